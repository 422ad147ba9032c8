"""Workloads: the scene presets of include/mpm_scenes.h loaded into a GPU context.

Named workloads follow the preset test numbers:
    c0  100  2D snowball 64^2 (CPU-only case; the GPU path is 3D)
    c1  101  3D snowball 128^3, ~237k particles
    c2  102  two colliding snowballs 256^3, ~1.94M particles
    c3  103  snow slab crash 512^3, ~21.5M particles
    c4  104  batch of 64 scenes, ~14.8M particles
"""
import numpy as np

from . import capi

WORKLOADS = {"c0": 100, "c1": 101, "c2": 102, "c3": 103, "c4": 104}


def scenes(test_number, seed=0, scene_indices=None, preset=None):
    """[(desc, info, particles)] for every scene of a preset (or the given indices).
    `preset`: the sampler to call (default capi.preset, from the GPU library)."""
    preset = preset or capi.preset
    desc, info, parts = preset(test_number, 0, seed)
    count = info.scene_count
    idx = list(range(count)) if scene_indices is None else list(scene_indices)
    out = []
    for i in idx:
        out.append((desc, info, parts) if i == 0 else preset(test_number, i, seed))
    return out


def make_context(test_number, precision="fp32", seed=0, scene_indices=None, use_graphs=True, chunk=0,
                 max_blocks=0, extra_particles=0):
    """A Context holding the preset's scenes, initialised. Returns (ctx, scene_list)."""
    sc = scenes(test_number, seed, scene_indices)
    n_total = sum(s[1].n_particles for s in sc)
    ctx = capi.Context(precision=precision, max_particles=n_total + extra_particles, max_scenes=max(1, len(sc)),
                       use_graphs=use_graphs, chunk=chunk, max_blocks=max_blocks)
    for desc, info, p in sc:
        sid = ctx.add_scene(desc)
        ctx.add_particles(sid, p["X"], p["V"], p["mass"], p["lambda0"], p["mu0"])
    ctx.initialize()
    return ctx, sc


def ball_scene(n=32, center=(0.5, 0.6, 0.5), radius=0.15, velocity=(0.0, -3.0, 0.0), ppc_axis=2, seed=1,
               E=1.4e5, nu=0.2, density=400.0):
    """A small seeded snowball with the preset solver settings (for tests and the smoke check)."""
    desc, _, _ = capi.preset(101)
    desc.counts[0] = desc.counts[1] = desc.counts[2] = n
    dx = 1.0 / n
    w = 2.0 * dx
    for b in range(desc.n_barriers):   # re-place the walls 2dx from the faces for this grid
        br = desc.barriers[b]
        for a in range(3):
            if br.normal[a] > 0.5:
                br.surface[a] = w
            elif br.normal[a] < -0.5:
                br.surface[a] = 1 - w
    rng = np.random.default_rng(seed)
    lo = max(0, int((min(center) - radius) * n) - 1)
    hi = min(n, int((max(center) + radius) * n) + 2)
    g = np.arange(lo, hi)
    cells = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    k = ppc_axis
    sub = np.stack(np.meshgrid(*[np.arange(k)] * 3, indexing="ij"), -1).reshape(-1, 3)
    X = ((cells[:, None, :] + (sub[None, :, :] + rng.random((len(cells), len(sub), 3))) / k) * dx).reshape(-1, 3)
    X = X[((X - np.asarray(center)) ** 2).sum(1) < radius * radius]
    N = len(X)
    mu0 = E / (2 * (1 + nu))
    lam0 = E * nu / ((1 + nu) * (1 - 2 * nu))
    parts = dict(X=X, V=np.tile(np.asarray(velocity, float), (N, 1)), mass=np.full(N, density * dx ** 3 / k ** 3),
                 lambda0=np.full(N, lam0), mu0=np.full(N, mu0))
    return desc, parts


def block_box_scene(n=64, lo=16, hi=48, velocity=(0.0, -1.0, 0.0), seed=0, E=1.4e5, nu=0.2, density=400.0):
    """A box of cells [lo, hi)^3 that fills whole 4^3-cell blocks (lo and hi multiples of
    4) with exactly 8 particles per cell, one in the middle half of each sub-cell, so that no
    particle changes cell for the first substeps: every work item is a full block, the
    case the transfer kernels' shared-memory cell order is laid out for (compare a ball,
    whose surface blocks are partly filled)."""
    desc, _ = ball_scene(n=n)
    dx = 1.0 / n
    rng = np.random.default_rng(seed)
    g = np.arange(lo, hi)
    cells = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    sub = np.stack(np.meshgrid(*[np.arange(2)] * 3, indexing="ij"), -1).reshape(-1, 3)
    X = ((cells[:, None, :] + (sub[None] + 0.25 + 0.5 * rng.random((len(cells), 8, 3))) / 2) * dx).reshape(-1, 3)
    N = len(X)
    parts = dict(X=X, V=np.tile(np.asarray(velocity, float), (N, 1)), mass=np.full(N, density * dx ** 3 / 8),
                 lambda0=np.full(N, E * nu / ((1 + nu) * (1 - 2 * nu))), mu0=np.full(N, E / (2 * (1 + nu))))
    return desc, parts


def run_scene(kind="box", precision="fp32", substeps=3, dt=1e-4, use_graphs=False):
    """Runs `substeps` substeps of a single-scene context holding block_box_scene() ("box")
    or a radius-0.25 ball on the same 64^3 grid ("ball"); eager substeps by default, so that
    a profiler sees every kernel launch. Returns the context."""
    desc, parts = block_box_scene() if kind == "box" else ball_scene(n=64, radius=0.25)
    ctx = capi.Context(precision=precision, max_particles=len(parts["mass"]), max_scenes=1, use_graphs=use_graphs)
    ctx.add_scene(desc)
    ctx.add_particles(0, parts["X"], parts["V"], parts["mass"], parts["lambda0"], parts["mu0"])
    ctx.initialize()
    ctx.step(dt, substeps)
    ctx.synchronize()
    return ctx


def shard_scenes(n_scenes, world_size, rank):
    """Scenes of rank `rank` when `n_scenes` independent scenes are split across `world_size`
    GPUs: contiguous, balanced ranges (the batch has no data exchange between scenes)."""
    base, extra = divmod(n_scenes, world_size)
    start = rank * base + min(rank, extra)
    return list(range(start, start + base + (1 if rank < extra else 0)))
