"""Barrier contact under GPU parity: the grid collision (Grid_Based_Collision_Helper.h:57-85,
MPM_Plane_Barrier.h:13-32), Project (Project_Helper.h:30-45, intended semantics) and the
out-of-domain removal of G2P (MPM_Example.cpp:654-660), each against the CPU oracle in
FP32, mixed and FP64.

Every scene starts with particles whose stencils reach nodes inside a barrier half-space,
so the collision rule runs on Interior nodes from the first substep:
  ground  a ball dropped at 6 m/s onto the sticky ground (v* = 0 inside it)
  wall    a ball thrown at 4 m/s into the +x wall, given friction mu = 0.3 (the friction
          branch and the stop branch of the collision rule)
  slab    a slab falling onto the 30-degree slip plane of the slab preset, on a 32^3 grid
  out     a ball thrown at 12 m/s through the +x face with no wall there: particles leave
          the cell domain [dx/2, 1-dx/2]^3 and are removed
Checked per test:
- on the first substep, from the same particles: v* after the collision rule on the same
  Interior node set, more than ten of those nodes inside the barrier's half-space (v* = 0
  there for the sticky ground), within 1e-9 (FP64) or 1e-5 (FP32, mixed) of the largest |v*|;
- over the run: the CG ran (the iteration total is positive) and took the same number of
  iterations as the oracle on every substep (FP64 exactly, FP32 and mixed within one);
- after the run: X, V, Fe, Jp and the removed set.
Tolerances after the run: FP64 1e-9 (in units of dx for positions); FP32 and mixed 1e-4 dx
for positions (the oracle's own FP32 and FP64 runs differ by 1-4e-5 dx here; float atomics
reorder sums on the GPU). Grid values after many FP32 substeps are not compared: FLIP
carries the particles' rounding differences into v = mv/m, which amplifies them at nodes of
small mass on the surface of the body.
"""
import numpy as np
import pytest

import oracle_lib
from non_ficks_diffusion_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

DT = 1e-4
TOL = {"fp64": 1e-9, "mixed": 1e-4, "fp32": 1e-4}
ITER_SLACK = {"fp64": 0, "mixed": 1, "fp32": 1}


def slab_on_plane(n=32, cy=0.39, velocity=(0.0, -4.0, 0.0), seed=33):
    """The slab preset's 0.5 x 0.08 x 0.5 slab and 30-degree slip plane (normal
    (-1/2, sqrt(3)/2, 0) through (0.5, 0.2, 0.5)) on an n^3 grid, with the slab lowered to
    y = cy so that its lower corner meets the plane at once; ground and walls 2 dx from the
    faces, 8 particles per cell."""
    d, _ = workloads.ball_scene(n=n)
    k = d.n_barriers
    b = d.barriers[k]
    b.normal[0], b.normal[1], b.normal[2] = -0.5, np.sqrt(3.0) / 2.0, 0.0
    b.surface[0], b.surface[1], b.surface[2] = 0.5, 0.2, 0.5
    b.mu, b.sticky = 0.0, 0
    d.n_barriers = k + 1
    dx = 1.0 / n
    rng = np.random.default_rng(seed)
    lo, hi = np.array([0.25, cy - 0.04, 0.25]), np.array([0.75, cy + 0.04, 0.75])
    g = [np.arange(int(np.floor(lo[a] * n)), int(np.ceil(hi[a] * n))) for a in range(3)]
    cells = np.stack(np.meshgrid(*g, indexing="ij"), -1).reshape(-1, 3)
    sub = np.stack(np.meshgrid(*[np.arange(2)] * 3, indexing="ij"), -1).reshape(-1, 3)
    X = ((cells[:, None, :] + (sub[None] + rng.random((len(cells), 8, 3))) / 2) * dx).reshape(-1, 3)
    X = X[np.all((X > lo) & (X < hi), 1)]
    N = len(X)
    E, nu, rho = 1.4e5, 0.2, 400.0
    parts = dict(X=X, V=np.tile(np.asarray(velocity, float), (N, 1)), mass=np.full(N, rho * dx ** 3 / 8),
                 lambda0=np.full(N, E * nu / ((1 + nu) * (1 - 2 * nu))), mu0=np.full(N, E / (2 * (1 + nu))))
    return d, parts


def contact_scene(name):
    """(desc, particles, substeps, index of the barrier the scene is about)."""
    if name == "ground":
        d, p = workloads.ball_scene(n=32, center=(0.5, 0.17, 0.5), radius=0.1, velocity=(0.0, -6.0, 0.0), seed=31)
        return d, p, 30, 0
    if name == "wall":
        d, p = workloads.ball_scene(n=32, center=(0.82, 0.5, 0.5), radius=0.1, velocity=(4.0, -2.0, 1.0), seed=32)
        for b in range(d.n_barriers):
            if d.barriers[b].normal[0] < -0.5:
                d.barriers[b].mu = 0.3
                wall = b
        return d, p, 30, wall
    if name == "slab":
        d, p = slab_on_plane()
        return d, p, 30, d.n_barriers - 1
    if name == "out":
        d, p = workloads.ball_scene(n=32, center=(0.85, 0.5, 0.5), radius=0.1, velocity=(12.0, 0.0, 0.0), seed=34)
        d.n_barriers = 1      # the sticky ground only: nothing stops the ball at the +x face
        return d, p, 60, None
    raise ValueError(name)


def inside_barrier(desc, b, coords):
    """Nodes (cell coordinates) whose centre lies in barrier b's half-space (x - s).n < 0."""
    dx = 1.0 / np.asarray(desc.counts[:3], float)
    x = (coords + 0.5) * dx
    br = desc.barriers[b]
    return ((x - np.asarray(br.surface[:3])) * np.asarray(br.normal[:3])).sum(1) < 0


def _ctx(desc, parts, prec):
    ctx = capi.Context(precision=prec, max_particles=len(parts["mass"]), max_scenes=1)
    sid = ctx.add_scene(desc)
    ctx.add_particles(sid, parts["X"], parts["V"], parts["mass"], parts["lambda0"], parts["mu0"])
    ctx.initialize()
    return ctx


def _match_nodes(g, r):
    gi = {tuple(c): i for i, c in enumerate(g["coords"])}
    ri = {tuple(c): i for i, c in enumerate(r["coords"])}
    assert set(gi) == set(ri), "Interior node sets differ"
    keys = sorted(ri)
    return np.array([gi[k] for k in keys]), np.array([ri[k] for k in keys])


@pytest.mark.parametrize("prec", ["fp32", "mixed", "fp64"])
@pytest.mark.parametrize("scene", ["ground", "wall", "slab"])
def test_collision_rule_on_first_substep(built_lib, scene, prec):
    desc, parts, _, barrier = contact_scene(scene)
    ctx = _ctx(desc, parts, prec)
    o = oracle_lib.oracle_from_desc(desc, parts, precision=capi.PRECISIONS[prec])
    ctx.step_partial(DT, 2)
    o.step(DT, 2)
    gn, rn = ctx.interior_nodes(), o.interior()
    a, b = _match_nodes(gn, rn)
    inside = inside_barrier(desc, barrier, rn["coords"][b])
    assert inside.sum() > 10, "no Interior node inside the barrier"
    if desc.barriers[barrier].sticky:
        assert np.all(gn["vs"][a][inside] == 0.0) and np.all(rn["vs"][b][inside] == 0.0)
    else:   # the normal component is gone where the body moves into the barrier
        n = np.asarray(desc.barriers[barrier].normal[:3])
        assert np.abs(rn["vs"][b][inside] @ n).max() < 1e-6
    scale = np.abs(rn["vs"]).max()
    tol = 1e-9 if prec == "fp64" else 1e-5
    assert np.abs(gn["vs"][a] - rn["vs"][b]).max() <= tol * scale


@pytest.mark.parametrize("prec", ["fp32", "mixed", "fp64"])
@pytest.mark.parametrize("scene", ["ground", "wall", "slab", "out"])
def test_barrier_contact_matches_oracle(built_lib, scene, prec):
    desc, parts, steps, barrier = contact_scene(scene)
    ctx = _ctx(desc, parts, prec)
    o = oracle_lib.oracle_from_desc(desc, parts, precision=capi.PRECISIONS[prec])
    gpu_iters, ora_iters = [], []
    for _ in range(steps):
        ctx.step(DT)
        o.step(DT)
        gpu_iters.append(ctx.stats()["cg_iterations"])
        ora_iters.append(o.stats()["cg_iterations"])
    slack = ITER_SLACK[prec]
    assert all(abs(a - b) <= slack for a, b in zip(gpu_iters, ora_iters)), (gpu_iters, ora_iters)
    if scene != "out" or prec != "fp64":       # FP64 free flight converges at iteration 0
        assert sum(ora_iters) > 0 and sum(gpu_iters) > 0

    g, r = ctx.particles(0), o.particles()
    dx = 1.0 / desc.counts[0]
    tol = TOL[prec]
    assert np.array_equal(g["valid"], r["valid"])
    if scene == "out":
        assert (~r["valid"]).sum() > 50, "particles should have left the cell domain"
    assert np.abs(g["X"] - r["X"]).max() <= tol * dx
    assert np.abs(g["V"] - r["V"]).max() <= tol * max(1.0, np.abs(r["V"]).max())
    assert np.abs(g["Fe"] - r["Fe"]).max() <= 10 * tol
    assert np.abs(g["Jp"] - r["Jp"]).max() <= 10 * tol
    if scene != "out":
        assert (r["Jp"] < 0.999).sum() > 10, "the impact should clamp some particles plastically"
