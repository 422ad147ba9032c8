"""Incremental binning (launch configuration incremental_sort = 1) against a numpy
restatement of the stable block sort (Group_Particles, MPM_Example.cpp:464-485), bit for
bit on every substep of GPU trajectories.

The substep's binning sorts the current slots by block, stably. In the incremental mode
only the slots whose block changed since the previous substep go through the radix
passes; the rest keep their order and the two are merged. The restatement here does not
know which mode ran: from the slot order before the substep (sort state: keys and
particle of every slot) and the particle positions it computes each slot's key, sorts the
slots stably by block, and lays every work item out as P2G stores it (cells in scatter
rank, pass-major; removed particles last in sorted order). The sort state after the
substep must equal that, key for key and slot for slot.

Trajectories: a ball landing on the sticky ground (FP32, FP64), a ball thrown out
through a face so that particles are removed and then allocated again, an 800K-particle
ball (hundreds of key-pass tiles and several tiles of moved particles), five scenes of
the 64-scene batch in one context (mixed precision, block ids offset per scene), a run
that switches between the full and the incremental sort every few substeps, eager
substeps, whole frames on the device, and 2,000 particles moved at once into one corner
(the merge's long-range path).
"""
import numpy as np
import pytest

from non_ficks_diffusion_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

DT = 1e-4
SENTINEL = np.uint32(0xFFFFFFFF)


def _block_bases(descs):
    bases = [0]
    for d in descs:
        nb = np.array(d.counts[:3]) // 4 + 2
        bases.append(bases[-1] + int(np.prod(nb)))
    return bases


def _cell_keys(X, counts, dtype):
    x = X.astype(dtype)
    c = np.floor(x * np.array(counts, dtype=dtype)).astype(np.int64)
    s = c + 4
    b, l = s >> 2, s & 3
    nb = np.array(counts) // 4 + 2
    gb = b[:, 0] + nb[0] * (b[:, 1] + nb[1] * b[:, 2])
    return gb, l[:, 0] | (l[:, 1] << 2) | (l[:, 2] << 4)


def _slot_keys(ctx, descs, order, scn, dtype):
    """Key of every slot of the current buffer from the particle positions (sentinel for
    removed particles)."""
    bases = _block_bases(descs)
    keys = np.full(len(order), SENTINEL, np.uint32)
    for s, d in enumerate(descs):
        p = ctx.particles(s)
        sel = np.flatnonzero(scn == s)
        loc = order[sel]
        ok = p["valid"][loc]
        gb, l = _cell_keys(p["X"][loc[ok]], list(d.counts[:3]), dtype)
        keys[sel[ok]] = ((gb + bases[s]) << 6 | l).astype(np.uint32)
    return keys


def _cell_rank():
    l = np.arange(64)
    bank = ((l & 3) + 6 * ((l >> 2) & 3) + 40 * (l >> 4)) % 32
    rank = np.empty(64, np.int64)
    rank[np.lexsort((l, bank))] = np.arange(64)
    return rank


RANK = _cell_rank()


def _pass_major(idx):
    n = len(idx)
    stride = (n + 31) // 32
    return np.asarray([idx[lane * stride + q] for q in range(stride) for lane in range(32) if lane * stride + q < n],
                      dtype=idx.dtype)


def _expected_layout(slot_keys, chunk):
    """Slots in the order P2G stores them after a stable sort by block."""
    perm = np.argsort(slot_keys >> 6, kind="stable")
    sk = slot_keys[perm]
    nv = int((sk != SENTINEL).sum())
    blk = sk[:nv] >> 6
    first = np.r_[True, blk[1:] != blk[:-1]] if nv else np.zeros(0, bool)
    start = np.maximum.accumulate(np.where(first, np.arange(nv), 0)) if nv else np.zeros(0, np.int64)
    heads = np.flatnonzero((np.arange(nv) - start) % chunk == 0)
    out = []
    for s, e in zip(heads, np.r_[heads[1:], nv]):
        item = perm[s:e]
        out.append(_pass_major(item[np.argsort(RANK[slot_keys[item] & 63], kind="stable")]))
    out.append(perm[nv:])
    return np.concatenate(out)


def _check_step(ctx, descs, dtype, step=lambda c: c.step(DT)):
    keys0, order0, scn0 = ctx.sort_state()
    sk = _slot_keys(ctx, descs, order0, scn0, dtype)
    want = _expected_layout(sk, ctx.launch_config()["chunk"])
    step(ctx)
    keys1, order1, scn1 = ctx.sort_state()
    nv = int((sk != SENTINEL).sum())
    assert np.array_equal(keys1[:nv], sk[want][:nv])
    assert np.all(keys1[nv:] == SENTINEL)
    assert np.array_equal(order1, order0[want])
    assert np.array_equal(scn1, scn0[want])
    moved = int(((keys0 >> 6) != (sk >> 6)).sum())
    return moved


def _ctx(descs_parts, prec, incremental=1, max_particles=None):
    n = sum(len(p["mass"]) for _, p in descs_parts)
    ctx = capi.Context(precision=prec, max_particles=max_particles or n, max_scenes=len(descs_parts))
    for d, p in descs_parts:
        sid = ctx.add_scene(d)
        ctx.add_particles(sid, p["X"], p["V"], p["mass"], p["lambda0"], p["mu0"])
    ctx.set_launch_config(incremental_sort=incremental)
    ctx.initialize()
    return ctx


DTYPE = {"fp32": np.float32, "mixed": np.float32, "fp64": np.float64}


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_incremental_sort_on_a_landing_ball(built_lib, prec):
    d, p = workloads.ball_scene(n=32, center=(0.5, 0.17, 0.5), radius=0.1, velocity=(0.0, -6.0, 0.0), seed=31)
    ctx = _ctx([(d, p)], prec)
    assert ctx.launch_config()["incremental_sort"] == 1
    moved = [_check_step(ctx, [d], DTYPE[prec]) for _ in range(30)]
    # the body moves between blocks on most substeps, but only a small part of it at once
    assert sum(m > 0 for m in moved) > 10 and max(moved) < len(p["mass"]) // 4


def test_incremental_sort_with_removed_and_allocated_particles(built_lib):
    d, p = workloads.ball_scene(n=32, center=(0.85, 0.5, 0.5), radius=0.1, velocity=(12.0, 0.0, 0.0), seed=34)
    d.n_barriers = 1          # nothing stops the ball at the +x face
    ctx = _ctx([(d, p)], "fp32")
    for _ in range(60):
        _check_step(ctx, [d], np.float32)
    assert (~ctx.particles(0)["valid"]).sum() > 60
    rng = np.random.default_rng(5)
    X = np.asarray((0.3, 0.5, 0.5)) + (rng.random((40, 3)) - 0.5) * 0.06
    ctx.allocate_particles(0, X, np.tile([0.0, -1.0, 0.0], (40, 1)), p["mass"][:40], p["lambda0"][:40], p["mu0"][:40])
    for _ in range(10):
        _check_step(ctx, [d], np.float32)


def test_incremental_sort_on_a_large_ball(built_lib):
    """About 800K particles: ~400 tiles of the moved-slot scan, and the first substep (whose
    previous keys come from the initial full grid build) moves no slot."""
    d, p = workloads.ball_scene(n=96, radius=0.3, velocity=(0.0, -3.0, 0.0))
    ctx = _ctx([(d, p)], "fp32")
    moved = [_check_step(ctx, [d], np.float32) for _ in range(6)]
    assert moved[0] == 0 and sum(moved) > 0


def _smallest_batch_scenes(k):
    sizes = []
    for s in range(64):
        d, i = capi.SceneDesc(), capi.PresetInfo()
        assert capi.lib().mpm_preset_scene(104, s, 0, capi.C.byref(d), capi.C.byref(i)) == capi.OK
        sizes.append(i.n_particles)
    return sorted(np.argsort(sizes)[:k].tolist())


def test_incremental_sort_on_batch_scenes(built_lib):
    ctx, scenes = workloads.make_context(104, precision="mixed", scene_indices=_smallest_batch_scenes(5))
    ctx.set_launch_config(incremental_sort=1)
    descs = [d for d, _, _ in scenes]
    moved = [_check_step(ctx, descs, np.float32) for _ in range(15)]
    assert sum(moved) > 0


def test_switching_between_full_and_incremental_sort(built_lib):
    d, p = workloads.ball_scene(n=32, center=(0.5, 0.17, 0.5), radius=0.1, velocity=(0.0, -6.0, 0.0), seed=31)
    ctx = _ctx([(d, p)], "fp32", incremental=0)
    ref = _ctx([(d, p)], "fp32", incremental=0)
    for k in range(24):
        ctx.set_launch_config(incremental_sort=(k // 4) % 2)
        _check_step(ctx, [d], np.float32)
        ref.step(DT)
    # the same trajectory as the context that always sorted fully, within FP32 rounding
    # (float atomics reorder sums)
    dx = 1.0 / d.counts[0]
    assert np.abs(ctx.particles(0)["X"] - ref.particles(0)["X"]).max() <= 2e-5 * dx


def test_incremental_sort_in_eager_substeps(built_lib):
    """Substeps launched one kernel at a time (no CUDA graph) go through the same binning."""
    d, p = workloads.ball_scene(n=32, center=(0.5, 0.17, 0.5), radius=0.1, velocity=(0.0, -6.0, 0.0), seed=31)
    ctx = capi.Context(precision="fp32", max_particles=len(p["mass"]), max_scenes=1, use_graphs=False)
    ctx.add_scene(d)
    ctx.add_particles(0, p["X"], p["V"], p["mass"], p["lambda0"], p["mu0"])
    ctx.set_launch_config(incremental_sort=1)
    ctx.initialize()
    for _ in range(12):
        _check_step(ctx, [d], np.float32)


def test_frames_on_the_device_with_incremental_sort(built_lib):
    """mpm_advance_to_time runs whole frames as one graph launch (nested conditional nodes);
    with the incremental binning inside it the run follows the full-sort run: the same
    substep counts, and FP64 positions equal within 1e-9 dx (float atomics reorder sums)."""
    d, p = workloads.ball_scene(n=32, center=(0.5, 0.2, 0.5), radius=0.1, velocity=(1.0, -4.0, 0.5), seed=5)
    runs = []
    for inc in (0, 1):
        ctx = _ctx([(d, p)], "fp64", incremental=inc)
        ks = [ctx.advance_to_time(t) for t in (0.01, 0.02, 0.03)]
        runs.append((ks, ctx.particles(0)))
        keys, order, scn = ctx.sort_state()
        assert np.all(np.diff((keys >> 6).astype(np.int64)) >= 0)
    (ka, ga), (kb, gb) = runs
    assert ka == kb and sum(ka) > 20
    assert np.array_equal(ga["valid"], gb["valid"])
    assert np.abs(ga["X"] - gb["X"]).max() <= 1e-9 / 32


def test_incremental_sort_after_a_mass_move(built_lib):
    """2,000 particles moved at once into a few blocks (mpm_set_particles between substeps):
    their merge ranks crowd into one merge tile, beyond the 256 that the merge stages 32 at
    a time, so that tile takes the per-slot binary search."""
    d, p = workloads.ball_scene(n=32, center=(0.5, 0.5, 0.5), radius=0.15, velocity=(0.0, 0.0, 0.0), seed=9)
    ctx = _ctx([(d, p)], "fp64")
    _check_step(ctx, [d], np.float64)
    q = ctx.particles(0)
    n = len(q["mass"])
    X = np.ascontiguousarray(q["X"])
    rng = np.random.default_rng(2)
    sel = rng.choice(n, 2000, replace=False)
    X[sel] = np.asarray((0.3, 0.3, 0.3)) + rng.random((2000, 3)) * (2.0 / 32)   # into a 2x2x2-cell corner
    ctx.set_particles(0, X=X, V=np.ascontiguousarray(q["V"]))
    moved = _check_step(ctx, [d], np.float64)
    assert moved >= 2000
    for _ in range(3):
        _check_step(ctx, [d], np.float64)
