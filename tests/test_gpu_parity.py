"""GPU parity tests: the sm_103a path through the C ABI against the CPU oracle.

Integer work (cell keys, the stable sort, active blocks, the Interior set, flag counts) is
compared bit for bit; floating-point results within the tolerances written in each test.
Tolerances: FP64 GPU vs FP64 oracle 1e-9 (relative, or in units of dx for positions) —
only summation order differs; FP32 and mixed vs the oracle of the same precision 2e-5 —
float atomics reorder sums and the CG may stop one iteration apart.
"""
import re

import numpy as np
import pytest

import oracle_lib
from non_ficks_diffusion_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-9, "mixed": 2e-5, "fp32": 2e-5}


def _ctx(desc, parts, prec, graphs=True, chunk=512):
    ctx = capi.Context(precision=prec, max_particles=len(parts["mass"]), max_scenes=1, use_graphs=graphs, chunk=chunk)
    sid = ctx.add_scene(desc)
    ctx.add_particles(sid, parts["X"], parts["V"], parts["mass"], parts["lambda0"], parts["mu0"])
    ctx.initialize()
    return ctx


def _oracle(desc, parts, prec):
    return oracle_lib.oracle_from_desc(desc, parts, precision=capi.PRECISIONS[prec])


def _expected_keys(X, counts, dtype):
    x = X.astype(dtype)
    c = np.floor(x * np.array(counts, dtype=dtype)).astype(np.int64)
    s = c + 4
    b, l = s >> 2, s & 3
    nb = np.array(counts) // 4 + 2
    gb = b[:, 0] + nb[0] * (b[:, 1] + nb[1] * b[:, 2])
    return ((gb << 6) | l[:, 0] | (l[:, 1] << 2) | (l[:, 2] << 4)).astype(np.uint32)


@pytest.fixture(scope="module")
def ball():
    return workloads.ball_scene(n=32, radius=0.12)


@pytest.fixture(scope="module")
def big_ball():
    """About 800K particles: hundreds of binning segments and of 4096-key sort tiles, so
    the look-backs between segments and between tiles run (the small ball fits in one)."""
    return workloads.ball_scene(n=96, radius=0.3)


@pytest.mark.parametrize("scene", ["ball", "big_ball"])
@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_sort_is_stable_and_bit_exact(built_lib, request, scene, prec):
    desc, parts = request.getfixturevalue(scene)
    ctx = _ctx(desc, parts, prec)
    keys, order, scn = ctx.sort_state()
    exp = _expected_keys(parts["X"], list(desc.counts), np.float32 if prec == "fp32" else np.float64)
    perm = np.argsort(exp >> 6, kind="stable")      # stable, by block
    assert np.array_equal(keys, exp[perm])
    assert np.array_equal(order, perm)
    assert np.all(scn == 0)


def _cell_rank():
    """Scatter order of a block's 64 cells: by shared-memory bank of the tile address
    x + 6y + 40z (mod 32), then by cell index."""
    l = np.arange(64)
    bank = ((l & 3) + 6 * ((l >> 2) & 3) + 40 * (l >> 4)) % 32
    rank = np.empty(64, np.int64)
    rank[np.lexsort((l, bank))] = np.arange(64)
    return rank


def _stored_order(ordered):
    """A work item's storage order: warp pass q gives lane L the ordered slot L*stride + q,
    stored at position run[q] + L (run[q] = valid slots of the passes before q)."""
    n = len(ordered)
    stride = (n + 31) // 32
    out = []
    for q in range(stride):
        for lane in range(32):
            k = lane * stride + q
            if k < n:
                out.append(ordered[k])
    return np.asarray(out, dtype=ordered.dtype)


@pytest.mark.parametrize("scene,chunk", [("ball", 64), ("ball", 512), ("big_ball", 64), ("big_ball", 1024)])
def test_p2g_writes_work_items_in_cell_order(built_lib, request, scene, chunk):
    """After a substep the keys are those of the sorted particles, ordered by block and,
    inside each work item, by the scatter rank of the cell, stored pass-major so that a
    warp's lanes read consecutive positions: P2G wrote the new buffer in that order."""
    desc, parts = request.getfixturevalue(scene)
    ctx = _ctx(desc, parts, "fp32", chunk=chunk)
    ctx.step(1e-4)
    keys, _, _ = ctx.sort_state()
    k0 = _expected_keys(parts["X"], list(desc.counts), np.float32)
    exp = k0[np.argsort(k0 >> 6, kind="stable")]
    n = len(exp)
    blk = exp >> 6
    first = np.r_[True, blk[1:] != blk[:-1]]
    start = np.maximum.accumulate(np.where(first, np.arange(n), 0))
    heads = np.flatnonzero((np.arange(n) - start) % chunk == 0)
    rank = _cell_rank()
    want = np.concatenate([_stored_order(exp[s:e][np.argsort(rank[exp[s:e] & 63], kind="stable")])
                           for s, e in zip(heads, np.r_[heads[1:], n])])
    assert np.array_equal(keys[:n], want)


@pytest.mark.parametrize("scene,chunk", [("ball", 64), ("ball", 512), ("big_ball", 256)])
def test_active_blocks_bit_exact(built_lib, request, scene, chunk):
    """The active blocks are exactly those that some particle's 3x3x3 stencil reaches
    (a particle at local cell l reaches the block below on an axis when l == 0 and the
    block above when l == 3), whatever the work-item size."""
    desc, parts = request.getfixturevalue(scene)
    ctx = _ctx(desc, parts, "fp32", chunk=chunk)
    got = {tuple(b) for b in ctx.active_blocks()}
    keys = _expected_keys(parts["X"], list(desc.counts), np.float32)
    keys = keys[keys != 0xFFFFFFFF]
    nb = np.array(desc.counts) // 4 + 2
    g = (keys >> 6).astype(np.int64)
    b = np.stack([g % nb[0], (g // nb[0]) % nb[1], g // (nb[0] * nb[1])], 1)
    l = keys & 63
    loc = np.stack([l & 3, (l >> 2) & 3, l >> 4], 1)
    exp = set()
    for ox in (-1, 0, 1):
        for oy in (-1, 0, 1):
            for oz in (-1, 0, 1):
                sel = np.ones(len(keys), bool)
                for a, o in enumerate((ox, oy, oz)):
                    if o == -1:
                        sel &= loc[:, a] == 0
                    elif o == 1:
                        sel &= loc[:, a] == 3
                nbrs = np.unique(b[sel] + np.array([ox, oy, oz]) - 1, axis=0)
                exp.update(map(tuple, nbrs.tolist()))
    assert got == exp


def _match_nodes(g, r):
    gi = {tuple(c): i for i, c in enumerate(g["coords"])}
    ri = {tuple(c): i for i, c in enumerate(r["coords"])}
    assert set(gi) == set(ri), "Interior node sets differ"
    keys = sorted(ri)
    return np.array([gi[k] for k in keys]), np.array([ri[k] for k in keys])


@pytest.mark.parametrize("prec", ["fp32", "mixed", "fp64"])
def test_rasterize_interior_set_and_values(built_lib, ball, prec):
    desc, parts = ball
    ctx = _ctx(desc, parts, prec)
    o = _oracle(desc, parts, prec)
    ctx.step_partial(1e-4, 1)
    o.step(1e-4, 1)
    g, r = ctx.interior_nodes(), o.interior()
    a, b = _match_nodes(g, r)
    tol = TOL[prec]
    assert np.allclose(g["m"][a], r["m"][b], rtol=tol, atol=0)
    scale = np.abs(r["v"]).max()
    assert np.abs(g["v"][a] - r["v"][b]).max() <= tol * scale
    assert np.array_equal(ctx.flag_counts(), o.flag_counts())


@pytest.mark.parametrize("prec", ["fp32", "mixed", "fp64"])
def test_explicit_force_and_collision(built_lib, ball, prec):
    desc, parts = ball
    ctx = _ctx(desc, parts, prec)
    o = _oracle(desc, parts, prec)
    ctx.step(1e-4, 2)
    for _ in range(2):
        o.step(1e-4)
    ctx.step_partial(1e-4, 2)
    o.step(1e-4, 2)
    g, r = ctx.interior_nodes(), o.interior()
    a, b = _match_nodes(g, r)
    scale = np.abs(r["vs"]).max()
    assert np.abs(g["vs"][a] - r["vs"][b]).max() <= TOL[prec] * scale


@pytest.mark.parametrize("prec", ["fp32", "mixed", "fp64"])
def test_cg_solution(built_lib, ball, prec):
    desc, parts = ball
    ctx = _ctx(desc, parts, prec)
    o = _oracle(desc, parts, prec)
    ctx.step_partial(1e-4, 3)
    o.step(1e-4, 3)
    g, r = ctx.interior_nodes(), o.interior()
    a, b = _match_nodes(g, r)
    scale = np.abs(r["vs"]).max()
    assert np.abs(g["vs"][a] - r["vs"][b]).max() <= TOL[prec] * scale
    gs, os_ = ctx.stats(), o.stats()
    assert abs(gs["cg_iterations"] - os_["cg_iterations"]) <= (0 if prec == "fp64" else 1)


@pytest.mark.parametrize("prec", ["fp32", "mixed", "fp64"])
@pytest.mark.parametrize("graphs", [True, False])
def test_substeps_match_oracle(built_lib, ball, prec, graphs):
    desc, parts = ball
    ctx = _ctx(desc, parts, prec, graphs=graphs)
    o = _oracle(desc, parts, prec)
    steps = 6
    ctx.step(1e-4, steps)
    for _ in range(steps):
        o.step(1e-4)
    g, r = ctx.particles(0), o.particles()
    dx = 1.0 / desc.counts[0]
    assert np.array_equal(g["valid"], r["valid"])
    assert np.abs(g["X"] - r["X"]).max() <= TOL[prec] * dx
    assert np.abs(g["V"] - r["V"]).max() <= TOL[prec] * max(1.0, np.abs(r["V"]).max())
    assert np.abs(g["Fe"] - r["Fe"]).max() <= 10 * TOL[prec]
    assert np.abs(g["Jp"] - r["Jp"]).max() <= 10 * TOL[prec]
    assert np.allclose(g["V0"], r["V0"], rtol=TOL[prec])


def test_batched_scenes_equal_separate_runs(built_lib):
    descs = []
    for i, (n, c, v) in enumerate([(32, (0.5, 0.6, 0.5), (0, -3, 0)), (16, (0.4, 0.5, 0.6), (1, -2, 0)),
                                   (64, (0.5, 0.4, 0.5), (0, -1, 2))]):
        descs.append(workloads.ball_scene(n=n, center=c, radius=0.1, velocity=v, seed=i + 3))
    total = sum(len(p["mass"]) for _, p in descs)
    ctx = capi.Context(precision="fp64", max_particles=total, max_scenes=3)
    for d, p in descs:
        sid = ctx.add_scene(d)
        ctx.add_particles(sid, p["X"], p["V"], p["mass"], p["lambda0"], p["mu0"])
    ctx.initialize()
    ctx.step(1e-4, 4)
    for i, (d, p) in enumerate(descs):
        single = _ctx(d, p, "fp64")
        single.step(1e-4, 4)
        a, b = ctx.particles(i), single.particles(0)
        assert np.abs(a["X"] - b["X"]).max() <= 1e-12
        assert ctx.stats(i)["cg_iterations"] == single.stats(0)["cg_iterations"]


def test_set_get_particles_roundtrip(built_lib, ball):
    desc, parts = ball
    ctx = _ctx(desc, parts, "fp64")
    ctx.step(1e-4, 2)
    p = ctx.particles(0)
    n = len(p["X"])
    X = np.ascontiguousarray(p["X"] + 1e-3)
    V = np.ascontiguousarray(p["V"] * 0.5)
    Fe = np.ascontiguousarray(p["Fe"].reshape(n, 9))
    ctx.set_particles(0, X=X, V=V, Fe=Fe, Jp=np.ascontiguousarray(p["Jp"]))
    q = ctx.particles(0)
    assert np.array_equal(q["X"], X) and np.array_equal(q["V"], V)
    assert np.array_equal(q["Fe"].reshape(n, 9), Fe) and np.array_equal(q["Jp"], p["Jp"])
    assert np.array_equal(q["mass"], p["mass"]) and np.array_equal(q["V0"], p["V0"])


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_direct_and_staged_host_transfers_agree(built_lib, ball, monkeypatch, dtype):
    """mpm_set_particles / mpm_get_particles read and write host arrays in place where the
    GPU can reach them, and go through a device staging copy otherwise
    (MPM_HOST_DIRECT=0 forces the copy). Both must move exactly the same values."""
    desc, parts = ball
    a = _ctx(desc, parts, "fp64")
    monkeypatch.setenv("MPM_HOST_DIRECT", "0")
    b = _ctx(desc, parts, "fp64")
    monkeypatch.delenv("MPM_HOST_DIRECT")
    a.step(1e-4, 2)
    p = a.particles(0)
    n = len(p["X"])
    arrays = {k: np.ascontiguousarray(v.reshape(n, -1) if k == "Fe" else v, dtype=dtype)
              for k, v in dict(X=p["X"] * 0.999 + 5e-4, V=p["V"], Fe=p["Fe"], Jp=p["Jp"], V0=p["V0"], mass=p["mass"],
                               lambda0=parts["lambda0"], mu0=parts["mu0"]).items()}
    arrays["valid"] = (np.arange(n) % 7 != 0).astype(np.int32)      # every 7th particle removed
    a.set_particles(0, **arrays)
    b.set_particles(0, **arrays)
    qa, qb = a.particles(0, dtype), b.particles(0, dtype)
    for k in ("X", "V", "Fe", "Jp", "V0", "mass", "lambda0", "mu0", "valid"):
        assert np.array_equal(qa[k], qb[k]), k
    assert np.array_equal(qa["valid"], arrays["valid"]) and np.array_equal(qa["lambda0"], arrays["lambda0"])
    assert np.array_equal(qa["X"], arrays["X"]) and np.array_equal(qa["Fe"].reshape(n, 9), arrays["Fe"])
    a.step(1e-4, 2)
    b.step(1e-4, 2)
    ra, rb = a.particles(0), b.particles(0)
    assert np.abs(ra["X"] - rb["X"]).max() <= 1e-9 / desc.counts[0]
    gone = arrays["valid"] == 0
    assert np.array_equal(ra["X"][gone], arrays["X"][gone].astype(np.float64)) and not ra["valid"][gone].any()


@pytest.mark.parametrize("pinned", [True, False])
def test_batched_host_transfers_equal_per_scene_calls(built_lib, pinned, monkeypatch):
    """mpm_set_particles_batch / mpm_get_particles_batch over three scenes move exactly what
    the per-scene calls move, in place (pinned host arrays) and through the staging copy
    (MPM_HOST_DIRECT=0), including a scene given twice and the removed flags."""
    import torch
    if not pinned:
        monkeypatch.setenv("MPM_HOST_DIRECT", "0")
    balls = [workloads.ball_scene(n=32, center=c, radius=0.08, seed=s)
             for c, s in (((0.3, 0.5, 0.5), 1), ((0.6, 0.4, 0.5), 2), ((0.5, 0.7, 0.4), 3))]
    n_all = sum(len(p["mass"]) for _, p in balls)
    ctxs = []
    for _ in range(2):
        ctx = capi.Context(precision="fp32", max_particles=n_all, max_scenes=3)
        for d, p in balls:
            sid = ctx.add_scene(d)
            ctx.add_particles(sid, p["X"], p["V"], p["mass"], p["lambda0"], p["mu0"])
        ctx.initialize()
        ctx.step(1e-4, 2)
        ctxs.append(ctx)
    a, b = ctxs

    def buf(shape):
        return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy() if pinned else np.empty(shape, np.float32)
    ins, outs_a, outs_b, keep = [], [], [], []
    for s, (d, p) in enumerate(balls):
        q = a.particles(s, np.float32)
        n = len(q["mass"])
        h = {k: buf(v.shape if k != "Fe" else (n, 9)) for k, v in q.items() if k in ("X", "V", "Fe", "Jp", "mass", "V0")}
        for k in h:
            h[k][...] = (q[k].reshape(n, 9) if k == "Fe" else q[k]) * (1.0 + 1e-3 * s)
        valid = (np.arange(n) % (5 + s) != 0).astype(np.int32)
        ins.append(capi.particle_arrays(n, np.float32, **h, valid=valid))
        oa = {k: buf(v.shape) for k, v in h.items()}
        ob = {k: buf(v.shape) for k, v in h.items()}
        va, vb = np.empty(n, np.int32), np.empty(n, np.int32)
        outs_a.append(capi.particle_arrays(n, np.float32, **oa, valid=va))
        outs_b.append(capi.particle_arrays(n, np.float32, **ob, valid=vb))
        keep.append((h, valid, oa, ob, va, vb))
    L = capi.lib()
    ids = [0, 1, 2, 1]                      # scene 1 twice: the second copy wins, as in calls one by one
    arr = (capi.ParticleArrays * 4)(*[ins[i] for i in ids])
    assert L.mpm_set_particles_batch(a.h, 4, (capi.C.c_int * 4)(*ids), arr) == capi.OK
    for i in ids:
        assert L.mpm_set_particles(b.h, i, capi.C.byref(ins[i])) == capi.OK
    outa = (capi.ParticleArrays * 3)(*outs_a)
    assert L.mpm_get_particles_batch(a.h, 3, (capi.C.c_int * 3)(0, 1, 2), outa) == capi.OK
    for i in range(3):
        assert L.mpm_get_particles(b.h, i, capi.C.byref(outs_b[i])) == capi.OK
    for h, valid, oa, ob, va, vb in keep:
        for k in oa:
            assert np.array_equal(oa[k], ob[k]) and np.array_equal(oa[k], h[k]), k
        assert np.array_equal(va, vb) and np.array_equal(va, valid)
    assert L.mpm_set_particles_batch(a.h, 1, (capi.C.c_int * 1)(5), arr) == capi.BAD_ARG


@pytest.mark.parametrize("prec", ["fp32", "mixed", "fp64"])
def test_eos_fluid_ball_matches_oracle(built_lib, prec):
    """The EOS fluid material (test 19's branch) on the GPU against the oracle: explicit
    pressure force, its CG term and the density update, which lives in the Jp slot."""
    desc, parts = workloads.ball_scene(n=32, radius=0.12, velocity=(0.5, -2.0, 0.0), seed=4)
    desc.material, desc.bulk_modulus, desc.eos_gamma = capi.MATERIAL_EOS_FLUID, 50.0, 7.0
    ctx = _ctx(desc, parts, prec)
    o = _oracle(desc, parts, prec)
    steps = 6
    ctx.step(1e-4, steps)
    for _ in range(steps):
        o.step(1e-4)
    g, r = ctx.particles(0), o.particles()
    dx = 1.0 / desc.counts[0]
    assert not np.allclose(r["Jp"], 1.0)
    assert np.abs(g["X"] - r["X"]).max() <= TOL[prec] * dx
    assert np.abs(g["V"] - r["V"]).max() <= TOL[prec] * max(1.0, np.abs(r["V"]).max())
    assert np.abs(g["Jp"] - r["Jp"]).max() <= 10 * TOL[prec]
    assert np.array_equal(g["Fe"], r["Fe"])


@pytest.mark.parametrize("prec", ["fp32", "mixed", "fp64"])
def test_colliding_balls_with_plastic_flow(built_lib, prec):
    """Two balls closing at 16 m/s: the snow plasticity clamp is active for many particles,
    exercising the clamped SVD path (FP64 Jacobi in the mixed and FP64 variants)."""
    da, pa = workloads.ball_scene(n=32, center=(0.39, 0.5, 0.5), radius=0.1, velocity=(8.0, 0, 0), seed=11)
    db, pb = workloads.ball_scene(n=32, center=(0.61, 0.5, 0.5), radius=0.1, velocity=(-8.0, 0, 0), seed=12)
    parts = {k: np.concatenate([pa[k], pb[k]]) for k in pa}
    ctx = _ctx(da, parts, prec)
    o = _oracle(da, parts, prec)
    steps = 30
    ctx.step(1e-4, steps)
    for _ in range(steps):
        o.step(1e-4)
    g, r = ctx.particles(0), o.particles()
    assert (r["Jp"] < 0.999).sum() > 100, "the plasticity clamp should be active"
    dx = 1.0 / 32
    tol = {"fp64": 1e-9, "mixed": 2e-4, "fp32": 2e-4}[prec]
    assert np.array_equal(g["valid"], r["valid"])
    assert np.abs(g["X"] - r["X"]).max() <= tol * dx
    assert np.abs(g["Jp"] - r["Jp"]).max() <= 10 * tol
    assert np.abs(g["Fe"] - r["Fe"]).max() <= 10 * tol


def test_autotune_restores_the_state_and_keeps_a_candidate(built_lib, ball):
    desc, parts = ball
    ctx = _ctx(desc, parts, "fp32")
    ctx.step(1e-4, 2)
    before, n0 = ctx.particles(0), ctx.stats()["substeps"]
    r = ctx.autotune(1e-4, substeps=2)
    after = ctx.particles(0)
    for k in ("X", "V", "Fe", "Jp", "V0", "valid"):
        assert np.array_equal(before[k], after[k]), k
    assert ctx.stats()["substeps"] == n0
    ch = r["chosen"]
    assert ch == ctx.launch_config()
    assert ch["chunk"] in (256, 512, 1024, 2048) and ch["grid_per_sm"] in (4, 8, 12, 16)
    assert ch["node_grid_per_sm"] in (1, 2, 4, 8) and ch["hessian_warp_items"] in (0, 1, 2)
    assert all(ch[k] in (3, 4, 5, 6) for k in ("ctas_hessian", "ctas_p2g", "ctas_g2p"))
    assert r["trials"] >= 1 and 0 < r["ms_per_substep"] <= r["ms_per_substep_initial"]
    # the tuned context continues like an untuned one, within the FP32 tolerance
    ref = _ctx(desc, parts, "fp32")
    ref.step(1e-4, 2)
    ctx.step(1e-4, 3)
    ref.step(1e-4, 3)
    dx = 1.0 / desc.counts[0]
    assert np.abs(ctx.particles(0)["X"] - ref.particles(0)["X"]).max() <= TOL["fp32"] * dx


def test_launch_config_is_validated(built_lib, ball):
    desc, parts = ball
    ctx = _ctx(desc, parts, "fp32")
    for bad in ({"chunk": 16}, {"ctas_hessian": 7}, {"grid_per_sm": 0}, {"node_grid_per_sm": 65},
                {"hessian_warp_items": 3}, {"incremental_sort": 2}):
        with pytest.raises(capi.MPMError):
            ctx.set_launch_config(**bad)
    ctx.set_launch_config(chunk=256, ctas_p2g=5)
    assert ctx.launch_config()["chunk"] == 256 and ctx.launch_config()["ctas_p2g"] == 5
    ctx.step(1e-4, 2)
    ref = _ctx(desc, parts, "fp32")
    ref.step(1e-4, 2)
    dx = 1.0 / desc.counts[0]
    assert np.abs(ctx.particles(0)["X"] - ref.particles(0)["X"]).max() <= TOL["fp32"] * dx


def test_nonfinite_position_names_its_scene(built_lib):
    """A NaN velocity supplied by the host (the failure is made on the host; positions are
    range-checked on upload, velocities are not) turns scene 1's positions non-finite in the
    first substep. G2P's check (or the next key pass) reports MPM_NONFINITE; a scene named
    in the message must be scene 1."""
    da, pa = workloads.ball_scene(n=16, center=(0.3, 0.5, 0.5), radius=0.1, seed=21)
    db, pb = workloads.ball_scene(n=16, center=(0.7, 0.5, 0.5), radius=0.1, seed=22)
    pb = dict(pb)
    V = pb["V"].copy()
    V[5, 0] = np.nan
    pb["V"] = V
    ctx = capi.Context(precision="fp32", max_particles=len(pa["mass"]) + len(pb["mass"]), max_scenes=2)
    for d, p in ((da, pa), (db, pb)):
        sid = ctx.add_scene(d)
        ctx.add_particles(sid, p["X"], p["V"], p["mass"], p["lambda0"], p["mu0"])
    ctx.initialize()
    with pytest.raises(capi.MPMError) as ei:
        for _ in range(3):
            ctx.step(1e-4)
    assert ei.value.status == capi.NONFINITE
    named = re.search(r"highest scene index with one: (-?\d+)", str(ei.value))
    assert named is None or named.group(1) == "1", str(ei.value)


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_hessian_forms_match_oracle(built_lib, prec):
    """The Hessian product with work items per CTA, per warp and chosen per launch: the same
    CG iterations and particles as the oracle on the colliding balls (plastic flow, many CG
    iterations)."""
    da, pa = workloads.ball_scene(n=32, center=(0.39, 0.5, 0.5), radius=0.1, velocity=(8.0, 0, 0), seed=11)
    _, pb = workloads.ball_scene(n=32, center=(0.61, 0.5, 0.5), radius=0.1, velocity=(-8.0, 0, 0), seed=12)
    parts = {k: np.concatenate([pa[k], pb[k]]) for k in pa}
    o = _oracle(da, parts, prec)
    steps = 20
    its_o = []
    for _ in range(steps):
        o.step(1e-4)
        its_o.append(o.stats()["cg_iterations"])
    r = o.particles()
    assert sum(its_o) > steps
    dx = 1.0 / 32
    tol = {"fp64": 1e-9, "fp32": 2e-4}[prec]
    for form in (0, 1, 2):
        ctx = _ctx(da, parts, prec)
        ctx.set_launch_config(hessian_warp_items=form)
        its = []
        for _ in range(steps):
            ctx.step(1e-4)
            its.append(ctx.stats()["cg_iterations"])
        g = ctx.particles(0)
        assert all(abs(a - b) <= (0 if prec == "fp64" else 1) for a, b in zip(its, its_o)), (form, its, its_o)
        assert np.abs(g["X"] - r["X"]).max() <= tol * dx, form
