"""Failure reporting on the GPU, made without faulting the GPU: each failure comes from the
host's inputs (a CG iteration cap of one, a node-block capacity far too small) or from a
device wait given a short limit on a flag that nothing sets. The reference has no error
channel: its CG stops silently at the cap (MPM_CG_System.h:233-234) and capacity does not
exist (SPGrid grows). Each test also checks that the context reports the failure through
its status and message and, where the state stays valid, keeps working afterwards."""
import numpy as np
import pytest

import oracle_lib
from non_ficks_diffusion_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def _colliding_balls(cg_max_iters):
    da, pa = workloads.ball_scene(n=32, center=(0.39, 0.5, 0.5), radius=0.1, velocity=(8.0, 0, 0), seed=11)
    _, pb = workloads.ball_scene(n=32, center=(0.61, 0.5, 0.5), radius=0.1, velocity=(-8.0, 0, 0), seed=12)
    parts = {k: np.concatenate([pa[k], pb[k]]) for k in pa}
    da.cg_max_iters = cg_max_iters
    return da, parts


def _ctx(desc, parts, prec="fp32", **kw):
    ctx = capi.Context(precision=prec, max_particles=len(parts["mass"]), max_scenes=1, **kw)
    sid = ctx.add_scene(desc)
    ctx.add_particles(sid, parts["X"], parts["V"], parts["mass"], parts["lambda0"], parts["mu0"])
    return ctx


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("graphs", [True, False])
def test_cg_iteration_cap_reports_not_converged(built_lib, prec, graphs):
    """cg_max_iters = 1 on two balls colliding at 16 m/s: every substep stops its CG after
    one iteration, the call returns MPM_CG_NOT_CONVERGED, and the substep still completes,
    as in the oracle with the same cap."""
    desc, parts = _colliding_balls(cg_max_iters=1)
    ctx = _ctx(desc, parts, prec, use_graphs=graphs)
    ctx.initialize()
    o = oracle_lib.oracle_from_desc(desc, parts, precision=capi.PRECISIONS[prec])
    for k in range(8):
        st = ctx.step(1e-4)
        o.step(1e-4)
        s = ctx.stats()
        assert st == capi.CG_NOT_CONVERGED
        assert s["cg_iterations"] == 1 and not s["cg_converged"] and s["substeps"] == k + 1
        assert o.stats()["cg_iterations"] == 1 and not o.stats()["converged"]
    g, r = ctx.particles(0), o.particles()
    assert np.isfinite(g["X"]).all()
    tol = {"fp32": 1e-4, "fp64": 1e-9}[prec]
    assert np.abs(g["X"] - r["X"]).max() <= tol / desc.counts[0]


def test_block_capacity_reports_capacity(built_lib):
    """A node-block capacity of 8 for a ball whose stencils reach about 200 blocks: the grid
    build flags the overflow (blocks past the capacity get no node storage and every lookup
    of them reads 'inactive'), and mpm_initialize returns MPM_CAPACITY with its message."""
    desc, parts = workloads.ball_scene(n=32, radius=0.12)
    ctx = _ctx(desc, parts, max_blocks=8)
    with pytest.raises(capi.MPMError) as ei:
        ctx.initialize()
    assert ei.value.status == capi.CAPACITY
    assert "capacity exceeded" in str(ei.value)
    ctx.close()
    # the same scene with the derived capacity initialises and steps
    ok = _ctx(desc, parts)
    ok.initialize()
    assert ok.step(1e-4) == capi.OK


@pytest.mark.parametrize("spin_limit", [1, 1000, 20000])
def test_lookback_wait_gives_up_and_reports(built_lib, spin_limit):
    """One look-back of the binning scans on a status array whose predecessor never
    publishes, its wait limited to spin_limit polls: the wait gives up, the device flag is
    set, the call returns MPM_CUDA_ERROR naming the look-back, and the context goes on
    stepping normally afterwards."""
    desc, parts = workloads.ball_scene(n=32, radius=0.12)
    ctx = _ctx(desc, parts)
    ctx.initialize()
    before = ctx.particles(0)
    st = ctx.L.mpm_selftest_lookback_wait(ctx.h, spin_limit)
    assert st == capi.CUDA_ERROR
    assert b"look-back wait exceeded its limit" in ctx.L.mpm_last_error(ctx.h)
    assert ctx.L.mpm_selftest_lookback_wait(ctx.h, 0) == capi.BAD_ARG
    after = ctx.particles(0)
    assert np.array_equal(before["X"], after["X"])
    assert ctx.step(1e-4, 2) == capi.OK
    assert np.isfinite(ctx.particles(0)["X"]).all()
