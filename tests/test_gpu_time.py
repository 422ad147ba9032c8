"""Device-side CFL time stepping (mpm_advance_to_time) against the same rule driven from the
host (MPM_Driver::Advance_To_Target_Time, MPM_Driver.cpp:55-80): per substep
dt = clamp(cfl dx / max(max_v, 1e-2), 1e-6, 5e-3), the smallest over the scenes, with the
end-of-frame split. The host loop reads max_v with mpm_max_particle_velocity and issues
fixed-dt substeps, so both arms must take the same substeps and agree to the FP64 bar.
The oracle arm runs the reference's own loop (Max_Particle_Velocity, the dt rule and
Advance_Step, restated on the CPU) beside the device loop over a ball that hits the ground:
the same substep count, the same clock, and positions within the precision's bar."""
import numpy as np
import pytest

import oracle_lib
from non_ficks_diffusion_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def _ctx(scenes, prec, graphs=True):
    total = sum(len(p["mass"]) for _, p in scenes)
    ctx = capi.Context(precision=prec, max_particles=total, max_scenes=len(scenes), use_graphs=graphs)
    for d, p in scenes:
        sid = ctx.add_scene(d)
        ctx.add_particles(sid, p["X"], p["V"], p["mass"], p["lambda0"], p["mu0"])
    ctx.initialize()
    return ctx


def _host_cfl(ctx, scenes, target, cfl, prec):
    """The reference's loop, one fixed-dt substep at a time."""
    f = np.float32 if prec == "fp32" else np.float64
    dxs = [float(f(1.0) / f(d.counts[0])) for d, _ in scenes]
    k = 0
    while True:
        dt = min(max(1e-6, min(5e-3, cfl * dx / max(ctx.max_velocity(s), 1e-2))) for s, dx in enumerate(dxs))
        rem = target - ctx.time
        last = rem < dt * 1.001
        if last:
            dt = rem
        elif rem < 2 * dt:
            dt = rem * 0.5
        ctx.step(dt)
        k += 1
        if last:
            return k


def _scenes():
    return [workloads.ball_scene(n=32, radius=0.12, velocity=(0.0, -3.0, 0.0)),
            workloads.ball_scene(n=64, center=(0.4, 0.5, 0.6), radius=0.08, velocity=(2.0, -1.0, 0.0), seed=5)]


@pytest.mark.parametrize("graphs", [True, False])
@pytest.mark.parametrize("nscenes", [1, 2])
def test_device_cfl_matches_host_loop(built_lib, graphs, nscenes):
    scenes = _scenes()[:nscenes]
    target, cfl = 0.002, 0.02
    a = _ctx(scenes, "fp64", graphs)
    b = _ctx(scenes, "fp64")
    ka = a.advance_to_time(target, cfl)
    kb = _host_cfl(b, scenes, target, cfl, "fp64")
    assert ka == kb and ka > 3
    assert a.time == target and abs(b.time - target) < 1e-15
    assert a.stats()["substeps"] == kb
    for s, (d, _) in enumerate(scenes):
        pa, pb = a.particles(s), b.particles(s)
        assert np.abs(pa["X"] - pb["X"]).max() <= 1e-9 / d.counts[0]
        assert np.abs(pa["V"] - pb["V"]).max() <= 1e-9 * max(1.0, np.abs(pb["V"]).max())
    # a second advance continues from the clock; fixed-dt substeps afterwards still work
    a.advance_to_time(target + 0.001, cfl)
    assert a.time == target + 0.001
    a.step(1e-4)
    assert abs(a.time - (target + 0.0011)) < 1e-15


def test_substep_cap_and_past_targets(built_lib):
    scenes = _scenes()[:1]
    ctx = _ctx(scenes, "fp32")
    assert ctx.advance_to_time(1.0, 0.1, max_substeps=3) == 3
    t = ctx.time
    assert 0 < t < 1.0 and ctx.stats()["substeps"] == 3
    assert ctx.advance_to_time(t * 0.5) == 0 and ctx.time == t
    with pytest.raises(capi.MPMError):
        ctx.advance_to_time(2.0, cfl=0.0)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-9), ("fp32", 1e-4)])
def test_device_cfl_matches_oracle_driver_loop(built_lib, prec, tol):
    """Two 1/240 s advances with cfl 0.1: a ball at 6 m/s meets the sticky ground during
    the first, so max_v and with it dt change from substep to substep."""
    desc, parts = workloads.ball_scene(n=32, center=(0.5, 0.2, 0.5), radius=0.1, velocity=(1.0, -6.0, 0.0), seed=41)
    ctx = _ctx([(desc, parts)], prec)
    o = oracle_lib.oracle_from_desc(desc, parts, precision=capi.PRECISIONS[prec])
    t_o = 0.0
    for j in (1, 2):
        target = j / 240.0
        kg = ctx.advance_to_time(target, 0.1)
        ko, t_o = o.advance_to_time(t_o, target, 0.1)
        assert kg == ko and kg > 5
        assert ctx.time == target and abs(t_o - target) <= (1e-15 if prec == "fp64" else 1e-6)
    g, r = ctx.particles(0), o.particles()
    dx = 1.0 / desc.counts[0]
    assert np.array_equal(g["valid"], r["valid"])
    assert np.abs(g["X"] - r["X"]).max() <= tol * dx
    assert abs(ctx.max_velocity() - o.max_velocity()) <= tol * max(1.0, o.max_velocity())
