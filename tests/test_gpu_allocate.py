"""New particles in a running scene (mpm_allocate_particles) against the oracle's restatement of
Allocate_Particle (MPM_Example.cpp:959-975): the slot of a removed particle is reused, the
particle is reset (Fe = I, Jp = 1) and gets its first-touch volume from the grid density
before it moves (Process_Waiting_Particles, MPM_Example.cpp:827-840).

- A ball thrown through the +x face loses ~100 particles to the cell-domain check; 50 new
  particles then take the removed slots of lowest insertion index, in the GPU and in the
  oracle alike, and both run on: the same slots, the same removed set, X, V and V0 within
  the precision's bar (FP64 1e-9 dx, FP32 1e-4 dx).
- Reserve slots: particles added with valid = 0 before mpm_initialize hold slots for later
  allocation; particles allocated into them get the same volumes as the same particles
  present from the start.
- Asking for more particles than the scene has removed ones returns MPM_CAPACITY.
"""
import numpy as np
import pytest

import oracle_lib
from non_ficks_diffusion_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

DT = 1e-4


def _new_particles(n=50, seed=7, center=(0.3, 0.5, 0.5)):
    rng = np.random.default_rng(seed)
    X = np.asarray(center) + (rng.random((n, 3)) - 0.5) * 0.06
    E, nu, m = 1.4e5, 0.2, 400.0 / 32 ** 3 / 8
    return dict(X=X, V=np.tile([0.0, -1.0, 0.0], (n, 1)), mass=np.full(n, m),
                lambda0=np.full(n, E * nu / ((1 + nu) * (1 - 2 * nu))), mu0=np.full(n, E / (2 * (1 + nu))))


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-9), ("fp32", 1e-4)])
def test_allocated_particles_reuse_removed_slots_like_the_oracle(built_lib, prec, tol):
    desc, parts = workloads.ball_scene(n=32, center=(0.85, 0.5, 0.5), radius=0.1, velocity=(12.0, 0.0, 0.0), seed=34)
    desc.n_barriers = 1          # nothing stops the ball at the +x face
    ctx = capi.Context(precision=prec, max_particles=len(parts["mass"]), max_scenes=1)
    ctx.add_scene(desc)
    ctx.add_particles(0, parts["X"], parts["V"], parts["mass"], parts["lambda0"], parts["mu0"])
    ctx.initialize()
    o = oracle_lib.oracle_from_desc(desc, parts, precision=capi.PRECISIONS[prec])
    for _ in range(60):
        ctx.step(DT)
        o.step(DT)
    removed = ~o.particles()["valid"]
    assert removed.sum() > 60 and np.array_equal(~ctx.particles(0)["valid"], removed)
    new = _new_particles()
    ids = ctx.allocate_particles(0, new["X"], new["V"], new["mass"], new["lambda0"], new["mu0"])
    ids_o = o.allocate_particles(new["X"], new["V"], new["mass"], new["lambda0"], new["mu0"])
    assert np.array_equal(ids, ids_o)
    assert np.array_equal(np.sort(ids), np.flatnonzero(removed)[:len(ids)])
    g = ctx.particles(0)
    stored = new["X"].astype(np.float32).astype(np.float64) if prec == "fp32" else new["X"]
    assert g["valid"][ids].all() and np.array_equal(g["X"][ids], stored)
    assert np.all(g["V0"][ids] > 0) and np.all(g["Jp"][ids] == 1.0)
    for _ in range(15):
        ctx.step(DT)
        o.step(DT)
    g, r = ctx.particles(0), o.particles()
    dx = 1.0 / desc.counts[0]
    assert np.array_equal(g["valid"], r["valid"])
    assert np.abs(g["X"] - r["X"]).max() <= tol * dx
    assert np.abs(g["V"] - r["V"]).max() <= tol * max(1.0, np.abs(r["V"]).max())
    assert np.allclose(g["V0"][ids], r["V0"][ids], rtol=10 * tol, atol=0)


def test_reserve_slots_take_the_volumes_of_particles_present_from_the_start(built_lib):
    desc, parts = workloads.ball_scene(n=32, radius=0.1, seed=3)
    new = _new_particles(n=64, center=(0.5, 0.3, 0.5))
    n0, n1 = len(parts["mass"]), len(new["mass"])
    both = {k: np.concatenate([parts[k], new[k]]) for k in parts}
    a = capi.Context(precision="fp64", max_particles=n0 + n1, max_scenes=1)
    a.add_scene(desc)
    valid = np.r_[np.ones(n0, np.int32), np.zeros(n1, np.int32)]
    a.add_particles(0, both["X"], both["V"], both["mass"], both["lambda0"], both["mu0"], valid=valid)
    a.initialize()
    assert not a.particles(0)["valid"][n0:].any()
    ids = a.allocate_particles(0, new["X"], new["V"], new["mass"], new["lambda0"], new["mu0"])
    assert np.array_equal(ids, np.arange(n0, n0 + n1))
    b = capi.Context(precision="fp64", max_particles=n0 + n1, max_scenes=1)
    b.add_scene(desc)
    b.add_particles(0, both["X"], both["V"], both["mass"], both["lambda0"], both["mu0"])
    b.initialize()
    pa, pb = a.particles(0), b.particles(0)
    assert pa["valid"].all()
    assert np.allclose(pa["V0"][n0:], pb["V0"][n0:], rtol=1e-12, atol=0)
    with pytest.raises(capi.MPMError) as ei:
        a.allocate_particles(0, new["X"][:1], new["V"][:1], new["mass"][:1], new["lambda0"][:1], new["mu0"][:1])
    assert ei.value.status == capi.CAPACITY
    a.step(DT, 3)
    b.step(DT, 3)
    # the two bodies are far apart, so every volume agrees and the runs continue alike
    assert np.allclose(a.particles(0)["V0"], pb["V0"], rtol=1e-12, atol=0)
    assert np.abs(a.particles(0)["X"] - b.particles(0)["X"]).max() <= 1e-9 / 32
