"""The CPU oracle's substep: conservation laws, determinism, the restated CG, barriers and
removal, in 2D and 3D, plus the committed scene fixture."""
import os

import numpy as np
import pytest

import oracle_lib as O
from non_ficks_diffusion_gb300 import capi, workloads

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def ball_params(n=16, barriers=True, gravity=(0, -9.8, 0), d=3, **kw):
    w = 2.0 / n
    bars = []
    if barriers:
        bars = [((0, 1, 0)[:d], (0, w, 0)[:d], 0.0, 1), ((1, 0, 0)[:d], (w, 0, 0)[:d], 0.0, 0),
                ((-1, 0, 0)[:d], (1 - w, 0, 0)[:d], 0.0, 0)]
    return O.scene_params((n,) * d, gravity[:d], barriers=bars, **kw)


def ball_particles(n=16, d=3, r=0.2, c=0.5, v=(1.0, -3.0, 0.5), seed=7, ppc=2, strain=0.0):
    rng = np.random.default_rng(seed)
    dx = 1.0 / n
    g = np.arange(n)
    cells = np.stack(np.meshgrid(*[g] * d, indexing="ij"), -1).reshape(-1, d)
    sub = np.stack(np.meshgrid(*[np.arange(ppc)] * d, indexing="ij"), -1).reshape(-1, d)
    X = ((cells[:, None, :] + (sub[None, :, :] + rng.random((len(cells), len(sub), d))) / ppc) * dx).reshape(-1, d)
    X = X[((X - c) ** 2).sum(1) < r * r]
    N = len(X)
    E, nu = 1.4e5, 0.2
    V = np.tile(np.asarray(v[:d], float), (N, 1))
    V[:, 1] += strain * (X[:, 1] - c)          # a stretching velocity field, so the CG has work
    return dict(X=X, V=V, mass=np.full(N, 400 * dx ** d / ppc ** d),
                lambda0=np.full(N, E * nu / ((1 + nu) * (1 - 2 * nu))), mu0=np.full(N, E / (2 * (1 + nu))))


def make(params, parts, prec=2, d=3, threads=0):
    o = O.Oracle(d, prec, params, threads)
    o.add_particles(parts["X"], parts["V"], parts["mass"], parts["lambda0"], parts["mu0"])
    o.initialize()
    return o


@pytest.mark.parametrize("d", [2, 3])
def test_p2g_conserves_mass_and_momentum(d):
    parts = ball_particles(d=d)
    o = make(ball_params(d=d), parts, d=d)
    o.step(1e-4, stop_after=1)
    g = o.interior()
    assert np.isclose(g["m"].sum(), parts["mass"].sum(), rtol=1e-12)
    p_grid = (g["m"][:, None] * g["v"]).sum(0)
    p_part = (parts["mass"][:, None] * parts["V"]).sum(0)
    assert np.allclose(p_grid, p_part, rtol=1e-12)


@pytest.mark.parametrize("d", [2, 3])
def test_free_fall_momentum(d):
    """Without barriers, internal forces cancel: the total momentum changes by M g t."""
    parts = ball_particles(d=d, v=(0.3, -1.0, 0.2))
    o = make(ball_params(d=d, barriers=False), parts, d=d)
    steps, dt = 10, 1e-4
    for _ in range(steps):
        o.step(dt)
    p = o.particles()
    m = parts["mass"]
    mom = (m[:, None] * p["V"]).sum(0)
    g = np.array([0, -9.8, 0][:d])
    exp = (m[:, None] * parts["V"]).sum(0) + m.sum() * g * steps * dt
    assert np.allclose(mom, exp, rtol=1e-6, atol=1e-12 * m.sum())


def test_deterministic_across_thread_counts():
    parts = ball_particles()
    res = []
    for t in (1, 3, 8):
        o = make(ball_params(), parts, threads=t)
        for _ in range(4):
            o.step(1e-4)
        res.append(o.particles())
    for r in res[1:]:
        assert np.abs(r["X"] - res[0]["X"]).max() < 1e-14
        assert np.abs(r["Fe"] - res[0]["Fe"]).max() < 1e-12


def test_cg_reaches_tolerance_and_precisions_agree():
    parts = ball_particles(n=32, r=0.15, v=(0, -3, 0), strain=40.0)
    out = {}
    for prec in (0, 1, 2):
        o = make(ball_params(n=32, cg_rel_tol=1e-7), parts, prec=prec)
        for _ in range(3):
            o.step(1e-4)
        s = o.stats()
        if prec == 2:
            assert s["converged"] and s["cg_residual"] <= s["cg_tolerance"] and s["cg_iterations"] >= 1
        out[prec] = o.particles()
    dx = 1 / 32
    assert np.abs(out[1]["X"] - out[2]["X"]).max() < 1e-5 * dx
    assert np.abs(out[0]["X"] - out[2]["X"]).max() < 1e-5 * dx


def test_cg_iteration_limit():
    parts = ball_particles(n=32, r=0.15, v=(0, -3, 0), strain=40.0)
    o = make(ball_params(n=32, cg_rel_tol=1e-14, cg_max_iters=2), parts)
    o.step(1e-4)
    s = o.stats()
    assert s["cg_iterations"] == 2 and not s["converged"]


def test_sticky_ground_holds_the_ball():
    n = 16
    parts = ball_particles(n=n, r=0.12, c=0.3, v=(0, -4.0, 0))
    o = make(ball_params(n=n), parts)
    for _ in range(300):
        o.step(1e-4)
    p = o.particles()
    assert p["valid"].all()
    assert p["X"][:, 1].min() > 2.0 / n - 1.0 / n


def test_particles_leaving_the_domain_are_removed():
    parts = ball_particles(n=16, r=0.08, c=0.5)
    X = parts["X"].copy()
    X[0] = [1 - 0.6 / 16, 0.5, 0.5]
    V = parts["V"].copy()
    V[0] = [50.0, 0, 0]
    parts.update(X=X, V=V)
    o = make(ball_params(n=16, barriers=False, gravity=(0, 0, 0), plastic=0), parts)
    o.step(1e-3)
    p = o.particles()
    assert not p["valid"][0] and p["valid"][1:].all()


def test_flag_counts_consistent():
    o = make(ball_params(), ball_particles())
    o.step(1e-4, stop_after=1)
    dirichlet, interior, both = o.flag_counts()
    assert both == interior and interior <= dirichlet and interior == len(o.interior()["m"])


def test_2d_snowball_preset_runs():
    desc, info, parts = capi.preset(100)
    assert info.dim == 2 and 2800 < info.n_particles < 3100
    o = O.oracle_from_desc(desc, parts, precision=0, dim=2)
    for _ in range(20):
        o.step(info.dt)
    p = o.particles()
    assert np.isfinite(p["X"]).all() and p["valid"].all()
    assert o.stats()["converged"]


def test_golden_scene_fixture():
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden
    g = np.load(os.path.join(GOLDEN, "oracle_scene.npz"))
    params, parts = make_golden.ball()
    assert np.array_equal(parts["X"], g["X0"])
    o = make(params, parts, threads=1)
    iters = [o.step(1e-4) for _ in range(5)]
    p = o.particles()
    assert iters == list(g["iters"])
    assert np.abs(p["X"] - g["X"]).max() < 1e-13
    assert np.abs(p["V"] - g["V"]).max() < 1e-10
    assert np.abs(p["Fe"] - g["Fe"]).max() < 1e-12
    assert np.allclose(p["Jp"], g["Jp"], rtol=1e-13) and np.allclose(p["V0"], g["V0"], rtol=1e-13)
    o.step(1e-4, 1)
    nodes = o.interior()
    assert np.array_equal(nodes["coords"], g["coords"])
    assert np.allclose(nodes["m"], g["m"], rtol=1e-13)


def test_eos_fluid_free_fall_momentum_and_density():
    """EOS fluid particles (MPM_Example.cpp:737-745): the pressure force is coef * grad w,
    whose node sum vanishes, so without barriers the momentum changes by M g t; the density
    (kept in the Jp slot) follows rho /= 1 + dt tr(grad v)."""
    parts = ball_particles(v=(0.3, -1.0, 0.2))
    o = make(ball_params(barriers=False, eos=1, bulk_modulus=50.0, eos_gamma=7.0), parts)
    steps, dt = 8, 1e-4
    for _ in range(steps):
        o.step(dt)
    p = o.particles()
    m = parts["mass"]
    exp = (m[:, None] * parts["V"]).sum(0) + m.sum() * np.array([0, -9.8, 0]) * steps * dt
    assert np.allclose((m[:, None] * p["V"]).sum(0), exp, rtol=1e-6, atol=1e-12 * m.sum())
    assert np.all(np.isfinite(p["Jp"])) and not np.allclose(p["Jp"], 1.0)
    assert np.array_equal(p["Fe"], np.tile(np.eye(3), (len(m), 1, 1)))


def test_eos_fluid_preset_19():
    desc, info, parts = capi.preset(19)
    assert desc.material == capi.MATERIAL_EOS_FLUID and desc.bulk_modulus == 1.0 and desc.eos_gamma == 7.0
    assert info.n_particles == 20000 and desc.n_barriers == 5
    o = O.oracle_from_desc(desc, parts, precision=0)
    for _ in range(5):
        o.step(info.dt)
    assert o.stats()["converged"] and np.isfinite(o.particles()["X"]).all()
