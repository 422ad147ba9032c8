"""The CPU oracle's per-particle math, pinned by identities and finite differences.

The reference ships no tests or golden vectors and cannot be built (Nova is not vendored),
so the oracle is pinned by the mathematics it restates: P = dPsi/dF
(MPM_Constitutive_Model.cpp:55-67), Times_dP_dF = dP (:71-76), dR and the cofactor
derivative (MPM_Constitutive_Model.h:28-69), the SVD convention of
Fast_Singular_Value_Decomposition, the quadratic B-spline (MPM_Particle.h:79-100) against
the reference's own N2/dN2 (MPM_Example.h:23-60), and the snow plasticity step. The
committed fixtures (tests/golden/make_golden.py) then freeze these results.
"""
import os

import numpy as np
import pytest

import oracle_lib as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
rng = np.random.default_rng(12345)


def random_F(d, scale):
    return np.eye(d) + scale * rng.standard_normal((d, d))


@pytest.mark.parametrize("d", [2, 3])
def test_svd_convention(d):
    cases = [random_F(d, s) for s in (0.01, 0.1, 0.5) for _ in range(10)]
    cases += [np.eye(d), np.diag(np.arange(1, d + 1) * 0.3), -np.eye(d), np.diag([1.0] * (d - 1) + [-0.5])]
    th = 0.7
    Rz = np.eye(d)
    Rz[:2, :2] = [[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]]
    cases.append(Rz)
    cases.append(Rz @ np.diag([1.0] * d) * 1.1)
    for F in cases:
        U, s, V = O.svd(F)
        assert np.allclose(U @ np.diag(s) @ V.T, F, atol=1e-12)
        assert np.allclose(U.T @ U, np.eye(d), atol=1e-12) and np.allclose(V.T @ V, np.eye(d), atol=1e-12)
        assert np.isclose(np.linalg.det(U), 1.0) and np.isclose(np.linalg.det(V), 1.0)
        assert np.all(s[:-1] >= 0) and np.all(np.diff(np.abs(s)) <= 1e-12) and s[0] >= s[1]
        assert np.sign(s[-1]) == np.sign(np.linalg.det(F)) or abs(s[-1]) < 1e-12
        assert np.allclose(np.sort(np.abs(s)), np.sort(np.linalg.svd(F)[1]), atol=1e-12)


def test_svd_float32_accuracy():
    import ctypes as C
    L = O.lib()
    for _ in range(50):
        F = random_F(3, 0.05).astype(np.float32)
        U, s, V = (np.zeros((3, 3), np.float32), np.zeros(3, np.float32), np.zeros((3, 3), np.float32))
        fp = C.POINTER(C.c_float)
        L.oracle_svd_f32(F.ctypes.data_as(fp), U.ctypes.data_as(fp), s.ctypes.data_as(fp), V.ctypes.data_as(fp))
        assert np.abs(U.astype(np.float64) @ np.diag(s) @ V.T - F).max() < 2e-6


def fd(f, F, h=1e-6):
    d = F.shape[0]
    G = np.zeros_like(F)
    for i in range(d):
        for j in range(d):
            E = np.zeros_like(F)
            E[i, j] = h
            G[i, j] = (f(F + E) - f(F - E)) / (2 * h)
    return G


@pytest.mark.parametrize("d", [2, 3])
def test_P_is_gradient_of_psi(d):
    for s in (0.02, 0.2):
        F = random_F(d, s)
        lam, mu = 3.0, 2.0
        _, P = O.psi_P(F, lam, mu)
        assert np.allclose(P, fd(lambda G: O.psi_P(G, lam, mu)[0], F), atol=1e-7)


@pytest.mark.parametrize("d", [2, 3])
def test_dP_is_derivative_of_P(d):
    for s in (0.02, 0.2):
        F = random_F(d, s)
        dF = rng.standard_normal((d, d))
        h = 1e-6
        num = (O.psi_P(F + h * dF, 3.0, 2.0)[1] - O.psi_P(F - h * dF, 3.0, 2.0)[1]) / (2 * h)
        assert np.allclose(O.dP(F, 3.0, 2.0, dF), num, atol=1e-7)


@pytest.mark.parametrize("d", [2, 3])
def test_dR_is_derivative_of_polar_rotation(d):
    for s in (0.02, 0.3):
        F = random_F(d, s)
        dF = rng.standard_normal((d, d))
        R, dR = O.polar_dR(F, dF)
        h = 1e-6
        num = (O.polar_dR(F + h * dF, dF)[0] - O.polar_dR(F - h * dF, dF)[0]) / (2 * h)
        assert np.allclose(dR, num, atol=1e-7)
        assert np.allclose(R.T @ R, np.eye(d), atol=1e-12)
        S = R.T @ F
        assert np.allclose(S, S.T, atol=1e-12)


@pytest.mark.parametrize("d", [2, 3])
def test_cofactor_and_derivative(d):
    F = random_F(d, 0.2)
    dF = rng.standard_normal((d, d))
    Cm, dC = O.cofactor(F, dF)
    assert np.allclose(Cm, np.linalg.det(F) * np.linalg.inv(F).T, atol=1e-12)
    h = 1e-6
    num = (O.cofactor(F + h * dF, dF)[0] - O.cofactor(F - h * dF, dF)[0]) / (2 * h)
    assert np.allclose(dC, num, atol=1e-8)


def n2(x):
    """N2 of the reference (MPM_Example.h:23-29), the unused quadratic B-spline evaluator."""
    ax = abs(x)
    return 0.75 - x * x if ax < 0.5 else (0.5 * (1.5 - ax) ** 2 if ax < 1.5 else 0.0)


def dn2(x):
    """dN2 of the reference (MPM_Example.h:37-44)."""
    sign = 1.0 if x >= 0 else -1.0
    ax = abs(x)
    return -2 * x if ax < 0.5 else (x - 1.5 * sign if ax < 1.5 else 0.0)


def test_bspline_weights():
    inv_dx = 64.0
    for x in np.linspace(0.5, 1.5, 101)[:-1]:
        w, dw = O.weights(x, inv_dx)
        assert abs(w.sum() - 1.0) < 1e-14 and abs(dw.sum()) < 1e-10
        # linear reproduction: sum_i w_i (i - x) = 0 with nodes at 0, 1, 2 relative to c-1
        assert abs((w * (np.arange(3) - x)).sum()) < 1e-14
        # node k sits at distance x-k from the particle (in cells)
        for k in range(3):
            assert abs(w[k] - n2(x - k)) < 1e-14
            assert abs(dw[k] - inv_dx * dn2(x - k)) < 1e-9   # gradient with respect to the particle position


def test_plasticity_step():
    pp = dict(hardening=10.0, cy=0.975, sy=1.0075)
    F = np.diag([1.02, 0.96, 1.0]) @ np.array([[1, 0.01, 0], [0, 1, 0.02], [0.01, 0, 1]])
    Jp = 0.99
    Fn, jp, lam, mu = O.plasticity(F, Jp, 3e4, 2e4, **pp)
    U, s, V = O.svd(F)
    sh = np.clip(s, pp["cy"], pp["sy"])
    assert np.allclose(Fn, U @ np.diag(sh) @ V.T, atol=1e-12)
    # the reference's Fp <- V S_hat^-1 U^T Fe Fp, of which only det() is used
    Fp0 = np.diag([Jp, 1.0, 1.0])
    Fp = V @ np.diag(1 / sh) @ U.T @ F @ Fp0
    assert np.isclose(jp, np.linalg.det(Fp), rtol=1e-12)
    e = np.exp(pp["hardening"] * (1 - jp))
    assert np.isclose(lam, 3e4 * e) and np.isclose(mu, 2e4 * e)
    # no clamp inside the band: Fe unchanged, Jp unchanged
    G = np.eye(3) + 1e-3 * np.array([[0, 1, 0], [-1, 0, 0], [0, 0, 1]])
    Gn, jp2, _, _ = O.plasticity(G, 0.97, 3e4, 2e4, **pp)
    assert np.allclose(Gn, G, atol=1e-14) and jp2 == 0.97
    # elastic particles keep the Lame parameters
    _, _, l3, m3 = O.plasticity(F, 0.5, 3e4, 2e4, plastic=0)
    assert l3 == 3e4 and m3 == 2e4


def test_golden_math_fixture():
    g = np.load(os.path.join(GOLDEN, "oracle_math.npz"))
    for d, count in ((3, 5), (2, 3)):
        for k in range(count):
            F, dF = g["F%d_%d" % (d, k)], g["dF%d_%d" % (d, k)]
            U, s, V = O.svd(F)
            assert np.allclose(s, g["s%d_%d" % (d, k)], rtol=0, atol=1e-13)
            psi, P = O.psi_P(F, 3.0e4, 2.0e4)
            assert np.allclose(psi, g["psi%d_%d" % (d, k)], rtol=1e-12, atol=1e-9)
            assert np.allclose(P, g["P%d_%d" % (d, k)], rtol=1e-12, atol=1e-8)
            assert np.allclose(O.dP(F, 3.0e4, 2.0e4, dF), g["dP%d_%d" % (d, k)], rtol=1e-11, atol=1e-7)
            assert np.allclose(O.polar_dR(F, dF)[1], g["dR%d_%d" % (d, k)], atol=1e-12)
            assert np.allclose(O.cofactor(F, dF)[1], g["dC%d_%d" % (d, k)], atol=1e-13)
    for x, w, dw in zip(g["wx"], g["w"], g["dw"]):
        a, b = O.weights(x, 64.0)
        assert np.array_equal(a, w) and np.array_equal(b, dw)
    Fn, jp, lam, mu = O.plasticity(g["plastic_F_in"], 0.99, 3.0e4, 2.0e4)
    assert np.allclose(Fn, g["plastic_F_out"], atol=1e-14)
    assert np.allclose([jp, lam, mu], g["plastic_out"], rtol=1e-13)
