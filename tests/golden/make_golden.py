"""Generates tests/golden/*.npz: known-answer vectors for the CPU oracle.

The reference ships no tests or golden data and cannot be built here (it needs the
un-vendored Nova library), so these fixtures are produced by the oracle itself, after the
oracle passed the finite-difference and identity checks of tests/test_oracle_math.py. They
pin the oracle against later changes:
  oracle_math.npz   SVD, Psi, P, dP/dF:dF, dR and the cofactor derivative at fixed matrices;
                    B-spline weights on a grid of x; the plasticity step at fixed inputs.
  oracle_scene.npz  a 16^3 ball (FP64 oracle) after 5 substeps: positions, velocities, Fe, Jp,
                    V0, CG iterations, and the Interior node set after the grid build.
Run: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle_lib as O  # noqa: E402


def matrices():
    rng = np.random.default_rng(20261203)
    F3 = [np.eye(3), np.diag([1.01, 0.99, 1.002]), np.eye(3) + 0.05 * rng.standard_normal((3, 3)),
          np.eye(3) + 0.3 * rng.standard_normal((3, 3)), np.array([[0.9, 0.2, 0.0], [-0.1, 1.1, 0.05], [0.0, 0.1, 0.95]])]
    F2 = [np.eye(2), np.diag([1.02, 0.97]), np.eye(2) + 0.1 * rng.standard_normal((2, 2))]
    dF3 = rng.standard_normal((len(F3), 3, 3))
    dF2 = rng.standard_normal((len(F2), 2, 2))
    return F3, F2, dF3, dF2


def make_math(path):
    F3, F2, dF3, dF2 = matrices()
    out = {}
    for d, Fs, dFs in ((3, F3, dF3), (2, F2, dF2)):
        for k, (F, dF) in enumerate(zip(Fs, dFs)):
            U, s, V = O.svd(F)
            psi, P = O.psi_P(F, 3.0e4, 2.0e4)
            out["F%d_%d" % (d, k)] = F
            out["dF%d_%d" % (d, k)] = dF
            out["s%d_%d" % (d, k)] = s
            out["usvt%d_%d" % (d, k)] = U @ np.diag(s) @ V.T
            out["psi%d_%d" % (d, k)] = np.array(psi)
            out["P%d_%d" % (d, k)] = P
            out["dP%d_%d" % (d, k)] = O.dP(F, 3.0e4, 2.0e4, dF)
            out["dR%d_%d" % (d, k)] = O.polar_dR(F, dF)[1]
            out["dC%d_%d" % (d, k)] = O.cofactor(F, dF)[1]
    xs = np.linspace(0.5, 1.5, 41)[:-1]
    out["wx"] = xs
    out["w"] = np.array([O.weights(x, 64.0)[0] for x in xs])
    out["dw"] = np.array([O.weights(x, 64.0)[1] for x in xs])
    Fp = np.array([[1.02, 0.01, 0.0], [0.0, 0.96, 0.02], [0.01, 0.0, 1.0]])
    Fn, jp, lam, mu = O.plasticity(Fp, 0.99, 3.0e4, 2.0e4)
    out["plastic_F_in"], out["plastic_F_out"] = Fp, Fn
    out["plastic_out"] = np.array([jp, lam, mu])
    np.savez(path, **out)


def ball(n=16):
    rng = np.random.default_rng(7)
    dx = 1.0 / n
    c, r = np.array([0.5, 0.5, 0.5]), 0.2
    g = np.arange(n)
    cells = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    sub = np.stack(np.meshgrid(*[np.arange(2)] * 3, indexing="ij"), -1).reshape(-1, 3)
    X = ((cells[:, None, :] + (sub[None, :, :] + rng.random((len(cells), 8, 3))) / 2) * dx).reshape(-1, 3)
    X = X[((X - c) ** 2).sum(1) < r * r]
    N = len(X)
    E, nu = 1.4e5, 0.2
    mu0, lam0 = E / (2 * (1 + nu)), E * nu / ((1 + nu) * (1 - 2 * nu))
    parts = dict(X=X, V=np.tile([1.0, -3.0, 0.5], (N, 1)), mass=np.full(N, 400 * dx ** 3 / 8),
                 lambda0=np.full(N, lam0), mu0=np.full(N, mu0))
    w = 2 * dx
    bars = [((0, 1, 0), (0, w, 0), 0.0, 1), ((1, 0, 0), (w, 0, 0), 0.0, 0), ((-1, 0, 0), (1 - w, 0, 0), 0.0, 0),
            ((0, -1, 0), (0, 1 - w, 0), 0.0, 0), ((0, 0, 1), (0, 0, w), 0.0, 0), ((0, 0, -1), (0, 0, 1 - w), 0.3, 0)]
    params = O.scene_params((n, n, n), (0, -9.8, 0), barriers=bars)
    return params, parts


def make_scene(path):
    params, parts = ball()
    o = O.Oracle(3, 2, params, threads=1)
    o.add_particles(parts["X"], parts["V"], parts["mass"], parts["lambda0"], parts["mu0"])
    o.initialize()
    iters = [o.step(1e-4) for _ in range(5)]
    p = o.particles()
    o.step(1e-4, 1)
    nodes = o.interior()
    np.savez(path, X0=parts["X"], V0_in=parts["V"], X=p["X"], V=p["V"], Fe=p["Fe"], Jp=p["Jp"], V0=p["V0"],
             valid=p["valid"], iters=np.array(iters), coords=nodes["coords"], m=nodes["m"])


if __name__ == "__main__":
    make_math(os.path.join(HERE, "oracle_math.npz"))
    make_scene(os.path.join(HERE, "oracle_scene.npz"))
    print("wrote", os.listdir(HERE))
