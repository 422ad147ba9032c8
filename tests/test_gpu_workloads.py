"""Parity on the benchmark workloads themselves, through the C ABI against the CPU oracle.

Two colliding snowballs (preset 102: 256^3, 1.94M particles, mixed precision). The spec
reports this workload's error against FP64. The GPU runs FP64 up to just before the balls
meet; from that state the GPU (FP64 and mixed) and the FP64 oracle run 80 more substeps
through the first contact. Bars: mixed within 1e-3 dx of the FP64 oracle (the spec's bar),
FP64 within 1e-8 dx with the same CG iteration count on every substep.

Batch of 64 scenes (preset 104, mixed precision). Five of its scenes run together in one
context and each against its own mixed-precision oracle for 20 substeps: per scene X, V, Fe,
Jp within 1e-4 dx (or relative), the removed set exactly, CG iterations within two on every
substep. (Totals are not compared: for a scene in free fall the FP32 residual is rounding
noise near the relative tolerance, and the GPU's separable stencil sums carry less of it
than the oracle's, so the GPU stops earlier: 0-1 iterations per substep against 1-2.)
"""
import os

import numpy as np
import pytest

import oracle_lib
from non_ficks_diffusion_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

DT = 1e-4
THREADS = os.cpu_count()


def _state_ctx(desc, st, prec):
    """A context holding one scene whose particles start from the state `st` (X, V, Fe, Jp,
    V0, mass, lambda0, mu0)."""
    n = len(st["mass"])
    ctx = capi.Context(precision=prec, max_particles=n, max_scenes=1)
    sid = ctx.add_scene(desc)
    ctx.add_particles(sid, st["X"], st["V"], st["mass"], st["lambda0"], st["mu0"], Fe=st["Fe"].reshape(n, 9),
                      Jp=st["Jp"], V0=st["V0"])
    ctx.initialize()
    return ctx


def test_colliding_snowballs_through_first_contact(built_lib):
    desc, info, parts = capi.preset(102)
    dx = 1.0 / desc.counts[0]
    approach, window = 250, 80
    a = capi.Context(precision="fp64", max_particles=len(parts["mass"]), max_scenes=1)
    a.add_scene(desc)
    a.add_particles(0, parts["X"], parts["V"], parts["mass"], parts["lambda0"], parts["mu0"])
    a.initialize()
    a.step(DT, approach)
    st = a.particles(0)
    assert st["valid"].all()
    gap = st["X"][parts["mu0"] > parts["mu0"].min(), 0].min() - st["X"][parts["mu0"] == parts["mu0"].min(), 0].max()
    assert 0 < gap < 3 * dx, "the balls should be about to meet (gap %g)" % gap

    o = oracle_lib.Oracle(3, 2, oracle_lib.params_from_desc(desc), THREADS)
    o.add_particles(st["X"], st["V"], st["mass"], st["lambda0"], st["mu0"], st["Fe"].reshape(-1, 9), st["Jp"], st["V0"])
    o.initialize()
    m = _state_ctx(desc, st, "mixed")
    it_gpu, it_ora = [], []
    for _ in range(window):
        a.step(DT)
        m.step(DT)
        o.step(DT)
        it_gpu.append(a.stats()["cg_iterations"])
        it_ora.append(o.stats()["cg_iterations"])
    r, g64, gm = o.particles(), a.particles(0), m.particles(0)
    # contact happened: the closest particles of the two balls now overlap in x
    assert (r["Jp"] < 0.999).sum() > 1000, "the contact should clamp particles plastically"
    assert it_gpu == it_ora
    assert np.array_equal(g64["valid"], r["valid"]) and np.array_equal(gm["valid"], r["valid"])
    assert np.abs(g64["X"] - r["X"]).max() <= 1e-8 * dx
    err_mixed = np.abs(gm["X"] - r["X"]).max() / dx
    assert err_mixed <= 1e-3, "mixed precision %.3g dx from the FP64 oracle" % err_mixed


def _smallest_batch_scenes(k):
    sizes = []
    for s in range(64):
        d, i = capi.SceneDesc(), capi.PresetInfo()
        assert capi.lib().mpm_preset_scene(104, s, 0, capi.C.byref(d), capi.C.byref(i)) == capi.OK
        sizes.append(i.n_particles)
    return sorted(np.argsort(sizes)[:k].tolist())


def test_batch_scenes_match_mixed_oracle(built_lib):
    idx = _smallest_batch_scenes(5)
    ctx, scenes = workloads.make_context(104, precision="mixed", scene_indices=idx)
    assert len({d.counts[0] for d, _, _ in scenes}) >= 1
    oracles = [oracle_lib.oracle_from_desc(d, p, precision=1, threads=THREADS) for d, _, p in scenes]
    steps = 20
    for _ in range(steps):
        ctx.step(DT)
        its, _ = ctx.cg_iterations()
        for s, o in enumerate(oracles):
            o.step(DT)
            assert abs(int(its[s]) - o.stats()["cg_iterations"]) <= 2
    for s, ((d, _, p), o) in enumerate(zip(scenes, oracles)):
        g, r = ctx.particles(s), o.particles()
        dx = 1.0 / d.counts[0]
        assert np.array_equal(g["valid"], r["valid"])
        assert np.abs(g["X"] - r["X"]).max() <= 1e-4 * dx, "scene %d" % idx[s]
        assert np.abs(g["V"] - r["V"]).max() <= 1e-4 * max(1.0, np.abs(r["V"]).max())
        assert np.abs(g["Fe"] - r["Fe"]).max() <= 1e-3
        assert np.abs(g["Jp"] - r["Jp"]).max() <= 1e-3
