"""The C ABI without a GPU: the library loads and exports every entry point declared in
include/*.h, argument checks that run before any CUDA call, the scene presets
(Standard_Tests surface) and the C++ driver executable."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from non_ficks_diffusion_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in ("mpm_gb300.h", "mpm_scenes.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        names += re.findall(r"MPM_API\s+[\w\s\*]+?\b(mpm_\w+)\s*\(", text)
    return names


def test_library_exports_every_declared_symbol(built_lib):
    L = C.CDLL(built_lib)
    names = declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(capi.SIGNATURES), "ctypes binding and headers disagree"


def test_status_strings_and_defaults(built_lib):
    L = capi.lib()
    assert L.mpm_status_string(capi.OK) == b"ok"
    assert L.mpm_status_string(capi.CAPACITY) == b"capacity exceeded"
    d = capi.default_scene()
    # reference constants: MPM_Example.cpp:77-82, Standard_Tests.h:82-85, MPM_Constitutive_Model.h:20
    assert list(d.gravity) == [0.0, -2.0, 0.0] and d.flip == 0.9
    assert d.cg_abs_tol == 1e-7 and d.cg_max_iters == 10000 and d.cg_min_iters == 0
    assert d.compression_yield == 0.95 and d.stretching_yield == 1.01 and d.hardening == 10.0
    cfg = capi.Config()
    L.mpm_default_config(C.byref(cfg))
    assert cfg.precision == capi.FP32 and cfg.use_graphs == 1 and cfg.chunk == 1024


@pytest.mark.parametrize("field,value", [("precision", 7), ("max_scenes", 0), ("max_scenes", 100000),
                                         ("max_particles", 0), ("chunk", 8)])
def test_create_rejects_bad_config_before_touching_the_gpu(built_lib, field, value):
    L = capi.lib()
    cfg = capi.Config()
    L.mpm_default_config(C.byref(cfg))
    setattr(cfg, field, value)
    h = C.c_void_p()
    assert L.mpm_create(C.byref(cfg), C.byref(h)) == capi.BAD_ARG
    assert not h.value


def test_null_arguments(built_lib):
    L = capi.lib()
    assert L.mpm_create(None, None) == capi.BAD_ARG
    assert L.mpm_advance_step(None, 1e-4) == capi.BAD_ARG
    assert L.mpm_get_stats(None, 0, None) == capi.BAD_ARG
    assert L.mpm_destroy(None) == capi.OK


def test_presets_are_deterministic_and_sized(built_lib):
    expect = {100: (2, 2959), 101: (3, 237144), 102: (3, 1943114)}
    for t, (dim, n) in expect.items():
        d1, i1, p1 = capi.preset(t, 0, 0)
        d2, i2, p2 = capi.preset(t, 0, 0)
        assert i1.dim == dim and i1.n_particles == n
        assert np.array_equal(p1["X"], p2["X"])
        assert (p1["X"] >= 0).all() and (p1["X"] <= 1).all()
        assert i1.dt == 1e-4 and list(d1.gravity[:2]) == [0.0, -9.8]
        assert d1.cg_rel_tol == 1e-5 and d1.cg_max_iters == 50 and d1.cg_abs_tol == 0.0
        assert np.isclose(d1.compression_yield, 0.975) and np.isclose(d1.stretching_yield, 1.0075)
        ground = d1.barriers[0]
        assert ground.sticky == 1 and np.isclose(ground.surface[1], 2.0 / d1.counts[0])
    _, _, p3 = capi.preset(100, 0, 1)
    assert not np.array_equal(p3["X"], capi.preset(100, 0, 0)[2]["X"])   # the seed matters
    # C2: the second sphere is 1.5x stiffer
    _, _, p = capi.preset(102)
    assert np.isclose(p["mu0"].max() / p["mu0"].min(), 1.5)


def test_batch_preset_distribution(built_lib):
    L = capi.lib()
    total, counts = 0, []
    for s in range(64):
        d, i = capi.SceneDesc(), capi.PresetInfo()
        assert L.mpm_preset_scene(104, s, 0, C.byref(d), C.byref(i)) == capi.OK
        assert i.scene_count == 64 and d.counts[0] in (64, 128, 256)
        assert 5 <= d.hardening <= 10
        counts.append(i.n_particles)
        total += i.n_particles
    assert 12e6 < total < 18e6 and min(counts) >= 1e4 * 0.9 and max(counts) <= 1.1e6
    d, i = capi.SceneDesc(), capi.PresetInfo()
    assert L.mpm_preset_scene(104, 64, 0, C.byref(d), C.byref(i)) == capi.BAD_ARG
    assert L.mpm_preset_scene(999, 0, 0, C.byref(d), C.byref(i)) == capi.BAD_ARG


def test_slab_preset_has_inclined_plane(built_lib):
    d, i = capi.SceneDesc(), capi.PresetInfo()
    assert capi.lib().mpm_preset_scene(103, 0, 0, C.byref(d), C.byref(i)) == capi.OK
    assert 21e6 < i.n_particles < 22e6 and d.counts[0] == 512
    plane = d.barriers[d.n_barriers - 1]
    assert np.isclose(plane.normal[0], -0.5) and np.isclose(plane.normal[1], np.sqrt(3) / 2) and plane.mu == 0


def test_driver_executable_parses_options(built_lib):
    exe = os.path.join(os.path.dirname(built_lib), "mpm_3d")
    r = subprocess.run([exe, "-bogus"], capture_output=True, text=True)
    assert r.returncode == 2 and "unknown option" in r.stderr


def test_oracle_library_draws_the_same_scenes(built_lib):
    """The CPU baseline draws its scenes from the oracle library's copy of the host-only
    sampler (so that process loads no GPU code); both copies give the same scenes."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    for t, idx in ((100, 0), (101, 0), (104, 3), (104, 17)):
        d1, i1, p1 = capi.preset(t, idx, 0)
        d2, i2, p2 = oracle_lib.preset(t, idx, 0)
        assert bytes(d1) == bytes(d2) and i1.n_particles == i2.n_particles
        for k in p1:
            assert np.array_equal(p1[k], p2[k]), k
