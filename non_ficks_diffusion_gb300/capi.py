"""ctypes binding of the C ABI in include/mpm_gb300.h and include/mpm_scenes.h.

The library is the in-tree build non_ficks_diffusion_gb300/_lib/libmpm_gb300.so; loading
fails loudly if it is missing (there is no CPU fallback). Compute calls need a CUDA GPU.
"""
import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_lib", "libmpm_gb300.so")

MPM_MAX_BARRIERS = 16
MPM_MAX_SCENES = 256
OK, CG_NOT_CONVERGED, NONFINITE, CAPACITY, BAD_ARG, CUDA_ERROR, NOT_READY = range(7)
FP32, MIXED, FP64 = 0, 1, 2
F32, F64 = 0, 1
PRECISIONS = {"fp32": FP32, "mixed": MIXED, "fp64": FP64}


class Config(C.Structure):
    _fields_ = [("precision", C.c_int), ("device", C.c_int), ("use_graphs", C.c_int), ("max_scenes", C.c_int),
                ("max_particles", C.c_longlong), ("max_blocks", C.c_longlong), ("chunk", C.c_int)]


class Barrier(C.Structure):
    _fields_ = [("normal", C.c_double * 3), ("surface", C.c_double * 3), ("mu", C.c_double), ("sticky", C.c_int)]


class SceneDesc(C.Structure):
    _fields_ = [("counts", C.c_int * 3), ("gravity", C.c_double * 3), ("flip", C.c_double),
                ("cg_abs_tol", C.c_double), ("cg_rel_tol", C.c_double), ("cg_max_iters", C.c_int),
                ("cg_min_iters", C.c_int), ("project", C.c_int), ("plastic", C.c_int), ("hardening", C.c_double),
                ("compression_yield", C.c_double), ("stretching_yield", C.c_double), ("hardening_max", C.c_double),
                ("n_barriers", C.c_int), ("barriers", Barrier * MPM_MAX_BARRIERS), ("material", C.c_int),
                ("bulk_modulus", C.c_double), ("eos_gamma", C.c_double)]


MATERIAL_SNOW, MATERIAL_EOS_FLUID = 0, 1


class ParticleArrays(C.Structure):
    _fields_ = [("n", C.c_longlong), ("dtype", C.c_int), ("X", C.c_void_p), ("V", C.c_void_p), ("mass", C.c_void_p),
                ("lambda0", C.c_void_p), ("mu0", C.c_void_p), ("Fe", C.c_void_p), ("Jp", C.c_void_p),
                ("V0", C.c_void_p), ("valid", C.POINTER(C.c_int))]


class Stats(C.Structure):
    _fields_ = [("n_particles", C.c_longlong), ("n_valid", C.c_longlong), ("n_active_blocks", C.c_longlong),
                ("n_interior", C.c_longlong), ("cg_iterations", C.c_int), ("cg_converged", C.c_int),
                ("cg_residual", C.c_double), ("cg_tolerance", C.c_double), ("substeps", C.c_longlong),
                ("gpu_launches", C.c_longlong)]


class LaunchConfig(C.Structure):
    _fields_ = [("chunk", C.c_int), ("ctas_hessian", C.c_int), ("ctas_p2g", C.c_int), ("ctas_g2p", C.c_int),
                ("grid_per_sm", C.c_int), ("node_grid_per_sm", C.c_int), ("hessian_warp_items", C.c_int),
                ("incremental_sort", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class TuneResult(C.Structure):
    _fields_ = [("chosen", LaunchConfig), ("initial", LaunchConfig), ("ms_per_substep", C.c_double),
                ("ms_per_substep_initial", C.c_double), ("trials", C.c_int)]


class PresetInfo(C.Structure):
    _fields_ = [("dim", C.c_int), ("scene_count", C.c_int), ("n_particles", C.c_longlong), ("dt", C.c_double),
                ("frame_dt", C.c_double), ("density", C.c_double)]


# Every entry point of include/mpm_gb300.h and include/mpm_scenes.h: name -> (restype, argtypes)
_vp, _ip, _dp, _lp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_longlong)
SIGNATURES = {
    "mpm_status_string": (C.c_char_p, [C.c_int]),
    "mpm_default_config": (None, [C.POINTER(Config)]),
    "mpm_default_scene": (None, [C.POINTER(SceneDesc)]),
    "mpm_create": (C.c_int, [C.POINTER(Config), C.POINTER(_vp)]),
    "mpm_destroy": (C.c_int, [_vp]),
    "mpm_last_error": (C.c_char_p, [_vp]),
    "mpm_add_scene": (C.c_int, [_vp, C.POINTER(SceneDesc), _ip]),
    "mpm_add_particles": (C.c_int, [_vp, C.c_int, C.POINTER(ParticleArrays)]),
    "mpm_initialize": (C.c_int, [_vp]),
    "mpm_advance_step": (C.c_int, [_vp, C.c_double]),
    "mpm_advance_steps": (C.c_int, [_vp, C.c_int, C.c_double]),
    "mpm_advance_step_partial": (C.c_int, [_vp, C.c_double, C.c_int]),
    "mpm_max_particle_velocity": (C.c_int, [_vp, C.c_int, _dp]),
    "mpm_get_particles": (C.c_int, [_vp, C.c_int, C.POINTER(ParticleArrays)]),
    "mpm_set_particles": (C.c_int, [_vp, C.c_int, C.POINTER(ParticleArrays)]),
    "mpm_get_particles_batch": (C.c_int, [_vp, C.c_int, _ip, C.POINTER(ParticleArrays)]),
    "mpm_set_particles_batch": (C.c_int, [_vp, C.c_int, _ip, C.POINTER(ParticleArrays)]),
    "mpm_allocate_particles": (C.c_int, [_vp, C.c_int, C.POINTER(ParticleArrays), _ip]),
    "mpm_get_stats": (C.c_int, [_vp, C.c_int, C.POINTER(Stats)]),
    "mpm_flag_counts": (C.c_int, [_vp, C.c_int, _lp]),
    "mpm_get_interior_nodes": (C.c_int, [_vp, C.c_int, C.c_longlong, _ip, _dp, _dp, _dp, _lp]),
    "mpm_get_active_blocks": (C.c_int, [_vp, C.c_int, C.c_longlong, _ip, _lp]),
    "mpm_get_sort": (C.c_int, [_vp, C.c_longlong, C.POINTER(C.c_uint32), _ip, _ip, _lp]),
    "mpm_synchronize": (C.c_int, [_vp]),
    "mpm_stream": (_vp, [_vp]),
    "mpm_set_timing": (C.c_int, [_vp, C.c_int]),
    "mpm_get_phase_times": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_char_p), _dp, _lp]),
    "mpm_time_steps": (C.c_int, [_vp, C.c_int, C.c_double, _dp]),
    "mpm_get_time": (C.c_int, [_vp, _dp]),
    "mpm_set_time": (C.c_int, [_vp, C.c_double]),
    "mpm_advance_to_time": (C.c_int, [_vp, C.c_double, C.c_double, C.c_int, _ip]),
    "mpm_get_launch_config": (C.c_int, [_vp, C.POINTER(LaunchConfig)]),
    "mpm_set_launch_config": (C.c_int, [_vp, C.POINTER(LaunchConfig)]),
    "mpm_autotune": (C.c_int, [_vp, C.c_double, C.c_int, C.POINTER(TuneResult)]),
    "mpm_preset_scene": (C.c_int, [C.c_int, C.c_int, C.c_ulonglong, C.POINTER(SceneDesc), C.POINTER(PresetInfo)]),
    "mpm_preset_particles": (C.c_int, [C.c_int, C.c_int, C.c_ulonglong, C.c_longlong, _dp, _dp, _dp, _dp, _dp]),
    "mpm_get_cg_iterations": (C.c_int, [_vp, C.c_int, _ip, _lp, _ip]),
    "mpm_selftest_lookback_wait": (C.c_int, [_vp, C.c_int]),
    "mpm_sort_pairs_noalloc": (C.c_int, [_vp, _vp, _vp, _vp, C.c_longlong, C.c_int, C.c_int, _vp]),
}

_lib = None


def lib():
    """Load the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libmpm_gb300.so is not built (run non_ficks_diffusion_gb300.build.build())")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        _lib = L
    return _lib


class MPMError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (lib().mpm_status_string(status).decode(), msg))
        self.status = status


def _ptr(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def preset(test_number, scene_index=0, seed=0, lib=None):
    """Scene description, info and FP64 particle arrays of a Standard_Tests preset. `lib`:
    another loaded library that exports the scene sampler (default: this package's)."""
    L = lib if lib is not None else globals()["lib"]()
    desc, info = SceneDesc(), PresetInfo()
    st = L.mpm_preset_scene(test_number, scene_index, seed, C.byref(desc), C.byref(info))
    if st != OK:
        raise MPMError(st, "preset %d/%d" % (test_number, scene_index))
    n, d = info.n_particles, info.dim
    X, V = np.zeros((n, d)), np.zeros((n, d))
    m, lam, mu = np.zeros(n), np.zeros(n), np.zeros(n)
    st = L.mpm_preset_particles(test_number, scene_index, seed, n, _ptr(X), _ptr(V), _ptr(m), _ptr(lam), _ptr(mu))
    if st != OK:
        raise MPMError(st, "preset particles")
    return desc, info, dict(X=X, V=V, mass=m, lambda0=lam, mu0=mu)


def default_scene():
    d = SceneDesc()
    globals()["lib"]().mpm_default_scene(C.byref(d))
    return d


def particle_arrays(n, dtype=np.float64, **arrays):
    """ParticleArrays over numpy arrays (kept alive in the returned object's _keep)."""
    pa = ParticleArrays()
    pa.n = n
    pa.dtype = F64 if dtype == np.float64 else F32
    keep = []
    for k in ("X", "V", "mass", "lambda0", "mu0", "Fe", "Jp", "V0"):
        a = arrays.get(k)
        if a is not None:
            assert a.dtype == dtype and a.flags.c_contiguous
            keep.append(a)
            setattr(pa, k, a.ctypes.data)
    if arrays.get("valid") is not None:
        keep.append(arrays["valid"])
        pa.valid = arrays["valid"].ctypes.data_as(C.POINTER(C.c_int))
    pa._keep = keep
    return pa


class Context:
    """One GPU context over the C ABI."""

    def __init__(self, precision="fp32", max_particles=1 << 20, max_scenes=64, use_graphs=True, chunk=0,
                 max_blocks=0, device=0):
        self.L = lib()
        cfg = Config()
        self.L.mpm_default_config(C.byref(cfg))
        cfg.precision = PRECISIONS[precision] if isinstance(precision, str) else precision
        cfg.max_particles, cfg.max_scenes = int(max_particles), int(max_scenes)
        cfg.use_graphs, cfg.chunk, cfg.max_blocks, cfg.device = int(use_graphs), int(chunk), int(max_blocks), int(device)
        h = C.c_void_p()
        st = self.L.mpm_create(C.byref(cfg), C.byref(h))
        if st != OK:
            raise MPMError(st, "mpm_create")
        self.h = h
        self.scene_sizes = []

    def close(self):
        if getattr(self, "h", None):
            self.L.mpm_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, st, what, allow=(OK,)):
        if st not in allow:
            raise MPMError(st, "%s: %s" % (what, self.L.mpm_last_error(self.h).decode()))
        return st

    def add_scene(self, desc):
        sid = C.c_int()
        self._check(self.L.mpm_add_scene(self.h, C.byref(desc), C.byref(sid)), "mpm_add_scene")
        self.scene_sizes.append(0)
        return sid.value

    def add_particles(self, scene, X, V, mass, lambda0, mu0, Fe=None, Jp=None, V0=None, valid=None):
        c = lambda a, w=None: None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape((len(mass),) + w if w else (-1,))
        n = len(mass)
        arrays = dict(X=c(X, (3,)), V=c(V, (3,)), mass=c(mass), lambda0=c(lambda0), mu0=c(mu0),
                      Fe=None if Fe is None else np.ascontiguousarray(Fe, dtype=np.float64).reshape(n, 9),
                      Jp=c(Jp), V0=c(V0),
                      valid=None if valid is None else np.ascontiguousarray(valid, dtype=np.int32))
        pa = particle_arrays(n, np.float64, **arrays)
        self._check(self.L.mpm_add_particles(self.h, scene, C.byref(pa)), "mpm_add_particles")
        self.scene_sizes[scene] += n

    def initialize(self):
        self._check(self.L.mpm_initialize(self.h), "mpm_initialize")

    def allocate_particles(self, scene, X, V, mass, lambda0, mu0):
        """New particles in the slots of the scene's removed particles (Allocate_Particle);
        returns their insertion indices in the scene."""
        c = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        n = len(mass)
        pa = particle_arrays(n, np.float64, X=c(X).reshape(n, 3), V=c(V).reshape(n, 3), mass=c(mass),
                             lambda0=c(lambda0), mu0=c(mu0))
        ids = np.zeros(n, np.int32)
        self._check(self.L.mpm_allocate_particles(self.h, scene, C.byref(pa), _ptr(ids, C.c_int)), "mpm_allocate_particles")
        return ids

    def step(self, dt, k=1):
        return self._check(self.L.mpm_advance_steps(self.h, k, dt), "mpm_advance_steps", (OK, CG_NOT_CONVERGED))

    def step_partial(self, dt, stop_after):
        return self._check(self.L.mpm_advance_step_partial(self.h, dt, stop_after), "partial", (OK, CG_NOT_CONVERGED))

    @property
    def time(self):
        t = C.c_double()
        self._check(self.L.mpm_get_time(self.h, C.byref(t)), "mpm_get_time")
        return t.value

    def set_time(self, t):
        self._check(self.L.mpm_set_time(self.h, t), "mpm_set_time")

    def advance_to_time(self, target, cfl=0.1, max_substeps=1 << 20):
        """The reference's CFL time stepping to `target` on the device; returns the substeps."""
        n = C.c_int()
        self._check(self.L.mpm_advance_to_time(self.h, target, cfl, max_substeps, C.byref(n)), "mpm_advance_to_time",
                    (OK, CG_NOT_CONVERGED))
        return n.value

    def launch_config(self):
        L = LaunchConfig()
        self._check(self.L.mpm_get_launch_config(self.h, C.byref(L)), "mpm_get_launch_config")
        return L.as_dict()

    def set_launch_config(self, **kw):
        L = LaunchConfig(**{**self.launch_config(), **kw})
        self._check(self.L.mpm_set_launch_config(self.h, C.byref(L)), "mpm_set_launch_config")

    def autotune(self, dt, substeps=3):
        """Times candidate launch configurations on this context's scenes and keeps the
        fastest; the particle state is left as it was."""
        r = TuneResult()
        self._check(self.L.mpm_autotune(self.h, dt, substeps, C.byref(r)), "mpm_autotune")
        return {"chosen": r.chosen.as_dict(), "initial": r.initial.as_dict(), "ms_per_substep": r.ms_per_substep,
                "ms_per_substep_initial": r.ms_per_substep_initial, "trials": r.trials}

    def time_steps(self, k, dt):
        ms = C.c_double()
        st = self._check(self.L.mpm_time_steps(self.h, k, dt, C.byref(ms)), "mpm_time_steps", (OK, CG_NOT_CONVERGED))
        return ms.value, st

    def particles(self, scene, dtype=np.float64):
        n = self.scene_sizes[scene]
        out = dict(X=np.zeros((n, 3), dtype), V=np.zeros((n, 3), dtype), Fe=np.zeros((n, 3, 3), dtype),
                   Jp=np.zeros(n, dtype), V0=np.zeros(n, dtype), mass=np.zeros(n, dtype), lambda0=np.zeros(n, dtype),
                   mu0=np.zeros(n, dtype), valid=np.zeros(n, np.int32))
        pa = particle_arrays(n, dtype, **out)
        self._check(self.L.mpm_get_particles(self.h, scene, C.byref(pa)), "mpm_get_particles")
        out["valid"] = out["valid"].astype(bool)
        return out

    def set_particles(self, scene, **arrays):
        n = self.scene_sizes[scene]
        dtype = arrays["X"].dtype
        pa = particle_arrays(n, dtype, **arrays)
        self._check(self.L.mpm_set_particles(self.h, scene, C.byref(pa)), "mpm_set_particles")

    def stats(self, scene=0):
        s = Stats()
        self._check(self.L.mpm_get_stats(self.h, scene, C.byref(s)), "mpm_get_stats")
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def flag_counts(self, scene=0):
        out = np.zeros(3, np.int64)
        self._check(self.L.mpm_flag_counts(self.h, scene, _ptr(out, C.c_longlong)), "mpm_flag_counts")
        return out

    def interior_nodes(self, scene=0):
        n = C.c_longlong()
        self._check(self.L.mpm_get_interior_nodes(self.h, scene, 0, None, None, None, None, C.byref(n)), "interior")
        k = n.value
        coords, m, v, vs = np.zeros((k, 3), np.int32), np.zeros(k), np.zeros((k, 3)), np.zeros((k, 3))
        self._check(self.L.mpm_get_interior_nodes(self.h, scene, k, _ptr(coords, C.c_int), _ptr(m), _ptr(v), _ptr(vs),
                                                  C.byref(n)), "interior")
        return dict(coords=coords, m=m, v=v, vs=vs)

    def active_blocks(self, scene=0):
        n = C.c_longlong()
        self._check(self.L.mpm_get_active_blocks(self.h, scene, 0, None, C.byref(n)), "blocks")
        c = np.zeros((n.value, 3), np.int32)
        self._check(self.L.mpm_get_active_blocks(self.h, scene, n.value, _ptr(c, C.c_int), C.byref(n)), "blocks")
        return c

    def sort_state(self):
        n = C.c_longlong()
        self._check(self.L.mpm_get_sort(self.h, 0, None, None, None, C.byref(n)), "sort")
        k = n.value
        keys, order, scn = np.zeros(k, np.uint32), np.zeros(k, np.int32), np.zeros(k, np.int32)
        self._check(self.L.mpm_get_sort(self.h, k, keys.ctypes.data_as(C.POINTER(C.c_uint32)), _ptr(order, C.c_int),
                                        _ptr(scn, C.c_int), C.byref(n)), "sort")
        return keys, order, scn

    def cg_iterations(self):
        """Per scene: CG iterations and Interior node count of the last substep."""
        ns = C.c_int()
        self._check(self.L.mpm_get_cg_iterations(self.h, 0, None, None, C.byref(ns)), "cg iterations")
        it, nn = np.zeros(ns.value, np.int32), np.zeros(ns.value, np.int64)
        if ns.value:
            self._check(self.L.mpm_get_cg_iterations(self.h, ns.value, _ptr(it, C.c_int), _ptr(nn, C.c_longlong),
                                                     C.byref(ns)), "cg iterations")
        return it, nn

    def max_velocity(self, scene=0):
        v = C.c_double()
        self._check(self.L.mpm_max_particle_velocity(self.h, scene, C.byref(v)), "vmax")
        return v.value

    def set_timing(self, on):
        self._check(self.L.mpm_set_timing(self.h, int(on)), "timing")

    def phase_times(self):
        names = (C.c_char_p * 16)()
        ms, launches = np.zeros(16), np.zeros(16, np.int64)
        k = self.L.mpm_get_phase_times(self.h, 16, names, _ptr(ms), _ptr(launches, C.c_longlong))
        return {names[i].decode(): (ms[i], int(launches[i])) for i in range(k)}

    def stream(self):
        return self.L.mpm_stream(self.h)

    def synchronize(self):
        self._check(self.L.mpm_synchronize(self.h), "sync")
