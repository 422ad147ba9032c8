"""ctypes binding of the CPU oracle (oracle/liboracle.so) for the tests and the bench's
CPU-baseline leg. The oracle is the checker; nothing in the product imports this file."""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
from oracle import build_oracle  # noqa: E402

MAX_BARRIERS = 16


class Barrier(C.Structure):
    _fields_ = [("normal", C.c_double * 3), ("surface", C.c_double * 3), ("mu", C.c_double), ("sticky", C.c_int)]


class Plasticity(C.Structure):
    _fields_ = [("plastic", C.c_int), ("hardening", C.c_double), ("compression_yield", C.c_double),
                ("stretching_yield", C.c_double), ("hardening_max", C.c_double)]


class SceneParams(C.Structure):
    _fields_ = [("counts", C.c_int * 3), ("gravity", C.c_double * 3), ("flip", C.c_double),
                ("cg_abs_tol", C.c_double), ("cg_rel_tol", C.c_double), ("cg_max_iters", C.c_int),
                ("cg_min_iters", C.c_int), ("project", C.c_int), ("plasticity", Plasticity),
                ("n_barriers", C.c_int), ("barriers", Barrier * MAX_BARRIERS), ("eos", C.c_int),
                ("bulk_modulus", C.c_double), ("eos_gamma", C.c_double)]


class StepStats(C.Structure):
    _fields_ = [("cg_iterations", C.c_int), ("converged", C.c_int), ("cg_residual", C.c_double),
                ("cg_tolerance", C.c_double), ("n_interior", C.c_longlong), ("n_removed", C.c_longlong)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        vp, dp, ip, lp = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_longlong)
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [C.c_int, C.c_int, C.POINTER(SceneParams), C.c_int]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_sizeof_scene_params.restype = C.c_int
        L.oracle_add_particles.argtypes = [vp, C.c_longlong, dp, dp, dp, dp, dp, dp, dp, dp]
        L.oracle_initialize.argtypes = [vp]
        L.oracle_allocate_particles.argtypes = [vp, C.c_longlong, dp, dp, dp, dp, dp, ip]
        L.oracle_advance_step.restype = C.c_int
        L.oracle_advance_step.argtypes = [vp, C.c_double, C.c_int]
        L.oracle_run_substeps.restype = C.c_double
        L.oracle_run_substeps.argtypes = [vp, C.c_int, C.c_double]
        L.oracle_num_particles.restype = C.c_longlong
        L.oracle_num_particles.argtypes = [vp]
        L.oracle_num_simulated.restype = C.c_longlong
        L.oracle_num_simulated.argtypes = [vp]
        L.oracle_get_particles.argtypes = [vp, dp, dp, dp, dp, dp, ip]
        L.oracle_get_cells.argtypes = [vp, ip]
        L.oracle_num_interior.restype = C.c_longlong
        L.oracle_num_interior.argtypes = [vp]
        L.oracle_get_interior.argtypes = [vp, ip, dp, dp, dp, dp]
        L.oracle_flag_counts.argtypes = [vp, lp]
        L.oracle_last_stats.argtypes = [vp, C.POINTER(StepStats)]
        L.oracle_max_particle_velocity.restype = C.c_double
        L.oracle_max_particle_velocity.argtypes = [vp]
        L.oracle_advance_to_time.restype = C.c_int
        L.oracle_advance_to_time.argtypes = [vp, dp, C.c_double, C.c_double, C.c_int]
        # the scene sampler (host-only; the same source as the GPU library's)
        from non_ficks_diffusion_gb300 import capi
        for name in ("mpm_preset_scene", "mpm_preset_particles", "mpm_default_scene"):
            f = getattr(L, name)
            f.restype, f.argtypes = capi.SIGNATURES[name]
        L.oracle_svd.argtypes = [C.c_int, dp, dp, dp, dp]
        fp = C.POINTER(C.c_float)
        L.oracle_svd_f32.argtypes = [fp, fp, fp, fp]
        L.oracle_psi_P.restype = C.c_double
        L.oracle_psi_P.argtypes = [C.c_int, dp, C.c_double, C.c_double, dp]
        L.oracle_dP.argtypes = [C.c_int, dp, C.c_double, C.c_double, dp, dp]
        L.oracle_polar_dR.argtypes = [C.c_int, dp, dp, dp, dp]
        L.oracle_cofactor.argtypes = [C.c_int, dp, dp, dp, dp]
        L.oracle_plasticity.argtypes = [C.c_int, dp, dp, C.c_double, C.c_double, C.POINTER(Plasticity), dp]
        L.oracle_weights.argtypes = [C.c_double, C.c_double, dp, dp]
        L.oracle_weights_f32.argtypes = [C.c_float, C.c_float, fp, fp]
        assert L.oracle_sizeof_scene_params() == C.sizeof(SceneParams)
        _lib = L
    return _lib


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


def scene_params(counts, gravity, flip=0.9, cg_abs_tol=0.0, cg_rel_tol=1e-5, cg_max_iters=50, cg_min_iters=0,
                 project=1, plastic=1, hardening=10.0, compression_yield=1 - 2.5e-2, stretching_yield=1 + 7.5e-3,
                 hardening_max=3.4028234663852886e38, barriers=(), eos=0, bulk_modulus=1e7, eos_gamma=7.0):
    p = SceneParams()
    for a in range(3):
        p.counts[a] = int(counts[a]) if a < len(counts) else 1
        p.gravity[a] = float(gravity[a]) if a < len(gravity) else 0.0
    p.flip, p.cg_abs_tol, p.cg_rel_tol = flip, cg_abs_tol, cg_rel_tol
    p.cg_max_iters, p.cg_min_iters, p.project = cg_max_iters, cg_min_iters, project
    p.plasticity = Plasticity(plastic, hardening, compression_yield, stretching_yield, hardening_max)
    p.eos, p.bulk_modulus, p.eos_gamma = int(eos), float(bulk_modulus), float(eos_gamma)
    p.n_barriers = len(barriers)
    for i, b in enumerate(barriers):
        n, s, mu, sticky = b
        for a in range(3):
            p.barriers[i].normal[a] = n[a] if a < len(n) else 0.0
            p.barriers[i].surface[a] = s[a] if a < len(s) else 0.0
        p.barriers[i].mu, p.barriers[i].sticky = mu, int(sticky)
    return p


class Oracle:
    """One scene simulated by the CPU oracle. precision: 0 fp32, 1 mixed, 2 fp64."""

    def __init__(self, d, precision, params, threads=0):
        self.L = lib()
        self.d = d
        self.params = params
        self.h = self.L.oracle_create(d, precision, C.byref(params), threads)
        assert self.h

    def __del__(self):
        if getattr(self, "h", None):
            self.L.oracle_destroy(self.h)
            self.h = None

    def add_particles(self, X, V, mass, lambda0, mu0, Fe=None, Jp=None, V0=None):
        c = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        X, V, mass, lambda0, mu0, Fe, Jp, V0 = map(c, (X, V, mass, lambda0, mu0, Fe, Jp, V0))
        n = len(mass)
        self.L.oracle_add_particles(self.h, n, _p(X), _p(V), _p(mass), _p(lambda0), _p(mu0), _p(Fe), _p(Jp), _p(V0))

    def initialize(self):
        self.L.oracle_initialize(self.h)

    def allocate_particles(self, X, V, mass, lambda0, mu0):
        """Allocate_Particle for each new particle; returns the indices they took."""
        c = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        X, V, mass, lambda0, mu0 = map(c, (X, V, mass, lambda0, mu0))
        ids = np.zeros(len(mass), dtype=np.int32)
        self.L.oracle_allocate_particles(self.h, len(mass), _p(X), _p(V), _p(mass), _p(lambda0), _p(mu0),
                                         _p(ids, C.c_int))
        return ids

    def step(self, dt, stop_after=0):
        return self.L.oracle_advance_step(self.h, dt, stop_after)

    def run(self, k, dt):
        return self.L.oracle_run_substeps(self.h, k, dt)

    def particles(self):
        n = self.L.oracle_num_particles(self.h)
        d = self.d
        X, V = np.zeros((n, d)), np.zeros((n, d))
        Fe, Jp, V0 = np.zeros((n, d, d)), np.zeros(n), np.zeros(n)
        valid = np.zeros(n, dtype=np.int32)
        self.L.oracle_get_particles(self.h, _p(X), _p(V), _p(Fe), _p(Jp), _p(V0), _p(valid, C.c_int))
        return dict(X=X, V=V, Fe=Fe, Jp=Jp, V0=V0, valid=valid.astype(bool))

    def cells(self):
        n = self.L.oracle_num_particles(self.h)
        c = np.zeros((n, self.d), dtype=np.int32)
        self.L.oracle_get_cells(self.h, _p(c, C.c_int))
        return c

    def interior(self):
        n = self.L.oracle_num_interior(self.h)
        d = self.d
        coords = np.zeros((n, d), dtype=np.int32)
        m, v, vs, f = np.zeros(n), np.zeros((n, d)), np.zeros((n, d)), np.zeros((n, d))
        self.L.oracle_get_interior(self.h, _p(coords, C.c_int), _p(m), _p(v), _p(vs), _p(f))
        return dict(coords=coords, m=m, v=v, vs=vs, f=f)

    def flag_counts(self):
        out = np.zeros(3, dtype=np.int64)
        self.L.oracle_flag_counts(self.h, out.ctypes.data_as(C.POINTER(C.c_longlong)))
        return out

    def stats(self):
        s = StepStats()
        self.L.oracle_last_stats(self.h, C.byref(s))
        return dict(cg_iterations=s.cg_iterations, converged=bool(s.converged), cg_residual=s.cg_residual,
                    cg_tolerance=s.cg_tolerance, n_interior=s.n_interior, n_removed=s.n_removed)

    def max_velocity(self):
        return self.L.oracle_max_particle_velocity(self.h)

    def advance_to_time(self, time, target, cfl=0.1, max_substeps=1 << 20):
        """The reference's CFL substep loop from `time` to `target` (MPM_Driver.cpp:55-80);
        returns (substeps, new time)."""
        t = C.c_double(time)
        k = self.L.oracle_advance_to_time(self.h, C.byref(t), target, cfl, max_substeps)
        return k, t.value


def preset(test_number, scene_index=0, seed=0):
    """A scene preset drawn by the oracle library's copy of the scene sampler (the GPU
    library is not loaded)."""
    from non_ficks_diffusion_gb300 import capi
    return capi.preset(test_number, scene_index, seed, lib=lib())


# ---- math kernels ----
def svd(F):
    F = np.ascontiguousarray(F, dtype=np.float64)
    d = F.shape[0]
    U, s, V = np.zeros((d, d)), np.zeros(d), np.zeros((d, d))
    lib().oracle_svd(d, _p(F), _p(U), _p(s), _p(V))
    return U, s, V


def psi_P(F, lam, mu):
    F = np.ascontiguousarray(F, dtype=np.float64)
    P = np.zeros_like(F)
    psi = lib().oracle_psi_P(F.shape[0], _p(F), lam, mu, _p(P))
    return psi, P


def dP(F, lam, mu, dF):
    F = np.ascontiguousarray(F, dtype=np.float64)
    dF = np.ascontiguousarray(dF, dtype=np.float64)
    out = np.zeros_like(F)
    lib().oracle_dP(F.shape[0], _p(F), lam, mu, _p(dF), _p(out))
    return out


def polar_dR(F, dF):
    F = np.ascontiguousarray(F, dtype=np.float64)
    dF = np.ascontiguousarray(dF, dtype=np.float64)
    R, dR = np.zeros_like(F), np.zeros_like(F)
    lib().oracle_polar_dR(F.shape[0], _p(F), _p(dF), _p(R), _p(dR))
    return R, dR


def cofactor(F, dF):
    F = np.ascontiguousarray(F, dtype=np.float64)
    dF = np.ascontiguousarray(dF, dtype=np.float64)
    Cm, dC = np.zeros_like(F), np.zeros_like(F)
    lib().oracle_cofactor(F.shape[0], _p(F), _p(dF), _p(Cm), _p(dC))
    return Cm, dC


def plasticity(F, Jp, lambda0, mu0, plastic=1, hardening=10.0, cy=0.975, sy=1.0075, hmax=3.4028234663852886e38):
    F = np.array(F, dtype=np.float64)
    jp = np.array([Jp], dtype=np.float64)
    lm = np.zeros(2)
    pp = Plasticity(plastic, hardening, cy, sy, hmax)
    lib().oracle_plasticity(F.shape[0], _p(F), _p(jp), lambda0, mu0, C.byref(pp), _p(lm))
    return F, jp[0], lm[0], lm[1]


def weights(x, one_over_dx):
    w, dw = np.zeros(3), np.zeros(3)
    lib().oracle_weights(x, one_over_dx, _p(w), _p(dw))
    return w, dw


def params_from_desc(desc, dim=3):
    """SceneParams equivalent of a C-ABI mpm_scene_desc (non_ficks_diffusion_gb300.capi.SceneDesc)."""
    bars = []
    for i in range(desc.n_barriers):
        b = desc.barriers[i]
        bars.append((tuple(b.normal[:dim]), tuple(b.surface[:dim]), b.mu, b.sticky))
    return scene_params(tuple(desc.counts[:dim]), tuple(desc.gravity[:dim]), flip=desc.flip, cg_abs_tol=desc.cg_abs_tol,
                        cg_rel_tol=desc.cg_rel_tol, cg_max_iters=desc.cg_max_iters, cg_min_iters=desc.cg_min_iters,
                        project=desc.project, plastic=desc.plastic, hardening=desc.hardening,
                        compression_yield=desc.compression_yield, stretching_yield=desc.stretching_yield,
                        hardening_max=desc.hardening_max, barriers=bars, eos=desc.material == 1,
                        bulk_modulus=desc.bulk_modulus, eos_gamma=desc.eos_gamma)


def oracle_from_desc(desc, parts, precision=2, threads=0, dim=3):
    """An initialised oracle for the scene `desc` with particle dict `parts` (X, V, mass, lambda0, mu0)."""
    o = Oracle(dim, precision, params_from_desc(desc, dim), threads)
    o.add_particles(parts["X"], parts["V"], parts["mass"], parts["lambda0"], parts["mu0"],
                    parts.get("Fe"), parts.get("Jp"), parts.get("V0"))
    o.initialize()
    return o
