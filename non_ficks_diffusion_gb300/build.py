"""Builds the in-tree C-ABI library libmpm_gb300.so (sm_103a CUDA kernels + host C++) and
the mpm_3d driver executable, with nvcc and g++ directly (no cmake).

    python -m non_ficks_diffusion_gb300.build [--force]
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
INC = os.path.join(ROOT, "include")
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OUT = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT, "libmpm_gb300.so")
EXE = os.path.join(OUT, "mpm_3d")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["mpm_capi.cu", "mpm_noalloc.cu"]
HOST_SOURCES = ["standard_tests.cpp"]
EXE_SOURCES = ["mpm_3d_main.cpp"]


def _deps():
    out = []
    for d in (CSRC, HOST, INC):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".cpp", ".h")):
                out.append(os.path.join(d, f))
    return out


def _stale(target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(p) > t for p in _deps() + [os.path.abspath(__file__)])


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def build(force=False, verbose=False):
    """Compile the library (and driver) if missing or older than the sources; returns the .so path."""
    if not force and not _stale(LIB) and os.path.exists(EXE):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    jobs = []
    for s in CU_SOURCES:
        o = os.path.join(objdir, s + ".o")
        jobs.append((o, [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                         "-Xcompiler", "-fvisibility=hidden", "-I" + INC, "-I" + CSRC,
                                         "-c", os.path.join(CSRC, s), "-o", o]))
    for s in HOST_SOURCES:
        o = os.path.join(objdir, s + ".o")
        jobs.append((o, ["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-I" + INC,
                         "-c", os.path.join(HOST, s), "-o", o]))
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(lambda j: _run(j[1], verbose), jobs))
    objs = [j[0] for j in jobs]
    tmp = LIB + ".tmp.%d" % os.getpid()
    _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs, verbose)
    os.replace(tmp, LIB)
    exe_src = [os.path.join(HOST, s) for s in EXE_SOURCES if os.path.exists(os.path.join(HOST, s))]
    if exe_src:
        tmpx = EXE + ".tmp.%d" % os.getpid()
        _run(["g++", "-O2", "-std=c++17", "-I" + INC, "-o", tmpx] + exe_src +
             ["-L" + OUT, "-lmpm_gb300", "-Wl,-rpath,$ORIGIN"], verbose)
        os.replace(tmpx, EXE)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
