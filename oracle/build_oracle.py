"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/oracle_capi.cpp into oracle/_build/liboracle.so with g++ and OpenMP,
together with the package's host-only scene sampler (non_ficks_diffusion_gb300/host/
standard_tests.cpp), so that the CPU baseline draws the same scenes without loading the
GPU library. The flags are portable (no -march=native) so the same source builds on x86_64
and on aarch64 and gives the same results on both.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
ROOT = os.path.dirname(HERE)
SOURCES = [os.path.join(HERE, "oracle_capi.cpp"),
           os.path.join(ROOT, "non_ficks_diffusion_gb300", "host", "standard_tests.cpp")]
HEADERS = [os.path.join(HERE, "mpm_oracle.h"), os.path.join(ROOT, "include", "mpm_scenes.h"),
           os.path.join(ROOT, "include", "mpm_gb300.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in SOURCES + HEADERS + [os.path.abspath(__file__)])


def build(force=False, verbose=False):
    """Compile the oracle library if it is missing or older than its sources."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
           "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-o", tmp] + SOURCES
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
