"""One full frame (1/24 s at dt = 1e-4: 417 substeps) of the 3D snowball on 128^3 (preset
101, 237k particles): the GPU's FP32, mixed and FP64 paths against the FP64 oracle.

Bar: particle positions within 1e-3 dx of the FP64 oracle for FP32 and mixed, 1e-9 dx for
FP64, and the same removed set. The ball is in free fall for the whole frame, so the FP64
CG needs no iteration; the FP32 paths iterate on rounding noise at low-mass nodes and
still stay far inside the bar.
"""
import numpy as np
import pytest

import oracle_lib
from non_ficks_diffusion_gb300 import workloads

pytestmark = pytest.mark.gpu

STEPS = 417
BAR = {"fp32": 1e-3, "mixed": 1e-3, "fp64": 1e-9}


@pytest.fixture(scope="module")
def fp64_frame():
    desc, info, p = workloads.scenes(101)[0]
    o = oracle_lib.oracle_from_desc(desc, p, precision=2)
    for _ in range(STEPS):
        o.step(info.dt)
    return desc, info, o.particles()


@pytest.mark.parametrize("prec", ["fp32", "mixed", "fp64"])
def test_one_frame_against_fp64_oracle(built_lib, fp64_frame, prec):
    desc, info, ref = fp64_frame
    ctx, _ = workloads.make_context(101, precision=prec)
    ctx.step(info.dt, STEPS)
    g = ctx.particles(0)
    dx = 1.0 / desc.counts[0]
    assert np.array_equal(g["valid"], ref["valid"])
    assert np.abs(g["X"] - ref["X"]).max() <= BAR[prec] * dx
