"""Host-side checks of the per-particle routines the sm_103a kernels share (mpm_math.cuh),
built by nvcc as host code and run on the CPU: the plasticity update, stress, stress
differential and weights against the oracle; the mixed-precision polar refinement against
an FP64 pass; the FP64 SVD warm-started from the FP32 one; the FP32 SVD; the near-diagonal
Jacobi rotation series against the closed form; the whole mixed update against FP64."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "non_ficks_diffusion_gb300", "csrc")
ORACLE = os.path.join(ROOT, "oracle")


def _run_host_check(tmp_path_factory, source, includes):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path_factory.mktemp("math") / os.path.splitext(source)[0])
    subprocess.run([nvcc, "-O2", "-std=c++17"] + ["-I" + d for d in includes] +
                   ["-x", "cu", os.path.join(HERE, "host", source), "-o", exe], check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    return {k: float(v) for k, v in zip(out[::2], out[1::2])}


@pytest.fixture(scope="module")
def math_check(tmp_path_factory):
    return _run_host_check(tmp_path_factory, "math_check.cu", [CSRC])


@pytest.fixture(scope="module")
def device_vs_oracle(tmp_path_factory):
    return _run_host_check(tmp_path_factory, "device_vs_oracle.cu", [CSRC, ORACLE])


def test_device_math_matches_the_oracle(device_vs_oracle):
    """The kernels' plasticity update, stress, stress differential and B-spline weights,
    built as host code, against the oracle's restatement of the reference on 20,000 random
    deformation gradients (75 % of them clamped)."""
    assert device_vs_oracle["fp64_update"] < 1e-12
    assert device_vs_oracle["fp64_P"] < 1e-14
    assert device_vs_oracle["fp64_dP"] < 1e-12
    assert device_vs_oracle["weights"] == 0.0
    assert device_vs_oracle["mixed_update_spacings"] <= 4


def test_mixed_polar_refinement_matches_fp64_pass(math_check):
    # the FP32 result equals one FP64 pass from the same FP32 rotation, rounded to FP32
    assert math_check["polar_mixed_ulp"] <= 1.0
    # orthonormal to the FP32 rounding of the rotation it starts from
    assert math_check["polar_orth"] < 2e-6


def test_mixed_determinant_matches_fp64_rounding(math_check):
    """det Fe of the mixed variant, evaluated in FP32 with error-free transformations,
    equals the FP64 determinant of the same FP32 matrix rounded to FP32 on 200,000 cases
    (near-rotations inside the yield band and general matrices)."""
    assert math_check["det_mismatch"] == 0


def test_fp64_svd_from_fp32_warm_start(math_check):
    assert math_check["svd_recon"] < 1e-14
    assert math_check["svd_orth"] < 1e-14


def test_fp32_svd_cold_start(math_check):
    # the first stage of every precision: a few FP32 spacings of reconstruction error
    assert math_check["svd32_recon"] < 2e-6
    assert math_check["svd32_orth"] < 2e-6


def test_near_diagonal_rotation_series(math_check):
    assert math_check["rot_small"] < 1e-15


def test_mixed_plasticity_update_against_fp64(math_check):
    """Mixed (FP32 state, FP64 SVD/polar) against FP64 on the same FP32 inputs, most of
    them clamped: within a few FP32 spacings. The mixed rotation keeps the FP32
    orthonormality of the rotation it refines, so a few percent of entries differ by more
    than one spacing."""
    assert math_check["upd_clamped"] > 0.5
    assert math_check["upd_ulp"] <= 4
    assert math_check["upd_frac_gt1"] < 0.06
