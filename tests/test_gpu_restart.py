"""Frame output and restart through the host driver (mpm_3d, MPM_Driver.cpp:18-32 and
MPM_Example.cpp:1049-1079): the full-state checkpoint continues a run exactly, and the
reference's own particle record (X, V, mass, volume) restarts it the reference's lossy way."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from non_ficks_diffusion_gb300 import build

pytestmark = pytest.mark.gpu


def _read_record(path):
    """Read_Write_MPM_Particles.h:33-46: size_t count, then X, V (3 floats), mass, volume."""
    with open(path, "rb") as f:
        n = int(np.frombuffer(f.read(8), np.uint64)[0])
        rec = np.frombuffer(f.read(n * 32), np.float32).reshape(n, 8)
    return rec


def _run(out, *args):
    r = subprocess.run([build.EXE, "-test_number", "19", "-precision", "fp64", "-o", out, *args],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr


def test_checkpoint_restart_continues_the_run(built_lib, tmp_path):
    out = str(tmp_path / "run")
    _run(out, "-last_frame", "2")
    full = _read_record(os.path.join(out, "2", "particles"))
    assert os.path.exists(os.path.join(out, "1", "checkpoint")) and len(full) == 20000
    shutil.rmtree(os.path.join(out, "2"))
    _run(out, "-last_frame", "2", "-restart", "1")
    again = _read_record(os.path.join(out, "2", "particles"))
    assert again.shape == full.shape
    # FP64 both ways; the record is FP32, and only the order of float atomics differs
    assert np.abs(again[:, :6] - full[:, :6]).max() <= 1e-5
    assert np.array_equal(again[:, 6], full[:, 6])


def test_reference_record_restart(built_lib, tmp_path):
    out = str(tmp_path / "run")
    _run(out, "-last_frame", "1")
    os.remove(os.path.join(out, "1", "checkpoint"))
    _run(out, "-last_frame", "2", "-restart", "1")
    rec = _read_record(os.path.join(out, "2", "particles"))
    assert len(rec) == 20000 and np.isfinite(rec).all()
