"""The reference arm of bench.py (the oracle on the host cores) prints one JSON line with
the fields the bench contract asks for, on the default workload (the 64-scene batch) and
with the same `config` the GPU arm prints; it loads no GPU code and needs no GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = """
import runpy, sys
sys.argv = ["bench.py"] + sys.argv[1:]
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print("LOADED_GPU_LIBRARY=%d" % ("libmpm_gb300" in maps))
"""


def _run(args):
    out = subprocess.run([sys.executable, "-c", PROBE] + args, cwd=ROOT, check=True, capture_output=True, text=True,
                         timeout=900).stdout
    lines = [l for l in out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    return json.loads(lines[0]), out


def test_reference_arm_prints_one_contract_line(built_lib):
    d, out = _run(["--impl", "reference", "--steps", "1", "--warmup", "0"])
    assert "LOADED_GPU_LIBRARY=0" in out
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["value"] > 0 and d["steps"] == 1 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    c = d["config"]
    assert c["preset"] == 104 and c["scenes"] == 64 and c["particles"] == 14758197 and c["precision"] == "mixed"
    assert "scenes 0,8,16,24,32,40,48,56" in d["cpu_baseline"]["sample"]


def test_gpu_and_reference_arms_share_the_config(built_lib):
    sys.path.insert(0, ROOT)
    import bench
    from non_ficks_diffusion_gb300 import workloads
    sl = workloads.scenes(101)
    assert bench.workload_config("c1", "fp32", sl, 1e-4) == bench.workload_config("c1", "fp32",
                                                                                bench.reference_scenes("c1"), 1e-4)


def test_c0_runs_the_2d_configuration_on_the_cpu(built_lib):
    d, out = _run(["--workload", "c0", "--frames", "2"])
    assert "LOADED_GPU_LIBRARY=0" in out
    assert d["impl"] == "reference" and d["config"]["preset"] == 100 and d["config"]["frames"] == 2
    assert d["steps"] == 834 and d["n_gpus"] == 0          # 417 substeps per 1/24 s frame at dt = 1e-4
    assert d["c0"]["valid_particles"] == d["config"]["particles"] == 2959
