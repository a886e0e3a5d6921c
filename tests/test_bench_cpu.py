"""CPU check of bench.py's reference arm: `--impl reference` times the oracle port of the
reference loops on the host cores (no GPU) and prints one JSON line with the contract's
keys, on the same workload, metric and unit as the GPU arm."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# runs the arm as `python bench.py ...` would, then reports whether the process mapped the
# project's CUDA library (the reference arm must not)
_RUN = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3']; "
        "runpy.run_path('bench.py', run_name='__main__'); "
        "print('MAPPED', any('libsinogb300' in ln for ln in open('/proc/self/maps')))")


def test_reference_arm_prints_contract_line():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-c", _RUN], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "MAPPED False" in r.stdout, r.stdout[-500:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["steps"] == 1 and line["warmup"] >= 3
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["config"]["workload"] == "fdk_ctfanflat_512x512x256_from_512x384x720"
    sys.path.insert(0, ROOT)
    import bench
    assert line["config"] == bench._config(1)  # the GPU arm's config object
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
