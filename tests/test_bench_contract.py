"""The benchmark's JSON line keeps the fields its consumers read.  The
reference arm (the oracle on the host cores) runs here without a GPU; the
GPU arm's line is checked on the GPU machine by the benchmark run itself."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REQUIRED = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
            "vs_baseline", "dtype", "data", "config")


def test_reference_arm_line():
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    for k in REQUIRED:
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["n_gpus"] == 1
    assert d["warmup"] >= 3 and d["steps"] == 1
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert isinstance(d["config"], dict) and "workload" in d["config"]


def test_roofline_traffic_figure_is_readable():
    # bench.py scales the committed k_rows capture's DRAM bytes to its launch
    sys.path.insert(0, ROOT)
    import bench
    per_window = bench.read_traffic()
    assert per_window is not None and 5e5 < per_window < 2e6, per_window
