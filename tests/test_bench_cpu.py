"""The benchmark's CPU arms (no GPU needed): the JSON line of `bench.py --impl reference` for a grid
config and for the batched form, and the served form's `unavailable` line."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench(*args):
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), *args], cwd=REPO, check=True,
                         capture_output=True, text=True, timeout=600).stdout
    lines = [ln for ln in out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out
    return json.loads(lines[0])


def _check_reference_line(d, steps, warmup):
    assert d["impl"] == "reference"
    assert d["unit"] == "tets/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["steps"] == steps and d["warmup"] == warmup and d["ms_per_step"] > 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "tets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_grid_config():
    d = _bench("--impl", "reference", "--config", "ia-small", "--steps", "2", "--warmup", "3")
    _check_reference_line(d, 2, 3)
    assert d["config"]["workload"].startswith("ia-")
    # the whole workload, not a sample of it
    assert "the whole grid (%d tets)" % d["config"]["tets"] in d["config"]["sample"]


def test_reference_arm_batch_all_cores():
    d = _bench("--impl", "reference", "--config", "batch", "--batch-n", "16", "--steps", "1", "--warmup", "3")
    _check_reference_line(d, 1, 3)
    assert d["cpu_baseline"]["cores"] == (os.cpu_count() or 1)
    assert d["config"]["problems"] == 16 and "16 of 16 grids" in d["config"]["sample"]


def test_reference_arm_serve_unavailable():
    d = _bench("--impl", "reference", "--config", "serve")
    assert d["impl"] == "reference" and "unavailable" in d


def test_warmup_floor():
    """Fewer than three warm-up steps are raised to three."""
    d = _bench("--impl", "reference", "--config", "ia-small", "--steps", "1", "--warmup", "1")
    assert d["warmup"] == 3
