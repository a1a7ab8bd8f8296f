"""The reference arm of bench.py (`--impl reference`: the reference's CPU
path, the oracle port, on the host cores) prints one JSON line with the
metric, unit and config of the GPU arm, its own cpu_baseline and an e2e
object without host<->device copies.  Runs on the small 2-D Laplacian, so
it takes about a second on the CPU."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "lap2d_100", "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "converged eigenpairs/s (resid <= 1e-10 ||A||)" and d["unit"] == "eigenpairs/s"
    assert d["higher_is_better"] is True and d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 0
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["workload"] == "lap2d_100" and d["config"]["n"] == 10000
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert cb["value"] == d["value"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_roofline_inputs_from_committed_profiles():
    # the GPU arm's roofline takes the DRAM/algorithmic traffic ratio of the
    # dominant CGS kernel from the committed ncu summaries, and the FP64
    # share of the hybrid projection from its 5 + 3 panel split
    sys.path.insert(0, ROOT)
    import bench
    for k in ("cgs_proj", "cgs_apply"):
        r = bench.read_traffic_ratio(k)
        assert r is not None and 0.8 < r < 1.3, (k, r)
    s = bench.cgs_fp64_share("cgs_proj", 20, 60)
    assert 0.6 < s < 0.65, s
    assert bench.cgs_fp64_share("cgs_proj", 7, 8) == 5 / 8   # one full panel
