"""bench.py's CPU-side contract: the reference arm's JSON line and the helpers
the GPU arm uses to fill its roofline, checked without a GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--events", "40",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["unit"] == "events/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["config"]["events"] == 40 and "workload" in d["config"]
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_profiled_traffic_reads_the_committed_capture():
    sys.path.insert(0, ROOT)
    import bench
    traffic, src = bench.profiled_traffic("scale", 10000)
    assert traffic is not None and traffic > 10000 * 34_000          # above the algorithmic bytes
    assert src.startswith("profiles/") and "B/event x 10000 events" in src
    assert bench.profiled_traffic("batched", 10) == (None, None)
