"""The CPU reference arm of the benchmark: the oracle port (bit-identical to
the reference's solver) timed on every host core as independent replicas of a
bounded solve, printed as one JSON line with the contract's keys.  CPU only."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "cfg1",
                        "--steps", "2", "--warmup", "1", "--ref-seconds", "1", "--ref-threads", "2"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "unknown-iters/s" and d["higher_is_better"]
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 1
    cb = d["cpu_baseline"]
    assert cb["cores"] == 2 and cb["kind"] == "port" and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_host_threads_respects_memory():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.host_threads(1.0) >= 1
    assert bench.host_threads(1e18) == 1
