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
    assert "CGSolve (" in cb["sample"] and "host_cores" in cb and "cpu_model" in cb
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_host_threads_respects_memory():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.host_threads(1.0) >= 1
    assert bench.host_threads(1e18) == 1


def test_parity_job_compares_with_the_oracle():
    """The default line's parity leg: a spawned process rebuilds the workload
    from its seeds, runs the oracle's full FP64 solves and compares them with
    the solutions saved by the parent (here the oracle's own, so 0 error)."""
    sys.path.insert(0, ROOT)
    import argparse
    import numpy as np
    import bench
    from oracle.oracle import Oracle
    params = {"workload": "cfg2", "points": 1500, "qprecond": 1}
    g, qp, hp, props, _ = bench.make_workload(argparse.Namespace(**params))
    o = Oracle("port")
    q, _ = o.cgsolveq(qp, props)
    h, _ = o.cgsolve(hp, props)
    jobs = bench.ParityJobs()
    try:
        np.savez(os.path.join(jobs.dir, "gpu_cfg2.npz"), q=q, h=h)
        jobs.start("cfg2", params)
        res = jobs.results(timeout_s=300)
    finally:
        jobs.close()
    r = res["cfg2"]
    assert "error" not in r, r
    assert r["q"]["rel_l2"] == 0.0 and r["h"]["rel_l2"] == 0.0
    assert r["q"]["iters_oracle"] > 2 and r["h"]["iters_oracle"] > 2


def test_roofline_traffic_names_the_kernel_of_the_form():
    """The mixed lines name the batched kernel of the form the autotuner
    picked (the one-pass form has a kernel of its own, qprecond 0/1 only) and
    scale that kernel's measured bytes per unknown-iteration."""
    sys.path.insert(0, ROOT)
    import bench
    assert bench.batch_kernel_name(1, 2) == "batch_kernel<1, 1>"
    assert bench.batch_kernel_name(1, 1) == "batch_kernel<1, 0>"
    assert bench.batch_kernel_name(1, 0) == "batch_kernel<1, 0>"
    assert bench.batch_kernel_name(2, 2) == "batch_kernel<2, 0>"
    for k in ("cgsolveq_kernel<1>", "batch_kernel<1, 0>", "batch_kernel<1, 1>"):
        assert bench.traffic(k, 1000) == 1000 * bench.MEASURED_TRAFFIC_PER_UNKNOWN_ITER[k]
    assert bench.traffic("batch_kernel<2, 0>", 1000) is None
