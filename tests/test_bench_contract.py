"""bench.py's JSON contract, checked on the parts that run without a GPU:
the reference arm's line (the CPU port of the reference path, full size of
the requested shape, no extrapolation) and the host-side problem
construction, at small sizes."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    sys.path.insert(0, ROOT)
    import bench
    return bench


def test_reference_arm_line_keys():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--workload", "plain_ls", "--steps", "2", "--warmup", "0", "--m", "12000", "--n", "40"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "impl",
                "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["status"] == "finished"
    assert line["steps"] == len(line["runs"]) == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    # the measured time is the mean of the full-size solves, not a scaled sample
    mean = sum(r["seconds"] for r in line["runs"]) / 2
    assert abs(line["value"] - 1.0 / mean) < 1e-9 * line["value"]
    bench = _bench()
    args = bench.parse(["--workload", "plain_ls", "--m", "12000", "--n", "40"])
    assert line["config"] == bench.workload_config(args, bench.workload(args), 1)
    # the port converged to the LAPACK residual
    for r in line["runs"]:
        assert r["rel_residual"] < 1e-3


def test_workloads_and_host_problem():
    import numpy as np
    bench = _bench()
    args = bench.parse([])
    wl = bench.workload(args)
    assert args.workload == "precision_ls"
    assert (wl["m"], wl["n"], wl["d"], wl["f32"], wl["kappa"]) == (1048576, 1024, 4096, True, 1e6)
    args = bench.parse(["--workload", "precision_ls", "--m", "3000", "--n", "30"])
    wl = bench.workload(args)
    A, b = bench.make_problem_host(wl)
    assert A.shape == (3000, 30) and A.flags.f_contiguous and b.shape == (3000,)
    # FP32-stored workload: every entry is exactly an FP32 value
    assert np.array_equal(A, A.astype(np.float32).astype(np.float64))
    s = np.linalg.svd(A, compute_uv=False)
    assert abs(s[0] - 1.0) < 1e-6 and abs(s[0] / s[-1] / 1e6 - 1.0) < 1e-2
