"""bench.py's JSON contract, checked on the parts that run without a GPU:
the reference arm's line (the CPU port of the reference path) and the
LAPACK timing beside the CPU baseline, at a small size."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line_keys():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0", "--m", "12000", "--n", "40"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "impl",
                "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    sys.path.insert(0, ROOT)
    import bench
    assert line["config"]["workload"] == bench.workload_name(12000, 40)


def test_lapack_sample_scales_with_rows():
    sys.path.insert(0, ROOT)
    import bench
    t, v = bench.lapack_sample(40000, 40, 4000)
    assert t > 0 and abs(v - 1.0 / (t * 10)) < 1e-12
