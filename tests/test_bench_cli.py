"""CPU tests of bench.py's command line: the reference arm (the FP64 oracle
on the host cores) prints one JSON line with the fields the benchmark
contract asks for, and the slice-count overrides name the workload."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--small", "--steps", "1", "--warmup", "0"],
                         cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["value"] > 0 and line["unit"] == "iter/s" and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"]["workload"].startswith("N=256 Nz=16 Nzp=8")


def test_workload_overrides():
    sys.path.insert(0, ROOT)
    import bench

    class A:
        small = False
        nz = 2
        nzp = 2

    w = bench.workload_of(A())
    assert (w["n"], w["nz"], w["nzp"], w["ntheta"], w["m"]) == (1024, 2, 2, 2880, 16)
    assert bench.workload_name(w) == "N=1024 Nz=2 Nzp=2 Ntheta=2880 Nrot=8 M=16 titer=4"

    class B:
        small = False
        nz = None
        nzp = None

    assert bench.workload_of(B()) == bench.WORKLOAD
