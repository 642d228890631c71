"""The dense front kernels of the multifrontal factorisation (blocked LU with
pivoting among the fully-summed rows, triangular inverses, packed GEMM),
compiled from their source with the host compiler and checked against naive
loops: LU reconstruction, inverses, bit-identical results for one and four
threads, and the singular-pivot report."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "pecs_gb300" / "csrc"


def test_dense_front_kernels(tmp_path):
    exe = tmp_path / "dense_check"
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-pthread", f"-I{CSRC}",
                        str(ROOT / "tests" / "dense_check.cpp"), str(CSRC / "dense.cpp"),
                        "-o", str(exe)], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("OK")
