"""The exact Riemann solver's powers of pressure ratios (n-th roots by
Newton's method and integer powers where n = 2 gamma / (gamma - 1) is an
integer) against pow() with the solver's FP64 exponents, for gamma = 1.4, 5/3
and 1.2, plus the pow() fallbacks (tests/cpp/root_check.cu, compiled by nvcc
as host code)."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_roots_match_pow(tmp_path):
    from finitevolumesolver_gb300 import build
    try:
        nvcc = build._nvcc()
    except RuntimeError:
        pytest.skip("nvcc not found")
    exe = tmp_path / "root_check"
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-x", "cu",
                        "-I", str(ROOT / "finitevolumesolver_gb300" / "csrc"),
                        str(ROOT / "tests" / "cpp" / "root_check.cu"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "fail 0" in r.stdout
