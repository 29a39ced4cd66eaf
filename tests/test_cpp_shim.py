"""The header-only C++17 shim (include/fvs_gpu.hpp) compiles against the C
ABI, links with libfvs_gb300.so, and raises fvs_gpu::Error with the
library's status code; on a GPU its context-level members run a uniform
patch through stable dt, fluxes, update and CompleteFromCons."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _build(tmp_path):
    from finitevolumesolver_gb300 import build
    lib = build.build()
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    exe = tmp_path / "shim_check"
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", "-Werror", str(ROOT / "tests" / "cpp" / "shim_check.cpp"),
           "-I", str(ROOT / "include"), "-I", str(cuda / "include"),
           "-L", str(lib.parent), "-lfvs_gb300", f"-Wl,-rpath,{lib.parent}",
           "-L", str(cuda / "lib64"), "-L", str(cuda / "lib"), "-lcudart",
           f"-Wl,-rpath,{cuda / 'lib64'}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_compiles_links_and_reports_errors(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("the no-device path needs a machine without a GPU")
    exe = _build(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "raised 2" in r.stdout


@pytest.mark.gpu
def test_shim_runs_a_patch_on_the_gpu(tmp_path, torch_cuda):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe), "gpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
