"""The header-only C++17 shim (include/fvs_gpu.hpp) compiles against the C
ABI, links with libfvs_gb300.so, and raises fvs_gpu::Error with the
library's status code; on a GPU its context-level members run a uniform
patch through stable dt, fluxes, update and CompleteFromCons, and a level of
non-uniform patches on separate streams bit for bit like the oracle."""
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


@pytest.mark.gpu
def test_shim_level_of_random_patches_matches_oracle(tmp_path, torch_cuda, orc):
    import numpy as np
    from finitevolumesolver_gb300 import workloads
    exe = _build(tmp_path)
    nx, ny, g, npatch, dx = 24, 10, 2, 3, 1.0 / 64
    NX, NY = nx + 2 * g, ny + 2 * g
    scr = []
    for p in range(npatch):
        cons = workloads.random_state((NY, NX), 2, seed=50 + p, v=0.8).reshape(4, 1, NY, NX)
        scr.append(orc.complete_from_cons(2, cons.reshape(4, -1)).reshape(6, 1, NY, NX))
    inp = tmp_path / "in.bin"
    out = tmp_path / "out.bin"
    np.concatenate([np.array([nx, ny, g, npatch, dx], dtype=np.float64)] +
                   [s.ravel() for s in scr]).tofile(inp)
    r = subprocess.run([str(exe), "patches", str(inp), str(out)], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    res = np.fromfile(out)
    m = orc.method()
    cbox = ([-g, -g], [nx + g, ny + g])
    dts = [orc.compute_stable_dt(m, 2, s, cbox, dx, 0, window_rule=1) for s in scr]
    dt = min(dts)
    assert res[0] == dt
    nflux = 4 * (nx + 1) * ny
    off = 1
    for s in scr:
        flux = res[off:off + nflux].reshape(4, 1, ny, nx + 1)
        off += nflux
        got = res[off:off + s.size].reshape(s.shape)
        off += s.size
        ref_f = orc.compute_numeric_fluxes(m, 2, s, cbox, ([0, 0], [nx + 1, ny]), 0.5 * dt, dx, 0)
        np.testing.assert_array_equal(flux, ref_f)
        # update of the valid cells in place, then CompleteFromCons everywhere
        cons = np.ascontiguousarray(s[:4])
        upd = orc.update_conservatively(([0, 0], [nx, ny]), cons, cbox, ref_f,
                                        ([0, 0], [nx + 1, ny]), 0.5 * dt, dx, 0)
        cons[:, :, g:g + ny, g:g + nx] = upd
        ref = orc.complete_from_cons(2, cons.reshape(4, -1)).reshape(s.shape)
        np.testing.assert_array_equal(got, ref)
