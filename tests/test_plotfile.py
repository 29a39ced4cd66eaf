"""AMReX plotfile output (the layout fub::amrex::WritePlotFile produces through
amrex::WriteMultiLevelPlotfile).  On the CPU: the library's writer
(csrc/fvs_plotfile.cpp) builds a two-level file that the test reader parses
field by field.  On the GPU: the uniform-grid, cut-cell and AMR solvers write
their Complete state computed on the device, which must equal the oracle's
CompleteFromCons of the downloaded state bit for bit."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads

import plotfile_reader

ROOT = Path(__file__).resolve().parents[1]


def test_writer_layout(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    csrc = ROOT / "finitevolumesolver_gb300" / "csrc"
    exe = tmp_path / "plotfile_check"
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", str(csrc),
                        str(ROOT / "tests" / "cpp" / "plotfile_check.cpp"),
                        str(csrc / "fvs_plotfile.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "plt00003"
    r = subprocess.run([str(exe), str(out)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    pf = plotfile_reader.read(out)
    assert pf["version"] == "HyperCLaw-V1.1"
    assert pf["vars"] == ["Density", "Momentum_0", "Momentum_1", "Energy", "Pressure",
                          "SpeedOfSound"]
    assert pf["dim"] == 2 and pf["time"] == 0.125
    assert pf["prob_lo"] == [0.0, 0.0] and pf["prob_hi"] == [1.0, 0.75]
    assert pf["ratios"] == [2]
    assert pf["domains"] == [((0, 0), (7, 5)), ((0, 0), (15, 11))]
    assert pf["steps"] == [3, 6]
    assert pf["dx"] == [[0.125, 0.125], [0.0625, 0.0625]]
    assert pf["coord"] == 0 and pf["bwidth"] == 0
    L0, L1 = pf["levels"]
    assert L0["step"] == 3 and L1["step"] == 6 and L0["time"] == 0.125
    assert L0["path"] == "Level_0/Cell" and L1["path"] == "Level_1/Cell"
    assert L0["boxes"] == [((0, 0), (3, 5)), ((4, 0), (7, 5))]
    assert L0["real_boxes"][1] == [(0.5, 1.0), (0.0, 0.75)]
    assert L1["real_boxes"][0] == [(0.25, 0.625), (0.125, 0.375)]
    for l, L in enumerate(pf["levels"]):
        for b, ((lo, hi), data) in enumerate(zip(L["boxes"], L["data"])):
            nx, ny = hi[0] - lo[0] + 1, hi[1] - lo[1] + 1
            j, i = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
            want = np.stack([1000.0 * c + 100 * l + 10 * b + i + 0.5 * j for c in range(6)])
            np.testing.assert_array_equal(data, want)
            np.testing.assert_array_equal(L["min"][b], want.reshape(6, -1).min(axis=1))
            np.testing.assert_array_equal(L["max"][b], want.reshape(6, -1).max(axis=1))


def _complete(orc, rank, cons):
    return orc.complete_from_cons(rank, cons.reshape(rank + 2, -1))


@pytest.mark.gpu
@pytest.mark.parametrize("rank,n", [(1, 300), (2, 96), (3, 40)])
def test_uniform_solver_plotfile(fvs, orc, tmp_path, rank, n):
    shape = (n,) * rank
    cons = workloads.random_state(tuple(reversed(shape)), rank, seed=rank)
    cons = cons.reshape((rank + 2,) + (1,) * (3 - rank) + tuple(reversed(shape)))
    s = fvs.Solver([n] * rank, [1.0 / n] * rank, "periodic")
    s.upload(cons)
    s.run(cfl=0.8, t_end=10.0, max_steps=2, log_len=2)
    s.write_plotfile(tmp_path / "plt")
    state = s.download()
    s.close()
    pf = plotfile_reader.read(tmp_path / "plt")
    assert pf["dim"] == rank and len(pf["levels"]) == 1 and pf["steps"] == [2]
    assert pf["vars"][0] == "Density" and pf["vars"][-1] == "SpeedOfSound"
    assert pf["vars"][1] == ("Momentum" if rank == 1 else "Momentum_0")
    full = _complete(orc, rank, state).reshape((rank + 4,) + tuple(reversed(shape)))
    L = pf["levels"][0]
    covered = 0
    for (lo, hi), data in zip(L["boxes"], L["data"]):
        sl = tuple(slice(lo[d], hi[d] + 1) for d in reversed(range(rank)))
        np.testing.assert_array_equal(data, full[(slice(None),) + sl])
        covered += data[0].size
    assert covered == n ** rank
    assert pf["time"] > 0


@pytest.mark.gpu
def test_cut_cell_plotfile(fvs, orc, tmp_path):
    n = 80
    circles = [[0.45, 0.5, 0.17], [0.8, 0.3, 0.1]]
    s = fvs.Solver([n, n], [1.0 / n, 1.0 / n], "transmissive")
    s.set_embedded_circles(circles)
    rng = np.random.default_rng(4)
    rho = rng.uniform(0.5, 1.5, (n, n))
    p = rng.uniform(0.5, 1.5, (n, n))
    cons = workloads.cons_from_prim(rho, [rng.uniform(-0.3, 0.3, (n, n)),
                                          rng.uniform(-0.3, 0.3, (n, n))], p)
    s.upload(cons.reshape(4, 1, n, n))
    s.run(cfl=0.5, t_end=10.0, max_steps=2, log_len=2)
    s.write_plotfile(tmp_path / "plt")
    state = s.download().reshape(4, n, n)
    g = s.cutcell_geometry()
    s.close()
    G = g["ghost"]
    alpha = g["alpha"][G:-G, G:-G]
    normal = g["normal"][:, G:-G, G:-G]
    pf = plotfile_reader.read(tmp_path / "plt")
    assert pf["vars"] == ["Density", "Momentum_0", "Momentum_1", "Energy", "Pressure",
                          "SpeedOfSound", "Boundary_X", "Boundary_Y", "vfrac"]
    full = _complete(orc, 2, state).reshape(6, n, n)
    live = (alpha > 0) & (state[0] > 0)
    want = np.where(live, full, 0.0)
    cut = (alpha > 0) & (alpha < 1)
    bx = np.where(cut, -normal[0], 0.0)
    by = np.where(cut, -normal[1], 0.0)
    rows = 0
    for (lo, hi), data in zip(pf["levels"][0]["boxes"], pf["levels"][0]["data"]):
        sl = slice(lo[1], hi[1] + 1)
        np.testing.assert_array_equal(data[:6], want[:, sl])
        np.testing.assert_array_equal(data[6], bx[sl])
        np.testing.assert_array_equal(data[7], by[sl])
        np.testing.assert_array_equal(data[8], alpha[sl])
        rows += hi[1] - lo[1] + 1
    assert rows == n


@pytest.mark.gpu
def test_amr_plotfile(fvs, orc, tmp_path):
    h, acons = workloads.amr_blast_2d(32, 3, target=40, sizes=(8,))
    a = fvs.AmrSolver(h)
    a.upload(acons)
    a.run(cfl=0.8, t_end=10.0, max_steps=2, log_len=2)
    a.write_plotfile(tmp_path / "plt")
    state = a.download()
    a.close()
    pf = plotfile_reader.read(tmp_path / "plt")
    assert len(pf["levels"]) == h.nlevels and pf["steps"] == [2 << l for l in range(h.nlevels)]
    assert pf["ratios"] == [2] * (h.nlevels - 1)
    off = 0
    seen = [0] * h.nlevels
    for p, lev in enumerate(h.levels):
        x0, y0, x1, y1 = h.boxes[p]
        nx, ny = x1 - x0, y1 - y0
        patch = state[off:off + 4 * nx * ny].reshape(4, ny, nx)
        off += 4 * nx * ny
        L = pf["levels"][lev]
        b = seen[lev]
        seen[lev] += 1
        assert L["boxes"][b] == ((x0, y0), (x1 - 1, y1 - 1))
        want = _complete(orc, 2, patch).reshape(6, ny, nx)
        np.testing.assert_array_equal(L["data"][b], want)
