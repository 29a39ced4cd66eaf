"""Reader of AMReX plotfile directories for the tests: the "HyperCLaw-V1.1"
Header, each level's VisMF Cell_H and the FABs of Cell_D_* (an ASCII line
with the number format, box and component count, then the values component
by component, x fastest)."""
from __future__ import annotations

import re
from pathlib import Path

import numpy as np

_BOX = re.compile(r"\(\(([-\d,]+)\) \(([-\d,]+)\) \(([-\d,]+)\)\)")
_FAB = re.compile(r"^FAB \(\((\d+), \(([\d ]+)\)\),\((\d+), \(([\d ]+)\)\)\)"
                  r"\(\(([-\d,]+)\) \(([-\d,]+)\) \(([-\d,]+)\)\) (\d+)\n$")


def _boxes(text):
    return [(tuple(int(v) for v in lo.split(",")), tuple(int(v) for v in hi.split(",")))
            for lo, hi, _ in _BOX.findall(text)]


def read(path):
    path = Path(path)
    it = iter((path / "Header").read_text().split("\n"))
    pf = {"version": next(it)}
    nvars = int(next(it))
    pf["vars"] = [next(it) for _ in range(nvars)]
    pf["dim"] = dim = int(next(it))
    pf["time"] = float(next(it))
    finest = int(next(it))
    pf["prob_lo"] = [float(x) for x in next(it).split()]
    pf["prob_hi"] = [float(x) for x in next(it).split()]
    pf["ratios"] = [int(x) for x in next(it).split()]
    pf["domains"] = _boxes(next(it))
    pf["steps"] = [int(x) for x in next(it).split()]
    pf["dx"] = [[float(x) for x in next(it).split()] for _ in range(finest + 1)]
    pf["coord"] = int(next(it))
    pf["bwidth"] = int(next(it))
    levels = []
    for _ in range(finest + 1):
        lev, nb, t = next(it).split()
        L = {"level": int(lev), "time": float(t), "step": int(next(it)), "real_boxes": []}
        for _ in range(int(nb)):
            L["real_boxes"].append([tuple(float(v) for v in next(it).split())
                                    for _ in range(dim)])
        L["path"] = next(it)
        levels.append(L)
    pf["levels"] = levels
    for L in levels:
        _read_level(path, L, nvars, dim)
    return pf


def _read_level(path, L, nvars, dim):
    cell_h = (path / (L["path"] + "_H")).read_text().split("\n")
    assert cell_h[0] == "1" and cell_h[1] == "1", cell_h[:2]
    assert int(cell_h[2]) == nvars and cell_h[3] == "0"
    m = re.match(r"\((\d+) 0$", cell_h[4])
    nb = int(m.group(1))
    L["boxes"] = _boxes("\n".join(cell_h[5:5 + nb]))
    assert cell_h[5 + nb] == ")"
    assert int(cell_h[6 + nb]) == nb
    fods = [cell_h[7 + nb + b].split() for b in range(nb)]
    k = 7 + 2 * nb
    assert cell_h[k] == ""
    mm = []
    for _ in range(2):
        k += 1
        assert cell_h[k] == f"{nb},{nvars}"
        rows = [[float(v) for v in cell_h[k + 1 + b].rstrip(",").split(",")] for b in range(nb)]
        mm.append(np.array(rows))
        k += nb + 1
        assert cell_h[k] == ""
    L["min"], L["max"] = mm
    L["data"] = []
    level_dir = path / Path(L["path"]).parent
    for b, (tag, fname, off) in enumerate(fods):
        assert tag == "FabOnDisk:"
        with open(level_dir / fname, "rb") as f:
            f.seek(int(off))
            line = f.readline().decode()
            m = _FAB.match(line)
            assert m, line
            assert m.group(1) == "8" and m.group(2) == "64 11 52 0 1 12 0 1023"
            assert m.group(4) == "8 7 6 5 4 3 2 1"  # little-endian doubles
            lo = tuple(int(v) for v in m.group(5).split(","))
            hi = tuple(int(v) for v in m.group(6).split(","))
            assert (lo, hi) == L["boxes"][b]
            assert int(m.group(8)) == nvars
            ext = [h - l + 1 for l, h in zip(lo, hi)]
            n = int(np.prod(ext))
            a = np.frombuffer(f.read(8 * n * nvars), dtype="<f8")
            L["data"].append(a.reshape((nvars,) + tuple(reversed(ext))))
