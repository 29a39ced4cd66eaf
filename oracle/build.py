"""Builds the CPU oracle (test infrastructure) as oracle/liboracle.so.

g++ -O2 -ffp-contract=off -fno-fast-math: IEEE arithmetic without FMA
contraction, the same behaviour as the reference's x86-64 build (which sets
no -march and no fast-math).  -ffp-contract=off matters on aarch64, where gcc
contracts a*b+c into FMA by default.
"""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
LIB_PATH = ORACLE_DIR / "liboracle.so"
SOURCES = ["fvs_oracle.cpp", "fvs_oracle_cutcell.cpp", "fvs_oracle_amr.cpp"]
HEADERS = ["fvs_oracle.hpp", "fvs_oracle_riemann.hpp"]
FLAGS = ["-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
         "-fPIC", "-shared", "-Wall"]


def build(force: bool = False) -> Path:
    cxx = shutil.which("g++") or "g++"
    deps = [ORACLE_DIR / s for s in SOURCES + HEADERS]
    if not force and LIB_PATH.exists() and all(
            d.stat().st_mtime <= LIB_PATH.stat().st_mtime for d in deps):
        return LIB_PATH
    cmd = [cxx, *FLAGS, *[str(ORACLE_DIR / s) for s in SOURCES], "-o", str(LIB_PATH)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stderr}")
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
