"""Builds libfvs_gb300.so (the CUDA kernels and the C ABI) in-tree with nvcc.

Only sm_103a (GB300) is targeted.  The exact-FP64 translation unit is
compiled with -fmad=false so that its arithmetic matches the reference's
no-FMA x86-64 build bit for bit.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR / "csrc"
INCLUDE = PKG_DIR.parent / "include"
BUILD_DIR = PKG_DIR / "_build"
LIB_PATH = PKG_DIR / "libfvs_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
          "-I", str(INCLUDE), "-I", str(CSRC)]

# (source, extra flags)
UNITS = [
    ("fvs_kernels_exact.cu", ["-fmad=false"]),
    ("fvs_kernels_fast.cu", []),
    ("fvs_kernels_df64.cu", []),
    ("fvs_kernels_godunov.cu", ["-fmad=false"]),
    ("fvs_kernels_cutcell.cu", ["-fmad=false"]),
    ("fvs_kernels_cutcell_mixed.cu", []),
    ("fvs_capi.cu", []),
    ("fvs_noalloc.cu", ["-fmad=false"]),
    ("fvs_host_patch.cu", []),
    ("fvs_mlp_train.cu", []),
    ("fvs_amr.cu", []),
    ("fvs_amr_exact.cu", ["-fmad=false"]),
    ("fvs_amr_fast.cu", []),
    ("fvs_plotfile.cpp", []),
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfvs_gb300")


def _sources_newer(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile every translation unit for sm_103a and link the shared library."""
    nvcc = _nvcc()
    BUILD_DIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    jobs = []
    objs = []
    for src, extra in UNITS:
        obj = BUILD_DIR / (Path(src).stem + ".o")
        objs.append(obj)
        if force or _sources_newer(obj, [CSRC / src, *headers]):
            cmd = [nvcc, *ARCH, *COMMON, *extra, "-c", str(CSRC / src), "-o", str(obj)]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _sources_newer(LIB_PATH, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", str(LIB_PATH), *map(str, objs), "-lcudart"]
        run(cmd)
    return LIB_PATH


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB_PATH)
