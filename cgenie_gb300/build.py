"""Build the CUDA library libgb_goldstein.so in-tree for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into
cgenie_gb300/_lib/libgb_goldstein.so (static CUDA runtime, C-ABI only).
The FP64 step is compiled with -fmad=false so that no multiply-add is
contracted: its doubles are the reference's non-FMA IEEE results.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(OUT_DIR, "libgb_goldstein.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]
# per-file extra flags
SOURCES = {
    "tstep_fp64.cu": ["-fmad=false"],
    "tstep_fp32.cu": [],
    "gb_goldstein.cu": ["-fmad=false"],
    "ensemble.cu": [],
    "biogem_coupling.cu": ["-fmad=false"],
    "surface_step.cu": ["-fmad=false"],
    "momentum.cu": ["-fmad=false"],
    "restart.cu": ["-fmad=false"],
    "timeseries.cu": ["-fmad=false"],
    "trace.cu": [],
}


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _deps() -> list[str]:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return files


def _needs_build() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(f) > t for f in _deps()) or os.path.getmtime(__file__) > t


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    """Compile every CUDA source for sm_103a and link the shared library."""
    if not force and not _needs_build():
        return LIB_PATH
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    extra = list(extra or [])

    def compile_one(name: str) -> str:
        src = os.path.join(CSRC, name)
        obj = os.path.join(OBJ_DIR, name.replace(".cu", ".o"))
        cmd = [nvcc(), *ARCH, *COMMON, *SOURCES[name], *extra, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
