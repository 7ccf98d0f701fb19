"""Builds the engine's shared library (libcudancorr_gb300.so) in-tree.

The CUDA sources under csrc/ are compiled for sm_103a only, in parallel, and
linked into cudancorr_gb300/lib/. No PyTorch extension machinery is involved:
the library exposes the C ABI of include/ncorr_gb300.h and is loaded with
ctypes (Python) or linked directly (C/C++).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "lib"
OBJ = PKG / "lib" / "obj"
LIBNAME = "libcudancorr_gb300.so"

SOURCES = ["cell_list.cu", "triangles_launch.cu", "sched.cu", "capi.cu", "sched_api.cu", "batch.cu", "rppi.cu", "utils.cu"]
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code: no implicit FMA contraction, so that host arithmetic (bin
# edges, tables, coordinates) gives the same bits on x86 and Arm hosts.
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and pathlib.Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, verbose: bool, obj_dir: pathlib.Path = None, defines=()) -> pathlib.Path:
    obj = (obj_dir or OBJ) / (pathlib.Path(src).stem + ".o")
    cmd = [nvcc(), *GENCODE, *FLAGS, *[f"-D{d}" for d in defines], "-c", str(CSRC / src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, file=sys.stderr)
    return obj


def library_path() -> pathlib.Path:
    return OUT / LIBNAME


def build(verbose: bool = False, force: bool = False, out: pathlib.Path = None, defines=()) -> pathlib.Path:
    """Compiles (when stale) and returns the path of the shared library.

    `out` and `defines` build a variant of the library (tuning constants set
    with -D) into another directory."""
    out_dir = pathlib.Path(out) if out else OUT
    obj_dir = out_dir / "obj"
    obj_dir.mkdir(parents=True, exist_ok=True)
    lib = out_dir / LIBNAME
    deps = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "ncorr_gb300.h"]
    if lib.exists() and not force:
        newest = max(p.stat().st_mtime for p in deps)
        if lib.stat().st_mtime >= newest:
            return lib
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, obj_dir, defines), SOURCES))
    tmp = lib.with_suffix(".so.tmp")
    cmd = [nvcc(), *GENCODE, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
