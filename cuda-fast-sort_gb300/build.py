"""Builds libgbsort.so (sm_103a) in-tree: cuda-fast-sort_gb300/lib/libgbsort.so.

    python cuda-fast-sort_gb300/build.py [--jobs N] [--force]

Every translation unit under csrc/ compiles in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3``; objects go to
cuda-fast-sort_gb300/_build/ and are reused while they are newer than every
source and header.  No cmake, no relocatable device code.
"""

from __future__ import annotations

import argparse
import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libgbsort.so")
INCLUDE = os.path.join(REPO, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2",
                     "-I", INCLUDE, "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libgbsort")


def _newest(paths) -> float:
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _compile(src: str, headers_mtime: float, force: bool, verbose: bool, obj_dir: str,
             defines: list[str], src_dir: str = CSRC) -> str:
    obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= max(headers_mtime, os.path.getmtime(src)):
        return obj
    cmd = [nvcc()] + NVCC_FLAGS + ["-I", src_dir] + [f"-D{d}" for d in defines] + ["-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(jobs: int | None = None, force: bool = False, verbose: bool = False, defines: list[str] | None = None,
          out_dir: str | None = None, csrc: str | None = None) -> str:
    """Builds the library; `defines` (-D...), `out_dir` and `csrc` (another
    source directory) produce a variant build for tuning experiments."""
    defines = defines or []
    src_dir = csrc or CSRC
    obj_dir = os.path.join(out_dir, "obj") if out_dir else BUILD
    lib = os.path.join(out_dir, "libgbsort.so") if out_dir else LIB
    os.makedirs(obj_dir, exist_ok=True)
    os.makedirs(os.path.dirname(lib), exist_ok=True)
    sources = sorted(glob.glob(os.path.join(src_dir, "*.cu")) + glob.glob(os.path.join(src_dir, "*.cpp")))
    headers = (glob.glob(os.path.join(src_dir, "*.cuh")) + glob.glob(os.path.join(src_dir, "*.h"))
               + glob.glob(os.path.join(INCLUDE, "*.h")))
    hm = _newest(headers + [os.path.abspath(__file__)])
    jobs = jobs or max(1, min(len(sources), os.cpu_count() or 4))
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, hm, force, verbose, obj_dir, defines, src_dir), sources))
    if force or not os.path.exists(lib) or os.path.getmtime(lib) < _newest(objs):
        tmp = lib + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
    return lib


CUB_SRC = os.path.join(PKG, "compare", "cub_compare.cu")
CUB_LIB = os.path.join(LIBDIR, "libcubcompare.so")


def build_cub_compare() -> str:
    """Benchmark comparator: cub::DeviceRadixSort from the CUDA toolkit, built
    as its own library (not part of libgbsort)."""
    os.makedirs(LIBDIR, exist_ok=True)
    if os.path.exists(CUB_LIB) and os.path.getmtime(CUB_LIB) >= os.path.getmtime(CUB_SRC):
        return CUB_LIB
    tmp = CUB_LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", CUB_SRC, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CUB comparator build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, CUB_LIB)
    return CUB_LIB


SHIM_TEST_SRC = os.path.join(REPO, "tests", "cpp", "rsort_shim_test.cpp")
SHIM_TEST_BIN = os.path.join(BUILD, "rsort_shim_test")


def build_shim_test() -> str:
    """Compiles the C++ program that uses include/rsort/rsort.cuh (the drop-in
    header) against libgbsort.so, the way a reference user would."""
    os.makedirs(BUILD, exist_ok=True)
    if os.path.exists(SHIM_TEST_BIN) and os.path.getmtime(SHIM_TEST_BIN) >= _newest(
            [SHIM_TEST_SRC, LIB, os.path.join(INCLUDE, "rsort", "rsort.cuh"), os.path.join(INCLUDE, "gbsort.h")]):
        return SHIM_TEST_BIN
    cmd = [nvcc(), "-O2", "-std=c++17", "-x", "c++", SHIM_TEST_SRC, "-I", INCLUDE, "-o", SHIM_TEST_BIN,
           "-L", LIBDIR, "-lgbsort", f"-Xlinker=-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"shim test build failed:\n{r.stdout}\n{r.stderr}")
    return SHIM_TEST_BIN


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("-D", dest="defines", action="append", default=[], help="extra preprocessor define")
    ap.add_argument("--out-dir", default=None, help="variant build directory")
    ap.add_argument("--csrc", default=None, help="alternative source directory")
    a = ap.parse_args()
    print(build(a.jobs, a.force, a.verbose, a.defines, a.out_dir, a.csrc))
