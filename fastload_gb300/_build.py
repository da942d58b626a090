"""Builds the FastLoad GB300 CUDA library and the CPU oracle in-tree.

The library is compiled for sm_103a only (``-gencode arch=compute_103a,
code=sm_103a``), one translation unit per ``csrc/*.cu`` file in parallel, and
linked into ``fastload_gb300/_lib/libfastload_gb300.so`` against the shared
CUDA runtime (the same one PyTorch loads).  Rebuilds only when a source or
header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJDIR = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIBNAME = "libfastload_gb300.so"
ORACLE_DIR = os.path.join(ROOT, "oracle")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr", "-I", INCLUDE]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the FastLoad GB300 library needs the CUDA toolkit to build")


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def _sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps() -> list[str]:
    return (_sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
            + [os.path.abspath(__file__)])


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str) -> str:
    obj = os.path.join(OBJDIR, os.path.basename(src).replace(".cu", ".o"))
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    return obj


def build_library(force: bool = False, verbose: bool = False) -> str:
    """Compiles csrc/*.cu for sm_103a and links the shared library."""
    target = lib_path()
    if not force and not _stale(target, _deps()):
        return target
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    tmp = target + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs, "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, target)
    if verbose:
        print(f"built {target}", file=sys.stderr)
    return target


def build_oracle(reference_src: str | None = None) -> None:
    """Builds oracle/liboracle.so and, when reference_src names the
    reference's src/ directory (argument, else the FL_REFERENCE_SRC
    environment variable; no default), oracle/_ref/libfastload_ref.so from
    those sources (test infrastructure only)."""
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "all"], check=True)
    ref_src = reference_src or os.environ.get("FL_REFERENCE_SRC")
    if ref_src and os.path.isdir(ref_src):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, "ref", f"REF_SRC={ref_src}"], check=True)


if __name__ == "__main__":
    build_library(force="--force" in sys.argv, verbose=True)
    build_oracle()
