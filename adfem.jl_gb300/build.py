"""Build libadfem_gpu.so (sm_103a) in-tree with nvcc.

Every translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo`` and linked into
``adfem.jl_gb300/lib/libadfem_gpu.so`` (static CUDA runtime, C ABI only).
Objects go to ``adfem.jl_gb300/_build``.  Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libadfem_gpu.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-fvisibility=hidden,-O3,-ffp-contract=off", "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


CHECKS_BUILD = os.path.join(HERE, "_build_checks")
CHECKS_LIB = os.path.join(LIBDIR, "libadfem_gpu_checks.so")


def _compile(src: str, extra: list[str], build_dir: str = BUILD, always: bool = False) -> str:
    obj = os.path.join(build_dir, os.path.basename(src) + ".o")
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep and not always:
        return obj
    cmd = [nvcc()] + NVCC_FLAGS + extra + ["-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stdout + r.stderr))
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False, ptxas_info: bool = False, checks: bool = False) -> str:
    """Build the library; checks=True builds the debug variant instead (-DADFEM_CHECKS: kernels
    check the indices they compute and record failures, see checks.cuh) as
    lib/libadfem_gpu_checks.so, with its objects in _build_checks."""
    build_dir, lib = (CHECKS_BUILD, CHECKS_LIB) if checks else (BUILD, LIB)
    os.makedirs(build_dir, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    extra = (["-Xptxas", "-v"] if ptxas_info else []) + (["-DADFEM_CHECKS"] if checks else [])
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(16, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, build_dir, ptxas_info), srcs))
    if (not os.path.exists(lib)) or any(os.path.getmtime(o) > os.path.getmtime(lib) for o in objs) or ptxas_info:
        tmp = lib + ".tmp%d" % os.getpid()
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stdout + r.stderr))
        os.replace(tmp, lib)
    if verbose:
        print("built", lib)
    return lib


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv, checks="--checks" in sys.argv)
