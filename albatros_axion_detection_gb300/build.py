"""Build the in-tree CUDA library ``lib/libalbatros_gb300.so`` for sm_103a.

Each ``csrc/*.cu`` is compiled to an object in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo`` and the objects
are linked into one shared library with a plain C ABI (include/albatros_gb300.h).
The library is rebuilt only when a source or header is newer than it.

    python -m albatros_axion_detection_gb300.build [--force] [--verbose]
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
OUTDIR = os.path.join(PKG, "lib")
LIB = os.path.join(OUTDIR, "libalbatros_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(verbose: bool):
    f = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I", os.path.join(ROOT, "include"), *ARCH]
    if verbose:
        f += ["-Xptxas", "-v"]
    return f


def _stale(srcs, deps) -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in list(srcs) + list(deps))


def build(force: bool = False, verbose: bool = False) -> str:
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    deps = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    if not force and not _stale(srcs, deps):
        return LIB
    os.makedirs(os.path.join(OUTDIR, "obj"), exist_ok=True)
    cc = nvcc()
    flags = _flags(verbose)

    def compile_one(src):
        obj = os.path.join(OUTDIR, "obj", os.path.basename(src) + ".o")
        cmd = [cc, *flags, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    r = subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
