"""Build libcssg.so (CUDA kernels + C ABI) in-tree for sm_103a.

Each .cu file is compiled by its own nvcc process (in parallel), then linked with ``nvcc -shared``.  The walk's
translation unit is compiled with ``-fmad=false`` so its edge-crossing arithmetic matches the CPU restatement
operation for operation; host code (mesh preprocessing) is compiled with ``-ffp-contract=off`` for the same reason
(aarch64 g++ would otherwise fuse multiply-adds in the edge frames and normals).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(OUT_DIR, "libcssg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr"]
PER_FILE = {"walk.cu": ["-fmad=false"]}
SOURCES = ["mesh.cu", "walk.cu", "geodesic.cu", "geodesic_outlined.cu", "lanes.cu", "system.cu", "diag.cu", "mlp.cu",
           "noalloc.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcssg.so")


def _stale(srcs, out):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    deps = [os.path.join(CSRC, s) for s in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "cssg.h"),
                                                                 os.path.abspath(__file__)]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, extra=None) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and not _stale(SOURCES, LIB_PATH):
        return LIB_PATH
    cc = nvcc()
    extra = list(extra or [])

    def compile_one(src):
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *COMMON, *PER_FILE.get(src, []), *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None))
