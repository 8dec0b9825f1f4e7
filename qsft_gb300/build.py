"""Build the CUDA library ``qsft_gb300/lib/libqsft_gb300.so`` for sm_103a.

Each translation unit under ``csrc/`` is compiled by nvcc in parallel, then
linked into one shared library with a C ABI (``include/qsft_gb300.h``).  The
library is loaded in-tree by ``qsft_gb300._lib`` with ctypes.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libqsft_gb300.so")
ARCH = "103a"
SOURCES = ["eval.cu", "eval_tc.cu", "eval_gemm.cu", "gwht.cu", "noise.cu", "peel.cu", "abi.cu", "noalloc.cu",
           "reproject.cu"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _flags():
    return ["-std=c++17", "-O3", "-lineinfo", f"-gencode=arch=compute_{ARCH},code=sm_{ARCH}",
            "-Xcompiler", "-fPIC", "-DQSFT_ARCH=103", "--expt-relaxed-constexpr",
            "-I", os.path.join(HERE, "..", "include")]


def _stale(src, obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + deps)


def build(verbose=False, force=False, extra=()):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "qsft_gb300.h"))
    cc = nvcc()
    jobs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, s.replace(".cu", ".o"))
        if force or _stale(src, obj, deps):
            jobs.append([cc, *_flags(), *extra, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(run, jobs))
    for cmd, r in results:
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    objs = [os.path.join(OBJ, s.replace(".cu", ".o")) for s in SOURCES]
    if force or jobs or not os.path.exists(LIB):
        cmd = [cc, "-shared", f"-gencode=arch=compute_{ARCH},code=sm_{ARCH}", *objs, "-o", LIB]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))
