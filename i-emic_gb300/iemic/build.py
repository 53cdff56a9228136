"""Build the in-tree CUDA library ``libiemic_gb300.so`` for sm_103a.

Each translation unit is compiled by nvcc in parallel and linked into one
shared library under ``i-emic_gb300/iemic/_build``. The assembly kernels are
compiled with ``-fmad=false`` so their FP64 arithmetic is not contracted into
fused multiply-adds (bit-identical to the unfused reference arithmetic).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libiemic_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code computes the grid and metric tables in FP64; -ffp-contract=off keeps
# GCC from fusing multiply-adds there (it does by default on aarch64), so the
# tables round exactly like the reference's unfused Fortran arithmetic.
COMMON = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
          "-Xcompiler", "-fno-strict-aliasing", "-Xcompiler", "-ffp-contract=off"]
# per-file extra flags
EXTRA = {"thcm_assembly.cu": ["-fmad=false"]}
SOURCES = ["ocean.cu", "thcm_assembly.cu", "krylov.cu", "ndlu.cu", "solver.cu", "continuation.cu", "noalloc.cu", "adjoint.cu"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    return [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(ROOT), "include", "iemic_gb300.h"))
    deps.append(__file__)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [cc] + ARCH + COMMON + EXTRA.get(src, []) + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-8000:]))
        return obj

    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr[-8000:])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
