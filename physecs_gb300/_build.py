"""Build libpsx.so (the CUDA hot path and its C ABI) in-tree with nvcc for sm_103a.

Every translation unit is compiled in parallel with
  -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo -fmad=false
and host code with -ffp-contract=off: no fused multiply-add anywhere, IEEE
division and square root, so kernels round like the reference's CPU code.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libpsx.so")
SOURCES = ["prims.cu", "broadphase.cu", "narrowphase.cu", "solver.cu", "world.cu", "server.cu", "query.cu", "meshbvh.cu",
           "carry.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
                "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
                "-Xptxas", "-warn-spills", "-I" + os.path.join(os.path.dirname(HERE), "include")]


# glibc's float acosf, which the servo rows reproduce (csrc/libm_f32.cuh), is compiled
# with fused multiply-adds on aarch64 hosts and without on x86-64 ones
import platform as _platform
if _platform.machine() in ("aarch64", "arm64"):
    FLAGS = FLAGS + ["-DPSX_LIBM_FUSED"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "psx.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, jobs=5):
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()

    def one(name):
        src = os.path.join(CSRC, name)
        obj = os.path.join(OUT, name + ".o")
        if not _stale(obj, src):
            return obj, ""
        cmd = [cc] + FLAGS + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (name, (r.stdout + r.stderr)[-8000:]))
        return obj, r.stderr

    with ThreadPoolExecutor(jobs) as ex:
        res = list(ex.map(one, SOURCES))
    objs = [o for o, _ in res]
    if verbose:
        for _, log in res:
            if log:
                print(log)
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [cc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + (r.stdout + r.stderr)[-4000:])
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv))
