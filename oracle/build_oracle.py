#!/usr/bin/env python3
"""Build the CPU oracle (oracle/port/*.cpp) into oracle/_build/liborc.so.

ORACLE (test infrastructure only).  Plain g++, -ffp-contract=off so every
float operation rounds exactly as the reference's does (the reference is
compiled the same way by oracle/ref/build_ref.py).  Host-portable: no
architecture flags, builds on x86-64 and aarch64 alike.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liborc.so")
SRCS = ["collide_util.cpp", "gjk_epa.cpp", "collide.cpp", "collide_tri.cpp", "world.cpp", "query.cpp", "port_capi.cpp"]
FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function",
         "-I" + os.path.join(REPO, "include")]


def build(jobs=6):
    os.makedirs(OUT, exist_ok=True)

    def one(src):
        obj = os.path.join(OUT, src + ".o")
        path = os.path.join(HERE, "port", src)
        if os.path.exists(obj) and os.path.getmtime(obj) >= max(
                os.path.getmtime(path), *[os.path.getmtime(os.path.join(HERE, "port", h))
                                          for h in os.listdir(os.path.join(HERE, "port")) if h.endswith(".h")],
                os.path.getmtime(os.path.join(REPO, "include", "psx.h"))):
            return obj
        cmd = ["g++"] + FLAGS + ["-c", path, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle compile failed: %s\n%s" % (" ".join(cmd), r.stderr[-6000:]))
        return obj

    with ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(one, SRCS))
    r = subprocess.run(["g++", "-shared", "-o", LIB] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle link failed:\n" + r.stderr[-4000:])
    return LIB


if __name__ == "__main__":
    print(build())
