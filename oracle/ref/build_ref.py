#!/usr/bin/env python3
"""Build the unmodified Physecs reference into oracle/_ref/ (test infrastructure).

Recipe (no reference build system is run):
  1. copy the reference's src/, include/ and vendored glm / EnTT headers from
     the reference checkout into oracle/_ref/tree/ (gitignored; never committed);
  2. apply purely mechanical MSVC->GCC spelling fixes to that copy:
       * ``x.m128_f32[i]`` / ``x.m128_i32[i]`` / ``x.m128i_i32[i]`` lane access
         -> ``((float*)&(x))[i]`` / ``((int*)&(x))[i]``;
       * the free ``__m128`` operator overloads in include/Physecs/SIMD.h:155-186
         are fenced with ``#ifdef _MSC_VER`` (GCC's built-in vector operators
         perform the same IEEE lane arithmetic);
       * ``ConstraintList``'s in-class ``__m128i`` initialiser becomes a
         constructor (GCC rejects the NSDMI inside the variant);
       * ``class Scene`` / ``class Constraint1DContainer`` gain a leading
         ``public:`` so the fixture driver can read the pair list and the
         contact constraints;
     no arithmetic expression is changed;
  3. compile every reference .cpp plus oracle/ref/ref_capi.cpp into
     oracle/_ref/libphysecs_ref.so with g++ -std=c++23 -O2 -ffp-contract=off
     and EnTT's ENTT_PACKED_PAGE raised to 131072 (see build()).

When the reference checkout is absent (e.g. on a machine that only received
the prepared copy), step 1-2 are skipped and the existing copy is compiled.
"""
import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
REPO = os.path.dirname(ORACLE)
OUT = os.path.join(ORACLE, "_ref")
TREE = os.path.join(OUT, "tree")
# the reference checkout: PSX_REFERENCE, else a `reference` directory beside this repository
REFERENCE = os.environ.get("PSX_REFERENCE") or os.path.join(os.path.dirname(REPO), "reference")

LANE_RE = re.compile(r"([A-Za-z_][A-Za-z0-9_]*(?:(?:\.|->)[A-Za-z_][A-Za-z0-9_]*)*)\.(m128_f32|m128_i32|m128i_i32)\[")


def _lane(m):
    ty = "float" if m.group(2) == "m128_f32" else "int"
    return "((%s*)&(%s))[" % (ty, m.group(1))


def _patch(path, fn):
    with open(path) as f:
        s = f.read()
    t = fn(s)
    if t != s:
        with open(path, "w") as f:
            f.write(t)


def prepare_tree():
    if os.path.isdir(TREE):
        shutil.rmtree(TREE)
    os.makedirs(TREE)
    for sub in ("src", "include"):
        shutil.copytree(os.path.join(REFERENCE, sub), os.path.join(TREE, sub))
    shutil.copytree(os.path.join(REFERENCE, "vendor", "glm 0.9.9.8", "glm"), os.path.join(TREE, "vendor", "glm"))
    os.makedirs(os.path.join(TREE, "vendor", "entt"))
    shutil.copy(os.path.join(REFERENCE, "vendor", "entt-3.12.2", "single_include", "entt", "entt.hpp"),
                os.path.join(TREE, "vendor", "entt", "entt.hpp"))
    for root, _, files in os.walk(os.path.join(TREE)):
        if "vendor" in root:
            continue
        for name in files:
            if name.endswith((".h", ".cpp")):
                _patch(os.path.join(root, name), lambda s: LANE_RE.sub(_lane, s))

    def simd(s):
        a = s.index("inline __m128 operator+ (__m128 a, __m128 b)")
        b = s.index("inline Vec3W operator* (__m128 a, const Vec3W &b)")
        return s[:a] + "#ifdef _MSC_VER\n    " + s[a:b] + "#endif\n    " + s[b:]
    _patch(os.path.join(TREE, "include", "Physecs", "SIMD.h"), simd)

    def container(s):
        s = s.replace("__m128i lanes = _mm_setzero_si128();",
                      "__m128i lanes;\n            ConstraintList() : lanes(_mm_setzero_si128()) {}")
        s = s.replace("class Constraint1DContainer {", "class Constraint1DContainer { public:")
        return s
    _patch(os.path.join(TREE, "include", "Physecs", "Constraint1DContainer.h"), container)
    _patch(os.path.join(TREE, "include", "Physecs", "Physecs.h"),
           lambda s: s.replace("    class Scene {\n", "    class Scene { public:\n", 1))


def build(jobs=8, verbose=False, portable=None):
    """portable: emulate SSE on GCC vector extensions (default: on hosts other than x86)."""
    if os.path.isdir(REFERENCE):
        prepare_tree()
    elif not os.path.isdir(TREE):
        raise RuntimeError("reference sources unavailable: neither %s nor %s exist" % (REFERENCE, TREE))
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    shim_dir = HERE
    inc = [
        "-I" + os.path.join(TREE, "src"),
        "-I" + os.path.join(TREE, "include", "Physecs"),
        "-I" + os.path.join(TREE, "include", "Physecs", "Joints"),
        "-I" + os.path.join(TREE, "include"),
        "-I" + os.path.join(TREE, "vendor"),
        "-I" + os.path.join(TREE, "vendor", "entt"),
        "-I" + os.path.join(REPO, "include"),
        "-I" + shim_dir,
    ]
    # ENTT_PACKED_PAGE: simulate() indexes the first EnTT page of
    # RigidBodyDynamicComponent storage as if it were the whole array
    # (src/Physecs.cpp:117,444,495,524), which is only valid while every dynamic
    # body sits in page 0.  EnTT's own configuration macro raises the page size
    # so scenes up to 131072 dynamic bodies stay inside it; no source changes.
    flags = ["-std=c++23", "-O2", "-fPIC", "-ffp-contract=off", "-DGLM_FORCE_INLINE", "-DPHYSECS_EXPORTS",
             "-DENTT_PACKED_PAGE=131072",
             "-w", "-include", os.path.join(shim_dir, "ref_shim.h")]
    import platform
    if portable is None:
        portable = platform.machine() not in ("x86_64", "AMD64", "i686")
    out_dir = OUT
    if portable:
        inc = ["-I" + os.path.join(HERE, "arm_include")] + inc
        flags += ["-DPSX_SSE_PORTABLE"]
        if platform.machine() in ("x86_64", "AMD64", "i686"):
            out_dir = os.path.join(OUT, "portable")   # validation build of the emulation on x86
            objdir = os.path.join(out_dir, "obj")
            os.makedirs(objdir, exist_ok=True)
    else:
        flags += ["-msse4.2"]
    srcs = []
    for root, _, files in os.walk(os.path.join(TREE, "src")):
        for name in sorted(files):
            if name.endswith(".cpp") and name not in ("Constraint1D.cpp", "Constraint1DW.cpp"):
                srcs.append(os.path.join(root, name))
    srcs.append(os.path.join(HERE, "ref_capi.cpp"))

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(os.path.dirname(src)) + "_" + os.path.basename(src) + ".o")
        cmd = ["g++"] + flags + inc + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s: %s" % (os.path.basename(src), " | ".join(r.stderr.strip().splitlines()[-12:])))
        return obj

    with ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(compile_one, srcs))
    lib = os.path.join(out_dir, "libphysecs_ref.so")
    r = subprocess.run(["g++", "-shared", "-o", lib] + objs + ["-lpthread"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
