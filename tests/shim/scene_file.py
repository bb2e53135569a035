"""Scene files and builds for tests/shim/drive_scene.cpp (test infrastructure).

drive_scene.cpp is one Physecs application source compiled twice: against the reference
(its headers and the library built from its sources under oracle/_ref) and against
include/physecs_gb300/Physecs.h with libpsx.so.  This module writes the scene file both
builds read, compiles them, and runs them.
"""
from __future__ import annotations

import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "drive_scene.cpp")

OP_KINEMATIC, OP_PATCH, OP_JOINT, OP_VELOCITY = 1, 2, 3, 4
OP_DESTROY, OP_CLEAR, OP_ADD_SPHERE, OP_DESTROY_JOINT, OP_SPAWN_SPHERE = 5, 6, 7, 8, 9


def tree():
    from oracle.ref import build_ref
    return build_ref.TREE


def write_scene(path, s, frames, ops=()):
    """The SceneData `s` (no triangle meshes), `frames` frames, and ops = [(frame, op, index,
    values up to 8 floats)] applied before the given frame, in list order."""
    a = s.arrays
    nb, nc = len(a["pos"]), len(a["col_type"])
    assert len(a["tri_index_start"]) <= 1, "triangle meshes are not written"
    ops = sorted(ops, key=lambda o: o[0])
    counts = np.array([nb, nc, len(a["convex_vert_start"]) - 1, len(a["face_normal"]), len(a["face_indices"]),
                       len(a["convex_verts"]), len(a["joint_type"]), s.num_substeps, s.num_iterations, frames, len(ops),
                       sum(1 for o in ops if o[1] == OP_SPAWN_SPHERE), 0], np.int32)
    parts = [counts, np.array([s.gravity], np.float32),
             a["flags"].astype(np.uint32), a["pos"], a["quat"], a["vel"], a["ang_vel"], a["inv_mass"], a["com"],
             a["inv_inertia"], a["collider_start"].astype(np.int32),
             a["col_pos"], a["col_quat"], a["col_type"].astype(np.int32), a["col_params"], a["col_mesh"].astype(np.int32),
             a["col_material"], a["col_is_trigger"].astype(np.uint8), a["col_enable_sim"].astype(np.uint8),
             a["col_data"].astype(np.int32),
             a["convex_vert_start"], a["convex_verts"], a["convex_face_start"], a["face_index_start"], a["face_indices"],
             a["face_normal"], a["face_centroid"],
             a["joint_type"], a["joint_body0"], a["joint_body1"], a["joint_frames"], a["joint_params"]]
    oi = np.zeros((len(ops), 4), np.int32)
    of = np.zeros((len(ops), 8), np.float32)
    for k, (fr, op, idx, vals) in enumerate(ops):
        oi[k, :3] = fr, op, idx
        of[k, :len(vals)] = vals
    parts += [oi, of]
    with open(path, "wb") as f:
        for p in parts:
            p = np.ascontiguousarray(p)
            if p.dtype == np.float64:
                p = p.astype(np.float32)
            f.write(p.tobytes())


def _common():
    return ["-O2", "-DENTT_PACKED_PAGE=131072", "-DGLM_FORCE_INLINE", "-w"]


def build_shim():
    """The application against physecs_gb300/Physecs.h and libpsx.so."""
    from physecs_gb300 import _build
    lib = _build.build()
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "drive_shim")
    t = tree()
    cmd = (["g++", "-std=c++20"] + _common() +
           ["-I" + os.path.join(t, "include", "Physecs"), "-I" + os.path.join(t, "vendor"),
            "-I" + os.path.join(t, "vendor", "entt"), "-I" + os.path.join(ROOT, "include"),
            SRC, "-o", exe, "-L" + os.path.dirname(lib), "-lpsx", "-Wl,-rpath," + os.path.dirname(lib)])
    _run(cmd)
    return exe


def build_reference():
    """The same application against the reference's headers and library."""
    from oracle.ref import build_ref
    lib = os.path.join(build_ref.OUT, "libphysecs_ref.so")
    if not os.path.exists(lib):
        lib = build_ref.build()
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "drive_reference")
    t = tree()
    flags = ["-std=c++23", "-ffp-contract=off", "-include", os.path.join(build_ref.HERE, "ref_shim.h")]
    inc = ["-I" + os.path.join(t, "include", "Physecs"), "-I" + os.path.join(t, "include", "Physecs", "Joints"),
           "-I" + os.path.join(t, "include"), "-I" + os.path.join(t, "vendor"), "-I" + os.path.join(t, "vendor", "entt"),
           "-I" + os.path.join(ROOT, "include"), "-I" + build_ref.HERE]
    if platform.machine() not in ("x86_64", "AMD64", "i686"):
        inc = ["-I" + os.path.join(build_ref.HERE, "arm_include")] + inc
        flags += ["-DPSX_SSE_PORTABLE"]
    else:
        flags += ["-msse4.2"]
    cmd = (["g++"] + flags + _common() + ["-DDRIVE_REFERENCE"] + inc +
           [SRC, "-o", exe, lib, "-lpthread", "-Wl,-rpath," + os.path.dirname(lib)])
    _run(cmd)
    return exe


def build_layout_check():
    """A program printing the component layouts, compiled against the reference's headers,
    EnTT, psx.h and physecs_gb300/Physecs.h."""
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "layout_check")
    t = tree()
    _run(["g++", "-std=c++20"] + _common() +
         ["-I" + os.path.join(t, "include", "Physecs"), "-I" + os.path.join(t, "vendor"),
          "-I" + os.path.join(t, "vendor", "entt"), "-I" + os.path.join(ROOT, "include"),
          os.path.join(HERE, "layout_check.cpp"), "-o", exe])
    return exe


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n%s\n%s" % (" ".join(cmd), (r.stdout + r.stderr)[-6000:]))


def run(exe, scene_path, out_path, n_bodies, frames, timeout=600):
    """Runs a build; returns (returncode, stderr, states (frames, bodies, 13) or None)."""
    r = subprocess.run([exe, scene_path, out_path], capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        return r.returncode, r.stderr, None
    st = np.fromfile(out_path, np.float32).reshape(frames, n_bodies, 13)
    return 0, r.stderr, st
