"""ctypes mirror of ``psx_scene_desc`` (include/psx.h) built from a SceneData."""
from __future__ import annotations

import ctypes as C
import numpy as np

_f = C.POINTER(C.c_float)
_i = C.POINTER(C.c_int32)
_u = C.POINTER(C.c_uint32)
_b = C.POINTER(C.c_uint8)


class PsxSceneDesc(C.Structure):
    _fields_ = [
        ("n_bodies", C.c_int32), ("entity", _u), ("flags", _u), ("pos", _f), ("quat", _f), ("vel", _f),
        ("ang_vel", _f), ("inv_mass", _f), ("com", _f), ("inv_inertia", _f), ("collider_start", _i),
        ("n_colliders", C.c_int32), ("col_pos", _f), ("col_quat", _f), ("col_type", _i), ("col_params", _f),
        ("col_mesh", _i), ("col_material", _f), ("col_is_trigger", _b), ("col_enable_sim", _b), ("col_data", _i),
        ("n_convex", C.c_int32), ("convex_vert_start", _i), ("convex_verts", _f), ("convex_face_start", _i),
        ("face_index_start", _i), ("face_indices", _i), ("face_normal", _f), ("face_centroid", _f),
        ("n_trimesh", C.c_int32), ("tri_vert_start", _i), ("tri_verts", _f), ("tri_index_start", _i),
        ("tri_indices", _u),
        ("n_joints", C.c_int32), ("joint_type", _i), ("joint_body0", _i), ("joint_body1", _i),
        ("joint_frames", _f), ("joint_params", _f),
        ("num_substeps", C.c_int32), ("num_iterations", C.c_int32), ("gravity", C.c_float),
    ]


_PTR_TYPES = {np.float32: _f, np.int32: _i, np.uint32: _u, np.uint8: _b}


def make_desc(scene) -> PsxSceneDesc:
    """Build a psx_scene_desc that points into ``scene.arrays`` (kept alive by the caller)."""
    a = scene.arrays
    d = PsxSceneDesc()
    for name, ty in PsxSceneDesc._fields_:
        if name in a:
            arr = a[name]
            assert arr.flags["C_CONTIGUOUS"], name
            ptr_t = _PTR_TYPES[arr.dtype.type]
            setattr(d, name, arr.ctypes.data_as(ptr_t))
    d.n_bodies = len(a["pos"])
    d.n_colliders = len(a["col_type"])
    d.n_convex = len(a["convex_vert_start"]) - 1
    d.n_trimesh = len(a["tri_vert_start"]) - 1
    d.n_joints = len(a["joint_type"])
    d.num_substeps = scene.num_substeps
    d.num_iterations = scene.num_iterations
    d.gravity = scene.gravity
    return d
