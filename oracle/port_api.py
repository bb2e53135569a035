"""ctypes access to the CPU oracle (oracle/_build/liborc.so).

ORACLE (test infrastructure only): imported by tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg, never by the physecs_gb300 product.  The
interface mirrors oracle/ref/ref_api.RefScene so restatement and reference
can be compared call for call.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liborc.so")
_lib = None


def build():
    from oracle.build_oracle import build as _b
    return _b()


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = C.CDLL(LIB)
        p = "orc_scene_"
        getattr(_lib, p + "create").restype = C.c_void_p
        getattr(_lib, p + "create").argtypes = [C.c_void_p]
        getattr(_lib, p + "destroy").argtypes = [C.c_void_p]
        getattr(_lib, p + "step").argtypes = [C.c_void_p, C.c_float]
        getattr(_lib, p + "set_knobs").argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float]
        for fn in ("read", "write"):
            getattr(_lib, p + fn).argtypes = [C.c_void_p] + [C.c_void_p] * 4
        getattr(_lib, p + "pairs").argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        getattr(_lib, p + "bounds").argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        getattr(_lib, p + "contacts").argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        getattr(_lib, p + "collide").argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        getattr(_lib, p + "joint_colors").argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        _lib.orc_collider_bounds.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        _lib.orc_scene_set_contact_order.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        _lib.orc_scene_order_error.argtypes = [C.c_void_p]
        _lib.orc_scene_contact_keys.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        _lib.orc_scene_raycast.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_scene_overlap.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int]
        _lib.orc_scene_overlap_mtd.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                               C.c_int]
        _lib.orc_scene_trigger_events.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        _lib.orc_trimesh_build.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        _lib.orc_scene_apply_deltas.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        _lib.orc_scene_create_body.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_scene_destroy_body.argtypes = [C.c_void_p, C.c_int]
        _lib.orc_scene_add_collider.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        _lib.orc_scene_clear_colliders.argtypes = [C.c_void_p, C.c_int]
        _lib.orc_scene_create_joint.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        _lib.orc_scene_destroy_joint.argtypes = [C.c_void_p, C.c_int]
        _lib.orc_scene_set_joint_params.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        _lib.orc_scene_set_contact_filter.argtypes = [C.c_void_p, C.c_void_p]
        _lib.orc_scene_set_can_collide.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
        _lib.orc_character_move.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                                            C.c_void_p]
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class OracleScene:
    """The CPU restatement of physecs::Scene::simulate over a SceneData."""

    h = None

    def __init__(self, scene):
        from physecs_gb300.desc import make_desc
        self.scene = scene
        self._desc = make_desc(scene)
        self.h = lib().orc_scene_create(C.byref(self._desc))
        self.n = len(scene.arrays["pos"])

    def close(self):
        if self.h:
            lib().orc_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def step(self, dt=None, frames=1):
        dt = self.scene.dt if dt is None else dt
        for _ in range(frames):
            lib().orc_scene_step(self.h, dt)

    def set_knobs(self, substeps, iterations, gravity):
        lib().orc_scene_set_knobs(self.h, substeps, iterations, gravity)

    def state(self):
        n = self.n
        pos, quat = np.zeros((n, 3), np.float32), np.zeros((n, 4), np.float32)
        vel, ang = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)
        lib().orc_scene_read(self.h, _p(pos), _p(quat), _p(vel), _p(ang))
        return dict(pos=pos, quat=quat, vel=vel, ang_vel=ang)

    def write_state(self, st):
        arrs = [np.ascontiguousarray(st[k], np.float32) for k in ("pos", "quat", "vel", "ang_vel")]
        lib().orc_scene_write(self.h, *[_p(a) for a in arrs])

    def pairs(self):
        cap = 1 << 16
        while True:
            out = np.zeros((cap, 4), np.int32)
            n = lib().orc_scene_pairs(self.h, _p(out), cap)
            if n <= cap:
                return out[:n]
            cap = n

    def bounds(self):
        cap = self.scene.arrays["col_type"].size
        ids = np.zeros((cap, 2), np.int32)
        b = np.zeros((cap, 6), np.float32)
        n = lib().orc_scene_bounds(self.h, _p(ids), _p(b), cap)
        return ids[:n], b[:n]

    def contacts(self):
        cap = 1 << 16
        while True:
            ids = np.zeros((cap, 4), np.int32)
            f = np.zeros((cap, 56), np.float32)
            n = lib().orc_scene_contacts(self.h, _p(ids), _p(f), cap)
            if n <= cap:
                return ids[:n], f[:n]
            cap = n

    def raycast(self, rays, accept=None):
        """Scene::raycastClosest per ray; rays: (n, 8) {unused, origin, dir, max distance};
        accept: per body (nonzero: accepted) or None.  Returns {body, collider, distance, pos}."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = len(rays)
        ids = np.zeros((max(n, 1), 2), np.int32)
        f = np.zeros((max(n, 1), 4), np.float32)
        acc = None if accept is None else np.ascontiguousarray(accept, np.uint8)
        lib().orc_scene_raycast(self.h, n, _p(rays), _p(acc) if acc is not None else None, _p(ids), _p(f))
        return {"body": ids[:n, 0].copy(), "collider": ids[:n, 1].copy(), "distance": f[:n, 0].copy(), "pos": f[:n, 1:4].copy()}

    def overlap(self, pos, quat, type_, params, mesh=-1, filt=0, cap=4096):
        """Scene::overlap for one shape: list of (body, collider) in collider order."""
        pose = np.ascontiguousarray(list(pos) + list(quat), np.float32)
        prm = np.ascontiguousarray((list(params) + [0.0, 0.0, 0.0])[:3], np.float32)
        out = np.zeros((cap, 2), np.int32)
        m = lib().orc_scene_overlap(self.h, _p(pose), int(type_), _p(prm), int(mesh), int(filt), _p(out), cap)
        return [tuple(map(int, r)) for r in out[:min(m, cap)]]

    def overlap_mtd(self, pos, quat, type_, params, mesh=-1, cap=4096):
        """Scene::overlapWithMinTranslationalDistance for one shape: list of
        (body, collider, normal (3,), mtd)."""
        pose = np.ascontiguousarray(list(pos) + list(quat), np.float32)
        prm = np.ascontiguousarray((list(params) + [0.0, 0.0, 0.0])[:3], np.float32)
        ids = np.zeros((cap, 2), np.int32)
        f = np.zeros((cap, 4), np.float32)
        m = lib().orc_scene_overlap_mtd(self.h, _p(pose), int(type_), _p(prm), int(mesh), _p(ids), _p(f), cap)
        return [(int(ids[k, 0]), int(ids[k, 1]), f[k, :3].copy(), f[k, 3]) for k in range(min(m, cap))]

    FILTER = C.CFUNCTYPE(C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32)

    def set_contact_filter(self, fn):
        """Scene::setContactFilter: fn(is_trigger0, data0, is_trigger1, data1) -> 0 COLLISION /
        1 TRIGGER, or None for the default filter."""
        self._filter = None if fn is None else self.FILTER(lambda a, b, c, d: int(fn(bool(a), b, bool(c), d)))
        lib().orc_scene_set_contact_filter(self.h, C.cast(self._filter, C.c_void_p) if self._filter else None)

    def set_can_collide(self, body0, body1, can_collide):
        lib().orc_scene_set_can_collide(self.h, int(body0), int(body1), int(bool(can_collide)))

    def move_character(self, body, height, radius, translation, max_step_height=0.3, slope_limit=0.70710677,
                       iterations=2):
        """CharacterController::move for `body`; returns its CharacterCollisionFlags value."""
        t = np.ascontiguousarray(translation, np.float32)
        return lib().orc_character_move(self.h, int(body), height, radius, max_step_height, slope_limit, int(iterations),
                                        _p(t))

    def create_body(self, body_scene):
        """A new entity from the single body of `body_scene` (a SceneData whose meshes
        are not used: collider mesh indices refer to this scene's).  Returns (body index,
        entity value)."""
        from physecs_gb300.desc import make_desc
        d = make_desc(body_scene)
        ent = C.c_uint32()
        b = lib().orc_scene_create_body(self.h, C.byref(d), C.byref(ent))
        self.n = max(self.n, b + 1)
        return b, ent.value

    def create_joint(self, jtype, body0, body1, frames, params=None):
        """Scene::createJoint between frames: frames = 14 floats (anchor 0 position and
        orientation, anchor 1 position and orientation), params = 8 floats.  Returns the
        joint index."""
        f = np.ascontiguousarray(frames, np.float32).ravel()
        p = np.zeros(8, np.float32) if params is None else np.ascontiguousarray(params, np.float32).ravel()
        return lib().orc_scene_create_joint(self.h, int(jtype), int(body0), int(body1), _p(f), _p(p))

    def set_joint_params(self, j, params):
        """The joint classes' setters: joint j's 8-float parameter block is replaced."""
        p = np.zeros(8, np.float32)
        p[:len(params)] = params
        lib().orc_scene_set_joint_params(self.h, int(j), _p(p))

    def destroy_joint(self, j):
        """Scene::destroyJoint of joint j."""
        lib().orc_scene_destroy_joint(self.h, int(j))

    def add_collider(self, body, collider_scene):
        """Scene::addCollider: the first collider of `collider_scene` (a SceneData; its
        mesh indices refer to this scene's meshes) joins body `body`."""
        from physecs_gb300.desc import make_desc
        d = make_desc(collider_scene)
        lib().orc_scene_add_collider(self.h, int(body), C.byref(d))

    def clear_colliders(self, body):
        """Scene::clearColliders of body `body`."""
        lib().orc_scene_clear_colliders(self.h, int(body))

    def destroy_body(self, b):
        """registry.destroy of body b's entity; its state then reads as zeros."""
        lib().orc_scene_destroy_body(self.h, int(b))

    def apply_deltas(self, deltas):
        """Registry deltas in array order: a (n, 17) float32 array in psx_body_delta layout
        (physecs_gb300.api.pack_deltas)."""
        d = np.ascontiguousarray(deltas, np.float32)
        lib().orc_scene_apply_deltas(self.h, len(d), _p(d))

    def trigger_events(self):
        """Drain the trigger events of the frames stepped so far: an (n, 6) int32 array of
        (frame, kind 0 enter / 1 exit, body0, collider0, body1, collider1), in step order."""
        out = np.zeros((0, 6), np.int32)
        n = lib().orc_scene_trigger_events(self.h, None, 0)
        if n:
            out = np.zeros((n, 6), np.int32)
            lib().orc_scene_trigger_events(self.h, _p(out), n)
        return out

    def collide(self, pairs):
        pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 4)
        cap = max(16, 8 * len(pairs))
        while True:
            ids = np.zeros((cap, 4), np.int32)
            f = np.zeros((cap, 28), np.float32)
            n = lib().orc_scene_collide(self.h, len(pairs), _p(pairs), _p(ids), _p(f), cap)
            if n <= cap:
                return ids[:n], f[:n]
            cap = n

    def joint_colors(self):
        cap = max(1, len(self.scene.arrays["joint_type"]))
        out = np.zeros((cap, 2), np.int32)
        n = lib().orc_scene_joint_colors(self.h, _p(out), cap)
        return out[:n]

    def set_contact_order(self, keys):
        """Solve the next step's contacts in this order (rows {e0, c0, e1, c1, tri})."""
        k = np.ascontiguousarray(keys, np.int32).reshape(-1, 5)
        self._order_keys = k
        lib().orc_scene_set_contact_order(self.h, len(k), _p(k))

    def order_error(self):
        return lib().orc_scene_order_error(self.h)

    def contact_keys(self):
        cap = 1 << 16
        while True:
            out = np.zeros((cap, 5), np.int32)
            n = lib().orc_scene_contact_keys(self.h, _p(out), cap)
            if n <= cap:
                return out[:n]
            cap = n


def trimesh_build(verts, indices):
    """TriangleMesh(vertices, indices) of the restatement: (triangles (n, 20) uint32 words,
    nodes (m, 8) uint32 words) in psx_trimesh_triangle / psx_trimesh_node layout."""
    v = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
    ix = np.ascontiguousarray(indices, np.uint32).ravel()
    nt = len(ix) // 3
    tris = np.zeros((max(nt, 1), 20), np.uint32)
    nodes = np.zeros((max(1, 2 * nt - 1), 8), np.uint32)
    n = lib().orc_trimesh_build(_p(v), len(v), _p(ix), len(ix), _p(tris), _p(nodes))
    return tris[:nt], nodes[:n]
