"""Python face of the GB300 simulation hot path: ctypes over libpsx.so (include/psx.h).

``World`` mirrors physecs::Scene (Physecs include/Physecs/Physecs.h:199-229) for one
or many scenes: ``step(dt)`` is ``simulate(dt)``, ``set_knobs`` is
setNumSubSteps / setNumIterations / setGravity, and body state moves between host
arrays and device memory explicitly, the way the reference reads and writes its
EnTT components.  There is no CPU fallback: if the CUDA library is missing or no
GPU is present, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .desc import PsxSceneDesc, make_desc

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libpsx.so")

PSX_STATUS = {0: "OK", 1: "INVALID_ARG", 2: "OUT_OF_MEMORY", 3: "CAPACITY", 4: "TIMEOUT", 5: "CUDA", 6: "NOT_READY"}
EXPORTS = ["psx_world_create", "psx_world_destroy", "psx_world_step", "psx_world_step_timed", "psx_world_synchronize", "psx_world_set_knobs",
           "psx_world_read_bodies", "psx_world_write_bodies", "psx_world_simulate_host", "psx_world_counts",
           "psx_world_get_pairs", "psx_world_get_contacts", "psx_world_get_bounds", "psx_last_error_string",
           "psx_scene_create", "psx_scene_destroy", "psx_scene_simulate", "psx_world_read_bodies_noalloc",
           "psx_server_create", "psx_server_destroy", "psx_server_admit", "psx_server_tick", "psx_server_read",
           "psx_server_release", "psx_server_stats", "psx_server_tick_begin", "psx_server_tick_end", "psx_server_world",
           "psx_server_tick_stages", "psx_server_device_bytes", "psx_server_trigger_events",
           "psx_world_tune", "psx_world_launch_config", "psx_world_raycast", "psx_world_overlap",
           "psx_world_overlap_mtd", "psx_world_trigger_events", "psx_trimesh_build", "psx_world_update_trimesh",
           "psx_world_apply_deltas", "psx_world_move_characters", "psx_world_set_contact_filter",
           "psx_world_set_can_collide", "psx_world_narrow_counts", "psx_pin_host", "psx_unpin_host", "psx_world_set_wait_limit",
           "psx_world_set_joint_params", "psx_world_recreate"]

_lib = None


class PsxError(RuntimeError):
    pass


LAUNCH_FIELDS = ["convex_warps", "convex_blocks_per_sm", "analytic_threads", "analytic_blocks_per_sm",
                 "contacts_threads", "solver_smem_kb", "large_scene_solver",
                 "gjk_blocks_per_sm", "epa_lanes", "solver_threads_min", "epa_full_only", "large_threads"]


class PsxLaunchConfig(C.Structure):
    _fields_ = [(n, C.c_int32) for n in LAUNCH_FIELDS]


class PsxWorldOpts(C.Structure):
    _fields_ = [("pairs_per_collider", C.c_int32), ("manifolds_per_collider", C.c_int32),
                ("block_scene_max_dyn", C.c_int32), ("use_graph", C.c_int32), ("device", C.c_int32),
                ("launch", C.c_void_p)]


class PsxSceneCarry(C.Structure):
    _fields_ = [("from_scene", C.c_int32), ("collider_from", C.c_void_p), ("joint_from", C.c_void_p),
                ("joint_color", C.c_void_p)]


class PsxServerOpts(C.Structure):
    _fields_ = [("n_classes", C.c_int32), ("class_bodies", C.c_void_p), ("class_slots", C.c_void_p),
                ("mesh_pool", C.c_void_p), ("pairs_per_collider", C.c_int32), ("manifolds_per_collider", C.c_int32),
                ("device", C.c_int32), ("eager", C.c_int32), ("profile", C.c_int32),
                ("hbm_budget", C.c_int64), ("launch", C.c_void_p), ("triggers", C.c_int32)]


def load():
    """Load libpsx.so (building it first when this checkout has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import _build
        _build.build()
    lib = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    lib.psx_world_create.argtypes = [C.POINTER(PsxSceneDesc), C.c_int32, C.POINTER(PsxWorldOpts), C.POINTER(vp)]
    lib.psx_world_destroy.argtypes = [vp]
    lib.psx_world_step.argtypes = [vp, C.c_float, C.c_int32]
    lib.psx_world_synchronize.argtypes = [vp]
    lib.psx_world_set_wait_limit.argtypes = [vp, C.c_int64]
    lib.psx_world_set_joint_params.argtypes = [vp, C.c_int32, C.c_int32, vp]
    lib.psx_world_recreate.argtypes = [vp, C.POINTER(PsxSceneDesc), C.c_int32, C.POINTER(PsxSceneCarry), C.POINTER(vp)]
    lib.psx_world_set_knobs.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.c_float]
    lib.psx_world_read_bodies.argtypes = [vp, vp, vp, vp, vp]
    lib.psx_world_write_bodies.argtypes = [vp, vp, vp, vp, vp]
    lib.psx_world_read_bodies_noalloc.argtypes = [vp, vp, vp, vp, vp]
    lib.psx_world_simulate_host.argtypes = [vp, C.c_float, vp, vp, vp, vp]
    lib.psx_world_counts.argtypes = [vp, vp]
    lib.psx_world_narrow_counts.argtypes = [vp, vp]
    lib.psx_world_step_timed.argtypes = [vp, C.c_float, C.c_int32, vp, vp, vp]
    lib.psx_world_get_pairs.argtypes = [vp, vp, C.c_int32]
    lib.psx_world_get_pairs.restype = C.c_int32
    lib.psx_world_get_contacts.argtypes = [vp, vp, vp, vp, C.c_int32]
    lib.psx_world_get_contacts.restype = C.c_int32
    lib.psx_world_get_bounds.argtypes = [vp, vp, C.c_int32]
    lib.psx_world_get_bounds.restype = C.c_int32
    lib.psx_last_error_string.restype = C.c_char_p
    lib.psx_server_create.argtypes = [C.POINTER(PsxServerOpts), C.POINTER(vp)]
    lib.psx_server_destroy.argtypes = [vp]
    lib.psx_server_admit.argtypes = [vp, C.POINTER(PsxSceneDesc), C.c_int32, C.c_float, vp]
    lib.psx_server_tick.argtypes = [vp, vp, C.c_int32, vp]
    lib.psx_server_tick_begin.argtypes = [vp]
    lib.psx_world_tune.argtypes = [vp, C.c_int32, vp]
    lib.psx_server_world.argtypes = [vp]
    lib.psx_server_world.restype = vp
    lib.psx_server_tick_end.argtypes = [vp, vp, C.c_int32, vp]
    lib.psx_server_read.argtypes = [vp, C.c_int32, vp, vp, vp, vp]
    lib.psx_server_release.argtypes = [vp, C.c_int32]
    lib.psx_world_trigger_events.argtypes = [vp, vp, C.c_int32, vp, vp]
    lib.psx_server_trigger_events.argtypes = [vp, vp, C.c_int32, vp, vp]
    lib.psx_trimesh_build.argtypes = [C.c_int32, vp, C.c_int32, vp, C.c_int32, vp, vp, vp]
    lib.psx_world_update_trimesh.argtypes = [vp, C.c_int32, C.c_int32, vp]
    lib.psx_world_apply_deltas.argtypes = [vp, C.c_int32, vp]
    lib.psx_world_set_contact_filter.argtypes = [vp, vp]
    lib.psx_pin_host.argtypes = [vp, C.c_size_t]
    lib.psx_unpin_host.argtypes = [vp]
    lib.psx_world_set_can_collide.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    lib.psx_world_move_characters.argtypes = [vp, C.c_int32, vp, C.c_float, vp]
    lib.psx_server_stats.argtypes = [vp, vp]
    _lib = lib
    return lib


def _check(status):
    if status != 0:
        msg = load().psx_last_error_string().decode(errors="replace")
        raise PsxError("psx %s: %s" % (PSX_STATUS.get(status, status), msg))


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class World:
    """One or many scenes resident on the GPU, stepped together."""

    h = None

    def __init__(self, scenes, pairs_per_collider=0, manifolds_per_collider=0, block_scene_max_dyn=0, use_graph=False,
                 device=0, launch=None):
        """launch: dict of psx_launch_config fields (missing or 0: default shapes)."""
        lib = load()
        if not isinstance(scenes, (list, tuple)):
            scenes = [scenes]
        self.scenes = list(scenes)
        arr = (PsxSceneDesc * len(scenes))()
        for i, s in enumerate(scenes):
            arr[i] = make_desc(s)
        self._descs = arr
        self._launch = None
        if launch:
            self._launch = PsxLaunchConfig(*[int(launch.get(n, 0)) for n in LAUNCH_FIELDS])
        opts = PsxWorldOpts(pairs_per_collider, manifolds_per_collider, block_scene_max_dyn, 1 if use_graph else 0,
                            device, C.cast(C.pointer(self._launch), C.c_void_p) if self._launch is not None else None)
        h = C.c_void_p()
        _check(lib.psx_world_create(arr, len(scenes), C.byref(opts), C.byref(h)))
        self.h = h
        self.n_bodies = sum(len(s.arrays["pos"]) for s in scenes)
        self.body_start = np.cumsum([0] + [len(s.arrays["pos"]) for s in scenes])

    def close(self):
        if self.h:
            load().psx_world_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, dt=None, frames=1):
        dt = self.scenes[0].dt if dt is None else dt
        _check(load().psx_world_step(self.h, C.c_float(dt), frames))

    def step_timed(self, dt=None, frames=1):
        """Step `frames` frames timed with CUDA events on the world's stream.
        Returns (total_ms, stage_ms[5], kernels queued)."""
        dt = self.scenes[0].dt if dt is None else dt
        tot = np.zeros(1, np.float32)
        st = np.zeros(5, np.float32)
        k = np.zeros(1, np.int64)
        _check(load().psx_world_step_timed(self.h, C.c_float(dt), frames, _p(tot), _p(st), _p(k)))
        return float(tot[0]), st.astype(np.float64), int(k[0])

    def synchronize(self):
        _check(load().psx_world_synchronize(self.h))

    def recreate(self, scenes, carry):
        """psx_world_recreate: this world's scenes replaced by `scenes` (SceneData, their
        current state), carrying over, per scene, what carry[i] = {"from_scene", "collider_from",
        "joint_from", "joint_color"} maps (arrays, or None).  This World then holds the new
        world; the old one is destroyed."""
        lib = load()
        if not isinstance(scenes, (list, tuple)):
            scenes = [scenes]
        arr = (PsxSceneDesc * len(scenes))()
        for i, s in enumerate(scenes):
            arr[i] = make_desc(s)
        keep = []
        car = (PsxSceneCarry * len(scenes))()
        for i, c in enumerate(carry):
            fields = []
            for k in ("collider_from", "joint_from", "joint_color"):
                v = c.get(k)
                if v is None:
                    fields.append(None)
                else:
                    a = np.ascontiguousarray(v, np.int32)
                    keep.append(a)
                    fields.append(a.ctypes.data_as(C.c_void_p))
            car[i] = PsxSceneCarry(int(c.get("from_scene", -1)), *fields)
        h = C.c_void_p()
        _check(lib.psx_world_recreate(self.h, arr, len(scenes), car, C.byref(h)))
        lib.psx_world_destroy(self.h)
        self.h = h
        self.scenes = list(scenes)
        self._descs = arr
        self.n_bodies = sum(len(s.arrays["pos"]) for s in scenes)
        self.body_start = np.cumsum([0] + [len(s.arrays["pos"]) for s in scenes])

    def set_joint_params(self, joint, params, scene=0):
        """psx_world_set_joint_params: the 8-float parameter block of a scene's joint."""
        p = np.zeros(8, np.float32)
        p[:len(params)] = params
        _check(load().psx_world_set_joint_params(self.h, scene, joint, _p(p)))

    def set_wait_limit(self, polls):
        """psx_world_set_wait_limit: polls of a grid-barrier wait before it gives up
        (0: the default, about half a second)."""
        _check(load().psx_world_set_wait_limit(self.h, int(polls)))

    def tune(self, frames=2):
        """psx_world_tune: pick the kernels' launch shapes on this world's frames (they
        advance the world).  Returns the chosen configuration as a dict."""
        c = PsxLaunchConfig()
        _check(load().psx_world_tune(self.h, frames, C.byref(c)))
        return {n: int(getattr(c, n)) for n in LAUNCH_FIELDS}

    def launch_config(self):
        """psx_world_launch_config: the launch shapes in effect, as a dict."""
        c = PsxLaunchConfig()
        _check(load().psx_world_launch_config(self.h, C.byref(c)))
        return {n: int(getattr(c, n)) for n in LAUNCH_FIELDS}

    def set_knobs(self, substeps, iterations, gravity, scene=-1):
        _check(load().psx_world_set_knobs(self.h, scene, substeps, iterations, C.c_float(gravity)))

    def read_bodies(self):
        n = self.n_bodies
        st = dict(pos=np.zeros((n, 3), np.float32), quat=np.zeros((n, 4), np.float32),
                  vel=np.zeros((n, 3), np.float32), ang_vel=np.zeros((n, 3), np.float32))
        _check(load().psx_world_read_bodies(self.h, _p(st["pos"]), _p(st["quat"]), _p(st["vel"]), _p(st["ang_vel"])))
        return st

    def write_bodies(self, st):
        a = [np.ascontiguousarray(st[k], np.float32) for k in ("pos", "quat", "vel", "ang_vel")]
        _check(load().psx_world_write_bodies(self.h, *[_p(x) for x in a]))

    def simulate_host(self, dt, st):
        """End-to-end simulate through host buffers (upload, one frame, download) in place."""
        _check(load().psx_world_simulate_host(self.h, C.c_float(dt), _p(st["pos"]), _p(st["quat"]), _p(st["vel"]),
                                              _p(st["ang_vel"])))

    def counts(self):
        c = np.zeros(12, np.int32)
        _check(load().psx_world_counts(self.h, _p(c)))
        keys = ["bodies", "colliders", "dynamic", "joints", "scenes", "pairs", "manifolds", "error", "points", "rows",
                "simulated", "kernels"]
        return dict(zip(keys, (int(v) for v in c)))

    def narrow_counts(self):
        """psx_world_narrow_counts: the last frame's convex pairs and the EPA tiers they reached."""
        c = np.zeros(4, np.int32)
        _check(load().psx_world_narrow_counts(self.h, _p(c)))
        return dict(zip(["convex", "epa", "past_lane", "past_group"], (int(v) for v in c)))

    def pairs(self):
        n = self.counts()["pairs"]
        out = np.zeros((max(n, 1), 5), np.int32)
        m = load().psx_world_get_pairs(self.h, _p(out), len(out))
        return out[:m]

    def contacts(self):
        n = self.counts()["manifolds"]
        ids = np.zeros((max(n, 1), 8), np.int32)
        f = np.zeros((max(n, 1), 56), np.float32)
        meta = np.zeros((max(n, 1), 2), np.int32)
        m = load().psx_world_get_contacts(self.h, _p(ids), _p(f), _p(meta), len(ids))
        return ids[:m], f[:m], meta[:m]

    def bounds(self):
        n = self.counts()["colliders"]
        b = np.zeros((n, 6), np.float32)
        load().psx_world_get_bounds(self.h, _p(b), n)
        return b

    def raycast(self, rays, accept=None):
        """psx_world_raycast.  rays: (n, 8) float rows {scene, origin xyz, dir xyz, max
        distance}; accept: one value per world body (nonzero: the filter accepts its
        entity) or None for every entity.  Returns {body, collider, entity, distance, pos}
        arrays; body -1 where a ray hits nothing."""
        rays = np.asarray(rays, np.float64).reshape(-1, 8)
        n = len(rays)
        buf = np.zeros((n, 8), np.float32)
        buf[:, 1:] = rays[:, 1:]
        buf.view(np.int32)[:, 0] = rays[:, 0].astype(np.int32)
        out = np.zeros((max(n, 1), 7), np.float32)   # psx_ray_hit: 7 words
        acc = None if accept is None else np.ascontiguousarray(accept, np.uint8)
        _check(load().psx_world_raycast(self.h, n, _p(buf), _p(acc) if acc is not None else None, _p(out)))
        out = out[:n]
        iv = out.view(np.int32)
        return {"body": iv[:, 0].copy(), "collider": iv[:, 1].copy(), "entity": out.view(np.uint32)[:, 2].copy(),
                "distance": out[:, 3].copy(), "pos": out[:, 4:7].copy()}

    def overlap(self, queries, cap=64):
        """psx_world_overlap.  queries: list of dicts {scene, pos, quat, type, params,
        mesh (convex index within the scene), filter}.  Returns (counts, hits): hits[i] is
        a list of (body, collider, entity) for query i, at most cap of them."""
        n = len(queries)
        buf = self._shapes(queries)
        hits = np.zeros((max(n * cap, 1), 3), np.int32)
        counts = np.zeros(max(n, 1), np.int32)
        _check(load().psx_world_overlap(self.h, n, _p(buf), cap, _p(hits), _p(counts)))
        res = []
        for i in range(n):
            m = min(int(counts[i]), cap)
            res.append([(int(b), int(c), int(np.uint32(e))) for b, c, e in hits[i * cap:i * cap + m]])
        return counts[:n].copy(), res

    @staticmethod
    def _shapes(queries):
        n = len(queries)
        buf = np.zeros((max(n, 1), 14), np.float32)
        iv = buf.view(np.int32)
        for i, q in enumerate(queries):
            iv[i, 0] = q["scene"]
            buf[i, 1:4] = q["pos"]
            buf[i, 4:8] = q.get("quat", (0.0, 0.0, 0.0, 1.0))
            iv[i, 8] = q["type"]
            prm = list(q.get("params", (0.0, 0.0, 0.0))) + [0.0, 0.0, 0.0]
            buf[i, 9:12] = prm[:3]
            iv[i, 12] = q.get("mesh", -1)
            iv[i, 13] = q.get("filter", 0)
        return buf

    def overlap_mtd(self, queries, cap=64):
        """psx_world_overlap_mtd.  queries as overlap (the filter is not used).  Returns
        (counts, hits): hits[i] is a list of (body, collider, entity, normal (3,), mtd)."""
        n = len(queries)
        buf = self._shapes(queries)
        hits = np.zeros((max(n * cap, 1), 7), np.float32)   # psx_overlap_mtd_hit: 7 words
        counts = np.zeros(max(n, 1), np.int32)
        _check(load().psx_world_overlap_mtd(self.h, n, _p(buf), cap, _p(hits), _p(counts)))
        iv, uv = hits.view(np.int32), hits.view(np.uint32)
        res = []
        for i in range(n):
            m = min(int(counts[i]), cap)
            res.append([(int(iv[k, 0]), int(iv[k, 1]), int(uv[k, 2]), hits[k, 3:6].copy(), hits[k, 6])
                        for k in range(i * cap, i * cap + m)])
        return counts[:n].copy(), res

    def apply_deltas(self, deltas):
        """psx_world_apply_deltas: registry changes in array order, ahead of the next frame;
        deltas is pack_deltas' (n, 17) array or a list of its dicts."""
        d = pack_deltas(deltas) if isinstance(deltas, (list, tuple)) else np.ascontiguousarray(deltas, np.float32)
        _check(load().psx_world_apply_deltas(self.h, len(d), _p(d)))

    CONTACT_FILTER = C.CFUNCTYPE(C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32)

    def set_contact_filter(self, fn):
        """psx_world_set_contact_filter (Scene::setContactFilter): fn(is_trigger0, data0,
        is_trigger1, data1) -> 0 COLLISION / 1 TRIGGER, or None for the default filter."""
        self._filter = None if fn is None else self.CONTACT_FILTER(lambda a, b, c, d: int(fn(bool(a), b, bool(c), d)))
        _check(load().psx_world_set_contact_filter(self.h, C.cast(self._filter, C.c_void_p) if self._filter else None))

    def set_can_collide(self, body0, body1, can_collide, scene=0):
        """psx_world_set_can_collide (Scene::setCanCollide) for two bodies of one scene."""
        _check(load().psx_world_set_can_collide(self.h, scene, body0, body1, int(bool(can_collide))))

    def move_characters(self, chars, translations, dt=1.0 / 60.0):
        """psx_world_move_characters.  chars: dicts {scene, body, height, radius,
        max_step_height (0.3), slope_limit (cos 45 deg), iterations (2)}; translations: (n, 3).
        Returns the flags (n,) uint8."""
        n = len(chars)
        buf = np.zeros((max(n, 1), 10), np.float32)
        iv = buf.view(np.int32)
        t = np.asarray(translations, np.float32).reshape(-1, 3)
        for i, c in enumerate(chars):
            iv[i, 0], iv[i, 1] = c.get("scene", 0), c["body"]
            buf[i, 2], buf[i, 3] = c["height"], c["radius"]
            buf[i, 4], buf[i, 5] = c.get("max_step_height", 0.3), c.get("slope_limit", 0.70710677)
            iv[i, 6] = c.get("iterations", 2)
            buf[i, 7:10] = t[i]
        flags = np.zeros(max(n, 1), np.uint8)
        _check(load().psx_world_move_characters(self.h, n, _p(buf), C.c_float(dt), _p(flags)))
        return flags[:n]

    def update_trimesh(self, scene, mesh, vertices):
        """psx_world_update_trimesh: new vertices (same count) for triangle mesh `mesh` of
        `scene`, its BVH rebuilt on the device and its colliders' bounds recomputed."""
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        _check(load().psx_world_update_trimesh(self.h, scene, mesh, _p(v)))

    # ---------------------------------------------------------------- trigger events

    def trigger_events(self, cap=4096):
        """psx_world_trigger_events until the queue is empty.  Returns (events, lost):
        events is an (n, 9) int64 array of (frame, kind 0 enter / 1 exit, scene, body0,
        collider0, body1, collider1, entity0, entity1) in delivery order; lost counts the
        events dropped because the device log overflowed between two drains."""
        return _drain_events(load().psx_world_trigger_events, self.h, cap)

    def _listeners(self, kind, scene):
        if not hasattr(self, "_trigger_listeners"):
            self._trigger_listeners = ({}, {})
        return self._trigger_listeners[kind].setdefault(scene, [])

    def add_on_trigger_enter_callback(self, listener, scene=0):
        """Scene::addOnTriggerEnterCallback (src/Physecs.cpp:772-774) for one scene of the
        world: listener.on_trigger_enter(entity0, collider_index0, entity1, collider_index1)
        runs for each pair of that scene that starts to overlap, from dispatch_trigger_events."""
        self._listeners(0, scene).append(listener)

    def add_on_trigger_exit_callback(self, listener, scene=0):
        """Scene::addOnTriggerExitCallback (src/Physecs.cpp:776-778): listener.on_trigger_exit(...)."""
        self._listeners(1, scene).append(listener)

    def remove_on_trigger_enter_callback(self, listener, scene=0):
        """Scene::removeOnTriggerEnterCallback (src/Physecs.cpp:780-782); ValueError if absent."""
        self._listeners(0, scene).remove(listener)

    def remove_on_trigger_exit_callback(self, listener, scene=0):
        """Scene::removeOnTriggerExitCallback (src/Physecs.cpp:784-786); ValueError if absent."""
        self._listeners(1, scene).remove(listener)

    def dispatch_trigger_events(self):
        """Drains the trigger events and calls the listeners as Scene::simulate does at the
        end of each frame (src/Physecs.cpp:537-552): frame by frame, every entering pair
        calls every enter listener of its scene in registration order, then every exiting
        pair every exit listener.  Returns the drained events (see trigger_events); raises
        PsxError after the dispatch when events were lost to the device log's capacity."""
        ev, lost = self.trigger_events()
        for _frame, kind, scene, _b0, c0, _b1, c1, e0, e1 in ev.tolist():
            for ls in list(self._listeners(kind, scene)):
                if kind == 0:
                    ls.on_trigger_enter(e0, c0, e1, c1)
                else:
                    ls.on_trigger_exit(e0, c0, e1, c1)
        if lost:
            raise PsxError("psx CAPACITY: %d trigger events were lost before this drain" % lost)
        return ev


def _drain_events(fn, h, cap):
    """Calls fn (psx_world_trigger_events or psx_server_trigger_events) until its queue is
    empty; returns the events as an (n, 9) int64 array and the count lost."""
    chunks, lost = [], 0
    out = np.zeros((cap, 9), np.int32)   # psx_trigger_event: 9 words
    n, nl = C.c_int32(), C.c_int64()
    while True:
        _check(fn(h, _p(out), cap, C.byref(n), C.byref(nl)))
        lost += nl.value
        ev = out[:n.value].astype(np.int64)
        ev[:, 7:9] = out[:n.value, 7:9].view(np.uint32)
        chunks.append(ev)
        if n.value < cap:
            break
    return np.concatenate(chunks), lost


class Server:
    """Continuous batching of scene requests (psx_server_*): admit, tick, read, release.

    classes: [(bodies per slot, slots)] in ascending size; mesh_pool: a scene whose
    convex meshes the requests may use; triggers: the requests' trigger colliders raise
    events (trigger_events)."""

    h = None

    def __init__(self, classes, mesh_pool=None, device=0, pairs_per_collider=0, manifolds_per_collider=0, eager=False,
                 profile=False, hbm_budget=0, launch=None, triggers=False):
        lib = load()
        self._cb = np.ascontiguousarray([c[0] for c in classes], np.int32)
        self._cs = np.ascontiguousarray([c[1] for c in classes], np.int32)
        self._pool_scene = mesh_pool
        self._pool = make_desc(mesh_pool) if mesh_pool is not None else None
        opts = PsxServerOpts(len(classes), self._cb.ctypes.data, self._cs.ctypes.data,
                             C.cast(C.pointer(self._pool), C.c_void_p) if self._pool is not None else None,
                             pairs_per_collider, manifolds_per_collider, device, 1 if eager else 0,
                             1 if profile else 0, int(hbm_budget), None, 1 if triggers else 0)
        if launch:
            self._launch = PsxLaunchConfig(*[int(launch.get(n, 0)) for n in LAUNCH_FIELDS])
            opts.launch = C.cast(C.pointer(self._launch), C.c_void_p)
        h = C.c_void_p()
        _check(lib.psx_server_create(C.byref(opts), C.byref(h)))
        self.h = h
        self.n_bodies = {}
        self._caps = [int(c[0]) for c in classes]
        self._free = [int(c[1]) for c in classes]
        self._cls = {}

    def close(self):
        if self.h:
            load().psx_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def admit(self, scene, frames, dt=None, desc=None):
        """Returns the slot, or None when no free slot fits (PSX_ERR_CAPACITY).  desc: the
        scene's psx_scene_desc when the caller has built it already."""
        dt = scene.dt if dt is None else dt
        need = max(len(scene.arrays["pos"]), len(scene.arrays["col_type"]) - 1)
        cls = next((c for c, cap in enumerate(self._caps) if cap >= need and self._free[c] > 0), None)
        if cls is None:
            return None          # the library would answer PSX_ERR_CAPACITY; skip the call
        d = make_desc(scene) if desc is None else desc
        slot = C.c_int32(-1)
        st = load().psx_server_admit(self.h, C.byref(d), frames, C.c_float(dt), C.byref(slot))
        if st == 3:
            return None
        _check(st)
        self._free[cls] -= 1
        self._cls[slot.value] = cls
        self.n_bodies[slot.value] = len(scene.arrays["pos"])
        return slot.value

    def tick(self):
        """One frame of every running request; returns the slots that finished."""
        self.tick_begin()
        return self.tick_end()

    def tick_begin(self):
        """Upload the requests admitted since the last tick and launch a frame (no wait)."""
        _check(load().psx_server_tick_begin(self.h))

    def tick_end(self):
        """Wait for the frame in flight; returns the slots that finished."""
        done = np.zeros(max(1, len(self.n_bodies) + 64), np.int32)
        n = C.c_int32(0)
        _check(load().psx_server_tick_end(self.h, _p(done), len(done), C.byref(n)))
        if n.value > len(done):
            raise PsxError("tick: more finished slots than the result buffer holds")
        return done[:n.value].tolist()

    def read(self, slot):
        n = self.n_bodies[slot]
        st = dict(pos=np.zeros((n, 3), np.float32), quat=np.zeros((n, 4), np.float32),
                  vel=np.zeros((n, 3), np.float32), ang_vel=np.zeros((n, 3), np.float32))
        _check(load().psx_server_read(self.h, slot, _p(st["pos"]), _p(st["quat"]), _p(st["vel"]), _p(st["ang_vel"])))
        return st

    def release(self, slot):
        _check(load().psx_server_release(self.h, slot))
        self.n_bodies.pop(slot, None)
        cls = self._cls.pop(slot, None)
        if cls is not None:
            self._free[cls] += 1

    def device_bytes(self):
        """psx_server_device_bytes: device memory the server holds."""
        out = np.zeros(1, np.int64)
        _check(load().psx_server_device_bytes(self.h, _p(out)))
        return int(out[0])

    def tick_stages(self):
        """psx_server_tick_stages (servers made with profile=True): the last finished tick's
        stage times in ms: uploads, broadphase, narrowphase, rows, solver, bounds."""
        out = np.zeros(6, np.float32)
        _check(load().psx_server_tick_stages(self.h, _p(out)))
        return out

    def trigger_events(self, cap=4096):
        """psx_server_trigger_events until the queue is empty: (events, lost) as
        World.trigger_events gives them, with scene = the request's slot and frames, bodies,
        colliders and entities the request's own."""
        return _drain_events(load().psx_server_trigger_events, self.h, cap)

    def stats(self):
        out = np.zeros(6, np.int64)
        _check(load().psx_server_stats(self.h, _p(out)))
        return dict(zip(["running", "finished", "free", "bodies", "body_frames", "slots"], (int(v) for v in out)))


def trimesh_build(vertices, indices, device=0):
    """psx_trimesh_build: physecs::TriangleMesh(vertices, indices) built on the GPU.
    Returns (triangles (n, 20) uint32 words, nodes (m, 8) uint32 words) in the
    psx_trimesh_triangle / psx_trimesh_node layouts."""
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    ix = np.ascontiguousarray(indices, np.uint32).ravel()
    nt = len(ix) // 3
    tris = np.zeros((max(nt, 1), 20), np.uint32)
    nodes = np.zeros((max(1, 2 * nt - 1), 8), np.uint32)
    n = C.c_int32()
    _check(load().psx_trimesh_build(device, _p(v), len(v), _p(ix), len(ix), _p(tris), _p(nodes), C.byref(n)))
    return tris[:nt], nodes[:n.value]


DELTA_POSE, DELTA_VELOCITY, DELTA_KINEMATIC = 1, 2, 4


def pack_deltas(deltas):
    """psx_body_delta records, (n, 17) float32 (int fields as their bits), from dicts
    {scene, body, pos + quat (a patched pose), vel + ang_vel (written velocities),
    kinematic (Scene::setIsKinematic)}; absent keys leave that part out."""
    out = np.zeros((len(deltas), 17), np.float32)
    iv = out.view(np.int32)
    for i, d in enumerate(deltas):
        mask = 0
        iv[i, 0], iv[i, 1] = d.get("scene", 0), d["body"]
        if d.get("pos") is not None:
            mask |= DELTA_POSE
            out[i, 4:7], out[i, 7:11] = d["pos"], d.get("quat", (0.0, 0.0, 0.0, 1.0))
        if d.get("vel") is not None:
            mask |= DELTA_VELOCITY
            out[i, 11:14], out[i, 14:17] = d["vel"], d.get("ang_vel", (0.0, 0.0, 0.0))
        if d.get("kinematic") is not None:
            mask |= DELTA_KINEMATIC
            iv[i, 3] = int(bool(d["kinematic"]))
        iv[i, 2] = mask
    return out


def pin_host(*arrays):
    """psx_pin_host for numpy arrays (e.g. the dict of read_bodies), so that the body
    copies of read_bodies / write_bodies / simulate_host run at the host link's speed.
    Release them with unpin_host before they are freed."""
    for a in arrays:
        _check(load().psx_pin_host(a.ctypes.data_as(C.c_void_p), a.nbytes))


def unpin_host(*arrays):
    for a in arrays:
        _check(load().psx_unpin_host(a.ctypes.data_as(C.c_void_p)))
