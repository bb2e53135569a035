"""A host-side mirror of a scene through topology changes (test infrastructure).

The oracle edits its scene in place (OracleScene.destroy_body / create_body / add_collider /
clear_colliders / create_joint / destroy_joint).  The device takes topology changes as a
new world built from the scene as it now is (psx_world_recreate), told which colliders and
joints continue from the old world.  SceneMirror applies the same edits to a description
of the scene and produces, after each batch of edits, that description (a SceneData with
the bodies' current state) and the carry maps.

Body indices follow the oracle's: a destroyed body keeps its index as an entity without
components (no colliders, static, zero state), and a created body takes the next index.
Joints are listed in creation order without the destroyed ones, which keeps each colour's
joints in the order the reference's colour lists hold them; their colours follow
Scene::addJoint / destroyJoint (src/Physecs.cpp:690-723): the lowest colour free at both
bodies, freed again when the joint is destroyed.
"""
from __future__ import annotations

import numpy as np

from physecs_gb300 import scenes

COL_KEYS = [("col_pos", 3), ("col_quat", 4), ("col_type", 1), ("col_params", 4), ("col_mesh", 1), ("col_material", 3),
            ("col_is_trigger", 1), ("col_enable_sim", 1), ("col_data", 1)]


def _colliders_of(a, b):
    out = []
    for c in range(a["collider_start"][b], a["collider_start"][b + 1]):
        out.append({k: np.array(a[k][c]).reshape(-1).copy() for k, _ in COL_KEYS})
    return out


class SceneMirror:
    def __init__(self, s):
        self.base = s
        a = s.arrays
        self.bodies = []
        for b in range(len(a["pos"])):
            cols = _colliders_of(a, b)
            prev = list(range(a["collider_start"][b], a["collider_start"][b + 1]))
            self.bodies.append({"entity": int(a["entity"][b]), "flags": int(a["flags"][b]), "inv_mass": float(a["inv_mass"][b]),
                                "com": a["com"][b].copy(), "inv_inertia": a["inv_inertia"][b].copy(),
                                "cols": cols, "prev": prev, "init": None})
        self.bits = np.zeros(len(a["pos"]), np.uint32)
        self.joints = []
        for j in range(len(a["joint_type"])):
            self._add_joint(int(a["joint_type"][j]), int(a["joint_body0"][j]), int(a["joint_body1"][j]),
                            a["joint_frames"][j].copy(), a["joint_params"][j].copy(), prev=j)

    def _add_joint(self, t, b0, b1, frames, params, prev=-1):
        u = int(self.bits[b0] | self.bits[b1]) & 0xff
        c = 0
        while u & (1 << c):
            c += 1
        self.bits[b0] |= 1 << c
        self.bits[b1] |= 1 << c
        self.joints.append({"type": t, "b0": b0, "b1": b1, "frames": np.asarray(frames, np.float32).ravel(),
                            "params": np.asarray(params, np.float32).ravel(), "color": c, "alive": True, "prev": prev})
        return len(self.joints) - 1

    # ---- the oracle's edits
    def destroy_body(self, b):
        B = self.bodies[b]
        B.update(flags=0, inv_mass=0.0, cols=[], prev=[], dead=True)

    def create_body(self, sp, entity):
        a = sp.arrays
        self.bodies.append({"entity": int(entity), "flags": int(a["flags"][0]), "inv_mass": float(a["inv_mass"][0]),
                            "com": a["com"][0].copy(), "inv_inertia": a["inv_inertia"][0].copy(),
                            "cols": _colliders_of(a, 0), "prev": [-1] * int(a["collider_start"][1]),
                            "init": {k: a[k][0].copy() for k in ("pos", "quat", "vel", "ang_vel")}})
        self.bits = np.append(self.bits, np.uint32(0))
        return len(self.bodies) - 1

    def add_collider(self, b, cs):
        self.bodies[b]["cols"] += _colliders_of(cs.arrays, 0)[:1]
        self.bodies[b]["prev"] += [-1]

    def clear_colliders(self, b):
        self.bodies[b]["cols"] = []
        self.bodies[b]["prev"] = []

    def create_joint(self, t, b0, b1, frames, params=None):
        return self._add_joint(t, b0, b1, frames, np.zeros(8, np.float32) if params is None else params)

    def destroy_joint(self, j):
        J = self.joints[j]
        if not J["alive"]:
            return
        J["alive"] = False
        self.bits[J["b0"]] &= ~np.uint32(1 << J["color"])
        self.bits[J["b1"]] &= ~np.uint32(1 << J["color"])

    # ---- the scene as it now is
    def build(self, state):
        """(SceneData, carry) for psx_world_recreate; `state` holds the current pose and
        velocities of the bodies the old world had (new bodies start from their own)."""
        n = len(self.bodies)
        a = {"entity": np.zeros(n, np.uint32), "flags": np.zeros(n, np.uint32), "pos": np.zeros((n, 3), np.float32),
             "quat": np.zeros((n, 4), np.float32), "vel": np.zeros((n, 3), np.float32),
             "ang_vel": np.zeros((n, 3), np.float32), "inv_mass": np.zeros(n, np.float32),
             "com": np.zeros((n, 3), np.float32), "inv_inertia": np.zeros((n, 9), np.float32),
             "collider_start": np.zeros(n + 1, np.int32)}
        cols, prev = [], []
        n_old = len(state["pos"])
        for b, B in enumerate(self.bodies):
            a["entity"][b] = B["entity"]
            a["flags"][b] = B["flags"]
            a["inv_mass"][b] = B["inv_mass"]
            a["com"][b] = B["com"]
            a["inv_inertia"][b] = B["inv_inertia"]
            if B.get("dead"):
                a["quat"][b] = (0, 0, 0, 1)
            elif b < n_old:
                for k in ("pos", "quat", "vel", "ang_vel"):
                    a[k][b] = state[k][b]
            else:
                for k in ("pos", "quat", "vel", "ang_vel"):
                    a[k][b] = B["init"][k]
            cols += B["cols"]
            prev += B["prev"]
            a["collider_start"][b + 1] = len(cols)
        for k, w in COL_KEYS:
            dt = self.base.arrays[k].dtype
            a[k] = (np.concatenate([c[k] for c in cols]).astype(dt).reshape(-1, w) if cols
                    else np.zeros((0, w), dt))
            if w == 1:
                a[k] = a[k].ravel()
        for k in ("convex_vert_start", "convex_verts", "convex_face_start", "face_index_start", "face_indices",
                  "face_normal", "face_centroid", "tri_vert_start", "tri_verts", "tri_index_start", "tri_indices"):
            a[k] = self.base.arrays[k]
        alive = [j for j, J in enumerate(self.joints) if J["alive"]]
        a["joint_type"] = np.array([self.joints[j]["type"] for j in alive], np.int32)
        a["joint_body0"] = np.array([self.joints[j]["b0"] for j in alive], np.int32)
        a["joint_body1"] = np.array([self.joints[j]["b1"] for j in alive], np.int32)
        a["joint_frames"] = np.array([self.joints[j]["frames"] for j in alive], np.float32).reshape(-1, 14)
        a["joint_params"] = np.array([self.joints[j]["params"] for j in alive], np.float32).reshape(-1, 8)
        carry = {"from_scene": 0, "collider_from": np.asarray(prev, np.int32),
                 "joint_from": np.array([self.joints[j]["prev"] for j in alive], np.int32),
                 "joint_color": np.array([self.joints[j]["color"] for j in alive], np.int32)}
        s = scenes.SceneData(self.base.name + "_edited")
        s.num_substeps, s.num_iterations, s.gravity, s.dt = (self.base.num_substeps, self.base.num_iterations,
                                                             self.base.gravity, self.base.dt)
        s.arrays = {k: np.ascontiguousarray(v) for k, v in a.items()}
        # the next build continues from this one
        k = 0
        for B in self.bodies:
            B["prev"] = list(range(k, k + len(B["cols"])))
            k += len(B["cols"])
        for i, j in enumerate(alive):
            self.joints[j]["prev"] = i
        return s, carry
