"""Seeded synthetic scenes for the Physecs simulation hot path.

Physecs publishes no benchmark data, so every workload here is generated from
a seed.  Random numbers come from SplitMix64 (Steele, Lea, Flood 2014) so the
same seed gives the same scene on every machine and numpy version:
    seed = 0x5EED0000 + config * 2**20 + scene_index.

A scene is a plain set of numpy arrays laid out like ``psx_scene_desc``
(include/psx.h), i.e. like the reference's EnTT registry: bodies in entity
creation order, each with a transform, colliders and optional dynamics
(include/Physecs/Components.h:6-17, src/Transform.h:6-10).

Mass properties follow physecs::computeCOMAndInvInertiaTensor
(src/MassUtil.cpp:73-183) evaluated in float64 and stored as float32; they are
scene inputs, so the reference and the GPU path read identical values.
"""
from __future__ import annotations

import math
import numpy as np

SPHERE, CAPSULE, BOX, CONVEX_MESH, TRIANGLE_MESH = 0, 1, 2, 3, 4
BODY_DYNAMIC, BODY_KINEMATIC = 1, 2
JOINT_FIXED, JOINT_REVOLUTE, JOINT_SPHERICAL, JOINT_PRISMATIC, JOINT_UNIVERSAL, JOINT_GEAR, JOINT_SERVO = range(7)
JOINT_PARAMS = 8
DENSITY = 1000.0
IDENTITY_Q = (0.0, 0.0, 0.0, 1.0)

_M64 = (1 << 64) - 1


class SplitMix64:
    """SplitMix64 stream; floats are (x >> 11) * 2**-53."""

    def __init__(self, seed: int):
        self.state = seed & _M64

    def next_u64(self, n: int) -> np.ndarray:
        inc = 0x9E3779B97F4A7C15
        k = np.arange(1, n + 1, dtype=np.uint64)
        with np.errstate(over="ignore"):
            z = np.uint64(self.state) + k * np.uint64(inc)
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
        self.state = (self.state + n * inc) & _M64
        return z

    def uniform(self, n: int, lo=0.0, hi=1.0) -> np.ndarray:
        u = (self.next_u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))
        return lo + (hi - lo) * u

    def normal(self, n: int) -> np.ndarray:
        m = (n + 1) // 2
        u1 = self.uniform(m)
        u2 = self.uniform(m)
        r = np.sqrt(-2.0 * np.log(np.maximum(u1, 1e-300)))
        z = np.concatenate([r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)])
        return z[:n]

    def quaternions(self, n: int) -> np.ndarray:
        """Uniform random rotations (Shoemake 1992), stored x, y, z, w."""
        u1, u2, u3 = self.uniform(n), self.uniform(n), self.uniform(n)
        a, b = np.sqrt(1.0 - u1), np.sqrt(u1)
        q = np.stack([a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2),
                      b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)], axis=1)
        return q


def scene_seed(config: int, index: int = 0) -> int:
    return 0x5EED0000 + config * (1 << 20) + index


# ----------------------------------------------------------------------------
# geometry assets
# ----------------------------------------------------------------------------

def convex_hull(points: np.ndarray):
    """Convex hull of a small point set by exhaustive facet search.

    Returns (vertices, faces) in ConvexMesh form (include/Physecs/ConvexMesh.h:7-34):
    vertices are the hull points, every face is a CCW (outward) triangle with its
    unit normal and centroid.  Points must be in general position (no four
    coplanar), which holds with probability one for random sphere samples.
    """
    p = np.asarray(points, dtype=np.float64)
    n = len(p)
    faces = []
    for i in range(n):
        for j in range(i + 1, n):
            for k in range(j + 1, n):
                nrm = np.cross(p[j] - p[i], p[k] - p[i])
                d = (p - p[i]) @ nrm
                d[[i, j, k]] = 0.0
                if np.all(d <= 1e-12):
                    faces.append((i, j, k))
                elif np.all(d >= -1e-12):
                    faces.append((i, k, j))
    used = sorted({v for f in faces for v in f})
    remap = {v: t for t, v in enumerate(used)}
    verts = p[used]
    out = []
    for f in faces:
        a, b, c = (remap[v] for v in f)
        nrm = np.cross(verts[b] - verts[a], verts[c] - verts[a])
        nrm /= np.linalg.norm(nrm)
        out.append(([a, b, c], nrm, (verts[a] + verts[b] + verts[c]) / 3.0))
    return verts, out


def box_hull(he):
    """A box as a ConvexMesh with quad faces (for box-vs-hull equivalence checks)."""
    hx, hy, hz = he
    v = np.array([[sx * hx, sy * hy, sz * hz] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)], dtype=np.float64)
    def idx(sx, sy, sz):
        return ((sx > 0) << 2) | ((sy > 0) << 1) | (sz > 0)
    quads = [
        ([idx(1, -1, -1), idx(1, 1, -1), idx(1, 1, 1), idx(1, -1, 1)], (1, 0, 0)),
        ([idx(-1, -1, -1), idx(-1, -1, 1), idx(-1, 1, 1), idx(-1, 1, -1)], (-1, 0, 0)),
        ([idx(-1, 1, -1), idx(-1, 1, 1), idx(1, 1, 1), idx(1, 1, -1)], (0, 1, 0)),
        ([idx(-1, -1, -1), idx(1, -1, -1), idx(1, -1, 1), idx(-1, -1, 1)], (0, -1, 0)),
        ([idx(-1, -1, 1), idx(1, -1, 1), idx(1, 1, 1), idx(-1, 1, 1)], (0, 0, 1)),
        ([idx(-1, -1, -1), idx(-1, 1, -1), idx(1, 1, -1), idx(1, -1, -1)], (0, 0, -1)),
    ]
    faces = [(q, np.array(nrm, dtype=np.float64), v[q].mean(axis=0)) for q, nrm in quads]
    return v, faces


def heightfield(rng: SplitMix64, cells=256, spacing=1.0, amplitude=4.0, lattice=16):
    """Value-noise terrain as a TriangleMesh: (cells+1)^2 vertices, 2*cells^2 triangles, CCW from +y."""
    nv = cells + 1
    coarse = cells // lattice + 2
    lat = rng.uniform(coarse * coarse, -1.0, 1.0).reshape(coarse, coarse)
    g = np.arange(nv) / lattice
    i0 = np.floor(g).astype(int)
    t = g - i0
    s = t * t * (3 - 2 * t)
    h = (lat[i0][:, i0] * np.outer(1 - s, 1 - s) + lat[i0 + 1][:, i0] * np.outer(s, 1 - s)
         + lat[i0][:, i0 + 1] * np.outer(1 - s, s) + lat[i0 + 1][:, i0 + 1] * np.outer(s, s))
    h = amplitude * h
    xs = (np.arange(nv) - cells / 2) * spacing
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    verts = np.stack([X.ravel(), h.ravel(), Z.ravel()], axis=1)
    i = np.arange(cells)
    I, J = np.meshgrid(i, i, indexing="ij")
    v00 = (I * nv + J).ravel()
    v10 = ((I + 1) * nv + J).ravel()
    v01 = (I * nv + J + 1).ravel()
    v11 = ((I + 1) * nv + J + 1).ravel()
    # (x,z) grid: +x along i, +z along j; CCW seen from +y means (a, b, c) with cross(b-a, c-a).y > 0
    t0 = np.stack([v00, v01, v10], axis=1)
    t1 = np.stack([v10, v01, v11], axis=1)
    idx = np.stack([t0, t1], axis=1).reshape(-1, 3)
    return verts.astype(np.float32), idx.astype(np.uint32), float(h.max())


# ----------------------------------------------------------------------------
# mass properties (src/MassUtil.cpp:7-183), single collider at the body origin
# ----------------------------------------------------------------------------

def mass_sphere(r):
    v = 4.0 * math.pi * r ** 3 / 3.0
    m = DENSITY * v
    i = 2.0 * m * r * r / 5.0
    return m, np.zeros(3), np.diag([i, i, i])


def mass_capsule(hh, r):
    vc = 2 * r * r * math.pi * hh
    vs = 4 * r ** 3 * math.pi / 3.0
    v = vc + vs
    m = DENSITY * v
    mc, ms = vc * m / v, vs * m / v
    ixx = mc * (hh * hh / 3.0 + r * r / 4.0) + ms * (hh * hh + 3.0 * hh * r / 4.0 + 2 * r * r / 5.0)
    iyy = mc * r * r / 2.0 + ms * 2 * r * r / 5.0
    return m, np.zeros(3), np.diag([ixx, iyy, ixx])


def mass_box(he):
    x, y, z = (float(e) for e in he)
    m = DENSITY * 8.0 * x * y * z
    k = m / 12.0
    return m, np.zeros(3), np.diag([k * (y * y + z * z), k * (x * x + z * z), k * (x * x + y * y)])


def _tet_inertia(mass, v):
    d = np.zeros(3)
    for i in range(4):
        for j in range(i + 1):
            d += v[j] * v[i]
    a, b, c = (d[1] + d[2]) / 10.0, (d[0] + d[2]) / 10.0, (d[0] + d[1]) / 10.0
    ap = bp = cp = 0.0
    for i in range(4):
        for j in range(4):
            mult = 2.0 if i == j else 1.0
            ap += mult * v[i][1] * v[j][2]
            bp += mult * v[i][0] * v[j][2]
            cp += mult * v[i][0] * v[j][1]
    ap, bp, cp = ap / 20.0, bp / 20.0, cp / 20.0
    I = np.array([[a, -bp, -cp], [-bp, b, -ap], [-cp, -ap, c]])
    return mass * I


def mass_convex(verts, faces, scale):
    sv = np.asarray(verts, dtype=np.float64) * np.asarray(scale, dtype=np.float64)
    center = sv.mean(axis=0)
    tets = []
    com = np.zeros(3)
    vol = 0.0
    for idx, _, _ in faces:
        v0 = sv[idx[0]]
        for i in range(1, len(idx) - 1):
            v1, v2 = sv[idx[i]], sv[idx[i + 1]]
            tv = abs(np.dot(np.cross(v0 - center, v1 - center), v2 - center)) / 6.0
            com += (center + v0 + v1 + v2) / 4.0 * tv
            vol += tv
            tets.append((tv, v0, v1, v2))
    com /= vol
    mass = DENSITY * vol
    I = np.zeros((3, 3))
    d = -com
    for tv, v0, v1, v2 in tets:
        I += _tet_inertia(mass * tv / vol, [center + d, v0 + d, v1 + d, v2 + d])
    return mass, com, I


# ----------------------------------------------------------------------------
# scene container
# ----------------------------------------------------------------------------

class SceneData:
    """Numpy arrays in psx_scene_desc layout (include/psx.h)."""

    def __init__(self, name="scene"):
        self.name = name
        self.num_substeps, self.num_iterations, self.gravity = 4, 8, 9.81
        self.dt = 1.0 / 60.0
        self._bodies = []     # list of dict chunks (vectorised)
        self._cols = []
        self.convex = []      # (verts (n,3), faces [(idx list, normal, centroid)])
        self.trimesh = []     # (verts (n,3), indices (k,))
        self._joints = []

    # bodies are appended in chunks to keep big scenes vectorised
    def add_bodies(self, pos, quat, flags, inv_mass, com, inv_inertia, col_type, col_params,
                   col_mesh=None, vel=None, ang_vel=None, material=(0.5, 0.0, 0.0),
                   col_pos=None, col_quat=None, enable_sim=None):
        n = len(pos)
        base = self.n_bodies
        zeros3 = np.zeros((n, 3))
        self._bodies.append(dict(
            pos=np.asarray(pos, np.float64).reshape(n, 3),
            quat=np.asarray(quat, np.float64).reshape(n, 4),
            flags=np.broadcast_to(np.asarray(flags, np.uint32), (n,)).copy(),
            inv_mass=np.broadcast_to(np.asarray(inv_mass, np.float64), (n,)).copy(),
            com=np.broadcast_to(np.asarray(com, np.float64), (n, 3)).copy(),
            inv_inertia=np.broadcast_to(np.asarray(inv_inertia, np.float64).reshape(-1, 9), (n, 9)).copy(),
            vel=zeros3 if vel is None else np.asarray(vel, np.float64).reshape(n, 3),
            ang_vel=zeros3 if ang_vel is None else np.asarray(ang_vel, np.float64).reshape(n, 3),
        ))
        mat = np.broadcast_to(np.asarray(material, np.float64), (n, 3)).copy()
        self._cols.append(dict(
            pos=np.zeros((n, 3)) if col_pos is None else np.broadcast_to(np.asarray(col_pos, np.float64), (n, 3)).copy(),
            quat=np.tile(np.asarray(IDENTITY_Q), (n, 1)) if col_quat is None else np.broadcast_to(np.asarray(col_quat, np.float64), (n, 4)).copy(),
            type=np.broadcast_to(np.asarray(col_type, np.int32), (n,)).copy(),
            params=np.broadcast_to(np.asarray(col_params, np.float64).reshape(-1, 4), (n, 4)).copy(),
            mesh=np.full(n, -1, np.int32) if col_mesh is None else np.broadcast_to(np.asarray(col_mesh, np.int32), (n,)).copy(),
            material=mat,
            enable=np.ones(n, np.uint8) if enable_sim is None else np.broadcast_to(np.asarray(enable_sim, np.uint8), (n,)).copy(),
        ))
        return base

    def add_joints(self, jtype, body0, body1, frames, params=None):
        n = len(body0)
        p = np.zeros((n, JOINT_PARAMS)) if params is None else np.asarray(params, np.float64).reshape(n, JOINT_PARAMS)
        self._joints.append(dict(type=np.broadcast_to(np.asarray(jtype, np.int32), (n,)).copy(),
                                 body0=np.asarray(body0, np.int32), body1=np.asarray(body1, np.int32),
                                 frames=np.asarray(frames, np.float64).reshape(n, 14), params=p))

    @property
    def n_bodies(self):
        return sum(len(c["pos"]) for c in self._bodies)

    def finalize(self):
        """Concatenate chunks into the flat float32 / int32 arrays of psx_scene_desc."""
        def cat(chunks, key, dtype):
            if not chunks:
                return np.zeros((0,), dtype)
            return np.ascontiguousarray(np.concatenate([c[key] for c in chunks]).astype(dtype))
        b, c, j = self._bodies, self._cols, self._joints
        a = {}
        a["pos"] = cat(b, "pos", np.float32)
        n = len(a["pos"])
        a["entity"] = np.arange(n, dtype=np.uint32)
        a["flags"] = cat(b, "flags", np.uint32)
        a["quat"] = cat(b, "quat", np.float32)
        a["vel"] = cat(b, "vel", np.float32)
        a["ang_vel"] = cat(b, "ang_vel", np.float32)
        a["inv_mass"] = cat(b, "inv_mass", np.float32)
        a["com"] = cat(b, "com", np.float32)
        a["inv_inertia"] = cat(b, "inv_inertia", np.float32)
        a["collider_start"] = np.arange(n + 1, dtype=np.int32)  # one collider per body
        a["col_pos"] = cat(c, "pos", np.float32)
        a["col_quat"] = cat(c, "quat", np.float32)
        a["col_type"] = cat(c, "type", np.int32)
        a["col_params"] = cat(c, "params", np.float32)
        a["col_mesh"] = cat(c, "mesh", np.int32)
        a["col_material"] = cat(c, "material", np.float32)
        a["col_enable_sim"] = cat(c, "enable", np.uint8)
        a["col_is_trigger"] = np.zeros(n, np.uint8)
        a["col_data"] = np.zeros(n, np.int32)
        # convex meshes
        vs, vstart, fstart, fis, fidx, fn, fc = [], [0], [0], [0], [], [], []
        for verts, faces in self.convex:
            vs.append(np.asarray(verts, np.float32))
            vstart.append(vstart[-1] + len(verts))
            for idx, nrm, cen in faces:
                fidx.extend(int(i) for i in idx)
                fis.append(len(fidx))
                fn.append(nrm)
                fc.append(cen)
            fstart.append(len(fn))
        a["convex_vert_start"] = np.asarray(vstart, np.int32)
        a["convex_verts"] = np.concatenate(vs).astype(np.float32) if vs else np.zeros((0, 3), np.float32)
        a["convex_face_start"] = np.asarray(fstart, np.int32)
        a["face_index_start"] = np.asarray(fis, np.int32)
        a["face_indices"] = np.asarray(fidx, np.int32)
        a["face_normal"] = np.asarray(fn, np.float32).reshape(-1, 3)
        a["face_centroid"] = np.asarray(fc, np.float32).reshape(-1, 3)
        # triangle meshes
        tv, tvs, ti, tis = [], [0], [], [0]
        for verts, idx in self.trimesh:
            tv.append(np.asarray(verts, np.float32))
            tvs.append(tvs[-1] + len(verts))
            ti.append(np.asarray(idx, np.uint32).ravel())
            tis.append(tis[-1] + ti[-1].size)
        a["tri_vert_start"] = np.asarray(tvs, np.int32)
        a["tri_verts"] = np.concatenate(tv).astype(np.float32) if tv else np.zeros((0, 3), np.float32)
        a["tri_index_start"] = np.asarray(tis, np.int32)
        a["tri_indices"] = np.concatenate(ti).astype(np.uint32) if ti else np.zeros(0, np.uint32)
        # joints
        a["joint_type"] = cat(j, "type", np.int32)
        a["joint_body0"] = cat(j, "body0", np.int32)
        a["joint_body1"] = cat(j, "body1", np.int32)
        a["joint_frames"] = cat(j, "frames", np.float32)
        a["joint_params"] = cat(j, "params", np.float32)
        for k, v in a.items():
            a[k] = np.ascontiguousarray(v)
        self.arrays = a
        return self

    @property
    def n_dynamic(self):
        f = self.arrays["flags"]
        return int(np.count_nonzero((f & BODY_DYNAMIC) & ~(f & BODY_KINEMATIC)))


def _inv3(I):
    return np.linalg.inv(I).T.ravel()  # column-major storage of inv(I)


# ----------------------------------------------------------------------------
# configs
# ----------------------------------------------------------------------------

def _ground_box(s: SceneData, he, top_y=0.0, material=(0.5, 0.0, 0.0)):
    return s.add_bodies(pos=[[0.0, top_y - he[1], 0.0]], quat=[IDENTITY_Q], flags=0, inv_mass=0.0,
                        com=np.zeros(3), inv_inertia=np.zeros(9), col_type=BOX,
                        col_params=[he[0], he[1], he[2], 0.0], material=material)


def pyramid(rows=20, half=0.5, gap=0.01, substeps=4, iterations=8, dt=1.0 / 60.0):
    """Config 1: a 2-D box pyramid in the x-y plane on a static 100x1x100 m ground box."""
    s = SceneData("pyramid%d" % rows)
    s.num_substeps, s.num_iterations, s.dt = substeps, iterations, dt
    _ground_box(s, (50.0, 0.5, 50.0))
    m, com, I = mass_box((half, half, half))
    pos = []
    pitch = 2 * half + gap
    for r in range(rows):
        n = rows - r
        for i in range(n):
            pos.append([(i - (n - 1) / 2.0) * pitch, half + r * pitch, 0.0])
    pos = np.asarray(pos)
    s.add_bodies(pos=pos, quat=np.tile(IDENTITY_Q, (len(pos), 1)), flags=BODY_DYNAMIC, inv_mass=1.0 / m,
                 com=com, inv_inertia=_inv3(I), col_type=BOX, col_params=[half, half, half, 0.0])
    return s.finalize()


def _hull_pool(rng: SplitMix64, count=32, points=16):
    pool = []
    for _ in range(count):
        p = rng.normal(points * 3).reshape(points, 3)
        p /= np.linalg.norm(p, axis=1, keepdims=True)
        pool.append(convex_hull(p))
    return pool


_HULL_UNIT = {}


def _hull_unit_props(mesh):
    """Unit-scale mass, COM and inverse inertia (column-major) of a pool hull; cached.
    The entry holds the mesh itself, so its id cannot be reused by another mesh while
    the entry lives."""
    key = id(mesh)
    hit = _HULL_UNIT.get(key)
    if hit is None or hit[0] is not mesh:
        verts, faces = mesh
        m, com, I = mass_convex(verts, faces, (1.0, 1.0, 1.0))
        hit = (mesh, (m, com, np.linalg.inv(I).T.ravel()))
        _HULL_UNIT[key] = hit
    return hit[1]


def _mixed_bodies(s: SceneData, rng: SplitMix64, centers: np.ndarray, hull_base: int, hull_pool,
                  mix=(0.4, 0.3, 0.2, 0.1), material=(0.5, 0.0, 0.0)):
    """Append len(centers) dynamic bodies with the config-2 shape mix and size distributions.

    Mass properties follow src/MassUtil.cpp for one collider at the body origin; a hull
    scaled uniformly by s has mass m1*s^3, COM com1*s and inertia I1*s^5."""
    n = len(centers)
    u = rng.uniform(n)
    c = np.cumsum(mix)
    kind = np.where(u < c[0], BOX, np.where(u < c[1], SPHERE, np.where(u < c[2], CAPSULE, CONVEX_MESH)))
    q = rng.quaternions(n)
    a, b, cc = rng.uniform(n), rng.uniform(n), rng.uniform(n)
    hp = (rng.next_u64(n) % np.uint64(len(hull_pool))).astype(np.int64)
    params = np.zeros((n, 4))
    mesh = np.full(n, -1, np.int32)
    inv_mass = np.zeros(n)
    com = np.zeros((n, 3))
    invI = np.zeros((n, 9))
    def diag_inv(sel, dx, dy, dz):
        invI[sel, 0], invI[sel, 4], invI[sel, 8] = 1.0 / dx, 1.0 / dy, 1.0 / dz
    sel = kind == BOX
    if sel.any():
        hx, hy, hz = 0.25 + 0.75 * a[sel], 0.25 + 0.75 * b[sel], 0.25 + 0.75 * cc[sel]
        params[sel, 0], params[sel, 1], params[sel, 2] = hx, hy, hz
        m = DENSITY * 8.0 * hx * hy * hz
        k = m / 12.0
        inv_mass[sel] = 1.0 / m
        diag_inv(sel, k * (hy * hy + hz * hz), k * (hx * hx + hz * hz), k * (hx * hx + hy * hy))
    sel = kind == SPHERE
    if sel.any():
        r = 0.25 + 0.5 * a[sel]
        params[sel, 0] = r
        m = DENSITY * 4.0 * math.pi * r ** 3 / 3.0
        i = 2.0 * m * r * r / 5.0
        inv_mass[sel] = 1.0 / m
        diag_inv(sel, i, i, i)
    sel = kind == CAPSULE
    if sel.any():
        r, hh = 0.2 + 0.3 * a[sel], 0.25 + 0.75 * b[sel]
        params[sel, 0], params[sel, 1] = hh, r
        vc = 2 * r * r * math.pi * hh
        vs = 4 * r ** 3 * math.pi / 3.0
        m = DENSITY * (vc + vs)
        mc, ms = vc * m / (vc + vs), vs * m / (vc + vs)
        ixx = mc * (hh * hh / 3.0 + r * r / 4.0) + ms * (hh * hh + 3.0 * hh * r / 4.0 + 2 * r * r / 5.0)
        iyy = mc * r * r / 2.0 + ms * 2 * r * r / 5.0
        inv_mass[sel] = 1.0 / m
        diag_inv(sel, ixx, iyy, ixx)
    for i in np.nonzero(kind == CONVEX_MESH)[0]:
        sc = 0.5 + a[i]
        params[i, :3] = sc
        h = int(hp[i])
        mesh[i] = hull_base + h
        m1, com1, inv1 = _hull_unit_props(hull_pool[h])
        inv_mass[i] = 1.0 / (m1 * sc ** 3)
        com[i] = com1 * sc
        invI[i] = inv1 / sc ** 5
    return s.add_bodies(pos=centers, quat=q, flags=BODY_DYNAMIC, inv_mass=inv_mass, com=com,
                        inv_inertia=invI, col_type=kind.astype(np.int32), col_params=params, col_mesh=mesh,
                        material=material)


def _jittered_grid(rng: SplitMix64, nx, ny, nz, pitch, base):
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    g = np.stack([ix.ravel() - (nx - 1) / 2.0, iy.ravel(), iz.ravel() - (nz - 1) / 2.0], axis=1) * pitch
    g = g + rng.uniform(g.size, -0.25, 0.25).reshape(g.shape)
    return g + np.asarray(base)


def large_mixed(n_bodies=65536, cells=256, seed=None):
    """Config 2: mixed shapes on a jittered 1.5 m grid above a value-noise heightfield."""
    rng = SplitMix64(scene_seed(2) if seed is None else seed)
    s = SceneData("large_mixed%d" % n_bodies)
    verts, idx, hmax = heightfield(rng, cells=cells)
    s.trimesh.append((verts, idx))
    s.add_bodies(pos=[[0.0, 0.0, 0.0]], quat=[IDENTITY_Q], flags=0, inv_mass=0.0, com=np.zeros(3),
                 inv_inertia=np.zeros(9), col_type=TRIANGLE_MESH, col_params=[0.0, 0.0, 0.0, 0.0], col_mesh=0)
    pool = _hull_pool(rng)
    s.convex.extend(pool)
    ny = max(1, int(round(n_bodies ** (1 / 3) / 2)))
    nxz = int(math.ceil(math.sqrt(n_bodies / ny)))
    centers = _jittered_grid(rng, nxz, ny, nxz, 1.5, [0.0, hmax + 6.0, 0.0])[:n_bodies]
    _mixed_bodies(s, rng, centers, 0, pool)
    return s.finalize()


def _chain(s: SceneData, rng: SplitMix64, anchor_body, anchor_pos, top, links, kinds, r=0.1, hh=0.25, omega=True):
    """A hanging capsule chain under a static anchor; joint kinds per link from ``kinds``."""
    m, com, I = mass_capsule(hh, r)
    pitch = 2 * (hh + r)
    centers = np.array([[top[0], top[1] - (hh + r) - k * pitch, top[2]] for k in range(links)])
    av = rng.normal(3 * links).reshape(links, 3) if omega else np.zeros((links, 3))
    first = s.add_bodies(pos=centers, quat=np.tile(IDENTITY_Q, (links, 1)), flags=BODY_DYNAMIC, inv_mass=1.0 / m,
                         com=com, inv_inertia=_inv3(I), col_type=CAPSULE, col_params=[hh, r, 0.0, 0.0], ang_vel=av)
    axes = rng.quaternions(links)
    frames = np.zeros((links, 14))
    params = np.zeros((links, JOINT_PARAMS))
    b0 = np.zeros(links, np.int32)
    b1 = np.arange(first, first + links, dtype=np.int32)
    for k in range(links):
        q = axes[k] if kinds[k] in (JOINT_REVOLUTE, JOINT_PRISMATIC, JOINT_UNIVERSAL) else np.asarray(IDENTITY_Q)
        if k == 0:
            b0[k] = anchor_body
            frames[k, 0:3] = np.asarray(top) - np.asarray(anchor_pos)  # anchor body is unrotated
        else:
            b0[k] = first + k - 1
            frames[k, 0:3] = [0.0, -(hh + r), 0.0]
        frames[k, 3:7] = q
        frames[k, 7:10] = [0.0, hh + r, 0.0]
        frames[k, 10:14] = q
        if kinds[k] == JOINT_PRISMATIC:
            params[k, 0], params[k, 1] = 0.2, -0.2
    s.add_joints(np.asarray(kinds, np.int32), b0, b1, frames, params)
    return first


def joint_chains(n_chains=2048, links=32, substeps=8, iterations=4, seed=None):
    """Config 3: capsule chains hanging from one static ceiling, mixed joint kinds."""
    rng = SplitMix64(scene_seed(3) if seed is None else seed)
    s = SceneData("chains%dx%d" % (n_chains, links))
    s.num_substeps, s.num_iterations = substeps, iterations
    gx = 64 if n_chains >= 64 else n_chains
    gz = int(math.ceil(n_chains / gx))
    ceiling_y = links * 0.7 + 5.0
    s.add_bodies(pos=[[0.0, 0.0, 0.0]], quat=[IDENTITY_Q], flags=0, inv_mass=0.0, com=np.zeros(3), inv_inertia=np.zeros(9),
                 col_type=BOX, col_params=[gx * 0.5 + 1.0, 0.1, gz * 0.5 + 1.0, 0.0],
                 col_pos=[0.0, ceiling_y + 0.2, 0.0])
    for c in range(n_chains):
        u = rng.uniform(links)
        kinds = np.where(u < 0.4, JOINT_REVOLUTE, np.where(u < 0.7, JOINT_SPHERICAL, np.where(
            u < 0.85, JOINT_PRISMATIC, np.where(u < 0.95, JOINT_UNIVERSAL, JOINT_FIXED))))
        top = [(c % gx - (gx - 1) / 2.0) * 1.0, ceiling_y, (c // gx - (gz - 1) / 2.0) * 1.0]
        _chain(s, rng, 0, [0.0, 0.0, 0.0], top, links, kinds)
    return s.finalize()


def _batch_bodies(rng):
    return int(round(math.exp(rng.uniform(1, math.log(16), math.log(2048))[0])))


def batch_scene_bodies(index, config=4):
    """The mixed-shape body count of batch_scene(index, config=config) without building it."""
    return _batch_bodies(SplitMix64(scene_seed(config, index)))


def batch_scene(index, n_bodies=None, config=4, chain_prob=0.1, pool=None):
    """One config-4 scene: mixed shapes dropped on a ground box, sometimes with an 8-link revolute chain."""
    rng = SplitMix64(scene_seed(config, index))
    if n_bodies is None:
        n_bodies = _batch_bodies(rng)
    s = SceneData("batch%d_%d" % (config, index))
    ny = max(1, int(round(n_bodies ** (1 / 3))))
    nxz = int(math.ceil(math.sqrt(n_bodies / ny)))
    ext = nxz * 0.75 + 3.0
    _ground_box(s, (ext, 0.5, ext))
    if pool is None:
        pool = _hull_pool(SplitMix64(scene_seed(config, 1 << 19)), count=8)
    s.convex.extend(pool)
    centers = _jittered_grid(rng, nxz, ny, nxz, 1.5, [0.0, 1.5, 0.0])[:n_bodies]
    _mixed_bodies(s, rng, centers, 0, pool)
    if rng.uniform(1)[0] < chain_prob:
        top = [ext - 1.0, 8 * 0.7 + 2.0, ext - 1.0]
        _chain(s, rng, 0, [0.0, -0.5, 0.0], top, 8, [JOINT_REVOLUTE] * 8, omega=False)
    return s.finalize()


def batch_scenes(count=4096, config=4, chain_prob=0.1):
    pool = _hull_pool(SplitMix64(scene_seed(config, 1 << 19)), count=8)
    return [batch_scene(i, config=config, chain_prob=chain_prob, pool=pool) for i in range(count)]


def serving_request(index, pool=None, n_max=8192):
    """Config 5 request: N log-uniform in [8, n_max] bodies, K uniform in [1, 120] frames."""
    rng = SplitMix64(scene_seed(5, index))
    n = int(round(math.exp(rng.uniform(1, math.log(8), math.log(n_max))[0])))
    k = int(1 + (rng.next_u64(1)[0] % np.uint64(120)))
    s = batch_scene(index, n_bodies=n, config=5, chain_prob=0.0, pool=pool)
    return s, k


def pair_scene(shape0, params0, pose0, shape1, params1, pose1, mesh0=None, mesh1=None, dynamic=(True, True)):
    """Two bodies at explicit poses, for narrowphase known-answer tests."""
    s = SceneData("pair")
    meshes = {}
    for i, (shape, params, pose, mesh, dyn) in enumerate(((shape0, params0, pose0, mesh0, dynamic[0]),
                                                          (shape1, params1, pose1, mesh1, dynamic[1]))):
        mid = -1
        if mesh is not None:
            if shape == CONVEX_MESH:
                mid = len(s.convex)
                s.convex.append(mesh)
            else:
                mid = len(s.trimesh)
                s.trimesh.append(mesh)
        p = list(params) + [0.0] * (4 - len(params))
        s.add_bodies(pos=[pose[0]], quat=[pose[1]], flags=BODY_DYNAMIC if dyn else 0, inv_mass=1.0 if dyn else 0.0,
                     com=np.zeros(3), inv_inertia=np.eye(3).ravel() if dyn else np.zeros(9), col_type=shape,
                     col_params=p, col_mesh=mid)
    return s.finalize()


# ----------------------------------------------------------------------------
# character controllers
# ----------------------------------------------------------------------------

def strip_colliders(s, bodies):
    """The scene with the colliders of `bodies` removed: such a body is an entity with a
    transform and an empty collider list (a character controller's entity)."""
    a = s.arrays
    cs = a["collider_start"]
    keep = np.ones(cs[-1], bool)
    for b in bodies:
        keep[cs[b]:cs[b + 1]] = False
    per_body = np.diff(cs).copy()
    per_body[list(bodies)] = 0
    for k in list(a):
        if k.startswith("col_") and len(a[k]) == len(keep):
            a[k] = np.ascontiguousarray(a[k][keep])
    a["collider_start"] = np.concatenate([[0], np.cumsum(per_body)]).astype(np.int32)
    return s


def character_scene(seed=61, n_chars=24, n_balls=10):
    """Character entities (transforms without colliders) among static walls, a ramp and
    resting dynamic bodies on a ground box."""
    rng = np.random.default_rng(seed)
    s = SceneData("characters%d" % seed)
    _ground_box(s, (12.0, 0.5, 12.0))
    walls = [([0, 1, 6], [6, 1, 0.3]), ([6, 1, 0], [0.3, 1, 6]), ([-4, 0.5, -4], [1.5, 0.5, 1.5])]
    for p, he in walls:
        s.add_bodies(pos=[p], quat=[IDENTITY_Q], flags=0, inv_mass=0.0, com=np.zeros(3), inv_inertia=np.zeros(9),
                     col_type=BOX, col_params=list(he) + [0.0])
    ang = 0.35
    s.add_bodies(pos=[[-3, 0.6, 3]], quat=[[np.sin(ang / 2), 0, 0, np.cos(ang / 2)]], flags=0, inv_mass=0.0,
                 com=np.zeros(3), inv_inertia=np.zeros(9), col_type=BOX, col_params=[2, 0.2, 2, 0])
    m, com, inertia = mass_sphere(0.4)
    balls = rng.uniform(-5, 5, (n_balls, 3))
    balls[:, 1] = 0.4 + 0.9 * (np.arange(n_balls) // 10)
    s.add_bodies(pos=balls, quat=[IDENTITY_Q] * n_balls, flags=BODY_DYNAMIC, inv_mass=1.0 / m, com=com,
                 inv_inertia=np.linalg.inv(inertia).T.ravel(), col_type=SPHERE, col_params=[0.4, 0, 0, 0])
    pc = rng.uniform(-6, 6, (n_chars, 3))
    pc[:, 1] = rng.uniform(0.0, 0.3, n_chars)
    first = s.add_bodies(pos=pc, quat=[IDENTITY_Q] * n_chars, flags=0, inv_mass=0.0, com=np.zeros(3),
                         inv_inertia=np.zeros(9), col_type=SPHERE, col_params=[0.1, 0, 0, 0])
    s = s.finalize()
    return strip_colliders(s, range(first, first + n_chars)), list(range(first, first + n_chars))


def character_moves(n_chars, frames, seed=62):
    """Seeded translations per frame and character: a walk in a heading that turns, plus a
    downward pull."""
    rng = np.random.default_rng(seed)
    head = rng.uniform(0, 2 * np.pi, n_chars)
    out = []
    for _ in range(frames):
        head += rng.normal(0, 0.3, n_chars)
        t = np.stack([0.12 * np.cos(head), np.full(n_chars, -0.05), 0.12 * np.sin(head)], 1).astype(np.float32)
        out.append(t)
    return out
