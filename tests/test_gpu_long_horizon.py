"""Long horizons on the GPU against the oracle.

A simulation of many frames is chaotic: the GPU solves each colour's contacts in
parallel, so its Gauss-Seidel order differs from the reference's serial order, and
that difference grows until two runs no longer agree body by body.  Long runs are
therefore judged by properties of the motion, each compared with the oracle (which
reproduces the reference bit for bit) on the same scene:
  * stack survival: the frame at which some box of a pyramid has moved 0.1 m;
  * penetration: the 99th percentile of contact penetration in each frame, and its
    largest value over the run;
  * energy: total mechanical energy (kinetic, rotational and potential) relative to
    its start, sampled every 10 frames.
The reference itself does not keep these stacks standing (its friction is formed
from the velocities at the start of each substep), so survival is compared, not
required.  Every run is deterministic, on the GPU and on the CPU, so the bounds
below do not vary between runs.  The GPU path runs its own colour order here, as a
user would.
"""
import numpy as np
import pytest

from physecs_gb300 import scenes

pytestmark = pytest.mark.gpu


def _rot(q):
    """(n, 4) quaternions (x, y, z, w) -> (n, 3, 3) rotation matrices."""
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], -2)


def energy(scene, st):
    """(total, kinetic) mechanical energy of the simulated bodies:
    1/2 m v^2 + 1/2 w^T I w + m g y_com, in joules."""
    a = scene.arrays
    fl = a["flags"].astype(np.int64)
    dyn = ((fl & scenes.BODY_DYNAMIC) != 0) & ((fl & scenes.BODY_KINEMATIC) == 0)
    R = _rot(st["quat"][dyn].astype(np.float64))
    m = 1.0 / a["inv_mass"][dyn].astype(np.float64)
    inv_i = a["inv_inertia"][dyn].astype(np.float64).reshape(-1, 3, 3).transpose(0, 2, 1)   # column-major
    i_local = np.linalg.inv(inv_i)
    v = st["vel"][dyn].astype(np.float64)
    wl = np.einsum("nji,nj->ni", R, st["ang_vel"][dyn].astype(np.float64))   # R^T w
    com = st["pos"][dyn].astype(np.float64) + np.einsum("nij,nj->ni", R, a["com"][dyn].astype(np.float64))
    ke = 0.5 * m * (v * v).sum(1) + 0.5 * np.einsum("ni,nij,nj->n", wl, i_local, wl)
    pe = m * scene.gravity * com[:, 1]
    return float((ke + pe).sum()), float(ke.sum())


def penetration_p99(f):
    """99th percentile of max(0, -separation) over a frame's contact points; the
    separation along the normal at the last row update is column 7 of each point."""
    c = f[:, [8 + 12 * k + 7 for k in range(4)]].astype(np.float64)
    live = np.abs(f[:, [8 + 12 * k + j for k in range(4) for j in range(6)]]).reshape(len(f), 4, 6).sum(2) > 0
    pen = np.maximum(0.0, -c[live])
    return float(np.percentile(pen, 99)) if pen.size else 0.0


def run(scene, frames):
    """The same scene on the GPU and in the oracle: per-frame penetration, energy /
    start energy and the largest body displacement every 10 frames."""
    from oracle.port_api import OracleScene
    from physecs_gb300.api import World
    dyn = (scene.arrays["flags"] & scenes.BODY_DYNAMIC) != 0
    out = {}
    for kind in ("gpu", "oracle"):
        sim = World([scene]) if kind == "gpu" else OracleScene(scene)
        read = sim.read_bodies if kind == "gpu" else sim.state
        st0 = read()
        e0, _ = energy(scene, st0)
        pen, e, ke, disp = [], [], [], []
        for t in range(1, frames + 1):
            sim.step()
            pen.append(penetration_p99(sim.contacts()[1]))
            if t % 10 == 0:
                st = read()
                a, b = energy(scene, st)
                e.append(a / e0)
                ke.append(b / abs(e0))
                disp.append(float(np.abs(st["pos"][dyn] - st0["pos"][dyn]).max()))
        assert np.isfinite(read()["pos"]).all(), kind
        if kind == "gpu":
            assert sim.counts()["error"] == 0
        sim.close()
        surv = next((10 * (i + 1) for i, d in enumerate(disp) if d > 0.1), frames + 10)
        out[kind] = dict(pen=np.asarray(pen), e=np.asarray(e), ke=np.asarray(ke), disp=np.asarray(disp), surv=surv)
    return out["gpu"], out["oracle"]


def test_pyramid_20_rows_600_frames(gpu_lib, oracle_lib):
    """The 20-layer pyramid (210 unit cubes, 4 substeps x 8 iterations), 600 frames: it
    starts moving when the reference's does, collapses to the same energy, and its
    penetration stays at the reference's."""
    g, o = run(scenes.pyramid(), 600)
    assert abs(g["surv"] - o["surv"]) <= 20, (g["surv"], o["surv"])
    assert g["pen"].max() <= 1.25 * o["pen"].max() + 0.005, (g["pen"].max(), o["pen"].max())
    assert np.percentile(g["pen"], 50) <= 1.5 * np.percentile(o["pen"], 50) + 0.002
    assert np.abs(g["e"] - o["e"]).max() <= 0.2, np.abs(g["e"] - o["e"]).max()
    assert abs(g["e"][-1] - o["e"][-1]) <= 0.05, (g["e"][-1], o["e"][-1])
    assert g["ke"][-1] <= 0.01 and o["ke"][-1] <= 0.01


def test_pyramid_5_rows_600_frames(gpu_lib, oracle_lib):
    """A 5-layer pyramid slides apart slowly in the reference; on the GPU it slides as
    slowly, keeps its energy and its penetration stays at the reference's."""
    g, o = run(scenes.pyramid(rows=5), 600)
    assert abs(g["surv"] - o["surv"]) <= 30, (g["surv"], o["surv"])
    assert g["disp"][-1] <= 2.0 * o["disp"][-1] + 0.1, (g["disp"][-1], o["disp"][-1])
    assert np.abs(g["e"] - o["e"]).max() <= 0.01
    assert g["pen"].max() <= 1.5 * o["pen"].max() + 0.002, (g["pen"].max(), o["pen"].max())


def test_chains_600_frames(gpu_lib, oracle_lib):
    """Eight 32-link chains with every joint kind (8 substeps x 4 iterations), 600 frames.
    The reference's joints add energy in the first frames; the GPU's add the same, and
    both settle to the same level."""
    g, o = run(scenes.joint_chains(n_chains=8, links=32), 600)
    assert abs(g["e"].max() - o["e"].max()) <= 0.2 * o["e"].max(), (g["e"].max(), o["e"].max())
    assert abs(g["e"][-1] - o["e"][-1]) <= 0.3 * abs(o["e"][-1]), (g["e"][-1], o["e"][-1])
    assert abs(g["e"][-10:].mean() - o["e"][-10:].mean()) <= 0.3 * abs(o["e"][-10:].mean())
    assert g["pen"].max() <= 1.25 * o["pen"].max() + 0.01, (g["pen"].max(), o["pen"].max())


def test_mixed_pile_300_frames(gpu_lib, oracle_lib):
    """About 400 mixed bodies (boxes, spheres, capsules, convex hulls and an 8-link chain
    where the scene has one) dropped on a ground box, 300 frames.  Bodies leave the
    ground box over its edges in both runs; penetration and energy stay at the
    reference's."""
    g, o = run(scenes.batch_scene(3, n_bodies=400), 300)
    assert g["pen"].max() <= 1.25 * o["pen"].max() + 0.005, (g["pen"].max(), o["pen"].max())
    assert np.percentile(g["pen"], 50) <= 1.5 * np.percentile(o["pen"], 50) + 0.002
    assert np.abs(g["e"] - o["e"]).max() <= 0.15, np.abs(g["e"] - o["e"]).max()
    assert abs(g["ke"][-1] - o["ke"][-1]) <= 0.3 * abs(o["ke"][-1]) + 0.01, (g["ke"][-1], o["ke"][-1])
