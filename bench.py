#!/usr/bin/env python3
"""Benchmark of the GB300 simulation hot path (physecs::Scene::simulate).

Metric: body-substeps/s = simulated bodies x substeps x frames / wall seconds.
Default workload: the batched form, 4096 independent scenes in one world, each
with N log-uniform in [16, 2048] bodies (box / sphere / capsule / convex hull mix,
uniform random orientations, dropped on a per-scene ground box, 10% of scenes
with an 8-link revolute chain), dt = 1/60 s, 4 substeps, 8 iterations, FP32.
Scenes are seeded synthetic data (Physecs publishes no dataset).

One step = one frame of every scene.  The timed region is bracketed by a
barrier and device synchronisation and timed with CUDA events on the world's
own stream; the working set (bodies, contacts, rows: GBs) exceeds the 129 MB L2,
so no flush is needed between steps.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
Under torchrun each rank simulates its own 4096 scenes (weak scaling, no
data-path collective); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "body-substeps/s"
DT = 1.0 / 60.0


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


class Dist:
    """Barrier and max-reduction over ranks (torch.distributed when launched with several ranks)."""

    def __init__(self, world, local):
        self.world = world
        self.pg = None
        if world > 1:
            import torch
            import torch.distributed as td
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(local)
            td.init_process_group(backend=backend)
            self.td, self.torch, self.backend = td, torch, backend

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, v):
        if self.world == 1:
            return v
        t = self.torch.tensor([v], dtype=self.torch.float64,
                              device="cuda" if self.backend == "nccl" else "cpu")
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if self.world == 1:
            return v
        t = self.torch.tensor([v], dtype=self.torch.float64,
                              device="cuda" if self.backend == "nccl" else "cpu")
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def frame_window(args):
    """The frames of the batched workload that are timed: every arm first runs --warmup
    frames and --e2e-steps frames untimed (the GPU arm's end-to-end leg), then times
    --steps frames of every scene."""
    first = args.warmup + args.e2e_steps + 1
    return first, first + args.steps - 1


def workload_config(name, n_scenes, args=None):
    """The workload's description.  The GPU arm and the reference arm print the same
    dict for the batched workload: same scenes, same timed frames."""
    if name == "batched":
        cfg = {"workload": "batched: %d independent scenes per GPU, N log-uniform in [16,2048] bodies, "
                           "box/sphere/capsule/hull 40/30/20/10 on a ground box, 10%% with an 8-link revolute chain, "
                           "dt=1/60 s, 4 substeps, 8 iterations" % n_scenes, "scenes": n_scenes,
               "hulls": "8 seeded 16-point hulls shared by the scenes' hull bodies, each scaled U[0.5,1.5]",
               "l2": "working set larger than L2 (no flush)"}
        if args is not None:
            a, b = frame_window(args)
            cfg["timed_frames"] = "frames %d-%d of every scene, after %d untimed frames" % (a, b, a - 1)
        return cfg
    if name == "large":
        return {"workload": "large single scene: 65536 mixed bodies over a 256x256-cell heightfield, dt=1/60, 4x8",
                "scenes": 1}
    if name == "chains":
        return {"workload": "2048 capsule chains x 32 links, mixed joints, dt=1/60, 8 substeps x 4 iterations",
                "scenes": 1, "pairs_per_collider": 16}
    return {"workload": "20-row box pyramid (210 cubes) on a ground box, dt=1/60, 4x8", "scenes": 1}


def build_workload(name, rank, n_scenes, args=None, world=1):
    """The scenes of `rank`.  Batched: the workload is world x n_scenes seeded scenes,
    split over the ranks by body count (physecs_gb300.shard), so each GPU holds about
    n_scenes scenes' worth of bodies whatever the number of GPUs (weak scaling)."""
    from physecs_gb300 import scenes
    if name == "batched":
        from physecs_gb300.shard import partition
        ids = list(range(world * n_scenes))
        part = partition([scenes.batch_scene_bodies(i) for i in ids], world)[rank] if world > 1 else ids
        pool = scenes._hull_pool(scenes.SplitMix64(scenes.scene_seed(4, 1 << 19)), count=8)
        ss = [scenes.batch_scene(i, pool=pool) for i in part]
    elif name == "large":
        ss = [scenes.large_mixed()]
    elif name == "chains":
        ss = [scenes.joint_chains()]
    else:
        ss = [scenes.pyramid()]
    return ss, workload_config(name, n_scenes, args)


def simulated_bodies(ss):
    return sum(s.n_dynamic for s in ss)


# ---------------------------------------------------------------- CPU side

def _cpu_proc(kind, scene_ids, warm, frames, barrier, conn):
    """One host core: the CPU implementation on its share of the batched scenes.  Builds
    its scenes, runs the untimed frames, waits for every other core, then times
    `frames` frames.  Sends (seconds, body-substeps)."""
    sys.path.insert(0, ROOT)
    try:
        from physecs_gb300 import scenes
        if kind == "reference":
            from oracle.ref.ref_api import RefScene as Sim
        else:
            from oracle.port_api import OracleScene as Sim
        pool = scenes._hull_pool(scenes.SplitMix64(scenes.scene_seed(4, 1 << 19)), count=8)
        sims, work = [], 0
        for idx in scene_ids:
            s = scenes.batch_scene(idx, pool=pool)
            sims.append(Sim(s))
            work += s.n_dynamic * s.num_substeps
        for sim in sims:
            sim.step(DT, warm)
    except BaseException:
        barrier.abort()
        raise
    barrier.wait()
    t = time.perf_counter()
    for sim in sims:
        sim.step(DT, frames)
    conn.send((time.perf_counter() - t, work * frames))
    conn.close()


def cpu_throughput(kind, scene_ids, warm, frames, procs):
    """body-substeps/s of the CPU implementation over the batched scenes `scene_ids`:
    `warm` untimed frames, then `frames` timed frames, on `procs` spawned processes (one
    per host core, numThreads = 0 in each) whose timed regions start together.  Scenes
    are assigned longest first to the least loaded process (by body count).  Returns
    (value, slowest process's timed seconds, processes used)."""
    import heapq
    import multiprocessing as mp
    from physecs_gb300 import scenes
    procs = max(1, min(procs, len(scene_ids)))
    sizes = sorted(((scenes.batch_scene_bodies(i), i) for i in scene_ids), reverse=True)
    heap = [(0, k) for k in range(procs)]
    chunks = [[] for _ in range(procs)]
    for n, i in sizes:
        load, k = heapq.heappop(heap)
        chunks[k].append(i)
        heapq.heappush(heap, (load + n, k))
    chunks = [sorted(c) for c in chunks if c]
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(len(chunks))
    conns, ps = [], []
    for c in chunks:
        parent, child = ctx.Pipe(duplex=False)
        p = ctx.Process(target=_cpu_proc, args=(kind, c, warm, frames, barrier, child))
        p.start()
        conns.append(parent)
        ps.append(p)
    res = [c.recv() for c in conns]
    for p in ps:
        p.join()
    wall = max(r[0] for r in res)
    work = sum(r[1] for r in res)
    return work / wall, wall, len(chunks)


def cpu_kind():
    try:
        from oracle.ref import ref_api
        if ref_api.available():
            return "reference"
    except Exception:
        pass
    return "port"



# ---------------------------------------------------------------- serving

SERVE_LAUNCH = None                # launch shapes of the serving world (None: the defaults)
SERVE_HBM_BUDGET = 120 * 10 ** 9   # device bytes the serving slots may hold (requests stay resident)
SERVE_CLASSES = [(17, 96), (33, 96), (65, 96), (129, 96), (257, 96), (513, 96), (1025, 64), (2049, 48), (4097, 32),
                 (8193, 24)]
# requests of at most 1000 bodies (the latency target's class)
SERVE_CLASSES_SMALL = [(17, 48), (33, 48), (65, 48), (129, 48), (257, 32), (513, 24), (1025, 16)]
# the same requests with the slot budget sized for a frame latency target: fewer slots,
# so that a full server's tick stays near 2 ms
SERVE_CLASSES_SLO = [(17, 16), (33, 16), (65, 16), (129, 12), (257, 8), (513, 6), (1025, 4)]


def serving_requests(count, rank=0, n_max=8192):
    """Seeded serving requests (N log-uniform in [8, n_max] bodies, K uniform in [1, 120] frames)."""
    from physecs_gb300 import scenes
    pool = scenes._hull_pool(scenes.SplitMix64(scenes.scene_seed(5, 1 << 19)), count=8)
    reqs = [scenes.serving_request(rank * count + i, pool=pool, n_max=n_max) for i in range(count)]
    ps = scenes.SceneData("pool")
    ps.convex.extend(pool)
    import numpy as np
    ps.add_bodies(pos=[[0, 0, 0]], quat=[scenes.IDENTITY_Q], flags=0, inv_mass=0.0, com=np.zeros(3),
                  inv_inertia=np.zeros(9), col_type=scenes.SPHERE, col_params=[0.5, 0, 0, 0], col_mesh=-1)
    return reqs, ps.finalize()


def _serve(srv, reqs, arrivals, t_end, max_backlog=None, descs=None):
    """Drive the server: while a tick runs on the GPU, admit the requests that have
    arrived and read and release the finished ones; then wait for the tick and start
    the next.  arrivals[i] is request i's arrival (seconds from start) or None for a
    permanent backlog.  Returns (frame latencies s, request latencies s, body-substeps
    run, wall s).  A frame's latency runs from the moment it could start (for the first
    frame, the start of the tick in which the request joins the batch; for the others,
    the previous frame's result) to its result being ready.  Waiting for a slot counts
    in the request latency (arrival to final result)."""
    import collections
    import numpy as np
    n_slots = srv.stats()["slots"]
    last = np.zeros(n_slots)              # admission time, then the previous frame's ready time
    arrival = np.zeros(n_slots)
    wps = np.zeros(n_slots)               # body-substeps per frame of the slot's request
    on = np.zeros(n_slots, bool)
    first = np.zeros(n_slots, np.int64)   # first tick that simulates the slot's request
    t0 = time.perf_counter()
    queue = collections.deque()
    nxt = 0
    frame_lat, req_lat = [], []
    work = 0.0
    ticks = 0
    in_flight = False
    finished = []
    joining = []
    while True:
        now = time.perf_counter() - t0
        if now >= t_end:
            break
        # ---- host work, beside the tick in flight
        for slot in finished:
            srv.read(slot)
            srv.release(slot)
        finished = []
        if arrivals is None:
            while len(queue) < (max_backlog or 64):
                queue.append((nxt % len(reqs), now)); nxt += 1
        else:
            while nxt < len(arrivals) and arrivals[nxt] <= now:
                queue.append((nxt % len(reqs), arrivals[nxt])); nxt += 1
        waiting = collections.deque()      # first come, first served among the requests a free slot fits
        while queue:
            i, ta = queue.popleft()
            s, k = reqs[i]
            slot = srv.admit(s, k, desc=descs[i] if descs else None)
            if slot is None:
                waiting.append((i, ta))
                continue
            on[slot] = True
            arrival[slot] = ta
            wps[slot] = s.n_dynamic * s.num_substeps
            first[slot] = ticks + 1
            joining.append(slot)
        queue = waiting
        # ---- finish the tick in flight, start the next
        if in_flight:
            done = srv.tick_end()
            t_ready = time.perf_counter() - t0
            ran = on & (first <= ticks)
            frame_lat.append(t_ready - last[ran])
            last[ran] = t_ready
            work += float(wps[ran].sum())
            for slot in done:
                req_lat.append(t_ready - arrival[slot])
                on[slot] = False
                finished.append(slot)
            in_flight = False
        if on.any():
            srv.tick_begin()
            # a request is admitted when it joins the running batch: the start of its first tick
            last[joining] = time.perf_counter() - t0
            joining = []
            ticks += 1
            in_flight = True
        else:
            time.sleep(0.0005)
    if in_flight:
        srv.tick_end()
    wall = time.perf_counter() - t0
    for slot in finished:
        srv.release(slot)
    for slot in np.nonzero(on)[0]:        # requests still running when the window closes are dropped
        srv.release(int(slot))
    fl = np.concatenate(frame_lat) if frame_lat else np.zeros(0)
    return fl, req_lat, work, wall


def run_serve_ticks(args):
    """Profiling form of the serving workload: a fixed number of ticks of a profiled
    (eagerly launched) server that keeps --serve-running requests in flight, admitted in
    seed order as slots free up.  No wall clock decides anything, so the same command
    launches the same kernels with or without a profiler.  Prints the ticks' stage times."""
    import numpy as np
    from physecs_gb300.api import Server
    from physecs_gb300.desc import make_desc
    small = args.serve_max_bodies <= 1000
    classes = SERVE_CLASSES_SMALL if small else SERVE_CLASSES
    reqs, pool_scene = serving_requests(2 * args.serve_ticks + 64, 0, n_max=args.serve_max_bodies)
    srv = Server(classes, mesh_pool=pool_scene, hbm_budget=SERVE_HBM_BUDGET, profile=True,
                 launch=json.loads(args.launch) if args.launch else SERVE_LAUNCH)
    nxt, live, stages = 0, set(), []
    for _ in range(args.serve_ticks):
        while len(live) < args.serve_running and nxt < len(reqs):
            slot = srv.admit(reqs[nxt][0], reqs[nxt][1], desc=make_desc(reqs[nxt][0]))
            if slot is None:
                break
            live.add(slot)
            nxt += 1
        for slot in srv.tick():
            live.discard(slot)
            srv.release(slot)
        stages.append(srv.tick_stages().copy())
    st = np.array(stages)
    names = ["uploads", "broadphase", "narrowphase", "rows", "solver", "bounds"]
    pct = lambda a, q: float(np.percentile(a, q))
    print(json.dumps({"workload": "serving ticks (profiled, eager)", "ticks": args.serve_ticks,
                      "running": args.serve_running, "requests": nxt,
                      "tick_ms": {"p50": pct(st.sum(1), 50), "p99": pct(st.sum(1), 99)},
                      "stage_ms": {n: {"p50": pct(st[:, i], 50), "p99": pct(st[:, i], 99)} for i, n in enumerate(names)}}))


def run_serving(args, rank, world, local):
    import numpy as np
    from physecs_gb300.api import Server
    small = args.serve_max_bodies <= 1000
    classes = (SERVE_CLASSES_SLO if args.serve_slo else SERVE_CLASSES_SMALL) if small else SERVE_CLASSES
    reqs, pool_scene = serving_requests(384 * world, 0, n_max=args.serve_max_bodies)
    if world > 1:
        # one request stream for every GPU's server, split by a deterministic router
        from physecs_gb300.shard import Router
        router = Router(world)
        reqs = [r for r in reqs if router.route(r[0].n_dynamic * r[1]) == rank]
    from physecs_gb300.desc import make_desc
    descs = [make_desc(s) for s, _ in reqs]          # the clients' packed requests
    launch = json.loads(args.launch) if args.launch else SERVE_LAUNCH
    srv = Server(classes, mesh_pool=pool_scene, device=local if world > 1 else 0, hbm_budget=SERVE_HBM_BUDGET,
                 launch=launch)
    # saturated throughput: a permanent backlog keeps every fitting slot busy
    backlog = 2 * sum(c[1] for c in classes)   # enough waiting requests to keep every class busy
    _serve(srv, reqs, None, 3.0, backlog, descs)
    _, _, work_sat, wall_sat = _serve(srv, reqs, None, max(5.0, args.serve_seconds / 3), backlog, descs)
    sat = work_sat / wall_sat
    mean_work = float(np.mean([s.n_dynamic * s.num_substeps * k for s, k in reqs]))
    lam = args.serve_load * sat / mean_work          # requests per second
    rng = np.random.default_rng(5 + rank)
    arrivals = np.cumsum(rng.exponential(1.0 / lam, size=int(lam * args.serve_seconds * 1.5) + 16))
    fl, rl, work, wall = _serve(srv, reqs, list(arrivals), args.serve_seconds, None, descs)
    fl, rl = np.asarray(fl) * 1e3, np.asarray(rl) * 1e3
    line = {
        "metric": "serving frame latency p99" + (" (N <= %d bodies)" % args.serve_max_bodies if small else ""),
        "value": float(np.percentile(fl, 99)), "unit": "ms", "n_gpus": world,
        "steps": len(fl), "warmup": 1, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (f64 in GJK/EPA)", "data": "synthetic (seeded SplitMix64 requests)",
        "config": {"workload": "serving: Poisson request stream at %.0f%% of saturated throughput, N log-uniform in "
                               "[8,%d] bodies, K uniform in [1,120] frames, dt=1/60, 4x8" % (100 * args.serve_load,
                                                                                             args.serve_max_bodies),
                   "slot_classes": classes, "seconds": args.serve_seconds, "launch": launch,
                   "hbm_budget_gb": SERVE_HBM_BUDGET / 1e9, "device_gb": srv.device_bytes() / 1e9},
        "p50_ms": float(np.percentile(fl, 50)), "p99_ms": float(np.percentile(fl, 99)),
        "request_p50_ms": float(np.percentile(rl, 50)) if len(rl) else None,
        "request_p99_ms": float(np.percentile(rl, 99)) if len(rl) else None,
        "lambda_req_per_s": lam, "saturated_body_substeps_per_s": sat,
        "served_body_substeps_per_s": work / wall, "requests_finished": int(len(rl)),
    }
    if rank == 0:
        print(json.dumps(line))
    srv.close()
    return 0

# ---------------------------------------------------------------- main

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="batched", choices=["batched", "large", "chains", "pyramid", "serving",
                                                                 "trimesh_bvh", "registry"])
    ap.add_argument("--mesh-cells", type=int, default=256, help="trimesh_bvh: heightfield cells per side")
    ap.add_argument("--serve-seconds", type=float, default=20.0)
    ap.add_argument("--serve-load", type=float, default=0.7)
    ap.add_argument("--serve-max-bodies", type=int, default=8192)
    ap.add_argument("--serve-slo", action="store_true", help="slot budget sized for the 2 ms frame target")
    ap.add_argument("--serve-ticks", type=int, default=0,
                    help="serving: run this many profiled ticks with --serve-running requests in flight instead")
    ap.add_argument("--serve-running", type=int, default=90)
    ap.add_argument("--scenes", type=int, default=4096)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--plain-scenes", type=int, default=64)
    ap.add_argument("--cpu-stride", type=int, default=8, help="cpu_baseline: every n-th scene of the workload")
    ap.add_argument("--eager", action="store_true", help="launch every frame's kernels instead of a CUDA graph")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the default kernel launch shapes")
    ap.add_argument("--launch", default=None, help="kernel launch shapes as JSON (psx_launch_config fields); no tuning")
    args = ap.parse_args()
    rank, world, local = dist_info()
    assert args.warmup >= 3, "at least three warm-up steps"

    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload == "serving" and args.serve_ticks > 0:
        return run_serve_ticks(args)
    if args.workload == "serving":
        return run_serving(args, rank, world, local)
    if args.workload == "trimesh_bvh":
        return run_trimesh_bvh(args, rank)
    if args.workload == "registry":
        return run_registry(args, rank)

    dist = Dist(world, local)
    from physecs_gb300.api import World
    ss, cfg = build_workload(args.workload, rank, args.scenes, args, world)
    n_sim = simulated_bodies(ss)
    substeps = ss[0].num_substeps
    dev = local if world > 1 else 0
    use_graph = not args.eager      # the frame is captured once and replayed as a CUDA graph
    launch = json.loads(args.launch) if args.launch else None
    if launch is None and not args.no_tune and len(ss) > 1:
        # warm-up includes the autotuner: it picks launch shapes on a throwaway world's
        # frames, stepped first to where the timed frames begin (early frames carry other
        # contact loads), and the measured world is created afresh with them
        w = World(ss, device=dev)
        w.step(DT, frame_window(args)[0] - 1)
        launch = w.tune(frames=2)
        w.close()
    # the swinging chains touch their neighbours: up to about 8 broadphase pairs per collider
    # (495,571 pairs for 65,537 colliders at frame 25), so their world gets twice the default room
    ppc = 16 if args.workload == "chains" else 0
    w = World(ss, device=dev, launch=launch, use_graph=use_graph, pairs_per_collider=ppc)
    for _ in range(args.warmup):
        w.step(DT)
    w.synchronize()
    # end to end through the public call, host arrays in and out every step; run ahead of
    # the device-timed frames, so on the earlier frames of the same scenes
    e2e_value = None
    if args.e2e_steps > 0:
        from physecs_gb300.api import pin_host, unpin_host
        st = w.read_bodies()
        pin_host(*st.values())        # the step's inputs and results live in page-locked host memory
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            w.simulate_host(DT, st)
        e2e_s = (time.perf_counter() - t0) / args.e2e_steps
        unpin_host(*st.values())
        e2e_s = dist.max(e2e_s)
        e2e_value = dist.sum(n_sim * substeps) / e2e_s
    dist.barrier()
    with ClockSampler(local) as clk:
        total_ms, stage_ms, kernels = w.step_timed(DT, args.steps)
    dist.barrier()
    t_max = dist.max(total_ms)
    work = n_sim * substeps * args.steps
    value = dist.sum(work) / (t_max / 1000.0)
    counts = w.counts()
    if counts["error"]:
        raise RuntimeError("device error bits %d" % counts["error"])

    # roofline of the solver (one launch per frame covers every substep)
    pts, rows = counts["points"], counts["rows"]
    alg_bytes = substeps * (156.0 * n_sim + 52.0 * pts + 76.0 * rows)
    solver_s = stage_ms[3] / 1000.0 / args.steps
    achieved = alg_bytes / solver_s / 1e9
    peak, peak_src = measured_peaks()
    traffic = None
    tp = os.path.join(ROOT, "profiles", "solver_traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            tj = json.load(f)
        if tj.get("workload") == args.workload and tj.get("bytes_per_body_frame"):
            traffic = float(tj["bytes_per_body_frame"]) * n_sim

    # end to end through the public API with host buffers: upload, one frame, download of
    # pos (3 floats), quat (4), vel (3) and ang_vel (3) for every body, each way
    nb = w.n_bodies
    h2d = 4 * (3 + 4 + 3 + 3) * nb

    # the plain path: the same scenes, one world per scene (each replaying its own frame
    # graph), stepped one scene at a time
    plain = None
    if args.workload == "batched" and args.plain_scenes > 0 and rank == 0:
        sub = ss[:args.plain_scenes]
        ws = [World([s], use_graph=use_graph) for s in sub]
        for x in ws:
            x.step(DT, 3)
        for x in ws:
            x.synchronize()
        t0 = time.perf_counter()
        frames = 3
        for x in ws:
            x.step(DT, frames)
            x.synchronize()
        pt = time.perf_counter() - t0
        plain = simulated_bodies(sub) * substeps * frames / pt
        for x in ws:
            x.close()

    cpu = None
    first, last = frame_window(args)
    if rank == 0 and world == 1 and not args.no_cpu and args.workload == "batched":
        try:
            # the reference built from its own sources when available, else the oracle port;
            # one spawned process per host core, each scene with numThreads = 0; a uniform
            # sample of the scenes over the same frames as the GPU arm
            kind = cpu_kind()
            ids = list(range(0, args.scenes, args.cpu_stride))
            v, wall, procs = cpu_throughput(kind, ids, first - 1, args.steps, max(1, os.cpu_count() or 1))
            cpu = {"value": v, "unit": METRIC, "cores": procs, "kind": kind,
                   "sample": "every %d-th of the %d scenes (%d scenes), frames %d-%d after %d untimed, one process "
                             "per core (%.1f s timed per process)" % (args.cpu_stride, args.scenes, len(ids), first, last,
                                                                      first - 1, wall)}
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": METRIC, "cores": 0, "kind": "port", "sample": "failed: %s" % e}

    clocks = clk.summary()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 in GJK/EPA)",
            "data": "synthetic (seeded SplitMix64 scenes)",
            "config": cfg,
            "parallelism": ("scene shards over %d GPUs (body-balanced)" % world) if world > 1 else "single GPU",
            "frame": "CUDA graph replay" if use_graph else "eager launches",
            "launch": launch,
            "counts": {"simulated_bodies": n_sim, "contact_points": pts, "joint_rows": rows, "pairs": counts["pairs"],
                       "manifolds": counts["manifolds"]},
            "stage_ms_per_step": {k: v / args.steps for k, v in zip(
                ["broadphase", "narrowphase", "contact_joint_rows", "solver", "bounds"], stage_ms)},
            "roofline": {"kernel": "k_solve_block (solver, all substeps of a frame)", "bound": "hbm",
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_source": peak_src, "traffic": traffic,
                         "algorithmic_bytes": alg_bytes},
            # the largest stage is the narrowphase, whose top kernel (EPA, f64 polytope for
            # parity) is bound by the FP64 pipe rather than by HBM or the tensor cores; the
            # largest kernel family is the solver, which the roofline above describes
            "dominant_kernel": {"kernel": "k_convex_epa_flat (narrowphase stage's top kernel)", "bound": "fp64 pipe",
                                "narrowphase_ms_per_step": stage_ms[1] / args.steps,
                                "fp64_pipe_active": 0.398,
                                "source": "profiles/k_convex_epa_flat_512.md (ncu --set full, 512 scenes)"},
            "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d},
            "plain_gpu_scene_by_scene": None if plain is None else {"value": plain, "unit": METRIC,
                                                                    "scenes": min(args.plain_scenes, len(ss))},
            "batched_vs_plain": None if plain is None else value / plain,
            "gpu_launches": kernels,
            "clocks": clocks,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))
    w.close()
    dist.close()


def run_trimesh_bvh(args, rank):
    """The triangle-mesh BVH build (TriangleMesh's constructor, src/TriangleMesh.cpp:144-164)
    of one value-noise heightfield of --mesh-cells^2 cells.  value: a terrain edit,
    psx_world_update_trimesh on a world that holds the mesh (new vertices uploaded, BVH
    rebuilt on the device, collider bounds refreshed); e2e: psx_trimesh_build from host
    arrays to host arrays.  Beside them, the reference's constructor on one host core."""
    import numpy as np
    from physecs_gb300 import scenes
    from physecs_gb300.api import World, trimesh_build
    if rank != 0:
        return 0
    cells = args.mesh_cells
    s = scenes.large_mixed(n_bodies=64, cells=cells, seed=scenes.scene_seed(2, 99))
    a = s.arrays
    v = a["tri_verts"].copy()
    ix = a["tri_indices"].copy()
    v2 = v.copy()
    v2[:, 1] = v2[:, 1] * np.float32(0.5)
    w = World([s])
    for i in range(args.warmup):
        w.update_trimesh(0, 0, v2 if i % 2 == 0 else v)
        trimesh_build(v, ix)
    upd, std = [], []
    for i in range(args.steps):
        t = time.perf_counter()
        w.update_trimesh(0, 0, v2 if i % 2 == 0 else v)
        upd.append(time.perf_counter() - t)
        t = time.perf_counter()
        trimesh_build(v, ix)
        std.append(time.perf_counter() - t)
    w.close()
    kind = cpu_kind()
    if kind == "reference":
        from oracle.ref.ref_api import trimesh_build as cpu_build
    else:
        from oracle.port_api import trimesh_build as cpu_build
    cpu = []
    for _ in range(3):
        t = time.perf_counter()
        cpu_build(v, ix)
        cpu.append(time.perf_counter() - t)
    nt, nv = len(ix) // 3, len(v)
    ms = 1e3 * statistics.median(upd)
    line = {
        "metric": "triangle-mesh BVH build time", "value": ms, "unit": "ms", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "none", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (value-noise heightfield)",
        "config": {"workload": "trimesh_bvh: heightfield %dx%d cells, %d triangles, %d vertices" % (cells, cells, nt, nv),
                   "value": "psx_world_update_trimesh (vertex upload + device build + collider bounds)"},
        "e2e": {"value": 1e3 * statistics.median(std), "unit": "ms", "h2d_bytes_per_step": 16 * nv + 16 * nt,
                "d2h_bytes_per_step": 80 * nt + 32 * (2 * nt - 1), "call": "psx_trimesh_build"},
        "cpu_baseline": {"value": 1e3 * statistics.median(cpu), "unit": "ms", "cores": 1, "kind": kind,
                         "sample": "3 builds of the same mesh (TriangleMesh's constructor)"},
        "gpu_launches": None,
    }
    print(json.dumps(line))
    return 0


def run_registry(args, rank):
    """Registry changes at scale, between frames of a batched world: --scenes scenes, one
    character entity among their bodies each.  value: psx_world_apply_deltas of a batch
    that patches the pose and writes the velocities of a tenth of the bodies (host fold,
    one upload, one kernel); e2e: psx_world_move_characters of every scene's character.
    Beside them, the reference doing the same through its registry and its
    CharacterController, one scene after another on one host core, on a sample."""
    import numpy as np
    from physecs_gb300.scenes import character_moves, character_scene
    from physecs_gb300.api import World, pack_deltas
    if rank != 0:
        return 0
    n = args.scenes
    base, chars = character_scene(n_chars=1, n_balls=200)
    ss = [base] * n
    w = World(ss)
    nb = len(base.arrays["pos"])
    rng = np.random.default_rng(3)
    dyn = np.nonzero(base.arrays["flags"] & 1)[0]
    k = max(1, nb // 10)

    def batch():
        rows = []
        for sc in range(n):
            for b in rng.choice(dyn, min(k, len(dyn)), replace=False):
                rows.append({"scene": sc, "body": int(b), "pos": rng.uniform(-5, 5, 3) + [0, 3, 0], "quat": [0, 0, 0, 1],
                             "vel": rng.normal(0, 1, 3), "ang_vel": [0, 0, 0]})
        return pack_deltas(rows)
    batches = [batch() for _ in range(args.steps + args.warmup)]
    moves = character_moves(n, args.steps + args.warmup)
    specs = [{"scene": sc, "body": chars[0], "height": 1.0, "radius": 0.3} for sc in range(n)]
    dts, cts = [], []
    for i in range(args.steps + args.warmup):
        w.synchronize()
        t = time.perf_counter()
        w.apply_deltas(batches[i])
        w.synchronize()
        t1 = time.perf_counter()
        w.move_characters(specs, moves[i])
        t2 = time.perf_counter()
        w.step(DT)
        if i >= args.warmup:
            dts.append(t1 - t)
            cts.append(t2 - t1)
    w.synchronize()
    err = w.counts()["error"]
    w.close()
    if err:
        raise RuntimeError("device error bits %d" % err)
    # the reference on a sample of the scenes (the same per-scene work)
    kind = cpu_kind()
    sample = min(n, 32)
    ref_d = ref_c = None
    if kind == "reference":
        from oracle.ref.ref_api import RefScene
        sims = [RefScene(base) for _ in range(sample)]
        per = len(batches[0]) // n
        td = tc = 0.0
        for i, r in enumerate(sims):
            part = batches[0][i * per:(i + 1) * per]
            t = time.perf_counter()
            r.apply_deltas(part)
            td += time.perf_counter() - t
            t = time.perf_counter()
            r.move_character(chars[0], 1.0, 0.3, moves[0][i])
            tc += time.perf_counter() - t
        ref_d, ref_c = 1e3 * td * n / sample, 1e3 * tc * n / sample
    nd = len(batches[0])
    line = {
        "metric": "registry delta batch time", "value": 1e3 * statistics.median(dts), "unit": "ms", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.median(dts), "higher_is_better": False,
        "scaling": "none", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded deltas and walks)",
        "config": {"workload": "registry: %d scenes of %d bodies, %d pose+velocity deltas per batch, %d characters"
                               % (n, nb, nd, n),
                   "value": "psx_world_apply_deltas", "e2e": "psx_world_move_characters"},
        "e2e": {"value": 1e3 * statistics.median(cts), "unit": "ms", "h2d_bytes_per_step": 40 * n, "d2h_bytes_per_step": n,
                "call": "psx_world_move_characters"},
        "cpu_baseline": {"value": ref_d, "unit": "ms", "cores": 1, "kind": kind,
                         "characters_ms": ref_c,
                         "sample": "%d scenes through the reference's registry and CharacterController, scaled to %d"
                                   % (sample, n)},
        "gpu_launches": None,
    }
    print(json.dumps(line))
    return 0


def run_reference(args, rank, world):
    """The reference's own CPU implementation (built from its sources; the oracle port
    where it is absent) on the host cores: the GPU arm's workload and frame window, every
    scene, one process per host core.  Under torchrun only rank 0 runs."""
    if rank != 0:
        return 0
    if args.workload in ("pyramid", "large", "chains"):
        return run_reference_single(args)
    if args.workload != "batched":
        print(json.dumps({"impl": "reference", "unavailable": "the reference arm runs the simulation workloads only"}))
        return 0
    kind = cpu_kind()
    procs = max(1, os.cpu_count() or 1)
    first, last = frame_window(args)
    ids = list(range(args.scenes))
    t0 = time.perf_counter()
    value, wall, used = cpu_throughput(kind, ids, first - 1, args.steps, procs)
    total_s = time.perf_counter() - t0
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "impl": "reference", "data": "synthetic (seeded SplitMix64 scenes)",
        "config": workload_config("batched", args.scenes, args),
        "parallelism": "%d host cores, one process per core (numThreads=0 each), scenes assigned by body count" % used,
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": used, "kind": kind,
                         "sample": "all %d scenes, frames %d-%d after %d untimed frames (%.0f s in all)"
                                   % (args.scenes, first, last, first - 1, total_s)},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_reference_single(args):
    """The reference on one large scene (pyramid, large, chains): one Scene with the
    reference's own thread pool over every host core (Scene(registry, numThreads)), the
    GPU arm's untimed frames first, then --steps timed frames."""
    kind = cpu_kind()
    ss, cfg = build_workload(args.workload, 0, 1, args)
    s = ss[0]
    threads = max(1, os.cpu_count() or 1)
    if kind == "reference":
        from oracle.ref.ref_api import RefScene
        sim = RefScene(s, num_threads=threads)
    else:
        from oracle.port_api import OracleScene
        sim, threads = OracleScene(s), 1
    warm = args.warmup + args.e2e_steps
    sim.step(DT, warm)
    t0 = time.perf_counter()
    sim.step(DT, args.steps)
    wall = time.perf_counter() - t0
    value = s.n_dynamic * s.num_substeps * args.steps / wall
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
        "dtype": "f32", "impl": "reference", "data": "synthetic (seeded SplitMix64 scenes)", "config": cfg,
        "parallelism": "one scene, the reference's thread pool over %d host threads" % threads,
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": kind,
                         "sample": "frames %d-%d after %d untimed frames" % (warm + 1, warm + args.steps, warm)},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    main()
