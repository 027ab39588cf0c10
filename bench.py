"""Benchmark: body-steps/s of the GPU world step on the 100k-body mixed scene.

Workload (one "step" = one B2world::step(1/60, 8, 3) of the whole scene):
  100k-body mixed scene: 50k circles (r 0.1-0.5 m) + 50k convex 3-8-gons (extent 0.1-0.6 m)
  seeded uniformly in a 1000 x 1000 m box of static edge walls, density 1, friction 0.4,
  v ~ N(0,1), gravity -10, dt = 1/60, 8 velocity / 3 position iterations, sleeping off,
  continuous physics off. Synthetic data from a seeded splitmix64 stream.

Legs
  value       device-resident throughput: N_dynamic * K / (sum of per-step device times),
              each step bracketed by CUDA events on the world's stream; an L2 flush
              (a 256 MiB write) runs between steps outside the timed events.
  e2e         the same steps through the public API with host buffers: b2g_step plus a
              read of every body's state (position, angle, velocities) into host memory
              after every step (b2g_get_body_states_async: the copy of step k overlaps
              step k + 1; the last copy is waited for), timed on the host clock around the
              whole loop.
  cpu_baseline the oracle (a faithful single-threaded CPU restatement of box2d-rs's step,
              libm sin/cos) timed on this host on a bounded sample of the same workload.
  --impl reference  times that CPU restatement alone (the real Rust crate cannot be built
              without cargo) and prints the reference line.
Multi-GPU (torchrun): the single world does not shard, so each rank steps its own replica
("replicas only"); value is all ranks' body-steps over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "box2d-rs_gb300"))

import b2g  # noqa: E402
import scenes  # noqa: E402
import shard  # noqa: E402

WORKLOAD = "mixed-100k: 50k circles + 50k 3-8-gons, 1000x1000 m walled box, 8/3 iterations, dt=1/60"
METRIC = "body-steps/s @100k bodies (mixed scene)"


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


SORT_PASSES = 4  # one world: 31 key bits (15-bit Morton cells per axis + the large-static bit), 8-bit digits


def bytes_model(st, scene_stats, vi, pi):
    """Algorithmic HBM bytes of one step by kernel phase (SoA layout of csrc/b2g_internal.h), from the
    step's own device counts `st` (b2g_get_step_stats).

    k_solve        per dynamic body: integrate velocities 72 B, integrate positions 48 B, write-back 40 B;
                   per proxy: fixture sync 76 B + shape bytes; per constraint slot: init + warm start
                   320 B, velocity iteration 208 B, position iteration 128 B, store 16 B
    k_collide      per contact: 116 B state + 2 shapes (polygon 16 B/vertex + 12, circle 12, edge 36)
    bp_sort        per proxy: bounds 24 B + keys 28 B + 4 radix passes x 24 B (key + payload read and
                   written); nothing when the pass keeps the hierarchy (hierarchy_age > 0)
    bp_hierarchy   per proxy: build 36 B, leaves 36 B, refit 68 B, four-way records 144 B; per contact:
                   row index 12 B. A pass that keeps the hierarchy: per proxy its moved flag 1 B, per moved
                   proxy 140 B (leaf index and fat AABB read; the leaf, its parent's binary record and two
                   four-way records located and written), per contact the row index 12 B
    bp_traverse    per fetched node 80 B (four child boxes + children), per checked leaf 32 B (its
                   payload, proxy ids, moved flags, contact row and key), per proxy 5 B (payload and
                   moved flag), per new pair 20 B
    merge          per contact: 2 x 108 B (read and written)
    """
    nf, nb = scene_stats["n_fixtures"], scene_stats["n_dynamic"]
    nc, ncons = st["contacts"], st["constraints"]
    shape = scene_stats["shape_bytes_mean"]
    rebuilt = st.get("hierarchy_age", 0) == 0
    return {
        "solver": nb * (72 + 48 + 40) + ncons * (320 + 208 * vi + 128 * pi + 16) + nf * (76 + shape),
        "collide": nc * (116 + 2 * shape),
        "bp_sort": nf * (24 + 28 + SORT_PASSES * 24) if rebuilt else 0,
        "bp_hierarchy": (nf * (36 + 36 + 68 + 144) if rebuilt else nf + st.get("bp_moved_proxies", 0) * 140) + nc * 12,
        "bp_traverse": st["bp_node_visits"] * 80 + st["bp_leaf_checks"] * 32 + nf * 5 + st["new_pairs"] * 20,
        "merge": nc * 2 * 108,
    }


# the kernel that dominates each phase (the phase's CUDA-event time is charged to it)
PHASE_KERNEL = {"solver": "k_solve", "collide": "k_collide", "bp_sort": "k_radix_coop",
                "bp_hierarchy": "k_bp_refit", "bp_traverse": "k_bp_traverse", "merge": "k_merge_old"}


def scene_stats(scene):
    f = scene["fixtures"]
    st = f["shape_type"]
    shape = np.where(st == b2g.CIRCLE, 12, np.where(st == b2g.EDGE, 36, 16 * np.maximum(f["vertex_count"], 4) + 12))
    return {"n_dynamic": scene["n_dynamic"], "n_fixtures": len(f), "shape_bytes_mean": float(shape.mean())}


def run_cpu_baseline(scene, skip, budget_s=30.0, max_steps=60):
    """Time the oracle (libm trig, single thread) on the bench's window of the same workload: the
    oracle steps the scene `skip` steps untimed, then is timed for up to `max_steps` steps or
    `budget_s` seconds (at least 3 steps)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.set_trig(True)
    w = oracle.OracleWorld(gravity=scene["gravity"], allow_sleep=False)
    scenes.build_world(w, scene)
    if skip > 0:
        w.steps(scene["dt"], scene["vi"], scene["pi"], skip)
    steps = 0
    t0 = time.perf_counter()
    while steps < max_steps and (steps < 3 or time.perf_counter() - t0 < budget_s):
        w.step(scene["dt"], scene["vi"], scene["pi"])
        steps += 1
    dt = time.perf_counter() - t0
    w.close()
    return {"value": scene["n_dynamic"] * steps / dt, "unit": "body-steps/s", "cores": 1, "kind": "port",
            "sample": f"steps {skip + 1}-{skip + steps} of the mixed-100k scene after {skip} untimed steps "
                      f"(oracle, libm sin/cos, 1 thread, {dt:.1f} s timed)"}


def snapshot(world):
    """Post-step state of a GPU world, enough for the oracle to continue from it."""
    aabbs, _ = world.get_proxies()
    return {"bodies": world.get_body_states(), "aabbs": aabbs, "contacts": world.get_contacts()}


def run_cpu_on_snapshots(scene, snaps, budget_s=24.0):
    """Time the oracle (libm sin/cos, 1 thread) for a few steps from each GPU snapshot, so the
    CPU sample covers the same part of the trajectory as the timed GPU steps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.set_trig(True)
    dt = scene["dt"]
    total_steps, total_s, where = 0, 0.0, []
    per_snap = budget_s / max(1, len(snaps))
    for step_index, snap in snaps:
        w = oracle.OracleWorld(gravity=scene["gravity"], allow_sleep=False)
        scenes.build_world(w, scene)
        w.import_state(snap["bodies"], snap["aabbs"], snap["contacts"], np.float32(1.0) / dt)
        n = 0
        t0 = time.perf_counter()
        while n < 20 and (n < 2 or time.perf_counter() - t0 < per_snap):
            w.step(dt, scene["vi"], scene["pi"])
            n += 1
        total_s += time.perf_counter() - t0
        total_steps += n
        where.append(f"{n}@{step_index}")
        w.close()
    return {"value": scene["n_dynamic"] * total_steps / total_s, "unit": "body-steps/s", "cores": 1, "kind": "port",
            "sample": f"oracle (libm sin/cos, 1 thread) stepped from GPU snapshots of the timed window: "
                      f"steps@step-index {', '.join(where)}; {total_s:.1f} s"}


def timed_steps(world, scene, steps, flush, torch):
    """Sum of per-step device times (CUDA events on the world's stream), L2 flushed between steps."""
    total = 0.0
    for _ in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        world.step(scene["dt"], scene["vi"], scene["pi"])
        total += world.get_profile()["step"]
    return total


def tune_blocks_per_sm(torch, flush, t, dt, vi, pi, turns=3, steps=3):
    """After b2g_autotune (which times back-to-back steps with warm caches): choose among its pick, the
    default configuration and both with 512 solver threads per block, on the scratch world `t`, the
    way this bench times a step (device time, L2 flushed before it); the candidates take turns.
    Returns the launch configuration to use (one block per SM: the part-local solve gives each block
    an SM's shared memory)."""
    tuned = t.get_launch_config()
    default = {"coop_blocks_per_sm": 1, "collide_block": 128, "traverse_block": 256, "solver_block": 256,
               "collide_group": 0}
    cands = []
    for base in (dict(tuned, coop_blocks_per_sm=1), default):
        for sb in (256, 512):
            c = dict(base, solver_block=sb)
            if c not in cands:
                cands.append(c)
    total = [0.0] * len(cands)
    for _ in range(turns):
        for i, c in enumerate(cands):
            t.set_launch_config(**c)
            for _ in range(2):  # the step graph's captures for both contact-buffer parities
                t.step(dt, vi, pi)
            for _ in range(steps):
                flush.fill_(1.0)
                torch.cuda.synchronize()
                t.step(dt, vi, pi)
                total[i] += t.get_profile()["step"]  # device time (CUDA events), as timed_steps
    return cands[min(range(len(cands)), key=lambda i: total[i])]


def run_batched(torch, flush, device, num_worlds=4096, steps=300, warmup=3, per_bucket=6, rank=0, world_size=1,
                autotune=True):
    """Batched uneven worlds: one world batch stepped together vs. the same worlds stepped one
    at a time. The sequential time is the sum over all worlds of each world's mean step time,
    estimated from `per_bucket` worlds of every log2 size bucket, each timed over the same
    steps as the batch. With several ranks each steps its contiguous range of the worlds
    (shard.py) and the batch time is the slowest rank's."""
    full = scenes.batched(num_worlds=num_worlds, steps=steps)
    part = shard.shard_scene(full, rank, world_size) if world_size > 1 else full
    if autotune:
        t = b2g.B2world(gravity=part["gravity"], num_worlds=part["num_worlds"], device=device)
        t.set_allow_sleeping(False)
        scenes.build_world(t, part)
        for _ in range(warmup + steps // 2):
            t.step(part["dt"], part["vi"], part["pi"])
        t.autotune(part["dt"], part["vi"], part["pi"], 6)
        tuned = tune_blocks_per_sm(torch, flush, t, part["dt"], part["vi"], part["pi"])
        t.close()
    w = b2g.B2world(gravity=part["gravity"], num_worlds=part["num_worlds"], device=device)
    w.set_allow_sleeping(False)
    scenes.build_world(w, part)
    if autotune:
        w.set_launch_config(**tuned)
    for _ in range(warmup):
        w.step(part["dt"], part["vi"], part["pi"])
    w.synchronize()
    launch_config = w.get_launch_config()
    if world_size > 1:
        torch.distributed.barrier()
    batch_ms = timed_steps(w, part, steps, flush, torch)
    counts = w.get_counts()
    w.close()
    if world_size > 1:
        t = torch.tensor([batch_ms], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        batch_ms = float(t[0])
    scene = full
    if rank != 0:
        return None
    sizes = scene["world_body_counts"]
    bucket = np.floor(np.log2(sizes)).astype(int)
    bodies, fixtures = scene["bodies"], scene["fixtures"]
    world_of_body = bodies["world_index"]
    est_ms, sampled = 0.0, []
    for b in np.unique(bucket):
        members = np.nonzero(bucket == b)[0]
        pick = members[np.linspace(0, len(members) - 1, min(per_bucket, len(members))).astype(int)]
        ms = []
        for wi in pick:
            bidx = np.nonzero(world_of_body == wi)[0]
            remap = np.full(len(bodies), -1, np.int64)
            remap[bidx] = np.arange(len(bidx))
            fidx = np.nonzero(remap[fixtures["body"]] >= 0)[0]
            bd = bodies[bidx].copy()
            bd["world_index"] = 0
            fx = fixtures[fidx].copy()
            fx["body"] = remap[fx["body"]]
            single = b2g.B2world(gravity=scene["gravity"], device=device)
            single.set_allow_sleeping(False)
            single.create_bodies(bd)
            single.create_fixtures(fx)
            sub = dict(scene, bodies=bd, fixtures=fx)
            for _ in range(warmup):
                single.step(scene["dt"], scene["vi"], scene["pi"])
            single.synchronize()
            ms.append(timed_steps(single, sub, steps, flush, torch) / steps)
            single.close()
        est_ms += len(members) * float(np.mean(ms)) * steps
        sampled.append({"bodies": f"{2 ** b}-{2 ** (b + 1) - 1}", "worlds": int(len(members)),
                        "sampled": int(len(pick)), "ms_per_step": float(np.mean(ms))})
    batched = num_worlds * steps / (batch_ms / 1e3)
    sequential = num_worlds * steps / (est_ms / 1e3)
    return {"metric": "world-steps/s, 4096 uneven worlds (16-2048 bodies)", "value": batched,
            "ranks": world_size, "sharding": "contiguous world ranges, no collective" if world_size > 1 else None,
            "launch_config": launch_config,
            "unit": "world-steps/s", "body_steps_per_s": scene["n_dynamic"] * steps / (batch_ms / 1e3),
            "bodies": scene["n_dynamic"], "steps": steps, "ms_per_step": batch_ms / steps,
            "sequential_single_world_gpu": {"value": sequential, "unit": "world-steps/s",
                                            "estimate": "sum over worlds of the mean per-step time of sampled worlds "
                                                        "in the same log2 size bucket", "buckets": sampled},
            "speedup_vs_sequential": batched / sequential, "contacts_last_step": counts["contacts"],
            "l2": "256 MiB flush between timed steps"}


def _stack_loss_grad(world, scene):
    """dL/d(final state) of L = sum over worlds of |centre of mass of the stack - target|^2."""
    st = world.get_body_states()
    d = np.zeros(world.body_count, b2g.BODY_STATE)
    stacks = scene.get("stacks", [scene.get("stack")])
    targets = scene.get("targets", [scene.get("target")])
    for stack, target in zip(stacks, targets):
        com = st["world_center"][stack].astype(np.float64).mean(0)
        d["world_center"][stack] = 2.0 * (com - target) / len(stack)
    return d


def _toi_pairs(n, seed):
    """n random pairs of moving shapes for the time-of-impact leg: circles (r 0.1-0.6), 3-8-gons
    (radius 0.2-0.7 with jitter) and edges (up to 3 m), sweeps moving up to 4 m and turning up to
    3 rad; the same mix as tests/test_toi.py, generated with array operations."""
    rng = np.random.default_rng(seed)

    def defs():
        d = b2g.fixture_defs(n)
        kind = rng.integers(0, 3, n)
        c, p, e = kind == 0, kind == 1, kind == 2
        d["shape_type"][c] = b2g.CIRCLE
        d["radius"][c] = rng.uniform(0.1, 0.6, int(c.sum()))
        d["vertices"][c, 0] = rng.uniform(-0.2, 0.2, (int(c.sum()), 2))
        d["shape_type"][p] = b2g.POLYGON
        d["polygon_mode"][p] = b2g.POLYGON_HULL
        k = rng.integers(3, 9, n)
        ang = np.sort(rng.uniform(0, 2 * np.pi, (n, 8)), axis=1)
        rad = rng.uniform(0.2, 0.7, (n, 8))
        verts = np.stack([rad * np.cos(ang), rad * np.sin(ang)], 2).astype(np.float32)
        verts[np.arange(8)[None, :] >= k[:, None]] = 0.0
        d["vertices"][p] = verts[p]
        d["vertex_count"][p] = k[p]
        d["shape_type"][e] = b2g.EDGE
        a = rng.uniform(-2, 2, (n, 2)).astype(np.float32)
        d["vertices"][e, 1] = a[e]
        d["vertices"][e, 2] = (a + rng.uniform(-3, 3, (n, 2)))[e]
        return d

    def sweeps(spread):
        s = np.zeros(n, b2g.SWEEP)
        s["local_center"] = rng.uniform(-0.1, 0.1, (n, 2))
        s["c0"] = rng.uniform(-spread, spread, (n, 2))
        s["c"] = s["c0"] + rng.uniform(-spread, spread, (n, 2))
        s["a0"] = rng.uniform(-10, 10, n)
        s["a"] = s["a0"] + rng.uniform(-3, 3, n)
        return s

    return defs(), sweeps(4.0), defs(), sweeps(1.0)


def run_toi(n=1_000_000, sample=100_000, repeats=3):
    """Batched time of impact (b2g_time_of_impact): pairs per second through the C ABI (host shape
    set-up, copies and the kernel, host clock), the oracle's single-thread rate on a sample, and
    whether the sample's results are bit-identical."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    da, sa, db, sb = _toi_pairs(n, 11)
    b2g.time_of_impact(da[:1000], sa[:1000], db[:1000], sb[:1000])  # load and warm up
    best = float("inf")
    for _ in range(repeats):
        t0 = time.perf_counter()
        got = b2g.time_of_impact(da, sa, db, sb)
        best = min(best, time.perf_counter() - t0)
    oracle.build()
    oracle.set_trig(False)
    try:
        t0 = time.perf_counter()
        ref = oracle.time_of_impact(da[:sample], sa[:sample], db[:sample], sb[:sample])
        cpu = time.perf_counter() - t0
    finally:
        oracle.set_trig(True)
    same = bool(np.array_equal(got[:sample]["state"], ref["state"]) and
                np.array_equal(got[:sample]["t"].view(np.uint32), ref["t"].view(np.uint32)))
    return {"pairs": n, "pairs_per_s": n / best, "cpu_pairs_per_s": sample / cpu, "cpu_sample": sample,
            "cpu_cores": 1, "sample_bit_identical": same,
            "states": np.bincount(got["state"], minlength=5).tolist()}


def run_continuous(torch, flush, device, skip=300, steps=60, warmup=3, cpu_budget_s=8.0):
    """The mixed-100k scene with continuous physics on (B2world::solve_toi after every step, the
    reference's default): bodies reach the floor edge at up to ~100 m/s, hundreds of
    time-of-impact events per step. GPU: device time of `steps` steps after `skip` untimed ones
    (L2 flushed between steps). CPU: the oracle (libm sin/cos, 1 thread, continuous on) stepped from
    the GPU's state at the start of the window."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    scene = scenes.mixed()
    w = b2g.B2world(gravity=scene["gravity"], device=device)
    w.set_allow_sleeping(False)
    w.set_continuous_physics(True)
    scenes.build_world(w, scene)
    dt, vi, pi = scene["dt"], scene["vi"], scene["pi"]
    for _ in range(skip):
        w.step(dt, vi, pi)
    w.synchronize()
    aabbs, _ = w.get_proxies()
    snap = {"bodies": w.get_body_states(), "aabbs": aabbs, "contacts": w.get_contacts()}
    for _ in range(warmup):
        w.step(dt, vi, pi)
    w.synchronize()
    e0 = w.get_toi_stats()[0]
    total, toi_ms, iters = 0.0, 0.0, []
    for _ in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        w.step(dt, vi, pi)
        prof = w.get_profile()
        total += prof["step"]
        toi_ms += prof["solve_toi"]
        iters.append(w.get_toi_stats()[1])
    events = w.get_toi_stats()[0] - e0
    restarts = w.get_toi_stats()[2]
    n_dyn = scene["n_dynamic"]
    w.close()

    oracle.set_trig(True)
    o = oracle.OracleWorld(gravity=scene["gravity"], allow_sleep=False, continuous=True)
    scenes.build_world(o, scene)
    o.import_state(snap["bodies"], snap["aabbs"], snap["contacts"], np.float32(1.0) / dt)
    n, t0 = 0, time.perf_counter()
    while n < 5 and (n < 1 or time.perf_counter() - t0 < cpu_budget_s):
        o.step(dt, vi, pi)
        n += 1
    cpu_s = time.perf_counter() - t0
    cpu_events = o.toi_events()
    o.close()
    return {"metric": "body-steps/s with continuous physics", "value": n_dyn * steps / (total / 1000.0),
            "unit": "body-steps/s", "ms_per_step": total / steps, "solve_toi_ms_per_step": toi_ms / steps,
            "window": f"steps {skip + warmup}-{skip + warmup + steps} of the mixed-100k scene",
            "toi_events_per_step": events / steps, "pass_iterations_max": max(iters), "restarts": restarts,
            "cpu_baseline": {"value": n_dyn * n / cpu_s, "unit": "body-steps/s", "cores": 1, "kind": "port",
                             "sample": f"oracle (libm sin/cos, 1 thread, solve_toi on) stepped {n} steps from the "
                                       f"GPU's state at step {skip}: {cpu_events / n:.0f} events per step, "
                                       f"{cpu_s:.1f} s"}}


def run_pile(torch, flush, device, steps=20, warmup=3, cpu=True, n_boxes=250_000, scene_steps=1000,
             cpu_budget_s=20.0):
    """High-contact pile: 250k boxes (half-extents 0.05-0.2 m) dropped into a 100 x 400 m walled container,
    1000 steps. The last `steps` steps of the 1000 are timed (device time, L2 flushed between steps),
    when the pile holds its most contact points. CPU: the oracle (libm sin/cos, 1 thread) stepped from
    the GPU's state at the start of the window. The world starts with 16M contacts and 4M new pairs of
    capacity and grows them as needed (b2g_set_auto_grow)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    scene = scenes.pile(n_boxes=n_boxes, steps=scene_steps)
    dt, vi, pi = scene["dt"], scene["vi"], scene["pi"]
    w = b2g.B2world(gravity=scene["gravity"], device=device, contact_capacity=16_000_000, pair_capacity=4_000_000)
    w.set_allow_sleeping(False)
    w.set_auto_grow(True)  # the falling column's stretched fat AABBs overlap many boxes below them
    scenes.build_world(w, scene)
    skip = scene_steps - steps - warmup
    for _ in range(skip):
        w.step(dt, vi, pi)
    w.synchronize()
    snap = snapshot(w)
    for _ in range(warmup):
        w.step(dt, vi, pi)
    w.synchronize()
    total = 0.0
    fine = dict.fromkeys(b2g.B2world.PHASES + b2g.B2world.TREE_PHASES, 0.0)
    stats = scene_stats(scene)
    byts = {}
    for _ in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        w.step(dt, vi, pi)
        total += w.get_profile()["step"]
        for ph, v in w.get_phase_times(tree_split=True).items():
            fine[ph] += v
        for ph, v in bytes_model(w.get_step_stats(), stats, vi, pi).items():
            byts[ph] = byts.get(ph, 0) + v
    st = w.get_step_stats()
    contacts = w.get_contacts()
    points = int(contacts["point_count"][contacts["touching"] != 0].sum())
    w.close()
    peak, _ = load_peaks()
    solver_ach = byts["solver"] / (fine["solver"] / 1e3) / 1e9 if fine["solver"] > 0 else None
    out = {"metric": "body-steps/s, high-contact pile", "value": n_boxes * steps / (total / 1e3),
           "unit": "body-steps/s", "ms_per_step": total / steps,
           "window": f"steps {skip + warmup + 1}-{scene_steps} of the {scene_steps}-step pile",
           "contact_points": points, "contacts": st["contacts"], "constraints": st["constraints"],
           "colours": st["colours"], "parts": st["parts"],
           "phase_ms_per_step": {k: v / steps for k, v in fine.items()},
           "solver_roofline": {"achieved": solver_ach, "peak": peak, "unit": "GB/s",
                               "frac": solver_ach / peak if solver_ach else None},
           "capacities": {"initial_contacts": 16_000_000, "initial_pairs": 4_000_000,
                          "contacts": st["contact_capacity"], "pairs": st["pair_capacity"],
                          "grows": st["capacity_grows"]}}
    if cpu:
        import oracle

        oracle.set_trig(True)
        o = oracle.OracleWorld(gravity=scene["gravity"], allow_sleep=False)
        scenes.build_world(o, scene)
        o.import_state(snap["bodies"], snap["aabbs"], snap["contacts"], np.float32(1.0) / dt)
        n, t0 = 0, time.perf_counter()
        while n < 10 and (n < 1 or time.perf_counter() - t0 < cpu_budget_s):
            o.step(dt, vi, pi)
            n += 1
        cpu_s = time.perf_counter() - t0
        o.close()
        out["cpu_baseline"] = {"value": n_boxes * n / cpu_s, "unit": "body-steps/s", "cores": 1, "kind": "port",
                               "sample": f"oracle (libm sin/cos, 1 thread) stepped {n} steps from the GPU's state at "
                                         f"step {skip}: {cpu_s:.1f} s"}
    return out


def run_adjoint(torch, flush, device, steps=240, seeds=512, repeats=3):
    """Differentiable throw-and-stack (64 boxes + a circle projectile, loss = squared distance of the
    stack's centre of mass from a target after `steps` steps): device time of the plain forward
    steps, of the same steps while recording the tape, and wall time of the backward pass over
    the tape (checkpoints every 16 steps, solver iterations recomputed); one world, and `seeds`
    worlds stepped as one batch."""
    out = {"workload": f"throw-and-stack: 8x8 boxes (half 0.25 m) + circle r 0.5 m, {steps} steps, dt 1/60, "
                       "8/3 iterations, checkpoint every 16 steps"}
    for name, scene in (("single_world", scenes.throw_stack(steps=steps)),
                        (f"batched_{seeds}_worlds", scenes.throw_stack_batch(seeds=seeds, steps=steps))):
        def fresh():
            w = b2g.B2world(gravity=scene["gravity"], num_worlds=scene["num_worlds"], device=device)
            w.set_allow_sleeping(False)
            scenes.build_world(w, scene)
            return w

        w = fresh()
        fwd_ms = timed_steps(w, scene, steps, flush, torch)
        w.close()
        w = fresh()
        w.tape_begin(steps)
        taped_ms = timed_steps(w, scene, steps, flush, torch)
        w.tape_end()
        d_final = _stack_loss_grad(w, scene)
        times = []
        for _ in range(repeats):  # the first call also allocates the work buffers
            flush.fill_(1.0)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            w.backward(d_final)
            times.append(time.perf_counter() - t0)
        info = w.tape_info()
        w.close()
        bwd_ms = 1e3 * min(times[1:] if len(times) > 1 else times)
        out[name] = {"worlds": int(scene["num_worlds"]), "dynamic_bodies": int(scene["n_dynamic"]),
                     "forward_ms_per_step": fwd_ms / steps, "taped_forward_ms_per_step": taped_ms / steps,
                     "backward_ms_per_step": bwd_ms / steps,
                     "backward_over_forward": bwd_ms / fwd_ms,
                     "taped_forward_plus_backward_over_forward": (taped_ms + bwd_ms) / fwd_ms,
                     "tape_slots": info["slots"], "device_bytes": info["device_bytes"],
                     "replay_mismatches": info["replay_mismatches"]}
    return out


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


SCENE_STEPS = 600  # the mixed-100k configuration runs 600 steps; the timed window is centred on its middle


def window_skip(args):
    """Untimed steps before the warm-up: --skip-steps, else the window of `steps` timed steps is centred
    on step 300 of the 600-step scene (the whole trajectory when steps >= 600)."""
    if args.skip_steps is not None:
        return args.skip_steps
    return max(0, SCENE_STEPS // 2 - args.warmup - args.steps // 2)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--scale", type=float, default=1.0, help="fraction of the 100k bodies (testing only)")
    ap.add_argument("--no-graphs", action="store_true", help="launch kernels directly instead of CUDA graphs")
    ap.add_argument("--batched-steps", type=int, default=300, help="steps of the 4096-world leg (0 skips it)")
    ap.add_argument("--adjoint-steps", type=int, default=240, help="steps of the differentiable leg (0 skips it)")
    ap.add_argument("--toi-pairs", type=int, default=1_000_000, help="pairs of the time-of-impact leg (0 skips it)")
    ap.add_argument("--continuous-steps", type=int, default=60,
                    help="timed steps of the continuous-physics leg (0 skips it)")
    ap.add_argument("--pile-steps", type=int, default=20, help="timed steps of the high-contact pile leg (0 skips it)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch configuration")
    ap.add_argument("--skip-steps", type=int, default=None,
                    help="untimed steps before the warm-up (default: centre the timed window on step 300)")
    ap.add_argument("--profile-window", action="store_true",
                    help="bracket the timed steps with cudaProfilerStart/Stop (ncu --profile-from-start off)")
    args = ap.parse_args()
    rank, world_size, local_rank = dist_info()
    n_half = int(50_000 * args.scale)
    scene = scenes.mixed(n_circles=n_half, n_polygons=n_half)
    stats = scene_stats(scene)
    skip = window_skip(args)
    first = skip + args.warmup + 1
    window = f"steps {first}-{first + args.steps - 1} of the {SCENE_STEPS}-step scene"
    config = {"workload": f"{WORKLOAD}; timed window: {window}", "bodies": stats["n_dynamic"],
              "fixtures": stats["n_fixtures"], "window": window,
              "velocity_iterations": 8, "position_iterations": 3, "dt": 1 / 60, "sleep": False,
              "continuous": False, "l2": "256 MiB flush between timed steps", "parallelism": "replicas",
              "cuda_graphs": not args.no_graphs}

    if args.impl == "reference":
        if rank != 0:
            return
        cb = run_cpu_baseline(scene, skip + args.warmup, budget_s=30.0, max_steps=max(args.steps, 3))
        line = {"metric": METRIC, "value": cb["value"], "unit": "body-steps/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "impl": "reference",
                "dtype": "f32", "data": "synthetic (seeded splitmix64)", "config": config, "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "vs_baseline": None,
                "note": "box2d-rs cannot be compiled here (no Rust toolchain); timed its faithful C++ restatement "
                        "on the same window of the same scene"}
        print(json.dumps(line))
        return

    import torch

    torch.cuda.set_device(local_rank)
    if world_size > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    dt, vi, pi = scene["dt"], scene["vi"], scene["pi"]
    if not args.no_autotune:
        # tune on a scratch world of the same scene, advanced to the middle of the timed window;
        # the measured world inherits the choice through the size-bucket cache
        t = b2g.B2world(gravity=scene["gravity"], device=local_rank)
        t.set_allow_sleeping(False)
        scenes.build_world(t, scene)
        for _ in range(skip + args.warmup + args.steps // 2):
            t.step(dt, vi, pi)
        t.autotune(dt, vi, pi, 6)
        tuned = tune_blocks_per_sm(torch, flush, t, dt, vi, pi)
        t.close()
    w = b2g.B2world(gravity=scene["gravity"], device=local_rank)
    w.set_allow_sleeping(False)
    w.set_continuous_physics(False)
    w.set_graph_capture(not args.no_graphs)
    if not args.no_autotune:
        w.set_launch_config(**tuned)
    scenes.build_world(w, scene)
    for _ in range(skip + args.warmup):
        w.step(dt, vi, pi)
    w.synchronize()
    config["launch_config"] = w.get_launch_config()

    sampler = ClockSampler(local_rank)
    if world_size > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler.start()
    if args.profile_window:
        torch.cuda.profiler.start()
    launches0 = w._lib.b2g_get_launch_count()
    total_ms = 0.0
    fine_ms = dict.fromkeys(b2g.B2world.PHASES + b2g.B2world.TREE_PHASES, 0.0)
    bytes_total = {}
    work = {"bp_node_visits": 0, "bp_leaf_checks": 0, "bp_moved_proxies": 0, "new_pairs": 0, "contacts": 0,
            "constraints": 0, "interior_slots": 0, "colours": 0, "hierarchy_rebuilds": 0,
            "bp_warp_max_visits": 0, "bp_warp_max_checks": 0}
    snap_at = set(int(x) for x in np.linspace(0, args.steps - 1, 4)) if rank == 0 and not args.no_cpu_baseline else set()
    snaps = []
    for k in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        w.step(dt, vi, pi)
        p = w.get_profile()  # synchronizes the world's stream; event times of this step
        total_ms += p["step"]
        for ph, v in w.get_phase_times(tree_split=True).items():
            fine_ms[ph] += v
        st = w.get_step_stats()  # this step's work counts (outside the timed events)
        st["hierarchy_rebuilds"] = int(st["hierarchy_age"] == 0)
        for key in work:
            work[key] += st[key]
        for ph, v in bytes_model(st, stats, vi, pi).items():
            bytes_total[ph] = bytes_total.get(ph, 0) + v
        if k in snap_at:  # outside the timed events: the state after this step
            snaps.append((skip + args.warmup + k + 1, snapshot(w)))
    launches = w._lib.b2g_get_launch_count() - launches0
    torch.cuda.synchronize()
    if args.profile_window:
        torch.cuda.profiler.stop()
    clocks = sampler.stop()
    counts = w.get_counts()
    w.close()

    # e2e: a fresh world over the same step window, stepped through the API with every body's
    # state read back into host memory each step (b2g_get_body_states_async)
    e2e_steps = args.e2e_steps if args.e2e_steps is not None else args.steps
    w = b2g.B2world(gravity=scene["gravity"], device=local_rank)
    w.set_allow_sleeping(False)
    w.set_continuous_physics(False)
    w.set_graph_capture(not args.no_graphs)
    if not args.no_autotune:
        w.set_launch_config(**tuned)
    scenes.build_world(w, scene)
    for _ in range(skip + args.warmup):
        w.step(dt, vi, pi)
    w.synchronize()
    # every step's states are copied into host memory (two buffers alternate); the copy of step k
    # runs on a second stream while step k + 1 is computed, and the last one is waited for
    states = [np.zeros(w.body_count, b2g.BODY_STATE) for _ in range(2)]
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        w.step(dt, vi, pi)
        w.get_body_states_async(states[k & 1])
    w.wait_body_states()
    e2e_s = time.perf_counter() - t0
    d2h = w.body_count * 32  # one b2g_body_state (32 bytes) per body
    w.close()

    if world_size > 1:
        t = torch.tensor([total_ms, e2e_s], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms, e2e_s = float(t[0]), float(t[1])
    units = stats["n_dynamic"] * args.steps * world_size
    value = units / (total_ms / 1e3)
    e2e_value = stats["n_dynamic"] * e2e_steps * world_size / e2e_s

    peak, peak_kind = load_peaks()
    # per phase: algorithmic bytes per step / the phase's mean CUDA-event time per step
    phase_time = {"solver": fine_ms["solver"], "collide": fine_ms["collide"], "bp_sort": fine_ms["bp_sort"],
                  "bp_hierarchy": fine_ms["bp_hierarchy"], "bp_traverse": fine_ms["bp_traverse"],
                  "merge": fine_ms["contact_merge"]}
    traffic_rec = {}
    tf = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if os.path.exists(tf):
        with open(tf) as f:
            rec = json.load(f)
        if rec.get("workload") == WORKLOAD and rec.get("window") == window:
            traffic_rec = rec.get("dram_bytes_per_launch", {})
    phases = {}
    for ph, ms in phase_time.items():
        if ms <= 0:
            continue
        b = bytes_total.get(ph, 0) / args.steps
        ach = b / (ms / args.steps / 1e3) / 1e9
        kern = PHASE_KERNEL[ph]
        phases[ph] = {"kernel": kern, "ms_per_step": ms / args.steps, "algorithmic_bytes_per_step": b,
                      "achieved": ach, "frac": ach / peak, "traffic": traffic_rec.get(kern)}
    dominant = max(phases, key=lambda k: phases[k]["ms_per_step"])
    d = phases[dominant]
    line = {
        "metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": world_size, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded splitmix64)",
        "config": config,
        "e2e": {"value": e2e_value, "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": d2h,
                "steps": e2e_steps, "window": window,
                "h2d_note": "B2world::step takes no per-step host input (dt and the iteration counts are scalar "
                            "arguments of b2g_step); every body's state is read back to host memory every step"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": d["kernel"], "kernel_phase": dominant, "achieved": d["achieved"],
                     "peak": peak, "unit": "GB/s", "frac": d["frac"], "peak_kind": peak_kind,
                     "traffic": d["traffic"], "algorithmic_bytes_per_launch": d["algorithmic_bytes_per_step"],
                     "traffic_note": ("DRAM bytes per launch from one ncu capture of the same window "
                                      "(profiles/roofline_traffic.json)") if d["traffic"] else None},
        "roofline_phases": phases,
        "work_per_step": {k: v / args.steps for k, v in work.items()},
        "phase_ms_per_step": {k: v / args.steps for k, v in fine_ms.items()},
        "counts_last_step": counts,
        "clocks": clocks,
    }
    if args.batched_steps > 0:
        line["batched"] = run_batched(torch, flush, local_rank, steps=args.batched_steps, warmup=args.warmup,
                                      rank=rank, world_size=world_size, autotune=not args.no_autotune)
    if args.adjoint_steps > 0 and rank == 0:
        line["adjoint"] = run_adjoint(torch, flush, local_rank, steps=args.adjoint_steps)
    if args.toi_pairs > 0 and rank == 0:
        line["time_of_impact"] = run_toi(args.toi_pairs)
    if args.continuous_steps > 0 and rank == 0:
        line["continuous"] = run_continuous(torch, flush, local_rank, steps=args.continuous_steps,
                                            warmup=args.warmup)
    if args.pile_steps > 0 and rank == 0:
        line["c3_pile"] = run_pile(torch, flush, local_rank, steps=args.pile_steps, warmup=args.warmup,
                                   cpu=not args.no_cpu_baseline)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = run_cpu_on_snapshots(scene, snaps)
    if rank == 0:
        print(json.dumps(line))
    if world_size > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
