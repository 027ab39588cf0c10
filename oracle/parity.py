"""Lockstep parity harness — TEST INFRASTRUCTURE ONLY.

Builds one scene into the GPU world (b2g.B2world) and into the oracle (the CPU
restatement of box2d-rs's step), then steps both: after each GPU step the GPU's
solve order (its constraint colouring) is handed to the oracle's ordering hook, so
the oracle solves every island in the same Gauss-Seidel order, and the two states are
compared. Used by tests/ and by __graft_entry__.smoke().
"""
from __future__ import annotations

import os
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, _HERE)
sys.path.insert(0, os.path.join(os.path.dirname(_HERE), "box2d-rs_gb300"))

import b2g  # noqa: E402
import oracle  # noqa: E402
import scenes  # noqa: E402

BODY_FIELDS = ("position", "angle", "linear_velocity", "angular_velocity", "world_center")


def make_pair(scene, record_pairs=True, record_events=False, warm_starting=True):
    oracle.set_trig(False)  # the project's correctly rounded sin/cos, which the GPU uses
    gpu = b2g.B2world(gravity=scene["gravity"], num_worlds=scene.get("num_worlds", 1))
    gpu.set_allow_sleeping(scene.get("allow_sleep", False))
    gpu.set_warm_starting(warm_starting)
    gpu.set_continuous_physics(False)
    gpu.set_record_pairs(record_pairs)
    gpu.set_contact_events(record_events)
    ora = oracle.OracleWorld(gravity=scene["gravity"], allow_sleep=scene.get("allow_sleep", False),
                             warm_starting=warm_starting, record_events=record_events)
    scenes.build_world(gpu, scene)
    scenes.build_world(ora, scene)
    return gpu, ora


def body_diff(a, b):
    """Largest absolute and relative difference over all body state fields."""
    worst_abs, worst_rel = 0.0, 0.0
    for f in BODY_FIELDS:
        x = np.asarray(a[f], np.float64)
        y = np.asarray(b[f], np.float64)
        d = np.abs(x - y)
        if d.size:
            worst_abs = max(worst_abs, float(d.max()))
            worst_rel = max(worst_rel, float((d / np.maximum(1.0, np.abs(y))).max()))
    return worst_abs, worst_rel


def pair_set(pairs):
    p = np.asarray(pairs, np.uint32).reshape(-1, 2)
    if len(p) == 0:
        return set()
    return set(map(tuple, np.unique(p, axis=0).tolist()))


def contact_map(contacts):
    return {(int(c["fixture_a"]), int(c["fixture_b"])): c for c in contacts}


def manifold_diff(gpu_contacts, ora_contacts):
    """Compare live contacts by fixture pair. Returns (missing/extra keys, id mismatches, max point diff)."""
    g = contact_map(gpu_contacts)
    o = contact_map(ora_contacts)
    key_mismatch = set(g) ^ set(o)
    id_mismatch = 0
    worst = 0.0
    for k in set(g) & set(o):
        a, b = g[k], o[k]
        if int(a["touching"]) != int(b["touching"]) or int(a["point_count"]) != int(b["point_count"]):
            id_mismatch += 1
            continue
        n = int(a["point_count"])
        if n == 0:
            continue
        if int(a["manifold_type"]) != int(b["manifold_type"]):
            id_mismatch += 1
            continue
        if list(a["point_id"][:n]) != list(b["point_id"][:n]):
            id_mismatch += 1
        for f in ("local_normal", "local_point"):
            worst = max(worst, float(np.abs(a[f].astype(np.float64) - b[f]).max()))
        worst = max(worst, float(np.abs(a["point_local"][:n].astype(np.float64) - b["point_local"][:n]).max()))
        worst = max(worst, float(np.abs(a["normal_impulse"][:n].astype(np.float64) - b["normal_impulse"][:n]).max()))
        worst = max(worst, float(np.abs(a["tangent_impulse"][:n].astype(np.float64) - b["tangent_impulse"][:n]).max()))
    return key_mismatch, id_mismatch, worst


def lockstep(scene, steps, check_pairs=True, check_contacts=True, resync=False, on_step=None):
    """Step GPU and oracle in lockstep; returns per-step records of the differences."""
    gpu, ora = make_pair(scene, record_pairs=check_pairs)
    dt, vi, pi = scene["dt"], scene["vi"], scene["pi"]
    out = []
    for k in range(steps):
        gpu.step(dt, vi, pi)
        order = gpu.get_solver_order()
        ora.set_solver_order(order)
        ora.step(dt, vi, pi)
        rec = {"step": k, "hook_misses": ora.hook_misses(), "constraints": len(order)}
        gs = gpu.get_body_states()
        os_ = ora.get_body_states()
        rec["body_abs"], rec["body_rel"] = body_diff(gs, os_)
        rec["bitexact_bodies"] = all(np.array_equal(gs[f], os_[f]) for f in BODY_FIELDS)
        if check_pairs:
            gp, op = pair_set(gpu.get_pairs()), pair_set(ora.get_pairs())
            rec["pairs_equal"] = gp == op
            rec["pairs"] = len(gp)
            rec["pair_sym_diff"] = len(gp ^ op)
        if check_contacts:
            km, im, worst = manifold_diff(gpu.get_contacts(), ora.get_contacts())
            rec["contact_key_mismatch"] = len(km)
            rec["contact_id_mismatch"] = im
            rec["manifold_max_diff"] = worst
        ga, _ = gpu.get_proxies()
        oa, _, _ = ora.get_proxies()
        rec["fat_aabb_equal"] = bool(np.array_equal(ga, oa))
        out.append(rec)
        if on_step is not None:
            on_step(rec)
    return out, gpu, ora
