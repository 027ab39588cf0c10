"""Generate tests/golden/golden_oracle.npz from the oracle (CPU restatement of box2d-rs).

The reference is Rust and cannot be built here (no cargo), so the golden vectors are the
oracle's own outputs on seeded inputs, committed so that (a) the oracle built on another
machine (the Arm GPU host) must reproduce them bit for bit, and (b) the GPU path is
checked against them in addition to the live oracle. All trigonometry uses the project's
correctly rounded sin/cos (identical on host and device).

Contents
  narrow_*        manifolds of 3000 random shape pairs (all five routines) at random poses
  pyr_*           8-row pyramid: body states after 30, 60 and 120 steps of 8/3
  mix_*           400-body mixed scene in a 20 m box: body states after 60 steps and the
                  sorted pair set of the last broadphase pass
Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "box2d-rs_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import b2g  # noqa: E402
import oracle  # noqa: E402
import scenes  # noqa: E402

OUT = os.path.join(HERE, "golden_oracle.npz")


def random_shape_pairs(n=3000, seed=21):
    """Shape pairs covering circle-circle, polygon-circle, polygon-polygon, edge-circle and
    edge-polygon (one- and two-sided edges), posed so that most pairs touch or nearly touch."""
    rng = scenes.SplitMix64(seed)
    da = b2g.fixture_defs(n)
    db = b2g.fixture_defs(n)
    kinds = rng.integers(n, 0, 4)
    sizes_a = rng.uniform(n, 0.2, 1.0)
    sizes_b = rng.uniform(n, 0.2, 1.0)
    nv_a = rng.integers(n, 3, 8)
    nv_b = rng.integers(n, 3, 8)
    va = scenes._polygon_vertices(rng, n, sizes_a, nv_a)
    vb = scenes._polygon_vertices(rng, n, sizes_b, nv_b)
    boxes = rng.integers(2 * n, 0, 1).reshape(n, 2)
    xa = np.zeros((n, 3), np.float32)
    xb = np.zeros((n, 3), np.float32)
    xa[:, 0] = rng.uniform(n, -1.0, 1.0)
    xa[:, 1] = rng.uniform(n, -1.0, 1.0)
    xa[:, 2] = rng.uniform(n, -3.2, 3.2)
    dist = rng.uniform(n, 0.0, 1.6)
    ang = rng.uniform(n, 0.0, 2.0 * np.pi)
    xb[:, 0] = xa[:, 0] + dist * np.cos(ang)
    xb[:, 1] = xa[:, 1] + dist * np.sin(ang)
    xb[:, 2] = rng.uniform(n, -3.2, 3.2)
    one_sided = rng.integers(n, 0, 1)
    for i in range(n):
        k = int(kinds[i])
        a, b = da[i : i + 1], db[i : i + 1]
        if k == 0:  # circle-circle
            a["shape_type"] = b2g.CIRCLE
            a["radius"] = sizes_a[i] * 0.5
            a["vertices"][0, 0] = (0.1, -0.05)
            b["shape_type"] = b2g.CIRCLE
            b["radius"] = sizes_b[i] * 0.5
        elif k == 1:  # polygon-circle
            a["shape_type"] = b2g.POLYGON
            a["vertex_count"] = nv_a[i]
            a["vertices"] = va[i]
            b["shape_type"] = b2g.CIRCLE
            b["radius"] = sizes_b[i] * 0.5
            b["vertices"][0, 0] = (0.02, 0.03)
        elif k == 2:  # polygon-polygon (hull or box)
            for d, v, nv, s, bx in ((a, va, nv_a, sizes_a, boxes[i, 0]), (b, vb, nv_b, sizes_b, boxes[i, 1])):
                d["shape_type"] = b2g.POLYGON
                if bx:
                    d["polygon_mode"] = b2g.POLYGON_BOX
                    d["box_half_extents"] = (s[i] * 0.6, s[i] * 0.4)
                else:
                    d["vertex_count"] = nv[i]
                    d["vertices"] = v[i]
        else:  # edge-circle or edge-polygon
            a["shape_type"] = b2g.EDGE
            a["vertices"][0, 0] = (-2.5, 0.3)
            a["vertices"][0, 1] = (-1.5, 0.0)
            a["vertices"][0, 2] = (1.5, 0.0)
            a["vertices"][0, 3] = (2.5, 0.4)
            a["one_sided"] = one_sided[i]
            xa[i] = (0.0, 0.0, 0.0)
            xb[i, 0] = dist[i] * 1.5 - 1.2
            xb[i, 1] = sizes_b[i] * 0.4 + 0.1 * np.cos(ang[i])
            if i % 2 == 0:
                b["shape_type"] = b2g.CIRCLE
                b["radius"] = sizes_b[i] * 0.5
            else:
                b["shape_type"] = b2g.POLYGON
                b["vertex_count"] = nv_b[i]
                b["vertices"] = vb[i]
    return da, xa, db, xb


def run_narrow(da, xa, db, xb):
    out = np.zeros(len(da), b2g.CONTACT_INFO)
    for i in range(len(da)):
        out[i] = oracle.collide(da[i : i + 1], xa[i], db[i : i + 1], xb[i])
    return out


def run_world(scene, steps, snapshots):
    w = oracle.OracleWorld(gravity=scene["gravity"])
    scenes.build_world(w, scene)
    res = {}
    for k in range(1, steps + 1):
        w.step(scene["dt"], scene["vi"], scene["pi"])
        if k in snapshots:
            res[k] = w.get_body_states()
    return res, w


def compute():
    oracle.set_trig(False)
    try:
        da, xa, db, xb = random_shape_pairs()
        out = {"narrow_def_a": da.view(np.uint8), "narrow_xf_a": xa, "narrow_def_b": db.view(np.uint8),
               "narrow_xf_b": xb, "narrow_out": run_narrow(da, xa, db, xb).view(np.uint8)}
        pyr = scenes.pyramid(rows=8, steps=120)
        res, _ = run_world(pyr, 120, (30, 60, 120))
        for k, v in res.items():
            out[f"pyr_{k}"] = v.view(np.uint8)
        mix = scenes.mixed(n_circles=200, n_polygons=200, size=20.0, seed=9)
        res, w = run_world(mix, 60, (60,))
        out["mix_60"] = res[60].view(np.uint8)
        p = w.get_pairs()
        out["mix_pairs"] = np.unique(p, axis=0) if len(p) else np.zeros((0, 2), np.uint32)
    finally:
        oracle.set_trig(True)
    return out


if __name__ == "__main__":
    np.savez_compressed(OUT, **compute())
    print("wrote", OUT, os.path.getsize(OUT), "bytes")
