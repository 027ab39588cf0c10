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


class MultiOracle:
    """One oracle world per world of a batched scene, addressed with the batch's global ids.

    The reference has one world per B2world; a batch of independent worlds is checked by
    running each in its own oracle and mapping body/fixture ids. Creation order inside each
    world follows the batch's order, so proxy ids keep the same relative order."""

    def __init__(self, scene, worlds=None, **kw):
        """worlds: the batch's worlds to restate (default all); the others are left out and their
        bodies and fixtures read as zeros."""
        bodies, fixtures = scene["bodies"], scene["fixtures"]
        wi = bodies["world_index"]
        self.n_bodies, self.n_fixtures = len(bodies), len(fixtures)
        self.worlds = []
        self.world_ids = list(range(scene["num_worlds"])) if worlds is None else [int(x) for x in worlds]
        self.fix_world = np.full(len(fixtures), -1, np.int64)
        self.fix_local = np.zeros(len(fixtures), np.int64)
        for w in self.world_ids:
            bidx = np.nonzero(wi == w)[0]
            remap = np.full(len(bodies), -1, np.int64)
            remap[bidx] = np.arange(len(bidx))
            fidx = np.nonzero(remap[fixtures["body"]] >= 0)[0]
            bd = bodies[bidx].copy()
            bd["world_index"] = 0
            fx = fixtures[fidx].copy()
            fx["body"] = remap[fx["body"]]
            o = oracle.OracleWorld(gravity=scene["gravity"], **kw)
            o.create_bodies(bd)
            o.create_fixtures(fx)
            self.fix_world[fidx] = w
            self.fix_local[fidx] = np.arange(len(fidx))
            self.worlds.append((o, bidx, fidx))

    def step(self, dt, vi, pi):
        for o, _, _ in self.worlds:
            o.step(dt, vi, pi)

    def body_mask(self):
        m = np.zeros(self.n_bodies, bool)
        for _, bidx, _ in self.worlds:
            m[bidx] = True
        return m

    def fixture_mask(self):
        return self.fix_world >= 0

    def import_state(self, bodies, fat_aabbs, contacts, inv_dt0):
        """Each restated world continues from its part of a batch's post-step state."""
        c = np.asarray(contacts)
        cw = self.fix_world[c["fixture_a"].astype(np.int64)] if len(c) else np.zeros(0, np.int64)
        for k, (o, bidx, fidx) in enumerate(self.worlds):
            cc = c[cw == self.world_ids[k]].copy()
            cc["fixture_a"] = self.fix_local[cc["fixture_a"].astype(np.int64)]
            cc["fixture_b"] = self.fix_local[cc["fixture_b"].astype(np.int64)]
            o.import_state(bodies[bidx], np.asarray(fat_aabbs)[fidx], cc, inv_dt0)

    def set_solver_order(self, pairs):
        p = np.asarray(pairs, np.int64).reshape(-1, 2)
        w = self.fix_world[p[:, 0]] if len(p) else np.zeros(0, np.int64)
        for k, (o, _, _) in enumerate(self.worlds):
            sel = p[w == self.world_ids[k]]
            o.set_solver_order(np.stack([self.fix_local[sel[:, 0]], self.fix_local[sel[:, 1]]], 1) if len(sel) else None)

    def hook_misses(self):
        return sum(o.hook_misses() for o, _, _ in self.worlds)

    def set_key_order(self, flag):
        for o, _, _ in self.worlds:
            o.set_key_order(flag)

    def get_awake(self):
        out = np.zeros(self.n_bodies, np.uint8)
        for o, bidx, _ in self.worlds:
            out[bidx] = o.get_awake()
        return out

    def toi_events(self):
        return sum(o.toi_events() for o, _, _ in self.worlds)

    def close(self):
        for o, _, _ in self.worlds:
            o.close()

    def get_body_states(self):
        out = np.zeros(self.n_bodies, b2g.BODY_STATE)
        for o, bidx, _ in self.worlds:
            out[bidx] = o.get_body_states()
        return out

    def get_pairs(self):
        res = [fidx[o.get_pairs()] for o, _, fidx in self.worlds]
        res = [r.reshape(-1, 2) for r in res if len(r)]
        if not res:
            return np.zeros((0, 2), np.uint32)
        p = np.concatenate(res)
        return np.stack([p.min(1), p.max(1)], 1).astype(np.uint32)

    def get_contacts(self):
        res = []
        for o, _, fidx in self.worlds:
            c = o.get_contacts().copy()
            c["fixture_a"] = fidx[c["fixture_a"]]
            c["fixture_b"] = fidx[c["fixture_b"]]
            res.append(c)
        return np.concatenate(res) if res else np.zeros(0, b2g.CONTACT_INFO)

    def get_proxies(self):
        aabbs = np.zeros((self.n_fixtures, 4), np.float32)
        moved = np.zeros(self.n_fixtures, np.uint8)
        ids = np.zeros(self.n_fixtures, np.int32)
        for o, _, fidx in self.worlds:
            a, m, i = o.get_proxies()
            aabbs[fidx], moved[fidx], ids[fidx] = a, m, i
        return aabbs, moved, ids


def make_pair(scene, record_pairs=True, record_events=False, warm_starting=True):
    oracle.set_trig(False)  # the project's correctly rounded sin/cos, which the GPU uses
    gpu = b2g.B2world(gravity=scene["gravity"], num_worlds=scene.get("num_worlds", 1))
    gpu.set_allow_sleeping(scene.get("allow_sleep", False))
    gpu.set_warm_starting(warm_starting)
    continuous = bool(scene.get("continuous", False))
    gpu.set_continuous_physics(continuous)
    gpu.set_toi_schedule(scene.get("toi_schedule", b2g.TOI_SIDE_BY_SIDE))
    gpu.set_record_pairs(record_pairs)
    gpu.set_contact_events(record_events)
    gpu.set_part_solve(scene.get("part_solve", True))
    kw = dict(allow_sleep=scene.get("allow_sleep", False), warm_starting=warm_starting, record_events=record_events,
              continuous=continuous)
    scenes.build_world(gpu, scene)
    if scene.get("num_worlds", 1) > 1:
        ora = MultiOracle(scene, **kw)
    else:
        ora = oracle.OracleWorld(gravity=scene["gravity"], **kw)
        scenes.build_world(ora, scene)
    # the contact-list order choices (collide's wake order, solve_toi's ties and island order)
    # follow the GPU's key order
    ora.set_key_order(True)
    if scene.get("joints") is not None and len(scene["joints"]):
        assert scene.get("num_worlds", 1) == 1, "joints are checked on single worlds"
        ora.set_joint_order(gpu.get_joint_order())
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


def _sorted_by_pair(c):
    c = np.asarray(c)
    return c[np.lexsort((c["fixture_b"], c["fixture_a"]))] if len(c) else c


def manifold_diff_fast(gpu_contacts, ora_contacts):
    """manifold_diff with array operations, for tables of hundreds of thousands of contacts. Returns
    (number of fixture pairs in one table only, id mismatches, max point/impulse difference)."""
    g, o = _sorted_by_pair(gpu_contacts), _sorted_by_pair(ora_contacts)
    kg = (g["fixture_a"].astype(np.uint64) << np.uint64(32)) | g["fixture_b"].astype(np.uint64)
    ko = (o["fixture_a"].astype(np.uint64) << np.uint64(32)) | o["fixture_b"].astype(np.uint64)
    common, ig, io = np.intersect1d(kg, ko, assume_unique=True, return_indices=True)
    key_mismatch = len(kg) + len(ko) - 2 * len(common)
    a, b = g[ig], o[io]
    same_head = (a["touching"] == b["touching"]) & (a["point_count"] == b["point_count"])
    n = a["point_count"]
    typed = same_head & (n > 0)
    type_ok = ~typed | (a["manifold_type"] == b["manifold_type"])
    ids_ok = np.ones(len(a), bool)
    for j in range(2):
        sel = typed & type_ok & (n > j)
        ids_ok &= ~sel | (a["point_id"][:, j] == b["point_id"][:, j])
    id_mismatch = int((~same_head).sum() + (~type_ok).sum() + (same_head & type_ok & ~ids_ok).sum())
    worst = 0.0
    cmp = typed & type_ok
    if cmp.any():
        aa, bb = a[cmp], b[cmp]
        for f in ("local_normal", "local_point"):
            worst = max(worst, float(np.abs(aa[f].astype(np.float64) - bb[f]).max()))
        nn = aa["point_count"]
        for j in range(2):
            sel = nn > j
            if sel.any():
                for f in ("point_local",):
                    worst = max(worst, float(np.abs(aa[f][sel, j].astype(np.float64) - bb[f][sel, j]).max()))
                for f in ("normal_impulse", "tangent_impulse"):
                    worst = max(worst, float(np.abs(aa[f][sel, j].astype(np.float64) - bb[f][sel, j]).max()))
    return key_mismatch, id_mismatch, worst


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


def drop_transient(contacts, aabbs):
    """Contacts without a manifold whose two fat AABBs no longer overlap are left out. With
    continuous physics the GPU solves independent time-of-impact events side by side, and a pair of
    two such bodies can be found (or missed) at a moment their fat AABBs overlap in one order of the
    events and not in the other; such a contact never gets a manifold and the next collide removes
    it. Contacts that overlap at the end of the step are found in either order."""
    c = np.asarray(contacts)
    if len(c) == 0:
        return c
    a = aabbs[c["fixture_a"].astype(np.int64)]
    b = aabbs[c["fixture_b"].astype(np.int64)]
    apart = (b[:, 0] - a[:, 2] > 0) | (b[:, 1] - a[:, 3] > 0) | (a[:, 0] - b[:, 2] > 0) | (a[:, 1] - b[:, 3] > 0)
    keep = ~apart | (c["touching"] != 0) | (c["point_count"] > 0)
    return c[keep]


def _pair_keys(pairs, fix_mask=None):
    p = np.asarray(pairs, np.int64).reshape(-1, 2)
    if fix_mask is not None and len(p):
        p = p[fix_mask[p[:, 0]] & fix_mask[p[:, 1]]]
    if len(p) == 0:
        return np.zeros(0, np.int64)
    return np.unique(np.minimum(p[:, 0], p[:, 1]) << 32 | np.maximum(p[:, 0], p[:, 1]))


def _restrict_contacts(c, fix_mask):
    c = np.asarray(c)
    if fix_mask is None or len(c) == 0:
        return c
    return c[fix_mask[c["fixture_a"].astype(np.int64)]]


def lockstep_window(scene, steps, skip=0, worlds=None, check_pairs=True, part_solve=None):
    """Lockstep parity on a window of a scene: the GPU steps `skip` steps alone, the oracle imports its
    post-step state (bodies, fat AABBs, the contact table with manifolds and impulses, the warm-start
    ratio), then both step `steps` more, the oracle in the GPU's solve order. For a batched scene,
    `worlds` selects the worlds the oracle restates (the GPU steps every world); only those worlds'
    bodies, proxies, pairs and contacts are compared. Array comparisons throughout, so it scales to
    the configurations' full sizes. Returns per-step records."""
    oracle.set_trig(False)
    nw = scene.get("num_worlds", 1)
    gpu = b2g.B2world(gravity=scene["gravity"], num_worlds=nw,
                      contact_capacity=scene.get("contact_capacity", 0), pair_capacity=scene.get("pair_capacity", 0))
    gpu.set_allow_sleeping(False)
    gpu.set_record_pairs(check_pairs)
    gpu.set_auto_grow(bool(scene.get("auto_grow", False)))
    if part_solve is not None:
        gpu.set_part_solve(part_solve)
    scenes.build_world(gpu, scene)
    dt, vi, pi = scene["dt"], scene["vi"], scene["pi"]
    for _ in range(skip):
        gpu.step(dt, vi, pi)
    if nw > 1:
        ora = MultiOracle(scene, worlds=worlds, allow_sleep=False)
        bmask, fmask = ora.body_mask(), ora.fixture_mask()
    else:
        ora = oracle.OracleWorld(gravity=scene["gravity"], allow_sleep=False)
        scenes.build_world(ora, scene)
        bmask, fmask = None, None
    ora.set_key_order(True)
    if skip > 0:
        aabbs, _ = gpu.get_proxies()
        ora.import_state(gpu.get_body_states(), aabbs, gpu.get_contacts(), np.float32(1.0) / dt)
    out = []
    for k in range(steps):
        gpu.step(dt, vi, pi)
        order = gpu.get_solver_order()
        ora.set_solver_order(order)
        ora.step(dt, vi, pi)
        rec = {"step": skip + k + 1, "hook_misses": ora.hook_misses(), "constraints": len(order)}
        gs, os_ = gpu.get_body_states(), ora.get_body_states()
        if bmask is not None:
            gs, os_ = gs[bmask], os_[bmask]
        rec["body_abs"], rec["body_rel"] = body_diff(gs, os_)
        rec["bitexact_bodies"] = all(np.array_equal(gs[f], os_[f]) for f in BODY_FIELDS)
        if check_pairs:
            gp, op = _pair_keys(gpu.get_pairs(), fmask), _pair_keys(ora.get_pairs(), fmask)
            rec["pairs_equal"] = bool(np.array_equal(gp, op))
            rec["pairs"] = int(len(gp))
        ga, _ = gpu.get_proxies()
        oa, _, _ = ora.get_proxies()
        if fmask is not None:
            ga, oa = ga[fmask], oa[fmask]
        rec["fat_aabb_equal"] = bool(np.array_equal(ga, oa))
        gc = _restrict_contacts(gpu.get_contacts(), fmask)
        oc = ora.get_contacts()
        km, im, worst = manifold_diff_fast(gc, oc)
        rec["contacts"] = int(len(gc))
        rec["contact_key_mismatch"] = km
        rec["contact_id_mismatch"] = im
        rec["manifold_max_diff"] = worst
        out.append(rec)
    gpu.close()
    if hasattr(ora, "close"):
        ora.close()
    return out


def lockstep(scene, steps, check_pairs=True, check_contacts=True, resync=False, on_step=None, before_step=None):
    """Step GPU and oracle in lockstep; returns per-step records of the differences."""
    gpu, ora = make_pair(scene, record_pairs=check_pairs)
    continuous = bool(scene.get("continuous", False))
    dt, vi, pi = scene["dt"], scene["vi"], scene["pi"]
    out = []
    for k in range(steps):
        if before_step is not None:
            before_step(k, gpu, ora)  # the same world edits on both sides
        gpu.step(dt, vi, pi)
        order = gpu.get_solver_order()
        ora.set_solver_order(order)
        ora.step(dt, vi, pi)
        rec = {"step": k, "hook_misses": ora.hook_misses(), "constraints": len(order)}
        gs = gpu.get_body_states()
        os_ = ora.get_body_states()
        rec["body_abs"], rec["body_rel"] = body_diff(gs, os_)
        rec["bitexact_bodies"] = all(np.array_equal(gs[f], os_[f]) for f in BODY_FIELDS)
        rec["awake_equal"] = bool(np.array_equal(gpu.get_awake(), ora.get_awake()))
        if getattr(gpu, "joint_count", 0):
            rec["joint_impulses_equal"] = bool(np.array_equal(gpu.get_joint_impulses(), ora.get_joint_impulses()))
        rec["awake"] = int(gpu.get_awake().sum())
        if check_pairs:
            gp, op = pair_set(gpu.get_pairs()), pair_set(ora.get_pairs())
            rec["pairs_equal"] = gp == op
            rec["pairs"] = len(gp)
            rec["pair_sym_diff"] = len(gp ^ op)
        ga, _ = gpu.get_proxies()
        oa, _, _ = ora.get_proxies()
        rec["fat_aabb_equal"] = bool(np.array_equal(ga, oa))
        if check_contacts:
            gc, oc = gpu.get_contacts(), ora.get_contacts()
            if continuous:
                gc, oc = drop_transient(gc, ga), drop_transient(oc, oa)
            km, im, worst = manifold_diff(gc, oc)
            rec["contact_key_mismatch"] = len(km)
            rec["contact_id_mismatch"] = im
            rec["manifold_max_diff"] = worst
        out.append(rec)
        if on_step is not None:
            on_step(rec)
    return out, gpu, ora


def energy(states, mass, gravity):
    """Kinetic energy (translation + rotation about the centre of mass) and potential energy
    (-m g.c) summed over all bodies; mass is b2g.B2world.get_mass_data() (static bodies have 0)."""
    m = mass[:, 0].astype(np.float64)
    inertia = mass[:, 2].astype(np.float64)
    v = states["linear_velocity"].astype(np.float64)
    w = states["angular_velocity"].astype(np.float64)
    c = states["world_center"].astype(np.float64)
    ke = 0.5 * float((m * (v * v).sum(1) + inertia * w * w).sum())
    pe = -float((m * (c @ np.asarray(gravity, np.float64))).sum())
    return ke, pe


def separations(contacts, states, radius, fixture_body):
    """Separation of every touching manifold point, from each contact's local manifold and the
    bodies' current transforms, as B2positionSolverManifold::initialize computes it
    (b2_contact_solver_private.rs:600-642). radius: per fixture; fixture_body: body per fixture."""
    out = []
    p = states["position"].astype(np.float64)
    a = states["angle"].astype(np.float64)
    for ct in contacts:
        n = int(ct["point_count"])
        if not ct["touching"] or n == 0:
            continue
        fa, fb = int(ct["fixture_a"]), int(ct["fixture_b"])
        ba, bb = int(fixture_body[fa]), int(fixture_body[fb])
        ra, rb = float(radius[fa]), float(radius[fb])

        def xf(b, v):
            s, c = np.sin(a[b]), np.cos(a[b])
            return np.array([c * v[0] - s * v[1] + p[b, 0], s * v[0] + c * v[1] + p[b, 1]])

        def rot(b, v):
            s, c = np.sin(a[b]), np.cos(a[b])
            return np.array([c * v[0] - s * v[1], s * v[0] + c * v[1]])

        ln, lp = ct["local_normal"].astype(np.float64), ct["local_point"].astype(np.float64)
        pts = ct["point_local"].astype(np.float64)
        mt = int(ct["manifold_type"])
        for j in range(n):
            if mt == 0:
                pa, pb = xf(ba, lp), xf(bb, pts[0])
                out.append(float(np.linalg.norm(pb - pa)) - ra - rb)
            elif mt == 1:
                nrm, plane, clip = rot(ba, ln), xf(ba, lp), xf(bb, pts[j])
                out.append(float((clip - plane) @ nrm) - ra - rb)
            else:
                nrm, plane, clip = rot(bb, ln), xf(bb, lp), xf(ba, pts[j])
                out.append(float((clip - plane) @ nrm) - ra - rb)
    return np.array(out)
