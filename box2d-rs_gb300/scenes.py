"""Seeded synthetic scenes with the shapes and sizes of the benchmark workloads.

No public dataset is involved: every scene is generated here from a splitmix64
stream, so the GPU world and the CPU oracle receive identical f32 inputs.

  pyramid        20-row box pyramid (box2d-rs examples/testbed/tests/pyramid.rs:50-89),
                 210 boxes, half-extent 0.5, density 5, friction 0.6, edge ground 80 m
  mixed          50k circles (r 0.1-0.5) + 50k convex 3-8-gons (extent 0.1-0.6) in a
                 1000 x 1000 m box of static edge walls, density 1, friction 0.4, v ~ N(0,1)
  pile           boxes (half-extents 0.05-0.2, random angle) dropped into a 100 x 400 m
                 walled container, density 1, friction 0.6
  batched        independent worlds with log-uniform 16-2048 bodies each (circles, boxes,
                 3-8-gons of size 0.1-0.6) above their own ground
  throw_stack    8 x 8 stack of boxes (half-extent 0.25) and a circle projectile (r 0.5)
  hello_world    box2d-rs tests/test.rs:26-102
  toi_rain       fast bodies (60-250 m/s) onto thin static plates, for continuous physics
  bridge         30 planks joined by revolute joints, bodies dropped on it, a motor and limits
"""
from __future__ import annotations

import math

import numpy as np

import b2g

F32 = np.float32
MASK64 = (1 << 64) - 1


class SplitMix64:
    """splitmix64 (Steele, Lea, Flood 2014) producing numpy arrays of uniforms."""

    def __init__(self, seed: int):
        self.state = np.uint64(seed & MASK64)

    def next_u64(self, n: int) -> np.ndarray:
        with np.errstate(over="ignore"):
            inc = np.uint64(0x9E3779B97F4A7C15)
            z = self.state + inc * np.arange(1, n + 1, dtype=np.uint64)
            self.state = z[-1] if n > 0 else self.state
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
        return z

    def uniform(self, n, lo=0.0, hi=1.0) -> np.ndarray:
        u = (self.next_u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))
        return lo + (hi - lo) * u

    def normal(self, n) -> np.ndarray:
        u1 = self.uniform(n)
        u2 = self.uniform(n)
        return np.sqrt(-2.0 * np.log1p(-u1)) * np.array([math.cos(2.0 * math.pi * t) for t in u2])

    def integers(self, n, lo, hi_inclusive) -> np.ndarray:
        span = hi_inclusive - lo + 1
        return lo + (self.next_u64(n) % np.uint64(span)).astype(np.int64)


def _scene(name, bodies, fixtures, steps, gravity=(0.0, -10.0), dt=1.0 / 60.0, vi=8, pi=3, num_worlds=1, **extra):
    s = {
        "name": name,
        "bodies": bodies,
        "fixtures": fixtures,
        "gravity": gravity,
        "dt": F32(dt),
        "vi": vi,
        "pi": pi,
        "steps": steps,
        "num_worlds": num_worlds,
        "allow_sleep": False,
        "n_dynamic": int((bodies["type"] == b2g.DYNAMIC).sum()),
    }
    s.update(extra)
    return s


def _walls(body, corners, friction):
    """Two-sided edges along a closed polyline of corners."""
    n = len(corners)
    f = b2g.fixture_defs(n)
    f["body"] = body
    f["shape_type"] = b2g.EDGE
    for i in range(n):
        f["vertices"][i, 1] = corners[i]
        f["vertices"][i, 2] = corners[(i + 1) % n]
    f["friction"] = friction
    return f


_ANGLE_COS = np.zeros((9, 8))
_ANGLE_SIN = np.zeros((9, 8))
for _n in range(3, 9):
    for _k in range(_n):
        _ANGLE_COS[_n, _k] = math.cos(2.0 * math.pi * _k / _n)
        _ANGLE_SIN[_n, _k] = math.sin(2.0 * math.pi * _k / _n)


def _polygon_vertices(rng: SplitMix64, count: int, extents: np.ndarray, nverts: np.ndarray) -> np.ndarray:
    """Convex n-gons with vertices at angles 2*pi*k/n and radii extent*(0.8..1.0).

    The angles come from a table of libm cos/sin values, so the vertices are identical on
    every machine; unused vertex slots stay zero."""
    jitter = rng.uniform(count * 8, 0.8, 1.0).reshape(count, 8)
    n = np.asarray(nverts, np.int64).reshape(-1)
    r = np.asarray(extents, np.float64).reshape(-1, 1) * jitter
    used = np.arange(8)[None, :] < n[:, None]
    out = np.zeros((count, 8, 2), np.float32)
    out[:, :, 0] = np.where(used, r * _ANGLE_COS[n], 0.0)
    out[:, :, 1] = np.where(used, r * _ANGLE_SIN[n], 0.0)
    return out


def pyramid(rows=20, friction=0.6, steps=600):
    """20-row pyramid of 210 boxes on a two-sided edge ground (pyramid.rs:50-89)."""
    n = rows * (rows + 1) // 2
    bodies = b2g.body_defs(n + 1)
    bodies["allow_sleep"] = 0
    bodies[0]["type"] = b2g.STATIC
    fixtures = b2g.fixture_defs(n + 1)
    fixtures[0]["body"] = 0
    fixtures[0]["shape_type"] = b2g.EDGE
    fixtures[0]["vertices"][1] = (-40.0, 0.0)
    fixtures[0]["vertices"][2] = (40.0, 0.0)
    fixtures[0]["friction"] = friction
    x = np.array([-7.0, 0.75], F32)
    dx = np.array([0.5625, 1.25], F32)
    dy = np.array([1.125, 0.0], F32)
    k = 1
    for i in range(rows):
        y = x.copy()
        for _ in range(i, rows):
            bodies[k]["type"] = b2g.DYNAMIC
            bodies[k]["position"] = y
            fixtures[k]["body"] = k
            fixtures[k]["shape_type"] = b2g.POLYGON
            fixtures[k]["polygon_mode"] = b2g.POLYGON_BOX
            fixtures[k]["box_half_extents"] = (0.5, 0.5)
            fixtures[k]["density"] = 5.0
            fixtures[k]["friction"] = friction
            y = (y + dy).astype(F32)
            k += 1
        x = (x + dx).astype(F32)
    return _scene("pyramid", bodies, fixtures, steps)


def mixed(n_circles=50_000, n_polygons=50_000, size=1000.0, seed=2, steps=600, gravity=(0.0, -10.0)):
    """Mixed circles + convex polygons in a square box of edge walls."""
    rng = SplitMix64(seed)
    n = n_circles + n_polygons
    bodies = b2g.body_defs(n + 1)
    bodies["allow_sleep"] = 0
    bodies[0]["type"] = b2g.STATIC
    dyn = bodies[1:]
    dyn["type"] = b2g.DYNAMIC
    margin = 1.0
    dyn["position"][:, 0] = rng.uniform(n, margin, size - margin)
    dyn["position"][:, 1] = rng.uniform(n, margin, size - margin)
    dyn["angle"] = rng.uniform(n, 0.0, 2.0 * math.pi)
    dyn["linear_velocity"][:, 0] = rng.normal(n)
    dyn["linear_velocity"][:, 1] = rng.normal(n)
    walls = _walls(0, [(0.0, 0.0), (size, 0.0), (size, size), (0.0, size)], 0.4)
    fix = b2g.fixture_defs(n)
    fix["body"] = np.arange(1, n + 1)
    fix["density"] = 1.0
    fix["friction"] = 0.4
    order = rng.uniform(n).argsort(kind="stable")  # interleave circles and polygons
    is_circle = np.zeros(n, bool)
    is_circle[order[:n_circles]] = True
    ci = np.nonzero(is_circle)[0]
    pi_ = np.nonzero(~is_circle)[0]
    fix["shape_type"][ci] = b2g.CIRCLE
    fix["radius"][ci] = rng.uniform(len(ci), 0.1, 0.5)
    fix["shape_type"][pi_] = b2g.POLYGON
    fix["polygon_mode"][pi_] = b2g.POLYGON_HULL
    nv = rng.integers(len(pi_), 3, 8)
    fix["vertex_count"][pi_] = nv
    fix["vertices"][pi_] = _polygon_vertices(rng, len(pi_), rng.uniform(len(pi_), 0.1, 0.6), nv)
    fixtures = np.concatenate([walls, fix])
    return _scene("mixed", bodies, fixtures, steps, gravity=gravity)


def pile(n_boxes=250_000, width=100.0, height=400.0, seed=3, steps=1000, spacing=0.6):
    """Boxes on a jittered grid above a walled container; they fall in and settle."""
    rng = SplitMix64(seed)
    bodies = b2g.body_defs(n_boxes + 1)
    bodies["allow_sleep"] = 0
    cols = int((width - 2 * spacing) / spacing)
    idx = np.arange(n_boxes)
    dyn = bodies[1:]
    dyn["type"] = b2g.DYNAMIC
    dyn["position"][:, 0] = spacing + (idx % cols) * spacing + rng.uniform(n_boxes, -0.01, 0.01)
    dyn["position"][:, 1] = spacing + (idx // cols) * spacing
    dyn["angle"] = rng.uniform(n_boxes, 0.0, 2.0 * math.pi)
    walls = _walls(0, [(0.0, height), (0.0, 0.0), (width, 0.0), (width, height)], 0.6)[:3]
    fix = b2g.fixture_defs(n_boxes)
    fix["body"] = np.arange(1, n_boxes + 1)
    fix["shape_type"] = b2g.POLYGON
    fix["polygon_mode"] = b2g.POLYGON_BOX
    fix["box_half_extents"][:, 0] = rng.uniform(n_boxes, 0.05, 0.2)
    fix["box_half_extents"][:, 1] = rng.uniform(n_boxes, 0.05, 0.2)
    fix["density"] = 1.0
    fix["friction"] = 0.6
    return _scene("pile", bodies, np.concatenate([walls, fix]), steps)


def batched(num_worlds=4096, lo=16, hi=2048, seed=4, steps=300):
    """Independent worlds; world w has log-uniform(lo, hi) dynamic bodies above its own ground."""
    rng = SplitMix64(seed)
    counts = np.exp(rng.uniform(num_worlds, math.log(lo), math.log(hi))).astype(np.int64)
    counts = np.clip(counts, lo, hi)
    total = int(counts.sum()) + num_worlds
    bodies = b2g.body_defs(total)
    bodies["allow_sleep"] = 0
    fixtures = b2g.fixture_defs(total)
    kinds = rng.integers(total, 0, 2)          # 0 circle, 1 box, 2 n-gon
    sizes = rng.uniform(total, 0.1, 0.6)
    halfx = rng.uniform(total, 0.05, 0.3)
    halfy = rng.uniform(total, 0.05, 0.3)
    nv = rng.integers(total, 3, 8)
    verts = _polygon_vertices(rng, total, sizes, nv)
    angles = rng.uniform(total, 0.0, 2.0 * math.pi)
    jit = rng.uniform(2 * total, -0.05, 0.05).reshape(total, 2)
    k = 0
    spacing = 1.3
    for w in range(num_worlds):
        n = int(counts[w])
        cols = int(math.ceil(math.sqrt(n)))
        half = 0.5 * cols * spacing + 5.0
        bodies[k]["type"] = b2g.STATIC
        bodies[k]["world_index"] = w
        fixtures[k]["body"] = k
        fixtures[k]["shape_type"] = b2g.EDGE
        fixtures[k]["vertices"][1] = (-half, 0.0)
        fixtures[k]["vertices"][2] = (half, 0.0)
        fixtures[k]["friction"] = 0.6
        ground = k
        k += 1
        j = np.arange(n)
        sl = slice(k, k + n)
        bodies[sl]["type"] = b2g.DYNAMIC
        bodies[sl]["world_index"] = w
        bodies[sl]["position"][:, 0] = -0.5 * cols * spacing + (j % cols) * spacing + jit[sl, 0]
        bodies[sl]["position"][:, 1] = 1.0 + (j // cols) * spacing + jit[sl, 1]
        bodies[sl]["angle"] = angles[sl]
        f = fixtures[sl]
        f["body"] = np.arange(k, k + n)
        f["density"] = 1.0
        f["friction"] = 0.6
        kd = kinds[sl]
        c = kd == 0
        f["shape_type"][c] = b2g.CIRCLE
        f["radius"][c] = 0.5 * sizes[sl][c]
        b = kd == 1
        f["shape_type"][b] = b2g.POLYGON
        f["polygon_mode"][b] = b2g.POLYGON_BOX
        f["box_half_extents"][b, 0] = halfx[sl][b]
        f["box_half_extents"][b, 1] = halfy[sl][b]
        g = kd == 2
        f["shape_type"][g] = b2g.POLYGON
        f["polygon_mode"][g] = b2g.POLYGON_HULL
        f["vertex_count"][g] = nv[sl][g]
        f["vertices"][g] = verts[sl][g]
        fixtures[sl] = f
        k += n
        del ground
    return _scene("batched", bodies, fixtures, steps, num_worlds=num_worlds, world_body_counts=counts)


def throw_stack(seed=5, steps=240, rows=8, cols=8, half=0.25, projectile_velocity=(12.0, 3.0)):
    """8 x 8 box stack and a circle projectile thrown at it, above an edge ground."""
    rng = SplitMix64(seed)
    n = rows * cols
    bodies = b2g.body_defs(n + 2)
    bodies["allow_sleep"] = 0
    fixtures = b2g.fixture_defs(n + 2)
    fixtures[0]["body"] = 0
    fixtures[0]["shape_type"] = b2g.EDGE
    fixtures[0]["vertices"][1] = (-40.0, 0.0)
    fixtures[0]["vertices"][2] = (40.0, 0.0)
    fixtures[0]["friction"] = 0.6
    j = np.arange(n)
    sl = slice(1, n + 1)
    bodies[sl]["type"] = b2g.DYNAMIC
    bodies[sl]["position"][:, 0] = 4.0 + (j % cols) * (2 * half + 0.01)
    bodies[sl]["position"][:, 1] = half + (j // cols) * (2 * half + 0.005)
    f = fixtures[sl]
    f["body"] = np.arange(1, n + 1)
    f["shape_type"] = b2g.POLYGON
    f["polygon_mode"] = b2g.POLYGON_BOX
    f["box_half_extents"] = (half, half)
    f["density"] = 1.0
    f["friction"] = 0.6
    fixtures[sl] = f
    p = n + 1
    bodies[p]["type"] = b2g.DYNAMIC
    bodies[p]["position"] = (-4.0, 2.0)
    bodies[p]["linear_velocity"] = projectile_velocity
    fixtures[p]["body"] = p
    fixtures[p]["shape_type"] = b2g.CIRCLE
    fixtures[p]["radius"] = 0.5
    fixtures[p]["density"] = 2.0
    fixtures[p]["friction"] = 0.6
    target = np.array([6.0 + rng.uniform(1)[0], 1.0 + rng.uniform(1)[0]], F32)
    return _scene("throw_stack", bodies, fixtures, steps, target=target, stack=np.arange(1, n + 1),
                  projectile=p)


def throw_stack_batch(seeds=512, steps=240):
    """`seeds` throw-and-stack worlds in one batch: world s is throw_stack(seed=s) with its
    projectile velocity drawn per seed (vx in [10, 14], vy in [2, 4]) and its own target."""
    bodies, fixtures, targets, stacks, projectiles = [], [], [], [], []
    nb = 0
    for s in range(seeds):
        rng = SplitMix64(1000003 * (s + 1))
        v = (float(10.0 + 4.0 * rng.uniform(1)[0]), float(2.0 + 2.0 * rng.uniform(1)[0]))
        sc = throw_stack(seed=s + 1, steps=steps, projectile_velocity=v)
        b = sc["bodies"].copy()
        b["world_index"] = s
        f = sc["fixtures"].copy()
        f["body"] += nb
        bodies.append(b)
        fixtures.append(f)
        targets.append(sc["target"])
        stacks.append(sc["stack"] + nb)
        projectiles.append(sc["projectile"] + nb)
        nb += len(b)
    return _scene("throw_stack_batch", np.concatenate(bodies), np.concatenate(fixtures), steps, num_worlds=seeds,
                  targets=np.array(targets, F32), stacks=np.array(stacks), projectiles=np.array(projectiles))


def hello_world():
    """box2d-rs tests/test.rs:26-102: a 1x1 box (density 1, friction 0.3) dropped on a 50x10 box ground."""
    bodies = b2g.body_defs(2)
    bodies[0]["position"] = (0.0, -10.0)
    bodies[1]["type"] = b2g.DYNAMIC
    bodies[1]["position"] = (0.0, 4.0)
    fixtures = b2g.fixture_defs(2)
    fixtures[0]["body"] = 0
    fixtures[0]["shape_type"] = b2g.POLYGON
    fixtures[0]["polygon_mode"] = b2g.POLYGON_BOX
    fixtures[0]["box_half_extents"] = (50.0, 10.0)
    fixtures[1]["body"] = 1
    fixtures[1]["shape_type"] = b2g.POLYGON
    fixtures[1]["polygon_mode"] = b2g.POLYGON_BOX
    fixtures[1]["box_half_extents"] = (1.0, 1.0)
    fixtures[1]["density"] = 1.0
    fixtures[1]["friction"] = 0.3
    s = _scene("hello_world", bodies, fixtures, 60, vi=6, pi=2)
    s["allow_sleep"] = True
    return s


def toi_rain(n=64, seed=7, steps=120, bullets=2, kinematic=True):
    """Fast bodies rained onto thin static plates (continuous physics): circles, boxes and 3-8-gons
    with downward speeds of 60-250 m/s over 0.1 m thick static boxes and an edge floor, so that a
    step without time of impact would carry them through; a few bullets and a sliding kinematic
    plate add the dynamic-versus-bullet and kinematic cases."""
    rng = SplitMix64(seed)
    nk = 1 if kinematic else 0
    ns = 4
    bodies = b2g.body_defs(ns + nk + n)
    bodies["allow_sleep"] = 0
    fixtures = []
    # statics: floor edge, thin plate, two thin walls
    f = b2g.fixture_defs(1)
    f["body"] = 0
    f["shape_type"] = b2g.EDGE
    f["vertices"][0, 1] = (-30.0, -4.0)
    f["vertices"][0, 2] = (30.0, -4.0)
    f["friction"] = 0.5
    fixtures.append(f)
    for b, pos, half in ((1, (0.0, 0.0), (20.0, 0.05)), (2, (-20.0, 10.0), (0.05, 12.0)), (3, (20.0, 10.0), (0.05, 12.0))):
        bodies[b]["position"] = pos
        f = b2g.fixture_defs(1)
        f["body"] = b
        f["shape_type"] = b2g.POLYGON
        f["polygon_mode"] = b2g.POLYGON_BOX
        f["box_half_extents"] = half
        f["friction"] = 0.5
        fixtures.append(f)
    if kinematic:
        k = ns
        bodies[k]["type"] = b2g.KINEMATIC
        bodies[k]["position"] = (-8.0, 6.0)
        bodies[k]["linear_velocity"] = (3.0, 0.0)
        bodies[k]["angular_velocity"] = 0.2
        f = b2g.fixture_defs(1)
        f["body"] = k
        f["shape_type"] = b2g.POLYGON
        f["polygon_mode"] = b2g.POLYGON_BOX
        f["box_half_extents"] = (3.0, 0.05)
        f["friction"] = 0.5
        fixtures.append(f)
    first = ns + nk
    idx = np.arange(first, first + n)
    bodies["type"][idx] = b2g.DYNAMIC
    px = rng.uniform(n, -18.0, 18.0)
    py = rng.uniform(n, 8.0, 40.0)
    vx = rng.uniform(n, -20.0, 20.0)
    vy = -rng.uniform(n, 60.0, 250.0)
    ang = rng.uniform(n, 0.0, 2.0 * math.pi)
    bodies["position"][idx] = np.stack([px, py], 1).astype(F32)
    bodies["angle"][idx] = ang.astype(F32)
    bodies["linear_velocity"][idx] = np.stack([vx, vy], 1).astype(F32)
    bodies["angular_velocity"][idx] = rng.uniform(n, -5.0, 5.0).astype(F32)
    if bullets:
        bodies["bullet"][idx[:bullets]] = 1
    kind = rng.integers(n, 0, 2)
    size = rng.uniform(n, 0.15, 0.5)
    nv = rng.integers(n, 3, 8)
    verts = _polygon_vertices(rng, n, size, nv)
    f = b2g.fixture_defs(n)
    f["body"] = idx
    f["density"] = 1.0
    f["friction"] = 0.4
    for i in range(n):
        if kind[i] == 0:
            f[i]["shape_type"] = b2g.CIRCLE
            f[i]["radius"] = size[i]
        elif kind[i] == 1:
            f[i]["shape_type"] = b2g.POLYGON
            f[i]["polygon_mode"] = b2g.POLYGON_BOX
            f[i]["box_half_extents"] = (size[i], 0.6 * size[i])
        else:
            f[i]["shape_type"] = b2g.POLYGON
            f[i]["vertex_count"] = nv[i]
            f[i]["vertices"][: nv[i]] = verts[i, : nv[i]]
    fixtures.append(f)
    return _scene("toi_rain", bodies, np.concatenate(fixtures), steps, continuous=True)


def toi_rain_batch(seeds=(7, 8, 9, 10), n=32, steps=90):
    """Independent toi_rain worlds in one batch (continuous physics per world)."""
    bodies, fixtures, offset = [], [], 0
    for w, seed in enumerate(seeds):
        s = toi_rain(n=n, seed=seed, steps=steps)
        b = s["bodies"].copy()
        b["world_index"] = w
        f = s["fixtures"].copy()
        f["body"] += offset
        offset += len(b)
        bodies.append(b)
        fixtures.append(f)
    return _scene("toi_rain_batch", np.concatenate(bodies), np.concatenate(fixtures), steps, num_worlds=len(seeds),
                  continuous=True)


def bridge(planks=30, seed=13, steps=240, drops=24):
    """A bridge of planks joined by revolute joints between two static posts (box2d-rs testbed
    bridge), with circles and boxes dropped on it; a motorised wheel and a hinged flap with limits
    on the side."""
    rng = SplitMix64(seed)
    n_extra = 2
    bodies = b2g.body_defs(1 + planks + drops + n_extra)
    bodies["allow_sleep"] = 0
    fixtures = [b2g.edge_fixture(0, (-40.0, 0.0), (40.0, 0.0))]
    joints = []
    x0 = -14.5
    for i in range(planks):
        b = 1 + i
        bodies[b]["type"] = b2g.DYNAMIC
        bodies[b]["position"] = (x0 + 1.0 * i, 5.0)
        fixtures.append(b2g.box_fixture(b, 0.5, 0.125, density=20.0, friction=0.2))
        prev = 0 if i == 0 else b - 1
        anchor = (x0 - 0.5 + 1.0 * i, 5.0)
        la = anchor if prev == 0 else (0.5, 0.0)
        joints.append(b2g.revolute_joint(prev, b, la, (-0.5, 0.0)))
    joints.append(b2g.revolute_joint(planks, 0, (0.5, 0.0), (x0 - 0.5 + 1.0 * planks, 5.0)))
    first = 1 + planks
    px = rng.uniform(drops, -12.0, 12.0)
    py = rng.uniform(drops, 8.0, 20.0)
    for k in range(drops):
        b = first + k
        bodies[b]["type"] = b2g.DYNAMIC
        bodies[b]["position"] = (px[k], py[k])
        if k % 2:
            fixtures.append(b2g.circle_fixture(b, 0.4, density=1.0, friction=0.4))
        else:
            fixtures.append(b2g.box_fixture(b, 0.4, 0.3, density=1.0, friction=0.4))
    wheel, flap = first + drops, first + drops + 1
    bodies[wheel]["type"] = b2g.DYNAMIC
    bodies[wheel]["position"] = (22.0, 3.0)
    fixtures.append(b2g.box_fixture(wheel, 2.0, 0.2, density=2.0, friction=0.5))
    joints.append(b2g.revolute_joint(0, wheel, (22.0, 3.0), (0.0, 0.0), motor=(2.0, 500.0)))
    bodies[flap]["type"] = b2g.DYNAMIC
    bodies[flap]["position"] = (-22.0, 6.0)
    fixtures.append(b2g.box_fixture(flap, 1.5, 0.1, density=1.0, friction=0.5))
    joints.append(b2g.revolute_joint(0, flap, (-23.5, 6.0), (-1.5, 0.0), limits=(-0.6, 0.3),
                                     motor=(-1.0, 5.0)))
    return _scene("bridge", bodies, np.concatenate(fixtures), steps, joints=np.concatenate(joints))


def gears(steps=240, drops=12, seed=17):
    """The box2d-rs testbed's gear joints (examples/testbed/tests/gear_joint.rs) with the gears' body_a /
    body_b set to their joints' second bodies: a box hanging from a static disc with a disc hinged to
    its lower end, geared to the box (the box is both A and D of that gear); a disc and a larger disc
    hinged to the ground and geared 2:1, the larger one geared to a box sliding on a vertical prismatic
    joint with limits. Boxes and circles dropped on top give them contacts to push through."""
    rng = SplitMix64(seed)
    bodies = b2g.body_defs(7 + drops)
    bodies["allow_sleep"] = 0
    fixtures = [b2g.edge_fixture(0, (50.0, 0.0), (-50.0, 0.0))]
    # the first group: static disc 1, hanging box 2, disc 3
    bodies[1]["position"] = (10.0, 9.0)
    fixtures.append(b2g.circle_fixture(1, 1.0, density=5.0))
    bodies[2]["type"], bodies[2]["position"] = b2g.DYNAMIC, (10.0, 8.0)
    fixtures.append(b2g.box_fixture(2, 0.5, 5.0, density=5.0))
    bodies[3]["type"], bodies[3]["position"] = b2g.DYNAMIC, (10.0, 6.0)
    bodies[3]["angular_velocity"] = 1.5
    fixtures.append(b2g.circle_fixture(3, 2.0, density=5.0))
    # the second group: disc 4 and disc 5 hinged to the ground, box 6 on a vertical slider
    bodies[4]["type"], bodies[4]["position"] = b2g.DYNAMIC, (-3.0, 12.0)
    fixtures.append(b2g.circle_fixture(4, 1.0, density=5.0))
    bodies[5]["type"], bodies[5]["position"] = b2g.DYNAMIC, (0.0, 12.0)
    fixtures.append(b2g.circle_fixture(5, 2.0, density=5.0))
    bodies[6]["type"], bodies[6]["position"] = b2g.DYNAMIC, (2.5, 12.0)
    fixtures.append(b2g.box_fixture(6, 0.5, 5.0, density=5.0))
    joints = [
        b2g.revolute_joint(1, 2, (0.0, 0.0), (0.0, 1.0)),      # 0: static disc - box at (10, 9)
        b2g.revolute_joint(2, 3, (0.0, -2.0), (0.0, 0.0)),     # 1: box - disc at (10, 6)
        b2g.gear_joint(0, 1, 2, 3, ratio=2.0),                 # 2: body_a = 2, body_b = 3
        b2g.revolute_joint(0, 4, (-3.0, 12.0), (0.0, 0.0)),    # 3: ground - disc 4
        b2g.revolute_joint(0, 5, (0.0, 12.0), (0.0, 0.0)),     # 4: ground - disc 5
        b2g.prismatic_joint(0, 6, (2.5, 12.0), (0.0, 0.0), (0.0, 1.0), limits=(-5.0, 5.0)),  # 5
        b2g.gear_joint(3, 4, 4, 5, ratio=2.0),                 # 6
        b2g.gear_joint(4, 5, 5, 6, ratio=-1.0 / 2.0),          # 7
    ]
    px = rng.uniform(drops, -6.0, 12.0)
    py = rng.uniform(drops, 18.0, 30.0)
    for k in range(drops):
        b = 7 + k
        bodies[b]["type"] = b2g.DYNAMIC
        bodies[b]["position"] = (px[k], py[k])
        if k % 2:
            fixtures.append(b2g.circle_fixture(b, 0.5, density=1.0, friction=0.4))
        else:
            fixtures.append(b2g.box_fixture(b, 0.5, 0.4, density=1.0, friction=0.4))
    return _scene("gears", bodies, np.concatenate(fixtures), steps, joints=np.concatenate(joints))


def build_world(world, scene):
    """Create a scene's bodies, fixtures and joints in a B2world or OracleWorld."""
    world.create_bodies(scene["bodies"])
    world.create_fixtures(scene["fixtures"])
    if scene.get("joints") is not None and len(scene["joints"]):
        world.create_joints(scene["joints"])
    return world
