"""ctypes binding of liboracle_adj.so — TEST INFRASTRUCTURE ONLY.

The host reference of the differentiable step (b2_adjoint_ref.cpp): it takes a tape exported
from a GPU world (b2g.B2world.tape_step / tape_checkpoint / get_mass_data) and runs
  replay_f32(init)      the taped solver steps sequentially in f32 (must land bit-exactly on
                        the GPU's recorded final state) and records every discrete decision;
  forward_f64(init)     the same steps in f64 with those decisions frozen;
  backward_f64(init, g) the f64 reverse pass: dL/d(initial state) from dL/d(final state).
States are (n_bodies, 6) arrays: centre x, y, angle, vx, vy, w.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboracle_adj.so")
_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle_adj.so"], check=True)
    lib = ctypes.CDLL(LIB_PATH)
    vp, i32 = ctypes.c_void_p, ctypes.c_int32
    lib.ora_adj_create.argtypes = [i32, vp, i32, vp, vp, vp]
    lib.ora_adj_create.restype = vp
    lib.ora_adj_destroy.argtypes = [vp]
    lib.ora_adj_destroy.restype = None
    for name in ("ora_adj_replay_f32", "ora_adj_forward_f64"):
        getattr(lib, name).argtypes = [vp, vp, vp]
        getattr(lib, name).restype = ctypes.c_int
    lib.ora_adj_backward_f64.argtypes = [vp, vp, vp, vp]
    lib.ora_adj_backward_f64.restype = ctypes.c_int
    lib.ora_adj_backward_f64_anchored.argtypes = [vp, vp, vp]
    lib.ora_adj_backward_f64_anchored.restype = ctypes.c_int
    _lib = lib
    return lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def export_tape(world, body_defs):
    """The tape of `world` (a b2g.B2world after tape_end) as plain arrays: body_static (n, 10)
    float32 (mass, 1/mass, inertia, 1/inertia, linear and angular damping, gravity scale, local
    centre x, y, type), steps (b2g.TAPE_STEP), cols int32 (each step's num_colours + 1 colour-group
    offsets, concatenated), slots (b2g.TAPE_SLOT).
    body_defs: the b2g.BODY_DEF array the bodies were created from."""
    import b2g

    T = world.tape_info()["steps"]
    mass = world.get_mass_data()
    bs = np.zeros((world.body_count, 10), np.float32)
    bs[:, 0:4] = mass[:, 0:4]
    bs[:, 4] = body_defs["linear_damping"]
    bs[:, 5] = body_defs["angular_damping"]
    bs[:, 6] = body_defs["gravity_scale"]
    bs[:, 7:9] = mass[:, 4:6]
    bs[:, 9] = body_defs["type"]
    steps = np.zeros(T, b2g.TAPE_STEP)
    cols = []
    slots = []
    for t in range(T):
        st, col, sl = world.tape_step(t)
        steps[t] = st
        cols.append(np.asarray(col, np.int32))
        slots.append(sl)
    slots = np.concatenate(slots) if slots else np.zeros(0, b2g.TAPE_SLOT)
    cols = np.concatenate(cols) if cols else np.zeros(0, np.int32)
    return {"body_static": bs, "steps": steps, "cols": cols, "slots": slots}


def flat_cols(steps, cols):
    """Colour-group offsets as one concatenated int32 array; a (steps, 257) array (one row per
    step, num_colours + 1 used) is flattened."""
    cols = np.asarray(cols, np.int32)
    if cols.ndim == 1:
        return cols
    nc = np.asarray(steps["num_colours"], np.int64)
    return np.concatenate([cols[t, : nc[t] + 1] for t in range(len(nc))]) if len(nc) else np.zeros(0, np.int32)


class AdjointRef:
    def __init__(self, body_static, steps, cols, slots):
        """Build the reference from an exported tape (see export_tape)."""
        self._lib = load()
        cols = flat_cols(steps, cols)
        nc = np.asarray(steps["num_colours"], np.int64)
        if len(cols) != int((nc + 1).sum()):
            raise ValueError("cols must hold num_colours + 1 offsets per step")
        self._keep = tuple(np.ascontiguousarray(a) for a in (body_static, steps, cols, slots))
        bs, steps, cols, slots = self._keep
        self.n = len(bs)
        self.steps = len(steps)
        self._h = self._lib.ora_adj_create(self.n, _p(bs), self.steps, _p(steps), _p(cols), _p(slots))

    @classmethod
    def from_world(cls, world, body_defs):
        t = export_tape(world, body_defs)
        return cls(t["body_static"], t["steps"], t["cols"], t["slots"])

    def close(self):
        if self._h:
            self._lib.ora_adj_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def replay_f32(self, init):
        """Final state of the f32 replay and the number of carried impulses that differed from
        the recorded ones (0 when the tape's carry links are right)."""
        init = np.ascontiguousarray(init, np.float32)
        out = np.zeros((self.n, 6), np.float32)
        mismatches = self._lib.ora_adj_replay_f32(self._h, _p(init), _p(out))
        return out, mismatches

    def forward_f64(self, init):
        init = np.ascontiguousarray(init, np.float64)
        out = np.zeros((self.n, 6), np.float64)
        assert self._lib.ora_adj_forward_f64(self._h, _p(init), _p(out)) == 0
        return out

    def backward_f64(self, init, d_final):
        init = np.ascontiguousarray(init, np.float64)
        d_final = np.ascontiguousarray(d_final, np.float64)
        out = np.zeros((self.n, 6), np.float64)
        assert self._lib.ora_adj_backward_f64(self._h, _p(init), _p(d_final), _p(out)) == 0
        return out

    def backward_f64_anchored(self, d_final):
        """The f64 reverse pass along the f32 replay's trajectory (call replay_f32 first): every step is
        linearised at the f32 state it started from, so only the reverse pass's own rounding separates
        it from the GPU's f32 gradient."""
        d_final = np.ascontiguousarray(d_final, np.float64)
        out = np.zeros((self.n, 6), np.float64)
        assert self._lib.ora_adj_backward_f64_anchored(self._h, _p(d_final), _p(out)) == 0
        return out


def state_from_checkpoint(ck):
    """(n, 8) checkpoint rows (cx, cy, a, -, vx, vy, w, -) -> (n, 6) state."""
    return np.ascontiguousarray(ck[:, [0, 1, 2, 4, 5, 6]])
