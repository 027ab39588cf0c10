"""The host reference of the differentiable step on a recorded GPU tape (CPU only).

tests/golden/tape_throw_stack.npz holds a 64-step tape of a 4 x 4 throw-and-stack world recorded
on a GB300 together with the GPU's backward result (tests/golden/make_tape_golden.py). Checks:
  * the host f32 replay of the tape lands on the GPU's final state bit for bit, and every
    impulse carried between steps through the tape's carry links equals the recorded one;
  * the host f64 reverse pass matches central differences of the f64 frozen-decision forward
    (1e-5 relative, plus 1e-7 of the largest entry for differencing noise);
  * the recorded GPU f32 gradient is within 1e-3 relative (2-norm) of the f64 reverse pass.
"""
import os

import numpy as np
import pytest

import adjoint_ref

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tape_throw_stack.npz")


@pytest.fixture(scope="module")
def tape():
    z = np.load(GOLDEN)
    ref = adjoint_ref.AdjointRef(z["body_static"], z["steps"], z["cols"], z["slots"])
    yield z, ref
    ref.close()


def _loss(c, stack, target):
    com = c[stack].mean(0)
    g = np.zeros((len(c), 2))
    g[stack] = 2.0 * (com - target) / len(stack)
    return float(((com - target) ** 2).sum()), g


def test_replay_is_bit_exact_with_the_gpu(tape):
    z, ref = tape
    init = adjoint_ref.state_from_checkpoint(z["init"])
    fin = adjoint_ref.state_from_checkpoint(z["final"])
    rep, carry_mismatches = ref.replay_f32(init)
    assert np.array_equal(rep.view(np.uint32), fin.view(np.uint32))
    assert carry_mismatches == 0
    assert int(z["replay_mismatches"]) == 0


def test_f64_reverse_pass_matches_central_differences(tape):
    z, ref = tape
    stack, target = z["stack"], z["target"]
    init = adjoint_ref.state_from_checkpoint(z["init"]).astype(np.float64)
    ref.replay_f32(init.astype(np.float32))
    _, gc = _loss(ref.forward_f64(init)[:, :2], stack, target)
    gd = np.zeros((len(init), 6))
    gd[:, :2] = gc
    g = ref.backward_f64(init, gd)
    gmax = np.abs(g).max()
    proj = int(z["projectile"])
    probes = [(proj, k) for k in range(6)] + [(int(b), k) for b in stack[[0, 3, 9, 15]] for k in range(6)]
    for b, k in probes:
        h = 1e-5 * max(1.0, abs(init[b, k]))
        xp, xm = init.copy(), init.copy()
        xp[b, k] += h
        xm[b, k] -= h
        fd = (_loss(ref.forward_f64(xp)[:, :2], stack, target)[0] -
              _loss(ref.forward_f64(xm)[:, :2], stack, target)[0]) / (2 * h)
        assert abs(fd - g[b, k]) <= 1e-5 * abs(fd) + 1e-7 * gmax, (b, k, fd, g[b, k])


def test_recorded_gpu_gradient_matches_f64(tape):
    z, ref = tape
    stack, target = z["stack"], z["target"]
    init = adjoint_ref.state_from_checkpoint(z["init"]).astype(np.float64)
    ref.replay_f32(init.astype(np.float32))
    # the GPU was given dL/d(final) from its own f32 final state
    gd = np.zeros((len(init), 6))
    gd[:, 0:2] = z["d_final"]["world_center"]
    g = ref.backward_f64(init, gd)
    gg = z["gpu_grad"]
    g_gpu = np.stack([gg["world_center"][:, 0], gg["world_center"][:, 1], gg["angle"], gg["linear_velocity"][:, 0],
                      gg["linear_velocity"][:, 1], gg["angular_velocity"]], 1).astype(np.float64)
    rel = np.linalg.norm(g_gpu - g) / np.linalg.norm(g)
    assert rel <= 1e-3, rel


def test_anchored_reverse_pass_matches_the_recorded_gpu_gradient(tape):
    """The f64 reverse pass linearised along the f32 replay's own trajectory (every step starts from
    the f32 state it started from on the GPU): only the reverse pass's rounding separates it from the
    GPU's f32 gradient, so the two agree far below 1e-3."""
    z, ref = tape
    init = adjoint_ref.state_from_checkpoint(z["init"])
    ref.replay_f32(init)
    gd = np.zeros((len(init), 6))
    gd[:, 0:2] = z["d_final"]["world_center"]
    g = ref.backward_f64_anchored(gd)
    gg = z["gpu_grad"]
    g_gpu = np.stack([gg["world_center"][:, 0], gg["world_center"][:, 1], gg["angle"], gg["linear_velocity"][:, 0],
                      gg["linear_velocity"][:, 1], gg["angular_velocity"]], 1).astype(np.float64)
    rel = np.linalg.norm(g_gpu - g) / np.linalg.norm(g)
    assert rel <= 1e-4, rel
    # the unanchored f64 pass over this short tape lands on nearly the same gradient
    g64 = ref.backward_f64(init.astype(np.float64), gd)
    assert np.linalg.norm(g64 - g) / np.linalg.norm(g) <= 1e-3
