"""Generate tests/golden/tape_throw_stack.npz (needs a GPU and the built libb2g.so).

Scene: throw_stack with a 4 x 4 box stack (half-extent 0.25 m) and the circle projectile, 64
steps at dt = 1/60 with 8/3 iterations, taped from the first step (checkpoints every 16 steps).
Saved: the exported tape (body static data, step parameters, colour offsets, slots), the
initial and final solver states, the loss's target and stack, and the GPU's backward result for
dL/d(final) of the stack centre-of-mass loss. The CPU tests replay this tape with the host
reference (bit-exact final state), check the f64 reverse pass against central differences and
compare the recorded GPU gradient with it.

Usage: python tests/golden/make_tape_golden.py [out.npz]
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "box2d-rs_gb300"), os.path.join(ROOT, "oracle")]

import numpy as np  # noqa: E402

import adjoint_ref  # noqa: E402
import b2g  # noqa: E402
import scenes  # noqa: E402

STEPS = 64


def main(out):
    sc = scenes.throw_stack(rows=4, cols=4, steps=STEPS, projectile_velocity=(9.0, 2.0))
    w = b2g.B2world(gravity=(0.0, -10.0))
    w.set_allow_sleeping(False)
    w.create_bodies(sc["bodies"])
    w.create_fixtures(sc["fixtures"])
    w.tape_begin(STEPS, 16)
    for _ in range(STEPS):
        w.step(1.0 / 60.0, 8, 3)
    w.tape_end()
    stack, target = sc["stack"], sc["target"].astype(np.float64)
    final = w.get_body_states()
    com = final["world_center"][stack].astype(np.float64).mean(0)
    d = np.zeros(w.body_count, b2g.BODY_STATE)
    d["world_center"][stack] = 2.0 * (com - target) / len(stack)
    g = w.backward(d)
    info = w.tape_info()
    tape = adjoint_ref.export_tape(w, sc["bodies"])
    np.savez_compressed(
        out, **tape, init=w.tape_checkpoint(0), final=w.tape_checkpoint(-1), stack=stack, target=target,
        projectile=np.int64(sc["projectile"]), d_final=d, gpu_grad=g,
        replay_mismatches=np.int64(info["replay_mismatches"]))
    print(out, info)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden", "tape_throw_stack.npz"))
