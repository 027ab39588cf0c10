"""Finite-difference check of the hand-written reverse-mode functions (CPU, double precision).

tests/adjoint_unit.cpp wraps every forward function of the differentiable step (velocity
integration, constraint initialisation with the world manifold, warm start, the velocity update
with friction cone and 1-point / 2-point block normal solve, position integration with its
clamps, the non-linear position update) as a map of flat vectors and compares the adjoint with
a central difference, with the discrete decisions frozen from the forward evaluation.
"""
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_adjoint_functions_match_finite_differences():
    src = os.path.join(ROOT, "tests", "adjoint_unit.cpp")
    inc = os.path.join(ROOT, "box2d-rs_gb300", "csrc")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "adjoint_unit")
        subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-I", inc, src, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = [l for l in out.stdout.splitlines() if "rel err" in l]
    assert len(lines) >= 90
    # every decision state of the 2-point block solver that the random cases reach is covered
    assert any("/1" in l for l in lines) and any("/3" in l for l in lines)
