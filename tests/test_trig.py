"""sin/cos: the float fast path of b2g_sincosf returns the same bits as the double evaluation
b2g_sincosf_ref.

CPU: every 251st float with 0 < |x| <= 8192 (tests/trig_check.cpp; the same program with stride 1
covers all 2,348,810,240 such floats). GPU: every float in that range on the device, plus the
device results against the host's on a 4M sample (tests/trig_check_gpu.cu).
"""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "box2d-rs_gb300", "csrc")


def test_fast_path_matches_double_evaluation_cpu():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "trig_check")
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-pthread", "-I", INC,
                        os.path.join(ROOT, "tests", "trig_check.cpp"), "-o", exe], check=True)
        out = subprocess.run([exe, "251", "4"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    checked = int(out.stdout.split()[1])
    assert checked > 9_000_000


@pytest.mark.gpu
def test_fast_path_matches_double_evaluation_gpu_exhaustive():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "trig_check_gpu")
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "--fmad=false",
                        "-ftz=false", "-prec-div=true", "-prec-sqrt=true", "-Xcompiler", "-ffp-contract=off",
                        "-I", INC, os.path.join(ROOT, "tests", "trig_check_gpu.cu"), "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "mismatches 0" in out.stdout
