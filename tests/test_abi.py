"""The C ABI library builds, loads and exports every entry point declared in include/b2g.h,
with struct layouts matching the Python mirror. No compute calls (runs without a GPU)."""
import ctypes
import os
import re
import subprocess

import numpy as np

import b2g

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "b2g.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\**(b2g_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("b2g_world_create", "b2g_world_destroy", "b2g_create_bodies", "b2g_create_fixtures", "b2g_step",
                 "b2g_get_body_states", "b2g_get_events", "b2g_get_profile", "b2g_get_solver_order", "b2g_get_pairs",
                 "b2g_collide_pairs"):
        assert must in names


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(b2g.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", b2g.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (b2g_\w+)", out))
    assert set(declared_functions()) <= exported


def test_struct_layouts(built, tmp_path):
    src = str(tmp_path / "sizeof.c")
    exe = str(tmp_path / "sizeof")
    code = """#include <stdio.h>
#include <stddef.h>
#include "b2g.h"
int main(void){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(b2g_world_def), sizeof(b2g_body_def),
 sizeof(b2g_fixture_def), sizeof(b2g_body_state), sizeof(b2g_contact_info), sizeof(b2g_contact_event),
 sizeof(b2g_profile), sizeof(b2g_counts), sizeof(b2g_tape_slot), sizeof(b2g_tape_step), sizeof(b2g_tape_info), sizeof(b2g_ray_hit), sizeof(b2g_launch_config),
 sizeof(b2g_sweep), sizeof(b2g_toi_output), sizeof(b2g_joint_def), sizeof(b2g_contact_impulse), sizeof(b2g_step_stats),
 sizeof(b2g_contact_edit), offsetof(b2g_joint_def, joint2));
 return 0;}"""
    try:
        with open(src, "w") as f:
            f.write(code)
        subprocess.run(["gcc", "-I" + os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        sizes = list(map(int, subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()))
    finally:
        for p in (src, exe):
            if os.path.exists(p):
                os.remove(p)
    assert sizes == [ctypes.sizeof(b2g.WorldDef), b2g.BODY_DEF.itemsize, b2g.FIXTURE_DEF.itemsize,
                     b2g.BODY_STATE.itemsize, b2g.CONTACT_INFO.itemsize, b2g.EVENT.itemsize,
                     ctypes.sizeof(b2g.Profile), ctypes.sizeof(b2g.Counts), b2g.TAPE_SLOT.itemsize,
                     b2g.TAPE_STEP.itemsize, ctypes.sizeof(b2g.TapeInfo), b2g.RAY_HIT.itemsize,
                     ctypes.sizeof(b2g.LaunchConfig), b2g.SWEEP.itemsize, b2g.TOI_OUTPUT.itemsize,
                     b2g.JOINT_DEF.itemsize, b2g.CONTACT_IMPULSE.itemsize, ctypes.sizeof(b2g.StepStats),
                     ctypes.sizeof(b2g.ContactEdit), b2g.JOINT_DEF.fields["joint2"][1]]


def test_invalid_arguments_are_rejected_without_a_device(built):
    lib = b2g.load_library()
    assert lib.b2g_world_create(None, None) == -1
    assert lib.b2g_world_destroy(None) == -1
    assert lib.b2g_step(None, ctypes.c_float(0.016), 8, 3) == -1
    d = b2g.WorldDef(b2g.Vec2(0, -10), 0, 0, 0, 0, 0, 0)  # num_worlds = 0
    h = ctypes.c_void_p()
    assert lib.b2g_world_create(ctypes.byref(d), ctypes.byref(h)) == -1
    assert lib.b2g_version() >= 1


def test_default_defs_match_reference_defaults():
    bd = b2g.body_defs(1)[0]
    assert bd["type"] == b2g.STATIC and bd["gravity_scale"] == 1.0 and bd["awake"] and bd["enabled"]
    fd = b2g.fixture_defs(1)[0]
    assert np.isclose(fd["friction"], 0.2) and fd["restitution"] == 0.0 and fd["restitution_threshold"] == 1.0
    assert fd["category_bits"] == 1 and fd["mask_bits"] == 0xFFFF and fd["group_index"] == 0
    assert np.isclose(fd["radius"], 0.01)
