"""The allocation-free manifold entry point against the allocating one, through the C ABI.

b2g_collide_pairs_noalloc serves callers that cannot allocate memory (a frame loop with a fixed
time budget, or a host program whose device memory belongs to its own pool allocator). It
must return exactly what b2g_collide_pairs returns for the same shape pairs, also on a second
call in a row (its scratch array keeps the previous call's contents), and must refuse more
pairs than its fixed scratch holds.
"""
import ctypes
import os
import sys

import numpy as np
import pytest

import b2g

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MAX_PAIRS = 16384  # B2G_NOALLOC_MAX_PAIRS in include/b2g.h
TOL = 1e-5


def _noalloc(lib, da, xa, db, xb):
    da = np.ascontiguousarray(da, b2g.FIXTURE_DEF)
    db = np.ascontiguousarray(db, b2g.FIXTURE_DEF)
    xa = np.ascontiguousarray(xa, np.float32)
    xb = np.ascontiguousarray(xb, np.float32)
    out = np.zeros(len(da), b2g.CONTACT_INFO)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rc = lib.b2g_collide_pairs_noalloc(p(da), p(xa), p(db), p(xb), len(da), p(out))
    return rc, out


def _same(out, ref):
    assert np.array_equal(out["point_count"], ref["point_count"])
    t = ref["point_count"] > 0
    assert np.array_equal(out["manifold_type"][t], ref["manifold_type"][t])
    for i in np.nonzero(t)[0]:
        n = ref["point_count"][i]
        assert list(out["point_id"][i][:n]) == list(ref["point_id"][i][:n]), i
        for f in ("local_normal", "local_point"):
            assert np.abs(out[f][i].astype(np.float64) - ref[f][i]).max() <= TOL, (i, f)
        assert np.abs(out["point_local"][i][:n].astype(np.float64) - ref["point_local"][i][:n]).max() <= TOL, i


def test_noalloc_matches_allocating_entry_point(built):
    sys.path.insert(0, GOLDEN)
    import make_golden

    lib = b2g.load_library()
    lib.b2g_collide_pairs_noalloc.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int32, ctypes.c_void_p]
    lib.b2g_collide_pairs_noalloc.restype = ctypes.c_int
    # two calls in a row, the second one smaller, so stale entries of the first stay in the scratch
    for seed, n in ((101, 3000), (202, 1200)):
        da, xa, db, xb = make_golden.random_shape_pairs(n=n, seed=seed)
        ref = b2g.collide_pairs(da, xa, db, xb)
        rc, out = _noalloc(lib, da, xa, db, xb)
        assert rc == 0
        _same(out, ref)
        assert (out["point_count"] > 0).sum() > n // 4


def test_noalloc_rejects_more_than_its_scratch(built):
    lib = b2g.load_library()
    lib.b2g_collide_pairs_noalloc.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int32, ctypes.c_void_p]
    lib.b2g_collide_pairs_noalloc.restype = ctypes.c_int
    n = MAX_PAIRS + 1
    d = b2g.fixture_defs(n)
    d["shape_type"] = b2g.CIRCLE
    d["radius"] = 0.5
    x = np.zeros((n, 3), np.float32)
    rc, _ = _noalloc(lib, d, x, d, x)
    assert rc == -3  # B2G_ERR_CAPACITY
    rc, out = _noalloc(lib, d[:MAX_PAIRS], x[:MAX_PAIRS], d[:MAX_PAIRS], x[:MAX_PAIRS])
    assert rc == 0 and (out["point_count"] == 1).all()
