"""prt_b200_nearest_hits_noalloc: the nearest-hit call for programs that must not
allocate device memory once running (e.g. a renderer whose frame loop forbids
cudaMalloc).  It must give exactly what prt_b200_nearest_hits gives, call after call,
while staging everything in the library's fixed device array.

Kept in a file of its own, collected last, so a failure here cannot hide other tests.
"""
import ctypes

import numpy as np
import pytest

from portablert_gb300 import _lib, hitreg, workloads

pytestmark = pytest.mark.gpu

MAX_RAYS = 65536  # the documented per-call limit of the fixed array


def _call(L, fn, ctx, rays, lay):
    out = np.zeros(len(rays) * lay.size, np.uint8)
    rc = fn(ctx, rays.ctypes.data, len(rays), lay.mask, lay.size, lay.offsets8(),
            out.ctypes.data)
    return rc, out


def test_noalloc_matches_allocating_call_twice():
    L = _lib.load()
    if not L.prt_b200_available():
        raise RuntimeError("no compute capability 10.3 device visible")
    ctx = ctypes.c_void_p()
    _lib.check(L.prt_b200_create(0, ctypes.byref(ctx)), None, L)
    try:
        tris = workloads.soup_tris(12, 4096)
        _lib.check(L.prt_b200_set_tris(ctx, tris.ctypes.data, len(tris)), ctx, L)
        cases = [(hitreg.TAGS, workloads.soup_rays(21, 50_000)),
                 (("t", "primitive_id", "valid"), workloads.soup_rays(22, MAX_RAYS))]
        wants = []
        for tags, rays in cases:
            lay = hitreg.layout(tags)
            rc_a, want = _call(L, L.prt_b200_nearest_hits, ctx, rays, lay)
            _lib.check(rc_a, ctx, L)
            wants.append(want)
        # From here on the first device buffer growth anywhere in the process fails (the
        # library's host-side allocation-failure injector).  The no-alloc calls must not
        # meet it, and it must still be armed after them.
        _lib.check(L.prt_b200_set_option(ctx, b"fail_alloc_after", 1), ctx, L)
        try:
            for (tags, rays), want in zip(cases, wants):  # two calls in a row
                lay = hitreg.layout(tags)
                rc_b, got = _call(L, L.prt_b200_nearest_hits_noalloc, ctx, rays, lay)
                _lib.check(rc_b, ctx, L)
                # The parity tolerance of this project is bit equality.
                assert np.array_equal(got, want)
                rec = got.view(lay.numpy_dtype())
                assert (rec["valid"] != 0).sum() > 0
            # Still armed: a set_tris that must grow its triangle buffer meets it.
            bigger = workloads.soup_tris(13, 8192)
            rc = L.prt_b200_set_tris(ctx, bigger.ctypes.data, len(bigger))
            assert rc == 6, rc  # PRT_ERR_OOM: the no-alloc calls made no growth
        finally:
            L.prt_b200_set_option(ctx, b"fail_alloc_after", 0)
        _lib.check(L.prt_b200_set_tris(ctx, tris.ctypes.data, len(tris)), ctx, L)
        too_many = workloads.soup_rays(23, MAX_RAYS + 1)
        rc, _ = _call(L, L.prt_b200_nearest_hits_noalloc, ctx, too_many,
                      hitreg.layout(hitreg.TAGS))
        assert rc == 7  # PRT_ERR_LIMIT
        assert b"65536" in L.prt_b200_last_error(ctx)
    finally:
        L.prt_b200_destroy(ctx)
