"""The two traversal passes: batches whose rays all have finite reciprocals run in the
regular pass (plain slab test only), the others are left to the deferred pass (with the
conservative test for zero direction components and non-finite rays).  Mixed queries
must give every ray the exhaustive search's record, whichever pass took its batch."""
import numpy as np
import pytest

from portablert_gb300 import hitreg, workloads as W

pytestmark = pytest.mark.gpu

TAGS = hitreg.TAGS


def _same(got, want):
    assert np.array_equal(got["valid"], want["valid"])
    v = want["valid"] != 0
    assert np.array_equal(got["t"].view(np.uint32), want["t"].view(np.uint32))
    assert np.array_equal(got["primitive_id"][v], want["primitive_id"][v])
    for f in ("u", "v", "px", "py", "pz"):
        a, b = got[f][v], want[f][v]
        assert ((a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))).all(), f


def _mixed_rays(n, seed):
    rays = W.soup_rays(seed, n).copy()
    # One ray with a zero direction component in every 7th batch of 32, a ray with a
    # zero component and an origin on a grid plane in every 11th, a NaN ray in one.
    for b in range(0, n // 32, 7):
        rays[32 * b + 5, 3] = 0.0
    for b in range(3, n // 32, 11):
        rays[32 * b + 17, 4] = 0.0
        rays[32 * b + 17, 1] = 0.0
    rays[32 * 4 + 9, 0] = np.nan
    return rays


@pytest.mark.parametrize("leaf", [1, 4])
def test_mixed_batches_against_exhaustive_search(gpu_backend, oracle_lib, leaf):
    tris = W.soup_tris(31, 20_000)
    rays = _mixed_rays(32 * 300 + 13, 32)
    want = oracle_lib.brute_force(tris, rays)
    try:
        gpu_backend.set_option("leaf_size", leaf)
        gpu_backend.set_tris(tris)
        for fmt in (0, 1):
            gpu_backend.set_option("node_format", fmt)
            _same(gpu_backend.nearest_hits(rays, TAGS), want)
    finally:
        gpu_backend.set_option("leaf_size", 1)
        gpu_backend.set_option("node_format", 0)


def test_every_batch_deferred(gpu_backend, oracle_lib):
    tris = W.soup_tris(33, 5_000)
    rays = W.soup_rays(34, 4_000).copy()
    rays[::32, 5] = 0.0  # the first ray of every batch
    gpu_backend.set_tris(tris)
    _same(gpu_backend.nearest_hits(rays, TAGS), oracle_lib.brute_force(tris, rays))


def test_counting_run_equals_plain(gpu_backend):
    tris = W.soup_tris(35, 30_000)
    rays = _mixed_rays(32 * 100, 36)
    gpu_backend.set_tris(tris)
    plain = gpu_backend.nearest_hits(rays, TAGS)
    try:
        gpu_backend.set_option("count_visits", 1)
        counted = gpu_backend.nearest_hits(rays, TAGS)
    finally:
        gpu_backend.set_option("count_visits", 0)
    assert plain.tobytes() == counted.tobytes()
