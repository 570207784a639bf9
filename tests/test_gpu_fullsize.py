"""Parity at the measured configurations' own sizes (the bench's workloads), where the
kernels' bookkeeping (traversal pool size, 27-bit work items, deferred-pass counters,
the SAH build's task tiers) takes the values it takes in the measurements.

* The 1,048,576-triangle heightfield (1024 x 512 quads, seed 1) with every one of its
  2,073,600 pinhole primary rays and 4,194,304 cosine secondary rays, offset 0.01 along
  the normal and offset 0 (from the hit points themselves), all five tags, against the
  oracle's restatement of the reference's CPU backend (its own SAH tree and traversal).
* The 8,388,608-triangle clustered soup (seed 2) with 16,777,216 random rays: FP32 and
  compressed nodes byte-identical on every ray, and a ray sample against the oracle's
  exhaustive search over all triangles.
"""
import numpy as np
import pytest

from parity import check
from portablert_gb300 import hitreg, workloads as W

pytestmark = pytest.mark.gpu

TAGS = hitreg.TAGS


def test_heightfield_every_ray(gpu_backend, oracle_lib):
    import os

    cores = os.cpu_count() or 1
    tris = W.heightfield_tris(seed=1)
    prim = W.camera_rays()
    assert len(tris) == 1_048_576 and len(prim) == 2_073_600
    gpu_backend.set_tris(tris)
    assert gpu_backend.stat("build_sah") == 1.0
    hp = gpu_backend.nearest_hits(prim, TAGS)
    bvh = oracle_lib.BVH(tris)
    rep = check(hp, bvh.nearest_hits(prim, threads=cores), TAGS, tris, prim, oracle_lib, cores)
    assert rep["n_bad"] == 0, rep
    assert rep["hits"] > 400_000
    for delta in (0.01, 0.0):
        sec = W.secondary_rays(tris, prim, hp["valid"] != 0, hp["primitive_id"],
                               np.stack([hp["px"], hp["py"], hp["pz"]], 1), 4_194_304,
                               delta=delta, seed=1)
        hs = gpu_backend.nearest_hits(sec, TAGS)
        rep = check(hs, bvh.nearest_hits(sec, threads=cores), TAGS, tris, sec, oracle_lib,
                    cores)
        assert rep["n_bad"] == 0, (delta, rep)
        assert rep["hits"] > 0


def test_clustered_soup_every_ray_both_formats_and_a_sample_exhaustively(gpu_backend,
                                                                         oracle_lib):
    import os

    import torch

    n_t, n_r = 8_388_608, 16_777_216
    tags = ("uv", "t", "primitive_id", "valid")
    lay = hitreg.layout(tags)
    d_t = torch.empty(n_t * 9, dtype=torch.float32, device="cuda")
    d_r = torch.empty(n_r * 6, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    W.generate_dev(gpu_backend, W.GEN_CLUSTER_TRIS, 2, n_t, d_t.data_ptr(), 256)
    W.generate_dev(gpu_backend, W.GEN_RANDOM_RAYS, 2, n_r, d_r.data_ptr(), 12.0)
    gpu_backend.sync()
    gpu_backend.set_tris_dev(d_t.data_ptr(), n_t)
    outs = []
    try:
        for fmt in (0, 1):
            gpu_backend.set_option("node_format", fmt)
            o = torch.zeros(n_r * lay.size, dtype=torch.uint8, device="cuda")
            torch.cuda.synchronize()
            gpu_backend.nearest_hits_dev(d_r.data_ptr(), n_r, o.data_ptr(), tags)
            gpu_backend.sync()
            outs.append(o)
    finally:
        gpu_backend.set_option("node_format", 0)
    assert torch.equal(outs[0], outs[1])
    got = outs[0].cpu().numpy().view(lay.numpy_dtype())
    assert (got["valid"] != 0).sum() > 4_000_000
    idx = np.sort(np.random.default_rng(77).choice(n_r, size=512, replace=False))
    tris = d_t.cpu().numpy().reshape(n_t, 9)
    rays = np.ascontiguousarray(d_r.cpu().numpy().reshape(n_r, 6)[idx])
    cores = os.cpu_count() or 1
    want = oracle_lib.brute_force(tris, rays, threads=cores)
    rep = check(got[idx], want, tags, tris, rays, oracle_lib, cores)
    assert rep["n_bad"] == 0, rep
    assert rep["hits"] > 100
