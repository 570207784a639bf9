"""Batches: many scenes built in one pass and queried by one launch (prt_b200_batch_*).
Every answer must be byte-identical to nearest_hits on that scene alone."""
import numpy as np
import pytest

from portablert_gb300 import hitreg, workloads

pytestmark = pytest.mark.gpu

TAGSETS = [hitreg.TAGS, ("t", "primitive_id", "valid"), ("uv",), ("p", "valid"),
           ("t", "primitive_id", "uv", "valid"), ("valid",), ("primitive_id",)]


def _torch():
    import torch

    assert torch.cuda.is_available()
    return torch


def _dev(torch, a):
    """Device copy of a numpy array, finished before the library's stream reads it."""
    t = torch.from_numpy(a).cuda()
    torch.cuda.synchronize()
    return t


def _scenes(seed, sizes, n_rays):
    tris = [workloads.soup_tris(seed + s, n) for s, n in enumerate(sizes)]
    rays = [workloads.soup_rays(seed + s, m) for s, m in enumerate(n_rays)]
    return tris, rays


def _queries(torch, rays, tagsets):
    from portablert_gb300.batch import make_query

    qs, keep = [], []
    for s, r in enumerate(rays):
        tags = tagsets[s % len(tagsets)]
        lay = hitreg.layout(tags)
        d_r = _dev(torch, r)
        d_o = torch.zeros(max(len(r), 1) * lay.size, dtype=torch.uint8, device="cuda")
        qs.append(make_query(s, d_r.data_ptr(), len(r), d_o.data_ptr(), tags))
        keep.append((d_r, d_o, tags, lay))
    torch.cuda.synchronize()
    return qs, keep


def _alone(backend, tris, rays, tags):
    backend.set_tris(tris)
    return backend.nearest_hits(rays, tags).view(np.uint8)


def _check(backend, tris, rays, keep):
    for s, (d_r, d_o, tags, lay) in enumerate(keep):
        got = d_o.cpu().numpy()[: len(rays[s]) * lay.size]
        want = _alone(backend, tris[s], rays[s], tags)
        assert np.array_equal(got, want), f"scene {s}"


def test_batch_matches_each_scene_alone(gpu_backend):
    torch = _torch()
    from portablert_gb300.batch import Batch

    sizes = [0, 1, 2, 7, 64, 500, 3000, 1, 4096, 33]
    n_rays = [50, 100, 1000, 31, 32, 33, 5000, 64, 2048, 999]
    tris, rays = _scenes(100, sizes, n_rays)
    off = np.cumsum([0] + sizes)
    d_tris = _dev(torch, np.concatenate(tris))
    b = Batch(gpu_backend)
    try:
        b.set_tris_dev(d_tris.data_ptr(), off)
        assert b.stat("n_scenes") == len(sizes)
        qs, keep = _queries(torch, rays, TAGSETS)
        b.query_dev(qs)
        b.sync()
        torch.cuda.synchronize()
        _check(gpu_backend, tris, rays, keep)
    finally:
        b.close()


@pytest.mark.parametrize("fmt", [0, 1])
def test_batch_graph_replay_matches(gpu_backend, fmt):
    torch = _torch()
    from portablert_gb300.batch import Batch

    sizes = list(workloads.batch_sizes(40, seed=9, tri_range=(16, 4000), ray_range=(64, 3000))[0])
    n_rays = list(workloads.batch_sizes(40, seed=9, tri_range=(16, 4000), ray_range=(64, 3000))[1])
    tris, rays = _scenes(300, sizes, n_rays)
    off = np.cumsum([0] + sizes)
    d_tris = _dev(torch, np.concatenate(tris))
    gpu_backend.set_option("node_format", fmt)
    b = Batch(gpu_backend)
    try:
        qs, keep = _queries(torch, rays, TAGSETS)
        for _ in range(2):  # capture + launch, then replay
            for _, d_o, _, _ in keep:
                d_o.zero_()
            torch.cuda.synchronize()
            b.run_graph(d_tris.data_ptr(), off, qs)
            b.sync()
            torch.cuda.synchronize()
            _check(gpu_backend, tris, rays, keep)
        assert b.stat("depth") >= 1 and b.stat("n_nodes") >= len(sizes)
        # the graph-built arena answers direct queries too
        for _, d_o, _, _ in keep:
            d_o.zero_()
        torch.cuda.synchronize()
        b.query_dev(qs)
        b.sync()
        torch.cuda.synchronize()
        _check(gpu_backend, tris, rays, keep)
    finally:
        b.close()
        gpu_backend.set_option("node_format", 0)


def test_batch_of_many_small_scenes_vs_oracle(gpu_backend, oracle_lib):
    torch = _torch()
    from portablert_gb300.batch import Batch, make_query

    tri_n, ray_n = workloads.batch_sizes(256, seed=5, tri_range=(16, 2048), ray_range=(64, 1024))
    tris = [workloads.soup_tris(1000 + s, int(n)) for s, n in enumerate(tri_n)]
    rays = [workloads.soup_rays(1000 + s, int(m)) for s, m in enumerate(ray_n)]
    off = np.cumsum([0] + [len(t) for t in tris])
    d_tris = _dev(torch, np.concatenate(tris))
    all_rays = np.concatenate(rays)
    d_rays = _dev(torch, all_rays)
    roff = np.cumsum([0] + [len(r) for r in rays])
    lay = hitreg.layout(hitreg.TAGS)
    d_out = torch.zeros(len(all_rays) * lay.size, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    qs = [make_query(s, d_rays.data_ptr() + 24 * int(roff[s]), len(rays[s]),
                     d_out.data_ptr() + lay.size * int(roff[s]), hitreg.TAGS)
          for s in range(len(tris))]
    b = Batch(gpu_backend)
    try:
        b.set_tris_dev(d_tris.data_ptr(), off)
        b.query_dev(qs)
        b.sync()
        got = d_out.cpu().numpy().view(lay.numpy_dtype())
    finally:
        b.close()
    for s in range(0, len(tris), 17):
        bf = oracle_lib.brute_force(tris[s], rays[s])
        g = got[roff[s]:roff[s + 1]]
        assert np.array_equal(g["valid"], bf["valid"])
        v = bf["valid"] != 0
        assert np.array_equal(g["t"].view(np.uint32), bf["t"].view(np.uint32))
        assert np.array_equal(g["primitive_id"][v], bf["primitive_id"][v])
