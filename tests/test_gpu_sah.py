"""The binned-SAH build (option build_sah): every field of every record equals the
oracle's exhaustive search and the LBVH build's records, whatever the scene -- sizes at
each boundary of the builder's tiers (32 and 512 triangles, 2048-triangle chunks),
identical triangles (no plane separates them), non-finite vertices and a scene whose
planes would nest deeper than the depth guard -- and the tree needs fewer node visits
than the LBVH on the heightfield and the soup."""
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


@pytest.fixture
def sah(gpu_backend):
    gpu_backend.set_option("build_sah", 1)  # the default for set_tris
    gpu_backend.set_option("build_small", 0)  # the binned-SAH builder at every size
    yield gpu_backend
    gpu_backend.set_option("build_small", 1)
    gpu_backend.set_option("leaf_size", 1)
    gpu_backend.set_option("node_format", 0)


@pytest.mark.parametrize("n", [1, 2, 3, 31, 32, 33, 64, 512, 513, 1024, 1025, 2048, 2049,
                               5000, 40_000])
def test_sizes_against_exhaustive_search(sah, oracle_lib, n):
    tris = W.soup_tris(9000 + n, n)
    rays = W.soup_rays(9100 + n, 4000)
    want = oracle_lib.brute_force(tris, rays)
    for leaf in (1, 8):
        sah.set_option("leaf_size", leaf)
        sah.set_tris(tris)
        assert sah.stat("build_sah") == 1.0
        for fmt in (0, 1):
            sah.set_option("node_format", fmt)
            _same(sah.nearest_hits(rays, TAGS), want)


def test_identical_triangles_split_into_halves(sah, oracle_lib):
    one = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32)
    tris = np.repeat(one, 3000, 0)
    tris[1500:] += np.float32(0.25)  # two stacks of identical triangles
    rays = np.concatenate([np.tile([[0.2, 0.2, -1, 0, 0, 1]], (50, 1)),
                           W.soup_rays(1, 500)]).astype(np.float32)
    sah.set_tris(tris)
    got = sah.nearest_hits(rays, TAGS)
    _same(got, oracle_lib.brute_force(tris, rays))
    assert got["primitive_id"][0] == 0  # ties in t go to the smaller id


def test_non_finite_vertices(sah, oracle_lib):
    tris = W.soup_tris(5, 3000)
    tris[7, 4] = np.nan
    tris[1200, 0] = np.inf
    tris[2999, 8] = -np.inf
    rays = W.soup_rays(6, 3000)
    sah.set_tris(tris)
    _same(sah.nearest_hits(rays, TAGS), oracle_lib.brute_force(tris, rays))


def test_depth_guard(sah, oracle_lib):
    """Triangles at x = 1.5^k: every SAH plane cuts off the farthest one, so the binary
    tree would be a chain; past 48 levels the builder splits into halves (or, if the
    8-wide tree still exceeds 32 levels, set_tris falls back to the LBVH)."""
    k = np.arange(200, dtype=np.float64)
    x = 1.5 ** (k / 4)
    tris = np.zeros((200, 9), np.float32)
    tris[:, 0] = x
    tris[:, 3] = x + 0.001 * x
    tris[:, 6] = x
    tris[:, 7] = 1.0
    tris[:, [2, 5, 8]] = 0.0
    rays = np.stack([x * 1.0005, np.full_like(x, 0.1), np.full_like(x, -1),
                     np.zeros_like(x), np.zeros_like(x), np.ones_like(x)], 1).astype(np.float32)
    sah.set_tris(tris)
    got = sah.nearest_hits(rays, TAGS)
    _same(got, oracle_lib.brute_force(tris, rays))
    assert (got["valid"] != 0).sum() > 100


@pytest.mark.parametrize("scene", ["heightfield", "soup"])
def test_equals_lbvh_with_fewer_visits(gpu_backend, scene):
    if scene == "heightfield":
        tris = W.heightfield_tris(3, 256, 128)
        rays = W.camera_rays(320, 240)
    else:
        tris = W.soup_tris(77, 200_000)
        rays = W.soup_rays(78, 20_000)
    res = {}
    try:
        gpu_backend.set_option("count_visits", 1)
        gpu_backend.set_option("build_small", 0)
        for sah in (0, 1):
            gpu_backend.set_option("build_sah", sah)
            gpu_backend.set_tris(tris)
            out = gpu_backend.nearest_hits(rays, TAGS)
            res[sah] = (out, gpu_backend.stat("visits_nodes"), gpu_backend.stat("n_nodes"))
    finally:
        gpu_backend.set_option("count_visits", 0)
        gpu_backend.set_option("build_sah", 1)
        gpu_backend.set_option("build_small", 1)
    assert res[0][0].tobytes() == res[1][0].tobytes()
    assert res[1][1] < res[0][1], (res[1][1], res[0][1])


def test_many_scenes_in_one_sah_build(gpu_backend, oracle_lib):
    """batch_set_tris_dev builds every scene's SAH tree in the same launches (tasks of all
    scenes side by side): each scene's records equal its exhaustive search."""
    import torch

    from portablert_gb300.batch import Batch, make_query

    sizes = [0, 1, 2, 33, 1025, 2049, 5000, 40_000, 3]
    tris = [W.soup_tris(9300 + s, n) for s, n in enumerate(sizes)]
    rays = [W.soup_rays(9400 + s, 1500) for s in range(len(sizes))]
    off = np.cumsum([0] + sizes)
    d_tris = torch.from_numpy(np.concatenate(tris)).cuda()
    lay = hitreg.layout(TAGS)
    keep, qs = [], []
    for s, r in enumerate(rays):
        d_r = torch.from_numpy(r).cuda()
        d_o = torch.zeros(len(r) * lay.size, dtype=torch.uint8, device="cuda")
        qs.append(make_query(s, d_r.data_ptr(), len(r), d_o.data_ptr(), TAGS))
        keep.append((d_r, d_o))
    torch.cuda.synchronize()
    b = Batch(gpu_backend)
    try:
        b.set_tris_dev(d_tris.data_ptr(), off)
        assert b.stat("build_sah") == 1.0
        b.query_dev(qs)
        b.sync()
        torch.cuda.synchronize()
        for s in range(len(sizes)):
            got = keep[s][1].cpu().numpy().view(lay.numpy_dtype())
            _same(got, oracle_lib.brute_force(tris[s], rays[s]))
    finally:
        b.close()
