"""The one-block build of small scenes (option build_small, prt_build_small.cu: Morton
order, PLOC, the collapse and the re-layout in one launch): every field of every record
equals the oracle's exhaustive search and the binned-SAH build's records, at sizes from 1
to the largest it takes (4,096), for both collapses, leaf sizes 1 to 8 and both node
formats; identical and non-finite triangles, equal Morton codes, points, segments and a
flat scene; a scene of 4,097 triangles goes to the binned-SAH build; a chain too deep
for the traversal falls back to the LBVH."""
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
def small(gpu_backend):
    gpu_backend.set_option("build_sah", 1)
    gpu_backend.set_option("build_small", 1)
    yield gpu_backend
    gpu_backend.set_option("leaf_size", 1)
    gpu_backend.set_option("node_format", 0)
    gpu_backend.set_option("collapse_cost", 1)
    gpu_backend.set_option("build_small", 1)


@pytest.mark.parametrize("n", [1, 2, 3, 9, 17, 31, 32, 33, 100, 1000, 2049, 4095, 4096])
def test_sizes_against_exhaustive_search(small, oracle_lib, n):
    tris = W.soup_tris(9500 + n, n)
    rays = W.soup_rays(9600 + n, 3000)
    want = oracle_lib.brute_force(tris, rays)
    for cost in (1, 0):
        small.set_option("collapse_cost", cost)
        for leaf in (1, 8):
            small.set_option("leaf_size", leaf)
            small.set_tris(tris)
            assert small.stat("build_small") == 1.0
            assert small.stat("build_sah") == 1.0
            for fmt in (0, 1):
                small.set_option("node_format", fmt)
                _same(small.nearest_hits(rays, TAGS), want)


def test_one_more_goes_to_the_sah_build(small, oracle_lib):
    tris = W.soup_tris(9700, 4097)
    rays = W.soup_rays(9701, 2000)
    small.set_tris(tris)
    assert small.stat("build_small") == 0.0 and small.stat("build_sah") == 1.0
    _same(small.nearest_hits(rays, TAGS), oracle_lib.brute_force(tris, rays))


def test_equals_the_sah_build_on_the_small_configuration(small):
    """The small configuration's scene (4,096 triangles, seed 0) and 65,536 rays: the same
    records from both builders, and node visits of the same order."""
    tris = W.soup_tris(0, 4096)
    rays = W.soup_rays(1, 65_536)
    out, visits = {}, {}
    try:
        small.set_option("count_visits", 1)
        for one_block in (1, 0):
            small.set_option("build_small", one_block)
            small.set_tris(tris)
            assert small.stat("build_small") == float(one_block)
            out[one_block] = small.nearest_hits(rays, TAGS)
            visits[one_block] = small.stat("visits_nodes")
    finally:
        small.set_option("count_visits", 0)
    assert out[0].tobytes() == out[1].tobytes()
    assert visits[1] < 1.25 * visits[0], (visits[1], visits[0])


def test_identical_triangles(small, oracle_lib):
    one = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32)
    tris = np.repeat(one, 3000, 0)
    tris[1500:] += np.float32(0.25)
    rays = np.concatenate([np.tile([[0.2, 0.2, -1, 0, 0, 1]], (50, 1)),
                           W.soup_rays(1, 500)]).astype(np.float32)
    small.set_tris(tris)
    assert small.stat("build_small") == 1.0
    got = small.nearest_hits(rays, TAGS)
    _same(got, oracle_lib.brute_force(tris, rays))
    assert got["primitive_id"][0] == 0  # ties in t go to the smaller id


def test_non_finite_vertices(small, oracle_lib):
    tris = W.soup_tris(5, 3000)
    tris[7, 4] = np.nan
    tris[1200, 0] = np.inf
    tris[2999, 8] = -np.inf
    rays = W.soup_rays(6, 3000)
    for cost in (1, 0):
        small.set_option("collapse_cost", cost)
        small.set_tris(tris)
        assert small.stat("build_small") == 1.0
        _same(small.nearest_hits(rays, TAGS), oracle_lib.brute_force(tris, rays))


def test_all_non_finite(small, oracle_lib):
    tris = np.full((40, 9), np.nan, np.float32)
    rays = W.soup_rays(8, 200)
    small.set_tris(tris)
    _same(small.nearest_hits(rays, TAGS), oracle_lib.brute_force(tris, rays))


def test_chain_scene(small, oracle_lib):
    """Triangles at x = 1.5^(k/4): clusters merge one at a time into a deep binary chain;
    the tree is still exact, and if its 8-wide form were deeper than the traversal's 32
    levels set_tris would fall back to the LBVH."""
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
    small.set_tris(tris)
    assert small.stat("depth") <= 32
    got = small.nearest_hits(rays, TAGS)
    _same(got, oracle_lib.brute_force(tris, rays))
    assert (got["valid"] != 0).sum() > 100


@pytest.mark.parametrize("n", [37, 4096])
def test_every_leaf_size(small, oracle_lib, n):
    """Leaf sizes 2 to 7 (1 and 8 above): leaves of several triangles take the counts the
    clusters carry (exact up to the largest leaf) and the permutation's subtree walk."""
    tris = W.soup_tris(9800 + n, n)
    rays = W.soup_rays(9801 + n, 2000)
    want = oracle_lib.brute_force(tris, rays)
    for leaf in range(2, 8):
        small.set_option("leaf_size", leaf)
        small.set_tris(tris)
        assert small.stat("build_small") == 1.0
        _same(small.nearest_hits(rays, TAGS), want)


def test_morton_ties_and_degenerate_triangles(small, oracle_lib):
    """Groups of triangles with one centroid (equal Morton codes, which the sort keeps in
    index order), zero-area triangles (points and segments) and a flat scene (one axis of
    zero extent, so every code has one coordinate's bits zero)."""
    rng = np.random.default_rng(77)
    base = W.soup_tris(78, 512)
    tris = np.concatenate([np.repeat(base[:64], 40, 0),  # 2,560 triangles, 64 centroids
                           base[64:]])
    tris[100] = [1, 1, 1, 1, 1, 1, 1, 1, 1]          # a point
    tris[200] = [0, 0, 0, 1, 1, 1, 2, 2, 2]          # a segment
    flat = tris.copy()
    flat[:, [2, 5, 8]] = 0.5
    rays = np.concatenate([W.soup_rays(79, 2000),
                           np.column_stack([rng.uniform(-1, 2, (500, 2)), np.full(500, -1.0),
                                            np.zeros((500, 2)), np.ones(500)])]).astype(np.float32)
    for scene in (tris, flat):
        small.set_tris(scene)
        assert small.stat("build_small") == 1.0
        _same(small.nearest_hits(rays, TAGS), oracle_lib.brute_force(scene, rays))
