"""Randomised scenes with awkward geometry against the oracle's exhaustive search.

The GPU's answer is, by construction, the exhaustive one: the smallest t over triangles
that Moller-Trumbore accepts and whose own box passes the reference slab test, ties to
the smaller primitive id (orc_brute_force).  So every field must match bit for bit, for
every ray, whatever the tree -- across both builders (binned SAH, LBVH), both collapses
(least expected cost, largest child first), leaf sizes and node formats.  The scenes mix
integer-grid vertices (coplanar and axis-aligned faces, shared edges), collinear and
repeated-vertex triangles and scales from 1e-20 to 1e20; the rays include zero
direction components, origins on grid planes and tiny or huge direction lengths."""
import numpy as np
import pytest

from portablert_gb300 import hitreg

pytestmark = pytest.mark.gpu

TAGS = hitreg.TAGS


def _scene(rng, n):
    kind = rng.integers(4)
    if kind == 0:  # soup
        c = rng.uniform(-1, 1, (n, 1, 3))
        t = c + rng.uniform(-0.1, 0.1, (n, 3, 3))
    elif kind == 1:  # integer grid: coplanar faces, shared edges, axis-aligned planes
        t = rng.integers(-4, 5, (n, 3, 3)).astype(np.float64)
    elif kind == 2:  # degenerate: collinear or repeated vertices among regular ones
        t = rng.uniform(-1, 1, (n, 3, 3))
        k = rng.random(n) < 0.3
        t[k, 2] = t[k, 0] + rng.uniform(0, 1, (k.sum(), 1)) * (t[k, 1] - t[k, 0])
        r = rng.random(n) < 0.1
        t[r, 1] = t[r, 0]
    else:  # thin slivers along an axis
        t = rng.uniform(-1, 1, (n, 3, 3))
        ax = rng.integers(3)
        t[:, :, ax] = np.round(t[:, :, ax] * 2) / 2
    scale = 10.0 ** rng.choice([-20, -3, 0, 0, 0, 3, 20])
    return (t * scale).reshape(n, 9).astype(np.float32), scale


def _rays(rng, m, scale):
    o = rng.uniform(-3, 3, (m, 3))
    d = rng.uniform(-1, 1, (m, 3)) - o  # through the scene's region
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    kind = rng.integers(4, size=m)
    z = kind == 1  # one or two zero direction components
    d[z, rng.integers(3, size=z.sum())] = 0.0
    zz = (kind == 1) & (rng.random(m) < 0.3)
    d[zz, rng.integers(3, size=zz.sum())] = 0.0
    g = kind == 2  # origins on integer grid planes, axis-aligned directions
    o[g] = np.round(o[g])
    d[g] = np.eye(3)[rng.integers(3, size=g.sum())] * rng.choice([-1.0, 1.0], (g.sum(), 1))
    s = kind == 3  # direction lengths far from 1
    d[s] *= 10.0 ** rng.choice([-30, -6, 6, 30], (s.sum(), 1))
    rays = np.concatenate([o * scale, d], 1).astype(np.float32)
    rays[np.all(rays[:, 3:] == 0, 1), 5] = 1.0  # no all-zero directions
    return rays


def _check(got, want):
    assert np.array_equal(got["valid"], want["valid"])
    v = want["valid"] != 0
    assert np.array_equal(got["t"].view(np.uint32), want["t"].view(np.uint32))
    assert np.array_equal(got["primitive_id"][v], want["primitive_id"][v])
    for f in ("u", "v", "px", "py", "pz"):
        a, b = got[f][v], want[f][v]
        same = (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))
        assert same.all(), f


@pytest.mark.parametrize("seed", range(48))
def test_fuzz_against_exhaustive_search(gpu_backend, oracle_lib, seed):
    rng = np.random.default_rng(7000 + seed)
    tris, scale = _scene(rng, int(rng.integers(1, 2500)))
    rays = _rays(rng, 3000, scale)
    want = oracle_lib.brute_force(tris, rays)
    try:
        # binned-SAH and LBVH builds, collapsed by least cost or largest child first
        for sah, cc in ((1, 1), (0, 1), (0, 0), (1, 0)):
            gpu_backend.set_option("build_sah", sah)
            gpu_backend.set_option("collapse_cost", cc)
            for leaf in (1, 4, 8):
                gpu_backend.set_option("leaf_size", leaf)
                gpu_backend.set_tris(tris)
                for fmt in (0, 1):
                    gpu_backend.set_option("node_format", fmt)
                    got = gpu_backend.nearest_hits(rays, TAGS)
                    _check(got, want)
    finally:
        gpu_backend.set_option("build_sah", 1)
        gpu_backend.set_option("collapse_cost", 1)
        gpu_backend.set_option("leaf_size", 1)
        gpu_backend.set_option("node_format", 0)
