"""Parity of the CUDA path (through the C ABI) with the reference.

Reference answers come from (a) the golden vectors written by the reference's own CPU
backend and (b) the C restatement of it (oracle/), which tests/test_oracle_pin.py pins
to those vectors.  Rules (tests/parity.py): valid / primitive_id / t / u / v / p
bit-exact; exact ties in t may name another triangle with the same t; tree-dependent
rays (zero x direction starting on a triangle's lower x face) must equal the leaf-only
answer, which the reference's answer is bounded by.
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN_SETS, ROOT, load_c0_golden, load_golden
from parity import _same_float, check, compare, exact_vs_leaf_only
from portablert_gb300 import hitreg, workloads

pytestmark = pytest.mark.gpu

FULL_TAGS = hitreg.TAGS


def _exact_vs_leaf_only(got, bf, tags=FULL_TAGS):
    return exact_vs_leaf_only(got, bf, tags)


def _check_against_reference(got, ref, tris, rays, oracle, tags=FULL_TAGS):
    rep = check(got, ref, tags, tris, rays, oracle)
    assert rep["n_bad"] == 0, f"{rep['n_bad']} rays differ from the reference, e.g. {rep['bad'][:5]}"
    return rep, rep["tree_dependent"]


@pytest.mark.parametrize("name", GOLDEN_SETS)
def test_golden_sets_match_reference(gpu_backend, oracle_lib, name):
    g = load_golden(name)
    gpu_backend.set_tris(g["tris"])
    got = gpu_backend.nearest_hits(g["rays"], FULL_TAGS)
    _check_against_reference(got, g["full"], g["tris"], g["rays"], oracle_lib)
    bf = oracle_lib.brute_force(g["tris"], g["rays"])
    assert _exact_vs_leaf_only(got, bf).size == 0


def test_kat_through_python_api(gpu_backend):
    g = load_golden("kat")
    gpu_backend.set_tris(g["tris"])
    h = gpu_backend.nearest_hits(g["rays"], FULL_TAGS)
    assert h["valid"][0] == 1 and h["valid"][1] == 0
    assert abs(h["t"][0] - 1.0) <= 1e-4 and abs(h["u"][0] - 0.3) <= 1e-4
    assert abs(h["v"][0] - 0.5) <= 1e-4 and h["primitive_id"][0] == 0
    assert abs(h["px"][0] - 0.1) <= 1e-4
    assert np.isinf(h["t"][1])
    hv = gpu_backend.nearest_hits(g["rays"], ("valid",))
    assert hv["valid"].tolist() == [1, 0]


def test_soup_small_config_bit_exact(gpu_backend, oracle_lib):
    """4,096-triangle soup, 65,536 rays, tags t/primitive_id/uv/valid."""
    tris, rays = workloads.soup(seed=0, n_tris=4096, n_rays=65536)
    tags = ("t", "primitive_id", "uv", "valid")
    gpu_backend.set_tris(tris)
    got = gpu_backend.nearest_hits(rays, tags)
    ref = oracle_lib.BVH(tris).nearest_hits(rays)
    rep, _ = _check_against_reference(got, ref, tris, rays, oracle_lib, tags)
    assert rep["hits"] > 30000
    # And against the reference's own records for exactly these inputs (golden fixture).
    g = load_c0_golden(tris, rays)
    rep, _ = _check_against_reference(got, g["full"], tris, rays, oracle_lib, tags)
    assert rep["hits"] == int((g["full"]["valid"] != 0).sum())


@pytest.mark.parametrize("tags", hitreg.TAG_COMBOS, ids=hitreg.hitreg_name)
def test_every_tag_combination(gpu_backend, oracle_lib, tags):
    g = load_golden("soup_small")
    gpu_backend.set_tris(g["tris"])
    got = gpu_backend.nearest_hits(g["rays"], tags)
    assert got.dtype.itemsize == hitreg.layout(tags).size
    _check_against_reference(got, g["full"], g["tris"], g["rays"], oracle_lib, tags)
    # Bytes the reference leaves unwritten are zero in ours except for present fields.
    lay = hitreg.layout(tags)
    raw = got.view(np.uint8).reshape(-1, lay.size)
    present = np.zeros(lay.size, bool)
    for name in got.dtype.names:
        off = got.dtype.fields[name][1]
        present[off: off + got.dtype.fields[name][0].itemsize] = True
    assert (raw[:, ~present] == 0).all()


@pytest.mark.parametrize("leaf_size", [1, 2, 4, 8])
@pytest.mark.parametrize("fmt", [0, 1])
def test_leaf_size_and_node_format_do_not_change_answers(gpu_backend, oracle_lib, leaf_size,
                                                         fmt):
    tris, rays = workloads.soup(seed=7, n_tris=6000, n_rays=20000)
    gpu_backend.set_option("leaf_size", leaf_size)
    gpu_backend.set_option("node_format", fmt)
    try:
        gpu_backend.set_tris(tris)
        got = gpu_backend.nearest_hits(rays, FULL_TAGS)
    finally:
        gpu_backend.set_option("leaf_size", 4)
        gpu_backend.set_option("node_format", 0)
    bf = oracle_lib.brute_force(tris, rays)
    assert _exact_vs_leaf_only(got, bf).size == 0


def test_heightfield_primary_and_secondary(gpu_backend, oracle_lib):
    tris = workloads.heightfield_tris(seed=1, nx=256, nz=128)
    prim = workloads.camera_rays(320, 180)
    gpu_backend.set_tris(tris)
    hp = gpu_backend.nearest_hits(prim, FULL_TAGS)
    bvh = oracle_lib.BVH(tris)
    ref = bvh.nearest_hits(prim)
    _check_against_reference(hp, ref, tris, prim, oracle_lib)
    for delta in (0.0, 0.01):
        sec = workloads.secondary_rays(tris, prim, hp["valid"] != 0, hp["primitive_id"],
                                       np.stack([hp["px"], hp["py"], hp["pz"]], 1), 20000,
                                       delta=delta)
        hs = gpu_backend.nearest_hits(sec, FULL_TAGS)
        rs = bvh.nearest_hits(sec)
        _check_against_reference(hs, rs, tris, sec, oracle_lib)


def test_clustered_soup(gpu_backend, oracle_lib):
    tris = workloads.cluster_tris(seed=2, n_tris=60_000)
    rays = workloads.random_rays(seed=2, n_rays=20_000)
    tags = ("t", "primitive_id", "valid")
    for fmt in (0, 1):
        gpu_backend.set_option("node_format", fmt)
        gpu_backend.set_tris(tris)
        got = gpu_backend.nearest_hits(rays, tags)
        bf = oracle_lib.brute_force(tris, rays)
        assert _exact_vs_leaf_only(got, bf, tags).size == 0
    gpu_backend.set_option("node_format", 0)


def test_empty_scene_and_empty_batch(gpu_backend):
    gpu_backend.set_tris(np.zeros((0, 9), np.float32))
    rays = workloads.soup_rays(3, 100)
    h = gpu_backend.nearest_hits(rays, FULL_TAGS)
    assert (h["valid"] == 0).all() and np.isinf(h["t"]).all()
    gpu_backend.set_tris(workloads.soup_tris(3, 10))
    assert gpu_backend.nearest_hits(np.zeros((0, 6), np.float32), FULL_TAGS).shape == (0,)


def test_non_finite_inputs_do_not_fail(gpu_backend, oracle_lib):
    tris = workloads.soup_tris(9, 2000)
    tris[5, 3] = np.nan
    tris[17, 0] = np.inf
    tris[33, 8] = -np.inf
    rays = workloads.soup_rays(9, 5000)
    rays[0, 3:] = 0.0
    rays[1, 3] = np.nan
    rays[2, 0] = np.inf
    rays[3, 3:] = [1e-40, 0.0, 1.0]
    gpu_backend.set_tris(tris)
    got = gpu_backend.nearest_hits(rays, FULL_TAGS)
    bf = oracle_lib.brute_force(tris, rays)
    assert _exact_vs_leaf_only(got, bf).size == 0


def test_errors_are_reported(gpu_backend):
    from portablert_gb300 import _lib
    from portablert_gb300.backend import B200Backend

    fresh = B200Backend(0)
    fresh.init()
    with pytest.raises(_lib.PrtError) as e:
        fresh.nearest_hits(workloads.soup_rays(1, 4), FULL_TAGS)
    assert e.value.code == 4
    with pytest.raises(_lib.PrtError):
        fresh.set_option("leaf_size", 9)
    fresh.shutdown()


def test_cpp_api_kat_and_all_combos():
    """portableRT's C++ API (select_backend / set_tris / nearest_hits<Tags...>) over the
    B200 backend: the validation example's known answers, and all 31 tag combinations
    (plus reordered tag lists) byte-compatible with the reference's records."""
    from portablert_gb300 import build

    exe = build.build_cpp_test()
    r = subprocess.run([exe, "kat"], capture_output=True, text=True, check=True)
    import json

    k = json.loads(r.stdout)
    assert k["backend"] == "B200" and k["hit"]["valid"] == 1 and k["miss_valid"] == 0
    assert abs(k["hit"]["t"] - 1.0) <= 1e-4 and abs(k["hit"]["u"] - 0.3) <= 1e-4
    assert abs(k["hit"]["v"] - 0.5) <= 1e-4 and k["hit"]["primitive_id"] == 0
    assert k["filtered_hit_valid"] == 1 and k["filtered_miss_valid"] == 0
    g = load_golden("soup_small")
    with tempfile.TemporaryDirectory() as d:
        tp, rp = os.path.join(d, "t.f32"), os.path.join(d, "r.f32")
        g["tris"].tofile(tp)
        g["rays"].tofile(rp)
        subprocess.run([exe, "dump", tp, rp, d], capture_output=True, text=True, check=True)
        full = g["full"]
        v = full["valid"] != 0
        for tags in hitreg.TAG_COMBOS:
            lay = hitreg.layout(tags)
            rec = np.fromfile(os.path.join(d, hitreg.hitreg_name(tags) + ".bin"),
                              dtype=lay.numpy_dtype())
            assert len(rec) == len(full)
            if "valid" in tags:
                assert np.array_equal(rec["valid"], full["valid"])
            if "t" in tags:
                assert _same_float(rec["t"], full["t"]).all()
            if "primitive_id" in tags:
                assert np.array_equal(rec["primitive_id"][v], full["primitive_id"][v])
        same = hitreg.layout(FULL_TAGS)
        a = np.fromfile(os.path.join(d, "uv_t_primitive_id_p_valid.bin"), np.uint8)
        b = np.fromfile(os.path.join(d, "order_t_primitive_id_uv_p_valid.bin"), np.uint8)
        assert same.size == 32 and np.array_equal(a, b)
