"""Parity rules between a backend's hit records and the reference's (TEST
INFRASTRUCTURE: the checker used by tests/ and by bench.py's CPU-baseline leg).

* ``valid`` and ``primitive_id`` bit-exact; t, u, v, p bit-exact (the kernels use the
  reference's operation order without FMA, so no ulp tolerance is needed: TOL_ULP = 0).
* A ray whose closest accepted triangles tie in t may report any of them: such rays
  are listed, and checked by equal t and by re-running the reference arithmetic on the
  reported triangle (it must be accepted with exactly that t, u and v).
* Misses: only t (= +inf) and valid are compared; the reference leaves u, v and
  primitive_id unwritten there.
"""
from __future__ import annotations

import numpy as np

TOL_ULP = 0


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _same_float(a, b):
    """Bit-identical, treating every NaN as equal (NaN payloads differ by platform)."""
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    both_nan = np.isnan(a) & np.isnan(b)
    return (_bits(a) == _bits(b)) | both_nan


def tri_box_pass(tri, ray):
    """The reference slab test (bvh.hpp:195-222) on one triangle's own box, in numpy
    float32 with the select min/max."""
    t = np.asarray(tri, np.float32).reshape(3, 3)
    o = np.asarray(ray[:3], np.float32)
    d = np.asarray(ray[3:], np.float32)

    def rmin(a, b):
        return b if b < a else a

    def rmax(a, b):
        return b if a < b else a

    lo = [rmin(t[0, k], rmin(t[1, k], t[2, k])) for k in range(3)]
    hi = [rmax(t[0, k], rmax(t[1, k], t[2, k])) for k in range(3)]
    with np.errstate(all="ignore"):
        f = [np.float32(1.0) / d[k] for k in range(3)]
        ts = [np.float32((np.float32(lo[k]) - o[k]) * f[k]) for k in range(3)] + \
             [np.float32((np.float32(hi[k]) - o[k]) * f[k]) for k in range(3)]
    t1, t3, t5, t2, t4, t6 = ts
    tmin = rmax(rmax(rmin(t1, t2), rmin(t3, t4)), rmin(t5, t6))
    tmax = rmin(rmin(rmax(t1, t2), rmax(t3, t4)), rmax(t5, t6))
    return not (tmax < 0) and not (tmin > tmax)


def compare(got, want, tags, tris, rays, oracle=None):
    """Checks `got` (structured array, fields per `tags`) against `want` (the reference's
    full records).  Returns a report dict; report['bad'] lists failing ray indices."""
    tags = set(tags)
    n = len(want)
    wv = want["valid"] != 0
    ok = np.ones(n, bool)
    if "valid" in tags:
        ok &= (got["valid"] != 0) == wv
    if "t" in tags:
        ok &= _same_float(got["t"], want["t"]) | (~wv & np.isinf(got["t"]) & (got["t"] > 0))
    same_pid = np.ones(n, bool)
    if "primitive_id" in tags:
        same_pid = got["primitive_id"] == want["primitive_id"]
    exact = np.ones(n, bool)
    if "uv" in tags:
        exact &= _same_float(got["u"], want["u"]) & _same_float(got["v"], want["v"])
    if "p" in tags:
        for f in ("px", "py", "pz"):
            exact &= _same_float(got[f], want[f])
    hit_ok = same_pid & exact
    ties = []
    if "primitive_id" in tags:
        for i in np.flatnonzero(wv & ~hit_ok):
            # A different triangle is allowed only on an exact tie in t.
            pid = int(got["primitive_id"][i])
            if oracle is None or pid >= len(tris):
                continue
            acc, t, u, v = oracle.intersect_tri(tris[pid], rays[i])
            if acc and tri_box_pass(tris[pid], rays[i]) and \
                    np.float32(t) == np.float32(want["t"][i]):
                if "uv" in tags and not (np.float32(u) == got["u"][i] and
                                         np.float32(v) == got["v"][i]):
                    continue
                hit_ok[i] = True
                ties.append(int(i))
    ok &= ~wv | hit_ok
    bad = np.flatnonzero(~ok)
    return {"n": n, "hits": int(wv.sum()), "ties": ties, "bad": bad.tolist(),
            "n_bad": int(bad.size)}


def exact_vs_leaf_only(got, bf, tags):
    """Indices where `got` differs from the order-independent leaf-only answer `bf`
    (exhaustive search, ties -> lower primitive id), which is what the kernels compute
    by construction; every present field bit for bit."""
    v = bf["valid"] != 0
    bad = np.zeros(len(bf), bool)
    if "valid" in tags:
        bad |= (got["valid"] != 0) != v
    if "t" in tags:
        bad |= ~_same_float(got["t"], bf["t"])
    if "primitive_id" in tags:
        bad |= v & (got["primitive_id"] != bf["primitive_id"])
    if "uv" in tags:
        bad |= v & ~(_same_float(got["u"], bf["u"]) & _same_float(got["v"], bf["v"]))
    if "p" in tags:
        for f in ("px", "py", "pz"):
            bad |= v & ~_same_float(got[f], bf[f])
    return np.flatnonzero(bad)


def tree_dependent_rays(tris, rays, oracle, threads=0):
    """(mask, leaf-only answers) of the rays whose reference answer depends on the
    reference's own tree (oracle.cpu.tree_dependent).  Only a ray whose x reciprocal is
    infinite can be one (a zero x direction starting on a triangle's lower x face makes
    the reference slab test NaN), so only those are searched exhaustively."""
    with np.errstate(divide="ignore"):
        cand = np.flatnonzero(np.isinf(np.float32(1.0) / rays[:, 3]))
    dep = np.zeros(len(rays), bool)
    bf = np.zeros(len(rays), oracle.HIT_DTYPE)
    if cand.size:
        d, a, _ = oracle.tree_dependent(tris, rays[cand], threads)
        dep[cand] = d
        bf[cand] = a
    return dep, bf


def check(got, want, tags, tris, rays, oracle, threads=0):
    """The full parity outcome of `got` against the reference's records `want`:
    compare() for every ray, except that a tree-dependent ray must instead equal the
    leaf-only answer bit for bit.  Returns {n, hits, n_bad, bad (first 20), ties,
    tree_dependent}."""
    dep, bf = tree_dependent_rays(tris, rays, oracle, threads)
    rep = compare(got, want, tags, tris, rays, oracle)
    bad = [i for i in rep["bad"] if not dep[i]]
    idx = np.flatnonzero(dep)
    if idx.size:
        bad += idx[exact_vs_leaf_only(got[idx], bf[idx], tags)].tolist()
    return {"n": rep["n"], "hits": rep["hits"], "n_bad": len(bad), "bad": sorted(bad)[:20],
            "ties": len(rep["ties"]), "tree_dependent": int(dep.sum())}
