"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE).

Loads ``oracle/_build/liboracle.so`` (the C restatement in ``prt_oracle.c``) and, where
it was built, runs ``oracle/_ref/ref_oracle`` (the reference's own CPU backend).  Only
tests, the smoke check and the CPU-baseline leg of bench.py use this module.
"""
from __future__ import annotations

import ctypes
import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ref_oracle")

HIT_DTYPE = np.dtype({
    "names": ["u", "v", "t", "primitive_id", "valid", "px", "py", "pz"],
    "formats": ["<f4", "<f4", "<f4", "<u4", "u1", "<f4", "<f4", "<f4"],
    "offsets": [0, 4, 8, 12, 16, 20, 24, 28],
    "itemsize": 32,
})

STATS_DTYPE = np.dtype([
    ("best_t", "<f4"), ("n_best", "<u4"), ("pid_min", "<u4"), ("pid_max", "<u4"),
    ("second_t", "<f4"), ("n_accepted", "<u4"), ("n_nodes", "<u4"), ("pad", "<u4"),
    ("t64", "<f8"),
])
assert STATS_DTYPE.itemsize == 40

NODE_DTYPE = np.dtype([("is_leaf", "<u4"), ("tri", "<u4"), ("left", "<u4"), ("right", "<u4"),
                       ("lo", "<f4", 3), ("hi", "<f4", 3)])

_lib = None


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, sz = ctypes.c_void_p, ctypes.c_size_t
        L.orc_bvh_build.restype = vp
        L.orc_bvh_build.argtypes = [vp, sz]
        L.orc_bvh_free.argtypes = [vp]
        L.orc_bvh_node_count.restype = sz
        L.orc_bvh_node_count.argtypes = [vp]
        L.orc_bvh_nodes.argtypes = [vp, vp]
        L.orc_nearest_hits.argtypes = [vp, vp, sz, vp, ctypes.c_int]
        L.orc_hit_stats.argtypes = [vp, vp, sz, vp, ctypes.c_int]
        L.orc_brute_force.argtypes = [vp, sz, vp, sz, vp, ctypes.c_int]
        L.orc_brute_force_robust.argtypes = [vp, sz, vp, sz, vp, ctypes.c_int]
        L.orc_intersect_tri.argtypes = [vp, vp, vp, vp, vp]
        L.orc_intersect_tri.restype = ctypes.c_int
        L.orc_ray_box.argtypes = [vp, vp, vp]
        L.orc_ray_box.restype = ctypes.c_int
        L.orc_camera_rays.argtypes = [vp, vp]
        L.orc_lambert.argtypes = [vp, vp, vp, sz, vp]
        _lib = L
    return _lib


def _f32(a, cols):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.ndim != 2 or a.shape[1] != cols:
        a = a.reshape(-1, cols)
    return a


class BVH:
    """The reference's BVH2, built by the restated SAH builder."""

    def __init__(self, tris):
        self.tris = _f32(tris, 9)
        self.h = lib().orc_bvh_build(self.tris.ctypes.data, self.tris.shape[0])

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_bvh_free(self.h)
            self.h = None

    def nodes(self) -> np.ndarray:
        n = lib().orc_bvh_node_count(self.h)
        out = np.zeros(n, NODE_DTYPE)
        lib().orc_bvh_nodes(self.h, out.ctypes.data)
        return out

    def nearest_hits(self, rays, threads: int = 0) -> np.ndarray:
        rays = _f32(rays, 6)
        out = np.zeros(rays.shape[0], HIT_DTYPE)
        lib().orc_nearest_hits(self.h, rays.ctypes.data, rays.shape[0], out.ctypes.data, threads)
        return out

    def stats(self, rays, threads: int = 0) -> np.ndarray:
        rays = _f32(rays, 6)
        out = np.zeros(rays.shape[0], STATS_DTYPE)
        lib().orc_hit_stats(self.h, rays.ctypes.data, rays.shape[0], out.ctypes.data, threads)
        return out


def brute_force(tris, rays, threads: int = 0) -> np.ndarray:
    tris, rays = _f32(tris, 9), _f32(rays, 6)
    out = np.zeros(rays.shape[0], HIT_DTYPE)
    lib().orc_brute_force(tris.ctypes.data, tris.shape[0], rays.ctypes.data, rays.shape[0],
                          out.ctypes.data, threads)
    return out


def brute_force_robust(tris, rays, threads: int = 0) -> np.ndarray:
    tris, rays = _f32(tris, 9), _f32(rays, 6)
    out = np.zeros(rays.shape[0], HIT_DTYPE)
    lib().orc_brute_force_robust(tris.ctypes.data, tris.shape[0], rays.ctypes.data,
                                 rays.shape[0], out.ctypes.data, threads)
    return out


def tree_dependent(tris, rays, threads: int = 0):
    """(mask, leaf-only answers, robust answers): mask marks the rays whose reference
    answer depends on the reference's tree (see orc_brute_force_robust)."""
    a = brute_force(tris, rays, threads)
    b = brute_force_robust(tris, rays, threads)
    diff = (a["valid"] != b["valid"]) | (a["t"].view(np.uint32) != b["t"].view(np.uint32)) | \
        ((a["valid"] != 0) & (a["primitive_id"] != b["primitive_id"]))
    return diff, a, b


def intersect_tri(tri9, ray6):
    tri, ray = _f32(tri9, 9)[0], _f32(ray6, 6)[0]
    t, u, v = (ctypes.c_float(0), ctypes.c_float(0), ctypes.c_float(0))
    ok = lib().orc_intersect_tri(tri.ctypes.data, ray.ctypes.data, ctypes.byref(t),
                                 ctypes.byref(u), ctypes.byref(v))
    return bool(ok), t.value, u.value, v.value


def ref_available() -> bool:
    return os.path.exists(REF_BIN)


def run_reference(tris, rays, combos: bool = False, repeat: int = 1):
    """Run the reference's CPU backend on (tris, rays).  Returns (full records,
    {combo name: raw bytes}, timing dict)."""
    if not ref_available():
        raise RuntimeError("oracle/_ref/ref_oracle is not built")
    tris, rays = _f32(tris, 9), _f32(rays, 6)
    with tempfile.TemporaryDirectory() as d:
        tp, rp = os.path.join(d, "tris.f32"), os.path.join(d, "rays.f32")
        tris.tofile(tp)
        rays.tofile(rp)
        cmd = [REF_BIN, tp, rp, d, "--repeat", str(repeat)] + (["--combos"] if combos else [])
        res = subprocess.run(cmd, check=True, capture_output=True, text=True)
        timing = json.loads(res.stdout.strip().splitlines()[-1])
        full = np.fromfile(os.path.join(d, "full.bin"), dtype=HIT_DTYPE)
        raw = {}
        if combos:
            for f in os.listdir(d):
                if f.endswith(".bin") and f != "full.bin":
                    with open(os.path.join(d, f), "rb") as fh:
                        raw[f[:-4]] = fh.read()
    return full, raw, timing


def camera_rays(width, height, form, pos, sensor_size, sensor_dist=0.0, sensor_z=0.0,
                cos_a=1.0, sin_a=0.0) -> np.ndarray:
    """The examples' pinhole sensor camera (orc_camera_rays)."""
    class _Cam(ctypes.Structure):
        _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                    ("form", ctypes.c_uint32), ("pad", ctypes.c_uint32),
                    ("pos", ctypes.c_float * 3), ("sensor_size", ctypes.c_float),
                    ("sensor_dist", ctypes.c_float), ("sensor_z", ctypes.c_float),
                    ("cos_a", ctypes.c_float), ("sin_a", ctypes.c_float)]
    c = _Cam(width, height, form, 0, (ctypes.c_float * 3)(*pos), sensor_size, sensor_dist,
             sensor_z, cos_a, sin_a)
    out = np.zeros((width * height, 6), np.float32)
    lib().orc_camera_rays(ctypes.byref(c), out.ctypes.data)
    return out


def lambert(tris, rays, hits) -> np.ndarray:
    """RGBA8 Lambert image of full hit records (orc_lambert)."""
    tris, rays = _f32(tris, 9), _f32(rays, 6)
    hits = np.ascontiguousarray(hits, dtype=HIT_DTYPE)
    out = np.zeros((len(rays), 4), np.uint8)
    lib().orc_lambert(tris.ctypes.data, rays.ctypes.data, hits.ctypes.data, len(rays),
                      out.ctypes.data)
    return out
