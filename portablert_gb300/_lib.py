"""ctypes binding of libprt_b200.so (the C ABI declared in include/prt_b200.h).

The library is the only compute path: if it is missing this module raises instead of
falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

LIB_PATH = _build.LIB

# Every symbol include/prt_b200.h declares.
EXPORTS = (
    "prt_b200_available", "prt_b200_create", "prt_b200_destroy", "prt_b200_last_error",
    "prt_b200_device_name", "prt_b200_set_tris", "prt_b200_set_tris_dev",
    "prt_b200_nearest_hits", "prt_b200_nearest_hits_dev", "prt_b200_sync",
    "prt_b200_set_option", "prt_b200_get_stat", "prt_b200_nearest_hits_noalloc",
    "prt_b200_batch_create", "prt_b200_batch_destroy", "prt_b200_batch_set_tris_dev",
    "prt_b200_batch_query_dev", "prt_b200_batch_run_graph", "prt_b200_batch_sync",
    "prt_b200_batch_stat", "prt_b200_generate", "prt_b200_t_error",
    "prt_b200_server_create", "prt_b200_server_destroy", "prt_b200_server_submit",
    "prt_b200_server_wait", "prt_b200_server_stat", "prt_b200_server_last_error",
    "prt_b200_nearest_hits_camera", "prt_b200_camera_rays", "prt_b200_shade_lambert",
    "prt_b200_obj_load", "prt_b200_gltf_load", "prt_b200_free", "prt_b200_probe_read",
)


class Query(ctypes.Structure):
    """prt_b200_query (include/prt_b200.h)."""
    _fields_ = [("scene", ctypes.c_uint32), ("field_mask", ctypes.c_uint32),
                ("rays", ctypes.c_void_p), ("n_rays", ctypes.c_uint64),
                ("out", ctypes.c_void_p), ("rec_size", ctypes.c_uint32),
                ("offs", ctypes.c_uint8 * 8)]

class Camera(ctypes.Structure):
    """prt_b200_camera (include/prt_b200.h): the examples' pinhole sensor camera."""
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("form", ctypes.c_uint32), ("pad", ctypes.c_uint32),
                ("pos", ctypes.c_float * 3), ("sensor_size", ctypes.c_float),
                ("sensor_dist", ctypes.c_float), ("sensor_z", ctypes.c_float),
                ("cos_a", ctypes.c_float), ("sin_a", ctypes.c_float)]


CAMERA_PLANE, CAMERA_PLANE_SENSOR_NORM, CAMERA_ROTATED = 0, 1, 2

PRT_OK = 0
ERRORS = {1: "PRT_ERR_ARG", 2: "PRT_ERR_CUDA", 3: "PRT_ERR_NO_DEVICE", 4: "PRT_ERR_NO_SCENE",
          5: "PRT_ERR_DEVICE", 6: "PRT_ERR_OOM", 7: "PRT_ERR_LIMIT"}

_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads the library and declares the signatures (no CUDA call is made)."""
    global _lib
    if _lib is not None and path == LIB_PATH:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build the CUDA extension first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    L = ctypes.CDLL(path)
    vp, c_int, c_u64, c_u32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint32
    L.prt_b200_available.restype = c_int
    L.prt_b200_available.argtypes = []
    L.prt_b200_create.restype = c_int
    L.prt_b200_create.argtypes = [c_int, ctypes.POINTER(vp)]
    L.prt_b200_destroy.restype = None
    L.prt_b200_destroy.argtypes = [vp]
    L.prt_b200_last_error.restype = ctypes.c_char_p
    L.prt_b200_last_error.argtypes = [vp]
    L.prt_b200_device_name.restype = c_int
    L.prt_b200_device_name.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    L.prt_b200_set_tris.restype = c_int
    L.prt_b200_set_tris.argtypes = [vp, vp, c_u64]
    L.prt_b200_set_tris_dev.restype = c_int
    L.prt_b200_set_tris_dev.argtypes = [vp, vp, c_u64]
    L.prt_b200_nearest_hits.restype = c_int
    L.prt_b200_nearest_hits.argtypes = [vp, vp, c_u64, c_u32, c_u32, ctypes.c_char_p, vp]
    L.prt_b200_nearest_hits_dev.restype = c_int
    L.prt_b200_nearest_hits_dev.argtypes = [vp, vp, c_u64, c_u32, c_u32, ctypes.c_char_p, vp, vp]
    L.prt_b200_sync.restype = c_int
    L.prt_b200_sync.argtypes = [vp]
    L.prt_b200_nearest_hits_noalloc.restype = c_int
    L.prt_b200_nearest_hits_noalloc.argtypes = [vp, vp, c_u64, c_u32, c_u32, ctypes.c_char_p, vp]
    qp = ctypes.POINTER(Query)
    L.prt_b200_batch_create.restype = c_int
    L.prt_b200_batch_create.argtypes = [vp, ctypes.POINTER(vp)]
    L.prt_b200_batch_destroy.restype = None
    L.prt_b200_batch_destroy.argtypes = [vp]
    L.prt_b200_batch_set_tris_dev.restype = c_int
    L.prt_b200_batch_set_tris_dev.argtypes = [vp, vp, ctypes.POINTER(c_u64), c_u32]
    L.prt_b200_batch_query_dev.restype = c_int
    L.prt_b200_batch_query_dev.argtypes = [vp, qp, c_u32, vp]
    L.prt_b200_batch_run_graph.restype = c_int
    L.prt_b200_batch_run_graph.argtypes = [vp, vp, ctypes.POINTER(c_u64), c_u32, qp, c_u32, vp]
    L.prt_b200_batch_sync.restype = c_int
    L.prt_b200_batch_sync.argtypes = [vp]
    L.prt_b200_batch_stat.restype = c_int
    L.prt_b200_batch_stat.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)]
    L.prt_b200_generate.restype = c_int
    L.prt_b200_generate.argtypes = [vp, c_int, c_u64, c_u64, ctypes.c_double, vp, vp]
    L.prt_b200_server_create.restype = c_int
    L.prt_b200_server_create.argtypes = [vp, vp, ctypes.POINTER(c_u64), c_u32, c_u64, c_u32,
                                         ctypes.POINTER(vp)]
    L.prt_b200_server_destroy.restype = None
    L.prt_b200_server_destroy.argtypes = [vp]
    L.prt_b200_server_submit.restype = c_int
    L.prt_b200_server_submit.argtypes = [vp, c_u32, vp, c_u64, c_u32, c_u32, ctypes.c_char_p, vp,
                                         ctypes.POINTER(c_u64)]
    L.prt_b200_server_wait.restype = c_int
    L.prt_b200_server_wait.argtypes = [vp, c_u64, ctypes.POINTER(ctypes.c_double)]
    L.prt_b200_server_stat.restype = c_int
    L.prt_b200_server_stat.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)]
    L.prt_b200_server_last_error.restype = ctypes.c_char_p
    L.prt_b200_server_last_error.argtypes = [vp]
    L.prt_b200_obj_load.restype = c_int
    L.prt_b200_obj_load.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.POINTER(ctypes.c_float)),
                                    ctypes.POINTER(c_u64)]
    L.prt_b200_gltf_load.restype = c_int
    L.prt_b200_gltf_load.argtypes = L.prt_b200_obj_load.argtypes
    L.prt_b200_free.restype = None
    L.prt_b200_free.argtypes = [vp]
    cp = ctypes.POINTER(Camera)
    L.prt_b200_nearest_hits_camera.restype = c_int
    L.prt_b200_nearest_hits_camera.argtypes = [vp, cp, c_u32, c_u32, ctypes.c_char_p, vp, vp]
    L.prt_b200_camera_rays.restype = c_int
    L.prt_b200_camera_rays.argtypes = [vp, cp, vp, vp]
    L.prt_b200_shade_lambert.restype = c_int
    L.prt_b200_shade_lambert.argtypes = [vp, cp, vp, c_u64, vp, c_u32, c_u32, ctypes.c_char_p, vp,
                                         vp]
    L.prt_b200_t_error.restype = c_int
    L.prt_b200_t_error.argtypes = [vp, vp, c_u64, vp, c_u64, vp, c_u32, c_u32, ctypes.c_char_p,
                                   ctypes.POINTER(ctypes.c_double)]
    L.prt_b200_probe_read.restype = c_int
    L.prt_b200_probe_read.argtypes = [vp, vp, c_u64, c_int, ctypes.POINTER(ctypes.c_float)]
    L.prt_b200_set_option.restype = c_int
    L.prt_b200_set_option.argtypes = [vp, ctypes.c_char_p, ctypes.c_int64]
    L.prt_b200_get_stat.restype = c_int
    L.prt_b200_get_stat.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)]
    if path == LIB_PATH:
        _lib = L
    return L


class PrtError(RuntimeError):
    """A non-zero status from the C ABI (the reference throws std::runtime_error)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def check(rc: int, ctx=None, L=None) -> None:
    if rc != PRT_OK:
        L = L or load()
        msg = L.prt_b200_last_error(ctx)
        raise PrtError(rc, msg.decode() if msg else "")
