"""Python mirror of portableRT's backend interface for the GB300 backend.

portableRT (include/portableRT/backend.hpp) exposes ``available_backends()``,
``select_backend()``, ``Backend::set_tris(Tris)``, ``Backend::device_name()`` and the
free function ``nearest_hits<Tags...>(rays)`` returning ``std::vector<HitReg<Tags...>>``.
This module offers the same calls over the C ABI of libprt_b200.so, with numpy arrays
in place of the std::vectors: triangles ``(n, 9)`` float32, rays ``(m, 6)`` float32,
hits a structured array whose bytes are exactly ``HitReg<Tags...>``.

Errors raise ``PrtError`` (a RuntimeError), as the reference throws std::runtime_error.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib, hitreg

ALL_TAGS = hitreg.TAGS


class B200Backend:
    """The GB300 backend (registered under the name "B200", like the C++ class)."""

    def __init__(self, device: int = 0):
        self._name = "B200"
        self.device = device
        self.ctx = None
        self._L = None

    # -- Backend interface (backend.hpp:16-23) --------------------------------------
    def name(self) -> str:
        return self._name

    def is_available(self) -> bool:
        try:
            return bool(_lib.load().prt_b200_available())
        except (OSError, RuntimeError):
            return False

    def init(self) -> None:
        if self.ctx is not None:
            return
        L = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(L.prt_b200_create(self.device, ctypes.byref(h)), None, L)
        self.ctx, self._L = h, L

    def shutdown(self) -> None:
        if self.ctx is not None:
            self._L.prt_b200_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.shutdown()
        except Exception:
            pass

    def device_name(self) -> str:
        self._need()
        buf = ctypes.create_string_buffer(256)
        self._check(self._L.prt_b200_device_name(self.ctx, buf, 256))
        return buf.value.decode()

    def set_tris(self, tris) -> None:
        self._need()
        t = np.ascontiguousarray(np.asarray(tris, dtype=np.float32).reshape(-1, 9))
        self._check(self._L.prt_b200_set_tris(self.ctx, t.ctypes.data, t.shape[0]))

    def set_tris_dev(self, ptr: int, n: int) -> None:
        self._need()
        self._check(self._L.prt_b200_set_tris_dev(self.ctx, ptr, n))

    def nearest_hits(self, rays, tags=ALL_TAGS) -> np.ndarray:
        """HitReg<tags...> records for every ray (host arrays, synchronous)."""
        self._need()
        r = np.ascontiguousarray(np.asarray(rays, dtype=np.float32).reshape(-1, 6))
        lay = hitreg.layout(tags)
        out = np.zeros(r.shape[0], dtype=lay.numpy_dtype())
        self._check(self._L.prt_b200_nearest_hits(self.ctx, r.ctypes.data, r.shape[0], lay.mask,
                                                  lay.size, lay.offsets8(), out.ctypes.data))
        return out

    def nearest_hits_dev(self, rays_ptr: int, n: int, out_ptr: int, tags=ALL_TAGS,
                         stream: int = 0) -> None:
        """Device-resident call: queues the traversal on `stream` (0 = the backend's)."""
        self._need()
        lay = hitreg.layout(tags)
        self._check(self._L.prt_b200_nearest_hits_dev(self.ctx, rays_ptr, n, lay.mask, lay.size,
                                                      lay.offsets8(), out_ptr, stream or None))

    def sync(self) -> None:
        self._need()
        self._check(self._L.prt_b200_sync(self.ctx))

    # -- the examples' camera and shading, on the device ------------------------------------
    def nearest_hits_camera(self, cam, out_ptr: int, tags=ALL_TAGS, stream: int = 0) -> None:
        """Records of the camera's width x height rays (built on the device) to out_ptr."""
        self._need()
        lay = hitreg.layout(tags)
        self._check(self._L.prt_b200_nearest_hits_camera(self.ctx, ctypes.byref(cam), lay.mask,
                                                         lay.size, lay.offsets8(), out_ptr,
                                                         stream or None))

    def camera_rays(self, cam, out_ptr: int, stream: int = 0) -> None:
        self._need()
        self._check(self._L.prt_b200_camera_rays(self.ctx, ctypes.byref(cam), out_ptr,
                                                 stream or None))

    def shade_lambert(self, records_ptr: int, tags, rgba_ptr: int, cam=None, rays_ptr: int = 0,
                      n: int = 0, stream: int = 0) -> None:
        """RGBA8 Lambert image of device records (t and primitive_id needed)."""
        self._need()
        lay = hitreg.layout(tags)
        self._check(self._L.prt_b200_shade_lambert(
            self.ctx, ctypes.byref(cam) if cam is not None else None, rays_ptr or None, n,
            records_ptr, lay.mask, lay.size, lay.offsets8(), rgba_ptr, stream or None))

    def t_error(self, tris_ptr: int, n_tris: int, rays_ptr: int, n_rays: int, out_ptr: int,
                tags) -> dict:
        """FP64 score of the t values in a device record buffer (prt_b200_t_error)."""
        self._need()
        lay = hitreg.layout(tags)
        r = (ctypes.c_double * 6)()
        self._check(self._L.prt_b200_t_error(self.ctx, tris_ptr, n_tris, rays_ptr, n_rays,
                                             out_ptr, lay.mask, lay.size, lay.offsets8(), r))
        return {"max_abs": r[0], "max_rel": r[1], "mean_abs": r[2], "scored": int(r[3]),
                "exact": int(r[4]), "unscored": int(r[5])}

    def probe_read_gbs(self, buf_ptr: int, nbytes: int, passes: int = 50) -> float:
        """Read bandwidth (GB/s) of the traversal's 32-byte loads over a device buffer
        (prt_b200_probe_read): under the L2 capacity the L2 -> SM bandwidth."""
        self._need()
        ms = ctypes.c_float()
        self._check(self._L.prt_b200_probe_read(self.ctx, buf_ptr, nbytes, passes,
                                                ctypes.byref(ms)))
        return nbytes * passes / (ms.value / 1e3) / 1e9

    # -- tuning and statistics ----------------------------------------------------------
    def set_option(self, key: str, value: int) -> None:
        self._need()
        self._check(self._L.prt_b200_set_option(self.ctx, key.encode(), int(value)))

    def stat(self, key: str) -> float:
        self._need()
        v = ctypes.c_double()
        self._check(self._L.prt_b200_get_stat(self.ctx, key.encode(), ctypes.byref(v)))
        return v.value

    # -----------------------------------------------------------------------------------
    def _need(self):
        if self.ctx is None:
            self.init()

    def _check(self, rc):
        _lib.check(rc, self.ctx, self._L)


# -- the registry (backend.hpp:39-95, src/backend.cpp:50-56) ------------------------------
_all = []
_available = []
selected_backend = None


def _register(b) -> None:
    if b.is_available():
        _available.append(b)
    _all.append(b)


def all_backends():
    if not _all:
        _register(B200Backend())
    return list(_all)


def available_backends():
    all_backends()
    return list(_available)


def select_backend(b) -> None:
    """Shuts the previous backend down and initialises `b` (backend.cpp:50-56)."""
    global selected_backend
    if selected_backend is not None and selected_backend is not b:
        selected_backend.shutdown()
    selected_backend = b
    b.init()


def nearest_hits(rays, *tags) -> np.ndarray:
    """portableRT::nearest_hits<Tags...>(rays); no tags means all five."""
    if selected_backend is None:
        raise RuntimeError("Unknown backend")
    return selected_backend.nearest_hits(rays, tags or ALL_TAGS)
