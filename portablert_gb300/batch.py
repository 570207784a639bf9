"""Many scenes on the device at once (the prt_b200_batch_* C ABI).

A ``Batch`` builds S scenes in one pass and answers a list of queries -- (scene, rays,
output, tags) with device buffers -- with one persistent launch, optionally as one CUDA
graph together with the build.  Each answer is what ``B200Backend.nearest_hits`` gives
for that scene alone.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib, hitreg


def make_query(scene: int, rays_ptr: int, n_rays: int, out_ptr: int, tags) -> _lib.Query:
    lay = hitreg.layout(tags)
    q = _lib.Query()
    q.scene = scene
    q.field_mask = lay.mask
    q.rays = rays_ptr
    q.n_rays = n_rays
    q.out = out_ptr
    q.rec_size = lay.size
    q.offs[:] = list(lay.offsets8())
    return q


class Batch:
    def __init__(self, backend):
        backend._need()
        self.backend = backend
        self._L = backend._L
        h = ctypes.c_void_p()
        _lib.check(self._L.prt_b200_batch_create(backend.ctx, ctypes.byref(h)), backend.ctx,
                   self._L)
        self.h = h

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self._L.prt_b200_batch_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        _lib.check(rc, self.backend.ctx, self._L)

    @staticmethod
    def _offsets(tri_off):
        off = np.ascontiguousarray(np.asarray(tri_off, dtype=np.uint64))
        return off, off.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), len(off) - 1

    def set_tris_dev(self, tris_ptr: int, tri_off) -> None:
        off, p, s = self._offsets(tri_off)
        self._check(self._L.prt_b200_batch_set_tris_dev(self.h, tris_ptr, p, s))

    def query_dev(self, queries, stream: int = 0) -> None:
        arr = queries if isinstance(queries, ctypes.Array) else (_lib.Query * len(queries))(*queries)
        self._check(self._L.prt_b200_batch_query_dev(self.h, arr, len(queries), stream or None))

    def run_graph(self, tris_ptr: int, tri_off, queries, stream: int = 0) -> None:
        off, p, s = self._offsets(tri_off)
        arr = queries if isinstance(queries, ctypes.Array) else (_lib.Query * len(queries))(*queries)
        self._check(self._L.prt_b200_batch_run_graph(self.h, tris_ptr, p, s, arr, len(queries),
                                                     stream or None))

    def sync(self) -> None:
        self._check(self._L.prt_b200_batch_sync(self.h))

    def stat(self, key: str) -> float:
        v = ctypes.c_double()
        self._check(self._L.prt_b200_batch_stat(self.h, key.encode(), ctypes.byref(v)))
        return v.value
