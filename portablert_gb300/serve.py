"""Request server over resident scenes (the prt_b200_server_* C ABI).

Scenes are built once and stay in HBM; requests (scene, rays, tags) are admitted in
arrival order while their device buffers fit a memory budget and run as waves -- one
persistent launch per group of admitted requests -- on several streams at once.  Each
request's records are what ``B200Backend.nearest_hits`` gives on its scene alone.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib, hitreg


class Server:
    def __init__(self, backend, tris_ptr: int, tri_off, budget_bytes: int, lanes: int = 4):
        backend._need()
        self.backend = backend
        self._L = backend._L
        off = np.ascontiguousarray(np.asarray(tri_off, dtype=np.uint64))
        h = ctypes.c_void_p()
        rc = self._L.prt_b200_server_create(backend.ctx, tris_ptr,
                                            off.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                            len(off) - 1, int(budget_bytes), int(lanes),
                                            ctypes.byref(h))
        _lib.check(rc, backend.ctx, self._L)
        self.h = h
        self._keep = {}

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self._L.prt_b200_server_destroy(self.h)
        self.h = None
        self._keep = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != _lib.PRT_OK:
            msg = self._L.prt_b200_server_last_error(self.h)
            raise _lib.PrtError(rc, msg.decode() if msg else "")

    def submit_ptr(self, scene: int, rays_ptr: int, n: int, tags, out_ptr: int) -> int:
        """Queues a request on host buffers given by address (kept alive by the caller)."""
        lay = hitreg.layout(tags)
        t = ctypes.c_uint64()
        self._check(self._L.prt_b200_server_submit(self.h, scene, ctypes.c_void_p(rays_ptr), n,
                                                   lay.mask, lay.size, lay.offsets8(),
                                                   ctypes.c_void_p(out_ptr), ctypes.byref(t)))
        return t.value

    def submit(self, scene: int, rays, tags):
        """Queues a request on numpy rays; returns (ticket, records array filled when
        wait(ticket) returns)."""
        lay = hitreg.layout(tags)
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        out = np.zeros(len(rays), dtype=lay.numpy_dtype())
        t = self.submit_ptr(scene, rays.ctypes.data, len(rays), tags, out.ctypes.data)
        self._keep[t] = (rays, out)
        return t, out

    def wait(self, ticket: int) -> float:
        """Blocks until the request is answered; returns its latency in ms."""
        ms = ctypes.c_double()
        rc = self._L.prt_b200_server_wait(self.h, ticket, ctypes.byref(ms))
        self._keep.pop(ticket, None)
        self._check(rc)
        return ms.value

    def stat(self, key: str) -> float:
        v = ctypes.c_double()
        self._check(self._L.prt_b200_server_stat(self.h, key.encode(), ctypes.byref(v)))
        return v.value
