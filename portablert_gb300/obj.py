"""Wavefront OBJ meshes as triangle soups (prt_b200_obj_load), and a writer for the
synthetic meshes the tests and the bench use."""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib


def load_obj(path: str) -> np.ndarray:
    """n x 9 float32 triangles of every face (polygons as fans), in file order."""
    return load_soup("prt_b200_obj_load", path)


def load_soup(entry: str, path: str) -> np.ndarray:
    """n x 9 float32 triangles from one of the library's mesh readers (`entry`: its C
    name), copied out of the library's array, which is then freed."""
    L = _lib.load()
    p = ctypes.POINTER(ctypes.c_float)()
    n = ctypes.c_uint64()
    rc = getattr(L, entry)(str(path).encode(), ctypes.byref(p), ctypes.byref(n))
    _lib.check(rc, None, L)
    try:
        out = np.ctypeslib.as_array(p, shape=(n.value * 9,)).copy() if n.value else \
            np.zeros(0, np.float32)
    finally:
        L.prt_b200_free(p)
    return out.reshape(-1, 9)


def write_obj(path: str, vertices: np.ndarray, faces: np.ndarray) -> None:
    """Vertices (m x 3) and 0-based triangle faces (k x 3) as OBJ text."""
    with open(path, "w") as f:
        f.write(f"# {len(vertices)} vertices, {len(faces)} faces\n")
        for v in np.asarray(vertices, np.float64):
            f.write(f"v {v[0]:.7e} {v[1]:.7e} {v[2]:.7e}\n")
        for t in np.asarray(faces, np.int64):
            f.write(f"f {t[0] + 1} {t[1] + 1} {t[2] + 1}\n")


def blob_mesh(n_lat: int = 50, n_lon: int = 50, centre=(-0.017, 0.11, 0.0), radius=0.06,
              seed: int = 3):
    """A closed, bumpy sphere-like mesh (vertices, faces) the size and place of the
    examples' bunny (about 0.16 wide, centred near (-0.02, 0.11, 0)); 2 n_lon (n_lat - 1)
    triangles.  Bumps: 6 sinusoids of the direction with seeded frequencies."""
    rng = np.random.default_rng(seed)
    fr = rng.uniform(2.0, 7.0, (6, 3))
    ph = rng.uniform(0.0, 2.0 * math.pi, 6)
    th = np.linspace(0.0, math.pi, n_lat + 1)
    ph_lon = np.linspace(0.0, 2.0 * math.pi, n_lon, endpoint=False)
    T, P = np.meshgrid(th[1:-1], ph_lon, indexing="ij")
    d = np.stack([np.sin(T) * np.cos(P), np.cos(T), np.sin(T) * np.sin(P)], -1).reshape(-1, 3)
    d = np.concatenate([[[0.0, 1.0, 0.0]], d, [[0.0, -1.0, 0.0]]])
    r = radius * (1.0 + 0.08 * np.sin(d @ fr.T + ph).sum(1) / 3.0)
    verts = np.asarray(centre) + d * r[:, None]
    faces = []
    ring = lambda i, j: 1 + i * n_lon + (j % n_lon)
    for j in range(n_lon):
        faces.append((0, ring(0, j + 1), ring(0, j)))
    for i in range(n_lat - 2):
        for j in range(n_lon):
            a, b, c, e = ring(i, j), ring(i, j + 1), ring(i + 1, j), ring(i + 1, j + 1)
            faces += [(a, b, c), (b, e, c)]
    last = len(verts) - 1
    for j in range(n_lon):
        faces.append((last, ring(n_lat - 2, j), ring(n_lat - 2, j + 1)))
    return verts, np.asarray(faces, np.int64)
