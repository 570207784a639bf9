"""Writes the golden vectors in tests/golden/ by running the reference's own CPU backend.

Run in a container that has the portableRT sources (oracle/Makefile `ref` target builds
oracle/_ref/ref_oracle from them):

    make -C oracle ref && python tests/golden/make_golden.py

Each set is an .npz with the inputs (`tris` n x 9, `rays` m x 6, float32) and the
reference's FullHitReg records (`full`, raw 32-byte records) plus, for `soup_small`,
the raw records of all 31 tag combinations (`combo_<name>`).  Bytes the reference
leaves indeterminate (absent fields, padding, u/v/primitive_id of misses) are stored
as written but are never compared.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import cpu  # noqa: E402
from portablert_gb300 import workloads as W  # noqa: E402


def kat():
    tris = np.array([[-1, -1, 0, 1, -1, 0, 0, 1, 0]], np.float32)
    rays = np.array([[0.1, 0, -1, 0, 0, 1], [-2, 0, -1, 0, 0, 1]], np.float32)
    return tris, rays


def grid_tris(n=8, z=0.0, flip=False):
    t = []
    for j in range(n):
        for i in range(n):
            v00, v10 = (i, j, z), (i + 1, j, z)
            v01, v11 = (i, j + 1, z), (i + 1, j + 1, z)
            a, b = (v00, v10, v01), (v10, v11, v01)
            if flip:
                a, b = a[::-1], b[::-1]
            t.append(sum(a, ()))
            t.append(sum(b, ()))
    return np.array(t, np.float32)


def axis_grid():
    """Integer grids at z=0 and z=1: axis-aligned rays land on vertices and edges and
    start on the triangles' bounding planes (the exact-zero direction cases)."""
    tris = np.concatenate([grid_tris(8, 0.0), grid_tris(8, 1.0, flip=True)])
    rays = []
    for y2 in range(0, 17):
        for x2 in range(0, 17):
            x, y = x2 / 2.0, y2 / 2.0
            rays.append((x, y, -1.0, 0.0, 0.0, 1.0))
            rays.append((x, y, 2.0, 0.0, 0.0, -1.0))
            rays.append((x, y, 0.5, 0.0, 0.0, 1.0))   # starts between the layers
            rays.append((x, y, 0.0, 0.0, 0.0, 1.0))   # starts on the lower layer
    for k in range(0, 9):
        rays.append((-1.0, float(k), 0.0, 1.0, 0.0, 0.0))   # in the plane z = 0
        rays.append((float(k), -1.0, 1.0, 0.0, 1.0, 0.0))   # in the plane z = 1
        rays.append((-1.0, float(k), 0.5, 1.0, 0.0, 0.0))   # between the planes
        rays.append((float(k), float(k), -1.0, 0.0, 1e-40, 1.0))  # denormal component
        rays.append((float(k), 0.5, -1.0, -0.0, 0.0, 1.0))  # negative zero
    s = W.Stream(11, 1)
    o = s.uniform(-1.0, 9.0, (200, 3))
    d = s.uniform(-1.0, 1.0, (200, 3))
    rays = np.concatenate([np.array(rays, np.float32), np.concatenate([o, d], 1)])
    return tris, rays.astype(np.float32)


def inside_soup():
    """Origins inside the soup: hits behind the origin (negative t) are accepted when
    the triangle's box reaches past the origin."""
    tris = W.soup_tris(21, 3000)
    s = W.Stream(21, 5)
    o = s.uniform(-1.0, 1.0, (3000, 3))
    d = W._normalize32(s.uniform(-1.0, 1.0, (3000, 3)))
    return tris, np.concatenate([o, d], 1).astype(np.float32)


def duplicates():
    """The same triangles repeated, some with their vertices rotated: exact ties."""
    s = W.Stream(31, 3)
    c = s.uniform(-0.3, 0.3, (60, 1, 3))
    base = (c + s.uniform(-0.3, 0.3, (60, 3, 3))).astype(np.float32).reshape(-1, 9)
    rot = base.reshape(-1, 3, 3)[:, [1, 2, 0], :].reshape(-1, 9)
    tris = np.concatenate([base, base, rot, base[::-1]]).astype(np.float32)
    return tris, W.soup_rays(31, 3000)


def one_tri():
    tris = np.array([[0.2, -0.4, 0.1, 0.9, 0.3, -0.2, -0.5, 0.6, 0.4]], np.float32)
    rays = W.soup_rays(41, 1500)
    extra = np.array([[0.2, -0.4, -3, 0, 0, 1], [0.9, 0.3, 3, 0, 0, -1],
                      [-0.5, 0.6, 0.4, 1, 0, 0], [0.0, 0.0, 0.0, 0, 0, 1]], np.float32)
    return tris, np.concatenate([rays, extra])


def two_tris():
    tris = np.array([[-0.6, -0.5, 0.0, 0.7, -0.4, 0.1, 0.0, 0.8, -0.1],
                     [-0.5, 0.5, 0.3, 0.6, 0.4, 0.2, 0.1, -0.7, 0.35]], np.float32)
    return tris, W.soup_rays(51, 1500)


def zero_tris():
    return np.zeros((0, 9), np.float32), W.soup_rays(61, 64)


def soup_small():
    return W.soup(seed=0, n_tris=512, n_rays=4096)


SETS = {
    "kat": kat,
    "axis_grid": axis_grid,
    "inside_soup": inside_soup,
    "duplicates": duplicates,
    "one_tri": one_tri,
    "two_tris": two_tris,
    "zero_tris": zero_tris,
    "soup_small": soup_small,
}


C0_TAGS = ("t", "primitive_id", "uv", "valid")


def c0_soup():
    """The small configuration exactly: 4,096-triangle soup and 65,536 rays (seed 0).
    Inputs are not stored (the seeded generator rebuilds them; their SHA-256 pins it);
    of the reference's records only the configuration's tags are kept (p is zeroed, as
    are u, v and primitive_id of misses, which the reference leaves unwritten)."""
    import hashlib

    tris, rays = W.soup(seed=0, n_tris=4096, n_rays=65536)
    full, _, _ = cpu.run_reference(tris, rays)
    full = full.copy()
    for f in ("px", "py", "pz"):
        full[f] = 0
    miss = full["valid"] == 0
    for f in ("u", "v", "primitive_id"):
        full[f][miss] = 0
    np.savez_compressed(os.path.join(HERE, "c0_soup.npz"),
                        full=full.view(np.uint8).reshape(-1, 32), tags=np.array(C0_TAGS),
                        tris_sha256=hashlib.sha256(tris.tobytes()).hexdigest(),
                        rays_sha256=hashlib.sha256(rays.tobytes()).hexdigest())
    print("c0_soup", tris.shape[0], rays.shape[0], int((~miss).sum()), "hits")


def main():
    if not cpu.ref_available():
        raise SystemExit("build oracle/_ref/ref_oracle first (make -C oracle ref)")
    c0_soup()
    for name, fn in SETS.items():
        tris, rays = fn()
        combos = name == "soup_small"
        full, raw, timing = cpu.run_reference(tris, rays, combos=combos)
        arrays = {"tris": tris, "rays": rays, "full": full.view(np.uint8).reshape(-1, 32)}
        if combos:
            for k, v in raw.items():
                arrays["combo_" + k] = np.frombuffer(v, np.uint8)[: 512 * 32].copy()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        print(name, tris.shape[0], rays.shape[0], int(full["valid"].sum()), "hits")


if __name__ == "__main__":
    main()
