"""Seeded synthetic scenes and ray batches for the nearest-hit workloads.

No public benchmark or dataset is attached to portableRT's ray-query path, so these
deterministic generators define the workloads.  All randomness comes from SplitMix64
(Steele, Lea, Flood 2014): output k of a stream is ``mix(state0 + k * gamma)``, which
vectorises in numpy.  A uniform in [0, 1) is ``(x >> 40) * 2**-24`` (exact in FP32),
mapped to [a, b) as ``a + (b - a) * u`` in FP32.  Gaussians use Box-Muller in double
and are rounded to FP32.

Workloads (triangles are ``n x 9`` float32 = v0, v1, v2; rays are ``m x 6`` float32 =
origin, direction, the AoS layouts of ``portableRT::Tri`` and ``portableRT::Ray``):

* ``soup``: triangle centres uniform in [-1, 1]^3, vertex offsets uniform in
  [-0.05, 0.05]^3; ray origins on the sphere of radius 3, aimed at a point uniform in
  [-0.5, 0.5]^3.  4,096 triangles / 65,536 rays is the small case.
* ``heightfield``: 1024 x 512 quads over [-4, 4] x [-2, 2], two triangles per quad,
  height = sum of 8 sinusoids (frequency in [0.5, 8], phase and heading in [0, 2 pi),
  amplitude 1/f); 1920 x 1080 pinhole camera from (0, 3, -6) at the origin, 60 degree
  vertical field of view; secondary rays leave primary hit points with cosine-weighted
  directions about the geometric normal that faces the primary ray.
* ``clusters``: 256 Gaussian clusters (centres in [-10, 10]^3, sigma in [0.1, 1]),
  triangle edges uniform in [-0.02, 0.02]^3; ray origins in [-12, 12]^3 with
  directions uniform on the sphere.
* ``batch_sizes``: per-scene triangle and ray counts, log-uniform, for many small
  soup scenes.
"""
from __future__ import annotations

import math

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _mix(z: np.ndarray) -> np.ndarray:
    z = z.astype(np.uint64, copy=True)
    with np.errstate(over="ignore"):
        z ^= z >> np.uint64(30)
        z *= _M1
        z ^= z >> np.uint64(27)
        z *= _M2
        z ^= z >> np.uint64(31)
    return z


class Stream:
    """One SplitMix64 stream, identified by (seed, stream id)."""

    def __init__(self, seed: int, sid: int):
        s = np.array([(seed & 0xFFFFFFFF) | ((sid & 0xFFFFFFFF) << 32)], dtype=np.uint64)
        self.state = _mix(s)[0]

    def u64(self, n: int) -> np.ndarray:
        k = np.arange(1, n + 1, dtype=np.uint64)
        with np.errstate(over="ignore"):
            z = self.state + _GAMMA * k
            self.state = self.state + _GAMMA * np.uint64(n)
        return _mix(z)

    def u01(self, shape) -> np.ndarray:
        n = int(np.prod(shape))
        x = (self.u64(n) >> np.uint64(40)).astype(np.float32) * np.float32(2.0 ** -24)
        return x.reshape(shape)

    def uniform(self, a: float, b: float, shape) -> np.ndarray:
        a32, b32 = np.float32(a), np.float32(b)
        return (a32 + (b32 - a32) * self.u01(shape)).astype(np.float32)

    def u01_f64(self, shape) -> np.ndarray:
        n = int(np.prod(shape))
        return ((self.u64(n) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53).reshape(shape)

    def gauss(self, shape) -> np.ndarray:
        """Standard normals (double) by Box-Muller, one pair of uniforms per value."""
        n = int(np.prod(shape))
        u1 = 1.0 - self.u01_f64((n,))  # (0, 1]
        u2 = self.u01_f64((n,))
        g = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)
        return g.reshape(shape)


def _normalize32(v: np.ndarray) -> np.ndarray:
    v = v.astype(np.float32)
    n = np.sqrt(v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2])
    return (v / n[:, None]).astype(np.float32)


def soup_tris(seed: int, n_tris: int) -> np.ndarray:
    s = Stream(seed, 1)
    c = s.uniform(-1.0, 1.0, (n_tris, 1, 3))
    off = s.uniform(-0.05, 0.05, (n_tris, 3, 3))
    return (c + off).astype(np.float32).reshape(n_tris, 9)


def soup_rays(seed: int, n_rays: int) -> np.ndarray:
    s = Stream(seed, 2)
    g = s.gauss((n_rays, 3)).astype(np.float32)
    origin = (np.float32(3.0) * _normalize32(g)).astype(np.float32)
    target = s.uniform(-0.5, 0.5, (n_rays, 3))
    d = _normalize32(target - origin)
    return np.concatenate([origin, d], axis=1).astype(np.float32)


def soup(seed: int = 0, n_tris: int = 4096, n_rays: int = 65536):
    return soup_tris(seed, n_tris), soup_rays(seed, n_rays)


# ---------------------------------------------------------------- heightfield

HF_NX, HF_NZ = 1024, 512
HF_SECONDARY, HF_DELTA = 4_194_304, 0.01 # secondary rays of the heightfield workload
CAM_EYE = (0.0, 3.0, -6.0)
CAM_W, CAM_H = 1920, 1080


def heightfield_params(seed: int = 1):
    s = Stream(seed, 1)
    f = 0.5 + 7.5 * s.u01_f64((8,))
    phase = 2.0 * np.pi * s.u01_f64((8,))
    heading = 2.0 * np.pi * s.u01_f64((8,))
    return f, phase, heading


def heightfield_tris(seed: int = 1, nx: int = HF_NX, nz: int = HF_NZ) -> np.ndarray:
    f, phase, heading = heightfield_params(seed)
    xs = -4.0 + 8.0 * np.arange(nx + 1, dtype=np.float64) / nx
    zs = -2.0 + 4.0 * np.arange(nz + 1, dtype=np.float64) / nz
    X, Z = np.meshgrid(xs, zs)  # shape (nz+1, nx+1), row j = z index
    H = np.zeros_like(X)
    for k in range(8):
        H += np.sin(f[k] * (X * math.cos(heading[k]) + Z * math.sin(heading[k])) + phase[k]) / f[k]
    V = np.stack([X, H, Z], axis=-1).astype(np.float32)  # (nz+1, nx+1, 3)
    v00 = V[:-1, :-1]
    v10 = V[:-1, 1:]
    v01 = V[1:, :-1]
    v11 = V[1:, 1:]
    t0 = np.concatenate([v00, v10, v01], axis=-1)  # (nz, nx, 9)
    t1 = np.concatenate([v10, v11, v01], axis=-1)
    tris = np.stack([t0, t1], axis=2).reshape(-1, 9)  # quad q = j*nx + i -> tris 2q, 2q+1
    return np.ascontiguousarray(tris, dtype=np.float32)


def camera_rays(width: int = CAM_W, height: int = CAM_H, eye=CAM_EYE, target=(0.0, 0.0, 0.0),
                up=(0.0, 1.0, 0.0), vfov_deg: float = 60.0) -> np.ndarray:
    """Pinhole rays through pixel centres, row-major from the top-left pixel."""
    eye = np.asarray(eye, np.float64)
    fwd = np.asarray(target, np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, np.asarray(up, np.float64))
    right /= np.linalg.norm(right)
    upv = np.cross(right, fwd)
    th = math.tan(math.radians(vfov_deg) / 2.0)
    aspect = width / height
    px = (2.0 * (np.arange(width) + 0.5) / width - 1.0) * th * aspect
    py = (1.0 - 2.0 * (np.arange(height) + 0.5) / height) * th
    PX, PY = np.meshgrid(px, py)  # (height, width)
    d = fwd[None, None, :] + PX[..., None] * right + PY[..., None] * upv
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    d = d.reshape(-1, 3).astype(np.float32)
    o = np.broadcast_to(eye.astype(np.float32), d.shape)
    return np.ascontiguousarray(np.concatenate([o, d], axis=1), dtype=np.float32)


def _onb(n: np.ndarray):
    """Orthonormal basis about unit normals n (Duff et al. 2017, branchless)."""
    sign = np.where(n[:, 2] >= 0.0, 1.0, -1.0)
    a = -1.0 / (sign + n[:, 2])
    b = n[:, 0] * n[:, 1] * a
    t = np.stack([1.0 + sign * n[:, 0] * n[:, 0] * a, sign * b, -sign * n[:, 0]], axis=1)
    bt = np.stack([b, sign + n[:, 1] * n[:, 1] * a, -n[:, 1]], axis=1)
    return t, bt


def secondary_rays(tris: np.ndarray, primary: np.ndarray, hit_valid: np.ndarray,
                   hit_pid: np.ndarray, hit_p: np.ndarray, n_rays: int, delta: float = 0.01,
                   seed: int = 1) -> np.ndarray:
    """Cosine-hemisphere rays from primary hit points.

    Ray k starts at the (k mod H)-th valid primary hit in pixel order (H = number of
    valid hits).  The origin is the hit point ``p`` moved by ``delta`` along the
    geometric normal that faces the primary ray (``delta = 0`` keeps ``p`` exactly).
    """
    idx = np.flatnonzero(hit_valid)
    if idx.size == 0:
        raise ValueError("no primary hits")
    src = idx[np.arange(n_rays) % idx.size]
    tri = tris[hit_pid[src]].astype(np.float64)
    e1 = tri[:, 3:6] - tri[:, 0:3]
    e2 = tri[:, 6:9] - tri[:, 0:3]
    n = np.cross(e1, e2)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    dprim = primary[src, 3:6].astype(np.float64)
    flip = np.einsum("ij,ij->i", n, dprim) > 0.0
    n[flip] = -n[flip]
    p = hit_p[src].astype(np.float32)
    if delta != 0.0:
        origin = (p.astype(np.float64) + delta * n).astype(np.float32)
    else:
        origin = p
    s = Stream(seed, 3)
    u1 = s.u01_f64((n_rays,))
    u2 = s.u01_f64((n_rays,))
    r = np.sqrt(u1)
    phi = 2.0 * np.pi * u2
    lx, ly, lz = r * np.cos(phi), r * np.sin(phi), np.sqrt(np.maximum(0.0, 1.0 - u1))
    t, bt = _onb(n)
    d = lx[:, None] * t + ly[:, None] * bt + lz[:, None] * n
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.ascontiguousarray(np.concatenate([origin, d.astype(np.float32)], axis=1),
                                dtype=np.float32)


# ---------------------------------------------------------------- clustered soup

def cluster_tris(seed: int = 2, n_tris: int = 8_388_608, n_clusters: int = 256) -> np.ndarray:
    s = Stream(seed, 1)
    centre = s.uniform(-10.0, 10.0, (n_clusters, 3))
    sigma = s.uniform(0.1, 1.0, (n_clusters,))
    cid = np.minimum((s.u01((n_tris,)) * np.float32(n_clusters)).astype(np.int64),
                     n_clusters - 1)
    g = s.gauss((n_tris, 3)).astype(np.float32)
    v0 = (centre[cid] + sigma[cid, None] * g).astype(np.float32)
    v1 = (v0 + s.uniform(-0.02, 0.02, (n_tris, 3))).astype(np.float32)
    v2 = (v0 + s.uniform(-0.02, 0.02, (n_tris, 3))).astype(np.float32)
    return np.ascontiguousarray(np.concatenate([v0, v1, v2], axis=1), dtype=np.float32)


def random_rays(seed: int = 2, n_rays: int = 16_777_216, extent: float = 12.0) -> np.ndarray:
    s = Stream(seed, 2)
    o = s.uniform(-extent, extent, (n_rays, 3))
    d = _normalize32(s.gauss((n_rays, 3)).astype(np.float32))
    return np.ascontiguousarray(np.concatenate([o, d], axis=1), dtype=np.float32)


# ---------------------------------------------------------------- many small scenes

def log_uniform_int(s: Stream, lo: int, hi: int, n: int) -> np.ndarray:
    u = s.u01_f64((n,))
    return np.floor(np.exp(math.log(lo) + u * (math.log(hi) - math.log(lo)))).astype(np.int64)


def batch_sizes(n_scenes: int = 4096, seed: int = 3, tri_range=(16, 65_536),
                ray_range=(64, 262_144)):
    s = Stream(seed, 7)
    return (log_uniform_int(s, tri_range[0], tri_range[1], n_scenes),
            log_uniform_int(s, ray_range[0], ray_range[1], n_scenes))


# ---------------------------------------------------------------- device generation

GEN_SOUP_TRIS, GEN_SOUP_RAYS, GEN_CLUSTER_TRIS, GEN_RANDOM_RAYS = 0, 1, 2, 3


def generate_dev(backend, kind: int, seed: int, n: int, out_ptr: int, param: float = 0.0,
                 stream: int | None = None) -> None:
    """Writes the generator `kind` (GEN_*) for `seed` straight into device memory at
    out_ptr (prt_b200_generate): n x 9 floats for triangles, n x 6 for rays.  Queued on
    `stream` (None = the backend context's stream)."""
    import ctypes

    backend._need()
    backend._check(backend._L.prt_b200_generate(backend.ctx, int(kind), int(seed), int(n),
                                                float(param), ctypes.c_void_p(out_ptr),
                                                ctypes.c_void_p(stream) if stream else None))


# ---------------------------------------------------------------- command line

def run_clustered(n_rays: int = 1_048_576, repeats: int = 2) -> dict:
    """The clustered soup (8,388,608 triangles, seed 2) with `n_rays` random rays (seed 2),
    generated on the device: one set_tris, then `repeats` nearest_hits_dev passes with
    FP32 nodes and `repeats` with compressed nodes (tags uv, t, primitive_id, valid) --
    the launches a profiler capture of either node format selects from."""
    import torch

    from . import backend, hitreg

    b = backend.B200Backend(0)
    b.init()
    n_t = 8_388_608
    tags = ("uv", "t", "primitive_id", "valid")
    lay = hitreg.layout(tags)
    d_t = torch.empty(n_t * 9, dtype=torch.float32, device="cuda")
    d_r = torch.empty(n_rays * 6, dtype=torch.float32, device="cuda")
    out = torch.zeros(n_rays * lay.size, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    generate_dev(b, GEN_CLUSTER_TRIS, 2, n_t, d_t.data_ptr(), 256)
    generate_dev(b, GEN_RANDOM_RAYS, 2, n_rays, d_r.data_ptr(), 12.0)
    b.sync()
    b.set_tris_dev(d_t.data_ptr(), n_t)
    for fmt in (0, 1):
        b.set_option("node_format", fmt)
        for _ in range(repeats):
            b.nearest_hits_dev(d_r.data_ptr(), n_rays, out.data_ptr(), tags)
        b.sync()
    b.set_option("node_format", 0)
    b.set_option("count_visits", 1)
    b.nearest_hits_dev(d_r.data_ptr(), n_rays, out.data_ptr(), tags)
    b.sync()
    res = {"nodes": b.stat("n_nodes"), "depth": b.stat("depth"),
           "node_visits_per_ray": b.stat("visits_nodes") / n_rays,
           "tri_tests_per_ray": b.stat("visits_tris") / n_rays}
    b.shutdown()
    return res


def heightfield_workload(primary_hits):
    """The heightfield workload: 1,048,576 triangles (seed 1), 1920x1080 pinhole primary
    rays and HF_SECONDARY cosine secondary rays (seed 1) leaving the primary hits offset
    by HF_DELTA.  primary_hits(tris, prim) returns the primary rays' records as a dict of
    fields (valid, primitive_id, px, py, pz)."""
    tris = heightfield_tris(seed=1)
    prim = camera_rays()
    h = primary_hits(tris, prim)
    sec = secondary_rays(tris, prim, h["valid"] != 0, h["primitive_id"],
                         np.stack([h["px"], h["py"], h["pz"]], 1), HF_SECONDARY,
                         delta=HF_DELTA, seed=1)
    rays = np.ascontiguousarray(np.concatenate([prim, sec]), dtype=np.float32)
    return tris, prim, rays


def run_heightfield(repeats: int = 2) -> dict:
    """The heightfield workload (all five tags): one set_tris, then `repeats`
    nearest_hits_dev passes with FP32 nodes and `repeats` with compressed nodes over all
    6,267,904 rays -- the launches a profiler capture of the regular pass selects from
    (the primary-ray pass that makes the secondary rays comes first)."""
    import torch

    from . import backend, hitreg

    b = backend.B200Backend(0)
    b.init()

    def primary_hits(tris, prim):
        b.set_tris(tris)
        return b.nearest_hits(prim, hitreg.TAGS)

    tris, prim, rays = heightfield_workload(primary_hits)
    n = len(rays)
    lay = hitreg.layout(hitreg.TAGS)
    d_r = torch.from_numpy(rays).cuda()
    out = torch.zeros(n * lay.size, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    for fmt in (0, 1):
        b.set_option("node_format", fmt)
        for _ in range(repeats):
            b.nearest_hits_dev(d_r.data_ptr(), n, out.data_ptr(), hitreg.TAGS)
        b.sync()
    b.set_option("node_format", 0)
    b.set_option("count_visits", 1)
    b.nearest_hits_dev(d_r.data_ptr(), n, out.data_ptr(), hitreg.TAGS)
    b.sync()
    res = {"rays": n, "nodes": b.stat("n_nodes"), "depth": b.stat("depth"),
           "node_visits_per_ray": b.stat("visits_nodes") / n,
           "tri_tests_per_ray": b.stat("visits_tris") / n}
    b.shutdown()
    return res


def run_heightfield_build(repeats: int = 2) -> dict:
    """set_tris_dev of the 1,048,576-triangle heightfield (seed 1) `repeats` times with the
    default SAH build: the launches a profiler capture of the build selects from."""
    import torch

    from . import backend

    b = backend.B200Backend(0)
    b.init()
    tris = heightfield_tris(seed=1)
    d = torch.from_numpy(tris).cuda()
    torch.cuda.synchronize()
    ms = []
    for _ in range(repeats):
        b.set_tris_dev(d.data_ptr(), len(tris))
        ms.append(b.stat("build_ms"))
    res = {"build_ms": ms, "nodes": b.stat("n_nodes"), "depth": b.stat("depth")}
    b.shutdown()
    return res


def run_soup_build(n_tris: int = 4096, repeats: int = 2) -> dict:
    """set_tris of the small configuration's soup (seed 0, n_tris triangles) `repeats`
    times with the default SAH build."""
    from . import backend

    b = backend.B200Backend(0)
    b.init()
    tris = soup_tris(0, n_tris)
    ms = []
    for _ in range(repeats):
        b.set_tris(tris)
        ms.append(b.stat("build_ms"))
    res = {"build_ms": ms, "nodes": b.stat("n_nodes"), "depth": b.stat("depth")}
    b.shutdown()
    return res


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description="run a workload on cuda:0")
    ap.add_argument("workload",
                    choices=["clustered", "heightfield", "heightfield-build", "soup-build"])
    ap.add_argument("--tris", type=int, default=4096)
    ap.add_argument("--rays", type=int, default=1_048_576)
    ap.add_argument("--repeats", type=int, default=2)
    args = ap.parse_args()
    if args.workload == "clustered":
        print(run_clustered(args.rays, args.repeats))
    elif args.workload == "heightfield":
        print(run_heightfield(args.repeats))
    elif args.workload == "soup-build":
        print(run_soup_build(args.tris, args.repeats))
    else:
        print(run_heightfield_build(args.repeats))
