"""Autotuner for batched builds and queries (many scenes, one graph).

The knobs are the options of the C ABI that change speed and never answers:

* ``leaf_size``   most triangles per leaf of the 8-wide tree (the build): larger leaves
                  trade node visits for triangle tests (a test costs about a quarter
                  of a visit), which pays in dense scenes;
* ``node_format`` FP32 or compressed 8-bit child boxes (the traversal's node bytes);
* ``block``       threads per traversal block (warps per block: shared memory per
                  block against blocks per SM);
* ``pool_depth``  the tree depth the graph's traversal pool is sized for (the pool is
                  the warp's traversal stack; smaller pools raise occupancy).

The tree width is fixed at 8 by the node layout.  Each candidate is captured as a
graph (build + query), replayed ``reps`` times with CUDA events around each replay,
and scored by its fastest replay; the winner is kept in a JSON cache keyed by the
device name and a signature of the workload (scene count, triangle and ray totals,
record layouts), so a later run of the same workload skips the search.  Each
candidate runs first with the pool sized for any tree (32 levels), which measures the
depth its build reaches, and then with the pool sized for exactly that depth.
"""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np

DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build",
                             "autotune.json")

KNOBS = ("leaf_size", "node_format", "block", "pool_depth")


def signature(tri_off, queries) -> str:
    off = np.asarray(tri_off, dtype=np.uint64)
    h = hashlib.sha1()
    h.update(off.tobytes())
    for q in queries:
        h.update(np.array([q.scene, q.field_mask, q.n_rays, q.rec_size], np.uint64).tobytes())
    return f"S{len(off) - 1}-T{int(off[-1])}-R{sum(int(q.n_rays) for q in queries)}-{h.hexdigest()[:16]}"


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, data):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def apply(backend, cfg: dict) -> None:
    backend.set_option("build_compressed", 1 if cfg["node_format"] == 1 else 0)
    for k in KNOBS:
        backend.set_option(k, int(cfg[k]))


def time_graph(batch, backend, d_tris_ptr, tri_off, qarr, stream, reps: int):
    """Milliseconds of each of `reps` replays (after the capture run) of build + query."""
    import torch

    batch.run_graph(d_tris_ptr, tri_off, qarr, stream.cuda_stream)
    batch.sync()
    out = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.run_graph(d_tris_ptr, tri_off, qarr, stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        out.append(e0.elapsed_time(e1))
    batch.sync()
    return out


def candidates(formats=(0, 1), leaf_sizes=(1, 2, 4, 8), blocks=(64, 128)):
    for fmt in formats:
        for leaf in leaf_sizes:
            for blk in blocks:
                yield {"node_format": fmt, "leaf_size": leaf, "block": blk}


def tune_batch(backend, d_tris_ptr: int, tri_off, queries, stream=None, reps: int = 3,
               formats=(0, 1), leaf_sizes=(1, 2, 4, 8), blocks=(64, 128), cache=DEFAULT_CACHE,
               refresh: bool = False, log=None) -> dict:
    """Best knob set for this batch (and the timings of every candidate tried).

    Leaves the backend's options set to the winner.  `queries` is a list or ctypes
    array of prt_b200_query.  Returns {"config": {...}, "ms": best, "tried": [...],
    "cached": bool}."""
    sig = signature(tri_off, queries)
    key = f"{backend.device_name()}|{sig}|{','.join(map(str, formats))}"
    data = _load(cache) if cache else {}
    if not refresh and key in data:
        best = data[key]
        apply(backend, best["config"])
        return dict(best, cached=True)
    import torch

    from . import _lib
    from .batch import Batch

    stream = stream or torch.cuda.Stream()

    qarr = queries if not isinstance(queries, list) else (_lib.Query * len(queries))(*queries)
    tried = []
    b = Batch(backend)
    try:
        for cand in candidates(formats, leaf_sizes, blocks):
            # First with the pool sized for any tree (learning this build's depth), then
            # with the pool sized for exactly that depth.
            pools, seen = [0], set()
            while pools:
                pd = pools.pop(0)
                cfg = dict(cand, pool_depth=pd)
                apply(backend, cfg)
                try:
                    ms = time_graph(b, backend, d_tris_ptr, tri_off, qarr, stream, reps)
                except _lib.PrtError as e:  # a pool too small reports an error, never a wrong answer
                    tried.append({"config": cfg, "ms": None, "error": str(e)})
                    continue
                d = int(b.stat("depth"))
                tried.append({"config": cfg, "ms": min(ms), "depth": d})
                if log:
                    log(f"autotune {cfg} -> {min(ms):.3f} ms (depth {d})")
                seen.add(pd)
                if pd == 0 and d < 32 and d not in seen:
                    pools.append(d)
    finally:
        b.close()
    tried_ok = [t for t in tried if t["ms"] is not None]
    if not tried_ok:
        raise RuntimeError("autotune: every candidate failed: " + tried[-1]["error"])
    best = min(tried_ok, key=lambda t: t["ms"])
    res = {"config": best["config"], "ms": best["ms"], "tried": tried}
    if cache:
        data[key] = res
        _store(cache, data)
    apply(backend, res["config"])
    return dict(res, cached=False)
