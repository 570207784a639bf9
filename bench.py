"""Nearest-hit throughput of the GB300 backend on the 1M-triangle heightfield.

Workload (one "step" = one nearest_hits pass over the whole ray batch, inputs resident
in HBM): 1024 x 512-quad heightfield (1,048,576 triangles), 1920 x 1080 pinhole primary
rays (2,073,600) plus 4,194,304 cosine-hemisphere secondary rays leaving the primary
hits 0.01 above the surface, all five filter tags (32-byte records), 8-wide FP32 nodes.
Inputs are synthetic (seeded generators in portablert_gb300/workloads.py).

Prints one JSON line (driver contract): value = Mrays/s over the timed steps (CUDA
events on the launching stream, L2 flushed between steps), e2e = the same through the
host-buffer C ABI call (rays copied in and records copied out every step), roofline of
the traversal kernel against the measured HBM bandwidth, the CPU baseline (the oracle
port of the reference CPU backend on this host's cores, bounded sample), and the SM
clocks sampled during the timed region.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from portablert_gb300 import hitreg, workloads  # noqa: E402

METRIC = "nearest-hit Mrays/s"
N_SECONDARY = 4_194_304
DELTA = 0.01
TAGS = hitreg.TAGS


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic():
    """DRAM bytes per launch from the committed ncu summary, if one exists."""
    p = os.path.join(ROOT, "profiles", "traverse_heightfield_traffic.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            if line.startswith("dram_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    return None


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int = 0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(prim_hits_fn):
    tris = workloads.heightfield_tris(seed=1)
    prim = workloads.camera_rays()
    h = prim_hits_fn(tris, prim)
    sec = workloads.secondary_rays(tris, prim, h["valid"] != 0, h["primitive_id"],
                                   np.stack([h["px"], h["py"], h["pz"]], 1), N_SECONDARY,
                                   delta=DELTA, seed=1)
    rays = np.ascontiguousarray(np.concatenate([prim, sec]), dtype=np.float32)
    return tris, prim, rays


def workload_config(n_tris, n_prim, n_rays):
    return {"workload": f"heightfield {n_tris:,} tris (1024x512 quads); {n_prim:,} pinhole "
                        f"primary + {n_rays - n_prim:,} cosine secondary rays (offset {DELTA}); "
                        "all five tags (32 B records)",
            "n_tris": n_tris, "n_rays": n_rays, "n_primary": n_prim,
            "tags": list(TAGS), "nodes": "fp32 8-wide", "l2": "flushed between steps (512 MB write)"}


# --------------------------------------------------------------------------- CPU side

def cpu_baseline(tris, rays, sample_rays: int, seed: int = 0):
    """The oracle port of the reference CPU backend on this host: SAH build (1 thread,
    as the reference) and nearest_hits on all online cores over a ray sample."""
    from oracle import cpu as orc

    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(len(rays), size=min(sample_rays, len(rays)), replace=False))
    sample = np.ascontiguousarray(rays[idx])
    t0 = time.perf_counter()
    bvh = orc.BVH(tris)
    build_s = time.perf_counter() - t0
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    bvh.nearest_hits(sample, threads=cores)
    q = time.perf_counter() - t0
    return bvh, {"value": len(sample) / q / 1e6, "unit": "Mrays/s", "cores": cores,
                 "kind": "port", "build_mtris_s": len(tris) / build_s / 1e6,
                 "sample": f"{len(sample):,} rays drawn uniformly from the batch; SAH build of "
                           f"all {len(tris):,} tris on 1 thread ({build_s:.1f} s)"}


def run_reference(args, world, rank):
    """--impl reference: the reference's CPU algorithm (oracle port: the reference's own
    build is x86-only here) timed on this host, bounded sample per step."""
    if rank != 0:
        return
    from oracle import cpu as orc

    orc.build()
    tris = workloads.heightfield_tris(seed=1)
    prim = workloads.camera_rays()
    bvh = orc.BVH(tris)
    ph = bvh.nearest_hits(prim)
    sec = workloads.secondary_rays(tris, prim, ph["valid"] != 0, ph["primitive_id"],
                                   np.stack([ph["px"], ph["py"], ph["pz"]], 1), N_SECONDARY,
                                   delta=DELTA, seed=1)
    rays = np.concatenate([prim, sec])
    cores = os.cpu_count() or 1
    sample_n = 65_536
    rng = np.random.default_rng(0)
    for _ in range(args.warmup):
        bvh.nearest_hits(rays[rng.choice(len(rays), sample_n, replace=False)], threads=cores)
    ts = []
    for _ in range(args.steps):
        s = np.ascontiguousarray(rays[np.sort(rng.choice(len(rays), sample_n, replace=False))])
        t0 = time.perf_counter()
        bvh.nearest_hits(s, threads=cores)
        ts.append(time.perf_counter() - t0)
    total = sum(ts)
    value = sample_n * args.steps / total / 1e6
    out = {"metric": METRIC, "value": value, "unit": "Mrays/s", "impl": "reference",
           "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": workload_config(len(tris), len(prim), len(rays)),
           "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": cores, "kind": "port",
                            "sample": f"{sample_n:,} random rays of the batch per step"},
           "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# --------------------------------------------------------------------------- GPU side

def run_gpu(args, world, rank):
    import torch

    from portablert_gb300.backend import B200Backend

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    b = B200Backend(dev)
    b.init()
    lay = hitreg.layout(TAGS)

    def prim_hits(tris, prim):
        b.set_tris(tris)
        return b.nearest_hits(prim, TAGS)

    tris, prim, rays = make_workload(prim_hits)
    n = len(rays)
    # Build timing (device-only, the scene already resident as input).
    d_tris = torch.from_numpy(tris).cuda()
    build_ms = []
    for _ in range(3):
        b.set_tris_dev(d_tris.data_ptr(), len(tris))
        build_ms.append(b.stat("build_ms"))
    build_dev_ms = float(np.median(build_ms))
    del d_tris
    t0 = time.perf_counter()
    b.set_tris(tris)
    build_e2e_ms = 1e3 * (time.perf_counter() - t0)

    d_rays = torch.from_numpy(rays).cuda()
    d_out = torch.empty(n * lay.size, dtype=torch.uint8, device="cuda")
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    # A dedicated stream: the kernels, the events and the L2 flush all go on it (the
    # legacy default stream has handle 0, which the C ABI reads as "context stream").
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream
    assert sptr != 0

    def step():
        b.nearest_hits_dev(d_rays.data_ptr(), n, d_out.data_ptr(), TAGS, sptr)

    # Visit counts for the algorithmic-byte roofline (a separate counting pass).
    b.set_option("count_visits", 1)
    step()
    b.sync()
    v_nodes, v_tris = b.stat("visits_nodes") / n, b.stat("visits_tris") / n
    b.set_option("count_visits", 0)
    node_size = b.stat("node_size")

    for _ in range(max(3, args.warmup)):
        step()
    b.sync()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    for s, e in ev:
        flush.zero_()
        s.record(stream)
        step()
        e.record(stream)
    torch.cuda.synchronize()
    b.sync()
    clk = clocks.stop()
    ms = [s.elapsed_time(e) for s, e in ev]
    total_ms = float(sum(ms))
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    torch.cuda.synchronize()
    mrays = world * n * args.steps / (total_ms / 1e3) / 1e6

    # End to end through the host-buffer C ABI call (pinned host memory).
    h_rays = torch.from_numpy(rays).pin_memory()
    h_out = torch.empty(n * lay.size, dtype=torch.uint8).pin_memory()
    rec = np.frombuffer(h_out.numpy().data, dtype=lay.numpy_dtype(), count=n)  # view
    L, ctx = b._L, b.ctx
    off = lay.offsets8()

    def e2e_step():
        rc = L.prt_b200_nearest_hits(ctx, h_rays.data_ptr(), n, lay.mask, lay.size, off,
                                     h_out.data_ptr())
        if rc:
            raise RuntimeError(L.prt_b200_last_error(ctx))

    for _ in range(2):
        e2e_step()
    e2e_t = []
    for _ in range(max(1, min(args.steps, 5))):
        t0 = time.perf_counter()
        e2e_step()
        e2e_t.append(time.perf_counter() - t0)
    e2e = n / float(np.median(e2e_t)) / 1e6
    assert rec["valid"].sum() > 0

    # Roofline of the traversal kernel (algorithmic bytes per launch / launch time).
    b_ray = 24 + lay.size + v_nodes * node_size + v_tris * 48
    per_launch_s = total_ms / 1e3 / args.steps
    achieved = n * b_ray / per_launch_s / 1e9
    peak, peak_kind = measured_peaks()
    traffic = committed_traffic()

    # Compressed nodes on the same batch (same hits; checked in the tests).
    b.set_option("node_format", 1)
    for _ in range(3):
        step()
    ev2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    for s, e in ev2:
        flush.zero_()
        s.record(stream)
        step()
        e.record(stream)
    torch.cuda.synchronize()
    b.sync()
    comp_ms = float(sum(s.elapsed_time(e) for s, e in ev2))
    comp_node_size = b.stat("node_size")
    b.set_option("node_format", 0)

    out = {"metric": METRIC, "value": mrays, "unit": "Mrays/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic", "config": workload_config(len(tris), len(prim), n),
           "e2e": {"value": e2e, "unit": "Mrays/s", "h2d_bytes_per_step": 24 * n,
                   "d2h_bytes_per_step": lay.size * n},
           "gpu_launches": args.steps,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "traffic": traffic,
                        "peak_source": peak_kind,
                        "bytes_per_ray": b_ray, "node_visits_per_ray": v_nodes,
                        "tri_tests_per_ray": v_tris, "node_bytes": node_size},
           "build": {"mtris_s_device": len(tris) / build_dev_ms / 1e3,
                     "mtris_s_e2e": len(tris) / build_e2e_ms / 1e3,
                     "ms_device": build_dev_ms, "nodes": b.stat("n_nodes"),
                     "depth": b.stat("depth")},
           "compressed": {"value": world * n * args.steps / (comp_ms / 1e3) / 1e6,
                          "unit": "Mrays/s", "node_bytes": comp_node_size},
           "clocks": clk}
    if rank == 0 and not args.no_cpu:
        _, cb = cpu_baseline(tris, rays, sample_rays=131_072)
        out["cpu_baseline"] = cb
    if rank == 0:
        print(json.dumps(out), flush=True)
    b.shutdown()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="b200", choices=["b200", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, world, rank)
    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    run_gpu(args, world, rank)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
