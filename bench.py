"""Nearest-hit throughput of the GB300 backend on the 1M-triangle heightfield.

Workload (one "step" = one nearest_hits pass over the whole ray batch, inputs resident
in HBM): 1024 x 512-quad heightfield (1,048,576 triangles), 1920 x 1080 pinhole primary
rays (2,073,600) plus 4,194,304 cosine-hemisphere secondary rays leaving the primary
hits 0.01 above the surface, all five filter tags (32-byte records), 8-wide FP32 nodes.
Inputs are synthetic (seeded generators in portablert_gb300/workloads.py).

Prints one JSON line (driver contract): value = Mrays/s over the timed steps (CUDA
events on the launching stream, L2 flushed between steps), e2e = the same through the
host-buffer C ABI call (rays read from and records written to host memory within every
timed call), rooflines of the traversal kernel (instruction issue, L2, HBM) with the one
that binds, the build's roofline, parity of every timed ray against the oracle port of
the reference CPU backend (run in the CPU-baseline leg, which also times that port on
this host's cores on a bounded sample), the other configurations' legs, and the SM
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

METRIC = "nearest-hit Mrays/s (plain vs compressed BVH, same hits); build Mtris/s; p99 ms"
N_SECONDARY = workloads.HF_SECONDARY
DELTA = workloads.HF_DELTA
TAGS = hitreg.TAGS


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


PROFILE = os.path.join("profiles", "traverse_heightfield_traffic.txt")


def committed_profile(key: str, text: bool = False):
    """A figure (DRAM bytes, warp instructions per launch, L2 hit rate, the commit it was
    captured at) from the committed ncu summary of the heightfield traversal, if any."""
    p = os.path.join(ROOT, PROFILE)
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            if line.startswith(key + ":"):
                v = line.split(":", 1)[1].strip()
                return v if text else float(v)
    return None


def traversal_rooflines(n, per_launch_s, b_ray, v_nodes, v_tris, node_size, rec_size, peak,
                        peak_kind, l2_peak, sms, sm_mhz):
    """The regular traversal pass against each resource that could bound it; `bound` is
    the one it comes closest to.

    * issue: warp instructions per launch (ncu, committed summary) over the launch time,
      against 4 issue slots per SM per cycle at the median SM clock of the timed region;
    * l2: the node and triangle bytes the traversal requests (visits x 256 B + tests x
      48 B per ray) against the read bandwidth of its own 32-byte loads from an
      L2-resident buffer (prt_b200_probe_read, measured in this run);
    * hbm: DRAM bytes per launch (ncu, committed summary) against the measured HBM peak;
      beside it the per-ray algorithmic bytes (24 B ray + record + node and triangle
      fetches) against the same peak, which exceeds 1 because L2 serves most fetches."""
    traffic = committed_profile("dram_bytes_per_launch")
    inst = committed_profile("warp_instructions_per_launch")
    at = committed_profile("captured_at", text=True)
    src = f"{PROFILE} (ncu, traversal of commit {at})"
    alg = n * b_ray / per_launch_s / 1e9
    fetch = n * (v_nodes * node_size + v_tris * 48) / per_launch_s / 1e9
    res = {
        "issue": {"achieved": inst / per_launch_s / 1e9 if inst else None,
                  "peak": sms * 4 * sm_mhz * 1e6 / 1e9, "unit": "G warp-instructions/s",
                  "warp_instructions_per_ray": inst / n if inst else None,
                  "warp_instructions_per_node_visit": inst / n / v_nodes if inst else None,
                  "source": src, "sm_mhz": sm_mhz, "sms": sms},
        "l2": {"achieved": fetch, "peak": l2_peak, "unit": "GB/s",
               "bytes_per_ray": v_nodes * node_size + v_tris * 48,
               "peak_source": "prt_b200_probe_read: 32-byte loads over a 48 MiB buffer, "
                              "this run"},
        "hbm": {"achieved": traffic / per_launch_s / 1e9 if traffic else None, "peak": peak,
                "unit": "GB/s", "traffic": traffic, "traffic_source": src,
                "peak_source": peak_kind, "l2_hit_rate_pct": committed_profile("l2_hit_rate_pct"),
                "algorithmic": {"achieved": alg, "frac": alg / peak, "bytes_per_ray": b_ray,
                                "node_visits_per_ray": v_nodes, "tri_tests_per_ray": v_tris,
                                "node_bytes": node_size,
                                "io_floor_frac": n * (24 + rec_size) / per_launch_s / 1e9 / peak}},
    }
    for r in res.values():
        r["frac"] = r["achieved"] / r["peak"] if r["achieved"] and r["peak"] else None
    bound = max((k for k in res if res[k]["frac"] is not None), key=lambda k: res[k]["frac"])
    top = res[bound]
    return {"bound": bound, "achieved": top["achieved"], "peak": top["peak"],
            "unit": top["unit"], "frac": top["frac"], "traffic": traffic,
            "traffic_source": src, **res}


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


class NvmlSampler:
    """SM clock and clock-event reasons read through NVML (libnvidia-ml, ctypes; reads
    only) every millisecond while the timed region runs -- nvidia-smi's 50 ms period
    sees one or two samples of a 32 ms region.  Falls back to ClockSampler when NVML
    cannot be loaded."""

    # nvmlClocksEventReason bits (nvml.h)
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, device: int = 0, period_s: float = 0.001):
        self.device, self.period = device, period_s
        self.samples, self.reasons, self.max_mhz = [], 0, None
        self.fallback = None
        self.stop_evt = threading.Event()
        try:
            import ctypes

            L = ctypes.CDLL("libnvidia-ml.so.1")
            if L.nvmlInit_v2() != 0:
                raise OSError("nvmlInit failed")
            h = ctypes.c_void_p()
            if L.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(device), ctypes.byref(h)) != 0:
                raise OSError("no NVML handle")
            fn = getattr(L, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                L.nvmlDeviceGetCurrentClocksThrottleReasons
            self.L, self.h, self.reason_fn, self.ct = L, h, fn, ctypes
            mx = ctypes.c_uint()
            if L.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:  # 1 = NVML_CLOCK_SM
                self.max_mhz = float(mx.value)
        except (OSError, AttributeError):
            self.L = None
            self.fallback = ClockSampler(device)

    def _run(self):
        ct = self.ct
        mhz, r = ct.c_uint(), ct.c_ulonglong()
        while not self.stop_evt.is_set():
            if self.L.nvmlDeviceGetClockInfo(self.h, 1, ct.byref(mhz)) == 0:
                self.samples.append(float(mhz.value))
            if self.reason_fn(self.h, ct.byref(r)) == 0:
                self.reasons |= int(r.value)
            time.sleep(self.period)

    def start(self):
        if self.fallback:
            return self.fallback.start()
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()

    def stop(self):
        if self.fallback:
            return self.fallback.stop()
        self.stop_evt.set()
        self.t.join()
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(self.samples)), "sm_max_mhz": self.max_mhz,
                "sm_min_mhz": float(min(self.samples)),
                "reasons": sorted(n for bit, n in self.REASONS.items() if self.reasons & bit),
                "samples": len(self.samples), "source": "NVML, 1 ms period"}


def make_workload(prim_hits_fn):
    return workloads.heightfield_workload(prim_hits_fn)


def workload_config(n_tris, n_prim, n_rays):
    return {"workload": f"heightfield {n_tris:,} tris (1024x512 quads); {n_prim:,} pinhole "
                        f"primary + {n_rays - n_prim:,} cosine secondary rays (offset {DELTA}); "
                        "all five tags (32 B records)",
            "n_tris": n_tris, "n_rays": n_rays, "n_primary": n_prim,
            "tags": list(TAGS), "nodes": "fp32 8-wide", "l2": "flushed between steps (512 MB write)"}


# --------------------------------------------------------------------------- ranks
#
# N > 1 (torchrun, one process per GPU): every rank runs a full replica -- the scene is
# replicated and each rank traces its own copy of the rays; the only collectives are the
# barrier before the timed region and the maximum of the timed totals after it.


def sync_ranks(world: int) -> None:
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """The largest x over all ranks (the job's time is its slowest rank's)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_mrays(world: int, n_per_rank: int, steps: int, max_total_ms: float) -> float:
    """Whole-job Mrays/s: the rays of all ranks over the slowest rank's time."""
    return world * n_per_rank * steps / (max_total_ms / 1e3) / 1e6


BUILD_BYTES_PER_TRI = 432  # the canonical LBVH pipeline's algorithmic bytes per triangle
NODE_BYTES_WRITTEN = 256 + 96  # each 8-wide node in FP32 and in compressed form


def build_roofline(n_tris, n_nodes, ms, lbvh_ms, lbvh_nodes, peak, peak_kind):
    """The build against HBM bandwidth: algorithmic bytes = 432 B per triangle (scene
    bounds, Morton codes, four radix passes, hierarchy, refit, collapse, re-layout) plus
    the 8-wide nodes written in both formats, over the device-timed build."""
    def one(nodes, t_ms):
        byt = BUILD_BYTES_PER_TRI * n_tris + NODE_BYTES_WRITTEN * nodes
        ach = byt / (t_ms / 1e3) / 1e9
        return {"bytes": byt, "bytes_per_tri": byt / n_tris, "ms": t_ms, "achieved": ach,
                "frac": ach / peak}
    r = {"bound": "hbm", "unit": "GB/s", "peak": peak, "peak_source": peak_kind}
    r.update(one(n_nodes, ms))
    r["lbvh"] = one(lbvh_nodes, lbvh_ms)
    return r


# --------------------------------------------------------------------------- CPU side

def cpu_baseline(tris, rays, sample_rays: int, seed: int = 0, got=None, tags=TAGS):
    """The oracle port of the reference CPU backend on this host: SAH build (1 thread,
    as the reference) and nearest_hits on all online cores over a ray sample.

    With `got` (the GPU's records of the whole batch) the oracle then answers every ray
    of the batch (untimed) and the parity rules (oracle/parity.py) are applied to all of
    them: the third value returned is that report."""
    from oracle import cpu as orc
    from oracle import parity

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
    rep = None
    if got is not None:
        t0 = time.perf_counter()
        want = bvh.nearest_hits(rays, threads=cores)
        rep = parity.check(got, want, tags, tris, rays, orc, threads=cores)
        rep["checked_against"] = ("oracle port of the reference CPU backend (pinned bit for "
                                  "bit to the reference's golden records), every ray")
        rep["check_s"] = time.perf_counter() - t0
    return bvh, {"value": len(sample) / q / 1e6, "unit": "Mrays/s", "cores": cores,
                 "kind": "port", "build_mtris_s": len(tris) / build_s / 1e6,
                 "sample": f"{len(sample):,} rays drawn uniformly from the batch; SAH build of "
                           f"all {len(tris):,} tris on 1 thread ({build_s:.1f} s)"}, rep


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


# --------------------------------------------------------------------------- other configs

C0_TAGS = ("uv", "t", "primitive_id", "valid")


def _events(torch, stream, fn, reps):
    ms = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    return ms


def leg_small(b, stream, steps):
    """The small configuration: 4,096-triangle soup (seed 0), 65,536 rays, tags
    uv/t/primitive_id/valid.  At this size a call is bound by launch and copy latency:
    the device time of one query and one build (CUDA events), and the host-buffer call
    timed on the host clock."""
    import torch

    tris, rays = workloads.soup(0, 4096, 65536)
    n = len(rays)
    lay = hitreg.layout(C0_TAGS)
    d_t = torch.from_numpy(tris).cuda()
    d_r = torch.from_numpy(rays).cuda()
    d_o = torch.empty(n * lay.size, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    bms = []
    for _ in range(max(3, steps)):
        b.set_tris_dev(d_t.data_ptr(), len(tris))
        bms.append(b.stat("build_ms"))
    q = lambda: b.nearest_hits_dev(d_r.data_ptr(), n, d_o.data_ptr(), C0_TAGS, stream.cuda_stream)
    for _ in range(3):
        q()
    b.sync()
    ms = float(np.median(_events(torch, stream, q, max(10, steps))))
    b.sync()
    for _ in range(3):
        b.nearest_hits(rays, C0_TAGS)
    ts = []
    for _ in range(max(10, steps)):
        t0 = time.perf_counter()
        b.nearest_hits(rays, C0_TAGS)
        ts.append(time.perf_counter() - t0)
    e2e_ms = 1e3 * float(np.median(ts))
    return {"workload": "soup 4,096 tris (seed 0), 65,536 rays; tags uv, t, primitive_id, valid",
            "query_ms": ms, "mrays_s": n / ms / 1e3, "build_ms": float(np.median(bms)),
            "build_mtris_s": len(tris) / float(np.median(bms)) / 1e3,
            "e2e_ms": e2e_ms, "e2e_mrays_s": n / e2e_ms / 1e3}


def leg_batch(b, stream, steps, n_scenes=4096, log=None):
    """4,096 soup scenes (triangles log-uniform in [16, 65536], rays log-uniform in
    [64, 262144], seeds 1000+s, tags uv/t/primitive_id/valid) built and queried as one
    CUDA graph with the autotuned knobs and compressed nodes, beside the same batch
    with FP32 nodes and the plain per-scene path (set_tris + nearest_hits per scene,
    FP32).  Inputs (1.2 GB triangles, 3.2 GB rays) exceed L2, so no flush is needed."""
    import torch

    from portablert_gb300 import autotune, _lib
    from portablert_gb300.batch import Batch, make_query

    tri_n, ray_n = workloads.batch_sizes(n_scenes, seed=3)
    toff = np.concatenate([[0], np.cumsum(tri_n)]).astype(np.uint64)
    roff = np.concatenate([[0], np.cumsum(ray_n)]).astype(np.int64)
    T, R = int(toff[-1]), int(roff[-1])
    lay = hitreg.layout(C0_TAGS)
    d_tris = torch.empty(T * 9, dtype=torch.float32, device="cuda")
    d_rays = torch.empty(R * 6, dtype=torch.float32, device="cuda")
    d_out = torch.zeros(R * lay.size, dtype=torch.uint8, device="cuda")
    d_plain = torch.zeros(R * lay.size, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    tp, rp, op = d_tris.data_ptr(), d_rays.data_ptr(), d_out.data_ptr()
    for s in range(n_scenes):
        workloads.generate_dev(b, workloads.GEN_SOUP_TRIS, 1000 + s, int(tri_n[s]),
                               tp + 36 * int(toff[s]))
        workloads.generate_dev(b, workloads.GEN_SOUP_RAYS, 1000 + s, int(ray_n[s]),
                               rp + 24 * int(roff[s]))
    b.sync()
    qs = [make_query(s, rp + 24 * int(roff[s]), int(ray_n[s]), op + lay.size * int(roff[s]),
                     C0_TAGS) for s in range(n_scenes)]
    qarr = (_lib.Query * n_scenes)(*qs)
    res = {"workload": f"{n_scenes} soup scenes, {T:,} tris, {R:,} rays (log-uniform sizes); "
                       "tags uv, t, primitive_id, valid (20 B records)",
           "n_scenes": n_scenes, "n_tris": T, "n_rays": R}
    out = {}
    for name, fmts in (("compressed", (1,)), ("fp32", (0,))):
        tuned = autotune.tune_batch(b, tp, toff, qarr, stream=stream, formats=fmts, reps=2,
                                    log=log)
        bt = Batch(b)
        try:
            graph_ms = autotune.time_graph(bt, b, tp, toff, qarr, stream, max(3, steps))
            q_ms = _events(torch, stream, lambda: bt.query_dev(qarr, stream.cuda_stream),
                           max(3, steps))
            bt.sync()
            depth, nodes = bt.stat("depth"), bt.stat("n_nodes")
        finally:
            bt.close()
        g, q = float(np.median(graph_ms)), float(np.median(q_ms))
        out[name] = {"graph_ms": g, "query_ms": q, "build_ms": g - q,
                     "mrays_s_graph": R / g / 1e3, "mrays_s_query": R / q / 1e3,
                     "mtris_s_build": T / max(g - q, 1e-6) / 1e3, "depth": depth,
                     "nodes": nodes, "autotuned": tuned["config"],
                     "autotune_cached": tuned["cached"],
                     "autotune_tried": len(tuned.get("tried", []))}
        if name == "compressed":
            torch.cuda.synchronize()
            batched = d_out.clone()
    # The plain path: one scene at a time through set_tris_dev + nearest_hits_dev (FP32,
    # LBVH trees as the batch builds), timed on the host clock around the whole loop.
    autotune.apply(b, {"node_format": 0, "leaf_size": 1, "block": 128, "pool_depth": 0})
    b.set_option("build_compressed", 1)
    b.set_option("build_sah", 0)
    pp = d_plain.data_ptr()
    t0 = time.perf_counter()
    for s in range(n_scenes):
        b.set_tris_dev(tp + 36 * int(toff[s]), int(tri_n[s]))
        b.nearest_hits_dev(rp + 24 * int(roff[s]), int(ray_n[s]), pp + lay.size * int(roff[s]),
                           C0_TAGS, stream.cuda_stream)
    b.sync()
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    b.set_option("build_sah", 1)
    out["plain_per_scene"] = {"ms": 1e3 * plain_s, "mrays_s": R / plain_s / 1e6,
                              "mtris_s_with_queries": T / plain_s / 1e6}
    res.update(out)
    # Records of the compressed graph and of the FP32 graph against the plain path's.
    res["identical"] = {"compressed_graph_vs_plain": bool(torch.equal(batched, d_plain)),
                        "fp32_graph_vs_plain": bool(torch.equal(d_out, d_plain))}
    res["speedup_vs_plain_per_scene"] = (out["compressed"]["mrays_s_graph"] /
                                         out["plain_per_scene"]["mrays_s"])
    res["speedup_vs_fp32_batched"] = (out["compressed"]["mrays_s_graph"] /
                                      out["fp32"]["mrays_s_graph"])
    del d_tris, d_rays, d_out, d_plain, batched
    torch.cuda.empty_cache()
    return res


def precision_parity(d_t, d_r, d_out, n_t, n_r, lay, k, seed=5):
    """The CPU leg's check of the clustered soup: k rays drawn uniformly from the batch,
    answered by the oracle's exhaustive search over all triangles (the reference's
    answer up to ties and tree-dependent rays, which the parity rules handle) and
    compared with the GPU's records of those rays."""
    from oracle import cpu as orc
    from oracle import parity

    t0 = time.perf_counter()
    idx = np.sort(np.random.default_rng(seed).choice(n_r, size=k, replace=False))
    tris = d_t.cpu().numpy().reshape(n_t, 9)
    rays = np.ascontiguousarray(d_r.cpu().numpy().reshape(n_r, 6)[idx])
    got = d_out.cpu().numpy().view(lay.numpy_dtype()).reshape(-1)[idx]
    cores = os.cpu_count() or 1
    want = orc.brute_force(tris, rays, threads=cores)
    rep = parity.check(got, want, lay.tags, tris, rays, orc, threads=cores)
    rep["checked_against"] = (f"oracle exhaustive search over all {n_t:,} triangles, "
                              f"{k:,} rays drawn uniformly from the batch")
    rep["check_s"] = time.perf_counter() - t0
    return rep


def leg_precision(b, stream, steps, check_rays=0):
    """The clustered soup: 8,388,608 tris in 256 Gaussian clusters, 16,777,216 random
    rays, tags uv/t/primitive_id/valid; FP32 against compressed nodes (records must be
    byte-identical) and the FP64 t error of the answers."""
    import torch

    n_t, n_r = 8_388_608, 16_777_216
    lay = hitreg.layout(C0_TAGS)
    d_t = torch.empty(n_t * 9, dtype=torch.float32, device="cuda")
    d_r = torch.empty(n_r * 6, dtype=torch.float32, device="cuda")
    outs = [torch.zeros(n_r * lay.size, dtype=torch.uint8, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    workloads.generate_dev(b, workloads.GEN_CLUSTER_TRIS, 2, n_t, d_t.data_ptr(), 256)
    workloads.generate_dev(b, workloads.GEN_RANDOM_RAYS, 2, n_r, d_r.data_ptr(), 12.0)
    b.sync()
    bms = []
    for _ in range(3):
        b.set_tris_dev(d_t.data_ptr(), n_t)
        bms.append(b.stat("build_ms"))
    res = {"workload": f"clustered soup {n_t:,} tris (256 clusters), {n_r:,} random rays; "
                       "tags uv, t, primitive_id, valid", "n_tris": n_t, "n_rays": n_r,
           "build_ms": float(np.median(bms)),
           "build_mtris_s": n_t / float(np.median(bms)) / 1e3}
    for fmt, name in ((0, "fp32"), (1, "compressed")):
        b.set_option("node_format", fmt)
        o = outs[fmt]
        step = lambda: b.nearest_hits_dev(d_r.data_ptr(), n_r, o.data_ptr(), C0_TAGS,
                                          stream.cuda_stream)
        for _ in range(2):
            step()
        b.sync()
        ms = _events(torch, stream, step, max(3, steps))
        b.sync()
        res[name] = {"mrays_s": n_r / float(np.median(ms)) / 1e3, "ms": float(np.median(ms)),
                     "node_bytes": b.stat("node_size")}
    b.set_option("node_format", 0)
    res["identical"] = bool(torch.equal(outs[0], outs[1]))
    sc = b.t_error(d_t.data_ptr(), n_t, d_r.data_ptr(), n_r, outs[0].data_ptr(), C0_TAGS)
    res["t_error_vs_fp64"] = sc
    res["compressed_over_fp32"] = res["compressed"]["mrays_s"] / res["fp32"]["mrays_s"]
    if check_rays:
        res["parity"] = precision_parity(d_t, d_r, outs[0], n_t, n_r, lay, check_rays)
    del d_t, d_r, outs
    torch.cuda.empty_cache()
    return res


SIZE_CLASSES = (("rays<=64Ki", 0, 65_536), ("64Ki<rays<=512Ki", 65_536, 524_288),
                ("rays>512Ki", 524_288, 1 << 40))


def latency_by_size(lat, nrays):
    """p50 / p99 latency (ms) of the requests in each size class."""
    out = {}
    for name, lo, hi in SIZE_CLASSES:
        m = (nrays > lo) & (nrays <= hi)
        if m.any():
            out[name] = {"n": int(m.sum()), "p50_ms": float(np.percentile(lat[m], 50)),
                         "p99_ms": float(np.percentile(lat[m], 99)),
                         "max_ms": float(lat[m].max())}
    return out


def leg_serving(b, stream, loads=(0.3, 0.6, 0.9), n_req=600, log=None, lanes=4, persistent=1):
    """64 resident soup scenes (sizes log-uniform in [16, 1,048,576], seeds 5000+s) and
    a request stream (seed 9000): scene uniform, rays log-uniform in [1,024, 1,048,576],
    tags uniform over the 31 combinations; Poisson arrivals at fractions of the measured
    capacity.  Latency = submit to records in (pinned) host memory, from the server's
    own clock; the memory budget for request buffers is 2 GiB.  persistent=1 (the
    default): requests are folded into one running launch; 0: waves on `lanes` lanes."""
    import threading

    import torch

    from portablert_gb300.serve import Server

    n_sc = 64
    sizes = workloads.log_uniform_int(workloads.Stream(5000, 11), 16, 1_048_576, n_sc)
    toff = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    T = int(toff[-1])
    d_tris = torch.empty(T * 9, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    for s_ in range(n_sc):
        workloads.generate_dev(b, workloads.GEN_SOUP_TRIS, 5000 + s_, int(sizes[s_]),
                               d_tris.data_ptr() + 36 * int(toff[s_]))
    pool_n = 2 * 1_048_576
    d_pool = torch.empty(pool_n * 6, dtype=torch.float32, device="cuda")
    workloads.generate_dev(b, workloads.GEN_SOUP_RAYS, 9001, pool_n, d_pool.data_ptr())
    b.sync()
    h_pool = d_pool.cpu().pin_memory()
    del d_pool
    slots = 32
    h_out = torch.empty(slots * 1_048_576 * 32, dtype=torch.uint8).pin_memory()
    rs = workloads.Stream(9000, 1)
    total = n_req * (1 + len(loads))
    scene = np.minimum((rs.u01((total,)) * n_sc).astype(np.int64), n_sc - 1)
    nray = workloads.log_uniform_int(rs, 1024, 1_048_576, total)
    combo = np.minimum((rs.u01((total,)) * 31).astype(np.int64), 30)
    start = (rs.u01((total,)) * (pool_n - 1_048_576)).astype(np.int64)

    def run(idx, rate):
        """Submits requests idx at Poisson times of `rate` per second (0 = at once,
        bounded only by the 32 output slots); returns latencies and the span."""
        lat = [0.0] * len(idx)
        free = [threading.Event() for _ in range(slots)]
        for e in free:
            e.set()
        tickets = [None] * len(idx)
        ready = [threading.Event() for _ in idx]

        def waiter():
            for j in range(len(idx)):
                ready[j].wait()
                lat[j] = srv.wait(tickets[j])
                free[j % slots].set()

        th = threading.Thread(target=waiter)
        th.start()
        gaps = -np.log(1.0 - np.random.default_rng(9002).random(len(idx))) / rate if rate else None
        t0 = time.perf_counter()
        due = t0
        for j, i in enumerate(idx):
            if rate:
                due += gaps[j]
                while time.perf_counter() < due:
                    pass
            free[j % slots].wait()
            free[j % slots].clear()
            tags = hitreg.TAG_COMBOS[int(combo[i])]
            n = int(nray[i])
            tickets[j] = srv.submit_ptr(int(scene[i]), h_pool.data_ptr() + 24 * int(start[i]), n,
                                        tags, h_out.data_ptr() + (j % slots) * 1_048_576 * 32)
            ready[j].set()
        th.join()
        span = time.perf_counter() - t0
        return np.array(lat), span

    res = {"workload": f"{n_sc} resident soup scenes ({T:,} tris); requests of 1,024 to "
                       "1,048,576 rays (log-uniform), uniform scene and tag set; Poisson "
                       "arrivals", "n_scenes": n_sc, "n_tris": T, "budget_bytes": 2 << 30,
           "mode": ("persistent: requests folded into one running launch, three queues by "
                    "size" if persistent else f"waves on {lanes} lanes"),
           "lanes": lanes}
    b.set_option("serve_persistent", persistent)
    # Leaf size of the resident scenes, chosen by capacity on the first requests (the
    # largest, densest scenes take most of the GPU time and favour larger leaves).
    trial = {}
    for leaf in (1, 4, 8):
        b.set_option("leaf_size", leaf)
        srv = Server(b, d_tris.data_ptr(), toff, budget_bytes=2 << 30, lanes=lanes)
        try:
            run(list(range(40)), 0)
            _, span = run(list(range(200)), 0)
            trial[leaf] = float(nray[:200].sum()) / span / 1e6
        finally:
            srv.close()
    best_leaf = max(trial, key=trial.get)
    res["leaf_size"] = {"chosen": best_leaf, "trial_mrays_s": trial}
    b.set_option("leaf_size", best_leaf)
    srv = Server(b, d_tris.data_ptr(), toff, budget_bytes=2 << 30, lanes=lanes)
    b.set_option("leaf_size", 1)
    try:
        idx = list(range(n_req))
        run(idx[:50], 0)  # warm-up
        lat, span = run(idx, 0)
        rays = float(nray[idx].sum())
        cap_mrays = rays / span / 1e6
        cap_rps = n_req / span
        res["capacity"] = {"mrays_s": cap_mrays, "requests_s": cap_rps,
                           "p50_ms": float(np.percentile(lat, 50)),
                           "p99_ms": float(np.percentile(lat, 99)),
                           "by_size": latency_by_size(lat, nray[idx])}
        res["loads"] = []
        for k, f in enumerate(loads):
            idx = list(range(n_req * (k + 1), n_req * (k + 2)))
            w0 = srv.stat("waves")
            lat, span = run(idx, f * cap_rps)
            rays = float(nray[idx].sum())
            res["loads"].append({"offered_fraction": f, "offered_requests_s": f * cap_rps,
                                 "mrays_s": rays / span / 1e6,
                                 "p50_ms": float(np.percentile(lat, 50)),
                                 "p99_ms": float(np.percentile(lat, 99)),
                                 "max_ms": float(lat.max()),
                                 "by_size": latency_by_size(lat, nray[idx]),
                                 "waves": srv.stat("waves") - w0})
            if log:
                log(f"serving load {f}: {res['loads'][-1]}")
        # Work per ray on the largest scene (counting pass, 65,536 rays of the pool).
        big = int(np.argmax(sizes))
        b.set_tris_dev(d_tris.data_ptr() + 36 * int(toff[big]), int(sizes[big]))
        b.set_option("count_visits", 1)
        b.nearest_hits(h_pool.numpy().reshape(-1, 6)[:65536], ("valid",))
        res["largest_scene"] = {"n_tris": int(sizes[big]), "leaf_size": 1,
                                "node_visits_per_ray": b.stat("visits_nodes") / 65536,
                                "tri_tests_per_ray": b.stat("visits_tris") / 65536}
        b.set_option("count_visits", 0)
        res["max_in_flight_waves"] = srv.stat("max_in_flight_waves")
        res["max_wave_requests"] = srv.stat("max_wave_requests")
        res["peak_bytes"] = srv.stat("peak_bytes")
    finally:
        srv.close()
    del d_tris, h_out, h_pool
    torch.cuda.empty_cache()
    return res


BUNNY_OBJ = os.path.join(ROOT, "tests", "golden", "bunny.obj")


def leg_camera(b, stream, steps, size=4096, log=None):
    """The examples' bunny set-up (4096 x 4096 pinhole sensor rays from (0, -0.02, -0.3),
    sensor 0.05 wide at 0.05) on the examples' own bunny mesh (tests/golden/bunny.obj,
    4,968 triangles) read through the OBJ reader: rays built inside the traversal (no ray
    buffer) against the same rays from a buffer, the Lambert shading pass, and a frame
    rendered to pinned host memory (camera -> hits -> RGBA8 -> host).  The valid mask is
    compared with the one the bunny program writes (tests/golden/bunny_mesh.npz).  At
    this scale the examples' Lambert leaves normals unnormalised (|N| < 0.001) and the
    image is black, as the reference's would be; the cost is the same."""
    import torch

    from portablert_gb300 import obj
    from portablert_gb300._lib import Camera

    tris = obj.load_obj(BUNNY_OBJ)
    b.set_tris(tris)
    cam = Camera()
    cam.width = cam.height = size
    cam.form = 0
    cam.pos[:] = [0.0, -0.02, -0.3]
    cam.sensor_size, cam.sensor_dist = 0.05, 0.05
    cam.sensor_z = float(np.float32(-0.3) + np.float32(0.05))
    n = size * size
    tags = ("t", "primitive_id", "valid")
    lay = hitreg.layout(tags)
    rec = torch.empty(n * lay.size, dtype=torch.uint8, device="cuda")
    rays = torch.empty(n * 6, dtype=torch.float32, device="cuda")
    rgba = torch.empty(n * 4, dtype=torch.uint8, device="cuda")
    h_rgba = torch.empty(n * 4, dtype=torch.uint8).pin_memory()
    sp = stream.cuda_stream
    torch.cuda.synchronize()
    b.camera_rays(cam, rays.data_ptr(), sp)
    fused = lambda: b.nearest_hits_camera(cam, rec.data_ptr(), tags, sp)
    buffered = lambda: b.nearest_hits_dev(rays.data_ptr(), n, rec.data_ptr(), tags, sp)
    shade = lambda: b.shade_lambert(rec.data_ptr(), tags, rgba.data_ptr(), cam=cam, stream=sp)

    def frame():  # all on `stream`, which is torch's current stream here
        fused()
        shade()
        h_rgba.copy_(rgba, non_blocking=True)

    res = {"workload": f"the examples' bunny ({len(tris):,} tris, OBJ), {size}x{size} pinhole "
                       "sensor rays of the examples' bunny set-up; tags t, primitive_id, valid",
           "n_tris": len(tris), "n_rays": n}
    for name, fn in (("fused_camera", fused), ("ray_buffer", buffered), ("shade", shade)):
        for _ in range(3):
            fn()
        b.sync()
        ms = float(np.median(_events(torch, stream, fn, max(3, steps))))
        b.sync()
        res[name] = {"ms": ms, "mrays_s": n / ms / 1e3}
    for _ in range(2):
        frame()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    k = max(3, min(steps, 10))
    for _ in range(k):
        frame()
    torch.cuda.synchronize()
    fms = 1e3 * (time.perf_counter() - t0) / k
    res["frame_to_host"] = {"ms": fms, "fps": 1e3 / fms, "mrays_s": n / fms / 1e3,
                            "d2h_bytes": 4 * n}
    fused()
    torch.cuda.synchronize()
    recs = rec.cpu().numpy().view(lay.numpy_dtype())
    res["hit_pixels"] = int((recs["valid"] != 0).sum())
    if size == 4096:
        z = np.load(os.path.join(ROOT, "tests", "golden", "bunny_mesh.npz"))
        res["mask_equals_bunny_program"] = bool(
            np.array_equal(np.packbits(recs["valid"] != 0), z["mask_bits"]))
    del rec, rays, rgba, h_rgba
    torch.cuda.empty_cache()
    return res


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
    sah_used = b.stat("build_sah")
    # The LBVH build of the same scene (option build_sah = 0), for comparison.
    b.set_option("build_sah", 0)
    lbvh_ms = []
    for _ in range(3):
        b.set_tris_dev(d_tris.data_ptr(), len(tris))
        lbvh_ms.append(b.stat("build_ms"))
    lbvh_nodes = b.stat("n_nodes")
    b.set_option("build_sah", 1)
    lbvh_ms = float(np.median(lbvh_ms))
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
    sync_ranks(world)
    torch.cuda.synchronize()
    clocks = NvmlSampler(dev)
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
    # The records of the timed steps: checked against the oracle (every ray, CPU leg),
    # against the host-buffer call and against compressed nodes below.
    fp32_out = d_out.clone()
    total_ms = max_over_ranks(float(sum(ms)), world)
    torch.cuda.synchronize()
    mrays = aggregate_mrays(world, n, args.steps, total_ms)

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
    in_place = b.stat("in_place") == 1.0
    assert rec["valid"].sum() > 0
    got_host = fp32_out.cpu()
    e2e_identical = bool(torch.equal(h_out, got_host))

    def timed(f, k):
        f()
        ts = []
        for _ in range(k):
            t0 = time.perf_counter()
            f()
            ts.append(time.perf_counter() - t0)
        return n / float(np.median(ts)) / 1e6

    # The same call through the chunked copy pipeline (option host_direct = 0).
    b.set_option("host_direct", 0)
    e2e_copy = timed(e2e_step, max(1, min(args.steps, 5)))
    b.set_option("host_direct", 1)
    # The same call on pageable memory (what portableRT's std::vector API passes).
    pg_out = np.zeros(n * lay.size, np.uint8)

    def e2e_pageable_step():
        rc = L.prt_b200_nearest_hits(ctx, rays.ctypes.data, n, lay.mask, lay.size, off,
                                     pg_out.ctypes.data)
        if rc:
            raise RuntimeError(L.prt_b200_last_error(ctx))

    e2e_pageable = timed(e2e_pageable_step, max(1, min(args.steps, 5)))
    pg_in_place = b.stat("in_place") == 1.0
    b.set_option("host_direct", 0)
    e2e_pageable_copy = timed(e2e_pageable_step, max(1, min(args.steps, 5)))
    b.set_option("host_direct", 1)

    # Rooflines of the traversal kernel: issue, L2 and HBM (traversal_rooflines).
    b_ray = 24 + lay.size + v_nodes * node_size + v_tris * 48
    per_launch_s = total_ms / 1e3 / args.steps
    peak, peak_kind = measured_peaks()
    probe = torch.empty(48 << 20, dtype=torch.uint8, device="cuda")
    probe.random_(0, 256)
    torch.cuda.synchronize()
    l2_peak = max(b.probe_read_gbs(probe.data_ptr(), probe.numel(), 50) for _ in range(3))
    del probe
    sm_mhz = clk["sm_mhz"] or 2070.0
    roof = traversal_rooflines(n, per_launch_s, b_ray, v_nodes, v_tris, node_size, lay.size,
                               peak, peak_kind, l2_peak, b.stat("sms"), sm_mhz)

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
    comp_identical = bool(torch.equal(d_out, fp32_out))
    del fp32_out
    b.set_option("node_format", 0)

    # Coherent and incoherent rays apart (the primary rays, the offset secondary rays),
    # and the literal secondary rays (offset 0: they start on the surface they leave, and
    # under the reference's semantics nearly all hit it again at t ~ 0).
    def time_range(ptr, count, k=10):
        for _ in range(3):
            b.nearest_hits_dev(ptr, count, d_out.data_ptr(), TAGS, sptr)
        b.sync()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(k)]
        for s, e in evs:
            flush.zero_()
            s.record(stream)
            b.nearest_hits_dev(ptr, count, d_out.data_ptr(), TAGS, sptr)
            e.record(stream)
        torch.cuda.synchronize()
        return count / (sum(s.elapsed_time(e) for s, e in evs) / k) / 1e3

    n_prim = len(prim)
    coherence = {"primary": {"n": n_prim, "mrays_s": time_range(d_rays.data_ptr(), n_prim)},
                 "secondary_offset": {"n": n - n_prim, "delta": DELTA,
                                      "mrays_s": time_range(d_rays.data_ptr() + 24 * n_prim,
                                                            n - n_prim)}}
    if rank == 0:
        hp = b.nearest_hits(prim, TAGS)
        lit = workloads.secondary_rays(tris, prim, hp["valid"] != 0, hp["primitive_id"],
                                       np.stack([hp["px"], hp["py"], hp["pz"]], 1),
                                       N_SECONDARY, delta=0.0, seed=1)
        d_lit = torch.from_numpy(np.ascontiguousarray(lit, dtype=np.float32)).cuda()
        torch.cuda.synchronize()
        coherence["secondary_literal"] = {"n": len(lit), "delta": 0.0,
                                          "mrays_s": time_range(d_lit.data_ptr(), len(lit))}
        del d_lit

    out = {"metric": METRIC, "value": mrays, "unit": "Mrays/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic",
           "config": dict(workload_config(len(tris), len(prim), n),
                          knobs={"leaf_size": int(b.stat("leaf_size")), "block_threads": 128,
                                 "width": 8, "node_format": "fp32",
                                 "build": "binned SAH, 8-wide collapse by least cost"}),
           "e2e": {"value": e2e, "unit": "Mrays/s", "h2d_bytes_per_step": 24 * n,
                   "d2h_bytes_per_step": lay.size * n, "host_memory": "pinned",
                   "path": ("in place: the traversal reads each ray from and writes each "
                            "record to the caller's host buffers over the host link")
                   if in_place else "chunked copy pipeline",
                   "copy_pipeline_value": e2e_copy,
                   "pageable_value": e2e_pageable,
                   "pageable_path": "in place" if pg_in_place else "chunked copy pipeline",
                   "pageable_copy_pipeline_value": e2e_pageable_copy,
                   "records_identical_to_device_run": e2e_identical},
           # per step: the regular pass and the deferred pass of k_trace8
           "gpu_launches": 2 * args.steps,
           "roofline": roof,
           "build": {"roofline": build_roofline(len(tris), b.stat("n_nodes"), build_dev_ms,
                                                lbvh_ms, lbvh_nodes, peak, peak_kind),
                     "mtris_s_device": len(tris) / build_dev_ms / 1e3,
                     "mtris_s_e2e": len(tris) / build_e2e_ms / 1e3,
                     "ms_device": build_dev_ms, "nodes": b.stat("n_nodes"),
                     "depth": b.stat("depth"),
                     "method": "binned SAH" if sah_used else "LBVH (SAH fell back)",
                     "lbvh": {"ms_device": lbvh_ms, "mtris_s_device": len(tris) / lbvh_ms / 1e3,
                              "nodes": lbvh_nodes}},
           "compressed": {"value": world * n * args.steps / (comp_ms / 1e3) / 1e6,
                          "unit": "Mrays/s", "node_bytes": comp_node_size,
                          "records_identical_to_fp32": comp_identical},
           "coherence": coherence,
           "clocks": clk}
    del d_rays, d_out, flush
    torch.cuda.empty_cache()
    # The other configurations are measured on rank 0 only (replicas would repeat them).
    legs = set(args.legs.split(",")) if args.legs and rank == 0 else set()
    log = (lambda m: print(m, file=sys.stderr, flush=True)) if args.verbose else None
    if "small" in legs:
        out["small"] = leg_small(b, stream, min(args.steps, 20))
    if "precision" in legs:
        out["precision"] = leg_precision(b, stream, min(args.steps, 10),
                                         check_rays=0 if args.no_cpu else 512)
    if "batch" in legs:
        out["batch"] = leg_batch(b, stream, min(args.steps, 10), log=log)
    if "serving" in legs:
        out["serving"] = leg_serving(b, stream, log=log)
    if "camera" in legs:
        out["camera"] = leg_camera(b, stream, min(args.steps, 10), log=log)
    if rank == 0 and not args.no_cpu:
        got = got_host.numpy().view(lay.numpy_dtype()).reshape(-1)
        _, cb, rep = cpu_baseline(tris, rays, sample_rays=131_072, got=got)
        out["cpu_baseline"] = cb
        out["parity"] = rep
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
    ap.add_argument("--legs", default="small,precision,batch,serving,camera",
                    help="other configurations to measure: small, precision, batch, serving, "
                         "camera "
                         "(comma list; 'none' for the heightfield alone)")
    ap.add_argument("--verbose", action="store_true")
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
