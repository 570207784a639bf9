"""Request server: every request's records equal nearest_hits on its scene alone, in
any mix of scenes, sizes and tag sets, with requests arriving from several threads
while others run; admission respects the memory budget."""
import threading
import time

import numpy as np
import pytest

from portablert_gb300 import hitreg, workloads
from portablert_gb300._lib import PrtError

pytestmark = pytest.mark.gpu

COMBOS = hitreg.TAG_COMBOS


def _fields_equal(a, b, lay):
    for f in lay.numpy_dtype().names:
        x, y = a[f], b[f]
        if x.dtype.kind == "f":
            x, y = x.view(np.uint32), y.view(np.uint32)
        if not np.array_equal(x, y):
            return f
    return None


def _server(backend, d_tris, off, persistent=1, **kw):
    """A server in persistent mode (requests folded into one running launch) or wave mode
    (each group of admitted requests one launch on a lane)."""
    from portablert_gb300.serve import Server

    backend.set_option("serve_persistent", persistent)
    try:
        return Server(backend, d_tris.data_ptr(), off, **kw)
    finally:
        backend.set_option("serve_persistent", 1)


def _scenes(torch, sizes, seed):
    tris = [workloads.soup_tris(seed + s, n) for s, n in enumerate(sizes)]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    d = torch.from_numpy(np.concatenate(tris)).cuda()
    torch.cuda.synchronize()
    return tris, off, d


@pytest.mark.parametrize("persistent", [1, 0])
def test_mix_equals_alone(gpu_backend, persistent):
    import torch

    sizes = [16, 300, 5000, 40_000, 1, 2, 120_000, 777]
    tris, off, d_tris = _scenes(torch, sizes, 5000)
    rng = np.random.default_rng(9000)
    reqs = []
    for i in range(60):
        s = int(rng.integers(len(sizes)))
        n = int(np.exp(rng.uniform(np.log(1), np.log(300_000))))
        tags = COMBOS[int(rng.integers(len(COMBOS)))]
        reqs.append((s, workloads.soup_rays(9100 + i, n), tags))
    srv = _server(gpu_backend, d_tris, off, persistent, budget_bytes=64 << 20, lanes=4)
    results = [None] * len(reqs)
    try:
        def client(k):
            for i in range(k, len(reqs), 3):
                s, rays, tags = reqs[i]
                # pinned host buffers, so copies do not hold up the scheduler
                h_r = torch.from_numpy(rays).pin_memory()
                lay = hitreg.layout(tags)
                h_o = torch.zeros(len(rays) * lay.size, dtype=torch.uint8).pin_memory()
                t = srv.submit_ptr(s, h_r.data_ptr(), len(rays), tags, h_o.data_ptr())
                results[i] = (t, h_r, h_o)
                time.sleep(0.0005 * (i % 4))
        th = [threading.Thread(target=client, args=(k,)) for k in range(3)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        lat = [srv.wait(r[0]) for r in results]
        assert all(x >= 0 for x in lat)
        assert srv.stat("completed") == len(reqs)
        assert srv.stat("waves") >= (1 if persistent else 2)
        assert srv.stat("peak_bytes") <= srv.stat("budget_bytes")
        assert srv.stat("bytes_in_use") == 0
    finally:
        srv.close()
    for i, (s, rays, tags) in enumerate(reqs):
        lay = hitreg.layout(tags)
        got = results[i][2].numpy().view(lay.numpy_dtype())
        gpu_backend.set_tris(tris[s])
        want = gpu_backend.nearest_hits(rays, tags)
        bad = _fields_equal(got, want, lay)
        assert bad is None, (i, s, len(rays), tags, bad)


@pytest.mark.parametrize("persistent", [1, 0])
@pytest.mark.parametrize("host_direct", [1, 0])
def test_budget_admission_and_limits(gpu_backend, host_direct, persistent):
    """host_direct 1: records go straight to the host buffers and only rays take budget;
    0: records are staged in the budget region too and copied out.  At most two requests
    are admitted at once, in waves or in the running launch."""
    import torch

    tris, off, d_tris = _scenes(torch, [2000, 3000], 5100)
    tags = ("t", "primitive_id", "valid")
    lay = hitreg.layout(tags)
    n = 20_000  # 480,000 B of rays (+ 320,000 B of records when staged) per request
    per = ((24 * n + 255) // 256) * 256 + (0 if host_direct else lay.size * n)
    budget = 2 * per + 1000  # two requests fit at once, not three
    gpu_backend.set_option("host_direct", host_direct)
    try:
        srv = _server(gpu_backend, d_tris, off, persistent, budget_bytes=budget, lanes=4)
    finally:
        gpu_backend.set_option("host_direct", 1)
    try:
        subs = [srv.submit(i % 2, workloads.soup_rays(5200 + i, n), tags) for i in range(9)]
        for t, _ in subs:
            srv.wait(t)
        assert srv.stat("peak_bytes") <= budget
        if persistent:
            assert srv.stat("max_in_flight_waves") <= 2  # requests admitted at once
        else:
            assert srv.stat("waves") >= 5  # at most two requests per wave
            assert srv.stat("max_wave_requests") <= 2
        for i, (_, out) in enumerate(subs):
            gpu_backend.set_tris(tris[i % 2])
            want = gpu_backend.nearest_hits(workloads.soup_rays(5200 + i, n), tags)
            assert _fields_equal(out, want, lay) is None
        with pytest.raises(PrtError):  # can never fit
            srv.submit(0, workloads.soup_rays(1, 3 * n), tags)
        with pytest.raises(PrtError):
            srv.submit(7, workloads.soup_rays(1, 10), tags)  # no such scene
        t, out = srv.submit(1, np.zeros((0, 6), np.float32), tags)  # empty request
        assert srv.wait(t) >= 0 and len(out) == 0
        with pytest.raises(PrtError):
            srv.wait(123456789)
    finally:
        srv.close()


@pytest.mark.parametrize("leaf,fmt,per_warp,persistent",
                         [(1, 0, 1, 0), (8, 0, 2, 0), (4, 1, 2, 0), (8, 1, 0, 0), (1, 1, 3, 0),
                          (1, 0, 1, 1), (8, 0, 1, 1), (4, 1, 1, 1), (1, 1, 1, 1)])
def test_wave_kernels_equal_alone(gpu_backend, leaf, fmt, per_warp, persistent):
    """Every traversal variant a server can run -- leaf sizes, node formats, wave warps
    bounded to 1-3 batches of 32 rays or unbounded (0), and the running launch of
    persistent mode -- gives each request the records of nearest_hits on its scene
    alone."""
    import torch

    sizes = [3000, 50_000, 7, 200_000]
    tris, off, d_tris = _scenes(torch, sizes, 5800 + leaf)
    tags = hitreg.TAGS
    lay = hitreg.layout(tags)
    try:
        gpu_backend.set_option("leaf_size", leaf)
        gpu_backend.set_option("node_format", fmt)
        gpu_backend.set_option("serve_batches_per_warp", per_warp)
        srv = _server(gpu_backend, d_tris, off, persistent, budget_bytes=128 << 20, lanes=3)
        try:
            reqs = [(i % len(sizes), workloads.soup_rays(5900 + i, [33, 70_000, 1, 9_999][i % 4]))
                    for i in range(12)]
            subs = [srv.submit(s, r, tags) for s, r in reqs]
            for t, _ in subs:
                assert srv.wait(t) >= 0
        finally:
            srv.close()
        for (s, r), (_, out) in zip(reqs, subs):
            gpu_backend.set_tris(tris[s])
            bad = _fields_equal(out, gpu_backend.nearest_hits(r, tags), lay)
            assert bad is None, (s, len(r), bad)
    finally:
        gpu_backend.set_option("leaf_size", 1)
        gpu_backend.set_option("node_format", 0)
        gpu_backend.set_option("serve_batches_per_warp", 1)


def test_requests_finish_alone_not_with_their_wave(gpu_backend):
    """Wave mode, one lane, so requests queued behind a running wave share the next one:
    the wave runs its small requests first and each finishes when its own rays are
    stored, not when the 1.5M-ray request on the dense scene is done."""
    import torch

    tris, off, d_tris = _scenes(torch, [300_000, 2_000], 6100)
    # Records go to the host buffers in place, so a request takes only its rays' bytes
    # of the budget: 19.2 MB for the first, 36 MB for the large one, under 1 MB for the
    # small ones.  With 40 MB the first runs alone (the large one does not fit beside it
    # and the small ones queue behind the large one), and the next wave takes the rest.
    srv = _server(gpu_backend, d_tris, off, 0, budget_bytes=40 << 20, lanes=1)
    tags = ("t", "primitive_id", "valid")
    lay = hitreg.layout(tags)
    try:
        big_rays = workloads.soup_rays(6201, 1_500_000)
        small = [(i % 2, workloads.soup_rays(6300 + i, 2_000 + 131 * i)) for i in range(8)]
        blocker = srv.submit(0, workloads.soup_rays(6200, 800_000), tags)
        big = srv.submit(0, big_rays, tags)
        subs = [srv.submit(s, r, tags) for s, r in small]
        srv.wait(blocker[0])
        lat = [srv.wait(t) for t, _ in subs]
        big_lat = srv.wait(big[0])
        assert srv.stat("max_wave_requests") >= 1 + len(small)
        assert max(lat) < big_lat, (lat, big_lat)
        for (s, r), (_, out) in zip(small, subs):
            gpu_backend.set_tris(tris[s])
            assert _fields_equal(out, gpu_backend.nearest_hits(r, tags), lay) is None
        gpu_backend.set_tris(tris[0])
        assert _fields_equal(big[1], gpu_backend.nearest_hits(big_rays, tags), lay) is None
    finally:
        srv.close()


@pytest.mark.parametrize("persistent", [1, 0])
def test_close_with_requests_queued(gpu_backend, persistent):
    import torch

    _, off, d_tris = _scenes(torch, [50_000], 5300)
    srv = _server(gpu_backend, d_tris, off, persistent, budget_bytes=32 << 20, lanes=2)
    keep = [srv.submit(0, workloads.soup_rays(5400 + i, 100_000), ("valid",)) for i in range(6)]
    srv.close()  # answers or fails every queued request, joins its threads
    assert keep


@pytest.mark.parametrize("persistent", [1, 0])
def test_small_requests_take_the_express_lane(gpu_backend, persistent):
    """Small requests queued behind a large one on a dense scene go to the express lane
    (wave mode: lane 0, highest priority) or the express queue (persistent mode: warps
    take its batches first), finish before the large one and still equal their answers
    alone."""
    import torch

    tris, off, d_tris = _scenes(torch, [300_000, 2_000], 5500)
    srv = _server(gpu_backend, d_tris, off, persistent, budget_bytes=256 << 20, lanes=3)
    tags = ("t", "primitive_id", "valid")
    lay = hitreg.layout(tags)
    try:
        big = srv.submit(0, workloads.soup_rays(5600, 1_500_000), tags)
        small = [(i % 2, workloads.soup_rays(5700 + i, 5_000 + 97 * i)) for i in range(12)]
        subs = [srv.submit(s, r, tags) for s, r in small]
        lat = [srv.wait(t) for t, _ in subs]
        big_lat = srv.wait(big[0])
        assert srv.stat("express_waves") >= 1
        assert min(lat) <= big_lat
        for (s, r), (_, out) in zip(small, subs):
            gpu_backend.set_tris(tris[s])
            assert _fields_equal(out, gpu_backend.nearest_hits(r, tags), lay) is None
    finally:
        srv.close()


def test_running_launch_stops_when_idle_and_starts_again(gpu_backend):
    """Persistent mode: the running launch ends after 5 ms without work and the next
    request starts another; answers stay equal to nearest_hits alone."""
    import torch

    tris, off, d_tris = _scenes(torch, [20_000], 6500)
    srv = _server(gpu_backend, d_tris, off, 1, budget_bytes=64 << 20, lanes=1)
    tags = hitreg.TAGS
    lay = hitreg.layout(tags)
    try:
        outs = []
        for k in range(3):
            rays = workloads.soup_rays(6600 + k, 50_000)
            t, out = srv.submit(0, rays, tags)
            srv.wait(t)
            outs.append((rays, out))
            time.sleep(0.05)  # long enough for the launch to stop
        assert srv.stat("waves") >= 3  # one launch per burst
        gpu_backend.set_tris(tris[0])
        for rays, out in outs:
            assert _fields_equal(out, gpu_backend.nearest_hits(rays, tags), lay) is None
    finally:
        srv.close()


def test_fault_fails_unfinished_requests_then_serves(gpu_backend):
    """Persistent mode, failure injected on the host (option fail_serve_after): the third
    request is published as if one of its batches had faulted (it never completes) and
    the fault flag rises.  The server stops its launch once the other published work is
    done (their answers stay right), fails the third request with PRT_ERR_DEVICE, resets
    its queues and then serves again."""
    import torch

    tris, off, d_tris = _scenes(torch, [300_000, 3_000], 6700)
    gpu_backend.set_option("fail_serve_after", 3)
    try:
        srv = _server(gpu_backend, d_tris, off, 1, budget_bytes=256 << 20, lanes=1)
    finally:
        gpu_backend.set_option("fail_serve_after", 0)
    tags = ("t", "primitive_id", "valid")
    lay = hitreg.layout(tags)
    try:
        reqs = [(0, workloads.soup_rays(6800 + i, 400_000)) for i in range(6)]
        subs = [srv.submit(s, r, tags) for s, r in reqs]
        codes = []
        for t, _ in subs:
            try:
                srv.wait(t)
                codes.append(0)
            except PrtError as e:
                codes.append(e.code)
        assert codes == [0, 0, 5, 0, 0, 0], codes  # PRT_ERR_DEVICE for the third
        gpu_backend.set_tris(tris[0])
        for (s, r), (_, out), c in zip(reqs, subs, codes):
            if c == 0:
                assert _fields_equal(out, gpu_backend.nearest_hits(r, tags), lay) is None
        rays = workloads.soup_rays(6900, 20_000)
        t, out = srv.submit(1, rays, tags)
        srv.wait(t)
        gpu_backend.set_tris(tris[1])
        assert _fields_equal(out, gpu_backend.nearest_hits(rays, tags), lay) is None
    finally:
        srv.close()
