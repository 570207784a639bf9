"""The host-buffer call (prt_b200_nearest_hits) either traverses the caller's buffers in
place (option host_direct, when the device can reach them: pinned memory, and pageable
memory where the device reads the host's page tables) or splits large batches into
chunks whose copies and traversals overlap on several streams.  Its records must be
byte-identical to one device-buffer launch over the same rays, for pageable and pinned
host memory, chunk counts from one to eight, ragged last chunks and every node format."""
import numpy as np
import pytest

from portablert_gb300 import hitreg, workloads

pytestmark = pytest.mark.gpu


def _device_records(torch, backend, rays, tags):
    lay = hitreg.layout(tags)
    d_r = torch.from_numpy(rays).cuda()
    d_o = torch.zeros(len(rays) * lay.size, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    backend.nearest_hits_dev(d_r.data_ptr(), len(rays), d_o.data_ptr(), tags)
    backend.sync()
    return d_o.cpu().numpy()


@pytest.mark.parametrize("n_rays", [(1 << 15) - 1, 8 * (1 << 15) + 1, 5 * (1 << 18) + 77,
                                    2_500_001])
@pytest.mark.parametrize("fmt", [0, 1])
@pytest.mark.parametrize("chunks,ramp", [(8, 1), (3, 0), (16, 1)])
def test_chunked_host_call_equals_device_call(gpu_backend, n_rays, fmt, chunks, ramp):
    import torch

    tris = workloads.soup_tris(41, 20_000)
    rays = workloads.soup_rays(42, n_rays)
    gpu_backend.set_option("node_format", fmt)
    gpu_backend.set_option("pipe_chunks", chunks)
    gpu_backend.set_option("pipe_ramp", ramp)
    gpu_backend.set_option("host_direct", 0)  # the copy pipeline
    try:
        gpu_backend.set_tris(tris)
        for tags in [hitreg.TAGS, ("t", "primitive_id", "valid"), ("valid",)]:
            want = _device_records(torch, gpu_backend, rays, tags)
            got = gpu_backend.nearest_hits(rays, tags).view(np.uint8).reshape(-1)
            assert np.array_equal(got, want), tags
    finally:
        gpu_backend.set_option("node_format", 0)
        gpu_backend.set_option("pipe_chunks", 8)
        gpu_backend.set_option("pipe_ramp", 1)
        gpu_backend.set_option("host_direct", 1)


@pytest.mark.parametrize("rays_mem,out_mem", [("pinned", "pinned"), ("pageable", "pageable"),
                                              ("pinned", "pageable"), ("pageable", "pinned")])
@pytest.mark.parametrize("direct", [1, 0])
def test_host_call_in_place_and_copied(gpu_backend, rays_mem, out_mem, direct):
    """Both forms of the host-buffer call, on every mix of pinned and pageable buffers,
    the output starting at an odd address (byte stores) or aligned."""
    import ctypes

    import torch

    tris = workloads.soup_tris(47, 8_000)
    rays = workloads.soup_rays(48, 300_001)
    gpu_backend.set_tris(tris)
    for tags in [hitreg.TAGS, ("valid",)]:
        lay = hitreg.layout(tags)
        want = _device_records(torch, gpu_backend, rays, tags)
        r = torch.from_numpy(rays).pin_memory() if rays_mem == "pinned" else rays
        r_ptr = r.data_ptr() if rays_mem == "pinned" else rays.ctypes.data
        for shift in (0, 1):
            size = len(rays) * lay.size + 1
            if out_mem == "pinned":
                o = torch.zeros(size, dtype=torch.uint8).pin_memory()
                o_ptr = o.data_ptr() + shift
            else:
                o = np.zeros(size, np.uint8)
                o_ptr = o.ctypes.data + shift
            L = gpu_backend._L
            try:
                gpu_backend.set_option("host_direct", direct)
                gpu_backend._check(L.prt_b200_nearest_hits(
                    gpu_backend.ctx, ctypes.c_void_p(r_ptr), len(rays), lay.mask, lay.size,
                    lay.offsets8(), ctypes.c_void_p(o_ptr)))
            finally:
                gpu_backend.set_option("host_direct", 1)
            got = (o.numpy() if out_mem == "pinned" else o)[shift:shift + len(rays) * lay.size]
            assert np.array_equal(got, want), (tags, shift)


def test_host_call_with_device_buffers_runs_in_place(gpu_backend):
    """Device memory handed to the host-buffer call is traversed where it is."""
    import ctypes

    import torch

    tris = workloads.soup_tris(49, 3_000)
    rays = workloads.soup_rays(50, 70_001)
    gpu_backend.set_tris(tris)
    lay = hitreg.layout(hitreg.TAGS)
    want = _device_records(torch, gpu_backend, rays, hitreg.TAGS)
    d_r = torch.from_numpy(rays).cuda()
    d_o = torch.zeros(len(rays) * lay.size, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    L = gpu_backend._L
    gpu_backend._check(L.prt_b200_nearest_hits(
        gpu_backend.ctx, ctypes.c_void_p(d_r.data_ptr()), len(rays), lay.mask, lay.size,
        lay.offsets8(), ctypes.c_void_p(d_o.data_ptr())))
    assert gpu_backend.stat("in_place") == 1.0
    assert np.array_equal(d_o.cpu().numpy(), want)


@pytest.mark.parametrize("rays_mem", ["pinned", "pageable"])
def test_host_rays_at_a_four_byte_offset_are_copied(gpu_backend, rays_mem):
    """Rays starting 4 bytes past an 8-byte boundary (a float array at an odd index) are
    not traversed in place, since the traversal reads them in 8-byte pairs: the call
    copies them into its aligned staging buffer and gives the same records; the same
    rays 8-byte aligned are traversed in place."""
    import ctypes

    import torch

    tris = workloads.soup_tris(51, 4_000)
    rays = workloads.soup_rays(52, 40_001)
    gpu_backend.set_tris(tris)
    lay = hitreg.layout(hitreg.TAGS)
    want = _device_records(torch, gpu_backend, rays, hitreg.TAGS)
    flat = np.zeros(rays.size + 2, np.float32)
    buf = torch.from_numpy(flat).pin_memory() if rays_mem == "pinned" else flat
    base = buf.data_ptr() if rays_mem == "pinned" else flat.ctypes.data
    assert base % 8 == 0
    host = buf.numpy() if rays_mem == "pinned" else flat
    size = len(rays) * lay.size
    o = torch.zeros(size, dtype=torch.uint8).pin_memory() if rays_mem == "pinned" else \
        np.zeros(size, np.uint8)
    o_ptr = o.data_ptr() if rays_mem == "pinned" else o.ctypes.data
    L = gpu_backend._L
    for k in (1, 2):
        host[:] = 0.0
        host[k:k + rays.size] = rays.reshape(-1)
        o[:] = 0
        gpu_backend._check(L.prt_b200_nearest_hits(
            gpu_backend.ctx, ctypes.c_void_p(base + 4 * k), len(rays), lay.mask, lay.size,
            lay.offsets8(), ctypes.c_void_p(o_ptr)))
        if k == 1:
            assert gpu_backend.stat("in_place") == 0.0, rays_mem
        elif rays_mem == "pinned":  # pageable memory is reachable only on some hosts
            assert gpu_backend.stat("in_place") == 1.0
        got = o.numpy() if rays_mem == "pinned" else o
        assert np.array_equal(got, want), (k, rays_mem)


def test_chunked_host_call_pinned_buffers(gpu_backend):
    import ctypes

    import torch

    tris = workloads.soup_tris(43, 5_000)
    rays = workloads.soup_rays(44, 3 * (1 << 18) + 5)
    gpu_backend.set_tris(tris)
    lay = hitreg.layout(hitreg.TAGS)
    h_r = torch.from_numpy(rays).pin_memory()
    h_o = torch.zeros(len(rays) * lay.size, dtype=torch.uint8).pin_memory()
    L = gpu_backend._L
    gpu_backend.set_option("host_direct", 0)  # the copy pipeline
    try:
        gpu_backend._check(L.prt_b200_nearest_hits(
            gpu_backend.ctx, ctypes.c_void_p(h_r.data_ptr()), len(rays), lay.mask, lay.size,
            lay.offsets8(), ctypes.c_void_p(h_o.data_ptr())))
    finally:
        gpu_backend.set_option("host_direct", 1)
    want = _device_records(torch, gpu_backend, rays, hitreg.TAGS)
    assert np.array_equal(h_o.numpy(), want)


def test_counting_run_is_one_chunk_and_equal(gpu_backend):
    import torch

    tris = workloads.soup_tris(45, 3_000)
    rays = workloads.soup_rays(46, 3 * (1 << 18))
    gpu_backend.set_tris(tris)
    want = _device_records(torch, gpu_backend, rays, hitreg.TAGS)
    gpu_backend.set_option("count_visits", 1)
    try:
        got = gpu_backend.nearest_hits(rays, hitreg.TAGS).view(np.uint8).reshape(-1)
        assert np.array_equal(got, want)
        assert gpu_backend.stat("visits_nodes") >= len(rays)
    finally:
        gpu_backend.set_option("count_visits", 0)


def test_rebuild_waits_for_queries_on_caller_streams(gpu_backend):
    """set_tris_dev right after nearest_hits_dev on a caller's stream (no sync between):
    the rebuild must not overwrite the scene the queued query is reading."""
    import torch

    scenes = [workloads.soup_tris(60 + s, 20_000 + 3_000 * s) for s in range(6)]
    rays = [workloads.soup_rays(70 + s, 400_000) for s in range(6)]
    want = []
    for t, r in zip(scenes, rays):
        gpu_backend.set_tris(t)
        want.append(gpu_backend.nearest_hits(r, hitreg.TAGS).view(np.uint8).reshape(-1))
    lay = hitreg.layout(hitreg.TAGS)
    d_t = [torch.from_numpy(t).cuda() for t in scenes]
    d_r = [torch.from_numpy(r).cuda() for r in rays]
    d_o = [torch.zeros(len(r) * lay.size, dtype=torch.uint8, device="cuda") for r in rays]
    torch.cuda.synchronize()
    st = torch.cuda.Stream()
    for s in range(len(scenes)):
        gpu_backend.set_tris_dev(d_t[s].data_ptr(), len(scenes[s]))
        gpu_backend.nearest_hits_dev(d_r[s].data_ptr(), len(rays[s]), d_o[s].data_ptr(),
                                     hitreg.TAGS, st.cuda_stream)
    gpu_backend.sync()
    for s in range(len(scenes)):
        assert np.array_equal(d_o[s].cpu().numpy(), want[s]), s


def test_queries_on_two_streams_at_once(gpu_backend):
    """Queries queued on two callers' streams may run at the same time: each stream has
    its own ray counter."""
    import torch

    tris = workloads.soup_tris(80, 30_000)
    gpu_backend.set_tris(tris)
    ra, rb = workloads.soup_rays(81, 1_500_000), workloads.soup_rays(82, 900_000)
    wa = gpu_backend.nearest_hits(ra, hitreg.TAGS).view(np.uint8).reshape(-1)
    wb = gpu_backend.nearest_hits(rb, hitreg.TAGS).view(np.uint8).reshape(-1)
    lay = hitreg.layout(hitreg.TAGS)
    da, db = torch.from_numpy(ra).cuda(), torch.from_numpy(rb).cuda()
    oa = torch.zeros(len(ra) * lay.size, dtype=torch.uint8, device="cuda")
    ob = torch.zeros(len(rb) * lay.size, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    for _ in range(3):
        gpu_backend.nearest_hits_dev(da.data_ptr(), len(ra), oa.data_ptr(), hitreg.TAGS,
                                     s1.cuda_stream)
        gpu_backend.nearest_hits_dev(db.data_ptr(), len(rb), ob.data_ptr(), hitreg.TAGS,
                                     s2.cuda_stream)
    gpu_backend.sync()
    assert np.array_equal(oa.cpu().numpy(), wa)
    assert np.array_equal(ob.cpu().numpy(), wb)
