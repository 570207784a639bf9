"""Failure detection without a GPU fault: host-side injection of device allocation
failures (option "fail_alloc_after").  A failure at any allocation of set_tris, of a
host-buffer nearest_hits, of a batch build or of a server's creation returns
PRT_ERR_OOM; the half-built scene is not queried (PRT_ERR_NO_SCENE); the same context
then builds and answers exactly as one that never failed.  The injected failure is a
status returned before anything is launched, so nothing reaches the GPU."""
import numpy as np
import pytest

from portablert_gb300 import backend, batch, hitreg, serve, workloads
from portablert_gb300._lib import PrtError

# A blocked call (the server's creation once deadlocked on the context's lock when an
# allocation failed) ends the run with every thread's stack instead of hanging it.
pytestmark = [pytest.mark.gpu, pytest.mark.timeout(300, method="thread")]

OOM, NO_SCENE = 6, 4


def _fresh():
    b = backend.B200Backend(0)
    b.init()
    return b


class Armed:
    """The k-th device buffer growth inside the block fails; disarmed on exit."""

    def __init__(self, b, k):
        self.b, self.k = b, k

    def __enter__(self):
        self.b.set_option("fail_alloc_after", self.k)

    def __exit__(self, *exc):
        self.b.set_option("fail_alloc_after", 0)


def _attempt(fn):
    """True if fn() succeeded, False if it failed with PRT_ERR_OOM."""
    try:
        fn()
        return True
    except PrtError as e:
        assert e.code == OOM, e
        return False


def test_set_tris_fails_at_each_allocation_then_recovers():
    tris = workloads.soup_tris(61, 3000)
    rays = workloads.soup_rays(62, 4000)
    b = _fresh()
    try:
        b.set_tris(tris)
        want = b.nearest_hits(rays).view(np.uint8)
    finally:
        b.shutdown()
    failed = 0
    for k in range(1, 80):
        b = _fresh()
        try:
            with Armed(b, k):
                ok = _attempt(lambda: b.set_tris(tris))
            if not ok:
                failed += 1
                with pytest.raises(PrtError) as ei:
                    b.nearest_hits(rays)
                assert ei.value.code == NO_SCENE
                b.set_tris(tris)
            assert np.array_equal(b.nearest_hits(rays).view(np.uint8), want), k
        finally:
            b.shutdown()
        if ok:
            break
    assert ok and failed >= 20, failed  # every growth of a build was met once


def test_host_call_staging_fails_then_recovers():
    tris = workloads.soup_tris(63, 2000)
    rays = workloads.soup_rays(64, 100_003)
    ref = _fresh()
    try:
        ref.set_tris(tris)
        want = ref.nearest_hits(rays).view(np.uint8)  # 32-byte records, one per ray
    finally:
        ref.shutdown()
    b = _fresh()
    try:
        b.set_tris(tris)
        # The copy pipeline from the first query on.  A call grows the rays' staging
        # buffer, then the records', when its batch is larger than any before: the first
        # call fails the first growth, the second (twice the rays) the second growth.
        b.set_option("host_direct", 0)
        for k, m in ((1, 50_001), (2, 100_003)):
            with Armed(b, k):
                assert not _attempt(lambda: b.nearest_hits(rays[:m])), k
            got = b.nearest_hits(rays[:m]).view(np.uint8)
            assert np.array_equal(got, want[:32 * m]), k
    finally:
        b.shutdown()


def test_batch_build_fails_at_each_allocation_then_recovers():
    import torch

    tri_list = [workloads.soup_tris(70 + s, 500 + 300 * s) for s in range(3)]
    tri_off = np.cumsum([0] + [len(t) for t in tri_list]).astype(np.uint64)
    d_tris = torch.from_numpy(np.concatenate(tri_list)).cuda()
    rays = workloads.soup_rays(80, 3000)
    d_rays = torch.from_numpy(rays).cuda()
    lay = hitreg.layout(hitreg.TAGS)

    def run(bt):
        outs = [torch.zeros(len(rays) * lay.size, dtype=torch.uint8, device="cuda")
                for _ in range(3)]
        torch.cuda.synchronize()
        qs = [batch.make_query(s, d_rays.data_ptr(), len(rays), outs[s].data_ptr(), hitreg.TAGS)
              for s in range(3)]
        bt.query_dev(qs)
        bt.sync()
        return [o.cpu().numpy() for o in outs]

    b = _fresh()
    try:
        bt = batch.Batch(b)
        bt.set_tris_dev(d_tris.data_ptr(), tri_off)
        want = run(bt)
        bt.close()
        failed = 0
        for k in range(1, 80):
            bt = batch.Batch(b)
            try:
                with Armed(b, k):
                    ok = _attempt(lambda: bt.set_tris_dev(d_tris.data_ptr(), tri_off))
                if not ok:
                    failed += 1
                    with pytest.raises(PrtError) as ei:
                        run(bt)
                    assert ei.value.code == NO_SCENE
                    bt.set_tris_dev(d_tris.data_ptr(), tri_off)
                got = run(bt)
                assert all(np.array_equal(g, w) for g, w in zip(got, want)), k
            finally:
                bt.close()
            if ok:
                break
        assert ok and failed >= 20, failed
    finally:
        b.shutdown()


def test_server_creation_fails_cleanly_then_serves():
    import torch

    tri_list = [workloads.soup_tris(90 + s, 800) for s in range(2)]
    tri_off = np.cumsum([0] + [len(t) for t in tri_list]).astype(np.uint64)
    d_tris = torch.from_numpy(np.concatenate(tri_list)).cuda()
    rays = workloads.soup_rays(95, 2000)
    b = _fresh()
    try:
        failed = 0
        for k in range(1, 120):
            with Armed(b, k):
                try:
                    srv = serve.Server(b, d_tris.data_ptr(), tri_off, 1 << 24, lanes=3)
                except PrtError as e:
                    assert e.code == OOM, e
                    failed += 1
                    continue
            srv.close()
            break
        assert failed >= 20, failed
        srv = serve.Server(b, d_tris.data_ptr(), tri_off, 1 << 24, lanes=3)
        try:
            for s in range(2):
                t, out = srv.submit(s, rays, hitreg.TAGS)
                srv.wait(t)
                ref = _fresh()
                try:
                    ref.set_tris(tri_list[s])
                    assert np.array_equal(out.view(np.uint8),
                                          ref.nearest_hits(rays).view(np.uint8)), s
                finally:
                    ref.shutdown()
        finally:
            srv.close()
    finally:
        b.shutdown()
