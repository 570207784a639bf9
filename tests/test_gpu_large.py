"""Large scenes: a 33.5M-triangle soup (above 2^25, exercising the wide index paths of
the sort, the collapse and the traversal's 27-bit work items) against the oracle's
exhaustive search on a ray sample, FP32 against compressed nodes, and the size limit."""
import numpy as np
import pytest

from parity import compare
from portablert_gb300 import hitreg, workloads as W
from portablert_gb300._lib import PrtError

pytestmark = pytest.mark.gpu

TAGS = hitreg.TAGS


def test_33m_triangle_soup(gpu_backend, oracle_lib):
    import torch

    n_t, n_r = (1 << 25) + 12345, 4096
    d_t = torch.empty(n_t * 9, dtype=torch.float32, device="cuda")
    d_r = torch.empty(n_r * 6, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    W.generate_dev(gpu_backend, W.GEN_SOUP_TRIS, 7, n_t, d_t.data_ptr())
    W.generate_dev(gpu_backend, W.GEN_SOUP_RAYS, 8, n_r, d_r.data_ptr())
    gpu_backend.sync()
    gpu_backend.set_tris_dev(d_t.data_ptr(), n_t)
    assert gpu_backend.stat("n_tris") == n_t
    lay = hitreg.layout(TAGS)
    outs = []
    for fmt in (0, 1):
        gpu_backend.set_option("node_format", fmt)
        o = torch.zeros(n_r * lay.size, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        gpu_backend.nearest_hits_dev(d_r.data_ptr(), n_r, o.data_ptr(), TAGS)
        gpu_backend.sync()
        outs.append(o)
    gpu_backend.set_option("node_format", 0)
    assert torch.equal(outs[0], outs[1])
    got = outs[0].cpu().numpy().view(lay.numpy_dtype())
    assert (got["valid"] != 0).mean() > 0.5
    # Exhaustive search over all triangles for a sample of the rays.
    tris = d_t.cpu().numpy().reshape(n_t, 9)
    rays = d_r.cpu().numpy().reshape(n_r, 6)
    idx = np.arange(0, n_r, 64)
    want = oracle_lib.brute_force(tris, rays[idx])
    rep = compare(got[idx], want, TAGS, tris, rays[idx], oracle_lib)
    assert rep["n_bad"] == 0, rep["bad"][:10]
    assert int(got["primitive_id"][got["valid"] != 0].max()) > (1 << 24)


def test_size_limit_refused_before_any_work(gpu_backend):
    import torch

    d = torch.zeros(64, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    with pytest.raises(PrtError) as e:
        gpu_backend.set_tris_dev(d.data_ptr(), 1 << 27)  # one more than the limit
    assert e.value.code == 7  # PRT_ERR_LIMIT
