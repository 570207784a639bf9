"""Precision: compressed 8-bit nodes give the FP32 nodes' answers at full size, and the
FP64 t scorer (prt_b200_t_error) agrees with the CPU oracle's double-precision t."""
import numpy as np
import pytest

from portablert_gb300 import hitreg, workloads as W
from portablert_gb300._lib import PrtError

pytestmark = pytest.mark.gpu

TAGS = ("uv", "t", "primitive_id", "valid")


def _run(torch, backend, d_rays, n, tags=TAGS):
    lay = hitreg.layout(tags)
    d_o = torch.zeros(n * lay.size, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    backend.nearest_hits_dev(d_rays.data_ptr(), n, d_o.data_ptr(), tags)
    backend.sync()
    return d_o


def test_t_error_agrees_with_oracle(gpu_backend, oracle_lib):
    import torch

    tris, rays = W.soup(0, 4096, 65536)
    gpu_backend.set_tris(tris)
    d_t = torch.from_numpy(tris).cuda()
    d_r = torch.from_numpy(rays).cuda()
    d_o = _run(torch, gpu_backend, d_r, len(rays))
    got = gpu_backend.t_error(d_t.data_ptr(), len(tris), d_r.data_ptr(), len(rays),
                              d_o.data_ptr(), TAGS)
    rec = d_o.cpu().numpy().view(hitreg.layout(TAGS).numpy_dtype())
    st = oracle_lib.BVH(tris).stats(rays)
    v = rec["valid"] != 0
    assert (st["n_best"][v] == 1).all()  # no ties in this scene: one triangle per hit
    t32 = rec["t"][v].astype(np.float64)
    t64 = st["t64"][v]
    err = np.abs(t32 - t64)
    assert got["scored"] == int(v.sum()) and got["unscored"] == 0
    assert got["max_abs"] == err.max()
    assert got["exact"] == int((rec["t"][v] == t64.astype(np.float32)).sum())
    assert got["mean_abs"] == pytest.approx(err.mean(), rel=1e-9)
    rel = err[t64 != 0] / np.abs(t64[t64 != 0])
    assert got["max_rel"] == rel.max()


def test_t_error_counts_unscorable_and_checks_fields(gpu_backend):
    import torch

    tris, rays = W.soup(3, 100, 1000)
    gpu_backend.set_tris(tris)
    d_t = torch.from_numpy(tris).cuda()
    d_r = torch.from_numpy(rays).cuda()
    d_o = _run(torch, gpu_backend, d_r, len(rays))
    lay = hitreg.layout(TAGS)
    rec = d_o.cpu().numpy().view(lay.numpy_dtype()).copy()
    v = np.flatnonzero(rec["valid"])
    assert len(v) > 10
    rec["primitive_id"][v[:7]] = len(tris) + 5
    d_bad = torch.from_numpy(rec.view(np.uint8).copy()).cuda()
    torch.cuda.synchronize()
    got = gpu_backend.t_error(d_t.data_ptr(), len(tris), d_r.data_ptr(), len(rays),
                              d_bad.data_ptr(), TAGS)
    assert got["unscored"] == 7 and got["scored"] == len(v) - 7
    with pytest.raises(PrtError):
        gpu_backend.t_error(d_t.data_ptr(), len(tris), d_r.data_ptr(), len(rays),
                            d_o.data_ptr(), ("uv", "valid"))


@pytest.mark.parametrize("n_tris,n_rays", [(1 << 20, 1 << 21), (8_388_608, 16_777_216)])
def test_compressed_equals_fp32_clustered(gpu_backend, n_tris, n_rays):
    """The precision workload (clustered soup, random rays) at full size: the compressed
    tree's records are byte-identical to the FP32 tree's."""
    import torch

    d_t = torch.empty(n_tris * 9, dtype=torch.float32, device="cuda")
    d_r = torch.empty(n_rays * 6, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    W.generate_dev(gpu_backend, W.GEN_CLUSTER_TRIS, 2, n_tris, d_t.data_ptr(), 256)
    W.generate_dev(gpu_backend, W.GEN_RANDOM_RAYS, 2, n_rays, d_r.data_ptr(), 12.0)
    gpu_backend.sync()
    gpu_backend.set_tris_dev(d_t.data_ptr(), n_tris)
    a = _run(torch, gpu_backend, d_r, n_rays)
    gpu_backend.set_option("node_format", 1)
    try:
        b = _run(torch, gpu_backend, d_r, n_rays)
    finally:
        gpu_backend.set_option("node_format", 0)
    assert torch.equal(a, b)
    lay = hitreg.layout(TAGS)
    rec = a.view(-1, lay.size)
    assert int(rec[:, lay.off_valid].sum()) > n_rays // 100
    sc = gpu_backend.t_error(d_t.data_ptr(), n_tris, d_r.data_ptr(), n_rays, a.data_ptr(), TAGS)
    assert sc["unscored"] == 0 and sc["scored"] > 0
    assert np.isfinite(sc["max_abs"]) and 0 <= sc["exact"] <= sc["scored"]
