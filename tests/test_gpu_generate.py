"""Device generators (prt_b200_generate) against the numpy generators in workloads.py.
Values drawn from integers and FP32 arithmetic are bit-identical; values that pass
through log/cos in double may differ where the two math libraries round differently,
which after rounding to FP32 is rare and at most a few ulp."""
import numpy as np
import pytest

from portablert_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _ulps(a, b):
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7FFFFFFF), ia)
    ib = np.where(ib < 0, -(ib & 0x7FFFFFFF), ib)
    return np.abs(ia - ib)


def _gen(backend, kind, seed, n, width, param=0.0):
    import torch

    out = torch.empty(n * width, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    W.generate_dev(backend, kind, seed, n, out.data_ptr(), param)
    backend.sync()
    return out.cpu().numpy().reshape(n, width)


def test_soup_tris_bit_identical(gpu_backend):
    for seed, n in [(0, 4096), (1007, 3), (5, 100_000)]:
        assert np.array_equal(_gen(gpu_backend, W.GEN_SOUP_TRIS, seed, n, 9),
                              W.soup_tris(seed, n))


@pytest.mark.parametrize("kind,fn,width,param", [
    (W.GEN_SOUP_RAYS, lambda s, n: W.soup_rays(s, n), 6, 0.0),
    (W.GEN_RANDOM_RAYS, lambda s, n: W.random_rays(s, n, 12.0), 6, 12.0),
    (W.GEN_CLUSTER_TRIS, lambda s, n: W.cluster_tris(s, n, 256), 9, 256.0),
])
def test_gaussian_generators_match(gpu_backend, kind, fn, width, param):
    for seed, n in [(2, 65_536), (1234, 7)]:
        got = _gen(gpu_backend, kind, seed, n, width, param)
        want = fn(seed, n)
        assert np.isfinite(got).all()
        u = _ulps(got.reshape(-1), want.reshape(-1))
        assert u.max() <= 4, (int(u.max()), int(np.argmax(u)))
        assert (u == 0).mean() >= 0.9999
