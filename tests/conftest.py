import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU and the built CUDA library")


def load_golden(name):
    from oracle.cpu import HIT_DTYPE

    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    out = {k: z[k] for k in z.files}
    out["full"] = out["full"].reshape(-1).view(HIT_DTYPE)
    return out


def load_c0_golden(tris, rays):
    """The reference's records for the small configuration (4,096-triangle soup, 65,536
    rays, seed 0; tags t, primitive_id, uv, valid).  The inputs are regenerated by the
    seeded generator; their SHA-256 must match the one stored with the records."""
    import hashlib

    from oracle.cpu import HIT_DTYPE

    z = np.load(os.path.join(GOLDEN, "c0_soup.npz"))
    assert hashlib.sha256(np.ascontiguousarray(tris).tobytes()).hexdigest() == str(z["tris_sha256"])
    assert hashlib.sha256(np.ascontiguousarray(rays).tobytes()).hexdigest() == str(z["rays_sha256"])
    return {"full": z["full"].reshape(-1).view(HIT_DTYPE), "tags": tuple(z["tags"].tolist())}


GOLDEN_SETS = ("kat", "axis_grid", "inside_soup", "duplicates", "one_tri", "two_tris",
               "zero_tris", "soup_small")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import cpu

    cpu.build()
    return cpu


@pytest.fixture(scope="session")
def gpu_backend():
    """The GB300 backend through the C ABI.  Fails (not skips) when the library or the
    device is missing, so a GPU run can never pass on a fallback."""
    from portablert_gb300 import _lib
    from portablert_gb300.backend import B200Backend

    _lib.load()
    b = B200Backend(0)
    if not b.is_available():
        raise RuntimeError("no compute capability 10.3 device visible")
    b.init()
    yield b
    b.shutdown()
