"""Option overrides from the environment (PRT_B200_<OPTION>): a new context takes them
as if prt_b200_set_option had been called, the answers stay the reference's, and an
out-of-range value fails creation with the option's message.  Each case runs in a child
process so that the environment of the test session is untouched."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT
from portablert_gb300 import workloads

pytestmark = pytest.mark.gpu

CHILD = """
import ctypes, sys
import numpy as np
from portablert_gb300 import _lib, backend, workloads
L = _lib.load()
h = ctypes.c_void_p()
rc = L.prt_b200_create(0, ctypes.byref(h))
if rc:
    print(rc, (L.prt_b200_last_error(None) or b"").decode())
    sys.exit(0)
L.prt_b200_destroy(h)
b = backend.B200Backend(0)
b.init()
b.set_tris(workloads.soup_tris(101, 5000))
hits = b.nearest_hits(workloads.soup_rays(102, 20000))
np.save(sys.argv[1], hits.view(np.uint8))
print(0, int(b.stat("leaf_size")), int(b.stat("build_sah")))
b.shutdown()
"""


def _child(tmp_path, env_extra):
    out = tmp_path / "hits.npy"
    env = dict(os.environ, **env_extra)
    r = subprocess.run([sys.executable, "-c", CHILD, str(out)], capture_output=True, text=True,
                       env=env, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout.split("\n")[0].split(" ", 1), out


def test_environment_overrides_apply(gpu_backend, tmp_path):
    gpu_backend.set_tris(workloads.soup_tris(101, 5000))
    want = gpu_backend.nearest_hits(workloads.soup_rays(102, 20000)).view(np.uint8)
    (rc, rest), out = _child(tmp_path, {"PRT_B200_LEAF_SIZE": "4", "PRT_B200_BUILD_SAH": "0"})
    assert rc == "0", rest
    assert rest.split() == ["4", "0"]  # leaf size 4, an LBVH tree
    assert np.array_equal(np.load(out), want)


def test_out_of_range_environment_override_fails_creation(tmp_path):
    (rc, rest), _ = _child(tmp_path, {"PRT_B200_BLOCK": "33"})
    assert rc == "1" and "block" in rest, (rc, rest)
