"""The examples' camera and the bunny set-up pinned against portableRT's own example
programs (fixtures written by tests/golden/make_examples_golden.py from the reference's
examples/validation and examples/bunny, compiled unmodified)."""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
from oracle.refdir import reference_path

F32 = np.float32
REF_EXAMPLES = os.path.join(ROOT, "oracle", "_ref")


def validation_camera(oracle_lib):
    return oracle_lib.camera_rays(1024, 1024, 1, (0.0, 0.0, -0.5), 0.05, 0.05,
                                  float(F32(-0.5) + F32(0.05)))


def bunny_camera_args():
    return (4096, 4096, 0, (0.0, -0.02, -0.3), 0.05, 0.05, float(F32(-0.3) + F32(0.05)))


def test_oracle_camera_equals_validation_program(oracle_lib):
    z = np.load(os.path.join(GOLDEN, "camera_validation.npz"))
    rays = validation_camera(oracle_lib)
    assert len(rays) == int(z["n"])
    assert np.array_equal(rays[z["idx"]].view(np.uint32), z["rays"].view(np.uint32))
    assert hashlib.sha256(rays.tobytes()).hexdigest() == str(z["sha256"])


def test_oracle_equals_bunny_program(oracle_lib):
    z = np.load(os.path.join(GOLDEN, "bunny_blob.npz"))
    rays = oracle_lib.camera_rays(*bunny_camera_args())
    hits = oracle_lib.BVH(z["tris"]).nearest_hits(rays)
    mask = np.where(hits["valid"] != 0, 255, 0).astype(np.uint8)
    assert np.array_equal(np.packbits(mask != 0), z["mask_bits"])
    assert hashlib.sha256(mask.tobytes()).hexdigest() == str(z["sha256"])


def test_oracle_equals_bunny_program_on_the_bunny(oracle_lib):
    """The examples' own bunny mesh (tests/golden/bunny.obj) through the OBJ reader, the
    oracle's camera and traversal: the bunny program's valid mask bit for bit."""
    from portablert_gb300 import obj

    z = np.load(os.path.join(GOLDEN, "bunny_mesh.npz"))
    path = os.path.join(GOLDEN, "bunny.obj")
    with open(path, "rb") as f:
        assert hashlib.sha256(f.read()).hexdigest() == str(z["obj_sha256"])
    tris = obj.load_obj(path)
    rays = oracle_lib.camera_rays(*bunny_camera_args())
    hits = oracle_lib.BVH(tris).nearest_hits(rays)
    mask = np.where(hits["valid"] != 0, 255, 0).astype(np.uint8)
    assert np.array_equal(np.packbits(mask != 0), z["mask_bits"])
    assert hashlib.sha256(mask.tobytes()).hexdigest() == str(z["sha256"])


@pytest.mark.skipif(not os.path.isdir(reference_path("examples")),
                    reason="the reference's example sources are not present")
def test_fixtures_match_the_programs_run_now():
    sys.path.insert(0, ROOT)
    from portablert_gb300 import obj

    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "examples"], check=True)
    z = np.load(os.path.join(GOLDEN, "camera_validation.npz"))
    with tempfile.TemporaryDirectory() as td:
        mesh = os.path.join(td, "blob.obj")
        v, f = obj.blob_mesh(60, 84)
        obj.write_obj(mesh, v, f)
        out = os.path.join(td, "rays.bin")
        subprocess.run([os.path.join(REF_EXAMPLES, "validation_example"), out], cwd=td,
                       env=dict(os.environ, PRT_STUB_OBJ=mesh), check=True,
                       stdout=subprocess.DEVNULL)
        rays = np.fromfile(out, np.float32)
    assert hashlib.sha256(rays.tobytes()).hexdigest() == str(z["sha256"])
