"""Writes the fixtures that pin the examples' camera (and, for the bunny set-up, the
whole pipeline) against portableRT's own example programs.

Runs the reference's examples/validation and examples/bunny programs, compiled
unmodified by `make -C oracle examples` (oracle/stubs/ stands in for tinyobjloader and
stb), on a generated bunny-sized mesh:

* camera_validation.npz: the validation program's 1,048,576 rays -- the SHA-256 of their
  bytes and every 1021st ray;
* bunny_blob.npz: the mesh's triangles (as read through the OBJ reader) and the valid
  mask the bunny program writes for its 4096 x 4096 camera, bit-packed, with its SHA-256;
* bunny.obj: the examples' own mesh (examples/common/bunny.obj, 4,968 triangles), copied
  as test data, and bunny_mesh.npz: the valid mask the bunny program writes for it (the
  program run unmodified on that file), bit-packed, with the SHA-256 of mask and file.

    python tests/golden/make_examples_golden.py      (needs the reference tree)
"""
import hashlib
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.refdir import reference_path  # noqa: E402
from portablert_gb300 import obj  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref")


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "examples"], check=True)
    with tempfile.TemporaryDirectory() as td:
        mesh = os.path.join(td, "blob.obj")
        v, f = obj.blob_mesh(60, 84)
        obj.write_obj(mesh, v, f)
        tris = obj.load_obj(mesh)
        env = dict(os.environ, PRT_STUB_OBJ=mesh)
        rays_path = os.path.join(td, "rays.bin")
        subprocess.run([os.path.join(REF_BIN, "validation_example"), rays_path], env=env,
                       cwd=td, check=True, stdout=subprocess.DEVNULL)
        rays = np.fromfile(rays_path, np.float32).reshape(-1, 6)
        mask_path = os.path.join(td, "mask.bin")
        env["PRT_STUB_IMAGE"] = mask_path
        subprocess.run([os.path.join(REF_BIN, "bunny_example")], env=env, cwd=td, check=True,
                       input=b"0\n", stdout=subprocess.DEVNULL)
        mask = np.fromfile(mask_path, np.uint8)
    bunny_src = reference_path("examples", "common", "bunny.obj")
    bunny_dst = os.path.join(HERE, "bunny.obj")
    shutil.copyfile(bunny_src, bunny_dst)
    with tempfile.TemporaryDirectory() as td:
        env = dict(os.environ, PRT_STUB_OBJ=bunny_dst,
                   PRT_STUB_IMAGE=os.path.join(td, "mask.bin"))
        subprocess.run([os.path.join(REF_BIN, "bunny_example")], env=env, cwd=td, check=True,
                       input=b"0\n", stdout=subprocess.DEVNULL)
        bmask = np.fromfile(os.path.join(td, "mask.bin"), np.uint8)
    with open(bunny_dst, "rb") as f:
        obj_sha = hashlib.sha256(f.read()).hexdigest()
    np.savez_compressed(os.path.join(HERE, "bunny_mesh.npz"),
                        mask_bits=np.packbits(bmask != 0), n=len(bmask),
                        sha256=hashlib.sha256(bmask.tobytes()).hexdigest(), obj_sha256=obj_sha)
    print(f"bunny.obj: mask {len(bmask)} ({int((bmask != 0).sum())} lit)")
    idx = np.arange(0, len(rays), 1021)
    np.savez_compressed(os.path.join(HERE, "camera_validation.npz"),
                        sha256=hashlib.sha256(rays.tobytes()).hexdigest(), n=len(rays),
                        idx=idx, rays=rays[idx])
    np.savez_compressed(os.path.join(HERE, "bunny_blob.npz"), tris=tris,
                        mask_bits=np.packbits(mask != 0), n=len(mask),
                        sha256=hashlib.sha256(mask.tobytes()).hexdigest())
    print(f"validation rays {len(rays)}, bunny mask {len(mask)} ({int((mask != 0).sum())} lit)")


if __name__ == "__main__":
    main()
