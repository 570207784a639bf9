"""The examples' camera built on the device, traversal fused with it, and the headless
Lambert shading: bit-identical to the CPU oracle's restatement of the examples."""
import math

import numpy as np
import pytest

from parity import compare
from portablert_gb300 import gltf, hitreg, obj
from portablert_gb300._lib import Camera

pytestmark = pytest.mark.gpu

TAGS = hitreg.TAGS
F32 = np.float32


def _cameras(w, h):
    """The bunny (form 0), validation (form 1) and sponza (form 2) set-ups."""
    bunny = dict(width=w, height=h, form=0, pos=(0.0, -0.02, -0.3), sensor_size=0.05,
                 sensor_dist=0.05, sensor_z=float(F32(-0.3) + F32(0.05)))
    valid = dict(width=w, height=h, form=1, pos=(0.0, 0.0, -0.5), sensor_size=0.05,
                 sensor_dist=0.05, sensor_z=float(F32(-0.5) + F32(0.05)))
    a = F32(-1.58)
    sponza = dict(width=w, height=h, form=2, pos=(0.3, 0.1, -0.05), sensor_size=0.05,
                  sensor_dist=0.05, cos_a=float(F32(math.cos(a))), sin_a=float(F32(math.sin(a))))
    return [bunny, valid, sponza]


def _ccam(d):
    c = Camera()
    c.width, c.height, c.form = d["width"], d["height"], d["form"]
    c.pos[:] = list(d["pos"])
    c.sensor_size, c.sensor_dist = d["sensor_size"], d.get("sensor_dist", 0.0)
    c.sensor_z, c.cos_a, c.sin_a = d.get("sensor_z", 0.0), d.get("cos_a", 1.0), d.get("sin_a", 0.0)
    return c


def _ocam(oracle_lib, d):
    return oracle_lib.camera_rays(d["width"], d["height"], d["form"], d["pos"], d["sensor_size"],
                                  d.get("sensor_dist", 0.0), d.get("sensor_z", 0.0),
                                  d.get("cos_a", 1.0), d.get("sin_a", 0.0))


def _mesh(tmp_path_factory, **kw):
    v, f = obj.blob_mesh(40, 48, **kw)
    p = tmp_path_factory.mktemp("mesh") / "blob.obj"
    obj.write_obj(str(p), v, f)
    return obj.load_obj(str(p))


@pytest.fixture(scope="module")
def blob(tmp_path_factory):
    """Bunny-sized: the examples' lambert_shade leaves normals of such small triangles
    unnormalised (|N| < 0.001), so its image is black, as the reference's would be."""
    return _mesh(tmp_path_factory)


@pytest.fixture(scope="module")
def big_blob(tmp_path_factory):
    """Radius 1 at z = 3, in front of a camera at the origin: normals are normalised."""
    return _mesh(tmp_path_factory, centre=(0.0, 0.0, 3.0), radius=1.0)


def _front_cameras(w, h):
    plane = dict(width=w, height=h, form=0, pos=(0.0, 0.0, 0.0), sensor_size=0.05,
                 sensor_z=0.05)
    a = F32(0.2)
    rot = dict(width=w, height=h, form=2, pos=(0.0, 0.1, 0.0), sensor_size=0.05,
               sensor_dist=0.05, cos_a=float(F32(math.cos(a))), sin_a=float(F32(math.sin(a))))
    return [plane, rot]


def test_camera_rays_equal_oracle(gpu_backend, oracle_lib):
    import torch

    for d in _cameras(97, 61) + _cameras(256, 256):
        n = d["width"] * d["height"]
        out = torch.empty(n * 6, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        gpu_backend.camera_rays(_ccam(d), out.data_ptr())
        gpu_backend.sync()
        got = out.cpu().numpy().reshape(n, 6)
        want = _ocam(oracle_lib, d)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), d


@pytest.mark.parametrize("scene", ["bunny_sized", "unit_sized"])
def test_fused_camera_traversal_and_shading(gpu_backend, oracle_lib, blob, big_blob, scene):
    import torch

    mesh, cams = (blob, _cameras(320, 200)) if scene == "bunny_sized" else \
        (big_blob, _front_cameras(320, 200))
    gpu_backend.set_tris(mesh)
    bvh = oracle_lib.BVH(mesh)
    lay = hitreg.layout(TAGS)
    for d in cams:
        n = d["width"] * d["height"]
        cam = _ccam(d)
        rec = torch.zeros(n * lay.size, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        gpu_backend.nearest_hits_camera(cam, rec.data_ptr(), TAGS)
        gpu_backend.sync()
        got = rec.cpu().numpy().view(lay.numpy_dtype())
        rays = _ocam(oracle_lib, d)
        want = bvh.nearest_hits(rays)
        assert (want["valid"] != 0).sum() > n // 50, d  # the mesh is in view
        rep = compare(got, want, TAGS, mesh, rays, oracle_lib)
        assert rep["n_bad"] == 0, rep["bad"][:10]
        # Lambert from the fused camera and from a ray buffer: both equal the oracle's
        # shading of the same hits (the GPU's records, so exact ties in t shade alike).
        hits = np.zeros(n, oracle_lib.HIT_DTYPE)
        for f in ("t", "primitive_id", "valid"):
            hits[f] = got[f]
        want_rgba = oracle_lib.lambert(mesh, rays, hits)
        if scene == "unit_sized":
            assert len(np.unique(want_rgba[:, 0])) > 20  # shading varies over the image
        for use_cam in (True, False):
            rgba = torch.zeros(n * 4, dtype=torch.uint8, device="cuda")
            d_rays = torch.from_numpy(rays).cuda()
            torch.cuda.synchronize()
            if use_cam:
                gpu_backend.shade_lambert(rec.data_ptr(), TAGS, rgba.data_ptr(), cam=cam)
            else:
                gpu_backend.shade_lambert(rec.data_ptr(), TAGS, rgba.data_ptr(),
                                          rays_ptr=d_rays.data_ptr(), n=n)
            gpu_backend.sync()
            assert np.array_equal(rgba.cpu().numpy().reshape(n, 4), want_rgba), (d, use_cam)


def test_sponza_setup_on_a_gltf_scene(gpu_backend, oracle_lib, tmp_path):
    """The sponza example's path end to end on a .glb scene: the glTF reader's soup,
    set_tris, the rotating camera (form 2) fused into the traversal, and the Lambert
    image -- records and pixels equal the oracle's on the same soup."""
    import torch

    v, f = obj.blob_mesh(40, 48, centre=(0.0, 0.0, 3.0), radius=1.0)
    p = tmp_path / "scene.glb"
    gltf.write_gltf(str(p), v, f, "u32", "glb")
    mesh = gltf.load_gltf(str(p))
    assert np.array_equal(mesh, v.astype(np.float32)[f].reshape(-1, 9))
    gpu_backend.set_tris(mesh)
    bvh = oracle_lib.BVH(mesh)
    lay = hitreg.layout(TAGS)
    d = _front_cameras(160, 100)[1]
    n = d["width"] * d["height"]
    cam = _ccam(d)
    rec = torch.zeros(n * lay.size, dtype=torch.uint8, device="cuda")
    rgba = torch.zeros(n * 4, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    gpu_backend.nearest_hits_camera(cam, rec.data_ptr(), TAGS)
    gpu_backend.shade_lambert(rec.data_ptr(), TAGS, rgba.data_ptr(), cam=cam)
    gpu_backend.sync()
    got = rec.cpu().numpy().view(lay.numpy_dtype())
    rays = _ocam(oracle_lib, d)
    want = bvh.nearest_hits(rays)
    assert (want["valid"] != 0).sum() > n // 50
    rep = compare(got, want, TAGS, mesh, rays, oracle_lib)
    assert rep["n_bad"] == 0, rep["bad"][:10]
    hits = np.zeros(n, oracle_lib.HIT_DTYPE)
    for k in ("t", "primitive_id", "valid"):
        hits[k] = got[k]
    assert np.array_equal(rgba.cpu().numpy().reshape(n, 4), oracle_lib.lambert(mesh, rays, hits))


def test_camera_arguments_checked(gpu_backend):
    import torch

    from portablert_gb300._lib import PrtError

    gpu_backend.set_tris(np.array([[-1, -1, 0, 1, -1, 0, 0, 1, 0]], np.float32))
    out = torch.zeros(64, dtype=torch.uint8, device="cuda")
    bad = _ccam(dict(width=0, height=4, form=0, pos=(0, 0, -1), sensor_size=0.05))
    with pytest.raises(PrtError):
        gpu_backend.nearest_hits_camera(bad, out.data_ptr(), TAGS)
    bad = _ccam(dict(width=4, height=4, form=7, pos=(0, 0, -1), sensor_size=0.05))
    with pytest.raises(PrtError):
        gpu_backend.camera_rays(bad, out.data_ptr())
    with pytest.raises(PrtError):  # records without primitive_id cannot be shaded
        gpu_backend.shade_lambert(out.data_ptr(), ("t", "valid"), out.data_ptr(),
                                  rays_ptr=out.data_ptr(), n=1)


def test_device_camera_equals_validation_program(gpu_backend):
    """The validation program's 1024 x 1024 rays, built on the device (SHA-256 of all
    of them against the fixture written from the reference's own program)."""
    import hashlib
    import os

    import torch

    from conftest import GOLDEN

    z = np.load(os.path.join(GOLDEN, "camera_validation.npz"))
    d = dict(width=1024, height=1024, form=1, pos=(0.0, 0.0, -0.5), sensor_size=0.05,
             sensor_dist=0.05, sensor_z=float(F32(-0.5) + F32(0.05)))
    out = torch.empty(1024 * 1024 * 6, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    gpu_backend.camera_rays(_ccam(d), out.data_ptr())
    gpu_backend.sync()
    assert hashlib.sha256(out.cpu().numpy().tobytes()).hexdigest() == str(z["sha256"])


def test_bunny_mesh_equals_bunny_program(gpu_backend):
    """The examples' own bunny (tests/golden/bunny.obj) read through the OBJ reader and
    traced by the fused camera traversal at 4096 x 4096: the bunny program's valid mask
    (the program run unmodified on that file) bit for bit."""
    import os

    import torch

    from conftest import GOLDEN
    from portablert_gb300 import obj

    z = np.load(os.path.join(GOLDEN, "bunny_mesh.npz"))
    tris = obj.load_obj(os.path.join(GOLDEN, "bunny.obj"))
    assert tris.shape == (4968, 9)
    gpu_backend.set_tris(tris)
    d = dict(width=4096, height=4096, form=0, pos=(0.0, -0.02, -0.3), sensor_size=0.05,
             sensor_dist=0.05, sensor_z=float(F32(-0.3) + F32(0.05)))
    tags = ("valid",)
    lay = hitreg.layout(tags)
    rec = torch.zeros(4096 * 4096 * lay.size, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    gpu_backend.nearest_hits_camera(_ccam(d), rec.data_ptr(), tags)
    gpu_backend.sync()
    valid = rec.cpu().numpy().view(lay.numpy_dtype())["valid"]
    assert int((valid != 0).sum()) == 2_914_808
    assert np.array_equal(np.packbits(valid != 0), z["mask_bits"])


def test_bunny_setup_equals_bunny_program(gpu_backend):
    """The bunny program's 4096 x 4096 valid mask on the fixture mesh, from the fused
    camera traversal."""
    import os

    import torch

    from conftest import GOLDEN

    z = np.load(os.path.join(GOLDEN, "bunny_blob.npz"))
    gpu_backend.set_tris(z["tris"])
    d = dict(width=4096, height=4096, form=0, pos=(0.0, -0.02, -0.3), sensor_size=0.05,
             sensor_dist=0.05, sensor_z=float(F32(-0.3) + F32(0.05)))
    tags = ("valid",)
    lay = hitreg.layout(tags)
    rec = torch.zeros(4096 * 4096 * lay.size, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    gpu_backend.nearest_hits_camera(_ccam(d), rec.data_ptr(), tags)
    gpu_backend.sync()
    valid = rec.cpu().numpy().view(lay.numpy_dtype())["valid"]
    assert np.array_equal(np.packbits(valid != 0), z["mask_bits"])
