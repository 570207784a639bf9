"""OBJ reader (prt_b200_obj_load, host code in the library): reference forms, fans,
negative indices, errors, and the examples' own bunny mesh where the reference tree is
present."""
import os

import numpy as np
import pytest

from oracle.refdir import reference_path
from portablert_gb300 import obj
from portablert_gb300._lib import PrtError

BUNNY = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bunny.obj")
REF_BUNNY = reference_path("examples", "common", "bunny.obj")


def _py_parse(text):
    """Straightforward restatement used as the expectation."""
    verts, tris = [], []
    for ln in text.splitlines():
        p = ln.split()
        if not p:
            continue
        if p[0] == "v":
            with np.errstate(over="ignore"):  # beyond float's range rounds to inf
                verts.append([np.float32(float(x)) for x in p[1:4]])
        elif p[0] == "f":
            idx = []
            for r in p[1:]:
                k = int(r.split("/")[0])
                idx.append(k - 1 if k > 0 else len(verts) + k)
            for k in range(1, len(idx) - 1):
                tris.append(verts[idx[0]] + verts[idx[k]] + verts[idx[k + 1]])
    return np.asarray(tris, np.float32).reshape(-1, 9)


def test_forms_fans_and_negative_indices(tmp_path):
    text = """# comment
mtllib x.mtl
o thing
v 0 0 0
v 1.5 0 0 1.0
v 0 2.25e-1 0
v 1 1 -3.0000001
vt 0.1 0.2
vn 0 0 1
g part
s off
f 1 2 3
f 1/1 2/1 4/1
f 1//1 3//1 4//1
f 1/1/1 2/1/1 4/1/1 3/1/1
f -4 -3 -2
usemtl red
f 2 3 4"""
    p = tmp_path / "m.obj"
    p.write_text(text)
    got = obj.load_obj(str(p))
    want = _py_parse(text)
    assert got.shape == (7, 9)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_round_trip_of_a_generated_mesh(tmp_path):
    v, f = obj.blob_mesh(20, 24)
    p = tmp_path / "blob.obj"
    obj.write_obj(str(p), v, f)
    got = obj.load_obj(str(p))
    assert np.array_equal(got.view(np.uint32), _py_parse(p.read_text()).view(np.uint32))
    assert len(got) == len(f)


@pytest.mark.parametrize("text", ["v 0 0 0\nv 1 0 0\nf 1 2\n", "v 0 0 0\nf 1 2 3\n",
                                  "v 0 0\n", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 0 1 2\n",
                                  "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 x\n"])
def test_errors(tmp_path, text):
    p = tmp_path / "bad.obj"
    p.write_text(text)
    with pytest.raises(PrtError):
        obj.load_obj(str(p))
    with pytest.raises(PrtError):
        obj.load_obj(str(tmp_path / "missing.obj"))


def test_empty_file(tmp_path):
    p = tmp_path / "e.obj"
    p.write_text("# nothing\n")
    assert obj.load_obj(str(p)).shape == (0, 9)


def test_examples_bunny():
    """The examples' own mesh (tests/golden/bunny.obj, a copy of examples/common/bunny.obj)."""
    got = obj.load_obj(BUNNY)
    with open(BUNNY) as f:
        want = _py_parse(f.read())
    assert got.shape == (4968, 9)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.skipif(not os.path.exists(REF_BUNNY), reason="reference examples not present")
def test_bunny_fixture_is_the_examples_mesh():
    with open(BUNNY, "rb") as a, open(REF_BUNNY, "rb") as b:
        assert a.read() == b.read()


def test_number_forms_round_like_python(tmp_path):
    """Signs, exponents, long mantissas (correct rounding to double, then to float),
    values beyond double's range, inf and nan: each coordinate equals Python's float()
    rounded to float32, whatever the process's C locale."""
    nums = ["+1.5", "-2e3", "1E-2", ".5", "5.", "-0", "0.1000000000000000055511151231257827",
            "3.4028235677973366e38", "3.4028236e38", "1.4e-45", "7e-46", "1e400", "-1e400",
            "1e-400", "inf", "-INF", "Infinity", "123456789012345678901234567890",
            "0.333333333333333333333333333333333333333333333", "nan"]
    while len(nums) % 3:
        nums.append("0")
    lines = [f"v {nums[i]} {nums[i + 1]} {nums[i + 2]}" for i in range(0, len(nums), 3)]
    nv = len(lines)
    lines += [f"f {a + 1} {b + 1} {c + 1}" for a, b, c in
              [(k, (k + 1) % nv, (k + 2) % nv) for k in range(nv)]]
    text = "\n".join(lines) + "\n"
    p = tmp_path / "n.obj"
    p.write_text(text)
    got = obj.load_obj(str(p))
    want = _py_parse(text)
    assert got.shape == want.shape
    nan_g, nan_w = np.isnan(got), np.isnan(want)
    assert np.array_equal(nan_g, nan_w)
    assert np.array_equal(got[~nan_g].view(np.uint32), want[~nan_w].view(np.uint32))


@pytest.mark.parametrize("text", ["v 1 2\n3 4 5\nf 1 1 1\n", "v 1 2 +-3\n", "v 1 2 -\n",
                                  "v 1 2 e5\n"])
def test_a_vertex_never_borrows_from_the_next_line_or_a_bad_number(tmp_path, text):
    p = tmp_path / "bad.obj"
    p.write_text(text)
    with pytest.raises(PrtError):
        obj.load_obj(str(p))
