"""glTF reader (prt_b200_gltf_load, host code in the library): the sponza example's
extraction (examples/sponza/main.cpp:35-101) on .gltf files with file and data: buffers
and on .glb files; strides, offsets, skipped primitives; errors for everything the
example would read out of bounds for; a JSON parser that takes what the format allows
and refuses the rest; mutated files that must fail cleanly, never crash."""
import base64
import json
import struct

import numpy as np
import pytest

from portablert_gb300 import gltf, obj
from portablert_gb300._lib import PrtError

IDX = {5121: ("<B", 1), 5123: ("<H", 2), 5125: ("<I", 4)}


def _expected(doc, buffers):
    """The example's loop restated in Python (honouring byteStride, which the example
    only meets as absent or 12): every mesh, every TRIANGLES primitive with POSITION and
    indices, triangles of consecutive index triples."""
    out = []
    for mesh in doc.get("meshes", []):
        for prim in mesh.get("primitives", []):
            if prim.get("mode", 4) != 4:
                continue
            if "POSITION" not in prim.get("attributes", {}) or "indices" not in prim:
                continue

            def view(acc_i, elem):
                a = doc["accessors"][acc_i]
                if "bufferView" not in a:
                    return None, 0, a["count"]
                v = doc["bufferViews"][a["bufferView"]]
                data = buffers[v["buffer"]]
                start = v.get("byteOffset", 0) + a.get("byteOffset", 0)
                return (data, start, v.get("byteStride", elem)), 1, a["count"]

            (pv, has_p, n_p) = view(prim["attributes"]["POSITION"], 12)
            ia = doc["accessors"][prim["indices"]]
            fmt, size = IDX[ia["componentType"]]
            (iv, has_i, n_i) = view(prim["indices"], size)
            for t in range(n_i // 3):
                tri = []
                for k in range(3):
                    j = 3 * t + k
                    idx = struct.unpack_from(fmt, iv[0], iv[1] + iv[2] * j)[0] if has_i else 0
                    assert idx < n_p
                    if has_p:
                        tri += struct.unpack_from("<3f", pv[0], pv[1] + pv[2] * idx)
                    else:
                        tri += [0.0, 0.0, 0.0]
                out.append(tri)
    return np.asarray(out, np.float32).reshape(-1, 9)


def _same(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("buffer", ["file", "embed", "glb"])
@pytest.mark.parametrize("index_type", ["u8", "u16", "u32"])
def test_round_trip_of_the_writer(tmp_path, buffer, index_type):
    v, f = obj.blob_mesh(10, 12)  # 110 vertices: fits u8 indices
    p = tmp_path / ("m.glb" if buffer == "glb" else "m.gltf")
    gltf.write_gltf(str(p), v, f, index_type, buffer)
    got = gltf.load_gltf(str(p))
    want = v.astype(np.float32)[f].reshape(-1, 9)
    assert _same(got, want)


def _rich_document(tmp_path):
    """Two meshes, two buffers (a file with an escaped name and a data: URI), and every
    rule of the loop: interleaved positions (byteStride 24), accessor and view offsets,
    u8/u16/u32 indices, a trailing index pair that makes no triangle, a LINES primitive,
    a primitive without indices, one without POSITION, an accessor without a view."""
    rng = np.random.default_rng(7)
    pos = rng.normal(size=(40, 3)).astype(np.float32)
    nrm = rng.normal(size=(40, 3)).astype(np.float32)
    inter = np.concatenate([pos, nrm], 1).tobytes()  # 24-byte stride
    packed = pos[10:].tobytes()
    i16 = rng.integers(0, 40, 14).astype(np.uint16).tobytes() + b"\0\0"  # 14 = 4 tris + 2
    i8 = rng.integers(0, 30, 9).astype(np.uint8).tobytes() + b"\0" * 3
    i32 = rng.integers(0, 30, 12).astype(np.uint32).tobytes()
    b0 = b"\xAB" * 8 + inter + i16       # 8 bytes of padding before the first view
    b1 = packed + i8 + i32 + bytes([2, 0, 1, 0])
    (tmp_path / "my mesh.bin").write_bytes(b0)
    o_i16 = 8 + len(inter)
    o_i8, o_i32 = len(packed), len(packed) + len(i8)
    doc = {
        "asset": {"version": "2.0"},
        "buffers": [{"uri": "my%20mesh.bin", "byteLength": len(b0)},
                    {"uri": "data:application/gltf-buffer;base64," +
                     base64.b64encode(b1).decode(), "byteLength": len(b1)}],
        "bufferViews": [
            {"buffer": 0, "byteOffset": 8, "byteLength": len(inter), "byteStride": 24},
            {"buffer": 0, "byteOffset": o_i16, "byteLength": 28},
            {"buffer": 1, "byteOffset": 0, "byteLength": len(packed)},
            {"buffer": 1, "byteOffset": o_i8, "byteLength": 9},
            {"buffer": 1, "byteOffset": o_i32, "byteLength": len(i32)},
            {"buffer": 1, "byteOffset": o_i32 + len(i32), "byteLength": 3},
        ],
        "accessors": [
            {"bufferView": 0, "componentType": 5126, "count": 40, "type": "VEC3"},
            {"bufferView": 1, "componentType": 5123, "count": 14, "type": "SCALAR"},
            {"bufferView": 2, "byteOffset": 12, "componentType": 5126, "count": 29,
             "type": "VEC3"},
            {"bufferView": 3, "componentType": 5121, "count": 9, "type": "SCALAR"},
            {"bufferView": 4, "byteOffset": 4, "componentType": 5125, "count": 9,
             "type": "SCALAR"},
            {"componentType": 5126, "count": 3, "type": "VEC3"},
            {"bufferView": 5, "componentType": 5121, "count": 3, "type": "SCALAR"},
        ],
        "meshes": [
            {"name": "café 😀", "primitives": [
                {"attributes": {"POSITION": 0, "NORMAL": 0}, "indices": 1},
                {"attributes": {"POSITION": 0}, "indices": 1, "mode": 1},
                {"attributes": {"POSITION": 0}},
                {"attributes": {"NORMAL": 0}, "indices": 1}]},
            {"primitives": [
                {"attributes": {"POSITION": 2}, "indices": 3, "mode": 4},
                {"attributes": {"POSITION": 2}, "indices": 4},
                {"attributes": {"POSITION": 5}, "indices": 6}]},
        ],
        "materials": [{"pbrMetallicRoughness": {"baseColorFactor": ["@TINY@", 0.5, 1E+2, -0.0],
                                                "metallicFactor": "@HUGE@"}}],
        "extensionsUsed": ["KHR_materials_unlit"],
    }
    return doc, [b0, b1]


def _dump(doc, **kw) -> str:
    """JSON text of doc with numbers beyond double's range where the placeholders are
    (only in a field the reader does not use)."""
    return json.dumps(doc, **kw).replace('"@TINY@"', "1e-400").replace('"@HUGE@"', "-1e400")


def test_every_rule_of_the_loop(tmp_path):
    doc, bufs = _rich_document(tmp_path)
    p = tmp_path / "rich.gltf"
    p.write_text(_dump(doc, ensure_ascii=True, indent="\t"))  # \u escapes, surrogate pair
    got = gltf.load_gltf(str(p))
    want = _expected(doc, bufs)
    assert len(want) == 4 + 3 + 3 + 1
    assert _same(got, want)


def test_glb_with_two_buffers(tmp_path):
    """A .glb whose buffer 0 is the BIN chunk and buffer 1 a data: URI."""
    doc, (b0, b1) = _rich_document(tmp_path)
    doc["buffers"][0] = {"byteLength": len(b0)}
    js = _dump(doc, ensure_ascii=False).encode()
    js += b" " * (-len(js) % 4)
    bin_ = b0 + b"\0" * (-len(b0) % 4)
    body = struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(bin_),
                                                                      0x004E4942) + bin_
    p = tmp_path / "two.glb"
    p.write_bytes(struct.pack("<III", 0x46546C67, 2, 12 + len(body)) + body)
    assert _same(gltf.load_gltf(str(p)), _expected(doc, [b0, b1]))


def test_only_buffer_0_of_a_glb_is_its_bin_chunk(tmp_path):
    """A second buffer without a URI does not alias the BIN chunk: it has no bytes, so
    its byteLength is an error."""
    v, f = obj.blob_mesh(6, 8)
    p = tmp_path / "g.glb"
    gltf.write_gltf(str(p), v, f, "u16", "glb")
    data = p.read_bytes()
    js_len = struct.unpack_from("<I", data, 12)[0]
    doc = json.loads(data[20:20 + js_len])
    doc["buffers"].append({"byteLength": 16})
    js = json.dumps(doc).encode()
    js += b" " * (-len(js) % 4)
    rest = data[20 + js_len:]
    body = struct.pack("<II", len(js), 0x4E4F534A) + js + rest
    q = tmp_path / "h.glb"
    q.write_bytes(struct.pack("<III", 0x46546C67, 2, 12 + len(body)) + body)
    with pytest.raises(PrtError, match="buffer 1: shorter than its byteLength"):
        gltf.load_gltf(str(q))


def test_empty_documents(tmp_path):
    for i, doc in enumerate([{"asset": {"version": "2.0"}},
                             {"asset": {"version": "2.0"}, "meshes": []},
                             {"meshes": [{"primitives": []}], "buffers": []}]):
        p = tmp_path / f"e{i}.gltf"
        p.write_text(json.dumps(doc))
        assert gltf.load_gltf(str(p)).shape == (0, 9)


def _small(tmp_path, edit=None, name="s.gltf"):
    """A valid one-triangle document (positions, u16 indices in one data: buffer), with
    `edit(doc)` applied before it is written."""
    blob = struct.pack("<9f", 0, 0, 0, 1, 0, 0, 0, 1, 0) + struct.pack("<3H", 0, 1, 2) + b"\0\0"
    doc = {"asset": {"version": "2.0"},
           "buffers": [{"uri": "data:application/octet-stream;base64," +
                        base64.b64encode(blob).decode(), "byteLength": len(blob)}],
           "bufferViews": [{"buffer": 0, "byteLength": 36}, {"buffer": 0, "byteOffset": 36,
                                                             "byteLength": 6}],
           "accessors": [{"bufferView": 0, "componentType": 5126, "count": 3, "type": "VEC3"},
                         {"bufferView": 1, "componentType": 5123, "count": 3,
                          "type": "SCALAR"}],
           "meshes": [{"primitives": [{"attributes": {"POSITION": 0}, "indices": 1}]}]}
    if edit:
        edit(doc)
    p = tmp_path / name
    p.write_text(json.dumps(doc))
    return p


def test_the_small_document_loads(tmp_path):
    got = gltf.load_gltf(str(_small(tmp_path)))
    assert got.tolist() == [[0, 0, 0, 1, 0, 0, 0, 1, 0]]


def _set(path, value):
    def edit(doc):
        node = doc
        for k in path[:-1]:
            node = node[k]
        node[path[-1]] = value
    return edit


@pytest.mark.parametrize("edit,words", [
    (_set(["accessors", 1, "count"], 6), "past the end of its bufferView"),
    (_set(["accessors", 0, "byteOffset"], 4), "past the end of its bufferView"),
    (_set(["bufferViews", 1, "byteLength"], 40), "past the end of its buffer"),
    (_set(["buffers", 0, "byteLength"], 100), "shorter than its byteLength"),
    (_set(["accessors", 0, "count"], 2), "beyond 2 positions"),
    (_set(["accessors", 0, "componentType"], 5123), "unsupported componentType"),
    (_set(["accessors", 0, "type"], "VEC4"), "type must be VEC3"),
    (_set(["accessors", 1, "componentType"], 5126), "unsupported componentType"),
    (_set(["accessors", 1, "sparse"], {"count": 1}), "sparse"),
    (_set(["accessors", 1, "count"], -3), "non-negative integer"),
    (_set(["accessors", 1, "count"], 1.5), "non-negative integer"),
    (_set(["meshes", 0, "primitives", 0, "indices"], 7), "missing accessor"),
    (_set(["accessors", 0, "bufferView"], 9), "missing bufferView"),
    (_set(["bufferViews", 0, "buffer"], 3), "missing buffer"),
    (_set(["bufferViews", 0, "byteStride"], 8), "byteStride"),
    (_set(["extensionsRequired"], ["KHR_draco_mesh_compression"]), "KHR_draco_mesh_compression"),
    (_set(["buffers", 0, "uri"], "https://example.com/b.bin"), "relative file names"),
    (_set(["buffers", 0, "uri"], "data:application/octet-stream,abc"), "base64"),
    (_set(["buffers", 0, "uri"], "data:application/octet-stream;base64,AB$C"), "bad base64"),
    (_set(["buffers", 0, "uri"], "missing.bin"), "cannot open"),
    (_set(["meshes"], {"a": 1}), "meshes is not an array"),
])
def test_errors_name_the_cause(tmp_path, edit, words):
    p = _small(tmp_path, edit)
    with pytest.raises(PrtError, match=words):
        gltf.load_gltf(str(p))


@pytest.mark.parametrize("text", [
    "", "{", "}", "[1, 2]", '{"a": }', '{"a" 1}', '{"a": 1,}', '{"a": [1 2]}', '{"a": 01}',
    '{"a": 1.}', '{"a": .5}', '{"a": +1}', '{"a": 1e}', '{"a": tru}', '{"a": "x}',
    '{"a": "\\q"}', '{"a": "\\ud800"}', '{"a": "\\udc00"}', '{"a": "\\u12g4"}',
    '{"a": "tab\there"}', '{"a": 1} x', "[" * 100 + "]" * 100, '{"a": NaN}',
])
def test_malformed_json_is_refused(tmp_path, text):
    p = tmp_path / "bad.gltf"
    p.write_text(text)
    with pytest.raises(PrtError):
        gltf.load_gltf(str(p))


def test_json_the_format_allows(tmp_path):
    """White space of every kind, escapes, repeated members (the last one counts),
    unknown members and extensions that are only used: all accepted."""
    p = _small(tmp_path)
    doc = json.loads(p.read_text())
    text = json.dumps(doc, indent=" ").replace("\n", "\r\n")
    text = text.replace('"asset"', '"\\u0061sset"', 1)
    text = text.replace('"meshes"', '"extras": {"k": [true, false, null, -0.0, 1E-3, "\\/\\b\\f\\n\\r\\t\\"\\\\"]}, "meshes"', 1)
    text = text.replace('"indices": 1', '"indices": 0, "indices": 1', 1)
    p.write_text(text)
    assert gltf.load_gltf(str(p)).tolist() == [[0, 0, 0, 1, 0, 0, 0, 1, 0]]


def test_glb_container_errors(tmp_path):
    good = tmp_path / "g.glb"
    v, f = obj.blob_mesh(6, 8)
    gltf.write_gltf(str(good), v, f, "u16", "glb")
    data = good.read_bytes()
    cases = {
        "version": data[:4] + struct.pack("<I", 1) + data[8:],
        "truncated": data[:len(data) - 40],
        "first chunk not JSON": data[:16] + struct.pack("<I", 0x004E4942) + data[20:],
        "header only": data[:12],
    }
    for name, blob in cases.items():
        p = tmp_path / f"{name.replace(' ', '_')}.glb"
        p.write_bytes(blob)
        with pytest.raises(PrtError):
            gltf.load_gltf(str(p))


def test_mutated_files_fail_cleanly(tmp_path):
    """Seeded byte flips and truncations of a valid .glb and .gltf: each call returns a
    soup or raises PrtError, and the process never crashes (the same corpus runs under
    AddressSanitizer in test_mesh_readers_asan.py)."""
    rng = np.random.default_rng(11)
    v, f = obj.blob_mesh(6, 8)
    g = tmp_path / "m.glb"
    gltf.write_gltf(str(g), v, f, "u16", "glb")
    t = _small(tmp_path, name="t.gltf")
    sources = [g.read_bytes(), t.read_bytes()]
    outcomes = {"ok": 0, "error": 0}
    for i in range(400):
        data = bytearray(sources[i % 2])
        if rng.random() < 0.3:
            data = data[:int(rng.integers(0, len(data)))]
        for _ in range(int(rng.integers(1, 6))):
            if data:
                data[int(rng.integers(0, len(data)))] = int(rng.integers(0, 256))
        p = tmp_path / ("x.glb" if i % 2 == 0 else "x.gltf")
        p.write_bytes(bytes(data))
        try:
            gltf.load_gltf(str(p))
            outcomes["ok"] += 1
        except PrtError:
            outcomes["error"] += 1
    assert outcomes["error"] > 0 and sum(outcomes.values()) == 400
