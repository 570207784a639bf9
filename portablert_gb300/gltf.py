"""glTF 2.0 meshes as triangle soups (prt_b200_gltf_load), and a writer of indexed
triangle meshes as .gltf (external or embedded buffer) or .glb files.

The reader follows the sponza example's extraction (examples/sponza/main.cpp:35-101):
every mesh in order, each TRIANGLES primitive with POSITION and indices, triangles of
consecutive index triples, mesh-space positions.
"""
from __future__ import annotations

import base64
import json
import os
import struct

import numpy as np

from .obj import load_soup

_INDEX_TYPES = {"u8": (5121, np.uint8), "u16": (5123, np.uint16), "u32": (5125, np.uint32)}


def load_gltf(path: str) -> np.ndarray:
    """n x 9 float32 triangles of every indexed TRIANGLES primitive, in file order."""
    return load_soup("prt_b200_gltf_load", path)


def _pad4(b: bytes, fill: bytes = b"\0") -> bytes:
    return b + fill * (-len(b) % 4)


def write_gltf(path: str, vertices: np.ndarray, faces: np.ndarray, index_type: str = "u32",
               buffer: str = "file") -> None:
    """Vertices (m x 3) and 0-based triangle faces (k x 3) as one mesh with one
    primitive.  `index_type`: "u8", "u16" or "u32".  `buffer`: "file" (a .bin beside
    the .gltf), "embed" (a base64 data: URI) or "glb" (a binary .glb; `path` should end
    in .glb)."""
    ctype, dt = _INDEX_TYPES[index_type]
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    f = np.ascontiguousarray(faces, np.int64).reshape(-1)
    if len(f) and (f.min() < 0 or f.max() >= len(v) or f.max() > np.iinfo(dt).max):
        raise ValueError("face index out of range for the vertices or the index type")
    pos = v.tobytes()
    idx = _pad4(f.astype(dt).tobytes())
    blob = pos + idx
    lo = v.min(0).tolist() if len(v) else [0.0] * 3
    hi = v.max(0).tolist() if len(v) else [0.0] * 3
    doc = {
        "asset": {"version": "2.0", "generator": "portablert_gb300.gltf"},
        "buffers": [{"byteLength": len(blob)}],
        "bufferViews": [{"buffer": 0, "byteOffset": 0, "byteLength": len(pos), "target": 34962},
                        {"buffer": 0, "byteOffset": len(pos), "byteLength": len(f) * dt().itemsize,
                         "target": 34963}],
        "accessors": [{"bufferView": 0, "componentType": 5126, "count": len(v), "type": "VEC3",
                       "min": lo, "max": hi},
                      {"bufferView": 1, "componentType": ctype, "count": len(f),
                       "type": "SCALAR"}],
        "meshes": [{"primitives": [{"attributes": {"POSITION": 0}, "indices": 1}]}],
        "nodes": [{"mesh": 0}],
        "scenes": [{"nodes": [0]}],
        "scene": 0,
    }
    if buffer == "glb":
        js = _pad4(json.dumps(doc).encode(), b" ")
        body = struct.pack("<II", len(js), 0x4E4F534A) + js + \
            struct.pack("<II", len(blob), 0x004E4942) + blob
        with open(path, "wb") as out:
            out.write(struct.pack("<III", 0x46546C67, 2, 12 + len(body)) + body)
        return
    if buffer == "embed":
        doc["buffers"][0]["uri"] = ("data:application/octet-stream;base64," +
                                    base64.b64encode(blob).decode())
    elif buffer == "file":
        name = os.path.splitext(os.path.basename(path))[0] + ".bin"
        doc["buffers"][0]["uri"] = name
        with open(os.path.join(os.path.dirname(os.path.abspath(path)), name), "wb") as out:
            out.write(blob)
    else:
        raise ValueError(f"unknown buffer kind {buffer!r}")
    with open(path, "w") as out:
        json.dump(doc, out)
