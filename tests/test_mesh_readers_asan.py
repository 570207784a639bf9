"""The mesh readers (prt_obj.cu, prt_gltf.cu: host code only) compiled with
AddressSanitizer and UndefinedBehaviorSanitizer and run over a seeded corpus of valid,
truncated and byte-flipped .gltf, .glb and .obj files: every file must give a status,
with no invalid memory access, leak or undefined behaviour reported."""
import base64
import json
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from portablert_gb300 import gltf, obj

CSRC = os.path.join(ROOT, "portablert_gb300", "csrc")

DRIVER = r"""
#include <cstdio>
#include <cstring>
#include <string>
#include "prt_b200.h"
namespace prt {
static std::string g_err;
void set_global_error(const std::string &msg) { g_err = msg; }
}
int main(int argc, char **argv) {
	for (int i = 1; i < argc; ++i) {
		float *t = nullptr;
		uint64_t n = 0;
		const size_t len = std::strlen(argv[i]);
		const bool is_obj = len > 4 && std::strcmp(argv[i] + len - 4, ".obj") == 0;
		const int rc = is_obj ? prt_b200_obj_load(argv[i], &t, &n)
		                      : prt_b200_gltf_load(argv[i], &t, &n);
		double sum = 0.0;
		for (uint64_t k = 0; k < 9 * n; ++k)
			sum += t[k] == t[k] ? 0.0 : 1.0;  // touches every float the reader returned
		std::printf("%d %llu %g\n", rc, (unsigned long long)n, sum);
		prt_b200_free(t);
	}
	return 0;
}
"""


def _corpus(tmp_path):
    rng = np.random.default_rng(5)
    v, f = obj.blob_mesh(6, 8)
    seeds = []
    for kind, name in (("glb", "a.glb"), ("embed", "b.gltf"), ("file", "c.gltf")):
        p = tmp_path / name
        gltf.write_gltf(str(p), v, f, "u16", kind)
        seeds.append((p.read_bytes(), os.path.splitext(name)[1]))
    o = tmp_path / "d.obj"
    obj.write_obj(str(o), v, f)
    seeds.append((o.read_bytes(), ".obj"))
    paths = [str(tmp_path / n) for n in ("a.glb", "b.gltf", "c.gltf", "d.obj")]
    for i in range(600):
        data, ext = seeds[i % len(seeds)]
        data = bytearray(data)
        if rng.random() < 0.3:
            data = data[:int(rng.integers(0, len(data) + 1))]
        for _ in range(int(rng.integers(1, 8))):
            if data:
                data[int(rng.integers(0, len(data)))] = int(rng.integers(0, 256))
        p = tmp_path / f"m{i}{ext}"
        p.write_bytes(bytes(data))
        paths.append(str(p))
    # Hand-made edge cases: deep nesting, a huge count, an index past the end.
    deep = tmp_path / "deep.gltf"
    deep.write_text("[" * 5000 + "]" * 5000)
    big = tmp_path / "big.gltf"
    blob = base64.b64encode(b"\0" * 48).decode()
    big.write_text(json.dumps({
        "buffers": [{"uri": "data:;base64," + blob, "byteLength": 48}],
        "bufferViews": [{"buffer": 0, "byteLength": 48}],
        "accessors": [{"bufferView": 0, "componentType": 5126, "count": 2 ** 50, "type": "VEC3"},
                      {"bufferView": 0, "componentType": 5125, "count": 12, "type": "SCALAR"}],
        "meshes": [{"primitives": [{"attributes": {"POSITION": 0}, "indices": 1}]}]}))
    glb_len = tmp_path / "len.glb"
    glb_len.write_bytes(struct.pack("<IIIII", 0x46546C67, 2, 0xFFFFFFFF, 0xFFFFFFF0, 0x4E4F534A))
    return paths + [str(deep), str(big), str(glb_len)]


def test_mesh_readers_under_sanitizers(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    exe = tmp_path / "readers"
    drv = tmp_path / "driver.cpp"
    drv.write_text(DRIVER)
    cmd = [gxx, "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=undefined", f"-I{os.path.join(ROOT, 'include')}",
           "-x", "c++", os.path.join(CSRC, "prt_gltf.cu"), os.path.join(CSRC, "prt_obj.cu"),
           "-x", "none", str(drv), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "asan" in r.stderr.lower():
        pytest.skip("AddressSanitizer runtime not available")
    assert r.returncode == 0, r.stderr
    paths = _corpus(tmp_path)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0",
               UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([str(exe)] + paths, capture_output=True, text=True, env=env,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr, \
        r.stderr[-3000:]
    lines = r.stdout.split("\n")
    rcs = [int(ln.split()[0]) for ln in lines if ln]
    assert len(rcs) == len(paths)
    assert rcs[:4] == [0, 0, 0, 0]  # the unmutated files load
    assert set(rcs) <= {0, 1, 6}
    assert rcs[-3:] == [1, 1, 1]    # deep nesting, huge count, bad GLB length: errors
