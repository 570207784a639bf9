"""Host-side logic of the request server that needs no GPU: its budget allocator."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_range_allocator(tmp_path):
    exe = tmp_path / "range_alloc_test"
    src = os.path.join(ROOT, "tests", "cpp", "range_alloc_test.cpp")
    inc = os.path.join(ROOT, "portablert_gb300", "csrc")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", inc, src, "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "ok" in out.stdout
