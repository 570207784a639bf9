"""Host-side logic of the request server that needs no GPU: its budget allocator."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("sanitize", [False, True])
def test_range_allocator(tmp_path, sanitize):
    """The allocator's randomized test, plain and under AddressSanitizer and UBSan."""
    exe = tmp_path / "range_alloc_test"
    src = os.path.join(ROOT, "tests", "cpp", "range_alloc_test.cpp")
    inc = os.path.join(ROOT, "portablert_gb300", "csrc")
    flags = ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined", "-g"] \
        if sanitize else []
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall"] + flags + ["-I", inc, src, "-o",
                                                                        str(exe)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        if sanitize and "asan" in r.stderr.lower():
            pytest.skip("AddressSanitizer runtime not available")
        pytest.fail(r.stderr)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "ok" in out.stdout
    assert "runtime error" not in out.stderr
