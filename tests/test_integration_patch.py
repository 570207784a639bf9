"""The drop-in: portableRT patched with portablert_gb300/integration/portableRT-b200.patch
(plus the three backend files) builds its own example programs with the B200 backend in
the variant, and they run.  Needs the portableRT sources, so it only runs where they
are present; without a GPU the B200 backend registers as unavailable and the CPU
backend answers, exactly as the reference's registry intends."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT
from oracle.refdir import REFERENCE_DIR
from portablert_gb300 import build

REF = REFERENCE_DIR
PATCH = os.path.join(ROOT, "portablert_gb300", "integration", "portableRT-b200.patch")

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")),
                                reason="portableRT sources not present")


def _patched_tree(tmp_path):
    dst = tmp_path / "portableRT"
    shutil.copytree(REF, dst)
    subprocess.run(["patch", "-p1", "-i", PATCH], cwd=dst, check=True, capture_output=True)
    shutil.copy(os.path.join(ROOT, "include", "prt_b200.h"), dst / "include" / "prt_b200.h")
    shutil.copy(os.path.join(ROOT, "include", "portableRT", "intersect_b200.hpp"),
                dst / "include" / "portableRT" / "intersect_b200.hpp")
    shutil.copy(os.path.join(ROOT, "portablert_gb300", "src", "intersect_b200.cpp"),
                dst / "src" / "intersect_b200.cpp")
    return dst


@pytest.mark.parametrize("example", ["simple", "triangle"])
def test_reference_examples_build_and_run_with_b200(tmp_path, example):
    lib = build.build_library()
    tree = _patched_tree(tmp_path)
    exe = tmp_path / example
    cmd = ["g++", "-O2", "-std=c++17", "-DUSE_B200", "-include", "cstdint", "-include",
           "iostream", "-include", "stdexcept", f"-I{tree / 'include'}",
           str(tree / "examples" / example / "main.cpp"), str(tree / "src" / "backend.cpp"),
           str(tree / "src" / "intersect_cpu.cpp"), str(tree / "src" / "intersect_b200.cpp"),
           "-o", str(exe), f"-L{os.path.dirname(lib)}", "-lprt_b200",
           f"-Wl,-rpath,{os.path.dirname(lib)}", "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert "Testing CPU" in out.stdout
    if example == "simple":
        assert "Ray 1: 1" in out.stdout and "Ray 2: 0" in out.stdout


def test_b200_is_registered_in_all_backends(tmp_path):
    lib = build.build_library()
    tree = _patched_tree(tmp_path)
    src = tmp_path / "list.cpp"
    src.write_text(
        "#include <portableRT/portableRT.hpp>\n"
        "int main() { for (auto *b : portableRT::all_backends()) std::cout << b->name() << '\\n';"
        " return 0; }\n")
    exe = tmp_path / "list"
    cmd = ["g++", "-O2", "-std=c++17", "-DUSE_B200", "-include", "cstdint", "-include",
           "iostream", "-include", "stdexcept", f"-I{tree / 'include'}", str(src),
           str(tree / "src" / "backend.cpp"), str(tree / "src" / "intersect_cpu.cpp"),
           str(tree / "src" / "intersect_b200.cpp"), "-o", str(exe),
           f"-L{os.path.dirname(lib)}", "-lprt_b200", f"-Wl,-rpath,{os.path.dirname(lib)}",
           "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60).stdout.split()
    assert "B200" in out and "CPU" in out
