"""CPU-only checks of the C ABI library: it loads, exports every symbol the header
declares, and reports (not crashes) when no GPU is present.  No compute call is made."""
import ctypes
import os
import re
import subprocess
import sys

import pytest

from conftest import ROOT
from portablert_gb300 import _lib, build, hitreg

HEADER = os.path.join(ROOT, "include", "prt_b200.h")


def declared_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"\b(prt_b200_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    build.build_library()
    return _lib.load()


def test_header_and_binding_agree():
    assert declared_functions() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (prt_b200_\w+)", out))
    missing = set(declared_functions()) - exported
    assert not missing, missing
    for name in declared_functions():
        assert hasattr(lib, name)


def test_no_gpu_is_reported_not_fatal(lib):
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    assert lib.prt_b200_available() == 0
    h = ctypes.c_void_p()
    rc = lib.prt_b200_create(0, ctypes.byref(h))
    assert rc == 3 and not h.value
    assert b"10.3" in lib.prt_b200_last_error(None)


def test_null_context_is_an_argument_error(lib):
    assert lib.prt_b200_set_tris(None, None, 0) == 1
    lay = hitreg.layout(hitreg.TAGS)
    assert lib.prt_b200_nearest_hits(None, None, 0, lay.mask, lay.size, lay.offsets8(),
                                     None) == 1
    assert lib.prt_b200_set_option(None, b"leaf_size", 4) == 1


def test_query_struct_layout_matches_header(tmp_path):
    src = tmp_path / "q.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "prt_b200.h"\n'
        'int main(void) { printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(prt_b200_query),'
        ' offsetof(prt_b200_query, rays), offsetof(prt_b200_query, n_rays),'
        ' offsetof(prt_b200_query, out), offsetof(prt_b200_query, rec_size),'
        ' offsetof(prt_b200_query, offs)); return 0; }\n')
    exe = tmp_path / "q"
    subprocess.run(["gcc", f"-I{os.path.join(ROOT, 'include')}", str(src), "-o", str(exe)],
                   check=True)
    c_side = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                             check=True).stdout.split()]
    Q = _lib.Query
    assert c_side == [ctypes.sizeof(Q), Q.rays.offset, Q.n_rays.offset, Q.out.offset,
                      Q.rec_size.offset, Q.offs.offset]


def test_cpp_api_compiles_and_links():
    exe = build.build_cpp_test()
    assert os.path.exists(exe)


def test_python_registry_mirrors_the_reference():
    """portableRT's registry calls (backend.hpp:39-95, backend.cpp:50-56) in the Python
    mirror: one backend named "B200", listed as available only where a device is, and
    nearest_hits before select_backend is the reference's "Unknown backend" error."""
    import numpy as np
    import torch

    from portablert_gb300 import backend

    everything = backend.all_backends()
    assert [b.name() for b in everything] == ["B200"]
    avail = backend.available_backends()
    if not torch.cuda.is_available():
        assert avail == []
    saved, backend.selected_backend = backend.selected_backend, None
    try:
        with pytest.raises(RuntimeError, match="Unknown backend"):
            backend.nearest_hits(np.zeros((1, 6), np.float32))
    finally:
        backend.selected_backend = saved


def test_exceptions_become_statuses(tmp_path):
    """The guard every C entry point runs its body under (prt_ctx.cuh): a body that runs
    out of host memory, or throws anything else, returns PRT_ERR_OOM with a message
    instead of letting the exception cross the C boundary; a body that returns passes
    its status through.  Host code only (no CUDA call is made)."""
    from portablert_gb300 import build as b

    src = tmp_path / "g.cu"
    src.write_text(
        '#include <cstdio>\n#include <new>\n#include <stdexcept>\n'
        f'#include "{os.path.join(ROOT, "portablert_gb300", "csrc", "prt_ctx.cuh")}"\n'
        'int main() {\n'
        '  prt::ErrorText err;\n'
        '  int a = prt::guarded(&err, "one", [&]() -> int { throw std::bad_alloc(); });\n'
        '  std::string ma = err.get();\n'
        '  int b = prt::guarded(&err, "two", [&]() -> int { throw std::runtime_error("x"); });\n'
        '  std::string mb = err.get();\n'
        '  int c = prt::guarded(&err, "three", [&]() -> int { throw 7; });\n'
        '  std::string mc = err.get();\n'
        '  int d = prt::guarded(&err, "four", [&]() -> int { return PRT_ERR_LIMIT; });\n'
        '  int e = prt::guarded(nullptr, "five", [&]() -> int { throw std::bad_alloc(); });\n'
        '  std::printf("%d %d %d %d %d|%s|%s|%s\\n", a, b, c, d, e, ma.c_str(), mb.c_str(),'
        ' mc.c_str());\n'
        '  return 0;\n}\n')
    exe = tmp_path / "g"
    r = subprocess.run([b.nvcc(), "-std=c++17", str(src), "-o", str(exe)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.strip()
    codes, ma, mb, mc = out.split("|")
    assert codes.split() == ["6", "6", "6", "7", "6"]
    assert ma == "one: out of host memory"
    assert mb == "two: x"
    assert mc == "three: unexpected exception"


def _option_lists():
    src = open(os.path.join(ROOT, "portablert_gb300", "csrc", "prt_capi.cu")).read()
    body = src[src.index("int prt_b200_set_option("):src.index("int prt_b200_get_stat(")]
    accepted = re.findall(r'k == "(\w+)"', body)
    table = src[src.index("kOptionKeys[] = {"):]
    table = table[:table.index("};")]
    env_keys = re.findall(r'"(\w+)"', table)
    hdr = open(HEADER).read()
    documented = re.findall(r'^ \*   "(\w+)"', hdr, re.M)
    return accepted, env_keys, documented


TEST_HOOKS = {"fail_alloc_after", "fail_serve_after"}  # set_option only: no environment override


def test_every_option_is_documented_and_settable_from_the_environment():
    accepted, env_keys, documented = _option_lists()
    assert sorted(set(accepted) - TEST_HOOKS) == sorted(env_keys)
    assert not TEST_HOOKS & set(env_keys)
    assert set(accepted) <= set(documented), set(accepted) - set(documented)


def _create_in_child(env_extra):
    """prt_b200_create(0) in a fresh process with extra environment: (status, message)."""
    code = (
        "import ctypes, sys\n"
        "from portablert_gb300 import _lib\n"
        "L = _lib.load()\n"
        "h = ctypes.c_void_p()\n"
        "rc = L.prt_b200_create(0, ctypes.byref(h))\n"
        "print(rc)\n"
        "print((L.prt_b200_last_error(None) or b'').decode())\n"
        "if h.value: L.prt_b200_destroy(h)\n")
    env = dict(os.environ, **env_extra)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                       cwd=ROOT, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")
    return int(lines[0]), lines[1]


@pytest.mark.parametrize("value", ["abc", "", "4x", "1.5", "99999999999999999999"])
def test_malformed_environment_override_is_an_argument_error(lib, value):
    rc, msg = _create_in_child({"PRT_B200_LEAF_SIZE": value})
    assert rc == 1 and "PRT_B200_LEAF_SIZE" in msg, (rc, msg)


def test_wellformed_environment_override_passes_the_syntax_check(lib):
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present (the GPU tests apply the override)")
    except ImportError:
        pass
    rc, msg = _create_in_child({"PRT_B200_LEAF_SIZE": " 4", "PRT_B200_BUILD_SAH": "-0"})
    assert rc == 3 and "10.3" in msg, (rc, msg)  # reached the device check
