"""HitReg<Tags...> layouts: the Python rules, the compat header and (where present) the
reference header give the same sizes and offsets for all 31 tag combinations."""
import os
import subprocess
import tempfile

import pytest

from conftest import ROOT
from oracle.refdir import reference_path
from portablert_gb300 import hitreg

# Measured with offsetof on portableRT's hitreg.hpp (g++ 13, x86-64):
# tags -> (size, u, v, t, primitive_id, valid, px)
EXPECTED = {
    "uv": (16, 0, 4, 8, 9, 10, 11), "t": (16, 0, 1, 4, 8, 9, 10),
    "primitive_id": (12, 0, 1, 2, 4, 8, 9), "p": (20, 0, 1, 2, 3, 4, 8),
    "valid": (8, 0, 1, 2, 3, 4, 5), "uv_t": (20, 0, 4, 8, 12, 13, 14),
    "uv_primitive_id": (20, 0, 4, 8, 12, 16, 17), "uv_p": (24, 0, 4, 8, 9, 10, 12),
    "uv_valid": (16, 0, 4, 8, 9, 10, 11), "t_primitive_id": (16, 0, 1, 4, 8, 12, 13),
    "t_p": (24, 0, 1, 4, 8, 9, 12), "t_valid": (16, 0, 1, 4, 8, 9, 10),
    "primitive_id_p": (24, 0, 1, 2, 4, 8, 12), "primitive_id_valid": (12, 0, 1, 2, 4, 8, 9),
    "p_valid": (20, 0, 1, 2, 3, 4, 8), "uv_t_primitive_id": (20, 0, 4, 8, 12, 16, 17),
    "uv_t_p": (28, 0, 4, 8, 12, 13, 16), "uv_t_valid": (20, 0, 4, 8, 12, 13, 14),
    "uv_primitive_id_p": (32, 0, 4, 8, 12, 16, 20),
    "uv_primitive_id_valid": (20, 0, 4, 8, 12, 16, 17), "uv_p_valid": (24, 0, 4, 8, 9, 10, 12),
    "t_primitive_id_p": (28, 0, 1, 4, 8, 12, 16), "t_primitive_id_valid": (16, 0, 1, 4, 8, 12, 13),
    "t_p_valid": (24, 0, 1, 4, 8, 9, 12), "primitive_id_p_valid": (24, 0, 1, 2, 4, 8, 12),
    "uv_t_primitive_id_p": (32, 0, 4, 8, 12, 16, 20),
    "uv_t_primitive_id_valid": (20, 0, 4, 8, 12, 16, 17), "uv_t_p_valid": (28, 0, 4, 8, 12, 13, 16),
    "uv_primitive_id_p_valid": (32, 0, 4, 8, 12, 16, 20),
    "t_primitive_id_p_valid": (28, 0, 1, 4, 8, 12, 16),
    "uv_t_primitive_id_p_valid": (32, 0, 4, 8, 12, 16, 20),
}


def test_31_combos_in_canonical_order():
    assert len(hitreg.TAG_COMBOS) == 31
    assert [hitreg.hitreg_name(c) for c in hitreg.TAG_COMBOS] == list(EXPECTED)


@pytest.mark.parametrize("tags", hitreg.TAG_COMBOS, ids=hitreg.hitreg_name)
def test_python_layout(tags):
    L = hitreg.layout(tags)
    assert (L.size, L.off_u, L.off_v, L.off_t, L.off_pid, L.off_valid, L.off_px) == \
        EXPECTED[hitreg.hitreg_name(tags)]
    assert hitreg.layout(tuple(reversed(tags))) == L  # order-independent


PROBE = r"""
#include <cstddef>
#include <cstdio>
#include <portableRT/hitreg.hpp>
using namespace portableRT; using namespace portableRT::filter;
template <class... T> void row(const char *n) {
  using R = HitReg<T...>;
  std::printf("%s %zu %zu %zu %zu %zu %zu %zu\n", n, sizeof(R), offsetof(R, u), offsetof(R, v),
              offsetof(R, t), offsetof(R, primitive_id), offsetof(R, valid), offsetof(R, px));
}
int main() {
@ROWS@
}
"""


def _probe(include_dir, extra=()):
    lines = []
    for c in hitreg.TAG_COMBOS:
        lines.append(f'  row<{", ".join(c)}>("{hitreg.hitreg_name(c)}");')
    src = PROBE.replace("@ROWS@", "\n".join(lines))
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "probe.cpp")
        open(p, "w").write(src)
        exe = os.path.join(d, "probe")
        subprocess.run(["g++", "-std=c++17", *extra, f"-I{include_dir}", p, "-o", exe],
                       check=True, capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return {ln.split()[0]: tuple(int(x) for x in ln.split()[1:]) for ln in out.splitlines()}


def test_compat_header_layout_matches():
    got = _probe(os.path.join(ROOT, "portablert_gb300", "compat"))
    assert got == EXPECTED


@pytest.mark.skipif(not os.path.isdir(reference_path("include")),
                    reason="portableRT sources not present")
def test_reference_header_layout_matches():
    got = _probe(reference_path("include"), extra=("-include", "cstdint", "-include", "iostream"))
    assert got == EXPECTED


def test_batch_query_record_carries_the_layout():
    """make_query fills a prt_b200_query with the HitReg layout of its tags (the C side
    reads the same field mask, record size and offsets a single query would use)."""
    from portablert_gb300 import hitreg
    from portablert_gb300.batch import Batch, make_query

    for tags in (hitreg.TAGS, ("valid",), ("t", "primitive_id", "uv", "valid")):
        lay = hitreg.layout(tags)
        q = make_query(7, 0x1000, 123, 0x2000, tags)
        assert (q.scene, q.rays, q.n_rays, q.out) == (7, 0x1000, 123, 0x2000)
        assert q.field_mask == lay.mask and q.rec_size == lay.size
        assert list(q.offs) == list(lay.offsets8())
    off, ptr, s = Batch._offsets([0, 5, 5, 12])
    assert s == 3 and off.dtype.name == "uint64" and ptr[3] == 12
