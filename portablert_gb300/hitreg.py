"""Hit-record layout of portableRT's filter-tagged ``HitReg<Tags...>``.

``HitRegImpl`` (include/portableRT/hitreg.hpp:29-44 in portableRT) declares, in this
order, ``u, v, t, primitive_id, valid, px, py, pz``.  A field whose tag is absent has
type ``Empty`` (one byte, alignment 1); present floats and the uint32 id are four
bytes aligned to four, ``valid`` is a one-byte ``bool``.  The record is therefore a
plain C struct laid out by the usual rules, which this module reproduces so that the
CUDA kernels can write exactly the bytes the C++ caller's ``std::vector`` expects.

The tag set is order-independent: ``HitReg<t, uv>`` and ``HitReg<uv, t>`` are the
same type (hitreg.hpp:56-59), so everything here keys on the set of tags.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass

import numpy as np

TAGS = ("uv", "t", "primitive_id", "p", "valid")

# Bit per tag in the C-ABI field mask (include/prt_b200.h).
FIELD_BIT = {"uv": 1, "t": 2, "primitive_id": 4, "p": 8, "valid": 16}

# The 31 combinations in portableRT's canonical order (hitreg.hpp:146-177).
TAG_COMBOS = tuple(
    c for n in range(1, 6) for c in itertools.combinations(TAGS, n)
)


def canonical(tags) -> tuple:
    """Tags in canonical order (the order of TAG_COMBOS), duplicates removed."""
    s = set(tags)
    bad = s - set(TAGS)
    if bad:
        raise ValueError(f"unknown filter tags: {sorted(bad)}")
    return tuple(t for t in TAGS if t in s)


def hitreg_name(tags) -> str:
    """portableRT::hitreg_name<Tags...>() for tags given in canonical order."""
    return "_".join(canonical(tags))


def field_mask(tags) -> int:
    m = 0
    for t in canonical(tags):
        m |= FIELD_BIT[t]
    return m


@dataclass(frozen=True)
class Layout:
    tags: tuple
    size: int
    align: int
    off_u: int
    off_v: int
    off_t: int
    off_pid: int
    off_valid: int
    off_px: int

    @property
    def mask(self) -> int:
        return field_mask(self.tags)

    def offsets8(self) -> bytes:
        """Offsets in the order the C-ABI takes them: u, v, t, primitive_id, valid,
        px, py, pz (one byte each; records are at most 32 bytes)."""
        py = self.off_px + (4 if "p" in self.tags else 1)
        pz = py + (4 if "p" in self.tags else 1)
        return bytes([self.off_u, self.off_v, self.off_t, self.off_pid, self.off_valid,
                      self.off_px, py, pz])

    def numpy_dtype(self) -> np.dtype:
        """A structured dtype with the present fields at their offsets."""
        names, formats, offsets = [], [], []
        if "uv" in self.tags:
            names += ["u", "v"]; formats += ["<f4", "<f4"]; offsets += [self.off_u, self.off_v]
        if "t" in self.tags:
            names.append("t"); formats.append("<f4"); offsets.append(self.off_t)
        if "primitive_id" in self.tags:
            names.append("primitive_id"); formats.append("<u4"); offsets.append(self.off_pid)
        if "valid" in self.tags:
            names.append("valid"); formats.append("u1"); offsets.append(self.off_valid)
        if "p" in self.tags:
            names += ["px", "py", "pz"]; formats += ["<f4"] * 3
            offsets += [self.off_px, self.off_px + 4, self.off_px + 8]
        return np.dtype({"names": names, "formats": formats, "offsets": offsets,
                         "itemsize": self.size})


def layout(tags) -> Layout:
    """Struct layout of HitReg<tags...> under the C/C++ struct rules."""
    tags = canonical(tags)
    has = set(tags)
    # (name, size, align) in declaration order; absent fields are 1-byte Empty.
    fields = [
        ("u", 4 if "uv" in has else 1),
        ("v", 4 if "uv" in has else 1),
        ("t", 4 if "t" in has else 1),
        ("primitive_id", 4 if "primitive_id" in has else 1),
        ("valid", 1),
        ("px", 4 if "p" in has else 1),
        ("py", 4 if "p" in has else 1),
        ("pz", 4 if "p" in has else 1),
    ]
    off = {}
    cur = 0
    max_align = 1
    for name, size in fields:
        align = size  # 4-byte members align to 4, one-byte members to 1
        cur = (cur + align - 1) // align * align
        off[name] = cur
        cur += size
        max_align = max(max_align, align)
    size = (cur + max_align - 1) // max_align * max_align
    return Layout(tags, size, max_align, off["u"], off["v"], off["t"], off["primitive_id"],
                  off["valid"], off["px"])


FULL = layout(TAGS)
assert FULL.size == 32 and FULL.off_px == 20
