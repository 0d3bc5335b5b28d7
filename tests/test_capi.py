"""The C-ABI library builds, loads without a GPU and exports every declared symbol (CPU)."""

from __future__ import annotations

import re
from pathlib import Path

import pytest

from conftest import ROOT


def _declared() -> set[str]:
    text = (ROOT / "include" / "xkgpu.h").read_text()
    return set(re.findall(r"^\s*(?:xk_status|const char\*)\s+(xk_\w+)\s*\(", text, flags=re.M))


@pytest.fixture(scope="module")
def lib():
    from xkgpu import _lib as L
    from xkgpu import build

    build.build()
    return L.load()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert "xk_pair_step" in names and len(names) >= 14
    for n in sorted(names):
        assert hasattr(lib, n), n


def test_binding_covers_header(lib):
    from xkgpu import _lib as L

    assert _declared() == set(L.exported_symbols())
    assert lib.xk_version().startswith(b"xkgpu")


def test_struct_layouts_match_header():
    import ctypes as C

    from xkgpu import _lib as L

    # field order and sizes as declared in include/xkgpu.h (LP64)
    assert C.sizeof(L.Section) == 9 * 8
    assert C.sizeof(L.Mesh) == 8 + 6 * 8
    assert C.sizeof(L.Pairs) == 8 + 23 * 8
    assert C.sizeof(L.Pairs32) == 16 + 26 * 8 + 2 * 4 + 8
    assert C.sizeof(L.BeamPlan) == 8 + 4 * 8 + 8 + 8 + 8  # chain_ordered and beam_ctas_per_sm (int32)
    assert L.BeamPlan.chain_ordered.offset == 56 and L.BeamPlan.beam_ctas_per_sm.offset == 60
    assert C.sizeof(L.ContactParams) == 6 * 8 + 8 + 5 * 8
    assert C.sizeof(L.BPParams) == 8 + 3 * 4 + 4 + 8 + 8
    assert C.sizeof(L.ContactPattern) == 16 + 5 * 8 + 10 * 8 + 2 * 8 + 7 * 8 + 3 * 8 + 2 * 4
    assert C.sizeof(L.System) == 8 + 13 * 8


def test_argument_checks_before_any_launch(lib):
    """Malformed calls are refused on the host with XK_ERR_ARG, before any device work (no GPU needed)."""
    import ctypes as C

    lib.xk_mlp_forward_tcgen05.restype = C.c_int
    lib.xk_mlp_forward_tcgen05.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.xk_last_error.restype = C.c_char_p
    # null parameters, negative count, misaligned feature rows
    assert lib.xk_mlp_forward_tcgen05(None, None, 0, None, None, None) == 1
    assert lib.xk_mlp_forward_tcgen05(0x1000, 0x2000, -1, 0x3000, 0x4000, None) == 1
    assert lib.xk_mlp_forward_tcgen05(0x1000, 0x2004, 8, 0x3000, 0x4000, None) == 1
    assert b"16-byte aligned" in lib.xk_last_error()
    # the device linear solve: null system, check interval below one
    from xkgpu import _lib as L

    assert lib.xk_bicgstab(None, None, None, None, None, 10, 1, 1e-8, None, None, None) == 1
    s = L.System(4, 0, 0x1000, 0x2000, 0x3000, 0x1000, 0x1000, 0x1000)
    assert lib.xk_bicgstab(C.byref(s), 0x1000, 0x2000, 0x3000, 0x4000, 10, 0, 1e-8, None, None, None) == 1
    assert lib.xk_system_spmv(None, 0x1000, 0x2000, None) == 1
