"""The C-ABI library builds for sm_103a, loads without a GPU and exports every
entry point declared in include/crg.h (no compute calls)."""
from __future__ import annotations

import ctypes as C
import re

from conftest import ROOT
from crg import _build, _lib


def declared_symbols():
    text = (ROOT / "include" / "crg.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(crg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    syms = declared_symbols()
    assert len(syms) >= 12
    for s in syms:
        assert hasattr(lib, s), s
        assert s in _lib.SIGNATURES, f"{s} missing from the ctypes binding"


def test_binding_covers_only_declared_symbols():
    assert set(_lib.SIGNATURES) == set(declared_symbols())


def test_cpu_safe_entry_points():
    lib = _lib.load()
    assert lib.crg_abi_version() == 2
    assert lib.crg_status_string(0) == b"ok"
    assert lib.crg_status_string(2) == b"dimension mismatch"
    # argument validation happens before any device work
    assert lib.crg_build(None, None, None, None) == _lib.CRG_ERR_INVALID_ARGUMENT
    assert b"NULL" in lib.crg_last_error()
    assert lib.crg_regridder_release(None) == 0


def test_se_entry_points_validate_before_device_work():
    """The SE builds check the space, the FV grid and the rule degree on the
    host (the reference's errors: reference_rule's "not available", :416-506)."""
    lib = _lib.load()
    out = C.c_void_p()
    assert lib.crg_build_se_to_fv(None, None, None, C.byref(out)) == _lib.CRG_ERR_INVALID_ARGUMENT
    fv = _lib.crg_grid_desc()
    fv.manifold = _lib.CRG_SPHERICAL
    space = _lib.crg_se_space()
    space.elements.manifold = _lib.CRG_SPHERICAL
    space.nq = 9
    assert lib.crg_build_se_to_fv(C.byref(fv), C.byref(space), None, C.byref(out)) == _lib.CRG_ERR_INVALID_ARGUMENT
    assert b"nq = 9" in lib.crg_last_error()
    space.nq = 4
    opts = _lib.crg_se_opts(9, 0, 0.0, None)
    assert lib.crg_build_fv_to_se(C.byref(space), C.byref(fv), C.byref(opts), C.byref(out)) == \
        _lib.CRG_ERR_INVALID_ARGUMENT
    assert b"degree 9 not available" in lib.crg_last_error()
    space.elements.manifold = _lib.CRG_PLANAR
    assert lib.crg_build_se_to_fv(C.byref(fv), C.byref(space), None, C.byref(out)) == _lib.CRG_ERR_INVALID_ARGUMENT
    assert b"spherical" in lib.crg_last_error()
    assert out.value is None


def test_build_is_sm103a_and_in_tree():
    assert any("sm_103a" in f for f in _build.ARCH_FLAGS)
    assert "--fmad=false" in _build.NVCC_FLAGS
    assert _build.LIB_PATH.is_relative_to(ROOT)
