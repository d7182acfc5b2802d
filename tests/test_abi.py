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


def test_loader_checks_the_abi_version(monkeypatch):
    """load() compares the library's crg_abi_version() with CRG_ABI_VERSION of
    include/crg.h and refuses a library built for another version."""
    lib = _lib.load()
    assert _lib.abi_version() == lib.crg_abi_version() == 2
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "abi_version", lambda: 3)
    try:
        _lib.load(build_if_missing=False)
    except RuntimeError as e:
        assert "ABI version 2" in str(e) and "declares 3" in str(e)
    else:
        raise AssertionError("a library of another ABI version was accepted")
    monkeypatch.undo()
    assert _lib.load() is lib


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


def _curvi(nx, ny, pts, manifold=None):
    d = _lib.crg_grid_desc()
    d.kind = _lib.CRG_GRID_CURVILINEAR
    d.manifold = _lib.CRG_SPHERICAL if manifold is None else manifold
    d.nblocks = 1
    d.ncells = nx * ny
    bx = (C.c_int64 * 1)(nx)
    by = (C.c_int64 * 1)(ny)
    d.block_nx = C.cast(bx, C.POINTER(C.c_int64))
    d.block_ny = C.cast(by, C.POINTER(C.c_int64))
    d.points = pts.ctypes.data
    return d, (bx, by, pts)


def test_build_checks_grid_descriptors_before_device_work():
    """crg_build and crg_build_batch refuse malformed grids with the reference's
    error classes (ArgumentError / DimensionMismatch, src/regridder/regrid.jl:242-245,
    :289-296) before any CUDA call, so they answer the same without a GPU."""
    import numpy as np

    lib = _lib.load()
    pts = np.zeros((3, 3, 3))
    good, keep = _curvi(2, 2, pts)
    out = C.c_void_p()

    def build(dst, src=good):
        st = lib.crg_build(C.byref(dst), C.byref(src), None, C.byref(out))
        assert out.value is None
        return st, lib.crg_last_error().decode()

    bad, k1 = _curvi(2, 2, pts)
    bad.manifold = 7
    st, msg = build(good, bad)
    assert st == _lib.CRG_ERR_INVALID_ARGUMENT and "manifold" in msg
    bad, k1 = _curvi(2, 2, pts)
    bad.nblocks = 0
    assert build(bad) == (_lib.CRG_ERR_INVALID_ARGUMENT, "destination grid: nblocks = 0 must be in 1..12")
    bad, k1 = _curvi(2, 2, pts)
    bad.ncells = 5
    st, msg = build(bad)
    assert st == _lib.CRG_ERR_DIMENSION_MISMATCH and "ncells = 5" in msg
    bad, k1 = _curvi(0, 2, pts)
    st, msg = build(good, bad)
    assert st == _lib.CRG_ERR_INVALID_ARGUMENT and msg.startswith("source grid: block 0 has 0 x 2 cells")
    bad, k1 = _curvi(2, 2, pts)
    bad.points = None
    assert build(bad)[0] == _lib.CRG_ERR_INVALID_ARGUMENT
    bad, k1 = _curvi(2, 2, pts)
    bad.ncells = -1
    assert build(bad)[0] == _lib.CRG_ERR_NOT_SUPPORTED
    cells = _lib.crg_grid_desc()
    cells.kind = _lib.CRG_GRID_CELLS
    cells.manifold = _lib.CRG_SPHERICAL
    cells.ncells = 4
    cells.max_verts = 9
    st, msg = build(cells)
    assert st == _lib.CRG_ERR_INVALID_ARGUMENT and "max_verts = 9" in msg
    cells.max_verts = 4
    st, msg = build(cells)
    assert st == _lib.CRG_ERR_INVALID_ARGUMENT and "cell_verts is NULL" in msg
    cells.kind = 5
    assert build(cells)[0] == _lib.CRG_ERR_INVALID_ARGUMENT
    # a batch names the failing item and leaves every output NULL
    dsts = (_lib.crg_grid_desc * 2)(good, good)
    bad, k1 = _curvi(2, 2, pts)
    bad.nblocks = 13
    srcs = (_lib.crg_grid_desc * 2)(good, bad)
    outs = (C.c_void_p * 2)(1, 1)
    assert lib.crg_build_batch(2, dsts, srcs, None, 1, outs) == _lib.CRG_ERR_INVALID_ARGUMENT
    assert lib.crg_last_error().decode().startswith("pair 1: source grid: nblocks = 13")
    assert list(outs) == [None, None]


def test_plain_c_caller(tmp_path):
    """include/crg.h is C99 (no C++ needed by a caller), the library links
    from C, and its GPU-free answers come back through the C ABI."""
    import shutil
    import subprocess

    if shutil.which("gcc") is None:
        import pytest

        pytest.skip("no C compiler")
    lib = _lib.load()
    assert lib is not None
    exe = tmp_path / "c_abi_caller"
    build = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                            "-I", str(ROOT / "include"), str(ROOT / "tests" / "c_abi_caller.c"),
                            str(_build.LIB_PATH), f"-Wl,-rpath,{_build.LIB_PATH.parent}", "-o", str(exe)],
                           capture_output=True, text=True)
    assert build.returncode == 0, build.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, run.stderr
    assert "c abi ok" in run.stdout
