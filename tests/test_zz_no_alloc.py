"""crg_apply_noalloc: the batched apply for callers that cannot allocate device
memory (for example an application whose memory pool already owns the whole
GPU, or one that allocates everything up front and forbids allocation while it
runs).  It keeps its scratch in a fixed static array, so it is checked here
through the C ABI against crg_apply on two calls in a row -- the second call
must not see anything the first one left in the shared scratch -- and for its
refusals (host buffers, a regridder too large for the scratch).

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from crg import Regridder, _lib, grids

pytestmark = pytest.mark.gpu

TOL = 1e-6  # the FP32 tolerance of the apply tests (identical kernels: expected bit-equal)


def _call(fn, R, transpose, x, K, y, stream=None, dtype=_lib.CRG_F32):
    return fn(C.c_void_p(R._h.ptr), transpose, dtype, C.c_void_p(x.data_ptr()), K, 1, C.c_void_p(y.data_ptr()),
              K, 1, K, 1, C.c_void_p(stream) if stream else None)


def test_noalloc_matches_apply_on_consecutive_calls(cuda):
    import torch

    lib = _lib.load()
    # 10-degree cells over HEALPix 32: forward rows of ~30 entries are cut between
    # work blocks, so the static scratch carries partial sums
    R = Regridder(grids.lonlat_regular(10.0, 10.0), grids.healpix_grid(32), normalize=True)
    assert R.info["carry_slots"][0] > 0
    nd, ns = R.shape
    gen = torch.Generator(device="cuda").manual_seed(5)
    # 64 fields: the merge-path kernel; 8: the narrow one (both through the scratch)
    for K, transpose, nin, nout in ((64, 0, ns, nd), (64, 1, nd, ns), (8, 0, ns, nd), (8, 1, nd, ns)):
        for _ in range(2):  # two calls in a row share the static scratch
            x = torch.randn((nin, K), generator=gen, device="cuda")
            ref = torch.empty((nout, K), device="cuda")
            got = torch.full((nout, K), float("nan"), device="cuda")
            assert _call(lib.crg_apply, R, transpose, x, K, ref) == _lib.CRG_OK
            st = _call(lib.crg_apply_noalloc, R, transpose, x, K, got)
            assert st == _lib.CRG_OK, lib.crg_last_error().decode()
            torch.cuda.synchronize()
            err = (got - ref).abs().max().item() / ref.abs().max().item()
            assert err <= TOL
            assert torch.equal(got, ref)


def test_noalloc_refusals(cuda):
    import torch

    lib = _lib.load()
    R = Regridder(grids.healpix_grid(8), grids.lonlat_regular(5.0, 5.0), normalize=True)
    nd, ns = R.shape
    K = 8
    # host buffers would need staging memory
    xh = torch.zeros((ns, K))
    yh = torch.zeros((nd, K))
    assert _call(lib.crg_apply_noalloc, R, 0, xh, K, yh) == _lib.CRG_ERR_NOT_SUPPORTED
    assert b"device pointers" in lib.crg_last_error()
    # a regridder whose cut rows need more than the static scratch's 32,768 pieces:
    # 30-degree cells over a 0.15-degree source, about 40,000 entries per row
    big = Regridder(grids.lonlat_regular(30.0, 30.0), grids.lonlat_regular(0.15, 0.15), normalize=True)
    assert big.info["carry_slots"][0] > 32768
    x = torch.zeros((big.shape[1], K), device="cuda")
    y = torch.zeros((big.shape[0], K), device="cuda")
    assert _call(lib.crg_apply_noalloc, big, 0, x, K, y) == _lib.CRG_ERR_NOT_SUPPORTED
    assert b"static scratch" in lib.crg_last_error()


def test_noalloc_bf16_and_no_device_allocation(cuda):
    """BF16 fields through the allocation-free path equal crg_apply's, and a
    call changes the device's free memory by nothing (after a first call on
    the same regridder, and with the stream drained on both sides)."""
    import torch

    lib = _lib.load()
    R = Regridder(grids.lonlat_regular(10.0, 10.0), grids.healpix_grid(32), normalize=True)
    nd, ns = R.shape
    K = 32
    gen = torch.Generator(device="cuda").manual_seed(9)
    for dtype, code in ((torch.bfloat16, _lib.CRG_BF16), (torch.float32, _lib.CRG_F32)):
        for transpose, nin, nout in ((0, ns, nd), (1, nd, ns)):
            x = torch.randn((nin, K), generator=gen, device="cuda").to(dtype)
            ref = torch.empty((nout, K), dtype=dtype, device="cuda")
            got = torch.full((nout, K), float("nan"), dtype=dtype, device="cuda")
            assert _call(lib.crg_apply, R, transpose, x, K, ref, dtype=code) == _lib.CRG_OK
            assert _call(lib.crg_apply_noalloc, R, transpose, x, K, got, dtype=code) == _lib.CRG_OK
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            got.fill_(float("nan"))
            torch.cuda.synchronize()
            assert _call(lib.crg_apply_noalloc, R, transpose, x, K, got, dtype=code) == _lib.CRG_OK
            torch.cuda.synchronize()
            assert torch.cuda.mem_get_info()[0] == free0, "crg_apply_noalloc changed the free device memory"
            assert torch.equal(got, ref), (dtype, transpose)
