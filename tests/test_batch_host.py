"""Host logic of the batch entry points (regrid_batch_ / ApplyPlan): how each
(dst, R, src[, dims]) item becomes a crg_apply_item -- strides, field counts,
direction -- and which items are refused before the library is called.  A
regridder view with a dummy handle stands in for a built one (no GPU)."""
from __future__ import annotations

import types

import numpy as np
import pytest

from crg import ArgumentError, DimensionMismatch, Regridder, _lib
from crg.batch import _items


def _fake(nd=5, ns=7, transposed=False):
    return Regridder(None, None, _view=dict(info={"n_dst": nd, "n_src": ns}, _transposed=transposed,
                                            _h=types.SimpleNamespace(ptr=4096)))


def test_items_carry_strides_and_direction():
    R = _fake()
    arr, keep = _items([(np.zeros(5), R, np.ones(7)),
                        (np.zeros((5, 8), np.float32), R, np.ones((7, 8), np.float32)),
                        (np.zeros((8, 5)), R, np.ones((8, 7)), 2),
                        (np.zeros(7), _fake(transposed=True), np.ones(5))], True, "batch")
    a = arr[0]
    assert (a.regridder, a.transpose, a.dtype, a.nfields, a.normalize, a.adjoint) == (4096, 0, _lib.CRG_F64, 1, 1, 0)
    assert (a.src_stride_cell, a.dst_stride_cell) == (1, 1)
    b = arr[1]  # cell-major: the 8 fields of a cell side by side
    assert (b.dtype, b.nfields, b.src_stride_cell, b.src_stride_field, b.dst_stride_cell, b.dst_stride_field) == \
        (_lib.CRG_F32, 8, 8, 1, 8, 1)
    c = arr[2]  # dims = 2: each field's cells contiguous
    assert (c.nfields, c.src_stride_cell, c.src_stride_field, c.dst_stride_cell, c.dst_stride_field) == (8, 1, 7, 1, 5)
    assert arr[3].transpose == 1
    assert len(keep) == 12


def test_items_refusals():
    R = _fake()
    with pytest.raises(ArgumentError, match="item 0: expected a Regridder"):
        _items([(np.zeros(5), object(), np.ones(7))], True, "batch")
    with pytest.raises(ArgumentError, match="item 0: source and destination dtypes differ"):
        _items([(np.zeros(5), R, np.ones(7, np.float32))], True, "batch")
    with pytest.raises(DimensionMismatch, match="item 1: source has 6 cells, expected 7"):
        _items([(np.zeros(5), R, np.ones(7)), (np.zeros(5), R, np.ones(6))], True, "batch")
    with pytest.raises(DimensionMismatch, match="3 source fields but 4 destination fields"):
        _items([(np.zeros((5, 4)), R, np.ones((7, 3)))], True, "batch")
    with pytest.raises(DimensionMismatch, match="along dims=2"):
        _items([(np.zeros((4, 5)), R, np.ones((7, 4)), 2)], True, "batch")
    with pytest.raises(ArgumentError, match="1-D or 2-D"):
        _items([(np.zeros((5, 2, 2)), R, np.ones((7, 2, 2)))], True, "batch")
    with pytest.raises(ArgumentError, match="plan fields must be CUDA tensors"):
        _items([(np.zeros(5), R, np.ones(7))], True, "plan")
