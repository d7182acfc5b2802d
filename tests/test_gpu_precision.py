"""Precision of the FP32 and BF16 applies against the FP64 oracle on a
cubed-sphere C48 (13,824 cells) -> 1-degree lon-lat (64,800 cells) map:
64 fields sum_{l <= 32} a_lm Y_lm (a_lm ~ N(0, 1)) + 0.1 U[0, 1), weights
built in FP64 and stored in FP32, FP32 accumulation.  Reports (printed with
-s) and bounds the maximum absolute error (relative to the largest value)
and the error of the area-weighted mean (conservation, relative to the
area-weighted mean magnitude), forward and through transpose(R)."""
from __future__ import annotations

import json

import numpy as np
import oracle
import pytest
from conftest import cell_centres, sh_fields

from crg import Regridder, regrid_, workloads
from test_gpu_parity import assert_parity

pytestmark = pytest.mark.gpu

K = 64


@pytest.fixture(scope="module")
def c2(cuda):
    dst, src = workloads.precision()
    R = Regridder(dst, src, normalize=True)
    O = oracle.OracleRegridder(dst, src, normalize=True)
    S = sh_fields(cell_centres(src), K, 32, seed=48, noise=0.1)   # (K, n_src)
    D = sh_fields(cell_centres(dst), K, 32, seed=49, noise=0.1)   # (K, n_dst): input of transpose(R)
    return R, O, S, D


def test_matrix_parity(c2):
    """The matrix whose FP32 copy is measured here equals the oracle's."""
    R, O, _, _ = c2
    assert_parity(R, O)


def _gpu(RR, X, dtype, layout):
    import torch

    x = torch.from_numpy(X).to(dtype)
    n_out = RR.shape[0]
    if layout == "cell_major":
        y = torch.empty((n_out, K), dtype=dtype, device="cuda")
        regrid_(y, RR, x.T.contiguous().cuda(), dims=1)
        return y.double().cpu().numpy().T, x.double().numpy()
    y = torch.empty((K, n_out), dtype=dtype, device="cuda")
    regrid_(y, RR, x.cuda(), dims=2)
    return y.double().cpu().numpy(), x.double().numpy()


@pytest.mark.parametrize("layout", ["cell_major", "field_major"])
@pytest.mark.parametrize("dtype,tol_max,tol_mean", [("float32", 1e-6, 1e-6), ("bfloat16", 8e-3, 8e-3)])
def test_precision_against_fp64_oracle(c2, dtype, tol_max, tol_mean, layout):
    import torch

    R, O, S, D = c2
    report = {"dtype": dtype, "layout": layout}
    for name, RR, X, transpose in (("forward", R, S, False), ("transpose", R.transpose(), D, True)):
        got, xq = _gpu(RR, X, getattr(torch, dtype), layout)
        ref = O.apply(xq, transpose=transpose)          # FP64 on the values the GPU saw
        a_out = O.src_areas if transpose else O.dst_areas
        a_in = O.dst_areas if transpose else O.src_areas
        max_err = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
        # area-weighted means, relative to the area-weighted mean magnitude (a
        # field's mean can be near zero; its magnitude cannot)
        scale = np.abs(ref) @ a_out
        mean_err = float(np.max(np.abs(got @ a_out - ref @ a_out) / scale))
        cons_in = float(np.max(np.abs(got @ a_out - xq @ a_in) / scale))
        report[name] = {"max_abs_err_rel": max_err, "mean_rel_err_vs_fp64": mean_err,
                        "mean_rel_err_vs_input": cons_in}
        assert max_err <= tol_max, (name, max_err)
        assert mean_err <= tol_mean, (name, mean_err)
    print(json.dumps(report))
