"""Parity at the sizes of the measured configurations, GPU against the oracle.

- large: HEALPix nside 256 nested <-> 0.25-degree lon-lat, the headline
  regridder.  Nonzero pattern (colptr, rowval) identical, areas bit-identical
  (held to 1e-12 relative at worst), both area vectors likewise; then 128 FP32
  fields (degree-64 harmonics + N(0, 0.1)) applied forward with R and back with
  transpose(R) in one call each, checked on 8 of the fields against the
  oracle's FP64 apply of the same (FP32-rounded) inputs.
- batches: all 32 jittered lon-lat pairs of 0.4 to 4 degrees, built as one
  batch, each matrix against the oracle's, and each pair's FP32 fields (1 to
  512 of them) applied by one captured plan against the oracle's FP64 apply.
- derivatives: jittered C96 <- 1-degree lon-lat.

FP32 bounds: max |got - oracle| <= 1e-6 of max |oracle|, and the area-weighted
mean within 1e-6 of the oracle's, relative to the area-weighted mean magnitude
sum(|oracle| a) / sum(a) (a field's mean can be near zero, its magnitude
cannot).  Reference: keep area > 0 and sparse(dst, src)
(src/regridder/intersection_areas.jl:115-121); d = (A s) ./ a_d
(src/regridder/regrid.jl:95-118).
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from crg import ApplyPlan, Regridder, build_batch, regrid_, workloads
from test_gpu_parity import assert_parity

pytestmark = pytest.mark.gpu

F32_MAX_REL = 1e-6
F32_MEAN_REL = 1e-6


def _check_fp32(got, ref, areas, what):
    """got, ref: (fields, cells) float64; areas of the output cells."""
    max_err = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
    scale = np.abs(ref) @ areas
    mean_err = float(np.max(np.abs(got @ areas - ref @ areas) / scale))
    assert max_err <= F32_MAX_REL, (what, "max", max_err)
    assert mean_err <= F32_MEAN_REL, (what, "mean", mean_err)
    return max_err, mean_err


@pytest.fixture(scope="module")
def large(cuda):
    hp, ll = workloads.large()
    R = Regridder(hp, ll, normalize=True)
    O = oracle.OracleRegridder(hp, ll, normalize=True)
    return hp, ll, R, O


def test_large_build_parity(large):
    _, _, R, O = large
    assert R.info["clip_overflows"] == 0
    assert R.shape == (786432, 1036800)
    assert_parity(R, O)


def test_large_apply_128_fields(large):
    import torch

    hp, ll, R, O = large
    K = 128
    dev = torch.device("cuda", 0)
    src = workloads.harmonic_fields(workloads.cell_centres(ll), K, 64, 1, 0.1, dev).T.contiguous()   # (ns, K)
    dsrc = workloads.harmonic_fields(workloads.cell_centres(hp), K, 64, 2, 0.1, dev).T.contiguous()  # (nd, K)
    out_f = torch.empty((R.shape[0], K), device=dev)
    out_r = torch.empty((R.shape[1], K), device=dev)
    regrid_(out_f, R, src, dims=1)
    regrid_(out_r, R.transpose(), dsrc, dims=1)
    pick = np.arange(0, K, K // 8)
    for name, x, y, transpose, a_out in (("forward", src, out_f, False, O.dst_areas),
                                         ("transpose", dsrc, out_r, True, O.src_areas)):
        xs = x[:, pick].T.double().cpu().numpy()
        ref = O.apply(xs, transpose=transpose)
        got = y[:, pick].T.double().cpu().numpy()
        _check_fp32(got, ref, a_out, name)


def test_derivatives_build_parity(cuda):
    dst, src = workloads.derivatives()
    assert_parity(Regridder(dst, src, normalize=True), oracle.OracleRegridder(dst, src, normalize=True))


def test_batch_pairs_parity_and_plan(cuda, monkeypatch):
    import torch

    pairs, ks = workloads.batch_pairs()
    Rs = build_batch(pairs, normalize=True, nthreads=8)
    dev = torch.device("cuda", 0)
    gen = torch.Generator(device=dev).manual_seed(5)
    items, xs = [], []
    for R, K in zip(Rs, ks):
        nd, ns = R.shape
        x = torch.randn((ns, K), generator=gen, device=dev)
        y = torch.full((nd, K), float("nan"), device=dev)
        items.append((y, R, x, 1))
        xs.append(x)
    # default: the small matrices with more than 128 fields in the persistent
    # launch, every other pair its own tuned apply on a graph branch
    plan = ApplyPlan(items)
    assert plan.info["batched_items"] == sum(K > 128 for K in ks), plan.info
    # every pair of 32 fields or more in the one persistent launch
    monkeypatch.setenv("CRG_PLAN_BATCH", "all")
    plan_all = ApplyPlan(items)
    monkeypatch.delenv("CRG_PLAN_BATCH")
    # (2 to 31 fields keep their own applies on the narrow merge-path kernel)
    assert plan_all.info["batched_items"] == sum(K == 1 or K >= 32 for K in ks), plan_all.info
    plan.launch()
    torch.cuda.synchronize()
    got = [y.clone() for y, _, _, _ in items]
    for y, _, _, _ in items:
        y.fill_(float("nan"))
    plan_all.launch()
    torch.cuda.synchronize()
    for (dst, src), R, K, g, (y, _, x, _) in zip(pairs, Rs, ks, got, items):
        assert torch.equal(g, y), f"pair {R.shape} K={K}: the two plans differ"
        O = oracle.OracleRegridder(dst, src, normalize=True)
        assert_parity(R, O)
        ref = O.apply(x.T.double().cpu().numpy())
        _check_fp32(y.T.double().cpu().numpy(), ref, O.dst_areas, f"pair {R.shape} K={K}")
