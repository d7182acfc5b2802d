"""crg.autograd on the GPU: the torch.autograd Functions return what the
library's own pullback entry points return (crg_apply_adjoint,
crg_area_grad and its swapped-build source form), and the field Function
passes torch.autograd.gradcheck in FP64 (the apply is linear, so central
differences are exact up to rounding)."""
from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import crg.autograd as ad  # noqa: E402
from crg import Regridder, grids, regrid_, regrid_adjoint_, regrid_pullback  # noqa: E402

pytestmark = pytest.mark.gpu


def test_regrid_ad_cell_major_fp32_matches_the_adjoint_apply(cuda):
    R = Regridder(grids.cubed_sphere(8, jitter=0.1, seed=2), grids.lonlat_regular(10.0, 10.0), normalize=True)
    nd, ns = R.shape
    g = torch.Generator(device=cuda).manual_seed(0)
    s = torch.randn(ns, 64, generator=g, device=cuda, requires_grad=True)
    w = torch.randn(nd, 64, generator=g, device=cuda)
    d = ad.regrid_ad(R, s)
    ref = torch.empty(nd, 64, device=cuda)
    regrid_(ref, R, s.detach())
    assert torch.equal(d, ref)
    (d * w).sum().backward()
    s_bar = torch.empty(ns, 64, device=cuda)
    regrid_adjoint_(s_bar, R, w.contiguous())
    assert torch.equal(s.grad, s_bar)


def test_regrid_ad_gradcheck_fp64_both_directions(cuda):
    R = Regridder(grids.lonlat_regular(30.0, 30.0), grids.lonlat_regular(20.0, 20.0), normalize=True)
    g = torch.Generator(device=cuda).manual_seed(1)
    for Rd in (R, R.transpose()):
        s = torch.randn(2, Rd.shape[1], generator=g, device=cuda, dtype=torch.float64, requires_grad=True)
        assert torch.autograd.gradcheck(lambda x: ad.regrid_ad(Rd, x, dims=2), (s,))


def test_regrid_vertices_ad_matches_the_pullback(cuda):
    dst, src = grids.cubed_sphere(6, jitter=0.15, seed=4), grids.lonlat_regular(15.0, 15.0)
    rng = np.random.default_rng(8)
    s0 = rng.standard_normal(src.ncells)
    w = rng.standard_normal(dst.ncells)
    s = torch.tensor(s0, requires_grad=True)
    V = torch.tensor(ad.grid_points(dst), requires_grad=True)
    W = torch.tensor(ad.grid_points(src), requires_grad=True)
    d = ad.regrid_vertices_ad(s, V, W, dst, src)
    R = Regridder(dst, src, normalize=True)
    d_ref = np.zeros(dst.ncells)
    regrid_(d_ref, R, s0)
    assert np.array_equal(d.detach().numpy(), d_ref)
    (torch.tensor(w) * d * d).sum().backward()
    s_bar, v_bar, w_bar = regrid_pullback(R, dst, src, s0, 2.0 * w * d_ref, wrt_src=True)
    assert np.array_equal(s.grad.numpy(), s_bar)  # the FP64 adjoint apply sums in a fixed order
    # shared corners accumulate with atomics, so the vertex cotangents agree to rounding only
    for got, want in ((V.grad.numpy(), v_bar), (W.grad.numpy(), w_bar)):
        assert got.shape == want.shape
        scale = np.max(np.abs(want))
        assert scale > 0
        assert np.max(np.abs(got - want)) <= 1e-12 * scale
