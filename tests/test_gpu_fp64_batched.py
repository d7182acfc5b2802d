"""Many FP64 fields in one launch, at the reference's precision.

Cell-major FP64 fields (the fields of a cell side by side) go through one
kernel for all fields; every field must still have the bits of the
reference's regrid! -- one stdlib CSC mul! per slice, then ./ a_d
(src/regridder/regrid.jl:95-118, the N-D loop :303-318) -- as the oracle
computes it, and of the one-field GPU apply.  Field counts below, at and above
the 128 a lane group covers, aligned and not; R and transpose(R); with and
without normalisation; the adjoint against one-field adjoints; and 8, 24 and
128 fields of the large configuration (HEALPix 256 <-> 0.25 degree), whose
polar rows hold hundreds of entries.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import c1_grids
from crg import Regridder, regrid_, regrid_adjoint_, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c1(cuda):
    dst, src = c1_grids()
    return Regridder(dst, src, normalize=True), oracle.OracleRegridder(dst, src, normalize=True)


def _cm(R, X, transpose, normalize):
    """Apply to the (K, n) fields X laid out cell-major on the device; (K, n_out)."""
    import torch

    RR = R.transpose() if transpose else R
    x = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()
    y = torch.full((RR.shape[0], X.shape[0]), float("nan"), dtype=torch.float64, device="cuda")
    regrid_(y, RR, x, dims=1, normalize=normalize)
    return y.T.cpu().numpy()


@pytest.mark.parametrize("K", [2, 7, 8, 16, 24, 32, 64, 128, 130, 300])
@pytest.mark.parametrize("transpose", [False, True])
@pytest.mark.parametrize("normalize", [True, False])
def test_cell_major_fp64_bit_exact(c1, K, transpose, normalize):
    R, O = c1
    rng = np.random.default_rng(K + 100 * transpose)
    X = rng.standard_normal((K, R.shape[0] if transpose else R.shape[1]))
    got = _cm(R, X, transpose, normalize)
    assert np.array_equal(got, O.apply(X, transpose=transpose, normalize=normalize))


@pytest.mark.parametrize("K", [5, 128])
def test_cell_major_fp64_adjoint_matches_one_field(c1, K):
    import torch

    R, _ = c1
    rng = np.random.default_rng(7)
    G = rng.standard_normal((K, R.shape[0]))
    g = torch.from_numpy(np.ascontiguousarray(G.T)).cuda()
    out = torch.full((R.shape[1], K), float("nan"), dtype=torch.float64, device="cuda")
    regrid_adjoint_(out, R, g, dims=1)
    for k in range(K):
        one = torch.empty(R.shape[1], dtype=torch.float64, device="cuda")
        regrid_adjoint_(one, R, torch.from_numpy(G[k]).cuda())
        assert torch.equal(out[:, k], one), k


@pytest.fixture(scope="module")
def large(cuda):
    hp, ll = workloads.large()
    return hp, ll, Regridder(hp, ll, normalize=True), oracle.OracleRegridder(hp, ll, normalize=True)


@pytest.mark.parametrize("K", [8, 24, 128])
def test_large_fields_fp64(large, K):
    """The large configuration's polar rows (hundreds of entries) at 8 and 24
    fields, which run the batched-entry candidates of the row kernel, and at
    128."""
    import torch

    hp, ll, R, O = large
    dev = torch.device("cuda", 0)
    for transpose, g in ((False, ll), (True, hp)):
        x = workloads.harmonic_fields(workloads.cell_centres(g), K, 16, 3 + transpose, 0.1, dev).double()
        y = torch.empty((R.shape[1] if transpose else R.shape[0], K), dtype=torch.float64, device=dev)
        regrid_(y, R.transpose() if transpose else R, x.T.contiguous(), dims=1)
        pick = np.arange(0, K, max(1, K // 8))
        ref = O.apply(x[pick].cpu().numpy(), transpose=transpose)
        assert np.array_equal(y[:, pick].T.cpu().numpy(), ref)
