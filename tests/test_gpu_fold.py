"""Folded (tripolar) grids on the GPU: with the fold-row partner slots as
ghosts the build matches the oracle bit for bit in both directions, ghost
slots get no entries, and regridding onto the folded grid followed by the
fold mirror (device kernel) reproduces constants in every slot, as the
reference's finalize_regridding! for Oceananigans fields does."""
from __future__ import annotations

import numpy as np
import oracle
import pytest
from test_gpu_parity import assert_parity

from crg import Regridder, grids, mirror_fold_, regrid_

pytestmark = pytest.mark.gpu

NX, NY = 96, 40


@pytest.mark.parametrize("direction", ["folded_source", "folded_destination"])
def test_folded_grid_parity_and_mirror(cuda, direction):
    import torch

    gh = grids.fold_ghosts(grids.folded_lonlat(NX, NY, 70.0))
    other = grids.healpix_grid(16)
    dst, src = (other, gh) if direction == "folded_source" else (gh, other)
    R = Regridder(dst, src, normalize=True)
    O = oracle.OracleRegridder(dst, src, normalize=True)
    assert_parity(R, O)
    ghosts = np.flatnonzero(gh.nverts == 0)
    if direction == "folded_source":
        assert np.all(np.diff(R.csc_arrays()[0])[ghosts] == 0)
        y = torch.empty((dst.ncells, 40), device="cuda")
        regrid_(y, R, torch.ones((src.ncells, 40), device="cuda"))
        assert torch.allclose(y, torch.ones_like(y), atol=1e-5)
        return
    assert R.info["empty_rows"][0] == len(ghosts)
    for layout in ("cell_major", "field_major"):
        if layout == "cell_major":
            y = torch.full((dst.ncells, 40), float("nan"), device="cuda")
            regrid_(y, R, torch.ones((src.ncells, 40), device="cuda"), dims=1)
            mirror_fold_(y, NX, NY, dims=1)
        else:
            y = torch.full((40, dst.ncells), float("nan"), device="cuda")
            regrid_(y, R, torch.ones((40, src.ncells), device="cuda"), dims=2)
            mirror_fold_(y, NX, NY, dims=2)
        assert torch.allclose(y, torch.ones_like(y), atol=1e-5), layout
    # FP64, one field: ghost slots are 0/0 before the mirror, the partner's value after it
    s = np.random.default_rng(9).standard_normal(src.ncells)
    d = torch.zeros(dst.ncells, dtype=torch.float64, device="cuda")
    regrid_(d, R, torch.from_numpy(s).cuda())
    assert torch.isnan(d[torch.from_numpy(ghosts).cuda()]).all()
    mirror_fold_(d, NX, NY)
    ref = O.apply(s)
    mirror_fold_(ref, NX, NY)
    assert np.array_equal(d.cpu().numpy(), ref)
