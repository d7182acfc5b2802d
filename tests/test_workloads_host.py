"""The synthetic workloads on CPU: the five configurations' grids have the
sizes the benchmark and the parity tests quote, the batched case draws its 32
pairs and field counts from the stated distributions (seeded, so the GPU
tests and the bench see the same pairs), and the spherical-harmonic fields are
band-limited as stated."""
from __future__ import annotations

import itertools

import numpy as np
import pytest

from crg import workloads


def test_configuration_sizes():
    assert [g.ncells for g in workloads.small_fp64()] == [120 * 60, 180 * 90]
    assert [g.ncells for g in workloads.precision()] == [360 * 180, 6 * 48 * 48]
    assert [g.ncells for g in workloads.derivatives()] == [6 * 96 * 96, 360 * 180]
    assert [g.ncells for g in workloads.large()] == [12 * 256 * 256, 1440 * 720]


def test_batch_pairs_follow_their_distributions():
    pairs, ks = workloads.batch_pairs()
    assert len(pairs) == len(ks) == 32
    cells = [g.ncells for p in pairs for g in p]
    assert (min(cells), max(cells), sum(ks)) == (4_232, 331_298, 2_669)
    assert all(1 <= k <= 512 for k in ks)
    for g in itertools.chain.from_iterable(pairs):
        # global lon-lat of r = 0.4..4 degrees: round(360 / r) columns, round(180 / r) rows
        ny, nx = g.blocks[0].shape[0] - 1, g.blocks[0].shape[1] - 1
        assert nx * ny == g.ncells and 90 <= nx <= 900 and 45 <= ny <= 450 and abs(nx - 2 * ny) <= 1
    again, ks2 = workloads.batch_pairs()
    assert ks2 == ks and [g.ncells for p in again for g in p] == cells


def _monomials(x, deg):
    cols = [np.ones(len(x))]
    for d in range(1, deg + 1):
        for a in range(d + 1):
            for b in range(d + 1 - a):
                c = d - a - b
                cols.append(x[:, 0] ** a * x[:, 1] ** b * x[:, 2] ** c)
    return np.stack(cols, axis=1)


@pytest.mark.parametrize("lmax", [0, 1, 3])
def test_harmonic_fields_are_band_limited(lmax):
    """Without noise, a field of degree <= lmax is a polynomial of degree <=
    lmax in (x, y, z) on the sphere: least squares on those monomials leaves a
    rounding-level residual (and lmax = 0 is the constant c00 Ybar00)."""
    pytest.importorskip("torch")
    rng = np.random.default_rng(1)
    x = rng.standard_normal((400, 3))
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    f = workloads.harmonic_fields(x, 3, lmax, seed=5, noise=0.0, device="cpu").double().numpy()
    assert f.shape == (3, 400)
    M = _monomials(x, lmax)
    coef, *_ = np.linalg.lstsq(M, f.T, rcond=None)
    resid = np.abs(M @ coef - f.T).max() / np.abs(f).max()
    assert resid < 1e-6  # the fields are returned in FP32
    if lmax == 0:
        assert np.all(f == f[:, :1])
    g = workloads.harmonic_fields(x, 3, lmax, seed=5, noise=0.0, device="cpu")
    assert np.array_equal(g.numpy(), f.astype(np.float32))
