"""Batches of regridders: crg_build_batch (concurrent builds) must give the
same matrices as one-at-a-time builds, and an ApplyPlan (one CUDA graph for
the applies of a whole batch) the same fields as one-at-a-time applies --
bit for bit, since both run the same kernels.  The pairs follow the batched
workload: jittered global lon-lat grids of uneven resolutions (cells moved by
U(-0.2, 0.2) widths, convex), plus a HEALPix and a cubed-sphere pair."""
from __future__ import annotations

import numpy as np
import pytest

from crg import ApplyPlan, ArgumentError, Regridder, build_batch, grids, regrid_, regrid_batch_

pytestmark = pytest.mark.gpu


def _jittered(rng, res):
    nx, ny = int(round(360.0 / res)), int(round(180.0 / res))
    while True:
        g = grids.lonlat_jittered(nx, ny, 0.2, int(rng.integers(1 << 31)))
        if grids.convex_cells(g).all():
            return g


@pytest.fixture(scope="module")
def pairs(cuda):
    rng = np.random.default_rng(33)
    out = []
    for _ in range(6):
        r = np.exp(rng.uniform(np.log(2.0), np.log(8.0), size=2))
        out.append((_jittered(rng, r[0]), _jittered(rng, r[1])))
    out.append((grids.healpix_grid(16), grids.lonlat_regular(3.0, 3.0)))
    out.append((grids.lonlat_regular(5.0, 5.0), grids.cubed_sphere(12, jitter=0.1, seed=2)))
    return out


def test_build_batch_equals_single_builds(pairs):
    batch = build_batch(pairs, normalize=True, nthreads=4)
    assert len(batch) == len(pairs)
    for (dst, src), Rb in zip(pairs, batch):
        Rs = Regridder(dst, src, normalize=True)
        for a, b in zip(Rb.csc_arrays(), Rs.csc_arrays()):
            assert np.array_equal(a, b)
        assert np.array_equal(Rb.dst_areas, Rs.dst_areas) and np.array_equal(Rb.src_areas, Rs.src_areas)
        assert Rb.info["normalizer"] == Rs.info["normalizer"]


def test_build_batch_failure_releases_everything(pairs):
    # a 9-gon: more vertices than the library's cells take (max_verts 3..8)
    t = np.linspace(0.0, 2.0 * np.pi, 10)[:-1]
    bad = grids.Grid("cells", grids.PLANAR, cells=np.stack([np.cos(t), np.sin(t)], axis=1)[None])
    with pytest.raises(ArgumentError, match="pair 1"):
        build_batch([pairs[0], (bad, bad), pairs[1]], nthreads=2)


def test_apply_plan_equals_single_applies(pairs):
    import torch

    Rs = build_batch(pairs, normalize=True)
    gen = torch.Generator(device="cuda").manual_seed(8)
    specs = [(1, torch.float64, 1), (40, torch.float32, 1), (7, torch.float32, 2), (64, torch.bfloat16, 1),
             (128, torch.float32, 1), (3, torch.float64, 2), (33, torch.float32, 1), (256, torch.float32, 1)]
    items, refs = [], []
    for k, ((K, dt, dims), R) in enumerate(zip(specs, Rs)):
        RR = R.transpose() if k % 3 == 2 else R
        n_out, n_in = RR.shape
        if K == 1:
            shape_in, shape_out = (n_in,), (n_out,)
        elif dims == 1:
            shape_in, shape_out = (n_in, K), (n_out, K)
        else:
            shape_in, shape_out = (K, n_in), (K, n_out)
        x = torch.randn(shape_in, generator=gen, device="cuda").to(dt)
        y = torch.full(shape_out, float("nan"), device="cuda").to(dt)
        items.append((y, RR, x, dims))
        refs.append((RR, x, dims))
    plan = ApplyPlan(items)
    for round_ in range(2):
        if round_:  # new values in the same buffers: the replay reads them
            for _, _, x, _ in items:
                x.copy_(torch.randn(x.shape, generator=gen, device="cuda").to(x.dtype))
        plan.launch()
        torch.cuda.synchronize()
        for (y, _, _, _), (RR, x, dims) in zip(items, refs):
            expect = torch.empty_like(y)
            regrid_(expect, RR, x, dims=dims)
            torch.cuda.synchronize()
            assert torch.equal(y, expect)


def test_apply_plan_rejects_host_fields(pairs):
    import torch

    R = Regridder(*pairs[-1])
    with pytest.raises(ArgumentError):
        ApplyPlan([(torch.zeros(R.shape[0]), R, torch.zeros(R.shape[1]))])


def test_regrid_batch_equals_single_applies(pairs):
    """crg_apply_batch: host (numpy, pinned torch) and CUDA fields, R and
    transpose(R) of the same handle at once (separate staging per direction),
    bit for bit the single applies."""
    import torch

    Rs = build_batch(pairs[:4], normalize=True)
    rng = np.random.default_rng(5)
    items, refs = [], []
    for k, R in enumerate(Rs):
        for RR in (R, R.transpose()):
            n_out, n_in = RR.shape
            K = 1 + 37 * k
            x = rng.standard_normal((n_in, K)).astype(np.float32)
            if k % 3 == 0:
                src, dst = x, np.full((n_out, K), np.nan, np.float32)
            elif k % 3 == 1:
                src = torch.from_numpy(x).pin_memory()
                dst = torch.full((n_out, K), float("nan")).pin_memory()
            else:
                src, dst = torch.from_numpy(x).cuda(), torch.full((n_out, K), float("nan"), device="cuda")
            items.append((dst, RR, src, 1))
            refs.append((RR, x))
    regrid_batch_(items, nthreads=3)
    torch.cuda.synchronize()
    for (dst, _, _, _), (RR, x) in zip(items, refs):
        expect = np.empty((RR.shape[0], x.shape[1]), np.float32)
        regrid_(expect, RR, x)
        got = dst.cpu().numpy() if hasattr(dst, "cpu") else dst
        assert np.array_equal(got, expect)


def test_regrid_batch_names_the_failing_item(pairs):
    R = Regridder(*pairs[0])
    good = (np.zeros(R.shape[0]), R, np.ones(R.shape[1]))
    bad = (np.zeros(R.shape[0] + 1), R, np.ones(R.shape[1]))
    with pytest.raises(Exception, match="item 1|cells"):
        regrid_batch_([good, bad])


@pytest.mark.parametrize("same_copy", [False, True])
def test_regrid_batch_host_pipeline(pairs, same_copy):
    """Host fields in every item: one chunk pipeline over the items (distinct
    matrix copies), or threads when a matrix copy repeats; bit for bit the
    single applies either way, cell-major and field-major."""
    import torch

    R1, R2 = build_batch(pairs[6:8], normalize=True)
    rng = np.random.default_rng(9)
    specs = [(R1, 1), (R1.transpose(), 2), (R2, 1)] if not same_copy else [(R1, 1), (R1, 2)]
    items, refs = [], []
    for RR, dims in specs:
        n_out, n_in = RR.shape
        K = 160
        x = rng.standard_normal((n_in, K) if dims == 1 else (K, n_in)).astype(np.float32)
        src = torch.from_numpy(x).pin_memory()
        dst = torch.full((n_out, K) if dims == 1 else (K, n_out), float("nan")).pin_memory()
        items.append((dst, RR, src, dims))
        refs.append((RR, x, dims))
    regrid_batch_(items)
    for (dst, _, _, _), (RR, x, dims) in zip(items, refs):
        expect = np.empty(dst.shape, np.float32)
        regrid_(expect, RR, x, dims=dims)
        assert np.array_equal(dst.numpy(), expect)


@pytest.mark.parametrize("normalize", [True, False])
def test_apply_plan_persistent_launch(pairs, normalize, monkeypatch):
    """With CRG_PLAN_BATCH=all, one persistent launch (plus one for cut and
    empty rows per field type) runs every single-field FP32 / BF16 item and
    every cell-major one of 32 fields or more (2 to 31 fields keep their own
    applies on the narrow merge-path kernel): field
    counts on both sides of the merge-path threshold (32), aligned or not
    (K % 4), R and transpose(R), a regridder with empty rows; FP64 and
    field-major items stay their own applies.  Bit for bit the single applies."""
    import torch

    Rs = build_batch(pairs, normalize=True)
    # a destination partly outside the source (rows without entries in R)
    part = Regridder(grids.lonlat_grid(np.arange(0.0, 361.0, 10.0), np.arange(-90.0, 91.0, 10.0)),
                     grids.lonlat_grid(np.arange(0.0, 181.0, 6.0), np.arange(-30.0, 31.0, 6.0)), normalize=True)
    gen = torch.Generator(device="cuda").manual_seed(12)
    specs = [(1, torch.float32, 1), (3, torch.float32, 1), (7, torch.bfloat16, 1), (12, torch.float32, 1),
             (32, torch.float32, 1), (33, torch.float32, 1), (100, torch.float32, 1), (128, torch.bfloat16, 1),
             (200, torch.float32, 1), (512, torch.float32, 1), (64, torch.float64, 1), (20, torch.float32, 2)]
    regs = [R if k % 2 == 0 else R.transpose() for k, R in enumerate(Rs)] + [part, part.transpose()]
    items, expect_batched = [], 0
    for k, (K, dt, dims) in enumerate(specs + specs[:2]):
        RR = regs[k % len(regs)] if k < len(specs) else regs[len(Rs) + k - len(specs)]
        n_out, n_in = RR.shape
        shape_in, shape_out = ((n_in, K), (n_out, K)) if dims == 1 else ((K, n_in), (K, n_out))
        if K == 1:
            shape_in, shape_out = (n_in,), (n_out,)
        x = torch.randn(shape_in, generator=gen, device="cuda").to(dt)
        y = torch.full(shape_out, float("nan"), device="cuda").to(dt)
        items.append((y, RR, x, dims))
        # 2 to 31 fields run k_cm_narrow in their own apply
        expect_batched += dt != torch.float64 and (K == 1 or (dims == 1 and K >= 32))
    monkeypatch.setenv("CRG_PLAN_BATCH", "all")  # every item the persistent launch can run
    plan = ApplyPlan(items, normalize=normalize)
    monkeypatch.delenv("CRG_PLAN_BATCH")
    info = plan.info
    assert info["batched_items"] == expect_batched
    for _ in range(2):
        for y, _, _, _ in items:
            y.fill_(float("nan"))
        plan.launch()
        torch.cuda.synchronize()
        for y, RR, x, dims in items:
            ref = torch.empty_like(y)
            regrid_(ref, RR, x, dims=dims, normalize=normalize)
            torch.cuda.synchronize()
            assert torch.equal(y, ref), (tuple(y.shape), y.dtype)
