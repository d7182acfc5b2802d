"""GPU parity: the CUDA build and apply against the CPU oracle, through the
C ABI.  Nonzero patterns must be bit-exact; the FP64 clip/area arithmetic is a
fixed operation sequence, so areas are expected bit-identical and are held to
1e-12 relative at worst; FP64 apply follows the reference's summation order.
"""
from __future__ import annotations

import json

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, c1_grids
from crg import Regridder, grids, regrid, regrid_, regrid_adjoint_
from crg.regridder import ArgumentError, DimensionMismatch

pytestmark = pytest.mark.gpu

AREA_RTOL = 1e-12


def assert_parity(R, O, exact=True):
    colptr, rowval, nzval = R.csc_arrays()
    assert R.nnz == O.nnz
    assert np.array_equal(colptr, O.colptr), "column pointers differ"
    assert np.array_equal(rowval, O.rowval), "row indices differ"
    scale = np.maximum(np.abs(O.nzval), 1e-300)
    assert np.max(np.abs(nzval - O.nzval) / scale, initial=0) <= AREA_RTOL
    assert np.allclose(R.dst_areas, O.dst_areas, rtol=AREA_RTOL, atol=0)
    assert np.allclose(R.src_areas, O.src_areas, rtol=AREA_RTOL, atol=0)
    if exact:
        assert np.array_equal(nzval, O.nzval), "areas are not bit-identical"
        assert np.array_equal(R.dst_areas, O.dst_areas) and np.array_equal(R.src_areas, O.src_areas)


def test_readme_known_answer_gpu(cuda):
    g = json.loads((GOLDEN / "readme_planar.json").read_text())["readme"]
    R = Regridder(grids.polygon_grid(g["dst"]), grids.polygon_grid(g["src"]), normalize=False)
    assert np.array_equal(R.intersections.toarray(), np.array(g["matrix"]))
    assert np.array_equal(R.src_areas, g["src_areas"]) and np.array_equal(R.dst_areas, g["dst_areas"])


def test_simple_jl_exact_conservation_gpu(cuda):
    g = json.loads((GOLDEN / "readme_planar.json").read_text())["simple_jl"]
    R = Regridder(grids.polygon_grid(g["dst"]), grids.polygon_grid(g["src"]), normalize=False)
    A = R.intersections
    assert np.array_equal(np.asarray(A.sum(axis=1)).ravel(), R.dst_areas)
    assert np.array_equal(np.asarray(A.sum(axis=0)).ravel(), R.src_areas)
    v2 = np.array(g["values_on_src"], float)
    v1 = np.zeros(4)
    regrid_(v1, R, v2)
    assert np.sum(v1 * R.dst_areas) == np.sum(v2 * R.src_areas)
    back = np.zeros(5)
    regrid_(back, R.transpose(), v1)
    assert np.sum(back * R.src_areas) == np.sum(v2 * R.src_areas)


CASES = {
    "C1_lonlat2_to_lonlat3_shifted": c1_grids,
    "lonlat4_to_healpix16": lambda: (grids.healpix_grid(16), grids.lonlat_regular(4.0, 4.0)),
    "healpix16_to_lonlat4": lambda: (grids.lonlat_regular(4.0, 4.0), grids.healpix_grid(16)),
    "lonlat4_to_healpix8_ring": lambda: (grids.healpix_grid(8, "ring"), grids.lonlat_regular(4.0, 4.0)),
    "lonlat4_to_cs12": lambda: (grids.cubed_sphere(12), grids.lonlat_regular(4.0, 4.0)),
    "cs8_to_lonlat5": lambda: (grids.lonlat_regular(5.0, 5.0), grids.cubed_sphere(8)),
    "jittered_lonlat": lambda: (grids.lonlat_jittered(60, 30, 0.2, 3), grids.lonlat_jittered(90, 45, 0.2, 4)),
    "jittered_cs_to_lonlat2": lambda: (grids.cubed_sphere(16, jitter=0.15, seed=5), grids.lonlat_regular(2.0, 2.0)),
    "coincident_lonlat4_lonlat2": lambda: (grids.lonlat_regular(4.0, 4.0), grids.lonlat_regular(2.0, 2.0)),
    "identical_healpix8": lambda: (grids.healpix_grid(8), grids.healpix_grid(8)),
    # RingGrids full grids (cells numbered ring by ring from the north) and a permuted numbering
    "full_clenshaw12_to_full_gaussian16": lambda: (grids.full_gaussian_grid(16), grids.full_clenshaw_grid(12)),
    "reordered_lonlat5_to_healpix8": lambda: (grids.healpix_grid(8), grids.reorder_cells(
        grids.lonlat_regular(5.0, 5.0), np.random.default_rng(5).permutation(72 * 36))),
    # rows of ~400 and ~8,100 entries: the shared-memory and global-memory row sorts
    "lonlat10_from_lonlat0.5": lambda: (grids.lonlat_regular(10.0, 10.0), grids.lonlat_regular(0.5, 0.5)),
    "lonlat45_from_lonlat0.5": lambda: (grids.lonlat_regular(45.0, 45.0), grids.lonlat_regular(0.5, 0.5)),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("normalize", [False, True])
def test_build_parity(cuda, name, normalize):
    dst, src = CASES[name]()
    R = Regridder(dst, src, normalize=normalize)
    O = oracle.OracleRegridder(dst, src, normalize=normalize)
    assert R.info["clip_overflows"] == 0
    assert_parity(R, O)


def test_planar_regular_grids(cuda):
    """Planar RegularGrid on both sides (test/regridding.jl:131-211 style)."""
    dst = grids.regular_grid(np.linspace(0, 1, 9), np.linspace(0, 1, 9))
    src = grids.regular_grid(np.linspace(0, 1, 5), np.linspace(0, 1, 5))
    R = Regridder(dst, src)
    O = oracle.OracleRegridder(dst, src)
    assert_parity(R, O)
    s = np.arange(1.0, 17.0)
    d = np.zeros(64)
    regrid_(d, R, s)
    assert np.array_equal(d, O.apply(s))


def test_empty_and_tiny(cuda):
    # no overlap at all: empty matrix, zero output
    a = grids.polygon_grid([[(0, 0), (1, 0), (1, 1), (0, 1)]])
    b = grids.polygon_grid([[(5, 5), (6, 5), (6, 6), (5, 6)], [(2, 2), (3, 2), (3, 3)]])
    R = Regridder(a, b)
    assert R.nnz == 0 and R.intersections.shape == (1, 2)
    d = np.full(1, 7.0)
    regrid_(d, R, np.array([1.0, 2.0]), normalize=False)
    assert d[0] == 0.0
    # one spherical cell on each side
    one = grids.lonlat_grid([0.0, 10.0], [0.0, 10.0])
    R1 = Regridder(one, one)
    O1 = oracle.OracleRegridder(one, one)
    assert_parity(R1, O1)


# ----------------------------------------------------------------- apply

@pytest.fixture(scope="module")
def c1(cuda):
    dst, src = c1_grids()
    return Regridder(dst, src, normalize=True), oracle.OracleRegridder(dst, src, normalize=True)


def test_apply_f64_bit_exact(c1):
    """regrid! in FP64: the reference's column-scatter mul! then ./ a_d; the
    row gather accumulates in the same order, so results are bit-identical."""
    R, O = c1
    rng = np.random.default_rng(11)
    s = rng.random(R.shape[1])
    d = np.zeros(R.shape[0])
    regrid_(d, R, s)
    assert np.array_equal(d, O.apply(s))
    # transpose(R) shares the matrices
    g = rng.random(R.shape[0])
    back = np.zeros(R.shape[1])
    regrid_(back, R.transpose(), g)
    assert np.array_equal(back, O.apply(g, transpose=True))
    # without normalisation
    regrid_(d, R, s, normalize=False)
    assert np.array_equal(d, O.apply(s, normalize=False))


def test_apply_f64_many_fields_layouts(c1):
    import torch

    R, O = c1
    rng = np.random.default_rng(12)
    K = 7
    S = rng.random((K, R.shape[1]))
    ref = O.apply(S)
    # field-major (dims=2 over a (K, N) array) on the device
    st = torch.from_numpy(S).cuda()
    dt = torch.zeros((K, R.shape[0]), dtype=torch.float64, device="cuda")
    regrid_(dt, R, st, dims=2)
    assert np.array_equal(dt.cpu().numpy(), ref)
    # cell-major (dims=1 over an (N, K) array) on the host
    Sc = np.ascontiguousarray(S.T)
    Dc = np.zeros((R.shape[0], K))
    regrid_(Dc, R, Sc, dims=1)
    assert np.array_equal(Dc.T, ref)


@pytest.mark.parametrize("dtype,tol", [("float32", 1e-5), ("bfloat16", 2e-2)])
@pytest.mark.parametrize("layout", ["cell_major", "field_major"])
def test_apply_low_precision(c1, dtype, tol, layout):
    """FP32 weights, FP32/BF16 fields, FP32 accumulation against the FP64 oracle:
    max abs error relative to max|d| and the relative error of the conserved
    area-weighted mean."""
    import torch

    R, O = c1
    K = 64
    rng = np.random.default_rng(13)
    S = rng.random((K, R.shape[1]))
    ref = O.apply(S)
    tdt = getattr(torch, dtype)
    if layout == "field_major":
        st = torch.from_numpy(S).to("cuda", tdt)
        dt = torch.zeros((K, R.shape[0]), dtype=tdt, device="cuda")
        regrid_(dt, R, st, dims=2)
        got = dt.double().cpu().numpy()
    else:
        st = torch.from_numpy(np.ascontiguousarray(S.T)).to("cuda", tdt)
        dt = torch.zeros((R.shape[0], K), dtype=tdt, device="cuda")
        regrid_(dt, R, st, dims=1)
        got = dt.double().cpu().numpy().T
    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    assert err <= tol
    if dtype == "float32":
        cons_ref = ref @ R.dst_areas
        cons = got @ R.dst_areas
        assert np.max(np.abs(cons - cons_ref) / np.abs(cons_ref)) <= 1e-6


def test_apply_device_equals_host(c1):
    import torch

    R, O = c1
    rng = np.random.default_rng(14)
    S = rng.standard_normal((3, R.shape[1])).astype(np.float32)
    host = np.zeros((3, R.shape[0]), np.float32)
    regrid_(host, R, S, dims=2)
    dev = torch.zeros((3, R.shape[0]), dtype=torch.float32, device="cuda")
    regrid_(dev, R, torch.from_numpy(S).cuda(), dims=2)
    assert np.array_equal(host, dev.cpu().numpy())


def test_constant_field_preserved(cuda):
    """test/usecases/constant_field.jl:41-77 and fullclenshaw.jl:19-31: ones stay
    ones on covered cells, forward and via transpose."""
    for dst, src in [(grids.healpix_grid(16), grids.lonlat_regular(4.0, 4.0)),
                     (grids.cubed_sphere(12), grids.lonlat_jittered(90, 45, 0.2, 9))]:
        R = Regridder(dst, src, normalize=True)
        d = regrid(R, np.ones(R.shape[1]))
        assert np.max(np.abs(d - 1)) < 1e-10
        s = regrid(R.transpose(), np.ones(R.shape[0]))
        assert np.max(np.abs(s - 1)) < 1e-10


def test_nd_dims_semantics(c1):
    """N-D regrid! (test/regridding.jl:127-203): every slice along the other
    axes equals the 1-D result; dims selects the spatial axis."""
    R, O = c1
    ns, nd = R.shape[1], R.shape[0]
    rng = np.random.default_rng(15)
    s3 = rng.random((3, ns, 2))
    d3 = np.zeros((3, nd, 2))
    regrid_(d3, R, s3, dims=2)
    for a in range(3):
        for b in range(2):
            assert np.array_equal(d3[a, :, b], O.apply(s3[a, :, b]))
    with pytest.raises(ArgumentError):
        regrid_(d3, R, s3, dims=4)
    with pytest.raises(DimensionMismatch):
        regrid_(np.zeros((3, nd, 3)), R, s3, dims=2)


def test_strided_vector_routes(c1):
    """test/regridding.jl:131-211: dense and strided vectors give the same
    result (==), strided ones through the regridder's temporaries."""
    R, O = c1
    ns, nd = R.shape[1], R.shape[0]
    s = np.random.default_rng(16).random(ns)
    ref = np.zeros(nd)
    regrid_(ref, R, s)
    big_s = np.zeros(2 * ns)
    big_s[::2] = s
    big_d = np.zeros(2 * nd)
    R.src_temp[:] = np.nan
    R.dst_temp[:] = np.nan
    regrid_(big_d[::2], R, big_s[::2])
    assert np.array_equal(big_d[::2], ref)
    assert not np.isnan(R.src_temp).any() and not np.isnan(R.dst_temp).any()


def test_adjoint_dot_product(c1):
    """<W s, g> == <s, W^T g> for the normalised forward map and for transpose(R)."""
    R, O = c1
    rng = np.random.default_rng(17)
    for RR in (R, R.transpose()):
        s = rng.standard_normal(RR.shape[1])
        g = rng.standard_normal(RR.shape[0])
        d = regrid(RR, s)
        gs = np.zeros(RR.shape[1])
        regrid_adjoint_(gs, RR, g)
        lhs, rhs = d @ g, s @ gs
        assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)


def test_transpose_shares_handle(c1):
    R, _ = c1
    T = R.transpose()
    assert T.src_areas is R.dst_areas and T.dst_areas is R.src_areas
    assert T.src_temp is R.dst_temp and T.dst_temp is R.src_temp
    assert T.shape == (R.shape[1], R.shape[0])
    assert (T.intersections != R.intersections.T).nnz == 0
    del R  # the view keeps the handle alive
    assert T.transpose().nnz == T.nnz


BATCHED_CASES = {
    # fine destination over coarse source: short rows, none cut
    "healpix32_from_lonlat3": lambda: (grids.healpix_grid(32), grids.lonlat_regular(3.0, 3.0)),
    # coarse destination over a fine source: long rows cut across tasks
    "lonlat20_from_lonlat0.5": lambda: (grids.lonlat_regular(20.0, 20.0), grids.lonlat_regular(0.5, 0.5)),
    "cs6_from_healpix64": lambda: (grids.cubed_sphere(6), grids.healpix_grid(64)),
    # global destination over a regional source: destination rows without entries
    "lonlat5_from_regional1": lambda: (grids.lonlat_regular(5.0, 5.0),
                                       grids.lonlat_grid(np.arange(10.5, 51.0, 1.0), np.arange(-20.5, 31.0, 1.0))),
}


@pytest.mark.parametrize("case", list(BATCHED_CASES))
@pytest.mark.parametrize("K,layout,dtype", [(128, "cell_major", "float32"), (200, "cell_major", "float32"),
                                            (40, "cell_major", "bfloat16"), (128, "field_major", "float32"),
                                            (37, "field_major", "bfloat16"), (16, "field_major", "float32")])
def test_apply_batched_paths(cuda, case, K, layout, dtype):
    """Batched FP32/BF16 SpMM (merge-path cell-major, row kernels, field-major
    through transposes) against the FP64 oracle, forward, transpose and adjoint."""
    import torch

    dst, src = BATCHED_CASES[case]()
    R = Regridder(dst, src, normalize=True)
    O = oracle.OracleRegridder(dst, src, normalize=True)
    # FP32 accumulation over rows of up to ~1600 entries (20-degree cells over 0.5 degrees)
    tol = 1e-5 if dtype == "float32" else 2e-2
    tdt = getattr(torch, dtype)
    rng = np.random.default_rng(21)
    for transpose in (False, True):
        RR = R.transpose() if transpose else R
        nin, nout = RR.shape[1], RR.shape[0]
        S = rng.standard_normal((K, nin))
        Sq = torch.from_numpy(S).to(tdt)  # the values the GPU sees
        ref = O.apply(Sq.double().numpy(), transpose=transpose)
        # NaN-filled outputs: every row, with entries or without, must be written
        if layout == "field_major":
            x = Sq.cuda()
            y = torch.full((K, nout), float("nan"), dtype=tdt, device="cuda")
            regrid_(y, RR, x, dims=2)
            got = y.double().cpu().numpy()
        else:
            x = Sq.T.contiguous().cuda()
            y = torch.full((nout, K), float("nan"), dtype=tdt, device="cuda")
            regrid_(y, RR, x, dims=1)
            got = y.double().cpu().numpy().T
        err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
        assert err <= tol, (transpose, err)
    # adjoint in FP32/BF16 against the dense transpose of the normalised map
    A = R.intersections.tocsr()
    W = A.multiply(1.0 / R.dst_areas[:, None]).tocsr()
    G = rng.standard_normal((K, R.shape[0]))
    Gq = torch.from_numpy(G).to(tdt)
    ref = (W.T @ Gq.double().numpy().T).T
    if layout == "field_major":
        y = torch.zeros((K, R.shape[1]), dtype=tdt, device="cuda")
        regrid_adjoint_(y, R, Gq.cuda(), dims=2)
        got = y.double().cpu().numpy()
    else:
        y = torch.zeros((R.shape[1], K), dtype=tdt, device="cuda")
        regrid_adjoint_(y, R, Gq.T.contiguous().cuda(), dims=1)
        got = y.double().cpu().numpy().T
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) <= tol


@pytest.mark.parametrize("K,layout", [(128, "cell_major"), (200, "cell_major"), (8, "field_major"),
                                      (130, "cell_strided")])
def test_host_pipeline_matches_device(cuda, K, layout):
    """Host fields go through the chunked copy/apply/copy pipeline; the result
    equals the apply on device fields (bit for bit where every chunk runs the
    device path's kernel, within FP32 rounding where a short last chunk takes
    another one), and a strided host destination keeps its other elements."""
    import torch

    R = Regridder(grids.healpix_grid(32), grids.lonlat_regular(2.0, 2.0), normalize=True)
    nd, ns = R.shape
    rng = np.random.default_rng(K)
    if layout == "field_major":
        S = rng.standard_normal((K, ns)).astype(np.float32)
        host = np.zeros((K, nd), np.float32)
        regrid_(host, R, S, dims=2)
        dev = torch.zeros((K, nd), device="cuda")
        regrid_(dev, R, torch.from_numpy(S).cuda(), dims=2)
        got, ref = host, dev.cpu().numpy()
    else:
        S = rng.standard_normal((ns, K)).astype(np.float32)
        if layout == "cell_strided":
            big = np.full((nd, K + 6), 7.0, np.float32)
            host = big[:, 3:3 + K]
        else:
            host = np.zeros((nd, K), np.float32)
        regrid_(host, R, S, dims=1)
        dev = torch.zeros((nd, K), device="cuda")
        regrid_(dev, R, torch.from_numpy(S).cuda(), dims=1)
        got, ref = host, dev.cpu().numpy()
        if layout == "cell_strided":
            assert np.all(big[:, :3] == 7.0) and np.all(big[:, 3 + K:] == 7.0)
    if K == 128 or layout == "field_major":
        assert np.array_equal(got, ref)
    else:
        assert np.max(np.abs(got - ref)) <= 1e-6 * np.max(np.abs(ref))


@pytest.mark.parametrize("dtype,tol", [("float32", 1e-5), ("bfloat16", 2e-2)])
def test_field_major_both_kernels(cuda, dtype, tol):
    """Field-major fields with >= 32 fields: the first apply of a direction
    times the row kernel and the transposes around the cell-major kernel and
    keeps the faster; every apply (the timed first one and the later ones)
    matches the FP64 oracle."""
    import torch

    dst, src = grids.healpix_grid(64), grids.lonlat_regular(1.0, 1.0)
    R = Regridder(dst, src, normalize=True)
    O = oracle.OracleRegridder(dst, src, normalize=True)
    tdt = getattr(torch, dtype)
    rng = np.random.default_rng(64)
    for transpose in (False, True):
        RR = R.transpose() if transpose else R
        K = 45  # not a multiple of 4: the transposed copy pads to 48
        Sq = torch.from_numpy(rng.standard_normal((K, RR.shape[1]))).to(tdt)
        ref = O.apply(Sq.double().numpy(), transpose=transpose)
        for _ in range(3):
            y = torch.full((K, RR.shape[0]), float("nan"), dtype=tdt, device="cuda")
            regrid_(y, RR, Sq.cuda(), dims=2)
            err = np.max(np.abs(y.double().cpu().numpy() - ref)) / np.max(np.abs(ref))
            assert err <= tol, (transpose, err)


def test_concurrent_applies_on_two_streams(cuda):
    """One handle applied at the same time from two host threads on two
    streams (read-only matrices, per-call temporaries) gives each thread the
    result of a lone apply."""
    import threading

    import torch

    R = Regridder(grids.healpix_grid(64), grids.lonlat_regular(1.0, 1.0), normalize=True)
    nd, ns = R.shape
    gen = torch.Generator(device="cuda").manual_seed(4)
    xs = [torch.randn((ns, 64), generator=gen, device="cuda") for _ in range(2)]
    refs = []
    for x in xs:
        y = torch.empty((nd, 64), device="cuda")
        regrid_(y, R, x)
        refs.append(y)
    torch.cuda.synchronize()
    outs = [torch.empty((nd, 64), device="cuda") for _ in range(2)]
    errors = []

    def work(k):
        try:
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                for _ in range(20):
                    regrid_(outs[k], R, xs[k], stream=s)
            s.synchronize()
        except Exception as e:  # surfaced below
            errors.append(e)

    threads = [threading.Thread(target=work, args=(k,)) for k in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for y, ref in zip(outs, refs):
        assert torch.equal(y, ref)


def _kahan_segments(indptr, data):
    """Kahan sums of each CSR segment in stored order (the operation order of
    the library's row sums)."""
    out = np.empty(len(indptr) - 1)
    for r in range(len(indptr) - 1):
        s = c = 0.0
        for v in data[indptr[r]:indptr[r + 1]]:
            y = v - c
            t = s + y
            c = (t - s) - y
            s = t
        out[r] = s
    return out


def test_row_col_sums_on_request_from_threads(cuda):
    """Row / column sums are computed on the first request, once, even when
    several threads ask at the same time; they are the Kahan sums of A in
    column (row) order and agree with the cell areas as the reference's area
    test asks (lib/ConservativeRegriddingTestHelpers/src/ConservativeRegriddingTestHelpers.jl:70-73)."""
    from concurrent.futures import ThreadPoolExecutor

    dst, src = c1_grids()
    R = Regridder(dst, src, normalize=True)
    A = R.intersections
    csr = A.tocsr()
    csr.sort_indices()
    csc = A.tocsc()
    csc.sort_indices()
    want_r, want_c = _kahan_segments(csr.indptr, csr.data), _kahan_segments(csc.indptr, csc.data)
    with ThreadPoolExecutor(4) as ex:
        got = list(ex.map(lambda _: R.row_col_sums(), range(4)))
    for rs, cs in got:
        assert np.array_equal(rs, want_r) and np.array_equal(cs, want_c)
    tol = np.sqrt(np.finfo(np.float64).eps)
    assert np.allclose(want_r, R.dst_areas, rtol=tol, atol=0)
    # the destination grid starts at -89.6 degrees: source cells reaching below it are not covered
    t, _ = src.cell_table()
    covered = t[:, :4, 2].min(axis=1) > np.sin(np.radians(-89.6)) + 1e-12
    assert 0 < (~covered).sum() < 400
    assert np.allclose(want_c[covered], R.src_areas[covered], rtol=tol, atol=0)
    assert np.all(want_c[~covered] < R.src_areas[~covered])
    rs2, cs2 = R.transpose().row_col_sums()  # the transpose view shares the handle's sums
    assert np.array_equal(rs2, want_r) and np.array_equal(cs2, want_c)


@pytest.mark.parametrize("dtype,K", [("bfloat16", 128), ("bfloat16", 64), ("bfloat16", 40), ("bfloat16", 200),
                                     ("bfloat16", 45), ("float32", 33), ("float32", 130), ("float32", 128)])
@pytest.mark.parametrize("case", ["cut_rows", "empty_rows"])
def test_low_precision_apply_cut_and_empty_rows(cuda, dtype, K, case):
    """FP32 / BF16 cell-major fields (FP32 accumulation) against the FP64 apply
    of the same rounded inputs, on matrices with rows cut between merge-path
    tasks (10-degree cells over HEALPix 32: ~30 entries per row) and with rows
    that have no entries (a destination partly outside the source), both
    directions: within the output rounding.  Field counts that are not a
    multiple of 4 take the merge path's strided lane layout."""
    import torch

    tol = 8e-3 if dtype == "bfloat16" else 2e-6

    if case == "cut_rows":
        R = Regridder(grids.lonlat_regular(10.0, 10.0), grids.healpix_grid(32), normalize=True)
        assert R.info["cut_rows"][0] > 0
    else:
        R = Regridder(grids.lonlat_grid(np.arange(0.0, 361.0, 10.0), np.arange(-90.0, 91.0, 10.0)),
                      grids.lonlat_grid(np.arange(0.0, 181.0, 6.0), np.arange(-30.0, 31.0, 6.0)), normalize=True)
        assert R.info["empty_rows"][0] > 0
    gen = torch.Generator(device="cuda").manual_seed(K)
    A = R.intersections
    for RR, counts in ((R, A.getnnz(axis=1)), (R.transpose(), A.getnnz(axis=0))):
        n_out, n_in = RR.shape
        x = torch.randn((n_in, K), generator=gen, device="cuda").to(getattr(torch, dtype))
        y = torch.full((n_out, K), float("nan"), device="cuda").to(getattr(torch, dtype))
        regrid_(y, RR, x, dims=1)
        ref = torch.empty((n_out, K), dtype=torch.float64, device="cuda")
        regrid_(ref, RR, x.double(), dims=1)
        err = (y.double() - ref).abs().max().item()
        assert np.isfinite(err) and err <= tol * ref.abs().max().item(), err
        empty = torch.from_numpy(np.asarray(counts) == 0).cuda()
        assert bool((y[empty] == 0).all())


@pytest.mark.parametrize("dtype", ["float32", "bfloat16"])
@pytest.mark.parametrize("case", ["cut_rows", "empty_rows", "polar_rows"])
def test_narrow_fields(cuda, dtype, case):
    """2 to 31 cell-major fields run the narrow merge-path kernel (several
    entries per warp load, a segmented scan per chunk of a task, rows continued
    across chunks and cut across tasks), one field the row kernel: against the
    FP64 apply of the same rounded inputs within the output rounding, both
    directions, K = 1 (a vector) .. 31, aligned rows or not; rows without
    entries are zero; applying again gives the same bits.  Matrices: rows cut
    between tasks (10-degree cells over HEALPix 32), rows without entries, and
    HEALPix 64 over 0.5-degree cells, whose polar rows hold hundreds of entries."""
    import torch

    tol = 8e-3 if dtype == "bfloat16" else 2e-6
    if case == "cut_rows":
        R = Regridder(grids.lonlat_regular(10.0, 10.0), grids.healpix_grid(32), normalize=True)
        assert R.info["cut_rows"][0] > 0
    elif case == "empty_rows":
        R = Regridder(grids.lonlat_grid(np.arange(0.0, 361.0, 10.0), np.arange(-90.0, 91.0, 10.0)),
                      grids.lonlat_grid(np.arange(0.0, 181.0, 6.0), np.arange(-30.0, 31.0, 6.0)), normalize=True)
        assert R.info["empty_rows"][0] > 0
    else:
        R = Regridder(grids.healpix_grid(64), grids.lonlat_regular(0.5, 0.5), normalize=True)
        assert R.intersections.getnnz(axis=1).max() > 200
    A = R.intersections
    dt = getattr(torch, dtype)
    for K in (1, 2, 3, 4, 5, 7, 8, 12, 16, 17, 24, 31):
        gen = torch.Generator(device="cuda").manual_seed(100 + K)
        for RR, counts in ((R, A.getnnz(axis=1)), (R.transpose(), A.getnnz(axis=0))):
            n_out, n_in = RR.shape
            shp_in, shp_out = ((n_in,), (n_out,)) if K == 1 else ((n_in, K), (n_out, K))
            x = torch.randn(shp_in, generator=gen, device="cuda").to(dt)
            y = torch.full(shp_out, float("nan"), device="cuda").to(dt)
            regrid_(y, RR, x, dims=1)
            ref = torch.empty(shp_out, dtype=torch.float64, device="cuda")
            regrid_(ref, RR, x.double(), dims=1)
            err = (y.double() - ref).abs().max().item()
            assert np.isfinite(err) and err <= tol * ref.abs().max().item(), (K, err)
            empty = torch.from_numpy(np.asarray(counts) == 0).cuda()
            assert bool((y[empty] == 0).all())
            y2 = torch.empty_like(y)
            regrid_(y2, RR, x, dims=1)
            assert torch.equal(y, y2), K
