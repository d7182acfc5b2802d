"""Host logic of crg.autograd (the torch.autograd counterparts of the
rrules), on the CPU: the library calls are replaced by dense stand-ins with
known derivatives, and torch.autograd.gradcheck compares each Function's
backward with central differences of its forward.  This checks what the
Functions add -- argument order, shapes, layouts of the vertex arrays,
``dims``, and which cotangents are returned -- not the kernels (the GPU tests
do that)."""
from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import crg.autograd as ad  # noqa: E402
from crg import grids  # noqa: E402


class _DenseR:
    def __init__(self, A, a_d):
        self.A, self.a_d = A, a_d
        self.shape = tuple(A.shape)


def _fake_regrid(R, src, dims=1, normalize=True):
    x = torch.movedim(src, dims - 1, 0)
    y = torch.tensordot(R.A, x, dims=1)
    if normalize:
        y = y / R.a_d.reshape((-1,) + (1,) * (y.dim() - 1))
    return torch.movedim(y, 0, dims - 1)


def _fake_adjoint_(s_bar, R, g, dims=1, normalize=True):
    gg = torch.movedim(g, dims - 1, 0)
    if normalize:
        gg = gg / R.a_d.reshape((-1,) + (1,) * (gg.dim() - 1))
    s_bar.copy_(torch.movedim(torch.tensordot(R.A.T, gg, dims=1), 0, dims - 1))
    return s_bar


@pytest.mark.parametrize("dims,shape", [(1, (7,)), (1, (7, 3)), (2, (4, 7)), (2, (2, 7, 3))])
def test_regrid_function_backward_is_the_adjoint(monkeypatch, dims, shape):
    monkeypatch.setattr(ad, "regrid", _fake_regrid)
    monkeypatch.setattr(ad, "regrid_adjoint_", _fake_adjoint_)
    g = torch.Generator().manual_seed(0)
    R = _DenseR(torch.rand(5, 7, generator=g, dtype=torch.float64),
                1.0 + torch.rand(5, generator=g, dtype=torch.float64))
    s = torch.randn(shape, generator=g, dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(lambda x: ad.regrid_ad(R, x, dims=dims), (s,))
    # an expanded (zero-stride) cotangent, as sum() produces
    ad.regrid_ad(R, s, dims=dims).sum().backward()
    ones = torch.ones(shape[:dims - 1] + (5,) + shape[dims:], dtype=torch.float64)
    assert torch.allclose(s.grad, _fake_adjoint_(torch.empty(shape, dtype=torch.float64), R, ones, dims))


class _VertexR:
    """d = alpha(V) * (beta(W) . s) with alpha = B vec(V), beta = C vec(W)."""

    B = C = None

    def __init__(self, dst, src, normalize=False):
        self.v = ad.grid_points(dst).reshape(-1)
        self.w = ad.grid_points(src).reshape(-1)
        self.alpha = self.B @ self.v
        self.beta = self.C @ self.w
        self.shape = (len(self.alpha), len(self.beta))
        self.vshape = ad.grid_points(dst).shape
        self.wshape = ad.grid_points(src).shape


def _fake_regrid_(d, R, s):
    d[...] = R.alpha * (R.beta @ s)
    return d


def _fake_pullback(R, dst, src, s, g, wrt_src=False):
    s_bar = R.beta * (R.alpha @ g)
    v_bar = (R.B.T @ g * (R.beta @ s)).reshape(R.vshape)
    if not wrt_src:
        return s_bar, v_bar
    return s_bar, v_bar, (R.C.T @ s * (R.alpha @ g)).reshape(R.wshape)


def test_vertex_regrid_function_cotangents(monkeypatch):
    dst = grids.regular_grid([0.0, 1.0, 2.0, 3.0], [0.0, 1.0, 2.0])          # curvilinear, 6 cells
    src = grids.polygon_grid([[(0, 0), (2, 0), (2, 2), (0, 2)],
                              [(2, 0), (3, 0), (3, 2)],
                              [(2, 0), (3, 2), (2, 2)]])                       # per-cell polygons, 3 cells
    rng = np.random.default_rng(3)
    V0, W0 = ad.grid_points(dst), ad.grid_points(src)
    assert V0.shape == (12, 2) and W0.shape == (3, 4, 2)
    _VertexR.B = rng.standard_normal((dst.ncells, V0.size))
    _VertexR.C = rng.standard_normal((src.ncells, W0.size))
    monkeypatch.setattr(ad, "Regridder", _VertexR)
    monkeypatch.setattr(ad, "regrid_", _fake_regrid_)
    monkeypatch.setattr(ad, "regrid_pullback", _fake_pullback)
    s = torch.tensor(rng.standard_normal(src.ncells), requires_grad=True)
    V = torch.tensor(V0, requires_grad=True)
    W = torch.tensor(W0, requires_grad=True)
    f = lambda s, V, W: ad.regrid_vertices_ad(s, V, W, dst, src)
    assert torch.autograd.gradcheck(f, (s, V, W))
    # only some inputs need a cotangent: the others come back as None
    W2 = torch.tensor(W0)
    out = f(s, V, W2)
    out.sum().backward()
    assert W2.grad is None and V.grad is not None
    # the forward saw the tensors' coordinates, not the grids' own
    moved = V0.copy()
    moved[4] += 0.25
    d = ad.regrid_vertices_ad(torch.tensor(rng.standard_normal(3)), torch.tensor(moved), W2, dst, src)
    assert d.shape == (6,)
    assert np.allclose(_VertexR(ad._with_points(dst, moved), src).alpha, _VertexR.B @ moved.reshape(-1))


def test_with_points_keeps_topology_and_checks_shape():
    g = grids.cubed_sphere(3)
    p = ad.grid_points(g)
    q = ad._with_points(g, p * 2.0)
    assert q.kind == "curvilinear" and q.block_shapes == g.block_shapes and q.full_sphere
    assert np.array_equal(q.points_flat(), p * 2.0)
    with pytest.raises(ad.DimensionMismatch):
        ad._with_points(g, p[:-1])
    with pytest.raises(ad.ArgumentError):
        ad.regrid_vertices_ad(torch.zeros(1), torch.zeros(1), torch.zeros(1), g, grids.regular_grid([0, 1], [0, 1]))
