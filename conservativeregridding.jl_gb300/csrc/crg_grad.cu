// crg_grad.cu -- derivatives of the regridder's areas with respect to the
// destination grid's vertices.
//
// The reference has no derivatives (no ChainRulesCore dependency,
// Project.toml:10-23).  For a differentiable regrid!, d = (A s) ./ a with
// A_ij = area(src_j clipped by dst_i) and a_i = area(dst_i), the cotangent of
// the destination vertices is
//   sum_ij u_i s_j dA_ij/dV + sum_i c_i da_i/dV,  u_i = g_i / a_i, c_i = -g_i d_i / a_i
// for an output cotangent g.  k_area_grad evaluates the first sum over the
// nonzeros of A (one thread per entry), k_cell_area_grad the second (one
// thread per destination cell), both by forward-mode derivatives of the same
// FP64 clip and area as the build (crg_dual.cuh), one destination vertex (its
// x, y, z) per pass, accumulating into the vertex array with atomics (the
// summation order, and so the last bits, may differ between runs).
#include <cuda_runtime.h>
#include <stdint.h>

#include "crg_dual.cuh"
#include "crg_internal.cuh"

namespace crg {

namespace {

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

constexpr int kGradCap = 2 * CRG_MAXV;  // a convex n-gon clipped by a convex m-gon has at most n + m vertices

// Vertices of one grid as laid out by the caller (crg_grid_desc), on the device.
struct GridView {
  int kind = 0, dim = 3, maxv = 4, nblocks = 0;
  int64_t ncells = 0, nslots = 0;  // nslots: points (curvilinear) or ncells * maxv vertex slots (cells)
  int64_t cell_off[kMaxGridBlocks + 1] = {};
  int64_t point_off[kMaxGridBlocks] = {};
  int64_t nx[kMaxGridBlocks] = {};
  const double* pts = nullptr;   // curvilinear: [points][dim]
  const double* cv = nullptr;    // cells: [ncells][maxv][dim]
  const int32_t* cn = nullptr;   // cells: vertex counts, or NULL for maxv each
};

// Vertices of cell c (z = 0 on the plane) and, when ids is not NULL, the slot
// of each vertex in the caller's vertex array; returns the vertex count.
__device__ int cell_vertices(const GridView& g, int64_t c, d3* v, int64_t* ids) {
  if (g.kind == CRG_GRID_CURVILINEAR) {
    int b = 0;
    while (b + 1 < g.nblocks && c >= g.cell_off[b + 1]) b++;
    const int64_t loc = c - g.cell_off[b], nx = g.nx[b];
    const int64_t i = loc % nx, j = loc / nx;
    const int64_t p[4] = {i + j * (nx + 1), (i + 1) + j * (nx + 1), (i + 1) + (j + 1) * (nx + 1),
                          i + (j + 1) * (nx + 1)};
    for (int k = 0; k < 4; ++k) {
      const int64_t slot = g.point_off[b] + p[k];
      const double* q = g.pts + slot * g.dim;
      v[k] = d3{q[0], q[1], g.dim == 3 ? q[2] : 0.0};
      if (ids) ids[k] = slot;
    }
    return 4;
  }
  const int n = g.cn ? g.cn[c] : g.maxv;
  for (int k = 0; k < n; ++k) {
    const int64_t slot = c * g.maxv + k;
    const double* q = g.cv + slot * g.dim;
    v[k] = d3{q[0], q[1], g.dim == 3 ? q[2] : 0.0};
    if (ids) ids[k] = slot;
  }
  return n;
}

template <bool kSph>
__global__ void __launch_bounds__(128) k_area_grad(const int32_t* __restrict__ erow, const int32_t* __restrict__ idx,
                                                   int64_t nnz, GridView dg, GridView sg,
                                                   const double* __restrict__ u, const double* __restrict__ s,
                                                   double* __restrict__ grad, unsigned long long* __restrict__ bad) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nnz) return;
  const int32_t i = erow[e], j = idx[e];
  const double coef = u[i] * s[j];
  if (coef == 0.0) return;
  d3 dv[CRG_MAXV], sv[CRG_MAXV];
  int64_t did[CRG_MAXV];
  const int nd = cell_vertices(dg, i, dv, did);
  const int ns = cell_vertices(sg, j, sv, nullptr);
  if (nd < 3 || ns < 3) return;
  const double sig = kSph ? orient_sph(sv, ns) : orient_pl(sv, ns);
  D3n<3> clip[CRG_MAXV];
  D3n<3> bufA[kGradCap], bufB[kGradCap];
  for (int kk = 0; kk < nd; ++kk) {
    for (int q = 0; q < nd; ++q) clip[q] = d3n_const<3>(dv[q]);
    clip[kk].x.d[0] = 1.0;
    clip[kk].y.d[1] = 1.0;
    clip[kk].z.d[2] = 1.0;
    for (int q = 0; q < ns; ++q) bufA[q] = d3n_const<3>(sv[q]);
    D3n<3>* res;
    const int m = clip_polygon_n<kSph, 3, kGradCap>(bufA, bufB, ns, clip, nd, &res);
    if (m < 0) {
      atomicAdd(bad, 1ull);
      return;
    }
    const Dn<3> a = kSph ? area_sph_signed_n(res, m) : area_pl_signed_n(res, m);
    for (int c = 0; c < dg.dim; ++c) atomicAdd(grad + did[kk] * dg.dim + c, coef * sig * a.d[c]);
  }
}

template <bool kSph>
__global__ void __launch_bounds__(128) k_cell_area_grad(GridView dg, const double* __restrict__ cw,
                                                        double* __restrict__ grad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= dg.ncells) return;
  const double coef = cw[i];
  if (coef == 0.0) return;
  d3 dv[CRG_MAXV];
  int64_t did[CRG_MAXV];
  const int nd = cell_vertices(dg, i, dv, did);
  if (nd < 3) return;
  const double orient = kSph ? orient_sph(dv, nd) : orient_pl(dv, nd);
  D3n<3> v[CRG_MAXV];
  for (int kk = 0; kk < nd; ++kk) {
    for (int q = 0; q < nd; ++q) v[q] = d3n_const<3>(dv[q]);
    v[kk].x.d[0] = 1.0;
    v[kk].y.d[1] = 1.0;
    v[kk].z.d[2] = 1.0;
    const Dn<3> a = kSph ? area_sph_signed_n(v, nd) : area_pl_signed_n(v, nd);
    for (int c = 0; c < dg.dim; ++c) atomicAdd(grad + did[kk] * dg.dim + c, coef * orient * a.d[c]);
  }
}

// device copy of a host array (or the device pointer itself)
template <class T> struct Staged {
  T* p = nullptr;
  cudaStream_t st = nullptr;
  const T* get(const T* src, size_t n, cudaStream_t s) {
    if (!src || n == 0 || is_device_pointer(src)) return src;
    st = s;
    CRG_CHECK_CUDA(cudaMallocAsync((void**)&p, n * sizeof(T), s));
    CRG_CHECK_CUDA(cudaMemcpyAsync(p, src, n * sizeof(T), cudaMemcpyHostToDevice, s));
    return p;
  }
  ~Staged() {
    if (p) cudaFreeAsync(p, st);
  }
};

GridView view_of(const crg_grid_desc* g, Staged<double>& sp, Staged<int32_t>& sn, cudaStream_t st) {
  CRG_REQUIRE(g != nullptr, CRG_ERR_INVALID_ARGUMENT, "grid descriptor is NULL");
  GridView v;
  v.kind = g->kind;
  v.dim = g->manifold == CRG_SPHERICAL ? 3 : 2;
  v.ncells = g->ncells;
  if (g->kind == CRG_GRID_CURVILINEAR) {
    CRG_REQUIRE(g->nblocks >= 1 && g->nblocks <= kMaxGridBlocks, CRG_ERR_INVALID_ARGUMENT,
                "nblocks = %d must be in 1..%d", g->nblocks, kMaxGridBlocks);
    CRG_REQUIRE(g->block_nx && g->block_ny && g->points, CRG_ERR_INVALID_ARGUMENT, "curvilinear grid arrays are NULL");
    v.nblocks = g->nblocks;
    v.maxv = 4;
    int64_t cells = 0, pts = 0;
    for (int b = 0; b < g->nblocks; ++b) {
      CRG_REQUIRE(g->block_nx[b] >= 1 && g->block_ny[b] >= 1, CRG_ERR_INVALID_ARGUMENT, "block %d is empty", b);
      v.cell_off[b] = cells;
      v.point_off[b] = pts;
      v.nx[b] = g->block_nx[b];
      cells += g->block_nx[b] * g->block_ny[b];
      pts += (g->block_nx[b] + 1) * (g->block_ny[b] + 1);
    }
    v.cell_off[g->nblocks] = cells;
    CRG_REQUIRE(cells == g->ncells, CRG_ERR_DIMENSION_MISMATCH, "ncells = %lld but the blocks hold %lld cells",
                (long long)g->ncells, (long long)cells);
    v.nslots = pts;
    v.pts = sp.get(g->points, (size_t)pts * v.dim, st);
  } else if (g->kind == CRG_GRID_CELLS) {
    CRG_REQUIRE(g->max_verts >= 3 && g->max_verts <= CRG_MAXV, CRG_ERR_INVALID_ARGUMENT,
                "max_verts = %d must be in 3..%d", g->max_verts, CRG_MAXV);
    CRG_REQUIRE(g->cell_verts || g->ncells == 0, CRG_ERR_INVALID_ARGUMENT, "cell_verts is NULL");
    v.maxv = g->max_verts;
    v.nslots = g->ncells * g->max_verts;
    v.cv = sp.get(g->cell_verts, (size_t)v.nslots * v.dim, st);
    v.cn = sn.get(g->cell_nverts, (size_t)g->ncells, st);
  } else {
    CRG_REQUIRE(false, CRG_ERR_INVALID_ARGUMENT, "unknown grid kind %d", g->kind);
  }
  return v;
}

}  // namespace

void area_grad_impl(const crg_regridder* r, const crg_grid_desc* dst, const crg_grid_desc* src, const double* u,
                    const double* s, const double* c, double* grad, cudaStream_t st) {
  CRG_REQUIRE(r != nullptr, CRG_ERR_INVALID_ARGUMENT, "regridder is NULL");
  CRG_REQUIRE(grad != nullptr, CRG_ERR_INVALID_ARGUMENT, "gradient array is NULL");
  CRG_REQUIRE((u == nullptr) == (s == nullptr), CRG_ERR_INVALID_ARGUMENT,
              "row_weight and src_field are given together (or both NULL)");
  check_grid_desc(dst, "destination");
  check_grid_desc(src, "source");
  int dev = 0;
  CRG_CHECK_CUDA(cudaGetDevice(&dev));
  CRG_REQUIRE(dev == r->device, CRG_ERR_INVALID_ARGUMENT, "regridder lives on device %d but device %d is current",
              r->device, dev);
  CRG_REQUIRE(dst && src && dst->manifold == r->manifold && src->manifold == r->manifold, CRG_ERR_INVALID_ARGUMENT,
              "the grids' manifold differs from the regridder's");
  Staged<double> dp, spts, su, ss, sc;
  Staged<int32_t> dn, sn;
  const GridView dg = view_of(dst, dp, dn, st);
  const GridView sg = view_of(src, spts, sn, st);
  CRG_REQUIRE(dg.ncells == r->nd && sg.ncells == r->ns, CRG_ERR_DIMENSION_MISMATCH,
              "grids have %lld x %lld cells, the regridder %lld x %lld", (long long)dg.ncells,
              (long long)sg.ncells, (long long)r->nd, (long long)r->ns);
  const double* du = su.get(u, (size_t)r->nd, st);
  const double* ds = ss.get(s, (size_t)r->ns, st);
  const double* dc = sc.get(c, (size_t)r->nd, st);
  const size_t nout = (size_t)dg.nslots * dg.dim;
  const bool host_out = !is_device_pointer(grad);
  double* g = grad;
  if (host_out) CRG_CHECK_CUDA(cudaMallocAsync((void**)&g, nout * sizeof(double) + 8, st));
  unsigned long long* bad = nullptr;
  CRG_CHECK_CUDA(cudaMallocAsync((void**)&bad, sizeof(unsigned long long), st));
  CRG_CHECK_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned long long), st));
  if (nout) CRG_CHECK_CUDA(cudaMemsetAsync(g, 0, nout * sizeof(double), st));
  const bool sph = r->manifold == CRG_SPHERICAL;
  if (du && r->nnz) {
    if (sph)
      k_area_grad<true><<<nblk(r->nnz, 128), 128, 0, st>>>(r->fwd.erow, r->fwd.idx, r->nnz, dg, sg, du, ds, g, bad);
    else
      k_area_grad<false><<<nblk(r->nnz, 128), 128, 0, st>>>(r->fwd.erow, r->fwd.idx, r->nnz, dg, sg, du, ds, g, bad);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
  if (dc && dg.ncells) {
    if (sph) k_cell_area_grad<true><<<nblk(dg.ncells, 128), 128, 0, st>>>(dg, dc, g);
    else k_cell_area_grad<false><<<nblk(dg.ncells, 128), 128, 0, st>>>(dg, dc, g);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
  unsigned long long hbad = 0;
  CRG_CHECK_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(hbad), cudaMemcpyDeviceToHost, st));
  if (host_out && nout) CRG_CHECK_CUDA(cudaMemcpyAsync(grad, g, nout * sizeof(double), cudaMemcpyDeviceToHost, st));
  CRG_CHECK_CUDA(cudaFreeAsync(bad, st));
  if (host_out) CRG_CHECK_CUDA(cudaFreeAsync(g, st));
  CRG_CHECK_CUDA(cudaStreamSynchronize(st));
  CRG_REQUIRE(hbad == 0, CRG_ERR_GEOMETRY, "%llu pairs exceeded the clipped-polygon capacity of %d vertices",
              hbad, kGradCap);
}

}  // namespace crg
