// crg_api.cu -- the extern "C" boundary declared in include/crg.h.
// No C++ exception crosses it: every entry point catches and returns a status.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "crg_internal.cuh"

namespace crg {

namespace {
thread_local char g_err[1024] = "";
}

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

namespace {

template <class F>
crg_status guarded(F&& f) {
  try {
    f();
    return CRG_OK;
  } catch (const Fail& e) {
    return e.st;
  } catch (const std::bad_alloc&) {
    set_error("host allocation failed");
    return CRG_ERR_OUT_OF_MEMORY;
  } catch (...) {
    set_error("unexpected internal error");
    return CRG_ERR_INTERNAL;
  }
}

// Copy a device int32 pointer array (n+1 entries) to int64 with a base shift.
__global__ void k_widen_ptr(const int32_t* __restrict__ in, int64_t n, int64_t base, int64_t* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (int64_t)in[i] + base;
}

void export_csr(const DevCsr& c, int32_t base, int64_t* ptr, int64_t* idx, double* val) {
  CRG_REQUIRE(base == 0 || base == 1, CRG_ERR_INVALID_ARGUMENT, "index_base must be 0 or 1");
  CRG_REQUIRE(ptr && (c.nnz == 0 || (idx && val)), CRG_ERR_INVALID_ARGUMENT, "output arrays must not be NULL");
  const int64_t np = c.nrows + 1, nnz = c.nnz;
  int64_t* dptr = nullptr;
  int64_t* didx = nullptr;
  CRG_CHECK_CUDA(cudaMalloc(&dptr, sizeof(int64_t) * np));
  CRG_CHECK_CUDA(cudaMalloc(&didx, sizeof(int64_t) * (nnz > 0 ? nnz : 1)));
  k_widen_ptr<<<(unsigned)((np + 255) / 256), 256>>>(c.ptr, np, base, dptr);
  if (nnz) k_widen_ptr<<<(unsigned)((nnz + 255) / 256), 256>>>(c.idx, nnz, base, didx);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(ptr, dptr, sizeof(int64_t) * np, cudaMemcpyDefault);
  if (e == cudaSuccess && nnz) e = cudaMemcpy(idx, didx, sizeof(int64_t) * nnz, cudaMemcpyDefault);
  if (e == cudaSuccess && nnz) e = cudaMemcpy(val, c.val, sizeof(double) * nnz, cudaMemcpyDefault);
  cudaFree(dptr);
  cudaFree(didx);
  CRG_CHECK_CUDA(e);
}

// ESMF offline weights from the CSC of A (rows of the transposed copy):
// entry k of source column j gives row = its destination cell, col = j,
// S = A_ij / a_i (ESMF "destarea" normalisation).
__global__ void k_esmf_entries(const int32_t* __restrict__ cptr, const int32_t* __restrict__ rows,
                               const double* __restrict__ val, int64_t ncols, const double* __restrict__ dst_area,
                               int64_t base, int64_t* __restrict__ row, int64_t* __restrict__ col,
                               double* __restrict__ S) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ncols) return;
  for (int32_t k = cptr[j]; k < cptr[j + 1]; ++k) {
    const int32_t i = rows[k];
    row[k] = i + base;
    col[k] = j + base;
    S[k] = val[k] / dst_area[i];
  }
}

__global__ void k_ratio(const double* __restrict__ a, const double* __restrict__ b, int64_t n, double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] / b[i];
}

void export_esmf(const crg_regridder* r, int32_t base, int64_t* row, int64_t* col, double* S, double* frac_a,
                 double* frac_b, double* area_a, double* area_b) {
  CRG_REQUIRE(r != nullptr, CRG_ERR_INVALID_ARGUMENT, "regridder is NULL");
  CRG_REQUIRE(base == 0 || base == 1, CRG_ERR_INVALID_ARGUMENT, "index_base must be 0 or 1");
  const int64_t nnz = r->nnz, na = r->ns, nb = r->nd;
  CRG_REQUIRE(nnz == 0 || (row && col && S), CRG_ERR_INVALID_ARGUMENT, "row, col and S must not be NULL");
  // device scratch: [nnz] row | [nnz] col | [nnz] S | [na] frac_a | [nb] frac_b
  char* buf = nullptr;
  const size_t bytes = sizeof(int64_t) * 2 * nnz + sizeof(double) * (nnz + na + nb) + 64;
  CRG_CHECK_CUDA(cudaMalloc(&buf, bytes));
  int64_t* drow = reinterpret_cast<int64_t*>(buf);
  int64_t* dcol = drow + nnz;
  double* dS = reinterpret_cast<double*>(dcol + nnz);
  double* dfa = dS + nnz;
  double* dfb = dfa + na;
  ensure_row_col_sums(r);
  if (na) k_esmf_entries<<<(unsigned)((na + 255) / 256), 256>>>(r->rev.ptr, r->rev.idx, r->rev.val, na, r->dst_area,
                                                                base, drow, dcol, dS);
  if (na) k_ratio<<<(unsigned)((na + 255) / 256), 256>>>(r->col_sum, r->src_area, na, dfa);
  if (nb) k_ratio<<<(unsigned)((nb + 255) / 256), 256>>>(r->row_sum, r->dst_area, nb, dfb);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && nnz) e = cudaMemcpy(row, drow, sizeof(int64_t) * nnz, cudaMemcpyDefault);
  if (e == cudaSuccess && nnz) e = cudaMemcpy(col, dcol, sizeof(int64_t) * nnz, cudaMemcpyDefault);
  if (e == cudaSuccess && nnz) e = cudaMemcpy(S, dS, sizeof(double) * nnz, cudaMemcpyDefault);
  if (e == cudaSuccess && frac_a && na) e = cudaMemcpy(frac_a, dfa, sizeof(double) * na, cudaMemcpyDefault);
  if (e == cudaSuccess && frac_b && nb) e = cudaMemcpy(frac_b, dfb, sizeof(double) * nb, cudaMemcpyDefault);
  if (e == cudaSuccess && area_a && na) e = cudaMemcpy(area_a, r->src_area, sizeof(double) * na, cudaMemcpyDefault);
  if (e == cudaSuccess && area_b && nb) e = cudaMemcpy(area_b, r->dst_area, sizeof(double) * nb, cudaMemcpyDefault);
  cudaFree(buf);
  CRG_CHECK_CUDA(e);
}

}  // namespace
}  // namespace crg

using namespace crg;

extern "C" {

crg_status crg_build(const crg_grid_desc* dst, const crg_grid_desc* src, const crg_build_opts* opts,
                     crg_regridder** out) {
  return guarded([&] {
    CRG_REQUIRE(out != nullptr, CRG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    *out = build_impl(dst, src, opts);
  });
}

crg_status crg_regridder_retain(crg_regridder* r) {
  return guarded([&] {
    CRG_REQUIRE(r != nullptr, CRG_ERR_INVALID_ARGUMENT, "regridder is NULL");
    r->refs.fetch_add(1);
  });
}

crg_status crg_regridder_release(crg_regridder* r) {
  return guarded([&] {
    if (!r) return;
    if (r->refs.fetch_sub(1) == 1) free_regridder(r);
  });
}

crg_status crg_regridder_info(const crg_regridder* r, crg_info* out) {
  return guarded([&] {
    CRG_REQUIRE(r && out, CRG_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = r->info;
  });
}

crg_status crg_apply(const crg_regridder* r, int32_t transpose, int32_t dtype, const void* src, int64_t ssc,
                     int64_t ssf, void* dst, int64_t dsc, int64_t dsf, int64_t nfields, int32_t normalize,
                     void* stream) {
  return guarded([&] {
    apply_impl(r, transpose, dtype, false, src, ssc, ssf, dst, dsc, dsf, nfields, normalize, (cudaStream_t)stream);
  });
}

crg_status crg_apply_adjoint(const crg_regridder* r, int32_t transpose, int32_t dtype, const void* gdst, int64_t gsc,
                             int64_t gsf, void* gsrc, int64_t osc, int64_t osf, int64_t nfields, int32_t normalize,
                             void* stream) {
  return guarded([&] {
    apply_impl(r, transpose, dtype, true, gdst, gsc, gsf, gsrc, osc, osf, nfields, normalize, (cudaStream_t)stream);
  });
}

crg_status crg_build_batch(int64_t n, const crg_grid_desc* dst, const crg_grid_desc* src, const crg_build_opts* opts,
                           int32_t nthreads, crg_regridder** out) {
  return guarded([&] { build_batch_impl(n, dst, src, opts, nthreads, out); });
}

crg_status crg_apply_plan_create(int64_t n, const crg_apply_item* items, crg_apply_plan** out) {
  return guarded([&] {
    CRG_REQUIRE(out != nullptr, CRG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    *out = apply_plan_impl(n, items);
  });
}

crg_status crg_apply_plan_launch(crg_apply_plan* plan, void* stream) {
  return guarded([&] { apply_plan_launch_impl(plan, (cudaStream_t)stream); });
}

crg_status crg_apply_plan_destroy(crg_apply_plan* plan) {
  return guarded([&] { apply_plan_destroy_impl(plan); });
}

crg_status crg_apply_plan_info(const crg_apply_plan* plan, int64_t* kernels, int64_t* batched_items) {
  return guarded([&] { apply_plan_info_impl(plan, kernels, batched_items); });
}

crg_status crg_area_grad(const crg_regridder* r, const crg_grid_desc* dst, const crg_grid_desc* src,
                         const double* row_weight, const double* src_field, const double* area_weight, double* grad,
                         void* stream) {
  return guarded([&] {
    area_grad_impl(r, dst, src, row_weight, src_field, area_weight, grad, (cudaStream_t)stream);
  });
}

crg_status crg_apply_noalloc(const crg_regridder* r, int32_t transpose, int32_t dtype, const void* src, int64_t ssc,
                             int64_t ssf, void* dst, int64_t dsc, int64_t dsf, int64_t nfields, int32_t normalize,
                             void* stream) {
  return guarded([&] {
    apply_noalloc_impl(r, transpose, dtype, src, ssc, ssf, dst, dsc, dsf, nfields, normalize, (cudaStream_t)stream);
  });
}

crg_status crg_get_csc(const crg_regridder* r, int32_t index_base, int64_t* colptr, int64_t* rowval, double* nzval) {
  return guarded([&] {
    CRG_REQUIRE(r != nullptr, CRG_ERR_INVALID_ARGUMENT, "regridder is NULL");
    export_csr(r->rev, index_base, colptr, rowval, nzval);
  });
}

crg_status crg_get_csr(const crg_regridder* r, int32_t index_base, int64_t* rowptr, int64_t* colval, double* nzval) {
  return guarded([&] {
    CRG_REQUIRE(r != nullptr, CRG_ERR_INVALID_ARGUMENT, "regridder is NULL");
    export_csr(r->fwd, index_base, rowptr, colval, nzval);
  });
}

crg_status crg_get_areas(const crg_regridder* r, double* dst_areas, double* src_areas) {
  return guarded([&] {
    CRG_REQUIRE(r != nullptr, CRG_ERR_INVALID_ARGUMENT, "regridder is NULL");
    if (dst_areas && r->nd) CRG_CHECK_CUDA(cudaMemcpy(dst_areas, r->dst_area, sizeof(double) * r->nd, cudaMemcpyDefault));
    if (src_areas && r->ns) CRG_CHECK_CUDA(cudaMemcpy(src_areas, r->src_area, sizeof(double) * r->ns, cudaMemcpyDefault));
  });
}

crg_status crg_get_row_col_sums(const crg_regridder* r, double* row_sums, double* col_sums) {
  return guarded([&] {
    CRG_REQUIRE(r != nullptr, CRG_ERR_INVALID_ARGUMENT, "regridder is NULL");
    ensure_row_col_sums(r);
    if (row_sums && r->nd) CRG_CHECK_CUDA(cudaMemcpy(row_sums, r->row_sum, sizeof(double) * r->nd, cudaMemcpyDefault));
    if (col_sums && r->ns) CRG_CHECK_CUDA(cudaMemcpy(col_sums, r->col_sum, sizeof(double) * r->ns, cudaMemcpyDefault));
  });
}

crg_status crg_mirror_fold(int32_t dtype, void* field, int64_t stride_cell, int64_t stride_field, int64_t nfields,
                           int64_t nx, int64_t ny, void* stream) {
  return guarded([&] { mirror_fold_impl(dtype, field, stride_cell, stride_field, nfields, nx, ny, (cudaStream_t)stream); });
}

crg_status crg_get_esmf_weights(const crg_regridder* r, int32_t index_base, int64_t* row, int64_t* col, double* S,
                                double* frac_a, double* frac_b, double* area_a, double* area_b) {
  return guarded([&] { export_esmf(r, index_base, row, col, S, frac_a, frac_b, area_a, area_b); });
}

crg_status crg_apply_batch(int64_t n, const crg_apply_item* items, int32_t nthreads, void* stream) {
  return guarded([&] { apply_batch_impl(n, items, nthreads, (cudaStream_t)stream); });
}

crg_status crg_build_se_to_fv(const crg_grid_desc* dst, const crg_se_space* src, const crg_se_opts* opts,
                              crg_regridder** out) {
  return guarded([&] {
    CRG_REQUIRE(out != nullptr, CRG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    *out = build_se_impl(dst, src, opts, false);
  });
}

crg_status crg_build_fv_to_se(const crg_se_space* dst, const crg_grid_desc* src, const crg_se_opts* opts,
                              crg_regridder** out) {
  return guarded([&] {
    CRG_REQUIRE(out != nullptr, CRG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    *out = build_se_impl(src, dst, opts, true);
  });
}

crg_status crg_se_nodes(const crg_se_space* space, const crg_se_opts* opts, double* points, double* weights) {
  return guarded([&] { se_nodes_impl(space, opts, points, weights); });
}

crg_status crg_se_dss(int32_t dtype, void* field, int64_t stride_node, int64_t stride_field, int64_t nfields,
                      const int32_t* group_ptr, const int32_t* group_nodes, const double* weights, int64_t ngroups,
                      void* stream) {
  return guarded([&] {
    se_dss_impl(dtype, field, stride_node, stride_field, nfields, group_ptr, group_nodes, weights, ngroups,
                (cudaStream_t)stream);
  });
}

const char* crg_last_error(void) { return g_err; }

const char* crg_status_string(crg_status s) {
  switch (s) {
    case CRG_OK: return "ok";
    case CRG_ERR_INVALID_ARGUMENT: return "invalid argument";
    case CRG_ERR_DIMENSION_MISMATCH: return "dimension mismatch";
    case CRG_ERR_CUDA: return "CUDA error";
    case CRG_ERR_OUT_OF_MEMORY: return "out of memory";
    case CRG_ERR_NOT_SUPPORTED: return "not supported";
    case CRG_ERR_GEOMETRY: return "geometry capacity exceeded";
    case CRG_ERR_INTERNAL: return "internal error";
  }
  return "unknown status";
}

int32_t crg_abi_version(void) { return CRG_ABI_VERSION; }

}  // extern "C"
