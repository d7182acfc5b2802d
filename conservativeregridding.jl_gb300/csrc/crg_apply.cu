// crg_apply.cu -- applying the regridder: d = (A s) ./ a_d and its transpose.
//
// Replaces regrid! (src/regridder/regrid.jl:63-118): the stdlib CSC mul!
// (single-threaded column scatter, :95-98) followed by the division by the
// destination areas (:104-118), the one-mul!-per-slice N-D loop
// (NDSliceLoop, :225-318), and regrid!(dst, transpose(R), src)
// (src/regridder/regridder.jl:49-50).  A is stored twice (CSR rows = dst and
// rows = src), so every direction is a row gather with no atomics.
//
// Kernels:
//   k_spmv_f64      FP64, one thread per (row, field), summation in ascending
//                   column order from 0.0 -- the same sequence as the
//                   reference's column-scatter mul! for each row -- then the
//                   optional division by the row area.
//   k_spmv_f64_k    FP64, 2-4 cell-major fields: the same per field, a thread
//                   per row with all its fields.
//   k_cm_rows_f64   FP64, more cell-major fields: G lanes per row, 4 fields
//                   per lane, the same per field; up to 32 fields the
//                   autotuner also times batches of 4 or 8 entries per group.
//   k_cm_nnz        FP32/BF16 fields stored cell-major (the fields of one cell
//                   side by side), >= 32 of them: merge-path over ~64-entry
//                   tasks, a warp per task, 4 fields per lane, B gathers of a
//                   source cell's field vector in flight (+ k_cm_fixup for
//                   rows cut between tasks, k_zero_empty_cm for empty rows).
//   k_cm_narrow     cell-major, 2-31 fields: the same tasks in chunks of
//                   64 / G entries (G lanes of 4 fields each per lane group,
//                   two entries per group), a segmented scan per chunk.
//   k_cm_rows       cell-major, fewer fields with CRG_SPMM_PATH=rows: G lanes
//                   per row, RB rows per lane group, 4 fields per lane.
//   k_fm_rows       field-major (spatial index contiguous per field): a row
//                   per lane; with >= 32 fields the first apply of a direction
//                   may choose k_transpose + the cell-major path instead.
//   k_spmm_rows     cell-major without 16-byte alignment or a multiple of 4 fields.
//   k_spmm_generic  any strides, one thread per (row, field).
#include <cuda_bf16.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "crg_div.cuh"
#include "crg_internal.cuh"

namespace crg {

namespace {

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// ------------------------------------------------------------------ element IO

template <class T> __device__ __forceinline__ float ld1(const T* p);
template <> __device__ __forceinline__ float ld1<float>(const float* p) { return __ldg(p); }
template <> __device__ __forceinline__ float ld1<__nv_bfloat16>(const __nv_bfloat16* p) { return __bfloat162float(__ldg(p)); }

template <class T> __device__ __forceinline__ void st1(T* p, float v);
template <> __device__ __forceinline__ void st1<float>(float* p, float v) { *p = v; }
template <> __device__ __forceinline__ void st1<__nv_bfloat16>(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }

// 4 consecutive elements (16 B FP32 / 8 B BF16, aligned)
template <class T> __device__ __forceinline__ float4 ld4(const T* p);
template <> __device__ __forceinline__ float4 ld4<float>(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
template <> __device__ __forceinline__ float4 ld4<__nv_bfloat16>(const __nv_bfloat16* p) {
  // a BF16 value is the upper half of its FP32 value
  const uint2 u = __ldg(reinterpret_cast<const uint2*>(p));
  return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xffff0000u), __uint_as_float(u.y << 16),
                     __uint_as_float(u.y & 0xffff0000u));
}

template <class T> __device__ __forceinline__ void st4(T* p, float4 v);
template <> __device__ __forceinline__ void st4<float>(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
template <> __device__ __forceinline__ void st4<__nv_bfloat16>(__nv_bfloat16* p, float4 v) {
  __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y), b = __floats2bfloat162_rn(v.z, v.w);
  uint2 u;
  u.x = *reinterpret_cast<uint32_t*>(&a);
  u.y = *reinterpret_cast<uint32_t*>(&b);
  *reinterpret_cast<uint2*>(p) = u;
}

// ------------------------------------------------------------------ FP64

__global__ void k_spmv_f64(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                           const double* __restrict__ val, int64_t nrows, const double* __restrict__ x, int64_t xsc,
                           int64_t xsf, double* __restrict__ y, int64_t ysc, int64_t ysf, int64_t f0,
                           const double* __restrict__ row_div, const double* __restrict__ col_div) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int64_t f = f0 + blockIdx.y;
  const double* xf = x + f * xsf;
  double acc = 0.0;
  int32_t k = __ldg(ptr + r);
  const int32_t k1 = __ldg(ptr + r + 1);
  // four entries' loads issued before their (ordered) sums: the row's gathers
  // overlap instead of waiting one after another
  for (; k + 4 <= k1; k += 4) {
    int32_t j[4];
    double v[4], xv[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      j[q] = __ldg(idx + k + q);
      v[q] = __ldg(val + k + q);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) xv[q] = xf[(int64_t)j[q] * xsc];
    if (col_div) {
#pragma unroll
      for (int q = 0; q < 4; ++q) xv[q] = xv[q] / __ldg(col_div + j[q]);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) acc = acc + v[q] * xv[q];
  }
  for (; k < k1; ++k) {
    const int32_t jj = __ldg(idx + k);
    double xx = xf[(int64_t)jj * xsc];
    if (col_div) xx = xx / __ldg(col_div + jj);
    acc = acc + __ldg(val + k) * xx;
  }
  if (row_div) acc = acc / row_div[r];
  y[r * ysc + f * ysf] = acc;
}

// FP64 fields side by side (cell-major), many of them: G lanes per row, 4
// fields per lane (two 16-byte loads when aligned), the row's (column,
// weight) entries loaded G at a time (KB = 0) or in batches of KB and
// broadcast by shuffles.  Each field
// is summed exactly as k_spmv_f64 sums it -- acc = 0, then acc + (w x) per
// entry in ascending column order, each operation rounded once -- and divided
// by the row area, so every field has the bits of the one-field apply (and of
// the reference's mul! then ./ areas).  The division by column areas of the
// adjoint is applied to the input beforehand (k_div_cols_f64), the same
// quotient k_spmv_f64 forms per entry.
template <int G, bool kVec, int KB>
__global__ void __launch_bounds__(256) k_cm_rows_f64(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                                     const double* __restrict__ val, int64_t nrows,
                                                     const double* __restrict__ x, int64_t xs, double* __restrict__ y,
                                                     int64_t ys, int64_t nf, const double* __restrict__ row_div,
                                                     const double* __restrict__ row_rcp) {
  const int lane = threadIdx.x & 31;
  const int g = lane % G;
  const int gbase = lane - g;
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gbase);
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  if (r >= nrows) return;  // the whole lane group shares r
  const int32_t k0 = __ldg(ptr + r), n = __ldg(ptr + r + 1) - k0;
  const double div = row_div ? __ldg(row_div + r) : 1.0;
  const double rcp = row_div ? __ldg(row_rcp + r) : 1.0;  // RN(1 / div): the quotients correct from it
  for (int64_t f0 = 0; f0 < nf; f0 += (int64_t)G * 4) {
    const int64_t f = f0 + (int64_t)g * 4;
    const bool on = f < nf;
    const bool full = kVec && f + 4 <= nf;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    if constexpr (KB > 0) {
      // Batches of KB entries (the autotuner's candidates up to 32 fields),
      // entry kb + u G + e held by lane e of the group.  The next batch's
      // (column, weight) pairs load while this batch's gathers are in flight,
      // and the sums follow in entry order: a polar row of hundreds of entries
      // costs one gather latency per KB entries instead of an index and a
      // gather latency per G.
      static_assert(KB % G == 0, "a batch is a whole number of entries per lane");
      constexpr int kB = KB, U = kB / G;
      int32_t bj[U];
      double bw[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int e = u * G + g;
        bj[u] = e < n ? __ldg(idx + k0 + e) : 0;
        bw[u] = e < n ? __ldg(val + k0 + e) : 0.0;
      }
      for (int kb = 0; kb < n; kb += kB) {
        int32_t nj[U];
        double nw[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int e = kb + kB + u * G + g;
          nj[u] = e < n ? __ldg(idx + k0 + e) : 0;
          nw[u] = e < n ? __ldg(val + k0 + e) : 0.0;
        }
        double xv[kB][4], wv[kB];
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
          for (int e = 0; e < G; ++e) {
            const int m = u * G + e;
            const int64_t j = __shfl_sync(gmask, bj[u], gbase + e);
            wv[m] = __shfl_sync(gmask, bw[u], gbase + e);
            const bool ok = on && kb + m < n;
            const double* xp = x + j * xs + f;
            if (ok && full) {
              const double2 a = __ldg(reinterpret_cast<const double2*>(xp));
              const double2 b = __ldg(reinterpret_cast<const double2*>(xp) + 1);
              xv[m][0] = a.x; xv[m][1] = a.y; xv[m][2] = b.x; xv[m][3] = b.y;
            } else {
#pragma unroll
              for (int q = 0; q < 4; ++q) xv[m][q] = (ok && f + q < nf) ? __ldg(xp + q) : 0.0;
            }
          }
#pragma unroll
        for (int m = 0; m < kB; ++m)
          if (kb + m < n) {
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[q] = __dadd_rn(acc[q], __dmul_rn(wv[m], xv[m][q]));
          }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          bj[u] = nj[u];
          bw[u] = nw[u];
        }
      }
    } else {
      // the group's lanes load G entries at a time
      for (int kb = 0; kb < n; kb += G) {
        const bool in = kb + g < n;
        const int32_t myj = in ? __ldg(idx + k0 + kb + g) : 0;
        const double myv = in ? __ldg(val + k0 + kb + g) : 0.0;
        const int ne = min(G, n - kb);
#pragma unroll 4
        for (int e = 0; e < ne; ++e) {
          const int64_t j = __shfl_sync(gmask, myj, gbase + e);
          const double wv = __shfl_sync(gmask, myv, gbase + e);
          if (!on) continue;
          const double* xp = x + j * xs + f;
          double xv[4];
          if (full) {
            const double2 a = __ldg(reinterpret_cast<const double2*>(xp));
            const double2 b = __ldg(reinterpret_cast<const double2*>(xp) + 1);
            xv[0] = a.x; xv[1] = a.y; xv[2] = b.x; xv[3] = b.y;
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) xv[q] = f + q < nf ? __ldg(xp + q) : 0.0;
          }
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[q] = __dadd_rn(acc[q], __dmul_rn(wv, xv[q]));
        }
      }
    }
    if (!on) continue;
    double* yp = y + r * ys + f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const double o = row_div ? div_rn_by(acc[q], div, rcp) : acc[q];
      if (full || f + q < nf) yp[q] = o;
    }
  }
}

// Two to four cell-major FP64 fields (nf <= NF): one thread per row, all its fields,
// the row's entries U at a time (their loads issued before the ordered sums),
// each field summed in entry order from 0.0 and its quotient by the row area
// formed as k_cm_rows_f64 forms it.  With a lane per row the FP64 warp
// instructions carry 32 rows' operations; k_cm_rows_f64 at one lane per row
// walked a row's entries one load after another.
template <int NF, int U>
__global__ void __launch_bounds__(128) k_spmv_f64_k(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                                    const double* __restrict__ val, int64_t nrows,
                                                    const double* __restrict__ x, int64_t xs, double* __restrict__ y,
                                                    int64_t ys, int nf, const double* __restrict__ row_div,
                                                    const double* __restrict__ row_rcp) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  double acc[NF];
#pragma unroll
  for (int q = 0; q < NF; ++q) acc[q] = 0.0;
  int32_t k = __ldg(ptr + r);
  const int32_t k1 = __ldg(ptr + r + 1);
  for (; k + U <= k1; k += U) {
    double v[U], xv[U][NF];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      v[u] = __ldg(val + k + u);
      const double* xp = x + (int64_t)__ldg(idx + k + u) * xs;
#pragma unroll
      for (int q = 0; q < NF; ++q) xv[u][q] = q < nf ? __ldg(xp + q) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int q = 0; q < NF; ++q) acc[q] = acc[q] + v[u] * xv[u][q];
  }
  for (; k < k1; ++k) {
    const double vk = __ldg(val + k);
    const double* xp = x + (int64_t)__ldg(idx + k) * xs;
#pragma unroll
    for (int q = 0; q < NF; ++q) acc[q] = acc[q] + vk * (q < nf ? __ldg(xp + q) : 0.0);
  }
  double* yp = y + r * ys;
  if (row_div) {
    const double div = __ldg(row_div + r), rcp = __ldg(row_rcp + r);
#pragma unroll
    for (int q = 0; q < NF; ++q)
      if (q < nf) yp[q] = div_rn_by(acc[q], div, rcp);
  } else {
#pragma unroll
    for (int q = 0; q < NF; ++q)
      if (q < nf) yp[q] = acc[q];
  }
}

// x'[c, f] = x[c, f] / col_div[c] for the adjoint's input (cell-major).
__global__ void k_div_cols_f64(const double* __restrict__ x, int64_t xs, int64_t ncells, int64_t nf,
                               const double* __restrict__ col_div, double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncells * nf) return;
  const int64_t c = i / nf, f = i - c * nf;
  out[i] = __ddiv_rn(x[c * xs + f], __ldg(col_div + c));
}

// ------------------------------------------------------------------ cell-major fields

// One row (entries k0..k1) without 4-field vectors: lane g of a group of G
// takes fields f0 + g + G t (t < 4) of each block of 4 G fields, so that each
// scalar load of the group reads consecutive elements.  Every field is summed
// in entry order from zero.
template <class T>
__device__ __forceinline__ void rows_strided(const int32_t* __restrict__ idx, const float* __restrict__ w, int32_t k0,
                                             int32_t k1, const T* __restrict__ x, int64_t xs, T* __restrict__ y,
                                             int64_t nf, int g, int G) {
  for (int64_t f0 = 0; f0 < nf; f0 += (int64_t)G * 4) {
    const int64_t f = f0 + g;
    float a[4] = {0.f, 0.f, 0.f, 0.f};
    for (int32_t q = k0; q < k1; ++q) {
      const int64_t j = __ldg(idx + q);
      const float ww = __ldg(w + q);
      const T* xp = x + j * xs + f;
#pragma unroll
      for (int t = 0; t < 4; ++t)
        if (f + (int64_t)t * G < nf) a[t] = fmaf(ww, ld1<T>(xp + (int64_t)t * G), a[t]);
    }
#pragma unroll
    for (int t = 0; t < 4; ++t)
      if (f + (int64_t)t * G < nf) st1<T>(y + f + (int64_t)t * G, a[t]);
  }
}

// k_spmm_rows with rows of 4-field vectors: lane g takes fields 4 g, 4 g + 4 G, ...
template <class T, int G>
__device__ __forceinline__ void spmm_rows_vec(const int32_t* __restrict__ idx, const float* __restrict__ w, int32_t k0,
                                              int32_t k1, const T* __restrict__ x, int64_t xsc, T* __restrict__ yr,
                                              int64_t nf, int g) {
  for (int64_t f = (int64_t)g * 4; f < nf; f += (int64_t)G * 4) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    const bool full = f + 4 <= nf;
    for (int32_t k = k0; k < k1; ++k) {
      const int64_t j = idx[k];
      const float ww = __ldg(w + k);
      const T* xp = x + j * xsc + f;
      float4 v;
      if (full) {
        v = ld4<T>(xp);
      } else {
        v.x = ld1<T>(xp);
        v.y = f + 1 < nf ? ld1<T>(xp + 1) : 0.f;
        v.z = f + 2 < nf ? ld1<T>(xp + 2) : 0.f;
        v.w = f + 3 < nf ? ld1<T>(xp + 3) : 0.f;
      }
      acc.x = fmaf(ww, v.x, acc.x);
      acc.y = fmaf(ww, v.y, acc.y);
      acc.z = fmaf(ww, v.z, acc.z);
      acc.w = fmaf(ww, v.w, acc.w);
    }
    T* yp = yr + f;
    if (full) {
      st4<T>(yp, acc);
    } else {
      st1<T>(yp, acc.x);
      if (f + 1 < nf) st1<T>(yp + 1, acc.y);
      if (f + 2 < nf) st1<T>(yp + 2, acc.z);
      if (f + 3 < nf) st1<T>(yp + 3, acc.w);
    }
  }
}

template <class T, int G, bool kVec>
__global__ void __launch_bounds__(256) k_spmm_rows(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                                   const float* __restrict__ w, int64_t nrows, const T* __restrict__ x,
                                                   int64_t xsc, T* __restrict__ y, int64_t ysc, int64_t nf) {
  const int g = threadIdx.x % G;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  if (r >= nrows) return;
  const int32_t k0 = ptr[r], k1 = ptr[r + 1];
  if constexpr (!kVec) {
    rows_strided<T>(idx, w, k0, k1, x, xsc, y + r * ysc, nf, g, G);
  } else {
    spmm_rows_vec<T, G>(idx, w, k0, k1, x, xsc, y + r * ysc, nf, g);
  }
}

// Cell-major fields, G lanes per row group (4 fields per lane, G*4 fields per
// pass), RB consecutive rows per group processed together.  The rows'
// (column, weight) entries are loaded G at a time by the group's lanes with
// one coalesced load per row and broadcast by shuffles, so the gathers of all
// RB rows are in flight together before the FMAs.
template <class T, int G, int RB>
__global__ void __launch_bounds__(256, 4) k_cm_rows(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                                    const float* __restrict__ w, int64_t nrows,
                                                    const int32_t* __restrict__ order, const T* __restrict__ x,
                                                    int64_t xs, T* __restrict__ y, int64_t ys, int64_t nf) {
  const int lane = threadIdx.x & 31;
  const int g = lane % G;
  const int gbase = lane - g;
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gbase);
  const int64_t grp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t r0 = grp * RB;
  if (r0 >= nrows) return;
  int32_t rr[RB], k0[RB], nn[RB];
#pragma unroll
  for (int q = 0; q < RB; ++q) {
    const int64_t ri = r0 + q;
    rr[q] = ri < nrows ? (order ? order[ri] : (int32_t)ri) : -1;
    k0[q] = rr[q] >= 0 ? __ldg(ptr + rr[q]) : 0;
    nn[q] = rr[q] >= 0 ? __ldg(ptr + rr[q] + 1) - k0[q] : 0;
  }
  int nmax = 0;
#pragma unroll
  for (int q = 0; q < RB; ++q) nmax = max(nmax, nn[q]);
  // every lane of the group runs every pass (the shuffles need the whole
  // group); lanes past the last field only skip their stores
  for (int64_t f0 = 0; f0 < nf; f0 += (int64_t)G * 4) {
    const int64_t fl = f0 + (int64_t)g * 4;
    const bool on = fl < nf;
    const int64_t f = on ? fl : 0;
    float4 acc[RB];
#pragma unroll
    for (int q = 0; q < RB; ++q) acc[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int kb = 0; kb < nmax; kb += G) {
      int32_t myj[RB];
      float myw[RB];
#pragma unroll
      for (int q = 0; q < RB; ++q) {
        const bool in = kb + g < nn[q];
        myj[q] = in ? __ldg(idx + k0[q] + kb + g) : 0;
        myw[q] = in ? __ldg(w + k0[q] + kb + g) : 0.f;
      }
      const int ne = min(G, nmax - kb);
      for (int e = 0; e < ne; e += 2) {
        float4 v[RB][2];
        float ww[RB][2];
#pragma unroll
        for (int q = 0; q < RB; ++q) {
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int src = gbase + min(e + h, G - 1);
            const int32_t j = __shfl_sync(gmask, myj[q], src);
            ww[q][h] = __shfl_sync(gmask, myw[q], src);
            const bool live = (kb + e + h) < nn[q];
            ww[q][h] = live ? ww[q][h] : 0.f;
            v[q][h] = live ? ld4<T>(x + (int64_t)j * xs + f) : make_float4(0.f, 0.f, 0.f, 0.f);
          }
        }
#pragma unroll
        for (int q = 0; q < RB; ++q)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            acc[q].x = fmaf(ww[q][h], v[q][h].x, acc[q].x);
            acc[q].y = fmaf(ww[q][h], v[q][h].y, acc[q].y);
            acc[q].z = fmaf(ww[q][h], v[q][h].z, acc[q].z);
            acc[q].w = fmaf(ww[q][h], v[q][h].w, acc[q].w);
          }
      }
    }
    if (on) {
#pragma unroll
      for (int q = 0; q < RB; ++q)
        if (rr[q] >= 0) st4<T>(y + (int64_t)rr[q] * ys + f, acc[q]);
    }
  }
}

// Field-major fields: one lane per row, so a warp reads and writes 32
// consecutive cells of each field.  The row's entries stay in registers (up to
// kFmE at a time) while the lane sweeps the fields 4 at a time, keeping
// 4 * entries gathers in flight.
constexpr int kFmE = 8;

template <class T>
__global__ void __launch_bounds__(256, 4) k_fm_rows(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                                    const float* __restrict__ w, int64_t nrows,
                                                    const int32_t* __restrict__ order, const T* __restrict__ x,
                                                    int64_t xs, T* __restrict__ y, int64_t ys, int64_t nf) {
  const int64_t ri = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (ri >= nrows) return;
  const int64_t r = order ? order[ri] : ri;
  const int32_t k0 = __ldg(ptr + r), k1 = __ldg(ptr + r + 1);
  if (k1 - k0 <= kFmE) {
    // common case: all entries in registers for the whole field sweep
    const int n = k1 - k0;
    int32_t jj[kFmE];
    float ww[kFmE];
#pragma unroll
    for (int e = 0; e < kFmE; ++e) {
      jj[e] = e < n ? __ldg(idx + k0 + e) : 0;
      ww[e] = e < n ? __ldg(w + k0 + e) : 0.f;
    }
    int64_t f = 0;
    for (; f + 4 <= nf; f += 4) {
      float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll
      for (int e = 0; e < kFmE; ++e) {
        if (e < n) {
          const T* xp = x + f * xs + jj[e];
          a0 = fmaf(ww[e], ld1<T>(xp), a0);
          a1 = fmaf(ww[e], ld1<T>(xp + xs), a1);
          a2 = fmaf(ww[e], ld1<T>(xp + 2 * xs), a2);
          a3 = fmaf(ww[e], ld1<T>(xp + 3 * xs), a3);
        }
      }
      T* yp = y + f * ys + r;
      st1<T>(yp, a0); st1<T>(yp + ys, a1); st1<T>(yp + 2 * ys, a2); st1<T>(yp + 3 * ys, a3);
    }
    for (; f < nf; ++f) {
      float a = 0.f;
#pragma unroll
      for (int e = 0; e < kFmE; ++e)
        if (e < n) a = fmaf(ww[e], ld1<T>(x + f * xs + jj[e]), a);
      st1<T>(y + f * ys + r, a);
    }
    return;
  }
  // long rows: entries re-read (from cache) for every group of 4 fields
  for (int64_t f = 0; f < nf; f += 4) {
    const int nq = (int)(nf - f < 4 ? nf - f : 4);
    float a[4] = {0.f, 0.f, 0.f, 0.f};
    for (int32_t k = k0; k < k1; ++k) {
      const int32_t j = __ldg(idx + k);
      const float wk = __ldg(w + k);
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (q < nq) a[q] = fmaf(wk, ld1<T>(x + (f + q) * xs + j), a[q]);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (q < nq) st1<T>(y + (f + q) * ys + r, a[q]);
  }
}

// ------------------------------------------------------------------ generic strides

template <class T>
__global__ void k_spmm_generic(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                               const float* __restrict__ w, int64_t nrows, const T* __restrict__ x, int64_t xsc,
                               int64_t xsf, T* __restrict__ y, int64_t ysc, int64_t ysf, int64_t f0) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int64_t f = f0 + blockIdx.y;
  float acc = 0.f;
  for (int32_t k = ptr[r]; k < ptr[r + 1]; ++k) acc = fmaf(w[k], ld1<T>(x + (int64_t)idx[k] * xsc + f * xsf), acc);
  st1<T>(y + r * ysc + f * ysf, acc);
}

int num_sms() {
  static int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
  }();
  return n;
}

// ------------------------------------------------------------------ merge-path (cell-major)

// Each warp walks tasks of about kTaskNnz consecutive entries.  Lanes load 32
// (column, weight) entries with one coalesced load each, and the warp reads
// which of them start a row from the row-start bitmap (one bit per entry);
// then every entry is broadcast and the whole warp gathers that cell's 128
// fields (4 per lane, 16-byte loads); 8 gathers are issued before they are
// consumed.  Rows are accumulated in entry order and written when the row
// changes (to the next row, or to nextrow[row] when some rows have no
// entries); a row that began in an earlier task or continues into a later one
// is written to the task's carry slot (0 = first row, 1 = last row) for
// k_cm_fixup.
//
// The gathers in flight hold the raw loads (16 bytes of 4 FP32 fields, 8 bytes
// of 4 BF16 fields), converted to FP32 when consumed.  kInFlight is the count
// of the persistent batch launch (k_batch_apply, at kBatchMinBlocks blocks per
// SM); the autotuner's candidates (CmVariant) set those of k_cm_nnz.
template <class T> struct CmGather;
template <> struct CmGather<float> {
  using Raw = float4;
  static constexpr int kInFlight = 4;
  // (offset, weight) pairs by two shuffles per entry (latency-bound: the
  // shared-memory staging measured 0.402 against 0.396 ms per step)
  static constexpr bool kStage = false;
  // k_batch_apply holds the vector, strided and row paths at once; at 4 blocks
  // per SM (64 registers) it spills a little, and still beats 3 blocks (0.58
  // against 0.73 ms for a batch of 32 uneven pairs)
  static constexpr int kBatchMinBlocks = 4;
  static __device__ __forceinline__ Raw load(const char* base, uint32_t off) {
    return __ldg(reinterpret_cast<const float4*>(base + off));
  }
  static __device__ __forceinline__ float4 widen(Raw r) { return r; }
};
template <> struct CmGather<__nv_bfloat16> {
  using Raw = uint2;
  static constexpr int kInFlight = 8;
  // (offset, weight) pairs by one broadcast shared load per entry: the BF16
  // kernel is closer to its issue limit (0.320 against 0.333 ms per step)
  static constexpr bool kStage = true;
  static constexpr int kBatchMinBlocks = 3;
  static __device__ __forceinline__ Raw load(const char* base, uint32_t off) {
    return __ldg(reinterpret_cast<const uint2*>(base + off));
  }
  // a BF16 value is the upper half of its FP32 value: one shift (the element
  // in the low half) and one mask (the element in the high half) per pair
  static __device__ __forceinline__ float4 widen(Raw u) {
    return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xffff0000u),
                       __uint_as_float(u.y << 16), __uint_as_float(u.y & 0xffff0000u));
  }
};

// Rows that are not 16-byte 4-vectors (a field count or stride not a multiple
// of 4): lane l takes fields f0 + l + 32 t (t < 4) of a 128-field pass, bit t
// of `onm` set when that field exists, so that each of the four scalar loads
// of a gather reads 32 consecutive elements across the warp.
template <class T>
__device__ __forceinline__ float4 cm_strided_load(const char* base, uint32_t off, int onm) {
  const T* p = reinterpret_cast<const T*>(base + off);
  float4 v;
  v.x = (onm & 1) ? ld1<T>(p) : 0.f;
  v.y = (onm & 2) ? ld1<T>(p + 32) : 0.f;
  v.z = (onm & 4) ? ld1<T>(p + 64) : 0.f;
  v.w = (onm & 8) ? ld1<T>(p + 96) : 0.f;
  return v;
}

// One merge-path task of one 128-field pass, by one warp.  `xb` is the lane's
// base (its first field of cell 0), `fo` that field, `onm` which of its 4
// fields exist (bit t); B gathers are in flight.  kVec: the lane's fields are
// fo .. fo + 3 (16-byte FP32 / 8-byte BF16 vectors); otherwise fo + 32 t.
// `stg`: the warp's 64-slot staging in shared memory; with CmGather<T>::kStage
// each 32-entry chunk's (source offset, weight) pairs go there, so that an
// entry costs one broadcast 8-byte shared load instead of two shuffles.
template <class T, bool kGaps, int B, bool kVec = true>
__device__ __forceinline__ void cm_task(int64_t task, const int4* __restrict__ tasks, const int2* __restrict__ tslot,
                                        const int32_t* __restrict__ idx, const uint32_t* __restrict__ rbits,
                                        const int32_t* __restrict__ nextrow, const float* __restrict__ w,
                                        const char* xb, uint32_t cstride, T* __restrict__ y, int64_t ys, int64_t fo,
                                        int onm, float* __restrict__ carry, int lane, uint2* __restrict__ stg) {
  using G = CmGather<T>;
  using Raw = typename std::conditional<kVec, typename G::Raw, float4>::type;
  const int4 tr = __ldg(tasks + task);
  const int32_t e0 = tr.x, e1 = tr.y;
  if (e0 >= e1) return;  // warp-uniform
  const int32_t first = tr.z & 0x7fffffff;
  // rows written to the carry slots: the first row if it began in an earlier
  // task, the last row if it continues into a later one (-1: no such row)
  const int32_t carry_first = tr.z < 0 ? first : -1;
  const int32_t carry_last = tr.w < 0 ? (tr.w & 0x7fffffff) : -1;
  const int2 slot = (tr.z | tr.w) < 0 ? __ldg(tslot + task) : make_int2(-1, -1);
  int32_t cur = first;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  auto flush = [&](int32_t row) {
    if (!onm) return;
    if (row == carry_first || row == carry_last) {
      float* c = carry + (int64_t)(row == carry_first ? slot.x : slot.y) * 128;
      if (kVec) {
        *reinterpret_cast<float4*>(c + lane * 4) = acc;
      } else {
        c += lane;
        if (onm & 1) c[0] = acc.x;
        if (onm & 2) c[32] = acc.y;
        if (onm & 4) c[64] = acc.z;
        if (onm & 8) c[96] = acc.w;
      }
    } else if (kVec) {
      st4<T>(y + (int64_t)row * ys + fo, acc);
    } else {
      T* yp = y + (int64_t)row * ys + fo;
      if (onm & 1) st1<T>(yp, acc.x);
      if (onm & 2) st1<T>(yp + 32, acc.y);
      if (onm & 4) st1<T>(yp + 64, acc.z);
      if (onm & 8) st1<T>(yp + 96, acc.w);
    }
  };
  // the chunk at c0: lane's byte offset of its source cell and weight, and
  // the row starts among the chunk's entries (bit k: entry c0 + k)
  auto load = [&](int32_t c0, uint32_t& starts, uint32_t& o, float& wt) {
    const int32_t e = c0 + lane;
    const bool valid = e < e1;
    o = valid ? (uint32_t)__ldg(idx + e) * cstride : 0u;
    wt = valid ? __ldg(w + e) : 0.f;
    starts = __funnelshift_r(__ldg(rbits + (c0 >> 5)), __ldg(rbits + (c0 >> 5) + 1), (uint32_t)c0 & 31u);
    if (e1 - c0 < 32) starts &= (1u << (e1 - c0)) - 1u;
  };
  uint32_t starts;
  uint32_t myo;
  float myw;
  load(e0, starts, myo, myw);
  starts &= ~1u;  // entry e0 belongs to row `first` (already current)
  // slots 0..31 and 32..63 alternate between chunks; the warp barrier after a
  // chunk's pairs are written also ends every read of the other half
  int half = 0;
  if constexpr (G::kStage) {
    __syncwarp();
    stg[lane] = make_uint2(myo, __float_as_uint(myw));
    __syncwarp();
  }
  for (int32_t c0 = e0; c0 < e1; c0 += 32) {
    // the next chunk's entries load while this one is gathered
    uint32_t nstarts = 0u, no = 0u;
    float nwt = 0.f;
    if (c0 + 32 < e1) load(c0 + 32, nstarts, no, nwt);
    const unsigned newrow = starts;
    const int n = e1 - c0 < 32 ? e1 - c0 : 32;
    const uint2* sp = stg + half;
    // B entries of the chunk from entry k: their gathers first, then their FMAs
    auto group = [&](int k, int nn) {
      Raw v[B];
      float ww[B];
#pragma unroll
      for (int h = 0; h < B; ++h) {
        uint32_t o;
        if constexpr (G::kStage) {
          const uint2 ow = sp[(k + h) & 31];
          o = ow.x;
          ww[h] = __uint_as_float(ow.y);
        } else {
          o = __shfl_sync(0xffffffffu, myo, (k + h) & 31);
          ww[h] = __shfl_sync(0xffffffffu, myw, (k + h) & 31);
        }
        // past-the-end entries load cell 0 with weight 0
        if constexpr (kVec) v[h] = G::load(xb, o);
        else v[h] = cm_strided_load<T>(xb, o, onm);
      }
#pragma unroll
      for (int h = 0; h < B; ++h) {
        if (k + h >= nn) break;  // no FMA with past-the-end data (0 * Inf would poison the row)
        if ((newrow >> (k + h)) & 1u) {
          flush(cur);
          // kGaps: the next row with entries (nextrow), when the layout has one
          cur = kGaps ? (nextrow ? __ldg(nextrow + cur) : cur + 1) : cur + 1;
          acc = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        float4 xv;
        if constexpr (kVec) xv = G::widen(v[h]);
        else xv = v[h];
        acc.x = fmaf(ww[h], xv.x, acc.x);
        acc.y = fmaf(ww[h], xv.y, acc.y);
        acc.z = fmaf(ww[h], xv.z, acc.z);
        acc.w = fmaf(ww[h], xv.w, acc.w);
      }
    };
    if (n == 32) {
      // a full chunk, unrolled: shuffle lanes and row-start bits are constants
#pragma unroll
      for (int k = 0; k < 32; k += B) group(k, 32);
    } else {
      for (int k = 0; k < n; k += B) group(k, n);
    }
    starts = nstarts;
    if constexpr (G::kStage) {
      half ^= 32;
      stg[half + lane] = make_uint2(no, __float_as_uint(nwt));
      __syncwarp();
    } else {
      myo = no;
      myw = nwt;
    }
  }
  flush(cur);
}

// The lane's field base of one 128-field pass starting at f0, its first
// field and which of its 4 fields exist.
template <class T, bool kVec>
__device__ __forceinline__ const char* cm_lane_base(const T* x, int64_t f0, int64_t nf, int lane, int64_t& fo,
                                                    int& onm) {
  if (kVec) {
    const int64_t f = f0 + (int64_t)lane * 4;
    onm = f < nf ? 0xf : 0;  // nf is a multiple of 4
    fo = f < nf ? f : f0;
  } else {
    const int64_t rem = nf - f0 - lane;
    onm = (rem > 0 ? 1 : 0) | (rem > 32 ? 2 : 0) | (rem > 64 ? 4 : 0) | (rem > 96 ? 8 : 0);
    fo = rem > 0 ? f0 + lane : f0;
  }
  return reinterpret_cast<const char*>(x + fo);
}

template <class T, bool kGaps, int B = CmGather<T>::kInFlight, int MINB = 3, bool kVec = true>
__global__ void __launch_bounds__(256, MINB)
    k_cm_nnz(const int4* __restrict__ tasks, const int2* __restrict__ tslot, const int32_t* __restrict__ idx,
             const uint32_t* __restrict__ rbits, const int32_t* __restrict__ nextrow, const float* __restrict__ w,
             int64_t ntasks, const T* __restrict__ x,
             int64_t xs, T* __restrict__ y, int64_t ys, int64_t f0, int64_t nf, float* __restrict__ carry) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int64_t fo;
  int onm;
  // per-lane base of this lane's fields; cell j adds j * xs elements (32-bit byte offset)
  const char* xb = cm_lane_base<T, kVec>(x, f0, nf, lane, fo, onm);
  const uint32_t cstride = (uint32_t)(xs * (int64_t)sizeof(T));
  __shared__ uint2 s_stage[CmGather<T>::kStage ? 8 : 1][64];
  uint2* stg = CmGather<T>::kStage ? s_stage[threadIdx.x >> 5] : nullptr;
  for (int64_t task = gw; task < ntasks; task += nw)
    cm_task<T, kGaps, B, kVec>(task, tasks, tslot, idx, rbits, nextrow, w, xb, cstride, y, ys, fo, onm, carry, lane,
                               stg);
}

// Rows cut between tasks: sum their pieces in task order (deterministic).
template <class T>
__global__ void k_cm_fixup(const int32_t* __restrict__ split, int64_t nsplit, const float* __restrict__ carry,
                           T* __restrict__ y, int64_t ys, int64_t f0, int64_t nf) {
  const int64_t wi = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wi >= nsplit) return;
  const int32_t row = split[3 * wi], s0 = split[3 * wi + 1], pieces = split[3 * wi + 2];
  const int64_t f = f0 + (int64_t)lane * 4;
  if (f >= nf) return;
  float4 s = *reinterpret_cast<const float4*>(carry + (int64_t)s0 * 128 + lane * 4);
  for (int32_t k = 1; k < pieces; ++k) {
    const float4 c = *reinterpret_cast<const float4*>(carry + (int64_t)(s0 + k) * 128 + lane * 4);
    s.x += c.x; s.y += c.y; s.z += c.z; s.w += c.w;
  }
  st4<T>(y + (int64_t)row * ys + f, s);
}

// The same for rows that are not 4-vectors: lane l sums fields l + 32 t of the
// pass, as cm_task's strided layout wrote them.
template <class T>
__global__ void k_cm_fixup_s(const int32_t* __restrict__ split, int64_t nsplit, const float* __restrict__ carry,
                             T* __restrict__ y, int64_t ys, int64_t f0, int64_t nf) {
  const int64_t wi = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wi >= nsplit) return;
  const int32_t row = split[3 * wi], s0 = split[3 * wi + 1], pieces = split[3 * wi + 2];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int p = lane + 32 * t;
    if (f0 + p >= nf) break;
    float acc = carry[(int64_t)s0 * 128 + p];
    for (int32_t k = 1; k < pieces; ++k) acc += carry[(int64_t)(s0 + k) * 128 + p];
    st1<T>(y + (int64_t)row * ys + f0 + p, acc);
  }
}

// The merge-path kernel over all 128-field passes, the fixup of rows cut
// between tasks, and zeros for rows without entries.  `carry` holds
// nslots * 128 floats when the layout has rows cut between tasks.
//
// The autotuner's candidates for this kernel (index 0 is the default): the
// gathers in flight per warp and the blocks of 8 warps per SM (the register
// cap follows: 80 registers at 3, 64 at 4, 128 at 2).  Every candidate sums
// the same entries in the same order, so the choice never changes a result.
constexpr int kCmVariants = 4;
template <class T> struct CmVariant;
template <> struct CmVariant<float> {
  static constexpr int B[kCmVariants] = {4, 8, 16, 12};
  static constexpr int MINB[kCmVariants] = {4, 3, 2, 2};
};
template <> struct CmVariant<__nv_bfloat16> {
  static constexpr int B[kCmVariants] = {8, 16, 4, 24};
  static constexpr int MINB[kCmVariants] = {3, 3, 4, 2};
};

template <class T>
void cm_nnz_passes(const DevCsr& c, const float* w, const T* x, int64_t xs, T* y, int64_t ys, int64_t nf,
                   float* carry, cudaStream_t st, int variant = 0, bool vec = true);

// The device part of an autotuner key: name and SM count of the current device.
std::string device_key() {
  static std::mutex mu;
  static std::vector<std::string> names;
  int dev = 0;
  CRG_CHECK_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if ((int)names.size() <= dev) names.resize(dev + 1);
  if (names[dev].empty()) {
    cudaDeviceProp prop;
    CRG_CHECK_CUDA(cudaGetDeviceProperties(&prop, dev));
    char b[320];
    snprintf(b, sizeof b, "%s/%dsm", prop.name, prop.multiProcessorCount);
    for (char* q = b; *q; ++q)
      if (*q == ' ' || *q == '\t') *q = '_';
    names[dev] = b;
  }
  return names[dev];
}

std::string matrix_key(const char* family, const DevCsr& c, const char* dtype, int64_t nf) {
  char b[256];
  snprintf(b, sizeof b, "%s %s rows=%lld cols=%lld nnz=%lld %s K=%lld", family, device_key().c_str(),
           (long long)c.nrows, (long long)c.ncols, (long long)c.nnz, dtype, (long long)nf);
  return b;
}

// The fastest of n candidates for `key`: the cached choice, else (outside
// stream capture) each candidate run once to warm up and twice timed with
// CUDA events on `st`, in turn, and the choice stored.  Candidate 0 when the
// tuner is off or the stream is capturing.  run(i) must leave the same result
// for every i.
template <class F>
int tune_choose(const std::string& key, int n, cudaStream_t st, F run) {
  int choice = 0;
  if (n <= 1 || !tune_enabled()) return 0;
  if (tune_lookup(key, choice)) return choice < n ? choice : 0;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CRG_CHECK_CUDA(cudaStreamIsCapturing(st, &cs));
  if (cs != cudaStreamCaptureStatusNone) return 0;
  std::vector<cudaEvent_t> ev(2 * n, nullptr);
  struct Guard {
    std::vector<cudaEvent_t>& v;
    ~Guard() {
      for (auto e : v)
        if (e) cudaEventDestroy(e);
    }
  } guard{ev};
  for (auto& e : ev) CRG_CHECK_CUDA(cudaEventCreate(&e));
  std::vector<float> ms(n, 0.f);
  for (int i = 0; i < n; ++i) run(i);
  for (int rep = 0; rep < 2; ++rep) {
    for (int i = 0; i < n; ++i) {
      CRG_CHECK_CUDA(cudaEventRecord(ev[2 * i], st));
      run(i);
      CRG_CHECK_CUDA(cudaEventRecord(ev[2 * i + 1], st));
    }
    CRG_CHECK_CUDA(cudaEventSynchronize(ev[2 * n - 1]));
    for (int i = 0; i < n; ++i) {
      float t = 0.f;
      CRG_CHECK_CUDA(cudaEventElapsedTime(&t, ev[2 * i], ev[2 * i + 1]));
      ms[i] += t;
    }
  }
  for (int i = 1; i < n; ++i)
    if (ms[i] < ms[choice]) choice = i;
  tune_store(key, choice, ms.data(), n);
  return choice;
}

template <class T> const char* dtype_name();
template <> const char* dtype_name<float>() { return "f32"; }
template <> const char* dtype_name<__nv_bfloat16>() { return "bf16"; }

template <class T>
void launch_cm_nnz(const DevCsr& c, const float* w, const T* x, int64_t xs, T* y, int64_t ys, int64_t nf,
                   cudaStream_t st, bool vec) {
  float* carry = nullptr;
  if (c.nslots) CRG_CHECK_CUDA(cudaMallocAsync((void**)&carry, sizeof(float) * c.nslots * 128, st));
  const int v = tune_choose(matrix_key(vec ? "cm_nnz" : "cm_nnz_strided", c, dtype_name<T>(), nf), kCmVariants, st,
                            [&](int i) { cm_nnz_passes<T>(c, w, x, xs, y, ys, nf, carry, st, i, vec); });
  cm_nnz_passes<T>(c, w, x, xs, y, ys, nf, carry, st, v, vec);
  if (carry) CRG_CHECK_CUDA(cudaFreeAsync(carry, st));
}

// Merge-path tasks for cell-major fields, 2 to 31 per cell: G lanes (4 fields
// each) per lane group, every lane group taking two consecutive entries of a
// chunk of 64 / G, so that a warp gathers 64 / G source rows per two loads and
// a polar row of hundreds of entries is spread over its tasks like any other.
// A lane group adds its two entries' products when they share a row; a
// segmented inclusive scan over the groups (Kogge-Stone, rows from erow) then
// sums every row's run of entries inside the chunk; the group holding a row's
// last entry of the chunk adds what earlier chunks carried and writes the row
// -- to its carry slot when the row is cut between tasks (k_cm_fixup sums
// those).  The chunk's last row stays open until the next chunk shows whether
// it continues.  Order of the FP32 sums: pairs, then a fixed scan tree per
// chunk, the chunks in entry order: the same bits for a given matrix and field
// count (the chunk's width follows the lanes per entry), every time.
template <class T, int G, bool kVec>
__global__ void __launch_bounds__(256, 4)
    k_cm_narrow(const int4* __restrict__ tasks, const int2* __restrict__ tslot, const int32_t* __restrict__ idx,
                const int32_t* __restrict__ erow, const float* __restrict__ w, int64_t ntasks,
                const T* __restrict__ x, int64_t xs, T* __restrict__ y, int64_t ys, int64_t nf,
                float* __restrict__ carry) {
  constexpr int E = 32 / G;
  constexpr unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31, i = lane / G, g = lane % G;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int f = 4 * g;  // the lane's first field
  const int onm = (f < nf ? 1 : 0) | (f + 1 < nf ? 2 : 0) | (f + 2 < nf ? 4 : 0) | (f + 3 < nf ? 8 : 0);
  for (int64_t task = gw; task < ntasks; task += nw) {
    const int4 tr = __ldg(tasks + task);
    const int32_t e0 = tr.x, e1 = tr.y;
    if (e0 >= e1) continue;  // warp-uniform
    const int32_t carry_first = tr.z < 0 ? (tr.z & 0x7fffffff) : -1;
    const int32_t carry_last = tr.w < 0 ? (tr.w & 0x7fffffff) : -1;
    const int2 slot = (tr.z | tr.w) < 0 ? __ldg(tslot + task) : make_int2(-1, -1);
    auto write = [&](int32_t row, float4 v) {
      if (!onm) return;
      if (row == carry_first || row == carry_last) {
        float* c = carry + (int64_t)(row == carry_first ? slot.x : slot.y) * 128 + f;
        if (onm & 1) c[0] = v.x;
        if (onm & 2) c[1] = v.y;
        if (onm & 4) c[2] = v.z;
        if (onm & 8) c[3] = v.w;
      } else if (kVec) {
        st4<T>(y + (int64_t)row * ys + f, v);
      } else {
        T* yp = y + (int64_t)row * ys + f;
        if (onm & 1) st1<T>(yp, v.x);
        if (onm & 2) st1<T>(yp + 1, v.y);
        if (onm & 4) st1<T>(yp + 2, v.z);
        if (onm & 8) st1<T>(yp + 3, v.w);
      }
    };
    int32_t open_row = -1;  // the row the previous chunk ended in, not written yet
    float4 open = make_float4(0.f, 0.f, 0.f, 0.f);
    // entry e of the task for this lane group: its row (-1 past the task's
    // end), source cell and weight, and its gathered fields
    auto meta = [&](int32_t e, int32_t& row, int32_t& col, float& wt) {
      const bool valid = e < e1;
      row = valid ? __ldg(erow + e) : -1;
      col = valid ? __ldg(idx + e) : 0;
      wt = valid ? __ldg(w + e) : 0.f;
    };
    auto gather = [&](int32_t row, int32_t col) {
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (row >= 0 && onm) {
        const T* xp = x + (int64_t)col * xs + f;
        if (kVec) {
          v = ld4<T>(xp);
        } else {
          v.x = (onm & 1) ? ld1<T>(xp) : 0.f;
          v.y = (onm & 2) ? ld1<T>(xp + 1) : 0.f;
          v.z = (onm & 4) ? ld1<T>(xp + 2) : 0.f;
          v.w = (onm & 8) ? ld1<T>(xp + 3) : 0.f;
        }
      }
      return v;
    };
    auto add = [](float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); };
    auto mul = [](float wt, float4 v) { return make_float4(wt * v.x, wt * v.y, wt * v.z, wt * v.w); };
    // Chunks of 2 E entries: lane group i takes entries 2i (a) and 2i + 1 (b).
    // The next chunk's indices and gathers are in flight while a chunk is summed.
    int32_t ra, ca, rb, cb;
    float wa, wb;
    meta(e0 + 2 * i, ra, ca, wa);
    meta(e0 + 2 * i + 1, rb, cb, wb);
    float4 va = gather(ra, ca), vb = gather(rb, cb);
    for (int32_t c0 = e0; c0 < e1; c0 += 2 * E) {
      int32_t na, nca, nb, ncb;
      float nwa, nwb;
      meta(c0 + 2 * E + 2 * i, na, nca, nwa);
      meta(c0 + 2 * E + 2 * i + 1, nb, ncb, nwb);
      const float4 nva = gather(na, nca), nvb = gather(nb, ncb);
      const float4 pa = mul(wa, va), pb = mul(wb, vb);
      const int32_t row0 = __shfl_sync(kFull, ra, 0);
      // the open row ended where this chunk begins: write it (group 0)
      if (open_row >= 0 && row0 != open_row) {
        if (i == 0) write(open_row, open);
        open_row = -1;
      }
      // a starts a run: the chunk's first entry, or a row change from the
      // previous entry (b of group i - 1); the group's last run (the one b is
      // in) starts inside it when b's row differs from a's, or at a
      const int32_t prev = __shfl_up_sync(kFull, rb, G);
      const bool head_a = i == 0 || ra != prev;
      const bool same = ra == rb;
      bool h = !same || head_a;
      float4 t = same ? add(pa, pb) : pb;
      // segmented inclusive scan of the groups' last runs
#pragma unroll
      for (int d = 1; d < E; d <<= 1) {
        const float qx = __shfl_up_sync(kFull, t.x, d * G), qy = __shfl_up_sync(kFull, t.y, d * G);
        const float qz = __shfl_up_sync(kFull, t.z, d * G), qw = __shfl_up_sync(kFull, t.w, d * G);
        const bool qh = __shfl_up_sync(kFull, h ? 1 : 0, d * G) != 0;
        if (i >= d && !h) {
          t = make_float4(qx + t.x, qy + t.y, qz + t.z, qw + t.w);
          h = qh;
        }
      }
      // a's run, when it ends at a: the previous group's scan (same run) + pa
      const float4 sp = make_float4(__shfl_up_sync(kFull, t.x, G), __shfl_up_sync(kFull, t.y, G),
                                    __shfl_up_sync(kFull, t.z, G), __shfl_up_sync(kFull, t.w, G));
      if (ra >= 0 && !same) {
        float4 ta = head_a ? pa : add(sp, pa);
        if (ra == open_row) ta = add(open, ta);
        write(ra, ta);
      }
      // b's run so far (with what earlier chunks carried); written when the
      // next entry starts another row, kept open at the chunk's end
      if (rb == open_row) t = add(open, t);
      const int32_t next = __shfl_down_sync(kFull, ra, G);
      if (rb >= 0 && i < E - 1 && next != rb) write(rb, t);
      const int last = (E - 1) * G + g;
      open_row = __shfl_sync(kFull, rb, last);  // -1 when the chunk was not full: all its rows are written
      open = make_float4(__shfl_sync(kFull, t.x, last), __shfl_sync(kFull, t.y, last),
                         __shfl_sync(kFull, t.z, last), __shfl_sync(kFull, t.w, last));
      ra = na;
      rb = nb;
      wa = nwa;
      wb = nwb;
      va = nva;
      vb = nvb;
    }
    if (open_row >= 0 && i == 0) write(open_row, open);
  }
}

// Rows without entries produce zero output (the row gather writes nothing for them).
template <class T>
__global__ void k_zero_empty_cm(const int32_t* __restrict__ ptr, int64_t n, T* __restrict__ y, int64_t ys, int64_t nf) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n || ptr[r + 1] > ptr[r]) return;
  for (int64_t f = 0; f < nf; ++f) st1<T>(y + r * ys + f, 0.f);
}

template <class T, int V, bool kVec>
void cm_nnz_launch(const DevCsr& c, const float* w, const T* x, int64_t xs, T* y, int64_t ys, int64_t f0, int64_t nf,
                   float* carry, cudaStream_t st) {
  constexpr int B = CmVariant<T>::B[V], MINB = CmVariant<T>::MINB[V];
  const int64_t warps = std::min<int64_t>(c.ntasks, (int64_t)num_sms() * 8 * MINB);  // MINB blocks of 8 warps per SM
  if (c.nextrow)
    k_cm_nnz<T, true, B, MINB, kVec><<<nblk(warps * 32, 256), 256, 0, st>>>(
        c.tasks, c.tslot, c.idx, c.rbits, c.nextrow, w, c.ntasks, x, xs, y, ys, f0, nf, carry);
  else
    k_cm_nnz<T, false, B, MINB, kVec><<<nblk(warps * 32, 256), 256, 0, st>>>(
        c.tasks, c.tslot, c.idx, c.rbits, nullptr, w, c.ntasks, x, xs, y, ys, f0, nf, carry);
}

template <class T, bool kVec>
void cm_nnz_variant(int variant, const DevCsr& c, const float* w, const T* x, int64_t xs, T* y, int64_t ys,
                    int64_t f0, int64_t nf, float* carry, cudaStream_t st) {
  switch (variant) {
    case 1: cm_nnz_launch<T, 1, kVec>(c, w, x, xs, y, ys, f0, nf, carry, st); break;
    case 2: cm_nnz_launch<T, 2, kVec>(c, w, x, xs, y, ys, f0, nf, carry, st); break;
    case 3: cm_nnz_launch<T, 3, kVec>(c, w, x, xs, y, ys, f0, nf, carry, st); break;
    default: cm_nnz_launch<T, 0, kVec>(c, w, x, xs, y, ys, f0, nf, carry, st); break;
  }
}

template <class T>
void cm_nnz_passes(const DevCsr& c, const float* w, const T* x, int64_t xs, T* y, int64_t ys, int64_t nf,
                   float* carry, cudaStream_t st, int variant, bool vec) {
  for (int64_t f0 = 0; f0 < nf; f0 += 128) {
    if (c.ntasks) {
      if (vec) cm_nnz_variant<T, true>(variant, c, w, x, xs, y, ys, f0, nf, carry, st);
      else cm_nnz_variant<T, false>(variant, c, w, x, xs, y, ys, f0, nf, carry, st);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
    if (c.nsplit) {
      if (vec) k_cm_fixup<T><<<nblk(c.nsplit * 32, 256), 256, 0, st>>>(c.split, c.nsplit, carry, y, ys, f0, nf);
      else k_cm_fixup_s<T><<<nblk(c.nsplit * 32, 256), 256, 0, st>>>(c.split, c.nsplit, carry, y, ys, f0, nf);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
  }
  if (c.nempty) {
    k_zero_empty_cm<T><<<nblk(c.nrows, 256), 256, 0, st>>>(c.ptr, c.nrows, y, ys, nf);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
}

// 2 to 31 cell-major fields: k_cm_narrow over
// the merge-path tasks, then the cut rows' sums and the empty rows.  `carry`:
// scratch of c.nslots * 128 floats, or NULL to take it from the stream's pool.
template <class T>
void launch_cm_narrow(const DevCsr& c, const float* w, const T* x, int64_t xs, T* y, int64_t ys, int64_t nf,
                      cudaStream_t st, bool vec, float* carry_given = nullptr) {
  float* carry = carry_given;
  if (!carry && c.nslots) CRG_CHECK_CUDA(cudaMallocAsync((void**)&carry, sizeof(float) * c.nslots * 128, st));
  if (c.ntasks) {
    const int64_t lanes = (nf + 3) / 4;
    int G = 1;
    while (G < lanes) G <<= 1;
    const int64_t warps = std::min<int64_t>(c.ntasks, (int64_t)num_sms() * 8 * 4);
    const unsigned blocks = nblk(warps * 32, 256);
#define CRG_NARROW(GG)                                                                                          \
  if (vec)                                                                                                      \
    k_cm_narrow<T, GG, true><<<blocks, 256, 0, st>>>(c.tasks, c.tslot, c.idx, c.erow, w, c.ntasks, x, xs, y, ys, nf, \
                                                     carry);                                                    \
  else                                                                                                          \
    k_cm_narrow<T, GG, false><<<blocks, 256, 0, st>>>(c.tasks, c.tslot, c.idx, c.erow, w, c.ntasks, x, xs, y, ys,   \
                                                      nf, carry);
    switch (G) {
      case 1: CRG_NARROW(1) break;
      case 2: CRG_NARROW(2) break;
      case 4: CRG_NARROW(4) break;
      default: CRG_NARROW(8) break;
    }
#undef CRG_NARROW
    CRG_CHECK_CUDA(cudaGetLastError());
  }
  if (c.nsplit) {
    if (vec) k_cm_fixup<T><<<nblk(c.nsplit * 32, 256), 256, 0, st>>>(c.split, c.nsplit, carry, y, ys, 0, nf);
    else k_cm_fixup_s<T><<<nblk(c.nsplit * 32, 256), 256, 0, st>>>(c.split, c.nsplit, carry, y, ys, 0, nf);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
  if (c.nempty) {
    k_zero_empty_cm<T><<<nblk(c.nrows, 256), 256, 0, st>>>(c.ptr, c.nrows, y, ys, nf);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
  if (!carry_given && carry) CRG_CHECK_CUDA(cudaFreeAsync(carry, st));
}

// Kernel choice for FP32/BF16 fields.  CRG_SPMM_PATH selects an alternative
// for tuning and profiling: "rows" (the row kernels for every layout, no
// merge-path, no transposes); unset = automatic.
enum class SpmmPath { kAuto, kRows };

inline SpmmPath spmm_path() {
  static const SpmmPath p = [] {
    const char* e = getenv("CRG_SPMM_PATH");
    return (e && strcmp(e, "rows") == 0) ? SpmmPath::kRows : SpmmPath::kAuto;
  }();
  return p;
}

// Whether launch_f32 applies these fields with k_cm_narrow: 2 to 31 fields
// side by side (at 32 it measured the same as the merge path: 0.303 ms for the
// HEALPix 256 <-> 0.25-degree step).  A single field keeps the row kernel's sequential row sums,
// the same as each field of a field-major apply (whose host pipeline applies
// its fields in chunks, down to one field at a time).
bool narrow_path(SpmmPath path, bool cell_major, int64_t nf) {
  return path == SpmmPath::kAuto && cell_major && nf < 32;
}

// k_cm_rows with RB rows per lane group; the autotuner picks RB (the
// candidates 2, 1, 4; every row is summed in entry order whatever RB).
template <class T>
void cm_rows_rb(const DevCsr& c, const float* w, const T* x, int64_t xs, T* y, int64_t ys, int64_t nf, int RB,
                cudaStream_t st);

template <class T>
void launch_cm_rows(const DevCsr& c, const float* w, const T* x, int64_t xs, T* y, int64_t ys, int64_t nf,
                    cudaStream_t st) {
  static const int kRB[3] = {2, 1, 4};
  const int v = tune_choose(matrix_key("cm_rows", c, dtype_name<T>(), nf), 3, st,
                            [&](int i) { cm_rows_rb<T>(c, w, x, xs, y, ys, nf, kRB[i], st); });
  cm_rows_rb<T>(c, w, x, xs, y, ys, nf, kRB[v], st);
}

template <class T>
void cm_rows_rb(const DevCsr& c, const float* w, const T* x, int64_t xs, T* y, int64_t ys, int64_t nf, int RB,
                cudaStream_t st) {
  const int64_t n = c.nrows;
  const int64_t lanes = (std::min<int64_t>(nf, 128) + 3) / 4;
  int G = 1;
  while (G < lanes) G <<= 1;
  const unsigned blocks = nblk((n + RB - 1) / RB * G, 256);
#define CRG_CM(GG, RR) k_cm_rows<T, GG, RR><<<blocks, 256, 0, st>>>(c.ptr, c.idx, w, n, nullptr, x, xs, y, ys, nf)
#define CRG_CM_RB(GG) \
  if (RB == 1) CRG_CM(GG, 1); else if (RB == 2) CRG_CM(GG, 2); else CRG_CM(GG, 4);
  switch (G) {
    case 1: CRG_CM_RB(1) break;
    case 2: CRG_CM_RB(2) break;
    case 4: CRG_CM_RB(4) break;
    case 8: CRG_CM_RB(8) break;
    case 16: CRG_CM_RB(16) break;
    default: CRG_CM_RB(32) break;
  }
#undef CRG_CM_RB
#undef CRG_CM
  CRG_CHECK_CUDA(cudaGetLastError());
}

// out[j * ldo + i] = in[i * ldi + j] for i < rows, j < cols: 32 x 32 tiles
// through shared memory, coalesced on both sides.
template <class T>
__global__ void k_transpose(const T* __restrict__ in, int64_t ldi, T* __restrict__ out, int64_t ldo, int64_t rows,
                            int64_t cols) {
  __shared__ T tile[32][33];
  const int64_t bi = (int64_t)blockIdx.y * 32, bj = (int64_t)blockIdx.x * 32;
  for (int k = threadIdx.y; k < 32; k += 8) {
    const int64_t i = bi + k, j = bj + threadIdx.x;
    if (i < rows && j < cols) tile[k][threadIdx.x] = in[i * ldi + j];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += 8) {
    const int64_t j = bj + k, i = bi + threadIdx.x;
    if (i < rows && j < cols) out[j * ldo + i] = tile[threadIdx.x][k];
  }
}

// The same for 4-aligned shapes: 64 x 64 tiles, 4-element vectors on both
// sides (16-byte loads and stores for FP32), 256 threads.  Each thread reads
// 4 consecutive columns of a row and writes 4 consecutive rows of a column.
template <class T> struct Vec4Of;
template <> struct Vec4Of<float> { using type = float4; };
template <> struct Vec4Of<__nv_bfloat16> { using type = uint2; };

template <class T>
__global__ void __launch_bounds__(256)
    k_transpose4(const T* __restrict__ in, int64_t ldi, T* __restrict__ out, int64_t ldo, int64_t rows,
                 int64_t cols) {
  using V = typename Vec4Of<T>::type;
  __shared__ T tile[64][65];
  const int64_t bi = (int64_t)blockIdx.y * 64, bj = (int64_t)blockIdx.x * 64;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // 16 vectors across, 16 rows down
  for (int k = ty; k < 64; k += 16) {
    const int64_t i = bi + k, j = bj + 4 * tx;
    if (i < rows && j < cols) {
      union { V v; T e[4]; } u;
      u.v = *reinterpret_cast<const V*>(in + i * ldi + j);  // cols % 4 == 0: all four inside
#pragma unroll
      for (int q = 0; q < 4; ++q) tile[k][4 * tx + q] = u.e[q];
    }
  }
  __syncthreads();
  for (int k = ty; k < 64; k += 16) {
    const int64_t j = bj + k, i = bi + 4 * tx;
    if (j < cols && i < rows) {
      union { V v; T e[4]; } u;
#pragma unroll
      for (int q = 0; q < 4; ++q) u.e[q] = tile[4 * tx + q][k];
      *reinterpret_cast<V*>(out + j * ldo + i) = u.v;  // rows % 4 == 0
    }
  }
}

template <class T>
void launch_transpose(const T* in, int64_t ldi, T* out, int64_t ldo, int64_t rows, int64_t cols, cudaStream_t st) {
  const size_t vb = 4 * sizeof(T);
  if (rows % 4 == 0 && cols % 4 == 0 && ldi % 4 == 0 && ldo % 4 == 0 && (uintptr_t)in % vb == 0 &&
      (uintptr_t)out % vb == 0) {
    for (int64_t r0 = 0; r0 < rows; r0 += 64 * 65535) {
      const int64_t rr = std::min<int64_t>(rows - r0, 64 * 65535);
      dim3 grid(nblk(cols, 64), nblk(rr, 64));
      k_transpose4<T><<<grid, 256, 0, st>>>(in + r0 * ldi, ldi, out + r0, ldo, rr, cols);
    }
    CRG_CHECK_CUDA(cudaGetLastError());
    return;
  }
  for (int64_t r0 = 0; r0 < rows; r0 += 32 * 65535) {
    const int64_t rr = std::min<int64_t>(rows - r0, 32 * 65535);
    dim3 grid(nblk(cols, 32), nblk(rr, 32));
    k_transpose<T><<<grid, dim3(32, 8), 0, st>>>(in + r0 * ldi, ldi, out + r0, ldo, rr, cols);
  }
  CRG_CHECK_CUDA(cudaGetLastError());
}

// One launch of k_cm_rows_f64: G lanes per row, batches of KB entries (0: G
// at a time).
template <int G, int KB>
void cm_f64_rows(const DevCsr& c, bool vec, const double* x, int64_t xs, double* y, int64_t ys, int64_t nf,
                 const double* rdiv, const double* rinv, cudaStream_t st) {
  const unsigned blocks = nblk(c.nrows * G, 256);
  if (vec)
    k_cm_rows_f64<G, true, KB><<<blocks, 256, 0, st>>>(c.ptr, c.idx, c.val, c.nrows, x, xs, y, ys, nf, rdiv, rinv);
  else
    k_cm_rows_f64<G, false, KB><<<blocks, 256, 0, st>>>(c.ptr, c.idx, c.val, c.nrows, x, xs, y, ys, nf, rdiv, rinv);
  CRG_CHECK_CUDA(cudaGetLastError());
}

// The autotuner's candidates for k_cm_rows_f64 with G lanes per row (index 0
// is the default): 0 loads G entries at a time; 1 batches of 8 entries (2 to
// 8 lanes per row); 2 batches of 4 (2 or 4 lanes per row).  Every candidate
// sums each field in entry order, so the choice never changes a result.
int cm_f64_variants(int G) { return G >= 2 && G <= 4 ? 3 : (G == 8 ? 2 : 1); }

template <int G>
void cm_f64_variant(int v, const DevCsr& c, bool vec, const double* x, int64_t xs, double* y, int64_t ys,
                    int64_t nf, const double* rdiv, const double* rinv, cudaStream_t st) {
  if constexpr (G >= 2 && G <= 8) {
    if (v == 1) return cm_f64_rows<G, 8>(c, vec, x, xs, y, ys, nf, rdiv, rinv, st);
  }
  if constexpr (G >= 2 && G <= 4) {
    if (v == 2) return cm_f64_rows<G, 4>(c, vec, x, xs, y, ys, nf, rdiv, rinv, st);
  }
  cm_f64_rows<G, 0>(c, vec, x, xs, y, ys, nf, rdiv, rinv, st);
}

// Cell-major FP64 fields (more than one): k_cm_rows_f64, G lanes per row.
// With the adjoint's column division, the input is divided once per element
// into a temporary first.
void launch_cm_f64(const DevCsr& c, bool adjoint, const double* div, const double* div_inv, const double* x,
                   int64_t xs, double* y, int64_t ys, int64_t nf, cudaStream_t st) {
  const int64_t n = c.nrows;
  if (n == 0 || nf == 0) return;
  const double* xin = x;
  int64_t xin_s = xs;
  double* tmp = nullptr;
  if (adjoint && div) {
    CRG_CHECK_CUDA(cudaMallocAsync((void**)&tmp, sizeof(double) * ((size_t)c.ncols * nf + 4), st));
    if (c.ncols) {
      k_div_cols_f64<<<nblk(c.ncols * nf, 256), 256, 0, st>>>(x, xs, c.ncols, nf, div, tmp);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
    xin = tmp;
    xin_s = nf;
  }
  const double* rdiv = adjoint ? nullptr : div;
  const double* rinv = adjoint ? nullptr : div_inv;
  if (nf <= 4) {
    // (at 8 fields this measured 0.91 against 0.79 ms per step for k_cm_rows_f64)
    const unsigned b = nblk(n, 128);
    if (nf <= 2) k_spmv_f64_k<2, 4><<<b, 128, 0, st>>>(c.ptr, c.idx, c.val, n, xin, xin_s, y, ys, (int)nf, rdiv, rinv);
    else k_spmv_f64_k<4, 4><<<b, 128, 0, st>>>(c.ptr, c.idx, c.val, n, xin, xin_s, y, ys, (int)nf, rdiv, rinv);
    CRG_CHECK_CUDA(cudaGetLastError());
    if (tmp) CRG_CHECK_CUDA(cudaFreeAsync(tmp, st));
    return;
  }
  const bool vec = nf % 4 == 0 && xin_s % 2 == 0 && ys % 2 == 0 && (uintptr_t)xin % 16 == 0 && (uintptr_t)y % 16 == 0;
  const int64_t lanes = (std::min<int64_t>(nf, 128) + 3) / 4;
  int G = 1;
  while (G < lanes) G <<= 1;
  auto run = [&](int v) {
    switch (G) {
      case 1: cm_f64_variant<1>(v, c, vec, xin, xin_s, y, ys, nf, rdiv, rinv, st); break;
      case 2: cm_f64_variant<2>(v, c, vec, xin, xin_s, y, ys, nf, rdiv, rinv, st); break;
      case 4: cm_f64_variant<4>(v, c, vec, xin, xin_s, y, ys, nf, rdiv, rinv, st); break;
      case 8: cm_f64_variant<8>(v, c, vec, xin, xin_s, y, ys, nf, rdiv, rinv, st); break;
      case 16: cm_f64_variant<16>(v, c, vec, xin, xin_s, y, ys, nf, rdiv, rinv, st); break;
      default: cm_f64_variant<32>(v, c, vec, xin, xin_s, y, ys, nf, rdiv, rinv, st); break;
    }
  };
  run(tune_choose(matrix_key(vec ? "cm_f64" : "cm_f64_strided", c, "f64", nf), cm_f64_variants(G), st, run));
  if (tmp) CRG_CHECK_CUDA(cudaFreeAsync(tmp, st));
}

template <class T>
void launch_f32(const DevCsr& c, bool normalize, bool adjoint, const T* x, int64_t xsc, int64_t xsf, T* y,
                int64_t ysc, int64_t ysf, int64_t nf, cudaStream_t st, std::atomic<int>* fm_choice = nullptr);

// Field-major fields through the cell-major kernels: transpose the input to
// (cells, fields), apply, transpose the output back.  Fields are padded to a
// multiple of 4 (zeros) so the cell-major path takes its vector kernels.
template <class T>
void field_major_via_cells(const DevCsr& c, bool normalize, bool adjoint, const T* x, int64_t xsf, T* y, int64_t ysf,
                           int64_t nf, cudaStream_t st) {
  const int64_t nin = c.ncols, nout = c.nrows, nfp = (nf + 3) / 4 * 4;
  T* xt = nullptr;
  T* yt = nullptr;
  CRG_CHECK_CUDA(cudaMallocAsync((void**)&xt, sizeof(T) * (nin * nfp + 4), st));
  CRG_CHECK_CUDA(cudaMallocAsync((void**)&yt, sizeof(T) * (nout * nfp + 4), st));
  if (nfp != nf) CRG_CHECK_CUDA(cudaMemsetAsync(xt, 0, sizeof(T) * nin * nfp, st));
  launch_transpose<T>(x, xsf, xt, nfp, nf, nin, st);
  launch_f32<T>(c, normalize, adjoint, xt, nfp, 1, yt, nfp, 1, nfp, st);
  launch_transpose<T>(yt, nfp, y, ysf, nout, nf, st);
  CRG_CHECK_CUDA(cudaFreeAsync(xt, st));
  CRG_CHECK_CUDA(cudaFreeAsync(yt, st));
}

template <class T>
void launch_f32(const DevCsr& c, bool normalize, bool adjoint, const T* x, int64_t xsc, int64_t xsf, T* y,
                int64_t ysc, int64_t ysf, int64_t nf, cudaStream_t st, std::atomic<int>* fm_choice) {
  const int64_t n = c.nrows;
  if (n == 0 || nf == 0) return;
  const float* w = normalize ? (adjoint ? c.adj32 : c.wn32) : c.val32;
  const bool cell_major = (xsf == 1 && ysf == 1) && nf > 1;
  const bool field_major = (xsc == 1 && ysc == 1);
  const int es = (int)sizeof(T);
  // 4-field vectors: 16-byte (FP32) / 8-byte (BF16) aligned loads and stores
  const bool vec4 = nf % 4 == 0 && xsc % 4 == 0 && ysc % 4 == 0 && (uintptr_t)x % (4 * es) == 0 &&
                    (uintptr_t)y % (4 * es) == 0;
  const SpmmPath path = spmm_path();
  // the merge-path kernel addresses source cells with 32-bit byte offsets
  const bool span32 = (double)c.ncols * (double)xsc * es < 4.0e9;
  if (path == SpmmPath::kAuto && cell_major && nf >= 32 && span32) {
    // merge-path over entries (4-field vectors when the rows allow, else each
    // lane's fields strided by 32); rows with no entries are zeroed separately
    launch_cm_nnz<T>(c, w, x, xsc, y, ysc, nf, st, vec4);
    return;
  }
  if (narrow_path(path, cell_major, nf)) {
    // fewer fields: the same tasks, several entries per warp load
    launch_cm_narrow<T>(c, w, x, xsc, y, ysc, nf, st, vec4);
    return;
  }
  {
    if (cell_major && vec4) {
      launch_cm_rows<T>(c, w, x, xsc, y, ysc, nf, st);
      CRG_CHECK_CUDA(cudaGetLastError());
      return;
    }
    if (field_major) {
      auto rows = [&]() {
        k_fm_rows<T><<<nblk(n, 256), 256, 0, st>>>(c.ptr, c.idx, w, n, nullptr, x, xsf, y, ysf, nf);
        CRG_CHECK_CUDA(cudaGetLastError());
      };
      auto cells = [&]() { field_major_via_cells<T>(c, normalize, adjoint, x, xsf, y, ysf, nf, st); };
      // With 32 fields or more the field-major gathers may touch many cache
      // lines per warp (rows whose columns are far apart in the source
      // numbering); then two transposes around the cell-major kernel win.
      // The first such apply of a direction times both (twice, after their
      // first launches) and keeps the faster; during stream capture, or
      // without a place to keep the choice, the row kernel runs.
      int choice = (path == SpmmPath::kAuto && nf >= 32 && fm_choice) ? fm_choice->load() : 1;
      if (choice == 0) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        CRG_CHECK_CUDA(cudaStreamIsCapturing(st, &cs));
        if (cs != cudaStreamCaptureStatusNone) {
          choice = 1;
        } else {
          cudaEvent_t e[5];
          for (auto& ev : e) CRG_CHECK_CUDA(cudaEventCreate(&ev));
          rows();
          cells();
          CRG_CHECK_CUDA(cudaEventRecord(e[0], st));
          rows();
          CRG_CHECK_CUDA(cudaEventRecord(e[1], st));
          cells();
          CRG_CHECK_CUDA(cudaEventRecord(e[2], st));
          CRG_CHECK_CUDA(cudaEventSynchronize(e[2]));
          float t_rows = 0.f, t_cells = 0.f;
          CRG_CHECK_CUDA(cudaEventElapsedTime(&t_rows, e[0], e[1]));
          CRG_CHECK_CUDA(cudaEventElapsedTime(&t_cells, e[1], e[2]));
          for (auto& ev : e) cudaEventDestroy(ev);
          fm_choice->store(t_cells < t_rows ? 2 : 1);
          return;  // y holds the result of the last variant
        }
      }
      if (choice == 2) cells();
      else rows();
      return;
    }
  }
  if (cell_major) {
    const bool vec = (xsc % 4 == 0) && (ysc % 4 == 0) && (nf % 4 == 0) &&
                     ((uintptr_t)x % (4 * sizeof(T)) == 0) && ((uintptr_t)y % (4 * sizeof(T)) == 0);
    int64_t lanes = (std::min<int64_t>(nf, 128) + 3) / 4;
    int G = 1;
    while (G < lanes) G <<= 1;
    const unsigned blocks = nblk(n * G, 256);
#define CRG_ROWS_CASE(GG)                                                                                  \
  case GG:                                                                                                 \
    if (vec) k_spmm_rows<T, GG, true><<<blocks, 256, 0, st>>>(c.ptr, c.idx, w, n, x, xsc, y, ysc, nf);     \
    else k_spmm_rows<T, GG, false><<<blocks, 256, 0, st>>>(c.ptr, c.idx, w, n, x, xsc, y, ysc, nf);        \
    break;
    switch (G) {
      CRG_ROWS_CASE(1)
      CRG_ROWS_CASE(2)
      CRG_ROWS_CASE(4)
      CRG_ROWS_CASE(8)
      CRG_ROWS_CASE(16)
      CRG_ROWS_CASE(32)
    }
#undef CRG_ROWS_CASE
  } else {
    for (int64_t f0 = 0; f0 < nf; f0 += 65535) {
      dim3 grid(nblk(n, 256), (unsigned)std::min<int64_t>(65535, nf - f0));
      k_spmm_generic<T><<<grid, 256, 0, st>>>(c.ptr, c.idx, w, n, x, xsc, xsf, y, ysc, ysf, f0);
    }
  }
  CRG_CHECK_CUDA(cudaGetLastError());
}

size_t elem_size(int dtype) { return dtype == CRG_F64 ? 8 : (dtype == CRG_F32 ? 4 : 2); }

// ------------------------------------------------------------------ one launch for a batch
//
// The applies of many regridders (cell-major FP32 or BF16 fields, device
// memory) as one grid of work units: merge-path items contribute one unit per
// task and 128-field pass (the body of k_cm_nnz), row items one unit per
// group of 32 / G rows (the body of k_spmm_rows, G lanes per row).  Every
// warp takes units u = warp, warp + warps, ... and finds the unit's item by a
// binary search in the items' first units.  A second launch sums the cut rows
// of every merge-path item (k_cm_fixup's body) and zeroes their empty rows.
// Each item's result has the bits of its own crg_apply: the same tasks, cut
// rows and fixup order, or the same sequential row sums.

struct BatchItem {
  int64_t unit0;   // first unit of the item
  int32_t kind;    // 0 merge-path, 1 rows
  int32_t gaps;    // merge-path: some rows have no entries (nextrow)
  int32_t lg;      // rows: log2 of the lanes per row
  int32_t vec;     // 4-field vector access (merge-path items: else the strided lane layout)
  int64_t ntasks;  // merge-path: tasks per 128-field pass
  int64_t nrows, nf, xs, ys, nslots;
  const int4* tasks;
  const int2* tslot;
  const uint32_t* rbits;
  const int32_t* nextrow;
  const int32_t* ptr;
  const int32_t* idx;
  const float* w;
  const void* x;
  void* y;
  float* carry;  // merge-path: [passes][nslots][128]
};

struct FinishItem {
  int64_t unit0;
  int32_t kind;  // 0 fixup of cut rows (nsplit units per pass), 1 zero rows without entries (32 rows per unit)
  int32_t vec;   // fixup: the carry slots hold the 4-vector lane layout (else the strided one)
  int64_t nsplit, nslots, nrows, nf, ys;
  const int32_t* split;
  const float* carry;
  const int32_t* ptr;
  void* y;
};

// index of the item holding unit u: the last i with unit0[i] <= u
__device__ __forceinline__ int batch_find(const int64_t* __restrict__ unit0, int n, int64_t u) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(unit0 + mid) <= u) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// k_spmm_rows for one group of rows: lane -> (row, g), fields f = 4 g, 4 g + 4 G, ...;
// each field summed in entry order, as the row kernels do.
template <class T>
__device__ __forceinline__ float4 ld4_tail(const T* xp, int64_t f, int64_t nf, bool full) {
  if (full) return ld4<T>(xp);
  float4 v;
  v.x = ld1<T>(xp);
  v.y = f + 1 < nf ? ld1<T>(xp + 1) : 0.f;
  v.z = f + 2 < nf ? ld1<T>(xp + 2) : 0.f;
  v.w = f + 3 < nf ? ld1<T>(xp + 3) : 0.f;
  return v;
}

template <class T>
__device__ __forceinline__ void st4_tail(T* yp, float4 acc, int64_t f, int64_t nf, bool full) {
  if (full) {
    st4<T>(yp, acc);
  } else {
    st1<T>(yp, acc.x);
    if (f + 1 < nf) st1<T>(yp + 1, acc.y);
    if (f + 2 < nf) st1<T>(yp + 2, acc.z);
    if (f + 3 < nf) st1<T>(yp + 3, acc.w);
  }
}

// One group of rows of a row item: G lanes per row (lane group g = lane % G),
// fields in blocks of 4 G -- 4 consecutive fields per lane when the rows are
// 4-vectors, else 4 fields strided by G (contiguous scalar loads across the
// group).  The group loads G of the row's (column, weight) entries at once and
// broadcasts them by shuffles; 4 entries' gathers are issued before their
// FMAs.  Every field is summed in entry order from zero, as the row kernels
// of crg_apply do.
template <class T>
__device__ __forceinline__ void rows_unit(const BatchItem* __restrict__ itp, int64_t k, int lane) {
  const int lg = itp->lg;
  const int G = 1 << lg;
  const int g = lane & (G - 1);
  const int gbase = lane - g;
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gbase);
  const int64_t r = k * (32 >> lg) + (lane >> lg);
  if (r >= itp->nrows) return;  // the whole lane group shares r
  const int64_t nf = itp->nf, xs = itp->xs;
  const bool vec = itp->vec != 0;
  const int32_t* __restrict__ idx = itp->idx;
  const float* __restrict__ w = itp->w;
  const T* __restrict__ x = static_cast<const T*>(itp->x);
  T* __restrict__ y = static_cast<T*>(itp->y) + r * itp->ys;
  const int32_t k0 = __ldg(itp->ptr + r), n = __ldg(itp->ptr + r + 1) - k0;
  for (int64_t f0 = 0; f0 < nf; f0 += (int64_t)G * 4) {
    // this lane's 4 fields: f + s * t, t < 4
    const int64_t f = vec ? f0 + (int64_t)g * 4 : f0 + g;
    const int64_t s = vec ? 1 : G;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int kb = 0; kb < n; kb += G) {
      const bool in = kb + g < n;
      const int32_t myj = in ? __ldg(idx + k0 + kb + g) : 0;
      const float myw = in ? __ldg(w + k0 + kb + g) : 0.f;
      const int ne = min(G, n - kb);
      for (int e = 0; e < ne; e += 4) {
        float4 v[4];
        float ww[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const int src = gbase + min(e + h, G - 1);
          const int64_t j = __shfl_sync(gmask, myj, src);
          ww[h] = __shfl_sync(gmask, myw, src);
          const T* xp = x + j * xs + f;
          if (e + h >= ne) {
            v[h] = make_float4(0.f, 0.f, 0.f, 0.f);
          } else if (vec) {
            v[h] = ld4<T>(xp);
          } else {
            v[h].x = f < nf ? ld1<T>(xp) : 0.f;
            v[h].y = f + s < nf ? ld1<T>(xp + s) : 0.f;
            v[h].z = f + 2 * s < nf ? ld1<T>(xp + 2 * s) : 0.f;
            v[h].w = f + 3 * s < nf ? ld1<T>(xp + 3 * s) : 0.f;
          }
        }
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          if (e + h >= ne) break;
          acc.x = fmaf(ww[h], v[h].x, acc.x);
          acc.y = fmaf(ww[h], v[h].y, acc.y);
          acc.z = fmaf(ww[h], v[h].z, acc.z);
          acc.w = fmaf(ww[h], v[h].w, acc.w);
        }
      }
    }
    if (vec) {
      if (f < nf) st4<T>(y + f, acc);
    } else {
      if (f < nf) st1<T>(y + f, acc.x);
      if (f + s < nf) st1<T>(y + f + s, acc.y);
      if (f + 2 * s < nf) st1<T>(y + f + 2 * s, acc.z);
      if (f + 3 * s < nf) st1<T>(y + f + 3 * s, acc.w);
    }
  }
}

// The items of a batch: units 0 .. nunits-1 are merge-path units, one per
// task and 128-field pass (the default gathers in flight and blocks per SM of
// k_cm_nnz); units nunits .. nunits+nrunits-1 are row units of the other items
// (a warp per group of 32 / G rows, rows_unit).  One grid-stride loop over
// both: the warps stay resident, and the row units fill the end of the launch
// instead of waiting for SM slots the persistent warps hold.
template <class T>
__global__ void __launch_bounds__(256, CmGather<T>::kBatchMinBlocks) k_batch_apply(const BatchItem* __restrict__ items,
                                                        const int64_t* __restrict__ unit0, int nitems,
                                                        int64_t nunits, const BatchItem* __restrict__ ritems,
                                                        const int64_t* __restrict__ runit0, int nritems,
                                                        int64_t nrunits) {
  constexpr int B = CmGather<T>::kInFlight;
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  __shared__ uint2 s_stage[CmGather<T>::kStage ? 8 : 1][64];
  uint2* stg = CmGather<T>::kStage ? s_stage[threadIdx.x >> 5] : nullptr;
  for (int64_t u = gw; u < nunits + nrunits; u += nw) {
    if (u >= nunits) {
      const int64_t v = u - nunits;
      const BatchItem* rtp = ritems + batch_find(runit0, nritems, v);
      rows_unit<T>(rtp, v - rtp->unit0, lane);
      continue;
    }
    const BatchItem* itp = items + batch_find(unit0, nitems, u);
    const int64_t ntasks = itp->ntasks, k = u - itp->unit0;
    const int64_t pass = k / ntasks, task = k - pass * ntasks;
    int64_t fo;
    int onm;
    const T* x = static_cast<const T*>(itp->x);
    const uint32_t cstride = (uint32_t)(itp->xs * (int64_t)sizeof(T));
    float* carry = itp->carry ? itp->carry + pass * itp->nslots * 128 : nullptr;
    T* y = static_cast<T*>(itp->y);
    // nextrow is NULL unless the item has rows without entries (checked per row change)
    const int32_t* nextrow = itp->gaps ? itp->nextrow : nullptr;
    if (itp->vec) {
      const char* xb = cm_lane_base<T, true>(x, pass * 128, itp->nf, lane, fo, onm);
      cm_task<T, true, B, true>(task, itp->tasks, itp->tslot, itp->idx, itp->rbits, nextrow, itp->w, xb, cstride, y,
                                itp->ys, fo, onm, carry, lane, stg);
    } else {
      const char* xb = cm_lane_base<T, false>(x, pass * 128, itp->nf, lane, fo, onm);
      cm_task<T, true, B, false>(task, itp->tasks, itp->tslot, itp->idx, itp->rbits, nextrow, itp->w, xb, cstride,
                                 y, itp->ys, fo, onm, carry, lane, stg);
    }
  }
}

template <class T>
__global__ void k_batch_finish(const FinishItem* __restrict__ items, const int64_t* __restrict__ unit0, int nitems,
                               int64_t nunits) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t u = gw; u < nunits; u += nw) {
    const FinishItem& it = items[batch_find(unit0, nitems, u)];
    const int64_t k = u - it.unit0;
    T* __restrict__ y = static_cast<T*>(it.y);
    if (it.kind == 0) {
      // k_cm_fixup / k_cm_fixup_s: the pieces of cut row s in task order
      const int64_t pass = k / it.nsplit, sp = k - pass * it.nsplit;
      const int32_t row = __ldg(it.split + 3 * sp), s0 = __ldg(it.split + 3 * sp + 1),
                    pieces = __ldg(it.split + 3 * sp + 2);
      const float* c = it.carry + pass * it.nslots * 128;
      if (it.vec) {
        const int64_t f = pass * 128 + (int64_t)lane * 4;
        if (f >= it.nf) continue;
        float4 acc = *reinterpret_cast<const float4*>(c + (int64_t)s0 * 128 + lane * 4);
        for (int32_t q = 1; q < pieces; ++q) {
          const float4 d = *reinterpret_cast<const float4*>(c + (int64_t)(s0 + q) * 128 + lane * 4);
          acc.x += d.x; acc.y += d.y; acc.z += d.z; acc.w += d.w;
        }
        st4<T>(y + (int64_t)row * it.ys + f, acc);
      } else {
        for (int t = 0; t < 4; ++t) {
          const int p = lane + 32 * t;
          if (pass * 128 + p >= it.nf) break;
          float acc = c[(int64_t)s0 * 128 + p];
          for (int32_t q = 1; q < pieces; ++q) acc += c[(int64_t)(s0 + q) * 128 + p];
          st1<T>(y + (int64_t)row * it.ys + pass * 128 + p, acc);
        }
      }
    } else {
      // k_zero_empty_cm: rows without entries
      const int64_t r = k * 32 + lane;
      if (r >= it.nrows || __ldg(it.ptr + r + 1) > __ldg(it.ptr + r)) continue;
      for (int64_t f = 0; f < it.nf; ++f) st1<T>(y + r * it.ys + f, 0.f);
    }
  }
}

}  // namespace

// The device tables of a batch (one allocation) and its launches.
struct BatchLaunch {
  void* mem = nullptr;
  int device = 0;
  struct Part {
    int dtype = CRG_F32;
    const BatchItem* items = nullptr;  // merge-path items
    const int64_t* unit0 = nullptr;
    int nitems = 0;
    int64_t nunits = 0;
    const BatchItem* ritems = nullptr;  // row items
    const int64_t* runit0 = nullptr;
    int nritems = 0;
    int64_t nrunits = 0;
    const FinishItem* fitems = nullptr;
    const int64_t* funit0 = nullptr;
    int nfitems = 0;
    int64_t nfunits = 0;
  };
  std::vector<Part> parts;  // one per field type present
};

BatchLaunch* batch_prepare(int64_t n, const crg_apply_item* items, std::vector<char>& handled, bool all) {
  handled.assign((size_t)n, 0);
  std::vector<BatchItem> bi[2], ri[2];  // merge-path items, row items
  std::vector<FinishItem> fi[2];
  std::vector<int64_t> carry_off[2];  // per merge-path item: float offset of its carry, -1 none
  int64_t units[2] = {0, 0}, runits[2] = {0, 0}, funits[2] = {0, 0}, carry_floats = 0;
  int dev = 0;
  CRG_CHECK_CUDA(cudaGetDevice(&dev));
  for (int64_t k = 0; k < n; ++k) {
    const crg_apply_item& it = items[k];
    const crg_regridder* r = it.regridder;
    if (!r || !(it.dtype == CRG_F32 || it.dtype == CRG_BF16) || r->device != dev || it.nfields < 1) continue;
    const bool t = it.transpose != 0;
    const DevCsr& c = it.adjoint ? (t ? r->fwd : r->rev) : (t ? r->rev : r->fwd);
    const int64_t nf = it.nfields;
    if (c.nrows == 0) {
      handled[k] = 1;  // nothing to write
      continue;
    }
    const int64_t ssc = it.src_stride_cell, ssf = it.src_stride_field, dsc = it.dst_stride_cell,
                  dsf = it.dst_stride_field;
    // fields side by side (or one field), device memory, positive strides
    if (!(nf == 1 || (ssf == 1 && dsf == 1))) continue;
    if (!it.dst || (c.ncols > 0 && !it.src) || dsc <= 0 || (c.ncols > 0 && ssc <= 0)) continue;
    if (!is_device_pointer(it.dst) || (c.ncols > 0 && !is_device_pointer(it.src))) continue;
    const int d = it.dtype == CRG_BF16 ? 1 : 0;
    const int es = d ? 2 : 4;
    const float* w = it.normalize ? (it.adjoint ? c.adj32 : c.wn32) : c.val32;
    const bool cell_major = ssf == 1 && dsf == 1 && nf > 1;
    const bool vec4 = nf % 4 == 0 && ssc % 4 == 0 && dsc % 4 == 0 && (uintptr_t)it.src % (4 * es) == 0 &&
                      (uintptr_t)it.dst % (4 * es) == 0;
    const bool span32 = (double)c.ncols * (double)ssc * es < 4.0e9;
    BatchItem b{};
    b.nrows = c.nrows;
    b.nf = nf;
    b.xs = ssc;
    b.ys = dsc;
    b.ptr = c.ptr;
    b.idx = c.idx;
    b.w = w;
    b.x = it.src;
    b.y = it.dst;
    const int64_t passes = (nf + 127) / 128;
    // crg_apply runs fewer than 32 fields with k_cm_narrow, whose sums the row
    // units would not reproduce: those items keep their own applies
    if (narrow_path(spmm_path(), cell_major, nf)) continue;
    const bool merge_path = spmm_path() == SpmmPath::kAuto && cell_major && nf >= 32 && span32;
    // Measured on 32 uneven pairs: the persistent launch runs a small matrix's
    // many 128-field passes side by side (3x its own launch), but a large
    // matrix or a row-kernel item runs 10-25% (2-3x) faster in its own tuned
    // launch on a graph branch.
    const int64_t resident = (int64_t)num_sms() * 8 *
                             (d ? CmGather<__nv_bfloat16>::kBatchMinBlocks : CmGather<float>::kBatchMinBlocks);
    if (!all && !(merge_path && passes >= 2 && c.ntasks < resident)) continue;
    if (merge_path) {
      // the merge path, as launch_cm_nnz runs it
      b.kind = 0;
      b.gaps = c.nextrow != nullptr;
      b.vec = vec4;
      b.ntasks = c.ntasks;
      b.nslots = c.nslots;
      b.tasks = c.tasks;
      b.tslot = c.tslot;
      b.rbits = c.rbits;
      b.nextrow = c.nextrow;
      const int64_t nu = c.ntasks * passes;
      if (nu > 0) {
        b.unit0 = units[d];
        units[d] += nu;
        carry_off[d].push_back(c.nslots ? carry_floats : -1);
        carry_floats += c.nslots * 128 * passes;
        bi[d].push_back(b);
      }
      FinishItem f{};
      f.nsplit = c.nsplit;
      f.nslots = c.nslots;
      f.nrows = c.nrows;
      f.nf = nf;
      f.ys = dsc;
      f.split = c.split;
      f.ptr = c.ptr;
      f.y = it.dst;
      if (c.nsplit && nu > 0) {
        f.kind = 0;
        f.vec = vec4;
        f.unit0 = funits[d];
        f.carry = reinterpret_cast<const float*>((intptr_t)carry_off[d].back());  // offset until allocation
        funits[d] += c.nsplit * passes;
        fi[d].push_back(f);
      }
      if (c.nempty) {
        f.kind = 1;
        f.carry = nullptr;
        f.unit0 = funits[d];
        funits[d] += (c.nrows + 31) / 32;
        fi[d].push_back(f);
      }
    } else {
      // the row kernels: G lanes per row, as launch_f32 picks them
      b.kind = 1;
      b.vec = vec4;
      const int64_t lanes = (std::min<int64_t>(nf, 128) + 3) / 4;
      int lg = 0;
      while ((1 << lg) < lanes) ++lg;
      b.lg = lg;
      b.unit0 = runits[d];
      runits[d] += (c.nrows + (32 >> lg) - 1) / (32 >> lg);
      ri[d].push_back(b);
    }
    handled[k] = 1;
  }
  // one allocation: [items][unit0] per part, carry
  size_t bytes = 0;
  auto take = [&](size_t b) {
    const size_t at = bytes;
    bytes += (b + 255) / 256 * 256;
    return at;
  };
  size_t off_items[2], off_u0[2], off_r[2], off_ru0[2], off_f[2], off_fu0[2];
  for (int d = 0; d < 2; ++d) {
    off_items[d] = take(bi[d].size() * sizeof(BatchItem));
    off_u0[d] = take(bi[d].size() * sizeof(int64_t));
    off_r[d] = take(ri[d].size() * sizeof(BatchItem));
    off_ru0[d] = take(ri[d].size() * sizeof(int64_t));
    off_f[d] = take(fi[d].size() * sizeof(FinishItem));
    off_fu0[d] = take(fi[d].size() * sizeof(int64_t));
  }
  const size_t off_carry = take((size_t)carry_floats * sizeof(float));
  BatchLaunch* L = new BatchLaunch;
  L->device = dev;
  try {
    if (bytes) CRG_CHECK_CUDA(cudaMalloc(&L->mem, bytes));
    char* base = static_cast<char*>(L->mem);
    float* carry = reinterpret_cast<float*>(base + off_carry);
    for (int d = 0; d < 2; ++d) {
      if (bi[d].empty() && ri[d].empty() && fi[d].empty()) continue;
      size_t mp = 0;
      for (auto& b : bi[d])
        if (b.kind == 0) {
          const int64_t o = carry_off[d][mp++];
          b.carry = o >= 0 ? carry + o : nullptr;
        }
      for (auto& f : fi[d])
        if (f.kind == 0) f.carry = carry + (intptr_t)f.carry;
      std::vector<int64_t> u0(bi[d].size()), ru0(ri[d].size()), fu0(fi[d].size());
      for (size_t q = 0; q < bi[d].size(); ++q) u0[q] = bi[d][q].unit0;
      for (size_t q = 0; q < ri[d].size(); ++q) ru0[q] = ri[d][q].unit0;
      for (size_t q = 0; q < fi[d].size(); ++q) fu0[q] = fi[d][q].unit0;
      auto up = [&](size_t off, const void* src, size_t nb) {
        if (nb) CRG_CHECK_CUDA(cudaMemcpy(base + off, src, nb, cudaMemcpyHostToDevice));
      };
      up(off_items[d], bi[d].data(), bi[d].size() * sizeof(BatchItem));
      up(off_u0[d], u0.data(), u0.size() * sizeof(int64_t));
      up(off_r[d], ri[d].data(), ri[d].size() * sizeof(BatchItem));
      up(off_ru0[d], ru0.data(), ru0.size() * sizeof(int64_t));
      up(off_f[d], fi[d].data(), fi[d].size() * sizeof(FinishItem));
      up(off_fu0[d], fu0.data(), fu0.size() * sizeof(int64_t));
      BatchLaunch::Part p;
      p.dtype = d ? CRG_BF16 : CRG_F32;
      p.items = reinterpret_cast<const BatchItem*>(base + off_items[d]);
      p.unit0 = reinterpret_cast<const int64_t*>(base + off_u0[d]);
      p.nitems = (int)bi[d].size();
      p.nunits = units[d];
      p.ritems = reinterpret_cast<const BatchItem*>(base + off_r[d]);
      p.runit0 = reinterpret_cast<const int64_t*>(base + off_ru0[d]);
      p.nritems = (int)ri[d].size();
      p.nrunits = runits[d];
      p.fitems = reinterpret_cast<const FinishItem*>(base + off_f[d]);
      p.funit0 = reinterpret_cast<const int64_t*>(base + off_fu0[d]);
      p.nfitems = (int)fi[d].size();
      p.nfunits = funits[d];
      L->parts.push_back(p);
    }
  } catch (...) {
    batch_free(L);
    throw;
  }
  return L;
}

void batch_enqueue(const BatchLaunch* L, cudaStream_t st) {
  const int64_t max_warps = (int64_t)num_sms() * 24;  // three blocks of 8 warps per SM
  for (const auto& p : L->parts) {
    if (p.nunits + p.nrunits) {
      const int minb =
          p.dtype == CRG_F32 ? CmGather<float>::kBatchMinBlocks : CmGather<__nv_bfloat16>::kBatchMinBlocks;
      const int64_t warps = std::min<int64_t>(p.nunits + p.nrunits, (int64_t)num_sms() * 8 * minb);
      if (p.dtype == CRG_F32)
        k_batch_apply<float><<<nblk(warps * 32, 256), 256, 0, st>>>(p.items, p.unit0, p.nitems, p.nunits, p.ritems,
                                                                    p.runit0, p.nritems, p.nrunits);
      else
        k_batch_apply<__nv_bfloat16><<<nblk(warps * 32, 256), 256, 0, st>>>(p.items, p.unit0, p.nitems, p.nunits,
                                                                            p.ritems, p.runit0, p.nritems, p.nrunits);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
    if (p.nfunits) {
      const int64_t warps = std::min<int64_t>(p.nfunits, max_warps);
      if (p.dtype == CRG_F32)
        k_batch_finish<float><<<nblk(warps * 32, 256), 256, 0, st>>>(p.fitems, p.funit0, p.nfitems, p.nfunits);
      else
        k_batch_finish<__nv_bfloat16><<<nblk(warps * 32, 256), 256, 0, st>>>(p.fitems, p.funit0, p.nfitems,
                                                                              p.nfunits);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
  }
}

int batch_launches(const BatchLaunch* L) {
  int n = 0;
  for (const auto& p : L->parts) n += (p.nunits + p.nrunits > 0) + (p.nfunits > 0);
  return n;
}

void batch_free(BatchLaunch* L) {
  if (!L) return;
  if (L->mem) cudaFree(L->mem);
  delete L;
}

namespace {

}  // namespace

// Whether an apply with host fields runs as the chunked pipeline, and its chunk.
HostChunks host_chunks(size_t es, int64_t nin, int64_t nf, int64_t ssc, int64_t ssf, int64_t dsc, int64_t dsf,
                       bool src_host, bool dst_host) {
  HostChunks h;
  h.cm = ssf == 1 && dsf == 1 && nf > 1;
  const bool fm = ssc == 1 && dsc == 1 && nf > 1 && !h.cm;
  // CRG_HOST_CHUNK_BYTES (64..4096, default 256) sets the cell-major row width for tuning
  static const int64_t row_bytes = [] {
    const char* e = getenv("CRG_HOST_CHUNK_BYTES");
    const int64_t v = e ? atoll(e) : 256;
    return (v >= 64 && v <= 4096) ? v : 256;
  }();
  h.chunk = h.cm ? std::max<int64_t>(4, row_bytes / (int64_t)es / 4 * 4) : (nf + 3) / 4;
  h.ok = src_host && dst_host && nin > 0 && (h.cm || fm) && nf >= 2 * h.chunk;
  return h;
}

bool host_pipeline_item(const crg_apply_item& it) {
  const crg_regridder* r = it.regridder;
  if (!r || it.nfields < 1 || !(it.dtype == CRG_F64 || it.dtype == CRG_F32 || it.dtype == CRG_BF16)) return false;
  const bool t = it.transpose != 0;
  const DevCsr& c = it.adjoint ? (t ? r->fwd : r->rev) : (t ? r->rev : r->fwd);
  if (c.nrows == 0) return false;
  const bool src_host = c.ncols > 0 && it.src && !is_device_pointer(it.src);
  const bool dst_host = it.dst && !is_device_pointer(it.dst);
  return host_chunks(elem_size(it.dtype), c.ncols, it.nfields, it.src_stride_cell, it.src_stride_field,
                     it.dst_stride_cell, it.dst_stride_field, src_host, dst_host).ok;
}

// Bytes of an item's first chunk in and last chunk out: the parts of the
// pipeline that overlap nothing when the item comes first or last.
void host_pipeline_ends(const crg_apply_item& it, size_t& fill, size_t& drain) {
  const crg_regridder* r = it.regridder;
  const bool t = it.transpose != 0;
  const DevCsr& c = it.adjoint ? (t ? r->fwd : r->rev) : (t ? r->rev : r->fwd);
  const size_t es = elem_size(it.dtype);
  const HostChunks h = host_chunks(es, c.ncols, it.nfields, it.src_stride_cell, it.src_stride_field,
                                   it.dst_stride_cell, it.dst_stride_field, true, true);
  const int64_t chunk = std::max<int64_t>(1, h.chunk);
  const int64_t last = it.nfields - (it.nfields - 1) / chunk * chunk;
  fill = (size_t)c.ncols * (size_t)std::min<int64_t>(chunk, it.nfields) * es;
  drain = (size_t)c.nrows * (size_t)last * es;
}

int host_pipeline_dir(const crg_apply_item& it) {
  const crg_regridder* r = it.regridder;
  const bool t = it.transpose != 0;
  const DevCsr& c = it.adjoint ? (t ? r->fwd : r->rev) : (t ? r->rev : r->fwd);
  return &c == &r->rev ? 1 : 0;
}

void apply_impl(const crg_regridder* rc, int transpose, int dtype, bool adjoint, const void* src, int64_t ssc,
                int64_t ssf, void* dst, int64_t dsc, int64_t dsf, int64_t nf, int normalize, cudaStream_t st,
                HostPipe* pipe) {
  crg_regridder* r = const_cast<crg_regridder*>(rc);
  CRG_REQUIRE(r != nullptr, CRG_ERR_INVALID_ARGUMENT, "regridder is NULL");
  CRG_REQUIRE(dtype == CRG_F64 || dtype == CRG_F32 || dtype == CRG_BF16, CRG_ERR_INVALID_ARGUMENT, "unknown dtype %d",
              dtype);
  CRG_REQUIRE(nf >= 0, CRG_ERR_INVALID_ARGUMENT, "nfields must be >= 0");
  CRG_REQUIRE(ssc >= 0 && ssf >= 0 && dsc >= 0 && dsf >= 0, CRG_ERR_INVALID_ARGUMENT, "strides must be >= 0");
  const bool t = transpose != 0;
  // direction: which copy of A is read, and which area vector divides
  const DevCsr& c = adjoint ? (t ? r->fwd : r->rev) : (t ? r->rev : r->fwd);
  const double* div = normalize ? (t ? r->src_area : r->dst_area) : nullptr;
  const double* div_inv = normalize ? (t ? r->src_area_inv : r->dst_area_inv) : nullptr;
  const int64_t nin = c.ncols, nout = c.nrows;
  if (nf == 0 || nout == 0) return;
  CRG_REQUIRE(dst != nullptr && (src != nullptr || nin == 0), CRG_ERR_INVALID_ARGUMENT, "field pointer is NULL");
  CRG_REQUIRE(nin == 0 || (ssc > 0 || nin == 1), CRG_ERR_INVALID_ARGUMENT, "source cell stride must be > 0");
  CRG_REQUIRE(dsc > 0 || nout == 1, CRG_ERR_INVALID_ARGUMENT, "destination cell stride must be > 0");
  CRG_REQUIRE(nf == 1 || (ssf > 0 && dsf > 0), CRG_ERR_INVALID_ARGUMENT, "field stride must be > 0");
  int dev = 0;
  CRG_CHECK_CUDA(cudaGetDevice(&dev));
  CRG_REQUIRE(dev == r->device, CRG_ERR_INVALID_ARGUMENT, "regridder lives on device %d but device %d is current",
              r->device, dev);

  const size_t es = elem_size(dtype);
  const int64_t in_span = nin > 0 ? (nin - 1) * ssc + (nf - 1) * ssf + 1 : 0;
  const int64_t out_span = (nout - 1) * dsc + (nf - 1) * dsf + 1;
  const bool src_host = nin > 0 && !is_device_pointer(src);
  const bool dst_host = !is_device_pointer(dst);

  // the field-major kernel choice of this matrix copy and dtype
  std::atomic<int>* choice = &r->fm_choice[&c == &r->rev ? 1 : 0][dtype == CRG_BF16 ? 1 : 0];
  // the apply on device buffers
  auto compute = [&](const void* x, int64_t xsc, int64_t xsf, void* y, int64_t ysc, int64_t ysf, int64_t n,
                     cudaStream_t s) {
    if (dtype == CRG_F64 && xsf == 1 && ysf == 1 && n > 1 && spmm_path() == SpmmPath::kAuto) {
      launch_cm_f64(c, adjoint, div, div_inv, (const double*)x, xsc, (double*)y, ysc, n, s);
    } else if (dtype == CRG_F64) {
      const double* cdiv = adjoint ? div : nullptr;
      const double* rdiv = adjoint ? nullptr : div;
      for (int64_t f0 = 0; f0 < n; f0 += 65535) {
        dim3 grid(nblk(nout, 128), (unsigned)std::min<int64_t>(65535, n - f0));
        k_spmv_f64<<<grid, 128, 0, s>>>(c.ptr, c.idx, c.val, nout, (const double*)x, xsc, xsf, (double*)y, ysc, ysf,
                                        f0, rdiv, cdiv);
      }
      CRG_CHECK_CUDA(cudaGetLastError());
    } else if (dtype == CRG_F32) {
      launch_f32<float>(c, normalize, adjoint, (const float*)x, xsc, xsf, (float*)y, ysc, ysf, n, s, choice);
    } else {
      launch_f32<__nv_bfloat16>(c, normalize, adjoint, (const __nv_bfloat16*)x, xsc, xsf, (__nv_bfloat16*)y, ysc, ysf,
                                n, s, choice);
    }
  };
  if (!src_host && !dst_host) {
    compute(src, ssc, ssf, dst, dsc, dsf, nf, st);
    return;
  }

  const int dir = &c == &r->rev ? 1 : 0;
  std::unique_lock<std::mutex> lock(r->stage_mu[dir], std::defer_lock);
  if (!pipe) lock.lock();  // a batch pipeline holds the staging locks of its items
  auto stage = [&](size_t need) {
    if (r->stage_bytes[dir] < need) {
      if (r->stage[dir]) CRG_CHECK_CUDA(cudaFree(r->stage[dir]));
      r->stage[dir] = nullptr;
      r->stage_bytes[dir] = 0;
      CRG_CHECK_CUDA(cudaMalloc(&r->stage[dir], need));
      r->stage_bytes[dir] = need;
    }
    return (char*)r->stage[dir];
  };
  cudaStream_t& copy_in = r->copy_in[dir];
  cudaStream_t& copy_out = r->copy_out[dir];

  // Host fields in both directions, fields side by side (cell-major) or
  // whole fields contiguous (field-major): a pipeline over chunks of fields.
  // Chunk k+1 moves to the device while chunk k is applied and chunk k-1
  // moves back, on two copy streams, so the two directions of the host link
  // run at once.  Cell-major chunks are 2-D copies of 256-byte rows (full link
  // speed); each chunk is applied as a contiguous (cells, fields) block.
  const HostChunks hc = host_chunks(es, nin, nf, ssc, ssf, dsc, dsf, src_host, dst_host);
  const bool cm = hc.cm;
  const int64_t chunk = hc.chunk;
  CRG_REQUIRE(!pipe || hc.ok, CRG_ERR_INTERNAL, "a batch pipeline item does not fit the chunked host pipeline");
  if (hc.ok) {
    const int64_t nchunks = (nf + chunk - 1) / chunk;
    const size_t in_bytes = ((size_t)nin * nf * es + 255) / 256 * 256;
    char* din = stage(in_bytes + (size_t)nout * nf * es + 256);
    char* dout = din + in_bytes;
    if (!pipe) {
      if (!copy_in) CRG_CHECK_CUDA(cudaStreamCreateWithFlags(&copy_in, cudaStreamNonBlocking));
      if (!copy_out) CRG_CHECK_CUDA(cudaStreamCreateWithFlags(&copy_out, cudaStreamNonBlocking));
    }
    // a batch pipeline runs every item's chunks on its own three streams, in order
    cudaStream_t cin = pipe ? pipe->cin : copy_in, cout = pipe ? pipe->cout : copy_out;
    if (pipe) st = pipe->cst;
    std::vector<cudaEvent_t> local;
    std::vector<cudaEvent_t>& ev = pipe ? pipe->events : local;
    const size_t e0 = ev.size();
    struct Events {
      std::vector<cudaEvent_t>& v;
      bool own;
      ~Events() {
        if (own)
          for (auto e : v)
            if (e) cudaEventDestroy(e);
      }
    } guard{local, true};
    ev.resize(e0 + 2 * nchunks + 1, nullptr);
    for (size_t k = e0; k < ev.size(); ++k) CRG_CHECK_CUDA(cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming));
    auto E = [&](int64_t k) { return ev[e0 + k]; };
    if (!pipe) {
      // the copies start after the work the caller queued on its stream
      CRG_CHECK_CUDA(cudaEventRecord(E(2 * nchunks), st));
      CRG_CHECK_CUDA(cudaStreamWaitEvent(cin, E(2 * nchunks), 0));
    }
    const char* hs = (const char*)src;
    char* hd = (char*)dst;
    for (int64_t k = 0; k < nchunks; ++k) {
      const int64_t f0 = k * chunk, fc = std::min(chunk, nf - f0);
      char* xk = din + (size_t)f0 * nin * es;
      char* yk = dout + (size_t)f0 * nout * es;
      if (cm)
        CRG_CHECK_CUDA(cudaMemcpy2DAsync(xk, fc * es, hs + f0 * es, ssc * es, fc * es, nin, cudaMemcpyHostToDevice,
                                         cin));
      else
        CRG_CHECK_CUDA(cudaMemcpy2DAsync(xk, nin * es, hs + f0 * ssf * es, ssf * es, nin * es, fc,
                                         cudaMemcpyHostToDevice, cin));
      CRG_CHECK_CUDA(cudaEventRecord(E(2 * k), cin));
      CRG_CHECK_CUDA(cudaStreamWaitEvent(st, E(2 * k), 0));
      if (cm) compute(xk, fc, 1, yk, fc, 1, fc, st);
      else compute(xk, 1, nin, yk, 1, nout, fc, st);
      CRG_CHECK_CUDA(cudaEventRecord(E(2 * k + 1), st));
      CRG_CHECK_CUDA(cudaStreamWaitEvent(cout, E(2 * k + 1), 0));
      if (cm)
        CRG_CHECK_CUDA(cudaMemcpy2DAsync(hd + f0 * es, dsc * es, yk, fc * es, fc * es, nout, cudaMemcpyDeviceToHost,
                                         cout));
      else
        CRG_CHECK_CUDA(cudaMemcpy2DAsync(hd + f0 * dsf * es, dsf * es, yk, nout * es, nout * es, fc,
                                         cudaMemcpyDeviceToHost, cout));
    }
    if (!pipe) {
      CRG_CHECK_CUDA(cudaStreamSynchronize(cout));
      CRG_CHECK_CUDA(cudaStreamSynchronize(st));
    }
    return;
  }

  // Otherwise: one copy in, the apply, one copy out.
  char* base = stage((src_host ? (size_t)in_span * es : 0) + (dst_host ? (size_t)out_span * es : 0) + 256);
  const void* xs = src;
  void* ys = dst;
  if (src_host) {
    CRG_CHECK_CUDA(cudaMemcpyAsync(base, src, (size_t)in_span * es, cudaMemcpyHostToDevice, st));
    xs = base;
    base += ((size_t)in_span * es + 255) / 256 * 256;
  }
  if (dst_host) {
    // a strided destination keeps the elements between ours: bring them along
    if (out_span != nout * nf)
      CRG_CHECK_CUDA(cudaMemcpyAsync(base, dst, (size_t)out_span * es, cudaMemcpyHostToDevice, st));
    ys = base;
  }
  compute(xs, ssc, ssf, ys, dsc, dsf, nf, st);
  if (dst_host) CRG_CHECK_CUDA(cudaMemcpyAsync(dst, ys, (size_t)out_span * es, cudaMemcpyDeviceToHost, st));
  CRG_CHECK_CUDA(cudaStreamSynchronize(st));
}

// ------------------------------------------------------------------ folded grids

namespace {

// Fold row of a RightCenterFolded (tripolar) grid, cells numbered i + j * nx:
// the primary slots r = 1..nq and nh+1..nh+nq (1-based) hold the values, their
// partners nx+1-r are ghost slots of the same physical cells and get a copy.
template <class T>
__global__ void k_mirror_fold(T* __restrict__ f, int64_t sc, int64_t sf, int64_t nfields, int64_t nx, int64_t nq,
                              int64_t nh, int64_t off) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = blockIdx.y;
  if (q >= 2 * nq || k >= nfields) return;
  const int64_t r = q < nq ? q + 1 : q - nq + nh + 1;
  f[(off + nx - r) * sc + k * sf] = f[(off + r - 1) * sc + k * sf];
}

template <class T>
void mirror_host(T* f, int64_t sc, int64_t sf, int64_t nfields, int64_t nx, int64_t nq, int64_t nh, int64_t off) {
  for (int64_t k = 0; k < nfields; ++k)
    for (int64_t q = 0; q < 2 * nq; ++q) {
      const int64_t r = q < nq ? q + 1 : q - nq + nh + 1;
      f[(off + nx - r) * sc + k * sf] = f[(off + r - 1) * sc + k * sf];
    }
}

}  // namespace

void mirror_fold_impl(int dtype, void* field, int64_t sc, int64_t sf, int64_t nfields, int64_t nx, int64_t ny,
                      cudaStream_t st) {
  CRG_REQUIRE(dtype == CRG_F64 || dtype == CRG_F32 || dtype == CRG_BF16, CRG_ERR_INVALID_ARGUMENT, "unknown dtype %d",
              dtype);
  CRG_REQUIRE(nx > 0 && ny > 0 && nx % 4 == 0, CRG_ERR_INVALID_ARGUMENT,
              "a folded grid needs nx a positive multiple of 4 (got nx = %lld, ny = %lld)", (long long)nx,
              (long long)ny);
  CRG_REQUIRE(field != nullptr && sc > 0 && nfields >= 1 && (nfields == 1 || sf > 0), CRG_ERR_INVALID_ARGUMENT,
              "field pointer, strides or field count invalid");
  CRG_REQUIRE(nfields <= 65535 || !is_device_pointer(field), CRG_ERR_NOT_SUPPORTED, "at most 65535 fields per call");
  const int64_t nq = nx / 4, nh = nx / 2, off = (ny - 1) * nx;
  if (!is_device_pointer(field)) {
    // the caller's queued work on this field comes first (nothing can be queued without a device)
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) cudaGetLastError();
    else CRG_CHECK_CUDA(e);
    if (dtype == CRG_F64) mirror_host((double*)field, sc, sf, nfields, nx, nq, nh, off);
    else if (dtype == CRG_F32) mirror_host((float*)field, sc, sf, nfields, nx, nq, nh, off);
    else mirror_host((__nv_bfloat16*)field, sc, sf, nfields, nx, nq, nh, off);
    return;
  }
  dim3 grid(nblk(2 * nq, 128), (unsigned)nfields);
  if (dtype == CRG_F64) k_mirror_fold<double><<<grid, 128, 0, st>>>((double*)field, sc, sf, nfields, nx, nq, nh, off);
  else if (dtype == CRG_F32) k_mirror_fold<float><<<grid, 128, 0, st>>>((float*)field, sc, sf, nfields, nx, nq, nh, off);
  else
    k_mirror_fold<__nv_bfloat16><<<grid, 128, 0, st>>>((__nv_bfloat16*)field, sc, sf, nfields, nx, nq, nh, off);
  CRG_CHECK_CUDA(cudaGetLastError());
}

}  // namespace crg

// ------------------------------------------------------------------ allocation-free apply
//
// crg_apply_noalloc runs the merge-path kernels above with their carry buffer
// in a statically declared device array instead of memory allocated per call,
// for callers that must not allocate device memory.  Each carry slot holds
// 128 FP32 partial sums of one piece of a row cut between tasks.

static __device__ __align__(256) float g_noalloc_carry[CRG_NOALLOC_SCRATCH_BYTES / sizeof(float)];

namespace crg {

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
// per device: the context the address was looked up in, and the address
void* g_noalloc_ctx[kMaxDevices] = {};
float* g_noalloc_ptr[kMaxDevices] = {};

// cuCtxGetCurrent through the runtime's driver entry point (no link against
// the driver library): the identity of the current context, so that an address
// looked up before a cudaDeviceReset (which makes a new primary context, where
// the array may lie elsewhere) is never reused.
using CtxGetCurrentFn = int (*)(void**);
CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<CtxGetCurrentFn>(f);
  }();
  return fn;
}

// Device address of g_noalloc_carry in the current context of device `dev`
// (the host-side name is only a stand-in, not a device address).  Looked up
// once per context: the lookup also loads this file's module, which reserves
// the array.
float* noalloc_scratch(int dev) {
  CRG_REQUIRE(dev >= 0 && dev < kMaxDevices, CRG_ERR_NOT_SUPPORTED, "device %d is beyond the supported %d", dev,
              kMaxDevices);
  const CtxGetCurrentFn get = ctx_get_current();
  CRG_REQUIRE(get != nullptr, CRG_ERR_CUDA, "cuCtxGetCurrent is not available from the driver");
  void* ctx = nullptr;
  CRG_REQUIRE(get(&ctx) == 0 && ctx != nullptr, CRG_ERR_CUDA, "no current CUDA context on device %d", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev] || g_noalloc_ctx[dev] != ctx) {
    void* p = nullptr;
    CRG_CHECK_CUDA(cudaGetSymbolAddress(&p, g_noalloc_carry));
    CRG_REQUIRE(p != nullptr, CRG_ERR_CUDA, "cudaGetSymbolAddress returned a null scratch address");
    g_noalloc_ptr[dev] = static_cast<float*>(p);
    g_noalloc_ctx[dev] = ctx;
  }
  return g_noalloc_ptr[dev];
}

}  // namespace

// Called by every build on the regridder's device: loads this file's module
// (reserving the static scratch of crg_apply_noalloc) while the caller is
// still setting up, rather than at its first allocation-free apply, when its
// own pool may already hold the whole GPU.
void noalloc_prepare(int dev) { (void)noalloc_scratch(dev); }

void apply_noalloc_impl(const crg_regridder* r, int transpose, int dtype, const void* src, int64_t ssc, int64_t ssf,
                        void* dst, int64_t dsc, int64_t dsf, int64_t nf, int normalize, cudaStream_t st) {
  CRG_REQUIRE(r != nullptr, CRG_ERR_INVALID_ARGUMENT, "regridder is NULL");
  CRG_REQUIRE(dtype == CRG_F32 || dtype == CRG_BF16, CRG_ERR_NOT_SUPPORTED,
              "crg_apply_noalloc supports CRG_F32 and CRG_BF16 fields (got dtype %d)", dtype);
  CRG_REQUIRE(nf > 0 && nf % 4 == 0, CRG_ERR_NOT_SUPPORTED, "nfields must be a positive multiple of 4 (got %lld)",
              (long long)nf);
  CRG_REQUIRE(ssf == 1 && dsf == 1, CRG_ERR_NOT_SUPPORTED,
              "crg_apply_noalloc needs the fields of a cell side by side (field strides 1)");
  CRG_REQUIRE(ssc >= nf && dsc >= nf && ssc % 4 == 0 && dsc % 4 == 0, CRG_ERR_NOT_SUPPORTED,
              "cell strides must be >= nfields and multiples of 4");
  const size_t es = dtype == CRG_F32 ? 4 : 2;
  CRG_REQUIRE(src && dst && (uintptr_t)src % (4 * es) == 0 && (uintptr_t)dst % (4 * es) == 0, CRG_ERR_NOT_SUPPORTED,
              "field pointers must be non-NULL and %d-byte aligned", (int)(4 * es));
  CRG_REQUIRE(is_device_pointer(src) && is_device_pointer(dst), CRG_ERR_NOT_SUPPORTED,
              "crg_apply_noalloc takes device pointers only (host fields would need staging memory)");
  int dev = 0;
  CRG_CHECK_CUDA(cudaGetDevice(&dev));
  CRG_REQUIRE(dev == r->device, CRG_ERR_INVALID_ARGUMENT, "regridder lives on device %d but device %d is current",
              r->device, dev);
  const bool t = transpose != 0;
  const DevCsr& c = t ? r->rev : r->fwd;
  const size_t need = (size_t)c.nslots * 128 * sizeof(float);
  CRG_REQUIRE(need <= CRG_NOALLOC_SCRATCH_BYTES, CRG_ERR_NOT_SUPPORTED,
              "this regridder cuts %lld long rows into %lld pieces and needs %zu bytes of scratch; the static "
              "scratch of crg_apply_noalloc holds %u bytes (%lld pieces)",
              (long long)c.nsplit, (long long)c.nslots, need, (unsigned)CRG_NOALLOC_SCRATCH_BYTES,
              (long long)(CRG_NOALLOC_SCRATCH_BYTES / (128 * sizeof(float))));
  CRG_REQUIRE((double)c.ncols * (double)ssc * (double)es < 4.0e9, CRG_ERR_NOT_SUPPORTED,
              "source fields span 4 GB or more");
  float* carry = noalloc_scratch(dev);
  const float* w = normalize ? c.wn32 : c.val32;
  // the kernels crg_apply takes for these fields, with the static scratch
  if (nf < 32) {
    if (dtype == CRG_F32)
      launch_cm_narrow<float>(c, w, (const float*)src, ssc, (float*)dst, dsc, nf, st, true, carry);
    else
      launch_cm_narrow<__nv_bfloat16>(c, w, (const __nv_bfloat16*)src, ssc, (__nv_bfloat16*)dst, dsc, nf, st, true,
                                      carry);
    return;
  }
  if (dtype == CRG_F32)
    cm_nnz_passes<float>(c, w, (const float*)src, ssc, (float*)dst, dsc, nf, carry, st);
  else
    cm_nnz_passes<__nv_bfloat16>(c, w, (const __nv_bfloat16*)src, ssc, (__nv_bfloat16*)dst, dsc, nf, carry, st);
}

}  // namespace crg
