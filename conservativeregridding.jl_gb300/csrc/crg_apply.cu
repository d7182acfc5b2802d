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
//   k_spmm_rows     FP32/BF16 fields stored cell-major (the fields of one cell
//                   side by side): G lanes per row, each lane owns 4
//                   consecutive fields (128-bit FP32 / 64-bit BF16 loads),
//                   FP32 accumulation, weights read once per row.
//   k_spmm_tile     FP32/BF16 fields stored field-major (dims = 1): a block
//                   owns 128 consecutive rows, stages their (column, weight)
//                   entries in shared memory once, then sweeps all fields.
//   k_spmm_generic  any strides, one thread per (row, field).
#include <cuda_bf16.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>

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
  uint2 u = __ldg(reinterpret_cast<const uint2*>(p));
  __nv_bfloat162 a = *reinterpret_cast<__nv_bfloat162*>(&u.x);
  __nv_bfloat162 b = *reinterpret_cast<__nv_bfloat162*>(&u.y);
  float2 fa = __bfloat1622float2(a), fb = __bfloat1622float2(b);
  return make_float4(fa.x, fa.y, fb.x, fb.y);
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
  for (int32_t k = ptr[r]; k < ptr[r + 1]; ++k) {
    int32_t j = idx[k];
    double xv = xf[(int64_t)j * xsc];
    if (col_div) xv = xv / col_div[j];
    acc = acc + val[k] * xv;
  }
  if (row_div) acc = acc / row_div[r];
  y[r * ysc + f * ysf] = acc;
}

// ------------------------------------------------------------------ cell-major fields

template <class T, int G, bool kVec>
__global__ void __launch_bounds__(256) k_spmm_rows(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                                   const float* __restrict__ w, int64_t nrows, const T* __restrict__ x,
                                                   int64_t xsc, T* __restrict__ y, int64_t ysc, int64_t nf) {
  const int g = threadIdx.x % G;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  if (r >= nrows) return;
  const int32_t k0 = ptr[r], k1 = ptr[r + 1];
  for (int64_t f = (int64_t)g * 4; f < nf; f += (int64_t)G * 4) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    const bool full = kVec && f + 4 <= nf;
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
    T* yp = y + r * ysc + f;
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

// ------------------------------------------------------------------ field-major fields

constexpr int kFmRows = 128;
constexpr int kFmEntries = 4096;  // shared-memory capacity (32 KB)
constexpr int kFmF = 8;           // fields per sweep step

template <class T>
__global__ void __launch_bounds__(kFmRows) k_spmm_tile(const int32_t* __restrict__ ptr,
                                                          const int32_t* __restrict__ idx,
                                                          const float* __restrict__ w, int64_t nrows,
                                                          const T* __restrict__ x, int64_t xsf, T* __restrict__ y,
                                                          int64_t ysf, int64_t nf) {
  __shared__ int32_t s_idx[kFmEntries];
  __shared__ float s_w[kFmEntries];
  const int64_t r0 = (int64_t)blockIdx.x * kFmRows;
  const int64_t r = r0 + threadIdx.x;
  const int64_t rend = min(nrows, r0 + kFmRows);
  const int32_t e0 = ptr[r0], e1 = ptr[rend];
  const bool staged = (e1 - e0) <= kFmEntries;
  if (staged) {
    for (int32_t e = e0 + threadIdx.x; e < e1; e += kFmRows) {
      s_idx[e - e0] = idx[e];
      s_w[e - e0] = w[e];
    }
  }
  __syncthreads();
  if (r >= nrows) return;
  const int32_t k0 = ptr[r], k1 = ptr[r + 1];
  for (int64_t f0 = 0; f0 < nf; f0 += kFmF) {
    float acc[kFmF];
#pragma unroll
    for (int q = 0; q < kFmF; ++q) acc[q] = 0.f;
    const int nq = (int)(nf - f0 < kFmF ? nf - f0 : kFmF);
    for (int32_t k = k0; k < k1; ++k) {
      const int64_t j = staged ? s_idx[k - e0] : idx[k];
      const float ww = staged ? s_w[k - e0] : w[k];
      const T* xp = x + f0 * xsf + j;
#pragma unroll
      for (int q = 0; q < kFmF; ++q)
        if (q < nq) acc[q] = fmaf(ww, ld1<T>(xp + q * xsf), acc[q]);
    }
    T* yp = y + f0 * ysf + r;
#pragma unroll
    for (int q = 0; q < kFmF; ++q)
      if (q < nq) st1<T>(yp + q * ysf, acc[q]);
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

// ------------------------------------------------------------------ staged tiles

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <class T> __device__ __forceinline__ float4 lds4(const T* p);
template <> __device__ __forceinline__ float4 lds4<float>(const float* p) { return *reinterpret_cast<const float4*>(p); }
template <> __device__ __forceinline__ float4 lds4<__nv_bfloat16>(const __nv_bfloat16* p) {
  uint2 u = *reinterpret_cast<const uint2*>(p);
  float2 a = __bfloat1622float2(*reinterpret_cast<__nv_bfloat162*>(&u.x));
  float2 b = __bfloat1622float2(*reinterpret_cast<__nv_bfloat162*>(&u.y));
  return make_float4(a.x, a.y, b.x, b.y);
}

template <class T, int KC>
__host__ __device__ constexpr int stage_stride() { return KC + 16 / (int)sizeof(T); }

template <class T, bool kFM, int KC>
constexpr size_t tiled_smem() {
  return (size_t)kTileUMax * stage_stride<T, KC>() * sizeof(T) + (kFM ? (size_t)kTileRows * (KC + 1) * sizeof(float) : 0);
}

// One CTA per staged tile.  For each chunk of KC fields: copy the tile's
// distinct source columns into shared memory (cp.async; 16-byte pieces of a
// cell's contiguous fields when cell-major, 4-byte gathers when field-major),
// then G = KC/4 lanes per row accumulate 4 fields each from shared memory in
// FP32 and write the row (cell-major) or stage it and write field by field
// (field-major, so the stores are runs of consecutive cells).
template <class T, bool kFM, int KC>
__global__ void __launch_bounds__(256, 2) k_spmm_tiled(const int2* __restrict__ tiles, const int32_t* __restrict__ uoff,
                                                       const int32_t* __restrict__ ucol,
                                                       const int32_t* __restrict__ rows,
                                                       const int32_t* __restrict__ lptr,
                                                       const uint16_t* __restrict__ lcol,
                                                       const float* __restrict__ lw, const T* __restrict__ x,
                                                       int64_t xs, T* __restrict__ y, int64_t ys, int64_t nf) {
  constexpr int SP = stage_stride<T, KC>();
  constexpr int G = KC / 4;
  constexpr int RPW = 32 / G;
  constexpr int OS = KC + 1;
  extern __shared__ __align__(16) unsigned char smem[];
  T* stage = reinterpret_cast<T*>(smem);
  float* outs = reinterpret_cast<float*>(smem + (size_t)kTileUMax * SP * sizeof(T));
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane % G, sub = lane / G;
  const int2 tr = tiles[blockIdx.x];
  const int p0 = tr.x, nr = tr.y - tr.x;
  const int u0 = uoff[blockIdx.x], u = uoff[blockIdx.x + 1] - u0;
  for (int64_t f0 = 0; f0 < nf; f0 += KC) {
    const int kc = (int)(nf - f0 < KC ? nf - f0 : KC);
    if (!kFM) {
      const int cpc = kc * (int)sizeof(T) / 16;
      for (int i = tid; i < u * cpc; i += 256) {
        const int c = i / cpc, q = i - c * cpc;
        cp_async16(stage + c * SP + q * (16 / (int)sizeof(T)), x + (int64_t)__ldg(ucol + u0 + c) * xs + f0 + q * (16 / (int)sizeof(T)));
      }
    } else {
      for (int i = tid; i < u * kc; i += 256) {
        const int f = i / u, c = i - f * u;
        const T* src = x + (f0 + f) * xs + __ldg(ucol + u0 + c);
        if (sizeof(T) == 4) cp_async4(stage + c * SP + f, src);
        else stage[c * SP + f] = *src;
      }
    }
    cp_async_wait_all();
    __syncthreads();
    for (int rb = warp * RPW + sub; rb < nr; rb += 8 * RPW) {
      const int p = p0 + rb;
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
      if (g * 4 < kc) {
        const int k1 = lptr[p + 1];
        for (int k = lptr[p]; k < k1; ++k) {
          const int lc = lcol[k];
          const float w = lw[k];
          const float4 v = lds4<T>(stage + lc * SP + g * 4);
          acc.x = fmaf(w, v.x, acc.x);
          acc.y = fmaf(w, v.y, acc.y);
          acc.z = fmaf(w, v.z, acc.z);
          acc.w = fmaf(w, v.w, acc.w);
        }
        if (!kFM) {
          st4<T>(y + (int64_t)rows[p] * ys + f0 + g * 4, acc);
        } else {
          float* o = outs + rb * OS + g * 4;
          o[0] = acc.x; o[1] = acc.y; o[2] = acc.z; o[3] = acc.w;
        }
      }
    }
    if (kFM) {
      __syncthreads();
      for (int i = tid; i < kc * nr; i += 256) {
        const int f = i / nr, r = i - f * nr;
        st1<T>(y + (f0 + f) * ys + rows[p0 + r], outs[r * OS + f]);
      }
    }
    __syncthreads();
  }
}

// Rows left out of the tiles (too many distinct columns), cell-major fields:
// one warp per row, 4 fields per lane.
template <class T>
__global__ void __launch_bounds__(256) k_direct_cm(const int32_t* __restrict__ pos, int64_t npos,
                                                   const int32_t* __restrict__ rows, const int32_t* __restrict__ ptr,
                                                   const int32_t* __restrict__ idx, const float* __restrict__ w,
                                                   const T* __restrict__ x, int64_t xs, T* __restrict__ y, int64_t ys,
                                                   int64_t nf) {
  const int64_t wi = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wi >= npos) return;
  const int32_t r = rows[pos[wi]];
  const int32_t k0 = ptr[r], k1 = ptr[r + 1];
  for (int64_t f = (int64_t)lane * 4; f < nf; f += 128) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int32_t k = k0; k < k1; ++k) {
      const float4 v = ld4<T>(x + (int64_t)idx[k] * xs + f);
      const float ww = w[k];
      acc.x = fmaf(ww, v.x, acc.x);
      acc.y = fmaf(ww, v.y, acc.y);
      acc.z = fmaf(ww, v.z, acc.z);
      acc.w = fmaf(ww, v.w, acc.w);
    }
    st4<T>(y + (int64_t)r * ys + f, acc);
  }
}

// Rows left out of the tiles, field-major fields: one warp per row, lanes
// split the row's entries, warp reduction per field.
template <class T>
__global__ void __launch_bounds__(256) k_direct_fm(const int32_t* __restrict__ pos, int64_t npos,
                                                   const int32_t* __restrict__ rows, const int32_t* __restrict__ ptr,
                                                   const int32_t* __restrict__ idx, const float* __restrict__ w,
                                                   const T* __restrict__ x, int64_t xs, T* __restrict__ y, int64_t ys,
                                                   int64_t nf) {
  const int64_t wi = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wi >= npos) return;
  const int32_t r = rows[pos[wi]];
  const int32_t k0 = ptr[r], k1 = ptr[r + 1];
  for (int64_t f = 0; f < nf; ++f) {
    float acc = 0.f;
    for (int32_t k = k0 + lane; k < k1; k += 32) acc = fmaf(w[k], ld1<T>(x + f * xs + idx[k]), acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) st1<T>(y + f * ys + r, acc);
  }
}

template <class T, bool kFM, int KC>
void launch_tiled_kc(const DevCsr& c, bool normalize, bool adjoint, const T* x, int64_t xs, T* y, int64_t ys,
                     int64_t nf, cudaStream_t st) {
  const DevTiles& tl = c.tiles;
  const float* lw = normalize ? (adjoint ? tl.lw_adj : tl.lw_wn) : tl.lw_val;
  const float* w = normalize ? (adjoint ? c.adj32 : c.wn32) : c.val32;
  constexpr size_t smem = tiled_smem<T, kFM, KC>();
  static bool configured = false;  // per template instance
  if (!configured) {
    CRG_CHECK_CUDA(cudaFuncSetAttribute(k_spmm_tiled<T, kFM, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured = true;
  }
  if (tl.ngood) {
    k_spmm_tiled<T, kFM, KC><<<(unsigned)tl.ngood, 256, smem, st>>>(tl.tiles, tl.uoff, tl.ucol, tl.rows, tl.lptr, tl.lcol,
                                                                     lw, x, xs, y, ys, nf);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
  if (tl.ndirect) {
    const unsigned blocks = nblk(tl.ndirect * 32, 256);
    if (kFM) k_direct_fm<T><<<blocks, 256, 0, st>>>(tl.direct, tl.ndirect, tl.rows, c.ptr, c.idx, w, x, xs, y, ys, nf);
    else k_direct_cm<T><<<blocks, 256, 0, st>>>(tl.direct, tl.ndirect, tl.rows, c.ptr, c.idx, w, x, xs, y, ys, nf);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
}

template <class T, bool kFM>
void launch_tiled(const DevCsr& c, bool normalize, bool adjoint, const T* x, int64_t xs, T* y, int64_t ys, int64_t nf,
                  cudaStream_t st) {
  if (nf >= 128) launch_tiled_kc<T, kFM, 128>(c, normalize, adjoint, x, xs, y, ys, nf, st);
  else if (nf >= 64) launch_tiled_kc<T, kFM, 64>(c, normalize, adjoint, x, xs, y, ys, nf, st);
  else launch_tiled_kc<T, kFM, 32>(c, normalize, adjoint, x, xs, y, ys, nf, st);
}

// Kernel choice for FP32/BF16 fields.  CRG_SPMM_PATH selects an alternative
// for tuning and profiling: "tiled" (shared-memory staged tiles) or "legacy"
// (first-generation row kernels); unset = the register-blocked row kernels.
enum class SpmmPath { kRows, kTiled, kLegacy };

inline SpmmPath spmm_path() {
  static const SpmmPath p = [] {
    const char* e = getenv("CRG_SPMM_PATH");
    if (e && strcmp(e, "tiled") == 0) return SpmmPath::kTiled;
    if (e && strcmp(e, "legacy") == 0) return SpmmPath::kLegacy;
    return SpmmPath::kRows;
  }();
  return p;
}

template <class T>
void launch_cm_rows(const DevCsr& c, const float* w, const T* x, int64_t xs, T* y, int64_t ys, int64_t nf,
                    cudaStream_t st) {
  const int64_t n = c.nrows;
  const int64_t lanes = (std::min<int64_t>(nf, 128) + 3) / 4;
  int G = 1;
  while (G < lanes) G <<= 1;
  static const int RB = [] {
    const char* e = getenv("CRG_SPMM_RB");
    int v = e ? atoi(e) : 2;
    return (v == 1 || v == 2 || v == 4) ? v : 2;
  }();
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
}

template <class T>
void launch_f32(const DevCsr& c, bool normalize, bool adjoint, const T* x, int64_t xsc, int64_t xsf, T* y,
                int64_t ysc, int64_t ysf, int64_t nf, cudaStream_t st) {
  const int64_t n = c.nrows;
  if (n == 0 || nf == 0) return;
  const float* w = normalize ? (adjoint ? c.adj32 : c.wn32) : c.val32;
  const bool cell_major = (xsf == 1 && ysf == 1) && nf > 1;
  const bool field_major = (xsc == 1 && ysc == 1);
  const int es = (int)sizeof(T);
  const int vecf = 16 / es;  // fields per 16 bytes
  // 4-field vectors: 16-byte (FP32) / 8-byte (BF16) aligned loads and stores
  const bool vec4 = nf % 4 == 0 && xsc % 4 == 0 && ysc % 4 == 0 && (uintptr_t)x % (4 * es) == 0 &&
                    (uintptr_t)y % (4 * es) == 0;
  const SpmmPath path = spmm_path();
  if (path == SpmmPath::kTiled) {
    if (cell_major && nf >= 16 && nf % vecf == 0 && xsc % vecf == 0 && ysc % 4 == 0 && (uintptr_t)x % 16 == 0 &&
        (uintptr_t)y % (4 * es) == 0) {
      launch_tiled<T, false>(c, normalize, adjoint, x, xsc, y, ysc, nf, st);
      return;
    }
    if (field_major && nf >= 16) {
      launch_tiled<T, true>(c, normalize, adjoint, x, xsf, y, ysf, nf, st);
      return;
    }
  }
  if (path == SpmmPath::kRows) {
    if (cell_major && vec4) {
      launch_cm_rows<T>(c, w, x, xsc, y, ysc, nf, st);
      CRG_CHECK_CUDA(cudaGetLastError());
      return;
    }
    if (field_major) {
      static const bool by_col = [] {
        const char* e = getenv("CRG_FM_ORDER");
        return !(e && strcmp(e, "natural") == 0);
      }();
      k_fm_rows<T><<<nblk(n, 256), 256, 0, st>>>(c.ptr, c.idx, w, n, by_col ? c.order_by_col : nullptr, x, xsf, y,
                                                ysf, nf);
      CRG_CHECK_CUDA(cudaGetLastError());
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
  } else if (field_major && nf > 1) {
    k_spmm_tile<T><<<nblk(n, kFmRows), kFmRows, 0, st>>>(c.ptr, c.idx, w, n, x, xsf, y, ysf, nf);
  } else {
    for (int64_t f0 = 0; f0 < nf; f0 += 65535) {
      dim3 grid(nblk(n, 256), (unsigned)std::min<int64_t>(65535, nf - f0));
      k_spmm_generic<T><<<grid, 256, 0, st>>>(c.ptr, c.idx, w, n, x, xsc, xsf, y, ysc, ysf, f0);
    }
  }
  CRG_CHECK_CUDA(cudaGetLastError());
}

size_t elem_size(int dtype) { return dtype == CRG_F64 ? 8 : (dtype == CRG_F32 ? 4 : 2); }

}  // namespace

void apply_impl(const crg_regridder* rc, int transpose, int dtype, bool adjoint, const void* src, int64_t ssc,
                int64_t ssf, void* dst, int64_t dsc, int64_t dsf, int64_t nf, int normalize, cudaStream_t st) {
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

  std::unique_lock<std::mutex> lock(r->stage_mu, std::defer_lock);
  const void* xs = src;
  void* ys = dst;
  if (src_host || dst_host) {
    lock.lock();
    size_t need = (src_host ? (size_t)in_span * es : 0) + (dst_host ? (size_t)out_span * es : 0) + 256;
    if (r->stage_bytes < need) {
      if (r->stage) CRG_CHECK_CUDA(cudaFree(r->stage));
      r->stage = nullptr;
      r->stage_bytes = 0;
      CRG_CHECK_CUDA(cudaMalloc(&r->stage, need));
      r->stage_bytes = need;
    }
    char* base = (char*)r->stage;
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
  }

  if (dtype == CRG_F64) {
    const double* cdiv = adjoint ? div : nullptr;
    const double* rdiv = adjoint ? nullptr : div;
    for (int64_t f0 = 0; f0 < nf; f0 += 65535) {
      dim3 grid(nblk(nout, 128), (unsigned)std::min<int64_t>(65535, nf - f0));
      k_spmv_f64<<<grid, 128, 0, st>>>(c.ptr, c.idx, c.val, nout, (const double*)xs, ssc, ssf, (double*)ys, dsc, dsf,
                                       f0, rdiv, cdiv);
    }
    CRG_CHECK_CUDA(cudaGetLastError());
  } else {
    if (dtype == CRG_F32)
      launch_f32<float>(c, normalize, adjoint, (const float*)xs, ssc, ssf, (float*)ys, dsc, dsf, nf, st);
    else
      launch_f32<__nv_bfloat16>(c, normalize, adjoint, (const __nv_bfloat16*)xs, ssc, ssf, (__nv_bfloat16*)ys, dsc,
                                dsf, nf, st);
  }

  if (dst_host) CRG_CHECK_CUDA(cudaMemcpyAsync(dst, ys, (size_t)out_span * es, cudaMemcpyDeviceToHost, st));
  if (src_host || dst_host) CRG_CHECK_CUDA(cudaStreamSynchronize(st));
}

}  // namespace crg
