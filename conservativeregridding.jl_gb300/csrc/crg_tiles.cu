// crg_tiles.cu -- row tiles with shared-memory column staging for the batched
// apply (built once per regridder direction).
//
// Rows are taken in the spatial (cube-face Morton) order of their cells.  A
// tile is a run of consecutive rows in that order; for each tile the sorted
// set of distinct source columns it touches is stored, and every entry gets a
// 16-bit index into that set.  At apply time a CTA copies the tile's source
// field columns into shared memory once and then reads them from there, so a
// source element crosses L2 -> SM about once per tile instead of once per
// nonzero.  Tiles start at kTileRows rows; a tile that touches more than
// kTileUMax columns (or holds more than kTileEMax entries) is split into four
// quarter tiles, down to single rows; single rows that are still too wide
// (a coarse cell over a fine grid) go to the direct-gather kernels.
#include <algorithm>
#include <vector>

#include "crg_internal.cuh"
#include "crg_scan.cuh"

namespace crg {

namespace {

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

constexpr int kThreads = 256;

// Column indices of rows [p0, p0+nr) gathered into s_col[0..E), padded with
// INT_MAX to a power of two P and sorted; returns E, or -1 if E > kTileEMax.
__device__ int load_tile_cols(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                              const int32_t* __restrict__ rows, int64_t p0, int nr, int32_t* s_col, int32_t* s_off,
                              int32_t* s_rowbeg) {
  const int tid = threadIdx.x;
  if (tid < nr) {
    int32_t r = rows[p0 + tid];
    s_rowbeg[tid] = ptr[r];
    s_off[tid + 1] = ptr[r + 1] - ptr[r];
  }
  if (tid == 0) s_off[0] = 0;
  __syncthreads();
  if (tid == 0)
    for (int i = 0; i < nr; ++i) s_off[i + 1] += s_off[i];
  __syncthreads();
  const int E = s_off[nr];
  if (E > kTileEMax) return -1;
  int P = 1;
  while (P < E) P <<= 1;
  for (int e = tid; e < P; e += kThreads) {
    if (e < E) {
      int lo = 0, hi = nr - 1;  // row i with s_off[i] <= e < s_off[i+1]
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (s_off[mid] <= e) lo = mid;
        else hi = mid - 1;
      }
      s_col[e] = idx[s_rowbeg[lo] + (e - s_off[lo])];
    } else {
      s_col[e] = 0x7fffffff;
    }
  }
  __syncthreads();
  for (int k = 2; k <= P; k <<= 1) {  // bitonic sort
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = tid; i < P; i += kThreads) {
        int ixj = i ^ j;
        if (ixj > i) {
          int32_t a = s_col[i], b = s_col[ixj];
          bool up = (i & k) == 0;
          if ((a > b) == up) { s_col[i] = b; s_col[ixj] = a; }
        }
      }
      __syncthreads();
    }
  }
  return E;
}

// Distinct-column count of candidate tiles cand[b] = [id*TR, id*TR+TR); -1 if too large.
__global__ void __launch_bounds__(kThreads) k_tile_count(const int32_t* __restrict__ ptr,
                                                        const int32_t* __restrict__ idx,
                                                        const int32_t* __restrict__ rows, int64_t nrows,
                                                        const int32_t* __restrict__ cand, int TR,
                                                        int32_t* __restrict__ u_out) {
  __shared__ int32_t s_col[kTileEMax];
  __shared__ int32_t s_off[kTileRows + 1];
  __shared__ int32_t s_rowbeg[kTileRows];
  __shared__ int s_red[kThreads / 32];
  const int64_t p0 = (int64_t)cand[blockIdx.x] * TR;
  const int nr = (int)(nrows - p0 < TR ? nrows - p0 : TR);
  const int E = load_tile_cols(ptr, idx, rows, p0, nr, s_col, s_off, s_rowbeg);
  if (E < 0) {
    if (threadIdx.x == 0) u_out[blockIdx.x] = -1;
    return;
  }
  int c = 0;
  for (int i = threadIdx.x; i < E; i += kThreads) c += (i == 0 || s_col[i] != s_col[i - 1]) ? 1 : 0;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int u = 0;
    for (int w = 0; w < kThreads / 32; ++w) u += s_red[w];
    u_out[blockIdx.x] = u <= kTileUMax ? u : -1;
  }
}

// Good tiles: distinct columns, 16-bit local column of every entry, and the
// three weight arrays permuted into processing order.
__global__ void __launch_bounds__(kThreads) k_tile_fill(const int32_t* __restrict__ ptr,
                                                       const int32_t* __restrict__ idx,
                                                       const float* __restrict__ val32, const float* __restrict__ wn32,
                                                       const float* __restrict__ adj32,
                                                       const int32_t* __restrict__ rows,
                                                       const int2* __restrict__ tiles,
                                                       const int32_t* __restrict__ uoff,
                                                       const int32_t* __restrict__ lptr, int32_t* __restrict__ ucol,
                                                       uint16_t* __restrict__ lcol, float* __restrict__ lw_val,
                                                       float* __restrict__ lw_wn, float* __restrict__ lw_adj) {
  __shared__ int32_t s_col[kTileEMax];
  __shared__ int32_t s_uniq[kTileUMax];
  __shared__ int32_t s_off[kTileRows + 1];
  __shared__ int32_t s_rowbeg[kTileRows];
  __shared__ int32_t s_wcnt[kThreads / 32 + 1];
  const int2 tr = tiles[blockIdx.x];
  const int64_t p0 = tr.x;
  const int nr = tr.y - tr.x;
  const int E = load_tile_cols(ptr, idx, rows, p0, nr, s_col, s_off, s_rowbeg);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int base = 0;
  for (int c0 = 0; c0 < E; c0 += kThreads) {
    int i = c0 + tid;
    int flag = (i < E && (i == 0 || s_col[i] != s_col[i - 1])) ? 1 : 0;
    unsigned m = __ballot_sync(0xffffffffu, flag);
    int pre = __popc(m & ((1u << lane) - 1));
    if (lane == 0) s_wcnt[warp] = __popc(m);
    __syncthreads();
    if (tid == 0) {
      int run = 0;
      for (int w = 0; w < kThreads / 32; ++w) { int x = s_wcnt[w]; s_wcnt[w] = run; run += x; }
      s_wcnt[kThreads / 32] = run;
    }
    __syncthreads();
    if (flag) s_uniq[base + s_wcnt[warp] + pre] = s_col[i];
    base += s_wcnt[kThreads / 32];
    __syncthreads();
  }
  const int u = base;
  const int32_t u0 = uoff[blockIdx.x];
  for (int i = tid; i < u; i += kThreads) ucol[u0 + i] = s_uniq[i];
  for (int e = tid; e < E; e += kThreads) {
    int lo = 0, hi = nr - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (s_off[mid] <= e) lo = mid;
      else hi = mid - 1;
    }
    const int32_t src = s_rowbeg[lo] + (e - s_off[lo]);
    const int32_t col = idx[src];
    int a = 0, b = u - 1;
    while (a < b) {
      int mid = (a + b) >> 1;
      if (s_uniq[mid] < col) a = mid + 1;
      else b = mid;
    }
    const int32_t dk = lptr[p0 + lo] + (e - s_off[lo]);
    lcol[dk] = (uint16_t)a;
    lw_val[dk] = val32[src];
    lw_wn[dk] = wn32[src];
    lw_adj[dk] = adj32[src];
  }
}

// Rows keyed by their first (smallest) column; empty rows get key ncols.
__global__ void k_firstcol_hist(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx, int64_t n,
                                int64_t ncols, int32_t* __restrict__ cnt) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int32_t k = ptr[r];
  atomicAdd(&cnt[k < ptr[r + 1] ? idx[k] : ncols], 1);
}

__global__ void k_firstcol_scatter(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx, int64_t n,
                                   int64_t ncols, const int32_t* __restrict__ off, int32_t* __restrict__ fill,
                                   int32_t* __restrict__ order) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int32_t k = ptr[r];
  const int64_t key = k < ptr[r + 1] ? idx[k] : ncols;
  order[off[key] + atomicAdd(&fill[key], 1)] = (int32_t)r;
}

__global__ void k_len_perm(const int32_t* __restrict__ ptr, const int32_t* __restrict__ rows, int64_t n,
                           int32_t* __restrict__ len) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) {
    int32_t r = rows[p];
    len[p] = ptr[r + 1] - ptr[r];
  }
}

template <class T>
T* palloc(size_t n) {
  T* p = nullptr;
  CRG_CHECK_CUDA(cudaMalloc((void**)&p, (n ? n : 1) * sizeof(T)));
  return p;
}

template <class T>
T* upload(const std::vector<T>& v) {
  T* p = palloc<T>(v.size());
  if (!v.empty()) CRG_CHECK_CUDA(cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  return p;
}

}  // namespace

void free_tiles(DevTiles& t) {
  cudaFree(t.rows); cudaFree(t.lptr); cudaFree(t.lcol); cudaFree(t.lw_val); cudaFree(t.lw_wn); cudaFree(t.lw_adj);
  cudaFree(t.tiles); cudaFree(t.uoff); cudaFree(t.ucol); cudaFree(t.direct);
  t = DevTiles{};
}

void build_tiles(DevCsr& c, const int32_t* row_order, cudaStream_t st) {
  DevTiles& T = c.tiles;
  const int64_t n = c.nrows, nnz = c.nnz;
  // rows by first column: counting sort over ncols + 1 keys
  c.order_by_col = palloc<int32_t>((size_t)n);
  if (n > 0) {
    const int64_t nk = c.ncols + 1;
    int32_t *cnt = nullptr, *fill = nullptr;
    CRG_CHECK_CUDA(cudaMallocAsync((void**)&cnt, sizeof(int32_t) * (nk + 1), st));
    CRG_CHECK_CUDA(cudaMallocAsync((void**)&fill, sizeof(int32_t) * nk, st));
    CRG_CHECK_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (nk + 1), st));
    CRG_CHECK_CUDA(cudaMemsetAsync(fill, 0, sizeof(int32_t) * nk, st));
    k_firstcol_hist<<<nblk(n, 256), 256, 0, st>>>(c.ptr, c.idx, n, c.ncols, cnt);
    CRG_CHECK_CUDA(cudaGetLastError());
    exclusive_scan_i32(cnt, cnt, nk, st);
    k_firstcol_scatter<<<nblk(n, 256), 256, 0, st>>>(c.ptr, c.idx, n, c.ncols, cnt, fill, c.order_by_col);
    CRG_CHECK_CUDA(cudaGetLastError());
    CRG_CHECK_CUDA(cudaFreeAsync(cnt, st));
    CRG_CHECK_CUDA(cudaFreeAsync(fill, st));
  }
  T.rows = palloc<int32_t>((size_t)n);
  T.lptr = palloc<int32_t>((size_t)n + 1);
  T.lcol = palloc<uint16_t>((size_t)nnz);
  T.lw_val = palloc<float>((size_t)nnz);
  T.lw_wn = palloc<float>((size_t)nnz);
  T.lw_adj = palloc<float>((size_t)nnz);
  std::vector<int2> good;
  std::vector<int32_t> gu, direct;
  if (n > 0) {
    CRG_CHECK_CUDA(cudaMemcpyAsync(T.rows, row_order, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, st));
    k_len_perm<<<nblk(n, 256), 256, 0, st>>>(c.ptr, T.rows, n, T.lptr);
    CRG_CHECK_CUDA(cudaGetLastError());
    exclusive_scan_i32(T.lptr, T.lptr, n, st);
    // refinement: tiles of kTileRows, then quarters, down to single rows
    std::vector<int32_t> cand((size_t)((n + kTileRows - 1) / kTileRows));
    for (size_t i = 0; i < cand.size(); ++i) cand[i] = (int32_t)i;
    int32_t* dcand = nullptr;
    int32_t* du = nullptr;
    size_t cap = 0;
    for (int TR = kTileRows; TR >= 1 && !cand.empty(); TR /= 4) {
      if (cand.size() > cap) {
        if (dcand) { cudaFreeAsync(dcand, st); cudaFreeAsync(du, st); }
        cap = cand.size();
        CRG_CHECK_CUDA(cudaMallocAsync((void**)&dcand, sizeof(int32_t) * cap, st));
        CRG_CHECK_CUDA(cudaMallocAsync((void**)&du, sizeof(int32_t) * cap, st));
      }
      CRG_CHECK_CUDA(cudaMemcpyAsync(dcand, cand.data(), sizeof(int32_t) * cand.size(), cudaMemcpyHostToDevice, st));
      k_tile_count<<<(unsigned)cand.size(), kThreads, 0, st>>>(c.ptr, c.idx, T.rows, n, dcand, TR, du);
      CRG_CHECK_CUDA(cudaGetLastError());
      std::vector<int32_t> u(cand.size());
      CRG_CHECK_CUDA(cudaMemcpyAsync(u.data(), du, sizeof(int32_t) * u.size(), cudaMemcpyDeviceToHost, st));
      CRG_CHECK_CUDA(cudaStreamSynchronize(st));
      std::vector<int32_t> next;
      const int sub = TR / 4;
      for (size_t i = 0; i < cand.size(); ++i) {
        const int64_t p0 = (int64_t)cand[i] * TR, p1 = std::min<int64_t>(n, p0 + TR);
        if (u[i] >= 0) {
          good.push_back(make_int2((int)p0, (int)p1));
          gu.push_back(u[i]);
        } else if (TR > 1) {
          for (int j = 0; j < 4; ++j) {
            int64_t q = (int64_t)cand[i] * 4 + j;
            if (q * sub < n) next.push_back((int32_t)q);
          }
        } else {
          direct.push_back((int32_t)p0);
        }
      }
      cand.swap(next);
      if (TR == 1) break;
    }
    if (dcand) { cudaFreeAsync(dcand, st); cudaFreeAsync(du, st); }
  } else {
    CRG_CHECK_CUDA(cudaMemsetAsync(T.lptr, 0, sizeof(int32_t), st));
  }
  // process tiles in row order (neighbouring CTAs share source columns in L2)
  std::vector<size_t> order(good.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return good[a].x < good[b].x; });
  std::vector<int2> gs(good.size());
  std::vector<int32_t> uoff(good.size() + 1, 0);
  for (size_t i = 0; i < order.size(); ++i) {
    gs[i] = good[order[i]];
    uoff[i + 1] = uoff[i] + gu[order[i]];
  }
  std::sort(direct.begin(), direct.end());
  CRG_CHECK_CUDA(cudaStreamSynchronize(st));
  T.ngood = (int64_t)gs.size();
  T.ndirect = (int64_t)direct.size();
  T.nucol = uoff.back();
  T.tiles = upload(gs);
  T.uoff = upload(uoff);
  T.direct = upload(direct);
  T.ucol = palloc<int32_t>((size_t)T.nucol);
  if (T.ngood) {
    k_tile_fill<<<(unsigned)T.ngood, kThreads, 0, st>>>(c.ptr, c.idx, c.val32, c.wn32, c.adj32, T.rows, T.tiles,
                                                        T.uoff, T.lptr, T.ucol, T.lcol, T.lw_val, T.lw_wn, T.lw_adj);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
}

}  // namespace crg
