// crg_tiles.cu -- row tiles for the staged batched apply (built once per
// regridder direction).
//
// Rows are taken in the spatial (cube-face Morton) order of their cells.  A
// tile is a run of consecutive rows in that order; per tile the library keeps
// (a) the sorted distinct source columns it touches, with a 16-bit index into
// that set for every entry -- the staging unit for fields stored cell-major,
// where one column is the contiguous vector of a cell's fields -- and (b) the
// sorted distinct 4-cell chunks (column >> 2) with a 16-bit index
// 4 * chunk + (column & 3) for every entry -- the staging unit for fields
// stored field-major, where a chunk is one aligned 16-byte (FP32) piece of a
// field.  At apply time a CTA copies a tile's pieces into shared memory with
// asynchronous copies and computes from there.  Tiles start at kTileRows rows;
// a tile touching more than kTileUMax columns (or holding more than kTileEMax
// entries) is split into quarters down to single rows; single rows that are
// still too wide (a coarse cell over a fine grid) go to direct-gather kernels.
#include <algorithm>
#include <vector>

#include <stdlib.h>
#include <string.h>

#include "crg_internal.cuh"
#include "crg_scan.cuh"

namespace crg {

namespace {

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

constexpr int kThreads = 256;

// Column indices of rows [p0, p0+nr) gathered into s_col[0..E), padded with
// INT_MAX to a power of two and sorted; returns E, or -1 if E > kTileEMax.
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

__device__ __forceinline__ int block_count(int c, int* s_red) {
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = c;
  __syncthreads();
  int t = 0;
  for (int w = 0; w < kThreads / 32; ++w) t += s_red[w];
  __syncthreads();
  return t;
}

// Candidate tiles [id*TR, id*TR+TR): distinct columns and distinct chunks
// (-1 in u_out when the tile has to be split).
__global__ void __launch_bounds__(kThreads) k_tile_count(const int32_t* __restrict__ ptr,
                                                        const int32_t* __restrict__ idx,
                                                        const int32_t* __restrict__ rows, int64_t nrows,
                                                        const int32_t* __restrict__ cand, int TR,
                                                        int32_t* __restrict__ u_out, int32_t* __restrict__ c_out) {
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
  int cu = 0, cc = 0;
  for (int i = threadIdx.x; i < E; i += kThreads) {
    cu += (i == 0 || s_col[i] != s_col[i - 1]) ? 1 : 0;
    cc += (i == 0 || (s_col[i] >> 2) != (s_col[i - 1] >> 2)) ? 1 : 0;
  }
  const int u = block_count(cu, s_red);
  const int nc = block_count(cc, s_red);
  if (threadIdx.x == 0) {
    u_out[blockIdx.x] = u <= kTileUMax ? u : -1;
    c_out[blockIdx.x] = nc;
  }
}

// Order-preserving compaction of the flagged keys of s_col[0..E) into out.
__device__ int compact_sorted(const int32_t* s_col, int E, int shift, int32_t* out, int32_t* s_wcnt) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int base = 0;
  for (int c0 = 0; c0 < E; c0 += kThreads) {
    int i = c0 + tid;
    int flag = (i < E && (i == 0 || (s_col[i] >> shift) != (s_col[i - 1] >> shift))) ? 1 : 0;
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
    if (flag) out[base + s_wcnt[warp] + pre] = s_col[i] >> shift;
    base += s_wcnt[kThreads / 32];
    __syncthreads();
  }
  return base;
}

__device__ __forceinline__ int lower_bound(const int32_t* a, int n, int32_t key) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Good tiles: distinct columns and chunks, the two 16-bit local indices of
// every entry, and the three weight arrays permuted into processing order.
__global__ void __launch_bounds__(kThreads) k_tile_fill(const int32_t* __restrict__ ptr,
                                                       const int32_t* __restrict__ idx,
                                                       const float* __restrict__ val32, const float* __restrict__ wn32,
                                                       const float* __restrict__ adj32,
                                                       const int32_t* __restrict__ rows,
                                                       const int32_t* __restrict__ desc,
                                                       const int32_t* __restrict__ lptr, int32_t* __restrict__ ucol,
                                                       int32_t* __restrict__ uchunk, uint16_t* __restrict__ lcol,
                                                       uint16_t* __restrict__ lchk, float* __restrict__ lw_val,
                                                       float* __restrict__ lw_wn, float* __restrict__ lw_adj) {
  __shared__ int32_t s_col[kTileEMax];
  __shared__ int32_t s_uniq[kTileUMax];
  __shared__ int32_t s_chunk[kTileUMax];
  __shared__ int32_t s_off[kTileRows + 1];
  __shared__ int32_t s_rowbeg[kTileRows];
  __shared__ int32_t s_wcnt[kThreads / 32 + 1];
  const int32_t* d = desc + (int64_t)blockIdx.x * kDescInts;
  const int64_t p0 = d[kDescP0];
  const int nr = d[kDescNr];
  const int E = load_tile_cols(ptr, idx, rows, p0, nr, s_col, s_off, s_rowbeg);
  const int u = compact_sorted(s_col, E, 0, s_uniq, s_wcnt);
  const int nc = compact_sorted(s_col, E, 2, s_chunk, s_wcnt);
  const int tid = threadIdx.x;
  for (int i = tid; i < u; i += kThreads) ucol[d[kDescU0] + i] = s_uniq[i];
  for (int i = tid; i < nc; i += kThreads) uchunk[d[kDescC0] + i] = s_chunk[i];
  for (int e = tid; e < E; e += kThreads) {
    int lo = 0, hi = nr - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (s_off[mid] <= e) lo = mid;
      else hi = mid - 1;
    }
    const int32_t src = s_rowbeg[lo] + (e - s_off[lo]);
    const int32_t col = idx[src];
    const int32_t dk = lptr[p0 + lo] + (e - s_off[lo]);
    lcol[dk] = (uint16_t)lower_bound(s_uniq, u, col);
    lchk[dk] = (uint16_t)(4 * lower_bound(s_chunk, nc, col >> 2) + (col & 3));
    lw_val[dk] = val32[src];
    lw_wn[dk] = wn32[src];
    lw_adj[dk] = adj32[src];
  }
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
T* upload(const std::vector<T>& v, cudaStream_t st) {
  T* p = keep_alloc<T>(v.size(), st);
  if (!v.empty()) {
    CRG_CHECK_CUDA(cudaMemcpyAsync(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st));
    CRG_CHECK_CUDA(cudaStreamSynchronize(st));
  }
  return p;
}

}  // namespace

void free_tiles(DevTiles& t) {
  cudaFree(t.rows); cudaFree(t.lptr); cudaFree(t.lcol); cudaFree(t.lchk);
  cudaFree(t.lw_val); cudaFree(t.lw_wn); cudaFree(t.lw_adj);
  cudaFree(t.desc); cudaFree(t.ucol); cudaFree(t.uchunk); cudaFree(t.direct);
  t = DevTiles{};
}

void build_tiles(DevCsr& c, const int32_t* row_order, cudaStream_t st) {
  DevTiles& T = c.tiles;
  const int64_t n = c.nrows, nnz = c.nnz;
  T.rows = keep_alloc<int32_t>((size_t)n, st);
  T.lptr = keep_alloc<int32_t>((size_t)n + 1, st);
  T.lcol = keep_alloc<uint16_t>((size_t)nnz + 2, st);  // +2: read as 32-bit words
  T.lchk = keep_alloc<uint16_t>((size_t)nnz + 2, st);
  T.lw_val = keep_alloc<float>((size_t)nnz, st);
  T.lw_wn = keep_alloc<float>((size_t)nnz, st);
  T.lw_adj = keep_alloc<float>((size_t)nnz, st);
  struct Good { int32_t p0, p1, u, nc; };
  std::vector<Good> good;
  std::vector<int32_t> direct;
  std::vector<int32_t> hlptr((size_t)n + 1, 0);
  if (n > 0) {
    CRG_CHECK_CUDA(cudaMemcpyAsync(T.rows, row_order, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, st));
    k_len_perm<<<nblk(n, 256), 256, 0, st>>>(c.ptr, T.rows, n, T.lptr);
    CRG_CHECK_CUDA(cudaGetLastError());
    exclusive_scan_i32(T.lptr, T.lptr, n, st);
    CRG_CHECK_CUDA(cudaMemcpyAsync(hlptr.data(), T.lptr, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToHost, st));
    // refinement: tiles of kTileRows, then quarters, down to single rows
    std::vector<int32_t> cand((size_t)((n + kTileRows - 1) / kTileRows));
    for (size_t i = 0; i < cand.size(); ++i) cand[i] = (int32_t)i;
    int32_t *dcand = nullptr, *du = nullptr, *dc = nullptr;
    size_t cap = 0;
    for (int TR = kTileRows; TR >= 1 && !cand.empty(); TR /= 4) {
      if (cand.size() > cap) {
        if (dcand) { cudaFreeAsync(dcand, st); cudaFreeAsync(du, st); cudaFreeAsync(dc, st); }
        cap = cand.size();
        CRG_CHECK_CUDA(cudaMallocAsync((void**)&dcand, sizeof(int32_t) * cap, st));
        CRG_CHECK_CUDA(cudaMallocAsync((void**)&du, sizeof(int32_t) * cap, st));
        CRG_CHECK_CUDA(cudaMallocAsync((void**)&dc, sizeof(int32_t) * cap, st));
      }
      CRG_CHECK_CUDA(cudaMemcpyAsync(dcand, cand.data(), sizeof(int32_t) * cand.size(), cudaMemcpyHostToDevice, st));
      k_tile_count<<<(unsigned)cand.size(), kThreads, 0, st>>>(c.ptr, c.idx, T.rows, n, dcand, TR, du, dc);
      CRG_CHECK_CUDA(cudaGetLastError());
      std::vector<int32_t> u(cand.size()), nc(cand.size());
      CRG_CHECK_CUDA(cudaMemcpyAsync(u.data(), du, sizeof(int32_t) * u.size(), cudaMemcpyDeviceToHost, st));
      CRG_CHECK_CUDA(cudaMemcpyAsync(nc.data(), dc, sizeof(int32_t) * nc.size(), cudaMemcpyDeviceToHost, st));
      CRG_CHECK_CUDA(cudaStreamSynchronize(st));
      std::vector<int32_t> next;
      const int sub = TR / 4;
      for (size_t i = 0; i < cand.size(); ++i) {
        const int64_t p0 = (int64_t)cand[i] * TR, p1 = std::min<int64_t>(n, p0 + TR);
        if (u[i] >= 0) {
          good.push_back(Good{(int32_t)p0, (int32_t)p1, u[i], nc[i]});
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
    if (dcand) { cudaFreeAsync(dcand, st); cudaFreeAsync(du, st); cudaFreeAsync(dc, st); }
  } else {
    CRG_CHECK_CUDA(cudaMemsetAsync(T.lptr, 0, sizeof(int32_t), st));
  }
  // descriptors in row order, so neighbouring work shares source columns in L2
  std::sort(good.begin(), good.end(), [](const Good& a, const Good& b) { return a.p0 < b.p0; });
  std::vector<int32_t> desc(good.size() * kDescInts);
  int64_t uacc = 0, cacc = 0;
  for (size_t i = 0; i < good.size(); ++i) {
    int32_t* d = &desc[i * kDescInts];
    d[kDescP0] = good[i].p0;
    d[kDescNr] = good[i].p1 - good[i].p0;
    d[kDescU0] = (int32_t)uacc;
    d[kDescNu] = good[i].u;
    d[kDescE0] = hlptr[good[i].p0];
    d[kDescNe] = hlptr[good[i].p1] - hlptr[good[i].p0];
    d[kDescC0] = (int32_t)cacc;
    d[kDescNc] = good[i].nc;
    uacc += good[i].u;
    cacc += good[i].nc;
  }
  std::sort(direct.begin(), direct.end());
  T.ngood = (int64_t)good.size();
  T.ndirect = (int64_t)direct.size();
  T.nucol = uacc;
  T.nuchunk = cacc;
  T.desc = upload(desc, st);
  T.direct = upload(direct, st);
  T.ucol = keep_alloc<int32_t>((size_t)uacc, st);
  T.uchunk = keep_alloc<int32_t>((size_t)cacc, st);
  if (T.ngood) {
    k_tile_fill<<<(unsigned)T.ngood, kThreads, 0, st>>>(c.ptr, c.idx, c.val32, c.wn32, c.adj32, T.rows, T.desc,
                                                        T.lptr, T.ucol, T.uchunk, T.lcol, T.lchk, T.lw_val, T.lw_wn,
                                                        T.lw_adj);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
}

}  // namespace crg

// ---------------------------------------------------------------------------
// Merge-path layout: the entries of a direction are cut into tasks of
// kTaskNnz consecutive entries (CSR order).  Rows whose entries straddle a task
// boundary are listed with the first and last task they touch, so the apply
// can combine their per-task partial sums in task order afterwards.

namespace crg {

namespace {

__global__ void k_expand_rows(const int32_t* __restrict__ ptr, int64_t n, int32_t* __restrict__ erow,
                              int* __restrict__ nempty) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int32_t a = ptr[r], b = ptr[r + 1];
  for (int32_t k = a; k < b; ++k) erow[k] = (int32_t)r;
  if (a == b) atomicAdd(nempty, 1);
}

// Start of task k: entry k * task_nnz moved up to the next row start, unless
// it falls inside a row longer than long_row (that row is then cut and its
// pieces summed by k_cm_fixup).  bound[ntasks] = nnz.
__global__ void k_task_bounds(const int32_t* __restrict__ ptr, const int32_t* __restrict__ erow, int64_t nnz,
                              int64_t ntasks, int task_nnz, int long_row, int32_t* __restrict__ bound) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k > ntasks) return;
  if (k == ntasks) {
    bound[k] = (int32_t)nnz;
    return;
  }
  const int64_t e = k * task_nnz;
  const int32_t r = erow[e], a = ptr[r], b = ptr[r + 1];
  bound[k] = (a == e || b - a > long_row) ? (int32_t)e : b;
}

// last task whose start is <= e
__device__ int64_t task_of_entry(const int32_t* __restrict__ bound, int64_t ntasks, int64_t e) {
  int64_t lo = 0, hi = ntasks - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (bound[mid] <= e) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Task records, and a flag on every task that ends a row begun in an earlier task.
__global__ void k_task_records(const int32_t* __restrict__ ptr, const int32_t* __restrict__ erow,
                               const int32_t* __restrict__ bound, int64_t ntasks, int4* __restrict__ tasks,
                               int32_t* __restrict__ ends) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntasks) return;
  const int32_t e0 = bound[t], e1 = bound[t + 1];
  if (e0 >= e1) {  // only the last task can be empty
    tasks[t] = make_int4(e0, e0, 0, 0);
    ends[t] = 0;
    return;
  }
  const int32_t first = erow[e0], last = erow[e1 - 1];
  const uint32_t fs = ptr[first] < e0 ? 1u : 0u, ls = ptr[last + 1] > e1 ? 1u : 0u;
  tasks[t] = make_int4(e0, e1, (int32_t)((uint32_t)first | (fs << 31)), (int32_t)((uint32_t)last | (ls << 31)));
  ends[t] = (fs && !(first == last && ls)) ? 1 : 0;
}

// Cut row number pos[t] ends in task t: its row, first task and number of
// pieces (one carry slot per piece).
__global__ void k_split_fill(const int32_t* __restrict__ ptr, const int32_t* __restrict__ bound, int64_t ntasks,
                             const int4* __restrict__ tasks, const int32_t* __restrict__ pos,
                             int32_t* __restrict__ split, int32_t* __restrict__ span) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntasks || pos[t + 1] == pos[t]) return;
  const int32_t row = tasks[t].z & 0x7fffffff;
  const int64_t t0 = task_of_entry(bound, ntasks, ptr[row]);
  int32_t* s = split + 3 * (int64_t)pos[t];
  s[0] = row;
  s[1] = (int32_t)t0;  // replaced by the first slot in k_slot_fill
  s[2] = (int32_t)(t - t0 + 1);
  span[pos[t]] = (int32_t)(t - t0 + 1);
}

// Slots of cut row s are base[s] .. base[s] + pieces - 1 in task order: the
// row's first task writes its last-row slot, the later tasks their first-row slot.
__global__ void k_slot_fill(int32_t* __restrict__ split, int64_t nsplit, const int32_t* __restrict__ base,
                            int2* __restrict__ tslot) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsplit) return;
  const int32_t t0 = split[3 * s + 1], pieces = split[3 * s + 2], b = base[s];
  tslot[t0].y = b;
  for (int32_t k = 1; k < pieces; ++k) tslot[t0 + k].x = b + k;
  split[3 * s + 1] = b;
}

}  // namespace

void build_merge_path(DevCsr& c, cudaStream_t st) {
  const int64_t n = c.nrows, nnz = c.nnz;
  c.erow = keep_alloc<int32_t>((size_t)nnz, st);
  // CRG_TASK_NNZ (32..1024) sets the nominal task length for tuning; CRG_TASK_CUT=fixed
  // cuts every task at exactly that length (rows spanning tasks everywhere)
  static const int task_nnz = [] {
    const char* e = getenv("CRG_TASK_NNZ");
    const int v = e ? atoi(e) : kTaskNnz;
    return (v >= 32 && v <= 1024) ? v : kTaskNnz;
  }();
  static const int long_row = [] {
    const char* e = getenv("CRG_TASK_CUT");
    return (e && strcmp(e, "fixed") == 0) ? -1 : task_nnz / 4;
  }();
  c.ntasks = (nnz + task_nnz - 1) / task_nnz;
  c.tasks = keep_alloc<int4>((size_t)c.ntasks, st);
  c.tslot = keep_alloc<int2>((size_t)c.ntasks, st);
  c.nsplit = 0;
  c.nslots = 0;
  c.nempty = n;
  if (n == 0 || nnz == 0) return;
  int32_t* work = nullptr;  // [1] empty rows | [ntasks + 1] bounds | [ntasks + 1] split positions
  CRG_CHECK_CUDA(cudaMallocAsync((void**)&work, sizeof(int32_t) * (2 * c.ntasks + 3), st));
  int32_t* nempty = work;
  int32_t* bound = work + 1;
  int32_t* pos = bound + c.ntasks + 1;
  CRG_CHECK_CUDA(cudaMemsetAsync(nempty, 0, sizeof(int32_t), st));
  k_expand_rows<<<nblk(n, 256), 256, 0, st>>>(c.ptr, n, c.erow, nempty);
  CRG_CHECK_CUDA(cudaGetLastError());
  k_task_bounds<<<nblk(c.ntasks + 1, 256), 256, 0, st>>>(c.ptr, c.erow, nnz, c.ntasks, task_nnz, long_row, bound);
  CRG_CHECK_CUDA(cudaGetLastError());
  k_task_records<<<nblk(c.ntasks, 256), 256, 0, st>>>(c.ptr, c.erow, bound, c.ntasks, c.tasks, pos);
  CRG_CHECK_CUDA(cudaGetLastError());
  exclusive_scan_i32(pos, pos, c.ntasks, st);
  int32_t counts[2] = {0, 0};
  CRG_CHECK_CUDA(cudaMemcpyAsync(&counts[0], pos + c.ntasks, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  CRG_CHECK_CUDA(cudaMemcpyAsync(&counts[1], nempty, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  CRG_CHECK_CUDA(cudaStreamSynchronize(st));
  c.nsplit = counts[0];
  c.nempty = counts[1];
  CRG_CHECK_CUDA(cudaMemsetAsync(c.tslot, 0xff, sizeof(int2) * c.ntasks, st));  // -1: row not cut
  c.split = keep_alloc<int32_t>((size_t)3 * c.nsplit, st);
  if (c.nsplit) {
    int32_t* span = nullptr;  // [nsplit + 1] pieces per cut row, scanned to first slots
    CRG_CHECK_CUDA(cudaMallocAsync((void**)&span, sizeof(int32_t) * (c.nsplit + 1), st));
    k_split_fill<<<nblk(c.ntasks, 256), 256, 0, st>>>(c.ptr, bound, c.ntasks, c.tasks, pos, c.split, span);
    CRG_CHECK_CUDA(cudaGetLastError());
    exclusive_scan_i32(span, span, c.nsplit, st);
    k_slot_fill<<<nblk(c.nsplit, 256), 256, 0, st>>>(c.split, c.nsplit, span, c.tslot);
    CRG_CHECK_CUDA(cudaGetLastError());
    int32_t nslots = 0;
    CRG_CHECK_CUDA(cudaMemcpyAsync(&nslots, span + c.nsplit, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CRG_CHECK_CUDA(cudaFreeAsync(span, st));
    CRG_CHECK_CUDA(cudaStreamSynchronize(st));
    c.nslots = nslots;
  }
  CRG_CHECK_CUDA(cudaFreeAsync(work, st));
}

}  // namespace crg
