// crg_build.cu -- device build of the regridder.
//
// Replaces Regridder(dst, src; normalize) of ConservativeRegridding.jl
// (src/regridder/regridder.jl:105-163):
//   K1 per-cell geometry: vertex tables, bounding balls, exact cell areas
//      (areas: regridder.jl:165-178; caps: src/trees/grids.jl:245-287)
//   K2 spatial order (cube-face Morton key, counting sort) and an implicit
//      binary hierarchy of axis-aligned boxes over leaves of 8 cells
//   K3 level-synchronous dual traversal of the two hierarchies with
//      warp-aggregated compaction of node pairs, then leaf-cell pair tests
//      (replaces the multithreaded dual DFS of
//      src/utils/MultithreadedDualDepthFirstSearch.jl:12-65 and
//      src/regridder/intersection_areas.jl:48-65)
//   K4 FP64 clip + area of every candidate pair (intersection_areas.jl:4-32)
//   K5 counting-sort assembly into CSR (rows = dst) and CSR of A^T, sorted
//      inside rows -- the pattern of SparseArrays.sparse(i_dst, i_src, area)
//      (intersection_areas.jl:115-121) -- plus normalize! and the derived
//      FP32 weights used by the apply kernels.
#include <stdlib.h>
#include <stdarg.h>
#include <stdio.h>

#include <algorithm>
#include <vector>

#include "crg_div.cuh"
#include "crg_geom.cuh"
#include "crg_internal.cuh"
#include "crg_scan.cuh"

namespace crg {

namespace {

constexpr int kLeaf = 8;          // cells per hierarchy leaf
constexpr int kMaxBlocks = kMaxGridBlocks;
constexpr int kMaxLevels = 40;
constexpr int kSortShift = 10;    // bins of the counting sort = key >> kSortShift

// ------------------------------------------------------------------ buffers

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// ------------------------------------------------------------------ K1: cell tables

struct BlockInfo {
  int nblocks;
  int dim;
  int64_t cell_off[kMaxBlocks + 1];
  int64_t point_off[kMaxBlocks];
  int64_t nx[kMaxBlocks];
};

// The expand kernels write each cell's vertices in FP64 and, rounded to
// nearest, in FP32 (the screening tests read those, converting nothing per pair).
__device__ __forceinline__ void put_vertex(double* o, float4* o4, double x, double y, double z) {
  o[0] = x;
  o[1] = y;
  o[2] = z;
  *o4 = make_float4((float)x, (float)y, (float)z, 0.f);
}

__global__ void k_expand_curvi(const double* __restrict__ pts, BlockInfo bi, int64_t ncells, double* __restrict__ v,
                               float4* __restrict__ v4, int8_t* __restrict__ nv) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  int b = 0;
  while (b + 1 < bi.nblocks && c >= bi.cell_off[b + 1]) b++;
  int64_t loc = c - bi.cell_off[b];
  int64_t nx = bi.nx[b];
  int64_t i = loc % nx, j = loc / nx;
  int64_t p[4] = {i + j * (nx + 1), (i + 1) + j * (nx + 1), (i + 1) + (j + 1) * (nx + 1), i + (j + 1) * (nx + 1)};
  for (int k = 0; k < 4; ++k) {
    const double* q = pts + (bi.point_off[b] + p[k]) * bi.dim;
    put_vertex(v + (c * 4 + k) * 3, v4 + c * 4 + k, q[0], q[1], bi.dim == 3 ? q[2] : 0.0);
  }
  nv[c] = 4;
}

__global__ void k_expand_cells(const double* __restrict__ cv, const int32_t* __restrict__ cn, int maxv, int dim,
                               int64_t ncells, double* __restrict__ v, float4* __restrict__ v4,
                               int8_t* __restrict__ nv, int32_t* __restrict__ bad) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  int n = cn ? cn[c] : maxv;
  // 0 vertices: a ghost slot (no geometry, no area, never a candidate)
  if ((n != 0 && n < 3) || n > maxv) {
    atomicAdd(bad, 1);
    n = n < 3 ? 0 : maxv;
  }
  for (int k = 0; k < maxv; ++k) {
    const double* q = cv + (c * maxv + k) * dim;
    put_vertex(v + (c * maxv + k) * 3, v4 + c * maxv + k, q[0], q[1], dim == 3 ? q[2] : 0.0);
  }
  nv[c] = (int8_t)n;
}

__device__ __forceinline__ uint32_t spread_bits14(uint32_t x) {
  // interleave: bit k of x -> bit 2k
  x &= 0x3fffu;
  x = (x | (x << 8)) & 0x00ff00ffu;
  x = (x | (x << 4)) & 0x0f0f0f0fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

__device__ __forceinline__ uint32_t spread_bits16(uint32_t x) {
  x &= 0xffffu;
  x = (x | (x << 8)) & 0x00ff00ffu;
  x = (x | (x << 4)) & 0x0f0f0f0fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

__device__ __forceinline__ uint32_t q14(float u) {  // u in [-1, 1]
  float t = (u + 1.0f) * 8191.5f;
  t = t < 0.0f ? 0.0f : (t > 16383.0f ? 16383.0f : t);
  return (uint32_t)t;
}

// Cube-face Morton key of a direction: face (3 bits) | 2 x 14 bits.  Any
// deterministic key serves (it only orders the cells of the hierarchy), so it
// is computed in FP32.
__device__ __forceinline__ uint32_t sphere_key(float x, float y, float z) {
  float ax = fabsf(x), ay = fabsf(y), az = fabsf(z);
  uint32_t face;
  float u, v, m;
  if (ax >= ay && ax >= az) { face = x >= 0 ? 0 : 1; m = ax; u = y; v = z; }
  else if (ay >= az) { face = y >= 0 ? 2 : 3; m = ay; u = x; v = z; }
  else { face = z >= 0 ? 4 : 5; m = az; u = x; v = y; }
  if (!(m > 0.0f)) return 0;
  u /= m; v /= m;
  return (face << 28) | spread_bits14(q14(u)) | (spread_bits14(q14(v)) << 1);
}

// Per-cell exact area, bounding volume and (spherical) order key.
// Spherical bounds: a ball in R^3 around c = normalize(sum v) with chord
// radius rho = max |c - v_k|; the cell (great-circle edges) lies in the
// spherical cap that ball cuts out whenever rho < sqrt(2), and rho = 2 is used
// otherwise.  The ball is computed in FP32 from the FP32-rounded vertices q_k
// (GB300's FP64 rate is a small fraction of its FP32 rate; only the area needs
// FP64): c is stored as computed, |v_k - q_k| <= 2^-24, and the FP32 distance
// |c - q_k| is within 2^-21 of its value relative, so rho (1 + 4e-6) + 4e-6,
// rounded up, bounds every |c - v_k|.  Planar bounds: the box of the FP64
// vertices rounded outward.  The float tests on these bounds are therefore a
// superset of the exact ones.
template <bool kSph>
__global__ void k_cell_geom(const double* __restrict__ v, const float4* __restrict__ v4,
                            const int8_t* __restrict__ nv, int maxv, int64_t ncells,
                            double* __restrict__ area, float4* __restrict__ bound, uint32_t* __restrict__ key,
                            int8_t* __restrict__ ori) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  d3 p[CRG_MAXV];
  int n = nv[c];
  for (int k = 0; k < n; ++k) {
    const double* q = v + (c * maxv + k) * 3;
    p[k].x = q[0]; p[k].y = q[1]; p[k].z = q[2];
  }
  // the orientation every clip of this cell uses, computed once, and the area
  // (signed area times orientation: the same values as cell_area)
  double o = 1.0, a = 0.0;
  if (n >= 3) {
    if (kSph) {
      a = area_orient_sph(p, n, o);
    } else {
      a = area_pl_signed(p, n);
      o = a >= 0.0 ? 1.0 : -1.0;
    }
  }
  area[c] = a * o;
  ori[c] = (int8_t)(o > 0.0 ? 1 : -1);
  if (n == 0) {  // a ghost slot: a bound that overlaps nothing (negative radius / inverted box)
    bound[c] = kSph ? make_float4(0.f, 0.f, 1.f, -4.f) : make_float4(INFINITY, INFINITY, -INFINITY, -INFINITY);
    if (kSph) key[c] = sphere_key(0.f, 0.f, 1.f);
    return;
  }
  if (kSph) {
    const float4* q = v4 + c * maxv;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    for (int k = 0; k < n; ++k) { sx += q[k].x; sy += q[k].y; sz += q[k].z; }
    const float nr = sqrtf(sx * sx + sy * sy + sz * sz);
    float cx = 0.f, cy = 0.f, cz = 1.f;
    if (nr > 0.f) {
      const float inr = 1.0f / nr;
      cx = sx * inr; cy = sy * inr; cz = sz * inr;
    }
    float rho2 = 0.f;
    for (int k = 0; k < n; ++k) {
      const float dx = q[k].x - cx, dy = q[k].y - cy, dz = q[k].z - cz;
      rho2 = fmaxf(rho2, dx * dx + dy * dy + dz * dz);
    }
    float rho = sqrtf(rho2);
    if (!(rho < 1.4f) || !(nr > 0.f)) rho = 2.f;
    const float rf = __fadd_ru(__fmul_ru(rho, 1.000004f), 4e-6f);
    bound[c] = make_float4(cx, cy, cz, rf);
    key[c] = sphere_key(cx, cy, cz);
  } else {
    double x0 = p[0].x, x1 = p[0].x, y0 = p[0].y, y1 = p[0].y;
    for (int k = 1; k < n; ++k) {
      x0 = fmin(x0, p[k].x); x1 = fmax(x1, p[k].x);
      y0 = fmin(y0, p[k].y); y1 = fmax(y1, p[k].y);
    }
    bound[c] = make_float4(__double2float_rd(x0), __double2float_rd(y0), __double2float_ru(x1), __double2float_ru(y1));
  }
}

// Planar keys after the global box is known (computed on the host from a
// reduction): 2 x 16-bit Morton of the box centre.
__global__ void k_planar_keys(const float4* __restrict__ bound, int64_t ncells, float4 gbox, uint32_t* __restrict__ key) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  float4 b = bound[c];
  float cx = 0.5f * (b.x + b.z), cy = 0.5f * (b.y + b.w);
  float wx = gbox.z - gbox.x, wy = gbox.w - gbox.y;
  float ux = wx > 0 ? (cx - gbox.x) / wx : 0.f, uy = wy > 0 ? (cy - gbox.y) / wy : 0.f;
  ux = fminf(fmaxf(ux, 0.f), 1.f);
  uy = fminf(fmaxf(uy, 0.f), 1.f);
  uint32_t qx = (uint32_t)(ux * 65535.f), qy = (uint32_t)(uy * 65535.f);
  key[c] = spread_bits16(qx) | (spread_bits16(qy) << 1);
}

// Block-wise min/max of planar boxes -> per-block partials.
__global__ void k_box_partials(const float4* __restrict__ bound, int64_t ncells, float4* __restrict__ part) {
  __shared__ float4 sh[256];
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float4 b = c < ncells ? bound[c] : make_float4(INFINITY, INFINITY, -INFINITY, -INFINITY);
  sh[threadIdx.x] = b;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      float4 o = sh[threadIdx.x + s];
      float4 m = sh[threadIdx.x];
      m.x = fminf(m.x, o.x); m.y = fminf(m.y, o.y); m.z = fmaxf(m.z, o.z); m.w = fmaxf(m.w, o.w);
      sh[threadIdx.x] = m;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// ------------------------------------------------------------------ K2: order + hierarchy

__global__ void k_hist(const uint32_t* __restrict__ key, int64_t n, int shift, int32_t* __restrict__ cnt) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) atomicAdd(&cnt[key[c] >> shift], 1);
}

__global__ void k_bin_scatter(const uint32_t* __restrict__ key, int64_t n, int shift, const int32_t* __restrict__ off,
                              int32_t* __restrict__ fill, int32_t* __restrict__ perm) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  uint32_t b = key[c] >> shift;
  int32_t slot = off[b] + atomicAdd(&fill[b], 1);
  perm[slot] = (int32_t)c;
}

// Sort each bin by (key, cell index): bins are tiny, insertion sort per thread.
// Inside the bins of the counting sort, cells go in (key, index) order: the
// pair is packed as key << 32 | index and sorted in place.  Bins of up to
// kBinSmall cells: one thread, insertion sort on the contiguous words; larger
// bins are listed for k_bin_sort_large (bitonic, shared memory up to
// kBinLarge words, which covers any realistic grid; larger bins fail loudly).
constexpr int kBinSmall = 32;
constexpr int kBinLarge = 4096;

__global__ void k_bin_pack(const uint32_t* __restrict__ key, const int32_t* __restrict__ perm, int64_t n,
                           uint64_t* __restrict__ w) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) w[i] = ((uint64_t)key[perm[i]] << 32) | (uint32_t)perm[i];
}

__global__ void k_bin_sort(uint64_t* __restrict__ w, const int32_t* __restrict__ off, int64_t nbins,
                           int32_t* __restrict__ large, int32_t* __restrict__ nlarge) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbins) return;
  const int32_t lo = off[b], hi = off[b + 1];
  if (hi - lo > kBinSmall) {
    large[atomicAdd(nlarge, 1)] = (int32_t)b;
    return;
  }
  for (int32_t i = lo + 1; i < hi; ++i) {
    const uint64_t x = w[i];
    int32_t j = i - 1;
    while (j >= lo && w[j] > x) {
      w[j + 1] = w[j];
      --j;
    }
    w[j + 1] = x;
  }
}

__global__ void __launch_bounds__(256) k_bin_sort_large(uint64_t* __restrict__ w, const int32_t* __restrict__ off,
                                                        const int32_t* __restrict__ large,
                                                        unsigned long long* __restrict__ too_big) {
  __shared__ uint64_t sk[kBinLarge];
  const int32_t b = large[blockIdx.x];
  const int32_t lo = off[b], len = off[b + 1] - lo;
  if (len > kBinLarge) {  // block-uniform
    if (threadIdx.x == 0) atomicAdd(too_big, 1ull);
    return;
  }
  int n2 = 64;
  while (n2 < len) n2 <<= 1;
  for (int i = threadIdx.x; i < n2; i += blockDim.x) sk[i] = i < len ? w[lo + i] : ~0ull;
  __syncthreads();
  for (int sz = 2; sz <= n2; sz <<= 1)
    for (int j = sz >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n2; i += blockDim.x) {
        const int p = i ^ j;
        if (p > i) {
          const uint64_t a = sk[i], c = sk[p];
          if (((i & sz) == 0) ? a > c : a < c) {
            sk[i] = c;
            sk[p] = a;
          }
        }
      }
      __syncthreads();
    }
  for (int i = threadIdx.x; i < len; i += blockDim.x) w[lo + i] = sk[i];
}

__global__ void k_bin_unpack(const uint64_t* __restrict__ w, int64_t n, int32_t* __restrict__ perm) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) perm[i] = (int32_t)(uint32_t)(w[i] & 0xffffffffu);
}

// Leaf boxes (level 0) and the per-cell bounds in sorted order.
template <bool kSph>
__global__ void k_leaves(const float4* __restrict__ bound, const int32_t* __restrict__ perm, int64_t ncells,
                         int64_t nleaves, float4* __restrict__ lo, float4* __restrict__ hi,
                         float4* __restrict__ sbound) {
  int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nleaves) return;
  float4 a = make_float4(INFINITY, INFINITY, INFINITY, 0.f), b = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.f);
  int64_t e = min(ncells, (l + 1) * kLeaf);
  for (int64_t s = l * kLeaf; s < e; ++s) {
    float4 q = bound[perm[s]];
    sbound[s] = q;
    float x0, y0, z0, x1, y1, z1;
    if (kSph) {
      x0 = __fsub_rd(q.x, q.w); x1 = __fadd_ru(q.x, q.w);
      y0 = __fsub_rd(q.y, q.w); y1 = __fadd_ru(q.y, q.w);
      z0 = __fsub_rd(q.z, q.w); z1 = __fadd_ru(q.z, q.w);
    } else {
      x0 = q.x; y0 = q.y; x1 = q.z; y1 = q.w; z0 = 0.f; z1 = 0.f;
    }
    a.x = fminf(a.x, x0); a.y = fminf(a.y, y0); a.z = fminf(a.z, z0);
    b.x = fmaxf(b.x, x1); b.y = fmaxf(b.y, y1); b.z = fmaxf(b.z, z1);
  }
  lo[l] = a;
  hi[l] = b;
}

// Levels l0 + 1 .. l0 + nup (nup <= kUp) of the box hierarchy in one launch:
// node i of level l + 1 bounds nodes 2i and 2i + 1 of level l, so each block
// reduces its 2^kUp nodes of level l0 through shared memory, one level per
// step, and writes every level it forms (min / max are exact: the boxes are
// those of a launch per level).
constexpr int kUp = 9;  // 512 nodes of level l0 per block of 256 threads
struct LevelTable {
  int64_t off[kMaxLevels];
  int64_t cnt[kMaxLevels];
};

__global__ void __launch_bounds__(256)
    k_levels_up(float4* __restrict__ lo, float4* __restrict__ hi, LevelTable lt, int l0, int nup) {
  __shared__ float4 slo[1 << kUp], shi[1 << kUp];
  int64_t cb = (int64_t)blockIdx.x << kUp;  // this block's first node of the current level
  for (int k = threadIdx.x; k < (1 << kUp); k += blockDim.x)
    if (cb + k < lt.cnt[l0]) {
      slo[k] = lo[lt.off[l0] + cb + k];
      shi[k] = hi[lt.off[l0] + cb + k];
    }
  __syncthreads();
  int64_t nc = lt.cnt[l0];
  for (int u = 1; u <= nup; ++u) {
    const int l = l0 + u;
    const int pw = (1 << kUp) >> u;  // this block's parents at level l
    const int64_t pb = cb >> 1;
    const int k = threadIdx.x;
    const bool have = k < pw && pb + k < lt.cnt[l];  // then child 2k exists
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
    if (have) {
      a = slo[2 * k];
      b = shi[2 * k];
      if (cb + 2 * k + 1 < nc) {
        const float4 c = slo[2 * k + 1], d = shi[2 * k + 1];
        a.x = fminf(a.x, c.x); a.y = fminf(a.y, c.y); a.z = fminf(a.z, c.z);
        b.x = fmaxf(b.x, d.x); b.y = fmaxf(b.y, d.y); b.z = fmaxf(b.z, d.z);
      }
    }
    __syncthreads();
    if (have) {
      slo[k] = a;
      shi[k] = b;
      lo[lt.off[l] + pb + k] = a;
      hi[lt.off[l] + pb + k] = b;
    }
    __syncthreads();
    nc = lt.cnt[l];
    cb = pb;
  }
}

struct Tree {
  int nlev = 0;                 // number of levels, leaves are level 0, root is nlev-1
  int64_t off[kMaxLevels] = {}; // node offset of each level in lo/hi
  int64_t cnt[kMaxLevels] = {}; // nodes per level
  int64_t ncells = 0;
  const float4* lo = nullptr;
  const float4* hi = nullptr;
  const float4* sbound = nullptr;  // per-cell bounds in sorted order
  const int32_t* perm = nullptr;   // sorted position -> cell index
};

// ------------------------------------------------------------------ K3: dual traversal

__device__ __forceinline__ uint32_t pack_node(int lev, int64_t idx) { return ((uint32_t)lev << 27) | (uint32_t)idx; }
__device__ __forceinline__ int node_lev(uint32_t p) { return (int)(p >> 27); }
__device__ __forceinline__ int64_t node_idx(uint32_t p) { return (int64_t)(p & 0x07ffffffu); }

__device__ __forceinline__ bool box_overlap(float4 alo, float4 ahi, float4 blo, float4 bhi) {
  return alo.x <= bhi.x && blo.x <= ahi.x && alo.y <= bhi.y && blo.y <= ahi.y && alo.z <= bhi.z && blo.z <= ahi.z;
}

struct TreeView {
  int64_t off[kMaxLevels];
  int64_t cnt[kMaxLevels];
  const float4* lo;
  const float4* hi;
};

// Warp-aggregated append of `k` items (k per lane may differ); returns the
// first output slot of this lane.
__device__ __forceinline__ int64_t warp_append(int k, unsigned long long* counter) {
  const int lane = threadIdx.x & 31;
  int incl = k;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  int total = __shfl_sync(0xffffffffu, incl, 31);
  unsigned long long base = 0;
  if (lane == 31 && total > 0) base = atomicAdd(counter, (unsigned long long)total);
  base = __shfl_sync(0xffffffffu, base, 31);
  return (int64_t)base + incl - k;
}

// One level of the dual traversal.  Each frontier pair (dst node, src node)
// expands the non-leaf side(s); child pairs whose boxes overlap go to the next
// frontier, or to the leaf-pair list when both children are leaves.
// One level of the dual traversal.  nin < 0: the frontier size is *nin_dev
// (written by the previous level on the device).  Appends past the capacities
// are dropped and raise *overflow (the host then runs the level loop).
__global__ void k_traverse(const uint2* __restrict__ in, int64_t nin, const unsigned long long* __restrict__ nin_dev,
                           TreeView td, TreeView ts, uint2* __restrict__ next, unsigned long long* __restrict__ nnext,
                           int64_t cap_next, uint2* __restrict__ leaves, unsigned long long* __restrict__ nleaves,
                           int64_t cap_leaves, int* __restrict__ overflow) {
  if (nin < 0) {
    // levels launched back to back (input count on the device): after a level
    // overflowed, its output is incomplete, so the later levels do nothing
    // (the host then restarts with the per-level loop); otherwise the count is
    // within the input buffer, which has the capacity of the output one
    // (one value per warp: the flag may be set while this level runs)
    if (__shfl_sync(0xffffffffu, *(volatile int*)overflow, 0)) return;
    nin = (int64_t)*nin_dev;
    if (nin > cap_next) nin = cap_next;
  }
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t nloop = (nin + 31) / 32 * 32;
  for (int64_t it = tid; it < ((nloop + stride - 1) / stride) * stride; it += stride) {
    uint2 outs[4];
    int nout = 0;
    if (it < nin) {
      uint2 pr = in[it];
      int la = node_lev(pr.x), lb = node_lev(pr.y);
      int64_t ia = node_idx(pr.x), ib = node_idx(pr.y);
      uint32_t ca[2], cb[2];
      int na = 0, nb = 0;
      if (la > 0) {
        ca[na++] = pack_node(la - 1, 2 * ia);
        if (2 * ia + 1 < td.cnt[la - 1]) ca[na++] = pack_node(la - 1, 2 * ia + 1);
      } else {
        ca[na++] = pr.x;
      }
      if (lb > 0) {
        cb[nb++] = pack_node(lb - 1, 2 * ib);
        if (2 * ib + 1 < ts.cnt[lb - 1]) cb[nb++] = pack_node(lb - 1, 2 * ib + 1);
      } else {
        cb[nb++] = pr.y;
      }
      for (int a = 0; a < na; ++a) {
        int64_t ga = td.off[node_lev(ca[a])] + node_idx(ca[a]);
        float4 alo = td.lo[ga], ahi = td.hi[ga];
        for (int b = 0; b < nb; ++b) {
          int64_t gb = ts.off[node_lev(cb[b])] + node_idx(cb[b]);
          if (box_overlap(alo, ahi, ts.lo[gb], ts.hi[gb])) outs[nout++] = make_uint2(ca[a], cb[b]);
        }
      }
    }
    // split into leaf pairs and internal pairs
    int nl = 0, ni = 0;
    for (int k = 0; k < nout; ++k) {
      if (node_lev(outs[k].x) == 0 && node_lev(outs[k].y) == 0) nl++;
      else ni++;
    }
    int64_t pi = warp_append(ni, nnext);
    int64_t pl = warp_append(nl, nleaves);
    if (pi + ni > cap_next || pl + nl > cap_leaves) {
      if (nout) atomicExch(overflow, 1);
      continue;
    }
    for (int k = 0; k < nout; ++k) {
      if (node_lev(outs[k].x) == 0 && node_lev(outs[k].y) == 0) leaves[pl++] = outs[k];
      else next[pi++] = outs[k];
    }
  }
}

template <bool kSph>
__device__ __forceinline__ bool cell_test(float4 a, float4 b) {
  if (kSph) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    float r = a.w + b.w;
    return r >= 0.f && d2 <= r * r * 1.000002f;  // a ghost slot's negative radius meets nothing
  }
  return a.x <= b.z && b.x <= a.z && a.y <= b.w && b.y <= a.w;
}

// Leaf pair -> number of cell pairs whose bounds intersect.
template <bool kSph>
__global__ void k_leaf_count(const uint2* __restrict__ lp, int64_t nlp, const float4* __restrict__ dsb, int64_t nd,
                             const float4* __restrict__ ssb, int64_t ns, int32_t* __restrict__ cnt) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nlp) return;
  uint2 p = lp[t];
  int64_t d0 = node_idx(p.x) * kLeaf, s0 = node_idx(p.y) * kLeaf;
  int64_t d1 = min(nd, d0 + kLeaf), s1 = min(ns, s0 + kLeaf);
  float4 db[kLeaf];
  int ndc = (int)(d1 - d0);
  for (int k = 0; k < ndc; ++k) db[k] = dsb[d0 + k];
  int c = 0;
  for (int64_t s = s0; s < s1; ++s) {
    float4 sb = ssb[s];
    for (int k = 0; k < ndc; ++k) c += cell_test<kSph>(db[k], sb) ? 1 : 0;
  }
  cnt[t] = c;
}

template <bool kSph>
__global__ void k_leaf_emit(const uint2* __restrict__ lp, int64_t nlp, const float4* __restrict__ dsb,
                            const int32_t* __restrict__ dperm, int64_t nd, const float4* __restrict__ ssb,
                            const int32_t* __restrict__ sperm, int64_t ns, const int32_t* __restrict__ off,
                            int2* __restrict__ cand) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nlp) return;
  uint2 p = lp[t];
  int64_t d0 = node_idx(p.x) * kLeaf, s0 = node_idx(p.y) * kLeaf;
  int64_t d1 = min(nd, d0 + kLeaf), s1 = min(ns, s0 + kLeaf);
  float4 db[kLeaf];
  int ndc = (int)(d1 - d0);
  for (int k = 0; k < ndc; ++k) db[k] = dsb[d0 + k];
  int32_t o = off[t];
  for (int64_t s = s0; s < s1; ++s) {
    float4 sb = ssb[s];
    int32_t sc = sperm[s];
    for (int k = 0; k < ndc; ++k)
      if (cell_test<kSph>(db[k], sb)) cand[o++] = make_int2(dperm[d0 + k], sc);
  }
}

// ------------------------------------------------------------------ K4: clip + area

// Every destination edge's half-space, once per cell (the clip of each pair reads it).
// Separation filter of the candidate pairs (spherical).  A pair whose source
// cell lies strictly outside one destination edge half-space has no overlap:
// the FP64 clip would empty the polygon at that edge, so the pair is dropped
// before it.  Decided in FP32: with n32 the plane normal rounded from FP64 and
// w32 = v32 - ca32 from rounded unit vectors, |s32 - n.(v - ca)| stays below
// 2^-21 |n32|_1 (1 + |w32|_inf) (inputs 2^-24 relative, the dot product 3
// roundings, the FP64 normal's own error far smaller), so s32 < -B with
// B = 2^-18 |n32|_1 (1 + |w32|_1) is outside by an 8x margin.
//
// The same tests give each kept pair its class: the mask of destination edges
// that may cut the source cell (neither all vertices clearly inside nor all
// outside), and the vertex count of the clipped polygon as FP32 side tests
// predict it (only a grouping key: the FP64 clip decides).  Clipping the
// pairs grouped by class lets the lanes of a warp meet their crossing points
// at the same stages and run the area's fan over the same number of
// triangles.
constexpr int kMaskClasses = 256;  // cut masks of up to 8 edges
constexpr int kSizeClasses = 16;   // predicted vertex counts 0 .. 15 (15: 15 or more)
constexpr int kClasses = kMaskClasses * kSizeClasses;  // class kClasses = dropped

__global__ void __launch_bounds__(256)
    k_separated(const int2* __restrict__ cand, int64_t nc, const float4* __restrict__ dv4,
                const int8_t* __restrict__ dnv, int dmaxv, const float4* __restrict__ sv4,
                const int8_t* __restrict__ snv, const int8_t* __restrict__ sori, int smaxv,
                const float4* __restrict__ planes32, uint16_t* __restrict__ cls) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc) return;
  const int2 pr = cand[t];
  const int nd = dnv[pr.x], ns = snv[pr.y];
  if (nd < 3 || ns < 3) {  // no polygon: never an entry
    cls[t] = kClasses;
    return;
  }
  float4 v[CRG_MAXV];
  const float4* q = sv4 + (int64_t)pr.y * smaxv;
  for (int i = 0; i < ns; ++i) v[i] = q[i];
  const float4* c = dv4 + (int64_t)pr.x * dmaxv;
  const float4* pl = planes32 + (int64_t)pr.x * dmaxv;
  int sep = 0, mask = 0;
  uint64_t sp = 0;  // bit 8 k + i: subject vertex i on the inner side of destination edge k (plain FP32 sign)
  for (int k = 0; k < nd && !sep; ++k) {
    const float4 p = pl[k], a = c[k];  // n32 (w = |n32|_1) and ca32
    int out = 1, in = 1;
    for (int i = 0; i < ns; ++i) {
      const float wx = v[i].x - a.x, wy = v[i].y - a.y, wz = v[i].z - a.z;
      const float s = fmaf(p.x, wx, fmaf(p.y, wy, p.z * wz));
      const float B = 3.814697265625e-06f * p.w * (1.0f + fabsf(wx) + fabsf(wy) + fabsf(wz));  // 2^-18
      out &= s < -B;
      in &= s > B;
      if (s >= 0.f) sp |= 1ull << (8 * k + i);
    }
    sep = out;
    if (!in) mask |= 1 << k;
  }
  if (sep) {
    cls[t] = kClasses;
    return;
  }
  // The vertex count of the intersection of two convex polygons (general
  // position): the subject's vertices inside the destination cell, the
  // destination's vertices inside the subject, and one per pair of edges that
  // cross (each edge's endpoints on either side of the other's great circle).
  uint64_t sq = 0;  // bit 8 j + k: destination vertex k on the inner side of subject edge j
  const float sg = (float)sori[pr.y];
  for (int j = 0; j < ns; ++j) {
    const float4 a = v[j], b = v[j + 1 == ns ? 0 : j + 1];
    const float ex = b.x - a.x, ey = b.y - a.y, ez = b.z - a.z;
    const float nx = sg * (a.y * ez - a.z * ey), ny = sg * (a.z * ex - a.x * ez), nz = sg * (a.x * ey - a.y * ex);
    for (int k = 0; k < nd; ++k) {
      const float4 d = c[k];
      const float s = fmaf(nx, d.x - a.x, fmaf(ny, d.y - a.y, nz * (d.z - a.z)));
      if (s >= 0.f) sq |= 1ull << (8 * j + k);
    }
  }
  uint32_t allp = (1u << ns) - 1u, allq = (1u << nd) - 1u;
  for (int k = 0; k < nd; ++k) allp &= (uint32_t)(sp >> (8 * k)) & 0xffu;
  for (int j = 0; j < ns; ++j) allq &= (uint32_t)(sq >> (8 * j)) & 0xffu;
  int m = __popc(allp) + __popc(allq);
  for (int j = 0; j < ns; ++j) {
    const int j1 = j + 1 == ns ? 0 : j + 1;
    const uint32_t rq = (uint32_t)(sq >> (8 * j)) & 0xffu;  // destination vertices vs subject edge j
    for (int k = 0; k < nd; ++k) {
      const int k1 = k + 1 == nd ? 0 : k + 1;
      const uint32_t rp = (uint32_t)(sp >> (8 * k)) & 0xffu;  // subject vertices vs destination edge k
      m += (((rp >> j) ^ (rp >> j1)) & ((rq >> k) ^ (rq >> k1)) & 1u) ? 1 : 0;
    }
  }
  cls[t] = (uint16_t)((mask & (kMaskClasses - 1)) | (min(m, kSizeClasses - 1) << 8));
}

__global__ void __launch_bounds__(256)
    k_class_count(const uint16_t* __restrict__ cls, int64_t nc, int32_t* __restrict__ cnt) {
  __shared__ int32_t h[kClasses + 1];
  for (int i = threadIdx.x; i <= kClasses; i += blockDim.x) h[i] = 0;
  __syncthreads();
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nc) atomicAdd(&h[cls[t]], 1);
  __syncthreads();
  for (int i = threadIdx.x; i < kClasses; i += blockDim.x)
    if (h[i]) atomicAdd(&cnt[i], h[i]);
}

// Kept pairs grouped by class: each block reserves its range of every class
// (any order inside a class: the clip results do not depend on it).
__global__ void __launch_bounds__(256)
    k_class_scatter(const int2* __restrict__ cand, const uint16_t* __restrict__ cls, int64_t nc,
                    const int32_t* __restrict__ off, int32_t* __restrict__ fill, int2* __restrict__ out) {
  __shared__ int32_t h[kClasses + 1], base[kClasses + 1];
  for (int i = threadIdx.x; i <= kClasses; i += blockDim.x) h[i] = 0;
  __syncthreads();
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int b = t < nc ? cls[t] : kClasses;
  const int r = b < kClasses ? atomicAdd(&h[b], 1) : 0;
  __syncthreads();
  for (int i = threadIdx.x; i < kClasses; i += blockDim.x) base[i] = h[i] ? atomicAdd(&fill[i], h[i]) : 0;
  __syncthreads();
  if (b < kClasses) out[off[b] + base[b] + r] = cand[t];
}

__global__ void k_edge_planes(const double* __restrict__ v, const int8_t* __restrict__ nv,
                              const int8_t* __restrict__ ori, int maxv, int64_t ncells, double4_32a* __restrict__ planes,
                              float4* __restrict__ planes32) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  const int n = nv[c];
  const double* q = v + c * maxv * 3;
  for (int k = 0; k < n; ++k) {
    const int k1 = k + 1 == n ? 0 : k + 1;
    d3 nrm;
    double eb;
    edge_plane(d3{q[3 * k], q[3 * k + 1], q[3 * k + 2]}, d3{q[3 * k1], q[3 * k1 + 1], q[3 * k1 + 2]}, (double)ori[c],
               nrm, eb);
    planes[c * maxv + k] = make_double4_32a(nrm.x, nrm.y, nrm.z, eb);
    const float nx = (float)nrm.x, ny = (float)nrm.y, nz = (float)nrm.z;
    planes32[c * maxv + k] = make_float4(nx, ny, nz, fabsf(nx) + fabsf(ny) + fabsf(nz));
  }
}

// 5 blocks of 128 per SM (96 registers, a few bytes spilled): 3.31 against
// 3.37 ms at the 128 registers the compiler takes unbounded (4 blocks).
template <bool kSph>
__global__ void __launch_bounds__(128, 5) k_clip(const int2* __restrict__ cand, int64_t nc, const double* __restrict__ dv,
                                              const int8_t* __restrict__ dnv, const int8_t* __restrict__ dori,
                                              int dmaxv, const double* __restrict__ sv,
                                              const int8_t* __restrict__ snv, const int8_t* __restrict__ sori,
                                              int smaxv, double* __restrict__ area,
                                              int32_t* __restrict__ rowcnt, int32_t* __restrict__ colcnt,
                                              unsigned long long* __restrict__ overflow,
                                              const double4_32a* __restrict__ dplanes,
                                              const float4* __restrict__ dplanes32, const float4* __restrict__ dv4,
                                              const float4* __restrict__ sv4) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc) return;
  int2 pr = cand[t];
  d3 clip[CRG_MAXV];
  d3 bufA[CRG_MAXC], bufB[CRG_MAXC];
  int nd = dnv[pr.x], ns = snv[pr.y];
  const double* q = dv + (int64_t)pr.x * dmaxv * 3;
  for (int k = 0; k < nd; ++k) { clip[k].x = q[3 * k]; clip[k].y = q[3 * k + 1]; clip[k].z = q[3 * k + 2]; }
  q = sv + (int64_t)pr.y * smaxv * 3;
  for (int k = 0; k < ns; ++k) { bufA[k].x = q[3 * k]; bufA[k].y = q[3 * k + 1]; bufA[k].z = q[3 * k + 2]; }
  const double sig = sori[pr.y];  // the subject's orientation (k_cell_geom)
  double a = 0.0;
  if (nd >= 3 && ns >= 3) {
    d3* res;
    float4 fa[kSph ? CRG_MAXC : 1], fb[kSph ? CRG_MAXC : 1];
    Screen32 s32{nullptr, nullptr, fa, fb};
    if (kSph) {
      s32.planes = dplanes32 + (int64_t)pr.x * dmaxv;
      s32.clip = dv4 + (int64_t)pr.x * dmaxv;
      const float4* q4 = sv4 + (int64_t)pr.y * smaxv;
      for (int k = 0; k < ns; ++k) fa[k] = q4[k];
    }
    int m = clip_polygon_oriented<kSph>(bufA, bufB, ns, clip, nd, (double)dori[pr.x], &res,
                                        kSph ? dplanes + (int64_t)pr.x * dmaxv : nullptr, kSph ? &s32 : nullptr);
    if (m < 0) {
      atomicAdd(overflow, 1ull);
    } else {
      a = (kSph ? area_sph_signed(res, m) : area_pl_signed(res, m)) * sig;
    }
  }
  area[t] = a;
  if (a > 0.0) {
    atomicAdd(&rowcnt[pr.x], 1);
    atomicAdd(&colcnt[pr.y], 1);
  }
}

// ------------------------------------------------------------------ K5: assembly

__global__ void k_scatter_pairs(const int2* __restrict__ cand, const double* __restrict__ area, int64_t nc,
                                const int32_t* __restrict__ rowptr, int32_t* __restrict__ rowfill,
                                const int32_t* __restrict__ colptr, int32_t* __restrict__ colfill,
                                int32_t* __restrict__ fidx, double* __restrict__ fval, int32_t* __restrict__ ridx,
                                double* __restrict__ rval) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc) return;
  double a = area[t];
  if (!(a > 0.0)) return;
  int2 pr = cand[t];
  int32_t p = rowptr[pr.x] + atomicAdd(&rowfill[pr.x], 1);
  fidx[p] = pr.y;
  fval[p] = a;
  int32_t q = colptr[pr.y] + atomicAdd(&colfill[pr.y], 1);
  ridx[q] = pr.x;
  rval[q] = a;
}

// Sorting each row segment by column (columns are distinct within a row, so
// any correct sort gives the same result).  Rows of up to 32 entries: one warp
// each, a bitonic network across the lanes.  Longer rows: one block each, a
// bitonic network over the row padded to a power of two, in shared memory up
// to kRowSortSmem entries and in a global scratch beyond.
constexpr int kRowSortSmem = 4096;
constexpr int kRowSortThreads = 256;

// Rows of up to 8 entries: one thread each, an odd-even transposition network
// of 8 elements in registers (missing entries are +inf keys).
__global__ void k_row_sort_small(const int32_t* __restrict__ ptr, int64_t nrows, int32_t* __restrict__ idx,
                                 double* __restrict__ val) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int32_t lo = ptr[r], len = ptr[r + 1] - lo;
  if (len < 2 || len > 8) return;
  int32_t k[8];
  double v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    k[i] = i < len ? idx[lo + i] : INT32_MAX;
    v[i] = i < len ? val[lo + i] : 0.0;
  }
#pragma unroll
  for (int round = 0; round < 8; ++round)
#pragma unroll
    for (int i = round & 1; i + 1 < 8; i += 2)
      if (k[i + 1] < k[i]) {
        const int32_t tk = k[i]; k[i] = k[i + 1]; k[i + 1] = tk;
        const double tv = v[i]; v[i] = v[i + 1]; v[i + 1] = tv;
      }
#pragma unroll
  for (int i = 0; i < 8; ++i)
    if (i < len) {
      idx[lo + i] = k[i];
      val[lo + i] = v[i];
    }
}

// Rows of 9..32 entries (listed): one warp each, a bitonic network across the lanes.
__global__ void k_row_sort_warp(const int32_t* __restrict__ ptr, const int32_t* __restrict__ rows, int64_t nlist,
                                int32_t* __restrict__ idx, double* __restrict__ val) {
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= nlist) return;  // warp-uniform
  const int32_t r = rows[w];
  const int32_t lo = ptr[r], len = ptr[r + 1] - lo;
  int32_t key = lane < len ? idx[lo + lane] : INT32_MAX;
  double v = lane < len ? val[lo + lane] : 0.0;
  for (int k = 2; k <= 32; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      const int32_t pk = __shfl_xor_sync(0xffffffffu, key, j);
      const double pv = __shfl_xor_sync(0xffffffffu, v, j);
      const bool up = (lane & k) == 0, lower = (lane & j) == 0;
      if (lower == up ? pk < key : pk > key) {
        key = pk;
        v = pv;
      }
    }
  }
  if (lane < len) {
    idx[lo + lane] = key;
    val[lo + lane] = v;
  }
}

// rows longer than 8 entries: 9..32 (a warp each), up to shared-memory size
// (a block each) and longer (global memory)
__global__ void k_row_classes(const int32_t* __restrict__ ptr, int64_t nrows, int32_t* __restrict__ warp,
                              int32_t* __restrict__ mid, int32_t* __restrict__ longr, int32_t* __restrict__ counts) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int32_t len = ptr[r + 1] - ptr[r];
  if (len <= 8) return;
  if (len <= 32) warp[atomicAdd(&counts[2], 1)] = (int32_t)r;
  else if (len <= kRowSortSmem) mid[atomicAdd(&counts[0], 1)] = (int32_t)r;
  else longr[atomicAdd(&counts[1], 1)] = (int32_t)r;
}

// bitonic network over n2 (a power of two) keys/values in k[], v[] (shared or global)
__device__ void bitonic_block(int32_t* k, double* v, int n2) {
  for (int sz = 2; sz <= n2; sz <<= 1) {
    for (int j = sz >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n2; i += blockDim.x) {
        const int p = i ^ j;
        if (p > i) {
          const bool up = (i & sz) == 0;
          const int32_t a = k[i], b = k[p];
          if (up ? a > b : a < b) {
            k[i] = b;
            k[p] = a;
            const double t = v[i];
            v[i] = v[p];
            v[p] = t;
          }
        }
      }
      __syncthreads();
    }
  }
}

__global__ void __launch_bounds__(kRowSortThreads) k_row_sort_block(const int32_t* __restrict__ ptr,
                                                                    const int32_t* __restrict__ rows,
                                                                    int32_t* __restrict__ idx,
                                                                    double* __restrict__ val) {
  __shared__ int32_t sk[kRowSortSmem];
  __shared__ double sv[kRowSortSmem];
  const int32_t r = rows[blockIdx.x];
  const int32_t lo = ptr[r], len = ptr[r + 1] - lo;
  int n2 = 64;
  while (n2 < len) n2 <<= 1;
  for (int i = threadIdx.x; i < n2; i += blockDim.x) {
    sk[i] = i < len ? idx[lo + i] : INT32_MAX;
    sv[i] = i < len ? val[lo + i] : 0.0;
  }
  __syncthreads();
  bitonic_block(sk, sv, n2);
  for (int i = threadIdx.x; i < len; i += blockDim.x) {
    idx[lo + i] = sk[i];
    val[lo + i] = sv[i];
  }
}

// long rows: each block owns the scratch window [off[b], off[b] + n2) of k/v
__global__ void __launch_bounds__(1024) k_row_sort_long(const int32_t* __restrict__ ptr,
                                                        const int32_t* __restrict__ rows,
                                                        const int64_t* __restrict__ off, int32_t* __restrict__ idx,
                                                        double* __restrict__ val, int32_t* __restrict__ gk,
                                                        double* __restrict__ gv) {
  const int32_t r = rows[blockIdx.x];
  const int32_t lo = ptr[r], len = ptr[r + 1] - lo;
  int n2 = kRowSortSmem;
  while (n2 < len) n2 <<= 1;
  int32_t* k = gk + off[blockIdx.x];
  double* v = gv + off[blockIdx.x];
  for (int i = threadIdx.x; i < n2; i += blockDim.x) {
    k[i] = i < len ? idx[lo + i] : INT32_MAX;
    v[i] = i < len ? val[lo + i] : 0.0;
  }
  __syncthreads();
  bitonic_block(k, v, n2);
  for (int i = threadIdx.x; i < len; i += blockDim.x) {
    idx[lo + i] = k[i];
    val[lo + i] = v[i];
  }
}

__global__ void k_long_windows(const int32_t* __restrict__ ptr, const int32_t* __restrict__ rows, int64_t n,
                               int64_t* __restrict__ off) {
  // sequential prefix over the (few) long rows
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  int64_t o = 0;
  for (int64_t b = 0; b < n; ++b) {
    off[b] = o;
    const int32_t len = ptr[rows[b] + 1] - ptr[rows[b]];
    int64_t n2 = kRowSortSmem;
    while (n2 < len) n2 <<= 1;
    o += n2;
  }
  off[n] = o;
}

__global__ void k_max_val(const double* __restrict__ v, int64_t n, unsigned long long* __restrict__ mx) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double m = 0.0;  // maximum(A) of a SparseMatrixCSC includes its implicit zeros; values are > 0 here
  for (; i < n; i += (int64_t)gridDim.x * blockDim.x) m = fmax(m, v[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(mx, (unsigned long long)__double_as_longlong(m));
}

// normalize!: both CSR copies of A and both area vectors divided by max(A),
// one launch over the four arrays back to back.
// Each thread takes kDivPer elements (grid-stride) and the IEEE reciprocal of
// max(A) once: the quotients come from Markstein's correction, checked, with
// the IEEE division where the check fails (crg_div.cuh) -- the bits of v / m.
constexpr int kDivPer = 8;
__global__ void k_div_by(double* __restrict__ a, double* __restrict__ b, int64_t nnz, double* __restrict__ c,
                         int64_t nc, double* __restrict__ d, int64_t nd, const unsigned long long* __restrict__ mx) {
  const double m = __longlong_as_double((long long)*mx);
  const double rcp = 1.0 / m;
  const int64_t total = 2 * nnz + nc + nd;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < total; j += stride) {
    int64_t i = j;
    double* v;
    if (i < nnz) {
      v = a;
    } else if ((i -= nnz) < nnz) {
      v = b;
    } else if ((i -= nnz) < nc) {
      v = c;
    } else {
      i -= nc;
      v = d;
    }
    v[i] = div_rn_by(v[i], m, rcp);
  }
}

// FP32 copies of the entries and of the normalised / adjoint weights, one
// thread per entry (erow: the row of each entry): val32 = A, wn32 = A / area_row,
// adj32 = A / area_col, each formed in FP64 as A times the FP64 reciprocal of the
// area (one reciprocal per cell, k_recip: FP64 division is a long sequence on
// GB300's FP64 pipe) and rounded to FP32.  The product is within 2^-52 of the
// quotient, relative, so the weight is the rounded quotient except when that lies
// within 2^-52 of an FP32 rounding midpoint, and then one FP32 ulp from it.
__global__ void k_recip(const double* __restrict__ v, int64_t n, double* __restrict__ r) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) r[i] = 1.0 / v[i];
}

__global__ void k_derive(const int32_t* __restrict__ erow, const int32_t* __restrict__ idx,
                         const double* __restrict__ val, int64_t nnz, const double* __restrict__ inv_row,
                         const double* __restrict__ inv_col, float* __restrict__ val32, float* __restrict__ wn32,
                         float* __restrict__ adj32) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nnz) return;
  const double a = val[k];
  val32[k] = (float)a;
  wn32[k] = (float)(a * inv_row[erow[k]]);
  adj32[k] = (float)(a * inv_col[idx[k]]);
}

// Kahan-summed rows of A, entries in column order.
__global__ void k_row_sums(const int32_t* __restrict__ ptr, const double* __restrict__ val, int64_t nrows,
                           double* __restrict__ rowsum) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  double s = 0.0, comp = 0.0;
  for (int32_t k = ptr[r]; k < ptr[r + 1]; ++k) {
    const double y = val[k] - comp;
    const double t = s + y;
    comp = (t - s) - y;
    s = t;
  }
  rowsum[r] = s;
}

// ------------------------------------------------------------------ host helpers

struct DevGrid {
  CellTable tab;
  DBuf<double> v;
  DBuf<float4> v4;
  DBuf<int8_t> nv;
  DBuf<int8_t> ori;
  int64_t ncells = 0;
};

void upload_grid(const crg_grid_desc* g, DevGrid& out, cudaStream_t st) {
  CRG_REQUIRE(g != nullptr, CRG_ERR_INVALID_ARGUMENT, "grid descriptor is NULL");
  CRG_REQUIRE(g->manifold == CRG_PLANAR || g->manifold == CRG_SPHERICAL, CRG_ERR_INVALID_ARGUMENT,
              "unknown manifold %d", g->manifold);
  CRG_REQUIRE(g->ncells >= 0 && g->ncells < (int64_t)1 << 31, CRG_ERR_NOT_SUPPORTED,
              "ncells = %lld is outside [0, 2^31)", (long long)g->ncells);
  const int dim = g->manifold == CRG_SPHERICAL ? 3 : 2;
  out.ncells = g->ncells;
  if (g->kind == CRG_GRID_CURVILINEAR) {
    CRG_REQUIRE(g->nblocks >= 1 && g->nblocks <= kMaxBlocks, CRG_ERR_INVALID_ARGUMENT,
                "nblocks = %d must be in 1..%d", g->nblocks, kMaxBlocks);
    CRG_REQUIRE(g->block_nx && g->block_ny && g->points, CRG_ERR_INVALID_ARGUMENT, "curvilinear grid arrays are NULL");
    BlockInfo bi{};
    bi.nblocks = g->nblocks;
    bi.dim = dim;
    int64_t cells = 0, pts = 0;
    for (int b = 0; b < g->nblocks; ++b) {
      CRG_REQUIRE(g->block_nx[b] >= 1 && g->block_ny[b] >= 1, CRG_ERR_INVALID_ARGUMENT,
                  "block %d has %lld x %lld cells", b, (long long)g->block_nx[b], (long long)g->block_ny[b]);
      bi.cell_off[b] = cells;
      bi.point_off[b] = pts;
      bi.nx[b] = g->block_nx[b];
      cells += g->block_nx[b] * g->block_ny[b];
      pts += (g->block_nx[b] + 1) * (g->block_ny[b] + 1);
    }
    bi.cell_off[g->nblocks] = cells;
    CRG_REQUIRE(cells == g->ncells, CRG_ERR_DIMENSION_MISMATCH,
                "ncells = %lld but the blocks hold %lld cells", (long long)g->ncells, (long long)cells);
    const double* dpts = g->points;
    DBuf<double> staged;
    if (!is_device_pointer(g->points)) {
      staged.alloc((size_t)pts * dim, st);
      CRG_CHECK_CUDA(cudaMemcpyAsync(staged.p, g->points, sizeof(double) * pts * dim, cudaMemcpyHostToDevice, st));
      dpts = staged.p;
    }
    out.tab.n = cells;
    out.tab.maxv = 4;
    out.v.alloc((size_t)cells * 4 * 3, st);
    out.v4.alloc((size_t)cells * 4, st);
    out.nv.alloc((size_t)cells, st);
    if (cells) {
      k_expand_curvi<<<nblk(cells, 256), 256, 0, st>>>(dpts, bi, cells, out.v.p, out.v4.p, out.nv.p);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
  } else if (g->kind == CRG_GRID_CELLS) {
    CRG_REQUIRE(g->max_verts >= 3 && g->max_verts <= CRG_MAXV, CRG_ERR_INVALID_ARGUMENT,
                "max_verts = %d must be in 3..%d", g->max_verts, CRG_MAXV);
    CRG_REQUIRE(g->cell_verts || g->ncells == 0, CRG_ERR_INVALID_ARGUMENT, "cell_verts is NULL");
    const int64_t n = g->ncells, mv = g->max_verts;
    const double* dcv = g->cell_verts;
    const int32_t* dcn = g->cell_nverts;
    DBuf<double> s1;
    DBuf<int32_t> s2;
    if (n && !is_device_pointer(g->cell_verts)) {
      s1.alloc((size_t)n * mv * dim, st);
      CRG_CHECK_CUDA(cudaMemcpyAsync(s1.p, g->cell_verts, sizeof(double) * n * mv * dim, cudaMemcpyHostToDevice, st));
      dcv = s1.p;
    }
    if (n && dcn && !is_device_pointer(dcn)) {
      s2.alloc((size_t)n, st);
      CRG_CHECK_CUDA(cudaMemcpyAsync(s2.p, dcn, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
      dcn = s2.p;
    }
    out.tab.n = n;
    out.tab.maxv = (int)mv;
    out.v.alloc((size_t)n * mv * 3, st);
    out.v4.alloc((size_t)n * mv, st);
    out.nv.alloc((size_t)n, st);
    DBuf<int32_t> bad(1, st);
    bad.zero();
    if (n) {
      k_expand_cells<<<nblk(n, 256), 256, 0, st>>>(dcv, dcn, (int)mv, dim, n, out.v.p, out.v4.p, out.nv.p, bad.p);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
    int32_t hbad = 0;
    CRG_CHECK_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CRG_CHECK_CUDA(cudaStreamSynchronize(st));
    CRG_REQUIRE(hbad == 0, CRG_ERR_INVALID_ARGUMENT, "%d cells have a vertex count outside 3..max_verts (or 0)",
                hbad);
  } else {
    CRG_REQUIRE(false, CRG_ERR_INVALID_ARGUMENT, "unknown grid kind %d", g->kind);
  }
  out.tab.v = out.v.p;
  out.tab.v4 = out.v4.p;
  out.tab.nv = out.nv.p;
  out.ori.alloc((size_t)out.tab.n, st);  // filled with the cell geometry
  out.tab.ori = out.ori.p;
}

struct HostTree {
  Tree t;
  DBuf<float4> bound, sbound, lo, hi;
  DBuf<uint32_t> key;
  DBuf<int32_t> perm;
};

// K1 + K2 for one grid.  `area_out` receives the exact cell areas.
void build_tree(const DevGrid& g, bool sph, double* area_out, HostTree& h, cudaStream_t st) {
  const int64_t n = g.ncells;
  h.t.ncells = n;
  h.bound.alloc((size_t)n, st);
  h.key.alloc((size_t)n, st);
  if (n == 0) return;
  if (sph) {
    k_cell_geom<true><<<nblk(n, 128), 128, 0, st>>>(g.tab.v, g.tab.v4, g.tab.nv, g.tab.maxv, n, area_out, h.bound.p,
                                                     h.key.p, g.tab.ori);
    CRG_CHECK_CUDA(cudaGetLastError());
  } else {
    k_cell_geom<false><<<nblk(n, 128), 128, 0, st>>>(g.tab.v, g.tab.v4, g.tab.nv, g.tab.maxv, n, area_out,
                                                      h.bound.p, h.key.p, g.tab.ori);
    CRG_CHECK_CUDA(cudaGetLastError());
    int64_t nb = nblk(n, 256);
    DBuf<float4> part((size_t)nb, st);
    k_box_partials<<<(unsigned)nb, 256, 0, st>>>(h.bound.p, n, part.p);
    CRG_CHECK_CUDA(cudaGetLastError());
    std::vector<float4> hp((size_t)nb);
    CRG_CHECK_CUDA(cudaMemcpyAsync(hp.data(), part.p, sizeof(float4) * nb, cudaMemcpyDeviceToHost, st));
    CRG_CHECK_CUDA(cudaStreamSynchronize(st));
    float4 gb = make_float4(INFINITY, INFINITY, -INFINITY, -INFINITY);
    for (auto& b : hp) {
      gb.x = std::min(gb.x, b.x); gb.y = std::min(gb.y, b.y);
      gb.z = std::max(gb.z, b.z); gb.w = std::max(gb.w, b.w);
    }
    k_planar_keys<<<nblk(n, 256), 256, 0, st>>>(h.bound.p, n, gb, h.key.p);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
  // counting sort by the top key bits, then sort inside bins
  const int64_t nbins = ((int64_t)1 << (32 - kSortShift));
  DBuf<int32_t> cnt((size_t)nbins + 1, st), fill((size_t)nbins, st);
  cnt.zero();
  fill.zero();
  k_hist<<<nblk(n, 256), 256, 0, st>>>(h.key.p, n, kSortShift, cnt.p);
  CRG_CHECK_CUDA(cudaGetLastError());
  exclusive_scan_i32(cnt.p, cnt.p, nbins, st);
  h.perm.alloc((size_t)n, st);
  k_bin_scatter<<<nblk(n, 256), 256, 0, st>>>(h.key.p, n, kSortShift, cnt.p, fill.p, h.perm.p);
  CRG_CHECK_CUDA(cudaGetLastError());
  {
    DBuf<uint64_t> w((size_t)n, st);
    DBuf<int32_t> large((size_t)nbins + 1, st);  // [nbins] large bins | [1] their count
    DBuf<unsigned long long> too_big(1, st);
    CRG_CHECK_CUDA(cudaMemsetAsync(large.p + nbins, 0, sizeof(int32_t), st));
    too_big.zero();
    if (n) k_bin_pack<<<nblk(n, 256), 256, 0, st>>>(h.key.p, h.perm.p, n, w.p);
    k_bin_sort<<<nblk(nbins, 256), 256, 0, st>>>(w.p, cnt.p, nbins, large.p, large.p + nbins);
    CRG_CHECK_CUDA(cudaGetLastError());
    int32_t hl = 0;
    CRG_CHECK_CUDA(cudaMemcpyAsync(&hl, large.p + nbins, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CRG_CHECK_CUDA(cudaStreamSynchronize(st));
    if (hl) {
      k_bin_sort_large<<<(unsigned)hl, 256, 0, st>>>(w.p, cnt.p, large.p, too_big.p);
      CRG_CHECK_CUDA(cudaGetLastError());
      unsigned long long hb = 0;
      CRG_CHECK_CUDA(cudaMemcpyAsync(&hb, too_big.p, sizeof(hb), cudaMemcpyDeviceToHost, st));
      CRG_CHECK_CUDA(cudaStreamSynchronize(st));
      CRG_REQUIRE(hb == 0, CRG_ERR_NOT_SUPPORTED, "%llu Morton bins hold more than %d cells", hb, kBinLarge);
    }
    if (n) k_bin_unpack<<<nblk(n, 256), 256, 0, st>>>(w.p, n, h.perm.p);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
  // hierarchy
  int64_t nleaves = (n + kLeaf - 1) / kLeaf;
  int64_t total = 0;
  int nlev = 0;
  for (int64_t c = nleaves;; c = (c + 1) / 2) {
    CRG_REQUIRE(nlev < kMaxLevels, CRG_ERR_INTERNAL, "hierarchy too deep");
    h.t.off[nlev] = total;
    h.t.cnt[nlev] = c;
    total += c;
    nlev++;
    if (c == 1) break;
  }
  h.t.nlev = nlev;
  CRG_REQUIRE(nleaves < ((int64_t)1 << 27), CRG_ERR_NOT_SUPPORTED, "too many cells for the hierarchy");
  h.lo.alloc((size_t)total, st);
  h.hi.alloc((size_t)total, st);
  h.sbound.alloc((size_t)n, st);
  if (sph)
    k_leaves<true><<<nblk(nleaves, 128), 128, 0, st>>>(h.bound.p, h.perm.p, n, nleaves, h.lo.p, h.hi.p, h.sbound.p);
  else
    k_leaves<false><<<nblk(nleaves, 128), 128, 0, st>>>(h.bound.p, h.perm.p, n, nleaves, h.lo.p, h.hi.p, h.sbound.p);
  CRG_CHECK_CUDA(cudaGetLastError());
  LevelTable lt{};
  for (int l = 0; l < nlev; ++l) {
    lt.off[l] = h.t.off[l];
    lt.cnt[l] = h.t.cnt[l];
  }
  for (int l0 = 0; l0 + 1 < nlev;) {
    const int nup = std::min(kUp, nlev - 1 - l0);
    const int64_t blocks = (h.t.cnt[l0] + (1 << kUp) - 1) >> kUp;
    k_levels_up<<<(unsigned)blocks, 256, 0, st>>>(h.lo.p, h.hi.p, lt, l0, nup);
    CRG_CHECK_CUDA(cudaGetLastError());
    l0 += nup;
  }
  h.t.lo = h.lo.p;
  h.t.hi = h.hi.p;
  h.t.sbound = h.sbound.p;
  h.t.perm = h.perm.p;
}

TreeView view_of(const Tree& t) {
  TreeView v{};
  for (int l = 0; l < kMaxLevels; ++l) { v.off[l] = t.off[l]; v.cnt[l] = t.cnt[l]; }
  v.lo = t.lo;
  v.hi = t.hi;
  return v;
}

// Capacity of the frontier and leaf-pair buffers of the traversal's levels
// launched back to back.  CRG_TRAVERSE_CAPACITY (>= 1, read at every build)
// lowers it, to exercise the per-level fallback a frontier too large for the
// buffers takes.
int64_t traverse_capacity(int64_t dflt) {
  const char* e = getenv("CRG_TRAVERSE_CAPACITY");
  if (e) {
    const long long v = atoll(e);
    if (v >= 1 && v < dflt) return (int64_t)v;
  }
  return dflt;
}

// K3 host loop.  Returns the candidate list (dst cell, src cell).
void dual_traverse(const HostTree& D, const HostTree& S, bool sph, DBuf<int2>& cand, int64_t& ncand, cudaStream_t st) {
  ncand = 0;
  if (D.t.ncells == 0 || S.t.ncells == 0) return;
  TreeView tv_d = view_of(D.t), tv_s = view_of(S.t);
  DBuf<unsigned long long> counters(2, st);
  DBuf<int> counters_ovf(1, st);
  counters_ovf.zero();
  DBuf<uint2> front, next, leafp;
  size_t front_cap = 1024, leaf_cap = 1 << 16;
  front.alloc(front_cap, st);
  next.alloc(front_cap * 4, st);
  leafp.alloc(leaf_cap, st);
  int64_t nleaf = 0;
  uint2 root = make_uint2(((uint32_t)(D.t.nlev - 1) << 27), ((uint32_t)(S.t.nlev - 1) << 27));
  int64_t nfront = 1;
  if (D.t.nlev == 1 && S.t.nlev == 1) {
    CRG_CHECK_CUDA(cudaMemcpyAsync(leafp.p, &root, sizeof(uint2), cudaMemcpyHostToDevice, st));
    nleaf = 1;
    nfront = 0;
  } else {
    CRG_CHECK_CUDA(cudaMemcpyAsync(front.p, &root, sizeof(uint2), cudaMemcpyHostToDevice, st));
  }
  // All levels launched back to back (pairs of a level are all at the same
  // two tree levels, so there are max(levels) - 1 of them), the frontier sizes
  // kept on the device: one host round trip instead of one per level.
  if (nfront > 0) {
    const int steps = std::max(D.t.nlev, S.t.nlev) - 1;
    const int64_t cap = traverse_capacity(std::max<int64_t>(1 << 16, 2 * (D.t.ncells + S.t.ncells)));
    DBuf<uint2> fa((size_t)cap, st), fb((size_t)cap, st), fl((size_t)cap, st);
    DBuf<unsigned long long> cnt((size_t)steps + 2, st);
    DBuf<int> ovf(1, st);
    cnt.zero();
    ovf.zero();
    const unsigned long long one = 1ull;
    CRG_CHECK_CUDA(cudaMemcpyAsync(cnt.p, &one, sizeof(one), cudaMemcpyHostToDevice, st));
    CRG_CHECK_CUDA(cudaMemcpyAsync(fa.p, &root, sizeof(uint2), cudaMemcpyHostToDevice, st));
    for (int l = 0; l < steps; ++l) {
      uint2* in = (l & 1) ? fb.p : fa.p;
      uint2* out = (l & 1) ? fa.p : fb.p;
      k_traverse<<<152 * 8, 256, 0, st>>>(in, -1, cnt.p + l, tv_d, tv_s, out, cnt.p + l + 1, cap, fl.p,
                                          cnt.p + steps + 1, cap, ovf.p);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
    unsigned long long hl[2] = {0ull, 0ull};
    int hov = 0;
    CRG_CHECK_CUDA(cudaMemcpyAsync(hl, cnt.p + steps, sizeof(hl), cudaMemcpyDeviceToHost, st));
    CRG_CHECK_CUDA(cudaMemcpyAsync(&hov, ovf.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CRG_CHECK_CUDA(cudaStreamSynchronize(st));
    if (!hov && hl[0] == 0) {  // every pair reached the leaves within the capacities
      nleaf = (int64_t)hl[1];
      nfront = 0;
      std::swap(leafp.p, fl.p);
      std::swap(leafp.n, fl.n);
    }
  }
  while (nfront > 0) {
    if (next.n < (size_t)nfront * 4) next.alloc((size_t)nfront * 8, st);
    if (leafp.n < (size_t)(nleaf + nfront * 4)) {
      DBuf<uint2> bigger((size_t)(nleaf + nfront * 4) * 2, st);
      if (nleaf) CRG_CHECK_CUDA(cudaMemcpyAsync(bigger.p, leafp.p, sizeof(uint2) * nleaf, cudaMemcpyDeviceToDevice, st));
      std::swap(bigger.p, leafp.p);
      std::swap(bigger.n, leafp.n);
    }
    unsigned long long hc[2] = {0ull, (unsigned long long)nleaf};
    CRG_CHECK_CUDA(cudaMemcpyAsync(counters.p, hc, sizeof(hc), cudaMemcpyHostToDevice, st));
    int64_t blocks = std::min<int64_t>(nblk(nfront, 256), 152 * 16);
    k_traverse<<<(unsigned)blocks, 256, 0, st>>>(front.p, nfront, nullptr, tv_d, tv_s, next.p, counters.p,
                                                 (int64_t)next.n, leafp.p, counters.p + 1, (int64_t)leafp.n,
                                                 counters_ovf.p);
    CRG_CHECK_CUDA(cudaGetLastError());
    int hov = 0;
    CRG_CHECK_CUDA(cudaMemcpyAsync(hc, counters.p, sizeof(hc), cudaMemcpyDeviceToHost, st));
    CRG_CHECK_CUDA(cudaMemcpyAsync(&hov, counters_ovf.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CRG_CHECK_CUDA(cudaStreamSynchronize(st));
    // the buffers hold 4 pairs per input pair, the most one pair can make
    CRG_REQUIRE(hov == 0, CRG_ERR_INTERNAL, "dual traversal overflowed its per-level buffers");
    nfront = (int64_t)hc[0];
    nleaf = (int64_t)hc[1];
    std::swap(front.p, next.p);
    std::swap(front.n, next.n);
  }
  if (nleaf == 0) return;
  // A leaf pair yields at most kLeaf^2 candidates, so below 2^32 / kLeaf^2 leaf
  // pairs the int32 scan of their counts cannot pass 2^32, and a total of 2^31
  // or more shows as negative (checked after the scan).
  CRG_REQUIRE(nleaf < ((int64_t)1 << 32) / (kLeaf * kLeaf), CRG_ERR_NOT_SUPPORTED,
              "%lld leaf pairs: the candidate count could overflow int32", (long long)nleaf);
  DBuf<int32_t> cnt((size_t)nleaf + 1, st);
  if (sph)
    k_leaf_count<true><<<nblk(nleaf, 128), 128, 0, st>>>(leafp.p, nleaf, D.t.sbound, D.t.ncells, S.t.sbound, S.t.ncells, cnt.p);
  else
    k_leaf_count<false><<<nblk(nleaf, 128), 128, 0, st>>>(leafp.p, nleaf, D.t.sbound, D.t.ncells, S.t.sbound, S.t.ncells, cnt.p);
  CRG_CHECK_CUDA(cudaGetLastError());
  exclusive_scan_i32(cnt.p, cnt.p, nleaf, st);
  int32_t tot = 0;
  CRG_CHECK_CUDA(cudaMemcpyAsync(&tot, cnt.p + nleaf, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  CRG_CHECK_CUDA(cudaStreamSynchronize(st));
  CRG_REQUIRE(tot >= 0, CRG_ERR_NOT_SUPPORTED, "candidate count overflows int32");
  ncand = tot;
  cand.alloc((size_t)(tot > 0 ? tot : 1), st);
  if (tot == 0) return;
  if (sph)
    k_leaf_emit<true><<<nblk(nleaf, 128), 128, 0, st>>>(leafp.p, nleaf, D.t.sbound, D.t.perm, D.t.ncells, S.t.sbound,
                                                       S.t.perm, S.t.ncells, cnt.p, cand.p);
  else
    k_leaf_emit<false><<<nblk(nleaf, 128), 128, 0, st>>>(leafp.p, nleaf, D.t.sbound, D.t.perm, D.t.ncells, S.t.sbound,
                                                        S.t.perm, S.t.ncells, cnt.p, cand.p);
  CRG_CHECK_CUDA(cudaGetLastError());
}

struct Events {
  cudaEvent_t e[5] = {};
  Events() {
    for (auto& x : e) CRG_CHECK_CUDA(cudaEventCreate(&x));
  }
  ~Events() {
    for (auto& x : e) if (x) cudaEventDestroy(x);
  }
};

}  // namespace

bool is_device_pointer(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Sorts the columns (and values) of every row of a CSR ascending.
void sort_rows(const RowSet* sets, int nsets, cudaStream_t st) {
  // per set: [nrows] mid rows | [nrows] long rows | [nrows] 9..32-entry rows; then [3] counts per set
  std::vector<int64_t> base((size_t)nsets + 1, 0);
  for (int k = 0; k < nsets; ++k) base[k + 1] = base[k] + 3 * sets[k].nrows;
  DBuf<int32_t> lists((size_t)base[nsets] + 3 * nsets, st);
  int32_t* counts = lists.p + base[nsets];
  CRG_CHECK_CUDA(cudaMemsetAsync(counts, 0, 3 * nsets * sizeof(int32_t), st));
  for (int k = 0; k < nsets; ++k) {
    const RowSet& r = sets[k];
    if (r.nrows == 0) continue;
    int32_t* l = lists.p + base[k];
    k_row_sort_small<<<nblk(r.nrows, 256), 256, 0, st>>>(r.ptr, r.nrows, r.idx, r.val);
    k_row_classes<<<nblk(r.nrows, 256), 256, 0, st>>>(r.ptr, r.nrows, l + 2 * r.nrows, l, l + r.nrows, counts + 3 * k);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
  std::vector<int32_t> h((size_t)3 * nsets);
  CRG_CHECK_CUDA(cudaMemcpyAsync(h.data(), counts, sizeof(int32_t) * 3 * nsets, cudaMemcpyDeviceToHost, st));
  CRG_CHECK_CUDA(cudaStreamSynchronize(st));  // one wait for all sets
  for (int k = 0; k < nsets; ++k) {
    const RowSet& r = sets[k];
    const int32_t* hk = h.data() + 3 * k;
    int32_t* l = lists.p + base[k];
    if (hk[2]) {
      k_row_sort_warp<<<nblk((int64_t)hk[2] * 32, 256), 256, 0, st>>>(r.ptr, l + 2 * r.nrows, hk[2], r.idx, r.val);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
    if (hk[0]) {
      k_row_sort_block<<<(unsigned)hk[0], kRowSortThreads, 0, st>>>(r.ptr, l, r.idx, r.val);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
    if (hk[1]) {
      DBuf<int64_t> off(hk[1] + 1, st);
      k_long_windows<<<1, 1, 0, st>>>(r.ptr, l + r.nrows, hk[1], off.p);
      CRG_CHECK_CUDA(cudaGetLastError());
      int64_t total = 0;
      CRG_CHECK_CUDA(cudaMemcpyAsync(&total, off.p + hk[1], sizeof(total), cudaMemcpyDeviceToHost, st));
      CRG_CHECK_CUDA(cudaStreamSynchronize(st));
      DBuf<int32_t> gk(total, st);
      DBuf<double> gv(total, st);
      k_row_sort_long<<<(unsigned)hk[1], 1024, 0, st>>>(r.ptr, l + r.nrows, off.p, r.idx, r.val, gk.p, gv.p);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
  }
}

void sort_rows(const int32_t* ptr, int64_t nrows, int32_t* idx, double* val, cudaStream_t st) {
  const RowSet one{ptr, nrows, idx, val};
  sort_rows(&one, 1, st);
}

void free_csr(DevCsr& c) {
  cudaFree(c.erow);
  cudaFree(c.rbits);
  cudaFree(c.nextrow);
  cudaFree(c.split);
  cudaFree(c.tasks);
  cudaFree(c.tslot);
  cudaFree(c.ptr); cudaFree(c.idx); cudaFree(c.val); cudaFree(c.val32); cudaFree(c.wn32); cudaFree(c.adj32);
  c = DevCsr{};
}

void free_regridder(crg_regridder* r) {
  if (!r) return;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaSetDevice(r->device);
  free_csr(r->fwd);
  free_csr(r->rev);
  cudaFree(r->dst_area);
  cudaFree(r->src_area);
  cudaFree(r->dst_area_inv);
  cudaFree(r->src_area_inv);
  cudaFree(r->row_sum);
  cudaFree(r->col_sum);
  for (int d = 0; d < 2; ++d) {
    if (r->stage[d]) cudaFree(r->stage[d]);
    if (r->copy_in[d]) cudaStreamDestroy(r->copy_in[d]);
    if (r->copy_out[d]) cudaStreamDestroy(r->copy_out[d]);
  }
  cudaSetDevice(dev);
  delete r;
}

// ------------------------------------------------------------------ shared build stages

struct PairSearch::Impl {
  DevGrid gd, gs;
  HostTree td, ts;
  DBuf<int2> cand, kept;
  DBuf<double4_32a> planes;
  DBuf<float4> planes32;
};

PairSearch::PairSearch() : impl(new Impl) {}
PairSearch::~PairSearch() { delete impl; }

void PairSearch::upload(const crg_grid_desc* dst, const crg_grid_desc* src, cudaStream_t st) {
  CRG_REQUIRE(dst && src, CRG_ERR_INVALID_ARGUMENT, "dst and src grids must not be NULL");
  CRG_REQUIRE(dst->manifold == src->manifold, CRG_ERR_INVALID_ARGUMENT,
              "Destination and source manifolds must be the same (got %d and %d); promote planar lon/lat to the sphere first",
              dst->manifold, src->manifold);
  sph = dst->manifold == CRG_SPHERICAL;
  upload_grid(dst, impl->gd, st);
  upload_grid(src, impl->gs, st);
  nd = impl->gd.ncells;
  ns = impl->gs.ncells;
  dtab = impl->gd.tab;
  stab = impl->gs.tab;
}

void PairSearch::search(double* dst_area, double* src_area, cudaStream_t st) {
  build_tree(impl->gd, sph, dst_area, impl->td, st);
  build_tree(impl->gs, sph, src_area, impl->ts, st);
  dual_traverse(impl->td, impl->ts, sph, impl->cand, nc, st);
  nc_search = nc;
  cand = impl->cand.p;
  if (sph && nc && nd) {
    impl->planes.alloc((size_t)nd * dtab.maxv, st);
    impl->planes32.alloc((size_t)nd * dtab.maxv, st);
    k_edge_planes<<<nblk(nd, 128), 128, 0, st>>>(dtab.v, dtab.nv, dtab.ori, dtab.maxv, nd, impl->planes.p,
                                                 impl->planes32.p);
    CRG_CHECK_CUDA(cudaGetLastError());
    dplanes = impl->planes.p;
    dplanes32 = impl->planes32.p;
    // drop the pairs separated by a destination edge, group the rest by class
    DBuf<int32_t> cnt(kClasses + 1, st), off(kClasses + 1, st), fill(kClasses + 1, st);
    DBuf<uint16_t> cls((size_t)nc + 1, st);
    cnt.zero();
    fill.zero();
    k_separated<<<nblk(nc, 256), 256, 0, st>>>(cand, nc, dtab.v4, dtab.nv, dtab.maxv, stab.v4, stab.nv, stab.ori,
                                               stab.maxv, dplanes32, cls.p);
    CRG_CHECK_CUDA(cudaGetLastError());
    k_class_count<<<nblk(nc, 256), 256, 0, st>>>(cls.p, nc, cnt.p);
    CRG_CHECK_CUDA(cudaGetLastError());
    exclusive_scan_i32(cnt.p, off.p, kClasses, st);
    int32_t nk = 0;
    CRG_CHECK_CUDA(cudaMemcpyAsync(&nk, off.p + kClasses, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CRG_CHECK_CUDA(cudaStreamSynchronize(st));
    impl->kept.alloc((size_t)nk + 1, st);
    k_class_scatter<<<nblk(nc, 256), 256, 0, st>>>(cand, cls.p, nc, off.p, fill.p, impl->kept.p);
    CRG_CHECK_CUDA(cudaGetLastError());
    nc = nk;
    cand = impl->kept.p;
  }
}

void ensure_row_col_sums(const crg_regridder* Rc) {
  crg_regridder* R = const_cast<crg_regridder*>(Rc);  // the sums are a cache: R stays logically read-only
  std::lock_guard<std::mutex> lock(R->sums_mu);
  if (R->sums_ready) return;
  int dev = 0;
  CRG_CHECK_CUDA(cudaGetDevice(&dev));
  struct Restore {
    int d;
    ~Restore() { cudaSetDevice(d); }
  } restore{dev};
  CRG_CHECK_CUDA(cudaSetDevice(R->device));
  cudaStream_t st = nullptr;
  CRG_CHECK_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  cudaError_t e = cudaSuccess;
  if (!R->row_sum) e = cudaMalloc((void**)&R->row_sum, sizeof(double) * (R->nd + 4));
  if (e == cudaSuccess && !R->col_sum) e = cudaMalloc((void**)&R->col_sum, sizeof(double) * (R->ns + 4));
  if (e == cudaSuccess && R->nd) k_row_sums<<<nblk(R->nd, 256), 256, 0, st>>>(R->fwd.ptr, R->fwd.val, R->nd, R->row_sum);
  if (e == cudaSuccess && R->ns) k_row_sums<<<nblk(R->ns, 256), 256, 0, st>>>(R->rev.ptr, R->rev.val, R->ns, R->col_sum);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  CRG_CHECK_CUDA(e);
  R->sums_ready = true;
}

void finish_build(crg_regridder* R, cudaStream_t st) {
  const int64_t nd = R->nd, ns = R->ns, nnz = R->nnz;
  for (DevCsr* c : {&R->fwd, &R->rev}) {
    c->val32 = keep_alloc<float>((size_t)nnz, st);
    c->wn32 = keep_alloc<float>((size_t)nnz, st);
    c->adj32 = keep_alloc<float>((size_t)nnz, st);
  }
  DBuf<int32_t> dcounts(6, st);
  build_merge_path(R->fwd, dcounts.p, st);  // also the row of every entry
  build_merge_path(R->rev, dcounts.p + 3, st);
  // the reciprocals of the final areas, kept for the FP64 apply's quotients
  R->dst_area_inv = keep_alloc<double>((size_t)nd, st);
  R->src_area_inv = keep_alloc<double>((size_t)ns, st);
  if (nd) k_recip<<<nblk(nd, 256), 256, 0, st>>>(R->dst_area, nd, R->dst_area_inv);
  if (ns) k_recip<<<nblk(ns, 256), 256, 0, st>>>(R->src_area, ns, R->src_area_inv);
  CRG_CHECK_CUDA(cudaGetLastError());
  if (nnz) {
    k_derive<<<nblk(nnz, 256), 256, 0, st>>>(R->fwd.erow, R->fwd.idx, R->fwd.val, nnz, R->dst_area_inv,
                                             R->src_area_inv, R->fwd.val32, R->fwd.wn32, R->fwd.adj32);
    k_derive<<<nblk(nnz, 256), 256, 0, st>>>(R->rev.erow, R->rev.idx, R->rev.val, nnz, R->src_area_inv,
                                             R->dst_area_inv, R->rev.val32, R->rev.wn32, R->rev.adj32);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
  int32_t hc[6];
  CRG_CHECK_CUDA(cudaMemcpyAsync(hc, dcounts.p, sizeof(hc), cudaMemcpyDeviceToHost, st));
  CRG_CHECK_CUDA(cudaStreamSynchronize(st));
  finish_merge_path(R->fwd, hc, st);
  finish_merge_path(R->rev, hc + 3, st);
  noalloc_prepare(R->device);
  crg_info& I = R->info;
  const DevCsr* cs[2] = {&R->fwd, &R->rev};
  for (int d = 0; d < 2; ++d) {
    I.merge_tasks[d] = cs[d]->ntasks;
    I.cut_rows[d] = cs[d]->nsplit;
    I.carry_slots[d] = cs[d]->nslots;
    I.empty_rows[d] = cs[d]->nempty;
  }
}

void check_grid_desc(const crg_grid_desc* g, const char* which) {
  CRG_REQUIRE(g != nullptr, CRG_ERR_INVALID_ARGUMENT, "%s grid descriptor is NULL", which);
  CRG_REQUIRE(g->manifold == CRG_PLANAR || g->manifold == CRG_SPHERICAL, CRG_ERR_INVALID_ARGUMENT,
              "%s grid: unknown manifold %d", which, g->manifold);
  CRG_REQUIRE(g->ncells >= 0 && g->ncells < (int64_t)1 << 31, CRG_ERR_NOT_SUPPORTED,
              "%s grid: ncells = %lld is outside [0, 2^31)", which, (long long)g->ncells);
  if (g->kind == CRG_GRID_CURVILINEAR) {
    CRG_REQUIRE(g->nblocks >= 1 && g->nblocks <= kMaxBlocks, CRG_ERR_INVALID_ARGUMENT,
                "%s grid: nblocks = %d must be in 1..%d", which, g->nblocks, kMaxBlocks);
    CRG_REQUIRE(g->block_nx && g->block_ny && g->points, CRG_ERR_INVALID_ARGUMENT,
                "%s grid: curvilinear grid arrays are NULL", which);
    int64_t cells = 0;
    for (int b = 0; b < g->nblocks; ++b) {
      const int64_t nx = g->block_nx[b], ny = g->block_ny[b];
      CRG_REQUIRE(nx >= 1 && ny >= 1 && nx < (int64_t)1 << 31 && ny < (int64_t)1 << 31, CRG_ERR_INVALID_ARGUMENT,
                  "%s grid: block %d has %lld x %lld cells", which, b, (long long)nx, (long long)ny);
      cells += nx * ny;  // < 2^62 + 2^31: no overflow
      CRG_REQUIRE(cells <= g->ncells, CRG_ERR_DIMENSION_MISMATCH,
                  "%s grid: ncells = %lld but the blocks hold more cells", which, (long long)g->ncells);
    }
    CRG_REQUIRE(cells == g->ncells, CRG_ERR_DIMENSION_MISMATCH, "%s grid: ncells = %lld but the blocks hold %lld cells",
                which, (long long)g->ncells, (long long)cells);
  } else if (g->kind == CRG_GRID_CELLS) {
    CRG_REQUIRE(g->max_verts >= 3 && g->max_verts <= CRG_MAXV, CRG_ERR_INVALID_ARGUMENT,
                "%s grid: max_verts = %d must be in 3..%d", which, g->max_verts, CRG_MAXV);
    CRG_REQUIRE(g->cell_verts || g->ncells == 0, CRG_ERR_INVALID_ARGUMENT, "%s grid: cell_verts is NULL", which);
  } else {
    CRG_REQUIRE(false, CRG_ERR_INVALID_ARGUMENT, "%s grid: unknown grid kind %d", which, g->kind);
  }
}

crg_regridder* build_impl(const crg_grid_desc* dst, const crg_grid_desc* src, const crg_build_opts* opts) {
  CRG_REQUIRE(dst && src, CRG_ERR_INVALID_ARGUMENT, "dst and src grids must not be NULL");
  CRG_REQUIRE(dst->manifold == src->manifold, CRG_ERR_INVALID_ARGUMENT,
              "Destination and source manifolds must be the same (got %d and %d); promote planar lon/lat to the sphere first",
              dst->manifold, src->manifold);
  CRG_REQUIRE(!opts || opts->flags == 0, CRG_ERR_INVALID_ARGUMENT, "crg_build_opts.flags must be 0");
  check_grid_desc(dst, "destination");
  check_grid_desc(src, "source");
  const bool sph = dst->manifold == CRG_SPHERICAL;
  cudaStream_t st = opts ? (cudaStream_t)opts->stream : nullptr;
  const int normalize = opts ? opts->normalize : 0;

  crg_regridder* R = new crg_regridder();
  try {
    CRG_CHECK_CUDA(cudaGetDevice(&R->device));
    R->manifold = dst->manifold;
    Events ev;
    CRG_CHECK_CUDA(cudaEventRecord(ev.e[0], st));

    PairSearch ps;
    ps.upload(dst, src, st);
    const int64_t nd = ps.nd, ns = ps.ns;
    R->nd = nd;
    R->ns = ns;
    R->dst_area = keep_alloc<double>((size_t)nd, st);
    R->src_area = keep_alloc<double>((size_t)ns, st);
    ps.search(R->dst_area, R->src_area, st);
    const int64_t nc = ps.nc;
    R->ncand = ps.nc_search;
    CRG_CHECK_CUDA(cudaEventRecord(ev.e[1], st));

    // K4
    DBuf<double> area((size_t)(nc > 0 ? nc : 1), st);
    DBuf<int32_t> rowcnt((size_t)nd + 1, st), colcnt((size_t)ns + 1, st);
    DBuf<unsigned long long> ovf(1, st);
    rowcnt.zero();
    colcnt.zero();
    ovf.zero();
    if (nc) {
      const CellTable &D = ps.dtab, &S = ps.stab;
      if (sph)
        k_clip<true><<<nblk(nc, 128), 128, 0, st>>>(ps.cand, nc, D.v, D.nv, D.ori, D.maxv, S.v, S.nv, S.ori, S.maxv,
                                                    area.p, rowcnt.p, colcnt.p, ovf.p, ps.dplanes, ps.dplanes32,
                                                    D.v4, S.v4);
      else
        k_clip<false><<<nblk(nc, 128), 128, 0, st>>>(ps.cand, nc, D.v, D.nv, D.ori, D.maxv, S.v, S.nv, S.ori, S.maxv,
                                                     area.p, rowcnt.p, colcnt.p, ovf.p, nullptr, nullptr, nullptr,
                                                     nullptr);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
    CRG_CHECK_CUDA(cudaEventRecord(ev.e[2], st));

    // K5
    R->fwd.nrows = nd; R->fwd.ncols = ns;
    R->rev.nrows = ns; R->rev.ncols = nd;
    R->fwd.ptr = keep_alloc<int32_t>((size_t)nd + 1, st);
    R->rev.ptr = keep_alloc<int32_t>((size_t)ns + 1, st);
    exclusive_scan_i32(rowcnt.p, R->fwd.ptr, nd, st);
    exclusive_scan_i32(colcnt.p, R->rev.ptr, ns, st);
    int32_t hnnz = 0;
    unsigned long long hovf = 0;
    CRG_CHECK_CUDA(cudaMemcpyAsync(&hnnz, R->fwd.ptr + nd, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CRG_CHECK_CUDA(cudaMemcpyAsync(&hovf, ovf.p, sizeof(hovf), cudaMemcpyDeviceToHost, st));
    CRG_CHECK_CUDA(cudaStreamSynchronize(st));
    CRG_REQUIRE(hovf == 0, CRG_ERR_GEOMETRY,
                "%llu candidate pairs exceeded the clipped-polygon capacity of %d vertices (non-convex cells?)",
                (unsigned long long)hovf, CRG_MAXC);
    const int64_t nnz = hnnz;
    R->nnz = nnz;
    R->fwd.nnz = R->rev.nnz = nnz;
    R->fwd.idx = keep_alloc<int32_t>((size_t)nnz, st);
    R->fwd.val = keep_alloc<double>((size_t)nnz, st);
    R->rev.idx = keep_alloc<int32_t>((size_t)nnz, st);
    R->rev.val = keep_alloc<double>((size_t)nnz, st);
    rowcnt.zero();
    colcnt.zero();
    if (nc) {
      k_scatter_pairs<<<nblk(nc, 256), 256, 0, st>>>(ps.cand, area.p, nc, R->fwd.ptr, rowcnt.p, R->rev.ptr, colcnt.p,
                                                     R->fwd.idx, R->fwd.val, R->rev.idx, R->rev.val);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
    const RowSet both[2] = {{R->fwd.ptr, nd, R->fwd.idx, R->fwd.val}, {R->rev.ptr, ns, R->rev.idx, R->rev.val}};
    sort_rows(both, 2, st);

    // normalize! (regridder.jl:54-62)
    DBuf<unsigned long long> mx(1, st);
    mx.zero();
    if (nnz) {
      k_max_val<<<(unsigned)std::min<int64_t>(nblk(nnz, 256), 152 * 8), 256, 0, st>>>(R->fwd.val, nnz, mx.p);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
    // max(A) is read back with the build's last synchronisation (the divisions read it on the device)
    unsigned long long hmx = 0;
    CRG_CHECK_CUDA(cudaMemcpyAsync(&hmx, mx.p, sizeof(hmx), cudaMemcpyDeviceToHost, st));
    R->normalized = normalize;
    if (normalize && 2 * nnz + nd + ns) {
      k_div_by<<<nblk((2 * nnz + nd + ns + kDivPer - 1) / kDivPer, 256), 256, 0, st>>>(
          R->fwd.val, R->rev.val, nnz, R->dst_area, nd, R->src_area, ns, mx.p);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
    finish_build(R, st);
    CRG_CHECK_CUDA(cudaEventRecord(ev.e[3], st));
    CRG_CHECK_CUDA(cudaEventSynchronize(ev.e[3]));
    double maxA;
    memcpy(&maxA, &hmx, sizeof(double));
    R->normalizer = normalize ? maxA : 1.0;
    float t01 = 0, t12 = 0, t23 = 0, t03 = 0;
    cudaEventElapsedTime(&t01, ev.e[0], ev.e[1]);
    cudaEventElapsedTime(&t12, ev.e[1], ev.e[2]);
    cudaEventElapsedTime(&t23, ev.e[2], ev.e[3]);
    cudaEventElapsedTime(&t03, ev.e[0], ev.e[3]);
    crg_info& I = R->info;
    I.n_dst = nd; I.n_src = ns; I.nnz = nnz; I.n_candidates = ps.nc_search; I.n_clipped = ps.nc;
    I.manifold = R->manifold; I.normalized = normalize;
    I.normalizer = R->normalizer;
    I.t_build_ms = t03; I.t_search_ms = t01; I.t_clip_ms = t12; I.t_assemble_ms = t23;
    I.clip_overflows = (int64_t)hovf;
    I.device = R->device;
    // temporaries are freed stream-ordered by the DBuf destructors
  } catch (...) {
    free_regridder(R);
    throw;
  }
  return R;
}

}  // namespace crg
