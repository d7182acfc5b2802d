// crg_scan.cu -- three-phase exclusive scan (block scan, scan of block sums,
// add-back), recursive over the block sums.
#include "crg_internal.cuh"
#include "crg_scan.cuh"

namespace crg {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;  // 2048

__device__ __forceinline__ int32_t warp_incl_scan(int32_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Scans one tile per block; writes exclusive prefixes and the tile total.
__global__ void k_scan_tiles(const int32_t* __restrict__ in, int32_t* __restrict__ out, int64_t n,
                             int32_t* __restrict__ tile_sums) {
  __shared__ int32_t warp_tot[kScanThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int32_t v[kScanItems];
  int32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + k;
    v[k] = i < n ? in[i] : 0;
    s += v[k];
  }
  int32_t incl = warp_incl_scan(s);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int32_t w = lane < kScanThreads / 32 ? warp_tot[lane] : 0;
    int32_t wi = warp_incl_scan(w);
    if (lane < kScanThreads / 32) warp_tot[lane] = wi - w;
    if (lane == kScanThreads / 32 - 1 && tile_sums) tile_sums[blockIdx.x] = wi;
  }
  __syncthreads();
  int32_t run = warp_tot[warp] + incl - s;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + k;
    int32_t x = v[k];
    if (i < n) out[i] = run;
    run += x;
  }
}

__global__ void k_add_tile_offsets(int32_t* __restrict__ out, int64_t n, const int32_t* __restrict__ offs) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += offs[i / kScanTile];
}

__global__ void k_write_total(const int32_t* __restrict__ in, const int32_t* __restrict__ out, int64_t n,
                              int32_t* __restrict__ total) {
  *total = n > 0 ? out[n - 1] + in[n - 1] : 0;
}

void scan_rec(const int32_t* in, int32_t* out, int64_t n, cudaStream_t st) {
  if (n <= 0) return;
  int64_t ntiles = (n + kScanTile - 1) / kScanTile;
  int32_t* sums = nullptr;
  if (ntiles > 1) CRG_CHECK_CUDA(cudaMallocAsync(&sums, sizeof(int32_t) * (ntiles + 1), st));
  k_scan_tiles<<<(unsigned)ntiles, kScanThreads, 0, st>>>(in, out, n, sums);
  CRG_CHECK_CUDA(cudaGetLastError());
  if (ntiles > 1) {
    scan_rec(sums, sums, ntiles, st);
    k_add_tile_offsets<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, sums);
    CRG_CHECK_CUDA(cudaGetLastError());
    CRG_CHECK_CUDA(cudaFreeAsync(sums, st));
  }
}

}  // namespace

void exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, cudaStream_t st) {
  // The total must be taken from the input before an in-place scan overwrites it.
  int32_t* last = nullptr;
  CRG_CHECK_CUDA(cudaMallocAsync(&last, sizeof(int32_t), st));
  if (n > 0) CRG_CHECK_CUDA(cudaMemcpyAsync(last, in + (n - 1), sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
  scan_rec(in, out, n, st);
  // out[n] = out[n-1] + last input
  k_write_total<<<1, 1, 0, st>>>(last, out + (n > 0 ? n - 1 : 0), n > 0 ? 1 : 0, out + n);
  CRG_CHECK_CUDA(cudaGetLastError());
  CRG_CHECK_CUDA(cudaFreeAsync(last, st));
}

}  // namespace crg
