// crg_layout.cu -- the merge-path layout of each direction of a regridder
// (built once per direction, read by every batched cell-major apply).
#include <stdlib.h>
#include <string.h>

#include "crg_internal.cuh"
#include "crg_scan.cuh"

// ---------------------------------------------------------------------------
// Merge-path layout: the entries of a direction are cut into tasks of
// kTaskNnz consecutive entries (CSR order).  Rows whose entries straddle a task
// boundary are listed with the first and last task they touch, so the apply
// can combine their per-task partial sums in task order afterwards.

namespace crg {

namespace {

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

__global__ void k_expand_rows(const int32_t* __restrict__ ptr, int64_t n, int32_t* __restrict__ erow,
                              uint32_t* __restrict__ rbits, int* __restrict__ nempty) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int32_t a = ptr[r], b = ptr[r + 1];
  for (int32_t k = a; k < b; ++k) erow[k] = (int32_t)r;
  if (a == b)
    atomicAdd(nempty, 1);
  else
    atomicOr(rbits + (a >> 5), 1u << (a & 31));
}

// Row that follows r in entry order (nrows after the last row with entries).
__global__ void k_next_rows(const int32_t* __restrict__ ptr, const int32_t* __restrict__ erow, int64_t n,
                            int64_t nnz, int32_t* __restrict__ nextrow) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int32_t b = ptr[r + 1];
  nextrow[r] = b < nnz ? erow[b] : (int32_t)n;
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
__global__ void k_slot_fill(int32_t* __restrict__ split, const int32_t* __restrict__ nsplit,
                            const int32_t* __restrict__ base, int2* __restrict__ tslot) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= *nsplit) return;
  const int32_t t0 = split[3 * s + 1], pieces = split[3 * s + 2], b = base[s];
  tslot[t0].y = b;
  for (int32_t k = 1; k < pieces; ++k) tslot[t0 + k].x = b + k;
  split[3 * s + 1] = b;
}

}  // namespace

// Enqueued without waiting on the host: the buffers whose length depends on
// the cut rows are sized by the task count (no more rows than tasks can be
// cut), and the counts (cut rows, empty rows, carry slots) go to dcounts[0..2]
// for finish_merge_path, after the caller's one synchronisation for both
// directions.
void build_merge_path(DevCsr& c, int32_t* dcounts, cudaStream_t st) {
  const int64_t n = c.nrows, nnz = c.nnz;
  c.erow = keep_alloc<int32_t>((size_t)nnz, st);
  const size_t nwords = (size_t)(nnz >> 5) + 2;
  c.rbits = keep_alloc<uint32_t>(nwords, st);
  CRG_CHECK_CUDA(cudaMemsetAsync(c.rbits, 0, sizeof(uint32_t) * nwords, st));
  CRG_CHECK_CUDA(cudaMemsetAsync(dcounts, 0, 3 * sizeof(int32_t), st));
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
  const int64_t nt = c.ntasks;
  int32_t* work = nullptr;  // [ntasks + 1] bounds | [ntasks + 1] split positions | [ntasks + 1] pieces
  CRG_CHECK_CUDA(cudaMallocAsync((void**)&work, sizeof(int32_t) * (3 * nt + 3), st));
  int32_t* bound = work;
  int32_t* pos = bound + nt + 1;
  int32_t* span = pos + nt + 1;
  k_expand_rows<<<nblk(n, 256), 256, 0, st>>>(c.ptr, n, c.erow, c.rbits, dcounts + 1);
  CRG_CHECK_CUDA(cudaGetLastError());
  k_task_bounds<<<nblk(nt + 1, 256), 256, 0, st>>>(c.ptr, c.erow, nnz, nt, task_nnz, long_row, bound);
  CRG_CHECK_CUDA(cudaGetLastError());
  k_task_records<<<nblk(nt, 256), 256, 0, st>>>(c.ptr, c.erow, bound, nt, c.tasks, pos);
  CRG_CHECK_CUDA(cudaGetLastError());
  exclusive_scan_i32(pos, pos, nt, st);  // pos[nt] = cut rows
  CRG_CHECK_CUDA(cudaMemcpyAsync(dcounts, pos + nt, sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
  // the next non-empty row of each row (kept only when some row is empty)
  c.nextrow = keep_alloc<int32_t>((size_t)n, st);
  k_next_rows<<<nblk(n, 256), 256, 0, st>>>(c.ptr, c.erow, n, nnz, c.nextrow);
  CRG_CHECK_CUDA(cudaGetLastError());
  CRG_CHECK_CUDA(cudaMemsetAsync(c.tslot, 0xff, sizeof(int2) * nt, st));  // -1: row not cut
  c.split = keep_alloc<int32_t>((size_t)3 * nt, st);
  CRG_CHECK_CUDA(cudaMemsetAsync(span, 0, sizeof(int32_t) * (nt + 1), st));
  k_split_fill<<<nblk(nt, 256), 256, 0, st>>>(c.ptr, bound, nt, c.tasks, pos, c.split, span);
  CRG_CHECK_CUDA(cudaGetLastError());
  exclusive_scan_i32(span, span, nt, st);  // first slots; span[nt] = carry slots
  k_slot_fill<<<nblk(nt, 256), 256, 0, st>>>(c.split, pos + nt, span, c.tslot);
  CRG_CHECK_CUDA(cudaGetLastError());
  CRG_CHECK_CUDA(cudaMemcpyAsync(dcounts + 2, span + nt, sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
  CRG_CHECK_CUDA(cudaFreeAsync(work, st));
}

void finish_merge_path(DevCsr& c, const int32_t* hcounts, cudaStream_t st) {
  if (c.nrows == 0 || c.nnz == 0) return;
  c.nsplit = hcounts[0];
  c.nempty = hcounts[1];
  c.nslots = hcounts[2];
  if (c.nempty == 0) {
    CRG_CHECK_CUDA(cudaFreeAsync(c.nextrow, st));
    c.nextrow = nullptr;
  }
}

}  // namespace crg
