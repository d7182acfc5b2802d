// crg_internal.cuh -- internal types shared by the build, apply and ABI units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "crg.h"

namespace crg {

// Sets the thread-local message returned by crg_last_error().
void set_error(const char* fmt, ...);

struct Fail {
  crg_status st;
};

#define CRG_CHECK_CUDA(expr)                                                              \
  do {                                                                                    \
    cudaError_t e_ = (expr);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      ::crg::set_error("CUDA error %s (%s) at %s:%d", cudaGetErrorName(e_),               \
                       cudaGetErrorString(e_), __FILE__, __LINE__);                       \
      throw ::crg::Fail{e_ == cudaErrorMemoryAllocation ? CRG_ERR_OUT_OF_MEMORY : CRG_ERR_CUDA}; \
    }                                                                                     \
  } while (0)

#define CRG_REQUIRE(cond, status, ...)        \
  do {                                        \
    if (!(cond)) {                            \
      ::crg::set_error(__VA_ARGS__);          \
      throw ::crg::Fail{status};              \
    }                                         \
  } while (0)

constexpr int kMaxGridBlocks = 12;  // curvilinear blocks per grid (cube faces and more)

// Device CSR of one direction.  rows = dst cells for the forward copy,
// src cells for the reverse copy (A^T).
struct DevCsr {
  int64_t nrows = 0, ncols = 0, nnz = 0;
  int32_t* ptr = nullptr;    // [nrows + 1]
  int32_t* idx = nullptr;    // [nnz] column indices, ascending in each row
  double* val = nullptr;     // [nnz] A entries (FP64)
  float* val32 = nullptr;    // [nnz] A entries (FP32)
  float* wn32 = nullptr;     // [nnz] A_rc / area_row (FP32): normalised weights of this direction
  float* adj32 = nullptr;    // [nnz] A_rc / area_col (FP32): adjoint weights of the other direction
  // merge-path layout: runs of about kTaskNnz entries per task, cut at row
  // starts except inside rows longer than kTaskNnz / 4
  int32_t* erow = nullptr;   // [nnz] row of each entry
  uint32_t* rbits = nullptr; // [nnz / 32 + 2] bit e set when entry e starts its row
  int32_t* nextrow = nullptr;  // [nrows] next row with entries (only when some rows have none)
  int64_t ntasks = 0;
  int4* tasks = nullptr;     // [ntasks] x = first entry, y = end entry,
                             //   z = first row | (row began in an earlier task) << 31,
                             //   w = last row | (row continues into a later task) << 31
  int2* tslot = nullptr;     // [ntasks] carry slots of the first / last row when they are cut (-1: none)
  int32_t* split = nullptr;  // [nsplit][3] rows cut between tasks: row, first carry slot, number of slots
  int64_t nsplit = 0;
  int64_t nslots = 0;        // carry slots (128 floats each) of all cut rows
  int64_t nempty = 0;        // rows without entries
};

constexpr int kTaskNnz = 64;  // nominal entries per merge-path task

// Per-cell vertex table on the device: [n][maxv] unit vectors (z = 0 planar).
struct CellTable {
  int64_t n = 0;
  int maxv = 0;
  double* v = nullptr;   // [n * maxv * 3]
  float4* v4 = nullptr;  // [n * maxv] the same vertices rounded to FP32 (w = 0)
  int8_t* nv = nullptr;  // [n]
  int8_t* ori = nullptr;  // [n] +1 counter-clockwise seen from outside (or from +z), -1 clockwise
};

// Device memory a regridder keeps, allocated in stream order (no device-wide
// synchronisation, so builds on different streams overlap) with four spare
// elements (a 16-byte load or copy of an array's last entries stays inside);
// freed with cudaFree when the regridder is released.
template <class T>
T* keep_alloc(size_t n, cudaStream_t st) {
  T* p = nullptr;
  CRG_CHECK_CUDA(cudaMallocAsync((void**)&p, (n + 4) * sizeof(T), st));
  return p;
}

// Stream-ordered temporary device buffer, freed (in stream order) when it goes out of scope.
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t st = nullptr;
  DBuf() = default;
  DBuf(size_t n_, cudaStream_t s) { alloc(n_, s); }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  void alloc(size_t n_, cudaStream_t s) {
    release();
    st = s;
    n = n_;
    if (n) CRG_CHECK_CUDA(cudaMallocAsync((void**)&p, n * sizeof(T), s));
  }
  void zero() {
    if (n) CRG_CHECK_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), st));
  }
  void release() {
    if (p) cudaFreeAsync(p, st);
    p = nullptr;
    n = 0;
  }
  ~DBuf() { release(); }
};

}  // namespace crg

struct crg_regridder {
  std::atomic<int> refs{1};
  int device = 0;
  int manifold = CRG_SPHERICAL;
  int normalized = 0;
  int64_t nd = 0, ns = 0, nnz = 0, ncand = 0;
  double normalizer = 1.0;
  crg::DevCsr fwd;  // CSR of A (rows = dst)
  crg::DevCsr rev;  // CSR of A^T (rows = src)
  double* dst_area = nullptr;   // [nd]
  double* src_area = nullptr;   // [ns]
  // RN(1 / area) per cell, of the final (normalised) areas: the FP64 apply of
  // several fields corrects its quotients from these
  double* dst_area_inv = nullptr;  // [nd]
  double* src_area_inv = nullptr;  // [ns]
  // [nd] / [ns] Kahan row / column sums of A, computed on first request
  // (ensure_row_col_sums) under sums_mu
  double* row_sum = nullptr;
  double* col_sum = nullptr;
  std::mutex sums_mu;
  bool sums_ready = false;
  crg_info info{};
  // staging for host-memory fields in crg_apply
  // per matrix copy ([0] A, [1] A^T), so that an apply of R and one of
  // transpose(R) with host fields can run at the same time
  std::mutex stage_mu[2];
  void* stage[2] = {nullptr, nullptr};
  size_t stage_bytes[2] = {0, 0};
  cudaStream_t copy_in[2] = {nullptr, nullptr};   // host -> device copies of the chunked host-field pipeline
  cudaStream_t copy_out[2] = {nullptr, nullptr};  // device -> host copies of it
  // field-major apply per matrix copy (fwd, rev) and dtype (FP32, BF16):
  // 0 not yet timed, 1 row kernel, 2 transposes around the cell-major kernel
  std::atomic<int> fm_choice[2][2] = {};
};

namespace crg {
// crg_build_impl lives in crg_build.cu; apply entry points in crg_apply.cu.
crg_regridder* build_impl(const crg_grid_desc* dst, const crg_grid_desc* src, const crg_build_opts* opts);
// Host-only checks of a grid descriptor (kind, manifold, sizes, NULL arrays),
// run by the entry points before any device work; `which` names the grid in
// the message.
void check_grid_desc(const crg_grid_desc* g, const char* which);
void free_regridder(crg_regridder* r);
// Streams and events shared by the applies of a batch with host fields: the
// chunks of all items form one pipeline (copies in on cin, applies on cst,
// copies out on cout, in item order).  Owned by the batch.
struct HostPipe {
  cudaStream_t cin = nullptr, cst = nullptr, cout = nullptr;
  std::vector<cudaEvent_t> events;
};
struct HostChunks {
  bool ok = false, cm = false;
  int64_t chunk = 0;
};
void apply_impl(const crg_regridder* r, int transpose, int dtype, bool adjoint, const void* src, int64_t ssc,
                int64_t ssf, void* dst, int64_t dsc, int64_t dsf, int64_t nfields, int normalize, cudaStream_t st,
                HostPipe* pipe = nullptr);
// whether an item's apply runs as the chunked host pipeline, and which matrix copy it reads
bool host_pipeline_item(const crg_apply_item& it);
int host_pipeline_dir(const crg_apply_item& it);
void host_pipeline_ends(const crg_apply_item& it, size_t& fill, size_t& drain);
bool is_device_pointer(const void* p);
void apply_noalloc_impl(const crg_regridder* r, int transpose, int dtype, const void* src, int64_t ssc, int64_t ssf,
                        void* dst, int64_t dsc, int64_t dsf, int64_t nf, int normalize, cudaStream_t st);
// The applies of a batch that one persistent launch can run (cell-major FP32 /
// BF16 fields or single fields, device memory): their device tables, built
// once; handled[k] = 1 for the items it covers (the others need their own
// crg_apply).  batch_enqueue queues its launches on st: one persistent launch
// over the merge-path and row units of every item, then one for cut rows and
// empty rows.
struct BatchLaunch;
// all = false: only the merge-path items of several 128-field passes and fewer
// tasks than the GPU holds warps (whose own launches run the passes one after
// another, latency-bound); all = true: every item the launch can run.
BatchLaunch* batch_prepare(int64_t n, const crg_apply_item* items, std::vector<char>& handled, bool all);
void batch_enqueue(const BatchLaunch* L, cudaStream_t st);
int batch_launches(const BatchLaunch* L);
void batch_free(BatchLaunch* L);
// The autotuner's table of choices (crg_tune.cu): the fastest candidate of a
// kernel family per key, persisted to a small file.
bool tune_enabled();
bool tune_lookup(const std::string& key, int& choice);
void tune_store(const std::string& key, int choice, const float* ms, int n);
// Loads the module that holds crg_apply_noalloc's static scratch on device
// `dev` (current) and caches its address; every build calls it.
void noalloc_prepare(int dev);
// The merge-path layout of one direction, enqueued without host waits; its
// counts land in dcounts[0..2] (device) and finish_merge_path takes them from
// a host copy once the stream has reached them.
void build_merge_path(DevCsr& c, int32_t* dcounts, cudaStream_t st);
void finish_merge_path(DevCsr& c, const int32_t* hcounts, cudaStream_t st);
// Each row segment of a CSR sorted by column (values follow), for several
// CSRs with one host wait between classifying the rows and sorting them.
struct RowSet {
  const int32_t* ptr;
  int64_t nrows;
  int32_t* idx;
  double* val;
};
void sort_rows(const RowSet* sets, int nsets, cudaStream_t st);
void sort_rows(const int32_t* ptr, int64_t nrows, int32_t* idx, double* val, cudaStream_t st);

// The search stage every build shares: both grids' cell tables on the device,
// their exact cell areas, the candidate (dst cell, src cell) pairs of the dual
// traversal and the edge half-spaces of the destination cells (spherical).
// upload() first (cell counts become known), then search().
struct PairSearch {
  struct Impl;
  Impl* impl = nullptr;
  bool sph = true;
  int64_t nd = 0, ns = 0, nc = 0;
  int64_t nc_search = 0;                   // pairs of the traversal, before the separation filter
  CellTable dtab, stab;
  const int2* cand = nullptr;              // [nc] pairs that may overlap
  const double4_32a* dplanes = nullptr;    // spherical: [nd * dtab.maxv]
  const float4* dplanes32 = nullptr;       // spherical: the normals rounded to FP32, w = |n32|_1
  PairSearch();
  ~PairSearch();
  PairSearch(const PairSearch&) = delete;
  PairSearch& operator=(const PairSearch&) = delete;
  void upload(const crg_grid_desc* dst, const crg_grid_desc* src, cudaStream_t st);
  // cell areas into dst_area [nd] and src_area [ns] (device memory)
  void search(double* dst_area, double* src_area, cudaStream_t st);
};

// FP32 weights and the merge-path layouts of both directions of R (after its
// matrix and areas are final).
void finish_build(crg_regridder* R, cudaStream_t st);
// The Kahan row and column sums of A (row_sum, col_sum), computed the first
// time they are asked for; safe to call from several threads.
void ensure_row_col_sums(const crg_regridder* R);
// crg_build_se_to_fv / crg_build_fv_to_se (crg_se.cu)
crg_regridder* build_se_impl(const crg_grid_desc* fv, const crg_se_space* se, const crg_se_opts* opts,
                             bool se_is_dst);
void se_nodes_impl(const crg_se_space* se, const crg_se_opts* opts, double* points, double* weights);
void se_dss_impl(int dtype, void* field, int64_t sn, int64_t sf, int64_t nfields, const int32_t* group_ptr,
                 const int32_t* group_nodes, const double* weights, int64_t ngroups, cudaStream_t st);
void area_grad_impl(const crg_regridder* r, const crg_grid_desc* dst, const crg_grid_desc* src, const double* u,
                    const double* s, const double* c, double* grad, cudaStream_t st);
void mirror_fold_impl(int dtype, void* field, int64_t sc, int64_t sf, int64_t nfields, int64_t nx, int64_t ny,
                      cudaStream_t st);
void build_batch_impl(int64_t n, const crg_grid_desc* dst, const crg_grid_desc* src, const crg_build_opts* opts,
                      int nthreads, crg_regridder** out);
crg_apply_plan* apply_plan_impl(int64_t n, const crg_apply_item* items);
void apply_batch_impl(int64_t n, const crg_apply_item* items, int nthreads, cudaStream_t st);
void apply_plan_launch_impl(crg_apply_plan* p, cudaStream_t st);
void apply_plan_destroy_impl(crg_apply_plan* p);
void apply_plan_info_impl(const crg_apply_plan* p, int64_t* kernels, int64_t* batched_items);
}  // namespace crg
