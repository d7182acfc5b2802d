// crg_batch.cu -- many regridders at once: concurrent builds and a
// graph-captured apply of a whole batch.
//
// The reference builds and applies one Regridder at a time
// (src/regridder/regridder.jl:105-163, src/regridder/regrid.jl:63-118).  For
// workloads with many grid pairs the GPU work of one small pair is a series
// of short kernels separated by host synchronisations, so crg_build_batch
// runs the builds from several host threads, each on its own stream, and
// crg_apply_plan captures the applies of all pairs into one CUDA graph that
// replays with a single launch.
#include <atomic>
#include <string>
#include <thread>
#include <vector>

#include "crg_internal.cuh"

struct crg_apply_plan {
  cudaGraphExec_t exec = nullptr;
  std::vector<crg_regridder*> held;  // retained for the plan's lifetime
  int device = 0;
};

namespace crg {

void build_batch_impl(int64_t n, const crg_grid_desc* dst, const crg_grid_desc* src, const crg_build_opts* opts,
                      int nthreads, crg_regridder** out) {
  CRG_REQUIRE(n >= 0, CRG_ERR_INVALID_ARGUMENT, "n must be >= 0");
  CRG_REQUIRE(n == 0 || (dst && src && out), CRG_ERR_INVALID_ARGUMENT, "dst, src and out must not be NULL");
  for (int64_t k = 0; k < n; ++k) out[k] = nullptr;
  if (n == 0) return;
  int dev = 0;
  CRG_CHECK_CUDA(cudaGetDevice(&dev));
  const int workers = (int)std::min<int64_t>(n, nthreads > 0 ? nthreads : 8);
  std::vector<crg_status> status(n, CRG_OK);
  std::vector<std::string> message(n);
  std::atomic<int64_t> next{0};
  auto work = [&]() {
    cudaStream_t st = nullptr;
    if (cudaSetDevice(dev) != cudaSuccess || cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
      for (int64_t k = next.fetch_add(1); k < n; k = next.fetch_add(1)) {
        status[k] = CRG_ERR_CUDA;
        message[k] = "could not create a stream for a build worker";
      }
      return;
    }
    for (int64_t k = next.fetch_add(1); k < n; k = next.fetch_add(1)) {
      crg_build_opts o{};
      if (opts) o = *opts;
      o.stream = st;
      try {
        out[k] = build_impl(&dst[k], &src[k], &o);
      } catch (const Fail& e) {
        status[k] = e.st;
        message[k] = crg_last_error();
      } catch (...) {
        status[k] = CRG_ERR_INTERNAL;
        message[k] = "unexpected internal error";
      }
    }
    cudaStreamDestroy(st);
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < workers; ++t) pool.emplace_back(work);
  work();  // the calling thread works too
  for (auto& th : pool) th.join();
  for (int64_t k = 0; k < n; ++k) {
    if (status[k] != CRG_OK) {
      for (int64_t j = 0; j < n; ++j) {
        if (out[j]) free_regridder(out[j]);
        out[j] = nullptr;
      }
      set_error("pair %lld: %s", (long long)k, message[k].c_str());
      throw Fail{status[k]};
    }
  }
}

crg_apply_plan* apply_plan_impl(int64_t n, const crg_apply_item* items) {
  CRG_REQUIRE(n >= 1 && items, CRG_ERR_INVALID_ARGUMENT, "a plan needs at least one item");
  int dev = 0;
  CRG_CHECK_CUDA(cudaGetDevice(&dev));
  for (int64_t k = 0; k < n; ++k) {
    const crg_apply_item& it = items[k];
    CRG_REQUIRE(it.regridder, CRG_ERR_INVALID_ARGUMENT, "item %lld has no regridder", (long long)k);
    CRG_REQUIRE(it.dst && is_device_pointer(it.dst) && (!it.src || is_device_pointer(it.src)), CRG_ERR_NOT_SUPPORTED,
                "item %lld: a plan replays on the GPU alone, so fields must be device pointers", (long long)k);
  }
  // Capture: the origin stream forks one branch per item (their outputs are
  // distinct), so the graph runs small items side by side.
  std::vector<cudaStream_t> sts(n + 1, nullptr);
  std::vector<cudaEvent_t> evs(n + 1, nullptr);
  auto cleanup = [&]() {
    for (auto e : evs)
      if (e) cudaEventDestroy(e);
    for (auto s : sts)
      if (s) cudaStreamDestroy(s);
  };
  cudaGraph_t graph = nullptr;
  try {
    for (int64_t k = 0; k <= n; ++k) {
      CRG_CHECK_CUDA(cudaStreamCreateWithFlags(&sts[k], cudaStreamNonBlocking));
      CRG_CHECK_CUDA(cudaEventCreateWithFlags(&evs[k], cudaEventDisableTiming));
    }
    cudaStream_t origin = sts[n];
    CRG_CHECK_CUDA(cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal));
    try {
      CRG_CHECK_CUDA(cudaEventRecord(evs[n], origin));
      for (int64_t k = 0; k < n; ++k) {
        const crg_apply_item& it = items[k];
        CRG_CHECK_CUDA(cudaStreamWaitEvent(sts[k], evs[n], 0));
        apply_impl(it.regridder, it.transpose, it.dtype, it.adjoint != 0, it.src, it.src_stride_cell,
                   it.src_stride_field, it.dst, it.dst_stride_cell, it.dst_stride_field, it.nfields, it.normalize,
                   sts[k]);
        CRG_CHECK_CUDA(cudaEventRecord(evs[k], sts[k]));
        CRG_CHECK_CUDA(cudaStreamWaitEvent(origin, evs[k], 0));
      }
    } catch (...) {
      cudaStreamEndCapture(origin, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    CRG_CHECK_CUDA(cudaStreamEndCapture(origin, &graph));
  } catch (...) {
    cleanup();
    throw;
  }
  cleanup();
  crg_apply_plan* p = new crg_apply_plan;
  p->device = dev;
  const cudaError_t e = cudaGraphInstantiate(&p->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    delete p;
    CRG_CHECK_CUDA(e);
  }
  for (int64_t k = 0; k < n; ++k) {
    crg_regridder* r = const_cast<crg_regridder*>(items[k].regridder);
    r->refs.fetch_add(1);
    p->held.push_back(r);
  }
  return p;
}

void apply_plan_launch_impl(crg_apply_plan* p, cudaStream_t st) {
  CRG_REQUIRE(p != nullptr, CRG_ERR_INVALID_ARGUMENT, "plan is NULL");
  int dev = 0;
  CRG_CHECK_CUDA(cudaGetDevice(&dev));
  CRG_REQUIRE(dev == p->device, CRG_ERR_INVALID_ARGUMENT, "plan lives on device %d but device %d is current",
              p->device, dev);
  CRG_CHECK_CUDA(cudaGraphLaunch(p->exec, st));
}

void apply_plan_destroy_impl(crg_apply_plan* p) {
  if (!p) return;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  for (crg_regridder* r : p->held)
    if (r->refs.fetch_sub(1) == 1) free_regridder(r);
  delete p;
}

}  // namespace crg
