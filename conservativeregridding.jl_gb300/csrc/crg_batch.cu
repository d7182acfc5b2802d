// crg_batch.cu -- many regridders at once: concurrent builds, concurrent
// applies and a graph-captured apply of a whole batch.
//
// The reference builds and applies one Regridder at a time
// (src/regridder/regridder.jl:105-163, src/regridder/regrid.jl:63-118).  For
// workloads with many grid pairs the GPU work of one small pair is a series
// of short kernels separated by host synchronisations, so crg_build_batch
// runs the builds from several host threads, each on its own stream, and
// crg_apply_plan captures the applies of all pairs into one CUDA graph that
// replays with a single launch.  crg_apply_batch runs independent applies
// from several host threads: with host fields, the copies of one item
// overlap those of the others on both directions of the host link.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <string>
#include <thread>
#include <vector>

#include "crg_internal.cuh"

struct crg_apply_plan {
  cudaGraphExec_t exec = nullptr;
  std::vector<crg_regridder*> held;  // retained for the plan's lifetime
  int device = 0;
  crg::BatchLaunch* batch = nullptr;  // the items one persistent launch runs (tables, carry)
  int64_t kernels = 0;                 // kernel launches per replay
  int64_t batched = 0;                 // items run by the persistent launch
};

namespace crg {

void build_batch_impl(int64_t n, const crg_grid_desc* dst, const crg_grid_desc* src, const crg_build_opts* opts,
                      int nthreads, crg_regridder** out) {
  CRG_REQUIRE(n >= 0, CRG_ERR_INVALID_ARGUMENT, "n must be >= 0");
  CRG_REQUIRE(n == 0 || (dst && src && out), CRG_ERR_INVALID_ARGUMENT, "dst, src and out must not be NULL");
  for (int64_t k = 0; k < n; ++k) out[k] = nullptr;
  if (n == 0) return;
  for (int64_t k = 0; k < n; ++k) {
    char which[48];
    snprintf(which, sizeof which, "pair %lld: destination", (long long)k);
    check_grid_desc(&dst[k], which);
    snprintf(which, sizeof which, "pair %lld: source", (long long)k);
    check_grid_desc(&src[k], which);
  }
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

void apply_batch_impl(int64_t n, const crg_apply_item* items, int nthreads, cudaStream_t st) {
  CRG_REQUIRE(n >= 0, CRG_ERR_INVALID_ARGUMENT, "n must be >= 0");
  CRG_REQUIRE(n == 0 || items, CRG_ERR_INVALID_ARGUMENT, "items must not be NULL");
  for (int64_t k = 0; k < n; ++k)
    CRG_REQUIRE(items[k].regridder, CRG_ERR_INVALID_ARGUMENT, "item %lld has no regridder", (long long)k);
  if (n == 0) return;
  int dev = 0;
  CRG_CHECK_CUDA(cudaGetDevice(&dev));
  // Host fields in every item, each matrix copy once: one chunk pipeline over
  // all items (the copies in of an item follow those of the one before it on
  // one stream while that one's results go out on another).
  bool pipeline = n > 1;
  std::vector<std::mutex*> mus;
  for (int64_t k = 0; k < n && pipeline; ++k) {
    if (!host_pipeline_item(items[k])) pipeline = false;
    else mus.push_back(&const_cast<crg_regridder*>(items[k].regridder)->stage_mu[host_pipeline_dir(items[k])]);
  }
  if (pipeline) {
    std::sort(mus.begin(), mus.end());
    if (std::adjacent_find(mus.begin(), mus.end()) != mus.end()) pipeline = false;
  }
  if (pipeline) {
    std::vector<std::unique_lock<std::mutex>> locks;
    for (auto* m : mus) locks.emplace_back(*m);  // address order: no lock-order cycles
    HostPipe p;
    cudaEvent_t start = nullptr;
    auto cleanup = [&]() {
      for (cudaStream_t s : {p.cin, p.cst, p.cout})
        if (s) cudaStreamSynchronize(s);
      for (cudaStream_t s : {p.cin, p.cst, p.cout})
        if (s) cudaStreamDestroy(s);
      for (auto e : p.events)
        if (e) cudaEventDestroy(e);
      if (start) cudaEventDestroy(start);
    };
    try {
      for (cudaStream_t* s : {&p.cin, &p.cst, &p.cout}) CRG_CHECK_CUDA(cudaStreamCreateWithFlags(s, cudaStreamNonBlocking));
      CRG_CHECK_CUDA(cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
      CRG_CHECK_CUDA(cudaEventRecord(start, st));
      CRG_CHECK_CUDA(cudaStreamWaitEvent(p.cin, start, 0));
      CRG_CHECK_CUDA(cudaStreamWaitEvent(p.cst, start, 0));
      // items are independent: the one with the smallest first chunk in goes
      // first and, of the others, the one with the smallest last chunk out goes
      // last (the pipeline's fill and drain overlap nothing)
      std::vector<int64_t> order(n);
      std::vector<size_t> fill(n), drain(n);
      for (int64_t k = 0; k < n; ++k) {
        order[k] = k;
        host_pipeline_ends(items[k], fill[k], drain[k]);
      }
      const int64_t f = std::min_element(fill.begin(), fill.end()) - fill.begin();
      std::swap(order[0], order[f]);
      int64_t l = 1;
      for (int64_t k = 2; k < n; ++k)
        if (drain[order[k]] < drain[order[l]]) l = k;
      std::swap(order[l], order[n - 1]);
      for (int64_t q = 0; q < n; ++q) {
        const int64_t k = order[q];
        const crg_apply_item& it = items[k];
        try {
          apply_impl(it.regridder, it.transpose, it.dtype, it.adjoint != 0, it.src, it.src_stride_cell,
                     it.src_stride_field, it.dst, it.dst_stride_cell, it.dst_stride_field, it.nfields, it.normalize,
                     p.cst, &p);
        } catch (const Fail&) {
          const std::string m = crg_last_error();
          set_error("item %lld: %s", (long long)k, m.c_str());
          throw;
        }
      }
      CRG_CHECK_CUDA(cudaStreamSynchronize(p.cout));
      CRG_CHECK_CUDA(cudaStreamSynchronize(p.cst));
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
    return;
  }
  cudaEvent_t start = nullptr;
  CRG_CHECK_CUDA(cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
  const cudaError_t er = cudaEventRecord(start, st);
  if (er != cudaSuccess) {
    cudaEventDestroy(start);
    CRG_CHECK_CUDA(er);
  }
  const int workers = (int)std::min<int64_t>(n, nthreads > 0 ? nthreads : 4);
  std::vector<crg_status> status(n, CRG_OK);
  std::vector<std::string> message(n);
  std::vector<cudaEvent_t> done(workers, nullptr);
  std::atomic<int64_t> next{0};
  auto work = [&](int wi) {
    cudaStream_t s = nullptr;
    if (cudaSetDevice(dev) != cudaSuccess || cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamWaitEvent(s, start, 0) != cudaSuccess) {
      for (int64_t k = next.fetch_add(1); k < n; k = next.fetch_add(1)) {
        status[k] = CRG_ERR_CUDA;
        message[k] = "could not set up a stream for an apply worker";
      }
      if (s) cudaStreamDestroy(s);
      return;
    }
    for (int64_t k = next.fetch_add(1); k < n; k = next.fetch_add(1)) {
      const crg_apply_item& it = items[k];
      try {
        apply_impl(it.regridder, it.transpose, it.dtype, it.adjoint != 0, it.src, it.src_stride_cell,
                   it.src_stride_field, it.dst, it.dst_stride_cell, it.dst_stride_field, it.nfields, it.normalize, s);
      } catch (const Fail& e) {
        status[k] = e.st;
        message[k] = crg_last_error();
      } catch (...) {
        status[k] = CRG_ERR_INTERNAL;
        message[k] = "unexpected internal error";
      }
    }
    // the caller's stream continues after this worker's device work
    if (cudaEventCreateWithFlags(&done[wi], cudaEventDisableTiming) == cudaSuccess) cudaEventRecord(done[wi], s);
    cudaStreamDestroy(s);
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < workers; ++t) pool.emplace_back(work, t);
  work(0);  // the calling thread works too
  for (auto& th : pool) th.join();
  cudaEventDestroy(start);
  cudaError_t werr = cudaSuccess;
  for (auto e : done) {
    if (!e) continue;
    const cudaError_t w = cudaStreamWaitEvent(st, e, 0);
    if (werr == cudaSuccess) werr = w;
    cudaEventDestroy(e);
  }
  for (int64_t k = 0; k < n; ++k) {
    if (status[k] != CRG_OK) {
      set_error("item %lld: %s", (long long)k, message[k].c_str());
      throw Fail{status[k]};
    }
  }
  CRG_CHECK_CUDA(werr);
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
  // Items whose own apply cannot fill the GPU run as one persistent launch over
  // all their work units (plus one launch for the rows cut between tasks and
  // the empty rows); the others keep their own, autotuned applies as graph
  // branches beside it.  CRG_PLAN_BATCH=0 captures every item as its own apply,
  // CRG_PLAN_BATCH=all puts every item the persistent launch can run into it.
  std::vector<char> handled((size_t)n, 0);
  BatchLaunch* batch = nullptr;
  const char* pb = getenv("CRG_PLAN_BATCH");
  if (!(pb && strcmp(pb, "0") == 0)) batch = batch_prepare(n, items, handled, pb && strcmp(pb, "all") == 0);
  // Capture: the origin stream forks one branch per remaining item (their
  // outputs are distinct), so the graph runs small items side by side.
  std::vector<cudaStream_t> sts(n + 1, nullptr);  // [n]: the origin (and the batch's launches)
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
      if (k < n && handled[k]) continue;
      CRG_CHECK_CUDA(cudaStreamCreateWithFlags(&sts[k], cudaStreamNonBlocking));
      CRG_CHECK_CUDA(cudaEventCreateWithFlags(&evs[k], cudaEventDisableTiming));
    }
    cudaStream_t origin = sts[n];
    CRG_CHECK_CUDA(cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal));
    try {
      CRG_CHECK_CUDA(cudaEventRecord(evs[n], origin));
      for (int64_t k = 0; k < n; ++k) {
        if (handled[k]) continue;
        const crg_apply_item& it = items[k];
        CRG_CHECK_CUDA(cudaStreamWaitEvent(sts[k], evs[n], 0));
        apply_impl(it.regridder, it.transpose, it.dtype, it.adjoint != 0, it.src, it.src_stride_cell,
                   it.src_stride_field, it.dst, it.dst_stride_cell, it.dst_stride_field, it.nfields, it.normalize,
                   sts[k]);
        CRG_CHECK_CUDA(cudaEventRecord(evs[k], sts[k]));
      }
      if (batch) batch_enqueue(batch, origin);  // beside the items of their own applies
      for (int64_t k = 0; k < n; ++k)  // join the branches
        if (!handled[k]) CRG_CHECK_CUDA(cudaStreamWaitEvent(origin, evs[k], 0));
    } catch (...) {
      cudaStreamEndCapture(origin, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    CRG_CHECK_CUDA(cudaStreamEndCapture(origin, &graph));
  } catch (...) {
    cleanup();
    batch_free(batch);
    throw;
  }
  cleanup();
  size_t nnodes = 0;
  int64_t kernels = 0;
  if (cudaGraphGetNodes(graph, nullptr, &nnodes) == cudaSuccess && nnodes) {
    std::vector<cudaGraphNode_t> nodes(nnodes);
    if (cudaGraphGetNodes(graph, nodes.data(), &nnodes) == cudaSuccess)
      for (size_t q = 0; q < nnodes; ++q) {
        cudaGraphNodeType ty;
        if (cudaGraphNodeGetType(nodes[q], &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) ++kernels;
      }
  }
  crg_apply_plan* p = new crg_apply_plan;
  p->device = dev;
  p->batch = batch;
  p->kernels = kernels;
  for (int64_t k = 0; k < n; ++k) p->batched += batch && handled[k] ? 1 : 0;
  const cudaError_t e = cudaGraphInstantiate(&p->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    batch_free(batch);
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

void apply_plan_info_impl(const crg_apply_plan* p, int64_t* kernels, int64_t* batched_items) {
  CRG_REQUIRE(p != nullptr, CRG_ERR_INVALID_ARGUMENT, "plan is NULL");
  if (kernels) *kernels = p->kernels;
  if (batched_items) *batched_items = p->batched;
}

void apply_plan_destroy_impl(crg_apply_plan* p) {
  if (!p) return;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  batch_free(p->batch);
  for (crg_regridder* r : p->held)
    if (r->refs.fetch_sub(1) == 1) free_regridder(r);
  delete p;
}

}  // namespace crg
