// Test helper: the clip's exact-sign predicates and the FP64 apply's
// corrected quotients evaluated on the GPU for batches of inputs, so that
// tests can compare them with rational arithmetic and with IEEE division.
// Built by tests/test_gpu_predicates.py into a temporary folder.
#include "crg_div.cuh"
#include "crg_geom.cuh"

namespace {
__global__ void k_det3(const double* p, int n, int* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* q = p + 9 * i;
  const crg::d3 a{q[0], q[1], q[2]}, b{q[3], q[4], q[5]}, c{q[6], q[7], q[8]};
  out[3 * i] = crg::det3_sign_adapt(a, b, c);
  out[3 * i + 1] = crg::det3_sign_dd(a, b, c);
  out[3 * i + 2] = crg::det3_sign(a, b, c);
}

__global__ void k_div(const double* a, const double* d, int n, double* fast, double* ieee) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  fast[i] = crg::div_rn_by(a[i], d[i], __drcp_rn(d[i]));
  ieee[i] = __ddiv_rn(a[i], d[i]);
}
}  // namespace

// abc: n triples (a, b, c) of 3-vectors, 9 doubles each, in host memory.
// out: 3 ints per triple: the clip's sign, the double-double filter's sign (0 when
// it cannot decide) and the error-free expansion's sign.  Returns a cudaError_t.
extern "C" int crg_test_det3(const double* abc, int n, int* out) {
  double* d = nullptr;
  int* o = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(double) * 9 * (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc(&o, sizeof(int) * 3 * (size_t)n);
  if (e == cudaSuccess) e = cudaMemcpy(d, abc, sizeof(double) * 9 * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && n > 0) {
    k_det3<<<(n + 127) / 128, 128>>>(d, n, o);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, o, sizeof(int) * 3 * (size_t)n, cudaMemcpyDeviceToHost);
  cudaFree(d);
  cudaFree(o);
  return (int)e;
}

// a, d: n dividends and divisors in host memory.  fast: div_rn_by(a, d, RN(1/d));
// ieee: the IEEE quotient.  Returns a cudaError_t.
extern "C" int crg_test_div(const double* a, const double* d, int n, double* fast, double* ieee) {
  double* buf = nullptr;
  const size_t b = sizeof(double) * (size_t)n;
  cudaError_t e = cudaMalloc(&buf, 4 * b + 16);
  if (e == cudaSuccess) e = cudaMemcpy(buf, a, b, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(buf + n, d, b, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && n > 0) {
    k_div<<<(n + 127) / 128, 128>>>(buf, buf + n, n, buf + 2 * (size_t)n, buf + 3 * (size_t)n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(fast, buf + 2 * (size_t)n, b, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(ieee, buf + 3 * (size_t)n, b, cudaMemcpyDeviceToHost);
  cudaFree(buf);
  return (int)e;
}
