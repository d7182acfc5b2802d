// Test helper: the clip's exact-sign predicates evaluated on the GPU for a
// batch of point triples, so that tests can compare them with rational
// arithmetic.  Built by tests/test_gpu_predicates.py into a temporary folder.
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
