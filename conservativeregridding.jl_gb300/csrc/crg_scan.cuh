// crg_scan.cuh -- device exclusive prefix sums and small reductions used by the
// build (counting sorts, CSR/CSC row pointers).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace crg {

// Exclusive scan of int32 counts `in[0..n)` into `out[0..n]` (out[n] = total),
// on `st`.  `in` and `out` may alias.  Uses a stream-ordered temporary.
void exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, cudaStream_t st);

}  // namespace crg
