// crg_div.cuh -- correctly rounded quotients by a per-row divisor.
//
// regrid! divides every output element of a row by the row's area
// (src/regridder/regrid.jl:95-118: mul! then ./ a_d).  Bit parity with that
// needs the IEEE quotient, and an FP64 division issues eight FP64-pipe
// instructions per element on GB300 -- as many as four entries' products and
// sums.  When a row's divisor d serves several fields, its reciprocal is taken
// once (rcp = RN(1/d)) and each quotient comes from Markstein's correction
// (P. Markstein, IBM J. Res. Dev. 34(1), 1990):
//   q0 = RN(a * rcp),  e = a - q0 d (exact with fma),  q1 = RN(q0 + e rcp),
// followed by a check that q1 is RN(a/d): the exact residual r1 = a - q1 d
// (exact with fma when q1 is within an ulp of a/d) is below half an ulp of q1
// times |d|, strictly, and q1 is a normal number that is not a power of two
// (whose lower neighbour is half an ulp closer).  A quotient that fails the
// check (zeros, subnormals, powers of two, a residual near underflow, or a
// quotient not within half an ulp) takes the IEEE division in a separate,
// non-inlined function, so that the common path does not carry the division's
// instructions predicated off.  Either way the result is the IEEE quotient.
// Four FP64 instructions replace the division on the fast path; the check is
// integer arithmetic on the bit patterns.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace crg {

static __device__ __noinline__ double div_rn_slow(double a, double d) { return __ddiv_rn(a, d); }

// RN(a / d), given rcp = RN(1 / d).
__device__ __forceinline__ double div_rn_by(double a, double d, double rcp) {
  const double q0 = a * rcp;
  const double e = fma(-q0, d, a);
  const double q1 = fma(e, rcp, q0);
  const double r1 = fma(-q1, d, a);
  const uint64_t qb = (uint64_t)__double_as_longlong(q1);
  const uint64_t db = (uint64_t)__double_as_longlong(d) & 0x7fffffffffffffffull;
  const int eq = (int)((qb >> 52) & 0x7ff);
  const int ed = (int)(db >> 52);
  // half an ulp of q1 times |d|: |d| with its exponent moved by (eq - 1023) - 53
  const int eh = ed + eq - 1076;
  const bool normal = eq >= 1 && eq <= 2046 && ed >= 1 && ed <= 2046 && (qb & 0x000fffffffffffffull) != 0;
  const bool room = eh >= 60 && eh <= 2046;  // the half-ulp bound and the residual far from underflow
  const uint64_t hb = (db & 0x000fffffffffffffull) | ((uint64_t)(room ? eh : 1) << 52);
  const uint64_t rb = (uint64_t)__double_as_longlong(r1) & 0x7fffffffffffffffull;
  // non-negative doubles order as their bit patterns
  if (normal && room && rb < hb) return q1;
  return div_rn_slow(a, d);
}

}  // namespace crg
