// crg_geom.cuh -- FP64 polygon clipping and area on the GPU.
//
// These are the device counterparts of GeometryOps' ConvexConvexSutherlandHodgman
// clip and spherical/planar `area`, which ConservativeRegridding.jl calls per
// candidate pair in DefaultIntersectionOperator (src/regridder/regridder.jl:96-103)
// and per cell in `areas` (src/regridder/regridder.jl:165-178).
//
// Methods (published, restated here):
//  * Sutherland & Hodgman (1974) clipping of the subject (source cell) by each
//    edge of the convex clip polygon (destination cell).  On the sphere an edge
//    a->b is the great-circle half-space s(x) = n.(x - a) >= 0 with
//    n = a x (b - a) = a x b (sign flipped for clockwise clip polygons);
//    differences are taken first so that short edges keep full relative
//    precision.
//  * crossing of segment a->b with the clip plane: x = |s_a| b + |s_b| a
//    (both weights non-negative, so x lies on the minor arc), then normalised
//    by one reciprocal square root taken as 1 / sqrt and three products.
//  * polygon solid angle: fan from vertex 0; each triangle contributes the
//    complex factor D + iN of Van Oosterom & Strackee (1983),
//    N = a.((b-a) x (c-a)) = a.(b x c), D = 1 + a.b + b.c + c.a; the area is
//    2 arg(prod).  Orientation = sign of the fan sum of N.
//  * arctangent by octant / pi-8 reduction and the Maclaurin series
//    (Abramowitz & Stegun 4.4.42), with a table-chosen number of terms.
//
// Every operation is an IEEE-754 binary64 +,-,*,/,sqrt or an explicit fma in a
// fixed order, and the library is compiled with --fmad=false, so any CPU coding
// of the same sequence compiled without contraction gives identical bits.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define CRG_MAXV 8    // vertices of an input cell
#define CRG_MAXC 24   // capacity of a clipped polygon

namespace crg {

struct d3 { double x, y, z; };

__device__ __forceinline__ double ddot(d3 a, d3 b) { return fma(a.x, b.x, fma(a.y, b.y, a.z * b.z)); }

// Plain products (no fma): a x a and a x 0 are exactly zero.
__device__ __forceinline__ d3 dcross(d3 a, d3 b) {
  d3 r;
  r.x = a.y * b.z - a.z * b.y;
  r.y = a.z * b.x - a.x * b.z;
  r.z = a.x * b.y - a.y * b.x;
  return r;
}

// ---------------------------------------------------------------- exact signs
// Error-free transformations (Shewchuk 1997): TwoProduct via fma, TwoSum, and
// the sign of a sum of doubles from a non-overlapping expansion.  Only taken
// when an FP64 side value lies inside its rounding-error bound.

__device__ __forceinline__ void two_prod(double a, double b, double& p, double& e) {
  p = a * b;
  e = fma(a, b, -p);
}
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  double x = a + b, bv = x - a, av = x - bv;
  e = (a - av) + (b - bv);
  s = x;
}

static __device__ __noinline__ int exact_sign(const double* t, int n) {
  double e[32];
  int m = 0;
  for (int i = 0; i < n; ++i) {
    double q = t[i];
    int k = 0;
    for (int j = 0; j < m; ++j) {
      double sm, h;
      two_sum(q, e[j], sm, h);
      if (h != 0.0) e[k++] = h;
      q = sm;
    }
    if (q != 0.0) e[k++] = q;
    m = k;
  }
  return m == 0 ? 0 : (e[m - 1] > 0.0 ? 1 : -1);
}

__device__ __forceinline__ void prod3(double p, double q, double r, double sg, double* t) {
  double s1, e1;
  two_prod(p, q, s1, e1);
  two_prod(s1, r, t[0], t[1]);
  two_prod(e1, r, t[2], t[3]);
  for (int k = 0; k < 4; ++k) t[k] *= sg;
}

// sign of det[a; b; c] = a.(b x c), exactly
static __device__ __noinline__ int det3_sign(d3 a, d3 b, d3 c) {
  double t[24];
  prod3(a.x, b.y, c.z, 1.0, t + 0);
  prod3(a.x, b.z, c.y, -1.0, t + 4);
  prod3(a.y, b.z, c.x, 1.0, t + 8);
  prod3(a.y, b.x, c.z, -1.0, t + 12);
  prod3(a.z, b.x, c.y, 1.0, t + 16);
  prod3(a.z, b.y, c.x, -1.0, t + 20);
  return exact_sign(t, 24);
}

// p*q - r*w as the double-double s + lo (TwoProduct for both products, TwoSum
// of the heads, the tails added in FP64), and |p*q| + |r*w| for the bound.
// |s + lo - (p*q - r*w)| <= 4 u^2 (|p*q| + |r*w|), u = 2^-53.
__device__ __forceinline__ void minor_dd(double p, double q, double r, double w, double& s, double& lo,
                                         double& perm) {
  double p1, e1, p2, e2, t;
  two_prod(p, q, p1, e1);
  two_prod(r, w, p2, e2);
  two_sum(p1, -p2, s, t);
  lo = t + (e1 - e2);
  perm = fabs(p1) + fabs(p2);
}

// 2^-99 = 128 u^2: four times the worst-case error of det3_sign_adapt's
// double-double value relative to the permanent (< 32 u^2).
constexpr double kDetDD = 1.5777218104420236e-30;
// an absolute floor for bounds: covers rounding of products in the subnormal range
constexpr double kTiny = 1e-290;

// Sign of det[a; b; c] from a double-double evaluation (Dekker 1971 products,
// Shewchuk 1997 adaptive filtering), or 0 when that value cannot decide it.  The
// 2x2 minors of b, c are formed as double-doubles, multiplied by a's components
// with TwoProduct heads and FP64 tails, the three heads summed exactly and the
// eight tail terms (below 5 u perm in all) in FP64, four roundings deep.  The
// value differs from the determinant by at most 3 u^2 perm (minors) + 2 u^2 perm
// (tail products) + 20 u^2 perm (tail sum) + O(u^3), perm = sum_k |a_k|
// (|b_i c_j| + |b_j c_i|): outside 128 u^2 perm (+1e-290 for products in the
// subnormal range) its sign is the determinant's.
__device__ __forceinline__ int det3_sign_dd(d3 a, d3 b, d3 c) {
  double sx, lx, px, sy, ly, py, sz, lz, pz;
  minor_dd(b.y, c.z, b.z, c.y, sx, lx, px);
  minor_dd(b.z, c.x, b.x, c.z, sy, ly, py);
  minor_dd(b.x, c.y, b.y, c.x, sz, lz, pz);
  double hx, ex, hy, ey, hz, ez, s1, r1, s, r2;
  two_prod(a.x, sx, hx, ex);
  two_prod(a.y, sy, hy, ey);
  two_prod(a.z, sz, hz, ez);
  two_sum(hx, hy, s1, r1);
  two_sum(s1, hz, s, r2);
  const double tail = ((r1 + r2) + ((ex + ey) + ez)) + ((a.x * lx + a.y * ly) + a.z * lz);
  const double d = s + tail;
  const double perm = (fabs(a.x) * px + fabs(a.y) * py) + fabs(a.z) * pz;
  if (fabs(d) > kDetDD * perm + kTiny) return d > 0.0 ? 1 : -1;
  return 0;
}

__device__ __forceinline__ bool same_point(d3 p, d3 q) { return p.x == q.x && p.y == q.y && p.z == q.z; }

// The exact sign of det[a; b; c], the same as det3_sign's.  Two equal points
// give 0 at once (a vertex of one grid that is a vertex of the other: most of
// the exact-sign calls between grids that share vertices).  Otherwise the
// double-double filter decides unless the determinant is below 1e-30 of its
// terms (exactly zero, as for three points with one coordinate zero); then the
// error-free expansion does.  The filter costs about a tenth of the expansion
// where points lie on a great circle only up to the rounding of their
// coordinates (meridians of a lon-lat grid through another grid's vertices).
static __device__ __noinline__ int det3_sign_adapt(d3 a, d3 b, d3 c) {
  if (same_point(c, a) || same_point(c, b) || same_point(a, b)) return 0;
  const int s = det3_sign_dd(a, b, c);
  return s != 0 ? s : det3_sign(a, b, c);
}

// sign of (bx-ax)(vy-ay) - (by-ay)(vx-ax), exactly (0 at once for two equal points)
static __device__ __noinline__ int orient2_sign(double ax, double ay, double bx, double by, double vx, double vy) {
  if ((vx == ax && vy == ay) || (vx == bx && vy == by) || (ax == bx && ay == by)) return 0;
  double d[4][2];
  two_sum(bx, -ax, d[0][0], d[0][1]);
  two_sum(vy, -ay, d[1][0], d[1][1]);
  two_sum(by, -ay, d[2][0], d[2][1]);
  two_sum(vx, -ax, d[3][0], d[3][1]);
  double t[16];
  int n = 0;
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      two_prod(d[0][i], d[1][j], t[n], t[n + 1]);
      n += 2;
    }
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      two_prod(d[2][i], d[3][j], t[n], t[n + 1]);
      t[n] = -t[n];
      t[n + 1] = -t[n + 1];
      n += 2;
    }
  return exact_sign(t, 16);
}

constexpr double kU32 = 3.552713678800501e-15;  // 32 * 2^-53
constexpr double kU8 = 8.881784197001252e-16;   // 8 * 2^-53

__device__ __forceinline__ double settle(double s, double bound, int sg) {
  if (fabs(s) > bound) return s;
  if (sg == 0) return 0.0;
  double m = fmax(fabs(s), 2.2250738585072014e-308);
  return sg > 0 ? m : -m;
}

static __constant__ double kAtanC[20] = {
    1.0, 0.3333333333333333, 0.2, 0.14285714285714285, 0.1111111111111111,
    0.09090909090909091, 0.07692307692307693, 0.06666666666666667, 0.058823529411764705,
    0.05263157894736842, 0.047619047619047616, 0.043478260869565216, 0.04,
    0.037037037037037035, 0.034482758620689655, 0.03225806451612903, 0.030303030303030304,
    0.02857142857142857, 0.02702702702702703, 0.02564102564102564};
// kAtanTh[n]: the largest t^2 for which terms k = 0..n reach 2^-56 relative accuracy.
static __constant__ double kAtanTh[20] = {
    4.163336342344337e-17, 8.33000234328132e-09, 4.596981552458248e-06, 0.0001057159916729051,
    0.0006866613224549, 0.0023770807360687612, 0.005751393360079481, 0.011132588223807069,
    0.018578395538006495, 0.02795464321653044, 0.039019086539122956, 0.051485905388814555,
    0.06506692879763946, 0.07949448812181649, 0.09453198900334307, 0.10997706781109234,
    0.12566065265206888, 0.1414440078610017, 0.15721498531213599, 0.17288416032961332};

constexpr double kTanPi8 = 0.41421356237309503;
constexpr double kPi4 = 0.7853981633974483;
constexpr double kPi2 = 1.5707963267948966;
constexpr double kPi = 3.141592653589793;

__device__ __forceinline__ double atan_series(double t) {
  double z = t * t;
  int n = 0;
  while (n < 19 && z > kAtanTh[n]) n++;
  double p = kAtanC[n];
  for (int k = n - 1; k >= 0; --k) p = fma(p, -z, kAtanC[k]);
  return t * p;
}

__device__ __forceinline__ double atan2_crg(double y, double x) {
  double ay = fabs(y), ax = fabs(x);
  bool swap = ay > ax;
  double num = swap ? ax : ay, den = swap ? ay : ax;
  if (den == 0.0) return 0.0;
  double t = num / den;
  double r;
  if (t > kTanPi8) {
    double u = (t - 1.0) / (t + 1.0);
    r = kPi4 + atan_series(u);
  } else {
    r = atan_series(t);
  }
  if (swap) r = kPi2 - r;
  if (x < 0.0) r = kPi - r;
  if (y < 0.0) r = -r;
  return r;
}

// ---------------------------------------------------------------- sphere

__device__ __forceinline__ d3 dsub(d3 a, d3 b) { return d3{a.x - b.x, a.y - b.y, a.z - b.z}; }

// a.((b-a) x (c-a)) = a.(b x c) in the frame of a (full relative precision for tiny triangles)
__device__ __forceinline__ double triple(d3 a, d3 b, d3 c) { return ddot(a, dcross(dsub(b, a), dsub(c, a))); }

// sign of the fan sum of triple products: +1 counter-clockwise seen from outside
__device__ __forceinline__ double orient_sph(const d3* c, int n) {
  double s = 0.0;
  for (int k = 1; k + 1 < n; ++k) s = s + triple(c[0], c[k], c[k + 1]);
  return s >= 0.0 ? 1.0 : -1.0;
}

// Side of v w.r.t. the great circle ca -> cb: FP64 n.(v - ca) with
// n = ca x (cb - ca) pre-signed by the clip orientation; exact sign inside the
// error bound eb * |v - ca|_1.
__device__ __forceinline__ double side_sph(d3 nrm, d3 ca, d3 cb, double eb, int isig, d3 v) {
  d3 w = dsub(v, ca);
  double s = ddot(nrm, w);
  double bound = eb * (fabs(w.x) + fabs(w.y) + fabs(w.z)) + kTiny;
  if (fabs(s) > bound) return s;
  return settle(s, bound, isig * det3_sign_adapt(ca, cb, v));
}

// Crossing weights below 2^-400 are scaled by 2^600 (exactly) before they are
// combined.  They come from side values the exact sign settled to about
// DBL_MIN at both ends of an edge; unscaled, the squared norm of the combination
// underflows to 0 and the crossing point becomes infinite.  The normalisation
// removes the factor, and weights from 2^-400 up take the unscaled sequence.
constexpr double kIsectTiny = 0x1p-400, kIsectScale = 0x1p600;

// A vertex exactly on the clip line is passed through unchanged.
__device__ __forceinline__ d3 isect_sph(d3 a, double sa, d3 b, double sb) {
  if (sa == 0.0) return a;
  if (sb == 0.0) return b;
  double wa = fabs(sb), wb = fabs(sa);
  if (fmax(wa, wb) < kIsectTiny) {
    wa *= kIsectScale;
    wb *= kIsectScale;
  }
  d3 x;
  x.x = fma(wb, b.x, wa * a.x);
  x.y = fma(wb, b.y, wa * a.y);
  x.z = fma(wb, b.z, wa * a.z);
  // one reciprocal and three products: FP64 division is a long instruction sequence
  const double ir = 1.0 / sqrt(ddot(x, x));
  x.x = x.x * ir; x.y = x.y * ir; x.z = x.z * ir;
  return x;
}

// Signed solid angle of polygon v[0..m) (fan from v[0]).  Consecutive fan
// triangles share c - a and a.c (the next triangle's b - a and a.b): each is
// computed once, with the values triple() and ddot() give.
__device__ __forceinline__ double area_sph_signed(const d3* v, int m) {
  if (m < 3) return 0.0;
  double re = 1.0, im = 0.0;
  const d3 a = v[0];
  d3 db = dsub(v[1], a);
  double ab = ddot(a, v[1]);
  for (int k = 1; k + 1 < m; ++k) {
    const d3 b = v[k], c = v[k + 1];
    const d3 dc = dsub(c, a);
    const double N = ddot(a, dcross(db, dc));
    const double ac = ddot(c, a);
    const double D = ((1.0 + ab) + ddot(b, c)) + ac;
    const double re2 = fma(re, D, -(im * N));
    const double im2 = fma(re, N, im * D);
    re = re2; im = im2;
    db = dc;
    ab = ac;  // ddot(a, c) == ddot(c, a): the products commute exactly
  }
  return 2.0 * atan2_crg(im, re);
}

// area_sph_signed and orient_sph of the same polygon from one pass over the
// fan (the triple products are shared; the values are the same).
__device__ __forceinline__ double area_orient_sph(const d3* v, int m, double& ori) {
  double re = 1.0, im = 0.0, s = 0.0;
  const d3 a = v[0];
  d3 db = m > 1 ? dsub(v[1], a) : d3{0.0, 0.0, 0.0};
  double ab = m > 1 ? ddot(a, v[1]) : 0.0;
  for (int k = 1; k + 1 < m; ++k) {
    const d3 b = v[k], c = v[k + 1];
    const d3 dc = dsub(c, a);
    const double N = ddot(a, dcross(db, dc));
    s = s + N;
    const double ac = ddot(c, a);
    const double D = ((1.0 + ab) + ddot(b, c)) + ac;
    const double re2 = fma(re, D, -(im * N));
    const double im2 = fma(re, N, im * D);
    re = re2; im = im2;
    db = dc;
    ab = ac;
  }
  ori = s >= 0.0 ? 1.0 : -1.0;
  return m < 3 ? 0.0 : 2.0 * atan2_crg(im, re);
}

// ---------------------------------------------------------------- plane

__device__ __forceinline__ double cross2(double ax, double ay, double bx, double by) { return ax * by - ay * bx; }

// shoelace formula relative to v[0]
__device__ __forceinline__ double area_pl_signed(const d3* v, int m) {
  if (m < 3) return 0.0;
  double s = 0.0;
  for (int k = 1; k + 1 < m; ++k)
    s = s + cross2(v[k].x - v[0].x, v[k].y - v[0].y, v[k + 1].x - v[0].x, v[k + 1].y - v[0].y);
  return 0.5 * s;
}

__device__ __forceinline__ double orient_pl(const d3* c, int n) { return area_pl_signed(c, n) >= 0.0 ? 1.0 : -1.0; }

__device__ __forceinline__ double side_pl(d3 a, d3 b, double ex, double ey, int isig, d3 v) {
  double wx = v.x - a.x, wy = v.y - a.y;
  double s = cross2(ex, ey, wx, wy);
  if (isig < 0) s = -s;
  double bound = kU8 * (fabs(ex) * fabs(wy) + fabs(ey) * fabs(wx)) + kTiny;
  if (fabs(s) > bound) return s;
  return settle(s, bound, isig * orient2_sign(a.x, a.y, b.x, b.y, v.x, v.y));
}

__device__ __forceinline__ d3 isect_pl(d3 a, double sa, d3 b, double sb) {
  if (sa == 0.0) return a;
  if (sb == 0.0) return b;
  double wa = fabs(sb), wb = fabs(sa);
  if (fmax(wa, wb) < kIsectTiny) {  // as in isect_sph: the products would lose their bits
    wa *= kIsectScale;
    wb *= kIsectScale;
  }
  double w = wa + wb;
  d3 x;
  x.x = fma(wb, b.x, wa * a.x) / w;
  x.y = fma(wb, b.y, wa * a.y) / w;
  x.z = 0.0;
  return x;
}

// ---------------------------------------------------------------- clip

// Sutherland-Hodgman clip of `subj` (ns vertices, copied into buf A) by the
// convex polygon `clip` (nc vertices) of orientation `sig` (+1 / -1).  Ping-pongs between bufA and bufB;
// returns the vertex count and sets *res to the buffer holding the result, or
// returns -1 if a stage would exceed CRG_MAXC vertices.
// Great-circle half-space of the clip edge ca -> cb of a polygon of
// orientation sig: n = ca x (cb - ca) (negated when clockwise) and the error
// bound factor of n.(v - ca).
__device__ __forceinline__ void edge_plane(d3 ca, d3 cb, double sig, d3& nrm, double& eb) {
  d3 d1 = dsub(cb, ca);
  nrm = dcross(ca, d1);
  if (sig < 0.0) { nrm.x = -nrm.x; nrm.y = -nrm.y; nrm.z = -nrm.z; }
  eb = kU32 * (fabs(ca.x) + fabs(ca.y) + fabs(ca.z)) * (fabs(d1.x) + fabs(d1.y) + fabs(d1.z));
}

// FP32 inputs of the side screening, rounded once instead of per test: the
// clip edges' normals (w = |n32|_1) and start vertices, and the subject
// polygon beside its FP64 copy (a and b ping-pong with bufA and bufB; a holds
// the subject's vertices on entry).  Every value equals the rounding of the
// FP64 value it stands for, so the decisions are those of converting in place.
struct Screen32 {
  const float4* planes;
  const float4* clip;
  float4* a;
  float4* b;
};

// `planes`, when given (spherical only), holds edge_plane of every clip edge
// (x, y, z = n, w = eb), computed once per clip polygon; `s32`, when given
// (spherical only), the FP32 screening inputs.
template <bool kSpherical>
__device__ __forceinline__ int clip_polygon_oriented(d3* bufA, d3* bufB, int ns, const d3* clip, int nc, double sig,
                                                     d3** res, const double4_32a* planes = nullptr,
                                                     const Screen32* s32 = nullptr) {
  d3* in = bufA;
  d3* out = bufB;
  float4* in32 = s32 ? s32->a : nullptr;
  float4* out32 = s32 ? s32->b : nullptr;
  int n = ns;
  for (int k = 0; k < nc && n > 0; ++k) {
    d3 ca = clip[k], cb = clip[k + 1 == nc ? 0 : k + 1];
    const int isig = sig < 0.0 ? -1 : 1;
    d3 nrm{0.0, 0.0, 0.0};
    double ex = 0.0, ey = 0.0, eb = 0.0;
    if (kSpherical) {
      // half-space of edge ca -> cb: n = ca x (cb - ca), s(v) = n.(v - ca)
      if (planes) {
        const double4_32a p = planes[k];
        nrm = d3{p.x, p.y, p.z};
        eb = p.w;
      } else {
        edge_plane(ca, cb, sig, nrm, eb);
      }
    } else {
      ex = cb.x - ca.x; ey = cb.y - ca.y;
    }
    // The stage in three passes that emit exactly the vertex sequence of the
    // one-pass loop (edge i runs from vertex i-1 to vertex i): the sides of
    // all vertices, then the crossing points -- two for a convex polygon,
    // computed in fixed slots so the lanes of a warp run them together --
    // then the output sequence.
    //
    // On the sphere a side is first decided in FP32: with n32, w32 = v32 - ca32
    // rounded from the FP64 plane and unit vectors, |s32 - n.(v - ca)| stays
    // below 2^-21 |n32|_1 (1 + |w32|_inf), so |s32| > B = 2^-18 |n32|_1
    // (1 + |w32|_1) gives the exact sign with an 8x margin.  The FP64 side
    // (with its exact-sign fallback) is taken only where that test is
    // undecided and for the endpoints of the crossing edges, whose values
    // weight the crossing points: decisions and values are those of the
    // one-pass loop.
    double sv[CRG_MAXC];
    uint32_t inside = 0u, known = 0u;  // bit i: vertex i inside; sv[i] computed
    if (kSpherical) {
      float nx, ny, nz, n1, ax, ay, az;
      if (s32) {
        const float4 p = s32->planes[k], c = s32->clip[k];
        nx = p.x; ny = p.y; nz = p.z; n1 = p.w;
        ax = c.x; ay = c.y; az = c.z;
      } else {
        nx = (float)nrm.x; ny = (float)nrm.y; nz = (float)nrm.z;
        ax = (float)ca.x; ay = (float)ca.y; az = (float)ca.z;
        n1 = fabsf(nx) + fabsf(ny) + fabsf(nz);
      }
      for (int i = 0; i < n; ++i) {
        float vx, vy, vz;
        if (s32) {
          const float4 u = in32[i];
          vx = u.x; vy = u.y; vz = u.z;
        } else {
          vx = (float)in[i].x; vy = (float)in[i].y; vz = (float)in[i].z;
        }
        const float wx = vx - ax, wy = vy - ay, wz = vz - az;
        const float s32 = fmaf(nx, wx, fmaf(ny, wy, nz * wz));
        const float B = 3.814697265625e-06f * n1 * (1.0f + fabsf(wx) + fabsf(wy) + fabsf(wz));  // 2^-18
        if (s32 > B) {
          inside |= 1u << i;
        } else if (!(s32 < -B)) {
          sv[i] = side_sph(nrm, ca, cb, eb, isig, in[i]);
          known |= 1u << i;
          if (sv[i] >= 0.0) inside |= 1u << i;
        }
      }
    } else {
      for (int i = 0; i < n; ++i) {
        sv[i] = side_pl(ca, cb, ex, ey, isig, in[i]);
        known |= 1u << i;
        if (sv[i] >= 0.0) inside |= 1u << i;
      }
    }
    const int nin = __popc(inside);
    if (nin == n) continue;  // all inside: the stage returns the polygon unchanged
    if (nin == 0) {
      n = 0;
      break;
    }
    // FP64 side values where the crossing points need them.  A vertex the FP32
    // test decided is at least 0.8 B from the plane, far outside the FP64
    // bound, where side_sph returns the plain value n.(v - ca): that is taken
    // directly.
    auto side = [&](int i) -> double {
      if (!((known >> i) & 1u)) {
        sv[i] = kSpherical ? ddot(nrm, dsub(in[i], ca)) : side_pl(ca, cb, ex, ey, isig, in[i]);
        known |= 1u << i;
      }
      return sv[i];
    };
    auto isin = [&](int i) { return ((inside >> i) & 1u) != 0u; };
    int e0 = -1, e1 = -1, ncross = 0;
    for (int i = 0; i < n; ++i) {
      const int p = i == 0 ? n - 1 : i - 1;
      if (isin(i) != isin(p)) {
        if (ncross == 0) e0 = i;
        else e1 = i;
        ++ncross;
      }
    }
    d3 x0{0.0, 0.0, 0.0}, x1{0.0, 0.0, 0.0};
    if (ncross == 2) {
      const int p0 = e0 == 0 ? n - 1 : e0 - 1, p1 = e1 == 0 ? n - 1 : e1 - 1;
      const double s_p0 = side(p0), s_e0 = side(e0), s_p1 = side(p1), s_e1 = side(e1);
      x0 = kSpherical ? isect_sph(in[p0], s_p0, in[e0], s_e0) : isect_pl(in[p0], s_p0, in[e0], s_e0);
      x1 = kSpherical ? isect_sph(in[p1], s_p1, in[e1], s_e1) : isect_pl(in[p1], s_p1, in[e1], s_e1);
    }
    int m = 0;
    for (int i = 0; i < n; ++i) {
      const int p = i == 0 ? n - 1 : i - 1;
      const bool ci = isin(i), pi = isin(p);
      if (ci == pi) {
        if (ci) {
          if (m >= CRG_MAXC) return -1;
          if (s32) out32[m] = in32[i];
          out[m++] = in[i];
        }
        continue;
      }
      // a crossing edge (more than two only for non-convex input: computed here)
      d3 x;
      if (ncross == 2) {
        x = i == e0 ? x0 : x1;
      } else {
        const double sp = side(p), sc = side(i);
        x = kSpherical ? isect_sph(in[p], sp, in[i], sc) : isect_pl(in[p], sp, in[i], sc);
      }
      if (m >= CRG_MAXC) return -1;
      if (s32) out32[m] = make_float4((float)x.x, (float)x.y, (float)x.z, 0.f);
      out[m++] = x;
      if (ci) {
        if (m >= CRG_MAXC) return -1;
        if (s32) out32[m] = in32[i];
        out[m++] = in[i];
      }
    }
    d3* t = in; in = out; out = t;
    float4* t32 = in32; in32 = out32; out32 = t32;
    n = m;
  }
  *res = in;
  return n;
}

// clip_polygon_oriented with the clip polygon's orientation computed here
template <bool kSpherical>
__device__ __forceinline__ int clip_polygon(d3* bufA, d3* bufB, int ns, const d3* clip, int nc, d3** res) {
  const double sig = kSpherical ? orient_sph(clip, nc) : orient_pl(clip, nc);
  return clip_polygon_oriented<kSpherical>(bufA, bufB, ns, clip, nc, sig, res);
}

template <bool kSpherical>
__device__ __forceinline__ double cell_area(const d3* v, int n) {
  if (kSpherical) return area_sph_signed(v, n) * orient_sph(v, n);
  return area_pl_signed(v, n) * orient_pl(v, n);
}

}  // namespace crg
