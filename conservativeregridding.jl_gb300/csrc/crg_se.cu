// crg_se.cu -- regridders between a spectral-element (SE) space and a
// finite-volume (FV) grid on the sphere: the ClimaCore extension of the
// reference (ext/ConservativeRegriddingClimaCoreExt.jl).
//
//   SE -> FV, principled weights   se_to_fv_principled :416-486,
//                                  accumulate_principled_b :260-305
//   FV -> SE, L2 projection        fv_to_se_l2_projection :573-689,
//                                  compute_local_mass_matrix :522-560,
//                                  element_jacobian_at :221-237
//   node positions / weights       se_node_positions / se_node_weights :139-156
//   weighted DSS of the result     finalize_regridding! :709-715
//
// Element geometry.  Element e with corners c1..c4 (unit vectors, at the
// reference corners (-1,-1), (1,-1), (1,1), (-1,1)) maps (xi, eta) to
// X / |X| with the bilinear X = a + b xi + c eta + d xi eta,
//   a = (c1 + c2 + c3 + c4) / 4,  b = (-c1 + c2 + c3 - c4) / 4,
//   c = (-c1 - c2 + c3 + c4) / 4, d = (c1 - c2 + c3 - c4) / 4
// (the normalised bilinear element map; its edges are great-circle arcs, so
// the element is the quadrilateral the candidate search and the clip see).
// Inverse map: X(xi, eta) is parallel to the vector x exactly when
// X.(x x c) = 0 and X.(x x b) = 0, i.e.
//   A1 + B1 xi + D1 xi eta = 0,   A2 - B1 eta + D2 xi eta = 0
// with A1 = x.(c x a), B1 = x.(c x b), D1 = x.(c x d), A2 = x.(b x a),
// D2 = x.(b x d).  Eliminating xi gives the quadratic
//   (-B1 D1) eta^2 + (A2 D1 - B1^2 - D2 A1) eta + A2 B1 = 0,
// whose small root (the one in [-1, 1]) is taken in the cancellation-free
// form eta = -2 c0 / (b0 + sign(b0) sqrt(b0^2 - 4 a0 c0)); then
// xi = -A1 / (B1 + D1 eta).  Area element of the map on the unit sphere:
// J = |X.(X_xi x X_eta)| / |X|^3.
//
// Quadrature.  GLL nodes: Newton's method on f = x P_N - P_(N-1) (whose
// roots are +-1 and the zeros of P_N'; f' = (N + 1) P_N), started at the
// Chebyshev-Gauss-Lobatto points, weights 2 / (N (N + 1) P_N(x)^2).  Lagrange
// basis in product form phi_j(t) = c_j prod_(m != j) (t - x_m).  Triangle
// rules: Dunavant (1985), "High degree efficient symmetrical Gaussian
// quadrature rules for the triangle", degrees 1..8, as the reference's
// src/regridder/triangle_quadrature.jl selects them.
//
// Every floating-point operation here has a fixed order (explicit fma where
// used, no contraction), so the oracle's C restatement reproduces the
// matrices bit for bit.
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "crg_geom.cuh"
#include "crg_internal.cuh"
#include "crg_scan.cuh"

namespace crg {

namespace {

constexpr int kSeMaxNq = 8;
constexpr int kSeMaxTri = 16;   // points of the degree-8 rule
constexpr int kSeMaxMass = 12;  // GLL points of the mass rule for nq = 8
constexpr int kSeCoef = 27;     // a, b, c, d, c x a, c x b, c x d, b x a, b x d

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

struct SeRule {
  int nq = 0, ntri = 0;
  double x[kSeMaxNq];         // GLL nodes on [-1, 1]
  double w[kSeMaxNq];         // GLL weights
  double c[kSeMaxNq];         // 1 / prod_(m != j) (x_j - x_m)
  double tl[kSeMaxTri][3];    // triangle rule points (barycentric)
  double tw[kSeMaxTri];       // triangle rule weights (summing to 1)
};

struct SeMass {
  int nm = 0;
  double w[kSeMaxMass];               // GLL weights of the mass rule
  double L[kSeMaxMass][kSeMaxNq];     // L[p][a] = phi_a at mass point p
};

// ------------------------------------------------------------------ host rules

// Legendre P_N and P_(N-1) at t by the three-term recurrence.
void legendre2(int N, double t, double* pn, double* pn1) {
  double p0 = 1.0, p1 = t;
  for (int k = 2; k <= N; ++k) {
    const double p2 = ((double)(2 * k - 1) * t * p1 - (double)(k - 1) * p0) / (double)k;
    p0 = p1;
    p1 = p2;
  }
  *pn = p1;
  *pn1 = p0;
}

void gll_points(int n, double* x, double* w) {
  const int N = n - 1;
  for (int i = 0; i <= N; ++i) x[i] = -cos(3.14159265358979323846 * (double)i / (double)N);
  for (int it = 0; it < 100; ++it) {
    double dmax = 0.0;
    for (int i = 0; i <= N; ++i) {
      double pn, pn1;
      legendre2(N, x[i], &pn, &pn1);
      const double dx = (x[i] * pn - pn1) / ((double)n * pn);
      x[i] = x[i] - dx;
      dmax = std::max(dmax, fabs(dx));
    }
    if (dmax <= 1e-15) break;
  }
  x[0] = -1.0;
  x[N] = 1.0;
  for (int i = 0; i < n / 2; ++i) x[N - i] = -x[i];
  if (n % 2) x[N / 2] = 0.0;
  for (int i = 0; i <= N; ++i) {
    double pn, pn1;
    legendre2(N, x[i], &pn, &pn1);
    w[i] = 2.0 / ((double)(N * n) * (pn * pn));
  }
}

void lagrange_host(int nq, const double* x, const double* c, double t, double* phi) {
  double d[kSeMaxNq], suf[kSeMaxNq];
  for (int m = 0; m < nq; ++m) d[m] = t - x[m];
  suf[nq - 1] = 1.0;
  for (int j = nq - 1; j > 0; --j) suf[j - 1] = suf[j] * d[j];
  double pre = 1.0;
  for (int j = 0; j < nq; ++j) {
    phi[j] = (pre * suf[j]) * c[j];
    pre = pre * d[j];
  }
}

// Dunavant (1985) rules as symmetry orbits, weights normalised to sum 1:
// kind 0 the centroid, kind 1 the permutations of (a, b, b), kind 2 those of (a, b, c).
struct Orbit {
  int degree, kind;
  double w, a, b, c;
};

std::vector<Orbit> dunavant_orbits() {
  const double s15 = sqrt(15.0);
  const double b5p = (6.0 + s15) / 21.0, b5m = (6.0 - s15) / 21.0;
  return {
      {1, 0, 1.0, 0, 0, 0},
      {2, 1, 1.0 / 3.0, 2.0 / 3.0, 1.0 / 6.0, 0},
      {3, 0, -27.0 / 48.0, 0, 0, 0},
      {3, 1, 25.0 / 48.0, 0.6, 0.2, 0},
      {4, 1, 0.223381589678011, 0.108103018168070, 0.445948490915965, 0},
      {4, 1, 0.109951743655322, 0.816847572980459, 0.091576213509771, 0},
      {5, 0, 0.225, 0, 0, 0},
      {5, 1, (155.0 + s15) / 1200.0, 1.0 - 2.0 * b5p, b5p, 0},
      {5, 1, (155.0 - s15) / 1200.0, 1.0 - 2.0 * b5m, b5m, 0},
      {6, 1, 0.116786275726379, 0.501426509658179, 0.249286745170910, 0},
      {6, 1, 0.050844906370207, 0.873821971016996, 0.063089014491502, 0},
      {6, 2, 0.082851075618374, 0.053145049844817, 0.310352451033784, 0.636502499121399},
      {7, 0, -0.149570044467682, 0, 0, 0},
      {7, 1, 0.175615257433208, 0.479308067841920, 0.260345966079040, 0},
      {7, 1, 0.053347235608838, 0.869739794195568, 0.065130102902216, 0},
      {7, 2, 0.077113760890257, 0.048690315425316, 0.312865496004874, 0.638444188569810},
      {8, 0, 0.144315607677787, 0, 0, 0},
      {8, 1, 0.095091634267285, 0.081414823414554, 0.459292588292723, 0},
      {8, 1, 0.103217370534718, 0.658861384496480, 0.170569307751760, 0},
      {8, 1, 0.032458497623198, 0.898905543365938, 0.050547228317031, 0},
      {8, 2, 0.027230314174435, 0.008394777409958, 0.263112829634638, 0.728492392955404},
  };
}

// reference_rule(degree) (src/regridder/triangle_quadrature.jl:159-167): the
// rule of that degree, degrees below 1 take the degree-1 rule, above 8 fail.
int triangle_rule(int degree, double (*tl)[3], double* tw) {
  const int d = degree < 1 ? 1 : degree;
  CRG_REQUIRE(d <= 8, CRG_ERR_INVALID_ARGUMENT, "Triangle quadrature degree %d not available (max is 8).", degree);
  int n = 0;
  auto put = [&](double w, double l0, double l1, double l2) {
    tl[n][0] = l0; tl[n][1] = l1; tl[n][2] = l2;
    tw[n] = w;
    ++n;
  };
  for (const Orbit& o : dunavant_orbits()) {
    if (o.degree != d) continue;
    const double third = 1.0 / 3.0;
    if (o.kind == 0) {
      put(o.w, third, third, third);
    } else if (o.kind == 1) {
      put(o.w, o.a, o.b, o.b); put(o.w, o.b, o.a, o.b); put(o.w, o.b, o.b, o.a);
    } else {
      put(o.w, o.a, o.b, o.c); put(o.w, o.a, o.c, o.b); put(o.w, o.b, o.a, o.c);
      put(o.w, o.b, o.c, o.a); put(o.w, o.c, o.a, o.b); put(o.w, o.c, o.b, o.a);
    }
  }
  return n;
}

SeRule make_rule(int nq, int degree) {
  SeRule r;
  r.nq = nq;
  gll_points(nq, r.x, r.w);
  for (int j = 0; j < nq; ++j) {
    double prod = 1.0;
    for (int m = 0; m < nq; ++m)
      if (m != j) prod = prod * (r.x[j] - r.x[m]);
    r.c[j] = 1.0 / prod;
  }
  r.ntri = triangle_rule(degree, r.tl, r.tw);
  return r;
}

// GLL rule exact for the mass-matrix integrand of bidegree 3 (nq - 1):
// n = ceil((3 nq - 2) / 2) + 1 points (compute_local_mass_matrix :530-532).
SeMass make_mass(const SeRule& r) {
  SeMass m;
  m.nm = (3 * r.nq - 2 + 1) / 2 + 1;
  double x[kSeMaxMass];
  gll_points(m.nm, x, m.w);
  for (int p = 0; p < m.nm; ++p) lagrange_host(r.nq, r.x, r.c, x[p], m.L[p]);
  return m;
}

// ------------------------------------------------------------------ device geometry

__device__ __forceinline__ d3 ld3(const double* p) { return d3{p[0], p[1], p[2]}; }

// Element coefficients (a, b, c, d and the five cross products of the inverse map).
__global__ void k_se_coeffs(const double* __restrict__ v, const int8_t* __restrict__ nv, int maxv, int64_t nelem,
                            double* __restrict__ coef, int* __restrict__ bad) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nelem) return;
  if (nv[e] != 4) {
    atomicAdd(bad, 1);
    return;
  }
  const double* q = v + e * maxv * 3;
  const d3 c1 = ld3(q), c2 = ld3(q + 3), c3 = ld3(q + 6), c4 = ld3(q + 9);
  d3 a, b, c, d;
  a.x = 0.25 * ((c1.x + c2.x) + (c3.x + c4.x));
  a.y = 0.25 * ((c1.y + c2.y) + (c3.y + c4.y));
  a.z = 0.25 * ((c1.z + c2.z) + (c3.z + c4.z));
  b.x = 0.25 * ((c2.x - c1.x) + (c3.x - c4.x));
  b.y = 0.25 * ((c2.y - c1.y) + (c3.y - c4.y));
  b.z = 0.25 * ((c2.z - c1.z) + (c3.z - c4.z));
  c.x = 0.25 * ((c3.x - c2.x) + (c4.x - c1.x));
  c.y = 0.25 * ((c3.y - c2.y) + (c4.y - c1.y));
  c.z = 0.25 * ((c3.z - c2.z) + (c4.z - c1.z));
  d.x = 0.25 * ((c1.x - c2.x) + (c3.x - c4.x));
  d.y = 0.25 * ((c1.y - c2.y) + (c3.y - c4.y));
  d.z = 0.25 * ((c1.z - c2.z) + (c3.z - c4.z));
  const d3 out[9] = {a, b, c, d, dcross(c, a), dcross(c, b), dcross(c, d), dcross(b, a), dcross(b, d)};
  double* o = coef + e * kSeCoef;
  for (int k = 0; k < 9; ++k) {
    o[3 * k] = out[k].x;
    o[3 * k + 1] = out[k].y;
    o[3 * k + 2] = out[k].z;
  }
}

struct InvMap {
  d3 P, Q, R, S, U;  // c x a, c x b, c x d, b x a, b x d
};

__device__ __forceinline__ InvMap load_invmap(const double* __restrict__ g) {
  return InvMap{ld3(g + 12), ld3(g + 15), ld3(g + 18), ld3(g + 21), ld3(g + 24)};
}

__device__ __forceinline__ void se_inverse(const InvMap& m, d3 x, double& xi, double& eta) {
  const double A1 = ddot(x, m.P), B1 = ddot(x, m.Q), D1 = ddot(x, m.R), A2 = ddot(x, m.S), D2 = ddot(x, m.U);
  const double C2 = -B1;
  const double a0 = C2 * D1;
  const double b0 = fma(-D2, A1, fma(A2, D1, C2 * B1));
  const double c0 = A2 * B1;
  double disc = fma(b0, b0, -(4.0 * a0) * c0);
  if (disc < 0.0) disc = 0.0;
  const double q = b0 + copysign(sqrt(disc), b0);
  eta = q != 0.0 ? (-2.0 * c0) / q : 0.0;
  const double den = fma(D1, eta, B1);
  xi = den != 0.0 ? -A1 / den : 0.0;
}

template <int NQ>
__device__ __forceinline__ void lagrange_dev(const SeRule& r, int nq, double t, double* phi) {
  constexpr int M = NQ ? NQ : kSeMaxNq;
  double d[M], suf[M];
#pragma unroll
  for (int m = 0; m < M; ++m)
    if (m < nq) d[m] = t - r.x[m];
  suf[nq - 1] = 1.0;
#pragma unroll
  for (int j = M - 1; j > 0; --j)
    if (j < nq) suf[j - 1] = suf[j] * d[j];
  double pre = 1.0;
#pragma unroll
  for (int j = 0; j < M; ++j)
    if (j < nq) {
      phi[j] = (pre * suf[j]) * r.c[j];
      pre = pre * d[j];
    }
}

// Node positions and weighted Jacobians (W = J w_i w_j radius^2).
__global__ void k_se_nodes(const double* __restrict__ coef, int64_t nelem, const __grid_constant__ SeRule r, double r2,
                           double* __restrict__ pts, double* __restrict__ wj) {
  const int nq = r.nq, nq2 = nq * nq;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nelem * nq2) return;
  const int64_t e = t / nq2;
  const int k = (int)(t - e * nq2), i = k % nq, j = k / nq;
  const double* g = coef + e * kSeCoef;
  const d3 a = ld3(g), b = ld3(g + 3), c = ld3(g + 6), d = ld3(g + 9);
  const double xi = r.x[i], eta = r.x[j], xe = xi * eta;
  d3 X;
  X.x = ((a.x + b.x * xi) + c.x * eta) + d.x * xe;
  X.y = ((a.y + b.y * xi) + c.y * eta) + d.y * xe;
  X.z = ((a.z + b.z * xi) + c.z * eta) + d.z * xe;
  const double n2 = ddot(X, X);
  if (pts) {
    const double ir = 1.0 / sqrt(n2);
    pts[3 * t] = X.x * ir;
    pts[3 * t + 1] = X.y * ir;
    pts[3 * t + 2] = X.z * ir;
  }
  if (wj) {
    const d3 Xxi{b.x + d.x * eta, b.y + d.y * eta, b.z + d.z * eta};
    const d3 Xeta{c.x + d.x * xi, c.y + d.y * xi, c.z + d.z * xi};
    const double J = fabs(ddot(X, dcross(Xxi, Xeta))) / (n2 * sqrt(n2));
    wj[t] = ((J * r.w[i]) * r.w[j]) * r2;
  }
}

// ------------------------------------------------------------------ overlap integrals

// b(e, k)[i + j nq] = integral over cell k ∩ element e of phi_i(xi) phi_j(eta)
// for one candidate pair (accumulate_principled_b :260-305): clip the subject
// (src cell) by the clip polygon (dst cell), fan-triangulate the overlap from
// its normalised vertex sum, Dunavant rule on every triangle of positive area
// (signed by the subject's orientation), (xi, eta) by the inverse element map
// at each rule point.  Each triangle's rule points are summed on their own and
// the triangles added in fan order.  The work is split into triangle items so
// that the lanes of a warp run the same number of rule points:
//   k_se_overlap   per pair: the clip, the fan's centroid and triangle areas,
//                  the polygon kept in the pair's slot
//   k_se_items     per pair: its triangles of positive area as (pair, triangle) items
//   k_se_tri_b<nq> per item: the sum over its rule points
//   k_se_pair_sum  per pair and node: its items in fan order

__global__ void __launch_bounds__(128)
    k_se_overlap(const int2* __restrict__ cand, int64_t nc, const double* __restrict__ dv,
                 const int8_t* __restrict__ dnv, const int8_t* __restrict__ dori, int dmaxv,
                 const double* __restrict__ sv, const int8_t* __restrict__ snv, const int8_t* __restrict__ sori,
                 int smaxv, const double4_32a* __restrict__ dplanes, const float4* __restrict__ dplanes32,
                 const float4* __restrict__ dv4, const float4* __restrict__ sv4, double r2, double* __restrict__ poly,
                 double* __restrict__ cen_out, double* __restrict__ tarea, int32_t* __restrict__ nvert,
                 int32_t* __restrict__ tcount, unsigned long long* __restrict__ overflow) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc) return;
  const int2 pr = cand[t];
  d3 clip[CRG_MAXV];
  d3 bufA[CRG_MAXC], bufB[CRG_MAXC];
  const int nd = dnv[pr.x], ns = snv[pr.y];
  const double* q = dv + (int64_t)pr.x * dmaxv * 3;
  for (int k = 0; k < nd; ++k) clip[k] = ld3(q + 3 * k);
  q = sv + (int64_t)pr.y * smaxv * 3;
  for (int k = 0; k < ns; ++k) bufA[k] = ld3(q + 3 * k);
  const double sig = sori[pr.y];
  int m = 0;
  d3* res = bufA;
  if (nd >= 3 && ns >= 3) {
    float4 fa[CRG_MAXC], fb[CRG_MAXC];
    const float4* q4 = sv4 + (int64_t)pr.y * smaxv;
    for (int k = 0; k < ns; ++k) fa[k] = q4[k];
    const Screen32 s32{dplanes32 + (int64_t)pr.x * dmaxv, dv4 + (int64_t)pr.x * dmaxv, fa, fb};
    m = clip_polygon_oriented<true>(bufA, bufB, ns, clip, nd, (double)dori[pr.x], &res,
                                    dplanes + (int64_t)pr.x * dmaxv, &s32);
    if (m < 0) {
      atomicAdd(overflow, 1ull);
      m = 0;
    }
  }
  int n = 0;
  if (m >= 3) {
    d3 cs = res[0];
    for (int k = 1; k < m; ++k) {
      cs.x = cs.x + res[k].x;
      cs.y = cs.y + res[k].y;
      cs.z = cs.z + res[k].z;
    }
    const double ic = 1.0 / sqrt(ddot(cs, cs));
    const d3 cen{cs.x * ic, cs.y * ic, cs.z * ic};
    cen_out[3 * t] = cen.x; cen_out[3 * t + 1] = cen.y; cen_out[3 * t + 2] = cen.z;
    double* pp = poly + t * (3 * CRG_MAXC);
    double* ta = tarea + t * CRG_MAXC;
    for (int k = 0; k < m; ++k) {
      const d3 v1 = res[k], v2 = res[k + 1 == m ? 0 : k + 1];
      pp[3 * k] = v1.x; pp[3 * k + 1] = v1.y; pp[3 * k + 2] = v1.z;
      const double N = triple(cen, v1, v2);
      const double D = ((1.0 + ddot(cen, v1)) + ddot(v1, v2)) + ddot(v2, cen);
      const double At = ((2.0 * atan2_crg(N, D)) * sig) * r2;
      ta[k] = At;
      n += At > 0.0;
    }
  }
  nvert[t] = m;
  tcount[t] = n;
}

__global__ void k_se_items(const int32_t* __restrict__ nvert, const double* __restrict__ tarea,
                           const int32_t* __restrict__ toff, int64_t nc, int2* __restrict__ items) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc) return;
  const int m = nvert[t];
  int32_t o = toff[t];
  for (int k = 0; k < m; ++k)
    if (tarea[t * CRG_MAXC + k] > 0.0) items[o++] = make_int2((int32_t)t, k);
}

template <int NQ>
__global__ void __launch_bounds__(128)
    k_se_tri_b(const int2* __restrict__ items, int64_t nitems, const double* __restrict__ poly,
               const double* __restrict__ cenv, const double* __restrict__ tarea, const int32_t* __restrict__ nvert,
               const int2* __restrict__ cand, const double* __restrict__ coef, int se_is_dst,
               const __grid_constant__ SeRule r, double* __restrict__ tb) {
  constexpr int M = NQ ? NQ : kSeMaxNq;
  const int nq = NQ ? NQ : r.nq, nq2 = nq * nq;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nitems) return;
  const int2 item = items[t];
  const int64_t pair = item.x;
  const int k = item.y, k1 = k + 1 == nvert[pair] ? 0 : k + 1;
  const int2 pr = cand[pair];
  const InvMap im = load_invmap(coef + (int64_t)(se_is_dst ? pr.x : pr.y) * kSeCoef);
  const double* pp = poly + pair * (3 * CRG_MAXC);
  const d3 cen = ld3(cenv + 3 * pair), v1 = ld3(pp + 3 * k), v2 = ld3(pp + 3 * k1);
  const double At = tarea[pair * CRG_MAXC + k];
  double T[M * M];
#pragma unroll
  for (int k = 0; k < M * M; ++k) T[k] = 0.0;
  for (int g = 0; g < r.ntri; ++g) {
    const double l0 = r.tl[g][0], l1 = r.tl[g][1], l2 = r.tl[g][2];
    // the rule point l0 cen + l1 v1 + l2 v2; the inverse map is invariant
    // under scaling of x, so its projection onto the sphere is not needed
    d3 x;
    x.x = fma(l2, v2.x, fma(l1, v1.x, l0 * cen.x));
    x.y = fma(l2, v2.y, fma(l1, v1.y, l0 * cen.y));
    x.z = fma(l2, v2.z, fma(l1, v1.z, l0 * cen.z));
    double xi, eta;
    se_inverse(im, x, xi, eta);
    double fx[M], fy[M];
    lagrange_dev<NQ>(r, nq, xi, fx);
    lagrange_dev<NQ>(r, nq, eta, fy);
    const double wA = r.tw[g] * At;
#pragma unroll
    for (int i = 0; i < M; ++i)
      if (i < nq) fx[i] = wA * fx[i];
#pragma unroll
    for (int j = 0; j < M; ++j)
#pragma unroll
      for (int i = 0; i < M; ++i)
        if (i < nq && j < nq) T[i + j * nq] = fma(fx[i], fy[j], T[i + j * nq]);
  }
  double* o = tb + t * nq2;
#pragma unroll
  for (int k = 0; k < M * M; ++k)
    if (k < nq2) o[k] = T[k];
}

// One thread per (pair, node): the pair's items summed in fan order (the
// nq2 threads of a pair read consecutive sums of each item).
__global__ void k_se_pair_sum(const int32_t* __restrict__ toff, const int32_t* __restrict__ tcount, int64_t nc,
                              const double* __restrict__ tb, int nq2, double* __restrict__ bv) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc * nq2) return;
  const int64_t pair = t / nq2;
  const int k = (int)(t - pair * nq2);
  const int64_t a = toff[pair];
  const int n = tcount[pair];
  double s = 0.0;
  for (int j = 0; j < n; ++j) s = s + tb[(a + j) * nq2 + k];
  bv[t] = s;
}

// Nonzero sums of each pair.
__global__ void k_se_pair_nz(const double* __restrict__ bv, int64_t nc, int nq2, int32_t* __restrict__ cnt) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc) return;
  int nz = 0;
  for (int k = 0; k < nq2; ++k) nz += bv[t * nq2 + k] != 0.0;
  cnt[t] = nz;
}

// ------------------------------------------------------------------ L2 projection (FV -> SE)

// Pairs with entries grouped by one of their cells (by_x: the dst cell, else
// the src cell), keyed by the other; sort_rows then orders each group by that
// key (the pair index rides along as an exactly representable double).
__global__ void k_group_count(const int2* __restrict__ cand, const int32_t* __restrict__ cnt, int64_t nc, int by_x,
                              int32_t* __restrict__ gcnt) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc || cnt[t] == 0) return;
  atomicAdd(&gcnt[by_x ? cand[t].x : cand[t].y], 1);
}

__global__ void k_group_fill(const int2* __restrict__ cand, const int32_t* __restrict__ cnt, int64_t nc, int by_x,
                             const int32_t* __restrict__ gptr, int32_t* __restrict__ gfill, int32_t* __restrict__ key,
                             double* __restrict__ gpair) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc || cnt[t] == 0) return;
  const int2 pr = cand[t];
  const int32_t g = by_x ? pr.x : pr.y;
  const int32_t p = gptr[g] + atomicAdd(&gfill[g], 1);
  key[p] = by_x ? pr.y : pr.x;
  gpair[p] = (double)t;
}

// One block per element (fv_to_se_l2_projection :634-679).  Shared memory:
// Jn [nq2] nodal Jacobians | Jq [nm^2] at the mass points | M [nq2^2] mass
// matrix, then its covered rows/columns | Inv [nq2^2] | bfull [nq2] | f [nq2]
// | cov [nq2] (int) | pivot (int).
__global__ void __launch_bounds__(128)
    k_se_project(const int32_t* __restrict__ eptr, const double* __restrict__ epair, const double* __restrict__ wj,
                 const __grid_constant__ SeRule r, const __grid_constant__ SeMass ms, const double* __restrict__ bv,
                 double* __restrict__ pv, int32_t* __restrict__ cnt, int* __restrict__ singular) {
  extern __shared__ double sh[];
  const int nq = r.nq, nq2 = nq * nq, nm = ms.nm;
  const int e = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  const int32_t p0 = eptr[e], p1 = eptr[e + 1];
  if (p0 == p1) return;  // no overlaps: the element's nodes keep no entries
  double* Jn = sh;
  double* Jq = Jn + nq2;
  double* M = Jq + nm * nm;
  double* Inv = M + nq2 * nq2;
  double* bfull = Inv + nq2 * nq2;
  double* f = bfull + nq2;
  int* cov = reinterpret_cast<int*>(f + nq2);
  int* piv = cov + nq2;
  __shared__ int ncov;
  // element_jacobian_at: nodal J = W / (w_p w_q), Lagrange-interpolated
  for (int k = tid; k < nq2; k += nt) Jn[k] = wj[(int64_t)e * nq2 + k] / (r.w[k % nq] * r.w[k / nq]);
  __syncthreads();
  for (int k = tid; k < nm * nm; k += nt) {
    const int pp = k % nm, qq = k / nm;
    double s = 0.0;
    for (int qn = 0; qn < nq; ++qn)
      for (int pn = 0; pn < nq; ++pn) s = fma(Jn[pn + qn * nq] * ms.L[pp][pn], ms.L[qq][qn], s);
    Jq[k] = s;
  }
  __syncthreads();
  // M[(a,b),(i,j)] = sum_(q,p) w_p w_q J phi_a(xi_p) phi_i(xi_p) phi_b(eta_q) phi_j(eta_q),
  // by sum factorisation: G[q][a][i] = sum_p w_p w_q J phi_a(xi_p) phi_i(xi_p) first
  double* G = Inv;  // nm * nq2 doubles, free until the inverse is formed
  for (int k = tid; k < nm * nq2; k += nt) {
    const int qq = k / nq2, a = (k % nq2) % nq, i = (k % nq2) / nq;
    double s = 0.0;
    for (int pp = 0; pp < nm; ++pp)
      s = fma(((ms.w[pp] * ms.w[qq]) * Jq[pp + qq * nm]) * ms.L[pp][a], ms.L[pp][i], s);
    G[k] = s;
  }
  __syncthreads();
  for (int k = tid; k < nq2 * nq2; k += nt) {
    const int row = k / nq2, col = k % nq2;
    const int a = row % nq, b = row / nq, i = col % nq, j = col / nq;
    double s = 0.0;
    for (int qq = 0; qq < nm; ++qq) s = fma(G[qq * nq2 + a + i * nq] * ms.L[qq][b], ms.L[qq][j], s);
    M[k] = s;
  }
  for (int k = tid; k < nq2; k += nt) {
    double s = 0.0;
    for (int32_t p = p0; p < p1; ++p) s = s + bv[(int64_t)epair[p] * nq2 + k];
    bfull[k] = s;
  }
  __syncthreads();
  if (tid == 0) {
    int n = 0;
    for (int k = 0; k < nq2; ++k)
      if (bfull[k] != 0.0) cov[n++] = k;
    ncov = n;
  }
  __syncthreads();
  const int m = ncov;
  // Mc = M[cov, cov] (staged through Inv), every row scaled so that its sum
  // equals bfull: exact constant preservation (:650-663)
  for (int x = tid; x < m * m; x += nt) Inv[(x / m) * nq2 + x % m] = M[cov[x / m] * nq2 + cov[x % m]];
  __syncthreads();
  for (int x = tid; x < m * m; x += nt) M[(x / m) * nq2 + x % m] = Inv[(x / m) * nq2 + x % m];
  __syncthreads();
  for (int rc = tid; rc < m; rc += nt) {
    double rs = 0.0;
    for (int cc = 0; cc < m; ++cc) rs = rs + M[rc * nq2 + cc];
    if (rs != 0.0) {
      const double scale = bfull[cov[rc]] / rs;
      for (int cc = 0; cc < m; ++cc) M[rc * nq2 + cc] = M[rc * nq2 + cc] * scale;
    }
  }
  for (int k = tid; k < m * m; k += nt) Inv[(k / m) * nq2 + k % m] = (k / m == k % m) ? 1.0 : 0.0;
  __syncthreads();
  // Gauss-Jordan elimination with partial pivoting (first largest |pivot|)
  for (int k = 0; k < m; ++k) {
    if (tid == 0) {
      int p = k;
      double best = fabs(M[k * nq2 + k]);
      for (int rr = k + 1; rr < m; ++rr)
        if (fabs(M[rr * nq2 + k]) > best) {
          best = fabs(M[rr * nq2 + k]);
          p = rr;
        }
      *piv = best == 0.0 ? -1 : p;
    }
    __syncthreads();
    const int p = *piv;
    if (p < 0) {
      if (tid == 0) atomicAdd(singular, 1);
      return;
    }
    if (p != k)
      for (int cc = tid; cc < m; cc += nt) {
        double x = M[k * nq2 + cc];
        M[k * nq2 + cc] = M[p * nq2 + cc];
        M[p * nq2 + cc] = x;
        x = Inv[k * nq2 + cc];
        Inv[k * nq2 + cc] = Inv[p * nq2 + cc];
        Inv[p * nq2 + cc] = x;
      }
    __syncthreads();
    const double pk = M[k * nq2 + k];
    __syncthreads();
    for (int cc = tid; cc < m; cc += nt) {
      if (cc > k) M[k * nq2 + cc] = M[k * nq2 + cc] / pk;
      Inv[k * nq2 + cc] = Inv[k * nq2 + cc] / pk;
    }
    if (tid == 0) M[k * nq2 + k] = 1.0;
    for (int rr = tid; rr < m; rr += nt) f[rr] = M[rr * nq2 + k];
    __syncthreads();
    for (int x = tid; x < m * m; x += nt) {
      const int rr = x / m, cc = x % m;
      if (rr == k) continue;
      if (cc > k) M[rr * nq2 + cc] = M[rr * nq2 + cc] - f[rr] * M[k * nq2 + cc];
      if (cc == k) M[rr * nq2 + cc] = 0.0;
      Inv[rr * nq2 + cc] = Inv[rr * nq2 + cc] - f[rr] * Inv[k * nq2 + cc];
    }
    __syncthreads();
  }
  // every cell's column: Inv * b[cov]
  const int32_t np = p1 - p0;
  for (int x = tid; x < np * nq2; x += nt) {
    const int64_t t = (int64_t)epair[p0 + x / nq2];
    const int k = x % nq2;
    pv[t * nq2 + k] = 0.0;
  }
  __syncthreads();
  for (int x = tid; x < np * m; x += nt) {
    const int64_t t = (int64_t)epair[p0 + x / m];
    const int rc = x % m;
    double s = 0.0;
    for (int cc = 0; cc < m; ++cc) s = fma(Inv[rc * nq2 + cc], bv[t * nq2 + cov[cc]], s);
    pv[t * nq2 + cov[rc]] = s;
  }
  __syncthreads();
  for (int x = tid; x < np; x += nt) {
    const int64_t t = (int64_t)epair[p0 + x];
    int n = 0;
    for (int k = 0; k < nq2; ++k) n += pv[t * nq2 + k] != 0.0;
    cnt[t] = n;
  }
}

// Rows = FV cells: the cell's pairs in element order, each pair's nonzeros in
// node order (so every row comes out sorted); o = the pair's first position.
__global__ void k_pair_counts(const double* __restrict__ gpair, int64_t np, const int32_t* __restrict__ cnt,
                              int32_t* __restrict__ w) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a < np) w[a] = cnt[(int64_t)gpair[a]];
}

__global__ void k_cell_ptr(const int32_t* __restrict__ gptr, int64_t ncells, const int32_t* __restrict__ poff,
                           int32_t* __restrict__ ptr) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c <= ncells) ptr[c] = poff[gptr[c]];
}

__global__ void k_cell_rows(const double* __restrict__ gpair, const int32_t* __restrict__ gkey, int64_t np,
                            const int32_t* __restrict__ poff, const double* __restrict__ vals, int nq2,
                            int32_t* __restrict__ idx, double* __restrict__ val) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= np) return;
  const int64_t pair = (int64_t)gpair[a];
  const int64_t e = gkey[a];
  int32_t o = poff[a];
  for (int k = 0; k < nq2; ++k) {
    const double v = vals[pair * nq2 + k];
    if (v == 0.0) continue;
    idx[o] = (int32_t)(e * nq2 + k);
    val[o] = v;
    ++o;
  }
}

// Rows = nodes (e, k): the element's pairs in cell order, entry k of each.
__global__ void k_node_counts(const int32_t* __restrict__ eptr, const double* __restrict__ epair, int64_t nelem,
                              const double* __restrict__ vals, int nq2, int32_t* __restrict__ ncnt) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nelem * nq2) return;
  const int64_t e = t / nq2;
  const int k = (int)(t - e * nq2);
  int32_t n = 0;
  for (int32_t p = eptr[e]; p < eptr[e + 1]; ++p) n += vals[(int64_t)epair[p] * nq2 + k] != 0.0;
  ncnt[t] = n;
}

__global__ void k_node_rows(const int32_t* __restrict__ eptr, const int32_t* __restrict__ ecell,
                            const double* __restrict__ epair, int64_t nelem, const double* __restrict__ vals, int nq2,
                            const int32_t* __restrict__ nptr, int32_t* __restrict__ idx, double* __restrict__ val) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nelem * nq2) return;
  const int64_t e = t / nq2;
  const int k = (int)(t - e * nq2);
  int32_t o = nptr[t];
  for (int32_t p = eptr[e]; p < eptr[e + 1]; ++p) {
    const double v = vals[(int64_t)epair[p] * nq2 + k];
    if (v == 0.0) continue;
    idx[o] = ecell[p];
    val[o] = v;
    ++o;
  }
}

__global__ void k_fill(double* __restrict__ p, int64_t n, double v) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) p[t] = v;
}

__global__ void k_scale(double* __restrict__ p, int64_t n, double v) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) p[t] = p[t] * v;
}

// ------------------------------------------------------------------ DSS

template <class T> __device__ __forceinline__ double ldv(const T* p);
template <> __device__ __forceinline__ double ldv<double>(const double* p) { return *p; }
template <> __device__ __forceinline__ double ldv<float>(const float* p) { return (double)*p; }
template <> __device__ __forceinline__ double ldv<__nv_bfloat16>(const __nv_bfloat16* p) {
  return (double)__bfloat162float(*p);
}
template <class T> __device__ __forceinline__ void stv(T* p, double v);
template <> __device__ __forceinline__ void stv<double>(double* p, double v) { *p = v; }
template <> __device__ __forceinline__ void stv<float>(float* p, double v) { *p = (float)v; }
template <> __device__ __forceinline__ void stv<__nv_bfloat16>(__nv_bfloat16* p, double v) {
  *p = __float2bfloat16_rn((float)v);
}

template <class T>
__global__ void k_se_dss(T* __restrict__ fld, int64_t sn, int64_t sf, int64_t nfields, const int32_t* __restrict__ gptr,
                         const int32_t* __restrict__ gnodes, const double* __restrict__ w, int64_t ngroups) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ngroups) return;
  const int32_t a = gptr[g], b = gptr[g + 1];
  for (int64_t fi = blockIdx.y; fi < nfields; fi += gridDim.y) {
    double s = 0.0, W = 0.0;
    for (int32_t k = a; k < b; ++k) {
      const int64_t n = gnodes[k];
      s = s + w[n] * ldv<T>(fld + n * sn + fi * sf);
      W = W + w[n];
    }
    const double v = s / W;
    for (int32_t k = a; k < b; ++k) stv<T>(fld + (int64_t)gnodes[k] * sn + fi * sf, v);
  }
}

// ------------------------------------------------------------------ host

struct Events4 {
  cudaEvent_t e[4] = {};
  Events4() {
    for (auto& x : e) CRG_CHECK_CUDA(cudaEventCreate(&x));
  }
  ~Events4() {
    for (auto& x : e)
      if (x) cudaEventDestroy(x);
  }
};

void check_space(const crg_se_space* se, const crg_se_opts* opts) {
  CRG_REQUIRE(se != nullptr, CRG_ERR_INVALID_ARGUMENT, "SE space is NULL");
  CRG_REQUIRE(se->nq >= 2 && se->nq <= kSeMaxNq, CRG_ERR_INVALID_ARGUMENT, "nq = %d must be in 2..%d", se->nq,
              kSeMaxNq);
  CRG_REQUIRE(se->elements.manifold == CRG_SPHERICAL, CRG_ERR_INVALID_ARGUMENT,
              "spectral-element spaces are spherical (cubed-sphere meshes)");
  CRG_REQUIRE(!opts || opts->flags == 0, CRG_ERR_INVALID_ARGUMENT, "crg_se_opts.flags must be 0");
  CRG_REQUIRE(!opts || opts->radius >= 0.0, CRG_ERR_INVALID_ARGUMENT, "radius must be >= 0");
}

double radius2(const crg_se_opts* opts) {
  const double rad = (opts && opts->radius > 0.0) ? opts->radius : 1.0;
  return rad * rad;
}

// Element coefficients of an uploaded element table.
void element_coeffs(const CellTable& t, DBuf<double>& coef, cudaStream_t st) {
  coef.alloc((size_t)t.n * kSeCoef + 1, st);
  DBuf<int> bad(1, st);
  bad.zero();
  if (t.n) {
    k_se_coeffs<<<nblk(t.n, 128), 128, 0, st>>>(t.v, t.nv, t.maxv, t.n, coef.p, bad.p);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
  int hb = 0;
  CRG_CHECK_CUDA(cudaMemcpyAsync(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  CRG_CHECK_CUDA(cudaStreamSynchronize(st));
  CRG_REQUIRE(hb == 0, CRG_ERR_INVALID_ARGUMENT, "%d elements do not have 4 vertices", hb);
}

// Node weights of the space on the device: the caller's, or computed.
void node_weights(const crg_se_space* se, const SeRule& r, const DBuf<double>& coef, int64_t nelem, double r2,
                  double* out, cudaStream_t st) {
  const int64_t nn = nelem * r.nq * r.nq;
  if (nn == 0) return;
  if (se->node_weights) {
    CRG_CHECK_CUDA(cudaMemcpyAsync(out, se->node_weights, sizeof(double) * nn, cudaMemcpyDefault, st));
  } else {
    k_se_nodes<<<nblk(nn, 128), 128, 0, st>>>(coef.p, nelem, r, r2, nullptr, out);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
}

// Pairs with entries grouped by their element (by_x = the element is the dst
// cell) or by their FV cell, the other index ascending in each group.
struct Groups {
  DBuf<int32_t> ptr, key;
  DBuf<double> pair;
  int64_t n = 0;
};

void group_pairs(const PairSearch& ps, const int32_t* cnt, int64_t ngroups, bool by_x, Groups& g, cudaStream_t st) {
  const int64_t nc = ps.nc;
  DBuf<int32_t> gcnt((size_t)ngroups + 1, st), fill((size_t)ngroups + 1, st);
  g.ptr.alloc((size_t)ngroups + 1, st);
  gcnt.zero();
  fill.zero();
  if (nc) {
    k_group_count<<<nblk(nc, 256), 256, 0, st>>>(ps.cand, cnt, nc, by_x, gcnt.p);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
  exclusive_scan_i32(gcnt.p, g.ptr.p, ngroups, st);
  int32_t np = 0;
  CRG_CHECK_CUDA(cudaMemcpyAsync(&np, g.ptr.p + ngroups, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  CRG_CHECK_CUDA(cudaStreamSynchronize(st));
  g.n = np;
  g.key.alloc((size_t)np + 1, st);
  g.pair.alloc((size_t)np + 1, st);
  if (nc) {
    k_group_fill<<<nblk(nc, 256), 256, 0, st>>>(ps.cand, cnt, nc, by_x, g.ptr.p, fill.p, g.key.p, g.pair.p);
    CRG_CHECK_CUDA(cudaGetLastError());
  }
  sort_rows(g.ptr.p, ngroups, g.key.p, g.pair.p, st);
}

struct Overlaps {
  const int2* items;
  int64_t nitems;
  const double *poly, *cen, *tarea;
  const int32_t* nvert;
};

template <int NQ>
void launch_tri_b(const Overlaps& o, const PairSearch& ps, const double* coef, int se_is_dst, const SeRule& r,
                  double* tb, cudaStream_t st) {
  k_se_tri_b<NQ><<<nblk(o.nitems, 128), 128, 0, st>>>(o.items, o.nitems, o.poly, o.cen, o.tarea, o.nvert, ps.cand,
                                                      coef, se_is_dst, r, tb);
  CRG_CHECK_CUDA(cudaGetLastError());
}

}  // namespace

crg_regridder* build_se_impl(const crg_grid_desc* fv, const crg_se_space* se, const crg_se_opts* opts,
                             bool se_is_dst) {
  CRG_REQUIRE(fv != nullptr, CRG_ERR_INVALID_ARGUMENT, "FV grid is NULL");
  check_space(se, opts);
  CRG_REQUIRE(fv->manifold == CRG_SPHERICAL, CRG_ERR_INVALID_ARGUMENT,
              "the FV grid of an SE regridder must be spherical (got manifold %d)", fv->manifold);
  cudaStream_t st = opts ? (cudaStream_t)opts->stream : nullptr;
  const int nq = se->nq, nq2 = nq * nq;
  const int degree = (opts && opts->triangle_quad_degree) ? opts->triangle_quad_degree : 2 * (nq - 1);
  const SeRule rule = make_rule(nq, degree);
  const double r2 = radius2(opts);

  crg_regridder* R = new crg_regridder();
  try {
    CRG_CHECK_CUDA(cudaGetDevice(&R->device));
    R->manifold = CRG_SPHERICAL;
    Events4 ev;
    CRG_CHECK_CUDA(cudaEventRecord(ev.e[0], st));
    PairSearch ps;
    if (se_is_dst)
      ps.upload(&se->elements, fv, st);
    else
      ps.upload(fv, &se->elements, st);
    const int64_t nelem = se_is_dst ? ps.nd : ps.ns, nfv = se_is_dst ? ps.ns : ps.nd;
    CRG_REQUIRE(nelem * nq2 < ((int64_t)1 << 31), CRG_ERR_NOT_SUPPORTED, "%lld nodes exceed the 32-bit index range",
                (long long)(nelem * nq2));
    const int64_t nn = nelem * nq2;
    R->nd = se_is_dst ? nn : nfv;
    R->ns = se_is_dst ? nfv : nn;
    R->dst_area = keep_alloc<double>((size_t)R->nd, st);
    R->src_area = keep_alloc<double>((size_t)R->ns, st);
    DBuf<double> elem_area((size_t)nelem + 1, st);
    double* fv_area = se_is_dst ? R->src_area : R->dst_area;
    if (se_is_dst)
      ps.search(elem_area.p, fv_area, st);
    else
      ps.search(fv_area, elem_area.p, st);
    const int64_t nc = ps.nc;
    R->ncand = ps.nc_search;
    // A pair yields at most CRG_MAXC fan triangles and nq^2 <= 64 nonzeros, so
    // below 2^26 pairs the int32 scans of those counts cannot pass 2^32, and a
    // total of 2^31 or more shows as negative (checked after each scan).
    static_assert(CRG_MAXC <= kSeMaxNq * kSeMaxNq, "the pair bound covers the triangle count");
    CRG_REQUIRE(nc < ((int64_t)1 << 26), CRG_ERR_NOT_SUPPORTED,
                "%lld overlapping pairs: the per-pair counts could overflow int32", (long long)nc);
    DBuf<double> coef;
    element_coeffs(se_is_dst ? ps.dtab : ps.stab, coef, st);
    DBuf<double> wj((size_t)nn + 1, st);
    node_weights(se, rule, coef, nelem, r2, wj.p, st);
    CRG_CHECK_CUDA(cudaEventRecord(ev.e[1], st));

    DBuf<double> bv((size_t)nc * nq2 + 1, st);
    DBuf<int32_t> cnt((size_t)nc + 1, st);
    DBuf<unsigned long long> ovf(1, st);
    ovf.zero();
    if (nc) {
      const CellTable &D = ps.dtab, &S = ps.stab;
      DBuf<int32_t> tcount((size_t)nc + 1, st), toff((size_t)nc + 1, st), nvert((size_t)nc + 1, st);
      // per pair: the clipped polygon (CRG_MAXC vertex slots), its centroid and fan-triangle areas
      DBuf<double> poly((size_t)nc * 3 * CRG_MAXC, st), cen((size_t)nc * 3, st), tarea((size_t)nc * CRG_MAXC, st);
      k_se_overlap<<<nblk(nc, 128), 128, 0, st>>>(ps.cand, nc, D.v, D.nv, D.ori, D.maxv, S.v, S.nv, S.ori, S.maxv,
                                                  ps.dplanes, ps.dplanes32, D.v4, S.v4, r2, poly.p, cen.p, tarea.p,
                                                  nvert.p, tcount.p, ovf.p);
      CRG_CHECK_CUDA(cudaGetLastError());
      exclusive_scan_i32(tcount.p, toff.p, nc, st);
      unsigned long long hovf = 0;
      int32_t nitems = 0;
      CRG_CHECK_CUDA(cudaMemcpyAsync(&hovf, ovf.p, sizeof(hovf), cudaMemcpyDeviceToHost, st));
      CRG_CHECK_CUDA(cudaMemcpyAsync(&nitems, toff.p + nc, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
      CRG_CHECK_CUDA(cudaStreamSynchronize(st));
      CRG_REQUIRE(hovf == 0, CRG_ERR_GEOMETRY,
                  "%llu candidate pairs exceeded the clipped-polygon capacity of %d vertices (non-convex cells?)",
                  (unsigned long long)hovf, CRG_MAXC);
      CRG_REQUIRE(nitems >= 0, CRG_ERR_NOT_SUPPORTED, "the triangle count overflows int32");
      DBuf<int2> items((size_t)nitems + 1, st);
      DBuf<double> tb((size_t)nitems * nq2 + 1, st);
      k_se_items<<<nblk(nc, 128), 128, 0, st>>>(nvert.p, tarea.p, toff.p, nc, items.p);
      CRG_CHECK_CUDA(cudaGetLastError());
      if (nitems) {
        const Overlaps o{items.p, nitems, poly.p, cen.p, tarea.p, nvert.p};
        switch (nq) {
          case 2: launch_tri_b<2>(o, ps, coef.p, se_is_dst, rule, tb.p, st); break;
          case 3: launch_tri_b<3>(o, ps, coef.p, se_is_dst, rule, tb.p, st); break;
          case 4: launch_tri_b<4>(o, ps, coef.p, se_is_dst, rule, tb.p, st); break;
          case 5: launch_tri_b<5>(o, ps, coef.p, se_is_dst, rule, tb.p, st); break;
          default: launch_tri_b<0>(o, ps, coef.p, se_is_dst, rule, tb.p, st); break;
        }
      }
      k_se_pair_sum<<<nblk(nc * nq2, 256), 256, 0, st>>>(toff.p, tcount.p, nc, tb.p, nq2, bv.p);
      k_se_pair_nz<<<nblk(nc, 256), 256, 0, st>>>(bv.p, nc, nq2, cnt.p);
      CRG_CHECK_CUDA(cudaGetLastError());
    }

    const double* vals = bv.p;
    DBuf<double> pv;
    if (se_is_dst && nc) {
      // the overlapping pairs grouped by element, cells ascending
      Groups eg;
      group_pairs(ps, cnt.p, nelem, true, eg, st);
      const int32_t* eptr_p = eg.ptr.p;
      const double* epair_p = eg.pair.p;
      const SeMass mass = make_mass(rule);
      pv.alloc((size_t)nc * nq2 + 1, st);
      CRG_CHECK_CUDA(cudaMemsetAsync(pv.p, 0, sizeof(double) * nc * nq2, st));
      const size_t smem = sizeof(double) * (size_t)(nq2 + mass.nm * mass.nm + 2 * nq2 * nq2 + 2 * nq2) +
                          sizeof(int) * (size_t)(nq2 + 1);
      CRG_CHECK_CUDA(cudaFuncSetAttribute(k_se_project, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      DBuf<int> singular(1, st);
      singular.zero();
      if (nelem) {
        k_se_project<<<(unsigned)nelem, 128, smem, st>>>(eptr_p, epair_p, wj.p, rule, mass, bv.p, pv.p, cnt.p,
                                                         singular.p);
        CRG_CHECK_CUDA(cudaGetLastError());
      }
      int hs = 0;
      CRG_CHECK_CUDA(cudaMemcpyAsync(&hs, singular.p, sizeof(int), cudaMemcpyDeviceToHost, st));
      CRG_CHECK_CUDA(cudaStreamSynchronize(st));
      CRG_REQUIRE(hs == 0, CRG_ERR_GEOMETRY, "%d local mass matrices are singular", hs);
      vals = pv.p;
    }
    CRG_CHECK_CUDA(cudaEventRecord(ev.e[2], st));

    // Both CSR copies written in order: rows = FV cells from the pairs grouped
    // by cell (elements ascending), rows = nodes from the pairs grouped by
    // element (cells ascending).
    Groups cg, eg2;
    group_pairs(ps, cnt.p, nfv, !se_is_dst, cg, st);
    group_pairs(ps, cnt.p, nelem, se_is_dst, eg2, st);
    DBuf<int32_t> w((size_t)cg.n + 1, st), poff((size_t)cg.n + 1, st);
    if (cg.n) {
      k_pair_counts<<<nblk(cg.n, 256), 256, 0, st>>>(cg.pair.p, cg.n, cnt.p, w.p);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
    exclusive_scan_i32(w.p, poff.p, cg.n, st);
    int32_t m = 0;
    CRG_CHECK_CUDA(cudaMemcpyAsync(&m, poff.p + cg.n, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CRG_CHECK_CUDA(cudaStreamSynchronize(st));
    CRG_REQUIRE(m >= 0, CRG_ERR_NOT_SUPPORTED, "the nonzero count overflows int32");
    DevCsr& crows = se_is_dst ? R->rev : R->fwd;  // rows = FV cells
    DevCsr& nrows = se_is_dst ? R->fwd : R->rev;  // rows = nodes
    crows.nrows = nfv; crows.ncols = nn;
    nrows.nrows = nn; nrows.ncols = nfv;
    R->nnz = m;
    crows.nnz = nrows.nnz = m;
    crows.ptr = keep_alloc<int32_t>((size_t)nfv + 1, st);
    nrows.ptr = keep_alloc<int32_t>((size_t)nn + 1, st);
    for (DevCsr* c : {&crows, &nrows}) {
      c->idx = keep_alloc<int32_t>((size_t)m, st);
      c->val = keep_alloc<double>((size_t)m, st);
    }
    k_cell_ptr<<<nblk(nfv + 1, 256), 256, 0, st>>>(cg.ptr.p, nfv, poff.p, crows.ptr);
    CRG_CHECK_CUDA(cudaGetLastError());
    if (cg.n) {
      k_cell_rows<<<nblk(cg.n, 256), 256, 0, st>>>(cg.pair.p, cg.key.p, cg.n, poff.p, vals, nq2, crows.idx, crows.val);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
    DBuf<int32_t> ncnt((size_t)nn + 1, st);
    if (nn) {
      k_node_counts<<<nblk(nn, 256), 256, 0, st>>>(eg2.ptr.p, eg2.pair.p, nelem, vals, nq2, ncnt.p);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
    exclusive_scan_i32(ncnt.p, nrows.ptr, nn, st);
    if (nn) {
      k_node_rows<<<nblk(nn, 256), 256, 0, st>>>(eg2.ptr.p, eg2.key.p, eg2.pair.p, nelem, vals, nq2, nrows.ptr,
                                                 nrows.idx, nrows.val);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
    // areas: FV cells (scaled to the radius), node weights or ones
    if (r2 != 1.0 && nfv) {
      k_scale<<<nblk(nfv, 256), 256, 0, st>>>(fv_area, nfv, r2);
      CRG_CHECK_CUDA(cudaGetLastError());
    }
    if (se_is_dst) {
      if (nn) {
        k_fill<<<nblk(nn, 256), 256, 0, st>>>(R->dst_area, nn, 1.0);
        CRG_CHECK_CUDA(cudaGetLastError());
      }
    } else if (nn) {
      CRG_CHECK_CUDA(cudaMemcpyAsync(R->src_area, wj.p, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
    }
    finish_build(R, st);
    CRG_CHECK_CUDA(cudaEventRecord(ev.e[3], st));
    CRG_CHECK_CUDA(cudaEventSynchronize(ev.e[3]));
    float t01 = 0, t12 = 0, t23 = 0, t03 = 0;
    cudaEventElapsedTime(&t01, ev.e[0], ev.e[1]);
    cudaEventElapsedTime(&t12, ev.e[1], ev.e[2]);
    cudaEventElapsedTime(&t23, ev.e[2], ev.e[3]);
    cudaEventElapsedTime(&t03, ev.e[0], ev.e[3]);
    crg_info& I = R->info;
    I.n_dst = R->nd; I.n_src = R->ns; I.nnz = R->nnz; I.n_candidates = ps.nc_search; I.n_clipped = ps.nc;
    I.manifold = CRG_SPHERICAL; I.normalized = 0; I.normalizer = 1.0;
    I.t_build_ms = t03; I.t_search_ms = t01; I.t_clip_ms = t12; I.t_assemble_ms = t23;
    I.clip_overflows = 0;
    I.device = R->device;
  } catch (...) {
    free_regridder(R);
    throw;
  }
  return R;
}

void se_nodes_impl(const crg_se_space* se, const crg_se_opts* opts, double* points, double* weights) {
  check_space(se, opts);
  cudaStream_t st = opts ? (cudaStream_t)opts->stream : nullptr;
  const SeRule rule = make_rule(se->nq, 1);
  const int nq2 = se->nq * se->nq;
  PairSearch ps;  // only its upload: the element table
  ps.upload(&se->elements, &se->elements, st);
  const int64_t nelem = ps.nd, nn = nelem * nq2;
  DBuf<double> coef;
  element_coeffs(ps.dtab, coef, st);
  DBuf<double> pts((size_t)nn * 3 + 1, st), wj((size_t)nn + 1, st);
  if (nn) {
    k_se_nodes<<<nblk(nn, 128), 128, 0, st>>>(coef.p, nelem, rule, radius2(opts), pts.p, wj.p);
    CRG_CHECK_CUDA(cudaGetLastError());
    if (se->node_weights)
      CRG_CHECK_CUDA(cudaMemcpyAsync(wj.p, se->node_weights, sizeof(double) * nn, cudaMemcpyDefault, st));
    if (points) CRG_CHECK_CUDA(cudaMemcpyAsync(points, pts.p, sizeof(double) * nn * 3, cudaMemcpyDefault, st));
    if (weights) CRG_CHECK_CUDA(cudaMemcpyAsync(weights, wj.p, sizeof(double) * nn, cudaMemcpyDefault, st));
  }
  CRG_CHECK_CUDA(cudaStreamSynchronize(st));
}

void se_dss_impl(int dtype, void* field, int64_t sn, int64_t sf, int64_t nfields, const int32_t* group_ptr,
                 const int32_t* group_nodes, const double* weights, int64_t ngroups, cudaStream_t st) {
  CRG_REQUIRE(ngroups >= 0 && nfields >= 0, CRG_ERR_INVALID_ARGUMENT, "ngroups and nfields must be >= 0");
  if (ngroups == 0 || nfields == 0) return;
  CRG_REQUIRE(field && group_ptr && group_nodes && weights, CRG_ERR_INVALID_ARGUMENT, "NULL argument");
  CRG_REQUIRE(is_device_pointer(field) && is_device_pointer(group_ptr) && is_device_pointer(group_nodes) &&
                  is_device_pointer(weights),
              CRG_ERR_NOT_SUPPORTED, "crg_se_dss takes device pointers");
  const dim3 grid(nblk(ngroups, 128), (unsigned)std::min<int64_t>(nfields, 65535));
  switch (dtype) {
    case CRG_F64:
      k_se_dss<double><<<grid, 128, 0, st>>>((double*)field, sn, sf, nfields, group_ptr, group_nodes, weights, ngroups);
      break;
    case CRG_F32:
      k_se_dss<float><<<grid, 128, 0, st>>>((float*)field, sn, sf, nfields, group_ptr, group_nodes, weights, ngroups);
      break;
    case CRG_BF16:
      k_se_dss<__nv_bfloat16><<<grid, 128, 0, st>>>((__nv_bfloat16*)field, sn, sf, nfields, group_ptr, group_nodes,
                                                   weights, ngroups);
      break;
    default:
      CRG_REQUIRE(false, CRG_ERR_INVALID_ARGUMENT, "unknown dtype %d", dtype);
  }
  CRG_CHECK_CUDA(cudaGetLastError());
}

}  // namespace crg
