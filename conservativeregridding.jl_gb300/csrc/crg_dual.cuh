// crg_dual.cuh -- forward-mode derivatives of the clip and area of crg_geom.cuh.
//
// The reference has no derivatives (no ChainRulesCore dependency, and its
// build writes Float64 buffers, src/regridder/intersection_areas.jl:14), so
// these exist for the GPU library's area gradient only.  A Dn<N> carries a
// value and N partial derivatives.  Every function below computes its value
// part with exactly the operations, fma placement and branch decisions of the
// FP64 function of the same name in crg_geom.cuh, so the clipped polygon has
// the same combinatorial structure as in the build; the partials follow the
// calculus of each operation (the exact-sign fallback keeps the partials of
// the FP64 side value it settles).
#pragma once
#include "crg_geom.cuh"

namespace crg {

template <int N> struct Dn {
  double v;
  double d[N];
};

template <int N> __device__ __forceinline__ Dn<N> dn_const(double v) {
  Dn<N> r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = 0.0;
  return r;
}
template <int N> __device__ __forceinline__ Dn<N> dn_add(Dn<N> a, Dn<N> b) {
  Dn<N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N> __device__ __forceinline__ Dn<N> dn_sub(Dn<N> a, Dn<N> b) {
  Dn<N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N> __device__ __forceinline__ Dn<N> dn_neg(Dn<N> a) {
  Dn<N> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N> __device__ __forceinline__ Dn<N> dn_mul(Dn<N> a, Dn<N> b) {
  Dn<N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.v * b.d[i] + b.v * a.d[i];
  return r;
}
// a * b + c with the value rounded once, as fma
template <int N> __device__ __forceinline__ Dn<N> dn_fma(Dn<N> a, Dn<N> b, Dn<N> c) {
  Dn<N> r;
  r.v = fma(a.v, b.v, c.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.v * b.d[i] + b.v * a.d[i] + c.d[i];
  return r;
}
template <int N> __device__ __forceinline__ Dn<N> dn_div(Dn<N> a, Dn<N> b) {
  Dn<N> r;
  r.v = a.v / b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) / b.v;
  return r;
}
template <int N> __device__ __forceinline__ Dn<N> dn_sqrt(Dn<N> a) {
  Dn<N> r;
  r.v = sqrt(a.v);
  const double h = r.v > 0.0 ? 0.5 / r.v : 0.0;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = h * a.d[i];
  return r;
}
template <int N> __device__ __forceinline__ Dn<N> dn_abs(Dn<N> a) { return a.v < 0.0 ? dn_neg(a) : a; }
template <int N> __device__ __forceinline__ Dn<N> dn_scale(double s, Dn<N> a) {
  Dn<N> r;
  r.v = s * a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = s * a.d[i];
  return r;
}

template <int N> struct D3n {
  Dn<N> x, y, z;
};

template <int N> __device__ __forceinline__ d3 dval(const D3n<N>& a) { return d3{a.x.v, a.y.v, a.z.v}; }
template <int N> __device__ __forceinline__ D3n<N> d3n_const(d3 a) {
  return D3n<N>{dn_const<N>(a.x), dn_const<N>(a.y), dn_const<N>(a.z)};
}
template <int N> __device__ __forceinline__ D3n<N> d3n_sub(const D3n<N>& a, const D3n<N>& b) {
  return D3n<N>{dn_sub(a.x, b.x), dn_sub(a.y, b.y), dn_sub(a.z, b.z)};
}
template <int N> __device__ __forceinline__ Dn<N> d3n_dot(const D3n<N>& a, const D3n<N>& b) {
  return dn_fma(a.x, b.x, dn_fma(a.y, b.y, dn_mul(a.z, b.z)));
}
template <int N> __device__ __forceinline__ D3n<N> d3n_cross(const D3n<N>& a, const D3n<N>& b) {
  return D3n<N>{dn_sub(dn_mul(a.y, b.z), dn_mul(a.z, b.y)), dn_sub(dn_mul(a.z, b.x), dn_mul(a.x, b.z)),
                dn_sub(dn_mul(a.x, b.y), dn_mul(a.y, b.x))};
}
template <int N> __device__ __forceinline__ Dn<N> d3n_triple(const D3n<N>& a, const D3n<N>& b, const D3n<N>& c) {
  return d3n_dot(a, d3n_cross(d3n_sub(b, a), d3n_sub(c, a)));
}

// ---------------------------------------------------------------- sphere

template <int N>
__device__ __forceinline__ Dn<N> side_sph_n(const D3n<N>& nrm, const D3n<N>& ca, const D3n<N>& cb, double eb, int isig,
                                            const D3n<N>& v) {
  const D3n<N> w = d3n_sub(v, ca);
  Dn<N> s = d3n_dot(nrm, w);
  const double bound = eb * (fabs(w.x.v) + fabs(w.y.v) + fabs(w.z.v)) + kTiny;
  if (fabs(s.v) > bound) return s;
  s.v = settle(s.v, bound, isig * det3_sign_adapt(dval(ca), dval(cb), dval(v)));
  return s;
}

template <int N>
__device__ __forceinline__ D3n<N> isect_sph_n(const D3n<N>& a, const Dn<N>& sa, const D3n<N>& b, const Dn<N>& sb) {
  if (sa.v == 0.0) return a;
  if (sb.v == 0.0) return b;
  Dn<N> wa = dn_abs(sb), wb = dn_abs(sa);
  if (fmax(wa.v, wb.v) < kIsectTiny) {  // isect_sph's rescaling of tiny weights
    wa = dn_scale(kIsectScale, wa);
    wb = dn_scale(kIsectScale, wb);
  }
  D3n<N> x{dn_fma(wb, b.x, dn_mul(wa, a.x)), dn_fma(wb, b.y, dn_mul(wa, a.y)), dn_fma(wb, b.z, dn_mul(wa, a.z))};
  const Dn<N> ir = dn_div(dn_const<N>(1.0), dn_sqrt(d3n_dot(x, x)));
  return D3n<N>{dn_mul(x.x, ir), dn_mul(x.y, ir), dn_mul(x.z, ir)};
}

// 2 arg(prod (D + iN)); d atan2(y, x) = (x dy - y dx) / (x^2 + y^2)
template <int N> __device__ __forceinline__ Dn<N> area_sph_signed_n(const D3n<N>* v, int m) {
  if (m < 3) return dn_const<N>(0.0);
  Dn<N> re = dn_const<N>(1.0), im = dn_const<N>(0.0);
  const D3n<N> a = v[0];
  for (int k = 1; k + 1 < m; ++k) {
    const D3n<N> b = v[k], c = v[k + 1];
    const Dn<N> Nt = d3n_triple(a, b, c);
    const Dn<N> one = dn_const<N>(1.0);
    const Dn<N> D = dn_add(dn_add(dn_add(one, d3n_dot(a, b)), d3n_dot(b, c)), d3n_dot(c, a));
    const Dn<N> re2 = dn_fma(re, D, dn_neg(dn_mul(im, Nt)));
    const Dn<N> im2 = dn_fma(re, Nt, dn_mul(im, D));
    re = re2;
    im = im2;
  }
  Dn<N> r;
  r.v = 2.0 * atan2_crg(im.v, re.v);
  const double q = re.v * re.v + im.v * im.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = q > 0.0 ? 2.0 * (re.v * im.d[i] - im.v * re.d[i]) / q : 0.0;
  return r;
}

// ---------------------------------------------------------------- plane

template <int N> __device__ __forceinline__ Dn<N> cross2_n(Dn<N> ax, Dn<N> ay, Dn<N> bx, Dn<N> by) {
  return dn_sub(dn_mul(ax, by), dn_mul(ay, bx));
}

template <int N> __device__ __forceinline__ Dn<N> area_pl_signed_n(const D3n<N>* v, int m) {
  if (m < 3) return dn_const<N>(0.0);
  Dn<N> s = dn_const<N>(0.0);
  for (int k = 1; k + 1 < m; ++k)
    s = dn_add(s, cross2_n(dn_sub(v[k].x, v[0].x), dn_sub(v[k].y, v[0].y), dn_sub(v[k + 1].x, v[0].x),
                           dn_sub(v[k + 1].y, v[0].y)));
  return dn_scale(0.5, s);
}

template <int N>
__device__ __forceinline__ Dn<N> side_pl_n(const D3n<N>& a, const D3n<N>& b, const Dn<N>& ex, const Dn<N>& ey,
                                           int isig, const D3n<N>& v) {
  const Dn<N> wx = dn_sub(v.x, a.x), wy = dn_sub(v.y, a.y);
  Dn<N> s = cross2_n(ex, ey, wx, wy);
  if (isig < 0) s = dn_neg(s);
  const double bound = kU8 * (fabs(ex.v) * fabs(wy.v) + fabs(ey.v) * fabs(wx.v)) + kTiny;
  if (fabs(s.v) > bound) return s;
  s.v = settle(s.v, bound, isig * orient2_sign(a.x.v, a.y.v, b.x.v, b.y.v, v.x.v, v.y.v));
  return s;
}

template <int N>
__device__ __forceinline__ D3n<N> isect_pl_n(const D3n<N>& a, const Dn<N>& sa, const D3n<N>& b, const Dn<N>& sb) {
  if (sa.v == 0.0) return a;
  if (sb.v == 0.0) return b;
  Dn<N> wa = dn_abs(sb), wb = dn_abs(sa);
  if (fmax(wa.v, wb.v) < kIsectTiny) {
    wa = dn_scale(kIsectScale, wa);
    wb = dn_scale(kIsectScale, wb);
  }
  const Dn<N> w = dn_add(wa, wb);
  return D3n<N>{dn_div(dn_fma(wb, b.x, dn_mul(wa, a.x)), w), dn_div(dn_fma(wb, b.y, dn_mul(wa, a.y)), w),
                dn_const<N>(0.0)};
}

// ---------------------------------------------------------------- clip

// clip_polygon of crg_geom.cuh on D3n vertices, with capacity CAP.
template <bool kSpherical, int N, int CAP>
__device__ __forceinline__ int clip_polygon_n(D3n<N>* bufA, D3n<N>* bufB, int ns, const D3n<N>* clip, int nc,
                                              D3n<N>** res) {
  D3n<N>* in = bufA;
  D3n<N>* out = bufB;
  int n = ns;
  d3 cv[CRG_MAXV];
  for (int k = 0; k < nc; ++k) cv[k] = dval(clip[k]);
  const double sig = kSpherical ? orient_sph(cv, nc) : orient_pl(cv, nc);
  for (int k = 0; k < nc && n > 0; ++k) {
    const D3n<N> ca = clip[k], cb = clip[k + 1 == nc ? 0 : k + 1];
    const int isig = sig < 0.0 ? -1 : 1;
    D3n<N> nrm = d3n_const<N>(d3{0.0, 0.0, 0.0});
    Dn<N> ex = dn_const<N>(0.0), ey = dn_const<N>(0.0);
    double eb = 0.0;
    if (kSpherical) {
      const D3n<N> d1 = d3n_sub(cb, ca);
      nrm = d3n_cross(ca, d1);
      if (sig < 0.0) nrm = D3n<N>{dn_neg(nrm.x), dn_neg(nrm.y), dn_neg(nrm.z)};
      eb = kU32 * (fabs(ca.x.v) + fabs(ca.y.v) + fabs(ca.z.v)) * (fabs(d1.x.v) + fabs(d1.y.v) + fabs(d1.z.v));
    } else {
      ex = dn_sub(cb.x, ca.x);
      ey = dn_sub(cb.y, ca.y);
    }
    int m = 0;
    D3n<N> prev = in[n - 1];
    Dn<N> sp = kSpherical ? side_sph_n(nrm, ca, cb, eb, isig, prev) : side_pl_n(ca, cb, ex, ey, isig, prev);
    for (int i = 0; i < n; ++i) {
      const D3n<N> cur = in[i];
      const Dn<N> sc = kSpherical ? side_sph_n(nrm, ca, cb, eb, isig, cur) : side_pl_n(ca, cb, ex, ey, isig, cur);
      if (sc.v >= 0.0) {
        if (sp.v < 0.0) {
          if (m >= CAP) return -1;
          out[m++] = kSpherical ? isect_sph_n(prev, sp, cur, sc) : isect_pl_n(prev, sp, cur, sc);
        }
        if (m >= CAP) return -1;
        out[m++] = cur;
      } else if (sp.v >= 0.0) {
        if (m >= CAP) return -1;
        out[m++] = kSpherical ? isect_sph_n(prev, sp, cur, sc) : isect_pl_n(prev, sp, cur, sc);
      }
      prev = cur;
      sp = sc;
    }
    D3n<N>* t = in;
    in = out;
    out = t;
    n = m;
  }
  *res = in;
  return n;
}

}  // namespace crg
