/*
 * crg_oracle.c -- CPU oracle for the conservative-regridding hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: tests/, the smoke
 * check in __graft_entry__.py and the cpu_baseline / reference legs of
 * bench.py load it; the product library never links, includes or calls it.
 *
 * It restates, in plain C, what ConservativeRegridding.jl v0.2.5 does when it
 * builds and applies a regridder on the sphere (or the plane):
 *
 *   Regridder(dst, src; normalize)            src/regridder/regridder.jl:105-163
 *     treeify -> TopDownQuadtreeCursor /      src/trees/interfaces.jl:94-129
 *                Healpix tree / cubed sphere  ext/ConservativeRegriddingHealpixExt.jl:18-175,
 *                                             src/trees/wrappers.jl:140-159
 *     candidate search (threaded dual DFS)    src/utils/MultithreadedDualDepthFirstSearch.jl:12-65
 *       + GeometryOps STI.dual_depth_first_search (third party, restated below)
 *     bounding caps                           src/trees/grids.jl:245-287
 *     per-pair clip + area, keep area > 0     src/regridder/intersection_areas.jl:4-32,
 *                                             src/regridder/regridder.jl:96-103
 *     SparseArrays.sparse(i_dst,i_src,a)      src/regridder/intersection_areas.jl:115-121
 *     per-cell areas, normalize! by max(A)    src/regridder/regridder.jl:54-62,165-178
 *   regrid!(dst, R, src) = (A*s) ./ a_d       src/regridder/regrid.jl:63-118
 *   transpose(R)                              src/regridder/regridder.jl:49-50
 *
 * The polygon arithmetic itself lives in GeometryOps.jl (compat 0.1.33, not
 * vendored with the reference).  It is restated here from published methods:
 *   - Sutherland & Hodgman (1974) re-entrant convex polygon clipping, with
 *     great-circle half-spaces s(x) = n.(x - a), n = a x (b - a) = a x b, on
 *     the sphere (differences first, so short edges keep full precision);
 *   - the arc/plane crossing point x = |s_a| b + |s_b| a (both weights >= 0);
 *   - polygon solid angle as the sum over a vertex fan of the triangle solid
 *     angles of Van Oosterom & Strackee (1983), tan(W/2) = N / D with
 *     N = a.((b-a) x (c-a)), accumulated as the argument of the product of
 *     the complex numbers D + iN; orientation = sign of the fan sum of N;
 *   - arctangent by octant/pi-8 range reduction and the Maclaurin series
 *     atan t = sum (-1)^k t^(2k+1)/(2k+1) (Abramowitz & Stegun 4.4.42);
 *   - HEALPix pixel corners from the face/ring geometry of Gorski et al. (2005),
 *     ApJ 622:759.
 * The clip/area arithmetic follows a fixed operation order with explicit fma()
 * and is compiled with -ffp-contract=off, so an independent coding of the same
 * sequence (the CUDA kernels) reproduces it bit for bit.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OG_MAXV 8   /* max vertices of an input cell */
#define OG_MAXC 24  /* capacity of a clipped polygon */

typedef struct { double x, y, z; } v3;

/* ------------------------------------------------------------------------ */
/* Exact-order arithmetic (shared spec with the device code).               */
/* ------------------------------------------------------------------------ */

static inline double og_dot(v3 a, v3 b) { return fma(a.x, b.x, fma(a.y, b.y, a.z * b.z)); }

/* Plain products (no fma): a x a and a x 0 are exactly zero. */
static inline v3 og_cross(v3 a, v3 b) {
    v3 r;
    r.x = a.y * b.z - a.z * b.y;
    r.y = a.z * b.x - a.x * b.z;
    r.z = a.x * b.y - a.y * b.x;
    return r;
}

/* ---- exact signs (error-free transformations, Shewchuk 1997) ---- */

static inline void og_two_prod(double a, double b, double* p, double* e) { *p = a * b; *e = fma(a, b, -*p); }
static inline void og_two_sum(double a, double b, double* s, double* e) {
    double x = a + b, bv = x - a, av = x - bv;
    *e = (a - av) + (b - bv);
    *s = x;
}

/* Exact sign of t[0] + ... + t[n-1]: grow a non-overlapping expansion with
 * zero elimination; its largest component carries the sign. */
static int og_exact_sign(const double* t, int n) {
    double e[32];
    int m = 0;
    for (int i = 0; i < n; ++i) {
        double q = t[i];
        int k = 0;
        for (int j = 0; j < m; ++j) {
            double sm, h;
            og_two_sum(q, e[j], &sm, &h);
            if (h != 0.0) e[k++] = h;
            q = sm;
        }
        if (q != 0.0) e[k++] = q;
        m = k;
    }
    return m == 0 ? 0 : (e[m - 1] > 0.0 ? 1 : -1);
}

/* exact p*q*r as four doubles */
static inline void og_prod3(double p, double q, double r, double sg, double* t) {
    double s1, e1;
    og_two_prod(p, q, &s1, &e1);
    og_two_prod(s1, r, &t[0], &t[1]);
    og_two_prod(e1, r, &t[2], &t[3]);
    for (int k = 0; k < 4; ++k) t[k] *= sg;
}

/* sign of det[a; b; c] = a.(b x c), exactly */
static int og_det3_sign(v3 a, v3 b, v3 c) {
    double t[24];
    og_prod3(a.x, b.y, c.z, 1.0, t + 0);
    og_prod3(a.x, b.z, c.y, -1.0, t + 4);
    og_prod3(a.y, b.z, c.x, 1.0, t + 8);
    og_prod3(a.y, b.x, c.z, -1.0, t + 12);
    og_prod3(a.z, b.x, c.y, 1.0, t + 16);
    og_prod3(a.z, b.y, c.x, -1.0, t + 20);
    return og_exact_sign(t, 24);
}

/* sign of (bx-ax)(vy-ay) - (by-ay)(vx-ax), exactly */
static int og_orient2_sign(double ax, double ay, double bx, double by, double vx, double vy) {
    double d[4][2];
    og_two_sum(bx, -ax, &d[0][0], &d[0][1]);
    og_two_sum(vy, -ay, &d[1][0], &d[1][1]);
    og_two_sum(by, -ay, &d[2][0], &d[2][1]);
    og_two_sum(vx, -ax, &d[3][0], &d[3][1]);
    double t[16];
    int n = 0;
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) {
            og_two_prod(d[0][i], d[1][j], &t[n], &t[n + 1]);
            n += 2;
        }
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) {
            og_two_prod(d[2][i], d[3][j], &t[n], &t[n + 1]);
            t[n] = -t[n];
            t[n + 1] = -t[n + 1];
            n += 2;
        }
    return og_exact_sign(t, 16);
}

#define OG_U32 3.552713678800501e-15  /* 32 * 2^-53 */
#define OG_U8 8.881784197001252e-16   /* 8 * 2^-53 */
#define OG_TINY 1e-290

/* Decide the side value: keep the FP64 estimate s when it clears the error
 * bound, otherwise take the exact sign (0 -> exactly on the line). */
static inline double og_settle(double s, double bound, int exact_sign) {
    if (fabs(s) > bound) return s;
    if (exact_sign == 0) return 0.0;
    double m = fmax(fabs(s), 2.2250738585072014e-308);
    return exact_sign > 0 ? m : -m;
}

static const double OG_ATAN_C[20] = {
    1.0, 0.3333333333333333, 0.2, 0.14285714285714285, 0.1111111111111111,
    0.09090909090909091, 0.07692307692307693, 0.06666666666666667, 0.058823529411764705,
    0.05263157894736842, 0.047619047619047616, 0.043478260869565216, 0.04,
    0.037037037037037035, 0.034482758620689655, 0.03225806451612903, 0.030303030303030304,
    0.02857142857142857, 0.02702702702702703, 0.02564102564102564};
/* OG_ATAN_TH[n]: largest t^2 for which the terms k = 0..n reach 2^-56 relative. */
static const double OG_ATAN_TH[20] = {
    4.163336342344337e-17, 8.33000234328132e-09, 4.596981552458248e-06, 0.0001057159916729051,
    0.0006866613224549, 0.0023770807360687612, 0.005751393360079481, 0.011132588223807069,
    0.018578395538006495, 0.02795464321653044, 0.039019086539122956, 0.051485905388814555,
    0.06506692879763946, 0.07949448812181649, 0.09453198900334307, 0.10997706781109234,
    0.12566065265206888, 0.1414440078610017, 0.15721498531213599, 0.17288416032961332};

#define OG_TAN_PI_8 0.41421356237309503
#define OG_PI_4 0.7853981633974483
#define OG_PI_2 1.5707963267948966
#define OG_PI 3.141592653589793

/* atan(t) for |t| <= tan(pi/8): Maclaurin series, Horner in z = t^2. */
static double og_atan_series(double t) {
    double z = t * t;
    int n = 0;
    while (n < 19 && z > OG_ATAN_TH[n]) n++;
    double p = OG_ATAN_C[n];
    for (int k = n - 1; k >= 0; --k) p = fma(p, -z, OG_ATAN_C[k]);
    return t * p;
}

/* atan2 by octant reduction: |y|<=|x| swap, then t>tan(pi/8) -> (t-1)/(t+1) + pi/4. */
double og_atan2(double y, double x) {
    double ay = fabs(y), ax = fabs(x);
    int swap = ay > ax;
    double num = swap ? ax : ay, den = swap ? ay : ax;
    if (den == 0.0) return 0.0;
    double t = num / den;
    double r;
    if (t > OG_TAN_PI_8) {
        double u = (t - 1.0) / (t + 1.0);
        r = OG_PI_4 + og_atan_series(u);
    } else {
        r = og_atan_series(t);
    }
    if (swap) r = OG_PI_2 - r;
    if (x < 0.0) r = OG_PI - r;
    if (y < 0.0) r = -r;
    return r;
}

/* ---- spherical clip + area ---- */

static inline v3 og_sub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }

/* Triple product a.((b-a) x (c-a)) = a.(b x c), evaluated in the frame of a so
 * that tiny triangles keep full relative precision. */
static inline double og_triple(v3 a, v3 b, v3 c) { return og_dot(a, og_cross(og_sub(b, a), og_sub(c, a))); }

/* Orientation: sign of the fan sum of triple products (+1 counter-clockwise
 * seen from outside the sphere). */
static double og_orient_sph(const v3* c, int n) {
    double s = 0.0;
    for (int k = 1; k + 1 < n; ++k) s = s + og_triple(c[0], c[k], c[k + 1]);
    return s >= 0.0 ? 1.0 : -1.0;
}

/* Crossing weights below 2^-400 (side values settled to about DBL_MIN at both
 * ends of an edge) are scaled by 2^600, exactly, before they are combined:
 * unscaled, the squared norm underflows to 0 and the point becomes infinite.
 * The normalisation removes the factor; larger weights are left as they are. */
#define OG_ISECT_TINY 0x1p-400
#define OG_ISECT_SCALE 0x1p600

static inline v3 og_isect_sph(v3 a, double sa, v3 b, double sb) {
    if (sa == 0.0) return a;
    if (sb == 0.0) return b;
    double wa = fabs(sb), wb = fabs(sa);
    if (fmax(wa, wb) < OG_ISECT_TINY) { wa *= OG_ISECT_SCALE; wb *= OG_ISECT_SCALE; }
    v3 x;
    x.x = fma(wb, b.x, wa * a.x);
    x.y = fma(wb, b.y, wa * a.y);
    x.z = fma(wb, b.z, wa * a.z);
    /* normalised with one reciprocal and three products (one rounding more
       than three quotients, and the same sequence as the GPU coding) */
    double ir = 1.0 / sqrt(og_dot(x, x));
    x.x = x.x * ir; x.y = x.y * ir; x.z = x.z * ir;
    return x;
}

/* Side of v w.r.t. the great circle through ca, cb: FP64 value of
 * n.(v - ca) (n = ca x (cb - ca), pre-signed by the clip orientation) with an
 * exact sign whenever |value| <= eb * |v - ca|_1. */
static inline double og_side_sph(v3 nrm, v3 ca, v3 cb, double eb, int isig, v3 v) {
    v3 w = og_sub(v, ca);
    double s = og_dot(nrm, w);
    double bound = eb * (fabs(w.x) + fabs(w.y) + fabs(w.z)) + OG_TINY;
    if (fabs(s) > bound) return s;
    return og_settle(s, bound, isig * og_det3_sign(ca, cb, v));
}

/* Clip convex `subj` by convex `clip` (Sutherland-Hodgman); returns vertex
 * count, or -1 on capacity overflow. */
static int og_clip_sph(const v3* subj, int ns, const v3* clip, int nc, v3* res) {
    v3 ba[OG_MAXC], bb[OG_MAXC];
    v3* in = ba; v3* out = bb;
    for (int i = 0; i < ns; ++i) in[i] = subj[i];
    int n = ns;
    double sig = og_orient_sph(clip, nc);
    for (int k = 0; k < nc && n > 0; ++k) {
        /* half-space of edge c_k -> c_k+1: n = c_k x (c_k+1 - c_k), s(v) = n.(v - c_k) */
        v3 ck = clip[k], ck1 = clip[(k + 1) % nc];
        v3 d1 = og_sub(ck1, ck);
        v3 nrm = og_cross(ck, d1);
        if (sig < 0.0) { nrm.x = -nrm.x; nrm.y = -nrm.y; nrm.z = -nrm.z; }
        int isig = sig < 0.0 ? -1 : 1;
        double eb = OG_U32 * (fabs(ck.x) + fabs(ck.y) + fabs(ck.z)) * (fabs(d1.x) + fabs(d1.y) + fabs(d1.z));
        int m = 0;
        v3 prev = in[n - 1];
        double sp = og_side_sph(nrm, ck, ck1, eb, isig, prev);
        for (int i = 0; i < n; ++i) {
            v3 cur = in[i];
            double sc = og_side_sph(nrm, ck, ck1, eb, isig, cur);
            if (sc >= 0.0) {
                if (sp < 0.0) { if (m >= OG_MAXC) return -1; out[m++] = og_isect_sph(prev, sp, cur, sc); }
                if (m >= OG_MAXC) return -1;
                out[m++] = cur;
            } else if (sp >= 0.0) {
                if (m >= OG_MAXC) return -1;
                out[m++] = og_isect_sph(prev, sp, cur, sc);
            }
            prev = cur; sp = sc;
        }
        v3* t = in; in = out; out = t;
        n = m;
    }
    for (int i = 0; i < n; ++i) res[i] = in[i];
    return n;
}

/* Signed solid angle of a polygon (fan from vertex 0). */
static double og_area_sph_signed(const v3* v, int m) {
    if (m < 3) return 0.0;
    double re = 1.0, im = 0.0;
    v3 a = v[0];
    for (int k = 1; k + 1 < m; ++k) {
        v3 b = v[k], c = v[k + 1];
        double N = og_triple(a, b, c);
        double D = ((1.0 + og_dot(a, b)) + og_dot(b, c)) + og_dot(c, a);
        double re2 = fma(re, D, -(im * N));
        double im2 = fma(re, N, im * D);
        re = re2; im = im2;
    }
    return 2.0 * og_atan2(im, re);
}

/* ---- planar clip + area (z ignored) ---- */

static inline double og_cross2(double ax, double ay, double bx, double by) { return ax * by - ay * bx; }

static double og_area_pl_signed(const v3* v, int m);
static double og_orient_pl(const v3* c, int n) { return og_area_pl_signed(c, n) >= 0.0 ? 1.0 : -1.0; }

static inline v3 og_isect_pl(v3 a, double sa, v3 b, double sb) {
    if (sa == 0.0) return a;
    if (sb == 0.0) return b;
    double wa = fabs(sb), wb = fabs(sa);
    if (fmax(wa, wb) < OG_ISECT_TINY) { wa *= OG_ISECT_SCALE; wb *= OG_ISECT_SCALE; }
    double w = wa + wb;
    v3 x;
    x.x = fma(wb, b.x, wa * a.x) / w;
    x.y = fma(wb, b.y, wa * a.y) / w;
    x.z = 0.0;
    return x;
}

/* Side of v w.r.t. the directed line a -> b, signed by the clip orientation,
 * with an exact sign when the FP64 value is within its error bound. */
static inline double og_side_pl(v3 a, v3 b, double ex, double ey, int isig, v3 v) {
    double wx = v.x - a.x, wy = v.y - a.y;
    double s = og_cross2(ex, ey, wx, wy);
    if (isig < 0) s = -s;
    double bound = OG_U8 * (fabs(ex) * fabs(wy) + fabs(ey) * fabs(wx)) + OG_TINY;
    if (fabs(s) > bound) return s;
    return og_settle(s, bound, isig * og_orient2_sign(a.x, a.y, b.x, b.y, v.x, v.y));
}

static int og_clip_pl(const v3* subj, int ns, const v3* clip, int nc, v3* res) {
    v3 ba[OG_MAXC], bb[OG_MAXC];
    v3* in = ba; v3* out = bb;
    for (int i = 0; i < ns; ++i) in[i] = subj[i];
    int n = ns;
    double sig = og_orient_pl(clip, nc);
    for (int k = 0; k < nc && n > 0; ++k) {
        v3 a = clip[k], b = clip[(k + 1) % nc];
        double ex = b.x - a.x, ey = b.y - a.y;
        int isig = sig < 0.0 ? -1 : 1;
        int m = 0;
        v3 prev = in[n - 1];
        double sp = og_side_pl(a, b, ex, ey, isig, prev);
        for (int i = 0; i < n; ++i) {
            v3 cur = in[i];
            double sc = og_side_pl(a, b, ex, ey, isig, cur);
            if (sc >= 0.0) {
                if (sp < 0.0) { if (m >= OG_MAXC) return -1; out[m++] = og_isect_pl(prev, sp, cur, sc); }
                if (m >= OG_MAXC) return -1;
                out[m++] = cur;
            } else if (sp >= 0.0) {
                if (m >= OG_MAXC) return -1;
                out[m++] = og_isect_pl(prev, sp, cur, sc);
            }
            prev = cur; sp = sc;
        }
        v3* t = in; in = out; out = t;
        n = m;
    }
    for (int i = 0; i < n; ++i) res[i] = in[i];
    return n;
}

/* shoelace formula relative to v[0] */
static double og_area_pl_signed(const v3* v, int m) {
    if (m < 3) return 0.0;
    double s = 0.0;
    for (int k = 1; k + 1 < m; ++k)
        s = s + og_cross2(v[k].x - v[0].x, v[k].y - v[0].y, v[k + 1].x - v[0].x, v[k + 1].y - v[0].y);
    return 0.5 * s;
}

/* Intersection area of src cell (subject) with dst cell (clip); the reference's
 * DefaultIntersectionOperator (regridder.jl:96-103) passes (p_src, p_dst).
 * Returns the area signed by the subject's orientation, so a correct overlap
 * is positive; *ovf is set on clip capacity overflow. */
static double og_pair_area(int spherical, const v3* s, int ns, const v3* d, int nd, int* ovf) {
    v3 res[OG_MAXC];
    if (spherical) {
        int m = og_clip_sph(s, ns, d, nd, res);
        if (m < 0) { *ovf = 1; return 0.0; }
        return og_area_sph_signed(res, m) * og_orient_sph(s, ns);
    } else {
        int m = og_clip_pl(s, ns, d, nd, res);
        if (m < 0) { *ovf = 1; return 0.0; }
        return og_area_pl_signed(res, m) * og_orient_pl(s, ns);
    }
}

static double og_cell_area(int spherical, const v3* v, int n) {
    if (spherical) return og_area_sph_signed(v, n) * og_orient_sph(v, n);
    return og_area_pl_signed(v, n) * og_orient_pl(v, n);
}

/* ------------------------------------------------------------------------ */
/* Extents: spherical caps (grids.jl:245-287) and planar boxes.             */
/* ------------------------------------------------------------------------ */

typedef struct { v3 c; double r; double xmin, xmax, ymin, ymax; } og_ext;

static v3 og_normalize_libm(v3 a) {
    double n = sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    v3 r = {a.x / n, a.y / n, a.z / n};
    return r;
}

/* GeometryOps spherical_distance: angle between unit vectors. */
static double og_sdist(v3 a, v3 b) {
    v3 c = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    double s = sqrt(c.x * c.x + c.y * c.y + c.z * c.z);
    double d = a.x * b.x + a.y * b.y + a.z * b.z;
    return atan2(s, d);
}

/* GeometryOps UnitSpherical.slerp(a, b, 0.5) in its sin(t W)/sin(W) form:
 * (sin(W/2)/sin W)(a + b) with W the angle between a and b.  Coincident points
 * (W = 0, e.g. the repeated pole vertex of a lon-lat pole row) give `a`;
 * antipodal points give the (near) zero vector, whose spherical_distance to
 * any centre is atan2(0, 0) = 0. */
static v3 og_mid(v3 a, v3 b) {
    double w = og_sdist(a, b);
    if (w == 0.0) return a;
    double k = sin(0.5 * w) / sin(w);
    v3 s = {k * (a.x + b.x), k * (a.y + b.y), k * (a.z + b.z)};
    return s;
}

static og_ext og_full_sphere(void) {
    og_ext e;
    e.c.x = 0; e.c.y = 0; e.c.z = 1;
    e.r = nextafter(OG_PI, INFINITY);
    e.xmin = -INFINITY; e.xmax = INFINITY; e.ymin = -INFINITY; e.ymax = INFINITY;
    return e;
}

/* _spherical_cap(p1..p4, perimeter) grids.jl:256-273: centre = normalize(mean
 * of 4 corners); radius = 1.0001 * max distance to corners, edge midpoints and
 * perimeter points. */
typedef struct {
    double d;
    v3 c;
} og_capacc;

static og_capacc og_cap_begin(v3 p1, v3 p2, v3 p3, v3 p4) {
    og_capacc a;
    v3 m = {(p1.x + p2.x + p3.x + p4.x) / 4, (p1.y + p2.y + p3.y + p4.y) / 4, (p1.z + p2.z + p3.z + p4.z) / 4};
    a.c = og_normalize_libm(m);
    v3 pts[8] = {p1, p2, p3, p4, og_mid(p1, p2), og_mid(p2, p3), og_mid(p3, p4), og_mid(p4, p1)};
    double d = 0.0;
    for (int k = 0; k < 8; ++k) { double t = og_sdist(a.c, pts[k]); d = (t > d || t != t) ? t : d; }
    a.d = d;
    return a;
}
static inline void og_cap_add(og_capacc* a, v3 p) {
    double t = og_sdist(a->c, p);
    if (t > a->d || t != t) a->d = t;
}
static og_ext og_cap_end(og_capacc a) {
    og_ext e;
    e.c = a.c; e.r = a.d * 1.0001;
    e.xmin = e.xmax = e.ymin = e.ymax = 0;
    return e;
}

/* GeometryOps UnitSpherical._intersects(cap, cap): centre distance <= r1 + r2. */
static inline int og_pred(int spherical, const og_ext* a, const og_ext* b) {
    if (spherical) return og_sdist(a->c, b->c) <= a->r + b->r;
    return a->xmin <= b->xmax && b->xmin <= a->xmax && a->ymin <= b->ymax && b->ymin <= a->ymax;
}

/* ------------------------------------------------------------------------ */
/* HEALPix geometry (Gorski et al. 2005): nested pixel -> 4 corners N,W,S,E. */
/* ------------------------------------------------------------------------ */

static const int OG_JRLL[12] = {2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4};
static const int OG_JPLL[12] = {1, 3, 5, 7, 0, 2, 4, 6, 1, 3, 5, 7};

static int64_t og_compact_bits(int64_t v) {
    int64_t r = 0;
    for (int b = 0; b < 31; ++b) r |= ((v >> (2 * b)) & 1) << b;
    return r;
}

static void og_nest2xyf(int64_t nside, int64_t pix, int64_t* ix, int64_t* iy, int* face) {
    int64_t npface = nside * nside;
    *face = (int)(pix / npface);
    int64_t ipf = pix % npface;
    *ix = og_compact_bits(ipf);
    *iy = og_compact_bits(ipf >> 1);
}

/* face-normalised (x, y) in [0,1]^2 -> unit vector */
static v3 og_hp_loc2vec(double x, double y, int face) {
    double jr = OG_JRLL[face] - x - y;
    double nr, z, sth;
    if (jr < 1.0) {
        nr = jr;
        double tmp = nr * nr / 3.0;
        z = 1.0 - tmp;
        sth = sqrt(tmp * (2.0 - tmp));
    } else if (jr > 3.0) {
        nr = 4.0 - jr;
        double tmp = nr * nr / 3.0;
        z = tmp - 1.0;
        sth = sqrt(tmp * (2.0 - tmp));
    } else {
        nr = 1.0;
        z = (2.0 - jr) * 2.0 / 3.0;
        sth = sqrt((1.0 - z) * (1.0 + z));
    }
    double tmp = OG_JPLL[face] * nr + x - y;
    if (tmp < 0) tmp += 8;
    if (tmp >= 8) tmp -= 8;
    double phi = (nr < 1e-15) ? 0.0 : (OG_PI_4 * tmp) / nr;
    v3 v = {sth * cos(phi), sth * sin(phi), z};
    return v;
}

void og_healpix_corners(int64_t nside, int64_t pix_nested, double* out12) {
    int64_t ix, iy; int face;
    og_nest2xyf(nside, pix_nested, &ix, &iy, &face);
    double ns = (double)nside;
    v3 c[4];
    c[0] = og_hp_loc2vec((ix + 1) / ns, (iy + 1) / ns, face); /* N */
    c[1] = og_hp_loc2vec((ix) / ns, (iy + 1) / ns, face);     /* W */
    c[2] = og_hp_loc2vec((ix) / ns, (iy) / ns, face);         /* S */
    c[3] = og_hp_loc2vec((ix + 1) / ns, (iy) / ns, face);     /* E */
    for (int k = 0; k < 4; ++k) { out12[3 * k] = c[k].x; out12[3 * k + 1] = c[k].y; out12[3 * k + 2] = c[k].z; }
}

int64_t og_healpix_nest2ring(int64_t nside, int64_t pix_nested) {
    int64_t ix, iy; int face;
    og_nest2xyf(nside, pix_nested, &ix, &iy, &face);
    int64_t nl4 = 4 * nside, npix = 12 * nside * nside, ncap = 2 * nside * (nside - 1);
    int64_t jr = (int64_t)OG_JRLL[face] * nside - ix - iy - 1;
    int64_t nr, nbefore, kshift;
    if (jr < nside) { nr = jr; nbefore = 2 * nr * (nr - 1); kshift = 0; }
    else if (jr > 3 * nside) { nr = nl4 - jr; nbefore = npix - 2 * (nr + 1) * nr; kshift = 0; }
    else { nr = nside; nbefore = ncap + (jr - nside) * nl4; kshift = (jr - nside) & 1; }
    int64_t jp = ((int64_t)OG_JPLL[face] * nr + ix - iy + 1 + kshift) / 2;
    if (jp > nl4) jp -= nl4;
    if (jp < 1) jp += nl4;
    return nbefore + jp - 1;
}

/* ------------------------------------------------------------------------ */
/* Grids and trees.                                                         */
/* ------------------------------------------------------------------------ */

enum { OG_CURVI = 0, OG_HEALPIX = 1, OG_POLYS = 2 };

/* Grid description (host pointers).  Curvilinear blocks: point (i,j) of block
 * b at points[(block_point_off[b] + i + j*(nx+1)) * dim]; cell (i,j) has global
 * index block_cell_off[b] + i + j*nx and ring p(i,j),p(i+1,j),p(i+1,j+1),p(i,j+1)
 * (grids.jl:77-83, interfaces.jl:241-243, ClimaCoreExt.jl:56-61).  HEALPix and
 * polygon grids: poly_verts[(cell*maxv + k)*dim], nverts[cell] (NULL -> maxv). */
typedef struct {
    int32_t kind, manifold, nblocks, nested;
    int32_t maxv, full_sphere_root, dim, pad;
    int64_t ncells, nside;
    const int64_t* block_nx;
    const int64_t* block_ny;
    const int64_t* block_point_off;
    const int64_t* block_cell_off;
    const double* points;
    const int32_t* nverts;
    const double* poly_verts;
} og_grid;

typedef struct {
    int8_t type;  /* 0 toplevel multi-block, 1 quad range, 2 hp root, 3 hp node, 4 flat */
    int8_t full;  /* node_extent overridden by the full sphere (KnownFullSphereExtentWrapper) */
    int32_t block;
    int32_t level;
    int64_t i0, i1, j0, j1;
    int64_t pixel;
} og_node;

typedef struct {
    const og_grid* g;
    int spherical;
    int hp_L;              /* leaf level of the HEALPix tree */
    int64_t par_threshold_den; /* nthreads * 32 */
    og_ext* cell_ext;      /* cached leaf extents per global cell index */
    int64_t* hp_ring_of_nested; /* nested leaf pixel -> output index */
} og_tree;

static v3 og_gpoint(const og_grid* g, int b, int64_t i, int64_t j) {
    int64_t nx = g->block_nx[b];
    const double* p = g->points + (g->block_point_off[b] + i + j * (nx + 1)) * g->dim;
    v3 v = {p[0], p[1], g->dim == 3 ? p[2] : 0.0};
    return v;
}

/* Vertices of global cell `idx` in ring order; returns count. */
static int og_cell_verts(const og_grid* g, int64_t idx, v3* out) {
    if (g->kind == OG_CURVI) {
        int b = 0;
        while (b + 1 < g->nblocks && idx >= g->block_cell_off[b + 1]) b++;
        int64_t loc = idx - g->block_cell_off[b];
        int64_t nx = g->block_nx[b];
        int64_t i = loc % nx, j = loc / nx;
        out[0] = og_gpoint(g, b, i, j);
        out[1] = og_gpoint(g, b, i + 1, j);
        out[2] = og_gpoint(g, b, i + 1, j + 1);
        out[3] = og_gpoint(g, b, i, j + 1);
        return 4;
    }
    int n = g->nverts ? g->nverts[idx] : g->maxv;
    for (int k = 0; k < n; ++k) {
        const double* p = g->poly_verts + (idx * g->maxv + k) * g->dim;
        out[k].x = p[0]; out[k].y = p[1]; out[k].z = g->dim == 3 ? p[2] : 0.0;
    }
    return n;
}

/* cell_range_extent (grids.jl:279-287 spherical, :148-152 planar) over cells
 * [i0..i1] x [j0..j1] of block b. */
static og_ext og_range_extent(const og_tree* t, int b, int64_t i0, int64_t i1, int64_t j0, int64_t j1) {
    const og_grid* g = t->g;
    int64_t imin = i0, imax = i1 + 1, jmin = j0, jmax = j1 + 1;
    if (!t->spherical) {
        og_ext e;
        e.xmin = INFINITY; e.xmax = -INFINITY; e.ymin = INFINITY; e.ymax = -INFINITY;
        for (int64_t j = jmin; j <= jmax; ++j)
            for (int64_t i = imin; i <= imax; ++i) {
                v3 p = og_gpoint(g, b, i, j);
                if (p.x < e.xmin) e.xmin = p.x;
                if (p.x > e.xmax) e.xmax = p.x;
                if (p.y < e.ymin) e.ymin = p.y;
                if (p.y > e.ymax) e.ymax = p.y;
            }
        e.c.x = e.c.y = e.c.z = 0; e.r = 0;
        return e;
    }
    og_capacc a = og_cap_begin(og_gpoint(g, b, imin, jmin), og_gpoint(g, b, imax, jmin),
                               og_gpoint(g, b, imax, jmax), og_gpoint(g, b, imin, jmax));
    /* CurvilinearGridPerimeterPoints (grids.jl:205-232): west and east columns,
     * then the interiors of the south and north rows. */
    for (int64_t j = jmin; j <= jmax; ++j) { og_cap_add(&a, og_gpoint(g, b, imin, j)); og_cap_add(&a, og_gpoint(g, b, imax, j)); }
    for (int64_t i = imin + 1; i < imax; ++i) { og_cap_add(&a, og_gpoint(g, b, i, jmin)); og_cap_add(&a, og_gpoint(g, b, i, jmax)); }
    return og_cap_end(a);
}

/* circle_from_four_corners(corners, ()) with corners in (N,W,S,E) order as
 * returned for a HEALPix pixel; reordered raw[1],raw[3],raw[4],raw[2]
 * (grids.jl:245-251). */
static og_ext og_cap_from_hp_corners(const v3* c) {
    og_capacc a = og_cap_begin(c[0], c[2], c[3], c[1]);
    return og_cap_end(a);
}

static og_ext og_poly_extent(const og_tree* t, int64_t idx) {
    v3 v[OG_MAXV];
    int n = og_cell_verts(t->g, idx, v);
    og_ext e;
    if (n == 0) {
        /* a cell without vertices (a ghost slot, like the padding cells of the
           reference's folded grids) is in no extent: no pair ever tests true */
        e.c.x = e.c.y = 0; e.c.z = 1; e.r = -INFINITY;
        e.xmin = e.ymin = INFINITY; e.xmax = e.ymax = -INFINITY;
        return e;
    }
    if (!t->spherical) {
        e.xmin = INFINITY; e.xmax = -INFINITY; e.ymin = INFINITY; e.ymax = -INFINITY;
        for (int k = 0; k < n; ++k) {
            if (v[k].x < e.xmin) e.xmin = v[k].x;
            if (v[k].x > e.xmax) e.xmax = v[k].x;
            if (v[k].y < e.ymin) e.ymin = v[k].y;
            if (v[k].y > e.ymax) e.ymax = v[k].y;
        }
        e.c.x = e.c.y = e.c.z = 0; e.r = 0;
        return e;
    }
    /* ExplicitPolygonGrid{Spherical} cell_range_extent (grids.jl:133-146) over
     * the closed ring (first vertex repeated). */
    v3 s = {0, 0, 0};
    for (int k = 0; k <= n; ++k) { v3 p = v[k % n]; s.x += p.x; s.y += p.y; s.z += p.z; }
    s.x /= (n + 1); s.y /= (n + 1); s.z /= (n + 1);
    e.c = og_normalize_libm(s);
    double d = 0;
    for (int k = 0; k < n; ++k) { double q = og_sdist(e.c, v[k]); if (q > d || q != q) d = q; }
    e.r = d * 1.0001;
    e.xmin = e.xmax = e.ymin = e.ymax = 0;
    return e;
}

static int og_isleaf(const og_tree* t, const og_node* n) {
    switch (n->type) {
        case 1: return (n->i1 - n->i0 + 1) <= 2 && (n->j1 - n->j0 + 1) <= 2;
        case 3: return n->level == t->hp_L;
        case 4: return 1;
        default: return 0;
    }
}

static int og_children(const og_tree* t, const og_node* n, og_node* ch) {
    const og_grid* g = t->g;
    if (n->type == 0) {
        for (int b = 0; b < g->nblocks; ++b) {
            og_node c = {1, 0, b, 0, 0, g->block_nx[b] - 1, 0, g->block_ny[b] - 1, 0};
            ch[b] = c;
        }
        return g->nblocks;
    }
    if (n->type == 2) {
        for (int k = 0; k < 12; ++k) { og_node c = {3, 0, 0, 0, 0, 0, 0, 0, k}; ch[k] = c; }
        return 12;
    }
    if (n->type == 3) {
        for (int k = 0; k < 4; ++k) { og_node c = {3, 0, 0, n->level + 1, 0, 0, 0, 0, 4 * n->pixel + k}; ch[k] = c; }
        return 4;
    }
    /* type 1: TopDownQuadtreeCursor getchild (quadtree_cursors.jl:258-287) */
    int64_t li = n->i1 - n->i0 + 1, lj = n->j1 - n->j0 + 1;
    og_node base = *n; base.full = 0;
    if (li == 1) {
        int64_t s = lj / 2;
        ch[0] = base; ch[0].j1 = n->j0 + s - 1;
        ch[1] = base; ch[1].j0 = n->j0 + s;
        return 2;
    }
    if (lj == 1) {
        int64_t s = li / 2;
        ch[0] = base; ch[0].i1 = n->i0 + s - 1;
        ch[1] = base; ch[1].i0 = n->i0 + s;
        return 2;
    }
    int64_t si = li / 2, sj = lj / 2;
    for (int k = 0; k < 4; ++k) ch[k] = base;
    ch[0].i1 = n->i0 + si - 1; ch[0].j1 = n->j0 + sj - 1;
    ch[1].i1 = n->i0 + si - 1; ch[1].j0 = n->j0 + sj;
    ch[2].i0 = n->i0 + si;     ch[2].j1 = n->j0 + sj - 1;
    ch[3].i0 = n->i0 + si;     ch[3].j0 = n->j0 + sj;
    return 4;
}

static og_ext og_node_extent(const og_tree* t, const og_node* n) {
    if (n->full || n->type == 0 || n->type == 2) return og_full_sphere();
    if (n->type == 1) return og_range_extent(t, n->block, n->i0, n->i1, n->j0, n->j1);
    if (n->type == 3) {
        if (n->level == t->hp_L) return t->cell_ext[t->hp_ring_of_nested[n->pixel]];
        double c12[12];
        og_healpix_corners((int64_t)1 << n->level, n->pixel, c12);
        v3 c[4];
        for (int k = 0; k < 4; ++k) { c[k].x = c12[3 * k]; c[k].y = c12[3 * k + 1]; c[k].z = c12[3 * k + 2]; }
        return og_cap_from_hp_corners(c);
    }
    /* flat: union of all polygon extents */
    og_ext e;
    if (!t->spherical) {
        e.xmin = INFINITY; e.xmax = -INFINITY; e.ymin = INFINITY; e.ymax = -INFINITY;
        for (int64_t i = 0; i < t->g->ncells; ++i) {
            og_ext c = t->cell_ext[i];
            if (c.xmin < e.xmin) e.xmin = c.xmin;
            if (c.xmax > e.xmax) e.xmax = c.xmax;
            if (c.ymin < e.ymin) e.ymin = c.ymin;
            if (c.ymax > e.ymax) e.ymax = c.ymax;
        }
        e.c.x = e.c.y = e.c.z = 0; e.r = 0;
        return e;
    }
    return og_full_sphere();
}

/* leaf cells of a leaf node */
static int og_leaf_cells(const og_tree* t, const og_node* n, int64_t* idx, int cap) {
    const og_grid* g = t->g;
    if (n->type == 1) {
        int c = 0;
        int64_t nx = g->block_nx[n->block];
        for (int64_t j = n->j0; j <= n->j1; ++j)
            for (int64_t i = n->i0; i <= n->i1; ++i) idx[c++] = g->block_cell_off[n->block] + i + j * nx;
        return c;
    }
    if (n->type == 3) { idx[0] = t->hp_ring_of_nested[n->pixel]; return 1; }
    (void)cap;
    return -1; /* flat: all cells, handled by caller */
}

typedef struct { int64_t* a; int64_t n, cap; } og_vec;
static void og_push2(og_vec* v, int64_t x, int64_t y) {
    if (v->n + 2 > v->cap) {
        v->cap = v->cap ? 2 * v->cap : 1024;
        v->a = (int64_t*)realloc(v->a, sizeof(int64_t) * v->cap);
    }
    v->a[v->n++] = x; v->a[v->n++] = y;
}

static void og_leaf_pairs(const og_tree* t1, const og_node* n1, const og_tree* t2, const og_node* n2, og_vec* out) {
    int64_t c1[4], c2[4];
    int k1 = og_leaf_cells(t1, n1, c1, 4), k2 = og_leaf_cells(t2, n2, c2, 4);
    int64_t m1 = k1 < 0 ? t1->g->ncells : k1, m2 = k2 < 0 ? t2->g->ncells : k2;
    for (int64_t a = 0; a < m1; ++a) {
        int64_t i1 = k1 < 0 ? a : c1[a];
        for (int64_t b = 0; b < m2; ++b) {
            int64_t i2 = k2 < 0 ? b : c2[b];
            if (og_pred(t1->spherical, &t1->cell_ext[i1], &t2->cell_ext[i2])) og_push2(out, i1, i2);
        }
    }
}

/* GeometryOps STI.dual_depth_first_search restated: descend both trees while
 * the child extents intersect; emit leaf-cell pairs whose extents intersect. */
static void og_dual_dfs(const og_tree* t1, og_node n1, const og_tree* t2, og_node n2, og_vec* out) {
    int l1 = og_isleaf(t1, &n1), l2 = og_isleaf(t2, &n2);
    og_node ch1[12], ch2[12];
    if (l1 && l2) { og_leaf_pairs(t1, &n1, t2, &n2, out); return; }
    if (l1) {
        og_ext e1 = og_node_extent(t1, &n1);
        int k2 = og_children(t2, &n2, ch2);
        for (int b = 0; b < k2; ++b) {
            og_ext e2 = og_node_extent(t2, &ch2[b]);
            if (og_pred(t1->spherical, &e1, &e2)) og_dual_dfs(t1, n1, t2, ch2[b], out);
        }
        return;
    }
    if (l2) {
        og_ext e2 = og_node_extent(t2, &n2);
        int k1 = og_children(t1, &n1, ch1);
        for (int a = 0; a < k1; ++a) {
            og_ext e1 = og_node_extent(t1, &ch1[a]);
            if (og_pred(t1->spherical, &e1, &e2)) og_dual_dfs(t1, ch1[a], t2, n2, out);
        }
        return;
    }
    int k1 = og_children(t1, &n1, ch1), k2 = og_children(t2, &n2, ch2);
    og_ext e2s[12];
    for (int b = 0; b < k2; ++b) e2s[b] = og_node_extent(t2, &ch2[b]);
    for (int a = 0; a < k1; ++a) {
        og_ext e1 = og_node_extent(t1, &ch1[a]);
        for (int b = 0; b < k2; ++b)
            if (og_pred(t1->spherical, &e1, &e2s[b])) og_dual_dfs(t1, ch1[a], t2, ch2[b], out);
    }
}

/* should_parallelize (quadtree_cursors.jl:17-25, interfaces.jl:80-81) */
static int og_should_par(const og_tree* t, const og_node* n, const og_ext* e) {
    if (n->type == 1) {
        int64_t total = t->g->block_nx[n->block] * t->g->block_ny[n->block];
        int64_t th = total / t->par_threshold_den;
        if (th < 1) th = 1;
        return (n->i1 - n->i0 + 1) * (n->j1 - n->j0 + 1) <= th;
    }
    if (!t->spherical) return 0;
    return (2 * OG_PI * (1 - cos(e->r))) < OG_PI;
}

typedef struct { og_node a, b; } og_task;
typedef struct { og_task* t; int64_t n, cap; } og_tasks;

/* multithreaded_dual_depth_first_search (MultithreadedDualDepthFirstSearch.jl:12-42) */
static void og_mt_dfs(const og_tree* t1, og_node n1, og_ext e1, const og_tree* t2, og_node n2, og_ext e2, og_tasks* ts) {
    int push = og_isleaf(t1, &n1) || og_isleaf(t2, &n2) ||
               (og_should_par(t1, &n1, &e1) && og_should_par(t2, &n2, &e2));
    if (push) {
        if (ts->n == ts->cap) { ts->cap = ts->cap ? 2 * ts->cap : 256; ts->t = (og_task*)realloc(ts->t, sizeof(og_task) * ts->cap); }
        ts->t[ts->n].a = n1; ts->t[ts->n].b = n2; ts->n++;
        return;
    }
    og_node ch1[12], ch2[12];
    int k1 = og_children(t1, &n1, ch1), k2 = og_children(t2, &n2, ch2);
    og_ext e2s[12];
    for (int b = 0; b < k2; ++b) e2s[b] = og_node_extent(t2, &ch2[b]);
    for (int a = 0; a < k1; ++a) {
        og_ext ce1 = og_node_extent(t1, &ch1[a]);
        for (int b = 0; b < k2; ++b)
            if (og_pred(t1->spherical, &ce1, &e2s[b])) og_mt_dfs(t1, ch1[a], ce1, t2, ch2[b], e2s[b], ts);
    }
}

static og_node og_root(const og_grid* g) {
    og_node r;
    memset(&r, 0, sizeof(r));
    if (g->kind == OG_CURVI) {
        if (g->nblocks > 1) { r.type = 0; r.full = 1; }
        else { r.type = 1; r.block = 0; r.i1 = g->block_nx[0] - 1; r.j1 = g->block_ny[0] - 1; r.full = (int8_t)g->full_sphere_root; }
    } else if (g->kind == OG_HEALPIX) {
        r.type = 2; r.full = 1;
    } else {
        r.type = 4;
    }
    return r;
}

static void og_tree_init(og_tree* t, const og_grid* g, int nthreads) {
    memset(t, 0, sizeof(*t));
    t->g = g;
    t->spherical = g->manifold == 1;
    t->par_threshold_den = (int64_t)nthreads * 32;
    t->cell_ext = (og_ext*)malloc(sizeof(og_ext) * (g->ncells > 0 ? g->ncells : 1));
    if (g->kind == OG_HEALPIX) {
        int L = 0;
        while (((int64_t)1 << L) < g->nside) L++;
        t->hp_L = L;
        t->hp_ring_of_nested = (int64_t*)malloc(sizeof(int64_t) * g->ncells);
        for (int64_t p = 0; p < g->ncells; ++p)
            t->hp_ring_of_nested[p] = g->nested ? p : og_healpix_nest2ring(g->nside, p);
    }
    /* cache leaf extents: identical to recomputing them on every visit */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < g->ncells; ++i) {
        if (g->kind == OG_CURVI) {
            int b = 0;
            while (b + 1 < g->nblocks && i >= g->block_cell_off[b + 1]) b++;
            int64_t loc = i - g->block_cell_off[b], nx = g->block_nx[b];
            t->cell_ext[i] = og_range_extent(t, b, loc % nx, loc % nx, loc / nx, loc / nx);
        } else if (g->kind == OG_HEALPIX) {
            v3 c[OG_MAXV];
            og_cell_verts(g, i, c);
            t->cell_ext[i] = og_cap_from_hp_corners(c);
        } else {
            t->cell_ext[i] = og_poly_extent(t, i);
        }
    }
}

static void og_tree_free(og_tree* t) {
    free(t->cell_ext);
    free(t->hp_ring_of_nested);
}

/* ------------------------------------------------------------------------ */
/* Regridder build (regridder.jl:125-163).                                  */
/* ------------------------------------------------------------------------ */

typedef struct {
    int64_t nd, ns, nnz, ncand;
    int64_t* colptr;  /* CSC of A (nd x ns): column = src cell, rows sorted */
    int64_t* rowval;
    double* nzval;
    double* dst_areas;
    double* src_areas;
    int64_t clip_overflows;
} og_regridder;

/* Candidate search only: returns pairs (src, dst) in *out (2 per pair).
 * use_tree = 0 replaces the dual DFS by the exhaustive leaf test (for tests). */
int64_t og_candidates(const og_grid* dst, const og_grid* src, int use_tree, int nthreads, int64_t** out) {
    og_tree ts, td;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    int nth = omp_get_max_threads();
#else
    int nth = 1;
#endif
    og_tree_init(&ts, src, nth);
    og_tree_init(&td, dst, nth);
    og_vec all = {0, 0, 0};
    if (use_tree) {
        og_node rs = og_root(src), rd = og_root(dst);
        og_tasks tasks = {0, 0, 0};
        og_mt_dfs(&ts, rs, og_node_extent(&ts, &rs), &td, rd, og_node_extent(&td, &rd), &tasks);
        og_vec* per = (og_vec*)calloc(tasks.n > 0 ? tasks.n : 1, sizeof(og_vec));
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t k = 0; k < tasks.n; ++k) og_dual_dfs(&ts, tasks.t[k].a, &td, tasks.t[k].b, &per[k]);
        int64_t tot = 0;
        for (int64_t k = 0; k < tasks.n; ++k) tot += per[k].n;
        all.a = (int64_t*)malloc(sizeof(int64_t) * (tot > 0 ? tot : 1));
        for (int64_t k = 0; k < tasks.n; ++k) {
            if (per[k].n) memcpy(all.a + all.n, per[k].a, sizeof(int64_t) * per[k].n);
            all.n += per[k].n;
            free(per[k].a);
        }
        free(per);
        free(tasks.t);
    } else {
        int64_t nsrc = src->ncells;
        og_vec* per = (og_vec*)calloc(nsrc > 0 ? nsrc : 1, sizeof(og_vec));
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t i = 0; i < nsrc; ++i)
            for (int64_t j = 0; j < dst->ncells; ++j)
                if (og_pred(ts.spherical, &ts.cell_ext[i], &td.cell_ext[j])) og_push2(&per[i], i, j);
        int64_t tot = 0;
        for (int64_t k = 0; k < nsrc; ++k) tot += per[k].n;
        all.a = (int64_t*)malloc(sizeof(int64_t) * (tot > 0 ? tot : 1));
        for (int64_t k = 0; k < nsrc; ++k) {
            if (per[k].n) memcpy(all.a + all.n, per[k].a, sizeof(int64_t) * per[k].n);
            all.n += per[k].n;
            free(per[k].a);
        }
        free(per);
    }
    og_tree_free(&ts);
    og_tree_free(&td);
    *out = all.a;
    return all.n / 2;
}

void og_free_buffer(void* p) { free(p); }

/* SparseArrays.sparse(I=dst, J=src, V, nd, ns): CSC by counting sort on the
 * column, rows ascending within a column, duplicates combined with +. */
static void og_sparse(og_regridder* R, const int64_t* i_dst, const int64_t* i_src, const double* v, int64_t n) {
    int64_t nd = R->nd, ns = R->ns;
    int64_t* cnt = (int64_t*)calloc(ns + 1, sizeof(int64_t));
    for (int64_t k = 0; k < n; ++k) cnt[i_src[k] + 1]++;
    for (int64_t j = 0; j < ns; ++j) cnt[j + 1] += cnt[j];
    int64_t* pos = (int64_t*)malloc(sizeof(int64_t) * (ns + 1));
    memcpy(pos, cnt, sizeof(int64_t) * (ns + 1));
    int64_t* rows = (int64_t*)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
    double* vals = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
    for (int64_t k = 0; k < n; ++k) { int64_t p = pos[i_src[k]]++; rows[p] = i_dst[k]; vals[p] = v[k]; }
    /* sort rows within each column (insertion sort: columns are short) and combine duplicates */
    R->colptr = (int64_t*)malloc(sizeof(int64_t) * (ns + 1));
    R->rowval = (int64_t*)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
    R->nzval = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
    int64_t out = 0;
    R->colptr[0] = 0;
    for (int64_t j = 0; j < ns; ++j) {
        int64_t a = cnt[j], b = cnt[j + 1];
        for (int64_t p = a + 1; p < b; ++p) {
            int64_t r = rows[p]; double x = vals[p]; int64_t q = p - 1;
            while (q >= a && rows[q] > r) { rows[q + 1] = rows[q]; vals[q + 1] = vals[q]; q--; }
            rows[q + 1] = r; vals[q + 1] = x;
        }
        for (int64_t p = a; p < b; ++p) {
            if (out > R->colptr[j] && R->rowval[out - 1] == rows[p]) R->nzval[out - 1] += vals[p];
            else { R->rowval[out] = rows[p]; R->nzval[out] = vals[p]; out++; }
        }
        R->colptr[j + 1] = out;
    }
    R->nnz = out;
    (void)nd;
    free(cnt); free(pos); free(rows); free(vals);
}

og_regridder* og_build(const og_grid* dst, const og_grid* src, int normalize, int use_tree, int nthreads) {
    og_regridder* R = (og_regridder*)calloc(1, sizeof(og_regridder));
    R->nd = dst->ncells; R->ns = src->ncells;
    int spherical = (dst->manifold == 1) || (src->manifold == 1);
    int64_t* cand = NULL;
    int64_t nc = og_candidates(dst, src, use_tree, nthreads, &cand);
    R->ncand = nc;
    double* area = (double*)malloc(sizeof(double) * (nc > 0 ? nc : 1));
    int64_t ovf_total = 0;
    /* chunked per-pair clip + area (intersection_areas.jl:4-32, :86-113) */
#pragma omp parallel for schedule(dynamic, 4096) reduction(+ : ovf_total)
    for (int64_t k = 0; k < nc; ++k) {
        v3 s[OG_MAXV], d[OG_MAXV];
        int ns_ = og_cell_verts(src, cand[2 * k], s);
        int nd_ = og_cell_verts(dst, cand[2 * k + 1], d);
        int ovf = 0;
        area[k] = og_pair_area(spherical, s, ns_, d, nd_, &ovf);
        ovf_total += ovf;
    }
    R->clip_overflows = ovf_total;
    /* keep area > 0, concatenated in candidate order */
    int64_t m = 0;
    int64_t* id = (int64_t*)malloc(sizeof(int64_t) * (nc > 0 ? nc : 1));
    int64_t* is = (int64_t*)malloc(sizeof(int64_t) * (nc > 0 ? nc : 1));
    for (int64_t k = 0; k < nc; ++k)
        if (area[k] > 0) { is[m] = cand[2 * k]; id[m] = cand[2 * k + 1]; area[m] = area[k]; m++; }
    og_sparse(R, id, is, area, m);
    free(id); free(is); free(area); free(cand);
    /* per-cell areas (regridder.jl:165-178) */
    R->dst_areas = (double*)malloc(sizeof(double) * (R->nd > 0 ? R->nd : 1));
    R->src_areas = (double*)malloc(sizeof(double) * (R->ns > 0 ? R->ns : 1));
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < R->nd; ++i) { v3 v[OG_MAXV]; int n = og_cell_verts(dst, i, v); R->dst_areas[i] = og_cell_area(spherical, v, n); }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < R->ns; ++i) { v3 v[OG_MAXV]; int n = og_cell_verts(src, i, v); R->src_areas[i] = og_cell_area(spherical, v, n); }
    if (normalize) {
        /* normalize!(::Regridder) regridder.jl:54-62: maximum(A) includes implicit zeros */
        double mx = (R->nnz < R->nd * R->ns) ? 0.0 : -INFINITY;
        for (int64_t k = 0; k < R->nnz; ++k) if (R->nzval[k] > mx) mx = R->nzval[k];
        for (int64_t k = 0; k < R->nnz; ++k) R->nzval[k] /= mx;
        for (int64_t i = 0; i < R->nd; ++i) R->dst_areas[i] /= mx;
        for (int64_t i = 0; i < R->ns; ++i) R->src_areas[i] /= mx;
    }
    return R;
}

int64_t og_nnz(const og_regridder* R) { return R->nnz; }
int64_t og_ncand(const og_regridder* R) { return R->ncand; }
int64_t og_overflows(const og_regridder* R) { return R->clip_overflows; }

void og_get_csc(const og_regridder* R, int64_t* colptr, int64_t* rowval, double* nzval) {
    memcpy(colptr, R->colptr, sizeof(int64_t) * (R->ns + 1));
    if (R->nnz) {
        memcpy(rowval, R->rowval, sizeof(int64_t) * R->nnz);
        memcpy(nzval, R->nzval, sizeof(double) * R->nnz);
    }
}

void og_get_areas(const og_regridder* R, double* dst_areas, double* src_areas) {
    memcpy(dst_areas, R->dst_areas, sizeof(double) * R->nd);
    memcpy(src_areas, R->src_areas, sizeof(double) * R->ns);
}

void og_free(og_regridder* R) {
    if (!R) return;
    free(R->colptr); free(R->rowval); free(R->nzval); free(R->dst_areas); free(R->src_areas);
    free(R);
}

/* ------------------------------------------------------------------------ */
/* Apply (regrid.jl:63-118, regridder.jl:49-50).                            */
/* Fields: element (cell c, field f) at base[c*stride_cell + f*stride_field]. */
/* ------------------------------------------------------------------------ */

/* forward: mul!(y, A, x) as the stdlib CSC kernel (column scatter), then ./ a_d */
static void og_apply_fwd1(const og_regridder* R, const double* x, int64_t sx, double* y, int64_t sy, int normalize) {
    for (int64_t i = 0; i < R->nd; ++i) y[i * sy] = 0.0;
    for (int64_t j = 0; j < R->ns; ++j) {
        double xj = x[j * sx];
        for (int64_t k = R->colptr[j]; k < R->colptr[j + 1]; ++k) y[R->rowval[k] * sy] += R->nzval[k] * xj;
    }
    if (normalize) for (int64_t i = 0; i < R->nd; ++i) y[i * sy] = y[i * sy] / R->dst_areas[i];
}

/* transpose: mul!(y, transpose(A), x) column gather, then ./ a_s */
static void og_apply_rev1(const og_regridder* R, const double* x, int64_t sx, double* y, int64_t sy, int normalize) {
    for (int64_t j = 0; j < R->ns; ++j) {
        double acc = 0.0;
        for (int64_t k = R->colptr[j]; k < R->colptr[j + 1]; ++k) acc += R->nzval[k] * x[R->rowval[k] * sx];
        y[j * sy] = normalize ? acc / R->src_areas[j] : acc;
    }
}

/* One 1-D pass per field, as NDSliceLoop does (regrid.jl:303-318); fields are
 * spread over threads. */
void og_apply(const og_regridder* R, int transpose, const double* src, int64_t src_stride_cell, int64_t src_stride_field,
              double* dst, int64_t dst_stride_cell, int64_t dst_stride_field, int64_t nfields, int normalize, int nthreads) {
    /* nthreads applies to this call only (0: all threads) */
    const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int64_t f = 0; f < nfields; ++f) {
        if (!transpose) og_apply_fwd1(R, src + f * src_stride_field, src_stride_cell, dst + f * dst_stride_field, dst_stride_cell, normalize);
        else og_apply_rev1(R, src + f * src_stride_field, src_stride_cell, dst + f * dst_stride_field, dst_stride_cell, normalize);
    }
}

/* The same on Float32 fields, as the reference runs regrid! on Float32 arrays
 * with its SparseMatrixCSC{Float64}: SparseArrays' column scatter
 * (C[rv[j]] += nzv[j] * x[col], regrid.jl:95-98) promotes every product to
 * Float64 and rounds each updated entry back to Float32; the transpose's
 * column gather accumulates in Float64 and rounds once; the division by the
 * areas (regrid.jl:104-118) is Float64, rounded to Float32. */
static void og_apply_fwd1_f32(const og_regridder* R, const float* x, int64_t sx, float* y, int64_t sy, int normalize) {
    for (int64_t i = 0; i < R->nd; ++i) y[i * sy] = 0.0f;
    for (int64_t j = 0; j < R->ns; ++j) {
        double xj = (double)x[j * sx];
        for (int64_t k = R->colptr[j]; k < R->colptr[j + 1]; ++k) {
            float* yp = y + R->rowval[k] * sy;
            *yp = (float)((double)*yp + R->nzval[k] * xj);
        }
    }
    if (normalize) for (int64_t i = 0; i < R->nd; ++i) y[i * sy] = (float)((double)y[i * sy] / R->dst_areas[i]);
}

static void og_apply_rev1_f32(const og_regridder* R, const float* x, int64_t sx, float* y, int64_t sy, int normalize) {
    for (int64_t j = 0; j < R->ns; ++j) {
        double acc = 0.0;
        for (int64_t k = R->colptr[j]; k < R->colptr[j + 1]; ++k) acc += R->nzval[k] * (double)x[R->rowval[k] * sx];
        y[j * sy] = (float)(normalize ? acc / R->src_areas[j] : acc);
    }
}

void og_apply_f32(const og_regridder* R, int transpose, const float* src, int64_t src_stride_cell, int64_t src_stride_field,
                  float* dst, int64_t dst_stride_cell, int64_t dst_stride_field, int64_t nfields, int normalize, int nthreads) {
    const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int64_t f = 0; f < nfields; ++f) {
        if (!transpose) og_apply_fwd1_f32(R, src + f * src_stride_field, src_stride_cell, dst + f * dst_stride_field, dst_stride_cell, normalize);
        else og_apply_rev1_f32(R, src + f * src_stride_field, src_stride_cell, dst + f * dst_stride_field, dst_stride_cell, normalize);
    }
}

/* ------------------------------------------------------------------------ */
/* Test hooks for single geometric operations.                              */
/* ------------------------------------------------------------------------ */

double og_pair_area_hook(int spherical, const double* s, int ns, const double* d, int nd, int* ovf) {
    v3 sv[OG_MAXV], dv[OG_MAXV];
    int dim = spherical ? 3 : 2;
    for (int k = 0; k < ns; ++k) { sv[k].x = s[k * dim]; sv[k].y = s[k * dim + 1]; sv[k].z = spherical ? s[k * dim + 2] : 0; }
    for (int k = 0; k < nd; ++k) { dv[k].x = d[k * dim]; dv[k].y = d[k * dim + 1]; dv[k].z = spherical ? d[k * dim + 2] : 0; }
    *ovf = 0;
    return og_pair_area(spherical, sv, ns, dv, nd, ovf);
}

int og_det3_sign_hook(const double* a, const double* b, const double* c) {
    v3 va = {a[0], a[1], a[2]}, vb = {b[0], b[1], b[2]}, vc = {c[0], c[1], c[2]};
    return og_det3_sign(va, vb, vc);
}

int og_orient2_sign_hook(double ax, double ay, double bx, double by, double vx, double vy) {
    return og_orient2_sign(ax, ay, bx, by, vx, vy);
}

double og_cell_area_hook(int spherical, const double* v, int n) {
    v3 p[OG_MAXV];
    int dim = spherical ? 3 : 2;
    for (int k = 0; k < n; ++k) { p[k].x = v[k * dim]; p[k].y = v[k * dim + 1]; p[k].z = spherical ? v[k * dim + 2] : 0; }
    return og_cell_area(spherical, p, n);
}

/* ------------------------------------------------------------------------ */
/* Forward-mode derivatives of the clip and area (dual numbers).            */
/*                                                                          */
/* The reference has no derivatives: its build writes Float64 buffers      */
/* (src/regridder/intersection_areas.jl:14), so ForwardDiff cannot be       */
/* pushed through it.  This is that experiment done on the oracle instead:  */
/* every og_*_dn function runs exactly the value sequence of the FP64       */
/* function of the same name above (same operations, fma placement and     */
/* branch decisions, so the clipped polygon has the same structure) and     */
/* carries the partial derivatives with respect to the three coordinates of */
/* one vertex of the clip polygon (the destination cell).  It is the        */
/* oracle of the GPU area gradient's tests.                                 */
/* ------------------------------------------------------------------------ */

typedef struct { double v, d[3]; } og_dn;
typedef struct { og_dn x, y, z; } og_dv;

static inline og_dn dn_k(double v) { og_dn r = {v, {0.0, 0.0, 0.0}}; return r; }
static inline og_dn dn_add(og_dn a, og_dn b) {
    og_dn r; r.v = a.v + b.v;
    for (int i = 0; i < 3; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
static inline og_dn dn_sub(og_dn a, og_dn b) {
    og_dn r; r.v = a.v - b.v;
    for (int i = 0; i < 3; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
static inline og_dn dn_neg(og_dn a) {
    og_dn r; r.v = -a.v;
    for (int i = 0; i < 3; ++i) r.d[i] = -a.d[i];
    return r;
}
static inline og_dn dn_mul(og_dn a, og_dn b) {
    og_dn r; r.v = a.v * b.v;
    for (int i = 0; i < 3; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
/* a*b + c, the value rounded once as fma() */
static inline og_dn dn_fma(og_dn a, og_dn b, og_dn c) {
    og_dn r; r.v = fma(a.v, b.v, c.v);
    for (int i = 0; i < 3; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i] + c.d[i];
    return r;
}
static inline og_dn dn_div(og_dn a, og_dn b) {
    og_dn r; r.v = a.v / b.v;
    for (int i = 0; i < 3; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) / b.v;
    return r;
}
static inline og_dn dn_sqrt(og_dn a) {
    og_dn r; r.v = sqrt(a.v);
    double h = r.v > 0.0 ? 0.5 / r.v : 0.0;
    for (int i = 0; i < 3; ++i) r.d[i] = h * a.d[i];
    return r;
}
static inline og_dn dn_abs(og_dn a) { return a.v < 0.0 ? dn_neg(a) : a; }
static inline og_dn dn_scale(double k, og_dn a) {
    og_dn r; r.v = k * a.v;
    for (int i = 0; i < 3; ++i) r.d[i] = k * a.d[i];
    return r;
}

static inline v3 dv_val(og_dv a) { v3 r = {a.x.v, a.y.v, a.z.v}; return r; }
static inline og_dv dv_k(v3 a) { og_dv r = {dn_k(a.x), dn_k(a.y), dn_k(a.z)}; return r; }
static inline og_dv dv_sub(og_dv a, og_dv b) { og_dv r = {dn_sub(a.x, b.x), dn_sub(a.y, b.y), dn_sub(a.z, b.z)}; return r; }
/* og_dot */
static inline og_dn dv_dot(og_dv a, og_dv b) { return dn_fma(a.x, b.x, dn_fma(a.y, b.y, dn_mul(a.z, b.z))); }
/* og_cross (plain products) */
static inline og_dv dv_cross(og_dv a, og_dv b) {
    og_dv r;
    r.x = dn_sub(dn_mul(a.y, b.z), dn_mul(a.z, b.y));
    r.y = dn_sub(dn_mul(a.z, b.x), dn_mul(a.x, b.z));
    r.z = dn_sub(dn_mul(a.x, b.y), dn_mul(a.y, b.x));
    return r;
}
/* og_triple */
static inline og_dn dv_triple(og_dv a, og_dv b, og_dv c) { return dv_dot(a, dv_cross(dv_sub(b, a), dv_sub(c, a))); }

static og_dn og_side_sph_dn(og_dv nrm, og_dv ca, og_dv cb, double eb, int isig, og_dv v) {
    og_dv w = dv_sub(v, ca);
    og_dn s = dv_dot(nrm, w);
    double bound = eb * (fabs(w.x.v) + fabs(w.y.v) + fabs(w.z.v)) + OG_TINY;
    if (fabs(s.v) > bound) return s;
    /* settled to its exact sign; the partials stay those of the FP64 value */
    s.v = og_settle(s.v, bound, isig * og_det3_sign(dv_val(ca), dv_val(cb), dv_val(v)));
    return s;
}

static og_dv og_isect_sph_dn(og_dv a, og_dn sa, og_dv b, og_dn sb) {
    if (sa.v == 0.0) return a;
    if (sb.v == 0.0) return b;
    og_dn wa = dn_abs(sb), wb = dn_abs(sa);
    if (fmax(wa.v, wb.v) < OG_ISECT_TINY) { wa = dn_scale(OG_ISECT_SCALE, wa); wb = dn_scale(OG_ISECT_SCALE, wb); }
    og_dv x;
    x.x = dn_fma(wb, b.x, dn_mul(wa, a.x));
    x.y = dn_fma(wb, b.y, dn_mul(wa, a.y));
    x.z = dn_fma(wb, b.z, dn_mul(wa, a.z));
    og_dn ir = dn_div(dn_k(1.0), dn_sqrt(dv_dot(x, x)));
    x.x = dn_mul(x.x, ir); x.y = dn_mul(x.y, ir); x.z = dn_mul(x.z, ir);
    return x;
}

/* 2 arg(prod (D + iN)); d atan2(y, x) = (x dy - y dx) / (x^2 + y^2) */
static og_dn og_area_sph_signed_dn(const og_dv* v, int m) {
    if (m < 3) return dn_k(0.0);
    og_dn re = dn_k(1.0), im = dn_k(0.0);
    og_dv a = v[0];
    for (int k = 1; k + 1 < m; ++k) {
        og_dv b = v[k], c = v[k + 1];
        og_dn N = dv_triple(a, b, c);
        og_dn D = dn_add(dn_add(dn_add(dn_k(1.0), dv_dot(a, b)), dv_dot(b, c)), dv_dot(c, a));
        og_dn re2 = dn_fma(re, D, dn_neg(dn_mul(im, N)));
        og_dn im2 = dn_fma(re, N, dn_mul(im, D));
        re = re2; im = im2;
    }
    og_dn r;
    r.v = 2.0 * og_atan2(im.v, re.v);
    double q = re.v * re.v + im.v * im.v;
    for (int i = 0; i < 3; ++i) r.d[i] = q > 0.0 ? 2.0 * (re.v * im.d[i] - im.v * re.d[i]) / q : 0.0;
    return r;
}

static inline og_dn dn_cross2(og_dn ax, og_dn ay, og_dn bx, og_dn by) { return dn_sub(dn_mul(ax, by), dn_mul(ay, bx)); }

static og_dn og_side_pl_dn(og_dv a, og_dv b, og_dn ex, og_dn ey, int isig, og_dv v) {
    og_dn wx = dn_sub(v.x, a.x), wy = dn_sub(v.y, a.y);
    og_dn s = dn_cross2(ex, ey, wx, wy);
    if (isig < 0) s = dn_neg(s);
    double bound = OG_U8 * (fabs(ex.v) * fabs(wy.v) + fabs(ey.v) * fabs(wx.v)) + OG_TINY;
    if (fabs(s.v) > bound) return s;
    s.v = og_settle(s.v, bound, isig * og_orient2_sign(a.x.v, a.y.v, b.x.v, b.y.v, v.x.v, v.y.v));
    return s;
}

static og_dv og_isect_pl_dn(og_dv a, og_dn sa, og_dv b, og_dn sb) {
    if (sa.v == 0.0) return a;
    if (sb.v == 0.0) return b;
    og_dn wa = dn_abs(sb), wb = dn_abs(sa);
    if (fmax(wa.v, wb.v) < OG_ISECT_TINY) { wa = dn_scale(OG_ISECT_SCALE, wa); wb = dn_scale(OG_ISECT_SCALE, wb); }
    og_dn w = dn_add(wa, wb);
    og_dv x;
    x.x = dn_div(dn_fma(wb, b.x, dn_mul(wa, a.x)), w);
    x.y = dn_div(dn_fma(wb, b.y, dn_mul(wa, a.y)), w);
    x.z = dn_k(0.0);
    return x;
}

static og_dn og_area_pl_signed_dn(const og_dv* v, int m) {
    if (m < 3) return dn_k(0.0);
    og_dn s = dn_k(0.0);
    for (int k = 1; k + 1 < m; ++k)
        s = dn_add(s, dn_cross2(dn_sub(v[k].x, v[0].x), dn_sub(v[k].y, v[0].y),
                                dn_sub(v[k + 1].x, v[0].x), dn_sub(v[k + 1].y, v[0].y)));
    og_dn r; r.v = 0.5 * s.v;
    for (int i = 0; i < 3; ++i) r.d[i] = 0.5 * s.d[i];
    return r;
}

/* og_clip_sph / og_clip_pl on dual vertices; the orientation of the clip
 * polygon (a sign) is taken from the values. */
static int og_clip_dn(int spherical, const og_dv* subj, int ns, const og_dv* clip, int nc, og_dv* res) {
    og_dv ba[OG_MAXC], bb[OG_MAXC];
    og_dv* in = ba; og_dv* out = bb;
    v3 cv[OG_MAXV];
    for (int i = 0; i < ns; ++i) in[i] = subj[i];
    for (int k = 0; k < nc; ++k) cv[k] = dv_val(clip[k]);
    int n = ns;
    double sig = spherical ? og_orient_sph(cv, nc) : og_orient_pl(cv, nc);
    int isig = sig < 0.0 ? -1 : 1;
    for (int k = 0; k < nc && n > 0; ++k) {
        og_dv ca = clip[k], cb = clip[(k + 1) % nc];
        og_dv nrm = dv_k(cv[k]);
        og_dn ex = dn_k(0.0), ey = dn_k(0.0);
        double eb = 0.0;
        if (spherical) {
            og_dv d1 = dv_sub(cb, ca);
            nrm = dv_cross(ca, d1);
            if (sig < 0.0) { nrm.x = dn_neg(nrm.x); nrm.y = dn_neg(nrm.y); nrm.z = dn_neg(nrm.z); }
            eb = OG_U32 * (fabs(ca.x.v) + fabs(ca.y.v) + fabs(ca.z.v)) * (fabs(d1.x.v) + fabs(d1.y.v) + fabs(d1.z.v));
        } else {
            ex = dn_sub(cb.x, ca.x);
            ey = dn_sub(cb.y, ca.y);
        }
        int m = 0;
        og_dv prev = in[n - 1];
        og_dn sp = spherical ? og_side_sph_dn(nrm, ca, cb, eb, isig, prev) : og_side_pl_dn(ca, cb, ex, ey, isig, prev);
        for (int i = 0; i < n; ++i) {
            og_dv cur = in[i];
            og_dn sc = spherical ? og_side_sph_dn(nrm, ca, cb, eb, isig, cur) : og_side_pl_dn(ca, cb, ex, ey, isig, cur);
            if (sc.v >= 0.0) {
                if (sp.v < 0.0) {
                    if (m >= OG_MAXC) return -1;
                    out[m++] = spherical ? og_isect_sph_dn(prev, sp, cur, sc) : og_isect_pl_dn(prev, sp, cur, sc);
                }
                if (m >= OG_MAXC) return -1;
                out[m++] = cur;
            } else if (sp.v >= 0.0) {
                if (m >= OG_MAXC) return -1;
                out[m++] = spherical ? og_isect_sph_dn(prev, sp, cur, sc) : og_isect_pl_dn(prev, sp, cur, sc);
            }
            prev = cur; sp = sc;
        }
        og_dv* t = in; in = out; out = t;
        n = m;
    }
    for (int i = 0; i < n; ++i) res[i] = in[i];
    return n;
}

/* Slot of vertex k of cell idx in the grid's vertex array: the point index
 * ([points][dim], shared corners share a slot) of a curvilinear grid, or
 * idx*maxv + k ([cells][maxv][dim]) of a polygon grid. */
static int64_t og_vertex_slot(const og_grid* g, int64_t idx, int k) {
    if (g->kind != OG_CURVI) return idx * g->maxv + k;
    int b = 0;
    while (b + 1 < g->nblocks && idx >= g->block_cell_off[b + 1]) b++;
    int64_t loc = idx - g->block_cell_off[b];
    int64_t nx = g->block_nx[b];
    int64_t i = loc % nx + (k == 1 || k == 2), j = loc / nx + (k >= 2);
    return g->block_point_off[b] + i + j * (nx + 1);
}

/* Cell idx of g as dual vertices with vertex `seed` carrying the unit partials
 * (seed < 0: all constant). */
static int og_cell_dn(const og_grid* g, int64_t idx, int seed, og_dv* out) {
    v3 p[OG_MAXV];
    int n = og_cell_verts(g, idx, p);
    for (int k = 0; k < n; ++k) {
        out[k] = dv_k(p[k]);
        if (k == seed) { out[k].x.d[0] = 1.0; out[k].y.d[1] = 1.0; out[k].z.d[2] = 1.0; }
    }
    return n;
}

/* grad (zeroed first) = sum over the nonzeros of R of u_i s_j dA_ij/dV
 *                     + sum_i c_i da_i/dV,
 * with A_ij the unnormalised area of (destination cell i) ∩ (source cell j)
 * -- the clip of subject = source cell j by clip = destination cell i, signed
 * by the subject's orientation, as og_pair_area -- a_i the unnormalised area
 * of destination cell i, and V the destination vertices laid out as
 * og_vertex_slot numbers them (dim coordinates each: x, y, z on the sphere,
 * x, y on the plane).  u and s may both be NULL (area term only); c may be
 * NULL.  dst and src must be the grids R was built from.  Returns the number
 * of pairs whose clip overflowed (left out). */
int64_t og_area_grad(const og_regridder* R, const og_grid* dst, const og_grid* src, const double* u, const double* s,
                     const double* c, double* grad) {
    int spherical = dst->manifold == 1;
    int dim = dst->dim;
    int64_t nslots = dst->kind == OG_CURVI ? dst->block_point_off[dst->nblocks - 1] +
                                                 (dst->block_nx[dst->nblocks - 1] + 1) * (dst->block_ny[dst->nblocks - 1] + 1)
                                           : dst->ncells * dst->maxv;
    memset(grad, 0, (size_t)(nslots * dim) * sizeof(double));
    int64_t overflows = 0;
    og_dv sv[OG_MAXV], dv[OG_MAXV], res[OG_MAXC];
    v3 sp[OG_MAXV];
    for (int64_t j = 0; u && s && j < R->ns; ++j) {
        int nsv = og_cell_verts(src, j, sp);
        for (int k = 0; k < nsv; ++k) sv[k] = dv_k(sp[k]);
        double so = spherical ? og_orient_sph(sp, nsv) : og_orient_pl(sp, nsv);
        for (int64_t q = R->colptr[j]; q < R->colptr[j + 1]; ++q) {
            int64_t i = R->rowval[q];
            double w = u[i] * s[j];
            if (w == 0.0) continue;
            int ndv = og_cell_dn(dst, i, -1, dv);
            for (int k = 0; k < ndv; ++k) {
                int nd = og_cell_dn(dst, i, k, dv);
                int m = og_clip_dn(spherical, sv, nsv, dv, nd, res);
                if (m < 0) { overflows++; break; }
                og_dn a = spherical ? og_area_sph_signed_dn(res, m) : og_area_pl_signed_dn(res, m);
                int64_t slot = og_vertex_slot(dst, i, k);
                for (int e = 0; e < dim; ++e) grad[slot * dim + e] += w * so * a.d[e];
            }
        }
    }
    for (int64_t i = 0; c && i < R->nd; ++i) {
        if (c[i] == 0.0) continue;
        int nd = og_cell_dn(dst, i, -1, dv);
        v3 p[OG_MAXV];
        for (int k = 0; k < nd; ++k) p[k] = dv_val(dv[k]);
        double o = spherical ? og_orient_sph(p, nd) : og_orient_pl(p, nd);
        for (int k = 0; k < nd; ++k) {
            og_cell_dn(dst, i, k, dv);
            og_dn a = spherical ? og_area_sph_signed_dn(dv, nd) : og_area_pl_signed_dn(dv, nd);
            int64_t slot = og_vertex_slot(dst, i, k);
            for (int e = 0; e < dim; ++e) grad[slot * dim + e] += c[i] * o * a.d[e];
        }
    }
    return overflows;
}

int og_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Spectral-element <-> FV regridders: the ClimaCore extension              */
/* (ext/ConservativeRegriddingClimaCoreExt.jl).                             */
/*   SE -> FV principled weights   se_to_fv_principled :416-486,            */
/*                                 accumulate_principled_b :260-305         */
/*   FV -> SE L2 projection        fv_to_se_l2_projection :573-689,         */
/*                                 compute_local_mass_matrix :522-560,      */
/*                                 element_jacobian_at :221-237             */
/*   triangle rules                src/regridder/triangle_quadrature.jl     */
/* ClimaCore itself (GLL nodes, the element map, its inverse, the weighted  */
/* Jacobian) is not vendored; restated from published methods:             */
/*   - GLL nodes: Newton on f = x P_N - P_(N-1), f' = (N+1) P_N, from the   */
/*     Chebyshev-Gauss-Lobatto points; weights 2 / (N (N+1) P_N^2);         */
/*   - the normalised bilinear element map X / |X|, X = a + b xi + c eta +  */
/*     d xi eta, inverted exactly: X || x <=> X.(x x c) = X.(x x b) = 0, a   */
/*     quadratic in eta solved in the cancellation-free form;               */
/*   - area element J = |X.(X_xi x X_eta)| / |X|^3;                          */
/*   - Dunavant (1985) symmetric triangle rules, degrees 1..8;              */
/*   - Gauss-Jordan inversion with partial pivoting.                        */
/* Same operation order as the CUDA coding (crg_se.cu), so the matrices     */
/* agree bit for bit.                                                       */
/* ------------------------------------------------------------------------ */

#define OG_SE_MAXNQ 8
#define OG_SE_MAXTRI 16
#define OG_SE_MAXMASS 12

typedef struct {
    int nq, ntri;
    double x[OG_SE_MAXNQ], w[OG_SE_MAXNQ], c[OG_SE_MAXNQ];
    double tl[OG_SE_MAXTRI][3], tw[OG_SE_MAXTRI];
} og_se_rule;

static void og_legendre2(int N, double t, double* pn, double* pn1) {
    double p0 = 1.0, p1 = t;
    for (int k = 2; k <= N; ++k) {
        double p2 = ((double)(2 * k - 1) * t * p1 - (double)(k - 1) * p0) / (double)k;
        p0 = p1; p1 = p2;
    }
    *pn = p1; *pn1 = p0;
}

void og_se_gll(int n, double* x, double* w) {
    int N = n - 1;
    for (int i = 0; i <= N; ++i) x[i] = -cos(3.14159265358979323846 * (double)i / (double)N);
    for (int it = 0; it < 100; ++it) {
        double dmax = 0.0;
        for (int i = 0; i <= N; ++i) {
            double pn, pn1;
            og_legendre2(N, x[i], &pn, &pn1);
            double dx = (x[i] * pn - pn1) / ((double)n * pn);
            x[i] = x[i] - dx;
            if (fabs(dx) > dmax) dmax = fabs(dx);
        }
        if (dmax <= 1e-15) break;
    }
    x[0] = -1.0; x[N] = 1.0;
    for (int i = 0; i < n / 2; ++i) x[N - i] = -x[i];
    if (n % 2) x[N / 2] = 0.0;
    for (int i = 0; i <= N; ++i) {
        double pn, pn1;
        og_legendre2(N, x[i], &pn, &pn1);
        w[i] = 2.0 / ((double)(N * n) * (pn * pn));
    }
}

/* Lagrange basis on the nodes x, product form phi_j = c_j prod_(m != j) (t - x_m) */
static void og_se_lagrange(int nq, const double* x, const double* c, double t, double* phi) {
    double d[OG_SE_MAXNQ], suf[OG_SE_MAXNQ];
    for (int m = 0; m < nq; ++m) d[m] = t - x[m];
    suf[nq - 1] = 1.0;
    for (int j = nq - 1; j > 0; --j) suf[j - 1] = suf[j] * d[j];
    double pre = 1.0;
    for (int j = 0; j < nq; ++j) { phi[j] = (pre * suf[j]) * c[j]; pre = pre * d[j]; }
}

/* Dunavant (1985) orbits, weights summing to 1: kind 0 centroid, kind 1
 * permutations of (a, b, b), kind 2 permutations of (a, b, c). */
typedef struct { int degree, kind; double w, a, b, c; } og_orbit;

static int og_se_orbits(og_orbit* o) {
    double s15 = sqrt(15.0);
    double bp = (6.0 + s15) / 21.0, bm = (6.0 - s15) / 21.0;
    og_orbit t[] = {
        {1, 0, 1.0, 0, 0, 0},
        {2, 1, 1.0 / 3.0, 2.0 / 3.0, 1.0 / 6.0, 0},
        {3, 0, -27.0 / 48.0, 0, 0, 0},
        {3, 1, 25.0 / 48.0, 0.6, 0.2, 0},
        {4, 1, 0.223381589678011, 0.108103018168070, 0.445948490915965, 0},
        {4, 1, 0.109951743655322, 0.816847572980459, 0.091576213509771, 0},
        {5, 0, 0.225, 0, 0, 0},
        {5, 1, (155.0 + s15) / 1200.0, 1.0 - 2.0 * bp, bp, 0},
        {5, 1, (155.0 - s15) / 1200.0, 1.0 - 2.0 * bm, bm, 0},
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
    int n = (int)(sizeof(t) / sizeof(t[0]));
    memcpy(o, t, sizeof(t));
    return n;
}

/* reference_rule(degree) (triangle_quadrature.jl): points and weights (sum 1);
 * degrees below 1 take rule 1; returns -1 above 8. */
int og_se_tri_rule(int degree, double* tl, double* tw) {
    int d = degree < 1 ? 1 : degree;
    if (d > 8) return -1;
    og_orbit o[32];
    int no = og_se_orbits(o), n = 0;
    double third = 1.0 / 3.0;
#define OG_PUT(W, A, B, C) do { tl[3 * n] = (A); tl[3 * n + 1] = (B); tl[3 * n + 2] = (C); tw[n] = (W); n++; } while (0)
    for (int k = 0; k < no; ++k) {
        if (o[k].degree != d) continue;
        if (o[k].kind == 0) {
            OG_PUT(o[k].w, third, third, third);
        } else if (o[k].kind == 1) {
            OG_PUT(o[k].w, o[k].a, o[k].b, o[k].b); OG_PUT(o[k].w, o[k].b, o[k].a, o[k].b);
            OG_PUT(o[k].w, o[k].b, o[k].b, o[k].a);
        } else {
            OG_PUT(o[k].w, o[k].a, o[k].b, o[k].c); OG_PUT(o[k].w, o[k].a, o[k].c, o[k].b);
            OG_PUT(o[k].w, o[k].b, o[k].a, o[k].c); OG_PUT(o[k].w, o[k].b, o[k].c, o[k].a);
            OG_PUT(o[k].w, o[k].c, o[k].a, o[k].b); OG_PUT(o[k].w, o[k].c, o[k].b, o[k].a);
        }
    }
#undef OG_PUT
    return n;
}

static int og_se_rule_make(int nq, int degree, og_se_rule* r) {
    r->nq = nq;
    og_se_gll(nq, r->x, r->w);
    for (int j = 0; j < nq; ++j) {
        double prod = 1.0;
        for (int m = 0; m < nq; ++m) if (m != j) prod = prod * (r->x[j] - r->x[m]);
        r->c[j] = 1.0 / prod;
    }
    r->ntri = og_se_tri_rule(degree, &r->tl[0][0], r->tw);
    return r->ntri > 0 ? 0 : -1;
}

/* a, b, c, d of the bilinear map and c x a, c x b, c x d, b x a, b x d */
static void og_se_coeffs(const v3* q, double* g) {
    v3 c1 = q[0], c2 = q[1], c3 = q[2], c4 = q[3], a, b, c, d;
    a.x = 0.25 * ((c1.x + c2.x) + (c3.x + c4.x)); a.y = 0.25 * ((c1.y + c2.y) + (c3.y + c4.y));
    a.z = 0.25 * ((c1.z + c2.z) + (c3.z + c4.z));
    b.x = 0.25 * ((c2.x - c1.x) + (c3.x - c4.x)); b.y = 0.25 * ((c2.y - c1.y) + (c3.y - c4.y));
    b.z = 0.25 * ((c2.z - c1.z) + (c3.z - c4.z));
    c.x = 0.25 * ((c3.x - c2.x) + (c4.x - c1.x)); c.y = 0.25 * ((c3.y - c2.y) + (c4.y - c1.y));
    c.z = 0.25 * ((c3.z - c2.z) + (c4.z - c1.z));
    d.x = 0.25 * ((c1.x - c2.x) + (c3.x - c4.x)); d.y = 0.25 * ((c1.y - c2.y) + (c3.y - c4.y));
    d.z = 0.25 * ((c1.z - c2.z) + (c3.z - c4.z));
    v3 out[9] = {a, b, c, d, og_cross(c, a), og_cross(c, b), og_cross(c, d), og_cross(b, a), og_cross(b, d)};
    for (int k = 0; k < 9; ++k) { g[3 * k] = out[k].x; g[3 * k + 1] = out[k].y; g[3 * k + 2] = out[k].z; }
}

static inline v3 og_v3at(const double* p) { v3 r = {p[0], p[1], p[2]}; return r; }

void og_se_inverse(const double* g, v3 x, double* xi, double* eta) {
    double A1 = og_dot(x, og_v3at(g + 12)), B1 = og_dot(x, og_v3at(g + 15)), D1 = og_dot(x, og_v3at(g + 18));
    double A2 = og_dot(x, og_v3at(g + 21)), D2 = og_dot(x, og_v3at(g + 24));
    double C2 = -B1;
    double a0 = C2 * D1;
    double b0 = fma(-D2, A1, fma(A2, D1, C2 * B1));
    double c0 = A2 * B1;
    double disc = fma(b0, b0, -(4.0 * a0) * c0);
    if (disc < 0.0) disc = 0.0;
    double q = b0 + copysign(sqrt(disc), b0);
    *eta = q != 0.0 ? (-2.0 * c0) / q : 0.0;
    double den = fma(D1, *eta, B1);
    *xi = den != 0.0 ? -A1 / den : 0.0;
}

/* B[i + j nq] += integral over the overlap polygon res[0..m) of phi_i(xi) phi_j(eta):
 * each fan triangle's rule points summed on their own (T), the triangles
 * then added in fan order (the GPU coding's triangle items). */
static void og_se_poly_b(const og_se_rule* r, const double* g, const v3* res, int m, double sig, double r2,
                         double* B) {
    int nq = r->nq;
    if (m < 3) return;
    v3 cs = res[0];
    for (int k = 1; k < m; ++k) { cs.x = cs.x + res[k].x; cs.y = cs.y + res[k].y; cs.z = cs.z + res[k].z; }
    double ic = 1.0 / sqrt(og_dot(cs, cs));
    v3 cen = {cs.x * ic, cs.y * ic, cs.z * ic};
    for (int k = 0; k < m; ++k) {
        v3 v1 = res[k], v2 = res[k + 1 == m ? 0 : k + 1];
        double N = og_triple(cen, v1, v2);
        double D = ((1.0 + og_dot(cen, v1)) + og_dot(v1, v2)) + og_dot(v2, cen);
        double At = ((2.0 * og_atan2(N, D)) * sig) * r2;
        if (!(At > 0.0)) continue;
        double T[OG_SE_MAXNQ * OG_SE_MAXNQ];
        for (int q = 0; q < nq * nq; ++q) T[q] = 0.0;
        for (int gq = 0; gq < r->ntri; ++gq) {
            double l0 = r->tl[gq][0], l1 = r->tl[gq][1], l2 = r->tl[gq][2];
            /* the rule point; the inverse map does not depend on its length */
            v3 x;
            x.x = fma(l2, v2.x, fma(l1, v1.x, l0 * cen.x));
            x.y = fma(l2, v2.y, fma(l1, v1.y, l0 * cen.y));
            x.z = fma(l2, v2.z, fma(l1, v1.z, l0 * cen.z));
            double xi, eta, fx[OG_SE_MAXNQ], fy[OG_SE_MAXNQ];
            og_se_inverse(g, x, &xi, &eta);
            og_se_lagrange(nq, r->x, r->c, xi, fx);
            og_se_lagrange(nq, r->x, r->c, eta, fy);
            double wA = r->tw[gq] * At;
            for (int i = 0; i < nq; ++i) fx[i] = wA * fx[i];
            for (int j = 0; j < nq; ++j)
                for (int i = 0; i < nq; ++i) T[i + j * nq] = fma(fx[i], fy[j], T[i + j * nq]);
        }
        for (int q = 0; q < nq * nq; ++q) B[q] = B[q] + T[q];
    }
}

/* Node positions and weighted Jacobians of one element (W = J w_i w_j r2). */
static void og_se_elem_nodes(const double* g, const og_se_rule* r, double r2, double* pts, double* wj) {
    int nq = r->nq;
    v3 a = og_v3at(g), b = og_v3at(g + 3), c = og_v3at(g + 6), d = og_v3at(g + 9);
    for (int j = 0; j < nq; ++j)
        for (int i = 0; i < nq; ++i) {
            double xi = r->x[i], eta = r->x[j], xe = xi * eta;
            v3 X;
            X.x = ((a.x + b.x * xi) + c.x * eta) + d.x * xe;
            X.y = ((a.y + b.y * xi) + c.y * eta) + d.y * xe;
            X.z = ((a.z + b.z * xi) + c.z * eta) + d.z * xe;
            double n2 = og_dot(X, X);
            int k = i + j * nq;
            if (pts) {
                double ir = 1.0 / sqrt(n2);
                pts[3 * k] = X.x * ir; pts[3 * k + 1] = X.y * ir; pts[3 * k + 2] = X.z * ir;
            }
            if (wj) {
                v3 Xxi = {b.x + d.x * eta, b.y + d.y * eta, b.z + d.z * eta};
                v3 Xeta = {c.x + d.x * xi, c.y + d.y * xi, c.z + d.z * xi};
                double J = fabs(og_dot(X, og_cross(Xxi, Xeta))) / (n2 * sqrt(n2));
                wj[k] = ((J * r->w[i]) * r->w[j]) * r2;
            }
        }
}

/* Per-element L2 projection (fv_to_se_l2_projection :634-679): M^e from the
 * GLL rule of ceil((3 nq - 2) / 2) + 1 points and the interpolated Jacobian,
 * restricted to the nodes of nonzero total b, rows scaled to that total,
 * inverted; out[p][cov[rc]] = sum_cc Inv[rc][cc] b_p[cov[cc]].  Returns -1 if
 * singular. */
static int og_se_project(const og_se_rule* r, const double* wj_e, const double* const* b, int np, double** out) {
    int nq = r->nq, nq2 = nq * nq;
    int nm = (3 * nq - 2 + 1) / 2 + 1;
    double xm[OG_SE_MAXMASS], wm[OG_SE_MAXMASS], L[OG_SE_MAXMASS][OG_SE_MAXNQ];
    og_se_gll(nm, xm, wm);
    for (int p = 0; p < nm; ++p) og_se_lagrange(nq, r->x, r->c, xm[p], L[p]);
    double Jn[OG_SE_MAXNQ * OG_SE_MAXNQ], Jq[OG_SE_MAXMASS * OG_SE_MAXMASS];
    for (int k = 0; k < nq2; ++k) Jn[k] = wj_e[k] / (r->w[k % nq] * r->w[k / nq]);
    for (int k = 0; k < nm * nm; ++k) {
        int pp = k % nm, qq = k / nm;
        double s = 0.0;
        for (int qn = 0; qn < nq; ++qn)
            for (int pn = 0; pn < nq; ++pn) s = fma(Jn[pn + qn * nq] * L[pp][pn], L[qq][qn], s);
        Jq[k] = s;
    }
    double* M = (double*)malloc(sizeof(double) * nq2 * nq2);
    double* Inv = (double*)malloc(sizeof(double) * nq2 * nq2);
    /* sum factorisation: G[q][a][i] = sum_p w_p w_q J phi_a phi_i, then M */
    double* G = (double*)malloc(sizeof(double) * nm * nq2);
    for (int k = 0; k < nm * nq2; ++k) {
        int qq = k / nq2, a = (k % nq2) % nq, i = (k % nq2) / nq;
        double s = 0.0;
        for (int pp = 0; pp < nm; ++pp) s = fma(((wm[pp] * wm[qq]) * Jq[pp + qq * nm]) * L[pp][a], L[pp][i], s);
        G[k] = s;
    }
    for (int k = 0; k < nq2 * nq2; ++k) {
        int row = k / nq2, col = k % nq2;
        int a = row % nq, bb = row / nq, i = col % nq, j = col / nq;
        double s = 0.0;
        for (int qq = 0; qq < nm; ++qq) s = fma(G[qq * nq2 + a + i * nq] * L[qq][bb], L[qq][j], s);
        M[k] = s;
    }
    free(G);
    double bfull[OG_SE_MAXNQ * OG_SE_MAXNQ];
    int cov[OG_SE_MAXNQ * OG_SE_MAXNQ], m = 0;
    for (int k = 0; k < nq2; ++k) {
        double s = 0.0;
        for (int p = 0; p < np; ++p) s = s + b[p][k];
        bfull[k] = s;
    }
    for (int k = 0; k < nq2; ++k) if (bfull[k] != 0.0) cov[m++] = k;
    for (int x = 0; x < m * m; ++x) Inv[(x / m) * nq2 + x % m] = M[cov[x / m] * nq2 + cov[x % m]];
    for (int x = 0; x < m * m; ++x) M[(x / m) * nq2 + x % m] = Inv[(x / m) * nq2 + x % m];
    for (int rc = 0; rc < m; ++rc) {
        double rs = 0.0;
        for (int cc = 0; cc < m; ++cc) rs = rs + M[rc * nq2 + cc];
        if (rs != 0.0) {
            double scale = bfull[cov[rc]] / rs;
            for (int cc = 0; cc < m; ++cc) M[rc * nq2 + cc] = M[rc * nq2 + cc] * scale;
        }
    }
    for (int x = 0; x < m * m; ++x) Inv[(x / m) * nq2 + x % m] = (x / m == x % m) ? 1.0 : 0.0;
    for (int k = 0; k < m; ++k) {
        int p = k;
        double best = fabs(M[k * nq2 + k]);
        for (int rr = k + 1; rr < m; ++rr)
            if (fabs(M[rr * nq2 + k]) > best) { best = fabs(M[rr * nq2 + k]); p = rr; }
        if (best == 0.0) { free(M); free(Inv); return -1; }
        if (p != k)
            for (int cc = 0; cc < m; ++cc) {
                double t = M[k * nq2 + cc]; M[k * nq2 + cc] = M[p * nq2 + cc]; M[p * nq2 + cc] = t;
                t = Inv[k * nq2 + cc]; Inv[k * nq2 + cc] = Inv[p * nq2 + cc]; Inv[p * nq2 + cc] = t;
            }
        double pk = M[k * nq2 + k];
        for (int cc = 0; cc < m; ++cc) {
            if (cc > k) M[k * nq2 + cc] = M[k * nq2 + cc] / pk;
            Inv[k * nq2 + cc] = Inv[k * nq2 + cc] / pk;
        }
        M[k * nq2 + k] = 1.0;
        double f[OG_SE_MAXNQ * OG_SE_MAXNQ];
        for (int rr = 0; rr < m; ++rr) f[rr] = M[rr * nq2 + k];
        for (int rr = 0; rr < m; ++rr) {
            if (rr == k) continue;
            for (int cc = 0; cc < m; ++cc) {
                if (cc > k) M[rr * nq2 + cc] = M[rr * nq2 + cc] - f[rr] * M[k * nq2 + cc];
                if (cc == k) M[rr * nq2 + cc] = 0.0;
                Inv[rr * nq2 + cc] = Inv[rr * nq2 + cc] - f[rr] * Inv[k * nq2 + cc];
            }
        }
    }
    for (int p = 0; p < np; ++p) {
        for (int k = 0; k < nq2; ++k) out[p][k] = 0.0;
        for (int rc = 0; rc < m; ++rc) {
            double s = 0.0;
            for (int cc = 0; cc < m; ++cc) s = fma(Inv[rc * nq2 + cc], b[p][cov[cc]], s);
            out[p][cov[rc]] = s;
        }
    }
    free(M); free(Inv);
    return 0;
}

/* SE <-> FV build.  se_is_dst = 0: SE -> FV (rows = FV cells, columns = nodes),
 * 1: FV -> SE (rows = nodes, columns = FV cells).  node_weights may be NULL.
 * Returns NULL with *err set: 1 bad argument (rule degree, element without 4
 * vertices), 2 clip overflow, 3 singular mass matrix. */
og_regridder* og_build_se(const og_grid* fv, const og_grid* elems, int nq, int degree, double radius,
                          const double* node_weights, int se_is_dst, int use_tree, int nthreads, int* err) {
    *err = 0;
    og_se_rule rule;
    if (nq < 2 || nq > OG_SE_MAXNQ || og_se_rule_make(nq, degree ? degree : 2 * (nq - 1), &rule) != 0) { *err = 1; return NULL; }
    double r2 = (radius > 0.0 ? radius : 1.0);
    r2 = r2 * r2;
    int nq2 = nq * nq;
    int64_t nelem = elems->ncells, nfv = fv->ncells, nn = nelem * nq2;
    double* coef = (double*)malloc(sizeof(double) * 27 * (nelem > 0 ? nelem : 1));
    for (int64_t e = 0; e < nelem; ++e) {
        v3 v[OG_MAXV];
        if (og_cell_verts(elems, e, v) != 4) { free(coef); *err = 1; return NULL; }
        og_se_coeffs(v, coef + 27 * e);
    }
    double* wj = (double*)malloc(sizeof(double) * (nn > 0 ? nn : 1));
    if (node_weights) memcpy(wj, node_weights, sizeof(double) * nn);
    else for (int64_t e = 0; e < nelem; ++e) og_se_elem_nodes(coef + 27 * e, &rule, r2, NULL, wj + e * nq2);
    const og_grid* dst = se_is_dst ? elems : fv;
    const og_grid* src = se_is_dst ? fv : elems;
    int64_t* cand = NULL;
    int64_t nc = og_candidates(dst, src, use_tree, nthreads, &cand);
    double* bv = (double*)calloc((size_t)(nc > 0 ? nc : 1) * nq2, sizeof(double));
    int64_t ovf_total = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : ovf_total)
    for (int64_t k = 0; k < nc; ++k) {
        v3 s[OG_MAXV], d[OG_MAXV], res[OG_MAXC];
        int ns_ = og_cell_verts(src, cand[2 * k], s);
        int nd_ = og_cell_verts(dst, cand[2 * k + 1], d);
        if (ns_ < 3 || nd_ < 3) continue;
        int m = og_clip_sph(s, ns_, d, nd_, res);
        if (m < 0) { ovf_total += 1; continue; }
        int64_t e = se_is_dst ? cand[2 * k + 1] : cand[2 * k];
        og_se_poly_b(&rule, coef + 27 * e, res, m, og_orient_sph(s, ns_), r2, bv + k * nq2);
    }
    if (ovf_total) { free(coef); free(wj); free(cand); free(bv); *err = 2; return NULL; }
    double* vals = bv;
    double* pv = NULL;
    if (se_is_dst) {
        /* pairs with a nonzero b, grouped by element, cells ascending */
        int64_t* ecnt = (int64_t*)calloc(nelem + 1, sizeof(int64_t));
        char* has = (char*)calloc(nc > 0 ? nc : 1, 1);
        for (int64_t k = 0; k < nc; ++k) {
            for (int q = 0; q < nq2; ++q) if (bv[k * nq2 + q] != 0.0) { has[k] = 1; break; }
            if (has[k]) ecnt[cand[2 * k + 1] + 1]++;
        }
        for (int64_t e = 0; e < nelem; ++e) ecnt[e + 1] += ecnt[e];
        int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (nelem + 1));
        memcpy(fill, ecnt, sizeof(int64_t) * (nelem + 1));
        int64_t* plist = (int64_t*)malloc(sizeof(int64_t) * (ecnt[nelem] > 0 ? ecnt[nelem] : 1));
        for (int64_t k = 0; k < nc; ++k) if (has[k]) plist[fill[cand[2 * k + 1]]++] = k;
        for (int64_t e = 0; e < nelem; ++e) {  /* insertion sort by cell */
            for (int64_t p = ecnt[e] + 1; p < ecnt[e + 1]; ++p) {
                int64_t t = plist[p], q = p - 1;
                while (q >= ecnt[e] && cand[2 * plist[q]] > cand[2 * t]) { plist[q + 1] = plist[q]; q--; }
                plist[q + 1] = t;
            }
        }
        pv = (double*)calloc((size_t)(nc > 0 ? nc : 1) * nq2, sizeof(double));
        int bad = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : bad)
        for (int64_t e = 0; e < nelem; ++e) {
            int64_t np = ecnt[e + 1] - ecnt[e];
            if (np == 0) continue;
            const double** bp = (const double**)malloc(sizeof(double*) * np);
            double** op = (double**)malloc(sizeof(double*) * np);
            for (int64_t p = 0; p < np; ++p) {
                bp[p] = bv + plist[ecnt[e] + p] * nq2;
                op[p] = pv + plist[ecnt[e] + p] * nq2;
            }
            if (og_se_project(&rule, wj + e * nq2, bp, (int)np, op) != 0) bad += 1;
            free(bp); free(op);
        }
        free(ecnt); free(has); free(fill); free(plist);
        if (bad) { free(coef); free(wj); free(cand); free(bv); free(pv); *err = 3; return NULL; }
        vals = pv;
    }
    /* COO in pair order -> sparse() */
    int64_t m = 0;
    for (int64_t k = 0; k < nc * nq2; ++k) m += vals[k] != 0.0;
    int64_t* ir = (int64_t*)malloc(sizeof(int64_t) * (m > 0 ? m : 1));
    int64_t* ic = (int64_t*)malloc(sizeof(int64_t) * (m > 0 ? m : 1));
    double* iv = (double*)malloc(sizeof(double) * (m > 0 ? m : 1));
    int64_t o = 0;
    for (int64_t k = 0; k < nc; ++k) {
        int64_t e = se_is_dst ? cand[2 * k + 1] : cand[2 * k];
        int64_t cell = se_is_dst ? cand[2 * k] : cand[2 * k + 1];
        for (int q = 0; q < nq2; ++q) {
            double v = vals[k * nq2 + q];
            if (v == 0.0) continue;
            int64_t node = e * nq2 + q;
            ir[o] = se_is_dst ? node : cell;
            ic[o] = se_is_dst ? cell : node;
            iv[o] = v;
            o++;
        }
    }
    og_regridder* R = (og_regridder*)calloc(1, sizeof(og_regridder));
    R->nd = se_is_dst ? nn : nfv;
    R->ns = se_is_dst ? nfv : nn;
    R->ncand = nc;
    og_sparse(R, ir, ic, iv, m);
    R->dst_areas = (double*)malloc(sizeof(double) * (R->nd > 0 ? R->nd : 1));
    R->src_areas = (double*)malloc(sizeof(double) * (R->ns > 0 ? R->ns : 1));
    double* fva = se_is_dst ? R->src_areas : R->dst_areas;
    for (int64_t i = 0; i < nfv; ++i) { v3 v[OG_MAXV]; int n = og_cell_verts(fv, i, v); fva[i] = og_cell_area(1, v, n) * r2; }
    if (se_is_dst) for (int64_t i = 0; i < nn; ++i) R->dst_areas[i] = 1.0;
    else memcpy(R->src_areas, wj, sizeof(double) * nn);
    free(ir); free(ic); free(iv); free(coef); free(wj); free(cand); free(bv); free(pv);
    return R;
}

/* Hooks for the SE known-answer tests. */
void og_se_lagrange_hook(int nq, double t, double* phi) {
    og_se_rule r;
    og_se_rule_make(nq, 1, &r);
    og_se_lagrange(nq, r.x, r.c, t, phi);
}

void og_se_inverse_hook(const double* corners12, const double* x3, double* out2) {
    v3 q[4];
    for (int k = 0; k < 4; ++k) q[k] = og_v3at(corners12 + 3 * k);
    double g[27];
    og_se_coeffs(q, g);
    og_se_inverse(g, og_v3at(x3), &out2[0], &out2[1]);
}

void og_se_nodes_hook(const double* corners12, int nq, double radius, double* pts, double* wj) {
    v3 q[4];
    for (int k = 0; k < 4; ++k) q[k] = og_v3at(corners12 + 3 * k);
    double g[27];
    og_se_coeffs(q, g);
    og_se_rule r;
    og_se_rule_make(nq, 1, &r);
    double r2 = (radius > 0.0 ? radius : 1.0);
    og_se_elem_nodes(g, &r, r2 * r2, pts, wj);
}

/* b of one element over a given polygon (counter-clockwise unit vectors). */
int og_se_poly_b_hook(const double* corners12, const double* poly, int m, int nq, int degree, double* B) {
    v3 q[4], p[OG_MAXC];
    if (m > OG_MAXC) return -1;
    for (int k = 0; k < 4; ++k) q[k] = og_v3at(corners12 + 3 * k);
    for (int k = 0; k < m; ++k) p[k] = og_v3at(poly + 3 * k);
    double g[27];
    og_se_coeffs(q, g);
    og_se_rule r;
    if (og_se_rule_make(nq, degree ? degree : 2 * (nq - 1), &r) != 0) return -1;
    for (int k = 0; k < nq * nq; ++k) B[k] = 0.0;
    og_se_poly_b(&r, g, p, m, og_orient_sph(p, m), 1.0, B);
    return 0;
}
