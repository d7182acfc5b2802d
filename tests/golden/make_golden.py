"""Generate the golden fixtures under tests/golden/.

1. ``readme_planar.json``: the known answers of ConservativeRegridding.jl's
   README example (README.md:52-80, the "blue" 2x2 unit squares against the
   "orange" diamond + 4 triangles): every intersection is 0.5, source areas
   [0.5, 0.5, 2, 0.5, 0.5], destination areas [1, 1, 1, 1]; and the variant
   of test/usecases/simple.jl:9-51 (squares built from a 3x3 point lattice,
   rows sums == cell areas, mean conserved exactly).
2. ``sphere_areas.json``: spherical polygons and pairs whose areas are
   computed here at 60 significant digits with mpmath by an independent
   method -- Girard's theorem (interior-angle excess) on the polygon, and for
   pairs a Sutherland-Hodgman clip carried out in mpmath -- to pin the FP64
   area/clip arithmetic of the oracle and of the CUDA kernels.

Run from the repository root:  python tests/golden/make_golden.py
(needs mpmath; the committed JSON files are what the tests read).
"""
from __future__ import annotations

import json
import math
from pathlib import Path

import mpmath as mp

mp.mp.dps = 60
HERE = Path(__file__).resolve().parent


# ----------------------------------------------------------------- planar known answers

def readme_case():
    blue = [[(1, 1), (1, 0), (0, 0), (0, 1), (1, 1)],
            [(2, 1), (2, 0), (1, 0), (1, 1), (2, 1)],
            [(1, 2), (1, 1), (0, 1), (0, 2), (1, 2)],
            [(2, 2), (2, 1), (1, 1), (1, 2), (2, 2)]]
    orange = [[(0, 2), (1, 2), (0, 1), (0, 2)],
              [(1, 2), (2, 2), (2, 1), (1, 2)],
              [(0, 1), (1, 2), (2, 1), (1, 0), (0, 1)],
              [(0, 0), (0, 1), (1, 0), (0, 0)],
              [(1, 0), (2, 1), (2, 0), (1, 0)]]
    # README.md:68-76 (4x5 matrix, row = blue/dst cell, column = orange/src cell)
    matrix = [[0, 0, 0.5, 0.5, 0],
              [0, 0, 0.5, 0, 0.5],
              [0.5, 0, 0.5, 0, 0],
              [0, 0.5, 0.5, 0, 0]]
    return {"dst": blue, "src": orange, "matrix": matrix,
            "src_areas": [0.5, 0.5, 2.0, 0.5, 0.5], "dst_areas": [1.0, 1.0, 1.0, 1.0]}


def simple_jl_case():
    # test/usecases/simple.jl:10-25: gridpoints[(i, j)] for i, j in 0:2; polygons in
    # column-major (i fastest) order with ring g[i,j], g[i,j+1], g[i+1,j+1], g[i+1,j].
    g = {(i, j): (i, j) for i in range(3) for j in range(3)}
    polys1 = []
    for j in range(2):
        for i in range(2):
            polys1.append([g[(i, j)], g[(i, j + 1)], g[(i + 1, j + 1)], g[(i + 1, j)], g[(i, j)]])
    diamond = [(0, 1), (1, 2), (2, 1), (1, 0), (0, 1)]
    tris = [[(0, 0), (1, 0), (0, 1), (0, 0)], [(0, 1), (0, 2), (1, 2), (0, 1)],
            [(1, 2), (2, 1), (2, 2), (1, 2)], [(2, 1), (2, 0), (1, 0), (2, 1)]]
    return {"dst": polys1, "src": [diamond] + tris, "dst_areas": [1.0] * 4,
            "src_areas": [2.0, 0.5, 0.5, 0.5, 0.5], "values_on_src": [0, 0, 5, 0, 0]}


# ----------------------------------------------------------------- high-precision sphere

def mvec(p):
    return [mp.mpf(p[0]), mp.mpf(p[1]), mp.mpf(p[2])]


def mcross(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def mdot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def mnorm(a):
    n = mp.sqrt(mdot(a, a))
    return [x / n for x in a]


def girard_area(poly):
    """Spherical excess of a convex polygon: 2 pi minus the sum of the
    exterior (turning) angles between consecutive great-circle edges."""
    return girard_area_mp([mnorm(mvec(p)) for p in poly])


def orient(P):
    m = [sum(p[i] for p in P) for i in range(3)]
    s = mp.mpf(0)
    for k in range(len(P)):
        s += mdot(mcross(P[k], P[(k + 1) % len(P)]), m)
    return 1 if s >= 0 else -1


def mp_clip(subj, clip):
    S = [mnorm(mvec(p)) for p in subj]
    Cl = [mnorm(mvec(p)) for p in clip]
    sig = orient(Cl)
    for k in range(len(Cl)):
        if not S:
            break
        n = mcross(Cl[k], Cl[(k + 1) % len(Cl)])
        n = [sig * x for x in n]
        out = []
        prev = S[-1]
        sp = mdot(n, prev)
        for cur in S:
            sc = mdot(n, cur)
            if sc >= 0:
                if sp < 0:
                    out.append(mnorm([abs(sp) * cur[i] + abs(sc) * prev[i] for i in range(3)]))
                out.append(cur)
            elif sp >= 0:
                out.append(mnorm([abs(sp) * cur[i] + abs(sc) * prev[i] for i in range(3)]))
            prev, sp = cur, sc
        S = out
    return S


def sph(lon, lat):
    lo, la = math.radians(lon), math.radians(lat)
    return [math.cos(la) * math.cos(lo), math.cos(la) * math.sin(lo), math.sin(la)]


def quad(lon0, lon1, lat0, lat1):
    return [sph(lon0, lat0), sph(lon1, lat0), sph(lon1, lat1), sph(lon0, lat1)]


def sphere_cases():
    polys = {
        "octant": [[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]],
        "cell_2deg_equator": quad(10, 12, 0, 2),
        "cell_1deg_midlat": quad(30, 31, 45, 46),
        "cell_0.25deg_highlat": quad(100, 100.25, 80, 80.25),
        "cell_0.001deg": quad(-60, -59.999, -20, -19.999),
        "cell_large_60deg": quad(0, 60, -30, 30),
        "cell_cw_3deg": list(reversed(quad(200, 203, -10, -7))),
        "pentagon": [sph(0, 0), sph(5, -1), sph(8, 3), sph(4, 7), sph(-1, 4)],
        "polar_triangle": [sph(0, 88), sph(120, 88), sph(240, 88)],
    }
    pairs = {
        "overlap_shifted": (quad(0, 2, 0, 2), quad(0.7, 3.7, 0.4, 3.4)),
        "src_inside_dst": (quad(10.5, 11, 10.5, 11), quad(10, 12, 10, 12)),
        "dst_inside_src": (quad(10, 12, 10, 12), quad(10.5, 11, 10.5, 11)),
        "diamond_square": ([sph(1, 0), sph(2, 1), sph(1, 2), sph(0, 1)], quad(0, 1, 0, 1)),
        "polar_rows": (quad(0, 10, 80, 85), quad(5, 15, 82, 86)),
        "cw_subject": (list(reversed(quad(0, 2, 0, 2))), quad(1, 3, 1, 3)),
        "cw_clip": (quad(0, 2, 0, 2), list(reversed(quad(1, 3, 1, 3)))),
        "disjoint": (quad(0, 1, 0, 1), quad(2, 3, 2, 3)),
    }
    out_p = {}
    for k, p in polys.items():
        out_p[k] = {"verts": p, "area": mp.nstr(girard_area(p), 40)}
    out_q = {}
    for k, (s, d) in pairs.items():
        r = mp_clip(s, d)
        a = girard_area_mp(r) if len(r) >= 3 else mp.mpf(0)
        out_q[k] = {"src": s, "dst": d, "area": mp.nstr(a, 40)}
    return {"polygons": out_p, "pairs": out_q}


def girard_area_mp(P):
    Q = []
    for p in P:  # drop consecutive (near-)duplicate vertices
        if not Q or mp.sqrt(mdot([p[i] - Q[-1][i] for i in range(3)], [p[i] - Q[-1][i] for i in range(3)])) > mp.mpf(10) ** -40:
            Q.append(p)
    while len(Q) > 1 and mp.sqrt(mdot([Q[0][i] - Q[-1][i] for i in range(3)], [Q[0][i] - Q[-1][i] for i in range(3)])) <= mp.mpf(10) ** -40:
        Q.pop()
    P = Q
    n = len(P)
    if n < 3:
        return mp.mpf(0)
    ext = mp.mpf(0)
    for k in range(n):
        a, b, c = P[k - 1], P[k], P[(k + 1) % n]
        n1 = mcross(a, b)
        n2 = mcross(b, c)
        if mdot(n1, n1) == 0 or mdot(n2, n2) == 0:
            continue
        n1 = mnorm(n1)
        n2 = mnorm(n2)
        ext += mp.atan2(mdot(mcross(n1, n2), b), mdot(n1, n2))
    return abs(2 * mp.pi - abs(ext))


def main():
    (HERE / "readme_planar.json").write_text(json.dumps({"readme": readme_case(), "simple_jl": simple_jl_case()}, indent=1))
    (HERE / "sphere_areas.json").write_text(json.dumps(sphere_cases(), indent=1))
    print("wrote", HERE / "readme_planar.json", HERE / "sphere_areas.json")


if __name__ == "__main__":
    main()
