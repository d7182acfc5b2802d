"""The oracle's planar clip and area against exact rational arithmetic: the
intersection of two convex polygons (Sutherland & Hodgman 1974 with exact
side tests and exact crossing points, in fractions.Fraction) and its exact
shoelace area, for random convex pairs of either orientation, nested,
overlapping, touching and disjoint.  This pins the planar path independently
of the README example."""
from __future__ import annotations

from fractions import Fraction

import numpy as np
import pytest

import oracle


def _convex(rng, n, cx, cy, r, ccw=True):
    a = np.sort(rng.uniform(0.0, 2.0 * np.pi, n))
    p = np.stack([cx + r * np.cos(a), cy + r * np.sin(a)], axis=1)
    return p if ccw else p[::-1].copy()


def _exact_area(p):
    s = Fraction(0)
    for k in range(len(p)):
        (x0, y0), (x1, y1) = p[k], p[(k + 1) % len(p)]
        s += x0 * y1 - x1 * y0
    return s / 2


def _exact_clip(subj, clip):
    """Subject clipped by the convex clip polygon, all in Fractions."""
    if _exact_area(clip) < 0:
        clip = clip[::-1]
    out = list(subj)
    for k in range(len(clip)):
        (ax, ay), (bx, by) = clip[k], clip[(k + 1) % len(clip)]
        side = lambda v: (bx - ax) * (v[1] - ay) - (by - ay) * (v[0] - ax)
        inp, out = out, []
        if not inp:
            break
        prev = inp[-1]
        sp = side(prev)
        for cur in inp:
            sc = side(cur)
            if sc >= 0:
                if sp < 0:
                    t = sp / (sp - sc)
                    out.append((prev[0] + t * (cur[0] - prev[0]), prev[1] + t * (cur[1] - prev[1])))
                out.append(cur)
            elif sp >= 0:
                t = sp / (sp - sc)
                out.append((prev[0] + t * (cur[0] - prev[0]), prev[1] + t * (cur[1] - prev[1])))
            prev, sp = cur, sc
    return out


def _fr(p):
    return [(Fraction(float(x)), Fraction(float(y))) for x, y in p]


def test_random_convex_pairs_match_exact_rational_areas():
    rng = np.random.default_rng(11)
    worst, overlapping = 0.0, 0
    for trial in range(300):
        ns, nd = int(rng.integers(3, 9)), int(rng.integers(3, 9))
        s = _convex(rng, ns, rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(0.2, 1.5), bool(rng.integers(2)))
        d = _convex(rng, nd, rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(0.2, 1.5), bool(rng.integers(2)))
        got = oracle.pair_area(s, d, spherical=False)
        fs = _fr(s)
        exact = _exact_area(_exact_clip(fs, _fr(d)))
        if _exact_area(fs) < 0:  # the oracle signs the area by the subject's orientation
            exact = -exact
        exact = float(exact)
        overlapping += exact != 0.0
        scale = max(abs(float(_exact_area(fs))), 1e-300)
        err = abs(got - exact) / scale
        worst = max(worst, err)
        assert err < 4e-15, (trial, got, exact)
    assert overlapping >= 100 and worst < 4e-15


@pytest.mark.parametrize("shift,expect", [((0.0, 0.0), 1.0), ((0.5, 0.25), 0.375), ((1.0, 0.0), 0.0),
                                          ((1.0, 1.0), 0.0), ((3.0, 0.0), 0.0)])
def test_unit_squares_shifted(shift, expect):
    """Overlap of two unit squares: identical, partly overlapping, sharing an
    edge, sharing a corner, disjoint (the last three exactly 0)."""
    sq = np.array([(0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 1.0)])
    assert oracle.pair_area(sq + np.array(shift), sq, spherical=False) == expect
