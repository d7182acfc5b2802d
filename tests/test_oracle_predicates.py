"""The oracle's exact-sign predicates against rational arithmetic.  The clip
decides every side test whose floating-point value is inside its rounding
bound by these signs (Shewchuk-style error-free expansions), which is why
cells that only touch clip to exactly zero area.  Inputs are nearly
degenerate on purpose: points on (or one ulp off) the great circle through
two others, or on the line through two others, where the plain
floating-point determinant is dominated by rounding."""
from __future__ import annotations

from fractions import Fraction

import numpy as np

import oracle


def _sign(x):
    return int(x > 0) - int(x < 0)


def _det3_exact(a, b, c):
    a, b, c = ([Fraction(float(t)) for t in v] for v in (a, b, c))
    return _sign(a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0])
                 + a[2] * (b[0] * c[1] - b[1] * c[0]))


def _orient2_exact(a, b, v):
    a, b, v = ([Fraction(float(t)) for t in p] for p in (a, b, v))
    return _sign((b[0] - a[0]) * (v[1] - a[1]) - (b[1] - a[1]) * (v[0] - a[0]))


def _unit(rng):
    v = rng.standard_normal(3)
    return v / np.linalg.norm(v)


def test_det3_sign_is_exact_near_coplanar_points():
    rng = np.random.default_rng(4)
    disagree_plain = 0
    for _ in range(2000):
        a, b = _unit(rng), _unit(rng)
        c = rng.uniform(-1, 1) * a + rng.uniform(-1, 1) * b
        k = int(rng.integers(3))
        c[k] = np.nextafter(c[k], np.inf * rng.choice([-1, 1])) if rng.integers(2) else c[k]
        want = _det3_exact(a, b, c)
        assert oracle.det3_sign(a, b, c) == want
        disagree_plain += _sign(float(np.dot(a, np.cross(b, c)))) != want
    # exactly coplanar: zero; and plain arithmetic gets some of the signs above wrong
    for a, b in ((_unit(rng), _unit(rng)) for _ in range(50)):
        assert oracle.det3_sign(a, b, a) == 0 and oracle.det3_sign(a, b, b) == 0 and oracle.det3_sign(a, b, -a) == 0
    assert disagree_plain > 0


def test_det3_sign_in_general_position():
    rng = np.random.default_rng(5)
    for _ in range(500):
        a, b, c = _unit(rng), _unit(rng), _unit(rng)
        assert oracle.det3_sign(a, b, c) == _det3_exact(a, b, c)


def test_orient2_sign_is_exact_near_collinear_points():
    rng = np.random.default_rng(6)
    disagree_plain = 0
    for _ in range(2000):
        a, b = rng.uniform(-10, 10, 2), rng.uniform(-10, 10, 2)
        v = a + rng.uniform(-2, 3) * (b - a)
        if rng.integers(2):
            k = int(rng.integers(2))
            v[k] = np.nextafter(v[k], np.inf * rng.choice([-1, 1]))
        want = _orient2_exact(a, b, v)
        assert oracle.orient2_sign(a, b, v) == want
        plain = (b[0] - a[0]) * (v[1] - a[1]) - (b[1] - a[1]) * (v[0] - a[0])
        disagree_plain += _sign(plain) != want
    assert disagree_plain > 0
    assert oracle.orient2_sign((0.0, 0.0), (1.0, 1.0), (0.5, 0.5)) == 0
    assert oracle.orient2_sign((0.0, 0.0), (1.0, 0.0), (0.5, 5e-324)) == 1
