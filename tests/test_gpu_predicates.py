"""The clip's exact-sign predicate on the GPU against rational arithmetic.

A side value inside its FP64 rounding bound is settled by the exact sign of
det[a; b; c] (the reference clips with exact predicates, so cells that only
touch clip to zero area).  The GPU takes that sign from a double-double value
when it lies outside a certified error bound, and from the error-free expansion
otherwise (two equal points give 0 before either); all must give the sign of the
exact determinant of the doubles.
Cases: points on a great circle up to the rounding of their coordinates
(meridians and parallels built from cos/sin, near-coplanar combinations one ulp
off), exactly coplanar points, and lattice vectors whose determinant is +-1 ulp^2
of terms near 1 (continued-fraction convergents), where only the expansion can
decide.

The FP64 apply of several fields divides each output element by its row's area
with a reciprocal taken once per row and Markstein's correction, checked and
otherwise replaced by the IEEE division: every quotient must have the IEEE
bits, on random operands, near-midpoint quotients, divisors whose significand
is all ones, powers of two, zeros, subnormal and overflowing quotients.
The helper library is compiled from tests/gpu_predicates.cu."""
from __future__ import annotations

import ctypes
import itertools
import subprocess
from fractions import Fraction

import numpy as np
import pytest

from conftest import ROOT
from crg import _build

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def helpers(cuda, tmp_path_factory):
    out = tmp_path_factory.mktemp("pred") / "libcrg_test_pred.so"
    subprocess.run([_build._nvcc(), *_build.NVCC_FLAGS, *_build.ARCH_FLAGS, f"-I{_build.CSRC}", "-shared",
                    "-o", str(out), str(ROOT / "tests" / "gpu_predicates.cu")], check=True, capture_output=True)
    lib = ctypes.CDLL(str(out))
    lib.crg_test_det3.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    lib.crg_test_det3.restype = ctypes.c_int
    lib.crg_test_div.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.crg_test_div.restype = ctypes.c_int
    return lib


@pytest.fixture(scope="module")
def det3(helpers):
    lib = helpers

    def run(triples):
        t = np.ascontiguousarray(np.asarray(triples, dtype=np.float64).reshape(-1, 9))
        o = np.zeros((len(t), 3), dtype=np.int32)
        assert lib.crg_test_det3(t.ctypes.data, len(t), o.ctypes.data) == 0
        return o

    return run


def _exact(q):
    a, b, c = ([Fraction(float(x)) for x in q[i:i + 3]] for i in (0, 3, 6))
    d = a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) + a[2] * (b[0] * c[1] - b[1] * c[0])
    return int(d > 0) - int(d < 0)


def _unit(rng):
    v = rng.standard_normal(3)
    return v / np.linalg.norm(v)


def _sph(lat, lon):
    return np.array([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)])


def _cases():
    rng = np.random.default_rng(11)
    out = []
    for _ in range(1500):  # near-coplanar, one ulp off
        a, b = _unit(rng), _unit(rng)
        c = rng.uniform(-1, 1) * a + rng.uniform(-1, 1) * b
        k = int(rng.integers(3))
        if rng.integers(2):
            c[k] = np.nextafter(c[k], np.inf * rng.choice([-1, 1]))
        out += [(a, b, c), (c, a, b)]
    for _ in range(800):  # three points of one meridian; three points of one parallel
        lon = rng.uniform(0, 2 * np.pi)
        out.append(tuple(_sph(t, lon) for t in rng.uniform(-np.pi / 2, np.pi / 2, 3)))
        lat = rng.uniform(-1.5, 1.5)
        out.append(tuple(_sph(lat, l) for l in rng.uniform(0, 2 * np.pi, 3)))
    for _ in range(200):  # exactly coplanar
        a, b = _unit(rng), _unit(rng)
        out += [(a, b, a), (a, b, b), (a, b, -a), (a, b, 2 * a)]
    for _ in range(300):  # general position, also scaled far down
        a, b, c = _unit(rng), _unit(rng), _unit(rng)
        out += [(a, b, c), (a * 1e-150, b, c)]
    perms = list(itertools.permutations(range(3)))
    for _ in range(150):  # |h_n k_(n-1) - h_(n-1) k_n| = 1, terms up to 2^52
        x = rng.uniform(0.1, 10)
        h, k, r = [1, int(x)], [0, 1], x - int(x)
        while r > 1e-12 and max(h[-1], k[-1]) < 2**52:
            r = 1 / r
            q = int(r)
            r -= q
            h.append(q * h[-1] + h[-2])
            k.append(q * k[-1] + k[-2])
        for n in range(2, len(h)):
            sc = 2.0 ** -int(rng.integers(40, 60))
            p = perms[int(rng.integers(6))]
            a = np.array([rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(0.5, 2)])[list(p)]
            b = np.array([h[n] * sc, k[n] * sc, 0.0])[list(p)]
            c = np.array([h[n - 1] * sc, k[n - 1] * sc, 0.0])[list(p)]
            out.append((a, b, c))
    return np.array([np.concatenate(t) for t in out])


def test_det3_sign_exact_on_gpu(det3):
    cases = _cases()
    got = det3(cases)
    want = np.array([_exact(q) for q in cases])
    assert np.array_equal(got[:, 0], want)           # the clip's predicate
    assert np.array_equal(got[:, 2], want)           # the error-free expansion alone
    filt = got[:, 1]
    assert np.array_equal(filt[filt != 0], want[filt != 0])  # a certified filter sign is never wrong
    # both stages decide some cases: the filter most, the expansion the exact zeros and the lattices
    assert (filt != 0).sum() > 0.8 * len(cases) and ((filt == 0) & (want != 0)).sum() > 50
    assert ((filt == 0) & (want == 0)).sum() >= 800
    # the clip's predicate answers equal points at once; equal points all give 0
    eq = np.array([np.array_equal(q[0:3], q[6:9]) or np.array_equal(q[3:6], q[6:9]) or np.array_equal(q[0:3], q[3:6])
                   for q in cases])
    assert eq.sum() >= 400 and not want[eq].any()


def _div_cases():
    rng = np.random.default_rng(21)
    a = list(rng.standard_normal(20000) * 10.0 ** rng.integers(-30, 30, 20000))
    d = list(np.abs(rng.standard_normal(20000)) * 10.0 ** rng.integers(-12, 3, 20000))
    # quotients within two ulps either side of k / d for small integers k
    for _ in range(20000):
        dd = float(rng.uniform(0.5, 2.0)) * 2.0 ** int(rng.integers(-40, 5))
        aa = float(rng.integers(1, 1 << 20)) * dd
        for step in (-2, -1, 0, 1, 2):
            x = aa
            for _ in range(abs(step)):
                x = np.nextafter(x, np.inf if step > 0 else -np.inf)
            a.append(float(x))
            d.append(dd)
    ones = np.nextafter(2.0, 0.0)  # significand all ones
    for e in range(-60, 60, 7):
        for x in rng.standard_normal(200):
            a += [float(x), float(x) * 2.0 ** e, 2.0 ** e, -(2.0 ** e)]
            d += [float(ones * 2.0 ** (e // 2))] * 2 + [3.0, float(ones)]
    a += [0.0, -0.0, 1e-310, -1e-320, 1e300, 1e-300, 1.0, np.nextafter(1.0, 2.0)]
    d += [3.0, 3.0, 7.0, 3.0, 1e-10, 1e10, 1.0, 1.0]
    return np.array(a), np.array(d)


def test_corrected_quotient_is_ieee(helpers):
    a, d = _div_cases()
    fast, ieee = np.empty_like(a), np.empty_like(a)
    assert helpers.crg_test_div(a.ctypes.data, d.ctypes.data, len(a), fast.ctypes.data, ieee.ctypes.data) == 0
    with np.errstate(all="ignore"):
        host = a / d
    assert np.array_equal(ieee.view(np.uint64), host.view(np.uint64))
    assert np.array_equal(fast.view(np.uint64), ieee.view(np.uint64))
