"""The residual's double-double accumulation (boltzmann_gb300/csrc/dd_arith.h, used by k_residual
for points at their FP64 rounding floor), compiled for the host: sums of products with heavy
cancellation against exact rational arithmetic. The plain FP64 sum loses the result; the
double-double one keeps it to the error bound of the compensated sum."""
import ctypes
import os
import shutil
import subprocess
from fractions import Fraction

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    so = str(tmp_path_factory.mktemp("dd") / "dd_harness.so")
    r = subprocess.run([cxx, "-O2", "-ffp-contract=off", "-shared", "-fPIC",
                        os.path.join(HERE, "host", "dd_harness.cpp"), "-o", so], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = ctypes.CDLL(so)
    dp = ctypes.POINTER(ctypes.c_double)
    L.dd_dot.argtypes = [ctypes.c_int, dp, dp, dp]
    L.dd_dot2.argtypes = [ctypes.c_int, dp, dp, dp, dp]
    return L


def _p(x):
    return x.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _cancelling(rng, n, scale):
    """Products of size `scale` that cancel to a sum of order 1 (the residual of a
    Coulomb-dominated point: large collision and e-e terms, small difference)."""
    a = rng.uniform(-1.0, 1.0, n) * scale
    b = rng.uniform(-1.0, 1.0, n)
    b[-1] = 0.0
    s = sum(Fraction(x) * Fraction(y) for x, y in zip(a[:-1], b[:-1]))
    a[-1] = float(-s)  # the last product cancels the sum up to its own rounding
    b[-1] = 1.0
    return a, b


@pytest.mark.parametrize("scale", [1e8, 1e12])
def test_dd_dot_keeps_cancelled_sums(lib, scale):
    rng = np.random.default_rng(int(np.log10(scale)))
    for _ in range(20):
        a, b = _cancelling(rng, 257, scale)
        exact = sum(Fraction(x) * Fraction(y) for x, y in zip(a, b))
        out = np.zeros(2)
        lib.dd_dot(len(a), _p(a), _p(b), _p(out))
        got = Fraction(out[0]) + Fraction(out[1])
        mag = sum(abs(Fraction(x) * Fraction(y)) for x, y in zip(a, b))
        # the compensated dot product's bound (Ogita, Rump and Oishi, Dot2): gamma_n^2 of the
        # sum of |terms|, gamma_n ~ n u, u = 2^-53
        assert abs(got - exact) <= 2 * (len(a) * Fraction(2) ** -53) ** 2 * mag
        plain = Fraction(float(np.dot(a, b)))
        assert abs(got - exact) <= abs(plain - exact) or plain == exact


def test_dd_dot2_carries_the_low_part(lib):
    """(hi + lo) * b with the low part kept: the products of a double-double vector."""
    rng = np.random.default_rng(5)
    n = 100
    hi = rng.uniform(-1.0, 1.0, n) * 1e6
    lo = hi * rng.uniform(-1.0, 1.0, n) * 2.0 ** -60
    b = rng.uniform(-1.0, 1.0, n)
    exact = sum((Fraction(h) + Fraction(l)) * Fraction(y) for h, l, y in zip(hi, lo, b))
    out = np.zeros(2)
    lib.dd_dot2(n, _p(hi), _p(lo), _p(b), _p(out))
    got = Fraction(out[0]) + Fraction(out[1])
    mag = sum(abs((Fraction(h) + Fraction(l)) * Fraction(y)) for h, l, y in zip(hi, lo, b))
    assert abs(got - exact) <= 2 * (n * Fraction(2) ** -53) ** 2 * mag
