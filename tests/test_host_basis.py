"""The library's B-spline evaluation and sigma interpolation (shared host/device code in
bte_common.cuh), compiled for the host and compared with the oracle's SciPy-based
evaluation on the reference's knot vectors."""
import os
import subprocess

import numpy as np
import pytest
import scipy.interpolate

from helpers import oracle_ops

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    from boltzmann_gb300._build import nvcc
    exe = str(tmp_path_factory.mktemp("probe") / "bspline_probe")
    r = subprocess.run([nvcc(), "-O2", "-std=c++17", "-x", "cu", os.path.join(HERE, "host", "bspline_probe.cu"),
                        "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run_probe(exe, t, pts, xs, ys, q):
    nsp = len(t) - 4
    inp = "%d\n%s\n%d\n%s\n%d\n%s\n%s\n%d\n%s\n" % (
        nsp, " ".join("%.17e" % v for v in t), len(pts), " ".join("%.17e" % v for v in pts),
        len(xs), " ".join("%.17e" % v for v in xs), " ".join("%.17e" % v for v in ys), len(q),
        " ".join("%.17e" % v for v in q))
    out = subprocess.run([exe], input=inp, capture_output=True, text=True, check=True).stdout.split("\n")
    rows = [list(map(float, l.split())) for l in out[:len(pts)]]
    vals = np.array([float(v) for v in out[len(pts):len(pts) + len(q)]])
    return rows, vals


@pytest.mark.parametrize("n_sp,l_max", [(64, 1), (128, 2)])
def test_bspline_values_and_derivatives(probe, synthetic_xs, n_sp, l_max):
    o = oracle_ops(synthetic_xs, n_sp, l_max, False)
    B = o.basis
    rng = np.random.default_rng(1)
    pts = np.concatenate([rng.uniform(0, o.knots[-1], 300), o.knots[3:-3] + 1e-9, [0.0, o.knots[-1], -1.0,
                                                                                   o.knots[-1] * 1.01]])
    rows, _ = run_probe(probe, o.knots, pts, [0.0, 1.0], [0.0, 1.0], [0.5])
    for x, row in zip(pts, rows):
        span = int(row[0])
        vals = np.array(row[1:]).reshape(3, 4)
        for d in range(3):
            ref = np.array([B.eval(i, np.array([x]), d)[0] for i in range(B.num_p)])
            got = np.zeros(B.num_p)
            if span >= 0:
                for j in range(4):
                    got[span - 3 + j] = vals[d, j]
            scale = max(1.0, np.max(np.abs(ref)))
            assert np.max(np.abs(got - ref)) <= 1e-12 * scale, (x, d, got, ref)


def test_interp_matches_scipy(probe, synthetic_xs):
    from boltzmann_gb300.lxcat import read_cross_section_data
    data = read_cross_section_data(synthetic_xs)
    for k, v in data.items():
        e, s = v["energy"], v["cross section"]
        f = scipy.interpolate.interp1d(e, s, kind="linear", bounds_error=False, fill_value=(s[0], s[-1]))
        rng = np.random.default_rng(2)
        q = np.concatenate([10 ** rng.uniform(-6, 5, 500), e[::97], [e[0], e[-1], -1.0, 2e4]])
        _, got = run_probe(probe, np.array([0, 0, 0, 0, 1, 1, 1, 1.0]), [0.5], e, s, q)
        ref = f(q)
        assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)) < 1e-13, k
