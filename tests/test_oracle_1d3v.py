"""The 1D3V oracle (oracle/bte1d_oracle.py) against golden vectors of the reference's own
spectral 1D3V step (tests/golden/make_golden_1d3v.py): set-up operators, initial condition,
x-advection and v-space steps."""
import ast
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "bte1d_reference.npz")


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - b)) / np.max(np.abs(b)))


@pytest.fixture(scope="module")
def case(synthetic_xs):
    from oracle.bte1d_oracle import Oracle1D
    g = np.load(GOLD)
    p = ast.literal_eval(str(g["params"]))
    o = Oracle1D(synthetic_xs, p["Np"], p["Nr"], p["Nvt"], p["lmax"], p["ev_max"], p["Te"], p["L"], p["freq"], p["Tg"],
                 p["p0"])
    return o, g, p


@pytest.mark.parametrize("name", ["Dp", "xp_vt", "xp_vt_qw", "op_po2sh", "op_psh2o", "op_adv_x", "op_col_en",
                                  "op_col_gT", "op_adv_v"])
def test_setup_operators(case, name):
    o, g, _ = case
    assert rel(getattr(o, name), g[name]) < 1e-13


def test_initial_condition(case):
    o, g, _ = case
    assert rel(o.initial_condition(), g["v0"]) < 1e-12


def test_x_steps(case):
    o, g, p = case
    assert rel(o.step_x(g["v0"], 0.5 * p["dt"]), g["v1"]) < 1e-12
    assert rel(o.step_x(g["v2"], 0.5 * p["dt"]), g["v3"]) < 1e-12


def test_v_step(case):
    """The reference's GMRES stops at rtol 1e-12 (relative to ||b||); the oracle solves exactly."""
    o, g, p = case
    assert rel(o.step_v(g["E"], g["v1"], p["dt"]), g["v2"]) < 1e-10


def test_strang_step(case):
    o, g, p = case
    assert rel(o.step(g["E"], g["v0"], p["dt"]), g["v3"]) < 1e-10
