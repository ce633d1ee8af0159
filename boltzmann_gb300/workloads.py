"""Synthetic workloads for the batched 0D3V velocity-space solve.

No public data set is involved: every input is generated here from fixed seeds.

Cross sections (argon-like, analytic, tabulated to an LXCat file that the product and
the oracle both read):
  * elastic momentum transfer  sigma = 1e-19 * (0.1 + eps)^0.5 m^2, m/M = 1.36e-5;
  * excitation, threshold 11.55 eV, rising linearly to 1e-21 m^2 at 30 eV, held above;
  * ionization, threshold 15.76 eV, rising linearly to 3e-20 m^2 at 100 eV, held above.
The table has eps = 0, 4000 log-spaced energies in [1e-4, 1e4] eV and the exact break
points; the solvers interpolate it linearly and clamp at both ends, as
`BESolver/python/collisions.py:79` does. The process key of the elastic block is
"E + Ar -> E + Ar": the reference reads m/M from exactly that key (`collisions.py:77`).

Common settings follow the reference driver (`BESolver/python/bte_0d3v_batched_driver.py`):
sp_order 3, spline_qpts 5, E = (E/N) * n0 * 1e-21, Newton atol 1e-20, rtol 1e-14,
alpha_rho 0.5, line-search c 1e-4; n0 = 1 Torr / (k_B * 300 K); velocity grid up to
80 eV with no extension; normalisation temperature Te = 4 eV.
"""
from __future__ import annotations

import os
import tempfile

import numpy as np

from .lxcat import write_lxcat

TORR = 133.32236842105263
KB = 1.380649e-23
N0_1TORR_300K = TORR / (KB * 300.0)
TD = 1e-21
EV_MAX = 80.0
TE_NORM = 4.0

ELASTIC_KEY = "E + Ar -> E + Ar"


def _energy_grid(breaks):
    e = np.concatenate([[0.0], np.logspace(-4, 4, 4000), np.asarray(breaks, dtype=np.float64)])
    return np.unique(e)


def synthetic_processes():
    """The three analytic processes as LXCat blocks (elastic, excitation, ionization)."""
    e_el = _energy_grid([])
    s_el = 1e-19 * np.sqrt(0.1 + e_el)

    e_ex = _energy_grid([11.55, 30.0])
    s_ex = np.where(e_ex < 11.55, 0.0, 1e-21 * np.minimum((e_ex - 11.55) / (30.0 - 11.55), 1.0))

    e_io = _energy_grid([15.76, 100.0])
    s_io = np.where(e_io < 15.76, 0.0, 3e-20 * np.minimum((e_io - 15.76) / (100.0 - 15.76), 1.0))
    return [
        dict(kind="ELASTIC", species="Ar", param=1.36e-5, process=ELASTIC_KEY, energy=e_el, sigma=s_el),
        dict(kind="EXCITATION", species="Ar", target="Ar -> Ar*", param=11.55,
             process="E + Ar -> E + Ar*", energy=e_ex, sigma=s_ex),
        dict(kind="IONIZATION", species="Ar", target="Ar -> Ar^+", param=15.76,
             process="E + Ar -> E + E + Ar+", energy=e_io, sigma=s_io),
    ]


def write_synthetic_lxcat(path: str | None = None) -> str:
    """Write the analytic argon-like set to `path` (default: a temp file) and return it."""
    if path is None:
        fd, path = tempfile.mkstemp(prefix="eAr_synthetic_", suffix=".lxcat")
        os.close(fd)
    write_lxcat(path, synthetic_processes())
    return path


def batch_parameters(n_pts: int, seed: int, ion_deg_range=(-8.0, -3.0), ebyn_range=(0.0, 3.0), ee=True):
    """Per-point parameters: E/N log-uniform in 10^ebyn_range Td, ionization degree
    log-uniform in 10^ion_deg_range, n0 at 1 Torr / 300 K, Tg = 300 K, one species."""
    rng = np.random.default_rng(seed)
    ebyn = 10.0 ** rng.uniform(ebyn_range[0], ebyn_range[1], n_pts)
    ion = 10.0 ** rng.uniform(ion_deg_range[0], ion_deg_range[1], n_pts)
    n0 = np.full(n_pts, N0_1TORR_300K)
    return dict(
        n0=n0,
        ne=(ion * n0) if ee else np.zeros(n_pts),
        Tg=np.full(n_pts, 300.0),
        E=ebyn * n0 * TD,
        ns_by_n0=np.ones((1, n_pts)),
        EbyN=ebyn,
    )


# (N_sp, l_max, n_pts, e-e, seed, ionization-degree range); N_sp = number of B-splines,
# the reference's `Nr` argument is N_sp - 1.
CONFIGS = {
    "c1": dict(n_sp=64, l_max=1, n_pts=1, ee=False, seed=None, ion=None),
    "c2": dict(n_sp=128, l_max=2, n_pts=4096, ee=True, seed=20261203, ion=(-8.0, -3.0)),
    "c5": dict(n_sp=256, l_max=4, n_pts=16384, ee=True, seed=20261205, ion=(-6.0, -2.0)),
}


def config_parameters(name: str, n_pts: int | None = None):
    c = CONFIGS[name]
    n = c["n_pts"] if n_pts is None else n_pts
    if name == "c1":
        n0 = np.full(n, N0_1TORR_300K)
        return dict(n0=n0, ne=np.zeros(n), Tg=np.full(n, 300.0), E=100.0 * n0 * TD,
                    ns_by_n0=np.ones((1, n)), EbyN=np.full(n, 100.0))
    return batch_parameters(n, c["seed"], ion_deg_range=c["ion"], ee=c["ee"])


# Serving mix: Poisson arrivals of requests of 1..512 points on grids with N_sp in
# {64, 96, 128, 192, 256} and l_max in {1, 2, 3}; E/N and ionization degree as the batched
# workload; seed 20261204.
SERVE_N_SP = (64, 96, 128, 192, 256)
SERVE_L_MAX = (1, 2, 3)


def serving_requests(n_req: int, rate_per_s: float, seed: int = 20261204, max_points: int = 512,
                     n_sp_choices=SERVE_N_SP, l_max_choices=SERVE_L_MAX):
    """Requests as dicts (arrival time in s from the start, n_sp, l_max and the per-point
    parameters of batch_parameters). rate_per_s = inf gives every arrival at t = 0."""
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    for i in range(n_req):
        if np.isfinite(rate_per_s):
            t += rng.exponential(1.0 / rate_per_s)
        P = int(rng.integers(1, max_points + 1))
        n_sp = int(rng.choice(n_sp_choices))
        l_max = int(rng.choice(l_max_choices))
        prm = batch_parameters(P, int(rng.integers(0, 2**31 - 1)))
        out.append(dict(t=t, n_sp=n_sp, l_max=l_max, **prm))
    return out
