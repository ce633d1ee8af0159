"""Serving loop on the GPU: each request's result is the same alone and in a mix of requests
of several grid sizes arriving while others run, and equals the plain solve path
(bte_0d3v_batched.solve: e-e-off warm start, then e-e on) on the same points."""
import threading
import time

import numpy as np
import pytest

from helpers import gpu_solver, rel_l2_cols
from boltzmann_gb300.workloads import batch_parameters

pytestmark = pytest.mark.gpu

# The engine runs per point the same kernels, in the same order, as bte_solve_steady, so
# results agree to round-off (bitwise in practice).
TOL_SAME = 1e-12
GRIDS = [(32, 1), (40, 2)]


def _req(n_sp, l_max, P, seed):
    from boltzmann_gb300.serving import SolveRequest
    p = batch_parameters(P, seed)
    return SolveRequest(n_sp=n_sp, l_max=l_max, n0=p["n0"], ne=p["ne"], Tg=p["Tg"], E=p["E"], ns_by_n0=p["ns_by_n0"])


def _copy(r):
    from boltzmann_gb300.serving import SolveRequest
    return SolveRequest(n_sp=r.n_sp, l_max=r.l_max, n0=r.n0.copy(), ne=r.ne.copy(), Tg=r.Tg.copy(), E=r.E.copy(),
                        ns_by_n0=r.ns_by_n0.copy(), ee=r.ee)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_engine_matches_two_solve_calls(synthetic_xs, precision):
    from boltzmann_gb300.serving import BteServer, wait_all
    import torch
    n_sp, l_max, P = 40, 2, 6
    req = _req(n_sp, l_max, P, 7)
    with BteServer(synthetic_xs, [(n_sp, l_max)], precision=precision, capacity=16, fp64_capacity=4) as srv:
        srv.submit(req)
        wait_all([req], timeout=300)
    s, args = gpu_solver(synthetic_xs, n_sp, l_max, True, P, precision=precision)
    for k in ["n0", "ne", "ns_by_n0", "Tg", "E"]:
        s.set_boltzmann_parameter(0, k, getattr(req, k))
    f0 = torch.as_tensor(s.initialize(0, P), device="cuda")
    args.ee_collisions = 0
    ffw, _ = s.solve(0, f0, 1e-20, 1e-14, 100, "steady-state", 1e-16, 0.5, 1e-4)
    args.ee_collisions = 1
    ff, qoi = s.solve(0, ffw, 1e-20, 1e-14, 100, "steady-state", 1e-16, 0.5, 1e-4)
    ff = ff.cpu().numpy()
    assert np.all(req.qoi["status"] <= 1)
    assert float(np.max(rel_l2_cols(req.ff, ff))) < TOL_SAME
    for k in ("energy", "mobility", "diffusion"):
        ref = qoi[k].cpu().numpy()
        assert float(np.max(np.abs(req.qoi[k] - ref) / np.abs(ref))) < 1e-11


def test_result_same_alone_and_in_a_mix(synthetic_xs):
    from boltzmann_gb300.serving import BteServer, wait_all, latency_summary
    probe = _req(40, 2, 5, 11)
    with BteServer(synthetic_xs, GRIDS, precision="mixed", capacity=64, fp64_capacity=8,
                   hbm_budget_bytes=256 << 20) as srv:
        alone = srv.submit(_copy(probe))
        wait_all([alone], timeout=300)
        # the mix: requests on both grids arriving over time; the probe arrives while others run
        rng = np.random.default_rng(3)
        mix = []

        def feed():
            for i in range(12):
                g = GRIDS[i % 2]
                mix.append(srv.submit(_req(g[0], g[1], int(rng.integers(1, 24)), 100 + i)))
                time.sleep(0.01)

        t = threading.Thread(target=feed)
        t.start()
        time.sleep(0.03)
        in_mix = srv.submit(_copy(probe))
        t.join()
        wait_all(mix + [in_mix], timeout=600)
        summ = latency_summary(mix + [in_mix])
    assert in_mix.t_admit < max(r.t_done for r in mix)  # it really ran alongside others
    assert float(np.max(rel_l2_cols(in_mix.ff, alone.ff))) < TOL_SAME
    for k in ("energy", "mobility", "diffusion"):
        assert np.allclose(in_mix.qoi[k], alone.qoi[k], rtol=1e-11, atol=0)
    # coarse test grids: a few random points may end unconverged, as they do in the plain solve
    for r in mix:
        assert np.all((r.qoi["status"] >= 0) & (r.qoi["status"] <= 5))
        ok = r.qoi["status"] <= 1
        assert np.all(np.isfinite(r.ff[:, ok]))
    assert summ["p99_ms"] >= summ["p50_ms"] > 0


def test_tps_csv_requests_through_the_server(synthetic_xs, tmp_path):
    """Points read from a TPS CSV (the reference driver's `-input` file) and split into
    requests give, through the server, the plain solve path's results on the same points."""
    from boltzmann_gb300.lxcat import read_available_species
    from boltzmann_gb300.serving import BteServer, wait_all
    from boltzmann_gb300.tps_input import read_tps_csv, requests_from_tps
    import torch
    species = read_available_species(synthetic_xs)
    P, n_sp, l_max = 10, 32, 1
    p = batch_parameters(P, 23)
    path = tmp_path / "tps.csv"
    with open(path, "w") as f:
        f.write(",".join(["Tg", "n0", "ne/n0", "E"] + ["(%s)/n0" % s for s in species]) + "\n")
        for i in range(P):
            vals = [p["Tg"][i], p["n0"][i], p["ne"][i] / p["n0"][i], p["E"][i]] + [1.0] * len(species)
            f.write(",".join(repr(float(v)) for v in vals) + "\n")
    prm = read_tps_csv(str(path), species)
    reqs = requests_from_tps(prm, n_sp, l_max, max_points=4)
    assert [r.P for r in reqs] == [4, 4, 2]
    with BteServer(synthetic_xs, [(n_sp, l_max)], precision="fp64", capacity=8, fp64_capacity=4) as srv:
        for r in reqs:
            srv.submit(r)
        wait_all(reqs, timeout=300)
    s, args = gpu_solver(synthetic_xs, n_sp, l_max, True, P, precision="fp64")
    for k in ["n0", "ne", "ns_by_n0", "Tg", "E"]:
        s.set_boltzmann_parameter(0, k, prm[k])
    f0 = torch.as_tensor(s.initialize(0, P), device="cuda")
    args.ee_collisions = 0
    ffw, _ = s.solve(0, f0, 1e-20, 1e-14, 100, "steady-state", 1e-16, 0.5, 1e-4)
    args.ee_collisions = 1
    ff, _ = s.solve(0, ffw, 1e-20, 1e-14, 100, "steady-state", 1e-16, 0.5, 1e-4)
    ff = ff.cpu().numpy()
    got = np.concatenate([r.ff for r in reqs], axis=1)
    assert all(np.all(r.qoi["status"] <= 1) for r in reqs)
    assert float(np.max(rel_l2_cols(got, ff))) < TOL_SAME
