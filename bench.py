"""Benchmark: batched 0D3V steady-state EDF solves on GB300.

Workload (default): 4096 independent points, 128 cubic B-splines x l_max 2 (n = 384
unknowns, 385 x 385 bordered Newton systems), e-e Coulomb collisions on, E/N log-uniform
in [1, 1000] Td, ionization degree log-uniform in [1e-8, 1e-3] (seed 20261203), synthetic
analytic argon-like cross sections. One step = one full EDF solve of the whole batch as
the reference driver does it (Maxwellian start, e-e-off warm start, e-e-on solve, QoIs).

Headline: solves/s of the mixed form (FP32 Jacobian factorizations against the FP64
residual). The plain FP64 form runs the same workload for the ratio and the error check
(max relative L2 difference of the EDFs <= 1e-8).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
import types

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "EDF solves/s (batched 0D3V steady state, e-e on, mixed precision, <=1e-8 rel err vs plain FP64)"
UNIT = "solves/s"
ATOL, RTOL, MAXIT = 1e-20, 1e-14, 100
ALPHA_MIN, ALPHA_RHO, LS_C = 1e-16, 0.5, 1e-4


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n-pts", type=int, default=4096)
    ap.add_argument("--n-sp", type=int, default=128)
    ap.add_argument("--l-max", type=int, default=2)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--plain-steps", type=int, default=1, help="timed steps of the plain FP64 form")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-points", type=int, default=4, help="points per CPU reference sample solve")
    ap.add_argument("--cpu-slice-s", type=float, default=8.0, help="seconds of CPU work per reference-arm step")
    ap.add_argument("--serve-requests", type=int, default=32,
                    help="requests of the serving mix (Poisson arrivals, 1-512 points, 15 grid sizes); the "
                         "first requests of the 2000-request stream")
    ap.add_argument("--serve-loads", default="0.5,0.8,1.0",
                    help="Poisson offered loads of the lambda sweep, as fractions of the plain FP64 capacity")
    ap.add_argument("--serve-saturation-only", action="store_true",
                    help="serving: only the saturation runs (every request queued at t = 0), no Poisson sweep")
    ap.add_argument("--serve-budget-gb", type=float, default=16.0, help="HBM budget of admitted points")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-1d", action="store_true", help="skip the 1D3V (config 4) leg")
    ap.add_argument("--c5-points", type=int, default=2048, help="points of the config-5 sample (0: skip)")
    ap.add_argument("--c5-plain-points", type=int, default=2048,
                    help="points of the plain FP64 run of the config-5 sample (the same points, for a fair ratio)")
    ap.add_argument("--steps-1d", type=int, default=20)
    ap.add_argument("--steps-fvm", type=int, default=10)
    ap.add_argument("--no-fvm", action="store_true", help="skip the finite-volume 1D3V leg")
    ap.add_argument("--no-ref-points", action="store_true",
                    help="skip the errors against the reference's answers at the c2-shape fixture points")
    ap.add_argument("--krylov", type=int, default=0,
                    help="mixed form: GMRES on the FP32 factors before an FP64 hand-over (bte_solve_opts.krylov)")
    ap.add_argument("--refine", type=int, default=4, help="mixed form: FP64 refinement passes per Newton step")
    ap.add_argument("--lu64-kernel", type=int, default=0,
                    help="FP64 factorizations: 0 library choice, 1 one CTA per system, 6 split over many CTAs")
    ap.add_argument("--lu-kernel", type=int, default=0,
                    help="FP32 factorization of the mixed form: 0 library choice, 2 tensor cores, 3 SIMT left-looking")
    return ap.parse_args()


def workload_config(a, precision):
    return {
        "workload": "batched 0D3V steady-state EDF solve: %d points, %d B-splines x l_max %d (n=%d), e-e Coulomb on, "
                    "E/N log-uniform [1,1000] Td, ionization degree log-uniform [1e-8,1e-3], seed %d"
                    % (a.n_pts, a.n_sp, a.l_max, a.n_sp * (a.l_max + 1), a.seed),
        "n_pts_per_gpu": a.n_pts, "n_sp": a.n_sp, "l_max": a.l_max, "precision": precision,
        "step": "maxwellian init + e-e-off warm start + e-e-on Newton solve + QoIs",
        "cache": "inputs larger than L2: each step streams %.1f GB of Jacobians" % (
            a.n_pts * (a.n_sp * (a.l_max + 1) + 1) ** 2 * (4 if precision == "mixed" else 8) / 1e9),
        "parallelism": "points sharded across GPUs, no collective on the data path",
        "refine": a.refine, "krylov": a.krylov,
    }


def dist_init(n):
    if n <= 1 or "RANK" not in os.environ:
        return 0, 1
    import torch.distributed as dist
    backend = "nccl"
    dist.init_process_group(backend=backend)
    return dist.get_rank(), dist.get_world_size()


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws):
    from boltzmann_gb300.sharding import max_over_ranks as mor
    return mor(x, ws)


class Clocks:
    """nvidia-smi sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def make_solver(xs, a, precision, dev):
    from boltzmann_gb300.bte_0d3v_batched import bte_0d3v_batched, vspace_grid_extension
    from boltzmann_gb300.workloads import EV_MAX, TE_NORM
    args = types.SimpleNamespace(threads=1, sp_order=3, spline_qpts=5, ee_collisions=1, verbose=0, use_gpu=1,
                                 Efreq=0.0, dt=1e-3, cycles=1, solver_type="steady-state", l_max=a.l_max,
                                 Nr=a.n_sp - 1, n_pts=a.n_pts, precision=precision,
                                 lu_kernel=getattr(a, "lu_kernel", 0), krylov=getattr(a, "krylov", 0),
                                 refine=getattr(a, "refine", 4), lu64_kernel=getattr(a, "lu64_kernel", 0))
    s = bte_0d3v_batched(args, np.array([EV_MAX]), np.array([TE_NORM]), np.array([a.n_sp - 1]),
                         [[[l, 0] for l in range(a.l_max + 1)]], 1, [xs])
    s._dev_id = dev
    t0 = time.perf_counter()
    s.assemble_operators(0, vspace_ext=vspace_grid_extension.NONE)
    return s, args, time.perf_counter() - t0


def full_solve(s, args, f0):
    """One EDF solve of the batch: e-e-off warm start then e-e-on (bte_0d3v_batched_driver.py:192-204)."""
    args.ee_collisions = 0
    ff, _ = s.solve(0, f0, ATOL, RTOL, MAXIT, "steady-state", ALPHA_MIN, ALPHA_RHO, LS_C)
    args.ee_collisions = 1
    return s.solve(0, ff, ATOL, RTOL, MAXIT, "steady-state", ALPHA_MIN, ALPHA_RHO, LS_C)


def run_gb300(a, rank, ws):
    import torch
    from boltzmann_gb300 import _lib
    from boltzmann_gb300.workloads import write_synthetic_lxcat, batch_parameters
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    xs = write_synthetic_lxcat()
    prm = batch_parameters(a.n_pts, a.seed + 7919 * rank)
    s, args, t_setup = make_solver(xs, a, "mixed", dev)
    for k in ["n0", "ne", "ns_by_n0", "Tg", "E"]:
        s.set_boltzmann_parameter(0, k, prm[k])
    f0_host = s.initialize(0, a.n_pts)
    s.host_to_device_setup(dev, 0)
    f0 = torch.as_tensor(f0_host, device="cuda")
    stream = torch.cuda.current_stream()

    for _ in range(a.warmup):
        ff, q = full_solve(s, args, f0)
    torch.cuda.synchronize()
    barrier(ws)
    _lib.stats_reset(timing=True)
    clocks = Clocks(dev)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    step_ms = []
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(a.steps):
        e_a = torch.cuda.Event(enable_timing=True)
        e_b = torch.cuda.Event(enable_timing=True)
        e_a.record(stream)
        ff, q = full_solve(s, args, f0)
        e_b.record(stream)
        step_ms.append((e_a, e_b))
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(ws)
    st = _lib.stats()
    ms = ev0.elapsed_time(ev1) / a.steps
    ms = max_over_ranks(ms, ws)
    steps_ms = [x.elapsed_time(y) for x, y in step_ms]
    value = a.n_pts * ws / (ms / 1e3)
    status = q["status"].cpu().numpy()
    iters = q["iters"].cpu().numpy()
    ff_mixed = ff.detach().cpu().numpy()

    # end to end through the public API with host buffers (H2D of inputs, D2H of results inside)
    s2_params = {k: prm[k] for k in ["n0", "ne", "ns_by_n0", "Tg", "E"]}
    for k, v in s2_params.items():
        s.set_boltzmann_parameter(0, k, v)
    s.xp_module = np
    full_solve(s, args, f0_host)
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(a.steps):
        ff_h, q_h = full_solve(s, args, f0_host)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / a.steps, ws)
    n = f0_host.shape[0]
    h2d = f0_host.nbytes * 2 + 8 * (4 + 1) * a.n_pts * 2  # f0 + parameters, two solves per step
    d2h = (n * a.n_pts * 8 + (3 + len(q_h["rates"])) * a.n_pts * 8 + 2 * 4 * a.n_pts) * 2
    e2e = {"value": a.n_pts * ws / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
           "path": "bte_0d3v_batched.solve() with NumPy host arrays"}

    # plain FP64 form on the same batch: throughput and the error of the mixed form against it
    plain = None
    if not a.no_plain:
        sp, argsp, _ = make_solver(xs, a, "fp64", dev)
        for k in ["n0", "ne", "ns_by_n0", "Tg", "E"]:
            sp.set_boltzmann_parameter(0, k, prm[k])
        sp.host_to_device_setup(dev, 0)
        full_solve(sp, argsp, f0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(a.plain_steps):
            ffp, qp = full_solve(sp, argsp, f0)
        torch.cuda.synchronize()
        pms = (time.perf_counter() - t0) / a.plain_steps * 1e3
        ffp = ffp.detach().cpu().numpy()
        err = np.linalg.norm(ff_mixed - ffp, axis=0) / np.linalg.norm(ffp, axis=0)
        qerr = {k: float(np.max(np.abs(q[k].cpu().numpy() - qp[k].cpu().numpy()) / np.abs(qp[k].cpu().numpy())))
                for k in ("energy", "mobility", "diffusion")}
        worst = np.argsort(err)[-5:][::-1]
        plain = {"value": a.n_pts * ws / (pms / 1e3), "ms_per_step": pms,
                 "mixed_speedup": (a.n_pts * ws / (ms / 1e3)) / (a.n_pts * ws / (pms / 1e3)),
                 "edf_max_rel_err_mixed_vs_fp64": float(np.max(err)), "qoi_max_rel_err_mixed_vs_fp64": qerr,
                 "edf_rel_err_percentiles": {p: float(np.percentile(err, float(p))) for p in ("50", "90", "99", "99.9")},
                 "points_above_1e-8": int(np.sum(err > 1e-8)),
                 "worst_points": [{"EbyN_Td": float(prm["EbyN"][i]), "ion_deg": float(prm["ne"][i] / prm["n0"][i]),
                                   "err": float(err[i])} for i in worst],
                 "status_counts": {str(k): int(v) for k, v in zip(*np.unique(qp["status"].cpu().numpy(), return_counts=True))}}
        del sp
    os.unlink(xs)
    return dict(value=value, ms=ms, steps_ms=steps_ms, stats=st, clocks=clk, status=status, iters=iters, e2e=e2e,
                plain=plain, setup_s=t_setup)


def _serve_run(xs, specs, precision, a, rate=None):
    """One serving run: requests submitted at their arrival times (all at once if rate is None)."""
    from boltzmann_gb300.serving import BteServer, SolveRequest, wait_all, latency_summary
    grids = sorted({(r["n_sp"], r["l_max"]) for r in specs})
    mk = lambda r: SolveRequest(n_sp=r["n_sp"], l_max=r["l_max"], n0=r["n0"], ne=r["ne"], Tg=r["Tg"], E=r["E"],
                                ns_by_n0=r["ns_by_n0"])
    t_setup = time.perf_counter()
    srv = BteServer(xs, grids, precision=precision, hbm_budget_bytes=int(a.serve_budget_gb * (1 << 30)),
                    capacity=512, fp64_capacity=64)
    try:
        s0 = specs[0]
        warm = [srv.submit(mk(dict(n_sp=g[0], l_max=g[1], n0=s0["n0"][:2], ne=s0["ne"][:2], Tg=s0["Tg"][:2],
                                   E=s0["E"][:2], ns_by_n0=s0["ns_by_n0"][:, :2]))) for g in grids]
        wait_all(warm, timeout=600)
        t_setup = time.perf_counter() - t_setup
        t0 = time.perf_counter()
        reqs = []
        for r in specs:
            if rate is not None:
                dt = t0 + r["t"] - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
            reqs.append(srv.submit(mk(r)))
        wait_all(reqs, timeout=3600)
        summ = latency_summary(reqs)
        summ["peak_budget_used_gb"] = srv.peak_used / (1 << 30)
        summ["setup_s"] = t_setup
        summ["status_counts"] = {str(k): int(v) for k, v in zip(*np.unique(
            np.concatenate([q.qoi["status"] for q in reqs]), return_counts=True))}
    finally:
        srv.close()
    return summ, reqs


def serve_bench(a):
    """Serving mix: Poisson arrivals of requests of 1-512 points on grids N_sp in {64..256} x
    l_max in {1,2,3} (seed 20261204). Capacity of each form from a run with every request
    queued at t = 0; latency from Poisson arrivals at 80% of the plain FP64 capacity."""
    import torch
    from boltzmann_gb300.workloads import write_synthetic_lxcat, serving_requests
    xs = write_synthetic_lxcat()
    try:
        specs = serving_requests(a.serve_requests, float("inf"))
        pts = sum(len(r["n0"]) for r in specs)
        sat = {}
        for prec in ("mixed", "fp64"):
            summ, _ = _serve_run(xs, specs, prec, a)
            sat[prec] = summ
            torch.cuda.empty_cache()
        cap_fp64 = sat["fp64"]["solves_per_s"]
        if a.serve_saturation_only:
            return {"workload": "the first %d requests of the seeded 2000-request stream, all queued at t = 0; %d points"
                                % (len(specs), pts), "hbm_budget_gb": a.serve_budget_gb,
                    "saturation": {"mixed": sat["mixed"], "fp64": sat["fp64"],
                                   "mixed_over_fp64": sat["mixed"]["solves_per_s"] / cap_fp64}}
        # lambda sweep: Poisson arrivals at fractions of the plain FP64 capacity, both forms;
        # the 0.8 point is the one the error comparison uses
        loads = [float(x) for x in a.serve_loads.split(",") if x.strip()]
        if 0.8 not in loads:
            loads.append(0.8)
        sweep, res = [], {}
        for load in loads:
            rate = load * cap_fp64 / (pts / len(specs))  # requests per second
            specs_p = serving_requests(a.serve_requests, rate)
            row = {"offered_load_of_fp64_capacity": load, "rate_requests_per_s": rate,
                   "offered_solves_per_s": load * cap_fp64}
            for prec in ("mixed", "fp64"):
                summ, reqs = _serve_run(xs, specs_p, prec, a, rate=rate)
                row[prec] = summ
                if load == 0.8:
                    res[prec] = reqs
                torch.cuda.empty_cache()
            sweep.append(row)
        pois = next(r for r in sweep if r["offered_load_of_fp64_capacity"] == 0.8)
        rate = pois["rate_requests_per_s"]
        # per-point EDF difference over points both forms converged (status 0 or 1)
        err, n_unconv = [], 0
        for m, p in zip(res["mixed"], res["fp64"]):
            ok = (m.qoi["status"] <= 1) & (p.qoi["status"] <= 1)
            n_unconv += int(np.sum(~ok))
            err.append((np.linalg.norm(m.ff - p.ff, axis=0) / np.linalg.norm(p.ff, axis=0))[ok])
        err = np.concatenate(err)
    finally:
        os.unlink(xs)
    return {
        "workload": "the first %d requests of the seeded 2000-request stream (1-512 points, N_sp in "
                    "{64,96,128,192,256} x l_max in {1,2,3}, E/N log-uniform [1,1000] Td, ionization degree log-uniform "
                    "[1e-8,1e-3], e-e warm start then e-e on), seed 20261204; %d points" % (len(specs), pts),
        "hbm_budget_gb": a.serve_budget_gb,
        "saturation": {"mixed": sat["mixed"], "fp64": sat["fp64"],
                       "mixed_over_fp64": sat["mixed"]["solves_per_s"] / cap_fp64},
        "poisson": {"rate_requests_per_s": rate, "offered_solves_per_s": 0.8 * cap_fp64,
                    "mixed": pois["mixed"], "fp64": pois["fp64"]},
        "lambda_sweep": [{"load": r["offered_load_of_fp64_capacity"], "rate_requests_per_s": r["rate_requests_per_s"],
                          "mixed": {k: r["mixed"][k] for k in ("p50_ms", "p99_ms", "solves_per_s")},
                          "fp64": {k: r["fp64"][k] for k in ("p50_ms", "p99_ms", "solves_per_s")}} for r in sweep],
        "edf_rel_err_mixed_vs_fp64": {"max": float(err.max()), "p50": float(np.median(err)),
                                      "p99": float(np.percentile(err, 99)), "points_above_1e-8": int(np.sum(err > 1e-8)),
                                      "points_compared": int(err.size), "points_unconverged_in_either": n_unconv},
    }


def bench_reference_points(a):
    """The mixed and plain forms on the points of the c2-shape reference fixture
    (tests/golden/c2_shape_reference.npz: 128 B-splines x l_max 2, e-e on, 8 points, three of
    them at E/N < 10 Td and ionization above 1e-4), each EDF's relative L2 error against the
    reference's own solution of the same point, with the reference's final residual and the
    shift of its answer under rounding-level perturbations of its operators."""
    import torch
    from boltzmann_gb300.workloads import write_synthetic_lxcat
    g = dict(np.load(os.path.join(ROOT, "tests", "golden", "c2_shape_reference.npz")))
    P = g["ff"].shape[1]
    ns = types.SimpleNamespace(n_sp=int(g["n_sp"]), l_max=int(g["l_max"]), n_pts=P)
    xs = write_synthetic_lxcat()
    out = {"points": [{"EbyN_Td": float(e), "ion_deg": float(i)} for e, i in zip(g["EbyN"], g["ion_deg"])],
           "reference_rel_error": [float(x) for x in g["rel_error"]]}
    for k in ("resolution", "resolution_mass", "rosenbluth_swap_shift"):
        if k in g:
            out["reference_" + k] = [float(x) for x in g[k]]
    try:
        for prec in ("mixed", "fp64"):
            s, args, _ = make_solver(xs, ns, prec, 0)
            for k in ["n0", "ne", "ns_by_n0", "Tg", "E"]:
                s.set_boltzmann_parameter(0, k, g[k])
            ff, q = full_solve(s, args, torch.as_tensor(s.initialize(0, P), device="cuda"))
            ff = ff.cpu().numpy()
            out["edf_rel_err_%s" % prec] = [float(x) for x in np.linalg.norm(ff - g["ff"], axis=0)
                                            / np.linalg.norm(g["ff"], axis=0)]
            del s
    finally:
        os.unlink(xs)
    return out


def bench_c5(a):
    """Config 5 (256 B-splines x l_max 4: n = 1280, 1281 x 1281 bordered systems, e-e on, ionization
    degree 1e-6..1e-2, seed 20261205) on a sample of its 16384 points: one full EDF solve of
    the sample in the mixed form (its first solve: the time includes the workspace set-up), and
    the plain FP64 form on the first points for the error. The sample's wall time is set by its
    slowest points (a few run to max_iter), not by its size."""
    import torch
    from boltzmann_gb300.workloads import write_synthetic_lxcat, config_parameters, CONFIGS
    c = CONFIGS["c5"]
    xs = write_synthetic_lxcat()
    try:
        ns = types.SimpleNamespace(n_sp=c["n_sp"], l_max=c["l_max"], n_pts=a.c5_points)
        prm = config_parameters("c5", c["n_pts"])
        sub = {k: (v[..., :a.c5_points] if isinstance(v, np.ndarray) else v) for k, v in prm.items()}
        s, args, t_setup = make_solver(xs, ns, "mixed", 0)
        for k in ["n0", "ne", "ns_by_n0", "Tg", "E"]:
            s.set_boltzmann_parameter(0, k, sub[k])
        f0 = torch.as_tensor(s.initialize(0, a.c5_points), device="cuda")
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ff, q = full_solve(s, args, f0)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        ffm = ff.cpu().numpy()
        stm = q["status"].cpu().numpy()
        del s
        torch.cuda.empty_cache()
        m = a.c5_plain_points
        ns.n_pts = m
        sp, argsp, _ = make_solver(xs, ns, "fp64", 0)
        for k in ["n0", "ne", "ns_by_n0", "Tg", "E"]:
            sp.set_boltzmann_parameter(0, k, sub[k][..., :m])
        f0p = torch.as_tensor(sp.initialize(0, m), device="cuda")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ffp, qp = full_solve(sp, argsp, f0p)
        torch.cuda.synchronize()
        pms = (time.perf_counter() - t0) * 1e3
        ffp = ffp.cpu().numpy()
        stp = qp["status"].cpu().numpy()
        ok = (stm[:m] <= 1) & (stp <= 1)
        err_all = np.linalg.norm(ffm[:, :m] - ffp, axis=0) / np.linalg.norm(ffp, axis=0)
        err = err_all[ok]
        rem, rep = q["rel_error"].cpu().numpy()[:m], qp["rel_error"].cpu().numpy()
        worst = [int(i) for i in np.argsort(np.where(ok, err_all, -1.0))[-5:][::-1]]
        worst = [{"point": i, "EbyN_Td": float(sub["EbyN"][i]), "ion_deg": float(sub["ne"][i] / sub["n0"][i]),
                  "err": float(err_all[i]), "rel_error_mixed": float(rem[i]), "rel_error_fp64": float(rep[i]),
                  "iters_mixed": int(q["iters"].cpu().numpy()[i]), "iters_fp64": int(qp["iters"].cpu().numpy()[i])}
                 for i in worst]
        del sp
        torch.cuda.empty_cache()
    finally:
        os.unlink(xs)
    return {"workload": "config 5 sample: first %d of its 16384 points (256 B-splines x l_max 4, n = 1280, e-e on, "
                        "ionization degree 1e-6..1e-2, seed 20261205)" % a.c5_points,
            "value": a.c5_points / (ms / 1e3), "unit": "solves/s", "ms_per_step": ms, "setup_s": t_setup,
            "status_counts": {str(k): int(v) for k, v in zip(*np.unique(stm, return_counts=True))},
            "newton_iters": {"mean": float(np.mean(q["iters"].cpu().numpy())),
                             "max": int(np.max(q["iters"].cpu().numpy()))},
            "plain_fp64": {"points": m, "value": m / (pms / 1e3), "ms_per_step": pms,
                           "edf_rel_err_mixed_vs_fp64": {"max": float(err.max()) if err.size else None,
                                                         "p50": float(np.median(err)) if err.size else None,
                                                         "p99": float(np.percentile(err, 99)) if err.size else None,
                                                         "points_above_1e-8": int(np.sum(err > 1e-8)),
                                                         "points_compared": int(err.size),
                                                         "worst_points": worst}}}


C4 = dict(L=2.54e-2, V0=100.0, freq=13.56e6, Tg=300.0, p0=1.0, atol=1e-14, rtol=1e-10, gmres_rsrt=30,
          gmres_rsrt_iter=20, max_iter=300, Np=200, Nr=63, Nvt=16, lmax=1, dt=1e-3, ev_max=80.0, ev_extend=0,
          sp_order=3, spline_qpts=5, Te=4.0, xspace_type=1, vspace_type=1)


def c4_efield(xp, t, p):
    """Synthetic field of the 1D3V workload: (V0 / gap) sin(2 pi t) ramped over x, so that E
    varies along x (t in RF periods)."""
    return (p["V0"] / p["L"]) * np.sin(2 * np.pi * t) * 0.5 * (1.0 + xp)


def bench_1d(a, peaks):
    """1D3V (config 4: 200 Chebyshev points, 64 B-splines x l_max 1, 16 ordinates, dt = 1e-3 RF
    period): the fully implicit step, GMRES(30) to rtol 1e-10 over the coupled v-space +
    Chebyshev x-advection operator with inflow rows, right-preconditioned by the Lie split
    (per-point FP32 v-space blocks, then the backward-Euler x-advection); the Strang split beside
    it for comparison."""
    import torch
    from boltzmann_gb300.bte_1d3v import bte_1d3v
    from boltzmann_gb300.workloads import write_synthetic_lxcat
    xs = write_synthetic_lxcat()
    p = dict(C4, collisions=xs, solver_type="fully_implicit")
    try:
        t0 = time.perf_counter()
        b = bte_1d3v(p)
        t_setup = time.perf_counter() - t0
        v = b.initial_condition()
        dt, t = p["dt"], 0.25
        for _ in range(3):
            v = b.step(c4_efield(b.xp, t, p), v, None, t, dt)
            t += dt
        torch.cuda.synchronize()
        s = torch.cuda.current_stream()
        its, L0 = [], b.launches()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        ev[0].record(s)
        for _ in range(a.steps_1d):
            E = c4_efield(b.xp, t, p)
            v = b.step(E, v, None, t, dt)
            its.append(b.gmres_info["iterations"])
            t += dt
        ev[1].record(s)
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / a.steps_1d
        launches = (b.launches() - L0) / a.steps_1d
        # the coupled operator alone (the GMRES matvec): 2 kernels per application
        E = torch.as_tensor(c4_efield(b.xp, t, p), device="cuda")
        nmv = 50
        for _ in range(3):
            b.fim_mvec(E, v, dt)
        ev[0].record(s)
        for _ in range(nmv):
            b.fim_mvec(E, v, dt)
        ev[1].record(s)
        torch.cuda.synchronize()
        mv_ms = ev[0].elapsed_time(ev[1]) / nmv
        # the Strang split on the same state (x over dt/2, v over dt, x over dt/2), on its own
        # solver (the x-step keeps the factors of one step size)
        bs = bte_1d3v(dict(C4, collisions=xs))
        for _ in range(2):
            bs.step(c4_efield(bs.xp, t, p), v, None, t, dt)
        tx = tv = 0.0
        for _ in range(5):
            E = c4_efield(bs.xp, t, p)
            ev[0].record(s)
            v1 = bs.step_bte_x(v, t, 0.5 * dt)
            ev[1].record(s)
            v2 = bs.step_bte_v(E, v1, None, t, dt)
            ev[2].record(s)
            bs.step_bte_x(v2, t, 0.5 * dt)
            ev[3].record(s)
            torch.cuda.synchronize()
            tx += ev[0].elapsed_time(ev[1]) + ev[2].elapsed_time(ev[3])
            tv += ev[1].elapsed_time(ev[2])
        tx, tv = tx / 5, tv / 5
        del bs
        # end to end through the public API with host arrays
        vh = v.cpu().numpy()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(5):
            E = c4_efield(b.xp, t, p)
            vh = b.step(E, vh, None, t, dt).cpu().numpy()
        e2e_ms = (time.perf_counter() - t0) / 5 * 1e3
        Nr, Nvt, Nx, nsh = p["Nr"] + 1, p["Nvt"], p["Np"], p["lmax"] + 1
        n = Nr * nsh
        M = Nr * Nvt
        # the matvec's algorithmic work: Chebyshev derivative M Nx^2, radial advection Nr^2 Nvt Nx,
        # v-space 2 n^2 Nx, projections 2 M nsh Nx multiply-adds; state in + out
        mv_flops = 2.0 * (M * Nx * Nx + Nr * Nr * Nvt * Nx + 2 * n * n * Nx + 2 * M * nsh * Nx)
        mv_bytes = 2.0 * M * Nx * 8
        fp64 = FP64_NOMINAL_TFLOPS
        out = {
            "workload": "1D3V fully implicit step: 200 Chebyshev points x 64 B-splines x l_max 1 x 16 ordinates "
                        "(204,800 unknowns), GMRES(30) rtol 1e-10 on the coupled v-space + BE Chebyshev "
                        "x-advection operator with inflow rows, Lie-split preconditioner (FP32 per-point v blocks, "
                        "BE x-advection), E(x,t) = (V0/gap) sin(2 pi t) (1+x)/2",
            "value": 1e3 / ms, "unit": "steps/s", "ms_per_step": ms, "setup_s": t_setup,
            "gmres_iterations": {"mean": float(np.mean(its)), "max": int(np.max(its)), "min": int(np.min(its))},
            "gpu_launches_per_step": launches, "matvec_ms": mv_ms,
            "roofline_matvec": {"kernel": "k_fim_dx + k_fim_combine", "bound": "fp64",
                                "achieved": mv_flops / (mv_ms * 1e-3) / 1e12, "peak": fp64, "unit": "TFLOP/s",
                                "frac": mv_flops / (mv_ms * 1e-3) / 1e12 / fp64,
                                "peak_source": "nominal GB300 FP64 (no measured FP64 peak)",
                                "alg_flops": mv_flops, "alg_bytes": mv_bytes,
                                "hbm_gbs_achieved": mv_bytes / (mv_ms * 1e-3) / 1e9},
            "strang_split": {"ms_per_step": tx + tv, "x_steps_ms": tx, "v_step_ms": tv},
            "e2e": {"value": 1e3 / e2e_ms, "unit": "steps/s", "h2d_bytes_per_step": int(vh.nbytes + Nx * 8),
                    "d2h_bytes_per_step": int(vh.nbytes), "path": "bte_1d3v.step() with NumPy host arrays"},
        }
        if not a.no_cpu:
            import multiprocessing
            from oracle.bte1d_oracle import Oracle1D
            o = Oracle1D(xs, Nx, p["Nr"], Nvt, p["lmax"], p["ev_max"], p["Te"], p["L"], p["freq"], p["Tg"], p["p0"])
            vo = v.cpu().numpy()
            t0 = time.perf_counter()
            _, cits = o.step_fim_gmres(c4_efield(o.xp, t, p), vo, dt, rtol=p["rtol"], restart=p["gmres_rsrt"])
            sec = time.perf_counter() - t0
            out["cpu_baseline"] = {"value": 1.0 / sec, "unit": "steps/s", "cores": multiprocessing.cpu_count(),
                                   "kind": "port", "sample": "one fully implicit step of the same workload (NumPy "
                                   "matrix-free operator, SciPy GMRES(30) with the same Lie-split preconditioner, %d "
                                   "iterations)" % cits}
    finally:
        os.unlink(xs)
    return out


FVM_C4 = dict(L=2.54e-2, V0=100.0, freq=13.56e6, Tg=300.0, p0=1.0, atol=1e-14, rtol=1e-10, gmres_rsrt=30,
              gmres_rsrt_iter=20, Np=200, Nr=63, Nvt=16, lmax=1, dt=1e-3, ev_max=80.0, ev_extend=0, sp_order=3,
              spline_qpts=5, Te=4.0, xspace_type=0, vspace_type=0, solver_type="fully_implicit", adaptive_grid=1,
              pvr=2, pvt=2, px=2, ic_file="")


def bench_fvm(a, peaks):
    """The finite-volume 1D3V fully implicit step (the reference's solver_type "fully_implicit",
    bte_1d3v_solver.py:1890-2009) at the 1D3V workload's size: 200 upwind x points, the radial
    cells of 64 B-splines x 5 Gauss points, 16 ordinates; GMRES(30) rtol 1e-10 preconditioned
    by the op-split step. Its operator (k_fvm_mvec) is one read and one write of the state."""
    import torch
    from boltzmann_gb300.bte_1d3v_fvm import bte_1d3v_fvm
    from boltzmann_gb300.workloads import write_synthetic_lxcat
    xs = write_synthetic_lxcat()
    p = dict(FVM_C4, collisions=xs)
    try:
        t0 = time.perf_counter()
        b = bte_1d3v_fvm(p)
        dt = p["dt"]
        b.init(dt)
        t_setup = time.perf_counter() - t0
        v = b.initial_condition()
        t = 0.25
        for _ in range(3):
            v = b.step(c4_efield(b.xp, t, p), v, None, t, dt)
            t += dt
        torch.cuda.synchronize()
        s = torch.cuda.current_stream()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        its, L0 = [], b.launches()
        ev[0].record(s)
        for _ in range(a.steps_fvm):
            v = b.step(c4_efield(b.xp, t, p), v, None, t, dt)
            its.append(b.gmres_info["iterations"])
            t += dt
        ev[1].record(s)
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / a.steps_fvm
        launches = (b.launches() - L0) / a.steps_fvm
        E = c4_efield(b.xp, t, p)
        timing = {}
        for name, fn in (("matvec", lambda: b.rhs_mvec(E, v, dt)),
                         ("precond", lambda: b.step_op_split(E, v, None, t, dt))):
            for _ in range(3):
                fn()
            ev[0].record(s)
            for _ in range(30):
                fn()
            ev[1].record(s)
            torch.cuda.synchronize()
            timing[name] = ev[0].elapsed_time(ev[1]) / 30
        vh = v.cpu().numpy()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            vh = b.step(c4_efield(b.xp, t, p), vh, None, t, dt).cpu().numpy()
        e2e_ms = (time.perf_counter() - t0) / 3 * 1e3
        N = b.dof_vr * b.dof_vt * b.dof_x
        hbm = peaks.get("hbm_gbs") or 6800.0
        mv_bytes = 2.0 * N * 8                # state in, result out
        pc_bytes = 8.0 * N * 8                # collision solve in/out, three sweeps in place, x rows in/out
        out = {
            "workload": "1D3V finite-volume fully implicit step: %d upwind x points x %d radial cells x %d ordinates "
                        "(%d unknowns), stencil orders 2, GMRES(30) rtol 1e-10, op-split preconditioner"
                        % (b.dof_x, b.dof_vr, b.dof_vt, N),
            "value": 1e3 / ms, "unit": "steps/s", "ms_per_step": ms, "setup_s": t_setup,
            "gmres_iterations": {"mean": float(np.mean(its)), "max": int(np.max(its))},
            "gpu_launches_per_step": launches, "matvec_ms": timing["matvec"], "precond_ms": timing["precond"],
            "roofline_matvec": {"kernel": "k_fvm_moment + gain GEMM + k_fvm_mvec", "bound": "hbm",
                                "achieved": mv_bytes / (timing["matvec"] * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                                "frac": mv_bytes / (timing["matvec"] * 1e-3) / 1e9 / hbm, "alg_bytes": mv_bytes},
            "roofline_precond": {"kernel": "collision solve + coalesced v_r, v_theta, x sweeps", "bound": "hbm",
                                 "achieved": pc_bytes / (timing["precond"] * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                                 "frac": pc_bytes / (timing["precond"] * 1e-3) / 1e9 / hbm, "alg_bytes": pc_bytes},
            "e2e": {"value": 1e3 / e2e_ms, "unit": "steps/s", "h2d_bytes_per_step": int(vh.nbytes + b.dof_x * 8),
                    "d2h_bytes_per_step": int(vh.nbytes), "path": "bte_1d3v_fvm.step() with NumPy host arrays"},
        }
    finally:
        os.unlink(xs)
    return out


# the pipe each kernel family runs on: roofline denominators from MEASURED_PEAKS.json
# (HBM copy GB/s, dense bf16 TFLOP/s). The FP32 factorization runs its trailing updates as
# tcgen05 kind::tf32 MMAs, whose dense rate is half the bf16 rate; FP64 families run on the
# FP64 pipe, for which no measured peak exists (nominal 1.25 TFLOP/s on GB300).
FAMILY_PIPE = {"lu_factor": "tensor_tf32", "lu_factor_fp64": "fp64", "jacobian": "fp64", "refine": "fp64",
               "residual": "fp64", "lu_solve": "hbm", "other": "hbm"}
FP64_NOMINAL_TFLOPS = 1.25


def family_roofline(name, v, peaks):
    """Roofline of one kernel family: algorithmic flops and bytes per launch over its average
    launch time (CUDA events), bound by arithmetic intensity against the ridge point."""
    hbm = peaks.get("hbm_gbs") or 6800.0
    bf16 = peaks.get("bf16_tflops") or 1900.0
    pipe = FAMILY_PIPE.get(name, "hbm")
    n = max(v["launches"], 1)
    t = v["ms"] / 1e3 / n
    fl, by = v["flops"] / n, v["bytes"] / n
    gbs = by / t / 1e9 if t > 0 else 0.0
    tfs = fl / t / 1e12 if t > 0 else 0.0
    ai = fl / by if by > 0 else float("inf")
    if pipe == "tensor_tf32":
        pk, src = bf16 / 2, "MEASURED_PEAKS.json bf16_tflops / 2 (dense TF32 rate, of measured)"
    elif pipe == "fp64":
        pk, src = FP64_NOMINAL_TFLOPS, "nominal GB300 FP64 1.25 TFLOP/s (no measured FP64 peak)"
    else:
        pk, src = None, None
    ridge = pk * 1e12 / (hbm * 1e9) if pk else float("inf")
    both = {"frac_hbm": gbs / hbm, "frac_pipe": (tfs / pk) if pk else None}
    if pk and ai >= ridge:
        return {"kernel": name, "bound": "tensor" if pipe == "tensor_tf32" else "fp64", "achieved": tfs, "peak": pk,
                "unit": "TFLOP/s", "frac": tfs / pk, "peak_source": src, "arith_intensity": ai, "ridge": ridge,
                "hbm_gbs_achieved": gbs, "avg_launch_ms": t * 1e3, "alg_flops_per_launch": fl,
                "alg_bytes_per_launch": by, **both}
    return {"kernel": name, "bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks.get("hbm_gbs") else "fallback",
            "arith_intensity": ai, "ridge": ridge, "tflops_achieved": tfs, "avg_launch_ms": t * 1e3,
            "alg_flops_per_launch": fl, "alg_bytes_per_launch": by, "pipe_peak": pk, "pipe_peak_source": src, **both}


def roofline(st, peaks):
    """The dominant kernel family's roofline (the `roofline` object), with every family's
    beside it. `traffic` is DRAM read + write per launch of the dominant family from the ncu
    capture summarized in profiles/ (its DRAM bytes per algorithmic byte, scaled to this run's
    average launch)."""
    fams = {k: v for k, v in st.items() if isinstance(v, dict) and "ms" in v and v["launches"] > 0}
    dom = max(fams, key=lambda k: fams[k]["ms"])
    out = family_roofline(dom, fams[dom], peaks)
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        rec = json.load(open(tpath)).get(dom)
        if rec and rec.get("alg_bytes_per_launch"):
            traffic = rec["dram_bytes_per_launch"] / rec["alg_bytes_per_launch"] * out["alg_bytes_per_launch"]
    out["traffic"] = traffic
    out["families"] = {k: {kk: (round(vv, 6) if isinstance(vv, float) else vv)
                           for kk, vv in family_roofline(k, f, peaks).items()
                           if kk in ("bound", "achieved", "unit", "frac", "avg_launch_ms")} for k, f in fams.items()}
    out["families_ms"] = {k: round(f["ms"], 3) for k, f in fams.items()}
    return out


class CpuReferenceRun:
    """The reference's CPU algorithm on the host cores: the oracle port of the reference's
    bte_0d3v_batched (NumPy/OpenBLAS, all host threads) solving consecutive samples of
    `n_pts` points of the same seeded workload, each to the reference's own stop criterion
    (e-e-off solve from the Maxwellian, then the e-e-on solve from its result, batch-global
    loop up to max_iter = 100 or the line-search break). The solves advance in bounded time
    slices (whole Newton iterations), so a benchmark step is bounded while every sample still
    runs to the end; throughput = points of completed samples / seconds spent on them. The
    operator set-up (assembly, dense Coulomb tensor) is not timed."""

    def __init__(self, a, n_pts):
        import multiprocessing
        from oracle import bte_oracle as O
        from boltzmann_gb300.workloads import write_synthetic_lxcat, EV_MAX, TE_NORM
        self.O, self.a, self.n_pts = O, a, n_pts
        self.cores = multiprocessing.cpu_count()
        xs = write_synthetic_lxcat()
        t0 = time.perf_counter()
        try:
            self.ops = O.Operators(O.processes_from_lxcat(xs), EV_MAX, TE_NORM, a.n_sp, a.l_max, ee=True)
        finally:
            os.unlink(xs)
        self.setup_s = time.perf_counter() - t0
        self.done = []
        self.k = 0
        self._start()

    def _start(self):
        from boltzmann_gb300.workloads import batch_parameters
        O = self.O
        prm = batch_parameters(self.a.n_pts, self.a.seed)
        sl = slice(self.k * self.n_pts, (self.k + 1) * self.n_pts)
        P = O.Params(prm["n0"][sl], prm["ne"][sl], prm["Tg"][sl], prm["E"][sl], prm["ns_by_n0"][:, sl])
        self.gen = self._solve(P)
        self.spent = 0.0

    def _solve(self, P):
        O = self.O
        f0 = O.maxwellian_initial(self.ops, self.n_pts)
        ff, _, i1 = yield from O.steady_state_iterations(self.ops, P, f0, ATOL, RTOL, MAXIT, False, ALPHA_MIN,
                                                         ALPHA_RHO, LS_C)
        _, _, i2 = yield from O.steady_state_iterations(self.ops, P, ff, ATOL, RTOL, MAXIT, True, ALPHA_MIN,
                                                        ALPHA_RHO, LS_C)
        return i1, i2

    def run_slice(self, budget_s):
        """Newton iterations of the current sample (and the next ones) for about budget_s."""
        t0 = time.perf_counter()
        while True:
            t1 = time.perf_counter()
            try:
                next(self.gen)
                self.spent += time.perf_counter() - t1
            except StopIteration as stop:
                self.spent += time.perf_counter() - t1
                i1, i2 = stop.value
                self.done.append({"points": self.n_pts, "seconds": self.spent, "iters": [i1["iters"], i2["iters"]],
                                  "res_evals": [i1["res_evals"], i2["res_evals"]],
                                  "stop": [i1["status"], i2["status"]]})
                self.k += 1
                self._start()
            if time.perf_counter() - t0 >= budget_s:
                return

    def summary(self):
        pts = sum(d["points"] for d in self.done)
        sec = sum(d["seconds"] for d in self.done)
        return {"value": pts / sec if sec > 0 else None, "unit": UNIT, "cores": self.cores, "kind": "port",
                "sample": "%d completed sample(s) of %d consecutive points of the seeded c2 workload, each solved to "
                          "the reference's stop criterion (e-e off then e-e on, batch-global loop); Newton iterations "
                          "per sample %s, stop %s; oracle port of bte_0d3v_batched (NumPy, OpenBLAS on all %d host "
                          "threads); operator set-up %.1f s not timed"
                          % (len(self.done), self.n_pts, [d["iters"] for d in self.done],
                             [d["stop"] for d in self.done], self.cores, self.setup_s),
                "seconds": sec, "samples": self.done}


# Counts of the reference's batch-global loop on the cpu_baseline sample (the first 4 points of
# the seeded c2 workload), from running it to its stop criterion on the GPU host's cores (the
# reference arm, --impl reference, does so every time and reports them): Newton iterations and
# residual evaluations of the e-e-off and e-e-on phases. Late iterations backtrack their line
# search many times at the FP64 floor, so most of the e-e-on time is residual evaluations.
CPU_SAMPLE_COUNTS = {(128, 2, 4): {"iters": (83, 100), "res_evals": (778, 3328)}}


def cpu_baseline_run(a, reps=3):
    """cpu_baseline of the GPU arm, a bounded sample (the whole solve of the sample takes about
    ten minutes on the GPU host; the reference arm runs it): per phase of the same 4-point
    sample, the closures' set-up, one Newton linear step (Jacobian, batched inverse, product)
    and one residual evaluation of the oracle port of bte_0d3v_batched are timed, each `reps`
    times, and combined with the sample's measured counts (CPU_SAMPLE_COUNTS)."""
    import multiprocessing
    from oracle import bte_oracle as O
    from boltzmann_gb300.workloads import write_synthetic_lxcat, batch_parameters, EV_MAX, TE_NORM
    counts = CPU_SAMPLE_COUNTS.get((a.n_sp, a.l_max, a.cpu_points))
    if counts is None:
        return CpuReferenceRun(a, a.cpu_points).summary() | {"note": "no measured counts for this sample"}
    xs = write_synthetic_lxcat()
    t0 = time.perf_counter()
    try:
        ops = O.Operators(O.processes_from_lxcat(xs), EV_MAX, TE_NORM, a.n_sp, a.l_max, ee=True)
    finally:
        os.unlink(xs)
    t_setup = time.perf_counter() - t0
    prm = batch_parameters(a.n_pts, a.seed)
    sl = slice(0, a.cpu_points)
    P = O.Params(prm["n0"][sl], prm["ne"][sl], prm["Tg"][sl], prm["E"][sl], prm["ns_by_n0"][:, sl])
    f0 = O.maxwellian_initial(ops, a.cpu_points)
    h = f0 / np.dot(ops.u, f0)
    parts, sec = [], 0.0
    for k, ee in enumerate((False, True)):
        t1 = time.perf_counter()
        res, jac, _ = O.rhs_and_jacobian(ops, P, ee)
        t_close = time.perf_counter() - t1
        r = res(h)
        t1 = time.perf_counter()
        for _ in range(reps):
            Linv = np.linalg.inv(jac(h))
            np.dot(ops.Qmat, np.einsum("abc,ca->ba", Linv, -r))
        t_step = (time.perf_counter() - t1) / reps
        t1 = time.perf_counter()
        for _ in range(reps):
            res(h)
        t_res = (time.perf_counter() - t1) / reps
        sec += t_close + counts["iters"][k] * t_step + counts["res_evals"][k] * t_res
        parts.append({"closures_s": t_close, "step_s": t_step, "residual_s": t_res})
    return {"value": a.cpu_points / sec, "unit": UNIT, "cores": multiprocessing.cpu_count(), "kind": "port",
            "sample": "%d points of the seeded c2 workload through the oracle port of bte_0d3v_batched (NumPy, "
                      "OpenBLAS on all host threads): per phase (e-e off, e-e on) the closures' set-up, one Newton "
                      "step (%.3f s, %.3f s) and one residual evaluation (%.3f s, %.3f s) timed, combined with the "
                      "sample's measured counts: iterations %s, residual evaluations %s (the reference arm runs the "
                      "sample to its stop criterion); operator set-up %.1f s not timed"
                      % (a.cpu_points, parts[0]["step_s"], parts[1]["step_s"], parts[0]["residual_s"],
                         parts[1]["residual_s"], list(counts["iters"]), list(counts["res_evals"]), t_setup),
            "seconds_per_sample": sec, "phases": parts, "counts": counts}


def _autotune_report():
    from boltzmann_gb300 import autotune
    return {k: v for k, v in autotune.choices().items()}


def main():
    a = parse()
    rank, ws = dist_init(a.gpus)
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    if a.impl == "reference":
        if rank != 0:
            return
        # the reference's CPU algorithm: each step a bounded slice of consecutive sample solves,
        # each sample run to the reference's stop criterion (no extrapolation of iterations)
        run = CpuReferenceRun(a, a.cpu_points)
        for _ in range(a.warmup):
            run.run_slice(0.0)  # one Newton iteration each
        t0 = time.perf_counter()
        steps = 0
        for _ in range(a.steps):
            run.run_slice(a.cpu_slice_s)
            steps += 1
        while not run.done:  # the timed steps end only once a sample has completed
            run.run_slice(a.cpu_slice_s)
            steps += 1
        elapsed = time.perf_counter() - t0
        summ = run.summary()
        v = summ["value"]
        cfg = workload_config(a, "fp64")
        cfg["sample_points_per_solve"] = a.cpu_points
        line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": steps, "warmup": a.warmup,
                "ms_per_step": 1e3 * elapsed / steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
                "config": cfg, "cpu_baseline": summ,
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    r = run_gb300(a, rank, ws)
    if rank != 0:
        return
    serve = None if (a.no_serve or ws > 1) else serve_bench(a)
    one_d = None if (a.no_1d or ws > 1) else bench_1d(a, peaks)
    fvm = None if (a.no_fvm or ws > 1) else bench_fvm(a, peaks)
    c5 = None if (a.c5_points <= 0 or ws > 1) else bench_c5(a)
    ref_pts = None if (ws > 1 or a.no_ref_points) else bench_reference_points(a)
    cpu = None if a.no_cpu else cpu_baseline_run(a)
    st = r["stats"]
    steps_ms = sorted(r["steps_ms"])
    line = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": r["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "mixed: f32 Jacobian+LU (tf32 tensor-core updates), f64 residual/state, double-double "
                 "residual at the f64 floor", "data": "synthetic",
        "config": workload_config(a, "mixed"),
        "latency_ms": {"p50": float(np.percentile(steps_ms, 50)), "p99": float(np.percentile(steps_ms, 99)),
                       "unit": "batch solve of %d points" % a.n_pts},
        "e2e": r["e2e"], "gpu_launches": st["launches"],
        "fp64_fallback_points_per_step": st["fp64_fallback_points"] / a.steps,
        "fp64_fallback_reasons": st["fp64_fallback_reasons"],
        "roofline": roofline(st, peaks), "cpu_baseline": cpu, "clocks": r["clocks"],
        "plain_fp64": r["plain"], "serving": serve, "bte_1d3v": one_d, "bte_1d3v_fvm": fvm, "c5_sample": c5, "edf_rel_err_vs_reference": ref_pts, "setup_s": r["setup_s"],
        "newton_iters": {"mean": float(np.mean(r["iters"])), "max": int(np.max(r["iters"]))},
        "lu_autotune": _autotune_report(),
        "status_counts": {str(k): int(v) for k, v in zip(*np.unique(r["status"], return_counts=True))},
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
