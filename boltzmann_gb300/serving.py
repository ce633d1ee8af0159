"""Continuous-batching request loop for steady-state EDF solves.

The reference has no serving layer: its driver solves one batch of points per call
(`BESolver/python/bte_0d3v_batched_driver.py:151-204`). Here requests (a batch of points
on one velocity grid, any of several grid sizes) arrive at any time:

* Every grid keeps its operators and the running points' state resident on the device in a
  `bte_engine` (include/bte_gb300.h), driven by its own host thread on its own CUDA stream,
  so the work of different grids overlaps on the device.
* A request is admitted as soon as its grid has free slots and the server's HBM budget has
  room for its points' footprint (Jacobian, pivots and state per point). Requests of one
  grid are admitted in arrival order.
* Admitted points join the running ones at the next Newton iteration and leave when their
  own solve ends; the request completes when its last point does. Each point runs the
  reference driver's sequence (e-e off, then e-e on from that result), with the arithmetic
  of `bte_solve_steady`, so a request's result does not depend on what else is running.

Latency is measured from `submit` to the moment the request's results are on the host.
"""
from __future__ import annotations

import collections
import ctypes as C
import threading
import time
import types
from dataclasses import dataclass, field

import numpy as np

from . import _lib


@dataclass
class SolveRequest:
    """A steady-state solve of P points on the grid (n_sp, l_max). Parameter arrays follow the
    reference's `set_boltzmann_parameter` shapes: n0, ne, Tg, E (P,), ns_by_n0 (n_species, P)."""
    n_sp: int
    l_max: int
    n0: np.ndarray
    ne: np.ndarray
    Tg: np.ndarray
    E: np.ndarray
    ns_by_n0: np.ndarray
    ee: bool = True
    rid: int = -1
    # filled by the server
    ff: np.ndarray | None = None      # (n, P) normalized distributions
    qoi: dict | None = None           # energy, mobility, diffusion (P,), rates (n_proc, P), status, iters
    t_submit: float = 0.0
    t_admit: float = 0.0
    t_done: float = 0.0
    done: threading.Event = field(default_factory=threading.Event)
    error: str | None = None

    @property
    def P(self) -> int:
        return int(np.asarray(self.n0).shape[0])

    @property
    def latency(self) -> float:
        return self.t_done - self.t_submit


class EngineBackend:
    """One `bte_engine` of the C library on one grid; every call is made by the grid's worker
    thread, on the worker's stream."""

    def __init__(self, grid, info, capacity, fp64_capacity, opts, device):
        import torch
        self.torch = torch
        self.lib = _lib.load()
        self.grid, self.info, self.device = grid, info, device
        self.n = info["n"]
        self.n_proc = info["n_proc"]
        self.opts = opts
        h = C.c_void_p()
        _lib.check(self.lib.bte_engine_create(grid, int(capacity), int(fp64_capacity), C.byref(opts), C.byref(h)),
                   "bte_engine_create")
        self.h = h
        ints = (C.c_int * 4)()
        nb = C.c_size_t()
        _lib.check(self.lib.bte_engine_info(h, ints, C.byref(nb)), "bte_engine_info")
        self.capacity = ints[0]
        self.bytes_per_slot = nb.value / max(ints[0], 1)
        self._done = np.zeros(self.capacity, dtype=np.int32)
        self.stream = None

    def bind(self, stream):
        self.stream = stream

    def _s(self):
        return C.c_void_p(self.stream.cuda_stream)

    def free_slots(self) -> int:
        ints = (C.c_int * 4)()
        _lib.check(self.lib.bte_engine_info(self.h, ints, None), "bte_engine_info")
        return ints[1]

    def admit(self, req: SolveRequest) -> np.ndarray:
        torch = self.torch
        P = req.P
        dev = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")
        n0, ne, Tg, E = dev(req.n0), dev(req.ne), dev(req.Tg), dev(req.E)
        ns = dev(np.asarray(req.ns_by_n0, dtype=np.float64).reshape(-1, P))
        f0 = torch.empty((P, self.n), dtype=torch.float64, device="cuda")
        _lib.check(self.lib.bte_initialize(self.grid, P, _lib.ptr(f0), self._s()), "bte_initialize")
        slots = np.zeros(P, dtype=np.int32)
        _lib.check(self.lib.bte_engine_admit(self.h, P, _lib.ptr(n0), _lib.ptr(ne), _lib.ptr(ns), _lib.ptr(Tg),
                                             _lib.ptr(E), _lib.ptr(f0), int(bool(req.ee)),
                                             slots.ctypes.data_as(C.POINTER(C.c_int32)), self._s()),
                   "bte_engine_admit")
        req._dev = (n0, E)
        return slots

    def step(self) -> np.ndarray:
        nd = C.c_int()
        _lib.check(self.lib.bte_engine_step(self.h, C.byref(nd), self._done.ctypes.data_as(C.POINTER(C.c_int32)),
                                            self._s()), "bte_engine_step")
        return self._done[:nd.value].copy()

    def collect(self, req: SolveRequest, slots: np.ndarray) -> None:
        torch = self.torch
        P = len(slots)
        f = torch.empty((P, self.n), dtype=torch.float64, device="cuda")
        st = torch.empty(P, dtype=torch.int32, device="cuda")
        it = torch.empty(P, dtype=torch.int32, device="cuda")
        sl = np.ascontiguousarray(slots, dtype=np.int32)
        _lib.check(self.lib.bte_engine_collect(self.h, P, sl.ctypes.data_as(C.POINTER(C.c_int32)), _lib.ptr(f),
                                               _lib.ptr(st), _lib.ptr(it), self._s()), "bte_engine_collect")
        n0, E = req._dev
        q = {k: torch.empty(P, dtype=torch.float64, device="cuda") for k in ("energy", "mobility", "diffusion")}
        rates = torch.empty((self.n_proc, P), dtype=torch.float64, device="cuda")
        _lib.check(self.lib.bte_qoi(self.grid, P, _lib.ptr(f), _lib.ptr(n0), _lib.ptr(E), 1, _lib.ptr(q["energy"]),
                                    _lib.ptr(q["mobility"]), _lib.ptr(q["diffusion"]), _lib.ptr(rates), self._s()),
                   "bte_qoi")
        self.stream.synchronize()
        req.ff = f.t().contiguous().cpu().numpy()
        req.qoi = {k: v.cpu().numpy() for k, v in q.items()}
        req.qoi["rates"] = rates.cpu().numpy()
        req.qoi["status"] = st.cpu().numpy()
        req.qoi["iters"] = it.cpu().numpy()
        del req._dev

    def close(self):
        if self.h:
            self.lib.bte_engine_destroy(self.h)
            self.h = None


class _Worker:
    def __init__(self, key, backend):
        self.key = key
        self.backend = backend
        self.queue = collections.deque()
        self.running = 0            # points of admitted, unfinished requests
        self.owner = {}             # slot -> request
        self.pending = {}           # request id -> points still running
        self.slots = {}             # request id -> its slots
        self.admitting = []         # requests taken from the queue, not yet in the engine
        self.dead = None            # the error that stopped the worker
        self.thread = None


class BteServer:
    """Serve `SolveRequest`s on a fixed set of grids with continuous batching.

    grids: list of (n_sp, l_max); every grid is assembled once (with e-e operators) from
    `lxcat_file` and stays resident. hbm_budget_bytes bounds the device memory of the points
    admitted at any time (a request larger than the whole budget is admitted alone).
    `backend_factory(key)` may replace the CUDA engine (used by host-only tests). refine and
    krylov are the mixed form's refinement options (bte_solve_opts: FP64 refinement passes;
    GMRES on the FP32 factors for stalled points, 0 = bordered sizes above 512, -1 = never).
    autotune (mixed form): each grid's FP32 factorization kernel is the one
    boltzmann_gb300.autotune measured fastest for its bordered size.
    """

    def __init__(self, lxcat_file, grids, precision="mixed", hbm_budget_bytes=8 << 30, capacity=1024,
                 fp64_capacity=64, atol=1e-20, rtol=1e-14, max_iter=100, alpha_min=1e-16, alpha_rho=0.5,
                 line_search_c=1e-4, refine=4, ev_max=80.0, Te=4.0, device=0, backend_factory=None, krylov=0,
                 autotune=True):
        self.budget = int(hbm_budget_bytes)
        self.used = 0
        self.peak_used = 0
        self._cv = threading.Condition()
        self._stop = False
        self._rid = 0
        self.errors = []
        self.device = device
        keys = [(int(a), int(b)) for a, b in grids]
        self.keys = keys
        self._workers = {}
        self._solver = None
        if backend_factory is None:
            import torch
            from .bte_0d3v_batched import bte_0d3v_batched, vspace_grid_extension
            torch.cuda.set_device(device)
            args = types.SimpleNamespace(threads=1, sp_order=3, spline_qpts=5, ee_collisions=1, verbose=0,
                                         use_gpu=1, Efreq=0.0, dt=1e-3, cycles=1, solver_type="steady-state",
                                         l_max=max(k[1] for k in keys), Nr=max(k[0] for k in keys) - 1, n_pts=1,
                                         precision=precision)
            s = bte_0d3v_batched(args, np.full(len(keys), float(ev_max)), np.full(len(keys), float(Te)),
                                 np.array([k[0] - 1 for k in keys]), [[[l, 0] for l in range(k[1] + 1)] for k in keys],
                                 len(keys), [lxcat_file] * len(keys))
            s._dev_id = device
            for i in range(len(keys)):
                s.assemble_operators(i, vspace_ext=vspace_grid_extension.NONE)
            self._solver = s
            opts = _lib.SolveOpts(atol=float(atol), rtol=float(rtol), max_iter=int(max_iter),
                                  alpha_min=float(alpha_min), alpha_rho=float(alpha_rho),
                                  line_search_c=float(line_search_c), ee=1,
                                  precision=_lib.PREC_MIXED if precision == "mixed" else _lib.PREC_FP64,
                                  refine=int(refine), krylov=int(krylov))
            for i, k in enumerate(keys):
                o = opts
                if precision == "mixed" and autotune:
                    from . import autotune as at
                    o = _lib.SolveOpts.from_buffer_copy(opts)
                    o.lu_kernel = at.lu_kernel_for(s._grid_info[i]["n"] + 1, device=device)
                be = EngineBackend(s._grid[i], s._grid_info[i], capacity, fp64_capacity, o, device)
                self._workers[k] = _Worker(k, be)
        else:
            for k in keys:
                self._workers[k] = _Worker(k, backend_factory(k))
        for w in self._workers.values():
            w.thread = threading.Thread(target=self._run, args=(w,), daemon=True, name="bte-serve-%d-%d" % w.key)
            w.thread.start()

    # ------------------------------------------------------------------ client side
    def submit(self, req: SolveRequest) -> SolveRequest:
        key = (int(req.n_sp), int(req.l_max))
        if key not in self._workers:
            raise ValueError("no grid (n_sp=%d, l_max=%d) on this server" % key)
        if req.P < 1 or req.P > self._workers[key].backend.capacity:
            raise ValueError("request size %d outside [1, %d]" % (req.P, self._workers[key].backend.capacity))
        with self._cv:
            if self._stop:
                raise RuntimeError("server is closed")
            if self._workers[key].dead:
                raise RuntimeError("grid %s failed: %s" % (key, self._workers[key].dead))
            req.rid = self._rid
            self._rid += 1
            req.t_submit = time.perf_counter()
            self._workers[key].queue.append(req)
            self._cv.notify_all()
        return req

    def cancel(self, req: SolveRequest) -> bool:
        """Withdraw a request that is still queued: it completes at once with error "cancelled"
        and holds no slots or budget. A request already admitted runs to the end (its points
        share the engine's batched iterations); the call then returns False."""
        key = (int(req.n_sp), int(req.l_max))
        with self._cv:
            w = self._workers.get(key)
            idx = None if w is None else next((i for i, r in enumerate(w.queue) if r is req), None)
            if idx is None:
                return False
            del w.queue[idx]
            req.error = "cancelled"
            req.t_done = time.perf_counter()
            self._cv.notify_all()
        req.done.set()
        return True

    def close(self):
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        for w in self._workers.values():
            if w.thread is not None:
                w.thread.join()
        for w in self._workers.values():
            close = getattr(w.backend, "close", None)
            if close:
                close()
        self._workers = {}

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------------ worker side
    def _admissible(self, w, req, free):
        need = req.P * w.backend.bytes_per_slot
        if req.P > free:
            return False
        return self.used + need <= self.budget or self.used == 0

    def _run(self, w: _Worker):
        be = w.backend
        stream = None
        try:
            if hasattr(be, "torch"):
                be.torch.cuda.set_device(be.device)
                stream = be.torch.cuda.Stream()
                be.bind(stream)
            ctx = be.torch.cuda.stream(stream) if stream is not None else _null_ctx()
            with ctx:
                self._loop(w)
        except Exception as e:  # surface worker failures to waiting clients
            with self._cv:
                w.dead = repr(e)
                self.errors.append("%s: %r" % (w.key, e))
                # requests admitted on this grid (in admission or owning slots) give their HBM
                # reservation back, each once, so that other grids' requests are not held back
                held = {id(r): r for r in w.admitting}
                held.update({id(r): r for r in w.owner.values()})
                for r in held.values():
                    self.used -= int(r.P * be.bytes_per_slot)
                w.admitting, w.running = [], 0
                w.owner.clear()
                for r in list(w.queue) + list(held.values()):
                    r.error = repr(e)
                    r.done.set()
                w.queue.clear()
                self._cv.notify_all()

    def _loop(self, w: _Worker):
        be = w.backend
        while True:
            admitted = []
            with self._cv:
                while not self._stop and not w.queue and w.running == 0:
                    self._cv.wait()
                if self._stop and w.running == 0:
                    return
                free = be.free_slots()
                while w.queue and self._admissible(w, w.queue[0], free):
                    r = w.queue.popleft()
                    free -= r.P
                    self.used += int(r.P * be.bytes_per_slot)
                    self.peak_used = max(self.peak_used, self.used)
                    admitted.append(r)
                if not admitted and w.running == 0:
                    # the head request waits for budget held by other grids
                    self._cv.wait(timeout=0.05)
                    continue
            w.admitting = admitted
            for r in admitted:
                slots = be.admit(r)
                r.t_admit = time.perf_counter()
                w.slots[r.rid] = slots
                w.pending[r.rid] = len(slots)
                for s in slots:
                    w.owner[int(s)] = r
                w.running += r.P
            w.admitting = []
            if w.running == 0:
                continue
            for s in be.step():
                r = w.owner.pop(int(s))
                w.pending[r.rid] -= 1
                if w.pending[r.rid] == 0:
                    self._finish(w, r)

    def _finish(self, w: _Worker, r: SolveRequest):
        be = w.backend
        slots = w.slots.pop(r.rid)
        del w.pending[r.rid]
        be.collect(r, slots)
        r.t_done = time.perf_counter()
        w.running -= r.P
        with self._cv:
            self.used -= int(r.P * be.bytes_per_slot)
            self._cv.notify_all()
        r.done.set()


class _null_ctx:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def wait_all(reqs, timeout=None):
    """Block until every request is done; raise if one failed."""
    t_end = None if timeout is None else time.perf_counter() + timeout
    for r in reqs:
        left = None if t_end is None else max(0.0, t_end - time.perf_counter())
        if not r.done.wait(left):
            raise TimeoutError("request %d not done" % r.rid)
        if r.error:
            raise RuntimeError("request %d failed: %s" % (r.rid, r.error))


def latency_summary(reqs):
    lat = np.array([r.latency for r in reqs]) * 1e3
    pts = sum(r.P for r in reqs)
    t0 = min(r.t_submit for r in reqs)
    t1 = max(r.t_done for r in reqs)
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "requests": len(reqs), "points": int(pts),
            "solves_per_s": pts / (t1 - t0) if t1 > t0 else None, "wall_s": t1 - t0}
