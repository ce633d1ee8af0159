"""Host logic of the serving loop (admission by HBM footprint, continuous batching, request
bookkeeping) with a fake engine in place of the CUDA one: no GPU needed."""
import threading
import time

import numpy as np
import pytest

from boltzmann_gb300.serving import BteServer, SolveRequest, latency_summary, wait_all


class FakeEngine:
    """Each point finishes after a number of steps set by its E (1 + int(E) % 4); its result is
    a deterministic function of its own parameters, as a real per-point solve is."""

    def __init__(self, key, capacity=64, bytes_per_slot=1000, step_s=0.002, fail_on=None, fail_step=False):
        self.key = key
        self.capacity = capacity
        self.bytes_per_slot = bytes_per_slot
        self.step_s = step_s
        self.free = list(range(capacity))[::-1]
        self.left = {}
        self.points = {}
        self.fail_on = fail_on
        self.fail_step = fail_step
        self.steps = 0
        self.max_running = 0
        self.lock = threading.Lock()

    def free_slots(self):
        return len(self.free)

    def admit(self, req):
        if self.fail_on is not None and req.P == self.fail_on:
            raise RuntimeError("planted engine failure")
        assert req.P <= len(self.free)
        slots = np.array([self.free.pop() for _ in range(req.P)], dtype=np.int32)
        for i, s in enumerate(slots):
            self.left[int(s)] = 1 + int(req.E[i]) % 4
            self.points[int(s)] = (req.E[i], req.n0[i])
        self.max_running = max(self.max_running, len(self.left))
        return slots

    def step(self):
        time.sleep(self.step_s)
        if self.fail_step:
            raise RuntimeError("planted step failure")
        self.steps += 1
        done = []
        for s in list(self.left):
            self.left[s] -= 1
            if self.left[s] == 0:
                del self.left[s]
                done.append(s)
        return np.array(done, dtype=np.int32)

    def collect(self, req, slots):
        vals = np.array([self.points.pop(int(s)) for s in slots])
        req.ff = np.stack([vals[:, 0] * 2.0, vals[:, 1] + 1.0])
        req.qoi = {"status": np.zeros(len(slots), dtype=np.int32)}
        self.free.extend(int(s) for s in slots)


def make_req(rng, n_sp=64, l_max=1, P=None):
    P = int(rng.integers(1, 17)) if P is None else P
    return SolveRequest(n_sp=n_sp, l_max=l_max, n0=rng.uniform(1, 2, P), ne=np.zeros(P), Tg=np.full(P, 300.0),
                        E=rng.uniform(0, 100, P), ns_by_n0=np.ones((1, P)))


def test_all_requests_complete_with_their_own_results():
    rng = np.random.default_rng(0)
    engines = {}
    fac = lambda k: engines.setdefault(k, FakeEngine(k))
    with BteServer(None, [(64, 1), (96, 2)], backend_factory=fac) as srv:
        reqs = [srv.submit(make_req(rng, *(64, 1) if i % 2 else (96, 2))) for i in range(40)]
        wait_all(reqs, timeout=30)
    for r in reqs:
        assert np.array_equal(r.ff[0], r.E * 2.0) and np.array_equal(r.ff[1], r.n0 + 1.0)
        assert r.t_submit <= r.t_admit <= r.t_done
    s = latency_summary(reqs)
    assert s["requests"] == 40 and s["p99_ms"] >= s["p50_ms"] > 0


def test_hbm_budget_bounds_admitted_points():
    rng = np.random.default_rng(1)
    engines = {}
    fac = lambda k: engines.setdefault(k, FakeEngine(k, capacity=64, bytes_per_slot=1000))
    with BteServer(None, [(64, 1), (96, 2)], hbm_budget_bytes=20_000, backend_factory=fac) as srv:
        reqs = [srv.submit(make_req(rng, *(64, 1) if i % 2 else (96, 2), P=8)) for i in range(30)]
        wait_all(reqs, timeout=30)
        assert srv.peak_used <= 20_000
        assert srv.used == 0
    assert sum(e.max_running for e in engines.values()) <= 2 * 20


def test_request_larger_than_budget_runs_alone():
    rng = np.random.default_rng(2)
    fac = lambda k: FakeEngine(k, capacity=64, bytes_per_slot=1000)
    with BteServer(None, [(64, 1)], hbm_budget_bytes=5_000, backend_factory=fac) as srv:
        r = srv.submit(make_req(rng, P=32))
        wait_all([r], timeout=10)
    assert r.ff.shape == (2, 32)


def test_continuous_batching_admits_while_others_run():
    """A request that arrives while a long one runs is admitted before the long one ends, and
    finishes first."""
    rng = np.random.default_rng(3)
    eng = FakeEngine((64, 1), step_s=0.01)
    with BteServer(None, [(64, 1)], backend_factory=lambda k: eng) as srv:
        long = make_req(rng, P=4)
        long.E[:] = 43.0          # 1 + 43 % 4 = 4 steps each
        r1 = srv.submit(long)
        time.sleep(0.015)
        short = make_req(rng, P=2)
        short.E[:] = 0.0          # 1 step
        r2 = srv.submit(short)
        wait_all([r1, r2], timeout=10)
    assert r2.t_admit < r1.t_done
    assert r2.t_done < r1.t_done
    assert eng.max_running == 6


def test_fifo_within_a_grid_when_slots_are_short():
    rng = np.random.default_rng(4)
    eng = FakeEngine((64, 1), capacity=8)
    with BteServer(None, [(64, 1)], backend_factory=lambda k: eng) as srv:
        reqs = [srv.submit(make_req(rng, P=6)) for _ in range(5)]
        wait_all(reqs, timeout=10)
    admits = [r.t_admit for r in reqs]
    assert admits == sorted(admits)


def test_bad_requests_and_engine_failure():
    rng = np.random.default_rng(5)
    with BteServer(None, [(64, 1)], backend_factory=lambda k: FakeEngine(k, capacity=16, fail_on=3)) as srv:
        with pytest.raises(ValueError):
            srv.submit(make_req(rng, n_sp=96, l_max=2))   # no such grid
        with pytest.raises(ValueError):
            srv.submit(make_req(rng, P=17))              # beyond the engine's slots
        bad = srv.submit(make_req(rng, P=3))
        with pytest.raises(RuntimeError, match="planted"):
            wait_all([bad], timeout=10)
        assert srv.errors
        with pytest.raises(RuntimeError, match="failed"):
            srv.submit(make_req(rng, P=2))               # the grid's worker has stopped


def test_cancel_a_queued_request():
    """A request still queued behind a full engine can be withdrawn: it completes at once with
    error "cancelled", never reaches the engine, and the requests behind it still run. A request
    already admitted cannot be withdrawn."""
    rng = np.random.default_rng(8)
    eng = {}

    def factory(k):
        eng[k] = FakeEngine(k, capacity=16, step_s=0.05)
        return eng[k]

    with BteServer(None, [(64, 1)], backend_factory=factory) as srv:
        big = make_req(rng, P=16)
        big.E = np.full(16, 3.5)                       # four engine steps
        srv.submit(big)
        t0 = time.perf_counter()
        while big.t_admit == 0.0 and time.perf_counter() - t0 < 5:
            time.sleep(0.005)
        a, b = srv.submit(make_req(rng, P=8)), srv.submit(make_req(rng, P=8))
        assert srv.cancel(a)
        assert a.done.is_set() and a.error == "cancelled" and a.ff is None
        assert not srv.cancel(big)                     # already admitted
        wait_all([big, b], timeout=10)
        assert big.error is None and b.error is None and b.ff is not None
        assert not srv.cancel(b)                       # finished
        assert srv.used == 0


def test_failed_grid_returns_its_hbm_reservation():
    """A grid whose engine fails in a step after admitting a request gives that request's HBM
    reservation back: a request on another grid that needs more than the budget left beside
    the failed request's footprint is still admitted and finishes."""
    rng = np.random.default_rng(9)

    def factory(k):
        return FakeEngine(k, capacity=32, bytes_per_slot=1000, step_s=0.02, fail_step=(k == (64, 1)))

    with BteServer(None, [(64, 1), (96, 2)], hbm_budget_bytes=20_000, backend_factory=factory) as srv:
        bad = srv.submit(make_req(rng, 64, 1, P=15))
        with pytest.raises(RuntimeError, match="planted step"):
            wait_all([bad], timeout=10)
        other = srv.submit(make_req(rng, 96, 2, P=10))
        wait_all([other], timeout=10)
        assert other.ff is not None and other.error is None
        assert srv.used == 0
