"""The request loop (lc2_server_*) on the CPU: requests with a host objective
run the full scheduler (admission by budget, worker threads, latency
accounting) without a GPU. Each result equals the same registration run
alone; the budget and the active-request limit hold at every moment."""
import threading
import time

import numpy as np
import pytest

from lc2registration_gb300 import capi
from lc2registration_gb300.geometry import Geometry


def _toy(target_params, center, delay_s=0.0, probe=None):
    target = capi.params_to_matrix("2D", target_params, center).reshape(9)[:6]
    w = np.array([30, 30, 0.3, 30, 30, 0.3])

    def lc2(M):
        if probe is not None:
            probe()
        if delay_s:
            time.sleep(delay_s)
        d = M.reshape(-1, 9)[:, :6] - target
        return np.exp(-((d * w) ** 2).sum(axis=1) * 0.1)
    return lc2


def _cfg(side):
    g = Geometry((side, side, 1), (1, 1, 1), (0, 0, 0))
    return capi.make_config("2D", g, g, (1.0, 1.0), 3)


REG = dict(initial=[0, 0, 0, 1, 1, 0], lower=[-5, -5, -8, 0.9, 0.9, -0.05],
           upper=[5, 5, 8, 1.1, 1.1, 0.05], center=(8.0, 8.0), direct_entries=["translation"],
           direct_maxeval=30, rounds=[(["translation", "rotation"], 1e-5)])


def test_results_equal_alone_and_in_the_mix():
    rng = np.random.default_rng(0)
    targets = [[*rng.uniform(-3, 3, 2), rng.uniform(-5, 5), 1, 1, 0] for _ in range(12)]
    alone = [capi.register(None, mode="2D", lc2_of_matrices=_toy(t, (8.0, 8.0)), **REG)
             for t in targets]
    srv = capi.Server(budget_bytes=1 << 40, max_active=4)
    tickets = []
    for t in targets:
        tickets.append(srv.submit(_cfg(64), lc2_of_matrices=_toy(t, (8.0, 8.0), 0.001), **REG))
        time.sleep(rng.exponential(0.002))     # Poisson-like arrivals
    res = [srv.poll(t) for t in tickets]
    for a, r in zip(alone, res):
        assert r["status"] == 0
        np.testing.assert_array_equal(r["params"][:6], a["params"])
        assert r["lc2"] == a["lc2"] and r["evaluations"] == a["evaluations"]
        assert r["total_ms"] >= r["run_ms"] > 0 and r["queue_ms"] >= 0
    st = srv.stats()
    assert st["completed"] == 12 and st["failed"] == 0
    assert 0 < st["p50_ms"] <= st["p95_ms"] <= st["p99_ms"]
    assert st["peak_active"] <= 4
    srv.close()


def test_budget_and_concurrency_limits():
    held, peak = capi.context_bytes(_cfg(128))
    assert peak >= held > 128 * 128 * 4
    budget = int(peak * 2.5)                  # room for two at a time
    srv = capi.Server(budget_bytes=budget, max_active=8)
    lock = threading.Lock()
    running = {"now": 0, "max": 0}

    def obj(M, base=_toy([1, 1, 0, 1, 1, 0], (8.0, 8.0), 0.002)):
        with lock:
            running["now"] += 1
            running["max"] = max(running["max"], running["now"])
        try:
            return base(M)
        finally:
            with lock:
                running["now"] -= 1

    tickets = [srv.submit(_cfg(128), lc2_of_matrices=obj, **REG) for _ in range(6)]
    admissions = [srv.poll(t)["admission"] for t in tickets]
    st = srv.stats()
    assert st["peak_bytes"] <= budget
    assert st["peak_active"] == 2 and running["max"] <= 2
    assert admissions == sorted(admissions)  # strict arrival order
    srv.close()


def test_oversized_request_rejected_and_errors_reported():
    held, peak = capi.context_bytes(_cfg(64))
    srv = capi.Server(budget_bytes=peak - 1, max_active=2)
    with pytest.raises(capi.LC2Error, match="OUT_OF_MEMORY"):
        srv.submit(_cfg(64), lc2_of_matrices=_toy([0] * 6, (8.0, 8.0)), **REG)
    srv.close()
    srv = capi.Server(budget_bytes=1 << 40, max_active=2)

    def bad(M):
        raise ValueError("objective failed")
    t = srv.submit(_cfg(64), lc2_of_matrices=bad, **REG)
    with pytest.raises(ValueError, match="objective failed"):
        srv.poll(t)
    assert srv.stats()["failed"] == 1
    with pytest.raises(capi.LC2Error, match="unknown"):
        srv.poll(t)
    # a request without images and without a host objective is refused
    with pytest.raises(capi.LC2Error, match="without images"):
        srv.submit(_cfg(64), **REG)
    assert srv.drain(1000)
    srv.close()


def test_poll_timeout_and_drain():
    srv = capi.Server(budget_bytes=1 << 40, max_active=1)
    slow = _toy([1, 0, 0, 1, 1, 0], (8.0, 8.0), 0.02)
    t1 = srv.submit(_cfg(32), lc2_of_matrices=slow, **REG)
    t2 = srv.submit(_cfg(32), lc2_of_matrices=slow, **REG)
    assert srv.poll(t2, wait_ms=0) is None     # still queued behind t1
    assert not srv.drain(0)
    assert srv.drain(-1)
    r1, r2 = srv.poll(t1), srv.poll(t2)
    assert r1["admission"] == 0 and r2["admission"] == 1
    assert r2["queue_ms"] >= r1["run_ms"] * 0.5
    srv.close()


def test_stack_request_validation():
    import ctypes
    srv = capi.Server(budget_bytes=1 << 40, max_active=1)
    req = capi.lc2_stack_request()
    t = ctypes.c_longlong()
    assert srv._lib.lc2_server_submit_stack(srv._h, ctypes.byref(req), ctypes.byref(t)) == 1
    srv.close()
