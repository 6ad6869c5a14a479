"""Serving loop: continuous batching of independent requests.  A request's
result is the same alone and in a mix of others that arrive while it runs,
and the same as one uninterrupted run of the plain path; the trace driver's
host logic is tested without a GPU."""
import numpy as np
import pytest

from dmdgb import abi, systems
from dmdgb.serving import Server, TraceResult, poisson_arrivals
from helpers import dense_system


def test_poisson_arrivals_statistics():
    a = poisson_arrivals(20.0, 50.0, seed=3)
    assert np.all(np.diff(a) > 0) and a[0] >= 0 and a[-1] < 50.0
    assert abs(len(a) - 1000) < 4 * np.sqrt(1000)
    gaps = np.diff(a)
    assert abs(gaps.mean() - 0.05) < 0.01


def test_trace_summary():
    r = TraceResult(latencies=[1.0, 2.0, 3.0, 4.0], events=1000, wall=2.0)
    s = r.summary()
    assert s["p50_s"] == 2.5 and s["events_per_s"] == 500.0 and s["requests"] == 4


def _req(k):
    return systems.generate(systems.serving_request(k, seed=9))


@pytest.mark.gpu
def test_same_alone_and_in_mix(built):
    target = dense_system(seed=31)
    n = 30000
    with Server(max_slots=8, chunk_events=7000) as srv:
        rid = srv.submit(target, n)
        while srv.status(rid)["state"] != abi.REQ_DONE:
            srv.step()
        alone = srv.result(rid)
    with Server(max_slots=8, chunk_events=7000) as srv:
        others = [_req(k) for k in range(4)]
        ids = [srv.submit(others[0], 20000), srv.submit(others[1], 50000)]
        srv.step()                       # the first two are running
        rid = srv.submit(target, n)      # arrives while others are on the GPU
        srv.step()
        ids += [srv.submit(others[2], 9000), srv.submit(others[3], 40000)]
        while any(srv.status(i)["state"] not in (abi.REQ_DONE, abi.REQ_FAILED) for i in ids + [rid]):
            srv.step()
        mixed = srv.result(rid)
        assert all(srv.status(i)["state"] == abi.REQ_DONE for i in ids)
    for k in ("x", "y", "z", "vx", "vy", "vz", "bptnr", "identity"):
        assert np.array_equal(alone[k], mixed[k]), k
    assert alone["coll"] == mixed["coll"] == n
    for k in ("e_total", "temperature", "rg", "e2e"):
        assert alone["diag"][k] == mixed["diag"][k], k
    # and equal to one uninterrupted run of the plain path
    from dmdgb.engine import Engine
    with Engine(target) as eng:
        eng.run(n)
        st = eng.state()
    for k in ("x", "y", "z", "vx", "vy", "vz", "bptnr", "identity"):
        assert np.array_equal(alone[k], st[k]), k


@pytest.mark.gpu
def test_admission_by_memory(built):
    """With a device-memory budget for about two requests, the others wait
    in the queue and are admitted as the first ones finish."""
    reqs = [dense_system(seed=40 + k) for k in range(5)]
    with Server(max_slots=16, chunk_events=5000) as srv:
        ids = [srv.submit(r, 8000) for r in reqs]
        srv.step()                       # admits all five
        need = srv.stats()["bytes_used"] / 5
    with Server(max_slots=16, chunk_events=5000, hbm_budget=int(2.5 * need)) as srv:
        ids = [srv.submit(r, 8000) for r in reqs]
        srv.step()
        s = srv.stats()
        assert s["active"] == 2 and s["waiting"] == 3
        while any(srv.status(i)["state"] != abi.REQ_DONE for i in ids):
            srv.step()
        assert srv.stats()["bytes_used"] == 0
