"""Serving with continuous batching: each request's result is the same alone
and in the mix, requests queue against the HBM budget and are admitted as
resident scenarios finish."""
import numpy as np
import pytest

from sagesim_gb300 import SageSimError
from sagesim_gb300.serve import Server, serve_stream

from test_batch_gpu import make_scenarios, standalone  # noqa: E402

pytestmark = pytest.mark.gpu


def requests(count, seed):
    out = []
    for sc in make_scenarios(count, seed, nmin=2000, nmax=60000):
        sc = dict(sc)
        sc.pop("lids")
        out.append(sc)
    return out


def test_served_results_equal_standalone_and_queueing_happens():
    reqs = requests(30, 11)
    from sagesim_gb300.batch import Batch  # noqa: F401  (same pool code)
    sizes = [r["offsets"].size - 1 for r in reqs]
    budget = int(sum(sorted(sizes)[-6:]) * 64)  # a handful resident at once
    rng = np.random.default_rng(4)
    arrivals = np.cumsum(rng.exponential(0.005, size=len(reqs)))
    with Server(budget_bytes=budget, agent_slots=2_000_000, edge_slots=40_000_000, variant="B") as srv:
        out = serve_stream(srv, reqs, arrivals, chunk=8)
        assert srv.counts()["done"] == len(reqs)
    assert (out["latency_s"] > 0).all()
    for i, r in enumerate(reqs):
        want = standalone(r, "B", r["horizon"])
        assert np.array_equal(out["results"][i], want), "request %d" % i


def test_request_over_budget_is_refused():
    reqs = requests(1, 12)
    n = reqs[0]["offsets"].size - 1
    with Server(budget_bytes=n * 4, agent_slots=1_000_000, edge_slots=10_000_000) as srv:
        with pytest.raises(SageSimError, match="BUDGET"):
            srv.submit(**reqs[0])


def test_poll_and_take_result():
    r = requests(1, 13)[0]
    with Server(budget_bytes=1 << 30, agent_slots=1_000_000, edge_slots=10_000_000) as srv:
        rid = srv.submit(**r)
        assert srv.poll(rid)[0] == 0  # queued
        srv.step(5)
        st, tk = srv.poll(rid)
        assert st == 1 and tk == 5
        while srv.poll(rid)[0] != 2:
            srv.step(16)
        got = srv.take_result(rid)
        assert np.array_equal(got, standalone(r, "B", r["horizon"]))
        with pytest.raises(SageSimError):
            srv.poll(rid)
