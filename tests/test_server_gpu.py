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
        srv.set_tune()  # the defaults (class sweep + hybrid step) are accepted
        with pytest.raises(SageSimError):
            srv.set_tune(count_flavour=1024)
        rid = srv.submit(**r)
        assert srv.poll(rid) == (1, 0)  # room at once: placed on the device, running
        srv.step(5)
        st, tk = srv.poll(rid)
        assert st == 1 and tk == 5
        while srv.poll(rid)[0] != 2:
            srv.step(16)
        got = srv.take_result(rid)
        assert np.array_equal(got, standalone(r, "B", r["horizon"]))
        with pytest.raises(SageSimError):
            srv.poll(rid)


def est_bytes(r):
    """About the server's footprint of a request (22 B per agent slot, 4 B per
    CSR entry, the scatter's segment list of 2 nnz / 64 + 64 entries of 16 B,
    tile and segment tables)."""
    n, nnz = r["offsets"].size - 1, r["indices"].size
    return ((n + 32) & ~31) * 22 + nnz * 4 + (2 * nnz // 64 + 64) * 16 + ((n + 2047) // 2048 + 1) * 20 + 256


def test_bad_csr_is_refused_on_both_submission_paths():
    """Placed at once (CSR checked on the device) or queued behind a request
    that fills the budget (checked on the host): a bad CSR is SG_ERR_BAD_CSR,
    nothing of it stays, and later requests run as they would alone."""
    good, other = requests(2, 14)
    bad_index = dict(other, indices=other["indices"].copy())
    bad_index["indices"][-1] = other["offsets"].size - 1 + 5
    bad_order = dict(other, offsets=other["offsets"].copy())
    bad_order["offsets"][3] = bad_order["offsets"][4] + 1
    for placed_at_once in (True, False):
        budget = (1 << 30) if placed_at_once else est_bytes(good) + est_bytes(other) // 2
        with Server(budget_bytes=budget, agent_slots=1_000_000, edge_slots=10_000_000) as srv:
            if not placed_at_once:
                first = srv.submit(**good)
                assert srv.poll(first)[0] == 1
            for bad in (bad_index, bad_order):
                with pytest.raises(SageSimError, match="BAD_CSR"):
                    srv.submit(**bad)
            assert srv.counts()["queued"] == 0
            rid = srv.submit(**other)
            if not placed_at_once:
                assert srv.poll(rid)[0] == 0  # queued behind the first
            while srv.poll(rid)[0] != 2:
                srv.step(16)
            assert np.array_equal(srv.take_result(rid), standalone(other, "B", other["horizon"]))


def test_requests_with_logical_ids_alone_and_in_the_mix():
    """Requests relabelled for locality carry logical ids (the original agent
    ids, the key of every draw as in sagesim/model.py:656-667): served in a mix
    with plain requests, each result equals its standalone run, and mapped back
    through the relabelling it equals the oracle's run of the graph in its
    original order."""
    from oracle import oracle
    from sagesim_gb300 import graphs

    base = requests(12, 15)
    reqs, perms, originals = [], [], []
    for k, r in enumerate(base):
        if k % 2:
            off, idx = r["offsets"], r["indices"]
            n = off.size - 1
            perm, _ = graphs.partition_relabel(off, idx, 8, k)
            roff, ridx = graphs.permute_csr(off, idx, perm)
            rst = np.empty_like(r["state"])
            rst[perm] = r["state"]
            lids = np.empty(n, dtype=np.int64)
            lids[perm] = np.arange(n, dtype=np.int64)
            reqs.append(dict(r, offsets=roff, indices=ridx, state=rst, lids=lids))
            perms.append(perm)
        else:
            reqs.append(dict(r))
            perms.append(None)
        originals.append(r)
    sizes = [r["offsets"].size - 1 for r in reqs]
    budget = int(sum(sorted(sizes)[-5:]) * 64)  # a few resident at once: some requests queue
    arrivals = np.cumsum(np.random.default_rng(5).exponential(0.004, size=len(reqs)))
    with Server(budget_bytes=budget, agent_slots=2_000_000, edge_slots=40_000_000, variant="B") as srv:
        out = serve_stream(srv, reqs, arrivals, chunk=8)
    for i, r in enumerate(reqs):
        assert np.array_equal(out["results"][i], standalone(r, "B", r["horizon"])), "request %d" % i
        o = originals[i]
        want, _, _ = oracle.sir_run(2, o["offsets"], o["indices"], o["state"], o["seed"], 0, o["horizon"],
                                    o["beta"], o["gamma"])
        got = out["results"][i] if perms[i] is None else out["results"][i][perms[i]]
        assert np.array_equal(got, want), "request %d against the oracle" % i


def test_borrowed_requests_queue_without_host_copies():
    """Requests submitted with borrow=True: those that queue keep the caller's
    arrays (no host copy or host CSR pass) and are checked on the device when
    placed. Results equal the standalone runs; a borrowed request with a bad CSR
    that queued is refused at placement (status SG_REQ_FAILED, take_result
    raises SG_ERR_BAD_CSR) without disturbing the others."""
    from sagesim_gb300 import _native as N

    reqs = requests(10, 16)
    bad = dict(reqs[3], indices=reqs[3]["indices"].copy())
    bad["indices"][5] = bad["offsets"].size + 7  # outside [0, n)
    budget = est_bytes(reqs[0]) + 1  # one resident at a time: the rest queue
    with Server(budget_bytes=max(budget, max(est_bytes(r) for r in reqs) + 1), agent_slots=2_000_000,
                edge_slots=40_000_000) as srv:
        rids = [srv.submit(**r, borrow=True) for r in reqs]
        bad_rid = srv.submit(**bad, borrow=True)
        assert srv.poll(bad_rid)[0] == N.SG_REQ_QUEUED
        pending = set(rids)
        results = {}
        while pending or srv.poll(bad_rid)[0] == N.SG_REQ_QUEUED:
            srv.step(32)
            for rid in list(pending):
                if srv.poll(rid)[0] == N.SG_REQ_DONE:
                    results[rid] = srv.take_result(rid)
                    pending.discard(rid)
        assert srv.poll(bad_rid)[0] == N.SG_REQ_FAILED
        with pytest.raises(SageSimError, match="BAD_CSR"):
            srv.take_result(bad_rid)
    for rid, r in zip(rids, reqs):
        assert np.array_equal(results[rid], standalone(r, "B", r["horizon"])), rid
