"""Graph setup on the GPU (sg_set_graph_id_edges): agent ids mapped to buffer
indices through the HBM hash table, CSR rows built by sorting, compared with
the host-side CSR builders; refusals of repeated and unknown ids."""
import numpy as np
import pytest

from oracle import oracle
from sagesim_gb300 import Engine, SageSimError, graphs

pytestmark = pytest.mark.gpu


def _host_csr(n, s, d, symmetric, ordered):
    rows = [[] for _ in range(n)]
    seen = [set() for _ in range(n)]
    pairs = []
    for a, b in zip(s, d):
        pairs.append((a, b))
        if symmetric:
            pairs.append((b, a))
    for a, b in pairs:
        if b not in seen[a]:
            seen[a].add(b)
            rows[a].append(b)
    if not ordered:
        rows = [sorted(r) for r in rows]
    off = np.zeros(n + 1, dtype=np.int32)
    off[1:] = np.cumsum([len(r) for r in rows])
    idx = np.array([x for r in rows for x in r], dtype=np.int32)
    return off, idx


@pytest.mark.parametrize("symmetric", [True, False])
@pytest.mark.parametrize("ordered", [False, True])
def test_id_edges_match_host_builder(symmetric, ordered):
    rng = np.random.default_rng(4)
    n, m = 3000, 12000
    ids = rng.choice(2**40, size=n, replace=False).astype(np.int64) - 2**39  # sparse, negative too
    ia, ib = rng.integers(0, n, m), rng.integers(0, n, m)
    ia[:50], ib[:50] = ia[50:100], ib[50:100]  # repeated edges
    with Engine() as e:
        e.set_graph_from_ids(ids, ids[ia], ids[ib], symmetric=symmetric, ordered=ordered)
        off, idx = e.get_graph()
    woff, widx = _host_csr(n, ia.tolist(), ib.tolist(), symmetric, ordered)
    assert np.array_equal(off, woff)
    assert np.array_equal(idx, widx)


def test_large_graph_matches_generator_and_runs_sir():
    """A 10^6-agent BA graph given as an id edge list (ids = a permutation of
    0..n-1 times 7): the GPU build equals the generator's sorted CSR mapped
    through the same ids, and SIR on it matches the oracle."""
    n = 1_000_000
    off, idx = graphs.barabasi_albert(n, 4, 9)
    src = np.repeat(np.arange(n), np.diff(off))
    keep = src < idx  # each undirected edge once
    a, b = src[keep], idx[keep]
    perm = np.random.default_rng(9).permutation(n)
    ids = perm.astype(np.int64) * 7
    st0 = np.full(n, 1, dtype=np.int32)
    st0[graphs.initial_infected(n, 0.001, 9)] = 2
    with Engine() as e:
        e.set_graph_from_ids(ids, ids[a], ids[b], symmetric=True)
        goff, gidx = e.get_graph()
        assert np.array_equal(goff, off)
        rows_ok = all(np.array_equal(np.sort(idx[off[i]:off[i + 1]]), gidx[goff[i]:goff[i + 1]])
                      for i in range(0, n, 9973))
        assert rows_ok
        p = e.add_property("state", np.int32, init=st0)
        e.set_seed(9)
        e.add_sir(p, 0.05, 0.1, variant="B", strategy="count")
        e.run(0, 15, stats=False)
        got = e.get_property(p)
    ref, _, _ = oracle.sir_run(2, goff, gidx, st0, 9, 0, 15, 0.05, 0.1)
    assert np.array_equal(got, ref)


def test_repeated_and_unknown_ids_are_refused():
    with Engine() as e:
        with pytest.raises(SageSimError, match="twice"):
            e.set_graph_from_ids([5, 6, 5], [5], [6])
        with pytest.raises(SageSimError, match="not in the id list"):
            e.set_graph_from_ids([5, 6, 7], [5, 9], [6, 7])
        e.set_graph_from_ids([5, 6, 7], [], [])
        off, idx = e.get_graph()
        assert off.tolist() == [0, 0, 0, 0] and idx.size == 0


def test_model_set_edges_matches_reference_fixtures():
    """NetworkSpace.set_edges (GPU build) reproduces the reference trajectories:
    the 10^4-agent ER SIR-B fixture (undirected, sorted rows) and the ordered WS
    opinion fixture (directed edges in row order, first-connection order kept)."""
    import os

    from sagesim_gb300 import Breed, Model, NetworkSpace, OpinionStep, SIRStep

    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    d = np.load(os.path.join(gold, "er_c1.npz"))
    off, idx = d["offsets"], d["indices"]
    n = off.size - 1
    src = np.repeat(np.arange(n), np.diff(off))
    keep = src < idx
    m = Model(NetworkSpace())
    br = Breed("SIR")
    br.register_property("state", 1)
    br.register_step_func(SIRStep("B"), __file__, 0)
    m.register_breed(br)
    m.register_global_property("p_infection", 0.05)
    m.register_global_property("p_recovery", 0.1)
    m.set_seed(0)
    m.create_agents_bulk(br, n, state=d["state0"].astype(np.int32))
    m.get_space().set_edges(src[keep], idx[keep])
    m.setup()
    m.simulate(100)
    assert np.array_equal(m.get_property_array("state"), d["sir_b"][-1])

    d = np.load(os.path.join(gold, "opinion_ws.npz"))
    off, idx = d["offsets"], d["indices"]
    n = off.size - 1
    m = Model(NetworkSpace(ordered=True))
    br = Breed("Opinion")
    br.register_property("opinion", 0.0)
    br.register_property("weights", [0.0] * 8)
    br.register_step_func(OpinionStep(), __file__, 0)
    m.register_breed(br)
    m.register_global_property("noise_sigma", 0.01)
    m.set_seed(2)
    m.create_agents_bulk(br, n, opinion=d["opinion0"], weights=d["weights"])
    m.get_space().set_edges(np.repeat(np.arange(n), np.diff(off)), idx, directed=True)
    m.setup()
    m.simulate(int(d["ticks"][-1]))
    got, want = m.get_property_array("opinion"), d["history"][-1]
    rel = np.abs(got - want) / np.maximum(np.abs(want), 1e-30)
    assert ((rel <= 1e-6) | (np.abs(got - want) <= 1e-12)).all()
