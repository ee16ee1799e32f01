"""The CPU oracle against golden fixtures produced by the reference itself.

The fixtures come from tests/golden/make_golden.py, which runs the unmodified
SAGESim pipeline (codegen, fused kernel, Philox) on CPU; this pins the oracle
before it is trusted as the checker of the CUDA engine.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name))


def test_philox_uniform_bit_exact():
    d = json.load(open(os.path.join(GOLD, "philox_vectors.json")))
    v = np.array(d["uniform_k23"], dtype=np.int64)
    got = oracle.philox_k23(v[:, 0], v[:, 1], v[:, 2], v[:, 3])
    assert np.array_equal(got.astype(np.int64), v[:, 4])


def test_philox_normal_close():
    d = json.load(open(os.path.join(GOLD, "philox_vectors.json")))
    rows = d["normal"]
    a = np.array([r[:4] for r in rows], dtype=np.int64)
    want = np.array([r[4] for r in rows])
    got = oracle.rand_normal(a[:, 0], a[:, 1], a[:, 2], a[:, 3])
    # numpy's log/cos (reference run) vs libm's: a few ulp at most
    assert np.allclose(got, want, rtol=1e-13, atol=1e-13)


def test_threshold_equals_double_compare():
    rng = np.random.default_rng(0)
    ps = list(rng.random(200)) + [0.0, 1.0, 0.05, 0.1, 0.03, 0.07, 1e-9, 0.5, 2.0, -1.0,
                                   1.0 / 8388608.0, 3.0 / 8388608.0]
    ks = np.arange(0, 8388608, 997)
    for p in ps:
        K = oracle.threshold(p)
        assert np.array_equal(ks / 8388608.0 < p, ks < K), p


def chain_csr(n):
    src = np.concatenate([np.arange(n - 1), np.arange(1, n)])
    dst = np.concatenate([np.arange(1, n), np.arange(n - 1)])
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    off = np.zeros(n + 1, dtype=np.int32)
    np.add.at(off, src + 1, 1)
    return np.cumsum(off).astype(np.int32), dst.astype(np.int32)


@pytest.mark.parametrize("key,n,p,seed,ticks", [("det10", 10, (1.0, 1.0), 42, 5),
                                                 ("sto20_seed999", 20, (0.5, 0.3), 999, 10),
                                                 ("sto50_seed111", 50, (0.3, 0.2), 111, 20),
                                                 ("sto50_seed222", 50, (0.3, 0.2), 222, 20)])
def test_oracle_reference_chain(key, n, p, seed, ticks):
    """tests/test_simulation.py chain model: agent 0 infected, SIR-A step."""
    hist = load("chain.npz")[key]
    off, idx = chain_csr(n)
    st = np.ones(n, dtype=np.int32)
    st[0] = 2
    _, _, h = oracle.sir_run(1, off, idx, st, seed, 0, ticks, p[0], p[1], history=True)
    assert np.array_equal(h, hist)


def test_chain_known_answer():
    """The reference test's own assertion (tests/test_simulation.py:95-115)."""
    hist = load("chain.npz")["det10"]
    assert hist[-1].tolist() == [3, 3, 3, 3, 3, 2, 1, 1, 1, 1]


def undirected_csr(n, edges):
    """The reference test connects each DiGraph edge with connect_agents(a, b),
    whose default is undirected (sagesim/space.py:107-125)."""
    src = np.concatenate([edges[:, 0], edges[:, 1]])
    dst = np.concatenate([edges[:, 1], edges[:, 0]])
    key = np.unique(src.astype(np.int64) * n + dst)
    src, dst = key // n, key % n
    off = np.zeros(n + 1, dtype=np.int32)
    np.add.at(off, src + 1, 1)
    return np.cumsum(off).astype(np.int32), dst.astype(np.int32)


def test_oracle_hierarchy():
    """tests/test_double_buffer.py: SI (1 tick) and two-priority SIR (2 ticks), p=1."""
    d = load("hier.npz")
    off, idx = undirected_csr(111, d["edges"])
    st = np.ones(111, dtype=np.int32)
    st[0] = 2
    _, _, h = oracle.sir_run(1, off, idx, st, 0, 0, 1, 1.0, 0.0, history=True)
    assert np.array_equal(h, d["si_1tick"])
    # infection at priority 0 and recovery at priority 1 both read tick-start
    # state, so the pair is the one-step SIR with p_inf = p_rec = 1
    _, _, h = oracle.sir_run(1, off, idx, st, 0, 0, 2, 1.0, 1.0, history=True)
    assert np.array_equal(h, d["sir_2ticks"])
    assert (h[1][1:11] == 3).all() and (h[1][11:] == 2).all() and h[1][0] == 3


@pytest.mark.parametrize("variant,key", [(1, "sir_a"), (2, "sir_b")])
def test_oracle_er_c1(variant, key):
    d = load("er_c1.npz")
    st = d["state0"].astype(np.int32)
    _, _, h = oracle.sir_run(variant, d["offsets"], d["indices"], st, 0, 0, 100, 0.05, 0.1, history=True)
    ref = d[key]
    bad = np.argwhere(h != ref)
    assert bad.size == 0, "first mismatch (tick, agent) %s" % (bad[0],)


def test_oracle_breeds_and_logical_ids():
    """Two interleaved breeds (the reference sorts agents by breed) and explicit
    logical ids: RNG keys follow logical ids, not buffer positions."""
    d = load("ba_breeds.npz")
    n = d["breeds"].size
    lids = np.arange(n, dtype=np.int64)
    for a, l in d["lid_pairs"]:
        lids[a] = l
    st = d["state0"].astype(np.int32)
    _, _, h = oracle.sir_run(2, d["offsets"], d["indices"], st, 77, 0, 30, 0.08, 0.1, lids=lids,
                             history=True)
    assert np.array_equal(h, d["history"])


def test_oracle_opinion():
    """float32 opinion model, ordered neighbours: 1e-6 relative to the reference."""
    d = load("opinion_ws.npz")
    _, h = oracle.opinion_run(d["offsets"], d["indices"], d["weights"], d["opinion0"], 2, 0, 50, 0.01,
                              history=True)
    got = h[d["ticks"] - 1]
    want = d["history"]
    rel = np.abs(got - want) / np.maximum(np.abs(want), 1e-30)
    close = (rel <= 1e-6) | (np.abs(got - want) <= 1e-12)
    assert close.all(), "max rel %g" % rel[~close].max()
