"""Ensemble batch: every scenario bit-exact with its standalone plain run."""
import numpy as np
import pytest

from oracle import oracle
from sagesim_gb300 import Engine, SageSimError, graphs
from sagesim_gb300.batch import Batch

pytestmark = pytest.mark.gpu


def make_scenarios(count, seed, nmin=1000, nmax=30000, variant_lids=False):
    rng = np.random.default_rng(seed)
    out = []
    for s in range(count):
        n = int(10 ** rng.uniform(np.log10(nmin), np.log10(nmax)))
        kind = s % 3
        if kind == 0:
            off, idx = graphs.erdos_renyi(n, 8.0 / (n - 1), 1000 + s)
        elif kind == 1:
            off, idx = graphs.barabasi_albert(n, int(rng.integers(3, 7)), 1000 + s)
        else:
            off, idx = graphs.watts_strogatz(n, int(rng.choice([6, 8, 10, 12])), 0.1, 1000 + s)
        st = np.ones(n, dtype=np.int32)
        st[rng.choice(n, max(1, int(0.005 * n)), replace=False)] = 2
        lids = None
        if variant_lids and s % 4 == 1:
            lids = rng.permutation(n).astype(np.int64) + 17
        out.append(dict(offsets=off, indices=idx, state=st, seed=int(rng.integers(0, 2**31)),
                        beta=float(rng.uniform(0.01, 0.1)), gamma=float(rng.uniform(0.05, 0.2)),
                        horizon=int(rng.integers(20, 61)), lids=lids))
    return out


def standalone(sc, variant, ticks, symmetric=True):
    with Engine() as e:
        e.set_graph(sc["offsets"], sc["indices"], symmetric=symmetric)
        if sc.get("lids") is not None:
            e.set_logical_ids(sc["lids"])
        e.set_seed(sc["seed"])
        p = e.add_property("state", np.int32, init=sc["state"])
        e.add_sir(p, sc["beta"], sc["gamma"], variant=variant)
        e.run(0, ticks, stats=False)
        return e.get_property(p)


@pytest.mark.parametrize("strategy", ["count", "pull"])
@pytest.mark.parametrize("variant", ["A", "B"])
def test_batch_scenarios_match_standalone(strategy, variant):
    scs = make_scenarios(24, 5, variant_lids=True)
    with Batch() as b:
        sids = [b.add_scenario(variant=variant, **sc) for sc in scs]
        b.commit()
        b.set_tune(strategy=strategy)
        for _ in range(3):  # 3 x 25 ticks: every horizon (<= 60) is reached
            b.run(25, use_graph=True)
        b.synchronize()
        for sid, sc in zip(sids, scs):
            assert b.tick(sid) == sc["horizon"]
            want = standalone(sc, variant, sc["horizon"])
            assert np.array_equal(b.get_state(sid), want), "scenario %d" % sid


@pytest.mark.parametrize("flavours", [(48, 0, 48 | 64), (0, 48 | 128, 4), (56, 5, 49), (16, 0, 16), (48 | 256 | 4, 0, 48 | 256),
                                      (6, 48 | 256 | 6, 2), (48 | 256 | 512, 512, 4), (512, 48, 48 | 256 | 512 | 6)])
def test_batch_count_flavours_switch_between_runs(flavours):
    """Class bytes are kept by every count-strategy kernel and the activity bits
    are rebuilt at the start of every run, so the class sweep can take over from
    (or hand over to) the other count-step flavours between runs; every scenario
    still equals its standalone run."""
    scs = make_scenarios(16, 21, variant_lids=True)
    with Batch() as b:
        sids = [b.add_scenario(variant="B", **sc) for sc in scs]
        b.commit()
        for fl in flavours:
            b.set_tune(strategy="count", count_flavour=fl)
            b.run(25, use_graph=True)
        b.synchronize()
        for sid, sc in zip(sids, scs):
            assert np.array_equal(b.get_state(sid), standalone(sc, "B", sc["horizon"])), "scenario %d" % sid


def test_batch_matches_oracle_and_tuner_keeps_results():
    scs = make_scenarios(12, 9)
    with Batch() as b:
        sids = [b.add_scenario(variant="B", **sc) for sc in scs]
        b.commit()
        best = b.tune(4)
        assert best["strategy"] in ("count", "pull") and best["us_per_tick"] > 0
        b.run(60)
        b.synchronize()
        for sid, sc in zip(sids, scs):
            ref, _, _ = oracle.sir_run(2, sc["offsets"], sc["indices"], sc["state"], sc["seed"], 0,
                                       sc["horizon"], sc["beta"], sc["gamma"])
            assert np.array_equal(b.get_state(sid), ref), sid


def test_batch_directed_scenario_uses_transpose():
    rng = np.random.default_rng(3)
    n = 4000
    deg = rng.integers(0, 10, size=n)
    off = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
    idx = rng.integers(0, n, size=int(off[-1])).astype(np.int32)
    st = np.ones(n, dtype=np.int32)
    st[:40] = 2
    sc = dict(offsets=off, indices=idx, state=st, seed=5, beta=0.2, gamma=0.1, horizon=30)
    with Batch() as b:
        sid = b.add_scenario(variant="B", symmetric=False, **sc)
        sid2 = b.add_scenario(variant="B", **make_scenarios(1, 4)[0])
        b.commit()
        b.run(30)
        b.synchronize()
        assert np.array_equal(b.get_state(sid), standalone(sc, "B", 30, symmetric=False))
        assert b.tick(sid2) > 0


def test_batch_errors():
    sc = make_scenarios(1, 1)[0]
    with Batch() as b:
        b.add_scenario(variant="B", **sc)
        with pytest.raises(SageSimError):
            b.add_scenario(variant="A", **sc)
        bad = dict(sc)
        bad["indices"] = sc["indices"].copy()
        bad["indices"][0] = 10**8
        with pytest.raises(SageSimError, match="BAD_CSR"):
            b.add_scenario(variant="B", **bad)
        b.commit()
        with pytest.raises(SageSimError):
            b.add_scenario(variant="B", **sc)


def test_ensemble_members_up_to_a_million_agents_match_oracle():
    """Members of the 512-scenario ensemble's size range, the largest at 10^6
    agents, advanced together for its 365 ticks with the default tuned launch
    configuration: each equals the oracle (SIR-B, own seed and parameters)."""
    specs = [("ba", 1_000_000, 5, 31), ("ws", 600_000, 10, 0.1, 32), ("er", 400_000, 8.0 / 399_999, 33),
             ("ba", 3_000, 3, 34), ("er", 1_000, 8.0 / 999, 35)]
    rng = np.random.default_rng(36)
    scs = []
    for spec in specs:
        off, idx = graphs.generate(spec)
        n = off.size - 1
        st = np.ones(n, dtype=np.int32)
        st[rng.choice(n, max(1, int(0.005 * n)), replace=False)] = 2
        scs.append(dict(offsets=off, indices=idx, state=st, seed=int(rng.integers(0, 2**31)),
                        beta=float(rng.uniform(0.01, 0.1)), gamma=float(rng.uniform(0.05, 0.2)), horizon=365))
    with Batch() as b:
        sids = [b.add_scenario(variant="B", **sc) for sc in scs]
        b.commit()
        b.snapshot()
        b.tune(2)
        b.restore()
        b.run(365)
        b.synchronize()
        for sid, sc in zip(sids, scs):
            ref, _, _ = oracle.sir_run(2, sc["offsets"], sc["indices"], sc["state"], sc["seed"], 0, 365,
                                       sc["beta"], sc["gamma"])
            assert np.array_equal(b.get_state(sid), ref), sid
