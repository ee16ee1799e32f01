"""The benchmark's own workload against the oracle, every tick.

10,000,000 agents on a Barabasi-Albert graph (m=4, seed 1, 8.0e7 CSR entries),
relabelled by the 64-way locality partition with logical id = original agent
id, 0.1 % infected, beta 0.03, gamma 0.07, per-infected-neighbour SIR, 200
ticks: exactly what bench.py times. Code that only runs at this size is
covered here: the hybrid count step switching between its loop form and the
class sweep at its natural threshold (at least 24 tiles per SM), hub rows of
thousands of entries through the scatter's row segments, the count-init
scatter from 10,000 infected agents and the L2 window on the counts.

Reference semantics: tests/test_simulation.py:24-43 and
sagesim/model.py:2306-2408 (the step reads tick-start values, writes land
after every agent has stepped); the oracle is pinned to the reference's own
pipeline by tests/test_oracle_golden.py.
"""
import numpy as np
import pytest

import bench
from oracle import oracle
from sagesim_gb300 import Engine

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def workload():
    off, idx, st0, lids = bench.build_workload()
    assert off.size - 1 == 10_000_000 and int(off[-1]) == 79_999_968
    final, stats, _ = oracle.sir_run(2, off, idx, st0, bench.SEED, 0, bench.TICKS, bench.BETA, bench.GAMMA,
                                     bench.CODES, lids=lids)
    return off, idx, st0, lids, final, stats


def _engine(off, idx, st0, lids, strategy):
    e = Engine()
    e.set_graph(off, idx, symmetric=True)
    e.set_logical_ids(lids)
    e.set_seed(bench.SEED)
    p = e.add_property("state", np.int32, init=st0)
    e.add_sir(p, bench.BETA, bench.GAMMA, variant="B", strategy=strategy, codes=bench.CODES)
    return e, p


@pytest.mark.parametrize("strategy", ["count", "frontier", "pull"])
def test_headline_final_state_and_tick_statistics(workload, strategy):
    off, idx, st0, lids, want, want_stats = workload
    e, p = _engine(off, idx, st0, lids, strategy)
    with e:
        stats, _ = e.run(0, bench.TICKS, stats=True)
        got = e.get_property(p)
        if strategy == "count":
            active = e.last_run_active(bench.TICKS)
            n = off.size - 1
            # the hybrid step gave some ticks to its loop form (every agent
            # processed) and the rest to the class sweep
            assert (active >= n).any() and (active < n).any()
    bad = np.flatnonzero((stats != want_stats).any(axis=1))
    assert bad.size == 0, "tick statistics differ from tick %d: %s vs %s" % (
        bad[0], stats[bad[0]], want_stats[bad[0]])
    assert np.array_equal(got, want), "%d agents differ" % int((got != want).sum())


def test_headline_count_strategy_every_tick(workload):
    """The default configuration's state after every one of the 200 ticks: the
    run of t ticks from the initial state (graph replay, no statistics, as the
    benchmark times it) equals the oracle after t ticks."""
    off, idx, st0, lids, want_final, _ = workload
    e, p = _engine(off, idx, st0, lids, "count")
    with e:
        e.snapshot()
        st = st0.copy()
        for t in range(1, bench.TICKS + 1):
            st, _, _ = oracle.sir_run(2, off, idx, st, bench.SEED, t - 1, 1, bench.BETA, bench.GAMMA, bench.CODES,
                                      lids=lids)
            e.restore()
            e.run_async(0, t, use_graph=True)
            got = e.get_property(p)
            assert np.array_equal(got, st), "tick %d: %d agents differ" % (t - 1, int((got != st).sum()))
    assert np.array_equal(st, want_final)
