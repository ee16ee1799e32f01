"""Edge cases of the SIR tick on the GPU against the oracle, for the pull
strategy and the count strategy's step forms (loop form, class sweep, hybrid):
graphs without edges, a single agent, everyone infected at start, the
deterministic beta = gamma = 1 case, and a star whose hub row spans many
scatter segments."""
import numpy as np
import pytest

from oracle import oracle
from sagesim_gb300 import Engine, graphs

pytestmark = pytest.mark.gpu

# (strategy, count_flavour): loop form; class sweep and hybrid forced onto small graphs
FORMS = [("pull", None), ("count", 0), ("count", 4), ("count", 48), ("count", 48 | 256 | 4)]


def _csr(n, a, b):
    a = np.asarray(a, dtype=np.int64)
    b = np.asarray(b, dtype=np.int64)
    src = np.concatenate([a, b])
    dst = np.concatenate([b, a])
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    off = np.zeros(n + 1, dtype=np.int32)
    np.add.at(off, src + 1, 1)
    return np.cumsum(off).astype(np.int32), dst.astype(np.int32)


def _run(off, idx, st0, variant, beta, gamma, ticks, strategy, flavour, seed=3):
    with Engine() as e:
        e.set_graph(off, idx, symmetric=True)
        e.set_seed(seed)
        p = e.add_property("state", np.int32, init=st0)
        e.add_sir(p, beta, gamma, variant=variant, strategy=strategy)
        if flavour is not None:
            e.set_tune(count_flavour=flavour)
        stats, _ = e.run(0, ticks, stats=True)
        return e.get_property(p), stats


def _check(off, idx, st0, variant, beta, gamma, ticks, strategy, flavour):
    got, stats = _run(off, idx, st0, variant, beta, gamma, ticks, strategy, flavour)
    ref, rstats, _ = oracle.sir_run(1 if variant == "A" else 2, off, idx, st0, 3, 0, ticks, beta, gamma)
    assert np.array_equal(got, ref)
    assert np.array_equal(stats, rstats)
    return got


@pytest.mark.parametrize("strategy,flavour", FORMS)
@pytest.mark.parametrize("variant", ["A", "B"])
def test_no_edges(strategy, flavour, variant):
    n = 5000
    off = np.zeros(n + 1, dtype=np.int32)
    idx = np.zeros(0, dtype=np.int32)
    st0 = np.full(n, 1, dtype=np.int32)
    st0[::7] = 2
    got = _check(off, idx, st0, variant, 0.5, 0.3, 12, strategy, flavour)
    assert not np.any((st0 == 1) & (got != 1))  # nobody can be infected


@pytest.mark.parametrize("strategy,flavour", FORMS)
def test_single_agent(strategy, flavour):
    off = np.zeros(2, dtype=np.int32)
    idx = np.zeros(0, dtype=np.int32)
    got = _check(off, idx, np.array([2], dtype=np.int32), "B", 0.9, 0.5, 8, strategy, flavour)
    assert got[0] in (2, 3)


@pytest.mark.parametrize("strategy,flavour", FORMS)
def test_everyone_infected(strategy, flavour):
    off, idx = graphs.erdos_renyi(3000, 0.004, 5)
    st0 = np.full(off.size - 1, 2, dtype=np.int32)
    _check(off, idx, st0, "B", 0.2, 0.1, 15, strategy, flavour)


@pytest.mark.parametrize("strategy,flavour", FORMS)
@pytest.mark.parametrize("variant", ["A", "B"])
def test_beta_gamma_one_is_deterministic(strategy, flavour, variant):
    """beta = gamma = 1: every susceptible agent with an infected neighbour is
    infected and every infected agent recovers, each tick (a breadth-first wave)."""
    n = 4000
    off, idx = _csr(n, np.arange(n - 1), np.arange(1, n))  # a path
    st0 = np.full(n, 1, dtype=np.int32)
    st0[n // 2] = 2
    got = _check(off, idx, st0, variant, 1.0, 1.0, 10, strategy, flavour)
    wave = np.abs(np.arange(n) - n // 2)
    assert np.all(got[wave < 10] == 3) and np.all(got[wave == 10] == 2) and np.all(got[wave > 10] == 1)


@pytest.mark.parametrize("strategy,flavour", FORMS)
def test_star_with_huge_hub(strategy, flavour):
    """One hub joined to 300,000 leaves: the hub's transpose row spans more than
    a thousand scatter segments when it changes state."""
    n = 300_001
    off, idx = _csr(n, np.zeros(n - 1, dtype=np.int64), np.arange(1, n))
    st0 = np.full(n, 1, dtype=np.int32)
    st0[0] = 2
    st0[1::997] = 2
    _check(off, idx, st0, "B", 0.3, 0.2, 8, strategy, flavour)
