"""Engine vs CPU oracle on seeded inputs (CUDA path through the C ABI)."""
import numpy as np
import pytest

from oracle import oracle
from sagesim_gb300 import Engine, graphs

pytestmark = pytest.mark.gpu


def _init_state(n, frac, seed, codes=(1, 2, 3)):
    st = np.full(n, codes[0], dtype=np.int32)
    st[graphs.initial_infected(n, frac, seed)] = codes[1]
    return st


@pytest.mark.parametrize("variant", ["A", "B"])
@pytest.mark.parametrize("strategy", ["pull", "count"])
@pytest.mark.parametrize("kind", ["er", "ba"])
def test_sir_matches_oracle_every_tick(variant, strategy, kind):
    if kind == "er":
        off, idx = graphs.erdos_renyi(10000, 0.001, 0)
        beta, gamma = 0.05, 0.1
    else:
        off, idx = graphs.barabasi_albert(20000, 4, 1)
        beta, gamma = 0.03, 0.07
    n = off.size - 1
    st0 = _init_state(n, 0.01, 0)
    ticks = 60
    with Engine() as e:
        e.set_graph(off, idx, symmetric=True)
        e.set_seed(7)
        p = e.add_property("state", np.int32, init=st0)
        e.add_sir(p, beta, gamma, variant=variant, strategy=strategy)
        st = st0.copy()
        for t in range(ticks):
            stats, _ = e.run(t, 1)
            ref, rstats, _ = oracle.sir_run(1 if variant == "A" else 2, off, idx, st, 7, t, 1, beta, gamma)
            got = e.get_property(p)
            assert np.array_equal(got, ref), "tick %d: %d agents differ" % (t, int((got != ref).sum()))
            assert np.array_equal(stats, rstats), "tick %d stats %s vs %s" % (t, stats, rstats)
            st = ref
