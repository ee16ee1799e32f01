"""Engine vs CPU oracle on seeded inputs (CUDA path through the C ABI)."""
import numpy as np
import pytest

from oracle import oracle
from sagesim_gb300 import Engine, SageSimError, graphs

pytestmark = pytest.mark.gpu


def _init_state(n, frac, seed, codes=(1, 2, 3)):
    st = np.full(n, codes[0], dtype=np.int32)
    st[graphs.initial_infected(n, frac, seed)] = codes[1]
    return st


def csr_from_edges(n, a, b):
    """Symmetric CSR (duplicates kept out) from undirected edge arrays."""
    a = np.asarray(a, dtype=np.int64)
    b = np.asarray(b, dtype=np.int64)
    keep = a != b
    src = np.concatenate([a[keep], b[keep]])
    dst = np.concatenate([b[keep], a[keep]])
    key = np.unique(src * n + dst)
    src, dst = key // n, key % n
    off = np.zeros(n + 1, dtype=np.int32)
    np.add.at(off, src + 1, 1)
    return np.cumsum(off, dtype=np.int64).astype(np.int32), dst.astype(np.int32)


def hub_graph(seed=3):
    """BA graph plus three hubs of 2500-6000 neighbours: rows for every bin."""
    n = 30000
    off, idx = graphs.barabasi_albert(n, 3, seed)
    src = np.repeat(np.arange(n), np.diff(off))
    rng = np.random.default_rng(seed)
    a, b = [src], [idx]
    for h, deg in ((5, 6000), (17, 2500), (123, 4000)):
        nb = rng.choice(n, size=deg, replace=False)
        a.append(np.full(deg, h))
        b.append(nb)
    return csr_from_edges(n, np.concatenate(a), np.concatenate(b))


@pytest.mark.parametrize("variant", ["A", "B"])
@pytest.mark.parametrize("strategy", ["pull", "count", "frontier"])
@pytest.mark.parametrize("kind", ["er", "ba", "hubs", "directed"])
def test_sir_matches_oracle_every_tick(variant, strategy, kind):
    if kind == "er":
        off, idx = graphs.erdos_renyi(10000, 0.001, 0)
        beta, gamma = 0.05, 0.1
    elif kind == "ba":
        off, idx = graphs.barabasi_albert(20000, 4, 1)
        beta, gamma = 0.03, 0.07
    elif kind == "hubs":
        off, idx = hub_graph()
        assert np.diff(off).max() > 2048
        beta, gamma = 0.02, 0.1
    else:  # directed: rows are out-neighbours only, the count strategy needs the transpose
        n = 15000
        rng = np.random.default_rng(11)
        deg = rng.integers(0, 12, size=n)
        deg[7] = 3000
        off = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
        idx = rng.integers(0, n, size=int(off[-1])).astype(np.int32)
        beta, gamma = 0.1, 0.05
    n = off.size - 1
    st0 = _init_state(n, 0.01, 0)
    ticks = 60
    with Engine() as e:
        e.set_graph(off, idx, symmetric=(kind != "directed"))
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


COUNT_FLAVOURS = list(range(8)) + [8, 12, 16, 24, 48, 56, 63, 48 | 64, 48 | 128, 56 | 192, 48 | 256 | 4, 48 | 256 | 1,
                                   16 | 256, 48 | 256 | 6, 16 | 256 | 6,
                                   # flat draws: every tick, every tick with a row-per-lane scatter, and in
                                   # the hybrid's busy ticks (forced on this small graph)
                                   512, 512 | 8, 512 | 48 | 256, 512 | 48 | 256 | 6]


@pytest.mark.parametrize("flavour", COUNT_FLAVOURS)
@pytest.mark.parametrize("variant", ["A", "B"])
def test_count_step_flavours_identical(flavour, variant):
    """Every count-step flavour (8 agents per thread, warp-dense draws, lazy
    loads, class sweep, either scatter) gives the oracle's states; checked
    through the non-statistics path."""
    off, idx = hub_graph(5)
    n = off.size - 1
    st0 = _init_state(n, 0.01, 5)
    with Engine() as e:
        e.set_graph(off, idx, symmetric=True)
        e.set_seed(9)
        p = e.add_property("state", np.int32, init=st0)
        e.add_sir(p, 0.04, 0.08, variant=variant, strategy="count")
        e.set_tune(blocks_per_sm=4 + 4 * (flavour & 1), count_flavour=flavour)
        for t0 in (0, 15, 30):
            e.run_async(t0, 15, use_graph=(t0 > 0))
        e.synchronize()
        got = e.get_property(p)
    ref, _, _ = oracle.sir_run(1 if variant == "A" else 2, off, idx, st0, 9, 0, 45, 0.04, 0.08)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("flavour", [0, 16, 48, 48 | 64, 48 | 128, 48 | 256 | 4, 48 | 256 | 3, 48 | 256 | 6,
                                     512, 512 | 48 | 256])
@pytest.mark.parametrize("variant", ["A", "B"])
def test_count_dense_graph_with_statistics(flavour, variant):
    """A dense graph with many infected neighbours per agent and a small beta
    (long draw loops, every agent a candidate of the class sweep, activity bits
    rebuilt after busy ticks): states and per-tick statistics match the oracle."""
    off, idx = graphs.erdos_renyi(6000, 0.03, 2)
    n = off.size - 1
    st0 = _init_state(n, 0.4, 6)
    beta, gamma = 0.005, 0.05
    with Engine() as e:
        e.set_graph(off, idx, symmetric=True)
        e.set_seed(11)
        p = e.add_property("state", np.int32, init=st0)
        e.add_sir(p, beta, gamma, variant=variant, strategy="count")
        e.set_tune(blocks_per_sm=8, count_flavour=flavour)
        stats, _ = e.run(0, 12, stats=True)
        got = e.get_property(p)
    ref, rstats, _ = oracle.sir_run(1 if variant == "A" else 2, off, idx, st0, 11, 0, 12, beta, gamma)
    assert np.array_equal(got, ref)
    assert np.array_equal(stats, rstats)


@pytest.mark.parametrize("variant", ["A", "B"])
def test_flat_step_on_a_range_without_class_bytes(variant):
    """A count step over agents [37, n - 100): its tiles do not start at
    multiples of 32, so no class bytes are kept and the flat-draw step reads the
    states (scalar loads at unaligned tile edges); agents outside the range keep
    their state. Equal to the loop form, every tick's statistics included."""
    off, idx = hub_graph(9)
    n = off.size - 1
    st0 = _init_state(n, 0.02, 9)
    out = {}
    for fl in (4, 512):
        with Engine() as e:
            e.set_graph(off, idx, symmetric=True)
            e.set_seed(3)
            p = e.add_property("state", np.int32, init=st0)
            e.add_sir(p, 0.05, 0.08, variant=variant, strategy="count", begin=37, end=n - 100)
            e.set_tune(count_flavour=fl)
            stats, _ = e.run(0, 40, stats=True)
            out[fl] = (e.get_property(p), stats)
    assert np.array_equal(out[4][0], out[512][0]) and np.array_equal(out[4][1], out[512][1])
    assert np.array_equal(out[512][0][:37], st0[:37]) and np.array_equal(out[512][0][n - 100:], st0[n - 100:])
    assert not np.array_equal(out[512][0], st0)


@pytest.mark.parametrize("wpt_bits", [64, 128, 192, 256 | 4, 256 | 64 | 2])
@pytest.mark.parametrize("variant", ["A", "B"])
def test_class_sweep_statistics_on_power_law_graph(variant, wpt_bits):
    """Class sweep with statistics on a graph with hubs, through busy and quiet
    ticks (bits kept by the scatter, then rebuilt, then kept again)."""
    off, idx = hub_graph(7)
    n = off.size - 1
    st0 = _init_state(n, 0.002, 7)
    with Engine() as e:
        e.set_graph(off, idx, symmetric=True)
        e.set_seed(5)
        p = e.add_property("state", np.int32, init=st0)
        e.add_sir(p, 0.2, 0.1, variant=variant, strategy="count")
        e.set_tune(blocks_per_sm=16, count_flavour=48 | wpt_bits)
        stats, _ = e.run(0, 60, stats=True)
        got = e.get_property(p)
    ref, rstats, _ = oracle.sir_run(1 if variant == "A" else 2, off, idx, st0, 5, 0, 60, 0.2, 0.1)
    assert np.array_equal(got, ref)
    assert np.array_equal(stats, rstats)


def test_array_rows_bounds_and_snapshot():
    """An engine array (breed-local array storage) with its own row count: a
    compiled step reads tick-start values (double-buffered), reads 0 and drops
    writes outside the array, and get/set_property, snapshot and restore address
    its rows."""
    n, rows = 100, 40
    off, idx = graphs.erdos_renyi(n, 0.05, 3)
    with Engine() as e:
        e.set_graph(off, idx, symmetric=True)
        p = e.add_property("state", np.int32, init=np.zeros(n, dtype=np.int32))
        arr = e.add_array("sgbla_h", np.float32, 3, rows)
        imap = np.where(np.arange(n) < rows, np.arange(n), -1).astype(np.int32)
        pi = e.add_property("sgbla_h_idx", np.int32, init=imap, double_buffered=False)
        src = ("#define PROP_state %d\n#define PROP_sgbla_h %d\n#define PROP_sgbla_h_idx %d\n" % (p, arr, pi)) + """
__device__ void f(const sg_ctx &ctx, int i)
{
    const long long row = ctx.i32(PROP_sgbla_h_idx, i);
    const float v = ctx.arr_f32(PROP_sgbla_h, row, 0) + ctx.arr_f32(PROP_sgbla_h, row, 7) + 1.0f;
    ctx.set_arr_f32(PROP_sgbla_h, row, v, 0);
    ctx.set_arr_f32(PROP_sgbla_h, row, (float)ctx.tick, 2);
    ctx.set_arr_f32(PROP_sgbla_h, row + 1000, 5.0f, 0);
    ctx.set_arr_f32(PROP_sgbla_h, row, 9.0f, 3);
    ctx.set_i32(PROP_state, i, ctx.i32(PROP_state, i) + 1);
}
"""
        e.compile_step(src, "f", [arr, p])
        e.run(0, 5, stats=False)
        h = e.get_property(arr)
        assert h.shape == (rows, 3)
        assert (h[:, 0] == 5).all() and (h[:, 1] == 0).all() and (h[:, 2] == 4).all()
        assert (e.get_property(p) == 5).all()
        assert np.array_equal(e.get_property(arr, first=10, count=5), h[10:15])
        e.snapshot()
        e.run(5, 2, stats=False)
        assert (e.get_property(arr)[:, 0] == 7).all()
        e.restore()
        assert (e.get_property(arr)[:, 0] == 5).all()
        e.set_property(arr, np.ones((2, 3), dtype=np.float32), first=rows - 2)
        assert (e.get_property(arr)[rows - 2:] == 1).all()
        with pytest.raises(SageSimError):
            e.get_property(arr, first=rows - 1, count=2)
        a2 = e.add_array("a2", np.int32, 1, rows)
        with pytest.raises(SageSimError, match="agent property"):
            e.add_sir(a2, 0.1, 0.1)  # an array is not an agent property


def test_tick_history_across_runs():
    """sg_get_tick_history: consecutive runs add their per-tick S, I, R, E_S rows;
    a run from another tick starts a new history."""
    off, idx = graphs.erdos_renyi(5000, 0.002, 4)
    st0 = np.ones(5000, dtype=np.int32)
    st0[:50] = 2
    with Engine() as e:
        e.set_graph(off, idx, symmetric=True)
        p = e.add_property("state", np.int32, init=st0)
        e.add_sir(p, 0.1, 0.1, variant="B")
        e.snapshot()
        a, _ = e.run(0, 10)
        b, _ = e.run(10, 5)
        first, hist = e.tick_history()
        assert first == 0 and np.array_equal(hist, np.vstack([a, b]))
        e.restore()
        c, _ = e.run(0, 3)
        first, hist = e.tick_history()
        assert first == 0 and np.array_equal(hist, c) and np.array_equal(c, a[:3])
