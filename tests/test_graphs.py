"""Host-side graph generators, locality relabel and CSR permute (no GPU)."""
import numpy as np
import pytest

from sagesim_gb300 import graphs


def check_symmetric_simple(off, idx):
    n = off.size - 1
    src = np.repeat(np.arange(n), np.diff(off))
    assert (src != idx).all(), "self loop"
    key = src.astype(np.int64) * n + idx
    assert np.unique(key).size == key.size, "duplicate edge"
    rkey = idx.astype(np.int64) * n + src
    assert np.array_equal(np.sort(key), np.sort(rkey)), "not symmetric"


@pytest.mark.parametrize("gen", ["er", "ba", "ws"])
def test_generators_simple_symmetric_deterministic(gen):
    f = {"er": lambda: graphs.erdos_renyi(3000, 0.004, 9),
         "ba": lambda: graphs.barabasi_albert(3000, 4, 9),
         "ws": lambda: graphs.watts_strogatz(3000, 10, 0.1, 9)}[gen]
    off, idx = f()
    check_symmetric_simple(off, idx)
    off2, idx2 = f()
    assert np.array_equal(off, off2) and np.array_equal(idx, idx2)


def test_er_density():
    off, idx = graphs.erdos_renyi(10000, 0.001, 0)
    m = idx.size / 2
    exp = 0.001 * 10000 * 9999 / 2
    assert abs(m - exp) < 5 * np.sqrt(exp)


def test_ba_edges_and_hubs():
    n, m = 20000, 4
    off, idx = graphs.barabasi_albert(n, m, 1)
    assert idx.size == 2 * m * (n - m)
    deg = np.diff(off)
    assert deg[m:].min() >= m and deg.max() > 20 * m


def test_ws_degree():
    off, idx = graphs.watts_strogatz(5000, 10, 0.1, 2)
    assert idx.size == 5000 * 10


def test_partition_is_permutation_and_local():
    off, idx = graphs.barabasi_albert(20000, 3, 4)
    perm, part = graphs.partition_relabel(off, idx, 64, 1)
    assert np.array_equal(np.sort(perm), np.arange(perm.size))
    sizes = np.bincount(part, minlength=64)
    assert sizes.max() <= -(-perm.size // 64) + 1
    noff, nidx = graphs.permute_csr(off, idx, perm)
    check_symmetric_simple(noff, nidx)
    # a random 64-way split keeps 1/64 of the edges inside parts
    src = np.repeat(np.arange(perm.size), np.diff(off))
    inside = (part[perm[src]] == part[perm[idx]]).mean()
    assert inside > 10.0 / 64


def test_permute_preserves_row_order():
    off = np.array([0, 2, 3, 5], dtype=np.int32)
    idx = np.array([2, 1, 0, 1, 0], dtype=np.int32)
    perm = np.array([2, 0, 1], dtype=np.int32)
    noff, nidx = graphs.permute_csr(off, idx, perm)
    # old row 1 -> new row 0: [perm[0]] = [2]; old row 2 -> new row 1:
    # [perm[1], perm[0]] = [0, 2]; old row 0 -> new row 2: [perm[2], perm[1]] = [1, 0]
    assert noff.tolist() == [0, 1, 3, 5]
    assert nidx.tolist() == [2, 0, 2, 1, 0]


def test_bad_permutation_rejected():
    from sagesim_gb300 import SageSimError

    off = np.array([0, 1, 2], dtype=np.int32)
    idx = np.array([1, 0], dtype=np.int32)
    with pytest.raises(SageSimError):
        graphs.permute_csr(off, idx, np.array([0, 0], dtype=np.int32))


@pytest.mark.parametrize("n,m,seed", [(3, 4, 0), (5, 4, 1), (1000, 3, 7), (200_000, 4, 1), (50_000, 6, 2**63 + 5)])
def test_oracle_barabasi_albert_equals_the_engine_generator(n, m, seed):
    """The CPU baseline builds the benchmark's graph with oracle/'s own
    generator (no engine library in that process); both follow the same
    definition and must give the same CSR, row order included."""
    from oracle import oracle

    a_off, a_idx = oracle.barabasi_albert(n, m, seed)
    b_off, b_idx = graphs.barabasi_albert(n, m, seed)
    assert np.array_equal(a_off, b_off) and np.array_equal(a_idx, b_idx)
    assert np.array_equal(oracle.initial_infected(n, 0.01, seed % 2**32),
                          graphs.initial_infected(n, 0.01, seed % 2**32))
