"""sg_sir_run_noalloc: the SIR tick for callers that cannot allocate device memory.

Such callers (an embedding framework that owns all CUDA memory through its own
pool, code running while a stream is captured, a plugin whose contract forbids
allocation) hand the engine device pointers to the CSR and the state and get
the state back in place; every piece of scratch memory comes from a static
device array inside the library. This test allocates the inputs and outputs
itself (through torch, as such a caller would with its own allocator), calls
the entry point through the C ABI twice in a row on different graphs, and
checks each result against the regular engine entry point and against the
oracle (bit-exact, the tolerance every integer-state test here uses), also at
the entry point's largest agent count. It lives in a file collected last so
that a run stopping at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle
from sagesim_gb300 import Engine, _native, graphs

pytestmark = pytest.mark.gpu


def _reference_run(off, idx, st0, builtin, seed, tick0, nticks, beta, gamma):
    with Engine() as e:
        e.set_graph(off, idx, symmetric=True)
        e.set_seed(seed)
        p = e.add_property("state", np.int32, init=st0)
        e.add_sir(p, beta, gamma, variant="A" if builtin == _native.SG_BUILTIN_SIR_A else "B",
                  strategy="count")
        e.run(tick0, nticks, stats=False)
        return e.get_property(p)


def _noalloc_run(lib, torch, off, idx, st0, builtin, seed, tick0, nticks, beta, gamma):
    d_off = torch.from_numpy(off).cuda()
    d_idx = torch.from_numpy(idx).cuda()
    d_st = torch.from_numpy(st0.copy()).cuda()
    stream = torch.cuda.current_stream()
    rc = lib.sg_sir_run_noalloc(ctypes.c_void_p(d_off.data_ptr()), ctypes.c_void_p(d_idx.data_ptr()),
                                ctypes.c_void_p(d_st.data_ptr()), off.size - 1, builtin, seed, tick0,
                                nticks, beta, gamma, 1, 2, 3, ctypes.c_void_p(stream.cuda_stream))
    _native.check(rc)
    torch.cuda.synchronize()
    return d_st.cpu().numpy()


def _state(n, frac, seed):
    st = np.ones(n, dtype=np.int32)
    st[graphs.initial_infected(n, frac, seed)] = 2
    return st


def test_noalloc_matches_engine_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    lib = _native.load()
    # first call: 200k-agent BA graph, SIR-B, ticks 0..39
    off1, idx1 = graphs.barabasi_albert(200_000, 4, 21)
    st1 = _state(off1.size - 1, 0.005, 21)
    want1 = _reference_run(off1, idx1, st1, _native.SG_BUILTIN_SIR_B, 5, 0, 40, 0.05, 0.1)
    got1 = _noalloc_run(lib, torch, off1, idx1, st1, _native.SG_BUILTIN_SIR_B, 5, 0, 40, 0.05, 0.1)
    assert np.array_equal(got1, want1)
    # the oracle (draws keyed on the agent index, as the entry point keys them)
    assert np.array_equal(got1, oracle.sir_run(2, off1, idx1, st1, 5, 0, 40, 0.05, 0.1)[0])
    # second call right after, smaller ER graph (the scratch array still holds
    # the first call's counts and change lists), SIR-A, ticks 7..36
    off2, idx2 = graphs.erdos_renyi(150_000, 8.0 / 150_000, 22)
    st2 = _state(off2.size - 1, 0.01, 22)
    want2 = _reference_run(off2, idx2, st2, _native.SG_BUILTIN_SIR_A, 9, 7, 30, 0.2, 0.1)
    got2 = _noalloc_run(lib, torch, off2, idx2, st2, _native.SG_BUILTIN_SIR_A, 9, 7, 30, 0.2, 0.1)
    assert np.array_equal(got2, want2)
    assert np.array_equal(got2, oracle.sir_run(1, off2, idx2, st2, 9, 7, 30, 0.2, 0.1)[0])
    assert not np.array_equal(got2, st2)  # the epidemic moved


def test_noalloc_at_the_size_limit():
    """n == SG_NOALLOC_MAX_AGENTS exactly: every part of the scratch array
    (counts, change lists, tile counters, tile table, segment record) is used
    up to its last entry, twice in a row."""
    torch = pytest.importorskip("torch")
    lib = _native.load()
    n = 1048576  # SG_NOALLOC_MAX_AGENTS
    off, idx = graphs.erdos_renyi(n, 10.0 / n, 23)
    assert off.size - 1 == n
    st = _state(n, 0.002, 23)
    for tick0, nticks in ((0, 12), (12, 6)):
        want = _reference_run(off, idx, st, _native.SG_BUILTIN_SIR_B, 3, tick0, nticks, 0.08, 0.05)
        got = _noalloc_run(lib, torch, off, idx, st, _native.SG_BUILTIN_SIR_B, 3, tick0, nticks, 0.08, 0.05)
        assert np.array_equal(got, want)
        assert np.array_equal(got, oracle.sir_run(2, off, idx, st, 3, tick0, nticks, 0.08, 0.05)[0])
        assert not np.array_equal(got, st)
        st = got


def test_noalloc_rejects_sizes_beyond_the_limit():
    lib = _native.load()
    n = 1048576 + 1  # SG_NOALLOC_MAX_AGENTS + 1
    rc = lib.sg_sir_run_noalloc(None, None, None, n, _native.SG_BUILTIN_SIR_B, 0, 0, 1, 0.1, 0.1,
                                1, 2, 3, None)
    assert rc == _native.SG_ERR_INVALID
    assert "SG_NOALLOC_MAX_AGENTS" in _native.last_error(None)
