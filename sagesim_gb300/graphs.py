"""Seeded synthetic graphs (symmetric int32 CSR) and the locality relabel.

Wrappers of the host-side generators in the native library. SAGESim users
build graphs with networkx (e.g. tests/test_double_buffer.py:206-221) and
partition with METIS (sagesim/generate_partition.py:24-69); these give the
same kinds of graphs at 10^7 agents in seconds.
"""
import ctypes

import numpy as np

from . import _native as N


def _two_pass(fn, *args):
    lib = N.load()
    nnz = ctypes.c_int64()
    N.check(getattr(lib, fn)(*args, None, None, ctypes.byref(nnz)))
    n = args[0]
    off = np.empty(n + 1, dtype=np.int32)
    idx = np.empty(max(nnz.value, 1), dtype=np.int32)
    N.check(getattr(lib, fn)(*args, ctypes.c_void_p(off.ctypes.data), ctypes.c_void_p(idx.ctypes.data),
                             ctypes.byref(nnz)))
    return off, idx[:nnz.value]


def erdos_renyi(n, p, seed):
    return _two_pass("sg_graph_er", int(n), float(p), ctypes.c_uint64(seed))


def barabasi_albert(n, m, seed):
    return _two_pass("sg_graph_ba", int(n), int(m), ctypes.c_uint64(seed))


def watts_strogatz(n, k, p, seed):
    return _two_pass("sg_graph_ws", int(n), int(k), float(p), ctypes.c_uint64(seed))


def partition_relabel(offsets, indices, k=64, seed=0):
    """perm[old] = new (k-way graph-growing partition, BFS order inside parts)."""
    lib = N.load()
    off = np.ascontiguousarray(offsets, dtype=np.int32)
    idx = np.ascontiguousarray(indices, dtype=np.int32)
    n = off.size - 1
    perm = np.empty(n, dtype=np.int32)
    part = np.empty(n, dtype=np.int32)
    N.check(lib.sg_partition_relabel(n, ctypes.c_void_p(off.ctypes.data), ctypes.c_void_p(idx.ctypes.data),
                                     int(k), ctypes.c_uint64(seed), ctypes.c_void_p(perm.ctypes.data),
                                     ctypes.c_void_p(part.ctypes.data)))
    return perm, part


def permute_csr(offsets, indices, perm):
    """CSR with row perm[i] = row i, entries mapped through perm (order kept)."""
    lib = N.load()
    off = np.ascontiguousarray(offsets, dtype=np.int32)
    idx = np.ascontiguousarray(indices, dtype=np.int32)
    pm = np.ascontiguousarray(perm, dtype=np.int32)
    n = off.size - 1
    noff = np.empty(n + 1, dtype=np.int32)
    nidx = np.empty(max(idx.size, 1), dtype=np.int32)
    N.check(lib.sg_csr_permute(n, ctypes.c_void_p(off.ctypes.data), ctypes.c_void_p(idx.ctypes.data),
                               ctypes.c_void_p(pm.ctypes.data), ctypes.c_void_p(noff.ctypes.data),
                               ctypes.c_void_p(nidx.ctypes.data)))
    return noff, nidx[:idx.size]


def initial_infected(n, fraction, seed):
    """Indices of round(fraction * n) distinct agents (numpy PCG64, platform independent)."""
    k = int(round(fraction * n))
    return np.sort(np.random.default_rng(seed).choice(n, size=k, replace=False)).astype(np.int64)


def generate(spec):
    """One graph from a spec tuple: ("er", n, p, seed) | ("ba", n, m, seed) |
    ("ws", n, k, p, seed)."""
    kind = spec[0]
    if kind == "er":
        return erdos_renyi(*spec[1:])
    if kind == "ba":
        return barabasi_albert(*spec[1:])
    if kind == "ws":
        return watts_strogatz(*spec[1:])
    raise ValueError("unknown graph kind %r" % (kind,))


def generate_many(specs, processes=None):
    """Generates graphs in parallel worker processes (spawn start method, so it
    is safe after CUDA has been initialised in the calling process)."""
    import multiprocessing as mp
    import os

    if processes is None:
        processes = min(len(specs), os.cpu_count() or 1)
    if processes <= 1 or len(specs) <= 1:
        return [generate(s) for s in specs]
    ctx = mp.get_context("spawn")
    with ctx.Pool(processes) as pool:
        return pool.map(generate, specs, chunksize=1)
