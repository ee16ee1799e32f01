"""ctypes wrapper around oracle/_build/libsg_oracle.so (test infrastructure only).

The C restatement follows sagesim/math_utils.py:106-189 (Philox-2x32-10),
sagesim/math_utils.py:231-255 (Box-Muller normal) and the tick semantics of
sagesim/model.py:2306-2408 (double-buffered step, write-back after all
priorities). Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg import it.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libsg_oracle.so")
_lib = None

_i64 = ctypes.c_int64
_i32 = ctypes.c_int32
_p = ctypes.c_void_p


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
                os.path.join(_HERE, "sg_oracle.c")):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.sgo_philox_k23.restype = ctypes.c_uint32
        L.sgo_philox_k23.argtypes = [_i64, _i64, _i64, _i64]
        L.sgo_rand_uniform.restype = ctypes.c_double
        L.sgo_rand_uniform.argtypes = [_i64, _i64, _i64, _i64]
        L.sgo_rand_normal.restype = ctypes.c_double
        L.sgo_rand_normal.argtypes = [_i64, _i64, _i64, _i64]
        L.sgo_threshold.restype = ctypes.c_uint32
        L.sgo_threshold.argtypes = [ctypes.c_double]
        L.sgo_sir_run.restype = ctypes.c_int
        L.sgo_sir_run.argtypes = [ctypes.c_int, _i64, _p, _p, _p, _i64, _i64, _i32,
                                  ctypes.c_double, ctypes.c_double, _i32, _i32, _i32,
                                  _p, _p, _p, ctypes.c_int]
        L.sgo_opinion_run.restype = ctypes.c_int
        L.sgo_opinion_run.argtypes = [_i64, _p, _p, _p, _i64, _i64, _i32, ctypes.c_double,
                                      _i32, _p, _p, _p, ctypes.c_int]
        L.sgo_philox_batch.restype = None
        L.sgo_philox_batch.argtypes = [_i64, _p, _p, _p, _p, _p]
        L.sgo_normal_batch.restype = None
        L.sgo_normal_batch.argtypes = [_i64, _p, _p, _p, _p, _p]
        L.sgo_max_threads.restype = ctypes.c_int
        L.sgo_graph_ba.restype = ctypes.c_int
        L.sgo_graph_ba.argtypes = [_i64, _i32, ctypes.c_uint64, _p, _p, ctypes.POINTER(_i64)]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def philox_k23(seed, tick, lid, salt):
    seed, tick, lid, salt = (np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.int64), np.broadcast(seed, tick, lid, salt).shape)).ravel()
                             for v in (seed, tick, lid, salt))
    out = np.empty(seed.size, dtype=np.uint32)
    lib().sgo_philox_batch(seed.size, _ptr(seed), _ptr(tick), _ptr(lid), _ptr(salt), _ptr(out))
    return out


def rand_uniform(seed, tick, lid, salt):
    return philox_k23(seed, tick, lid, salt).astype(np.float64) / 8388608.0


def rand_normal(seed, tick, lid, salt):
    shape = np.broadcast(seed, tick, lid, salt).shape
    seed, tick, lid, salt = (np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.int64), shape)).ravel()
                             for v in (seed, tick, lid, salt))
    out = np.empty(seed.size, dtype=np.float64)
    lib().sgo_normal_batch(seed.size, _ptr(seed), _ptr(tick), _ptr(lid), _ptr(salt), _ptr(out))
    return out


def threshold(p):
    return int(lib().sgo_threshold(float(p)))


def sir_run(variant, offsets, indices, state, seed, tick0, nticks, beta, gamma,
            codes=(1, 2, 3), lids=None, history=False, nthreads=0):
    """Runs nticks SIR ticks on a copy of `state`.

    Returns (final_state int32[n], stats int64[nticks, 4], history int8[nticks, n] or None).
    stats rows: S, I, R after the tick and E_S (degree sum of tick-start S agents).
    """
    off = np.ascontiguousarray(offsets, dtype=np.int32)
    idx = np.ascontiguousarray(indices, dtype=np.int32)
    st = np.array(state, dtype=np.int32, copy=True)
    n = st.size
    if off.size != n + 1:
        raise ValueError("offsets must have n+1 entries")
    lid = None if lids is None else np.ascontiguousarray(lids, dtype=np.int64)
    stats = np.zeros((max(nticks, 0), 4), dtype=np.int64)
    hist = np.zeros((nticks, n), dtype=np.int8) if history else None
    rc = lib().sgo_sir_run(int(variant), n, _ptr(off), _ptr(idx), _ptr(lid), int(seed), int(tick0),
                           int(nticks), float(beta), float(gamma), int(codes[0]), int(codes[1]),
                           int(codes[2]), _ptr(st), _ptr(stats), _ptr(hist), int(nthreads))
    if rc != 0:
        raise MemoryError("oracle allocation failed")
    return st, stats, hist


def opinion_run(offsets, indices, weights, opinion, seed, tick0, nticks, sigma, lids=None,
                history=False, nthreads=0):
    off = np.ascontiguousarray(offsets, dtype=np.int32)
    idx = np.ascontiguousarray(indices, dtype=np.int32)
    w = np.ascontiguousarray(weights, dtype=np.float32)
    x = np.array(opinion, dtype=np.float32, copy=True)
    n = x.size
    width = w.shape[1] if w.ndim == 2 else 1
    lid = None if lids is None else np.ascontiguousarray(lids, dtype=np.int64)
    hist = np.zeros((nticks, n), dtype=np.float32) if history else None
    rc = lib().sgo_opinion_run(n, _ptr(off), _ptr(idx), _ptr(lid), int(seed), int(tick0), int(nticks),
                               float(sigma), int(width), _ptr(w), _ptr(x), _ptr(hist), int(nthreads))
    if rc != 0:
        raise MemoryError("oracle allocation failed")
    return x, hist


def max_threads():
    return int(lib().sgo_max_threads())


def barabasi_albert(n, m, seed):
    """Symmetric int32 CSR of the seeded Barabasi-Albert graph (sgo_graph_ba)."""
    nnz = _i64()
    rc = lib().sgo_graph_ba(int(n), int(m), int(seed) & (2**64 - 1), None, None, ctypes.byref(nnz))
    if rc != 0:
        raise ValueError("sgo_graph_ba: bad arguments")
    off = np.empty(int(n) + 1, dtype=np.int32)
    idx = np.empty(max(nnz.value, 1), dtype=np.int32)
    rc = lib().sgo_graph_ba(int(n), int(m), int(seed) & (2**64 - 1), _ptr(off), _ptr(idx), ctypes.byref(nnz))
    if rc != 0:
        raise MemoryError("sgo_graph_ba: out of memory")
    return off, idx[:nnz.value]


def initial_infected(n, fraction, seed):
    """Indices of round(fraction * n) distinct agents drawn by numpy's PCG64
    generator (the same draw the engine's input helpers make)."""
    k = int(round(fraction * n))
    return np.sort(np.random.default_rng(seed).choice(n, size=k, replace=False)).astype(np.int64)
