"""Thin object wrapper over the C-ABI engine (one scenario on one GPU).

`Engine` is what the drop-in `Model` drives; tests and bench.py use it
directly for large workloads. Arrays cross the boundary as numpy arrays (host
pointers); the engine copies them to device memory it owns.
"""
import ctypes

import numpy as np

from . import _native as N


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class Engine:
    """One plain engine: CSR graph, SoA properties, builtin/compiled steps."""

    def __init__(self, device=0, stream=None):
        self._lib = N.load()
        cfg = N.EngineCfg(device, 0, stream)
        h = ctypes.c_void_p()
        rc = self._lib.sg_engine_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != N.SG_OK:
            raise N.SageSimError(rc, N.last_error(None))
        self._h = h
        self.n = None
        self._props = {}

    # -- lifecycle --------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._lib.sg_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _ck(self, rc):
        return N.check(rc, self._h)

    # -- model ------------------------------------------------------------
    def set_graph(self, offsets, indices, ordered=False, symmetric=False):
        off = np.ascontiguousarray(offsets, dtype=np.int32)
        idx = np.ascontiguousarray(indices, dtype=np.int32)
        n = off.size - 1
        flags = (N.SG_GRAPH_ORDERED if ordered else 0) | (N.SG_GRAPH_SYMMETRIC if symmetric else 0)
        self._ck(self._lib.sg_set_graph_csr(self._h, _ptr(off), n, _ptr(idx) if idx.size else None,
                                            idx.size, flags))
        self.n = n

    def set_graph_from_ids(self, ids, src_ids, dst_ids, symmetric=True, ordered=False):
        """Graph from an edge list in agent ids, built on the GPU: ids[k] is the id of
        the agent at buffer index k; an HBM hash table maps the edges' ids to indices.
        symmetric adds both directions; ordered keeps rows in first-connection order
        (else sorted); repeated edges are dropped."""
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        src = np.ascontiguousarray(src_ids, dtype=np.int64)
        dst = np.ascontiguousarray(dst_ids, dtype=np.int64)
        if src.shape != dst.shape:
            raise ValueError("src_ids and dst_ids differ in length")
        flags = (N.SG_GRAPH_ORDERED if ordered else 0) | (N.SG_GRAPH_SYMMETRIC if symmetric else 0)
        self._ck(self._lib.sg_set_graph_id_edges(self._h, _ptr(ids) if ids.size else None, ids.size,
                                                 _ptr(src) if src.size else None, _ptr(dst) if dst.size else None,
                                                 src.size, flags))
        self.n = ids.size

    def get_graph(self):
        """(offsets, indices) of the engine's CSR, copied to the host."""
        nnz = ctypes.c_int64()
        self._ck(self._lib.sg_get_graph_csr(self._h, None, None, ctypes.byref(nnz)))
        off = np.empty(self.n + 1, dtype=np.int32)
        idx = np.empty(max(nnz.value, 1), dtype=np.int32)
        self._ck(self._lib.sg_get_graph_csr(self._h, _ptr(off), _ptr(idx), ctypes.byref(nnz)))
        return off, idx[:nnz.value]

    def set_logical_ids(self, lids):
        if lids is None:
            self._ck(self._lib.sg_set_logical_ids(self._h, None, self.n))
            return
        a = np.ascontiguousarray(lids, dtype=np.int64)
        self._ck(self._lib.sg_set_logical_ids(self._h, _ptr(a), a.size))

    def set_seed(self, seed):
        self._ck(self._lib.sg_set_seed(self._h, int(seed)))

    def set_globals(self, values):
        a = np.ascontiguousarray(values, dtype=np.float64)
        self._ck(self._lib.sg_set_globals_f64(self._h, _ptr(a) if a.size else None, a.size))

    def add_property(self, name, dtype, width=1, init=None, double_buffered=True):
        dt = N.SG_I32 if np.dtype(dtype) == np.int32 else N.SG_F32
        npdt = np.int32 if dt == N.SG_I32 else np.float32
        a = None
        if init is not None:
            a = np.ascontiguousarray(init, dtype=npdt).reshape(-1)
            if a.size != self.n * width:
                raise ValueError("init must hold n*width values")
        pid = ctypes.c_int32()
        self._ck(self._lib.sg_add_property(self._h, name.encode(), dt, int(width),
                                           1 if double_buffered else 0, _ptr(a), ctypes.byref(pid)))
        self._props[pid.value] = (npdt, int(width), self.n)
        return pid.value

    def add_array(self, name, dtype, width, rows, init=None, double_buffered=True):
        """A breed-local array: `rows` rows of `width` values (zeros unless init),
        addressed by row in steps and in get/set_property."""
        dt = N.SG_I32 if np.dtype(dtype) == np.int32 else N.SG_F32
        npdt = np.int32 if dt == N.SG_I32 else np.float32
        a = None
        if init is not None:
            a = np.ascontiguousarray(init, dtype=npdt).reshape(-1)
            if a.size != rows * width:
                raise ValueError("init must hold rows*width values")
        pid = ctypes.c_int32()
        self._ck(self._lib.sg_add_array(self._h, name.encode(), dt, int(width), int(rows),
                                        1 if double_buffered else 0, _ptr(a), ctypes.byref(pid)))
        self._props[pid.value] = (npdt, int(width), int(rows))
        return pid.value

    def set_property(self, prop, values, first=0):
        npdt, width, _ = self._props[prop]
        a = np.ascontiguousarray(values, dtype=npdt).reshape(-1)
        if a.size % width:
            raise ValueError("values must hold whole rows")
        self._ck(self._lib.sg_set_property(self._h, prop, _ptr(a), int(first), a.size // width))

    def set_property_ptr(self, prop, host_ptr, first, count):
        """Copies `count` rows from a raw host pointer (e.g. pinned memory)."""
        self._ck(self._lib.sg_set_property(self._h, prop, ctypes.c_void_p(host_ptr), int(first), int(count)))

    def get_property(self, prop, first=0, count=None):
        npdt, width, rows = self._props[prop]
        if count is None:
            count = rows - first
        out = np.empty(count * width, dtype=npdt)
        self._ck(self._lib.sg_get_property(self._h, prop, _ptr(out), int(first), int(count)))
        return out.reshape(count, width) if width > 1 else out

    def get_property_ptr(self, prop, host_ptr, first, count):
        self._ck(self._lib.sg_get_property(self._h, prop, ctypes.c_void_p(host_ptr), int(first), int(count)))

    def property_device_ptr(self, prop):
        p = ctypes.c_void_p()
        self._ck(self._lib.sg_property_device_ptr(self._h, prop, ctypes.byref(p)))
        return p.value

    # -- steps --------------------------------------------------------------
    @staticmethod
    def _params(builtin, state_prop, begin, end, beta=0.0, gamma=0.0, codes=(1, 2, 3),
                strategy="count", priority=0, aux_prop=-1, sigma=0.0):
        st = {"pull": N.SG_SIR_PULL, "count": N.SG_SIR_COUNT, "frontier": N.SG_SIR_FRONTIER}[strategy]
        return N.BuiltinParams(builtin, st, state_prop, aux_prop, codes[0], codes[1], codes[2],
                               priority, int(begin), int(end), float(beta), float(gamma), float(sigma))

    def add_sir(self, state_prop, beta, gamma, variant="B", strategy="count", codes=(1, 2, 3),
                begin=0, end=None, priority=0):
        builtin = N.SG_BUILTIN_SIR_A if variant == "A" else N.SG_BUILTIN_SIR_B
        p = self._params(builtin, state_prop, begin, self.n if end is None else end, beta, gamma,
                         codes, strategy, priority)
        sid = ctypes.c_int32()
        self._ck(self._lib.sg_add_builtin_step(self._h, ctypes.byref(p), ctypes.byref(sid)))
        return sid.value

    def update_sir(self, step_id, state_prop, beta, gamma, variant="B", strategy="count",
                   codes=(1, 2, 3), begin=0, end=None, priority=0):
        builtin = N.SG_BUILTIN_SIR_A if variant == "A" else N.SG_BUILTIN_SIR_B
        p = self._params(builtin, state_prop, begin, self.n if end is None else end, beta, gamma,
                         codes, strategy, priority)
        self._ck(self._lib.sg_update_builtin_step(self._h, step_id, ctypes.byref(p)))

    def add_opinion(self, opinion_prop, weights_prop, sigma, begin=0, end=None, priority=0):
        p = self._params(N.SG_BUILTIN_OPINION, opinion_prop, begin, self.n if end is None else end,
                         priority=priority, aux_prop=weights_prop, sigma=sigma, strategy="pull")
        sid = ctypes.c_int32()
        self._ck(self._lib.sg_add_builtin_step(self._h, ctypes.byref(p), ctypes.byref(sid)))
        return sid.value

    def compile_step(self, source, entry, written, begin=0, end=None, priority=0):
        w = np.ascontiguousarray(list(written), dtype=np.int32)
        sid = ctypes.c_int32()
        self._ck(self._lib.sg_compile_step(self._h, source.encode(), entry.encode(), int(priority),
                                           int(begin), int(self.n if end is None else end),
                                           _ptr(w) if w.size else None, w.size, ctypes.byref(sid)))
        return sid.value

    # -- execution ------------------------------------------------------------
    def run(self, tick0, nticks, stats=True):
        """Runs nticks synchronously; returns (per-tick stats int64[nticks, 4] or None, totals)."""
        st = np.zeros((max(nticks, 0), 4), dtype=np.int64) if stats else None
        tot = N.Stats()
        self._ck(self._lib.sg_run(self._h, int(tick0), int(nticks), _ptr(st) if stats and nticks else None,
                                  ctypes.byref(tot) if stats else None))
        return st, tot

    def run_async(self, tick0, nticks, use_graph=True):
        self._ck(self._lib.sg_run_async(self._h, int(tick0), int(nticks), 1 if use_graph else 0))

    def last_run_active(self, nticks):
        out = np.zeros(nticks, dtype=np.int64)
        self._ck(self._lib.sg_last_run_active(self._h, _ptr(out), int(nticks)))
        return out

    def synchronize(self):
        self._ck(self._lib.sg_synchronize(self._h))

    def tick_history(self):
        """(first tick, int64[ticks, 4] of S, I, R, E_S) recorded by consecutive
        run() calls with statistics."""
        rows, first = ctypes.c_int64(), ctypes.c_int64()
        self._ck(self._lib.sg_get_tick_history(self._h, None, 0, ctypes.byref(rows), ctypes.byref(first)))
        out = np.zeros((rows.value, 4), dtype=np.int64)
        if rows.value:
            self._ck(self._lib.sg_get_tick_history(self._h, _ptr(out), rows.value, ctypes.byref(rows),
                                                   ctypes.byref(first)))
        return first.value, out

    def snapshot(self):
        self._ck(self._lib.sg_snapshot(self._h))

    def restore(self):
        self._ck(self._lib.sg_restore(self._h))

    def set_tune(self, blocks_per_sm=16, thread_row=32, mega_row=2048, count_flavour=790):
        """Launch configuration of the SIR kernels (results are identical for all)."""
        t = N.Tune(N.SG_SIR_COUNT, blocks_per_sm, thread_row, mega_row, count_flavour, 0.0)
        self._ck(self._lib.sg_engine_set_tune(self._h, ctypes.byref(t)))

    def opinion_cosine_check(self, k0, n):
        """(split-table cosine, direct cos) of 2 pi k / 2^23 for k0 <= k < k0 + n."""
        split = np.empty(n, dtype=np.float64)
        direct = np.empty(n, dtype=np.float64)
        self._ck(self._lib.sg_opinion_cosine_check(self._h, int(k0), int(n), _ptr(split), _ptr(direct)))
        return split, direct

    def opinion_noise_check(self, x, k1, k2, sigma):
        """(result, pair-table result, slow flags) of the opinion step's noise term
        for opinions x and the normal draw's 23-bit integers k1, k2."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        k1 = np.ascontiguousarray(k1, dtype=np.uint32)
        k2 = np.ascontiguousarray(k2, dtype=np.uint32)
        n = len(x)
        if len(k1) != n or len(k2) != n:
            raise ValueError("x, k1 and k2 must have the same length")
        out = np.empty(n, dtype=np.float32)
        exact = np.empty(n, dtype=np.float32)
        slow = np.empty(n, dtype=np.uint8)
        self._ck(self._lib.sg_opinion_noise_check(self._h, float(sigma), n, _ptr(x), _ptr(k1), _ptr(k2),
                                                  _ptr(out), _ptr(exact), _ptr(slow)))
        return out, exact, slow.astype(bool)

    def profile(self, on=True):
        self._ck(self._lib.sg_profile_enable(self._h, 1 if on else 0))

    def profile_report(self):
        out = {}
        k = 0
        name = ctypes.create_string_buffer(128)
        launches = ctypes.c_int64()
        ms = ctypes.c_double()
        while self._lib.sg_profile_get(self._h, k, name, 128, ctypes.byref(launches), ctypes.byref(ms)) == 0:
            out[name.value.decode()] = (launches.value, ms.value)
            k += 1
        return out
