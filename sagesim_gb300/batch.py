"""Ensembles of independent SIR scenarios advanced together (one pool, one
launch per kernel per tick, CUDA-graph replay of the tick loop, autotuned
launch configuration). Each scenario stays bit-exact with its standalone
Engine run: own seed, logical ids, tick counter and horizon."""
import ctypes

import numpy as np

from . import _native as N


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def scenario_desc(offsets, indices, state, seed, beta, gamma, variant="B", horizon=0, lids=None,
                  codes=(1, 2, 3), symmetric=True, keep=None):
    """Builds a ScenarioDesc; `keep` collects the arrays that must outlive the call."""
    off = np.ascontiguousarray(offsets, dtype=np.int32)
    idx = np.ascontiguousarray(indices, dtype=np.int32)
    st = np.ascontiguousarray(state, dtype=np.int32)
    lid = None if lids is None else np.ascontiguousarray(lids, dtype=np.int64)
    if keep is not None:
        keep.extend([off, idx, st, lid])
    builtin = N.SG_BUILTIN_SIR_A if variant == "A" else N.SG_BUILTIN_SIR_B
    return N.ScenarioDesc(off.size - 1, idx.size, _p(off).value, _p(idx).value if idx.size else None,
                          _p(st).value, None if lid is None else _p(lid).value, int(seed), float(beta),
                          float(gamma), builtin, codes[0], codes[1], codes[2], int(horizon),
                          N.SG_GRAPH_SYMMETRIC if symmetric else 0)


STRATEGIES = {"pull": N.SG_SIR_PULL, "count": N.SG_SIR_COUNT}


class Batch:
    def __init__(self, device=0, stream=None):
        self._lib = N.load()
        h = ctypes.c_void_p()
        rc = self._lib.sg_batch_create(ctypes.byref(N.EngineCfg(device, 0, stream)), ctypes.byref(h))
        if rc != N.SG_OK:
            raise N.SageSimError(rc, N.last_error(None))
        self._h = h
        self._n = {}

    def _ck(self, rc):
        return N.check(rc, self._h, "sg_batch_last_error")

    def close(self):
        if getattr(self, "_h", None):
            self._lib.sg_batch_destroy(self._h)
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

    def add_scenario(self, offsets, indices, state, seed, beta, gamma, variant="B", horizon=0,
                     lids=None, codes=(1, 2, 3), symmetric=True):
        keep = []
        d = scenario_desc(offsets, indices, state, seed, beta, gamma, variant, horizon, lids, codes,
                          symmetric, keep)
        sid = ctypes.c_int32()
        self._ck(self._lib.sg_batch_add_scenario(self._h, ctypes.byref(d), ctypes.byref(sid)))
        self._n[sid.value] = d.n_agents
        return sid.value

    def commit(self):
        self._ck(self._lib.sg_batch_commit(self._h))

    def set_tune(self, strategy="count", blocks_per_sm=16, thread_row=32, mega_row=2048, count_flavour=272):
        t = N.Tune(STRATEGIES[strategy], blocks_per_sm, thread_row, mega_row, count_flavour, 0.0)
        self._ck(self._lib.sg_batch_set_tune(self._h, ctypes.byref(t)))

    def get_tune(self):
        t = N.Tune()
        self._ck(self._lib.sg_batch_get_tune(self._h, ctypes.byref(t)))
        return _tune_dict(t)

    def tune(self, ticks=8):
        t = N.Tune()
        self._ck(self._lib.sg_batch_tune(self._h, int(ticks), ctypes.byref(t)))
        return _tune_dict(t)

    def run(self, nticks, use_graph=True):
        self._ck(self._lib.sg_batch_run(self._h, int(nticks), 1 if use_graph else 0))

    def synchronize(self):
        self._ck(self._lib.sg_batch_synchronize(self._h))

    def get_state(self, sid):
        out = np.empty(self._n[sid], dtype=np.int32)
        self._ck(self._lib.sg_batch_get_state(self._h, sid, _p(out), out.size))
        return out

    def tick(self, sid):
        t = ctypes.c_int64()
        self._ck(self._lib.sg_batch_scenario_tick(self._h, sid, ctypes.byref(t)))
        return t.value

    def info(self):
        a, e, b = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self._ck(self._lib.sg_batch_info(self._h, ctypes.byref(a), ctypes.byref(e), ctypes.byref(b)))
        return {"agents": a.value, "nnz": e.value, "device_bytes": b.value}

    def snapshot(self):
        self._ck(self._lib.sg_batch_snapshot(self._h))

    def restore(self):
        self._ck(self._lib.sg_batch_restore(self._h))


def _tune_dict(t):
    inv = {v: k for k, v in STRATEGIES.items()}
    return {"strategy": inv[t.strategy], "blocks_per_sm": t.blocks_per_sm, "thread_row": t.thread_row,
            "mega_row": t.mega_row, "count_flavour": t.count_flavour, "us_per_tick": t.us_per_tick}
