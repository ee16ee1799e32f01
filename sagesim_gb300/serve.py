"""Serving SIR scenario requests with continuous batching.

Server wraps the C-ABI server: requests are queued, admitted against an HBM
budget as resident slots free up, advanced together with every other resident
scenario, and retired at their horizon. serve_stream() drives a server with a
timed arrival sequence (e.g. a Poisson stream) and measures, per request, the
latency from arrival to completion.
"""
import ctypes
import time

import numpy as np

from . import _native as N
from .batch import STRATEGIES, scenario_desc


class Server:
    def __init__(self, budget_bytes, agent_slots, edge_slots, max_resident=4096, variant="B", device=0,
                 stream=None):
        self._lib = N.load()
        builtin = N.SG_BUILTIN_SIR_A if variant == "A" else N.SG_BUILTIN_SIR_B
        cfg = N.ServerCfg(device, builtin, stream, int(budget_bytes), int(agent_slots), int(edge_slots),
                          int(max_resident), 0)
        h = ctypes.c_void_p()
        rc = self._lib.sg_server_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != N.SG_OK:
            raise N.SageSimError(rc, N.last_error(None))
        self._h = h
        self.variant = variant
        self._n = {}
        self._borrowed = {}  # rid -> arrays a borrowed request points into

    def _ck(self, rc):
        return N.check(rc, self._h, "sg_server_last_error")

    def close(self):
        if getattr(self, "_h", None):
            self._lib.sg_server_destroy(self._h)
            self._h = None
        self._borrowed = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, offsets, indices, state, seed, beta, gamma, horizon, codes=(1, 2, 3), lids=None,
               borrow=False):
        """Queues (or places at once) one scenario. lids: the logical id of every
        agent, the key of its random draws (sagesim/model.py:656-667); None keys
        the draws on the agent index, as the reference does by default.
        borrow: the arrays stay valid and unchanged until the request is placed
        (the server keeps references to them until its result is taken), so a
        queued request is neither copied nor checked on the host; its CSR is
        checked on the device when it is placed."""
        keep = []
        d = scenario_desc(offsets, indices, state, seed, beta, gamma, self.variant, horizon, lids, codes,
                          True, keep)
        if borrow:
            d.flags |= N.SG_REQ_BORROW
        rid = ctypes.c_int64()
        self._ck(self._lib.sg_server_submit(self._h, ctypes.byref(d), ctypes.byref(rid)))
        self._n[rid.value] = d.n_agents
        if borrow:
            self._borrowed[rid.value] = keep
        return rid.value

    def step(self, nticks):
        done = ctypes.c_int32()
        self._ck(self._lib.sg_server_step(self._h, int(nticks), ctypes.byref(done)))
        return done.value

    def poll(self, rid):
        st, tk = ctypes.c_int32(), ctypes.c_int64()
        self._ck(self._lib.sg_server_poll(self._h, rid, ctypes.byref(st), ctypes.byref(tk)))
        return st.value, tk.value

    def take_result(self, rid):
        out = np.empty(self._n.pop(rid), dtype=np.int32)
        self._borrowed.pop(rid, None)
        self._ck(self._lib.sg_server_take_result(self._h, rid, ctypes.c_void_p(out.ctypes.data), out.size))
        return out

    def counts(self):
        q, r, d, b = (ctypes.c_int64() for _ in range(4))
        self._ck(self._lib.sg_server_counts(self._h, ctypes.byref(q), ctypes.byref(r), ctypes.byref(d),
                                            ctypes.byref(b)))
        return {"queued": q.value, "resident": r.value, "done": d.value, "resident_bytes": b.value}

    def set_tune(self, strategy="count", blocks_per_sm=16, thread_row=32, mega_row=2048, count_flavour=272):
        t = N.Tune(STRATEGIES[strategy], blocks_per_sm, thread_row, mega_row, count_flavour, 0.0)
        self._ck(self._lib.sg_server_set_tune(self._h, ctypes.byref(t)))


def serve_stream(server, requests, arrivals, chunk=8, keep_results=True, clock=time.perf_counter, borrow=False):
    """Submits requests[i] (dict of Server.submit kwargs) at arrivals[i] seconds
    after the start, steps the server by `chunk` ticks while work remains, and
    returns per-request latency (completion - arrival, seconds), results and totals
    (with the host time spent in submit and in step). keep_results: keep every
    result (True), none (False) or those whose index is in the given set.
    borrow: submit with borrow=True (the requests' arrays outlive the stream)."""
    order = np.argsort(arrivals, kind="stable")
    t0 = clock()
    rid_of, req_of = {}, {}
    done_at = {}
    results = {}
    nxt = 0
    pending = 0
    agent_ticks = 0
    t_submit = t_step = 0.0
    while nxt < len(order) or pending:
        now = clock() - t0
        while nxt < len(order) and arrivals[order[nxt]] <= now:
            i = int(order[nxt])
            ts = clock()
            rid = server.submit(**requests[i], borrow=True) if borrow else server.submit(**requests[i])
            t_submit += clock() - ts
            rid_of[i] = rid
            req_of[rid] = i
            pending += 1
            nxt += 1
        if not pending:
            # idle until the next arrival
            wait = arrivals[order[nxt]] - (clock() - t0)
            if wait > 0:
                time.sleep(min(wait, 0.01))
            continue
        ts = clock()
        finished = server.step(chunk)
        t_step += clock() - ts
        if finished:
            tnow = clock() - t0
            for rid in list(req_of):
                st, _ = server.poll(rid)
                if st in (N.SG_REQ_DONE, N.SG_REQ_FAILED):
                    i = req_of.pop(rid)
                    done_at[i] = tnow
                    res = server.take_result(rid)  # raises for a request refused at placement
                    if keep_results is True or (keep_results and i in keep_results):
                        results[i] = res
                    agent_ticks += res.size * int(requests[i]["horizon"])
                    pending -= 1
    wall = clock() - t0
    lat = np.array([done_at[i] - arrivals[i] for i in range(len(requests))])
    return {"latency_s": lat, "results": results, "wall_s": wall, "agent_ticks": agent_ticks,
            "submit_s": t_submit, "step_s": t_step}
