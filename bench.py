"""Benchmark of the per-tick SIR agent step on one GB300.

Workload (default): 10,000,000 agents on a Barabasi-Albert graph (m=4, seed 1,
about 8.0e7 directed CSR entries), relabelled by a seeded 64-way locality
partition (logical ids keep the original agent ids as RNG keys), 0.1 %
initially infected, beta=0.03, gamma=0.07, per-infected-neighbour SIR, 200
ticks. One step = one simulate(200) from the initial state.

  value : agent-ticks/s with inputs resident in HBM (device timed, CUDA events)
  e2e   : the same through the C ABI with host buffers (pinned): the initial
          state is copied in and the final state read back every step
  roofline : the dominant kernel's algorithmic bytes / its CUDA-event duration
  parity_vs_oracle : every strategy's final state and per-tick S, I, R, E_S
                 equal the oracle's run of the same 200 ticks
  cpu_baseline : that oracle run (the C port of the reference tick, OpenMP on
                 all host cores), one whole simulate(200), timed

`--impl reference` times the reference's CPU implementation of this path. The
reference runs its step only as a CuPy GPU kernel (its use_gpu=False flag is
ignored), so its CPU implementation here is the C restatement of its tick in
oracle/ on all host cores, on the same workload: whole 200-tick runs, the
input built by oracle/ alone (no engine library in that process).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_AGENTS = 10_000_000
BA_M = 4
TICKS = 200
BETA, GAMMA = 0.03, 0.07
INFECTED_FRAC = 0.001
SEED = 1
# DRAM traffic per launch of the dominant kernel (dram__bytes_read.sum +
# dram__bytes_write.sum, averaged over all 200 ticks of one simulate, L2 contents kept
# from launch to launch as in the run), from
#   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum \
#       --cache-control none --clock-control none -k regex:sir_count_hybrid -c 200 \
#       --csv --log-file dram.csv python bench.py --profile-case
# keyed by (strategy, agents, kernel); the count step is one launch per tick (class
# sweep or flat draws). Re-measure when a kernel changes.
MEASURED_TRAFFIC = {("count", 10_000_000, "sir_count_step"): 27.999e6}
PARTS = 64
CODES = (1, 2, 3)
WORKLOAD = ("SIR per-infected-neighbour (salt 2+j trials), BA n=%d m=4 seed 1, 64-way locality relabel, "
            "0.1%% infected, beta 0.03 gamma 0.07, 200 ticks")


def _env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def build_workload(n=N_AGENTS):
    from sagesim_gb300 import graphs

    off, idx = graphs.barabasi_albert(n, BA_M, SEED)
    perm, _ = graphs.partition_relabel(off, idx, PARTS, SEED)
    roff, ridx = graphs.permute_csr(off, idx, perm)
    st = np.full(n, CODES[0], dtype=np.int32)
    st[graphs.initial_infected(n, INFECTED_FRAC, SEED)] = CODES[1]
    rst = np.empty_like(st)
    rst[perm] = st
    lids = np.empty(n, dtype=np.int64)
    lids[perm] = np.arange(n, dtype=np.int64)  # logical id = original agent id
    return roff, ridx, rst, lids


def build_reference_workload(n=N_AGENTS):
    """The same workload for the CPU reference arm, built by oracle/ only: the
    Barabasi-Albert graph in generation order with logical id = agent id, which
    is how SAGESim runs it on one rank (it has no locality relabel). The
    engine's relabelled run keys every draw on the same logical ids, so both
    give the same trajectory (agents permuted)."""
    from oracle import oracle

    off, idx = oracle.barabasi_albert(n, BA_M, SEED)
    st = np.full(n, CODES[0], dtype=np.int32)
    st[oracle.initial_infected(n, INFECTED_FRAC, SEED)] = CODES[1]
    return off, idx, st


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self._t.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ensemble_specs(count=512, seed=3):
    """Config 4: n log-uniform in [1e3, 1e6]; ER (mean degree 8), BA (m 3..6) or
    WS (k 6..12, p 0.1); beta U[0.01, 0.1], gamma U[0.05, 0.2]; 0.5 % infected."""
    rng = np.random.default_rng(seed)
    specs, params = [], []
    for s_ in range(count):
        n = int(10 ** rng.uniform(3, 6))
        kind = int(rng.integers(0, 3))
        gseed = int(rng.integers(0, 2**62))
        if kind == 0:
            specs.append(("er", n, 8.0 / (n - 1), gseed))
        elif kind == 1:
            specs.append(("ba", n, int(rng.integers(3, 7)), gseed))
        else:
            specs.append(("ws", n, int(rng.choice([6, 8, 10, 12])), 0.1, gseed))
        params.append(dict(seed=int(rng.integers(0, 2**31)), beta=float(rng.uniform(0.01, 0.1)),
                           gamma=float(rng.uniform(0.05, 0.2)), infected_seed=int(rng.integers(0, 2**31))))
    return specs, params


def max_over_ranks(value, dist=None, device=None):
    """The largest of every rank's value: a job of replicas ends with its slowest
    one (identity on a single process)."""
    if dist is None:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank, world, seconds):
    """Whole-job rate of `world` independent replicas that each process
    units_per_rank units, the slowest in `seconds`."""
    return world * units_per_rank / seconds


def pinned(a):
    """A page-locked host copy of numpy array `a` (through torch's pinned allocator)."""
    import torch

    t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    out = t.numpy()
    assert out.base is not None  # the view keeps the pinned tensor alive
    return out


def initial_state(n, frac, seed):
    st = np.full(n, CODES[0], dtype=np.int32)
    k = max(1, int(round(frac * n)))
    st[np.random.default_rng(seed).choice(n, size=k, replace=False)] = CODES[1]
    return st


def ensemble_section(stream, steps, device=0, ticks=365):
    """Batched ensemble vs the same scenarios run one after another on the plain
    engine (device time of the simulate() calls only), bit-exact compared."""
    import torch

    from sagesim_gb300 import Engine, graphs
    from sagesim_gb300.batch import Batch

    specs, params = ensemble_specs()
    t0 = time.perf_counter()
    gs = graphs.generate_many(specs)
    gen_s = time.perf_counter() - t0
    states = [initial_state(off.size - 1, 0.005, p["infected_seed"]) for (off, _), p in zip(gs, params)]
    agents = sum(off.size - 1 for off, _ in gs)
    nnz = sum(int(off[-1]) for off, _ in gs)
    with torch.cuda.stream(stream):
        b = Batch(device=device, stream=stream.cuda_stream)
        sids = [b.add_scenario(off, idx, st, p["seed"], p["beta"], p["gamma"], variant="B", horizon=ticks)
                for (off, idx), st, p in zip(gs, states, params)]
        b.commit()
        b.snapshot()
        tune = b.tune(4)
        b.restore()
        b.run(ticks)  # warm-up (graph capture)
        b.restore()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        stream.synchronize()
        ms_total = 0.0
        for _ in range(steps):
            b.restore()
            ev0.record(stream)
            b.run(ticks)
            ev1.record(stream)
            stream.synchronize()
            ms_total += ev0.elapsed_time(ev1)
        batched_ms = ms_total / steps
        finals = [b.get_state(sid) for sid in sids]
        info = b.info()
        b.close()
        # the same scenarios on the plain engine, one after another
        plain_ms = 0.0
        mismatches = 0
        for (off, idx), st, p, fin in zip(gs, states, params, finals):
            e = Engine(device=device, stream=stream.cuda_stream)
            e.set_graph(off, idx, symmetric=True)
            e.set_seed(p["seed"])
            pr = e.add_property("state", np.int32, init=st)
            e.add_sir(pr, p["beta"], p["gamma"], variant="B", strategy="count", codes=CODES)
            e.snapshot()
            e.run_async(0, ticks)  # warm-up (graph capture)
            e.restore()
            stream.synchronize()
            ev0.record(stream)
            e.run_async(0, ticks)
            ev1.record(stream)
            stream.synchronize()
            plain_ms += ev0.elapsed_time(ev1)
            mismatches += int(not np.array_equal(e.get_property(pr), fin))
            e.close()
    # checker: a dozen scenarios, the two largest among them, against the oracle
    from oracle import oracle

    by_size = np.argsort([off.size for off, _ in gs], kind="stable")
    pick = set(int(k) for k in by_size[-2:])
    pick |= set(int(k) for k in np.random.default_rng(3).choice(len(gs), 10, replace=False))
    oracle_ok = 0
    for k in sorted(pick):
        (off, idx), p = gs[k], params[k]
        want, _, _ = oracle.sir_run(2, off, idx, states[k], p["seed"], 0, ticks, p["beta"], p["gamma"], CODES)
        oracle_ok += int(np.array_equal(finals[k], want))
    return {"workload": "512 SIR scenarios (ER/BA/WS, n log-uniform 1e3..1e6, seed 3), 365 ticks",
            "oracle_checked": {"scenarios": len(pick), "bit_exact": oracle_ok,
                               "largest_agents": int(gs[int(by_size[-1])][0].size - 1)},
            "scenarios": len(gs), "agents": agents, "nnz": nnz, "graph_gen_s": gen_s,
            "batched_agent_ticks_per_s": agents * ticks / (batched_ms / 1e3), "batched_ms": batched_ms,
            "plain_sequential_agent_ticks_per_s": agents * ticks / (plain_ms / 1e3),
            "plain_sequential_ms": plain_ms, "speedup": plain_ms / batched_ms,
            "tune": tune, "bit_exact_scenarios": len(gs) - mismatches, "device_bytes": info["device_bytes"]}


def opinion_section(stream, steps, device=0, peak=None, n=2_000_000, ticks=500):
    """Config 3: opinion dynamics on WS n=2e6 k=10 p=0.1 (seed 2, ordered rows),
    opinions U[0,1), float32[8] weights N(0,1), noise sigma 0.01, 500 ticks.

    Returns agent-ticks/s (device, graph replay), the opinion kernel's roofline on
    its algorithmic bytes per tick (4N opinion read + 4N write + 32N weights + 4N
    row offsets + 4E neighbour indices, neighbour opinions counted as reuse), the
    largest relative difference from the oracle after 20 ticks, and the oracle's
    rate on the host cores."""
    import torch

    from oracle import oracle
    from sagesim_gb300 import Engine, graphs

    off, idx = graphs.watts_strogatz(n, 10, 0.1, 2)
    rng = np.random.default_rng(2)
    x0 = rng.random(n, dtype=np.float32)
    w = rng.standard_normal((n, 8), dtype=np.float32)
    nnz = int(off[-1])
    with torch.cuda.stream(stream):
        eng = Engine(device=device, stream=stream.cuda_stream)
        eng.set_graph(off, idx, ordered=True)
        eng.set_seed(2)
        px = eng.add_property("opinion", np.float32, init=x0)
        pw = eng.add_property("weights", np.float32, width=8, init=w)
        eng.add_opinion(px, pw, 0.01)
        eng.snapshot()
        eng.run(0, 20, stats=False)
        got20 = eng.get_property(px)
        for _ in range(2):
            eng.restore()
            eng.run_async(0, ticks, use_graph=True)
        stream.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            eng.restore()
            eng.run_async(0, ticks, use_graph=True)
        ev1.record(stream)
        stream.synchronize()
        ms = ev0.elapsed_time(ev1) / steps
        eng.restore()
        eng.profile(True)
        eng.run(0, ticks, stats=False)
        rep = eng.profile_report()
        eng.profile(False)
        eng.close()
    want20, _ = oracle.opinion_run(off, idx, w, x0, 2, 0, 20, 0.01)
    rel = np.abs(got20 - want20) / np.maximum(np.abs(want20), 1e-30)
    rel = np.where(np.abs(got20 - want20) <= 1e-12, 0.0, rel)
    t0 = time.perf_counter()
    oracle.opinion_run(off, idx, w, x0, 2, 0, 20, 0.01)
    cpu_dt = time.perf_counter() - t0
    launches, k_ms = rep.get("opinion", (ticks, ms))
    per_launch_s = k_ms / max(launches, 1) / 1e3
    alg = 4.0 * n + 4.0 * n + 32.0 * n + 4.0 * n + 4.0 * nnz
    achieved = alg / per_launch_s / 1e9
    out = {"workload": "opinion, WS n=2e6 k=10 p=0.1 seed 2 (ordered), float32[8] weights, sigma 0.01, "
                       "%d ticks" % ticks,
           "agent_ticks_per_s": n * ticks / (ms / 1e3), "ms_per_step": ms, "nnz": nnz,
           "max_rel_diff_vs_oracle_20_ticks": float(rel.max()), "within_1e-6": bool(rel.max() <= 1e-6),
           "roofline": {"bound": "hbm", "achieved": achieved, "unit": "GB/s", "per_launch_us": per_launch_s * 1e6,
                        "alg_bytes_per_launch": alg},
           "cpu_port_agent_ticks_per_s": n * 20 / cpu_dt, "cpu_cores": oracle.max_threads()}
    if peak:
        out["roofline"]["peak"] = peak
        out["roofline"]["frac"] = achieved / peak
    return out


def serving_section(stream, device=0, n_requests=1000, n_graphs=64):
    """Config 5: a stream of n_requests requests, Poisson arrivals at 200 req/s
    (seed 4), n log-uniform in [1e4, 5e6], BA or ER with mean degree 4..16,
    horizons U{50..365}, 150 GB admission budget. Graph structures come from a
    pool of n_graphs generated graphs; every fourth structure is relabelled by
    a 16-way locality partition and its requests carry logical ids (the
    original agent ids), so they must reproduce the run in the original order.
    Every request has its own seed, beta, gamma, initial infections and
    horizon. The Poisson stream gives the latencies (its throughput is bounded
    by the arrival rate); the same requests all arriving at once give the
    served form's capacity (burst_*). Every request's result is compared with
    its run on the plain engine, and a sample (relabelled ones among them) with
    the oracle run on the graph in its original order."""
    import torch

    from sagesim_gb300 import Engine, graphs
    from sagesim_gb300.serve import Server, serve_stream

    rng = np.random.default_rng(4)
    specs = []
    for g in range(n_graphs):
        n = int(10 ** rng.uniform(4, np.log10(5e6)))
        deg = float(rng.uniform(4, 16))
        if rng.random() < 0.5:
            specs.append(("ba", n, max(2, int(round(deg / 2))), int(rng.integers(0, 2**62))))
        else:
            specs.append(("er", n, deg / (n - 1), int(rng.integers(0, 2**62))))
    t0 = time.perf_counter()
    base = graphs.generate_many(specs)
    pool = []  # (offsets, indices, perm or None, lids or None) as requests see them
    for g, (off, idx) in enumerate(base):
        if g % 4 == 1:
            perm, _ = graphs.partition_relabel(off, idx, 16, g)
            roff, ridx = graphs.permute_csr(off, idx, perm)
            lids = np.empty(off.size - 1, dtype=np.int64)
            lids[perm] = np.arange(off.size - 1, dtype=np.int64)
            pool.append((roff, ridx, perm, lids))
        else:
            pool.append((off, idx, None, None))
    gen_s = time.perf_counter() - t0
    # requests arrive in page-locked host memory (a server's receive buffers), for
    # the served and the plain runs alike
    pool = [tuple(None if a is None else pinned(a) for a in entry) for entry in pool]
    arrivals = np.cumsum(rng.exponential(1.0 / 200.0, size=n_requests))
    reqs, gof, st_orig = [], [], []
    for i in range(n_requests):
        g = int(rng.integers(0, n_graphs))
        off, idx, perm, lids = pool[g]
        n = off.size - 1
        st = initial_state(n, 0.005, int(rng.integers(0, 2**31)))  # in the original order
        rst = st
        if perm is not None:
            rst = np.empty_like(st)
            rst[perm] = st
        gof.append(g)
        st_orig.append(st)
        reqs.append(dict(offsets=off, indices=idx, state=pinned(rst), seed=int(rng.integers(0, 2**31)),
                         beta=float(rng.uniform(0.01, 0.1)), gamma=float(rng.uniform(0.05, 0.2)),
                         horizon=int(rng.integers(50, 366)), lids=lids))
    with torch.cuda.stream(stream):
        srv = Server(budget_bytes=150 * 10**9, agent_slots=400_000_000, edge_slots=2_100_000_000,
                     max_resident=4096, variant="B", device=device, stream=stream.cuda_stream)
        out = serve_stream(srv, reqs, arrivals, chunk=8, borrow=True)
        srv.close()
        # capacity: the same requests all arriving at once
        srv = Server(budget_bytes=150 * 10**9, agent_slots=400_000_000, edge_slots=2_100_000_000,
                     max_resident=4096, variant="B", device=device, stream=stream.cuda_stream)
        burst = serve_stream(srv, reqs, np.zeros(n_requests), chunk=8, keep_results=False, borrow=True)
        srv.close()
        # plain sequential: each request alone on its own plain engine, as a user
        # of the engine API would run it: uploads, simulate and result read-back
        # (wall time), and the device time of its simulate alone
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        plain_ms, mismatches = 0.0, 0
        t0 = time.perf_counter()
        for i, r in enumerate(reqs):
            e = Engine(device=device, stream=stream.cuda_stream)
            e.set_graph(r["offsets"], r["indices"], symmetric=True)
            if r["lids"] is not None:
                e.set_logical_ids(r["lids"])
            e.set_seed(r["seed"])
            pr = e.add_property("state", np.int32, init=r["state"])
            e.add_sir(pr, r["beta"], r["gamma"], variant="B", strategy="count", codes=CODES)
            ev0.record(stream)
            e.run_async(0, r["horizon"], use_graph=False)
            ev1.record(stream)
            res = e.get_property(pr)
            plain_ms += ev0.elapsed_time(ev1)
            mismatches += int(not np.array_equal(res, out["results"][i]))
            e.close()
        plain_wall = time.perf_counter() - t0
    # checker: a sample of requests against the oracle on the graph in its original
    # order (no logical ids); relabelled results are mapped back through perm
    from oracle import oracle

    sample = [i for i in range(n_requests) if pool[gof[i]][2] is not None][:4]
    sample += [i for i in range(n_requests) if pool[gof[i]][2] is None][:4]
    oracle_ok = 0
    for i in sample:
        off, idx = base[gof[i]]
        perm = pool[gof[i]][2]
        r = reqs[i]
        want, _, _ = oracle.sir_run(2, off, idx, st_orig[i], r["seed"], 0, r["horizon"], r["beta"], r["gamma"],
                                    CODES)
        got = out["results"][i] if perm is None else out["results"][i][perm]
        oracle_ok += int(np.array_equal(got, want))
    lat = out["latency_s"]
    agent_ticks = out["agent_ticks"]
    return {"workload": "%d SIR requests, Poisson 200 req/s (seed 4), n 1e4..5e6 log-uniform, BA/ER "
                        "mean degree 4..16, horizons 50..365, 150 GB budget, %d graph structures (every "
                        "fourth relabelled, its requests carrying logical ids)" % (n_requests, n_graphs),
            "requests": n_requests, "with_logical_ids": int(sum(r["lids"] is not None for r in reqs)),
            "graph_gen_s": gen_s,
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "served_agent_ticks_per_s": agent_ticks / out["wall_s"], "wall_s": out["wall_s"],
            "arrival_span_s": float(arrivals[-1]), "submit_s": out["submit_s"], "step_s": out["step_s"],
            "burst_agent_ticks_per_s": burst["agent_ticks"] / burst["wall_s"], "burst_wall_s": burst["wall_s"],
            "burst_submit_s": burst["submit_s"], "burst_step_s": burst["step_s"],
            "burst_step_agent_ticks_per_s": burst["agent_ticks"] / burst["step_s"],
            "burst_p50_latency_s": float(np.percentile(burst["latency_s"], 50)),
            "burst_p99_latency_s": float(np.percentile(burst["latency_s"], 99)),
            "plain_sequential_agent_ticks_per_s": agent_ticks / (plain_ms / 1e3),
            "plain_sequential_wall_s": plain_wall,
            "plain_sequential_wall_agent_ticks_per_s": agent_ticks / plain_wall,
            "burst_vs_plain_over_wall": (burst["agent_ticks"] / burst["wall_s"]) / (agent_ticks / plain_wall),
            "bit_exact_requests": n_requests - mismatches,
            "oracle_checked": {"requests": len(sample), "bit_exact": oracle_ok}}


def algorithmic_bytes(kernel, n, st0, tick_stats, active, flat=True):
    """Compulsory DRAM bytes per launch of `kernel`, per tick of the run (int32 state).

    sir_pull          12 B per agent (state read/write, row offset) + 4 B per CSR
                      entry of the tick-start susceptible agents (E_S)
    sir_count_step    class sweep ticks: 1 B class read per agent,
                      1/8 B activity bit per agent, 4 B RNG key per candidate
                      (active[] = infected agents + susceptible agents with the
                      bit set), 4 B count per susceptible candidate, 9 B per
                      transition (state write, class write, change entry);
                      busy ticks (hybrid step): with flat draws (the default), 1 B
                      class read per agent, 4 B count per tick-start S agent, 4 B
                      RNG key per candidate (at most the tick-start I and S
                      agents: counted as all of them), 9 B per transition; with
                      the loop form, 4 B state read per agent, 4 B count read per
                      tick-start S agent, 8 B per transition
    frontier_step     20 B per active agent (list, state, count, mark, next list)
                      + 8 B per transition
    *_scatter         8 B per transition (change entry, transpose offsets) + 12 B
                      per transpose entry of a changed agent (index read, count
                      read-modify-write); recoveries' degree sum is estimated from
                      the infections' mean degree
    """
    S = tick_stats[:, 0].astype(np.float64)
    R = tick_stats[:, 2].astype(np.float64)
    S_start = np.concatenate([[float((st0 == CODES[0]).sum())], S[:-1]])
    R_start = np.concatenate([[float((st0 == CODES[2]).sum())], R[:-1]])
    inf = S_start - S
    rec = R - R_start
    changes = inf + rec
    E_S = tick_stats[:, 3].astype(np.float64)
    deg_inf = E_S - np.concatenate([E_S[1:], [E_S[-1]]])
    mean_deg = deg_inf.sum() / max(inf.sum(), 1.0)
    deg_changes = deg_inf + rec * mean_deg
    if kernel == "sir_pull":
        return 12.0 * n + 4.0 + 4.0 * E_S
    if kernel == "sir_count_step":
        # ticks the hybrid step gave to the loop form report every agent as processed
        I = tick_stats[:, 1].astype(np.float64)
        I_start = np.concatenate([[float((st0 == CODES[1]).sum())], I[:-1]])
        sweep = 1.125 * n + 4.0 * active + 4.0 * np.maximum(active - I_start, 0.0) + 9.0 * changes
        if flat:
            busy = 1.0 * n + 4.0 * S_start + 4.0 * (I_start + S_start) + 9.0 * changes
        else:
            busy = 4.0 * n + 4.0 * S_start + 8.0 * changes
        return np.where(active >= n, busy, sweep)
    if kernel == "frontier_step":
        return 20.0 * active + 8.0 * changes
    if kernel in ("sir_count_scatter", "frontier_scatter"):
        return 8.0 * changes + 12.0 * deg_changes
    # sir_count_init, once per run: state of every agent, offsets, CSR rows and
    # count write of the susceptible agents
    return np.array([4.0 * n + 12.0 * S_start[0] + 4.0 * E_S[0]])


def run_reference(args):
    """The reference arm: whole 200-tick runs of the C port of the reference
    tick (oracle/, OpenMP on every host core), input built by oracle/ only.
    One step = one simulate(200) from the initial state, timed on the host."""
    rank = _env_int("RANK", 0)
    if rank != 0:
        return
    from oracle import oracle

    off, idx, st = build_reference_workload()
    used = oracle.max_threads()
    for _ in range(max(args.warmup, 0)):
        oracle.sir_run(2, off, idx, st, SEED, 0, TICKS, BETA, GAMMA, CODES)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.sir_run(2, off, idx, st, SEED, 0, TICKS, BETA, GAMMA, CODES)
        times.append(time.perf_counter() - t0)
    s_step = float(np.sum(times)) / max(len(times), 1)
    v = N_AGENTS * TICKS / s_step
    line = {
        "impl": "reference", "metric": "SIR agent-ticks/s (BA 1e7, 200-tick simulate)", "value": v,
        "unit": "agent-ticks/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": s_step * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": WORKLOAD % N_AGENTS,
                   "order": "graph in generation order, logical id = agent id (the relabel is the engine's "
                            "layout; same trajectory)"},
        "cpu_baseline": {"value": v, "unit": "agent-ticks/s", "cores": used, "kind": "port",
                         "sample": "whole 200-tick simulate per step, %d steps (C port of the reference "
                                   "tick, OpenMP)" % args.steps},
        "e2e": {"value": v, "unit": "agent-ticks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def profile_case(args):
    """One simulate(200) through the engine, no timing: the command ncu wraps."""
    from sagesim_gb300 import Engine

    off, idx, st0, lids = build_workload(args.agents)
    with Engine() as eng:
        eng.set_graph(off, idx, symmetric=True)
        eng.set_logical_ids(lids)
        eng.set_seed(SEED)
        prop = eng.add_property("state", np.int32, init=st0)
        eng.add_sir(prop, BETA, GAMMA, variant="B", strategy=args.strategy, codes=CODES)
        if args.flavour >= 0:
            eng.set_tune(blocks_per_sm=args.bps, count_flavour=args.flavour)
        stats, _ = eng.run(0, TICKS, stats=args.profile_stats)
        active = eng.last_run_active(TICKS)
        final = eng.get_property(prop)
    print("profile case done: %d agents, %d ticks, %d infected or recovered at the end"
          % (args.agents, TICKS, int((final != CODES[0]).sum())))
    if args.profile_stats:
        for t in (0, 5, 10, 15, 20, 25, 30, 40, 60, 100, 150, 199):
            print("tick %3d  S %9d  I %9d  R %9d  E_S %10d  processed %9d" % ((t,) + tuple(stats[t]) + (active[t],)))


def profile_opinion(args):
    """Thirty ticks of the opinion workload (WS n=2e6), no timing: the command ncu wraps."""
    from sagesim_gb300 import Engine, graphs

    n = 2_000_000
    off, idx = graphs.watts_strogatz(n, 10, 0.1, 2)
    rng = np.random.default_rng(2)
    x0 = rng.random(n, dtype=np.float32)
    w = rng.standard_normal((n, 8), dtype=np.float32)
    with Engine() as eng:
        eng.set_graph(off, idx, ordered=True)
        eng.set_seed(2)
        px = eng.add_property("opinion", np.float32, init=x0)
        pw = eng.add_property("weights", np.float32, width=8, init=w)
        eng.add_opinion(px, pw, 0.01)
        eng.run(0, 30, stats=False)
        out = eng.get_property(px)
    print("opinion profile case done: %d agents, 30 ticks, mean opinion %.6f" % (n, float(out.mean())))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--strategy", default="count", choices=["count", "frontier", "pull"])
    ap.add_argument("--agents", type=int, default=N_AGENTS)
    ap.add_argument("--profile-stats", action="store_true",
                    help="with --profile-case: collect and print per-tick S/I/R/E_S")
    ap.add_argument("--flavour", type=int, default=-1, help="count-step flavour for --profile-case")
    ap.add_argument("--bps", type=int, default=16, help="blocks per SM for --profile-case")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the ensemble and serving sections")
    ap.add_argument("--profile-opinion", action="store_true",
                    help="run 30 ticks of the opinion workload and exit (for ncu captures)")
    ap.add_argument("--profile-case", action="store_true",
                    help="run one simulate(200) of --strategy and exit (for ncu captures)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.profile_case:
        profile_case(args)
        return
    if args.profile_opinion:
        profile_opinion(args)
        return

    import torch

    from sagesim_gb300 import Engine

    world = _env_int("WORLD_SIZE", 1)
    rank = _env_int("RANK", 0)
    local = _env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    n = args.agents
    off, idx, st0, lids = build_workload(n)
    nnz = int(off[-1])
    stream = torch.cuda.Stream(device=local)
    peak, peak_kind = peaks()

    def measure(strategy, steps, warmup):
        """Times `steps` simulate(200) calls of one strategy on its own engine."""
        with torch.cuda.stream(stream):
            eng = Engine(device=local, stream=stream.cuda_stream)
            eng.set_graph(off, idx, symmetric=True)
            eng.set_logical_ids(lids)
            eng.set_seed(SEED)
            prop = eng.add_property("state", np.int32, init=st0)
            eng.add_sir(prop, BETA, GAMMA, variant="B", strategy=strategy, codes=CODES)
            eng.snapshot()
            # trajectory statistics (untimed): E_S per tick for edge-visits/s and bytes
            tick_stats, totals = eng.run(0, TICKS, stats=True)
            run_launches = int(totals.kernel_launches)
            active = eng.last_run_active(TICKS).astype(np.float64)
            final = eng.get_property(prop)
            eng.restore()

            def step():
                eng.restore()
                eng.run_async(0, TICKS, use_graph=True)

            for _ in range(max(warmup, 3)):
                step()
            stream.synchronize()
            if dist:
                dist.barrier()
            clk = ClockSampler(local)
            clk.start()
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            stream.synchronize()
            ev0.record(stream)
            for _ in range(steps):
                step()
            ev1.record(stream)
            stream.synchronize()
            clocks = clk.stop()
            ms = max_over_ranks(ev0.elapsed_time(ev1), dist, "cuda")
            ms_step = ms / steps

            # end to end through the C ABI with pinned host buffers
            h_in = torch.from_numpy(st0).pin_memory()
            h_out = torch.empty(n, dtype=torch.int32).pin_memory()
            for _ in range(2):
                eng.set_property_ptr(prop, h_in.data_ptr(), 0, n)
                eng.run_async(0, TICKS, use_graph=True)
                eng.get_property_ptr(prop, h_out.data_ptr(), 0, n)
            t0 = time.perf_counter()
            for _ in range(steps):
                eng.set_property_ptr(prop, h_in.data_ptr(), 0, n)
                eng.run_async(0, TICKS, use_graph=True)
                eng.get_property_ptr(prop, h_out.data_ptr(), 0, n)
            e2e_s = max_over_ranks((time.perf_counter() - t0) / steps, dist, "cuda")
            if not np.array_equal(h_out.numpy(), final):
                raise RuntimeError("end-to-end result differs from the device-resident run")

            # dominant kernel: per-launch CUDA events (separate, profiled run)
            eng.restore()
            eng.profile(True)
            eng.run(0, TICKS, stats=False)
            rep = eng.profile_report()
            eng.profile(False)
            eng.close()
        dom_name, (dom_launches, dom_ms) = max(rep.items(), key=lambda kv: kv[1][1])
        E_S = tick_stats[:, 3].astype(np.float64)
        per_launch_ms = dom_ms / max(dom_launches, 1)
        # the contract's algorithmic bytes: one SIR tick of the reference's scan,
        # 12 N + 4 + 4 E_S (state read and write and row offset per agent, one CSR
        # index per neighbour of each susceptible agent); one launch of the
        # dominant step kernel advances one tick
        ref_bytes = float((12.0 * n + 4.0 + 4.0 * E_S).mean())
        achieved = ref_bytes / (per_launch_ms / 1e3) / 1e9
        # the kernel's own compulsory bytes (it does not scan rows; see algorithmic_bytes)
        own = float(algorithmic_bytes(dom_name, n, st0, tick_stats, active).mean())
        own_achieved = own / (per_launch_ms / 1e3) / 1e9
        traffic = MEASURED_TRAFFIC.get((strategy, n, dom_name))
        return {
            "value": replica_rate(n * TICKS, world, ms_step / 1e3), "ms_per_step": ms_step,
            "e2e": replica_rate(n * TICKS, world, e2e_s),
            "edge_visits_per_s": replica_rate(float(E_S.sum()), world, ms_step / 1e3),
            "launches": steps * run_launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "kernel": dom_name,
                         "peak_source": peak_kind, "per_launch_us": per_launch_ms * 1e3,
                         "alg_bytes_per_launch": ref_bytes,
                         "alg_bytes": "12N + 4 + 4 E_S per tick (one tick of the reference scan)",
                         "kernel_bytes_per_launch": own, "kernel_achieved": own_achieved,
                         "kernel_frac": own_achieved / peak},
            "kernels": {k: {"launches": v[0], "total_ms": v[1]} for k, v in rep.items()},
            "clocks": clocks, "final": final, "tick_stats": tick_stats,
        }

    results = {}
    for strategy in [args.strategy] + [s for s in ("count", "frontier", "pull") if s != args.strategy]:
        results[strategy] = measure(strategy, args.steps, args.warmup)
    head = results[args.strategy]

    # checker: the oracle runs the same 200 ticks on the host cores (rank 0); every
    # strategy's final state and per-tick S, I, R, E_S must equal it. The run is
    # timed: it is the CPU baseline (one whole simulate(200)).
    parity, cpu = None, None
    if rank == 0:
        from oracle import oracle

        t0 = time.perf_counter()
        want, want_stats, _ = oracle.sir_run(2, off, idx, st0, SEED, 0, TICKS, BETA, GAMMA, CODES, lids=lids)
        cpu_s = time.perf_counter() - t0
        parity = {s_: {"final_state": bool(np.array_equal(r_["final"], want)),
                       "tick_stats": bool(np.array_equal(r_["tick_stats"], want_stats))}
                  for s_, r_ in results.items()}
        cpu = {"value": n * TICKS / cpu_s, "unit": "agent-ticks/s", "cores": oracle.max_threads(), "kind": "port",
               "sample": "one whole 200-tick simulate of the same workload (%.2f s), C port of the reference "
                         "tick (oracle/), OpenMP" % cpu_s}

    extra = {}
    if rank == 0 and not args.no_extras:
        for name, fn in (("ensemble", lambda: ensemble_section(stream, max(1, min(args.steps, 3)), local)),
                         ("serving", lambda: serving_section(stream, local)),
                         ("opinion", lambda: opinion_section(stream, max(1, min(args.steps, 3)), local, peak))):
            try:
                extra[name] = fn()
            except Exception as exc:  # a failing extra section must not lose the headline line
                extra[name] = {"error": "%s: %s" % (type(exc).__name__, exc)}

    line = {
        "metric": "SIR agent-ticks/s (BA 1e7, 200-tick simulate)", "value": head["value"],
        "unit": "agent-ticks/s", "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3),
        "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": WORKLOAD % n,
                   "strategy": args.strategy, "nnz": nnz,
                   "l2": "inputs larger than L2 (CSR %.0f MB)" % (nnz * 4 / 1e6),
                   "parallelism": "replicas" if world > 1 else "single"},
        "edge_visits_per_s": head["edge_visits_per_s"],
        "e2e": {"value": head["e2e"], "unit": "agent-ticks/s", "h2d_bytes_per_step": 4 * n,
                "d2h_bytes_per_step": 4 * n},
        "gpu_launches": head["launches"],
        "roofline": head["roofline"],
        "kernels": head["kernels"],
        "clocks": head["clocks"],
        "cpu_baseline": cpu,
        "parity_vs_oracle": None if parity is None else all(p["final_state"] and p["tick_stats"]
                                                             for p in parity.values()),
        "parity_detail": parity,
        "strategies": {k: {kk: vv for kk, vv in v.items() if kk not in ("final", "clocks", "tick_stats")}
                       for k, v in results.items()},
    }
    line.update(extra)
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
