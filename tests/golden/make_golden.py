"""Generates the golden fixtures in tests/golden/ from the reference itself.

Runs the unmodified SAGESim package (its Model/Breed/NetworkSpace API, AST
codegen, generated fused kernel and Philox) on one host core, with the CPU
stand-ins of oracle/refshim for cupy, cupyx.jit, mpi4py and awkward. It needs
the reference source tree, so it runs only in the build container:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/reference

Outputs (committed; the tests read only these files):
  philox_vectors.json  rand_uniform_philox / rand_normal values for sampled and
                       edge-case counters
  chain.npz            the reference test chain (tests/test_simulation.py) and
                       stochastic chains, state after every tick
  hier.npz             the hierarchical DiGraph of tests/test_double_buffer.py
                       with its SI (1 tick) and two-priority SIR (2 ticks) runs
  db_priority.json     the double-buffer / no_double_buffer priority results
  er_c1.npz            10,000-agent ER graph (p=0.001, seed 0), 1% infected,
                       beta 0.05, gamma 0.1, Philox seed 0, 100 ticks, for the
                       reference test step (SIR-A) and the per-neighbour step
                       (SIR-B); state after every tick
  ba_breeds.npz        3,000-agent BA graph, two interleaved breeds, explicit
                       logical ids for some agents, SIR-B, 30 ticks
  bla_two_breeds.npz   1,500-agent BA graph, host and site breeds with
                       breed-local arrays (one double-buffered, one written in
                       place at a later priority), both arrays after ticks
                       1, 2, 3, 5, 10, 25
  measures_er.npz      1,500-agent ER graph, SIR with float32[4] protective
                       measures and a float32[5] state-history ring (list
                       properties read through row aliases), 25 ticks
  helpers_er.npz       1,000-agent ER graph, per-neighbour SIR written with the
                       device helpers of sagesim/utils.py, 30 ticks
  fraction_er.npz      1,500-agent ER graph, SIR with two properties that start
                       as whole numbers and are written fractions (immunity,
                       load), 25 ticks
  binding_er.npz       the INTEGRATION.md binding's extraction (GB300SIRModel.
                       gb300_inputs) of a 2,000-agent ER SIR model with some
                       logical ids, and the reference pipeline's own states of
                       that model after every one of 30 ticks
  opinion_ws.npz       2,000-agent WS graph (k=10, p=0.1, seed 2), ordered
                       neighbours, float32 opinion + float32[8] weights, 50 ticks
"""
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def setup_paths(reference):
    sys.dont_write_bytecode = True
    os.environ["SAGESIM_NUM_SMS"] = "1"
    sys.path.insert(0, os.path.join(ROOT, "oracle", "refshim"))
    sys.path.insert(0, reference)
    sys.path.insert(0, os.path.join(reference, "tests"))
    sys.path.insert(0, HERE)
    sys.path.insert(0, ROOT)


def states_by_agent(model, prop):
    """Current values of `prop` indexed by agent id (reads the device buffers)."""
    buf = model._gpu_buffers
    pidx = model._agent_factory._property_name_2_index[prop]
    vals = np.asarray(buf.property_tensors[pidx])[: buf.num_local_agents]
    ids = np.asarray(buf.all_agent_ids_list[: buf.num_local_agents]).astype(np.int64)
    out = np.empty_like(vals)
    out[ids] = vals
    return out


def run_ticks(model, prop, ticks, dtype):
    model._max_blocks_per_sm = 1
    model.setup(use_gpu=True)
    hist = []
    for _ in range(ticks):
        model.simulate(1, sync_workers_every_n_ticks=1)
        hist.append(states_by_agent(model, prop).astype(dtype))
    return np.stack(hist)


def clear_generated():
    for k in [k for k in sys.modules if k.startswith("step_func_code")]:
        del sys.modules[k]


def philox_vectors():
    from sagesim.math_utils import rand_normal, rand_uniform_philox

    rng = np.random.default_rng(123)
    cases = []
    edge = [(0, 0, 0, 0), (42, 0, 0, 1), (2**31 - 1, 2**31 - 1, 2**32 - 1, 7), (-1, 5, 3, 1),
            (7, -3, 11, 2), (1, 4294, 2**33 + 5, 1), (99, 10**9, 123456789, 1000002),
            (5, 0, 0, 73856093), (0, 1, 1, 2**32 + 3), (12345, 365, 999999, 9)]
    for c in edge:
        cases.append(c)
    for _ in range(246):
        cases.append((int(rng.integers(0, 2**31)), int(rng.integers(0, 10**6)),
                      int(rng.integers(0, 2**31)), int(rng.integers(0, 2000))))
    uni = []
    for s, t, l, sa in cases:
        u = rand_uniform_philox(s, t, l, sa)
        k = int(round(u * 8388608.0))
        assert k / 8388608.0 == u
        uni.append([s, t, l, sa, k])
    nor = []
    for s, t, l, sa in cases[:64]:
        nor.append([s, t, l, sa, float(rand_normal(s, t, l, sa))])
    with open(os.path.join(HERE, "philox_vectors.json"), "w") as f:
        json.dump({"uniform_k23": uni, "normal": nor,
                   "note": "k23 = rand_uniform_philox(seed, tick, agent, salt) * 2^23 from the "
                           "reference's sagesim/math_utils.py run on CPU"}, f)


def chains():
    import test_simulation as ts

    out = {}
    m = ts._build_chain_model(10, codefile="step_func_code_gold_chain.py")
    out["det10"] = run_ticks(m, "state", 5, np.int8)
    clear_generated()
    m = ts._build_chain_model(20, p_infection=0.5, p_recovery=0.3, seed=999,
                              codefile="step_func_code_gold_r.py")
    out["sto20_seed999"] = run_ticks(m, "state", 10, np.int8)
    clear_generated()
    for seed in (111, 222):
        m = ts._build_chain_model(50, p_infection=0.3, p_recovery=0.2, seed=seed,
                                  codefile="step_func_code_gold_d%d.py" % seed)
        out["sto50_seed%d" % seed] = run_ticks(m, "state", 20, np.int8)
        clear_generated()
    np.savez_compressed(os.path.join(HERE, "chain.npz"), **out)


def hierarchy():
    import test_double_buffer as tdb

    net = tdb._generate_hierarchical_network(111)
    edges = np.array(list(net.edges), dtype=np.int32)
    out = {"edges": edges}
    m = tdb._create_model_from_network(tdb.SIModel(p_infection=1.0), net)
    out["si_1tick"] = run_ticks(m, "state", 1, np.int8)
    clear_generated()
    m = tdb._create_model_from_network(tdb.SIRModel(p_infection=1.0, p_recovery=1.0), net)
    out["sir_2ticks"] = run_ticks(m, "state", 2, np.int8)
    clear_generated()
    np.savez_compressed(os.path.join(HERE, "hier.npz"), **out)


def db_priority():
    import test_double_buffer as tdb

    res = {}
    for name, cls in (("db", tdb._DBBreed), ("nodb", tdb._NoDBBreed), ("rbw_db", tdb._RBWDBBreed),
                      ("rbw_nodb", tdb._RBWNoDBBreed)):
        m = tdb._make_db_model(cls, "step_func_code_gold_%s.py" % name)
        m._max_blocks_per_sm = 1
        m.setup(use_gpu=True)
        m.simulate(1, sync_workers_every_n_ticks=1)
        res[name] = {"counter": float(m.get_agent_property_value(0, "counter")),
                     "result": float(m.get_agent_property_value(0, "result"))}
        clear_generated()
    with open(os.path.join(HERE, "db_priority.json"), "w") as f:
        json.dump(res, f, indent=1)


def build_sir_model(step, off, idx, state, seed, beta, gamma, breeds=None, lids=None,
                    codefile="step_func_code_gold_sir.py"):
    from sagesim.breed import Breed
    from sagesim.model import Model
    from sagesim.space import NetworkSpace

    model = Model(NetworkSpace(), step_function_file_path=codefile)
    nb = 1 if breeds is None else int(breeds.max()) + 1
    blist = []
    for b in range(nb):
        br = Breed("SIR%d" % b)
        br.register_property("state", 1)
        br.register_step_func(step, os.path.join(HERE, "ref_steps.py"), priority=0)
        model.register_breed(br)
        blist.append(br)
    model.register_global_property("p_infection", beta)
    model.register_global_property("p_recovery", gamma)
    model.set_seed(seed)
    n = off.size - 1
    for i in range(n):
        b = 0 if breeds is None else int(breeds[i])
        model.create_agent_of_breed(blist[b], state=int(state[i]))
    sp = model.get_space()
    for i in range(n):
        for k in range(off[i], off[i + 1]):
            sp.connect_agents(i, int(idx[k]), directed=True)
    if lids is not None:
        for aid, lid in lids.items():
            model.set_agent_logical_id(aid, lid)
    return model


def er_c1():
    import test_simulation as ts
    from ref_steps import sir_per_neighbour_step

    from sagesim_gb300 import graphs

    off, idx = graphs.erdos_renyi(10000, 0.001, 0)
    n = off.size - 1
    st = np.ones(n, dtype=np.int32)
    st[graphs.initial_infected(n, 0.01, 0)] = 2
    out = {"offsets": off, "indices": idx, "state0": st.astype(np.int8)}
    for name, step in (("sir_a", ts.sir_step_func), ("sir_b", sir_per_neighbour_step)):
        m = build_sir_model(step, off, idx, st, 0, 0.05, 0.1, codefile="step_func_code_gold_%s.py" % name)
        out[name] = run_ticks(m, "state", 100, np.int8)
        clear_generated()
    np.savez_compressed(os.path.join(HERE, "er_c1.npz"), **out)


def ba_breeds():
    from ref_steps import sir_per_neighbour_step

    from sagesim_gb300 import graphs

    off, idx = graphs.barabasi_albert(3000, 3, 5)
    n = off.size - 1
    rng = np.random.default_rng(5)
    breeds = (rng.random(n) < 0.4).astype(np.int32)
    st = np.ones(n, dtype=np.int32)
    st[rng.choice(n, 30, replace=False)] = 2
    lid_agents = rng.choice(n, 200, replace=False)
    lids = {int(a): int(v) for a, v in zip(lid_agents, rng.integers(0, 2**24, size=200))}
    m = build_sir_model(sir_per_neighbour_step, off, idx, st, 77, 0.08, 0.1, breeds=breeds, lids=lids,
                        codefile="step_func_code_gold_breeds.py")
    hist = run_ticks(m, "state", 30, np.int8)
    clear_generated()
    la = np.array(sorted(lids.items()), dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "ba_breeds.npz"), offsets=off, indices=idx, breeds=breeds,
                        state0=st.astype(np.int8), lid_pairs=la, history=hist)


def opinion_ws():
    from ref_steps import opinion_step
    from sagesim.breed import Breed
    from sagesim.model import Model
    from sagesim.space import NetworkSpace

    from sagesim_gb300 import graphs

    off, idx = graphs.watts_strogatz(2000, 10, 0.1, 2)
    n = off.size - 1
    rng = np.random.default_rng(2)
    x0 = rng.random(n, dtype=np.float32)
    w = rng.standard_normal((n, 8), dtype=np.float32)
    model = Model(NetworkSpace(ordered=True), step_function_file_path="step_func_code_gold_op.py")
    br = Breed("Opinion")
    br.register_property("opinion", 0.0)
    br.register_property("weights", [0.0] * 8)
    br.register_step_func(opinion_step, os.path.join(HERE, "ref_steps.py"), priority=0)
    model.register_breed(br)
    model.register_global_property("noise_sigma", 0.01)
    model.set_seed(2)
    for i in range(n):
        model.create_agent_of_breed(br, opinion=float(x0[i]), weights=[float(v) for v in w[i]])
    sp = model.get_space()
    for i in range(n):
        for k in range(off[i], off[i + 1]):
            sp.connect_agents(i, int(idx[k]), directed=True)
    hist = run_ticks(model, "opinion", 50, np.float32)
    clear_generated()
    keep = np.array([1, 2, 5, 10, 25, 50])
    np.savez_compressed(os.path.join(HERE, "opinion_ws.npz"), offsets=off, indices=idx, opinion0=x0,
                        weights=w, ticks=keep, history=hist[keep - 1])


def bla_two_breeds():
    from ref_steps import host_step, site_step
    from sagesim.breed import Breed
    from sagesim.model import Model
    from sagesim.space import NetworkSpace

    from sagesim_gb300 import graphs

    off, idx = graphs.barabasi_albert(1500, 3, 8)
    n = off.size - 1
    rng = np.random.default_rng(8)
    breeds = (rng.random(n) < 0.4).astype(np.int32)  # 1 = site
    st = np.ones(n, dtype=np.int32)
    hosts = np.flatnonzero(breeds == 0)
    st[rng.choice(hosts, 20, replace=False)] = 2
    model = Model(NetworkSpace(), step_function_file_path="step_func_code_gold_bla.py")
    host, site = Breed("Host"), Breed("Site")
    for br in (host, site):
        br.register_property("state", 1)
    path = os.path.join(HERE, "ref_steps.py")
    host.register_step_func(host_step, path, priority=0)
    site.register_step_func(site_step, path, priority=1, no_double_buffer=["load"])
    model.register_breed(host)
    model.register_breed(site)
    model.register_global_property("p_infection", 0.04)
    model.register_global_property("p_recovery", 0.1)
    model.register_breed_local_array("health", host, (4,))
    model.register_breed_local_array("load", site, (2, 2))
    model.set_seed(8)
    for i in range(n):
        model.create_agent_of_breed(site if breeds[i] else host, state=int(st[i]))
    sp = model.get_space()
    for i in range(n):
        for k in range(off[i], off[i + 1]):
            sp.connect_agents(i, int(idx[k]), directed=True)
    model._max_blocks_per_sm = 1
    model.setup(use_gpu=True)
    keep = [1, 2, 3, 5, 10, 25]
    health, load = [], []
    for t in range(1, keep[-1] + 1):
        model.simulate(1, sync_workers_every_n_ticks=1)
        if t in keep:
            health.append(np.asarray(model.get_breed_local_array("health"), dtype=np.float32))
            load.append(np.asarray(model.get_breed_local_array("load"), dtype=np.float32))
    clear_generated()
    np.savez_compressed(os.path.join(HERE, "bla_two_breeds.npz"), offsets=off, indices=idx, breeds=breeds,
                        state0=st.astype(np.int8), ticks=np.array(keep), health=np.stack(health),
                        load=np.stack(load))


def measures_er():
    from ref_steps import measures_step
    from sagesim.breed import Breed
    from sagesim.model import Model
    from sagesim.space import NetworkSpace

    from sagesim_gb300 import graphs

    off, idx = graphs.erdos_renyi(1500, 0.004, 9)
    n = off.size - 1
    rng = np.random.default_rng(9)
    st = np.ones(n, dtype=np.int32)
    st[rng.choice(n, 30, replace=False)] = 2
    meas = (rng.random((n, 4), dtype=np.float32) * np.float32(0.5)).astype(np.float32)
    model = Model(NetworkSpace(), step_function_file_path="step_func_code_gold_meas.py")
    br = Breed("SIR")
    br.register_property("state", 1)
    br.register_property("measures", [0.0] * 4)
    br.register_property("history", [0.0] * 5)
    br.register_step_func(measures_step, os.path.join(HERE, "ref_steps.py"), priority=0)
    model.register_breed(br)
    model.register_global_property("p_infection", 0.3)
    model.register_global_property("p_recovery", 0.1)
    model.set_seed(9)
    for i in range(n):
        model.create_agent_of_breed(br, state=int(st[i]), measures=[float(v) for v in meas[i]])
    sp = model.get_space()
    for i in range(n):
        for k in range(off[i], off[i + 1]):
            sp.connect_agents(i, int(idx[k]), directed=True)
    model._max_blocks_per_sm = 1
    model.setup(use_gpu=True)
    keep = [1, 2, 5, 10, 25]
    states, hist = [], []
    for t in range(1, keep[-1] + 1):
        model.simulate(1, sync_workers_every_n_ticks=1)
        if t in keep:
            states.append(states_by_agent(model, "state").astype(np.int8))
            hist.append(states_by_agent(model, "history").astype(np.float32))
    clear_generated()
    np.savez_compressed(os.path.join(HERE, "measures_er.npz"), offsets=off, indices=idx, state0=st.astype(np.int8),
                        measures=meas, ticks=np.array(keep), state=np.stack(states), history=np.stack(hist))


def helpers_er():
    from ref_steps import helpers_step
    from sagesim.breed import Breed
    from sagesim.model import Model
    from sagesim.space import NetworkSpace

    from sagesim_gb300 import graphs

    off, idx = graphs.erdos_renyi(1000, 0.006, 12)
    n = off.size - 1
    rng = np.random.default_rng(12)
    st = np.ones(n, dtype=np.int32)
    st[rng.choice(n, 15, replace=False)] = 2
    model = Model(NetworkSpace(), step_function_file_path="step_func_code_gold_helpers.py")
    br = Breed("SIR")
    br.register_property("state", 1)
    br.register_property("visits", 0.0)
    br.register_step_func(helpers_step, os.path.join(HERE, "ref_steps.py"), priority=0)
    model.register_breed(br)
    model.register_global_property("p_infection", 0.2)
    model.register_global_property("p_recovery", 0.1)
    model.set_seed(12)
    for i in range(n):
        model.create_agent_of_breed(br, state=int(st[i]))
    sp = model.get_space()
    for i in range(n):
        for k in range(off[i], off[i + 1]):
            sp.connect_agents(i, int(idx[k]), directed=True)
    hist = run_ticks(model, "state", 30, np.int8)
    visits = states_by_agent(model, "visits").astype(np.float32)
    clear_generated()
    np.savez_compressed(os.path.join(HERE, "helpers_er.npz"), offsets=off, indices=idx, state0=st.astype(np.int8),
                        history=hist, visits=visits)


def fraction_er():
    from ref_steps import fraction_step
    from sagesim.breed import Breed
    from sagesim.model import Model
    from sagesim.space import NetworkSpace

    from sagesim_gb300 import graphs

    off, idx = graphs.erdos_renyi(1500, 0.004, 13)
    n = off.size - 1
    rng = np.random.default_rng(13)
    st = np.ones(n, dtype=np.int32)
    st[rng.choice(n, 30, replace=False)] = 2
    load0 = rng.integers(0, 4, size=n).astype(np.int32)
    model = Model(NetworkSpace(), step_function_file_path="step_func_code_gold_frac.py")
    br = Breed("SIR")
    br.register_property("state", 1)
    br.register_property("immunity", 0)
    br.register_property("load", 0)
    br.register_step_func(fraction_step, os.path.join(HERE, "ref_steps.py"), priority=0)
    model.register_breed(br)
    model.register_global_property("p_infection", 0.4)
    model.register_global_property("p_recovery", 0.1)
    model.set_seed(13)
    for i in range(n):
        model.create_agent_of_breed(br, state=int(st[i]), load=int(load0[i]))
    sp = model.get_space()
    for i in range(n):
        for k in range(off[i], off[i + 1]):
            sp.connect_agents(i, int(idx[k]), directed=True)
    model._max_blocks_per_sm = 1
    model.setup(use_gpu=True)
    keep = [1, 2, 5, 10, 25]
    states, imm, load = [], [], []
    for t in range(1, keep[-1] + 1):
        model.simulate(1, sync_workers_every_n_ticks=1)
        if t in keep:
            states.append(states_by_agent(model, "state").astype(np.int8))
            imm.append(states_by_agent(model, "immunity").astype(np.float32))
            load.append(states_by_agent(model, "load").astype(np.float32))
    clear_generated()
    np.savez_compressed(os.path.join(HERE, "fraction_er.npz"), offsets=off, indices=idx, state0=st.astype(np.int8),
                        load0=load0, ticks=np.array(keep), state=np.stack(states), immunity=np.stack(imm),
                        load=np.stack(load))


def binding_model(cls, codefile):
    """The SIR model of the binding fixture, built through the reference's own
    API as a SAGESim user would (connect_agents on a set-based space)."""
    import test_simulation as ts
    from sagesim.breed import Breed

    from sagesim_gb300 import graphs

    off, idx = graphs.erdos_renyi(2000, 0.004, 17)
    n = off.size - 1
    rng = np.random.default_rng(17)
    st = np.ones(n, dtype=np.int32)
    st[rng.choice(n, 20, replace=False)] = 2
    from sagesim.space import NetworkSpace

    model = cls(NetworkSpace(), step_function_file_path=codefile)
    br = Breed("SIR")
    br.register_property("state", 1)
    br.register_step_func(ts.sir_step_func, ts.__file__, priority=0)
    model.register_breed(br)
    model.register_global_property("p_infection", 0.3)
    model.register_global_property("p_recovery", 0.1)
    model.set_seed(17)
    for i in range(n):
        model.create_agent_of_breed(br, state=int(st[i]))
    sp = model.get_space()
    for i in range(n):
        for k in range(off[i], off[i + 1]):
            if idx[k] > i:
                sp.connect_agents(i, int(idx[k]))
    for a in rng.choice(n, 100, replace=False):
        model.set_agent_logical_id(int(a), int(rng.integers(0, 2**24)))
    return model


def integration_binding_namespace():
    """Executes the two binding blocks of INTEGRATION.md (the engine side and the
    SAGESim side) in one namespace."""
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    ns = {}
    for tag in ("engine", "sagesim"):
        body = text.split("<!-- binding:%s -->" % tag, 1)[1].split("```python", 1)[1].split("```", 1)[0]
        exec(compile(body, "INTEGRATION.md:binding:" + tag, "exec"), ns)
    return ns


def binding_er():
    from sagesim.model import Model

    ns = integration_binding_namespace()
    x = binding_model(ns["GB300SIRModel"], "step_func_code_gold_bind0.py").gb300_inputs()
    clear_generated()
    hist = run_ticks(binding_model(Model, "step_func_code_gold_bind1.py"), "state", 30, np.int8)
    clear_generated()
    np.savez_compressed(os.path.join(HERE, "binding_er.npz"), history=hist,
                        **{"in_" + k: np.asarray(v) for k, v in x.items()})


def main():
    reference = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SAGESIM_REFERENCE", "")
    if not reference or not os.path.isdir(os.path.join(reference, "sagesim")):
        sys.exit("usage: make_golden.py <reference source tree>")
    setup_paths(reference)
    work = tempfile.mkdtemp(prefix="sg_golden_")
    os.chdir(work)  # the reference writes its generated step module into the CWD
    which = sys.argv[2:] or ["philox", "chain", "hier", "db", "er", "breeds", "bla", "measures", "helpers",
                             "fraction", "binding", "opinion"]
    jobs = {"philox": philox_vectors, "chain": chains, "hier": hierarchy, "db": db_priority,
            "er": er_c1, "breeds": ba_breeds, "bla": bla_two_breeds, "measures": measures_er, "helpers": helpers_er,
            "fraction": fraction_er, "binding": binding_er,
            "opinion": opinion_ws}
    for w in which:
        print("generating", w, flush=True)
        jobs[w]()


if __name__ == "__main__":
    main()
