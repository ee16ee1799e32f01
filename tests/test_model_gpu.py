"""The drop-in Model API on the GPU against fixtures produced by the reference.

Each case rebuilds, through Breed/Model/NetworkSpace, the model that
tests/golden/make_golden.py ran through SAGESim's own pipeline, and compares
the agent states tick by tick: bit-exact for integer state, 1e-6 relative for
float32 properties.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle
from sagesim_gb300 import Breed, CudaStep, Engine, Model, NetworkSpace, OpinionStep, SIRStep, graphs

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def gold(name):
    return np.load(os.path.join(GOLD, name))


class SIRBreed(Breed):
    def __init__(self, step, name="SIR"):
        super().__init__(name)
        self.register_property("state", 1)
        self.register_step_func(step, __file__, priority=0)


def sir_model(step, p_infection, p_recovery, seed, ordered=False):
    m = Model(NetworkSpace(ordered=ordered))
    breed = SIRBreed(step)
    m.register_breed(breed)
    m.register_global_property("p_infection", p_infection)
    m.register_global_property("p_recovery", p_recovery)
    m.set_seed(seed)
    return m, breed


def chain_model(n, p_inf, p_rec, seed, step=None):
    """tests/test_simulation.py:_build_chain_model with the builtin SIR step."""
    m, breed = sir_model(step or SIRStep("A"), p_inf, p_rec, seed)
    for _ in range(n):
        m.create_agent_of_breed(breed, state=1)
    m.set_agent_property_value(0, "state", 2)
    for i in range(n - 1):
        m.get_space().connect_agents(i, i + 1)
    return m


def states(m, n):
    return [m.get_agent_property_value(i, "state") for i in range(n)]


def test_deterministic_sir_chain_known_answer():
    """tests/test_simulation.py:95-115."""
    m = chain_model(10, 1.0, 1.0, 42)
    m.setup(use_gpu=True)
    m.simulate(5, sync_workers_every_n_ticks=1)
    assert states(m, 10) == [3, 3, 3, 3, 3, 2, 1, 1, 1, 1]


@pytest.mark.parametrize("key,n,p,seed,ticks", [("det10", 10, (1.0, 1.0), 42, 5),
                                                 ("sto20_seed999", 20, (0.5, 0.3), 999, 10),
                                                 ("sto50_seed111", 50, (0.3, 0.2), 111, 20),
                                                 ("sto50_seed222", 50, (0.3, 0.2), 222, 20)])
@pytest.mark.parametrize("strategy", ["count", "pull", "frontier"])
def test_chain_every_tick_matches_reference(key, n, p, seed, ticks, strategy):
    hist = gold("chain.npz")[key]
    m = chain_model(n, p[0], p[1], seed, SIRStep("A", strategy=strategy))
    m.setup()
    for t in range(ticks):
        m.simulate(1)
        assert m.get_property_array("state").tolist() == hist[t].tolist(), "tick %d" % t


def test_seed_reproducibility_and_sensitivity():
    """tests/test_simulation.py:117-159."""
    runs = {}
    for tag, seed in (("a", 999), ("b", 999), ("c", 111), ("d", 222)):
        m = chain_model(50, 0.3, 0.2, seed)
        m.setup()
        m.simulate(20)
        runs[tag] = states(m, 50)
    assert runs["a"] == runs["b"]
    assert runs["c"] != runs["d"]


def infect_src():
    return """
__device__ void infect(const sg_ctx &c, int i)
{
    if (c.i32(PROP_state, i) != 1) return;
    for (int k = 0; k < c.degree(i); ++k) {
        if (c.i32(PROP_state, c.neighbor(i, k)) == 2 && c.rand_uniform(i, 1) < c.g[G_p_infection]) {
            c.set_i32(PROP_state, i, 2);
            return;
        }
    }
}
"""


def recover_src():
    return """
__device__ void recover(const sg_ctx &c, int i)
{
    c.set_i32(PROP_dummy, i, c.i32(PROP_dummy, i) + 1);
    if (c.i32(PROP_state, i) == 2 && c.rand_uniform(i, 2) < c.g[G_p_recovery])
        c.set_i32(PROP_state, i, 3);
}
"""


def test_hierarchy_si_and_two_priority_sir():
    """tests/test_double_buffer.py:247-271 (SI one tick; infection at priority
    0 and recovery at priority 1, both double-buffered, two ticks)."""
    d = gold("hier.npz")
    edges = d["edges"]
    # SI: builtin SIR-A without recovery
    m, breed = sir_model(SIRStep("A"), 1.0, 0.0, 0)
    for _ in range(111):
        m.create_agent_of_breed(breed, state=1)
    m.set_agent_property_value(0, "state", 2)
    for a, b in edges:
        m.get_space().connect_agents(a, b)
    m.setup()
    m.simulate(1)
    assert m.get_property_array("state").tolist() == d["si_1tick"][0].tolist()

    # SIR with two compiled steps at two priorities and a dummy counter
    m = Model(NetworkSpace())
    br = Breed("Infection")
    br.register_property("state", 1)
    br.register_property("dummy", 0)
    br.register_step_func(CudaStep(infect_src(), "infect"), __file__, 0)
    br.register_step_func(CudaStep(recover_src(), "recover"), __file__, 1)
    m.register_breed(br)
    m.register_global_property("p_infection", 1.0)
    m.register_global_property("p_recovery", 1.0)
    for _ in range(111):
        m.create_agent_of_breed(br, state=1)
    m.set_agent_property_value(0, "state", 2)
    for a, b in edges:
        m.get_space().connect_agents(a, b)
    m.setup()
    for t in range(2):
        m.simulate(1)
        assert m.get_property_array("state").tolist() == d["sir_2ticks"][t].tolist()
    assert m.get_property_array("dummy").tolist() == [2] * 111


def db_model(first, second, nodb):
    write = CudaStep("__device__ void wc(const sg_ctx &c, int i) { c.set_i32(PROP_counter, i, 10); }", "wc")
    read = CudaStep("__device__ void rm(const sg_ctx &c, int i) "
                    "{ c.set_i32(PROP_result, i, c.i32(PROP_counter, i) * 2); }", "rm")
    steps = {"write": write, "read": read}
    m = Model(NetworkSpace())
    br = Breed("DB")
    br.register_property("counter", 0)
    br.register_property("result", 0)
    br.register_step_func(steps[first], __file__, 0, no_double_buffer=["counter"] if nodb else None)
    br.register_step_func(steps[second], __file__, 1)
    m.register_breed(br)
    m.create_agent_of_breed(br, counter=0, result=0)
    return m


@pytest.mark.parametrize("name,first,second,nodb", [("db", "write", "read", False),
                                                    ("nodb", "write", "read", True),
                                                    ("rbw_db", "read", "write", False),
                                                    ("rbw_nodb", "read", "write", True)])
def test_double_buffer_priority_semantics(name, first, second, nodb):
    """tests/test_double_buffer.py:282-312 (counter/result by priority order)."""
    want = json.load(open(os.path.join(GOLD, "db_priority.json")))[name]
    m = db_model(first, second, nodb)
    m.setup()
    m.simulate(1)
    assert m.get_agent_property_value(0, "counter") == want["counter"]
    assert m.get_agent_property_value(0, "result") == want["result"]


def er_model(step, d, seed=0):
    off, idx = d["offsets"], d["indices"]
    n = off.size - 1
    m, breed = sir_model(step, 0.05, 0.1, seed)
    m.create_agents_bulk(breed, n, state=d["state0"].astype(np.int32))
    m.get_space().set_csr(off, idx)
    return m


@pytest.mark.parametrize("variant,key", [("A", "sir_a"), ("B", "sir_b")])
@pytest.mark.parametrize("strategy", ["count", "pull", "frontier"])
def test_er_10k_every_tick_matches_reference(variant, key, strategy):
    """10,000-agent ER (p=0.001, seed 0), 1 % infected, 100 ticks."""
    d = gold("er_c1.npz")
    ref = d[key]
    m = er_model(SIRStep(variant, strategy=strategy), d)
    m.setup()
    for t in range(100):
        m.simulate(1)
        got = m.get_property_array("state")
        assert np.array_equal(got, ref[t]), "tick %d: %d agents differ" % (t, int((got != ref[t]).sum()))


def test_er_10k_one_call():
    d = gold("er_c1.npz")
    m = er_model(SIRStep("B"), d)
    m.setup()
    m.simulate(100)
    assert np.array_equal(m.get_property_array("state"), d["sir_b"][-1])


def test_compiled_sir_step_matches_reference():
    """The same SIR-A written as a CudaStep (NVRTC path) on the ER fixture."""
    src = """
__device__ void sir_a(const sg_ctx &c, int i)
{
    const int s = c.i32(PROP_state, i);
    const double u = c.rand_uniform(i, 1);
    if (s == 2 && u < c.g[G_p_recovery]) {
        c.set_i32(PROP_state, i, 3);
    } else if (s == 1) {
        for (int k = 0; k < c.degree(i); ++k)
            if (c.i32(PROP_state, c.neighbor(i, k)) == 2 && u < c.g[G_p_infection])
                c.set_i32(PROP_state, i, 2);
    }
}
"""
    d = gold("er_c1.npz")
    m = er_model(CudaStep(src, "sir_a"), d)
    m.setup()
    for t in (0, 9, 49, 99):
        m.simulate(t + 1 - m.tick)
        assert np.array_equal(m.get_property_array("state"), d["sir_a"][t]), t


def test_two_breeds_and_logical_ids():
    """Interleaved breeds (sorted into ranges) and explicit logical ids."""
    d = gold("ba_breeds.npz")
    off, idx, breeds = d["offsets"], d["indices"], d["breeds"]
    n = off.size - 1
    m = Model(NetworkSpace())
    bl = [SIRBreed(SIRStep("B"), "SIR0"), SIRBreed(SIRStep("B"), "SIR1")]
    for b in bl:
        m.register_breed(b)
    m.register_global_property("p_infection", 0.08)
    m.register_global_property("p_recovery", 0.1)
    m.set_seed(77)
    for i in range(n):
        m.create_agent_of_breed(bl[int(breeds[i])], state=int(d["state0"][i]))
    for i in range(n):
        for k in range(off[i], off[i + 1]):
            m.get_space().connect_agents(i, int(idx[k]), directed=True)
    for a, l in d["lid_pairs"]:
        m.set_agent_logical_id(int(a), int(l))
    m.setup()
    for t in range(30):
        m.simulate(1)
        assert np.array_equal(m.get_property_array("state"), d["history"][t]), t
    assert m.get_breed_data("SIR1", "state") == \
        d["history"][-1][np.flatnonzero(breeds == 1)].tolist()


def test_opinion_model_matches_reference():
    """float32 opinion + float32[8] weights on ordered neighbours (WS 2,000)."""
    d = gold("opinion_ws.npz")
    off, idx = d["offsets"], d["indices"]
    n = off.size - 1
    m = Model(NetworkSpace(ordered=True))
    br = Breed("Opinion")
    br.register_property("opinion", 0.0)
    br.register_property("weights", [0.0] * 8)
    br.register_step_func(OpinionStep(), __file__, 0)
    m.register_breed(br)
    m.register_global_property("noise_sigma", 0.01)
    m.set_seed(2)
    m.create_agents_bulk(br, n, opinion=d["opinion0"], weights=d["weights"])
    m.get_space().set_csr(off, idx)
    m.setup()
    for t, want in zip(d["ticks"], d["history"]):
        m.simulate(int(t) - m.tick)
        got = m.get_property_array("opinion")
        rel = np.abs(got - want) / np.maximum(np.abs(want), 1e-30)
        ok = (rel <= 1e-6) | (np.abs(got - want) <= 1e-12)
        assert ok.all(), "tick %d: max rel %g" % (t, rel[~ok].max())


def test_opinion_engine_vs_oracle_larger():
    """WS 200,000 agents, 100 ticks, engine builtin vs the CPU oracle."""
    off, idx = graphs.watts_strogatz(200_000, 10, 0.1, 2)
    n = off.size - 1
    rng = np.random.default_rng(2)
    x0 = rng.random(n, dtype=np.float32)
    w = rng.standard_normal((n, 8), dtype=np.float32)
    with Engine() as e:
        e.set_graph(off, idx, ordered=True)
        e.set_seed(2)
        px = e.add_property("opinion", np.float32, init=x0)
        pw = e.add_property("weights", np.float32, width=8, init=w)
        e.add_opinion(px, pw, 0.01)
        e.run(0, 100, stats=False)
        got = e.get_property(px)
    want, _ = oracle.opinion_run(off, idx, w, x0, 2, 0, 100, 0.01)
    rel = np.abs(got - want) / np.maximum(np.abs(want), 1e-30)
    ok = (rel <= 1e-6) | (np.abs(got - want) <= 1e-12)
    assert ok.all(), "max rel %g over %d agents" % (rel[~ok].max(), int((~ok).sum()))


def test_opinion_split_cosine_against_direct_cos():
    """The opinion step forms cos(2 pi k / 2^23), the Box-Muller angle of
    sagesim/math_utils.py:250-255, by angle addition from small tables of
    double-float pairs, in double-float arithmetic, instead of evaluating cos.
    Over all 2^23 values of k it stays within 2e-14 of the device's own cos of
    the reference's expression and of the oracle's libm cos (numpy here); with
    sigma * radius below 0.06 that moves the noise by under 1.2e-15, far below
    a float32 ulp of the result."""
    with Engine() as e:
        split, direct = e.opinion_cosine_check(0, 1 << 23)
    k = np.arange(1 << 23, dtype=np.float64)
    host = np.cos(6.283185307179586 * (k / 8388608.0))
    assert np.abs(split - direct).max() <= 2e-14
    assert np.abs(split - host).max() <= 2e-14
    assert np.abs(direct - host).max() <= 2e-15


@pytest.mark.parametrize("sigma", [0.01, 0.25])
def test_opinion_radius_correction_gives_the_pair_table_result(sigma):
    """The opinion step forms the Box-Muller radius as a float32 estimate plus a
    32-bit correction from a table (to 2^-41) and falls back to the double-float
    pair table only where that leaves the float32 rounding of x + sigma * r *
    cos open. Over every one of the 2^23 radii (opinions spread over [0, 1],
    near 0 and 1, tiny, negative, and tiny radii with tiny opinions, where
    float32 steps are finest) the result equals the pair-table result bit for
    bit, the fallback is rare but taken, and the result matches the reference's
    double expression (sagesim/math_utils.py:231-255) rounded to float32 within
    one ulp, almost always exactly."""
    rng = np.random.default_rng(11)
    n = 1 << 23
    q = n // 6
    x = np.concatenate([rng.random(q), rng.uniform(-0.1, 0.1, q), rng.uniform(0.9, 1.1, q),
                        10.0 ** -rng.uniform(1, 8, q), 10.0 ** -rng.uniform(5, 12, q),
                        rng.uniform(0.45, 0.55, n - 5 * q)]).astype(np.float32)
    k1 = rng.permutation(n).astype(np.uint32)  # every radius once
    k2 = rng.integers(0, 1 << 23, n, dtype=np.uint32)
    tiny = np.flatnonzero(k1 >= (1 << 23) - 4096)  # radii below 0.03 ...
    x[tiny] = (10.0 ** -rng.uniform(5, 12, tiny.size)).astype(np.float32)  # ... with tiny opinions
    with Engine() as e:
        out, exact, slow = e.opinion_noise_check(x, k1, k2, sigma)
    assert np.array_equal(out.view(np.uint32), exact.view(np.uint32))
    assert slow.any()  # about 60 of the 2^23 at sigma 0.01
    assert slow[:q].mean() < 1e-4, slow[:q].mean()
    assert slow.mean() < 1e-3, slow.mean()
    r = np.sqrt(-2.0 * np.log(k1 / 8388608.0 + 1e-10))
    c = np.cos(6.283185307179586 * (k2 / 8388608.0))
    want = np.clip((x.astype(np.float64) + sigma * (r * c)).astype(np.float32), 0.0, 1.0).astype(np.float32)
    want[want == 0] = 0.0
    ulp = np.abs(out.view(np.int32).astype(np.int64) - want.view(np.int32).astype(np.int64))
    assert ulp.max() <= 1
    assert (ulp != 0).mean() < 1e-5


def test_opinion_long_run_stays_within_tolerance():
    """500 ticks (the benchmark's run length) on a 50,000-agent WS graph: the
    opinions stay within 1e-6 relative of the oracle at ticks 100, 250 and 500."""
    off, idx = graphs.watts_strogatz(50_000, 10, 0.1, 4)
    n = off.size - 1
    rng = np.random.default_rng(4)
    x0 = rng.random(n, dtype=np.float32)
    w = rng.standard_normal((n, 8), dtype=np.float32)
    with Engine() as e:
        e.set_graph(off, idx, ordered=True)
        e.set_seed(4)
        px = e.add_property("opinion", np.float32, init=x0)
        pw = e.add_property("weights", np.float32, width=8, init=w)
        e.add_opinion(px, pw, 0.01)
        t, want = 0, x0
        for stop in (100, 250, 500):
            e.run(t, stop - t, stats=False)
            want, _ = oracle.opinion_run(off, idx, w, want, 4, t, stop - t, 0.01)
            t = stop
            got = e.get_property(px)
            rel = np.abs(got - want) / np.maximum(np.abs(want), 1e-30)
            ok = (rel <= 1e-6) | (np.abs(got - want) <= 1e-12)
            assert ok.all(), "tick %d: max rel %g over %d agents" % (t, rel[~ok].max(), int((~ok).sum()))


def test_set_property_between_simulates_and_reset():
    m = chain_model(10, 1.0, 1.0, 42)
    m.setup()
    m.simulate(2)
    m.set_agent_property_value(9, "state", 2)  # a second outbreak at the far end
    m.simulate(1)
    s = states(m, 10)
    assert s[9] == 3 and s[8] == 2 and s[2] == 3 and s[3] == 2
    m.reset()
    assert m.tick == 0
    assert m.get_agent_property_value(3, "state") == 2  # host store refreshed from the device
    m.simulate(1)
    assert states(m, 10)[4] == 2


def test_global_change_between_simulates():
    m = chain_model(10, 0.0, 0.0, 42)
    m.setup()
    m.simulate(3)
    assert states(m, 10) == [2] + [1] * 9
    m.set_global_property_value("p_infection", 1.0)
    m.simulate(1)
    assert states(m, 10)[:3] == [2, 2, 1]


@pytest.mark.parametrize("first", ["connect", "edges"])
@pytest.mark.parametrize("strategy", ["count", "pull", "frontier"])
def test_topology_edits_between_simulates(first, strategy):
    """Edges added and removed between simulate() calls take effect at the next
    call, with state and tick kept: the trajectory equals the oracle run on the
    first adjacency for 10 ticks, then on the edited one from tick 10."""
    rng = np.random.default_rng(11)
    n = 3000
    m, breed = sir_model(SIRStep("B", strategy=strategy), 0.06, 0.1, 17)
    state0 = np.ones(n, dtype=np.int32)
    state0[rng.choice(n, 30, replace=False)] = 2
    for a in range(n):
        m.create_agent_of_breed(breed, state=int(state0[a]))
    sp = m.get_space()
    src, dst = rng.integers(0, n, 6000), rng.integers(0, n, 6000)
    if first == "edges":
        sp.set_edges(src, dst)
    else:
        for a, b in zip(src, dst):
            sp.connect_agents(a, b)
    m.setup()
    off1, idx1 = sp._rows()
    m.simulate(10)
    want, _, _ = oracle.sir_run(2, off1, idx1, state0, 17, 0, 10, 0.06, 0.1)
    assert np.array_equal(m.get_property_array("state"), want)
    for a, b in zip(src[:2000], dst[:2000]):
        sp.disconnect_agents(a, b)
    for a, b in zip(rng.integers(0, n, 3000), rng.integers(0, n, 3000)):
        sp.connect_agents(a, b, directed=bool(a & 1))
    off2, idx2 = sp._rows()
    m.simulate(10)
    want, _, _ = oracle.sir_run(2, off2, idx2, want, 17, 10, 10, 0.06, 0.1)
    assert np.array_equal(m.get_property_array("state"), want)


class _PyStepRef:
    """Stands in for a CuPy-JIT rawkernel object: the translator needs only the
    function's name and the module path given to register_step_func."""

    def __init__(self, name):
        self.__name__ = name


REF_STEPS = os.path.join(GOLD, "ref_steps.py")


@pytest.mark.parametrize("strategy_ticks", [(0, 9, 49, 99)])
def test_python_dialect_sir_step_matches_reference(strategy_ticks):
    """The reference-dialect SIR-B step of tests/golden/ref_steps.py, translated
    from its Python source and compiled with NVRTC, reproduces the trajectory the
    reference's own pipeline produced from the same source (er_c1.npz)."""
    d = gold("er_c1.npz")
    off, idx = d["offsets"], d["indices"]
    n = off.size - 1
    m = Model(NetworkSpace())
    br = Breed("SIR")
    br.register_property("state", 1)
    br.register_step_func(_PyStepRef("sir_per_neighbour_step"), REF_STEPS, priority=0)
    m.register_breed(br)
    m.register_global_property("p_infection", 0.05)
    m.register_global_property("p_recovery", 0.1)
    m.set_seed(0)
    m.create_agents_bulk(br, n, state=d["state0"].astype(np.int32))
    m.get_space().set_csr(off, idx)
    m.setup()
    for t in strategy_ticks:
        m.simulate(t + 1 - m.tick)
        assert np.array_equal(m.get_property_array("state"), d["sir_b"][t]), t


def test_python_dialect_opinion_step_matches_reference():
    """The reference-dialect opinion step (float32 sums, float64 noise, clamp),
    translated and compiled, against the reference's opinion_ws.npz trajectory."""
    d = gold("opinion_ws.npz")
    off, idx = d["offsets"], d["indices"]
    n = off.size - 1
    m = Model(NetworkSpace(ordered=True))
    br = Breed("Opinion")
    br.register_property("opinion", 0.0)
    br.register_property("weights", [0.0] * 8)
    br.register_step_func(_PyStepRef("opinion_step"), REF_STEPS, 0)
    m.register_breed(br)
    m.register_global_property("noise_sigma", 0.01)
    m.set_seed(2)
    m.create_agents_bulk(br, n, opinion=d["opinion0"], weights=d["weights"])
    m.get_space().set_csr(off, idx)
    m.setup()
    for t, want in zip(d["ticks"], d["history"]):
        m.simulate(int(t) - m.tick)
        got = m.get_property_array("opinion")
        rel = np.abs(got - want) / np.maximum(np.abs(want), 1e-30)
        ok = (rel <= 1e-6) | (np.abs(got - want) <= 1e-12)
        assert ok.all(), "tick %d: max rel %g" % (t, rel[~ok].max())


def test_breed_local_arrays_match_reference():
    """Two breeds with breed-local arrays (sagesim/model.py:620-650,
    1215-1270): the hosts' double-buffered float32[4] array and the sites'
    in-place float32[2][2] array written at priority 1, both translated from the
    reference dialect, equal the reference pipeline's arrays bit for bit."""
    d = gold("bla_two_breeds.npz")
    off, idx, breeds, st = d["offsets"], d["indices"], d["breeds"], d["state0"]
    n = off.size - 1
    m = Model(NetworkSpace())
    host, site = Breed("Host"), Breed("Site")
    for br in (host, site):
        br.register_property("state", 1)
    host.register_step_func(_PyStepRef("host_step"), REF_STEPS, priority=0)
    site.register_step_func(_PyStepRef("site_step"), REF_STEPS, priority=1, no_double_buffer=["load"])
    m.register_breed(host)
    m.register_breed(site)
    m.register_global_property("p_infection", 0.04)
    m.register_global_property("p_recovery", 0.1)
    assert m.register_breed_local_array("health", host, (4,)) == 0
    assert m.register_breed_local_array("load", site, (2, 2)) == 1
    m.set_seed(8)
    for i in range(n):
        m.create_agent_of_breed(site if breeds[i] else host, state=int(st[i]))
    sp = m.get_space()
    for i in range(n):
        for k in range(off[i], off[i + 1]):
            sp.connect_agents(i, int(idx[k]), directed=True)
    m.setup()
    assert not m.get_breed_local_array("health").any()
    for j, t in enumerate(d["ticks"]):
        m.simulate(int(t) - m.tick)
        h, ld = m.get_breed_local_array("health"), m.get_breed_local_array("load")
        assert h.shape == d["health"][j].shape and ld.shape == d["load"][j].shape
        assert np.array_equal(h, d["health"][j]), "health, tick %d" % t
        assert np.array_equal(ld, d["load"][j]), "load, tick %d" % t
    m.reset()
    m.simulate(1)
    assert np.array_equal(m.get_breed_local_array("health"), d["health"][0])  # rebuilt from zeros


def test_save_load_breed_ids_and_neighbor_visible(tmp_path):
    """sagesim/model.py:1288-1309 (save / load), 492-515 (get_breed_agent_ids),
    398-409 (set_property_neighbor_visible): a saved model continues from its
    tick and state after loading, as the original does."""
    want = chain_model(30, 0.5, 0.3, 5)
    want.setup()
    want.simulate(7)
    m = chain_model(30, 0.5, 0.3, 5)
    m.set_property_neighbor_visible("state", False)
    with pytest.raises(ValueError):
        m.set_property_neighbor_visible("no_such_property", True)
    m.setup()
    with pytest.raises(RuntimeError):
        m.set_property_neighbor_visible("state", True)
    assert m.get_breed_agent_ids("SIR").tolist() == list(range(30))
    m.simulate(4)
    path = str(tmp_path / "model.pkl")
    m.save(m, path)
    loaded = m.load(path)
    assert loaded.tick == 4 and states(loaded, 30) == states(m, 30)
    loaded.simulate(3)
    m.simulate(3)
    assert states(loaded, 30) == states(m, 30) == states(want, 30)


def test_python_dialect_list_property_rows_match_reference():
    """A reference-dialect step that reads list properties through row aliases
    and len() (protective measures, a state-history ring), translated, against
    the reference pipeline's states and histories (measures_er.npz)."""
    d = gold("measures_er.npz")
    off, idx = d["offsets"], d["indices"]
    n = off.size - 1
    m = Model(NetworkSpace())
    br = Breed("SIR")
    br.register_property("state", 1)
    br.register_property("measures", [0.0] * 4)
    br.register_property("history", [0.0] * 5)
    br.register_step_func(_PyStepRef("measures_step"), REF_STEPS, 0)
    m.register_breed(br)
    m.register_global_property("p_infection", 0.3)
    m.register_global_property("p_recovery", 0.1)
    m.set_seed(9)
    m.create_agents_bulk(br, n, state=d["state0"].astype(np.int32), measures=d["measures"])
    m.get_space().set_csr(off, idx)
    m.setup()
    for j, t in enumerate(d["ticks"]):
        m.simulate(int(t) - m.tick)
        assert np.array_equal(m.get_property_array("state"), d["state"][j]), "state, tick %d" % t
        assert np.array_equal(m.get_property_array("history"), d["history"][j]), "history, tick %d" % t


def test_python_dialect_utils_helpers_match_reference():
    """A reference-dialect step written with sagesim/utils.py's device helpers
    (get_num_neighbors / get_neighbor on the CSR names, get_ / set_this_agent_
    data_from_tensor), translated, against the reference pipeline's every-tick
    states and final visit counters (helpers_er.npz)."""
    d = gold("helpers_er.npz")
    off, idx = d["offsets"], d["indices"]
    n = off.size - 1
    m = Model(NetworkSpace())
    br = Breed("SIR")
    br.register_property("state", 1)
    br.register_property("visits", 0.0)
    br.register_step_func(_PyStepRef("helpers_step"), REF_STEPS, 0)
    m.register_breed(br)
    m.register_global_property("p_infection", 0.2)
    m.register_global_property("p_recovery", 0.1)
    m.set_seed(12)
    m.create_agents_bulk(br, n, state=d["state0"].astype(np.int32))
    m.get_space().set_csr(off, idx)
    m.setup()
    for t in range(30):
        m.simulate(1)
        assert np.array_equal(m.get_property_array("state"), d["history"][t]), "tick %d" % t
    assert np.array_equal(m.get_property_array("visits"), d["visits"])


def test_python_dialect_float_remainder(tmp_path):
    """Float % in a translated step has Python's sign rule (numpy.remainder)."""
    mod = tmp_path / "fmod_step.py"
    mod.write_text('''
def fmod_step(tick, agent_index, d, agent_ids, breeds, locations, x, y):
    y[agent_index] = x[agent_index] % d
''')
    n = 64
    x = np.linspace(-7.3, 7.3, n).astype(np.float32)
    m = Model(NetworkSpace())
    br = Breed("B")
    br.register_property("x", 0.5)
    br.register_property("y", 0.5)
    br.register_step_func(_PyStepRef("fmod_step"), str(mod), 0)
    m.register_breed(br)
    m.register_global_property("d", -2.5)
    m.create_agents_bulk(br, n, x=x)
    m.get_space().set_csr(np.zeros(n + 1, dtype=np.int32), np.zeros(0, dtype=np.int32))
    m.setup()
    m.simulate(1)
    want = np.remainder(x.astype(np.float64), -2.5).astype(np.float32)
    assert np.array_equal(m.get_property_array("y"), want)


def test_python_dialect_step_writes_fractions_into_whole_number_properties():
    """Two properties start as whole numbers (an int default, int initial
    values) and a reference-dialect step stores fractions into them (immunity
    += 0.25, load = (load + k) / 2). The reference keeps both in float32; here
    they must not be truncated: states, immunity and load equal the reference
    pipeline's (fraction_er.npz) after ticks 1, 2, 5, 10, 25."""
    d = gold("fraction_er.npz")
    off, idx = d["offsets"], d["indices"]
    n = off.size - 1
    m = Model(NetworkSpace())
    br = Breed("SIR")
    br.register_property("state", 1)
    br.register_property("immunity", 0)
    br.register_property("load", 0)
    br.register_step_func(_PyStepRef("fraction_step"), REF_STEPS, 0)
    m.register_breed(br)
    m.register_global_property("p_infection", 0.4)
    m.register_global_property("p_recovery", 0.1)
    m.set_seed(13)
    m.create_agents_bulk(br, n, state=d["state0"].astype(np.int32), load=d["load0"])
    m.get_space().set_csr(off, idx)
    m.setup()
    for j, t in enumerate(d["ticks"]):
        m.simulate(int(t) - m.tick)
        assert np.array_equal(m.get_property_array("state"), d["state"][j]), "state, tick %d" % t
        assert np.array_equal(m.get_property_array("immunity"), d["immunity"][j]), "immunity, tick %d" % t
        assert np.array_equal(m.get_property_array("load"), d["load"][j]), "load, tick %d" % t
    assert (d["immunity"][-1] % 1 != 0).any() and (d["load"][-1] % 1 != 0).any()
