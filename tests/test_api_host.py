"""Drop-in API bookkeeping on the host (no GPU): Breed, NetworkSpace, CSR
builder, AgentFactory and Model before setup, and the host arrays setup()
hands the engine. Mirrors the reference's own unit tests
(tests/test_breed.py, tests/test_space.py, tests/test_csr.py,
tests/test_model_lifecycle.py)."""
from math import nan
from pathlib import Path

import numpy as np
import pytest

from sagesim_gb300 import Breed, CudaStep, Model, NetworkSpace, SIRStep
from sagesim_gb300.csr import build_csr_from_ragged, build_csr_values_only

STEP = SIRStep(variant="A")


# ---- Breed (tests/test_breed.py) ----
def test_register_property_scalar_and_list():
    b = Breed("TestBreed")
    b.register_property("health", 100)
    b.register_property("history", [0.0] * 10)
    assert b.properties["health"] == 100
    assert b.properties["history"] == [0.0] * 10


def test_register_step_func_and_no_double_buffer():
    b = Breed("TestBreed")
    b.register_property("counter", 0)
    b.register_property("result", 0)
    b.register_step_func(STEP, __file__, priority=0, no_double_buffer=["counter"])
    fn, path = b.step_funcs[0]
    assert fn is STEP and path == str(Path(__file__).resolve())
    assert "counter" in b.no_double_buffer_props and "result" not in b.no_double_buffer_props


def test_property_neighbor_visible_and_default_nan():
    b = Breed("TestBreed")
    b.register_property("state", 1, neighbor_visible=True)
    b.register_property("internal", 0, neighbor_visible=False)
    b.register_property("x")
    assert b.prop2neighbor_visible["state"] and not b.prop2neighbor_visible["internal"]
    assert b.properties["x"] != b.properties["x"]  # nan


# ---- NetworkSpace (tests/test_space.py) ----
def make_space(n=3, ordered=False):
    m = Model(NetworkSpace(ordered=ordered))
    b = Breed("B")
    b.register_property("state", 1)
    m.register_breed(b)
    for _ in range(n):
        m.create_agent_of_breed(b)
    return m, m.get_space()


def test_space_connect_disconnect():
    _, sp = make_space()
    assert sp._locations == [set(), set(), set()]
    sp.connect_agents(0, 1)
    assert 1 in sp._locations[0] and 0 in sp._locations[1]
    sp.connect_agents(1, 2, directed=True)
    assert 2 in sp._locations[1] and 1 not in sp._locations[2]
    sp.disconnect_agents(0, 1)
    assert 1 not in sp._locations[0] and 0 not in sp._locations[1]
    sp.connect_agents(0, 2)
    sp.disconnect_agents(0, 2, directed=True)
    assert 2 not in sp._locations[0] and 0 in sp._locations[2]


def test_ordered_space_keeps_insertion_order_without_duplicates():
    _, sp = make_space(4, ordered=True)
    for a, b in [(0, 3), (0, 1), (0, 3), (2, 0)]:
        sp.connect_agents(a, b)
    assert sp.get_location(0) == [3, 1, 2]


# ---- CSR (tests/test_csr.py golden arrays) ----
def test_csr_golden():
    off, val = build_csr_from_ragged([[5, 2], [8, 3, 1], [], [7, 4, 9, 6]])
    assert off.tolist() == [0, 2, 5, 5, 9] and val.tolist() == [5, 2, 8, 3, 1, 7, 4, 9, 6]
    off, val = build_csr_from_ragged([{5, 2}, {8}])
    assert off.tolist() == [0, 2, 3] and set(val[:2].tolist()) == {5, 2} and val[2] == 8
    off, val = build_csr_from_ragged([])
    assert off.tolist() == [0] and val.size == 0
    off, val = build_csr_from_ragged([[1], [], [2, 3]])
    assert off.tolist() == [0, 1, 1, 3] and val.tolist() == [1, 2, 3]
    off, _ = build_csr_from_ragged([[10, 20], [30]])
    assert build_csr_values_only([[100, 200], [300]], off).tolist() == [100, 200, 300]


# ---- Model lifecycle (tests/test_model_lifecycle.py, host parts) ----
def test_model_lifecycle_host():
    m, _ = make_space(0)
    b = list(m._agent_factory.breeds)[0]
    assert [m.create_agent_of_breed(b) for _ in range(5)] == [0, 1, 2, 3, 4]
    assert m._agent_factory.num_agents == 5
    m.set_agent_property_value(2, "state", 42)
    assert m.get_agent_property_value(2, "state") == 42
    m.register_global_property("rate", 0.5)
    assert m.get_global_property_value("rate") == 0.5
    m.set_global_property_value("rate", 0.9)
    assert m.get_global_property_value("rate") == 0.9
    m.set_seed(12345)
    assert m._seed == 12345
    with pytest.raises(Exception):
        m.register_breed(Breed("Late"))


def test_python_step_function_is_taken_as_reference_dialect():
    """A plain function is a step in SAGESim's Python dialect, translated at setup;
    one whose source cannot be found fails with the translator's message."""
    from sagesim_gb300.steps import PythonStep
    from sagesim_gb300.translate import StepTranslationError

    m, _ = make_space(2)
    b = list(m._agent_factory.breeds)[0]
    b.register_step_func(lambda *a: None, __file__, priority=0)
    m._collect_steps()
    step = m._steps[0][2]
    assert isinstance(step, PythonStep)
    with pytest.raises(StepTranslationError, match="no function"):
        step.translate([], ["state"], {"state": "i"})


def test_host_arrays_breed_sort_csr_and_logical_ids():
    """setup()'s host side: stable breed sort (sagesim/agent.py:438-473), CSR
    of buffer indices, float32 logical ids (sagesim/model.py:1085-1096)."""
    m = Model(NetworkSpace())
    b0, b1 = Breed("A"), Breed("B")
    for b in (b0, b1):
        b.register_property("state", 1)
        b.register_step_func(SIRStep("B"), __file__, 0)
        m.register_breed(b)
    m.register_global_property("p_infection", 0.1)
    m.register_global_property("p_recovery", 0.1)
    breeds = [0, 1, 0, 1, 1, 0]
    for i, bi in enumerate(breeds):
        m.create_agent_of_breed((b0, b1)[bi], state=1 + (i == 3))
    sp = m.get_space()
    for a, c in [(0, 1), (1, 2), (3, 4), (5, 0)]:
        sp.connect_agents(a, c)
    m.set_agent_logical_id(4, 2**24 + 1)  # rounds to 2^24 in float32
    m._collect_steps()
    m._build_host_arrays()
    assert m._order.tolist() == [0, 2, 5, 1, 3, 4]
    assert m._breed_ranges == {0: (0, 3), 1: (3, 6)}
    off, idx = m._csr
    pos = m._pos
    for a in range(6):
        row = set(idx[off[pos[a]]:off[pos[a] + 1]].tolist())
        assert row == {int(pos[c]) for c in sp._locations[a]}
    assert m._lids.tolist() == [0, 2, 5, 1, 3, 2**24]
    dt, w, col = m._props["state"]
    assert dt == np.int32 and w == 1 and col.tolist() == [1, 1, 1, 1, 2, 1]


def test_cuda_step_detects_writes():
    s = CudaStep("__device__ void f(const sg_ctx& c, int i){ c.set_i32(PROP_counter, i, 10); }", "f")
    assert s.writes == ("counter",)


def test_list_property_padded_with_nan():
    m = Model(NetworkSpace())
    b = Breed("B")
    b.register_property("w", [0.0, 0.0, 0.0])
    m.register_breed(b)
    m.create_agent_of_breed(b, w=[1.0, 2.0])
    m.create_agent_of_breed(b)
    m._collect_steps()
    m._build_host_arrays()
    dt, width, col = m._props["w"]
    assert width == 3 and dt == np.float32
    assert col[0, :2].tolist() == [1.0, 2.0] and np.isnan(col[0, 2]) and col[1].tolist() == [0, 0, 0]
    assert nan != nan


@pytest.mark.parametrize("ordered", [False, True])
@pytest.mark.parametrize("directed", [False, True])
def test_edge_list_rows_equal_connect_agents(ordered, directed):
    """set_edges leaves the rows connect_agents would (sagesim/space.py:107-125):
    repeated and self edges, both directions unless directed, first-connection
    order for an ordered space; later edits go through the same containers."""
    rng = np.random.default_rng(5)
    n = 40
    src = rng.integers(0, n, 300)
    dst = rng.integers(0, n, 300)
    src[:5], dst[:5] = 7, 7  # self edges
    _, a = make_space(n, ordered=ordered)
    for s, d in zip(src, dst):
        a.connect_agents(s, d, directed=directed)
    _, b = make_space(n, ordered=ordered)
    v = b._version
    b.set_edges(src, dst, directed=directed)
    assert b._version > v
    off, idx = b._rows()
    for i in range(n):
        row = idx[off[i]:off[i + 1]].tolist()
        assert (row == a.get_location(i)) if ordered else (set(row) == a.get_location(i))
    b.disconnect_agents(3, 4)
    a.disconnect_agents(3, 4)
    assert b._id_edges is None
    for i in range(n):
        assert b.get_location(i) == a.get_location(i)
    with pytest.raises(ValueError):
        b.set_edges([0], [n])
        b._rows()


def test_breed_local_array_registration():
    """sagesim/model.py:620-645: index in registration order; our checks refuse
    a repeated name, empty shapes and registration after setup."""
    m, _ = make_space(3)
    b = list(m._agent_factory.breeds)[0]
    assert m.register_breed_local_array("h", b, (4,)) == 0
    assert m.register_breed_local_array("g", b, 5) == 1
    assert m._breed_local_arrays[1]["shape_per_agent"] == (5,)
    with pytest.raises(ValueError):
        m.register_breed_local_array("h", b, (2,))
    with pytest.raises(ValueError):
        m.register_breed_local_array("z", b, (0,))
    with pytest.raises(RuntimeError):
        m.get_breed_local_array("h")
    m._is_setup = True
    with pytest.raises(RuntimeError):
        m.register_breed_local_array("late", b, (1,))


class _FakeEngine:
    """Records the graph a Model hands to its engine (host-side test double)."""

    def __init__(self):
        self.graphs = []

    def set_graph(self, off, idx, ordered=False):
        self.graphs.append((np.array(off), np.array(idx), ordered))

    def set_graph_from_ids(self, ids, src, dst, symmetric=True, ordered=False):
        self.graphs.append(("ids", np.array(ids), np.array(src), np.array(dst), symmetric, ordered))


def test_topology_edits_reach_the_engine_in_buffer_order():
    """After setup, an edit of the space bumps its version and the next
    simulate() hands the new CSR (buffer indices) to the engine; an unchanged
    space hands nothing."""
    m = Model(NetworkSpace())
    b0, b1 = Breed("A"), Breed("B")
    for b in (b0, b1):
        b.register_property("state", 1)
        m.register_breed(b)
    for i in range(6):
        m.create_agent_of_breed((b0, b1)[i % 2])
    sp = m.get_space()
    sp.connect_agents(0, 1)
    m._collect_steps()
    m._build_host_arrays()
    m._engine = fake = _FakeEngine()
    m._install_graph(fake)
    m._refresh_graph()
    assert len(fake.graphs) == 1
    sp.connect_agents(2, 5)
    sp.disconnect_agents(0, 1)
    m._refresh_graph()
    off, idx, _ = fake.graphs[-1]
    pos = m._pos
    rows = {a: set(idx[off[pos[a]]:off[pos[a] + 1]].tolist()) for a in range(6)}
    assert rows[2] == {pos[5]} and rows[5] == {pos[2]} and rows[0] == set() and rows[1] == set()
    sp.set_edges([0, 3], [4, 1], directed=True)
    m._refresh_graph()
    kind, ids, src, dst, sym, _ = fake.graphs[-1]
    assert kind == "ids" and ids.tolist() == m._order.tolist() and not sym
    assert src.tolist() == [0, 3] and dst.tolist() == [4, 1]
    m._refresh_graph()  # nothing changed since: nothing handed over
    assert len(fake.graphs) == 3


def test_model_pickles_without_an_engine():
    import pickle

    m = Model(NetworkSpace(ordered=True))
    b = Breed("SIR")
    b.register_property("state", 1)
    b.register_property("w", [0.0, 0.0])
    b.register_step_func(STEP, __file__, 0)
    m.register_breed(b)
    m.register_global_property("p_infection", 0.5)
    for i in range(4):
        m.create_agent_of_breed(b, state=1 + (i == 2), w=[i, -i])
    m.get_space().connect_agents(0, 3)
    m.register_breed_local_array("h", b, (2,))
    m._collect_steps()
    m._build_host_arrays()
    m2 = pickle.loads(pickle.dumps(m))
    assert m2._engine is None and m2._order.tolist() == m._order.tolist()
    assert m2.get_space().get_location(3) == [0]
    assert m2.get_agent_property_value(2, "state") == 2 and m2.get_agent_property_value(1, "w") == [1, -1]
    assert m2._breed_local_arrays[0]["shape_per_agent"] == (2,)


def test_property_types_follow_what_steps_write():
    """Whole-number properties stay int32 only when no Python-dialect step
    writes them (or a builtin SIR step, whose state is int32, does); a property
    a translated step writes is float32 as in the reference, so a stored
    fraction is kept; values outside int32 are float32."""
    here = Path(__file__).resolve().parent / "golden" / "ref_steps.py"

    class Ref:
        __name__ = "fraction_step"

    m = Model(NetworkSpace())
    br = Breed("SIR")
    br.register_property("state", 1)
    br.register_property("immunity", 0)
    br.register_property("load", 0)
    br.register_property("tag", 7)
    br.register_property("big", 0)
    br.register_step_func(Ref(), str(here), 0)
    m.register_breed(br)
    m.register_global_property("p_infection", 0.4)
    m.register_global_property("p_recovery", 0.1)
    for i in range(5):
        m.create_agent_of_breed(br, state=1, load=i, big=2**33 if i == 3 else 0)
    m._collect_steps()
    m._build_host_arrays()
    types = {k: v[0] for k, v in m._props.items()}
    assert types["immunity"] == np.float32 and types["load"] == np.float32 and types["state"] == np.float32
    assert types["tag"] == np.int32  # read by no step, written by none
    assert types["big"] == np.float32  # beyond int32

    m2 = Model(NetworkSpace())
    b2 = Breed("SIR")
    b2.register_property("state", 1)
    b2.register_step_func(SIRStep("B"), None, 0)
    m2.register_breed(b2)
    m2.register_global_property("p_infection", 0.4)
    m2.register_global_property("p_recovery", 0.1)
    for i in range(3):
        m2.create_agent_of_breed(b2, state=1)
    m2._collect_steps()
    m2._build_host_arrays()
    assert m2._props["state"][0] == np.int32  # the builtin SIR step needs int32 state
