"""The Python step-dialect translator on the host: output shape, typing rules
and refusals (compilation and results are checked on the GPU in
test_model_gpu.py)."""
import os

import pytest

from sagesim_gb300.translate import StepTranslationError, translate_step

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _tr(src, name="step", globals_=("p",), props=("state",), dtypes=None):
    return translate_step(src, name, list(globals_), list(props), dtypes or {"state": "i"})


def test_reference_dialect_steps_translate():
    src = open(os.path.join(GOLD, "ref_steps.py")).read()
    code, entry, writes = translate_step(src, "sir_per_neighbour_step", ["p_infection", "p_recovery"],
                                         ["state"], {"state": "i"})
    assert entry == "sg_py_sir_per_neighbour_step" and writes == ["state"]
    assert "ctx.degree((int)(sg_agent))" in code
    assert "ctx.rand_uniform((int)(sg_agent), (long long)(((long long)(2LL) + (long long)(u_j))))" in code
    assert "ctx.g[G_p_recovery]" in code
    code, _, writes = translate_step(src, "opinion_step", ["noise_sigma"], ["opinion", "weights"],
                                     {"opinion": "f", "weights": "f"})
    assert writes == ["opinion"]
    assert "float u_acc" in code and "double u_y" in code
    assert "ctx.f32(PROP_weights, (int)(sg_agent), (int)(u_j))" in code
    assert "ctx.rand_normal((int)(sg_agent), (long long)(1LL))" in code


def test_numpy_typing_rules():
    src = '''
def step(tick, agent_index, p, agent_ids, breeds, locations, state):
    a = 3
    b = a / 2
    c = a // 2
    d = cp.float32(1.5)
    e = d * 2.0
    f = d * a
    g = -7 % 3
'''
    code, _, _ = _tr(src)
    assert "long long u_a" in code
    assert "double u_b" in code and "((double)(u_a) / (double)(2LL))" in code
    assert "long long u_c" in code and "sg_py_floordiv" in code
    assert "float u_d" in code
    assert "float u_e" in code  # a float32 with a literal stays float32
    assert "double u_f" in code  # float32 with int64 becomes float64
    assert "sg_py_mod" in code


def test_loops_and_property_components():
    src = '''
def step(tick, agent_index, p, agent_ids, breeds, locations, state, weights):
    row = locations[agent_index]
    total = 0.0
    for k in range(len(row)):
        if cp.isnan(row[k]):
            break
        total += weights[agent_index][k] * p
    weights[agent_index, 0] = total
    if total > 1.0:
        return
'''
    code, _, writes = _tr(src, props=("state", "weights"), dtypes={"state": "i", "weights": "f"})
    assert writes == ["weights"]
    assert "for (u_k = (long long)(0LL);" in code
    assert "if (false)" in code  # CSR rows carry no NaN padding
    assert "ctx.set_f32(PROP_weights, (int)(sg_agent), (float)(u_total), (int)(0LL));" in code
    assert "return;" in code


@pytest.mark.parametrize("body,msg", [
    ("    x = [1, 2]\n", "unsupported expression"),
    ("    foo(1)\n", "expression statements"),
    ("    y = rand_uniform_philox(tick + 1, agent_index, 1)\n", "current tick"),
    ("    tick = 3\n", "cannot assign to parameter"),
    ("    for k in items:\n        pass\n", "range()"),
    ("    return 1\n", "returns nothing"),
])
def test_refusals_name_the_line(body, msg):
    src = "def step(tick, agent_index, p, agent_ids, breeds, locations, state):\n" + body
    with pytest.raises(StepTranslationError, match=msg):
        _tr(src)


def test_missing_function_and_short_signature():
    with pytest.raises(StepTranslationError, match="no function"):
        _tr("def other(tick, agent_index):\n    pass\n")
    with pytest.raises(StepTranslationError, match="expected"):
        _tr("def step(tick, agent_index):\n    pass\n", globals_=("a", "b"))


def test_breed_local_arrays():
    """Breed-local arrays come as (array, index map) parameter pairs after the
    properties (sagesim/model.py:1994-2008); elements are flattened row-major
    into the engine array, writes are reported as sgbla_<name>."""
    src = open(os.path.join(GOLD, "ref_steps.py")).read()
    arrays = [("health", (4,)), ("load", (2, 2))]
    code, _, writes = translate_step(src, "host_step", ["p_infection", "p_recovery"], ["state"], {"state": "i"},
                                     arrays=arrays)
    assert writes == ["sgbla_health"]
    assert "(long long)ctx.i32(PROP_sgbla_health_idx, (int)(sg_agent))" in code
    assert "ctx.arr_f32(PROP_sgbla_load, (long long)(u_r3), ((0LL) * 2LL + (long long)(1LL)) * 2LL + (long long)(0LL))" in code
    assert "ctx.set_arr_f32(PROP_sgbla_health, (long long)(u_row), (float)(u_e_n), (0LL) * 4LL + (long long)(3LL));" in code
    _, _, writes = translate_step(src, "site_step", ["p_infection", "p_recovery"], ["state"], {"state": "i"},
                                  arrays=arrays)
    assert writes == ["sgbla_load"]
    bad = '''
def step(tick, agent_index, p, agent_ids, breeds, locations, state, h, h_idx):
    h[h_idx[agent_index]] = 1.0
'''
    with pytest.raises(StepTranslationError, match="needs 2 indices"):
        translate_step(bad, "step", ["p"], ["state"], {"state": "i"}, arrays=[("h", (3,))])
    with pytest.raises(StepTranslationError, match="breed-local array parameters"):
        translate_step(bad, "step", ["p"], ["state"], {"state": "i"})
    bad = bad.replace("h[h_idx[agent_index]] = 1.0", "h_idx[agent_index] = 1")
    with pytest.raises(StepTranslationError):
        translate_step(bad, "step", ["p"], ["state"], {"state": "i"}, arrays=[("h", (3,))])


def test_list_property_row_aliases():
    """r = p[a] of a list property is an alias of that row: r[k] reads p[a][k],
    len(r) and len(p[a]) are the property's width; writes through an alias are
    refused; int ** small int literal stays an exact integer."""
    src = open(os.path.join(GOLD, "ref_steps.py")).read()
    code, _, writes = translate_step(src, "measures_step", ["p_infection", "p_recovery"],
                                     ["state", "measures", "history"], {"state": "i", "measures": "f", "history": "f"},
                                     prop_widths={"state": 1, "measures": 4, "history": 5})
    assert writes == ["history", "state"]
    assert "ctx.f32(PROP_measures, (int)(u_nb), (int)(u_b))" in code
    assert "(long long)ctx.width(PROP_measures)" in code and "(long long)ctx.width(PROP_history)" in code
    assert "pow(" not in code
    bad = '''
def step(tick, agent_index, p, agent_ids, breeds, locations, state, w):
    r = w[agent_index]
    r[0] = 1.0
'''
    with pytest.raises(StepTranslationError, match="row alias"):
        translate_step(bad, "step", ["p"], ["state", "w"], {"state": "i", "w": "f"}, prop_widths={"w": 3})


def test_utils_helpers():
    """sagesim/utils.py's device helpers: get_num_neighbors / get_neighbor read
    the CSR, get_ / set_this_agent_data_from_tensor are p[a] and p[a] = x."""
    src = open(os.path.join(GOLD, "ref_steps.py")).read()
    code, _, writes = translate_step(src, "helpers_step", ["p_infection", "p_recovery"], ["state", "visits"],
                                     {"state": "i", "visits": "f"})
    assert writes == ["state", "visits"]
    assert "ctx.degree((int)(sg_agent))" in code and "ctx.neighbor((int)(sg_agent), (int)(u_i))" in code
    assert "ctx.set_i32(PROP_state, (int)(sg_agent), (int)(3LL));" in code
    assert "ctx.i32(PROP_state, (int)(sg_agent))" in code


def test_float_remainder_has_python_sign():
    """x % y on floats follows Python / numpy (the result takes the divisor's
    sign): fmod, then the divisor added when the signs differ."""
    src = '''
def step(tick, agent_index, p, agent_ids, breeds, locations, x):
    a = 5.5 % 2.0
    b = x[agent_index] % cp.float32(0.25)
'''
    code, _, _ = translate_step(src, "step", ["p"], ["x"], {"x": "f"})
    assert "double u_a" in code and "u_a = (double)(sg_py_fmod((double)(5.5), (double)(2.0)));" in code
    assert "float u_b" in code and "sg_py_fmodf((float)(ctx.f32(PROP_x, (int)(sg_agent)))" in code
    assert "if (m != 0.0 && ((m < 0.0) != (b < 0.0))) m += b;" in code


def test_min_max_of_several_values_and_math_constants():
    """min/max fold left to right over any number of values; math.pi and
    math.e are Python floats (weak: float32 with them stays float32)."""
    src = '''
def step(tick, agent_index, g, agent_ids, breeds, locations, x):
    a = min(4, 2, 3)
    b = max(x[agent_index], 0.5, cp.float32(0.25))
    c = math.pi * 2
    d = x[agent_index] * math.e
'''
    code, _, _ = translate_step(src, "step", ["g"], ["x"], {"x": "f"})
    assert "long long u_a" in code and "float u_b" in code and "double u_c" in code and "float u_d" in code
    assert "3.141592653589793" in code and "(float)(2.718281828459045)" in code
    with pytest.raises(StepTranslationError, match="two or more"):
        translate_step(src.replace("min(4, 2, 3)", "min(4)"), "step", ["g"], ["x"], {"x": "f"})
