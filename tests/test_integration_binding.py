"""The SAGESim-side binding of INTEGRATION.md, run as written there.

Host side (no GPU): GB300SIRModel.gb300_inputs() reads a model built through
the reference's own API (Model / Breed / NetworkSpace.connect_agents /
set_agent_logical_id, run through the CPU stand-ins of oracle/refshim) and must
give the extraction recorded in tests/golden/binding_er.npz. It needs the
reference source tree, so it is skipped where that tree is absent; set
SAGESIM_REFERENCE to its path.

GPU side: the binding's engine half, gb300_sir_engine(), fed that recorded
extraction, must reproduce the reference pipeline's own states of the same
model after every one of 30 ticks (SAGESim's test SIR step,
tests/test_simulation.py:24-43, logical ids as RNG keys,
sagesim/model.py:656-667).
"""
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLD = os.path.join(HERE, "golden", "binding_er.npz")


def _binding_block(tag):
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    return text.split("<!-- binding:%s -->" % tag, 1)[1].split("```python", 1)[1].split("```", 1)[0]


def test_binding_extraction_from_a_reference_model(tmp_path):
    reference = os.environ.get("SAGESIM_REFERENCE", "/root/reference")
    if not os.path.isdir(os.path.join(reference, "sagesim")):
        pytest.skip("the reference source tree is not available here")
    out = tmp_path / "inputs.npz"
    # a child process: the CPU stand-ins for cupy / mpi4py must not leak into this one
    script = (
        "import os, sys, numpy as np\n"
        "sys.path.insert(0, %r)\n"
        "import make_golden as mg\n"
        "mg.setup_paths(%r)\n"
        "os.chdir(%r)\n"
        "ns = mg.integration_binding_namespace()\n"
        "x = mg.binding_model(ns['GB300SIRModel'], 'step_func_code_bind_test.py').gb300_inputs()\n"
        "np.savez(%r, **{k: np.asarray(v) for k, v in x.items()})\n"
    ) % (os.path.join(HERE, "golden"), reference, str(tmp_path), str(out))
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    got = np.load(out)
    want = np.load(GOLD)
    for k in ("offsets", "indices", "logical_ids", "seed", "state", "p_infection", "p_recovery"):
        assert np.array_equal(got[k], want["in_" + k]), k
    # what the extraction must hold, checked independently of the binding's code
    n = want["in_state"].size
    off, idx = got["offsets"], got["indices"]
    src = np.repeat(np.arange(n), np.diff(off))
    assert np.array_equal(np.sort(src.astype(np.int64) * n + idx), np.sort(idx.astype(np.int64) * n + src))
    assert int(got["seed"]) == 17 and float(got["p_infection"]) == 0.3 and float(got["p_recovery"]) == 0.1
    assert (got["logical_ids"] != np.arange(n)).sum() == 100
    assert (got["state"] == 2).sum() == 20


@pytest.mark.gpu
def test_binding_engine_reproduces_the_reference_pipeline():
    d = np.load(GOLD)
    x = {k[3:]: d[k] for k in d.files if k.startswith("in_")}
    x["seed"] = int(x["seed"])
    x["p_infection"] = float(x["p_infection"])
    x["p_recovery"] = float(x["p_recovery"])
    ns = {}
    exec(compile(_binding_block("engine"), "INTEGRATION.md:binding:engine", "exec"), ns)
    e, state = ns["gb300_sir_engine"](x)
    with e:
        for t in range(d["history"].shape[0]):
            e.run(t, 1, stats=False)  # what GB300SIRModel.worker_coroutine does per simulate(1)
            got = e.get_property(state)
            assert np.array_equal(got, d["history"][t]), "tick %d: %d agents differ" % (
                t, int((got != d["history"][t]).sum()))
