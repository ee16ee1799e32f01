"""The translator's CUDA C++ compiles for sm_103a (no GPU needed: nvcc
cross-compiles), wrapped the way the engine hands a compiled step to NVRTC:
the Philox and step-API headers, the PROP_ / G_ index macros, the step, and a
tile-walking kernel that calls it. Covers every reference-dialect step in
tests/golden/ref_steps.py and the float remainder helpers."""
import os
import shutil
import subprocess

import pytest

from sagesim_gb300.translate import translate_step

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")

# (step, globals, properties with dtype and width, breed-local arrays)
CASES = [
    ("sir_per_neighbour_step", ["p_infection", "p_recovery"], [("state", "i", 1)], []),
    ("opinion_step", ["noise_sigma"], [("opinion", "f", 1), ("weights", "f", 8)], []),
    ("host_step", ["p_infection", "p_recovery"], [("state", "i", 1)], [("health", (4,)), ("load", (2, 2))]),
    ("site_step", ["p_infection", "p_recovery"], [("state", "i", 1)], [("health", (4,)), ("load", (2, 2))]),
    ("measures_step", ["p_infection", "p_recovery"], [("state", "i", 1), ("measures", "f", 4), ("history", "f", 5)],
     []),
    ("helpers_step", ["p_infection", "p_recovery"], [("state", "i", 1), ("visits", "f", 1)], []),
]

FMOD = '''
def fmod_step(tick, agent_index, d, agent_ids, breeds, locations, x, y):
    y[agent_index] = x[agent_index] % d + cp.float32(x[agent_index] % cp.float32(0.5))
    y[agent_index] = max(y[agent_index], 0.0, min(d, math.pi, 4)) * math.e
'''


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def _unit(name, code, entry, props, globals_, arrays):
    defs, undefs = [], []
    names = [p[0] for p in props] + sum([["sgbla_" + a, "sgbla_%s_idx" % a] for a, _ in arrays], [])
    for k, pname in enumerate(names):
        defs.append("#define PROP_%s %d" % (pname, k))
        undefs.append("#undef PROP_%s" % pname)
    for k, g in enumerate(globals_):
        defs.append("#define G_%s %d" % (g, k))
        undefs.append("#undef G_%s" % g)
    # each unit's prelude helpers are static inline: wrap in a namespace per step
    return "\n".join(["namespace u_%s {" % name] + defs + [code] + [
        "}",
        'extern "C" __global__ void k_%s(sg_step_args a)' % name,
        "{",
        "    sg_ctx ctx;",
        "    ctx.tick = a.tick0 + a.r; ctx.key = a.key; ctx.c0b = sg_c0base(ctx.tick); ctx.r = a.r;",
        "    ctx.lids = a.lids; ctx.off = a.off; ctx.idx = a.idx; ctx.g = a.g; ctx.props = a.props;",
        "    for (int i = threadIdx.x; i < (int)a.n; i += blockDim.x) u_%s::%s(ctx, i);" % (name, entry),
        "}",
    ] + undefs)


def test_translated_steps_compile_for_sm_103a(tmp_path):
    nvcc = _nvcc()
    if not nvcc:
        pytest.skip("needs nvcc")
    src = open(os.path.join(GOLD, "ref_steps.py")).read()
    units = []
    for name, globals_, props, arrays in CASES:
        code, entry, _ = translate_step(src, name, globals_, [p[0] for p in props],
                                        {p[0]: p[1] for p in props}, arrays=arrays,
                                        prop_widths={p[0]: p[2] for p in props})
        units.append(_unit(name, code, entry, props, globals_, arrays))
    code, entry, _ = translate_step(FMOD, "fmod_step", ["d"], ["x", "y"], {"x": "f", "y": "f"})
    assert "sg_py_fmodf" in code and "sg_py_fmod(" in code
    units.append(_unit("fmod_step", code, entry, [("x", "f", 1), ("y", "f", 1)], ["d"], []))
    cu = tmp_path / "steps.cu"
    cu.write_text("\n".join([
        '#include "sg_philox.h"',
        '#include "sagesim_gb300_step.h"',
    ] + units))
    out = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "--fmad=false",
                          "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "sagesim_gb300", "csrc"),
                          "-c", str(cu), "-o", str(tmp_path / "steps.o")], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr[-3000:]
