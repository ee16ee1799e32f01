"""Step objects accepted by Breed.register_step_func.

SAGESim step functions are CuPy-JIT Python kernels (e.g.
tests/test_simulation.py:24-43). Here a step is one of:

  SIRStep      the hand-written SIR kernels. variant "A" is SAGESim's own SIR
               step (one Philox draw per agent per tick, salt 1: I recovers if
               u < p_recovery; S is infected if u < p_infection and any
               neighbour is infected); variant "B" draws once per infected
               neighbour (the j-th infected neighbour found draws salt 2 + j).
  OpinionStep  the float32 opinion update (weighted mean of the first `width`
               ordered neighbours, Philox N(0, sigma) noise, clamp to [0, 1]).
  CudaStep     any step written as a CUDA C++ device function against the
               sg_ctx API of include/sagesim_gb300_step.h, compiled with NVRTC
               into the tick kernel. Property and global indices are available
               as PROP_<name> and G_<name> macros.
  PythonStep   a step function in SAGESim's own Python dialect (a CuPy-JIT
               rawkernel or a plain function), translated to a CudaStep at
               setup (sagesim_gb300/translate.py). Any other object passed to
               register_step_func is taken as such a function.

Globals are referred to by the names given to Model.register_global_property,
as the reference passes them positionally by registration order
(sagesim/model.py:2226-2251).
"""
import re


class SIRStep:
    def __init__(self, variant="A", state="state", p_infection="p_infection",
                 p_recovery="p_recovery", codes=(1, 2, 3), strategy=None):
        if variant not in ("A", "B"):
            raise ValueError("variant must be 'A' or 'B'")
        if strategy not in (None, "count", "pull", "frontier"):
            raise ValueError("strategy must be None, 'count', 'pull' or 'frontier'")
        self.variant = variant
        self.state = state
        self.p_infection = p_infection
        self.p_recovery = p_recovery
        self.codes = tuple(int(c) for c in codes)
        self.strategy = strategy

    @property
    def writes(self):
        return (self.state,)

    def __repr__(self):
        return "SIRStep(variant=%r, state=%r)" % (self.variant, self.state)


class OpinionStep:
    def __init__(self, opinion="opinion", weights="weights", noise_sigma="noise_sigma"):
        self.opinion = opinion
        self.weights = weights
        self.noise_sigma = noise_sigma

    @property
    def writes(self):
        return (self.opinion,)


class CudaStep:
    """A CUDA C++ step: `source` defines `__device__ void <entry>(const sg_ctx&, int i)`."""

    _SET = re.compile(r"set_(?:i32|f32|arr_f32)\s*\(\s*PROP_(\w+)")

    def __init__(self, source, entry, writes=None):
        self.source = source
        self.entry = entry
        if writes is None:
            writes = sorted(set(self._SET.findall(source)))
        self._writes = tuple(writes)

    @property
    def writes(self):
        return self._writes


class PythonStep:
    """A step function in SAGESim's Python dialect, read from its module file
    (the path given to register_step_func) and translated to CUDA C++ when the
    model is set up, with the model's globals and properties mapped by position
    as the reference passes them."""

    def __init__(self, step_func, module_fpath=None):
        from .translate import find_step_source

        self.source, self.name = find_step_source(step_func, module_fpath)
        self._writes = None

    def translate(self, globals_, props, prop_dtypes, arrays=(), prop_widths=None):
        from .translate import translate_step

        src, entry, writes = translate_step(self.source, self.name, globals_, props, prop_dtypes,
                                            arrays=arrays, prop_widths=prop_widths)
        self._writes = tuple(writes)
        return CudaStep(src, entry, writes=list(writes))

    def written(self, globals_, props, arrays=(), prop_widths=None):
        """Names of the properties and arrays the step writes, found before the
        property types are settled (the step is translated once with every
        property taken as float32; only its casts depend on that)."""
        from .translate import translate_step

        _, _, writes = translate_step(self.source, self.name, globals_, props, {p: "f" for p in props},
                                      arrays=arrays, prop_widths=prop_widths)
        return set(writes)

    @property
    def writes(self):
        if self._writes is None:
            raise RuntimeError("PythonStep %s is translated at setup" % self.name)
        return self._writes

    def __repr__(self):
        return "PythonStep(%r)" % self.name
