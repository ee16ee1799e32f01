"""Breed: property registry and step functions by priority.

Same interface as sagesim/breed.py:8-99 (register_property with defaults,
max_dims and neighbor_visible; register_step_func with module path,
priority and no_double_buffer). Step functions here are the step objects of
sagesim_gb300.steps (builtin SIR / opinion steps, or CUDA C++ steps compiled
with NVRTC) instead of CuPy-JIT Python functions.
"""
import inspect
from collections import OrderedDict
from math import nan
from pathlib import Path


class Breed:
    def __init__(self, name):
        self._properties = OrderedDict()
        self._prop2pos = {}
        self._name = name
        self._step_funcs = {}
        self._breedidx = -1
        self._num_properties = 0
        self._prop2maxdims = {}
        self._prop2neighbor_visible = {}
        self._no_double_buffer_props = set()

    @property
    def name(self):
        return self._name

    @property
    def properties(self):
        return self._properties

    @property
    def step_funcs(self):
        return self._step_funcs

    @property
    def prop2neighbor_visible(self):
        return self._prop2neighbor_visible

    @property
    def no_double_buffer_props(self):
        return self._no_double_buffer_props

    def register_property(self, name, default=nan, max_dims=None, neighbor_visible=True):
        """sagesim/breed.py:40-61."""
        self._properties[name] = default
        self._prop2pos[name] = self._num_properties
        self._num_properties += 1
        self._prop2maxdims[name] = max_dims
        self._prop2neighbor_visible[name] = neighbor_visible

    def register_step_func(self, step_func, module_fpath=None, priority=0, no_double_buffer=None):
        """sagesim/breed.py:68-99: one step per priority; no_double_buffer names
        properties written in place (visible to later priorities in the same tick)."""
        if module_fpath is None:
            try:
                module_fpath = inspect.getfile(type(step_func))
            except TypeError:
                module_fpath = __file__
        self._step_funcs[priority] = (step_func, str(Path(module_fpath).resolve()))
        if no_double_buffer:
            self._no_double_buffer_props.update(no_double_buffer)
