"""Model: the drop-in SAGESim Model over the GB300 engine.

Public interface of sagesim/model.py:355-998 for the per-tick agent step:
register_breed, create_agent_of_breed, register/set/get_global_property,
set_seed, set_agent_logical_id, setup, simulate, get/set_agent_property_value,
get_breed_data, get_breed_agent_ids, register/get_breed_local_array,
set_property_neighbor_visible, reset, save, load. setup() does what the reference's setup() plus its
first-simulate buffer build do (sagesim/model.py:682-886, 1020-1274): agents
are stably sorted by breed (sagesim/agent.py:438-473), the NetworkSpace
becomes a device CSR of buffer indices, every property a structure-of-arrays
column (int32 when all its values are integers, float32 otherwise; list
properties are padded float32 rows, NaN-padded as in
sagesim/internal_utils.py:189-230), and every breed's steps are added to the
engine over that breed's index range. simulate() then runs the ticks on the
GPU with the tick counter continuing across calls (model.py:1576).
"""
import math
import pickle
import time

import numpy as np

from . import _native as N
from .agent import AgentFactory
from .breed import Breed  # noqa: F401  (re-exported for drop-in imports)
from .engine import Engine
from .steps import CudaStep, OpinionStep, PythonStep, SIRStep


class Model:
    def __init__(self, space, threads_per_block=32, step_function_file_path="step_func_code.py",
                 verbose_timing=False, agent_slack_factor=1.5, csr_slack_factor=2.0,
                 min_capacity=64, device=0):
        # threads_per_block, the generated-module path and the slack factors
        # are accepted for compatibility; the engine sizes its own buffers and
        # compiles steps in memory.
        self._threads_per_block = threads_per_block
        self._step_function_file_path = step_function_file_path
        self._verbose_timing = verbose_timing
        self._agent_slack_factor = agent_slack_factor
        self._csr_slack_factor = csr_slack_factor
        self._min_capacity = min_capacity
        self._device = device
        self._agent_factory = AgentFactory(space, verbose_timing=verbose_timing)
        self._is_setup = False
        self._global_tensors = []
        self._global_names = {}
        self._globals_dirty = True
        self._seed = int(np.random.randint(0, 2**31))
        self._logical_id_map = {}
        self.tick = 0
        self._engine = None
        self._breed_local_arrays = []
        self._neighbor_visible_override = {}
        self._tick_timings = []

    # ---- properties of the model ------------------------------------------------
    @property
    def verbose_timing(self):
        return self._verbose_timing

    @verbose_timing.setter
    def verbose_timing(self, value):
        self._verbose_timing = value

    def register_breed(self, breed):
        """sagesim/model.py:411-414."""
        if self._agent_factory.num_agents > 0:
            raise Exception("All breeds must be registered before agents are created!")
        self._agent_factory.register_breed(breed)

    def create_agent_of_breed(self, breed, add_to_space=True, rank=None, **kwargs):
        """sagesim/model.py:416-420."""
        agent_id = self._agent_factory.create_agent(breed, rank=rank, **kwargs)
        if add_to_space:
            self.get_space().add_agent(agent_id)
        return agent_id

    def create_agents_bulk(self, breed, count, **arrays):
        """Creates `count` agents at once (per-agent values from arrays); their
        adjacency must be installed with NetworkSpace.set_csr before setup()."""
        first = self._agent_factory.create_agents_bulk(breed, count, **arrays)
        self.get_space()._locations.extend([None] * count)
        return first

    def get_space(self):
        return self._agent_factory._space

    def get_agents_with(self, query):
        return self._agent_factory.get_agents_with(query)

    # ---- globals, seed, logical ids -------------------------------------------------
    def register_global_property(self, property_name, value):
        """sagesim/model.py:588-597 (stored as float64)."""
        idx = len(self._global_tensors)
        self._global_tensors.append(np.atleast_1d(np.asarray(value, dtype=np.float64)).copy())
        self._global_names[property_name] = idx
        self._globals_dirty = True
        return idx

    def set_global_property_value(self, property_name, value):
        idx = self._global_names[property_name]
        self._global_tensors[idx][:] = np.atleast_1d(np.asarray(value, dtype=np.float64))
        self._globals_dirty = True

    def get_global_property_value(self, property_name):
        arr = self._global_tensors[self._global_names[property_name]]
        return float(arr.flat[0]) if arr.size == 1 else arr.copy()

    @property
    def globals(self):
        return {n: self._global_tensors[i] for n, i in self._global_names.items()}

    def set_seed(self, seed):
        self._seed = int(seed)
        if self._engine is not None:
            self._engine.set_seed(self._seed)

    def set_agent_logical_id(self, agent_id, logical_id):
        """sagesim/model.py:656-667: RNG key of the agent (call before setup())."""
        self._logical_id_map[int(agent_id)] = int(logical_id)

    def load_partition(self, partition_file, format="auto"):
        """Accepted for compatibility. With one GPU there is no rank to assign;
        locality relabelling is graphs.partition_relabel + Engine-level input."""
        self._partition_file = partition_file

    def register_breed_local_array(self, name, breed, shape_per_agent, neighbor_visible=False):
        """sagesim/model.py:620-645: a float32 array with one row of
        shape_per_agent per agent of `breed`, zeros at setup. Every step function
        receives it after the properties as two parameters, the array and its
        index map (row of agent i = idx[i], -1 for agents of other breeds). A
        written array is double-buffered unless a step's no_double_buffer names
        it. neighbor_visible adds ghost rows across ranks in the reference; on one
        GPU every row is local."""
        if self._is_setup:
            raise RuntimeError("register breed-local arrays before setup()")
        shape = tuple(int(d) for d in np.atleast_1d(shape_per_agent))
        if not shape or min(shape) < 1:
            raise ValueError("shape_per_agent must hold positive sizes")
        if any(b["name"] == name for b in self._breed_local_arrays):
            raise ValueError("breed-local array %r is already registered" % name)
        self._breed_local_arrays.append({"name": name, "breed": breed, "shape_per_agent": shape,
                                         "neighbor_visible": bool(neighbor_visible)})
        return len(self._breed_local_arrays) - 1

    def get_breed_local_array(self, name):
        """sagesim/model.py:647-650: the array's current contents, shape
        (rows, *shape_per_agent), rows = the breed's agent count (at least 1)."""
        bla = next(b for b in self._breed_local_arrays if b["name"] == name)
        if self._engine is None:
            raise RuntimeError("breed-local arrays live on the device: call setup() first")
        a = self._engine.get_property(self._pid["sgbla_" + name])
        return a.reshape((-1,) + bla["shape_per_agent"])

    # ---- setup -------------------------------------------------------------------------
    def setup(self, use_gpu=True, skip_priority_barriers=False):
        """sagesim/model.py:682-886 plus the first-simulate buffer build."""
        self._use_gpu = use_gpu
        self._skip_priority_barriers = skip_priority_barriers
        self.tick = 0
        self._collect_steps()
        self._build_host_arrays()
        self._build_engine()
        self._is_setup = True

    def _collect_steps(self):
        af = self._agent_factory
        steps = []  # (priority, breed_idx, step, module_path)
        for breed in af.breeds:
            for priority, (fn, path) in breed.step_funcs.items():
                if not isinstance(fn, (SIRStep, OpinionStep, CudaStep, PythonStep)):
                    # SAGESim's own Python step function: translated at setup
                    fn = PythonStep(fn, path)
                steps.append((priority, breed._breedidx, fn, path))
        steps.sort(key=lambda s: (s[0], s[1]))
        self._steps = steps
        nodb = set()
        for breed in af.breeds:
            nodb |= set(breed.no_double_buffer_props)
        self._no_double_buffer = nodb

    def _build_host_arrays(self):
        """Host arrays in buffer order: CSR, properties, logical ids, breed ranges."""
        af = self._agent_factory
        n = af.num_agents
        breeds = np.asarray(af._agent2breed, dtype=np.int64)
        order = np.argsort(breeds, kind="stable")  # buffer index -> agent id
        pos = np.empty(n, dtype=np.int32)
        pos[order] = np.arange(n, dtype=np.int32)
        self._order, self._pos = order, pos
        nb = af._num_breeds
        counts = np.bincount(breeds, minlength=nb) if n else np.zeros(nb, dtype=np.int64)
        starts = np.concatenate([[0], np.cumsum(counts)])
        self._breed_ranges = {b: (int(starts[b]), int(starts[b + 1])) for b in range(nb)}

        space = self.get_space()
        self._id_edges = getattr(space, "_id_edges", None)
        if self._id_edges is not None:
            self._csr = None  # built on the GPU from the id edge list at engine build
        else:
            if any(c is None for c in space._locations) and space._csr is None:
                raise RuntimeError("agents created in bulk need NetworkSpace.set_csr or set_edges before setup()")
            off, idx = space._rows()
            if off.size - 1 != n:
                raise RuntimeError("the space holds %d agents, the model %d" % (off.size - 1, n))
            from .graphs import permute_csr

            self._csr = permute_csr(off, idx, pos) if n else (off, idx)

        lids = np.arange(n, dtype=np.int64)[order]  # agent id of each buffer slot
        if self._logical_id_map:
            keys = np.fromiter(self._logical_id_map.keys(), dtype=np.int64)
            vals = np.fromiter(self._logical_id_map.values(), dtype=np.int64)
            by_agent = np.arange(n, dtype=np.int64)
            by_agent[keys] = vals
            lids = by_agent[order]
        # the reference keeps ids and logical ids in float32 (model.py:1085-1096)
        lids = lids.astype(np.float32).astype(np.int64)
        self._lids = None if np.array_equal(lids, np.arange(n)) else lids

        self._props = {}  # name -> (numpy dtype, width, column in buffer order)
        for name, pidx in sorted(af._property_name_2_index.items(), key=lambda kv: kv[1]):
            if pidx < 2:
                continue
            col = af.column(name)
            default = af._property_name_2_defaults[name]
            if isinstance(default, (list, tuple, np.ndarray)) or (col and isinstance(col[0], (list, tuple, np.ndarray))):
                width = max([len(r) if isinstance(r, (list, tuple, np.ndarray)) else 1 for r in col] + [1])
                arr = np.full((n, width), np.nan, dtype=np.float32)
                for a, r in enumerate(col):
                    if isinstance(r, (list, tuple, np.ndarray)):
                        arr[a, :len(r)] = r
                    else:
                        arr[a, 0] = r
                self._props[name] = (np.float32, width, arr[order])
            else:
                vals = np.asarray(col)
                integral = vals.dtype.kind in "iub" or (
                    vals.dtype.kind == "f" and vals.size and np.all(np.isfinite(vals)) and
                    np.all(vals == np.round(vals)) and not isinstance(default, float))
                if integral and vals.size:
                    integral = bool(np.all(vals >= -2**31) and np.all(vals < 2**31))
                if integral:
                    self._props[name] = (np.int32, 1, vals.astype(np.int32)[order])
                else:
                    self._props[name] = (np.float32, 1, vals.astype(np.float32)[order])
        self._settle_written_types()

    def _settle_written_types(self):
        """The reference keeps every property in float32 (sagesim/internal_utils.py:
        189-230, sagesim/model.py:1085), so a step may store a fraction into a
        property that started as whole numbers. A property inferred as int32 stays
        int32 only when no Python-dialect step writes it, or when a builtin SIR
        step (whose state is int32) does; otherwise it is float32, as in the
        reference."""
        py_written, sir_written = set(), set()
        gnames = [k for k, _ in sorted(self._global_names.items(), key=lambda kv: kv[1])]
        arrays = [(b["name"], b["shape_per_agent"]) for b in self._breed_local_arrays]
        widths = {k: v[1] for k, v in self._props.items()}
        for _, _, fn, _ in self._steps:
            if isinstance(fn, PythonStep):
                py_written |= fn.written(gnames, list(self._props), arrays, widths)
            elif isinstance(fn, SIRStep):
                sir_written.add(fn.state)
        for name in sorted(py_written - sir_written):
            if name in self._props and self._props[name][0] == np.int32:
                dt, width, arr = self._props[name]
                self._props[name] = (np.float32, width, arr.astype(np.float32))

    def _global_offsets(self):
        offs, flat = {}, []
        for name, gi in self._global_names.items():
            offs[name] = len(flat)
            flat.extend(self._global_tensors[gi].ravel().tolist())
        return offs, np.asarray(flat, dtype=np.float64)

    def _scalar_global(self, name):
        if name not in self._global_names:
            raise KeyError("global %r is not registered" % name)
        return float(self._global_tensors[self._global_names[name]].flat[0])

    def _build_engine(self):
        if self._engine is not None:
            self._engine.close()
        e = Engine(device=self._device)
        self._install_graph(e)
        if self._lids is not None:
            e.set_logical_ids(self._lids)
        e.set_seed(self._seed)
        goffs, gflat = self._global_offsets()
        self._goffs = goffs
        e.set_globals(gflat)
        self._globals_dirty = False
        # Python-dialect steps: globals and properties mapped by position
        gnames = [k for k, _ in sorted(self._global_names.items(), key=lambda kv: kv[1])]
        pdt = {k: ("i" if v[0] == np.int32 else "f") for k, v in self._props.items()}
        arrays = [(b["name"], b["shape_per_agent"]) for b in self._breed_local_arrays]
        widths = {k: v[1] for k, v in self._props.items()}
        self._steps = [(pr, bi, (fn.translate(gnames, list(self._props), pdt, arrays, widths)
                                 if isinstance(fn, PythonStep) else fn), path) for pr, bi, fn, path in self._steps]
        self._pid = {}
        for name, (dt, width, arr) in self._props.items():
            self._pid[name] = e.add_property(name, dt, width, init=arr,
                                             double_buffered=name not in self._no_double_buffer)
        # breed-local arrays (sagesim/model.py:1215-1270): rows in breed-range
        # order, index map from buffer index to row
        n = self._order.size
        for bla in self._breed_local_arrays:
            b, en = self._breed_ranges.get(bla["breed"]._breedidx, (0, 0))
            width = int(np.prod(bla["shape_per_agent"]))
            key = "sgbla_" + bla["name"]
            self._pid[key] = e.add_array(key, np.float32, width, max(en - b, 1),
                                         double_buffered=bla["name"] not in self._no_double_buffer)
            idx_map = np.full(n, -1, dtype=np.int32)
            idx_map[b:en] = np.arange(en - b, dtype=np.int32)
            self._pid[key + "_idx"] = e.add_property(key + "_idx", np.int32, 1, init=idx_map,
                                                     double_buffered=False)
        writers = {}
        for _, bidx, fn, _ in self._steps:
            for w in fn.writes:
                writers.setdefault(w, []).append(fn)
        self._builtin_ids = []
        for priority, bidx, fn, _ in self._steps:
            b, en = self._breed_ranges[bidx]
            if isinstance(fn, SIRStep):
                if fn.strategy:
                    strategy = fn.strategy
                elif len(self._steps) == 1:
                    strategy = "frontier"  # the only step: active-list ticks, state in place
                elif len(writers.get(fn.state, [])) == 1:
                    strategy = "count"
                else:
                    strategy = "pull"
                sid = e.add_sir(self._pid[fn.state], self._scalar_global(fn.p_infection),
                                self._scalar_global(fn.p_recovery), variant=fn.variant, strategy=strategy,
                                codes=fn.codes, begin=b, end=en, priority=priority)
                self._builtin_ids.append((sid, fn, strategy, b, en, priority))
            elif isinstance(fn, OpinionStep):
                e.add_opinion(self._pid[fn.opinion], self._pid[fn.weights],
                              self._scalar_global(fn.noise_sigma), begin=b, end=en, priority=priority)
            else:
                defs = "".join("#define PROP_%s %d\n" % (k, v) for k, v in self._pid.items())
                defs += "".join("#define G_%s %d\n" % (k, v) for k, v in goffs.items())
                e.compile_step(defs + fn.source, fn.entry, [self._pid[w] for w in fn.writes],
                               begin=b, end=en, priority=priority)
        self._engine = e

    def _install_graph(self, e):
        """Hands the space's adjacency, in buffer order, to engine e."""
        space = self.get_space()
        if self._csr is None:
            src, dst, directed = self._id_edges
            # buffer slot k holds agent id self._order[k]; the engine maps ids on the GPU
            e.set_graph_from_ids(self._order.astype(np.int64), src, dst, symmetric=not directed,
                                 ordered=space.ordered)
        else:
            off, idx = self._csr
            e.set_graph(off, idx, ordered=space.ordered)
        self._graph_version = space._version

    def _refresh_graph(self):
        """Topology edited since the engine was built (connect_agents,
        disconnect_agents, set_csr, set_edges): the new adjacency replaces the
        device CSR; agent state and tick are kept."""
        space = self.get_space()
        if space._version == self._graph_version:
            return
        self._id_edges = space._id_edges
        if self._id_edges is not None:
            self._csr = None
        else:
            from .graphs import permute_csr

            off, idx = space._rows()
            n = self._order.size
            if off.size - 1 != n:
                raise RuntimeError("the space holds %d agents, the model %d" % (off.size - 1, n))
            self._csr = permute_csr(off, idx, self._pos) if n else (off, idx)
        self._install_graph(self._engine)

    def _refresh_globals(self):
        if not self._globals_dirty:
            return
        _, gflat = self._global_offsets()
        self._engine.set_globals(gflat)
        for sid, fn, strategy, b, en, priority in self._builtin_ids:
            self._engine.update_sir(sid, self._pid[fn.state], self._scalar_global(fn.p_infection),
                                    self._scalar_global(fn.p_recovery), variant=fn.variant,
                                    strategy=strategy, codes=fn.codes, begin=b, end=en, priority=priority)
        self._globals_dirty = False

    # ---- simulate ---------------------------------------------------------------------
    def simulate(self, ticks, sync_workers_every_n_ticks=1):
        """sagesim/model.py:961-998: runs `ticks` ticks from the current tick."""
        if not self._is_setup:
            raise RuntimeError("call setup() before simulate()")
        if self._engine is None:
            self._build_host_arrays()
            self._build_engine()
        self._refresh_globals()
        self._refresh_graph()
        t0 = time.perf_counter()
        _, tot = self._engine.run(self.tick, int(ticks), stats=self._verbose_timing)
        wall = time.perf_counter() - t0
        if self._verbose_timing:
            self._tick_timings.append({"ticks": ticks, "wall_s": wall, "device_ms": tot.device_ms})
            print("[SAGESim-GB300] ticks %d-%d: %.3f ms device, %.3f ms wall, %d edge visits"
                  % (self.tick, self.tick + ticks - 1, tot.device_ms, wall * 1e3, tot.edge_visits),
                  flush=True)
        self.tick += int(ticks)

    # ---- readout --------------------------------------------------------------------------
    def _value_from_engine(self, agent_id, name):
        dt, width, _ = self._props[name]
        v = self._engine.get_property(self._pid[name], int(self._pos[agent_id]), 1)
        if width > 1:
            return v.reshape(-1).tolist()
        return int(v[0]) if dt == np.int32 else float(v[0])

    def get_agent_property_value(self, id, property_name):
        """sagesim/model.py:422-450."""
        if self._engine is not None and property_name in self._props:
            return self._value_from_engine(id, property_name)
        if property_name == "locations":
            return self.get_space().get_location(id)
        return self._agent_factory.get_agent_property_value(property_name=property_name, agent_id=id)

    def set_agent_property_value(self, id, property_name, value):
        """sagesim/model.py:452-459. After setup the new value is written to the
        device in place (the reference instead rebuilds all device buffers from
        its host copy, which it has not refreshed since the last simulate)."""
        self._agent_factory.set_agent_property_value(property_name=property_name, agent_id=id,
                                                     value=value)
        if self._engine is not None and property_name in self._props:
            dt, width, _ = self._props[property_name]
            row = np.full(width, np.nan, dtype=dt) if width > 1 else np.array([value], dtype=dt)
            if width > 1:
                row[:len(value)] = value
            self._engine.set_property(self._pid[property_name], row, first=int(self._pos[id]))

    def get_breed_data(self, breed_name, property_name, local=False):
        """sagesim/model.py:464-490: the breed's values in buffer order."""
        bidx = self._agent_factory._breeds[breed_name]._breedidx
        b, e = self._breed_ranges[bidx] if self._is_setup else (0, 0)
        if self._engine is None:
            ids = [a for a in range(self._agent_factory.num_agents) if self._agent_factory._agent2breed[a] == bidx]
            return [self._agent_factory.get_agent_property_value(property_name, a) for a in ids]
        v = self._engine.get_property(self._pid[property_name], b, e - b)
        return v.tolist()

    def get_breed_agent_ids(self, breed_name, local=False):
        """sagesim/model.py:492-515: the breed's agent ids in buffer order, as
        the float32 values the reference keeps them in."""
        bidx = self._agent_factory._breeds[breed_name]._breedidx
        if not self._is_setup:
            raise RuntimeError("call setup() before get_breed_agent_ids()")
        b, e = self._breed_ranges.get(bidx, (0, 0))
        return self._order[b:e].astype(np.float32)

    def set_property_neighbor_visible(self, property_name, visible):
        """sagesim/model.py:398-409: the flag only selects what crosses ranks in
        the reference's ghost exchange; one GPU holds every agent, so it is
        recorded and changes nothing here."""
        if self._is_setup:
            raise RuntimeError("Cannot change neighbor_visible after setup()")
        af = self._agent_factory
        if property_name not in af._property_name_2_index:
            raise ValueError("Unknown property: %s" % property_name)
        self._neighbor_visible_override[property_name] = bool(visible)

    def _sync_to_host(self):
        """Copies the device values of every property into the host store."""
        af = self._agent_factory
        for name in self._props:
            vals = self.get_property_array(name)
            col = af.column(name)
            for a in range(len(col)):
                col[a] = vals[a].tolist() if vals.ndim > 1 else vals[a].item()

    def __getstate__(self):
        # the device engine is not picklable: its property values go to the
        # host store and the next simulate() builds a new engine from them
        if self._engine is not None:
            self._sync_to_host()
        state = self.__dict__.copy()
        state["_engine"] = None
        return state

    def save(self, app, fpath):
        """sagesim/model.py:1288-1298: pickles `app` (a Model) to fpath. Property
        values and the tick are kept; breed-local arrays restart from zeros
        when the loaded model next runs."""
        with open(fpath, "wb") as fout:
            pickle.dump(app, fout)

    def load(self, fpath):
        """sagesim/model.py:1300-1309: the model pickled at fpath."""
        with open(fpath, "rb") as fin:
            return pickle.load(fin)

    def get_property_array(self, property_name):
        """All agents' values by agent id as a numpy array (one device copy)."""
        v = self._engine.get_property(self._pid[property_name])
        out = np.empty_like(v)
        out[self._order] = v
        return out

    def reset(self):
        """sagesim/model.py:944-958: tick 0, device state copied back to the
        host store, device buffers freed (rebuilt on the next simulate)."""
        self.tick = 0
        if self._engine is not None:
            self._sync_to_host()
            self._engine.close()
            self._engine = None
        self._globals_dirty = True
