"""AgentFactory: host-side agent store of the drop-in API.

Mirrors sagesim/agent.py:24-473 for one process: property 0 is `breed`,
property 1 is `locations` (the agent's neighbour container in the space),
user properties follow in registration order; agent ids are creation order;
every agent holds every property (defaults from the registering breed). There
are no MPI ranks: the engine runs on one GPU. create_agents_bulk is an
addition that creates many agents from arrays without a Python call per
agent.
"""
from collections import OrderedDict
from copy import copy

import numpy as np


class AgentFactory:
    def __init__(self, space, verbose_timing=False):
        self._breeds = OrderedDict()
        self._space = space
        self._verbose_timing = verbose_timing
        self._space._agent_factory = self
        self._num_breeds = 0
        self._num_agents = 0
        self._property_name_2_agent_data_tensor = OrderedDict({"breed": [], "locations": []})
        self._property_name_2_defaults = OrderedDict({"breed": 0, "locations": []})
        self._property_name_2_index = {"breed": 0, "locations": 1}
        self._property_name_2_neighbor_visible = OrderedDict({"breed": True, "locations": False})
        self._agent2breed = []
        self._bulk = []  # (first_id, count, breed_idx, {name: array}) blocks from create_agents_bulk

    @property
    def breeds(self):
        return self._breeds.values()

    @property
    def num_agents(self):
        return self._num_agents

    @property
    def num_properties(self):
        return len(self._property_name_2_agent_data_tensor)

    def register_breed(self, breed):
        """sagesim/agent.py:280-309."""
        breed._breedidx = self._num_breeds
        self._num_breeds += 1
        self._breeds[breed.name] = breed
        for name, default in breed.properties.items():
            visible = breed.prop2neighbor_visible.get(name, True)
            if name in self._property_name_2_agent_data_tensor:
                self._property_name_2_defaults[name] = default
                self._property_name_2_neighbor_visible[name] = (
                    self._property_name_2_neighbor_visible.get(name, False) or visible)
            else:
                self._property_name_2_index[name] = len(self._property_name_2_agent_data_tensor)
                self._property_name_2_agent_data_tensor[name] = []
                self._property_name_2_defaults[name] = default
                self._property_name_2_neighbor_visible[name] = visible

    def _flush_bulk(self):
        """Appends bulk-created agents to the per-property lists (on first need)."""
        if not self._bulk:
            return
        for first, count, bidx, arrays in self._bulk:
            for name, col in self._property_name_2_agent_data_tensor.items():
                if name == "breed":
                    col.extend([bidx] * count)
                elif name == "locations":
                    col.extend(self._space._locations[first:first + count])
                elif name in arrays:
                    col.extend(arrays[name].tolist())
                else:
                    d = self._property_name_2_defaults[name]
                    col.extend(copy(d) for _ in range(count))
        self._bulk = []

    def create_agent(self, breed, rank=None, **kwargs):
        """sagesim/agent.py:311-370 (rank is accepted and ignored: one GPU)."""
        if breed.name not in self._breeds:
            raise ValueError("Fatal: unregistered breed %s" % breed.name)
        self._flush_bulk()
        agent_id = self._num_agents
        bidx = self._breeds[breed.name]._breedidx
        self._agent2breed.append(bidx)
        for name, col in self._property_name_2_agent_data_tensor.items():
            if name == "breed":
                col.append(bidx)
            else:
                col.append(kwargs.get(name, copy(self._property_name_2_defaults[name])))
        self._num_agents += 1
        return agent_id

    def create_agents_bulk(self, breed, count, **arrays):
        """Creates `count` agents of `breed`; keyword arrays give per-agent values.
        Returns the first new agent id (ids are consecutive)."""
        if breed.name not in self._breeds:
            raise ValueError("Fatal: unregistered breed %s" % breed.name)
        first = self._num_agents
        bidx = self._breeds[breed.name]._breedidx
        cols = {}
        for k, v in arrays.items():
            if k not in self._property_name_2_agent_data_tensor:
                raise ValueError("%s not a property of any breed" % k)
            a = np.asarray(v)
            if a.shape[0] != count:
                raise ValueError("%s has %d rows, expected %d" % (k, a.shape[0], count))
            cols[k] = a
        self._bulk.append((first, count, bidx, cols))
        self._agent2breed.extend([bidx] * count)
        self._num_agents += count
        return first

    def get_agent_property_value(self, property_name, agent_id):
        self._flush_bulk()
        return self._property_name_2_agent_data_tensor[property_name][agent_id]

    def set_agent_property_value(self, property_name, agent_id, value):
        if property_name not in self._property_name_2_agent_data_tensor:
            raise ValueError("%s not a property of any breed" % property_name)
        self._flush_bulk()
        col = self._property_name_2_agent_data_tensor[property_name]
        if property_name == "locations" and agent_id == len(col):
            col.append(value)  # NetworkSpace.add_agent links the container
            return
        col[agent_id] = value

    def get_agents_with(self, query):
        self._flush_bulk()
        names = list(self._property_name_2_agent_data_tensor.keys())
        out = {}
        for aid in range(self._num_agents):
            props = {n: self._property_name_2_agent_data_tensor[n][aid] for n in names}
            if query(**props):
                out[aid] = props
        return out

    def column(self, name):
        """All agents' values of a property as a list (agent-id order)."""
        self._flush_bulk()
        return self._property_name_2_agent_data_tensor[name]
