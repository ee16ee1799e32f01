"""NetworkSpace: agent adjacency as Python sets (or insertion-ordered lists).

Same interface and semantics as sagesim/space.py:50-145: add_agent links the
agent's `locations` property to its container; connect_agents is undirected
unless directed=True; ordered=True keeps insertion order and drops
duplicates. set_csr() and set_edges() are additions for large graphs: they
install a whole adjacency at once (CSR arrays or an edge list, in agent ids)
without per-edge Python calls.

Every change of the adjacency bumps a version counter; a Model that has been
set up installs the new adjacency at its next simulate() (the reference picks
up topology edits only when its device buffers are rebuilt).
"""
import numpy as np


class Space:
    def __init__(self, neighbor_compute_func, locations_max_dims, locations_defaults):
        self._neighbor_compute_func = neighbor_compute_func
        self._locations = []
        self._agent_factory = None
        self._csr = None
        self._id_edges = None
        self._version = 0


def _network_space_compute_neighbors(agent_locations):
    return agent_locations


class NetworkSpace(Space):
    def __init__(self, ordered=False):
        self._ordered = ordered
        if ordered:
            self._locations_set = {}
        super().__init__(_network_space_compute_neighbors, [0], [])

    @property
    def ordered(self):
        return self._ordered

    def add_agent(self, agent):
        container = [] if self._ordered else set()
        self._locations.append(container)
        if self._ordered:
            self._locations_set[agent] = set()
        if self._agent_factory is not None:
            self._agent_factory.set_agent_property_value("locations", agent, self._locations[agent])

    def bulk_add_agents(self, total_agents):
        if self._ordered:
            self._locations = [[] for _ in range(total_agents)]
            self._locations_set = {i: set() for i in range(total_agents)}
        else:
            self._locations = [set() for _ in range(total_agents)]

    def _materialize(self):
        """Turns an installed CSR or edge list back into per-agent containers
        (before edits)."""
        if self._id_edges is not None:
            self._csr = self._edges_to_csr()
            self._id_edges = None
        if self._csr is None:
            return
        off, idx = self._csr
        self._csr = None
        for i in range(off.size - 1):
            row = [int(v) for v in idx[off[i]:off[i + 1]]]
            if self._ordered:
                self._locations[i][:] = row
                self._locations_set[i] = set(row)
            else:
                self._locations[i].clear()
                self._locations[i].update(row)

    def get_location(self, agent_id):
        self._materialize()
        return self._locations[agent_id]

    def get_neighbors(self, agent_id):
        self._materialize()
        return self._neighbor_compute_func(self._locations)[agent_id]

    def connect_agents(self, agent_0, agent_1, directed=False):
        self._materialize()
        self._version += 1
        agent_0 = int(agent_0)
        agent_1 = int(agent_1)
        if self._ordered:
            if agent_1 not in self._locations_set[agent_0]:
                self._locations_set[agent_0].add(agent_1)
                self._locations[agent_0].append(agent_1)
            if not directed and agent_0 not in self._locations_set[agent_1]:
                self._locations_set[agent_1].add(agent_0)
                self._locations[agent_1].append(agent_0)
        else:
            self._locations[agent_0].add(agent_1)
            if not directed:
                self._locations[agent_1].add(agent_0)

    def disconnect_agents(self, agent_0, agent_1, directed=False):
        self._materialize()
        self._version += 1
        agent_0 = int(agent_0)
        agent_1 = int(agent_1)
        if self._ordered:
            if agent_1 in self._locations_set[agent_0]:
                self._locations_set[agent_0].discard(agent_1)
                self._locations[agent_0].remove(agent_1)
            if not directed and agent_0 in self._locations_set[agent_1]:
                self._locations_set[agent_1].discard(agent_0)
                self._locations[agent_1].remove(agent_0)
        else:
            self._locations[agent_0].discard(agent_1)
            if not directed:
                self._locations[agent_1].discard(agent_0)

    def set_csr(self, offsets, indices):
        """Installs the adjacency of agents 0..n-1 (rows of agent ids) at once."""
        off = np.ascontiguousarray(offsets, dtype=np.int32)
        idx = np.ascontiguousarray(indices, dtype=np.int32)
        if off.size - 1 != len(self._locations):
            raise ValueError("CSR has %d rows but the space holds %d agents"
                             % (off.size - 1, len(self._locations)))
        self._csr = (off, idx)
        self._id_edges = None
        self._version += 1

    def set_edges(self, src_ids, dst_ids, directed=False):
        """Installs the adjacency as an edge list in agent ids (any int64 ids the
        model's agents carry: creation-order ids here). The CSR is built on the GPU
        at setup: an open-addressing hash table in HBM maps ids to buffer indices
        (the reference's convert_agent_ids_to_indices, sagesim/model.py:31-110),
        and the rows are sorted (or kept in first-connection order for an ordered
        space), repeated edges dropped, as connect_agents would leave them."""
        src = np.ascontiguousarray(src_ids, dtype=np.int64)
        dst = np.ascontiguousarray(dst_ids, dtype=np.int64)
        if src.shape != dst.shape:
            raise ValueError("src_ids and dst_ids differ in length")
        self._id_edges = (src, dst, bool(directed))
        self._csr = None
        self._version += 1

    def _edges_to_csr(self):
        """CSR (agent ids) of the installed edge list, rows as connect_agents
        would leave them: each edge added in list order (both directions unless
        directed), repeats dropped, rows sorted or (ordered) in first-connection
        order."""
        src, dst, directed = self._id_edges
        n = len(self._locations)
        if src.size and (min(src.min(), dst.min()) < 0 or max(src.max(), dst.max()) >= n):
            raise ValueError("an edge names an agent id outside 0..%d" % (n - 1))
        if directed:
            rows, cols = src, dst
        else:  # edge k adds src->dst, then dst->src
            rows = np.stack([src, dst], axis=1).reshape(-1)
            cols = np.stack([dst, src], axis=1).reshape(-1)
        key = rows * np.int64(max(n, 1)) + cols
        _, first = np.unique(key, return_index=True)
        if self._ordered:
            first.sort()
            first = first[np.argsort(rows[first], kind="stable")]
        rows, cols = rows[first], cols[first]
        off = np.zeros(n + 1, dtype=np.int32)
        np.cumsum(np.bincount(rows, minlength=n), out=off[1:])
        return off, cols.astype(np.int32)

    def _rows(self):
        """(offsets, indices) by agent id, from the CSR or the containers."""
        if self._id_edges is not None:
            return self._edges_to_csr()
        if self._csr is not None:
            return self._csr
        from .csr import build_csr_from_ragged

        return build_csr_from_ragged(self._locations)
