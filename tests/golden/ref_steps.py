"""Step functions written in the reference's own dialect (CuPy-JIT Python).

Used only by make_golden.py, which runs them through the reference's real
Model.setup()/simulate() pipeline (AST rewrite, seed injection, double
buffering, fused kernel) on CPU to produce golden fixtures. They are user
model code for the reference, not part of this package.

sir_per_neighbour_step: per-infected-neighbour SIR. An infected agent recovers
  when philox(salt 1) < p_recovery. A susceptible agent scans its neighbours in
  CSR order; the j-th infected neighbour found (j = 0, 1, ...) draws
  philox(salt 2 + j) and the first draw below p_infection infects it.
host_step / site_step: two breeds with breed-local arrays and no property
  writes. Hosts keep health[row] = (status 0 S / 1 I / 2 R, decayed
  infected-neighbour count, ticks infected, sum of the neighbouring hosts'
  decayed counts) in a double-buffered float32[4] array (status read from the
  int property state - 1 at tick 0); a susceptible host is infected with
  probability p_infection * (decayed count + 0.1 * neighbouring sites' load).
  Sites (priority 1) write load[row][tick % 2] = (neighbouring hosts' ticks
  infected, infected neighbouring hosts at tick start) in place
  (no_double_buffer) and add 0.5 to the other slot's count.
measures_step: SIR with per-agent protective measures (a float32[4] list
  property) and a float32[5] state-history ring, in the style of the SIR example
  shipped with the reference but drawing philox(salt 1) instead of Python's
  random(): a susceptible agent is infected when some neighbour is infected and
  the draw is below p_infection * (1 - sum of pairwise products of the two
  agents' measures / 16); rows are read through local aliases and len().
helpers_step: per-neighbour SIR written with the device helpers of
  sagesim/utils.py (get_num_neighbors / get_neighbor on the CSR names,
  get_ / set_this_agent_data_from_tensor) plus a float32 visit counter.
fraction_step: SIR whose two extra properties start as whole numbers (an int
  default and int initial values) and are written fractions: a susceptible
  agent with infected neighbours gains 0.25 immunity per tick (up to 1) and is
  infected when philox(salt 1) < p_infection * (1 - immunity); every agent's
  load becomes (load + infected neighbours) / 2.
opinion_step: weighted mean of the first min(deg, 8) ordered neighbours'
  opinions (float32 arithmetic in row order, normalised by the sum of |w|),
  plus noise_sigma * rand_normal(salt 1) in float64, clamped to [0, 1].
"""
import cupy as cp
from cupyx import jit

from sagesim.math_utils import rand_normal, rand_uniform_philox
from sagesim.utils import (
    get_neighbor,
    get_num_neighbors,
    get_this_agent_data_from_tensor,
    set_this_agent_data_from_tensor,
)


@jit.rawkernel(device="cuda")
def sir_per_neighbour_step(
    tick, agent_index, p_infection, p_recovery,
    agent_ids, breeds, locations, state_tensor,
):
    neighbor_indices = locations[agent_index]
    agent_state = int(state_tensor[agent_index])
    if agent_state == 2:
        rand = rand_uniform_philox(tick, agent_index, 1)
        if rand < p_recovery:
            state_tensor[agent_index] = 3
    elif agent_state == 1:
        i = 0
        j = 0
        infected = False
        while i < len(neighbor_indices) and not infected:
            neighbor_index = int(neighbor_indices[i])
            if int(state_tensor[neighbor_index]) == 2:
                rand = rand_uniform_philox(tick, agent_index, 2 + j)
                if rand < p_infection:
                    state_tensor[agent_index] = 2
                    infected = True
                j += 1
            i += 1


@jit.rawkernel(device="cuda")
def opinion_step(
    tick, agent_index, noise_sigma,
    agent_ids, breeds, locations, opinion, weights,
):
    neighbor_indices = locations[agent_index]
    m = len(neighbor_indices)
    if m > 8:
        m = 8
    acc = cp.float32(0.0)
    norm = cp.float32(0.0)
    j = 0
    while j < m:
        w = cp.float32(weights[agent_index][j])
        nb = int(neighbor_indices[j])
        acc = cp.float32(acc + cp.float32(w * cp.float32(opinion[nb])))
        norm = cp.float32(norm + abs(w))
        j += 1
    x = cp.float32(opinion[agent_index])
    if norm > 0:
        x = cp.float32(acc / norm)
    z = rand_normal(tick, agent_index, 1)
    y = float(x) + noise_sigma * z
    if y < 0.0:
        y = 0.0
    if y > 1.0:
        y = 1.0
    opinion[agent_index] = y



@jit.rawkernel(device="cuda")
def host_step(
    tick, agent_index, p_infection, p_recovery,
    agent_ids, breeds, locations, state_tensor,
    health, health_idx, load, load_idx,
):
    row = health_idx[agent_index]
    neighbor_indices = locations[agent_index]
    k = 0
    e_n = cp.float32(0.0)
    site_load = cp.float32(0.0)
    i = 0
    while i < len(neighbor_indices):
        nb = int(neighbor_indices[i])
        r2 = health_idx[nb]
        if r2 >= 0:
            if tick == 0:
                s2 = int(state_tensor[nb]) - 1
            else:
                s2 = int(health[r2][0])
            if s2 == 1:
                k += 1
            e_n = cp.float32(e_n + health[r2][1])
        r3 = load_idx[nb]
        if r3 >= 0:
            site_load = cp.float32(site_load + load[r3][1][0])
        i += 1
    if tick == 0:
        s = int(state_tensor[agent_index]) - 1
    else:
        s = int(health[row][0])
    ex = cp.float32(health[row][1])
    health[row][1] = cp.float32(cp.float32(ex * cp.float32(0.5)) + cp.float32(k))
    health[row, 3] = e_n
    new = s
    if s == 1:
        health[row][2] += cp.float32(1.0)
        if rand_uniform_philox(tick, agent_index, 1) < p_recovery:
            new = 2
    elif s == 0:
        p = p_infection * (float(ex) + 0.1 * float(site_load))
        if rand_uniform_philox(tick, agent_index, 2) < p:
            new = 1
    health[row][0] = cp.float32(new)


@jit.rawkernel(device="cuda")
def site_step(
    tick, agent_index, p_infection, p_recovery,
    agent_ids, breeds, locations, state_tensor,
    health, health_idx, load, load_idx,
):
    row = load_idx[agent_index]
    neighbor_indices = locations[agent_index]
    tot = cp.float32(0.0)
    k = 0
    i = 0
    while i < len(neighbor_indices):
        nb = int(neighbor_indices[i])
        r2 = health_idx[nb]
        if r2 >= 0:
            tot = cp.float32(tot + health[r2][2])
            if int(health[r2][0]) == 1:
                k = k + 1
        i += 1
    slot = tick % 2
    load[row][slot][0] = tot
    load[row][slot][1] = cp.float32(k)
    load[row][1 - slot][1] += cp.float32(0.5)


@jit.rawkernel(device="cuda")
def measures_step(
    tick, agent_index, p_infection, p_recovery,
    agent_ids, breeds, locations, state_tensor, measures, history,
):
    neighbor_indices = locations[agent_index]
    rand = rand_uniform_philox(tick, agent_index, 1)
    agent_state = state_tensor[agent_index]
    own = measures[agent_index]
    if agent_state == 2 and rand < p_recovery:
        state_tensor[agent_index] = 3
    elif agent_state == 1:
        i = 0
        while i < len(neighbor_indices) and neighbor_indices[i] != -1:
            nb = neighbor_indices[i]
            theirs = measures[nb]
            safety = 0.0
            for a in range(len(own)):
                for b in range(len(theirs)):
                    safety += own[a] * theirs[b]
            scaled = safety / (len(own) ** 2)
            if state_tensor[nb] == 2 and rand < p_infection * (1 - scaled):
                state_tensor[agent_index] = 2
            i += 1
    slot = tick % len(history[agent_index])
    history[agent_index][slot] = state_tensor[agent_index]


@jit.rawkernel(device="cuda")
def helpers_step(
    tick, agent_index, p_infection, p_recovery,
    agent_ids, breeds, locations, state_tensor, visits,
):
    agent_state = int(get_this_agent_data_from_tensor(agent_index, state_tensor))
    if agent_state == 2:
        if rand_uniform_philox(tick, agent_index, 1) < p_recovery:
            set_this_agent_data_from_tensor(agent_index, state_tensor, 3)
    elif agent_state == 1:
        i = 0
        j = 0
        infected = False
        while i < get_num_neighbors(agent_index, neighbor_offsets) and not infected:
            nb = get_neighbor(agent_index, i, neighbor_offsets, neighbor_values)
            if int(state_tensor[nb]) == 2:
                if rand_uniform_philox(tick, agent_index, 2 + j) < p_infection:
                    set_this_agent_data_from_tensor(agent_index, state_tensor, 2)
                    infected = True
                j += 1
            i += 1
    visits[agent_index] = visits[agent_index] + 1


@jit.rawkernel(device="cuda")
def fraction_step(
    tick, agent_index, p_infection, p_recovery,
    agent_ids, breeds, locations, state_tensor, immunity, load,
):
    neighbor_ids = locations[agent_index]
    agent_state = int(state_tensor[agent_index])
    infected = 0
    i = 0
    while i < len(neighbor_ids) and neighbor_ids[i] != -1:
        if int(state_tensor[neighbor_ids[i]]) == 2:
            infected += 1
        i += 1
    load[agent_index] = (load[agent_index] + infected) / 2
    if agent_state == 2:
        if rand_uniform_philox(tick, agent_index, 1) < p_recovery:
            state_tensor[agent_index] = 3
    elif agent_state == 1:
        if infected > 0:
            if rand_uniform_philox(tick, agent_index, 1) < p_infection * (1.0 - immunity[agent_index]):
                state_tensor[agent_index] = 2
            if immunity[agent_index] < 1.0:
                immunity[agent_index] = immunity[agent_index] + 0.25
