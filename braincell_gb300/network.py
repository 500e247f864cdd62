"""Networks of cells joined by event-driven ExpSyn synapses.

Mirrors the reference's network surface (``network/core.py``): named
:class:`Population` objects wrap a :class:`~braincell_gb300.cell.Cell` whose
``pop_size`` replicas are the population members, and :class:`Connection` rows
join presynaptic members to a placed synapse of postsynaptic members with a
weight and a delay.  :meth:`Network.run` lowers everything into one batch and
runs it on the GPU: spikes (any CV of a source cell crossing 0 mV upward within a
step) are recorded by the step kernel and delivered by a delivery kernel between
launches into a ring of per-step synapse arrivals; a launch never spans more
steps than the shortest delay, so no event is due inside the launch that
produced it.  The event timing and the synapse dynamics follow
``network/engine.py:474-530``, ``network/delivery.py`` and ``synapse/markov.py:65``.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .batch import concat_batches, lower_cell
from .mech import ExpSyn

__all__ = ["Population", "Connection", "Network", "NetworkRunResult"]


@dataclass
class Population:
    """A named group of ``cell.pop_size`` identical cells."""

    name: str
    cell: object

    def __post_init__(self) -> None:
        if not isinstance(self.name, str) or not self.name:
            raise ValueError("Population name must be a non-empty string.")
        if len(tuple(self.cell.pop_size)) != 1 or int(self.cell.pop_size[0]) <= 0:
            raise ValueError(f"a population needs a one-dimensional pop_size > 0, got {self.cell.pop_size!r}.")

    @property
    def size(self) -> int:
        return int(self.cell.pop_size[0])


@dataclass
class Connection:
    """Contacts ``pre_population[pre_index] -> post_population[post_index].synapse``.

    ``synapse`` names a placed :class:`~braincell_gb300.mech.ExpSyn` (its ``name``)
    or gives its index in placement order.  ``weight`` (uS) defaults to the
    synapse's own ``weight``; ``delay`` is in ms (>= 0, a zero delay means
    next-step delivery).
    """

    pre_population: str
    post_population: str
    pre_index: object
    post_index: object
    synapse: object = 0
    weight: object | None = None
    delay: object = 0.0

    def __post_init__(self) -> None:
        self.pre_index = np.atleast_1d(np.asarray(self.pre_index, dtype=np.int64))
        self.post_index = np.atleast_1d(np.asarray(self.post_index, dtype=np.int64))
        if self.pre_index.shape != self.post_index.shape or self.pre_index.ndim != 1:
            raise ValueError("pre_index and post_index must be 1-D arrays of equal length.")

    @property
    def n_contact(self) -> int:
        return int(self.pre_index.size)


@dataclass
class NetworkRunResult:
    """Spikes per population as (member index, time in ms), time-ordered."""

    spikes: dict = field(default_factory=dict)
    steps: int = 0
    dt: float = 0.0


def _synapses_of(cell) -> list[ExpSyn]:
    out = []
    for locset, decls in cell.place_rules:
        for _ in locset.points(cell.morpho):
            out.extend(d for d in decls if isinstance(d, ExpSyn))
    return out


class Network:
    def __init__(self, populations, connections=()):
        pops = list(populations.values()) if isinstance(populations, dict) else list(populations)
        self.populations = {p.name: p for p in pops}
        if len(self.populations) != len(pops):
            raise ValueError("population names must be unique.")
        self.connections = list(connections)
        self._plan = None
        self._t_step = 0

    # ------------------------------------------------------------------ lowering
    def batch(self):
        """The whole network as one batch: populations in order, members as cells."""
        parts, cell_off, syn_off, syn_per_cell, syn_decl = [], {}, {}, {}, {}
        nc = ns = 0
        for name, pop in self.populations.items():
            b = lower_cell(pop.cell, replicas=pop.size)
            decls = _synapses_of(pop.cell)
            cell_off[name], syn_off[name] = nc, ns
            syn_per_cell[name], syn_decl[name] = len(decls), decls
            nc += pop.size
            ns += len(decls) * pop.size
            parts.append(b)
        batch = concat_batches(parts)
        pre, post, w, d = [], [], [], []
        for con in self.connections:
            for nm in (con.pre_population, con.post_population):
                if nm not in self.populations:
                    raise KeyError(f"unknown population {nm!r}")
            pp, qp = self.populations[con.pre_population], self.populations[con.post_population]
            if np.any(con.pre_index < 0) or np.any(con.pre_index >= pp.size):
                raise ValueError(f"pre_index out of range for population {pp.name!r}.")
            if np.any(con.post_index < 0) or np.any(con.post_index >= qp.size):
                raise ValueError(f"post_index out of range for population {qp.name!r}.")
            decls = syn_decl[qp.name]
            if isinstance(con.synapse, str):
                hits = [k for k, s in enumerate(decls) if s.name == con.synapse]
                if len(hits) != 1:
                    raise ValueError(f"population {qp.name!r} has {len(hits)} synapses named {con.synapse!r}.")
                k = hits[0]
            else:
                k = int(con.synapse)
                if not 0 <= k < len(decls):
                    raise ValueError(f"population {qp.name!r} has no synapse {k}.")
            n = con.n_contact
            weight = np.broadcast_to(np.asarray(decls[k].weight if con.weight is None else con.weight, float), (n,))
            delay = np.broadcast_to(np.asarray(con.delay, float), (n,))
            if np.any(delay < 0):
                raise ValueError("delays must be >= 0 ms.")
            pre.append(cell_off[pp.name] + con.pre_index)
            post.append(syn_off[qp.name] + con.post_index * syn_per_cell[qp.name] + k)
            w.append(weight)
            d.append(delay)
        if pre:
            batch.conn_pre = np.concatenate(pre).astype(np.int32)
            batch.conn_post = np.concatenate(post).astype(np.int64)
            batch.conn_weight = np.concatenate(w).astype(np.float64)
            batch.conn_delay = np.concatenate(d).astype(np.float64)
        self._cell_off = cell_off
        return batch

    # ------------------------------------------------------------------ running
    def init_state(self, **plan_options):
        from .runtime import Plan

        cells = [p.cell for p in self.populations.values()]
        precisions = {getattr(c, "solver_options", {}).get("precision", "f32") for c in cells}
        if len(precisions) > 1:
            raise ValueError(f"all populations of a network must share one precision, got {sorted(precisions)}.")
        plan_options.setdefault("precision", precisions.pop() if precisions else "f32")
        plan_options.setdefault("record_every", 0)
        self._plan = Plan(self.batch(), **plan_options)
        self._t_step = 0
        return self._plan

    def run(self, *, dt: float, duration: float, **plan_options) -> NetworkRunResult:
        """Run ``duration`` ms from the current state (initialising on first use)."""
        if self._plan is None:
            self.init_state(**plan_options)
        n = int(round(duration / dt))
        self._plan.run(n, dt)
        self._t_step += n
        return self.spikes(dt)

    def spikes(self, dt: float) -> NetworkRunResult:
        cells, steps = self.spike_records()
        out = {}
        order = np.lexsort((cells, steps))
        cells, steps = cells[order], steps[order]
        for name, pop in self.populations.items():
            c0 = self._cell_off[name]
            m = (cells >= c0) & (cells < c0 + pop.size)
            out[name] = (cells[m] - c0, steps[m] * dt)
        return NetworkRunResult(spikes=out, steps=self._t_step, dt=dt)

    def spike_records(self):
        """All (cell, step) spike records since the last reset."""
        plan = self._plan
        n = C.c_int64()
        _abi.check(plan._lib.bc_network_spikes(plan._h, None, None, 0, C.byref(n), plan._stream(None)))
        m = int(n.value)
        cells = np.zeros(m, np.int32)
        steps = np.zeros(m, np.int64)
        if m:
            _abi.check(plan._lib.bc_network_spikes(plan._h, cells.ctypes.data_as(C.POINTER(C.c_int32)),
                                                   steps.ctypes.data_as(C.POINTER(C.c_int64)), m, C.byref(n),
                                                   plan._stream(None)))
        return cells, steps

    def synapse_g(self) -> np.ndarray:
        plan = self._plan
        out = np.zeros(int(plan.batch.syn_cell.size))
        _abi.check(plan._lib.bc_synapse_download(plan._h, out.ctypes.data_as(C.POINTER(C.c_double)),
                                                 plan._stream(None)))
        return out
