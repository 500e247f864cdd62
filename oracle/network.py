"""Float64 CPU restatement of network event delivery between cells.

TEST INFRASTRUCTURE ONLY: the checker for the GPU network path, never imported by
the product.  Follows the reference's network run step
(``network/engine.py:474-530``):

1. ``write_arrivals`` -- events due this step are handed to their target synapses
   (``network/delivery.py:317-358``), which add them to ``g`` at the start of the
   step (``Cell._begin_step``, ``cell.py:2331-2346``);
2. every cell advances one staggered step;
3. ``enqueue_future_events`` -- the population spike of every presynaptic cell
   (any CV crossing, ``delivery.py:103-123``) is projected through its contacts
   into the ring slot ``delay_steps`` ahead (``delivery.py:361-394``).

With one ring of depth ``delay_steps + 1`` per delay group that slot is read
``max(delay_steps, 1)`` steps later, so a spike at step s arrives at step
``s + max(delay_steps, 1)`` (a zero delay means next-step delivery).  Delays are
quantised to steps with the reference's default ``"ceil"`` rule
(``network/lowering.py:185-226``).
"""

from __future__ import annotations

import math
from collections import defaultdict

import numpy as np

__all__ = ["delay_steps", "OracleNetwork"]


def delay_steps(delay_ms, dt: float) -> np.ndarray:
    """Delays in whole steps: ``ceil(delay / dt)``, exact multiples kept exact."""
    raw = np.asarray(delay_ms, dtype=np.float64) / float(dt)
    near = np.rint(raw)
    raw = np.where(np.isclose(raw, near, rtol=1e-7, atol=1e-7), near, raw)
    steps = np.ceil(raw - 1e-12).astype(np.int64)
    if np.any(steps < 0):
        raise ValueError("delays must be >= 0")
    return steps


class OracleNetwork:
    """Cells (``OracleCell`` objects, replica 0 of each) joined by ExpSyn contacts.

    ``contacts``: ``(pre_cell, post_cell, post_synapse, weight_uS, delay_ms)`` with
    cell indices into ``cells`` and the synapse index in the post cell's placed
    ExpSyn order.
    """

    def __init__(self, cells, contacts):
        self.cells = list(cells)
        self.contacts = [(int(a), int(b), int(k), float(w), float(d)) for a, b, k, w, d in contacts]
        self.t_step = 0
        self.pending: dict[int, dict[tuple[int, int], float]] = defaultdict(lambda: defaultdict(float))

    def run(self, dt: float, n_steps: int):
        """Return (spikes: list of (cell, step), traces [n_cells, n_steps] of probe 0 or CV 0)."""
        d_steps = delay_steps([c[4] for c in self.contacts], dt) if self.contacts else np.zeros(0, np.int64)
        out_by_pre = defaultdict(list)
        for (pre, post, k, w, _), ds in zip(self.contacts, d_steps):
            out_by_pre[pre].append((post, k, w, max(int(ds), 1)))
        pending = self.pending
        spikes = []
        traces = np.zeros((len(self.cells), n_steps))
        for s in range(n_steps):
            step = self.t_step
            due = pending.pop(step, {})
            for ci, oc in enumerate(self.cells):
                n_syn = len(oc.syn_points)
                if n_syn:
                    w = np.zeros((oc.P, n_syn))
                    for (post, k), val in due.items():
                        if post == ci:
                            w[:, k] += val
                    oc.add_events(w)
            for ci, oc in enumerate(self.cells):
                oc.step(dt, step * dt)
                traces[ci, s] = oc.V[0, self._probe_cv(oc)]
            for ci, oc in enumerate(self.cells):
                if oc.population_spike()[0]:
                    spikes.append((ci, step))
                    for post, k, w, ds in out_by_pre[ci]:
                        pending[step + ds][(post, k)] += w
            self.t_step += 1
        return spikes, traces

    @staticmethod
    def _probe_cv(oc) -> int:
        if oc.probe_points:
            hit = np.nonzero(oc.cv_mid == oc.probe_points[0])[0]
            if hit.size:
                return int(hit[0])
        return 0
