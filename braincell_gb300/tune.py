"""Autotuner for the tile plan of a batch.

The step kernel's speed depends on four plan options:
- ``tile_nodes``: how many cells share a CTA, hence CTAs per SM;
- ``threads_per_tile``: warps that take warp slots in parallel;
- ``lane_nodes``: the switch between shuffle-scanned chains and chains walked
  serially by one lane;
- ``steps_per_launch``: how many steps one launch fuses.

Their best values depend on the morphologies of the batch.  :func:`autotune` times
short runs of candidate plans on a seeded sample of the batch's cells, searching
coordinate-wise: first tile size x threads jointly (they set occupancy together),
then ``lane_nodes``, then ``steps_per_launch``.  It returns the keyword arguments
for :class:`~braincell_gb300.runtime.Plan`.

The measurement is injectable (``measure=``), so the search itself is testable
without a GPU.
"""

from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import Callable, Sequence

import numpy as np

from .batch import CellBatch

__all__ = ["TuneResult", "autotune", "sample_cells", "measure_plan"]

TILE_THREADS = ((2500, 512), (2000, 512), (2500, 384), (2000, 256), (1500, 256), (4800, 1024))
PORT_MAX_THREADS = 384
LANE_NODES = (10, 4, 1)
STEPS_PER_LAUNCH = (1000, 250)


@dataclass
class TuneResult:
    options: dict
    rate: float                       # compartment-steps/s of the chosen options on the sample
    trials: list = field(default_factory=list)  # (options, rate) in the order measured

    def __repr__(self) -> str:  # pragma: no cover - cosmetic
        return f"TuneResult(options={self.options}, rate={self.rate:.3e}, trials={len(self.trials)})"


def sample_cells(batch: CellBatch, max_cells: int, seed: int = 0) -> CellBatch:
    """A seeded random subset of at most ``max_cells`` cells of ``batch``."""
    if batch.n_cells <= max_cells:
        return batch
    rng = np.random.default_rng(seed)
    keep = np.sort(rng.choice(batch.n_cells, size=max_cells, replace=False))
    return batch.select(keep)


def measure_plan(batch: CellBatch, options: dict, *, steps: int = 200, dt: float = 0.025, device: int = 0,
                 precision: str = "f32") -> float:
    """Compartment-steps/s of ``batch`` under ``options`` (device time of ``steps`` steps)."""
    from .runtime import Plan

    plan = Plan(batch, precision=precision, device=device, record_every=0, **options)
    try:
        plan.run(min(steps, 20), dt)  # warm-up: staging, clocks
        ms = plan.run_timed(steps, dt)
        return plan.n_cv * steps / (ms * 1e-3)
    finally:
        plan.close()


def autotune(batch: CellBatch, *, steps: int = 200, dt: float = 0.025, device: int = 0, precision: str = "f32",
             max_cells: int = 1500, seed: int = 0,
             tile_threads: Sequence[tuple[int, int]] = TILE_THREADS,
             lane_nodes: Sequence[int] = LANE_NODES,
             steps_per_launch: Sequence[int] = STEPS_PER_LAUNCH,
             measure: Callable[[CellBatch, dict], float] | None = None,
             time_budget_s: float | None = None) -> TuneResult:
    """Choose plan options for ``batch``; see the module docstring.

    ``measure(sample, options) -> rate`` replaces the GPU timing when given.
    ``time_budget_s`` stops the search early (the best options so far are kept).
    """
    sample = sample_cells(batch, max_cells, seed)
    if sample.port_cell.size:  # the kernel variant with GRU ports runs at most 384 threads per tile
        tile_threads = [(tn, min(th, PORT_MAX_THREADS)) for tn, th in tile_threads]
    if measure is None:
        def measure(b, o):
            return measure_plan(b, o, steps=steps, dt=dt, device=device, precision=precision)
    t0 = time.perf_counter()
    trials: list = []
    cache: dict = {}

    def rate_of(opts: dict) -> float:
        key = tuple(sorted(opts.items()))
        if key not in cache:
            cache[key] = float(measure(sample, dict(opts)))
            trials.append((dict(opts), cache[key]))
        return cache[key]

    def out_of_time() -> bool:
        return time_budget_s is not None and time.perf_counter() - t0 > time_budget_s

    best = {"tile_nodes": tile_threads[0][0], "threads_per_tile": tile_threads[0][1],
            "threads_big": tile_threads[0][1] if sample.port_cell.size else 512,
            "lane_nodes": lane_nodes[0], "steps_per_launch": steps_per_launch[0]}
    best_rate = rate_of(best)
    for tn, th in tile_threads:
        if out_of_time():
            break
        cand = dict(best, tile_nodes=tn, threads_per_tile=th,
                    threads_big=th if sample.port_cell.size else max(th, 512))
        r = rate_of(cand)
        if r > best_rate:
            best, best_rate = cand, r
    for ln in lane_nodes:
        if out_of_time():
            break
        cand = dict(best, lane_nodes=ln)
        r = rate_of(cand)
        if r > best_rate:
            best, best_rate = cand, r
    for spl in steps_per_launch:
        if out_of_time():
            break
        cand = dict(best, steps_per_launch=spl)
        r = rate_of(cand)
        if r > best_rate:
            best, best_rate = cand, r
    return TuneResult(options=best, rate=best_rate, trials=trials)
