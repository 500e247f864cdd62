"""Autotuner search logic (with an injected measurement) and batch subsetting."""

import numpy as np
import pytest

from braincell_gb300 import tune
from braincell_gb300 import workloads as W
from braincell_gb300.batch import CellBatch


def _arrays_equal(a: CellBatch, b: CellBatch):
    assert a.n_regions == b.n_regions
    for k in CellBatch._DTYPES:
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k), err_msg=k)


def test_select_matches_building_the_subset():
    descs = W.uneven(12) + W.small(3)
    full = W.descs_to_batch(descs)
    idx = [13, 2, 7, 0]
    _arrays_equal(full.select(idx), W.descs_to_batch([descs[i] for i in idx]))
    _arrays_equal(full.select(np.arange(full.n_cells)), full)


def test_select_rejects_bad_indices():
    b = W.descs_to_batch(W.small(2))
    with pytest.raises(ValueError):
        b.select([2])


def test_sample_is_seeded_and_bounded():
    b = W.descs_to_batch(W.uneven(40))
    s1, s2 = tune.sample_cells(b, 10, seed=3), tune.sample_cells(b, 10, seed=3)
    assert s1.n_cells == 10
    _arrays_equal(s1, s2)
    assert tune.sample_cells(b, 100) is b


def test_coordinate_search_finds_the_best_options():
    best = {"tile_nodes": 2000, "threads_per_tile": 256, "lane_nodes": 4, "steps_per_launch": 250}

    def fake(sample, o):
        assert sample.n_cells == 20
        return 1e9 * (1 + sum(o[k] == v for k, v in best.items()))

    r = tune.autotune(W.descs_to_batch(W.uneven(30)), max_cells=20, measure=fake)
    for k, v in best.items():
        assert r.options[k] == v
    assert r.rate == 5e9
    # each distinct option set is measured once
    keys = [tuple(sorted(o.items())) for o, _ in r.trials]
    assert len(keys) == len(set(keys))


def test_time_budget_stops_the_search():
    r = tune.autotune(W.descs_to_batch(W.small(4)), measure=lambda s, o: 1.0, time_budget_s=0.0)
    assert len(r.trials) == 1 and r.options["tile_nodes"] == tune.TILE_THREADS[0][0]
