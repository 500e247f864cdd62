"""Schedule planning without a GPU (dry-run plans): tiles, phases, warp slots for
long chains, input validation."""

import numpy as np
import pytest

from braincell_gb300 import _abi
from braincell_gb300 import batch as _batch
from braincell_gb300 import catalogue as _catalogue
from braincell_gb300 import workloads as W
from braincell_gb300.batch import CellBatch
from braincell_gb300.runtime import Plan


def test_small_workload_plan(native_lib):
    b = W.descs_to_batch(W.small(16))
    p = Plan(b, dry_run=True)
    assert p.info["n_cells"] == 16 and p.info["n_cv"] == 16 * 113 and p.info["n_nodes"] == 16 * 129
    st = p.tile_stats()
    assert st[:, 0].sum() == 16 * 129
    assert np.all(st[:, 2] >= 1) and np.all(st[:, 3] > 0)
    assert np.all(st[:, 5] < 227 * 1024)


def test_uneven_sample_plan(native_lib):
    b = W.descs_to_batch(W.uneven(300))
    p = Plan(b, dry_run=True)
    st = p.tile_stats()
    n_nodes = (b.cell_ncv() + b.cell_nbranch() + 1).sum()
    assert st[:, 0].sum() == n_nodes == p.info["n_nodes"]
    assert set(np.unique(st[:, 4])) <= {0, 1, 2}
    # packed tiles respect the node budget
    packed = st[st[:, 4] == 0]
    assert np.all(packed[:, 0] <= p.info["tile_nodes"])


def test_long_chain_is_chunked_over_lanes(native_lib):
    # a 200-CV branch is one chain of ~201 nodes: its warp slot gives each lane a
    # chunk of ceil(201 / 32) = 7 nodes joined by a 5-step scan, so the critical
    # path (cost units: 4 per serial node, 8 per scan step) grows by far less than
    # a serial walk of the chain would add (4 * 201)
    d = W.small(1)[0]
    base = Plan(W.descs_to_batch([d]), dry_run=True).tile_stats()
    d.ncv = [1] + [200] + [8] * (len(d.parent) - 2)
    st = Plan(W.descs_to_batch([d]), dry_run=True).tile_stats()
    assert st[0, 0] == base[0, 0] + 192
    assert st[0, 3] - base[0, 3] <= 4 * 7 + 8 * 5


def test_phases_follow_chain_levels(native_lib):
    # binary tree of depth 3 under a one-CV soma: branch chains at levels 0..2 and
    # the soma chain on top -> 4 phases, whatever the number of cells in the tile
    for n in (1, 8):
        st = Plan(W.descs_to_batch(W.small(n)), dry_run=True).tile_stats()
        assert np.all(st[:, 2] == 4)


def _bad(b: CellBatch, **kw):
    for k, v in kw.items():
        setattr(b, k, v)
    return b


@pytest.mark.parametrize("mutate,msg", [
    (lambda b: _bad(b, branch_region=np.full_like(b.branch_region, 7)), "region"),
    (lambda b: _bad(b, region_mech=np.full_like(b.region_mech, 1 << 30)), "mechanism"),
    (lambda b: _bad(b, pulse_t_off=b.pulse_t_on - 1.0), "pulse_t_off"),
    (lambda b: _bad(b, probe_branch=np.full_like(b.probe_branch, 99)), "probe"),
])
def test_invalid_batches_rejected(native_lib, mutate, msg):
    b = mutate(W.descs_to_batch(W.small(2)))
    with pytest.raises(_abi.BCError, match=msg) as e:
        Plan(b, dry_run=True)
    assert e.value.status == _abi.BC_ERR_INVALID


def test_parent_order_and_radii_validation(native_lib):
    b = W.descs_to_batch(W.small(1))
    b.branch_parent = b.branch_parent.copy()
    b.branch_parent[1] = 5  # a parent that comes after its child
    with pytest.raises(_abi.BCError, match="precede"):
        Plan(b, dry_run=True)
    b = W.descs_to_batch(W.small(1))
    b.seg_r_prox = b.seg_r_prox.copy()
    b.seg_r_prox[3] = 0.0
    with pytest.raises(_abi.BCError, match="radii"):
        Plan(b, dry_run=True)


def test_dry_plan_has_no_device_state(native_lib):
    p = Plan(W.descs_to_batch(W.small(1)), dry_run=True)
    with pytest.raises(_abi.BCError, match="dry_run"):
        p.run(1, 0.025)


def _probe_plan(decls, field):
    from braincell_gb300 import Branch, Cell, Morphology
    from braincell_gb300.batch import lower_cell
    from braincell_gb300.mech import AllRegion, CableProperty, CVPerBranch, RootLocation, StateProbe
    from braincell_gb300.runtime import Plan

    m = Morphology.from_root(Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma"), name="soma")
    c = Cell(m, cv_policy=CVPerBranch())
    c.paint(AllRegion(), CableProperty(), *decls)
    c.place(RootLocation(0.5), StateProbe())
    b = lower_cell(c)
    b.probe_field[:] = field
    return Plan(b, dry_run=True)


def _decl(cls):
    from braincell_gb300.mech import Channel, Ion

    return Ion(cls) if cls == "CalciumDetailed" else Channel(cls)


# one case per view / current code, named by its kernel class (same-form classes share them)
_VIEW_CASES = sorted({(v, c) for (c, _f), v in _batch.PROBE_STATES.items() if c not in _catalogue.SAME_FORM})
_CUR_CASES = sorted({(v, c) for c, v in _batch.PROBE_CURRENTS.items() if c not in _catalogue.SAME_FORM})


@pytest.mark.parametrize("view,cls", _VIEW_CASES)
def test_planner_state_view_owner_table(view, cls):
    # the planner accepts a mechanism probe only where the mechanism owning the view is
    # painted (bc_plan.cpp owner table), whatever else is painted there
    from braincell_gb300 import _abi
    from braincell_gb300.mech import Channel

    _probe_plan([Channel("IL"), _decl(cls)], view).close()
    other = "KNI_Ya1989" if cls != "KNI_Ya1989" else "KM_RI2021_SC"
    with pytest.raises(_abi.BCError, match="no such mechanism"):
        _probe_plan([Channel("IL"), Channel(other)], view)


@pytest.mark.parametrize("code,cls", _CUR_CASES)
def test_planner_current_owner_table(code, cls):
    from braincell_gb300 import _abi
    from braincell_gb300.mech import Channel

    field = _abi.BC_PROBE_CURRENT + code
    _probe_plan([_decl(cls)], field).close()
    other = "HCN_HM1992" if cls != "HCN_HM1992" else "K_Leak"
    with pytest.raises(_abi.BCError, match="no such mechanism"):
        _probe_plan([Channel(other)], field)


@pytest.mark.parametrize("ion,members", [("na", ("Na_Ba2002", "Na_HH1952")),
                                         ("k", ("KDR_Ba2002", "K_Leak", "AHP_De1994", "K_HH1952", "KM_RI2021_SC",
                                                "KA1_HM1992", "KA2_HM1992", "KK2A_HM1992", "KK2B_HM1992",
                                                "KNI_Ya1989")),
                                         ("ca", ("CaL_IS2008", "CaT_HM1992"))])
def test_planner_ion_current_owner_table(ion, members):
    from braincell_gb300 import _abi
    from braincell_gb300.batch import ION_CURRENTS
    from braincell_gb300.mech import Channel

    field = _abi.BC_PROBE_CURRENT + ION_CURRENTS[ion]
    for cls in members:
        _probe_plan([Channel(cls)], field).close()
    with pytest.raises(_abi.BCError, match="no such mechanism"):
        _probe_plan([Channel("HCN_HM1992")], field)


@pytest.mark.parametrize("cls,variant", [("IL", _abi.BC_VARIANT_LEAN), ("Na_Ba2002", _abi.BC_VARIANT_LEAN),
                                         ("CaT_HM1992", _abi.BC_VARIANT_LEAN), ("Na_HH1952", _abi.BC_VARIANT_EXTRA),
                                         ("K_HH1952", _abi.BC_VARIANT_EXTRA), ("KM_RI2021_SC", _abi.BC_VARIANT_EXTRA),
                                         ("KA1_HM1992", _abi.BC_VARIANT_EXTRA), ("KA2_HM1992", _abi.BC_VARIANT_EXTRA),
                                         ("KK2A_HM1992", _abi.BC_VARIANT_EXTRA), ("KK2B_HM1992", _abi.BC_VARIANT_EXTRA),
                                         ("KNI_Ya1989", _abi.BC_VARIANT_EXTRA), ("K_TM1991", _abi.BC_VARIANT_LEAN)])
def test_kernel_variant_follows_the_painted_channels(cls, variant):
    # the lean kernel carries only the main mix: a plan with any channel outside it
    # must launch the extra variant, which is the one that evaluates those channels
    from braincell_gb300.mech import Channel

    p = _probe_plan([Channel(cls)], _abi.BC_STATE_V)
    assert p.info["kernel_variant"] == variant
    p.close()


def test_mechanism_probe_selects_the_extra_variant():
    from braincell_gb300.mech import Channel

    p = _probe_plan([Channel("Na_Ba2002")], _abi.BC_STATE_NA_P)
    assert p.info["kernel_variant"] == _abi.BC_VARIANT_EXTRA
    p.close()


def test_threaded_planner_matches_sequential(monkeypatch):
    # cells lower and decompose on host threads (BC_PLAN_THREADS); the plan must not
    # depend on how many
    b = W.descs_to_batch(W.uneven(700))
    kw = dict(precision="f32", tile_nodes=2500, threads_per_tile=512, threads_big=512, dry_run=True)
    out = []
    for n in ("1", "3", "8"):
        monkeypatch.setenv("BC_PLAN_THREADS", n)
        p = Plan(b, **kw)
        out.append((p.info, p.tile_stats()))
        p.close()
    for info, stats in out[1:]:
        assert info == out[0][0]
        np.testing.assert_array_equal(stats, out[0][1])


def test_threaded_planner_reports_the_first_failing_cell(monkeypatch):
    b = W.descs_to_batch(W.uneven(700))
    for c in (300, 650):  # a child listed before its parent in two cells
        k = int(b.cell_branch_offsets[c])
        assert int(b.cell_branch_offsets[c + 1]) - k >= 3
        b.branch_parent[k + 1] = 2
    msgs = []
    for n in ("1", "8"):
        monkeypatch.setenv("BC_PLAN_THREADS", n)
        with pytest.raises(_abi.BCError, match="cell 300") as e:
            Plan(b, dry_run=True)
        msgs.append(str(e.value))
    assert msgs[0] == msgs[1]


def test_ports_pick_the_lean_port_variant_unless_another_feature_needs_the_extra_one():
    # a plan whose only optional feature is its GRU ports runs the lean kernel with
    # ports; a mechanism probe beside the ports needs the extra variant's probe pass
    from dataclasses import replace

    from braincell_gb300 import surrogate as S
    from braincell_gb300 import workloads as W
    from braincell_gb300.runtime import Plan

    d = next(x for x in W.uneven(40, seed=1) if S.reduce_desc(x)[1])
    red, ports = S.reduce_desc(d)
    b = S.ports_to_batch([replace(red, probes=[(0, 0.5)])], [ports])
    p = Plan(b, precision="f32", dry_run=True, threads_per_tile=384, threads_big=384, threads_global=384)
    assert p.info["kernel_variant"] == _abi.BC_VARIANT_PORTS_LEAN
    p.close()
    b.probe_field = np.asarray([_abi.BC_STATE_NA_P], np.int32)
    p = Plan(b, precision="f32", dry_run=True, threads_per_tile=384, threads_big=384, threads_global=384)
    assert p.info["kernel_variant"] == _abi.BC_VARIANT_PORTS
    p.close()
