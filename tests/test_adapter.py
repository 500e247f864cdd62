"""The braincell-side lowering (``_spec_from_cell`` of the plugin) against stand-ins
that carry the reference ``Cell``'s post-discretisation attributes: the batch it
builds equals the one this package builds from the same declarations."""

from dataclasses import dataclass, field

import numpy as np
import pytest

from braincell_gb300 import workloads as W
from braincell_gb300.adapter import batch_from_reference_cell
from braincell_gb300.batch import _branch_regions, lower_cell
from oracle.staggered import OracleCell


@dataclass
class _MorphoBranch:  # morph/morphology.py MorphoBranch: geometry + attachment
    node_id: int
    parent_id: int | None
    parent_x: float
    child_x: float
    branch: object


@dataclass
class _Morpho:
    branches: tuple


@dataclass
class _Role:  # _discretization/base.py CVPointMechanism
    position: str
    mechanism: object


@dataclass
class _CV:  # _discretization/base.py CV (the fields the lowering reads)
    id: int
    branch_id: int
    prox: float
    dist: float
    cm: float
    ra: float
    v: float
    density_mech: tuple
    point_mech_roles: tuple = field(default_factory=tuple)


@dataclass
class _RefCell:
    morpho: _Morpho
    cvs: tuple
    pop_size: tuple


def _stand_in(cell):
    """A reference-shaped view of a declared cell: branches with node ids (given in a
    shuffled order map), CVs with their painted declarations and point roles."""
    m = cell.morpho
    parent = m.parent_index
    px = {e.child.index: (e.parent_x, e.child_x) for e in m.edges}
    ids = [100 + 7 * k for k in range(len(m))]
    nodes = tuple(_MorphoBranch(ids[k], None if parent[k] < 0 else ids[parent[k]], *px.get(k, (0.0, 0.0)),
                                branch=m.branches[k]) for k in range(len(m)))
    oc = OracleCell(cell)
    branch_region, regions = _branch_regions(cell)
    roles = {}
    for locset, decls in cell.place_rules:
        for (b, x) in locset.points(m):
            ids_b = oc.branch_cv_ids[b]
            if x <= 0.0:
                cv, pos = ids_b[0], "prox"
            elif x >= 1.0:
                cv, pos = ids_b[-1], "dist"
            else:
                cv, pos = oc._locate_cv(b, x), "mid"
            for d in decls:
                roles.setdefault(cv, []).append(_Role(pos, d))
    cvs = []
    for k in range(oc.n_cv):
        b = oc.cv_branch[k]
        cable, mechs = regions[int(branch_region[b])]
        cvs.append(_CV(k, b, oc.cv_prox[k], oc.cv_dist[k], cable.membrane_capacitance, cable.axial_resistivity,
                       cable.resting_potential, tuple(mechs), tuple(roles.get(k, ()))))
    return _RefCell(_Morpho(nodes), tuple(reversed(cvs)), cell.pop_size)


def _cells():
    d = W._small_desc(2)
    d.pulses = [(0, 0.5, 1.0, 9.0, 0.3), (3, 1.0, 2.0, 4.0, 0.1)]
    yield W.desc_to_cell(d, pop_size=3)
    u = W.uneven(indices=[5])[0]
    yield W.desc_to_cell(u)
    yield W.desc_to_cell(W.large(indices=[0], n_range=(300, 400), n_branches=20, n_pulses=5, duration=10.0)[0])


@pytest.mark.parametrize("cell", list(_cells()), ids=["small_x3", "uneven", "calcium"])
def test_reference_cell_lowers_like_the_declaration(cell):
    got = batch_from_reference_cell(_stand_in(cell))
    want = lower_cell(cell)
    for name in ("cell_branch_offsets", "branch_parent", "branch_parent_x", "branch_child_x", "branch_ncv",
                 "branch_seg_offsets", "seg_length", "seg_r_prox", "seg_r_dist"):
        np.testing.assert_array_equal(getattr(got, name), getattr(want, name), err_msg=name)
    # the same record on every branch (region numbering may differ)
    np.testing.assert_allclose(got.region_params[got.branch_region], want.region_params[want.branch_region], rtol=1e-12)
    np.testing.assert_array_equal(got.region_mech[got.branch_region], want.region_mech[want.branch_region])
    key = lambda b: sorted(zip(b.pulse_cell, b.pulse_branch, b.pulse_x, b.pulse_t_on, b.pulse_t_off, b.pulse_amp))
    assert key(got) == key(want)
    np.testing.assert_array_equal(np.sort(got.probe_branch), np.sort(want.probe_branch))


def test_branches_painted_below_branch_grain_are_rejected():
    cell = W.desc_to_cell(W._small_desc(0))
    ref = _stand_in(cell)
    cv0 = [c for c in ref.cvs if c.branch_id == 1][0]
    cv0.cm = 2.0
    with pytest.raises(NotImplementedError):
        batch_from_reference_cell(ref)


def test_unsupported_point_mechanisms_are_rejected():
    cell = W.desc_to_cell(W._small_desc(0))
    ref = _stand_in(cell)

    class ExpTwoSyn:  # a point mechanism the batch spec does not carry
        pass

    ref.cvs[0].point_mech_roles = (_Role("mid", ExpTwoSyn()),)
    with pytest.raises(NotImplementedError):
        batch_from_reference_cell(ref)
