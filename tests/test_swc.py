"""SWC reader against the reference reader's known answers, plus lowering of an
SWC morphology to the solver batch."""

import json
import os

import numpy as np
import pytest

from braincell_gb300 import Cell
from braincell_gb300.mech import AllRegion, CableProperty, Channel, CVPerBranch, branch_in
from braincell_gb300.runtime import Plan
from braincell_gb300.swc import parse_swc, read_swc

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "swc_known_answers.json")))["cases"]


def _by_name(m):
    return {n.name: n for n in (m.branch(i) for i in range(len(m)))}


def _edge_of(m, name):
    return next(e for e in m.edges if e.child.name == name)


@pytest.mark.parametrize("case", GOLD, ids=[c["ref"].split()[1] for c in GOLD])
def test_reference_known_answers(case):
    m = read_swc(case["swc"], text=True)
    names = _by_name(m)
    if "n_branches" in case:
        assert len(m) == case["n_branches"]
    if "root_name" in case:
        assert m.root.name == case["root_name"]
    if "root_length" in case:
        assert m.root.branch.length == pytest.approx(case["root_length"])
    if "edges" in case:
        assert [e.parent_x for e in m.edges] == case["edges"]
    if "child_x" in case:
        assert [e.child_x for e in m.edges] == case["child_x"]
    for nm, ty in case.get("types", {}).items():
        assert names[nm].branch.type == ty
    if "root_points" in case:
        np.testing.assert_allclose(m.root.branch.points, case["root_points"])
    if "axon_children" in case:
        kids = [e for e in m.edges if e.child.branch.type == "axon"]
        assert len(kids) == len(case["axon_children"])
        for e, exp in zip(kids, case["axon_children"]):
            np.testing.assert_allclose(e.child.branch.points, exp["points"])
            assert e.parent_x == exp["parent_x"]
    for nm, exp in case.get("branches", {}).items():
        e = _edge_of(m, nm)
        if "parent" in exp:
            assert e.parent.name == exp["parent"]
        if "parent_x" in exp:
            assert e.parent_x == exp["parent_x"]
        if "points" in exp:
            np.testing.assert_allclose(names[nm].branch.points, exp["points"])
    if "soma_center" in case:
        pts = m.root.branch.points
        np.testing.assert_allclose(pts[1], case["soma_center"])
        assert {tuple(p) for p in pts[[0, 2]]} == {tuple(map(float, p)) for p in case["soma_ends"]}
        d = names[case["dend"]].branch
        np.testing.assert_allclose(d.points[0], case["dend_first_point"])
        assert d.radii_proximal[0] == pytest.approx(d.radii_distal[0])
        assert d.radii_proximal[0] != pytest.approx(case["dend_radius_not"])
    if "n_soma_branches" in case:
        assert sum(1 for n in names.values() if n.branch.type == "soma") == case["n_soma_branches"]


@pytest.mark.parametrize("body,msg", [
    ("1 1 0 0 0 10 -1\n1 3 0 1 0 1 1", "twice"),
    ("1 1 0 0 0 10 -1\n2 3 0 1 0 1 7", "unknown parent"),
    ("1 1 0 0 0 10 -1\n2 3 0 1 0 1 -1", "exactly one root"),
    ("1 1 0 0 0 0 -1", "radius"),
    ("1 1 0 0 0 10", "7 fields"),
])
def test_malformed_swc_is_rejected(body, msg):
    with pytest.raises(ValueError, match=msg):
        read_swc(body, text=True)


def test_comments_and_blank_lines_are_skipped():
    rows = parse_swc("# header\n\n1 1 0 0 0 10 -1\n  # x\n2 3 0 10 0 2 1\n")
    assert [r.node_id for r in rows] == [1, 2]


_PYRAMID = os.path.join(os.path.dirname(__file__), "golden", "pyramid_small.swc")  # a small synthetic cell


def test_swc_cell_lowers_to_a_plan():
    m = read_swc(_PYRAMID)
    assert len(m) == 8  # soma, 3 basal, 3 apical (trunk + tuft), axon
    cell = Cell(m, cv_policy=CVPerBranch(), pop_size=3)
    cell.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.3, E=-70.0))
    cell.paint(branch_in("type", "soma"), Channel("Na_Ba2002", g_max=120.0), Channel("KDR_Ba2002", g_max=36.0))
    b = cell.batch()
    assert b.n_cells == 3 and b.n_cv == 3 * cell.n_cv
    p = Plan(b, dry_run=True)
    assert p.info["n_cv"] == b.n_cv
