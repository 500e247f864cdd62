"""Native lowering (geometry -> point tree -> axial coefficients) against the oracle's
restatement of the reference assembly, and the flat batch paths against each other."""

import numpy as np
import pytest

from braincell_gb300 import Branch, Cell, Morphology
from braincell_gb300 import workloads as W
from braincell_gb300.batch import concat_batches, lower_cell, native_lowering
from braincell_gb300.mech import AllRegion, CableProperty, Channel, CVPerBranchList, MaxCVLen, branch_in
from oracle.staggered import OracleCell


def _compare(cell, native_lib):
    oc = OracleCell(cell)
    nl = native_lowering(lower_cell(cell, replicas=1), 0)
    assert nl["cv_area"].shape[0] == oc.n_cv and nl["parent"].shape[0] == oc.n_point
    np.testing.assert_allclose(nl["cv_area"], oc.cv_area, rtol=1e-13)
    np.testing.assert_array_equal(nl["cv_node"], oc.cv_mid)
    np.testing.assert_array_equal(nl["parent"], oc.node_parent)
    rows = oc.point_to_row
    np.testing.assert_allclose(nl["diag"], oc.diag_ms[rows], rtol=1e-12)
    # lowers[row] = A[row, parent] = -alpha, uppers[row] = A[parent, row] = -beta
    np.testing.assert_allclose(-nl["alpha"], oc.lowers_ms[rows], rtol=1e-12, atol=0)
    np.testing.assert_allclose(-nl["beta"], oc.uppers_ms[rows], rtol=1e-12, atol=0)
    assert np.all((nl["region"] >= 0) == oc.is_mid)


def test_small_cell_lowering(native_lib):
    _compare(W.desc_to_cell(W.small(1)[0]), native_lib)


@pytest.mark.parametrize("i", [0, 3, 7, 15])
def test_uneven_cell_lowering(native_lib, i):
    _compare(W.desc_to_cell(W.uneven(indices=[i])[0]), native_lib)


def test_multisegment_jump_and_midpoint_attachment(native_lib):
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    m = Morphology.from_root(soma, name="soma")
    d1 = Branch.from_lengths(lengths=[30.0, 0.0, 40.0], radii_proximal=[2.0, 1.0, 1.5], radii_distal=[1.0, 1.5, 0.5],
                             type="dendrite")
    m.attach(parent="soma", child_branch=d1, child_name="d1", parent_x=1.0)
    d2 = Branch.from_lengths(lengths=[25.0, 25.0], radii_proximal=[1.0, 0.6], radii_distal=[0.8, 0.4], type="dendrite")
    m.attach(parent="d1", child_branch=d2, child_name="d2", parent_x=0.5)  # attaches at a CV midpoint
    d3 = Branch.from_lengths(lengths=[15.0], radii=[0.7, 0.5], type="dendrite")
    m.attach(parent="soma", child_branch=d3, child_name="d3", parent_x=0.0)  # at the root endpoint
    cell = Cell(m, cv_policy=CVPerBranchList((1, 5, 4, 3)))
    cell.paint(AllRegion(), CableProperty(axial_resistivity=150.0, membrane_capacitance=0.9))
    cell.paint(branch_in("type", "dendrite"), Channel("IL", g_max=0.2))
    _compare(cell, native_lib)


def test_max_cv_len_policy_counts():
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    m = Morphology.from_root(soma)
    m.attach(parent=0, child_branch=Branch.from_lengths(lengths=[100.0], radii=[1, 1], type="dendrite"))
    assert MaxCVLen(30.0).cv_counts(m).tolist() == [1, 5]  # ceil(100/30)=4 -> promoted to odd
    assert MaxCVLen(30.0, keep_odd=False).cv_counts(m).tolist() == [1, 4]


def test_descs_batch_equals_declared_cells():
    descs = W.uneven(indices=[1, 2, 5])
    fast = W.descs_to_batch(descs)
    slow = concat_batches([lower_cell(W.desc_to_cell(d)) for d in descs])
    for name in ("cell_branch_offsets", "branch_parent", "branch_ncv", "branch_region", "seg_length",
                 "seg_r_prox", "seg_r_dist", "region_mech", "pulse_branch", "pulse_x", "pulse_amp", "probe_x"):
        np.testing.assert_array_equal(getattr(fast, name), getattr(slow, name), err_msg=name)
    np.testing.assert_allclose(fast.region_params, slow.region_params, rtol=1e-15)


def test_large_descriptions_are_consistent():
    d = W.large(indices=[0], n_range=(300, 400), n_branches=20, n_pulses=30)[0]
    b = W.descs_to_batch([d])
    assert 300 <= b.n_cv <= 400 and b.pulse_cell.size == 30
    assert np.all(b.pulse_branch >= 1)
