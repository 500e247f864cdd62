"""bc_state_download_noalloc: the state download that allocates nothing.

Collected last (file name), so on a GPU it runs both after every other test and,
when run alone, in a fresh process where its first call does the scratch set-up.
Its values must equal bc_state_download's (same view kernel, same offsets) on two
calls in a row, for every state view, in both precisions.
"""

import ctypes as C

import numpy as np
import pytest

from braincell_gb300 import _abi
from braincell_gb300 import workloads as W
from braincell_gb300.runtime import Plan


def _download_noalloc(lib, plan, which):
    out = np.full(plan.n_cv, -7.0)
    st = lib.bc_state_download_noalloc(plan._h, which, out.ctypes.data_as(C.POINTER(C.c_double)), None)
    return st, out


def test_plan_above_capacity_is_rejected(native_lib):
    descs = W.uneven(480)
    plan = Plan(W.descs_to_batch(descs), dry_run=True)
    assert plan.n_cv > _abi.BC_NOALLOC_MAX_CV
    st, out = _download_noalloc(native_lib, plan, _abi.BC_STATE_V)
    assert st == _abi.BC_ERR_INVALID
    msg = native_lib.bc_last_error()
    assert b"BC_NOALLOC_MAX_CV" in msg and str(plan.n_cv).encode() in msg
    assert (out == -7.0).all()


def test_invalid_arguments_are_rejected(native_lib):
    plan = Plan(W.descs_to_batch(W.small(2)), dry_run=True)
    assert _download_noalloc(native_lib, plan, _abi.BC_NSTATE_VIEW)[0] == _abi.BC_ERR_INVALID
    assert _download_noalloc(native_lib, plan, -1)[0] == _abi.BC_ERR_INVALID
    st, _ = _download_noalloc(native_lib, plan, _abi.BC_STATE_V)
    assert st == _abi.BC_ERR_INVALID and b"dry_run" in native_lib.bc_last_error()
    assert native_lib.bc_state_download_noalloc(None, 0, None, None) == _abi.BC_ERR_INVALID


def _calcium_desc():
    return W.large(indices=[0], n_range=(300, 400), n_branches=20, n_pulses=60, duration=20.0)[0]


def _hh_batch():
    # a cell with the classic Hodgkin-Huxley channels, the M current and both A-current
    # and slow K2 components, so that every state view has values somewhere in the batch
    from braincell_gb300 import Branch, Cell, Morphology
    from braincell_gb300.batch import lower_cell
    from braincell_gb300.mech import AllRegion, CableProperty, Channel, CVPerBranch, branch_in

    m = Morphology.from_root(Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma"), name="soma")
    m.attach(parent="soma", child_branch=Branch.from_lengths(lengths=[100.0], radii=[1.0, 0.6], type="basal_dendrite"))
    c = Cell(m, cv_policy=CVPerBranch())
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.3, E=-54.4))
    c.paint(branch_in("type", "soma"), Channel("Na_HH1952"), Channel("K_HH1952", g_max=36.0))
    c.paint(branch_in("type", "basal_dendrite"), Channel("KM_RI2021_SC"), Channel("KA1_HM1992", g_max=3.0),
            Channel("KA2_HM1992", g_max=2.0), Channel("KK2A_HM1992", g_max=1.0), Channel("KK2B_HM1992", g_max=1.0),
            Channel("KNI_Ya1989"), Channel("Nav1p6_MA2020_GoC", g_max=2.0), Channel("Kca2p2_MA2020_GoC", g_max=1.0),
            Channel("Kca1p1_MA2020_GoC", g_max=1.0),  # and the Markov and cerebellar channels' state views
            Channel("Kv3p4_MA2020_GoC", g_max=0.5), Channel("Kv4p3_MA2020_GoC", g_max=0.5),
            Channel("Kv1p1_MA2020_GoC", g_max=0.2), Channel("Kir2p3_MA2020_GrC", g_max=0.2),
            Channel("HCN1_MA2020_GoC", g_max=0.05), Channel("HCN1_MA2024_PC", g_max=0.05),
            Channel("CaHVA_MA2020_GoC", g_max=0.05), Channel("Cav2p3_MA2020_GoC", g_max=0.05),
            Channel("Cav3p2_RI2021_SC", g_max=0.05),
            # and the extension channels' views
            Channel("HCN2_MA2020_GoC", g_max=0.05), Channel("Kv3p3_MA2024_PC", g_max=0.2),
            Channel("Kv2p2_0010_MA2020_GrC", g_max=0.2), Channel("Kv1p5_MA2024_PC", g_max=0.2),
            Channel("NaF_SU2015_DCN", g_max=0.2), Channel("NaP_SU2015_DCN", g_max=0.05),
            Channel("Na_ZH2019_IO", g_max=0.2), Channel("fKdr_SU2015_DCN", g_max=0.2),
            Channel("sKdr_SU2015_DCN", g_max=0.2), Channel("Kdr_ZH2019_IO", g_max=0.2),
            Channel("HCN_SU2015_DCN", g_max=0.05), Channel("HCN_ZH2019_IO", g_max=0.05),
            Channel("CaT_HP1992", g_max=0.05), Channel("CaHT_Re1993", g_max=0.05),
            Channel("CaL_SU2015_DCN", g_max=0.05), Channel("Kca3p1_MA2020_GoC", g_max=0.05),
            Channel("SK_SU2015_DCN", g_max=0.05), Channel("K_Kv_test", g_max=0.05),
            Channel("CaN_IS2008", g_max=0.05), Channel("Ca_ZH2019_IO", g_max=0.05),
            Channel("Nav_MA2020_GrC", g_max=0.2), Channel("Cav3p1_MA2020_GoC", g_max=1e-5),
            Channel("Cav3p3_RI2021_SC"), Channel("Cav1p2_MA2020_GoC", g_max=0.01), Channel("Cav1p3_MA2020_GoC"),
            Channel("Cav2p1_RI2021_SC", g_max=1e-6), Channel("CaHVA_SU2015_DCN"),
            Channel("CaLVA_SU2015_DCN", perm=1e-6))
    return lower_cell(c)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_noalloc_download_matches_download(native_lib, cuda_device, precision):
    from braincell_gb300.batch import concat_batches

    descs = W.small(4) + [_calcium_desc()] + W.uneven(indices=[0, 1])
    plan = Plan(concat_batches([W.descs_to_batch(descs), _hh_batch()]), precision=precision, device=cuda_device)
    assert plan.n_cv <= _abi.BC_NOALLOC_MAX_CV
    for segment in range(2):
        plan.run(300, 0.025)
        for name, which in _abi.STATE_NAMES.items():
            ref = plan.state(name)
            first = plan.state_into(name, np.empty(plan.n_cv))
            st, second = _download_noalloc(native_lib, plan, which)
            assert st == _abi.BC_OK, native_lib.bc_last_error()
            # bit-identical to the allocating download, NaN where the mechanism is absent
            np.testing.assert_array_equal(first, ref, err_msg=f"{name}, segment {segment}, first call")
            np.testing.assert_array_equal(second, ref, err_msg=f"{name}, segment {segment}, second call")
            assert np.isfinite(ref).any(), name
    plan.close()
