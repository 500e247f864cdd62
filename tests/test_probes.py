"""Mechanism probes (gate states, Ci) next to voltage probes: lowering on the host,
traces against the float64 oracle on the GPU."""

import numpy as np
import pytest

from braincell_gb300 import Branch, Cell, Morphology
from braincell_gb300 import _abi
from braincell_gb300.mech import (AllRegion, CableProperty, Channel, CurrentClamp, CurrentProbe, CVPerBranch, Ion,
                                  MechanismProbe, RootLocation, StateProbe, at, branch_in)


def _cell(precision="f64"):
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    m = Morphology.from_root(soma, name="soma")
    m.attach(parent="soma", child_branch=Branch.from_lengths(lengths=[150.0], radii=[1.0, 0.5], type="dendrite"),
             child_name="d0")
    c = Cell(m, cv_policy=CVPerBranch(6), precision=precision)
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.3, E=-70.0))
    c.paint(branch_in("type", "soma"), Channel("Na_Ba2002", g_max=120.0, name="na_soma"),
            Channel("KDR_Ba2002", g_max=36.0))
    c.paint(branch_in("type", "dendrite"), Channel("CaL_IS2008", g_max=2.0), Channel("CaT_HM1992", g_max=2.1),
            Channel("AHP_De1994", g_max=0.3),
            Ion("CalciumDetailed", C_rest=5e-5, tau=10.0, d=0.5, Ci_initializer=5e-5))
    c.place(RootLocation(0.5), CurrentClamp(delay=2.0, durations=20.0, amplitudes=0.6))
    c.place(RootLocation(0.5), StateProbe(name="v_soma"), MechanismProbe("na_soma", "p", name="na_p"),
            MechanismProbe("KDR_Ba2002", "p", name="kdr_p"))
    c.place(at(1, 0.3), StateProbe(name="v_dend"), MechanismProbe("CaL_IS2008", "q", name="cal_q"),
            MechanismProbe("CalciumDetailed", "Ci", name="ci"), MechanismProbe("AHP_De1994", "p", name="ahp_p"))
    return c


def test_mechanism_probe_lowering():
    b = _cell().batch()
    np.testing.assert_array_equal(
        b.probe_field, [0, _abi.BC_STATE_NA_P, _abi.BC_STATE_KDR_P, 0, _abi.BC_STATE_CAL_Q, _abi.BC_STATE_CA_CI,
                        _abi.BC_STATE_AHP_P])
    assert _cell().probe_names() == ["v_soma", "na_p", "kdr_p", "v_dend", "cal_q", "ci", "ahp_p"]


def test_mechanism_probe_errors(native_lib):
    from braincell_gb300._abi import BCError
    from braincell_gb300.runtime import Plan

    with pytest.raises(ValueError):
        MechanismProbe("", "p")
    c = _cell()
    c.place(RootLocation(0.5), MechanismProbe("CaL_IS2008", "p", name="bad"))  # no CaL on the soma
    with pytest.raises(KeyError):
        c.batch()
    c = _cell()
    c.place(at(1, 0.5), MechanismProbe("CaL_IS2008", "z", name="bad"))
    with pytest.raises(KeyError):
        c.batch()
    b = _cell().batch()
    b.probe_field = b.probe_field.copy()
    b.probe_field[0] = _abi.BC_STATE_CAL_P  # the soma has no CaL
    with pytest.raises(BCError, match="no such mechanism"):
        Plan(b, dry_run=True)
    b.probe_field[0] = _abi.BC_NSTATE_VIEW  # the first code past the state views
    with pytest.raises(BCError, match="probe_field"):
        Plan(b, dry_run=True)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("f64", 1e-6), ("f32", 2e-4)])
def test_mechanism_probes_match_oracle(native_lib, cuda_device, precision, tol):
    from braincell_gb300.runtime import Plan
    from oracle.staggered import OracleCell

    c = _cell(precision)
    n = 1600
    p = Plan(c.batch(), precision=precision, record_every=1)
    p.run(n, 0.025)
    gpu = p.traces()
    oc = OracleCell(_cell("f64"))
    ref, _ = oc.run(0.025, n)
    ref = ref[0]
    assert gpu.shape == ref.shape == (7, n)
    # FP64 over the whole run; FP32 before the first spike's upstroke (dV/dt > 10 mV/ms).
    # Voltages in mV, gates and Ci relative to their largest value.
    end = n if precision == "f64" else int(np.nonzero(np.diff(ref[0]) / 0.025 > 10.0)[0][0])
    for k in range(7):
        scale = 1.0 if k in (0, 3) else max(np.abs(ref[k]).max(), 1e-12)
        err = np.abs(gpu[k, :end] - ref[k, :end]).max()
        assert err <= tol * scale * (5.0 if precision == "f32" and k in (0, 3) else 1.0), (k, err)
    # the states moved (the soma spikes, Ci rises)
    assert ref[1].max() - ref[1].min() > 0.5 and ref[5].max() > 2 * ref[5][0]
    # mechanism probes do not produce spikes; the soma voltage probe does
    sp = p.spikes()
    assert len(sp[0]) >= 1 and all(len(sp[k]) == 0 for k in (1, 2, 4, 5, 6))


def _current_cell(precision="f64"):
    c = _cell(precision)
    c.place(RootLocation(0.5), CurrentProbe(mechanism="na_soma", name="i_na"), CurrentProbe(ion="k", name="i_k"))
    c.place(at(1, 0.3), CurrentProbe(mechanism="CaL_IS2008", name="i_cal"), CurrentProbe(ion="ca", name="i_ca"),
            CurrentProbe(mechanism="IL", name="i_leak"))
    return c


def test_current_probe_lowering_and_errors():
    b = _current_cell().batch()
    C = _abi.BC_PROBE_CURRENT
    np.testing.assert_array_equal(b.probe_field[7:], [C + _abi.BC_CUR_NA, C + _abi.BC_CUR_ION_K, C + _abi.BC_CUR_CAL,
                                                      C + _abi.BC_CUR_ION_CA, C + _abi.BC_CUR_IL])
    with pytest.raises(ValueError):
        CurrentProbe()
    c = _cell()
    c.place(RootLocation(0.5), CurrentProbe(ion="xx"))
    with pytest.raises(KeyError):
        c.batch()


@pytest.mark.gpu
def test_current_probes_match_oracle(native_lib, cuda_device):
    from braincell_gb300.runtime import Plan
    from oracle.staggered import OracleCell

    n = 1200
    p = Plan(_current_cell("f64").batch(), precision="f64", record_every=1)
    p.run(n, 0.025)
    gpu = p.traces()[7:]
    ref = OracleCell(_current_cell("f64")).run(0.025, n)[0][0][7:]
    for k in range(5):
        scale = max(np.abs(ref[k]).max(), 1e-12)
        assert np.abs(gpu[k] - ref[k]).max() <= 1e-6 * scale, (k, np.abs(gpu[k] - ref[k]).max(), scale)
    # the sodium current is inward (positive as g (E - V)) and large during the spikes
    assert ref[0].max() > 10.0
