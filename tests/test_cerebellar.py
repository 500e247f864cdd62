"""Cerebellar channels of the MA2020 / MA2024 / MA2025 / RI2021 models: Kv3p4, Kv4p3,
Kv1p1, Kir2p3, the two HCN1 forms and the calcium channels CaHVA, Cav2p3 and Cav3p2,
with the cell-type variants that share their kinetics.

CPU: the published known answers of the reference docstrings (Kv1p1's n_inf = 1/2 at
-45 mV and the half-maximal n^4 near -29.9 mV, channel/potassium.py:4570), and the
variants' parameter records against their base class's.  GPU: a soma / dendrite cell
carrying all six kernels against the float64 oracle (FP64 at 1e-8 mV over the whole run,
or within a 1e-9 ms time shift on the upstrokes; gate and current probes, spikes) and
FP32 against FP64; a dendrite with the three
calcium channels on a CalciumDetailed shell (their step-start current drives Ci).
"""

import numpy as np
import pytest

from braincell_gb300 import Branch, Cell, Morphology
from braincell_gb300 import _abi, catalogue
from braincell_gb300.mech import (AllRegion, CableProperty, Channel, CurrentClamp, CurrentProbe, CVPerBranch, Ion,
                                  MechanismProbe, RootLocation, StateProbe, at, branch_in)
from oracle import staggered as O

DT = 0.025
SHIFT_MS = 1e-9  # the spike-time bar: a trace may lead or lag the oracle's by this much


def _assert_close_up_to_shift(gpu, ref, atol, rtol=0.0, err_msg=""):
    """``|gpu - ref| <= atol + rtol |ref| + SHIFT_MS |d ref / dt|`` elementwise.

    On an upstroke V climbs ~400 mV/ms, so a spike that crosses 1e-10 ms earlier (the
    rounding of exp and of the current sums, amplified by the Na feedback) reads as
    4e-8 mV at a fixed sample: the comparison takes the time shift that the spike-time
    check already accepts, and stays at ``atol`` where the trace is slow."""
    gpu, ref = np.atleast_2d(gpu), np.atleast_2d(ref)
    slope = np.abs(np.gradient(ref, DT, axis=-1))
    bound = atol + rtol * np.abs(ref) + SHIFT_MS * slope
    bad = np.abs(gpu - ref) > bound
    assert not bad.any(), (f"{err_msg}: {int(bad.sum())} samples off, worst excess "
                           f"{float((np.abs(gpu - ref) - bound).max()):.3e}")


def test_kv11_published_known_answers():
    p = O._resolve(O.CHANNEL_DEFAULTS, Channel("Kv1p1_MA2020_GoC"))
    _, a, b = O.rates("Kv1p1_MA2020_GoC", np.array([-45.0]), p)["n"]
    assert abs(a[0] / (a[0] + b[0]) - 0.5) < 1e-15  # equal prefactors: n_inf = 1/2 at -45 mV
    lo, hi = -45.0, 0.0
    for _ in range(60):  # n_inf^4 = 1/2: "reaches half its maximum near -29.9 mV"
        mid = 0.5 * (lo + hi)
        _, a, b = O.rates("Kv1p1_MA2020_GoC", np.array([mid]), p)["n"]
        lo, hi = (mid, hi) if (a[0] / (a[0] + b[0])) ** 4 < 0.5 else (lo, mid)
    assert abs(lo + 29.9) < 0.1


def test_variants_run_on_their_base_kernel():
    cable = CableProperty()
    for base, variants in catalogue.KINETIC_VARIANTS.items():
        for name, own in variants.items():
            bits_v, rec_v = catalogue.region_record([Channel(name)], cable)
            bits_b, rec_b = catalogue.region_record([Channel(base, **own)], cable)
            assert bits_v == bits_b != 0
            np.testing.assert_array_equal(rec_v, rec_b)
    # Kv4p3's variants differ from the Golgi-cell class in their default temperature only
    _, r22 = catalogue.region_record([Channel("Kv4p3_MA2020_GoC")], cable)
    _, r30 = catalogue.region_record([Channel("Kv4p3_MA2020_GrC")], cable)
    assert r30[_abi.BC_P_KV43_PHI] == pytest.approx(r22[_abi.BC_P_KV43_PHI] * 3.0 ** 0.8, rel=1e-12)


def test_kv11_gating_current_is_not_accepted():
    with pytest.raises(ValueError, match="gating current"):
        catalogue.region_record([Channel("Kv1p1_MA2020_GoC", gateCurrent=1.0)], CableProperty())


def _cell(precision="f64"):
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    m = Morphology.from_root(soma, name="soma")
    m.attach(parent="soma", child_branch=Branch.from_lengths(lengths=[160.0], radii=[1.2, 0.6], type="dendrite"),
             child_name="d0")
    c = Cell(m, cv_policy=CVPerBranch(5), precision=precision)
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.1, E=-65.0))
    c.paint(branch_in("type", "soma"), Channel("Na_Ba2002", g_max=120.0), Channel("KDR_Ba2002", g_max=40.0),
            Channel("Kv3p4_MA2020_GoC", g_max=5.0), Channel("Kv4p3_MA2020_GrC", g_max=1.0, name="ka"),
            Channel("Kv1p1_MA2020_GoC", g_max=0.2), Channel("HCN1_MA2020_GoC", g_max=0.5, name="hcn_f"))
    c.paint(branch_in("type", "dendrite"), Channel("Kir2p3_MA2020_GrC", g_max=0.5),
            Channel("HCN1_MA2024_PC", g_max=0.3, name="hcn_h"))
    c.place(RootLocation(0.5), CurrentClamp(delay=2.0, durations=25.0, amplitudes=0.4))
    c.place(RootLocation(0.5), StateProbe(name="v"), MechanismProbe("Kv3p4_MA2020_GoC", "h", name="kv34_h"),
            MechanismProbe("ka", "a", name="kv43_a"), MechanismProbe("hcn_f", "o_slow", name="hcn_slow"),
            CurrentProbe(mechanism="ka", name="i_ka"), CurrentProbe(mechanism="hcn_f", name="i_hcn"),
            CurrentProbe(ion="k", name="i_k"))
    c.place(at(1, 0.5), StateProbe(name="v_dend"))
    return c


def test_cerebellar_probe_lowering():
    b = _cell().batch()
    base = _abi.BC_PROBE_CURRENT
    np.testing.assert_array_equal(b.probe_field, [0, _abi.BC_STATE_KV34_H, _abi.BC_STATE_KV43_A,
                                                  _abi.BC_STATE_HCN1F_SLOW, base + _abi.BC_CUR_KV43,
                                                  base + _abi.BC_CUR_HCN1F, base + _abi.BC_CUR_ION_K, 0])


@pytest.mark.gpu
def test_cerebellar_cell_f64_matches_oracle(native_lib, cuda_device):
    from braincell_gb300.runtime import Plan

    n = 1200
    p = Plan(_cell().batch(), precision="f64", record_every=1, device=cuda_device)
    p.run(n, DT)
    gpu = p.traces()
    oc = O.OracleCell(_cell())
    ref, osp = oc.run(DT, n)
    ref = ref[0]
    _assert_close_up_to_shift(gpu[0], ref[0], atol=1e-8, err_msg="V")
    _assert_close_up_to_shift(gpu[1:4], ref[1:4], atol=1e-10, err_msg="gates")
    _assert_close_up_to_shift(gpu[4:7], ref[4:7], atol=1e-9, rtol=1e-8, err_msg="currents")
    sp = p.spikes()[0]
    assert len(sp) == len(osp[0][0]) >= 2
    assert np.abs(np.asarray(sp) - np.asarray(osp[0][0])).max() <= 1e-9
    np.testing.assert_allclose(p.state("V"), oc.V[0], rtol=0, atol=1e-8)
    kd = p.state("Kir2p3_d")
    on = np.isfinite(kd)  # the dendrite's five CVs; NaN on the soma, which does not carry Kir2.3
    assert on.sum() == 5 and not on[:5].any()
    np.testing.assert_allclose(kd[on], oc.gates[("Kir2p3_MA2020_GrC", "d")][0, oc.cv_mid][on], rtol=0, atol=1e-10)
    p.close()


@pytest.mark.gpu
def test_cerebellar_cell_f32_meets_the_bar(native_lib, cuda_device):
    from braincell_gb300.runtime import Plan

    n = 1200
    out = {}
    for prec in ("f32", "f64"):
        p = Plan(_cell(prec).batch(), precision=prec, record_every=1, device=cuda_device)
        p.run(n, DT)
        out[prec] = (p.traces()[0], p.spikes()[0])
        p.close()
    (t32, s32), (t64, s64) = out["f32"], out["f64"]
    onset = int(np.nonzero(np.diff(t64) / DT > 10.0)[0][0]) + 1
    assert np.abs(t32[:onset] - t64[:onset]).max() <= 1e-3
    assert len(s32) == len(s64) >= 2
    assert np.abs(np.asarray(s32) - np.asarray(s64)).max() <= 0.05


def _ca_cell(precision="f64"):
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    m = Morphology.from_root(soma, name="soma")
    m.attach(parent="soma", child_branch=Branch.from_lengths(lengths=[150.0], radii=[1.0, 0.6], type="dendrite"),
             child_name="d0")
    c = Cell(m, cv_policy=CVPerBranch(5), precision=precision)
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.1, E=-65.0))
    c.paint(branch_in("type", "soma"), Channel("Na_Ba2002", g_max=120.0), Channel("KDR_Ba2002", g_max=40.0))
    c.paint(branch_in("type", "dendrite"), Channel("CaHVA_MA2020_GrC", g_max=0.5),
            Channel("Cav2p3_MA2020_GoC", g_max=0.3), Channel("Cav3p2_MA2024_PC", g_max=0.4, V_sh=5.0),
            Channel("Kv4p3_MA2020_GoC", g_max=0.5),
            Ion("CalciumDetailed", C_rest=5e-5, tau=20.0, d=0.5, Ci_initializer=5e-5))
    c.place(RootLocation(0.5), CurrentClamp(delay=2.0, durations=20.0, amplitudes=0.4), StateProbe(name="v"))
    c.place(at(1, 0.5), StateProbe(name="v_dend"), MechanismProbe("CalciumDetailed", "Ci", name="ci"),
            MechanismProbe("Cav3p2_MA2024_PC", "h", name="cav32_h"), CurrentProbe(ion="ca", name="i_ca"),
            CurrentProbe(mechanism="CaHVA_MA2020_GrC", name="i_hva"))
    return c


def test_calcium_channel_probe_lowering():
    b = _ca_cell().batch()
    base = _abi.BC_PROBE_CURRENT
    np.testing.assert_array_equal(b.probe_field, [0, 0, _abi.BC_STATE_CA_CI, _abi.BC_STATE_CAV32_H,
                                                  base + _abi.BC_CUR_ION_CA, base + _abi.BC_CUR_CAHVA])


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol_v,tol_ci", [("f64", 1e-8, 1e-12), ("f32", None, 1e-6)])
def test_calcium_channels_drive_the_shell_like_the_oracle(native_lib, cuda_device, precision, tol_v, tol_ci):
    from braincell_gb300.runtime import Plan

    n = 1000
    p = Plan(_ca_cell(precision).batch(), precision=precision, record_every=1, device=cuda_device)
    p.run(n, DT)
    gpu = p.traces()
    p.close()
    ref, osp = O.OracleCell(_ca_cell()).run(DT, n)
    ref = ref[0]
    assert ref[2].max() > 2.0 * ref[2][0]  # the shell fills from the dendritic channels
    if precision == "f64":
        _assert_close_up_to_shift(gpu[:2], ref[:2], atol=tol_v, err_msg="V")
        _assert_close_up_to_shift(gpu[3], ref[3], atol=1e-10, err_msg="Cav3p2 h")
        _assert_close_up_to_shift(gpu[4:], ref[4:], atol=1e-9, rtol=1e-8, err_msg="currents")
        _assert_close_up_to_shift(gpu[2], ref[2], atol=tol_ci, rtol=1e-9, err_msg="Ci")
    else:
        onset = int(np.nonzero(np.diff(ref[0]) / DT > 10.0)[0][0]) + 1
        assert np.abs(gpu[0][:onset] - ref[0][:onset]).max() <= 1e-3
        np.testing.assert_allclose(gpu[2][:onset], ref[2][:onset], rtol=1e-5, atol=tol_ci)
