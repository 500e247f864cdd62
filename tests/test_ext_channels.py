"""Extension channels (BC_M_EXT with BC_X_* bits in the record): HCN2_MA2020_GoC,
Kv3p3_MA2024_PC, Kv2p2_0010_MA2020_GrC, Kv1p5_MA2024_PC (and Kv1p5_MA2020_GrC on its
kernel), the SU2015 DCN sodium / potassium / HCN / CaL classes, the ZH2019 IO sodium /
potassium / HCN classes, CaT_HP1992 and CaHT_Re1993 driving a CalciumDetailed shell, the
calcium-gated Kca3p1 (and its BC / PC classes) and SK_SU2015_DCN, K_Kv_test, CaN_IS2008
(Ci-modulated, carried by calcium in its own E), Ca_ZH2019_IO (and its Frozen class), and
the Markov scheme Nav_MA2020_GrC, and Cav3p1 (GoC, PC and their _Frozen classes) with its
GHK drive, Cav3p3 (RI2021_SC, MA2024_PC and its _Frozen class) with its own, and the
Ci-inactivated Cav1p2 / Cav1p3 (and their BC classes), and Cav2p1 (SC, PC, BC) on the
shared GHK drive, and the SU2015 DCN CaHVA / CaLVA on their own drive (the DCN cell).

CPU: the records and their mask, the planner's check of the mask, and the owner
tables (through the planner tests).  GPU: a DCN-like cell and an IO-like cell
against the float64 oracle (FP64 at 1e-8 mV, or within a 1e-9 ms time shift on the
upstrokes; gate and current probes, spikes), and FP32 against FP64.
"""

import numpy as np
import pytest

from braincell_gb300 import Branch, Cell, Morphology, _abi, catalogue
from braincell_gb300.mech import (AllRegion, CableProperty, Channel, CurrentClamp, CurrentProbe, CVPerBranch, Ion,
                                  MechanismProbe, RootLocation, StateProbe, at, branch_in)
from oracle import staggered as O

DT = 0.025
SHIFT_MS = 1e-9


def _close(gpu, ref, atol, rtol=0.0, what=""):
    """|gpu - ref| <= atol + rtol |ref| + SHIFT_MS |d ref / dt| (the spike-time bar as a
    time shift on the fast upstrokes)."""
    gpu, ref = np.atleast_2d(gpu), np.atleast_2d(ref)
    bound = atol + rtol * np.abs(ref) + SHIFT_MS * np.abs(np.gradient(ref, DT, axis=-1))
    bad = np.abs(gpu - ref) > bound
    assert not bad.any(), f"{what}: {int(bad.sum())} samples off, worst {float((np.abs(gpu - ref) - bound).max()):.3e}"


def test_extension_records():
    cable = CableProperty()
    bits, rec = catalogue.region_record([Channel("HCN2_MA2020_GoC"), Channel("Kv1p5_MA2024_PC", temp=O._c2k(30.0)),
                                         Channel("Na_ZH2019_IO")], cable)
    assert bits == _abi.BC_M_EXT
    assert int(rec[_abi.BC_P_EXT_MASK]) == _abi.BC_X_HCN2 | _abi.BC_X_KV15 | _abi.BC_X_NAIO
    # HCN2's conductance carries its Q10 1.5 factor, its gates q10 3, both at 23 degC
    assert rec[_abi.BC_P_HCN2_G] == pytest.approx(0.08 * 1.5 ** (-0.1), rel=1e-12)
    assert rec[_abi.BC_P_HCN2_PHI] == pytest.approx(3.0 ** (-0.1), rel=1e-12)
    assert rec[_abi.BC_P_KV15_Q10] == pytest.approx(2.2 ** (-0.7), rel=1e-12)
    assert rec[_abi.BC_P_NAIO_G] == 70.0
    # the defaults of the reference classes, in mS/cm^2 (Kv3p3 0.005 S/cm^2, Kv1p5 0.13195e-3 S/cm^2)
    _, rec = catalogue.region_record([Channel("Kv3p3_MA2024_PC"), Channel("Kv1p5_MA2024_PC")], cable)
    assert rec[_abi.BC_P_KV33_G] == 5.0 and rec[_abi.BC_P_KV15_G] == pytest.approx(0.13195)
    # bits 24 and up go to a second record entry, so that both stay exact in an FP32 record
    _, rec = catalogue.region_record([Channel("HCN2_MA2020_GoC"), Channel("Cav2p1_RI2021_SC")], cable)
    assert rec[_abi.BC_P_EXT_MASK] == _abi.BC_X_HCN2 and rec[_abi.BC_P_EXT_MASK_HI] == _abi.BC_X_CAV21 >> 24
    assert catalogue.ext_mask(rec.astype(np.float32)) == _abi.BC_X_HCN2 | _abi.BC_X_CAV21
    # no extension channel: no mask, no bit
    bits, rec = catalogue.region_record([Channel("IL")], cable)
    assert not bits & _abi.BC_M_EXT and rec[_abi.BC_P_EXT_MASK] == 0.0
    with pytest.raises(ValueError, match="gating current"):
        catalogue.region_record([Channel("Kv3p3_MA2024_PC", gateCurrent=1.0)], cable)


def test_planner_checks_the_extension_mask(native_lib):
    from braincell_gb300.batch import lower_cell
    from braincell_gb300.runtime import Plan

    b = lower_cell(_io_cell())
    Plan(b, dry_run=True).close()
    for bad in (0.0, 0.5, float(_abi.BC_X_ALL + 1)):
        b2 = lower_cell(_io_cell())
        b2.region_params = b2.region_params.copy()
        b2.region_params[:, _abi.BC_P_EXT_MASK] = bad
        with pytest.raises(_abi.BCError, match="BC_P_EXT_MASK"):
            Plan(b2, dry_run=True)


def _dcn_cell(precision="f64"):
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    m = Morphology.from_root(soma, name="soma")
    m.attach(parent="soma", child_branch=Branch.from_lengths(lengths=[150.0], radii=[1.2, 0.6], type="dendrite"),
             child_name="d0")
    c = Cell(m, cv_policy=CVPerBranch(5), precision=precision)
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.05, E=-65.0))
    c.paint(branch_in("type", "soma"), Channel("NaF_SU2015_DCN", g_max=40.0), Channel("NaP_SU2015_DCN", g_max=0.2),
            Channel("fKdr_SU2015_DCN", g_max=15.0), Channel("sKdr_SU2015_DCN", g_max=4.0),
            Channel("HCN_SU2015_DCN", g_max=0.3))
    c.paint(branch_in("type", "dendrite"), Channel("Kv1p5_MA2024_PC", g_max=0.5), Channel("Kv3p3_MA2024_PC", g_max=1.0),
            Channel("Kv2p2_0010_MA2020_GrC", g_max=0.5), Channel("HCN2_MA2020_GoC", g_max=0.3),
            Channel("CaHVA_SU2015_DCN", perm=2e-4), Channel("CaLVA_SU2015_DCN", perm=5e-5))
    c.place(RootLocation(0.5), CurrentClamp(delay=2.0, durations=20.0, amplitudes=0.3), StateProbe(name="v"),
            MechanismProbe("NaF_SU2015_DCN", "h", name="naf_h"), CurrentProbe(mechanism="NaF_SU2015_DCN", name="i_naf"),
            CurrentProbe(ion="na", name="i_na"))
    c.place(at(1, 0.5), StateProbe(name="v_dend"), MechanismProbe("Kv1p5_MA2024_PC", "m", name="kv15_m"),
            MechanismProbe("HCN2_MA2020_GoC", "o_slow", name="hcn2_s"),
            CurrentProbe(mechanism="Kv1p5_MA2024_PC", name="i_kv15"), CurrentProbe(ion="k", name="i_k"),
            MechanismProbe("CaLVA_SU2015_DCN", "h", name="calva_h"), CurrentProbe(ion="ca", name="i_ca"))
    return c


def _io_cell(precision="f64"):
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    c = Cell(Morphology.from_root(soma, name="soma"), cv_policy=CVPerBranch(), precision=precision)
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.1, E=-65.0), Channel("Na_ZH2019_IO"),
            Channel("Kdr_ZH2019_IO"), Channel("HCN_ZH2019_IO"), Channel("Cav3p1Test_PC24", g_max=0.5))
    c.place(RootLocation(0.5), CurrentClamp(delay=2.0, durations=15.0, amplitudes=0.5), StateProbe(name="v"),
            MechanismProbe("Kdr_ZH2019_IO", "n", name="kdr_n"), MechanismProbe("HCN_ZH2019_IO", "q", name="hcn_q"),
            CurrentProbe(mechanism="Na_ZH2019_IO", name="i_na"), CurrentProbe(mechanism="Cav3p1Test_PC24", name="i_t"))
    return c


def _ca_cell(precision="f64"):
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    m = Morphology.from_root(soma, name="soma")
    m.attach(parent="soma", child_branch=Branch.from_lengths(lengths=[150.0], radii=[1.0, 0.6], type="dendrite"),
             child_name="d0")
    c = Cell(m, cv_policy=CVPerBranch(5), precision=precision)
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.1, E=-65.0))
    c.paint(branch_in("type", "soma"), Channel("Na_Ba2002", g_max=120.0), Channel("KDR_Ba2002", g_max=40.0),
            Channel("CaL_SU2015_DCN", g_max=0.5), Channel("Kv1p5_MA2020_GrC", g_max=1.0))
    c.paint(branch_in("type", "dendrite"), Channel("CaT_HP1992", g_max=0.5), Channel("CaHT_Re1993", g_max=0.5),
            Ion("CalciumDetailed", C_rest=5e-5, tau=20.0, d=0.5, Ci_initializer=5e-5))
    c.place(RootLocation(0.5), CurrentClamp(delay=2.0, durations=20.0, amplitudes=0.4), StateProbe(name="v"),
            MechanismProbe("CaL_SU2015_DCN", "h", name="cal_h"), CurrentProbe(mechanism="Kv1p5_MA2020_GrC", name="i_kv"))
    c.place(at(1, 0.5), StateProbe(name="v_dend"), MechanismProbe("CalciumDetailed", "Ci", name="ci"),
            MechanismProbe("CaT_HP1992", "p", name="cat_p"), MechanismProbe("CaHT_Re1993", "q", name="caht_q"),
            CurrentProbe(ion="ca", name="i_ca"), CurrentProbe(mechanism="CaHT_Re1993", name="i_caht"))
    return c


def _kca_cell(precision="f64"):
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    m = Morphology.from_root(soma, name="soma")
    m.attach(parent="soma", child_branch=Branch.from_lengths(lengths=[150.0], radii=[1.0, 0.6], type="dendrite"),
             child_name="d0")
    c = Cell(m, cv_policy=CVPerBranch(5), precision=precision)
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.1, E=-65.0))
    # the soma's SK sees the fixed Ci; the dendrite's Kca3p1 and SK the shell's Ci
    c.paint(branch_in("type", "soma"), Channel("Na_Ba2002", g_max=120.0), Channel("KDR_Ba2002", g_max=30.0),
            Channel("K_Kv_test", g_max=0.5), Channel("SK_SU2015_DCN", g_max=0.05))
    c.paint(branch_in("type", "dendrite"), Channel("CaHT_Re1993", g_max=1.0), Channel("Kca3p1_MA2024_PC", g_max=0.3),
            Channel("SK_SU2015_DCN", g_max=0.3),
            Ion("CalciumDetailed", C_rest=5e-5, tau=20.0, d=0.5, Ci_initializer=5e-5))
    c.place(RootLocation(0.5), CurrentClamp(delay=2.0, durations=20.0, amplitudes=0.5), StateProbe(name="v"),
            MechanismProbe("K_Kv_test", "n", name="kkv_n"), CurrentProbe(mechanism="SK_SU2015_DCN", name="i_sk_soma"))
    c.place(at(1, 0.5), StateProbe(name="v_dend"), MechanismProbe("CalciumDetailed", "Ci", name="ci"),
            MechanismProbe("Kca3p1_MA2024_PC", "p", name="kca31_p"), MechanismProbe("SK_SU2015_DCN", "z", name="sk_z"),
            CurrentProbe(ion="k", name="i_k"))
    return c


def _can_cell(precision="f64", frozen=True):
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    m = Morphology.from_root(soma, name="soma")
    m.attach(parent="soma", child_branch=Branch.from_lengths(lengths=[150.0], radii=[1.0, 0.6], type="dendrite"),
             child_name="d0")
    c = Cell(m, cv_policy=CVPerBranch(5), precision=precision)
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.1, E=-65.0))
    # Ca_ZH2019_IO with m_inf held out of the linearisation (the Frozen class) or in it
    io = Channel("Ca_ZH2019_IO_Frozen", g_max=0.5) if frozen else Channel("Ca_ZH2019_IO", g_max=0.5, freeze_m_inf=False)
    c.paint(branch_in("type", "soma"), Channel("Na_ZH2019_IO"), Channel("Kdr_ZH2019_IO"), io)
    c.paint(branch_in("type", "dendrite"), Channel("CaHT_Re1993", g_max=0.5), Channel("CaN_IS2008", g_max=0.5),
            Ion("CalciumDetailed", C_rest=5e-5, tau=20.0, d=0.5, Ci_initializer=5e-5))
    c.place(RootLocation(0.5), CurrentClamp(delay=2.0, durations=20.0, amplitudes=0.4), StateProbe(name="v"),
            CurrentProbe(mechanism="Ca_ZH2019_IO_Frozen" if frozen else "Ca_ZH2019_IO", name="i_caio"))
    c.place(at(1, 0.5), StateProbe(name="v_dend"), MechanismProbe("CalciumDetailed", "Ci", name="ci"),
            MechanismProbe("CaN_IS2008", "p", name="can_p"), CurrentProbe(mechanism="CaN_IS2008", name="i_can"),
            CurrentProbe(ion="ca", name="i_ca"))
    return c


def _can_cell_unfrozen(precision="f64"):
    return _can_cell(precision, frozen=False)


def _grc_cell(precision="f64"):
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    c = Cell(Morphology.from_root(soma, name="soma"), cv_policy=CVPerBranch(), precision=precision)
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.1, E=-65.0), Channel("Nav_MA2020_GrC", g_max=40.0),
            Channel("Kdr_ZH2019_IO", g_max=18.0), Channel("Kv2p2_0010_MA2020_GrC", g_max=1.0))
    c.place(RootLocation(0.5), CurrentClamp(delay=2.0, durations=15.0, amplitudes=0.4), StateProbe(name="v"),
            MechanismProbe("Nav_MA2020_GrC", "O", name="nav_o"), MechanismProbe("Nav_MA2020_GrC", "OB", name="nav_ob"),
            MechanismProbe("Nav_MA2020_GrC", "I3", name="nav_i3"), CurrentProbe(mechanism="Nav_MA2020_GrC", name="i_nav"),
            CurrentProbe(ion="na", name="i_na"))
    return c


def _cav31_cell(precision="f64"):
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    m = Morphology.from_root(soma, name="soma")
    m.attach(parent="soma", child_branch=Branch.from_lengths(lengths=[150.0], radii=[1.0, 0.6], type="dendrite"),
             child_name="d0")
    c = Cell(m, cv_policy=CVPerBranch(5), precision=precision)
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.1, E=-65.0))
    # the soma: the Frozen class on the fixed calcium ion; the dendrite: the GHK drive in
    # the linearisation, on a CalciumDetailed shell that it fills
    c.paint(branch_in("type", "soma"), Channel("Na_Ba2002", g_max=120.0), Channel("KDR_Ba2002", g_max=40.0),
            Channel("Cav3p1_MA2024_PC_Frozen", g_max=1e-4), Channel("Cav1p3_MA2025_BC", g_max=0.3),
            Channel("Cav2p1_RI2021_SC_Frozen", g_max=3e-5, V_sh=1.0))
    c.paint(branch_in("type", "dendrite"), Channel("Cav3p1_MA2020_GoC", g_max=2.5e-4),
            Channel("Cav3p3_RI2021_SC", perm=2e-4, g_scale=1.0, V_sh=3.0), Channel("Cav1p2_MA2020_GoC", g_max=0.5),
            Ion("CalciumDetailed", C_rest=5e-5, tau=20.0, d=0.5, Ci_initializer=5e-5))
    c.place(RootLocation(0.5), CurrentClamp(delay=2.0, durations=20.0, amplitudes=0.3), StateProbe(name="v"),
            CurrentProbe(mechanism="Cav3p1_MA2024_PC_Frozen", name="i_cav_soma"),
            CurrentProbe(mechanism="Cav2p1_RI2021_SC_Frozen", name="i_cav21_frozen"))
    c.place(at(1, 0.5), StateProbe(name="v_dend"), MechanismProbe("CalciumDetailed", "Ci", name="ci"),
            MechanismProbe("Cav3p1_MA2020_GoC", "p", name="cav_p"), MechanismProbe("Cav3p1_MA2020_GoC", "q", name="cav_q"),
            CurrentProbe(mechanism="Cav3p1_MA2020_GoC", name="i_cav"), CurrentProbe(ion="ca", name="i_ca"),
            MechanismProbe("Cav3p3_RI2021_SC", "l", name="cav33_l"), CurrentProbe(mechanism="Cav3p3_RI2021_SC",
                                                                                name="i_cav33"),
            MechanismProbe("Cav1p2_MA2020_GoC", "n", name="cav12_n"), CurrentProbe(mechanism="Cav1p2_MA2020_GoC",
                                                                                 name="i_cav12"))
    return c


def _cav33_frozen_cell(precision="f64"):
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    c = Cell(Morphology.from_root(soma, name="soma"), cv_policy=CVPerBranch(), precision=precision)
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.1, E=-65.0), Channel("Na_Ba2002", g_max=120.0),
            Channel("KDR_Ba2002", g_max=40.0), Channel("Cav3p3_MA2024_PC_Frozen", perm=2e-4, g_scale=1.0),
            Channel("Cav2p1_MA2025_BC", g_max=2e-5, V_sh=-2.0),
            Ion("CalciumDetailed", C_rest=5e-5, tau=20.0, d=0.5, Ci_initializer=5e-5))
    c.place(RootLocation(0.5), CurrentClamp(delay=2.0, durations=20.0, amplitudes=0.3), StateProbe(name="v"),
            MechanismProbe("CalciumDetailed", "Ci", name="ci"), CurrentProbe(ion="ca", name="i_ca"),
            MechanismProbe("Cav2p1_MA2025_BC", "m", name="cav21_m"), CurrentProbe(mechanism="Cav2p1_MA2025_BC",
                                                                                name="i_cav21"))
    return c


def test_kv15_grc_runs_on_the_pc_kernel():
    cable = CableProperty()
    assert catalogue.region_record([Channel("Kv1p5_MA2020_GrC", g_max=0.3)], cable)[1].tolist() == \
        catalogue.region_record([Channel("Kv1p5_MA2024_PC", g_max=0.3)], cable)[1].tolist()
    with pytest.raises(ValueError, match="gnonspec"):
        catalogue.region_record([Channel("Kv1p5_MA2020_GrC", gnonspec=1e-4)], cable)


@pytest.mark.gpu
@pytest.mark.parametrize("make,n", [(_dcn_cell, 1000), (_io_cell, 800), (_ca_cell, 1000), (_kca_cell, 1000),
                                    (_can_cell, 1000), (_can_cell_unfrozen, 1000), (_grc_cell, 800),
                                    (_cav31_cell, 1000), (_cav33_frozen_cell, 1000)],
                         ids=["dcn", "io", "ca", "kca", "can", "can_unfrozen", "grc", "cav31", "cav33_frozen"])
def test_extension_cells_f64_match_oracle(native_lib, cuda_device, make, n):
    from braincell_gb300.runtime import Plan

    p = Plan(make().batch(), precision="f64", record_every=1, device=cuda_device)
    p.run(n, DT)
    gpu, sp = p.traces(), p.spikes()[0]
    oc = O.OracleCell(make())
    ref, osp = oc.run(DT, n)
    ref = ref[0]
    fields = make().batch().probe_field
    for k, f in enumerate(fields):
        if f == _abi.BC_STATE_V:
            _close(gpu[k], ref[k], 1e-8, what=f"V probe {k}")
        elif f >= _abi.BC_PROBE_CURRENT:
            _close(gpu[k], ref[k], 1e-9, rtol=1e-8, what=f"current probe {k}")
        elif f == _abi.BC_STATE_CA_CI:
            _close(gpu[k], ref[k], 1e-12, rtol=1e-9, what=f"Ci probe {k}")
        else:
            _close(gpu[k], ref[k], 1e-10, what=f"state probe {k}")
    assert len(sp) == len(osp[0][0]) >= 2
    assert np.abs(np.asarray(sp) - np.asarray(osp[0][0])).max() <= 1e-9
    np.testing.assert_allclose(p.state("V"), oc.V[0], rtol=0, atol=1e-8)
    p.close()


@pytest.mark.gpu
@pytest.mark.parametrize("make", [_dcn_cell, _io_cell, _ca_cell, _kca_cell, _can_cell, _grc_cell, _cav31_cell,
                                  _cav33_frozen_cell],
                         ids=["dcn", "io", "ca", "kca", "can", "grc", "cav31", "cav33_cav21"])
def test_extension_cells_f32_meet_the_bar(native_lib, cuda_device, make):
    from braincell_gb300.runtime import Plan

    out = {}
    for prec in ("f32", "f64"):
        p = Plan(make(prec).batch(), precision=prec, record_every=1, device=cuda_device)
        p.run(800, DT)
        out[prec] = (p.traces()[0], p.spikes()[0])
        p.close()
    (t32, s32), (t64, s64) = out["f32"], out["f64"]
    onset = int(np.nonzero(np.diff(t64) / DT > 10.0)[0][0]) + 1
    assert np.abs(t32[:onset] - t64[:onset]).max() <= 1e-3
    assert len(s32) == len(s64) >= 2
    assert np.abs(np.asarray(s32) - np.asarray(s64)).max() <= 0.05
