"""Markov channels (Nav1p6_MA2020_GoC, Kca2p2_MA2020_GoC, Kca1p1_MA2020_GoC) on the
GPU against the float64 oracle (``oracle/markov.py``: the reference's Markov template
and its backward-Euler subsolver).

A soma with the resurgent Nav1.6 scheme, KDR and both calcium-activated K schemes on
a dynamic calcium shell, and a dendrite with CaL: FP64 traces of the voltage, of
Markov states and of the Kca currents at 1e-8 (states, mV) over the whole run, FP32
within 1e-3 mV before spike onset and 0.05 ms on spike times, the stationary
distribution after a reset, and the lane kernel on a population of such somata.
"""

import numpy as np
import pytest

from braincell_gb300 import Branch, Cell, Morphology
from braincell_gb300 import _abi
from braincell_gb300.mech import (AllRegion, CableProperty, Channel, CurrentClamp, CurrentProbe, CVPerBranch, Ion,
                                  MechanismProbe, RootLocation, StateProbe, at, branch_in)

DT = 0.025


def _cell(precision="f64", pop_size=1, amp=0.4, mech_probes=True, nav="Nav1p6_MA2020_GoC"):
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    m = Morphology.from_root(soma, name="soma")
    m.attach(parent="soma", child_branch=Branch.from_lengths(lengths=[120.0], radii=[1.0, 0.6], type="dendrite"),
             child_name="d0")
    c = Cell(m, cv_policy=CVPerBranch(4), precision=precision, pop_size=pop_size)
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.2, E=-65.0),
            Ion("CalciumDetailed", C_rest=5e-5, tau=20.0, d=0.5, Ci_initializer=5e-5))
    c.paint(branch_in("type", "soma"), Channel(nav, g_max=60.0, name="nav"),
            Channel("KDR_Ba2002", g_max=20.0), Channel("Kca2p2_MA2020_GoC", g_max=1.0, name="sk"),
            Channel("Kca1p1_MA2020_GoC", g_max=2.0, name="bk"), Channel("CaL_IS2008", g_max=1.0))
    c.paint(branch_in("type", "dendrite"), Channel("CaL_IS2008", g_max=2.0))
    c.place(RootLocation(0.5), CurrentClamp(delay=2.0, durations=30.0, amplitudes=amp))
    c.place(RootLocation(0.5), StateProbe(name="v"))
    if mech_probes:
        c.place(RootLocation(0.5), MechanismProbe("nav", "O", name="nav_o"), MechanismProbe("nav", "B", name="nav_b"),
                MechanismProbe("sk", "O2", name="sk_o2"), MechanismProbe("bk", "O4", name="bk_o4"),
                CurrentProbe(mechanism="bk", name="i_bk"), CurrentProbe(mechanism="sk", name="i_sk"),
                CurrentProbe(ion="na", name="i_na"))
    c.place(at(1, 0.5), StateProbe(name="v_dend"))
    return c


def test_markov_probe_lowering():
    b = _cell().batch()
    base = _abi.BC_PROBE_CURRENT
    np.testing.assert_array_equal(
        b.probe_field, [0, _abi.BC_STATE_NAV16_O, _abi.BC_STATE_NAV16_O + 1, _abi.BC_STATE_KCA22_C2 + 4,
                        _abi.BC_STATE_KCA11_C1 + 8, base + _abi.BC_CUR_KCA11, base + _abi.BC_CUR_KCA22,
                        base + _abi.BC_CUR_ION_NA, 0])
    assert (b.region_mech & _abi.BC_M_NAV16).any() and (b.region_mech & _abi.BC_M_KCA11).any()


def test_markov_plans_run_the_extra_variant_with_the_markov_slots(native_lib):
    from braincell_gb300.runtime import Plan

    p = Plan(_cell().batch(), dry_run=True)
    assert p.info["kernel_variant"] == _abi.BC_VARIANT_EXTRA and p.info["state_slots"] == 52
    p.close()


@pytest.mark.gpu
@pytest.mark.parametrize("nav", ["Nav1p6_MA2020_GoC", "Nav1p1_MA2025_BC"])
def test_markov_cell_f64_matches_oracle(native_lib, cuda_device, nav):
    # Nav1p1_MA2025_BC: the same 13-state scheme with its own Oon, epsilon and phi
    from braincell_gb300.runtime import Plan
    from oracle.staggered import OracleCell

    n = 1400
    p = Plan(_cell(nav=nav).batch(), precision="f64", record_every=1, device=cuda_device)
    p.run(n, DT)
    gpu = p.traces()[:, :]
    oc = OracleCell(_cell(nav=nav))
    ref, osp = oc.run(DT, n)
    ref = ref[0]
    assert gpu.shape == ref.shape == (9, n)
    np.testing.assert_allclose(gpu[[0, 8]], ref[[0, 8]], rtol=0, atol=1e-8)  # mV
    np.testing.assert_allclose(gpu[1:5], ref[1:5], rtol=0, atol=1e-10)      # occupancies
    np.testing.assert_allclose(gpu[5:8], ref[5:8], rtol=1e-8, atol=1e-9)    # uA/cm^2
    sp = p.spikes()[0]
    assert len(sp) == len(osp[0][0]) >= 2
    assert np.abs(np.asarray(sp) - np.asarray(osp[0][0])).max() <= 1e-9
    # after the run, every CV's voltage
    np.testing.assert_allclose(p.state("V"), oc.V[0], rtol=0, atol=1e-8)
    p.close()


@pytest.mark.gpu
def test_markov_reset_is_the_stationary_distribution(native_lib, cuda_device):
    from braincell_gb300.runtime import Plan
    from oracle import markov as MK

    p = Plan(_cell().batch(), precision="f64", device=cuda_device)
    p.reset()
    v0 = p.state("V")[0]
    for cls, name in (("Nav1p6_MA2020_GoC", "Nav1p6"), ("Kca2p2_MA2020_GoC", "Kca2p2"),
                      ("Kca1p1_MA2020_GoC", "Kca1p1")):
        sch = MK.SCHEMES[cls]
        prm = MK.scheme_params(cls, MK.MARKOV_DEFAULTS[cls])
        ss = MK.steady_state(sch, sch.rates(np.array([v0]), 5e-5, prm))
        for k in sch.independent:
            got = p.state(f"{name}_{k}")[0]
            assert abs(got - ss[k][0]) <= 1e-12, (cls, k)
    p.close()


@pytest.mark.gpu
def test_markov_cell_f32_meets_the_bar(native_lib, cuda_device):
    from braincell_gb300.runtime import Plan

    n = 1400
    out = {}
    for prec in ("f32", "f64"):
        p = Plan(_cell(prec).batch(), precision=prec, record_every=1, device=cuda_device)
        p.run(n, DT)
        out[prec] = (p.traces()[0], p.spikes()[0])
        p.close()
    (t32, s32), (t64, s64) = out["f32"], out["f64"]
    rate = np.diff(t64) / DT
    onset = int(np.nonzero(rate > 10.0)[0][0]) + 1
    assert np.abs(t32[:onset] - t64[:onset]).max() <= 1e-3
    assert len(s32) == len(s64) >= 2
    assert np.abs(np.asarray(s32) - np.asarray(s64)).max() <= 0.05


@pytest.mark.gpu
def test_markov_somata_on_lane_tiles_match_packed_tiles(native_lib, cuda_device):
    # the lane kernel's extra-channel path runs the same Markov solver as the tiles
    from braincell_gb300.batch import concat_batches
    from braincell_gb300.runtime import Plan

    cells = [_cell(amp=a, mech_probes=False) for a in np.linspace(0.1, 0.6, 24)]
    b = concat_batches([c.batch() for c in cells])
    res = []
    for lanes in (0, 100):
        p = Plan(b, precision="f64", record_every=1, device=cuda_device, lane_cell_nodes=lanes)
        assert ((p.tile_stats()[:, 4] == 3).all()) == bool(lanes)
        p.run(800, DT)
        res.append((p.traces(), p.state("V")))
        p.close()
    np.testing.assert_allclose(res[0][0], res[1][0], rtol=0, atol=1e-9)
    np.testing.assert_allclose(res[0][1], res[1][1], rtol=0, atol=1e-9)
