"""InitNernst ions (ion/_base.py:261-360): fixed Ci / Co with the reversal potential
stored once from the Nernst equation.  CPU: the catalogue's E against the textbook
value at the family defaults and against the oracle's; the E reaches the channel's
reversal slot.  GPU: a soma with Na / K / CaL on InitNernst ions against the float64
oracle."""

import numpy as np
import pytest

from braincell_gb300 import Branch, Cell, Morphology, _abi, catalogue
from braincell_gb300.mech import (AllRegion, CableProperty, Channel, CurrentClamp, CVPerBranch, Ion, RootLocation,
                                  StateProbe)
from oracle import staggered as O

# RT/F at 36 degC in mV: 8.314462618 * 309.15 / 96485.33212 * 1e3
RT_F_36 = 26.6404858


def test_init_nernst_reversal_potentials():
    cable = CableProperty()
    cases = {"SodiumInitNernst": (_abi.BC_P_ENA, RT_F_36 * np.log(140.0 / 10.0)),
             "PotassiumInitNernst": (_abi.BC_P_EK, RT_F_36 * np.log(2.5 / 54.4)),
             "CalciumInitNernst": (_abi.BC_P_ECA, RT_F_36 / 2.0 * np.log(2.0 / 5e-5))}
    for name, (slot, want) in cases.items():
        _, rec = catalogue.region_record([Ion(name)], cable)
        assert rec[slot] == pytest.approx(want, rel=1e-6), name
    # overrides of Ci / Co / temp enter the formula
    _, rec = catalogue.region_record([Ion("SodiumInitNernst", Ci=20.0, temp=O._c2k(20.0))], cable)
    assert rec[_abi.BC_P_ENA] == pytest.approx(1e3 * O.GAS_R * O._c2k(20.0) / O.FARADAY * np.log(7.0), rel=1e-12)
    with pytest.raises(ValueError, match="Nernst"):
        catalogue.region_record([Ion("PotassiumInitNernst", Ci=0.0)], cable)


def _cell(precision="f64"):
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    c = Cell(Morphology.from_root(soma, name="soma"), cv_policy=CVPerBranch(), precision=precision)
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.1, E=-65.0),
            Channel("Na_Ba2002", g_max=100.0), Channel("KDR_Ba2002", g_max=30.0), Channel("CaL_IS2008", g_max=1.0),
            Ion("SodiumInitNernst", Ci=12.0), Ion("PotassiumInitNernst", Ci=140.0, Co=5.0),
            Ion("CalciumInitNernst", Ci=1e-4))
    c.place(RootLocation(0.5), CurrentClamp(delay=1.0, durations=10.0, amplitudes=0.5), StateProbe(name="v"))
    return c


def test_oracle_takes_the_stored_nernst_potentials():
    oc = O.OracleCell(_cell())
    _, rec = catalogue.region_record([Ion("SodiumInitNernst", Ci=12.0)], CableProperty())
    assert oc.E_na[oc.cv_mid[0]] == pytest.approx(rec[_abi.BC_P_ENA], rel=1e-14)
    _, rec = catalogue.region_record([Ion("PotassiumInitNernst", Ci=140.0, Co=5.0)], CableProperty())
    assert oc.E_k[oc.cv_mid[0]] == pytest.approx(rec[_abi.BC_P_EK], rel=1e-14)


@pytest.mark.gpu
def test_init_nernst_cell_matches_oracle(native_lib, cuda_device):
    from braincell_gb300.runtime import Plan

    n = 600
    p = Plan(_cell().batch(), precision="f64", record_every=1, device=cuda_device)
    p.run(n, 0.025)
    gpu = p.traces()[0]
    sp = p.spikes()[0]
    p.close()
    ref, osp = O.OracleCell(_cell()).run(0.025, n)
    assert len(sp) == len(osp[0][0]) >= 1
    np.testing.assert_allclose(np.asarray(sp), np.asarray(osp[0][0]), rtol=0, atol=1e-9)
    # 1e-8 mV, or a time shift within the spike-time bar on the upstrokes
    slope = np.abs(np.gradient(ref[0, 0], 0.025))
    assert gpu.shape == ref[0, 0].shape
    assert (np.abs(gpu - ref[0, 0]) <= 1e-8 + 1e-9 * slope).all()
