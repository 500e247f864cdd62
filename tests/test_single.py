"""SingleCompartment on the GB300 step (``_single_compartment/base.py:252-278``).

CPU: the single-compartment oracle and the node-tree oracle agree on a one-CV cell
(two independent routes to the same staggered step).  GPU: ``update(I_ext)``
through the registered solver matches the oracle step for step, spikes included,
under a time-varying input.
"""

import math

import numpy as np
import pytest

from braincell_gb300 import SingleCompartment, environ
from braincell_gb300.mech import Channel, Ion
from oracle.single import OracleSingleCompartment
from oracle.staggered import OracleCell

DT = 0.025
LENGTH, RADIUS = 10.0, 5.0


def _hh():
    return dict(na=Channel("Na_HH1952"), k=Channel("K_HH1952"), leak=Channel("IL", g_max=0.3, E=-54.4))


def _calcium():
    return dict(na=Channel("Na_Ba2002", g_max=100.0), kdr=Channel("KDR_Ba2002", g_max=30.0),
                cat=Channel("CaT_HM1992", g_max=1.0), ahp=Channel("AHP_De1994", g_max=0.5),
                hcn=Channel("HCN_HM1992", g_max=0.05, E=-43.0), leak=Channel("IL", g_max=0.1, E=-70.0),
                ca=Ion("CalciumDetailed", C_rest=5e-5, tau=10.0, d=0.5, Ci_initializer=5e-5))


def _drive(k, n):
    """A time-varying input density (nA/cm^2): steps and a ramp, different per neuron."""
    t = k * DT
    base = np.linspace(5e3, 2.5e4, n)
    return np.where((t > 2.0) & (t < 30.0), base * (1.0 + 0.5 * math.sin(t / 3.0)), 0.0)


def _tree_cell(decls, i_na):
    from braincell_gb300 import Branch, Cell, Morphology
    from braincell_gb300.mech import AllRegion, CableProperty, CurrentClamp, CVPerBranch, RootLocation

    soma = Branch.from_lengths(lengths=[LENGTH], radii=[RADIUS, RADIUS], type="soma")
    c = Cell(Morphology.from_root(soma, name="soma"), cv_policy=CVPerBranch())
    c.paint(AllRegion(), CableProperty(resting_potential=-65.0), *decls)
    c.place(RootLocation(0.5), CurrentClamp(delay=0.0, durations=1e9, amplitudes=i_na))
    return c


@pytest.mark.parametrize("mix", [_hh, _calcium], ids=["hh", "calcium"])
def test_single_oracle_matches_tree_oracle(mix):
    decls = list(mix().values())
    dens = 1.5e4  # nA/cm^2
    area_cm2 = 2.0 * math.pi * RADIUS * LENGTH * 1e-8
    tree = OracleCell(_tree_cell(decls, dens * area_cm2))
    single = OracleSingleCompartment(1, decls, V_init=-65.0)
    spikes = 0
    for _ in range(1200):
        tree.step(DT)
        spikes += int(single.update(DT, dens)[0])
        assert abs(tree.V[0, 0] - single.V[0]) <= 1e-9
    assert spikes >= 2


def test_single_compartment_declarations():
    with pytest.raises(TypeError):
        SingleCompartment(3, na="Na_HH1952")
    with pytest.raises(ValueError):
        SingleCompartment(0, **_hh())
    sc = SingleCompartment((2, 3), **_hh())
    assert sc.varshape == (2, 3) and sc.n_compartment == 1
    assert sc.area == pytest.approx(2.0 * math.pi * 5.0 * 10.0)
    b = sc.batch(np.full(6, -65.0))
    assert b.n_cells == 6 and int(b.branch_ncv.sum()) == 6 and b.pulse_cell.size == 6


@pytest.mark.gpu
@pytest.mark.parametrize("mix", [_hh, _calcium], ids=["hh", "calcium"])
@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("lanes", [0, 3], ids=["tiles", "lanes"])
def test_single_compartment_update_matches_oracle(native_lib, cuda_device, mix, precision, lanes):
    # lanes = 3: every neuron (a 3-node tree) runs one per thread on the lane kernel;
    # the HH mix runs its out-of-line channels there
    n = 8
    v0 = np.linspace(-70.0, -60.0, n)
    sc = SingleCompartment(n, length=LENGTH, radius=RADIUS, V_initializer=v0,
                           solver_options=dict(precision=precision, device=cuda_device, lane_cell_nodes=lanes),
                           **mix())
    sc.init_state()
    assert (sc._runtime.tile_stats()[:, 4] == 3).all() == bool(lanes)
    oc = OracleSingleCompartment(n, list(mix().values()), V_init=v0)
    np.testing.assert_allclose(sc.V, oc.V, atol=1e-12 if precision == "f64" else 1e-5)
    tol = 1e-8 if precision == "f64" else None
    gpu_spk, ref_spk = [], []
    with environ.context(dt=DT):
        for k in range(1600):
            I = _drive(k, n)
            s = sc.update(I)
            r = oc.update(DT, I)
            gpu_spk.append(s.copy())
            ref_spk.append(r.copy())
            if tol is not None:
                assert np.abs(sc.V - oc.V).max() <= tol, f"step {k}"
    gpu_spk, ref_spk = np.asarray(gpu_spk), np.asarray(ref_spk)
    assert ref_spk.sum() >= n  # every neuron fires under this input
    if precision == "f64":
        np.testing.assert_array_equal(gpu_spk, ref_spk)
    else:
        # FP32: the same number of spikes per neuron, each within 2 steps (0.05 ms)
        for j in range(n):
            a, b = np.nonzero(gpu_spk[:, j])[0], np.nonzero(ref_spk[:, j])[0]
            assert a.size == b.size and np.abs(a - b).max() <= 2
    sc.close()


@pytest.mark.gpu
def test_single_compartment_reset_and_threshold(native_lib, cuda_device):
    sc = SingleCompartment(4, V_th=-20.0, V_initializer=-65.0, solver_options=dict(precision="f64"), **_hh())
    sc.init_state()
    with environ.context(dt=DT):
        fired = sum(sc.update(2.0e4).sum() for _ in range(400))
    assert fired >= 4
    v_mid = sc.V.copy()
    sc.reset_state()
    np.testing.assert_allclose(sc.V, -65.0, atol=1e-12)
    assert not np.allclose(v_mid, -65.0)
    assert sc.spike.sum() == 0
