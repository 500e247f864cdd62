"""The Cell front end dispatches to the registered GB300 integrator and keeps the
reference's step-level behaviours (quad/_staggered_test.py, _multi_compartment/cell_test.py)."""

import json
import os

import numpy as np
import pytest

from braincell_gb300 import Branch, Cell, Morphology, environ
from braincell_gb300 import workloads as W
from braincell_gb300.mech import CurrentClamp, CVPerBranch, RootLocation, StateProbe
from oracle.staggered import OracleCell

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_known_answers.json")))


@pytest.fixture(scope="module", autouse=True)
def _lib(native_lib, cuda_device):
    return native_lib


def _soma_cell(case, pop=1, precision="f64"):
    soma = Branch.from_lengths(lengths=[case["soma_length"]], radii=[case["soma_radius"]] * 2, type="soma")
    cell = Cell(Morphology.from_root(soma, name="soma"), pop_size=pop, cv_policy=CVPerBranch(),
                V_init=case.get("V_init"), precision=precision)
    cell.place(RootLocation(case["clamp_x"]),
               CurrentClamp(delay=case["delay"], durations=case["durations"], amplitudes=case["amplitudes"]))
    return cell


@pytest.mark.parametrize("case", GOLD["step_behaviour"][:2], ids=["endpoint", "multistep"])
def test_clamp_raises_voltage(case):
    cell = _soma_cell(case)
    cell.init_state()
    before = cell.V[0, 0]
    with environ.context(dt=case["dt"]):
        cell.update()
    assert cell.V[0, 0] > before
    oc = OracleCell(_soma_cell(case))
    oc.step(case["dt"], 0.0)
    assert abs(cell.V[0, 0] - oc.V[0, 0]) < 1e-9


def test_population_widening_is_neutral():
    case = GOLD["step_behaviour"][2]
    single, pop = _soma_cell(case), _soma_cell(case, pop=case["pop"])
    single.init_state()
    pop.init_state()
    with environ.context(dt=case["dt"]):
        single.update()
        pop.update()
    for m in range(case["pop"]):
        np.testing.assert_allclose(pop.V[m], single.V[0], rtol=case["rtol"], atol=case["atol"])


def test_cell_run_matches_update_loop_and_oracle():
    d = W._small_desc(0)
    d.pulses = [(0, 0.5, 1.0, 4.0, 0.5)]
    a = W.desc_to_cell(d, pop_size=2, precision="f64")
    res = a.run(dt=0.025, duration=5.0)
    assert res.time.shape == (200,) and set(res.traces) == {"probe_0"}
    tr = res.traces["probe_0"]
    assert tr.shape == (2, 200)
    b = W.desc_to_cell(d, precision="f64")
    b.init_state()
    with environ.context(dt=0.025):
        loop = []
        for _ in range(200):
            b.update()
            loop.append(b.V[0, 0])
    np.testing.assert_allclose(tr[0], np.asarray(loop), atol=1e-12)
    oc = OracleCell(W.desc_to_cell(d))
    otr, _ = oc.run(0.025, 200)
    np.testing.assert_allclose(tr[0], otr[0, 0], atol=1e-8)


def test_cell_declaration_errors():
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    cell = Cell(Morphology.from_root(soma))
    with pytest.raises(ValueError, match="probe"):
        cell.run(dt=0.025, duration=1.0)
    cell.place(RootLocation(0.5), StateProbe())
    cell.init_state()
    with pytest.raises(RuntimeError):
        cell.paint(RootLocation(0.5), CurrentClamp())
    with pytest.raises(ValueError, match="dt"):
        cell.update()
    with pytest.raises(ValueError):
        Cell(Morphology.from_root(soma), solver="no_such_solver")


def _swc_cell(precision):
    from braincell_gb300.mech import AllRegion, CableProperty, Channel, branch_in
    from braincell_gb300.swc import read_swc

    m = read_swc(os.path.join(os.path.dirname(__file__), "golden", "pyramid_small.swc"))
    cell = Cell(m, cv_policy=CVPerBranch(), pop_size=1, precision=precision)
    cell.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.3, E=-70.0))
    cell.paint(branch_in("type", "soma"), Channel("Na_Ba2002", g_max=120.0), Channel("KDR_Ba2002", g_max=36.0))
    cell.paint(branch_in("type", ("basal_dendrite", "apical_dendrite")), Channel("CaL_IS2008", g_max=2.0))
    cell.place(RootLocation(0.5), CurrentClamp(delay=1.0, durations=8.0, amplitudes=0.3))
    cell.place(RootLocation(0.5), StateProbe())
    return cell


def test_swc_morphology_matches_oracle():
    # a cell read from SWC (3-point soma, basal and apical trees, axon) through the
    # Cell front end: FP64 GPU run vs the float64 oracle
    cell = _swc_cell("f64")
    res = cell.run(dt=0.025, duration=10.0)
    tr = res.traces["probe_0"][0]
    oc = OracleCell(_swc_cell("f64"))
    otr, _ = oc.run(0.025, 400)
    np.testing.assert_allclose(tr, otr[0, 0], atol=1e-8)


def test_per_cv_spike_state_matches_oracle():
    # Cell.spike is the per-CV get_spike(last_V, V) of the last step (cell.py:2384-2386):
    # after every update(), and after a fused run that ends on a crossing step
    from braincell_gb300.runtime import Plan

    d = W._small_desc(0)
    d.pulses = [(0, 0.5, 1.0, 30.0, 1.2)]
    cell = W.desc_to_cell(d, precision="f64")
    cell.init_state()
    assert cell.spike.sum() == 0
    oc = OracleCell(W.desc_to_cell(d))
    crossing_steps = []
    with environ.context(dt=0.025):
        for k in range(800):
            s = cell.update()
            o = oc.step(0.025)
            np.testing.assert_array_equal(s[0], o[0], err_msg=f"step {k}")
            if o.sum():
                crossing_steps.append(k + 1)
    assert len(crossing_steps) >= 2
    n = crossing_steps[1]
    p = Plan(W.descs_to_batch([d]), precision="f64", steps_per_launch=37)
    p.run(n, 0.025)
    ref = OracleCell(W.desc_to_cell(d))
    for _ in range(n):
        spk = ref.step(0.025)
    assert spk.sum() >= 1
    np.testing.assert_array_equal(p.spike_state(0.0), spk[0])
    # an upload starts a fresh history: no crossing until the next step
    p.set_state("V", p.state("V"))
    assert p.spike_state(0.0).sum() == 0
    p.reset()
    assert p.spike_state(0.0).sum() == 0
