"""The float64 network oracle: delay quantisation, arrival timing, ExpSyn current."""

import numpy as np
import pytest

from braincell_gb300 import Branch, Cell, Morphology
from braincell_gb300.mech import AllRegion, CableProperty, Channel, CurrentClamp, CVPerBranch, ExpSyn, RootLocation, StateProbe
from oracle.network import OracleNetwork, delay_steps
from oracle.staggered import OracleCell


def test_delay_quantisation_is_ceil_with_exact_multiples_kept():
    np.testing.assert_array_equal(delay_steps([0.0, 0.025, 0.026, 1.0, 0.3], 0.025), [0, 1, 2, 40, 12])
    with pytest.raises(ValueError):
        delay_steps([-0.1], 0.025)


def soma_cell(clamp=0.0, syn=False):
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    c = Cell(Morphology.from_root(soma, name="soma"), cv_policy=CVPerBranch(), precision="f64")
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.3, E=-70.0),
            Channel("Na_Ba2002", g_max=120.0), Channel("KDR_Ba2002", g_max=36.0))
    if clamp:
        c.place(RootLocation(0.5), CurrentClamp(delay=1.0, durations=30.0, amplitudes=clamp))
    if syn:
        c.place(RootLocation(0.5), ExpSyn(tau=2.0, e=0.0))
    c.place(RootLocation(0.5), StateProbe())
    return c


def test_spike_reaches_the_target_synapse_after_the_delay():
    pre, post = OracleCell(soma_cell(clamp=1.5)), OracleCell(soma_cell(syn=True))
    spikes, traces = OracleNetwork([pre, post], [(0, 1, 0, 0.05, 1.0)]).run(0.025, 400)
    _, alone = OracleNetwork([OracleCell(soma_cell(clamp=1.5)), OracleCell(soma_cell(syn=True))], []).run(0.025, 400)
    s0 = min(s for c, s in spikes if c == 0)
    # the postsynaptic cell is untouched until the arrival step s0 + 40 (1 ms), then depolarised
    np.testing.assert_array_equal(traces[1, : s0 + 40], alone[1, : s0 + 40])
    assert traces[1, s0 + 40] != alone[1, s0 + 40]
    assert traces[1, s0 + 45] > alone[1, s0 + 45] + 0.5


def test_zero_delay_means_next_step():
    pre, post = OracleCell(soma_cell(clamp=1.5)), OracleCell(soma_cell(syn=True))
    net = OracleNetwork([pre, post], [(0, 1, 0, 0.05, 0.0)])
    net.run(0.025, 1)
    s = 1
    while not pre.population_spike()[0]:
        net.run(0.025, 1)
        s += 1
    g_before = post.syn_g.copy()
    net.run(0.025, 1)  # arrival at s: applied at the start of this step, then one dt of decay
    assert np.all(g_before == 0.0) and post.syn_g[0, 0] == pytest.approx(0.05 * np.exp(-0.025 / 2.0), rel=1e-12)
