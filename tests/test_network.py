"""Network lowering (CPU) and GPU event delivery against the float64 network oracle."""

import numpy as np
import pytest

from braincell_gb300 import Branch, Cell, Morphology
from braincell_gb300.mech import AllRegion, CableProperty, Channel, CurrentClamp, CVPerBranch, ExpSyn, RootLocation, StateProbe
from braincell_gb300.network import Connection, Network, Population
from braincell_gb300.runtime import Plan


def neuron(pop=1, clamp=0.0, precision="f64", n_dend=0):
    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    m = Morphology.from_root(soma, name="soma")
    for k in range(n_dend):
        m.attach(parent="soma", child_branch=Branch.from_lengths(lengths=[80.0], radii=[1.0, 0.6], type="basal_dendrite"))
    c = Cell(m, cv_policy=CVPerBranch(), pop_size=pop, precision=precision)
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.3, E=-70.0),
            Channel("Na_Ba2002", g_max=120.0), Channel("KDR_Ba2002", g_max=36.0))
    if clamp:
        c.place(RootLocation(0.5), CurrentClamp(delay=1.0, durations=40.0, amplitudes=clamp))
    c.place(RootLocation(0.5), ExpSyn(tau=2.0, e=0.0, weight=0.05, name="ampa"))
    c.place(RootLocation(0.5), StateProbe())
    return c


CONNS = [
    Connection("drv", "exc", [0, 0, 0], [0, 1, 2], synapse="ampa", weight=[0.2, 0.25, 0.3], delay=[1.0, 0.5, 2.0]),
    Connection("exc", "exc", [0], [1], synapse=0, delay=0.3),
    Connection("exc", "exc", [2], [0], synapse="ampa", weight=0.02, delay=0.0),
]


def test_network_batch_lowering():
    net = Network([Population("drv", neuron(1, clamp=1.5)), Population("exc", neuron(3))], CONNS)
    b = net.batch()
    assert b.n_cells == 4 and b.syn_cell.size == 4
    np.testing.assert_array_equal(b.conn_pre, [0, 0, 0, 1, 3])
    np.testing.assert_array_equal(b.conn_post, [1, 2, 3, 2, 1])
    np.testing.assert_allclose(b.conn_weight, [0.2, 0.25, 0.3, 0.05, 0.02])
    np.testing.assert_allclose(b.conn_delay, [1.0, 0.5, 2.0, 0.3, 0.0])
    p = Plan(b, dry_run=True)
    assert p.info["n_cells"] == 4
    # select keeps synapses and the connections among the kept cells
    sub = b.select([0, 1])
    np.testing.assert_array_equal(sub.conn_pre, [0])
    np.testing.assert_array_equal(sub.conn_post, [1])


def test_network_errors():
    with pytest.raises(KeyError):
        Network([Population("a", neuron(1))], [Connection("a", "b", [0], [0])]).batch()
    with pytest.raises(ValueError, match="post_index"):
        Network([Population("a", neuron(2))], [Connection("a", "a", [0], [5])]).batch()
    with pytest.raises(ValueError, match="synapses named"):
        Network([Population("a", neuron(2))], [Connection("a", "a", [0], [1], synapse="nmda")]).batch()
    b = Network([Population("a", neuron(2))], [Connection("a", "a", [0], [1], delay=0.1)]).batch()
    b.syn_x = np.array([1.0, 1.0])
    from braincell_gb300 import _abi
    with pytest.raises(_abi.BCError, match="inside a CV"):
        Plan(b, dry_run=True)


def _oracle_run(n_steps, dt=0.025, n_dend=0):
    from oracle.network import OracleNetwork
    from oracle.staggered import OracleCell

    cells = [OracleCell(neuron(1, clamp=1.5, n_dend=n_dend))] + [OracleCell(neuron(1, n_dend=n_dend)) for _ in range(3)]
    contacts = [(0, 1, 0, 0.2, 1.0), (0, 2, 0, 0.25, 0.5), (0, 3, 0, 0.3, 2.0), (1, 2, 0, 0.05, 0.3), (3, 1, 0, 0.02, 0.0)]
    return OracleNetwork(cells, contacts).run(dt, n_steps)


@pytest.mark.gpu
@pytest.mark.parametrize("steps_per_launch", [1000, 7])
def test_network_matches_oracle_f64(native_lib, cuda_device, steps_per_launch):
    n = 1200
    net = Network([Population("drv", neuron(1, clamp=1.5, n_dend=2)), Population("exc", neuron(3, n_dend=2))], CONNS)
    net.init_state(record_every=1, steps_per_launch=steps_per_launch)
    res = net.run(dt=0.025, duration=n * 0.025)
    spikes, traces = _oracle_run(n, n_dend=2)
    gpu_traces = net._plan.traces()
    np.testing.assert_allclose(gpu_traces, traces, atol=1e-8)
    cells, steps = net.spike_records()
    assert sorted(zip(cells.tolist(), steps.tolist())) == sorted(spikes)
    # every exc member received events and fired at least once
    assert set(res.spikes["exc"][0].tolist()) == {0, 1, 2}
    assert np.all(net.synapse_g() >= 0.0)


@pytest.mark.gpu
def test_network_f32_spike_steps():
    n = 1200
    net = Network([Population("drv", neuron(1, clamp=1.5, precision="f32")), Population("exc", neuron(3, precision="f32"))],
                  CONNS)
    net.init_state(record_every=1)
    net.run(dt=0.025, duration=n * 0.025)
    spikes, _ = _oracle_run(n)
    cells, steps = net.spike_records()
    got = sorted(zip(cells.tolist(), steps.tolist()))
    want = sorted(spikes)
    assert len(got) == len(want)
    for (c1, s1), (c2, s2) in zip(got, want):
        assert c1 == c2 and abs(s1 - s2) <= 2  # 0.05 ms
