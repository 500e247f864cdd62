"""Subtree-surrogate ports in the step kernel against the float64 oracle (closed loop).

A small cell keeps three leaf branches whose subtrees a GRU stands in for; the
oracle (``OracleCell.set_ports``) runs the same GRU in float64 with the kernels'
BF16 rounding points and injects the same port currents, so the whole loop --
voltage in, GRU step, implicit port conductance, current out -- is compared.
"""

import numpy as np
import pytest

from braincell_gb300 import workloads as W
from braincell_gb300.runtime import Plan
from oracle import gru as G
from oracle.staggered import OracleCell

pytestmark = pytest.mark.gpu

DT = 0.025
V_SCALE, Y_SCALE = 10.0, 5.0
WIDE = (V_SCALE, Y_SCALE, -1e4, 1e4, 1e9)


def _desc(amp=0.25):
    parent = [-1, 0, 1, 1, 0]
    length = [20.0, 100.0, 80.0, 60.0, 120.0]
    ncv = [1, 6, 4, 3, 5]
    rp, rd = W._finish_tree(parent, length, ncv)
    leak = ("IL", {"g_max": 0.3, "E": -70.0})
    return W.CellDesc(parent=parent, length=length, r_prox=rp, r_dist=rd, ncv=ncv,
                      types=["soma"] + ["dendrite"] * 4,
                      channels_soma=[leak, ("Na_Ba2002", {"g_max": 120.0}), ("KDR_Ba2002", {"g_max": 36.0})],
                      channels_dend=[leak, ("CaL_IS2008", {"g_max": 2.0}), ("HCN_HM1992", {"g_max": 0.01, "E": -43.0}),
                                     ("K_Leak", {"g_max": 0.005})],
                      pulses=[(0, 0.5, 2.0, 1e9, amp)])


PORTS = [
    dict(branch=2, g=0.004, e=-70.0, feat=(0.3, -0.2), stim=[]),
    dict(branch=3, g=0.006, e=-68.0, feat=(-0.5, 0.1), stim=[(5.0, 8.0, 0.05), (10.0, 11.0, 0.1)]),
    dict(branch=4, g=0.003, e=-72.0, feat=(0.0, 0.7), stim=[(3.0, 4.0, 0.08)]),
]


def _with_ports(batch, ports, cell=0):
    batch.port_cell = np.full(len(ports), cell, np.int32)
    batch.port_branch = np.array([p["branch"] for p in ports], np.int32)
    batch.port_g = np.array([p["g"] for p in ports])
    batch.port_e = np.array([p["e"] for p in ports])
    batch.port_feat = np.array([p["feat"] for p in ports], float)
    pp = [(k, *s) for k, p in enumerate(ports) for s in p["stim"]]
    batch.port_pulse_port = np.array([q[0] for q in pp], np.int32)
    batch.port_pulse_t_on = np.array([q[1] for q in pp], float)
    batch.port_pulse_t_off = np.array([q[2] for q in pp], float)
    batch.port_pulse_amp = np.array([q[3] for q in pp], float)
    return batch


def _run_pair(precision, n_steps, theta, amp=0.25, **kw):
    d = _desc(amp)
    b = _with_ports(W.descs_to_batch([d]), PORTS)
    p = Plan(b, precision=precision, record_every=1, **kw)
    p.set_surrogate(theta, WIDE)
    p.run(n_steps, DT)
    oc = OracleCell(W.desc_to_cell(d))
    oc.set_ports(PORTS, theta.astype(np.float64), V_SCALE, Y_SCALE)
    tr, sp = oc.run(DT, n_steps)
    return p, p.traces()[0], tr[0, 0], p.spikes()[0], np.asarray(sp[0][0])


def test_ports_closed_loop_f64_matches_oracle(native_lib, cuda_device):
    theta = G.init_params(11, scale=1.5).astype(np.float32)
    p, gpu, ora, gsp, osp = _run_pair("f64", 1200, theta, amp=0.05)
    # the GRU itself is FP32/BF16 in both runs: agreement is to its rounding, far below 1e-3 mV
    assert np.abs(gpu - ora).max() < 1e-4, np.abs(gpu - ora).max()
    assert np.abs(gpu[-1] - gpu[0]) > 1e-3  # the cell moved
    assert len(gsp) == len(osp)


def test_ports_closed_loop_f32_spiking(native_lib, cuda_device):
    theta = G.init_params(12, scale=1.0).astype(np.float32)
    p, gpu, ora, gsp, osp = _run_pair("f32", 2400, theta, amp=0.4)
    assert len(osp) >= 1
    assert len(gsp) == len(osp)
    assert np.abs(gsp - osp).max() < 0.05
    # before the first spike's upstroke (dV/dt above 10 mV/ms), to 1e-3 mV
    first = int(np.nonzero(np.diff(ora) / DT > 10.0)[0][0]) + 1
    assert np.abs(gpu[:first] - ora[:first]).max() < 1e-3


def test_ports_change_the_cell(native_lib, cuda_device):
    """A port with a GRU that outputs a constant +y feeds current: the soma depolarises."""
    theta = np.zeros(G.NPARAM, np.float32)
    d = _desc(0.0)
    base = Plan(W.descs_to_batch([d]), precision="f64", record_every=1)
    base.run(400, DT)
    theta[G.OFF_BO] = 4.0  # y = 4 -> I = g (e + 20 mV - V_end)
    b = _with_ports(W.descs_to_batch([d]), PORTS)
    p = Plan(b, precision="f64", record_every=1)
    p.set_surrogate(theta, WIDE)
    p.run(400, DT)
    assert p.traces()[0][-1] > base.traces()[0][-1] + 0.05


def test_envelope_flags_and_reset(native_lib, cuda_device):
    theta = G.init_params(13).astype(np.float32)
    d = _desc(0.3)
    b = _with_ports(W.descs_to_batch([d, d]), PORTS, cell=1)  # ports on the second cell only
    p = Plan(b, precision="f32", record_every=0)
    # an envelope the spiking cell leaves (|dV/dt| bound of 1 mV/ms)
    p.set_surrogate(theta, (V_SCALE, Y_SCALE, -50.0, 50.0, 1.0))
    p.run(1200, DT)
    np.testing.assert_array_equal(p.surrogate_flags(), [0, 1])
    p.reset()
    np.testing.assert_array_equal(p.surrogate_flags(), [0, 0])
    p.set_surrogate(theta, WIDE)
    p.run(200, DT)
    np.testing.assert_array_equal(p.surrogate_flags(), [0, 0])


def test_ports_need_a_gru(native_lib, cuda_device):
    from braincell_gb300._abi import BCError

    b = _with_ports(W.descs_to_batch([_desc()]), PORTS)
    p = Plan(b, precision="f32")
    with pytest.raises(BCError, match="bc_surrogate_set"):
        p.run(10, DT)


def test_ports_in_graph_and_big_tile_class(native_lib, cuda_device):
    """Same ports through a CUDA graph and through the one-cell tile class: same trace."""
    theta = G.init_params(14, scale=1.5).astype(np.float32)
    d = _desc(0.3)
    out = []
    for kw in (dict(), dict(use_graph=True), dict(tile_nodes=16, threads_big=256)):
        b = _with_ports(W.descs_to_batch([d]), PORTS)
        p = Plan(b, precision="f64", record_every=1, steps_per_launch=150, **kw)
        p.set_surrogate(theta, WIDE)
        p.run(700, DT)
        out.append(p.traces()[0])
    np.testing.assert_allclose(out[1], out[0], rtol=0, atol=1e-9)
    np.testing.assert_allclose(out[2], out[0], rtol=0, atol=1e-7)


def _soma_rms(traces, ref):
    return np.sqrt(np.mean((traces - ref) ** 2, axis=1))


def test_packaged_model_gains_over_the_method_without_it(native_lib, cuda_device):
    """On held-out cells of the 10k workload (seed 1, never trained on), the trained
    GRU ports track the FP64 plain solve's soma voltage better than the same ports
    with the network switched off (only the passive load), and far better than
    cutting the subtrees off."""
    from dataclasses import replace

    from braincell_gb300 import surrogate as S

    m = S.load_model(S.PACKAGED_MODEL)
    descs = W.uneven(40, seed=1)
    n = 4000
    full = [replace(d, probes=[(0, 0.5)]) for d in descs]
    ref = Plan(W.descs_to_batch(full), precision="f64", record_every=1)
    ref.run(n, DT)
    tr64 = ref.traces()
    gru = S.run_surrogate(descs, m, n, record_every=1, fallback=False)
    lin = S.run_surrogate(descs, None, n, record_every=1, fallback=False)
    red = [replace(S.reduce_desc(d)[0], probes=[(0, 0.5)]) for d in descs]
    cut = Plan(W.descs_to_batch(red), precision="f32", record_every=1)
    cut.run(n, DT)
    e_gru = np.median(_soma_rms(gru.traces, tr64))
    e_lin = np.median(_soma_rms(lin.traces, tr64))
    e_cut = np.median(_soma_rms(cut.traces(), tr64))
    assert gru.n_ports > 0 and gru.reduced_cv < 0.5 * gru.full_cv
    assert e_gru < 0.5 * e_lin, (e_gru, e_lin)
    assert e_lin < e_cut
    assert e_gru < 1.0  # mV, the somatic bar


def test_fallback_replaces_flagged_cells_with_the_full_solve(native_lib, cuda_device):
    from dataclasses import replace

    from braincell_gb300 import surrogate as S

    m = S.load_model(S.PACKAGED_MODEL)
    tight = replace(m, env_dvdt=0.5)  # most spiking cells leave this envelope
    descs = W.uneven(12, seed=1)
    r = S.run_surrogate(descs, tight, 2000, record_every=1, fallback=True)
    assert 0 < r.fallback_cells.size <= len(descs)
    fd = [replace(descs[i], probes=[(0, 0.5)]) for i in r.fallback_cells]
    full = Plan(W.descs_to_batch(fd), precision="f32", record_every=1, **S.fallback_plan_options(fd, threads=512))
    full.run(2000, DT)
    np.testing.assert_allclose(r.traces[r.fallback_cells], full.traces(), rtol=0, atol=1e-9)


def test_mixed_population_full_cells_match_the_plain_solve(native_lib, cuda_device):
    # a mixed population (some cells keep their full morphology from t = 0, the rest
    # run with ports and fallback): the full cells are exactly the plain solve's,
    # the port cells exactly those of an unmixed surrogate run
    from dataclasses import replace

    from braincell_gb300 import surrogate as S

    m = S.load_model(S.PACKAGED_MODEL)
    descs = W.uneven(20, seed=4)
    full_idx = np.array([1, 4, 5, 11, 17])
    r = S.run_surrogate(descs, m, 2000, record_every=1, fallback=True, full_cells=full_idx)
    assert np.array_equal(r.full_cells, full_idx) and not np.isin(r.fallback_cells, full_idx).any()
    fd = [replace(descs[i], probes=[(0, 0.5)]) for i in full_idx]
    ref = Plan(W.descs_to_batch(fd), precision="f32", record_every=1, **S.fallback_plan_options(fd, threads=512))
    ref.run(2000, DT)
    np.testing.assert_allclose(r.traces[full_idx], ref.traces(), rtol=0, atol=1e-9)
    # the port cells as in an unmixed run (tile packing changes the order of the GRU's
    # per-port partial sums, so agreement is to rounding, judged on the spikes)
    rest = np.setdiff1d(np.arange(len(descs)), full_idx)
    alone = S.run_surrogate([descs[i] for i in rest], m, 2000, record_every=1, fallback=True)
    for j, i in enumerate(rest):
        assert len(r.spikes[i]) == len(alone.spikes[j])
        if len(alone.spikes[j]):
            assert np.abs(np.asarray(r.spikes[i]) - np.asarray(alone.spikes[j])).max() <= 0.05
    assert np.array_equal(np.sort(r.fallback_cells), np.sort(rest[alone.fallback_cells]))


def test_training_pipeline_learns(native_lib, cuda_device):
    """Trajectories from the plain solver, GPU training with the library's kernels:
    a short run lowers the held-out loss."""
    from braincell_gb300 import surrogate as S

    m = S.train_surrogate(40, n_steps=1600, epochs=20, batch=64, window=200, lr=3e-3, val_frac=0.2, seed=5)
    assert m.info["n_traj"] > 20
    assert m.info["val_mse_after"] < 0.6 * m.info["val_mse_before"], m.info
    assert np.isfinite(m.theta).all()
