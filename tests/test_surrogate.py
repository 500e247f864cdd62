"""Subtree surrogate on the host: reduction, passive port load, port arrays, model files."""

import numpy as np
import pytest

from braincell_gb300 import surrogate as S
from braincell_gb300 import workloads as W
from braincell_gb300.batch import native_lowering


def _descs(n=12, seed=3):
    return W.uneven(n, seed=seed)


def test_reduction_conserves_compartments_and_moves_stimuli():
    for d in _descs():
        d = W.CellDesc(**{**d.__dict__, "pulses": list(d.pulses)})
        depth = S.branch_depths(d.parent)
        deep = [b for b in range(len(d.parent)) if depth[b] >= S.CUT_DEPTH]
        if deep:
            d.pulses.append((deep[0], 0.5, 3.0, 4.0, 0.1))
        red, ports = S.reduce_desc(d)
        assert sum(red.ncv) + sum(p.n_cv for p in ports) == sum(d.ncv)
        assert max(S.branch_depths(red.parent)) < S.CUT_DEPTH
        assert sorted(b for p in ports for b in p.subtree) == deep
        # every port sits on a kept branch that had removed children
        for p in ports:
            assert red.parent[p.branch] == (-1 if d.parent[p.branch_full] < 0 else
                                            [b for b in range(len(d.parent)) if depth[b] < S.CUT_DEPTH].index(
                                                d.parent[p.branch_full]))
            assert p.g > 0 and p.c_pf > 0
        if deep:
            assert sum(len(p.stim) for p in ports) == 1
            assert len(red.pulses) == len(d.pulses) - 1


def test_attachment_conductance_matches_native_lowering(native_lib):
    d = _descs(4)[0]
    _, ports = S.reduce_desc(d)
    low = native_lowering(W.descs_to_batch([d]), 0)
    cum = np.concatenate([[0], np.cumsum(d.ncv)])
    for p in ports:
        mid = low["cv_node"][cum[p.branch_full + 1] - 1]
        end = [i for i in range(len(low["parent"])) if low["parent"][i] == mid and low["region"][i] < 0][0]
        # boundary rows carry a 1 uF dummy capacitance: alpha = g / 1e-6 F * 1e-3 -> g (uS) = alpha * 1e3
        assert S._g_att(d, p.branch_full) == pytest.approx(low["alpha"][end] * 1e3, rel=1e-12)


def test_port_input_conductance_matches_a_linear_solve(native_lib):
    """The passive subtree load against the steady state of the lowered node tree."""
    d = _descs(8)[4]
    _, ports = S.reduce_desc(d)
    g_m, _ = S._membrane(d)
    low = native_lowering(W.descs_to_batch([d]), 0)
    n = len(low["parent"])
    cap = np.full(n, 1e-6)
    cap[low["cv_node"]] = low["cv_area"] * 1e-8 * 1.0 * 1e-6
    gmem = np.zeros(n)
    gmem[low["cv_node"]] = g_m * 1e-3 * low["cv_area"] * 1e-8  # S
    cum = np.concatenate([[0], np.cumsum(d.ncv)])
    kids = [[] for _ in range(n)]
    for i in range(n):
        if low["parent"][i] >= 0:
            kids[low["parent"][i]].append(i)
    for p in ports:
        mid = low["cv_node"][cum[p.branch_full + 1] - 1]
        end = [i for i in range(n) if low["parent"][i] == mid and low["region"][i] < 0][0]
        sub, stack = [], list(kids[end])
        while stack:
            i = stack.pop()
            sub.append(i)
            stack.extend(kids[i])
        idx = {v: k for k, v in enumerate(sub)}
        A = np.zeros((len(sub), len(sub)))
        rhs = np.zeros(len(sub))
        for v in sub:
            k = idx[v]
            A[k, k] += gmem[v]
            ge = low["alpha"][v] * cap[v] * 1e3  # S
            A[k, k] += ge
            par = low["parent"][v]
            if par == end:
                rhs[k] += ge * 1.0  # V_end = 1
            else:
                A[k, idx[par]] -= ge
                A[idx[par], idx[par]] += ge
                A[idx[par], k] -= ge
        vs = np.linalg.solve(A, rhs)
        g_in = sum(low["alpha"][v] * cap[v] * 1e3 * (1.0 - vs[idx[v]]) for v in kids[end])  # S
        assert p.g == pytest.approx(g_in * 1e6, rel=1e-9)


def test_ports_to_batch_and_plan_validation(native_lib):
    from braincell_gb300._abi import BCError
    from braincell_gb300.runtime import Plan

    descs = _descs(6)
    red, ports = zip(*[S.reduce_desc(d) for d in descs])
    b = S.ports_to_batch(list(red), list(ports))
    b.validate()
    assert b.port_cell.size == sum(len(p) for p in ports)
    p = Plan(b, dry_run=True)
    assert p.info["n_tiles"] >= 1
    bad = S.ports_to_batch(list(red), list(ports))
    bad.port_g = bad.port_g.copy()
    bad.port_g[0] = 0.0
    with pytest.raises(BCError, match="port g"):
        Plan(bad, dry_run=True)
    bad = S.ports_to_batch(list(red), list(ports))
    bad.port_branch = bad.port_branch.copy()
    bad.port_branch[0] = 10_000
    with pytest.raises(BCError, match="port_branch"):
        Plan(bad, dry_run=True)
    bad = S.ports_to_batch(list(red), list(ports))
    k = int(np.nonzero(np.bincount(bad.port_cell) >= 2)[0][0])
    i0, i1 = np.nonzero(bad.port_cell == k)[0][:2]
    bad.port_branch = bad.port_branch.copy()
    bad.port_branch[i1] = bad.port_branch[i0]
    with pytest.raises(BCError, match="two ports"):
        Plan(bad, dry_run=True)
    with pytest.raises(BCError, match="at most"):
        Plan(b, dry_run=True, threads_per_tile=1024)


def test_model_file_round_trip(tmp_path):
    m = S.load_model(S.PACKAGED_MODEL)
    assert m.theta.shape == (S.NPARAM,) and np.isfinite(m.theta).all()
    assert m.env_v[0] < 0 < m.env_v[1] and m.env_dvdt > 0
    f = tmp_path / "m.npz"
    S.save_model(m, str(f))
    m2 = S.load_model(str(f))
    np.testing.assert_array_equal(m2.theta, m.theta)
    np.testing.assert_array_equal(m2.norm(), m.norm())
    assert m2.info == m.info
