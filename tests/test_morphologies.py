"""Real reconstructed morphologies through Cell -> GPU, against the oracle.

The branch trees of five of the reference's morphologies (data/morphology: CA1,
bc, io, grc, branched_soma) were read with this package's SWC reader and stored
in tests/golden/morphologies.npz by tests/golden/make_morphology_fixtures.py.
Each is painted with the small configuration's channel mix (leak everywhere,
Na_Ba2002 / KDR_Ba2002 on soma and axon, CaL_IS2008 + HCN_HM1992 on dendrites),
discretised at most 20 um per CV, driven by a soma clamp, and run in FP64 against
the float64 oracle and in FP32 against the FP64 kernels.
"""

import os

import numpy as np
import pytest

from oracle.staggered import OracleCell

GOLD = os.path.join(os.path.dirname(__file__), "golden", "morphologies.npz")
NAMES = ("CA1", "bc", "io", "grc", "branched_soma")
TYPES = ("soma", "axon", "basal_dendrite", "apical_dendrite", "dendrite", "custom")
DT = 0.025


def _morphology(name):
    from braincell_gb300.morph import Branch, Morphology

    z = np.load(GOLD)
    par, px, cx = z[f"{name}__parent"], z[f"{name}__parent_x"], z[f"{name}__child_x"]
    typ, off = z[f"{name}__type"], z[f"{name}__seg_offsets"]
    L, rp, rd = z[f"{name}__lengths"], z[f"{name}__r_prox"], z[f"{name}__r_dist"]

    def branch(b):
        s = slice(int(off[b]), int(off[b + 1]))
        return Branch(lengths=L[s].copy(), radii_proximal=rp[s].copy(), radii_distal=rd[s].copy(), type=TYPES[typ[b]])

    m = Morphology.from_root(branch(0), name="root")
    for b in range(1, par.size):
        m.attach(parent=int(par[b]), child_branch=branch(b), child_name=f"b{b}", parent_x=float(px[b]),
                 child_x=float(cx[b]))
    return m


def _cell(name, precision="f64"):
    from braincell_gb300 import Cell
    from braincell_gb300.mech import (AllRegion, CableProperty, Channel, CurrentClamp, MaxCVLen, RootLocation,
                                      StateProbe, branch_in)

    c = Cell(_morphology(name), cv_policy=MaxCVLen(20.0), precision=precision)
    c.paint(AllRegion(), CableProperty(), Channel("IL", g_max=0.3, E=-70.0))
    c.paint(branch_in("type", ("soma", "axon")), Channel("Na_Ba2002", g_max=120.0), Channel("KDR_Ba2002", g_max=36.0))
    c.paint(branch_in("type", ("basal_dendrite", "apical_dendrite", "dendrite", "custom")),
            Channel("CaL_IS2008", g_max=2.0), Channel("HCN_HM1992", g_max=0.01, E=-43.0))
    c.place(RootLocation(0.5), CurrentClamp(delay=1.0, durations=8.0, amplitudes=1.0))
    c.place(RootLocation(0.5), StateProbe())
    return c


def _upstroke(trace):
    """Start of the first spike's upstroke (trace length if no spike)."""
    hit = np.nonzero((trace[1:] >= 0.0) & (trace[:-1] < 0.0))[0]
    if not hit.size:
        return trace.size
    calm = np.nonzero(np.diff(trace[:hit[0] + 1]) / DT <= 10.0)[0]
    return int(calm[-1]) + 1 if calm.size else 0


@pytest.mark.parametrize("name", NAMES)
def test_fixture_rebuilds_a_lowerable_morphology(name):
    z = np.load(GOLD)
    m = _morphology(name)
    assert len(m.branches) == z[f"{name}__parent"].size
    got = np.concatenate([b.lengths for b in m.branches])
    np.testing.assert_array_equal(got, z[f"{name}__lengths"])  # no segment added or dropped
    oc = OracleCell(_cell(name))
    assert oc.n_cv >= len(m.branches)
    if name == "CA1":
        assert len(m.branches) == 681 and abs(sum(b.length for b in m.branches) - 16095.0) < 1.0


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_real_morphology_f64_matches_oracle(native_lib, cuda_device, name):
    from braincell_gb300.batch import lower_cell
    from braincell_gb300.runtime import Plan

    n = 400
    p = Plan(lower_cell(_cell(name)), precision="f64", record_every=1, device=cuda_device)
    p.run(n, DT)
    tr = p.traces()[0]
    oc = OracleCell(_cell(name))
    otr, osp = oc.run(DT, n)
    assert np.abs(otr[0, 0] - tr).max() <= 1e-8
    assert np.abs(oc.V[0] - p.state("V")).max() <= 1e-8
    sp = p.spikes()[0]
    assert len(sp) == len(osp[0][0])
    if len(sp):
        assert np.abs(np.asarray(sp) - np.asarray(osp[0][0])).max() <= 1e-9
    p.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_real_morphology_f32_against_f64(native_lib, cuda_device, name):
    from braincell_gb300.batch import lower_cell
    from braincell_gb300.runtime import Plan

    out = {}
    for prec in ("f32", "f64"):
        p = Plan(lower_cell(_cell(name, prec)), precision=prec, record_every=1, device=cuda_device)
        p.run(800, DT)
        out[prec] = (p.traces()[0], p.spikes()[0])
        p.close()
    (t32, s32), (t64, s64) = out["f32"], out["f64"]
    u = _upstroke(t64)
    assert np.abs(t32[:u] - t64[:u]).max() <= 1e-3
    assert len(s32) == len(s64)
    if len(s64):
        assert np.abs(np.asarray(s32) - np.asarray(s64)).max() <= 0.05
