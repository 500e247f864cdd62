"""Physics known answers that do not depend on any reading of the reference.

The steady state of a passive cable under a DC current is the cable equation's
closed form.  A discretised cable with h << lambda must reproduce it to O((h /
lambda)^2): these tests pin the geometry, unit scaling, axial and membrane terms,
sealed ends and branch-point current conservation of the oracle's assembly (CPU)
and of the GPU kernels through the C-ABI (``-m gpu``), against

* a sealed-end cylinder fed at x = 0:
  V(x) - E = I R_inf cosh((L - x) / lambda) / sinh(L / lambda);
* a branched tree, by Rall's recursion for the input conductance of a cylinder
  with a distal load, G_in = G_inf (G_L + G_inf t) / (G_inf + G_L t), t = tanh(L /
  lambda), children's G_in summing at a branch point, and the voltage carried
  down each branch in closed form;

with lambda = sqrt(R_m a / (2 R_a)), R_inf = 1 / G_inf = R_a lambda / (pi a^2).
"""

import math

import numpy as np
import pytest

from oracle.staggered import OracleCell

G_LEAK = 0.3       # mS/cm^2
E_LEAK = -70.0     # mV
RA = 100.0         # ohm cm
I_NA = 0.1         # nA, injected at the root's x = 0 end

# (parent, length um, radius um, CVs)
CYLINDER = [(-1, 500.0, 1.0, 250)]
TREE = [(-1, 300.0, 1.2, 150), (0, 400.0, 0.8, 200), (0, 250.0, 0.5, 125), (1, 200.0, 0.6, 100),
        (1, 350.0, 0.4, 175)]


def _cell(tree, precision="f64"):
    from braincell_gb300 import Branch, Cell, Morphology
    from braincell_gb300.mech import (AllRegion, CableProperty, Channel, CurrentClamp, CVPerBranchList,
                                      RootLocation, StateProbe)

    root = Branch.from_lengths(lengths=[tree[0][1]], radii=[tree[0][2], tree[0][2]], type="dendrite")
    m = Morphology.from_root(root, name="b0")
    for k, (par, L, a, _) in enumerate(tree[1:], start=1):
        m.attach(parent=par, child_branch=Branch.from_lengths(lengths=[L], radii=[a, a], type="dendrite"),
                 child_name=f"b{k}", parent_x=1.0, child_x=0.0)
    c = Cell(m, cv_policy=CVPerBranchList(tuple(n for *_, n in tree)), precision=precision)
    c.paint(AllRegion(), CableProperty(resting_potential=E_LEAK, axial_resistivity=RA),
            Channel("IL", g_max=G_LEAK, E=E_LEAK))
    c.place(RootLocation(0.0), CurrentClamp(delay=0.0, durations=1e9, amplitudes=I_NA))
    c.place(RootLocation(0.5), StateProbe())
    return c


def _lam_ginf(a_um):
    rm = 1.0 / (G_LEAK * 1e-3)          # ohm cm^2
    a = a_um * 1e-4                      # cm
    lam = math.sqrt(rm * a / (2.0 * RA))  # cm
    ginf = math.pi * a * a / (RA * lam)  # S
    return lam, ginf


def analytic_midpoints(tree):
    """Steady-state V - E (mV) at every CV midpoint, branch by branch, CVs in order."""
    nb = len(tree)
    kids = [[k for k in range(nb) if tree[k][0] == b] for b in range(nb)]
    gin = [0.0] * nb
    for b in reversed(range(nb)):  # children have larger indices
        _, L, a, _ = tree[b]
        lam, ginf = _lam_ginf(a)
        gl = sum(gin[k] for k in kids[b])
        t = math.tanh(L * 1e-4 / lam)
        gin[b] = ginf * (gl + ginf * t) / (ginf + gl * t)
    vprox = [0.0] * nb
    vprox[0] = I_NA * 1e-9 / gin[0] * 1e3  # mV
    out = []
    for b in range(nb):
        _, L, a, n = tree[b]
        lam, ginf = _lam_ginf(a)
        gl = sum(gin[k] for k in kids[b])
        Lc = L * 1e-4
        den = math.cosh(Lc / lam) + gl / ginf * math.sinh(Lc / lam)
        y = (np.arange(n) + 0.5) / n * Lc
        out.append(vprox[b] * (np.cosh((Lc - y) / lam) + gl / ginf * np.sinh((Lc - y) / lam)) / den)
        for k in kids[b]:
            vprox[k] = vprox[b] / den
    return np.concatenate(out)


def test_single_cylinder_matches_rall_form():
    # the recursion reduces to the sealed-end closed form for one branch
    (_, L, a, n), = CYLINDER
    lam, ginf = _lam_ginf(a)
    x = (np.arange(n) + 0.5) / n * L * 1e-4
    want = I_NA * 1e-9 / ginf * np.cosh((L * 1e-4 - x) / lam) / math.sinh(L * 1e-4 / lam) * 1e3
    np.testing.assert_allclose(analytic_midpoints(CYLINDER), want, rtol=1e-12)


@pytest.mark.parametrize("tree", [CYLINDER, TREE], ids=["cylinder", "branched"])
def test_oracle_steady_state_matches_cable_theory(tree):
    oc = OracleCell(_cell(tree))
    assert len(oc.clamps_edge) == 1 and not oc.clamps_mid  # x = 0 is the root's endpoint node
    for _ in range(3):  # implicit Euler with a huge step lands on the steady state
        oc.step(1e9, t=0.0)
    got = oc.V[0] - E_LEAK
    want = analytic_midpoints(tree)
    assert want.min() > 1.0  # millivolts of depolarisation everywhere: a meaningful comparison
    np.testing.assert_allclose(got, want, rtol=2e-5)


def test_oracle_cable_error_is_second_order_in_the_cv_length():
    def err(tree):
        oc = OracleCell(_cell(tree))
        for _ in range(3):
            oc.step(1e9, t=0.0)
        return np.abs((oc.V[0] - E_LEAK) / analytic_midpoints(tree) - 1.0).max()

    fine = err(TREE)
    coarse = err([(p, L, a, n // 10) for p, L, a, n in TREE])
    assert 50.0 < coarse / fine < 200.0  # 10x the CV length: ~100x the error


@pytest.mark.gpu
@pytest.mark.parametrize("tree", [CYLINDER, TREE], ids=["cylinder", "branched"])
@pytest.mark.parametrize("precision,rtol", [("f64", 2e-5), ("f32", 1e-4)])
def test_gpu_steady_state_matches_cable_theory(native_lib, cuda_device, tree, precision, rtol):
    from braincell_gb300.batch import lower_cell
    from braincell_gb300.runtime import Plan

    p = Plan(lower_cell(_cell(tree, precision)), precision=precision, device=cuda_device)
    # 400 steps of 0.5 ms = 60 membrane time constants: converged far below the tolerance
    p.run(400, 0.5)
    got = p.state("V") - E_LEAK
    np.testing.assert_allclose(got, analytic_midpoints(tree), rtol=rtol)
    p.close()
