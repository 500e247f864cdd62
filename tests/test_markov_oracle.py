"""The oracle's Markov template and backward-Euler subsolver, pinned to the
reference's own known answers (CPU).

* ``quad/_backward_euler_test.py:71-86``: on dx/dt = -x / tau (tau 10 ms) one step of
  0.1 ms gives x0 / 1.01, and 1,000 steps of 0.01 ms land within 5e-4 of e^-1;
* ``channel/_base_test.py:1049-1065``: the stationary distribution of C <-> O -> I
  (0.2, 0.1; 0.05) is all in I;
* ``channel/_base_test.py:1177-1190``: C <-> O (0.2, 0.1) settles at O = 2/3;
* ``channel/_base_test.py:1117-1150``: the kinetics clip the independent states into
  [0, 1] and take the dependent state from the raw sum;
* ``channel/potassium_calcium_test.py:338-361``: Kca2p2's independent states are
  (C2, C3, C4, O1, O2), C1 is eliminated, and its steady state sums to 1.
"""

import math

import numpy as np

from oracle import markov as M


def _decay_scheme(k):
    # one independent state x = C draining into the dependent state at rate k:
    # dx/dt = -k x
    return M.MarkovScheme("decay", (("C", "D", "k", None),), "D", ("D",), "k", lambda V, Ci, p: {"k": k})


def test_backward_euler_one_step_is_the_implicit_solution():
    sch = _decay_scheme(0.1)
    y = M.backward_euler(sch, {"C": np.array([1.0])}, {"k": np.array([0.1])}, 0.1)
    assert abs(y["C"][0] - 1.0 / 1.01) < 1e-12


def test_backward_euler_converges_to_the_exact_decay():
    sch = _decay_scheme(0.1)
    y = {"C": np.array([1.0])}
    for _ in range(1000):
        y = M.backward_euler(sch, y, {"k": np.array([0.1])}, 0.01)
    assert abs(y["C"][0] - math.exp(-1.0)) < 5e-4


def test_substeps_split_the_step():
    sch = _decay_scheme(0.1)
    y = M.backward_euler(sch, {"C": np.array([1.0])}, {"k": np.array([0.1])}, 0.2, substeps=2)
    assert abs(y["C"][0] - 1.0 / 1.01 ** 2) < 1e-12


def _example():
    return M.MarkovScheme("example", (("C", "O", "open", "close"), ("O", "I", "inact", None)), "C", ("O",), "k",
                          lambda V, Ci, p: {"open": 0.2, "close": 0.1, "inact": 0.05})


def test_steady_state_of_an_absorbing_chain():
    r = {"open": np.array([0.2]), "close": np.array([0.1]), "inact": np.array([0.05])}
    ss = M.steady_state(_example(), r)
    assert abs(ss["I"][0] - 1.0) < 1e-12 and abs(ss["C"][0] + ss["O"][0]) < 1e-12


def test_steady_state_of_a_two_state_chain():
    sch = M.MarkovScheme("two", (("C", "O", "open", "close"),), "C", ("O",), "k", None)
    ss = M.steady_state(sch, {"open": np.array([0.2]), "close": np.array([0.1])})
    assert abs(ss["O"][0] - 2.0 / 3.0) < 1e-12


def test_kinetics_clip_independent_states_and_keep_the_raw_dependent_state():
    r = {"open": np.array([0.2]), "close": np.array([0.1]), "inact": np.array([0.05])}
    y = {"O": np.array([1.2]), "I": np.array([-0.1])}
    d = M.derivative(_example(), y, r)
    C = 1.0 - 1.2 + 0.1  # raw: -0.1
    assert abs(d["O"][0] - (C * 0.2 - 1.0 * 0.1 - 1.0 * 0.05)) < 1e-12
    assert abs(d["I"][0] - 1.0 * 0.05) < 1e-12


def test_jacobian_matches_finite_differences_inside_the_simplex():
    sch = M.SCHEMES["Nav1p6_MA2020_GoC"]
    p = M.scheme_params(sch.name, M.MARKOV_DEFAULTS[sch.name])
    V = np.array([-40.0])
    r = sch.rates(V, 5e-5, p)
    ss = M.steady_state(sch, r)
    y = {k: ss[k] * 0.9 + 0.1 / 13 for k in sch.independent}
    J = M.jacobian(sch, y, r)[0]
    f0 = M.derivative(sch, y, r)
    for j, kj in enumerate(sch.independent):
        h = 1e-7
        y2 = dict(y)
        y2[kj] = y[kj] + h
        f1 = M.derivative(sch, y2, r)
        for i, ki in enumerate(sch.independent):
            assert abs((f1[ki][0] - f0[ki][0]) / h - J[i, j]) < 1e-4 * max(1.0, abs(J[i, j]))


def test_channel_states_and_dependent_states():
    k22 = M.SCHEMES["Kca2p2_MA2020_GoC"]
    assert k22.independent == ("C2", "C3", "C4", "O1", "O2") and k22.dependent == "C1"
    nav = M.SCHEMES["Nav1p6_MA2020_GoC"]
    assert nav.dependent == "I6" and len(nav.independent) == 12
    k11 = M.SCHEMES["Kca1p1_MA2020_GoC"]
    assert k11.dependent == "C0" and len(k11.independent) == 9


def test_steady_states_are_stationary_probabilities():
    for name, sch in M.SCHEMES.items():
        p = M.scheme_params(name, M.MARKOV_DEFAULTS[name])
        V = np.array([-70.0, -40.0, 0.0])
        r = sch.rates(V, np.array([5e-5, 1e-4, 1e-3]), p)
        ss = M.steady_state(sch, r)
        np.testing.assert_allclose(sum(ss[k] for k in sch.states), 1.0, rtol=1e-12)
        assert min(float(np.min(ss[k])) for k in sch.states) >= 0.0
        d = M.derivative(sch, {k: ss[k] for k in sch.independent}, r)
        for k in sch.independent:
            np.testing.assert_allclose(d[k], 0.0, atol=1e-9)
        # a backward-Euler step from the steady state stays there
        y = M.backward_euler(sch, {k: ss[k] for k in sch.independent}, r, 0.025)
        for k in sch.independent:
            np.testing.assert_allclose(y[k], ss[k], atol=1e-12)


def test_nav16_rate_constants():
    # sodium.py:894-898: alfac = (Oon / Con)^(1/4), btfac = (Ooff / Coff)^(1/4); at 22 degC phi = 1
    sch = M.SCHEMES["Nav1p6_MA2020_GoC"]
    p = M.scheme_params(sch.name, M.MARKOV_DEFAULTS[sch.name])
    assert p["phi"] == 1.0
    r = sch.rates(np.array([0.0]), 5e-5, p)
    assert abs(r["f01"][0] - 600.0) < 1e-9 and abs(r["b04"][0] - 12.0) < 1e-9
    assert abs(r["fi5"][0] - 0.005 * 150.0) < 1e-12 and abs(r["bi5"][0] - 0.5 * 0.01) < 1e-12
