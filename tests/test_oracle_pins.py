"""Pins the float64 oracle to the reference's own known answers (tests/golden)."""

import json
import math
import os

import numpy as np
import pytest

from oracle import staggered as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_known_answers.json")))


def _radii(case):
    if "radii" in case:
        r = np.asarray(case["radii"])
        return r[:-1], r[1:]
    _, rp, rd = O.insert_radius_jumps(case["lengths"], case["radii_proximal"], case["radii_distal"])
    return rp, rd


def _lengths(case):
    if "radii" in case:
        return case["lengths"]
    return O.insert_radius_jumps(case["lengths"], case["radii_proximal"], case["radii_distal"])[0]


@pytest.mark.parametrize("case", GOLD["frusta"], ids=lambda c: c["src"].split()[-1])
def test_frusta(case):
    rp, rd = _radii(case)
    if "split_x" in case:
        x = case["split_x"]
        left = O.build_frusta(_lengths(case), rp, rd, 0.0, x)
        right = O.build_frusta(_lengths(case), rp, rd, x, 1.0)
        assert len(left) == case["n_left"] and len(right) == case["n_right"]
        assert left[-1].length_um == pytest.approx(case["left_last_length_um"])
        assert right[0].length_um == pytest.approx(case["right_first_length_um"])
        whole = O.build_frusta(_lengths(case), rp, rd, 0.0, 1.0)
        assert O.lateral_area_um2(left) + O.lateral_area_um2(right) == pytest.approx(O.lateral_area_um2(whole), abs=1e-4)
        return
    fr = O.build_frusta(_lengths(case), rp, rd, case["prox"], case["dist"])
    assert len(fr) == case["n"]
    assert [f.length_um for f in fr] == pytest.approx(case["length_um"])
    if "r_prox_um" in case:
        assert [f.r_prox_um for f in fr] == pytest.approx(case["r_prox_um"])
        assert [f.r_dist_um for f in fr] == pytest.approx(case["r_dist_um"])
    if "jump_index" in case:
        j = fr[case["jump_index"]]
        assert j.r_prox_um == pytest.approx(case["jump_r_prox_um"])
        assert j.r_dist_um == pytest.approx(case["jump_r_dist_um"])


def test_jump_branch_area_and_axial_factor():
    # geometry_test.py:95-115: the zero-length jump adds the annulus area but no axial resistance
    lengths, rp, rd = [10.0, 20.0], np.array([2.0, 4.0]), np.array([1.0, 2.0])
    fr = O.build_frusta(*O.insert_radius_jumps(lengths, rp, rd), 0.0, 1.0)
    expected = sum((L * 1e-4) / (math.pi * (a * 1e-4) * (b * 1e-4)) for L, a, b in zip(lengths, rp, rd))
    assert O.axial_factor_per_cm(fr) == pytest.approx(expected, abs=1e-9)
    area = sum(math.pi * (a + b) * math.sqrt(L * L + (b - a) ** 2) for L, a, b in zip(lengths, rp, rd))
    area += math.pi * (4.0 ** 2 - 1.0 ** 2)  # annulus of the 1 -> 4 um jump
    assert O.lateral_area_um2(fr) == pytest.approx(area, abs=1e-4)


@pytest.mark.parametrize("case", GOLD["frusta_rejects"], ids=lambda c: f"{c['prox']}-{c['dist']}")
def test_frusta_rejects(case):
    rp, rd = _radii(case)
    with pytest.raises(ValueError):
        O.build_frusta(case["lengths"], rp, rd, case["prox"], case["dist"])


@pytest.mark.parametrize("case", GOLD["frustum_scalars"], ids=lambda c: c["src"].split()[-1])
def test_frustum_scalars(case):
    fr = (O.Frustum(0.0, 1.0, case["length_um"], case["r0"], case["r1"]),)
    if "area_um2" in case:
        assert round(O.lateral_area_um2(fr) - case["area_um2"], case["area_places"]) == 0
    if "axial_factor_per_cm" in case:
        assert round(O.axial_factor_per_cm(fr) - case["axial_factor_per_cm"], case["axial_places"]) == 0
    if "midpoint_radius_um" in case:
        assert O.midpoint_radius_um(fr) == pytest.approx(case["midpoint_radius_um"])


@pytest.mark.parametrize("case", GOLD["peel_levels"], ids=lambda c: c["src"])
def test_peel_levels(case):
    lv = O.compute_peel_levels(np.asarray(case["node_parent"]), case["node_children"])
    assert lv.tolist() == case["levels"]


def test_peel_levels_cycle():
    c = GOLD["peel_levels_cycle"]
    with pytest.raises(ValueError, match="cycle"):
        O.compute_peel_levels(np.asarray(c["node_parent"]), c["node_children"])


def test_backsub_indices():
    a, b = GOLD["backsub_indices"]
    idx = O.build_backsub_indices(np.asarray(a["parent_lookup"]), a["n_nodes"])
    assert idx.shape[1] == a["ncols"] and int(idx[0, 0]) == a["idx00"]
    idx = O.build_backsub_indices(np.asarray(b["parent_lookup"]), b["n_nodes"])
    assert idx[0].tolist() == b["row0"] and int(idx[1, 0]) == b["idx10"]


def test_rate_known_answers():
    kdr, na = GOLD["rates"]
    r = O.rates("KDR_Ba2002", np.asarray([kdr["V"]]), {"V_sh": kdr["V_sh"]})
    assert float(r["p"][1][0]) == pytest.approx(kdr["alpha"], rel=1e-12)
    (v1, s1), (v2, s2) = na["pair"]
    a1 = O.rates("Na_Ba2002", np.asarray([v1]), {"V_sh": s1})["p"][1]
    a2 = O.rates("Na_Ba2002", np.asarray([v2]), {"V_sh": s2})["p"][1]
    assert abs(float(a1[0] - a2[0])) <= na["atol"]


def test_q10_factor():
    q = GOLD["q10"]
    phi = q["q10"] ** ((q["temp"] - q["temp_ref"]) / 10.0)
    assert phi == pytest.approx(q["phi"], abs=q["atol"])
    from braincell_gb300.catalogue import q10_phi

    assert q10_phi(q["q10"], q["temp"], q["temp_ref"]) == pytest.approx(q["phi"], abs=q["atol"])


def test_exprel():
    assert float(O.exprel(0.0)) == 1.0
    x = np.asarray([1e-8, -1e-3, 0.5, -3.0])
    assert np.allclose(O.exprel(x), np.expm1(x) / x, rtol=1e-14)


def _soma_cell(case, pop=1):
    from braincell_gb300 import Branch, Cell, Morphology
    from braincell_gb300.mech import CurrentClamp, CVPerBranch, RootLocation

    soma = Branch.from_lengths(lengths=[case["soma_length"]], radii=[case["soma_radius"]] * 2, type="soma")
    cell = Cell(Morphology.from_root(soma, name="soma"), pop_size=pop, cv_policy=CVPerBranch(),
                V_init=case.get("V_init"))
    cell.place(RootLocation(case["clamp_x"]),
               CurrentClamp(delay=case["delay"], durations=case["durations"], amplitudes=case["amplitudes"]))
    return cell


@pytest.mark.parametrize("case", GOLD["step_behaviour"][:2], ids=["endpoint", "multistep"])
def test_oracle_clamp_raises_voltage(case):
    oc = O.OracleCell(_soma_cell(case))
    before = oc.V[0, 0]
    oc.step(case["dt"], 0.0)
    assert oc.V[0, 0] > before


def test_oracle_population_widening_is_neutral():
    case = GOLD["step_behaviour"][2]
    single = O.OracleCell(_soma_cell(case))
    pop = O.OracleCell(_soma_cell(case, pop=case["pop"]))
    single.step(case["dt"], 0.0)
    pop.step(case["dt"], 0.0)
    for m in range(case["pop"]):
        np.testing.assert_allclose(pop.V[m], single.V[0], rtol=case["rtol"], atol=case["atol"])


def test_oracle_small_config_structure():
    """The small workload lowers to 129 points, 29 DHS levels, 8 back-substitution passes."""
    from braincell_gb300 import workloads as W

    oc = O.OracleCell(W.desc_to_cell(W.small(1)[0]))
    assert oc.n_cv == 113 and oc.n_point == 129
    assert len(oc.level_offsets) - 1 == 29
    assert oc.backsub.shape[0] == 8


def test_oracle_rest_is_steady_without_input():
    """With no stimulus the passive cell stays near rest and nothing diverges."""
    from braincell_gb300 import workloads as W

    d = W.small(1)[0]
    d.pulses = []
    oc = O.OracleCell(W.desc_to_cell(d))
    for _ in range(200):
        oc.step(0.025)
    assert np.all(np.isfinite(oc.V))
    assert np.all(np.abs(oc.V + 67.5) < 3.0)


def test_hh1952_rates_match_published_forms():
    # channel/sodium.py:293-330 and channel/potassium.py:341-380 docstrings: with the
    # default V_sh = -45 mV the rates are Hodgkin & Huxley's published forms
    from oracle.staggered import rates

    V = np.array([-80.0, -65.0, -52.5, -20.0, 10.0])
    na = rates("Na_HH1952", V, {"V_sh": -45.0})
    np.testing.assert_allclose(na["p"][1], 0.1 * (V + 40) / (1 - np.exp(-(V + 40) / 10)), rtol=1e-12)
    np.testing.assert_allclose(na["p"][2], 4 * np.exp(-(V + 65) / 18), rtol=1e-12)
    np.testing.assert_allclose(na["q"][1], 0.07 * np.exp(-(V + 65) / 20), rtol=1e-12)
    np.testing.assert_allclose(na["q"][2], 1 / (1 + np.exp(-(V + 35) / 10)), rtol=1e-12)
    k = rates("K_HH1952", V, {"V_sh": -45.0})
    np.testing.assert_allclose(k["p"][1], 0.01 * (V + 55) / (1 - np.exp(-(V + 55) / 10)), rtol=1e-12)
    np.testing.assert_allclose(k["p"][2], 0.125 * np.exp(-(V + 65) / 80), rtol=1e-12)
    # removable singularities: alpha_m(-40) = 1, alpha_n(-55) = 0.1 (potassium.py docstring)
    assert rates("Na_HH1952", np.array([-40.0]), {"V_sh": -45.0})["p"][1][0] == pytest.approx(1.0)
    assert rates("K_HH1952", np.array([-55.0]), {"V_sh": -45.0})["p"][1][0] == pytest.approx(0.1)


def test_km_rates_and_temperature_factor():
    # channel/potassium.py:1597-1748: n_inf = 1 / (1 + exp(-(V + 35) / 6)),
    # tau_n = 1 / (alpha_n + beta_n), gate q10 3 at 22 degC (phi = 3^0.8 at 30 degC)
    from braincell_gb300.catalogue import KM_Q10, KM_TEMP_REF, q10_phi
    from braincell_gb300.mech import celsius2kelvin
    from oracle.staggered import rates

    V = np.array([-60.0, -35.0, 0.0])
    r = rates("KM_RI2021_SC", V, {})
    np.testing.assert_allclose(r["n"][1], 1 / (1 + np.exp(-(V + 35) / 6)), rtol=1e-12)
    a, b = 0.0033 * np.exp((V + 30) / 40), 0.0033 * np.exp((V + 30) / -20)
    np.testing.assert_allclose(r["n"][2], 1 / (a + b), rtol=1e-12)
    assert q10_phi(KM_Q10, celsius2kelvin(30.0), KM_TEMP_REF) == pytest.approx(3.0 ** 0.8)
    assert q10_phi(3.0, celsius2kelvin(46.0), celsius2kelvin(36.0)) == pytest.approx(3.0)  # potassium_test.py:113-121


@pytest.mark.parametrize("cls,kern", [("Na_TM1991", "Na_Ba2002"), ("K_TM1991", "KDR_Ba2002"),
                                      ("CaHT_HM1992", "CaT_HM1992"), ("KM_MA2020_GoC", "KM_RI2021_SC"),
                                      ("KM_MA2020_GrC", "KM_RI2021_SC")])
def test_same_form_classes_match_their_kernel_class(cls, kern):
    # The TM1991 classes restate the Traub-Miles rates in terms of V_sh - V
    # (sodium.py:275-289, potassium.py:331-337) and CaHT_HM1992 repeats CaT_HM1992's
    # (calcium.py:645-663); with the same V_sh the gate rates are equal, which is why
    # the catalogue runs them on the kernel class with their own defaults.
    from braincell_gb300 import catalogue

    assert catalogue.kernel_class(cls) == kern
    p = dict(O.CHANNEL_DEFAULTS[cls])
    q = dict(O.CHANNEL_DEFAULTS[kern], **({"V_sh": p["V_sh"]} if "V_sh" in p else {}))
    if "V_sh" not in p:  # no shift parameter: the defaults themselves agree
        assert p == O.CHANNEL_DEFAULTS[kern]
        p["V_sh"] = 0.0
    V = np.concatenate([np.linspace(-120.0, 60.0, 721), p["V_sh"] + np.array([13.0, 15.0, 40.0, -80.0])])
    a, b = O.rates(cls, V, p), O.rates(kern, V, q)
    assert a.keys() == b.keys()
    for g in a:
        assert a[g][0] == b[g][0]
        for k in (1, 2):
            np.testing.assert_allclose(a[g][k], b[g][k], rtol=1e-12, atol=0.0)


def test_same_form_defaults_and_exclusion():
    from braincell_gb300 import _abi, catalogue
    from braincell_gb300.mech import CableProperty, Channel

    bits, rec = catalogue.region_record([Channel("Na_TM1991"), Channel("K_TM1991", g_max=5.0),
                                         Channel("CaHT_HM1992")], CableProperty())
    assert bits == _abi.BC_M_NA | _abi.BC_M_KDR | _abi.BC_M_CAT
    assert (rec[_abi.BC_P_NA_G], rec[_abi.BC_P_NA_VSH], rec[_abi.BC_P_NA_PHI]) == (120.0, -63.0, 1.0)
    assert (rec[_abi.BC_P_KDR_G], rec[_abi.BC_P_KDR_VSH], rec[_abi.BC_P_KDR_PHI]) == (5.0, -60.0, 1.0)
    assert rec[_abi.BC_P_CAT_VSH] == 25.0
    assert rec[_abi.BC_P_CAT_PHIP] == pytest.approx(3.55 ** 1.2) and rec[_abi.BC_P_CAT_PHIQ] == pytest.approx(3.0 ** 1.2)
    for pair in (("Na_TM1991", "Na_Ba2002"), ("KDR_Ba2002", "K_TM1991"), ("CaT_HM1992", "CaHT_HM1992")):
        with pytest.raises(ValueError, match="same kernel"):
            catalogue.region_record([Channel(pair[0]), Channel(pair[1])], CableProperty())


def test_a_current_rates():
    # KA1_HM1992 / KA2_HM1992 (potassium.py:592-611, :743-762): activation midpoints
    # -60 and -36 mV, the same inactivation in both classes, and tau_q applying the
    # expression strictly below V' = -63 and 19 ms at and above it (the branches do
    # not meet: about 23.4 ms just below, as the class docstring notes).
    p1, p2 = dict(O.CHANNEL_DEFAULTS["KA1_HM1992"]), dict(O.CHANNEL_DEFAULTS["KA2_HM1992"])
    assert O.rates("KA1_HM1992", np.array(-60.0), p1)["p"][1] == pytest.approx(0.5)
    assert O.rates("KA2_HM1992", np.array(-36.0), p2)["p"][1] == pytest.approx(0.5)
    V = np.linspace(-120.0, 40.0, 641)
    a, b = O.rates("KA1_HM1992", V, p1), O.rates("KA2_HM1992", V, p2)
    np.testing.assert_array_equal(a["q"][1], b["q"][1])
    np.testing.assert_array_equal(a["q"][2], b["q"][2])
    np.testing.assert_array_equal(a["p"][2], b["p"][2])
    assert float(O.rates("KA1_HM1992", np.array(-63.0), p1)["q"][2]) == 19.0
    below = float(O.rates("KA1_HM1992", np.array(-63.0 - 1e-9), p1)["q"][2])
    assert below == pytest.approx(23.4, abs=0.05)


def test_a_current_records():
    from braincell_gb300 import _abi, catalogue
    from braincell_gb300.mech import CableProperty, Channel, celsius2kelvin as T

    bits, rec = catalogue.region_record([Channel("KA1_HM1992"), Channel("KA2_HM1992", g_max=7.0, V_sh=2.0)],
                                        CableProperty())
    assert bits == _abi.BC_M_KA1 | _abi.BC_M_KA2
    assert list(rec[_abi.BC_P_KA1_G:_abi.BC_P_KA1_PHIQ + 1]) == [30.0, 0.0, 1.0, 1.0]
    assert list(rec[_abi.BC_P_KA2_G:_abi.BC_P_KA2_PHIQ + 1]) == [7.0, 2.0, 1.0, 1.0]
    bits, rec = catalogue.region_record([Channel("KK2A_HM1992", temp=T(26.0)), Channel("KK2B_HM1992", g_max=4.0)],
                                        CableProperty())
    assert bits == _abi.BC_M_KK2A | _abi.BC_M_KK2B
    assert list(rec[_abi.BC_P_KK2A_G:_abi.BC_P_KK2A_PHIQ + 1]) == [10.0, 0.0, 1.0, 1.0]  # q10 1: phi 1 at any temp
    assert list(rec[_abi.BC_P_KK2B_G:_abi.BC_P_KK2B_PHIQ + 1]) == [4.0, 0.0, 1.0, 1.0]


def test_deprecated_channel_names_resolve():
    # channel/__init__.py:49-86: the pre-rename names warn and give the renamed class
    from braincell_gb300 import catalogue
    from braincell_gb300.mech import CableProperty, Channel

    with pytest.warns(DeprecationWarning, match="use KA1_HM1992"):
        old = Channel("IKA1_HM1992", g_max=3.0)
    assert old.class_name == "KA1_HM1992" and old.instance_name == "KA1_HM1992"
    a = catalogue.region_record([old], CableProperty())
    b = catalogue.region_record([Channel("KA1_HM1992", g_max=3.0)], CableProperty())
    assert a[0] == b[0] and (a[1] == b[1]).all()


def test_slow_k2_rates():
    # KK2A_HM1992 / KK2B_HM1992 (potassium.py:881-895, :1023-1041): the same
    # activation and inactivation curves; KK2A's tau_q is 120 ms + a bell, KK2B's is
    # the bell strictly below V' = -70 (about 885 ms just below, as its docstring
    # notes) and 8.9 ms at and above.
    pa, pb = dict(O.CHANNEL_DEFAULTS["KK2A_HM1992"]), dict(O.CHANNEL_DEFAULTS["KK2B_HM1992"])
    V = np.linspace(-120.0, 40.0, 641)
    a, b = O.rates("KK2A_HM1992", V, pa), O.rates("KK2B_HM1992", V, pb)
    for k in (1, 2):
        np.testing.assert_array_equal(a["p"][k], b["p"][k])
    np.testing.assert_array_equal(a["q"][1], b["q"][1])
    assert float(O.rates("KK2B_HM1992", np.array(-70.0), pb)["q"][2]) == 8.9
    below = float(O.rates("KK2B_HM1992", np.array(-70.0 - 1e-9), pb)["q"][2])
    assert below == pytest.approx(885.0, rel=0.01)
    assert float(O.rates("KK2A_HM1992", np.array(-70.0), pa)["q"][2]) == pytest.approx(below + 120.0, rel=1e-6)
    assert O.rates("KK2A_HM1992", np.array(-43.0), pa)["p"][1] == pytest.approx(0.5)


def test_kni_rates_and_record():
    # KNI_Ya1989 (potassium.py:1156-1163): p_inf is 1/2 at V' = -35 mV, where
    # tau = tau_max / (3.3 + 1); tau_max is a constructor parameter in ms.
    from braincell_gb300 import _abi, catalogue
    from braincell_gb300.mech import CableProperty, Channel

    p = dict(O.CHANNEL_DEFAULTS["KNI_Ya1989"])
    r = O.rates("KNI_Ya1989", np.array(-35.0), p)["p"]
    assert r[1] == pytest.approx(0.5) and r[2] == pytest.approx(4000.0 / 4.3)
    bits, rec = catalogue.region_record([Channel("KNI_Ya1989", tau_max=2000.0, V_sh=-3.0)], CableProperty())
    assert bits == _abi.BC_M_KNI
    assert list(rec[_abi.BC_P_KNI_G:_abi.BC_P_KNI_TAUMAX + 1]) == [0.004, -3.0, 1.0, 2000.0]


# ------------------------------------------------------------------ defaults, phi, currents, calcium


@pytest.mark.parametrize("case", GOLD["defaults"], ids=lambda c: c["class"])
def test_reference_defaults(case):
    # the oracle and the product catalogue both hold the reference's constructor defaults
    from braincell_gb300 import catalogue

    oracle_table = O.CHANNEL_DEFAULTS if case["kind"] == "channel" else O.ION_DEFAULTS
    product_table = catalogue.CHANNELS if case["kind"] == "channel" else catalogue.IONS
    for k, v in case["values"].items():
        assert oracle_table[case["class"]][k] == pytest.approx(v, rel=1e-12), (case["src"], k)
        assert product_table[case["class"]][k] == pytest.approx(v, rel=1e-12), (case["src"], k)


@pytest.mark.parametrize("case", GOLD["gate_phi"], ids=lambda c: c["src"].split()[0])
def test_gate_phi_known_answers(case):
    from braincell_gb300 import catalogue
    from braincell_gb300.mech import CableProperty, Channel

    for cls in case["classes"]:
        p = O._resolve(O.CHANNEL_DEFAULTS, Channel(cls, **case["params"]))
        for key, phi in case["phi"].items():
            assert p[key] == pytest.approx(phi, abs=case["atol"]), (cls, key)
        # the product record carries the same factors (its phi slots)
        _, rec = catalogue.region_record([Channel(cls, **case["params"])], CableProperty())
        k = catalogue.kernel_class(cls)
        slots = {"CaT_HM1992": (_abi_slot("CAT_PHIP"), _abi_slot("CAT_PHIQ")),
                 "CaL_IS2008": (_abi_slot("CAL_PHIP"), _abi_slot("CAL_PHIQ")),
                 "HCN_HM1992": (_abi_slot("HCN_PHI"),)}[k]
        assert [rec[s] for s in slots] == pytest.approx(list(case["phi"].values()), abs=case["atol"])


def _abi_slot(name):
    from braincell_gb300 import _abi

    return getattr(_abi, "BC_P_" + name)


@pytest.mark.parametrize("case", GOLD["currents"], ids=lambda c: c["class"])
def test_current_known_answers(case):
    # HCN current g_max p (E - V), evaluated the way the oracle evaluates channel currents
    from braincell_gb300 import Branch, Cell, Morphology
    from braincell_gb300.mech import AllRegion, CableProperty, Channel

    soma = Branch.from_lengths(lengths=[20.0], radii=[10.0, 10.0], type="soma")
    c = Cell(Morphology.from_root(soma, name="soma"))
    c.paint(AllRegion(), CableProperty(resting_potential=case["V"]), Channel(case["class"], **case["params"]))
    oc = O.OracleCell(c)
    for g, v in case["gates"].items():
        oc.gates[(case["class"], g)][:] = v
    pv = oc.cv_to_point(oc.V)
    I, dI = oc._channel_currents(pv)
    mid = oc.cv_mid[0]
    assert I[0, mid] == pytest.approx(case["current"], abs=case["atol"])
    assert dI[0, mid] == pytest.approx(-case["params"]["g_max"] * case["gates"]["p"], abs=1e-12)


def test_calcium_detailed_known_answers():
    cases = {c["src"].split()[1]: c for c in GOLD["calcium_detailed"]}
    dflt = O.ION_DEFAULTS["CalciumDetailed"]
    c = cases["test_E_zero_when_internal_equals_external"]
    assert O.nernst_ca_mV(dflt["temp"], dflt["Co"], c["Ci"]) == pytest.approx(c["E"], abs=c["atol"])
    c = cases["test_derivative_without_current_matches_leak_formula"]
    got = O.ca_detailed_rate(c["I_ca"], c["Ci"], dflt["d"], c["tau"], c["C_rest"])
    assert got == pytest.approx(c["dCi_dt"], abs=c["atol"])
    c = cases["test_E_updates_with_C_dynamically"]
    assert O.nernst_ca_mV(dflt["temp"], dflt["Co"], c["Ci_high"]) < O.nernst_ca_mV(dflt["temp"], dflt["Co"], c["Ci_low"])
    # an inward calcium current only ever adds calcium; an outward one is clipped to no influx
    assert O.ca_detailed_rate(-5.0, 1e-4, 1.0, 5.0, 1e-4) == 0.0
    assert O.ca_detailed_rate(5.0, 1e-4, 1.0, 5.0, 1e-4) > 0.0


# ------------------------------------------------------------------ exp-Euler against the closed form


@pytest.mark.parametrize("name,gate", [("CaL_IS2008", "q"), ("Na_Ba2002", "p"), ("HCN_HM1992", "p"),
                                       ("KDR_Ba2002", "p")])
def test_gate_exp_euler_is_the_exact_exponential(name, gate):
    # at fixed V a gate ODE is linear, x' = (x_inf - x) / tau_eff, so one exp-Euler
    # step must equal the closed-form x_inf + (x - x_inf) exp(-dt / tau_eff)
    p = O._resolve(O.CHANNEL_DEFAULTS, _decl(name))
    phik = {g: k for g, _, k in O._GATES[name]}[gate]
    V = np.linspace(-90.0, 30.0, 25)
    kind, a, b = O.rates(name, V, p)[gate]
    if kind == "ab":
        xinf, tau = a / (a + b), 1.0 / (p[phik] * (a + b))
    else:
        xinf, tau = a, b / p[phik]
    for dt in (0.025, 0.5, 7.0):
        x0 = np.full_like(V, 0.3)
        got = O.gate_step(x0, kind, a, b, p[phik], dt)
        want = xinf + (x0 - xinf) * np.exp(-dt / tau)
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-15)


def _decl(name):
    from braincell_gb300.mech import Channel

    return Channel(name)
