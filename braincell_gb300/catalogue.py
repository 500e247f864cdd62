"""Mechanism catalogue: declaration -> per-region parameter record.

Every class name, parameter name and default below is the reference's:

* ``IL``          -- channel/leaky.py:144   (g_max 0.1 mS/cm^2, E -70 mV)
* ``K_Leak``      -- channel/potassium.py:1167 (g_max 0.005 mS/cm^2, E = E_K)
* ``Na_Ba2002``   -- channel/sodium.py:59   (g_max 90, q10 3, temp = temp_ref = 36 degC, V_sh -50)
* ``KDR_Ba2002``  -- channel/potassium.py:95 (g_max 10, q10 3, temp = temp_ref = 36 degC, V_sh -50)
* ``CaL_IS2008``  -- channel/calcium.py:790 (g_max 1, q10_p 3.55, q10_q 3, temp_ref 24 degC, V_sh 0)
* ``CaT_HM1992``  -- channel/calcium.py:222 (g_max 2, q10_p 3.55, q10_q 3, temp_ref 24 degC, V_sh -3)
* ``HCN_HM1992``  -- channel/hyperpolarization_activated.py:45 (g_max 10, E +43 mV, q10 1)
* ``AHP_De1994``  -- channel/potassium_calcium.py:78 (n 2, g_max 10, alpha 48, beta 0.09, phi 1)
* ``Na_HH1952``   -- channel/sodium.py:293  (g_max 120, q10 3, temp = temp_ref = 36 degC, V_sh -45)
* ``K_HH1952``    -- channel/potassium.py:341 (g_max 10, q10 3, temp = temp_ref = 36 degC, V_sh -45)
* ``KM_RI2021_SC``-- channel/potassium.py:1597 (g_max 0.25, temp 30 degC; gate q10 3 at 22 degC)
* ``Na_TM1991``   -- channel/sodium.py:174  (g_max 120, q10 1, temp = temp_ref = 36 degC, V_sh -63)
* ``K_TM1991``    -- channel/potassium.py:218 (g_max 10, q10 1, temp = temp_ref = 36 degC, V_sh -60)
* ``CaHT_HM1992`` -- channel/calcium.py:511 (g_max 2, q10_p 3.55, q10_q 3, temp_ref 24 degC, V_sh 25)
* ``KA1_HM1992``  -- channel/potassium.py:460 (g_max 30, q10_p = q10_q = 1, temp = temp_refs = 36 degC, V_sh 0)
* ``KA2_HM1992``  -- channel/potassium.py:614 (g_max 20, otherwise as KA1_HM1992)
* ``KK2A_HM1992`` -- channel/potassium.py:765 (g_max 10, q10_p = q10_q = 1, temp = temp_refs = 36 degC, V_sh 0)
* ``KK2B_HM1992`` -- channel/potassium.py:899 (as KK2A_HM1992)
* ``KNI_Ya1989``  -- channel/potassium.py:1045 (g_max 0.004, q10 1, temp = temp_ref = 36 degC, tau_max 4 s, V_sh 0)
* ``Nav1p6_MA2020_GoC`` -- channel/sodium.py:727 (Markov; g_max 16, temp 22 degC, phi = 3^((T - 22 degC) / 10))
* ``Nav1p1_MA2025_BC`` / ``Nav1p1_RI2021_SC`` -- channel/sodium.py:1188, :1351 (the Nav1.6 scheme with Oon 2.3,
  epsilon 1e-12, phi = 2.7^((T - 22 degC) / 10); g_max 8, temp 22 degC, gateCurrent 0)
* ``Kca2p2_MA2020_GoC`` -- channel/potassium_calcium.py:613 (Markov; g_max 38, q10_base 3, diff 3, temp 22 degC,
  phi = q10_base^((T - 23 degC) / 10))
* ``Kca1p1_MA2020_GoC`` -- channel/potassium_calcium.py:1107 (Markov; g_max 10, q10_base 3, temp 22 degC, phi as
  Kca2p2; alpha(V) = exp(0.73 F V / R T), beta(V) = exp(-0.67 F V / R T))
* ``Kv3p4_MA2020_GoC`` -- channel/potassium.py:4750 (g_max 4, temp 22 degC; gates q10 3 at 37 degC)
* ``Kv4p3_MA2020_GoC`` -- channel/potassium.py:4964 (g_max 3.2, temp 22 degC; gates q10 3 at 25.5 degC; the GrC / PC /
  BC / SC variants default to 30 degC)
* ``Kv1p1_MA2020_GoC`` -- channel/potassium.py:4570 (g_max 4, temp 22 degC, gateCurrent 0; gate q10 2.7 at 22 degC)
* ``Kir2p3_MA2020_GrC`` -- channel/potassium.py:5334 (g_max 0.9, temp 30 degC; gate q10 3 at 20 degC)
* ``HCN1_MA2020_GoC`` -- channel/hyperpolarization_activated.py:675 (g_max 0.05, E -20 mV, temp 22 degC; gates q10 3
  and g Q10 1.5, both at 23 degC)
* ``HCN1_MA2024_PC`` -- channel/hyperpolarization_activated.py:411 (g_max 0.1, E -34.4 mV, temp 23 degC; gate q10 3
  at 37 degC)
* ``CaHVA_MA2020_GoC`` / ``_GrC`` -- channel/calcium.py:4333, :4499 (g_max 0.46, temp 30 degC; gates q10 3 at 20 degC)
* ``Cav2p3_MA2020_GoC`` -- channel/calcium.py:4672 (g_max 0, temp 34 degC; gates without a temperature factor)
* ``Cav3p2_RI2021_SC`` -- channel/calcium.py:3636 (g_max 8e-4, V_sh 0, temp 36 degC; m phi 5^1.2, the h time constant
  carrying 3^1.2); the MA2025_BC and MA2024_PC classes inherit it

Extension channels (bit BC_M_EXT; the region's record lists them as BC_X_* bits in
BC_P_EXT_MASK, their parameters after it; conductances in mS/cm^2):
* ``HCN2_MA2020_GoC`` -- channel/hyperpolarization_activated.py:838 (g_max 0.08, E -20 mV, temp 22 degC; gates q10 3
  and g Q10 1.5 at 23 degC)
* ``Kv3p3_MA2024_PC`` -- channel/potassium.py:2937 (g_max 5, temp 22 degC, gateCurrent 0; gate q10 2.7 at 22 degC)
* ``Kv2p2_0010_MA2020_GrC`` -- channel/potassium.py:5664 (g_max 0.01, BBiD 10, unused by the rates)
* ``Kv1p5_MA2024_PC`` -- channel/potassium.py:2735 (g_max 0.13195, temp 37 degC, Tauact / Tauinactf / Tauinacts 1;
  rates scaled by 2.2^((T - 37 degC) / 10); current times 0.1 + 1 / (1 + exp(-(V - 15) / 13)))
* ``NaF_SU2015_DCN``, ``NaP_SU2015_DCN`` -- channel/sodium.py:402, :500 (g_max 0.01)
* ``Na_ZH2019_IO`` -- channel/sodium.py:598 (g_max 70)
* ``fKdr_SU2015_DCN``, ``sKdr_SU2015_DCN`` -- channel/potassium.py:1374, :1485 (g_max 0.01)
* ``Kdr_ZH2019_IO`` -- channel/potassium.py:6238 (g_max 18)
* ``HCN_SU2015_DCN`` -- channel/hyperpolarization_activated.py:1010 (g_max 0.01, E -45 mV)
* ``HCN_ZH2019_IO`` -- channel/hyperpolarization_activated.py:1109 (g_max 0.15, E -43 mV)
* ``CaT_HP1992`` -- channel/calcium.py:377 (g_max 1.75, temp 36 degC, q10_p 5 / q10_q 3 at 24 degC, V_sh -3 mV)
* ``CaHT_Re1993`` -- channel/calcium.py:667 (g_max 1, temp 36 degC, q10 2.3 at 23 degC, V_sh 0)
* ``CaL_SU2015_DCN`` -- channel/calcium.py:1066 (g_max 0.01, E 139 mV, qdeltat 1; not a calcium-ion channel)
* ``Kv1p5_MA2020_GrC`` -- channel/potassium_sodium.py:38 on Kv1p5_MA2024_PC's kernel (its nonspecific current,
  gnonspec, 0 by default: only 0 is built)
* ``Kca3p1_MA2020_GoC`` -- channel/potassium_calcium.py:299 (g_max 120; q10_base and temp accepted, unused); the
  MA2025_BC and MA2024_PC classes (:452, :533) repeat it
* ``SK_SU2015_DCN`` -- channel/potassium_calcium.py:189 (g_max 0.01, qdeltat 1)
* ``K_Kv_test`` -- channel/potassium.py:1239 (g_max 0, V_sh 0, Ra 0.02, Rb 0.006, q 9 mV, v12 25 mV; Q10_n 1)
* ``CaN_IS2008`` -- channel/calcium.py:108 (g_max 1, E 10 mV, temp 36 degC, q10 1 at 36 degC; current times
  Ci / (Ci + 0.2 mM), carried by the calcium ion)
* ``Cav3p1_MA2020_GoC`` -- channel/calcium.py:1972 (permeability g_max 2.5e-4 cm/s, temp 22 degC, q10 3 at 37 degC
  dividing the time constants; GHK drive at temp + 0.04 K); Cav3p1_MA2024_PC repeats it, the two _Frozen classes
  hold the drive out of the linearisation, and Cav3p1Test_PC24 (:2577) runs the gates with a fixed 1 mV drive
* ``Cav3p3_RI2021_SC`` -- channel/calcium.py:4033 (perm 1e-4 cm/s, g_scale 1e-5, temp 36 degC, V_sh 0; gates q10 2.3
  at 28 degC; GHK drive at temp - 0.01 K); Cav3p3_MA2024_PC repeats it and its _Frozen class holds the drive out of
  the linearisation
* ``Cav1p2_MA2020_GoC`` / ``Cav1p3_MA2020_GoC`` -- channel/calcium.py:1408, :1683 (g_max 0.2 / 0.005, temp 22 degC,
  q10 1 at 22 degC; n_inf = kf / (kf + Ci)); their MA2025_BC classes repeat them
* ``Cav2p1_RI2021_SC`` -- channel/calcium.py:2767 (permeability g_max 2.2e-4 cm/s, V_sh 0, temp 23 degC; gate q10 3 at
  23 degC; the shared GHK drive of channel/_base.py:47); the MA2024_PC and MA2025_BC classes repeat it, and the three
  _Frozen classes run the Cav3.1 model-file GHK at a stop-gradient V
* ``CaHVA_SU2015_DCN`` / ``CaLVA_SU2015_DCN`` -- channel/calcium.py:924, :1221 (perm 7.5e-6 / 1 cm/s, temp 36 degC,
  qdeltat 1; the model's drive (4.47814e6 V / T)(ci - co A) / 1000 / (1 - A), A = e^(-23.20764929 V / T); CaLVA on
  CaL_SU2015_DCN's gates)
* ``Nav_MA2020_GrC`` -- channel/sodium.py:1427 (g_max 13, temp 32 degC; phi 3^((T - 20 degC) / 10)): a Markov
  scheme on the Nav1.6 graph with its own rate constants
* ``Ca_ZH2019_IO`` / ``_Frozen`` -- channel/calcium.py:4837 (g_max 0.4, E 120 mV, mMidV -61 mV, freeze_m_inf true;
  the Frozen class pins it)

Same-form classes: Na_TM1991 has Na_Ba2002's Traub-Miles rate functions written
in terms of V_sh - V (sodium.py:275-289 against :154-170), K_TM1991 has
KDR_Ba2002's (potassium.py:331-337 against :208-214), and CaHT_HM1992 has
CaT_HM1992's (calcium.py:645-663 against :355-373); only their defaults differ.
KM_MA2020_GoC and KM_MA2020_GrC (potassium.py:4419, :5182) repeat KM_RI2021_SC's
rates, gate temperature factor and defaults.  The Markov channels' cell-type variants
repeat their base class unchanged (Nav1p6_MA2024_PC / _MA2025_BC / _RI2021_SC,
sodium.py:943-1190; Kca2p2 and Kca1p1 _MA2025_BC / _MA2020_GrC / _MA2024_PC /
_RI2021_SC, potassium_calcium.py).
Each fills the parameter record and kernel slot of its same-form class, so a
region cannot carry both classes of one pair.
* ions: ``SodiumFixed`` E 50 (ion/sodium.py:149), ``PotassiumFixed`` E -95
  (ion/potassium.py:151), ``CalciumFixed`` E 120 (ion/calcium.py:187) -- the
  defaults used when no ion is painted (_compute/ions.py:107-113);
  ``CalciumDetailed`` (ion/calcium.py:286: temp 36 degC, d 1 um, tau 5 ms,
  C_rest 2.4e-4 mM, Co 2 mM, Ci0 2.4e-4 mM); ``SodiumInitNernst``,
  ``PotassiumInitNernst`` and ``CalciumInitNernst`` (ion/_base.py:261: fixed Ci / Co,
  E = R T / (z F) ln(Co / Ci) set once, temp 36 degC and the family's Ci, Co, valence).

The gate temperature factor is ``phi = q10 ** ((temp - temp_ref) / 10 K)``
(channel/_base.py:517-532).
"""

from __future__ import annotations

import numpy as np

from . import _abi
from .mech import CableProperty, Channel, Ion, celsius2kelvin

__all__ = ["CHANNELS", "IONS", "SAME_FORM", "kernel_class", "region_record", "q10_phi"]

T36 = celsius2kelvin(36.0)
T24 = celsius2kelvin(24.0)
T22 = celsius2kelvin(22.0)
T30 = celsius2kelvin(30.0)
T37 = celsius2kelvin(37.0)
FARADAY = 96485.33212  # C/mol
GAS_R = 8.314462618  # J/(mol K)

CHANNELS: dict[str, dict[str, float]] = {
    "IL": {"g_max": 0.1, "E": -70.0},
    "K_Leak": {"g_max": 0.005},
    "Na_Ba2002": {"g_max": 90.0, "temp": T36, "q10": 3.0, "temp_ref": T36, "V_sh": -50.0},
    "KDR_Ba2002": {"g_max": 10.0, "temp": T36, "q10": 3.0, "temp_ref": T36, "V_sh": -50.0},
    "CaL_IS2008": {
        "g_max": 1.0, "temp": T36, "q10_p": 3.55, "temp_ref_p": T24, "q10_q": 3.0, "temp_ref_q": T24, "V_sh": 0.0,
    },
    "CaT_HM1992": {
        "g_max": 2.0, "temp": T36, "q10_p": 3.55, "temp_ref_p": T24, "q10_q": 3.0, "temp_ref_q": T24, "V_sh": -3.0,
    },
    "HCN_HM1992": {"g_max": 10.0, "E": 43.0, "temp": T36, "q10": 1.0, "temp_ref": T36},
    "AHP_De1994": {"n": 2.0, "g_max": 10.0, "alpha": 48.0, "beta": 0.09, "phi": 1.0},
    "Na_HH1952": {"g_max": 120.0, "temp": T36, "q10": 3.0, "temp_ref": T36, "V_sh": -45.0},
    "K_HH1952": {"g_max": 10.0, "temp": T36, "q10": 3.0, "temp_ref": T36, "V_sh": -45.0},
    "KM_RI2021_SC": {"g_max": 0.25, "temp": T30},
    "Na_TM1991": {"g_max": 120.0, "temp": T36, "q10": 1.0, "temp_ref": T36, "V_sh": -63.0},
    "K_TM1991": {"g_max": 10.0, "temp": T36, "q10": 1.0, "temp_ref": T36, "V_sh": -60.0},
    "CaHT_HM1992": {
        "g_max": 2.0, "temp": T36, "q10_p": 3.55, "temp_ref_p": T24, "q10_q": 3.0, "temp_ref_q": T24, "V_sh": 25.0,
    },
    "KM_MA2020_GoC": {"g_max": 0.25, "temp": T30},
    "KM_MA2020_GrC": {"g_max": 0.25, "temp": T30},
    "KA1_HM1992": {
        "g_max": 30.0, "temp": T36, "q10_p": 1.0, "temp_ref_p": T36, "q10_q": 1.0, "temp_ref_q": T36, "V_sh": 0.0,
    },
    "KA2_HM1992": {
        "g_max": 20.0, "temp": T36, "q10_p": 1.0, "temp_ref_p": T36, "q10_q": 1.0, "temp_ref_q": T36, "V_sh": 0.0,
    },
    "KK2A_HM1992": {
        "g_max": 10.0, "temp": T36, "q10_p": 1.0, "temp_ref_p": T36, "q10_q": 1.0, "temp_ref_q": T36, "V_sh": 0.0,
    },
    "KK2B_HM1992": {
        "g_max": 10.0, "temp": T36, "q10_p": 1.0, "temp_ref_p": T36, "q10_q": 1.0, "temp_ref_q": T36, "V_sh": 0.0,
    },
    "KNI_Ya1989": {"g_max": 0.004, "temp": T36, "q10": 1.0, "temp_ref": T36, "tau_max": 4e3, "V_sh": 0.0},
    "Nav1p6_MA2020_GoC": {"g_max": 16.0, "temp": T22},
    "Nav1p1_MA2025_BC": {"g_max": 8.0, "temp": T22, "gateCurrent": 0.0},
    "Nav1p1_RI2021_SC": {"g_max": 8.0, "temp": T22, "gateCurrent": 0.0},
    "Kca2p2_MA2020_GoC": {"g_max": 38.0, "q10_base": 3.0, "diff": 3.0, "temp": T22},
    "Kca1p1_MA2020_GoC": {"g_max": 10.0, "q10_base": 3.0, "temp": T22},
    "Kv3p4_MA2020_GoC": {"g_max": 4.0, "temp": T22},
    "Kv4p3_MA2020_GoC": {"g_max": 3.2, "temp": T22},
    "Kv1p1_MA2020_GoC": {"g_max": 4.0, "temp": T22, "gateCurrent": 0.0},
    "Kir2p3_MA2020_GrC": {"g_max": 0.9, "temp": T30},
    "HCN1_MA2020_GoC": {"g_max": 0.05, "E": -20.0, "temp": T22},
    "HCN1_MA2024_PC": {"g_max": 0.1, "E": -34.4, "temp": celsius2kelvin(23.0)},
    "CaHVA_MA2020_GoC": {"g_max": 0.46, "temp": T30},
    "Cav2p3_MA2020_GoC": {"g_max": 0.0, "temp": celsius2kelvin(34.0)},
    "Cav3p2_RI2021_SC": {"g_max": 8.0e-4, "V_sh": 0.0, "temp": T36},
    # extension channels (record entries after BC_P_EXT_MASK)
    "HCN2_MA2020_GoC": {"g_max": 0.08, "E": -20.0, "temp": T22},
    "Kv3p3_MA2024_PC": {"g_max": 5.0, "temp": T22, "gateCurrent": 0.0},
    "Kv2p2_0010_MA2020_GrC": {"g_max": 0.01, "BBiD": 10.0},
    "Kv1p5_MA2024_PC": {"g_max": 0.13195, "temp": celsius2kelvin(37.0), "Tauact": 1.0, "Tauinactf": 1.0,
                        "Tauinacts": 1.0},
    "NaF_SU2015_DCN": {"g_max": 0.01},
    "NaP_SU2015_DCN": {"g_max": 0.01},
    "Na_ZH2019_IO": {"g_max": 70.0},
    "fKdr_SU2015_DCN": {"g_max": 0.01},
    "sKdr_SU2015_DCN": {"g_max": 0.01},
    "Kdr_ZH2019_IO": {"g_max": 18.0},
    "HCN_SU2015_DCN": {"g_max": 0.01, "E": -45.0},
    "HCN_ZH2019_IO": {"g_max": 0.15, "E": -43.0},
    "CaT_HP1992": {"g_max": 1.75, "temp": T36, "q10_p": 5.0, "temp_ref_p": celsius2kelvin(24.0), "q10_q": 3.0,
                   "temp_ref_q": celsius2kelvin(24.0), "V_sh": -3.0},
    "CaHT_Re1993": {"g_max": 1.0, "temp": T36, "q10_p": 2.3, "temp_ref_p": celsius2kelvin(23.0), "q10_q": 2.3,
                    "temp_ref_q": celsius2kelvin(23.0), "V_sh": 0.0},
    "CaL_SU2015_DCN": {"g_max": 0.01, "E": 139.0, "qdeltat": 1.0},
    "Kca3p1_MA2020_GoC": {"g_max": 120.0, "q10_base": 3.0, "temp": T22},
    "SK_SU2015_DCN": {"g_max": 0.01, "qdeltat": 1.0},
    "K_Kv_test": {"g_max": 0.0, "V_sh": 0.0, "temp": celsius2kelvin(25.0), "Ra": 0.02, "Rb": 0.006, "q": 9.0,
                  "v12": 25.0},
    "CaN_IS2008": {"E": 10.0, "g_max": 1.0, "temp": T36, "q10": 1.0, "temp_ref": T36},
    "Ca_ZH2019_IO": {"g_max": 0.4, "E": 120.0, "mMidV": -61.0, "freeze_m_inf": 1.0},
    "Nav_MA2020_GrC": {"g_max": 13.0, "temp": celsius2kelvin(32.0)},
    # a permeability in cm/s (calcium.py:1972: 2.5e-4 cm/s)
    "Cav3p1_MA2020_GoC": {"g_max": 2.5e-4, "V_sh": 0.0, "temp": T22, "q10": 3.0, "temp_ref": celsius2kelvin(37.0)},
    # permeability perm in cm/s times g_scale (calcium.py:4033); no g_max parameter
    "Cav3p3_RI2021_SC": {"perm": 1.0e-4, "g_scale": 1.0e-5, "temp": T36, "V_sh": 0.0},
    # 0.0002 and 0.000005 S/cm^2 (calcium.py:1408, :1683); V_sh accepted, unused by the rates
    "Cav1p2_MA2020_GoC": {"g_max": 0.2, "V_sh": 0.0, "temp": T22, "q10": 1.0, "temp_ref": T22},
    "Cav1p3_MA2020_GoC": {"g_max": 0.005, "V_sh": 0.0, "temp": T22, "q10": 1.0, "temp_ref": T22},
    # a permeability in cm/s (calcium.py:2767: 2.2e-4 cm/s)
    "Cav2p1_RI2021_SC": {"g_max": 2.2e-4, "V_sh": 0.0, "temp": celsius2kelvin(23.0)},
    # permeabilities in cm/s (calcium.py:924, 7.5e-6; the CaLVA class, 1.0)
    "CaHVA_SU2015_DCN": {"perm": 7.5e-6, "temp": T36, "qdeltat": 1.0},
    "CaLVA_SU2015_DCN": {"perm": 1.0, "temp": T36, "qdeltat": 1.0},
}
# extension channels: class -> (BC_X_* bit, record entry of g_max, record entry of E or None)
_EXT = {
    "HCN2_MA2020_GoC": (_abi.BC_X_HCN2, _abi.BC_P_HCN2_G, _abi.BC_P_HCN2_E),
    "Kv3p3_MA2024_PC": (_abi.BC_X_KV33, _abi.BC_P_KV33_G, None),
    "Kv2p2_0010_MA2020_GrC": (_abi.BC_X_KV22, _abi.BC_P_KV22_G, None),
    "Kv1p5_MA2024_PC": (_abi.BC_X_KV15, _abi.BC_P_KV15_G, None),
    "NaF_SU2015_DCN": (_abi.BC_X_NAF, _abi.BC_P_NAF_G, None),
    "NaP_SU2015_DCN": (_abi.BC_X_NAP, _abi.BC_P_NAP_G, None),
    "Na_ZH2019_IO": (_abi.BC_X_NAIO, _abi.BC_P_NAIO_G, None),
    "fKdr_SU2015_DCN": (_abi.BC_X_FKDR, _abi.BC_P_FKDR_G, None),
    "sKdr_SU2015_DCN": (_abi.BC_X_SKDR, _abi.BC_P_SKDR_G, None),
    "Kdr_ZH2019_IO": (_abi.BC_X_KDRIO, _abi.BC_P_KDRIO_G, None),
    "HCN_SU2015_DCN": (_abi.BC_X_HCNDCN, _abi.BC_P_HCNDCN_G, _abi.BC_P_HCNDCN_E),
    "HCN_ZH2019_IO": (_abi.BC_X_HCNIO, _abi.BC_P_HCNIO_G, _abi.BC_P_HCNIO_E),
    "CaT_HP1992": (_abi.BC_X_CATHP, _abi.BC_P_CATHP_G, None),
    "CaHT_Re1993": (_abi.BC_X_CAHTRE, _abi.BC_P_CAHTRE_G, None),
    "CaL_SU2015_DCN": (_abi.BC_X_CALDCN, _abi.BC_P_CALDCN_G, _abi.BC_P_CALDCN_E),
    "Kca3p1_MA2020_GoC": (_abi.BC_X_KCA31, _abi.BC_P_KCA31_G, None),
    "SK_SU2015_DCN": (_abi.BC_X_SKDCN, _abi.BC_P_SKDCN_G, None),
    "K_Kv_test": (_abi.BC_X_KKV, _abi.BC_P_KKV_G, None),
    "CaN_IS2008": (_abi.BC_X_CAN, _abi.BC_P_CAN_G, _abi.BC_P_CAN_E),
    "Ca_ZH2019_IO": (_abi.BC_X_CAIO, _abi.BC_P_CAIO_G, _abi.BC_P_CAIO_E),
    "Nav_MA2020_GrC": (_abi.BC_X_NAVGRC, _abi.BC_P_NAVGRC_G, None),
    "Cav3p1_MA2020_GoC": (_abi.BC_X_CAV31, _abi.BC_P_CAV31_G, None),
    "Cav3p3_RI2021_SC": (_abi.BC_X_CAV33, _abi.BC_P_CAV33_G, None),
    "Cav1p2_MA2020_GoC": (_abi.BC_X_CAV12, _abi.BC_P_CAV12_G, None),
    "Cav1p3_MA2020_GoC": (_abi.BC_X_CAV13, _abi.BC_P_CAV13_G, None),
    "Cav2p1_RI2021_SC": (_abi.BC_X_CAV21, _abi.BC_P_CAV21_G, None),
    "CaHVA_SU2015_DCN": (_abi.BC_X_CAHVADCN, _abi.BC_P_CAHVADCN_G, None),
    "CaLVA_SU2015_DCN": (_abi.BC_X_CALVADCN, _abi.BC_P_CALVADCN_G, None),
}
# Cav3p1 classes with the GHK drive frozen for the linearisation (calcium.py, the
# _Frozen subclasses: the forward current is the base class's)
_GHK_FROZEN = ("Cav3p1_MA2020_GoC_Frozen", "Cav3p1_MA2024_PC_Frozen", "Cav3p3_MA2024_PC_Frozen",
               "Cav2p1_MA2024_PC_Frozen", "Cav2p1_MA2025_BC_Frozen", "Cav2p1_RI2021_SC_Frozen")
# cell-type variants with their base class's kinetics; own defaults where they differ
KINETIC_VARIANTS = {
    "Kv3p4_MA2020_GoC": {v: {} for v in ("Kv3p4_MA2020_GrC", "Kv3p4_MA2024_PC", "Kv3p4_MA2025_BC", "Kv3p4_RI2021_SC")},
    "Kv4p3_MA2020_GoC": {v: {"temp": T30} for v in ("Kv4p3_MA2020_GrC", "Kv4p3_MA2024_PC", "Kv4p3_MA2025_BC",
                                                      "Kv4p3_RI2021_SC")},
    "Kv1p1_MA2020_GoC": {v: {} for v in ("Kv1p1_MA2020_GrC", "Kv1p1_MA2024_PC", "Kv1p1_MA2025_BC", "Kv1p1_RI2021_SC")},
    "Kir2p3_MA2020_GrC": {v: {} for v in ("Kir2p3_MA2024_PC", "Kir2p3_MA2025_BC", "Kir2p3_RI2021_SC")},
    "HCN1_MA2024_PC": {v: {} for v in ("HCN1_MA2025_BC", "HCN1_RI2021_SC")},
    "CaHVA_MA2020_GoC": {"CaHVA_MA2020_GrC": {}},
    "Cav3p2_RI2021_SC": {v: {} for v in ("Cav3p2_MA2025_BC", "Cav3p2_MA2024_PC")},
    "Kca3p1_MA2020_GoC": {v: {} for v in ("Kca3p1_MA2025_BC", "Kca3p1_MA2024_PC")},
    "Cav1p2_MA2020_GoC": {"Cav1p2_MA2025_BC": {}},
    "Cav1p3_MA2020_GoC": {"Cav1p3_MA2025_BC": {}},
    "Cav2p1_RI2021_SC": {v: {} for v in ("Cav2p1_MA2024_PC", "Cav2p1_MA2025_BC")},
}
MARKOV_VARIANTS = {
    "Nav1p6_MA2020_GoC": ("Nav1p6_MA2024_PC", "Nav1p6_MA2025_BC", "Nav1p6_RI2021_SC"),
    "Kca2p2_MA2020_GoC": ("Kca2p2_MA2025_BC", "Kca2p2_MA2020_GrC", "Kca2p2_MA2024_PC", "Kca2p2_RI2021_SC"),
    "Kca1p1_MA2020_GoC": ("Kca1p1_MA2025_BC", "Kca1p1_MA2020_GrC", "Kca1p1_MA2024_PC", "Kca1p1_RI2021_SC"),
}
# class -> the class whose kernel (rate functions, parameter slots, states) it uses
SAME_FORM = {"Na_TM1991": "Na_Ba2002", "K_TM1991": "KDR_Ba2002", "CaHT_HM1992": "CaT_HM1992",
             "KM_MA2020_GoC": "KM_RI2021_SC", "KM_MA2020_GrC": "KM_RI2021_SC"}
for _base, _variants in MARKOV_VARIANTS.items():
    for _v in _variants:
        CHANNELS[_v] = dict(CHANNELS[_base])
        SAME_FORM[_v] = _base
for _base, _variants in KINETIC_VARIANTS.items():
    for _v, _own in _variants.items():
        CHANNELS[_v] = {**CHANNELS[_base], **_own}
        SAME_FORM[_v] = _base
# Kv1p5_MA2020_GrC (potassium_sodium.py:38-259) is Kv1p5_MA2024_PC's kinetics and K
# current plus a nonspecific current of conductance gnonspec, 0 by default; only
# gnonspec = 0 is built
CHANNELS["Kv1p5_MA2020_GrC"] = {**CHANNELS["Kv1p5_MA2024_PC"], "gnonspec": 0.0}
SAME_FORM["Kv1p5_MA2020_GrC"] = "Kv1p5_MA2024_PC"
# Cav3p1_MA2024_PC overrides nothing of Cav3p1_MA2020_GoC; the _Frozen classes differ
# only in the linearisation
for _v in ("Cav3p1_MA2024_PC", "Cav3p1_MA2020_GoC_Frozen", "Cav3p1_MA2024_PC_Frozen"):
    CHANNELS[_v] = dict(CHANNELS["Cav3p1_MA2020_GoC"])
    SAME_FORM[_v] = "Cav3p1_MA2020_GoC"
# Cav3p1Test_PC24 (calcium.py:2577): Cav3p1's gates, g_max in mS/cm^2 (2.5e-4 S/cm^2), a
# fixed 1 mV drive
CHANNELS["Cav3p1Test_PC24"] = {"g_max": 0.25, "temp": T22, "q10": 3.0, "temp_ref": celsius2kelvin(37.0)}
SAME_FORM["Cav3p1Test_PC24"] = "Cav3p1_MA2020_GoC"
# Cav3p3_MA2024_PC overrides nothing of Cav3p3_RI2021_SC; its _Frozen class differs only
# in the linearisation
for _v in ("Cav3p3_MA2024_PC", "Cav3p3_MA2024_PC_Frozen"):
    CHANNELS[_v] = dict(CHANNELS["Cav3p3_RI2021_SC"])
    SAME_FORM[_v] = "Cav3p3_RI2021_SC"
# the Cav2p1 _Frozen classes: Cav2p1's gates and defaults, the Cav3.1 model-file GHK at a
# stop-gradient V (their record differs from the base class's in the drive entries)
for _v in ("Cav2p1_MA2024_PC_Frozen", "Cav2p1_MA2025_BC_Frozen", "Cav2p1_RI2021_SC_Frozen"):
    CHANNELS[_v] = dict(CHANNELS["Cav2p1_RI2021_SC"])
    SAME_FORM[_v] = "Cav2p1_RI2021_SC"
# Ca_ZH2019_IO_Frozen (calcium.py) is Ca_ZH2019_IO with freeze_m_inf pinned to True
CHANNELS["Ca_ZH2019_IO_Frozen"] = dict(CHANNELS["Ca_ZH2019_IO"])
SAME_FORM["Ca_ZH2019_IO_Frozen"] = "Ca_ZH2019_IO"
# classes with a parameter record of their own on another class's kernel mechanism
_SHARED_KERNEL = {"Nav1p1_MA2025_BC": "Nav1p6_MA2020_GoC", "Nav1p1_RI2021_SC": "Nav1p6_MA2020_GoC"}
# gate temperature factors fixed by a class (not constructor parameters)
KM_Q10, KM_TEMP_REF = 3.0, T22
_ALIASES = {"leaky": "IL"}

IONS: dict[str, dict[str, float]] = {
    "SodiumFixed": {"E": 50.0},
    "PotassiumFixed": {"E": -95.0},
    "CalciumFixed": {"E": 120.0},
    "CalciumDetailed": {
        "temp": T36, "d": 1.0, "tau": 5.0, "C_rest": 2.4e-4, "Co": 2.0, "Ci_initializer": 2.4e-4,
    },
    # fixed Ci / Co with E set once from Nernst at init and reset (ion/_base.py:261-360);
    # the family defaults Ci, Co, valence: ion/sodium.py:82-84, ion/potassium.py:83-85,
    # ion/calcium.py:120-122, temp 36 C (ion/sodium.py:235)
    "SodiumInitNernst": {"temp": T36, "Ci": 10.0, "Co": 140.0, "valence": 1.0},
    "PotassiumInitNernst": {"temp": T36, "Ci": 54.4, "Co": 2.5, "valence": 1.0},
    "CalciumInitNernst": {"temp": T36, "Ci": 5e-5, "Co": 2.0, "valence": 2.0},
}
# the reversal-potential slot each fixed-E ion family sets
_E_SLOT = {"SodiumFixed": _abi.BC_P_ENA, "PotassiumFixed": _abi.BC_P_EK, "CalciumFixed": _abi.BC_P_ECA,
           "SodiumInitNernst": _abi.BC_P_ENA, "PotassiumInitNernst": _abi.BC_P_EK,
           "CalciumInitNernst": _abi.BC_P_ECA}


def nernst_mV(temp: float, valence: float, Co: float, Ci: float) -> float:
    """R T / (z F) ln(Co / Ci) in mV, the stored E of an InitNernst ion
    (ion/_base.py:350-356)."""
    if not (Co > 0.0 and Ci > 0.0) or valence == 0.0:
        raise ValueError(f"Nernst potential needs Co > 0, Ci > 0 and valence != 0 (got {Co}, {Ci}, {valence}).")
    return 1e3 * GAS_R * float(temp) / (float(valence) * FARADAY) * float(np.log(Co / Ci))


# classes whose record is (g_max, V_sh, phi_p, phi_q) at a base index: mechanism bit, base
_PQ_RECORDS = {
    "KA1_HM1992": (_abi.BC_M_KA1, _abi.BC_P_KA1_G), "KA2_HM1992": (_abi.BC_M_KA2, _abi.BC_P_KA2_G),
    "KK2A_HM1992": (_abi.BC_M_KK2A, _abi.BC_P_KK2A_G), "KK2B_HM1992": (_abi.BC_M_KK2B, _abi.BC_P_KK2B_G),
}


def ext_mask(rec) -> int:
    """The BC_X_* bits a record lists (BC_P_EXT_MASK, and BC_P_EXT_MASK_HI for bits 24 up)."""
    return int(rec[_abi.BC_P_EXT_MASK]) | (int(rec[_abi.BC_P_EXT_MASK_HI]) << 24)


def kernel_class(name: str) -> str:
    """The class whose kernel a channel class runs on (itself unless same-form)."""
    return SAME_FORM.get(name, name)


def q10_phi(q10: float, temp: float, temp_ref: float) -> float:
    return float(q10) ** ((float(temp) - float(temp_ref)) / 10.0)


def _params(table: dict, name: str, decl) -> dict[str, float]:
    out = dict(table[name])
    for k, v in decl.params.items():
        if k not in out:
            raise ValueError(f"{name} has no parameter {k!r}; known: {sorted(out)}.")
        out[k] = float(v)
    return out


def region_record(mechs, cable: CableProperty) -> tuple[int, np.ndarray]:
    """Return ``(mechanism_bits, params[BC_NPARAM])`` for one region.

    ``mechs`` is the ordered list of Channel / Ion declarations painted on the
    region; a later declaration of the same class replaces an earlier one.
    """
    rec = np.zeros(_abi.BC_NPARAM, dtype=np.float64)
    rec[_abi.BC_P_INVCM] = 1.0 / float(cable.membrane_capacitance)
    rec[_abi.BC_P_VREST] = float(cable.resting_potential)
    rec[_abi.BC_P_ENA] = IONS["SodiumFixed"]["E"]
    rec[_abi.BC_P_EK] = IONS["PotassiumFixed"]["E"]
    rec[_abi.BC_P_ECA] = IONS["CalciumFixed"]["E"]
    bits = 0
    kernel_owner: dict[str, str] = {}
    last: dict[str, object] = {}
    for m in mechs:
        last[m.class_name if m.class_name not in _ALIASES else _ALIASES[m.class_name]] = m
    for name, decl in last.items():
        if isinstance(decl, Ion):
            if name not in IONS:
                raise ValueError(f"Unsupported ion class {name!r}; supported: {sorted(IONS)}.")
            p = _params(IONS, name, decl)
            if name in _E_SLOT:
                rec[_E_SLOT[name]] = p["E"] if "E" in p else nernst_mV(p["temp"], p["valence"], p["Co"], p["Ci"])
            else:
                bits |= _abi.BC_M_CADET
                rec[_abi.BC_P_CA_D] = p["d"]
                rec[_abi.BC_P_CA_TAU] = p["tau"]
                rec[_abi.BC_P_CA_CREST] = p["C_rest"]
                rec[_abi.BC_P_CA_CO] = p["Co"]
                rec[_abi.BC_P_CA_TEMP] = p["temp"]
                rec[_abi.BC_P_CA_CI0] = p["Ci_initializer"]
            continue
        if not isinstance(decl, Channel):
            raise TypeError(f"Expected Channel or Ion declaration, got {type(decl).__name__}.")
        if name not in CHANNELS:
            raise ValueError(f"Unsupported channel class {name!r}; supported: {sorted(CHANNELS)}.")
        p = _params(CHANNELS, name, decl)
        kname = kernel_class(name)
        owner_key = _SHARED_KERNEL.get(kname, kname)
        if owner_key in kernel_owner:
            raise ValueError(f"{name} and {kernel_owner[owner_key]} run on the same kernel mechanism and cannot be "
                             "painted on one region.")
        kernel_owner[owner_key] = name
        name = kname
        if name == "IL":
            bits |= _abi.BC_M_IL
            rec[_abi.BC_P_IL_G], rec[_abi.BC_P_IL_E] = p["g_max"], p["E"]
        elif name == "K_Leak":
            bits |= _abi.BC_M_KLEAK
            rec[_abi.BC_P_KLEAK_G] = p["g_max"]
        elif name == "Na_Ba2002":
            bits |= _abi.BC_M_NA
            rec[_abi.BC_P_NA_G], rec[_abi.BC_P_NA_VSH] = p["g_max"], p["V_sh"]
            rec[_abi.BC_P_NA_PHI] = q10_phi(p["q10"], p["temp"], p["temp_ref"])
        elif name == "KDR_Ba2002":
            bits |= _abi.BC_M_KDR
            rec[_abi.BC_P_KDR_G], rec[_abi.BC_P_KDR_VSH] = p["g_max"], p["V_sh"]
            rec[_abi.BC_P_KDR_PHI] = q10_phi(p["q10"], p["temp"], p["temp_ref"])
        elif name == "CaL_IS2008":
            bits |= _abi.BC_M_CAL
            rec[_abi.BC_P_CAL_G], rec[_abi.BC_P_CAL_VSH] = p["g_max"], p["V_sh"]
            rec[_abi.BC_P_CAL_PHIP] = q10_phi(p["q10_p"], p["temp"], p["temp_ref_p"])
            rec[_abi.BC_P_CAL_PHIQ] = q10_phi(p["q10_q"], p["temp"], p["temp_ref_q"])
        elif name == "CaT_HM1992":
            bits |= _abi.BC_M_CAT
            rec[_abi.BC_P_CAT_G], rec[_abi.BC_P_CAT_VSH] = p["g_max"], p["V_sh"]
            rec[_abi.BC_P_CAT_PHIP] = q10_phi(p["q10_p"], p["temp"], p["temp_ref_p"])
            rec[_abi.BC_P_CAT_PHIQ] = q10_phi(p["q10_q"], p["temp"], p["temp_ref_q"])
        elif name == "HCN_HM1992":
            bits |= _abi.BC_M_HCN
            rec[_abi.BC_P_HCN_G], rec[_abi.BC_P_HCN_E] = p["g_max"], p["E"]
            rec[_abi.BC_P_HCN_PHI] = q10_phi(p["q10"], p["temp"], p["temp_ref"])
        elif name == "AHP_De1994":
            bits |= _abi.BC_M_AHP
            rec[_abi.BC_P_AHP_G], rec[_abi.BC_P_AHP_N] = p["g_max"], p["n"]
            rec[_abi.BC_P_AHP_ALPHA], rec[_abi.BC_P_AHP_BETA] = p["alpha"], p["beta"]
            rec[_abi.BC_P_AHP_PHI] = p["phi"]
        elif name == "Na_HH1952":
            bits |= _abi.BC_M_NAHH
            rec[_abi.BC_P_NAHH_G], rec[_abi.BC_P_NAHH_VSH] = p["g_max"], p["V_sh"]
            rec[_abi.BC_P_NAHH_PHI] = q10_phi(p["q10"], p["temp"], p["temp_ref"])
        elif name == "K_HH1952":
            bits |= _abi.BC_M_KHH
            rec[_abi.BC_P_KHH_G], rec[_abi.BC_P_KHH_VSH] = p["g_max"], p["V_sh"]
            rec[_abi.BC_P_KHH_PHI] = q10_phi(p["q10"], p["temp"], p["temp_ref"])
        elif name == "KM_RI2021_SC":
            bits |= _abi.BC_M_KM
            rec[_abi.BC_P_KM_G] = p["g_max"]
            rec[_abi.BC_P_KM_PHI] = q10_phi(KM_Q10, p["temp"], KM_TEMP_REF)
        elif name == "KNI_Ya1989":
            bits |= _abi.BC_M_KNI
            rec[_abi.BC_P_KNI_G], rec[_abi.BC_P_KNI_VSH] = p["g_max"], p["V_sh"]
            rec[_abi.BC_P_KNI_PHI] = q10_phi(p["q10"], p["temp"], p["temp_ref"])
            rec[_abi.BC_P_KNI_TAUMAX] = p["tau_max"]
        elif name == "Nav1p6_MA2020_GoC":
            bits |= _abi.BC_M_NAV16
            rec[_abi.BC_P_NAV16_G] = p["g_max"]
            rec[_abi.BC_P_NAV16_PHI] = q10_phi(3.0, p["temp"], T22)
            rec[_abi.BC_P_NAV16_OON], rec[_abi.BC_P_NAV16_EPS] = 0.75, 1.75
            rec[_abi.BC_P_NAV16_ALFAC] = (0.75 / 0.005) ** 0.25
        elif name in ("Nav1p1_MA2025_BC", "Nav1p1_RI2021_SC"):
            # the Nav1.6 scheme with Oon 2.3, epsilon 1e-12 and phi 2.7^((T - 22 degC) / 10)
            if p["gateCurrent"] != 0.0:
                raise ValueError(f"{decl.class_name}: the gating current (gateCurrent != 0) is not built.")
            bits |= _abi.BC_M_NAV16
            rec[_abi.BC_P_NAV16_G] = p["g_max"]
            rec[_abi.BC_P_NAV16_PHI] = q10_phi(2.7, p["temp"], T22)
            rec[_abi.BC_P_NAV16_OON], rec[_abi.BC_P_NAV16_EPS] = 2.3, 1e-12
            rec[_abi.BC_P_NAV16_ALFAC] = (2.3 / 0.005) ** 0.25
        elif name == "Kca2p2_MA2020_GoC":
            bits |= _abi.BC_M_KCA22
            rec[_abi.BC_P_KCA22_G], rec[_abi.BC_P_KCA22_DIFF] = p["g_max"], p["diff"]
            rec[_abi.BC_P_KCA22_PHI] = q10_phi(p["q10_base"], p["temp"], celsius2kelvin(23.0))
        elif name == "Kca1p1_MA2020_GoC":
            bits |= _abi.BC_M_KCA11
            rec[_abi.BC_P_KCA11_G] = p["g_max"]
            rec[_abi.BC_P_KCA11_PHI] = q10_phi(p["q10_base"], p["temp"], celsius2kelvin(23.0))
            rec[_abi.BC_P_KCA11_QO] = 0.73 * FARADAY * 1e-3 / (GAS_R * p["temp"])
            rec[_abi.BC_P_KCA11_QC] = -0.67 * FARADAY * 1e-3 / (GAS_R * p["temp"])
        elif name == "Kv3p4_MA2020_GoC":
            bits |= _abi.BC_M_KV34
            rec[_abi.BC_P_KV34_G] = p["g_max"]
            rec[_abi.BC_P_KV34_PHI] = q10_phi(3.0, p["temp"], T37)
        elif name == "Kv4p3_MA2020_GoC":
            bits |= _abi.BC_M_KV43
            rec[_abi.BC_P_KV43_G] = p["g_max"]
            rec[_abi.BC_P_KV43_PHI] = q10_phi(3.0, p["temp"], celsius2kelvin(25.5))
        elif name == "Kv1p1_MA2020_GoC":
            if p["gateCurrent"] != 0.0:
                raise ValueError(f"{decl.class_name}: the gating current (gateCurrent != 0) is not built.")
            bits |= _abi.BC_M_KV11
            rec[_abi.BC_P_KV11_G] = p["g_max"]
            rec[_abi.BC_P_KV11_PHI] = q10_phi(2.7, p["temp"], T22)
        elif name == "Kir2p3_MA2020_GrC":
            bits |= _abi.BC_M_KIR23
            rec[_abi.BC_P_KIR23_G] = p["g_max"]
            rec[_abi.BC_P_KIR23_PHI] = q10_phi(3.0, p["temp"], celsius2kelvin(20.0))
        elif name == "HCN1_MA2020_GoC":
            bits |= _abi.BC_M_HCN1F
            rec[_abi.BC_P_HCN1F_G] = p["g_max"] * q10_phi(1.5, p["temp"], celsius2kelvin(23.0))
            rec[_abi.BC_P_HCN1F_E] = p["E"]
            rec[_abi.BC_P_HCN1F_PHI] = q10_phi(3.0, p["temp"], celsius2kelvin(23.0))
        elif name == "HCN1_MA2024_PC":
            bits |= _abi.BC_M_HCN1H
            rec[_abi.BC_P_HCN1H_G], rec[_abi.BC_P_HCN1H_E] = p["g_max"], p["E"]
            rec[_abi.BC_P_HCN1H_PHI] = q10_phi(3.0, p["temp"], T37)
        elif name == "CaHVA_MA2020_GoC":
            bits |= _abi.BC_M_CAHVA
            rec[_abi.BC_P_CAHVA_G] = p["g_max"]
            rec[_abi.BC_P_CAHVA_PHI] = q10_phi(3.0, p["temp"], celsius2kelvin(20.0))
        elif name == "Cav2p3_MA2020_GoC":
            bits |= _abi.BC_M_CAV23
            rec[_abi.BC_P_CAV23_G] = p["g_max"]
        elif name == "Cav3p2_RI2021_SC":
            bits |= _abi.BC_M_CAV32
            rec[_abi.BC_P_CAV32_G], rec[_abi.BC_P_CAV32_VSH] = p["g_max"], p["V_sh"]
        elif name in _EXT:
            xbit, g_slot, e_slot = _EXT[name]
            bits |= _abi.BC_M_EXT
            mask = ext_mask(rec) | xbit  # two record reals, each exact in FP32
            rec[_abi.BC_P_EXT_MASK], rec[_abi.BC_P_EXT_MASK_HI] = float(mask & 0xFFFFFF), float(mask >> 24)
            g = p["g_scale"] * p["perm"] if name == "Cav3p3_RI2021_SC" else \
                (p["perm"] if name in ("CaHVA_SU2015_DCN", "CaLVA_SU2015_DCN") else p["g_max"])
            if name == "HCN2_MA2020_GoC":  # the conductance's own Q10 1.5 and the gates' q10 3, at 23 degC
                g *= q10_phi(1.5, p["temp"], celsius2kelvin(23.0))
                rec[_abi.BC_P_HCN2_PHI] = q10_phi(3.0, p["temp"], celsius2kelvin(23.0))
            elif name == "Kv3p3_MA2024_PC":
                if p["gateCurrent"] != 0.0:
                    raise ValueError(f"{decl.class_name}: the gating current (gateCurrent != 0) is not built.")
                rec[_abi.BC_P_KV33_PHI] = q10_phi(2.7, p["temp"], T22)
            elif name == "Kv1p5_MA2024_PC":
                if p.get("gnonspec", 0.0) != 0.0:
                    raise ValueError(f"{decl.class_name}: the nonspecific current (gnonspec != 0) is not built.")
                rec[_abi.BC_P_KV15_Q10] = q10_phi(2.2, p["temp"], celsius2kelvin(37.0))
                rec[_abi.BC_P_KV15_TACT] = p["Tauact"]
                rec[_abi.BC_P_KV15_TINF] = p["Tauinactf"]
                rec[_abi.BC_P_KV15_TINS] = p["Tauinacts"]
            elif name in ("CaT_HP1992", "CaHT_Re1993"):
                base = g_slot
                rec[base + 1] = p["V_sh"]
                rec[base + 2] = q10_phi(p["q10_p"], p["temp"], p["temp_ref_p"])
                rec[base + 3] = q10_phi(p["q10_q"], p["temp"], p["temp_ref_q"])
            elif name in ("CaHVA_SU2015_DCN", "CaLVA_SU2015_DCN"):
                if p["qdeltat"] != 1.0:
                    raise ValueError(f"{decl.class_name}: qdeltat other than 1 is not built.")
                rec[_abi.BC_P_CAHVADCN_T if name == "CaHVA_SU2015_DCN" else _abi.BC_P_CALVADCN_T] = p["temp"]
            elif name in ("CaL_SU2015_DCN", "SK_SU2015_DCN") and p["qdeltat"] != 1.0:
                raise ValueError(f"{decl.class_name}: qdeltat other than 1 is not built.")
            elif name == "CaN_IS2008":
                rec[_abi.BC_P_CAN_PHI] = q10_phi(p["q10"], p["temp"], p["temp_ref"])
            elif name == "Cav3p1_MA2020_GoC":
                rec[_abi.BC_P_CAV31_QT] = q10_phi(p["q10"], p["temp"], p["temp_ref"])
                rec[_abi.BC_P_CAV31_TGHK] = p["temp"] + 0.04  # the model file's Kelvin offset
                rec[_abi.BC_P_CAV31_FREEZE] = 2.0 if decl.class_name == "Cav3p1Test_PC24" else \
                    (1.0 if decl.class_name in _GHK_FROZEN else 0.0)
            elif name == "Cav3p3_RI2021_SC":
                rec[_abi.BC_P_CAV33_PHI] = q10_phi(2.3, p["temp"], celsius2kelvin(28.0))
                rec[_abi.BC_P_CAV33_TGHK] = p["temp"] - 0.01  # the model file's Kelvin offset
                rec[_abi.BC_P_CAV33_VSH] = p["V_sh"]
                rec[_abi.BC_P_CAV33_FREEZE] = 1.0 if decl.class_name in _GHK_FROZEN else 0.0
            elif name in ("Cav1p2_MA2020_GoC", "Cav1p3_MA2020_GoC"):
                rec[_abi.BC_P_CAV12_PHI if name == "Cav1p2_MA2020_GoC" else _abi.BC_P_CAV13_PHI] = \
                    q10_phi(p["q10"], p["temp"], p["temp_ref"])
            elif name == "Cav2p1_RI2021_SC":  # Gate q10 3 at 23 degC; the shared GHK at temp
                rec[_abi.BC_P_CAV21_VSH] = p["V_sh"]
                rec[_abi.BC_P_CAV21_PHI] = q10_phi(3.0, p["temp"], celsius2kelvin(23.0))
                # the _Frozen classes' drive is the Cav3.1 model-file GHK (at T + 0.04 K)
                frozen = decl.class_name in _GHK_FROZEN
                rec[_abi.BC_P_CAV21_TGHK] = p["temp"] + (0.04 if frozen else 0.0)
                rec[_abi.BC_P_CAV21_FROZEN] = 1.0 if frozen else 0.0
            elif name == "Nav_MA2020_GrC":  # phi = 3^((T - 20 degC) / 10) (sodium.py, __init__)
                rec[_abi.BC_P_NAVGRC_PHI] = q10_phi(3.0, p["temp"], celsius2kelvin(20.0))
            elif name == "Ca_ZH2019_IO":
                rec[_abi.BC_P_CAIO_MID] = p["mMidV"]
                frozen = decl.class_name == "Ca_ZH2019_IO_Frozen" or bool(p["freeze_m_inf"])
                rec[_abi.BC_P_CAIO_FREEZE] = 1.0 if frozen else 0.0
            elif name == "K_Kv_test":
                if p["q"] == 0.0:
                    raise ValueError(f"{decl.class_name}: q must not be 0.")
                for k, slot in (("V_sh", _abi.BC_P_KKV_VSH), ("Ra", _abi.BC_P_KKV_RA), ("Rb", _abi.BC_P_KKV_RB),
                                ("q", _abi.BC_P_KKV_Q), ("v12", _abi.BC_P_KKV_V12)):
                    rec[slot] = p[k]
            rec[g_slot] = g
            if e_slot is not None:
                rec[e_slot] = p["E"]
        elif name in _PQ_RECORDS:
            bit, base = _PQ_RECORDS[name]
            bits |= bit
            rec[base], rec[base + 1] = p["g_max"], p["V_sh"]
            rec[base + 2] = q10_phi(p["q10_p"], p["temp"], p["temp_ref_p"])
            rec[base + 3] = q10_phi(p["q10_q"], p["temp"], p["temp_ref_q"])
    ci_gated = bits & (_abi.BC_M_AHP | _abi.BC_M_KCA22 | _abi.BC_M_KCA11) or \
        ext_mask(rec) & (_abi.BC_X_KCA31 | _abi.BC_X_SKDCN | _abi.BC_X_CAN | _abi.BC_X_CAV31 |
                                         _abi.BC_X_CAV33 | _abi.BC_X_CAV12 | _abi.BC_X_CAV13 | _abi.BC_X_CAV21 |
                                         _abi.BC_X_CAHVADCN | _abi.BC_X_CALVADCN)
    if ext_mask(rec) & (_abi.BC_X_CAV31 | _abi.BC_X_CAV33 | _abi.BC_X_CAV21 | _abi.BC_X_CAHVADCN |
                        _abi.BC_X_CALVADCN) and \
            not bits & _abi.BC_M_CADET:
        rec[_abi.BC_P_CA_CO] = 2.0  # the GHK drive's Co: the fixed calcium ion's (ion/calcium.py:121)
    if ci_gated and not bits & _abi.BC_M_CADET:
        # AHP and the Kca channels read Ci from the calcium ion; with a fixed Ca ion
        # Ci is the class default.
        rec[_abi.BC_P_CA_CI0] = 5e-5
        rec[_abi.BC_P_CA_CREST] = 5e-5
    return bits, rec
