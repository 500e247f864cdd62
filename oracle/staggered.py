"""CPU float64 restatement of the reference staggered Cell step -- the oracle.

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` as the checker; never by the product.

Parity status: the reference (JAX + brainstate + brainunit) cannot be imported in
this build environment and ships no stored traces for the full Cell solve, so the
end-to-end solve is **parity unpinned**.  The pieces below are pinned against the
reference's own known-answer tests (see ``tests/test_oracle_pins.py``): frustum
clipping / area / axial factor / midpoint radius (``_discretization/geometry_test.py``),
peel levels and schedule groups (``_compute/scheduling_test.py``), recursive-doubling
indices (``quad/_staggered_test.py:182-200``), gate rate known answers and Q10
factors (``channel/*_test.py``), and the step-level behaviours the reference tests
assert (clamp raises V, population widening is neutral, replicas are identical).

Restated algorithm, in the reference's order:

* geometry -- ``_discretization/geometry.py:214-336`` (frusta, lateral area),
  ``:339-349`` (axial factor), ``:352-376`` (midpoint radius), ``:382-434`` (split),
  ``:614-736`` (per-CV assembly); ``_discretization/base.py:530-559`` (R = Ra * factor);
* node tree -- ``_discretization/node_build.py:58-285`` (midpoints + root endpoint +
  one terminal per branch; edge roles), ``:352-371`` (attachment node);
* scheduling -- ``_compute/scheduling.py:45-213`` (peel levels, row order, groups);
* DHS static source -- ``quad/_staggered.py:323-390`` (axial operator),
  ``:546-593`` (edge conductance, row capacitance), ``:596-612`` (edge order),
  ``:726-739`` (recursive-doubling table);
* one step -- ``quad/_staggered.py:54-154`` with ``cell.py:2261-2280`` (cached ion
  current), ``:763-795`` + ``cell.py:1907-1963`` (linearisation), ``:449-543``
  (numeric state, edge clamps, restore), ``:641-657`` (forward elimination),
  ``:742-760`` (back-substitution), ``cell.py:2157-2217`` (family order: ion self
  states, then channels) and ``quad/_exp_euler.py:330-478`` (y += dt*exprel(dt*l)*f);
* mechanisms -- ``channel/_base.py:517-674`` (HH template), the channel files named
  in :data:`CHANNEL_DEFAULTS`, ``ion/_base.py:463-506`` and ``ion/calcium.py:499-505``.

Where the reference differentiates with ``vector_grad`` the oracle writes the
derivative in closed form: every config current is ohmic in V with the gates held
fixed, so dI/dV = -sum(g * prod(x^p)), and every gate/Ci right-hand side is affine
in its own state, so d f / d x is the coefficient of x.

Units: um, mV, ms, nA, mS/cm^2 (so g*(E-V) is uA/cm^2 and dV/dt = I/cm in mV/ms),
uF/cm^2, ohm*cm, K, mM.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from oracle import markov as MK

__all__ = [
    "OracleCell",
    "Frustum",
    "build_frusta",
    "insert_radius_jumps",
    "lateral_area_um2",
    "axial_factor_per_cm",
    "midpoint_radius_um",
    "split_frusta",
    "compute_peel_levels",
    "build_backsub_indices",
    "exprel",
    "exp_euler",
    "gate_step",
    "nernst_ca_mV",
    "ca_detailed_rate",
    "rates",
    "CHANNEL_DEFAULTS",
    "ION_DEFAULTS",
]

EPS_PARAM = 1e-9
EPS_LEN_UM = 1e-6
FARADAY = 96485.33212  # C/mol (CODATA 2018)
GAS_R = 8.314462618  # J/(mol K)


def _c2k(c: float) -> float:
    return c + 273.15


# Defaults restated from the reference constructors.
CHANNEL_DEFAULTS = {
    "IL": dict(g_max=0.1, E=-70.0),  # channel/leaky.py:183-190
    "K_Leak": dict(g_max=0.005),  # channel/potassium.py:1210-1216
    "Na_Ba2002": dict(g_max=90.0, temp=_c2k(36.0), q10=3.0, temp_ref=_c2k(36.0), V_sh=-50.0),  # sodium.py:139-148
    "KDR_Ba2002": dict(g_max=10.0, temp=_c2k(36.0), q10=3.0, temp_ref=_c2k(36.0), V_sh=-50.0),  # potassium.py:191-200
    "CaL_IS2008": dict(g_max=1.0, temp=_c2k(36.0), q10_p=3.55, temp_ref_p=_c2k(24.0), q10_q=3.0,
                       temp_ref_q=_c2k(24.0), V_sh=0.0),  # calcium.py:(CaL __init__)
    "CaT_HM1992": dict(g_max=2.0, temp=_c2k(36.0), q10_p=3.55, temp_ref_p=_c2k(24.0), q10_q=3.0,
                       temp_ref_q=_c2k(24.0), V_sh=-3.0),  # calcium.py:(CaT __init__)
    "HCN_HM1992": dict(g_max=10.0, E=43.0, temp=_c2k(36.0), q10=1.0, temp_ref=_c2k(36.0)),  # hyperpol..:104-112
    "AHP_De1994": dict(n=2.0, g_max=10.0, alpha=48.0, beta=0.09, phi=1.0),  # potassium_calcium.py:163-172
    "Na_HH1952": dict(g_max=120.0, temp=_c2k(36.0), q10=3.0, temp_ref=_c2k(36.0), V_sh=-45.0),  # sodium.py:371-380
    "K_HH1952": dict(g_max=10.0, temp=_c2k(36.0), q10=3.0, temp_ref=_c2k(36.0), V_sh=-45.0),  # potassium.py:433-441
    "KM_RI2021_SC": dict(g_max=0.25, temp=_c2k(30.0)),  # potassium.py:1716-1721
    "Na_TM1991": dict(g_max=120.0, temp=_c2k(36.0), q10=1.0, temp_ref=_c2k(36.0), V_sh=-63.0),  # sodium.py:261-265
    "K_TM1991": dict(g_max=10.0, temp=_c2k(36.0), q10=1.0, temp_ref=_c2k(36.0), V_sh=-60.0),  # potassium.py:317-321
    "CaHT_HM1992": dict(g_max=2.0, temp=_c2k(36.0), q10_p=3.55, temp_ref_p=_c2k(24.0), q10_q=3.0,
                        temp_ref_q=_c2k(24.0), V_sh=25.0),  # calcium.py:627-633
    "KM_MA2020_GoC": dict(g_max=0.25, temp=_c2k(30.0)),  # potassium.py:4537-4538
    "KM_MA2020_GrC": dict(g_max=0.25, temp=_c2k(30.0)),  # potassium.py:5301-5302
    "KA1_HM1992": dict(g_max=30.0, temp=_c2k(36.0), q10_p=1.0, temp_ref_p=_c2k(36.0), q10_q=1.0,
                       temp_ref_q=_c2k(36.0), V_sh=0.0),  # potassium.py:574-580
    "KA2_HM1992": dict(g_max=20.0, temp=_c2k(36.0), q10_p=1.0, temp_ref_p=_c2k(36.0), q10_q=1.0,
                       temp_ref_q=_c2k(36.0), V_sh=0.0),  # potassium.py:725-731
    "KK2A_HM1992": dict(g_max=10.0, temp=_c2k(36.0), q10_p=1.0, temp_ref_p=_c2k(36.0), q10_q=1.0,
                        temp_ref_q=_c2k(36.0), V_sh=0.0),  # potassium.py:863-869
    "KK2B_HM1992": dict(g_max=10.0, temp=_c2k(36.0), q10_p=1.0, temp_ref_p=_c2k(36.0), q10_q=1.0,
                        temp_ref_q=_c2k(36.0), V_sh=0.0),  # potassium.py:1005-1011
    "KNI_Ya1989": dict(g_max=0.004, temp=_c2k(36.0), q10=1.0, temp_ref=_c2k(36.0), tau_max=4e3,
                       V_sh=0.0),  # potassium.py:1140-1145
}
CHANNEL_DEFAULTS.update({
    "Kv3p4_MA2020_GoC": dict(g_max=4.0, temp=_c2k(22.0)),  # potassium.py:4750 (__init__)
    "Kv4p3_MA2020_GoC": dict(g_max=3.2, temp=_c2k(22.0)),  # potassium.py:4964
    "Kv1p1_MA2020_GoC": dict(g_max=4.0, temp=_c2k(22.0), gateCurrent=0.0),  # potassium.py:4570
    "Kir2p3_MA2020_GrC": dict(g_max=0.9, temp=_c2k(30.0)),  # potassium.py:5334
    "HCN1_MA2020_GoC": dict(g_max=0.05, E=-20.0, temp=_c2k(22.0)),  # hyperpolarization_activated.py:675
    "HCN1_MA2024_PC": dict(g_max=0.1, E=-34.4, temp=_c2k(23.0)),  # hyperpolarization_activated.py:411
    "CaHVA_MA2020_GoC": dict(g_max=0.46, temp=_c2k(30.0)),  # calcium.py:4333
    "Cav2p3_MA2020_GoC": dict(g_max=0.0, temp=_c2k(34.0)),  # calcium.py:4672
    "Cav3p2_RI2021_SC": dict(g_max=8.0e-4, V_sh=0.0, temp=_c2k(36.0)),  # calcium.py:3636
})
# extension channels (conductances in mS/cm^2)
CHANNEL_DEFAULTS.update({
    "HCN2_MA2020_GoC": dict(g_max=0.08, E=-20.0, temp=_c2k(22.0)),  # hyperpolarization_activated.py:838
    "Kv3p3_MA2024_PC": dict(g_max=5.0, temp=_c2k(22.0), gateCurrent=0.0),  # potassium.py:2937 (0.005 S/cm^2)
    "Kv2p2_0010_MA2020_GrC": dict(g_max=0.01, BBiD=10.0),  # potassium.py:5664
    "Kv1p5_MA2024_PC": dict(g_max=0.13195, temp=_c2k(37.0), Tauact=1.0, Tauinactf=1.0,
                            Tauinacts=1.0),  # potassium.py:2735 (0.13195e-3 S/cm^2)
    "NaF_SU2015_DCN": dict(g_max=0.01),  # sodium.py:402
    "NaP_SU2015_DCN": dict(g_max=0.01),  # sodium.py:500
    "Na_ZH2019_IO": dict(g_max=70.0),  # sodium.py:598
    "fKdr_SU2015_DCN": dict(g_max=0.01),  # potassium.py:1374
    "sKdr_SU2015_DCN": dict(g_max=0.01),  # potassium.py:1485
    "Kdr_ZH2019_IO": dict(g_max=18.0),  # potassium.py:6238
    "HCN_SU2015_DCN": dict(g_max=0.01, E=-45.0),  # hyperpolarization_activated.py:1010
    "HCN_ZH2019_IO": dict(g_max=0.15, E=-43.0),  # hyperpolarization_activated.py:1109
    "CaT_HP1992": dict(g_max=1.75, temp=_c2k(36.0), q10_p=5.0, temp_ref_p=_c2k(24.0), q10_q=3.0,
                       temp_ref_q=_c2k(24.0), V_sh=-3.0),  # calcium.py:377
    "CaHT_Re1993": dict(g_max=1.0, temp=_c2k(36.0), q10_p=2.3, temp_ref_p=_c2k(23.0), q10_q=2.3,
                        temp_ref_q=_c2k(23.0), V_sh=0.0),  # calcium.py:667
    "CaL_SU2015_DCN": dict(g_max=0.01, E=139.0, qdeltat=1.0),  # calcium.py:1066
    "Kca3p1_MA2020_GoC": dict(g_max=120.0, q10_base=3.0, temp=_c2k(22.0)),  # potassium_calcium.py:299
    "SK_SU2015_DCN": dict(g_max=0.01, qdeltat=1.0),  # potassium_calcium.py:189
    "K_Kv_test": dict(g_max=0.0, V_sh=0.0, temp=_c2k(25.0), Ra=0.02, Rb=0.006, q=9.0, v12=25.0),  # potassium.py:1239
    "CaN_IS2008": dict(E=10.0, g_max=1.0, temp=_c2k(36.0), q10=1.0, temp_ref=_c2k(36.0)),  # calcium.py:108
    "Ca_ZH2019_IO": dict(g_max=0.4, E=120.0, mMidV=-61.0, freeze_m_inf=1.0),  # calcium.py:4837
    # permeability in cm/s (calcium.py:1972)
    "Cav3p1_MA2020_GoC": dict(g_max=2.5e-4, V_sh=0.0, temp=_c2k(22.0), q10=3.0, temp_ref=_c2k(37.0)),
    # permeability perm (cm/s) times g_scale (calcium.py:4033)
    "Cav3p3_RI2021_SC": dict(perm=1.0e-4, g_scale=1.0e-5, temp=_c2k(36.0), V_sh=0.0),
    "Cav1p2_MA2020_GoC": dict(g_max=0.2, V_sh=0.0, temp=_c2k(22.0), q10=1.0, temp_ref=_c2k(22.0)),  # calcium.py:1408
    "Cav1p3_MA2020_GoC": dict(g_max=0.005, V_sh=0.0, temp=_c2k(22.0), q10=1.0, temp_ref=_c2k(22.0)),  # :1683
    "Cav2p1_RI2021_SC": dict(g_max=2.2e-4, V_sh=0.0, temp=_c2k(23.0)),  # calcium.py:2767 (cm/s)
    # calcium.py:2577: Cav3p1's gates, g in mS/cm^2, current -g p^2 q (1 mV)
    "Cav3p1Test_PC24": dict(g_max=0.25, temp=_c2k(22.0), q10=3.0, temp_ref=_c2k(37.0)),
    "CaHVA_SU2015_DCN": dict(perm=7.5e-6, temp=_c2k(36.0), qdeltat=1.0),  # calcium.py:924 (cm/s)
    "CaLVA_SU2015_DCN": dict(perm=1.0, temp=_c2k(36.0), qdeltat=1.0),  # calcium.py:1221 (cm/s)
})


def su2015_drive(V, ci, co, temp):
    """The SU2015 DCN calcium drive (calcium.py:924-1064): (4.47814e6 V / T)(ci - co A) /
    1000 / (1 - A) mA/cm^2 per cm/s with A = e^-x, x = 23.20764929 V / T, written as
    c S(x)(ci - co A) uA/cm^2 per cm/s (c = 4.47814e6 / 23.20764929, S(x) = x / (1 - e^-x);
    the same value, finite at V = 0).  Returns (drive, d drive / dV per mV)."""
    c = 4.47814e6 / 23.20764929
    kx = 23.20764929 / temp
    x = kx * V
    a = np.exp(-x)
    small = np.abs(x) < 1e-4
    xs = np.where(small, 1.0, x)
    sx = np.where(small, 1.0 + x / 2.0, xs / (1.0 - np.exp(-xs)))
    den = 1.0 - np.exp(-xs)
    ds = np.where(small, 0.5 + x / 6.0, (den - xs * np.exp(-xs)) / den ** 2)
    num = ci - co * a
    return c * sx * num, c * kx * (ds * num + sx * co * a)


def ghk_codata_drive(V, ci, co, temp):
    """The shared ghk_flux (channel/_base.py:47) for z = 2 with the CODATA F and R of
    the CalciumDetailed restatement (FARADAY, GAS_R), the small branch at
    |1 - e^-zeta| <= 1e-6.  Returns (drive, d drive / dV per mV)."""
    zf = 2.0 * FARADAY
    k = zf / (GAS_R * temp) * 1e-3
    z = k * V
    em = np.exp(-z)
    num = ci - co * em
    den = 1.0 - em
    small = np.abs(den) <= 1e-6
    safe = np.where(small, 1.0, den)
    drive = np.where(small, zf * num * (1.0 + z / 2.0), zf * z * num / safe)
    dd = np.where(small, zf * k * (co * em * (1.0 + z / 2.0) + num / 2.0),
                  zf * k * ((num + z * co * em) / safe - z * num * em / safe ** 2))
    return drive, dd


def cav33_drive(V, ci, co, temp):
    """The Cav3.3 GHK drive (calcium.py:89-97) with the model file's F = 96520, R = 8.3134
    and T - 0.01 K; z = 2.  Returns (drive, d drive / dV per mV)."""
    zf = 2.0 * 96520.0
    k = zf / (8.3134 * (temp - 0.01)) * 1e-3
    w = k * V
    ep = np.exp(w)
    num = co - ci * ep
    den = ep - 1.0
    small = np.abs(den) < 1e-6
    safe = np.where(small, 1.0, den)
    drive = np.where(small, -zf * num * (1.0 - w / 2.0), -zf * num * w / safe)
    dd = np.where(small, -zf * k * (-ci * ep * (1.0 - w / 2.0) - num / 2.0),
                  -zf * k * ((num - ci * ep * w) / safe - num * w * ep / safe ** 2))
    return drive, dd


def cav31_drive(V, ci, co, temp):
    """The Cav3.1 GHK drive (calcium.py:78-86) with the model file's constants
    F = 9.6485e4, R = 8.3145 and T + 0.04 K; z = 2.  Returns (drive, d drive / dV per mV)
    for ci, co in mM and V in mV; -g drive (g in cm/s) is in uA/cm^2."""
    zf = 2.0 * 9.6485e4
    k = zf / (8.3145 * (temp + 0.04)) * 1e-3
    z = k * V
    em = np.exp(-z)
    num = ci - co * em
    den = 1.0 - em
    small = np.abs(den) < 1e-6
    safe = np.where(small, 1.0, den)
    drive = np.where(small, zf * num * (1.0 + z / 2.0), zf * z * num / safe)
    dd = np.where(small, zf * k * (co * em * (1.0 + z / 2.0) + num / 2.0),
                  zf * k * ((num + z * co * em) / safe - z * num * em / safe ** 2))
    return drive, dd


def can_modulation(Ci):
    """CaN_IS2008's current factor Ci / (Ci + 0.2 mM) (calcium.py:108-220)."""
    return Ci / (Ci + 0.2)


def caio_minf(V, mid):
    """Ca_ZH2019_IO's instantaneous m_inf = 1 / (1 + exp((mMidV - V) / 4.2))^3 and its
    V-derivative (calcium.py:4837-4979)."""
    t = 1.0 + np.exp((mid - V) / 4.2)
    return 1.0 / t ** 3, 3.0 * (t - 1.0) / (4.2 * t ** 4)
# cell-type variants that run their base class's kinetics, with their own defaults
# where they differ (each class body is the base's: potassium.py, hyperpolarization_activated.py)
_VARIANTS = {
    **{v: ("Kv3p4_MA2020_GoC", {}) for v in ("Kv3p4_MA2020_GrC", "Kv3p4_MA2024_PC", "Kv3p4_MA2025_BC",
                                              "Kv3p4_RI2021_SC")},
    **{v: ("Kv4p3_MA2020_GoC", {"temp": _c2k(30.0)}) for v in ("Kv4p3_MA2020_GrC", "Kv4p3_MA2024_PC",
                                                                "Kv4p3_MA2025_BC", "Kv4p3_RI2021_SC")},
    **{v: ("Kv1p1_MA2020_GoC", {}) for v in ("Kv1p1_MA2020_GrC", "Kv1p1_MA2024_PC", "Kv1p1_MA2025_BC",
                                              "Kv1p1_RI2021_SC")},
    **{v: ("Kir2p3_MA2020_GrC", {}) for v in ("Kir2p3_MA2024_PC", "Kir2p3_MA2025_BC", "Kir2p3_RI2021_SC")},
    **{v: ("HCN1_MA2024_PC", {}) for v in ("HCN1_MA2025_BC", "HCN1_RI2021_SC")},
    "CaHVA_MA2020_GrC": ("CaHVA_MA2020_GoC", {}),
    # potassium_sodium.py:38-259: Kv1p5_MA2024_PC's kinetics and K current, plus a
    # nonspecific current of conductance gnonspec (0 by default; only 0 is restated)
    "Kv1p5_MA2020_GrC": ("Kv1p5_MA2024_PC", {"gnonspec": 0.0}),
    **{v: ("Kca3p1_MA2020_GoC", {}) for v in ("Kca3p1_MA2025_BC", "Kca3p1_MA2024_PC")},
    "Ca_ZH2019_IO_Frozen": ("Ca_ZH2019_IO", {}),  # freeze_m_inf pinned to True (calcium.py, the subclass)
    # Cav3p1_MA2024_PC overrides nothing; the _Frozen classes hold the GHK drive out of the linearisation
    **{v: ("Cav3p1_MA2020_GoC", {}) for v in ("Cav3p1_MA2024_PC", "Cav3p1_MA2020_GoC_Frozen",
                                               "Cav3p1_MA2024_PC_Frozen")},
    **{v: ("Cav3p3_RI2021_SC", {}) for v in ("Cav3p3_MA2024_PC", "Cav3p3_MA2024_PC_Frozen")},
    "Cav1p2_MA2025_BC": ("Cav1p2_MA2020_GoC", {}), "Cav1p3_MA2025_BC": ("Cav1p3_MA2020_GoC", {}),
    **{v: ("Cav2p1_RI2021_SC", {}) for v in ("Cav2p1_MA2024_PC", "Cav2p1_MA2025_BC", "Cav2p1_MA2024_PC_Frozen",
                                              "Cav2p1_MA2025_BC_Frozen", "Cav2p1_RI2021_SC_Frozen")},
    **{v: ("Cav3p2_RI2021_SC", {}) for v in ("Cav3p2_MA2025_BC", "Cav3p2_MA2024_PC")},
}


def _base_class(name: str) -> str:
    return _VARIANTS[name][0] if name in _VARIANTS else name


# Markov channels (channel/_base.py:677-1125): restated in oracle/markov.py
CHANNEL_DEFAULTS.update({k: dict(v) for k, v in MK.MARKOV_DEFAULTS.items()})
ION_DEFAULTS = {
    "SodiumFixed": dict(E=50.0),
    "PotassiumFixed": dict(E=-95.0),
    "CalciumFixed": dict(E=120.0),
    "CalciumDetailed": dict(temp=_c2k(36.0), d=1.0, tau=5.0, C_rest=2.4e-4, Co=2.0, Ci_initializer=2.4e-4),
    # InitNernst ions: fixed Ci / Co, E stored from Nernst (ion/_base.py:350-356) with the
    # family defaults (ion/sodium.py:82-84, ion/potassium.py:83-85, ion/calcium.py:120-122)
    "SodiumInitNernst": dict(temp=_c2k(36.0), Ci=10.0, Co=140.0, valence=1),
    "PotassiumInitNernst": dict(temp=_c2k(36.0), Ci=54.4, Co=2.5, valence=1),
    "CalciumInitNernst": dict(temp=_c2k(36.0), Ci=5e-5, Co=2.0, valence=2),
}
_CA_FIXED_CI = 5e-5  # Calcium.default_Ci (ion/calcium.py:120)


# ----------------------------------------------------------------------------- geometry


@dataclass(frozen=True)
class Frustum:
    prox: float
    dist: float
    length_um: float
    r_prox_um: float
    r_dist_um: float


def insert_radius_jumps(lengths, r_prox, r_dist):
    """Zero-length jump segments at radius discontinuities (``morph/branch.py:440-500``)."""
    lengths = np.asarray(lengths, dtype=float)
    r_prox = np.asarray(r_prox, dtype=float)
    r_dist = np.asarray(r_dist, dtype=float)
    if lengths.size <= 1:
        return lengths, r_prox, r_dist
    disc = ~np.isclose(r_dist[:-1], r_prox[1:])
    L, P, D = [], [], []
    for i in range(lengths.size):
        L.append(lengths[i])
        P.append(r_prox[i])
        D.append(r_dist[i])
        if i < lengths.size - 1 and disc[i]:
            L.append(0.0)
            P.append(r_dist[i])
            D.append(r_prox[i + 1])
    return np.asarray(L), np.asarray(P), np.asarray(D)


def build_frusta(lengths, r_prox, r_dist, prox: float, dist: float) -> tuple[Frustum, ...]:
    """``_build_frusta`` (geometry.py:214-321) without 3-D points."""
    prox_f, dist_f = float(prox), float(dist)
    if not (0.0 - EPS_PARAM <= prox_f < dist_f - EPS_PARAM and dist_f <= 1.0 + EPS_PARAM):
        raise ValueError(f"CV bounds must satisfy 0 <= prox < dist <= 1, got {(prox, dist)!r}.")
    prox_f = max(0.0, min(1.0, prox_f))
    dist_f = max(0.0, min(1.0, dist_f))
    lengths = np.asarray(lengths, dtype=float)
    r_prox = np.asarray(r_prox, dtype=float)
    r_dist = np.asarray(r_dist, dtype=float)
    if np.any(r_prox <= 0.0) or np.any(r_dist <= 0.0):
        raise ValueError("All branch radii must be > 0.")
    total = float(np.sum(lengths))
    if total <= EPS_LEN_UM:
        raise ValueError("Branch total length must be > EPS_LEN_UM.")
    start_um, end_um = prox_f * total, dist_f * total
    seg_starts = np.concatenate(([0.0], np.cumsum(lengths)[:-1]))
    seg_ends = seg_starts + lengths
    out: list[Frustum] = []
    for i, seg_len in enumerate(lengths):
        s0, s1 = float(seg_starts[i]), float(seg_ends[i])
        rp, rd = float(r_prox[i]), float(r_dist[i])
        if seg_len <= EPS_LEN_UM:
            if np.isclose(rp, rd):
                continue
            # zero-length radius jump (geometry.py:198-211)
            if s0 < start_um - EPS_LEN_UM or s0 > end_um + EPS_LEN_UM:
                continue
            if s0 <= start_um + EPS_LEN_UM and not start_um <= EPS_LEN_UM:
                continue
            xj = max(prox_f, min(dist_f, s0 / total))
            out.append(Frustum(xj, xj, 0.0, rp, rd))
            continue
        left, right = max(s0, start_um), min(s1, end_um)
        if right - left <= EPS_LEN_UM:
            continue
        t0, t1 = (left - s0) / float(seg_len), (right - s0) / float(seg_len)
        r0, r1 = rp + (rd - rp) * t0, rp + (rd - rp) * t1
        x0 = max(prox_f, min(dist_f, left / total))
        x1 = max(prox_f, min(dist_f, right / total))
        out.append(Frustum(x0, x1, right - left, r0, r1))
    if not out:
        raise ValueError("CV produced no frusta.")
    return tuple(out)


def lateral_area_um2(frusta) -> float:
    total = 0.0
    for p in frusta:
        slant = math.sqrt(p.length_um ** 2 + (p.r_dist_um - p.r_prox_um) ** 2)
        total += math.pi * (p.r_prox_um + p.r_dist_um) * slant
    return total


def axial_factor_per_cm(frusta) -> float:
    f = 0.0
    for p in frusta:
        f += (p.length_um * 1e-4) / (math.pi * (p.r_prox_um * 1e-4) * (p.r_dist_um * 1e-4))
    return f


def midpoint_radius_um(frusta) -> float:
    total = sum(p.length_um for p in frusta)
    if total <= EPS_LEN_UM:
        return 0.5 * (frusta[0].r_prox_um + frusta[-1].r_dist_um)
    target, walked = 0.5 * total, 0.0
    for p in frusta:
        nxt = walked + p.length_um
        if nxt >= target - EPS_LEN_UM:
            if p.length_um <= EPS_LEN_UM:
                return 0.5 * (p.r_prox_um + p.r_dist_um)
            ratio = max(0.0, min(1.0, (target - walked) / p.length_um))
            return p.r_prox_um + (p.r_dist_um - p.r_prox_um) * ratio
        walked = nxt
    return frusta[-1].r_dist_um


def split_frusta(frusta, x: float):
    left, right = [], []
    for p in frusta:
        if p.dist <= x + EPS_PARAM:
            left.append(p)
            continue
        if p.prox >= x - EPS_PARAM:
            right.append(p)
            continue
        span = p.dist - p.prox
        if span <= EPS_PARAM:
            continue
        ratio = max(0.0, min(1.0, (x - p.prox) / span))
        ll = p.length_um * ratio
        lr = p.length_um - ll
        rm = p.r_prox_um + (p.r_dist_um - p.r_prox_um) * ratio
        if ll > EPS_LEN_UM:
            left.append(Frustum(p.prox, x, ll, p.r_prox_um, rm))
        if lr > EPS_LEN_UM:
            right.append(Frustum(x, p.dist, lr, rm, p.r_dist_um))
    return tuple(left), tuple(right)


# ----------------------------------------------------------------------------- schedule


def compute_peel_levels(node_parent: np.ndarray, node_children) -> np.ndarray:
    """``_compute_peel_levels`` (scheduling.py:120-159)."""
    n = len(node_parent)
    levels = np.full(n, -1, dtype=np.int32)
    remaining = np.asarray([len(c) for c in node_children], dtype=np.int32)
    frontier = [pid for pid in range(n) if remaining[pid] == 0]
    for pid in frontier:
        levels[pid] = 0
    cur = 0
    while cur < len(frontier):
        pid = frontier[cur]
        cur += 1
        par = int(node_parent[pid])
        if par < 0:
            continue
        cand = int(levels[pid]) + 1
        if levels[par] < cand:
            levels[par] = cand
        remaining[par] -= 1
        if remaining[par] == 0:
            frontier.append(par)
    if (levels < 0).any():
        raise ValueError("compute_peel_levels: cycle detected or node unreachable from any leaf.")
    return levels


def build_backsub_indices(parent_lookup: np.ndarray, n_nodes: int) -> np.ndarray:
    """``_build_backsub_indices`` (_staggered.py:726-739)."""
    parent_lookup = np.asarray(parent_lookup, dtype=np.int32)
    idx = []
    old, new = 0, 1
    k = np.arange(n_nodes + 1, dtype=np.int32)
    while new <= max(1, n_nodes):
        for _ in range(new - old):
            k = parent_lookup[k]
        old, new = new, 2 * new
        idx.append(k)
    return np.asarray(idx, dtype=np.int32)


# ----------------------------------------------------------------------------- rates


def exprel(x):
    """(e^x - 1)/x with exprel(0) = 1."""
    x = np.asarray(x, dtype=np.float64)
    small = np.abs(x) < 1e-300
    xs = np.where(small, 1.0, x)
    return np.where(small, 1.0, np.expm1(xs) / xs)


def exp_euler(x, f, lam, dt: float):
    """One exponential-Euler step of x' = f(x) with diagonal Jacobian lam:
    x + dt * exprel(dt * lam) * f (quad/_exp_euler.py:330-478)."""
    return x + dt * exprel(dt * lam) * f


def gate_step(x, kind: str, a, b, phi, dt: float):
    """Exp-Euler step of one HH gate (channel/_base.py:575-588): ``kind`` "ab" for
    x' = phi (a (1 - x) - b x), "it" for x' = phi (a - x) / b (a = x_inf, b = tau)."""
    if kind == "ab":
        f = phi * (a * (1.0 - x) - b * x)
        lam = -phi * (a + b)
    else:
        f = phi * (a - x) / b
        lam = -phi / b
    return exp_euler(x, f, lam, dt)


def nernst_ca_mV(temp, Co, Ci):
    """Calcium reversal potential (mV): R T / (2 F) ln(Co / Ci) (ion/_base.py:463-469)."""
    return 1e3 * GAS_R * temp / (2.0 * FARADAY) * np.log(Co / Ci)


def ca_detailed_rate(I_ca, Ci, d, tau, C_rest):
    """CalciumDetailed dCi/dt (mM/ms) (ion/calcium.py:499-505): the influx
    max(I_ca / (2 F d), 0) of the ion's total current I_ca = sum g (E_Ca - V)
    (uA/cm^2, positive inward), over a shell of depth d (um), plus the decay
    (C_rest - Ci) / tau."""
    drive = np.maximum(I_ca * 10.0 / (2.0 * FARADAY * d), 0.0)
    return drive + (C_rest - Ci) / tau


def _x_over_1mexp(x):
    """x / (1 - e^-x), with 1 + x / 2 for |x| < 1e-6 (channel/sodium.py:50-55)."""
    x = np.asarray(x, dtype=float)
    small = np.abs(x) < 1e-6
    safe = np.where(small, 1.0, x)
    return np.where(small, 1.0 + x / 2.0, safe / (1.0 - np.exp(-safe)))


def kv15_vfactor(V):
    """Kv1p5_MA2024_PC's voltage factor f(V) and f'(V) (potassium.py:2735-2935)."""
    s = 1.0 / (1.0 + np.exp(-(V - 15.0) / 13.0))
    return 0.1 + s, s * (1.0 - s) / 13.0


def rates(name: str, V, p: dict, Ci=None):
    """Gate rate functions, keyed by gate: returns {gate: ("ab", alpha, beta) | ("it", inf, tau)}."""
    if name == "Na_Ba2002":  # sodium.py:154-170
        Vp = V - p["V_sh"]
        return {
            "p": ("ab", 0.32 * 4.0 / exprel(-(Vp - 13.0) / 4.0), 0.28 * 5.0 / exprel((Vp - 40.0) / 5.0)),
            "q": ("ab", 0.128 * np.exp(-(Vp - 17.0) / 18.0), 4.0 / (1.0 + np.exp(-(Vp - 40.0) / 5.0))),
        }
    if name == "KDR_Ba2002":  # potassium.py:206-214
        Vp = V - p["V_sh"]
        return {"p": ("ab", 0.032 * 5.0 / exprel(-(Vp - 15.0) / 5.0), 0.5 * np.exp(-(Vp - 10.0) / 40.0))}
    if name == "CaL_IS2008":  # calcium.py:(CaL f_p_inf .. f_q_tau)
        Vs = V - p["V_sh"]
        return {
            "p": ("it", 1.0 / (1.0 + np.exp(-(Vs + 10.0) / 4.0)),
                  0.4 + 0.7 / (np.exp(-(Vs + 5.0) / 15.0) + np.exp((Vs + 5.0) / 15.0))),
            "q": ("it", 1.0 / (1.0 + np.exp((Vs + 25.0) / 2.0)),
                  300.0 + 100.0 / (np.exp((Vs + 40.0) / 9.5) + np.exp(-(Vs + 40.0) / 9.5))),
        }
    if name == "CaT_HM1992":  # calcium.py:(CaT f_p_inf .. f_q_tau)
        Vs = V - p["V_sh"]
        return {
            "p": ("it", 1.0 / (1.0 + np.exp(-(Vs + 59.0) / 6.2)),
                  1.0 / (np.exp(-(Vs + 132.0) / 16.7) + np.exp((Vs + 16.8) / 18.2)) + 0.612),
            "q": ("it", 1.0 / (1.0 + np.exp((Vs + 83.0) / 4.0)),
                  np.where(Vs >= -80.0, np.exp(-(Vs + 22.0) / 10.5) + 28.0, np.exp((Vs + 467.0) / 66.6))),
        }
    if name == "HCN_HM1992":  # hyperpolarization_activated.py:126-133
        return {"p": ("it", 1.0 / (1.0 + np.exp((V + 75.0) / 5.5)),
                      1.0 / (np.exp(-0.086 * V - 14.59) + np.exp(0.0701 * V - 1.87)))}
    if name == "AHP_De1994":  # potassium_calcium.py:181-186
        return {"p": ("ab", p["alpha"] * np.power(Ci, p["n"]), p["beta"] * np.ones_like(V))}
    if name == "Na_HH1952":  # sodium.py:384-399
        Vp = V - p["V_sh"]
        return {
            "p": ("ab", 1.0 / exprel(-(Vp - 5.0) / 10.0), 4.0 * np.exp(-(Vp + 20.0) / 18.0)),
            "q": ("ab", 0.07 * np.exp(-(Vp + 20.0) / 20.0), 1.0 / (1.0 + np.exp(-(Vp - 10.0) / 10.0))),
        }
    if name == "K_HH1952":  # potassium.py:450-456
        Vp = V - p["V_sh"]
        return {"p": ("ab", 0.1 / exprel(-(Vp + 10.0) / 10.0), 0.125 * np.exp(-(Vp + 20.0) / 80.0))}
    if name == "Na_TM1991":  # sodium.py:275-289, written as there (V_sh - V)
        t = p["V_sh"] - V
        return {
            "p": ("ab", 0.32 * 4.0 / exprel((13.0 + t) / 4.0), 0.28 * 5.0 / exprel((-t - 40.0) / 5.0)),
            "q": ("ab", 0.128 * np.exp((17.0 + t) / 18.0), 4.0 / (1.0 + np.exp(-(-t - 40.0) / 5.0))),
        }
    if name == "K_TM1991":  # potassium.py:331-337, written as there (V_sh - V)
        t = p["V_sh"] - V
        return {"p": ("ab", 0.032 * 5.0 / exprel((15.0 + t) / 5.0), 0.5 * np.exp((10.0 + t) / 40.0))}
    if name == "CaHT_HM1992":  # calcium.py:645-663
        Vs = V - p["V_sh"]
        return {
            "p": ("it", 1.0 / (1.0 + np.exp(-(Vs + 59.0) / 6.2)),
                  1.0 / (np.exp(-(Vs + 132.0) / 16.7) + np.exp((Vs + 16.8) / 18.2)) + 0.612),
            "q": ("it", 1.0 / (1.0 + np.exp((Vs + 83.0) / 4.0)),
                  np.where(Vs >= -80.0, np.exp(-(Vs + 22.0) / 10.5) + 28.0, np.exp((Vs + 467.0) / 66.6))),
        }
    if name in ("KA1_HM1992", "KA2_HM1992"):  # potassium.py:592-611 and :743-762
        Vs = V - p["V_sh"]
        mid, slope = (60.0, 8.5) if name == "KA1_HM1992" else (36.0, 20.0)
        return {
            "p": ("it", 1.0 / (1.0 + np.exp(-(Vs + mid) / slope)),
                  1.0 / (np.exp((Vs + 35.8) / 19.7) + np.exp(-(Vs + 79.7) / 12.7)) + 0.37),
            "q": ("it", 1.0 / (1.0 + np.exp((Vs + 78.0) / 6.0)),
                  np.where(Vs < -63.0, 1.0 / (np.exp((Vs + 46.0) / 5.0) + np.exp(-(Vs + 238.0) / 37.5)), 19.0)),
        }
    if name == "KNI_Ya1989":  # potassium.py:1156-1163
        t = V - p["V_sh"] + 35.0
        return {"p": ("it", 1.0 / (1.0 + np.exp(-(V - p["V_sh"] + 35.0) / 10.0)),
                      p["tau_max"] / (3.3 * np.exp(t / 20.0) + np.exp(-t / 20.0)))}
    if name in ("KK2A_HM1992", "KK2B_HM1992"):  # potassium.py:881-895 and :1023-1041
        Vs = V - p["V_sh"]
        bell = 1.0 / (np.exp((Vs - 1329.0) / 200.0) + np.exp(-(Vs + 130.0) / 7.1))
        qtau = bell + 120.0 if name == "KK2A_HM1992" else np.where(Vs < -70.0, bell, 8.9)
        return {
            "p": ("it", 1.0 / (1.0 + np.exp(-(Vs + 43.0) / 17.0)),
                  1.0 / (np.exp((Vs - 81.0) / 25.6) + np.exp(-(Vs + 132.0) / 18.0)) + 9.9),
            "q": ("it", 1.0 / (1.0 + np.exp((Vs + 58.0) / 10.6)), qtau),
        }
    if name == "Kv3p4_MA2020_GoC":  # potassium.py:4750: V' = V + 11 mV, times in s x 1000
        x = V + 11.0
        mt = np.where(x < -35.0, (3.4225e-5 + 0.00498 * np.exp(x / 28.29)) * 3.0,
                      0.00012851 + 1.0 / (np.exp((x + 100.7) / 12.9) + np.exp((x - 56.0) / -23.1)))
        ht = np.where(x > 0.0, 0.0012 + 0.0023 * np.exp(-0.141 * x),
                      1.2202e-05 + 0.012 * np.exp(-(((x + 56.3) / 49.6) ** 2)))
        return {"m": ("it", 1.0 / (1.0 + np.exp(-(x + 24.0) / 15.4)), 1000.0 * mt),
                "h": ("it", 0.31 + 0.69 / (1.0 + np.exp((x + 5.802) / 11.2)), 1000.0 * ht)}
    if name == "Kv4p3_MA2020_GoC":  # potassium.py:4964, sigm(x, y) = 1 / (exp(x / y) + 1) (:73-74)
        def sigm(x, y):
            return 1.0 / (np.exp(x / y) + 1.0)
        aa, ab = 0.8147 * sigm(V + 9.17203, -23.3271), 0.1655 / np.exp((V + 18.2791) / 19.4718)
        ba, bb = 0.0368 * sigm(V + 111.332, 12.8433), 0.0345 * sigm(V + 49.9537, -8.90123)
        return {"a": ("it", 1.0 / (1.0 + np.exp((V + 38.0) / -17.0)), 1.0 / (aa + ab)),
                "b": ("it", 1.0 / (1.0 + np.exp((V + 78.8) / 8.4)), 1.0 / (ba + bb))}
    if name == "Kv1p1_MA2020_GoC":  # potassium.py:4570
        return {"n": ("ab", 0.12889 * np.exp(-(V + 45.0) / -33.90877), 0.12889 * np.exp(-(V + 45.0) / 12.42101))}
    if name == "Kir2p3_MA2020_GrC":  # potassium.py:5334
        return {"d": ("ab", 0.13289 * np.exp((V + 83.94) / -24.3902), 0.16994 * np.exp((V + 83.94) / 35.714))}
    if name == "HCN1_MA2020_GoC":  # hyperpolarization_activated.py:675
        o = 1.0 / (1.0 + np.exp((V - -72.49) * 0.11305))
        r = 0.002096 * V + 0.97596
        return {"o_fast": ("it", r * o, np.exp(((0.01371 * V) - -3.368) * 2.30259)),
                "o_slow": ("it", (1.0 - r) * o, np.exp(((0.01451 * V) - -4.056) * 2.30259))}
    if name == "HCN1_MA2024_PC":  # hyperpolarization_activated.py:411, half voltages minus the 9.3 mV ljp
        vh, v1 = -90.3 - 9.3, -68.0 - 9.3
        return {"h": ("it", 1.0 / (1.0 + np.exp((V - vh) / 9.67)),
                      1.0 / (0.0018 * (np.exp((V - v1) / -22.0) + np.exp((V - v1) / 7.14))))}
    if name == "CaHVA_MA2020_GoC":  # calcium.py:4333
        return {"s": ("ab", 0.04944 * np.exp((V - -29.06) / 15.873), 0.08298 * np.exp((V - -18.66) / -25.641)),
                "u": ("ab", 0.0013 * np.exp((V - -48.0) / -18.183), 0.0013 * np.exp((V - -48.0) / 83.33))}
    if name == "Cav2p3_MA2020_GoC":  # calcium.py:4672
        one = np.ones_like(V)
        return {"m": ("it", 1.0 / (1.0 + np.exp((V + 48.5) / -3.0)), 50.0 * one),
                "h": ("it", 1.0 / (1.0 + np.exp((V + 53.0) / 1.0)), 5.0 * one)}
    if name == "Cav3p2_RI2021_SC":  # calcium.py:3636, on V + V_sh; tau_h carries 3^((36 - 24) / 10)
        Vs = V + p["V_sh"]
        phi_h = 3.0 ** ((36.0 - 24.0) / 10.0)
        term = (1942.0 + np.exp((Vs + 164.0) / 9.2)) / (1.0 + np.exp((Vs + 89.3) / 3.7))
        return {"m": ("it", 1.0 / (1.0 + np.exp(-(Vs + 54.8) / 7.4)),
                      1.9 + 1.0 / (np.exp((Vs + 37.0) / 11.9) + np.exp(-(Vs + 131.6) / 21.0))),
                "h": ("it", 1.0 / (1.0 + np.exp((Vs + 85.5) / 7.18)), 13.7 + term / phi_h)}
    if name == "HCN2_MA2020_GoC":  # hyperpolarization_activated.py:838-1008
        o = 1.0 / (1.0 + np.exp((V - -81.95) * 0.1661))
        r = np.where(V >= -64.70, 0.0, np.where(V <= -108.70, 1.0, -0.0227 * V + -1.4694))
        return {"o_fast": ("it", r * o, np.exp(((0.0269 * V) - -5.6111) * 2.3026)),
                "o_slow": ("it", (1.0 - r) * o, np.exp(((0.0152 * V) - -5.2944) * 2.3026))}
    if name == "Kv3p3_MA2024_PC":  # potassium.py:2937-3124
        return {"n": ("ab", 0.22 * np.exp(-(V + 16.0) / -26.5), 0.22 * np.exp(-(V + 16.0) / 26.5))}
    if name == "Kv2p2_0010_MA2020_GrC":  # potassium.py:5664-5804
        return {"m": ("it", 1.0 / (1.0 + np.exp((V - 5.0) / -12.0)), 130.0 / (1.0 + np.exp((V + 46.56) / -44.14))),
                "h": ("it", 1.0 / (1.0 + np.exp((V + 16.3) / 4.8)), 10000.0 / (1.0 + np.exp((V + 46.56) / -44.14)))}
    if name == "Kv1p5_MA2024_PC":  # potassium.py:2735-2935; q10 2.2 at 37 degC on the m and n rates
        q = 2.2 ** (((p["temp"] - _c2k(37.0))) / 10.0)
        am = q * 0.65 / (np.exp(-(V + 10.0) / 8.5) + np.exp(-(V - 30.0) / 59.0))
        bm = q * 0.65 / (2.5 + np.exp((V + 82.0) / 17.0))
        an = q * 0.001 / (2.4 + 10.9 * np.exp(-(V + 90.0) / 78.0))
        bn = q * 0.001 * np.exp((V - 168.0) / 16.0)
        return {"m": ("it", 1.0 / (1.0 + np.exp(-(V + 30.3) / 9.6)), 1.0 / (am + bm) / 3.0 * p["Tauact"]),
                "n": ("it", 0.25 + 1.0 / (1.35 + np.exp((V + 7.0) / 14.0)), 1.0 / (an + bn) / 3.0 * p["Tauinactf"]),
                "u": ("it", 0.1 + 1.0 / (1.1 + np.exp((V + 7.0) / 14.0)), 6800.0 * p["Tauinacts"] * np.ones_like(V))}
    if name == "NaF_SU2015_DCN":  # sodium.py:402-498 (qdeltat 1)
        return {"m": ("it", 1.0 / (1.0 + np.exp((V + 45.0) / -7.3)),
                      5.83 / (np.exp((V - 6.4) / -9.0) + np.exp((V + 97.0) / 17.0)) + 0.025),
                "h": ("it", 1.0 / (1.0 + np.exp((V + 42.0) / 5.9)),
                      16.67 / (np.exp((V - 8.3) / -29.0) + np.exp((V + 66.0) / 9.0)) + 0.2)}
    if name == "NaP_SU2015_DCN":  # sodium.py:500-596
        return {"m": ("it", 1.0 / (1.0 + np.exp((V + 70.0) / -4.1)), 50.0 * np.ones_like(V)),
                "h": ("it", 1.0 / (1.0 + np.exp((V + 80.0) / 4.0)), 1750.0 / (1.0 + np.exp((V + 65.0) / -8.0)) + 250.0)}
    if name == "Na_ZH2019_IO":  # sodium.py:598-725
        am, bm = _x_over_1mexp((V + 41.0) / 10.0), 9.0 * np.exp(-(V + 66.0) / 20.0)
        ah, bh = 5.0 * np.exp(-(V + 60.0) / 15.0), 10.0 * _x_over_1mexp((V + 50.0) / 10.0)
        return {"m": ("it", am / (am + bm), 0.001 * np.ones_like(V)), "h": ("it", ah / (ah + bh), 250.0 / (ah + bh))}
    if name == "fKdr_SU2015_DCN":  # potassium.py:1374-1483
        return {"m": ("it", 1.0 / (1.0 + np.exp((V + 40.0) / -7.8)),
                      13.9 / (np.exp((V + 40.0) / 12.0) + np.exp((V + 40.0) / -13.0)) + 0.1)}
    if name == "sKdr_SU2015_DCN":  # potassium.py:1485-1595
        return {"m": ("it", 1.0 / (1.0 + np.exp((V + 50.0) / -9.1)),
                      14.95 / (np.exp((V + 50.0) / 21.74) + np.exp((V + 50.0) / -13.91)) + 0.05)}
    if name == "Kdr_ZH2019_IO":  # potassium.py:6238-6374
        a, b = 10.0 * _x_over_1mexp((V + 41.0) / 10.0), 12.5 * np.exp(-(V + 51.0) / 80.0)
        return {"n": ("it", a / (a + b), 10.0 / (a + b))}
    if name == "HCN_SU2015_DCN":  # hyperpolarization_activated.py:1010-1107
        return {"m": ("it", 1.0 / (1.0 + np.exp((V + 80.0) / 5.0)), 400.0 * np.ones_like(V))}
    if name == "HCN_ZH2019_IO":  # hyperpolarization_activated.py:1109-1217
        return {"q": ("it", 1.0 / (1.0 + np.exp((V + 75.0) / 5.5)),
                      1.0 / (np.exp(-0.086 * V - 14.6) + np.exp(0.07 * V - 1.87)))}
    if name == "CaT_HP1992":  # calcium.py:377-509, on V - V_sh
        x = V - p["V_sh"]
        return {"p": ("it", 1.0 / (1.0 + np.exp(-(x + 52.0) / 7.4)),
                      3.0 + 1.0 / (np.exp((x + 27.0) / 10.0) + np.exp(-(x + 102.0) / 15.0))),
                "q": ("it", 1.0 / (1.0 + np.exp((x + 80.0) / 5.0)),
                      85.0 + 1.0 / (np.exp((x + 48.0) / 4.0) + np.exp(-(x + 407.0) / 50.0)))}
    if name == "CaHT_Re1993":  # calcium.py:667-788, t = V_sh - V; d / (e^(d/3.8) - 1) = 3.8 / exprel(d / 3.8)
        t = p["V_sh"] - V
        return {"p": ("ab", 0.055 * 3.8 / exprel((t - 27.0) / 3.8), 0.94 * np.exp((-75.0 + t) / 17.0)),
                "q": ("ab", 0.000457 * np.exp((-13.0 + t) / 50.0), 0.0065 / (np.exp((-15.0 + t) / 28.0) + 1.0))}
    if name == "CaL_SU2015_DCN":  # calcium.py:1066-1219
        ht = np.where(V < -81.0, 0.333 * np.exp((V + 466.0) / 66.0), 0.333 * np.exp((V + 21.0) / -10.5) + 9.32)
        return {"m": ("it", 1.0 / (1.0 + np.exp((V + 56.0) / -6.2)),
                      (0.333 / (np.exp((V + 131.0) / -16.7) + np.exp((V + 15.8) / 18.2)) + 0.204) / p["qdeltat"]),
                "h": ("it", 1.0 / (1.0 + np.exp((V + 80.0) / 4.0)), ht / p["qdeltat"])}
    if name == "Kca3p1_MA2020_GoC":  # potassium_calcium.py:299-450 (q10_base and temp unused)
        ci = np.asarray(Ci, dtype=float)
        c1 = 500.0 * 0.0013 / exprel((0.015 - ci) / 0.0013)
        c2 = 500.0 * 0.005 / (np.exp(0.005 / 0.0013) - 1.0)
        a = np.exp((V + 70.0) / 27.0) * np.where(ci < 0.01, c1, c2)
        return {"p": ("ab", a, 0.05 * np.ones_like(a))}
    if name == "SK_SU2015_DCN":  # potassium_calcium.py:189-297
        ci = np.asarray(Ci, dtype=float) * np.ones_like(V)
        return {"z": ("it", ci ** 4 / (ci ** 4 + 8.1e-15), np.where(ci < 0.005, 1.0 - 186.67 * ci, 0.0667) / p["qdeltat"])}
    if name == "K_Kv_test":  # potassium.py:1239-1372; y / (1 - e^(-y/q)) taken through its limit at y = 0
        y = V - p["V_sh"] - p["v12"]
        q = p["q"]
        denom = q * (p["Ra"] * _x_over_1mexp(y / q) + p["Rb"] * _x_over_1mexp(-y / q))
        return {"n": ("it", 1.0 / (1.0 + np.exp(-y / q)), 1.0 / denom)}
    if name == "Cav3p1Test_PC24":  # calcium.py:2577-2765: Cav3p1's rates
        return rates("Cav3p1_MA2020_GoC", V, p, Ci)
    if name == "Cav3p1_MA2020_GoC":  # calcium.py:1972-2202; the time constants divided by qt
        qt = p["q10"] ** ((p["temp"] - p["temp_ref"]) / 10.0)
        pt = np.where(V <= -90.0, 1.0, (1.0 + 1.0 / (np.exp((V + 40.0) / 9.0) + np.exp((V + 102.0) / -18.0))) / qt)
        return {"p": ("it", 1.0 / (1.0 + np.exp((V - -52.0) / -5.0)), pt),
                "q": ("it", 1.0 / (1.0 + np.exp((V - -72.0) / 7.0)), (15.0 + 1.0 / np.exp((V + 32.0) / 7.0)) / qt)}
    if name == "Cav3p3_RI2021_SC":  # calcium.py:4033-4255, on V - V_sh
        x = V - p["V_sh"]
        return {"n": ("it", 1.0 / (1.0 + np.exp(-(x - -41.5) / 6.2)),
                      np.where(x > -60.0, 7.2 + 0.02 * np.exp(-x / 14.7), 0.875 * np.exp((x + 120.0) / 41.0))),
                "l": ("it", 1.0 / (1.0 + np.exp(-(x - -69.8) / -6.1)),
                      np.where(x > -60.0, 79.5 + 2.0 * np.exp(-x / 9.3), 260.0))}
    if name == "CaHVA_SU2015_DCN":  # calcium.py:924-1064
        act = 31.746 / (np.exp((V - 5.0) / -13.89) + 1.0)
        cor = 3.97e-4 * 5.0 / exprel((V + 8.9) / 5.0)
        return {"m": ("it", 1.0 / (1.0 + np.exp((V + 34.5) / -9.0)), 1.0 / (act + cor) / p["qdeltat"])}
    if name == "CaLVA_SU2015_DCN":  # calcium.py:1221-1406: CaL_SU2015_DCN's gates
        return rates("CaL_SU2015_DCN", V, {"qdeltat": p["qdeltat"]})
    if name == "Cav2p1_RI2021_SC":  # calcium.py:2767-2953, on V - V_sh
        x = V - p["V_sh"]
        mt = np.where(x >= -40.0, 0.2702 + 1.1622 * np.exp(-((x + 26.798) ** 2) / 164.19), 0.6923 * np.exp(x / 1089.372))
        return {"m": ("it", 1.0 / (1.0 + np.exp(-(x - -29.458) / 8.429)), mt)}
    if name in ("Cav1p2_MA2020_GoC", "Cav1p3_MA2020_GoC"):  # calcium.py:1408-1599, :1683-1886
        ci = np.asarray(Ci, dtype=float) * np.ones_like(V)
        one = np.ones_like(V)
        if name == "Cav1p2_MA2020_GoC":
            minf, vdi, hinf_x = 1.0 / (1.0 + np.exp((V + 8.9) / -6.7)), 0.17, np.exp((V + 55.0) / 8.0)
            am, bm = 39800.0 * 9.005 / exprel((V + 8.124) / 9.005), 990.0 * np.exp(V / 31.4)
        else:
            minf, vdi, hinf_x = 1.0 / (np.exp((V - -40.0) / -5.0) + 1.0), 1.0, np.exp((V - -37.0) / 5.0)
            am, bm = 39800.0 * 15.005 / exprel((V + 67.24) / 15.005), 3500.0 * np.exp(V / 31.4)
        return {"m": ("it", minf, 1.0 / (am + bm)), "h": ("it", vdi / (1.0 + hinf_x) + (1.0 - vdi), 44.3 * one),
                "n": ("it", 0.0005 / (0.0005 + ci), 0.5 * one)}
    if name == "CaN_IS2008":  # calcium.py:108-220
        return {"p": ("it", 1.0 / (1.0 + np.exp(-(V + 43.0) / 5.2)),
                      2.7 / (np.exp(-(V + 55.0) / 15.0) + np.exp((V + 55.0) / 15.0)) + 1.6)}
    if name == "Ca_ZH2019_IO":  # calcium.py:4837-4979
        return {"h": ("it", 1.0 / (1.0 + np.exp((V + 85.5) / 8.6)),
                      40.0 + 30.0 * (1.0 / (1.0 + np.exp((V + 84.0) / 7.3))) * np.exp((V + 160.0) / 30.0))}
    if name in ("KM_RI2021_SC", "KM_MA2020_GoC", "KM_MA2020_GrC"):  # potassium.py:1735-1748, :4553-4567, :5317-5331
        a = 0.0033 * np.exp((V + 30.0) / 40.0)
        b = 0.0033 * np.exp((V + 30.0) / -20.0)
        return {"n": ("it", 1.0 / (1.0 + np.exp(-(V + 35.0) / 6.0)), 1.0 / (a + b))}
    raise KeyError(name)


_GATES = {  # (gate, power, phi-key)
    "Na_Ba2002": (("p", 3, "phi"), ("q", 1, "phi")),
    "KDR_Ba2002": (("p", 4, "phi"),),
    "CaL_IS2008": (("p", 2, "phi_p"), ("q", 1, "phi_q")),
    "CaT_HM1992": (("p", 2, "phi_p"), ("q", 1, "phi_q")),
    "HCN_HM1992": (("p", 1, "phi"),),
    "AHP_De1994": (("p", 2, "phi"),),
    "Na_HH1952": (("p", 3, "phi"), ("q", 1, "phi")),
    "K_HH1952": (("p", 4, "phi"),),
    "KM_RI2021_SC": (("n", 1, "phi"),),
    "KM_MA2020_GoC": (("n", 1, "phi"),),
    "KM_MA2020_GrC": (("n", 1, "phi"),),
    "Na_TM1991": (("p", 3, "phi"), ("q", 1, "phi")),
    "K_TM1991": (("p", 4, "phi"),),
    "CaHT_HM1992": (("p", 2, "phi_p"), ("q", 1, "phi_q")),
    "KA1_HM1992": (("p", 4, "phi_p"), ("q", 1, "phi_q")),
    "KA2_HM1992": (("p", 4, "phi_p"), ("q", 1, "phi_q")),
    "KK2A_HM1992": (("p", 1, "phi_p"), ("q", 1, "phi_q")),
    "KK2B_HM1992": (("p", 1, "phi_p"), ("q", 1, "phi_q")),
    "KNI_Ya1989": (("p", 1, "phi"),),
    "Kv3p4_MA2020_GoC": (("m", 3, "phi"), ("h", 1, "phi")),
    "Kv4p3_MA2020_GoC": (("a", 3, "phi"), ("b", 1, "phi")),
    "Kv1p1_MA2020_GoC": (("n", 4, "phi"),),
    "Kir2p3_MA2020_GrC": (("d", 1, "phi"),),
    "HCN1_MA2020_GoC": (("o_fast", 1, "phi"), ("o_slow", 1, "phi")),
    "HCN1_MA2024_PC": (("h", 1, "phi"),),
    "CaHVA_MA2020_GoC": (("s", 2, "phi"), ("u", 1, "phi")),
    "Cav2p3_MA2020_GoC": (("m", 3, "phi"), ("h", 1, "phi")),
    "Cav3p2_RI2021_SC": (("m", 2, "phi_m"), ("h", 1, "phi")),
    "HCN2_MA2020_GoC": (("o_fast", 1, "phi"), ("o_slow", 1, "phi")),
    "Kv3p3_MA2024_PC": (("n", 4, "phi"),),
    "Kv2p2_0010_MA2020_GrC": (("m", 1, "phi"), ("h", 1, "phi")),
    "Kv1p5_MA2024_PC": (("m", 3, "phi"), ("n", 1, "phi"), ("u", 1, "phi")),
    "NaF_SU2015_DCN": (("m", 3, "phi"), ("h", 1, "phi")),
    "NaP_SU2015_DCN": (("m", 3, "phi"), ("h", 1, "phi")),
    "Na_ZH2019_IO": (("m", 3, "phi"), ("h", 1, "phi")),
    "fKdr_SU2015_DCN": (("m", 4, "phi"),),
    "sKdr_SU2015_DCN": (("m", 4, "phi"),),
    "Kdr_ZH2019_IO": (("n", 4, "phi"),),
    "HCN_SU2015_DCN": (("m", 2, "phi"),),
    "HCN_ZH2019_IO": (("q", 1, "phi"),),
    "CaT_HP1992": (("p", 2, "phi_p"), ("q", 1, "phi_q")),
    "CaHT_Re1993": (("p", 2, "phi_p"), ("q", 1, "phi_q")),
    "CaL_SU2015_DCN": (("m", 2, "phi"), ("h", 1, "phi")),
    "Kca3p1_MA2020_GoC": (("p", 1, "phi"),),
    "SK_SU2015_DCN": (("z", 1, "phi"),),
    "K_Kv_test": (("n", 1, "phi"),),
    "CaN_IS2008": (("p", 1, "phi"),),
    "Ca_ZH2019_IO": (("h", 1, "phi"),),
    "Cav3p1_MA2020_GoC": (("p", 2, "phi"), ("q", 1, "phi")),
    "Cav3p1Test_PC24": (("p", 2, "phi"), ("q", 1, "phi")),
    "Cav3p3_RI2021_SC": (("n", 2, "phi"), ("l", 1, "phi")),
    "Cav1p2_MA2020_GoC": (("m", 1, "phi"), ("h", 1, "phi"), ("n", 1, "phi")),
    "Cav1p3_MA2020_GoC": (("m", 1, "phi"), ("h", 1, "phi"), ("n", 1, "phi")),
    "Cav2p1_RI2021_SC": (("m", 3, "phi"),),
    "CaHVA_SU2015_DCN": (("m", 3, "phi"),),
    "CaLVA_SU2015_DCN": (("m", 2, "phi"), ("h", 1, "phi")),
}
_ION_OF = {"Na_Ba2002": "na", "KDR_Ba2002": "k", "CaL_IS2008": "ca", "CaT_HM1992": "ca",
           "K_Leak": "k", "AHP_De1994": "k", "Na_HH1952": "na", "K_HH1952": "k", "KM_RI2021_SC": "k",
           "Na_TM1991": "na", "K_TM1991": "k", "CaHT_HM1992": "ca", "KA1_HM1992": "k", "KA2_HM1992": "k",
           "KM_MA2020_GoC": "k", "KM_MA2020_GrC": "k", "KK2A_HM1992": "k", "KK2B_HM1992": "k",
           "KNI_Ya1989": "k", "Nav1p6_MA2020_GoC": "na", "Kca2p2_MA2020_GoC": "k", "Kca1p1_MA2020_GoC": "k",
           "Kv3p4_MA2020_GoC": "k", "Kv4p3_MA2020_GoC": "k", "Kv1p1_MA2020_GoC": "k", "Kir2p3_MA2020_GrC": "k",
           "Nav1p1_MA2025_BC": "na", "Nav1p1_RI2021_SC": "na",
           "CaHVA_MA2020_GoC": "ca", "Cav2p3_MA2020_GoC": "ca", "Cav3p2_RI2021_SC": "ca",
           "Kv3p3_MA2024_PC": "k", "Kv2p2_0010_MA2020_GrC": "k", "Kv1p5_MA2024_PC": "k", "NaF_SU2015_DCN": "na",
           "NaP_SU2015_DCN": "na", "Na_ZH2019_IO": "na", "fKdr_SU2015_DCN": "k", "sKdr_SU2015_DCN": "k",
           "Kdr_ZH2019_IO": "k", "CaT_HP1992": "ca", "CaHT_Re1993": "ca", "Kca3p1_MA2020_GoC": "k",
           "SK_SU2015_DCN": "k", "K_Kv_test": "k", "CaN_IS2008": "ca", "Nav_MA2020_GrC": "na",
           "Cav3p1_MA2020_GoC": "ca", "Cav3p3_RI2021_SC": "ca", "Cav1p2_MA2020_GoC": "ca", "Cav1p3_MA2020_GoC": "ca",
           "Cav2p1_RI2021_SC": "ca", "CaHVA_SU2015_DCN": "ca", "CaLVA_SU2015_DCN": "ca",
           "Cav3p1Test_PC24": "ca"}
# calcium channels with a GHK current (-g gates drive) instead of an ohmic one
_GHK = ("Cav3p1_MA2020_GoC", "Cav3p3_RI2021_SC", "Cav2p1_RI2021_SC", "CaHVA_SU2015_DCN", "CaLVA_SU2015_DCN",
        "Cav3p1Test_PC24")
# channels with their own reversal potential (HHTypedNeuron root, not an ion)
_OWN_E = ("HCN_HM1992", "HCN1_MA2020_GoC", "HCN1_MA2024_PC", "HCN2_MA2020_GoC", "HCN_SU2015_DCN", "HCN_ZH2019_IO",
          "CaL_SU2015_DCN", "CaN_IS2008", "Ca_ZH2019_IO")


def _resolve(table: dict, decl) -> dict:
    base, own = _VARIANTS.get(decl.class_name, (decl.class_name, {}))
    p = {**table[base], **own}
    for k, v in decl.params.items():
        if k not in p:
            raise ValueError(f"{decl.class_name}: unknown parameter {k!r}.")
        p[k] = float(v)
    name = base
    if name in ("Na_Ba2002", "KDR_Ba2002", "HCN_HM1992", "Na_HH1952", "K_HH1952", "Na_TM1991", "K_TM1991",
                "KNI_Ya1989"):
        p["phi"] = p["q10"] ** ((p["temp"] - p["temp_ref"]) / 10.0)
    elif name in ("KM_RI2021_SC", "KM_MA2020_GoC", "KM_MA2020_GrC"):
        # Gate("n", q10=3.0, temp_ref=22 degC): potassium.py:1710, :4532, :5296
        p["phi"] = 3.0 ** ((p["temp"] - (273.15 + 22.0)) / 10.0)
    elif name in ("CaL_IS2008", "CaT_HM1992", "CaHT_HM1992", "KA1_HM1992", "KA2_HM1992", "KK2A_HM1992",
                  "KK2B_HM1992", "CaT_HP1992", "CaHT_Re1993"):
        p["phi_p"] = p["q10_p"] ** ((p["temp"] - p["temp_ref_p"]) / 10.0)
        p["phi_q"] = p["q10_q"] ** ((p["temp"] - p["temp_ref_q"]) / 10.0)
    elif name in MK.SCHEMES:
        p = MK.scheme_params(name, p)
    elif name == "Kv3p4_MA2020_GoC":  # Gate q10 3 at 37 degC
        p["phi"] = 3.0 ** ((p["temp"] - _c2k(37.0)) / 10.0)
    elif name == "Kv4p3_MA2020_GoC":  # Gate q10 3 at 25.5 degC
        p["phi"] = 3.0 ** ((p["temp"] - _c2k(25.5)) / 10.0)
    elif name == "Kv1p1_MA2020_GoC":  # Gate q10 2.7 at 22 degC
        if p["gateCurrent"] != 0.0:
            raise ValueError("Kv1p1 gating current not restated")
        p["phi"] = 2.7 ** ((p["temp"] - _c2k(22.0)) / 10.0)
    elif name == "Kir2p3_MA2020_GrC":  # Gate q10 3 at 20 degC
        p["phi"] = 3.0 ** ((p["temp"] - _c2k(20.0)) / 10.0)
    elif name == "HCN1_MA2020_GoC":  # gates q10 3 and the conductance Q10_diff 1.5, at 23 degC
        p["phi"] = 3.0 ** ((p["temp"] - _c2k(23.0)) / 10.0)
        p["gbar_phi"] = 1.5 ** ((p["temp"] - _c2k(23.0)) / 10.0)
    elif name == "HCN1_MA2024_PC":  # Gate q10 3 at 37 degC
        p["phi"] = 3.0 ** ((p["temp"] - _c2k(37.0)) / 10.0)
    elif name == "CaHVA_MA2020_GoC":  # Gates q10 3 at 20 degC
        p["phi"] = 3.0 ** ((p["temp"] - _c2k(20.0)) / 10.0)
    elif name == "Cav2p3_MA2020_GoC":  # Gates without q10 or phi: factor 1
        p["phi"] = 1.0
    elif name == "Cav3p2_RI2021_SC":  # Gate("m", phi=5^((36 - 24) / 10)); h: 1
        p["phi_m"] = 5.0 ** ((36.0 - 24.0) / 10.0)
        p["phi"] = 1.0
    elif name == "HCN2_MA2020_GoC":  # gates q10 3 and the conductance Q10_diff 1.5, at 23 degC
        p["phi"] = 3.0 ** ((p["temp"] - _c2k(23.0)) / 10.0)
        p["gbar_phi"] = 1.5 ** ((p["temp"] - _c2k(23.0)) / 10.0)
    if name == "Cav2p1_RI2021_SC":  # Gate q10 3 at 23 degC
        p["phi"] = 3.0 ** ((p["temp"] - _c2k(23.0)) / 10.0)
    if name in ("CaHVA_SU2015_DCN", "CaLVA_SU2015_DCN"):  # gates without a temperature factor; g = perm
        p["phi"] = 1.0
        p["g_max"] = p["perm"]
    if name in ("CaN_IS2008", "Cav1p2_MA2020_GoC", "Cav1p3_MA2020_GoC"):  # Gates (q10, temp_ref)
        p["phi"] = p["q10"] ** ((p["temp"] - p["temp_ref"]) / 10.0)
    if name in ("Cav3p1_MA2020_GoC", "Cav3p3_RI2021_SC", "Cav2p1_RI2021_SC"):  # _Frozen: drive out of the linearisation
        p["ghk_frozen"] = 1.0 if decl.class_name.endswith("_Frozen") else 0.0
    if name == "Cav3p1Test_PC24":  # Cav3p1's gates with the fixed 1 mV drive
        p["phi"] = 1.0
        p["ghk_frozen"] = 2.0
    if name == "Cav3p3_RI2021_SC":  # Gates q10 2.3 at 28 degC; g = g_scale perm
        p["phi"] = 2.3 ** ((p["temp"] - _c2k(28.0)) / 10.0)
        p["g_max"] = p["g_scale"] * p["perm"]
    if p.get("gnonspec", 0.0) != 0.0:
        raise ValueError("Kv1p5_MA2020_GrC's nonspecific current (gnonspec != 0) not restated")
    p.pop("gnonspec", None)
    if name == "Kv3p3_MA2024_PC":  # Gate q10 2.7 at 22 degC
        if p["gateCurrent"] != 0.0:
            raise ValueError("Kv3p3 gating current not restated")
        p["phi"] = 2.7 ** ((p["temp"] - _c2k(22.0)) / 10.0)
    elif name in ("Kv2p2_0010_MA2020_GrC", "Kv1p5_MA2024_PC", "NaF_SU2015_DCN", "NaP_SU2015_DCN", "Na_ZH2019_IO",
                  "fKdr_SU2015_DCN", "sKdr_SU2015_DCN", "Kdr_ZH2019_IO", "HCN_SU2015_DCN", "HCN_ZH2019_IO",
                  "CaL_SU2015_DCN", "Kca3p1_MA2020_GoC", "SK_SU2015_DCN", "K_Kv_test", "Ca_ZH2019_IO",
                  "Cav3p1_MA2020_GoC"):
        p["phi"] = 1.0  # gates without q10 or phi (Kv1p5's Q10 sits in its rates)
    return p


# ----------------------------------------------------------------------------- the cell


class OracleCell:
    """Float64 restatement of one reference ``Cell`` stepped with ``"staggered"``.

    ``cell`` is a declared :class:`braincell_gb300.cell.Cell` (morphology, CV
    policy, paint and place rules, population size); only its declarations are
    read.  States are dense over points with ``g = 0`` off the painted mask, as in
    ``_compute/bindings.py:569-757``.
    """

    MAX_GROUP = 256  # Cell.node_scheduling default (cell.py:1282)

    def __init__(self, cell, *, replicas: int | None = None) -> None:
        self.P = int(np.prod(cell.pop_size)) if replicas is None else int(replicas)
        self.V_th = float(cell.V_th)
        self._discretize(cell)
        self._node_tree()
        self._schedule()
        self._static_source()
        self._mechanisms(cell)
        self._points(cell)
        self.t_step = 0
        self.reset_state()

    # ------------------------------------------------------------ discretization
    def _discretize(self, cell) -> None:
        from braincell_gb300.mech import CableProperty

        morpho = cell.morpho
        self.morpho = morpho
        branches = morpho.branches
        counts = cell.cv_policy.cv_counts(morpho)
        # cable per branch: last painted CableProperty wins (default cable otherwise)
        cable = [CableProperty() for _ in branches]
        mech_by_branch: list[list] = [[] for _ in branches]
        for region, decls in cell.paint_rules:
            mask = region.branch_mask(morpho)
            for d in decls:
                for b in np.nonzero(mask)[0]:
                    if isinstance(d, CableProperty):
                        cable[b] = d
                    else:
                        mech_by_branch[b].append(d)
        self.cv_branch, self.cv_prox, self.cv_dist = [], [], []
        self.cv_area, self.cv_rprox, self.cv_rdist, self.cv_cm, self.cv_v = [], [], [], [], []
        self.branch_cv_ids: list[list[int]] = []
        self.branch_mechs = mech_by_branch
        cid = 0
        for b, br in enumerate(branches):
            ids = []
            n = int(counts[b])
            for k in range(n):
                prox, dist = k / n, (k + 1) / n
                fr = build_frusta(br.lengths, br.radii_proximal, br.radii_distal, prox, dist)
                area = lateral_area_um2(fr)
                left, right = split_frusta(fr, 0.5 * (prox + dist))
                fp = axial_factor_per_cm(left) if left else 0.0
                fd = axial_factor_per_cm(right) if right else 0.0
                ra = float(cable[b].axial_resistivity)
                self.cv_branch.append(b)
                self.cv_prox.append(prox)
                self.cv_dist.append(dist)
                self.cv_area.append(area)
                self.cv_rprox.append(ra * fp)
                self.cv_rdist.append(ra * fd)
                self.cv_cm.append(float(cable[b].membrane_capacitance))
                self.cv_v.append(float(cable[b].resting_potential))
                ids.append(cid)
                cid += 1
            self.branch_cv_ids.append(ids)
        self.n_cv = cid
        self.cv_area = np.asarray(self.cv_area)
        self.cv_cm = np.asarray(self.cv_cm)
        self.cv_v = np.asarray(self.cv_v)
        if cell.V_init is not None:
            self.cv_v[:] = float(cell.V_init)

    def _locate_cv(self, b: int, x: float) -> int:
        ids = self.branch_cv_ids[b]
        if x <= 0.0 + EPS_PARAM:
            return ids[0]
        if x >= 1.0 - EPS_PARAM:
            return ids[-1]
        for c in ids:
            if self.cv_prox[c] - EPS_PARAM <= x < self.cv_dist[c] - EPS_PARAM:
                return c
        for c in ids:
            if abs(x - self.cv_dist[c]) <= EPS_PARAM:
                return c
        raise ValueError(f"x={x} not owned by any CV of branch {b}.")

    def _node_tree(self) -> None:
        """``build_node_tree_from_cvs`` (node_build.py:58-285)."""
        morpho = self.morpho
        roles: list[set] = []
        cv_mid = np.full(self.n_cv, -1, dtype=np.int64)
        endpoint: dict[tuple[int, float], int] = {}
        edge_roles: dict[tuple[int, int], list] = {}
        edge_order: list[tuple[int, int]] = []

        def new_node(cv_id, pos):
            roles.append({(cv_id, pos)})
            return len(roles) - 1

        def add_edge(p, c, cv_id, half):
            key = (p, c)
            if key not in edge_roles:
                edge_roles[key] = []
                edge_order.append(key)
            if (cv_id, half) not in edge_roles[key]:
                edge_roles[key].append((cv_id, half))

        parent_x = {e.child.index: e.parent_x for e in morpho.edges}
        child_x = {e.child.index: e.child_x for e in morpho.edges}
        parent_of = {e.child.index: e.parent.index for e in morpho.edges}
        root = new_node(self.branch_cv_ids[0][0], "prox")
        endpoint[(0, 0.0)] = root
        for b in range(len(morpho.branches)):
            ids = self.branch_cv_ids[b]
            if b == 0:
                att, ax, order = root, 0.0, ids
            else:
                px = float(parent_x[b])
                pb = parent_of[b]
                if px <= EPS_PARAM:
                    att = endpoint[(pb, 0.0)]
                elif px >= 1.0 - EPS_PARAM:
                    att = endpoint[(pb, 1.0)]
                else:
                    att = int(cv_mid[self._locate_cv(pb, px)])
                ax = float(child_x[b])
                order = ids if ax <= EPS_PARAM else list(reversed(ids))
            entry = "prox" if ax <= EPS_PARAM else "dist"
            exit_ = "dist" if ax <= EPS_PARAM else "prox"
            roles[att].add((order[0], entry))
            endpoint[(b, float(ax))] = att
            for c in order:
                cv_mid[c] = new_node(c, "mid")
            term = new_node(order[-1], exit_)
            endpoint[(b, float(1.0 - ax))] = term
            for i, c in enumerate(order):
                mid = int(cv_mid[c])
                par = att if i == 0 else int(cv_mid[order[i - 1]])
                chi = term if i == len(order) - 1 else int(cv_mid[order[i + 1]])
                add_edge(par, mid, c, entry)
                add_edge(mid, chi, c, exit_)
        self.n_point = len(roles)
        self.cv_mid = cv_mid
        self.is_mid = np.zeros(self.n_point, dtype=bool)
        self.is_mid[cv_mid] = True
        self.endpoint = endpoint
        self.edges = []
        for key in edge_order:
            rl = sorted(edge_roles[key])
            self.edges.append((key[0], key[1], rl))

    def _schedule(self) -> None:
        n = self.n_point
        node_parent = np.full(n, -1, dtype=np.int32)
        children: list[list[int]] = [[] for _ in range(n)]
        for p, c, _ in self.edges:
            if node_parent[c] != -1:
                raise ValueError("node has two parents")
            node_parent[c] = p
            children[p].append(c)
        peel = compute_peel_levels(node_parent, children)
        order = np.lexsort((np.arange(n, dtype=np.int32), -peel)).astype(np.int32)
        row_of = np.empty(n, dtype=np.int32)
        row_of[order] = np.arange(n, dtype=np.int32)
        parent_rows = np.full(n, -1, dtype=np.int32)
        for row, pid in enumerate(order.tolist()):
            if node_parent[pid] >= 0:
                parent_rows[row] = row_of[node_parent[pid]]
        peels_ordered = peel[order]
        starts = [0] + [i for i in range(1, n) if peels_ordered[i] != peels_ordered[i - 1]] + [n]
        groups = []
        for a, b in zip(starts[:-1], starts[1:]):
            for s in range(a, b, self.MAX_GROUP):
                groups.append(row_of[order[s:min(b, s + self.MAX_GROUP)]])
        self.row_to_point = order
        self.point_to_row = row_of
        self.parent_rows = parent_rows
        self.groups = groups
        self.node_parent = node_parent
        self.peel = peel

    def _static_source(self) -> None:
        n = self.n_point
        row_of = self.point_to_row
        dyn_rows = row_of[self.cv_mid]
        cap_F = np.full(n, 1e-6)  # boundary rows: dummy 1 uF (_staggered.py:579-593)
        cap_F[dyn_rows] = self.cv_area * 1e-8 * self.cv_cm * 1e-6
        diag = np.zeros(n)
        A_pc = {}
        for p_id, c_id, rl in self.edges:
            pr, cr = int(row_of[p_id]), int(row_of[c_id])
            res = [self.cv_rprox[c] if h == "prox" else self.cv_rdist[c] for c, h in rl]
            br_ids = {self.cv_branch[c] for c, _ in rl}
            if len(res) > 1 and len(br_ids) == 1:
                g = 1.0 / sum(res)
            else:
                g = sum(1.0 / r for r in res)
            pc = g / cap_F[pr] * 1e-3  # ms^-1
            cc = g / cap_F[cr] * 1e-3
            diag[pr] += pc
            diag[cr] += cc
            A_pc[(pr, cr)] = -pc
            A_pc[(cr, pr)] = -cc
        lowers = np.zeros(n)
        uppers = np.zeros(n)
        for row, prow in enumerate(self.parent_rows.tolist()):
            if prow < 0:
                continue
            lowers[row] = A_pc[(row, prow)]
            uppers[row] = A_pc[(prow, row)]
        parent_lookup = np.empty(n + 1, dtype=np.int32)
        parent_lookup[:n] = np.where(self.parent_rows >= 0, self.parent_rows, n)
        parent_lookup[n] = n
        edges, level_size = [], []
        for grp in reversed(self.groups):
            le = [[int(r), int(self.parent_rows[r])] for r in grp.tolist() if self.parent_rows[r] >= 0]
            if le:
                edges.extend(le)
                level_size.append(len(le))
        self.dhs_edges = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
        self.level_offsets = np.cumsum([0] + level_size).astype(np.int64)
        self.backsub = build_backsub_indices(parent_lookup, n)
        self.dyn_rows = dyn_rows
        self.diag_ms = diag
        self.lowers_ms = lowers
        self.uppers_ms = uppers
        self.row_cap_uF = cap_F * 1e6

    # ------------------------------------------------------------ mechanisms
    def _mechanisms(self, cell) -> None:
        """Dense point-space parameters (g = 0 off the painted points)."""
        from braincell_gb300.mech import Channel, Ion

        n = self.n_point
        self.chan = {}  # name -> dict(param arrays over points, mask)
        self.E_na = np.full(n, ION_DEFAULTS["SodiumFixed"]["E"])
        self.E_k = np.full(n, ION_DEFAULTS["PotassiumFixed"]["E"])
        self.E_ca_fixed = np.full(n, ION_DEFAULTS["CalciumFixed"]["E"])
        self.ca_dyn = None
        for b, decls in enumerate(self.branch_mechs):
            last = {}
            for d in decls:
                last[("IL" if d.class_name == "leaky" else _base_class(d.class_name))] = d
            pts = self.cv_mid[self.branch_cv_ids[b]]
            for name, d in last.items():
                if isinstance(d, Ion):
                    p = _resolve(ION_DEFAULTS, d)
                    if name == "SodiumFixed":
                        self.E_na[pts] = p["E"]
                    elif name == "PotassiumFixed":
                        self.E_k[pts] = p["E"]
                    elif name == "CalciumFixed":
                        self.E_ca_fixed[pts] = p["E"]
                    elif name.endswith("InitNernst"):
                        e = 1e3 * GAS_R * p["temp"] / (p["valence"] * FARADAY) * np.log(p["Co"] / p["Ci"])
                        {"Sodium": self.E_na, "Potassium": self.E_k, "Calcium": self.E_ca_fixed}[
                            name[: -len("InitNernst")]][pts] = e
                    elif name == "CalciumDetailed":
                        if self.ca_dyn is None:
                            self.ca_dyn = {k: np.zeros(n) for k in ("d", "tau", "C_rest", "Co", "temp", "Ci0")}
                            self.ca_dyn["d"][:] = 1.0
                            self.ca_dyn["tau"][:] = 1.0
                            self.ca_dyn["C_rest"][:] = ION_DEFAULTS["CalciumDetailed"]["C_rest"]
                            self.ca_dyn["Co"][:] = ION_DEFAULTS["CalciumDetailed"]["Co"]
                            self.ca_dyn["temp"][:] = ION_DEFAULTS["CalciumDetailed"]["temp"]
                            self.ca_dyn["Ci0"][:] = _CA_FIXED_CI
                            self.ca_dyn["mask"] = np.zeros(n, dtype=bool)
                        for k, src in (("d", "d"), ("tau", "tau"), ("C_rest", "C_rest"), ("Co", "Co"),
                                       ("temp", "temp"), ("Ci0", "Ci_initializer")):
                            self.ca_dyn[k][pts] = p[src]
                        self.ca_dyn["mask"][pts] = True
                    else:
                        raise ValueError(f"unsupported ion {name}")
                    continue
                assert isinstance(d, Channel)
                p = _resolve(CHANNEL_DEFAULTS, d)
                if name not in self.chan:
                    # dense over points: conductance 0 off the painted mask, every other
                    # parameter broadcast from the first painted value (bindings.py:723-741)
                    self.chan[name] = {"mask": np.zeros(n, dtype=bool)}
                    for k, v in p.items():
                        self.chan[name][k] = np.zeros(n) if k == "g_max" else np.full(n, float(v))
                ch = self.chan[name]
                ch["mask"][pts] = True
                for k, v in p.items():
                    if k not in ch:
                        ch[k] = np.zeros(n)
                    ch[k][pts] = v
        # the fixed-Ca Ci seen by AHP where no dynamic calcium is painted
        self.Ci_fixed = np.full(n, _CA_FIXED_CI)

    def _points(self, cell) -> None:
        from braincell_gb300.mech import CurrentClamp, CurrentProbe, ExpSyn, MechanismProbe, StateProbe

        self.clamps_mid = []  # (point, t_on, t_off, amp_nA)
        self.clamps_edge = []
        self.probe_points = []
        self.probe_what = []  # None: V; else ("gate", channel, gate) or ("Ci",)
        self.syn_points, self.syn_tau, self.syn_e = [], [], []  # ExpSyn at CV midpoints
        for locset, decls in cell.place_rules:
            for (b, x) in locset.points(self.morpho):
                if x <= EPS_PARAM:
                    pid = self.endpoint[(b, 0.0)] if (b, 0.0) in self.endpoint else None
                elif x >= 1.0 - EPS_PARAM:
                    pid = self.endpoint[(b, 1.0)] if (b, 1.0) in self.endpoint else None
                else:
                    pid = int(self.cv_mid[self._locate_cv(b, x)])
                if pid is None:
                    raise ValueError("locset point not found")
                for d in decls:
                    if isinstance(d, CurrentClamp):
                        for (t_on, t_off, amp) in d.segments():
                            (self.clamps_mid if self.is_mid[pid] else self.clamps_edge).append((pid, t_on, t_off, amp))
                    elif isinstance(d, StateProbe):
                        self.probe_points.append(pid)
                        self.probe_what.append(None)
                    elif isinstance(d, MechanismProbe):
                        # probes.py:136-181: the named mechanism's (or ion's) field at the point
                        self.probe_points.append(pid)
                        self.probe_what.append(self._probe_key(cell, b, d))
                    elif isinstance(d, CurrentProbe):
                        # probes.py:184-258: a channel's current, or an ion's total
                        self.probe_points.append(pid)
                        if d.mechanism is not None:
                            key = self._probe_key(cell, b, MechanismProbe(d.mechanism, "p", name=d.name))
                            self.probe_what.append(("cur", key[1]))
                        else:
                            self.probe_what.append(("ion", d.ion))
                    elif isinstance(d, ExpSyn):
                        if not self.is_mid[pid]:
                            raise ValueError("ExpSyn must sit inside a CV, not on a branch end point.")
                        self.syn_points.append(pid)
                        self.syn_tau.append(d.tau)
                        self.syn_e.append(d.e)
        self.point_area_um2 = np.zeros(self.n_point)
        self.point_area_um2[self.cv_mid] = self.cv_area

    def _probe_key(self, cell, b: int, d):
        names = {}
        for region, decls in cell.paint_rules:
            if region.branch_mask(self.morpho)[b]:
                for m in decls:
                    if hasattr(m, "class_name"):
                        names[m.instance_name] = m.class_name
        if d.mechanism not in names:
            raise KeyError(f"no mechanism named {d.mechanism!r} at the probe")
        cls = _base_class(names[d.mechanism])
        if d.field == "Ci":
            return ("Ci",)
        return ("gate", cls, d.field)

    # ------------------------------------------------------------ surrogate ports
    def set_ports(self, ports, theta, v_scale: float, y_scale: float) -> None:
        """Subtree-surrogate ports (no counterpart in the reference).

        ``ports``: dicts with ``branch`` (the port feeds that branch's x = 1
        endpoint; its attachment CV is the branch's last CV), ``g`` (uS), ``e``
        (mV), ``feat`` (two floats) and ``stim`` [(t_on, t_off, amp_nA)].  Every
        step each port runs one GRU step (``oracle/gru.py``, BF16 rounding as the
        kernels) on ((V_att - e) / v_scale, S / 0.1 nA, feat) and injects
        g (e + y_scale y - V_end) nA into its endpoint row, the -g V_end part
        implicitly.
        """
        from oracle import gru as G

        row_of = np.empty(self.n_point, np.int64)
        row_of[self.row_to_point] = np.arange(self.n_point)
        self.ports = []
        for pt in ports:
            b = int(pt["branch"])
            end = self.endpoint[(b, 1.0)]
            att = int(self.branch_cv_ids[b][-1])
            self.ports.append(dict(row=int(row_of[end]), att=att, g=float(pt["g"]), e=float(pt["e"]),
                                   feat=np.asarray(pt["feat"], float), stim=list(pt.get("stim", ()))))
        self.port_theta = np.asarray(theta, float)
        self.port_norm = (float(v_scale), float(y_scale))
        self.port_h = np.zeros((self.P, len(self.ports), G.H))

    def _port_rows(self, diags, solves, V_n, t: float, dt: float) -> None:
        from oracle import gru as G

        v_scale, y_scale = self.port_norm
        P, K = self.P, len(self.ports)
        x = np.zeros((P, K, G.X))
        for k, pt in enumerate(self.ports):
            S = sum(amp for (t_on, t_off, amp) in pt["stim"] if t_on <= t < t_off)
            x[:, k, 0] = (V_n[:, pt["att"]] - pt["e"]) / v_scale
            x[:, k, 1] = S / 0.1  # nA, the stimulus input scale
            x[:, k, 2:] = pt["feat"]
        h, y = G.step(self.port_theta, x.reshape(P * K, G.X), self.port_h.reshape(P * K, G.H), quantize=True)
        self.port_h = h.reshape(P, K, G.H)
        y = y.reshape(P, K)
        for k, pt in enumerate(self.ports):
            gg = dt * pt["g"] * 1e-3  # uS on a row with the 1 uF dummy capacitance
            diags[:, pt["row"]] += gg
            solves[:, pt["row"]] += gg * (pt["e"] + y_scale * y[:, k])

    # ------------------------------------------------------------ state
    def reset_state(self) -> None:
        """``Cell.reset_state`` (cell.py:2529-2550) + ``HH.reset_state`` (channel/_base.py:560-573)."""
        P, n = self.P, self.n_point
        self.V = np.broadcast_to(self.cv_v, (P, self.n_cv)).copy()
        self.t_step = 0
        pv = self.cv_to_point(self.V)
        self.Ci = None
        if self.ca_dyn is not None:
            self.Ci = np.broadcast_to(self.ca_dyn["Ci0"], (P, n)).copy()
        self.gates = {}
        for name, ch in self.chan.items():
            if name not in _GATES:
                continue
            r = rates(name, pv, ch, Ci=self._ci_for_channels())
            for gate, _power, _phik in _GATES[name]:
                kind, a, b = r[gate]
                self.gates[(name, gate)] = (a / (a + b) if kind == "ab" else a) * np.ones((P, n))
        # Markov channels start at their stationary distribution at V_init
        # (Nav1p6 / Kca2p2 / Kca1p1 reset_state -> Markov.reset_steady_state)
        for name, ch in self.chan.items():
            if name not in MK.SCHEMES:
                continue
            sch = MK.SCHEMES[name]
            ss = MK.steady_state(sch, sch.rates(pv, self._ci_for_channels(), ch))
            for st in sch.independent:
                self.gates[(name, st)] = ss[st] * np.ones((P, n))
        self.spike = np.zeros((P, self.n_cv))
        self.syn_g = np.zeros((P, len(self.syn_points)))  # uS
        self.syn_pending = np.zeros((P, len(self.syn_points)))

    def add_events(self, weights) -> None:
        """Event weights (uS, ``[P, n_syn]``) applied at the start of the next step
        (``Cell._begin_step``, cell.py:2331-2346; ``ExpSyn.apply_discrete_events``,
        synapse/markov.py:104-106)."""
        self.syn_pending = self.syn_pending + np.asarray(weights, dtype=np.float64)

    def population_spike(self) -> np.ndarray:
        """One spike flag per replica: any CV crossed (network/delivery.py:103-123)."""
        return self.spike.any(axis=1)

    def cv_to_point(self, v):
        out = np.zeros(v.shape[:-1] + (self.n_point,))
        out[..., self.cv_mid] = v
        return out

    def _ci_for_channels(self):
        if self.Ci is None:
            return self.Ci_fixed
        return np.where(self.ca_dyn["mask"], self.Ci, self.Ci_fixed)

    def _ghk(self, name, ch, pv):
        """(drive, d drive / dV) of a GHK calcium channel at the point voltages."""
        if name == "Cav3p1_MA2020_GoC":
            return cav31_drive(pv, self._ci_for_channels(), self._co_for_channels(), ch["temp"])
        if name == "Cav3p1Test_PC24":  # the fixed 1 mV drive
            return np.ones_like(pv), np.zeros_like(pv)
        if name == "Cav2p1_RI2021_SC":  # the _Frozen classes: the Cav3.1 model-file helper (calcium.py, their current)
            args = (pv - ch["V_sh"], self._ci_for_channels(), self._co_for_channels(), ch["temp"])
            shared, nmodl = ghk_codata_drive(*args), cav31_drive(*args)
            fr = np.asarray(ch["ghk_frozen"]) != 0.0
            return np.where(fr, nmodl[0], shared[0]), np.where(fr, nmodl[1], shared[1])
        if name in ("CaHVA_SU2015_DCN", "CaLVA_SU2015_DCN"):
            return su2015_drive(pv, self._ci_for_channels(), self._co_for_channels(), ch["temp"])
        return cav33_drive(pv - ch["V_sh"], self._ci_for_channels(), self._co_for_channels(), ch["temp"])

    def _co_for_channels(self):
        """Co of the calcium ion: the dynamic shell's, else the fixed ion's 2 mM
        (ion/calcium.py:121)."""
        if self.ca_dyn is None:
            return 2.0
        return np.where(self.ca_dyn["mask"], self.ca_dyn["Co"], 2.0)

    def _E_ca(self):
        if self.Ci is None:
            return self.E_ca_fixed
        cd = self.ca_dyn
        nernst = nernst_ca_mV(cd["temp"], cd["Co"], np.where(cd["mask"], self.Ci, 1.0))
        return np.where(cd["mask"], nernst, self.E_ca_fixed)

    def _gate_product(self, name):
        if name == "CaN_IS2008":  # p Ci / (Ci + 0.2 mM)
            return can_modulation(self._ci_for_channels()) * self.gates[(name, "p")]
        if name in ("HCN1_MA2020_GoC", "HCN2_MA2020_GoC"):  # g (o_fast + o_slow) with the conductance's Q10 factor
            return self.chan[name]["gbar_phi"] * (self.gates[(name, "o_fast")] + self.gates[(name, "o_slow")])
        if name in MK.SCHEMES:  # the open occupancy of the raw stored states
            sch = MK.SCHEMES[name]
            return MK.open_fraction(sch, {st: self.gates[(name, st)] for st in sch.independent})
        prod = 1.0
        for gate, power, _ in _GATES[name]:
            x = self.gates[(name, gate)]
            prod = prod * (x if power == 1 else x ** power)
        return prod

    def _channel_currents(self, pv):
        """Total ionic current density and its V-derivative (uA/cm^2, uA/cm^2/mV) per point."""
        I = np.zeros_like(pv)
        dI = np.zeros_like(pv)
        E_ca = self._E_ca()
        E_of = {"na": self.E_na, "k": self.E_k, "ca": E_ca}
        for name, ch in self.chan.items():
            g = ch["g_max"]
            if name == "IL":
                E = ch["E"]
                fac = 1.0
            elif name == "K_Leak":
                E, fac = self.E_k, 1.0
            elif name in _OWN_E:
                E, fac = ch["E"], self._gate_product(name)
            else:
                E, fac = E_of[_ION_OF[name]], self._gate_product(name)
            geff = g * fac
            if name == "Kv1p5_MA2024_PC":  # g f(V) gates (E - V): dI/dV = g gates (f'(V) (E - V) - f(V))
                f, df = kv15_vfactor(pv)
                I = I + geff * f * (E - pv)
                dI = dI + geff * (df * (E - pv) - f)
                continue
            if name in _GHK:  # -g gates drive(V): dI/dV = -g gates d drive / dV
                drive, dd = self._ghk(name, ch, pv)
                I = I - geff * drive
                frozen = ch.get("ghk_frozen", 0.0)  # Cav2p1 has no _Frozen class built
                dI = dI - np.where(np.asarray(frozen) != 0.0, 0.0, geff * dd)
                continue
            if name == "Ca_ZH2019_IO":  # g m_inf(V) h (E - V); a frozen m_inf is out of the derivative
                m, dm = caio_minf(pv, ch["mMidV"])
                I = I + geff * m * (E - pv)
                frozen = ch["freeze_m_inf"] != 0.0
                dI = dI - geff * m + np.where(frozen, 0.0, geff * dm * (E - pv))
                continue
            I = I + geff * (E - pv)
            dI = dI - geff
        return I, dI

    def _probe_current(self, what, pid):
        """A current probe's value at point pid after the step (uA/cm^2)."""
        pv = self.cv_to_point(self.V)
        E_ca = self._E_ca()
        E_of = {"na": self.E_na, "k": self.E_k, "ca": E_ca}

        def one(name):
            ch = self.chan[name]
            if name == "IL":
                E, fac = ch["E"], 1.0
            elif name == "K_Leak":
                E, fac = self.E_k, 1.0
            elif name in _OWN_E:
                E, fac = ch["E"], self._gate_product(name)
            else:
                E, fac = E_of[_ION_OF[name]], self._gate_product(name)
            if name == "Kv1p5_MA2024_PC":
                fac = fac * kv15_vfactor(pv)[0]
            if name == "Ca_ZH2019_IO":
                fac = fac * caio_minf(pv, ch["mMidV"])[0]
            if name in _GHK:
                cur = -ch["g_max"] * fac * self._ghk(name, ch, pv)[0]
                return cur[:, pid] if np.ndim(cur) == 2 else np.full(self.P, float(cur))
            cur = ch["g_max"] * fac * (E - pv)
            return cur[:, pid] if np.ndim(cur) == 2 else np.full(self.P, float(cur))

        if what[0] == "cur":
            return one(what[1])
        total = np.zeros(self.P)
        for name in self.chan:
            if _ION_OF.get(name) == what[1]:
                total = total + one(name)
        return total

    def _ca_current(self, pv):
        """``Ion.current`` of the calcium ion (sum over its channels), uA/cm^2."""
        I = np.zeros_like(pv)
        E_ca = self._E_ca()
        for name in self.chan:
            if _ION_OF.get(name) == "ca":
                if name in _GHK:  # the GHK drive
                    ch = self.chan[name]
                    I = I - ch["g_max"] * self._gate_product(name) * self._ghk(name, ch, pv)[0]
                    continue
                E = self.chan[name]["E"] if name in _OWN_E else E_ca  # CaN_IS2008 carries calcium in its own E
                I = I + self.chan[name]["g_max"] * self._gate_product(name) * (E - pv)
        return I

    def _clamp_nA(self, clamps, t: float):
        cur = np.zeros((self.P, self.n_point))
        for pid, t_on, t_off, amp in clamps:
            lt = t  # absolute time; delay folded into t_on/t_off
            if t_on <= lt < t_off:
                cur[:, pid] += amp
        return cur

    # ------------------------------------------------------------ one step
    def step(self, dt: float, t: float | None = None) -> np.ndarray:
        """Advance one staggered step; returns the spike indicator ``(P, n_cv)``."""
        if t is None:
            t = self.t_step * dt
        P = self.P
        n = self.n_point
        V_n = self.V
        last_V = V_n
        pv = self.cv_to_point(V_n)
        # a2: cache ion total current at step start
        I_ca_cached = self._ca_current(pv) if self.Ci is not None else None
        # a6: linearise (point mode): derivative = I/C at midpoints, linear = dI/dV / C
        I_pt, dI_pt = self._channel_currents(pv)
        clamp_nA = self._clamp_nA(self.clamps_mid, t)
        safe_area = np.where(self.is_mid, self.point_area_um2, 1.0)
        I_pt = I_pt + np.where(self.is_mid, clamp_nA * 1e5 / safe_area, 0.0)
        if self.syn_points:
            # events of this step first, then the synapse current g (e - V) as a
            # total (nA) point current turned into a density like a clamp
            self.syn_g = self.syn_g + self.syn_pending
            self.syn_pending = np.zeros_like(self.syn_pending)
            for k, pid in enumerate(self.syn_points):
                g = self.syn_g[:, k] * 1e5 / self.point_area_um2[pid]  # uS -> mS/cm^2 over the CV
                I_pt[:, pid] += g * (self.syn_e[k] - pv[:, pid])
                dI_pt[:, pid] -= g
        C_pt = np.ones(n)
        C_pt[self.cv_mid] = self.cv_cm
        deriv = np.where(self.is_mid, I_pt / C_pt, 0.0)
        lin = np.where(self.is_mid, dI_pt / C_pt, 0.0)
        linear = lin[:, self.cv_mid]
        derivative = deriv[:, self.cv_mid]
        const = derivative - V_n * linear
        # a7: numeric state
        diags = np.broadcast_to(np.concatenate([self.diag_ms * dt, [1.0]]), (P, n + 1)).copy()
        diags[:, self.dyn_rows] += 1.0 - dt * linear
        solves = np.zeros((P, n + 1))
        solves[:, self.dyn_rows] = V_n + dt * const
        if self.clamps_edge:
            edge_nA = self._clamp_nA(self.clamps_edge, t)
            by_row = edge_nA[:, self.row_to_point]
            solves[:, :n] += dt * (by_row / self.row_cap_uF) * 1e-3
        if getattr(self, "ports", None):
            self._port_rows(diags, solves, V_n, t, dt)
        lowers = np.concatenate([self.lowers_ms * dt, [0.0]])
        uppers = np.concatenate([self.uppers_ms * dt, [0.0]])
        # a8: forward elimination, one level at a time (leaves first)
        E = self.dhs_edges
        for i in range(len(self.level_offsets) - 1):
            a, b = self.level_offsets[i], self.level_offsets[i + 1]
            ch, par = E[a:b, 0], E[a:b, 1]
            m = uppers[ch] / diags[:, ch]
            np.add.at(diags, (slice(None), par), -lowers[ch] * m)
            np.add.at(solves, (slice(None), par), -solves[:, ch] * m)
        # a9: recursive-doubling back substitution
        low = lowers.copy()
        low[0] = 0.0
        le = -low / diags
        se = solves / diags
        for k in self.backsub:
            se = se + le * se[:, k]
            le = le * le[:, k]
        # a10: restore midpoint voltage
        V_new = se[:, self.dyn_rows]
        self.V = V_new
        pv_new = self.cv_to_point(V_new)
        # runtime synapse dynamics after the voltage (quad/_staggered.py:144-145):
        # exp-Euler of g' = -g / tau, exact for this linear ODE
        for k in range(len(self.syn_points)):
            lam = -1.0 / self.syn_tau[k]
            self.syn_g[:, k] = self.syn_g[:, k] + dt * exprel(dt * lam) * (lam * self.syn_g[:, k])
        # a11 (a): dependent ion self states -- Ci with the cached step-start current
        if self.Ci is not None:
            cd = self.ca_dyn
            f = ca_detailed_rate(I_ca_cached, self.Ci, cd["d"], cd["tau"], cd["C_rest"])
            Ci_new = exp_euler(self.Ci, f, -1.0 / cd["tau"], dt)
            self.Ci = np.where(cd["mask"], Ci_new, self.Ci)
        # a11 (c): dependent channels, exp-Euler per gate at the new voltage (and new Ci)
        Ci_now = self._ci_for_channels()
        new_gates = {}
        for name, ch in self.chan.items():
            if name not in _GATES:
                continue
            r = rates(name, pv_new, ch, Ci=Ci_now)
            for gate, _power, phik in _GATES[name]:
                kind, a, b = r[gate]
                new_gates[(name, gate)] = gate_step(self.gates[(name, gate)], kind, a, b, ch[phik], dt)
        self.gates.update(new_gates)
        # a11 (d): independent channels through their own solver (cell.py:2204-2217):
        # Markov states by one backward-Euler step at the new voltage and Ci
        for name, ch in self.chan.items():
            if name not in MK.SCHEMES:
                continue
            sch = MK.SCHEMES[name]
            y = MK.backward_euler(sch, {st: self.gates[(name, st)] for st in sch.independent},
                                  sch.rates(pv_new, Ci_now, ch), dt)
            for st in sch.independent:
                self.gates[(name, st)] = y[st]
        # a16: spike = last_V < V_th <= V
        spk = ((V_new - self.V_th) >= 0.0) & ((self.V_th - last_V) > 0.0)
        self.spike = spk.astype(np.float64)
        self.t_step += 1
        return self.spike

    # ------------------------------------------------------------ time loop
    def run(self, dt: float, n_steps: int, record_every: int = 1):
        """Run ``n_steps``; return (probe traces [P, n_probe, n_rec], spike times per (P, probe))."""
        traces = []
        spikes = [[[] for _ in self.probe_points] for _ in range(self.P)]
        probe_cv = [int(np.nonzero(self.cv_mid == pid)[0][0]) if self.is_mid[pid] else None
                    for pid in self.probe_points]
        for s in range(n_steps):
            t = self.t_step * dt
            Vold = self.V.copy()
            self.step(dt, t)
            for j, c in enumerate(probe_cv):
                if c is None or (j < len(self.probe_what) and self.probe_what[j] is not None):
                    continue
                v0, v1 = Vold[:, c], self.V[:, c]
                hit = (v0 < self.V_th) & (v1 >= self.V_th)
                for p in np.nonzero(hit)[0]:
                    frac = (self.V_th - v0[p]) / (v1[p] - v0[p])
                    spikes[p][j].append(t + dt * frac)
            if (s + 1) % record_every == 0:
                row = []
                for j, c in enumerate(probe_cv):
                    what = self.probe_what[j] if j < len(self.probe_what) else None
                    pid = self.probe_points[j]
                    if what is None:
                        row.append(self.V[:, c] if c is not None else np.full(self.P, np.nan))
                    elif what[0] == "Ci":
                        row.append(self.Ci[:, pid])
                    elif what[0] in ("cur", "ion"):
                        row.append(self._probe_current(what, pid))
                    else:
                        row.append(self.gates[(what[1], what[2])][:, pid])
                traces.append(np.stack(row, axis=1))
        tr = np.stack(traces, axis=-1) if traces else np.zeros((self.P, len(probe_cv), 0))
        return tr, spikes
