"""The step kernel's FP64 rate structures (``bc_mech.cuh``), compiled for the host,
against the oracle's rate functions over a voltage grid: a CPU check of the device
rate arithmetic for every kernel channel, including the classes that only the GPU
parity tests exercise in a full simulation.  Needs nvcc (no GPU)."""

from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import staggered as O

HERE = os.path.dirname(os.path.abspath(__file__))

# harness index -> (oracle class, kernel parameters from the class defaults)
CASES = {
    0: ("Na_Ba2002", ("V_sh",)), 1: ("KDR_Ba2002", ("V_sh",)), 2: ("CaL_IS2008", ("V_sh",)),
    3: ("CaT_HM1992", ("V_sh",)), 4: ("HCN_HM1992", ()), 5: ("Na_HH1952", ("V_sh",)), 6: ("K_HH1952", ("V_sh",)),
    7: ("KM_RI2021_SC", ()), 8: ("KA1_HM1992", ("V_sh",)), 9: ("KA2_HM1992", ("V_sh",)),
    10: ("KK2A_HM1992", ("V_sh",)), 11: ("KK2B_HM1992", ("V_sh",)), 12: ("KNI_Ya1989", ("V_sh", "tau_max")),
    13: ("Kv3p4_MA2020_GoC", ()), 14: ("Kv4p3_MA2020_GoC", ()), 15: ("Kv1p1_MA2020_GoC", ()),
    16: ("Kir2p3_MA2020_GrC", ()), 17: ("HCN1_MA2020_GoC", ()), 18: ("HCN1_MA2024_PC", ()),
    19: ("CaHVA_MA2020_GoC", ()), 20: ("Cav2p3_MA2020_GoC", ()), 21: ("Cav3p2_RI2021_SC", ("V_sh",)),
    # extension channels
    22: ("HCN2_MA2020_GoC", ()), 23: ("Kv3p3_MA2024_PC", ()), 24: ("Kv2p2_0010_MA2020_GrC", ()),
    25: ("Kv1p5_MA2024_PC", ("q10f", "Tauact", "Tauinactf", "Tauinacts")), 26: ("NaF_SU2015_DCN", ()),
    27: ("NaP_SU2015_DCN", ()), 28: ("Na_ZH2019_IO", ()), 29: ("fKdr_SU2015_DCN", ()), 30: ("sKdr_SU2015_DCN", ()),
    31: ("Kdr_ZH2019_IO", ()), 32: ("HCN_SU2015_DCN", ()), 33: ("HCN_ZH2019_IO", ()),
    34: ("CaT_HP1992", ("V_sh",)), 35: ("CaHT_Re1993", ("V_sh",)), 36: ("CaL_SU2015_DCN", ()),
    37: ("Kca3p1_MA2020_GoC", ("Ci",)), 38: ("SK_SU2015_DCN", ("Ci",)),
    39: ("K_Kv_test", ("V_sh", "Ra", "Rb", "q", "v12")), 40: ("CaN_IS2008", ()), 41: ("Ca_ZH2019_IO", ()),
    42: ("Cav3p1_MA2020_GoC", ("qt",)), 44: ("Cav3p3_RI2021_SC", ("V_sh",)),
    46: ("Cav1p2_MA2020_GoC", ("Ci",)), 47: ("Cav1p3_MA2020_GoC", ("Ci",)), 48: ("Cav2p1_RI2021_SC", ("V_sh",)),
    50: ("CaHVA_SU2015_DCN", ()),
}


@pytest.fixture(scope="module")
def rates_lib(tmp_path_factory):
    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc is not available")
    out = str(tmp_path_factory.mktemp("rates") / "librates_host.so")
    cmd = [nvcc, "-x", "cu", "-shared", "-Xcompiler", "-fPIC", "-std=c++17", "-O2",
           "-gencode=arch=compute_103a,code=sm_103a", os.path.join(HERE, "rates_host.cu"), "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    lib = C.CDLL(out)
    lib.bc_test_rates.argtypes = [C.c_int, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double),
                                  C.POINTER(C.c_double)]
    lib.bc_test_rates.restype = C.c_int
    return lib


def _kernel(lib, which, V, prm):
    V = np.ascontiguousarray(V, np.float64)
    prm = np.ascontiguousarray(prm, np.float64)
    out = np.zeros((V.size, 6))
    dp = C.POINTER(C.c_double)
    assert lib.bc_test_rates(which, V.ctypes.data_as(dp), V.size, prm.ctypes.data_as(dp), out.ctypes.data_as(dp)) == 0
    return out


@pytest.mark.parametrize("which", sorted(CASES))
@pytest.mark.parametrize("shift", [0.0, 7.5])
def test_kernel_rates_match_oracle(rates_lib, which, shift):
    name, keys = CASES[which]
    p = dict(O.CHANNEL_DEFAULTS[name])
    if "V_sh" in keys:
        p["V_sh"] = p["V_sh"] + shift
    if name == "Kv1p5_MA2024_PC":  # a temperature off 37 degC and non-unit time-constant scales when shifted
        p["temp"] += shift
        p["Tauact"], p["Tauinacts"] = 1.0 + shift / 10.0, 1.0 + shift / 5.0
        p["q10f"] = 2.2 ** ((p["temp"] - O._c2k(37.0)) / 10.0)
    # a grid with the removable singularities of exprel and the branch points of the
    # piecewise time constants (KA -63, KK2B -70, CaT -80 relative to V_sh)
    V = np.linspace(-130.0, 60.0, 1901)
    if name == "Kv3p4_MA2020_GoC":  # the branch points of its time constants (V + 11 = -35 and 0)
        V = np.concatenate([V, [-46.0, -11.0]])
    if name == "HCN2_MA2020_GoC":  # the ends of r(V)'s linear piece
        V = np.concatenate([V, [-64.70, -108.70]])
    if name in ("Na_ZH2019_IO", "Kdr_ZH2019_IO"):  # the removable singularities of x / (1 - e^-x)
        V = np.concatenate([V, [-41.0, -50.0, -41.0 + 1e-7, -50.0 - 1e-7]])
    if name == "CaHT_Re1993":  # alpha_p's removable singularity at V = V_sh - 27 mV
        V = np.concatenate([V, p["V_sh"] - 27.0 + np.array([0.0, 1e-7, -1e-7])])
    if name == "CaL_SU2015_DCN":  # the branch point of h's time constant
        V = np.concatenate([V, [-81.0, -81.0 + 1e-9]])
    if "V_sh" in keys:
        V = np.concatenate([V, p["V_sh"] + np.array([13.0, 15.0, 40.0, -5.0, -63.0, -70.0, -80.0, -10.0])])
    # the calcium-gated classes at a Ci on each side of their branch points (0.005, 0.01 mM)
    p["Ci"] = {0.0: 2e-3, 7.5: 0.012}[shift] if name == "Kca3p1_MA2020_GoC" else \
        ({0.0: 1e-4, 7.5: 0.007}[shift] if name in ("SK_SU2015_DCN", "Cav1p2_MA2020_GoC", "Cav1p3_MA2020_GoC")
         else None)
    if name in ("Cav1p2_MA2020_GoC", "Cav1p3_MA2020_GoC"):  # m_alpha's removable singularity at V = -c
        V = np.concatenate([V, [-8.124, -67.24, -8.124 + 1e-7]])
    if name == "K_Kv_test":  # its removable singularity at V = V_sh + v12
        V = np.concatenate([V, p["V_sh"] + p["v12"] + np.array([0.0, 1e-7, -1e-7])])
    if name == "Cav3p3_RI2021_SC":  # the -60 mV branch point of its time constants
        V = np.concatenate([V, p["V_sh"] - 60.0 + np.array([0.0, 1e-9])])
    if name == "Cav3p1_MA2020_GoC":  # at a temperature off its reference, where qt != 1; the -90 mV branch point
        p["temp"] += shift
        p["qt"] = p["q10"] ** ((p["temp"] - p["temp_ref"]) / 10.0)
        V = np.concatenate([V, [-90.0, -90.0 + 1e-9]])
    got = _kernel(rates_lib, which, V, [p[k] for k in keys])
    ref = O.rates(name, V, p, Ci=p["Ci"])
    cols = [c for g in ref for c in (ref[g][1], ref[g][2])]
    for k, col in enumerate(cols):
        np.testing.assert_allclose(got[:, k], np.broadcast_to(col, V.shape), rtol=1e-12, atol=1e-300,
                                   err_msg=f"{name} rate column {k}")


@pytest.mark.parametrize("which", [43, 45, 49, 51], ids=["cav3p1", "cav3p3", "shared", "su2015"])
@pytest.mark.parametrize("ci,co,temp", [(5e-5, 2.0, 295.15), (1e-3, 2.0, 310.15), (2.0, 2.0, 300.0)])
def test_ghk_drive_matches_oracle(rates_lib, which, ci, co, temp):
    # the Cav3.1 / Cav3.3 GHK drives and their V-derivatives, across 0 mV (the small branch)
    fn, off = {43: (O.cav31_drive, 0.04), 45: (O.cav33_drive, -0.01), 49: (O.ghk_codata_drive, 0.0),
               51: (O.su2015_drive, 0.0)}[which]
    V = np.concatenate([np.linspace(-100.0, 60.0, 1601), [0.0, 1e-7, -1e-7, 1e-4]])
    got = _kernel(rates_lib, which, V, [ci, co, temp + off])  # the kernel takes the GHK temperature itself
    drive, dd = fn(V, ci, co, temp)
    # 1e-10: near 0 mV the regular branch divides by 1 - e^-zeta ~ 1e-5, so an ulp of exp
    # (the host's against numpy's) is amplified to ~1e-11 relative
    np.testing.assert_allclose(got[:, 0], drive, rtol=1e-10, atol=1e-9)
    # the derivative's two terms cancel as 1/(1 - e^-zeta)^2 near 0 mV: ~1e-6 relative there
    far = np.abs(V) > 1e-2
    np.testing.assert_allclose(got[far, 1], dd[far], rtol=1e-10, atol=1e-9)
    np.testing.assert_allclose(got[~far, 1], dd[~far], rtol=1e-4)
    # the derivative against a central difference away from the branch switch
    h = 1e-4
    Vs = np.linspace(-90.0, 50.0, 141) + 0.37
    fd = (fn(Vs + h, ci, co, temp)[0] - fn(Vs - h, ci, co, temp)[0]) / (2 * h)
    np.testing.assert_allclose(fn(Vs, ci, co, temp)[1], fd, rtol=1e-6, atol=1e-6)


def test_unknown_structure_is_rejected(rates_lib):
    assert rates_lib.bc_test_rates(99, None, 0, None, None) == 0  # no voltages: nothing to evaluate
    v = np.zeros(1)
    out = np.zeros(6)  # six rate entries per voltage
    dp = C.POINTER(C.c_double)
    assert rates_lib.bc_test_rates(99, v.ctypes.data_as(dp), 1, v.ctypes.data_as(dp), out.ctypes.data_as(dp)) == -1
