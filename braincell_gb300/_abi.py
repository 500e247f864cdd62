"""ctypes view of the C ABI declared in ``include/braincell_gb300.h``.

The shared library is built in-tree (``braincell_gb300/_native/libbraincell_gb300.so``)
by :func:`braincell_gb300.build.build_native`.  Loading fails loudly when it is
missing: there is no CPU fallback for the solver.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

__all__ = ["lib", "check", "BCError", "BatchSpec", "PlanOptions", "PlanInfo", "LIB_PATH"]

# ---------------------------------------------------------------- constants (mirror the header)
BC_OK = 0
BC_ERR_INVALID = 1
BC_ERR_CUDA = 2
BC_ERR_NONFINITE = 3
BC_ERR_CAPACITY = 4
BC_ERR_TIMEOUT = 5
BC_ERR_UNSUPPORTED = 6

BC_M_IL = 1 << 0
BC_M_KLEAK = 1 << 1
BC_M_NA = 1 << 2
BC_M_KDR = 1 << 3
BC_M_CAL = 1 << 4
BC_M_CAT = 1 << 5
BC_M_HCN = 1 << 6
BC_M_AHP = 1 << 7
BC_M_CADET = 1 << 8
BC_M_NAHH = 1 << 9
BC_M_KHH = 1 << 10
BC_M_KM = 1 << 11
BC_M_KA1 = 1 << 12
BC_M_KA2 = 1 << 13
BC_M_KK2A = 1 << 14
BC_M_KK2B = 1 << 15
BC_M_KNI = 1 << 16
BC_M_NAV16 = 1 << 17
BC_M_KCA22 = 1 << 18
BC_M_KCA11 = 1 << 19
BC_M_KV34 = 1 << 20
BC_M_KV43 = 1 << 21
BC_M_KV11 = 1 << 22
BC_M_KIR23 = 1 << 23
BC_M_HCN1F = 1 << 24
BC_M_HCN1H = 1 << 25
BC_M_CAHVA = 1 << 26
BC_M_CAV23 = 1 << 27
BC_M_CAV32 = 1 << 28
BC_M_EXT = 1 << 29  # extension channels, listed as BC_X_* bits in the record's BC_P_EXT_MASK
BC_M_ALL = 0x3FFFFFFF

BC_X_HCN2 = 1 << 0
BC_X_KV33 = 1 << 1
BC_X_KV22 = 1 << 2
BC_X_KV15 = 1 << 3
BC_X_NAF = 1 << 4
BC_X_NAP = 1 << 5
BC_X_NAIO = 1 << 6
BC_X_FKDR = 1 << 7
BC_X_SKDR = 1 << 8
BC_X_KDRIO = 1 << 9
BC_X_HCNDCN = 1 << 10
BC_X_HCNIO = 1 << 11
BC_X_CATHP = 1 << 12
BC_X_CAHTRE = 1 << 13
BC_X_CALDCN = 1 << 14
BC_X_KCA31 = 1 << 15
BC_X_SKDCN = 1 << 16
BC_X_KKV = 1 << 17
BC_X_CAN = 1 << 18
BC_X_CAIO = 1 << 19
BC_X_NAVGRC = 1 << 20
BC_X_CAV31 = 1 << 21
BC_X_CAV33 = 1 << 22
BC_X_CAV12 = 1 << 23
BC_X_CAV13 = 1 << 24
BC_X_CAV21 = 1 << 25
BC_X_CAHVADCN = 1 << 26
BC_X_CALVADCN = 1 << 27
BC_X_ALL = 0xFFFFFFF

BC_NPARAM = 168
BC_P_INVCM = 0
BC_P_VREST = 1
BC_P_ENA = 2
BC_P_EK = 3
BC_P_ECA = 4
BC_P_IL_G = 5
BC_P_IL_E = 6
BC_P_KLEAK_G = 7
BC_P_NA_G = 8
BC_P_NA_VSH = 9
BC_P_NA_PHI = 10
BC_P_KDR_G = 11
BC_P_KDR_VSH = 12
BC_P_KDR_PHI = 13
BC_P_CAL_G = 14
BC_P_CAL_VSH = 15
BC_P_CAL_PHIP = 16
BC_P_CAL_PHIQ = 17
BC_P_CAT_G = 18
BC_P_CAT_VSH = 19
BC_P_CAT_PHIP = 20
BC_P_CAT_PHIQ = 21
BC_P_HCN_G = 22
BC_P_HCN_E = 23
BC_P_HCN_PHI = 24
BC_P_AHP_G = 25
BC_P_AHP_N = 26
BC_P_AHP_ALPHA = 27
BC_P_AHP_BETA = 28
BC_P_AHP_PHI = 29
BC_P_CA_D = 30
BC_P_CA_TAU = 31
BC_P_CA_CREST = 32
BC_P_CA_CO = 33
BC_P_CA_TEMP = 34
BC_P_CA_CI0 = 35
BC_P_NAHH_G = 36
BC_P_NAHH_VSH = 37
BC_P_NAHH_PHI = 38
BC_P_KHH_G = 39
BC_P_KHH_VSH = 40
BC_P_KHH_PHI = 41
BC_P_KM_G = 42
BC_P_KM_PHI = 43
BC_P_KA1_G = 44
BC_P_KA1_VSH = 45
BC_P_KA1_PHIP = 46
BC_P_KA1_PHIQ = 47
BC_P_KA2_G = 48
BC_P_KA2_VSH = 49
BC_P_KA2_PHIP = 50
BC_P_KA2_PHIQ = 51
BC_P_KK2A_G = 52
BC_P_KK2A_VSH = 53
BC_P_KK2A_PHIP = 54
BC_P_KK2A_PHIQ = 55
BC_P_KK2B_G = 56
BC_P_KK2B_VSH = 57
BC_P_KK2B_PHIP = 58
BC_P_KK2B_PHIQ = 59
BC_P_KNI_G = 60
BC_P_KNI_VSH = 61
BC_P_KNI_PHI = 62
BC_P_KNI_TAUMAX = 63
BC_P_NAV16_G = 64
BC_P_NAV16_PHI = 65
BC_P_KCA22_G = 66
BC_P_KCA22_PHI = 67
BC_P_KCA22_DIFF = 68
BC_P_KCA11_G = 69
BC_P_KCA11_PHI = 70
BC_P_KCA11_QO = 71
BC_P_KCA11_QC = 72
BC_P_NAV16_OON = 73
BC_P_NAV16_ALFAC = 88
BC_P_NAV16_EPS = 89
BC_P_CAHVA_G = 90
BC_P_CAHVA_PHI = 91
BC_P_CAV23_G = 92
BC_P_CAV32_G = 93
BC_P_CAV32_VSH = 94
BC_P_KV34_G = 74
BC_P_KV34_PHI = 75
BC_P_KV43_G = 76
BC_P_KV43_PHI = 77
BC_P_KV11_G = 78
BC_P_KV11_PHI = 79
BC_P_KIR23_G = 80
BC_P_KIR23_PHI = 81
BC_P_HCN1F_G = 82
BC_P_HCN1F_E = 83
BC_P_HCN1F_PHI = 84
BC_P_HCN1H_G = 85
BC_P_HCN1H_E = 86
BC_P_HCN1H_PHI = 87
BC_P_EXT_MASK = 96
BC_P_HCN2_G = 97
BC_P_HCN2_E = 98
BC_P_HCN2_PHI = 99
BC_P_KV33_G = 100
BC_P_KV33_PHI = 101
BC_P_KV22_G = 102
BC_P_KV15_G = 103
BC_P_KV15_Q10 = 104
BC_P_KV15_TACT = 105
BC_P_KV15_TINF = 106
BC_P_KV15_TINS = 107
BC_P_NAF_G = 108
BC_P_NAP_G = 109
BC_P_NAIO_G = 110
BC_P_FKDR_G = 111
BC_P_SKDR_G = 112
BC_P_KDRIO_G = 113
BC_P_HCNDCN_G = 114
BC_P_HCNDCN_E = 115
BC_P_HCNIO_G = 116
BC_P_HCNIO_E = 117
BC_P_CATHP_G = 118
BC_P_CATHP_VSH = 119
BC_P_CATHP_PHIP = 120
BC_P_CATHP_PHIQ = 121
BC_P_CAHTRE_G = 122
BC_P_CAHTRE_VSH = 123
BC_P_CAHTRE_PHIP = 124
BC_P_CAHTRE_PHIQ = 125
BC_P_CALDCN_G = 126
BC_P_CALDCN_E = 127
BC_P_KCA31_G = 128
BC_P_SKDCN_G = 129
BC_P_KKV_G = 130
BC_P_KKV_VSH = 131
BC_P_KKV_RA = 132
BC_P_KKV_RB = 133
BC_P_KKV_Q = 134
BC_P_KKV_V12 = 135
BC_P_CAN_G = 136
BC_P_CAN_E = 137
BC_P_CAN_PHI = 138
BC_P_CAIO_G = 139
BC_P_CAIO_E = 140
BC_P_CAIO_MID = 141
BC_P_CAIO_FREEZE = 142
BC_P_NAVGRC_G = 143
BC_P_NAVGRC_PHI = 144
BC_P_CAV31_G = 145
BC_P_CAV31_QT = 146
BC_P_CAV31_TGHK = 147
BC_P_CAV31_FREEZE = 148
BC_P_CAV33_G = 149
BC_P_CAV33_PHI = 150
BC_P_CAV33_TGHK = 151
BC_P_CAV33_VSH = 152
BC_P_CAV33_FREEZE = 153
BC_P_CAV12_G = 154
BC_P_CAV12_PHI = 155
BC_P_CAV13_G = 156
BC_P_CAV13_PHI = 157
BC_P_CAV21_G = 158
BC_P_CAV21_VSH = 159
BC_P_CAV21_PHI = 160
BC_P_CAV21_TGHK = 161
BC_P_EXT_MASK_HI = 162
BC_P_CAHVADCN_G = 163
BC_P_CAHVADCN_T = 164
BC_P_CALVADCN_G = 165
BC_P_CALVADCN_T = 166
BC_P_CAV21_FROZEN = 167

BC_ABI_VERSION = 500

BC_VARIANT_LEAN = 0
BC_VARIANT_EXTRA = 1
BC_VARIANT_PORTS = 2
BC_VARIANT_PORTS_LEAN = 3

BC_PREC_F32 = 0
BC_PREC_F64 = 1

BC_GRU_HIDDEN = 64
BC_GRU_INPUTS = 4
BC_SURROGATE_NORM = 5

BC_PROBE_CURRENT = 128
BC_CUR_IL = 0
BC_CUR_KLEAK = 1
BC_CUR_NA = 2
BC_CUR_KDR = 3
BC_CUR_CAL = 4
BC_CUR_CAT = 5
BC_CUR_HCN = 6
BC_CUR_AHP = 7
BC_CUR_NAHH = 8
BC_CUR_KHH = 9
BC_CUR_KM = 10
BC_CUR_ION_NA = 11
BC_CUR_ION_K = 12
BC_CUR_ION_CA = 13
BC_CUR_KA1 = 14
BC_CUR_KA2 = 15
BC_CUR_KK2A = 16
BC_CUR_KK2B = 17
BC_CUR_KNI = 18
BC_CUR_NAV16 = 19
BC_CUR_KCA22 = 20
BC_CUR_KCA11 = 21
BC_CUR_KV34 = 22
BC_CUR_KV43 = 23
BC_CUR_KV11 = 24
BC_CUR_KIR23 = 25
BC_CUR_HCN1F = 26
BC_CUR_HCN1H = 27
BC_CUR_CAHVA = 28
BC_CUR_CAV23 = 29
BC_CUR_CAV32 = 30
BC_CUR_HCN2 = 31
BC_CUR_KV33 = 32
BC_CUR_KV22 = 33
BC_CUR_KV15 = 34
BC_CUR_NAF = 35
BC_CUR_NAP = 36
BC_CUR_NAIO = 37
BC_CUR_FKDR = 38
BC_CUR_SKDR = 39
BC_CUR_KDRIO = 40
BC_CUR_HCNDCN = 41
BC_CUR_HCNIO = 42
BC_CUR_CATHP = 43
BC_CUR_CAHTRE = 44
BC_CUR_CALDCN = 45
BC_CUR_KCA31 = 46
BC_CUR_SKDCN = 47
BC_CUR_KKV = 48
BC_CUR_CAN = 49
BC_CUR_CAIO = 50
BC_CUR_NAVGRC = 51
BC_CUR_CAV31 = 52
BC_CUR_CAV33 = 53
BC_CUR_CAV12 = 54
BC_CUR_CAV13 = 55
BC_CUR_CAV21 = 56
BC_CUR_CAHVADCN = 57
BC_CUR_CALVADCN = 58
BC_NCUR = 59

BC_STATE_V = 0
BC_STATE_NA_P = 1
BC_STATE_NA_Q = 2
BC_STATE_KDR_P = 3
BC_STATE_CAL_P = 4
BC_STATE_CAL_Q = 5
BC_STATE_CAT_P = 6
BC_STATE_CAT_Q = 7
BC_STATE_HCN_P = 8
BC_STATE_AHP_P = 9
BC_STATE_CA_CI = 10
BC_STATE_NAHH_P = 11
BC_STATE_NAHH_Q = 12
BC_STATE_KHH_P = 13
BC_STATE_KM_N = 14
BC_STATE_KA1_P = 15
BC_STATE_KA1_Q = 16
BC_STATE_KA2_P = 17
BC_STATE_KA2_Q = 18
BC_STATE_KK2A_P = 19
BC_STATE_KK2A_Q = 20
BC_STATE_KK2B_P = 21
BC_STATE_KK2B_Q = 22
BC_STATE_KNI_P = 23
BC_STATE_V_LAST = 24
BC_STATE_NAV16_C1 = 25
BC_STATE_NAV16_O = 35
BC_STATE_KCA22_C2 = 37
BC_STATE_KCA11_C1 = 42
BC_STATE_KV34_M = 51
BC_STATE_KV34_H = 52
BC_STATE_KV43_A = 53
BC_STATE_KV43_B = 54
BC_STATE_KV11_N = 55
BC_STATE_KIR23_D = 56
BC_STATE_HCN1F_FAST = 57
BC_STATE_HCN1F_SLOW = 58
BC_STATE_HCN1H_H = 59
BC_STATE_CAHVA_S = 60
BC_STATE_CAHVA_U = 61
BC_STATE_CAV23_M = 62
BC_STATE_CAV23_H = 63
BC_STATE_CAV32_M = 64
BC_STATE_CAV32_H = 65
BC_STATE_HCN2_FAST = 66
BC_STATE_HCN2_SLOW = 67
BC_STATE_KV33_N = 68
BC_STATE_KV22_M = 69
BC_STATE_KV22_H = 70
BC_STATE_KV15_M = 71
BC_STATE_KV15_N = 72
BC_STATE_KV15_U = 73
BC_STATE_NAF_M = 74
BC_STATE_NAF_H = 75
BC_STATE_NAP_M = 76
BC_STATE_NAP_H = 77
BC_STATE_NAIO_M = 78
BC_STATE_NAIO_H = 79
BC_STATE_FKDR_M = 80
BC_STATE_SKDR_M = 81
BC_STATE_KDRIO_N = 82
BC_STATE_HCNDCN_M = 83
BC_STATE_HCNIO_Q = 84
BC_STATE_CATHP_P = 85
BC_STATE_CATHP_Q = 86
BC_STATE_CAHTRE_P = 87
BC_STATE_CAHTRE_Q = 88
BC_STATE_CALDCN_M = 89
BC_STATE_CALDCN_H = 90
BC_STATE_KCA31_P = 91
BC_STATE_SKDCN_Z = 92
BC_STATE_KKV_N = 93
BC_STATE_CAN_P = 94
BC_STATE_CAIO_H = 95
BC_STATE_NAVGRC_C1 = 96
BC_STATE_NAVGRC_O = 106
BC_STATE_CAV31_P = 108
BC_STATE_CAV31_Q = 109
BC_STATE_CAV33_N = 110
BC_STATE_CAV33_L = 111
BC_STATE_CAV12_M = 112
BC_STATE_CAV13_M = 115
BC_STATE_CAV21_M = 118
BC_STATE_CAHVADCN_M = 119
BC_STATE_CALVADCN_M = 120
BC_STATE_CALVADCN_H = 121
BC_NSTATE_VIEW = 122
# the independent states of each Markov scheme, in view order (first appearance in
# the scheme's transition list, the dependent state left out)
MARKOV_STATES = {
    "Nav1p6_MA2020_GoC": (BC_STATE_NAV16_C1, ("C1", "C2", "C3", "C4", "C5", "I1", "I2", "I3", "I4", "I5", "O", "B")),
    "Kca2p2_MA2020_GoC": (BC_STATE_KCA22_C2, ("C2", "C3", "C4", "O1", "O2")),
    "Kca1p1_MA2020_GoC": (BC_STATE_KCA11_C1, ("C1", "C2", "C3", "C4", "O0", "O1", "O2", "O3", "O4")),
    "Nav_MA2020_GrC": (BC_STATE_NAVGRC_C1, ("C1", "C2", "C3", "C4", "C5", "I1", "I2", "I3", "I4", "I5", "O", "OB")),
}
BC_NOALLOC_MAX_CV = 262144

STATE_NAMES = {
    "V": BC_STATE_V,
    "Na_p": BC_STATE_NA_P,
    "Na_q": BC_STATE_NA_Q,
    "KDR_p": BC_STATE_KDR_P,
    "CaL_p": BC_STATE_CAL_P,
    "CaL_q": BC_STATE_CAL_Q,
    "CaT_p": BC_STATE_CAT_P,
    "CaT_q": BC_STATE_CAT_Q,
    "HCN_p": BC_STATE_HCN_P,
    "AHP_p": BC_STATE_AHP_P,
    "Ci": BC_STATE_CA_CI,
    "NaHH_p": BC_STATE_NAHH_P,
    "NaHH_q": BC_STATE_NAHH_Q,
    "KHH_p": BC_STATE_KHH_P,
    "KM_n": BC_STATE_KM_N,
    "KA1_p": BC_STATE_KA1_P,
    "KA1_q": BC_STATE_KA1_Q,
    "KA2_p": BC_STATE_KA2_P,
    "KA2_q": BC_STATE_KA2_Q,
    "KK2A_p": BC_STATE_KK2A_P,
    "KK2A_q": BC_STATE_KK2A_Q,
    "KK2B_p": BC_STATE_KK2B_P,
    "KK2B_q": BC_STATE_KK2B_Q,
    "KNI_p": BC_STATE_KNI_P,
    "V_last": BC_STATE_V_LAST,
    "Kv3p4_m": BC_STATE_KV34_M,
    "Kv3p4_h": BC_STATE_KV34_H,
    "Kv4p3_a": BC_STATE_KV43_A,
    "Kv4p3_b": BC_STATE_KV43_B,
    "Kv1p1_n": BC_STATE_KV11_N,
    "Kir2p3_d": BC_STATE_KIR23_D,
    "HCN1_o_fast": BC_STATE_HCN1F_FAST,
    "HCN1_o_slow": BC_STATE_HCN1F_SLOW,
    "HCN1_h": BC_STATE_HCN1H_H,
    "CaHVA_s": BC_STATE_CAHVA_S,
    "CaHVA_u": BC_STATE_CAHVA_U,
    "Cav2p3_m": BC_STATE_CAV23_M,
    "Cav2p3_h": BC_STATE_CAV23_H,
    "Cav3p2_m": BC_STATE_CAV32_M,
    "Cav3p2_h": BC_STATE_CAV32_H,
    "HCN2_o_fast": BC_STATE_HCN2_FAST,
    "HCN2_o_slow": BC_STATE_HCN2_SLOW,
    "Kv3p3_n": BC_STATE_KV33_N,
    "Kv2p2_m": BC_STATE_KV22_M,
    "Kv2p2_h": BC_STATE_KV22_H,
    "Kv1p5_m": BC_STATE_KV15_M,
    "Kv1p5_n": BC_STATE_KV15_N,
    "Kv1p5_u": BC_STATE_KV15_U,
    "NaF_m": BC_STATE_NAF_M,
    "NaF_h": BC_STATE_NAF_H,
    "NaP_m": BC_STATE_NAP_M,
    "NaP_h": BC_STATE_NAP_H,
    "NaIO_m": BC_STATE_NAIO_M,
    "NaIO_h": BC_STATE_NAIO_H,
    "fKdr_m": BC_STATE_FKDR_M,
    "sKdr_m": BC_STATE_SKDR_M,
    "KdrIO_n": BC_STATE_KDRIO_N,
    "HCNDCN_m": BC_STATE_HCNDCN_M,
    "HCNIO_q": BC_STATE_HCNIO_Q,
    "CaTHP_p": BC_STATE_CATHP_P,
    "CaTHP_q": BC_STATE_CATHP_Q,
    "CaHTRe_p": BC_STATE_CAHTRE_P,
    "CaHTRe_q": BC_STATE_CAHTRE_Q,
    "CaLDCN_m": BC_STATE_CALDCN_M,
    "CaLDCN_h": BC_STATE_CALDCN_H,
    "Kca3p1_p": BC_STATE_KCA31_P,
    "SKDCN_z": BC_STATE_SKDCN_Z,
    "KKv_n": BC_STATE_KKV_N,
    "CaN_p": BC_STATE_CAN_P,
    "CaIO_h": BC_STATE_CAIO_H,
    "Cav3p1_p": BC_STATE_CAV31_P,
    "Cav3p1_q": BC_STATE_CAV31_Q,
    "Cav3p3_n": BC_STATE_CAV33_N,
    "Cav3p3_l": BC_STATE_CAV33_L,
    "Cav1p2_m": BC_STATE_CAV12_M,
    "Cav1p2_h": BC_STATE_CAV12_M + 1,
    "Cav1p2_n": BC_STATE_CAV12_M + 2,
    "Cav1p3_m": BC_STATE_CAV13_M,
    "Cav1p3_h": BC_STATE_CAV13_M + 1,
    "Cav1p3_n": BC_STATE_CAV13_M + 2,
    "Cav2p1_m": BC_STATE_CAV21_M,
    "CaHVADCN_m": BC_STATE_CAHVADCN_M,
    "CaLVADCN_m": BC_STATE_CALVADCN_M,
    "CaLVADCN_h": BC_STATE_CALVADCN_H,
}
for _cls, (_base, _names) in MARKOV_STATES.items():
    for _k, _n in enumerate(_names):
        STATE_NAMES[f"{_cls.split('_')[0]}_{_n}"] = _base + _k

_p = C.POINTER


class BatchSpec(C.Structure):
    _fields_ = [
        ("n_cells", C.c_int64),
        ("n_branches", C.c_int64),
        ("n_segments", C.c_int64),
        ("n_regions", C.c_int32),
        ("cell_branch_offsets", _p(C.c_int64)),
        ("branch_parent", _p(C.c_int32)),
        ("branch_parent_x", _p(C.c_double)),
        ("branch_child_x", _p(C.c_double)),
        ("branch_ncv", _p(C.c_int32)),
        ("branch_region", _p(C.c_int32)),
        ("branch_seg_offsets", _p(C.c_int64)),
        ("seg_length", _p(C.c_double)),
        ("seg_r_prox", _p(C.c_double)),
        ("seg_r_dist", _p(C.c_double)),
        ("region_cm", _p(C.c_double)),
        ("region_ra", _p(C.c_double)),
        ("region_mech", _p(C.c_uint32)),
        ("region_params", _p(C.c_double)),
        ("n_pulses", C.c_int64),
        ("pulse_cell", _p(C.c_int32)),
        ("pulse_branch", _p(C.c_int32)),
        ("pulse_x", _p(C.c_double)),
        ("pulse_t_on", _p(C.c_double)),
        ("pulse_t_off", _p(C.c_double)),
        ("pulse_amp", _p(C.c_double)),
        ("n_probes", C.c_int64),
        ("probe_cell", _p(C.c_int32)),
        ("probe_branch", _p(C.c_int32)),
        ("probe_x", _p(C.c_double)),
        ("n_synapses", C.c_int64),
        ("syn_cell", _p(C.c_int32)),
        ("syn_branch", _p(C.c_int32)),
        ("syn_x", _p(C.c_double)),
        ("syn_tau", _p(C.c_double)),
        ("syn_e", _p(C.c_double)),
        ("n_connections", C.c_int64),
        ("conn_pre", _p(C.c_int32)),
        ("conn_post", _p(C.c_int64)),
        ("conn_weight", _p(C.c_double)),
        ("conn_delay", _p(C.c_double)),
        ("n_ports", C.c_int64),
        ("port_cell", _p(C.c_int32)),
        ("port_branch", _p(C.c_int32)),
        ("port_g", _p(C.c_double)),
        ("port_e", _p(C.c_double)),
        ("port_feat", _p(C.c_double)),
        ("n_port_pulses", C.c_int64),
        ("port_pulse_port", _p(C.c_int32)),
        ("port_pulse_t_on", _p(C.c_double)),
        ("port_pulse_t_off", _p(C.c_double)),
        ("port_pulse_amp", _p(C.c_double)),
        ("probe_field", _p(C.c_int32)),
    ]


class PlanOptions(C.Structure):
    _fields_ = [
        ("precision", C.c_int32),
        ("threads_per_tile", C.c_int32),
        ("tile_nodes", C.c_int32),
        ("lane_nodes", C.c_int32),
        ("steps_per_launch", C.c_int32),
        ("record_every", C.c_int32),
        ("max_spikes", C.c_int32),
        ("use_graph", C.c_int32),
        ("device", C.c_int32),
        ("threads_big", C.c_int32),
        ("threads_global", C.c_int32),
        ("narrow_lane_nodes", C.c_int32),
        ("reserved_b", C.c_float),
        ("dry_run", C.c_int32),
        ("lane_cell_nodes", C.c_int32),
        ("tile_order", C.c_int32),
    ]


class PlanInfo(C.Structure):
    _fields_ = [
        ("n_cells", C.c_int64),
        ("n_cv", C.c_int64),
        ("n_nodes", C.c_int64),
        ("n_tiles", C.c_int64),
        ("n_probes", C.c_int64),
        ("n_pulses", C.c_int64),
        ("threads_per_tile", C.c_int32),
        ("tile_nodes", C.c_int32),
        ("steps_per_launch", C.c_int32),
        ("precision", C.c_int32),
        ("smem_bytes_per_tile", C.c_int64),
        ("device_bytes", C.c_int64),
        ("max_phases", C.c_int64),
        ("max_chain_nodes", C.c_int64),
        ("state_slots", C.c_int32),
        ("n_smem_tiles", C.c_int32),
        ("n_launch_classes", C.c_int32),
        ("kernel_variant", C.c_int32),
        ("reserved", C.c_int32 * 4),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


# Exported symbols and their ctypes signatures (kept in step with the header).
SIGNATURES = {
    "bc_last_error": (C.c_char_p, []),
    "bc_version": (C.c_int32, []),
    "bc_default_options": (None, [_p(PlanOptions)]),
    "bc_plan_create": (C.c_int32, [_p(BatchSpec), _p(PlanOptions), _p(C.c_void_p)]),
    "bc_plan_destroy": (C.c_int32, [C.c_void_p]),
    "bc_plan_info": (C.c_int32, [C.c_void_p, _p(PlanInfo)]),
    "bc_plan_cell_ncv": (C.c_int32, [C.c_void_p, _p(C.c_int64)]),
    "bc_plan_tile_stats": (C.c_int32, [C.c_void_p, _p(C.c_int64)]),
    "bc_lower_cell": (
        C.c_int32,
        [_p(BatchSpec), C.c_int64, _p(C.c_int32), _p(C.c_int32), _p(C.c_double), _p(C.c_int32), _p(C.c_int32),
         _p(C.c_double), _p(C.c_double), _p(C.c_double), _p(C.c_int32)],
    ),
    "bc_reset": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "bc_run": (C.c_int32, [C.c_void_p, C.c_int64, C.c_double, C.c_void_p]),
    "bc_run_async": (C.c_int32, [C.c_void_p, C.c_int64, C.c_double, C.c_void_p]),
    "bc_check": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "bc_state_download": (C.c_int32, [C.c_void_p, C.c_int32, _p(C.c_double), C.c_void_p]),
    "bc_state_upload": (C.c_int32, [C.c_void_p, C.c_int32, _p(C.c_double), C.c_void_p]),
    "bc_state_download_noalloc": (C.c_int32, [C.c_void_p, C.c_int32, _p(C.c_double), C.c_void_p]),
    "bc_spike_state_download": (C.c_int32, [C.c_void_p, C.c_double, _p(C.c_double), C.c_void_p]),
    "bc_pulse_set_amp": (C.c_int32, [C.c_void_p, _p(C.c_double), C.c_void_p]),
    "bc_network_spikes": (C.c_int32, [C.c_void_p, _p(C.c_int32), _p(C.c_int64), C.c_int64, _p(C.c_int64), C.c_void_p]),
    "bc_synapse_download": (C.c_int32, [C.c_void_p, _p(C.c_double), C.c_void_p]),
    "bc_probe_count": (C.c_int32, [C.c_void_p, _p(C.c_int64)]),
    "bc_probe_download": (C.c_int32, [C.c_void_p, _p(C.c_double), C.c_int64, C.c_void_p]),
    "bc_spike_download": (C.c_int32, [C.c_void_p, _p(C.c_int32), _p(C.c_double), C.c_void_p]),
    "bc_probe_clear": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "bc_step_count": (C.c_int32, [C.c_void_p, _p(C.c_int64)]),
    "bc_debug_phase_cycles": (C.c_int32, [C.c_void_p, _p(C.c_uint64), C.c_int32]),
    "bc_run_timed": (C.c_int32, [C.c_void_p, C.c_int64, C.c_double, C.c_void_p, _p(C.c_double)]),
    "bc_gru_nparam": (C.c_int32, []),
    "bc_surrogate_set": (C.c_int32, [C.c_void_p, _p(C.c_float), _p(C.c_float), C.c_void_p]),
    "bc_surrogate_flags": (C.c_int32, [C.c_void_p, _p(C.c_int32), C.c_void_p]),
    "bc_gru_pack": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "bc_gru_forward": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int32,
                                   C.c_int64, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p]),
    "bc_gru_backward_workspace": (C.c_int64, [C.c_int32]),
    "bc_gru_backward": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int32,
                                    C.c_int64, C.c_int32, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p,
                                    C.c_void_p, C.c_void_p]),
    "bc_gru_grad_sqnorm": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "bc_gru_adam": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_float, C.c_float,
                                C.c_float, C.c_float, C.c_float, C.c_void_p]),
}

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_native", "libbraincell_gb300.so")

_lock = threading.Lock()
_lib = None


class BCError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[bc status {status}] {message}")
        self.status = status


def lib():
    """Load (once) and return the native library; raise if it was not built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"braincell_gb300 native library not found at {LIB_PATH}; build it with "
                "`python -c 'import braincell_gb300.build as b; b.build_native()'`. "
                "There is no CPU fallback for the GB300 solver."
            )
        handle = C.CDLL(LIB_PATH)
        for name, (restype, argtypes) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = restype
            fn.argtypes = argtypes
        # a library of another ABI version lays out its records differently
        # (parameter record size, state views): refuse it rather than misread it
        version = int(handle.bc_version())
        if version != BC_ABI_VERSION:
            raise ImportError(f"braincell_gb300 native library at {LIB_PATH} has ABI version {version}, this package "
                              f"expects {BC_ABI_VERSION}; rebuild it with "
                              "`python -c 'import braincell_gb300.build as b; b.build_native(force=True)'`.")
        _lib = handle
        return _lib


def check(status: int) -> None:
    if status != BC_OK:
        msg = lib().bc_last_error()
        raise BCError(int(status), msg.decode() if msg else "unknown error")
