/*
 * braincell_gb300 -- C ABI of the GB300 (sm_103a) multi-compartment Cell time step.
 *
 * This library replaces, for a batch of cells, the reference's staggered solver
 * path: `staggered_step` (braincell/quad/_staggered.py:54-154), i.e. the step-start
 * ion-current cache (cell.py:2261-2280), the DHS implicit-Euler voltage step
 * (_staggered.py:193-320: linearisation :763-795, numeric state :449-513, forward
 * elimination `comp_triang_raw` :641-657, back-substitution `comp_backsub_raw`
 * :742-760), and the family-ordered exponential-Euler update of ions and channels
 * (cell.py:2157-2217 -> quad/_exp_euler.py:330-478).  The one-time lowering it also
 * replaces is the geometry / node-tree / axial-matrix assembly:
 * _discretization/geometry.py:214-434,614-736, _discretization/base.py:530-559,
 * _discretization/node_build.py:58-285, quad/_staggered.py:323-390,546-593.
 *
 * Conventions: plain pointers and sizes, host memory unless stated, no torch types.
 * Every entry point returns a bc_status (0 = OK); bc_last_error() gives the text of
 * the most recent failure on the calling thread.  A plan is used from one host
 * thread at a time; device work is ordered on the CUDA stream passed in.
 *
 * Units: um, mV, ms, nA, mS/cm^2 (conductance density), uF/cm^2, ohm*cm, kelvin, mM.
 */
#ifndef BRAINCELL_GB300_H
#define BRAINCELL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status codes */
typedef int32_t bc_status;
#define BC_OK 0
#define BC_ERR_INVALID 1        /* bad argument / malformed spec (host-side check)      */
#define BC_ERR_CUDA 2           /* a CUDA runtime call failed                           */
#define BC_ERR_NONFINITE 3      /* a NaN/Inf voltage was detected by the kernel          */
#define BC_ERR_CAPACITY 4       /* a cell does not fit any supported tile                */
#define BC_ERR_TIMEOUT 5        /* a bounded device wait gave up                         */
#define BC_ERR_UNSUPPORTED 6    /* feature not available in this build / precision       */

/* ------------------------------------------------------------------ mechanisms */
/* Bit per mechanism present in a region (painted density mechanisms). */
#define BC_M_IL (1u << 0)        /* channel/leaky.py:144      g (E - V)                       */
#define BC_M_KLEAK (1u << 1)     /* channel/potassium.py:1167 g (E_K - V)                     */
#define BC_M_NA (1u << 2)        /* channel/sodium.py:59      Na_Ba2002   p^3 q, E_Na          */
#define BC_M_KDR (1u << 3)       /* channel/potassium.py:95   KDR_Ba2002  p^4, E_K             */
#define BC_M_CAL (1u << 4)       /* channel/calcium.py:790    CaL_IS2008  p^2 q, E_Ca          */
#define BC_M_CAT (1u << 5)       /* channel/calcium.py:222    CaT_HM1992  p^2 q, E_Ca          */
#define BC_M_HCN (1u << 6)       /* channel/hyperpolarization_activated.py:45 HCN_HM1992 p, E  */
#define BC_M_AHP (1u << 7)       /* channel/potassium_calcium.py:78 AHP_De1994 p^2, E_K, Ci   */
#define BC_M_CADET (1u << 8)     /* ion/calcium.py:286        CalciumDetailed (dynamic Ci)     */
#define BC_M_NAHH (1u << 9)      /* channel/sodium.py:293     Na_HH1952   p^3 q, E_Na          */
#define BC_M_KHH (1u << 10)      /* channel/potassium.py:341  K_HH1952    p^4, E_K             */
#define BC_M_KM (1u << 11)       /* channel/potassium.py:1597 KM_RI2021_SC n, E_K              */
#define BC_M_KA1 (1u << 12)      /* channel/potassium.py:460  KA1_HM1992  p^4 q, E_K           */
#define BC_M_KA2 (1u << 13)      /* channel/potassium.py:614  KA2_HM1992  p^4 q, E_K           */
#define BC_M_KK2A (1u << 14)     /* channel/potassium.py:765  KK2A_HM1992 p q, E_K             */
#define BC_M_KK2B (1u << 15)     /* channel/potassium.py:899  KK2B_HM1992 p q, E_K             */
#define BC_M_KNI (1u << 16)      /* channel/potassium.py:1045 KNI_Ya1989  p, E_K               */
/* Markov channels (channel/_base.py:677-1125), each advanced by one linearised
 * backward-Euler step (quad/_backward_euler.py:31-64) at the new V and Ci, after
 * the gates, as the reference's independent-integration family is. */
#define BC_M_NAV16 (1u << 17)    /* channel/sodium.py:727     Nav1p6_MA2020_GoC 13 states, g O, E_Na    */
#define BC_M_KCA22 (1u << 18)    /* channel/potassium_calcium.py:613 Kca2p2_MA2020_GoC 6 states, E_K */
#define BC_M_KCA11 (1u << 19)    /* channel/potassium_calcium.py:1107 Kca1p1_MA2020_GoC 10 states, E_K */
/* Cerebellar HH channels of the MA2020 / MA2024 / MA2025 / RI2021 models (each kernel
 * also serves the cell-type variants that share its kinetics). */
#define BC_M_KV34 (1u << 20)     /* channel/potassium.py:4750 Kv3p4_MA2020_GoC  m^3 h, E_K (V + 11 mV) */
#define BC_M_KV43 (1u << 21)     /* channel/potassium.py:4964 Kv4p3_MA2020_GoC  a^3 b, E_K          */
#define BC_M_KV11 (1u << 22)     /* channel/potassium.py:4570 Kv1p1_MA2020_GoC  n^4, E_K            */
#define BC_M_KIR23 (1u << 23)    /* channel/potassium.py:5334 Kir2p3_MA2020_GrC d, E_K              */
#define BC_M_HCN1F (1u << 24)    /* channel/hyperpolarization_activated.py:675 HCN1_MA2020_GoC
                                    o_fast + o_slow, own E, Q10 1.5 on g                             */
#define BC_M_HCN1H (1u << 25)    /* channel/hyperpolarization_activated.py:411 HCN1_MA2024_PC h, own E */
/* Cerebellar calcium channels: ohmic in E_Ca, their step-start current feeding a
 * CalciumDetailed shell like CaL and CaT. */
#define BC_M_CAHVA (1u << 26)    /* channel/calcium.py:4333 CaHVA_MA2020_GoC s^2 u, E_Ca              */
#define BC_M_CAV23 (1u << 27)    /* channel/calcium.py:4672 Cav2p3_MA2020_GoC m^3 h, E_Ca             */
#define BC_M_CAV32 (1u << 28)    /* channel/calcium.py:3636 Cav3p2_RI2021_SC m^2 h, E_Ca              */
/* Extension channels (extra kernel variant): a region that carries any sets
 * BC_M_EXT and lists them as BC_X_* bits in its record: bits 0-23 in BC_P_EXT_MASK,
 * bits 24 and up in BC_P_EXT_MASK_HI (each an integer below 2^24, exact in FP32);
 * their parameters follow BC_P_EXT_MASK. */
#define BC_M_EXT (1u << 29)
#define BC_M_ALL 0x3FFFFFFFu

#define BC_X_HCN2 (1u << 0)    /* channel/hyperpolarization_activated.py:838 HCN2_MA2020_GoC
                                  o_fast + o_slow, own E, Q10 1.5 on g                        */
#define BC_X_KV33 (1u << 1)    /* channel/potassium.py:2937 Kv3p3_MA2024_PC n^4, E_K          */
#define BC_X_KV22 (1u << 2)    /* channel/potassium.py:5664 Kv2p2_0010_MA2020_GrC m h, E_K    */
#define BC_X_KV15 (1u << 3)    /* channel/potassium.py:2735 Kv1p5_MA2024_PC m^3 n u f(V), E_K */
#define BC_X_NAF (1u << 4)     /* channel/sodium.py:402 NaF_SU2015_DCN m^3 h, E_Na            */
#define BC_X_NAP (1u << 5)     /* channel/sodium.py:500 NaP_SU2015_DCN m^3 h, E_Na            */
#define BC_X_NAIO (1u << 6)    /* channel/sodium.py:598 Na_ZH2019_IO m^3 h, E_Na              */
#define BC_X_FKDR (1u << 7)    /* channel/potassium.py:1374 fKdr_SU2015_DCN m^4, E_K          */
#define BC_X_SKDR (1u << 8)    /* channel/potassium.py:1485 sKdr_SU2015_DCN m^4, E_K          */
#define BC_X_KDRIO (1u << 9)   /* channel/potassium.py:6238 Kdr_ZH2019_IO n^4, E_K            */
#define BC_X_HCNDCN (1u << 10) /* channel/hyperpolarization_activated.py:1010 HCN_SU2015_DCN
                                  m^2, own E                                                  */
#define BC_X_HCNIO (1u << 11)  /* channel/hyperpolarization_activated.py:1109 HCN_ZH2019_IO
                                  q, own E                                                    */
#define BC_X_CATHP (1u << 12)  /* channel/calcium.py:377 CaT_HP1992 p^2 q, E_Ca (Ci drive)   */
#define BC_X_CAHTRE (1u << 13) /* channel/calcium.py:667 CaHT_Re1993 p^2 q, E_Ca (Ci drive)  */
#define BC_X_CALDCN (1u << 14) /* channel/calcium.py:1066 CaL_SU2015_DCN m^2 h, own E        */
#define BC_X_KCA31 (1u << 15)  /* channel/potassium_calcium.py:299 Kca3p1_MA2020_GoC p(V, Ci), E_K */
#define BC_X_SKDCN (1u << 16)  /* channel/potassium_calcium.py:189 SK_SU2015_DCN z(Ci), E_K  */
#define BC_X_KKV (1u << 17)    /* channel/potassium.py:1239 K_Kv_test n, E_K                 */
#define BC_X_CAN (1u << 18)    /* channel/calcium.py:108 CaN_IS2008 p Ci/(Ci + 0.2), own E
                                  (a calcium-ion current: joins the Ci drive)                 */
#define BC_X_CAIO (1u << 19)   /* channel/calcium.py:4837 Ca_ZH2019_IO m_inf(V)^1 h, own E   */
#define BC_X_NAVGRC (1u << 20) /* channel/sodium.py:1427 Nav_MA2020_GrC 13-state Markov scheme
                                  (the Nav1.6 graph), g O, E_Na                               */
#define BC_X_CAV31 (1u << 21)  /* channel/calcium.py:1972 Cav3p1_MA2020_GoC p^2 q, GHK drive
                                  (permeability g in cm/s; a calcium-ion current)            */
#define BC_X_CAV33 (1u << 22)  /* channel/calcium.py:4033 Cav3p3_RI2021_SC n^2 l, GHK drive
                                  (g_scale x perm in cm/s; a calcium-ion current)            */
#define BC_X_CAV12 (1u << 23)  /* channel/calcium.py:1408 Cav1p2_MA2020_GoC m h n(Ci), E_Ca    */
#define BC_X_CAV13 (1u << 24)  /* channel/calcium.py:1683 Cav1p3_MA2020_GoC m h n(Ci), E_Ca    */
#define BC_X_CAV21 (1u << 25)  /* channel/calcium.py:2767 Cav2p1_RI2021_SC m^3, GHK drive (the
                                  shared ghk_flux, channel/_base.py:47; g in cm/s)           */
#define BC_X_CAHVADCN (1u << 26) /* channel/calcium.py:924 CaHVA_SU2015_DCN m^3, SU2015 GHK drive */
#define BC_X_CALVADCN (1u << 27) /* channel/calcium.py:1221 CaLVA_SU2015_DCN m^2 h, same drive   */
#define BC_X_ALL 0xFFFFFFFu

/* Per-region parameter record (double[BC_NPARAM]); index names below. */
#define BC_NPARAM 168
#define BC_P_INVCM 0      /* 1 / membrane capacitance, cm^2/uF                 */
#define BC_P_VREST 1      /* voltage used by reset (mV)                        */
#define BC_P_ENA 2        /* fixed reversal potentials (mV)                    */
#define BC_P_EK 3
#define BC_P_ECA 4        /* used only when BC_M_CADET is absent               */
#define BC_P_IL_G 5
#define BC_P_IL_E 6
#define BC_P_KLEAK_G 7
#define BC_P_NA_G 8
#define BC_P_NA_VSH 9
#define BC_P_NA_PHI 10
#define BC_P_KDR_G 11
#define BC_P_KDR_VSH 12
#define BC_P_KDR_PHI 13
#define BC_P_CAL_G 14
#define BC_P_CAL_VSH 15
#define BC_P_CAL_PHIP 16
#define BC_P_CAL_PHIQ 17
#define BC_P_CAT_G 18
#define BC_P_CAT_VSH 19
#define BC_P_CAT_PHIP 20
#define BC_P_CAT_PHIQ 21
#define BC_P_HCN_G 22
#define BC_P_HCN_E 23
#define BC_P_HCN_PHI 24
#define BC_P_AHP_G 25
#define BC_P_AHP_N 26
#define BC_P_AHP_ALPHA 27
#define BC_P_AHP_BETA 28
#define BC_P_AHP_PHI 29
#define BC_P_CA_D 30      /* shell depth (um)                                  */
#define BC_P_CA_TAU 31    /* ms                                                */
#define BC_P_CA_CREST 32  /* mM                                                */
#define BC_P_CA_CO 33     /* mM                                                */
#define BC_P_CA_TEMP 34   /* K                                                 */
#define BC_P_CA_CI0 35    /* mM, reset value of Ci                             */
#define BC_P_NAHH_G 36
#define BC_P_NAHH_VSH 37
#define BC_P_NAHH_PHI 38
#define BC_P_KHH_G 39
#define BC_P_KHH_VSH 40
#define BC_P_KHH_PHI 41
#define BC_P_KM_G 42
#define BC_P_KM_PHI 43
#define BC_P_KA1_G 44
#define BC_P_KA1_VSH 45
#define BC_P_KA1_PHIP 46
#define BC_P_KA1_PHIQ 47
#define BC_P_KA2_G 48
#define BC_P_KA2_VSH 49
#define BC_P_KA2_PHIP 50
#define BC_P_KA2_PHIQ 51
#define BC_P_KK2A_G 52
#define BC_P_KK2A_VSH 53
#define BC_P_KK2A_PHIP 54
#define BC_P_KK2A_PHIQ 55
#define BC_P_KK2B_G 56
#define BC_P_KK2B_VSH 57
#define BC_P_KK2B_PHIP 58
#define BC_P_KK2B_PHIQ 59
#define BC_P_KNI_G 60
#define BC_P_KNI_VSH 61
#define BC_P_KNI_PHI 62
#define BC_P_KNI_TAUMAX 63  /* ms */
#define BC_P_NAV16_G 64
#define BC_P_NAV16_PHI 65   /* 3^((T - 22 degC) / 10)                               */
#define BC_P_KCA22_G 66
#define BC_P_KCA22_PHI 67   /* q10^((T - 23 degC) / 10)                             */
#define BC_P_KCA22_DIFF 68  /* divisor of the calcium-binding rates                 */
#define BC_P_KCA11_G 69
#define BC_P_KCA11_PHI 70   /* q10^((T - 23 degC) / 10)                             */
#define BC_P_KCA11_QO 71    /* Qo F / (R T) per mV: alpha(V) = exp(QO V)            */
#define BC_P_KCA11_QC 72    /* Qc F / (R T) per mV: beta(V) = exp(QC V)             */
#define BC_P_NAV16_OON 73   /* the Nav1.6 scheme's Oon (Nav1p6 0.75, Nav1p1 2.3)    */
#define BC_P_KV34_G 74
#define BC_P_KV34_PHI 75    /* 3^((T - 37 degC) / 10)                               */
#define BC_P_KV43_G 76
#define BC_P_KV43_PHI 77    /* 3^((T - 25.5 degC) / 10)                             */
#define BC_P_KV11_G 78
#define BC_P_KV11_PHI 79    /* 2.7^((T - 22 degC) / 10)                             */
#define BC_P_KIR23_G 80
#define BC_P_KIR23_PHI 81   /* 3^((T - 20 degC) / 10)                               */
#define BC_P_HCN1F_G 82     /* g_max x 1.5^((T - 23 degC) / 10)                     */
#define BC_P_HCN1F_E 83
#define BC_P_HCN1F_PHI 84   /* 3^((T - 23 degC) / 10)                               */
#define BC_P_HCN1H_G 85
#define BC_P_HCN1H_E 86
#define BC_P_HCN1H_PHI 87   /* 3^((T - 37 degC) / 10)                               */
#define BC_P_NAV16_ALFAC 88 /* (Oon / Con)^(1/4)                                    */
#define BC_P_NAV16_EPS 89   /* epsilon, the open -> blocked rate (Nav1p1: 1e-12)   */
#define BC_P_CAHVA_G 90
#define BC_P_CAHVA_PHI 91   /* 3^((T - 20 degC) / 10)                               */
#define BC_P_CAV23_G 92
#define BC_P_CAV32_G 93
#define BC_P_CAV32_VSH 94
/* 95: reserved (0) */
#define BC_P_EXT_MASK 96    /* BC_X_* bits 0-23 of the region's extension channels  */
#define BC_P_HCN2_G 97      /* g_max x 1.5^((T - 23 degC) / 10)                     */
#define BC_P_HCN2_E 98
#define BC_P_HCN2_PHI 99    /* 3^((T - 23 degC) / 10)                               */
#define BC_P_KV33_G 100
#define BC_P_KV33_PHI 101   /* 2.7^((T - 22 degC) / 10)                             */
#define BC_P_KV22_G 102
#define BC_P_KV15_G 103
#define BC_P_KV15_Q10 104   /* 2.2^((T - 37 degC) / 10), on the m and n rates       */
#define BC_P_KV15_TACT 105  /* Tauact, Tauinactf, Tauinacts: time-constant scales   */
#define BC_P_KV15_TINF 106
#define BC_P_KV15_TINS 107
#define BC_P_NAF_G 108
#define BC_P_NAP_G 109
#define BC_P_NAIO_G 110
#define BC_P_FKDR_G 111
#define BC_P_SKDR_G 112
#define BC_P_KDRIO_G 113
#define BC_P_HCNDCN_G 114
#define BC_P_HCNDCN_E 115
#define BC_P_HCNIO_G 116
#define BC_P_HCNIO_E 117
#define BC_P_CATHP_G 118
#define BC_P_CATHP_VSH 119
#define BC_P_CATHP_PHIP 120 /* q10_p^((T - temp_ref_p) / 10)                        */
#define BC_P_CATHP_PHIQ 121
#define BC_P_CAHTRE_G 122
#define BC_P_CAHTRE_VSH 123
#define BC_P_CAHTRE_PHIP 124
#define BC_P_CAHTRE_PHIQ 125
#define BC_P_CALDCN_G 126
#define BC_P_CALDCN_E 127
#define BC_P_KCA31_G 128
#define BC_P_SKDCN_G 129
#define BC_P_KKV_G 130
#define BC_P_KKV_VSH 131
#define BC_P_KKV_RA 132     /* 1/(mV ms) */
#define BC_P_KKV_RB 133
#define BC_P_KKV_Q 134      /* mV        */
#define BC_P_KKV_V12 135    /* mV        */
#define BC_P_CAN_G 136
#define BC_P_CAN_E 137
#define BC_P_CAN_PHI 138    /* q10^((T - temp_ref) / 10)                            */
#define BC_P_CAIO_G 139
#define BC_P_CAIO_E 140
#define BC_P_CAIO_MID 141   /* mMidV (mV)                                           */
#define BC_P_CAIO_FREEZE 142 /* 1: m_inf held out of the linearisation (freeze_m_inf) */
#define BC_P_NAVGRC_G 143
#define BC_P_NAVGRC_PHI 144 /* 3^((T - 20 degC) / 10)                               */
#define BC_P_CAV31_G 145    /* permeability (cm/s)                                  */
#define BC_P_CAV31_QT 146   /* q10^((T - temp_ref) / 10): the time constants' divisor */
#define BC_P_CAV31_TGHK 147 /* the GHK temperature T + 0.04 K                       */
#define BC_P_CAV31_FREEZE 148 /* 1: the drive held out of the linearisation (Frozen);
                                 2: Cav3p1Test_PC24's fixed 1 mV drive (g in mS/cm^2)  */
#define BC_P_CAV33_G 149    /* g_scale x perm (cm/s)                                */
#define BC_P_CAV33_PHI 150  /* 2.3^((T - 28 degC) / 10)                             */
#define BC_P_CAV33_TGHK 151 /* the GHK temperature T - 0.01 K                       */
#define BC_P_CAV33_VSH 152
#define BC_P_CAV33_FREEZE 153 /* 1: the drive held out of the linearisation (Frozen) */
#define BC_P_CAV12_G 154
#define BC_P_CAV12_PHI 155  /* q10^((T - temp_ref) / 10)                            */
#define BC_P_CAV13_G 156
#define BC_P_CAV13_PHI 157
#define BC_P_CAV21_G 158    /* permeability (cm/s)                                  */
#define BC_P_CAV21_VSH 159
#define BC_P_CAV21_PHI 160  /* 3^((T - 23 degC) / 10)                               */
#define BC_P_CAV21_TGHK 161 /* the GHK temperature T (K)                            */
#define BC_P_EXT_MASK_HI 162 /* BC_X_* bits 24 and up, shifted down by 24           */
#define BC_P_CAHVADCN_G 163 /* permeability perm (cm/s)                            */
#define BC_P_CAHVADCN_T 164 /* temperature (K) of its drive                         */
#define BC_P_CALVADCN_G 165
#define BC_P_CALVADCN_T 166
#define BC_P_CAV21_FROZEN 167 /* 1: the _Frozen classes' drive (the Cav3.1 model-file GHK
                                 at T + 0.04 K, in BC_P_CAV21_TGHK) held out of the
                                 linearisation                                        */

/* ------------------------------------------------------------------ batch spec */
/*
 * A batch of independent cells described at morphology level.  Cell c owns
 * branches [cell_branch_offsets[c], cell_branch_offsets[c+1]); branch indices in
 * branch_parent are cell-local (root = -1 and must be branch 0 of the cell).
 * Branch b owns segments [branch_seg_offsets[b], branch_seg_offsets[b+1]) and is
 * tiled into branch_ncv[b] uniform CVs (the reference's uniform CV policies).
 * Region r of cell c uses record region_params[(c*n_regions + r)*BC_NPARAM ...],
 * mechanisms region_mech[c*n_regions + r], cable region_cm / region_ra.
 */
typedef struct bc_batch_spec {
  int64_t n_cells;
  int64_t n_branches;
  int64_t n_segments;
  int32_t n_regions;
  const int64_t* cell_branch_offsets; /* [n_cells + 1]                          */
  const int32_t* branch_parent;       /* [n_branches] cell-local, -1 = root     */
  const double* branch_parent_x;      /* [n_branches]                           */
  const double* branch_child_x;       /* [n_branches] 0 or 1                    */
  const int32_t* branch_ncv;          /* [n_branches] >= 1                      */
  const int32_t* branch_region;       /* [n_branches] in [0, n_regions)         */
  const int64_t* branch_seg_offsets;  /* [n_branches + 1]                       */
  const double* seg_length;           /* [n_segments] um                        */
  const double* seg_r_prox;           /* [n_segments] um                        */
  const double* seg_r_dist;           /* [n_segments] um                        */
  const double* region_cm;            /* [n_cells * n_regions] uF/cm^2          */
  const double* region_ra;            /* [n_cells * n_regions] ohm*cm           */
  const uint32_t* region_mech;        /* [n_cells * n_regions] BC_M_* bits      */
  const double* region_params;        /* [n_cells * n_regions * BC_NPARAM]      */
  /* current-clamp segments: active for t_on <= t < t_off (absolute ms).       */
  int64_t n_pulses;
  const int32_t* pulse_cell;          /* [n_pulses]                             */
  const int32_t* pulse_branch;        /* [n_pulses] cell-local branch           */
  const double* pulse_x;              /* [n_pulses] location on the branch      */
  const double* pulse_t_on;           /* [n_pulses] ms                          */
  const double* pulse_t_off;          /* [n_pulses] ms                          */
  const double* pulse_amp;            /* [n_pulses] nA                          */
  /* probes: voltage recorded at (cell, branch, x); spikes detected there.     */
  int64_t n_probes;
  const int32_t* probe_cell;
  const int32_t* probe_branch;
  const double* probe_x;
  /* ExpSyn synapses (synapse/markov.py:65-117): state g (uS), g' = -g / tau; an
     arriving event adds its weight to g at the start of a step; current
     i = g (V - e) enters the CV holding the synapse as i / area.  Must sit
     inside a CV (0 < x < 1 on its branch).                                      */
  int64_t n_synapses;
  const int32_t* syn_cell;
  const int32_t* syn_branch;
  const double* syn_x;
  const double* syn_tau;              /* ms                                     */
  const double* syn_e;                /* mV                                     */
  /* connections (network/engine.py:474-530): when any CV of cell conn_pre
     crosses 0 mV upward within step s, conn_weight (uS) reaches synapse
     conn_post at step s + max(ceil(conn_delay / dt), 1).                        */
  int64_t n_connections;
  const int32_t* conn_pre;            /* cell index                             */
  const int64_t* conn_post;           /* synapse index                          */
  const double* conn_weight;          /* uS                                     */
  const double* conn_delay;           /* ms, >= 0                               */
  /* subtree-surrogate ports (no counterpart in the reference: the learned
     stand-in for distal dendritic subtrees).  Port k replaces a removed subtree
     of cell port_cell[k] that hung off the distal end (x = 1) of branch
     port_branch[k]: the port node is that endpoint, the attachment compartment
     is the branch's last CV.  Every step the port injects
       I = g (e + y_scale * y - V_end)   nA (g in uS, V in mV)
     into the endpoint row, its conductance part implicit, y being the output of
     the plan's GRU (bc_surrogate_set) fed with
       ((V_att - e) / v_scale, S / 0.1 nA, feat[0], feat[1]),
     S = the port's stimulus, i.e. the sum of its active port pulses (nA).      */
  int64_t n_ports;
  const int32_t* port_cell;
  const int32_t* port_branch;
  const double* port_g;               /* uS, > 0                                */
  const double* port_e;               /* mV                                     */
  const double* port_feat;            /* [n_ports][2] static features           */
  int64_t n_port_pulses;
  const int32_t* port_pulse_port;     /* port index                             */
  const double* port_pulse_t_on;      /* ms                                     */
  const double* port_pulse_t_off;     /* ms                                     */
  const double* port_pulse_amp;       /* nA                                     */
  /* what each probe records (mech/_point.py StateProbe / MechanismProbe /
     CurrentProbe, sampled as _multi_compartment/probes.py:44-258 does): a
     BC_STATE_* view -- 0 = V, else the named gate or Ci of the mechanism at the
     probe's CV -- or BC_PROBE_CURRENT + BC_CUR_* for a current density, after
     the step.  Null: every probe records V.                                    */
  const int32_t* probe_field;         /* [n_probes]                             */
} bc_batch_spec;

/* ------------------------------------------------------------------ plan options */
#define BC_PREC_F32 0 /* FP32 state + arithmetic, float-float (Kahan) V and Ci */
#define BC_PREC_F64 1 /* FP64 throughout: the on-GPU oracle run                 */

typedef struct bc_plan_options {
  int32_t precision;        /* BC_PREC_*                                             */
  int32_t threads_per_tile; /* CTA size (multiple of 32, <= 1024); 0 = auto          */
  int32_t tile_nodes;       /* node budget per tile (shared-memory size); 0 = auto   */
  int32_t lane_nodes;       /* nodes a lane walks serially inside a warp slot; longer
                               chains are spread over lanes joined by shuffle scans;
                               0 = auto (10)                                         */
  int32_t steps_per_launch; /* time steps fused per kernel launch; 0 = auto          */
  int32_t record_every;     /* probe sampling period in steps (>= 1)                 */
  int32_t max_spikes;       /* spike times kept per probe                            */
  int32_t use_graph;        /* 1: each bc_run replays a CUDA graph of its launches
                               (one kernel-node chain per launch class), built when
                               the launch pattern changes and otherwise only
                               re-parameterised; results are bit-identical        */
  int32_t device;           /* CUDA device ordinal                                   */
  int32_t threads_big;      /* CTA size for tiles holding one cell larger than
                               tile_nodes; 0 = auto                                   */
  int32_t threads_global;   /* CTA size for global-memory tiles; 0 = auto            */
  int32_t narrow_lane_nodes; /* lane_nodes for narrow phases (fewer nodes than one
                               warp slot per warp); 0 = auto (1)                  */
  float reserved_b;         /* must be 0                                             */
  int32_t dry_run;          /* 1: lower and schedule only (no CUDA calls); the plan
                               answers bc_plan_info / bc_plan_tile_stats only         */
  int32_t lane_cell_nodes;  /* cells of at most this many tree nodes run one per thread
                               (serial solve per cell, cells interleaved node by node in
                               global memory) instead of in packed tiles; plans without
                               synapses, connections, mechanism probes or ports; 0 = off */
  int32_t tile_order;       /* launch order of the tiles of a class: 0 = the order the
                               packer built them (largest cells first); 1 = longest
                               estimated step first (critical path, then nodes), so
                               the last wave of CTAs is made of short tiles         */
} bc_plan_options;

typedef struct bc_plan* bc_plan_t;

/* Plan statistics (host-side, filled by bc_plan_info). */
typedef struct bc_plan_info_t {
  int64_t n_cells, n_cv, n_nodes, n_tiles, n_probes, n_pulses;
  int32_t threads_per_tile, tile_nodes, steps_per_launch, precision;
  int64_t smem_bytes_per_tile;   /* dynamic shared memory per CTA                    */
  int64_t device_bytes;          /* device memory held by the plan                   */
  int64_t max_phases;            /* largest barrier-phase count of any tile          */
  int64_t max_chain_nodes;       /* longest per-thread node walk (critical path)     */
  int32_t state_slots;           /* per-node mechanism state slots                   */
  int32_t n_smem_tiles;          /* tiles resident in shared memory                  */
  int32_t n_launch_classes;      /* kernel launches per fused step block             */
  int32_t kernel_variant;        /* BC_VARIANT_* the plan launches                   */
  int32_t reserved[4];
} bc_plan_info_t;
/* Step-kernel variants: lean (the main channel mix only), extra (synapses, spike
 * sources, mechanism and current probes, the channels outside the main mix), ports
 * (extra plus subtree-surrogate GRU ports), ports on the lean kernel. */
#define BC_VARIANT_LEAN 0
#define BC_VARIANT_EXTRA 1
#define BC_VARIANT_PORTS 2
#define BC_VARIANT_PORTS_LEAN 3 /* ports on the lean kernel: plans with ports and no other
                                   optional feature (no synapses, mechanism probes or
                                   channels outside the main mix)                  */

/* ------------------------------------------------------------------ entry points */
/* Thread-local text of the last failure (never NULL). */
const char* bc_last_error(void);
/* ABI version: major * 10000 + minor * 100 + patch.  0.2.0: the 64-entry parameter
 * record, the A / K2 / KNI mechanisms, named plan-info fields.  0.3.0: the V_last
 * state view (BC_NSTATE_VIEW 25), bc_spike_state_download, bc_pulse_set_amp, the
 * workspace of bc_gru_backward (bit-reproducible gradients).  0.4.0: the Markov
 * channels (BC_M_NAV16 / KCA22 / KCA11, a 74-entry parameter record, state views
 * 25-50), lane tiles (bc_plan_options.lane_cell_nodes, tile_order), the cerebellar
 * HH and calcium channels (BC_M_KV34 .. CAV32, a 96-entry parameter record, state
 * views 51-65, BC_PROBE_CURRENT 128).  0.5.0: extension channels (BC_M_EXT with
 * BC_X_* bits in the record's BC_P_EXT_MASK / _HI, a 168-entry parameter record,
 * state views 66-121, current codes 31-58). */
#define BC_ABI_VERSION 500
int32_t bc_version(void);
/* Fill opts with defaults. */
void bc_default_options(bc_plan_options* opts);

/* Lower a batch (geometry -> CVs -> node tree -> axial coefficients), schedule it
 * into shared-memory tiles and allocate the device buffers.  Replaces the
 * reference's one-time lowering (Cell.init_state, cell.py:490-552) and the cached
 * DHS static source (_staggered.py:323-446). */
bc_status bc_plan_create(const bc_batch_spec* spec, const bc_plan_options* opts, bc_plan_t* out);
bc_status bc_plan_destroy(bc_plan_t plan);
bc_status bc_plan_info(bc_plan_t plan, bc_plan_info_t* info);

/* Per-tile schedule statistics, 6 int64 per tile in launch order: real nodes,
 * chain records, barrier phases, critical-path estimate (node visits of the
 * busiest thread summed over phases), launch class (0 packed shared-memory tile,
 * 1 single-cell shared-memory tile, 2 global-memory tile, 3 lane tile: one cell per
 * thread), shared bytes. */
bc_status bc_plan_tile_stats(bc_plan_t plan, int64_t* out /* [n_tiles * 6] */);

/* The native lowering of one cell, for checking against other assemblies (host
 * only, no CUDA).  Points are numbered like the reference's node tree
 * (_discretization/node_build.py:58-285).  Pass NULL arrays to query the sizes.
 *   cv_area [n_cv] um^2, cv_node [n_cv] midpoint point of each CV,
 *   parent [n_node], alpha / beta / diag [n_node] axial coefficients in 1/ms
 *   (row i: diag_i x_i - alpha_i x_parent - sum_c beta_c x_c), region [n_node]
 *   (-1 on boundary points). */
bc_status bc_lower_cell(const bc_batch_spec* spec, int64_t cell, int32_t* n_cv, int32_t* n_node, double* cv_area,
                        int32_t* cv_node, int32_t* parent, double* alpha, double* beta, double* diag,
                        int32_t* region);

/* Sizes of the host-side views (CV count per cell, in reference CV order). */
bc_status bc_plan_cell_ncv(bc_plan_t plan, int64_t* ncv_out /* [n_cells] */);

/* Reset all states: V = region V_rest, gates at steady state at V, Ci = Ci0,
 * spike counters and step counter cleared.  Mirrors Cell.reset_state
 * (cell.py:2529-2550) with HH.reset_state (channel/_base.py:560-573). */
bc_status bc_reset(bc_plan_t plan, void* stream);

/* Advance n_steps time steps of size dt (ms) from the plan's step counter, in
 * launches of steps_per_launch fused steps.  Mirrors n_steps calls of
 * staggered_step with t = t0 + k * dt.  Returns BC_ERR_NONFINITE if any probe
 * or node voltage became non-finite (checked when the call completes). */
bc_status bc_run(bc_plan_t plan, int64_t n_steps, double dt, void* stream);

/* Same as bc_run but enqueues only; no host synchronisation and no status check.
 * Use bc_check to read the device status later. */
bc_status bc_run_async(bc_plan_t plan, int64_t n_steps, double dt, void* stream);
bc_status bc_check(bc_plan_t plan, void* stream);

/* Read/write state in reference order (float64 host arrays).
 *   V per CV:         [n_cv]   (cell-major, CV ids as the reference numbers them)
 *   state per CV:     [n_cv * BC_NSTATE_VIEW], the named view below            */
#define BC_STATE_V 0
#define BC_STATE_NA_P 1
#define BC_STATE_NA_Q 2
#define BC_STATE_KDR_P 3
#define BC_STATE_CAL_P 4
#define BC_STATE_CAL_Q 5
#define BC_STATE_CAT_P 6
#define BC_STATE_CAT_Q 7
#define BC_STATE_HCN_P 8
#define BC_STATE_AHP_P 9
#define BC_STATE_CA_CI 10
#define BC_STATE_NAHH_P 11
#define BC_STATE_NAHH_Q 12
#define BC_STATE_KHH_P 13
#define BC_STATE_KM_N 14
#define BC_STATE_KA1_P 15
#define BC_STATE_KA1_Q 16
#define BC_STATE_KA2_P 17
#define BC_STATE_KA2_Q 18
#define BC_STATE_KK2A_P 19
#define BC_STATE_KK2A_Q 20
#define BC_STATE_KK2B_P 21
#define BC_STATE_KK2B_Q 22
#define BC_STATE_KNI_P 23
#define BC_STATE_V_LAST 24 /* V at the start of the last step taken (= V after a reset);
                              not a probe field                                    */
/* Markov states: the independent states of each scheme, in the order they first
   appear in its transition list (the dependent state is 1 - their sum).         */
#define BC_STATE_NAV16_C1 25 /* .. C5 29, I1 30 .. I5 34, O 35, B 36 (I6 dependent) */
#define BC_STATE_NAV16_O 35
#define BC_STATE_KCA22_C2 37 /* C3 38, C4 39, O1 40, O2 41 (C1 dependent)           */
#define BC_STATE_KCA11_C1 42 /* C2 43, C3 44, C4 45, O0 46 .. O4 50 (C0 dependent) */
#define BC_STATE_KV34_M 51
#define BC_STATE_KV34_H 52
#define BC_STATE_KV43_A 53
#define BC_STATE_KV43_B 54
#define BC_STATE_KV11_N 55
#define BC_STATE_KIR23_D 56
#define BC_STATE_HCN1F_FAST 57
#define BC_STATE_HCN1F_SLOW 58
#define BC_STATE_HCN1H_H 59
#define BC_STATE_CAHVA_S 60
#define BC_STATE_CAHVA_U 61
#define BC_STATE_CAV23_M 62
#define BC_STATE_CAV23_H 63
#define BC_STATE_CAV32_M 64
#define BC_STATE_CAV32_H 65
/* extension channels' gates */
#define BC_STATE_HCN2_FAST 66
#define BC_STATE_HCN2_SLOW 67
#define BC_STATE_KV33_N 68
#define BC_STATE_KV22_M 69
#define BC_STATE_KV22_H 70
#define BC_STATE_KV15_M 71
#define BC_STATE_KV15_N 72
#define BC_STATE_KV15_U 73
#define BC_STATE_NAF_M 74
#define BC_STATE_NAF_H 75
#define BC_STATE_NAP_M 76
#define BC_STATE_NAP_H 77
#define BC_STATE_NAIO_M 78
#define BC_STATE_NAIO_H 79
#define BC_STATE_FKDR_M 80
#define BC_STATE_SKDR_M 81
#define BC_STATE_KDRIO_N 82
#define BC_STATE_HCNDCN_M 83
#define BC_STATE_HCNIO_Q 84
#define BC_STATE_CATHP_P 85
#define BC_STATE_CATHP_Q 86
#define BC_STATE_CAHTRE_P 87
#define BC_STATE_CAHTRE_Q 88
#define BC_STATE_CALDCN_M 89
#define BC_STATE_CALDCN_H 90
#define BC_STATE_KCA31_P 91
#define BC_STATE_SKDCN_Z 92
#define BC_STATE_KKV_N 93
#define BC_STATE_CAN_P 94
#define BC_STATE_CAIO_H 95
#define BC_STATE_NAVGRC_C1 96 /* .. C5 100, I1 101 .. I5 105, O 106, OB 107 (I6 dependent) */
#define BC_STATE_NAVGRC_O 106
#define BC_STATE_CAV31_P 108
#define BC_STATE_CAV31_Q 109
#define BC_STATE_CAV33_N 110
#define BC_STATE_CAV33_L 111
#define BC_STATE_CAV12_M 112 /* M, H, N: 112 .. 114 */
#define BC_STATE_CAV13_M 115 /* M, H, N: 115 .. 117 */
#define BC_STATE_CAV21_M 118
#define BC_STATE_CAHVADCN_M 119
#define BC_STATE_CALVADCN_M 120
#define BC_STATE_CALVADCN_H 121
#define BC_NSTATE_VIEW 122
/* Current probes (mech/_point.py CurrentProbe, _multi_compartment/probes.py:184-258):
   probe_field = BC_PROBE_CURRENT + one of the codes below records that current
   density (uA/cm^2, outward negative as g (E - V)) after the step.             */
#define BC_PROBE_CURRENT 128
#define BC_CUR_IL 0
#define BC_CUR_KLEAK 1
#define BC_CUR_NA 2      /* Na_Ba2002   */
#define BC_CUR_KDR 3     /* KDR_Ba2002  */
#define BC_CUR_CAL 4     /* CaL_IS2008  */
#define BC_CUR_CAT 5     /* CaT_HM1992  */
#define BC_CUR_HCN 6     /* HCN_HM1992  */
#define BC_CUR_AHP 7     /* AHP_De1994  */
#define BC_CUR_NAHH 8    /* Na_HH1952   */
#define BC_CUR_KHH 9     /* K_HH1952    */
#define BC_CUR_KM 10     /* KM_RI2021_SC */
#define BC_CUR_ION_NA 11 /* sum over the sodium channels    */
#define BC_CUR_ION_K 12  /* sum over the potassium channels */
#define BC_CUR_ION_CA 13 /* sum over the calcium channels   */
#define BC_CUR_KA1 14    /* KA1_HM1992  */
#define BC_CUR_KA2 15    /* KA2_HM1992  */
#define BC_CUR_KK2A 16   /* KK2A_HM1992 */
#define BC_CUR_KK2B 17   /* KK2B_HM1992 */
#define BC_CUR_KNI 18    /* KNI_Ya1989  */
#define BC_CUR_NAV16 19  /* Nav1p6_MA2020_GoC */
#define BC_CUR_KCA22 20  /* Kca2p2_MA2020_GoC */
#define BC_CUR_KCA11 21  /* Kca1p1_MA2020_GoC */
#define BC_CUR_KV34 22   /* Kv3p4_MA2020_GoC  */
#define BC_CUR_KV43 23   /* Kv4p3_MA2020_GoC  */
#define BC_CUR_KV11 24   /* Kv1p1_MA2020_GoC  */
#define BC_CUR_KIR23 25  /* Kir2p3_MA2020_GrC */
#define BC_CUR_HCN1F 26  /* HCN1_MA2020_GoC   */
#define BC_CUR_HCN1H 27  /* HCN1_MA2024_PC    */
#define BC_CUR_CAHVA 28  /* CaHVA_MA2020_GoC  */
#define BC_CUR_CAV23 29  /* Cav2p3_MA2020_GoC */
#define BC_CUR_CAV32 30  /* Cav3p2_RI2021_SC  */
#define BC_CUR_HCN2 31   /* HCN2_MA2020_GoC        */
#define BC_CUR_KV33 32   /* Kv3p3_MA2024_PC        */
#define BC_CUR_KV22 33   /* Kv2p2_0010_MA2020_GrC  */
#define BC_CUR_KV15 34   /* Kv1p5_MA2024_PC        */
#define BC_CUR_NAF 35    /* NaF_SU2015_DCN         */
#define BC_CUR_NAP 36    /* NaP_SU2015_DCN         */
#define BC_CUR_NAIO 37   /* Na_ZH2019_IO           */
#define BC_CUR_FKDR 38   /* fKdr_SU2015_DCN        */
#define BC_CUR_SKDR 39   /* sKdr_SU2015_DCN        */
#define BC_CUR_KDRIO 40  /* Kdr_ZH2019_IO          */
#define BC_CUR_HCNDCN 41 /* HCN_SU2015_DCN         */
#define BC_CUR_HCNIO 42  /* HCN_ZH2019_IO          */
#define BC_CUR_CATHP 43  /* CaT_HP1992             */
#define BC_CUR_CAHTRE 44 /* CaHT_Re1993            */
#define BC_CUR_CALDCN 45 /* CaL_SU2015_DCN         */
#define BC_CUR_KCA31 46  /* Kca3p1_MA2020_GoC      */
#define BC_CUR_SKDCN 47  /* SK_SU2015_DCN          */
#define BC_CUR_KKV 48    /* K_Kv_test              */
#define BC_CUR_CAN 49    /* CaN_IS2008             */
#define BC_CUR_CAIO 50   /* Ca_ZH2019_IO           */
#define BC_CUR_NAVGRC 51 /* Nav_MA2020_GrC         */
#define BC_CUR_CAV31 52  /* Cav3p1_MA2020_GoC      */
#define BC_CUR_CAV33 53  /* Cav3p3_RI2021_SC       */
#define BC_CUR_CAV12 54  /* Cav1p2_MA2020_GoC      */
#define BC_CUR_CAV13 55  /* Cav1p3_MA2020_GoC      */
#define BC_CUR_CAV21 56  /* Cav2p1_RI2021_SC       */
#define BC_CUR_CAHVADCN 57 /* CaHVA_SU2015_DCN     */
#define BC_CUR_CALVADCN 58 /* CaLVA_SU2015_DCN     */
#define BC_NCUR 59
bc_status bc_state_download(bc_plan_t plan, int32_t which, double* out /* [n_cv] */, void* stream);
/* Set the amplitude (nA) of every current-clamp pulse of the batch spec, in spec
 * order (amp_nA[n_pulses]); times and locations are unchanged.  Takes effect from
 * the next step.  The time-varying input of a stepped model goes through this:
 * SingleCompartment.update(I_ext) (_single_compartment/base.py:252-278) passes a
 * new external current every step, which here is one pulse per neuron. */
bc_status bc_pulse_set_amp(bc_plan_t plan, const double* amp_nA, void* stream);
/* Per-CV spike indicator of the last step taken: out[k] = 1 where CV k's voltage
 * crossed v_th upward during that step (V_last < v_th <= V), else 0; all 0 after a
 * reset.  Replaces reading Cell.spike, which the reference sets every step from
 * get_spike(last_V, V) (_base.py:421-431, _multi_compartment/cell.py:2384-2386). */
bc_status bc_spike_state_download(bc_plan_t plan, double v_th, double* out /* [n_cv] */, void* stream);
bc_status bc_state_upload(bc_plan_t plan, int32_t which, const double* in /* [n_cv] */, void* stream);

/* bc_state_download without any allocation.  No counterpart in the reference: its
 * states are ordinary arrays the caller already holds.
 * Who needs it: a caller that reads state while simulations run on other streams
 * (a monitor, a closed-loop controller) and cannot afford cudaMalloc/cudaFree,
 * which synchronise the whole device and so stall every queued launch; and a
 * process whose device memory is already held by a caching allocator, where a
 * fresh cudaMalloc may fail.  bc_state_download allocates its offset tables and
 * value buffer per call; this variant uses one fixed scratch array in the
 * library's device image plus a host staging array of the same capacity, both
 * sized for BC_NOALLOC_MAX_CV compartments (24 bytes each on the device: 6 MiB).
 * Plans with more CVs are rejected with BC_ERR_INVALID (use bc_state_download).
 * The first call on each device looks up the scratch address (cudaGetSymbolAddress)
 * and caches it.  Never call it on a stream that is being captured into a CUDA
 * graph: it copies from pageable host memory and synchronises the stream, so it
 * returns BC_ERR_INVALID there.  The scratch is shared by every plan of the
 * process: calls that overlap in time (from several host threads) race on it, so
 * the caller must serialise them.  Returns once `out` holds the values (the stream
 * is synchronised, on failures too once anything was enqueued). */
#define BC_NOALLOC_MAX_CV 262144
bc_status bc_state_download_noalloc(bc_plan_t plan, int32_t which, double* out /* [n_cv] */, void* stream);

/* Probe outputs.  Traces: [n_probes, n_records] float64 where n_records is the
 * number of samples taken since the last bc_probe_clear.  Spikes: count per probe
 * and up to max_spikes upward 0 mV crossing times (ms, linear interpolation). */
bc_status bc_probe_count(bc_plan_t plan, int64_t* n_records);
bc_status bc_probe_download(bc_plan_t plan, double* traces, int64_t max_records, void* stream);
bc_status bc_spike_download(bc_plan_t plan, int32_t* counts /* [n_probes] */,
                            double* times /* [n_probes * max_spikes] */, void* stream);
bc_status bc_probe_clear(bc_plan_t plan, void* stream);

/* Network outputs.  Spike records (cell, step) of every cell of a plan with
 * connections, in the order the device produced them (by launch; within a
 * launch not sorted), since the last bc_reset; *n_out receives the number of
 * records (also when it exceeds cap, in which case only cap are copied).
 * Synapse conductances g (uS) in synapse order. */
bc_status bc_network_spikes(bc_plan_t plan, int32_t* cells, int64_t* steps, int64_t cap, int64_t* n_out,
                            void* stream);
bc_status bc_synapse_download(bc_plan_t plan, double* g /* [n_synapses] */, void* stream);

/* ------------------------------------------------- subtree surrogate (GRU ports)
 * No counterpart in the reference.  The GRU: hidden BC_GRU_HIDDEN, inputs
 * BC_GRU_INPUTS, parameters as one FP32 vector of bc_gru_nparam() entries:
 *   Wh [3H][H] | Wx [3H][X] | bx [3H] | bh [3H] | wo [H] | bo
 * (gate blocks r, z, n).  Weights are used as BF16 on the tensor cores.         */
#define BC_GRU_HIDDEN 64
#define BC_GRU_INPUTS 4
#define BC_SURROGATE_NORM 5 /* v_scale, y_scale, env_v_lo, env_v_hi, env_dvdt */
int32_t bc_gru_nparam(void);
/* Give the plan its GRU (host arrays) and enable its ports.  norm: v_scale (mV),
   y_scale (mV), the envelope of V_att - e (mV, lo / hi) and of |dV_att/dt|
   (mV/ms): a port input outside it flags the port's cell for the full solve. */
bc_status bc_surrogate_set(bc_plan_t plan, const float* params, const float* norm, void* stream);
/* flags[c] = 1 when a port of cell c saw an input outside the envelope since the
   last reset, else 0 (host array of n_cells).                                  */
bc_status bc_surrogate_flags(bc_plan_t plan, int32_t* flags, void* stream);

/* Training kernels (device pointers; stream-ordered).  x [n_seq][t_total][X]
   and y [n_seq][t_total] hold the sequences; a batch is the sequence ids
   seq[batch]; a window is steps t0 .. t0+T-1.  h [batch][H] carries the hidden
   state in and out.  wext [4H][H+16] / wht [H][3H]: BF16 pairs made by
   bc_gru_pack -- the extended weight matrix of the forward (recurrent weights,
   input weights and biases of the r, z, hn and input-n blocks) and the
   transposed recurrent weights of the backward.  acts [5][batch][T][H] and yout [batch][T] are the forward's
   saved activations (acts may be null when no backward follows).  loss (may be
   null) accumulates the sum of squared errors in FP64.  The backward adds the
   gradient of gscale/2 * sum (y - y_target)^2 into grads.                      */
bc_status bc_gru_pack(const float* params, uint32_t* wext, uint32_t* wht, void* stream);
bc_status bc_gru_forward(const float* params, const uint32_t* wext, const float* x, const float* y, int64_t t_total,
                         const int32_t* seq, int32_t batch, int64_t t0, int32_t T, float* h, float* acts,
                         float* yout, double* loss, void* stream);
/* The backward writes each CTA's gradient (16 sequences each) into its own row
   of workspace (bc_gru_backward_workspace(batch) floats, device memory, no
   initialisation needed) and then adds the rows to grads in a fixed order: the
   gradient is bit-reproducible from run to run.                              */
int64_t bc_gru_backward_workspace(int32_t batch);
bc_status bc_gru_backward(const float* params, const uint32_t* wht, const float* x, const float* y,
                          int64_t t_total, const int32_t* seq, int32_t batch, int64_t t0, int32_t T,
                          const float* acts, const float* yout, float gscale, float* grads, float* workspace,
                          void* stream);
bc_status bc_gru_grad_sqnorm(const float* grads, float* out, void* stream);
/* One Adam step (bias-corrected, step >= 1) on params with grads * clip_scale;
   clears grads.                                                                */
bc_status bc_gru_adam(float* params, float* grads, float* m, float* v, int64_t step, float lr, float beta1,
                      float beta2, float eps, float clip_scale, void* stream);

/* Current step counter (number of steps taken since reset). */
bc_status bc_step_count(bc_plan_t plan, int64_t* steps);

/* Timing helper for measurement: runs n_steps like bc_run_async between two CUDA
 * events recorded on the stream and returns the elapsed device milliseconds of the
 * solver kernels alone (ms_out). */
bc_status bc_run_timed(bc_plan_t plan, int64_t n_steps, double dt, void* stream, double* ms_out);

#ifdef __cplusplus
}
#endif
#endif /* BRAINCELL_GB300_H */
