// Extension channels: classes outside the mechanism bits of the main record,
// listed per region as BC_X_* bits in the record entry BC_P_EXT_MASK and run by
// the extra kernel variant.  Each is an exp-Euler HH channel as the others are
// (gates at the new V, ohmic current in its ion's E or its own E); Kv1p5's
// current carries a voltage factor, so its conductance term is the negative
// V-derivative of the current, as the reference's autodiff linearisation takes
// it (quad/_staggered.py:763-795).
//
// Rate functions, as published in the reference:
//   HCN2_MA2020_GoC        channel/hyperpolarization_activated.py:838-1008
//   Kv3p3_MA2024_PC        channel/potassium.py:2937-3124
//   Kv2p2_0010_MA2020_GrC  channel/potassium.py:5664-5804
//   Kv1p5_MA2024_PC        channel/potassium.py:2735-2935
//   NaF_SU2015_DCN         channel/sodium.py:402-498
//   NaP_SU2015_DCN         channel/sodium.py:500-596
//   Na_ZH2019_IO           channel/sodium.py:598-725
//   fKdr_SU2015_DCN        channel/potassium.py:1374-1483
//   sKdr_SU2015_DCN        channel/potassium.py:1485-1595
//   Kdr_ZH2019_IO          channel/potassium.py:6238-6374
//   HCN_SU2015_DCN         channel/hyperpolarization_activated.py:1010-1107
//   HCN_ZH2019_IO          channel/hyperpolarization_activated.py:1109-1217
//   CaT_HP1992             channel/calcium.py:377-509
//   CaHT_Re1993            channel/calcium.py:667-788
//   CaL_SU2015_DCN         channel/calcium.py:1066-1219
//   Kca3p1_MA2020_GoC      channel/potassium_calcium.py:299-450
//   SK_SU2015_DCN          channel/potassium_calcium.py:189-297
//   K_Kv_test              channel/potassium.py:1239-1372
//   CaN_IS2008             channel/calcium.py:108-220
//   Ca_ZH2019_IO           channel/calcium.py:4837-4979
//   Nav_MA2020_GrC         channel/sodium.py:1427-1666 (on the Markov solver of bc_mech.cuh)
//   Cav3p1_MA2020_GoC      channel/calcium.py:1972-2202 (GHK drive, calcium.py:78-86)
//   Cav3p3_RI2021_SC       channel/calcium.py:4033-4255 (GHK drive, calcium.py:89-97)
//   Cav1p2_MA2020_GoC      channel/calcium.py:1408-1599
//   Cav1p3_MA2020_GoC      channel/calcium.py:1683-1886
//   Cav2p1_RI2021_SC       channel/calcium.py:2767-2953 (GHK drive, channel/_base.py:47)
//   CaHVA_SU2015_DCN       channel/calcium.py:924-1064
//   CaLVA_SU2015_DCN       channel/calcium.py:1221-1406 (CaL_SU2015_DCN's gates)
// CaT_HP1992, CaHT_Re1993 and CaN_IS2008 (in its own E) carry calcium: their
// step-start current joins the calcium shell's drive, as CaL's and CaT's do.  Kca3p1 and SK read Ci: the new Ci
// of a dynamic calcium ion, else the fixed one (BC_P_CA_CI0), as AHP_De1994 does.
#pragma once

#include "bc_mech.cuh"

namespace bc {

// State slots, after the cerebellar channels' (a plan with extension channels
// carries kNumSlotsExt slots per node); view BC_STATE_* k sits in slot k + 1.
constexpr int kSlotHcn2F = 67;
constexpr int kSlotHcn2S = 68;
constexpr int kSlotKv33N = 69;
constexpr int kSlotKv22M = 70;
constexpr int kSlotKv22H = 71;
constexpr int kSlotKv15M = 72;
constexpr int kSlotKv15N = 73;
constexpr int kSlotKv15U = 74;
constexpr int kSlotNafM = 75;
constexpr int kSlotNafH = 76;
constexpr int kSlotNapM = 77;
constexpr int kSlotNapH = 78;
constexpr int kSlotNaioM = 79;
constexpr int kSlotNaioH = 80;
constexpr int kSlotFkdrM = 81;
constexpr int kSlotSkdrM = 82;
constexpr int kSlotKdrioN = 83;
constexpr int kSlotHcndcnM = 84;
constexpr int kSlotHcnioQ = 85;
constexpr int kSlotCathpP = 86;
constexpr int kSlotCathpQ = 87;
constexpr int kSlotCahtreP = 88;
constexpr int kSlotCahtreQ = 89;
constexpr int kSlotCaldcnM = 90;
constexpr int kSlotCaldcnH = 91;
constexpr int kSlotKca31P = 92;
constexpr int kSlotSkdcnZ = 93;
constexpr int kSlotKkvN = 94;
constexpr int kSlotCanP = 95;
constexpr int kSlotCaioH = 96;
constexpr int kSlotNavGrc = 97;  // C1..C5, I1..I5, O, OB in 97..108 (I6 dependent)
constexpr int kSlotCav31P = 109;
constexpr int kSlotCav31Q = 110;
constexpr int kSlotCav33N = 111;
constexpr int kSlotCav33L = 112;
constexpr int kSlotCav12 = 113;  // m, h, n
constexpr int kSlotCav13 = 116;  // m, h, n
constexpr int kSlotCav21M = 119;
constexpr int kSlotCahvadcnM = 120;
constexpr int kSlotCalvadcnM = 121;
constexpr int kSlotCalvadcnH = 122;
constexpr int kNumSlotsExt = 123;

// x / (1 - e^-x) = 1 / exprel(-x), finite at x = 0 (the reference's
// _x_over_one_minus_exp_neg_stable, channel/sodium.py:50-55)
template <typename Real>
__host__ __device__ __forceinline__ Real x_over_1mexp(Real x) {
  return Real(1) / exprel(-x);
}

// HCN2_MA2020_GoC: o_inf split by r(V), clamped to 0 above -64.7 mV and to 1
// below -108.7 mV; time constants exp((tC V - tD) tE).
template <typename Real>
struct Hcn2Rates {
  Real finf, ftau, sinf, stau;
  __host__ __device__ __forceinline__ explicit Hcn2Rates(Real v) {
    const Real o = Real(1) / (Real(1) + aexp((v + Real(81.95)) * Real(0.1661)));
    const Real r = v >= Real(-64.70) ? Real(0) : (v <= Real(-108.70) ? Real(1) : Real(-0.0227) * v - Real(1.4694));
    finf = r * o;
    sinf = (Real(1) - r) * o;
    ftau = aexp((Real(0.0269) * v + Real(5.6111)) * Real(2.3026));
    stau = aexp((Real(0.0152) * v + Real(5.2944)) * Real(2.3026));
  }
};

// Kv3p3_MA2024_PC: n, alpha / beta = 0.22 exp(-+(V + 16) / 26.5).
template <typename Real>
struct Kv33Rates {
  Real a, b;
  __host__ __device__ __forceinline__ explicit Kv33Rates(Real v) {
    a = Real(0.22) * aexp(-(v + Real(16)) / Real(-26.5));
    b = Real(0.22) * aexp(-(v + Real(16)) / Real(26.5));
  }
};

// Kv2p2_0010_MA2020_GrC: m and h, inf / tau.
template <typename Real>
struct Kv22Rates {
  Real minf, mtau, hinf, htau;
  __host__ __device__ __forceinline__ explicit Kv22Rates(Real v) {
    minf = Real(1) / (Real(1) + aexp((v - Real(5)) / Real(-12)));
    const Real d = Real(1) + aexp((v + Real(46.56)) / Real(-44.14));
    mtau = Real(130) / d;
    hinf = Real(1) / (Real(1) + aexp((v + Real(16.3)) / Real(4.8)));
    htau = Real(10000) / d;
  }
};

// Kv1p5_MA2024_PC: m^3 n u; the Q10 factor q scales the m and n rates, the
// Tau* parameters scale the time constants.
template <typename Real>
struct Kv15Rates {
  Real minf, mtau, ninf, ntau, uinf;
  __host__ __device__ __forceinline__ Kv15Rates(Real v, Real q, Real tact, Real tinf) {
    minf = Real(1) / (Real(1) + aexp(-(v + Real(30.3)) / Real(9.6)));
    const Real am = q * Real(0.65) / (aexp(-(v + Real(10)) / Real(8.5)) + aexp(-(v - Real(30)) / Real(59)));
    const Real bm = q * Real(0.65) / (Real(2.5) + aexp((v + Real(82)) / Real(17)));
    mtau = Real(1) / (am + bm) / Real(3) * tact;
    ninf = Real(0.25) + Real(1) / (Real(1.35) + aexp((v + Real(7)) / Real(14)));
    const Real an = q * Real(0.001) / (Real(2.4) + Real(10.9) * aexp(-(v + Real(90)) / Real(78)));
    const Real bn = q * Real(0.001) * aexp((v - Real(168)) / Real(16));
    ntau = Real(1) / (an + bn) / Real(3) * tinf;
    uinf = Real(0.1) + Real(1) / (Real(1.1) + aexp((v + Real(7)) / Real(14)));
  }
};
// u's time constant: 6800 ms x Tauinacts
constexpr double kKv15TauU = 6800.0;

// Kv1p5's voltage factor f(V) = 0.1 + s, s = 1 / (1 + exp(-(V - 15) / 13)), and
// its derivative s (1 - s) / 13.
template <typename Real>
__host__ __device__ __forceinline__ void kv15_vfactor(Real v, Real& f, Real& df) {
  const Real s = Real(1) / (Real(1) + aexp(-(v - Real(15)) / Real(13)));
  f = Real(0.1) + s;
  df = s * (Real(1) - s) / Real(13);
}

// NaF_SU2015_DCN: m^3 h, inf / tau (qdeltat = 1).
template <typename Real>
struct NafRates {
  Real minf, mtau, hinf, htau;
  __host__ __device__ __forceinline__ explicit NafRates(Real v) {
    minf = Real(1) / (Real(1) + aexp((v + Real(45)) / Real(-7.3)));
    mtau = Real(5.83) / (aexp((v - Real(6.4)) / Real(-9)) + aexp((v + Real(97)) / Real(17))) + Real(0.025);
    hinf = Real(1) / (Real(1) + aexp((v + Real(42)) / Real(5.9)));
    htau = Real(16.67) / (aexp((v - Real(8.3)) / Real(-29)) + aexp((v + Real(66)) / Real(9))) + Real(0.2);
  }
};

// NaP_SU2015_DCN: m^3 h, inf / tau, m's tau 50 ms.
template <typename Real>
struct NapRates {
  Real minf, mtau, hinf, htau;
  __host__ __device__ __forceinline__ explicit NapRates(Real v) {
    minf = Real(1) / (Real(1) + aexp((v + Real(70)) / Real(-4.1)));
    mtau = Real(50);
    hinf = Real(1) / (Real(1) + aexp((v + Real(80)) / Real(4)));
    htau = Real(1750) / (Real(1) + aexp((v + Real(65)) / Real(-8))) + Real(250);
  }
};

// Na_ZH2019_IO: m^3 h from alpha / beta, m's tau 0.001 ms, h's 250 / (a + b).
template <typename Real>
struct NaioRates {
  Real minf, mtau, hinf, htau;
  __host__ __device__ __forceinline__ explicit NaioRates(Real v) {
    const Real am = x_over_1mexp((v + Real(41)) / Real(10));
    const Real bm = Real(9) * aexp(-(v + Real(66)) / Real(20));
    const Real ah = Real(5) * aexp(-(v + Real(60)) / Real(15));
    const Real bh = Real(10) * x_over_1mexp((v + Real(50)) / Real(10));
    minf = am / (am + bm);
    mtau = Real(0.001);
    hinf = ah / (ah + bh);
    htau = Real(250) / (ah + bh);
  }
};

// fKdr / sKdr_SU2015_DCN: m^4, inf = 1 / (1 + exp((V + vh) / k)),
// tau = c / (exp((V + vh) / k1) + exp((V + vh) / k2)) + t0 (qdeltat = 1).
template <typename Real>
struct Su2015KdrRates {
  Real minf, mtau;
  __host__ __device__ __forceinline__ Su2015KdrRates(Real v, Real vh, Real k, Real c, Real k1, Real k2, Real t0) {
    const Real x = v + vh;
    minf = Real(1) / (Real(1) + aexp(x / k));
    mtau = c / (aexp(x / k1) + aexp(x / k2)) + t0;
  }
};
template <typename Real>
__host__ __device__ __forceinline__ Su2015KdrRates<Real> fkdr_rates(Real v) {
  return Su2015KdrRates<Real>(v, Real(40), Real(-7.8), Real(13.9), Real(12), Real(-13), Real(0.1));
}
template <typename Real>
__host__ __device__ __forceinline__ Su2015KdrRates<Real> skdr_rates(Real v) {
  return Su2015KdrRates<Real>(v, Real(50), Real(-9.1), Real(14.95), Real(21.74), Real(-13.91), Real(0.05));
}

// Kdr_ZH2019_IO: n^4 from alpha / beta, tau 10 / (a + b).
template <typename Real>
struct KdrioRates {
  Real ninf, ntau;
  __host__ __device__ __forceinline__ explicit KdrioRates(Real v) {
    const Real a = Real(10) * x_over_1mexp((v + Real(41)) / Real(10));
    const Real b = Real(12.5) * aexp(-(v + Real(51)) / Real(80));
    ninf = a / (a + b);
    ntau = Real(10) / (a + b);
  }
};

// HCN_SU2015_DCN: m^2, m's tau 400 ms.
template <typename Real>
struct HcndcnRates {
  Real minf, mtau;
  __host__ __device__ __forceinline__ explicit HcndcnRates(Real v) {
    minf = Real(1) / (Real(1) + aexp((v + Real(80)) / Real(5)));
    mtau = Real(400);
  }
};

// HCN_ZH2019_IO: q, tau = 1 / (exp(-0.086 V - 14.6) + exp(0.07 V - 1.87)).
template <typename Real>
struct HcnioRates {
  Real qinf, qtau;
  __host__ __device__ __forceinline__ explicit HcnioRates(Real v) {
    qinf = Real(1) / (Real(1) + aexp((v + Real(75)) / Real(5.5)));
    qtau = Real(1) / (aexp(Real(-0.086) * v - Real(14.6)) + aexp(Real(0.07) * v - Real(1.87)));
  }
};

// CaT_HP1992: p^2 q on V - V_sh, inf / tau.
template <typename Real>
struct CathpRates {
  Real pinf, ptau, qinf, qtau;
  __host__ __device__ __forceinline__ CathpRates(Real v, Real vsh) {
    const Real x = v - vsh;
    pinf = Real(1) / (Real(1) + aexp(-(x + Real(52)) / Real(7.4)));
    ptau = Real(3) + Real(1) / (aexp((x + Real(27)) / Real(10)) + aexp(-(x + Real(102)) / Real(15)));
    qinf = Real(1) / (Real(1) + aexp((x + Real(80)) / Real(5)));
    qtau = Real(85) + Real(1) / (aexp((x + Real(48)) / Real(4)) + aexp(-(x + Real(407)) / Real(50)));
  }
};

// CaHT_Re1993: p^2 q from alpha / beta of t = V_sh - V; alpha_p's
// d / (e^(d / 3.8) - 1) (d = t - 27) is 3.8 / exprel(d / 3.8), finite at d = 0.
template <typename Real>
struct CahtreRates {
  Real ap, bp, aq, bq;
  __host__ __device__ __forceinline__ CahtreRates(Real v, Real vsh) {
    const Real t = vsh - v;
    ap = Real(0.055 * 3.8) / exprel((t - Real(27)) / Real(3.8));
    bp = Real(0.94) * aexp((t - Real(75)) / Real(17));
    aq = Real(0.000457) * aexp((t - Real(13)) / Real(50));
    bq = Real(0.0065) / (aexp((t - Real(15)) / Real(28)) + Real(1));
  }
};

// CaL_SU2015_DCN: m^2 h, h's tau piecewise at -81 mV (qdeltat = 1).
template <typename Real>
struct CaldcnRates {
  Real minf, mtau, hinf, htau;
  __host__ __device__ __forceinline__ explicit CaldcnRates(Real v) {
    minf = Real(1) / (Real(1) + aexp((v + Real(56)) / Real(-6.2)));
    mtau = Real(0.333) / (aexp((v + Real(131)) / Real(-16.7)) + aexp((v + Real(15.8)) / Real(18.2))) + Real(0.204);
    hinf = Real(1) / (Real(1) + aexp((v + Real(80)) / Real(4)));
    htau = v < Real(-81) ? Real(0.333) * aexp((v + Real(466)) / Real(66))
                         : Real(0.333) * aexp((v + Real(21)) / Real(-10.5)) + Real(9.32);
  }
};

// Kca3p1_MA2020_GoC: p, alpha = exp((V + 70) / 27) c(Ci), beta = 0.05, with
// c = 500 (0.015 - Ci) / (exp((0.015 - Ci) / 0.0013) - 1) below Ci = 0.01 mM and its
// value at 0.01 above (temperature parameters accepted but unused, phi 1).
template <typename Real>
struct Kca31Rates {
  Real a, b;
  __host__ __device__ __forceinline__ Kca31Rates(Real v, Real ci) {
    const Real c = ci < Real(0.01) ? Real(500 * 0.0013) / exprel((Real(0.015) - ci) / Real(0.0013))
                                   : Real(500 * 0.0013) / exprel(Real(0.005 / 0.0013));
    a = aexp((v + Real(70)) / Real(27)) * c;
    b = Real(0.05);
  }
};

// SK_SU2015_DCN: z, inf = Ci^4 / (Ci^4 + 8.1e-15), tau = 1 - 186.67 Ci below
// Ci = 0.005 mM, else 0.0667 ms (qdeltat = 1).
template <typename Real>
struct SkdcnRates {
  Real zinf, ztau;
  __host__ __device__ __forceinline__ explicit SkdcnRates(Real ci) {
    const Real c2 = ci * ci;
    const Real c4 = c2 * c2;
    zinf = c4 / (c4 + Real(8.1e-15));
    ztau = ci < Real(0.005) ? Real(1) - Real(186.67) * ci : Real(0.0667);
  }
};

// K_Kv_test: n on y = V - V_sh - v12; inf = 1 / (1 + exp(-y / q)),
// 1 / tau = Ra y / (1 - e^(-y / q)) - Rb y / (1 - e^(y / q)), i.e.
// q (Ra x/(1 - e^-x) at x = y / q + Rb the same at -y / q), finite at y = 0.
template <typename Real>
struct KkvRates {
  Real ninf, ntau;
  __host__ __device__ __forceinline__ KkvRates(Real v, Real vsh, Real ra, Real rb, Real q, Real v12) {
    const Real y = v - vsh - v12;
    ninf = Real(1) / (Real(1) + aexp(-y / q));
    ntau = Real(1) / (q * (ra * x_over_1mexp(y / q) + rb * x_over_1mexp(-y / q)));
  }
};

// CaN_IS2008: p, inf / tau (its current carries Ci / (Ci + 0.2 mM)).
template <typename Real>
struct CanRates {
  Real pinf, ptau;
  __host__ __device__ __forceinline__ explicit CanRates(Real v) {
    pinf = Real(1) / (Real(1) + aexp(-(v + Real(43)) / Real(5.2)));
    ptau = Real(2.7) / (aexp(-(v + Real(55)) / Real(15)) + aexp((v + Real(55)) / Real(15))) + Real(1.6);
  }
};

// Ca_ZH2019_IO: h, inf / tau; the current's instantaneous m_inf = 1 / t^3 with
// t = 1 + exp((mMidV - V) / 4.2), and dm_inf/dV = 3 (t - 1) / (4.2 t^4).
template <typename Real>
struct CaioRates {
  Real hinf, htau;
  __host__ __device__ __forceinline__ explicit CaioRates(Real v) {
    hinf = Real(1) / (Real(1) + aexp((v + Real(85.5)) / Real(8.6)));
    htau = Real(40) + Real(30) * (Real(1) / (Real(1) + aexp((v + Real(84)) / Real(7.3)))) * aexp((v + Real(160)) / Real(30));
  }
};
template <typename Real>
__host__ __device__ __forceinline__ void caio_minf(Real v, Real mid, Real& m, Real& dm) {
  const Real t = Real(1) + aexp((mid - v) / Real(4.2));
  const Real t3 = t * t * t;
  m = Real(1) / t3;
  dm = Real(3) * (t - Real(1)) / (Real(4.2) * t3 * t);
}

// Nav_MA2020_GrC: the Nav1.6 transition graph (the same 13 states and 17 pairs, in
// the pair order of the Nav1.6 tables) with the GrC class's rates: alfa = A_a
// e^(V / 13.99), beta = A_b e^(-V / 13.99), teta = A_t e^(-V / 25), gamma, delta,
// epsilon, Con, Coff, Oon, Ooff constants, all times phi; a = (Oon / Con)^(1/4),
// b = (Ooff / Coff)^(1/4); the C->C rates n1..n4 alfa (back n4..n1 beta).
__device__ __forceinline__ MarkovGraph navgrc_graph() {
  return MarkovGraph{13, 17, 12, kSlotNavGrc, kNav16Src, kNav16Dst};
}
template <typename Real>
__device__ __forceinline__ void navgrc_rates(Real v, Real phi, Real* kf, Real* kb) {
  const Real alfa = phi * Real(353.91) * aexp(v / Real(13.99));
  const Real beta = phi * Real(1.272) * aexp(-v / Real(13.99));
  const Real teta = phi * Real(0.0201) * aexp(-v / Real(25));
  const Real gamma = phi * Real(150), delta = phi * Real(40), eps = phi * Real(1.75);
  const Real con = phi * Real(0.005), coff = phi * Real(0.5), oon = phi * Real(0.75), ooff = phi * Real(0.005);
  const Real a = dpow(oon / con, Real(0.25)), b = dpow(ooff / coff, Real(0.25));
  const Real n[4] = {Real(5.422), Real(3.279), Real(1.83), Real(0.738)};
  // pairs (Nav1.6 order): C1C2 C2C3 C3C4 C4C5 C1I1 I1I2 C2I2 I2I3 C3I3 I3I4 C4I4 I4I5 C5I5 C5O OB I5I6 OI6
  const int cc[4] = {0, 1, 2, 3}, ii[4] = {5, 7, 9, 11}, ci[5] = {4, 6, 8, 10, 12};
  Real ak = Real(1), bk = Real(1);
  for (int k = 0; k < 4; ++k) {
    kf[cc[k]] = n[k] * alfa;
    kb[cc[k]] = n[3 - k] * beta;
    kf[ii[k]] = n[k] * alfa * a;
    kb[ii[k]] = n[3 - k] * beta * b;
  }
  for (int k = 0; k < 5; ++k) {
    kf[ci[k]] = con * ak;
    kb[ci[k]] = coff * bk;
    ak *= a;
    bk *= b;
  }
  kf[13] = gamma;  // C5 -> O
  kb[13] = delta;
  kf[14] = eps;    // O -> OB
  kb[14] = teta;
  kf[15] = gamma;  // I5 -> I6
  kb[15] = delta;
  kf[16] = oon;    // O -> I6
  kb[16] = ooff;
}

// Cav3p1_MA2020_GoC: p^2 q; inf sigmoids, p's tau 1 ms at V <= -90 mV and
// (1 + 1 / (e^((V + 40) / 9) + e^((V + 102) / -18))) / qt above, q's
// (15 + 1 / e^((V + 32) / 7)) / qt.
template <typename Real>
struct Cav31Rates {
  Real pinf, ptau, qinf, qtau;
  __host__ __device__ __forceinline__ Cav31Rates(Real v, Real qt) {
    pinf = Real(1) / (Real(1) + aexp((v + Real(52)) / Real(-5)));
    qinf = Real(1) / (Real(1) + aexp((v + Real(72)) / Real(7)));
    ptau = v <= Real(-90) ? Real(1)
                          : (Real(1) + Real(1) / (aexp((v + Real(40)) / Real(9)) + aexp((v + Real(102)) / Real(-18)))) / qt;
    qtau = (Real(15) + Real(1) / aexp((v + Real(32)) / Real(7))) / qt;
  }
};

// The Cav3.1 GHK drive (calcium.py:78-86, with the model file's F = 9.6485e4 C/mol and
// R = 8.3145 J/(K mol)): z = 2, zeta = z F V / (R T), drive = z F zeta (ci - co e^-zeta)
// / (1 - e^-zeta), and z F (ci - co e^-zeta)(1 + zeta / 2) where |1 - e^-zeta| < 1e-6.
// With a permeability g in cm/s and ci, co in mM, -g drive is in uA/cm^2.  *dd
// receives d drive / dV (per mV), the derivative of the branch taken.
// The constant-field form z F zeta (ci - co e^-zeta) / (1 - e^-zeta) for z = 2 with
// the Faraday and gas constants F, R; `le` takes the small branch at |1 - e^-zeta|
// <= 1e-6 (the shared ghk_flux) rather than < 1e-6 (the Cav3.1 model file's helper).
template <typename Real>
__host__ __device__ __forceinline__ Real ghk_drive2(Real v, Real ci, Real co, Real tghk, double F, double R, bool le,
                                                   Real& dd) {
  const Real zf = Real(2 * F);
  const Real k = zf / (Real(R) * tghk) * Real(1e-3);  // zeta per mV
  const Real z = k * v;
  const Real em = aexp(-z);
  const Real num = ci - co * em;
  const Real den = Real(1) - em;
  const Real ad = den < Real(0) ? -den : den;
  if (le ? ad <= Real(1e-6) : ad < Real(1e-6)) {
    dd = zf * k * (co * em * (Real(1) + z / Real(2)) + num / Real(2));
    return zf * num * (Real(1) + z / Real(2));
  }
  dd = zf * k * ((num + z * co * em) / den - z * num * em / (den * den));
  return zf * z * num / den;
}
template <typename Real>
__host__ __device__ __forceinline__ Real cav31_drive(Real v, Real ci, Real co, Real tghk, Real& dd) {
  return ghk_drive2(v, ci, co, tghk, 9.6485e4, 8.3145, false, dd);
}
// the shared ghk_flux (channel/_base.py:47) with brainunit's CODATA constants
template <typename Real>
__host__ __device__ __forceinline__ Real ghk_codata_drive(Real v, Real ci, Real co, Real temp, Real& dd) {
  return ghk_drive2(v, ci, co, temp, kFaraday, kGasR, true, dd);
}

// Cav2p1_RI2021_SC: m^3 on V - V_sh; m_inf = 1 / (1 + e^(-(V + 29.458) / 8.429)), m_tau
// 0.2702 + 1.1622 e^(-(V + 26.798)^2 / 164.19) at V >= -40 mV, else 0.6923 e^(V / 1089.372).
template <typename Real>
struct Cav21Rates {
  Real minf, mtau;
  __host__ __device__ __forceinline__ Cav21Rates(Real v, Real vsh) {
    const Real x = v - vsh;
    minf = Real(1) / (Real(1) + aexp(-(x + Real(29.458)) / Real(8.429)));
    const Real y = x + Real(26.798);
    mtau = x >= Real(-40) ? Real(0.2702) + Real(1.1622) * aexp(-(y * y) / Real(164.19))
                          : Real(0.6923) * aexp(x / Real(1089.372));
  }
};

// Cav3p3_RI2021_SC: n^2 l on V - V_sh; inf sigmoids, piecewise time constants at -60 mV.
template <typename Real>
struct Cav33Rates {
  Real ninf, ntau, linf, ltau;
  __host__ __device__ __forceinline__ Cav33Rates(Real v, Real vsh) {
    const Real x = v - vsh;
    ninf = Real(1) / (Real(1) + aexp(-(x + Real(41.5)) / Real(6.2)));
    linf = Real(1) / (Real(1) + aexp(-(x + Real(69.8)) / Real(-6.1)));
    ntau = x > Real(-60) ? Real(7.2) + Real(0.02) * aexp(-x / Real(14.7)) : Real(0.875) * aexp((x + Real(120)) / Real(41));
    ltau = x > Real(-60) ? Real(79.5) + Real(2) * aexp(-x / Real(9.3)) : Real(260);
  }
};

// The Cav3.3 GHK drive (calcium.py:89-97, the model file's F = 96520 C/mol and
// R = 8.3134 J/(K mol)): z = 2, w = z F V / (R T), drive = -z F (co - ci e^w) w /
// (e^w - 1), and -z F (co - ci e^w)(1 - w / 2) where |e^w - 1| < 1e-6; *dd receives
// d drive / dV (per mV) of the branch taken.
template <typename Real>
__host__ __device__ __forceinline__ Real cav33_drive(Real v, Real ci, Real co, Real tghk, Real& dd) {
  const Real zf = Real(2 * 96520.0);
  const Real k = zf / (Real(8.3134) * tghk) * Real(1e-3);  // w per mV
  const Real w = k * v;
  const Real ep = aexp(w);
  const Real num = co - ci * ep;
  const Real den = ep - Real(1);
  const Real ad = den < Real(0) ? -den : den;
  if (ad < Real(1e-6)) {
    dd = -zf * k * (-ci * ep * (Real(1) - w / Real(2)) - num / Real(2));
    return -zf * num * (Real(1) - w / Real(2));
  }
  // d/dw [num w / den] = (-ci e^w w + num) / den - num w e^w / den^2
  dd = -zf * k * ((num - ci * ep * w) / den - num * w * ep / (den * den));
  return -zf * num * w / den;
}

// Cav1p2 / Cav1p3_MA2020_GoC: m h n, ohmic in E_Ca; m_inf = 1 / (1 + e^((V - vm) / km)),
// h_inf = VDI / (1 + e^((V - vh) / kh)) + 1 - VDI, n_inf = kf / (kf + Ci) (kf 5e-4 mM),
// m_tau = 1 / (A k / exprel((V + c) / k) + B e^(V / 31.4)) (the reference's
// A (V + c) / (e^((V + c) / k) - 1), finite at V = -c), h_tau 44.3 ms, n_tau 0.5 ms.
struct Cav1Consts {
  double vm, km, vh, kh, vdi, a, c, k, b;
};
// the two classes' constants: Cav1p2 (c12) and Cav1p3
__host__ __device__ __forceinline__ Cav1Consts cav1_consts(bool c12) {
  return c12 ? Cav1Consts{-8.9, -6.7, -55.0, 8.0, 0.17, 39800.0, 8.124, 9.005, 990.0}
             : Cav1Consts{-40.0, -5.0, -37.0, 5.0, 1.0, 39800.0, 67.24, 15.005, 3500.0};
}
template <typename Real>
struct Cav1Rates {
  Real minf, mtau, hinf, ninf;
  __host__ __device__ __forceinline__ Cav1Rates(Real v, Real ci, Cav1Consts q) {
    minf = Real(1) / (Real(1) + aexp((v - Real(q.vm)) / Real(q.km)));
    hinf = Real(q.vdi) / (Real(1) + aexp((v - Real(q.vh)) / Real(q.kh))) + (Real(1) - Real(q.vdi));
    ninf = Real(0.0005) / (Real(0.0005) + ci);
    const Real am = Real(q.a * q.k) / exprel((v + Real(q.c)) / Real(q.k));
    const Real bm = Real(q.b) * aexp(v / Real(31.4));
    mtau = Real(1) / (am + bm);
  }
};
constexpr double kCav1TauH = 44.3;
constexpr double kCav1TauN = 0.5;

// CaHVA_SU2015_DCN: m^3; m_inf = 1 / (1 + e^((V + 34.5) / -9)), m_tau = 1 / (31.746 /
// (e^((V - 5) / -13.89) + 1) + 3.97e-4 (V + 8.9) / (e^((V + 8.9) / 5) - 1)) (qdeltat 1),
// the second term as 3.97e-4 5 / exprel((V + 8.9) / 5).
template <typename Real>
struct CahvadcnRates {
  Real minf, mtau;
  __host__ __device__ __forceinline__ explicit CahvadcnRates(Real v) {
    minf = Real(1) / (Real(1) + aexp((v + Real(34.5)) / Real(-9)));
    const Real act = Real(31.746) / (aexp((v - Real(5)) / Real(-13.89)) + Real(1));
    const Real cor = Real(3.97e-4 * 5.0) / exprel((v + Real(8.9)) / Real(5));
    mtau = Real(1) / (act + cor);
  }
};

// The SU2015 DCN calcium drive (calcium.py:924-1064): A = e^-x, x = 23.20764929 V / T,
// (4.47814e6 V / T)(ci / 1000 - co A / 1000) / (1 - A) in mA/cm^2 per cm/s, i.e.
// c S(x)(ci - co A) uA/cm^2 per cm/s with c = 4.47814e6 / 23.20764929 and S(x) = x / (1 -
// e^-x) (the reference's expression, finite at V = 0).  *dd receives its V-derivative.
template <typename Real>
__host__ __device__ __forceinline__ Real su2015_drive(Real v, Real ci, Real co, Real temp, Real& dd) {
  const Real c = Real(4.47814e6 / 23.20764929);
  const Real kx = Real(23.20764929) / temp;  // x per mV
  const Real x = kx * v;
  const Real a = aexp(-x);
  const Real sx = x_over_1mexp(x);
  const Real ax = x < Real(0) ? -x : x;
  // S'(x) = (1 - e^-x - x e^-x) / (1 - e^-x)^2, 1/2 + x/6 near 0
  const Real den = Real(1) - a;
  const Real ds = ax < Real(1e-4) ? Real(0.5) + x / Real(6) : (den - x * a) / (den * den);
  const Real num = ci - co * a;
  dd = c * kx * (ds * num + sx * co * a);
  return c * sx * num;
}

// The region's BC_X_* bits: two record reals, each an integer below 2^24 (exact in FP32).
template <typename Real>
__host__ __device__ __forceinline__ uint32_t ext_mask(const Real* P) {
  return uint32_t(P[BC_P_EXT_MASK]) | (uint32_t(P[BC_P_EXT_MASK_HI]) << 24);
}

// One extension channel's current at v with the node's stored gates (0 where the
// region does not carry it); *gv receives -dI/dV when not null.
template <typename Real>
__device__ __forceinline__ Real ext_current(const Real* st, int N, const Real* P, uint32_t x, Real v, Real ci,
                                            Real eca, int code, Real* gv) {
  Real g = Real(0), e = Real(0), gd = Real(0);
  bool has = false;
  switch (code) {
    case BC_CUR_HCN2:
      if ((has = (x & BC_X_HCN2) != 0)) {
        g = P[BC_P_HCN2_G] * (st[kSlotHcn2F * N] + st[kSlotHcn2S * N]);
        e = P[BC_P_HCN2_E];
      }
      break;
    case BC_CUR_KV33:
      if ((has = (x & BC_X_KV33) != 0)) {
        const Real n2 = st[kSlotKv33N * N] * st[kSlotKv33N * N];
        g = P[BC_P_KV33_G] * n2 * n2;
        e = P[BC_P_EK];
      }
      break;
    case BC_CUR_KV22:
      if ((has = (x & BC_X_KV22) != 0)) {
        g = P[BC_P_KV22_G] * st[kSlotKv22M * N] * st[kSlotKv22H * N];
        e = P[BC_P_EK];
      }
      break;
    case BC_CUR_KV15:
      if ((has = (x & BC_X_KV15) != 0)) {
        const Real m = st[kSlotKv15M * N];
        const Real gg = P[BC_P_KV15_G] * m * m * m * st[kSlotKv15N * N] * st[kSlotKv15U * N];
        Real f, df;
        kv15_vfactor(v, f, df);
        e = P[BC_P_EK];
        g = gg * f;
        // I = gg f (E - V): -dI/dV = gg (f - f' (E - V))
        gd = gg * (f - df * (e - v));
      }
      break;
    case BC_CUR_NAF:
      if ((has = (x & BC_X_NAF) != 0)) {
        const Real m = st[kSlotNafM * N];
        g = P[BC_P_NAF_G] * m * m * m * st[kSlotNafH * N];
        e = P[BC_P_ENA];
      }
      break;
    case BC_CUR_NAP:
      if ((has = (x & BC_X_NAP) != 0)) {
        const Real m = st[kSlotNapM * N];
        g = P[BC_P_NAP_G] * m * m * m * st[kSlotNapH * N];
        e = P[BC_P_ENA];
      }
      break;
    case BC_CUR_NAIO:
      if ((has = (x & BC_X_NAIO) != 0)) {
        const Real m = st[kSlotNaioM * N];
        g = P[BC_P_NAIO_G] * m * m * m * st[kSlotNaioH * N];
        e = P[BC_P_ENA];
      }
      break;
    case BC_CUR_FKDR:
      if ((has = (x & BC_X_FKDR) != 0)) {
        const Real m2 = st[kSlotFkdrM * N] * st[kSlotFkdrM * N];
        g = P[BC_P_FKDR_G] * m2 * m2;
        e = P[BC_P_EK];
      }
      break;
    case BC_CUR_SKDR:
      if ((has = (x & BC_X_SKDR) != 0)) {
        const Real m2 = st[kSlotSkdrM * N] * st[kSlotSkdrM * N];
        g = P[BC_P_SKDR_G] * m2 * m2;
        e = P[BC_P_EK];
      }
      break;
    case BC_CUR_KDRIO:
      if ((has = (x & BC_X_KDRIO) != 0)) {
        const Real n2 = st[kSlotKdrioN * N] * st[kSlotKdrioN * N];
        g = P[BC_P_KDRIO_G] * n2 * n2;
        e = P[BC_P_EK];
      }
      break;
    case BC_CUR_HCNDCN:
      if ((has = (x & BC_X_HCNDCN) != 0)) {
        const Real m = st[kSlotHcndcnM * N];
        g = P[BC_P_HCNDCN_G] * m * m;
        e = P[BC_P_HCNDCN_E];
      }
      break;
    case BC_CUR_HCNIO:
      if ((has = (x & BC_X_HCNIO) != 0)) {
        g = P[BC_P_HCNIO_G] * st[kSlotHcnioQ * N];
        e = P[BC_P_HCNIO_E];
      }
      break;
    case BC_CUR_CATHP:
      if ((has = (x & BC_X_CATHP) != 0)) {
        const Real p = st[kSlotCathpP * N];
        g = P[BC_P_CATHP_G] * p * p * st[kSlotCathpQ * N];
        e = eca;
      }
      break;
    case BC_CUR_CAHTRE:
      if ((has = (x & BC_X_CAHTRE) != 0)) {
        const Real p = st[kSlotCahtreP * N];
        g = P[BC_P_CAHTRE_G] * p * p * st[kSlotCahtreQ * N];
        e = eca;
      }
      break;
    case BC_CUR_CALDCN:
      if ((has = (x & BC_X_CALDCN) != 0)) {
        const Real m = st[kSlotCaldcnM * N];
        g = P[BC_P_CALDCN_G] * m * m * st[kSlotCaldcnH * N];
        e = P[BC_P_CALDCN_E];
      }
      break;
    case BC_CUR_KCA31:
      if ((has = (x & BC_X_KCA31) != 0)) {
        g = P[BC_P_KCA31_G] * st[kSlotKca31P * N];
        e = P[BC_P_EK];
      }
      break;
    case BC_CUR_SKDCN:
      if ((has = (x & BC_X_SKDCN) != 0)) {
        g = P[BC_P_SKDCN_G] * st[kSlotSkdcnZ * N];
        e = P[BC_P_EK];
      }
      break;
    case BC_CUR_KKV:
      if ((has = (x & BC_X_KKV) != 0)) {
        g = P[BC_P_KKV_G] * st[kSlotKkvN * N];
        e = P[BC_P_EK];
      }
      break;
    case BC_CUR_CAN:
      if ((has = (x & BC_X_CAN) != 0)) {
        g = P[BC_P_CAN_G] * (ci / (ci + Real(0.2))) * st[kSlotCanP * N];
        e = P[BC_P_CAN_E];
      }
      break;
    case BC_CUR_NAVGRC:
      if ((has = (x & BC_X_NAVGRC) != 0)) {
        g = P[BC_P_NAVGRC_G] * st[(kSlotNavGrc + 10) * N];  // O
        e = P[BC_P_ENA];
      }
      break;
    case BC_CUR_CAV31:
      if ((has = (x & BC_X_CAV31) != 0)) {
        const Real p = st[kSlotCav31P * N];
        const Real gp = P[BC_P_CAV31_G] * p * p * st[kSlotCav31Q * N];
        // Cav3p1Test_PC24 (calcium.py:2577): the same gates with a fixed 1 mV drive
        if (P[BC_P_CAV31_FREEZE] == Real(2)) {
          if (gv) *gv = Real(0);
          return -gp;
        }
        Real dd;
        const Real drive = cav31_drive(v, ci, P[BC_P_CA_CO], P[BC_P_CAV31_TGHK], dd);
        // I = -g p^2 q drive: -dI/dV = g p^2 q d drive / dV, 0 with the drive frozen
        if (gv) *gv = P[BC_P_CAV31_FREEZE] != Real(0) ? Real(0) : gp * dd;
        return -gp * drive;
      }
      return Real(0);
    case BC_CUR_CAV33:
      if ((has = (x & BC_X_CAV33) != 0)) {
        const Real n = st[kSlotCav33N * N];
        const Real gp = P[BC_P_CAV33_G] * n * n * st[kSlotCav33L * N];
        Real dd;
        const Real drive = cav33_drive(v - P[BC_P_CAV33_VSH], ci, P[BC_P_CA_CO], P[BC_P_CAV33_TGHK], dd);
        if (gv) *gv = P[BC_P_CAV33_FREEZE] != Real(0) ? Real(0) : gp * dd;
        return -gp * drive;
      }
      return Real(0);
    case BC_CUR_CAV12:
    case BC_CUR_CAV13: {
      const bool c12 = code == BC_CUR_CAV12;
      if ((has = (x & (c12 ? BC_X_CAV12 : BC_X_CAV13)) != 0)) {
        const int s0 = c12 ? kSlotCav12 : kSlotCav13;
        g = P[c12 ? BC_P_CAV12_G : BC_P_CAV13_G] * st[s0 * N] * st[(s0 + 1) * N] * st[(s0 + 2) * N];
        e = eca;
      }
      break;
    }
    case BC_CUR_CAV21:
      if ((has = (x & BC_X_CAV21) != 0)) {
        const Real m = st[kSlotCav21M * N];
        const Real gp = P[BC_P_CAV21_G] * m * m * m;
        Real dd;
        // the _Frozen classes: the Cav3.1 model-file GHK at a stop-gradient V (row conductance 0)
        const bool frozen = P[BC_P_CAV21_FROZEN] != Real(0);
        const Real vs = v - P[BC_P_CAV21_VSH];
        const Real drive = frozen ? cav31_drive(vs, ci, P[BC_P_CA_CO], P[BC_P_CAV21_TGHK], dd)
                                  : ghk_codata_drive(vs, ci, P[BC_P_CA_CO], P[BC_P_CAV21_TGHK], dd);
        if (gv) *gv = frozen ? Real(0) : gp * dd;
        return -gp * drive;
      }
      return Real(0);
    case BC_CUR_CAHVADCN:
    case BC_CUR_CALVADCN: {
      const bool hva = code == BC_CUR_CAHVADCN;
      if ((has = (x & (hva ? BC_X_CAHVADCN : BC_X_CALVADCN)) != 0)) {
        Real gates;
        if (hva) {
          const Real m = st[kSlotCahvadcnM * N];
          gates = m * m * m;
        } else {
          const Real m = st[kSlotCalvadcnM * N];
          gates = m * m * st[kSlotCalvadcnH * N];
        }
        const Real gp = P[hva ? BC_P_CAHVADCN_G : BC_P_CALVADCN_G] * gates;
        Real dd;
        const Real drive = su2015_drive(v, ci, P[BC_P_CA_CO], P[hva ? BC_P_CAHVADCN_T : BC_P_CALVADCN_T], dd);
        if (gv) *gv = gp * dd;
        return -gp * drive;
      }
      return Real(0);
    }
    case BC_CUR_CAIO:
      if ((has = (x & BC_X_CAIO) != 0)) {
        Real m, dm;
        caio_minf(v, P[BC_P_CAIO_MID], m, dm);
        const Real gh = P[BC_P_CAIO_G] * st[kSlotCaioH * N];
        e = P[BC_P_CAIO_E];
        g = gh * m;
        // a frozen m_inf stays out of the linearisation, as the reference's stop_gradient does
        gd = P[BC_P_CAIO_FREEZE] != Real(0) ? g : gh * (m - dm * (e - v));
      }
      break;
  }
  if (!has) return Real(0);
  if (gv) *gv = (code == BC_CUR_KV15 || code == BC_CUR_CAIO) ? gd : g;
  return g * (e - v);
}

// Gate update of one node's extension channels at v (exp-Euler, as the others).
template <typename Real>
__device__ __forceinline__ void ext_gates(Real* st, int N, const Real* P, uint32_t x, Real v, Real ci, Real dt) {
  if (x & BC_X_HCN2) {
    const Hcn2Rates<Real> r(v);
    const Real phi = P[BC_P_HCN2_PHI];
    st[kSlotHcn2F * N] = gate_it(st[kSlotHcn2F * N], r.finf, r.ftau, phi, dt);
    st[kSlotHcn2S * N] = gate_it(st[kSlotHcn2S * N], r.sinf, r.stau, phi, dt);
  }
  if (x & BC_X_KV33) {
    const Kv33Rates<Real> r(v);
    st[kSlotKv33N * N] = gate_ab<Real, true>(st[kSlotKv33N * N], r.a, r.b, P[BC_P_KV33_PHI], dt);
  }
  if (x & BC_X_KV22) {
    const Kv22Rates<Real> r(v);
    st[kSlotKv22M * N] = gate_it(st[kSlotKv22M * N], r.minf, r.mtau, Real(1), dt);
    st[kSlotKv22H * N] = gate_it(st[kSlotKv22H * N], r.hinf, r.htau, Real(1), dt);
  }
  if (x & BC_X_KV15) {
    const Kv15Rates<Real> r(v, P[BC_P_KV15_Q10], P[BC_P_KV15_TACT], P[BC_P_KV15_TINF]);
    st[kSlotKv15M * N] = gate_it(st[kSlotKv15M * N], r.minf, r.mtau, Real(1), dt);
    st[kSlotKv15N * N] = gate_it(st[kSlotKv15N * N], r.ninf, r.ntau, Real(1), dt);
    st[kSlotKv15U * N] = gate_it(st[kSlotKv15U * N], r.uinf, Real(kKv15TauU) * P[BC_P_KV15_TINS], Real(1), dt);
  }
  if (x & BC_X_NAF) {
    const NafRates<Real> r(v);
    st[kSlotNafM * N] = gate_it(st[kSlotNafM * N], r.minf, r.mtau, Real(1), dt);
    st[kSlotNafH * N] = gate_it(st[kSlotNafH * N], r.hinf, r.htau, Real(1), dt);
  }
  if (x & BC_X_NAP) {
    const NapRates<Real> r(v);
    st[kSlotNapM * N] = gate_it(st[kSlotNapM * N], r.minf, r.mtau, Real(1), dt);
    st[kSlotNapH * N] = gate_it(st[kSlotNapH * N], r.hinf, r.htau, Real(1), dt);
  }
  if (x & BC_X_NAIO) {
    const NaioRates<Real> r(v);
    st[kSlotNaioM * N] = gate_it(st[kSlotNaioM * N], r.minf, r.mtau, Real(1), dt);
    st[kSlotNaioH * N] = gate_it(st[kSlotNaioH * N], r.hinf, r.htau, Real(1), dt);
  }
  if (x & BC_X_FKDR) {
    const Su2015KdrRates<Real> r = fkdr_rates(v);
    st[kSlotFkdrM * N] = gate_it(st[kSlotFkdrM * N], r.minf, r.mtau, Real(1), dt);
  }
  if (x & BC_X_SKDR) {
    const Su2015KdrRates<Real> r = skdr_rates(v);
    st[kSlotSkdrM * N] = gate_it(st[kSlotSkdrM * N], r.minf, r.mtau, Real(1), dt);
  }
  if (x & BC_X_KDRIO) {
    const KdrioRates<Real> r(v);
    st[kSlotKdrioN * N] = gate_it(st[kSlotKdrioN * N], r.ninf, r.ntau, Real(1), dt);
  }
  if (x & BC_X_HCNDCN) {
    const HcndcnRates<Real> r(v);
    st[kSlotHcndcnM * N] = gate_it(st[kSlotHcndcnM * N], r.minf, r.mtau, Real(1), dt);
  }
  if (x & BC_X_HCNIO) {
    const HcnioRates<Real> r(v);
    st[kSlotHcnioQ * N] = gate_it(st[kSlotHcnioQ * N], r.qinf, r.qtau, Real(1), dt);
  }
  if (x & BC_X_CATHP) {
    const CathpRates<Real> r(v, P[BC_P_CATHP_VSH]);
    st[kSlotCathpP * N] = gate_it(st[kSlotCathpP * N], r.pinf, r.ptau, P[BC_P_CATHP_PHIP], dt);
    st[kSlotCathpQ * N] = gate_it(st[kSlotCathpQ * N], r.qinf, r.qtau, P[BC_P_CATHP_PHIQ], dt);
  }
  if (x & BC_X_CAHTRE) {
    const CahtreRates<Real> r(v, P[BC_P_CAHTRE_VSH]);
    st[kSlotCahtreP * N] = gate_ab<Real, true>(st[kSlotCahtreP * N], r.ap, r.bp, P[BC_P_CAHTRE_PHIP], dt);
    st[kSlotCahtreQ * N] = gate_ab<Real, true>(st[kSlotCahtreQ * N], r.aq, r.bq, P[BC_P_CAHTRE_PHIQ], dt);
  }
  if (x & BC_X_CALDCN) {
    const CaldcnRates<Real> r(v);
    st[kSlotCaldcnM * N] = gate_it(st[kSlotCaldcnM * N], r.minf, r.mtau, Real(1), dt);
    st[kSlotCaldcnH * N] = gate_it(st[kSlotCaldcnH * N], r.hinf, r.htau, Real(1), dt);
  }
  if (x & BC_X_KCA31) {
    const Kca31Rates<Real> r(v, ci);
    st[kSlotKca31P * N] = gate_ab<Real, true>(st[kSlotKca31P * N], r.a, r.b, Real(1), dt);
  }
  if (x & BC_X_SKDCN) {
    const SkdcnRates<Real> r(ci);
    st[kSlotSkdcnZ * N] = gate_it(st[kSlotSkdcnZ * N], r.zinf, r.ztau, Real(1), dt);
  }
  if (x & BC_X_KKV) {
    const KkvRates<Real> r(v, P[BC_P_KKV_VSH], P[BC_P_KKV_RA], P[BC_P_KKV_RB], P[BC_P_KKV_Q], P[BC_P_KKV_V12]);
    st[kSlotKkvN * N] = gate_it(st[kSlotKkvN * N], r.ninf, r.ntau, Real(1), dt);
  }
  if (x & BC_X_CAN) {
    const CanRates<Real> r(v);
    st[kSlotCanP * N] = gate_it(st[kSlotCanP * N], r.pinf, r.ptau, P[BC_P_CAN_PHI], dt);
  }
  if (x & BC_X_CAIO) {
    const CaioRates<Real> r(v);
    st[kSlotCaioH * N] = gate_it(st[kSlotCaioH * N], r.hinf, r.htau, Real(1), dt);
  }
  if (x & BC_X_CAV31) {
    const Cav31Rates<Real> r(v, P[BC_P_CAV31_QT]);
    st[kSlotCav31P * N] = gate_it(st[kSlotCav31P * N], r.pinf, r.ptau, Real(1), dt);
    st[kSlotCav31Q * N] = gate_it(st[kSlotCav31Q * N], r.qinf, r.qtau, Real(1), dt);
  }
  if (x & BC_X_CAV33) {
    const Cav33Rates<Real> r(v, P[BC_P_CAV33_VSH]);
    const Real phi = P[BC_P_CAV33_PHI];
    st[kSlotCav33N * N] = gate_it(st[kSlotCav33N * N], r.ninf, r.ntau, phi, dt);
    st[kSlotCav33L * N] = gate_it(st[kSlotCav33L * N], r.linf, r.ltau, phi, dt);
  }
  for (int c = 0; c < 2; ++c) {
    if (!(x & (c == 0 ? BC_X_CAV12 : BC_X_CAV13))) continue;
    const int s0 = c == 0 ? kSlotCav12 : kSlotCav13;
    const Real phi = P[c == 0 ? BC_P_CAV12_PHI : BC_P_CAV13_PHI];
    const Cav1Rates<Real> r(v, ci, cav1_consts(c == 0));
    st[s0 * N] = gate_it(st[s0 * N], r.minf, r.mtau, phi, dt);
    st[(s0 + 1) * N] = gate_it(st[(s0 + 1) * N], r.hinf, Real(kCav1TauH), phi, dt);
    st[(s0 + 2) * N] = gate_it(st[(s0 + 2) * N], r.ninf, Real(kCav1TauN), phi, dt);
  }
  if (x & BC_X_CAV21) {
    const Cav21Rates<Real> r(v, P[BC_P_CAV21_VSH]);
    st[kSlotCav21M * N] = gate_it(st[kSlotCav21M * N], r.minf, r.mtau, P[BC_P_CAV21_PHI], dt);
  }
  if (x & BC_X_CAHVADCN) {
    const CahvadcnRates<Real> r(v);
    st[kSlotCahvadcnM * N] = gate_it(st[kSlotCahvadcnM * N], r.minf, r.mtau, Real(1), dt);
  }
  if (x & BC_X_CALVADCN) {
    const CaldcnRates<Real> r(v);
    st[kSlotCalvadcnM * N] = gate_it(st[kSlotCalvadcnM * N], r.minf, r.mtau, Real(1), dt);
    st[kSlotCalvadcnH * N] = gate_it(st[kSlotCalvadcnH * N], r.hinf, r.htau, Real(1), dt);
  }
  // the Markov scheme after the gates, by one linearised backward-Euler step
  if (x & BC_X_NAVGRC) {
    Real kf[17], kb[17];
    navgrc_rates(v, P[BC_P_NAVGRC_PHI], kf, kb);
    markov_advance(st, N, navgrc_graph(), kf, kb, dt);
  }
}

// A node's extension channels: gates at v (when advancing), then their G and I.
// ci and eca: Ci and E_Ca after this step's shell update (the calcium-gated and
// the calcium channels).
template <typename Real>
__device__ __noinline__ void ext_channels(Real* st, int N, const Real* P, Real v, Real ci, Real eca, Real dt,
                                          bool advance, Real& G, Real& I) {
  const uint32_t x = ext_mask(P);
  if (advance) ext_gates(st, N, P, x, v, ci, dt);
  for (int code = BC_CUR_HCN2; code <= BC_CUR_CALVADCN; ++code) {
    Real g = Real(0);
    const Real i = ext_current(st, N, P, x, v, ci, eca, code, &g);
    G += g;
    I += i;
  }
}

// The calcium current of the extension channels that carry calcium, at the
// step-start gates, v, Ci and E_Ca (their share of the calcium shell's drive).
template <typename Real>
__device__ __noinline__ Real ext_ca_current(const Real* st, int N, const Real* P, Real v, Real ci, Real eca) {
  const uint32_t x = ext_mask(P);
  return ext_current(st, N, P, x, v, ci, eca, BC_CUR_CATHP, (Real*)nullptr) +
         ext_current(st, N, P, x, v, ci, eca, BC_CUR_CAHTRE, (Real*)nullptr) +
         ext_current(st, N, P, x, v, ci, eca, BC_CUR_CAN, (Real*)nullptr) +
         ext_current(st, N, P, x, v, ci, eca, BC_CUR_CAV31, (Real*)nullptr) +
         ext_current(st, N, P, x, v, ci, eca, BC_CUR_CAV33, (Real*)nullptr) +
         ext_current(st, N, P, x, v, ci, eca, BC_CUR_CAV12, (Real*)nullptr) +
         ext_current(st, N, P, x, v, ci, eca, BC_CUR_CAV13, (Real*)nullptr) +
         ext_current(st, N, P, x, v, ci, eca, BC_CUR_CAV21, (Real*)nullptr) +
         ext_current(st, N, P, x, v, ci, eca, BC_CUR_CAHVADCN, (Real*)nullptr) +
         ext_current(st, N, P, x, v, ci, eca, BC_CUR_CALVADCN, (Real*)nullptr);
}

// Steady states of the extension channels' gates at v (HH.reset_state).
template <typename Real>
__device__ __forceinline__ void ext_steady(const Real* P, Real* st, int N, Real v) {
  const uint32_t x = ext_mask(P);
  if (x & BC_X_HCN2) {
    const Hcn2Rates<Real> r(v);
    st[kSlotHcn2F * N] = r.finf;
    st[kSlotHcn2S * N] = r.sinf;
  }
  if (x & BC_X_KV33) {
    const Kv33Rates<Real> r(v);
    st[kSlotKv33N * N] = r.a / (r.a + r.b);
  }
  if (x & BC_X_KV22) {
    const Kv22Rates<Real> r(v);
    st[kSlotKv22M * N] = r.minf;
    st[kSlotKv22H * N] = r.hinf;
  }
  if (x & BC_X_KV15) {
    const Kv15Rates<Real> r(v, P[BC_P_KV15_Q10], P[BC_P_KV15_TACT], P[BC_P_KV15_TINF]);
    st[kSlotKv15M * N] = r.minf;
    st[kSlotKv15N * N] = r.ninf;
    st[kSlotKv15U * N] = r.uinf;
  }
  if (x & BC_X_NAF) {
    const NafRates<Real> r(v);
    st[kSlotNafM * N] = r.minf;
    st[kSlotNafH * N] = r.hinf;
  }
  if (x & BC_X_NAP) {
    const NapRates<Real> r(v);
    st[kSlotNapM * N] = r.minf;
    st[kSlotNapH * N] = r.hinf;
  }
  if (x & BC_X_NAIO) {
    const NaioRates<Real> r(v);
    st[kSlotNaioM * N] = r.minf;
    st[kSlotNaioH * N] = r.hinf;
  }
  if (x & BC_X_FKDR) st[kSlotFkdrM * N] = fkdr_rates(v).minf;
  if (x & BC_X_SKDR) st[kSlotSkdrM * N] = skdr_rates(v).minf;
  if (x & BC_X_KDRIO) st[kSlotKdrioN * N] = KdrioRates<Real>(v).ninf;
  if (x & BC_X_HCNDCN) st[kSlotHcndcnM * N] = HcndcnRates<Real>(v).minf;
  if (x & BC_X_HCNIO) st[kSlotHcnioQ * N] = HcnioRates<Real>(v).qinf;
  if (x & BC_X_CATHP) {
    const CathpRates<Real> r(v, P[BC_P_CATHP_VSH]);
    st[kSlotCathpP * N] = r.pinf;
    st[kSlotCathpQ * N] = r.qinf;
  }
  if (x & BC_X_CAHTRE) {
    const CahtreRates<Real> r(v, P[BC_P_CAHTRE_VSH]);
    st[kSlotCahtreP * N] = r.ap / (r.ap + r.bp);
    st[kSlotCahtreQ * N] = r.aq / (r.aq + r.bq);
  }
  if (x & BC_X_CALDCN) {
    const CaldcnRates<Real> r(v);
    st[kSlotCaldcnM * N] = r.minf;
    st[kSlotCaldcnH * N] = r.hinf;
  }
  // the calcium-gated channels at the reset Ci
  if (x & BC_X_KCA31) {
    const Kca31Rates<Real> r(v, P[BC_P_CA_CI0]);
    st[kSlotKca31P * N] = r.a / (r.a + r.b);
  }
  if (x & BC_X_SKDCN) st[kSlotSkdcnZ * N] = SkdcnRates<Real>(P[BC_P_CA_CI0]).zinf;
  if (x & BC_X_KKV)
    st[kSlotKkvN * N] =
        KkvRates<Real>(v, P[BC_P_KKV_VSH], P[BC_P_KKV_RA], P[BC_P_KKV_RB], P[BC_P_KKV_Q], P[BC_P_KKV_V12]).ninf;
  if (x & BC_X_CAN) st[kSlotCanP * N] = CanRates<Real>(v).pinf;
  if (x & BC_X_CAIO) st[kSlotCaioH * N] = CaioRates<Real>(v).hinf;
  if (x & BC_X_CAV31) {
    const Cav31Rates<Real> r(v, P[BC_P_CAV31_QT]);
    st[kSlotCav31P * N] = r.pinf;
    st[kSlotCav31Q * N] = r.qinf;
  }
  if (x & BC_X_CAV33) {
    const Cav33Rates<Real> r(v, P[BC_P_CAV33_VSH]);
    st[kSlotCav33N * N] = r.ninf;
    st[kSlotCav33L * N] = r.linf;
  }
  for (int c = 0; c < 2; ++c) {  // at the reset Ci
    if (!(x & (c == 0 ? BC_X_CAV12 : BC_X_CAV13))) continue;
    const int s0 = c == 0 ? kSlotCav12 : kSlotCav13;
    const Cav1Rates<Real> r(v, P[BC_P_CA_CI0], cav1_consts(c == 0));
    st[s0 * N] = r.minf;
    st[(s0 + 1) * N] = r.hinf;
    st[(s0 + 2) * N] = r.ninf;
  }
  if (x & BC_X_CAV21) st[kSlotCav21M * N] = Cav21Rates<Real>(v, P[BC_P_CAV21_VSH]).minf;
  if (x & BC_X_CAHVADCN) st[kSlotCahvadcnM * N] = CahvadcnRates<Real>(v).minf;
  if (x & BC_X_CALVADCN) {
    const CaldcnRates<Real> r(v);
    st[kSlotCalvadcnM * N] = r.minf;
    st[kSlotCalvadcnH * N] = r.hinf;
  }
  if (x & BC_X_NAVGRC) {  // the stationary distribution (reset_steady_state)
    Real kf[17], kb[17];
    navgrc_rates(v, P[BC_P_NAVGRC_PHI], kf, kb);
    markov_steady(st, N, navgrc_graph(), kf, kb);
  }
}

}  // namespace bc
