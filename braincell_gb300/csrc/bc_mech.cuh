// Per-compartment mechanism arithmetic (device).  Rate functions and state
// equations are the reference's:
//   HH template      channel/_base.py:575-588 (alpha/beta or inf/tau derivative),
//                    :550-558 (gate product), :658-674 (ohmic current)
//   exp-Euler        quad/_exp_euler.py:461-465  y += dt * exprel(dt * lambda) * f
//   Na_Ba2002        channel/sodium.py:154-170
//   KDR_Ba2002       channel/potassium.py:206-214
//   CaL_IS2008       channel/calcium.py:(CaL f_p_inf .. f_q_tau)
//   CaT_HM1992       channel/calcium.py:(CaT f_p_inf .. f_q_tau)
//   HCN_HM1992       channel/hyperpolarization_activated.py:126-133
//   AHP_De1994       channel/potassium_calcium.py:181-186
//   Na_HH1952        channel/sodium.py:384-399
//   K_HH1952         channel/potassium.py:450-456
//   KM_RI2021_SC     channel/potassium.py:1735-1748
//   KA1_HM1992       channel/potassium.py:592-611, KA2_HM1992 :743-762
//   KK2A_HM1992      channel/potassium.py:881-895, KK2B_HM1992 :1023-1041
//   KNI_Ya1989       channel/potassium.py:1156-1163
//   CalciumDetailed  ion/calcium.py:499-505, Nernst E: ion/_base.py:463-469
//   Markov channels  channel/_base.py:677-1125 (template), quad/_backward_euler.py:31-64;
//                    Nav1p6_MA2020_GoC sodium.py:727-940, Kca2p2_MA2020_GoC
//                    potassium_calcium.py:613-790, Kca1p1_MA2020_GoC :1107-1353
// CUDA's own exp / expm1 / log are called; nothing of the math library is
// re-implemented here.
#pragma once

#include <cstdint>

#include "../../include/braincell_gb300.h"

namespace bc {

// Accurate functions (both precisions): used where FP32 rounding matters
// (exp-Euler decay factors, exprel near its removable singularity, Nernst log).
__device__ __forceinline__ float dexpm1(float x) { return expm1f(x); }
__host__ __device__ __forceinline__ double dexpm1(double x) { return expm1(x); }
__device__ __forceinline__ float dlog(float x) { return logf(x); }
__host__ __device__ __forceinline__ double dlog(double x) { return log(x); }
__device__ __forceinline__ float dpow(float x, float y) { return powf(x, y); }
__host__ __device__ __forceinline__ double dpow(double x, double y) { return pow(x, y); }
// The FP64 forms and the rate structures are also host functions, so that a host
// build of this header can check the FP64 rates against the oracle on a CPU; the
// FP32 forms stay device-only.
// Rate-function arithmetic: FP32 uses the hardware approximations (__expf, and
// a * rcp.approx(b) for a / b: a few ulp, far below what the rates need); FP64
// stays exact so the FP64 build remains an oracle-grade run of the same kernels.
__device__ __forceinline__ float rexp(float x) { return __expf(x); }
__device__ __forceinline__ float aexp(float x) { return expf(x); }
__host__ __device__ __forceinline__ double aexp(double x) { return exp(x); }
__host__ __device__ __forceinline__ double rexp(double x) { return exp(x); }
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rdiv(float a, float b) { return a * rcp_approx(b); }
__host__ __device__ __forceinline__ double rdiv(double a, double b) { return a / b; }

// e^x - 1 for the exp-Euler decay of a gate (x = dt * lambda <= 0).  FP32: for
// |x| < 1/4 the Taylor series of e^x - 1 to x^6 (truncation < 5e-8 relative, the
// float rounding level); otherwise __expf(x) - 1, which has no cancellation there.
// FP64: expm1.
__device__ __forceinline__ float decay_em1(float x) {
  const float p = x * (1.0f + x * (0.5f + x * (1.0f / 6.0f + x * (1.0f / 24.0f + x * (1.0f / 120.0f + x * (1.0f / 720.0f))))));
  return fabsf(x) < 0.25f ? p : __expf(x) - 1.0f;
}
__host__ __device__ __forceinline__ double decay_em1(double x) { return expm1(x); }

// exprel(x) = (e^x - 1) / x, exprel(0) = 1
template <typename Real>
__host__ __device__ __forceinline__ Real exprel(Real x) {
  return x == Real(0) ? Real(1) : dexpm1(x) / x;
}

// One exp-Euler step y += dt * exprel(dt * lam) * f of a gate whose right-hand
// side is affine in the gate: with lam = -phi (a + b) and f = -lam (x_inf - x) the
// step is x - expm1(dt * lam) * (x_inf - x).  kExact selects IEEE division and
// expm1 (the spike-generating Na / K gates) over the fast forms.
template <typename Real, bool kExact = false>
__device__ __forceinline__ Real gate_ab(Real x, Real a, Real b, Real phi, Real dt) {
  const Real s = a + b;
  if (kExact) return x - dexpm1(-dt * phi * s) * (a / s - x);
  const Real xinf = rdiv(a, s);
  return x - decay_em1(-dt * phi * s) * (xinf - x);
}

// Same step for a gate in inf/tau form: lam = -phi / tau, f = phi (inf - x) / tau.
template <typename Real>
__device__ __forceinline__ Real gate_it(Real x, Real inf, Real tau, Real phi, Real dt) {
  return x - decay_em1(-rdiv(dt * phi, tau)) * (inf - x);
}

template <typename Real>
struct NaRates {
  Real ap, bp, aq, bq;
  __host__ __device__ __forceinline__ NaRates(Real v, Real vsh) {
    const Real vp = v - vsh;
    ap = Real(0.32 * 4.0) / exprel(-(vp - Real(13)) * Real(1.0 / 4));
    bp = Real(0.28 * 5.0) / exprel((vp - Real(40)) * Real(1.0 / 5));
    aq = Real(0.128) * aexp(-(vp - Real(17)) * Real(1.0 / 18));
    bq = Real(4) / (Real(1) + aexp(-(vp - Real(40)) * Real(1.0 / 5)));
  }
};

template <typename Real>
struct KdrRates {
  Real a, b;
  __host__ __device__ __forceinline__ KdrRates(Real v, Real vsh) {
    const Real vp = v - vsh;
    a = Real(0.032 * 5.0) / exprel(-(vp - Real(15)) * Real(1.0 / 5));
    b = Real(0.5) * aexp(-(vp - Real(10)) * Real(1.0 / 40));
  }
};

// 1 / (e^-y + e^y) = z / (1 + z^2) with z = e^y
template <typename Real>
__host__ __device__ __forceinline__ Real inv_cosh2(Real y) {
  const Real z = rexp(y);
  return rdiv(z, Real(1) + z * z);
}

template <typename Real>
struct CaLRates {
  Real pinf, ptau, qinf, qtau;
  __host__ __device__ __forceinline__ CaLRates(Real v, Real vsh) {
    const Real vs = v - vsh;
    pinf = rdiv(Real(1), Real(1) + rexp(-(vs + Real(10)) * Real(1.0 / 4)));
    ptau = Real(0.4) + Real(0.7) * inv_cosh2((vs + Real(5)) * Real(1.0 / 15));
    qinf = rdiv(Real(1), Real(1) + rexp((vs + Real(25)) * Real(1.0 / 2)));
    qtau = Real(300) + Real(100) * inv_cosh2((vs + Real(40)) * Real(1.0 / 9.5));
  }
};

template <typename Real>
struct CaTRates {
  Real pinf, ptau, qinf, qtau;
  __host__ __device__ __forceinline__ CaTRates(Real v, Real vsh) {
    const Real vs = v - vsh;
    pinf = rdiv(Real(1), Real(1) + rexp(-(vs + Real(59)) * Real(1.0 / 6.2)));
    ptau = rdiv(Real(1), rexp(-(vs + Real(132)) * Real(1.0 / 16.7)) + rexp((vs + Real(16.8)) * Real(1.0 / 18.2))) + Real(0.612);
    qinf = rdiv(Real(1), Real(1) + rexp((vs + Real(83)) * Real(1.0 / 4)));
    qtau = vs >= Real(-80) ? rexp(-(vs + Real(22)) * Real(1.0 / 10.5)) + Real(28) : rexp((vs + Real(467)) * Real(1.0 / 66.6));
  }
};

template <typename Real>
struct HcnRates {
  Real pinf, ptau;
  __host__ __device__ __forceinline__ HcnRates(Real v) {
    pinf = rdiv(Real(1), Real(1) + rexp((v + Real(75)) * Real(1.0 / 5.5)));
    ptau = rdiv(Real(1), rexp(Real(-0.086) * v - Real(14.59)) + rexp(Real(0.0701) * v - Real(1.87)));
  }
};

template <typename Real>
struct NaHHRates {
  Real ap, bp, aq, bq;
  __host__ __device__ __forceinline__ NaHHRates(Real v, Real vsh) {
    const Real vp = v - vsh;
    ap = Real(1) / exprel(-(vp - Real(5)) * Real(0.1));
    bp = Real(4) * aexp(-(vp + Real(20)) * Real(1.0 / 18));
    aq = Real(0.07) * aexp(-(vp + Real(20)) * Real(0.05));
    bq = Real(1) / (Real(1) + aexp(-(vp - Real(10)) * Real(0.1)));
  }
};

template <typename Real>
struct KHHRates {
  Real a, b;
  __host__ __device__ __forceinline__ KHHRates(Real v, Real vsh) {
    const Real vp = v - vsh;
    a = Real(0.1) / exprel(-(vp + Real(10)) * Real(0.1));
    b = Real(0.125) * aexp(-(vp + Real(20)) * Real(1.0 / 80));
  }
};

template <typename Real>
struct KMRates {
  Real ninf, ntau;
  __host__ __device__ __forceinline__ KMRates(Real v) {
    ninf = rdiv(Real(1), Real(1) + rexp(-(v + Real(35)) * Real(1.0 / 6)));
    ntau = rdiv(Real(1), Real(0.0033) * rexp((v + Real(30)) * Real(1.0 / 40)) +
                             Real(0.0033) * rexp(-(v + Real(30)) * Real(1.0 / 20)));
  }
};

// KA1_HM1992 / KA2_HM1992 (A current): the two classes differ only in the
// activation midpoint and slope (KA1: -60 mV / 8.5, KA2: -36 mV / 20); V' = V - V_sh.
template <typename Real>
struct KARates {
  Real pinf, ptau, qinf, qtau;
  __host__ __device__ __forceinline__ KARates(Real v, Real vsh, Real pmid, Real pinv_slope) {
    const Real vp = v - vsh;
    pinf = rdiv(Real(1), Real(1) + rexp(-(vp + pmid) * pinv_slope));
    ptau = rdiv(Real(1), rexp((vp + Real(35.8)) * Real(1.0 / 19.7)) + rexp(-(vp + Real(79.7)) * Real(1.0 / 12.7))) +
           Real(0.37);
    qinf = rdiv(Real(1), Real(1) + rexp((vp + Real(78)) * Real(1.0 / 6)));
    qtau = vp < Real(-63)
               ? rdiv(Real(1), rexp((vp + Real(46)) * Real(0.2)) + rexp(-(vp + Real(238)) * Real(1.0 / 37.5)))
               : Real(19);
  }
};
// KK2A_HM1992 / KK2B_HM1992 (slow I_K2): the same activation and inactivation
// curves; tau_q is 120 ms + a bell for KK2A, and for KK2B the bell strictly below
// V' = -70 and 8.9 ms at and above it.
template <typename Real>
struct K2Rates {
  Real pinf, ptau, qinf, qtau;
  __host__ __device__ __forceinline__ K2Rates(Real v, Real vsh, bool b_form) {
    const Real vp = v - vsh;
    pinf = rdiv(Real(1), Real(1) + rexp(-(vp + Real(43)) * Real(1.0 / 17)));
    ptau = rdiv(Real(1), rexp((vp - Real(81)) * Real(1.0 / 25.6)) + rexp(-(vp + Real(132)) * Real(1.0 / 18))) +
           Real(9.9);
    qinf = rdiv(Real(1), Real(1) + rexp((vp + Real(58)) * Real(1.0 / 10.6)));
    const Real bell = rdiv(Real(1), rexp((vp - Real(1329)) * Real(0.005)) + rexp(-(vp + Real(130)) * Real(1.0 / 7.1)));
    qtau = b_form ? (vp < Real(-70) ? bell : Real(8.9)) : bell + Real(120);
  }
};
// KNI_Ya1989 (slow non-inactivating K): V' = V - V_sh, tau_max a parameter (ms).
template <typename Real>
struct KNIRates {
  Real pinf, ptau;
  __host__ __device__ __forceinline__ KNIRates(Real v, Real vsh, Real tau_max) {
    const Real x = v - vsh + Real(35);
    pinf = rdiv(Real(1), Real(1) + rexp(-x * Real(0.1)));
    ptau = rdiv(tau_max, Real(3.3) * rexp(x * Real(0.05)) + rexp(-x * Real(0.05)));
  }
};
constexpr double kKA1Mid = 60.0, kKA1InvSlope = 1.0 / 8.5;
constexpr double kKA2Mid = 36.0, kKA2InvSlope = 1.0 / 20.0;

// Fixed state slot of every mechanism state in the [slot][node] state array.
constexpr int kSlotNaP = 0;
constexpr int kSlotNaQ = 1;
constexpr int kSlotKdrP = 2;
constexpr int kSlotCalP = 3;
constexpr int kSlotCalQ = 4;
constexpr int kSlotCatP = 5;
constexpr int kSlotCatQ = 6;
constexpr int kSlotHcnP = 7;
constexpr int kSlotAhpP = 8;
constexpr int kSlotCaHi = 9;   // CalciumDetailed Ci, float-float high word
constexpr int kSlotCaLo = 10;  // low word
constexpr int kSlotNaHHP = 11;
constexpr int kSlotNaHHQ = 12;
constexpr int kSlotKHHP = 13;
constexpr int kSlotKMN = 14;
constexpr int kSlotKA1P = 15;
constexpr int kSlotKA1Q = 16;
constexpr int kSlotKA2P = 17;
constexpr int kSlotKA2Q = 18;
constexpr int kSlotKK2AP = 19;
constexpr int kSlotKK2AQ = 20;
constexpr int kSlotKK2BP = 21;
constexpr int kSlotKK2BQ = 22;
constexpr int kSlotKNIP = 23;
// membrane voltage at the start of the last step taken (float-float), written on
// the last step of every launch: the `last_V` of the per-CV spike indicator
constexpr int kSlotVLastHi = 24;
constexpr int kSlotVLastLo = 25;
constexpr int kNumSlots = 26;

constexpr double kFaraday = 96485.33212;   // C/mol
constexpr double kGasR = 8.314462618;      // J/(mol K)
// 1e3 * R / (2 F): Nernst slope for z = 2 in mV/K
constexpr double kNernstCa = 1e3 * kGasR / (2.0 * kFaraday);
// uA/cm^2 -> mM/ms influx per um of shell depth: 10 / (2 F)
constexpr double kCaDrive = 10.0 / (2.0 * kFaraday);

// ------------------------------------------------------- cerebellar HH channels
// Kv3p4_MA2020_GoC (channel/potassium.py:4750): m^3 h on V' = V + 11 mV (the
// junction potential), inf / tau forms in seconds scaled to ms.
template <typename Real>
struct Kv34Rates {
  Real minf, mtau, hinf, htau;
  __host__ __device__ __forceinline__ explicit Kv34Rates(Real v) {
    const Real x = v + Real(11);
    minf = Real(1) / (Real(1) + aexp(-(x + Real(24)) / Real(15.4)));
    const Real mt = x < Real(-35) ? (Real(3.4225e-5) + Real(0.00498) * aexp(x / Real(28.29))) * Real(3)
                                  : Real(0.00012851) + Real(1) / (aexp((x + Real(100.7)) / Real(12.9)) +
                                                                  aexp((x - Real(56)) / Real(-23.1)));
    mtau = Real(1000) * mt;
    hinf = Real(0.31) + Real(0.69) / (Real(1) + aexp((x + Real(5.802)) / Real(11.2)));
    const Real y = (x + Real(56.3)) / Real(49.6);
    const Real ht = x > Real(0) ? Real(0.0012) + Real(0.0023) * aexp(Real(-0.141) * x)
                                : Real(1.2202e-05) + Real(0.012) * aexp(-(y * y));
    htau = Real(1000) * ht;
  }
};

// Kv4p3_MA2020_GoC (channel/potassium.py:4964): a^3 b, inf sigmoids and
// tau = 1 / (alpha + beta) with sigm(x, y) = 1 / (exp(x / y) + 1) (:73-74).
template <typename Real>
struct Kv43Rates {
  Real ainf, atau, binf, btau;
  __host__ __device__ __forceinline__ explicit Kv43Rates(Real v) {
    const Real aa = Real(0.8147) / (aexp((v + Real(9.17203)) / Real(-23.3271)) + Real(1));
    const Real ab = Real(0.1655) / aexp((v + Real(18.2791)) / Real(19.4718));
    const Real ba = Real(0.0368) / (aexp((v + Real(111.332)) / Real(12.8433)) + Real(1));
    const Real bb = Real(0.0345) / (aexp((v + Real(49.9537)) / Real(-8.90123)) + Real(1));
    ainf = Real(1) / (Real(1) + aexp((v + Real(38)) / Real(-17)));
    atau = Real(1) / (aa + ab);
    binf = Real(1) / (Real(1) + aexp((v + Real(78.8)) / Real(8.4)));
    btau = Real(1) / (ba + bb);
  }
};

// Kv1p1_MA2020_GoC (channel/potassium.py:4570): n^4, alpha / beta form.
template <typename Real>
struct Kv11Rates {
  Real a, b;
  __host__ __device__ __forceinline__ explicit Kv11Rates(Real v) {
    a = Real(0.12889) * aexp((v + Real(45)) / Real(33.90877));
    b = Real(0.12889) * aexp(-(v + Real(45)) / Real(12.42101));
  }
};

// Kir2p3_MA2020_GrC (channel/potassium.py:5334): d, alpha / beta form.
template <typename Real>
struct Kir23Rates {
  Real a, b;
  __host__ __device__ __forceinline__ explicit Kir23Rates(Real v) {
    a = Real(0.13289) * aexp((v + Real(83.94)) / Real(-24.3902));
    b = Real(0.16994) * aexp((v + Real(83.94)) / Real(35.714));
  }
};

// HCN1_MA2020_GoC (channel/hyperpolarization_activated.py:675): two gates whose
// steady states split o_inf by r(V) = 0.002096 V + 0.97596.
template <typename Real>
struct Hcn1fRates {
  Real finf, ftau, sinf, stau;
  __host__ __device__ __forceinline__ explicit Hcn1fRates(Real v) {
    const Real o = Real(1) / (Real(1) + aexp((v + Real(72.49)) * Real(0.11305)));
    const Real r = Real(0.002096) * v + Real(0.97596);
    finf = r * o;
    sinf = (Real(1) - r) * o;
    ftau = aexp((Real(0.01371) * v + Real(3.368)) * Real(2.30259));
    stau = aexp((Real(0.01451) * v + Real(4.056)) * Real(2.30259));
  }
};

// HCN1_MA2024_PC (channel/hyperpolarization_activated.py:411): h, with the
// half-activation voltages shifted by the 9.3 mV junction potential.
template <typename Real>
struct Hcn1hRates {
  Real hinf, htau;
  __host__ __device__ __forceinline__ explicit Hcn1hRates(Real v) {
    hinf = Real(1) / (Real(1) + aexp((v + Real(99.6)) / Real(9.67)));
    htau = Real(1) / (Real(0.0018) * (aexp((v + Real(77.3)) / Real(-22)) + aexp((v + Real(77.3)) / Real(7.14))));
  }
};

// CaHVA_MA2020_GoC (channel/calcium.py:4333; the GrC class, :4499, is identical):
// s^2 u, alpha / beta exponentials.
template <typename Real>
struct CaHvaRates {
  Real sa, sb, ua, ub;
  __host__ __device__ __forceinline__ explicit CaHvaRates(Real v) {
    sa = Real(0.04944) * aexp((v + Real(29.06)) / Real(15.873));
    sb = Real(0.08298) * aexp((v + Real(18.66)) / Real(-25.641));
    ua = Real(0.0013) * aexp((v + Real(48)) / Real(-18.183));
    ub = Real(0.0013) * aexp((v + Real(48)) / Real(83.33));
  }
};

// Cav2p3_MA2020_GoC (channel/calcium.py:4672): m^3 h, fixed time constants.
template <typename Real>
struct Cav23Rates {
  Real minf, mtau, hinf, htau;
  __host__ __device__ __forceinline__ explicit Cav23Rates(Real v) {
    minf = Real(1) / (Real(1) + aexp((v + Real(48.5)) / Real(-3)));
    hinf = Real(1) / (Real(1) + aexp((v + Real(53)) / Real(1)));
    mtau = Real(50);
    htau = Real(5);
  }
};

// Cav3p2_RI2021_SC (channel/calcium.py:3636; the BC and PC classes inherit it): m^2 h
// on V + V_sh; the h time constant carries its own 36 degC factor 3^1.2.
template <typename Real>
struct Cav32Rates {
  Real minf, mtau, hinf, htau;
  __host__ __device__ __forceinline__ Cav32Rates(Real v0, Real vsh) {
    const Real v = v0 + vsh;
    minf = Real(1) / (Real(1) + aexp(-(v + Real(54.8)) / Real(7.4)));
    hinf = Real(1) / (Real(1) + aexp((v + Real(85.5)) / Real(7.18)));
    mtau = Real(1.9) + Real(1) / (aexp((v + Real(37)) / Real(11.9)) + aexp(-(v + Real(131.6)) / Real(21)));
    const Real phi_h = Real(3.7371928188465517);  // 3^((36 - 24) / 10)
    htau = Real(13.7) + (Real(1942) + aexp((v + Real(164)) / Real(9.2))) / (Real(1) + aexp((v + Real(89.3)) / Real(3.7))) /
                            phi_h;
  }
};
// Cav3p2's m gate temperature factor, 5^((36 - 24) / 10)
constexpr double kCav32PhiM = 6.898648307306074;

// ---------------------------------------------------------------- Markov channels
// The independent states of each scheme (channel/_base.py:677-1125: every state but
// the dependent one, which is 1 - their sum), in the order they first appear in the
// scheme's transition list.  Plans with a Markov channel carry kNumSlotsMarkov
// slots per node; the others kNumSlots.
constexpr int kSlotNav16 = 26;  // Nav1p6_MA2020_GoC: C1..C5, I1..I5, O, B
constexpr int kSlotKca22 = 38;  // Kca2p2_MA2020_GoC: C2, C3, C4, O1, O2
constexpr int kSlotKca11 = 43;  // Kca1p1_MA2020_GoC: C1..C4, O0..O4
constexpr int kNumSlotsMarkov = 52;
// Cerebellar HH channels (after the Markov states; plans with one carry
// kNumSlotsCerebellar slots per node)
constexpr int kSlotKv34M = 52;
constexpr int kSlotKv34H = 53;
constexpr int kSlotKv43A = 54;
constexpr int kSlotKv43B = 55;
constexpr int kSlotKv11N = 56;
constexpr int kSlotKir23D = 57;
constexpr int kSlotHcn1Fast = 58;
constexpr int kSlotHcn1Slow = 59;
constexpr int kSlotHcn1H = 60;
constexpr int kSlotCaHvaS = 61;
constexpr int kSlotCaHvaU = 62;
constexpr int kSlotCav23M = 63;
constexpr int kSlotCav23H = 64;
constexpr int kSlotCav32M = 65;
constexpr int kSlotCav32H = 66;
constexpr int kNumSlotsCerebellar = 67;
constexpr int kMarkovMaxStates = 13;

// A transition graph: states 0 .. ns-1 (dep is eliminated), pair k moves src -> dst
// at kf[k] * s[src] and back at kb[k] * s[dst].
struct MarkovGraph {
  int ns, np, dep, slot0;
  const int8_t* src;
  const int8_t* dst;
};

// sodium.py:840-858: C1 0 .. C5 4, I1 5 .. I5 9, O 10, B 11, I6 12
static __device__ __constant__ const int8_t kNav16Src[17] = {0, 1, 2, 3, 0, 5, 1, 6, 2, 7, 3, 8, 4, 4, 10, 9, 10};
static __device__ __constant__ const int8_t kNav16Dst[17] = {1, 2, 3, 4, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 11, 12, 12};
// potassium_calcium.py:717-724: C1 0, C2 1, C3 2, C4 3, O1 4, O2 5
static __device__ __constant__ const int8_t kKca22Src[5] = {0, 1, 2, 2, 3};
static __device__ __constant__ const int8_t kKca22Dst[5] = {1, 2, 3, 4, 5};
// potassium_calcium.py:1213-1228: C0 0 .. C4 4, O0 5 .. O4 9
static __device__ __constant__ const int8_t kKca11Src[13] = {0, 1, 2, 3, 5, 6, 7, 8, 0, 1, 2, 3, 4};
static __device__ __constant__ const int8_t kKca11Dst[13] = {1, 2, 3, 4, 6, 7, 8, 9, 5, 6, 7, 8, 9};

// Nav1.6-scheme rates (sodium.py:903-935; constants :874-898 with x3 = x5 = 1e12,
// x4 = -1e12 and the V shifts 0).  Oon, alfac = (Oon / Con)^(1/4) and epsilon come
// from the parameter record: Nav1p1_MA2025_BC (sodium.py:1188) runs the same scheme
// with Oon 2.3 and epsilon 1e-12.
template <typename Real>
__device__ __forceinline__ void nav16_rates(Real v, Real phi, Real oon, Real alfac, Real ep, Real* kf, Real* kb) {
  const Real al = Real(150), be = Real(3), ga = Real(150), de = Real(40), ze = Real(0.03);
  const Real con = Real(0.005), coff = Real(0.5), ooff = Real(0.005);
  const double bf[5] = {1.0, 0.31622776601683794, 0.1, 0.03162277660168379, 0.01};  // (Ooff / Coff)^(k/4)
  const Real ea = aexp(v / Real(20)) * phi, eb = aexp(v / Real(-20)) * phi;
  const Real e3 = aexp(v / Real(1e12)) * phi, e4 = aexp(v / Real(-1e12)) * phi, e6 = aexp(v / Real(-25)) * phi;
  const Real e5 = aexp(v / Real(1e12)) * phi;
  const Real a2 = alfac * alfac, a3 = a2 * alfac, a4 = a3 * alfac;
  const Real btfac = Real(bf[1]);
  // pair order: C1C2 C2C3 C3C4 C4C5 C1I1 I1I2 C2I2 I2I3 C3I3 I3I4 C4I4 I4I5 C5I5 C5O OB I5I6 OI6
  kf[0] = Real(4) * al * ea;  kb[0] = Real(1) * be * eb;
  kf[1] = Real(3) * al * ea;  kb[1] = Real(2) * be * eb;
  kf[2] = Real(2) * al * ea;  kb[2] = Real(3) * be * eb;
  kf[3] = Real(1) * al * ea;  kb[3] = Real(4) * be * eb;
  kf[4] = con * phi;          kb[4] = coff * phi;
  kf[5] = Real(4) * al * alfac * ea;  kb[5] = Real(1) * be * btfac * eb;
  kf[6] = con * alfac * phi;          kb[6] = coff * Real(bf[1]) * phi;
  kf[7] = Real(3) * al * alfac * ea;  kb[7] = Real(2) * be * btfac * eb;
  kf[8] = con * a2 * phi;             kb[8] = coff * Real(bf[2]) * phi;
  kf[9] = Real(2) * al * alfac * ea;  kb[9] = Real(3) * be * btfac * eb;
  kf[10] = con * a3 * phi;            kb[10] = coff * Real(bf[3]) * phi;
  kf[11] = Real(1) * al * alfac * ea; kb[11] = Real(4) * be * btfac * eb;
  kf[12] = con * a4 * phi;            kb[12] = coff * Real(bf[4]) * phi;
  kf[13] = ga * e3;                   kb[13] = de * e4;
  kf[14] = ep * e5;                   kb[14] = ze * e6;
  kf[15] = ga * e3;                   kb[15] = de * e4;
  kf[16] = oon * phi;                 kb[16] = ooff * phi;
}

// Kca2p2 rates (potassium_calcium.py:760-790; constants :740-753): the
// calcium-binding steps at k phi Ci / diff, the others at k phi.
template <typename Real>
__device__ __forceinline__ void kca22_rates(Real ci, Real phi, Real diff, Real* kf, Real* kb) {
  const Real c = phi * ci / diff;
  kf[0] = Real(200) * c;       kb[0] = Real(80e-3) * phi;
  kf[1] = Real(160) * c;       kb[1] = Real(80e-3) * phi;
  kf[2] = Real(80) * c;        kb[2] = Real(200e-3) * phi;
  kf[3] = Real(160e-3) * phi;  kb[3] = Real(1) * phi;
  kf[4] = Real(1.2) * phi;     kb[4] = Real(100e-3) * phi;
}

// Kca1p1 rates (potassium_calcium.py:1277-1353; constants :1243-1265): binding at
// (4 - i) Ci k1, unbinding at (i + 1) Kc k1 (closed) or (i + 1) Ko k1 (open),
// opening at pf_i exp(Qo F V / R T), closing at pb_i exp(Qc F V / R T), all x phi.
template <typename Real>
__device__ __forceinline__ void kca11_rates(Real v, Real ci, Real phi, Real qo, Real qc, Real* kf, Real* kb) {
  const double pf[5] = {2.39e-3, 7.0e-3, 40e-3, 295e-3, 557e-3};
  const double pb[5] = {3936e-3, 1152e-3, 659e-3, 486e-3, 92e-3};
  const Real on = Real(1e3) * phi * ci;
  const Real a = aexp(qo * v) * phi, b = aexp(qc * v) * phi;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    kf[i] = Real(4 - i) * on;
    kb[i] = Real(i + 1) * Real(11.0e-3 * 1e3) * phi;
    kf[4 + i] = Real(4 - i) * on;
    kb[4 + i] = Real(i + 1) * Real(1.1e-3 * 1e3) * phi;
  }
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    kf[8 + i] = Real(pf[i]) * a;
    kb[8 + i] = Real(pb[i]) * b;
  }
}

// Gaussian elimination with partial pivoting of the n x n system in A[.][0..n-1]
// with its right-hand side in A[.][n]; the solution replaces column n.
template <typename Real>
__device__ __forceinline__ void dense_solve(Real (*A)[kMarkovMaxStates + 1], int n) {
  for (int c = 0; c < n; ++c) {
    int piv = c;
    Real best = fabs(A[c][c]);
    for (int r = c + 1; r < n; ++r)
      if (fabs(A[r][c]) > best) {
        best = fabs(A[r][c]);
        piv = r;
      }
    if (piv != c)
      for (int k = c; k <= n; ++k) {
        const Real t = A[c][k];
        A[c][k] = A[piv][k];
        A[piv][k] = t;
      }
    for (int r = c + 1; r < n; ++r) {
      const Real l = A[r][c] / A[c][c];
      if (l != Real(0))
        for (int k = c + 1; k <= n; ++k) A[r][k] -= l * A[c][k];
    }
  }
  for (int c = n - 1; c >= 0; --c) {
    Real x = A[c][n];
    for (int k = c + 1; k < n; ++k) x -= A[c][k] * A[k][n];
    A[c][n] = x / A[c][c];
  }
}

// One linearised backward-Euler step (quad/_backward_euler.py:31-64) of a Markov
// scheme's independent states in slots slot0.. of the node's state column: the
// kinetics see each independent state clipped to [0, 1] and the dependent state as
// 1 - the raw sum (channel/_base.py:852-878, 1105-1125); J = df/dy there (d clip /
// dy = 1 on [0, 1], 0 outside); (I - dt J) dy = dt f; y += dy.
template <typename Real>
__device__ void markov_advance(Real* st, int N, const MarkovGraph& g, const Real* kf, const Real* kb, Real dt) {
  Real A[kMarkovMaxStates][kMarkovMaxStates + 1];
  Real s[kMarkovMaxStates], msk[kMarkovMaxStates];
  const int ni = g.ns - 1;
  Real sum = Real(0);
  for (int k = 0; k < g.ns; ++k) {
    if (k == g.dep) continue;
    const int j = k < g.dep ? k : k - 1;
    const Real y = st[(g.slot0 + j) * N];
    sum += y;
    s[k] = y < Real(0) ? Real(0) : (y > Real(1) ? Real(1) : y);
    msk[k] = (y >= Real(0) && y <= Real(1)) ? Real(1) : Real(0);
  }
  s[g.dep] = Real(1) - sum;
  msk[g.dep] = Real(0);
  for (int r = 0; r < ni; ++r)
    for (int c = 0; c <= ni; ++c) A[r][c] = Real(0);
  // A[.][0..ni-1] = J, A[.][ni] = f
  for (int p = 0; p < g.np; ++p) {
    const int a = g.src[p], b = g.dst[p];
    for (int dir = 0; dir < 2; ++dir) {
      const int by = dir ? b : a, to = dir ? a : b;
      const Real rate = dir ? kb[p] : kf[p];
      const Real fl = rate * s[by];
      const int rf = by == g.dep ? -1 : (by < g.dep ? by : by - 1);
      const int rt = to == g.dep ? -1 : (to < g.dep ? to : to - 1);
      if (rf >= 0) A[rf][ni] -= fl;
      if (rt >= 0) A[rt][ni] += fl;
      if (by == g.dep) {  // d s_dep / d y_j = -1 for every j
        if (rt >= 0)
          for (int c = 0; c < ni; ++c) A[rt][c] -= rate;
      } else {
        const Real d = rate * msk[by];
        A[rf][rf] -= d;
        if (rt >= 0) A[rt][rf] += d;
      }
    }
  }
  for (int r = 0; r < ni; ++r) {
    for (int c = 0; c < ni; ++c) A[r][c] = (r == c ? Real(1) : Real(0)) - dt * A[r][c];
    A[r][ni] *= dt;
  }
  dense_solve(A, ni);
  for (int j = 0; j < ni; ++j) st[(g.slot0 + j) * N] += A[j][ni];
}

// Stationary distribution of a scheme (channel/_base.py:1033-1091): the generator
// with the dependent state's row replaced by ones = 1, solved, clipped at 0 and
// renormalised; the independent states are stored.
template <typename Real>
__device__ void markov_steady(Real* st, int N, const MarkovGraph& g, const Real* kf, const Real* kb) {
  Real A[kMarkovMaxStates][kMarkovMaxStates + 1];
  const int n = g.ns;
  for (int r = 0; r < n; ++r)
    for (int c = 0; c <= n; ++c) A[r][c] = Real(0);
  for (int p = 0; p < g.np; ++p) {
    const int a = g.src[p], b = g.dst[p];
    A[a][a] -= kf[p];
    A[b][a] += kf[p];
    A[a][b] += kb[p];
    A[b][b] -= kb[p];
  }
  for (int c = 0; c < n; ++c) A[g.dep][c] = Real(1);
  A[g.dep][n] = Real(1);
  dense_solve(A, n);
  Real tot = Real(0);
  for (int k = 0; k < n; ++k) {
    A[k][n] = A[k][n] < Real(0) ? Real(0) : A[k][n];
    tot += A[k][n];
  }
  for (int k = 0; k < n; ++k) {
    if (k == g.dep) continue;
    st[(g.slot0 + (k < g.dep ? k : k - 1)) * N] = A[k][n] / tot;
  }
}

}  // namespace bc
