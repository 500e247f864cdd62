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

}  // namespace bc
