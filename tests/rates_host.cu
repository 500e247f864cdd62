// Test harness: the FP64 rate structures of the step kernel's mechanism header,
// compiled for the host, so that tests/test_rates_host.py can compare them with
// the oracle's rate functions on a CPU.  Not part of the library.
#include "../braincell_gb300/csrc/bc_ext.cuh"

using namespace bc;

// Kernel rate structure `which` at n voltages v (mV) with parameters prm (V_sh
// first; KNI: V_sh, tau_max; Kv1p5: its Q10 factor, Tauact, Tauinactf, Tauinacts;
// Kca3p1 and SK: Ci (mM); K_Kv_test: V_sh, Ra, Rb, q, v12).
// out[6 i .. 6 i + 5] receives the gate rates in the oracle's order: per gate
// (alpha, beta) or (inf, tau); unused entries are 0.
// Returns 0, or -1 for an unknown structure.
extern "C" int bc_test_rates(int which, const double* v, int n, const double* prm, double* out) {
  for (int i = 0; i < n; ++i) {
    double* o = out + 6 * i;
    o[0] = o[1] = o[2] = o[3] = o[4] = o[5] = 0.0;
    const double x = v[i];
    switch (which) {
      case 0: { const NaRates<double> r(x, prm[0]); o[0] = r.ap; o[1] = r.bp; o[2] = r.aq; o[3] = r.bq; break; }
      case 1: { const KdrRates<double> r(x, prm[0]); o[0] = r.a; o[1] = r.b; break; }
      case 2: { const CaLRates<double> r(x, prm[0]); o[0] = r.pinf; o[1] = r.ptau; o[2] = r.qinf; o[3] = r.qtau; break; }
      case 3: { const CaTRates<double> r(x, prm[0]); o[0] = r.pinf; o[1] = r.ptau; o[2] = r.qinf; o[3] = r.qtau; break; }
      case 4: { const HcnRates<double> r(x); o[0] = r.pinf; o[1] = r.ptau; break; }
      case 5: { const NaHHRates<double> r(x, prm[0]); o[0] = r.ap; o[1] = r.bp; o[2] = r.aq; o[3] = r.bq; break; }
      case 6: { const KHHRates<double> r(x, prm[0]); o[0] = r.a; o[1] = r.b; break; }
      case 7: { const KMRates<double> r(x); o[0] = r.ninf; o[1] = r.ntau; break; }
      case 8: {
        const KARates<double> r(x, prm[0], kKA1Mid, kKA1InvSlope);
        o[0] = r.pinf; o[1] = r.ptau; o[2] = r.qinf; o[3] = r.qtau;
        break;
      }
      case 9: {
        const KARates<double> r(x, prm[0], kKA2Mid, kKA2InvSlope);
        o[0] = r.pinf; o[1] = r.ptau; o[2] = r.qinf; o[3] = r.qtau;
        break;
      }
      case 10: { const K2Rates<double> r(x, prm[0], false); o[0] = r.pinf; o[1] = r.ptau; o[2] = r.qinf; o[3] = r.qtau; break; }
      case 11: { const K2Rates<double> r(x, prm[0], true); o[0] = r.pinf; o[1] = r.ptau; o[2] = r.qinf; o[3] = r.qtau; break; }
      case 12: { const KNIRates<double> r(x, prm[0], prm[1]); o[0] = r.pinf; o[1] = r.ptau; break; }
      case 13: { const Kv34Rates<double> r(x); o[0] = r.minf; o[1] = r.mtau; o[2] = r.hinf; o[3] = r.htau; break; }
      case 14: { const Kv43Rates<double> r(x); o[0] = r.ainf; o[1] = r.atau; o[2] = r.binf; o[3] = r.btau; break; }
      case 15: { const Kv11Rates<double> r(x); o[0] = r.a; o[1] = r.b; break; }
      case 16: { const Kir23Rates<double> r(x); o[0] = r.a; o[1] = r.b; break; }
      case 17: { const Hcn1fRates<double> r(x); o[0] = r.finf; o[1] = r.ftau; o[2] = r.sinf; o[3] = r.stau; break; }
      case 18: { const Hcn1hRates<double> r(x); o[0] = r.hinf; o[1] = r.htau; break; }
      case 19: { const CaHvaRates<double> r(x); o[0] = r.sa; o[1] = r.sb; o[2] = r.ua; o[3] = r.ub; break; }
      case 20: { const Cav23Rates<double> r(x); o[0] = r.minf; o[1] = r.mtau; o[2] = r.hinf; o[3] = r.htau; break; }
      case 21: { const Cav32Rates<double> r(x, prm[0]); o[0] = r.minf; o[1] = r.mtau; o[2] = r.hinf; o[3] = r.htau; break; }
      case 22: { const Hcn2Rates<double> r(x); o[0] = r.finf; o[1] = r.ftau; o[2] = r.sinf; o[3] = r.stau; break; }
      case 23: { const Kv33Rates<double> r(x); o[0] = r.a; o[1] = r.b; break; }
      case 24: { const Kv22Rates<double> r(x); o[0] = r.minf; o[1] = r.mtau; o[2] = r.hinf; o[3] = r.htau; break; }
      case 25: {
        const Kv15Rates<double> r(x, prm[0], prm[1], prm[2]);
        o[0] = r.minf; o[1] = r.mtau; o[2] = r.ninf; o[3] = r.ntau; o[4] = r.uinf; o[5] = kKv15TauU * prm[3];
        break;
      }
      case 26: { const NafRates<double> r(x); o[0] = r.minf; o[1] = r.mtau; o[2] = r.hinf; o[3] = r.htau; break; }
      case 27: { const NapRates<double> r(x); o[0] = r.minf; o[1] = r.mtau; o[2] = r.hinf; o[3] = r.htau; break; }
      case 28: { const NaioRates<double> r(x); o[0] = r.minf; o[1] = r.mtau; o[2] = r.hinf; o[3] = r.htau; break; }
      case 29: { const Su2015KdrRates<double> r = fkdr_rates(x); o[0] = r.minf; o[1] = r.mtau; break; }
      case 30: { const Su2015KdrRates<double> r = skdr_rates(x); o[0] = r.minf; o[1] = r.mtau; break; }
      case 31: { const KdrioRates<double> r(x); o[0] = r.ninf; o[1] = r.ntau; break; }
      case 32: { const HcndcnRates<double> r(x); o[0] = r.minf; o[1] = r.mtau; break; }
      case 33: { const HcnioRates<double> r(x); o[0] = r.qinf; o[1] = r.qtau; break; }
      case 34: { const CathpRates<double> r(x, prm[0]); o[0] = r.pinf; o[1] = r.ptau; o[2] = r.qinf; o[3] = r.qtau; break; }
      case 35: { const CahtreRates<double> r(x, prm[0]); o[0] = r.ap; o[1] = r.bp; o[2] = r.aq; o[3] = r.bq; break; }
      case 36: { const CaldcnRates<double> r(x); o[0] = r.minf; o[1] = r.mtau; o[2] = r.hinf; o[3] = r.htau; break; }
      case 37: { const Kca31Rates<double> r(x, prm[0]); o[0] = r.a; o[1] = r.b; break; }
      case 38: { const SkdcnRates<double> r(prm[0]); o[0] = r.zinf; o[1] = r.ztau; break; }
      case 39: {
        const KkvRates<double> r(x, prm[0], prm[1], prm[2], prm[3], prm[4]);
        o[0] = r.ninf; o[1] = r.ntau;
        break;
      }
      case 40: { const CanRates<double> r(x); o[0] = r.pinf; o[1] = r.ptau; break; }
      case 41: { const CaioRates<double> r(x); o[0] = r.hinf; o[1] = r.htau; break; }
      case 42: { const Cav31Rates<double> r(x, prm[0]); o[0] = r.pinf; o[1] = r.ptau; o[2] = r.qinf; o[3] = r.qtau; break; }
      case 46:
      case 47: {  // Cav1p2 / Cav1p3 at Ci = prm[0]: (m_inf, m_tau, h_inf, h_tau, n_inf, n_tau)
        const Cav1Rates<double> r(x, prm[0], cav1_consts(which == 46));
        o[0] = r.minf; o[1] = r.mtau; o[2] = r.hinf; o[3] = kCav1TauH; o[4] = r.ninf; o[5] = kCav1TauN;
        break;
      }
      case 48: { const Cav21Rates<double> r(x, prm[0]); o[0] = r.minf; o[1] = r.mtau; break; }
      case 49: {  // the shared GHK drive and its V-derivative at ci = prm[0], co = prm[1], T = prm[2]
        double dd;
        o[0] = ghk_codata_drive(x, prm[0], prm[1], prm[2], dd);
        o[1] = dd;
        break;
      }
      case 50: { const CahvadcnRates<double> r(x); o[0] = r.minf; o[1] = r.mtau; break; }
      case 51: {  // the SU2015 drive and its V-derivative at ci = prm[0], co = prm[1], T = prm[2]
        double dd;
        o[0] = su2015_drive(x, prm[0], prm[1], prm[2], dd);
        o[1] = dd;
        break;
      }
      case 44: { const Cav33Rates<double> r(x, prm[0]); o[0] = r.ninf; o[1] = r.ntau; o[2] = r.linf; o[3] = r.ltau; break; }
      case 45: {  // the Cav3.3 GHK drive and its V-derivative at ci = prm[0], co = prm[1], T = prm[2]
        double dd;
        o[0] = cav33_drive(x, prm[0], prm[1], prm[2], dd);
        o[1] = dd;
        break;
      }
      case 43: {  // the GHK drive and its V-derivative at ci = prm[0], co = prm[1], T = prm[2]
        double dd;
        o[0] = cav31_drive(x, prm[0], prm[1], prm[2], dd);
        o[1] = dd;
        break;
      }
      default: return -1;
    }
  }
  return 0;
}
