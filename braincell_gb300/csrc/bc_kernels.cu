// sm_103a kernels of the multi-compartment Cell time step.
//
// One CTA owns one tile (one or more whole cells).  For shared-memory tiles the
// tile's blob (voltages, axial coefficients, chain schedule, parameter records)
// is staged into shared memory with TMA bulk copies (cp.async.bulk + mbarrier),
// stays resident for `n_steps` fused time steps, and only the voltages are
// written back with a bulk store.  Mechanism states (gates, calcium) stream from
// a global [slot][node] array, read and written once per node per step.  Tiles
// too large for shared memory run the same code on their global-memory blob.
//
// Per time step (reference: quad/_staggered.py:54-154):
//   forward elimination   -- barrier-separated phases; in each, every thread walks
//                            its chains leaf -> root (comp_triang_raw, :641-657);
//   back-substitution     -- phases in reverse, chains root -> leaf (the O(n) sweep
//                            whose result equals comp_backsub_raw, :742-760);
//   per-node update       -- V += delta (float-float), CalciumDetailed Ci from the
//                            step-start current (cell.py:2261-2280, ion/calcium.py:
//                            499-505), gates by exp-Euler at the new V (cell.py:
//                            2157-2217), the next step's linearised row
//                            (_staggered.py:449-513, cell.py:1907-1963), clamp
//                            pulses (_compute/layouts.py:960-982) and probes.
// The voltage system is solved for the increment x = V_{n+1} - V_n; with the same
// matrix this gives the same V_{n+1} as the reference's direct form, and in FP32
// it keeps V to ~1e-5 mV over thousands of steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "bc_internal.h"
#include "bc_mech.cuh"

namespace bc {

constexpr int kStatusNonfinite = 1;
constexpr int kStatusTimeout = 2;
constexpr uint16_t kBoundary = 0xFFFF;
constexpr uint16_t kNoSpecial = 0xFFFF;

// ------------------------------------------------------------------ TMA helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// Bounded wait on phase `parity`; returns false if it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t max_iter) {
  for (uint32_t it = 0; it < max_iter; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void bulk_s2g(void* dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_commit_and_wait() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

constexpr uint32_t kBulkChunk = 32768;  // bytes per bulk copy instruction (multiple of 16)

// ------------------------------------------------------------------ tile view
// Per-node pairs, loaded and stored as one vector access.
template <typename Real>
struct PairOf;
template <>
struct PairOf<float> {
  using type = float2;
};
template <>
struct PairOf<double> {
  using type = double2;
};
template <typename Real>
using Pair = typename PairOf<Real>::type;

template <typename Real>
__device__ __forceinline__ Pair<Real> make_pair(Real a, Real b) {
  Pair<Real> p;
  p.x = a;
  p.y = b;
  return p;
}

template <typename Real>
struct TileView {
  Pair<Real>* v;   // (V_hi, V_lo)
  Pair<Real>* ab;  // (alpha, beta); (alpha dt, beta dt) once pre-scaled
  Pair<Real>* dr;  // (diagonal, rhs) of the row; (1 / pivot, rhs or x) during the sweeps
  Real* state;
  const Real *diag0, *params;
  const int32_t *child, *lists;
  const uint16_t *pidx, *spec;
  const ChainRec* chains;
  const SpecRec* specs;
  const uint32_t* mech;
  Real *scd, *scr, *sfill, *sh;
  int N, n_real, n_phases;

  __device__ __forceinline__ void bind(const TileDesc& td, unsigned char* base, unsigned char* scratch, void* gstate) {
    v = reinterpret_cast<Pair<Real>*>(base + td.off_v);
    ab = reinterpret_cast<Pair<Real>*>(base + td.off_ab);
    dr = reinterpret_cast<Pair<Real>*>(scratch + td.off_dr);
    state = reinterpret_cast<Real*>(gstate) + td.state_offset;
    diag0 = reinterpret_cast<const Real*>(base + td.off_diag0);
    params = reinterpret_cast<const Real*>(base + td.off_params);
    child = reinterpret_cast<const int32_t*>(base + td.off_child);
    lists = reinterpret_cast<const int32_t*>(base + td.off_lists);
    pidx = reinterpret_cast<const uint16_t*>(base + td.off_pidx);
    spec = reinterpret_cast<const uint16_t*>(base + td.off_spec);
    chains = reinterpret_cast<const ChainRec*>(base + td.off_chains);
    specs = reinterpret_cast<const SpecRec*>(base + td.off_specs);
    mech = reinterpret_cast<const uint32_t*>(base + td.off_mech);
    scd = reinterpret_cast<Real*>(scratch + td.off_scd);
    scr = reinterpret_cast<Real*>(scratch + td.off_scr);
    sfill = reinterpret_cast<Real*>(scratch + td.off_sfill);
    sh = reinterpret_cast<Real*>(scratch + td.off_sh);
    N = td.n_nodes;
    n_real = td.n_real_nodes;
    n_phases = td.n_phases;
  }
};

// Reciprocal of a Hines pivot.  FP32: the hardware approximation (about 1 ulp;
// pivots are >= 1 on membrane rows and O(dt * g / C) on boundary rows, far from
// the denormal range); FP64: IEEE round-to-nearest.
__device__ __forceinline__ float pivot_rcp(float d) { return __fdividef(1.0f, d); }
__device__ __forceinline__ double pivot_rcp(double d) { return __drcp_rn(d); }

// float-float accumulation: (hi, lo) += d
template <typename Real>
__device__ __forceinline__ void ff_add(Real& hi, Real& lo, Real d) {
  const Real s = hi + d;
  const Real bb = s - hi;
  const Real err = (hi - (s - bb)) + (d - bb);
  const Real t = lo + err;
  hi = s + t;
  lo = t - (hi - s);
}

// ------------------------------------------------------------------ mechanisms
// The mechanism states of one node, held in registers (absent ones are 0).
template <typename Real>
struct NodeStates {
  Real nap, naq, kdrp, calp, calq, catp, catq, hcnp, ahpp, cahi, calo;
};

template <typename Real>
__device__ __forceinline__ void load_states(const Real* st, int N, uint32_t m, NodeStates<Real>& s) {
  s.nap = s.naq = s.kdrp = s.calp = s.calq = s.catp = s.catq = s.hcnp = s.ahpp = s.cahi = s.calo = Real(0);
  if (m & BC_M_NA) {
    s.nap = st[kSlotNaP * N];
    s.naq = st[kSlotNaQ * N];
  }
  if (m & BC_M_KDR) s.kdrp = st[kSlotKdrP * N];
  if (m & BC_M_CAL) {
    s.calp = st[kSlotCalP * N];
    s.calq = st[kSlotCalQ * N];
  }
  if (m & BC_M_CAT) {
    s.catp = st[kSlotCatP * N];
    s.catq = st[kSlotCatQ * N];
  }
  if (m & BC_M_HCN) s.hcnp = st[kSlotHcnP * N];
  if (m & BC_M_AHP) s.ahpp = st[kSlotAhpP * N];
  if (m & BC_M_CADET) {
    s.cahi = st[kSlotCaHi * N];
    s.calo = st[kSlotCaLo * N];
  }
}

// One node's mechanisms.  `st` points at the node's slot-0 state (stride N).
// With advance = true the states move from (v_old) to (v_new) first: calcium
// from the step-start current (old gates, old V, old Ci), then every gate at
// v_new (and the new Ci).  Returns the membrane conductance G (mS/cm^2) and
// ionic current I (uA/cm^2) at v_new with the resulting states.
template <typename Real>
__device__ __forceinline__ void node_mechanisms_loaded(const NodeStates<Real>& s0, Real* st, int N, const Real* P,
                                                       uint32_t m, Real v_old, Real v_new, Real dt, bool advance,
                                                       Real& G, Real& I) {
  Real nap = s0.nap, naq = s0.naq, kdrp = s0.kdrp, calp = s0.calp, calq = s0.calq, catp = s0.catp, catq = s0.catq,
       hcnp = s0.hcnp, ahpp = s0.ahpp, cahi = s0.cahi, calo = s0.calo;
  if (advance) {
    if (m & BC_M_CADET) {
      const Real ci = cahi + calo;
      const Real eca = Real(kNernstCa) * P[BC_P_CA_TEMP] * dlog(P[BC_P_CA_CO] / ci);
      Real ica = Real(0);
      if (m & BC_M_CAL) ica += P[BC_P_CAL_G] * calp * calp * calq * (eca - v_old);
      if (m & BC_M_CAT) ica += P[BC_P_CAT_G] * catp * catp * catq * (eca - v_old);
      Real drive = ica * Real(kCaDrive) / P[BC_P_CA_D];
      drive = drive > Real(0) ? drive : Real(0);
      const Real tau = P[BC_P_CA_TAU];
      const Real f = drive + (P[BC_P_CA_CREST] - ci) / tau;
      ff_add(cahi, calo, dt * exprel(-dt / tau) * f);
      st[kSlotCaHi * N] = cahi;
      st[kSlotCaLo * N] = calo;
    }
    if (m & BC_M_NA) {
      const NaRates<Real> r(v_new, P[BC_P_NA_VSH]);
      const Real phi = P[BC_P_NA_PHI];
      nap = gate_ab<Real, true>(nap, r.ap, r.bp, phi, dt);
      naq = gate_ab<Real, true>(naq, r.aq, r.bq, phi, dt);
      st[kSlotNaP * N] = nap;
      st[kSlotNaQ * N] = naq;
    }
    if (m & BC_M_KDR) {
      const KdrRates<Real> r(v_new, P[BC_P_KDR_VSH]);
      kdrp = gate_ab<Real, true>(kdrp, r.a, r.b, P[BC_P_KDR_PHI], dt);
      st[kSlotKdrP * N] = kdrp;
    }
    if (m & BC_M_CAL) {
      const CaLRates<Real> r(v_new, P[BC_P_CAL_VSH]);
      calp = gate_it(calp, r.pinf, r.ptau, P[BC_P_CAL_PHIP], dt);
      calq = gate_it(calq, r.qinf, r.qtau, P[BC_P_CAL_PHIQ], dt);
      st[kSlotCalP * N] = calp;
      st[kSlotCalQ * N] = calq;
    }
    if (m & BC_M_CAT) {
      const CaTRates<Real> r(v_new, P[BC_P_CAT_VSH]);
      catp = gate_it(catp, r.pinf, r.ptau, P[BC_P_CAT_PHIP], dt);
      catq = gate_it(catq, r.qinf, r.qtau, P[BC_P_CAT_PHIQ], dt);
      st[kSlotCatP * N] = catp;
      st[kSlotCatQ * N] = catq;
    }
    if (m & BC_M_HCN) {
      const HcnRates<Real> r(v_new);
      hcnp = gate_it(hcnp, r.pinf, r.ptau, P[BC_P_HCN_PHI], dt);
      st[kSlotHcnP * N] = hcnp;
    }
    if (m & BC_M_AHP) {
      const Real ci = (m & BC_M_CADET) ? cahi + calo : P[BC_P_CA_CI0];
      const Real n = P[BC_P_AHP_N];
      const Real ci_n = n == Real(2) ? ci * ci : dpow(ci, n);
      ahpp = gate_ab(ahpp, P[BC_P_AHP_ALPHA] * ci_n, P[BC_P_AHP_BETA], P[BC_P_AHP_PHI], dt);
      st[kSlotAhpP * N] = ahpp;
    }
  }
  // currents at v_new
  const Real v = v_new;
  G = Real(0);
  I = Real(0);
  if (m & BC_M_IL) {
    const Real g = P[BC_P_IL_G];
    G += g;
    I += g * (P[BC_P_IL_E] - v);
  }
  if (m & BC_M_KLEAK) {
    const Real g = P[BC_P_KLEAK_G];
    G += g;
    I += g * (P[BC_P_EK] - v);
  }
  if (m & BC_M_NA) {
    const Real g = P[BC_P_NA_G] * nap * nap * nap * naq;
    G += g;
    I += g * (P[BC_P_ENA] - v);
  }
  if (m & BC_M_KDR) {
    const Real p2 = kdrp * kdrp;
    const Real g = P[BC_P_KDR_G] * p2 * p2;
    G += g;
    I += g * (P[BC_P_EK] - v);
  }
  if (m & (BC_M_CAL | BC_M_CAT)) {
    Real eca = P[BC_P_ECA];
    if (m & BC_M_CADET) eca = Real(kNernstCa) * P[BC_P_CA_TEMP] * dlog(P[BC_P_CA_CO] / (cahi + calo));
    if (m & BC_M_CAL) {
      const Real g = P[BC_P_CAL_G] * calp * calp * calq;
      G += g;
      I += g * (eca - v);
    }
    if (m & BC_M_CAT) {
      const Real g = P[BC_P_CAT_G] * catp * catp * catq;
      G += g;
      I += g * (eca - v);
    }
  }
  if (m & BC_M_HCN) {
    const Real g = P[BC_P_HCN_G] * hcnp;
    G += g;
    I += g * (P[BC_P_HCN_E] - v);
  }
  if (m & BC_M_AHP) {
    const Real g = P[BC_P_AHP_G] * ahpp * ahpp;
    G += g;
    I += g * (P[BC_P_EK] - v);
  }
}

template <typename Real>
__device__ __forceinline__ void node_mechanisms(Real* st, int N, const Real* P, uint32_t m, Real v_old, Real v_new,
                                                Real dt, bool advance, Real& G, Real& I) {
  NodeStates<Real> s;
  load_states(st, N, m, s);
  node_mechanisms_loaded(s, st, N, P, m, v_old, v_new, dt, advance, G, I);
}

// Steady state of every gate at v (HH.reset_state), Ci = Ci0.
template <typename Real>
__device__ __forceinline__ void steady_states(const Real* P, uint32_t m, Real* st, int N, Real v) {
  if (m & BC_M_CADET) {
    st[kSlotCaHi * N] = P[BC_P_CA_CI0];
    st[kSlotCaLo * N] = Real(0);
  }
  if (m & BC_M_NA) {
    const NaRates<Real> r(v, P[BC_P_NA_VSH]);
    st[kSlotNaP * N] = r.ap / (r.ap + r.bp);
    st[kSlotNaQ * N] = r.aq / (r.aq + r.bq);
  }
  if (m & BC_M_KDR) {
    const KdrRates<Real> r(v, P[BC_P_KDR_VSH]);
    st[kSlotKdrP * N] = r.a / (r.a + r.b);
  }
  if (m & BC_M_CAL) {
    const CaLRates<Real> r(v, P[BC_P_CAL_VSH]);
    st[kSlotCalP * N] = r.pinf;
    st[kSlotCalQ * N] = r.qinf;
  }
  if (m & BC_M_CAT) {
    const CaTRates<Real> r(v, P[BC_P_CAT_VSH]);
    st[kSlotCatP * N] = r.pinf;
    st[kSlotCatQ * N] = r.qinf;
  }
  if (m & BC_M_HCN) {
    const HcnRates<Real> r(v);
    st[kSlotHcnP * N] = r.pinf;
  }
  if (m & BC_M_AHP) {
    const Real ci = P[BC_P_CA_CI0];
    const Real n = P[BC_P_AHP_N];
    const Real a = P[BC_P_AHP_ALPHA] * (n == Real(2) ? ci * ci : dpow(ci, n));
    st[kSlotAhpP * N] = a / (a + P[BC_P_AHP_BETA]);
  }
}

// Row i of the next linear system: diag = 1 + dt (D + G / cm), rhs = dt I / cm
// on membrane rows; diag = dt D, rhs = 0 on boundary rows.
template <typename Real>
__device__ __forceinline__ void write_row(const TileView<Real>& tv, int i, uint16_t pr, Real dt, Real G, Real I) {
  if (pr == kBoundary) {
    tv.dr[i] = make_pair(dt * tv.diag0[i], Real(0));
  } else {
    const Real invcm = tv.params[size_t(pr) * BC_NPARAM + BC_P_INVCM];
    tv.dr[i] = make_pair(Real(1) + dt * (tv.diag0[i] + invcm * G), dt * invcm * I);
  }
}

// Clamp pulses active at `step` on node i (the thread that wrote row i adds them).
template <typename Real>
__device__ __forceinline__ void add_node_pulses(const TileView<Real>& tv, const PulseRec* pulses, const SpecRec& sr,
                                                int i, uint16_t pr, int64_t step, Real dt) {
  for (int k = sr.pulse_begin; k < sr.pulse_end; ++k) {
    const PulseRec p = pulses[k];
    if (step < p.on_step || step >= p.off_step) continue;
    if (pr == kBoundary)
      tv.dr[i].y += dt * Real(p.amp);
    else
      tv.dr[i].y += dt * tv.params[size_t(pr) * BC_NPARAM + BC_P_INVCM] * Real(p.amp);
  }
}

// ---------------------------------------------------------------- Hines sweeps
// Row i of the increment system (V_{n+1} = V_n + x):
//   d_i x_i - alpha_i x_parent - sum_c beta_c x_c = rhs_i - alpha_i Delta_i + sum_c beta_c Delta_c
// with Delta_i = V_i - V_parent (float-float).  Chains are walked bottom -> top;
// eliminating node i hands (cD, cR) = (alpha_i w, w r_i + beta_i Delta_i),
// w = beta_i / d_i, to its parent.  Per node a walk touches three pairs -- (d, r),
// (alpha dt, beta dt) and (V_hi, V_lo) -- loaded two nodes ahead, so that the
// shared-memory latency stays off the pivot recurrence.

__device__ __forceinline__ ChainRec load_rec(const ChainRec* recs, int c) {
  const int4* p = reinterpret_cast<const int4*>(recs + c);
  const int4 x = p[0], y = p[1];
  ChainRec r;
  r.start = x.x;
  r.count = x.y;
  r.top_parent = x.z;
  r.aux = x.w;
  r.n_child = y.x;
  r.kind = y.y;
  r.slot = y.z;
  r.first = y.w;
  return r;
}

// (alpha dt, beta dt) of node i: pre-scaled in shared-memory tiles, scaled here otherwise.
template <typename Real, bool kPre>
__device__ __forceinline__ Pair<Real> coef(const TileView<Real>& tv, int i, Real dt) {
  Pair<Real> c = tv.ab[i];
  if (!kPre) {
    c.x *= dt;
    c.y *= dt;
  }
  return c;
}

template <typename Real, bool kPre>
__device__ __forceinline__ void eliminate_regular(const TileView<Real>& tv, const ChainRec& ch, Real dt) {
  const int s0 = ch.start, end = ch.start + ch.count;
  Pair<Real> q = tv.dr[s0];
  Real D = q.x, R = q.y;
  for (int k = 0; k < ch.n_child; ++k) {
    D -= tv.scd[ch.aux + k];
    R += tv.scr[ch.aux + k];
  }
  Pair<Real> c = coef<Real, kPre>(tv, s0, dt), v = tv.v[s0];
  // node s0 + 1 (or the chain's parent, or -- at the root -- the node itself)
  const Pair<Real> v_top = ch.top_parent >= 0 ? tv.v[ch.top_parent] : tv.v[end - 1];
  Pair<Real> q1 = q, c1 = c, v1 = v_top;
  if (s0 + 1 < end) {
    q1 = tv.dr[s0 + 1];
    c1 = coef<Real, kPre>(tv, s0 + 1, dt);
    v1 = tv.v[s0 + 1];
  }
  for (int i = s0;; ++i) {
    Pair<Real> q2 = q1, c2 = c1, v2 = v_top;
    if (i + 2 < end) {
      q2 = tv.dr[i + 2];
      c2 = coef<Real, kPre>(tv, i + 2, dt);
      v2 = tv.v[i + 2];
    }
    const Real inv = pivot_rcp(D);
    const Real delta = (v.x - v1.x) + (v.y - v1.y);
    R -= c.x * delta;
    tv.dr[i] = make_pair(inv, R);
    const Real w = c.y * inv;
    if (i + 1 == end) {
      if (ch.slot >= 0) {
        tv.scd[ch.slot] = c.x * w;
        tv.scr[ch.slot] = w * R + c.y * delta;
      }
      break;
    }
    D = q1.x - c.x * w;
    R = q1.y + w * R + c.y * delta;
    c = c1;
    v = v1;
    q1 = q2;
    c1 = c2;
    v1 = v2;
  }
}

// One segment [a, b] of a split chain.  Nodes a .. b-1 are eliminated; the fill
// coefficient g_i of row i on x_o (o = top of the segment below) is kept in sfill,
// and the changes this causes in row o -- diagonal, right-hand side, and the
// coefficient H of x_b -- go to slot `slot` of scd / scr / sh.  Node b keeps its
// (not inverted) pivot for the reduced system.
template <typename Real, bool kPre>
__device__ __forceinline__ void eliminate_segment(const TileView<Real>& tv, const ChainRec& ch, Real dt) {
  const int a = ch.start, b = ch.start + ch.count - 1, end = b + 1;
  Pair<Real> q = tv.dr[a];
  Real D = q.x, R = q.y;
  Pair<Real> c = coef<Real, kPre>(tv, a, dt), v = tv.v[a];
  Real g = Real(0), h = Real(0), dd = Real(0), dr = Real(0);
  if (ch.first) {
    for (int k = 0; k < ch.n_child; ++k) {
      D -= tv.scd[ch.aux + k];
      R += tv.scr[ch.aux + k];
    }
  } else {
    const int o = ch.aux;
    const Pair<Real> co = coef<Real, kPre>(tv, o, dt);
    const Pair<Real> vo = tv.v[o];
    R += co.y * ((vo.x - v.x) + (vo.y - v.y));
    g = -co.y;
    h = -co.x;
  }
  const Pair<Real> v_top = ch.top_parent >= 0 ? tv.v[ch.top_parent] : tv.v[b];
  Pair<Real> q1 = q, c1 = c, v1 = v_top;
  if (a + 1 < end) {
    q1 = tv.dr[a + 1];
    c1 = coef<Real, kPre>(tv, a + 1, dt);
    v1 = tv.v[a + 1];
  }
  for (int i = a;; ++i) {
    Pair<Real> q2 = q1, c2 = c1, v2 = v_top;
    if (i + 2 < end) {
      q2 = tv.dr[i + 2];
      c2 = coef<Real, kPre>(tv, i + 2, dt);
      v2 = tv.v[i + 2];
    }
    const Real delta = (v.x - v1.x) + (v.y - v1.y);
    R -= c.x * delta;
    if (i == b) {
      tv.dr[i] = make_pair(D, R);
      tv.sfill[i] = g;
      break;
    }
    const Real inv = pivot_rcp(D);
    const Real w = c.y * inv;
    const Real hh = h * inv;
    dd -= hh * g;
    dr -= hh * R;
    h = hh * c.x;
    tv.dr[i] = make_pair(inv, R);
    tv.sfill[i] = g;
    D = q1.x - c.x * w;
    R = q1.y + w * R + c.y * delta;
    g = w * g;
    c = c1;
    v = v1;
    q1 = q2;
    c1 = c2;
    v1 = v2;
  }
  tv.scd[ch.slot] = dd;
  tv.scr[ch.slot] = dr;
  tv.sh[ch.slot] = h;
}

// Reduced system over the segment tops y_1 .. y_K (bottom to top):
//   row s: (d_s + dd_{s+1}) y_s + g_s y_{s-1} + H_{s+1} y_{s+1} = r_s + dr_{s+1}.
template <typename Real, bool kPre>
__device__ __forceinline__ void eliminate_reduced(const TileView<Real>& tv, const ChainRec& ch, Real dt) {
  const int K = ch.n_child;
  Real inv_prev = Real(0), f_prev = Real(0);
  int top = -1;
  ChainRec sg = load_rec(tv.chains, tv.child[ch.aux]);
  for (int s = 0; s < K; ++s) {
    top = sg.start + sg.count - 1;
    const Pair<Real> q = tv.dr[top];
    Real e = q.x, f = q.y;
    ChainRec up = sg;
    if (s + 1 < K) {
      up = load_rec(tv.chains, tv.child[ch.aux + s + 1]);
      e += tv.scd[up.slot];
      f += tv.scr[up.slot];
    }
    if (s > 0) {
      const Real mlt = tv.sfill[top] * inv_prev;
      e -= mlt * tv.sh[sg.slot];
      f -= mlt * f_prev;
    }
    inv_prev = pivot_rcp(e);
    f_prev = f;
    tv.dr[top] = make_pair(inv_prev, f);
    sg = up;
  }
  if (ch.slot >= 0) {
    const Pair<Real> c = coef<Real, kPre>(tv, top, dt);
    const Pair<Real> vt = tv.v[top], vp = tv.v[ch.top_parent];
    const Real w = c.y * inv_prev;
    tv.scd[ch.slot] = c.x * w;
    tv.scr[ch.slot] = w * f_prev + c.y * ((vt.x - vp.x) + (vt.y - vp.y));
  }
}

template <typename Real, bool kPre>
__device__ __forceinline__ void eliminate_rec(const TileView<Real>& tv, const ChainRec& ch, Real dt) {
  if (ch.kind == kChainRegular)
    eliminate_regular<Real, kPre>(tv, ch, dt);
  else if (ch.kind == kChainSegment)
    eliminate_segment<Real, kPre>(tv, ch, dt);
  else
    eliminate_reduced<Real, kPre>(tv, ch, dt);
}

template <typename Real, bool kPre>
__device__ __forceinline__ void backsub_rec(const TileView<Real>& tv, const ChainRec& ch, Real dt) {
  if (ch.kind == kChainReduced) {
    const int K = ch.n_child;
    ChainRec sg = load_rec(tv.chains, tv.child[ch.aux + K - 1]);
    int top = sg.start + sg.count - 1;
    const Real xp = ch.top_parent >= 0 ? tv.dr[ch.top_parent].y : Real(0);
    Pair<Real> q = tv.dr[top];
    Real y = (q.y + coef<Real, kPre>(tv, top, dt).x * xp) * q.x;
    tv.dr[top].y = y;
    for (int s = K - 2; s >= 0; --s) {
      const Real H = tv.sh[sg.slot];  // coefficient of y_{s+1} in row s, left by segment s+1
      sg = load_rec(tv.chains, tv.child[ch.aux + s]);
      top = sg.start + sg.count - 1;
      q = tv.dr[top];
      y = (q.y - H * y) * q.x;
      tv.dr[top].y = y;
    }
    return;
  }
  if (ch.kind == kChainSegment) {
    const int b = ch.start + ch.count - 1;
    if (b == ch.start) return;
    const Real yo = ch.first ? Real(0) : tv.dr[ch.aux].y;
    Real xn = tv.dr[b].y;
    int i = b - 1;
    Pair<Real> q = tv.dr[i];
    Real f = tv.sfill[i], al = coef<Real, kPre>(tv, i, dt).x;
    for (;; --i) {
      const bool nxt = i > ch.start;
      Pair<Real> qn = q;
      Real fn = Real(0), aln = Real(0);
      if (nxt) {
        qn = tv.dr[i - 1];
        fn = tv.sfill[i - 1];
        aln = coef<Real, kPre>(tv, i - 1, dt).x;
      }
      const Real x = (q.y - f * yo + al * xn) * q.x;
      tv.dr[i].y = x;
      xn = x;
      if (!nxt) break;
      q = qn;
      f = fn;
      al = aln;
    }
    return;
  }
  const int top = ch.start + ch.count - 1;
  Real dp = ch.top_parent >= 0 ? tv.dr[ch.top_parent].y : Real(0);
  Pair<Real> q = tv.dr[top];
  Real al = coef<Real, kPre>(tv, top, dt).x;
  Pair<Real> q1 = q;
  Real al1 = al;
  if (top - 1 >= ch.start) {
    q1 = tv.dr[top - 1];
    al1 = coef<Real, kPre>(tv, top - 1, dt).x;
  }
  for (int i = top;; --i) {
    Pair<Real> q2 = q1;
    Real al2 = al1;
    if (i - 2 >= ch.start) {
      q2 = tv.dr[i - 2];
      al2 = coef<Real, kPre>(tv, i - 2, dt).x;
    }
    const Real x = (q.y + al * dp) * q.x;
    tv.dr[i].y = x;
    dp = x;
    if (i == ch.start) break;
    q = q1;
    al = al1;
    q1 = q2;
    al1 = al2;
  }
}

// A thread's records of one phase, with the next record prefetched.
template <typename Real, bool kPre>
__device__ __forceinline__ void eliminate_list(const TileView<Real>& tv, int c0, int c1, Real dt) {
  if (c0 >= c1) return;
  ChainRec ch = load_rec(tv.chains, c0);
  for (int c = c0;; ++c) {
    const bool more = c + 1 < c1;
    ChainRec nx = ch;
    if (more) nx = load_rec(tv.chains, c + 1);
    eliminate_rec<Real, kPre>(tv, ch, dt);
    if (!more) break;
    ch = nx;
  }
}

template <typename Real, bool kPre>
__device__ __forceinline__ void backsub_list(const TileView<Real>& tv, int c0, int c1, Real dt) {
  if (c0 >= c1) return;
  ChainRec ch = load_rec(tv.chains, c1 - 1);
  for (int c = c1 - 1;; --c) {
    const bool more = c > c0;
    ChainRec nx = ch;
    if (more) nx = load_rec(tv.chains, c - 1);
    backsub_rec<Real, kPre>(tv, ch, dt);
    if (!more) break;
    ch = nx;
  }
}

template <typename Real>
__device__ __forceinline__ bool is_finite_real(Real x) {
  return isfinite(x);
}

// ------------------------------------------------------------------ the step kernel
template <typename Real, bool kSmem>
__global__ void __launch_bounds__(1024) tile_step_kernel(LaunchArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ int s_status;
  const TileDesc td = a.tiles[blockIdx.x];
  unsigned char* gblob = a.blob + td.blob_offset;
  unsigned char* base;
  unsigned char* scratch;
  if (threadIdx.x == 0) s_status = 0;
  if constexpr (kSmem) {
    base = smem;
    scratch = smem + td.blob_bytes;
    if (threadIdx.x == 0) {
      mbar_init(&bar, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      mbar_expect_tx(&bar, uint32_t(td.blob_bytes));
      for (uint32_t off = 0; off < uint32_t(td.blob_bytes); off += kBulkChunk) {
        const uint32_t n = min(kBulkChunk, uint32_t(td.blob_bytes) - off);
        bulk_g2s(smem + off, gblob + off, n, &bar);
      }
    }
    // Bounded wait; the give-up decision is made block-wide so that no thread is
    // left at a barrier that others skip.
    const int ok = __syncthreads_and(mbar_wait(&bar, 0, 1u << 22) ? 1 : 0);
    if (!ok) {
      // The copy never completed: record, wait once more (bounded) and leave.
      if (threadIdx.x == 0) {
        atomicOr(a.status, kStatusTimeout);
        mbar_wait(&bar, 0, 1u << 22);
      }
      return;
    }
  } else {
    base = gblob;
    scratch = a.scratch + td.scratch_offset;
    __syncthreads();
  }
  TileView<Real> tv;
  tv.bind(td, base, scratch, a.state);
  const Real dt = Real(a.dt);
  const int T = blockDim.x, tid = threadIdx.x;
  const PulseRec* pulses = a.pulses + td.pulse_offset;
  if constexpr (kSmem) {
    // the staged axial coefficients become (alpha dt, beta dt) for this launch
    for (int i = tid; i < tv.N; i += T) {
      Pair<Real> c = tv.ab[i];
      c.x *= dt;
      c.y *= dt;
      tv.ab[i] = c;
    }
  }

  // Prologue: the linear system of the first step from the current state.
  for (int i = tid; i < tv.n_real; i += T) {
    const uint16_t pr = tv.pidx[i];
    Real G = Real(0), I = Real(0);
    if (pr != kBoundary) {
      const Real v = tv.v[i].x;
      node_mechanisms(tv.state + i, tv.N, tv.params + size_t(pr) * BC_NPARAM, tv.mech[pr], v, v, dt, false, G, I);
    }
    write_row(tv, i, pr, dt, G, I);
    const uint16_t sp = tv.spec[i];
    if (sp != kNoSpecial) add_node_pulses(tv, pulses, tv.specs[sp], i, pr, a.step0, dt);
  }
  __syncthreads();

#ifdef BC_PHASE_TIMERS
  unsigned long long tm[4] = {0, 0, 0, 0};
  long long t_prev = clock64();
#define BC_TICK(slot)                                 \
  do {                                                \
    const long long t_now = clock64();                \
    tm[slot] += (unsigned long long)(t_now - t_prev); \
    t_prev = t_now;                                   \
  } while (0)
#else
#define BC_TICK(slot) \
  do {                \
  } while (0)
#endif
  for (int s = 0; s < a.n_steps; ++s) {
    const int64_t step = a.step0 + s;
    // forward elimination, leaves first
    for (int p = 0; p < tv.n_phases; ++p) {
      eliminate_list<Real, kSmem>(tv, tv.lists[p * (T + 1) + tid], tv.lists[p * (T + 1) + tid + 1], dt);
      __syncthreads();
    }
    BC_TICK(0);
    // back-substitution, root first
    for (int p = tv.n_phases - 1; p >= 0; --p) {
      backsub_list<Real, kSmem>(tv, tv.lists[p * (T + 1) + tid], tv.lists[p * (T + 1) + tid + 1], dt);
      __syncthreads();
    }
    BC_TICK(1);
    // V update, mechanism states, next row, probes and next pulses
    const bool last = s + 1 == a.n_steps;
    const int64_t k_since = step + 1 - a.trace_base;
    const bool record = a.record_every > 0 && k_since % a.record_every == 0;
    // The states live in global memory (L2): the next node's are loaded one
    // iteration ahead so that their latency overlaps this node's arithmetic.
    NodeStates<Real> cur;
    uint16_t pr_cur = kBoundary;
    if (tid < tv.n_real) {
      pr_cur = tv.pidx[tid];
      if (pr_cur != kBoundary) load_states(tv.state + tid, tv.N, tv.mech[pr_cur], cur);
    }
    for (int i = tid; i < tv.n_real; i += T) {
      NodeStates<Real> nxt;
      uint16_t pr_nxt = kBoundary;
      if (i + T < tv.n_real) {
        pr_nxt = tv.pidx[i + T];
        if (pr_nxt != kBoundary) load_states(tv.state + i + T, tv.N, tv.mech[pr_nxt], nxt);
      }
      const Pair<Real> vv = tv.v[i];
      Real hi = vv.x, lo = vv.y;
      const Real v_old = hi, lo_old = lo;
      ff_add(hi, lo, tv.dr[i].y);
      tv.v[i] = make_pair(hi, lo);
      if (!is_finite_real(hi)) s_status = kStatusNonfinite;
      const uint16_t pr = pr_cur;
      Real G = Real(0), I = Real(0);
      if (pr != kBoundary)
        node_mechanisms_loaded(cur, tv.state + i, tv.N, tv.params + size_t(pr) * BC_NPARAM, tv.mech[pr], v_old, hi, dt,
                               true, G, I);
      cur = nxt;
      pr_cur = pr_nxt;
      if (!last) write_row(tv, i, pr, dt, G, I);
      const uint16_t sp = tv.spec[i];
      if (sp != kNoSpecial) {
        const SpecRec sr = tv.specs[sp];
        if (sr.probe >= 0) {
          const double v1 = double(hi) + double(lo), v0 = double(v_old) + double(lo_old);
          if (v0 < 0.0 && v1 >= 0.0) {
            const int n = a.spike_count[sr.probe];
            if (n < a.max_spikes)
              a.spike_times[int64_t(sr.probe) * a.max_spikes + n] = double(step) * a.dt + a.dt * (0.0 - v0) / (v1 - v0);
            a.spike_count[sr.probe] = n + 1;
          }
          if (record) {
            const int64_t slot = k_since / a.record_every - 1;
            if (slot >= 0 && slot < a.trace_cap) a.traces[slot * a.n_probes_total + sr.probe] = v1;
          }
        }
        if (!last) add_node_pulses(tv, pulses, sr, i, pr, step + 1, dt);
      }
    }
    __syncthreads();
    BC_TICK(2);
  }
#ifdef BC_PHASE_TIMERS
  if (threadIdx.x == 0 && a.timers)
    for (int q = 0; q < 4; ++q) atomicAdd(a.timers + q, tm[q]);
#endif
  if (s_status) atomicOr(a.status, s_status);

  if constexpr (kSmem) {
    fence_proxy_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      for (uint32_t off = 0; off < uint32_t(td.dyn_bytes); off += kBulkChunk) {
        const uint32_t n = min(kBulkChunk, uint32_t(td.dyn_bytes) - off);
        bulk_s2g(gblob + off, smem + off, n);
      }
      bulk_commit_and_wait();
    }
  }
}

// Reset: V from the initial image, gates at steady state, Ci = Ci0.
template <typename Real>
__global__ void reset_kernel(LaunchArgs a, const double* vinit, const int64_t* vinit_off) {
  const TileDesc td = a.tiles[blockIdx.x];
  unsigned char* base = a.blob + td.blob_offset;
  TileView<Real> tv;
  tv.bind(td, base, base, a.state);  // scratch unused
  const double* vi = vinit + vinit_off[blockIdx.x];
  for (int i = threadIdx.x; i < tv.n_real; i += blockDim.x) {
    const Real v = Real(vi[i]);
    tv.v[i] = make_pair(v, Real(0));
    const uint16_t pr = tv.pidx[i];
    if (pr == kBoundary) continue;
    const Real* P = tv.params + size_t(pr) * BC_NPARAM;
    steady_states(P, tv.mech[pr], tv.state + i, tv.N, v);
  }
}

// Gather (write = false) or scatter (write = true) one named view.
__device__ __forceinline__ unsigned char* view_addr(unsigned char* blob, unsigned char* state, int64_t off) {
  return off >= kStateTag ? state + (off - kStateTag) : blob + off;
}

template <typename Real>
__global__ void view_kernel(unsigned char* blob, unsigned char* state, const int64_t* off_hi, const int64_t* off_lo,
                            double* view, int64_t n, bool write) {
  for (int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; k < n; k += int64_t(gridDim.x) * blockDim.x) {
    const int64_t oh = off_hi[k], ol = off_lo[k];
    if (oh < 0) {
      if (!write) view[k] = __longlong_as_double(0x7ff8000000000000LL);
      continue;
    }
    Real* hi = reinterpret_cast<Real*>(view_addr(blob, state, oh));
    Real* lo = ol >= 0 ? reinterpret_cast<Real*>(view_addr(blob, state, ol)) : nullptr;
    if (write) {
      *hi = Real(view[k]);
      if (lo) *lo = Real(view[k] - double(*hi));
    } else {
      view[k] = double(*hi) + (lo ? double(*lo) : 0.0);
    }
  }
}

// ------------------------------------------------------------------ launchers
template <typename Real, bool kSmem>
static int launch_impl(const LaunchArgs& a, int threads, size_t smem_bytes, cudaStream_t st) {
  auto k = tile_step_kernel<Real, kSmem>;
  if (kSmem) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_bytes));
    if (e != cudaSuccess) return int(e);
  }
  dim3 grid(a.n_tiles, 1, 1);
  k<<<grid, threads, kSmem ? smem_bytes : 0, st>>>(a);
  return int(cudaGetLastError());
}

int launch_tiles(const LaunchArgs& a, int precision, bool smem, int threads, size_t smem_bytes, void* stream) {
  if (a.n_tiles <= 0) return 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (precision == BC_PREC_F64)
    return smem ? launch_impl<double, true>(a, threads, smem_bytes, st)
                : launch_impl<double, false>(a, threads, smem_bytes, st);
  return smem ? launch_impl<float, true>(a, threads, smem_bytes, st)
              : launch_impl<float, false>(a, threads, smem_bytes, st);
}

int launch_reset_impl(const LaunchArgs& a, int precision, int threads, const double* vinit, const int64_t* voff,
                      void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (a.n_tiles <= 0) return 0;
  if (precision == BC_PREC_F64)
    reset_kernel<double><<<a.n_tiles, threads, 0, st>>>(a, vinit, voff);
  else
    reset_kernel<float><<<a.n_tiles, threads, 0, st>>>(a, vinit, voff);
  return int(cudaGetLastError());
}

int launch_view_impl(unsigned char* blob, unsigned char* state, int precision, const int64_t* off_hi,
                     const int64_t* off_lo, double* view, int64_t n, bool write, void* stream) {
  if (n <= 0) return 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int threads = 256;
  const int64_t blocks = std::min<int64_t>((n + threads - 1) / threads, 65535);
  if (precision == BC_PREC_F64)
    view_kernel<double><<<int(blocks), threads, 0, st>>>(blob, state, off_hi, off_lo, view, n, write);
  else
    view_kernel<float><<<int(blocks), threads, 0, st>>>(blob, state, off_hi, off_lo, view, n, write);
  return int(cudaGetLastError());
}

// Scratch of bc_state_download_noalloc, part of the module image (no allocation
// call): three 8-byte arrays of BC_NOALLOC_MAX_CV entries, 256-byte aligned.
static __device__ __align__(256) unsigned char g_noalloc_view_scratch[3 * 8 * size_t(BC_NOALLOC_MAX_CV)];

int noalloc_view_scratch_address(void** out) {
  return int(cudaGetSymbolAddress(out, g_noalloc_view_scratch));
}

}  // namespace bc
