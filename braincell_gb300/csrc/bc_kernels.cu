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

#include "bc_gru.cuh"
#include "bc_internal.h"
#include "bc_mech.cuh"
#include "bc_ext.cuh"

namespace bc {

constexpr int kStatusNonfinite = 1;
constexpr int kStatusTimeout = 2;
constexpr int kStatusRecordOverflow = 4;
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
  const SlotRec* slots;   // warp slots, phase by phase
  const int32_t* phase;    // [n_phases + 1] slot ranges
  const uint16_t *pidx, *spec, *crec;
  const ChainRec* chains;
  const SpecRec* specs;
  const uint32_t* mech;
  Real *scd, *scr;
  const int32_t* syn;       // tile synapse list (global synapse ids)
  const uint16_t* ncell;    // per node: tile-local cell (spike-source tiles only)
  const int32_t* srccell;   // per tile cell: global id of a spike source, -1 otherwise
  int32_t* stamp;           // per tile cell: last step with a crossing
  int N, n_real, n_phases, n_cells;
  int pstride;  // reals per parameter record
  bool has_src;

  __device__ __forceinline__ void bind(const TileDesc& td, unsigned char* base, unsigned char* scratch, void* gstate) {
    v = reinterpret_cast<Pair<Real>*>(base + td.off_v);
    ab = reinterpret_cast<Pair<Real>*>(base + td.off_ab);
    dr = reinterpret_cast<Pair<Real>*>(scratch + td.off_dr);
    state = reinterpret_cast<Real*>(gstate) + td.state_offset;
    diag0 = reinterpret_cast<const Real*>(base + td.off_diag0);
    params = reinterpret_cast<const Real*>(base + td.off_params);
    slots = reinterpret_cast<const SlotRec*>(base + td.off_slots);
    phase = reinterpret_cast<const int32_t*>(base + td.off_phase);
    crec = reinterpret_cast<const uint16_t*>(base + td.off_crec);
    pidx = reinterpret_cast<const uint16_t*>(base + td.off_pidx);
    spec = reinterpret_cast<const uint16_t*>(base + td.off_spec);
    chains = reinterpret_cast<const ChainRec*>(base + td.off_chains);
    specs = reinterpret_cast<const SpecRec*>(base + td.off_specs);
    mech = reinterpret_cast<const uint32_t*>(base + td.off_mech);
    scd = reinterpret_cast<Real*>(scratch + td.off_scd);
    scr = reinterpret_cast<Real*>(scratch + td.off_scr);
    syn = reinterpret_cast<const int32_t*>(base + td.off_syn);
    has_src = td.off_ncell >= 0;
    ncell = has_src ? reinterpret_cast<const uint16_t*>(base + td.off_ncell) : nullptr;
    srccell = has_src ? reinterpret_cast<const int32_t*>(base + td.off_srccell) : nullptr;
    stamp = has_src ? reinterpret_cast<int32_t*>(scratch + td.off_stamp) : nullptr;
    n_cells = td.n_cells;
    pstride = td.param_stride;
    N = td.n_nodes;
    n_real = td.n_real_nodes;
    n_phases = td.n_phases;
  }
};

// Reciprocal of a Hines pivot.  FP32: the hardware approximation (about 1 ulp;
// pivots are >= 1 on membrane rows and O(dt * g / C) on boundary rows, far from
// the denormal range); FP64: IEEE round-to-nearest.
__device__ __forceinline__ float pivot_rcp(float d) { return rcp_approx(d); }
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

// The cerebellar calcium channels' current density at v from the states in st and
// the calcium reversal potential eca: the step-start current the calcium shell
// integrates (with CaL and CaT), and the ohmic terms of the row.
template <typename Real>
__device__ __forceinline__ Real cerebellar_ca_current(const Real* st, int N, const Real* P, uint32_t m, Real v, Real eca,
                                                      Real* g_out) {
  Real g = Real(0);
  if (m & BC_M_CAHVA) {
    const Real s = st[kSlotCaHvaS * N];
    g += P[BC_P_CAHVA_G] * s * s * st[kSlotCaHvaU * N];
  }
  if (m & BC_M_CAV23) {
    const Real a = st[kSlotCav23M * N];
    g += P[BC_P_CAV23_G] * a * a * a * st[kSlotCav23H * N];
  }
  if (m & BC_M_CAV32) {
    const Real a = st[kSlotCav32M * N];
    g += P[BC_P_CAV32_G] * a * a * st[kSlotCav32H * N];
  }
  if (g_out) *g_out = g;
  return g * (eca - v);
}

// The value a mechanism probe records: state view `field` (a BC_STATE_* other
// than V) of the node whose states start at st, after the node's update.
template <typename Real>
__device__ __forceinline__ double probe_state(const Real* st, int N, int field) {
  if (field == BC_STATE_CA_CI) return double(st[kSlotCaHi * N]) + double(st[kSlotCaLo * N]);
  // slots 9, 10 hold Ci; the Markov views 25.. sit one above their slots 26..
  const int slot = field <= BC_STATE_AHP_P ? field - 1 : (field >= BC_STATE_NAV16_C1 ? field + 1 : field);
  return double(st[slot * N]);
}

// The value a current probe records: current density `code` (BC_CUR_*, uA/cm^2)
// of the node whose states start at st, at voltage v after the node's update,
// with the same terms as the step's currents.
template <typename Real>
__device__ __forceinline__ double probe_current(const Real* st, int N, const Real* P, uint32_t m, Real v, int code) {
  auto eca = [&]() -> Real {
    if (m & BC_M_CADET)
      return Real(kNernstCa) * P[BC_P_CA_TEMP] * dlog(P[BC_P_CA_CO] / (st[kSlotCaHi * N] + st[kSlotCaLo * N]));
    return P[BC_P_ECA];
  };
  auto cur = [&](int c) -> Real {
    switch (c) {
      case BC_CUR_IL:
        return (m & BC_M_IL) ? P[BC_P_IL_G] * (P[BC_P_IL_E] - v) : Real(0);
      case BC_CUR_KLEAK:
        return (m & BC_M_KLEAK) ? P[BC_P_KLEAK_G] * (P[BC_P_EK] - v) : Real(0);
      case BC_CUR_NA: {
        if (!(m & BC_M_NA)) return Real(0);
        const Real p = st[kSlotNaP * N];
        return P[BC_P_NA_G] * p * p * p * st[kSlotNaQ * N] * (P[BC_P_ENA] - v);
      }
      case BC_CUR_KDR: {
        if (!(m & BC_M_KDR)) return Real(0);
        const Real p2 = st[kSlotKdrP * N] * st[kSlotKdrP * N];
        return P[BC_P_KDR_G] * p2 * p2 * (P[BC_P_EK] - v);
      }
      case BC_CUR_CAL: {
        if (!(m & BC_M_CAL)) return Real(0);
        const Real p = st[kSlotCalP * N];
        return P[BC_P_CAL_G] * p * p * st[kSlotCalQ * N] * (eca() - v);
      }
      case BC_CUR_CAT: {
        if (!(m & BC_M_CAT)) return Real(0);
        const Real p = st[kSlotCatP * N];
        return P[BC_P_CAT_G] * p * p * st[kSlotCatQ * N] * (eca() - v);
      }
      case BC_CUR_HCN:
        return (m & BC_M_HCN) ? P[BC_P_HCN_G] * st[kSlotHcnP * N] * (P[BC_P_HCN_E] - v) : Real(0);
      case BC_CUR_AHP: {
        if (!(m & BC_M_AHP)) return Real(0);
        const Real p = st[kSlotAhpP * N];
        return P[BC_P_AHP_G] * p * p * (P[BC_P_EK] - v);
      }
      case BC_CUR_NAHH: {
        if (!(m & BC_M_NAHH)) return Real(0);
        const Real p = st[kSlotNaHHP * N];
        return P[BC_P_NAHH_G] * p * p * p * st[kSlotNaHHQ * N] * (P[BC_P_ENA] - v);
      }
      case BC_CUR_KHH: {
        if (!(m & BC_M_KHH)) return Real(0);
        const Real p2 = st[kSlotKHHP * N] * st[kSlotKHHP * N];
        return P[BC_P_KHH_G] * p2 * p2 * (P[BC_P_EK] - v);
      }
      case BC_CUR_KM:
        return (m & BC_M_KM) ? P[BC_P_KM_G] * st[kSlotKMN * N] * (P[BC_P_EK] - v) : Real(0);
      case BC_CUR_KA1: {
        if (!(m & BC_M_KA1)) return Real(0);
        const Real p2 = st[kSlotKA1P * N] * st[kSlotKA1P * N];
        return P[BC_P_KA1_G] * p2 * p2 * st[kSlotKA1Q * N] * (P[BC_P_EK] - v);
      }
      case BC_CUR_KA2: {
        if (!(m & BC_M_KA2)) return Real(0);
        const Real p2 = st[kSlotKA2P * N] * st[kSlotKA2P * N];
        return P[BC_P_KA2_G] * p2 * p2 * st[kSlotKA2Q * N] * (P[BC_P_EK] - v);
      }
      case BC_CUR_KK2A:
        return (m & BC_M_KK2A) ? P[BC_P_KK2A_G] * st[kSlotKK2AP * N] * st[kSlotKK2AQ * N] * (P[BC_P_EK] - v) : Real(0);
      case BC_CUR_KK2B:
        return (m & BC_M_KK2B) ? P[BC_P_KK2B_G] * st[kSlotKK2BP * N] * st[kSlotKK2BQ * N] * (P[BC_P_EK] - v) : Real(0);
      case BC_CUR_KNI:
        return (m & BC_M_KNI) ? P[BC_P_KNI_G] * st[kSlotKNIP * N] * (P[BC_P_EK] - v) : Real(0);
      case BC_CUR_NAV16:
        return (m & BC_M_NAV16) ? P[BC_P_NAV16_G] * st[(kSlotNav16 + 10) * N] * (P[BC_P_ENA] - v) : Real(0);
      case BC_CUR_KCA22:
        return (m & BC_M_KCA22)
                   ? P[BC_P_KCA22_G] * (st[(kSlotKca22 + 3) * N] + st[(kSlotKca22 + 4) * N]) * (P[BC_P_EK] - v)
                   : Real(0);
      case BC_CUR_KCA11: {
        if (!(m & BC_M_KCA11)) return Real(0);
        Real o = Real(0);
        for (int k = 4; k < 9; ++k) o += st[(kSlotKca11 + k) * N];
        return P[BC_P_KCA11_G] * o * (P[BC_P_EK] - v);
      }
      case BC_CUR_KV34: {
        if (!(m & BC_M_KV34)) return Real(0);
        const Real a = st[kSlotKv34M * N];
        return P[BC_P_KV34_G] * a * a * a * st[kSlotKv34H * N] * (P[BC_P_EK] - v);
      }
      case BC_CUR_KV43: {
        if (!(m & BC_M_KV43)) return Real(0);
        const Real a = st[kSlotKv43A * N];
        return P[BC_P_KV43_G] * a * a * a * st[kSlotKv43B * N] * (P[BC_P_EK] - v);
      }
      case BC_CUR_KV11: {
        if (!(m & BC_M_KV11)) return Real(0);
        const Real n2 = st[kSlotKv11N * N] * st[kSlotKv11N * N];
        return P[BC_P_KV11_G] * n2 * n2 * (P[BC_P_EK] - v);
      }
      case BC_CUR_KIR23:
        return (m & BC_M_KIR23) ? P[BC_P_KIR23_G] * st[kSlotKir23D * N] * (P[BC_P_EK] - v) : Real(0);
      case BC_CUR_HCN1F:
        return (m & BC_M_HCN1F)
                   ? P[BC_P_HCN1F_G] * (st[kSlotHcn1Fast * N] + st[kSlotHcn1Slow * N]) * (P[BC_P_HCN1F_E] - v)
                   : Real(0);
      case BC_CUR_HCN1H:
        return (m & BC_M_HCN1H) ? P[BC_P_HCN1H_G] * st[kSlotHcn1H * N] * (P[BC_P_HCN1H_E] - v) : Real(0);
      case BC_CUR_CAHVA:
        return cerebellar_ca_current(st, N, P, m & BC_M_CAHVA, v, eca(), (Real*)nullptr);
      case BC_CUR_CAV23:
        return cerebellar_ca_current(st, N, P, m & BC_M_CAV23, v, eca(), (Real*)nullptr);
      case BC_CUR_CAV32:
        return cerebellar_ca_current(st, N, P, m & BC_M_CAV32, v, eca(), (Real*)nullptr);
      default:
        // extension channels: the record's list exists only where BC_M_EXT is set
        if (c >= BC_CUR_HCN2 && c <= BC_CUR_CALVADCN && (m & BC_M_EXT)) {
          const Real ci = (m & BC_M_CADET) ? st[kSlotCaHi * N] + st[kSlotCaLo * N] : P[BC_P_CA_CI0];
          const bool ohmic_ca = c == BC_CUR_CATHP || c == BC_CUR_CAHTRE || c == BC_CUR_CAV12 || c == BC_CUR_CAV13;
          return ext_current(st, N, P, ext_mask(P), v, ci, ohmic_ca ? eca() : Real(0),
                             c, (Real*)nullptr);
        }
    }
    return Real(0);
  };
  switch (code) {
    case BC_CUR_ION_NA:
      return double(cur(BC_CUR_NA)) + double(cur(BC_CUR_NAHH)) + double(cur(BC_CUR_NAV16)) + double(cur(BC_CUR_NAF)) +
             double(cur(BC_CUR_NAP)) + double(cur(BC_CUR_NAIO)) + double(cur(BC_CUR_NAVGRC));
    case BC_CUR_ION_K:
      return double(cur(BC_CUR_KDR)) + double(cur(BC_CUR_KLEAK)) + double(cur(BC_CUR_AHP)) + double(cur(BC_CUR_KHH)) +
             double(cur(BC_CUR_KM)) + double(cur(BC_CUR_KA1)) + double(cur(BC_CUR_KA2)) + double(cur(BC_CUR_KK2A)) +
             double(cur(BC_CUR_KK2B)) + double(cur(BC_CUR_KNI)) + double(cur(BC_CUR_KCA22)) + double(cur(BC_CUR_KCA11)) +
             double(cur(BC_CUR_KV34)) + double(cur(BC_CUR_KV43)) + double(cur(BC_CUR_KV11)) + double(cur(BC_CUR_KIR23)) +
             double(cur(BC_CUR_KV33)) + double(cur(BC_CUR_KV22)) + double(cur(BC_CUR_KV15)) + double(cur(BC_CUR_FKDR)) +
             double(cur(BC_CUR_SKDR)) + double(cur(BC_CUR_KDRIO)) + double(cur(BC_CUR_KCA31)) + double(cur(BC_CUR_SKDCN)) +
             double(cur(BC_CUR_KKV));
    case BC_CUR_ION_CA:
      return double(cur(BC_CUR_CAL)) + double(cur(BC_CUR_CAT)) + double(cur(BC_CUR_CAHVA)) + double(cur(BC_CUR_CAV23)) +
             double(cur(BC_CUR_CAV32)) + double(cur(BC_CUR_CATHP)) + double(cur(BC_CUR_CAHTRE)) + double(cur(BC_CUR_CAN)) +
             double(cur(BC_CUR_CAV31)) + double(cur(BC_CUR_CAV33)) + double(cur(BC_CUR_CAV12)) + double(cur(BC_CUR_CAV13)) +
             double(cur(BC_CUR_CAV21)) + double(cur(BC_CUR_CAHVADCN)) + double(cur(BC_CUR_CALVADCN));
    default:
      return double(cur(code));
  }
}

// Channels outside the main workloads' mix (classic Hodgkin-Huxley Na / K, the
// M current, the A current, the slow K2 current, the slow non-inactivating K
// current): kept out of line so that their registers do not weigh on the common
// path; same exp-Euler steps and ohmic currents as the others.
constexpr uint32_t kCerebellarCaChannels = BC_M_CAHVA | BC_M_CAV23 | BC_M_CAV32;
constexpr uint32_t kCerebellarChannels =
    BC_M_KV34 | BC_M_KV43 | BC_M_KV11 | BC_M_KIR23 | BC_M_HCN1F | BC_M_HCN1H | kCerebellarCaChannels;
constexpr uint32_t kExtraChannels = BC_M_NAHH | BC_M_KHH | BC_M_KM | BC_M_KA1 | BC_M_KA2 | BC_M_KK2A | BC_M_KK2B |
                                   BC_M_KNI | BC_M_NAV16 | BC_M_KCA22 | BC_M_KCA11 | kCerebellarChannels | BC_M_EXT;

__device__ __forceinline__ MarkovGraph nav16_graph() { return MarkovGraph{13, 17, 12, kSlotNav16, kNav16Src, kNav16Dst}; }
__device__ __forceinline__ MarkovGraph kca22_graph() { return MarkovGraph{6, 5, 0, kSlotKca22, kKca22Src, kKca22Dst}; }
__device__ __forceinline__ MarkovGraph kca11_graph() { return MarkovGraph{10, 13, 0, kSlotKca11, kKca11Src, kKca11Dst}; }

// One A-current mechanism (p^4 q, E_K) in slots (sp, sq) with parameters from pg.
template <typename Real>
__device__ __forceinline__ void a_current(Real* st, int N, const Real* P, int sp, int sq, int pg, Real mid,
                                          Real inv_slope, Real v, Real dt, bool advance, Real& G, Real& I) {
  Real p = st[sp * N], q = st[sq * N];
  if (advance) {
    const KARates<Real> r(v, P[pg + 1], mid, inv_slope);
    p = gate_it(p, r.pinf, r.ptau, P[pg + 2], dt);
    q = gate_it(q, r.qinf, r.qtau, P[pg + 3], dt);
    st[sp * N] = p;
    st[sq * N] = q;
  }
  const Real p2 = p * p;
  const Real g = P[pg] * p2 * p2 * q;
  G += g;
  I += g * (P[BC_P_EK] - v);
}

// One slow K2 mechanism (p q, E_K) in slots (sp, sq) with parameters from pg.
template <typename Real>
__device__ __forceinline__ void k2_current(Real* st, int N, const Real* P, int sp, int sq, int pg, bool b_form, Real v,
                                           Real dt, bool advance, Real& G, Real& I) {
  Real p = st[sp * N], q = st[sq * N];
  if (advance) {
    const K2Rates<Real> r(v, P[pg + 1], b_form);
    p = gate_it(p, r.pinf, r.ptau, P[pg + 2], dt);
    q = gate_it(q, r.qinf, r.qtau, P[pg + 3], dt);
    st[sp * N] = p;
    st[sq * N] = q;
  }
  const Real g = P[pg] * p * q;
  G += g;
  I += g * (P[BC_P_EK] - v);
}

// The cerebellar HH channels: exp-Euler gates at v, ohmic currents (HCN1 with its
// own reversal potential; HCN1_MA2020_GoC's g carries its Q10 factor already; the
// calcium channels in E_Ca of the calcium ci after this step's shell update).
template <typename Real>
__device__ __forceinline__ void cerebellar_channels(Real* st, int N, const Real* P, uint32_t m, Real v, Real ci,
                                                    Real dt, bool advance, Real& G, Real& I) {
  if (m & BC_M_KV34) {
    Real a = st[kSlotKv34M * N], b = st[kSlotKv34H * N];
    if (advance) {
      const Kv34Rates<Real> r(v);
      a = gate_it(a, r.minf, r.mtau, P[BC_P_KV34_PHI], dt);
      b = gate_it(b, r.hinf, r.htau, P[BC_P_KV34_PHI], dt);
      st[kSlotKv34M * N] = a;
      st[kSlotKv34H * N] = b;
    }
    const Real g = P[BC_P_KV34_G] * a * a * a * b;
    G += g;
    I += g * (P[BC_P_EK] - v);
  }
  if (m & BC_M_KV43) {
    Real a = st[kSlotKv43A * N], b = st[kSlotKv43B * N];
    if (advance) {
      const Kv43Rates<Real> r(v);
      a = gate_it(a, r.ainf, r.atau, P[BC_P_KV43_PHI], dt);
      b = gate_it(b, r.binf, r.btau, P[BC_P_KV43_PHI], dt);
      st[kSlotKv43A * N] = a;
      st[kSlotKv43B * N] = b;
    }
    const Real g = P[BC_P_KV43_G] * a * a * a * b;
    G += g;
    I += g * (P[BC_P_EK] - v);
  }
  if (m & BC_M_KV11) {
    Real n = st[kSlotKv11N * N];
    if (advance) {
      const Kv11Rates<Real> r(v);
      n = gate_ab<Real, true>(n, r.a, r.b, P[BC_P_KV11_PHI], dt);
      st[kSlotKv11N * N] = n;
    }
    const Real n2 = n * n;
    const Real g = P[BC_P_KV11_G] * n2 * n2;
    G += g;
    I += g * (P[BC_P_EK] - v);
  }
  if (m & BC_M_KIR23) {
    Real d = st[kSlotKir23D * N];
    if (advance) {
      const Kir23Rates<Real> r(v);
      d = gate_ab<Real, true>(d, r.a, r.b, P[BC_P_KIR23_PHI], dt);
      st[kSlotKir23D * N] = d;
    }
    const Real g = P[BC_P_KIR23_G] * d;
    G += g;
    I += g * (P[BC_P_EK] - v);
  }
  if (m & BC_M_HCN1F) {
    Real f = st[kSlotHcn1Fast * N], sl = st[kSlotHcn1Slow * N];
    if (advance) {
      const Hcn1fRates<Real> r(v);
      f = gate_it(f, r.finf, r.ftau, P[BC_P_HCN1F_PHI], dt);
      sl = gate_it(sl, r.sinf, r.stau, P[BC_P_HCN1F_PHI], dt);
      st[kSlotHcn1Fast * N] = f;
      st[kSlotHcn1Slow * N] = sl;
    }
    const Real g = P[BC_P_HCN1F_G] * (f + sl);
    G += g;
    I += g * (P[BC_P_HCN1F_E] - v);
  }
  if (m & BC_M_HCN1H) {
    Real h = st[kSlotHcn1H * N];
    if (advance) {
      const Hcn1hRates<Real> r(v);
      h = gate_it(h, r.hinf, r.htau, P[BC_P_HCN1H_PHI], dt);
      st[kSlotHcn1H * N] = h;
    }
    const Real g = P[BC_P_HCN1H_G] * h;
    G += g;
    I += g * (P[BC_P_HCN1H_E] - v);
  }
  if (m & kCerebellarCaChannels) {
    if (advance) {
      if (m & BC_M_CAHVA) {
        const CaHvaRates<Real> r(v);
        st[kSlotCaHvaS * N] = gate_ab<Real, true>(st[kSlotCaHvaS * N], r.sa, r.sb, P[BC_P_CAHVA_PHI], dt);
        st[kSlotCaHvaU * N] = gate_ab<Real, true>(st[kSlotCaHvaU * N], r.ua, r.ub, P[BC_P_CAHVA_PHI], dt);
      }
      if (m & BC_M_CAV23) {
        const Cav23Rates<Real> r(v);
        st[kSlotCav23M * N] = gate_it(st[kSlotCav23M * N], r.minf, r.mtau, Real(1), dt);
        st[kSlotCav23H * N] = gate_it(st[kSlotCav23H * N], r.hinf, r.htau, Real(1), dt);
      }
      if (m & BC_M_CAV32) {
        const Cav32Rates<Real> r(v, P[BC_P_CAV32_VSH]);
        st[kSlotCav32M * N] = gate_it(st[kSlotCav32M * N], r.minf, r.mtau, Real(kCav32PhiM), dt);
        st[kSlotCav32H * N] = gate_it(st[kSlotCav32H * N], r.hinf, r.htau, Real(1), dt);
      }
    }
    const Real eca =
        (m & BC_M_CADET) ? Real(kNernstCa) * P[BC_P_CA_TEMP] * dlog(P[BC_P_CA_CO] / ci) : P[BC_P_ECA];
    Real g = Real(0);
    I += cerebellar_ca_current(st, N, P, m, v, eca, &g);
    G += g;
  }
}

template <typename Real>
__device__ __noinline__ void extra_channels(Real* st, int N, const Real* P, uint32_t m, Real v, Real ci, Real dt,
                                            bool advance,
                                            Real& G, Real& I) {
  if (m & BC_M_NAHH) {
    Real p = st[kSlotNaHHP * N], q = st[kSlotNaHHQ * N];
    if (advance) {
      const NaHHRates<Real> r(v, P[BC_P_NAHH_VSH]);
      const Real phi = P[BC_P_NAHH_PHI];
      p = gate_ab<Real, true>(p, r.ap, r.bp, phi, dt);
      q = gate_ab<Real, true>(q, r.aq, r.bq, phi, dt);
      st[kSlotNaHHP * N] = p;
      st[kSlotNaHHQ * N] = q;
    }
    const Real g = P[BC_P_NAHH_G] * p * p * p * q;
    G += g;
    I += g * (P[BC_P_ENA] - v);
  }
  if (m & BC_M_KHH) {
    Real p = st[kSlotKHHP * N];
    if (advance) {
      const KHHRates<Real> r(v, P[BC_P_KHH_VSH]);
      p = gate_ab<Real, true>(p, r.a, r.b, P[BC_P_KHH_PHI], dt);
      st[kSlotKHHP * N] = p;
    }
    const Real p2 = p * p;
    const Real g = P[BC_P_KHH_G] * p2 * p2;
    G += g;
    I += g * (P[BC_P_EK] - v);
  }
  if (m & BC_M_KM) {
    Real n = st[kSlotKMN * N];
    if (advance) {
      const KMRates<Real> r(v);
      n = gate_it(n, r.ninf, r.ntau, P[BC_P_KM_PHI], dt);
      st[kSlotKMN * N] = n;
    }
    const Real g = P[BC_P_KM_G] * n;
    G += g;
    I += g * (P[BC_P_EK] - v);
  }
  if (m & BC_M_KA1)
    a_current(st, N, P, kSlotKA1P, kSlotKA1Q, BC_P_KA1_G, Real(kKA1Mid), Real(kKA1InvSlope), v, dt, advance, G, I);
  if (m & BC_M_KA2)
    a_current(st, N, P, kSlotKA2P, kSlotKA2Q, BC_P_KA2_G, Real(kKA2Mid), Real(kKA2InvSlope), v, dt, advance, G, I);
  if (m & BC_M_KK2A) k2_current(st, N, P, kSlotKK2AP, kSlotKK2AQ, BC_P_KK2A_G, false, v, dt, advance, G, I);
  if (m & BC_M_KK2B) k2_current(st, N, P, kSlotKK2BP, kSlotKK2BQ, BC_P_KK2B_G, true, v, dt, advance, G, I);
  if (m & BC_M_KNI) {
    Real p = st[kSlotKNIP * N];
    if (advance) {
      const KNIRates<Real> r(v, P[BC_P_KNI_VSH], P[BC_P_KNI_TAUMAX]);
      p = gate_it(p, r.pinf, r.ptau, P[BC_P_KNI_PHI], dt);
      st[kSlotKNIP * N] = p;
    }
    const Real g = P[BC_P_KNI_G] * p;
    G += g;
    I += g * (P[BC_P_EK] - v);
  }
  if (m & kCerebellarChannels) cerebellar_channels(st, N, P, m, v, ci, dt, advance, G, I);
  // Markov channels: the reference's independent-integration family, advanced
  // after the gates (cell.py:2204-2217), each at the new V and Ci
  if (m & (BC_M_NAV16 | BC_M_KCA22 | BC_M_KCA11)) {
    Real kf[17], kb[17];
    if (m & BC_M_NAV16) {
      if (advance) {
        nav16_rates(v, P[BC_P_NAV16_PHI], P[BC_P_NAV16_OON], P[BC_P_NAV16_ALFAC], P[BC_P_NAV16_EPS], kf, kb);
        markov_advance(st, N, nav16_graph(), kf, kb, dt);
      }
      const Real g = P[BC_P_NAV16_G] * st[(kSlotNav16 + 10) * N];  // O
      G += g;
      I += g * (P[BC_P_ENA] - v);
    }
    if (m & BC_M_KCA22) {
      if (advance) {
        kca22_rates(ci, P[BC_P_KCA22_PHI], P[BC_P_KCA22_DIFF], kf, kb);
        markov_advance(st, N, kca22_graph(), kf, kb, dt);
      }
      const Real g = P[BC_P_KCA22_G] * (st[(kSlotKca22 + 3) * N] + st[(kSlotKca22 + 4) * N]);  // O1 + O2
      G += g;
      I += g * (P[BC_P_EK] - v);
    }
    if (m & BC_M_KCA11) {
      if (advance) {
        kca11_rates(v, ci, P[BC_P_KCA11_PHI], P[BC_P_KCA11_QO], P[BC_P_KCA11_QC], kf, kb);
        markov_advance(st, N, kca11_graph(), kf, kb, dt);
      }
      Real o = Real(0);
      for (int k = 4; k < 9; ++k) o += st[(kSlotKca11 + k) * N];  // O0 .. O4
      const Real g = P[BC_P_KCA11_G] * o;
      G += g;
      I += g * (P[BC_P_EK] - v);
    }
  }
  // the extension channels listed in the record (gates independent of the above),
  // the calcium ones in E_Ca of the calcium after this step's shell update
  if (m & BC_M_EXT) {
    const Real eca =
        (m & BC_M_CADET) ? Real(kNernstCa) * P[BC_P_CA_TEMP] * dlog(P[BC_P_CA_CO] / ci) : P[BC_P_ECA];
    ext_channels(st, N, P, v, ci, eca, dt, advance, G, I);
  }
}

// One node's mechanisms.  `st` points at the node's slot-0 state (stride N).
// With advance = true the states move from (v_old) to (v_new) first: calcium
// from the step-start current (old gates, old V, old Ci), then every gate at
// v_new (and the new Ci).  Returns the membrane conductance G (mS/cm^2) and
// ionic current I (uA/cm^2) at v_new with the resulting states.
template <typename Real, bool kExtra = true>
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
      if (kExtra && (m & kCerebellarCaChannels)) ica += cerebellar_ca_current(st, N, P, m, v_old, eca, (Real*)nullptr);
      if (kExtra && (m & BC_M_EXT)) ica += ext_ca_current(st, N, P, v_old, ci, eca);
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
  if (kExtra && (m & kExtraChannels)) {
    // the calcium the Markov Kca channels bind: the new Ci of a dynamic ion, else the fixed one
    const Real ci = (m & BC_M_CADET) ? cahi + calo : P[BC_P_CA_CI0];
    extra_channels(st, N, P, m, v_new, ci, dt, advance, G, I);
  }
}

template <typename Real, bool kExtra = true>
__device__ __forceinline__ void node_mechanisms(Real* st, int N, const Real* P, uint32_t m, Real v_old, Real v_new,
                                                Real dt, bool advance, Real& G, Real& I) {
  NodeStates<Real> s;
  load_states(st, N, m, s);
  node_mechanisms_loaded<Real, kExtra>(s, st, N, P, m, v_old, v_new, dt, advance, G, I);
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
  if (m & BC_M_NAHH) {
    const NaHHRates<Real> r(v, P[BC_P_NAHH_VSH]);
    st[kSlotNaHHP * N] = r.ap / (r.ap + r.bp);
    st[kSlotNaHHQ * N] = r.aq / (r.aq + r.bq);
  }
  if (m & BC_M_KHH) {
    const KHHRates<Real> r(v, P[BC_P_KHH_VSH]);
    st[kSlotKHHP * N] = r.a / (r.a + r.b);
  }
  if (m & BC_M_KM) st[kSlotKMN * N] = KMRates<Real>(v).ninf;
  if (m & BC_M_KA1) {
    const KARates<Real> r(v, P[BC_P_KA1_VSH], Real(kKA1Mid), Real(kKA1InvSlope));
    st[kSlotKA1P * N] = r.pinf;
    st[kSlotKA1Q * N] = r.qinf;
  }
  if (m & BC_M_KA2) {
    const KARates<Real> r(v, P[BC_P_KA2_VSH], Real(kKA2Mid), Real(kKA2InvSlope));
    st[kSlotKA2P * N] = r.pinf;
    st[kSlotKA2Q * N] = r.qinf;
  }
  if (m & BC_M_KK2A) {
    const K2Rates<Real> r(v, P[BC_P_KK2A_VSH], false);
    st[kSlotKK2AP * N] = r.pinf;
    st[kSlotKK2AQ * N] = r.qinf;
  }
  if (m & BC_M_KK2B) {
    const K2Rates<Real> r(v, P[BC_P_KK2B_VSH], true);
    st[kSlotKK2BP * N] = r.pinf;
    st[kSlotKK2BQ * N] = r.qinf;
  }
  if (m & BC_M_KNI) st[kSlotKNIP * N] = KNIRates<Real>(v, P[BC_P_KNI_VSH], P[BC_P_KNI_TAUMAX]).pinf;
  if (m & BC_M_KV34) {
    const Kv34Rates<Real> r(v);
    st[kSlotKv34M * N] = r.minf;
    st[kSlotKv34H * N] = r.hinf;
  }
  if (m & BC_M_KV43) {
    const Kv43Rates<Real> r(v);
    st[kSlotKv43A * N] = r.ainf;
    st[kSlotKv43B * N] = r.binf;
  }
  if (m & BC_M_KV11) {
    const Kv11Rates<Real> r(v);
    st[kSlotKv11N * N] = r.a / (r.a + r.b);
  }
  if (m & BC_M_KIR23) {
    const Kir23Rates<Real> r(v);
    st[kSlotKir23D * N] = r.a / (r.a + r.b);
  }
  if (m & BC_M_HCN1F) {
    const Hcn1fRates<Real> r(v);
    st[kSlotHcn1Fast * N] = r.finf;
    st[kSlotHcn1Slow * N] = r.sinf;
  }
  if (m & BC_M_HCN1H) st[kSlotHcn1H * N] = Hcn1hRates<Real>(v).hinf;
  if (m & BC_M_CAHVA) {
    const CaHvaRates<Real> r(v);
    st[kSlotCaHvaS * N] = r.sa / (r.sa + r.sb);
    st[kSlotCaHvaU * N] = r.ua / (r.ua + r.ub);
  }
  if (m & BC_M_CAV23) {
    const Cav23Rates<Real> r(v);
    st[kSlotCav23M * N] = r.minf;
    st[kSlotCav23H * N] = r.hinf;
  }
  if (m & BC_M_CAV32) {
    const Cav32Rates<Real> r(v, P[BC_P_CAV32_VSH]);
    st[kSlotCav32M * N] = r.minf;
    st[kSlotCav32H * N] = r.hinf;
  }
  if (m & BC_M_EXT) ext_steady(P, st, N, v);
  if (m & (BC_M_NAV16 | BC_M_KCA22 | BC_M_KCA11)) {
    // Markov channels start at their stationary distribution (reset_steady_state)
    Real kf[17], kb[17];
    const Real ci = P[BC_P_CA_CI0];
    if (m & BC_M_NAV16) {
      nav16_rates(v, P[BC_P_NAV16_PHI], P[BC_P_NAV16_OON], P[BC_P_NAV16_ALFAC], P[BC_P_NAV16_EPS], kf, kb);
      markov_steady(st, N, nav16_graph(), kf, kb);
    }
    if (m & BC_M_KCA22) {
      kca22_rates(ci, P[BC_P_KCA22_PHI], P[BC_P_KCA22_DIFF], kf, kb);
      markov_steady(st, N, kca22_graph(), kf, kb);
    }
    if (m & BC_M_KCA11) {
      kca11_rates(v, ci, P[BC_P_KCA11_PHI], P[BC_P_KCA11_QO], P[BC_P_KCA11_QC], kf, kb);
      markov_steady(st, N, kca11_graph(), kf, kb);
    }
  }
}

// Row i of the next linear system: diag = 1 + dt (D + G / cm), rhs = dt I / cm
// on membrane rows; diag = dt D, rhs = 0 on boundary rows.
template <typename Real>
__device__ __forceinline__ void write_row(const TileView<Real>& tv, int i, uint16_t pr, Real dt, Real G, Real I) {
  if (pr == kBoundary) {
    tv.dr[i] = make_pair(dt * tv.diag0[i], Real(0));
  } else {
    const Real invcm = tv.params[size_t(pr) * tv.pstride + BC_P_INVCM];
    tv.dr[i] = make_pair(Real(1) + dt * (tv.diag0[i] + invcm * G), dt * invcm * I);
  }
}

// ExpSyn synapses of a node (synapse/markov.py:65-117).  `g` is stored as the
// conductance at the start of a step including that step's events.  advance:
// one dt of decay (exp-Euler of g' = -g / tau, exact); then, unless `last`, the
// events due at `next_step` are added (their ring slot is cleared) and the
// synapse current g (e - V) at v (a total current spread over the CV) is added
// to the node's conductance G and current I for the next row.
template <typename Real>
__device__ __forceinline__ void node_synapses(const LaunchArgs& a, const TileView<Real>& tv, const SpecRec& sr,
                                              Real v, Real dt, bool advance, bool last, int64_t next_step, Real& G,
                                              Real& I) {
  Real* g_all = static_cast<Real*>(a.syn_g);
  const Real* tau = static_cast<const Real*>(a.syn_tau);
  const Real* e = static_cast<const Real*>(a.syn_e);
  const Real* scale = static_cast<const Real*>(a.syn_scale);
  Real* arr = static_cast<Real*>(a.arrivals);
  for (int k = sr.syn_begin; k < sr.syn_end; ++k) {
    const int32_t id = tv.syn[k];
    Real g = g_all[id];
    if (advance) g += decay_em1(-dt / tau[id]) * g;
    if (!last) {
      if (arr) {
        Real* slot = arr + (next_step % a.arr_slots) * a.n_syn + id;
        g += *slot;
        *slot = Real(0);
      }
      const Real gd = g * scale[id];
      G += gd;
      I += gd * (e[id] - v);
    }
    g_all[id] = g;
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
      tv.dr[i].y += dt * tv.params[size_t(pr) * tv.pstride + BC_P_INVCM] * Real(p.amp);
  }
}

// ---------------------------------------------------------------- Hines sweeps
// Row i of the increment system (V_{n+1} = V_n + x):
//   d_i x_i - alpha_i x_parent - sum_c beta_c x_c = rhs_i - alpha_i Delta_i + sum_c beta_c Delta_c
// with Delta_i = V_i - V_parent (float-float).  Along a chain (node k+1 is the
// parent of node k; a = alpha dt, b = beta dt) elimination is the recurrence
//   D_0 = d_0 - sum cD(children),  R_0 = r_0 + sum cR(children),
//   R'_k = R_k - a_k Delta_k,  w_k = b_k / D_k,
//   D_{k+1} = d_{k+1} - a_k b_k / D_k,  R_{k+1} = r_{k+1} + w_k R'_k + b_k Delta_k,
// the chain top hands (cD, cR) = (a w, w R' + b Delta) to its parent, and back-
// substitution is x_k = (R'_k + a_k x_{k+1}) / D_k.  All three are associative
// scans along the chain: D through the projective (Moebius) form
//   [p; q]_{k+1} = [[d_{k+1}, -a_k b_k], [1, 0]] [p; q]_k,  D = p / q,
// R' and x through affine maps.  Each phase's chains are packed into 32-lane warp
// slots.  In a "serial" slot every lane owns whole chains (at most lane_nodes
// nodes) and walks them one after another.  In a "scan" slot a chain spans
// several lanes: each lane composes the maps of its chunk, the lanes scan them
// with shuffles (segmented at chain bottoms going up, at chain tops going down),
// and each lane re-walks its chunk from the carry of its neighbours.

constexpr unsigned kFullMask = 0xffffffffu;

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

__device__ __forceinline__ float rabs(float x) { return fabsf(x); }
__device__ __forceinline__ double rabs(double x) { return fabs(x); }
__device__ __forceinline__ float rmax(float x, float y) { return fmaxf(x, y); }
__device__ __forceinline__ double rmax(double x, double y) { return fmax(x, y); }

// 2^-floor(log2 m) for m > 0 (exact scaling by a power of two; the exponent is
// clamped so that the result stays a normal number).
__device__ __forceinline__ float pow2_inv(float m) {
  int e = (__float_as_int(m) >> 23) & 0xff;
  e = min(max(e, 1), 253);
  return __int_as_float((254 - e) << 23);
}
__device__ __forceinline__ double pow2_inv(double m) {
  long long e = (__double_as_longlong(m) >> 52) & 0x7ff;
  e = min(max(e, 1LL), 2045LL);
  return __longlong_as_double((2046LL - e) << 52);
}

template <typename Real>
struct Mob {
  Real m00, m01, m10, m11;  // [[m00, m01], [m10, m11]]
};

// Rescale by a power of two: the projective ratio a map defines does not change,
// and the entries stay in range.
template <typename Real>
__device__ __forceinline__ void mob_norm(Mob<Real>& r) {
  const Real s = pow2_inv(rmax(rmax(rabs(r.m00), rabs(r.m01)), rmax(rabs(r.m10), rabs(r.m11))));
  r.m00 *= s;
  r.m01 *= s;
  r.m10 *= s;
  r.m11 *= s;
}

// hi * lo (hi is the later map).
template <typename Real>
__device__ __forceinline__ Mob<Real> mob_mul(const Mob<Real>& hi, const Mob<Real>& lo) {
  Mob<Real> r;
  r.m00 = hi.m00 * lo.m00 + hi.m01 * lo.m10;
  r.m01 = hi.m00 * lo.m01 + hi.m01 * lo.m11;
  r.m10 = hi.m10 * lo.m00 + hi.m11 * lo.m10;
  r.m11 = hi.m10 * lo.m01 + hi.m11 * lo.m11;
  return r;
}

template <typename Real>
__device__ __forceinline__ Mob<Real> mob_shfl_up(const Mob<Real>& m, int off) {
  Mob<Real> o;
  o.m00 = __shfl_up_sync(kFullMask, m.m00, off);
  o.m01 = __shfl_up_sync(kFullMask, m.m01, off);
  o.m10 = __shfl_up_sync(kFullMask, m.m10, off);
  o.m11 = __shfl_up_sync(kFullMask, m.m11, off);
  return o;
}

// Lane of the segment start at or below `lane` (bit l of `heads` marks a start).
__device__ __forceinline__ int seg_first(unsigned heads, int lane) {
  return 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
}
// Lane of the segment end at or above `lane` (bit l of `tops` marks an end).
__device__ __forceinline__ int seg_last(unsigned tops, int lane) {
  return lane + __ffs(tops >> lane) - 1;
}

// Inclusive segmented scan of Moebius maps over the lanes (lane order = chain
// order); `reach` = lane - first lane of the segment; 2^steps >= segment lanes.
// Inputs are normalised maps; a product of four of them stays far inside the
// FP32 range (each factor changes the scale by at most ~1e6 either way), so the
// partial products are renormalised after every second step only.
template <typename Real>
__device__ __forceinline__ Mob<Real> scan_mob(Mob<Real> m, int reach, int steps) {
  for (int s = 0, off = 1; s < steps; ++s, off <<= 1) {
    const Mob<Real> o = mob_shfl_up(m, off);
    if (off <= reach) m = mob_mul(m, o);
    if (s & 1) mob_norm(m);
  }
  return m;
}

// Inclusive segmented scan of affine maps x -> a x + b, later lanes applied last.
template <typename Real>
__device__ __forceinline__ void scan_aff_up(Real& a, Real& b, int reach, int steps) {
  for (int s = 0, off = 1; s < steps; ++s, off <<= 1) {
    const Real oa = __shfl_up_sync(kFullMask, a, off);
    const Real ob = __shfl_up_sync(kFullMask, b, off);
    if (off <= reach) {
      b = a * ob + b;
      a = a * oa;
    }
  }
}

// The same towards lower lanes (back-substitution runs from chain tops down);
// `reach` = last lane of the segment - lane.
template <typename Real>
__device__ __forceinline__ void scan_aff_down(Real& a, Real& b, int reach, int steps) {
  for (int s = 0, off = 1; s < steps; ++s, off <<= 1) {
    const Real oa = __shfl_down_sync(kFullMask, a, off);
    const Real ob = __shfl_down_sync(kFullMask, b, off);
    if (off <= reach) {
      b = a * ob + b;
      a = a * oa;
    }
  }
}

template <typename Real>
__device__ __forceinline__ Pair<Real> shfl_up_pair(const Pair<Real>& p, int off) {
  return make_pair<Real>(__shfl_up_sync(kFullMask, p.x, off), __shfl_up_sync(kFullMask, p.y, off));
}
template <typename Real>
__device__ __forceinline__ Pair<Real> shfl_down_pair(const Pair<Real>& p, int off) {
  return make_pair<Real>(__shfl_down_sync(kFullMask, p.x, off), __shfl_down_sync(kFullMask, p.y, off));
}

template <typename Real>
__device__ __forceinline__ Real vdelta(const Pair<Real>& v, const Pair<Real>& up) {
  return (v.x - up.x) + (v.y - up.y);
}

// Children's contributions pulled by a chain bottom: the first four slots are
// loaded together (predicated), further ones in a loop.
template <typename Real>
__device__ __forceinline__ void pull_children(const TileView<Real>& tv, const ChainRec& ch, Real& D, Real& R) {
  const int n = ch.n_child, a0 = ch.aux;
  Real cd[4], cr[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    cd[j] = j < n ? tv.scd[a0 + j] : Real(0);
    cr[j] = j < n ? tv.scr[a0 + j] : Real(0);
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    D -= cd[j];
    R += cr[j];
  }
  for (int j = 4; j < n; ++j) {
    D -= tv.scd[a0 + j];
    R += tv.scr[a0 + j];
  }
}

// Lane chunk of a warp slot: nodes [k0, k0 + len) (len = 0 for an idle lane).
__device__ __forceinline__ void lane_chunk(const SlotRec& sr, int lane, int& k0, int& len) {
  const int o0 = sr.off[lane];
  const int o1 = lane < 31 ? int(sr.off[lane + 1]) : int(sr.n_count);
  k0 = sr.n_begin + o0;
  len = o1 - o0;
}

// Elimination of one warp slot holding one node per lane.
template <typename Real, bool kPre>
__device__ __forceinline__ void eliminate_lanes(const TileView<Real>& tv, const SlotRec& sr, int lane, Real dt) {
  const bool valid = lane < sr.n_count;
  const int k = sr.n_begin + (valid ? lane : 0);
  const ChainRec ch = load_rec(tv.chains, tv.crec[k]);
  const bool head = !valid || k == ch.start;
  const bool tail = valid && k == ch.start + ch.count - 1;
  const Pair<Real> q = tv.dr[k];
  const Pair<Real> c = coef<Real, kPre>(tv, k, dt);
  const Pair<Real> v = tv.v[k];
  Pair<Real> vup = shfl_down_pair<Real>(v, 1);  // node k+1 sits in the next lane
  if (tail) vup = ch.top_parent >= 0 ? tv.v[ch.top_parent] : v;
  const Real delta = vdelta<Real>(v, vup);
  const Pair<Real> cp = shfl_up_pair<Real>(c, 1);  // node k-1 sits in the previous lane
  const Real deltap = __shfl_up_sync(kFullMask, delta, 1);
  Real D0 = q.x, R0 = q.y;
  if (head && valid) pull_children(tv, ch, D0, R0);
  Mob<Real> m;
  m.m10 = Real(1);
  m.m11 = Real(0);
  if (head) {
    m.m00 = D0;
    m.m01 = Real(0);
  } else {
    m.m00 = q.x;
    m.m01 = -cp.x * cp.y;
  }
  mob_norm(m);
  const int reach = lane - seg_first(__ballot_sync(kFullMask, head), lane);
  m = scan_mob(m, reach, sr.steps);
  const Real inv = m.m10 * pivot_rcp(m.m00);
  const Real w = c.y * inv;
  const Real wp = __shfl_up_sync(kFullMask, w, 1);
  Real a, b;
  if (head) {
    a = Real(0);
    b = R0 - c.x * delta;
  } else {
    a = wp;
    b = q.y + cp.y * deltap - c.x * delta;
  }
  scan_aff_up(a, b, reach, sr.steps);
  if (valid) {
    tv.dr[k] = make_pair(inv, b);
    if (tail && ch.slot >= 0) {
      tv.scd[ch.slot] = c.x * w;
      tv.scr[ch.slot] = w * b + c.y * delta;
    }
  }
}

// Back-substitution of one warp slot holding one node per lane.
template <typename Real, bool kPre>
__device__ __forceinline__ void backsub_lanes(const TileView<Real>& tv, const SlotRec& sr, int lane, Real dt) {
  const bool valid = lane < sr.n_count;
  const int k = sr.n_begin + (valid ? lane : 0);
  const ChainRec ch = load_rec(tv.chains, tv.crec[k]);
  const bool tail = valid && k == ch.start + ch.count - 1;
  const Pair<Real> q = tv.dr[k];  // (1 / D, R')
  Real A = coef<Real, kPre>(tv, k, dt).x * q.x, B = q.y * q.x;
  if (tail) {
    const Real xp = ch.top_parent >= 0 ? tv.dr[ch.top_parent].y : Real(0);
    B = A * xp + B;
    A = Real(0);
  }
  const bool top = !valid || tail;
  scan_aff_down(A, B, seg_last(__ballot_sync(kFullMask, top), lane) - lane, sr.steps);
  if (valid) tv.dr[k].y = B;
}

// Serial elimination of one whole chain by one lane.
template <typename Real, bool kPre>
__device__ __forceinline__ void eliminate_chain(const TileView<Real>& tv, const ChainRec& ch, Real dt) {
  const int s0 = ch.start, end = ch.start + ch.count;
  const Pair<Real> q = tv.dr[s0];
  Real D = q.x, R = q.y;
  pull_children(tv, ch, D, R);
  Pair<Real> c = coef<Real, kPre>(tv, s0, dt), v = tv.v[s0];
  // node s0 + 1 (or the chain's parent, or -- at the root -- the top node itself)
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
    const Real delta = vdelta<Real>(v, v1);
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

// Serial back-substitution of one whole chain by one lane (top down).
template <typename Real, bool kPre>
__device__ __forceinline__ void backsub_chain(const TileView<Real>& tv, const ChainRec& ch, Real dt) {
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

// A slot of whole chains: every lane walks the chains of its chunk one after another.
template <typename Real, bool kPre>
__device__ __forceinline__ void eliminate_serial(const TileView<Real>& tv, const SlotRec& sr, int lane, Real dt) {
  int k, len;
  lane_chunk(sr, lane, k, len);
  const int end = k + len;
  while (k < end) {
    const ChainRec ch = load_rec(tv.chains, tv.crec[k]);
    eliminate_chain<Real, kPre>(tv, ch, dt);
    k += ch.count;
  }
}

template <typename Real, bool kPre>
__device__ __forceinline__ void backsub_serial(const TileView<Real>& tv, const SlotRec& sr, int lane, Real dt) {
  int k0, len;
  lane_chunk(sr, lane, k0, len);
  int k = k0 + len - 1;
  while (k >= k0) {
    const ChainRec ch = load_rec(tv.chains, tv.crec[k]);
    backsub_chain<Real, kPre>(tv, ch, dt);
    k = ch.start - 1;
  }
}

// A slot of chains spread over several lanes each: every lane composes the maps
// of its chunk, the lanes scan them (segmented per chain), and every lane
// re-walks its chunk from the carry of the lanes below.
template <typename Real, bool kPre>
__device__ __forceinline__ void eliminate_scan(const TileView<Real>& tv, const SlotRec& sr, int lane, Real dt) {
  int k0, len;
  lane_chunk(sr, lane, k0, len);
  ChainRec ch{};
  if (len > 0) ch = load_rec(tv.chains, tv.crec[k0]);
  const int top = ch.start + ch.count - 1;
  const bool head = len > 0 && k0 == ch.start;
  const bool seg = head || len == 0;
  const int reach = lane - seg_first(__ballot_sync(kFullMask, seg), lane);
  Real D0 = Real(0), R0 = Real(0);
  if (head) {
    const Pair<Real> q = tv.dr[k0];
    D0 = q.x;
    R0 = q.y;
    pull_children(tv, ch, D0, R0);
  }
  // chunk map of the pivot recurrence
  Mob<Real> m{Real(1), Real(0), Real(0), Real(1)};
  for (int j = 0; j < len; ++j) {
    const int k = k0 + j;
    Mob<Real> e;
    e.m10 = Real(1);
    e.m11 = Real(0);
    if (k == ch.start) {
      e.m00 = D0;
      e.m01 = Real(0);
    } else {
      const Pair<Real> cp = coef<Real, kPre>(tv, k - 1, dt);
      e.m00 = tv.dr[k].x;
      e.m01 = -cp.x * cp.y;
    }
    m = mob_mul(e, m);
    mob_norm(m);
  }
  m = scan_mob(m, reach, sr.steps);
  const Mob<Real> mx = mob_shfl_up(m, 1);
  // re-walk: pivots of the chunk from the state after the lane below
  Real p = mx.m00, pq = mx.m10;
  for (int j = 0; j < len; ++j) {
    const int k = k0 + j;
    if (k == ch.start) {
      p = D0;
      pq = Real(1);
    } else {
      const Pair<Real> cp = coef<Real, kPre>(tv, k - 1, dt);
      const Real np = tv.dr[k].x * p - cp.x * cp.y * pq;
      pq = p;
      p = np;
      const Real s = pow2_inv(rmax(rabs(p), rabs(pq)));
      p *= s;
      pq *= s;
    }
    tv.dr[k].x = pq * pivot_rcp(p);  // 1 / D_k
  }
  __syncwarp();
  // chunk map of the right-hand-side recurrence R'_k = a_k R'_{k-1} + b_k
  Real fa = Real(1), fb = Real(0);
  for (int j = 0; j < len; ++j) {
    const int k = k0 + j;
    const Pair<Real> c = coef<Real, kPre>(tv, k, dt);
    const Pair<Real> v = tv.v[k];
    const Pair<Real> vup = k == top ? (ch.top_parent >= 0 ? tv.v[ch.top_parent] : v) : tv.v[k + 1];
    const Real delta = vdelta<Real>(v, vup);
    Real a, b;
    if (k == ch.start) {
      a = Real(0);
      b = R0 - c.x * delta;
    } else {
      const Pair<Real> cp = coef<Real, kPre>(tv, k - 1, dt);
      a = cp.y * tv.dr[k - 1].x;
      b = tv.dr[k].y + cp.y * vdelta<Real>(tv.v[k - 1], v) - c.x * delta;
    }
    tv.dr[k].y = b;
    fb = a * fb + b;
    fa = a * fa;
  }
  scan_aff_up(fa, fb, reach, sr.steps);
  Real r = __shfl_up_sync(kFullMask, fb, 1);
  for (int j = 0; j < len; ++j) {
    const int k = k0 + j;
    Real a = Real(0);
    if (k != ch.start) a = coef<Real, kPre>(tv, k - 1, dt).y * tv.dr[k - 1].x;
    r = a * r + tv.dr[k].y;
    tv.dr[k].y = r;
    if (k == top && ch.slot >= 0) {
      const Pair<Real> c = coef<Real, kPre>(tv, k, dt);
      const Pair<Real> v = tv.v[k];
      const Pair<Real> vup = ch.top_parent >= 0 ? tv.v[ch.top_parent] : v;
      const Real w = c.y * tv.dr[k].x;
      tv.scd[ch.slot] = c.x * w;
      tv.scr[ch.slot] = w * r + c.y * vdelta<Real>(v, vup);
    }
  }
}

template <typename Real, bool kPre>
__device__ __forceinline__ void backsub_scan(const TileView<Real>& tv, const SlotRec& sr, int lane, Real dt) {
  int k0, len;
  lane_chunk(sr, lane, k0, len);
  ChainRec ch{};
  if (len > 0) ch = load_rec(tv.chains, tv.crec[k0]);
  const int top = ch.start + ch.count - 1;
  const bool has_top = len > 0 && k0 + len - 1 == top;
  const bool seg_top = len == 0 || has_top;
  const int reach = seg_last(__ballot_sync(kFullMask, seg_top), lane) - lane;
  const Real xp = has_top && ch.top_parent >= 0 ? tv.dr[ch.top_parent].y : Real(0);
  Real fa = Real(1), fb = Real(0);
  for (int j = len - 1; j >= 0; --j) {
    const int k = k0 + j;
    const Pair<Real> q = tv.dr[k];
    Real A = coef<Real, kPre>(tv, k, dt).x * q.x, B = q.y * q.x;
    if (k == top) {
      B = A * xp + B;
      A = Real(0);
    }
    fb = A * fb + B;
    fa = A * fa;
  }
  scan_aff_down(fa, fb, reach, sr.steps);
  Real x = __shfl_down_sync(kFullMask, fb, 1);  // x of the node after this chunk
  for (int j = len - 1; j >= 0; --j) {
    const int k = k0 + j;
    const Pair<Real> q = tv.dr[k];
    const Real A = coef<Real, kPre>(tv, k, dt).x * q.x;
    x = k == top ? A * xp + q.y * q.x : A * x + q.y * q.x;
    tv.dr[k].y = x;
  }
}

template <typename Real, bool kPre>
__device__ __forceinline__ void eliminate_phase(const TileView<Real>& tv, int p, int warp, int n_warps, int lane,
                                                Real dt) {
  for (int s = tv.phase[p] + warp; s < tv.phase[p + 1]; s += n_warps) {
    const SlotRec& sr = tv.slots[s];
    if (sr.steps == 0)
      eliminate_serial<Real, kPre>(tv, sr, lane, dt);
    else if (sr.unit)
      eliminate_lanes<Real, kPre>(tv, sr, lane, dt);
    else
      eliminate_scan<Real, kPre>(tv, sr, lane, dt);
  }
}

template <typename Real, bool kPre>
__device__ __forceinline__ void backsub_phase(const TileView<Real>& tv, int p, int warp, int n_warps, int lane,
                                              Real dt) {
  for (int s = tv.phase[p] + warp; s < tv.phase[p + 1]; s += n_warps) {
    const SlotRec& sr = tv.slots[s];
    if (sr.steps == 0)
      backsub_serial<Real, kPre>(tv, sr, lane, dt);
    else if (sr.unit)
      backsub_lanes<Real, kPre>(tv, sr, lane, dt);
    else
      backsub_scan<Real, kPre>(tv, sr, lane, dt);
  }
}

// ------------------------------------------------------------ surrogate ports
// One GRU step per port of the tile and the port's terms in the row of step m
// (the port variant only).  The port injects I = g (e + y_scale y - V_end) into
// its endpoint row: the -g V_end part implicitly (diagonal), the rest at V^m.
// Inputs: ((V_att - e) / v_scale, S / 0.1 nA, feat0, feat1) with V_att the
// attachment CV's voltage at the start of step m and S the port's stimulus
// pulses active at step m (nA).
//
// Pass A (a thread per port) stages the inputs, checks the envelope (an input
// outside it flags the port's cell for the full solve) and adds the row terms
// that do not depend on y.  Pass B, after a barrier, deals work items (M tile of
// 16 ports, group jb of 8 hidden units) round-robin over the warps; lane
// (g, tq) holds ports g and g + 8 of the tile and units 8 jb + 2 tq, +1.  The
// hidden state is read from the half (m & 1) and written to the other half, so
// items do not race; each item adds its part of y's current atomically.
constexpr float kPortStimScale = 0.1f;  // nA

// Launch start / end: the tile's port records and envelope state between global
// memory and the tile scratch.
__device__ __forceinline__ void port_local_load(const PortRec* ports, int n_ports, const float* port_h,
                                                PortLocal* pl, int tid, int T) {
  for (int q = tid; q < n_ports; q += T) {
    const PortRec r = ports[q];
    PortLocal l;
    l.node = r.node;
    l.att = r.att;
    l.cell = r.cell;
    l.id = r.id;
    l.stim_begin = r.stim_begin;
    l.stim_end = r.stim_end;
    l.g = r.g;
    l.e = r.e;
    l.feat[0] = r.feat[0];
    l.feat[1] = r.feat[1];
    const float2 pv = *reinterpret_cast<const float2*>(port_h + size_t(r.id) * kPortStride + kPortVPrev);
    l.v_prev = pv.x;
    l.seen = pv.y;
    l.pad[0] = l.pad[1] = 0;
    pl[q] = l;
  }
}

__device__ __forceinline__ void port_local_store(int n_ports, float* port_h, const PortLocal* pl, int tid, int T) {
  for (int q = tid; q < n_ports; q += T)
    *reinterpret_cast<float2*>(port_h + size_t(pl[q].id) * kPortStride + kPortVPrev) =
        make_float2(pl[q].v_prev, pl[q].seen);
}

template <typename Real>
__device__ __forceinline__ void port_stage(PortLocal* pl, int n_ports, const PulseRec* stim, int32_t* flags,
                                          const GruWeights* __restrict__ W, const Pair<Real>* v, Pair<Real>* dr,
                                          PortStage* stage, int64_t m, Real dt, int tid, int T) {
  for (int q = tid; q < n_ports; q += T) {
    PortLocal& r = pl[q];
    const Pair<Real> va = v[r.att], ve = v[r.node];
    float S = 0.f;
    for (int k = r.stim_begin; k < r.stim_end; ++k) {
      const PulseRec pr = stim[k];
      if (m >= pr.on_step && m < pr.off_step) S += float(pr.amp);
    }
    const float vatt = float(va.x + va.y);
    const float dv = vatt - float(r.e);
    const float rate = r.seen != 0.f ? fabsf(vatt - r.v_prev) / float(dt) : 0.f;
    if (dv < W->env_v_lo || dv > W->env_v_hi || rate > W->env_dvdt) flags[r.cell] = 1;
    r.v_prev = vatt;
    r.seen = 1.f;
    const Real gg = Real(r.g) * Real(1e-3) * dt;  // uS -> row units (1 uF dummy capacitance)
    Pair<Real> row = dr[r.node];
    row.x += gg;
    row.y += gg * (Real(r.e) + Real(W->y_scale) * Real(W->bo) - (ve.x + ve.y));
    dr[r.node] = row;
    PortStage st;
    st.x[0] = dv / W->v_scale;
    st.x[1] = S * (1.0f / kPortStimScale);
    st.x[2] = r.feat[0];
    st.x[3] = r.feat[1];
    st.node = r.node;
    st.coef = float(gg) * W->y_scale;
    st.id = r.id;
    st.pad = 0;
    stage[q] = st;
  }
}

template <typename Real>
__device__ __forceinline__ void port_gru(const PortStage* stage, int n_ports, float* port_h, const uint2* wfrag,
                                        const float* wo_s, Pair<Real>* dr, int64_t m, int warp, int n_warps, int lane,
                                        unsigned long long* ptimers) {
#ifdef BC_PORT_TIMERS
  long long pt0 = clock64();
#define BC_PTICK(slot)                                                                                  \
  do {                                                                                                  \
    const long long pt1 = clock64();                                                                    \
    if (warp == 0 && lane == 0 && ptimers) atomicAdd(ptimers + (slot), (unsigned long long)(pt1 - pt0)); \
    pt0 = pt1;                                                                                          \
  } while (0)
#else
#define BC_PTICK(slot) \
  do {                 \
  } while (0)
#endif
  const int g = lane >> 2, tq = lane & 3;
  const int rd = int(m & 1), wr = rd ^ 1;
  // Work items: (M tile of 16 ports, range of N groups).  Each M tile is split
  // into as many ranges as there are warps for it (1..8), so every warp is busy;
  // the A operand is loaded once per item and reused across its N groups.
  const int n_mt = (n_ports + 15) >> 4;
  const int n_split = max(1, min(8, n_warps / max(n_mt, 1)));
  const int n_items = n_mt * n_split;
  for (int it = warp; it < n_items; it += n_warps) {
    const int mt = it / n_split, sp = it - mt * n_split;
    const int jb_begin = (sp * 8) / n_split, jb_end = ((sp + 1) * 8) / n_split;
    const int qa = mt * 16 + g, qb = qa + 8;
    const bool oka = qa < n_ports, okb = qb < n_ports;
    float* ha = oka ? port_h + size_t(stage[qa].id) * kPortStride : nullptr;
    float* hb = okb ? port_h + size_t(stage[qb].id) * kPortStride : nullptr;
    // A operand straight from the BF16 halves
    uint32_t ah[4][4];
    const uint32_t* ba = oka ? reinterpret_cast<const uint32_t*>(ha + kPortHBf) + rd * (kGruH / 2) : nullptr;
    const uint32_t* bb = okb ? reinterpret_cast<const uint32_t*>(hb + kPortHBf) + rd * (kGruH / 2) : nullptr;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      ah[kk][0] = oka ? ba[kk * 8 + tq] : 0u;
      ah[kk][1] = okb ? bb[kk * 8 + tq] : 0u;
      ah[kk][2] = oka ? ba[kk * 8 + 4 + tq] : 0u;
      ah[kk][3] = okb ? bb[kk * 8 + 4 + tq] : 0u;
    }
    uint32_t ax[4];
    {
      const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
      const float4 xa = oka ? *reinterpret_cast<const float4*>(stage[qa].x) : z4;
      const float4 xb = okb ? *reinterpret_cast<const float4*>(stage[qb].x) : z4;
      const float fa[4] = {xa.x, xa.y, xa.z, xa.w}, fb[4] = {xb.x, xb.y, xb.z, xb.w};
      xblock_frag(fa, fb, tq, ax);
    }
    BC_PTICK(0);
    float ysa = 0.0f, ysb = 0.0f;
#pragma unroll 1
    for (int jb = jb_begin; jb < jb_end; ++jb) {
      const int j0 = jb * 8 + 2 * tq;
      // FP32 values of this lane's two units (issued ahead of the products)
      const float2 z2 = make_float2(0.f, 0.f);
      const float2 hoa = oka ? *reinterpret_cast<const float2*>(ha + rd * kGruH + j0) : z2;
      const float2 hob = okb ? *reinterpret_cast<const float2*>(hb + rd * kGruH + j0) : z2;
      float acc[4][4];
      gru_preact_frag(wfrag + jb * (kGruFragSlots * 32), lane, ah, ax, acc);
      BC_PTICK(1);
      const float2 wo = *reinterpret_cast<const float2*>(wo_s + j0);
      const GruGate G0 = gru_gate(acc[0][0], acc[1][0], acc[2][0], acc[3][0], hoa.x);
      const GruGate G1 = gru_gate(acc[0][1], acc[1][1], acc[2][1], acc[3][1], hoa.y);
      const GruGate G2 = gru_gate(acc[0][2], acc[1][2], acc[2][2], acc[3][2], hob.x);
      const GruGate G3 = gru_gate(acc[0][3], acc[1][3], acc[2][3], acc[3][3], hob.y);
      if (oka) {
        *reinterpret_cast<float2*>(ha + wr * kGruH + j0) = make_float2(G0.h_new, G1.h_new);
        reinterpret_cast<uint32_t*>(ha + kPortHBf)[wr * (kGruH / 2) + j0 / 2] = pack_bf16(G0.h_new, G1.h_new);
      }
      if (okb) {
        *reinterpret_cast<float2*>(hb + wr * kGruH + j0) = make_float2(G2.h_new, G3.h_new);
        reinterpret_cast<uint32_t*>(hb + kPortHBf)[wr * (kGruH / 2) + j0 / 2] = pack_bf16(G2.h_new, G3.h_new);
      }
      ysa += wo.x * G0.h_new + wo.y * G1.h_new;
      ysb += wo.x * G2.h_new + wo.y * G3.h_new;
      BC_PTICK(2);
    }
    ysa += __shfl_xor_sync(kFullMask, ysa, 1);
    ysa += __shfl_xor_sync(kFullMask, ysa, 2);
    ysb += __shfl_xor_sync(kFullMask, ysb, 1);
    ysb += __shfl_xor_sync(kFullMask, ysb, 2);
    if (tq == 0) {
      if (oka) atomicAdd(&dr[stage[qa].node].y, Real(stage[qa].coef) * Real(ysa));
      if (okb) atomicAdd(&dr[stage[qb].node].y, Real(stage[qb].coef) * Real(ysb));
    }
    BC_PTICK(3);
  }
#undef BC_PTICK
}

template <typename Real>
__device__ __forceinline__ bool is_finite_real(Real x) {
  return isfinite(x);
}

// ------------------------------------------------------------------ the step kernel
// kVar: 0 = lean (no optional mechanism), 1 = extra (synapses, network,
// out-of-line channels), 2 = extra + subtree-surrogate ports, 3 = lean + ports
// (plans whose only optional feature is the ports).
// The port variants run at most BC_PORT_MAX_THREADS threads per CTA and ask for
// BC_PORT_MIN_CTAS resident CTAs per SM (their register budget).
template <typename Real, bool kSmem, int kVar>
__global__ void __launch_bounds__(kVar >= 2 ? BC_PORT_MAX_THREADS : 1024, kVar >= 2 ? BC_PORT_MIN_CTAS : 1)
    tile_step_kernel(LaunchArgs a) {
  constexpr bool kExtra = kVar == 1 || kVar == 2;
  constexpr bool kPorts = kVar >= 2;
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
  const int lane = tid & 31, warp = tid >> 5, n_warps = T >> 5;
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
      node_mechanisms<Real, kExtra>(tv.state + i, tv.N, tv.params + size_t(pr) * tv.pstride, tv.mech[pr], v, v, dt,
                                    false, G, I);
    }
    const uint16_t sp = tv.spec[i];
    if (sp != kNoSpecial) {
      const SpecRec sr = tv.specs[sp];
      if (kExtra && sr.syn_begin < sr.syn_end) node_synapses(a, tv, sr, tv.v[i].x, dt, false, false, a.step0, G, I);
    }
    write_row(tv, i, pr, dt, G, I);
    if (sp != kNoSpecial) add_node_pulses(tv, pulses, tv.specs[sp], i, pr, a.step0, dt);
  }
  if (tv.has_src)
    for (int c = tid; c < tv.n_cells; c += T) tv.stamp[c] = -1;
  __syncthreads();
  PortStage* pstage = nullptr;
  PortLocal* plocal = nullptr;
  uint2* wfrag = nullptr;
  float* wo_s = nullptr;
  if constexpr (kPorts) {
    if (td.n_ports > 0) {
      wfrag = reinterpret_cast<uint2*>(scratch + td.off_pstage);
      wo_s = reinterpret_cast<float*>(scratch + td.off_pstage + kGruFragBytes);
      pstage = reinterpret_cast<PortStage*>(scratch + td.off_pstage + kGruSmemBytes);
      plocal = reinterpret_cast<PortLocal*>(pstage + td.n_ports);
      gru_frag_fill(a.gru->wext, wfrag, tid, T);
      for (int j = tid; j < kGruH; j += T) wo_s[j] = a.gru->wo[j];
      port_local_load(a.ports + td.port_offset, td.n_ports, a.port_h, plocal, tid, T);
      __syncthreads();
      port_stage<Real>(plocal, td.n_ports, a.port_pulses, a.port_flags, a.gru, tv.v, tv.dr, pstage, a.step0, dt,
                       tid, T);
      __syncthreads();
      port_gru<Real>(pstage, td.n_ports, a.port_h, wfrag, wo_s, tv.dr, a.step0, warp, n_warps, lane, a.timers);
      __syncthreads();
    }
  }

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
      eliminate_phase<Real, kSmem>(tv, p, warp, n_warps, lane, dt);
      __syncthreads();
    }
    BC_TICK(0);
    // back-substitution, root first
    for (int p = tv.n_phases - 1; p >= 0; --p) {
      backsub_phase<Real, kSmem>(tv, p, warp, n_warps, lane, dt);
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
      if (last) {  // last_V of the per-CV spike indicator (cell.py:2384-2386)
        tv.state[size_t(kSlotVLastHi) * tv.N + i] = v_old;
        tv.state[size_t(kSlotVLastLo) * tv.N + i] = lo_old;
      }
      if (!is_finite_real(hi)) s_status = kStatusNonfinite;
      const uint16_t pr = pr_cur;
      Real G = Real(0), I = Real(0);
      if (pr != kBoundary)
        node_mechanisms_loaded<Real, kExtra>(cur, tv.state + i, tv.N, tv.params + size_t(pr) * tv.pstride, tv.mech[pr],
                                             v_old, hi, dt, true, G, I);
      cur = nxt;
      pr_cur = pr_nxt;
      const uint16_t sp = tv.spec[i];
      SpecRec sr;
      if (sp != kNoSpecial) {
        sr = tv.specs[sp];
        if (kExtra && sr.syn_begin < sr.syn_end) node_synapses(a, tv, sr, hi, dt, true, last, step + 1, G, I);
      }
      if (!last) write_row(tv, i, pr, dt, G, I);
      if (kExtra && tv.has_src && pr != kBoundary) {
        // a spike of the cell: any of its CVs crossing 0 mV upward in this step
        const uint16_t lc = tv.ncell[i];
        if (lc != 0xFFFF && Real(v_old + lo_old) < Real(0) && Real(hi + lo) >= Real(0))
          tv.stamp[lc] = int32_t(step & 0x7fffffff);
      }
      if (sp != kNoSpecial) {
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
    if (kExtra && record && td.n_xprobes > 0) {
      // mechanism probes (plans with them run the extra variant): state views after the update
      const ProbeRef* pl = reinterpret_cast<const ProbeRef*>(reinterpret_cast<const unsigned char*>(tv.specs) +
                                                             (td.off_plist - td.off_specs));
      const int64_t slot = k_since / a.record_every - 1;
      for (int q = tid; q < td.n_xprobes; q += T) {
        const ProbeRef r = pl[q];
        if (slot < 0 || slot >= a.trace_cap) continue;
        double val;
        if (r.field >= BC_PROBE_CURRENT) {
          const uint16_t pr = tv.pidx[r.node];
          const Pair<Real> vv = tv.v[r.node];
          val = probe_current(tv.state + r.node, tv.N, tv.params + size_t(pr) * tv.pstride, tv.mech[pr], vv.x + vv.y,
                              r.field - BC_PROBE_CURRENT);
        } else {
          val = probe_state(tv.state + r.node, tv.N, r.field);
        }
        a.traces[slot * a.n_probes_total + r.id] = val;
      }
    }
    if (kExtra && tv.has_src)
      for (int c = tid; c < tv.n_cells; c += T)
        if (tv.stamp[c] == int32_t(step & 0x7fffffff) && tv.srccell[c] >= 0) {
          const unsigned long long r = atomicAdd(a.rec_count, 1ull);
          if (int64_t(r) < a.rec_cap) {
            a.rec_cell[r] = tv.srccell[c];
            a.rec_step[r] = step;
          } else {
            s_status = kStatusRecordOverflow;
          }
        }
    BC_TICK(2);
    if constexpr (kPorts) {
      if (td.n_ports > 0 && !last) {
        port_stage<Real>(plocal, td.n_ports, a.port_pulses, a.port_flags, a.gru, tv.v, tv.dr, pstage, step + 1, dt,
                         tid, T);
        __syncthreads();
        BC_TICK(2);
        port_gru<Real>(pstage, td.n_ports, a.port_h, wfrag, wo_s, tv.dr, step + 1, warp, n_warps, lane, a.timers);
        __syncthreads();
      }
    }
    BC_TICK(3);
  }
#ifdef BC_PHASE_TIMERS
  if (threadIdx.x == 0 && a.timers)
    for (int q = 0; q < 4; ++q) atomicAdd(a.timers + q, tm[q]);
#endif
  if constexpr (kPorts) {
    if (td.n_ports > 0) port_local_store(td.n_ports, a.port_h, plocal, tid, T);
  }
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

// ------------------------------------------------------------------ lane tiles
// One small cell per thread: node v of the thread's cell is tile node v * L + lane
// (L = blockDim.x), so the threads of a warp touching "their" node v touch
// consecutive addresses of every per-node array (blob, solver scratch, states).
// Parents precede their children in the node order (v_parent < v), so elimination
// runs v = n-1 .. 1 folding each node into its parent, and back-substitution runs
// v = 0 .. n-1.  The rows are those of the tile kernel (increment form,
// float-float V); a thread touches only its own cell, so a step needs no barrier.
// Plans with lane tiles have no synapses, network, mechanism probes or ports;
// kExtra adds the channels outside the main mix.
template <typename Real, bool kExtra>
__global__ void __launch_bounds__(kLaneThreads, sizeof(Real) == 4 ? 8 : 4) lane_step_kernel(LaunchArgs a) {
  __shared__ int s_status;
  const TileDesc td = a.tiles[blockIdx.x];
  unsigned char* base = a.blob + td.blob_offset;
  TileView<Real> tv;
  tv.bind(td, base, a.scratch + td.scratch_offset, a.state);
  const int L = blockDim.x, lane = threadIdx.x;
  const int n = reinterpret_cast<const int32_t*>(base + td.off_lane_n)[lane];
  const uint16_t* par = tv.crec;  // parent v of each node
  const Real dt = Real(a.dt);
  const PulseRec* pulses = a.pulses + td.pulse_offset;
  if (lane == 0) s_status = 0;
  __syncthreads();
  // the rows of the first step from the current state
  for (int k = 0; k < n; ++k) {
    const int i = k * L + lane;
    const uint16_t pr = tv.pidx[i];
    Real G = Real(0), I = Real(0);
    if (pr != kBoundary) {
      NodeStates<Real> st;
      load_states(tv.state + i, tv.N, tv.mech[pr], st);
      const Real v = tv.v[i].x;
      node_mechanisms_loaded<Real, kExtra>(st, tv.state + i, tv.N, tv.params + size_t(pr) * tv.pstride, tv.mech[pr],
                                           v, v, dt, false, G, I);
    }
    write_row(tv, i, pr, dt, G, I);
    const uint16_t sp = tv.spec[i];
    if (sp != kNoSpecial) add_node_pulses(tv, pulses, tv.specs[sp], i, pr, a.step0, dt);
  }
  for (int s = 0; s < a.n_steps; ++s) {
    const int64_t step = a.step0 + s;
    // Elimination, deepest node first.  Node k's contribution to its parent stays
    // in registers (cD, cR) when the parent is node k - 1, the next one visited
    // (the common case along a branch); otherwise it is added to the parent's
    // row in memory, which only a later iteration reads.  Node k - 1's inputs are
    // loaded one iteration ahead: iteration k writes no row but its own and one of
    // a node below k - 1.
    Real cD = Real(0), cR = Real(0);
    if (n > 1) {
      int i = (n - 1) * L + lane;
      int pv = par[i];
      Pair<Real> q = tv.dr[i], c = coef<Real, false>(tv, i, dt), vi = tv.v[i], vp = tv.v[pv * L + lane];
      for (int k = n - 1; k >= 1; --k) {
        const int i1 = i - L;
        int pv1 = 0;
        Pair<Real> q1 = q, c1 = c, vi1 = vi, vp1 = vp;
        if (k > 1) {
          pv1 = par[i1];
          q1 = tv.dr[i1];
          c1 = coef<Real, false>(tv, i1, dt);
          vi1 = tv.v[i1];
          vp1 = tv.v[pv1 * L + lane];
        }
        const Real delta = vdelta<Real>(vi, vp);
        const Real inv = pivot_rcp(q.x - cD);
        const Real Rp = (q.y + cR) - c.x * delta;
        tv.dr[i] = make_pair(inv, Rp);
        const Real w = c.y * inv;
        const Real oD = c.x * w, oR = w * Rp + c.y * delta;
        if (pv == k - 1) {
          cD = oD;
          cR = oR;
        } else {
          const int ip = pv * L + lane;
          Pair<Real> pp = tv.dr[ip];
          pp.x -= oD;
          pp.y += oR;
          tv.dr[ip] = pp;
          cD = Real(0);
          cR = Real(0);
        }
        i = i1;
        pv = pv1;
        q = q1;
        c = c1;
        vi = vi1;
        vp = vp1;
      }
    }
    // the root, then back-substitution root first; x of node k - 1 stays in a
    // register for a child that follows its parent
    Real x_prev = Real(0);
    if (n > 0) {
      const Pair<Real> q = tv.dr[lane];
      const Real inv = pivot_rcp(q.x - cD);
      x_prev = (q.y + cR) * inv;
      tv.dr[lane] = make_pair(inv, x_prev);
    }
    if (n > 1) {
      int i = L + lane;
      int pv = par[i];
      Pair<Real> q = tv.dr[i];
      Real al = coef<Real, false>(tv, i, dt).x;
      for (int k = 1; k < n; ++k) {
        const int i1 = i + L;
        int pv1 = 0;
        Pair<Real> q1 = q;
        Real al1 = al;
        if (k + 1 < n) {
          pv1 = par[i1];
          q1 = tv.dr[i1];
          al1 = coef<Real, false>(tv, i1, dt).x;
        }
        const Real xp = pv == k - 1 ? x_prev : tv.dr[pv * L + lane].y;
        const Real x = (q.y + al * xp) * q.x;
        tv.dr[i].y = x;
        x_prev = x;
        i = i1;
        pv = pv1;
        q = q1;
        al = al1;
      }
    }
    // update: V += x, mechanisms, the next row, probes and next pulses; the next
    // node's region and states are loaded one iteration ahead
    const bool last = s + 1 == a.n_steps;
    const int64_t k_since = step + 1 - a.trace_base;
    const bool record = a.record_every > 0 && k_since % a.record_every == 0;
    NodeStates<Real> cur;
    uint16_t pr_cur = kBoundary;
    if (n > 0) {
      pr_cur = tv.pidx[lane];
      if (pr_cur != kBoundary) load_states(tv.state + lane, tv.N, tv.mech[pr_cur], cur);
    }
    for (int k = 0; k < n; ++k) {
      const int i = k * L + lane;
      NodeStates<Real> nxt;
      uint16_t pr_nxt = kBoundary;
      if (k + 1 < n) {
        pr_nxt = tv.pidx[i + L];
        if (pr_nxt != kBoundary) load_states(tv.state + i + L, tv.N, tv.mech[pr_nxt], nxt);
      }
      const Pair<Real> vv = tv.v[i];
      Real hi = vv.x, lo = vv.y;
      const Real v_old = hi, lo_old = lo;
      ff_add(hi, lo, tv.dr[i].y);
      tv.v[i] = make_pair(hi, lo);
      if (last) {  // last_V of the per-CV spike indicator
        tv.state[size_t(kSlotVLastHi) * tv.N + i] = v_old;
        tv.state[size_t(kSlotVLastLo) * tv.N + i] = lo_old;
      }
      if (!is_finite_real(hi)) s_status = kStatusNonfinite;
      const uint16_t pr = pr_cur;
      Real G = Real(0), I = Real(0);
      if (pr != kBoundary)
        node_mechanisms_loaded<Real, kExtra>(cur, tv.state + i, tv.N, tv.params + size_t(pr) * tv.pstride,
                                             tv.mech[pr], v_old, hi, dt, true, G, I);
      cur = nxt;
      pr_cur = pr_nxt;
      if (!last) write_row(tv, i, pr, dt, G, I);
      const uint16_t sp = tv.spec[i];
      if (sp != kNoSpecial) {
        const SpecRec sr = tv.specs[sp];
        if (sr.probe >= 0) {
          const double v1 = double(hi) + double(lo), v0 = double(v_old) + double(lo_old);
          if (v0 < 0.0 && v1 >= 0.0) {
            const int cnt = a.spike_count[sr.probe];
            if (cnt < a.max_spikes)
              a.spike_times[int64_t(sr.probe) * a.max_spikes + cnt] =
                  double(step) * a.dt + a.dt * (0.0 - v0) / (v1 - v0);
            a.spike_count[sr.probe] = cnt + 1;
          }
          if (record) {
            const int64_t slot = k_since / a.record_every - 1;
            if (slot >= 0 && slot < a.trace_cap) a.traces[slot * a.n_probes_total + sr.probe] = v1;
          }
        }
        if (!last) add_node_pulses(tv, pulses, sr, i, pr, step + 1, dt);
      }
    }
  }
  __syncthreads();
  if (lane == 0 && s_status) atomicOr(a.status, s_status);
}

static void* lane_kernel(int precision, bool extra) {
  if (precision == BC_PREC_F64)
    return extra ? reinterpret_cast<void*>(lane_step_kernel<double, true>)
                 : reinterpret_cast<void*>(lane_step_kernel<double, false>);
  return extra ? reinterpret_cast<void*>(lane_step_kernel<float, true>)
               : reinterpret_cast<void*>(lane_step_kernel<float, false>);
}

int launch_lanes(const LaunchArgs& a, int precision, int threads, bool extra, void* stream) {
  if (a.n_tiles <= 0) return 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (threads != kLaneThreads) return int(cudaErrorInvalidConfiguration);
  if (precision == BC_PREC_F64) {
    if (extra)
      lane_step_kernel<double, true><<<a.n_tiles, threads, 0, st>>>(a);
    else
      lane_step_kernel<double, false><<<a.n_tiles, threads, 0, st>>>(a);
  } else {
    if (extra)
      lane_step_kernel<float, true><<<a.n_tiles, threads, 0, st>>>(a);
    else
      lane_step_kernel<float, false><<<a.n_tiles, threads, 0, st>>>(a);
  }
  return int(cudaGetLastError());
}

int lane_node_params(const LaunchArgs* a, int precision, int threads, bool extra, cudaKernelNodeParams* np,
                     const LaunchArgs** hold) {
  if (threads != kLaneThreads) return int(cudaErrorInvalidConfiguration);
  *hold = a;
  np->func = lane_kernel(precision, extra);
  np->gridDim = dim3(a->n_tiles, 1, 1);
  np->blockDim = dim3(threads, 1, 1);
  np->sharedMemBytes = 0u;
  np->extra = nullptr;
  np->kernelParams = reinterpret_cast<void**>(const_cast<LaunchArgs**>(hold));
  return 0;
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
    tv.state[size_t(kSlotVLastHi) * tv.N + i] = v;  // no step taken: no crossing
    tv.state[size_t(kSlotVLastLo) * tv.N + i] = Real(0);
    const uint16_t pr = tv.pidx[i];
    if (pr == kBoundary) continue;
    const Real* P = tv.params + size_t(pr) * tv.pstride;
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
template <typename Real, bool kSmem, int kVar>
static int launch_impl(const LaunchArgs& a, int threads, size_t smem_bytes, cudaStream_t st) {
  auto k = tile_step_kernel<Real, kSmem, kVar>;
  if (kSmem) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_bytes));
    if (e != cudaSuccess) return int(e);
  }
  dim3 grid(a.n_tiles, 1, 1);
  k<<<grid, threads, kSmem ? smem_bytes : 0, st>>>(a);
  return int(cudaGetLastError());
}

template <int kVar>
static int launch_tiles_x(const LaunchArgs& a, int precision, bool smem, int threads, size_t smem_bytes,
                          cudaStream_t st) {
  if (precision == BC_PREC_F64)
    return smem ? launch_impl<double, true, kVar>(a, threads, smem_bytes, st)
                : launch_impl<double, false, kVar>(a, threads, smem_bytes, st);
  return smem ? launch_impl<float, true, kVar>(a, threads, smem_bytes, st)
              : launch_impl<float, false, kVar>(a, threads, smem_bytes, st);
}

int launch_tiles(const LaunchArgs& a, int precision, bool smem, int threads, size_t smem_bytes, int variant,
                 void* stream) {
  if (a.n_tiles <= 0) return 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  switch (variant) {
    case 0:
      return launch_tiles_x<0>(a, precision, smem, threads, smem_bytes, st);
    case 1:
      return launch_tiles_x<1>(a, precision, smem, threads, smem_bytes, st);
    case 2:
      return launch_tiles_x<2>(a, precision, smem, threads, smem_bytes, st);
    default:
      return launch_tiles_x<3>(a, precision, smem, threads, smem_bytes, st);
  }
}

// Kernel-node parameters of one tile launch for a CUDA graph: the same kernel,
// grid, block and shared memory as launch_tiles; `*a` is copied by the graph call
// that consumes the parameters.
template <typename Real, bool kSmem, int kVar>
static int node_impl(const LaunchArgs* a, int threads, size_t smem_bytes, cudaKernelNodeParams* np) {
  auto k = tile_step_kernel<Real, kSmem, kVar>;
  if (kSmem) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_bytes));
    if (e != cudaSuccess) return int(e);
  }
  np->func = reinterpret_cast<void*>(k);
  np->gridDim = dim3(a->n_tiles, 1, 1);
  np->blockDim = dim3(threads, 1, 1);
  np->sharedMemBytes = kSmem ? unsigned(smem_bytes) : 0u;
  np->extra = nullptr;
  return 0;
}

template <int kVar>
static int node_x(const LaunchArgs* a, int precision, bool smem, int threads, size_t smem_bytes,
                  cudaKernelNodeParams* np) {
  if (precision == BC_PREC_F64)
    return smem ? node_impl<double, true, kVar>(a, threads, smem_bytes, np)
                : node_impl<double, false, kVar>(a, threads, smem_bytes, np);
  return smem ? node_impl<float, true, kVar>(a, threads, smem_bytes, np)
              : node_impl<float, false, kVar>(a, threads, smem_bytes, np);
}

int tile_node_params(const LaunchArgs* a, int precision, bool smem, int threads, size_t smem_bytes, int variant,
                     cudaKernelNodeParams* np, const LaunchArgs** hold) {
  *hold = a;
  int e;
  switch (variant) {
    case 0:
      e = node_x<0>(a, precision, smem, threads, smem_bytes, np);
      break;
    case 1:
      e = node_x<1>(a, precision, smem, threads, smem_bytes, np);
      break;
    case 2:
      e = node_x<2>(a, precision, smem, threads, smem_bytes, np);
      break;
    default:
      e = node_x<3>(a, precision, smem, threads, smem_bytes, np);
      break;
  }
  np->kernelParams = reinterpret_cast<void**>(const_cast<LaunchArgs**>(hold));
  return e;
}

// Event delivery (network/delivery.py:361-394): each spike record (cell, step)
// of the last launch adds, for every connection of its cell, the weight into the
// ring slot of the arrival step step + max(delay, 1).  Several records can hit one
// slot: the additions are atomic, so their order (and the last bits of a sum of
// three or more weights) may vary between runs.
template <typename Real>
__global__ void deliver_kernel(const int32_t* rec_cell, const int64_t* rec_step, const unsigned long long* rec_count,
                               const unsigned long long* rec_done, int64_t rec_cap, const int64_t* out_ptr,
                               const int64_t* out_syn, const Real* out_w, const int32_t* out_d, Real* arrivals,
                               int64_t arr_slots, int64_t n_syn) {
  const int64_t r0 = int64_t(*rec_done);
  const int64_t r1 = min(int64_t(*rec_count), rec_cap);
  for (int64_t r = r0 + blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < r1; r += int64_t(gridDim.x) * blockDim.x) {
    const int32_t c = rec_cell[r];
    const int64_t s = rec_step[r];
    for (int64_t j = out_ptr[c]; j < out_ptr[c + 1]; ++j) {
      const int64_t arrive = s + max(out_d[j], 1);
      atomicAdd(arrivals + (arrive % arr_slots) * n_syn + out_syn[j], out_w[j]);
    }
  }
}

int launch_deliver_impl(int precision, const int32_t* rec_cell, const int64_t* rec_step,
                        const unsigned long long* rec_count, const unsigned long long* rec_done, int64_t rec_cap,
                        const int64_t* out_ptr, const int64_t* out_syn, const void* out_w, const int32_t* out_d,
                        void* arrivals, int64_t arr_slots, int64_t n_syn, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (precision == BC_PREC_F64)
    deliver_kernel<double><<<152, 256, 0, st>>>(rec_cell, rec_step, rec_count, rec_done, rec_cap, out_ptr, out_syn,
                                                static_cast<const double*>(out_w), out_d,
                                                static_cast<double*>(arrivals), arr_slots, n_syn);
  else
    deliver_kernel<float><<<152, 256, 0, st>>>(rec_cell, rec_step, rec_count, rec_done, rec_cap, out_ptr, out_syn,
                                               static_cast<const float*>(out_w), out_d, static_cast<float*>(arrivals),
                                               arr_slots, n_syn);
  return int(cudaGetLastError());
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
