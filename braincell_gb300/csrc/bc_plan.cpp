// Planner and C ABI of the GB300 Cell step.
//
// bc_plan_create lowers every cell (bc_lower.cpp), decomposes each point tree
// into chains (maximal single-child paths), groups the chains into barrier-
// separated phases by chain level (1 + the highest level of the chains hanging
// below a chain's bottom node), packs each phase's chains into 32-lane warp slots
// (one node per lane; a chain longer than 32 nodes gets a slot of its own with a
// chunk of nodes per lane), packs cells into shared-memory tiles by best-fit-
// decreasing on node count, lays each tile out as one contiguous 16-byte-aligned
// blob and uploads it.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <queue>
#include <string>
#include <thread>
#include <vector>

#include "../../include/braincell_gb300_debug.h"
#include "bc_internal.h"
#include "bc_mech.cuh"
#include "bc_ext.cuh"

namespace bc {

static thread_local std::string g_error = "";

void set_error(const std::string& msg) { g_error = msg; }

bc_status fail(bc_status code, const std::string& msg) {
  g_error = msg;
  return code;
}

#define BC_CUDA(call)                                                                     \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(BC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));       \
  } while (0)

static size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

struct CellSched;

}  // namespace bc

// launch classes: 0 packed shared-memory tiles, 1 one big cell per shared-memory
// tile, 2 global-memory tiles, 3 lane tiles (one small cell per thread)
constexpr int kMaxClasses = 4;
// Serial-walk lengths of the warp slots (lane_nodes / narrow_lane_nodes).  Swept on
// GB300 over the 10,000-cell uneven population (FP32, 1,000 steps per launch):
// lane_nodes 1 / 4 / 8 / 10 / 12 with narrow phases at 1 ran 2.18 / 2.24 / 2.35 /
// 2.38 / 2.33e10 compartment-steps/s; narrow phases at 2 instead of 1 cost 23%.
constexpr int kDefaultLaneNodes = 10;
constexpr int kDefaultNarrowLaneNodes = 1;

constexpr uint32_t kMarkovBits = BC_M_NAV16 | BC_M_KCA22 | BC_M_KCA11;
constexpr uint32_t kCerebellarBits = BC_M_KV34 | BC_M_KV43 | BC_M_KV11 | BC_M_KIR23 | BC_M_HCN1F | BC_M_HCN1H |
                                     BC_M_CAHVA | BC_M_CAV23 | BC_M_CAV32;

namespace bc {

// A region's mechanism bits, with its extension channels' BC_X_* bits (from the
// record) in the high word: the owner masks of state views and current probes.
constexpr uint64_t ext_bits(uint32_t x) { return uint64_t(x) << 32; }
static inline uint64_t region_bits(const bc_batch_spec& s, int64_t k) {
  uint64_t b = s.region_mech[k];
  if (b & BC_M_EXT)
    b |= ext_bits(uint32_t(s.region_params[k * BC_NPARAM + BC_P_EXT_MASK]) |
                  (uint32_t(s.region_params[k * BC_NPARAM + BC_P_EXT_MASK_HI]) << 24));
  return b;
}

// The mechanism bit that owns a BC_STATE_* view and the state slot holding it (V:
// in the tile blob, no slot; V_last: every node; Ci and V_last also have a low word).
static void state_view(int32_t which, uint64_t* bit, int* slot) {
  static const uint32_t kBit[BC_STATE_NAV16_C1] = {
      0,         BC_M_NA,   BC_M_NA,   BC_M_KDR,  BC_M_CAL,  BC_M_CAL,  BC_M_CAT,   BC_M_CAT,  BC_M_HCN,
      BC_M_AHP,  BC_M_CADET, BC_M_NAHH, BC_M_NAHH, BC_M_KHH, BC_M_KM,   BC_M_KA1,   BC_M_KA1,  BC_M_KA2,
      BC_M_KA2,  BC_M_KK2A, BC_M_KK2A, BC_M_KK2B, BC_M_KK2B, BC_M_KNI,  BC_M_ALL};
  static const int kSlot[BC_STATE_NAV16_C1] = {
      -1,         kSlotNaP,   kSlotNaQ,   kSlotKdrP,  kSlotCalP,  kSlotCalQ,  kSlotCatP,  kSlotCatQ,  kSlotHcnP,
      kSlotAhpP,  kSlotCaHi,  kSlotNaHHP, kSlotNaHHQ, kSlotKHHP,  kSlotKMN,   kSlotKA1P,  kSlotKA1Q,  kSlotKA2P,
      kSlotKA2Q,  kSlotKK2AP, kSlotKK2AQ, kSlotKK2BP, kSlotKK2BQ, kSlotKNIP,  kSlotVLastHi};
  if (which < BC_STATE_NAV16_C1) {
    *bit = kBit[which];
    *slot = kSlot[which];
    return;
  }
  // Markov views 25 .. 50 and the cerebellar gates 51 .. 65 sit in slots 26 .. 66
  static const uint32_t kCereb[BC_NSTATE_VIEW - BC_STATE_KV34_M] = {
      BC_M_KV34,  BC_M_KV34,  BC_M_KV43,  BC_M_KV43,  BC_M_KV11,  BC_M_KIR23, BC_M_HCN1F, BC_M_HCN1F,
      BC_M_HCN1H, BC_M_CAHVA, BC_M_CAHVA, BC_M_CAV23, BC_M_CAV23, BC_M_CAV32, BC_M_CAV32};
  // extension channels' states 66 .. 121 in slots 67 .. 122
  static const uint32_t kExt[BC_NSTATE_VIEW - BC_STATE_HCN2_FAST] = {
      BC_X_HCN2, BC_X_HCN2, BC_X_KV33, BC_X_KV22,  BC_X_KV22,  BC_X_KV15,  BC_X_KV15,
      BC_X_KV15, BC_X_NAF,  BC_X_NAF,  BC_X_NAP,   BC_X_NAP,   BC_X_NAIO,  BC_X_NAIO,
      BC_X_FKDR, BC_X_SKDR, BC_X_KDRIO, BC_X_HCNDCN, BC_X_HCNIO, BC_X_CATHP, BC_X_CATHP,
      BC_X_CAHTRE, BC_X_CAHTRE, BC_X_CALDCN, BC_X_CALDCN, BC_X_KCA31, BC_X_SKDCN, BC_X_KKV,
      BC_X_CAN, BC_X_CAIO, BC_X_NAVGRC, BC_X_NAVGRC, BC_X_NAVGRC, BC_X_NAVGRC, BC_X_NAVGRC, BC_X_NAVGRC,
      BC_X_NAVGRC, BC_X_NAVGRC, BC_X_NAVGRC, BC_X_NAVGRC, BC_X_NAVGRC, BC_X_NAVGRC, BC_X_CAV31, BC_X_CAV31,
      BC_X_CAV33, BC_X_CAV33, BC_X_CAV12, BC_X_CAV12, BC_X_CAV12, BC_X_CAV13, BC_X_CAV13, BC_X_CAV13,
      BC_X_CAV21, BC_X_CAHVADCN, BC_X_CALVADCN, BC_X_CALVADCN};
  if (which >= BC_STATE_HCN2_FAST)
    *bit = ext_bits(kExt[which - BC_STATE_HCN2_FAST]);
  else if (which >= BC_STATE_KV34_M)
    *bit = kCereb[which - BC_STATE_KV34_M];
  else
    *bit = which < BC_STATE_KCA22_C2 ? BC_M_NAV16 : (which < BC_STATE_KCA11_C1 ? BC_M_KCA22 : BC_M_KCA11);
  *slot = which + 1;
}

}  // namespace bc

struct LaunchClass {
  int first = 0, count = 0, threads = 256;
  bool smem = true;
  bool lane = false;  // lane tiles: one cell per thread (lane_step_kernel)
  size_t smem_bytes = 0;
};

struct bc_plan {
  std::vector<LaunchClass> classes;
  int precision = BC_PREC_F32;
  int device = 0;
  int threads = 128;
  int threads_global = 512;
  int tile_nodes = 0;
  int lane_nodes = 1;
  int narrow_lane_nodes = 1;
  int steps_per_launch = 1000;
  int record_every = 1;
  int max_spikes = 64;
  int use_graph = 0;
  bool extra = false;  // synapses, a network, mechanism probes, or a region using the out-of-line mechanism set
  int state_slots = 1;
  int64_t n_cells = 0, n_cv = 0, n_nodes = 0, n_probes = 0, n_pulses = 0;
  int64_t max_phases = 0, max_chain_nodes = 0;
  size_t real_size = 4;
  std::vector<bc::TileDesc> tiles;  // smem tiles first, then global tiles
  int n_smem_tiles = 0;
  size_t smem_bytes = 0;
  std::vector<int64_t> cell_ncv;
  std::vector<int32_t> cv_tile, cv_node;
  std::vector<uint64_t> cv_mech;  // region bits, extension channels' BC_X_* bits in the high word
  std::vector<bc::PulseRec> pulses;
  std::vector<int64_t> pulse_src;   // spec pulse id of each record (records are in tile / node order)
  std::vector<double> pulse_scale;  // record amp per nA
  double pulses_dt = -1.0;
  std::vector<double> probe_vrest;
  // synapses and connections (host copies; device mirrors below)
  int64_t n_synapses = 0, n_connections = 0;
  std::vector<double> syn_tau, syn_e, syn_scale, conn_delay;
  std::vector<int64_t> out_ptr, out_syn, out_order;  // CSR of connections by presynaptic cell
  std::vector<double> out_w;
  void* d_syn_g = nullptr;
  void* d_syn_tau = nullptr;
  void* d_syn_e = nullptr;
  void* d_syn_scale = nullptr;
  int64_t* d_out_ptr = nullptr;
  int64_t* d_out_syn = nullptr;
  void* d_out_w = nullptr;
  int32_t* d_out_d = nullptr;
  void* d_arrivals = nullptr;
  int64_t arr_slots = 0, net_k = 0;
  double net_dt = 0.0;  // dt the delays were quantised for (0: not yet)
  int32_t* d_rec_cell = nullptr;
  int64_t* d_rec_step = nullptr;
  unsigned long long* d_rec_count = nullptr;  // [0] produced, [1] delivered
  int64_t rec_cap = 0;
  // subtree-surrogate ports: records (tile order), stimulus pulses (nA), GRU
  int64_t n_ports = 0;
  std::vector<bc::PortRec> ports;
  std::vector<bc::PulseRec> port_pulses;
  double port_pulses_dt = -1.0;
  bc::PortRec* d_ports = nullptr;
  bc::PulseRec* d_port_pulses = nullptr;
  float* d_port_h = nullptr;
  int32_t* d_port_flags = nullptr;
  bc::GruWeights* d_gru = nullptr;
  bool gru_set = false;
  // device buffers
  unsigned char* d_blob = nullptr;
  size_t blob_bytes = 0;
  unsigned char* d_scratch = nullptr;
  size_t scratch_bytes = 0;
  unsigned char* d_state = nullptr;
  size_t state_bytes = 0;
  bc::TileDesc* d_tiles = nullptr;
  bc::PulseRec* d_pulses = nullptr;
  double* d_vinit = nullptr;
  int64_t* d_vinit_off = nullptr;
  double* d_traces = nullptr;
  int64_t trace_cap = 0;
  int64_t trace_origin = 0;
  int32_t* d_spike_count = nullptr;
  double* d_spike_times = nullptr;
  int32_t* d_status = nullptr;
  int64_t step = 0;
  size_t device_bytes = 0;
  // launch classes after the first run concurrently on these streams
  cudaStream_t aux[kMaxClasses - 1] = {nullptr, nullptr, nullptr};
  cudaStream_t init_stream = nullptr;  // highest priority: the initial reset
  int aux_prio = 0;                    // priority of the aux streams (that of the last caller's stream)
  bool dry = false;
  unsigned long long* d_timers = nullptr;
  std::vector<std::array<int64_t, 6>> tile_stats;
  cudaEvent_t ev_fork = nullptr, ev_join[kMaxClasses - 1] = {nullptr, nullptr, nullptr};
  // CUDA graph of one run (use_graph): per launch class a chain of kernel nodes,
  // rebuilt when the launch pattern changes, otherwise only re-parameterised.
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  std::vector<cudaGraphNode_t> graph_nodes;  // [launch][class]
  int64_t graph_launches = -1;
  int32_t graph_k = -1, graph_k_last = -1;
};

namespace bc {

template <typename T>
static bc_status dalloc(bc_plan* p, T** ptr, size_t count) {
  *ptr = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(ptr), count * sizeof(T));
  if (e != cudaSuccess) return fail(BC_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  p->device_bytes += count * sizeof(T);
  return BC_OK;
}

static void free_plan(bc_plan* p) {
  cudaFree(p->d_blob);
  cudaFree(p->d_scratch);
  cudaFree(p->d_state);
  cudaFree(p->d_tiles);
  cudaFree(p->d_pulses);
  cudaFree(p->d_vinit);
  cudaFree(p->d_vinit_off);
  cudaFree(p->d_traces);
  cudaFree(p->d_spike_count);
  cudaFree(p->d_spike_times);
  cudaFree(p->d_status);
  cudaFree(p->d_timers);
  cudaFree(p->d_syn_g);
  cudaFree(p->d_syn_tau);
  cudaFree(p->d_syn_e);
  cudaFree(p->d_syn_scale);
  cudaFree(p->d_out_ptr);
  cudaFree(p->d_out_syn);
  cudaFree(p->d_out_w);
  cudaFree(p->d_out_d);
  cudaFree(p->d_arrivals);
  cudaFree(p->d_rec_cell);
  cudaFree(p->d_rec_step);
  cudaFree(p->d_rec_count);
  cudaFree(p->d_ports);
  cudaFree(p->d_port_pulses);
  cudaFree(p->d_port_h);
  cudaFree(p->d_port_flags);
  cudaFree(p->d_gru);
  for (int k = 0; k < kMaxClasses - 1; ++k) {
    if (p->aux[k]) cudaStreamDestroy(p->aux[k]);
    if (p->ev_join[k]) cudaEventDestroy(p->ev_join[k]);
  }
  if (p->init_stream) cudaStreamDestroy(p->init_stream);
  if (p->ev_fork) cudaEventDestroy(p->ev_fork);
  if (p->graph_exec) cudaGraphExecDestroy(p->graph_exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  delete p;
}

// ------------------------------------------------------------------ chain schedule
struct Chain {
  std::vector<int32_t> nodes;  // bottom -> top (cell-local node ids)
  std::vector<int32_t> kids;   // chain ids (cell-local) whose top's parent is nodes[0]
  int32_t level = 0;
};

struct CellSched {
  std::vector<Chain> chains;   // ordered by level ascending
  int32_t max_level = 0;
};

// fn(i) for i in [0, n) on up to BC_PLAN_THREADS host threads (default: the
// hardware threads, at most 32), in chunks of 64 items; one thread when n is
// small.  fn must touch only item i's outputs and must not throw.  When a
// worker thread cannot be started, the threads already running (and the
// calling thread) take its share: the items are claimed from one counter.
template <class F>
static void parallel_for(int64_t n, F&& fn) {
  int64_t nt = int64_t(std::thread::hardware_concurrency());
  if (const char* e = std::getenv("BC_PLAN_THREADS")) nt = std::atoll(e);
  nt = std::max<int64_t>(1, std::min<int64_t>({nt, 32, (n + 63) / 64}));
  if (nt <= 1) {
    for (int64_t i = 0; i < n; ++i) fn(i);
    return;
  }
  std::atomic<int64_t> next{0};
  auto work = [&]() {
    for (;;) {
      const int64_t i0 = next.fetch_add(64);
      if (i0 >= n) return;
      for (int64_t i = i0; i < std::min<int64_t>(n, i0 + 64); ++i) fn(i);
    }
  };
  std::vector<std::thread> pool;
  try {
    pool.reserve(size_t(nt - 1));
    for (int64_t t = 1; t < nt; ++t) pool.emplace_back(work);
  } catch (const std::exception&) {
    // std::system_error (no thread) or bad_alloc: carry on with what started
  }
  work();
  for (auto& th : pool) th.join();
}

static void decompose(const LoweredCell& lc, CellSched& cs) {
  const int32_t n = lc.n_node;
  std::vector<int32_t> nchild(n, 0);
  for (int32_t i = 0; i < n; ++i)
    if (lc.parent[i] >= 0) nchild[lc.parent[i]]++;
  std::vector<int32_t> chain_of(n, -1);
  std::vector<Chain> chains;
  for (int32_t i = 0; i < n; ++i) {
    if (nchild[i] == 1) continue;  // interior of some chain
    Chain ch;
    int32_t cur = i;
    ch.nodes.push_back(cur);
    while (true) {
      const int32_t p = lc.parent[cur];
      if (p < 0 || nchild[p] != 1) break;
      cur = p;
      ch.nodes.push_back(cur);
    }
    for (int32_t v : ch.nodes) chain_of[v] = int32_t(chains.size());
    chains.push_back(std::move(ch));
  }
  // child chains: top's parent is a bottom of another chain
  for (size_t c = 0; c < chains.size(); ++c) {
    const int32_t top = chains[c].nodes.back();
    const int32_t p = lc.parent[top];
    if (p >= 0) chains[chain_of[p]].kids.push_back(int32_t(c));
  }
  // levels (iterative: process chains in order of decreasing depth)
  std::vector<int32_t> order(chains.size());
  std::iota(order.begin(), order.end(), 0);
  // depth of the bottom node from the root
  std::vector<int32_t> depth(n, -1);
  for (int32_t i = 0; i < n; ++i) {
    if (depth[i] >= 0) continue;
    std::vector<int32_t> path;
    int32_t cur = i;
    while (cur >= 0 && depth[cur] < 0) {
      path.push_back(cur);
      cur = lc.parent[cur];
    }
    int32_t d = cur >= 0 ? depth[cur] : -1;
    for (auto it = path.rbegin(); it != path.rend(); ++it) depth[*it] = ++d;
  }
  std::sort(order.begin(), order.end(),
            [&](int32_t a, int32_t b) { return depth[chains[a].nodes[0]] > depth[chains[b].nodes[0]]; });
  for (int32_t c : order) {
    int32_t lv = 0;
    for (int32_t k : chains[c].kids) lv = std::max(lv, chains[k].level + 1);
    chains[c].level = lv;
  }
  // reorder by level ascending, remap kid ids
  std::vector<int32_t> by_level(chains.size());
  std::iota(by_level.begin(), by_level.end(), 0);
  std::stable_sort(by_level.begin(), by_level.end(),
                   [&](int32_t a, int32_t b) { return chains[a].level < chains[b].level; });
  std::vector<int32_t> newid(chains.size());
  for (size_t k = 0; k < by_level.size(); ++k) newid[by_level[k]] = int32_t(k);
  cs.chains.clear();
  cs.chains.reserve(chains.size());
  cs.max_level = 0;
  for (int32_t old : by_level) {
    Chain ch = std::move(chains[old]);
    for (auto& k : ch.kids) k = newid[k];
    cs.max_level = std::max(cs.max_level, ch.level);
    cs.chains.push_back(std::move(ch));
  }
}

// ------------------------------------------------------------------ tile building
struct TileBuild {
  std::vector<int64_t> cells;  // global cell ids
  int cls = 0;                 // launch class
};

struct TileOut {
  TileDesc desc{};
  std::vector<unsigned char> blob;
  std::vector<double> vinit;
  std::vector<PulseRec> pulses;
  std::vector<int64_t> pulse_src;     // spec pulse id of each pulse record
  std::vector<double> pulse_scale;    // record amp per nA of the spec pulse
  std::vector<PortRec> ports;         // stim_begin / stim_end relative to port_pulses
  std::vector<PulseRec> port_pulses;  // amp in nA
  std::vector<std::pair<int64_t, int32_t>> cv_local;  // (global cv id, local node)
  std::vector<uint64_t> cv_mech;
  int64_t crit = 0;
};

struct BuildCtx {
  const bc_batch_spec* spec;
  const std::vector<LoweredCell>* cells;
  const std::vector<CellSched>* sched;
  const std::vector<int64_t>* cv_base;  // global cv id of each cell's first CV
  const std::vector<std::vector<int64_t>>* cell_pulses;
  const std::vector<std::vector<int64_t>>* cell_probes;
  const std::vector<std::vector<int32_t>>* pulse_node;  // per cell, node per pulse (parallel to cell_pulses)
  const std::vector<std::vector<int32_t>>* probe_node;
  const std::vector<std::vector<std::pair<int64_t, int32_t>>>* cell_syns;  // per cell: (synapse id, node)
  const std::vector<char>* is_src;                                        // per cell: source of a connection
  // per cell: (port id, endpoint node, attachment CV node); port pulses by port
  const std::vector<std::vector<std::array<int32_t, 3>>>* cell_ports;
  const std::vector<std::vector<int64_t>>* port_pulse_ids;
  int precision;
  int state_slots;
  int lane_nodes;  // nodes a lane walks serially in a warp slot
  int narrow_lane_nodes;  // the same in phases with fewer nodes than 32 x warps
  int param_stride;       // reals per parameter record in the tile blobs
};

template <typename Real>
static void put(std::vector<unsigned char>& b, size_t off, size_t idx, Real v) {
  std::memcpy(b.data() + off + idx * sizeof(Real), &v, sizeof(Real));
}

static bc_status build_tile(const BuildCtx& cx, const TileBuild& tb, int T, TileOut& out) {
  const bc_batch_spec& s = *cx.spec;
  const int R = s.n_regions;
  const size_t rs = cx.precision == BC_PREC_F64 ? 8 : 4;
  std::vector<int64_t> cell_list = tb.cells;
  std::vector<std::pair<int64_t, size_t>> cmap;
  for (size_t i = 0; i < cell_list.size(); ++i) cmap.push_back({cell_list[i], i});
  std::sort(cmap.begin(), cmap.end());
  // -------- chains -> phases -> warp slots
  // One record per chain.  The phase of a chain is its chain level (children first).
  // Inside a phase, chains of at most 32 nodes are packed first-fit-decreasing into
  // 32-lane warp slots, one node per lane; a longer chain gets a slot of its own in
  // which every lane takes a contiguous chunk of ceil(L / 32) nodes.
  struct CRef {
    int32_t li, chain, L;
  };
  struct RecSpec {
    int32_t li, chain, kind, seg, K, lo, hi;
  };
  int64_t n_real = 0;
  std::vector<std::vector<int32_t>> node_tile(cell_list.size());
  std::vector<std::vector<int32_t>> handle(cell_list.size());  // chain -> record
  for (size_t li = 0; li < cell_list.size(); ++li) {
    const LoweredCell& lc = (*cx.cells)[cell_list[li]];
    const CellSched& cs = (*cx.sched)[cell_list[li]];
    node_tile[li].assign(lc.n_node, -1);
    handle[li].assign(cs.chains.size(), -1);
    n_real += lc.n_node;
  }
  const int W = std::max(1, T / 32);
  const int C_wide = std::max(1, cx.lane_nodes);
  const int C_narrow = cx.narrow_lane_nodes > 0 ? cx.narrow_lane_nodes : C_wide;
  std::vector<ChainRec> chains;
  std::vector<RecSpec> rec_src;
  std::vector<SlotRec> slots;
  int32_t next_node = 0;
  int64_t crit = 0;
  std::vector<std::vector<CRef>> levels;
  for (size_t li = 0; li < cell_list.size(); ++li) {
    const CellSched& cs = (*cx.sched)[cell_list[li]];
    for (size_t k = 0; k < cs.chains.size(); ++k) {
      const int32_t lv = cs.chains[k].level;
      if (int(levels.size()) <= lv) levels.resize(lv + 1);
      levels[lv].push_back({int32_t(li), int32_t(k), int32_t(cs.chains[k].nodes.size())});
    }
  }
  const bool lane = tb.cls == 3;  // a lane tile has no chains, phases or warp slots
  std::vector<std::vector<CRef>> phases;
  for (auto& v : levels)
    if (!v.empty() && !lane) phases.push_back(std::move(v));
  const int n_phases = int(phases.size());
  std::vector<int32_t> phase_ptr(size_t(n_phases) + 1, 0);
  // A lane plan: the chains (whole, or one chain's part) of one lane.
  struct Lane {
    std::vector<CRef> whole;  // serial slots: whole chains
    int32_t nodes = 0;
  };
  struct Slot {
    bool scan = false;
    std::vector<Lane> lanes;              // serial slots
    std::vector<CRef> spread;             // scan slots: chains, each over `parts` lanes
    std::vector<std::vector<int32_t>> parts;  // per spread chain: part sizes
    int32_t used = 0, steps = 0, cost = 0;
  };
  for (int p = 0; p < n_phases; ++p) {
    std::vector<CRef>& v = phases[p];
    std::stable_sort(v.begin(), v.end(), [](const CRef& a, const CRef& b) { return a.L > b.L; });
    // a phase with fewer nodes than one unit slot per warp is latency-bound: short
    // chains there are walked serially (C_narrow) rather than scanned
    int64_t phase_nodes = 0;
    for (const CRef& c : v) phase_nodes += c.L;
    const int C = phase_nodes < int64_t(32) * W ? C_narrow : C_wide;
    std::vector<Slot> ps;
    // chains longer than a lane's share: split into near-equal parts over lanes
    std::vector<Lane> lanes;
    for (const CRef& c : v) {
      if (c.L > C) {
        int32_t m = (c.L + C - 1) / C;
        int32_t chunk = C;
        if (m > 32) {
          chunk = (c.L + 31) / 32;
          m = (c.L + chunk - 1) / chunk;
        }
        std::vector<int32_t> sizes(m);
        for (int32_t q = 0; q < m; ++q) sizes[q] = int32_t(int64_t(c.L) * (q + 1) / m - int64_t(c.L) * q / m);
        int32_t st = 0;
        while ((1 << st) < m) ++st;
        Slot* tgt = nullptr;
        for (Slot& s : ps)
          if (s.scan && s.used + m <= 32) {
            tgt = &s;
            break;
          }
        if (!tgt) {
          ps.emplace_back();
          tgt = &ps.back();
          tgt->scan = true;
        }
        tgt->spread.push_back(c);
        tgt->parts.push_back(sizes);
        tgt->used += m;
        tgt->steps = std::max(tgt->steps, st);
        tgt->cost = std::max<int32_t>(tgt->cost, 4 * sizes[0] + 8 * st);
        continue;
      }
      // whole chain: first lane with room (lanes fill to C nodes)
      bool placed = false;
      for (Lane& ln : lanes)
        if (ln.nodes + c.L <= C) {
          ln.whole.push_back(c);
          ln.nodes += c.L;
          placed = true;
          break;
        }
      if (!placed) {
        Lane ln;
        ln.whole.push_back(c);
        ln.nodes = c.L;
        lanes.push_back(std::move(ln));
      }
    }
    for (size_t q = 0; q < lanes.size(); q += 32) {
      Slot s;
      for (size_t r = q; r < std::min(lanes.size(), q + 32); ++r) {
        s.cost = std::max<int32_t>(s.cost, 2 * lanes[r].nodes);
        s.lanes.push_back(std::move(lanes[r]));
      }
      s.used = int32_t(s.lanes.size());
      ps.push_back(std::move(s));
    }
    // dearest slots first: warp w takes slots w, w + W, ...
    std::stable_sort(ps.begin(), ps.end(), [](const Slot& a, const Slot& b) { return a.cost > b.cost; });
    std::vector<int64_t> warp_cost(W, 0);
    phase_ptr[p] = int32_t(slots.size());
    for (size_t si = 0; si < ps.size(); ++si) {
      const Slot& s = ps[si];
      SlotRec sr{};
      sr.n_begin = next_node;
      sr.steps = uint8_t(s.scan ? std::max(1, s.steps) : 0);
      int lane = 0;
      auto emit_chain = [&](const CRef& c) {
        const Chain& ch = (*cx.sched)[cell_list[c.li]].chains[c.chain];
        ChainRec rec{};
        rec.start = next_node;
        rec.count = c.L;
        rec.kind = kChainRegular;
        rec.slot = -1;
        for (int32_t q = 0; q < c.L; ++q) node_tile[c.li][ch.nodes[q]] = next_node++;
        handle[c.li][c.chain] = int32_t(chains.size());
        chains.push_back(rec);
        rec_src.push_back({c.li, c.chain, kChainRegular, 0, 1, 0, c.L});
      };
      if (s.scan) {
        for (size_t ci = 0; ci < s.spread.size(); ++ci) {
          const int32_t base = next_node - sr.n_begin;
          int32_t o = base;
          for (int32_t sz : s.parts[ci]) {
            sr.off[lane++] = uint16_t(o);
            o += sz;
          }
          emit_chain(s.spread[ci]);
        }
      } else {
        for (const Lane& ln : s.lanes) {
          sr.off[lane++] = uint16_t(next_node - sr.n_begin);
          for (const CRef& c : ln.whole) emit_chain(c);
        }
      }
      if (next_node - sr.n_begin > 0x7fff) return fail(BC_ERR_CAPACITY, "a warp slot holds more than 32767 nodes");
      sr.n_count = int16_t(next_node - sr.n_begin);
      sr.unit = uint8_t(s.scan && sr.n_count == lane ? 1 : 0);
      for (; lane < 32; ++lane) sr.off[lane] = uint16_t(sr.n_count);
      slots.push_back(sr);
      warp_cost[si % W] += s.cost;
    }
    crit += *std::max_element(warp_cost.begin(), warp_cost.end());
  }
  phase_ptr[n_phases] = int32_t(slots.size());
  out.crit = crit;
  // lane tile: node v of the cell in lane l is tile node v * T + l
  std::vector<int32_t> lane_n;
  int32_t lane_kmax = 0;
  if (lane) {
    if (int64_t(cell_list.size()) > T) return fail(BC_ERR_INVALID, "internal: lane tile with more cells than threads");
    lane_n.assign(size_t(T), 0);
    for (size_t li = 0; li < cell_list.size(); ++li) {
      const LoweredCell& lc = (*cx.cells)[cell_list[li]];
      lane_n[li] = lc.n_node;
      lane_kmax = std::max(lane_kmax, lc.n_node);
      for (int32_t v = 0; v < lc.n_node; ++v) node_tile[li][v] = v * T + int32_t(li);
    }
    if (lane_kmax >= 0xFFFF) return fail(BC_ERR_CAPACITY, "a lane-tile cell has too many nodes");
    n_real = int64_t(lane_kmax) * T;
    out.crit = lane_kmax;
  }
  if (chains.size() >= 0xFFFF) return fail(BC_ERR_CAPACITY, "too many chains in one tile");
  // -------- links: parents and contribution slots
  // A record owns the consecutive contribution slots aux .. aux + n_child, one per
  // child chain; each child writes its (cD, cR) into its own slot.
  int32_t n_slots = 0;
  for (size_t k = 0; k < chains.size(); ++k) {
    const RecSpec& rsp = rec_src[k];
    const LoweredCell& lc = (*cx.cells)[cell_list[rsp.li]];
    const Chain& ch = (*cx.sched)[cell_list[rsp.li]].chains[rsp.chain];
    const int32_t chain_top_parent = lc.parent[ch.nodes.back()];
    ChainRec& rec = chains[k];
    rec.top_parent = chain_top_parent >= 0 ? node_tile[rsp.li][chain_top_parent] : -1;
    rec.first = 1;
    rec.aux = n_slots;
    rec.n_child = int32_t(ch.kids.size());
    n_slots += rec.n_child;
  }
  for (size_t k = 0; k < chains.size(); ++k) {
    const RecSpec& rsp = rec_src[k];
    const Chain& ch = (*cx.sched)[cell_list[rsp.li]].chains[rsp.chain];
    for (size_t j = 0; j < ch.kids.size(); ++j) {
      const int32_t kid_rec = handle[rsp.li][ch.kids[j]];
      if (kid_rec < 0) return fail(BC_ERR_INVALID, "internal: unresolved chain link");
      chains[kid_rec].slot = chains[k].aux + int32_t(j);
    }
  }
  // per-node record index
  std::vector<uint16_t> crec(size_t(n_real), 0);
  for (size_t k = 0; k < chains.size(); ++k)
    for (int32_t q = 0; q < chains[k].count; ++q) crec[size_t(chains[k].start + q)] = uint16_t(k);
  if (lane) {  // lane tiles: the parent's node index v within the cell (0xFFFF at the root)
    for (size_t li = 0; li < cell_list.size(); ++li) {
      const LoweredCell& lc = (*cx.cells)[cell_list[li]];
      for (int32_t v = 0; v < lc.n_node; ++v)
        crec[size_t(node_tile[li][v])] = lc.parent[v] >= 0 ? uint16_t(lc.parent[v]) : uint16_t(0xFFFF);
    }
  }
  // -------- special nodes: clamp pulses (sorted by node) and probes
  std::vector<std::pair<int32_t, int64_t>> tpulse, tprobe;  // (tile node, pulse / probe id)
  for (size_t li = 0; li < cell_list.size(); ++li) {
    const int64_t c = cell_list[li];
    const auto& pl = (*cx.cell_pulses)[c];
    const auto& pn = (*cx.pulse_node)[c];
    for (size_t k = 0; k < pl.size(); ++k) tpulse.push_back({node_tile[li][pn[k]], pl[k]});
    const auto& ql = (*cx.cell_probes)[c];
    const auto& qn = (*cx.probe_node)[c];
    for (size_t k = 0; k < ql.size(); ++k) tprobe.push_back({node_tile[li][qn[k]], ql[k]});
  }
  std::vector<std::pair<int32_t, int64_t>> tsyn;  // (tile node, synapse id)
  bool has_src = false;
  for (size_t li = 0; li < cell_list.size(); ++li) {
    const int64_t c = cell_list[li];
    for (const auto& sv : (*cx.cell_syns)[c]) tsyn.push_back({node_tile[li][sv.second], sv.first});
    has_src = has_src || (*cx.is_src)[c];
  }
  std::stable_sort(tsyn.begin(), tsyn.end(),
                   [](const std::pair<int32_t, int64_t>& x, const std::pair<int32_t, int64_t>& y) { return x.first < y.first; });
  std::stable_sort(tpulse.begin(), tpulse.end(),
                   [](const std::pair<int32_t, int64_t>& x, const std::pair<int32_t, int64_t>& y) { return x.first < y.first; });
  std::sort(tprobe.begin(), tprobe.end());
  std::vector<int32_t> spec_nodes;
  for (auto& x : tpulse) spec_nodes.push_back(x.first);
  for (auto& x : tprobe) spec_nodes.push_back(x.first);
  for (auto& x : tsyn) spec_nodes.push_back(x.first);
  std::sort(spec_nodes.begin(), spec_nodes.end());
  spec_nodes.erase(std::unique(spec_nodes.begin(), spec_nodes.end()), spec_nodes.end());
  if (spec_nodes.size() >= 0xFFFF) return fail(BC_ERR_CAPACITY, "too many clamped / probed / synapse points in one tile");
  if (cell_list.size() >= 0xFFFF) return fail(BC_ERR_CAPACITY, "too many cells in one tile");
  // -------- layout
  const int64_t N = (n_real + 3) & ~int64_t(3);
  const int S = cx.state_slots;
  const int64_t n_params = int64_t(cell_list.size()) * R;
  if (n_params >= 0xFFFF) return fail(BC_ERR_CAPACITY, "too many parameter records in one tile");
  TileDesc d{};
  d.param_stride = cx.param_stride;
  size_t off = 0;
  d.off_v = int32_t(off);
  off = align16(off + 2 * N * rs);
  d.dyn_bytes = int32_t(off);
  d.off_ab = int32_t(off);
  off = align16(off + 2 * N * rs);
  d.off_diag0 = int32_t(off);
  off = align16(off + N * rs);
  d.off_pidx = int32_t(off);
  off = align16(off + N * 2);
  d.off_spec = int32_t(off);
  off = align16(off + N * 2);
  d.off_specs = int32_t(off);
  off = align16(off + spec_nodes.size() * sizeof(SpecRec));
  d.off_chains = int32_t(off);
  off = align16(off + chains.size() * sizeof(ChainRec));
  d.off_slots = int32_t(off);
  off = align16(off + slots.size() * sizeof(SlotRec));
  d.off_phase = int32_t(off);
  off = align16(off + phase_ptr.size() * 4);
  d.off_crec = int32_t(off);
  off = align16(off + N * 2);
  d.off_params = int32_t(off);
  off = align16(off + size_t(n_params) * cx.param_stride * rs);
  d.off_mech = int32_t(off);
  off = align16(off + size_t(n_params) * 4);
  d.off_syn = int32_t(off);
  off = align16(off + tsyn.size() * 4);
  d.off_plist = int32_t(off);
  off = align16(off + tprobe.size() * sizeof(ProbeRef));
  d.off_lane_n = -1;
  d.lane_kmax = lane_kmax;
  if (lane) {
    d.off_lane_n = int32_t(off);
    off = align16(off + size_t(T) * 4);
  }
  d.n_cells = int32_t(cell_list.size());
  d.off_ncell = -1;
  d.off_srccell = -1;
  if (has_src) {
    d.off_ncell = int32_t(off);
    off = align16(off + size_t(N) * 2);
    d.off_srccell = int32_t(off);
    off = align16(off + cell_list.size() * 4);
  }
  if (off > size_t(0x7fffffff)) return fail(BC_ERR_CAPACITY, "tile blob exceeds 2 GiB");
  d.blob_bytes = int32_t(off);
  size_t so = 0;
  d.off_dr = int32_t(so);
  so = align16(so + 2 * N * rs);
  d.off_scd = int32_t(so);
  so = align16(so + size_t(std::max(n_slots, 1)) * rs);
  d.off_scr = int32_t(so);
  so = align16(so + size_t(std::max(n_slots, 1)) * rs);
  d.n_slots = n_slots;
  d.off_stamp = -1;
  if (has_src) {
    d.off_stamp = int32_t(so);
    so = align16(so + cell_list.size() * 4);
  }
  size_t n_tile_ports = 0;
  for (size_t li = 0; li < cell_list.size(); ++li) n_tile_ports += (*cx.cell_ports)[cell_list[li]].size();
  d.off_pstage = -1;
  if (n_tile_ports > 0) {
    d.off_pstage = int32_t(so);
    so = align16(so + size_t(kGruSmemBytes) + n_tile_ports * (sizeof(PortStage) + sizeof(PortLocal)));
  }
  d.scratch_bytes = int32_t(so);
  d.n_nodes = int32_t(N);
  d.n_real_nodes = int32_t(n_real);
  d.n_chains = int32_t(chains.size());
  d.n_phases = n_phases;
  d.n_params = int32_t(n_params);
  // -------- fill
  std::vector<unsigned char>& b = out.blob;
  b.assign(d.blob_bytes, 0);
  out.vinit.assign(n_real, 0.0);
  if (lane) {  // holes of the lane grid are boundary rows the kernel never visits
    std::vector<uint16_t> hole(size_t(N), 0xFFFF);
    std::memcpy(b.data() + d.off_pidx, hole.data(), hole.size() * 2);
    std::memcpy(b.data() + d.off_lane_n, lane_n.data(), lane_n.size() * 4);
  }
  auto putr = [&](size_t base_off, size_t idx, double v) {
    if (rs == 8)
      put<double>(b, base_off, idx, v);
    else
      put<float>(b, base_off, idx, float(v));
  };
  for (size_t li = 0; li < cell_list.size(); ++li) {
    const int64_t c = cell_list[li];
    const LoweredCell& lc = (*cx.cells)[c];
    for (int32_t v = 0; v < lc.n_node; ++v) {
      const int32_t j = node_tile[li][v];
      putr(d.off_v, 2 * size_t(j), lc.node_vrest[v]);
      putr(d.off_ab, 2 * size_t(j), lc.alpha[v]);
      putr(d.off_ab, 2 * size_t(j) + 1, lc.beta[v]);
      putr(d.off_diag0, j, lc.diag[v]);
      const uint16_t pi = lc.region[v] >= 0 ? uint16_t(li * R + lc.region[v]) : uint16_t(0xFFFF);
      std::memcpy(b.data() + d.off_pidx + size_t(j) * 2, &pi, 2);
      out.vinit[j] = lc.node_vrest[v];
    }
    for (int r = 0; r < R; ++r) {
      const int64_t rc = c * R + r;
      for (int k = 0; k < std::min(BC_NPARAM, cx.param_stride - 1); ++k)
        putr(d.off_params, (li * R + r) * cx.param_stride + k, s.region_params[rc * BC_NPARAM + k]);
      const uint32_t m = s.region_mech[rc];
      std::memcpy(b.data() + d.off_mech + (li * R + r) * 4, &m, 4);
    }
    // CV view map
    const int64_t base = (*cx.cv_base)[c];
    for (int32_t k = 0; k < lc.n_cv; ++k) {
      const int32_t v = lc.cv_node[k];
      out.cv_local.push_back({base + k, node_tile[li][v]});
      out.cv_mech.push_back(region_bits(s, c * R + lc.region[v]));
    }
  }
  // special records: pulses in node order, probe ids
  {
    std::vector<uint16_t> spec(N, 0xFFFF);
    std::vector<SpecRec> specs(spec_nodes.size());
    std::vector<int32_t> node_cell(n_real, -1), node_local(n_real, -1);
    for (size_t li = 0; li < cell_list.size(); ++li) {
      const LoweredCell& lc = (*cx.cells)[cell_list[li]];
      for (int32_t v = 0; v < lc.n_node; ++v) {
        node_cell[node_tile[li][v]] = int32_t(li);
        node_local[node_tile[li][v]] = v;
      }
    }
    for (size_t q = 0; q < spec_nodes.size(); ++q) {
      spec[spec_nodes[q]] = uint16_t(q);
      specs[q] = SpecRec{0, 0, -1, 0, 0, {0, 0, 0}};
    }
    size_t kp = 0;
    for (size_t q = 0; q < spec_nodes.size(); ++q) {
      const int32_t node = spec_nodes[q];
      specs[q].pulse_begin = int32_t(out.pulses.size());
      while (kp < tpulse.size() && tpulse[kp].first == node) {
        const int64_t pid = tpulse[kp].second;
        const size_t li = size_t(node_cell[node]);
        const LoweredCell& lc = (*cx.cells)[cell_list[li]];
        const int32_t v = node_local[node];
        PulseRec pr{};
        pr.node = node;
        pr.is_mid = lc.region[v] >= 0 ? 1 : 0;
        if (pr.is_mid) {
          double area = 0.0;
          for (int32_t k = 0; k < lc.n_cv; ++k)
            if (lc.cv_node[k] == v) {
              area = lc.cv_area[k];
              break;
            }
          out.pulse_scale.push_back(1e5 / area);  // nA -> uA/cm^2
        } else {
          out.pulse_scale.push_back(1e-3);  // nA -> mV/ms on a row with the 1 uF dummy capacitance
        }
        pr.amp = s.pulse_amp[pid] * out.pulse_scale.back();
        pr.t_on = s.pulse_t_on[pid];
        pr.t_off = s.pulse_t_off[pid];
        out.pulses.push_back(pr);
        out.pulse_src.push_back(pid);
        ++kp;
      }
      specs[q].pulse_end = int32_t(out.pulses.size());
    }
    size_t ks = 0;
    for (size_t q = 0; q < spec_nodes.size(); ++q) {
      specs[q].syn_begin = int32_t(ks);
      while (ks < tsyn.size() && tsyn[ks].first == spec_nodes[q]) ++ks;
      specs[q].syn_end = int32_t(ks);
    }
    std::vector<int32_t> syn_ids(tsyn.size());
    for (size_t k = 0; k < tsyn.size(); ++k) syn_ids[k] = int32_t(tsyn[k].second);
    if (!syn_ids.empty()) std::memcpy(b.data() + d.off_syn, syn_ids.data(), syn_ids.size() * 4);
    if (has_src) {
      std::vector<uint16_t> ncell(N, 0xFFFF);
      std::vector<int32_t> src(cell_list.size(), -1);
      for (int64_t j = 0; j < n_real; ++j) ncell[j] = uint16_t(node_cell[j]);
      for (size_t li = 0; li < cell_list.size(); ++li)
        if ((*cx.is_src)[cell_list[li]]) src[li] = int32_t(cell_list[li]);
      std::memcpy(b.data() + d.off_ncell, ncell.data(), ncell.size() * 2);
      std::memcpy(b.data() + d.off_srccell, src.data(), src.size() * 4);
    }
    {
      // probes in node order (tprobe is sorted): each special node owns a range
      std::vector<ProbeRef> plist;
      for (const auto& x : tprobe) {
        const int64_t pid = x.second;
        const int32_t field = s.probe_field ? s.probe_field[pid] : BC_STATE_V;
        if (field != BC_STATE_V) {
          plist.push_back(ProbeRef{x.first, int32_t(pid), field, 0});
        } else {
          SpecRec& sr = specs[spec[x.first]];
          if (sr.probe >= 0) return fail(BC_ERR_INVALID, "two voltage probes at the same point of a cell are not supported");
          sr.probe = int32_t(pid);
        }
      }
      d.n_xprobes = int32_t(plist.size());
      if (!plist.empty()) std::memcpy(b.data() + d.off_plist, plist.data(), plist.size() * sizeof(ProbeRef));
    }
    std::memcpy(b.data() + d.off_spec, spec.data(), spec.size() * 2);
    if (!specs.empty()) std::memcpy(b.data() + d.off_specs, specs.data(), specs.size() * sizeof(SpecRec));
  }
  // surrogate ports of the tile's cells (the plan assigns port_offset)
  for (size_t li = 0; li < cell_list.size(); ++li) {
    const int64_t c = cell_list[li];
    for (const auto& pt : (*cx.cell_ports)[c]) {
      PortRec r{};
      r.node = node_tile[li][pt[1]];
      r.att = node_tile[li][pt[2]];
      r.cell = int32_t(c);
      r.id = pt[0];
      r.g = s.port_g[pt[0]];
      r.e = s.port_e[pt[0]];
      r.feat[0] = float(s.port_feat[2 * size_t(pt[0])]);
      r.feat[1] = float(s.port_feat[2 * size_t(pt[0]) + 1]);
      r.stim_begin = int32_t(out.port_pulses.size());
      for (int64_t q : (*cx.port_pulse_ids)[pt[0]]) {
        PulseRec pr{};
        pr.node = r.node;
        pr.amp = s.port_pulse_amp[q];
        pr.t_on = s.port_pulse_t_on[q];
        pr.t_off = s.port_pulse_t_off[q];
        out.port_pulses.push_back(pr);
      }
      r.stim_end = int32_t(out.port_pulses.size());
      out.ports.push_back(r);
    }
  }
  d.n_ports = int32_t(out.ports.size());
  std::memcpy(b.data() + d.off_chains, chains.data(), chains.size() * sizeof(ChainRec));
  if (!slots.empty()) std::memcpy(b.data() + d.off_slots, slots.data(), slots.size() * sizeof(SlotRec));
  std::memcpy(b.data() + d.off_phase, phase_ptr.data(), phase_ptr.size() * 4);
  std::memcpy(b.data() + d.off_crec, crec.data(), crec.size() * 2);
  out.desc = d;
  return BC_OK;
}

static size_t max_optin_smem(int device) {
  int v = 0;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess) return 0;
  return size_t(v);
}

static size_t sm_smem(int device) {
  int v = 0;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device) != cudaSuccess) return 0;
  return size_t(v);
}

// First step index s with s * dt >= t (float64), for clamp windows.
static int64_t first_step_at(double t, double dt) {
  if (t <= 0.0) return 0;
  int64_t s = int64_t(std::floor(t / dt));
  if (s < 0) s = 0;
  while (s > 0 && double(s - 1) * dt >= t) --s;
  while (double(s) * dt < t) ++s;
  return s;
}

static bc_status update_pulses(bc_plan* p, double dt, void* stream) {
  if (!p->port_pulses.empty() && p->port_pulses_dt != dt) {
    for (auto& pr : p->port_pulses) {
      pr.on_step = first_step_at(pr.t_on, dt);
      pr.off_step = first_step_at(pr.t_off, dt);
    }
    BC_CUDA(cudaMemcpyAsync(p->d_port_pulses, p->port_pulses.data(), p->port_pulses.size() * sizeof(PulseRec),
                            cudaMemcpyHostToDevice, static_cast<cudaStream_t>(stream)));
    BC_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    p->port_pulses_dt = dt;
  }
  if (p->pulses.empty() || p->pulses_dt == dt) return BC_OK;
  for (auto& pr : p->pulses) {
    pr.on_step = first_step_at(pr.t_on, dt);
    pr.off_step = first_step_at(pr.t_off, dt);
  }
  BC_CUDA(cudaMemcpyAsync(p->d_pulses, p->pulses.data(), p->pulses.size() * sizeof(PulseRec), cudaMemcpyHostToDevice,
                          static_cast<cudaStream_t>(stream)));
  BC_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
  p->pulses_dt = dt;
  return BC_OK;
}

static bc_status ensure_traces(bc_plan* p, int64_t records, void* stream) {
  if (p->n_probes == 0 || records <= p->trace_cap) return BC_OK;
  int64_t cap = std::max<int64_t>(records, p->trace_cap * 2);
  double* nb = nullptr;
  BC_CUDA(cudaMalloc(reinterpret_cast<void**>(&nb), size_t(cap) * p->n_probes * sizeof(double)));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (p->d_traces && p->trace_cap > 0) {
    BC_CUDA(cudaMemcpyAsync(nb, p->d_traces, size_t(p->trace_cap) * p->n_probes * sizeof(double),
                            cudaMemcpyDeviceToDevice, st));
    BC_CUDA(cudaStreamSynchronize(st));
  }
  cudaFree(p->d_traces);
  p->device_bytes += size_t(cap - p->trace_cap) * p->n_probes * sizeof(double);
  p->d_traces = nb;
  p->trace_cap = cap;
  return BC_OK;
}

// Kernel variant of a plan (see launch_tiles).
static int kernel_variant(const bc_plan* p) {
  if (p->n_ports > 0) return p->extra ? BC_VARIANT_PORTS : BC_VARIANT_PORTS_LEAN;
  return p->extra ? BC_VARIANT_EXTRA : BC_VARIANT_LEAN;
}

static LaunchArgs base_args(bc_plan* p) {
  LaunchArgs a{};
  a.blob = p->d_blob;
  a.scratch = p->d_scratch;
  a.state = p->d_state;
  a.pulses = p->d_pulses;
  a.traces = p->d_traces;
  a.trace_cap = p->trace_cap;
  a.trace_base = p->trace_origin;
  a.n_probes_total = p->n_probes;
  a.record_every = p->record_every;
  a.max_spikes = p->max_spikes;
  a.spike_count = p->d_spike_count;
  a.spike_times = p->d_spike_times;
  a.status = p->d_status;
  a.state_slots = p->state_slots;
  a.timers = p->d_timers;
  a.syn_g = p->d_syn_g;
  a.syn_tau = p->d_syn_tau;
  a.syn_e = p->d_syn_e;
  a.syn_scale = p->d_syn_scale;
  a.arrivals = p->n_connections > 0 ? p->d_arrivals : nullptr;
  a.arr_slots = std::max<int64_t>(p->arr_slots, 1);
  a.n_syn = p->n_synapses;
  a.rec_cell = p->d_rec_cell;
  a.rec_step = p->d_rec_step;
  a.rec_count = p->d_rec_count;
  a.rec_cap = p->rec_cap;
  a.ports = p->d_ports;
  a.port_pulses = p->d_port_pulses;
  a.port_h = p->d_port_h;
  a.port_flags = p->d_port_flags;
  a.gru = p->d_gru;
  return a;
}

// Delays in whole steps for dt (network/lowering.py:185-226, "ceil": delays within
// 1e-7 of a whole number of steps count as that number), and the arrival ring:
// launches of at most the shortest delay (so a launch never receives an event its
// own spikes cause) and room for the longest delay past the current launch.
static bc_status prepare_network(bc_plan* p, double dt, void* stream) {
  if (p->n_connections == 0 || p->net_dt == dt) return BC_OK;
  if (p->net_dt != 0.0 && p->step != 0)
    return fail(BC_ERR_INVALID, "a network plan keeps its dt between resets; call bc_reset before changing dt");
  std::vector<int32_t> d(p->n_connections);
  int64_t dmin = INT64_MAX, dmax = 1;
  for (int64_t q = 0; q < p->n_connections; ++q) {
    double raw = p->conn_delay[p->out_order[q]] / dt;
    const double near = std::nearbyint(raw);
    if (std::fabs(raw - near) <= 1e-7 + 1e-7 * std::fabs(near)) raw = near;
    const double st = std::ceil(raw - 1e-12);
    if (st > 1e9) return fail(BC_ERR_INVALID, "connection delay too long for this dt");
    d[q] = int32_t(st);
    const int64_t eff = std::max<int64_t>(d[q], 1);
    dmin = std::min(dmin, eff);
    dmax = std::max(dmax, eff);
  }
  const int64_t k = std::min<int64_t>(p->steps_per_launch, dmin);
  const int64_t slots = k + dmax + 1;
  const size_t rs = p->real_size;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  BC_CUDA(cudaStreamSynchronize(s));
  cudaFree(p->d_arrivals);
  p->d_arrivals = nullptr;
  const size_t bytes = size_t(slots) * size_t(std::max<int64_t>(p->n_synapses, 1)) * rs;
  BC_CUDA(cudaMalloc(&p->d_arrivals, bytes));
  BC_CUDA(cudaMemsetAsync(p->d_arrivals, 0, bytes, s));
  BC_CUDA(cudaMemcpyAsync(p->d_out_d, d.data(), d.size() * 4, cudaMemcpyHostToDevice, s));
  BC_CUDA(cudaStreamSynchronize(s));
  p->arr_slots = slots;
  p->net_k = k;
  p->net_dt = dt;
  return BC_OK;
}

// The launches of one run as a CUDA graph: each launch class is a chain of
// kernel nodes (the classes hold independent cells, so the chains run side by
// side).  The graph is built when the number of launches or their step counts
// change; otherwise only the kernel arguments (first step, trace buffer, ...)
// of its nodes are updated before the replay.
static bc_status enqueue_run_graph(bc_plan* p, int64_t n_steps, double dt, void* stream) {
  const int32_t K = p->steps_per_launch;
  const int64_t L = (n_steps + K - 1) / K;
  const int32_t k_last = int32_t(n_steps - (L - 1) * K);
  const int nc = int(p->classes.size());
  std::vector<LaunchArgs> args(size_t(L) * nc);
  for (int64_t j = 0; j < L; ++j)
    for (int ci = 0; ci < nc; ++ci) {
      LaunchArgs a = base_args(p);
      a.step0 = p->step + j * K;
      a.n_steps = j + 1 == L ? k_last : K;
      a.dt = dt;
      a.tiles = p->d_tiles + p->classes[ci].first;
      a.n_tiles = p->classes[ci].count;
      args[size_t(j) * nc + ci] = a;
    }
  const bool rebuild = !p->graph_exec || p->graph_launches != L || p->graph_k != K || p->graph_k_last != k_last;
  if (rebuild) {
    if (p->graph_exec) cudaGraphExecDestroy(p->graph_exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    p->graph_exec = nullptr;
    p->graph = nullptr;
    p->graph_launches = -1;
    BC_CUDA(cudaGraphCreate(&p->graph, 0));
    p->graph_nodes.assign(size_t(L) * nc, nullptr);
    for (int64_t j = 0; j < L; ++j)
      for (int ci = 0; ci < nc; ++ci) {
        const LaunchClass& lcz = p->classes[ci];
        cudaKernelNodeParams np{};
        const LaunchArgs* hold = nullptr;
        int e = lcz.lane ? lane_node_params(&args[size_t(j) * nc + ci], p->precision, lcz.threads, p->extra, &np, &hold)
                         : tile_node_params(&args[size_t(j) * nc + ci], p->precision, lcz.smem, lcz.threads, lcz.smem_bytes,
                                            kernel_variant(p), &np, &hold);
        if (e) return fail(BC_ERR_CUDA, std::string("graph node: ") + cudaGetErrorString(cudaError_t(e)));
        cudaGraphNode_t dep = j > 0 ? p->graph_nodes[size_t(j - 1) * nc + ci] : nullptr;
        BC_CUDA(cudaGraphAddKernelNode(&p->graph_nodes[size_t(j) * nc + ci], p->graph, dep ? &dep : nullptr,
                                       dep ? 1 : 0, &np));
      }
    BC_CUDA(cudaGraphInstantiate(&p->graph_exec, p->graph, 0));
    p->graph_launches = L;
    p->graph_k = K;
    p->graph_k_last = k_last;
  } else {
    for (int64_t j = 0; j < L; ++j)
      for (int ci = 0; ci < nc; ++ci) {
        const LaunchClass& lcz = p->classes[ci];
        cudaKernelNodeParams np{};
        const LaunchArgs* hold = nullptr;
        int e = lcz.lane ? lane_node_params(&args[size_t(j) * nc + ci], p->precision, lcz.threads, p->extra, &np, &hold)
                         : tile_node_params(&args[size_t(j) * nc + ci], p->precision, lcz.smem, lcz.threads, lcz.smem_bytes,
                                            kernel_variant(p), &np, &hold);
        if (e) return fail(BC_ERR_CUDA, std::string("graph node: ") + cudaGetErrorString(cudaError_t(e)));
        BC_CUDA(cudaGraphExecKernelNodeSetParams(p->graph_exec, p->graph_nodes[size_t(j) * nc + ci], &np));
      }
  }
  BC_CUDA(cudaGraphLaunch(p->graph_exec, static_cast<cudaStream_t>(stream)));
  return BC_OK;
}

static bc_status enqueue_run(bc_plan* p, int64_t n_steps, double dt, void* stream) {
  if (n_steps < 0) return fail(BC_ERR_INVALID, "n_steps must be >= 0");
  if (!(dt > 0.0) || !std::isfinite(dt)) return fail(BC_ERR_INVALID, "dt must be a positive finite number (ms)");
  if (p->n_ports > 0 && !p->gru_set) return fail(BC_ERR_INVALID, "the plan has surrogate ports: call bc_surrogate_set first");
  bc_status st = update_pulses(p, dt, stream);
  if (st != BC_OK) return st;
  const int64_t recs = p->record_every > 0 ? (p->step + n_steps - p->trace_origin) / p->record_every : 0;
  st = ensure_traces(p, recs, stream);
  if (st != BC_OK) return st;
  st = prepare_network(p, dt, stream);
  if (st != BC_OK) return st;
  const bool net = p->n_connections > 0;
  if (p->use_graph && n_steps > 0 && !net) {
    st = enqueue_run_graph(p, n_steps, dt, stream);
    if (st == BC_OK) p->step += n_steps;
    return st;
  }
  const int64_t per_launch = net ? std::min<int64_t>(p->steps_per_launch, p->net_k) : p->steps_per_launch;
  if (p->classes.size() > 1) {
    // the forked class streams take the priority of the caller's stream; work still
    // queued on the streams they replace completes, and this run's forks are ordered
    // after it through the caller's stream (the last run joined into it)
    int prio = 0;
    BC_CUDA(cudaStreamGetPriority(static_cast<cudaStream_t>(stream), &prio));
    if (prio != p->aux_prio) {
      for (int k = 0; k < kMaxClasses - 1; ++k) {
        cudaStream_t ns = nullptr;
        BC_CUDA(cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, prio));
        if (p->aux[k]) cudaStreamDestroy(p->aux[k]);
        p->aux[k] = ns;
      }
      p->aux_prio = prio;
    }
  }
  int64_t done = 0;
  while (done < n_steps) {
    const int32_t k = int32_t(std::min<int64_t>(per_launch, n_steps - done));
    LaunchArgs a = base_args(p);
    a.step0 = p->step + done;
    a.n_steps = k;
    a.dt = dt;
    // Classes are independent cells: the first runs on the caller's stream, the
    // others on forked streams so their CTAs can share SMs.
    cudaStream_t main_st = static_cast<cudaStream_t>(stream);
    const int nc = int(p->classes.size());
    if (nc > 1) BC_CUDA(cudaEventRecord(p->ev_fork, main_st));
    for (int ci = 0; ci < nc; ++ci) {
      const LaunchClass& lcz = p->classes[ci];
      cudaStream_t st = main_st;
      if (ci > 0) {
        st = p->aux[ci - 1];
        BC_CUDA(cudaStreamWaitEvent(st, p->ev_fork, 0));
      }
      a.tiles = p->d_tiles + lcz.first;
      a.n_tiles = lcz.count;
      int e = lcz.lane ? launch_lanes(a, p->precision, lcz.threads, p->extra, st)
                       : launch_tiles(a, p->precision, lcz.smem, lcz.threads, lcz.smem_bytes, kernel_variant(p), st);
      if (e) return fail(BC_ERR_CUDA, std::string("tile kernel launch: ") + cudaGetErrorString(cudaError_t(e)));
      if (ci > 0) {
        BC_CUDA(cudaEventRecord(p->ev_join[ci - 1], st));
        BC_CUDA(cudaStreamWaitEvent(main_st, p->ev_join[ci - 1], 0));
      }
    }
    if (net) {
      // deliver this launch's spikes into the arrival ring, then mark them delivered
      int e = launch_deliver_impl(p->precision, p->d_rec_cell, p->d_rec_step, p->d_rec_count, p->d_rec_count + 1,
                                  p->rec_cap, p->d_out_ptr, p->d_out_syn, p->d_out_w, p->d_out_d, p->d_arrivals,
                                  p->arr_slots, p->n_synapses, stream);
      if (e) return fail(BC_ERR_CUDA, std::string("delivery kernel: ") + cudaGetErrorString(cudaError_t(e)));
      BC_CUDA(cudaMemcpyAsync(p->d_rec_count + 1, p->d_rec_count, sizeof(unsigned long long),
                              cudaMemcpyDeviceToDevice, main_st));
    }
    done += k;
  }
  p->step += n_steps;
  return BC_OK;
}

}  // namespace bc

using namespace bc;

extern "C" {

const char* bc_last_error(void) { return g_error.c_str(); }

int32_t bc_version(void) { return BC_ABI_VERSION; }

void bc_default_options(bc_plan_options* o) {
  std::memset(o, 0, sizeof(*o));
  o->precision = BC_PREC_F32;
  o->threads_per_tile = 0;
  o->tile_nodes = 0;
  o->lane_nodes = kDefaultLaneNodes;
  o->narrow_lane_nodes = kDefaultNarrowLaneNodes;
  o->steps_per_launch = 0;
  o->record_every = 1;
  o->max_spikes = 64;
  o->use_graph = 0;
  o->device = 0;
}

bc_status bc_plan_create(const bc_batch_spec* spec, const bc_plan_options* opts_in, bc_plan_t* out) {
  if (!spec || !out) return fail(BC_ERR_INVALID, "null argument");
  *out = nullptr;
  bc_plan_options opts;
  if (opts_in)
    opts = *opts_in;
  else
    bc_default_options(&opts);
  const bc_batch_spec& s = *spec;
  if (s.n_cells <= 0) return fail(BC_ERR_INVALID, "n_cells must be > 0");
  if (s.n_regions <= 0) return fail(BC_ERR_INVALID, "n_regions must be > 0");
  if (opts.precision != BC_PREC_F32 && opts.precision != BC_PREC_F64)
    return fail(BC_ERR_INVALID, "precision must be BC_PREC_F32 or BC_PREC_F64");
  if (opts.tile_order < 0 || opts.tile_order > 1) return fail(BC_ERR_INVALID, "tile_order must be 0 or 1");
  if (opts.threads_per_tile < 0 || opts.threads_per_tile > 1024 || opts.threads_per_tile % 32)
    return fail(BC_ERR_INVALID, "threads_per_tile must be 0 or a multiple of 32 up to 1024");
  if (opts.record_every < 0 || opts.max_spikes < 0) return fail(BC_ERR_INVALID, "record_every/max_spikes must be >= 0");
  if (s.cell_branch_offsets[0] != 0 || s.cell_branch_offsets[s.n_cells] != s.n_branches)
    return fail(BC_ERR_INVALID, "cell_branch_offsets must span [0, n_branches]");
  const bool dry = opts.dry_run != 0;
  if (!dry) BC_CUDA(cudaSetDevice(opts.device));
  bc_plan* p = new bc_plan();
  p->dry = dry;
  p->precision = opts.precision;
  p->device = opts.device;
  p->real_size = opts.precision == BC_PREC_F64 ? 8 : 4;
  p->record_every = opts.record_every;
  p->max_spikes = opts.max_spikes;
  p->use_graph = opts.use_graph;
  p->steps_per_launch = opts.steps_per_launch > 0 ? opts.steps_per_launch : 1000;
  p->lane_nodes = opts.lane_nodes > 0 ? opts.lane_nodes : kDefaultLaneNodes;
  p->narrow_lane_nodes = opts.narrow_lane_nodes > 0 ? opts.narrow_lane_nodes : kDefaultNarrowLaneNodes;
  p->n_cells = s.n_cells;
  // ---------------------------------------------------- lower
  std::vector<LoweredCell> cells(s.n_cells);
  std::vector<int64_t> cv_base(s.n_cells + 1, 0);
  {
    // cells lower independently; the failure reported is that of the first failing
    // cell in cell order, as a sequential pass would report it
    std::vector<bc_status> lst(s.n_cells, BC_OK);
    std::vector<std::string> lmsg(s.n_cells);
    parallel_for(s.n_cells, [&](int64_t c) {
      try {
        lst[c] = lower_cell(s, c, cells[c]);
        if (lst[c] != BC_OK) lmsg[c] = bc_last_error();
      } catch (const std::exception& ex) {
        lst[c] = BC_ERR_CAPACITY;
        lmsg[c] = std::string("lowering cell ") + std::to_string(c) + ": " + ex.what();
      }
    });
    for (int64_t c = 0; c < s.n_cells; ++c) {
      if (lst[c] != BC_OK) {
        delete p;
        return fail(lst[c], lmsg[c]);
      }
      cv_base[c + 1] = cv_base[c] + cells[c].n_cv;
      p->n_nodes += cells[c].n_node;
    }
  }
  p->n_cv = cv_base[s.n_cells];
  p->cell_ncv.resize(s.n_cells);
  for (int64_t c = 0; c < s.n_cells; ++c) p->cell_ncv[c] = cells[c].n_cv;
  for (int64_t k = 0; k < s.n_cells * s.n_regions; ++k)
    p->extra = p->extra || (s.region_mech[k] & (BC_M_NAHH | BC_M_KHH | BC_M_KM | BC_M_KA1 | BC_M_KA2 | BC_M_KK2A |
                                                 BC_M_KK2B | BC_M_KNI | kMarkovBits | kCerebellarBits | BC_M_EXT)) != 0;
  for (int64_t k = 0; k < s.n_cells * s.n_regions; ++k) {
    if (s.region_mech[k] & ~BC_M_ALL) {
      delete p;
      return fail(BC_ERR_INVALID, "unknown mechanism bits in region_mech");
    }
    if (s.region_mech[k] & BC_M_EXT) {
      // the record lists its extension channels: integers of known BC_X_* bits (low 24 and
      // the rest), not all 0
      const double lo = s.region_params[k * BC_NPARAM + BC_P_EXT_MASK];
      const double hi = s.region_params[k * BC_NPARAM + BC_P_EXT_MASK_HI];
      const bool ints = lo >= 0.0 && lo < 16777216.0 && lo == std::floor(lo) && hi >= 0.0 && hi < 256.0 &&
                        hi == std::floor(hi);
      const uint32_t x = ints ? uint32_t(lo) | (uint32_t(hi) << 24) : 0u;
      if (!ints || x == 0u || (x & ~BC_X_ALL)) {
        delete p;
        return fail(BC_ERR_INVALID, "a region with BC_M_EXT needs BC_X_* bits in its record's BC_P_EXT_MASK");
      }
    }
  }
  uint32_t all_bits = 0;
  for (int64_t k = 0; k < s.n_cells * s.n_regions; ++k) all_bits |= s.region_mech[k];
  // the Markov, cerebellar and extension states only where a plan has them
  const int S = (all_bits & BC_M_EXT) ? kNumSlotsExt
                                      : ((all_bits & kCerebellarBits) ? kNumSlotsCerebellar
                                                                      : ((all_bits & kMarkovBits) ? kNumSlotsMarkov : kNumSlots));
  p->state_slots = S;
  // ---------------------------------------------------- pulses / probes -> nodes
  std::vector<std::vector<int64_t>> cell_pulses(s.n_cells), cell_probes(s.n_cells);
  std::vector<std::vector<int32_t>> pulse_node(s.n_cells), probe_node(s.n_cells);
  for (int64_t k = 0; k < s.n_pulses; ++k) {
    const int64_t c = s.pulse_cell[k];
    if (c < 0 || c >= s.n_cells) {
      delete p;
      return fail(BC_ERR_INVALID, "pulse_cell out of range");
    }
    const int32_t v = locate_node(s, c, cells[c], s.pulse_branch[k], s.pulse_x[k]);
    if (v < 0) {
      delete p;
      return fail(BC_ERR_INVALID, "pulse location not found");
    }
    if (!(s.pulse_t_off[k] >= s.pulse_t_on[k])) {
      delete p;
      return fail(BC_ERR_INVALID, "pulse_t_off must be >= pulse_t_on");
    }
    cell_pulses[c].push_back(k);
    pulse_node[c].push_back(v);
  }
  p->probe_vrest.assign(s.n_probes, 0.0);
  for (int64_t k = 0; k < s.n_probes; ++k) {
    const int64_t c = s.probe_cell[k];
    if (c < 0 || c >= s.n_cells) {
      delete p;
      return fail(BC_ERR_INVALID, "probe_cell out of range");
    }
    const int32_t v = locate_node(s, c, cells[c], s.probe_branch[k], s.probe_x[k]);
    if (v < 0) {
      delete p;
      return fail(BC_ERR_INVALID, "probe location not found");
    }
    const int32_t field = s.probe_field ? s.probe_field[k] : BC_STATE_V;
    const bool is_current = field >= BC_PROBE_CURRENT && field < BC_PROBE_CURRENT + BC_NCUR;
    if (!is_current && (field < 0 || field >= BC_NSTATE_VIEW || field == BC_STATE_V_LAST)) {
      delete p;
      return fail(BC_ERR_INVALID, "probe_field is not a recordable BC_STATE_* view or a BC_PROBE_CURRENT code");
    }
    if (is_current) {
      static const uint64_t cur_owner[BC_NCUR] = {
          BC_M_IL,  BC_M_KLEAK, BC_M_NA,   BC_M_KDR, BC_M_CAL,           BC_M_CAT,
          BC_M_HCN, BC_M_AHP,   BC_M_NAHH, BC_M_KHH, BC_M_KM,
          BC_M_NA | BC_M_NAHH | BC_M_NAV16 | ext_bits(BC_X_NAF | BC_X_NAP | BC_X_NAIO | BC_X_NAVGRC),
          BC_M_KDR | BC_M_KLEAK | BC_M_AHP | BC_M_KHH | BC_M_KM | BC_M_KA1 | BC_M_KA2 | BC_M_KK2A | BC_M_KK2B | BC_M_KNI |
              BC_M_KCA22 | BC_M_KCA11 | BC_M_KV34 | BC_M_KV43 | BC_M_KV11 | BC_M_KIR23 |
              ext_bits(BC_X_KV33 | BC_X_KV22 | BC_X_KV15 | BC_X_FKDR | BC_X_SKDR | BC_X_KDRIO | BC_X_KCA31 |
                       BC_X_SKDCN | BC_X_KKV),
          BC_M_CAL | BC_M_CAT | BC_M_CAHVA | BC_M_CAV23 | BC_M_CAV32 | ext_bits(BC_X_CATHP | BC_X_CAHTRE | BC_X_CAN | BC_X_CAV31 | BC_X_CAV33 |
                                                                  BC_X_CAV12 | BC_X_CAV13 | BC_X_CAV21 |
                                                                  BC_X_CAHVADCN | BC_X_CALVADCN),
          BC_M_KA1,  BC_M_KA2, BC_M_KK2A, BC_M_KK2B, BC_M_KNI,
          BC_M_NAV16, BC_M_KCA22, BC_M_KCA11, BC_M_KV34, BC_M_KV43, BC_M_KV11, BC_M_KIR23, BC_M_HCN1F, BC_M_HCN1H,
          BC_M_CAHVA, BC_M_CAV23, BC_M_CAV32,
          ext_bits(BC_X_HCN2), ext_bits(BC_X_KV33), ext_bits(BC_X_KV22), ext_bits(BC_X_KV15), ext_bits(BC_X_NAF),
          ext_bits(BC_X_NAP), ext_bits(BC_X_NAIO), ext_bits(BC_X_FKDR), ext_bits(BC_X_SKDR), ext_bits(BC_X_KDRIO),
          ext_bits(BC_X_HCNDCN), ext_bits(BC_X_HCNIO), ext_bits(BC_X_CATHP), ext_bits(BC_X_CAHTRE),
          ext_bits(BC_X_CALDCN), ext_bits(BC_X_KCA31), ext_bits(BC_X_SKDCN), ext_bits(BC_X_KKV), ext_bits(BC_X_CAN),
          ext_bits(BC_X_CAIO), ext_bits(BC_X_NAVGRC), ext_bits(BC_X_CAV31), ext_bits(BC_X_CAV33), ext_bits(BC_X_CAV12),
          ext_bits(BC_X_CAV13), ext_bits(BC_X_CAV21), ext_bits(BC_X_CAHVADCN), ext_bits(BC_X_CALVADCN)};
      const int32_t rg = cells[c].region[v];
      if (rg < 0 || !(region_bits(s, c * s.n_regions + rg) & cur_owner[field - BC_PROBE_CURRENT])) {
        delete p;
        return fail(BC_ERR_INVALID, "probe current: no such mechanism at the probed location");
      }
    } else if (field != BC_STATE_V) {
      // the mechanism that owns the state must be present at the probed CV
      uint64_t owner = 0;
      int slot = -1;
      state_view(field, &owner, &slot);
      const int32_t rg = cells[c].region[v];
      if (rg < 0 || !(region_bits(s, c * s.n_regions + rg) & owner)) {
        delete p;
        return fail(BC_ERR_INVALID, "probe field: no such mechanism at the probed location");
      }
    }
    cell_probes[c].push_back(k);
    probe_node[c].push_back(v);
    p->probe_vrest[k] = cells[c].node_vrest[v];
  }
  p->n_probes = s.n_probes;
  p->n_pulses = s.n_pulses;
  // mechanism probes are recorded by the extra kernel variant only
  bool mech_probes = false;
  for (int64_t k = 0; s.probe_field && k < s.n_probes; ++k) mech_probes = mech_probes || s.probe_field[k] != BC_STATE_V;
  p->extra = p->extra || mech_probes;
  // ---------------------------------------------------- synapses / connections
  std::vector<std::vector<std::pair<int64_t, int32_t>>> cell_syns(s.n_cells);
  std::vector<char> is_src(s.n_cells, 0);
  if (s.n_synapses < 0 || s.n_connections < 0) {
    delete p;
    return fail(BC_ERR_INVALID, "n_synapses and n_connections must be >= 0");
  }
  std::vector<double> syn_scale(s.n_synapses, 0.0);
  for (int64_t k = 0; k < s.n_synapses; ++k) {
    const int64_t c = s.syn_cell[k];
    if (c < 0 || c >= s.n_cells) {
      delete p;
      return fail(BC_ERR_INVALID, "syn_cell out of range");
    }
    if (!(s.syn_tau[k] > 0.0) || !std::isfinite(s.syn_e[k])) {
      delete p;
      return fail(BC_ERR_INVALID, "synapse tau must be > 0 ms and e finite");
    }
    if (!(s.syn_x[k] > 0.0 && s.syn_x[k] < 1.0)) {
      delete p;
      return fail(BC_ERR_INVALID, "a synapse must sit inside a CV (0 < syn_x < 1)");
    }
    const int32_t v = locate_node(s, c, cells[c], s.syn_branch[k], s.syn_x[k]);
    int32_t cv = -1;
    for (int32_t q = 0; q < cells[c].n_cv && v >= 0; ++q)
      if (cells[c].cv_node[q] == v) cv = q;
    if (v < 0 || cv < 0) {
      delete p;
      return fail(BC_ERR_INVALID, "synapse location not found");
    }
    cell_syns[c].push_back({k, v});
    syn_scale[k] = 1e5 / cells[c].cv_area[cv];
  }
  for (int64_t j = 0; j < s.n_connections; ++j) {
    if (s.conn_pre[j] < 0 || s.conn_pre[j] >= s.n_cells || s.conn_post[j] < 0 || s.conn_post[j] >= s.n_synapses) {
      delete p;
      return fail(BC_ERR_INVALID, "connection pre cell or post synapse out of range");
    }
    if (!(s.conn_delay[j] >= 0.0) || !std::isfinite(s.conn_weight[j])) {
      delete p;
      return fail(BC_ERR_INVALID, "connection delay must be >= 0 ms and weight finite");
    }
  }
  // ---------------------------------------------------- surrogate ports
  std::vector<std::vector<std::array<int32_t, 3>>> cell_ports(s.n_cells);
  std::vector<std::vector<int64_t>> port_pulse_ids(std::max<int64_t>(s.n_ports, 0));
  if (s.n_ports < 0 || s.n_port_pulses < 0 || s.n_ports >= (int64_t(1) << 31)) {
    delete p;
    return fail(BC_ERR_INVALID, "n_ports and n_port_pulses must be >= 0");
  }
  for (int64_t k = 0; k < s.n_ports; ++k) {
    const int64_t c = s.port_cell[k];
    if (c < 0 || c >= s.n_cells) {
      delete p;
      return fail(BC_ERR_INVALID, "port_cell out of range");
    }
    if (!(s.port_g[k] > 0.0) || !std::isfinite(s.port_g[k]) || !std::isfinite(s.port_e[k]) ||
        !std::isfinite(s.port_feat[2 * k]) || !std::isfinite(s.port_feat[2 * k + 1])) {
      delete p;
      return fail(BC_ERR_INVALID, "port g must be > 0 and e, features finite");
    }
    const int32_t br = s.port_branch[k];
    const int32_t nb = int32_t(s.cell_branch_offsets[c + 1] - s.cell_branch_offsets[c]);
    if (br < 0 || br >= nb) {
      delete p;
      return fail(BC_ERR_INVALID, "port_branch out of range");
    }
    const int32_t ncv = s.branch_ncv[s.cell_branch_offsets[c] + br];
    const int32_t end = locate_node(s, c, cells[c], br, 1.0);
    const int32_t att = locate_node(s, c, cells[c], br, 1.0 - 0.5 / double(ncv));
    if (end < 0 || att < 0 || cells[c].region[att] < 0) {
      delete p;
      return fail(BC_ERR_INVALID, "port location not found");
    }
    for (const auto& q : cell_ports[c])
      if (q[1] == end) {
        delete p;
        return fail(BC_ERR_INVALID, "two ports at the same branch end are not supported");
      }
    cell_ports[c].push_back({int32_t(k), end, att});
  }
  for (int64_t q = 0; q < s.n_port_pulses; ++q) {
    const int64_t k = s.port_pulse_port[q];
    if (k < 0 || k >= s.n_ports) {
      delete p;
      return fail(BC_ERR_INVALID, "port_pulse_port out of range");
    }
    if (!(s.port_pulse_t_off[q] >= s.port_pulse_t_on[q]) || !std::isfinite(s.port_pulse_amp[q])) {
      delete p;
      return fail(BC_ERR_INVALID, "port pulse needs t_off >= t_on and a finite amplitude");
    }
    port_pulse_ids[k].push_back(q);
  }
  p->n_ports = s.n_ports;
  // every cell of a network records its spikes (the output of a network run);
  // only cells with connections have events to deliver
  if (s.n_connections > 0) std::fill(is_src.begin(), is_src.end(), char(1));
  p->n_synapses = s.n_synapses;
  p->n_connections = s.n_connections;
  p->extra = p->extra || s.n_synapses > 0 || s.n_connections > 0;
  p->syn_tau.assign(s.syn_tau, s.syn_tau + s.n_synapses);
  p->syn_e.assign(s.syn_e, s.syn_e + s.n_synapses);
  p->syn_scale = syn_scale;
  p->conn_delay.assign(s.conn_delay, s.conn_delay + s.n_connections);
  {
    // connections in CSR by presynaptic cell
    std::vector<int64_t> order(s.n_connections);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return s.conn_pre[a] < s.conn_pre[b]; });
    p->out_ptr.assign(s.n_cells + 1, 0);
    for (int64_t j = 0; j < s.n_connections; ++j) p->out_ptr[s.conn_pre[j] + 1]++;
    for (int64_t c = 0; c < s.n_cells; ++c) p->out_ptr[c + 1] += p->out_ptr[c];
    p->out_order = order;
    p->out_syn.resize(s.n_connections);
    p->out_w.resize(s.n_connections);
    for (int64_t q = 0; q < s.n_connections; ++q) {
      p->out_syn[q] = s.conn_post[order[q]];
      p->out_w[q] = s.conn_weight[order[q]];
    }
  }
  // ---------------------------------------------------- schedules
  std::vector<CellSched> sched(s.n_cells);
  {
    // as for the lowering: per-cell outcomes, the first failing cell reported
    std::vector<std::string> dmsg(s.n_cells);
    std::vector<char> dbad(s.n_cells, 0);
    parallel_for(s.n_cells, [&](int64_t c) {
      try {
        decompose(cells[c], sched[c]);
      } catch (const std::exception& ex) {
        dbad[c] = 1;
        dmsg[c] = std::string("scheduling cell ") + std::to_string(c) + ": " + ex.what();
      }
    });
    for (int64_t c = 0; c < s.n_cells; ++c)
      if (dbad[c]) {
        delete p;
        return fail(BC_ERR_CAPACITY, dmsg[c]);
      }
  }
  // ---------------------------------------------------- tile packing
  const size_t rs = p->real_size;
  const size_t smem_cap = dry ? size_t(232448) : max_optin_smem(opts.device);
  if (smem_cap == 0) {
    delete p;
    return fail(BC_ERR_CUDA, "could not query the shared-memory limit of the device");
  }
  const size_t static_smem = 1024;  // static shared memory of the kernel (mbarrier, status) + slack
  const size_t smem_budget = smem_cap - static_smem;
  // bytes per node (approx.) for packing: V hi/lo, states, alpha/beta/diag0, parent, pidx, scratch diag/rhs
  // shared bytes per node: V hi/lo, alpha/beta/diag0, scratch diag/rhs/fill (Real),
  // region index (2 B), plus ~1 chain record per 5 nodes (record, child slot, cD/cR/H)
  const double bpn = double(8 * rs + 2) + (28.0 + 4.0 + 3.0 * double(rs)) / 5.0;
  int tile_nodes = opts.tile_nodes;
  if (tile_nodes <= 0) tile_nodes = 900;
  tile_nodes = std::max(tile_nodes, 16);
  p->tile_nodes = tile_nodes;
  // Launch classes: 0 = packed shared-memory tiles (cells <= tile_nodes), 1 = one big
  // cell per shared-memory tile, 2 = global-memory tiles (too big for shared memory).
  const int T_packed = opts.threads_per_tile > 0 ? opts.threads_per_tile : 128;
  const int T_big = opts.threads_big > 0 ? opts.threads_big : 256;
  const int T_glob = opts.threads_global > 0 ? opts.threads_global : (s.n_ports > 0 ? BC_PORT_MAX_THREADS : 512);
  if (T_big % 32 || T_big > 1024 || T_glob % 32 || T_glob > 1024) {
    delete p;
    return fail(BC_ERR_INVALID, "thread counts must be multiples of 32 up to 1024");
  }
  if (s.n_ports > 0 && (T_packed > BC_PORT_MAX_THREADS || T_big > BC_PORT_MAX_THREADS || T_glob > BC_PORT_MAX_THREADS)) {
    delete p;
    return fail(BC_ERR_INVALID, "plans with surrogate ports run at most " + std::to_string(BC_PORT_MAX_THREADS) +
                                    " threads per tile");
  }
  const int class_threads[kMaxClasses] = {T_packed, T_big, T_glob, kLaneThreads};
  p->threads = T_packed;
  p->threads_global = T_glob;
  std::vector<int64_t> order(s.n_cells);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int64_t a, int64_t b) { return cells[a].n_node > cells[b].n_node; });
  std::vector<TileBuild> builds;
  std::vector<int64_t> fill;
  // Lane tiles: cells of at most lane_cell_nodes tree nodes, kLaneThreads per tile
  // in decreasing size (a tile's threads then walk near-equal trees).  The lane
  // kernel runs the channels (out-of-line ones included when the plan has them) and
  // voltage probes, but no synapses, network, mechanism probes or ports.
  std::vector<char> in_lane(s.n_cells, 0);
  const bool lane_ok = !mech_probes && s.n_synapses == 0 && s.n_connections == 0 && s.n_ports == 0;
  if (opts.lane_cell_nodes > 0 && lane_ok) {
    std::vector<int64_t> lane_cells;
    for (int64_t c : order)
      if (cells[c].n_node <= opts.lane_cell_nodes) lane_cells.push_back(c);
    for (size_t q = 0; q < lane_cells.size(); q += kLaneThreads) {
      TileBuild tb;
      tb.cls = 3;
      for (size_t r = q; r < std::min(lane_cells.size(), q + kLaneThreads); ++r) {
        tb.cells.push_back(lane_cells[r]);
        in_lane[lane_cells[r]] = 1;
      }
      builds.push_back(tb);
      fill.push_back(0);
    }
  }
  // best-fit decreasing: each cell goes to the open packed tile with the least room
  // that still holds it (free room -> tile index), else opens a new tile
  std::multimap<int64_t, size_t> room;
  for (int64_t c : order) {
    if (in_lane[c]) continue;
    const int64_t nn = cells[c].n_node;
    if (nn > tile_nodes) {
      TileBuild tb;
      tb.cells.push_back(c);
      tb.cls = 1;
      builds.push_back(tb);
      fill.push_back(nn);
      continue;
    }
    auto it = room.lower_bound(nn);
    if (it != room.end()) {
      const size_t t = it->second;
      room.erase(it);
      builds[t].cells.push_back(c);
      fill[t] += nn;
      if (tile_nodes - fill[t] > 0 && builds[t].cells.size() < 4096) room.emplace(tile_nodes - fill[t], t);
      continue;
    }
    TileBuild tb;
    tb.cells.push_back(c);
    tb.cls = 0;
    builds.push_back(tb);
    fill.push_back(nn);
    if (tile_nodes - nn > 0) room.emplace(tile_nodes - nn, builds.size() - 1);
  }
  BuildCtx cx{&s, &cells, &sched, &cv_base, &cell_pulses, &cell_probes, &pulse_node, &probe_node, &cell_syns, &is_src,
              &cell_ports, &port_pulse_ids, p->precision, S, p->lane_nodes, p->narrow_lane_nodes,
              p->extra ? ((all_bits & BC_M_EXT) ? kParamStride : kParamStrideExtra) : kParamStrideCore};
  std::vector<TileOut> outs;
  outs.reserve(builds.size());
  // Packed tiles: tile_nodes sets how many CTAs share an SM (by the per-node
  // estimate); the shared-memory budget of one tile is then that SM's share, so
  // tiles fill up to tile_nodes without lowering the occupancy.
  const size_t per_sm = dry ? size_t(233472) : sm_smem(opts.device);
  const size_t cta_reserve = 2 * static_smem;  // static shared memory + the system's per-CTA reserve
  // a tile with ports also holds the weight fragments of the GRU
  const size_t est = size_t(double(tile_nodes) * bpn) + 2048 + (s.n_ports > 0 ? size_t(kGruSmemBytes) : 0);
  const size_t ctas_per_sm = std::max<size_t>(1, per_sm / (est + cta_reserve));
  const size_t packed_budget =
      std::min(smem_budget, std::max(est, per_sm / ctas_per_sm > cta_reserve ? per_sm / ctas_per_sm - cta_reserve : est));
  for (size_t t = 0; t < builds.size(); ++t) {
    TileOut to;
    bc_status st = build_tile(cx, builds[t], class_threads[builds[t].cls], to);
    if (st != BC_OK) {
      delete p;
      return st;
    }
    const size_t need = size_t(to.desc.blob_bytes) + size_t(to.desc.scratch_bytes);
    const size_t limit = builds[t].cls == 0 ? packed_budget : smem_budget;
    if (builds[t].cls < 2 && need > limit) {
      if (builds[t].cells.size() > 1) {
        // split: move the last cells into the best-fitting packed tiles not built yet
        // (or new ones) and rebuild this one.  As many cells move at once as the
        // overflow's share of the tile (at least one), so a tile of many small cells
        // whose per-cell records outgrow the node estimate is rebuilt a few times,
        // not once per cell.
        const size_t n_in = builds[t].cells.size();
        size_t n_move = size_t(std::ceil(double(n_in) * double(need - limit) / double(need)));
        n_move = std::max<size_t>(1, std::min(n_move, n_in - 1));
        for (size_t q = 0; q < n_move; ++q) {
          const int64_t c = builds[t].cells.back();
          const int64_t nn = cells[c].n_node;
          builds[t].cells.pop_back();
          fill[t] -= nn;
          size_t dest = builds.size();
          for (auto it = room.lower_bound(nn); it != room.end(); ++it)
            if (it->second > t) {
              dest = it->second;
              room.erase(it);
              break;
            }
          if (dest == builds.size()) {
            TileBuild nb;
            nb.cls = 0;
            builds.push_back(nb);
            fill.push_back(0);
          }
          builds[dest].cells.push_back(c);
          fill[dest] += nn;
          if (tile_nodes - fill[dest] > 0 && builds[dest].cells.size() < 4096) room.emplace(tile_nodes - fill[dest], dest);
        }
        --t;
        continue;
      }
      builds[t].cls = need > smem_budget ? 2 : 1;
      st = build_tile(cx, builds[t], class_threads[builds[t].cls], to);
      if (st != BC_OK) {
        delete p;
        return st;
      }
    }
    outs.push_back(std::move(to));
  }
  // tiles ordered by class; one launch per class
  std::vector<size_t> tord;
  for (int cl = 0; cl < kMaxClasses; ++cl) {
    LaunchClass lcz;
    lcz.first = int(tord.size());
    lcz.threads = class_threads[cl];
    lcz.smem = cl < 2;
    lcz.lane = cl == 3;
    for (size_t t = 0; t < builds.size(); ++t)
      if (builds[t].cls == cl) {
        tord.push_back(t);
        const size_t need = size_t(outs[t].desc.blob_bytes) + size_t(outs[t].desc.scratch_bytes);
        if (lcz.smem) lcz.smem_bytes = std::max(lcz.smem_bytes, need);
      }
    if (opts.tile_order == 1) {
      // longest estimated step first: the block scheduler hands out CTAs in index
      // order, so the tiles left for the last, partly filled wave are the short ones
      std::stable_sort(tord.begin() + lcz.first, tord.end(), [&](size_t x, size_t y) {
        if (outs[x].crit != outs[y].crit) return outs[x].crit > outs[y].crit;
        return outs[x].desc.n_real_nodes > outs[y].desc.n_real_nodes;
      });
    }
    lcz.count = int(tord.size()) - lcz.first;
    if (lcz.count > 0) p->classes.push_back(lcz);
  }
  p->n_smem_tiles = 0;
  for (auto& lcz : p->classes)
    if (lcz.smem) p->n_smem_tiles += lcz.count;
  // ---------------------------------------------------- concatenate + upload
  size_t blob_total = 0, scratch_total = 0, vinit_total = 0;
  int64_t state_total = 0;
  std::vector<int64_t> vinit_off;
  p->tiles.clear();
  p->cv_tile.assign(p->n_cv, -1);
  p->cv_node.assign(p->n_cv, -1);
  p->cv_mech.assign(p->n_cv, 0);
  for (size_t k = 0; k < tord.size(); ++k) {
    TileOut& to = outs[tord[k]];
    TileDesc d = to.desc;
    d.blob_offset = int64_t(blob_total);
    blob_total = align16(blob_total + d.blob_bytes);
    d.state_offset = state_total;
    state_total += int64_t(S) * d.n_nodes;
    if (builds[tord[k]].cls >= 2) {  // global-memory and lane tiles: solver scratch in HBM
      d.scratch_offset = int64_t(scratch_total);
      scratch_total = align16(scratch_total + d.scratch_bytes);
    } else {
      p->smem_bytes = std::max(p->smem_bytes, size_t(d.blob_bytes) + size_t(d.scratch_bytes));
    }
    d.pulse_offset = int64_t(p->pulses.size());
    d.n_pulses = int32_t(to.pulses.size());
    p->pulses.insert(p->pulses.end(), to.pulses.begin(), to.pulses.end());
    p->pulse_src.insert(p->pulse_src.end(), to.pulse_src.begin(), to.pulse_src.end());
    p->pulse_scale.insert(p->pulse_scale.end(), to.pulse_scale.begin(), to.pulse_scale.end());
    d.port_offset = int64_t(p->ports.size());
    d.n_ports = int32_t(to.ports.size());
    for (PortRec r : to.ports) {
      r.stim_begin += int32_t(p->port_pulses.size());
      r.stim_end += int32_t(p->port_pulses.size());
      p->ports.push_back(r);
    }
    p->port_pulses.insert(p->port_pulses.end(), to.port_pulses.begin(), to.port_pulses.end());
    vinit_off.push_back(int64_t(vinit_total));
    vinit_total += to.vinit.size();
    for (size_t q = 0; q < to.cv_local.size(); ++q) {
      p->cv_tile[to.cv_local[q].first] = int32_t(k);
      p->cv_node[to.cv_local[q].first] = to.cv_local[q].second;
      p->cv_mech[to.cv_local[q].first] = to.cv_mech[q];
    }
    p->max_phases = std::max<int64_t>(p->max_phases, d.n_phases);
    p->max_chain_nodes = std::max<int64_t>(p->max_chain_nodes, to.crit);
    p->tiles.push_back(d);
  }
  std::vector<unsigned char> blob(blob_total, 0);
  std::vector<double> vinit(vinit_total);
  for (size_t k = 0; k < tord.size(); ++k) {
    const TileOut& to = outs[tord[k]];
    std::memcpy(blob.data() + p->tiles[k].blob_offset, to.blob.data(), to.blob.size());
    std::copy(to.vinit.begin(), to.vinit.end(), vinit.begin() + vinit_off[k]);
  }
  std::vector<int64_t> outs_crit(outs.size());
  for (size_t q = 0; q < outs.size(); ++q) outs_crit[q] = outs[q].crit;
  outs.clear();
  bc_status st = BC_OK;
#define BC_TRY(x)          \
  do {                     \
    st = (x);              \
    if (st != BC_OK) {     \
      free_plan(p);        \
      return st;           \
    }                      \
  } while (0)
#define BC_TRYC(call)                                                                                \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess) {                                                                         \
      free_plan(p);                                                                                  \
      return fail(BC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));                   \
    }                                                                                                \
  } while (0)
  p->tile_stats.clear();
  for (size_t k = 0; k < tord.size(); ++k) {
    const TileDesc& d = p->tiles[k];
    p->tile_stats.push_back({int64_t(d.n_real_nodes), int64_t(d.n_chains), int64_t(d.n_phases),
                             int64_t(outs_crit[tord[k]]), int64_t(builds[tord[k]].cls),
                             int64_t(d.blob_bytes) + int64_t(d.scratch_bytes)});
  }
  if (dry) {
    *out = p;
    return BC_OK;
  }
  p->blob_bytes = blob_total;
  p->scratch_bytes = scratch_total;
  BC_TRY(dalloc(p, &p->d_blob, blob_total));
  BC_TRY(dalloc(p, &p->d_scratch, scratch_total));
  p->state_bytes = size_t(state_total) * rs;
  BC_TRY(dalloc(p, &p->d_state, p->state_bytes));
  BC_TRY(dalloc(p, &p->d_tiles, p->tiles.size()));
  BC_TRY(dalloc(p, &p->d_pulses, p->pulses.size()));
  BC_TRY(dalloc(p, &p->d_vinit, vinit.size()));
  BC_TRY(dalloc(p, &p->d_vinit_off, vinit_off.size()));
  BC_TRY(dalloc(p, &p->d_spike_count, size_t(p->n_probes)));
  BC_TRY(dalloc(p, &p->d_spike_times, size_t(p->n_probes) * std::max(1, p->max_spikes)));
  BC_TRY(dalloc(p, &p->d_status, 1));
  BC_TRY(dalloc(p, &p->d_timers, 4));
  BC_TRYC(cudaMemset(p->d_timers, 0, 4 * sizeof(unsigned long long)));
  BC_TRYC(cudaMemcpy(p->d_blob, blob.data(), blob_total, cudaMemcpyHostToDevice));
  BC_TRYC(cudaMemcpy(p->d_tiles, p->tiles.data(), p->tiles.size() * sizeof(TileDesc), cudaMemcpyHostToDevice));
  BC_TRYC(cudaMemcpy(p->d_vinit, vinit.data(), vinit.size() * sizeof(double), cudaMemcpyHostToDevice));
  BC_TRYC(cudaMemcpy(p->d_vinit_off, vinit_off.data(), vinit_off.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
  BC_TRYC(cudaMemset(p->d_status, 0, sizeof(int32_t)));
  {
    // synapse parameters and the connection CSR, in the plan's precision
    auto up_real = [&](void** dst, const std::vector<double>& src) -> bc_status {
      const size_t n = std::max<size_t>(src.size(), 1);
      cudaError_t e = cudaMalloc(dst, n * rs);
      if (e != cudaSuccess) return fail(BC_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
      p->device_bytes += n * rs;
      std::vector<unsigned char> tmp(n * rs, 0);
      for (size_t k = 0; k < src.size(); ++k) {
        if (rs == 8)
          std::memcpy(tmp.data() + k * 8, &src[k], 8);
        else {
          const float f = float(src[k]);
          std::memcpy(tmp.data() + k * 4, &f, 4);
        }
      }
      e = cudaMemcpy(*dst, tmp.data(), n * rs, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return fail(BC_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
      return BC_OK;
    };
    BC_TRY(up_real(&p->d_syn_g, std::vector<double>(p->n_synapses, 0.0)));
    BC_TRY(up_real(&p->d_syn_tau, p->syn_tau));
    BC_TRY(up_real(&p->d_syn_e, p->syn_e));
    BC_TRY(up_real(&p->d_syn_scale, p->syn_scale));
    BC_TRY(up_real(&p->d_out_w, p->out_w));
    BC_TRY(dalloc(p, &p->d_out_ptr, p->out_ptr.size()));
    BC_TRY(dalloc(p, &p->d_out_syn, p->out_syn.size()));
    BC_TRY(dalloc(p, &p->d_out_d, size_t(p->n_connections)));
    BC_TRYC(cudaMemcpy(p->d_out_ptr, p->out_ptr.data(), p->out_ptr.size() * 8, cudaMemcpyHostToDevice));
    if (p->n_connections > 0)
      BC_TRYC(cudaMemcpy(p->d_out_syn, p->out_syn.data(), p->out_syn.size() * 8, cudaMemcpyHostToDevice));
    int64_t n_src = 0;
    for (int64_t c = 0; c + 1 < int64_t(p->out_ptr.size()); ++c) n_src += p->out_ptr[c + 1] > p->out_ptr[c];
    p->rec_cap = p->n_connections > 0 ? std::max<int64_t>(int64_t(1) << 16, 256 * n_src) : 1;
    BC_TRY(dalloc(p, &p->d_rec_cell, size_t(p->rec_cap)));
    BC_TRY(dalloc(p, &p->d_rec_step, size_t(p->rec_cap)));
    BC_TRY(dalloc(p, &p->d_rec_count, 2));
    BC_TRYC(cudaMemset(p->d_rec_count, 0, 2 * sizeof(unsigned long long)));
  }
  if (p->n_ports > 0) {
    BC_TRY(dalloc(p, &p->d_ports, p->ports.size()));
    BC_TRY(dalloc(p, &p->d_port_pulses, std::max<size_t>(p->port_pulses.size(), 1)));
    BC_TRY(dalloc(p, &p->d_port_h, size_t(p->n_ports) * kPortStride));
    BC_TRY(dalloc(p, &p->d_port_flags, size_t(p->n_cells)));
    BC_TRY(dalloc(p, &p->d_gru, 1));
    BC_TRYC(cudaMemcpy(p->d_ports, p->ports.data(), p->ports.size() * sizeof(PortRec), cudaMemcpyHostToDevice));
  }
  if (p->n_smem_tiles > 0 && p->smem_bytes + static_smem > smem_cap) {
    free_plan(p);
    return fail(BC_ERR_CAPACITY, "tile shared memory exceeds the device limit");
  }
  for (int k = 0; k < kMaxClasses - 1; ++k) {
    BC_TRYC(cudaStreamCreateWithFlags(&p->aux[k], cudaStreamNonBlocking));
    BC_TRYC(cudaEventCreateWithFlags(&p->ev_join[k], cudaEventDisableTiming));
  }
  BC_TRYC(cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming));
  int prio_least = 0, prio_greatest = 0;
  BC_TRYC(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest));
  BC_TRYC(cudaStreamCreateWithPriority(&p->init_stream, cudaStreamNonBlocking, prio_greatest));
  *out = p;
  // The initial reset runs on the plan's own non-blocking stream of the highest
  // priority: creating a plan waits neither for work other plans have queued on
  // the legacy stream nor, behind their pending blocks, for free SM slots.
  return bc_reset(p, p->init_stream);
}

bc_status bc_lower_cell(const bc_batch_spec* spec, int64_t cell, int32_t* n_cv, int32_t* n_node, double* cv_area,
                        int32_t* cv_node, int32_t* parent, double* alpha, double* beta, double* diag,
                        int32_t* region) {
  if (!spec || !n_cv || !n_node) return fail(BC_ERR_INVALID, "null argument");
  if (cell < 0 || cell >= spec->n_cells) return fail(BC_ERR_INVALID, "cell out of range");
  LoweredCell lc;
  bc_status st = lower_cell(*spec, cell, lc);
  if (st != BC_OK) return st;
  *n_cv = lc.n_cv;
  *n_node = lc.n_node;
  if (cv_area) std::copy(lc.cv_area.begin(), lc.cv_area.end(), cv_area);
  if (cv_node) std::copy(lc.cv_node.begin(), lc.cv_node.end(), cv_node);
  if (parent) std::copy(lc.parent.begin(), lc.parent.end(), parent);
  if (alpha) std::copy(lc.alpha.begin(), lc.alpha.end(), alpha);
  if (beta) std::copy(lc.beta.begin(), lc.beta.end(), beta);
  if (diag) std::copy(lc.diag.begin(), lc.diag.end(), diag);
  if (region) std::copy(lc.region.begin(), lc.region.end(), region);
  return BC_OK;
}

bc_status bc_plan_destroy(bc_plan_t p) {
  if (!p) return fail(BC_ERR_INVALID, "null plan");
  free_plan(p);
  return BC_OK;
}

bc_status bc_plan_info(bc_plan_t p, bc_plan_info_t* info) {
  if (!p || !info) return fail(BC_ERR_INVALID, "null argument");
  std::memset(info, 0, sizeof(*info));
  info->n_cells = p->n_cells;
  info->n_cv = p->n_cv;
  info->n_nodes = p->n_nodes;
  info->n_tiles = int64_t(p->tiles.size());
  info->n_probes = p->n_probes;
  info->n_pulses = p->n_pulses;
  info->threads_per_tile = p->threads;
  info->tile_nodes = p->tile_nodes;
  info->steps_per_launch = p->steps_per_launch;
  info->precision = p->precision;
  info->smem_bytes_per_tile = int64_t(p->smem_bytes);
  info->device_bytes = int64_t(p->device_bytes);
  info->max_phases = p->max_phases;
  info->max_chain_nodes = p->max_chain_nodes;
  info->state_slots = p->state_slots;
  info->n_smem_tiles = int32_t(p->n_smem_tiles);
  info->n_launch_classes = int32_t(p->classes.size());
  info->kernel_variant = kernel_variant(p);
  return BC_OK;
}

bc_status bc_plan_cell_ncv(bc_plan_t p, int64_t* ncv) {
  if (!p || !ncv) return fail(BC_ERR_INVALID, "null argument");
  std::copy(p->cell_ncv.begin(), p->cell_ncv.end(), ncv);
  return BC_OK;
}

#define BC_NEED_DEVICE(p) \
  if ((p)->dry) return fail(BC_ERR_INVALID, "plan was created with dry_run; it has no device state")

bc_status bc_reset(bc_plan_t p, void* stream) {
  if (!p) return fail(BC_ERR_INVALID, "null plan");
  BC_NEED_DEVICE(p);
  BC_CUDA(cudaSetDevice(p->device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  LaunchArgs a = base_args(p);
  a.tiles = p->d_tiles;
  a.n_tiles = int32_t(p->tiles.size());
  int e = launch_reset_impl(a, p->precision, 256, p->d_vinit, p->d_vinit_off, stream);
  if (e) return fail(BC_ERR_CUDA, std::string("reset kernel: ") + cudaGetErrorString(cudaError_t(e)));
  if (p->n_probes > 0) {
    BC_CUDA(cudaMemsetAsync(p->d_spike_count, 0, size_t(p->n_probes) * sizeof(int32_t), st));
  }
  BC_CUDA(cudaMemsetAsync(p->d_status, 0, sizeof(int32_t), st));
  if (p->n_synapses > 0) BC_CUDA(cudaMemsetAsync(p->d_syn_g, 0, size_t(p->n_synapses) * p->real_size, st));
  if (p->d_arrivals)
    BC_CUDA(cudaMemsetAsync(p->d_arrivals, 0,
                            size_t(p->arr_slots) * size_t(std::max<int64_t>(p->n_synapses, 1)) * p->real_size, st));
  BC_CUDA(cudaMemsetAsync(p->d_rec_count, 0, 2 * sizeof(unsigned long long), st));
  if (p->n_ports > 0) {
    BC_CUDA(cudaMemsetAsync(p->d_port_h, 0, size_t(p->n_ports) * kPortStride * sizeof(float), st));
    BC_CUDA(cudaMemsetAsync(p->d_port_flags, 0, size_t(p->n_cells) * sizeof(int32_t), st));
  }
  BC_CUDA(cudaStreamSynchronize(st));
  p->step = 0;
  p->trace_origin = 0;
  return BC_OK;
}

bc_status bc_network_spikes(bc_plan_t p, int32_t* cells, int64_t* steps, int64_t cap, int64_t* n_out,
                            void* stream) {
  if (!p || !n_out || (cap > 0 && (!cells || !steps))) return fail(BC_ERR_INVALID, "null argument");
  BC_NEED_DEVICE(p);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned long long n = 0;
  BC_CUDA(cudaMemcpyAsync(&n, p->d_rec_count, sizeof(n), cudaMemcpyDeviceToHost, s));
  BC_CUDA(cudaStreamSynchronize(s));
  *n_out = int64_t(n);
  const int64_t m = std::min<int64_t>(std::min<int64_t>(int64_t(n), cap), p->rec_cap);
  if (m > 0) {
    BC_CUDA(cudaMemcpyAsync(cells, p->d_rec_cell, size_t(m) * 4, cudaMemcpyDeviceToHost, s));
    BC_CUDA(cudaMemcpyAsync(steps, p->d_rec_step, size_t(m) * 8, cudaMemcpyDeviceToHost, s));
    BC_CUDA(cudaStreamSynchronize(s));
  }
  return BC_OK;
}

// BF16 of a finite float, round to nearest even (as the device conversion).
static uint16_t bf16_rne(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  u += 0x7fffu + ((u >> 16) & 1u);
  return uint16_t(u >> 16);
}

bc_status bc_surrogate_set(bc_plan_t p, const float* params, const float* norm, void* stream) {
  if (!p || !params || !norm) return fail(BC_ERR_INVALID, "null argument");
  if (p->n_ports == 0) return fail(BC_ERR_INVALID, "the plan has no surrogate ports");
  BC_NEED_DEVICE(p);
  BC_CUDA(cudaSetDevice(p->device));
  for (int k = 0; k < kGruNParam; ++k)
    if (!std::isfinite(params[k])) return fail(BC_ERR_INVALID, "non-finite GRU parameter");
  const float v_scale = norm[0], y_scale = norm[1], lo = norm[2], hi = norm[3], dvdt = norm[4];
  if (!(v_scale > 0.f) || !std::isfinite(v_scale) || !std::isfinite(y_scale) || !(hi >= lo) || !(dvdt > 0.f))
    return fail(BC_ERR_INVALID, "surrogate norm: v_scale > 0, finite y_scale, env_v_hi >= env_v_lo, env_dvdt > 0");
  // the extended weight matrix, as gru_pack_kernel builds it for training
  auto bf = [](float f) {
    const uint32_t u = uint32_t(bf16_rne(f)) << 16;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
  };
  auto value = [&](int n, int k) -> float {
    const int q = n / kGruH, u = n % kGruH;
    if (k < kGruH) return q < 3 ? params[kGruOffWh + (q * kGruH + u) * kGruH + k] : 0.0f;
    const int c = k - kGruH;
    const int xrow = q == 0 ? u : q == 1 ? kGruH + u : 2 * kGruH + u;
    if (c < 2 * kGruX) return q == 2 ? 0.0f : bf(params[kGruOffWx + xrow * kGruX + (c % kGruX)]);
    if (c < 2 * kGruX + 2) {
      const float bsum = q == 0   ? params[kGruOffBx + u] + params[kGruOffBh + u]
                         : q == 1 ? params[kGruOffBx + kGruH + u] + params[kGruOffBh + kGruH + u]
                         : q == 2 ? params[kGruOffBh + 2 * kGruH + u]
                                  : params[kGruOffBx + 2 * kGruH + u];
      const float hi = bf(bsum);
      return c == 2 * kGruX ? hi : bsum - hi;
    }
    return 0.0f;
  };
  GruWeights w{};
  for (int n = 0; n < kGruRows; ++n)
    for (int k = 0; k < kGruK; k += 2)
      w.wext[(n * kGruK + k) / 2] = uint32_t(bf16_rne(value(n, k))) | (uint32_t(bf16_rne(value(n, k + 1))) << 16);
  std::memcpy(w.wo, params + kGruOffWo, sizeof(w.wo));
  w.bo = params[kGruOffBo];
  w.v_scale = v_scale;
  w.y_scale = y_scale;
  w.env_v_lo = lo;
  w.env_v_hi = hi;
  w.env_dvdt = dvdt;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  BC_CUDA(cudaMemcpyAsync(p->d_gru, &w, sizeof(w), cudaMemcpyHostToDevice, st));
  BC_CUDA(cudaStreamSynchronize(st));
  p->gru_set = true;
  return BC_OK;
}

bc_status bc_surrogate_flags(bc_plan_t p, int32_t* flags, void* stream) {
  if (!p || !flags) return fail(BC_ERR_INVALID, "null argument");
  if (p->n_ports == 0) {
    std::fill(flags, flags + p->n_cells, 0);
    return BC_OK;
  }
  BC_NEED_DEVICE(p);
  BC_CUDA(cudaSetDevice(p->device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  BC_CUDA(cudaMemcpyAsync(flags, p->d_port_flags, size_t(p->n_cells) * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  BC_CUDA(cudaStreamSynchronize(st));
  return BC_OK;
}

bc_status bc_synapse_download(bc_plan_t p, double* g, void* stream) {
  if (!p || (!g && p->n_synapses > 0)) return fail(BC_ERR_INVALID, "null argument");
  BC_NEED_DEVICE(p);
  if (p->n_synapses == 0) return BC_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::vector<unsigned char> tmp(size_t(p->n_synapses) * p->real_size);
  BC_CUDA(cudaMemcpyAsync(tmp.data(), p->d_syn_g, tmp.size(), cudaMemcpyDeviceToHost, s));
  BC_CUDA(cudaStreamSynchronize(s));
  for (int64_t k = 0; k < p->n_synapses; ++k) {
    if (p->real_size == 8) {
      std::memcpy(&g[k], tmp.data() + k * 8, 8);
    } else {
      float f;
      std::memcpy(&f, tmp.data() + k * 4, 4);
      g[k] = double(f);
    }
  }
  return BC_OK;
}

bc_status bc_check(bc_plan_t p, void* stream) {
  if (!p) return fail(BC_ERR_INVALID, "null plan");
  BC_NEED_DEVICE(p);
  int32_t status = 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  BC_CUDA(cudaMemcpyAsync(&status, p->d_status, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  BC_CUDA(cudaStreamSynchronize(st));
  if (status & 2) return fail(BC_ERR_TIMEOUT, "a bounded device wait gave up (bulk copy did not complete)");
  if (status & 4) return fail(BC_ERR_CAPACITY, "the spike record buffer of the network run overflowed");
  if (status & 1) return fail(BC_ERR_NONFINITE, "non-finite membrane voltage");
  return BC_OK;
}

bc_status bc_run_async(bc_plan_t p, int64_t n_steps, double dt, void* stream) {
  if (!p) return fail(BC_ERR_INVALID, "null plan");
  BC_NEED_DEVICE(p);
  BC_CUDA(cudaSetDevice(p->device));
  return enqueue_run(p, n_steps, dt, stream);
}

bc_status bc_run(bc_plan_t p, int64_t n_steps, double dt, void* stream) {
  bc_status st = bc_run_async(p, n_steps, dt, stream);
  if (st != BC_OK) return st;
  return bc_check(p, stream);
}

bc_status bc_run_timed(bc_plan_t p, int64_t n_steps, double dt, void* stream, double* ms_out) {
  if (!p || !ms_out) return fail(BC_ERR_INVALID, "null argument");
  BC_NEED_DEVICE(p);
  BC_CUDA(cudaSetDevice(p->device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // prepare tables outside the timed region
  bc_status s0 = update_pulses(p, dt, stream);
  if (s0 != BC_OK) return s0;
  const int64_t recs = p->record_every > 0 ? (p->step + n_steps - p->trace_origin) / p->record_every : 0;
  s0 = ensure_traces(p, recs, stream);
  if (s0 != BC_OK) return s0;
  cudaEvent_t e0, e1;
  BC_CUDA(cudaEventCreate(&e0));
  BC_CUDA(cudaEventCreate(&e1));
  BC_CUDA(cudaEventRecord(e0, st));
  bc_status s1 = enqueue_run(p, n_steps, dt, stream);
  BC_CUDA(cudaEventRecord(e1, st));
  BC_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  BC_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms_out = ms;
  if (s1 != BC_OK) return s1;
  return bc_check(p, stream);
}

static bc_status view_offsets(bc_plan* p, int32_t which, std::vector<int64_t>& hi, std::vector<int64_t>& lo) {
  if (which < 0 || which >= BC_NSTATE_VIEW) return fail(BC_ERR_INVALID, "unknown state view");
  hi.assign(p->n_cv, -1);
  lo.assign(p->n_cv, -1);
  const size_t rs = p->real_size;
  for (int64_t k = 0; k < p->n_cv; ++k) {
    const TileDesc& d = p->tiles[p->cv_tile[k]];
    const int64_t j = p->cv_node[k];
    const int64_t base = d.blob_offset;
    if (which == BC_STATE_V) {
      hi[k] = base + d.off_v + 2 * j * rs;
      lo[k] = hi[k] + rs;
      continue;
    }
    uint64_t bit = 0;
    int slot = -1;
    state_view(which, &bit, &slot);
    if (which != BC_STATE_V_LAST && !(p->cv_mech[k] & bit)) slot = -1;
    const bool has_lo = which == BC_STATE_CA_CI || which == BC_STATE_V_LAST;
    if (slot < 0) continue;
    // states live in the separate state array: offsets are tagged by +state_tag
    const int lo_slot = which == BC_STATE_V_LAST ? kSlotVLastLo : kSlotCaLo;
    hi[k] = kStateTag + (d.state_offset + int64_t(slot) * d.n_nodes + j) * int64_t(rs);
    if (has_lo) lo[k] = kStateTag + (d.state_offset + int64_t(lo_slot) * d.n_nodes + j) * int64_t(rs);
  }
  return BC_OK;
}

static bc_status view_io(bc_plan* p, int32_t which, double* host, bool write, void* stream) {
  if (!p || !host) return fail(BC_ERR_INVALID, "null argument");
  BC_NEED_DEVICE(p);
  BC_CUDA(cudaSetDevice(p->device));
  std::vector<int64_t> hi, lo;
  bc_status st = view_offsets(p, which, hi, lo);
  if (st != BC_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t n = size_t(p->n_cv);
  int64_t *dhi = nullptr, *dlo = nullptr;
  double* dv = nullptr;
  BC_CUDA(cudaMalloc(reinterpret_cast<void**>(&dhi), n * 8));
  BC_CUDA(cudaMalloc(reinterpret_cast<void**>(&dlo), n * 8));
  BC_CUDA(cudaMalloc(reinterpret_cast<void**>(&dv), n * 8));
  cudaError_t e = cudaMemcpyAsync(dhi, hi.data(), n * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dlo, lo.data(), n * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && write) e = cudaMemcpyAsync(dv, host, n * 8, cudaMemcpyHostToDevice, s);
  int ke = 0;
  if (e == cudaSuccess)
    ke = launch_view_impl(p->d_blob, p->d_state, p->precision, dhi, dlo, dv, int64_t(n), write, stream);
  if (e == cudaSuccess && !ke && !write) e = cudaMemcpyAsync(host, dv, n * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(dhi);
  cudaFree(dlo);
  cudaFree(dv);
  if (ke) return fail(BC_ERR_CUDA, std::string("view kernel: ") + cudaGetErrorString(cudaError_t(ke)));
  if (e != cudaSuccess) return fail(BC_ERR_CUDA, std::string("state view: ") + cudaGetErrorString(e));
  return BC_OK;
}

bc_status bc_state_download(bc_plan_t p, int32_t which, double* out, void* stream) {
  return view_io(p, which, out, false, stream);
}

bc_status bc_state_upload(bc_plan_t p, int32_t which, const double* in, void* stream) {
  bc_status st = view_io(p, which, const_cast<double*>(in), true, stream);
  // a new voltage starts a fresh history: no step has crossed anything since
  if (st == BC_OK && which == BC_STATE_V) st = view_io(p, BC_STATE_V_LAST, const_cast<double*>(in), true, stream);
  return st;
}

bc_status bc_pulse_set_amp(bc_plan_t p, const double* amp_nA, void* stream) {
  if (!p || (!amp_nA && p->n_pulses > 0)) return fail(BC_ERR_INVALID, "null argument");
  BC_NEED_DEVICE(p);
  if (p->pulses.empty()) return BC_OK;
  BC_CUDA(cudaSetDevice(p->device));
  for (int64_t q = 0; q < p->n_pulses; ++q)
    if (!std::isfinite(amp_nA[q])) return fail(BC_ERR_INVALID, "bc_pulse_set_amp: non-finite amplitude");
  for (size_t k = 0; k < p->pulses.size(); ++k) p->pulses[k].amp = amp_nA[p->pulse_src[k]] * p->pulse_scale[k];
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the records also carry the step bounds of the last dt; pageable source: wait
  BC_CUDA(cudaMemcpyAsync(p->d_pulses, p->pulses.data(), p->pulses.size() * sizeof(PulseRec), cudaMemcpyHostToDevice,
                          st));
  BC_CUDA(cudaStreamSynchronize(st));
  return BC_OK;
}

bc_status bc_spike_state_download(bc_plan_t p, double v_th, double* out, void* stream) {
  if (!p || !out) return fail(BC_ERR_INVALID, "null argument");
  std::vector<double> last(size_t(p->n_cv));
  bc_status st = view_io(p, BC_STATE_V, out, false, stream);
  if (st == BC_OK && p->n_cv > 0) st = view_io(p, BC_STATE_V_LAST, last.data(), false, stream);
  if (st != BC_OK) return st;
  for (int64_t k = 0; k < p->n_cv; ++k) out[k] = (last[size_t(k)] < v_th && out[k] >= v_th) ? 1.0 : 0.0;
  return BC_OK;
}

// ------------------------------------------------------------------ no-allocation download
// Host staging of the offset tables, [hi | lo] with BC_NOALLOC_MAX_CV entries each
// (zero-initialised static storage; nothing is allocated at run time).
static int64_t g_noalloc_host_off[2 * size_t(BC_NOALLOC_MAX_CV)];
constexpr int kNoAllocDevices = 64;
static unsigned char* g_noalloc_scratch[kNoAllocDevices];
static std::mutex g_noalloc_setup_mu;

// One-time (per device) lookup of the scratch address; the caller has set the device.
static bc_status noalloc_scratch(int device, unsigned char** out) {
  if (device < 0 || device >= kNoAllocDevices) return fail(BC_ERR_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_setup_mu);
  if (!g_noalloc_scratch[device]) {
    void* addr = nullptr;
    const int e = noalloc_view_scratch_address(&addr);
    if (e != 0 || !addr)
      return fail(BC_ERR_CUDA, std::string("cudaGetSymbolAddress(no-allocation scratch): ") +
                                   cudaGetErrorString(cudaError_t(e)));
    g_noalloc_scratch[device] = static_cast<unsigned char*>(addr);
  }
  *out = g_noalloc_scratch[device];
  return BC_OK;
}

// Offsets of CV k in view `which`: the per-CV form of view_offsets.
static void noalloc_offset(const bc_plan* p, int32_t which, int64_t k, int64_t* hi, int64_t* lo) {
  const TileDesc& d = p->tiles[p->cv_tile[k]];
  const int64_t j = p->cv_node[k];
  const int64_t rs = int64_t(p->real_size);
  *hi = -1;
  *lo = -1;
  if (which == BC_STATE_V) {
    *hi = d.blob_offset + d.off_v + 2 * j * rs;
    *lo = *hi + rs;
    return;
  }
  uint64_t bit = 0;
  int slot = -1;
  state_view(which, &bit, &slot);
  if (which != BC_STATE_V_LAST && !(p->cv_mech[k] & bit)) return;
  *hi = kStateTag + (d.state_offset + int64_t(slot) * d.n_nodes + j) * rs;
  if (which == BC_STATE_CA_CI) *lo = kStateTag + (d.state_offset + int64_t(kSlotCaLo) * d.n_nodes + j) * rs;
  if (which == BC_STATE_V_LAST) *lo = kStateTag + (d.state_offset + int64_t(kSlotVLastLo) * d.n_nodes + j) * rs;
}

bc_status bc_state_download_noalloc(bc_plan_t p, int32_t which, double* out, void* stream) {
  if (!p || !out) return fail(BC_ERR_INVALID, "null argument");
  if (which < 0 || which >= BC_NSTATE_VIEW) return fail(BC_ERR_INVALID, "unknown state view");
  if (p->n_cv > BC_NOALLOC_MAX_CV)
    return fail(BC_ERR_INVALID, "bc_state_download_noalloc: plan has " + std::to_string(p->n_cv) +
                                    " CVs, above the fixed scratch capacity of " +
                                    std::to_string(BC_NOALLOC_MAX_CV) +
                                    " (BC_NOALLOC_MAX_CV); use bc_state_download");
  BC_NEED_DEVICE(p);
  BC_CUDA(cudaSetDevice(p->device));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // The call copies from pageable host memory and synchronises the stream, and
  // neither is allowed while the stream is being captured into a graph.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  BC_CUDA(cudaStreamIsCapturing(s, &cap));
  if (cap != cudaStreamCaptureStatusNone)
    return fail(BC_ERR_INVALID, "bc_state_download_noalloc: the stream is being captured; call it outside capture");
  unsigned char* scratch = nullptr;
  bc_status st = noalloc_scratch(p->device, &scratch);
  if (st != BC_OK) return st;
  const int64_t n = p->n_cv;
  if (n == 0) return BC_OK;
  int64_t* h_hi = g_noalloc_host_off;
  int64_t* h_lo = g_noalloc_host_off + BC_NOALLOC_MAX_CV;
  for (int64_t k = 0; k < n; ++k) noalloc_offset(p, which, k, &h_hi[k], &h_lo[k]);
  // Entries [0, n) of all three arrays are written before they are read (offsets by
  // the copies, values by the view kernel, which fills absent states with NaN), so
  // nothing has to start at zero.
  int64_t* d_hi = reinterpret_cast<int64_t*>(scratch);
  int64_t* d_lo = d_hi + BC_NOALLOC_MAX_CV;
  double* d_val = reinterpret_cast<double*>(d_lo + BC_NOALLOC_MAX_CV);
  // Once something is enqueued, every return waits for the stream first, so that
  // no copy or kernel of this call still uses the shared scratch when the next,
  // serialised call (perhaps on another stream) writes it.
  auto failed = [&](const std::string& what, cudaError_t e) {
    (void)cudaStreamSynchronize(s);
    return fail(BC_ERR_CUDA, what + ": " + cudaGetErrorString(e));
  };
  cudaError_t e = cudaMemcpyAsync(d_hi, h_hi, size_t(n) * 8, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return failed("offset upload", e);
  e = cudaMemcpyAsync(d_lo, h_lo, size_t(n) * 8, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return failed("offset upload", e);
  const int ke = launch_view_impl(p->d_blob, p->d_state, p->precision, d_hi, d_lo, d_val, n, false, stream);
  if (ke) return failed("view kernel", cudaError_t(ke));
  e = cudaMemcpyAsync(out, d_val, size_t(n) * 8, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return failed("value download", e);
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(BC_ERR_CUDA, std::string("cudaStreamSynchronize: ") + cudaGetErrorString(e));
  return BC_OK;
}

bc_status bc_probe_count(bc_plan_t p, int64_t* n) {
  if (!p || !n) return fail(BC_ERR_INVALID, "null argument");
  *n = p->record_every > 0 ? (p->step - p->trace_origin) / p->record_every : 0;
  if (*n > p->trace_cap) *n = p->trace_cap;
  return BC_OK;
}

bc_status bc_probe_download(bc_plan_t p, double* traces, int64_t max_records, void* stream) {
  if (!p || (!traces && max_records > 0)) return fail(BC_ERR_INVALID, "null argument");
  int64_t n = 0;
  bc_probe_count(p, &n);
  n = std::min(n, max_records);
  if (n <= 0 || p->n_probes == 0) return BC_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  BC_CUDA(cudaMemcpyAsync(traces, p->d_traces, size_t(n) * p->n_probes * sizeof(double), cudaMemcpyDeviceToHost, s));
  BC_CUDA(cudaStreamSynchronize(s));
  return BC_OK;
}

bc_status bc_spike_download(bc_plan_t p, int32_t* counts, double* times, void* stream) {
  if (!p) return fail(BC_ERR_INVALID, "null plan");
  if (p->n_probes == 0) return BC_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (counts)
    BC_CUDA(cudaMemcpyAsync(counts, p->d_spike_count, size_t(p->n_probes) * 4, cudaMemcpyDeviceToHost, s));
  if (times && p->max_spikes > 0)
    BC_CUDA(cudaMemcpyAsync(times, p->d_spike_times, size_t(p->n_probes) * p->max_spikes * 8, cudaMemcpyDeviceToHost, s));
  BC_CUDA(cudaStreamSynchronize(s));
  return BC_OK;
}

bc_status bc_probe_clear(bc_plan_t p, void* stream) {
  if (!p) return fail(BC_ERR_INVALID, "null plan");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->n_probes > 0) BC_CUDA(cudaMemsetAsync(p->d_spike_count, 0, size_t(p->n_probes) * 4, s));
  BC_CUDA(cudaStreamSynchronize(s));
  p->trace_origin = p->step;
  return BC_OK;
}

bc_status bc_plan_tile_stats(bc_plan_t p, int64_t* out) {
  if (!p || !out) return fail(BC_ERR_INVALID, "null argument");
  for (size_t k = 0; k < p->tile_stats.size(); ++k)
    for (int j = 0; j < 6; ++j) out[k * 6 + j] = p->tile_stats[k][j];
  return BC_OK;
}

bc_status bc_debug_phase_cycles(bc_plan_t p, uint64_t* out4, int32_t reset) {
  if (!p || !out4) return fail(BC_ERR_INVALID, "null argument");
  BC_NEED_DEVICE(p);
  BC_CUDA(cudaMemcpy(out4, p->d_timers, 4 * sizeof(uint64_t), cudaMemcpyDeviceToHost));
  if (reset) BC_CUDA(cudaMemset(p->d_timers, 0, 4 * sizeof(uint64_t)));
  return BC_OK;
}

bc_status bc_step_count(bc_plan_t p, int64_t* steps) {
  if (!p || !steps) return fail(BC_ERR_INVALID, "null argument");
  *steps = p->step;
  return BC_OK;
}

}  // extern "C"
