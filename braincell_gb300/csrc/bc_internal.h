// Internal structures shared by the host planner (bc_plan.cpp, bc_lower.cpp) and
// the device code (bc_kernels.cu).  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/braincell_gb300.h"

namespace bc {

// ----------------------------------------------------------------- errors
void set_error(const std::string& msg);
bc_status fail(bc_status code, const std::string& msg);

// ----------------------------------------------------------------- lowering
// One cell lowered to its point tree (node numbering as the reference's
// build_node_tree_from_cvs: root endpoint = 0, then per branch its CV
// midpoints in walk order followed by its terminal endpoint).
struct LoweredCell {
  int32_t n_cv = 0;
  int32_t n_node = 0;
  std::vector<int32_t> parent;   // [n_node] parent node, -1 root
  std::vector<double> alpha;     // [n_node] g_e / C_self    (ms^-1), 0 for root
  std::vector<double> beta;      // [n_node] g_e / C_parent  (ms^-1), 0 for root
  std::vector<double> diag;      // [n_node] sum of axial coefficients of the row (ms^-1)
  std::vector<int32_t> region;   // [n_node] region id, -1 for boundary (algebraic) rows
  std::vector<int32_t> cv_node;  // [n_cv]  midpoint node of each CV (reference CV order)
  std::vector<double> cv_area;   // [n_cv]  um^2
  std::vector<double> node_vrest;// [n_node] initial voltage
};

// Lower cell `c` of the batch.  Returns BC_OK or an error (message set).
bc_status lower_cell(const bc_batch_spec& spec, int64_t c, LoweredCell& out);

// Locate the node selected by (branch, x) in a lowered cell (midpoint of the
// owning CV for interior x, the branch endpoint node for x = 0 / 1).
int32_t locate_node(const bc_batch_spec& spec, int64_t c, const LoweredCell& lc, int32_t branch, double x);

// ----------------------------------------------------------------- device records
// Stride (in reals) of the per-(cell, region) parameter records in a tile blob: one
// more than BC_NPARAM, so that the records of different regions start in different
// shared-memory banks (the lanes of a warp read the records of their own nodes'
// regions; at a stride of 64 words they would all fall in one bank).
constexpr int kParamStride = BC_NPARAM + 1;
// Plans on the extra variant without extension channels read the entries before
// BC_P_EXT_MASK only, and plans on the lean variants only the main mix's (up to
// BC_P_CA_CI0): their records keep those, on an odd stride as well.
constexpr int kParamStrideExtra = BC_P_EXT_MASK + 1;
constexpr int kParamStrideCore = BC_P_CA_CI0 + 2;

// A chain: nodes [start, start+count) of the tile, bottom (deepest) first; node
// start+k+1 is the parent of node start+k and top_parent is the parent of the top
// node (-1 at a root).  The record owns the consecutive contribution slots
// aux .. aux + n_child, one per child chain, and writes its own contribution to
// the parent's slot `slot` (-1 at a root).  32 bytes, read as two 16-byte vectors.
struct ChainRec {
  int32_t start;
  int32_t count;
  int32_t top_parent;   // tile node that is the parent of the top node, -1 at a root
  int32_t aux;
  int32_t n_child;
  int32_t kind;
  int32_t slot;
  int32_t first;
};
constexpr int32_t kChainRegular = 0;

// A warp slot of one phase: nodes [n_begin, n_begin + n_count) in lane order.
// Lane l owns the chunk [n_begin + off[l], n_begin + off[l+1]) (the last used
// lane ends at n_count; idle lanes have off[l] = n_count).  steps = 0: every
// lane's chunk holds whole chains, walked serially; steps > 0: chains spread
// over up to 2^steps lanes each, joined by shuffle scans; unit = 1: one node
// per lane (lane l owns node n_begin + l).
struct SlotRec {
  int32_t n_begin;
  int16_t n_count;
  uint8_t steps;
  uint8_t unit;
  uint16_t off[32];
};

// Per-tile descriptor (global memory, read-only).
struct TileDesc {
  int64_t blob_offset;      // bytes into the plan's blob buffer (16-B aligned)
  int32_t blob_bytes;       // total bytes of the tile blob (dynamic + static)
  int32_t dyn_bytes;        // leading bytes written back (V, states)
  int32_t n_nodes;          // N (padded node count used for array strides)
  int32_t n_real_nodes;     // nodes actually used
  int32_t n_chains;
  int32_t n_phases;
  int32_t n_params;         // param records in this tile
  int32_t n_pulses;
  int64_t pulse_offset;     // into plan pulse array
  int32_t n_xprobes;        // mechanism probes of the tile (ProbeRef list at off_plist)
  int32_t param_stride;     // reals per parameter record (kParamStride or kParamStrideCore)
  int64_t probe_offset;     // into plan probe array
  // byte offsets inside the blob
  int32_t off_v;            // (V_hi, V_lo) pairs
  int32_t off_plist;        // the tile's mechanism-probe list (ProbeRef)
  int64_t state_offset;     // elements into the plan's global mechanism-state array ([slot][n_nodes])
  int32_t off_ab;           // (alpha, beta) pairs
  int32_t off_diag0, off_pidx, off_spec, off_specs;
  int32_t off_chains, off_slots, off_phase, off_crec, off_params, off_mech;
  int32_t scratch_bytes;    // diag/rhs/cD/cR scratch (shared memory after the blob)
  int32_t off_dr;           // (diagonal, rhs) pairs, inside the scratch area
  int32_t off_scd, off_scr;  // contribution slots, inside the scratch area
  int32_t n_slots;          // contribution slots (scd / scr / sh entries)
  int32_t n_cells;          // cells in the tile
  // network: tile synapse list (global ids), per-node tile-local cell index and
  // per-cell global id of spike sources (-1: not a source); off_ncell = -1 when
  // the tile has no spike source.  off_stamp: per-cell spike step (scratch).
  int32_t off_syn, off_ncell, off_srccell, off_stamp;
  int64_t scratch_offset;   // bytes into the plan's global scratch (global-resident tiles)
  int64_t port_offset;      // into the plan's port array (subtree-surrogate ports of this tile)
  int32_t n_ports;
  int32_t off_pstage;       // the GRU weight fragments and wo (kGruSmemBytes), then per-port staging
                            // records (PortStage), then PortLocal records, inside the
                            // scratch area; -1: none
  // lane tiles (one small cell per thread): node v of lane l is tile node v * L + l
  // (L = threads of the launch); crec holds each node's parent v (0xFFFF at the
  // root); off_lane_n: int32 node count per lane (0: no cell).  -1 otherwise.
  int32_t off_lane_n;
  int32_t lane_kmax;        // largest node count of the tile's cells (lane tiles)
};

// Threads (= cells) per lane tile.
constexpr int kLaneThreads = 128;

// ------------------------------------------------------------- subtree surrogate
// GRU sizes and the layout of its flat FP32 parameter vector (training master
// copy, host files): Wh [3H][H] | Wx [3H][X] | bx [3H] | bh [3H] | wo [H] | bo,
// gate blocks in the order r, z, n.
constexpr int kGruH = 64;
constexpr int kGruX = 4;
constexpr int kGru3H = 3 * kGruH;
constexpr int kGruOffWh = 0;
constexpr int kGruOffWx = kGruOffWh + kGru3H * kGruH;
constexpr int kGruOffBx = kGruOffWx + kGru3H * kGruX;
constexpr int kGruOffBh = kGruOffBx + kGru3H;
constexpr int kGruOffWo = kGruOffBh + kGru3H;
constexpr int kGruOffBo = kGruOffWo + kGruH;
constexpr int kGruNParam = kGruOffBo + 1;
// Extended K of the tensor-core products: h (H) plus a 16-wide block of inputs
// and biases; rows of the extended weight matrix: r, z, hn, nx (4H).
constexpr int kGruK = kGruH + 16;
constexpr int kGruRows = 4 * kGruH;
// Per-port recurrent state (floats): h [2][H] in FP32 (read / write halves
// alternate by step parity), then the same two halves as BF16 pairs (the
// tensor-core operand, H / 2 words each), then the attachment voltage of the
// last step and a "seen" mark.
constexpr int kPortHBf = 2 * kGruH;            // offset of the BF16 halves
constexpr int kPortVPrev = kPortHBf + kGruH;    // offset of (v_prev, seen)
constexpr int kPortStride = kPortVPrev + 4;
// A tile with ports holds the B fragments of the extended weight matrix in its
// scratch, fragment-major: for N group jb (8 units) there are 16 fragment slots,
// (block q < 3, k step kk < 5) at slot 5 q + kk and the nx block's x step at
// slot 15; a slot is 32 lanes x one (b0, b1) word pair, so a warp reads it as
// 256 contiguous bytes (no bank conflicts).  Rows that the slot omits (the nx
// rows' h steps) are zero in the row-major matrix.
constexpr int kGruFragSlots = 16;
constexpr int kGruFragPairs = 8 * kGruFragSlots * 32;                       // uint2 per tile
constexpr int kGruFragBytes = kGruFragPairs * 8;                            // 32 KB
constexpr int kGruSmemBytes = kGruFragBytes + kGruH * 4;                    // + output weights wo
__host__ __device__ constexpr int gru_frag_slot(int q, int kk) { return q < 3 ? 5 * q + kk : 15; }

// Launch shape of the kernel variant with ports: at most BC_PORT_MAX_THREADS
// threads per tile, register budget for BC_PORT_MIN_CTAS resident tiles per SM.
#ifndef BC_PORT_MAX_THREADS
#define BC_PORT_MAX_THREADS 768
#endif
#ifndef BC_PORT_MIN_CTAS
#define BC_PORT_MIN_CTAS 1
#endif

// Per-step staging of a port inside the tile's scratch: the GRU inputs, the
// endpoint node, the factor that turns y into the row's right-hand side and the
// port id (row of its hidden state).
struct PortStage {
  float x[4];
  int32_t node;
  float coef;
  int32_t id;
  int32_t pad;
};

// A port's record and envelope state in the tile's scratch for the length of a
// launch (copied in at the start, the envelope state written back at the end).
struct PortLocal {
  int32_t node, att, cell, id, stim_begin, stim_end;
  double g, e;
  float feat[2];
  float v_prev, seen;
  int32_t pad[2];
};

// Inference weights of a plan (global memory, read through L1).
struct GruWeights {
  uint32_t wext[kGruRows * kGruK / 2];  // BF16 pairs, row-major [4H][K]
  float wo[kGruH];
  float bo;
  float v_scale;    // mV: voltage input = (V_att - e) / v_scale
  float y_scale;    // mV: port current = g (e + y_scale y - V_end)
  float env_v_lo;   // envelope of V_att - e, mV
  float env_v_hi;
  float env_dvdt;   // bound of |dV_att/dt|, mV/ms
  float pad[2];
};

// A port: the stand-in for a removed subtree.  node: tile-local endpoint node it
// feeds; att: tile-local node of the attachment CV; cell: batch cell id;
// id: plan port id (recurrent state row); its stimulus pulses are
// stim_begin .. stim_end of the plan's port-pulse array (amp in nA).
struct PortRec {
  int32_t node;
  int32_t att;
  int32_t cell;
  int32_t id;
  int32_t stim_begin;
  int32_t stim_end;
  double g;        // uS
  double e;        // mV
  float feat[2];
};

struct PulseRec {
  int32_t node;      // tile-local node
  int32_t is_mid;    // 1: density term (rhs += dt*invcm*amp), 0: boundary row (rhs += dt*amp)
  int64_t on_step;   // active for on_step <= step < off_step
  int64_t off_step;
  double amp;        // midpoint: uA/cm^2 (nA * 1e5 / area_um2); boundary: nA * 1e-3 (mV/ms per uF)
  double t_on, t_off;
};

// A node with clamp pulses, a voltage probe and/or synapses: its pulses are
// pulse_begin .. pulse_end of the tile's pulse list (sorted by node), its voltage
// probe id is `probe` (-1: none), its synapses are entries syn_begin .. syn_end of
// the tile's synapse list (global synapse ids).
struct SpecRec {
  int32_t pulse_begin;
  int32_t pulse_end;
  int32_t probe;
  int32_t syn_begin;
  int32_t syn_end;
  int32_t pad[3];
};

// A mechanism probe of a tile: its node, plan probe id and BC_STATE_* view
// (recorded in a pass of its own after the update pass).
struct ProbeRef {
  int32_t node;
  int32_t id;
  int32_t field;
  int32_t pad;
};

// Kernel launch parameters (by value).
struct LaunchArgs {
  const TileDesc* tiles;
  int32_t n_tiles;
  unsigned char* blob;        // plan blob buffer
  unsigned char* scratch;     // global scratch (global-resident tiles)
  void* state;                // mechanism states, [slot][node] per tile (Real)
  const PulseRec* pulses;
  double* traces;             // [trace_cap][n_probes_total], record-major
  int64_t trace_cap;          // records that fit
  int64_t trace_base;         // step count at the last probe clear
  int64_t n_probes_total;
  int32_t record_every;
  int32_t max_spikes;
  int32_t* spike_count;       // [n_probes]
  double* spike_times;        // [n_probes * max_spikes]
  int32_t* status;            // device status word (BC_* codes, OR-ed bits)
  int64_t step0;              // global index of the first step of this launch
  int32_t n_steps;
  int32_t state_slots;
  double dt;
  unsigned long long* timers;  // [4] cycle sums (elimination, back-sub, update, other); phase-timer builds only
  // synapses (Real arrays indexed by global synapse id) and network delivery
  void* syn_g;                 // conductance, uS
  const void* syn_tau;         // ms
  const void* syn_e;           // mV
  const void* syn_scale;       // 1e5 / CV area: uS -> mS/cm^2
  void* arrivals;              // [arr_slots][n_syn] event weights due per step (null: no network)
  int64_t arr_slots;
  int64_t n_syn;
  int32_t* rec_cell;           // spike records (source cell, step)
  int64_t* rec_step;
  unsigned long long* rec_count;
  int64_t rec_cap;
  // subtree-surrogate ports
  const PortRec* ports;
  const PulseRec* port_pulses;
  float* port_h;               // [n_ports][kPortStride]
  int32_t* port_flags;         // [n_cells] envelope exits
  const GruWeights* gru;
};

// Host-callable launchers implemented in bc_kernels.cu.
// variant: 0 = the lean kernel; 1 = the plan uses synapses, a network, mechanism
// probes, or a mechanism of the out-of-line set (classic HH Na / K, M current);
// 2 = as 1 plus subtree-surrogate ports; 3 = the lean kernel plus ports (a plan
// whose only optional feature is its ports).
int launch_tiles(const LaunchArgs& a, int precision, bool smem, int threads, size_t smem_bytes, int variant,
                 void* stream);
// Kernel-node parameters of the same launch for a CUDA graph.  kernelParams
// points at *hold, which points at *a: both must stay valid until the graph
// call that consumes the parameters returns (it copies the argument).
int tile_node_params(const LaunchArgs* a, int precision, bool smem, int threads, size_t smem_bytes, int variant,
                     cudaKernelNodeParams* np, const LaunchArgs** hold);
// Lane tiles: each thread runs one whole small cell (serial Hines elimination
// and back-substitution over its nodes, then its update), no barriers in a step.
int launch_lanes(const LaunchArgs& a, int precision, int threads, bool extra, void* stream);
int lane_node_params(const LaunchArgs* a, int precision, int threads, bool extra, cudaKernelNodeParams* np,
                     const LaunchArgs** hold);
int launch_reset_impl(const LaunchArgs& a, int precision, int threads, const double* vinit, const int64_t* voff,
                      void* stream);
// View offsets: byte offsets into the blob, or kStateTag + byte offset into the state array.
constexpr int64_t kStateTag = int64_t(1) << 62;
int launch_view_impl(unsigned char* blob, unsigned char* state, int precision, const int64_t* off_hi,
                     const int64_t* off_lo, double* view, int64_t n, bool write, void* stream);
// Event delivery after a launch: every spike record in [*rec_done, *rec_count)
// adds the weights of its source cell's connections into the arrival ring.
int launch_deliver_impl(int precision, const int32_t* rec_cell, const int64_t* rec_step,
                        const unsigned long long* rec_count, const unsigned long long* rec_done, int64_t rec_cap,
                        const int64_t* out_ptr, const int64_t* out_syn, const void* out_w, const int32_t* out_d,
                        void* arrivals, int64_t arr_slots, int64_t n_syn, void* stream);
// Device address (on the current device) of the fixed scratch behind
// bc_state_download_noalloc: [hi offsets | lo offsets | values], BC_NOALLOC_MAX_CV
// 8-byte entries each.  Returns the cudaError_t of cudaGetSymbolAddress.
int noalloc_view_scratch_address(void** out);

}  // namespace bc
