// GRU building blocks shared by the subtree-surrogate port phase of the step
// kernel and by the training kernels, so that the network that was trained is
// evaluated with the same arithmetic.
//
// The cell (hidden H = 64, inputs X = 4) follows the usual GRU form:
//   r  = sigmoid(Wx_r x + bx_r + Wh_r h~ + bh_r)
//   z  = sigmoid(Wx_z x + bx_z + Wh_z h~ + bh_z)
//   hn = Wh_n h~ + bh_n
//   n  = tanh(Wx_n x + bx_n + r * hn)
//   h' = (1 - z) n + z h
//   y  = wo . h' + bo
// h is kept in FP32; h~ = bf16(h).  All four pre-activation blocks (r, z, hn and
// the input part of n, "nx") come out of mma.sync m16n8k16 BF16 tiles with FP32
// accumulation over an extended K of 80: k < 64 is h~ against Wh, and the
// 16-wide "x block" carries the inputs and the biases,
//   A columns: bf16(x0..x3) | bf16(x - bf16(x)) (x0..x3) | 1 | 1 | 0 ...
//   B rows   : bf16(Wx)     | bf16(Wx)                    | b_hi | b_lo | 0 ...
// so x reaches the product with about 16 significant bits and each bias as the
// sum of two BF16 halves; Wx itself is BF16.  The r and z rows carry the summed
// biases bx + bh, the hn rows bh_n (no inputs), the nx rows Wx_n and bx_n (no h).
// M tiles are 16 sequences (or ports); an N group is 8 hidden units of each of
// the four blocks.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "bc_internal.h"

namespace bc {

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&p);
}

__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// D = A B + D for one 16x8x16 BF16 tile (FP32 accumulators).
// Fragments (g = lane / 4, t = lane % 4):
//   A: a[0] (row g, cols 2t..2t+1), a[1] (row g+8), a[2] (row g, cols 2t+8..), a[3] (row g+8, cols 2t+8..)
//   B: b0 (k 2t..2t+1, col g), b1 (k 2t+8..2t+9, col g)
//   D: d[0..1] (row g, cols 2t, 2t+1), d[2..3] (row g+8, cols 2t, 2t+1)
__device__ __forceinline__ void mma_bf16_16816(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float ex2_approx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rcp_fast(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// sigmoid(x) = 1 / (1 + 2^(-x log2 e)) and tanh(x) = 1 - 2 / (1 + 2^(2 x log2 e)):
// one base-2 exponential and one reciprocal each (hardware approximations, both
// within a few ulp), saturating correctly at +-infinity.
constexpr float kLog2e = 1.4426950408889634f;
__device__ __forceinline__ float gru_sigmoid(float x) { return rcp_fast(1.0f + ex2_approx(-kLog2e * x)); }
__device__ __forceinline__ float gru_tanh(float x) { return 1.0f - 2.0f * rcp_fast(1.0f + ex2_approx(2.0f * kLog2e * x)); }

// A fragment of the x block for rows g (inputs xa) and g + 8 (inputs xb).
__device__ __forceinline__ void xblock_frag(const float* xa, const float* xb, int tq, uint32_t* a) {
  float a0, a1, b0, b1;
  if (tq < 2) {  // columns 2 tq, 2 tq + 1: bf16 of inputs 2 tq, 2 tq + 1
    a0 = xa[2 * tq];
    a1 = xa[2 * tq + 1];
    b0 = xb[2 * tq];
    b1 = xb[2 * tq + 1];
  } else {       // columns 4..7: the low halves of inputs 0..3
    const int i = 2 * (tq - 2);
    a0 = xa[i] - bf16_round(xa[i]);
    a1 = xa[i + 1] - bf16_round(xa[i + 1]);
    b0 = xb[i] - bf16_round(xb[i]);
    b1 = xb[i + 1] - bf16_round(xb[i + 1]);
  }
  a[0] = pack_bf16(a0, a1);
  a[1] = pack_bf16(b0, b1);
  const float one = tq == 0 ? 1.0f : 0.0f;  // columns 8, 9: the two bias halves
  a[2] = pack_bf16(one, one);
  a[3] = a[2];
}

// Pre-activations of N group jb (units 8 jb .. 8 jb + 7) for one M tile:
// acc[0] r, acc[1] z, acc[2] hn, acc[3] nx.  ah: A fragments of h~ (4 k steps),
// ax: the x block.  wext: BF16 pairs, row-major [4H][kGruK] (rows r, z, hn, nx).
__device__ __forceinline__ void gru_preact(const uint32_t* __restrict__ wext, int jb, int g, int tq,
                                           const uint32_t (*ah)[4], const uint32_t* ax, float (*acc)[4]) {
  constexpr int kRow = kGruK / 2;  // uint32 per row
#pragma unroll
  for (int q = 0; q < 4; ++q) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.0f;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const uint32_t* w = wext + size_t(q * kGruH + jb * 8 + g) * kRow;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) mma_bf16_16816(acc[q], ah[kk], __ldg(w + kk * 8 + tq), __ldg(w + kk * 8 + 4 + tq));
    mma_bf16_16816(acc[q], ax, __ldg(w + 32 + tq), __ldg(w + 36 + tq));
  }
  const uint32_t* w = wext + size_t(3 * kGruH + jb * 8 + g) * kRow;
  mma_bf16_16816(acc[3], ax, __ldg(w + 32 + tq), __ldg(w + 36 + tq));
}

// Copy the row-major extended matrix into the fragment-major layout of a tile's
// scratch (kGruFragPairs word pairs; see kGruFragSlots).
__device__ __forceinline__ void gru_frag_fill(const uint32_t* __restrict__ wext, uint2* frag, int tid, int T) {
  constexpr int kRow = kGruK / 2;
  for (int i = tid; i < kGruFragPairs; i += T) {
    const int lane = i & 31, slot = (i >> 5) % kGruFragSlots, jb = i / (32 * kGruFragSlots);
    const int q = slot < 15 ? slot / 5 : 3, kk = slot < 15 ? slot % 5 : 4;
    const uint32_t* w = wext + size_t(q * kGruH + jb * 8 + (lane >> 2)) * kRow + kk * 8 + (lane & 3);
    frag[i] = make_uint2(__ldg(w), __ldg(w + 4));
  }
}

// gru_preact with the B fragments of N group jb taken from the fragment-major
// copy (frag = the tile's copy + jb * 16 slots * 32 lanes): the same products
// in the same order, so the same results.
__device__ __forceinline__ void gru_preact_frag(const uint2* frag, int lane, const uint32_t (*ah)[4],
                                                const uint32_t* ax, float (*acc)[4]) {
#pragma unroll
  for (int q = 0; q < 4; ++q) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.0f;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const uint2 b = frag[gru_frag_slot(q, kk) * 32 + lane];
      mma_bf16_16816(acc[q], ah[kk], b.x, b.y);
    }
    const uint2 b = frag[gru_frag_slot(q, 4) * 32 + lane];
    mma_bf16_16816(acc[q], ax, b.x, b.y);
  }
  const uint2 b = frag[gru_frag_slot(3, 4) * 32 + lane];
  mma_bf16_16816(acc[3], ax, b.x, b.y);
}

struct GruGate {
  float r, z, n, hn, h_new;
};

__device__ __forceinline__ GruGate gru_gate(float pr, float pz, float hn, float nx, float h_old) {
  GruGate g;
  g.r = gru_sigmoid(pr);
  g.z = gru_sigmoid(pz);
  g.hn = hn;
  g.n = gru_tanh(nx + g.r * hn);
  g.h_new = g.n + g.z * (h_old - g.n);
  return g;
}

}  // namespace bc
