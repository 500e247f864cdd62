// Training kernels of the subtree-surrogate GRU: forward over a window of a
// batch of sequences (storing the activations), backward through time with the
// weight gradients accumulated in the same pass, Adam, and the BF16 packing of
// the recurrent weights.  One CTA owns an M tile of 16 sequences for the whole
// window; warp w owns hidden units [8w, 8w + 8) in the elementwise parts.
//
// Loss: mean over the window's (sequence, step) entries of (y - y_target)^2.
// Truncated BPTT: the hidden state is carried from window to window, the
// gradient is not.
#include <cuda_runtime.h>

#include <cmath>

#include "../../include/braincell_gb300.h"
#include "bc_gru.cuh"
#include "bc_internal.h"

namespace bc {
namespace {

constexpr int kRows = 16;      // sequences per CTA
constexpr int kWarps = 8;      // kGruH / 8
constexpr int kThreads = kWarps * 32;
constexpr int kHPad = kGruH + 8;        // fp32 row stride of the hidden tile
constexpr int kGPad = kGru3H + 8;       // bf16 row stride of dG [row][n]
constexpr int kRPad = kRows + 8;        // bf16 row stride of dG^T [n][row] and h^T [k][row]
constexpr int kDPad = kGruH + 4;        // fp32 row stride of dh [row][k]
// Row stride (floats) of the per-CTA gradient rows of the backward: kGruNParam
// rounded up to a multiple of 4, so that every row starts on a 16-byte boundary
// (the recurrent block is stored as float2 pairs).
constexpr int kPartialStride = (kGruNParam + 3) & ~3;

struct FwdArgs {
  const float* params;
  const uint32_t* wext;
  const float* x;
  const float* y;
  int64_t t_total;
  const int32_t* seq;
  int32_t batch;
  int64_t t0;
  int32_t T;
  float* h;
  float* acts;  // [5][batch][T][H] or null
  float* yout;  // [batch][T] or null
  double* loss;
};

struct BwdArgs {
  const float* params;
  const uint32_t* wht;
  const float* x;
  const float* y;
  int64_t t_total;
  const int32_t* seq;
  int32_t batch;
  int64_t t0;
  int32_t T;
  const float* acts;
  const float* yout;
  float gscale;
  float* partial;  // [gridDim.x][kPartialStride]: this CTA's gradient, every entry written
};

__device__ __forceinline__ size_t act_index(int k, int batch, int T, int b, int t, int j) {
  return ((size_t(k) * batch + b) * T + t) * kGruH + j;
}

__global__ void __launch_bounds__(kThreads) gru_fwd_kernel(FwdArgs a) {
  __shared__ __align__(16) float hs[2][kRows][kHPad];
  __shared__ float ypart[2][kWarps][kRows];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane >> 2, tq = lane & 3;
  const int b_base = blockIdx.x * kRows;
  const float* wo = a.params + kGruOffWo;
  const float bo = a.params[kGruOffBo];

  for (int i = threadIdx.x; i < kRows * kGruH; i += kThreads) {
    const int r = i / kGruH, j = i % kGruH;
    const int b = b_base + r;
    hs[0][r][j] = b < a.batch ? a.h[size_t(b) * kGruH + j] : 0.0f;
  }
  const int r0 = g, r1 = g + 8;
  const int b0 = b_base + r0, b1 = b_base + r1;
  const bool v0 = b0 < a.batch, v1 = b1 < a.batch;
  const int64_t s0 = v0 ? a.seq[b0] : 0, s1 = v1 ? a.seq[b1] : 0;
  double loss = 0.0;
  __syncthreads();

  for (int t = 0; t < a.T; ++t) {
    const int cur = t & 1, nxt = cur ^ 1;
    float x0[kGruX], x1[kGruX];
    const int64_t tt = a.t0 + t;
#pragma unroll
    for (int i = 0; i < kGruX; ++i) {
      x0[i] = v0 ? a.x[(s0 * a.t_total + tt) * kGruX + i] : 0.0f;
      x1[i] = v1 ? a.x[(s1 * a.t_total + tt) * kGruX + i] : 0.0f;
    }
    uint32_t ah[4][4], ax[4];
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const int c = kk * 16 + 2 * tq;
      const float2 p0 = *reinterpret_cast<const float2*>(&hs[cur][r0][c]);
      const float2 p1 = *reinterpret_cast<const float2*>(&hs[cur][r1][c]);
      const float2 p2 = *reinterpret_cast<const float2*>(&hs[cur][r0][c + 8]);
      const float2 p3 = *reinterpret_cast<const float2*>(&hs[cur][r1][c + 8]);
      ah[kk][0] = pack_bf16(p0.x, p0.y);
      ah[kk][1] = pack_bf16(p1.x, p1.y);
      ah[kk][2] = pack_bf16(p2.x, p2.y);
      ah[kk][3] = pack_bf16(p3.x, p3.y);
    }
    xblock_frag(x0, x1, tq, ax);
    float acc[4][4];
    gru_preact(a.wext, w, g, tq, ah, ax, acc);
    float ys0 = 0.0f, ys1 = 0.0f;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int row = e < 2 ? r0 : r1;
      const int j = 8 * w + 2 * tq + (e & 1);
      const float h_old = hs[cur][row][j];
      const GruGate G = gru_gate(acc[0][e], acc[1][e], acc[2][e], acc[3][e], h_old);
      hs[nxt][row][j] = G.h_new;
      if (e < 2)
        ys0 += wo[j] * G.h_new;
      else
        ys1 += wo[j] * G.h_new;
      const bool valid = e < 2 ? v0 : v1;
      if (a.acts && valid) {
        const int b = b_base + row;
        a.acts[act_index(0, a.batch, a.T, b, t, j)] = h_old;
        a.acts[act_index(1, a.batch, a.T, b, t, j)] = G.r;
        a.acts[act_index(2, a.batch, a.T, b, t, j)] = G.z;
        a.acts[act_index(3, a.batch, a.T, b, t, j)] = G.n;
        a.acts[act_index(4, a.batch, a.T, b, t, j)] = G.hn;
      }
    }
    ys0 += __shfl_xor_sync(0xffffffffu, ys0, 1);
    ys0 += __shfl_xor_sync(0xffffffffu, ys0, 2);
    ys1 += __shfl_xor_sync(0xffffffffu, ys1, 1);
    ys1 += __shfl_xor_sync(0xffffffffu, ys1, 2);
    if (tq == 0) {
      ypart[cur][w][r0] = ys0;
      ypart[cur][w][r1] = ys1;
    }
    __syncthreads();
    if (w == 0 && lane < kRows) {
      const int b = b_base + lane;
      if (b < a.batch) {
        float y = bo;
#pragma unroll
        for (int q = 0; q < kWarps; ++q) y += ypart[cur][q][lane];
        if (a.yout) a.yout[size_t(b) * a.T + t] = y;
        if (a.y) {
          const double err = double(y) - double(a.y[int64_t(a.seq[b]) * a.t_total + tt]);
          loss += err * err;
        }
      }
    }
  }
  __syncthreads();
  const int fin = a.T & 1;
  for (int i = threadIdx.x; i < kRows * kGruH; i += kThreads) {
    const int r = i / kGruH, j = i % kGruH;
    const int b = b_base + r;
    if (b < a.batch) a.h[size_t(b) * kGruH + j] = hs[fin][r][j];
  }
  if (a.loss && w == 0 && lane < kRows && loss != 0.0) atomicAdd(a.loss, loss);
}

__global__ void __launch_bounds__(kThreads) gru_bwd_kernel(BwdArgs a) {
  __shared__ __align__(16) __nv_bfloat16 dG[2][kRows][kGPad];
  __shared__ __align__(16) __nv_bfloat16 dGT[2][kGru3H][kRPad];
  __shared__ __align__(16) __nv_bfloat16 HT[2][kGruH][kRPad];
  __shared__ __align__(16) float dHs[2][kRows][kDPad];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane >> 2, tq = lane & 3;
  const int b_base = blockIdx.x * kRows;
  const float* wo = a.params + kGruOffWo;
  const int r0 = g, r1 = g + 8;
  const int b0 = b_base + r0, b1 = b_base + r1;
  const bool v0 = b0 < a.batch, v1 = b1 < a.batch;
  const int64_t s0 = v0 ? a.seq[b0] : 0, s1 = v1 ? a.seq[b1] : 0;

  float carry[4] = {0.0f, 0.0f, 0.0f, 0.0f};     // dL/dh' of this step from later steps
  float gwx[3][2][kGruX], gbx[3][2], gbh[3][2], gwo[2];
#pragma unroll
  for (int q = 0; q < 3; ++q)
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      gbx[q][u] = gbh[q][u] = 0.0f;
#pragma unroll
      for (int i = 0; i < kGruX; ++i) gwx[q][u][i] = 0.0f;
    }
  gwo[0] = gwo[1] = 0.0f;
  float gbo = 0.0f;
  float accw[12][4];
#pragma unroll
  for (int i = 0; i < 12; ++i)
#pragma unroll
    for (int e = 0; e < 4; ++e) accw[i][e] = 0.0f;
  const int mt = w >> 1, nt = w & 1;  // this warp's tile of the dh^T = Wh^T dG^T product

  for (int t = a.T - 1; t >= 0; --t) {
    const int cur = t & 1;
    const int64_t tt = a.t0 + t;
    float x0[kGruX], x1[kGruX];
#pragma unroll
    for (int i = 0; i < kGruX; ++i) {
      x0[i] = v0 ? a.x[(s0 * a.t_total + tt) * kGruX + i] : 0.0f;
      x1[i] = v1 ? a.x[(s1 * a.t_total + tt) * kGruX + i] : 0.0f;
    }
    const float dy0 = v0 ? a.gscale * (a.yout[size_t(b0) * a.T + t] - a.y[s0 * a.t_total + tt]) : 0.0f;
    const float dy1 = v1 ? a.gscale * (a.yout[size_t(b1) * a.T + t] - a.y[s1 * a.t_total + tt]) : 0.0f;
    float dh_dir[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int row = e < 2 ? r0 : r1;
      const bool valid = e < 2 ? v0 : v1;
      const int u = e & 1;
      const int j = 8 * w + 2 * tq + u;
      const int b = b_base + row;
      float h_old = 0.0f, r = 0.0f, z = 0.0f, n = 0.0f, hn = 0.0f;
      if (valid) {
        h_old = a.acts[act_index(0, a.batch, a.T, b, t, j)];
        r = a.acts[act_index(1, a.batch, a.T, b, t, j)];
        z = a.acts[act_index(2, a.batch, a.T, b, t, j)];
        n = a.acts[act_index(3, a.batch, a.T, b, t, j)];
        hn = a.acts[act_index(4, a.batch, a.T, b, t, j)];
      }
      const float dy = e < 2 ? dy0 : dy1;
      const float h_new = (1.0f - z) * n + z * h_old;
      const float dh = carry[e] + dy * wo[j];
      const float dn = dh * (1.0f - z);
      const float dz = dh * (h_old - n);
      dh_dir[e] = dh * z;
      const float dan = dn * (1.0f - n * n);
      const float dr = dan * hn;
      const float dar = dr * r * (1.0f - r);
      const float daz = dz * z * (1.0f - z);
      const float dhn = dan * r;
      const float* xr = e < 2 ? x0 : x1;
#pragma unroll
      for (int i = 0; i < kGruX; ++i) {
        gwx[0][u][i] += dar * xr[i];
        gwx[1][u][i] += daz * xr[i];
        gwx[2][u][i] += dan * xr[i];
      }
      gbx[0][u] += dar;
      gbx[1][u] += daz;
      gbx[2][u] += dan;
      gbh[0][u] += dar;
      gbh[1][u] += daz;
      gbh[2][u] += dhn;
      gwo[u] += dy * h_new;
      const __nv_bfloat16 qr = __float2bfloat16_rn(dar), qz = __float2bfloat16_rn(daz),
                          qn = __float2bfloat16_rn(dhn);
      dG[cur][row][j] = qr;
      dG[cur][row][kGruH + j] = qz;
      dG[cur][row][2 * kGruH + j] = qn;
      dGT[cur][j][row] = qr;
      dGT[cur][kGruH + j][row] = qz;
      dGT[cur][2 * kGruH + j][row] = qn;
      HT[cur][j][row] = __float2bfloat16_rn(h_old);
    }
    if (w == 0 && tq == 0) gbo += dy0 + dy1;
    __syncthreads();
    {
      // dh^T[k][row] = sum_n Wh^T[k][n] dG[row][n]: M = k (16 per tile), N = rows, K = 3H
      float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      const int kr0 = mt * 16 + g, kr1 = kr0 + 8;
#pragma unroll
      for (int kk = 0; kk < kGru3H / 16; ++kk) {
        const uint32_t af[4] = {a.wht[kr0 * (kGru3H / 2) + kk * 8 + tq], a.wht[kr1 * (kGru3H / 2) + kk * 8 + tq],
                                a.wht[kr0 * (kGru3H / 2) + kk * 8 + 4 + tq],
                                a.wht[kr1 * (kGru3H / 2) + kk * 8 + 4 + tq]};
        const uint32_t bb0 = *reinterpret_cast<const uint32_t*>(&dG[cur][nt * 8 + g][kk * 16 + 2 * tq]);
        const uint32_t bb1 = *reinterpret_cast<const uint32_t*>(&dG[cur][nt * 8 + g][kk * 16 + 2 * tq + 8]);
        mma_bf16_16816(c, af, bb0, bb1);
      }
      const int rr = nt * 8 + 2 * tq;
      dHs[cur][rr][kr0] = c[0];
      dHs[cur][rr + 1][kr0] = c[1];
      dHs[cur][rr][kr1] = c[2];
      dHs[cur][rr + 1][kr1] = c[3];
    }
    // dWh[n][k] += sum_row dG[row][n] h~[row][k]: M = n, N = k, K = 16 rows
#pragma unroll
    for (int i = 0; i < 12; ++i) {
      const int q = 12 * w + i;
      const int mi = q >> 3, ni = q & 7;
      const uint32_t af[4] = {*reinterpret_cast<const uint32_t*>(&dGT[cur][mi * 16 + g][2 * tq]),
                              *reinterpret_cast<const uint32_t*>(&dGT[cur][mi * 16 + g + 8][2 * tq]),
                              *reinterpret_cast<const uint32_t*>(&dGT[cur][mi * 16 + g][2 * tq + 8]),
                              *reinterpret_cast<const uint32_t*>(&dGT[cur][mi * 16 + g + 8][2 * tq + 8])};
      const uint32_t bb0 = *reinterpret_cast<const uint32_t*>(&HT[cur][ni * 8 + g][2 * tq]);
      const uint32_t bb1 = *reinterpret_cast<const uint32_t*>(&HT[cur][ni * 8 + g][2 * tq + 8]);
      mma_bf16_16816(accw[i], af, bb0, bb1);
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int row = e < 2 ? r0 : r1;
      const int j = 8 * w + 2 * tq + (e & 1);
      carry[e] = dh_dir[e] + dHs[cur][row][j];
    }
  }
  // This CTA's gradient goes to its own row of the partial buffer, each entry
  // written by exactly one lane; bc_gru_backward then sums the rows in CTA order,
  // so the gradient is the same bit for bit on every run.
  float* G = a.partial + size_t(blockIdx.x) * kPartialStride;
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    const int q = 12 * w + i;
    const int mi = q >> 3, ni = q & 7;
    const int n0 = mi * 16 + g, k0 = ni * 8 + 2 * tq;
    *reinterpret_cast<float2*>(&G[kGruOffWh + n0 * kGruH + k0]) = make_float2(accw[i][0], accw[i][1]);
    *reinterpret_cast<float2*>(&G[kGruOffWh + (n0 + 8) * kGruH + k0]) = make_float2(accw[i][2], accw[i][3]);
  }
  // the per-unit sums: reduce over the 8 lanes that share a unit (same tq)
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int j = 8 * w + 2 * tq + u;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
#pragma unroll
      for (int i = 0; i < kGruX; ++i) {
        float v = gwx[q][u][i];
        v += __shfl_xor_sync(0xffffffffu, v, 4);
        v += __shfl_xor_sync(0xffffffffu, v, 8);
        v += __shfl_xor_sync(0xffffffffu, v, 16);
        if (g == 0) G[kGruOffWx + (q * kGruH + j) * kGruX + i] = v;
      }
      float vb = gbx[q][u], vh = gbh[q][u];
      vb += __shfl_xor_sync(0xffffffffu, vb, 4);
      vb += __shfl_xor_sync(0xffffffffu, vb, 8);
      vb += __shfl_xor_sync(0xffffffffu, vb, 16);
      vh += __shfl_xor_sync(0xffffffffu, vh, 4);
      vh += __shfl_xor_sync(0xffffffffu, vh, 8);
      vh += __shfl_xor_sync(0xffffffffu, vh, 16);
      if (g == 0) {
        G[kGruOffBx + q * kGruH + j] = vb;
        G[kGruOffBh + q * kGruH + j] = vh;
      }
    }
    float vo = gwo[u];
    vo += __shfl_xor_sync(0xffffffffu, vo, 4);
    vo += __shfl_xor_sync(0xffffffffu, vo, 8);
    vo += __shfl_xor_sync(0xffffffffu, vo, 16);
    if (g == 0) G[kGruOffWo + j] = vo;
  }
  if (w == 0) {
    float vb = tq == 0 ? gbo : 0.0f;
#pragma unroll
    for (int s = 1; s < 32; s <<= 1) vb += __shfl_xor_sync(0xffffffffu, vb, s);
    if (lane == 0) G[kGruOffBo] = vb;
  }
}

// grads[i] += sum over the CTAs c = 0, 1, ... of partial[c][i], in that order.
__global__ void gru_grad_reduce_kernel(const float* partial, int n_cta, float* grads) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kGruNParam; i += gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int c = 0; c < n_cta; ++c) s += partial[size_t(c) * kPartialStride + i];
    grads[i] += s;
  }
}

// Adam on the FP32 master vector; the gradient is cleared for the next window.
__global__ void gru_adam_kernel(float* p, float* gr, float* m, float* v, int n, float lr, float b1, float b2, float eps,
                                float c1, float c2, float clip_scale) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = gr[i] * clip_scale;
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    gr[i] = 0.0f;
  }
}

__global__ void gru_sqnorm_kernel(const float* gr, int n, float* out) {
  float s = 0.0f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s += gr[i] * gr[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

// Extended weight matrix (BF16 pairs, [4H][K], rows r, z, hn, nx; see
// bc_gru.cuh) and the transposed recurrent block Wh^T [H][3H] for the backward.
__device__ __forceinline__ float wext_value(const float* p, int n, int k) {
  const int q = n / kGruH, u = n % kGruH;
  if (k < kGruH) return q < 3 ? p[kGruOffWh + (q * kGruH + u) * kGruH + k] : 0.0f;
  const int c = k - kGruH;
  const int xrow = q == 0 ? u : q == 1 ? kGruH + u : 2 * kGruH + u;  // Wx row of this block
  if (c < 2 * kGruX) return q == 2 ? 0.0f : bf16_round(p[kGruOffWx + xrow * kGruX + (c % kGruX)]);
  if (c < 2 * kGruX + 2) {
    const float bsum = q == 0   ? p[kGruOffBx + u] + p[kGruOffBh + u]
                       : q == 1 ? p[kGruOffBx + kGruH + u] + p[kGruOffBh + kGruH + u]
                       : q == 2 ? p[kGruOffBh + 2 * kGruH + u]
                                : p[kGruOffBx + 2 * kGruH + u];
    const float hi = bf16_round(bsum);
    return c == 2 * kGruX ? hi : bsum - hi;
  }
  return 0.0f;
}

__global__ void gru_pack_kernel(const float* p, uint32_t* wext, uint32_t* wht) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kGruRows * kGruK / 2; i += gridDim.x * blockDim.x) {
    const int n = i / (kGruK / 2), k = 2 * (i % (kGruK / 2));
    wext[i] = pack_bf16(wext_value(p, n, k), wext_value(p, n, k + 1));
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kGru3H * kGruH / 2; i += gridDim.x * blockDim.x) {
    const int kt = i / (kGru3H / 2), nt = 2 * (i % (kGru3H / 2));
    wht[i] = pack_bf16(p[kGruOffWh + nt * kGruH + kt], p[kGruOffWh + (nt + 1) * kGruH + kt]);
  }
}

bc_status launch_status(cudaError_t e, const char* what) {
  if (e != cudaSuccess) return fail(BC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return BC_OK;
}

}  // namespace
}  // namespace bc

using namespace bc;

extern "C" {

int32_t bc_gru_nparam(void) { return kGruNParam; }

bc_status bc_gru_pack(const float* params, uint32_t* wext, uint32_t* wht, void* stream) {
  if (!params || !wext || !wht) return fail(BC_ERR_INVALID, "bc_gru_pack: null buffer");
  gru_pack_kernel<<<40, 256, 0, static_cast<cudaStream_t>(stream)>>>(params, wext, wht);
  return launch_status(cudaGetLastError(), "gru_pack_kernel");
}

bc_status bc_gru_forward(const float* params, const uint32_t* wext, const float* x, const float* y, int64_t t_total,
                         const int32_t* seq, int32_t batch, int64_t t0, int32_t T, float* h, float* acts, float* yout,
                         double* loss, void* stream) {
  if (!params || !wext || !x || !seq || !h) return fail(BC_ERR_INVALID, "bc_gru_forward: null buffer");
  if (batch <= 0 || T <= 0 || t0 < 0 || t0 + T > t_total)
    return fail(BC_ERR_INVALID, "bc_gru_forward: window outside the sequences");
  if (acts && !yout) return fail(BC_ERR_INVALID, "bc_gru_forward: acts need yout");
  FwdArgs a{params, wext, x, y, t_total, seq, batch, t0, T, h, acts, yout, loss};
  gru_fwd_kernel<<<(batch + kRows - 1) / kRows, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(a);
  return launch_status(cudaGetLastError(), "gru_fwd_kernel");
}

int64_t bc_gru_backward_workspace(int32_t batch) {
  return batch > 0 ? int64_t((batch + kRows - 1) / kRows) * kPartialStride : 0;
}

bc_status bc_gru_backward(const float* params, const uint32_t* wht, const float* x, const float* y, int64_t t_total,
                          const int32_t* seq, int32_t batch, int64_t t0, int32_t T, const float* acts,
                          const float* yout, float gscale, float* grads, float* workspace, void* stream) {
  if (!params || !wht || !x || !y || !seq || !acts || !yout || !grads || !workspace)
    return fail(BC_ERR_INVALID, "bc_gru_backward: null buffer");
  if (batch <= 0 || T <= 0 || t0 < 0 || t0 + T > t_total)
    return fail(BC_ERR_INVALID, "bc_gru_backward: window outside the sequences");
  if (reinterpret_cast<uintptr_t>(workspace) % 16 != 0)
    return fail(BC_ERR_INVALID, "bc_gru_backward: workspace must be 16-byte aligned");
  const int n_cta = (batch + kRows - 1) / kRows;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  BwdArgs a{params, wht, x, y, t_total, seq, batch, t0, T, acts, yout, gscale, workspace};
  gru_bwd_kernel<<<n_cta, kThreads, 0, st>>>(a);
  bc_status s = launch_status(cudaGetLastError(), "gru_bwd_kernel");
  if (s != BC_OK) return s;
  gru_grad_reduce_kernel<<<(kGruNParam + 255) / 256, 256, 0, st>>>(workspace, n_cta, grads);
  return launch_status(cudaGetLastError(), "gru_grad_reduce_kernel");
}

bc_status bc_gru_grad_sqnorm(const float* grads, float* out, void* stream) {
  if (!grads || !out) return fail(BC_ERR_INVALID, "bc_gru_grad_sqnorm: null buffer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(float), s);
  if (e != cudaSuccess) return launch_status(e, "cudaMemsetAsync");
  gru_sqnorm_kernel<<<8, 256, 0, s>>>(grads, kGruNParam, out);
  return launch_status(cudaGetLastError(), "gru_sqnorm_kernel");
}

bc_status bc_gru_adam(float* params, float* grads, float* m, float* v, int64_t step, float lr, float beta1,
                      float beta2, float eps, float clip_scale, void* stream) {
  if (!params || !grads || !m || !v) return fail(BC_ERR_INVALID, "bc_gru_adam: null buffer");
  if (step < 1) return fail(BC_ERR_INVALID, "bc_gru_adam: step counts from 1");
  const float c1 = float(1.0 / (1.0 - std::pow(double(beta1), double(step))));
  const float c2 = float(1.0 / (1.0 - std::pow(double(beta2), double(step))));
  gru_adam_kernel<<<(kGruNParam + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      params, grads, m, v, kGruNParam, lr, beta1, beta2, eps, c1, c2, clip_scale);
  return launch_status(cudaGetLastError(), "gru_adam_kernel");
}

}  // extern "C"
