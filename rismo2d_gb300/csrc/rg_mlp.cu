// Learned Newton warm start (include/rg300_mlp.h): stencil features, the
// network's forward pass and the backward products of its 128-wide layers on
// the tensor cores (mma.sync m16n8k16, bf16 operands, fp32 accumulation), the
// output layer's backward and Adam in fp32.
//
// Network per node: x (128, bf16) -> [W1 x + b1 -> gelu -> bf16] -> [W2 ...]
// -> [W3 ...] -> W4 h3 + b4 (3 outputs).  The outputs are the deviation of
// the next time level from the linear extrapolation 2 L1 - L2 of the last
// two, in units of the output scales.  Weights live as fp32 masters and a
// bf16 copy used by every product; the backward pass differentiates the
// computed function with the bf16 roundings taken as identity.

#include "rg_internal.cuh"
#include "../../include/rg300_mlp.h"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

namespace {

constexpr int D = 128;           // input and hidden width
constexpr int NOUT = 3;
constexpr int K = RG_MLP_STENCIL;
constexpr int FPS = 8;           // features per stencil node
constexpr int KP = 136;          // padded shared-memory row (bf16): conflict-free fragment loads
constexpr int TILE = 64;         // nodes per forward tile (4 warps x 16 rows)
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + D * D, OFF_W2 = OFF_B1 + D, OFF_B2 = OFF_W2 + D * D;
constexpr int OFF_W3 = OFF_B2 + D, OFF_B3 = OFF_W3 + D * D, OFF_W4 = OFF_B3 + D, OFF_B4 = OFF_W4 + NOUT * D;
constexpr int NPARAM = OFF_B4 + NOUT;
static_assert(NPARAM == RG_MLP_NPARAM, "parameter layout");
constexpr int WB_LAYER = D * D;          // bf16 weights: W1, W2, W3, then W4 padded to 8 rows
constexpr int WB_TOTAL = 3 * WB_LAYER + 8 * D;
constexpr size_t FWD_SMEM = (size_t)(3 * D + 8) * KP * 2 + (size_t)2 * TILE * KP * 2 + (3 * D + 8) * 4;

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * expf(-0.5f * z * z) * 0.39894228040143268f;
}

__device__ __forceinline__ unsigned ld_b32(const __nv_bfloat16* p) { return *reinterpret_cast<const unsigned*>(p); }

// D += A (16x16, row) * B (16x8, col), bf16 in, fp32 accumulate
__device__ __forceinline__ void mma_bf16(float (&d)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                         unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// ---- features ---------------------------------------------------------------
// per stencil slot s (node m): dz, H1, U1, V1, dS, dU, dV (level 1 - level 2
// over the step scales), distance; then q_next - 1, q_prev - 1 (x10), zeros.
// Missing slots are zero.
__global__ void k_features(int n, const int* __restrict__ nodes, const int* __restrict__ stencil,
                           const float* __restrict__ dist, const double* __restrict__ zb,
                           const double* __restrict__ st,   // 6 x np: U1 V1 S1 U2 V2 S2
                           int np, float href, float uref, float zref, float ssU, float ssV, float ssS,
                           float qn, float qp, __nv_bfloat16* __restrict__ X) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)n * D;
       t += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(t / D), f = (int)(t % D);
    const int nd = nodes[r];
    float v = 0.0f;
    if (f < K * FPS) {
      const int s = f / FPS, c = f % FPS;
      const int m = stencil[(size_t)nd * K + s];
      if (m >= 0) {
        const double* U1 = st;
        const double* V1 = st + np;
        const double* S1 = st + 2 * (size_t)np;
        const double* U2 = st + 3 * (size_t)np;
        const double* V2 = st + 4 * (size_t)np;
        const double* S2 = st + 5 * (size_t)np;
        // differences in FP64 (levels and elevations are large numbers), scaling in FP32
        switch (c) {
          case 0: v = (float)(zb[m] - zb[nd]) / zref; break;
          case 1: v = (float)fmax(S1[m] - zb[m], 0.0) / href; break;
          case 2: v = (float)U1[m] / uref; break;
          case 3: v = (float)V1[m] / uref; break;
          case 4: v = (float)(S1[m] - S2[m]) / ssS; break;
          case 5: v = (float)(U1[m] - U2[m]) / ssU; break;
          case 6: v = (float)(V1[m] - V2[m]) / ssV; break;
          default: v = dist[(size_t)nd * K + s]; break;
        }
      }
    } else if (f == K * FPS) {
      v = 10.0f * (qn - 1.0f);
    } else if (f == K * FPS + 1) {
      v = 10.0f * (qp - 1.0f);
    }
    v = fminf(fmaxf(v, -30.0f), 30.0f);
    X[t] = __float2bfloat16_rn(v);
  }
}

// ---- forward: persistent CTAs, all weights in shared memory ------------------
// rows: optional row index into X (gather), else identity.  STORE keeps the
// pre-activations z (fp32) and activations h (bf16) of the three hidden layers.
template <bool STORE>
__global__ void __launch_bounds__(128) k_forward(int n, const int* __restrict__ rows,
                                                 const __nv_bfloat16* __restrict__ X,
                                                 const __nv_bfloat16* __restrict__ Wb, const float* __restrict__ P,
                                                 float* __restrict__ Y, float* __restrict__ Z,
                                                 __nv_bfloat16* __restrict__ H) {
  extern __shared__ __align__(16) unsigned char smem[];
  __nv_bfloat16* sw = reinterpret_cast<__nv_bfloat16*>(smem);        // (3*128 + 8) x KP
  __nv_bfloat16* sa = sw + (size_t)(3 * D + 8) * KP;                  // 2 x TILE x KP
  float* sb = reinterpret_cast<float*>(sa + (size_t)2 * TILE * KP);   // b1 b2 b3 b4(8)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, c = lane & 3;
  for (int i = tid; i < (3 * D + 8) * D; i += blockDim.x) {
    const int row = i / D, col = i % D;
    sw[(size_t)row * KP + col] = Wb[i];
  }
  for (int i = tid; i < 3 * D + 8; i += blockDim.x) {
    float b = 0.0f;
    if (i < D) b = P[OFF_B1 + i];
    else if (i < 2 * D) b = P[OFF_B2 + i - D];
    else if (i < 3 * D) b = P[OFF_B3 + i - 2 * D];
    else if (i - 3 * D < NOUT) b = P[OFF_B4 + i - 3 * D];
    sb[i] = b;
  }
  __syncthreads();
  const int ntiles = (n + TILE - 1) / TILE;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int r0 = tile * TILE;
    // input tile -> buffer 0 (rows beyond n are zero)
    for (int i = tid; i < TILE * (D / 8); i += blockDim.x) {
      const int rr = i / (D / 8), q = i % (D / 8);
      const int r = r0 + rr;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (r < n) {
        const long long src = rows ? rows[r] : r;
        v = *reinterpret_cast<const uint4*>(X + src * D + q * 8);
      }
      *reinterpret_cast<uint4*>(sa + (size_t)rr * KP + q * 8) = v;
    }
    __syncthreads();
    int in = 0;
    const int wr = warp * 16;   // this warp's 16 rows
    for (int l = 0; l < 3; l++) {
      const __nv_bfloat16* W = sw + (size_t)l * D * KP;
      const __nv_bfloat16* A = sa + (size_t)in * TILE * KP;
      __nv_bfloat16* O = sa + (size_t)(in ^ 1) * TILE * KP;
      float acc[16][4];
#pragma unroll
      for (int j = 0; j < 16; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
#pragma unroll
      for (int kk = 0; kk < D / 16; kk++) {
        const int k0 = kk * 16 + c * 2;
        const unsigned a0 = ld_b32(A + (size_t)(wr + g) * KP + k0);
        const unsigned a1 = ld_b32(A + (size_t)(wr + g + 8) * KP + k0);
        const unsigned a2 = ld_b32(A + (size_t)(wr + g) * KP + k0 + 8);
        const unsigned a3 = ld_b32(A + (size_t)(wr + g + 8) * KP + k0 + 8);
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const unsigned b0 = ld_b32(W + (size_t)(j * 8 + g) * KP + k0);
          const unsigned b1 = ld_b32(W + (size_t)(j * 8 + g) * KP + k0 + 8);
          mma_bf16(acc[j], a0, a1, a2, a3, b0, b1);
        }
      }
#pragma unroll
      for (int j = 0; j < 16; j++) {
#pragma unroll
        for (int h = 0; h < 2; h++) {          // rows g and g + 8
          const int rr = wr + g + 8 * h;
          const int r = r0 + rr;
          const int col = j * 8 + c * 2;
          const float z0 = acc[j][2 * h] + sb[l * D + col];
          const float z1 = acc[j][2 * h + 1] + sb[l * D + col + 1];
          const __nv_bfloat162 hv = __floats2bfloat162_rn(gelu(z0), gelu(z1));
          *reinterpret_cast<__nv_bfloat162*>(O + (size_t)rr * KP + col) = hv;
          if (STORE && r < n) {
            *reinterpret_cast<float2*>(Z + ((size_t)l * n + r) * D + col) = make_float2(z0, z1);
            *reinterpret_cast<__nv_bfloat162*>(H + ((size_t)l * n + r) * D + col) = hv;
          }
        }
      }
      __syncwarp();
      in ^= 1;
    }
    // output layer: one n-tile of 8 columns (rows 3..7 of W4 are zero)
    {
      const __nv_bfloat16* W = sw + (size_t)3 * D * KP;
      const __nv_bfloat16* A = sa + (size_t)in * TILE * KP;
      float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int kk = 0; kk < D / 16; kk++) {
        const int k0 = kk * 16 + c * 2;
        mma_bf16(acc, ld_b32(A + (size_t)(wr + g) * KP + k0), ld_b32(A + (size_t)(wr + g + 8) * KP + k0),
                 ld_b32(A + (size_t)(wr + g) * KP + k0 + 8), ld_b32(A + (size_t)(wr + g + 8) * KP + k0 + 8),
                 ld_b32(W + (size_t)g * KP + k0), ld_b32(W + (size_t)g * KP + k0 + 8));
      }
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int r = r0 + wr + g + 8 * h;
        const int col = c * 2;
        if (r < n) {
          if (col < NOUT) Y[(size_t)r * 4 + col] = acc[2 * h] + sb[3 * D + col];
          if (col + 1 < NOUT) Y[(size_t)r * 4 + col + 1] = acc[2 * h + 1] + sb[3 * D + col + 1];
          if (col == 2) Y[(size_t)r * 4 + 3] = 0.0f;
        }
      }
    }
    __syncthreads();
  }
}

// ---- backward ---------------------------------------------------------------
// dY = 2 (Y - T) m / count; block partial sums of the loss
__global__ void k_out_grad(int n, const int* __restrict__ rows, const float* __restrict__ Y,
                           const float* __restrict__ T, const float* __restrict__ M, float inv_cnt,
                           float* __restrict__ dY, double* __restrict__ lpart) {
  __shared__ double sh[256];
  double l = 0.0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const long long s = rows ? rows[r] : r;
    const float m = M[s];
    for (int j = 0; j < 4; j++) {
      float d = 0.0f;
      if (j < NOUT) {
        const float e = Y[(size_t)r * 4 + j] - T[s * 4 + j];
        d = 2.0f * e * m * inv_cnt;
        l += (double)e * e * m;
      }
      dY[(size_t)r * 4 + j] = d;
    }
  }
  sh[threadIdx.x] = l;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) lpart[blockIdx.x] = sh[0];
}

// dZ_prev[r][k] = (sum_j dZ[r][j] W[j][k]) * gelu'(Zprev[r][k]); W = the bf16
// weights (dout rows of 128), staged in shared memory
template <int DOUT>
__global__ void __launch_bounds__(128) k_back(int n, const float* __restrict__ dZ, int dz_stride,
                                               const __nv_bfloat16* __restrict__ Wb,
                                               const float* __restrict__ Zprev, float* __restrict__ dZprev) {
  __shared__ __nv_bfloat16 sw[DOUT * D];
  __shared__ float sd[8][DOUT];
  for (int i = threadIdx.x; i < DOUT * D; i += blockDim.x) sw[i] = Wb[i];
  __syncthreads();
  const int k = threadIdx.x;
  for (int r0 = blockIdx.x * 8; r0 < n; r0 += gridDim.x * 8) {
    for (int i = threadIdx.x; i < 8 * DOUT; i += blockDim.x) {
      const int rr = i / DOUT, j = i % DOUT;
      sd[rr][j] = (r0 + rr < n) ? dZ[(size_t)(r0 + rr) * dz_stride + j] : 0.0f;
    }
    __syncthreads();
    for (int rr = 0; rr < 8; rr++) {
      const int r = r0 + rr;
      if (r >= n) break;
      float s = 0.0f;
#pragma unroll 8
      for (int j = 0; j < DOUT; j++) s += sd[rr][j] * __bfloat162float(sw[j * D + k]);
      dZprev[(size_t)r * D + k] = s * gelu_grad(Zprev[(size_t)r * D + k]);
    }
    __syncthreads();
  }
}

// weight gradient partials: part[b][j*128 + k] = sum over the block's rows of
// dZ[r][j] * Hin[r][k]; part[b][DOUT*128 + j] = sum dZ[r][j].  Hin rows are
// gathered through `rows` when given (the network input of a shuffled batch).
template <int DOUT>
__global__ void __launch_bounds__(256) k_wgrad(int n, const float* __restrict__ dZ, int dz_stride,
                                                const __nv_bfloat16* __restrict__ Hin, const int* __restrict__ rows,
                                                int rows_per_block, float* __restrict__ part) {
  constexpr int NACC = (DOUT * D + 255) / 256;
  __shared__ float sd[32][DOUT];
  __shared__ float sh[32][D];
  float acc[NACC];
#pragma unroll
  for (int q = 0; q < NACC; q++) acc[q] = 0.0f;
  float bacc = 0.0f;
  const int rb = blockIdx.x * rows_per_block, re = min(n, rb + rows_per_block);
  for (int r0 = rb; r0 < re; r0 += 32) {
    const int cnt = min(32, re - r0);
    for (int i = threadIdx.x; i < 32 * DOUT; i += blockDim.x) {
      const int rr = i / DOUT, j = i % DOUT;
      sd[rr][j] = rr < cnt ? dZ[(size_t)(r0 + rr) * dz_stride + j] : 0.0f;
    }
    for (int i = threadIdx.x; i < 32 * D; i += blockDim.x) {
      const int rr = i / D, k = i % D;
      float v = 0.0f;
      if (rr < cnt) {
        const long long src = rows ? rows[r0 + rr] : (r0 + rr);
        v = __bfloat162float(Hin[src * D + k]);
      }
      sh[rr][k] = v;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NACC; q++) {
      const int idx = threadIdx.x + 256 * q;
      if (idx < DOUT * D) {
        const int j = idx / D, k = idx % D;
        float s = acc[q];
        for (int rr = 0; rr < cnt; rr++) s += sd[rr][j] * sh[rr][k];
        acc[q] = s;
      }
    }
    if (threadIdx.x < DOUT)
      for (int rr = 0; rr < cnt; rr++) bacc += sd[rr][threadIdx.x];
    __syncthreads();
  }
  float* out = part + (size_t)blockIdx.x * (DOUT * D + DOUT);
#pragma unroll
  for (int q = 0; q < NACC; q++) {
    const int idx = threadIdx.x + 256 * q;
    if (idx < DOUT * D) out[idx] = acc[q];
  }
  if (threadIdx.x < DOUT) out[DOUT * D + threadIdx.x] = bacc;
}

// ---- backward of the 128-wide layers on the tensor cores ----------------------
// The products take the upstream gradient dZ rounded to bf16 (the weights and
// activations already are), accumulate in fp32: mma.sync m16n8k16, A row-major
// 16x16, B col-major 16x8.  Operands are staged transposed in shared memory
// with padded rows, so every fragment is one 32-bit load without bank conflicts.

// weight gradient partials of a 128x128 layer: part[b][j*128 + k] = sum over the
// block's rows of dZ[r][j] * Hin[r][k]; part[b][128*128 + j] = sum dZ[r][j] (fp32).
// 8 warps, warp w owns output rows j = 16w..16w+15, all 128 columns.
__global__ void __launch_bounds__(256) k_wgrad_tc(int n, const float* __restrict__ dZ, int dz_stride,
                                                   const __nv_bfloat16* __restrict__ Hin, const int* __restrict__ rows,
                                                   int rows_per_block, float* __restrict__ part) {
  constexpr int RP = 40;                   // 32 rows of a chunk + 8 pad (80-byte rows)
  __shared__ __nv_bfloat16 sdT[D][RP];     // dZ^T of the chunk: [j][r]
  __shared__ __nv_bfloat16 shT[D][RP];     // Hin^T of the chunk: [k][r]
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, g = lane >> 2, c = lane & 3;
  float acc[16][4];
#pragma unroll
  for (int t = 0; t < 16; t++) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.0f;
  float bacc = 0.0f;
  const int rb = blockIdx.x * rows_per_block, re = min(n, rb + rows_per_block);
  for (int r0 = rb; r0 < re; r0 += 32) {
    const int cnt = min(32, re - r0);
    for (int i = threadIdx.x; i < 32 * D; i += blockDim.x) {
      const int rr = i / D, j = i % D;
      float v = 0.0f;
      __nv_bfloat16 h = __float2bfloat16_rn(0.0f);
      if (rr < cnt) {
        v = dZ[(size_t)(r0 + rr) * dz_stride + j];
        const long long src = rows ? rows[r0 + rr] : (r0 + rr);
        h = Hin[src * D + j];
      }
      sdT[j][rr] = __float2bfloat16_rn(v);
      shT[j][rr] = h;
    }
    if (threadIdx.x < D)
      for (int rr = 0; rr < cnt; rr++) bacc += dZ[(size_t)(r0 + rr) * dz_stride + threadIdx.x];
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < 2; ks++) {
      const int kc = 16 * ks + 2 * c;
      const unsigned a0 = ld_b32(&sdT[16 * w + g][kc]), a1 = ld_b32(&sdT[16 * w + g + 8][kc]);
      const unsigned a2 = ld_b32(&sdT[16 * w + g][kc + 8]), a3 = ld_b32(&sdT[16 * w + g + 8][kc + 8]);
#pragma unroll
      for (int t = 0; t < 16; t++) {
        const unsigned b0 = ld_b32(&shT[8 * t + g][kc]), b1 = ld_b32(&shT[8 * t + g][kc + 8]);
        mma_bf16(acc[t], a0, a1, a2, a3, b0, b1);
      }
    }
    __syncthreads();
  }
  float* out = part + (size_t)blockIdx.x * (D * D + D);
#pragma unroll
  for (int t = 0; t < 16; t++) {
    const int j0 = 16 * w + g, k0 = 8 * t + 2 * c;
    out[(size_t)j0 * D + k0] = acc[t][0];
    out[(size_t)j0 * D + k0 + 1] = acc[t][1];
    out[(size_t)(j0 + 8) * D + k0] = acc[t][2];
    out[(size_t)(j0 + 8) * D + k0 + 1] = acc[t][3];
  }
  if (threadIdx.x < D) out[D * D + threadIdx.x] = bacc;
}

// dZprev[r][k] = (sum_j dZ[r][j] W[j][k]) * gelu'(Zprev[r][k]) for a 128x128 layer;
// W^T staged once per block, 32-row tiles of dZ; warp w: rows 16(w%2).., columns 32(w/2)..
__global__ void __launch_bounds__(256) k_back_tc(int n, const float* __restrict__ dZ, int dz_stride,
                                                  const __nv_bfloat16* __restrict__ Wb,
                                                  const float* __restrict__ Zprev, float* __restrict__ dZprev) {
  __shared__ __nv_bfloat16 swT[D][KP];     // W^T: [k][j]
  __shared__ __nv_bfloat16 sa[32][KP];     // dZ rows of the tile: [r][j]
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, g = lane >> 2, c = lane & 3;
  for (int i = threadIdx.x; i < D * D; i += blockDim.x) swT[i % D][i / D] = Wb[i];
  const int mt = w & 1, nq = w >> 1;
  for (int r0 = blockIdx.x * 32; r0 < n; r0 += gridDim.x * 32) {
    for (int i = threadIdx.x; i < 32 * D; i += blockDim.x) {
      const int rr = i / D, j = i % D;
      sa[rr][j] = __float2bfloat16_rn(r0 + rr < n ? dZ[(size_t)(r0 + rr) * dz_stride + j] : 0.0f);
    }
    __syncthreads();
    float acc[4][4];
#pragma unroll
    for (int t = 0; t < 4; t++) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.0f;
#pragma unroll
    for (int ks = 0; ks < D / 16; ks++) {
      const int kc = 16 * ks + 2 * c;
      const unsigned a0 = ld_b32(&sa[16 * mt + g][kc]), a1 = ld_b32(&sa[16 * mt + g + 8][kc]);
      const unsigned a2 = ld_b32(&sa[16 * mt + g][kc + 8]), a3 = ld_b32(&sa[16 * mt + g + 8][kc + 8]);
#pragma unroll
      for (int t = 0; t < 4; t++) {
        const int n0 = 32 * nq + 8 * t;
        const unsigned b0 = ld_b32(&swT[n0 + g][kc]), b1 = ld_b32(&swT[n0 + g][kc + 8]);
        mma_bf16(acc[t], a0, a1, a2, a3, b0, b1);
      }
    }
#pragma unroll
    for (int t = 0; t < 4; t++) {
      const int k = 32 * nq + 8 * t + 2 * c;
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int r = r0 + 16 * mt + g + 8 * h;
        if (r < n) {
          const size_t o = (size_t)r * D + k;
          dZprev[o] = acc[t][2 * h] * gelu_grad(Zprev[o]);
          dZprev[o + 1] = acc[t][2 * h + 1] * gelu_grad(Zprev[o + 1]);
        }
      }
    }
    __syncthreads();
  }
}

// g[w_off + i] = sum_b part[b][i] (i < dout*128), g[b_off + j] = sum_b part[b][doutp*128 + j];
// a part row holds doutp >= dout output rows (the padded output layer)
__global__ void k_reduce_parts(int nb, int dout, int doutp, const float* __restrict__ part, float* __restrict__ g,
                               int w_off, int b_off) {
  const int stride = doutp * D + doutp;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < dout * D + dout; i += gridDim.x * blockDim.x) {
    const int src = i < dout * D ? i : doutp * D + (i - dout * D);
    float s = 0.0f;
    for (int b = 0; b < nb; b++) s += part[(size_t)b * stride + src];
    if (i < dout * D)
      g[w_off + i] = s;
    else
      g[b_off + i - dout * D] = s;
  }
}

__global__ void k_adam(int np, float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M1,
                       float* __restrict__ M2, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const float g = G[i];
    const float m = b1 * M1[i] + (1.0f - b1) * g;
    const float v = b2 * M2[i] + (1.0f - b2) * g * g;
    M1[i] = m;
    M2[i] = v;
    P[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
  }
}

// bf16 weight copies: W1, W2, W3 (128 x 128) and W4 padded to 8 rows
__global__ void k_to_bf16(const float* __restrict__ P, __nv_bfloat16* __restrict__ Wb) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < WB_TOTAL; i += gridDim.x * blockDim.x) {
    float v = 0.0f;
    if (i < WB_LAYER) v = P[OFF_W1 + i];
    else if (i < 2 * WB_LAYER) v = P[OFF_W2 + i - WB_LAYER];
    else if (i < 3 * WB_LAYER) v = P[OFF_W3 + i - 2 * WB_LAYER];
    else if (i - 3 * WB_LAYER < NOUT * D) v = P[OFF_W4 + i - 3 * WB_LAYER];
    Wb[i] = __float2bfloat16_rn(v);
  }
}

// the base of a prediction: 2 L1 - L2 where the node was wet at both levels, else L1
__host__ __device__ inline double extrapolate(double l1, double l2, bool wet2) { return wet2 ? 2.0 * l1 - l2 : l1; }

// targets and mask of appended samples; st: U1 V1 S1 U2 V2 S2 U0 V0 S0 (9 x np);
// target = (L0 - base) / output scale
__global__ void k_targets(int n, const int* __restrict__ nodes, const double* __restrict__ st, int np,
                          const int* __restrict__ wet2, float osU, float osV, float osS, float* __restrict__ T,
                          float* __restrict__ M) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const int nd = nodes[r];
    const bool w2 = wet2[nd] != 0;
    const float os[3] = {osU, osV, osS};
    for (int j = 0; j < 3; j++) {
      const double l1 = st[(size_t)j * np + nd], l2 = st[(size_t)(3 + j) * np + nd];
      const double l0 = st[(size_t)(6 + j) * np + nd];
      T[(size_t)r * 4 + j] = (float)((l0 - extrapolate(l1, l2, w2)) / os[j]);
    }
    T[(size_t)r * 4 + 3] = 0.0f;
    M[r] = 1.0f;
  }
}

}  // namespace

struct rg_mlp {
  int device = 0;
  cudaStream_t st = nullptr;
  std::string err;
  int num_sms = 1;
  int np = 0;
  DBuf<int> stencil;
  DBuf<float> dist;
  DBuf<double> zb;
  float in_ref[3] = {4.0f, 1.0f, 1.0f};
  float step_scale[3] = {0.01f, 0.01f, 0.001f};
  float out_scale[3] = {0.002f, 0.002f, 0.0002f};
  DBuf<float> P, G, M1, M2;
  DBuf<__nv_bfloat16> Wb;
  int adam_t = 0;
  // training set
  DBuf<__nv_bfloat16> X;
  DBuf<float> T, Mk;
  long long nsamp = 0;
  // scratch
  DBuf<double> sstate;
  DBuf<int> snodes, srows, swet;
  DBuf<__nv_bfloat16> sX, sH;
  DBuf<float> sY, sZ, sdY, sdA, sdB, spart, sT, sM;
  DBuf<double> slp;
};

namespace {

rg_status mfail(rg_mlp* m, rg_status s, const std::string& msg) {
  if (m) m->err = msg;
  return s;
}

#define MTRY(expr)                                                                                            \
  do {                                                                                                        \
    cudaError_t _e = (expr);                                                                                  \
    if (_e != cudaSuccess) return mfail(m, RG_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

int grid_of(rg_mlp* m, long long work, int block) {
  long long g = (work + block - 1) / block;
  g = std::min<long long>(g, (long long)m->num_sms * 8);
  return (int)std::max<long long>(g, 1);
}

template <class T>
cudaError_t ensure(DBuf<T>& b, size_t n) {
  if (b.n >= n && b.p) return cudaSuccess;
  return b.alloc(n);
}

cudaError_t refresh_bf16(rg_mlp* m) {
  k_to_bf16<<<grid_of(m, WB_TOTAL, 256), 256, 0, m->st>>>(m->P.p, m->Wb.p);
  return cudaGetLastError();
}

cudaError_t forward(rg_mlp* m, int n, const int* rows, const __nv_bfloat16* X, float* Y, bool store) {
  // the shared-memory attribute is a property of the device: set it once per device
  static bool attr[kMaxDevices] = {false};
  if (m->device < 0 || m->device >= kMaxDevices) return cudaErrorInvalidDevice;
  if (!attr[m->device]) {
    cudaError_t e = cudaFuncSetAttribute(k_forward<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FWD_SMEM);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_forward<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FWD_SMEM);
    if (e != cudaSuccess) return e;
    attr[m->device] = true;
  }
  const int ntiles = (n + TILE - 1) / TILE;
  const int grid = std::max(1, std::min(ntiles, m->num_sms));
  if (store)
    k_forward<true><<<grid, 128, FWD_SMEM, m->st>>>(n, rows, X, m->Wb.p, m->P.p, Y, m->sZ.p, m->sH.p);
  else
    k_forward<false><<<grid, 128, FWD_SMEM, m->st>>>(n, rows, X, m->Wb.p, m->P.p, Y, nullptr, nullptr);
  return cudaGetLastError();
}

// gradient of the masked mean squared error of one batch into m->G (the
// forward pass with stored activations must have run on the same rows)
rg_status backward(rg_mlp* m, int n, const int* rows, const __nv_bfloat16* X, const float* T, const float* M,
                   float inv_cnt, double* loss_sum) {
  const int gb = grid_of(m, n, 256);
  MTRY(ensure(m->sdY, (size_t)n * 4));
  MTRY(ensure(m->sdA, (size_t)n * D));
  MTRY(ensure(m->sdB, (size_t)n * D));
  MTRY(ensure(m->slp, (size_t)gb));
  k_out_grad<<<gb, 256, 0, m->st>>>(n, rows, m->sY.p, T, M, inv_cnt, m->sdY.p, m->slp.p);
  const int rpb = 512;
  const int nbw = (n + rpb - 1) / rpb;
  MTRY(ensure(m->spart, (size_t)nbw * (D * D + D)));
  const float* Z = m->sZ.p;
  const __nv_bfloat16* H = m->sH.p;
  // output layer: dW4 from h3 (part rows padded to 4), dZ3 through W4
  k_wgrad<4><<<nbw, 256, 0, m->st>>>(n, m->sdY.p, 4, H + (size_t)2 * n * D, nullptr, rpb, m->spart.p);
  k_reduce_parts<<<4, 256, 0, m->st>>>(nbw, NOUT, 4, m->spart.p, m->G.p, OFF_W4, OFF_B4);
  const int gbk = grid_of(m, (long long)n, 8);
  k_back<4><<<gbk, 128, 0, m->st>>>(n, m->sdY.p, 4, m->Wb.p + 3 * WB_LAYER, Z + (size_t)2 * n * D, m->sdA.p);
  const int gbt = std::min((n + 31) / 32, m->num_sms * 4);
  // hidden layers 3, 2: dW_l from h_{l-1}, dZ_{l-1} through W_l
  float* dz = m->sdA.p;
  float* dzn = m->sdB.p;
  for (int l = 3; l >= 2; l--) {
    k_wgrad_tc<<<nbw, 256, 0, m->st>>>(n, dz, D, H + (size_t)(l - 2) * n * D, nullptr, rpb, m->spart.p);
    const int woff = l == 3 ? OFF_W3 : OFF_W2, boff = l == 3 ? OFF_B3 : OFF_B2;
    k_reduce_parts<<<64, 256, 0, m->st>>>(nbw, D, D, m->spart.p, m->G.p, woff, boff);
    k_back_tc<<<gbt, 256, 0, m->st>>>(n, dz, D, m->Wb.p + (size_t)(l - 1) * WB_LAYER, Z + (size_t)(l - 2) * n * D,
                                      dzn);
    std::swap(dz, dzn);
  }
  // first layer: dW1 from the network input
  k_wgrad_tc<<<nbw, 256, 0, m->st>>>(n, dz, D, X, rows, rpb, m->spart.p);
  k_reduce_parts<<<64, 256, 0, m->st>>>(nbw, D, D, m->spart.p, m->G.p, OFF_W1, OFF_B1);
  MTRY(cudaGetLastError());
  if (loss_sum) {
    std::vector<double> lp(gb);
    MTRY(cudaMemcpyAsync(lp.data(), m->slp.p, gb * sizeof(double), cudaMemcpyDeviceToHost, m->st));
    MTRY(cudaStreamSynchronize(m->st));
    double s = 0;
    for (double v : lp) s += v;
    *loss_sum = s;
  }
  return RG_OK;
}

// features of `n` nodes into m->sX from host state arrays (levels 1, 2[, 0])
rg_status build_features(rg_mlp* m, int n, const int* nodes, const double* const* lv, int nlev, double qn,
                         double qp) {
  const int np = m->np;
  MTRY(ensure(m->sstate, (size_t)9 * np));
  MTRY(ensure(m->snodes, (size_t)std::max(n, 1)));
  MTRY(ensure(m->sX, (size_t)std::max(n, 1) * D));
  for (int i = 0; i < nlev; i++)
    MTRY(cudaMemcpyAsync(m->sstate.p + (size_t)i * np, lv[i], np * sizeof(double), cudaMemcpyHostToDevice, m->st));
  if (n > 0) {
    MTRY(cudaMemcpyAsync(m->snodes.p, nodes, n * sizeof(int), cudaMemcpyHostToDevice, m->st));
    k_features<<<grid_of(m, (long long)n * D, 256), 256, 0, m->st>>>(
        n, m->snodes.p, m->stencil.p, m->dist.p, m->zb.p, m->sstate.p, np, m->in_ref[0], m->in_ref[1], m->in_ref[2],
        m->step_scale[0], m->step_scale[1], m->step_scale[2], (float)qn, (float)qp, m->sX.p);
    MTRY(cudaGetLastError());
  }
  return RG_OK;
}

}  // namespace

extern "C" {

rg_status rg_mlp_create(int device, unsigned seed, rg_mlp** out) {
  if (!out) return RG_ERR_ARG;
  *out = nullptr;
  rg_mlp* m = new rg_mlp();
  if (device < 0) cudaGetDevice(&device);
  m->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = m->P.alloc(NPARAM);
  if (e == cudaSuccess) e = m->G.alloc(NPARAM);
  if (e == cudaSuccess) e = m->M1.alloc(NPARAM);
  if (e == cudaSuccess) e = m->M2.alloc(NPARAM);
  if (e == cudaSuccess) e = m->Wb.alloc(WB_TOTAL);
  if (e != cudaSuccess) {
    delete m;
    return RG_ERR_CUDA;
  }
  // seeded uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases, small output layer
  std::vector<float> p(NPARAM, 0.0f);
  std::mt19937 rng(seed);
  std::uniform_real_distribution<float> u(-1.0f, 1.0f);
  const float s = 1.0f / std::sqrt((float)D);
  for (int i = 0; i < D * D; i++) p[OFF_W1 + i] = u(rng) * s;
  for (int i = 0; i < D * D; i++) p[OFF_W2 + i] = u(rng) * s;
  for (int i = 0; i < D * D; i++) p[OFF_W3 + i] = u(rng) * s;
  for (int i = 0; i < NOUT * D; i++) p[OFF_W4 + i] = u(rng) * s * 0.1f;
  *out = m;
  return rg_mlp_set_params(m, p.data());
}

rg_status rg_mlp_destroy(rg_mlp* m) {
  if (!m) return RG_OK;
  cudaSetDevice(m->device);
  if (m->st) cudaStreamSynchronize(m->st);
  if (m->st) cudaStreamDestroy(m->st);
  delete m;
  return RG_OK;
}

const char* rg_mlp_last_error(rg_mlp* m) { return m ? m->err.c_str() : "null network"; }

rg_status rg_mlp_set_params(rg_mlp* m, const float* params) {
  if (!m || !params) return RG_ERR_ARG;
  MTRY(cudaSetDevice(m->device));
  MTRY(cudaMemcpyAsync(m->P.p, params, NPARAM * sizeof(float), cudaMemcpyHostToDevice, m->st));
  MTRY(cudaMemsetAsync(m->M1.p, 0, NPARAM * sizeof(float), m->st));
  MTRY(cudaMemsetAsync(m->M2.p, 0, NPARAM * sizeof(float), m->st));
  m->adam_t = 0;
  MTRY(refresh_bf16(m));
  MTRY(cudaStreamSynchronize(m->st));
  return RG_OK;
}

rg_status rg_mlp_get_params(rg_mlp* m, float* params) {
  if (!m || !params) return RG_ERR_ARG;
  MTRY(cudaSetDevice(m->device));
  MTRY(cudaMemcpyAsync(params, m->P.p, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, m->st));
  MTRY(cudaStreamSynchronize(m->st));
  return RG_OK;
}

rg_status rg_mlp_set_scales(rg_mlp* m, const float* in_ref3, const float* step_scale3, const float* out_scale3) {
  if (!m) return RG_ERR_ARG;
  for (int i = 0; i < 3; i++) {
    const float a = in_ref3 ? in_ref3[i] : m->in_ref[i];
    const float b = step_scale3 ? step_scale3[i] : m->step_scale[i];
    const float c = out_scale3 ? out_scale3[i] : m->out_scale[i];
    if (!(a > 0.0f) || !(b > 0.0f) || !(c > 0.0f)) return mfail(m, RG_ERR_ARG, "scales must be positive");
  }
  for (int i = 0; i < 3; i++) {
    if (in_ref3) m->in_ref[i] = in_ref3[i];
    if (step_scale3) m->step_scale[i] = step_scale3[i];
    if (out_scale3) m->out_scale[i] = out_scale3[i];
  }
  return RG_OK;
}

rg_status rg_mlp_set_mesh(rg_mlp* m, int np, const double* x, const double* y, const double* z, int ne,
                          const int* en) {
  if (!m || np <= 0 || !x || !y || !z || ne < 0 || (ne > 0 && !en)) return RG_ERR_ARG;
  // one-ring neighbours: nodes sharing a triangle
  std::vector<std::vector<int>> nb(np);
  for (int e = 0; e < ne; e++)
    for (int i = 0; i < 6; i++) {
      const int a = en[6 * e + i];
      if (a < 0 || a >= np) return mfail(m, RG_ERR_ARG, "rg_mlp_set_mesh: node index out of range");
      for (int j = 0; j < 6; j++)
        if (j != i) nb[a].push_back(en[6 * e + j]);
    }
  std::vector<int> sten((size_t)np * K, -1);
  std::vector<float> dist((size_t)np * K, 0.0f);
  for (int n = 0; n < np; n++) {
    std::vector<int>& v = nb[n];
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    auto d2 = [&](int a) { return (x[a] - x[n]) * (x[a] - x[n]) + (y[a] - y[n]) * (y[a] - y[n]); };
    std::stable_sort(v.begin(), v.end(), [&](int a, int b) { return d2(a) < d2(b); });
    if ((int)v.size() > K - 1) v.resize(K - 1);
    std::stable_sort(v.begin(), v.end(), [&](int a, int b) {
      return std::atan2(y[a] - y[n], x[a] - x[n]) < std::atan2(y[b] - y[n], x[b] - x[n]);
    });
    double dmax = 0.0;
    for (int a : v) dmax = std::max(dmax, std::sqrt(d2(a)));
    sten[(size_t)n * K] = n;
    for (size_t s = 0; s < v.size(); s++) {
      sten[(size_t)n * K + 1 + s] = v[s];
      dist[(size_t)n * K + 1 + s] = dmax > 0.0 ? (float)(std::sqrt(d2(v[s])) / dmax) : 0.0f;
    }
  }
  MTRY(cudaSetDevice(m->device));
  MTRY(m->stencil.alloc(sten.size()));
  MTRY(m->dist.alloc(dist.size()));
  MTRY(m->zb.alloc(np));
  MTRY(cudaMemcpyAsync(m->stencil.p, sten.data(), sten.size() * sizeof(int), cudaMemcpyHostToDevice, m->st));
  MTRY(cudaMemcpyAsync(m->dist.p, dist.data(), dist.size() * sizeof(float), cudaMemcpyHostToDevice, m->st));
  MTRY(cudaMemcpyAsync(m->zb.p, z, np * sizeof(double), cudaMemcpyHostToDevice, m->st));
  MTRY(cudaStreamSynchronize(m->st));
  m->np = np;
  return RG_OK;
}

rg_status rg_mlp_features(rg_mlp* m, int n, const int* nodes, const double* U1, const double* V1, const double* S1,
                          const double* U2, const double* V2, const double* S2, double q_next, double q_prev,
                          float* X_out) {
  if (!m || m->np == 0 || n < 0 || !nodes || !X_out) return RG_ERR_ARG;
  for (int i = 0; i < n; i++)
    if (nodes[i] < 0 || nodes[i] >= m->np) return mfail(m, RG_ERR_ARG, "rg_mlp_features: node out of range");
  MTRY(cudaSetDevice(m->device));
  const double* lv[6] = {U1, V1, S1, U2, V2, S2};
  rg_status s = build_features(m, n, nodes, lv, 6, q_next, q_prev);
  if (s != RG_OK) return s;
  std::vector<__nv_bfloat16> h((size_t)n * D);
  MTRY(cudaMemcpyAsync(h.data(), m->sX.p, h.size() * 2, cudaMemcpyDeviceToHost, m->st));
  MTRY(cudaStreamSynchronize(m->st));
  for (size_t i = 0; i < h.size(); i++) X_out[i] = __bfloat162float(h[i]);
  return RG_OK;
}

rg_status rg_mlp_clear_samples(rg_mlp* m) {
  if (!m) return RG_ERR_ARG;
  m->nsamp = 0;
  return RG_OK;
}

rg_status rg_mlp_add_samples(rg_mlp* m, const double* U2, const double* V2, const double* S2, const double* U1,
                             const double* V1, const double* S1, const double* U0, const double* V0, const double* S0,
                             const int* wet2, const int* wet1, const int* wet0, double q_next, double q_prev,
                             long long* added) {
  if (!m || m->np == 0 || !U2 || !V2 || !S2 || !U1 || !V1 || !S1 || !U0 || !V0 || !S0 || !wet2 || !wet1 || !wet0)
    return RG_ERR_ARG;
  MTRY(cudaSetDevice(m->device));
  std::vector<int> nodes;
  for (int i = 0; i < m->np; i++)
    if (wet1[i] && wet0[i]) nodes.push_back(i);
  const int n = (int)nodes.size();
  const double* lv[9] = {U1, V1, S1, U2, V2, S2, U0, V0, S0};
  rg_status s = build_features(m, n, nodes.data(), lv, 9, q_next, q_prev);
  if (s != RG_OK) return s;
  const long long need = m->nsamp + n;
  if ((long long)m->X.n < need * D) {
    // grow by half again, keeping the samples so far
    const long long cap = std::max<long long>(need, (long long)(m->X.n / D) * 3 / 2);
    DBuf<__nv_bfloat16> X2;
    DBuf<float> T2, M2;
    MTRY(X2.alloc((size_t)cap * D));
    MTRY(T2.alloc((size_t)cap * 4));
    MTRY(M2.alloc((size_t)cap));
    if (m->nsamp > 0) {
      MTRY(cudaMemcpyAsync(X2.p, m->X.p, (size_t)m->nsamp * D * 2, cudaMemcpyDeviceToDevice, m->st));
      MTRY(cudaMemcpyAsync(T2.p, m->T.p, (size_t)m->nsamp * 16, cudaMemcpyDeviceToDevice, m->st));
      MTRY(cudaMemcpyAsync(M2.p, m->Mk.p, (size_t)m->nsamp * 4, cudaMemcpyDeviceToDevice, m->st));
    }
    MTRY(cudaStreamSynchronize(m->st));
    std::swap(m->X.p, X2.p);
    std::swap(m->X.n, X2.n);
    std::swap(m->T.p, T2.p);
    std::swap(m->T.n, T2.n);
    std::swap(m->Mk.p, M2.p);
    std::swap(m->Mk.n, M2.n);
  }
  if (n > 0) {
    MTRY(ensure(m->swet, (size_t)m->np));
    MTRY(cudaMemcpyAsync(m->swet.p, wet2, (size_t)m->np * sizeof(int), cudaMemcpyHostToDevice, m->st));
    MTRY(cudaMemcpyAsync(m->X.p + (size_t)m->nsamp * D, m->sX.p, (size_t)n * D * 2, cudaMemcpyDeviceToDevice, m->st));
    k_targets<<<grid_of(m, n, 256), 256, 0, m->st>>>(n, m->snodes.p, m->sstate.p, m->np, m->swet.p, m->out_scale[0],
                                                     m->out_scale[1], m->out_scale[2], m->T.p + (size_t)m->nsamp * 4,
                                                     m->Mk.p + m->nsamp);
    MTRY(cudaGetLastError());
  }
  MTRY(cudaStreamSynchronize(m->st));
  m->nsamp = need;
  if (added) *added = n;
  return RG_OK;
}

rg_status rg_mlp_train(rg_mlp* m, int epochs, int batch, float lr, unsigned seed, double* loss_out) {
  if (!m || epochs < 0 || batch <= 0 || !(lr > 0.0f)) return RG_ERR_ARG;
  if (m->nsamp == 0) return mfail(m, RG_ERR_ARG, "rg_mlp_train: no samples");
  MTRY(cudaSetDevice(m->device));
  const long long ns = m->nsamp;
  const int bmax = (int)std::min<long long>(batch, ns);
  MTRY(ensure(m->sY, (size_t)bmax * 4));
  MTRY(ensure(m->sZ, (size_t)3 * bmax * D));
  MTRY(ensure(m->sH, (size_t)3 * bmax * D));
  MTRY(ensure(m->srows, (size_t)ns));
  std::vector<int> perm(ns);
  std::mt19937 rng(seed);
  for (int ep = 0; ep < epochs; ep++) {
    for (long long i = 0; i < ns; i++) perm[i] = (int)i;
    std::shuffle(perm.begin(), perm.end(), rng);
    MTRY(cudaMemcpyAsync(m->srows.p, perm.data(), ns * sizeof(int), cudaMemcpyHostToDevice, m->st));
    double lsum = 0.0;
    for (long long b0 = 0; b0 < ns; b0 += bmax) {
      const int n = (int)std::min<long long>(bmax, ns - b0);
      const int* rows = m->srows.p + b0;
      MTRY(forward(m, n, rows, m->X.p, m->sY.p, true));
      double l = 0.0;
      rg_status s = backward(m, n, rows, m->X.p, m->T.p, m->Mk.p, 1.0f / (float)n, &l);
      if (s != RG_OK) return s;
      lsum += l;
      m->adam_t++;
      const float b1 = 0.9f, b2 = 0.999f;
      const float c1 = 1.0f - std::pow(b1, (float)m->adam_t), c2 = 1.0f - std::pow(b2, (float)m->adam_t);
      k_adam<<<grid_of(m, NPARAM, 256), 256, 0, m->st>>>(NPARAM, m->P.p, m->G.p, m->M1.p, m->M2.p, lr, b1, b2,
                                                         1e-8f, c1, c2);
      MTRY(refresh_bf16(m));
    }
    if (loss_out) loss_out[ep] = lsum / (double)ns;
  }
  MTRY(cudaStreamSynchronize(m->st));
  return RG_OK;
}

rg_status rg_mlp_loss_grad(rg_mlp* m, int n, const float* X, const float* T, const float* mask, double* loss,
                           float* y_out, float* grad_out) {
  if (!m || n <= 0 || !X || !T || !mask) return RG_ERR_ARG;
  MTRY(cudaSetDevice(m->device));
  std::vector<__nv_bfloat16> xb((size_t)n * D);
  for (size_t i = 0; i < xb.size(); i++) xb[i] = __float2bfloat16_rn(X[i]);
  std::vector<float> t4((size_t)n * 4, 0.0f);
  double cnt = 0.0;
  for (int r = 0; r < n; r++) {
    for (int j = 0; j < NOUT; j++) t4[(size_t)r * 4 + j] = T[(size_t)r * NOUT + j];
    cnt += mask[r];
  }
  MTRY(ensure(m->sX, (size_t)n * D));
  MTRY(ensure(m->sT, (size_t)n * 4));
  MTRY(ensure(m->sM, (size_t)n));
  MTRY(ensure(m->sY, (size_t)n * 4));
  MTRY(ensure(m->sZ, (size_t)3 * n * D));
  MTRY(ensure(m->sH, (size_t)3 * n * D));
  MTRY(cudaMemcpyAsync(m->sX.p, xb.data(), xb.size() * 2, cudaMemcpyHostToDevice, m->st));
  MTRY(cudaMemcpyAsync(m->sT.p, t4.data(), t4.size() * 4, cudaMemcpyHostToDevice, m->st));
  MTRY(cudaMemcpyAsync(m->sM.p, mask, (size_t)n * 4, cudaMemcpyHostToDevice, m->st));
  MTRY(forward(m, n, nullptr, m->sX.p, m->sY.p, true));
  double l = 0.0;
  rg_status s = backward(m, n, nullptr, m->sX.p, m->sT.p, m->sM.p, (float)(1.0 / std::max(cnt, 1.0)), &l);
  if (s != RG_OK) return s;
  if (loss) *loss = l / std::max(cnt, 1.0);
  if (y_out) {
    std::vector<float> y((size_t)n * 4);
    MTRY(cudaMemcpyAsync(y.data(), m->sY.p, y.size() * 4, cudaMemcpyDeviceToHost, m->st));
    MTRY(cudaStreamSynchronize(m->st));
    for (int r = 0; r < n; r++)
      for (int j = 0; j < NOUT; j++) y_out[(size_t)r * NOUT + j] = y[(size_t)r * 4 + j];
  }
  if (grad_out) {
    MTRY(cudaMemcpyAsync(grad_out, m->G.p, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, m->st));
    MTRY(cudaStreamSynchronize(m->st));
  }
  return RG_OK;
}

rg_status rg_mlp_predict(rg_mlp* m, const double* U2, const double* V2, const double* S2, const double* U1,
                         const double* V1, const double* S1, const int* wet2, const int* wet1, double q_next,
                         double q_prev, double* U_out, double* V_out, double* S_out) {
  if (!m || m->np == 0 || !U2 || !V2 || !S2 || !U1 || !V1 || !S1 || !wet2 || !wet1 || !U_out || !V_out || !S_out)
    return RG_ERR_ARG;
  MTRY(cudaSetDevice(m->device));
  const int np = m->np;
  std::vector<int> nodes;
  for (int i = 0; i < np; i++)
    if (wet1[i]) nodes.push_back(i);
  const int n = (int)nodes.size();
  const double* lv[6] = {U1, V1, S1, U2, V2, S2};
  rg_status s = build_features(m, n, nodes.data(), lv, 6, q_next, q_prev);
  if (s != RG_OK) return s;
  std::vector<float> y((size_t)n * 4);
  if (n > 0) {
    MTRY(ensure(m->sY, (size_t)n * 4));
    MTRY(forward(m, n, nullptr, m->sX.p, m->sY.p, false));
    MTRY(cudaMemcpyAsync(y.data(), m->sY.p, y.size() * 4, cudaMemcpyDeviceToHost, m->st));
  }
  MTRY(cudaStreamSynchronize(m->st));
  for (int i = 0; i < np; i++) {
    U_out[i] = U1[i];
    V_out[i] = V1[i];
    S_out[i] = S1[i];
  }
  for (int r = 0; r < n; r++) {
    const int nd = nodes[r];
    const bool w2 = wet2[nd] != 0;
    U_out[nd] = extrapolate(U1[nd], U2[nd], w2) + (double)y[(size_t)r * 4 + 0] * m->out_scale[0];
    V_out[nd] = extrapolate(V1[nd], V2[nd], w2) + (double)y[(size_t)r * 4 + 1] * m->out_scale[1];
    S_out[nd] = extrapolate(S1[nd], S2[nd], w2) + (double)y[(size_t)r * 4 + 2] * m->out_scale[2];
  }
  return RG_OK;
}

}  // extern "C"
