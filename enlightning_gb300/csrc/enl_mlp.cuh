// Learned hybrid sensor: features, BF16 tensor-core MLP (mma.sync m16n8k16,
// FP32 accumulation), used both inside the fused stage kernel (inference) and
// by the training kernels in enl_mlp.cu.
//
// Network: 40 inputs -> 64 -> 64 -> 1 logit, GELU (erf form) on the hidden
// layers; p(WENO needed) = sigmoid(logit).  Parameters live as one FP32
// vector (layout below); kernels stage BF16 copies in shared memory with the
// weight matrices stored transposed ([out][in]) so that B fragments are
// single 32-bit loads.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace enl {

constexpr int kFeat = 40;     // input features
constexpr int kFeatPad = 48;  // K padded to a multiple of 16
constexpr int kHid = 64;
// FP32 parameter vector layout
constexpr int kOffW1 = 0;                       // W1[k][n], k < 40, n < 64
constexpr int kOffB1 = kOffW1 + kFeat * kHid;   // 2560
constexpr int kOffW2 = kOffB1 + kHid;           // W2[k][n], 64 x 64
constexpr int kOffB2 = kOffW2 + kHid * kHid;
constexpr int kOffW3 = kOffB2 + kHid;           // w3[k]
constexpr int kOffB3 = kOffW3 + kHid;
constexpr int kNParams = kOffB3 + 1;            // 6849

// Shared-memory image of the network (BF16 transposed matrices + FP32 vectors).
struct MlpSmem {
  __nv_bfloat16 w1t[kHid][kFeatPad];  // [n][k], k >= 40 zero
  __nv_bfloat16 w2t[kHid][kHid];      // [n][k]
  float b1[kHid], b2[kHid], w3[kHid];
  float b3;
};

// The same image built on the host (the stage kernel reads it from global
// memory through L1: the network runs on few cells, and keeping it out of
// shared memory keeps four stage blocks per SM).
inline void mlp_build_image(const float* P, MlpSmem& S) {
  for (int n = 0; n < kHid; ++n)
    for (int k = 0; k < kFeatPad; ++k) S.w1t[n][k] = __float2bfloat16_rn(k < kFeat ? P[kOffW1 + k * kHid + n] : 0.0f);
  for (int n = 0; n < kHid; ++n)
    for (int k = 0; k < kHid; ++k) S.w2t[n][k] = __float2bfloat16_rn(P[kOffW2 + k * kHid + n]);
  for (int e = 0; e < kHid; ++e) {
    S.b1[e] = P[kOffB1 + e];
    S.b2[e] = P[kOffB2 + e];
    S.w3[e] = __bfloat162float(__float2bfloat16_rn(P[kOffW3 + e]));
  }
  S.b3 = P[kOffB3];
}

__device__ __forceinline__ void mlp_stage_params(MlpSmem& S, const float* __restrict__ P, int tid, int nthr) {
  for (int e = tid; e < kHid * kFeatPad; e += nthr) {
    int n = e / kFeatPad, k = e % kFeatPad;
    S.w1t[n][k] = __float2bfloat16_rn(k < kFeat ? P[kOffW1 + k * kHid + n] : 0.0f);
  }
  for (int e = tid; e < kHid * kHid; e += nthr) {
    int n = e / kHid, k = e % kHid;
    S.w2t[n][k] = __float2bfloat16_rn(P[kOffW2 + k * kHid + n]);
  }
  for (int e = tid; e < kHid; e += nthr) {
    S.b1[e] = P[kOffB1 + e];
    S.b2[e] = P[kOffB2 + e];
    S.w3[e] = __bfloat162float(__float2bfloat16_rn(P[kOffW3 + e]));
  }
  if (tid == 0) S.b3 = P[kOffB3];
}

__device__ __forceinline__ void mma_bf16(float d[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// erf by Abramowitz & Stegun, Handbook of Mathematical Functions, 7.1.26:
// erf(x) = 1 - (a1 t + a2 t^2 + a3 t^3 + a4 t^4 + a5 t^5) exp(-x^2),
// t = 1 / (1 + p x) for x >= 0, odd in x, |error| <= 1.5e-7 in exact
// arithmetic (below 1e-6 here, in FP32 with the hardware reciprocal and
// exponential) — far below the BF16 rounding that every activation goes
// through next, in fewer instructions than the library's erff (the network
// evaluates 128 per cell).
__device__ __forceinline__ float erf_as(float x) {
  const float ax = fabsf(x);
  float t;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(t) : "f"(fmaf(0.3275911f, ax, 1.0f)));
  const float poly =
      t * fmaf(t, fmaf(t, fmaf(t, fmaf(t, 1.061405429f, -1.453152027f), 1.421413741f), -0.284496736f), 0.254829592f);
  return copysignf(fmaf(-poly, __expf(-ax * ax), 1.0f), x);
}
__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erf_as(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  // d/dx [x Phi(x)] = Phi(x) + x phi(x)
  const float inv_sqrt_2pi = 0.39894228040143268f;
  return 0.5f * (1.0f + erf_as(x * 0.70710678118654752f)) + x * inv_sqrt_2pi * __expf(-0.5f * x * x);
}

// Forward pass of 16 rows (one m-tile) held by one warp.  X: BF16 rows of
// stride ldx (>= 40 elements, 4-byte aligned), columns >= 40 read as zero.
// Returns in z1/z2 the pre-activations (FP32, C-fragment layout) and the
// logits of rows g and g+8 (valid in lanes with t == 0).
struct MlpFwd16 {
  float z1[8][4];  // layer-1 pre-activations, n-tile x C fragment
  float z2[8][4];  // layer-2 pre-activations
  float logit[2];  // rows g, g+8
};

__device__ __forceinline__ void mlp_forward16(const MlpSmem& S, const __nv_bfloat16* X, int ldx, int lane,
                                              MlpFwd16& F) {
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int q = 0; q < 4; ++q) F.z1[n][q] = S.b1[n * 8 + 2 * t + (q & 1)];
#pragma unroll
  for (int kc = 0; kc < 3; ++kc) {
    int c0 = kc * 16 + 2 * t, c1 = c0 + 8;
    uint32_t a0 = c0 < kFeat ? ld_pair(X + g * ldx + c0) : 0u;
    uint32_t a1 = c0 < kFeat ? ld_pair(X + (g + 8) * ldx + c0) : 0u;
    uint32_t a2 = c1 < kFeat ? ld_pair(X + g * ldx + c1) : 0u;
    uint32_t a3 = c1 < kFeat ? ld_pair(X + (g + 8) * ldx + c1) : 0u;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      uint32_t b0 = ld_pair(&S.w1t[n * 8 + g][kc * 16 + 2 * t]);
      uint32_t b1 = ld_pair(&S.w1t[n * 8 + g][kc * 16 + 2 * t + 8]);
      mma_bf16(F.z1[n], a0, a1, a2, a3, b0, b1);
    }
  }
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int q = 0; q < 4; ++q) F.z2[n][q] = S.b2[n * 8 + 2 * t + (q & 1)];
#pragma unroll
  for (int kc = 0; kc < 4; ++kc) {
    // A fragment of the hidden layer straight from the C fragments of
    // n-tiles 2kc (columns 0-7 of the chunk) and 2kc+1 (columns 8-15)
    uint32_t a0 = pack_bf16(gelu(F.z1[2 * kc][0]), gelu(F.z1[2 * kc][1]));
    uint32_t a1 = pack_bf16(gelu(F.z1[2 * kc][2]), gelu(F.z1[2 * kc][3]));
    uint32_t a2 = pack_bf16(gelu(F.z1[2 * kc + 1][0]), gelu(F.z1[2 * kc + 1][1]));
    uint32_t a3 = pack_bf16(gelu(F.z1[2 * kc + 1][2]), gelu(F.z1[2 * kc + 1][3]));
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      uint32_t b0 = ld_pair(&S.w2t[n * 8 + g][kc * 16 + 2 * t]);
      uint32_t b1 = ld_pair(&S.w2t[n * 8 + g][kc * 16 + 2 * t + 8]);
      mma_bf16(F.z2[n], a0, a1, a2, a3, b0, b1);
    }
  }
  float s0 = 0.f, s1 = 0.f;
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    int col = n * 8 + 2 * t;
    // hidden activations enter the last layer rounded to BF16, like the
    // inputs of the two tensor-core layers
    s0 += __bfloat162float(__float2bfloat16_rn(gelu(F.z2[n][0]))) * S.w3[col] +
          __bfloat162float(__float2bfloat16_rn(gelu(F.z2[n][1]))) * S.w3[col + 1];
    s1 += __bfloat162float(__float2bfloat16_rn(gelu(F.z2[n][2]))) * S.w3[col] +
          __bfloat162float(__float2bfloat16_rn(gelu(F.z2[n][3]))) * S.w3[col + 1];
  }
  s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
  s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
  s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
  s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
  F.logit[0] = s0 + S.b3;
  F.logit[1] = s1 + S.b3;
}

// Inference only, with the same arithmetic as mlp_forward16 (the same
// accumulation orders, so the same logits) and fewer live registers: the
// hidden layer is packed into BF16 A fragments before the second layer, which
// then runs one n-tile at a time into the logit sums.
__device__ __forceinline__ void mlp_logits16(const MlpSmem& S, const __nv_bfloat16* X, int ldx, int lane,
                                             float logit[2]) {
  const int g = lane >> 2, t = lane & 3;
  uint32_t h[4][4];  // gelu(layer 1) as A fragments, k-chunks of 16
  {
    float z1[8][4];
#pragma unroll
    for (int n = 0; n < 8; ++n)
#pragma unroll
      for (int q = 0; q < 4; ++q) z1[n][q] = S.b1[n * 8 + 2 * t + (q & 1)];
#pragma unroll
    for (int kc = 0; kc < 3; ++kc) {
      int c0 = kc * 16 + 2 * t, c1 = c0 + 8;
      uint32_t a0 = c0 < kFeat ? ld_pair(X + g * ldx + c0) : 0u;
      uint32_t a1 = c0 < kFeat ? ld_pair(X + (g + 8) * ldx + c0) : 0u;
      uint32_t a2 = c1 < kFeat ? ld_pair(X + g * ldx + c1) : 0u;
      uint32_t a3 = c1 < kFeat ? ld_pair(X + (g + 8) * ldx + c1) : 0u;
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        uint32_t b0 = ld_pair(&S.w1t[n * 8 + g][kc * 16 + 2 * t]);
        uint32_t b1 = ld_pair(&S.w1t[n * 8 + g][kc * 16 + 2 * t + 8]);
        mma_bf16(z1[n], a0, a1, a2, a3, b0, b1);
      }
    }
#pragma unroll
    for (int kc = 0; kc < 4; ++kc) {
      h[kc][0] = pack_bf16(gelu(z1[2 * kc][0]), gelu(z1[2 * kc][1]));
      h[kc][1] = pack_bf16(gelu(z1[2 * kc][2]), gelu(z1[2 * kc][3]));
      h[kc][2] = pack_bf16(gelu(z1[2 * kc + 1][0]), gelu(z1[2 * kc + 1][1]));
      h[kc][3] = pack_bf16(gelu(z1[2 * kc + 1][2]), gelu(z1[2 * kc + 1][3]));
    }
  }
  float s0 = 0.f, s1 = 0.f;
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    float z2[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) z2[q] = S.b2[n * 8 + 2 * t + (q & 1)];
#pragma unroll
    for (int kc = 0; kc < 4; ++kc) {
      uint32_t b0 = ld_pair(&S.w2t[n * 8 + g][kc * 16 + 2 * t]);
      uint32_t b1 = ld_pair(&S.w2t[n * 8 + g][kc * 16 + 2 * t + 8]);
      mma_bf16(z2, h[kc][0], h[kc][1], h[kc][2], h[kc][3], b0, b1);
    }
    int col = n * 8 + 2 * t;
    s0 += __bfloat162float(__float2bfloat16_rn(gelu(z2[0]))) * S.w3[col] +
          __bfloat162float(__float2bfloat16_rn(gelu(z2[1]))) * S.w3[col + 1];
    s1 += __bfloat162float(__float2bfloat16_rn(gelu(z2[2]))) * S.w3[col] +
          __bfloat162float(__float2bfloat16_rn(gelu(z2[3]))) * S.w3[col + 1];
  }
  s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
  s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
  s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
  s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
  logit[0] = s0 + S.b3;
  logit[1] = s1 + S.b3;
}

// ------------------------------------------------------------------------
// Features of one cell (40 values) from an FP32 perturbation accessor:
// for each direction (x, y) and each stencil offset m = -2..2:
//   [0] the hybrid sensor ratio of rho at i+m  (2|ab|+e)/(a^2+b^2+e)
//   [1] the same ratio on p with e * c^4 (p' ~ c^2 rho')
//   [2] the WENO5 smoothness indicator beta1 of rho at i+m, as b/(b+e)
//   [3] log1p(|rho(m+1) - rho(m-1)| / sqrt(e)) / 4
// ------------------------------------------------------------------------
template <class ACC>
__device__ __forceinline__ void cell_features(const ACC& A, float eps, float eps_p, float inv_sqrt_eps,
                                              float out[kFeat]) {
#pragma unroll
  for (int dir = 0; dir < 2; ++dir) {
    float r[7], p[7];
#pragma unroll
    for (int q = 0; q < 7; ++q) {
      r[q] = dir == 0 ? A.w(0, q - 3, 0) : A.w(0, 0, q - 3);
      p[q] = dir == 0 ? A.p(q - 3, 0) : A.p(0, q - 3);
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      float a = r[m + 1] - r[m], b = r[m + 2] - r[m + 1];
      float ap = p[m + 1] - p[m], bp = p[m + 2] - p[m + 1];
      float rr = __fdividef(fmaf(2.0f, fabsf(a * b), eps), fmaf(a, a, fmaf(b, b, eps)));
      float rp = __fdividef(fmaf(2.0f, fabsf(ap * bp), eps_p), fmaf(ap, ap, fmaf(bp, bp, eps_p)));
      float d2 = (r[m] - 2.0f * r[m + 1]) + r[m + 2], d1 = r[m] - r[m + 2];
      float beta = (13.0f / 12.0f) * d2 * d2 + 0.25f * d1 * d1;
      const int o = dir * 20 + m * 4;
      out[o + 0] = rr;
      out[o + 1] = rp;
      out[o + 2] = __fdividef(beta, beta + eps);
      out[o + 3] = 0.25f * log1pf(fabsf(d1) * inv_sqrt_eps);
    }
  }
}

}  // namespace enl
