// Learned hybrid sensor: training-data harvest from the plain FP64 method,
// BF16 tensor-core forward/backward kernels (FP32 accumulation), Adam.
//
// The reference's hybrid switch (fortran/rhs_hybrid_high_llf.m4:239-256)
// sends a level-0 cell to WENO when any of six density-ratio tests falls
// below 0.9999.  The learned sensor predicts from 40 stencil features
// (enl_mlp.cuh) whether WENO is needed, trained on the plain switch and on
// the local difference between the DRP and WENO right-hand sides.
#include <cstring>
#include <cstdio>

#include "enl_mlp.cuh"
#include "enl_rhs_cell.cuh"

namespace enl {

// ---------------------------------------------------------------------------
// Training: one block of 4 warps handles chunks of 64 samples (16 per warp).
// ---------------------------------------------------------------------------
constexpr int kChunk = 64;

struct TrainSmem {
  MlpSmem S;
  __nv_bfloat16 w2[kHid][kHid];  // W2 [k][n] (B operand of dH1 = dZ2 W2^T)
  __nv_bfloat16 xs[kChunk][kFeatPad];
  __nv_bfloat16 h1[kChunk][kHid];
  __nv_bfloat16 h2[kChunk][kHid];
  __nv_bfloat16 dz1[kChunk][kHid];
  __nv_bfloat16 dz2[kChunk][kHid];
  float dl[kChunk];
};

__device__ __forceinline__ uint32_t pack_two(const __nv_bfloat16 lo, const __nv_bfloat16 hi) {
  __nv_bfloat162 v;
  v.x = lo;
  v.y = hi;
  return *reinterpret_cast<uint32_t*>(&v);
}

__global__ void __launch_bounds__(128) mlp_grad_kernel(const __nv_bfloat16* __restrict__ X,
                                                       const float* __restrict__ y, const float* __restrict__ wgt,
                                                       long N, const float* __restrict__ P, float* grad,
                                                       double* loss_sum) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  TrainSmem& T = *reinterpret_cast<TrainSmem*>(sm_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t = lane & 3;
  mlp_stage_params(T.S, P, tid, 128);
  for (int e = tid; e < kHid * kHid; e += 128) {
    int k = e / kHid, n = e % kHid;
    T.w2[k][n] = __float2bfloat16_rn(P[kOffW2 + k * kHid + n]);
  }
  // per-thread accumulators of the block's weight gradients
  float aw2[8][4], aw1[8][4];
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int q = 0; q < 4; ++q) aw2[n][q] = aw1[n][q] = 0.f;
  float ab1[2] = {0.f, 0.f}, ab2[2] = {0.f, 0.f}, aw3[2] = {0.f, 0.f}, ab3 = 0.f;
  double lsum = 0.0;
  __syncthreads();
  for (long c0 = (long)blockIdx.x * kChunk; c0 < N; c0 += (long)gridDim.x * kChunk) {
    for (int e = tid; e < kChunk * kFeatPad; e += 128) {
      int r = e / kFeatPad, k = e % kFeatPad;
      long s = c0 + r;
      T.xs[r][k] = (s < N && k < kFeat) ? X[s * kFeat + k] : __float2bfloat16_rn(0.0f);
    }
    __syncthreads();
    // forward, 16 rows per warp
    MlpFwd16 F;
    mlp_forward16(T.S, &T.xs[warp * 16][0], kFeatPad, lane, F);
    const int r0 = warp * 16 + g, r1 = r0 + 8;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      int col = n * 8 + 2 * t;
      T.h1[r0][col] = __float2bfloat16_rn(gelu(F.z1[n][0]));
      T.h1[r0][col + 1] = __float2bfloat16_rn(gelu(F.z1[n][1]));
      T.h1[r1][col] = __float2bfloat16_rn(gelu(F.z1[n][2]));
      T.h1[r1][col + 1] = __float2bfloat16_rn(gelu(F.z1[n][3]));
      T.h2[r0][col] = __float2bfloat16_rn(gelu(F.z2[n][0]));
      T.h2[r0][col + 1] = __float2bfloat16_rn(gelu(F.z2[n][1]));
      T.h2[r1][col] = __float2bfloat16_rn(gelu(F.z2[n][2]));
      T.h2[r1][col + 1] = __float2bfloat16_rn(gelu(F.z2[n][3]));
    }
    // BCE-with-logits gradient of rows r0, r1 (lanes t == 0 hold the logits)
    float dl0 = 0.f, dl1 = 0.f;
    if (t == 0) {
      long s0 = c0 + r0, s1 = c0 + r1;
      float z0 = F.logit[0], z1 = F.logit[1];
      if (s0 < N) {
        float w = wgt[s0], yy = y[s0];
        dl0 = w * (1.0f / (1.0f + __expf(-z0)) - yy);
        lsum += (double)(w * (fmaxf(z0, 0.f) - yy * z0 + log1pf(__expf(-fabsf(z0)))));
      }
      if (s1 < N) {
        float w = wgt[s1], yy = y[s1];
        dl1 = w * (1.0f / (1.0f + __expf(-z1)) - yy);
        lsum += (double)(w * (fmaxf(z1, 0.f) - yy * z1 + log1pf(__expf(-fabsf(z1)))));
      }
      T.dl[r0] = dl0;
      T.dl[r1] = dl1;
    }
    dl0 = __shfl_sync(0xffffffffu, dl0, lane & ~3);
    dl1 = __shfl_sync(0xffffffffu, dl1, lane & ~3);
    // dZ2 = (dl w3) * gelu'(z2), C-fragment layout
    float dz2[8][4];
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      int col = n * 8 + 2 * t;
      dz2[n][0] = dl0 * T.S.w3[col] * gelu_grad(F.z2[n][0]);
      dz2[n][1] = dl0 * T.S.w3[col + 1] * gelu_grad(F.z2[n][1]);
      dz2[n][2] = dl1 * T.S.w3[col] * gelu_grad(F.z2[n][2]);
      dz2[n][3] = dl1 * T.S.w3[col + 1] * gelu_grad(F.z2[n][3]);
      T.dz2[r0][col] = __float2bfloat16_rn(dz2[n][0]);
      T.dz2[r0][col + 1] = __float2bfloat16_rn(dz2[n][1]);
      T.dz2[r1][col] = __float2bfloat16_rn(dz2[n][2]);
      T.dz2[r1][col + 1] = __float2bfloat16_rn(dz2[n][3]);
    }
    // dH1 = dZ2 W2^T on the tensor cores (A = dZ2 from registers)
    float dh1[8][4];
#pragma unroll
    for (int n = 0; n < 8; ++n)
#pragma unroll
      for (int q = 0; q < 4; ++q) dh1[n][q] = 0.f;
#pragma unroll
    for (int kc = 0; kc < 4; ++kc) {
      uint32_t a0 = pack_bf16(dz2[2 * kc][0], dz2[2 * kc][1]);
      uint32_t a1 = pack_bf16(dz2[2 * kc][2], dz2[2 * kc][3]);
      uint32_t a2 = pack_bf16(dz2[2 * kc + 1][0], dz2[2 * kc + 1][1]);
      uint32_t a3 = pack_bf16(dz2[2 * kc + 1][2], dz2[2 * kc + 1][3]);
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        // B(kk = hidden-2 index, col = hidden-1 index) = W2[col][kk]
        uint32_t b0 = ld_pair(&T.w2[n * 8 + g][kc * 16 + 2 * t]);
        uint32_t b1 = ld_pair(&T.w2[n * 8 + g][kc * 16 + 2 * t + 8]);
        mma_bf16(dh1[n], a0, a1, a2, a3, b0, b1);
      }
    }
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      int col = n * 8 + 2 * t;
      T.dz1[r0][col] = __float2bfloat16_rn(dh1[n][0] * gelu_grad(F.z1[n][0]));
      T.dz1[r0][col + 1] = __float2bfloat16_rn(dh1[n][1] * gelu_grad(F.z1[n][1]));
      T.dz1[r1][col] = __float2bfloat16_rn(dh1[n][2] * gelu_grad(F.z1[n][2]));
      T.dz1[r1][col + 1] = __float2bfloat16_rn(dh1[n][3] * gelu_grad(F.z1[n][3]));
    }
    __syncthreads();
    // weight gradients, reduction over the 64 samples on the tensor cores:
    // dW2[k][n] = sum_s H1[s][k] dZ2[s][n] (warp w: rows k of m-tile w)
    // dW1[k][n] = sum_s X[s][k] dZ1[s][n]  (warps 0-2: m-tiles of k < 48)
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      const int s0 = ks * 16 + 2 * t;
      const int m0 = warp * 16 + g;
      uint32_t a0 = pack_two(T.h1[s0][m0], T.h1[s0 + 1][m0]);
      uint32_t a1 = pack_two(T.h1[s0][m0 + 8], T.h1[s0 + 1][m0 + 8]);
      uint32_t a2 = pack_two(T.h1[s0 + 8][m0], T.h1[s0 + 9][m0]);
      uint32_t a3 = pack_two(T.h1[s0 + 8][m0 + 8], T.h1[s0 + 9][m0 + 8]);
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        const int nn = n * 8 + g;
        uint32_t b0 = pack_two(T.dz2[s0][nn], T.dz2[s0 + 1][nn]);
        uint32_t b1 = pack_two(T.dz2[s0 + 8][nn], T.dz2[s0 + 9][nn]);
        mma_bf16(aw2[n], a0, a1, a2, a3, b0, b1);
      }
      if (warp < 3) {
        uint32_t c0_ = pack_two(T.xs[s0][m0], T.xs[s0 + 1][m0]);
        uint32_t c1_ = pack_two(T.xs[s0][m0 + 8], T.xs[s0 + 1][m0 + 8]);
        uint32_t c2_ = pack_two(T.xs[s0 + 8][m0], T.xs[s0 + 9][m0]);
        uint32_t c3_ = pack_two(T.xs[s0 + 8][m0 + 8], T.xs[s0 + 9][m0 + 8]);
#pragma unroll
        for (int n = 0; n < 8; ++n) {
          const int nn = n * 8 + g;
          uint32_t b0 = pack_two(T.dz1[s0][nn], T.dz1[s0 + 1][nn]);
          uint32_t b1 = pack_two(T.dz1[s0 + 8][nn], T.dz1[s0 + 9][nn]);
          mma_bf16(aw1[n], c0_, c1_, c2_, c3_, b0, b1);
        }
      }
    }
    // bias and last-layer gradients on the CUDA cores (2 columns per lane)
    if (warp == 3) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        int col = lane * 2 + h;
        float sb1 = 0.f, sb2 = 0.f, sw3 = 0.f;
        for (int s = 0; s < kChunk; ++s) {
          sb1 += __bfloat162float(T.dz1[s][col]);
          sb2 += __bfloat162float(T.dz2[s][col]);
          sw3 += T.dl[s] * __bfloat162float(T.h2[s][col]);
        }
        ab1[h] += sb1;
        ab2[h] += sb2;
        aw3[h] += sw3;
      }
      if (lane == 0)
        for (int s = 0; s < kChunk; ++s) ab3 += T.dl[s];
    }
    __syncthreads();
  }
  // flush the block's partial gradients
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const int col = n * 8 + 2 * t;
    const int k0 = warp * 16 + g, k1 = k0 + 8;
    atomicAdd(&grad[kOffW2 + k0 * kHid + col], aw2[n][0]);
    atomicAdd(&grad[kOffW2 + k0 * kHid + col + 1], aw2[n][1]);
    atomicAdd(&grad[kOffW2 + k1 * kHid + col], aw2[n][2]);
    atomicAdd(&grad[kOffW2 + k1 * kHid + col + 1], aw2[n][3]);
    if (warp < 3) {
      if (k0 < kFeat) {
        atomicAdd(&grad[kOffW1 + k0 * kHid + col], aw1[n][0]);
        atomicAdd(&grad[kOffW1 + k0 * kHid + col + 1], aw1[n][1]);
      }
      if (k1 < kFeat) {
        atomicAdd(&grad[kOffW1 + k1 * kHid + col], aw1[n][2]);
        atomicAdd(&grad[kOffW1 + k1 * kHid + col + 1], aw1[n][3]);
      }
    }
  }
  if (warp == 3) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      atomicAdd(&grad[kOffB1 + lane * 2 + h], ab1[h]);
      atomicAdd(&grad[kOffB2 + lane * 2 + h], ab2[h]);
      atomicAdd(&grad[kOffW3 + lane * 2 + h], aw3[h]);
    }
    if (lane == 0) atomicAdd(&grad[kOffB3], ab3);
  }
  if (loss_sum) {
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (lane == 0) atomicAdd(loss_sum, lsum);
  }
}

// Inference on a feature matrix (evaluation and tests): logits of N rows.
__global__ void __launch_bounds__(128) mlp_forward_kernel(const __nv_bfloat16* __restrict__ X, long N,
                                                          const float* __restrict__ P, float* __restrict__ logit) {
  __shared__ MlpSmem S;
  __shared__ __align__(16) __nv_bfloat16 xs[kChunk][kFeatPad];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  mlp_stage_params(S, P, tid, 128);
  __syncthreads();
  for (long c0 = (long)blockIdx.x * kChunk; c0 < N; c0 += (long)gridDim.x * kChunk) {
    for (int e = tid; e < kChunk * kFeatPad; e += 128) {
      int r = e / kFeatPad, k = e % kFeatPad;
      long s = c0 + r;
      xs[r][k] = (s < N && k < kFeat) ? X[s * kFeat + k] : __float2bfloat16_rn(0.0f);
    }
    __syncthreads();
    MlpFwd16 F;
    mlp_forward16(S, &xs[warp * 16][0], kFeatPad, lane, F);
    if ((lane & 3) == 0) {
      long s0 = c0 + warp * 16 + (lane >> 2);
      if (s0 < N) logit[s0] = F.logit[0];
      if (s0 + 8 < N) logit[s0 + 8] = F.logit[1];
    }
    __syncthreads();
  }
}

// Adam on the FP32 master parameters; the gradient is a sum over samples and
// is scaled by inv_n (1 / total sample weight).
__global__ void adam_kernel(float* P, const float* grad, float* m, float* v, int n, float lr, float b1, float b2,
                            float eps, float inv_n, int step) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float gr = grad[i] * inv_n;
  float mm = b1 * m[i] + (1.f - b1) * gr;
  float vv = b2 * v[i] + (1.f - b2) * gr * gr;
  m[i] = mm;
  v[i] = vv;
  float mh = mm / (1.f - powf(b1, (float)step));
  float vh = vv / (1.f - powf(b2, (float)step));
  P[i] -= lr * mh / (sqrtf(vh) + eps);
}

}  // namespace enl

using namespace enl;

// Largest |erf_as(x) - erff(x)| over n points evenly spread in [-6, 6]
// (bits of a non-negative float: ordered as unsigned integers).
__global__ void erf_check_kernel(int n, unsigned* max_bits) {
  float m = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float x = -6.0f + 12.0f * (float)i / (float)(n - 1);
    m = fmaxf(m, fabsf(erf_as(x) - erff(x)));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(max_bits, __float_as_uint(m));
}

extern "C" {

int enl_mlp_erf_error(double* max_err) {
  if (!max_err) return ENL_ERR_ARG;
  unsigned* d = nullptr;
  if (cudaMalloc(&d, sizeof(unsigned)) != cudaSuccess) return ENL_ERR_CUDA;
  cudaMemsetAsync(d, 0, sizeof(unsigned), stream());
  erf_check_kernel<<<256, 256, 0, stream()>>>(1 << 22, d);
  unsigned h = 0;
  cudaMemcpyAsync(&h, d, sizeof(unsigned), cudaMemcpyDeviceToHost, stream());
  cudaStreamSynchronize(stream());
  cudaFree(d);
  float f;
  memcpy(&f, &h, sizeof(f));
  *max_err = f;
  return check_launch("mlp erf check");
}

int enl_mlp_nparams(void) { return kNParams; }

int enl_mlp_grad(const void* X, const float* y, const float* wgt, long n, const float* params, float* grad,
                 double* loss_sum) {
  if (!X || !y || !wgt || !params || !grad || n < 0) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  if (n == 0) return ENL_OK;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem));
    attr = true;
  }
  int nsm = 148;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0);
  long chunks = (n + kChunk - 1) / kChunk;
  int blocks = (int)std::min<long>(chunks, (long)nsm * 4);
  mlp_grad_kernel<<<blocks, 128, sizeof(TrainSmem), stream()>>>((const __nv_bfloat16*)X, y, wgt, n, params, grad,
                                                               loss_sum);
  return check_launch("mlp_grad");
}

int enl_mlp_forward(const void* X, long n, const float* params, float* logits) {
  if (!X || !params || !logits || n < 0) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  if (n == 0) return ENL_OK;
  int nsm = 148;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0);
  long chunks = (n + kChunk - 1) / kChunk;
  int blocks = (int)std::min<long>(chunks, (long)nsm * 8);
  mlp_forward_kernel<<<blocks, 128, 0, stream()>>>((const __nv_bfloat16*)X, n, params, logits);
  return check_launch("mlp_forward");
}

int enl_mlp_adam(float* params, const float* grad, float* m, float* v, float lr, float beta1, float beta2, float eps,
                 float inv_n, int step) {
  if (!params || !grad || !m || !v || step < 1) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  adam_kernel<<<(kNParams + 255) / 256, 256, 0, stream()>>>(params, grad, m, v, kNParams, lr, beta1, beta2, eps, inv_n,
                                                          step);
  return check_launch("mlp_adam");
}

}  // extern "C"
