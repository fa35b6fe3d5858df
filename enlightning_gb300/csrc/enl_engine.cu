// Batched multi-level engine: canvases, device tile tables, fused persistent
// stage kernel with TMA halo staging, ghost fill, coarsening, CUDA graph.
//
// Reference semantics restated here:
//   stage loop       SAMRAI MethodOfLinesIntegrator (driven at main.C:448),
//                    coefficients input.txt:130-133
//   singleStep       enlightning.C:459-583 (rhs -> runge_kutta ->
//                    update_state -> absorbing envelope)
//   physical ghosts  enlightning.C:790-1013
//   coarse-fine      LINEAR_REFINE / CONSERVATIVE_COARSEN registered at
//                    enlightning.C:259-288 (arithmetic defined in this file:
//                    bilinear in cell centres, 2x2 average)
//   tag_cells        fortran/tag_cells.m4:58-108
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <vector>

#include "enl_fast.cuh"
#include "enl_mlp.cuh"
#include "enl_rhs_cell.cuh"
#include "enl_tma.cuh"

namespace enl {

RhsConst make_rhs_const(const double* xlo, const double* dx, double alpha, double kappa, double mu,
                        double muB, double R, double T_star_n, double tau_n, const double* tol, int level,
                        double c, double c_lr);

constexpr int kL = ENL_MAX_LEVELS;
constexpr int kTW = 32, kTH = 8;                 // tile interior (cells)
constexpr int kBW = kTW + 6, kBH = kTH + 6;      // halo box
constexpr int kNF = 7;                           // stored fields
constexpr int kTileElems = kNF * kBH * kBW;      // 3724
constexpr int kTileBytes64 = kTileElems * 8;     // 29792
// Shared-memory layout of the stage kernel.  A TMA destination must start on
// a 128-byte boundary, so every region is padded to a multiple of 128 bytes.
constexpr int align128(int b) { return (b + 127) / 128 * 128; }
constexpr int kStageBufBytes = align128(kTileBytes64);            // 29824
constexpr int kTile32Bytes = align128(kTileElems * 4);            // 14976
constexpr int kOffTile32 = 2 * kStageBufBytes;
constexpr int kOffMlp = kOffTile32 + kTile32Bytes;
constexpr int kWaitIters = 1 << 22;              // bounded mbarrier polls

struct StageArgs {
  CUtensorMap tmap[kL];  // input buffer, per level
  double* in[kL];
  double* out[kL];
  const double* un[kL];  // u^n (current buffer)
  const double* h0[kL];
  long pitch[kL], fstride[kL];
  RhsConst P[kL];
  FastConst F[kL];
  double rho0, p0, T0, c, c_lr, gm1_over_2rho0, c_p, c_v, R, ylo, dy[kL];
  double a1, a2, bdt, beta;
  const double* dt_dev;  // adaptive time step in device memory (or null)
  const int4* tiles;
  const int* ntiles;
  int* counter;
  int* health;
  unsigned long long* stats;  // [level][3]: weno cells, cells, cells decided by the plain-sensor fallback
  const float* mlp;           // learned-sensor parameters (FP32 vector) or null
  float margin;               // |p - 0.5| <= margin -> plain sensor decides
  float feat_eps, feat_eps_p, feat_inv_sqrt_eps;
};

// Shared-memory accessors centred on one cell of the staged halo tile.
struct SAcc64 {
  const double* t;  // tile base
  int c;            // (row)*kBW + col of the centre
  __device__ double w(int k, int di, int dj) const { return t[k * (kBH * kBW) + c + dj * kBW + di]; }
  __device__ double p(int di, int dj) const { return t[5 * (kBH * kBW) + c + dj * kBW + di]; }
  __device__ double t_(int di, int dj) const { return t[6 * (kBH * kBW) + c + dj * kBW + di]; }
  __device__ double tT(int di, int dj) const { return t_(di, dj); }
};
struct SAcc64R {  // adapter with the accessor names rhs_cell expects
  SAcc64 a;
  __device__ double w(int k, int di, int dj) const { return a.w(k, di, dj); }
  __device__ double p(int di, int dj) const { return a.p(di, dj); }
  __device__ double t(int di, int dj) const { return a.tT(di, dj); }
};
struct SAcc32 {
  const float* t;
  int c;
  __device__ float w(int k, int di, int dj) const { return t[k * (kBH * kBW) + c + dj * kBW + di]; }
  __device__ float p(int di, int dj) const { return t[5 * (kBH * kBW) + c + dj * kBW + di]; }
  __device__ float t_(int di, int dj) const { return t[6 * (kBH * kBW) + c + dj * kBW + di]; }
};
struct SAcc32R {
  SAcc32 a;
  __device__ float w(int k, int di, int dj) const { return a.w(k, di, dj); }
  __device__ float p(int di, int dj) const { return a.p(di, dj); }
  __device__ float t(int di, int dj) const { return a.t_(di, dj); }
};

__device__ __forceinline__ void raise_health(int* h, int code) { atomicCAS(h, 0, code); }

// ---------------------------------------------------------------------------
// Fused persistent stage kernel: per tile, TMA-stage the (32+6)x(8+6) halo box
// of all 7 fields, decide WENO/DRP per cell, compact the cells so that each
// warp runs one branch, compute KK, and finish the cell in place:
// w = a1*u^n + a2*w + beta*dt*KK, then p and T (update_state).
// ---------------------------------------------------------------------------
template <int SCHEME, int ORDER, bool LLF, bool FAST>
__global__ void __launch_bounds__(256, 2) stage_kernel(const __grid_constant__ StageArgs A) {
  // dynamic shared memory: two FP64 staging buffers (TMA destinations, the
  // next tile's copy overlaps the current tile's compute) + one FP32 tile
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* stage_buf[2] = {reinterpret_cast<double*>(smem_raw),
                          reinterpret_cast<double*>(smem_raw + kStageBufBytes)};
  float* tile32 = reinterpret_cast<float*>(smem_raw + kOffTile32);
  // learned sensor (FAST + hybrid only): network image and feature tile
  MlpSmem* mlp_s = reinterpret_cast<MlpSmem*>(smem_raw + kOffMlp);
  __nv_bfloat16* feat = reinterpret_cast<__nv_bfloat16*>(smem_raw + kOffMlp + align128((int)sizeof(MlpSmem)));
  __shared__ unsigned char s_flag[256];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ int s_t[2];
  __shared__ int s_cnt[2][8];
  __shared__ int s_list[256];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ntiles = *A.ntiles;
  auto issue = [&](int t, int b) {
    const int4 td = A.tiles[t];
    // a tiled TMA copy needs x * 8 bytes to be a multiple of 16 (x even);
    // set_patches only accepts even patch origins and tiles are 32 wide
    if (td.x & 1) {
      raise_health(A.health, ENL_ERR_STATE);
      return false;
    }
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&mbar[b], kTileBytes64);
    // canvas column of cell i0-3 is i0 (ghost offset 3); i0 is even
    tma_load_3d(stage_buf[b], &A.tmap[td.z & 0xff], td.x, td.y, 0, &mbar[b]);
    return true;
  };
  // TMA destinations must start on 128-byte boundaries; refuse to run otherwise
  if ((smem_u32(smem_raw) & 127u) != 0u) {
    if (tid == 0) raise_health(A.health, ENL_ERR_STATE);
    return;
  }
  const bool learned = FAST && SCHEME == kHybrid && A.mlp != nullptr;
  if (learned) mlp_stage_params(*mlp_s, A.mlp, tid, 256);
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_mbar_init();
    int t = atomicAdd(A.counter, 1);
    if (t < ntiles && !issue(t, 0)) t = ntiles;
    s_t[0] = t;
  }
  __syncthreads();
  uint32_t phase[2] = {0u, 0u};
  int b = 0;
  int t = s_t[0];
  while (t < ntiles) {
    if (tid == 0) {
      int nt = atomicAdd(A.counter, 1);
      if (nt < ntiles && !issue(nt, b ^ 1)) nt = ntiles;
      s_t[b ^ 1] = nt;
    }
    double* tile = stage_buf[b];
    const int4 td = A.tiles[t];
    const int lvl = td.z & 0xff, w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    const int i0 = td.x, j0 = td.y;
    if (!mbar_wait_bounded(&mbar[b], phase[b], kWaitIters)) {
      if (tid == 0) raise_health(A.health, ENL_ERR_TIMEOUT);
      // let copies in flight land (bounded) before the block leaves
      mbar_wait_bounded(&mbar[b], phase[b], kWaitIters);
      mbar_wait_bounded(&mbar[b ^ 1], phase[b ^ 1], kWaitIters);
      break;
    }
    phase[b] ^= 1u;
    const double bdt = A.dt_dev ? A.beta * (*A.dt_dev) : A.bdt;
    if (FAST) {
      const float rho0 = (float)A.rho0;
      for (int e = tid; e < kTileElems; e += 256) {
        int k = e / (kBH * kBW);
        double v = tile[e];
        double amb = k == 0 ? A.rho0 : (k == 4 ? A.rho0 * A.T0 : (k == 5 ? A.p0 : (k == 6 ? A.T0 : 0.0)));
        tile32[e] = (float)(v - amb);
      }
      (void)rho0;
      __syncthreads();
    }
    const int tx = lane, ty = warp;
    const bool valid = tx < w && ty < h;
    const int cc = (ty + 3) * kBW + (tx + 3);
    int flag = 0;
    int fallback = 0;
    if (learned && lvl == 0) {
      // learned switch: features -> BF16 MLP on the tensor cores (one warp per
      // tile row, two m16 tiles) -> p; cells with |p - 0.5| <= margin fall
      // back to the plain sensor
      float fv[kFeat];
      if (valid) {
        SAcc32R acc{SAcc32{tile32, cc}};
        cell_features(acc, A.feat_eps, A.feat_eps_p, A.feat_inv_sqrt_eps, fv);
      } else {
#pragma unroll
        for (int q = 0; q < kFeat; ++q) fv[q] = 0.f;
      }
#pragma unroll
      for (int q = 0; q < kFeat; q += 2)
        *reinterpret_cast<uint32_t*>(feat + tid * kFeat + q) = pack_bf16(fv[q], fv[q + 1]);
      __syncwarp();
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        MlpFwd16 F;
        mlp_forward16(*mlp_s, feat + (warp * 32 + half * 16) * kFeat, kFeat, lane, F);
        if ((lane & 3) == 0) {
          int c0 = warp * 32 + half * 16 + (lane >> 2);
          s_flag[c0] = (unsigned char)(F.logit[0] > 0.f ? 2 : 1) | (fabsf(F.logit[0]) <= A.margin ? 4 : 0);
          s_flag[c0 + 8] = (unsigned char)(F.logit[1] > 0.f ? 2 : 1) | (fabsf(F.logit[1]) <= A.margin ? 4 : 0);
        }
      }
      __syncwarp();
      if (valid) {
        unsigned char d = s_flag[tid];
        if (d & 4) {
          SAcc32R acc{SAcc32{tile32, cc}};
          flag = sensor_fast(acc, A.F[lvl]);
          fallback = 1;
        } else {
          flag = (d & 2) ? 1 : 0;
        }
      }
    } else if (valid) {
      if (FAST) {
        SAcc32R acc{SAcc32{tile32, cc}};
        flag = SCHEME == kWeno ? 1 : (SCHEME == kDrp ? 0 : sensor_fast(acc, A.F[lvl]));
      } else {
        SAcc64R acc{SAcc64{tile, cc}};
        flag = rhs_switch<SCHEME, ORDER, LLF>(acc, A.P[lvl]);
      }
    }
    const int nfb = learned ? __syncthreads_count(fallback) : 0;
    // compaction: DRP cells first, then WENO cells, each in tile order
    unsigned bd = __ballot_sync(0xffffffffu, valid && !flag);
    unsigned bw = __ballot_sync(0xffffffffu, valid && flag);
    if (lane == 0) {
      s_cnt[0][warp] = __popc(bd);
      s_cnt[1][warp] = __popc(bw);
    }
    __syncthreads();
    int nd = 0, nw = 0, od = 0, ow = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      if (q < warp) {
        od += s_cnt[0][q];
        ow += s_cnt[1][q];
      }
      nd += s_cnt[0][q];
      nw += s_cnt[1][q];
    }
    if (valid) {
      unsigned lt = (1u << lane) - 1u;
      int pos = flag ? (nd + ow + __popc(bw & lt)) : (od + __popc(bd & lt));
      s_list[pos] = (ty << 5) | tx | (flag << 16);
    }
    if (tid == 0 && A.stats) {
      atomicAdd(&A.stats[3 * lvl + 0], (unsigned long long)nw);
      atomicAdd(&A.stats[3 * lvl + 1], (unsigned long long)(nd + nw));
      if (nfb) atomicAdd(&A.stats[3 * lvl + 2], (unsigned long long)nfb);
    }
    __syncthreads();
    if (tid < nd + nw) {
      const int e = s_list[tid];
      const int cx = e & 31, cy = (e >> 5) & 0xff, f = (e >> 16) & 1;
      const int c2 = (cy + 3) * kBW + (cx + 3);
      const int gi = i0 + cx, gj = j0 + cy;  // level index
      const long g = (long)(gj + 3) * A.pitch[lvl] + (gi + 3);
      const long fs = A.fstride[lvl];
      const double* un = A.un[lvl];
      double* out = A.out[lvl];
      double wn[5];
      if (FAST) {
        SAcc32R acc{SAcc32{tile32, c2}};
        float H[5], K[5];
        H[0] = (float)A.h0[lvl][g];
        sources_fast(acc, A.F[lvl], H);
        fluxes_fast<ORDER, LLF>(acc, A.F[lvl], gj, f, H, K);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          double win = tile[k * (kBH * kBW) + c2];
          wn[k] = fma(bdt, (double)K[k], fma(A.a1, un[k * fs + g], A.a2 * win));
        }
        // update_state in perturbation form (update_state.m4:90-105)
        const float rp = (float)(wn[0] - A.rho0);
        const float inv_r = 1.0f / (float)wn[0];
        const float s = (float)wn[3] * inv_r;
        const float h = (float)(A.ylo + A.dy[lvl] * ((double)gj + 0.5));
        const float ccl = (float)A.c + (float)A.c_lr * h;
        const float pp = (ccl * ccl) * ((rp + (float)A.gm1_over_2rho0 * (rp * rp)) + (float)wn[3] / (float)A.c_p);
        const float x = (s + (float)A.R * log1pf(rp / (float)A.rho0)) / (float)A.c_v;
        const float tp = (float)A.T0 * expm1f(x);
        out[5 * fs + g] = A.p0 + (double)pp;
        out[6 * fs + g] = A.T0 + (double)tp;
      } else {
        SAcc64R acc{SAcc64{tile, c2}};
        double H[5], K[5];
        H[0] = A.h0[lvl][g];
        rhs_sources(acc, A.P[lvl], H);
        rhs_fluxes<SCHEME, ORDER, LLF>(acc, A.P[lvl], gj, f, H, K);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          double win = tile[k * (kBH * kBW) + c2];
          wn[k] = __dadd_rn(__dadd_rn(__dmul_rn(A.a1, un[k * fs + g]), __dmul_rn(A.a2, win)),
                            __dmul_rn(bdt, K[k]));
        }
        const double hgt = __dadd_rn(A.ylo, __dmul_rn(A.dy[lvl], (double)gj + 0.5));
        const double cc_ = __dadd_rn(A.c, __dmul_rn(A.c_lr, hgt));
        const double d = __dsub_rn(wn[0], A.rho0);
        const double s = __ddiv_rn(wn[3], wn[0]);
        const double inner = __dadd_rn(__dadd_rn(d, __dmul_rn(A.gm1_over_2rho0, __dmul_rn(d, d))),
                                       __dmul_rn(__ddiv_rn(wn[0], A.c_p), s));
        out[5 * fs + g] = __dadd_rn(__dmul_rn(__dmul_rn(cc_, cc_), inner), A.p0);
        out[6 * fs + g] = A.T0 * exp((s - A.R * log(A.rho0 / wn[0])) / A.c_v);
      }
#pragma unroll
      for (int k = 0; k < 5; ++k) out[k * fs + g] = wn[k];
      if (!(wn[0] > 0.0) || !isfinite(wn[0] + wn[1] + wn[2] + wn[3] + wn[4])) raise_health(A.health, ENL_ERR_NONFINITE);
    }
    __syncthreads();  // this staging buffer is refilled two tiles later
    t = s_t[b ^ 1];
    b ^= 1;
  }
}

// ---------------------------------------------------------------------------
// Ghost fill and transfer kernels (canvas form)
// ---------------------------------------------------------------------------
struct CanvasView {
  double* base;
  long pitch, fstride;
  int nx, ny;
  __device__ double& at(int k, int i, int j) const { return base[k * fstride + (long)(j + 3) * pitch + (i + 3)]; }
};

// Physical ghost band of one level (enlightning.C:830-1008 for the patch that
// touches each side): edge ghosts copy the first interior cell of their row or
// column, corners copy the interior corner cell; the normal momentum is
// negated on REFLECT sides (both momenta in a corner of two REFLECT sides).
__global__ void physbc_kernel(CanvasView V, int nfields, int bcL, int bcR, int bcB, int bcT) {
  const int nx = V.nx, ny = V.ny;
  const long nedge_x = 3L * ny, nedge_y = 3L * nx;
  const long total = (2 * nedge_x + 2 * nedge_y + 36) * nfields;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    int k = (int)(t % nfields);
    long r = t / nfields;
    int i, j, si, sj;
    bool negu = false, negv = false;
    if (r < 2 * nedge_x) {
      int side = (int)(r / nedge_x);
      long q = r % nedge_x;
      j = (int)(q / 3);
      int d = (int)(q % 3);
      sj = j;
      if (side == 0) { i = -1 - d; si = 0; negu = bcL == kReflect; }
      else { i = nx + d; si = nx - 1; negu = bcR == kReflect; }
    } else if (r < 2 * nedge_x + 2 * nedge_y) {
      r -= 2 * nedge_x;
      int side = (int)(r / nedge_y);
      long q = r % nedge_y;
      i = (int)(q / 3);
      int d = (int)(q % 3);
      si = i;
      if (side == 0) { j = -1 - d; sj = 0; negv = bcB == kReflect; }
      else { j = ny + d; sj = ny - 1; negv = bcT == kReflect; }
    } else {
      r -= 2 * nedge_x + 2 * nedge_y;
      int corner = (int)(r / 9), q = (int)(r % 9);
      int dx = q % 3, dy = q / 3;
      int xs = corner & 1, ys = corner >> 1;
      i = xs ? nx + dx : -1 - dx;
      j = ys ? ny + dy : -1 - dy;
      si = xs ? nx - 1 : 0;
      sj = ys ? ny - 1 : 0;
      negu = (xs ? bcR : bcL) == kReflect;
      negv = (ys ? bcT : bcB) == kReflect;
    }
    double v = V.at(k, si, sj);
    if ((k == 1 && negu) || (k == 2 && negv)) v = -v;
    V.at(k, i, j) = v;
  }
}

// Independent problems: every patch of the table is a domain of its own, and
// its 3-cell band is filled by the single-patch rule of enlightning.C:830-1008
// (edges from the first interior cell, corners from the interior corner, the
// normal momenta negated on REFLECT sides).  One block per patch.
__global__ void physbc_patches_kernel(CanvasView V, const int4* patches, int off, int cnt, int bcL, int bcR,
                                      int bcB, int bcT) {
  for (int p = blockIdx.x; p < cnt; p += gridDim.x) {
    const int4 b = patches[off + p];
    const int w = b.y - b.x + 1, h = b.w - b.z + 1;
    const int nband = 6 * h + 6 * w + 36;
    for (int t = threadIdx.x; t < nband * kNF; t += blockDim.x) {
      int k = t % kNF, r = t / kNF;
      int i, j, si, sj;
      bool negu = false, negv = false;
      if (r < 6 * h) {
        int side = r / (3 * h), q = r % (3 * h);
        j = b.z + q / 3;
        int d = q % 3;
        sj = j;
        if (side == 0) { i = b.x - 1 - d; si = b.x; negu = bcL == kReflect; }
        else { i = b.y + 1 + d; si = b.y; negu = bcR == kReflect; }
      } else if (r < 6 * h + 6 * w) {
        r -= 6 * h;
        int side = r / (3 * w), q = r % (3 * w);
        i = b.x + q / 3;
        int d = q % 3;
        si = i;
        if (side == 0) { j = b.z - 1 - d; sj = b.z; negv = bcB == kReflect; }
        else { j = b.w + 1 + d; sj = b.w; negv = bcT == kReflect; }
      } else {
        r -= 6 * h + 6 * w;
        int corner = r / 9, q = r % 9;
        int xs = corner & 1, ys = corner >> 1;
        i = xs ? b.y + 1 + q % 3 : b.x - 1 - q % 3;
        j = ys ? b.w + 1 + q / 3 : b.z - 1 - q / 3;
        si = xs ? b.y : b.x;
        sj = ys ? b.w : b.z;
        negu = (xs ? bcR : bcL) == kReflect;
        negv = (ys ? bcT : bcB) == kReflect;
      }
      double v = V.at(k, si, sj);
      if ((k == 1 && negu) || (k == 2 && negv)) v = -v;
      V.at(k, i, j) = v;
    }
  }
}

// Coarse-fine ghosts: bilinear interpolation in cell centres from the
// coarser canvas.  One warp per halo row segment (j, i_begin, i_end).
__device__ __forceinline__ void refine_weights(int I, int r, int& ic, double& f) {
  // fine cell centre in coarse index coordinates: (I + 0.5)/r - 0.5
  double xc = ((double)I + 0.5) / (double)r - 0.5;
  double fl = floor(xc);
  ic = (int)fl;
  f = xc - fl;
}

__global__ void interp_kernel(CanvasView F, CanvasView C, int ratio, const int4* segs, const int* meta, int moff,
                              int mcnt, int nfields) {
  const int off = meta[moff], cnt = meta[mcnt];
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  for (int s = gw; s < cnt; s += warps) {
    int4 sg = segs[off + s];
    int J = sg.x;
    int jc;
    double fy;
    refine_weights(J, ratio, jc, fy);
    for (int I = sg.y + lane; I <= sg.z; I += 32) {
      int ic;
      double fx;
      refine_weights(I, ratio, ic, fx);
      for (int k = 0; k < nfields; ++k) {
        double c00 = C.at(k, ic, jc), c10 = C.at(k, ic + 1, jc), c01 = C.at(k, ic, jc + 1), c11 = C.at(k, ic + 1, jc + 1);
        double lo = (1.0 - fx) * c00 + fx * c10;
        double hi = (1.0 - fx) * c01 + fx * c11;
        F.at(k, I, J) = (1.0 - fy) * lo + fy * hi;
      }
    }
  }
}

// Generic tile-list kernels: one block of 256 threads per 32x8 tile.
// Coarsening: coarse cell = mean of its ratio x ratio fine cells (7 fields).
__global__ void coarsen_kernel(CanvasView C, CanvasView F, int ratio, const int4* tiles, const int* meta, int moff,
                               int mcnt) {
  const int off = meta[moff], cnt = meta[mcnt];
  for (int t = blockIdx.x; t < cnt; t += gridDim.x) {
    int4 td = tiles[off + t];
    int w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (tx >= w || ty >= h) continue;
    int I = td.x + tx, J = td.y + ty;
    double inv = 1.0 / (double)(ratio * ratio);
    for (int k = 0; k < kNF; ++k) {
      double s = 0.0;
      for (int b = 0; b < ratio; ++b)
        for (int a = 0; a < ratio; ++a) s += F.at(k, I * ratio + a, J * ratio + b);
      C.at(k, I, J) = s * inv;
    }
  }
}

// Copy patch interiors between two buffers of the same level (7 fields).
__global__ void copy_tiles_kernel(CanvasView dst, CanvasView src, const int4* tiles, int off, int cnt) {
  for (int t = blockIdx.x; t < cnt; t += gridDim.x) {
    int4 td = tiles[off + t];
    int w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (tx >= w || ty >= h) continue;
    for (int k = 0; k < kNF; ++k) dst.at(k, td.x + tx, td.y + ty) = src.at(k, td.x + tx, td.y + ty);
  }
}

// Bilinear fill of whole boxes (new fine data after a regrid).
__global__ void refine_box_kernel(CanvasView F, CanvasView C, int ratio, int ilo, int jlo, int w, int h) {
  long n = (long)w * h;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    int I = ilo + (int)(t % w), J = jlo + (int)(t / w);
    int ic, jc;
    double fx, fy;
    refine_weights(I, ratio, ic, fx);
    refine_weights(J, ratio, jc, fy);
    for (int k = 0; k < kNF; ++k) {
      double lo = (1.0 - fx) * C.at(k, ic, jc) + fx * C.at(k, ic + 1, jc);
      double hi = (1.0 - fx) * C.at(k, ic, jc + 1) + fx * C.at(k, ic + 1, jc + 1);
      F.at(k, I, J) = (1.0 - fy) * lo + fy * hi;
    }
  }
}

// tag_cells.m4:58-108 over the tiles of one level, bit-exact.
__device__ __forceinline__ bool ratio_below_e(double fm, double f0, double fp, double ep) {
  double t1 = __dsub_rn(f0, fm);
  double t2 = __dsub_rn(fp, f0);
  double num = __dadd_rn(__dmul_rn(2.0, fabs(__dmul_rn(t1, t2))), ep);
  double den = __dadd_rn(__dadd_rn(__dmul_rn(t1, t1), __dmul_rn(t2, t2)), ep);
  return __ddiv_rn(num, den) < Lit::c0_9999;
}

__global__ void tag_tiles_kernel(int* tags, CanvasView W, CanvasView H, const int4* tiles, int off, int cnt,
                                 double ep0, double ep1) {
  for (int t = blockIdx.x; t < cnt; t += gridDim.x) {
    int4 td = tiles[off + t];
    int w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (tx >= w || ty >= h) continue;
    int i = td.x + tx, j = td.y + ty;
    bool tg = ratio_below_e(H.at(0, i - 1, j), H.at(0, i, j), H.at(0, i + 1, j), ep0) ||
              ratio_below_e(H.at(0, i, j - 1), H.at(0, i, j), H.at(0, i, j + 1), ep0) ||
              ratio_below_e(W.at(0, i - 1, j), W.at(0, i, j), W.at(0, i + 1, j), ep1) ||
              ratio_below_e(W.at(0, i, j - 1), W.at(0, i, j), W.at(0, i, j + 1), ep1);
    tags[(long)j * W.nx + i] = tg ? 1 : 0;
  }
}

// Absorbing envelope per patch (enlightning.C:634-786, loop-exit rules kept):
// one thread per patch row (L/R) or column (B/T).  Patches come from a table
// (ilo, ihi, jlo, jhi); the envelope distance uses the level's cell centres.
struct AbsorbArgs {
  double dx0, dx1, gxlo0, gxlo1, gxhi0, gxhi1, w2, p0, T0, rho0;
};

__device__ __forceinline__ double env_(double d, double w2) {
  return __dadd_rn(-exp(__dmul_rn(__ddiv_rn(-log(2.0), w2), __dmul_rn(d, d))), 1.0);
}
__device__ __forceinline__ double relax_(double q, double amb, double tmp) {
  return __dadd_rn(__dmul_rn(__dsub_rn(q, amb), tmp), amb);
}

__global__ void absorb_patches_kernel(CanvasView V, const int4* patches, int off, int cnt, int dir, AbsorbArgs A) {
  const double ep = 1.0e-8;
  // grid-stride over (patch, row/column); the host passes a bound on rows
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x;; t += (long)gridDim.x * blockDim.x) {
    long acc = 0;
    int p = -1, r = 0;
    for (int q = 0; q < cnt; ++q) {
      int4 b = patches[off + q];
      int n = dir < 2 ? (b.w - b.z + 1) : (b.y - b.x + 1);
      if (t < acc + n) {
        p = q;
        r = (int)(t - acc);
        break;
      }
      acc += n;
    }
    if (p < 0) return;
    int4 b = patches[off + p];
    auto apply = [&](int i, int j, double tmp) {
      V.at(5, i, j) = relax_(V.at(5, i, j), A.p0, tmp);
      V.at(6, i, j) = relax_(V.at(6, i, j), A.T0, tmp);
      V.at(0, i, j) = relax_(V.at(0, i, j), A.rho0, tmp);
      V.at(1, i, j) = __dmul_rn(V.at(1, i, j), tmp);
      V.at(2, i, j) = __dmul_rn(V.at(2, i, j), tmp);
      V.at(3, i, j) = __dmul_rn(V.at(3, i, j), tmp);
      V.at(4, i, j) = relax_(V.at(4, i, j), __dmul_rn(A.T0, A.rho0), tmp);
    };
    if (dir < 2) {
      int j = b.z + r;
      auto dist = [&](int i) {
        double xc = A.gxlo0 + A.dx0 * ((double)i + 0.5);
        return dir == 0 ? (xc - A.gxlo0) : (A.gxhi0 - xc);
      };
      double tmp = (r == 0) ? env_(dist(dir == 0 ? b.x : b.y), A.w2) : 0.0;
      for (int n = 0; fabs(1.0 - tmp) > ep && n <= b.y - b.x; ++n) {
        int i = dir == 0 ? b.x + n : b.y - n;
        tmp = env_(dist(i), A.w2);
        apply(i, j, tmp);
      }
    } else {
      int i = b.x + r;
      auto dist = [&](int j) {
        double yc = A.gxlo1 + A.dx1 * ((double)j + 0.5);
        return dir == 2 ? (yc - A.gxlo1) : (A.gxhi1 - yc);
      };
      double tmp = env_(dist(dir == 2 ? b.z : b.w), A.w2);
      for (int n = 0; fabs(1.0 - tmp) > ep && n <= b.w - b.z; ++n) {
        int j = dir == 2 ? b.z + n : b.w - n;
        tmp = env_(dist(j), A.w2);
        apply(i, j, tmp);
      }
    }
  }
}

// Plain path RK update on a canvas patch (runge_kutta.m4:60-63), in place on
// the stage buffer, and update_state on the same cells.
__global__ void rk_plain_kernel(CanvasView S, CanvasView U, CanvasView K, int ilo, int jlo, int w, int h, double a1,
                                double a2, double bdt, double beta, const double* dt_dev) {
  int ci = blockIdx.x * blockDim.x + threadIdx.x, cj = blockIdx.y * blockDim.y + threadIdx.y;
  if (ci >= w || cj >= h) return;
  if (dt_dev) bdt = beta * (*dt_dev);
  int i = ilo + ci, j = jlo + cj;
  for (int k = 0; k < 5; ++k)
    S.at(k, i, j) = __dadd_rn(__dadd_rn(__dmul_rn(a1, U.at(k, i, j)), __dmul_rn(a2, S.at(k, i, j))),
                              __dmul_rn(bdt, K.at(k, i, j)));
}

struct EosArgs {
  double rho0, c, gm1_over_2rho0, c_p, p0, T0, c_lr, c_v, R, ylo, dy;
};

__global__ void eos_plain_kernel(CanvasView S, int ilo, int jlo, int w, int h, EosArgs E) {
  int ci = blockIdx.x * blockDim.x + threadIdx.x, cj = blockIdx.y * blockDim.y + threadIdx.y;
  if (ci >= w || cj >= h) return;
  int i = ilo + ci, j = jlo + cj;
  double w0 = S.at(0, i, j), w3 = S.at(3, i, j);
  // update_state.m4:88 uses the patch's xlo and (j - ifirst1); with the level
  // origin that is the same centre height.
  double height = __dadd_rn(E.ylo, __dmul_rn(E.dy, (double)j + 0.5));
  double cc = __dadd_rn(E.c, __dmul_rn(E.c_lr, height));
  double d = __dsub_rn(w0, E.rho0);
  double s = __ddiv_rn(w3, w0);
  double inner = __dadd_rn(__dadd_rn(d, __dmul_rn(E.gm1_over_2rho0, __dmul_rn(d, d))), __dmul_rn(__ddiv_rn(w0, E.c_p), s));
  S.at(5, i, j) = __dadd_rn(__dmul_rn(__dmul_rn(cc, cc), inner), E.p0);
  S.at(6, i, j) = E.T0 * exp((s - E.R * log(E.rho0 / w0)) / E.c_v);
}

// ---------------------------------------------------------------------------
// Source painting, enlightning.C:2140-2307 (addSource), one thread per cell of
// the level's patch tiles.  POINT and SINE overwrite; LIGHTNING accumulates
// every channel segment with the capsule-union rule H <- H + t - (H/A) t.
// ---------------------------------------------------------------------------
struct PaintArgs {
  int type, mode;
  double amp, inv_s2ln2;   // log(2) / spread^2
  double pos0, pos1, sine_amp, sine_freq, drive;  // drive: sin(omega*(n+1-n0)*dt)
  double xlo0, xlo1, dx0, dx1;
  const double* segs;      // (x0, y0, x1, y1) per segment
  int nseg;
};

// Per-segment constants (host-computed once, like the reference computes them
// once per segment): x0, y0, x1, y1, theta, tan(pi/2 - theta), sin, cos,
// orientation, and a culling box outside which all three Gaussian terms
// underflow to exactly 0 (so skipping the segment there changes nothing).
constexpr int kSegStride = 13;

__device__ double capsule_union(double H, double xc0, double xc1, const PaintArgs& A) {
  for (int k = 0; k < A.nseg; ++k) {
    const double* s = A.segs + kSegStride * k;
    if (xc0 < s[9] || xc0 > s[10] || xc1 < s[11] || xc1 > s[12]) continue;
    const int orientation = (int)s[8];
    const double theta = s[4], tn = s[5];
    double line0 = tn * (xc0 - s[0]) + s[1];
    double line1 = tn * (xc0 - s[2]) + s[3];
    if (((orientation == 1) && (xc1 >= line0)) || ((orientation == 2) && (xc1 <= line0))) {
      double d0 = xc0 - s[0], d1 = xc1 - s[1];
      double t = A.amp * exp(-A.inv_s2ln2 * (d0 * d0 + d1 * d1));
      H = H + t - (H / A.amp) * t;
    }
    if (((orientation == 1) && (xc1 <= line1)) || ((orientation == 2) && (xc1 >= line1))) {
      double d0 = xc0 - s[2], d1 = xc1 - s[3];
      double t = A.amp * exp(-A.inv_s2ln2 * (d0 * d0 + d1 * d1));
      H = H + t - (H / A.amp) * t;
    }
    if (((orientation == 1) && (xc1 < line0) && (xc1 > line1)) ||
        ((orientation == 2) && (xc1 > line0) && (xc1 < line1))) {
      double d = s[6] * (xc0 - s[0]) + s[7] * (xc1 - s[1]);
      double t = A.amp * exp(-A.inv_s2ln2 * (d * d));
      H = H + t - (H / A.amp) * t;
    }
    (void)theta;
  }
  return H;
}

__global__ void paint_kernel(CanvasView H, const int4* tiles, int off, int cnt, PaintArgs A) {
  for (int t = blockIdx.x; t < cnt; t += gridDim.x) {
    int4 td = tiles[off + t];
    int w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (tx >= w || ty >= h) continue;
    int i = td.x + tx, j = td.y + ty;
    double xc0 = A.xlo0 + A.dx0 * ((double)i + 0.5);
    double xc1 = A.xlo1 + A.dx1 * ((double)j + 0.5);
    double x0 = xc0 - A.pos0, x1 = xc1 - A.pos1;
    double& out = H.at(0, i, j);
    if (A.type == 10) {  // POINT (PULSE) / DRIVEN point
      double v = A.amp * exp(-A.inv_s2ln2 * (x0 * x0 + x1 * x1));
      out = A.mode == 20 ? v * A.drive : v;
    } else if (A.type == 20) {  // SINE
      double d = x0 - A.sine_amp * sin(A.sine_freq * x1);
      out = A.amp * exp(-A.inv_s2ln2 * (d * d));
    } else {  // LIGHTNING
      out = capsule_union(out, xc0, xc1, A);
    }
  }
}

// Overpressure dp (read from H0) -> state at s = 0, c_lr = 0, inverting
// update_state.m4:90-94: dp/c^2 = drho + (gamma-1)/(2 rho0) drho^2; T from
// update_state.m4:103-105; rho*T_n = rho*T (nitrogen mode in equilibrium).
__global__ void overpressure_state_kernel(CanvasView S, CanvasView H, const int4* tiles, int off, int cnt,
                                          double rho0, double c, double gm1_over_2rho0, double p0, double T0,
                                          double R, double c_v) {
  for (int t = blockIdx.x; t < cnt; t += gridDim.x) {
    int4 td = tiles[off + t];
    int w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (tx >= w || ty >= h) continue;
    int i = td.x + tx, j = td.y + ty;
    double dp = H.at(0, i, j);
    double k = gm1_over_2rho0;
    double x = dp / (c * c);
    double drho = (-1.0 + sqrt(1.0 + 4.0 * k * x)) / (2.0 * k);
    double rho = rho0 + drho;
    double T = T0 * exp((0.0 - R * log(rho0 / rho)) / c_v);
    S.at(0, i, j) = rho;
    S.at(1, i, j) = 0.0;
    S.at(2, i, j) = 0.0;
    S.at(3, i, j) = 0.0;
    S.at(4, i, j) = rho * T;
    S.at(5, i, j) = (c * c) * (drho + k * (drho * drho)) + p0;
    S.at(6, i, j) = T;
    H.at(0, i, j) = 0.0;
  }
}

// Block map of tags for regridding: map[by][bx] = 1 if any tagged cell lies
// within `buf` cells of the block (tag buffering folded into the reduction).
__global__ void tag_block_kernel(const int* tags, int nx, int ny, int B, int buf, unsigned char* map, int nbx,
                                 int nby) {
  long n = (long)nbx * nby;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    int bx = (int)(t % nbx), by = (int)(t / nbx);
    int i0 = max(0, bx * B - buf), i1 = min(nx - 1, (bx + 1) * B - 1 + buf);
    int j0 = max(0, by * B - buf), j1 = min(ny - 1, (by + 1) * B - 1 + buf);
    unsigned char any = 0;
    for (int j = j0; j <= j1 && !any; ++j)
      for (int i = i0; i <= i1; ++i)
        if (tags[(long)j * nx + i]) {
          any = 1;
          break;
        }
    map[t] = any;
  }
}

// ---------------------------------------------------------------------------
// Adaptive time step: dt = cfl * dx_min / max over every patch cell of every
// level of max(|u|, |v|) + c (the reference's LLF speed, rhs_hybrid_high_llf
// .m4:270-284, with c_lr = 0).  Block-level max with warp shuffles, one
// 64-bit atomicMax per block (non-negative doubles order like their bits).
// ---------------------------------------------------------------------------
struct SpeedArgs {
  CanvasView lev[kL];
  const int4* tiles;
  const int* ntiles;
  double c;
  unsigned long long* smax_bits;
};

__global__ void speed_kernel(SpeedArgs A) {
  __shared__ double s_w[8];
  const int n = *A.ntiles;
  double m = 0.0;
  for (int t = blockIdx.x; t < n; t += gridDim.x) {
    int4 td = A.tiles[t];
    int lvl = td.z & 0xff, w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (tx < w && ty < h) {
      const CanvasView& V = A.lev[lvl];
      int i = td.x + tx, j = td.y + ty;
      double r = V.at(0, i, j);
      double s = fmax(fabs(V.at(1, i, j) / r), fabs(V.at(2, i, j) / r)) + A.c;
      if (!(s == s)) s = 1e300;  // NaN state: force a tiny dt, health check reports it
      m = fmax(m, s);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? s_w[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) atomicMax(A.smax_bits, (unsigned long long)__double_as_longlong(m));
  }
}

__global__ void dt_kernel(unsigned long long* smax_bits, double* dt, double* time, double cfl_dxmin,
                          double dt_max) {
  double smax = __longlong_as_double((long long)*smax_bits);
  double d = smax > 0.0 ? cfl_dxmin / smax : dt_max;
  *dt = fmin(d, dt_max);
  *time += *dt;
  *smax_bits = 0ull;
}

// Pack / unpack the patch interiors of every level (7 fields) into a dense
// buffer: field k of the cell (tx, ty) of tile t sits at
// k*total + off[t] + ty*w + tx.  Used to exchange the hierarchy state with
// host memory.
struct PackArgs {
  CanvasView lev[kL];
  const int4* tiles;
  const long long* off;
  int ntiles;
  long long total;
  double* packed;
  int unpack;
};

__global__ void pack_kernel(PackArgs A) {
  for (int t = blockIdx.x; t < A.ntiles; t += gridDim.x) {
    int4 td = A.tiles[t];
    int lvl = td.z & 0xff, w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (tx >= w || ty >= h) continue;
    long long o = A.off[t] + ty * w + tx;
    const CanvasView& V = A.lev[lvl];
    for (int k = 0; k < kNF; ++k) {
      double& c = V.at(k, td.x + tx, td.y + ty);
      double& p = A.packed[k * A.total + o];
      if (A.unpack) c = p;
      else p = c;
    }
  }
}

// ---------------------------------------------------------------------------
// Training-data harvest for the learned sensor (hybrid_high_llf, level 0):
// per cell the 40 features, the exact plain switch, and the local difference
// between the DRP and WENO right-hand sides,
//   err = max_k dt |KK_drp,k - KK_weno,k| / scale_k,
// computed in FP64 from the current buffer (ghosts filled by the caller).
// Every WENO-flagged cell is kept; DRP cells are kept with probability
// keep0 (hash of the cell and `seed`).
// ---------------------------------------------------------------------------
struct HarvestArgs {
  CanvasView V;
  CanvasView H;
  RhsConst P;
  float eps, eps_p, inv_sqrt_eps, rho0, p0, T0;
  const int4* tiles;
  int off, cnt;
  double dt;
  double inv_scale[5];
  unsigned keep0, seed;
  __nv_bfloat16* X;
  float* lab;  // (flag, err) per row
  unsigned long long* count;
  long cap;
};

struct CanvasAcc64 {
  const CanvasView* V;
  int i, j;
  __device__ double w(int k, int di, int dj) const { return V->at(k, i + di, j + dj); }
  __device__ double p(int di, int dj) const { return V->at(5, i + di, j + dj); }
  __device__ double t(int di, int dj) const { return V->at(6, i + di, j + dj); }
};
struct CanvasAcc32 {
  const CanvasView* V;
  int i, j;
  double rho0, p0;
  __device__ float w(int k, int di, int dj) const { return (float)(V->at(k, i + di, j + dj) - (k == 0 ? rho0 : 0.0)); }
  __device__ float p(int di, int dj) const { return (float)(V->at(5, i + di, j + dj) - p0); }
};

__global__ void harvest_kernel(HarvestArgs A) {
  for (int t = blockIdx.x; t < A.cnt; t += gridDim.x) {
    int4 td = A.tiles[A.off + t];
    int w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (tx >= w || ty >= h) continue;
    int i = td.x + tx, j = td.y + ty;
    CanvasAcc64 a64{&A.V, i, j};
    int flag = rhs_switch<kHybrid, 5, true>(a64, A.P);
    if (!flag) {
      unsigned hsh = (unsigned)i * 73856093u ^ (unsigned)j * 19349663u ^ A.seed * 83492791u;
      hsh ^= hsh >> 13;
      hsh *= 0x5bd1e995u;
      hsh ^= hsh >> 15;
      if (hsh > A.keep0) continue;
    }
    double H[5], Kd[5], Kw[5];
    H[0] = A.H.at(0, i, j);
    rhs_sources(a64, A.P, H);
    double H2[5] = {H[0], H[1], H[2], H[3], H[4]};
    rhs_fluxes<kHybrid, 5, true>(a64, A.P, j, 0, H, Kd);
    rhs_fluxes<kHybrid, 5, true>(a64, A.P, j, 1, H2, Kw);
    double err = 0.0;
#pragma unroll
    for (int k = 0; k < 5; ++k) err = fmax(err, A.dt * fabs(Kd[k] - Kw[k]) * A.inv_scale[k]);
    unsigned long long idx = atomicAdd(A.count, 1ull);
    if ((long)idx >= A.cap) continue;
    CanvasAcc32 a32{&A.V, i, j, (double)A.rho0, (double)A.p0};
    float fv[kFeat];
    cell_features(a32, A.eps, A.eps_p, A.inv_sqrt_eps, fv);
    for (int q = 0; q < kFeat; ++q) A.X[(long)idx * kFeat + q] = __float2bfloat16_rn(fv[q]);
    A.lab[2 * idx] = (float)flag;
    A.lab[2 * idx + 1] = (float)err;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int launch_rhs_pitched(int variant, const double* w, const double* pres, const double* temp, long pitch,
                       long fstride, const double* H0, double* KK, long opitch, long ofstride, int nx, int ny,
                       const RhsConst& P);

struct Level {
  int nx = 0, ny = 0;
  long pitch = 0, fstride = 0;
  double* buf[3] = {nullptr, nullptr, nullptr};
  double* h0 = nullptr;
  double* kk = nullptr;
  double dx[2] = {0, 0};
  std::vector<int4> patches;
  CUtensorMap tmap[3];
  CanvasView view(int which) const {
    double* b = which < 3 ? buf[which] : h0;
    return CanvasView{b, pitch, fstride, nx, ny};
  }
};

// meta layout (device ints)
enum {
  M_NTILES = 0,
  M_HALO_OFF = 1,      // +level
  M_HALO_CNT = 1 + kL,
  M_CT_OFF = 1 + 2 * kL,
  M_CT_CNT = 1 + 3 * kL,
  M_SIZE = 1 + 4 * kL
};

template <typename T>
struct DevArray {
  T* p = nullptr;
  size_t cap = 0;
  bool ensure(size_t n) {  // returns true if reallocated
    if (n <= cap) return false;
    if (p) cudaFree(p);
    cap = std::max<size_t>(n, 2 * cap);
    cudaMalloc(&p, cap * sizeof(T));
    return true;
  }
  ~DevArray() {
    if (p) cudaFree(p);
  }
};

struct Engine {
  enl_engine_config cfg;
  Level lev[kL];
  // tables
  std::vector<int4> h_tiles;                 // stage tiles, all levels
  std::vector<int> tile_off, tile_cnt;       // per level (in h_tiles)
  std::vector<int4> h_halo;                  // halo segments, all levels
  std::vector<int4> h_ctiles;                // coarsen tiles (coarse index), all fine levels
  std::vector<int4> h_patchtab;              // patch boxes, all levels
  std::vector<int> patch_off, patch_cnt;
  int h_meta[M_SIZE];
  DevArray<int4> d_tiles, d_halo, d_ctiles, d_patchtab;
  int* d_meta = nullptr;
  int* d_counters = nullptr;   // 3 stage counters
  int* d_health = nullptr;
  unsigned long long* d_stats = nullptr;
  cudaGraphExec_t graph = nullptr;
  bool graph_valid = false;
  int* d_tags[kL] = {nullptr, nullptr, nullptr, nullptr};  // tag scratch per level
  unsigned char* d_bmap = nullptr;
  size_t bmap_cap = 0;
  double* d_segs = nullptr;
  size_t segs_cap = 0;
  float* d_mlp = nullptr;    // learned-sensor parameters
  float margin = 0.f;
  int adaptive = 0;          // device-computed dt
  double cfl = 0.5;
  double* d_dt = nullptr;    // [0] = dt of the current step, [1] = simulated time
  int profile = 0;            // time each stage-kernel launch with events
  cudaEvent_t pev[6] = {};
  double prof_ms = 0.0;
  long long prof_launches = 0, prof_cells = 0;
  DevArray<long long> d_tileoff;
  std::vector<long long> h_tileoff;
  double* d_packed = nullptr;
  size_t packed_cap = 0;
  unsigned long long* d_smax = nullptr;
  int nsm = 148;
  int stage_blocks = 0;
  size_t smem_bytes = 0;
};

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

static int make_tmap(CUtensorMap* m, double* base, long pitch, long fstride, int nyc) {
  auto fn = encode_fn();
  if (!fn) return ENL_ERR_CUDA;
  cuuint64_t dims[3] = {(cuuint64_t)pitch, (cuuint64_t)nyc, (cuuint64_t)kNF};
  cuuint64_t strides[2] = {(cuuint64_t)(pitch * 8), (cuuint64_t)(fstride * 8)};
  cuuint32_t box[3] = {(cuuint32_t)kBW, (cuuint32_t)kBH, (cuuint32_t)kNF};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, base, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? ENL_OK : ENL_ERR_CUDA;
}

static void tiles_of_box(int4 b, int level, int pid, std::vector<int4>& out) {
  for (int j = b.z; j <= b.w; j += kTH)
    for (int i = b.x; i <= b.y; i += kTW) {
      int w = std::min(kTW, b.y - i + 1), h = std::min(kTH, b.w - j + 1);
      out.push_back(make_int4(i, j, level | (w << 8) | (h << 16), pid));
    }
}

// Row segments of the cells within distance 3 (Chebyshev) of the patch union,
// inside [0,nx)x[0,ny), not covered by any patch.
static void halo_segments(const std::vector<int4>& P, int nx, int ny, std::vector<int4>& out) {
  std::map<int, std::vector<std::pair<int, int>>> grow, cover;
  for (auto& b : P) {
    for (int j = std::max(0, b.z - 3); j <= std::min(ny - 1, b.w + 3); ++j)
      grow[j].push_back({std::max(0, b.x - 3), std::min(nx - 1, b.y + 3)});
    for (int j = b.z; j <= b.w; ++j) cover[j].push_back({b.x, b.y});
  }
  for (auto& kv : grow) {
    int j = kv.first;
    auto g = kv.second;
    std::sort(g.begin(), g.end());
    std::vector<std::pair<int, int>> gm;  // merged grown intervals
    for (auto& iv : g) {
      if (!gm.empty() && iv.first <= gm.back().second + 1) gm.back().second = std::max(gm.back().second, iv.second);
      else gm.push_back(iv);
    }
    std::vector<std::pair<int, int>> cv;
    auto it = cover.find(j);
    if (it != cover.end()) {
      cv = it->second;
      std::sort(cv.begin(), cv.end());
    }
    for (auto& iv : gm) {
      int a = iv.first;
      for (auto& c : cv) {
        if (c.second < a || c.first > iv.second) continue;
        if (c.first > a) out.push_back(make_int4(j, a, c.first - 1, 0));
        a = std::max(a, c.second + 1);
      }
      if (a <= iv.second) out.push_back(make_int4(j, a, iv.second, 0));
    }
  }
}

static int rebuild_tables(Engine* E) {
  const int nl = E->cfg.nlevels;
  E->h_tiles.clear();
  E->h_halo.clear();
  E->h_ctiles.clear();
  E->h_patchtab.clear();
  E->tile_off.assign(nl, 0);
  E->tile_cnt.assign(nl, 0);
  E->patch_off.assign(nl, 0);
  E->patch_cnt.assign(nl, 0);
  memset(E->h_meta, 0, sizeof(E->h_meta));
  for (int l = 0; l < nl; ++l) {
    E->tile_off[l] = (int)E->h_tiles.size();
    E->patch_off[l] = (int)E->h_patchtab.size();
    int pid = 0;
    for (auto& b : E->lev[l].patches) {
      tiles_of_box(b, l, pid++, E->h_tiles);
      E->h_patchtab.push_back(b);
    }
    E->tile_cnt[l] = (int)E->h_tiles.size() - E->tile_off[l];
    E->patch_cnt[l] = (int)E->h_patchtab.size() - E->patch_off[l];
    E->h_meta[M_HALO_OFF + l] = (int)E->h_halo.size();
    if (l > 0) halo_segments(E->lev[l].patches, E->lev[l].nx, E->lev[l].ny, E->h_halo);
    E->h_meta[M_HALO_CNT + l] = (int)E->h_halo.size() - E->h_meta[M_HALO_OFF + l];
    E->h_meta[M_CT_OFF + l] = (int)E->h_ctiles.size();
    if (l > 0) {
      int r = E->cfg.ratio;
      for (auto& b : E->lev[l].patches) {
        int4 cb = make_int4(b.x / r, (b.y + 1) / r - 1, b.z / r, (b.w + 1) / r - 1);
        tiles_of_box(cb, l, 0, E->h_ctiles);
      }
    }
    E->h_meta[M_CT_CNT + l] = (int)E->h_ctiles.size() - E->h_meta[M_CT_OFF + l];
  }
  E->h_meta[M_NTILES] = (int)E->h_tiles.size();
  E->h_tileoff.resize(E->h_tiles.size());
  long long acc = 0;
  for (size_t q = 0; q < E->h_tiles.size(); ++q) {
    E->h_tileoff[q] = acc;
    int4 td = E->h_tiles[q];
    acc += (long long)((td.z >> 8) & 0xff) * ((td.z >> 16) & 0xff);
  }
  E->d_tileoff.ensure(std::max<size_t>(E->h_tileoff.size(), 1));
  if (!E->h_tileoff.empty())
    cudaMemcpyAsync(E->d_tileoff.p, E->h_tileoff.data(), E->h_tileoff.size() * sizeof(long long),
                    cudaMemcpyHostToDevice, stream());
  bool grew = false;
  grew |= E->d_tiles.ensure(std::max<size_t>(E->h_tiles.size(), 1));
  grew |= E->d_halo.ensure(std::max<size_t>(E->h_halo.size(), 1));
  grew |= E->d_ctiles.ensure(std::max<size_t>(E->h_ctiles.size(), 1));
  grew |= E->d_patchtab.ensure(std::max<size_t>(E->h_patchtab.size(), 1));
  if (grew) E->graph_valid = false;
  cudaStream_t s = stream();
  if (!E->h_tiles.empty())
    cudaMemcpyAsync(E->d_tiles.p, E->h_tiles.data(), E->h_tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, s);
  if (!E->h_halo.empty())
    cudaMemcpyAsync(E->d_halo.p, E->h_halo.data(), E->h_halo.size() * sizeof(int4), cudaMemcpyHostToDevice, s);
  if (!E->h_ctiles.empty())
    cudaMemcpyAsync(E->d_ctiles.p, E->h_ctiles.data(), E->h_ctiles.size() * sizeof(int4), cudaMemcpyHostToDevice,
                    s);
  if (!E->h_patchtab.empty())
    cudaMemcpyAsync(E->d_patchtab.p, E->h_patchtab.data(), E->h_patchtab.size() * sizeof(int4),
                    cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(E->d_meta, E->h_meta, sizeof(E->h_meta), cudaMemcpyHostToDevice, s);
  // the host vectors are reused; wait so they are not modified under the copy
  cudaStreamSynchronize(s);
  return check_launch("engine tables");
}

static StageArgs stage_args(Engine* E, int stage, double dt) {
  StageArgs A;
  memset(&A, 0, sizeof(A));
  const auto& c = E->cfg;
  int in = stage == 0 ? 0 : stage;          // cur, S0, S1
  int out = stage == 2 ? 0 : stage + 1;     // S0, S1, cur
  for (int l = 0; l < c.nlevels; ++l) {
    Level& L = E->lev[l];
    A.tmap[l] = L.tmap[in];
    A.in[l] = L.buf[in];
    A.out[l] = L.buf[out];
    A.un[l] = L.buf[0];
    A.h0[l] = L.h0;
    A.pitch[l] = L.pitch;
    A.fstride[l] = L.fstride;
    double xlo[2] = {c.xlo[0], c.xlo[1]};
    A.P[l] = make_rhs_const(xlo, L.dx, c.weno_alpha, c.kappa, c.mu, c.muB, c.R, c.T_star_n, c.tau_n, c.tol, l, c.c,
                            c.c_lr);
    const RhsConst& P = A.P[l];
    FastConst F;
    F.inv_dx0 = (float)P.inv_dx0;
    F.inv_dx1 = (float)P.inv_dx1;
    F.inv_dx0sq = (float)P.inv_dx0sq;
    F.inv_dx1sq = (float)P.inv_dx1sq;
    F.inv_2dx0 = (float)P.inv_2dx0;
    F.inv_2dx1 = (float)P.inv_2dx1;
    F.inv_4dxdy = (float)P.inv_4dxdy;
    F.kappa = (float)c.kappa;
    F.mu = (float)c.mu;
    F.muB = (float)c.muB;
    F.R078 = (float)(Lit::c0_78 * c.R);
    F.T_star_n = (float)c.T_star_n;
    F.inv_tau_n = (float)(1.0 / c.tau_n);
    F.alpha = (float)c.weno_alpha;
    F.c = (float)c.c;
    F.c_lr = (float)c.c_lr;
    F.ylo = (float)c.xlo[1];
    F.dy = (float)L.dx[1];
    F.sensor_eps = (float)P.sensor_eps;
    F.rho0 = (float)c.rho0;
    F.T0 = (float)c.T0;
    F.level = l;
    A.F[l] = F;
    A.dy[l] = L.dx[1];
  }
  A.rho0 = c.rho0;
  A.p0 = c.p0;
  A.T0 = c.T0;
  A.c = c.c;
  A.c_lr = c.c_lr;
  A.gm1_over_2rho0 = (c.gamma1 - 1.0) / (2.0 * c.rho0);
  A.c_p = c.c_p;
  A.c_v = c.c_v;
  A.R = c.R;
  A.ylo = c.xlo[1];
  A.a1 = c.rk_alpha1[stage];
  A.a2 = c.rk_alpha2[stage];
  A.bdt = c.rk_beta[stage] * dt;
  A.beta = c.rk_beta[stage];
  A.dt_dev = E->adaptive ? E->d_dt : nullptr;
  A.tiles = E->d_tiles.p;
  A.ntiles = E->d_meta + M_NTILES;
  A.counter = E->d_counters + stage;
  A.health = E->d_health;
  A.stats = E->d_stats;
  A.mlp = (E->cfg.learned && E->cfg.precision == ENL_PREC_FP32) ? E->d_mlp : nullptr;
  A.margin = E->margin;
  A.feat_eps = (float)A.P[0].sensor_eps;
  A.feat_eps_p = (float)(A.P[0].sensor_eps * (c.c * c.c) * (c.c * c.c));
  A.feat_inv_sqrt_eps = (float)(1.0 / sqrt(A.P[0].sensor_eps));
  return A;
}

typedef void (*StageFn)(StageArgs);

template <bool FAST>
static StageFn pick_stage(int variant) {
  switch (variant) {
    case 0: return stage_kernel<kHybrid, 5, true, FAST>;
    case 1: return stage_kernel<kHybrid, 5, false, FAST>;
    case 2: return stage_kernel<kHybrid, 3, true, FAST>;
    case 3: return stage_kernel<kHybrid, 3, false, FAST>;
    case 4: return stage_kernel<kWeno, 5, true, FAST>;
    case 5: return stage_kernel<kWeno, 5, false, FAST>;
    case 6: return stage_kernel<kWeno, 3, true, FAST>;
    case 7: return stage_kernel<kWeno, 3, false, FAST>;
    default: return stage_kernel<kDrp, 5, false, FAST>;
  }
}

static int fill_level(Engine* E, int l, int which) {
  cudaStream_t s = stream();
  const auto& c = E->cfg;
  Level& L = E->lev[l];
  if (l > 0) {
    interp_kernel<<<E->nsm * 4, 256, 0, s>>>(L.view(which), E->lev[l - 1].view(which), c.ratio, E->d_halo.p,
                                             E->d_meta, M_HALO_OFF + l, M_HALO_CNT + l, kNF);
  }
  if (c.independent) {
    if (E->patch_cnt[l])
      physbc_patches_kernel<<<E->patch_cnt[l], 256, 0, s>>>(L.view(which), E->d_patchtab.p, E->patch_off[l],
                                                            E->patch_cnt[l], c.bc[0], c.bc[1], c.bc[2], c.bc[3]);
  } else {
    physbc_kernel<<<E->nsm * 2, 256, 0, s>>>(L.view(which), kNF, c.bc[0], c.bc[1], c.bc[2], c.bc[3]);
  }
  return ENL_OK;
}

static int fill_all(Engine* E, int which) {
  for (int l = 0; l < E->cfg.nlevels; ++l) fill_level(E, l, which);
  return check_launch("fill");
}

static int absorb_all(Engine* E, int which) {
  const auto& c = E->cfg;
  if (!(c.bc[0] == kAbsorb || c.bc[1] == kAbsorb || c.bc[2] == kAbsorb || c.bc[3] == kAbsorb)) return ENL_OK;
  cudaStream_t s = stream();
  for (int l = 0; l < c.nlevels; ++l) {
    Level& L = E->lev[l];
    if (E->patch_cnt[l] == 0) continue;
    AbsorbArgs A{L.dx[0], L.dx[1], c.xlo[0], c.xlo[1], c.xlo[0] + L.dx[0] * L.nx, c.xlo[1] + L.dx[1] * L.ny,
                 c.absorb_width * c.absorb_width, c.p0, c.T0, c.rho0};
    long rows = 0, cols = 0;
    for (int q = 0; q < E->patch_cnt[l]; ++q) {
      int4 b = E->h_patchtab[E->patch_off[l] + q];
      rows += b.w - b.z + 1;
      cols += b.y - b.x + 1;
    }
    for (int dir = 0; dir < 4; ++dir) {
      if (c.bc[dir] != kAbsorb) continue;
      long n = dir < 2 ? rows : cols;
      absorb_patches_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(L.view(which), E->d_patchtab.p,
                                                                       E->patch_off[l], E->patch_cnt[l], dir, A);
    }
  }
  return check_launch("absorb");
}

static int coarsen_all(Engine* E) {
  cudaStream_t s = stream();
  for (int l = E->cfg.nlevels - 1; l > 0; --l)
    coarsen_kernel<<<E->nsm * 4, 256, 0, s>>>(E->lev[l - 1].view(0), E->lev[l].view(0), E->cfg.ratio, E->d_ctiles.p,
                                             E->d_meta, M_CT_OFF + l, M_CT_CNT + l);
  return check_launch("coarsen");
}

static double finest_dx(Engine* E) {
  const Level& L = E->lev[E->cfg.nlevels - 1];
  return L.dx[0] < L.dx[1] ? L.dx[0] : L.dx[1];
}

static void adaptive_dt(Engine* E, double dt_max) {
  if (!E->adaptive) return;
  SpeedArgs S;
  memset(&S, 0, sizeof(S));
  for (int l = 0; l < E->cfg.nlevels; ++l) S.lev[l] = E->lev[l].view(0);
  S.tiles = E->d_tiles.p;
  S.ntiles = E->d_meta + M_NTILES;
  S.c = E->cfg.c;
  S.smax_bits = E->d_smax;
  speed_kernel<<<E->nsm * 4, 256, 0, stream()>>>(S);
  dt_kernel<<<1, 1, 0, stream()>>>(E->d_smax, E->d_dt, E->d_dt + 1, E->cfl * finest_dx(E), dt_max);
}

static int step_fused(Engine* E, double dt) {
  cudaStream_t s = stream();
  cudaMemsetAsync(E->d_counters, 0, 3 * sizeof(int), s);
  adaptive_dt(E, dt);
  StageFn fn = E->cfg.precision == ENL_PREC_FP32 ? pick_stage<true>(E->cfg.variant) : pick_stage<false>(E->cfg.variant);
  for (int st = 0; st < 3; ++st) {
    int in = st == 0 ? 0 : st;
    int out = st == 2 ? 0 : st + 1;
    fill_all(E, in);
    StageArgs A = stage_args(E, st, dt);
    void* args[] = {&A};
    if (E->profile) cudaEventRecord(E->pev[2 * st], s);
    cudaLaunchKernel((const void*)fn, dim3(E->stage_blocks), dim3(256), args, E->smem_bytes, s);
    if (E->profile) cudaEventRecord(E->pev[2 * st + 1], s);
    absorb_all(E, out);
  }
  coarsen_all(E);
  if (E->profile) {
    cudaEventSynchronize(E->pev[5]);
    long long cells = 0;
    for (auto& td : E->h_tiles) cells += (long long)((td.z >> 8) & 0xff) * ((td.z >> 16) & 0xff);
    for (int st = 0; st < 3; ++st) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, E->pev[2 * st], E->pev[2 * st + 1]);
      E->prof_ms += ms;
      E->prof_launches += 1;
      E->prof_cells += cells;
    }
  }
  return check_launch("engine step");
}

static int step_plain(Engine* E, double dt) {
  cudaStream_t s = stream();
  const auto& c = E->cfg;
  const int nl = c.nlevels;
  adaptive_dt(E, dt);
  // copy current -> scratch (patch interiors)
  for (int l = 0; l < nl; ++l)
    if (E->tile_cnt[l])
      copy_tiles_kernel<<<E->tile_cnt[l], 256, 0, s>>>(E->lev[l].view(1), E->lev[l].view(0), E->d_tiles.p,
                                                       E->tile_off[l], E->tile_cnt[l]);
  for (int st = 0; st < 3; ++st) {
    fill_all(E, 1);
    // rhs of every patch first (each patch reads its neighbours' cells as
    // ghosts, which SAMRAI copied before the stage), then the updates
    for (int l = 0; l < nl; ++l) {
      Level& L = E->lev[l];
      double xlo[2] = {c.xlo[0], c.xlo[1]};
      RhsConst P = make_rhs_const(xlo, L.dx, c.weno_alpha, c.kappa, c.mu, c.muB, c.R, c.T_star_n, c.tau_n, c.tol, l,
                                  c.c, c.c_lr);
      for (auto& b : L.patches) {
        int nx = b.y - b.x + 1, ny = b.w - b.z + 1;
        long g0 = (long)(b.z) * L.pitch + b.x;  // canvas offset of cell (ilo-3, jlo-3)
        long c0 = (long)(b.z + 3) * L.pitch + (b.x + 3);
        // the plain kernel computes the LLF height from the row inside the
        // patch; shift ylo to the patch's lower edge
        RhsConst Pp = P;
        Pp.ylo = c.xlo[1] + L.dx[1] * (double)b.z;
        launch_rhs_pitched(c.variant, L.buf[1] + g0, L.buf[1] + 5 * L.fstride + g0, L.buf[1] + 6 * L.fstride + g0,
                           L.pitch, L.fstride, L.h0 + c0, L.kk + c0, L.pitch, L.fstride, nx, ny, Pp);
      }
    }
    for (int l = 0; l < nl; ++l) {
      Level& L = E->lev[l];
      EosArgs Ea{c.rho0, c.c, (c.gamma1 - 1.0) / (2.0 * c.rho0), c.c_p, c.p0, c.T0, c.c_lr, c.c_v, c.R, c.xlo[1],
                 L.dx[1]};
      CanvasView K{L.kk, L.pitch, L.fstride, L.nx, L.ny};
      for (auto& b : L.patches) {
        int nx = b.y - b.x + 1, ny = b.w - b.z + 1;
        dim3 blk(32, 4), grd((nx + 31) / 32, (ny + 3) / 4);
        rk_plain_kernel<<<grd, blk, 0, s>>>(L.view(1), L.view(0), K, b.x, b.z, nx, ny, c.rk_alpha1[st],
                                            c.rk_alpha2[st], c.rk_beta[st] * dt, c.rk_beta[st],
                                            E->adaptive ? E->d_dt : nullptr);
        eos_plain_kernel<<<grd, blk, 0, s>>>(L.view(1), b.x, b.z, nx, ny, Ea);
      }
    }
    absorb_all(E, 1);
  }
  for (int l = 0; l < nl; ++l)
    if (E->tile_cnt[l])
      copy_tiles_kernel<<<E->tile_cnt[l], 256, 0, s>>>(E->lev[l].view(0), E->lev[l].view(1), E->d_tiles.p,
                                                       E->tile_off[l], E->tile_cnt[l]);
  coarsen_all(E);
  return check_launch("engine plain step");
}

}  // namespace enl

using namespace enl;

extern "C" {

int enl_engine_create(const enl_engine_config* cfg, void** out) {
  if (!cfg || !out || cfg->nlevels < 1 || cfg->nlevels > kL || cfg->ratio < 2 || cfg->nx0 < 8 || cfg->ny0 < 8 ||
      cfg->variant < 0 || cfg->variant > 8 ||
      (cfg->independent && (cfg->nlevels != 1 || cfg->bc[0] == kAbsorb || cfg->bc[1] == kAbsorb ||
                            cfg->bc[2] == kAbsorb || cfg->bc[3] == kAbsorb))) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  Engine* E = new Engine();
  E->cfg = *cfg;
  cudaDeviceGetAttribute(&E->nsm, cudaDevAttrMultiProcessorCount, 0);
  int rr = 1;
  for (int l = 0; l < cfg->nlevels; ++l) {
    Level& L = E->lev[l];
    L.nx = cfg->nx0 * rr;
    L.ny = cfg->ny0 * rr;
    L.dx[0] = cfg->dx0[0] / rr;
    L.dx[1] = cfg->dx0[1] / rr;
    L.pitch = ((L.nx + 6 + 15) / 16) * 16;
    long rows = L.ny + 6;
    L.fstride = ((L.pitch * rows + 31) / 32) * 32;
    size_t bytes = (size_t)L.fstride * kNF * sizeof(double);
    for (int b = 0; b < 3; ++b) {
      if (cudaMalloc(&L.buf[b], bytes) != cudaSuccess) {
        set_error(ENL_ERR_CUDA);
        enl_engine_destroy(E);
        return ENL_ERR_CUDA;
      }
      cudaMemset(L.buf[b], 0, bytes);
      if (make_tmap(&L.tmap[b], L.buf[b], L.pitch, L.fstride, (int)rows) != ENL_OK) {
        set_error(ENL_ERR_CUDA);
        enl_engine_destroy(E);
        return ENL_ERR_CUDA;
      }
    }
    cudaMalloc(&L.h0, (size_t)L.fstride * sizeof(double));
    cudaMemset(L.h0, 0, (size_t)L.fstride * sizeof(double));
    rr *= cfg->ratio;
  }
  cudaMalloc(&E->d_meta, sizeof(E->h_meta));
  cudaMemset(E->d_meta, 0, sizeof(E->h_meta));
  cudaMalloc(&E->d_counters, 4 * sizeof(int));
  cudaMalloc(&E->d_health, sizeof(int));
  cudaMemset(E->d_health, 0, sizeof(int));
  cudaMalloc(&E->d_stats, 3 * kL * sizeof(unsigned long long));
  cudaMemset(E->d_stats, 0, 3 * kL * sizeof(unsigned long long));
  cudaMalloc(&E->d_dt, 2 * sizeof(double));
  cudaMemset(E->d_dt, 0, 2 * sizeof(double));
  cudaMalloc(&E->d_smax, sizeof(unsigned long long));
  cudaMemset(E->d_smax, 0, sizeof(unsigned long long));
  E->smem_bytes = 2 * kStageBufBytes + (cfg->precision == ENL_PREC_FP32 ? kTile32Bytes : 0);
  if (cfg->precision == ENL_PREC_FP32 && cfg->learned)
    E->smem_bytes += align128((int)sizeof(MlpSmem)) + 256 * kFeat * sizeof(__nv_bfloat16);
  StageFn fn = cfg->precision == ENL_PREC_FP32 ? pick_stage<true>(cfg->variant) : pick_stage<false>(cfg->variant);
  cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)E->smem_bytes);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)fn, 256, E->smem_bytes);
  E->stage_blocks = E->nsm * std::max(1, per_sm);
  E->tile_off.assign(cfg->nlevels, 0);
  E->tile_cnt.assign(cfg->nlevels, 0);
  E->patch_off.assign(cfg->nlevels, 0);
  E->patch_cnt.assign(cfg->nlevels, 0);
  if (check_launch("engine create") != ENL_OK) {
    enl_engine_destroy(E);
    return ENL_ERR_CUDA;
  }
  *out = E;
  return ENL_OK;
}

int enl_engine_destroy(void* e) {
  Engine* E = (Engine*)e;
  if (!E) return ENL_OK;
  for (int l = 0; l < kL; ++l) {
    for (int b = 0; b < 3; ++b)
      if (E->lev[l].buf[b]) cudaFree(E->lev[l].buf[b]);
    if (E->lev[l].h0) cudaFree(E->lev[l].h0);
    if (E->lev[l].kk) cudaFree(E->lev[l].kk);
  }
  if (E->d_meta) cudaFree(E->d_meta);
  if (E->d_counters) cudaFree(E->d_counters);
  if (E->d_health) cudaFree(E->d_health);
  if (E->d_stats) cudaFree(E->d_stats);
  for (int l = 0; l < kL; ++l)
    if (E->d_tags[l]) cudaFree(E->d_tags[l]);
  if (E->d_bmap) cudaFree(E->d_bmap);
  if (E->d_dt) cudaFree(E->d_dt);
  if (E->d_mlp) cudaFree(E->d_mlp);
  if (E->d_packed) cudaFree(E->d_packed);
  for (int q = 0; q < 6; ++q)
    if (E->pev[q]) cudaEventDestroy(E->pev[q]);
  if (E->d_smax) cudaFree(E->d_smax);
  if (E->d_segs) cudaFree(E->d_segs);
  if (E->graph) cudaGraphExecDestroy(E->graph);
  delete E;
  return ENL_OK;
}

int enl_engine_buffer(void* e, int level, int which, double** base, long* pitch, long* fstride, int* nx, int* ny) {
  Engine* E = (Engine*)e;
  if (!E || level < 0 || level >= E->cfg.nlevels || which < 0 || which > 3) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  Level& L = E->lev[level];
  if (base) *base = which < 3 ? L.buf[which] : L.h0;
  if (pitch) *pitch = L.pitch;
  if (fstride) *fstride = L.fstride;
  if (nx) *nx = L.nx;
  if (ny) *ny = L.ny;
  return ENL_OK;
}

int enl_engine_set_patches(void* e, int level, int npatch, const int* boxes) {
  Engine* E = (Engine*)e;
  if (!E || level < 0 || level >= E->cfg.nlevels || npatch < 0 || (npatch > 0 && !boxes)) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  Level& L = E->lev[level];
  std::vector<int4> P;
  for (int q = 0; q < npatch; ++q) {
    int4 b = make_int4(boxes[4 * q], boxes[4 * q + 1], boxes[4 * q + 2], boxes[4 * q + 3]);
    if (b.x < 0 || b.z < 0 || b.y >= L.nx || b.w >= L.ny || b.y < b.x || b.w < b.z || (b.x & 1)) {
      set_error(ENL_ERR_ARG);
      return ENL_ERR_ARG;
    }
    P.push_back(b);
  }
  L.patches = P;
  return rebuild_tables(E);
}

int enl_engine_refine_init(void* e, int level, int nbox, const int* boxes) {
  Engine* E = (Engine*)e;
  if (!E || level < 1 || level >= E->cfg.nlevels || nbox < 0 || (nbox > 0 && !boxes)) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  cudaStream_t s = stream();
  Level& L = E->lev[level];
  for (int q = 0; q < nbox; ++q) {
    int ilo = boxes[4 * q], ihi = boxes[4 * q + 1], jlo = boxes[4 * q + 2], jhi = boxes[4 * q + 3];
    if (ilo < 0 || jlo < 0 || ihi >= L.nx || jhi >= L.ny || ihi < ilo || jhi < jlo) {
      set_error(ENL_ERR_ARG);
      return ENL_ERR_ARG;
    }
    long n = (long)(ihi - ilo + 1) * (jhi - jlo + 1);
    refine_box_kernel<<<(unsigned)std::min<long>((n + 255) / 256, 4096), 256, 0, s>>>(
        L.view(0), E->lev[level - 1].view(0), E->cfg.ratio, ilo, jlo, ihi - ilo + 1, jhi - jlo + 1);
  }
  return check_launch("refine_init");
}

int enl_engine_fill(void* e, int which) {
  Engine* E = (Engine*)e;
  if (!E || which < 0 || which > 2) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  return fill_all(E, which);
}

int enl_engine_step(void* e, double dt) {
  Engine* E = (Engine*)e;
  if (!E) return ENL_ERR_ARG;
  if (E->h_tiles.empty()) {
    set_error(ENL_ERR_STATE);
    return ENL_ERR_STATE;
  }
  return step_fused(E, dt);
}

int enl_engine_step_plain(void* e, double dt) {
  Engine* E = (Engine*)e;
  if (!E) return ENL_ERR_ARG;
  if (E->h_tiles.empty()) {
    set_error(ENL_ERR_STATE);
    return ENL_ERR_STATE;
  }
  for (int l = 0; l < E->cfg.nlevels; ++l) {
    Level& L = E->lev[l];
    if (!L.kk) {
      if (cudaMalloc(&L.kk, (size_t)L.fstride * 5 * sizeof(double)) != cudaSuccess) {
        set_error(ENL_ERR_CUDA);
        return ENL_ERR_CUDA;
      }
      cudaMemset(L.kk, 0, (size_t)L.fstride * 5 * sizeof(double));
    }
  }
  return step_plain(E, dt);
}

int enl_engine_graph_capture(void* e, double dt) {
  Engine* E = (Engine*)e;
  if (!E || E->h_tiles.empty()) {
    set_error(ENL_ERR_STATE);
    return ENL_ERR_STATE;
  }
  cudaStream_t s = stream();
  if (s == nullptr) {  // capture needs a non-legacy stream
    set_error(ENL_ERR_STATE);
    return ENL_ERR_STATE;
  }
  cudaGraph_t g;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  step_fused(E, dt);
  if (cudaStreamEndCapture(s, &g) != cudaSuccess) {
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  if (E->graph) cudaGraphExecDestroy(E->graph);
  E->graph = nullptr;
  cudaError_t r = cudaGraphInstantiate(&E->graph, g, 0);
  cudaGraphDestroy(g);
  if (r != cudaSuccess) {
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  E->graph_valid = true;
  return ENL_OK;
}

int enl_engine_graph_replay(void* e, int nsteps) {
  Engine* E = (Engine*)e;
  if (!E || !E->graph || !E->graph_valid) {
    set_error(ENL_ERR_STATE);
    return ENL_ERR_STATE;
  }
  cudaStream_t s = stream();
  for (int k = 0; k < nsteps; ++k)
    if (cudaGraphLaunch(E->graph, s) != cudaSuccess) {
      set_error(ENL_ERR_CUDA);
      return ENL_ERR_CUDA;
    }
  return ENL_OK;
}

int enl_engine_tag(void* e, int level, int* tags) {
  Engine* E = (Engine*)e;
  if (!E || level < 0 || level >= E->cfg.nlevels || !tags) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  cudaStream_t s = stream();
  Level& L = E->lev[level];
  fill_all(E, 0);
  // source ghosts: the same physical rule on the H0 canvas (one field)
  physbc_kernel<<<E->nsm, 256, 0, s>>>(L.view(3), 1, E->cfg.bc[0], E->cfg.bc[1], E->cfg.bc[2], E->cfg.bc[3]);
  cudaMemsetAsync(tags, 0, (size_t)L.nx * L.ny * sizeof(int), s);
  const double xi = 1.0;
  const double* tol = E->cfg.tol;
  double ep0 = ((Lit::c0_9 * tol[0]) * (xi * xi)) / (1.0 - Lit::c0_9 * (tol[0] * tol[0]));
  double ep1 = ((Lit::c0_9 * tol[1]) * (xi * xi)) / (1.0 - Lit::c0_9 * (tol[1] * tol[1]));
  if (E->tile_cnt[level])
    tag_tiles_kernel<<<E->tile_cnt[level], 256, 0, s>>>(tags, L.view(0), L.view(3), E->d_tiles.p, E->tile_off[level],
                                                        E->tile_cnt[level], ep0, ep1);
  return check_launch("engine tag");
}

int enl_engine_stats(void* e, long long* counts) {
  Engine* E = (Engine*)e;
  if (!E || !counts) return ENL_ERR_ARG;
  unsigned long long h[3 * kL];
  cudaMemcpyAsync(h, E->d_stats, sizeof(h), cudaMemcpyDeviceToHost, stream());
  cudaStreamSynchronize(stream());
  for (int q = 0; q < 3 * kL; ++q) counts[q] = (long long)h[q];
  cudaMemsetAsync(E->d_stats, 0, sizeof(h), stream());
  return check_launch("engine stats");
}

int enl_engine_health(void* e) {
  Engine* E = (Engine*)e;
  if (!E) return ENL_ERR_ARG;
  int h = 0;
  cudaMemcpyAsync(&h, E->d_health, sizeof(int), cudaMemcpyDeviceToHost, stream());
  cudaStreamSynchronize(stream());
  cudaMemsetAsync(E->d_health, 0, sizeof(int), stream());
  return h;
}

int enl_engine_launches_per_step(void* e, int plain) {
  Engine* E = (Engine*)e;
  if (!E) return -1;
  const auto& c = E->cfg;
  int nl = c.nlevels;
  int fills = nl + (nl - 1);  // physbc per level + interp per fine level
  int nabs = 0;
  for (int d = 0; d < 4; ++d) nabs += c.bc[d] == kAbsorb;
  int absorbs = 0;
  for (int l = 0; l < nl; ++l) absorbs += E->patch_cnt[l] ? nabs : 0;
  if (!plain) return 3 * (fills + 1 + absorbs) + (nl - 1);
  int npatch = 0, copies = 0;
  for (int l = 0; l < nl; ++l) {
    npatch += (int)E->lev[l].patches.size();
    copies += E->tile_cnt[l] ? 1 : 0;
  }
  return 3 * (fills + 3 * npatch + absorbs) + 2 * copies + (nl - 1);
}

int enl_engine_paint_source(void* e, int level, int type, int mode, double amp, double spread, const double* pos,
                            double sine_amp, double sine_freq, int nseg, const double* segs, double drive) {
  Engine* E = (Engine*)e;
  if (!E || level < 0 || level >= E->cfg.nlevels || !(type == 10 || type == 20 || type == 30) ||
      !(mode == 10 || mode == 20) || spread <= 0 || (type == 30 && (nseg < 0 || (nseg > 0 && !segs))) ||
      (type != 30 && !pos)) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  cudaStream_t s = stream();
  Level& L = E->lev[level];
  PaintArgs A;
  memset(&A, 0, sizeof(A));
  A.type = type;
  A.mode = mode;
  A.amp = amp;
  A.inv_s2ln2 = log(2.0) / (spread * spread);
  if (pos) {
    A.pos0 = pos[0];
    A.pos1 = pos[1];
  }
  A.sine_amp = sine_amp;
  A.sine_freq = sine_freq;
  A.drive = drive;
  A.xlo0 = E->cfg.xlo[0];
  A.xlo1 = E->cfg.xlo[1];
  A.dx0 = L.dx[0];
  A.dx1 = L.dx[1];
  if (type == 30 && nseg > 0) {
    size_t need = (size_t)nseg * kSegStride;
    std::vector<double> pre(need);
    const double PI_ = 3.14159265358979323846264338;
    // exp(-ln2 d^2/spread^2) underflows to 0 beyond d = 32.8 spread
    const double cull = 40.0 * spread;
    for (int k = 0; k < nseg; ++k) {
      const double* c = segs + 4 * k;
      double* o = pre.data() + (size_t)kSegStride * k;
      double theta = -atan((c[3] - c[1]) / (c[2] - c[0]));
      int orientation = 0;
      if (((c[0] > c[2]) && (c[1] > c[3])) || ((c[0] <= c[2]) && (c[1] >= c[3]))) orientation = 1;
      else if (((c[0] >= c[2]) && (c[1] <= c[3])) || ((c[0] < c[2]) && (c[1] < c[3]))) orientation = 2;
      o[0] = c[0];
      o[1] = c[1];
      o[2] = c[2];
      o[3] = c[3];
      o[4] = theta;
      o[5] = tan(PI_ / 2.0 - theta);
      o[6] = sin(theta);
      o[7] = cos(theta);
      o[8] = orientation;
      o[9] = std::min(c[0], c[2]) - cull;
      o[10] = std::max(c[0], c[2]) + cull;
      o[11] = std::min(c[1], c[3]) - cull;
      o[12] = std::max(c[1], c[3]) + cull;
    }
    if (need > E->segs_cap) {
      if (E->d_segs) cudaFree(E->d_segs);
      if (cudaMalloc(&E->d_segs, need * sizeof(double)) != cudaSuccess) {
        E->d_segs = nullptr;
        E->segs_cap = 0;
        set_error(ENL_ERR_CUDA);
        return ENL_ERR_CUDA;
      }
      E->segs_cap = need;
    }
    cudaMemcpyAsync(E->d_segs, pre.data(), need * sizeof(double), cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
    A.segs = E->d_segs;
    A.nseg = nseg;
  }
  if (E->tile_cnt[level])
    paint_kernel<<<E->tile_cnt[level], 256, 0, s>>>(L.view(3), E->d_tiles.p, E->tile_off[level], E->tile_cnt[level],
                                                    A);
  return check_launch("paint_source");
}

int enl_engine_state_from_overpressure(void* e, int level) {
  Engine* E = (Engine*)e;
  if (!E || level < 0 || level >= E->cfg.nlevels) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  const auto& c = E->cfg;
  Level& L = E->lev[level];
  if (E->tile_cnt[level])
    overpressure_state_kernel<<<E->tile_cnt[level], 256, 0, stream()>>>(
        L.view(0), L.view(3), E->d_tiles.p, E->tile_off[level], E->tile_cnt[level], c.rho0, c.c,
        (c.gamma1 - 1.0) / (2.0 * c.rho0), c.p0, c.T0, c.R, c.c_v);
  return check_launch("state_from_overpressure");
}

int enl_engine_tag_blocks(void* e, int level, int block, int buffer, unsigned char* map_host, int* nbx_out,
                          int* nby_out) {
  Engine* E = (Engine*)e;
  if (!E || level < 0 || level >= E->cfg.nlevels || block < 1 || buffer < 0) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  Level& L = E->lev[level];
  int nbx = (L.nx + block - 1) / block, nby = (L.ny + block - 1) / block;
  if (nbx_out) *nbx_out = nbx;
  if (nby_out) *nby_out = nby;
  if (!map_host) return ENL_OK;  // size query
  cudaStream_t s = stream();
  if (!E->d_tags[level]) {
    if (cudaMalloc(&E->d_tags[level], (size_t)L.nx * L.ny * sizeof(int)) != cudaSuccess) {
      E->d_tags[level] = nullptr;
      set_error(ENL_ERR_CUDA);
      return ENL_ERR_CUDA;
    }
  }
  size_t nb = (size_t)nbx * nby;
  if (nb > E->bmap_cap) {
    if (E->d_bmap) cudaFree(E->d_bmap);
    if (cudaMalloc(&E->d_bmap, nb) != cudaSuccess) {
      E->d_bmap = nullptr;
      E->bmap_cap = 0;
      set_error(ENL_ERR_CUDA);
      return ENL_ERR_CUDA;
    }
    E->bmap_cap = nb;
  }
  int st = enl_engine_tag(e, level, E->d_tags[level]);
  if (st != ENL_OK) return st;
  tag_block_kernel<<<E->nsm * 4, 256, 0, s>>>(E->d_tags[level], L.nx, L.ny, block, buffer, E->d_bmap, nbx, nby);
  cudaMemcpyAsync(map_host, E->d_bmap, nb, cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  return check_launch("tag_blocks");
}

int enl_engine_set_adaptive_dt(void* e, int on, double cfl) {
  Engine* E = (Engine*)e;
  if (!E || cfl <= 0.0 || cfl >= 1.0) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  E->adaptive = on ? 1 : 0;
  E->cfl = cfl;
  E->graph_valid = false;  // kernel arguments change
  return ENL_OK;
}

int enl_engine_time(void* e, double* dt_last, double* sim_time) {
  Engine* E = (Engine*)e;
  if (!E) return ENL_ERR_ARG;
  double h[2];
  cudaMemcpyAsync(h, E->d_dt, sizeof(h), cudaMemcpyDeviceToHost, stream());
  cudaStreamSynchronize(stream());
  if (dt_last) *dt_last = h[0];
  if (sim_time) *sim_time = h[1];
  return check_launch("engine time");
}

static long long packed_cells(Engine* E) {
  if (E->h_tiles.empty()) return 0;
  int4 td = E->h_tiles.back();
  return E->h_tileoff.back() + (long long)((td.z >> 8) & 0xff) * ((td.z >> 16) & 0xff);
}

int enl_engine_packed_size(void* e, long long* ndoubles) {
  Engine* E = (Engine*)e;
  if (!E || !ndoubles) return ENL_ERR_ARG;
  *ndoubles = packed_cells(E) * kNF;
  return ENL_OK;
}

static int pack_common(Engine* E, double* host, int unpack) {
  long long cells = packed_cells(E);
  if (cells == 0) return ENL_OK;
  size_t need = (size_t)cells * kNF;
  if (need > E->packed_cap) {
    if (E->d_packed) cudaFree(E->d_packed);
    if (cudaMalloc(&E->d_packed, need * sizeof(double)) != cudaSuccess) {
      E->d_packed = nullptr;
      E->packed_cap = 0;
      set_error(ENL_ERR_CUDA);
      return ENL_ERR_CUDA;
    }
    E->packed_cap = need;
  }
  cudaStream_t s = stream();
  PackArgs A;
  memset(&A, 0, sizeof(A));
  for (int l = 0; l < E->cfg.nlevels; ++l) A.lev[l] = E->lev[l].view(0);
  A.tiles = E->d_tiles.p;
  A.off = E->d_tileoff.p;
  A.ntiles = (int)E->h_tiles.size();
  A.total = cells;
  A.packed = E->d_packed;
  A.unpack = unpack;
  if (unpack) cudaMemcpyAsync(E->d_packed, host, need * sizeof(double), cudaMemcpyHostToDevice, s);
  pack_kernel<<<std::min(A.ntiles, E->nsm * 8), 256, 0, s>>>(A);
  if (!unpack) cudaMemcpyAsync(host, E->d_packed, need * sizeof(double), cudaMemcpyDeviceToHost, s);
  return check_launch(unpack ? "engine upload" : "engine download");
}

int enl_engine_download(void* e, double* host) {
  Engine* E = (Engine*)e;
  if (!E || !host) return ENL_ERR_ARG;
  return pack_common(E, host, 0);
}

int enl_engine_upload(void* e, const double* host) {
  Engine* E = (Engine*)e;
  if (!E || !host) return ENL_ERR_ARG;
  return pack_common(E, const_cast<double*>(host), 1);
}

int enl_engine_profile(void* e, int on, double* ms_total, long long* launches, long long* cells) {
  Engine* E = (Engine*)e;
  if (!E) return ENL_ERR_ARG;
  if (ms_total) *ms_total = E->prof_ms;
  if (launches) *launches = E->prof_launches;
  if (cells) *cells = E->prof_cells;
  E->prof_ms = 0.0;
  E->prof_launches = 0;
  E->prof_cells = 0;
  if (on && !E->pev[0])
    for (int q = 0; q < 6; ++q) cudaEventCreate(&E->pev[q]);
  E->profile = on ? 1 : 0;
  return check_launch("engine profile");
}

int enl_engine_set_mlp(void* e, const float* params_host, float margin) {
  Engine* E = (Engine*)e;
  if (!E || !params_host || margin < 0.f) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  if (!(E->cfg.precision == ENL_PREC_FP32 && E->cfg.learned)) {
    set_error(ENL_ERR_STATE);
    return ENL_ERR_STATE;
  }
  if (!E->d_mlp && cudaMalloc(&E->d_mlp, kNParams * sizeof(float)) != cudaSuccess) {
    E->d_mlp = nullptr;
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  cudaMemcpyAsync(E->d_mlp, params_host, kNParams * sizeof(float), cudaMemcpyHostToDevice, stream());
  cudaStreamSynchronize(stream());
  E->margin = margin;
  return check_launch("set_mlp");
}

int enl_engine_harvest(void* e, int level, double dt, const double* scale, double keep0, unsigned seed, void* X,
                       float* labels, long capacity, unsigned long long* count_dev) {
  Engine* E = (Engine*)e;
  if (!E || level < 0 || level >= E->cfg.nlevels || !scale || !X || !labels || !count_dev || capacity < 0) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  const auto& c = E->cfg;
  Level& L = E->lev[level];
  fill_all(E, 0);
  HarvestArgs A;
  memset(&A, 0, sizeof(A));
  A.V = L.view(0);
  A.H = L.view(3);
  double xlo[2] = {c.xlo[0], c.xlo[1]};
  A.P = make_rhs_const(xlo, L.dx, c.weno_alpha, c.kappa, c.mu, c.muB, c.R, c.T_star_n, c.tau_n, c.tol, 0, c.c,
                       c.c_lr);
  A.eps = (float)A.P.sensor_eps;
  A.eps_p = (float)(A.P.sensor_eps * (c.c * c.c) * (c.c * c.c));
  A.inv_sqrt_eps = (float)(1.0 / sqrt(A.P.sensor_eps));
  A.rho0 = (float)c.rho0;
  A.p0 = (float)c.p0;
  A.T0 = (float)c.T0;
  A.tiles = E->d_tiles.p;
  A.off = E->tile_off[level];
  A.cnt = E->tile_cnt[level];
  A.dt = dt;
  for (int k = 0; k < 5; ++k) A.inv_scale[k] = 1.0 / scale[k];
  A.keep0 = (unsigned)(std::min(1.0, std::max(0.0, keep0)) * 4294967295.0);
  A.seed = seed;
  A.X = (__nv_bfloat16*)X;
  A.lab = labels;
  A.count = count_dev;
  A.cap = capacity;
  if (A.cnt) harvest_kernel<<<std::min(A.cnt, E->nsm * 16), 256, 0, stream()>>>(A);
  return check_launch("harvest");
}

}  // extern "C"
