// FP32 perturbation-form cell routine of the batched fast path.
//
// The state stays FP64 in HBM.  Each stage converts its halo tile to
// perturbations about the ambient state (rho - rho0, rho u, rho v, rho s,
// rho T_n - rho0 T0, p - p0, T - T0) in single precision and evaluates the
// same right-hand side as fortran/rhs_hybrid_high_llf.m4:121-358:
//   * constant parts cancel exactly in every flux difference and WENO
//     reconstruction (both are translation invariant), so only the variations
//     carry rounding error;
//   * T - T_n and T / T_n - 1 are formed from perturbations
//     ((rho T_n - rho0 T0) - (rho - rho0) T0) / rho, which avoids cancellation;
//   * the hybrid switch uses the division-free form of the ratio test.
// The caller stages per-tile planes of the velocities u = rho u / rho,
// v = rho v / rho and of the fluxes F_k = u w_k (+ p for k = 1) and
// G_k = v w_k (+ p for k = 2) at every halo position, so each cell reads
// them instead of recomputing them for every stencil point.
#pragma once
#include "enl_physics.cuh"

namespace enl {

// Single-precision reciprocal of the hardware (rcp.approx, within 1 ulp);
// every use is inside the FP32 perturbation path, whose error budget is
// orders of magnitude above that.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

struct FastConst {
  float inv_dx0, inv_dx1, inv_dx0sq, inv_dx1sq, inv_2dx0, inv_2dx1, inv_4dxdy;
  float kappa, mu, muB, R078, T_star_n, inv_tau_n;
  float alpha, c, c_lr, ylo, dy;
  float sensor_eps;
  float rho0, T0, rho0T0;
  int level;
};

// acc.w(k, di, dj): perturbation field k (0..4), acc.p: p - p0, acc.t: T - T0,
// acc.u / acc.v: velocities, acc.fx(k, di) / acc.gy(k, dj): fluxes F_k, G_k
// along the cell's row / column.
template <class ACC>
__device__ __forceinline__ int sensor_fast(const ACC& A, const FastConst& P) {
  if (P.level != 0) return 1;
  const float thr = 0.9999f;
  int tag = 0;
#pragma unroll
  for (int dir = 0; dir < 2; ++dir) {
    float r[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) r[q] = dir == 0 ? A.w(0, q - 2, 0) : A.w(0, 0, q - 2);
#pragma unroll
    for (int q = 1; q <= 3; ++q) {
      float t1 = r[q] - r[q - 1], t2 = r[q + 1] - r[q];
      float num = fmaf(2.0f, fabsf(t1 * t2), P.sensor_eps);
      float den = fmaf(t1, t1, fmaf(t2, t2, P.sensor_eps));
      if (num < thr * den) tag = 1;
    }
  }
  return tag;
}

template <class ACC>
__device__ __forceinline__ void sources_fast(const ACC& A, const FastConst& P, float H[5]) {
  float u[3][3], v[3][3];
#pragma unroll
  for (int dj = -1; dj <= 1; ++dj)
#pragma unroll
    for (int di = -1; di <= 1; ++di) {
      u[dj + 1][di + 1] = A.u(di, dj);
      v[dj + 1][di + 1] = A.v(di, dj);
    }
  const float inv_c = rcp_approx(P.rho0 + A.w(0, 0, 0));
  const float c43 = 4.0f / 3.0f, c23 = 2.0f / 3.0f;
  float u_dxx = ((u[1][0] - 2.0f * u[1][1]) + u[1][2]) * P.inv_dx0sq;
  float u_dyy = ((u[0][1] - 2.0f * u[1][1]) + u[2][1]) * P.inv_dx1sq;
  float v_dxy = (((v[2][2] - v[0][2]) - v[2][0]) + v[0][0]) * P.inv_4dxdy;
  H[1] = P.muB * (u_dxx + v_dxy) + P.mu * ((c43 * u_dxx - c23 * v_dxy) + (u_dyy + v_dxy));
  float v_dyy = ((v[0][1] - 2.0f * v[1][1]) + v[2][1]) * P.inv_dx1sq;
  float v_dxx = ((v[1][0] - 2.0f * v[1][1]) + v[1][2]) * P.inv_dx0sq;
  float u_dyx = (((u[2][2] - u[0][2]) - u[2][0]) + u[0][0]) * P.inv_4dxdy;
  H[2] = P.muB * (v_dyy + u_dyx) + P.mu * ((u_dyx + v_dxx) + (c43 * v_dyy - c23 * u_dyx));

  float ux = (u[1][2] - u[1][0]) * P.inv_2dx0;
  float uy = (u[2][1] - u[0][1]) * P.inv_2dx1;
  float vy = (v[2][1] - v[0][1]) * P.inv_2dx1;
  float vx = (v[1][2] - v[1][0]) * P.inv_2dx0;
  float tp = A.t(0, 0);
  float Tc = P.T0 + tp;
  float tx = (A.t(1, 0) - A.t(-1, 0)) * P.inv_2dx0;
  float ty = (A.t(0, 1) - A.t(0, -1)) * P.inv_2dx1;
  float txx = ((A.t(-1, 0) - 2.0f * tp) + A.t(1, 0)) * P.inv_dx0sq;
  float tyy = ((A.t(0, -1) - 2.0f * tp) + A.t(0, 1)) * P.inv_dx1sq;
  float rp = A.w(0, 0, 0);
  float rho = P.rho0 + rp;
  float Tn_p = fmaf(-rp, P.T0, A.w(4, 0, 0)) * inv_c;   // T_n - T0
  float T_n = P.T0 + Tn_p;
  float dT = tp - Tn_p;                                 // T - T_n
  float Mn = dT * P.inv_tau_n;
  float inv_Tn = rcp_approx(T_n);
  float tmp1 = P.T_star_n * inv_Tn;
  float c_vn = (P.R078 * (tmp1 * tmp1)) * __expf(-tmp1);
  float A_n = (dT * inv_Tn) * c_vn;
  float phi_xx = c43 * ux - c23 * vy, phi_xy = uy + vx, phi_yy = c43 * vy - c23 * ux;
  float inv_T = rcp_approx(Tc), inv_T2 = inv_T * inv_T;
  float s0 = ux + vy;
  float sigma = (((P.muB * inv_T) * (s0 * s0) +
                  (P.mu * 0.5f * inv_T) * ((phi_xx * phi_xx + 2.0f * (phi_xy * phi_xy)) + phi_yy * phi_yy)) +
                 (P.kappa * inv_T2) * (tx * tx + ty * ty)) +
                (rho * inv_T) * (A_n * Mn);
  float cond = ((-(P.kappa * (tx * tx)) * inv_T2 + (P.kappa * txx) * inv_T) - (P.kappa * (ty * ty)) * inv_T2) +
               (P.kappa * tyy) * inv_T;
  H[3] = (sigma - ((rho * inv_Tn) * c_vn) * Mn) + cond;
  H[4] = (rho * P.inv_tau_n) * dT;
}

// LLF-split WENO derivative of field k at the cell, plus its source term hk:
// KK_k = hk - (dF/dx + dG/dy), from the staged fluxes and the cell's speeds.
// Out of line by default: one copy of the code for the five fields keeps the
// caller's registers and code size small (ENL_WENO_INLINE inlines it).
#ifdef ENL_WENO_INLINE
#define ENL_WENO_FN __device__ __forceinline__
#else
#define ENL_WENO_FN __device__ __noinline__
#endif
template <int ORDER, class ACC>
ENL_WENO_FN float weno_field(const ACC A, const FastConst& P, int k, float af, float ag, float hk) {
  float fp[7], fm[7], gp[7], gm[7];
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    float wx = A.w(k, q - 3, 0), wy = A.w(k, 0, q - 3);
    float F = A.fx(k, q - 3), G = A.gy(k, q - 3);
    fp[q] = 0.5f * fmaf(af, wx, F);
    fm[q] = 0.5f * fmaf(-af, wx, F);
    gp[q] = 0.5f * fmaf(ag, wy, G);
    gm[q] = 0.5f * fmaf(-ag, wy, G);
  }
  float dfx, dgy;
  if (ORDER == 5) {
    dfx = ((weno5f<true>(fp[0], fp[1], fp[2], fp[3], fp[4]) + weno5f<false>(fm[1], fm[2], fm[3], fm[4], fm[5])) -
           weno5f<true>(fp[1], fp[2], fp[3], fp[4], fp[5])) -
          weno5f<false>(fm[2], fm[3], fm[4], fm[5], fm[6]);
    dgy = ((weno5f<true>(gp[0], gp[1], gp[2], gp[3], gp[4]) + weno5f<false>(gm[1], gm[2], gm[3], gm[4], gm[5])) -
           weno5f<true>(gp[1], gp[2], gp[3], gp[4], gp[5])) -
          weno5f<false>(gm[2], gm[3], gm[4], gm[5], gm[6]);
  } else {
    dfx = ((weno3f<true>(fp[1], fp[2], fp[3]) + weno3f<false>(fm[2], fm[3], fm[4])) -
           weno3f<true>(fp[2], fp[3], fp[4])) -
          weno3f<false>(fm[3], fm[4], fm[5]);
    dgy = ((weno3f<true>(gp[1], gp[2], gp[3]) + weno3f<false>(gm[2], gm[3], gm[4])) -
           weno3f<true>(gp[2], gp[3], gp[4])) -
          weno3f<false>(gm[3], gm[4], gm[5]);
  }
  return fmaf(dfx, P.inv_dx0, fmaf(dgy, P.inv_dx1, hk));
}

template <int ORDER, bool LLF, class ACC>
__device__ __forceinline__ void fluxes_fast(const ACC& A, const FastConst& P, int row, int tag, float H[5],
                                            float KK[5]) {
  // ambient parts of w_k: only rho (k = 0) and rho T_n (k = 4) have one;
  // the fluxes (staged planes) use the full value, the split and the
  // stencil use variations.
  if (tag == 0) {
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      float fx = 0.f, gy = 0.f;
#pragma unroll
      for (int m = 3; m >= 1; --m) {
        const float a = m == 1 ? (float)Lit::a1 : (m == 2 ? (float)Lit::a2 : (float)Lit::a3);
        fx = fmaf(a, A.fx(k, m) - A.fx(k, -m), fx);
        gy = fmaf(a, A.gy(k, m) - A.gy(k, -m), gy);
      }
      KK[k] = (H[k] - fx * P.inv_dx0) - gy * P.inv_dx1;
    }
    return;
  }
  float ux[7], vy[7];
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    ux[q] = A.u(q - 3, 0);
    vy[q] = A.v(0, q - 3);
  }
  float af, ag;
  if (LLF) {
    const int qr = ORDER == 5 ? 3 : 2;
    float mx = 0.f;
#pragma unroll
    for (int q = 3 - qr; q <= 3 + qr; ++q) mx = fmaxf(mx, fabsf(ux[q]));
    af = (mx + P.c) + P.c_lr * (P.ylo + P.dy * ((float)row + 0.5f));
    ag = 0.f;
#pragma unroll
    for (int q = 3 - qr; q <= 3 + qr; ++q)
      ag = fmaxf(ag, (fabsf(vy[q]) + P.c) + P.c_lr * (P.ylo + P.dy * ((float)(row + q - 3) + 0.5f)));
  } else {
    af = P.alpha;
    ag = P.alpha;
  }
  // one out-of-line call per field keeps this function's H and KK indexed by
  // constants (registers) and the code of the five fields shared
  KK[0] = weno_field<ORDER>(A, P, 0, af, ag, H[0]);
  KK[1] = weno_field<ORDER>(A, P, 1, af, ag, H[1]);
  KK[2] = weno_field<ORDER>(A, P, 2, af, ag, H[2]);
  KK[3] = weno_field<ORDER>(A, P, 3, af, ag, H[3]);
  KK[4] = weno_field<ORDER>(A, P, 4, af, ag, H[4]);
}

}  // namespace enl
