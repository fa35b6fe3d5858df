// Per-cell physics of the hybrid WENO/DRP right-hand side, FP64 and FP32.
//
// Restates fortran/rhs_hybrid_high_llf.m4:114-360 (and the eight sibling
// variants) for one cell.  The arithmetic is reorganised for the GPU where the
// result stays within rounding of the reference:
//   * one reciprocal of rho per stencil point; F_k = u * w_k (+ p for k = 1),
//     which equals the reference's w0*(w1/w0)*(wk/w0) up to rounding;
//   * WENO weights with one division per reconstruction (FP64) instead of six;
//   * constant divisors (dx, 2dx, dx^2, 4 dx dy, tau_n) become multiplications.
// The hybrid switch and tag_cells are kept bit-exact: they use only rho
// differences, evaluated with explicitly rounded operations (no FMA) in the
// reference's order, so their decisions match the Fortran bit for bit.
#pragma once
#include "enl_common.cuh"

namespace enl {

enum Scheme { kHybrid = 0, kWeno = 1, kDrp = 2 };

// Launch-constant parameters of the RHS (derived from the rhs_ arguments).
struct RhsConst {
  double inv_dx0, inv_dx1;          // 1/dx, 1/dy
  double inv_dx0sq, inv_dx1sq;      // 1/dx^2, 1/dy^2
  double inv_2dx0, inv_2dx1;        // 1/(2dx), 1/(2dy)
  double inv_4dxdy;                 // 1/(4 dx dy)
  double kappa, mu, muB, R, T_star_n, inv_tau_n;
  double alpha;                     // fixed split speed (weno_alpha)
  double c, c_lr;                   // sound speed and lapse rate
  double ylo, dy;                   // height of row j: ylo + dy*((j - jfirst) + 0.5)
  double sensor_eps;                // ep of the hybrid sensor (tolerance(2))
  int level;
};

// ------------------------------------------------------------------------
// Exact hybrid sensor (rhs_hybrid_high_llf.m4:239-256).  r[0..4] = rho at
// offsets -2..2 along one direction.  Returns 1 if any of the three ratio
// tests at offsets -1, 0, 1 falls below 0.9999.
// ------------------------------------------------------------------------
__device__ __forceinline__ int sensor_line_exact(const double r[5], double ep) {
  int tag = 0;
#pragma unroll
  for (int q = 1; q <= 3; ++q) {
    double t1 = __dsub_rn(r[q], r[q - 1]);
    double t2 = __dsub_rn(r[q + 1], r[q]);
    double num = __dadd_rn(__dmul_rn(2.0, fabs(__dmul_rn(t1, t2))), ep);
    double den = __dadd_rn(__dadd_rn(__dmul_rn(t1, t1), __dmul_rn(t2, t2)), ep);
    double rr = __ddiv_rn(num, den);
    if (rr < Lit::c0_9999) tag = 1;
  }
  return tag;
}

// ------------------------------------------------------------------------
// WENO reconstructions.  wenop/wenom of rhs_hybrid_high_llf.m4:365-433 and
// the WENO3 pair of rhs_hybrid_low_llf.m4:349-397.
// ------------------------------------------------------------------------
// FP64, one division: omega_k = d_k * prod_{j!=k} q_j / sum_k(...).
template <bool PLUS>
__device__ __forceinline__ double weno5(double a, double b, double c, double d, double e) {
  // a..e = fgm2, fgm1, fg0, fgp1, fgp2
  const double k1312 = Lit::c13_12;
  double t0 = fma(-2.0, d, c) + e, s0 = fma(3.0, c, fma(-4.0, d, e));
  double t1 = fma(-2.0, c, b) + d, s1 = b - d;
  double t2 = fma(-2.0, b, a) + c, s2 = fma(-4.0, b, a) + 3.0 * c;
  double q0 = fma(k1312, t0 * t0, 0.25 * (s0 * s0)) + Lit::weno_eps;
  double q1 = fma(k1312, t1 * t1, 0.25 * (s1 * s1)) + Lit::weno_eps;
  double q2 = fma(k1312, t2 * t2, 0.25 * (s2 * s2)) + Lit::weno_eps;
  q0 *= q0;
  q1 *= q1;
  q2 *= q2;
  const double d0 = PLUS ? Lit::c0_3 : Lit::c0_1;
  const double d2 = PLUS ? Lit::c0_1 : Lit::c0_3;
  double n0 = d0 * (q1 * q2), n1 = Lit::c0_6 * (q0 * q2), n2 = d2 * (q0 * q1);
  double f0, f1, f2;
  if (PLUS) {
    f0 = fma(2.0, c, 5.0 * d) - e;
    f1 = fma(5.0, c, -b) + 2.0 * d;
    f2 = fma(2.0, a, -7.0 * b) + 11.0 * c;
  } else {
    f0 = fma(11.0, c, -7.0 * d) + 2.0 * e;
    f1 = fma(2.0, b, 5.0 * c) - d;
    f2 = fma(5.0, b, -a) + 2.0 * c;
  }
  double num = fma(n0, f0, fma(n1, f1, n2 * f2));
  return Lit::c1_6 * (num / ((n0 + n1) + n2));
}

template <bool PLUS>
__device__ __forceinline__ double weno3(double b, double c, double d) {
  // b, c, d = fgm1, fg0, fgp1
  double e0 = d - c, e1 = c - b;
  double q0 = fma(e0, e0, Lit::weno_eps), q1 = fma(e1, e1, Lit::weno_eps);
  q0 *= q0;
  q1 *= q1;
  const double z0 = PLUS ? Lit::c2_3 : Lit::c1_3;
  const double z1 = PLUS ? Lit::c1_3 : Lit::c2_3;
  double n0 = z0 * q1, n1 = z1 * q0;
  double f0 = PLUS ? (c + d) : fma(3.0, c, -d);
  double f1 = PLUS ? fma(3.0, c, -b) : (b + c);
  return 0.5 * (fma(n0, f0, n1 * f1) / (n0 + n1));
}

// FP32 variants (batched fast path): reciprocals instead of the product form,
// which would overflow single precision for strong shocks.
template <bool PLUS>
__device__ __forceinline__ float weno5f(float a, float b, float c, float d, float e) {
  const float k1312 = 13.0f / 12.0f;
  const float eps = 10.0e-6f;
  float t0 = fmaf(-2.0f, d, c) + e, s0 = fmaf(3.0f, c, fmaf(-4.0f, d, e));
  float t1 = fmaf(-2.0f, c, b) + d, s1 = b - d;
  float t2 = fmaf(-2.0f, b, a) + c, s2 = fmaf(-4.0f, b, a) + 3.0f * c;
  float q0 = fmaf(k1312, t0 * t0, 0.25f * (s0 * s0)) + eps;
  float q1 = fmaf(k1312, t1 * t1, 0.25f * (s1 * s1)) + eps;
  float q2 = fmaf(k1312, t2 * t2, 0.25f * (s2 * s2)) + eps;
  const float d0 = PLUS ? 0.3f : 0.1f;
  const float d2 = PLUS ? 0.1f : 0.3f;
  float z0 = __fdividef(d0, q0 * q0), z1 = __fdividef(0.6f, q1 * q1), z2 = __fdividef(d2, q2 * q2);
  float f0, f1, f2;
  if (PLUS) {
    f0 = fmaf(2.0f, c, 5.0f * d) - e;
    f1 = fmaf(5.0f, c, -b) + 2.0f * d;
    f2 = fmaf(2.0f, a, -7.0f * b) + 11.0f * c;
  } else {
    f0 = fmaf(11.0f, c, -7.0f * d) + 2.0f * e;
    f1 = fmaf(2.0f, b, 5.0f * c) - d;
    f2 = fmaf(5.0f, b, -a) + 2.0f * c;
  }
  float num = fmaf(z0, f0, fmaf(z1, f1, z2 * f2));
  return (1.0f / 6.0f) * __fdividef(num, (z0 + z1) + z2);
}

template <bool PLUS>
__device__ __forceinline__ float weno3f(float b, float c, float d) {
  float e0 = d - c, e1 = c - b;
  float q0 = fmaf(e0, e0, 10.0e-6f), q1 = fmaf(e1, e1, 10.0e-6f);
  const float c0 = PLUS ? (2.0f / 3.0f) : (1.0f / 3.0f);
  const float c1 = PLUS ? (1.0f / 3.0f) : (2.0f / 3.0f);
  float z0 = __fdividef(c0, q0 * q0), z1 = __fdividef(c1, q1 * q1);
  float f0 = PLUS ? (c + d) : fmaf(3.0f, c, -d);
  float f1 = PLUS ? fmaf(3.0f, c, -b) : (b + c);
  return 0.5f * __fdividef(fmaf(z0, f0, z1 * f1), z0 + z1);
}

// ------------------------------------------------------------------------
// Viscous, entropy-production and relaxation sources H1..H4
// (rhs_hybrid_high_llf.m4:161-237).  Inputs: u, v on the 3x3 box (index
// [dj+1][di+1]), temperature on the 5-point cross (tc, txm, txp, tym, typ),
// rho and rho*T_n at the centre, 1/rho at the centre.
// ------------------------------------------------------------------------
template <typename T>
struct SrcIn {
  T u[3][3], v[3][3];
  T tc, txm, txp, tym, typ;
  T rho, rhoTn, inv_rho;
};

__device__ __forceinline__ void sources_f64(const SrcIn<double>& s, const RhsConst& P, double H[5]) {
  const double c43 = Lit::c4_3, c23 = Lit::c2_3;
  double u_dxx = ((s.u[1][0] - 2.0 * s.u[1][1]) + s.u[1][2]) * P.inv_dx0sq;
  double u_dyy = ((s.u[0][1] - 2.0 * s.u[1][1]) + s.u[2][1]) * P.inv_dx1sq;
  double v_dxy = (((s.v[2][2] - s.v[0][2]) - s.v[2][0]) + s.v[0][0]) * P.inv_4dxdy;
  H[1] = P.muB * (u_dxx + v_dxy) + P.mu * ((c43 * u_dxx - c23 * v_dxy) + (u_dyy + v_dxy));
  double v_dyy = ((s.v[0][1] - 2.0 * s.v[1][1]) + s.v[2][1]) * P.inv_dx1sq;
  double v_dxx = ((s.v[1][0] - 2.0 * s.v[1][1]) + s.v[1][2]) * P.inv_dx0sq;
  double u_dyx = (((s.u[2][2] - s.u[0][2]) - s.u[2][0]) + s.u[0][0]) * P.inv_4dxdy;
  H[2] = P.muB * (v_dyy + u_dyx) + P.mu * ((u_dyx + v_dxx) + (c43 * v_dyy - c23 * u_dyx));

  double ux = (s.u[1][2] - s.u[1][0]) * P.inv_2dx0;
  double uy = (s.u[2][1] - s.u[0][1]) * P.inv_2dx1;
  double vy = (s.v[2][1] - s.v[0][1]) * P.inv_2dx1;
  double vx = (s.v[1][2] - s.v[1][0]) * P.inv_2dx0;
  double Tc = s.tc;
  double tx = (s.txp - s.txm) * P.inv_2dx0;
  double ty = (s.typ - s.tym) * P.inv_2dx1;
  double txx = ((s.txm - 2.0 * Tc) + s.txp) * P.inv_dx0sq;
  double tyy = ((s.tym - 2.0 * Tc) + s.typ) * P.inv_dx1sq;
  double T_n = s.rhoTn * s.inv_rho;
  double Mn = (Tc - T_n) * P.inv_tau_n;
  double inv_Tn = 1.0 / T_n;
  double tmp1 = P.T_star_n * inv_Tn;
  double c_vn = ((Lit::c0_78 * P.R) * (tmp1 * tmp1)) * exp(-tmp1);
  double A_n = (Tc * inv_Tn - 1.0) * c_vn;
  double phi_xx = c43 * ux - c23 * vy;
  double phi_xy = uy + vx;
  double phi_yy = c43 * vy - c23 * ux;
  double inv_T = 1.0 / Tc;
  double inv_T2 = inv_T * inv_T;
  double s0 = ux + vy;
  double sigma = (((P.muB * inv_T) * (s0 * s0) +
                   (P.mu * 0.5 * inv_T) * ((phi_xx * phi_xx + 2.0 * (phi_xy * phi_xy)) + phi_yy * phi_yy)) +
                  (P.kappa * inv_T2) * (tx * tx + ty * ty)) +
                 (s.rho * inv_T) * (A_n * Mn);
  double cond = ((-(P.kappa * (tx * tx)) * inv_T2 + (P.kappa * txx) * inv_T) -
                 (P.kappa * (ty * ty)) * inv_T2) +
                (P.kappa * tyy) * inv_T;
  H[3] = (sigma - ((s.rho * inv_Tn) * c_vn) * Mn) + cond;
  H[4] = (s.rho * P.inv_tau_n) * (Tc - T_n);
}

}  // namespace enl
