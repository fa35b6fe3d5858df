// FP64 cell routine of the batched engine, reading per-tile planes.
//
// Same right-hand side as fortran/rhs_hybrid_high_llf.m4:121-358 (and the
// eight sibling variants), in FP64, for a cell of a staged halo tile whose
// velocities u = rho u / rho, v = rho v / rho (every halo position) and
// fluxes F_k = u w_k (+ p for k = 1), G_k = v w_k (+ p for k = 2) (interior
// rows / columns) the block computed once into shared memory.  On this GPU
// the FP64 pipe does two fused multiply-adds per clock per SM while FP32 and
// integer work is ~60x cheaper, so the routine spends FP64 operations only
// where the value needs them:
//   * reciprocals are an FP32 hardware seed refined in FP64 (rcp64: three
//     fused multiply-adds, within a couple of units in the last place) and
//     constant divisors are multiplications;
//   * velocities and fluxes come from the planes (a cell used to divide 23
//     times);
//   * the hybrid switch decides bit for bit as the reference's division
//     would (sensor_line_fast), dividing only ratios that lie within 2^-44 of
//     the threshold.
// Results stay within rounding of the reference's (the engine is held to the
// oracle at 1e-12 relative L2 per field).
#pragma once
#include "enl_fast.cuh"

namespace enl {

// Reciprocal of a double.  For positive normal x within the float exponent
// range, the double's exponent and top 20 mantissa bits are moved into a
// float by integer operations, the hardware single-precision reciprocal gives
// a seed r with |1 - x r| < 2^-19, and one Newton step with its cubic term,
// r (1 + e + e^2) with e = 1 - x r, leaves |1 - x r'| = |e|^3 < 2^-57, below
// FP64 rounding.  Zero, negative, non-finite and out-of-range arguments take
// the division.  All bit manipulation is on unsigned integers, so no shift
// overflows.
__device__ __forceinline__ double rcp64(double x) {
  const unsigned hi = (unsigned)__double2hiint(x);
  const unsigned e = hi >> 20;  // sign and biased exponent
  if (e - (1023u - 125u) > 250u) return 1.0 / x;
  const float xf = __uint_as_float((hi - ((1023u - 127u) << 20)) << 3);
  const unsigned rb = __float_as_uint(rcp_approx(xf));
  const double r = __hiloint2double((int)((rb >> 3) + ((1023u - 127u) << 20)), (int)(rb << 29));
  const double ee = fma(-x, r, 1.0);
  return fma(r, fma(ee, ee, ee), r);
}

// The hybrid switch of rhs_hybrid_high_llf.m4:239-256 along one direction,
// r[0..4] = rho at offsets -2..2; the same decision as sensor_line_exact bit
// for bit.  Each ratio num / den (both >= ep > 0, rounded as the reference
// rounds them) is first estimated as num * rcp64(den), within 2^-50 of the
// exact quotient; the reference's correctly rounded quotient is below the
// threshold c when the estimate is below c (1 - 2^-44) and not below it when
// the estimate is above c (1 + 2^-44).  Only ratios in between are divided.
// Two zero differences give num = den = ep, a ratio of 1: no WENO.
__device__ __forceinline__ int sensor_line_fast(const double r[5], double ep) {
  constexpr double kLo = Lit::c0_9999 * (1.0 - 0x1p-44);
  constexpr double kHi = Lit::c0_9999 * (1.0 + 0x1p-44);
  double t[4], sq[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    t[q] = __dsub_rn(r[q + 1], r[q]);
    sq[q] = __dmul_rn(t[q], t[q]);
  }
  int tag = 0;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const double t1 = t[q], t2 = t[q + 1];
    const unsigned long long mag =
        ((unsigned long long)__double_as_longlong(t1) | (unsigned long long)__double_as_longlong(t2)) << 1;
    if (mag != 0ull) {  // (both differences zero, of either sign: ratio 1)
      const double num = __dadd_rn(__dmul_rn(2.0, fabs(__dmul_rn(t1, t2))), ep);
      const double den = __dadd_rn(__dadd_rn(sq[q], sq[q + 1]), ep);
      // positive quotient: its bit pattern orders as its value
      const unsigned long long qb = (unsigned long long)__double_as_longlong(num * rcp64(den));
      if (qb < (unsigned long long)__double_as_longlong(kLo)) tag = 1;
      else if (qb <= (unsigned long long)__double_as_longlong(kHi) && __ddiv_rn(num, den) < Lit::c0_9999) tag = 1;
    }
  }
  return tag;
}

// FP64 planes of a 38 x 14 halo tile (rows of kBW64 doubles): u and v at
// every position, F_0..4 on the 8 interior rows, G_0..4 on the 32 interior
// columns (rows of 32).
constexpr int kBW64 = 38, kBH64 = 14;
constexpr int kPos64 = kBW64 * kBH64;       // 532
constexpr int kPl64F = 8 * kBW64;           // 304
constexpr int kPl64G = kBH64 * 32;          // 448
constexpr int kPl64OffV = kPos64, kPl64OffF = 2 * kPos64, kPl64OffG = kPl64OffF + 5 * kPl64F;
constexpr int kPl64Elems = kPl64OffG + 5 * kPl64G;  // 4824 doubles

// Accessor of one cell: the staged tile (7 fields, planes of kPos64) and the
// planes, centred on the cell.
struct SAcc64P {
  const double* t;
  const double* pl;
  int c;       // (cy + 3) * kBW64 + cx + 3
  int cf, cg;  // cy * kBW64 + cx + 3 in the F planes, (cy + 3) * 32 + cx in the G planes
  __device__ double w(int k, int di, int dj) const { return t[k * kPos64 + c + dj * kBW64 + di]; }
  __device__ double p(int di, int dj) const { return t[5 * kPos64 + c + dj * kBW64 + di]; }
  __device__ double t_(int di, int dj) const { return t[6 * kPos64 + c + dj * kBW64 + di]; }
  __device__ double u(int di, int dj) const { return pl[c + dj * kBW64 + di]; }
  __device__ double v(int di, int dj) const { return pl[kPl64OffV + c + dj * kBW64 + di]; }
  __device__ double fx(int k, int di) const { return pl[kPl64OffF + k * kPl64F + cf + di]; }
  __device__ double gy(int k, int dj) const { return pl[kPl64OffG + k * kPl64G + cg + dj * 32]; }
};
__device__ __forceinline__ SAcc64P acc64p(const double* t, const double* pl, int cx, int cy) {
  return SAcc64P{t, pl, (cy + 3) * kBW64 + cx + 3, cy * kBW64 + cx + 3, (cy + 3) * 32 + cx};
}

// Switch of one cell (SCHEME as in enl_physics.cuh).
template <int SCHEME>
__device__ __forceinline__ int switch64(const SAcc64P& A, const RhsConst& P) {
  if (SCHEME == kWeno) return 1;
  if (SCHEME == kDrp) return 0;
  if (P.level != 0) return 1;
  double r[5];
#pragma unroll
  for (int q = 0; q < 5; ++q) r[q] = A.w(0, q - 2, 0);
  int tag = sensor_line_fast(r, P.sensor_eps);
#pragma unroll
  for (int q = 0; q < 5; ++q) r[q] = A.w(0, 0, q - 2);
  return tag | sensor_line_fast(r, P.sensor_eps);
}

// Viscous, entropy-production and relaxation sources H1..H4
// (rhs_hybrid_high_llf.m4:161-237) from the planes.
__device__ __forceinline__ void sources64(const SAcc64P& A, const RhsConst& P, double H[5]) {
  const double c43 = Lit::c4_3, c23 = Lit::c2_3;
  double u[3][3], v[3][3];
#pragma unroll
  for (int dj = -1; dj <= 1; ++dj)
#pragma unroll
    for (int di = -1; di <= 1; ++di) {
      u[dj + 1][di + 1] = A.u(di, dj);
      v[dj + 1][di + 1] = A.v(di, dj);
    }
  double u_dxx = ((u[1][0] - 2.0 * u[1][1]) + u[1][2]) * P.inv_dx0sq;
  double u_dyy = ((u[0][1] - 2.0 * u[1][1]) + u[2][1]) * P.inv_dx1sq;
  double v_dxy = (((v[2][2] - v[0][2]) - v[2][0]) + v[0][0]) * P.inv_4dxdy;
  H[1] = P.muB * (u_dxx + v_dxy) + P.mu * ((c43 * u_dxx - c23 * v_dxy) + (u_dyy + v_dxy));
  double v_dyy = ((v[0][1] - 2.0 * v[1][1]) + v[2][1]) * P.inv_dx1sq;
  double v_dxx = ((v[1][0] - 2.0 * v[1][1]) + v[1][2]) * P.inv_dx0sq;
  double u_dyx = (((u[2][2] - u[0][2]) - u[2][0]) + u[0][0]) * P.inv_4dxdy;
  H[2] = P.muB * (v_dyy + u_dyx) + P.mu * ((u_dyx + v_dxx) + (c43 * v_dyy - c23 * u_dyx));

  double ux = (u[1][2] - u[1][0]) * P.inv_2dx0;
  double uy = (u[2][1] - u[0][1]) * P.inv_2dx1;
  double vy = (v[2][1] - v[0][1]) * P.inv_2dx1;
  double vx = (v[1][2] - v[1][0]) * P.inv_2dx0;
  const double Tc = A.t_(0, 0), txm = A.t_(-1, 0), txp = A.t_(1, 0), tym = A.t_(0, -1), typ = A.t_(0, 1);
  double tx = (txp - txm) * P.inv_2dx0;
  double ty = (typ - tym) * P.inv_2dx1;
  double txx = ((txm - 2.0 * Tc) + txp) * P.inv_dx0sq;
  double tyy = ((tym - 2.0 * Tc) + typ) * P.inv_dx1sq;
  const double rho = A.w(0, 0, 0);
  double T_n = A.w(4, 0, 0) * rcp64(rho);
  double Mn = (Tc - T_n) * P.inv_tau_n;
  double inv_Tn = rcp64(T_n);
  double tmp1 = P.T_star_n * inv_Tn;
  double c_vn = ((Lit::c0_78 * P.R) * (tmp1 * tmp1)) * exp(-tmp1);
  double A_n = (Tc * inv_Tn - 1.0) * c_vn;
  double phi_xx = c43 * ux - c23 * vy;
  double phi_xy = uy + vx;
  double phi_yy = c43 * vy - c23 * ux;
  double inv_T = rcp64(Tc);
  double inv_T2 = inv_T * inv_T;
  double s0 = ux + vy;
  double sigma = (((P.muB * inv_T) * (s0 * s0) +
                   (P.mu * 0.5 * inv_T) * ((phi_xx * phi_xx + 2.0 * (phi_xy * phi_xy)) + phi_yy * phi_yy)) +
                  (P.kappa * inv_T2) * (tx * tx + ty * ty)) +
                 (rho * inv_T) * (A_n * Mn);
  double cond = ((-(P.kappa * (tx * tx)) * inv_T2 + (P.kappa * txx) * inv_T) - (P.kappa * (ty * ty)) * inv_T2) +
                (P.kappa * tyy) * inv_T;
  H[3] = (sigma - ((rho * inv_Tn) * c_vn) * Mn) + cond;
  H[4] = (rho * P.inv_tau_n) * (Tc - T_n);
}

// WENO reconstructions with the seeded reciprocal for the weights' sum
// (the same formulas as weno5 / weno3 of enl_physics.cuh).
template <bool PLUS>
__device__ __forceinline__ double weno5r(double a, double b, double c, double d, double e) {
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
  return (Lit::c1_6 * num) * rcp64((n0 + n1) + n2);
}

template <bool PLUS>
__device__ __forceinline__ double weno3r(double b, double c, double d) {
  double e0 = d - c, e1 = c - b;
  double q0 = fma(e0, e0, Lit::weno_eps), q1 = fma(e1, e1, Lit::weno_eps);
  q0 *= q0;
  q1 *= q1;
  const double z0 = PLUS ? Lit::c2_3 : Lit::c1_3;
  const double z1 = PLUS ? Lit::c1_3 : Lit::c2_3;
  double n0 = z0 * q1, n1 = z1 * q0;
  double f0 = PLUS ? (c + d) : fma(3.0, c, -d);
  double f1 = PLUS ? fma(3.0, c, -b) : (b + c);
  return (0.5 * fma(n0, f0, n1 * f1)) * rcp64(n0 + n1);
}

// LLF-split WENO derivative of field k plus its source hk (out of line: one
// copy of the code for the five fields).
template <int ORDER>
__device__ __noinline__ double weno_field64(const SAcc64P A, const RhsConst& P, int k, double af, double ag,
                                            double hk) {
  double fp[7], fm[7], gp[7], gm[7];
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    const double wx = A.w(k, q - 3, 0), wy = A.w(k, 0, q - 3);
    const double F = A.fx(k, q - 3), G = A.gy(k, q - 3);
    fp[q] = 0.5 * fma(af, wx, F);
    fm[q] = 0.5 * fma(-af, wx, F);
    gp[q] = 0.5 * fma(ag, wy, G);
    gm[q] = 0.5 * fma(-ag, wy, G);
  }
  double dfx, dgy;
  if (ORDER == 5) {
    dfx = ((weno5r<true>(fp[0], fp[1], fp[2], fp[3], fp[4]) + weno5r<false>(fm[1], fm[2], fm[3], fm[4], fm[5])) -
           weno5r<true>(fp[1], fp[2], fp[3], fp[4], fp[5])) -
          weno5r<false>(fm[2], fm[3], fm[4], fm[5], fm[6]);
    dgy = ((weno5r<true>(gp[0], gp[1], gp[2], gp[3], gp[4]) + weno5r<false>(gm[1], gm[2], gm[3], gm[4], gm[5])) -
           weno5r<true>(gp[1], gp[2], gp[3], gp[4], gp[5])) -
          weno5r<false>(gm[2], gm[3], gm[4], gm[5], gm[6]);
  } else {
    dfx = ((weno3r<true>(fp[1], fp[2], fp[3]) + weno3r<false>(fm[2], fm[3], fm[4])) -
           weno3r<true>(fp[2], fp[3], fp[4])) -
          weno3r<false>(fm[3], fm[4], fm[5]);
    dgy = ((weno3r<true>(gp[1], gp[2], gp[3]) + weno3r<false>(gm[2], gm[3], gm[4])) -
           weno3r<true>(gp[2], gp[3], gp[4])) -
          weno3r<false>(gm[3], gm[4], gm[5]);
  }
  return fma(dfx, P.inv_dx0, fma(dgy, P.inv_dx1, hk));
}

// KK[0..4] of the cell given the switch (H[0] holds the source H0).
template <int ORDER, bool LLF>
__device__ __forceinline__ void fluxes64(const SAcc64P& A, const RhsConst& P, int cj, int tag, double H[5],
                                         double KK[5]) {
  if (tag == 0) {
    // Tam-Webb DRP, rhs_hybrid_high_llf.m4:258-268
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      double fx = 0.0, gy = 0.0;
#pragma unroll
      for (int m = 3; m >= 1; --m) {
        const double a = m == 1 ? Lit::a1 : (m == 2 ? Lit::a2 : Lit::a3);
        fx = fma(a, A.fx(k, m) - A.fx(k, -m), fx);
        gy = fma(a, A.gy(k, m) - A.gy(k, -m), gy);
      }
      KK[k] = (H[k] - fx * P.inv_dx0) - gy * P.inv_dx1;
    }
    return;
  }
  // split speeds, rhs_hybrid_high_llf.m4:270-284
  double af, ag;
  if (LLF) {
    const int qr = ORDER == 5 ? 3 : 2;
    double mx = 0.0;
#pragma unroll
    for (int q = -qr; q <= qr; ++q) mx = fmax(mx, fabs(A.u(q, 0)));
    const double hrow = P.ylo + P.dy * ((double)cj + 0.5);
    af = (mx + P.c) + P.c_lr * hrow;
    ag = 0.0;
#pragma unroll
    for (int q = -qr; q <= qr; ++q) {
      const double h = P.ylo + P.dy * ((double)(cj + q) + 0.5);
      ag = fmax(ag, (fabs(A.v(0, q)) + P.c) + P.c_lr * h);
    }
  } else {
    af = P.alpha;
    ag = P.alpha;
  }
  KK[0] = weno_field64<ORDER>(A, P, 0, af, ag, H[0]);
  KK[1] = weno_field64<ORDER>(A, P, 1, af, ag, H[1]);
  KK[2] = weno_field64<ORDER>(A, P, 2, af, ag, H[2]);
  KK[3] = weno_field64<ORDER>(A, P, 3, af, ag, H[3]);
  KK[4] = weno_field64<ORDER>(A, P, 4, af, ag, H[4]);
}

// Accessor of the learned switch's features on an FP64 tile: density and
// pressure as single-precision perturbations (the features use differences
// and ratios of differences only).
struct SAcc64Feat {
  const double* t;
  int c;
  double rho0, p0;
  __device__ float w(int k, int di, int dj) const {
    return (float)(t[k * kPos64 + c + dj * kBW64 + di] - (k == 0 ? rho0 : 0.0));
  }
  __device__ float p(int di, int dj) const { return (float)(t[5 * kPos64 + c + dj * kBW64 + di] - p0); }
};

}  // namespace enl
