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
// every position, the half fluxes F_0..4 / 2 on the 8 interior rows and
// G_0..4 / 2 on the 32 interior columns (rows of 32).
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

// WENO5 reconstruction (the formulas of weno5 in enl_physics.cuh) from its
// five inputs and the squares of its three second differences tt0..tt2
// (S0 = c,d,e; S1 = b,c,d; S2 = a,b,c), arranged for the FP64 pipe:
//   * the weights omega_k = (d_k / q_k) / sum_j (d_j / q_j) do not change
//     when every q_k is multiplied by the same number, so with
//     q_k = (13/12 t_k^2 + s_k^2 / 4 + eps)^2 the routine uses 16 q_k =
//     (13/3 t_k^2 + s_k^2 + 4 eps)^2, formed by two fused multiply-adds and
//     a square;
//   * omega_k f_k / 6 = P_k (d_k f_k / 6) / sum_j d_j P_j with P_k the product
//     of the other two q: the linear weights d_k and the 1/6 go into the
//     candidate polynomials' coefficients (compile-time constants), and the
//     normalisation is one seeded reciprocal.
// The result agrees with weno5 to rounding.
template <bool PLUS>
__device__ __forceinline__ double weno5q(double a, double b, double c, double d, double e, double tt0, double tt1,
                                         double tt2) {
  constexpr double k4 = 4.0 * Lit::c13_12;        // exact
  constexpr double eps4 = 4.0 * Lit::weno_eps;    // exact
  const double s0 = fma(3.0, c, fma(-4.0, d, e)), s1 = b - d, s2 = fma(3.0, c, fma(-4.0, b, a));
  double q0 = fma(k4, tt0, fma(s0, s0, eps4));
  double q1 = fma(k4, tt1, fma(s1, s1, eps4));
  double q2 = fma(k4, tt2, fma(s2, s2, eps4));
  q0 *= q0;
  q1 *= q1;
  q2 *= q2;
  constexpr double d0 = PLUS ? Lit::c0_3 : Lit::c0_1;
  constexpr double d1 = Lit::c0_6;
  constexpr double d2 = PLUS ? Lit::c0_1 : Lit::c0_3;
  constexpr double w0 = d0 * Lit::c1_6, w1 = d1 * Lit::c1_6, w2 = d2 * Lit::c1_6;
  const double P0 = q1 * q2, P1 = q0 * q2, P2 = q0 * q1;
  const double den = fma(d0, P0, fma(d1, P1, d2 * P2));
  double g0, g1, g2;  // d_k f_k / 6
  if (PLUS) {
    g0 = fma(2.0 * w0, c, fma(5.0 * w0, d, -w0 * e));
    g1 = fma(-w1, b, fma(5.0 * w1, c, (2.0 * w1) * d));
    g2 = fma(2.0 * w2, a, fma(-7.0 * w2, b, (11.0 * w2) * c));
  } else {
    g0 = fma(11.0 * w0, c, fma(-7.0 * w0, d, (2.0 * w0) * e));
    g1 = fma(2.0 * w1, b, fma(5.0 * w1, c, -w1 * d));
    g2 = fma(-w2, a, fma(5.0 * w2, b, (2.0 * w2) * c));
  }
  const double num = fma(P0, g0, fma(P1, g1, P2 * g2));
  return num * rcp64(den);
}

// The two WENO5 reconstructions of one sign along one direction of a cell:
// x[0..5] are the split fluxes at offsets -3..2; lo is the reconstruction
// from x[0..4], hi from x[1..5].  The two stencils share two of their three
// second differences and those differences' squares.
template <bool PLUS>
__device__ __forceinline__ void weno5_pair(const double x[6], double& lo, double& hi) {
  double tt[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const double t = fma(-2.0, x[j + 1], x[j]) + x[j + 2];
    tt[j] = t * t;
  }
  lo = weno5q<PLUS>(x[0], x[1], x[2], x[3], x[4], tt[2], tt[1], tt[0]);
  hi = weno5q<PLUS>(x[1], x[2], x[3], x[4], x[5], tt[3], tt[2], tt[1]);
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
// The planes hold half fluxes F/2, G/2, and ha, hb are half the split
// speeds: fma(ha, w, F/2) is 0.5 fma(af, w, F) exactly (halving is exact),
// one multiplication fewer per split flux.
template <int ORDER>
__device__ __noinline__ double weno_field64(const SAcc64P A, const RhsConst& P, int k, double ha, double hb,
                                            double hk) {
  double fp[7], fm[7], gp[7], gm[7];
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    const double wx = A.w(k, q - 3, 0), wy = A.w(k, 0, q - 3);
    const double Fh = A.fx(k, q - 3), Gh = A.gy(k, q - 3);
    fp[q] = fma(ha, wx, Fh);
    fm[q] = fma(-ha, wx, Fh);
    gp[q] = fma(hb, wy, Gh);
    gm[q] = fma(-hb, wy, Gh);
  }
  double dfx, dgy;
  if (ORDER == 5) {
    double fpl, fph, fml, fmh, gpl, gph, gml, gmh;
    weno5_pair<true>(fp, fpl, fph);
    weno5_pair<false>(fm + 1, fml, fmh);
    weno5_pair<true>(gp, gpl, gph);
    weno5_pair<false>(gm + 1, gml, gmh);
    dfx = ((fpl + fml) - fph) - fmh;
    dgy = ((gpl + gml) - gph) - gmh;
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
      // half fluxes in the planes: the coefficients are doubled (exactly)
      double fx = 0.0, gy = 0.0;
#pragma unroll
      for (int m = 3; m >= 1; --m) {
        const double a = 2.0 * (m == 1 ? Lit::a1 : (m == 2 ? Lit::a2 : Lit::a3));
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
    if (P.c_lr == 0.0) {
      // (x + c) + 0 h is x + c, and x + c rounds monotonically in x: the
      // maximum of the sums is the sum with the maximum (same doubles)
      af = mx + P.c;
      double mv = 0.0;
#pragma unroll
      for (int q = -qr; q <= qr; ++q) mv = fmax(mv, fabs(A.v(0, q)));
      ag = mv + P.c;
    } else {
      const double hrow = P.ylo + P.dy * ((double)cj + 0.5);
      af = (mx + P.c) + P.c_lr * hrow;
      ag = 0.0;
#pragma unroll
      for (int q = -qr; q <= qr; ++q) {
        const double h = P.ylo + P.dy * ((double)(cj + q) + 0.5);
        ag = fmax(ag, (fabs(A.v(0, q)) + P.c) + P.c_lr * h);
      }
    }
  } else {
    af = P.alpha;
    ag = P.alpha;
  }
  const double ha = 0.5 * af, hb = 0.5 * ag;
  KK[0] = weno_field64<ORDER>(A, P, 0, ha, hb, H[0]);
  KK[1] = weno_field64<ORDER>(A, P, 1, ha, hb, H[1]);
  KK[2] = weno_field64<ORDER>(A, P, 2, ha, hb, H[2]);
  KK[3] = weno_field64<ORDER>(A, P, 3, ha, hb, H[3]);
  KK[4] = weno_field64<ORDER>(A, P, 4, ha, hb, H[4]);
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
