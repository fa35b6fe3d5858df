// One cell of the right-hand side in FP64: switch, sources, DRP or WENO.
// fortran/rhs_hybrid_high_llf.m4:121-358 and the eight sibling variants.
#pragma once
#include "enl_physics.cuh"

namespace enl {

// ACC provides  double w(int k, int di, int dj), double p(int di, int dj),
// double t(int di, int dj)  relative to the cell being computed.
// cj = row index of the cell inside its patch (for the LLF height term).
template <int SCHEME, int ORDER, bool LLF, class ACC>
__device__ __forceinline__ int rhs_switch(const ACC& A, const RhsConst& P) {
  if (SCHEME == kWeno) return 1;
  if (SCHEME == kDrp) return 0;
  if (P.level != 0) return 1;
  double r[5];
#pragma unroll
  for (int q = 0; q < 5; ++q) r[q] = A.w(0, q - 2, 0);
  int tag = sensor_line_exact(r, P.sensor_eps);
#pragma unroll
  for (int q = 0; q < 5; ++q) r[q] = A.w(0, 0, q - 2);
  tag |= sensor_line_exact(r, P.sensor_eps);
  return tag;
}

template <class ACC>
__device__ __forceinline__ void rhs_sources(const ACC& A, const RhsConst& P, double H[5]) {
  SrcIn<double> s;
#pragma unroll
  for (int dj = -1; dj <= 1; ++dj)
#pragma unroll
    for (int di = -1; di <= 1; ++di) {
      double ir = 1.0 / A.w(0, di, dj);
      s.u[dj + 1][di + 1] = A.w(1, di, dj) * ir;
      s.v[dj + 1][di + 1] = A.w(2, di, dj) * ir;
      if (di == 0 && dj == 0) s.inv_rho = ir;
    }
  s.tc = A.t(0, 0);
  s.txm = A.t(-1, 0);
  s.txp = A.t(1, 0);
  s.tym = A.t(0, -1);
  s.typ = A.t(0, 1);
  s.rho = A.w(0, 0, 0);
  s.rhoTn = A.w(4, 0, 0);
  sources_f64(s, P, H);
}

// Computes KK[0..4] (H[0] must hold the source) given the switch.
template <int SCHEME, int ORDER, bool LLF, class ACC>
__device__ __forceinline__ void rhs_fluxes(const ACC& A, const RhsConst& P, int cj, int tag,
                                           double H[5], double KK[5]) {
  // velocities along the x row and y column, q = -3..3
  double ux[7], vy[7];
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    ux[q] = A.w(1, q - 3, 0) / A.w(0, q - 3, 0);
    vy[q] = A.w(2, 0, q - 3) / A.w(0, 0, q - 3);
  }
  if (tag == 0) {
    // Tam-Webb DRP, rhs_hybrid_high_llf.m4:258-268.
#pragma unroll 1
    for (int k = 0; k < 5; ++k) {
      double fx = 0.0, gy = 0.0;
#pragma unroll
      for (int m = 3; m >= 1; --m) {
        const double a = m == 1 ? Lit::a1 : (m == 2 ? Lit::a2 : Lit::a3);
        double fp = ux[3 + m] * A.w(k, m, 0), fm = ux[3 - m] * A.w(k, -m, 0);
        double gp = vy[3 + m] * A.w(k, 0, m), gm = vy[3 - m] * A.w(k, 0, -m);
        if (k == 1) {
          fp += A.p(m, 0);
          fm += A.p(-m, 0);
        }
        if (k == 2) {
          gp += A.p(0, m);
          gm += A.p(0, -m);
        }
        fx = fma(a, fp - fm, fx);
        gy = fma(a, gp - gm, gy);
      }
      KK[k] = (H[k] - fx * P.inv_dx0) - gy * P.inv_dx1;
    }
    return;
  }
  // WENO: split speeds, rhs_hybrid_high_llf.m4:270-284.
  double af, ag;
  if (LLF) {
    const int qr = ORDER == 5 ? 3 : 2;
    double mx = 0.0;
#pragma unroll
    for (int q = 3 - qr; q <= 3 + qr; ++q) mx = fmax(mx, fabs(ux[q]));
    double hrow = P.ylo + P.dy * ((double)cj + 0.5);
    af = (mx + P.c) + P.c_lr * hrow;
    ag = 0.0;
#pragma unroll
    for (int q = 3 - qr; q <= 3 + qr; ++q) {
      double h = P.ylo + P.dy * ((double)(cj + q - 3) + 0.5);
      ag = fmax(ag, (fabs(vy[q]) + P.c) + P.c_lr * h);
    }
  } else {
    af = P.alpha;
    ag = P.alpha;
  }
#pragma unroll 1
  for (int k = 0; k < 5; ++k) {
    double fp[7], fm[7], gp[7], gm[7];
#pragma unroll
    for (int q = 0; q < 7; ++q) {
      double wx = A.w(k, q - 3, 0), wy = A.w(k, 0, q - 3);
      double F = ux[q] * wx, G = vy[q] * wy;
      if (k == 1) F += A.p(q - 3, 0);
      if (k == 2) G += A.p(0, q - 3);
      fp[q] = 0.5 * fma(af, wx, F);
      fm[q] = 0.5 * fma(-af, wx, F);
      gp[q] = 0.5 * fma(ag, wy, G);
      gm[q] = 0.5 * fma(-ag, wy, G);
    }
    double dfx, dgy;
    if (ORDER == 5) {
      // pf1: fp[-3..1], mf1: fm[-2..2], pf2: fp[-2..2], mf2: fm[-1..3]
      double pf1 = weno5<true>(fp[0], fp[1], fp[2], fp[3], fp[4]);
      double mf1 = weno5<false>(fm[1], fm[2], fm[3], fm[4], fm[5]);
      double pf2 = weno5<true>(fp[1], fp[2], fp[3], fp[4], fp[5]);
      double mf2 = weno5<false>(fm[2], fm[3], fm[4], fm[5], fm[6]);
      double pg1 = weno5<true>(gp[0], gp[1], gp[2], gp[3], gp[4]);
      double mg1 = weno5<false>(gm[1], gm[2], gm[3], gm[4], gm[5]);
      double pg2 = weno5<true>(gp[1], gp[2], gp[3], gp[4], gp[5]);
      double mg2 = weno5<false>(gm[2], gm[3], gm[4], gm[5], gm[6]);
      dfx = ((pf1 + mf1) - pf2) - mf2;
      dgy = ((pg1 + mg1) - pg2) - mg2;
    } else {
      // rhs_hybrid_low_llf.m4:286-337: pf1 fp[-2..0], mf1 fm[-1..1],
      // pf2 fp[-1..1], mf2 fm[0..2]
      double pf1 = weno3<true>(fp[1], fp[2], fp[3]);
      double mf1 = weno3<false>(fm[2], fm[3], fm[4]);
      double pf2 = weno3<true>(fp[2], fp[3], fp[4]);
      double mf2 = weno3<false>(fm[3], fm[4], fm[5]);
      double pg1 = weno3<true>(gp[1], gp[2], gp[3]);
      double mg1 = weno3<false>(gm[2], gm[3], gm[4]);
      double pg2 = weno3<true>(gp[2], gp[3], gp[4]);
      double mg2 = weno3<false>(gm[3], gm[4], gm[5]);
      dfx = ((pf1 + mf1) - pf2) - mf2;
      dgy = ((pg1 + mg1) - pg2) - mg2;
    }
    KK[k] = fma(dfx, P.inv_dx0, fma(dgy, P.inv_dx1, H[k]));
  }
}

}  // namespace enl
