// ===========================================================================
// CPU ORACLE -- test infrastructure only.
//
// A line-by-line C++ restatement of Enlightning's per-patch time advance, used
// by the tests, by __graft_entry__.smoke() and by bench.py's CPU baseline as
// the checker of the CUDA library.  It is never linked into, called by, or
// shipped with the product library (enlightning_gb300/).
//
// What it restates (reference paths are relative to the jonrood/enlightning
// tree):
//   rhs (9 variants)  fortran/rhs_hybrid_high_llf.m4:28-433 and siblings
//                      rhs_hybrid_high.m4, rhs_hybrid_low_llf.m4, rhs_hybrid_low.m4,
//                      rhs_weno_high_llf.m4, rhs_weno_high.m4, rhs_weno_low_llf.m4,
//                      rhs_weno_low.m4, rhs_drp.m4
//   runge_kutta        fortran/runge_kutta.m4:57-66
//   update_state       fortran/update_state.m4:87-107
//   tag_cells          fortran/tag_cells.m4:58-108
//   absorbing envelope enlightning.C:634-786
//   physical BC fill   enlightning.C:790-1013
//   tau_n / tau_o      enlightning.C:217-234
//
// Arithmetic conventions (so that results are bit-identical to a gfortran
// build without FMA contraction):
//   * Fortran evaluates a op b op c left to right and honours parentheses;
//     every expression below keeps that association.
//   * x**2 is x*x.
//   * Un-suffixed Fortran real literals (0.79926643, 13.0/12.0, 0.9, 0.9999,
//     10.0e-6, 0.78, 4.0/3.0, ...) are REAL*4 constants, widened to double when
//     they meet a double operand.  lit() reproduces that (switchable with
//     ora_set_f32_literals for a -fdefault-real-8 style build).
//   * Built with -ffp-contract=off -fno-fast-math.
//
// Parity pin: the reference ships no tests and no golden data, and no Fortran
// compiler exists on either machine.  The golden fixtures in tests/golden/ are
// produced by executing the reference's own Fortran source text with a
// Fortran-77 subset interpreter (tests/golden/f77interp.py); this oracle is
// checked against them bit for bit.  The C++ parts (absorb, BC fill) are
// pinned to the reference's own C++: oracle/ref_bc.py compiles the text of
// enlightning::setAbsorbingBoundaryConditions and
// enlightning::setPhysicalBoundaryConditions unchanged against stand-ins for
// the SAMRAI types (oracle/samrai_stub.h), tests/golden/make_bc_golden.py
// records its outputs, and ora_absorb / ora_phys_bc match them bit for bit.
// SAMRAI's own boundary-box construction is restated in the stand-ins (SAMRAI
// is not available), so that part stays unpinned.
// ===========================================================================
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdlib>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

int g_f32_literals = 1;

inline double lit(float f, double d) { return g_f32_literals ? (double)f : d; }

// ------------------------------------------------------------------------
// Operation counting: the RHS cell routine is a template on its real type so
// that the same source yields per-branch FP64 operation counts.
// ------------------------------------------------------------------------
struct OpCount { double add, mul, div, tr, cmp; };
OpCount g_ops;

struct CR {
  double v;
  CR() : v(0) {}
  CR(double x) : v(x) {}
};
inline CR operator+(CR a, CR b) { g_ops.add++; return CR(a.v + b.v); }
inline CR operator-(CR a, CR b) { g_ops.add++; return CR(a.v - b.v); }
inline CR operator*(CR a, CR b) { g_ops.mul++; return CR(a.v * b.v); }
inline CR operator/(CR a, CR b) { g_ops.div++; return CR(a.v / b.v); }
inline CR operator-(CR a) { return CR(-a.v); }
inline bool operator<(CR a, CR b) { g_ops.cmp++; return a.v < b.v; }
inline bool operator>(CR a, CR b) { g_ops.cmp++; return a.v > b.v; }
inline CR rexp(CR a) { g_ops.tr++; return CR(std::exp(a.v)); }
inline CR rabs(CR a) { return CR(std::fabs(a.v)); }
inline double val(CR a) { return a.v; }

inline double rexp(double a) { return std::exp(a); }
inline double rabs(double a) { return std::fabs(a); }
inline double val(double a) { return a; }

// Scheme selection, mirrors the nine rhs_*.m4 files.
enum Scheme { HYBRID = 0, WENO = 1, DRP = 2 };
struct Variant { int scheme; int order; int llf; };

Variant decode_variant(int v) {
  // v = scheme*4 + (order==3)*2 + (!llf); drp ignores order/llf.
  Variant r;
  r.scheme = v / 4;
  r.order = ((v >> 1) & 1) ? 3 : 5;
  r.llf = (v & 1) ? 0 : 1;
  return r;
}

// Ghosted (SAMRAI CellData, depth-major) layout helper.
struct Box {
  int if0, il0, if1, il1, g0, g1;
  int nxg() const { return il0 - if0 + 1 + 2 * g0; }
  int nyg() const { return il1 - if1 + 1 + 2 * g1; }
  long idx(int i, int j, int k) const {
    return ((long)k * nyg() + (j - if1 + g1)) * nxg() + (i - if0 + g0);
  }
};

// WENO5 reconstructions, rhs_hybrid_high_llf.m4:365-433.
template <class R>
R wenom5(R fgm2, R fgm1, R fg0, R fgp1, R fgp2) {
  const R ep = lit(10.0e-6f, 10.0e-6);
  const R c1312 = lit(13.0f / 12.0f, 13.0 / 12.0);
  const R q = 0.25;
  const R two = 2.0, three = 3.0, four = 4.0, five = 5.0, seven = 7.0, eleven = 11.0;
  R t;
  t = (fg0 - two * fgp1) + fgp2;
  R s = (three * fg0 - four * fgp1) + fgp2;
  R beta0 = c1312 * (t * t) + q * (s * s);
  t = (fgm1 - two * fg0) + fgp1;
  s = fgm1 - fgp1;
  R beta1 = c1312 * (t * t) + q * (s * s);
  t = (fgm2 - two * fgm1) + fg0;
  s = (fgm2 - four * fgm1) + three * fg0;
  R beta2 = c1312 * (t * t) + q * (s * s);
  R e0 = ep + beta0, e1 = ep + beta1, e2 = ep + beta2;
  R zeta0 = R(lit(0.1f, 0.1)) / (e0 * e0);
  R zeta1 = R(lit(0.6f, 0.6)) / (e1 * e1);
  R zeta2 = R(lit(0.3f, 0.3)) / (e2 * e2);
  R sigma = (zeta0 + zeta1) + zeta2;
  R omega0 = zeta0 / sigma, omega1 = zeta1 / sigma, omega2 = zeta2 / sigma;
  const R sixth = lit(1.0f / 6.0f, 1.0 / 6.0);
  R f0 = sixth * ((eleven * fg0 - seven * fgp1) + two * fgp2);
  R f1 = sixth * ((two * fgm1 + five * fg0) - fgp1);
  R f2 = sixth * ((-fgm2 + five * fgm1) + two * fg0);
  return (omega0 * f0 + omega1 * f1) + omega2 * f2;
}

template <class R>
R wenop5(R fgm2, R fgm1, R fg0, R fgp1, R fgp2) {
  const R ep = lit(10.0e-6f, 10.0e-6);
  const R c1312 = lit(13.0f / 12.0f, 13.0 / 12.0);
  const R q = 0.25;
  const R two = 2.0, three = 3.0, four = 4.0, five = 5.0, seven = 7.0, eleven = 11.0;
  R t;
  t = (fg0 - two * fgp1) + fgp2;
  R s = (three * fg0 - four * fgp1) + fgp2;
  R beta0 = c1312 * (t * t) + q * (s * s);
  t = (fgm1 - two * fg0) + fgp1;
  s = fgm1 - fgp1;
  R beta1 = c1312 * (t * t) + q * (s * s);
  t = (fgm2 - two * fgm1) + fg0;
  s = (fgm2 - four * fgm1) + three * fg0;
  R beta2 = c1312 * (t * t) + q * (s * s);
  R e0 = ep + beta0, e1 = ep + beta1, e2 = ep + beta2;
  R zeta0 = R(lit(0.3f, 0.3)) / (e0 * e0);
  R zeta1 = R(lit(0.6f, 0.6)) / (e1 * e1);
  R zeta2 = R(lit(0.1f, 0.1)) / (e2 * e2);
  R sigma = (zeta0 + zeta1) + zeta2;
  R omega0 = zeta0 / sigma, omega1 = zeta1 / sigma, omega2 = zeta2 / sigma;
  const R sixth = lit(1.0f / 6.0f, 1.0 / 6.0);
  R f0 = sixth * ((two * fg0 + five * fgp1) - fgp2);
  R f1 = sixth * ((-fgm1 + five * fg0) + two * fgp1);
  R f2 = sixth * ((two * fgm2 - seven * fgm1) + eleven * fg0);
  return (omega0 * f0 + omega1 * f1) + omega2 * f2;
}

// WENO3 reconstructions, rhs_hybrid_low_llf.m4:349-397 (ep written 10e-6 there,
// the same REAL*4 value as 10.0e-6).
template <class R>
R wenom3(R fgm1, R fg0, R fgp1) {
  const R ep = lit(10.0e-6f, 10.0e-6);
  R d0 = fgp1 - fg0, d1 = fg0 - fgm1;
  R beta0 = d0 * d0, beta1 = d1 * d1;
  R e0 = ep + beta0, e1 = ep + beta1;
  R zeta0 = R(lit(1.0f / 3.0f, 1.0 / 3.0)) / (e0 * e0);
  R zeta1 = R(lit(2.0f / 3.0f, 2.0 / 3.0)) / (e1 * e1);
  R sigma = zeta0 + zeta1;
  R omega0 = zeta0 / sigma, omega1 = zeta1 / sigma;
  const R h = 0.5, three = 3.0;
  R f0 = h * (three * fg0 - fgp1);
  R f1 = h * (fgm1 + fg0);
  return omega0 * f0 + omega1 * f1;
}

template <class R>
R wenop3(R fgm1, R fg0, R fgp1) {
  const R ep = lit(10.0e-6f, 10.0e-6);
  R d0 = fgp1 - fg0, d1 = fg0 - fgm1;
  R beta0 = d0 * d0, beta1 = d1 * d1;
  R e0 = ep + beta0, e1 = ep + beta1;
  R zeta0 = R(lit(2.0f / 3.0f, 2.0 / 3.0)) / (e0 * e0);
  R zeta1 = R(lit(1.0f / 3.0f, 1.0 / 3.0)) / (e1 * e1);
  R sigma = zeta0 + zeta1;
  R omega0 = zeta0 / sigma, omega1 = zeta1 / sigma;
  const R h = 0.5, three = 3.0;
  R f0 = h * (fg0 + fgp1);
  R f1 = h * (-fgm1 + three * fg0);
  return omega0 * f0 + omega1 * f1;
}

struct RhsParams {
  double xlo[2], dx[2];
  double alpha, kappa, mu, muB, R, T_star_n, tau_n;
  double tol[3];
  int level;
  double c, c_lr;
};

// One cell of the RHS.  Returns the WENO/DRP switch (1 = WENO) and writes the
// five KK components.  rhs_hybrid_high_llf.m4:121-358 (and siblings).
template <class R>
int rhs_cell(const Variant& var, const Box& b, const RhsParams& P, const double* w_n,
             const double* H0, const double* pres, const double* temp, int i, int j,
             double out[5]) {
  auto W = [&](int ii, int jj, int k) -> R { return R(w_n[b.idx(ii, jj, k)]); };
  auto PR = [&](int ii, int jj) -> R { return R(pres[b.idx(ii, jj, 0)]); };
  auto TE = [&](int ii, int jj) -> R { return R(temp[b.idx(ii, jj, 0)]); };
  const R two = 2.0, four = 4.0, one = 1.0;
  const R dx0 = P.dx[0], dx1 = P.dx[1];

  // Fluxes F (x) and G (y) at q = -3..3, rhs_hybrid_high_llf.m4:123-157.
  R F[7][5], G[7][5];
  for (int q = -3; q <= 3; ++q) {
    R a0 = W(i + q, j, 0), a1 = W(i + q, j, 1), a2 = W(i + q, j, 2), a3 = W(i + q, j, 3),
      a4 = W(i + q, j, 4);
    R u = a1 / a0;
    F[q + 3][0] = a0 * u;
    F[q + 3][1] = a0 * (u * u) + PR(i + q, j);
    F[q + 3][2] = (a0 * u) * (a2 / a0);
    F[q + 3][3] = (a0 * u) * (a3 / a0);
    F[q + 3][4] = (a0 * u) * (a4 / a0);
    R b0 = W(i, j + q, 0), b1 = W(i, j + q, 1), b2 = W(i, j + q, 2), b3 = W(i, j + q, 3),
      b4 = W(i, j + q, 4);
    R v = b2 / b0;
    G[q + 3][0] = b0 * v;
    G[q + 3][1] = (b0 * v) * (b1 / b0);
    G[q + 3][2] = b0 * (v * v) + PR(i, j + q);
    G[q + 3][3] = (b0 * v) * (b3 / b0);
    G[q + 3][4] = (b0 * v) * (b4 / b0);
  }

  R H[5];
  H[0] = R(H0[(long)(j - b.if1) * (b.il0 - b.if0 + 1) + (i - b.if0)]);

  auto U = [&](int ii, int jj) -> R { return W(ii, jj, 1) / W(ii, jj, 0); };
  auto V = [&](int ii, int jj) -> R { return W(ii, jj, 2) / W(ii, jj, 0); };
  const R c43 = lit(4.0f / 3.0f, 4.0 / 3.0), c23 = lit(2.0f / 3.0f, 2.0 / 3.0);
  const R muB = P.muB, mu = P.mu, kappa = P.kappa;

  // Viscous terms, rhs_hybrid_high_llf.m4:161-197.
  R u_dprime_x = ((U(i - 1, j) - two * U(i, j)) + U(i + 1, j)) / (dx0 * dx0);
  R u_dprime_y = ((U(i, j - 1) - two * U(i, j)) + U(i, j + 1)) / (dx1 * dx1);
  R v_dprime_xy = (((V(i + 1, j + 1) - V(i + 1, j - 1)) - V(i - 1, j + 1)) + V(i - 1, j - 1)) /
                  ((four * dx0) * dx1);
  R phi_xx_prime_x = c43 * u_dprime_x - c23 * v_dprime_xy;
  R phi_xy_prime_y = u_dprime_y + v_dprime_xy;
  H[1] = muB * (u_dprime_x + v_dprime_xy) + mu * (phi_xx_prime_x + phi_xy_prime_y);

  R v_dprime_y = ((V(i, j - 1) - two * V(i, j)) + V(i, j + 1)) / (dx1 * dx1);
  R v_dprime_x = ((V(i - 1, j) - two * V(i, j)) + V(i + 1, j)) / (dx0 * dx0);
  R u_dprime_yx = (((U(i + 1, j + 1) - U(i + 1, j - 1)) - U(i - 1, j + 1)) + U(i - 1, j - 1)) /
                  ((four * dx0) * dx1);
  R phi_yx_prime_x = u_dprime_yx + v_dprime_x;
  R phi_yy_prime_y = c43 * v_dprime_y - c23 * u_dprime_yx;
  H[2] = muB * (v_dprime_y + u_dprime_yx) + mu * (phi_yx_prime_x + phi_yy_prime_y);

  // Entropy production and relaxation, rhs_hybrid_high_llf.m4:200-237.
  R u_prime_x = (U(i + 1, j) - U(i - 1, j)) / (two * dx0);
  R u_prime_y = (U(i, j + 1) - U(i, j - 1)) / (two * dx1);
  R v_prime_y = (V(i, j + 1) - V(i, j - 1)) / (two * dx1);
  R v_prime_x = (V(i + 1, j) - V(i - 1, j)) / (two * dx0);
  R Tc = TE(i, j);
  R t_prime_x = (TE(i + 1, j) - TE(i - 1, j)) / (two * dx0);
  R t_prime_y = (TE(i, j + 1) - TE(i, j - 1)) / (two * dx1);
  R t_dprime_x = ((TE(i - 1, j) - two * Tc) + TE(i + 1, j)) / (dx0 * dx0);
  R t_dprime_y = ((TE(i, j - 1) - two * Tc) + TE(i, j + 1)) / (dx1 * dx1);
  R w0 = W(i, j, 0);
  R T_n = W(i, j, 4) / w0;
  R Mn = (Tc - T_n) / R(P.tau_n);
  R tmp1 = R(P.T_star_n) / T_n;
  R c_vn = (R(lit(0.78f, 0.78)) * R(P.R)) * (tmp1 * tmp1) * rexp(-tmp1);
  R A_n = (Tc / T_n - one) * c_vn;
  R phi_xx = c43 * u_prime_x - c23 * v_prime_y;
  R phi_xy_yx = u_prime_y + v_prime_x;
  R phi_yy = c43 * v_prime_y - c23 * u_prime_x;
  R s0 = u_prime_x + v_prime_y;
  R sigma = (((muB / Tc) * (s0 * s0) +
              (mu / (two * Tc)) * ((phi_xx * phi_xx + two * (phi_xy_yx * phi_xy_yx)) + phi_yy * phi_yy)) +
             (kappa / (Tc * Tc)) * (t_prime_x * t_prime_x + t_prime_y * t_prime_y)) +
            (w0 / Tc) * (A_n * Mn);
  R cond = ((-((kappa * (t_prime_x * t_prime_x)) / (Tc * Tc)) + (kappa * t_dprime_x) / Tc) -
            (kappa * (t_prime_y * t_prime_y)) / (Tc * Tc)) +
           (kappa * t_dprime_y) / Tc;
  H[3] = (sigma - ((w0 / T_n) * c_vn) * Mn) + cond;
  H[4] = (w0 / R(P.tau_n)) * (Tc - T_n);

  // Switch, rhs_hybrid_high_llf.m4:239-256.
  int tag;
  if (var.scheme == WENO) {
    tag = 1;
  } else if (var.scheme == DRP) {
    tag = 0;
  } else {
    tag = 1;
    if (P.level == 0) {
      tag = 0;
      const R xi = 1.0;
      const R c09 = lit(0.9f, 0.9);
      R tl = P.tol[2];
      R ep = ((c09 * tl) * (xi * xi)) / (one - c09 * (tl * tl));
      const R thr = lit(0.9999f, 0.9999);
      for (int q = -1; q <= 1; ++q) {
        R t1 = W(i + q, j, 0) - W(i - 1 + q, j, 0);
        R t2 = W(i + 1 + q, j, 0) - W(i + q, j, 0);
        R rx = (two * rabs(t1 * t2) + ep) / ((t1 * t1 + t2 * t2) + ep);
        if (rx < thr) tag = 1;
        t1 = W(i, j + q, 0) - W(i, j - 1 + q, 0);
        t2 = W(i, j + 1 + q, 0) - W(i, j + q, 0);
        R ry = (two * rabs(t1 * t2) + ep) / ((t1 * t1 + t2 * t2) + ep);
        if (ry < thr) tag = 1;
      }
    }
  }

  if (tag == 0) {
    // DRP, rhs_hybrid_high_llf.m4:258-268 (Tam-Webb 7-point).
    const R a1 = lit(0.79926643f, 0.79926643), a2 = lit(-0.18941314f, -0.18941314),
            a3 = lit(0.02651995f, 0.02651995);
    for (int k = 0; k < 5; ++k) {
      R fx = (((((-(a3 * F[0][k]) - a2 * F[1][k]) - a1 * F[2][k]) + a1 * F[4][k]) + a2 * F[5][k]) +
              a3 * F[6][k]);
      R gy = (((((-(a3 * G[0][k]) - a2 * G[1][k]) - a1 * G[2][k]) + a1 * G[4][k]) + a2 * G[5][k]) +
              a3 * G[6][k]);
      R kk = (fx / (-dx0) + gy / (-dx1)) + H[k];
      out[k] = val(kk);
    }
    return 0;
  }

  // WENO branch: split speed, rhs_hybrid_high_llf.m4:270-284.
  R af, ag;
  if (var.llf) {
    af = 0.0;
    ag = 0.0;
    const int qr = (var.order == 5) ? 3 : 2;
    const R c = P.c, c_lr = P.c_lr, half = 0.5;
    for (int q = -qr; q <= qr; ++q) {
      R height = R(P.xlo[1]) + dx1 * (R((double)(j - b.if1)) + half);
      R sf = (rabs(U(i + q, j)) + c) + c_lr * height;
      if (sf > af) af = sf;
      height = R(P.xlo[1]) + dx1 * (R((double)(j - b.if1 + q)) + half);
      R sg = (rabs(V(i, j + q)) + c) + c_lr * height;
      if (sg > ag) ag = sg;
    }
  } else {
    af = P.alpha;
    ag = P.alpha;
  }

  const R half = 0.5;
  for (int k = 0; k < 5; ++k) {
    // Split fluxes fp(q) = 0.5*(F + a w), fm(q) = 0.5*(F - a w) at q = -3..3.
    auto fpx = [&](int q) { return half * (F[q + 3][k] + af * W(i + q, j, k)); };
    auto fmx = [&](int q) { return half * (F[q + 3][k] - af * W(i + q, j, k)); };
    auto fpy = [&](int q) { return half * (G[q + 3][k] + ag * W(i, j + q, k)); };
    auto fmy = [&](int q) { return half * (G[q + 3][k] - ag * W(i, j + q, k)); };
    R pf1, mf1, pf2, mf2, pg1, mg1, pg2, mg2;
    if (var.order == 5) {
      // rhs_hybrid_high_llf.m4:287-353: interfaces i-1/2 (ii=i-1 and ii=i)
      // and i+1/2 (ii=i and ii=i+1).
      pf1 = wenop5<R>(fpx(-3), fpx(-2), fpx(-1), fpx(0), fpx(1));
      mf1 = wenom5<R>(fmx(-2), fmx(-1), fmx(0), fmx(1), fmx(2));
      pf2 = wenop5<R>(fpx(-2), fpx(-1), fpx(0), fpx(1), fpx(2));
      mf2 = wenom5<R>(fmx(-1), fmx(0), fmx(1), fmx(2), fmx(3));
      pg1 = wenop5<R>(fpy(-3), fpy(-2), fpy(-1), fpy(0), fpy(1));
      mg1 = wenom5<R>(fmy(-2), fmy(-1), fmy(0), fmy(1), fmy(2));
      pg2 = wenop5<R>(fpy(-2), fpy(-1), fpy(0), fpy(1), fpy(2));
      mg2 = wenom5<R>(fmy(-1), fmy(0), fmy(1), fmy(2), fmy(3));
    } else {
      // rhs_hybrid_low_llf.m4:286-337.
      pf1 = wenop3<R>(fpx(-2), fpx(-1), fpx(0));
      mf1 = wenom3<R>(fmx(-1), fmx(0), fmx(1));
      pf2 = wenop3<R>(fpx(-1), fpx(0), fpx(1));
      mf2 = wenom3<R>(fmx(0), fmx(1), fmx(2));
      pg1 = wenop3<R>(fpy(-2), fpy(-1), fpy(0));
      mg1 = wenom3<R>(fmy(-1), fmy(0), fmy(1));
      pg2 = wenop3<R>(fpy(-1), fpy(0), fpy(1));
      mg2 = wenom3<R>(fmy(0), fmy(1), fmy(2));
    }
    R kk = ((((pf1 + mf1) - pf2) - mf2) / dx0 + (((pg1 + mg1) - pg2) - mg2) / dx1) + H[k];
    out[k] = val(kk);
  }
  return 1;
}

}  // namespace

extern "C" {

void ora_set_f32_literals(int on) { g_f32_literals = on ? 1 : 0; }

// Variant ids: 0 hybrid_high_llf, 1 hybrid_high, 2 hybrid_low_llf, 3 hybrid_low,
// 4 weno_high_llf, 5 weno_high, 6 weno_low_llf, 7 weno_low, 8 drp.
//
// rhs: enlightningfort.h:23-49 argument meaning.  flags (nullable, nx*ny ints)
// receives the per-cell WENO(1)/DRP(0) switch; opcounts (nullable, nx*ny*5
// doubles) receives add/mul/div/transcendental/compare counts per cell.
void ora_rhs(int variant, int if0, int il0, int if1, int il1, int g0, int g1, const double* xlo,
             const double* dx, const double* w_n, const double* H0, double* KK, const double* pres,
             const double* temp, double alpha, double kappa, double mu, double muB, double R,
             double T_star_n, double T_star_o, double tau_n, double tau_o, const double* tol,
             int level, double c, double c_lr, int nequ, int* flags, double* opcounts) {
  (void)T_star_o;
  (void)tau_o;
  (void)nequ;
  Variant var = decode_variant(variant);
  Box b{if0, il0, if1, il1, g0, g1};
  RhsParams P;
  P.xlo[0] = xlo[0];
  P.xlo[1] = xlo[1];
  P.dx[0] = dx[0];
  P.dx[1] = dx[1];
  P.alpha = alpha;
  P.kappa = kappa;
  P.mu = mu;
  P.muB = muB;
  P.R = R;
  P.T_star_n = T_star_n;
  P.tau_n = tau_n;
  P.tol[0] = tol[0];
  P.tol[1] = tol[1];
  P.tol[2] = tol[2];
  P.level = level;
  P.c = c;
  P.c_lr = c_lr;
  const int nx = il0 - if0 + 1, ny = il1 - if1 + 1;
  const long n2 = (long)nx * ny;
  if (opcounts) {
    // Instrumented pass (serial: the counters are global).
    for (int j = if1; j <= il1; ++j)
      for (int i = if0; i <= il0; ++i) {
        double out[5];
        long cidx = (long)(j - if1) * nx + (i - if0);
        g_ops = OpCount{0, 0, 0, 0, 0};
        int tag = rhs_cell<CR>(var, b, P, w_n, H0, pres, temp, i, j, out);
        opcounts[cidx * 5 + 0] = g_ops.add;
        opcounts[cidx * 5 + 1] = g_ops.mul;
        opcounts[cidx * 5 + 2] = g_ops.div;
        opcounts[cidx * 5 + 3] = g_ops.tr;
        opcounts[cidx * 5 + 4] = g_ops.cmp;
        for (int k = 0; k < 5; ++k) KK[k * n2 + cidx] = out[k];
        if (flags) flags[cidx] = tag;
      }
    return;
  }
  // Cells are independent; rows are shared out over host threads.
#pragma omp parallel for schedule(dynamic, 1)
  for (int j = if1; j <= il1; ++j) {
    for (int i = if0; i <= il0; ++i) {
      double out[5];
      long cidx = (long)(j - if1) * nx + (i - if0);
      int tag = rhs_cell<double>(var, b, P, w_n, H0, pres, temp, i, j, out);
      for (int k = 0; k < 5; ++k) KK[k * n2 + cidx] = out[k];
      if (flags) flags[cidx] = tag;
    }
  }
}

// Number of host threads the parallel loops use (1 = serial).
void ora_set_threads(int n);

// runge_kutta.m4:57-66.  w_n ghosted, ww and KK interior-only.
void ora_runge_kutta(int if0, int il0, int if1, int il1, int g0, int g1, double dt, double alpha_1,
                     double alpha_2, double beta, double* w_n, const double* ww, const double* KK,
                     int nequ) {
  Box b{if0, il0, if1, il1, g0, g1};
  const int nx = il0 - if0 + 1, ny = il1 - if1 + 1;
  for (int k = 0; k < nequ; ++k)
    for (int j = if1; j <= il1; ++j)
      for (int i = if0; i <= il0; ++i) {
        long c = ((long)k * ny + (j - if1)) * nx + (i - if0);
        long g = b.idx(i, j, k);
        w_n[g] = (alpha_1 * ww[c] + alpha_2 * w_n[g]) + (beta * dt) * KK[c];
      }
}

// update_state.m4:87-107.
void ora_update_state(const double* dx, const double* xlo, int if0, int il0, int if1, int il1,
                      int g0, int g1, const double* w_n, double* pres, double* temp, double rho0,
                      double c, double gamma1, double c_p, double p0, double T0, double c_lr,
                      double c_v, double R_tilde, double M, double R, int nequ) {
  (void)R_tilde;
  (void)M;
  (void)nequ;
  Box b{if0, il0, if1, il1, g0, g1};
  for (int j = if1; j <= il1; ++j) {
    double xc1 = xlo[1] + dx[1] * ((double)(j - if1) + 0.5);
    for (int i = if0; i <= il0; ++i) {
      double w0 = w_n[b.idx(i, j, 0)], w3 = w_n[b.idx(i, j, 3)];
      double cc = c + c_lr * xc1;
      double d = w0 - rho0;
      pres[b.idx(i, j, 0)] =
          (cc * cc) * ((d + ((gamma1 - 1.0) / (2.0 * rho0)) * (d * d)) + (w0 / c_p) * (w3 / w0)) + p0;
      temp[b.idx(i, j, 0)] = T0 * std::exp((w3 / w0 - R * std::log(rho0 / w0)) / c_v);
    }
  }
}

// tag_cells.m4:58-108.  H0 and w_n ghosted; tags interior-only.
void ora_tag_cells(int if0, int il0, int if1, int il1, int g0, int g1, int* tags,
                   const double* w_n, const double* H0, int refine_tag_val, const double* tol,
                   int nequ) {
  (void)nequ;
  Box b{if0, il0, if1, il1, g0, g1};
  const int nx = il0 - if0 + 1;
  auto T = [&](int i, int j) -> int& { return tags[(long)(j - if1) * nx + (i - if0)]; };
  for (int j = if1; j <= il1; ++j)
    for (int i = if0; i <= il0; ++i) T(i, j) = 0;
  const double xi = 1.0;
  const double thr = lit(0.9999f, 0.9999), c09 = lit(0.9f, 0.9);
  for (int pass = 0; pass < 2; ++pass) {
    const double* f = pass == 0 ? H0 : w_n;
    double ep = ((c09 * tol[pass]) * (xi * xi)) / (1.0 - c09 * (tol[pass] * tol[pass]));
    for (int dir = 0; dir < 2; ++dir)
      for (int j = if1; j <= il1; ++j)
        for (int i = if0; i <= il0; ++i) {
          int di = dir == 0 ? 1 : 0, dj = dir == 0 ? 0 : 1;
          double t1 = f[b.idx(i, j, 0)] - f[b.idx(i - di, j - dj, 0)];
          double t2 = f[b.idx(i + di, j + dj, 0)] - f[b.idx(i, j, 0)];
          double r = (2.0 * std::fabs(t1 * t2) + ep) / ((t1 * t1 + t2 * t2) + ep);
          if (r < thr) T(i, j) = refine_tag_val;
        }
  }
}

// Absorbing envelope, enlightning.C:634-786.  bc[4] = L,R,B,T with 20 = ABSORB.
// Arrays ghosted (w_n 5 fields, pres, temp).
void ora_absorb(int if0, int il0, int if1, int il1, int g0, int g1, const double* patch_xlo,
                const double* dx, const double* grid_xlo, const double* grid_xhi, const int* bc,
                double absorb_width, double p0, double T0, double rho0, double* w_n, double* pres,
                double* temp) {
  const int ABSORB = 20;
  if (!(bc[0] == ABSORB || bc[1] == ABSORB || bc[2] == ABSORB || bc[3] == ABSORB)) return;
  Box b{if0, il0, if1, il1, g0, g1};
  const double ep = 1.0e-8;
  const double W2 = absorb_width * absorb_width;
  auto apply = [&](int i, int j, double tmp) {
    long id = b.idx(i, j, 0);
    long area = (long)b.nxg() * b.nyg();
    pres[id] = (pres[id] - p0) * tmp + p0;
    temp[id] = (temp[id] - T0) * tmp + T0;
    w_n[0 * area + id] = (w_n[0 * area + id] - rho0) * tmp + rho0;
    w_n[1 * area + id] = w_n[1 * area + id] * tmp;
    w_n[2 * area + id] = w_n[2 * area + id] * tmp;
    w_n[3 * area + id] = w_n[3 * area + id] * tmp;
    w_n[4 * area + id] = (w_n[4 * area + id] - T0 * rho0) * tmp + T0 * rho0;
  };
  auto env = [&](double d) { return -std::exp(-std::log(2.0) / W2 * (d * d)) + 1.0; };
  double tmp;
  if (bc[0] == ABSORB) {
    double xc0 = patch_xlo[0] + dx[0] * 0.5;
    tmp = env(xc0 - grid_xlo[0]);
    for (int j = if1; j <= il1; ++j) {
      for (int i = if0; (std::fabs(1.0 - tmp) > ep) && (i <= il0); ++i) {
        xc0 = patch_xlo[0] + dx[0] * ((double)(i - if0) + 0.5);
        tmp = env(xc0 - grid_xlo[0]);
        apply(i, j, tmp);
      }
      tmp = 0;
    }
  }
  if (bc[1] == ABSORB) {
    double xc0 = patch_xlo[0] + dx[0] * ((double)(il0 - if0) + 0.5);
    tmp = env(grid_xhi[0] - xc0);
    for (int j = if1; j <= il1; ++j) {
      for (int i = il0; (std::fabs(1.0 - tmp) > ep) && (i >= if0); --i) {
        xc0 = patch_xlo[0] + dx[0] * ((double)(i - if0) + 0.5);
        tmp = env(grid_xhi[0] - xc0);
        apply(i, j, tmp);
      }
      tmp = 0;
    }
  }
  if (bc[2] == ABSORB) {
    double xc1 = patch_xlo[1] + dx[1] * 0.5;
    tmp = env(xc1 - grid_xlo[1]);
    for (int j = if1; (std::fabs(1.0 - tmp) > ep) && (j <= il1); ++j) {
      xc1 = patch_xlo[1] + dx[1] * ((double)(j - if1) + 0.5);
      tmp = env(xc1 - grid_xlo[1]);
      for (int i = if0; i <= il0; ++i) apply(i, j, tmp);
    }
  }
  if (bc[3] == ABSORB) {
    double xc1 = patch_xlo[1] + dx[1] * ((double)(il1 - if1) + 0.5);
    tmp = env(grid_xhi[1] - xc1);
    for (int j = il1; (std::fabs(1.0 - tmp) > ep) && (j >= if1); --j) {
      xc1 = patch_xlo[1] + dx[1] * ((double)(j - if1) + 0.5);
      tmp = env(grid_xhi[1] - xc1);
      for (int i = if0; i <= il0; ++i) apply(i, j, tmp);
    }
  }
}

// Physical-boundary ghost fill, enlightning.C:790-1013, under SAMRAI's
// boundary-box rules: an edge box on every patch side that lies on the domain
// boundary (spanning the patch interior tangentially), and a node box at every
// corner adjacent to at least one such side.  touches[4] = L,R,B,T.  fw0/fw1 =
// ghost width to fill.  bc[4] = L,R,B,T with 10 = REFLECT.  Arrays ghosted:
// w_n (5 fields), pres, temp, source.
void ora_phys_bc(int if0, int il0, int if1, int il1, int g0, int g1, const int* touches,
                 const int* bc, int fw0, int fw1, double* w_n, double* pres, double* temp,
                 double* source) {
  const int REFLECT = 10;
  Box b{if0, il0, if1, il1, g0, g1};
  long area = (long)b.nxg() * b.nyg();
  auto copy = [&](int i, int j, int si, int sj, int neg_k, bool neg) {
    long d = b.idx(i, j, 0), s = b.idx(si, sj, 0);
    pres[d] = pres[s];
    temp[d] = temp[s];
    source[d] = source[s];
    for (int k = 0; k < 5; ++k) {
      w_n[k * area + d] = w_n[k * area + s];
      if (k == neg_k && neg) w_n[k * area + d] = -w_n[k * area + d];
    }
  };
  // Edges, processed in SAMRAI's location order 0..3.
  if (touches[0]) {  // left: fill box i in [if0-fw0, if0-1], j in [if1, il1]
    int fi = if0 - fw0, li = if0 - 1;
    for (int j = if1; j <= il1; ++j)
      for (int i = li; i >= fi; --i) copy(i, j, i + 1, j, 1, i == li && bc[0] == REFLECT);
  }
  if (touches[1]) {
    int fi = il0 + 1, li = il0 + fw0;
    for (int j = if1; j <= il1; ++j)
      for (int i = fi; i <= li; ++i) copy(i, j, i - 1, j, 1, i == fi && bc[1] == REFLECT);
  }
  if (touches[2]) {
    int fj = if1 - fw1, lj = if1 - 1;
    for (int j = lj; j >= fj; --j)
      for (int i = il0; i >= if0; --i) copy(i, j, i, j + 1, 2, j == lj && bc[2] == REFLECT);
  }
  if (touches[3]) {
    int fj = il1 + 1, lj = il1 + fw1;
    for (int j = fj; j <= lj; ++j)
      for (int i = if0; i <= il0; ++i) copy(i, j, i, j - 1, 2, j == fj && bc[3] == REFLECT);
  }
  // Nodes: 0 = (x lo, y lo), 1 = (x hi, y lo), 2 = (x lo, y hi), 3 = (x hi, y hi).
  for (int loc = 0; loc < 4; ++loc) {
    int xs = loc & 1, ys = (loc >> 1) & 1;
    bool present = touches[xs ? 1 : 0] || touches[ys ? 3 : 2];
    if (!present) continue;
    int fi = xs ? il0 + 1 : if0 - fw0, li = xs ? il0 + fw0 : if0 - 1;
    int fj = ys ? il1 + 1 : if1 - fw1, lj = ys ? il1 + fw1 : if1 - 1;
    if (!xs) {
      for (int j = fj; j <= lj; ++j)
        for (int i = li; i >= fi; --i) copy(i, j, i + 1, j, 1, i == li && bc[0] == REFLECT);
    } else {
      for (int j = fj; j <= lj; ++j)
        for (int i = fi; i <= li; ++i) copy(i, j, i - 1, j, 1, i == fi && bc[1] == REFLECT);
    }
  }
}

// tau_n and tau_o from enlightning.C:217-234.
void ora_relaxation_times(double p0, double T0, double RH, double* tau_n, double* tau_o) {
  const double PI = 3.14159265358979323846264338;
  const double T_ref = T0, p_ref = p0;
  const double zeta = 10.79586 * (1 - (273.16 / T0)) - 5.02808 * std::log10(T0 / 273.16) +
                      (1.50474e-4) * (1 - std::pow(10, (-8.29692 * ((T0 / 273.16) - 1)))) -
                      (4.2873e-4) * (1 - std::pow(10, (-4.76955 * ((273.16 / T0) - 1)))) -
                      2.2195983;
  const double p_vp = p_ref * std::pow(10, zeta);
  const double h = (RH * p_vp) / p0;
  const double eta = 4.17 * (std::pow(T_ref / T0, 1.0 / 3.0) - 1);
  const double f_n = (p0 / p_ref) * (std::pow((T_ref / T0), 0.5) * (9 + 280 * h * std::exp(-eta)));
  const double f_o = (p0 / p_ref) * (24 + (4.04e4) * h * ((0.02 + h) / (0.391 + h)));
  *tau_n = 1 / (2 * PI * f_n);
  *tau_o = 1 / (2 * PI * f_o);
}

}  // extern "C"

extern "C" {
void ora_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void)n;
#endif
}
int ora_get_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
}

// Source painting, enlightning.C:2140-2307 (addSource) for one patch of nx*ny
// cells with lower corner xlo and spacing dx; H is interior-only (nx*ny).
// type 10 POINT, 20 SINE, 30 LIGHTNING; mode 10 PULSE, 20 DRIVEN (POINT, the
// value times `drive`).  LIGHTNING accumulates onto H with the capsule-union
// rule of enlightning.C:2214-2281.
extern "C" void ora_paint_source(int nx, int ny, const double* xlo, const double* dx, double* H, int type,
                                 int mode, double amp, double spread, const double* pos, double sine_amp,
                                 double sine_freq, int nseg, const double* segs, double drive) {
  const double PI = 3.14159265358979323846264338;
  auto SQ = [](double x) { return x * x; };
  for (int j = 0; j < ny; ++j) {
    double xc1 = xlo[1] + dx[1] * ((double)j + 0.5);
    for (int i = 0; i < nx; ++i) {
      double xc0 = xlo[0] + dx[0] * ((double)i + 0.5);
      double& out = H[(long)j * nx + i];
      if (type == 10) {
        double x0 = xc0 - pos[0], x1 = xc1 - pos[1];
        double v = amp * std::exp(-std::log(2.0) / SQ(spread) * (x0 * x0 + x1 * x1));
        out = mode == 20 ? v * drive : v;
      } else if (type == 20) {
        double x0 = xc0 - pos[0], x1 = xc1 - pos[1];
        out = amp * std::exp(-std::log(2.0) / SQ(spread) * SQ((x0)-sine_amp * std::sin(sine_freq * (x1))));
      } else {
        for (int k = 0; k < nseg; ++k) {
          const double* c = segs + 4 * k;
          int orientation = 0;
          double theta = -std::atan((c[3] - c[1]) / (c[2] - c[0]));
          if (((c[0] > c[2]) && (c[1] > c[3])) || ((c[0] <= c[2]) && (c[1] >= c[3]))) orientation = 1;
          else if (((c[0] >= c[2]) && (c[1] <= c[3])) || ((c[0] < c[2]) && (c[1] < c[3]))) orientation = 2;
          double line0 = std::tan(PI / 2.0 - theta) * (xc0 - c[0]) + c[1];
          double line1 = std::tan(PI / 2.0 - theta) * (xc0 - c[2]) + c[3];
          if (((orientation == 1) && (xc1 >= line0)) || ((orientation == 2) && (xc1 <= line0))) {
            double t = amp * std::exp(-std::log(2.0) / SQ(spread) * (SQ(xc0 - c[0]) + SQ(xc1 - c[1])));
            out = out + t - (out / amp) * t;
          }
          if (((orientation == 1) && (xc1 <= line1)) || ((orientation == 2) && (xc1 >= line1))) {
            double t = amp * std::exp(-std::log(2.0) / SQ(spread) * (SQ(xc0 - c[2]) + SQ(xc1 - c[3])));
            out = out + t - (out / amp) * t;
          }
          if (((orientation == 1) && (xc1 < line0) && (xc1 > line1)) ||
              ((orientation == 2) && (xc1 > line0) && (xc1 < line1))) {
            double t = amp * std::exp(-std::log(2.0) / SQ(spread) *
                                      (SQ(std::sin(theta) * (xc0 - c[0]) + std::cos(theta) * (xc1 - c[1]))));
            out = out + t - (out / amp) * t;
          }
        }
      }
    }
  }
}

