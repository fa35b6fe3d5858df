// Per-patch FP64 kernels behind the drop-in F77 entry points.
//
//   rhs_           fortran/rhs_*.m4           (rhs_plain_kernel)
//   runge_kutta_   fortran/runge_kutta.m4     (runge_kutta_kernel)
//   update_state_  fortran/update_state.m4    (update_state_kernel)
//   tag_cells_     fortran/tag_cells.m4       (tag_cells_kernel)
//   enl_phys_bc    enlightning.C:790-1013     (phys_bc_edge_kernel, phys_bc_node_kernel)
//   enl_absorb     enlightning.C:634-786      (absorb_x_kernel, absorb_y_kernel)
//
// Every kernel addresses its patch through a pitched view (first stored cell,
// row pitch, field stride) so that the same code serves SAMRAI's contiguous
// CellData arrays and patches embedded in a larger level array.
#include <cmath>
#include <cstdio>

#include "enl_rhs_cell.cuh"

namespace enl {

int rhs_variant();

// Global-memory accessor centred on one cell.
struct GAcc {
  const double* wp;  // field 0 at the centre cell
  const double* pr;  // pressure at the centre cell
  const double* te;  // temperature at the centre cell
  long pitch, fstride;
  __device__ double w(int k, int di, int dj) const { return __ldg(wp + k * fstride + dj * pitch + di); }
  __device__ double p(int di, int dj) const { return __ldg(pr + dj * pitch + di); }
  __device__ double t(int di, int dj) const { return __ldg(te + dj * pitch + di); }
};

template <int SCHEME, int ORDER, bool LLF>
__global__ void __launch_bounds__(128) rhs_plain_kernel(const double* __restrict__ w, const double* __restrict__ pres,
                                         const double* __restrict__ temp, long pitch, long fstride, int g0,
                                         int g1, const double* __restrict__ H0, double* __restrict__ KK,
                                         long opitch, long ofstride, int nx, int ny, RhsConst P,
                                         int* __restrict__ flags) {
  int ci = blockIdx.x * blockDim.x + threadIdx.x;
  int cj = blockIdx.y * blockDim.y + threadIdx.y;
  if (ci >= nx || cj >= ny) return;
  long c = (long)(cj + g1) * pitch + (ci + g0);
  GAcc A{w + c, pres + c, temp + c, pitch, fstride};
  int tag = rhs_switch<SCHEME, ORDER, LLF>(A, P);
  double H[5], K[5];
  H[0] = H0[(long)cj * opitch + ci];
  rhs_sources(A, P, H);
  rhs_fluxes<SCHEME, ORDER, LLF>(A, P, cj, tag, H, K);
  long o = (long)cj * opitch + ci;
#pragma unroll
  for (int k = 0; k < 5; ++k) KK[k * ofstride + o] = K[k];
  if (flags) flags[o] = tag;
}

// runge_kutta.m4:60-63, association kept: (a1*ww + a2*w_n) + (beta*dt)*KK.
__global__ void runge_kutta_kernel(double* __restrict__ wn, long pitch, long fstride, int g0, int g1,
                                   const double* __restrict__ ww, const double* __restrict__ KK,
                                   long ipitch, long ifstride, int nx, int ny, int nequ, double a1,
                                   double a2, double bdt) {
  int ci = blockIdx.x * blockDim.x + threadIdx.x;
  int cj = blockIdx.y * blockDim.y + threadIdx.y;
  if (ci >= nx || cj >= ny) return;
  long g = (long)(cj + g1) * pitch + (ci + g0);
  long c = (long)cj * ipitch + ci;
  for (int k = 0; k < nequ; ++k) {
    double v = __dadd_rn(__dadd_rn(__dmul_rn(a1, ww[k * ifstride + c]), __dmul_rn(a2, wn[k * fstride + g])),
                         __dmul_rn(bdt, KK[k * ifstride + c]));
    wn[k * fstride + g] = v;
  }
}

struct StateConst {
  double rho0, c, gm1_over_2rho0, c_p, p0, T0, c_lr, c_v, R, ylo, dy;
};

// update_state.m4:87-107.
__device__ __forceinline__ void eos_f64(double w0, double w3, double height, const StateConst& S, double& p,
                                        double& T) {
  double cc = __dadd_rn(S.c, __dmul_rn(S.c_lr, height));
  double d = __dsub_rn(w0, S.rho0);
  double s = __ddiv_rn(w3, w0);
  double inner = __dadd_rn(__dadd_rn(d, __dmul_rn(S.gm1_over_2rho0, __dmul_rn(d, d))), __dmul_rn(__ddiv_rn(w0, S.c_p), s));
  p = __dadd_rn(__dmul_rn(__dmul_rn(cc, cc), inner), S.p0);
  T = S.T0 * exp((s - S.R * log(S.rho0 / w0)) / S.c_v);
}

__global__ void update_state_kernel(const double* __restrict__ w, double* __restrict__ pres,
                                    double* __restrict__ temp, long pitch, long fstride, int g0, int g1,
                                    int nx, int ny, StateConst S) {
  int ci = blockIdx.x * blockDim.x + threadIdx.x;
  int cj = blockIdx.y * blockDim.y + threadIdx.y;
  if (ci >= nx || cj >= ny) return;
  long g = (long)(cj + g1) * pitch + (ci + g0);
  double height = __dadd_rn(S.ylo, __dmul_rn(S.dy, (double)cj + 0.5));
  double p, T;
  eos_f64(w[g], w[3 * fstride + g], height, S, p, T);
  pres[g] = p;
  temp[g] = T;
}

// tag_cells.m4:58-108, bit-exact (explicitly rounded operations).
__device__ __forceinline__ bool ratio_below(double fm, double f0, double fp, double ep) {
  double t1 = __dsub_rn(f0, fm);
  double t2 = __dsub_rn(fp, f0);
  double num = __dadd_rn(__dmul_rn(2.0, fabs(__dmul_rn(t1, t2))), ep);
  double den = __dadd_rn(__dadd_rn(__dmul_rn(t1, t1), __dmul_rn(t2, t2)), ep);
  return __ddiv_rn(num, den) < Lit::c0_9999;
}

__global__ void tag_cells_kernel(int* __restrict__ tags, long tpitch, const double* __restrict__ w,
                                 const double* __restrict__ H0, long pitch, int g0, int g1, int nx, int ny,
                                 int tag_val, double ep0, double ep1) {
  int ci = blockIdx.x * blockDim.x + threadIdx.x;
  int cj = blockIdx.y * blockDim.y + threadIdx.y;
  if (ci >= nx || cj >= ny) return;
  long g = (long)(cj + g1) * pitch + (ci + g0);
  bool t = ratio_below(H0[g - 1], H0[g], H0[g + 1], ep0) || ratio_below(H0[g - pitch], H0[g], H0[g + pitch], ep0) ||
           ratio_below(w[g - 1], w[g], w[g + 1], ep1) || ratio_below(w[g - pitch], w[g], w[g + pitch], ep1);
  tags[(long)cj * tpitch + ci] = t ? tag_val : 0;
}

// Physical-boundary fill, enlightning.C:830-944 (edges).  Each ghost cell of
// an edge box receives the first interior cell of its row/column (the
// reference's cascading copy), the normal momentum negated on REFLECT sides.
// One thread per (tangential cell, ghost depth, field).  The fields array
// holds w_n (5), pressure, temperature, source: 8 pointers.
struct PatchFields8 {
  double* f[8];
};

__global__ void phys_bc_edge_kernel(PatchFields8 F, long pitch, int nx, int ny, int g0, int g1, int side,
                                    int fill, int reflect) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int tan_n = (side < 2) ? ny : nx;
  int total = tan_n * fill * 8;
  if (t >= total) return;
  int k = t % 8;
  int d = (t / 8) % fill;       // depth 0 = adjacent ghost
  int s = t / (8 * fill);       // tangential index
  int i, j, si, sj;
  if (side == 0) { j = s + g1; i = g0 - 1 - d; si = g0; sj = j; }
  else if (side == 1) { j = s + g1; i = g0 + nx + d; si = g0 + nx - 1; sj = j; }
  else if (side == 2) { i = s + g0; j = g1 - 1 - d; si = i; sj = g1; }
  else { i = s + g0; j = g1 + ny + d; si = i; sj = g1 + ny - 1; }
  double v = F.f[k][(long)sj * pitch + si];
  int neg_k = (side < 2) ? 1 : 2;
  if (k == neg_k && reflect) v = -v;
  F.f[k][(long)j * pitch + i] = v;
}

// Nodes (corners), enlightning.C:948-1008: copy along x from the cell next
// to the corner box (an edge ghost or a neighbour-filled ghost), x-momentum
// negated when the adjacent x side is REFLECT.
__global__ void phys_bc_node_kernel(PatchFields8 F, long pitch, int nx, int ny, int g0, int g1, int loc,
                                    int fill0, int fill1, int reflect_x) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int total = fill0 * fill1 * 8;
  if (t >= total) return;
  int k = t % 8;
  int dx = (t / 8) % fill0;
  int dy = t / (8 * fill0);
  int xs = loc & 1, ys = (loc >> 1) & 1;
  int j = ys ? (g1 + ny + dy) : (g1 - 1 - dy);
  int i = xs ? (g0 + nx + dx) : (g0 - 1 - dx);
  int si = xs ? (g0 + nx - 1) : g0;
  double v = F.f[k][(long)j * pitch + si];
  if (k == 1 && reflect_x) v = -v;
  F.f[k][(long)j * pitch + i] = v;
}

// Absorbing envelope, enlightning.C:671-783, including the loop-exit rules:
// along x each row runs from the boundary side while the previous envelope
// value differs from 1 by more than 1e-8 (the first row starts from the
// envelope of the first cell, later rows from tmp = 0); along y the same rule
// runs over rows.  dir: 0 = L, 1 = R (one thread per row); 2 = B, 3 = T (one
// thread per column, each walking the rows).
struct AbsorbConst {
  double xlo0, xlo1, dx0, dx1, gxlo0, gxlo1, gxhi0, gxhi1, w2, p0, T0, rho0;
};

// -exp(-log(2.0) / SQUARE(W) * SQUARE(d)) + 1 (enlightning.C:676).
__device__ __forceinline__ double envelope(double d, double w2) {
  return __dadd_rn(-exp(__dmul_rn(__ddiv_rn(-log(2.0), w2), __dmul_rn(d, d))), 1.0);
}

// (q - q_amb) * tmp + q_amb, rounded as written (no contraction).
__device__ __forceinline__ double relax_to(double q, double amb, double tmp) {
  return __dadd_rn(__dmul_rn(__dsub_rn(q, amb), tmp), amb);
}

__device__ __forceinline__ void absorb_apply(PatchFields8 F, long g, double tmp, const AbsorbConst& A) {
  F.f[5][g] = relax_to(F.f[5][g], A.p0, tmp);
  F.f[6][g] = relax_to(F.f[6][g], A.T0, tmp);
  F.f[0][g] = relax_to(F.f[0][g], A.rho0, tmp);
  F.f[1][g] = __dmul_rn(F.f[1][g], tmp);
  F.f[2][g] = __dmul_rn(F.f[2][g], tmp);
  F.f[3][g] = __dmul_rn(F.f[3][g], tmp);
  F.f[4][g] = relax_to(F.f[4][g], __dmul_rn(A.T0, A.rho0), tmp);
}

__global__ void absorb_kernel(PatchFields8 F, long pitch, int nx, int ny, int g0, int g1, int dir,
                              AbsorbConst A) {
  const double ep = 1.0e-8;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (dir < 2) {
    if (t >= ny) return;
    int cj = t;
    double tmp;
    auto xdist = [&](int ci) {
      double xc = A.xlo0 + A.dx0 * ((double)ci + 0.5);
      return dir == 0 ? (xc - A.gxlo0) : (A.gxhi0 - xc);
    };
    tmp = (cj == 0) ? envelope(xdist(dir == 0 ? 0 : nx - 1), A.w2) : 0.0;
    for (int n = 0; (fabs(1.0 - tmp) > ep) && n < nx; ++n) {
      int ci = dir == 0 ? n : nx - 1 - n;
      tmp = envelope(xdist(ci), A.w2);
      absorb_apply(F, (long)(cj + g1) * pitch + (ci + g0), tmp, A);
    }
  } else {
    if (t >= nx) return;
    int ci = t;
    auto ydist = [&](int cj) {
      double yc = A.xlo1 + A.dx1 * ((double)cj + 0.5);
      return dir == 2 ? (yc - A.gxlo1) : (A.gxhi1 - yc);
    };
    double tmp = envelope(ydist(dir == 2 ? 0 : ny - 1), A.w2);
    for (int n = 0; (fabs(1.0 - tmp) > ep) && n < ny; ++n) {
      int cj = dir == 2 ? n : ny - 1 - n;
      tmp = envelope(ydist(cj), A.w2);
      absorb_apply(F, (long)(cj + g1) * pitch + (ci + g0), tmp, A);
    }
  }
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------

RhsConst make_rhs_const(const double* xlo, const double* dx, double alpha, double kappa, double mu,
                        double muB, double R, double T_star_n, double tau_n, const double* tol, int level,
                        double c, double c_lr) {
  RhsConst P;
  P.inv_dx0 = 1.0 / dx[0];
  P.inv_dx1 = 1.0 / dx[1];
  P.inv_dx0sq = 1.0 / (dx[0] * dx[0]);
  P.inv_dx1sq = 1.0 / (dx[1] * dx[1]);
  P.inv_2dx0 = 1.0 / (2.0 * dx[0]);
  P.inv_2dx1 = 1.0 / (2.0 * dx[1]);
  P.inv_4dxdy = 1.0 / ((4.0 * dx[0]) * dx[1]);
  P.kappa = kappa;
  P.mu = mu;
  P.muB = muB;
  P.R = R;
  P.T_star_n = T_star_n;
  P.inv_tau_n = 1.0 / tau_n;
  P.alpha = alpha;
  P.c = c;
  P.c_lr = c_lr;
  P.ylo = xlo[1];
  P.dy = dx[1];
  // ep = 0.9*tolerance(2)*(xi**2)/(1-0.9*(tolerance(2)**2)), xi = 1
  // (rhs_hybrid_high_llf.m4:114-115); this file is built without FMA
  // contraction of host code so the value is the reference's.
  const double xi = 1.0;
  P.sensor_eps = ((Lit::c0_9 * tol[2]) * (xi * xi)) / (1.0 - Lit::c0_9 * (tol[2] * tol[2]));
  P.level = level;
  return P;
}

static int launch_rhs(int variant, dim3 grid, dim3 block, const double* w, const double* pres,
                      const double* temp, long pitch, long fstride, int g0, int g1, const double* H0,
                      double* KK, long opitch, long ofstride, int nx, int ny, const RhsConst& P, int* flags) {
  cudaStream_t s = stream();
#define ENL_RHS_CASE(ID, SCH, ORD, LLF_)                                                              \
  case ID:                                                                                           \
    rhs_plain_kernel<SCH, ORD, LLF_><<<grid, block, 0, s>>>(w, pres, temp, pitch, fstride, g0, g1, H0, \
                                                            KK, opitch, ofstride, nx, ny, P, flags); \
    break;
  switch (variant) {
    ENL_RHS_CASE(0, kHybrid, 5, true)
    ENL_RHS_CASE(1, kHybrid, 5, false)
    ENL_RHS_CASE(2, kHybrid, 3, true)
    ENL_RHS_CASE(3, kHybrid, 3, false)
    ENL_RHS_CASE(4, kWeno, 5, true)
    ENL_RHS_CASE(5, kWeno, 5, false)
    ENL_RHS_CASE(6, kWeno, 3, true)
    ENL_RHS_CASE(7, kWeno, 3, false)
    ENL_RHS_CASE(8, kDrp, 5, false)
    default:
      set_error(ENL_ERR_ARG);
      return ENL_ERR_ARG;
  }
#undef ENL_RHS_CASE
  return check_launch("rhs");
}

// Pitched launch used by the engine's plain path: w points at the first stored
// cell (ghost width 3 on both sides of the patch).
int launch_rhs_pitched(int variant, const double* w, const double* pres, const double* temp, long pitch,
                       long fstride, const double* H0, double* KK, long opitch, long ofstride, int nx, int ny,
                       const RhsConst& P) {
  dim3 block(32, 4);
  dim3 grid((nx + block.x - 1) / block.x, (ny + block.y - 1) / block.y);
  return launch_rhs(variant, grid, block, w, pres, temp, pitch, fstride, 3, 3, H0, KK, opitch, ofstride, nx, ny, P,
                    nullptr);
}

}  // namespace enl

using namespace enl;

static inline dim3 grid2d(int nx, int ny, dim3 b) { return dim3((nx + b.x - 1) / b.x, (ny + b.y - 1) / b.y); }

extern "C" {

int enl_rhs(int variant, int ifirst0, int ilast0, int ifirst1, int ilast1, int gcw0, int gcw1,
            const double* xlo, const double* dx, const double* w_n, long w_pitch, long w_fstride,
            const double* source, double* rhs, long out_pitch, long out_fstride, const double* pressure,
            const double* temperature, double weno_alpha, double kappa, double mu, double muB, double R,
            double T_star_n, double tau_n, const double* tag_tolerance, int level, double c, double c_lr,
            int* flags) {
  int nx = ilast0 - ifirst0 + 1, ny = ilast1 - ifirst1 + 1;
  if (nx <= 0 || ny <= 0 || gcw0 < 3 || gcw1 < 3 || !w_n || !rhs || !source || !pressure || !temperature ||
      !xlo || !dx || !tag_tolerance || w_pitch < nx + 2 * gcw0 || out_pitch < nx) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  RhsConst P = make_rhs_const(xlo, dx, weno_alpha, kappa, mu, muB, R, T_star_n, tau_n, tag_tolerance, level,
                              c, c_lr);
  dim3 block(32, 4);
  return launch_rhs(variant, grid2d(nx, ny, block), block, w_n, pressure, temperature, w_pitch, w_fstride,
                    gcw0, gcw1, source, rhs, out_pitch, out_fstride, nx, ny, P, flags);
}

void rhs_(const int& ifirst0, const int& ilast0, const int& ifirst1, const int& ilast1, const int& gcw0,
          const int& gcw1, const double* xlo, const double* dx, const double* w_n, const double* source,
          double* rhs, const double* pressure, const double* temperature, const double& weno_alpha,
          const double& kappa, const double& mu, const double& muB, const double& R, const double& T_star_n,
          const double& T_star_o, const double& tau_n, const double& tau_o, const double* tag_tolerance,
          const int& level, const double& c, const double& c_lr, const int& nequ) {
  (void)T_star_o;
  (void)tau_o;
  if (nequ != kNequ) {
    set_error(ENL_ERR_ARG);
    return;
  }
  int nx = ilast0 - ifirst0 + 1, ny = ilast1 - ifirst1 + 1;
  long pitch = nx + 2 * gcw0, fstride = pitch * (ny + 2 * gcw1);
  enl_rhs(rhs_variant(), ifirst0, ilast0, ifirst1, ilast1, gcw0, gcw1, xlo, dx, w_n, pitch, fstride, source,
          rhs, nx, (long)nx * ny, pressure, temperature, weno_alpha, kappa, mu, muB, R, T_star_n, tau_n,
          tag_tolerance, level, c, c_lr, nullptr);
}

void runge_kutta_(const int& ifirst0, const int& ilast0, const int& ifirst1, const int& ilast1,
                  const int& gcw0, const int& gcw1, const double& dt, const double& alpha_1,
                  const double& alpha_2, const double& beta, double* w_n, const double* w, const double* rhs,
                  const int& nequ) {
  int nx = ilast0 - ifirst0 + 1, ny = ilast1 - ifirst1 + 1;
  if (nx <= 0 || ny <= 0 || nequ < 1 || !w_n || !w || !rhs) {
    set_error(ENL_ERR_ARG);
    return;
  }
  long pitch = nx + 2 * gcw0, fstride = pitch * (ny + 2 * gcw1);
  dim3 block(32, 4);
  runge_kutta_kernel<<<grid2d(nx, ny, block), block, 0, stream()>>>(
      w_n, pitch, fstride, gcw0, gcw1, w, rhs, nx, (long)nx * ny, nx, ny, nequ, alpha_1, alpha_2,
      beta * dt);
  check_launch("runge_kutta");
}

void update_state_(const double* dx, const double* xlo, const int& ifirst0, const int& ilast0,
                   const int& ifirst1, const int& ilast1, const int& gcw0, const int& gcw1, const double* w_n,
                   double* pressure, double* temperature, const double& rho0, const double& c,
                   const double& gamma1, const double& c_p, const double& p0, const double& T0,
                   const double& c_lr, const double& c_v, const double& R_tilde, const double& M,
                   const double& R, const int& nequ) {
  (void)R_tilde;
  (void)M;
  (void)nequ;
  int nx = ilast0 - ifirst0 + 1, ny = ilast1 - ifirst1 + 1;
  if (nx <= 0 || ny <= 0 || !w_n || !pressure || !temperature || !dx || !xlo) {
    set_error(ENL_ERR_ARG);
    return;
  }
  long pitch = nx + 2 * gcw0, fstride = pitch * (ny + 2 * gcw1);
  StateConst S{rho0, c, (gamma1 - 1.0) / (2.0 * rho0), c_p, p0, T0, c_lr, c_v, R, xlo[1], dx[1]};
  dim3 block(32, 4);
  update_state_kernel<<<grid2d(nx, ny, block), block, 0, stream()>>>(w_n, pressure, temperature, pitch,
                                                                       fstride, gcw0, gcw1, nx, ny, S);
  check_launch("update_state");
}

void tag_cells_(const int& ifirst0, const int& ilast0, const int& ifirst1, const int& ilast1, const int& gcw0,
                const int& gcw1, int* tags, const double* w_n, const double* source, const int& refine_tag_val,
                const double* tag_tolerance, const int& nequ) {
  (void)nequ;
  int nx = ilast0 - ifirst0 + 1, ny = ilast1 - ifirst1 + 1;
  if (nx <= 0 || ny <= 0 || gcw0 < 1 || gcw1 < 1 || !tags || !w_n || !source || !tag_tolerance) {
    set_error(ENL_ERR_ARG);
    return;
  }
  long pitch = nx + 2 * gcw0;
  const double xi = 1.0;
  double ep0 = ((Lit::c0_9 * tag_tolerance[0]) * (xi * xi)) / (1.0 - Lit::c0_9 * (tag_tolerance[0] * tag_tolerance[0]));
  double ep1 = ((Lit::c0_9 * tag_tolerance[1]) * (xi * xi)) / (1.0 - Lit::c0_9 * (tag_tolerance[1] * tag_tolerance[1]));
  dim3 block(32, 4);
  tag_cells_kernel<<<grid2d(nx, ny, block), block, 0, stream()>>>(tags, nx, w_n, source, pitch, gcw0, gcw1, nx,
                                                                    ny, refine_tag_val, ep0, ep1);
  check_launch("tag_cells");
}

int enl_phys_bc(int ifirst0, int ilast0, int ifirst1, int ilast1, int gcw0, int gcw1, const int* touches,
                const int* bc, int fill0, int fill1, double* w_n, double* pressure, double* temperature,
                double* source) {
  int nx = ilast0 - ifirst0 + 1, ny = ilast1 - ifirst1 + 1;
  if (nx <= 0 || ny <= 0 || !touches || !bc || fill0 < 0 || fill1 < 0 || fill0 > gcw0 || fill1 > gcw1 || !w_n ||
      !pressure || !temperature || !source) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  long pitch = nx + 2 * gcw0, fstride = pitch * (ny + 2 * gcw1);
  PatchFields8 F;
  for (int k = 0; k < 5; ++k) F.f[k] = w_n + k * fstride;
  F.f[5] = pressure;
  F.f[6] = temperature;
  F.f[7] = source;
  cudaStream_t s = stream();
  for (int side = 0; side < 4; ++side) {
    if (!touches[side]) continue;
    int fill = side < 2 ? fill0 : fill1;
    int n = ((side < 2) ? ny : nx) * fill * 8;
    if (n == 0) continue;
    phys_bc_edge_kernel<<<(n + 127) / 128, 128, 0, s>>>(F, pitch, nx, ny, gcw0, gcw1, side, fill,
                                                        bc[side] == kReflect);
  }
  for (int loc = 0; loc < 4; ++loc) {
    int xs = loc & 1, ys = (loc >> 1) & 1;
    if (!(touches[xs ? 1 : 0] || touches[ys ? 3 : 2])) continue;
    int n = fill0 * fill1 * 8;
    if (n == 0) continue;
    phys_bc_node_kernel<<<(n + 127) / 128, 128, 0, s>>>(F, pitch, nx, ny, gcw0, gcw1, loc, fill0, fill1,
                                                        bc[xs ? 1 : 0] == kReflect);
  }
  return check_launch("phys_bc");
}

int enl_absorb(int ifirst0, int ilast0, int ifirst1, int ilast1, int gcw0, int gcw1, const double* patch_xlo,
               const double* dx, const double* grid_xlo, const double* grid_xhi, const int* bc,
               double absorb_width, double p0, double T0, double rho0, double* w_n, double* pressure,
               double* temperature) {
  int nx = ilast0 - ifirst0 + 1, ny = ilast1 - ifirst1 + 1;
  if (nx <= 0 || ny <= 0 || !patch_xlo || !dx || !grid_xlo || !grid_xhi || !bc || !w_n || !pressure ||
      !temperature) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  if (!(bc[0] == kAbsorb || bc[1] == kAbsorb || bc[2] == kAbsorb || bc[3] == kAbsorb)) return ENL_OK;
  long pitch = nx + 2 * gcw0, fstride = pitch * (ny + 2 * gcw1);
  PatchFields8 F;
  for (int k = 0; k < 5; ++k) F.f[k] = w_n + k * fstride;
  F.f[5] = pressure;
  F.f[6] = temperature;
  F.f[7] = nullptr;
  AbsorbConst A{patch_xlo[0], patch_xlo[1], dx[0], dx[1], grid_xlo[0], grid_xlo[1], grid_xhi[0], grid_xhi[1],
                absorb_width * absorb_width, p0, T0, rho0};
  cudaStream_t s = stream();
  for (int dir = 0; dir < 4; ++dir) {
    if (bc[dir] != kAbsorb) continue;
    int n = dir < 2 ? ny : nx;
    absorb_kernel<<<(n + 127) / 128, 128, 0, s>>>(F, pitch, nx, ny, gcw0, gcw1, dir, A);
  }
  return check_launch("absorb");
}

}  // extern "C"
