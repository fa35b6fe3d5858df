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
#include <array>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include "enl_cell64.cuh"
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
// The single-precision tile has rows of 40 (a TMA box row must span a
// multiple of 16 bytes: 38 floats do not, 40 do); columns 38, 39 are unused.
constexpr int kBW32 = 40;
constexpr int kPlane32 = kBH * kBW32;            // 560
constexpr int kTile32Elems = kNF * kPlane32;     // 3920
constexpr int kTileBytes32 = kTile32Elems * 4;   // 15680
// Shared-memory layout of the stage kernel.  A TMA destination must start on
// a 128-byte boundary, so every region is padded to a multiple of 128 bytes.
//   FP64 state:  [FP64 box A][FP64 box B][FP32 tile (FAST)][planes (FAST)]
//   FP32 state:  [FP32 tile A][FP32 tile B][planes]
// (the learned switch's features use the planes' space during its review)
constexpr int align128(int b) { return (b + 127) / 128 * 128; }
constexpr int kStageBufBytes = align128(kTileBytes64);            // 29824
constexpr int kTile32Bytes = align128(kTileBytes32);              // 15744
// per-tile planes of the FP32 path: u and v over the whole halo box (rows of
// kBW32), the x-fluxes F_0..4 on the 8 interior rows (rows of kBW32), the
// y-fluxes G_0..4 on the 32 interior columns (rows of 32)
constexpr int kPlaneF = kTH * kBW32;             // 320
constexpr int kPlaneG = kBH * kTW;               // 448
constexpr int kPlOffV = kPlane32, kPlOffF = 2 * kPlane32, kPlOffG = kPlOffF + 5 * kPlaneF;
constexpr int kPlanesBytes = align128((kPlOffG + 5 * kPlaneG) * 4);   // 19840
// With ENL_STAGE_UN_TMA 1, FP32 storage prefetches u^n (5 fields) and H0 of
// the tile interior with the halo box: boxes of 40 x 8 (x starts at the
// aligned column of cell i0 - 3).  By default (0) each cell loads them from
// the canvases (coalesced rows), which keeps the staging buffers small
// enough for 4 resident blocks.
#ifndef ENL_STAGE_UN_TMA
#define ENL_STAGE_UN_TMA 0
#endif
constexpr bool kUnTma = ENL_STAGE_UN_TMA != 0;
// FP32 storage without staged u^n: prefetch (to L2) the u^n and H0 values of
// each thread's cell when its tile starts.  Measured on the 3-level line
// source: hybrid 0.342 ms per launch against 0.349 ms without.
#ifndef ENL_PREFETCH_UN
#define ENL_PREFETCH_UN 1
#endif
#ifndef ENL_PREFETCH_OP
#define ENL_PREFETCH_OP "prefetch.global.L2"
#endif
constexpr int kUnBytes = 5 * kTH * kBW32 * 4;    // 6400
constexpr int kH0Bytes = kTH * kBW32 * 4;        // 1280
constexpr int kBufS = kTile32Bytes + (kUnTma ? kUnBytes + kH0Bytes : 0);  // per staging buffer
constexpr int kOffTile32 = 2 * kStageBufBytes;
constexpr int kOffPlanes = kOffTile32 + kTile32Bytes;
constexpr int kSmemFast64 = kOffPlanes + kPlanesBytes;   // dynamic shared memory, FP64 storage + FP32 rhs
constexpr int kOffPlanesS = 2 * kBufS;
// FP64 right-hand side: [FP64 box A][FP64 box B][FP64 planes]
constexpr int kOffPlanes64 = 2 * kStageBufBytes;
constexpr int kPlanes64Bytes = align128(kPl64Elems * 8);               // 38656
constexpr int kSmem64 = kOffPlanes64 + kPlanes64Bytes;                  // dynamic shared memory, FP64
static_assert(kBH * kBW == kPos64 && kBW == kBW64, "FP64 planes follow the staged box");
constexpr int kSmemFast32 = kOffPlanesS + kPlanesBytes;  // dynamic shared memory, FP32 storage
constexpr unsigned long long kWaitNs = 200000000ull;  // bounded mbarrier waits: 0.2 s of wall time
// learned switch: cells per network chunk (8 warps x 16 cells); their BF16
// features take the planes' place for the review, and the planes are built
// again after it
constexpr int kFeatRows = 128;
static_assert(kFeatRows * kFeat * 2 <= kPlanesBytes, "the features fit where the planes go");
static_assert(kFeatRows * kFeat * 2 <= align128(kPl64Elems * 8), "the features fit where the FP64 planes go");
// Resident stage blocks per SM with FP32 storage (bounds the registers per
// thread: 4 blocks of 256 threads leave 64, 3 leave 80).  Four blocks need
// the smaller staging buffers of ENL_STAGE_UN_TMA 0 (4 x 56 KB of shared
// memory); measured on the 3-level line source, 4 blocks without the u^n
// boxes run the stage in 0.346 ms against 0.371 ms for 3 blocks with them.
#ifndef ENL_STAGE_BLOCKS_F32
#define ENL_STAGE_BLOCKS_F32 4
#endif
constexpr int kStageBlocksF32 = ENL_STAGE_BLOCKS_F32;


// Absorbing envelope (enlightning.C:634-786) as per-level tables: for each
// side, env[i] = 1 - exp(-ln2 d^2 / w^2) at the distance d of cell centre i
// (column for L/R, row for B/T) from that side of the domain; null where the
// side is not ABSORB.  The tables are computed on the host once per engine.
struct AbsorbTables {
  const double* env[kL][4];
  const float* envf[kL][4];           // the same factors rounded to float
  const unsigned char* cont[kL][4];   // |1 - env| > 1e-8: the walk goes on past this cell
  // cells whose factor is not exactly 1: index < act (L, B) or >= act (R, T)
  int act[kL][4];
};

// The reference walks every patch row from the L (R) side inwards and stops
// after the first cell whose factor is within 1e-8 of 1 (on the first row it
// does not start at all when the edge cell's factor is); B and T do the same
// with whole rows.  The factors grow monotonically inwards, so whether cell
// (i, j) of patch b is reached follows from its neighbour towards the side:
// the walk is evaluated per cell.  The sides that reach the cell are returned
// (0..3 = L, R, B, T) in the reference's order.
// Bit s set when the walk from side s (0..3 = L, R, B, T) reaches the cell;
// `mask` limits the test to the sides that can reach the cell's tile
// (absorb_tile_mask).  Callers apply the sides in the reference's order.
__device__ __forceinline__ int absorb_reach(const AbsorbTables& T, int lvl, int i, int j, const int4& b,
                                            int mask = 15) {
  int r = 0;
  const unsigned char* c = T.cont[lvl][0];
  if ((mask & 1) && c && (j != b.z || c[b.x]) && (i == b.x || c[i - 1])) r |= 1;
  c = T.cont[lvl][1];
  if ((mask & 2) && c && (j != b.z || c[b.y]) && (i == b.y || c[i + 1])) r |= 2;
  c = T.cont[lvl][2];
  if ((mask & 4) && c && c[b.z] && (j == b.z || c[j - 1])) r |= 4;
  c = T.cont[lvl][3];
  if ((mask & 8) && c && c[b.w] && (j == b.w || c[j + 1])) r |= 8;
  return r;
}

// Sides whose walk can reach some cell of the w x h tile at (i0, j0) of patch
// b with a factor other than exactly 1: the continuation tests are monotone,
// so the tile's cell nearest to each side decides.  (The walk from a patch's
// own edge reaches its first cell even far from the domain side, where the
// factor is exactly 1; the batched engine leaves such cells as they are,
// which is the reference's (q - q_amb) * 1 + q_amb except for a last-place
// rounding when q is beyond twice its ambient value.)
__device__ __forceinline__ int absorb_tile_mask(const AbsorbTables& T, int lvl, int i0, int j0, int w, int h,
                                                const int4& b) {
  int m = 0;
  const unsigned char* c = T.cont[lvl][0];
  if (c && i0 < T.act[lvl][0] && (i0 == b.x || c[i0 - 1])) m |= 1;
  c = T.cont[lvl][1];
  if (c && i0 + w - 1 >= T.act[lvl][1] && (i0 + w - 1 == b.y || c[i0 + w])) m |= 2;
  c = T.cont[lvl][2];
  if (c && j0 < T.act[lvl][2] && c[b.z] && (j0 == b.z || c[j0 - 1])) m |= 4;
  c = T.cont[lvl][3];
  if (c && j0 + h - 1 >= T.act[lvl][3] && c[b.w] && (j0 + h - 1 == b.w || c[j0 + h])) m |= 8;
  return m;
}

// Per-tile values computed once by thread 0 and read by every thread after
// the next barrier.
struct TileInfo {
  int4 box;       // the tile's patch
  int absorb;     // absorb_tile_mask
  float bdtf;     // beta * dt in single precision
};

// (q - ambient) * tmp + ambient, rounding like the reference's statement
__device__ __forceinline__ double relax_(double q, double amb, double tmp) {
  return __dadd_rn(__dmul_rn(__dsub_rn(q, amb), tmp), amb);
}

// update_state (update_state.m4:90-105) on absolute FP64 values, with the
// reference's rounding; height = centre height of the cell row.
struct EosConst64 {
  double rho0, c, c_lr, gm1_over_2rho0, c_p, p0, T0, c_v, R;
  double inv_c_p, inv_c_v;  // 1/c_p, 1/c_v (eos_fast64)
};
__device__ __forceinline__ void eos_abs64(const EosConst64& E, double w0, double w3, double height, double& p,
                                          double& T) {
  const double cc = __dadd_rn(E.c, __dmul_rn(E.c_lr, height));
  const double d = __dsub_rn(w0, E.rho0);
  const double s = __ddiv_rn(w3, w0);
  const double inner =
      __dadd_rn(__dadd_rn(d, __dmul_rn(E.gm1_over_2rho0, __dmul_rn(d, d))), __dmul_rn(__ddiv_rn(w0, E.c_p), s));
  p = __dadd_rn(__dmul_rn(__dmul_rn(cc, cc), inner), E.p0);
  T = E.T0 * exp((s - E.R * log(E.rho0 / w0)) / E.c_v);
}

// The same as the batched FP64 engine computes it (stage epilogue and state
// upload alike, so the two agree bit for bit): one seeded reciprocal of rho
// (rcp64) instead of two divisions, constant divisors as factors, every
// operation explicitly rounded (no contraction differences between call
// sites).  Within a few units in the last place of eos_abs64.
__device__ __forceinline__ double row_height64(double ylo, double dy, int j) {
  return __dadd_rn(ylo, __dmul_rn(dy, (double)j + 0.5));
}
__device__ __forceinline__ void eos_fast64(const EosConst64& E, double w0, double w3, double height, double& p,
                                           double& T) {
  const double cc = __dadd_rn(E.c, __dmul_rn(E.c_lr, height));
  const double ir = rcp64(w0);
  const double d = __dsub_rn(w0, E.rho0);
  const double s = __dmul_rn(w3, ir);
  const double inner =
      __dadd_rn(__dadd_rn(d, __dmul_rn(E.gm1_over_2rho0, __dmul_rn(d, d))), __dmul_rn(__dmul_rn(w0, E.inv_c_p), s));
  p = __dadd_rn(__dmul_rn(__dmul_rn(cc, cc), inner), E.p0);
  T = __dmul_rn(E.T0, exp(__dmul_rn(__dsub_rn(s, __dmul_rn(E.R, log(__dmul_rn(E.rho0, ir)))), E.inv_c_v)));
}

// The same in single-precision perturbation form: rp = rho - rho0, w3 = rho s;
// returns p - p0 and T - T0 (log1p/expm1 keep small perturbations exact).
struct EosConst32 {
  float rho0, c, c_lr, gm1_over_2rho0, inv_c_p, T0, inv_c_v, R, inv_rho0;
};
// Every operation is explicitly rounded, so the result does not depend on
// how the compiler contracts it at each call site (the stage epilogue and the
// state upload must agree bit for bit).
__device__ __forceinline__ void eos_pert32(const EosConst32& E, float rp, float w3, float height, float& pp,
                                           float& tp) {
  const float s = __fmul_rn(w3, rcp_approx(__fadd_rn(E.rho0, rp)));
  const float ccl = __fmaf_rn(E.c_lr, height, E.c);
  const float inner = __fadd_rn(__fmaf_rn(E.gm1_over_2rho0, __fmul_rn(rp, rp), rp), __fmul_rn(w3, E.inv_c_p));
  pp = __fmul_rn(__fmul_rn(ccl, ccl), inner);
  const float x = __fmul_rn(__fmaf_rn(E.R, log1pf(__fmul_rn(rp, E.inv_rho0)), s), E.inv_c_v);
  tp = __fmul_rn(E.T0, expm1f(x));
}
// Centre height of cell row j in single precision.
__device__ __forceinline__ float row_height32(float ylo, float dy, int j) {
  return __fmaf_rn(dy, __fadd_rn((float)j, 0.5f), ylo);
}

struct StageArgs {
  CUtensorMap tmap[kL];     // input buffer, per level (halo box)
  CUtensorMap tmap_un[kL];  // FP32 storage: u^n interior box
  CUtensorMap tmap_h0[kL];  // FP32 storage: H0 interior box
  int un_is_in;             // stage 1: u^n is the staged input itself
  // canvases in the engine's storage type (double, or float perturbations)
  void* in[kL];
  void* out[kL];
  const void* un[kL];  // u^n (current buffer)
  const void* h0[kL];
  long pitch[kL], fstride[kL];
  RhsConst P[kL];
  FastConst F[kL];
  double rho0, p0, T0, c, c_lr, gm1_over_2rho0, c_p, c_v, R, ylo, dy[kL];
  int uniform;              // uniform tiles reuse a computed cell (c_lr == 0 and not dense)
  const int* tile_base;     // first table entry of the launch's tiles (null: 0)
  int learned_levels;       // levels whose plain-WENO cells the network reviews
  int tile_order;           // 0 finest level first (table from its end), 1 level 0
                            // first, 2 the two ends alternately
  int chunk;                // a block claims runs of `chunk` consecutive tiles (>= 1)
  EosConst32 E32;  // FP32-storage epilogue
  EosConst64 E64;  // FP64 epilogue
  double a1, a2, bdt, beta;
  const double* dt_dev;  // adaptive time step in device memory (or null)
  float a1f, a2f, bdtf, betaf;
  const float* dtf_dev;  // the same time step rounded to float (FP32 storage)
  const int4* tiles;
  const int* ntiles;
  int* counter;
  unsigned long long* counter64;  // tile order 3: packed level-0 / finest-end claims
  int nsm;                        // SMs (the grid's first wave of blocks)
  int* health;
  unsigned long long* stats;  // [level][4]: weno cells, cells, cells decided by the plain-sensor fallback,
                              // cells of uniform tiles stored from the cache
  AbsorbTables absorb;        // absorbing envelope, applied to each finished cell
  bool any_absorb;
  const int4* patchtab;       // patch boxes of all levels (tile .w = index)
  const MlpSmem* mlp;         // learned-sensor network image (global memory) or null
  float margin;               // |p - 0.5| <= margin -> plain sensor decides
  float feat_eps, feat_eps_p, feat_inv_sqrt_eps;
  // uniform-tile skipping (null when off).  Records of the current step,
  // per table index: stage 1 writes rec_un_out and rec_out, stage 2 writes
  // rec_out.  In stages 2 and 3 the launch runs over a list of tiles: tiles
  // holds their descriptors, gti their table indices (null: the table
  // itself), and the first uniform tile computed per level is published in
  // gcache (GUni<S>[kL]) for the skipped tiles (skip_phase).
  void* rec_out;
  void* rec_un_out;
  const int* gti;
  void* gcache;
  // the skipped tiles, taken eight at a time (one per warp) by blocks that
  // have run out of tiles to compute: their table indices (skip_n of them),
  // the previous stage's records (their keys), and the list of those without
  // a cached or published result (left_n, for a second launch)
  const int* skip_gti;
  const int* skip_n;
  int* skip_counter;
  const int4* tiles_all;  // the tile table (descriptors of the skipped tiles)
  const void* rec_in;
  const void* rec_un_in;
  int* left_n;
  int4* left_td;
  int* left_gti;
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
struct SAcc32 {  // single-precision tile and its planes
  const float* t;
  const float* pl;  // u, v, F_0..4, G_0..4
  int c;            // (row)*kBW32 + col of the centre in the halo box
  int cf, cg;       // the centre in the F planes (cy*kBW32 + cx + 3) and G planes ((cy+3)*32 + cx)
  __device__ float w(int k, int di, int dj) const { return t[k * kPlane32 + c + dj * kBW32 + di]; }
  __device__ float p(int di, int dj) const { return t[5 * kPlane32 + c + dj * kBW32 + di]; }
  __device__ float t_(int di, int dj) const { return t[6 * kPlane32 + c + dj * kBW32 + di]; }
  __device__ float u(int di, int dj) const { return pl[c + dj * kBW32 + di]; }
  __device__ float v(int di, int dj) const { return pl[kPlOffV + c + dj * kBW32 + di]; }
  __device__ float fx(int k, int di) const { return pl[kPlOffF + k * kPlaneF + cf + di]; }
  __device__ float gy(int k, int dj) const { return pl[kPlOffG + k * kPlaneG + cg + dj * kTW]; }
};
__device__ __forceinline__ SAcc32 acc32(const float* t, const float* pl, int cx, int cy) {
  return SAcc32{t, pl, (cy + 3) * kBW32 + (cx + 3), cy * kBW32 + cx + 3, (cy + 3) * kTW + cx};
}
struct SAcc32R {
  SAcc32 a;
  __device__ float w(int k, int di, int dj) const { return a.w(k, di, dj); }
  __device__ float p(int di, int dj) const { return a.p(di, dj); }
  __device__ float t(int di, int dj) const { return a.t_(di, dj); }
  __device__ float u(int di, int dj) const { return a.u(di, dj); }
  __device__ float v(int di, int dj) const { return a.v(di, dj); }
  __device__ float fx(int k, int di) const { return a.fx(k, di); }
  __device__ float gy(int k, int dj) const { return a.gy(k, dj); }
};

__device__ __forceinline__ void raise_health(int* h, int code) { atomicCAS(h, 0, code); }

// Per-block cache of the result of a uniform tile: a tile whose staged halo
// box holds one value per field, bit for bit, and whose cells share their
// u^n and H0 values (and lie in no absorbing band, with c_lr = 0) has the
// same inputs in every cell, so every cell computes the same outputs.  The
// first such tile of a level is computed in full and its cell (0, 0) records
// its inputs (key) and outputs (res); a later uniform tile of the level with
// the same key stores res without computing it.  The results are those of
// the full computation by construction.
template <typename S>
struct UniEntry {
  S key[13];  // the 7 staged fields, u^n (5), H0
  S res[7];   // the 7 stored fields of a cell
  int weno;   // the switch decision
  int valid;
};
__device__ __forceinline__ bool same_bits(double a, double b) {
  return __double_as_longlong(a) == __double_as_longlong(b);
}
__device__ __forceinline__ bool same_bits(float a, float b) { return __float_as_int(a) == __float_as_int(b); }

// Records of one step for skipping uniform tiles.  Within a step nothing but
// the stage kernels writes patch interiors (ghost fills write ghosts, the
// coarsening follows the last stage), so what stage 1 and stage 2 record
// about the tiles they wrote still holds when the next stage reads it:
//   OutRec: the tile's stored outputs, when every cell of the tile holds the
//           same 7 values (a uniform tile, from the cache or computed);
//   UnRec:  the tile's u^n (5 fields) and H0, when uniform over its cells and
//           the tile lies in no absorbing band (from stage 1's uniform test).
// A tile of stage 2 or 3 whose own input record and its eight neighbours'
// (all in its patch, each reaching at least 3 cells into the halo) hold the
// same values has a uniform halo box with those values: with a matching
// cache entry its outputs are the entry's, and the box is not loaded.
template <typename S>
struct alignas(16) OutRec {
  S v[7];
  int valid;
};
template <typename S>
struct alignas(16) UnRec {
  S v[6];  // u^n (5 fields), H0
  int valid;
};
static_assert(sizeof(OutRec<double>) == 64 && sizeof(UnRec<double>) == 64, "FP64 records: 64 bytes");
static_assert(sizeof(OutRec<float>) == 32 && sizeof(UnRec<float>) == 32, "FP32 records: 32 bytes");

// Per tile: 1 when the stage's input records prove the tile's halo box
// uniform (nbr[8 t .. 8 t + 7]: the tiles whose interiors hold its halo, or
// -1 first when they do not).  Block b takes tiles [256 b, 256 b + 256) and
// writes its count of tiles to compute and to skip to bcnt[b].
constexpr int kFlagThreads = 256;
template <typename S>
__global__ void __launch_bounds__(kFlagThreads) skip_flags_kernel(const int* nbr, const int* ntiles,
                                                                  const OutRec<S>* rin, const UnRec<S>* run,
                                                                  unsigned char* flag, int2* bcnt) {
  const int n = *ntiles;
  const int t = blockIdx.x * kFlagThreads + threadIdx.x;
  if (blockIdx.x * kFlagThreads >= n) return;  // (the whole block: no barrier below is left half-way)
  bool ok = false;
  if (t < n) {
    const int4 n0 = reinterpret_cast<const int4*>(nbr)[2 * t], n1 = reinterpret_cast<const int4*>(nbr)[2 * t + 1];
    ok = n0.x >= 0 && run[t].valid != 0 && rin[t].valid != 0;
    if (ok) {
      const OutRec<S> c = rin[t];
      const int q[8] = {n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, n1.z, n1.w};
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const OutRec<S> r = rin[q[m]];
        ok = ok && r.valid != 0;
#pragma unroll
        for (int k = 0; k < 7; ++k) ok = ok && same_bits(r.v[k], c.v[k]);
      }
    }
    flag[t] = ok ? 1 : 0;
  }
  const int nskip = __syncthreads_count(ok);
  if (threadIdx.x == 0) bcnt[blockIdx.x] = make_int2(min(kFlagThreads, n - blockIdx.x * kFlagThreads) - nskip, nskip);
}

// Input k of a uniform tile: the staged fields (0..6), u^n (7..11: the staged
// fields 0..4 in stage 1, else the first cell's values) and H0 (12).
template <typename S, int kPl>
__device__ __forceinline__ S uni_key(const S* box, const S* first, int un_is_in, int k) {
  return k < 7 ? box[k * kPl] : (k < 12 ? (un_is_in ? box[(k - 7) * kPl] : first[k - 7]) : first[5]);
}

// The uniform-tile test of the stage kernel, in two out-of-line parts (the
// stage kernel's cell computation keeps its registers) around one block
// barrier in the kernel.  uniform_probe: this thread's part of the test, after
// the tile's halo box has landed in `box` (kPl elements per field, rows of
// kRow): its share of the box equals each field's first element, and its
// cell's u^n and H0 equal those of the first cell of its warp, whose values
// lane 0 writes to wl[warp] (the caller loaded them before the tile's wait,
// zero in stage 1 where u^n is the staged box).  uniform_hit, after the barrier's AND of the
// probes: 0 when the tile is not uniform; 1 when it is and the level's cache
// entry holds its inputs (the cached outputs are stored into every cell of
// the tile and counted); 2 when it is uniform and must be computed (the
// caller's cell (0, 0) then fills the entry).  Neither contains a barrier.
template <typename S, int kPl, int kRow>
__device__ __noinline__ bool uniform_probe(const S* box, S (*wl)[6], int w, int h, S u0, S u1, S u2, S u3, S u4,
                                           S hv) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool valid = lane < w && warp < h;
  const S v[6] = {u0, u1, u2, u3, u4, hv};  // u^n (5 fields) and H0 of this thread's cell
  // the staged box 16 bytes at a time, every element against its field's
  // first element (bit patterns OR-ed together: zero when all equal)
  bool ok;
  if constexpr (std::is_same<S, double>::value) {
    static_assert(kRow == 38 && kPl == 532, "FP64 box: rows of 38, 14 rows");
    const double2* b2 = reinterpret_cast<const double2*>(box);
    unsigned long long acc = 0ull;
    for (int q = tid; q < kNF * (kPl / 2); q += 256) {
      const int k = q / (kPl / 2);
      const unsigned long long ref = (unsigned long long)__double_as_longlong(box[k * kPl]);
      const double2 x = b2[q];
      acc |= ((unsigned long long)__double_as_longlong(x.x) ^ ref) | ((unsigned long long)__double_as_longlong(x.y) ^ ref);
    }
    ok = acc == 0ull;
  } else {
    static_assert(kRow == 40 && kPl == 560, "FP32 box: rows of 40 (38 used), 14 rows");
    const float4* b4 = reinterpret_cast<const float4*>(box);
    unsigned acc = 0u;
    for (int q = tid; q < kNF * (kPl / 4); q += 256) {
      const int k = q / (kPl / 4), cv = (q - k * (kPl / 4)) % (kRow / 4);
      const unsigned ref = __float_as_uint(box[k * kPl]);
      const float4 x = b4[q];
      unsigned d = (__float_as_uint(x.x) ^ ref) | (__float_as_uint(x.y) ^ ref);
      if (cv != kRow / 4 - 1) d |= (__float_as_uint(x.z) ^ ref) | (__float_as_uint(x.w) ^ ref);  // columns 38, 39 unused
      acc |= d;
    }
    ok = acc == 0u;
  }
  // every lane takes part in the shuffle (a lane without a cell included:
  // the full-mask shuffle waits for all 32), only cells compare
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const S first = __shfl_sync(0xffffffffu, v[k], 0);
    if (valid && !same_bits(v[k], first)) ok = false;
    if (lane == 0 && valid) wl[warp][k] = v[k];
  }
  return ok;
}

template <typename S, int kPl>
__device__ __noinline__ int uniform_hit(const StageArgs& A, const S* box, const UniEntry<S>* uc, const S (*wl)[6],
                                        unsigned* stats, int lvl, int i0, int j0, int w, int h) {
  for (int q = 1; q < h; ++q)
#pragma unroll
    for (int k = 0; k < 6; ++k)
      if (!same_bits(wl[q][k], wl[0][k])) return 0;
  const UniEntry<S>& U = uc[lvl];
  bool hit = U.valid != 0;
#pragma unroll
  for (int k = 0; k < 13; ++k) hit = hit && same_bits(uni_key<S, kPl>(box, wl[0], A.un_is_in, k), U.key[k]);
  if (!hit) return 2;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (lane < w && warp < h) {
    S* out = static_cast<S*>(A.out[lvl]);
    const long fs = A.fstride[lvl];
    const long gc = (long)(j0 + warp + 3) * A.pitch[lvl] + (i0 + lane + 3);
#pragma unroll
    for (int k = 0; k < kNF; ++k) out[k * fs + gc] = U.res[k];
  }
  if (tid == 0) {
    stats[4 * lvl + 0] += U.weno ? (unsigned)(w * h) : 0u;
    stats[4 * lvl + 1] += (unsigned)(w * h);
    stats[4 * lvl + 3] += (unsigned)(w * h);
  }
  return 1;
}

// The cache entry of a uniform tile computed in full: its inputs and the
// outputs of its cell (0, 0).
template <typename S, int kPl>
__device__ __noinline__ void uniform_record(UniEntry<S>* U, const S* box, const S* first, int un_is_in, S w0, S w1,
                                            S w2, S w3, S w4, S pv, S tv, int weno) {
#pragma unroll
  for (int k = 0; k < 13; ++k) U->key[k] = uni_key<S, kPl>(box, first, un_is_in, k);
  U->res[0] = w0;
  U->res[1] = w1;
  U->res[2] = w2;
  U->res[3] = w3;
  U->res[4] = w4;
  U->res[5] = pv;
  U->res[6] = tv;
  U->weno = weno;
  U->valid = 1;
}

// The first uniform tile a stage launch computes on a level publishes its
// inputs and outputs (the block-cache entry it just filled) for the skipped
// tiles that blocks without that entry take at the end of the launch: state
// 0 empty, 1 being written, 2 complete.
template <typename S>
struct GUni {
  S key[13];
  S res[7];
  int weno;
  int state;
};
template <typename S>
__device__ __forceinline__ void publish_uniform(GUni<S>* G, const UniEntry<S>& U) {
  if (atomicCAS(&G->state, 0, 1) != 0) return;
#pragma unroll
  for (int k = 0; k < 13; ++k) G->key[k] = U.key[k];
#pragma unroll
  for (int k = 0; k < 7; ++k) G->res[k] = U.res[k];
  G->weno = U.weno;
  __threadfence();
  atomicExch(&G->state, 2);
}

// A computed uniform tile's record: the outputs of its first cell.
template <typename S, typename W>
__device__ __forceinline__ void record_out(OutRec<S>* ro, const W* wn, S pv, S tv) {
#pragma unroll
  for (int k = 0; k < 5; ++k) ro->v[k] = (S)wn[k];
  ro->v[5] = pv;
  ro->v[6] = tv;
  ro->valid = 1;
}

// The skipped tiles of a stage launch (stages 2 and 3 with skipping), taken
// by blocks that have run out of tiles to compute, eight per claim, one per
// warp: lanes 0..12 load the tile's key from the previous stage's records;
// the block's cache entry for the level, or else the launch's published
// result, with that key gives the outputs of every cell (stored eight rows of
// 32, and recorded for the next stage), as a cache hit of the full path
// would; a tile with neither goes to the list of the second launch.  Called
// by the whole block after its last computed tile (all its copies landed).
template <typename S>
__device__ __noinline__ void skip_phase(const StageArgs& A, const UniEntry<S>* uc, unsigned* stats, int* s_claim) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ns = *A.skip_n;
  const OutRec<S>* rin = static_cast<const OutRec<S>*>(A.rec_in);
  const UnRec<S>* run = static_cast<const UnRec<S>*>(A.rec_un_in);
  OutRec<S>* rout = static_cast<OutRec<S>*>(A.rec_out);
  const GUni<S>* gc = static_cast<const GUni<S>*>(A.gcache);
  for (;;) {
    __syncthreads();  // (the claim slot is free)
    if (tid == 0) s_claim[0] = atomicAdd(A.skip_counter, 8);
    __syncthreads();
    const int q = s_claim[0] + warp;
    if (q - warp >= ns) break;
    if (q >= ns) continue;
    const int gi = A.skip_gti[q];
    const int4 td = A.tiles_all[gi];
    const int lvl = td.z & 0xff, w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    S kv = S(0);
    if (lane < 7) kv = rin[gi].v[lane];
    else if (lane < 13) kv = run[gi].v[lane - 7];
    // the block's cache entry first, then the published result (read after
    // its completed state, past L1)
    const UniEntry<S>& U = uc[lvl];
    bool hit = __all_sync(0xffffffffu, U.valid != 0 && (lane >= 13 || same_bits(kv, U.key[lane])));
    S rv = S(0);
    int weno = 0;
    if (hit) {
      if (lane < 7) rv = U.res[lane];
      weno = U.weno;
    } else {
      const GUni<S>* G = gc + lvl;
      const int state = *reinterpret_cast<const volatile int*>(&G->state);
      __threadfence();
      const volatile S* gk = G->key;
      hit = __all_sync(0xffffffffu, state == 2 && (lane >= 13 || same_bits(kv, (S)gk[lane])));
      if (hit) {
        if (lane < 7) rv = ((const volatile S*)G->res)[lane];
        weno = *reinterpret_cast<const volatile int*>(&G->weno);
      }
    }
    if (hit) {
      S res[7];
#pragma unroll
      for (int k = 0; k < 7; ++k) res[k] = __shfl_sync(0xffffffffu, rv, k);
      if (lane < w) {
        S* o = static_cast<S*>(A.out[lvl]) + (long)(td.y + 3) * A.pitch[lvl] + (td.x + lane + 3);
        for (int r = 0; r < h; ++r)
#pragma unroll
          for (int k = 0; k < kNF; ++k) o[k * A.fstride[lvl] + (long)r * A.pitch[lvl]] = res[k];
      }
      if (lane == 0) {
        if (weno) atomicAdd(&stats[4 * lvl + 0], (unsigned)(w * h));
        atomicAdd(&stats[4 * lvl + 1], (unsigned)(w * h));
        atomicAdd(&stats[4 * lvl + 3], (unsigned)(w * h));
      }
      if (rout && lane < 8) {
        if (lane < 7) rout[gi].v[lane] = rv;
        else rout[gi].valid = 1;
      }
    } else if (lane == 0) {
      const int k = atomicAdd(A.left_n, 1);
      A.left_td[k] = td;
      A.left_gti[k] = gi;
    }
  }
}

// ---------------------------------------------------------------------------
// Fused persistent stage kernel: per tile, TMA-stage the (32+6)x(8+6) halo box
// of all 7 fields, decide WENO/DRP per cell, compact the cells so that each
// warp runs one branch, compute KK, and finish the cell in place:
// w = a1*u^n + a2*w + beta*dt*KK, then p and T (update_state).
//
// S is the storage type of the canvases.  S = double: absolute values, the
// right-hand side in FP64 from per-tile FP64 planes (FAST = false) or in FP32
// perturbation form after a conversion of the staged box (FAST = true).
// S = float (FAST only): the canvases hold perturbations about the ambient
// state, the box is staged straight into the FP32 tile and the whole cell
// update is single precision.
// ---------------------------------------------------------------------------
template <int SCHEME, int ORDER, bool LLF, bool FAST, typename S>
__global__ void __launch_bounds__(256, std::is_same<S, float>::value ? kStageBlocksF32 : 2)
    stage_kernel(const __grid_constant__ StageArgs A) {
  constexpr bool kF32S = std::is_same<S, float>::value;
  static_assert(!kF32S || FAST, "single-precision storage runs the FP32 right-hand side");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // TMA destinations: two FP64 boxes (FP64 storage) or two FP32 tiles (FP32
  // storage); the next tile's copy overlaps the current tile's compute
  unsigned char* dst[2] = {smem_raw, smem_raw + (kF32S ? kBufS : kStageBufBytes)};
  float* tile32_conv = reinterpret_cast<float*>(smem_raw + kOffTile32);  // FP64 storage, FAST
  float* planes = reinterpret_cast<float*>(smem_raw + (kF32S ? kOffPlanesS : kOffPlanes));  // FAST
  double* planes64 = reinterpret_cast<double*>(smem_raw + kOffPlanes64);  // FP64 right-hand side
  // learned sensor (hybrid only): features of up to kFeatRows cells at a
  // time in the planes' place; the network image stays in global memory
  __nv_bfloat16* feat = reinterpret_cast<__nv_bfloat16*>(FAST ? (void*)planes : (void*)planes64);
  __shared__ unsigned char s_flag[256];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ int s_t[2];
  __shared__ int4 s_td[2];  // descriptors of the staged tiles
  __shared__ int s_ti[2];   // their table indices
  __shared__ unsigned s_stats[4 * kL];
  __shared__ int s_cnt[2][8];
  __shared__ int s_list[256];
  __shared__ TileInfo s_tile;
  __shared__ UniEntry<S> s_uc[kL];
  __shared__ S s_wl[8][6];  // per warp: u^n (5 fields) and H0 of its first cell
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ntiles = *A.ntiles;
  const int tbase = A.tile_base ? *A.tile_base : 0;
  // the block's next tile: the rest of its run of A.chunk consecutive tiles
  // (neighbours in the table: the next tile to the right in a patch row),
  // then a new run from the counter
  auto claim_next = [&](int cur) -> int {
    if (A.tile_order == 3) {
      // two streams on one packed counter (level-0 claims in the low half,
      // finest-end claims in the high half): the first wave of blocks (one
      // per SM) takes tiles from the finest end of the table, the second
      // from level 0, so an SM keeps an FP64-heavy block while fine tiles
      // remain; a claim is valid while the streams have not met (each side's
      // indices are distinct, and an index claimed by one side after the
      // other claimed it would see the sum reach ntiles)
      const bool from_end = ((blockIdx.x / A.nsm) & 1) == 0;
      const unsigned long long old = atomicAdd(A.counter64, from_end ? (1ull << 32) : 1ull);
      const unsigned long long f = old & 0xffffffffull, bk = old >> 32;
      if (f + bk >= (unsigned long long)ntiles) return ntiles;
      return from_end ? ntiles - 1 - (int)bk : (int)f;
    }
    if (cur >= 0 && (cur + 1) % A.chunk != 0 && cur + 1 < ntiles) return cur + 1;
    return atomicAdd(A.counter, A.chunk);
  };
  auto issue = [&](int t, int b) {
    // claim order -> table index (the table runs level 0 to the finest);
    // order 2 takes the two ends alternately, so that fine-level WENO tiles
    // (FP64-bound) and level-0 tiles (memory-bound) run side by side
    const int ti = (A.tile_order == 1 || A.tile_order == 3) ? t  // order 3 claims table indices
                   : A.tile_order == 2 ? ((t & 1) ? (t >> 1) : ntiles - 1 - (t >> 1))
                                       : ntiles - 1 - t;
    const int4 td = A.tiles[tbase + ti];
    const int gi = A.gti ? A.gti[tbase + ti] : tbase + ti;
    s_td[b] = td;
    s_ti[b] = gi;
    // a tiled TMA copy needs x * sizeof(S) to be a multiple of 16: x even for
    // doubles, a multiple of 4 for floats; set_patches only accepts such
    // patch origins and tiles are 32 wide
    if (td.x & (kF32S ? 3 : 1)) {
      raise_health(A.health, ENL_ERR_STATE);
      return false;
    }
    fence_proxy_async_smem();
    const int lv = td.z & 0xff;
    if constexpr (kF32S) {
      // halo box, and the interior rows of u^n (unless u^n is the input) and H0;
      // canvas column of cell i0-3 is i0, canvas row of cell j0 is j0+3
      if (kUnTma) {
        mbar_arrive_expect_tx(&mbar[b], kTileBytes32 + (A.un_is_in ? 0 : kUnBytes) + kH0Bytes);
        tma_load_3d(dst[b], &A.tmap[lv], td.x, td.y, 0, &mbar[b]);
        if (!A.un_is_in) tma_load_3d(dst[b] + kTile32Bytes, &A.tmap_un[lv], td.x, td.y + 3, 0, &mbar[b]);
        tma_load_3d(dst[b] + kTile32Bytes + kUnBytes, &A.tmap_h0[lv], td.x, td.y + 3, 0, &mbar[b]);
      } else {
        mbar_arrive_expect_tx(&mbar[b], kTileBytes32);
        tma_load_3d(dst[b], &A.tmap[lv], td.x, td.y, 0, &mbar[b]);
      }
    } else {
      mbar_arrive_expect_tx(&mbar[b], kTileBytes64);
      // canvas column of cell i0-3 is i0 (ghost offset 3)
      tma_load_3d(dst[b], &A.tmap[lv], td.x, td.y, 0, &mbar[b]);
    }
    return true;
  };
  // TMA destinations must start on 128-byte boundaries; refuse to run otherwise
  if ((smem_u32(smem_raw) & 127u) != 0u) {
    if (tid == 0) raise_health(A.health, ENL_ERR_STATE);
    return;
  }
  const bool learned = SCHEME == kHybrid && A.mlp != nullptr;
  if (tid < kL) s_uc[tid].valid = 0;
  if (tid == 0) {
    for (int q = 0; q < 4 * kL; ++q) s_stats[q] = 0u;
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_mbar_init();
    int t = claim_next(-1);
    if (t < ntiles && !issue(t, 0)) t = ntiles;
    s_t[0] = t;
  }
  __syncthreads();
  uint32_t phase[2] = {0u, 0u};
  int b = 0;
  int t = s_t[0];
  while (t < ntiles) {
    if (tid == 0) {
      int nt = claim_next(t);
      if (nt < ntiles && !issue(nt, b ^ 1)) nt = ntiles;
      s_t[b ^ 1] = nt;
    }
    const double* tile = reinterpret_cast<const double*>(dst[b]);  // FP64 storage
    float* tile32 = kF32S ? reinterpret_cast<float*>(dst[b]) : tile32_conv;
    const int4 td = s_td[b];
    const int gti = s_ti[b];
    const int lvl = td.z & 0xff, w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    const int i0 = td.x, j0 = td.y;
    const int tx = lane, ty = warp;
    const bool valid = tx < w && ty < h;
    // u^n and H0 of this thread's cell, for the uniform-tile test: loaded
    // before the wait, so that their latency overlaps it
    S un_c[5] = {S(0), S(0), S(0), S(0), S(0)}, h0_c = S(0);
    if (A.uniform && valid) {
      const long g = (long)(j0 + ty + 3) * A.pitch[lvl] + (i0 + tx + 3);
      h0_c = static_cast<const S*>(A.h0[lvl])[g];
      if (!A.un_is_in)
#pragma unroll
        for (int k = 0; k < 5; ++k) un_c[k] = static_cast<const S*>(A.un[lvl])[k * A.fstride[lvl] + g];
    }
#if ENL_PREFETCH_UN
    if constexpr (kF32S && !kUnTma) {
      // u^n and H0 of this thread's cell are read in the epilogue: start
      // their way towards the SM now
      if (!A.uniform && valid) {
        const long g = (long)(j0 + ty + 3) * A.pitch[lvl] + (i0 + tx + 3);
        const float* h0p = static_cast<const float*>(A.h0[lvl]) + g;
        asm volatile(ENL_PREFETCH_OP " [%0];" ::"l"(h0p));
        if (!A.un_is_in) {
          const float* up = static_cast<const float*>(A.un[lvl]) + g;
#pragma unroll
          for (int k = 0; k < 5; ++k) asm volatile(ENL_PREFETCH_OP " [%0];" ::"l"(up + k * A.fstride[lvl]));
        }
      }
    }
#endif
    if (!mbar_wait_timed(&mbar[b], phase[b], kWaitNs)) {
      if (tid == 0) raise_health(A.health, ENL_ERR_TIMEOUT);
      // let copies in flight land (bounded) before the block leaves
      mbar_wait_timed(&mbar[b], phase[b], kWaitNs);
      mbar_wait_timed(&mbar[b ^ 1], phase[b ^ 1], kWaitNs);
      break;
    }
    phase[b] ^= 1u;
    // beta*dt of this stage (dt from the device CFL reduction when adaptive)
    const double bdt = kF32S ? 0.0 : (A.dt_dev ? A.beta * (*A.dt_dev) : A.bdt);
    if (tid == 0) {
      const int4 pb = A.patchtab[td.w];
      s_tile.box = pb;
      s_tile.absorb = A.any_absorb ? absorb_tile_mask(A.absorb, lvl, i0, j0, w, h, pb) : 0;
      s_tile.bdtf = A.dtf_dev ? A.betaf * (*A.dtf_dev) : A.bdtf;
    }
    // ---- uniform tile: one value per staged field, shared u^n and H0 ----
    constexpr int kPl = kF32S ? kPlane32 : kBH * kBW;  // elements per staged field
    int ucode = 0;
    if (A.uniform) {
      const S* box = reinterpret_cast<const S*>(dst[b]);
      const bool ok = uniform_probe<S, kPl, kF32S ? kBW32 : kBW>(box, s_wl, w, h, un_c[0], un_c[1], un_c[2],
                                                                 un_c[3], un_c[4], h0_c);
      const bool all = __syncthreads_and(ok) != 0;  // (also publishes s_tile and s_wl)
      if (all && s_tile.absorb == 0) ucode = uniform_hit<S, kPl>(A, box, s_uc, s_wl, s_stats, lvl, i0, j0, w, h);
      // this step's records of the tile (a computed uniform tile, ucode 2,
      // records its outputs where its first cell records the cache entry)
      if (tid == 0 && A.rec_un_out) {
        UnRec<S>* rn = static_cast<UnRec<S>*>(A.rec_un_out) + gti;
        if (ucode != 0)
#pragma unroll
          for (int k = 0; k < 6; ++k) rn->v[k] = uni_key<S, kPl>(box, s_wl[0], A.un_is_in, 7 + k);
        rn->valid = ucode != 0 ? 1 : 0;
      }
      if (tid == 0 && A.rec_out && ucode != 2) {
        OutRec<S>* ro = static_cast<OutRec<S>*>(A.rec_out) + gti;
        if (ucode == 1)
#pragma unroll
          for (int k = 0; k < 7; ++k) ro->v[k] = s_uc[lvl].res[k];
        ro->valid = ucode == 1 ? 1 : 0;
      }
    }
    // a uniform tile whose outputs came from the cache (ucode 1) goes to the
    // end of the tile; one missing from the cache (ucode 2) is computed in
    // full and its cell (0, 0) fills the entry (after the barriers that
    // follow, when no thread reads it)
    const bool uni = ucode == 2;
    if (ucode != 1) {
      if (FAST && !kF32S) {
        // FP64 box (rows of kBW) -> FP32 perturbations (rows of kBW32)
        for (int e = tid; e < kTileElems; e += 256) {
          const int k = e / (kBH * kBW), r = e - k * (kBH * kBW);
          const int row = r / kBW, col = r - row * kBW;
          double v = tile[e];
          double amb = k == 0 ? A.rho0 : (k == 4 ? A.rho0 * A.T0 : (k == 5 ? A.p0 : (k == 6 ? A.T0 : 0.0)));
          tile32[k * kPlane32 + row * kBW32 + col] = (float)(v - amb);
        }
        __syncthreads();
      }
      // switch first: it reads the staged density only, so the barrier that
      // completes the planes also tells whether the tile has a WENO cell
      int flag = 0;
      if (valid) {
        if constexpr (FAST) {
          SAcc32R acc{acc32(tile32, planes, tx, ty)};
          flag = SCHEME == kWeno ? 1 : (SCHEME == kDrp ? 0 : sensor_fast(acc, A.F[lvl]));
        } else {
          flag = switch64<SCHEME>(acc64p(tile, planes64, tx, ty), A.P[lvl]);
        }
      }
      unsigned bd = __ballot_sync(0xffffffffu, valid && !flag);
      unsigned bw = __ballot_sync(0xffffffffu, valid && flag);
      // planes of u, v and the fluxes at every halo position of the tile
      auto build_planes = [&]() {
        if constexpr (FAST) {
          const float rho0f = A.F[lvl].rho0, rT0f = A.F[lvl].rho0T0;
          // kBH * kBW = 532 positions: the 20 of the third pass fall on the last
          // warp, not on warp 0, which also stages the next tile
          for (int e = 255 - tid; e < kBH * kBW; e += 256) {
            const int row = e / kBW, col = e - row * kBW, o = row * kBW32 + col;
            const float ir = rcp_approx(rho0f + tile32[o]);
            const float u = tile32[kPlane32 + o] * ir, v = tile32[2 * kPlane32 + o] * ir;
            const float pp = tile32[5 * kPlane32 + o];
            planes[o] = u;
            planes[kPlOffV + o] = v;
            float wk[5];
#pragma unroll
            for (int k = 0; k < 5; ++k) wk[k] = tile32[k * kPlane32 + o] + (k == 0 ? rho0f : (k == 4 ? rT0f : 0.0f));
            if (row >= 3 && row < 3 + kTH) {  // x-fluxes on the interior rows
#pragma unroll
              for (int k = 0; k < 5; ++k)
                planes[kPlOffF + k * kPlaneF + (row - 3) * kBW32 + col] = fmaf(u, wk[k], k == 1 ? pp : 0.0f);
            }
            if (col >= 3 && col < 3 + kTW) {  // y-fluxes on the interior columns
#pragma unroll
              for (int k = 0; k < 5; ++k)
                planes[kPlOffG + k * kPlaneG + row * kTW + (col - 3)] = fmaf(v, wk[k], k == 2 ? pp : 0.0f);
            }
          }
        } else {
          // FP64: one seeded reciprocal of rho per halo position; the flux
          // planes hold half fluxes, formed from u/2, v/2 and p/2 (halving
          // is exact, so each is F/2 or G/2 of the same double)
          for (int e = 255 - tid; e < kPos64; e += 256) {
            const int row = e / kBW64, col = e - row * kBW64;
            const double ir = rcp64(tile[e]);
            const double u = tile[kPos64 + e] * ir, v = tile[2 * kPos64 + e] * ir;
            const double hp = 0.5 * tile[5 * kPos64 + e];
            planes64[e] = u;
            planes64[kPl64OffV + e] = v;
            if (row >= 3 && row < 3 + kTH) {
              const double hu = 0.5 * u;
#pragma unroll
              for (int k = 0; k < 5; ++k)
                planes64[kPl64OffF + k * kPl64F + (row - 3) * kBW64 + col] =
                    k == 1 ? fma(hu, tile[kPos64 + e], hp) : hu * tile[k * kPos64 + e];
            }
            if (col >= 3 && col < 3 + kTW) {
              const double hv = 0.5 * v;
#pragma unroll
              for (int k = 0; k < 5; ++k)
                planes64[kPl64OffG + k * kPl64G + row * kTW + (col - 3)] =
                    k == 2 ? fma(hv, tile[2 * kPos64 + e], hp) : hv * tile[k * kPos64 + e];
            }
          }
        }
      };
      // the learned review (tiles with WENO cells on level 0, or on every
      // level: on the fine levels the plain decision is WENO for every cell)
      // keeps its features where the planes are and rebuilds them after it
      const bool review = learned && lvl < A.learned_levels;
      build_planes();
      // compaction counts: DRP cells first, then WENO cells, each in tile order
      int nd = 0, nw = 0, od = 0, ow = 0;
      if constexpr (SCHEME == kWeno) {  // every cell WENO: the natural order
        __syncthreads();
        nw = w * h;
      } else if (!__syncthreads_or(bw != 0u)) {
        nd = w * h;  // no WENO cell: the natural order, no counts needed
      } else {
        if (lane == 0) {
          s_cnt[0][warp] = __popc(bd);
          s_cnt[1][warp] = __popc(bw);
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          if (q < warp) {
            od += s_cnt[0][q];
            ow += s_cnt[1][q];
          }
          nd += s_cnt[0][q];
          nw += s_cnt[1][q];
        }
      }
      int nfb = 0;
      if (review && nw > 0) {
        // learned switch: it refines the plain one and can only send cells the
        // plain switch put on WENO back to DRP.  Those cells (numbered in tile
        // order by the counts above) go through the BF16 MLP on the tensor
        // cores in chunks of kFeatRows, one warp per 16 cells; cells with
        // |logit| <= margin keep the plain decision.  Tiles without such cells
        // pay nothing; tiles with them build their planes twice.
        const int slot = ow + __popc(bw & ((1u << lane) - 1u));
        for (int c0 = 0; c0 < nw; c0 += kFeatRows) {
          if (valid && flag && slot >= c0 && slot < c0 + kFeatRows) {
            float fv[kFeat];
            if constexpr (FAST) {
              SAcc32R acc{acc32(tile32, planes, tx, ty)};
              cell_features(acc, A.feat_eps, A.feat_eps_p, A.feat_inv_sqrt_eps, fv);
            } else {
              SAcc64Feat acc{tile, (ty + 3) * kBW64 + tx + 3, A.rho0, A.p0};
              cell_features(acc, A.feat_eps, A.feat_eps_p, A.feat_inv_sqrt_eps, fv);
            }
#pragma unroll
            for (int q = 0; q < kFeat; q += 2)
              *reinterpret_cast<uint32_t*>(feat + (slot - c0) * kFeat + q) = pack_bf16(fv[q], fv[q + 1]);
            s_list[slot - c0] = tid;
          }
          __syncthreads();
          const int g0 = warp * 16;
          if (g0 < kFeatRows && c0 + g0 < nw) {
            float logit[2];
            mlp_logits16(*A.mlp, feat + g0 * kFeat, kFeat, lane, logit);
            if ((lane & 3) == 0) {
#pragma unroll
              for (int hh = 0; hh < 2; ++hh) {
                const int sl = g0 + (lane >> 2) + 8 * hh;
                if (c0 + sl < nw)
                  s_flag[s_list[sl]] =
                      (unsigned char)(logit[hh] > 0.f ? 2 : 1) | (fabsf(logit[hh]) <= A.margin ? 4 : 0);
              }
            }
          }
          __syncthreads();
        }
        int fallback = 0;
        if (valid && flag) {
          const unsigned char d = s_flag[tid];
          if (d & 4) fallback = 1;       // plain decision (WENO) kept
          else flag = (d & 2) ? 1 : 0;
        }
        nfb = __syncthreads_count(fallback);  // also orders the counts' reuse below
        bd = __ballot_sync(0xffffffffu, valid && !flag);
        bw = __ballot_sync(0xffffffffu, valid && flag);
        if (lane == 0) {
          s_cnt[0][warp] = __popc(bd);
          s_cnt[1][warp] = __popc(bw);
        }
        __syncthreads();
        nd = nw = od = ow = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          if (q < warp) {
            od += s_cnt[0][q];
            ow += s_cnt[1][q];
          }
          nd += s_cnt[0][q];
          nw += s_cnt[1][q];
        }
        build_planes();  // the features took the planes' place
        __syncthreads();
      }
      // a tile without WENO cells keeps its natural order (no list, no barrier)
      const bool direct = SCHEME == kWeno || nw == 0;  // one branch for the whole tile
      if (valid && !direct) {
        unsigned lt = (1u << lane) - 1u;
        int pos = flag ? (nd + ow + __popc(bw & lt)) : (od + __popc(bd & lt));
        s_list[pos] = (ty << 5) | tx | (flag << 16);
      }
      if (tid == 0) {  // per-block counts, added to A.stats when the block leaves
        s_stats[4 * lvl + 0] += (unsigned)nw;
        s_stats[4 * lvl + 1] += (unsigned)(nd + nw);
        s_stats[4 * lvl + 2] += (unsigned)nfb;
      }
      if (!direct) __syncthreads();
      if (direct ? valid : (tid < nd + nw)) {
        const int e = direct ? ((ty << 5) | tx | (SCHEME == kWeno ? 1 << 16 : 0)) : s_list[tid];
        const int cx = e & 31, cy = (e >> 5) & 0xff, f = (e >> 16) & 1;
        const int c2 = (cy + 3) * kBW + (cx + 3);
        const int c32 = (cy + 3) * kBW32 + (cx + 3);
        const int gi = i0 + cx, gj = j0 + cy;  // level index
        const long g = (long)(gj + 3) * A.pitch[lvl] + (gi + 3);
        const long fs = A.fstride[lvl];
        // the uniform tile's first cell records the tile's inputs and outputs
        const bool record = uni && cx == 0 && cy == 0;
        if constexpr (kF32S) {
          // single precision throughout: perturbations in, perturbations out
          // u^n and H0 of this cell from the prefetched interior boxes
          const float* unb = reinterpret_cast<const float*>(dst[b] + kTile32Bytes);
          const float* h0b = reinterpret_cast<const float*>(dst[b] + kTile32Bytes + kUnBytes);
          const int ci = cy * kBW32 + cx + 3;
          float* out = static_cast<float*>(A.out[lvl]);
          SAcc32R acc{acc32(tile32, planes, cx, cy)};
          float H[5], K[5], wn[5];
          H[0] = kUnTma ? h0b[ci] : static_cast<const float*>(A.h0[lvl])[g];
          sources_fast(acc, A.F[lvl], H);
          fluxes_fast<ORDER, LLF>(acc, A.F[lvl], gj, f, H, K);
          const float a1 = A.a1f, a2 = A.a2f, bdtf = s_tile.bdtf;
#pragma unroll
          for (int k = 0; k < 5; ++k) {
            const float w = tile32[k * kPlane32 + c32];
            const float u0 = A.un_is_in ? w : (kUnTma ? unb[k * (kTH * kBW32) + ci]
                                                     : static_cast<const float*>(A.un[lvl])[k * fs + g]);
            wn[k] = fmaf(bdtf, K[k], fmaf(a1, u0, a2 * w));
          }
          // update_state in perturbation form (update_state.m4:90-105)
          const FastConst& F = A.F[lvl];
          const float rho = F.rho0 + wn[0];
          float pq, tp;
          eos_pert32(A.E32, wn[0], wn[3], row_height32(F.ylo, F.dy, gj), pq, tp);
          if (s_tile.absorb) {  // perturbations relax towards 0
            const int reach = absorb_reach(A.absorb, lvl, gi, gj, s_tile.box, s_tile.absorb);
#pragma unroll
            for (int sd = 0; sd < 4; ++sd) {
              if (!(reach & (1 << sd))) continue;
              const float t_ = A.absorb.envf[lvl][sd][sd < 2 ? gi : gj];
#pragma unroll
              for (int k = 0; k < 5; ++k) wn[k] *= t_;
              pq *= t_;
              tp *= t_;
            }
          }
#pragma unroll
          for (int k = 0; k < 5; ++k) out[k * fs + g] = wn[k];
          out[5 * fs + g] = pq;
          out[6 * fs + g] = tp;
          if (record) {
            uniform_record<S, kPl>(&s_uc[lvl], reinterpret_cast<const S*>(dst[b]), s_wl[0], A.un_is_in, wn[0], wn[1],
                                   wn[2], wn[3], wn[4], pq, tp, f);
            if (A.rec_out) record_out<S>(static_cast<OutRec<S>*>(A.rec_out) + gti, wn, pq, tp);
            if (A.gcache) publish_uniform<S>(static_cast<GUni<S>*>(A.gcache) + lvl, s_uc[lvl]);
          }
          if (!(rho > 0.f) || !isfinite(wn[0] + wn[1] + wn[2] + wn[3] + wn[4])) raise_health(A.health, ENL_ERR_NONFINITE);
        } else {
          const double* un = static_cast<const double*>(A.un[lvl]);
          double* out = static_cast<double*>(A.out[lvl]);
          double wn[5], pv, tv;
          if constexpr (FAST) {
            SAcc32R acc{acc32(tile32, planes, cx, cy)};
            float H[5], K[5];
            H[0] = (float)static_cast<const double*>(A.h0[lvl])[g];
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
            pv = A.p0 + (double)pp;
            tv = A.T0 + (double)tp;
          } else {
            SAcc64P acc = acc64p(tile, planes64, cx, cy);
            double H[5], K[5];
            H[0] = static_cast<const double*>(A.h0[lvl])[g];
            sources64(acc, A.P[lvl], H);
            fluxes64<ORDER, LLF>(acc, A.P[lvl], gj, f, H, K);
#pragma unroll
            for (int k = 0; k < 5; ++k) {
              double win = tile[k * (kBH * kBW) + c2];
              wn[k] = (A.a1 * un[k * fs + g] + A.a2 * win) + bdt * K[k];
            }
            // update_state (update_state.m4:90-105), as the state upload computes it
            eos_fast64(A.E64, wn[0], wn[3], row_height64(A.ylo, A.dy[lvl], gj), pv, tv);
          }
          if (s_tile.absorb) {  // absolute values relax towards the ambient state
            const int reach = absorb_reach(A.absorb, lvl, gi, gj, s_tile.box, s_tile.absorb);
            const double rT = __dmul_rn(A.T0, A.rho0);
#pragma unroll
            for (int sd = 0; sd < 4; ++sd) {
              if (!(reach & (1 << sd))) continue;
              const double fa = A.absorb.env[lvl][sd][sd < 2 ? gi : gj];
              pv = relax_(pv, A.p0, fa);
              tv = relax_(tv, A.T0, fa);
              wn[0] = relax_(wn[0], A.rho0, fa);
              wn[1] = __dmul_rn(wn[1], fa);
              wn[2] = __dmul_rn(wn[2], fa);
              wn[3] = __dmul_rn(wn[3], fa);
              wn[4] = relax_(wn[4], rT, fa);
            }
          }
          out[5 * fs + g] = pv;
          out[6 * fs + g] = tv;
#pragma unroll
          for (int k = 0; k < 5; ++k) out[k * fs + g] = wn[k];
          if (record) {
            uniform_record<S, kPl>(&s_uc[lvl], reinterpret_cast<const S*>(dst[b]), s_wl[0], A.un_is_in, wn[0], wn[1],
                                   wn[2], wn[3], wn[4], pv, tv, f);
            if (A.rec_out) record_out<S>(static_cast<OutRec<S>*>(A.rec_out) + gti, wn, pv, tv);
            if (A.gcache) publish_uniform<S>(static_cast<GUni<S>*>(A.gcache) + lvl, s_uc[lvl]);
          }
          if (!(wn[0] > 0.0) || !isfinite(wn[0] + wn[1] + wn[2] + wn[3] + wn[4]))
            raise_health(A.health, ENL_ERR_NONFINITE);
        }
      }
    }
    __syncthreads();  // this staging buffer is refilled two tiles later
    t = s_t[b ^ 1];
    b ^= 1;
  }
  if (A.skip_gti) skip_phase<S>(A, s_uc, s_stats, s_t);
  if (tid == 0 && A.stats)
    for (int q = 0; q < 4 * kL; ++q)
      if (s_stats[q]) atomicAdd(&A.stats[q], (unsigned long long)s_stats[q]);
}

// ---------------------------------------------------------------------------
// Uniform-tile skipping, stages 2 and 3: after skip_flags_kernel, the tile
// table is split into the tiles to compute (their descriptors and table
// indices, in table order, so the schedule's tile orders still apply) and the
// tiles to skip; the stage launch computes the first list, publishes its
// first uniform result per level and stores the cached or published result
// into the skipped tiles whose records carry the same key (skip_phase); the
// others go to a second stage launch (usually empty).
// counts: [0] tiles to compute, [1] tiles to skip, [2] passed on.
// Block b (of the flag pass's blocks) writes the entries of its 256 tiles at
// the offsets that the counts of the blocks before it give; block 0 also
// writes the totals.
__global__ void __launch_bounds__(kFlagThreads) skip_lists_kernel(const unsigned char* flag, const int* ntiles,
                                                                  const int2* bcnt, const int4* tiles,
                                                                  int4* full_td, int* full_gti, int* skip_gti,
                                                                  int* counts) {
  __shared__ int s_red[2][kFlagThreads / 32];
  __shared__ int s_wf[kFlagThreads / 32], s_ws[kFlagThreads / 32];
  const int n = *ntiles, nb = (n + kFlagThreads - 1) / kFlagThreads;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if ((int)blockIdx.x >= nb) return;
  // offsets of this block: sums over the blocks before it (block 0 sums all
  // of them for the totals)
  const int upto = blockIdx.x == 0 ? nb : (int)blockIdx.x;
  int of = 0, os = 0;
  for (int q = tid; q < upto; q += kFlagThreads) {
    const int2 c = bcnt[q];
    of += c.x;
    os += c.y;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    of += __shfl_xor_sync(0xffffffffu, of, o);
    os += __shfl_xor_sync(0xffffffffu, os, o);
  }
  if (lane == 0) {
    s_red[0][warp] = of;
    s_red[1][warp] = os;
  }
  // this block's tiles: rank within the block by ballots
  const int t = blockIdx.x * kFlagThreads + tid;
  const bool in = t < n;
  const bool sk = in && flag[t] != 0;
  const unsigned bs = __ballot_sync(0xffffffffu, sk), bf = __ballot_sync(0xffffffffu, in && !sk);
  if (lane == 0) {
    s_wf[warp] = __popc(bf);
    s_ws[warp] = __popc(bs);
  }
  __syncthreads();
  of = 0;
  os = 0;
  int pf = 0, ps = 0;
#pragma unroll
  for (int q = 0; q < kFlagThreads / 32; ++q) {
    of += s_red[0][q];
    os += s_red[1][q];
    if (q < warp) {
      pf += s_wf[q];
      ps += s_ws[q];
    }
  }
  if (blockIdx.x == 0) {
    if (tid == 0) {
      counts[0] = of;
      counts[1] = os;
      counts[2] = 0;
    }
    of = os = 0;  // block 0 starts both lists
  }
  const unsigned lt = (1u << lane) - 1u;
  if (sk) {
    skip_gti[os + ps + __popc(bs & lt)] = t;
  } else if (in) {
    const int p = of + pf + __popc(bf & lt);
    full_td[p] = tiles[t];
    full_gti[p] = t;
  }
}

// ---------------------------------------------------------------------------
// Ghost fill and transfer kernels (canvas form)
// ---------------------------------------------------------------------------
// A level canvas in storage type S: absolute values (double) or
// perturbations about the ambient state (float).
template <typename S>
struct CanvasT {
  S* base;
  long pitch, fstride;
  int nx, ny;
  __device__ S& at(int k, int i, int j) const { return base[k * fstride + (long)(j + 3) * pitch + (i + 3)]; }
};
using CanvasView = CanvasT<double>;

// Physical ghost band of one level (enlightning.C:830-1008 for the patch that
// touches each side): edge ghosts copy the first interior cell of their row or
// column, corners copy the interior corner cell; the normal momentum is
// negated on REFLECT sides (both momenta in a corner of two REFLECT sides).
// sides: bit d set (0..3 = L, R, B, T) fills that side's band; a corner is
// filled when both of its sides are.
template <typename S>
__global__ void physbc_kernel(CanvasT<S> V, int nfields, int bcL, int bcR, int bcB, int bcT, int sides = 15) {
  // 32-bit index arithmetic: a band holds 6 (nx + ny) + 36 cells, far below
  // 2^31 / 7 for any canvas the engine allocates
  const int nx = V.nx, ny = V.ny;
  const int nedge_x = 3 * ny, nedge_y = 3 * nx;
  const int nband = 2 * nedge_x + 2 * nedge_y + 36;
  const int total = nband * nfields;
  // field-major: neighbouring threads fill neighbouring band cells of one field
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int k = t / nband;
    int r = t - k * nband;
    int i, j, si, sj;
    bool negu = false, negv = false;
    if (r < 2 * nedge_x) {
      int side = r >= nedge_x ? 1 : 0;
      int q = r - side * nedge_x;
      j = q / 3;
      int d = q - 3 * j;
      sj = j;
      if (!(sides & (1 << side))) continue;
      if (side == 0) { i = -1 - d; si = 0; negu = bcL == kReflect; }
      else { i = nx + d; si = nx - 1; negu = bcR == kReflect; }
    } else if (r < 2 * nedge_x + 2 * nedge_y) {
      r -= 2 * nedge_x;
      int side = r >= nedge_y ? 1 : 0;
      int q = r - side * nedge_y;
      i = q / 3;
      int d = q - 3 * i;
      si = i;
      if (!(sides & (4 << side))) continue;
      if (side == 0) { j = -1 - d; sj = 0; negv = bcB == kReflect; }
      else { j = ny + d; sj = ny - 1; negv = bcT == kReflect; }
    } else {
      r -= 2 * nedge_x + 2 * nedge_y;
      int corner = r / 9, q = r % 9;
      int dx = q % 3, dy = q / 3;
      int xs = corner & 1, ys = corner >> 1;
      if (!(sides & (1 << xs)) || !(sides & (4 << ys))) continue;
      i = xs ? nx + dx : -1 - dx;
      j = ys ? ny + dy : -1 - dy;
      si = xs ? nx - 1 : 0;
      sj = ys ? ny - 1 : 0;
      negu = (xs ? bcR : bcL) == kReflect;
      negv = (ys ? bcT : bcB) == kReflect;
    }
    S v = V.at(k, si, sj);
    if ((k == 1 && negu) || (k == 2 && negv)) v = -v;
    V.at(k, i, j) = v;
  }
}

// Independent problems: every patch of the table is a domain of its own, and
// its 3-cell band is filled by the single-patch rule of enlightning.C:830-1008
// (edges from the first interior cell, corners from the interior corner, the
// normal momenta negated on REFLECT sides).  blockIdx.y picks the patch, the
// blocks along x share its band (neighbouring threads: neighbouring band
// cells of one field).
constexpr int kBandBlocksPerPatch = 32;
template <typename S>
__global__ void physbc_patches_kernel(CanvasT<S> V, const int4* patches, int off, int cnt, int bcL, int bcR,
                                      int bcB, int bcT) {
  for (int p = blockIdx.y; p < cnt; p += gridDim.y) {
    const int4 b = patches[off + p];
    const int w = b.y - b.x + 1, h = b.w - b.z + 1;
    const int nband = 6 * h + 6 * w + 36;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nband * kNF; t += gridDim.x * blockDim.x) {
      int k = t / nband, r = t - k * nband;
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
      S v = V.at(k, si, sj);
      if ((k == 1 && negu) || (k == 2 && negv)) v = -v;
      V.at(k, i, j) = v;
    }
  }
}

// Coarse-fine ghosts: bilinear interpolation in cell centres from the
// coarser canvas.  One warp per halo row segment (j, i_begin, i_end).
// Weights in the storage type: for a power-of-two ratio every step is exact
// in float as well as in double (I < 2^22).
template <typename S>
__device__ __forceinline__ void refine_weights(int I, int r, int& ic, S& f) {
  // fine cell centre in coarse index coordinates: (I + 0.5)/r - 0.5 (for a
  // power-of-two ratio the product with 1/r is the same number, exactly)
  S xc = ((r & (r - 1)) == 0 ? ((S)I + (S)0.5) * ((S)1 / (S)r) : ((S)I + (S)0.5) / (S)r) - (S)0.5;
  S fl = floor(xc);
  ic = (int)fl;
  f = xc - fl;
}

// One warp per halo chunk (a row run of at most 32 cells of the level's halo,
// the tables split longer runs), one lane per cell: a lane finds its cell
// without a search and has its 4 x nfields loads in flight together.
// Consecutive chunks go to different blocks, so a halo of a few hundred
// chunks still spreads over every SM.  All 4 x 7 coarse loads of a lane are
// issued before its first store (a store could alias a later load, so the
// compiler would not move those loads above it).
template <typename S>
__global__ void interp_kernel(CanvasT<S> F, CanvasT<S> C, int ratio, const int4* segs, const int* meta, int moff,
                              int mcnt) {
  const int off = meta[moff], cnt = meta[mcnt];
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  for (int q = (threadIdx.x >> 5) * gridDim.x + blockIdx.x; q < cnt; q += gridDim.x * wpb) {
    const int4 sg = segs[off + q];
    const int J = sg.x, I = sg.y + lane;
    if (I > sg.z) continue;
    int jc, ic;
    S fy, fx;
    refine_weights(J, ratio, jc, fy);
    refine_weights(I, ratio, ic, fx);
    S c00[kNF], c10[kNF], c01[kNF], c11[kNF];
#pragma unroll
    for (int k = 0; k < kNF; ++k) {
      c00[k] = C.at(k, ic, jc);
      c10[k] = C.at(k, ic + 1, jc);
      c01[k] = C.at(k, ic, jc + 1);
      c11[k] = C.at(k, ic + 1, jc + 1);
    }
#pragma unroll
    for (int k = 0; k < kNF; ++k) {
      S lo_ = ((S)1 - fx) * c00[k] + fx * c10[k];
      S hi_ = ((S)1 - fx) * c01[k] + fx * c11[k];
      F.at(k, I, J) = ((S)1 - fy) * lo_ + fy * hi_;
    }
  }
}

// Generic tile-list kernels: one block of 256 threads per 32x8 tile.
// Coarsening: coarse cell = mean of its ratio x ratio fine cells (7 fields).
// A block takes one field of one tile, so the few tiles a fine level covers
// still spread over every SM; at ratio 2 a thread's four loads are issued
// together (the sum keeps the row-major order of the general loop).
template <typename S>
__global__ void coarsen_kernel(CanvasT<S> C, CanvasT<S> F, int ratio, const int4* tiles, const int* meta, int moff,
                               int mcnt) {
  const int off = meta[moff], cnt = meta[mcnt];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const S inv = (S)1 / (S)(ratio * ratio);
  for (int t = blockIdx.x; t < cnt * kNF; t += gridDim.x) {
    const int tile = t / kNF, k = t - tile * kNF;
    const int4 td = tiles[off + tile];
    const int w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    if (tx >= w || ty >= h) continue;
    const int I = td.x + tx, J = td.y + ty;
    S s = 0;
    if (ratio == 2) {
      const S f00 = F.at(k, 2 * I, 2 * J), f10 = F.at(k, 2 * I + 1, 2 * J);
      const S f01 = F.at(k, 2 * I, 2 * J + 1), f11 = F.at(k, 2 * I + 1, 2 * J + 1);
      s += f00;
      s += f10;
      s += f01;
      s += f11;
    } else {
      for (int b = 0; b < ratio; ++b)
        for (int a = 0; a < ratio; ++a) s += F.at(k, I * ratio + a, J * ratio + b);
    }
    C.at(k, I, J) = s * inv;
  }
}

// Copy patch interiors between two buffers of the same level (7 fields).
template <typename S>
__global__ void copy_tiles_kernel(CanvasT<S> dst, CanvasT<S> src, const int4* tiles, int off, int cnt) {
  for (int t = blockIdx.x; t < cnt; t += gridDim.x) {
    int4 td = tiles[off + t];
    int w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (tx >= w || ty >= h) continue;
    for (int k = 0; k < kNF; ++k) dst.at(k, td.x + tx, td.y + ty) = src.at(k, td.x + tx, td.y + ty);
  }
}

// Bilinear fill of whole boxes (new fine data after a regrid).
template <typename S>
// blockIdx.y picks the box (ilo, ihi, jlo, jhi) of `boxes`; the blocks along
// x share its cells.
__global__ void refine_box_kernel(CanvasT<S> F, CanvasT<S> C, int ratio, const int4* boxes, int nbox) {
  for (int q = blockIdx.y; q < nbox; q += gridDim.y) {
  const int4 bx = boxes[q];
  const int ilo = bx.x, jlo = bx.z, w = bx.y - bx.x + 1, h = bx.w - bx.z + 1;
  long n = (long)w * h;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    int I = ilo + (int)(t % w), J = jlo + (int)(t / w);
    int ic, jc;
    S fx, fy;
    refine_weights(I, ratio, ic, fx);
    refine_weights(J, ratio, jc, fy);
    for (int k = 0; k < kNF; ++k) {
      S lo = ((S)1 - fx) * C.at(k, ic, jc) + fx * C.at(k, ic + 1, jc);
      S hi = ((S)1 - fx) * C.at(k, ic, jc + 1) + fx * C.at(k, ic + 1, jc + 1);
      F.at(k, I, J) = ((S)1 - fy) * lo + fy * hi;
    }
  }
  }
}

// tag_cells.m4:58-108 over the tiles of one level, bit-exact.
// Decided bit for bit as the reference's division would, with the estimate
// of the hybrid switch (sensor_line_fast): two zero differences give the
// ratio ep / ep, 1 or NaN, never below the threshold (most cells of a mostly
// quiet level); otherwise, for a tolerance ep above 2^-1000 (num and den are
// then normal, at least ep), an estimate num * rcp64(den) within 2^-50 of the
// quotient decides unless it lies within 2^-44 of the threshold, and only
// those ratios are divided.
__device__ __forceinline__ bool ratio_below_e(double fm, double f0, double fp, double ep) {
  constexpr double kLo = Lit::c0_9999 * (1.0 - 0x1p-44);
  constexpr double kHi = Lit::c0_9999 * (1.0 + 0x1p-44);
  const double t1 = __dsub_rn(f0, fm);
  const double t2 = __dsub_rn(fp, f0);
  const unsigned long long mag =
      ((unsigned long long)__double_as_longlong(t1) | (unsigned long long)__double_as_longlong(t2)) << 1;
  if (mag == 0ull) return false;
  const double num = __dadd_rn(__dmul_rn(2.0, fabs(__dmul_rn(t1, t2))), ep);
  const double den = __dadd_rn(__dadd_rn(__dmul_rn(t1, t1), __dmul_rn(t2, t2)), ep);
  if (!(ep > 0x1p-1000)) return __ddiv_rn(num, den) < Lit::c0_9999;
  // a positive quotient (or NaN, whose pattern is above kHi): its bit
  // pattern orders as its value
  const unsigned long long qb = (unsigned long long)__double_as_longlong(num * rcp64(den));
  if (qb < (unsigned long long)__double_as_longlong(kLo)) return true;
  return qb <= (unsigned long long)__double_as_longlong(kHi) && __ddiv_rn(num, den) < Lit::c0_9999;
}

// The same test in single precision for FP32 storage (FP64 division is slow
// on this part and the fast engine's tags need no bit-exactness); 0.9999f is
// the reference's REAL*4 literal itself.
__device__ __forceinline__ bool ratio_below_f(float fm, float f0, float fp, float ep) {
  const float t1 = f0 - fm, t2 = fp - f0;
  const float num = fmaf(2.0f, fabsf(t1 * t2), ep);
  const float den = fmaf(t1, t1, fmaf(t2, t2, ep));
  return __fdiv_rn(num, den) < 0.9999f;
}

// The ratio test depends on differences only, so it reads perturbation
// storage as it is.
template <typename S>
// tags (when not null) gets 1 / 0 per patch cell; mask (when not null) gets
// the tagged cells as bits of per-block words (block B x B cells, bit
// r*B + c for cell (c, r) of the block, B <= 8; the words zeroed before).
__global__ void tag_tiles_kernel(int* tags, CanvasT<S> W, CanvasT<S> H, const int4* tiles, int off, int cnt,
                                 double ep0, double ep1, unsigned long long* mask = nullptr, int B = 1,
                                 int nbx = 0) {
  for (int t = blockIdx.x; t < cnt; t += gridDim.x) {
    int4 td = tiles[off + t];
    int w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (tx >= w || ty >= h) continue;
    int i = td.x + tx, j = td.y + ty;
    bool tg;
    if constexpr (std::is_same<S, float>::value) {
      const float e0 = (float)ep0, e1 = (float)ep1;
      tg = ratio_below_f(H.at(0, i - 1, j), H.at(0, i, j), H.at(0, i + 1, j), e0) ||
           ratio_below_f(H.at(0, i, j - 1), H.at(0, i, j), H.at(0, i, j + 1), e0) ||
           ratio_below_f(W.at(0, i - 1, j), W.at(0, i, j), W.at(0, i + 1, j), e1) ||
           ratio_below_f(W.at(0, i, j - 1), W.at(0, i, j), W.at(0, i, j + 1), e1);
    } else {
      tg = ratio_below_e(H.at(0, i - 1, j), H.at(0, i, j), H.at(0, i + 1, j), ep0) ||
           ratio_below_e(H.at(0, i, j - 1), H.at(0, i, j), H.at(0, i, j + 1), ep0) ||
           ratio_below_e(W.at(0, i - 1, j), W.at(0, i, j), W.at(0, i + 1, j), ep1) ||
           ratio_below_e(W.at(0, i, j - 1), W.at(0, i, j), W.at(0, i, j + 1), ep1);
    }
    if (tags) tags[(long)j * W.nx + i] = tg ? 1 : 0;
    if (mask && tg) {
      const int bx = i / B, by = j / B;
      atomicOr(&mask[(long)by * nbx + bx], 1ull << ((j - by * B) * B + (i - bx * B)));
    }
  }
}

// Absorbing envelope of the plain path (enlightning.C:634-786): one thread
// per patch cell of every level, the same per-cell rule and tables as the
// fused stage kernel; amb[] is the ambient state in storage terms.
struct AbsorbTileArgs {
  AbsorbTables T;
  CanvasView lev[kL];
  const int4* tiles;
  const int4* patchtab;
  int ntiles;
  double p0, T0, rho0;
};

__global__ void absorb_tiles_kernel(AbsorbTileArgs A) {
  for (int t = blockIdx.x; t < A.ntiles; t += gridDim.x) {
    const int4 td = A.tiles[t];
    const int lvl = td.z & 0xff, w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (tx >= w || ty >= h) continue;
    const int i = td.x + tx, j = td.y + ty;
    const int reach = absorb_reach(A.T, lvl, i, j, A.patchtab[td.w]);
    const CanvasView& V = A.lev[lvl];
    const double rT = __dmul_rn(A.T0, A.rho0);
#pragma unroll
    for (int sd = 0; sd < 4; ++sd) {
      if (!(reach & (1 << sd))) continue;
      const double fa = A.T.env[lvl][sd][sd < 2 ? i : j];
      V.at(5, i, j) = relax_(V.at(5, i, j), A.p0, fa);
      V.at(6, i, j) = relax_(V.at(6, i, j), A.T0, fa);
      V.at(0, i, j) = relax_(V.at(0, i, j), A.rho0, fa);
      V.at(1, i, j) = __dmul_rn(V.at(1, i, j), fa);
      V.at(2, i, j) = __dmul_rn(V.at(2, i, j), fa);
      V.at(3, i, j) = __dmul_rn(V.at(3, i, j), fa);
      V.at(4, i, j) = relax_(V.at(4, i, j), rT, fa);
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
  // update_state.m4:88 uses the patch's xlo and (j - ifirst1); with the level
  // origin that is the same centre height.
  const double height = __dadd_rn(E.ylo, __dmul_rn(E.dy, (double)j + 0.5));
  const EosConst64 K{E.rho0, E.c, E.c_lr, E.gm1_over_2rho0, E.c_p, E.p0, E.T0, E.c_v, E.R, 1.0 / E.c_p, 1.0 / E.c_v};
  double p, T;
  eos_abs64(K, S.at(0, i, j), S.at(3, i, j), height, p, T);
  S.at(5, i, j) = p;
  S.at(6, i, j) = T;
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

template <typename S>
__global__ void paint_kernel(CanvasT<S> H, const int4* tiles, int off, int cnt, PaintArgs A) {
  for (int t = blockIdx.x; t < cnt; t += gridDim.x) {
    int4 td = tiles[off + t];
    int w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (tx >= w || ty >= h) continue;
    int i = td.x + tx, j = td.y + ty;
    double xc0 = A.xlo0 + A.dx0 * ((double)i + 0.5);
    double xc1 = A.xlo1 + A.dx1 * ((double)j + 0.5);
    double x0 = xc0 - A.pos0, x1 = xc1 - A.pos1;
    S& out = H.at(0, i, j);
    if (A.type == 10) {  // POINT (PULSE) / DRIVEN point
      double v = A.amp * exp(-A.inv_s2ln2 * (x0 * x0 + x1 * x1));
      out = (S)(A.mode == 20 ? v * A.drive : v);
    } else if (A.type == 20) {  // SINE
      double d = x0 - A.sine_amp * sin(A.sine_freq * x1);
      out = (S)(A.amp * exp(-A.inv_s2ln2 * (d * d)));
    } else {  // LIGHTNING
      out = (S)capsule_union((double)out, xc0, xc1, A);
    }
  }
}

// Overpressure dp (read from H0) -> state at s = 0, c_lr = 0, inverting
// update_state.m4:90-94: dp/c^2 = drho + (gamma-1)/(2 rho0) drho^2; T from
// update_state.m4:103-105; rho*T_n = rho*T (nitrogen mode in equilibrium).
template <typename S>
__global__ void overpressure_state_kernel(CanvasT<S> V, CanvasT<S> H, const int4* tiles, int off, int cnt,
                                          double rho0, double c, double gm1_over_2rho0, double p0, double T0,
                                          double R, double c_v, double a0, double a4,
                                          double a5, double a6) {
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
    // a0, a4, a5, a6: ambient parts held out of the storage (0 for absolute)
    V.at(0, i, j) = (S)(rho - a0);
    V.at(1, i, j) = 0;
    V.at(2, i, j) = 0;
    V.at(3, i, j) = 0;
    V.at(4, i, j) = (S)(rho * T - a4);
    V.at(5, i, j) = (S)(((c * c) * (drho + k * (drho * drho)) + p0) - a5);
    V.at(6, i, j) = (S)(T - a6);
    H.at(0, i, j) = 0;
  }
}

// Block map of tags for regridding: map[by][bx] = 1 if any tagged cell lies
// within `buf` cells of the block (tag buffering folded into the reduction).
// Warp-wide bounding box of the blocks with any != 0, merged into bbox by
// lane 0 (all 32 lanes call it).
__device__ __forceinline__ void bbox_merge(int* bbox, unsigned char any, int bx, int by) {
  if (__ballot_sync(0xffffffffu, any)) {
    const int x0 = __reduce_min_sync(0xffffffffu, any ? bx : 0x7fffffff);
    const int x1 = __reduce_max_sync(0xffffffffu, any ? bx : -1);
    const int y0 = __reduce_min_sync(0xffffffffu, any ? by : 0x7fffffff);
    const int y1 = __reduce_max_sync(0xffffffffu, any ? by : -1);
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&bbox[0], x0);
      atomicMax(&bbox[1], x1);
      atomicMin(&bbox[2], y0);
      atomicMax(&bbox[3], y1);
    }
  }
}

// Block map from the per-block tag words (B <= 8; tag_tiles_kernel sets
// them): a block is tagged when its own cells or the cells
// of its 8 neighbours within `buf` (<= B) cells of it hold a tag.  rowm[d] /
// colm[d] select the rows / columns of the neighbour at offset d - 1 that lie
// within the buffer.  Same map as tag_block_kernel.
__global__ void tag_dilate_kernel(const unsigned long long* __restrict__ mask, int nbx, int nby,
                                  unsigned long long rm0, unsigned long long rm2, unsigned long long cm0,
                                  unsigned long long cm2, unsigned char* map, int* bbox) {
  const long n = (long)nbx * nby;
  const long stride = (long)gridDim.x * blockDim.x;
  for (long t0 = blockIdx.x * (long)blockDim.x; t0 < n; t0 += stride) {  // trip count uniform per warp
    const long t = t0 + threadIdx.x;
    unsigned char any = 0;
    int bx = 0, by = 0;
    if (t < n) {
      bx = (int)(t % nbx);
      by = (int)(t / nbx);
      const unsigned long long all = ~0ull;
      const unsigned long long rm[3] = {rm0, all, rm2}, cm[3] = {cm0, all, cm2};
      unsigned long long hit = 0;
#pragma unroll
      for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
          const int x = bx + dx, y = by + dy;
          if (x >= 0 && x < nbx && y >= 0 && y < nby) hit |= mask[(long)y * nbx + x] & rm[dy + 1] & cm[dx + 1];
        }
      any = hit != 0;
      map[t] = any;
    }
    bbox_merge(bbox, any, bx, by);
  }
}

// Block map in one pass, any block size and buffer: each block scans its
// buffered window.  bbox (device, 4 ints: min bx, max bx, min by, max by;
// preset to an empty box) receives the bounding box of the tagged blocks.
__global__ void tag_block_kernel(const int* tags, int nx, int ny, int B, int buf, unsigned char* map, int nbx,
                                 int nby, int* bbox) {
  const long n = (long)nbx * nby;
  const long stride = (long)gridDim.x * blockDim.x;
  for (long t0 = blockIdx.x * (long)blockDim.x; t0 < n; t0 += stride) {  // trip count uniform per warp
    const long t = t0 + threadIdx.x;
    unsigned char any = 0;
    int bx = 0, by = 0;
    if (t < n) {
      bx = (int)(t % nbx);
      by = (int)(t / nbx);
      const int i0 = max(0, bx * B - buf), i1 = min(nx - 1, (bx + 1) * B - 1 + buf);
      const int j0 = max(0, by * B - buf), j1 = min(ny - 1, (by + 1) * B - 1 + buf);
      for (int j = j0; j <= j1 && !any; ++j)
        for (int i = i0; i <= i1; ++i)
          if (tags[(long)j * nx + i]) {
            any = 1;
            break;
          }
      map[t] = any;
    }
    bbox_merge(bbox, any, bx, by);
  }
}

// ---------------------------------------------------------------------------
// Adaptive time step: dt = cfl * dx_min / max over every patch cell of every
// level of max(|u|, |v|) + c (the reference's LLF speed, rhs_hybrid_high_llf
// .m4:270-284, with c_lr = 0).  Block-level max with warp shuffles, one
// 64-bit atomicMax per block (non-negative doubles order like their bits).
// ---------------------------------------------------------------------------
template <typename S>
struct SpeedArgs {
  CanvasT<S> lev[kL];
  const int4* tiles;
  const int* ntiles;
  double c;
  int ec;          // c >= 2^ec (binary exponent of c); -4096 when c is not a positive normal
  double rho_off;  // ambient density held out of the storage (0 for absolute)
  unsigned long long* smax_bits;
};

// max(|rho u|, |rho v|) / |rho| is max(|u|, |v|) bit for bit (a correctly
// rounded division is monotonic), with one division instead of two.  With
// perturbation storage the speed is formed in single precision.  With FP64
// storage the FP64 pipe (1/64 of the FP32 rate on this GPU, compares and
// conversions included) is kept out of the per-cell work: magnitudes are
// compared as integers, a quotient provably below a quarter unit in the last
// place of c (exponents alone show it) contributes c exactly, and the rest
// divide in FP64 only when a single-precision estimate, built from the
// doubles' exponent and leading mantissa bits, says they may hold the block's
// maximum (FP64 division costs about nine fused multiply-adds).  The maximum
// is the same double as dividing every cell.
// Each block takes kSpeedTiles tiles per pass with all their loads in flight
// together (the pass is a chain of dependent loads: descriptor, then fields).
constexpr int kSpeedTiles = 4;

// Single-precision value of a non-negative double whose biased exponent e
// lies in [1023 - 120, 1023 + 120]: exponent rebiased, mantissa truncated to
// 23 bits (relative error below 2^-23, never above the double).
__device__ __forceinline__ float f32_of_bits(unsigned long long u, int e) {
  return __int_as_float(((e - 896) << 23) | (int)((u >> 29) & 0x7fffffu));
}

template <typename S>
__global__ void speed_kernel(SpeedArgs<S> A) {
  __shared__ double s_w[8];
  __shared__ float s_e[8];
  const int n = *A.ntiles;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  double m = 0.0;
  float mf = 0.f;          // FP32 storage: the largest speed
  bool nan_seen = false;   // FP32 storage: a NaN speed (forces a tiny dt)
  bool zero_q = false;     // FP64 storage: a cell whose speed is exactly c
  float m64est = 0.f;      // FP64 storage: the largest quotient estimate of the pass
  const float roff = (float)A.rho_off, cf = (float)A.c;
  float cand_q[kSpeedTiles];
  double av[kSpeedTiles], bv[kSpeedTiles];
#pragma unroll
  for (int u = 0; u < kSpeedTiles; ++u) cand_q[u] = -1.f;
  for (int t0 = blockIdx.x; t0 < n; t0 += kSpeedTiles * gridDim.x) {
    int4 td[kSpeedTiles];
#pragma unroll
    for (int u = 0; u < kSpeedTiles; ++u) {
      const int t = t0 + u * gridDim.x;
      td[u] = t < n ? A.tiles[t] : make_int4(0, 0, 0, 0);  // w = h = 0: no cell
    }
    S r[kSpeedTiles], mu[kSpeedTiles], mv[kSpeedTiles];
    bool ok[kSpeedTiles];
#pragma unroll
    for (int u = 0; u < kSpeedTiles; ++u) {
      const int lvl = td[u].z & 0xff, w = (td[u].z >> 8) & 0xff, h = (td[u].z >> 16) & 0xff;
      ok[u] = tx < w && ty < h;
      if (ok[u]) {
        const CanvasT<S>& V = A.lev[lvl];
        const int i = td[u].x + tx, j = td[u].y + ty;
        r[u] = V.at(0, i, j);
        mu[u] = V.at(1, i, j);
        mv[u] = V.at(2, i, j);
      }
    }
#pragma unroll
    for (int u = 0; u < kSpeedTiles; ++u) {
      if (!ok[u]) continue;
      if constexpr (std::is_same<S, float>::value) {
        const float sf = fmaxf(fabsf(mu[u]), fabsf(mv[u])) / fabsf(roff + r[u]) + cf;
        if (sf == sf) mf = fmaxf(mf, sf);
        else nan_seen = true;
      } else {
        constexpr unsigned long long kAbs = 0x7fffffffffffffffull, kInf = 0x7ff0000000000000ull;
        unsigned long long ua = (unsigned long long)__double_as_longlong(mu[u]) & kAbs;
        unsigned long long uv = (unsigned long long)__double_as_longlong(mv[u]) & kAbs;
        // fmax: a NaN operand yields the other one
        if (ua > kInf) ua = uv;
        else if (uv > kInf) uv = ua;
        const unsigned long long qa = ua > uv ? ua : uv;
        const unsigned long long qb = (unsigned long long)__double_as_longlong(r[u]) & kAbs;
        const int ea = (int)(qa >> 52), eb = (int)(qb >> 52);
        bool odd = true;
        if (qb != 0 && qb <= kInf) {  // |rho| > 0, not NaN
          // a < 2^(ea-1022) and b >= 2^(eb-1023) (b normal): the quotient is
          // below 2^(ec-54), a quarter ulp of c, so q + c rounds to c
          if (qa == 0 || (ea < 2047 && eb >= 1 && eb < 2047 && ea - eb <= A.ec - 55)) {
            zero_q = true;
            odd = false;
          } else if (ea >= 903 && ea <= 1143 && eb >= 903 && eb <= 1143) {
            const float qe = __fdividef(f32_of_bits(qa, ea), f32_of_bits(qb, eb));
            if (qe > 0.f && qe < 1e30f) {
              cand_q[u] = qe;
              m64est = fmaxf(m64est, qe);
              odd = false;
            }
          }
        }
        const double a = __longlong_as_double((long long)qa), b = __longlong_as_double((long long)qb);
        if (odd) {
          // outside the estimate's range: zero or subnormal density, infinite
          // or NaN values, quotients beyond single precision
          double q = a / b;
          if (!(q == q)) q = 1e300;  // NaN state: force a tiny dt, health check reports it
          m = fmax(m, q + A.c);
        }
        av[u] = a;
        bv[u] = b;
      }
    }
    if constexpr (!std::is_same<S, float>::value) {
      // the block's largest estimate; a cell can hold the largest exact
      // quotient only if its estimate is within the estimates' relative error
      // (below 2^-21: two truncations to 23 mantissa bits and the approximate
      // division; taken here as 1e-5) of that maximum: only those divide in
      // FP64, so the maximum is the same double as dividing everywhere
      float bm = m64est;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) bm = fmaxf(bm, __shfl_xor_sync(0xffffffffu, bm, o));
      if ((threadIdx.x & 31) == 0) s_e[threadIdx.x >> 5] = bm;
      __syncthreads();
      bm = s_e[0];
#pragma unroll
      for (int w = 1; w < 8; ++w) bm = fmaxf(bm, s_e[w]);
      __syncthreads();
      const float thr = bm * (1.0f - 1e-5f);
#pragma unroll
      for (int u = 0; u < kSpeedTiles; ++u) {
        if (cand_q[u] >= 0.f && cand_q[u] >= thr) m = fmax(m, av[u] / bv[u] + A.c);
        cand_q[u] = -1.f;
      }
      m64est = 0.f;
    }
  }
  if constexpr (std::is_same<S, float>::value) {
    m = (double)mf;
    if (nan_seen) m = fmax(m, 1e300);
  } else if (zero_q) {
    m = fmax(m, A.c);
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

__global__ void dt_kernel(unsigned long long* smax_bits, double* dt, double* time, float* dt_f, double cfl_dxmin,
                          double dt_max) {
  double smax = __longlong_as_double((long long)*smax_bits);
  double d = smax > 0.0 ? cfl_dxmin / smax : dt_max;
  *dt = fmin(d, dt_max);
  *dt_f = (float)*dt;  // for the FP32 stage epilogue
  *time += *dt;
  *smax_bits = 0ull;
}

// ---------------------------------------------------------------------------
// Virtual microphones, enlightning::recordAudio (enlightning.C:2392-2506):
// after a step, every patch of every level whose physical extent
// [xlo, xhi] x [ylo, yhi] (closed) contains a microphone records the
// pressure at i = int((x - xlo)/dx), j = int((y - ylo)/dy), read as element
// j*nx + i of the patch interior, as the reference indexes it (a microphone
// on a patch's upper edge therefore reads the first cell of the next row;
// past the last row the reference reads outside the array, recorded here as
// NaN).  One thread per (microphone, patch); matches are appended to a
// device buffer with the iteration, level and patch index, so the host can
// restore the reference's file order (level, then patch, per microphone).
// ---------------------------------------------------------------------------
struct MicRecord {
  int iteration, mic, level, patch;
  double p;
};

template <typename S>
struct MicArgs {
  CanvasT<S> lev[kL];
  double dx[kL][2];
  double xlo0, xlo1, p_off;
  const int4* patchtab;
  const int* patch_first;       // device: first patch-table index per level, then the total
  int nmics;
  const double* mics;           // x, y per microphone
  const int* iteration;         // device counter of completed steps
  MicRecord* rec;
  unsigned long long* count;
  long long cap;
};

template <typename S>
__global__ void mic_kernel(MicArgs<S> A) {
  const int it = *A.iteration + 1;  // the step just completed
  const int npatch = A.patch_first[kL];
  const long long n = (long long)A.nmics * npatch;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(t % A.nmics), pi = (int)(t / A.nmics);
    int lvl = 0;
    while (lvl + 1 < kL && pi >= A.patch_first[lvl + 1]) ++lvl;
    const int4 b = A.patchtab[pi];
    const double dx = A.dx[lvl][0], dy = A.dx[lvl][1];
    // patch extent as SAMRAI's CartesianPatchGeometry forms it (no fused multiply-add)
    const double xl = __dadd_rn(A.xlo0, __dmul_rn(dx, (double)b.x));
    const double xh = __dadd_rn(A.xlo0, __dmul_rn(dx, (double)(b.y + 1)));
    const double yl = __dadd_rn(A.xlo1, __dmul_rn(dy, (double)b.z));
    const double yh = __dadd_rn(A.xlo1, __dmul_rn(dy, (double)(b.w + 1)));
    const double mx = A.mics[2 * k], my = A.mics[2 * k + 1];
    if (!(mx >= xl && mx <= xh && my >= yl && my <= yh)) continue;
    const int nx = b.y - b.x + 1, ny = b.w - b.z + 1;
    const int i = (int)__ddiv_rn(__dsub_rn(mx, xl), dx), j = (int)__ddiv_rn(__dsub_rn(my, yl), dy);
    const long long idx = (long long)j * nx + i;
    double p = __longlong_as_double(0x7ff8000000000000LL);  // NaN
    if (idx >= 0 && idx < (long long)nx * ny)
      p = A.p_off + (double)A.lev[lvl].at(5, b.x + (int)(idx % nx), b.z + (int)(idx / nx));
    const unsigned long long slot = atomicAdd(A.count, 1ull);
    if ((long long)slot < A.cap) A.rec[slot] = MicRecord{it, k, lvl, pi, p};
  }
}

// Advances the device iteration counter after mic_kernel has read it (the
// next launch on the stream).
__global__ void mic_advance_kernel(int* iteration) { *iteration += 1; }

// Pack / unpack the patch interiors of every level (7 fields) into a dense
// buffer: field k of the cell (tx, ty) of tile t sits at
// k*total + off[t] + ty*w + tx.  Used to exchange the hierarchy state with
// host memory.
template <typename S>
struct PackArgs {
  CanvasT<S> lev[kL];
  const int4* tiles;
  const long long* off;
  int ntiles;
  long long total;
  S* packed;
  int unpack;
  int nfields;          // 7: every stored field; 5: the conserved state only
  double ylo, dy[kL];   // cell-row heights (update_state after a 5-field unpack)
  EosConst64 E64;
  EosConst32 E32;
};

// One block per 32x8 tile; all NF loads of a cell are issued before its
// stores.
template <typename S, int NF, bool UNPACK>
__global__ void pack_kernel(PackArgs<S> A) {
  for (int t = blockIdx.x; t < A.ntiles; t += gridDim.x) {
    const int4 td = A.tiles[t];
    const int lvl = td.z & 0xff, w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (tx >= w || ty >= h) continue;
    const long long o = A.off[t] + ty * w + tx;
    const CanvasT<S>& V = A.lev[lvl];
    const int i = td.x + tx, j = td.y + ty;
    S v[NF];
    if (UNPACK) {
#pragma unroll
      for (int k = 0; k < NF; ++k) v[k] = A.packed[k * A.total + o];
#pragma unroll
      for (int k = 0; k < NF; ++k) V.at(k, i, j) = v[k];
      if (NF == 5) {  // p and T follow from the state (update_state)
        if constexpr (std::is_same<S, float>::value) {
          float pp, tp;
          eos_pert32(A.E32, v[0], v[3], row_height32((float)A.ylo, (float)A.dy[lvl], j), pp, tp);
          V.at(5, i, j) = pp;
          V.at(6, i, j) = tp;
        } else {
          double pv, tv;
          eos_fast64(A.E64, v[0], v[3], row_height64(A.ylo, A.dy[lvl], j), pv, tv);
          V.at(5, i, j) = pv;
          V.at(6, i, j) = tv;
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < NF; ++k) v[k] = V.at(k, i, j);
#pragma unroll
      for (int k = 0; k < NF; ++k) A.packed[k * A.total + o] = v[k];
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
template <typename S>
struct HarvestArgs {
  CanvasT<S> V;
  CanvasT<S> H;
  double amb_off[kNF];  // ambient parts held out of the storage (0 for absolute)
  RhsConst P;
  float eps, eps_p, inv_sqrt_eps, rho0, p0, T0;
  double rho0_d, p0_d;
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

// Absolute values: the storage plus its held-out ambient part (adding 0.0
// to a double is exact).
template <typename S>
struct CanvasAcc64 {
  const CanvasT<S>* V;
  const double* off;
  int i, j;
  __device__ double w(int k, int di, int dj) const { return off[k] + (double)V->at(k, i + di, j + dj); }
  __device__ double p(int di, int dj) const { return off[5] + (double)V->at(5, i + di, j + dj); }
  __device__ double t(int di, int dj) const { return off[6] + (double)V->at(6, i + di, j + dj); }
};
// Perturbations of rho and p as the stage kernel's FP32 tile holds them;
// d0 = off[0] - rho0 and d5 = off[5] - p0 are exactly 0 for perturbation
// storage and -rho0, -p0 for absolute storage.
template <typename S>
struct CanvasAcc32 {
  const CanvasT<S>* V;
  int i, j;
  double d0, d5;
  __device__ float w(int k, int di, int dj) const {
    return (float)((double)V->at(k, i + di, j + dj) + (k == 0 ? d0 : 0.0));
  }
  __device__ float p(int di, int dj) const { return (float)((double)V->at(5, i + di, j + dj) + d5); }
};

template <typename S>
__global__ void harvest_kernel(HarvestArgs<S> A) {
  for (int t = blockIdx.x; t < A.cnt; t += gridDim.x) {
    int4 td = A.tiles[A.off + t];
    int w = (td.z >> 8) & 0xff, h = (td.z >> 16) & 0xff;
    int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    if (tx >= w || ty >= h) continue;
    int i = td.x + tx, j = td.y + ty;
    CanvasAcc64<S> a64{&A.V, A.amb_off, i, j};
    int flag = rhs_switch<kHybrid, 5, true>(a64, A.P);
    if (!flag) {
      unsigned hsh = (unsigned)i * 73856093u ^ (unsigned)j * 19349663u ^ A.seed * 83492791u;
      hsh ^= hsh >> 13;
      hsh *= 0x5bd1e995u;
      hsh ^= hsh >> 15;
      if (hsh > A.keep0) continue;
    }
    double H[5], Kd[5], Kw[5];
    H[0] = (double)A.H.at(0, i, j);
    rhs_sources(a64, A.P, H);
    double H2[5] = {H[0], H[1], H[2], H[3], H[4]};
    rhs_fluxes<kHybrid, 5, true>(a64, A.P, j, 0, H, Kd);
    rhs_fluxes<kHybrid, 5, true>(a64, A.P, j, 1, H2, Kw);
    double err = 0.0;
#pragma unroll
    for (int k = 0; k < 5; ++k) err = fmax(err, A.dt * fabs(Kd[k] - Kw[k]) * A.inv_scale[k]);
    unsigned long long idx = atomicAdd(A.count, 1ull);
    if ((long)idx >= A.cap) continue;
    CanvasAcc32<S> a32{&A.V, i, j, A.amb_off[0] - A.rho0_d, A.amb_off[5] - A.p0_d};
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
  void* buf[3] = {nullptr, nullptr, nullptr};  // storage type of the engine
  void* h0 = nullptr;
  double* kk = nullptr;                        // plain path (FP64 storage only)
  double dx[2] = {0, 0};
  std::vector<int4> patches;
  CUtensorMap tmap[3];
  CUtensorMap tmap_un, tmap_h0;  // FP32 storage: interior boxes of u^n and H0
  template <typename S>
  CanvasT<S> view(int which) const {
    void* b = which < 3 ? buf[which] : h0;
    return CanvasT<S>{static_cast<S*>(b), pitch, fstride, nx, ny};
  }
  double* buf64(int which) const { return static_cast<double*>(buf[which]); }
};

// meta layout (device ints)
enum {
  M_NTILES = 0,
  M_HALO_OFF = 1,      // +level
  M_HALO_CNT = 1 + kL,
  M_CT_OFF = 1 + 2 * kL,
  M_CT_CNT = 1 + 3 * kL,
  M_PATCH_OFF = 1 + 4 * kL,  // kL + 1 entries: first patch-table index of each level, then the total
  M_HALO_NCELL = 2 + 5 * kL,  // +level: halo cells to interpolate
  M_TILE_OFF = 2 + 6 * kL,    // +level: first stage tile of the level
  M_TILE_CNT = 2 + 7 * kL,    // +level: stage tiles of the level
  M_SIZE = 2 + 8 * kL
};

template <typename T>
struct DevArray {
  T* p = nullptr;
  size_t cap = 0;
  // Room for n elements.  Returns true if the array was reallocated (its old
  // contents are gone).  When the allocation fails, p is null and cap 0:
  // callers check p before any copy or launch.
  bool ensure(size_t n) {
    if (n <= cap) return false;
    if (p) cudaFree(p);
    p = nullptr;
    // headroom, so that regrids rarely outgrow a table (and a captured graph)
    const size_t want = std::max<size_t>(n + n / 2, 2 * cap);
    cap = 0;
    if (cudaMalloc(&p, want * sizeof(T)) != cudaSuccess) {
      p = nullptr;
      cudaGetLastError();  // reported as ENL_ERR_CUDA by the caller
      return true;
    }
    cap = want;
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
  int tables_from = 0;            // first level whose tables are out of date
  bool tables_on_device = false;  // the device tables hold the kept levels
  // the sides (bit d: 0..3 = L, R, B, T) of the level's physical ghost band
  // that a step reads (by its own patches' stencils or by the next level's
  // halo interpolation)
  int bc_read[kL] = {15, 15, 15, 15};
  DevArray<int4> d_tiles, d_halo, d_ctiles, d_patchtab;
  DevArray<int4> d_rboxes;  // boxes of the last refine_init
  void* rbox_host = nullptr;  // their pinned staging
  size_t rbox_cap = 0;
  cudaEvent_t rbox_ev = nullptr;
  int* d_meta = nullptr;
  int* d_counters = nullptr;   // stage counters: 3 for the all-level launches, 3 per level
  unsigned long long* d_counters64 = nullptr;  // the same, packed two-stream claims (tile order 3)
  int* d_health = nullptr;
  unsigned long long* d_stats = nullptr;
  cudaGraphExec_t graph = nullptr;
  bool graph_valid = false;
  int* d_tags[kL] = {nullptr, nullptr, nullptr, nullptr};  // tag scratch per level
  unsigned char* d_bmap = nullptr;
  int* d_bbox = nullptr;  // bounding box of the tagged blocks of the last block map
  size_t bmap_cap = 0;
  unsigned long long* d_bmask = nullptr;  // per-block tag bits (block map first pass)
  size_t bmask_cap = 0;
  double* d_segs = nullptr;
  size_t segs_cap = 0;
  MlpSmem* d_mlp = nullptr;  // learned-sensor network image (BF16 transposed weights)
  float margin = 0.f;
  int adaptive = 0;          // device-computed dt
  double cfl = 0.5;
  double* d_dt = nullptr;    // [0] = dt of the current step, [1] = simulated time
  int profile = 0;            // 1: time each stage-kernel launch with events; 2: also the other kernels
  cudaEvent_t pev[6] = {};
  double prof_ms = 0.0;
  long long prof_launches = 0, prof_cells = 0;
  // per-class timing of the step's other kernels (profile 2): 0 interp,
  // 1 physical band fill, 2 coarsen, 3 CFL maximum (speed + dt), and with
  // uniform-tile skipping 4 the flag pass and lists, 5 the second stage
  // launch
  static constexpr int kKev = 128;
  cudaEvent_t kev[2 * kKev] = {};
  int kev_cls[kKev] = {};
  int kev_n = 0;
  static constexpr int kCls = 6;
  double kev_bytes[kKev] = {};
  double kcls_ms[kCls] = {};
  double kcls_bytes[kCls] = {};
  long long kcls_n[kCls] = {};
  // per level, from the tables: distinct coarse cells the halo interpolation
  // reads, coarse cells the coarsening writes, band cells of the per-patch
  // fill, patch cells
  long long n_halo_coarse[kL] = {}, n_ccells[kL] = {}, n_pband[kL] = {}, n_cells[kL] = {};
  DevArray<long long> d_tileoff;
  std::vector<long long> h_tileoff;
  // host exchange (upload/download): two device staging slots per direction,
  // copies on the engine's own streams, ordered with the library stream by
  // events (see pack_common)
  struct Xfer {
    void* dev[2] = {nullptr, nullptr};
    size_t cap[2] = {0, 0};                 // bytes
    cudaEvent_t copied[2] = {};             // the slot's copy is done
    cudaEvent_t used[2] = {};               // the slot's kernel (pack / unpack) is done
    bool pending[2] = {false, false};       // download: the slot's copy may be in flight
    int slot = 0;
  } xin, xout;
  cudaStream_t s_in = nullptr, s_out = nullptr;
  // downloads whose copy to the host may still run: an upload from an
  // overlapping host range waits for them
  struct HostWrite {
    const void* host;
    size_t bytes;
    cudaEvent_t done;
  };
  std::vector<HostWrite> host_writes;
  std::vector<cudaEvent_t> spare_events;
  unsigned long long* d_smax = nullptr;
  // virtual microphones
  int nmics = 0;
  double* d_mics = nullptr;
  int* d_mic_it = nullptr;
  MicRecord* d_mic_rec = nullptr;
  unsigned long long* d_mic_count = nullptr;
  long long mic_cap = 0;
  int nsm = 148;
  int stage_blocks = 0;
  size_t smem_bytes = 0;
  // stage-kernel schedule (enl_engine_set_schedule / enl_engine_autotune):
  // resident blocks per SM of the persistent grid (the occupancy limit by
  // default) and the length of the tile runs a block claims
  int samrai_order = 0;  // enl_engine_set_level_order
  int max_blocks_per_sm = 1;
  int sched_bps = 0;  // 0: max_blocks_per_sm
  int sched_chunk = 1;
  // uniform-tile skipping in stages 2 and 3 (with reuse): per tile the
  // neighbour stride (tiles per row of its patch, 0 when a neighbour lies
  // outside the patch), this step's records and the skip flags
  int skip = 1;
  DevArray<int> d_nbr;
  std::vector<int> h_nbr;
  DevArray<unsigned char> d_rec_o1, d_rec_o2, d_rec_un, d_skip;
  DevArray<int2> d_bcnt;                       // per flag-pass block: tiles to compute, to skip
  DevArray<int4> d_full_td, d_left_td;         // descriptors of the tiles to compute / passed on
  DevArray<int> d_full_gti, d_skip_gti, d_left_gti;
  int* d_skipcnt = nullptr;                    // [0] to compute, [1] to skip, [2] passed on
  void* d_gcache = nullptr;                    // GUni<S>[kL]: published uniform results
  // storage: FP64 absolute values, or FP32 perturbations about the ambient
  // state (absolute = off[k] + stored)
  bool f32s = false;
  size_t esize = 8;
  double* d_env[kL][4] = {};  // absorbing-envelope tables (null: side not ABSORB)
  int env_act[kL][4] = {};    // AbsorbTables::act
  double regrid_ms[5] = {0, 0, 0, 0, 0};  // host wall time of enl_engine_regrid phases
  void* stage_host = nullptr;  // pinned staging of the tables
  size_t stage_cap = 0;
  cudaEvent_t stage_ev = nullptr;
  float* d_envf[kL][4] = {};
  unsigned char* d_cont[kL][4] = {};
  double off[kNF] = {0, 0, 0, 0, 0, 0, 0};
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

// Halo-box tensor map of one canvas: a (38 or 40) x 14 x 7 box of doubles
// (rows of kBW) or floats (rows of kBW32, so that a row spans 160 bytes).
// Any other box: `fields` planes of the canvas, a box_w x box_h x box_f box.
static int make_tmap(CUtensorMap* m, void* base, long pitch, long fstride, int nyc, bool f32, int fields = kNF,
                     int box_w = 0, int box_h = kBH, int box_f = kNF) {
  auto fn = encode_fn();
  if (!fn) return ENL_ERR_CUDA;
  const cuuint64_t es = f32 ? 4 : 8;
  if (box_w == 0) box_w = f32 ? kBW32 : kBW;
  cuuint64_t dims[3] = {(cuuint64_t)pitch, (cuuint64_t)nyc, (cuuint64_t)fields};
  cuuint64_t strides[2] = {(cuuint64_t)(pitch * es), (cuuint64_t)(fstride * es)};
  cuuint32_t box[3] = {(cuuint32_t)box_w, (cuuint32_t)box_h, (cuuint32_t)box_f};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(m, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, base, dims,
                  strides, box, estr,
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
// inside [0,nx)x[0,ny), not covered by any patch, in row order and, within a
// row, left to right.  Rows where no patch starts or ends (grown or not) have
// the same segments, so they are computed once per band of such rows, from
// the patches whose grown rows hold the band (a sweep over the patches in
// order of their first grown row): O(bands x active patches), not
// O(rows x patches).
static void halo_segments(const std::vector<int4>& P, int nx, int ny, std::vector<int4>& out) {
  if (P.empty()) return;
  std::vector<int> cuts;  // first rows of the bands
  cuts.reserve(4 * P.size());
  for (auto& b : P) {
    cuts.push_back(std::max(0, b.z - 3));
    cuts.push_back(b.z);
    cuts.push_back(b.w + 1);
    cuts.push_back(std::min(ny, b.w + 4));
  }
  std::sort(cuts.begin(), cuts.end());
  cuts.erase(std::unique(cuts.begin(), cuts.end()), cuts.end());
  std::vector<int> order(P.size()), active;
  for (size_t q = 0; q < P.size(); ++q) order[q] = (int)q;
  std::sort(order.begin(), order.end(), [&](int a, int b) { return P[a].z < P[b].z; });
  size_t next = 0;
  std::vector<std::pair<int, int>> g, gm, cv;
  std::vector<int4> seg;  // one row's segments (.x = row, filled per row)
  for (size_t k = 0; k + 1 < cuts.size(); ++k) {
    const int r0 = cuts[k], r1 = std::min(cuts[k + 1], ny);  // rows [r0, r1)
    if (r0 >= r1) continue;
    while (next < order.size() && std::max(0, P[order[next]].z - 3) <= r0) active.push_back(order[next++]);
    active.erase(std::remove_if(active.begin(), active.end(),
                                [&](int q) { return std::min(ny - 1, P[q].w + 3) < r0; }),
                 active.end());
    g.clear();
    cv.clear();
    for (int q : active) {
      const int4& b = P[q];
      g.push_back({std::max(0, b.x - 3), std::min(nx - 1, b.y + 3)});
      if (r0 >= b.z && r0 <= b.w) cv.push_back({b.x, b.y});
    }
    if (g.empty()) continue;
    std::sort(g.begin(), g.end());
    gm.clear();  // merged grown intervals
    for (auto& iv : g) {
      if (!gm.empty() && iv.first <= gm.back().second + 1) gm.back().second = std::max(gm.back().second, iv.second);
      else gm.push_back(iv);
    }
    std::sort(cv.begin(), cv.end());
    seg.clear();
    for (auto& iv : gm) {
      int a = iv.first;
      for (auto& c : cv) {
        if (c.second < a || c.first > iv.second) continue;
        if (c.first > a) seg.push_back(make_int4(0, a, c.first - 1, 0));
        a = std::max(a, c.second + 1);
      }
      if (a <= iv.second) seg.push_back(make_int4(0, a, iv.second, 0));
    }
    for (int j = r0; j < r1; ++j)
      for (const int4& q : seg) out.push_back(make_int4(j, q.y, q.z, 0));
  }
}

// The eight neighbours of every tile of one level (table entries [t0, t1)),
// 8 table indices per tile in the order skip_flags_kernel reads them (above
// left, above, above right, left, right, below left, below, below right; rows
// counted downwards in j), when its halo box lies in their interiors, else
// -1 in the first slot: tiles of the same patch row-major around a tile whose
// neighbours reach at least 3 cells into its box, and, across patches, full
// 32 x 8 tiles on the level's 32 x 8 grid whose eight grid neighbours are
// such tiles too (the base level's patches are aligned to it).
static void level_neighbours(const std::vector<int4>& tiles, const std::vector<int4>& patches, int t0, int t1,
                             std::vector<int>& out) {
  out.resize((size_t)8 * t1, -1);
  for (int t = t0; t < t1; ++t) out[(size_t)8 * t] = -1;
  // within a patch
  int t = t0;
  for (const int4& b : patches) {
    const int W = b.y - b.x + 1, H = b.w - b.z + 1;
    const int nc = (W + kTW - 1) / kTW, nr = (H + kTH - 1) / kTH;
    for (int r = 0; r < nr; ++r)
      for (int c = 0; c < nc; ++c, ++t) {
        const bool inner = c >= 1 && r >= 1 && c + 1 < nc && r + 1 < nr &&
                           std::min(kTW, W - kTW * (c + 1)) >= 3 && std::min(kTH, H - kTH * (r + 1)) >= 3;
        if (!inner) continue;
        const int q[8] = {t - nc - 1, t - nc, t - nc + 1, t - 1, t + 1, t + nc - 1, t + nc, t + nc + 1};
        for (int m = 0; m < 8; ++m) out[(size_t)8 * t + m] = q[m];
      }
  }
  // across patches, on the 32 x 8 grid (over the bounding box of the full,
  // aligned tiles)
  auto full = [&](const int4& td) {
    return (td.x % kTW) == 0 && (td.y % kTH) == 0 && ((td.z >> 8) & 0xff) == kTW && ((td.z >> 16) & 0xff) == kTH;
  };
  int gx0 = INT_MAX, gy0 = INT_MAX, gx1 = INT_MIN, gy1 = INT_MIN;
  for (int u = t0; u < t1; ++u)
    if (full(tiles[u])) {
      gx0 = std::min(gx0, tiles[u].x / kTW);
      gx1 = std::max(gx1, tiles[u].x / kTW);
      gy0 = std::min(gy0, tiles[u].y / kTH);
      gy1 = std::max(gy1, tiles[u].y / kTH);
    }
  if (gx0 > gx1) return;
  const int gw = gx1 - gx0 + 1, gh = gy1 - gy0 + 1;
  std::vector<int> grid((size_t)gw * gh, -1);
  for (int u = t0; u < t1; ++u)
    if (full(tiles[u])) grid[(size_t)(tiles[u].y / kTH - gy0) * gw + (tiles[u].x / kTW - gx0)] = u;
  for (int u = t0; u < t1; ++u) {
    if (!full(tiles[u]) || out[(size_t)8 * u] >= 0) continue;
    const int gx = tiles[u].x / kTW - gx0, gy = tiles[u].y / kTH - gy0;
    if (gx < 1 || gy < 1 || gx + 1 >= gw || gy + 1 >= gh) continue;
    int q[8], m = 0;
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx)
        if (dx || dy) q[m++] = grid[(size_t)(gy + dy) * gw + (gx + dx)];
    bool all = true;
    for (int k = 0; k < 8; ++k) all = all && q[k] >= 0;
    if (all)
      for (int k = 0; k < 8; ++k) out[(size_t)8 * u + k] = q[k];
  }
}

// Coarse index of the lower of the two coarse cells a fine cell
// interpolates from: floor((I + 1/2)/r - 1/2), as refine_weights.
static int coarse_lo(int I, int r) {
  const int n = 2 * I + 1 - r, d = 2 * r;
  return n >= 0 ? n / d : -((-n + d - 1) / d);
}

// Sizes the profile mode's byte counts use, for level l of the tables.
static void level_counts(Engine* E, int l) {
  const int r = E->cfg.ratio;
  long long hc = 0;
  if (l > 0) {
    // distinct coarse cells under the halo's 2 x 2 stencils: row intervals
    // per coarse row, merged
    std::vector<int3> iv;
    const int off = E->h_meta[M_HALO_OFF + l], cnt = E->h_meta[M_HALO_CNT + l];
    iv.reserve(2 * (size_t)cnt);
    for (int q = off; q < off + cnt; ++q) {
      const int4 sg = E->h_halo[q];
      const int jc = coarse_lo(sg.x, r), a = coarse_lo(sg.y, r), b = coarse_lo(sg.z, r) + 1;
      iv.push_back(make_int3(jc, a, b));
      iv.push_back(make_int3(jc + 1, a, b));
    }
    std::sort(iv.begin(), iv.end(), [](const int3& u, const int3& v) { return u.x != v.x ? u.x < v.x : u.y < v.y; });
    for (size_t k = 0; k < iv.size();) {
      int row = iv[k].x, lo = iv[k].y, hi = iv[k].z;
      for (++k; k < iv.size() && iv[k].x == row && iv[k].y <= hi + 1; ++k) hi = std::max(hi, iv[k].z);
      hc += hi - lo + 1;
    }
  }
  E->n_halo_coarse[l] = hc;
  long long cc = 0;
  for (int q = E->h_meta[M_CT_OFF + l]; q < E->h_meta[M_CT_OFF + l] + E->h_meta[M_CT_CNT + l]; ++q)
    cc += (long long)((E->h_ctiles[q].z >> 8) & 0xff) * ((E->h_ctiles[q].z >> 16) & 0xff);
  E->n_ccells[l] = cc;
  long long pb = 0, pc = 0;
  for (const int4& b : E->lev[l].patches) {
    const long long w = b.y - b.x + 1, h = b.w - b.z + 1;
    pb += 6 * (w + h) + 36;
    pc += w * h;
  }
  E->n_pband[l] = pb;
  E->n_cells[l] = pc;
}

// Band cells physbc_kernel fills on a level for a mask of sides.
static long long band_cells(int nx, int ny, int sides) {
  long long n = 0;
  for (int side = 0; side < 4; ++side)
    if (sides & (1 << side)) n += 3LL * (side < 2 ? ny : nx);
  for (int xs = 0; xs < 2; ++xs)
    for (int ys = 0; ys < 2; ++ys)
      if ((sides & (1 << xs)) && (sides & (4 << ys))) n += 9;
  return n;
}

// Host and device patch, tile, halo and coarsen tables.  Levels below
// E->tables_from are unchanged since the last rebuild: their entries (at the
// front of every table) are kept on the host and, unless a device table was
// reallocated, on the device; only the rest is rebuilt and copied.
static int rebuild_tables(Engine* E) {
  const int nl = E->cfg.nlevels;
  const int l0 = std::min(E->tables_from, nl);
  if (l0 == 0) {
    E->tile_off.assign(nl, 0);
    E->tile_cnt.assign(nl, 0);
    E->patch_off.assign(nl, 0);
    E->patch_cnt.assign(nl, 0);
    memset(E->h_meta, 0, sizeof(E->h_meta));
  }
  // truncate every table to the kept levels
  const size_t keep_tiles = l0 < nl ? (size_t)E->tile_off[l0] : E->h_tiles.size();
  const size_t keep_pt = l0 < nl ? (size_t)E->patch_off[l0] : E->h_patchtab.size();
  const size_t keep_halo = l0 < nl ? (size_t)E->h_meta[M_HALO_OFF + l0] : E->h_halo.size();
  const size_t keep_ct = l0 < nl ? (size_t)E->h_meta[M_CT_OFF + l0] : E->h_ctiles.size();
  E->h_tiles.resize(keep_tiles);
  E->h_tileoff.resize(keep_tiles);
  E->h_nbr.resize((size_t)8 * keep_tiles);
  E->h_patchtab.resize(keep_pt);
  E->h_halo.resize(keep_halo);
  E->h_ctiles.resize(keep_ct);
  for (int l = l0; l < nl; ++l) {
    E->tile_off[l] = (int)E->h_tiles.size();
    E->patch_off[l] = (int)E->h_patchtab.size();
    for (auto& b : E->lev[l].patches) {
      // tile .w = index of the patch in the all-level patch table
      tiles_of_box(b, l, (int)E->h_patchtab.size(), E->h_tiles);
      E->h_patchtab.push_back(b);
    }
    level_neighbours(E->h_tiles, E->lev[l].patches, E->tile_off[l], (int)E->h_tiles.size(), E->h_nbr);
    E->tile_cnt[l] = (int)E->h_tiles.size() - E->tile_off[l];
    E->patch_cnt[l] = (int)E->h_patchtab.size() - E->patch_off[l];
    E->h_meta[M_HALO_OFF + l] = (int)E->h_halo.size();
    if (l > 0) {
      // row runs, split into chunks of at most 32 cells (one warp each)
      std::vector<int4> runs;
      halo_segments(E->lev[l].patches, E->lev[l].nx, E->lev[l].ny, runs);
      for (const int4& g : runs)
        for (int a = g.y; a <= g.z; a += 32) E->h_halo.push_back(make_int4(g.x, a, std::min(g.z, a + 31), 0));
    }
    E->h_meta[M_HALO_CNT + l] = (int)E->h_halo.size() - E->h_meta[M_HALO_OFF + l];
    int ncell = 0;  // .w = halo cells of the level before this chunk (for reading the tables)
    for (size_t q = E->h_meta[M_HALO_OFF + l]; q < E->h_halo.size(); ++q) {
      E->h_halo[q].w = ncell;
      ncell += E->h_halo[q].z - E->h_halo[q].y + 1;
    }
    E->h_meta[M_HALO_NCELL + l] = ncell;
    E->h_meta[M_CT_OFF + l] = (int)E->h_ctiles.size();
    if (l > 0) {
      int r = E->cfg.ratio;
      for (auto& b : E->lev[l].patches) {
        int4 cb = make_int4(b.x / r, (b.y + 1) / r - 1, b.z / r, (b.w + 1) / r - 1);
        tiles_of_box(cb, l, 0, E->h_ctiles);
      }
    }
    E->h_meta[M_CT_CNT + l] = (int)E->h_ctiles.size() - E->h_meta[M_CT_OFF + l];
    level_counts(E, l);
  }
  E->h_meta[M_NTILES] = (int)E->h_tiles.size();
  for (int l = 0; l < kL; ++l) {
    E->h_meta[M_TILE_OFF + l] = l < nl ? E->tile_off[l] : (int)E->h_tiles.size();
    E->h_meta[M_TILE_CNT + l] = l < nl ? E->tile_cnt[l] : 0;
  }
  for (int l = 0; l < kL; ++l) E->h_meta[M_PATCH_OFF + l] = l < nl ? E->patch_off[l] : (int)E->h_patchtab.size();
  E->h_meta[M_PATCH_OFF + kL] = (int)E->h_patchtab.size();
  E->h_tileoff.resize(E->h_tiles.size());
  long long acc = 0;
  if (keep_tiles > 0) {
    const int4 td = E->h_tiles[keep_tiles - 1];
    acc = E->h_tileoff[keep_tiles - 1] + (long long)((td.z >> 8) & 0xff) * ((td.z >> 16) & 0xff);
  }
  for (size_t q = keep_tiles; q < E->h_tiles.size(); ++q) {
    E->h_tileoff[q] = acc;
    int4 td = E->h_tiles[q];
    acc += (long long)((td.z >> 8) & 0xff) * ((td.z >> 16) & 0xff);
  }
  E->tables_from = nl;
  // independent problems: the band fill takes the patch counts as launch
  // arguments, so a captured step does not survive new patches
  if (E->cfg.independent) E->graph_valid = false;
  // Which levels' physical ghost bands a step reads: those with a patch
  // within 3 cells (the stencil reach) of a side, and those under a finer
  // level with a patch within 3 + ratio fine cells of a side (its halo cells
  // interpolate from coarse cells one beyond the halo).  The others keep
  // their band fill out of the step.
  {
    auto near = [&](int l, int m) {  // sides within m cells of a patch of level l
      const Level& L = E->lev[l];
      int sides = 0;
      for (const int4& b : L.patches)
        sides |= (b.x < m ? 1 : 0) | (b.y > L.nx - 1 - m ? 2 : 0) | (b.z < m ? 4 : 0) | (b.w > L.ny - 1 - m ? 8 : 0);
      return sides;
    };
    for (int l = 0; l < nl; ++l) {
      const int r = near(l, 3) | (l + 1 < nl ? near(l + 1, 3 + E->cfg.ratio) : 0);
      if (r != E->bc_read[l]) E->graph_valid = false;  // the step's launches change
      E->bc_read[l] = r;
    }
  }
  bool grew = false;
  const bool off_grew = E->d_tileoff.ensure(std::max<size_t>(E->h_tileoff.size(), 1));
  grew |= E->d_tiles.ensure(std::max<size_t>(E->h_tiles.size(), 1));
  grew |= E->d_halo.ensure(std::max<size_t>(E->h_halo.size(), 1));
  grew |= E->d_ctiles.ensure(std::max<size_t>(E->h_ctiles.size(), 1));
  grew |= E->d_patchtab.ensure(std::max<size_t>(E->h_patchtab.size(), 1));
  {
    const size_t nt = std::max<size_t>(E->h_tiles.size(), 1), rb = E->f32s ? 32 : 64;
    grew |= E->d_nbr.ensure(8 * nt);
    grew |= E->d_skip.ensure(nt);
    grew |= E->d_rec_o1.ensure(nt * rb);
    grew |= E->d_rec_o2.ensure(nt * rb);
    grew |= E->d_rec_un.ensure(nt * rb);
    grew |= E->d_full_td.ensure(nt);
    grew |= E->d_left_td.ensure(nt);
    grew |= E->d_full_gti.ensure(nt);
    grew |= E->d_skip_gti.ensure(nt);
    grew |= E->d_left_gti.ensure(nt);
    // one count per flag-pass block over the skip flags' capacity (the
    // passes' grids, fixed while the arrays keep their size)
    grew |= E->d_bcnt.ensure((E->d_skip.cap + kFlagThreads - 1) / kFlagThreads);
  }
  if (grew) E->graph_valid = false;
  if (!E->d_nbr.p || !E->d_skip.p || !E->d_rec_o1.p || !E->d_rec_o2.p || !E->d_rec_un.p || !E->d_full_td.p ||
      !E->d_left_td.p || !E->d_full_gti.p || !E->d_skip_gti.p || !E->d_left_gti.p || !E->d_bcnt.p) {
    E->tables_on_device = false;
    E->graph_valid = false;
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  if (!E->d_tileoff.p || !E->d_tiles.p || !E->d_halo.p || !E->d_ctiles.p || !E->d_patchtab.p) {
    E->tables_on_device = false;
    E->graph_valid = false;
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  // entries kept on the device: none when a table was reallocated (its old
  // contents are gone) or when the tables were never copied
  const bool keep_dev = !grew && !off_grew && E->tables_on_device;
  const size_t k_tiles = keep_dev ? keep_tiles : 0, k_halo = keep_dev ? keep_halo : 0,
               k_ct = keep_dev ? keep_ct : 0, k_pt = keep_dev ? keep_pt : 0;
  // one pinned staging buffer for all tables, copied asynchronously; the
  // previous rebuild's copies must have left it before it is rewritten
  const size_t b_nbr = (E->h_nbr.size() - (size_t)8 * k_tiles) * sizeof(int);
  const size_t b_off = (E->h_tileoff.size() - k_tiles) * sizeof(long long),
               b_tiles = (E->h_tiles.size() - k_tiles) * sizeof(int4),
               b_halo = (E->h_halo.size() - k_halo) * sizeof(int4), b_ct = (E->h_ctiles.size() - k_ct) * sizeof(int4),
               b_pt = (E->h_patchtab.size() - k_pt) * sizeof(int4), b_meta = sizeof(E->h_meta);
  const size_t need = b_nbr + b_off + b_tiles + b_halo + b_ct + b_pt + b_meta;
  if (E->stage_ev) cudaEventSynchronize(E->stage_ev);
  if (need > E->stage_cap) {
    if (E->stage_host) cudaFreeHost(E->stage_host);
    E->stage_cap = need + need / 2;
    if (cudaHostAlloc(&E->stage_host, E->stage_cap, cudaHostAllocDefault) != cudaSuccess) {
      E->stage_host = nullptr;
      E->stage_cap = 0;
      set_error(ENL_ERR_CUDA);
      return ENL_ERR_CUDA;
    }
  }
  if (!E->stage_ev) cudaEventCreateWithFlags(&E->stage_ev, cudaEventDisableTiming);
  cudaStream_t s = stream();
  unsigned char* h = static_cast<unsigned char*>(E->stage_host);
  auto put = [&](void* dst, const void* src, size_t n) {
    if (!n) return;
    memcpy(h, src, n);
    cudaMemcpyAsync(dst, h, n, cudaMemcpyHostToDevice, s);
    h += n;
  };
  put(E->d_tileoff.p + k_tiles, E->h_tileoff.data() + k_tiles, b_off);
  put(E->d_nbr.p + (size_t)8 * k_tiles, E->h_nbr.data() + (size_t)8 * k_tiles, b_nbr);
  put(E->d_tiles.p + k_tiles, E->h_tiles.data() + k_tiles, b_tiles);
  put(E->d_halo.p + k_halo, E->h_halo.data() + k_halo, b_halo);
  put(E->d_ctiles.p + k_ct, E->h_ctiles.data() + k_ct, b_ct);
  put(E->d_patchtab.p + k_pt, E->h_patchtab.data() + k_pt, b_pt);
  put(E->d_meta, E->h_meta, b_meta);
  cudaEventRecord(E->stage_ev, s);
  E->tables_on_device = true;
  return check_launch("engine tables");
}

static bool any_absorb(const Engine* E);
static AbsorbTables absorb_tables(const Engine* E);

static EosConst32 eos_const32(const enl_engine_config& c) {
  EosConst32 e;
  e.rho0 = (float)c.rho0;
  e.c = (float)c.c;
  e.c_lr = (float)c.c_lr;
  e.gm1_over_2rho0 = (float)((c.gamma1 - 1.0) / (2.0 * c.rho0));
  e.inv_c_p = (float)(1.0 / c.c_p);
  e.T0 = (float)c.T0;
  e.inv_c_v = (float)(1.0 / c.c_v);
  e.R = (float)c.R;
  e.inv_rho0 = (float)(1.0 / c.rho0);
  return e;
}

static EosConst64 eos_const64(const enl_engine_config& c) {
  return EosConst64{c.rho0, c.c, c.c_lr, (c.gamma1 - 1.0) / (2.0 * c.rho0), c.c_p, c.p0, c.T0, c.c_v, c.R,
                    1.0 / c.c_p, 1.0 / c.c_v};
}

// level < 0: the launch covers every tile of every level; otherwise the
// tiles of that level only (the per-level stage order)
// Uniform-tile skipping: with uniform-tile reuse (c_lr = 0, not dense) and
// the schedule's skipping on.
static bool skip_on(const Engine* E) {
  return E->skip && !E->cfg.dense && E->cfg.c_lr == 0.0 && !E->samrai_order && E->d_skipcnt && E->d_gcache;
}

static StageArgs stage_args(Engine* E, int stage, double dt, int level = -1) {
  StageArgs A;
  memset(&A, 0, sizeof(A));
  const auto& c = E->cfg;
  int in = stage == 0 ? 0 : stage;          // cur, S0, S1
  int out = stage == 2 ? 0 : stage + 1;     // S0, S1, cur
  for (int l = 0; l < c.nlevels; ++l) {
    Level& L = E->lev[l];
    A.tmap[l] = L.tmap[in];
    A.tmap_un[l] = L.tmap_un;
    A.tmap_h0[l] = L.tmap_h0;
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
    F.rho0T0 = F.rho0 * F.T0;
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
  A.uniform = (!c.dense && c.c_lr == 0.0) ? 1 : 0;
  A.tile_order = c.tile_order;
  A.chunk = std::max(1, E->sched_chunk);
  A.R = c.R;
  A.ylo = c.xlo[1];
  A.un_is_in = in == 0 ? 1 : 0;
  A.a1 = c.rk_alpha1[stage];
  A.a2 = c.rk_alpha2[stage];
  A.bdt = c.rk_beta[stage] * dt;
  A.beta = c.rk_beta[stage];
  A.E32 = eos_const32(c);
  A.E64 = eos_const64(c);
  A.dt_dev = E->adaptive ? E->d_dt : nullptr;
  A.dtf_dev = E->adaptive ? reinterpret_cast<const float*>(E->d_dt + 2) : nullptr;
  A.a1f = (float)A.a1;
  A.a2f = (float)A.a2;
  A.betaf = (float)A.beta;
  A.bdtf = (float)A.bdt;
  A.absorb = absorb_tables(E);
  A.any_absorb = any_absorb(E);
  A.patchtab = E->d_patchtab.p;
  A.tiles = E->d_tiles.p;
  A.ntiles = E->d_meta + (level < 0 ? M_NTILES : M_TILE_CNT + level);
  A.tile_base = level < 0 ? nullptr : E->d_meta + M_TILE_OFF + level;
  A.counter = E->d_counters + (level < 0 ? stage : 3 * (1 + level) + stage);
  A.counter64 = E->d_counters64 + (level < 0 ? stage : 3 * (1 + level) + stage);
  A.nsm = E->nsm;
  A.health = E->d_health;
  A.stats = E->d_stats;
  A.mlp = E->cfg.learned ? E->d_mlp : nullptr;  // null until set_mlp
  A.learned_levels = E->cfg.learned == 2 ? kL : 1;
  A.margin = E->margin;
  A.feat_eps = (float)A.P[0].sensor_eps;
  A.feat_eps_p = (float)(A.P[0].sensor_eps * (c.c * c.c) * (c.c * c.c));
  A.feat_inv_sqrt_eps = (float)(1.0 / sqrt(A.P[0].sensor_eps));
  if (skip_on(E)) {
    // stage 1 records its outputs and u^n / H0, stage 2 its outputs; stages
    // 2 and 3 run over the list of tiles to compute (skip_stage_t) and
    // publish their uniform results for the skipped ones
    if (stage == 0) {
      A.rec_out = E->d_rec_o1.p;
      A.rec_un_out = E->d_rec_un.p;
    } else {
      A.rec_out = stage == 1 ? E->d_rec_o2.p : nullptr;
      A.tiles = E->d_full_td.p;
      A.gti = E->d_full_gti.p;
      A.ntiles = E->d_skipcnt;
      A.gcache = E->d_gcache;
    }
  }
  return A;
}

typedef void (*StageFn)(StageArgs);

template <bool FAST, typename S>
static StageFn pick_stage_t(int variant) {
  switch (variant) {
    case 0: return stage_kernel<kHybrid, 5, true, FAST, S>;
    case 1: return stage_kernel<kHybrid, 5, false, FAST, S>;
    case 2: return stage_kernel<kHybrid, 3, true, FAST, S>;
    case 3: return stage_kernel<kHybrid, 3, false, FAST, S>;
    case 4: return stage_kernel<kWeno, 5, true, FAST, S>;
    case 5: return stage_kernel<kWeno, 5, false, FAST, S>;
    case 6: return stage_kernel<kWeno, 3, true, FAST, S>;
    case 7: return stage_kernel<kWeno, 3, false, FAST, S>;
    default: return stage_kernel<kDrp, 5, false, FAST, S>;
  }
}

static StageFn pick_stage(int precision, int variant) {
  if (precision == ENL_PREC_FP32_STATE) return pick_stage_t<true, float>(variant);
  if (precision == ENL_PREC_FP32) return pick_stage_t<true, double>(variant);
  return pick_stage_t<false, double>(variant);
}

// Events around one launch of a kernel class (profile mode 2, direct steps),
// with the launch's algorithmic bytes (each cell value read or written once).
static int kt_begin(Engine* E, int cls, double bytes) {
  if (E->profile < 2 || E->kev_n >= Engine::kKev) return -1;
  const int q = E->kev_n;
  for (int k = 0; k < 2; ++k)
    if (!E->kev[2 * q + k] && cudaEventCreate(&E->kev[2 * q + k]) != cudaSuccess) {
      E->kev[2 * q + k] = nullptr;
      cudaGetLastError();
      return -1;
    }
  E->kev_n = q + 1;
  E->kev_cls[q] = cls;
  E->kev_bytes[q] = bytes;
  cudaEventRecord(E->kev[2 * q], stream());
  return q;
}
static void kt_end(Engine* E, int q) {
  if (q >= 0) cudaEventRecord(E->kev[2 * q + 1], stream());
}
static void kt_collect(Engine* E) {
  for (int q = 0; q < E->kev_n; ++q) {
    float ms = 0.f;
    cudaEventSynchronize(E->kev[2 * q + 1]);
    cudaEventElapsedTime(&ms, E->kev[2 * q], E->kev[2 * q + 1]);
    E->kcls_ms[E->kev_cls[q]] += ms;
    E->kcls_bytes[E->kev_cls[q]] += E->kev_bytes[q];
    E->kcls_n[E->kev_cls[q]] += 1;
  }
  E->kev_n = 0;
}

template <typename S>
static int fill_level(Engine* E, int l, int which, bool skip_unread, int src_which = -1) {
  cudaStream_t s = stream();
  const auto& c = E->cfg;
  Level& L = E->lev[l];
  if (l > 0) {
    // coarse-fine ghosts from buffer src_which of the coarser level (the
    // same buffer unless given)
    const int src = src_which < 0 ? which : src_which;
    // writes the halo cells, reads the coarse cells under their stencils
    const int q = kt_begin(E, 0, (double)kNF * sizeof(S) * (E->h_meta[M_HALO_NCELL + l] + E->n_halo_coarse[l]));
    interp_kernel<S><<<E->nsm * 4, 256, 0, s>>>(L.view<S>(which), E->lev[l - 1].view<S>(src), c.ratio,
                                                E->d_halo.p, E->d_meta, M_HALO_OFF + l, M_HALO_CNT + l);
    kt_end(E, q);
  }
  if (c.independent) {
    if (E->patch_cnt[l]) {
      // each band cell: one source value read, one ghost written
      const int q = kt_begin(E, 1, 2.0 * kNF * sizeof(S) * E->n_pband[l]);
      physbc_patches_kernel<S><<<dim3(kBandBlocksPerPatch, std::min(E->patch_cnt[l], 65535)), 256, 0, s>>>(
          L.view<S>(which), E->d_patchtab.p, E->patch_off[l], E->patch_cnt[l], c.bc[0], c.bc[1], c.bc[2], c.bc[3]);
      kt_end(E, q);
    }
  } else if (!skip_unread || E->bc_read[l]) {
    const int q = kt_begin(E, 1, 2.0 * kNF * sizeof(S) * band_cells(L.nx, L.ny, skip_unread ? E->bc_read[l] : 15));
    physbc_kernel<S><<<E->nsm * 4, 256, 0, s>>>(L.view<S>(which), kNF, c.bc[0], c.bc[1], c.bc[2], c.bc[3],
                                                skip_unread ? E->bc_read[l] : 15);
    kt_end(E, q);
  }
  return ENL_OK;
}

// Ghosts of levels 0..last (a level's fill reads only the coarser levels).
// skip_unread (the fused step): band fills only of the sides the step reads;
// every other fill (tagging, regrid, the API) fills whole bands.
static int fill_all(Engine* E, int which, int last = kL, bool skip_unread = false) {
  for (int l = 0; l < E->cfg.nlevels && l <= last; ++l) {
    if (E->f32s) fill_level<float>(E, l, which, skip_unread);
    else fill_level<double>(E, l, which, skip_unread);
  }
  return check_launch("fill");
}

static bool any_absorb(const Engine* E) {
  const auto& c = E->cfg;
  return c.bc[0] == kAbsorb || c.bc[1] == kAbsorb || c.bc[2] == kAbsorb || c.bc[3] == kAbsorb;
}

static AbsorbTables absorb_tables(const Engine* E) {
  AbsorbTables T;
  for (int l = 0; l < kL; ++l)
    for (int d = 0; d < 4; ++d) {
      T.env[l][d] = E->d_env[l][d];
      T.envf[l][d] = E->d_envf[l][d];
      T.cont[l][d] = E->d_cont[l][d];
      T.act[l][d] = E->env_act[l][d];
    }
  return T;
}

// Envelope tables of every level, host-computed with the reference's formula
// 1 - exp(-ln2 / w^2 * d^2) and the level's cell centres.
static int build_absorb_tables(Engine* E) {
  const auto& c = E->cfg;
  const double W2 = c.absorb_width * c.absorb_width;
  for (int l = 0; l < c.nlevels; ++l) {
    Level& L = E->lev[l];
    const int n[4] = {L.nx, L.nx, L.ny, L.ny};
    for (int d = 0; d < 4; ++d) {
      if (c.bc[d] != kAbsorb) continue;
      std::vector<double> h(n[d]);
      const int ax = d < 2 ? 0 : 1;
      const double lo = c.xlo[ax], hi = c.xlo[ax] + L.dx[ax] * (ax == 0 ? L.nx : L.ny);
      for (int q = 0; q < n[d]; ++q) {
        const double xc = lo + L.dx[ax] * ((double)q + 0.5);
        const double dist = (d == 0 || d == 2) ? (xc - lo) : (hi - xc);
        h[q] = -std::exp(-std::log(2.0) / W2 * (dist * dist)) + 1.0;
      }
      std::vector<float> hf(n[d]);
      std::vector<unsigned char> hc(n[d]);
      for (int q = 0; q < n[d]; ++q) {
        hf[q] = (float)h[q];
        hc[q] = std::fabs(1.0 - h[q]) > 1.0e-8 ? 1 : 0;  // the reference's loop test
      }
      // cells from the side inwards up to the last factor that is not exactly 1
      int act = (d == 0 || d == 2) ? 0 : n[d];
      for (int q = 0; q < n[d]; ++q)
        if (h[q] != 1.0) {
          if (d == 0 || d == 2) act = std::max(act, q + 1);
          else act = std::min(act, q);
        }
      E->env_act[l][d] = act;
      if (cudaMalloc(&E->d_env[l][d], n[d] * sizeof(double)) != cudaSuccess ||
          cudaMalloc(&E->d_envf[l][d], n[d] * sizeof(float)) != cudaSuccess ||
          cudaMalloc(&E->d_cont[l][d], n[d]) != cudaSuccess)
        return ENL_ERR_CUDA;
      cudaMemcpy(E->d_env[l][d], h.data(), n[d] * sizeof(double), cudaMemcpyHostToDevice);
      cudaMemcpy(E->d_envf[l][d], hf.data(), n[d] * sizeof(float), cudaMemcpyHostToDevice);
      cudaMemcpy(E->d_cont[l][d], hc.data(), n[d], cudaMemcpyHostToDevice);
    }
  }
  return ENL_OK;
}

// Plain path only (FP64 storage); the fused path applies the envelope in the
// stage kernel.
static int absorb_all(Engine* E, int which) {
  if (!any_absorb(E) || E->h_tiles.empty()) return ENL_OK;
  const auto& c = E->cfg;
  AbsorbTileArgs A;
  memset(&A, 0, sizeof(A));
  A.T = absorb_tables(E);
  for (int l = 0; l < c.nlevels; ++l) A.lev[l] = E->lev[l].view<double>(which);
  A.tiles = E->d_tiles.p;
  A.patchtab = E->d_patchtab.p;
  A.ntiles = (int)E->h_tiles.size();
  A.p0 = c.p0;
  A.T0 = c.T0;
  A.rho0 = c.rho0;
  absorb_tiles_kernel<<<std::min(A.ntiles, E->nsm * 16), 256, 0, stream()>>>(A);
  return check_launch("absorb");
}

template <typename S>
static void coarsen_all_t(Engine* E) {
  for (int l = E->cfg.nlevels - 1; l > 0; --l) {
    // reads ratio^2 fine values per coarse value written
    const int q = kt_begin(E, 2, (double)kNF * sizeof(S) * (E->cfg.ratio * E->cfg.ratio + 1) * E->n_ccells[l]);
    coarsen_kernel<S><<<E->nsm * 4, 256, 0, stream()>>>(E->lev[l - 1].view<S>(0), E->lev[l].view<S>(0), E->cfg.ratio,
                                                       E->d_ctiles.p, E->d_meta, M_CT_OFF + l, M_CT_CNT + l);
    kt_end(E, q);
  }
}

static int coarsen_all(Engine* E) {
  if (E->f32s) coarsen_all_t<float>(E);
  else coarsen_all_t<double>(E);
  return check_launch("coarsen");
}

static double finest_dx(Engine* E) {
  const Level& L = E->lev[E->cfg.nlevels - 1];
  return L.dx[0] < L.dx[1] ? L.dx[0] : L.dx[1];
}

template <typename S>
static void speed_t(Engine* E) {
  SpeedArgs<S> A;
  memset(&A, 0, sizeof(A));
  for (int l = 0; l < E->cfg.nlevels; ++l) A.lev[l] = E->lev[l].view<S>(0);
  A.tiles = E->d_tiles.p;
  A.ntiles = E->d_meta + M_NTILES;
  A.c = E->cfg.c;
  int ec = 0;
  A.ec = (std::isnormal(A.c) && A.c > 0.0) ? (std::frexp(A.c, &ec), ec - 1) : -4096;
  A.rho_off = E->off[0];
  A.smax_bits = E->d_smax;
  speed_kernel<S><<<E->nsm * 8, 256, 0, stream()>>>(A);
}

static void adaptive_dt(Engine* E, double dt_max) {
  if (!E->adaptive) return;
  // reads rho, rho u, rho v of every patch cell
  long long cells = 0;
  for (int l = 0; l < E->cfg.nlevels; ++l) cells += E->n_cells[l];
  const int q = kt_begin(E, 3, 3.0 * (E->f32s ? 4 : 8) * cells);
  if (E->f32s) speed_t<float>(E);
  else speed_t<double>(E);
  dt_kernel<<<1, 1, 0, stream()>>>(E->d_smax, E->d_dt, E->d_dt + 1, reinterpret_cast<float*>(E->d_dt + 2), E->cfl * finest_dx(E), dt_max);
  kt_end(E, q);
}

template <typename S>
static void mics_t(Engine* E) {
  MicArgs<S> A;
  memset(&A, 0, sizeof(A));
  for (int l = 0; l < E->cfg.nlevels; ++l) {
    A.lev[l] = E->lev[l].view<S>(0);
    A.dx[l][0] = E->lev[l].dx[0];
    A.dx[l][1] = E->lev[l].dx[1];
  }
  A.xlo0 = E->cfg.xlo[0];
  A.xlo1 = E->cfg.xlo[1];
  A.p_off = E->off[5];
  A.patchtab = E->d_patchtab.p;
  A.patch_first = E->d_meta + M_PATCH_OFF;
  A.nmics = E->nmics;
  A.mics = E->d_mics;
  A.iteration = E->d_mic_it;
  A.rec = E->d_mic_rec;
  A.count = E->d_mic_count;
  A.cap = E->mic_cap;
  mic_kernel<S><<<E->nsm, 256, 0, stream()>>>(A);
  mic_advance_kernel<<<1, 1, 0, stream()>>>(E->d_mic_it);
}

// Microphones sample the state a step leaves (after coarsening), as the
// reference calls recordAudio after advanceHierarchy (main.C:482-486).
static void record_mics(Engine* E) {
  if (E->nmics <= 0) return;
  if (E->f32s) mics_t<float>(E);
  else mics_t<double>(E);
}

// RK stage `stage` (1 or 2) with skipping: flags and lists from the previous
// stage's records, the launch over the tiles to compute (its blocks then
// store the skipped tiles, skip_phase), and a launch over the skipped tiles
// without a cached or published result (usually none).
template <typename S>
static void skip_stage_t(Engine* E, int stage, StageFn fn, const StageArgs& A0) {
  cudaStream_t s = stream();
  const OutRec<S>* rin = reinterpret_cast<const OutRec<S>*>(stage == 1 ? E->d_rec_o1.p : E->d_rec_o2.p);
  const UnRec<S>* run = reinterpret_cast<const UnRec<S>*>(E->d_rec_un.p);
  const int nbk = (int)E->d_bcnt.cap;
  cudaMemsetAsync(E->d_gcache, 0, kL * sizeof(GUni<S>), s);
  int q = kt_begin(E, 4, 0.0);
  skip_flags_kernel<S><<<nbk, kFlagThreads, 0, s>>>(E->d_nbr.p, E->d_meta + M_NTILES, rin, run, E->d_skip.p,
                                                     E->d_bcnt.p);
  skip_lists_kernel<<<nbk, kFlagThreads, 0, s>>>(E->d_skip.p, E->d_meta + M_NTILES, E->d_bcnt.p, E->d_tiles.p,
                                                 E->d_full_td.p, E->d_full_gti.p, E->d_skip_gti.p, E->d_skipcnt);
  kt_end(E, q);
  StageArgs A = A0;
  A.skip_gti = E->d_skip_gti.p;
  A.skip_n = E->d_skipcnt + 1;
  A.skip_counter = E->d_counters + 6 + stage;
  A.tiles_all = E->d_tiles.p;
  A.rec_in = rin;
  A.rec_un_in = run;
  A.left_n = E->d_skipcnt + 2;
  A.left_td = E->d_left_td.p;
  A.left_gti = E->d_left_gti.p;
  void* args[] = {&A};
  cudaLaunchKernel((const void*)fn, dim3(E->stage_blocks), dim3(256), args, E->smem_bytes, s);
  StageArgs B = A0;
  B.tiles = E->d_left_td.p;
  B.gti = E->d_left_gti.p;
  B.ntiles = E->d_skipcnt + 2;
  B.counter = E->d_counters + 3 + stage;
  B.counter64 = E->d_counters64 + 3 + stage;
  B.gcache = nullptr;
  void* bargs[] = {&B};
  q = kt_begin(E, 5, 0.0);
  cudaLaunchKernel((const void*)fn, dim3(E->stage_blocks), dim3(256), bargs, E->smem_bytes, s);
  kt_end(E, q);
}

static int step_fused(Engine* E, double dt) {
  cudaStream_t s = stream();
  cudaMemsetAsync(E->d_counters, 0, 3 * (1 + kL) * sizeof(int), s);
  cudaMemsetAsync(E->d_counters64, 0, 3 * (1 + kL) * sizeof(unsigned long long), s);
  adaptive_dt(E, dt);
  StageFn fn = pick_stage(E->cfg.precision, E->cfg.variant);
  for (int st = 0; st < 3; ++st) {
    int in = st == 0 ? 0 : st;
    int out = st == 2 ? 0 : st + 1;
    if (E->samrai_order) {
      // SAMRAI's MethodOfLinesIntegrator order (main.C:448): per stage the
      // levels coarsest first, each filling its ghosts -- coarse-fine ones
      // from the coarser level already advanced in this stage -- and then
      // advancing; one launch per level
      if (E->profile) cudaEventRecord(E->pev[2 * st], s);
      for (int l = 0; l < E->cfg.nlevels; ++l) {
        if (l > 0) {
          // the coarser level's ghosts in its advanced buffer, as SAMRAI's
          // refine schedule rebuilds them (from the levels below, already
          // advanced, and the physical boundary) before interpolating
          if (E->f32s) fill_level<float>(E, l - 1, out, false);
          else fill_level<double>(E, l - 1, out, false);
        }
        if (E->f32s) fill_level<float>(E, l, in, true, out);
        else fill_level<double>(E, l, in, true, out);
        StageArgs A = stage_args(E, st, dt, l);
        void* args[] = {&A};
        cudaLaunchKernel((const void*)fn, dim3(E->stage_blocks), dim3(256), args, E->smem_bytes, s);
      }
      if (E->profile) cudaEventRecord(E->pev[2 * st + 1], s);
      continue;
    }
    fill_all(E, in, kL, true);
    StageArgs A = stage_args(E, st, dt);
    void* args[] = {&A};
    if (E->profile) cudaEventRecord(E->pev[2 * st], s);
    if (st > 0 && skip_on(E)) {
      if (E->f32s) skip_stage_t<float>(E, st, fn, A);
      else skip_stage_t<double>(E, st, fn, A);
    } else {
      cudaLaunchKernel((const void*)fn, dim3(E->stage_blocks), dim3(256), args, E->smem_bytes, s);
    }
    if (E->profile) cudaEventRecord(E->pev[2 * st + 1], s);
    (void)out;
  }
  coarsen_all(E);
  record_mics(E);
  if (E->profile) {
    kt_collect(E);
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

// Plain path: FP64 storage only (enl_engine_step_plain refuses FP32 storage).
static int step_plain(Engine* E, double dt) {
  cudaStream_t s = stream();
  const auto& c = E->cfg;
  const int nl = c.nlevels;
  adaptive_dt(E, dt);
  // copy current -> scratch (patch interiors)
  for (int l = 0; l < nl; ++l)
    if (E->tile_cnt[l])
      copy_tiles_kernel<double><<<E->tile_cnt[l], 256, 0, s>>>(E->lev[l].view<double>(1), E->lev[l].view<double>(0),
                                                               E->d_tiles.p, E->tile_off[l], E->tile_cnt[l]);
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
        const double* b1 = L.buf64(1);
        launch_rhs_pitched(c.variant, b1 + g0, b1 + 5 * L.fstride + g0, b1 + 6 * L.fstride + g0, L.pitch, L.fstride,
                           static_cast<const double*>(L.h0) + c0, L.kk + c0, L.pitch, L.fstride, nx, ny, Pp);
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
        rk_plain_kernel<<<grd, blk, 0, s>>>(L.view<double>(1), L.view<double>(0), K, b.x, b.z, nx, ny,
                                            c.rk_alpha1[st], c.rk_alpha2[st], c.rk_beta[st] * dt, c.rk_beta[st],
                                            E->adaptive ? E->d_dt : nullptr);
        eos_plain_kernel<<<grd, blk, 0, s>>>(L.view<double>(1), b.x, b.z, nx, ny, Ea);
      }
    }
    absorb_all(E, 1);
  }
  for (int l = 0; l < nl; ++l)
    if (E->tile_cnt[l])
      copy_tiles_kernel<double><<<E->tile_cnt[l], 256, 0, s>>>(E->lev[l].view<double>(0), E->lev[l].view<double>(1),
                                                               E->d_tiles.p, E->tile_off[l], E->tile_cnt[l]);
  coarsen_all(E);
  record_mics(E);
  if (E->profile >= 2) kt_collect(E);  // the other kernels' events of this step
  return check_launch("engine plain step");
}

}  // namespace enl

using namespace enl;

template <typename S>
static int harvest_t(Engine* E, int level, double dt, const double* scale, double keep0, unsigned seed, void* X,
                     float* labels, long capacity, unsigned long long* count_dev) {
  const auto& c = E->cfg;
  Level& L = E->lev[level];
  HarvestArgs<S> A;
  memset(&A, 0, sizeof(A));
  A.V = L.view<S>(0);
  A.H = L.view<S>(3);
  for (int k = 0; k < kNF; ++k) A.amb_off[k] = E->off[k];
  double xlo[2] = {c.xlo[0], c.xlo[1]};
  A.P = make_rhs_const(xlo, L.dx, c.weno_alpha, c.kappa, c.mu, c.muB, c.R, c.T_star_n, c.tau_n, c.tol, 0, c.c,
                       c.c_lr);
  A.eps = (float)A.P.sensor_eps;
  A.eps_p = (float)(A.P.sensor_eps * (c.c * c.c) * (c.c * c.c));
  A.inv_sqrt_eps = (float)(1.0 / sqrt(A.P.sensor_eps));
  A.rho0 = (float)c.rho0;
  A.p0 = (float)c.p0;
  A.rho0_d = c.rho0;
  A.p0_d = c.p0;
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
  if (A.cnt) harvest_kernel<S><<<std::min(A.cnt, E->nsm * 16), 256, 0, stream()>>>(A);
  return check_launch("harvest");
}

extern "C" {

int enl_engine_create(const enl_engine_config* cfg, void** out) {
  if (!cfg || !out || cfg->nlevels < 1 || cfg->nlevels > kL || cfg->ratio < 2 || cfg->nx0 < 8 || cfg->ny0 < 8 ||
      cfg->variant < 0 || cfg->variant > 8 || cfg->precision < ENL_PREC_FP64 || cfg->precision > ENL_PREC_FP32_STATE ||
      cfg->tile_order < 0 || cfg->tile_order > 3 || cfg->learned < 0 || cfg->learned > 2 ||
      (cfg->independent && (cfg->nlevels != 1 || cfg->bc[0] == kAbsorb || cfg->bc[1] == kAbsorb ||
                            cfg->bc[2] == kAbsorb || cfg->bc[3] == kAbsorb))) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  Engine* E = new Engine();
  E->cfg = *cfg;
  E->f32s = cfg->precision == ENL_PREC_FP32_STATE;
  E->esize = E->f32s ? sizeof(float) : sizeof(double);
  if (E->f32s) {
    E->off[0] = cfg->rho0;
    E->off[4] = cfg->rho0 * cfg->T0;
    E->off[5] = cfg->p0;
    E->off[6] = cfg->T0;
  }
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
    size_t bytes = (size_t)L.fstride * kNF * E->esize;
    for (int b = 0; b < 3; ++b) {
      if (cudaMalloc(&L.buf[b], bytes) != cudaSuccess) {
        set_error(ENL_ERR_CUDA);
        enl_engine_destroy(E);
        return ENL_ERR_CUDA;
      }
      cudaMemset(L.buf[b], 0, bytes);
      if (make_tmap(&L.tmap[b], L.buf[b], L.pitch, L.fstride, (int)rows, E->f32s) != ENL_OK) {
        set_error(ENL_ERR_CUDA);
        enl_engine_destroy(E);
        return ENL_ERR_CUDA;
      }
    }
    cudaMalloc(&L.h0, (size_t)L.fstride * E->esize);
    cudaMemset(L.h0, 0, (size_t)L.fstride * E->esize);
    if (E->f32s && (make_tmap(&L.tmap_un, L.buf[0], L.pitch, L.fstride, (int)rows, true, kNF, kBW32, kTH, 5) != ENL_OK ||
                    make_tmap(&L.tmap_h0, L.h0, L.pitch, L.fstride, (int)rows, true, 1, kBW32, kTH, 1) != ENL_OK)) {
      set_error(ENL_ERR_CUDA);
      enl_engine_destroy(E);
      return ENL_ERR_CUDA;
    }
    rr *= cfg->ratio;
  }
  if (any_absorb(E) && build_absorb_tables(E) != ENL_OK) {
    set_error(ENL_ERR_CUDA);
    enl_engine_destroy(E);
    return ENL_ERR_CUDA;
  }
  cudaMalloc(&E->d_meta, sizeof(E->h_meta));
  cudaMemset(E->d_meta, 0, sizeof(E->h_meta));
  cudaMalloc(&E->d_counters, 3 * (1 + kL) * sizeof(int));
  cudaMalloc(&E->d_counters64, 3 * (1 + kL) * sizeof(unsigned long long));
  if (cudaMalloc(&E->d_skipcnt, 4 * sizeof(int)) != cudaSuccess) E->d_skipcnt = nullptr;
  if (cudaMalloc(&E->d_gcache, kL * sizeof(GUni<double>)) != cudaSuccess) E->d_gcache = nullptr;
  cudaGetLastError();  // (skipping stays off without them)
  cudaMalloc(&E->d_health, sizeof(int));
  cudaMemset(E->d_health, 0, sizeof(int));
  cudaMalloc(&E->d_stats, 4 * kL * sizeof(unsigned long long));
  cudaMemset(E->d_stats, 0, 4 * kL * sizeof(unsigned long long));
  cudaMalloc(&E->d_dt, 3 * sizeof(double));  // dt, simulated time, dt as float
  cudaMemset(E->d_dt, 0, 3 * sizeof(double));
  cudaMalloc(&E->d_smax, sizeof(unsigned long long));
  cudaMemset(E->d_smax, 0, sizeof(unsigned long long));
  if (E->f32s) E->smem_bytes = kSmemFast32;
  else E->smem_bytes = cfg->precision == ENL_PREC_FP32 ? kSmemFast64 : kSmem64;
  // (the learned switch keeps its features in the planes' place: no more)
  StageFn fn = pick_stage(cfg->precision, cfg->variant);
  cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)E->smem_bytes);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)fn, 256, E->smem_bytes);
  E->max_blocks_per_sm = std::max(1, per_sm);
  E->stage_blocks = E->nsm * E->max_blocks_per_sm;
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
  for (int l = 0; l < kL; ++l)
    for (int d = 0; d < 4; ++d)
    {
      if (E->d_env[l][d]) cudaFree(E->d_env[l][d]);
      if (E->d_envf[l][d]) cudaFree(E->d_envf[l][d]);
      if (E->d_cont[l][d]) cudaFree(E->d_cont[l][d]);
    }
  if (E->d_meta) cudaFree(E->d_meta);
  if (E->d_counters) cudaFree(E->d_counters);
  if (E->d_counters64) cudaFree(E->d_counters64);
  if (E->d_skipcnt) cudaFree(E->d_skipcnt);
  if (E->d_gcache) cudaFree(E->d_gcache);
  if (E->d_health) cudaFree(E->d_health);
  if (E->d_stats) cudaFree(E->d_stats);
  for (int l = 0; l < kL; ++l)
    if (E->d_tags[l]) cudaFree(E->d_tags[l]);
  if (E->d_bmap) cudaFree(E->d_bmap);
  if (E->d_bbox) cudaFree(E->d_bbox);
  if (E->d_bmask) cudaFree(E->d_bmask);
  if (E->d_dt) cudaFree(E->d_dt);
  if (E->d_mlp) cudaFree(E->d_mlp);
  for (Engine::Xfer* X : {&E->xin, &E->xout})
    for (int q = 0; q < 2; ++q) {
      if (X->copied[q]) {
        cudaEventSynchronize(X->copied[q]);
        cudaEventDestroy(X->copied[q]);
      }
      if (X->used[q]) {
        cudaEventSynchronize(X->used[q]);
        cudaEventDestroy(X->used[q]);
      }
      if (X->dev[q]) cudaFree(X->dev[q]);
    }
  for (auto& w : E->host_writes) {
    cudaEventSynchronize(w.done);
    cudaEventDestroy(w.done);
  }
  for (cudaEvent_t ev : E->spare_events) cudaEventDestroy(ev);
  if (E->s_in) cudaStreamDestroy(E->s_in);
  if (E->s_out) cudaStreamDestroy(E->s_out);
  for (int q = 0; q < 6; ++q)
    if (E->pev[q]) cudaEventDestroy(E->pev[q]);
  for (int q = 0; q < 2 * Engine::kKev; ++q)
    if (E->kev[q]) cudaEventDestroy(E->kev[q]);
  if (E->d_smax) cudaFree(E->d_smax);
  if (E->rbox_ev) {
    cudaEventSynchronize(E->rbox_ev);
    cudaEventDestroy(E->rbox_ev);
  }
  if (E->rbox_host) cudaFreeHost(E->rbox_host);
  if (E->stage_ev) {
    cudaEventSynchronize(E->stage_ev);
    cudaEventDestroy(E->stage_ev);
  }
  if (E->stage_host) cudaFreeHost(E->stage_host);
  if (E->d_mics) cudaFree(E->d_mics);
  if (E->d_mic_it) cudaFree(E->d_mic_it);
  if (E->d_mic_rec) cudaFree(E->d_mic_rec);
  if (E->d_mic_count) cudaFree(E->d_mic_count);
  if (E->d_segs) cudaFree(E->d_segs);
  if (E->graph) cudaGraphExecDestroy(E->graph);
  delete E;
  return ENL_OK;
}

int enl_engine_buffer(void* e, int level, int which, void** base, long* pitch, long* fstride, int* nx, int* ny) {
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
    // tile origins feed TMA x coordinates: 16-byte aligned rows of the box
    const int xmask = E->f32s ? 3 : 1;
    if (b.x < 0 || b.z < 0 || b.y >= L.nx || b.w >= L.ny || b.y < b.x || b.w < b.z || (b.x & xmask)) {
      set_error(ENL_ERR_ARG);
      return ENL_ERR_ARG;
    }
    P.push_back(b);
  }
  L.patches = P;
  E->tables_from = std::min(E->tables_from, level);
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
  long most = 0;
  for (int q = 0; q < nbox; ++q) {
    int ilo = boxes[4 * q], ihi = boxes[4 * q + 1], jlo = boxes[4 * q + 2], jhi = boxes[4 * q + 3];
    if (ilo < 0 || jlo < 0 || ihi >= L.nx || jhi >= L.ny || ihi < ilo || jhi < jlo) {
      set_error(ENL_ERR_ARG);
      return ENL_ERR_ARG;
    }
    most = std::max(most, (long)(ihi - ilo + 1) * (jhi - jlo + 1));
  }
  if (nbox == 0) return ENL_OK;
  // every box in one launch: the boxes go to the device through a pinned
  // staging buffer of their own (its previous copy has left it)
  const size_t bytes = (size_t)nbox * sizeof(int4);
  // the previous refine's kernel has finished with both the device boxes and
  // their staging (rbox_ev follows its launch, on whatever stream it ran)
  if (E->rbox_ev) cudaEventSynchronize(E->rbox_ev);
  E->d_rboxes.ensure(nbox);
  if (!E->d_rboxes.p) {
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  if (bytes > E->rbox_cap) {
    if (E->rbox_host) cudaFreeHost(E->rbox_host);
    E->rbox_cap = bytes + bytes / 2;
    if (cudaHostAlloc(&E->rbox_host, E->rbox_cap, cudaHostAllocDefault) != cudaSuccess) {
      E->rbox_host = nullptr;
      E->rbox_cap = 0;
      set_error(ENL_ERR_CUDA);
      return ENL_ERR_CUDA;
    }
  }
  if (!E->rbox_ev) cudaEventCreateWithFlags(&E->rbox_ev, cudaEventDisableTiming);
  memcpy(E->rbox_host, boxes, bytes);
  cudaMemcpyAsync(E->d_rboxes.p, E->rbox_host, bytes, cudaMemcpyHostToDevice, s);
  const dim3 g((unsigned)std::min<long>((most + 255) / 256, 1024), (unsigned)std::min(nbox, 65535));
  if (E->f32s)
    refine_box_kernel<float><<<g, 256, 0, s>>>(L.view<float>(0), E->lev[level - 1].view<float>(0), E->cfg.ratio,
                                               E->d_rboxes.p, nbox);
  else
    refine_box_kernel<double><<<g, 256, 0, s>>>(L.view<double>(0), E->lev[level - 1].view<double>(0), E->cfg.ratio,
                                                E->d_rboxes.p, nbox);
  cudaEventRecord(E->rbox_ev, s);
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
  if (E->h_tiles.empty() || E->f32s) {
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
  const int profile = E->profile;  // event timing waits on the host: not in a graph
  E->profile = 0;
  step_fused(E, dt);
  E->profile = profile;
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

int enl_engine_graph_valid(void* e) {
  Engine* E = (Engine*)e;
  if (!E) return 0;
  return (E->graph && E->graph_valid) ? 1 : 0;
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

// tag_cells on the patch cells of `level` (ghosts of levels 0..level filled
// first): into the int map tags and/or the block mask (see tag_tiles_kernel).
static int tag_level(Engine* E, int level, int* tags, unsigned long long* mask, int B, int nbx) {
  cudaStream_t s = stream();
  Level& L = E->lev[level];
  fill_all(E, 0, level);
  // source ghosts: the same physical rule on the H0 canvas (one field)
  if (E->f32s)
    physbc_kernel<float><<<E->nsm, 256, 0, s>>>(L.view<float>(3), 1, E->cfg.bc[0], E->cfg.bc[1], E->cfg.bc[2],
                                                E->cfg.bc[3]);
  else
    physbc_kernel<double><<<E->nsm, 256, 0, s>>>(L.view<double>(3), 1, E->cfg.bc[0], E->cfg.bc[1], E->cfg.bc[2],
                                                 E->cfg.bc[3]);
  if (tags) cudaMemsetAsync(tags, 0, (size_t)L.nx * L.ny * sizeof(int), s);
  const double xi = 1.0;
  const double* tol = E->cfg.tol;
  double ep0 = ((Lit::c0_9 * tol[0]) * (xi * xi)) / (1.0 - Lit::c0_9 * (tol[0] * tol[0]));
  double ep1 = ((Lit::c0_9 * tol[1]) * (xi * xi)) / (1.0 - Lit::c0_9 * (tol[1] * tol[1]));
  if (E->tile_cnt[level])
    if (E->f32s)
      tag_tiles_kernel<float><<<E->tile_cnt[level], 256, 0, s>>>(tags, L.view<float>(0), L.view<float>(3),
                                                                 E->d_tiles.p, E->tile_off[level],
                                                                 E->tile_cnt[level], ep0, ep1, mask, B, nbx);
    else
      tag_tiles_kernel<double><<<E->tile_cnt[level], 256, 0, s>>>(tags, L.view<double>(0), L.view<double>(3),
                                                                  E->d_tiles.p, E->tile_off[level],
                                                                  E->tile_cnt[level], ep0, ep1, mask, B, nbx);
  return check_launch("engine tag");
}

int enl_engine_tag(void* e, int level, int* tags) {
  Engine* E = (Engine*)e;
  if (!E || level < 0 || level >= E->cfg.nlevels || !tags) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  return tag_level(E, level, tags, nullptr, 1, 0);
}

int enl_engine_stats(void* e, long long* counts) {
  Engine* E = (Engine*)e;
  if (!E || !counts) return ENL_ERR_ARG;
  unsigned long long h[4 * kL];
  cudaMemcpyAsync(h, E->d_stats, sizeof(h), cudaMemcpyDeviceToHost, stream());
  cudaStreamSynchronize(stream());
  for (int q = 0; q < 4 * kL; ++q) counts[q] = (long long)h[q];
  cudaMemsetAsync(E->d_stats, 0, sizeof(h), stream());
  return check_launch("engine stats");
}

int enl_engine_skipped_tiles(void* e, long long* flagged, long long* written, long long* tiles) {
  Engine* E = (Engine*)e;
  if (!E || !flagged) return ENL_ERR_ARG;
  const size_t n = E->h_tiles.size();
  *flagged = 0;
  if (written) *written = 0;
  if (tiles) *tiles = (long long)n;
  if (!skip_on(E) || n == 0) return ENL_OK;
  int h[3] = {0, 0, 0};
  cudaMemcpyAsync(h, E->d_skipcnt, sizeof(h), cudaMemcpyDeviceToHost, stream());
  cudaStreamSynchronize(stream());
  *flagged = h[1];
  if (written) *written = (long long)h[1] - h[2];
  return check_launch("engine skipped tiles");
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
  const int dt = (E->adaptive ? 2 : 0) + (E->nmics > 0 ? 2 : 0);  // speed + dt update; microphones
  // fused: the stage kernel applies the absorbing envelope itself, and the
  // band fill of a level whose band the step does not read is left out
  if (!plain) {
    int bands = 0;
    for (int l = 0; l < nl; ++l) bands += (c.independent || E->bc_read[l] != 0) ? 1 : 0;
    // SAMRAI order: one stage launch per level, and the coarser level's
    // ghosts rebuilt before each finer level (a band fill, and an
    // interpolation below level 1)
    const int refresh = E->samrai_order ? (nl - 1) + (nl > 2 ? nl - 2 : 0) : 0;
    return 3 * (bands + (nl - 1) + (E->samrai_order ? nl : 1) + refresh) + (nl - 1) + dt +
           (skip_on(E) ? 6 : 0);  // stages 2 and 3: flags, lists, second launch
  }
  const int absorbs = any_absorb(E) ? 1 : 0;
  int npatch = 0, copies = 0;
  for (int l = 0; l < nl; ++l) {
    npatch += (int)E->lev[l].patches.size();
    copies += E->tile_cnt[l] ? 1 : 0;
  }
  return 3 * (fills + 3 * npatch + absorbs) + 2 * copies + (nl - 1) + dt;
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
    if (E->f32s)
      paint_kernel<float><<<E->tile_cnt[level], 256, 0, s>>>(L.view<float>(3), E->d_tiles.p, E->tile_off[level],
                                                             E->tile_cnt[level], A);
    else
      paint_kernel<double><<<E->tile_cnt[level], 256, 0, s>>>(L.view<double>(3), E->d_tiles.p, E->tile_off[level],
                                                              E->tile_cnt[level], A);
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
  if (E->tile_cnt[level]) {
    const unsigned g = (unsigned)E->tile_cnt[level];
    const double k = (c.gamma1 - 1.0) / (2.0 * c.rho0);
    if (E->f32s)
      overpressure_state_kernel<float><<<g, 256, 0, stream()>>>(
          L.view<float>(0), L.view<float>(3), E->d_tiles.p, E->tile_off[level], E->tile_cnt[level], c.rho0, c.c, k,
          c.p0, c.T0, c.R, c.c_v, E->off[0], E->off[4], E->off[5], E->off[6]);
    else
      overpressure_state_kernel<double><<<g, 256, 0, stream()>>>(
          L.view<double>(0), L.view<double>(3), E->d_tiles.p, E->tile_off[level], E->tile_cnt[level], c.rho0, c.c,
          k, c.p0, c.T0, c.R, c.c_v, 0.0, 0.0, 0.0, 0.0);
  }
  return check_launch("state_from_overpressure");
}

// tag_cells on `level` and its block map (tags buffered by `buffer` cells)
// into E->d_bmap, with the tagged blocks' bounding box in E->d_bbox; no copy
// to the host and no synchronisation.
static int tag_blocks_device(Engine* E, int level, int block, int buffer) {
  Level& L = E->lev[level];
  const int nbx = (L.nx + block - 1) / block, nby = (L.ny + block - 1) / block;
  cudaStream_t s = stream();
  const bool two_pass = block <= 8 && buffer <= block;
  if (!two_pass && !E->d_tags[level]) {
    if (cudaMalloc(&E->d_tags[level], (size_t)L.nx * L.ny * sizeof(int)) != cudaSuccess) {
      E->d_tags[level] = nullptr;
      set_error(ENL_ERR_CUDA);
      return ENL_ERR_CUDA;
    }
  }
  const size_t nb = (size_t)nbx * nby;
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
  if (!E->d_bbox && cudaMalloc(&E->d_bbox, 4 * sizeof(int)) != cudaSuccess) {
    E->d_bbox = nullptr;
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  static const int empty[4] = {0x7fffffff, -1, 0x7fffffff, -1};
  cudaMemcpyAsync(E->d_bbox, empty, sizeof(empty), cudaMemcpyHostToDevice, s);
  if (two_pass) {
    // the tag kernel sets the tagged cells' bits in per-block words, then
    // each block takes in the buffer from its 8 neighbours' words
    if (nb > E->bmask_cap) {
      if (E->d_bmask) cudaFree(E->d_bmask);
      if (cudaMalloc(&E->d_bmask, nb * sizeof(unsigned long long)) != cudaSuccess) {
        E->d_bmask = nullptr;
        E->bmask_cap = 0;
        set_error(ENL_ERR_CUDA);
        return ENL_ERR_CUDA;
      }
      E->bmask_cap = nb;
    }
    unsigned long long rows_hi = 0, rows_lo = 0, cols_hi = 0, cols_lo = 0;
    for (int r = 0; r < block; ++r)
      for (int c = 0; c < block; ++c) {
        const unsigned long long bit = 1ull << (r * block + c);
        if (r >= block - buffer) rows_hi |= bit;  // last rows: in the window of the block at j + 1
        if (r < buffer) rows_lo |= bit;           // first rows: in the window of the block at j - 1
        if (c >= block - buffer) cols_hi |= bit;
        if (c < buffer) cols_lo |= bit;
      }
    cudaMemsetAsync(E->d_bmask, 0, nb * sizeof(unsigned long long), s);
    const int st = tag_level(E, level, nullptr, E->d_bmask, block, nbx);
    if (st != ENL_OK) return st;
    const unsigned g = (unsigned)std::min<size_t>((nb + 255) / 256, (size_t)E->nsm * 8);
    tag_dilate_kernel<<<g, 256, 0, s>>>(E->d_bmask, nbx, nby, rows_hi, rows_lo, cols_hi, cols_lo, E->d_bmap, E->d_bbox);
  } else {
    const int st = tag_level(E, level, E->d_tags[level], nullptr, 1, 0);
    if (st != ENL_OK) return st;
    tag_block_kernel<<<E->nsm * 4, 256, 0, s>>>(E->d_tags[level], L.nx, L.ny, block, buffer, E->d_bmap, nbx, nby,
                                                E->d_bbox);
  }
  return check_launch("tag_blocks");
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
  int st = tag_blocks_device(E, level, block, buffer);
  if (st != ENL_OK) return st;
  cudaMemcpyAsync(map_host, E->d_bmap, (size_t)nbx * nby, cudaMemcpyDeviceToHost, stream());
  cudaStreamSynchronize(stream());
  return check_launch("tag_blocks");
}

}  // extern "C"

// The bounded mbarrier wait of the stage kernel on a barrier that completes
// (arrive = 1: one arrival) or that nothing completes (arrive = 0): out gets
// ENL_OK or, after `polls` polls, ENL_ERR_TIMEOUT.  No copy is in flight, so
// giving up leaves nothing behind.
__global__ void bounded_wait_check_kernel(int polls, int arrive, int* out) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (arrive) mbar_arrive(&bar);
    *out = mbar_wait_bounded(&bar, 0u, polls) ? ENL_OK : ENL_ERR_TIMEOUT;
  }
}

// Rectangles covering box a minus box r (inclusive boxes as int4 ilo, ihi,
// jlo, jhi): bottom and top slabs, then the left and right pieces between.
static void box_subtract(const int4& a, const int4& r, std::vector<int4>& out) {
  if (r.y < a.x || r.x > a.y || r.w < a.z || r.z > a.w) {
    out.push_back(a);
    return;
  }
  if (a.z < r.z) out.push_back(make_int4(a.x, a.y, a.z, r.z - 1));
  if (a.w > r.w) out.push_back(make_int4(a.x, a.y, r.w + 1, a.w));
  const int j0 = std::max(a.z, r.z), j1 = std::min(a.w, r.w);
  if (a.x < r.x) out.push_back(make_int4(a.x, r.x - 1, j0, j1));
  if (a.y > r.y) out.push_back(make_int4(r.y + 1, a.y, j0, j1));
}

extern "C" {

int enl_engine_regrid(void* e, int level, int block, int tag_buffer, int nest_blocks, double efficiency,
                      int min_size, int max_size) {
  Engine* E = (Engine*)e;
  if (!E || level < 0 || level + 1 >= E->cfg.nlevels || block < 1 || tag_buffer < 0 || nest_blocks < 0 ||
      min_size < 1 || max_size < 1) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  using clk = std::chrono::steady_clock;
  auto ms = [](clk::time_point a, clk::time_point b) { return std::chrono::duration<double, std::milli>(b - a).count(); };
  const auto t0 = clk::now();
  cudaStreamSynchronize(stream());  // the steps already queued (timed apart from the regrid's own work)
  const auto t1 = clk::now();
  // tags of `level` folded into blocks on the device; only the window of the
  // tagged blocks' bounding box, grown by the nesting erosion, comes back
  const Level& C = E->lev[level];
  const int nbx = (C.nx + block - 1) / block, nby = (C.ny + block - 1) / block;
  int st = tag_blocks_device(E, level, block, tag_buffer);
  if (st != ENL_OK) return st;
  int bb[4];
  cudaMemcpyAsync(bb, E->d_bbox, sizeof(bb), cudaMemcpyDeviceToHost, stream());
  cudaStreamSynchronize(stream());
  const auto t2 = clk::now();
  // The clusterer works inside the bounding box of the tags that survive the
  // nesting mask, and eroding a block reads `passes` blocks around it: a
  // window of the tags' bounding box grown by `passes` (clamped to the map,
  // where the full map has its edge too) gives the boxes of the full map.
  const int passes = level > 0 ? nest_blocks : 0;
  const int cell = block * E->cfg.ratio;  // level+1 cells per block side
  std::vector<int> cb(4 * 1024);
  int nb = 0, wx0 = 0, wy0 = 0;
  if (bb[1] >= bb[0] && bb[3] >= bb[2]) {
    wx0 = std::max(0, bb[0] - passes);
    wy0 = std::max(0, bb[2] - passes);
    const int wx1 = std::min(nbx - 1, bb[1] + passes), wy1 = std::min(nby - 1, bb[3] + passes);
    const int ww = wx1 - wx0 + 1, wh = wy1 - wy0 + 1;
    std::vector<unsigned char> bmap((size_t)ww * wh), allowed((size_t)ww * wh, 0);
    cudaMemcpy2DAsync(bmap.data(), ww, E->d_bmap + (size_t)wy0 * nbx + wx0, nbx, ww, wh, cudaMemcpyDeviceToHost,
                      stream());
    // blocks lying wholly inside a patch of `level`, in window coordinates
    for (const int4& b : C.patches) {
      const int bx0 = std::max((b.x + block - 1) / block, wx0), bx1 = std::min((b.y + 1) / block - 1, wx1);
      const int by0 = std::max((b.z + block - 1) / block, wy0), by1 = std::min((b.w + 1) / block - 1, wy1);
      for (int j = by0; j <= by1; ++j)
        for (int i = bx0; i <= bx1; ++i) allowed[(size_t)(j - wy0) * ww + (i - wx0)] = 1;
    }
    cudaStreamSynchronize(stream());
    st = check_launch("regrid tags");
    if (st != ENL_OK) return st;
    for (;;) {
      st = enl_cluster_tags(bmap.data(), allowed.data(), ww, wh, passes, efficiency, std::max(1, min_size / cell),
                            std::max(1, max_size / cell), cb.data(), (int)(cb.size() / 4), &nb);
      if (st == ENL_OK) break;
      if (nb * 4 <= (int)cb.size()) {
        set_error(st);
        return st;
      }
      cb.resize((size_t)nb * 4);
    }
  }
  const Level& F = E->lev[level + 1];
  const auto t3 = clk::now();
  std::vector<int4> fine;
  for (int q = 0; q < nb; ++q) {
    const int4 fb = make_int4((wx0 + cb[4 * q]) * cell, std::min(F.nx, (wx0 + cb[4 * q + 1] + 1) * cell) - 1,
                              (wy0 + cb[4 * q + 2]) * cell, std::min(F.ny, (wy0 + cb[4 * q + 3] + 1) * cell) - 1);
    if (fb.y >= fb.x && fb.w >= fb.z) fine.push_back(fb);
  }
  // new fine cells (not covered by the old fine patches) are interpolated
  std::vector<int4> fresh;
  for (const int4& b : fine) {
    std::vector<int4> pieces{b}, next;
    for (const int4& r : F.patches) {
      next.clear();
      for (const int4& p : pieces) box_subtract(p, r, next);
      pieces.swap(next);
    }
    fresh.insert(fresh.end(), pieces.begin(), pieces.end());
  }
  std::vector<int> flat(4 * fine.size()), flat2(4 * fresh.size());
  for (size_t q = 0; q < fine.size(); ++q) {
    flat[4 * q] = fine[q].x;
    flat[4 * q + 1] = fine[q].y;
    flat[4 * q + 2] = fine[q].z;
    flat[4 * q + 3] = fine[q].w;
  }
  for (size_t q = 0; q < fresh.size(); ++q) {
    flat2[4 * q] = fresh[q].x;
    flat2[4 * q + 1] = fresh[q].y;
    flat2[4 * q + 2] = fresh[q].z;
    flat2[4 * q + 3] = fresh[q].w;
  }
  st = enl_engine_set_patches(e, level + 1, (int)fine.size(), flat.data());
  if (st != ENL_OK) return st;
  const auto t4 = clk::now();
  st = enl_engine_refine_init(e, level + 1, (int)fresh.size(), flat2.data());
  const auto t5 = clk::now();
  const double ph[5] = {ms(t0, t1), ms(t1, t2), ms(t2, t3), ms(t3, t4), ms(t4, t5)};
  for (int q = 0; q < 5; ++q) E->regrid_ms[q] += ph[q];
  return st;
}

int enl_halo_segments(const int* boxes, int nbox, int nx, int ny, int* segs, int max_segs, int* nseg) {
  if (nbox < 0 || (nbox > 0 && !boxes) || nx < 1 || ny < 1 || max_segs < 0 || (max_segs > 0 && !segs) || !nseg) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  std::vector<int4> P(nbox), out;
  for (int q = 0; q < nbox; ++q) P[q] = make_int4(boxes[4 * q], boxes[4 * q + 1], boxes[4 * q + 2], boxes[4 * q + 3]);
  halo_segments(P, nx, ny, out);
  *nseg = (int)out.size();
  for (int q = 0; q < (int)out.size() && q < max_segs; ++q) {
    segs[3 * q] = out[q].x;
    segs[3 * q + 1] = out[q].y;
    segs[3 * q + 2] = out[q].z;
  }
  if ((int)out.size() > max_segs) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  return ENL_OK;
}

int enl_tile_neighbours(const int* boxes, int nbox, int* tiles, int* nbr, int max_tiles, int* ntiles) {
  if (nbox < 0 || (nbox > 0 && !boxes) || max_tiles < 0 || (max_tiles > 0 && (!tiles || !nbr)) || !ntiles) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  std::vector<int4> P(nbox), T;
  for (int q = 0; q < nbox; ++q) {
    P[q] = make_int4(boxes[4 * q], boxes[4 * q + 1], boxes[4 * q + 2], boxes[4 * q + 3]);
    if (P[q].y < P[q].x || P[q].w < P[q].z) {
      set_error(ENL_ERR_ARG);
      return ENL_ERR_ARG;
    }
    tiles_of_box(P[q], 0, q, T);
  }
  std::vector<int> N;
  level_neighbours(T, P, 0, (int)T.size(), N);
  *ntiles = (int)T.size();
  if ((int)T.size() > max_tiles) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  for (size_t t = 0; t < T.size(); ++t) {
    tiles[4 * t] = T[t].x;
    tiles[4 * t + 1] = T[t].y;
    tiles[4 * t + 2] = (T[t].z >> 8) & 0xff;
    tiles[4 * t + 3] = (T[t].z >> 16) & 0xff;
    for (int m = 0; m < 8; ++m) nbr[8 * t + m] = N[8 * t + m];
  }
  return ENL_OK;
}

int enl_check_bounded_wait(int polls, int arrive) {
  if (polls < 1) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  int* d = nullptr;
  if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) {
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  cudaStream_t s = stream();
  bounded_wait_check_kernel<<<1, 32, 0, s>>>(polls, arrive, d);
  int h = ENL_ERR_CUDA;
  cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  cudaFree(d);
  const int st = check_launch("bounded wait check");
  return st != ENL_OK ? st : h;
}

int enl_engine_regrid_timing(void* e, double* ms5) {
  Engine* E = (Engine*)e;
  if (!E || !ms5) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  for (int q = 0; q < 5; ++q) {
    ms5[q] = E->regrid_ms[q];
    E->regrid_ms[q] = 0.0;
  }
  return ENL_OK;
}

int enl_engine_get_patches(void* e, int level, int* boxes, int max_boxes, int* npatch) {
  Engine* E = (Engine*)e;
  if (!E || level < 0 || level >= E->cfg.nlevels || !npatch || max_boxes < 0 || (max_boxes > 0 && !boxes)) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  const auto& P = E->lev[level].patches;
  *npatch = (int)P.size();
  for (int q = 0; q < (int)P.size() && q < max_boxes; ++q) {
    boxes[4 * q] = P[q].x;
    boxes[4 * q + 1] = P[q].y;
    boxes[4 * q + 2] = P[q].z;
    boxes[4 * q + 3] = P[q].w;
  }
  return (int)P.size() <= max_boxes ? ENL_OK : ENL_ERR_ARG;
}

int enl_engine_set_mics(void* e, int nmics, const double* xy, long long capacity, int iteration) {
  Engine* E = (Engine*)e;
  if (!E || nmics < 0 || (nmics > 0 && (!xy || capacity < 1))) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  if (E->d_mics) cudaFree(E->d_mics);
  if (E->d_mic_rec) cudaFree(E->d_mic_rec);
  E->d_mics = nullptr;
  E->d_mic_rec = nullptr;
  E->nmics = 0;
  E->mic_cap = 0;
  E->graph_valid = false;  // the step gains or loses the sampling launches
  if (nmics == 0) return ENL_OK;
  if (!E->d_mic_it && cudaMalloc(&E->d_mic_it, sizeof(int)) != cudaSuccess) E->d_mic_it = nullptr;
  if (!E->d_mic_count && cudaMalloc(&E->d_mic_count, sizeof(unsigned long long)) != cudaSuccess)
    E->d_mic_count = nullptr;
  if (!E->d_mic_it || !E->d_mic_count || cudaMalloc(&E->d_mics, 2 * nmics * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&E->d_mic_rec, capacity * sizeof(MicRecord)) != cudaSuccess) {
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  cudaStream_t s = stream();
  cudaMemcpyAsync(E->d_mics, xy, 2 * nmics * sizeof(double), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(E->d_mic_it, &iteration, sizeof(int), cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(E->d_mic_count, 0, sizeof(unsigned long long), s);
  cudaStreamSynchronize(s);
  E->nmics = nmics;
  E->mic_cap = capacity;
  return check_launch("set_mics");
}

int enl_engine_mic_records(void* e, void* host, long long max, long long* n, long long* dropped) {
  Engine* E = (Engine*)e;
  if (!E || !n || max < 0 || (max > 0 && !host)) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  *n = 0;
  if (dropped) *dropped = 0;
  if (E->nmics <= 0) return ENL_OK;
  cudaStream_t s = stream();
  unsigned long long cnt = 0;
  cudaMemcpyAsync(&cnt, E->d_mic_count, sizeof(cnt), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  const long long stored = std::min<long long>((long long)cnt, E->mic_cap);
  const long long take = std::min(stored, max);
  if (take > 0) cudaMemcpyAsync(host, E->d_mic_rec, take * sizeof(MicRecord), cudaMemcpyDeviceToHost, s);
  cudaMemsetAsync(E->d_mic_count, 0, sizeof(unsigned long long), s);
  cudaStreamSynchronize(s);
  *n = take;
  if (dropped) *dropped = (long long)cnt - take;
  return check_launch("mic_records");
}

// ---------------------------------------------------------------------------
// Stage-kernel schedule and its autotuner.  The reference balances patches
// over MPI ranks with SAMRAI's load balancer (main.C:268-301); here all
// patches of all levels share one persistent grid, and what decides the
// balance is how the grid's blocks take tiles.  A schedule is
//   [0] resident blocks per SM of the persistent grid (0: occupancy limit),
//   [1] tile order: 0 finest level first, 1 level 0 first, 2 the two ends
//       of the tile table alternately, 3 two streams (each SM's first block
//       from the finest end, its second from level 0),
//   [2] uniform-tile reuse: 2 on, with stages 2 and 3 skipping the halo box
//       of tiles this step's records prove uniform; 1 on, every box loaded
//       and tested; 0 every tile computed cell by cell (results identical
//       in all three),
//   [3] run length: a block claims this many consecutive tiles at a time
//       (1, 2, 4: 32x8, 64x8, 128x8 cells of a patch row per claim).
// ---------------------------------------------------------------------------
static int apply_schedule(Engine* E, const int* v) {
  if (v[0] < 0 || v[0] > E->max_blocks_per_sm || v[1] < 0 || v[1] > 3 || v[2] < 0 || v[2] > 2 || v[3] < 1 ||
      v[3] > 16)
    return ENL_ERR_ARG;
  E->sched_bps = v[0];
  E->cfg.tile_order = v[1];
  E->cfg.dense = v[2] ? 0 : 1;
  E->skip = v[2] == 2 ? 1 : 0;
  E->sched_chunk = v[3];
  E->stage_blocks = E->nsm * (v[0] ? v[0] : E->max_blocks_per_sm);
  E->graph_valid = false;  // grid size and kernel arguments change
  return ENL_OK;
}

static void get_schedule(const Engine* E, int* v) {
  v[0] = E->sched_bps ? E->sched_bps : E->max_blocks_per_sm;
  v[1] = E->cfg.tile_order;
  v[2] = E->cfg.dense ? 0 : (E->skip ? 2 : 1);
  v[3] = E->sched_chunk;
}

int enl_engine_set_schedule(void* e, const int* sched, int n) {
  Engine* E = (Engine*)e;
  if (!E || !sched || n < 4) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  const int r = apply_schedule(E, sched);
  if (r != ENL_OK) set_error(r);
  return r;
}

int enl_engine_get_schedule(void* e, int* sched, int n) {
  Engine* E = (Engine*)e;
  if (!E || !sched || n < 5) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  get_schedule(E, sched);
  sched[4] = E->max_blocks_per_sm;
  return ENL_OK;
}

// Times every candidate schedule on the engine's current hierarchy and
// state: for each, the state is put back to where it was, one step runs
// untimed and `steps` steps are timed with CUDA events on the engine's
// stream; the three fastest and the schedule in force are timed once more
// and the fastest of that second round is applied.  The state (current
// canvases of every level), time step, simulated time, statistics and health
// word are restored afterwards, and microphones record nothing meanwhile, so
// tuning leaves the simulation where it was.  tried (4 ints per candidate)
// and ms (milliseconds per step, the best of the candidate's rounds) receive
// up to `cap` candidates; *ntried their number.  Device memory for one copy
// of the current canvases is allocated for the duration of the call.
int enl_engine_autotune(void* e, double dt, int steps, int cap, int* tried, float* ms, int* ntried) {
  Engine* E = (Engine*)e;
  if (!E || steps < 1 || cap < 0 || (cap > 0 && (!tried || !ms))) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  if (E->h_tiles.empty()) {
    set_error(ENL_ERR_STATE);
    return ENL_ERR_STATE;
  }
  cudaStream_t s = stream();
  const int nl = E->cfg.nlevels;
  // snapshot
  std::vector<void*> snap(nl, nullptr);
  size_t extra = 3 * sizeof(double) + 4 * kL * sizeof(unsigned long long) + sizeof(int);
  void* snap_misc = nullptr;
  bool ok = cudaMalloc(&snap_misc, extra) == cudaSuccess;
  for (int l = 0; ok && l < nl; ++l)
    ok = cudaMalloc(&snap[l], (size_t)kNF * E->lev[l].fstride * E->esize) == cudaSuccess;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  ok = ok && cudaEventCreate(&ev[0]) == cudaSuccess && cudaEventCreate(&ev[1]) == cudaSuccess;
  auto release = [&]() {
    for (void* p : snap)
      if (p) cudaFree(p);
    if (snap_misc) cudaFree(snap_misc);
    for (auto& x : ev)
      if (x) cudaEventDestroy(x);
  };
  if (!ok) {
    cudaGetLastError();
    release();
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  unsigned char* misc = static_cast<unsigned char*>(snap_misc);
  const size_t o_stats = 3 * sizeof(double), o_health = o_stats + 4 * kL * sizeof(unsigned long long);
  auto save_restore = [&](bool save) {
    for (int l = 0; l < nl; ++l) {
      const size_t bytes = (size_t)kNF * E->lev[l].fstride * E->esize;
      if (save) cudaMemcpyAsync(snap[l], E->lev[l].buf[0], bytes, cudaMemcpyDeviceToDevice, s);
      else cudaMemcpyAsync(E->lev[l].buf[0], snap[l], bytes, cudaMemcpyDeviceToDevice, s);
    }
    struct {
      void* dev;
      size_t off, bytes;
    } m[3] = {{E->d_dt, 0, 3 * sizeof(double)},
              {E->d_stats, o_stats, 4 * kL * sizeof(unsigned long long)},
              {E->d_health, o_health, sizeof(int)}};
    for (auto& x : m) {
      if (save) cudaMemcpyAsync(misc + x.off, x.dev, x.bytes, cudaMemcpyDeviceToDevice, s);
      else cudaMemcpyAsync(x.dev, misc + x.off, x.bytes, cudaMemcpyDeviceToDevice, s);
    }
  };
  const int nmics = E->nmics;
  const int profile = E->profile;
  E->nmics = 0;
  E->profile = 0;
  int current[4];
  get_schedule(E, current);
  save_restore(true);
  // candidates: the upper half of the occupancy range, the four orders, reuse
  // with skipping and off (and reuse without skipping on single-tile runs)
  // when the configuration allows reuse, runs of 1, 2, 4 tiles
  std::vector<std::array<int, 4>> cand;
  const bool reuse_ok = E->cfg.c_lr == 0.0;
  for (int bps = (E->max_blocks_per_sm + 1) / 2; bps <= E->max_blocks_per_sm; ++bps)
    for (int order = 0; order <= 3; ++order)
      for (int reuse = reuse_ok ? 2 : 0; reuse >= 0; --reuse)
        for (int chunk : {1, 2, 4})
          if ((order != 3 || chunk == 1) && (reuse != 1 || chunk == 1))  // the two-stream order claims single tiles
            cand.push_back({bps, order, reuse, chunk});
  std::vector<float> best(cand.size(), 1e30f);
  int rc = ENL_OK;
  auto time_one = [&](size_t k) -> float {
    apply_schedule(E, cand[k].data());
    save_restore(false);
    rc = step_fused(E, dt);
    cudaEventRecord(ev[0], s);
    for (int q = 0; q < steps && rc == ENL_OK; ++q) rc = step_fused(E, dt);
    cudaEventRecord(ev[1], s);
    cudaEventSynchronize(ev[1]);
    float t = 0.f;
    cudaEventElapsedTime(&t, ev[0], ev[1]);
    return t / steps;
  };
  for (size_t k = 0; k < cand.size() && rc == ENL_OK; ++k) best[k] = time_one(k);
  if (rc == ENL_OK) {
    // second round: the three fastest and the schedule in force
    std::vector<size_t> idx(cand.size());
    for (size_t k = 0; k < idx.size(); ++k) idx[k] = k;
    std::sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return best[a] < best[b]; });
    std::vector<size_t> again(idx.begin(), idx.begin() + std::min<size_t>(3, idx.size()));
    for (size_t k = 0; k < cand.size(); ++k)
      if (cand[k][0] == current[0] && cand[k][1] == current[1] && cand[k][2] == current[2] &&
          cand[k][3] == current[3] && std::find(again.begin(), again.end(), k) == again.end())
        again.push_back(k);
    for (size_t k : again) {
      if (rc != ENL_OK) break;
      best[k] = std::min(best[k], time_one(k));
    }
  }
  size_t win = 0;
  for (size_t k = 1; k < cand.size(); ++k)
    if (best[k] < best[win]) win = k;
  save_restore(false);
  cudaStreamSynchronize(s);
  E->nmics = nmics;
  E->profile = profile;
  if (rc == ENL_OK) apply_schedule(E, cand[win].data());
  else apply_schedule(E, current);
  const int n = (int)std::min<size_t>(cand.size(), (size_t)cap);
  for (int k = 0; k < n; ++k) {
    for (int q = 0; q < 4; ++q) tried[4 * k + q] = cand[k][q];
    ms[k] = best[k];
  }
  if (ntried) *ntried = (int)cand.size();
  release();
  if (rc != ENL_OK) return rc;
  return check_launch("engine autotune");
}

int enl_engine_set_level_order(void* e, int samrai) {
  Engine* E = (Engine*)e;
  if (!E || samrai < 0 || samrai > 1) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  E->samrai_order = samrai;
  E->graph_valid = false;  // the step's launches change
  return ENL_OK;
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

int enl_engine_set_time(void* e, double dt_last, double sim_time) {
  Engine* E = (Engine*)e;
  if (!E) return ENL_ERR_ARG;
  const double h[2] = {dt_last, sim_time};
  const float hf = (float)dt_last;
  cudaMemcpyAsync(E->d_dt, h, sizeof(h), cudaMemcpyHostToDevice, stream());
  cudaMemcpyAsync(E->d_dt + 2, &hf, sizeof(float), cudaMemcpyHostToDevice, stream());
  cudaStreamSynchronize(stream());
  return check_launch("engine set_time");
}

static long long packed_cells(Engine* E) {
  if (E->h_tiles.empty()) return 0;
  int4 td = E->h_tiles.back();
  return E->h_tileoff.back() + (long long)((td.z >> 8) & 0xff) * ((td.z >> 16) & 0xff);
}

int enl_engine_packed_size(void* e, long long* nelems) {
  Engine* E = (Engine*)e;
  if (!E || !nelems) return ENL_ERR_ARG;
  *nelems = packed_cells(E) * kNF;
  return ENL_OK;
}

int enl_engine_storage(void* e, int* elem_bytes, double* offsets) {
  Engine* E = (Engine*)e;
  if (!E) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  if (elem_bytes) *elem_bytes = (int)E->esize;
  if (offsets)
    for (int k = 0; k < kNF; ++k) offsets[k] = E->off[k];
  return ENL_OK;
}

}  // extern "C"

template <typename S>
static void pack_t(Engine* E, long long cells, int unpack, int nfields, void* packed) {
  PackArgs<S> A;
  memset(&A, 0, sizeof(A));
  for (int l = 0; l < E->cfg.nlevels; ++l) {
    A.lev[l] = E->lev[l].view<S>(0);
    A.dy[l] = E->lev[l].dx[1];
  }
  A.nfields = nfields;
  A.ylo = E->cfg.xlo[1];
  A.E64 = eos_const64(E->cfg);
  A.E32 = eos_const32(E->cfg);
  A.tiles = E->d_tiles.p;
  A.off = E->d_tileoff.p;
  A.ntiles = (int)E->h_tiles.size();
  A.total = cells;
  A.packed = static_cast<S*>(packed);
  A.unpack = unpack;
  const unsigned g = (unsigned)std::max(1, std::min(A.ntiles, 1 << 30));
  if (nfields == 5) {
    if (unpack) pack_kernel<S, 5, true><<<g, 256, 0, stream()>>>(A);
    else pack_kernel<S, 5, false><<<g, 256, 0, stream()>>>(A);
  } else {
    if (unpack) pack_kernel<S, kNF, true><<<g, 256, 0, stream()>>>(A);
    else pack_kernel<S, kNF, false><<<g, 256, 0, stream()>>>(A);
  }
}

extern "C" {

// Host exchange.  An upload copies the host data into a device staging slot
// on the engine's upload stream, and the library stream waits for that copy
// before the unpack kernel; a download packs on the library stream into a
// slot and copies it to the host on the download stream.  Slots alternate,
// so the copies of one exchange overlap the kernels of the steps around it;
// a slot is reused only after its previous kernel and copy are done, and an
// upload whose host range overlaps a pending download waits for that
// download.  The host memory stays in use until enl_engine_sync.
static bool overlap(const void* a, size_t na, const void* b, size_t nb) {
  const char *pa = static_cast<const char*>(a), *pb = static_cast<const char*>(b);
  return na && nb && pa < pb + nb && pb < pa + na;
}

static int xfer_slot(Engine* E, Engine::Xfer& X, size_t bytes, int& q) {
  if (!E->s_in && (cudaStreamCreateWithFlags(&E->s_in, cudaStreamNonBlocking) != cudaSuccess ||
                   cudaStreamCreateWithFlags(&E->s_out, cudaStreamNonBlocking) != cudaSuccess)) {
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  q = X.slot;
  X.slot ^= 1;
  if (!X.copied[q] && (cudaEventCreateWithFlags(&X.copied[q], cudaEventDisableTiming) != cudaSuccess ||
                       cudaEventCreateWithFlags(&X.used[q], cudaEventDisableTiming) != cudaSuccess)) {
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  if (bytes > X.cap[q]) {
    // the slot's previous kernel and copy must be done before it is freed
    cudaEventSynchronize(X.used[q]);
    cudaEventSynchronize(X.copied[q]);
    if (X.dev[q]) cudaFree(X.dev[q]);
    if (cudaMalloc(&X.dev[q], bytes) != cudaSuccess) {
      X.dev[q] = nullptr;
      X.cap[q] = 0;
      set_error(ENL_ERR_CUDA);
      return ENL_ERR_CUDA;
    }
    X.cap[q] = bytes;
  }
  return ENL_OK;
}

static int pack_common(Engine* E, void* host, long long host_bytes, int unpack, int nfields) {
  long long cells = packed_cells(E);
  if (cells == 0) return ENL_OK;
  const size_t bytes = (size_t)cells * nfields * E->esize;
  if (host_bytes < 0 || (size_t)host_bytes < bytes) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  cudaStream_t s = stream();
  Engine::Xfer& X = unpack ? E->xin : E->xout;
  int q = 0;
  int st = xfer_slot(E, X, bytes, q);
  if (st != ENL_OK) return st;
  if (unpack) {
    // the slot's previous unpack has read it; downloads into this host range
    // that may still run have written it (finished ones are dropped)
    cudaStreamWaitEvent(E->s_in, X.used[q], 0);
    if (cudaGetLastError() != cudaSuccess) {  // report earlier failures before the queries below
      set_error(ENL_ERR_CUDA);
      return ENL_ERR_CUDA;
    }
    auto& W = E->host_writes;
    for (size_t r = 0; r < W.size();) {
      if (cudaEventQuery(W[r].done) == cudaSuccess) {
        E->spare_events.push_back(W[r].done);
        W[r] = W.back();
        W.pop_back();
        continue;
      }
      if (overlap(host, bytes, W[r].host, W[r].bytes)) cudaStreamWaitEvent(E->s_in, W[r].done, 0);
      ++r;
    }
    cudaGetLastError();  // a cudaErrorNotReady of the queries is not an error
    cudaMemcpyAsync(X.dev[q], host, bytes, cudaMemcpyHostToDevice, E->s_in);
    cudaEventRecord(X.copied[q], E->s_in);
    cudaStreamWaitEvent(s, X.copied[q], 0);
    if (E->f32s) pack_t<float>(E, cells, 1, nfields, X.dev[q]);
    else pack_t<double>(E, cells, 1, nfields, X.dev[q]);
    cudaEventRecord(X.used[q], s);
  } else {
    // the slot's previous copy to the host has read it
    if (X.pending[q]) cudaStreamWaitEvent(s, X.copied[q], 0);
    if (E->f32s) pack_t<float>(E, cells, 0, nfields, X.dev[q]);
    else pack_t<double>(E, cells, 0, nfields, X.dev[q]);
    cudaEventRecord(X.used[q], s);
    // (earlier uploads have been read: their unpack precedes this pack)
    cudaStreamWaitEvent(E->s_out, X.used[q], 0);
    cudaMemcpyAsync(host, X.dev[q], bytes, cudaMemcpyDeviceToHost, E->s_out);
    cudaEventRecord(X.copied[q], E->s_out);
    X.pending[q] = true;
    cudaEvent_t done = nullptr;
    if (!E->spare_events.empty()) {
      done = E->spare_events.back();
      E->spare_events.pop_back();
    } else if (cudaEventCreateWithFlags(&done, cudaEventDisableTiming) != cudaSuccess) {
      set_error(ENL_ERR_CUDA);
      return ENL_ERR_CUDA;
    }
    cudaEventRecord(done, E->s_out);
    E->host_writes.push_back({host, bytes, done});
  }
  return check_launch(unpack ? "engine upload" : "engine download");
}

int enl_engine_sync(void* e) {
  Engine* E = (Engine*)e;
  if (!E) return ENL_ERR_ARG;
  if (E->s_in) cudaStreamSynchronize(E->s_in);
  if (E->s_out) cudaStreamSynchronize(E->s_out);
  cudaStreamSynchronize(stream());
  return check_launch("engine sync");
}

int enl_engine_download(void* e, void* host, long long host_bytes) {
  Engine* E = (Engine*)e;
  if (!E || !host) return ENL_ERR_ARG;
  return pack_common(E, host, host_bytes, 0, kNF);
}

int enl_engine_upload(void* e, const void* host, long long host_bytes) {
  Engine* E = (Engine*)e;
  if (!E || !host) return ENL_ERR_ARG;
  return pack_common(E, const_cast<void*>(host), host_bytes, 1, kNF);
}

int enl_engine_download_state(void* e, void* host, long long host_bytes) {
  Engine* E = (Engine*)e;
  if (!E || !host) return ENL_ERR_ARG;
  return pack_common(E, host, host_bytes, 0, 5);
}

int enl_engine_upload_state(void* e, const void* host, long long host_bytes) {
  Engine* E = (Engine*)e;
  if (!E || !host) return ENL_ERR_ARG;
  return pack_common(E, const_cast<void*>(host), host_bytes, 1, 5);
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
  for (int k = 0; k < Engine::kCls; ++k) {
    E->kcls_ms[k] = E->kcls_bytes[k] = 0.0;
    E->kcls_n[k] = 0;
  }
  if (on && !E->pev[0])
    for (int q = 0; q < 6; ++q) cudaEventCreate(&E->pev[q]);
  E->profile = on <= 0 ? 0 : on >= 2 ? 2 : 1;
  return check_launch("engine profile");
}

int enl_engine_profile_kernels(void* e, double* ms, double* bytes, long long* launches) {
  Engine* E = (Engine*)e;
  if (!E) return ENL_ERR_ARG;
  for (int k = 0; k < Engine::kCls; ++k) {
    if (ms) ms[k] = E->kcls_ms[k];
    if (bytes) bytes[k] = E->kcls_bytes[k];
    if (launches) launches[k] = E->kcls_n[k];
  }
  return ENL_OK;
}

int enl_engine_set_mlp(void* e, const float* params_host, float margin) {
  Engine* E = (Engine*)e;
  if (!E || !params_host || margin < 0.f) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  if (!E->cfg.learned) {
    set_error(ENL_ERR_STATE);
    return ENL_ERR_STATE;
  }
  if (!E->d_mlp && cudaMalloc(&E->d_mlp, sizeof(MlpSmem)) != cudaSuccess) {
    E->d_mlp = nullptr;
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  MlpSmem img;
  mlp_build_image(params_host, img);
  cudaMemcpyAsync(E->d_mlp, &img, sizeof(MlpSmem), cudaMemcpyHostToDevice, stream());
  cudaStreamSynchronize(stream());
  if (E->margin != margin) E->graph_valid = false;  // the margin is a kernel argument
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
  fill_all(E, 0);
  if (E->f32s) return harvest_t<float>(E, level, dt, scale, keep0, seed, X, labels, capacity, count_dev);
  return harvest_t<double>(E, level, dt, scale, keep0, seed, X, labels, capacity, count_dev);
}


}  // extern "C"
