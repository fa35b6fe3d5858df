/*
 * enlightning_gpu.h -- C-ABI of the GB300 (sm_103a) implementation of
 * Enlightning's per-patch time advance.
 *
 * Part 1 is the drop-in boundary: the four Fortran entry points that
 * enlightning.C calls through enlightningfort.h, with the same symbol names
 * (gfortran mangling of SAMRAI_F77_FUNC: lower case + trailing underscore),
 * the same argument order and the same meaning.  As in the reference every
 * scalar is passed by reference (a C++ reference, or a pointer from C, which
 * is the same ABI).  The difference is where the data lives:
 *   - patch arrays (w_n, source, rhs, pressure, temperature, tags, ww) are
 *     DEVICE pointers in SAMRAI CellData layout (depth-major, i fastest);
 *   - the small geometry arrays (xlo, dx, tag_tolerance) are HOST pointers,
 *     as SAMRAI's CartesianPatchGeometry hands them out.
 * Calls are asynchronous on the library stream (enl_set_stream); the caller
 * synchronises before reading results on the host.  The Fortran routines have
 * no error channel, so these return void; failures are recorded in a sticky
 * error word read with enl_get_last_error().
 *
 * Part 2 adds status-returning entry points (0 = success, nonzero = an
 * ENL_ERR_* code) that the reference has no counterpart for: explicit scheme
 * selection, switch-flag export, the physical-boundary fill and absorbing
 * envelope of enlightning.C as device kernels, the fused stage, the batched
 * multi-level engine and the learned sensor.
 */
#ifndef ENLIGHTNING_GPU_H
#define ENLIGHTNING_GPU_H

#ifdef __cplusplus
#define ENL_REF(T) const T&
extern "C" {
#else
#define ENL_REF(T) const T*
#endif

/* ---------------------------------------------------------------------- */
/* Status codes                                                            */
/* ---------------------------------------------------------------------- */
#define ENL_OK 0
#define ENL_ERR_ARG 1        /* invalid argument (sizes, variant, null)    */
#define ENL_ERR_CUDA 2       /* a CUDA runtime call or launch failed       */
#define ENL_ERR_NONFINITE 3  /* the health check found rho <= 0 or NaN      */
#define ENL_ERR_TIMEOUT 4    /* a bounded device-side wait gave up          */
#define ENL_ERR_STATE 5      /* call order violated (e.g. no engine levels) */

/* RHS scheme ids (the reference picks one at build time, makefile:6). */
#define ENL_HYBRID_HIGH_LLF 0 /* fortran/rhs_hybrid_high_llf.m4 (default) */
#define ENL_HYBRID_HIGH 1     /* fortran/rhs_hybrid_high.m4               */
#define ENL_HYBRID_LOW_LLF 2  /* fortran/rhs_hybrid_low_llf.m4            */
#define ENL_HYBRID_LOW 3      /* fortran/rhs_hybrid_low.m4                */
#define ENL_WENO_HIGH_LLF 4   /* fortran/rhs_weno_high_llf.m4             */
#define ENL_WENO_HIGH 5       /* fortran/rhs_weno_high.m4                 */
#define ENL_WENO_LOW_LLF 6    /* fortran/rhs_weno_low_llf.m4              */
#define ENL_WENO_LOW 7        /* fortran/rhs_weno_low.m4                  */
#define ENL_DRP 8             /* fortran/rhs_drp.m4                       */

/* ====================================================================== */
/* Part 1: drop-in F77 entry points (enlightningfort.h:22-102)             */
/* ====================================================================== */

/* Replaces SAMRAI_F77_FUNC(rhs, RHS), enlightningfort.h:23-49
 * (fortran/rhs_*.m4).  Scheme = the one chosen with enl_set_rhs_variant
 * (default ENL_HYBRID_HIGH_LLF, the reference makefile's default).
 * w_n, pressure, temperature: ghosted (gcw0, gcw1); source, rhs: interior. */
void rhs_(ENL_REF(int) ifirst0, ENL_REF(int) ilast0, ENL_REF(int) ifirst1,
          ENL_REF(int) ilast1, ENL_REF(int) gcw0, ENL_REF(int) gcw1,
          const double* xlo, const double* dx, const double* w_n,
          const double* source, double* rhs, const double* pressure,
          const double* temperature, ENL_REF(double) weno_alpha,
          ENL_REF(double) kappa, ENL_REF(double) mu, ENL_REF(double) muB,
          ENL_REF(double) R, ENL_REF(double) T_star_n,
          ENL_REF(double) T_star_o, ENL_REF(double) tau_n,
          ENL_REF(double) tau_o, const double* tag_tolerance,
          ENL_REF(int) level, ENL_REF(double) c, ENL_REF(double) c_lr,
          ENL_REF(int) nequ);

/* Replaces SAMRAI_F77_FUNC(runge_kutta, RUNGE_KUTTA), enlightningfort.h:51-64
 * (fortran/runge_kutta.m4:57-66): w_n = alpha_1*w + alpha_2*w_n + beta*dt*rhs
 * over the interior.  w_n ghosted; w and rhs interior-only. */
void runge_kutta_(ENL_REF(int) ifirst0, ENL_REF(int) ilast0,
                  ENL_REF(int) ifirst1, ENL_REF(int) ilast1, ENL_REF(int) gcw0,
                  ENL_REF(int) gcw1, ENL_REF(double) dt, ENL_REF(double) alpha_1,
                  ENL_REF(double) alpha_2, ENL_REF(double) beta, double* w_n,
                  const double* w, const double* rhs, ENL_REF(int) nequ);

/* Replaces SAMRAI_F77_FUNC(update_state, UPDATE_STATE), enlightningfort.h:66-88
 * (fortran/update_state.m4:87-107).  Note dx comes before xlo here. */
void update_state_(const double* dx, const double* xlo, ENL_REF(int) ifirst0,
                   ENL_REF(int) ilast0, ENL_REF(int) ifirst1,
                   ENL_REF(int) ilast1, ENL_REF(int) gcw0, ENL_REF(int) gcw1,
                   const double* w_n, double* pressure, double* temperature,
                   ENL_REF(double) rho0, ENL_REF(double) c,
                   ENL_REF(double) gamma1, ENL_REF(double) c_p,
                   ENL_REF(double) p0, ENL_REF(double) T0,
                   ENL_REF(double) c_lr, ENL_REF(double) c_v,
                   ENL_REF(double) R_tilde, ENL_REF(double) M,
                   ENL_REF(double) R, ENL_REF(int) nequ);

/* Replaces SAMRAI_F77_FUNC(tag_cells, TAG_CELLS), enlightningfort.h:90-101
 * (fortran/tag_cells.m4:58-108).  tags interior-only (int); w_n and source
 * ghosted.  Bit-exact with the reference. */
void tag_cells_(ENL_REF(int) ifirst0, ENL_REF(int) ilast0,
                ENL_REF(int) ifirst1, ENL_REF(int) ilast1, ENL_REF(int) gcw0,
                ENL_REF(int) gcw1, int* tags, const double* w_n,
                const double* source, ENL_REF(int) refine_tag_val,
                const double* tag_tolerance, ENL_REF(int) nequ);

/* ====================================================================== */
/* Part 2: library control and extended entry points                      */
/* ====================================================================== */

/* Stream all calls enqueue on (a cudaStream_t; NULL = legacy default). */
int enl_set_stream(void* stream);
/* Sticky error word: first ENL_ERR_* recorded since the last call. */
int enl_get_last_error(void);
const char* enl_error_string(int code);
/* Scheme used by rhs_ (ENL_* id).  The reference fixes it at build time. */
int enl_set_rhs_variant(int variant);
int enl_get_rhs_variant(void);

/* rhs_ with an explicit scheme, an optional per-cell switch output
 * (flags: device int[nx*ny], 1 = WENO, 0 = DRP; may be NULL) and explicit
 * row pitches so patches stored inside a larger array can be addressed.
 * w_pitch/w_fstride: elements between rows / fields of w_n (pressure and
 * temperature share w_pitch and hold one field each); out_pitch/out_fstride
 * likewise for rhs, source uses out_pitch.  Everything else as rhs_.
 * Follows fortran/rhs_<variant>.m4. */
int enl_rhs(int variant, int ifirst0, int ilast0, int ifirst1, int ilast1,
            int gcw0, int gcw1, const double* xlo, const double* dx,
            const double* w_n, long w_pitch, long w_fstride,
            const double* source, double* rhs, long out_pitch,
            long out_fstride, const double* pressure,
            const double* temperature, double weno_alpha, double kappa,
            double mu, double muB, double R, double T_star_n, double tau_n,
            const double* tag_tolerance, int level, double c, double c_lr,
            int* flags);

/* Physical-boundary ghost fill of one patch, enlightning.C:790-1013.
 * touches[4] (host): patch side lies on the domain boundary (L, R, B, T).
 * bc[4] (host): 10 = REFLECT, 20 = ABSORB.  fill0/fill1: ghost width to fill.
 * Arrays ghosted (SAMRAI layout): w_n (5 fields), pressure, temperature,
 * source. */
int enl_phys_bc(int ifirst0, int ilast0, int ifirst1, int ilast1, int gcw0,
                int gcw1, const int* touches, const int* bc, int fill0,
                int fill1, double* w_n, double* pressure, double* temperature,
                double* source);

/* Absorbing envelope of one patch, enlightning.C:634-786 (including its loop
 * exit rules).  patch_xlo, dx, grid_xlo, grid_xhi, bc: host arrays. */
int enl_absorb(int ifirst0, int ilast0, int ifirst1, int ilast1, int gcw0,
               int gcw1, const double* patch_xlo, const double* dx,
               const double* grid_xlo, const double* grid_xhi, const int* bc,
               double absorb_width, double p0, double T0, double rho0,
               double* w_n, double* pressure, double* temperature);

/* ====================================================================== */
/* Part 3: batched multi-level engine                                      */
/* ====================================================================== */
/* All patches of all AMR levels advance together.  Each level is stored as
 * one ghosted canvas covering the whole level index space (3 ghost cells on
 * every side, 7 FP64 fields: rho, rho*u, rho*v, rho*s, rho*T_n, p, T), with
 * three such buffers (current, stage A, stage B) plus the source H0.
 * Patches are index boxes into the canvas: same-level ghost exchange is a
 * read of the neighbour's cells, coarse-fine ghosts are filled by bilinear
 * interpolation from the coarser canvas (the reference registers
 * LINEAR_REFINE, enlightning.C:259-288), physical ghosts by the rule of
 * enlightning.C:790-1013, and fine data is averaged onto the coarse level
 * after every step (CONSERVATIVE_COARSEN).  One RK3 step = per stage: ghost
 * fill of every level, then one persistent kernel over a device tile list
 * that fuses rhs + runge_kutta + update_state; the absorbing envelope and the
 * coarsening follow.  The whole step can be captured once as a CUDA graph and
 * replayed until the next regrid (the tile and halo tables are device data,
 * so a regrid rewrites them without a new capture unless they outgrow their
 * capacity). */

#define ENL_MAX_LEVELS 4
#define ENL_PREC_FP64 0   /* RHS in FP64: same results as the plain path   */
#define ENL_PREC_FP32 1   /* RHS in FP32 perturbation form, FP64 state     */
#define ENL_PREC_FP32_STATE 2 /* FP32 throughout: canvases hold FP32
                             perturbations about the ambient state (rho -
                             rho0, rho u, rho v, rho s, rho T_n - rho0 T0,
                             p - p0, T - T0); no plain path            */

typedef struct {
  int nlevels;            /* 1..ENL_MAX_LEVELS                              */
  int ratio;              /* refinement ratio between levels (2)            */
  int nx0, ny0;           /* level-0 cells                                   */
  double xlo[2];          /* domain lower corner (m)                         */
  double dx0[2];          /* level-0 cell size (m)                           */
  int bc[4];              /* L, R, B, T: 10 = REFLECT, 20 = ABSORB           */
  int variant;            /* ENL_* scheme id                                 */
  int precision;          /* ENL_PREC_FP64, ENL_PREC_FP32, ENL_PREC_FP32_STATE */
  int learned;            /* 1: learned switch on level 0 (reviews the plain
                             switch's WENO cells); 2: on every level (on the
                             fine levels, where the reference always uses
                             WENO, it reviews every cell); 0: off          */
  double weno_alpha, kappa, mu, muB, R, T_star_n, tau_n, c, c_lr;
  double tol[3];
  double rho0, gamma1, c_p, p0, T0, c_v;
  double absorb_width;
  double rk_alpha1[3], rk_alpha2[3], rk_beta[3];
  int independent;        /* 1: every level-0 patch is its own domain whose
                             sides are physical boundaries (batched independent
                             problems; nlevels must be 1, patches >= 6 cells
                             apart on the canvas)                         */
  int dense;              /* 0 (default): a stage tile whose staged inputs are
                             bitwise uniform (one value per field over the
                             halo box, shared u^n and H0, no absorbing band,
                             c_lr = 0) stores the outputs the block computed
                             for an earlier tile with the same inputs, which
                             are the outputs every one of its cells would
                             compute; 1: every tile is computed cell by cell.
                             The states are identical either way.          */
  int tile_order;         /* order in which the stage kernel's blocks claim
                             tiles: 0 (default) finest level first (the WENO
                             tiles of the fine levels start first and the
                             cheaper coarse tiles balance the end), 1 level 0
                             first, 2 finest and level-0 tiles alternately,
                             3 two streams: each SM's first block takes tiles
                             from the finest end, its second from level 0.
                             Every order gives the same states.            */
} enl_engine_config;

/* Create / destroy.  Allocates the canvases of every level (device memory). */
int enl_engine_create(const enl_engine_config* cfg, void** engine);
int enl_engine_destroy(void* engine);
/* Device canvas of one level: which = 0 current, 1 stage A, 2 stage B,
 * 3 source H0.  Cell (i, j) of the level (i, j >= -3) is element
 * base[k*fstride + (j+3)*pitch + (i+3)] of field k, in the storage type of
 * the engine (enl_engine_storage). */
int enl_engine_buffer(void* engine, int level, int which, void** base,
                      long* pitch, long* fstride, int* nx, int* ny);
/* Storage of the canvases and of the packed state: element size (8 = double,
 * 4 = float) and, per field, the ambient value held out of the storage
 * (absolute value = offsets[k] + stored value; all 0 for FP64 storage).
 * offsets may be NULL. */
int enl_engine_storage(void* engine, int* elem_bytes, double* offsets);
/* Patch boxes of one level, (ilo, ihi, jlo, jhi) per patch in that level's
 * index space, host array of 4*npatch ints.  Level l > 0 boxes must be
 * properly nested in level l-1 (after coarsening).  ilo must be even (a
 * multiple of 4 with FP32 storage): tile rows are TMA copies. */
int enl_engine_set_patches(void* engine, int level, int npatch, const int* boxes);
/* Fill the cells of the given boxes of `level` (current buffer) by bilinear
 * interpolation from level-1 (new fine data after a regrid). */
int enl_engine_refine_init(void* engine, int level, int nbox, const int* boxes);
/* Ghost fill of buffer `which` on every level (physical + coarse-fine). */
int enl_engine_fill(void* engine, int which);
/* One RK3 step of the batched fused path (kernel launches on the stream). */
int enl_engine_step(void* engine, double dt);
/* One RK3 step of the plain path: per patch, unfused FP64 rhs, runge_kutta
 * and update_state launches (what enlightning.C issues through the F77
 * entry points), same storage and ghost fill.  FP64 storage only
 * (ENL_ERR_STATE otherwise). */
int enl_engine_step_plain(void* engine, double dt);
/* Capture one fused step as a CUDA graph, then replay it nsteps times.
 * Kernels read tile, halo and patch tables from device memory, so a regrid
 * (enl_engine_set_patches) keeps the graph valid unless a table outgrows its
 * capacity; enl_engine_graph_valid (1/0) tells whether a new capture is
 * needed. */
int enl_engine_graph_capture(void* engine, double dt);
int enl_engine_graph_replay(void* engine, int nsteps);
int enl_engine_graph_valid(void* engine);
/* tag_cells over the patches of `level` (fortran/tag_cells.m4), into a
 * device int array of nx*ny (level index space, row pitch nx); cells outside
 * the patches are 0.  Fills ghosts of the current buffer and H0 first. */
int enl_engine_tag(void* engine, int level, int* tags);
/* Counters of the last steps: per level, cells advanced with WENO, cells in
 * total, cells the learned switch left to the plain switch, and cells of
 * uniform tiles whose outputs came from the block's cache (host array of
 * 4*ENL_MAX_LEVELS long long), then reset. */
int enl_engine_stats(void* engine, long long* counts);
/* Uniform-tile skipping in the last step's RK stage 3 (schedule reuse 2):
 * tiles whose halo box the records of stage 2 proved uniform (flagged), of
 * those the tiles stored from a cached or published result without loading
 * their box (written; the others took the full path in a second launch,
 * which happens when blocks reach them before any block has computed a
 * tile with their key), and the tiles of the hierarchy.  written and tiles
 * may be NULL.  Synchronises the library stream.  0 when skipping is off. */
int enl_engine_skipped_tiles(void* engine, long long* flagged, long long* written, long long* tiles);
/* Health word: 0, or the first code a kernel raised since the last call:
 * ENL_ERR_NONFINITE (rho <= 0 or non-finite state), ENL_ERR_TIMEOUT (a
 * bounded wait gave up), ENL_ERR_STATE (a TMA precondition failed and the
 * copy was not issued). */
int enl_engine_health(void* engine);
/* Number of kernel launches one enl_engine_step issues (for accounting). */
int enl_engine_launches_per_step(void* engine, int plain);

/* Adaptive time step computed on the device at the start of every step:
 * dt = cfl * (finest dx) / max over all patch cells of max(|u|,|v|) + c, a
 * warp-shuffle max reduction; stage kernels read dt from device memory, so a
 * captured graph stays valid.  The dt passed to enl_engine_step is then an
 * upper bound.  Off by default (the reference uses cfl*dx/c,
 * enlightning.C:433-456). */
int enl_engine_set_adaptive_dt(void* engine, int on, double cfl);
/* Last device dt and accumulated simulated time (adaptive mode). */
int enl_engine_time(void* engine, double* dt_last, double* sim_time);
/* Restore them (restart). */
int enl_engine_set_time(void* engine, double dt_last, double sim_time);

/* State exchange with host memory: the current buffer's patch interiors of
 * every level, packed (7 fields, tile order: level by level, patch by patch,
 * 32x8 tiles row-major).  Elements are of the storage type
 * (enl_engine_storage: doubles, or FP32 perturbations);
 * enl_engine_packed_size gives their number.  host_bytes is the size of the
 * host buffer (ENL_ERR_ARG, and nothing copied, when it is smaller than the
 * packed state).  Asynchronous: the host copies run on the engine's own
 * upload and download streams and are ordered with the kernels on the
 * library stream by events (an upload is what the next step reads; a
 * download holds the state after the work enqueued before it), so they
 * overlap the steps around them.  Two device staging slots per direction
 * alternate.  Host memory should be pinned; a host buffer stays in use until
 * enl_engine_sync returns (do not change an upload's source or read a
 * download's target before).  An upload from host memory that a pending
 * download writes waits for that download. */
int enl_engine_packed_size(void* engine, long long* nelems);
int enl_engine_download(void* engine, void* host, long long host_bytes);
int enl_engine_upload(void* engine, const void* host, long long host_bytes);
/* The same with the conserved state only (rho, rho u, rho v, rho s,
 * rho T_n: 5 of the 7 fields, nelems * 5/7 elements); the upload recomputes
 * p and T on the device with update_state (update_state.m4:90-105). */
int enl_engine_download_state(void* engine, void* host, long long host_bytes);
int enl_engine_upload_state(void* engine, const void* host, long long host_bytes);
/* Wait for the engine's host copies and the library stream. */
int enl_engine_sync(void* engine);

/* Stage-kernel timing: with on = 1 every direct (not graph) enl_engine_step
 * brackets its three stage-kernel launches with CUDA events on the stream;
 * on = 2 also brackets every launch of the step's other kernels.  Returns
 * (and resets, with the per-class figures below) the accumulated
 * stage-kernel milliseconds, launches and cells advanced by them since the
 * previous call. */
int enl_engine_profile(void* engine, int on, double* ms_total,
                       long long* launches, long long* cells);

/* Per-class figures of profile mode 2 since the last enl_engine_profile
 * call, six entries each: 0 coarse-fine halo interpolation, 1 physical
 * band fill, 2 coarsening, 3 CFL maximum (speed + dt kernels), and with
 * uniform-tile skipping (schedule reuse 2, RK stages 2 and 3) 4 the flag
 * pass and tile lists, 5 the second stage launch (bytes 0 for these two;
 * their time is also inside the stage figures of enl_engine_profile).  bytes are
 * algorithmic: every cell value the launch must read or write, once
 * (interpolation: the halo cells written and the distinct coarse cells
 * under their 2 x 2 stencils; band fill: one read and one write per band
 * cell; coarsening: ratio^2 fine reads and one write per coarse cell; CFL:
 * rho, rho u, rho v of every patch cell), 7 fields of the storage type. */
int enl_engine_profile_kernels(void* engine, double* ms, double* bytes,
                               long long* launches);

/* Stage order across levels.  samrai = 0 (default): in every RK stage all
 * levels fill their ghosts from the same stage input and advance in one
 * launch.  samrai = 1: the order of SAMRAI's MethodOfLinesIntegrator, which
 * the reference drives (main.C:448): per stage the levels go coarsest first,
 * each filling its ghosts (coarse-fine ones interpolated from the coarser
 * level after that level's update in the same stage) and then advancing, one
 * launch per level.  Invalidates a captured graph. */
int enl_engine_set_level_order(void* engine, int samrai);

/* Stage-kernel schedule.  Replaces SAMRAI's patch-to-rank load balancing
 * (main.C:268-301): every patch of every level shares one persistent grid,
 * and the schedule decides how its blocks take the tiles.
 *   sched[0] resident blocks per SM (0 = the occupancy limit),
 *   sched[1] tile order (as enl_engine_config.tile_order),
 *   sched[2] uniform-tile reuse: 2 on (the default), with RK stages 2 and 3
 *            skipping the halo box of a tile whose own and neighbours'
 *            records from the previous stage of the step prove it uniform;
 *            1 on, every tile's box loaded and tested; 0 off (as
 *            enl_engine_config.dense = 1),
 *   sched[3] run length: tiles a block claims at a time (1..16; consecutive
 *            tiles of a patch row, so 2 and 4 claim 64x8 and 128x8 cells).
 * Every schedule gives the same states.  Setting one invalidates a captured
 * graph.  get_schedule writes sched[0..3] (sched[0] as the actual count) and
 * sched[4] = the occupancy limit; n is the length of the array (>= 4 to set,
 * >= 5 to get). */
int enl_engine_set_schedule(void* engine, const int* sched, int n);
int enl_engine_get_schedule(void* engine, int* sched, int n);
/* Autotuner: times candidate schedules (blocks per SM in the upper half of
 * the occupancy range x the four tile orders x reuse 2 and 0 x runs of 1, 2, 4
 * tiles, and reuse 1 with runs of 1) on the current hierarchy and state, `steps` timed steps each after
 * one untimed step, with CUDA events on the library stream; the three
 * fastest and the schedule in force are timed again and the fastest is
 * applied.  The current canvases, time step, simulated time, statistics and
 * health word are restored after every candidate and at the end, and
 * microphones record nothing meanwhile: the simulation is left where it
 * was.  tried[4*k..4*k+3] and ms[k] (milliseconds per step, best of the
 * candidate's rounds) receive up to cap candidates; *ntried (may be NULL)
 * their number.  Allocates one copy of the current canvases for the call. */
int enl_engine_autotune(void* engine, double dt, int steps, int cap, int* tried,
                        float* ms, int* ntried);

/* ---------------------------------------------------------------------- */
/* Learned hybrid sensor                                                   */
/* ---------------------------------------------------------------------- */
/* A 40 -> 64 -> 64 -> 1 MLP (GELU) replacing the hybrid switch of
 * fortran/rhs_hybrid_high_llf.m4:239-256 on level 0 of the FP32 engine.
 * Parameters are one FP32 vector of enl_mlp_nparams() floats: W1[40][64],
 * b1[64], W2[64][64], b2[64], w3[64], b3.  Kernels compute with BF16 weights
 * and activations on the tensor cores, FP32 accumulation.  Cells whose logit
 * is within +-margin of 0 are decided by the plain switch. */
int enl_mlp_nparams(void);
/* The network's GELU uses erf by Abramowitz & Stegun 7.1.26 (|error| <=
 * 1.5e-7 in exact arithmetic, evaluated in FP32); this returns its largest
 * difference from the CUDA math library's erff over 4M points in [-6, 6]. */
int enl_mlp_erf_error(double* max_err);
/* Logits of n feature rows (device BF16 [n][40]) into device float[n]. */
int enl_mlp_forward(const void* X, long n, const float* params, float* logits);
/* Sums over the n rows of the weighted BCE-with-logits loss gradient
 * (device arrays; grad is accumulated into, loss_sum too, may be NULL). */
int enl_mlp_grad(const void* X, const float* y, const float* weight, long n,
                 const float* params, float* grad, double* loss_sum);
/* One Adam step on the device parameters (grad scaled by inv_n). */
int enl_mlp_adam(float* params, const float* grad, float* m, float* v,
                 float lr, float beta1, float beta2, float eps, float inv_n,
                 int step);
/* Install the network (host FP32 vector) in an engine created with
 * learned = 1 (any precision). */
int enl_engine_set_mlp(void* engine, const float* params_host, float margin);
/* Harvest training rows from a level of the engine (plain FP64 arithmetic):
 * features (device BF16 [capacity][40]), labels (device float [capacity][2]
 * = plain switch, max_k dt|KK_drp - KK_weno|/scale_k), count_dev (device
 * counter, incremented).  WENO-flagged cells are all kept, DRP cells with
 * probability keep0. */
int enl_engine_harvest(void* engine, int level, double dt, const double* scale,
                       double keep0, unsigned seed, void* X, float* labels,
                       long capacity, unsigned long long* count_dev);

/* Source painting on the H0 canvas of one level over its patches, as
 * enlightning::addSource does (enlightning.C:2140-2307): type 10 = POINT,
 * 20 = SINE, 30 = LIGHTNING; mode 10 = PULSE, 20 = DRIVEN (POINT only; the
 * painted value is multiplied by `drive` = sin(omega*(n+1-n0)*dt)).  amp and
 * spread as src_amp / src_spread (Gaussian exp(-ln2 r^2/spread^2)); pos (host,
 * 2 doubles) for POINT and SINE; segs (host, 4*nseg doubles x0,y0,x1,y1) for
 * LIGHTNING, accumulated in order with the capsule-union rule. */
int enl_engine_paint_source(void* engine, int level, int type, int mode,
                            double amp, double spread, const double* pos,
                            double sine_amp, double sine_freq, int nseg,
                            const double* segs, double drive);
/* Read H0 of a level as an overpressure and write the corresponding ambient-
 * entropy state (inverse of update_state.m4:90-94) into the current buffer on
 * the level's patches; H0 is zeroed.  Builds synthetic initial conditions. */
int enl_engine_state_from_overpressure(void* engine, int level);
/* Regrid helper: tag_cells on `level`, then a block map (host array of
 * nbx*nby bytes, block x block cells per entry) marking blocks with a tagged
 * cell within `buffer` cells.  With map_host == NULL only nbx, nby are set. */
int enl_engine_tag_blocks(void* engine, int level, int block, int buffer,
                          unsigned char* map_host, int* nbx, int* nby);
/* One regrid of level+1 from the tags of `level` (SAMRAI's gridding step
 * for the reference, main.C:489-502) in one call: enl_engine_tag_blocks,
 * proper nesting inside the patches of `level` (eroded by nest_blocks blocks
 * for level > 0), enl_cluster_tags, fine boxes (block * ratio cells per block
 * side, sizes min_size..max_size fine cells), enl_engine_set_patches and
 * enl_engine_refine_init of the cells the old fine patches did not cover. */
int enl_engine_regrid(void* engine, int level, int block, int tag_buffer,
                      int nest_blocks, double efficiency, int min_size,
                      int max_size);
/* Host wall time (ms) spent in enl_engine_regrid since the last call, by
 * phase: waiting for the steps already queued, device tagging with the block
 * map read back, clustering, tables, refine launches; then reset. */
int enl_engine_regrid_timing(void* engine, double* ms5);

/* The stage kernel's bounded mbarrier wait, on its own: one block waits on a
 * barrier that one arrival completes (arrive = 1) or that nothing completes
 * (arrive = 0).  Returns ENL_OK, or ENL_ERR_TIMEOUT once `polls` polls have
 * passed — the way a copy that never lands is reported instead of hanging
 * the GPU (the context stays usable). */
int enl_check_bounded_wait(int polls, int arrive);
/* Patch boxes of a level (host array of 4*max_boxes ints); npatch = count. */
int enl_engine_get_patches(void* engine, int level, int* boxes, int max_boxes,
                           int* npatch);

/* Virtual microphones, enlightning::recordAudio (enlightning.C:2392-2506):
 * with nmics > 0, every enl_engine_step (and graph replay) ends by sampling
 * the pressure for each microphone (xy: host, x0, y0, x1, y1, ... in metres)
 * in every patch of every level whose closed extent contains it, at
 * i = int((x - patch xlo)/dx), j = int((y - patch ylo)/dy), read as element
 * j*nx + i of the patch interior as the reference indexes it (NaN where
 * that falls past the patch).  Records go to a device buffer of `capacity`
 * entries; `iteration` is the number of the last completed step (the next
 * step records iteration + 1).  nmics = 0 turns sampling off.  Setting or
 * clearing microphones invalidates a captured graph. */
typedef struct {
  int iteration, mic, level, patch; /* patch: index over all levels, level-major */
  double p;
} enl_mic_record;
int enl_engine_set_mics(void* engine, int nmics, const double* xy,
                        long long capacity, int iteration);
/* Copy up to max records (in device arrival order) to host memory and empty
 * the buffer; dropped = records lost to a full buffer. */
int enl_engine_mic_records(void* engine, void* host, long long max,
                           long long* n, long long* dropped);

/* Host-side clustering of a tag map (nx*ny bytes, row-major, e.g. the block
 * map of enl_engine_tag_blocks) into boxes (ilo, ihi, jlo, jhi) in map
 * coordinates, as SAMRAI's BergerRigoutsos does for the reference
 * (main.C:261-265, input.txt:123-127): boxes cover every tag inside
 * `allowed` (NULL: everywhere; proper nesting), after nest_erode erosions
 * of `allowed` by the 3x3 square (cells outside the map count as allowed),
 * never cover a disallowed cell, reach `efficiency` tagged fraction or
 * cannot be cut further, and have no side longer than max_size.  Writes at
 * most max_boxes boxes and the count needed to nboxes (ENL_ERR_ARG when
 * that exceeds max_boxes).  No GPU involved. */
int enl_cluster_tags(const unsigned char* tags, const unsigned char* allowed,
                     int nx, int ny, int nest_erode, double efficiency,
                     int min_size, int max_size, int* boxes, int max_boxes,
                     int* nboxes);

/* Arithmetic ceilings of the current device, measured now (no counterpart in
 * the reference; it states the FP64 ceiling that bounds the FP64 right-hand
 * side).  Writes out[0] = FP64 fused multiply-add rate (TFLOP/s, 2 flops per
 * FMA), out[1] = correctly rounded FP64 divisions (G/s), out[2] = FP32 fused
 * multiply-add rate (TFLOP/s), each the best of three launches of
 * independent dependency chains over every SM.  n >= 3.  Synchronous; takes
 * some tens of milliseconds. */
int enl_measure_fp_peaks(double* out, int n);

/* Host-side: the coarse-fine halo of a level's patches (nbox boxes ilo, ihi,
 * jlo, jhi) — the cells of [0,nx)x[0,ny) within 3 cells (Chebyshev) of the
 * patch union and in no patch — as row segments (j, i_begin, i_end) in row
 * order, left to right, the cells the engine interpolates from the coarser
 * level.  Writes at most max_segs segments (3 ints each) and the count
 * needed to nseg (ENL_ERR_ARG when that exceeds max_segs).  No GPU
 * involved. */
int enl_halo_segments(const int* boxes, int nbox, int nx, int ny, int* segs,
                      int max_segs, int* nseg);

/* Host-side: the 32x8 stage tiles of one level's patches (nbox boxes ilo,
 * ihi, jlo, jhi; per patch row-major from its corner) and, per tile, the
 * table indices of the eight tiles whose interiors hold its 3-cell halo
 * ring, as the uniform-tile skipping uses them (above left, above, above
 * right, left, right, below left, below, below right), or -1 in the first
 * slot when the engine does not skip that tile.  tiles receives (i0, j0,
 * width, height) per tile, nbr 8 ints per tile; at most max_tiles tiles, the
 * count needed in ntiles (ENL_ERR_ARG when that exceeds max_tiles).  No GPU
 * involved. */
int enl_tile_neighbours(const int* boxes, int nbox, int* tiles, int* nbr, int max_tiles,
                        int* ntiles);

/* ---------------------------------------------------------------------------
 * Allocation-free stable time step of one patch.  No counterpart in the
 * reference (its dt, enlightning.C:433-456, needs no reduction); it is for
 * callers that cannot allocate device memory when they need a time step.
 * dt_out (device, 1 double) = min(dt_max, cfl * min(dx) / max over the patch
 * interior of max(|u|,|v|) + c), the same value as the engine's device CFL
 * reduction.  w_n as in rhs_ (SAMRAI layout, ghosts gcw0/gcw1).  Scratch is a
 * static device array of 4096 partial maxima, one per 32x8 tile: patches of
 * more than 4096 tiles (1,048,576 cells) are refused with ENL_ERR_ARG.  All
 * calls share that array, so calls that overlap on the GPU race; the first
 * call on a device looks up its address and belongs before any stream
 * capture (the address is cached per device and context; after a
 * cudaDeviceReset the next call looks it up again).  A non-finite or non-positive
 * density in the interior makes dt_out a quiet NaN, never a small finite
 * step.  Runs on the stream set with enl_set_stream.
 * ------------------------------------------------------------------------- */
int enl_cfl_dt_static(int ifirst0, int ilast0, int ifirst1, int ilast1,
                      int gcw0, int gcw1, const double* w_n, const double* dx,
                      double c, double cfl, double dt_max, double* dt_out);

#ifdef __cplusplus
}
#endif
#endif /* ENLIGHTNING_GPU_H */
