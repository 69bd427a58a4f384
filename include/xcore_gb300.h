/*
 * xcore_gb300.h -- C ABI of the GB300 (sm_103a) drop-in for the per-timestep
 * hot path of xcore.jl (aelligp/xcore.jl).
 *
 * The reference's "operator API" is a set of plain Julia functions that mutate
 * caller-allocated state structs in place (src/phsevo.jl, src/fluidmech.jl,
 * src/noise.jl, src/update.jl, src/store.jl, src/diagnose.jl).  This library
 * keeps that state resident in GPU memory inside an opaque context with the
 * reference's field names and sizes (column-major, z the leading dimension,
 * src/state.jl:101-122, 218-258; src/noise.jl:82-92), and exports one entry
 * point per reference function.  Julia binds them with ccall (the binding is
 * xcore.jl_gb300/julia/XcoreGPU.jl); no torch or CUDA types appear in any
 * signature.
 *
 * Conventions
 *  - Every function returns an xc_status; on failure xc_last_error() holds a
 *    one-line message for the calling thread.  Nothing throws across the ABI.
 *  - A context owns its device buffers and a non-blocking CUDA stream; all work
 *    of that context is ordered on that stream.  A context is not thread safe;
 *    separate contexts are independent.  Functions that return host scalars
 *    synchronise the stream; the others only enqueue work.
 *  - The library never frees caller memory.  Host arrays passed in are read or
 *    written during the call only.
 *  - There is no CPU fallback: without a usable CUDA device every call that
 *    needs one returns XC_NO_DEVICE.
 */
#ifndef XCORE_GB300_H
#define XCORE_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum xc_status {
  XC_OK = 0,
  XC_BAD_ARG = 1,        /* size / scheme / BC argument the reference rejects
                            (@assert and ArgumentError, advect.jl:378-385,421;
                            ghosts.jl:35,47; timing.jl:35) */
  XC_NOT_CONVERGED = 2,  /* iterative Stokes solve hit its iteration limit */
  XC_NAN = 3,            /* non-finite residual (diagnose.jl:80 raises) */
  XC_TIMEOUT = 4,        /* a bounded device wait gave up */
  XC_CUDA = 5,           /* a CUDA runtime call failed */
  XC_NO_DEVICE = 6       /* no CUDA device available */
} xc_status;

/* advection schemes, par.ADVN (src/parameters.jl:74; advect.jl:346-355) */
typedef enum xc_scheme {
  XC_CENTR = 0, XC_UPWD1 = 1, XC_QUICK = 2, XC_FROMM = 3,
  XC_WENO3 = 4, XC_WENO5 = 5, XC_TVDIM = 6
} xc_scheme;

/* boundary conditions per axis (ghosts.jl:18-51) */
typedef enum xc_bc { XC_PERIODIC = 0, XC_CLOSED = 1 } xc_bc;

/* time integrators, par.TINT (src/timing.jl:18-36) */
typedef enum xc_tint { XC_BE1IM = 0, XC_BD2IM = 1, XC_CN2SI = 2, XC_BD2SI = 3 } xc_tint;

/* Stokes solver kinds (the reference always factorises with UMFPACK,
   fluidmech.jl:512-522; these replace that solve) */
typedef enum xc_solver_kind {
  XC_SOLVER_FGMRES_FP64 = 0,   /* FP64 FGMRES + FP64 multigrid / Schur preconditioner */
  XC_SOLVER_MIXED = 1          /* FP32 FGMRES + FP32 multigrid inside FP64 iterative refinement */
} xc_solver_kind;

/*
 * Scalars of Parameters{Float64} (src/parameters.jl:12-89) and Scales
 * (src/scales.jl:13-57) that the path reads, plus the boundary keywords of
 * run! (src/run.jl:174-180).  Scales are computed by the caller (they are
 * one-off host scalars in the reference) and passed in.
 */
typedef struct xc_params {
  int Nz, Nx;              /* grid.Nz, grid.Nx (src/grid.jl:311-334) */
  double h, D;             /* grid.h, par.D */
  double rhom0, rhox0, d0, g0, etam0, etax0;
  double AA[4], BB[4], CC[4];  /* 2x2 rheology matrices, row-major [11,12,21,22] */
  double Xi, Ptop, alpha, gamma, CFL, dtmax, etacntr;
  int open_sgr;            /* 0/1 */
  /* scales */
  double L0, l0, L0h, l0h, D0, txi0, G0, bnd_w, dt0;
  int ADVN;                /* xc_scheme */
  int TINT;                /* xc_tint */
  int xBC, zBC;            /* xc_bc; the reference default is periodic x, closed z */
  int sds, top_cnv, bot_cnv, open_cnv;   /* fluidmech! keywords (fluidmech.jl:71-80) */
  int weno_weights;        /* WENO5 nonlinear weights (advect.jl:35-53): 0 the reference's form,
                              three divisions for the weights and one to normalise them, bit for
                              bit; 1 the same weights over a common denominator, one division per
                              reconstruction (within a few ulps of the reference: its 1e-12 stencil
                              tolerance) */
} xc_params;

typedef struct xc_solver_opts {
  int kind;          /* xc_solver_kind */
  double rtol;       /* relative residual target of the (scaled) saddle system */
  int maxit;         /* outer iteration cap */
  int restart;       /* FGMRES restart length */
  double inner_rtol; /* mixed: relative reduction per FP32 inner solve */
  int inner_maxit;   /* mixed: FP32 FGMRES iterations per refinement pass */
  /* preconditioner knobs (0 selects the default) */
  int smooth_sweeps;       /* velocity Jacobi sweeps before each coarse correction, and after it
                              unless post_sweeps is given (default 1 before, 2 after; 4 and 4 for MMS) */
  double omega_velocity;   /* damping of the velocity Jacobi smoother (0.7) */
  double schur_mass;       /* weight c of the c*eta/rho term added to the Schur inverse (0.5) */
  int schur_full_diagonal; /* 1: pressure Laplacian from the full velocity diagonal, no mass term */
  int coarse_cells;        /* a velocity level of at most this many cells is the coarsest, a pressure
                              level of a quarter of it (16; 256 for MMS) */
  int coarse_sweeps;       /* Jacobi sweeps on a coarsest level that is not solved with its dense
                              inverse (above 64 unknowns, or jacobi_coarse): 4 (Nz + Nx), at
                              least 32; 200 for MMS */
  int small_cells;         /* levels of at most this many cells run their V-cycle in one CTA
                              (256; -1: none) */
  int pressure_sweeps;     /* pressure-multigrid Jacobi sweeps before and after each coarse
                              correction (2) */
  int inner_gs_passes;     /* mixed: Gram-Schmidt passes of the FP32 inner solve (1; 1 or 2) */
  int serial_launch;       /* 1: plain stream order inside the solver's CUDA graphs instead of
                              programmatic dependent launch (same results) */
  int coarse_viscosity_mean; /* cell viscosity of a coarse multigrid level from its four fine
                                cells: 0 arithmetic (default), 1 geometric, 2 harmonic */
  int tiled_sweep;         /* 1: FP32 velocity sweeps from shared-memory tiles instead of per-row
                              reads (same results; measured 5% slower at 1024^2) */
  int post_sweeps;         /* velocity post-smoothing sweeps on the large levels (2) */
  int outer_solver;        /* mixed: 2 plain iterative refinement x += S dy per inner solve (default),
                              1 FP64 FGMRES whose preconditioner is the FP32 inner solve (measured
                              4% slower at 1024^2: the inner solves' corrections are nearly
                              independent, so keeping them gains no iterations) */
  int fused_pressure_cells; /* pressure-multigrid levels of at most this many cells fuse the first
                               sweep, residual and restriction (descent) and the prolongation and
                               first post sweep (ascent) into one launch each; larger levels launch
                               each operation (same results either way; default and -1: none,
                               measured no faster) */
  int stage_small_levels;  /* 1: the one-CTA V-cycles of the small levels stage them in shared
                              memory instead of reading global memory (same results; measured
                              1.5% slower at 1024^2) */
  int jacobi_coarse;       /* 1: Jacobi sweeps (coarse_sweeps) on the coarsest levels even where they
                              have at most 64 unknowns, which by default are solved with their
                              dense inverse (formed and inverted on the device once per solve) */
  int row_block_sweep;     /* 1: FP32 velocity sweeps with four consecutive rows along z per thread
                              and an interior path without boundary tests (same operations as the
                              default one row per thread; measured 20% slower at 1024^2: the
                              strided per-thread rows cost more L1 wavefronts than the shared
                              loads save) */
  int learned;             /* mixed solver, plain refinement: preconditioner of the FP32 inner
                              solves.  0 the multigrid V-cycles; 1 the learned network
                              (xc_set_learned_preconditioner) in their place, an inner solve that
                              misses inner_rtol redone with the multigrid; 2 the V-cycles followed
                              by the network on the residual they leave.  The FP64 residual of
                              the refinement judges every pass either way. */
  int device_givens;       /* 1: the FGMRES least-squares update (Givens rotations, back
                              substitution) on the device, each Arnoldi step a conditional CUDA
                              graph whose gate kernel skips it once the cycle has stopped, the
                              host queueing the next step before the current one ends (same
                              iterations; measured 7% slower at 1024^2: an IF node costs more
                              than the host round trip it removes).  0: on the host, one
                              synchronisation per Arnoldi step */
  int cluster_cells;       /* velocity multigrid levels below the finest with more than small_cells
                              and at most this many cells run their part of the V-cycle in one
                              launch of a thread-block cluster (16 CTAs; cluster barriers between
                              the operations, the same per-unknown operations as the per-level
                              launches).  0 or -1: none (default; measured 1.7% slower at 1024^2
                              with 16384, even with 4096: the programmatic launches already hide
                              most of the per-level launch gaps) */
} xc_solver_opts;

typedef struct xc_solver_stats {
  int iterations;          /* FP64 FGMRES iterations, or FP32 inner iterations in total */
  int refinements;         /* mixed: FP64 refinement passes */
  double rel_residual;     /* final ||RR - LL x|| / ||RR|| of the scaled system, FP64 */
  int converged;           /* 1 when rel_residual <= rtol */
  double seconds;          /* device time of the solve */
  int learned_fallbacks;   /* inner solves of the learned preconditioner redone with the multigrid */
  int device_givens_steps; /* Arnoldi steps whose least-squares update ran on the device (conditional
                              graphs, device_givens = 1; 0 where those graphs cannot be built) */
} xc_solver_stats;

#define XC_MAX_SWEEPS 64
typedef struct xc_step_stats {
  double resnorm[XC_MAX_SWEEPS];  /* compute_resnorm per Picard sweep (diagnose.jl:57-71) */
  double resnorm0;         /* the loop's reference residual at the end (run.jl:246-249) */
  int sweeps;              /* Picard sweeps run */
  int solver_iterations;   /* summed over sweeps */
  double solver_rel_residual;  /* worst final residual over the sweeps */
  double dt_next;          /* update_dt (update.jl:494-502) */
  int unconverged_solves;  /* Stokes solves that stopped at their iteration cap above their rtol */
  int picard_converged;    /* xc_step_converge: 1 when the loop ended on rtol / atol, 0 on maxit
                              (or after the 3 sweeps of a loop that never met them); xc_step: 0 */
} xc_step_stats;

typedef struct xc_ctx xc_ctx;

/* ------------------------------------------------------------------ */
/* context and fields                                                  */
/* ------------------------------------------------------------------ */

/* Allocate device state for one grid, all fields zero (FluidState /
   PhaseState / NoiseState constructors, src/state.jl:101-122, 218-258,
   src/noise.jl:61-93, incl. the Gaussian filter precompute noise.jl:68-78). */
int xc_ctx_create(const xc_params* par, xc_ctx** out);
int xc_ctx_destroy(xc_ctx* ctx);

/* Field registry: ids 0..xc_field_count()-1 name every state field. */
int xc_field_count(void);
const char* xc_field_name(int id);
int xc_field_id(const char* name);            /* -1 when unknown */
/* rows, cols and element size (8 = Float64, 1 = Bool) of a field */
int xc_field_shape(const xc_ctx* ctx, int id, int* rows, int* cols, int* elem_bytes);
/* Device address of a field (column-major, leading dimension = rows). */
int xc_field_device_ptr(const xc_ctx* ctx, int id, void** dev_ptr);
/* Work in place on the caller's device array for field `id`: every later
   call reads and writes dev_ptr (xc_field_shape's rows x cols, column-major,
   16-byte aligned) instead of the context's own copy -- a CuArray of the
   reference's FluidState / PhaseState (state.jl:74-258) bound field by field
   makes the library a zero-copy drop-in on the caller's state.  The memory
   stays the caller's: it must outlive the binding, and the library never
   frees it.  dev_ptr = NULL unbinds (the context's own copy, with the values
   it held before the binding, is used again).  Synchronises the context
   first, so no queued work sees the switch. */
int xc_field_bind(xc_ctx* ctx, int id, void* dev_ptr);
/* Copy a whole field host -> device / device -> host (synchronous). */
int xc_field_upload(xc_ctx* ctx, int id, const void* host);
int xc_field_download(xc_ctx* ctx, int id, void* host);
/* Wait for all work of the context. */
int xc_synchronize(xc_ctx* ctx);

/* ------------------------------------------------------------------ */
/* one entry point per reference function                              */
/* ------------------------------------------------------------------ */

/* store_previous!(fluid, phase)                         src/store.jl:13-30 */
int xc_store_previous(xc_ctx* ctx);
/* store_noise!(ns)                                      src/noise.jl:115-120 */
int xc_store_noise(xc_ctx* ctx);
/* snapshot!(res, phase, fluid)                          src/diagnose.jl:42-49 */
int xc_snapshot(xc_ctx* ctx);
/* phsevo!(phase, fluid, grid, par, scales; ADVN, xBC, zBC, a1..b3, dt, alpha)
                                                         src/phsevo.jl:164-214
   coefs = (a1, a2, a3, b1, b2, b3); scheme = xc_scheme (par.ADVN when < 0) */
int xc_phsevo(xc_ctx* ctx, int scheme, const double coefs[6], double dt, double alpha);
/* fluidmech!(fluid, grid, par; phase, sds, top_cnv, bot_cnv, open_cnv, xBC,
   zBC, dt, a1..b3)                                      src/fluidmech.jl:71-534
   The UMFPACK factorisation is replaced by the iterative solver in opts
   (NULL = FP64 FGMRES to rtol 1e-10).  stats may be NULL. */
int xc_fluidmech(xc_ctx* ctx, const double coefs[6], double dt,
                 const xc_solver_opts* opts, xc_solver_stats* stats);
/* fluidmech! in MMS mode (bnchm_data != nothing): src_* and *_exact arrays are
   host arrays sized like W (Nz+1,Nx+2), U (Nz+2,Nx+1), P (Nz+2,Nx+2); a context
   with open_cnv set returns XC_BAD_ARG here.
                                                         src/fluidmech.jl:115,218,243,320,421-476 */
int xc_fluidmech_mms(xc_ctx* ctx, const double* src_W, const double* src_U, const double* src_P,
                     const double* W_exact, const double* U_exact, const double* P_exact,
                     const double coefs[6], double dt,
                     const xc_solver_opts* opts, xc_solver_stats* stats);
/* noise!(ns, phase, grid, par, scales, dt; first_iter)  src/noise.jl:138-239
   The white noise that the reference draws with randn!(ns.rng, ...) on the
   first sweep (noise.jl:154-157) is passed in: re/rs are host (Nz, Nx) arrays
   copied in when first_iter != 0; NULL keeps the draws already on the device. */
int xc_noise(xc_ctx* ctx, double dt, int first_iter, const double* re, const double* rs);
/* update_phase_velocities!(phase, fluid, ns, grid, par; xBC, zBC)
   incl. update_segregation_speed!                       src/store.jl:47-105 */
int xc_update_phase_velocities(xc_ctx* ctx);
/* update!(phase, fluid, grid, par, scales; xBC, zBC)    src/update.jl:525-538 */
int xc_update(xc_ctx* ctx);
/* dt = update_dt(phase, fluid, grid, par, dt_prev)      src/update.jl:494-502 */
int xc_update_dt(xc_ctx* ctx, double dt_prev, double* dt_out);
/* (resnorm, res_mass, res_mmnt) = compute_resnorm(res, phase, fluid, dt)
                                                         src/diagnose.jl:57-71 */
int xc_resnorm(xc_ctx* ctx, double dt, double out[3]);
/* FP64 conservation sums of record_history!             src/history.jl:121-145
   out = {sumB, sumM, sumX, sumGx, top_aX, bot_aX, top_aM, bot_aM,
          top_dX, bot_dX, top_dM, bot_dM} */
int xc_conservation_sums(xc_ctx* ctx, double out[12]);
/* Field statistics of record_history!                  src/history.jl:183-222
   out[0..3]   x: min, mean, max, std (corrected)
   out[4..21]  V, vx, vm, xie, xix, xis: min, rms, max each
   out[22..57] Ra, Rc, ReD, Red, ks, ke, kx, eta, etamix, etae, etas, etat:
               min, geomean (exp(mean(log(max(a, eps))))), max each */
int xc_history_stats(xc_ctx* ctx, double out[58]);
/* The field statistics print_step! prints beyond record_history!'s
                                                         src/diagnose.jl:92-182
   (on the raw fields; the reference divides each by a scale first, which
   min, max and geomean commute with):
   out[0..2]   m: min, mean, max
   out[3..23]  rho, V, vx, vm, xie, xix, xis: min, geomean, max each, with
               geomean = exp(sum(log(max(a, 1e-300))) / length(a)) (diagnose.jl:10) */
int xc_print_step_stats(xc_ctx* ctx, double out[24]);
/* Fresh-start initialize! (src/run.jl:71-140) with the initial crystal
   fraction x (host (Nz,Nx)) in place of the MersenneTwister perturbation
   (run.jl:98-108) and the first white-noise draw re/rs. */
int xc_initialize(xc_ctx* ctx, const double* x_init, const double* re, const double* rs);
/* One outer time step of run! (src/run.jl:204-274) with a fixed number of
   Picard sweeps: time_coefs, store_previous!, store_noise!, `sweeps`
   (1..XC_MAX_SWEEPS) sweeps of phsevo! -> fluidmech! -> noise! ->
   update_phase_velocities! -> update! -> compute_resnorm, then update_dt.  This
   is the reference's loop with maxit = sweeps >= 3 and rtol = atol = 0.
   re/rs are the step's white-noise draw (host arrays, or NULL to keep the
   device ones).  stats may be NULL.
   Status: XC_NAN (and the step abandoned after that sweep, as report_iter
   raises, diagnose.jl:80) when a sweep's residual norm is NaN; otherwise the
   whole step is done and XC_NOT_CONVERGED is returned when any Stokes solve
   of it stopped at its iteration cap above its rtol (the reference's direct
   solve has no such case), XC_OK when every solve converged. */
int xc_step(xc_ctx* ctx, int step, double dt, int sweeps, const double* re, const double* rs,
            const xc_solver_opts* opts, xc_step_stats* stats);
/* The same step with run!'s own Picard loop (src/run.jl:220-250): at least 3
   sweeps, then further sweeps while resnorm / resnorm0 >= rtol, resnorm >=
   atol and fewer than maxit sweeps were run; resnorm0 is the first sweep's
   norm and is raised whenever a sweep's norm exceeds it (both + 1e-32).  The
   reference's defaults are rtol 1e-4, atol 1e-9, maxit 15
   (src/parameters.jl:76-78); maxit is capped at XC_MAX_SWEEPS.  Statuses as
   for xc_step; stats->picard_converged tells whether the loop met its
   tolerances. */
int xc_step_converge(xc_ctx* ctx, int step, double dt, double rtol, double atol, int maxit,
                     const double* re, const double* rs, const xc_solver_opts* opts,
                     xc_step_stats* stats);

/* ------------------------------------------------------------------ */
/* ensembles: independent contexts advanced together                   */
/* ------------------------------------------------------------------ */

/* The loop of run! (src/run.jl:204-275) over many independent instances at
   once (uneven grid sizes, parameters and noise seeds; no reference
   counterpart beyond that loop).  Each explicit stage of a Picard sweep is one
   CUDA graph launch for the whole ensemble -- store_previous! /
   store_noise! / snapshot! / phsevo!; noise!; update_phase_velocities! /
   update! / compute_resnorm's reductions; update_dt's reductions -- the
   graph holding every member's kernels of that stage as parallel branches,
   while the members' Stokes solves run concurrently on `threads` host
   threads (0: one per member).  Members must be distinct contexts on one
   device and must not be used elsewhere during a step, and the ensemble must
   be destroyed before them. */
typedef struct xc_ensemble xc_ensemble;
int xc_ensemble_create(xc_ctx* const* members, int n, int threads, xc_ensemble** out);
int xc_ensemble_destroy(xc_ensemble* ens);
/* One time step of every member: xc_step(members[i], steps[i], dts[i],
   sweeps, re[i], rs[i], opts, &stats[i]) for all i, with the same kernels,
   arguments and order per member, so each member ends bit-identical to that
   call.  re / rs (arrays of n host pointers, or NULL; an entry may be NULL)
   are the members' white-noise draws; stats (n entries) may be NULL.
   Status: XC_NAN when a sweep's residual norm is NaN in any member (the
   ensemble step stops after that sweep), the first member's error otherwise,
   XC_NOT_CONVERGED when the step was completed but some member's Stokes
   solve stopped at its iteration cap. */
int xc_ensemble_step(xc_ensemble* ens, const int* steps, const double* dts, int sweeps,
                     const double* const* re, const double* const* rs, const xc_solver_opts* opts,
                     xc_step_stats* stats);

/* ------------------------------------------------------------------ */
/* stencil-level entry points on caller device pointers                */
/* (sizes exactly as the reference's; stream = cudaStream_t or NULL)   */
/* ------------------------------------------------------------------ */

/* fill_ghosts!(f, halo; zBC, xBC), f is (Nz+2halo, Nx+2halo)   src/kernels/ghosts.jl:18-51 */
int xc_fill_ghosts(double* f, int Nz, int Nx, int halo, int zBC, int xBC, void* stream);
/* advect!(adv, f_halo, u, w, h, scheme)                          src/kernels/advect.jl:374-425
   f_halo (Nz+2g, Nx+2g); u (Nz, Nx+1) or (Nz, Nx+3) for tvdim; w (Nz+1, Nx) or (Nz+3, Nx) */
int xc_advect(double* adv, const double* f_halo, const double* u, const double* w,
              int Nz, int Nx, double h, int scheme, void* stream);
/* advect_with_flux!(adv, qx, qz, f_halo, u, w, h, scheme; xBC, zBC)
   qx (Nz+2, Nx+1), qz (Nz+1, Nx+2)                                src/kernels/advect.jl:717-798 */
int xc_advect_with_flux(double* adv, double* qx, double* qz, const double* f_halo,
                        const double* u, const double* w, int Nz, int Nx, double h,
                        int scheme, int xBC, int zBC, void* stream);
/* advect_centered_with_flux!(adv, qx, qz, f, u, w, h, scheme; xBC, zBC):
   f (Nz, Nx) without halo; ghost fill fused into the tile load  src/phsevo.jl:90-128 */
int xc_advect_centered_with_flux(double* adv, double* qx, double* qz, const double* f,
                                 const double* u, const double* w, int Nz, int Nx, double h,
                                 int scheme, int xBC, int zBC, void* stream);
/* diffus!(dff, f_halo, k_halo, h; halo=1)                        src/kernels/diffus.jl:109-121 */
int xc_diffus(double* dff, const double* f_halo, const double* k_halo, int Nz, int Nx,
              double h, void* stream);
/* diffus_with_flux!(dff, qx, qz, f_halo, k_halo, h; halo=1, xBC, zBC)
                                                                 src/kernels/diffus.jl:169-211 */
int xc_diffus_with_flux(double* dff, double* qx, double* qz, const double* f_halo,
                        const double* k_halo, int Nz, int Nx, double h, int xBC, int zBC,
                        void* stream);

/* The CFL step of xc_update_dt for callers that cannot let a library allocate
   device memory (no counterpart in the reference).  A process whose device
   memory is owned by its own pool -- a Julia session using CUDA.jl, or a
   framework with a caching allocator -- cannot have a library call cudaMalloc
   behind its back, and cudaMalloc / cudaFree would also synchronise the whole
   device inside its time-step loop.  This call allocates nothing: kx (Nz,Nx),
   Wx, Wm (Nz+1,Nx+2), Ux, Um (Nz+2,Nx+1) are the caller's device arrays and
   dt_out is one caller-owned double in device memory; block partials live in
   a fixed 80 KiB static device array that every device loading the library
   holds until exit.  Limit: at most 2048 * 4096 = 8,388,608 elements per
   array (about 2894 x 2894 cells); larger grids return XC_BAD_ARG.  The first
   call on each device looks up the array's device address
   (cudaGetSymbolAddress) and keeps it, so make that first call before any
   stream capture; the kept address dies with the device's primary context,
   so do not call this again after a cudaDeviceReset (or a release of the
   primary context) in the same process.  All calls share the array: calls
   that overlap on the GPU race and must not be issued.  Nothing carries over
   between calls.  Maxima and the final min / max follow Julia (a NaN input
   gives a NaN step), as xc_update_dt does.  Stream-ordered on `stream`; no
   host synchronisation. */
int xc_update_dt_noalloc(const double* kx, const double* Wx, const double* Wm, const double* Ux,
                         const double* Um, int Nz, int Nx, double h, double CFL, double dtmax,
                         double dt_prev, double* dt_out, void* stream);

/* time_coefs(Float64, TINT, step) -> (a1, a2, a3, b1, b2, b3)    src/timing.jl:18-36 */
int xc_time_coefs(int tint, int step, double out[6]);

/* ------------------------------------------------------------------ */
/* learned preconditioner network (no counterpart in the reference)    */
/* ------------------------------------------------------------------ */
/* One 3x3 convolution of the preconditioner's U-Net on the tensor cores,
   on caller device pointers: y = relu?(conv3x3(x, w) + bias), BF16 operands,
   FP32 accumulation, zero padding.  x: NHWC BF16 [B][H][W][Cin]; w: BF16
   [Cout][9][Cin] (tap 3 (dy + 1) + (dx + 1)); bias: FP32 [Cout] or NULL;
   y: NHWC BF16 [B][H][W][Cout] and/or y_f32 FP32 (either may be NULL).
   Cin, Cout in {16, 32, 64, 128}; W a multiple of 128, or a power of two
   below 128 with H a multiple of 128 / W; pointers 16-byte aligned.
   Synchronises the stream; XC_TIMEOUT if a bounded wait in the kernel ran
   out. */
int xc_nn_conv3x3(const void* x, const void* w, const float* bias, void* y, float* y_f32, int B, int H, int W,
                  int Cin, int Cout, int relu, void* stream);
/* Its weight gradient: dw (FP32 [Cout][9][Cin]) = sum over pixels p of
   dy[p][co] * x[p + off(tap)][ci] (zero outside the image).  Same shapes and
   rules; synchronises the stream. */
int xc_nn_conv3x3_wgrad(const void* x, const void* dy, float* dw, int B, int H, int W, int Cin, int Cout,
                        void* stream);

/* The U-Net: 4 levels (16, 32, 64, 128 channels), two 3x3 convolutions with
   ReLU per level on the way down, 2x2 average pooling, nearest upsampling of
   a 3x3 convolution plus an additive skip and one 3x3 convolution with ReLU
   per level on the way up, a final 3x3 convolution to FP32.  Inputs and
   outputs are FP32 NHWC arrays [batch][H][W][in_ch] / [..][out_ch] on the
   device; H, W multiples of 8 whose four levels tile into 128-pixel tiles
   (e.g. 256, 512, 1024, 2048).  Weights start He-normal from `seed`. */
typedef struct xc_nn xc_nn;
int xc_nn_create(int H, int W, int batch, int in_ch, int out_ch, unsigned long long seed, xc_nn** out);
int xc_nn_destroy(xc_nn* net);
/* FP32 parameter count of the flat block [w_0 b_0 w_1 b_1 ...] (weights
   [Cout][9][Cin] per layer, each block 16-byte aligned) */
long long xc_nn_param_count(const xc_nn* net);
/* per layer: weight and bias offsets into the block, and (Cin, Cout, level,
   relu); 15 layers */
int xc_nn_layout(const xc_nn* net, long long woff[15], long long boff[15], int spec[60]);
int xc_nn_get_params(xc_nn* net, float* host);
int xc_nn_set_params(xc_nn* net, const float* host);
int xc_nn_get_grads(xc_nn* net, float* host);
/* out = net(in); synchronises the stream (NULL = the network's own) */
int xc_nn_forward(xc_nn* net, const float* in, float* out, void* stream);
/* loss = mean over pixels of sum over out_ch of (net(in) - target)^2 and its
   parameter gradient (xc_nn_get_grads); synchronises */
int xc_nn_loss_grad(xc_nn* net, const float* in, const float* target, float* loss, void* stream);
/* xc_nn_loss_grad followed by one Adam step (beta 0.9, 0.999) at rate lr */
int xc_nn_train_step(xc_nn* net, const float* in, const float* target, float lr, float* loss, void* stream);

/* The learned preconditioner of a context's mixed Stokes solver (no
   counterpart in the reference; it replaces, with the multigrid, the LU of
   fluidmech.jl:512-523): a network of this context's grid size (Nz, Nx
   tiling as xc_nn_create requires; in 4 channels, out 3) with the given
   FP32 parameter block of xc_nn_param_count values (trained at any grid size:
   the weights do not depend on it).  params = NULL removes it.  Selected per
   solve by xc_solver_opts.learned. */
int xc_set_learned_preconditioner(xc_ctx* ctx, const float* params, long long nparams);
/* One training pair from the context's last FP64 fluidmech operator: v is a
   device FP32 vector of the scaled saddle system (length NW + NU + NP, the
   layout of W, U, P one after the other, column-major).  The right-hand side
   r is v itself, or with after_vcycle = 1 the residual v - S LL S M(v) that
   one FP64 V-cycle M of the multigrid preconditioner leaves; the plain FP64
   solver (FGMRES with the multigrid preconditioner, from zero, to rtol, at
   most maxit iterations) solves S LL S z = r; in = the network input
   [Nz][Nx][4] of r (at unit norm) and the viscosity, target = z on the
   interior unknowns [Nz][Nx][3] (device FP32).  Synchronises;
   XC_NOT_CONVERGED when the solve missed rtol. */
int xc_learned_sample(xc_ctx* ctx, const float* v, int after_vcycle, float* in, float* target, double rtol,
                      int maxit, int* iterations);
/* y = S LL S v with the context's last fluidmech operator (device FP32
   vectors, applied in FP64); synchronises. */
int xc_stokes_apply_scaled(xc_ctx* ctx, const float* v, float* y);

/* ------------------------------------------------------------------ */
/* instrumentation (no counterpart in the reference)                   */
/* ------------------------------------------------------------------ */
/* The context's CUDA stream (cudaStream_t), for events recorded by a caller. */
void* xc_stream(xc_ctx* ctx);
/* Kernels launched by this library since load (host-side count). */
long long xc_launch_count(void);
/* Time one kernel of the path on the context's current state with CUDA
   events on the context stream: `iters` back-to-back launches after one
   warm-up launch (kernel 1: each launch timed alone after a 256 MiB write
   that evicts L2; kernels 2, 3: back to back over copies of the operands that
   together exceed twice the L2).  which: 0 WENO5/QUICK advect-with-flux of X (phsevo!),
   1 FP64 Stokes operator apply, 2 FP32 velocity Jacobi sweep (finest level,
   one row per thread as the mixed solver runs it), 3 FP64 velocity Jacobi
   sweep, 4 FFT line filter (z pass of psie), 5 the FP32 sweep with four rows
   per thread (row_block_sweep).
   out = {ms per launch, algorithmic bytes per
   launch, algorithmic flops per launch, units per launch}.  Kernels 1-3 need
   a previous xc_fluidmech call (2 needs the mixed solver). */
int xc_bench_kernel(xc_ctx* ctx, int which, int iters, double out[4]);

/* Last error message of the calling thread ("" when none). */
const char* xc_last_error(void);
/* Library version string. */
const char* xc_version(void);

#ifdef __cplusplus
}
#endif
#endif /* XCORE_GB300_H */
