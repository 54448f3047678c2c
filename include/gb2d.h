/*
 * gb2d.h — C ABI of the GB300 (sm_103a) level-set / ghost-fluid projection path.
 *
 * Drop-in target: the calls EULERIAN_FLUID_SOLVER_2D makes into its advection,
 * reinitialisation and projection members (reference ByungJoonLee/2D_Engine):
 *   Levelset_Advection(dt, tid)        EULERIAN_FLUID_SOLVER_2D.h:1896-2045
 *   Reinitialization(dt, tid)          EULERIAN_FLUID_SOLVER_2D.h:2402-2445
 *   Velocity_Advection(dt, tid)        EULERIAN_FLUID_SOLVER_2D.h:1886-1889
 *   Projection(dt, tid)                EULERIAN_FLUID_SOLVER_2D.h:2359-2363
 *   level-set/reinit TVD-RK3 blocks    EULERIAN_FLUID_SOLVER_2D.h:1694-1741
 *   SolveForRK(dt, tid), its gravity /   EULERIAN_FLUID_SOLVER_2D.h:1857-1879, 3249-3268,
 *   sourcing / wall stages, velocity RK3     2082-2097, 2227-2263, 1753-1794
 *   AdvanceOneTimeStepThread (order 3)    EULERIAN_FLUID_SOLVER_2D.h:1140, 1694-1794
 *   CFLOneTimeStep, AdvanceOneFrame       EULERIAN_FLUID_SOLVER_2D.h:3517-3637, SIMULATION_WORLD.h:1094-1146
 *   LEVELSET_2D::ComputeCurvaturesThread  LEVELSET_2D.h:898-990
 *   POISSON_SOLVER::Solve + PCG_METHOD    POISSON_SOLVER.cpp:127-145, PCG_METHOD.cpp:176-264
 * Plain pointers and sizes only.  Every call returns a status (GB2D_OK = 0,
 * negative on error); gb2d_last_error() gives the message.  A context owns one
 * CUDA stream and its device buffers; it is not re-entrant (one host thread
 * at a time), matching how the reference runs these on its head thread.
 *
 * Host arrays use the reference's ghost-inclusive ARRAY_2D layout
 * (ARRAY_2D.h:140-146): row-major, i fastest, element (i, j) of a field with
 * ghost width g and interior width nI at [(i+g) + (j+g)*(nI+2g)], i.e. the
 * FIELD_STRUCTURE_2D::array_for_this.values pointer can be passed as is.
 */
#ifndef GB2D_H
#define GB2D_H

#ifdef __cplusplus
extern "C" {
#endif

#define GB2D_OK 0
#define GB2D_ERR_ARG (-1)          /* invalid argument or size */
#define GB2D_ERR_CUDA (-2)         /* CUDA runtime error (message names it) */
#define GB2D_ERR_NONFINITE (-3)    /* NaN/Inf met in a reduction */
#define GB2D_ERR_MAX_ITERS (-4)    /* solver stopped at its iteration cap above tolerance */
#define GB2D_ERR_ZERO_GRADIENT (-5)/* curvature denominator zero (reference exits: LEVELSET_2D.h:869-873) */
#define GB2D_ERR_NO_DEVICE (-6)
#define GB2D_ERR_TOO_LARGE (-7)    /* size above a fixed maximum (gb2d_poisson_solve_noalloc) */

/* Field identifiers and their ghost widths (EULERIAN_FLUID_SOLVER_2D.h:350-384,
 * PROJECTION_2D.h:207-213, LEVELSET_2D.h:64-79). */
#define GB2D_FIELD_PHI 0   /* level set, nodes ni x nj, ghost 2 */
#define GB2D_FIELD_U 1     /* x-face velocity (ni+1) x nj, ghost 2 */
#define GB2D_FIELD_V 2     /* y-face velocity ni x (nj+1), ghost 2 */
#define GB2D_FIELD_UA 3    /* advecting x-velocity copy (ghost 3): velocity_field_mac_ghost_x */
#define GB2D_FIELD_VA 4    /* advecting y-velocity copy (ghost 3): velocity_field_mac_ghost_y */
#define GB2D_FIELD_P 5     /* pressure, ghost 1 */
#define GB2D_FIELD_KAPPA 6 /* curvature, no ghost */
#define GB2D_FIELD_DENSITY 7 /* node density of DetermineDensity (EULERIAN_FLUID_SOLVER_2D.h:81,379), ghost 2 */

#define GB2D_PRECISION_FP64 0  /* FP64 everywhere: reproduces the reference's FP64 results */
#define GB2D_PRECISION_MIXED 1 /* FP32 where it only affects speed, FP64 where it sets the result (see gb2d_solve_opts) */

#define GB2D_SOLVER_MGPCG 0       /* multigrid-preconditioned CG */
#define GB2D_SOLVER_PCG_JACOBI 1  /* diagonal-preconditioned CG (simple FP64 parity solver) */

typedef struct gb2d_ctx gb2d_ctx;

/* Node grid as GRID_STRUCTURE_2D (GRID_STRUCTURE_2D.h:88-123): dx = (x_max-x_min)/(ni-1). */
typedef struct {
  int ni, nj;
  double x_min, y_min, x_max, y_max;
} gb2d_grid;

/* Physical and scheme constants read by the reference from its .sim script
 * (EULERIAN_FLUID_SOLVER_2D.h:170-262, ADVECTION_2D.cpp:4-18). */
typedef struct {
  double water_density;    /* phi > 0 (air_bubble_rising) */
  double air_density;      /* phi <= 0 */
  double surface_tension;  /* jump jc = sigma * kappa */
  double weno_epsilon;     /* WENO weight epsilon (1e-6) */
  int reinit_iterations;   /* iteration_number_for_reinitialization */
  int reinit_scaling;      /* scaling_number_for_reinitialization: dtau = dx/scaling */
  int advection_precision; /* explicit stencils (WENO5 advection, reinitialisation, ENO3 velocity advection,
                              viscosity): GB2D_PRECISION_FP64 reproduces the reference's FP64 results;
                              MIXED evaluates their fluxes in FP32 from FP64 differences, state and
                              updates FP64 */
} gb2d_params;

/* Constants of the stages SolveForRK runs around the projection (gravity, viscosity;
 * EULERIAN_FLUID_SOLVER_2D.h:180-194, 246).  A new context starts with the script
 * defaults: water_viscosity 1, air_viscosity 0, gravity (0, -9.8), cfl_number 0.5,
 * viscosity 0. */
typedef struct {
  double water_viscosity;  /* phi > 0 */
  double air_viscosity;    /* phi <= 0 */
  double gravity_x, gravity_y;
  double cfl_number;       /* CFLOneTimeStep's dt = cfl_number / CFL (script default 0.5) */
  int viscosity;           /* 1: explicit delta-function viscosity (VISCOSITY_2D::ApplyViscosity,
                              VISCOSITY_2D.h:460-532).  0: none, which is what the reference runs for
                              air/water even with is_viscosity_active: it never configures that
                              solver for air/water (only the oil/water branch calls its
                              InitializeFromScriptBlock, EULERIAN_FLUID_SOLVER_2D.h:645-669), so its
                              use_delta_function_formulation stays off and ApplyViscosity does nothing */
} gb2d_flow_params;

/* Pressure-solve options (replace PROJECTION block's tolerance/max_iteration/
 * poisson_solver_type, PROJECTION_2D.h:132-160). */
typedef struct {
  int solver;           /* GB2D_SOLVER_* */
  int precision;        /* GB2D_PRECISION_*: the CG (x, r, p, A p) is FP64 either way; MIXED runs the
                           preconditioner (V-cycle or Jacobi) in FP32 */
  double tolerance;     /* stop at ||b - A p||_2 / ||b||_2 <= tolerance */
  int max_iterations;   /* cap on Krylov iterations (all restarts together) */
  int mg_smooth;        /* red-black Gauss-Seidel sweeps before and after each coarse correction (0 = 2) */
} gb2d_solve_opts;

typedef struct {
  int iterations;        /* Krylov iterations done */
  int outer_iterations;  /* CG starts: 1, or more if the true residual had drifted above the tolerance */
  double rel_residual;   /* final FP64 ||b - A p|| / ||b|| */
  double max_velocity_x; /* max |u| after the update (PROJECTION_2D::max_velocity_x) */
  double max_velocity_y;
} gb2d_solve_stats;

/* Context lifetime.  Allocates every device buffer up front (no allocation in later calls). */
int gb2d_create(const gb2d_grid* grid, const gb2d_params* params, gb2d_ctx** out);
int gb2d_destroy(gb2d_ctx* ctx);
const char* gb2d_last_error(const gb2d_ctx* ctx);
/* Ghost-inclusive host extents of a field: *ires x *jres doubles. */
int gb2d_field_extent(const gb2d_grid* grid, int field, int* ires, int* jres);

/* Host <-> device state transfer of one ghost-inclusive field (blocking). */
int gb2d_set_field(gb2d_ctx* ctx, int field, const double* host);
int gb2d_get_field(gb2d_ctx* ctx, int field, double* host);
/* Device address of a whole field (for callers that keep their own device state).
 * PHI, and U / V after a viscosity pass, are double-buffered: the address is valid
 * until the next call that advances the state. */
int gb2d_field_device_ptr(gb2d_ctx* ctx, int field, double** dptr);
int gb2d_synchronize(gb2d_ctx* ctx);
/* Run the context's work on a caller-owned CUDA stream (a cudaStream_t passed as
 * void*); NULL returns to the context's own stream. */
int gb2d_set_stream(gb2d_ctx* ctx, void* stream);
/* Tile shape of the pressure solver's tiled smoothing levels (a tuning knob; no
 * counterpart in the reference): plan < 0 the per-level rule, 0-3 one shape for every
 * tiled level (64x16, 32x16, 32x8, 32x32 cells).  Different plans sum the preconditioner's
 * dot products in different orders, so their results differ by rounding. */
int gb2d_set_tile_plan(gb2d_ctx* ctx, int plan);

/* Kernel probe for roofline measurement: while enabled, the pressure solver
 * brackets every launch of its finest-level smoother (one launch = every red-black
 * sweep of one side of the V-cycle) with CUDA events on the context stream.  gb2d_probe_read returns the launches
 * seen, their summed event time and the algorithmic bytes of one launch
 * (every array the half sweep must read or write, once). */
int gb2d_probe_enable(gb2d_ctx* ctx, int enable);
int gb2d_probe_read(gb2d_ctx* ctx, int* launches, double* total_ms, double* bytes_per_launch);
/* Kernels this library has launched in this process so far (all contexts). */
int gb2d_kernel_launches(unsigned long long* count);
/* Arithmetic peaks of the current device in TFLOP/s (2 flops per FMA), measured by
 * timing independent FMA chains on every SM (about 0.1 s in total on a GB300): the
 * denominators of the ALU roofline of the WENO5 and reinitialisation sweeps.
 * GB2D_ERR_CUDA if a launch fails, GB2D_ERR_NO_DEVICE without a device. */
int gb2d_alu_peaks(double* fp64_tflops, double* fp32_tflops);

/* Self-check of the exact FP64 division by 3 and 6 used in the WENO5 kernels
 * (three FP64 operations instead of a division): compares it bit for bit with
 * the IEEE division on 2 n pseudo-random inputs (every exponent, NaN and
 * infinity included) and stores the number of differing results.  No
 * counterpart in the reference (diagnostics). */
int gb2d_check_exact_division(unsigned long long n, unsigned long long seed, unsigned long long* mismatches);

/* Multigrid layout of the pressure solver for one precision (GB2D_PRECISION_FP64
 * or GB2D_PRECISION_MIXED, whose V-cycles run in FP32): the number of levels, the
 * first level handled by the thread-block-cluster tail kernel (-1 when the
 * single-CTA tail is used instead) and that cluster's CTA count.  No counterpart
 * in the reference (diagnostics). */
int gb2d_solver_layout(gb2d_ctx* ctx, int precision, int* levels, int* cluster_top, int* cluster_ctas);

/* One multigrid V-cycle of the pressure solver's preconditioner, z = M r, for the
 * system last assembled on this context (gb2d_poisson_assemble or a projection):
 * precision GB2D_PRECISION_FP64 or GB2D_PRECISION_MIXED (FP32 levels, r narrowed
 * to FP32 as the solver does), mg_smooth red-black sweeps per side (0 = 2).  r, z:
 * host ni x nj, row-major, no ghosts.  No counterpart in the reference
 * (diagnostics: the smoothing kernels are compared through it). */
int gb2d_preconditioner_apply(gb2d_ctx* ctx, int precision, int mg_smooth, const double* r, double* z);

/* Device-resident checkpoint of the step state (PHI with its ghosts, U, V, UA,
 * VA, P): save copies it to a second set of device buffers (allocated on the
 * first save), restore copies it back.  Asynchronous on the context stream. */
int gb2d_checkpoint_save(gb2d_ctx* ctx);
int gb2d_checkpoint_restore(gb2d_ctx* ctx);

/* One Levelset_Advection: WENO5 sweep with the advecting copies UA/VA, then phi's
 * ghost extrapolation (a1, a5, a7). */
int gb2d_levelset_advection(gb2d_ctx* ctx, double dt);
/* One Reinitialization: S = phi/sqrt(phi^2+dx^2), reinit_iterations WENO5-Godunov sweeps (a2, a6). */
int gb2d_reinitialization(gb2d_ctx* ctx);
/* LEVELSET_2D::FastSweepingMethodOriginal(sweeps) (LEVELSET_2D.h:281-384), the
 * reinitialisation of scripts with fastsweeping_reinitialization (EULERIAN_FLUID_SOLVER_2D.h:2404-2408,
 * called there with 4): nodes with |phi| < 2 dx stay fixed, the others take sweeps
 * Gauss-Seidel sweeps of Zhao's upwind distance update (directions ++, -+, --, +- in turn),
 * with phi's ghosts extrapolated before and after. */
int gb2d_fast_sweeping(gb2d_ctx* ctx, int sweeps);
/* Level-set TVD-RK3 followed by reinit TVD-RK3, as one step of the reference (a4). */
int gb2d_levelset_rk3(gb2d_ctx* ctx, double dt);
/* One Velocity_Advection: refresh UA/VA from U/V, ENO3 on both MAC components (a3). */
int gb2d_velocity_advection(gb2d_ctx* ctx, double dt);
/* ComputeCurvaturesThread: extrapolate phi's ghosts, write KAPPA (a8). */
int gb2d_curvature(gb2d_ctx* ctx);
/* One PROJECTION_2D::Solve(dt): density, divergence, sigma*kappa jump, matrix-free
 * ghost-fluid Poisson system, solve (P is the warm start), GFM velocity update (a9-a14). */
int gb2d_projection(gb2d_ctx* ctx, double dt, const gb2d_solve_opts* opts, gb2d_solve_stats* stats);
/* gb2d_projection on a state held in host memory: copies PHI, U, V and the warm-start P
 * in, projects, and copies P, U, V out, in the ghost-inclusive layouts of gb2d_set_field
 * (a null input keeps the context's field, a null output is not copied).  One call
 * instead of seven: U, V and P stream in on a copy stream while the curvature, face
 * weights and diagonal compute from PHI, and P streams out while the velocity update
 * runs.  Page-locked host buffers let the copies overlap; pageable ones work too.
 * Returns when the outputs are in place, with gb2d_projection's status. */
int gb2d_projection_host(gb2d_ctx* ctx, double dt, const gb2d_solve_opts* opts, const double* phi, const double* u,
                         const double* v, const double* p, double* p_out, double* u_out, double* v_out,
                         gb2d_solve_stats* stats);

/* Flow constants for the stages below (see gb2d_flow_params). */
int gb2d_set_flow_params(gb2d_ctx* ctx, const gb2d_flow_params* flow);
/* ApplyGraivity (EULERIAN_FLUID_SOLVER_2D.h:3249-3268): every U and V face, walls
 * included, gains dt * gravity. */
int gb2d_apply_gravity(gb2d_ctx* ctx, double dt);
/* Sourcing (:2082-2097): DetermineDensity (:2162-2180) into DENSITY, then the
 * explicit viscosity if gb2d_flow_params.viscosity is set. */
int gb2d_sourcing(gb2d_ctx* ctx, double dt);
/* SetupBoundaryConditionForVelocity (:2227-2263): zero normal velocity on the walls. */
int gb2d_velocity_boundary(gb2d_ctx* ctx);
/* SolveForRK (:1857-1879): Velocity_Advection, gravity, sourcing and wall
 * conditions (one fused pass), Projection. */
int gb2d_solve_for_rk(gb2d_ctx* ctx, double dt, const gb2d_solve_opts* opts, gb2d_solve_stats* stats);
/* AdvanceOneTimeStepThread with order_for_time_advancing = 3 (:1694-1794): level-set
 * and reinitialisation TVD-RK3, then the velocity TVD-RK3 over three SolveForRK
 * stages.  stats: iterations and outer_iterations summed over the three
 * projections, rel_residual the largest, the velocity maxima the last.  A stage
 * that stops at the iteration cap does not end the step; the call then returns
 * GB2D_ERR_MAX_ITERS after the step. */
int gb2d_advance_time_step(gb2d_ctx* ctx, double dt, const gb2d_solve_opts* opts, gb2d_solve_stats* stats);

/* CFLOneTimeStep (EULERIAN_FLUID_SOLVER_2D.h:3517-3637) from U, V and KAPPA as they
 * stand (run gb2d_curvature first, as SIMULATION_WORLD::AdvanceOneFrame does):
 * cfl_number / CFL, or 0 where CFL is 0.  rates (may be NULL) receives the
 * advection, gravity, viscosity and surface-tension rates c_f, g_f, v_f, s_f. */
int gb2d_cfl_time_step(gb2d_ctx* ctx, double* dt, double* rates);
/* SIMULATION_WORLD::AdvanceOneFrame (SIMULATION_WORLD.h:1094-1146, 1194-1207):
 * curvature, dt = CFLOneTimeStep() * cfl (the previous dt in place of a zero
 * CFLOneTimeStep), then gb2d_advance_time_step(dt).  *dt: the previous time step
 * in, the step taken out. */
int gb2d_advance_frame(gb2d_ctx* ctx, double cfl, double* dt, const gb2d_solve_opts* opts, gb2d_solve_stats* stats);

/* Adjoints (vector-Jacobian products) for gradients of a scalar loss L; no counterpart in
 * the reference, which has no derivative code.  Host arrays in the field layouts; FP64.
 *
 * gb2d_weno5_adjoint: one gb2d_levelset_advection (WENO5 sweep, its ghost copy and the
 * ghost extrapolation) linearised at the current PHI, UA, VA, i.e. at the step's input.
 * lam_phi = dL/dphi' of the step's output (PHI layout); writes mu_phi = dL/dphi (PHI
 * layout) and, if non-NULL, mu_ua / mu_va = dL/dUA, dL/dVA (UA / VA layouts).  The WENO5
 * weights are differentiated; the upwind switch on the sign of the face-averaged
 * velocity is held at its current side.  Allocates about 16 doubles per node on the
 * first call. */
int gb2d_weno5_adjoint(gb2d_ctx* ctx, double dt, const double* lam_phi, double* mu_phi, double* mu_ua, double* mu_va);
/* gb2d_projection_adjoint: the last gb2d_projection, linearised at its level set and
 * assembled system (PHI unchanged since), with respect to its intermediate velocity.
 * lam_u, lam_v = dL/dU', dL/dV' of the projected velocity, lam_p = dL/dp (P layout, may be
 * NULL); writes mu_u, mu_v = dL/dU*, dL/dV*.  Applies the transposed pressure gradient,
 * solves the same symmetric system with opts, applies the transposed divergence. */
int gb2d_projection_adjoint(gb2d_ctx* ctx, double dt, const double* lam_u, const double* lam_v, const double* lam_p, double* mu_u,
                            double* mu_v, const gb2d_solve_opts* opts, gb2d_solve_stats* stats);

/* The same loss's derivatives with respect to the two densities (water_density, air_density
 * of gb2d_params), through the face weights of A, the jump fluxes of the right-hand side and
 * the velocity update's 1/rho: dL/drho = sum lam du'/drho|p + z (db/drho - dA/drho p).  Call
 * right after gb2d_projection_adjoint, which leaves z and the cotangents in the context. */
int gb2d_projection_density_gradient(gb2d_ctx* ctx, double dt, double* d_water_density, double* d_air_density);
/* dL/dphi of the same loss, after gb2d_projection_adjoint and before the state changes: the
 * projection's dependence on the level set through the face weights (the |phi|-weighted
 * harmonic mean of 1/rho in A and in the jump fluxes of b), the jump fluxes' |phi|-weighted
 * interpolation of sigma kappa, the curvature kappa(phi) (zero slope where clamped), and the
 * velocity update's interface faces (|phi|-weighted jump, smeared-Heaviside density); the
 * phases (signs of phi) are piecewise constant.  The ghost extrapolation the projection
 * starts with is reversed, so d_phi (PHI's layout, ghost 2) is the gradient with respect to
 * the PHI the projection was given. */
int gb2d_projection_phi_gradient(gb2d_ctx* ctx, double dt, double* d_phi);
/* VJP of the last gb2d_velocity_advection (the FP64 forms of ENO3; call before UA / VA
 * change): lam_u, lam_v (U, V layouts) are the cotangents of the advected U, V; mu_ua, mu_va
 * (UA, VA layouts, ghost 3) receive the cotangents of the advecting copies that step read
 * (both as advected values and as advecting velocities).  The advected U, V also pass lam_u,
 * lam_v straight through (u' = u - dt (...)), and UA / VA are the ghost-filled copies of U / V
 * (FillGhostCellsFrom): a caller maps mu_ua, mu_va back onto U, V through that copy's transpose. */
int gb2d_velocity_advection_adjoint(gb2d_ctx* ctx, double dt, const double* lam_u, const double* lam_v, double* mu_ua,
                                    double* mu_va);
/* One WENO5-Godunov reinitialisation sweep (the sweep gb2d_reinitialization repeats) of phi_in
 * (PHI's layout) with the given S (ni x nj, S = phi / sqrt(phi^2 + dx^2) of the level set the
 * Reinitialization started from) into phi_out, in the context's advection precision; the
 * context's own PHI is not touched.  With gb2d_reinit_sweep_adjoint, the building block of a
 * differentiable Reinitialization (the sweeps' S is held, and its own derivative is the
 * caller's). */
int gb2d_reinit_sweep_apply(gb2d_ctx* ctx, const double* phi_in, const double* sign, double* phi_out);
/* VJP of that sweep (FP64 form) at phi_in, sign: lam (PHI's layout) -> mu_phi (PHI's layout) and
 * mu_sign (ni x nj, the cotangent of S). */
int gb2d_reinit_sweep_adjoint(gb2d_ctx* ctx, const double* phi_in, const double* sign, const double* lam, double* mu_phi,
                              double* mu_sign);
/* VJP of gb2d_sourcing's explicit viscosity (ApplyViscosity, VISCOSITY_2D.h:460-532; FP64 form)
 * at the context's PHI, U, V (the stage's inputs): lam_u, lam_v (U / V layouts) -> mu_u, mu_v
 * (U / V layouts) and mu_phi (PHI's layout: the smeared viscosities and the face densities
 * depend on the level set, read on the interior and the ghost-1 ring) and, if d_density is not
 * null, d_density[0..1] = dL/d water_density, dL/d air_density (through dt / rho of each face).
 * Uses gb2d_flow_params' viscosities. */
int gb2d_viscosity_adjoint(gb2d_ctx* ctx, double dt, const double* lam_u, const double* lam_v, double* mu_u, double* mu_v,
                           double* mu_phi, double* d_density);

/* Batches: many independent simulations of uneven grid sizes on one GPU (no counterpart
 * in the reference, which runs one simulation per process).  Each instance is a full
 * context with its own stream; host worker threads drive disjoint sets of instances frame
 * by frame so that small grids overlap on the GPU.  Instances are placed on workers
 * longest-first by cost per frame (cells until gb2d_batch_autotune has measured them).
 * Set each instance's fields through gb2d_batch_context; the contexts belong to the batch.
 * workers <= 0 picks min(host threads, 16). */
typedef struct gb2d_batch gb2d_batch;
typedef struct {
  int frames;                /* frames advanced per instance */
  int instances;
  long long cg_iterations;   /* summed over every projection of every instance */
  double max_rel_residual;   /* largest final relative residual of any projection */
  double wall_ms;            /* host wall time of the call (all work finished) */
  double cell_frames_per_s;  /* sum of instance cells x frames / wall time */
} gb2d_batch_stats;
int gb2d_batch_create(int n, const gb2d_grid* grids, const gb2d_params* params, const gb2d_flow_params* flows, int workers,
                      gb2d_batch** out);
int gb2d_batch_destroy(gb2d_batch* batch);
const char* gb2d_batch_last_error(const gb2d_batch* batch);
int gb2d_batch_size(const gb2d_batch* batch, int* n, int* workers);
int gb2d_batch_context(gb2d_batch* batch, int k, gb2d_ctx** ctx);
/* Autotuner: for each distinct grid size, time one frame (gb2d_advance_frame with cfl)
 * with 1, 2 and 3 red-black sweeps per V-cycle side under each of four tile plans (the
 * per-level rule, 32x16, 32x8 and 64x16 tiles on every tiled level) from the instance's
 * current state (restored afterwards), keep the fastest schedule for every instance of that
 * size (sweeps in smooth_out[k], may be NULL; both through gb2d_batch_schedule) and re-place
 * the instances on the workers by the measured times. */
int gb2d_batch_autotune(gb2d_batch* batch, double cfl, const gb2d_solve_opts* opts, int* smooth_out);
/* gb2d_advance_frame for every instance, frames times.  dts[k]: instance k's previous time
 * step in, its last step out.  opts' mg_smooth is replaced per instance by the tuned value. */
int gb2d_batch_advance(gb2d_batch* batch, int frames, double cfl, double* dts, const gb2d_solve_opts* opts, gb2d_batch_stats* stats);
/* The same run as gb2d_batch_advance in one graph launch: every instance is an independent
 * branch of one CUDA graph, a WHILE node over its frames whose body is the instance's frame
 * run on the device (the CFL step formed on the GPU, each CG solve a nested WHILE node), so
 * the host takes part only before and after the run.  The graph is captured on the first
 * call and again when frames, cfl, opts or the tuned schedules change (stats->wall_ms
 * excludes the capture).  The instances' fields and dts equal gb2d_batch_advance's bit for
 * bit (each solve takes at most the host loop's first pass and one restart). */
int gb2d_batch_run_graph(gb2d_batch* batch, int frames, double cfl, double* dts, const gb2d_solve_opts* opts, gb2d_batch_stats* stats);
/* Instance k's tuned schedule: red-black sweeps per V-cycle side and tile plan (-1: the
 * per-level rule; 0-3: one tile shape, 64x16, 32x16, 32x8 or 32x32, for every tiled level). */
int gb2d_batch_schedule(const gb2d_batch* batch, int k, int* sweeps, int* tile_plan);

/* The general jump-condition Poisson problem (a15; POISSON_SOLVER::Solve with density, bc,
 * div, levelset, jc_on_solution, jc_on_derivative, POISSON_SOLVER.cpp:127-145, and its
 * builder :714-976, as POISSON_EQUATION_TEST uses it): on the context's grid, with the
 * coefficient 1/density, boundary codes bc (>= 0 unknown, -1 Dirichlet, -4 Neumann),
 * right-hand side -div, jumps [u] = jc_solution and [beta du/dn] = jc_derivative across
 * levelset = 0 (normals from the level set as LEVELSET_2D::ComputeNormals forms them).
 * density, bc (int), div, jc_solution, jc_derivative, pressure: P layout (ghost 1);
 * levelset: PHI layout (ghost 2).  pressure holds the Dirichlet values and the warm start
 * and receives the solution; normal_x / normal_y (P layout, may be NULL) receive the
 * normals.  Uses the context's system buffers (a later gb2d_projection rebuilds them). */
int gb2d_jump_poisson_solve(gb2d_ctx* ctx, const double* density, const int* bc, const double* div, const double* levelset,
                            const double* jc_solution, const double* jc_derivative, double* pressure, double* normal_x,
                            double* normal_y, const gb2d_solve_opts* opts, gb2d_solve_stats* stats);

/* Standalone pieces of the pressure system for parity checks and for
 * POISSON_SOLVER_2D-style use (a10, a15).  gb2d_poisson_assemble runs the
 * curvature step (which extrapolates phi's ghosts) and builds the system of the
 * current state as PROJECTION_2D would, then copies out face weights bx
 * ((ni+1) x nj), by (ni x (nj+1)), diag and rhs (ni x nj); any output may be NULL. */
int gb2d_poisson_assemble(gb2d_ctx* ctx, double dt, double* bx, double* by, double* diag, double* rhs);
/* y = A x with the assembled operator, summed in the reference CSR row order. */
int gb2d_poisson_apply(gb2d_ctx* ctx, const double* x, double* y);
/* Solve A x = rhs with the assembled operator; x is the warm start (ni x nj). */
int gb2d_poisson_solve(gb2d_ctx* ctx, const double* rhs, double* x, const gb2d_solve_opts* opts, gb2d_solve_stats* stats);

/* Allocation-free solve for callers that cannot allocate device memory: hosts that
 * reserve all GPU memory for their own pool and forbid cudaMalloc/cudaFree after
 * start-up, or that must not allocate inside a frame because allocation can
 * synchronise the device.  No counterpart in the reference (its PCG allocates
 * its vectors on every call, PCG_METHOD.cpp:180-200).
 * FP64 Jacobi-preconditioned CG on an assembled system given as DEVICE pointers
 * in the layout gb2d_poisson_assemble returns (bx (ni+1) x nj, by ni x (nj+1),
 * diag, rhs ni x nj); x is the device warm start and receives the solution.
 * Stops at ||b - A x|| / ||b|| <= tolerance or after max_iterations.  stream is a
 * cudaStream_t as void* (NULL = the default stream); the call returns after the
 * solve has finished on that stream.  Scratch is one file-scope device array of
 * about 2.1 MB that every GPU loading the library keeps until exit; at most
 * GB2D_NOALLOC_MAX_CELLS unknowns, larger sizes return GB2D_ERR_TOO_LARGE.  The
 * first call on a device looks up the array's address with that device current
 * (make it before any stream capture) and keeps it for the process: after a
 * cudaDeviceReset, or from another context on that device, do not call it again.
 * A warm start that already meets the tolerance returns GB2D_OK after zero
 * iterations with x unchanged.  All calls share the array and keep the last
 * call's contents, so calls that overlap on the GPU race. */
#define GB2D_NOALLOC_MAX_CELLS 65536
int gb2d_poisson_solve_noalloc(int ni, int nj, double dx, double dy, const double* bx, const double* by, const double* diag,
                               const double* rhs, double* x, double tolerance, int max_iterations, void* stream, int* iterations,
                               double* rel_residual);

#ifdef __cplusplus
}
#endif
#endif /* GB2D_H */
