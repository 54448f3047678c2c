/*
 * gb2d_oracle — CPU restatement of the reference hot path (ByungJoonLee/2D_Engine).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU path is compared with;
 * it is never the product.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load it.
 *
 * Parity pinning: every function here is checked bit-for-bit (or to the stated
 * tolerance for the iterative solve) against outputs of the reference itself,
 * stored as golden fixtures under tests/golden/ and produced by
 * tests/golden/make_golden.py from the headless reference build in oracle/ref/.
 *
 * Array layout is the reference's ARRAY_2D (ARRAY_2D.h:140-146): row-major,
 * i fastest, ghost cells included, element (i, j) of a field with ghost width g
 * and interior extent nI at [(i + g) + (j + g) * (nI + 2g)].
 *   phi : node grid ni x nj, ghost 2      ((ni+4) x (nj+4))
 *   u   : x-faces (ni+1) x nj, ghost 2     ((ni+5) x (nj+4))
 *   v   : y-faces ni x (nj+1), ghost 2     ((ni+4) x (nj+5))
 *   ua  : advecting x-velocity, ghost 3    ((ni+7) x (nj+6))
 *   va  : advecting y-velocity, ghost 3    ((ni+6) x (nj+7))
 *   p   : pressure, ghost 1                ((ni+2) x (nj+2))
 *   kappa : curvature, no ghost            (ni x nj)
 * All arithmetic is IEEE double with no contraction (build with -ffp-contract=off).
 */
#ifndef GB2D_ORACLE_H
#define GB2D_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int ni, nj;                      /* pressure / level-set nodes */
  double x_min, y_min, x_max, y_max;
} or_grid;

typedef struct {
  double water_density;            /* phi > 0  (air_bubble_rising, PROJECTION_2D.h:350-358) */
  double air_density;              /* phi <= 0 */
  double surface_tension;          /* jc = sigma * kappa (PROJECTION_2D.h:826-833) */
  double weno_epsilon;             /* 1e-6 in the scripts */
  int reinit_iterations;           /* iteration_number_for_reinitialization */
  int reinit_scaling;              /* scaling_number_for_reinitialization: dtau = dx / scaling */
  double pcg_tolerance;            /* stop when r.z < tol^2 (PCG_METHOD.cpp:254) */
  int pcg_max_iterations;
  double pcg_rel_residual;         /* > 0: also stop once ||r||_2 <= this * ||b||_2 (CPU-baseline
                                      timing to a relative residual; the reference has no such test) */
} or_params;

/* Flow constants of SolveForRK's sourcing stages (EULERIAN_FLUID_SOLVER_2D.h:170-262). */
typedef struct {
  double water_viscosity;          /* phi > 0 */
  double air_viscosity;            /* phi <= 0 */
  double gravity_x, gravity_y;     /* ApplyGraivity adds dt * gravity */
  int viscosity;                   /* 1: explicit delta-function viscosity (VISCOSITY_2D.h:460-532);
                                      0: none, which is what the reference's air/water setup runs
                                      (its viscosity solver is never configured) */
} or_flow;

typedef struct {
  int iterations;
  double residual;                 /* sqrt(r.z) at exit, as the reference prints it */
  double max_velocity_x, max_velocity_y;
} or_stats;

/* Status codes (shared meaning with the GPU ABI). */
#define OR_OK 0
#define OR_BAD_ARG (-1)
#define OR_NO_MEMORY (-2)
#define OR_ZERO_GRADIENT (-3)

/* a7 ghost fills. */
void or_fill_ghost_copy(double* dst, int gd, const double* src, int gs, int nI, int nJ, int g);
void or_fill_ghost_extrapolate(double* f, int g, int nI, int nJ);

/* a1+a5: one Levelset_Advection call (WENO5 forward-Euler sweep + ghost extrapolation). */
int or_levelset_advection(const or_grid* gr, const or_params* pr, double* phi, const double* ua, const double* va, double dt);
/* a2+a6: one Reinitialization call (S = phi/sqrt(phi^2+dx^2), then reinit_iterations sweeps). */
int or_reinitialization(const or_grid* gr, const or_params* pr, double* phi);
/* a4: level-set TVD-RK3 then reinit TVD-RK3, as EULERIAN_FLUID_SOLVER_2D.h:1694-1741. */
int or_levelset_rk3(const or_grid* gr, const or_params* pr, double* phi, const double* ua, const double* va, double dt);
/* a3: one Velocity_Advection call (ENO3 on both MAC components; refreshes ua, va first). */
int or_velocity_advection(const or_grid* gr, const or_params* pr, double* u, double* v, double* ua, double* va, double dt);
/* a8: ComputeCurvaturesThread (fills phi's ghosts, writes kappa). */
int or_curvature(const or_grid* gr, double* phi, double* kappa);
/* a9-a14: one PROJECTION_2D::Solve(dt, tid); p is the warm start and the result. */
int or_projection(const or_grid* gr, const or_params* pr, double* phi, double* u, double* v, double* p, double* kappa, double dt, or_stats* st);
/* The same projection as three calls, so that its PCG can run in slices of
 * iterations: begin (curvature, assembly, IC(0) factor, first residual), iterate
 * (at most `count` PCG iterations; returns how many ran, *done = 1 once a stop
 * test holds), finish (remaining iterations, VectorToGrid, velocity update).  The
 * arrays passed to begin must stay valid until finish; free releases the run. */
typedef struct or_projection_run or_projection_run;
int or_projection_begin(const or_grid* gr, const or_params* pr, double* phi, double* u, double* v, double* p, double* kappa, double dt,
                        or_projection_run** run);
int or_projection_iterate(or_projection_run* run, int count, int* done);
int or_projection_finish(or_projection_run* run, or_stats* st);
void or_projection_free(or_projection_run* run);

/* Rest of SolveForRK (EULERIAN_FLUID_SOLVER_2D.h:1857-1879). */
int or_apply_gravity(const or_grid* gr, const or_flow* fl, double* u, double* v, double dt);
/* DetermineDensity into density (ghost 2; may be null), then the viscosity if fl->viscosity. */
int or_sourcing(const or_grid* gr, const or_params* pr, const or_flow* fl, const double* phi, double* u, double* v, double* density, double dt);
void or_velocity_bc(const or_grid* gr, double* u, double* v);
int or_solve_for_rk(const or_grid* gr, const or_params* pr, const or_flow* fl, double* phi, double* u, double* v, double* ua,
                    double* va, double* p, double* kappa, double* density, double dt, or_stats* st);
/* AdvanceOneTimeStepThread, order 3 (EULERIAN_FLUID_SOLVER_2D.h:1694-1794). */
int or_time_step(const or_grid* gr, const or_params* pr, const or_flow* fl, double* phi, double* u, double* v, double* ua,
                 double* va, double* p, double* kappa, double* density, double dt, or_stats* st);

/* CFLOneTimeStep (EULERIAN_FLUID_SOLVER_2D.h:3517-3637) with kappa from or_curvature;
 * rates (may be null) receives c_f, g_f, v_f, s_f. */
double or_cfl_time_step(const or_grid* gr, const or_params* pr, const or_flow* fl, const double* u, const double* v,
                        const double* kappa, double cfl_number, double rates[4]);

/* General jump-condition Poisson problem (POISSON_SOLVER::Solve with density, bc, div,
 * levelset, jc_on_solution, jc_on_derivative; POISSON_SOLVER.cpp:127-145, 714-976).
 * or_normals: LEVELSET_2D::ComputeNormals(thread_id) (copy-fills phi's ghosts, writes unit
 * normals nx, ny on the nodes; ghost 1).  or_jump_poisson_assemble: the system in the grid
 * layout, full cells (bc >= 0) as the builder writes them, every other node an identity
 * row scaled by 1/dx^2 holding its pressure; bc codes: >= 0 full, -1 Dirichlet, -4 Neumann. */
void or_normals(const or_grid* gr, double* phi, double* nx, double* ny);
int or_jump_poisson_assemble(const or_grid* gr, const double* pressure, const double* density, const int* bc, const double* div,
                             const double* phi, const double* nx, const double* ny, const double* jc_solution,
                             const double* jc_derivative, double* bx, double* by, double* diag, double* rhs);

/* LEVELSET_2D::FastSweepingMethodOriginal(sweeps) (LEVELSET_2D.h:281-384, 507-589). */
int or_fast_sweeping(const or_grid* gr, double* phi, int sweeps);

/* a10 in matrix-free form.  bx: x-faces (ni+1) x nj (face i between nodes i-1 and i),
 * by: y-faces ni x (nj+1), diag, rhs: ni x nj.  phi must already hold the ghost
 * state of the projection (or_curvature fills it).  kappa: ni x nj. */
int or_poisson_assemble(const or_grid* gr, const or_params* pr, const double* phi, const double* u, const double* v, const double* kappa, double dt,
                        double* bx, double* by, double* diag, double* rhs);
/* Matrix-free operator apply in the reference CSR row order (l, r, b, t, diag). */
void or_poisson_apply(const or_grid* gr, const double* bx, const double* by, const double* diag, const double* x, double* y);
/* The reference PCG with IC(0) (PCG_METHOD.cpp:176-264) on the matrix-free system.
 * x: warm start in, solution out (ni x nj).  max_iterations < 0 keeps pr's value. */
int or_pcg_ic0(const or_grid* gr, const or_params* pr, const double* bx, const double* by, const double* diag, const double* rhs, double* x, or_stats* st);

#ifdef __cplusplus
}
#endif
#endif
