// Internal declarations shared by the gb2d translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "gb2d.h"

namespace gb2d {

constexpr int kThreads = 256;       // threads per block for grid-stride kernels
constexpr int kMaxPartials = 1216;  // 152 SMs x 8: reduction partial sums per pass
constexpr int kCoarseMax = 64;      // coarsest multigrid level (<= 64 cells) is solved by a dense inverse
constexpr int kMaxLevels = 16;

// Grid spacing of one (sub)grid, computed as GRID_STRUCTURE_2D::Initialize does.
struct Space {
  double dx, dy, odx, ody, o2dx, o2dy, odx2, ody2;
};
Space make_space(int ires, int jres, double x_min, double y_min, double x_max, double y_max);

// Ghost-inclusive field view on the device.
struct DField {
  double* a;
  int g, nI, nJ, ld;
};
__host__ __device__ inline DField dfield(double* a, int g, int nI, int nJ) { return DField{a, g, nI, nJ, nI + 2 * g}; }
#define GB_AT(f, i, j) ((f).a[((i) + (f).g) + (size_t)((j) + (f).g) * (f).ld])

// FP32 <-> FP64 moves as bit manipulations on the integer pipes (FP64 issue
// slots, which conversions use, are scarce on this part).
// Exact FP32 -> FP64 (every FP32 value is an FP64 value); FP32 subnormals, below
// 1.2e-38, become signed zero.
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  unsigned long long bits = (unsigned long long)(u >> 31) << 63;
  if (e != 0u) {
    const unsigned long long E = e == 0xffu ? 0x7ffull : (unsigned long long)(e + 896u);
    bits |= (E << 52) | ((unsigned long long)(u & 0x7fffffu) << 29);
  }
  return __longlong_as_double((long long)bits);
}
__device__ __forceinline__ double widen(double d) { return d; }

// FP64 -> FP32 by truncation of the significand (the preconditioner's input
// only); magnitudes below the FP32 normal range become signed zero, above it
// infinity.
__device__ __forceinline__ float narrow(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned s = (unsigned)(b >> 63) << 31;
  const int E = (int)((b >> 52) & 0x7ffull);
  const int e = E - 896;
  unsigned bits;
  if (E == 0x7ff)
    bits = s | 0x7f800000u | (unsigned)((b >> 29) & 0x7fffffull) | ((b & 0xfffffffffffffull) ? 0x400000u : 0u);
  else if (e <= 0)
    bits = s;
  else if (e >= 255)
    bits = s | 0x7f800000u;
  else
    bits = s | ((unsigned)e << 23) | (unsigned)((b >> 29) & 0x7fffffull);
  return __uint_as_float(bits);
}

// ---- level construction -----------------------------------------------------

// Grid-stride loop over an nI x nJ index space on a 2D grid (x: columns, y:
// rows): no integer division per element.
#define GB_FOR_IJ(i, j, nI, nJ)                            \
  for (int j = blockIdx.y; j < (nJ); j += gridDim.y)       \
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (nI); i += gridDim.x * blockDim.x)

// Launch grid for GB_FOR_IJ with kThreads-wide blocks: columns covered, rows
// folded so that at most 152 x 16 blocks are launched.
inline dim3 grid_ij(int nI, int nJ) {
  unsigned gx = (unsigned)((nI + kThreads - 1) / kThreads), gy = (unsigned)nJ;
  if (gx < 1) gx = 1;
  if (gy < 1) gy = 1;
  while (gx * gy > 152u * 16u && gy > 1) gy = (gy + 1) / 2;
  return dim3(gx, gy);
}

// One multigrid level (cell-centred view of the node grid), padded with a zero
// ring: cell (i, j) at (i+1) + (j+1)*ld, ld = nI + 2.  cx at the same index is the
// conductance of the face between (i-1, j) and (i, j) (i = 0..nI), cy the face
// between (i, j-1) and (i, j).  Wall faces carry zero conductance.
template <typename T>
struct Level {
  int nI, nJ, ld;
  T *cx, *cy, *dg, *idg, *sh;  // sh = dg - sum of face conductances (pin / dx != dy terms)
  T *x, *b;                    // correction and right-hand side
  T* xa;                       // second correction buffer: tiled sweeps read one and write the other
};

// Device-resident solver scalars (deterministic reductions land here).
struct Scalars {
  double rz_new;   // r.z of the latest preconditioned residual
  double rz_cur;   // r.z belonging to the current search direction
  double alpha;    // step length for the current direction
  double beta;     // rz_new / rz_cur
  double rr;       // ||r||^2 of the latest update
  double thr2;     // ||r||^2 at which the running solve stops
  double bb;       // ||b||^2
  int flag;        // non-finite / zero-gradient detections
  int pad;
  int iters;       // CG iterations of the device-driven loop so far
  int max_it;      // its cap
  unsigned long long maxu_bits, maxv_bits;  // max |u|, |v| of the velocity update
  unsigned long long cfl_bits[3];           // max |u|, |v|, |kappa| for the CFL time step
  double cfl[5];                            // CFL dt, c_f, g_f, v_f, s_f
  // Frames run on the device (gb2d_batch_run_graph): the time step of the running frame,
  // which the kernels read in place of a host value, and the instance's totals.
  double dt_frame;
  double g_rr, g_bb;               // true ||r||^2 and ||b||^2 of the latest solve
  double g_rel2_max;               // largest ||r||^2 / ||b||^2 at the end of a solve
  unsigned long long g_iters;      // CG iterations of every solve
  int g_frames;                    // frames of the current run so far
  int g_capped;                    // a solve stopped at its iteration cap
};

// A time step given by value, or (p non-null) read on the device when the kernel runs: the
// frame's CFL step computed on the GPU.
struct DtArg {
  double v;
  const double* p;
  __device__ __forceinline__ double get() const { return p ? *p : v; }
};

struct Solver;  // defined in gb2d_solver.cu

// Kernels launched by this library (process-wide), reported by gb2d_kernel_launches.
// Launches made while this thread captures a graph count into t_capture_count instead
// (they run, and are counted, when the graph is launched).
extern std::atomic<unsigned long long> g_launches;
extern thread_local unsigned long long* t_capture_count;
#define GB_LAUNCHED(n) \
  (::gb2d::t_capture_count ? (void)(*::gb2d::t_capture_count += (n)) : (void)(::gb2d::g_launches += (n)))

// Event brackets around one kernel's launches (roofline measurement).
struct Probe {
  int on = 0, n = 0, cap = 0;
  cudaEvent_t* ev = nullptr;     // 2 * cap events
  double* bytes_each = nullptr;  // algorithmic bytes of each probed launch
};

}  // namespace gb2d

struct gb2d_ctx {
  gb2d_grid grid;
  gb2d_params prm;
  gb2d_flow_params flow;
  gb2d::Space base, xs, ys;
  cudaStream_t stream;
  cudaStream_t own_stream;
  cudaStream_t side;              // second stream for independent setup branches
  cudaEvent_t ev_fork, ev_join;   // fork / join of the side stream
  cudaStream_t side2;             // third stream: the preconditioner hierarchy built during the assembly
  cudaEvent_t ev_fork2, ev_join2, ev_pre0;  // ev_pre0: the FP64 finest level is built
  int device_loop;                // run each CG solve as one graph launch (a device-side WHILE loop)
  int asm_reuse;                  // the next projection keeps the phi-dependent assembly and solver levels
  // While a device-driven frame is captured (gb2d_batch_run_graph): the kernels take the time
  // step from dt_dev, nothing reads back to the host, and each solve loops on the device.
  const double* dt_dev;
  int graph_mode;
  cudaStream_t body_stream;       // captures the bodies of the device loops (created on first use)
  cudaStream_t xfer;              // host copies that overlap the projection (gb2d_projection_host)
  cudaEvent_t ev_xfer0, ev_xfer;
  gb2d::Probe probe;
  // Level-set buffers (ghost 2): current index into phi_buf.
  double* phi_buf[4];
  int phi_cur;
  double *u, *v, *ua, *va, *p, *kappa;
  double *u_alt, *v_alt;    // second face buffers: the viscosity pass writes them, then they swap with u, v
  double *u_keep, *v_keep;  // velocity TVD-RK3 stage-0 copies (water_velocity_field_*_rk_3rd)
  double* density;          // DetermineDensity's node density, ghost 2
  // Adjoint work buffers (allocated by the first adjoint call)
  double *adj_coef, *adj_gvel;        // WENO5 stencil coefficients (14 per node), velocity shares (2 per node)
  double *adj_lam_phi, *adj_mu_phi;   // cotangents of phi (ghost 2)
  double *adj_lam_u, *adj_lam_v;      // cotangents of U, V (ghost 2)
  double *adj_mu_u, *adj_mu_v;        // results for U/V (ghost 2) or UA/VA (ghost 3)
  double* adj_lam_p;                  // cotangent of p (ghost 1)
  double* adj_eno;                    // ENO3 adjoint: 16 coefficients per face of both MAC grids
  // General jump-Poisson inputs (allocated by the first gb2d_jump_poisson_solve)
  double *jmp_dens, *jmp_div, *jmp_js, *jmp_jd, *jmp_nx, *jmp_ny, *jmp_phi;
  int* jmp_bc;
  double* sign;  // reinit S (interior)
  // Assembled pressure system (FP64): faces bx ((ni+1) x nj), by (ni x (nj+1)), diag/rhs (ni x nj).
  double *bx, *by, *diag, *rhs;
  const double* sys_shift;  // diagonal beyond the face conductances (ni x nj), or null: the projection's structure
  double *tmp_a, *tmp_b;  // compact scratch for the standalone Poisson calls
  double* xw;             // padded solution buffer for gb2d_poisson_solve
  double* ckpt[6];        // checkpoint copies of phi, u, v, ua, va, p (allocated on first save)
  int ckpt_phi_cur;
  double* host_stage;  // pinned staging for small reads
  gb2d::Scalars* sc;   // device scalars
  gb2d::Solver* solver;
  char err[512];
};

namespace gb2d {

// ---- gb2d_exact.cu (FP64 kernels compiled without FMA contraction) ----
void launch_fill_ghost_copy(cudaStream_t s, double* dst, int gd, const double* src, int gs, int nI, int nJ, int g);
unsigned long long check_div_by(unsigned long long n, unsigned long long seed, int* cuda_error);
void launch_extrapolate_ghosts(cudaStream_t s, double* f, int g, int nI, int nJ);
void launch_weno5_advect(cudaStream_t s, const gb2d_ctx* c, const double* src, double* dst, double dt, int mixed);
void launch_reinit_sign(cudaStream_t s, const gb2d_ctx* c, const double* phi, double* S);
void launch_reinit_sweep(cudaStream_t s, const gb2d_ctx* c, const double* src, double* dst, const double* S, double dtau, int mixed);
void launch_blend(cudaStream_t s, const gb2d_ctx* c, const double* keep, double* phi, double c0, double c1);
void launch_eno3(cudaStream_t s, const gb2d_ctx* c, double dt);
void launch_curvature(cudaStream_t s, const gb2d_ctx* c, const double* phi, double* kappa, int* flag);
void launch_faces(cudaStream_t s, const gb2d_ctx* c, const double* phi, double dt);
void launch_diag(cudaStream_t s, const gb2d_ctx* c, double dt);
void launch_rhs(cudaStream_t s, const gb2d_ctx* c, const double* phi, double dt);
void launch_poisson_apply_exact(cudaStream_t s, const gb2d_ctx* c, const double* x, double* y);
void launch_velocity_update(cudaStream_t s, const gb2d_ctx* c, const double* phi, double dt, Scalars* sc);
void launch_copy_interior(cudaStream_t s, const double* src, int gs, double* dst, int gd, int nI, int nJ);
// FastSweepingMethodOriginal on the current level set (c->tmp_a holds the fixed band).
void launch_fast_sweeping(cudaStream_t s, gb2d_ctx* c, int sweeps);

// ---- gb2d_flow.cu (FP64, compiled without FMA contraction) ----
// Gravity (grav), viscosity (visc) and wall conditions (bc) over the face grids, and
// DetermineDensity into density (may be null).  With visc the result lands in the
// alternate face buffers, which then swap with c->u / c->v.
void launch_flow(cudaStream_t s, gb2d_ctx* c, double dt, int grav, int visc, int bc, double* density);
// u = c0 * u_keep + c1 * u on every face of both grids (velocity TVD-RK3).
void launch_face_blend(cudaStream_t s, gb2d_ctx* c, double c0, double c1);
// CFLOneTimeStep into c->sc->cfl (dt, c_f, g_f, v_f, s_f).
void launch_cfl(cudaStream_t s, gb2d_ctx* c);
// The frame's time step on the device, as gb2d_advance_frame forms it on the host:
// c->sc->dt_frame = (CFL step, or the previous dt_frame when that is zero) * cfl.
void launch_frame_dt(cudaStream_t s, gb2d_ctx* c, double cfl);

// ---- gb2d_api.cu ----
// One gb2d_advance_frame captured on c->stream for the device (no host reads; see gb2d_api.cu).
int frame_capture(gb2d_ctx* c, double cfl, const gb2d_solve_opts* o);

// ---- gb2d_adjoint.cu ----
int adjoint_buffers(gb2d_ctx* c);
// VJP of one level-set advection sweep at the current PHI, UA, VA: adj_lam_phi (consumed)
// -> adj_mu_phi; velocity cotangents into mu_ua / mu_va (UA/VA layout) when non-null.
void launch_weno5_adjoint(cudaStream_t s, gb2d_ctx* c, double dt, double* mu_ua, double* mu_va);
// Projection adjoint: c->rhs = dL/dp from adj_lam_u/v (and adj_lam_p); then, after the
// solve into the padded z, adj_mu_u/v = lam + D^T z.
void launch_projection_adjoint_rhs(cudaStream_t s, gb2d_ctx* c, double dt, int with_lam_p);
void launch_projection_adjoint_vel(cudaStream_t s, gb2d_ctx* c, double dt, const double* z);
// dL/d(water density), dL/d(air density) after the projection adjoint (z in c->xw).
int density_gradient(gb2d_ctx* c, double dt, double* d_water, double* d_air);
// dL/dphi (phi's layout, ghost 2) after the projection adjoint, into host_out.
int phi_gradient(gb2d_ctx* c, double dt, double* host_out);
// VJP of the last velocity advection (the FP64 forms of ENO3) at the current UA, VA: cotangents
// adj_lam_u / adj_lam_v of the advected U, V -> adj_mu_u / adj_mu_v on UA / VA (ghost 3).
int eno3_adjoint(gb2d_ctx* c, double dt);
// VJP of one reinitialisation sweep (FP64 form) at phi (device, ghost 2) and S (device, ni x nj):
// lam (device, ghost 2) -> mu (device, ghost 2) and the cotangent of S into gs (device, ni x nj).
int reinit_sweep_vjp(gb2d_ctx* c, const double* phi, const double* sign, const double* lam, double* mu, double* gs);
int viscosity_vjp(gb2d_ctx* c, double dt, const double* lu, const double* lv, double* mu, double* mv, double* mp,
                  double* d_density);

// ---- gb2d_jump.cu (FP64, compiled without FMA contraction) ----
int jump_buffers(gb2d_ctx* c);
// Normals of jmp_phi, then the jump system (xw holds the pressure with its boundary values)
// into c->bx, by, diag, rhs, and its diagonal shift into c->tmp_b.
void launch_jump_assemble(cudaStream_t s, gb2d_ctx* c);

// ---- gb2d_solver.cu ----
Solver* solver_create(int ni, int nj, char* err, size_t errlen);
void solver_destroy(Solver* s);
// Solve A x = rhs (system held in ctx->bx/by/diag) with x (ni x nj, FP64, compact) as warm start.
int solver_solve(gb2d_ctx* c, const double* rhs, double* x, const gb2d_solve_opts* o, gb2d_solve_stats* st);
// With MG-PCG options: start building the solver's levels from ctx->bx/by/diag (complete
// on ctx->stream) on ctx->side2 (the FP64 finest level, then the FP32 hierarchy or the
// FP64 coarse levels and dense inverse); the next solver_solve joins them instead of
// building them.  Jacobi-PCG: no-op.
void solver_prebuild(gb2d_ctx* c, const gb2d_solve_opts* o);
// Abandon a started prebuild (an error before the solve): ctx->stream waits for it.
void solver_drop_prebuild(gb2d_ctx* c);
// The next solver_solve keeps its levels (built by the previous solve from the same
// ctx->bx/by/diag) and refreshes only the right-hand side.
void solver_keep_levels(gb2d_ctx* c);
void solver_layout(const Solver* S, int mixed, int* levels, int* cluster_top, int* cluster_ctas);
// Tile shapes of the smoothing levels: < 0 the default per-level rule, 0-3 one shape for all.
void solver_set_tile_plan(gb2d_ctx* c, int plan);
// Kernels of one CG iteration in the loop body of the latest device-driven solve capture.
unsigned long long solver_body_nodes(const gb2d_ctx* c);
// One multigrid V-cycle (nu sweeps per side, FP32 levels when prec) of the assembled
// system in ctx->bx/by/diag applied to r: z = M r (device, compact ni x nj FP64).
int solver_precondition(gb2d_ctx* c, int prec, int nu, const double* r_dev, double* z_dev);

}  // namespace gb2d

#define GB2D_CUDA_TRY(ctx, expr)                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (expr);                                                                      \
    if (e_ != cudaSuccess) {                                                                      \
      snprintf((ctx)->err, sizeof((ctx)->err), "%s: %s (%s:%d)", #expr, cudaGetErrorString(e_),   \
               __FILE__, __LINE__);                                                               \
      return GB2D_ERR_CUDA;                                                                       \
    }                                                                                             \
  } while (0)
