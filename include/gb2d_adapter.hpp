// gb2d_adapter.hpp — C++ host-side mirror of the reference solver's step
// interface on top of the C ABI in gb2d.h.
//
// EULERIAN_FLUID_SOLVER_2D (ByungJoonLee/2D_Engine) calls its level-set,
// reinitialisation, velocity-advection and projection members from every
// worker thread, with barriers inside (EULERIAN_FLUID_SOLVER_2D.h:1140-1796).
// GB2D_FLUID_STEP keeps those member names and arguments: the head thread
// (thread_id == 0) issues the GPU work, and the caller's barrier (passed in as a
// callable, MULTITHREADING::Sync in the reference) makes the other threads wait,
// as BEGIN_HEAD_THREAD_WORK/END_HEAD_THREAD_WORK do (MACROS.h:74-75).
// Errors print to std::cerr and exit, as the reference does on a failed
// curvature (LEVELSET_2D.h:869-873).
//
// The arrays handed to Upload/Download are the reference's ghost-inclusive
// ARRAY_2D storage (FIELD_STRUCTURE_2D::array_for_this.values).
#ifndef GB2D_ADAPTER_HPP
#define GB2D_ADAPTER_HPP

#include <cstdlib>
#include <functional>
#include <iostream>

#include "gb2d.h"

class GB2D_FLUID_STEP {
 public:
  typedef std::function<void(int)> SYNC;  // barrier across worker threads (MULTITHREADING::Sync)

  GB2D_FLUID_STEP(const gb2d_grid& grid, const gb2d_params& params, const gb2d_solve_opts& solve, SYNC sync = SYNC())
      : ctx_(0), solve_(solve), sync_(sync) {
    Check(gb2d_create(&grid, &params, &ctx_), "gb2d_create");
  }
  ~GB2D_FLUID_STEP() {
    if (ctx_) gb2d_destroy(ctx_);
  }
  GB2D_FLUID_STEP(const GB2D_FLUID_STEP&) = delete;
  GB2D_FLUID_STEP& operator=(const GB2D_FLUID_STEP&) = delete;

  // Host <-> device state (ghost-inclusive reference arrays).
  void Upload(int field, const double* values) { Check(gb2d_set_field(ctx_, field, values), "gb2d_set_field"); }
  void Download(int field, double* values) { Check(gb2d_get_field(ctx_, field, values), "gb2d_get_field"); }

  // EULERIAN_FLUID_SOLVER_2D::Levelset_Advection(dt, thread_id) (:1896-2045)
  void Levelset_Advection(const double& dt, const int& thread_id) {
    if (thread_id == 0) Check(gb2d_levelset_advection(ctx_, dt), "Levelset_Advection");
    Sync(thread_id);
  }
  // EULERIAN_FLUID_SOLVER_2D::Reinitialization(dt, thread_id) (:2402-2445); dt is unused there too.
  void Reinitialization(const double& dt, const int& thread_id) {
    (void)dt;
    if (thread_id == 0) Check(gb2d_reinitialization(ctx_), "Reinitialization");
    Sync(thread_id);
  }
  // The level-set and reinitialisation TVD-RK3 blocks of AdvanceOneTimeStepThread (:1694-1741).
  void Levelset_RK3(const double& dt, const int& thread_id) {
    if (thread_id == 0) Check(gb2d_levelset_rk3(ctx_, dt), "Levelset_RK3");
    Sync(thread_id);
  }
  // EULERIAN_FLUID_SOLVER_2D::Velocity_Advection(dt, thread_id) (:1886-1889)
  void Velocity_Advection(const double& dt, const int& thread_id) {
    if (thread_id == 0) Check(gb2d_velocity_advection(ctx_, dt), "Velocity_Advection");
    Sync(thread_id);
  }
  // EULERIAN_FLUID_SOLVER_2D::Projection(dt, thread_id) (:2359-2363)
  void Projection(const double& dt, const int& thread_id) {
    if (thread_id == 0) Solved(gb2d_projection(ctx_, dt, &solve_, &stats_), "Projection");
    Sync(thread_id);
  }
  // Projection(dt, thread_id) on a state kept in the reference's own host arrays (the
  // array_for_this.values of the level set, the two MAC velocity fields and the pressure):
  // phi, U, V and the warm-start p go in, and the projected U, V and p come back in place,
  // in one call whose copies overlap the GPU work (gb2d_projection_host).
  void ProjectionOnHost(const double& dt, const int& thread_id, const double* phi, double* u, double* v, double* p) {
    if (thread_id == 0) Solved(gb2d_projection_host(ctx_, dt, &solve_, phi, u, v, p, p, u, v, &stats_), "Projection");
    Sync(thread_id);
  }

  // Constants of gravity, viscosity and the CFL time step (gb2d_flow_params).
  void SetFlowParams(const gb2d_flow_params& flow) { Check(gb2d_set_flow_params(ctx_, &flow), "gb2d_set_flow_params"); }
  // EULERIAN_FLUID_SOLVER_2D::SolveForRK(dt, thread_id) (:1857-1879)
  void SolveForRK(const double& dt, const int& thread_id) {
    if (thread_id == 0) Solved(gb2d_solve_for_rk(ctx_, dt, &solve_, &stats_), "SolveForRK");
    Sync(thread_id);
  }
  // EULERIAN_FLUID_SOLVER_2D::AdvanceOneTimeStepThread(dt, thread_id), order 3 (:1140, 1694-1794)
  void AdvanceOneTimeStepThread(const double& dt, const int& thread_id) {
    if (thread_id == 0) Solved(gb2d_advance_time_step(ctx_, dt, &solve_, &stats_), "AdvanceOneTimeStepThread");
    Sync(thread_id);
  }
  // EULERIAN_FLUID_SOLVER_2D::CFLOneTimeStep() (:3517-3637), with the curvature as it stands;
  // head thread only, like SIMULATION_WORLD::DetermineTimeStep.
  double CFLOneTimeStep() {
    double dt = 0, rates[4];
    Check(gb2d_cfl_time_step(ctx_, &dt, rates), "CFLOneTimeStep");
    c_f = rates[0];
    g_f = rates[1];
    v_f = rates[2];
    s_f = rates[3];
    return dt;
  }
  // SIMULATION_WORLD::AdvanceOneFrame (SIMULATION_WORLD.h:1094-1146): curvature, dt = CFL step * cfl,
  // one time step.  dt: the previous step in, the step taken out.
  void AdvanceOneFrame(const double& cfl, double& dt) { Solved(gb2d_advance_frame(ctx_, cfl, &dt, &solve_, &stats_), "AdvanceOneFrame"); }

  const gb2d_solve_stats& LastSolveStats() const { return stats_; }
  gb2d_ctx* Context() const { return ctx_; }

  double max_velocity_x = 0, max_velocity_y = 0;  // PROJECTION_2D::max_velocity_x/_y
  double c_f = 0, g_f = 0, v_f = 0, s_f = 0;       // rates of the last CFLOneTimeStep

 private:
  void Sync(int thread_id) {
    if (sync_) sync_(thread_id);
  }
  // A solve stopped at its iteration cap is not fatal (PCG_METHOD.cpp:253).
  void Solved(int rc, const char* what) {
    if (rc != GB2D_ERR_MAX_ITERS) Check(rc, what);
    max_velocity_x = stats_.max_velocity_x;
    max_velocity_y = stats_.max_velocity_y;
  }
  void Check(int rc, const char* what) {
    if (rc != GB2D_OK) {
      std::cerr << what << " failed (" << rc << "): " << (ctx_ ? gb2d_last_error(ctx_) : "no context") << std::endl;
      std::exit(1);
    }
  }

  gb2d_ctx* ctx_;
  gb2d_solve_opts solve_;
  gb2d_solve_stats stats_ = {};
  SYNC sync_;
};

#endif  // GB2D_ADAPTER_HPP
