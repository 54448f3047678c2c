/*
 * Headless driver around the reference solver (ByungJoonLee/2D_Engine), built
 * by oracle/ref/Makefile straight from the reference's own sources into
 * oracle/_ref/libref2d.so.  It is test infrastructure only: the golden-vector
 * generator (tests/golden/make_golden.py) and the oracle-vs-reference checks
 * call it to obtain outputs of the reference itself.
 *
 * It replaces what SIMULATION_WORLD.h:86-307 and :1094-1146 do (script parsing,
 * GLUT, timers) with direct construction of EULERIAN_FLUID_SOLVER_2D
 * (EULERIAN_FLUID_SOLVER_2D.h:159-727) from a SCRIPT_BLOCK whose values this
 * file fills in, then exposes the solver's own step functions:
 *   Levelset_Advection (:1896), Reinitialization (:2402), Velocity_Advection
 *   (:1886), Projection (:2359), AdvanceOneTimeStepThread (:1140), SolveForRK
 *   (:1857), ApplyGraivity (:3249), Sourcing (:2082), SetupBoundaryConditionForVelocity
 *   (:2227),
 *   LEVELSET_2D::ComputeCurvaturesThread (LEVELSET_2D.h:898).
 * Every call runs on one worker (thread_id 0 of a 1-thread MULTITHREADING),
 * which is how the reference's head thread runs the pressure solve anyway
 * (PROJECTION_2D.h:250-254).
 */
#include <cstdio>
#include <cstdlib>
#include <map>
#include <sstream>
#include <streambuf>
#include <string>

#include "EULERIAN_FLUID_SOLVER_2D.h"
#include "POISSON_EQUATION_TEST.h"

/* ---- SCRIPT_BLOCK accessors (declared in SCRIPT_READER.h:112-160) ----------
 * The reference implements these with a regex parser (SCRIPT_READER.cpp); the
 * driver stores already-typed text values, so plain lookups are enough. */
static SCRIPT_BLOCK g_empty_block;

const SCRIPT_VALUE* SCRIPT_BLOCK::SearchValue(const vector<SCRIPT_VALUE*>* vals, const char* name) const {
  for (size_t k = 0; k < vals->size(); ++k)
    if ((*vals)[k]->value_name == name) return (*vals)[k];
  return 0;
}
const SCRIPT_BLOCK& SCRIPT_BLOCK::FindBlock(const char* name) const {
  for (size_t k = 0; k < child_blocks.size(); ++k)
    if (child_blocks[k]->block_name == name) return *child_blocks[k];
  return g_empty_block;
}
int SCRIPT_BLOCK::GetInteger(const char* name, const int& dflt) const {
  const SCRIPT_VALUE* v = SearchValue(&values, name);
  return v ? atoi(v->val.c_str()) : dflt;
}
T SCRIPT_BLOCK::GetFloat(const char* name, const T& dflt) const {
  const SCRIPT_VALUE* v = SearchValue(&values, name);
  return v ? strtod(v->val.c_str(), 0) : dflt;
}
VT SCRIPT_BLOCK::GetVector2(const char* name, const VT& dflt) const {
  const SCRIPT_VALUE* v = SearchValue(&values, name);
  if (!v) return dflt;
  double a = 0, b = 0;
  sscanf(v->val.c_str(), "%lf %lf", &a, &b);
  return VT(a, b);
}
VI SCRIPT_BLOCK::GetInt2(const char* name, const VI& dflt) const {
  const SCRIPT_VALUE* v = SearchValue(&values, name);
  if (!v) return dflt;
  int a = 0, b = 0;
  sscanf(v->val.c_str(), "%d %d", &a, &b);
  return VI(a, b);
}
bool SCRIPT_BLOCK::GetBoolean(const char* name, const bool dflt) const {
  const SCRIPT_VALUE* v = SearchValue(&values, name);
  return v ? (v->val == "true") : dflt;
}
const char* SCRIPT_BLOCK::GetString(const char* name, const char* dflt) const {
  const SCRIPT_VALUE* v = SearchValue(&values, name);
  return v ? v->val.c_str() : dflt;
}

namespace {

struct NullBuffer : std::streambuf {
  int overflow(int c) override { return c; }
};
NullBuffer g_null;

void put(SCRIPT_BLOCK& b, const char* name, const std::string& val) {
  SCRIPT_VALUE* v = new SCRIPT_VALUE;
  v->value_name = name;
  v->val = val;
  v->val_type = SCRIPT_VALUE::TYPE_NONE;
  b.values.push_back(v);
}
std::string num(double x) {
  char buf[64];
  snprintf(buf, sizeof buf, "%.17g", x);
  return buf;
}
SCRIPT_BLOCK* child(SCRIPT_BLOCK& b, const char* name) {
  SCRIPT_BLOCK* c = new SCRIPT_BLOCK;
  c->block_name = name;
  b.child_blocks.push_back(c);
  return c;
}

struct RefSim {
  MULTITHREADING mt;
  WORLD_DISCRETIZATION_2D world;
  EULERIAN_FLUID_SOLVER_2D solver;
  SCRIPT_BLOCK block;
#ifdef REF_GPU
  ~RefSim() { delete solver.gpu_step; }
#endif
};

ARRAY_2D<T>* field(RefSim* s, int id) {
  EULERIAN_FLUID_SOLVER_2D& f = s->solver;
  switch (id) {
    case 0: return &f.water_levelset->signed_distance_field.array_for_this;  // phi, ghost 2
    case 1: return &f.water_velocity_field_mac_x->array_for_this;            // U faces, ghost 2
    case 2: return &f.water_velocity_field_mac_y->array_for_this;            // V faces, ghost 2
    case 3: return &f.vector_field_mac_ghost_x.array_for_this;               // advecting U, ghost 3
    case 4: return &f.vector_field_mac_ghost_y.array_for_this;               // advecting V, ghost 3
    case 5: return &f.water_projection->pressure_field.array_for_this;       // p, ghost 1
    case 6: return &f.water_levelset->curvature.array_for_this;              // kappa, ghost 0
    case 7: return &f.water_projection->projection_density_field.array_for_this;  // rho, ghost 1
    case 8: return &f.water_projection->jc_on_solution.array_for_this;       // sigma*kappa, ghost 1
    case 9: return &f.water_projection->divergence_field.array_for_this;     // div/dt, ghost 1
    case 10: return &f.sign_function.array_for_this;                         // reinit S, ghost 3
    case 11: return &f.scalar_field_ghost.array_for_this;                    // WENO scratch, ghost 3
    case 12: return &f.density_field.array_for_this;                         // node density, ghost 2
    case 13: return &f.water_velocity_field_x_rk_3rd.array_for_this;         // velocity RK3 keep, x
    case 14: return &f.water_velocity_field_y_rk_3rd.array_for_this;         // velocity RK3 keep, y
    default: return 0;
  }
}

}  // namespace

extern "C" {

/* prm: [0] water_density (phi > 0), [1] air_density (phi <= 0), [2] water_viscosity,
 * [3] air_viscosity, [4] surface_tension, [5] gravity_x, [6] gravity_y,
 * [7] PCG tolerance on sqrt(r.z) (PCG_METHOD.cpp:254), [8] PCG max_iteration,
 * [9] iteration_number_for_reinitialization, [10] scaling_number_for_reinitialization,
 * [11] cfl_number, [12] WENO epsilon. */
void* ref_create(int ni, int nj, double x_min, double y_min, double x_max, double y_max, const double* prm) {
  std::cout.rdbuf(&g_null);
  RefSim* s = new RefSim;
  s->mt.Initialize(1);
  s->world.large_bubble = true;
  s->world.small_bubble = false;
  s->world.air_water_simulation = true;

  SCRIPT_BLOCK& b = s->block;
  put(b, "ghost_width", "3");
  put(b, "fastsweeping_reinitialization", "false");
  put(b, "sussmanstyle_reinitialization", "true");
  put(b, "scaling_number_for_reinitialization", num(prm[10]));
  put(b, "iteration_number_for_reinitialization", num(prm[9]));
  put(b, "water_viscosity", num(prm[2]));
  put(b, "air_viscosity", num(prm[3]));
  put(b, "gravity", num(prm[5]) + " " + num(prm[6]));
  put(b, "water_density", num(prm[0]));
  put(b, "air_density", num(prm[1]));
  put(b, "surface_tension", num(prm[4]));
  put(b, "order_for_time_advancing", "3");
  put(b, "cfl_number", num(prm[11]));
  put(b, "use_mac_grid", "true");
  put(b, "is_velocity_advection_active", "true");
  put(b, "is_sourcing_active", "true");
  put(b, "is_projection_active", "true");
  put(b, "is_levelset_advection_active", "true");
  put(b, "is_viscosity_active", "true");
  put(b, "use_delta_function_formulation", "true");
  put(b, "use_jump_condition_on_viscosity", "false");
  put(b, "CSF_model", "false");
  put(b, "curvature_by_normal_vector", "false");
  put(b, "curvature_by_levelset", "true");
  SCRIPT_BLOCK* la = child(b, "LEVELSET_ADVECTION");
  put(*la, "use_5th_weno", "true");
  put(*la, "epsilon", num(prm[12]));
  SCRIPT_BLOCK* va = child(b, "VELOCITY_ADVECTION");
  put(*va, "use_3rd_eno_v", "true");
  SCRIPT_BLOCK* pr = child(b, "PROJECTION");
  put(*pr, "tolerance", num(prm[7]));
  put(*pr, "max_iteration", num(prm[8]));
  put(*pr, "air_bubble_rising", "true");
  put(*pr, "poisson_solver_type", "PCG");
  put(*pr, "Neumann_Boundary_Condition", "true");

  GRID_STRUCTURE_2D grid(ni, nj, 0, 0, x_min, y_min, x_max, y_max);
  s->solver.world_discretization = &s->world;
  s->solver.air_water_simulation = true;
  s->solver.InitializeFromScriptBlock(grid, b, &s->mt);
  /* For air/water the reference constructs its VISCOSITY_2D (EULERIAN_FLUID_SOLVER_2D.h:646-652)
   * but never calls VISCOSITY_2D::InitializeFromScriptBlock (only the oil/water branch does,
   * :668), and the constructor's initialiser list (VISCOSITY_2D.h:107-111) leaves
   * use_delta_function_formulation unset.  With it false, ApplyViscosity does nothing for
   * air/water; the driver sets it so, making that behaviour deterministic.
   * ref_configure_viscosity(h, 1) runs the configuration step the air/water branch skips. */
  s->solver.viscosity_solver->use_delta_function_formulation = false;
  return s;
}

/* Configure the viscosity solver as VISCOSITY_2D::InitializeFromScriptBlock (VISCOSITY_2D.h:117-276)
 * would for this script (enable = 1), so that ApplyViscosity applies the delta-function
 * formulation (:460-532) with the script's viscosities and densities; enable = 0 returns
 * to the reference's as-shipped air/water behaviour (no viscous term). */
void ref_configure_viscosity(void* h, int enable) {
  RefSim* s = static_cast<RefSim*>(h);
  VISCOSITY_2D* vs = s->solver.viscosity_solver;
  if (!enable) {
    vs->use_delta_function_formulation = false;
    return;
  }
  SCRIPT_BLOCK blk;
  for (size_t k = 0; k < s->block.values.size(); ++k) {
    const SCRIPT_VALUE* v = s->block.values[k];
    if (v->value_name != "use_delta_function_formulation") put(blk, v->value_name.c_str(), v->val);
  }
  put(blk, "use_delta_function_formulation", "true");
  SCRIPT_BLOCK* pw = child(blk, "PROJECTION_WATER");
  put(*pw, "air_bubble_rising", "true");
  SCRIPT_BLOCK* pr = child(blk, "PROJECTION");
  put(*pr, "poisson_solver_type", "PCG");
  vs->air_water_simulation = true;
  vs->oil_water_simulation = false;
  vs->InitializeFromScriptBlock(blk);
}

void ref_destroy(void* h) { delete static_cast<RefSim*>(h); }

/* Shape of a ghost-inclusive array: start indices (negative = ghost width) and extents. */
int ref_field_shape(void* h, int id, int* i_start, int* j_start, int* i_res, int* j_res) {
  ARRAY_2D<T>* a = field(static_cast<RefSim*>(h), id);
  if (!a) return -1;
  *i_start = a->i_start;
  *j_start = a->j_start;
  *i_res = a->i_res;
  *j_res = a->j_res;
  return 0;
}
int ref_get_field(void* h, int id, double* out) {
  ARRAY_2D<T>* a = field(static_cast<RefSim*>(h), id);
  if (!a) return -1;
  for (int k = 0; k < a->ij_res; ++k) out[k] = a->values[k];
  return 0;
}
int ref_set_field(void* h, int id, const double* in) {
  ARRAY_2D<T>* a = field(static_cast<RefSim*>(h), id);
  if (!a) return -1;
  for (int k = 0; k < a->ij_res; ++k) a->values[k] = in[k];
  return 0;
}

void ref_levelset_advection(void* h, double dt) { static_cast<RefSim*>(h)->solver.Levelset_Advection(dt, 0); }
void ref_reinitialization(void* h, double dt) { static_cast<RefSim*>(h)->solver.Reinitialization(dt, 0); }
void ref_velocity_advection(void* h, double dt) { static_cast<RefSim*>(h)->solver.Velocity_Advection(dt, 0); }
void ref_projection(void* h, double dt) { static_cast<RefSim*>(h)->solver.Projection(dt, 0); }
void ref_curvature(void* h) { static_cast<RefSim*>(h)->solver.water_levelset->ComputeCurvaturesThread(0); }
void ref_fast_sweeping(void* h, int sweeps) { static_cast<RefSim*>(h)->solver.water_levelset->FastSweepingMethodOriginal(sweeps); }
void ref_apply_gravity(void* h, double dt) { static_cast<RefSim*>(h)->solver.ApplyGraivity(dt, 0); }
void ref_sourcing(void* h, double dt) { static_cast<RefSim*>(h)->solver.Sourcing(dt, 0); }
void ref_velocity_bc(void* h) { static_cast<RefSim*>(h)->solver.SetupBoundaryConditionForVelocity(); }
void ref_solve_for_rk(void* h, double dt) { static_cast<RefSim*>(h)->solver.SolveForRK(dt, 0); }
void ref_step(void* h, double dt) { static_cast<RefSim*>(h)->solver.AdvanceOneTimeStepThread(dt, 0); }
double ref_cfl_dt(void* h) { return static_cast<RefSim*>(h)->solver.CFLOneTimeStep(); }

/* ---- POISSON_EQUATION_TEST (POISSON_EQUATION_TEST.h) -------------------------
 * The jump-condition Poisson tests 3 and 5 on [-1,1]^2 with n x n nodes, Dirichlet
 * boundaries and PCG, set up as SIMULATION_WORLD does for
 * poisson_equation_with_jump_condition (SIMULATION_WORLD.h:379-384 and the interface
 * level sets at :913-943), then solved by POISSON_EQUATION_TEST::Solve (:288-311). */
struct RefPoisson {
  MULTITHREADING mt;
  WORLD_DISCRETIZATION_2D world;
  POISSON_EQUATION_TEST test;
};

/* Test 8's interface as SIMULATION_WORLD builds it (SIMULATION_WORLD.h:945-1070): the
 * distance to 8000 samples of the five-petal curve r = 0.5 + 0.2 sin(5 theta) about
 * (0.02 sqrt 5, 0.02 sqrt 5), signed by comparing the node with that curve at the
 * node's own polar angle about the origin (the reference's test, kept as it is). */
static T star_levelset(T x, T y) {
  const int samples = 8000;
  const T c = (T)0.02 * sqrt((T)5);
  T best = 0;
  for (int p = 0; p < samples; ++p) {
    const T th = (T)2 * PI * p / samples;
    const T px = c + ((T)0.5 + (T)0.2 * sin(5 * th)) * cos(th);
    const T py = c + ((T)0.5 + (T)0.2 * sin(5 * th)) * sin(th);
    const T d = sqrt(POW2(x - px) + POW2(y - py));
    if (p == 0 || d <= best) best = d;
  }
  const T ratio = y / x;
  T ang;
  if (x >= (T)0 && y >= (T)0)
    ang = atan(ratio);
  else if (x <= (T)0 && y >= (T)0)
    ang = PI + atan(ratio);
  else if (x <= (T)0 && y <= (T)0)
    ang = PI + atan(ratio);
  else
    ang = 2 * PI + atan(ratio);
  const T side = POW2(x - 0.02 * sqrt(5)) + POW2(y - 0.02 * sqrt(5)) - POW2(0.5 + 0.2 * sin(5 * ang));
  if (side > 0) return best;
  if (side < 0) return -best;
  return 0;  // on the curve, or a NaN test (the origin's angle): the reference leaves 0
}

void* ref_poisson_create(int test_number, int n, double tolerance, int max_iteration) {
  std::cout.rdbuf(&g_null);
  if (test_number != 3 && test_number != 5 && test_number != 8) return 0;
  RefPoisson* r = new RefPoisson;
  r->mt.Initialize(1);
  r->world.poisson_equation_with_jump_condition_test = true;
  r->world.grid_1d = false;
  r->world.grid_2d = true;
  r->world.world_grid.Initialize(n, n, 0, 0, -1, -1, 1, 1);
  r->test.world_discretization = &r->world;
  r->test.test_number = test_number;
  r->test.grid_1d = false;
  r->test.grid_2d = true;
  SCRIPT_BLOCK b;
  put(b, "tolerance", num(tolerance));
  put(b, "max_iteration", num(max_iteration));
  put(b, "poisson_solver_type", "PCG");
  put(b, "Dirichlet_Boundary_Condition", "true");
  put(b, "Neumann_Boundary_Condition", "false");
  r->test.InitializeFromBlock(b, &r->mt);
  LEVELSET_2D& ls = *r->test.interface_levelset_2d;
  GRID_STRUCTURE_2D& g = ls.grid;
  for (int j = g.j_start; j <= g.j_end; ++j)
    for (int i = g.i_start; i <= g.i_end; ++i) {
      T x = g.x_min + i * g.dx, y = g.y_min + j * g.dy;
      if (test_number == 3)
        ls(i, j) = sqrt(POW2(x - (T)0.5) + POW2(y - (T)0.5)) - (T)0.25;
      else if (test_number == 5)
        ls(i, j) = sqrt(POW2(x) + POW2(y)) - (T)0.5;
      else
        ls(i, j) = star_levelset(x, y);
    }
  ls.FillGhostCellsFromThreaded(&(ls.phi), false);
  return r;
}

void ref_poisson_destroy(void* h) { delete static_cast<RefPoisson*>(h); }

double ref_poisson_solve(void* h) {
  RefPoisson* r = static_cast<RefPoisson*>(h);
  r->test.Solve(0);
  return r->test.l2_norm;
}

/* Fields after ref_poisson_solve, ghost-inclusive: 0 solution (ghost 1), 1 true solution,
 * 2 beta, 3 rhs, 4 jc_on_solution, 5 jc_on_derivative, 6 boundary condition (as double),
 * 7 interface level set (ghost 2), 8 / 9 normal x / y (ghost 1). */
int ref_poisson_field(void* h, int id, int* i_res, int* j_res, double* out) {
  RefPoisson* r = static_cast<RefPoisson*>(h);
  POISSON_EQUATION_TEST& t = r->test;
  const ARRAY_2D<T>* a = 0;
  switch (id) {
    case 0: a = &t.solution_2d.array_for_this; break;
    case 1: a = &t.true_solution_2d.array_for_this; break;
    case 2: a = &t.beta_2d.array_for_this; break;
    case 3: a = &t.rhs_2d.array_for_this; break;
    case 4: a = &t.jc_on_solution_2d.array_for_this; break;
    case 5: a = &t.jc_on_derivative_2d.array_for_this; break;
    case 7: a = &t.interface_levelset_2d->signed_distance_field.array_for_this; break;
    default: break;
  }
  if (a) {
    *i_res = a->i_res;
    *j_res = a->j_res;
    if (out)
      for (int k = 0; k < a->ij_res; ++k) out[k] = a->values[k];
    return 0;
  }
  if (id == 6) {
    const ARRAY_2D<int>& bc = t.boundary_condition_2d.array_for_this;
    *i_res = bc.i_res;
    *j_res = bc.j_res;
    if (out)
      for (int k = 0; k < bc.ij_res; ++k) out[k] = bc.values[k];
    return 0;
  }
  if (id == 8 || id == 9) {
    const ARRAY_2D<VT>& nv = t.interface_levelset_2d->normal.array_for_this;
    *i_res = nv.i_res;
    *j_res = nv.j_res;
    if (out)
      for (int k = 0; k < nv.ij_res; ++k) out[k] = id == 8 ? nv.values[k].x : nv.values[k].y;
    return 0;
  }
  return -1;
}

int ref_poisson_test_system(void* h, int* n, int* nnz, int* row_ptr, int* col, double* val, double* b, int* iterations) {
  POISSON_SOLVER& ps = static_cast<RefPoisson*>(h)->test.poisson_solver;
  *n = ps.A.N;
  *nnz = ps.A.nz;
  if (row_ptr) for (int k = 0; k <= ps.A.N; ++k) row_ptr[k] = ps.A.row_ptr[k];
  if (col) for (int k = 0; k < ps.A.nz; ++k) col[k] = ps.A.column_index[k];
  if (val) for (int k = 0; k < ps.A.nz; ++k) val[k] = ps.A.values[k];
  if (b) for (int k = 0; k < ps.b.num_dimension; ++k) b[k] = ps.b[k];
  if (iterations) *iterations = ps.linear_solver->num_iteration;
  return 0;
}

/* Linear system of the most recent projection (POISSON_SOLVER.cpp:714-976):
 * call with null arrays to get n and nnz, then again to copy. */
int ref_poisson_system(void* h, int* n, int* nnz, int* row_ptr, int* col, double* val, double* b, double* x) {
  POISSON_SOLVER& ps = static_cast<RefSim*>(h)->solver.water_projection->poisson_solver;
  *n = ps.A.N;
  *nnz = ps.A.nz;
  if (row_ptr) for (int k = 0; k <= ps.A.N; ++k) row_ptr[k] = ps.A.row_ptr[k];
  if (col) for (int k = 0; k < ps.A.nz; ++k) col[k] = ps.A.column_index[k];
  if (val) for (int k = 0; k < ps.A.nz; ++k) val[k] = ps.A.values[k];
  if (b) for (int k = 0; k < ps.b.num_dimension; ++k) b[k] = ps.b[k];
  if (x) for (int k = 0; k < ps.x.num_dimension; ++k) x[k] = ps.x[k];
  return 0;
}
#ifdef REF_GPU
/* The drop-in (built by `make -C oracle/ref gpu` on a copy of EULERIAN_FLUID_SOLVER_2D.h
 * with the hooks of oracle/ref/patch_gpu_step.py, linked against libgb2d.so): the
 * solver's GB2D_FLUID_STEP is built from its own grid and script constants, as
 * INTEGRATION.md shows a maintainer doing at the end of InitializeFromScriptBlock, and
 * loaded with the solver's current state; from then on AdvanceOneTimeStepThread,
 * CFLOneTimeStep and the four step members run on the GPU.  ref_gpu_download copies the
 * device state back into the reference's arrays. */
int ref_enable_gpu(void* h, int mixed, double tolerance) {
  RefSim* s = static_cast<RefSim*>(h);
  EULERIAN_FLUID_SOLVER_2D& f = s->solver;
  const GRID_STRUCTURE_2D& g = f.base_grid;
  const int prec = mixed ? GB2D_PRECISION_MIXED : GB2D_PRECISION_FP64;
  gb2d_grid gg = {g.i_res, g.j_res, g.x_min, g.y_min, g.x_max, g.y_max};
  gb2d_params p = {f.water_density, f.air_density, f.surface_tension, f.advecting_field_variables->epsilon,
                   f.iteration_number_for_reinitialization, f.scaling_number_for_reinitialization, prec};
  gb2d_solve_opts o = {GB2D_SOLVER_MGPCG, prec, tolerance, 100000, 2};
  delete f.gpu_step;
  f.gpu_step = new GB2D_FLUID_STEP(gg, p, o, [s](int tid) { s->mt.Sync(tid); });
  gb2d_flow_params fl = {f.water_viscosity, f.air_viscosity, f.gravity.x, f.gravity.y, f.cfl_number,
                         f.viscosity_solver->use_delta_function_formulation ? 1 : 0};
  f.gpu_step->SetFlowParams(fl);
  for (int id = 0; id <= 5; ++id) f.gpu_step->Upload(id, field(s, id)->values);
  return 0;
}
int ref_gpu_download(void* h) {
  RefSim* s = static_cast<RefSim*>(h);
  if (!s->solver.gpu_step) return -1;
  for (int id = 0; id <= 5; ++id) s->solver.gpu_step->Download(id, field(s, id)->values);
  return 0;
}
#endif

int ref_pcg_info(void* h, int* iterations, double* residual) {
  LINEAR_SOLVER* ls = static_cast<RefSim*>(h)->solver.water_projection->poisson_solver.linear_solver;
  *iterations = ls->num_iteration;
  *residual = ls->residual;
  return 0;
}

}  // extern "C"
