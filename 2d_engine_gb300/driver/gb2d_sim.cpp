// gb2d_sim — headless replacement for SIMULATION_WORLD (SIMULATION_WORLD.h:86-307,
// 1094-1207 of ByungJoonLee/2D_Engine) for air/water scripts: it reads an unchanged .sim
// script, builds the state as InitializeFromScript does, and advances frames as
// AdvanceOneFrameThread does (curvature, dt = CFLOneTimeStep() * CFL, time step), all
// through the gb2d C ABI on one GPU.  Fields are written as .npy files (the reference's
// ghost-inclusive ARRAY_2D layout, rows = j).
//
//   gb2d_sim SCRIPT [--frames N] [--out DIR] [--every K] [--dry-run]
//
// Keys read (reference defaults where the script omits them):
//   SIMULATION_WORLD: dt (0.01), max_dt (100), CFL (0), last_frame,
//     FLUID_SOLVER_OPTIONS.air_water_simulation (must be true)
//   SIMULATION_WORLD.WORLD_DISCRETIZATION.AIR_WATER_SIMULATION: large_bubble / small_bubble
//     and GRID_STRUCTURE_2D_LARGE / _SMALL (base_grid_resolution, base_grid_min/max)
//   FLUID_SOLVER_UNIFORM.AIR_WATER_SIMULATION: water/air density (1), water (1) / air (0)
//     viscosity, surface_tension (1), gravity ((0,-9.8)), cfl_number (0.5),
//     iteration_number_for_reinitialization (10), scaling_number_for_reinitialization (5),
//     LEVELSET_ADVECTION.epsilon ((float)1e-6)
//   GB300 (a block the reference does not read): precision "fp64" | "mixed" ("mixed"),
//     solver_tolerance (relative residual, 1e-8), max_iteration (10000), viscosity (false:
//     the reference's air/water runs apply none), output_every (0: last frame only), and an
//     optional bubble_center / bubble_radius in place of the script's large/small bubble.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "gb2d.h"
#include "script.hpp"

namespace {

struct Config {
  double dt = 0.01, max_dt = 100, cfl = 0;
  int last_frame = 1000000;
  gb2d_grid grid = {0, 0, 0, 0, 0, 0};
  gb2d_params params = {};
  gb2d_flow_params flow = {};
  gb2d_solve_opts opts = {};
  double cx = 0, cy = 0, radius = 0;  // bubble: sqrt((x-cx)^2 + (y-cy)^2) - radius
  std::string bubble;
  int every = 0;
};

void die(const std::string& msg) {
  std::fprintf(stderr, "gb2d_sim: %s\n", msg.c_str());
  std::exit(1);
}

Config load(const std::string& path) {
  std::unique_ptr<gb2d_script::Block> root = gb2d_script::ReadScript(path);
  const gb2d_script::Block& world = root->FindBlock("SIMULATION_WORLD");
  Config c;
  c.dt = world.GetFloat("dt", 0.01);
  c.max_dt = world.GetFloat("max_dt", 100);
  c.cfl = world.GetFloat("CFL", 0);
  c.last_frame = world.GetInteger("last_frame", 1000000);
  if (!world.GetBoolean("fluid_solver", false) || !world.FindBlock("FLUID_SOLVER_OPTIONS").GetBoolean("air_water_simulation", false))
    die("only air/water fluid scripts are supported (fluid_solver and FLUID_SOLVER_OPTIONS.air_water_simulation)");
  const gb2d_script::Block& wd = world.FindBlock("WORLD_DISCRETIZATION").FindBlock("AIR_WATER_SIMULATION");
  const bool large = wd.GetBoolean("large_bubble", false), small = wd.GetBoolean("small_bubble", false);
  if (!large && !small) die("WORLD_DISCRETIZATION.AIR_WATER_SIMULATION needs large_bubble or small_bubble");
  const gb2d_script::Block& gb = wd.FindBlock(large ? "GRID_STRUCTURE_2D_LARGE" : "GRID_STRUCTURE_2D_SMALL");
  int ni = 0, nj = 0;
  gb.GetInt2("base_grid_resolution", ni, nj);
  double x0 = 0, y0 = 0, x1 = 0, y1 = 0;
  gb.GetVector2("base_grid_min", x0, y0);
  gb.GetVector2("base_grid_max", x1, y1);
  c.grid = {ni, nj, x0, y0, x1, y1};
  // SIMULATION_WORLD.h:408-425: the large bubble sqrt(x^2 + (y+0.5)^2) - 1/3, the small one
  // sqrt(x^2 + (y+0.005)^2) - 1/300
  if (large) {
    c.cx = 0, c.cy = -0.5, c.radius = 1.0 / 3.0, c.bubble = "large_bubble";
  } else {
    c.cx = 0, c.cy = -0.005, c.radius = 1.0 / 300.0, c.bubble = "small_bubble";
  }

  const gb2d_script::Block& fs = root->FindBlock("FLUID_SOLVER_UNIFORM").FindBlock("AIR_WATER_SIMULATION");
  c.params.water_density = fs.GetFloat("water_density", 1);
  c.params.air_density = fs.GetFloat("air_density", 1);
  c.params.surface_tension = fs.GetFloat("surface_tension", 1);
  c.params.weno_epsilon = fs.FindBlock("LEVELSET_ADVECTION").GetFloat("epsilon", (double)1e-6f);
  c.params.reinit_iterations = fs.GetInteger("iteration_number_for_reinitialization", 10);
  c.params.reinit_scaling = fs.GetInteger("scaling_number_for_reinitialization", 5);
  c.flow.water_viscosity = fs.GetFloat("water_viscosity", 1);
  c.flow.air_viscosity = fs.GetFloat("air_viscosity", 0);
  c.flow.gravity_x = 0;
  c.flow.gravity_y = -9.8;
  fs.GetVector2("gravity", c.flow.gravity_x, c.flow.gravity_y);
  c.flow.cfl_number = fs.GetFloat("cfl_number", 0.5);

  const gb2d_script::Block& g3 = root->FindBlock("GB300");
  const std::string prec = g3.GetString("precision", "mixed");
  if (prec != "mixed" && prec != "fp64") die("GB300.precision must be \"mixed\" or \"fp64\"");
  const int p = prec == "mixed" ? GB2D_PRECISION_MIXED : GB2D_PRECISION_FP64;
  c.params.advection_precision = p;
  c.flow.viscosity = g3.GetBoolean("viscosity", false) ? 1 : 0;
  c.opts.solver = GB2D_SOLVER_MGPCG;
  c.opts.precision = p;
  c.opts.tolerance = g3.GetFloat("solver_tolerance", 1e-8);
  c.opts.max_iterations = g3.GetInteger("max_iteration", 10000);
  c.opts.mg_smooth = 2;
  c.every = g3.GetInteger("output_every", 0);
  if (g3.Has("bubble_radius")) {
    g3.GetVector2("bubble_center", c.cx, c.cy);
    c.radius = g3.GetFloat("bubble_radius", c.radius);
    c.bubble = "bubble_center/bubble_radius";
  }
  return c;
}

// .npy version 1.0, little-endian float64, C order.
void write_npy(const std::string& path, const std::vector<double>& a, int rows, int cols) {
  std::string hdr = "{'descr': '<f8', 'fortran_order': False, 'shape': (" + std::to_string(rows) + ", " + std::to_string(cols) + "), }";
  size_t total = 10 + hdr.size() + 1;
  hdr.append((64 - total % 64) % 64, ' ');
  hdr += '\n';
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) die("cannot write " + path);
  const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
  const unsigned short len = (unsigned short)hdr.size();
  std::fwrite(magic, 1, 8, f);
  const unsigned char l2[2] = {(unsigned char)(len & 0xff), (unsigned char)(len >> 8)};
  std::fwrite(l2, 1, 2, f);
  std::fwrite(hdr.data(), 1, hdr.size(), f);
  std::fwrite(a.data(), sizeof(double), a.size(), f);
  std::fclose(f);
}

void check(gb2d_ctx* ctx, int rc, const char* what) {
  if (rc != GB2D_OK && rc != GB2D_ERR_MAX_ITERS)
    die(std::string(what) + " failed (" + std::to_string(rc) + "): " + (ctx ? gb2d_last_error(ctx) : "no context"));
}

void dump(gb2d_ctx* ctx, const Config& c, const std::string& out, int frame) {
  const struct {
    int field;
    const char* name;
  } fields[] = {{GB2D_FIELD_PHI, "phi"}, {GB2D_FIELD_U, "u"}, {GB2D_FIELD_V, "v"}, {GB2D_FIELD_P, "p"}};
  for (const auto& f : fields) {
    int ir = 0, jr = 0;
    check(ctx, gb2d_field_extent(&c.grid, f.field, &ir, &jr), "gb2d_field_extent");
    std::vector<double> a((size_t)ir * jr);
    check(ctx, gb2d_get_field(ctx, f.field, a.data()), "gb2d_get_field");
    char name[64];
    std::snprintf(name, sizeof name, "/%s_%06d.npy", f.name, frame);
    write_npy(out + name, a, jr, ir);
  }
}

}  // namespace

int main(int argc, char** argv) {
  std::string script, out = "gb2d_sim_out";
  int frames = -1, every = -1;
  bool dry = false;
  for (int k = 1; k < argc; ++k) {
    std::string a = argv[k];
    if (a == "--frames" && k + 1 < argc)
      frames = std::atoi(argv[++k]);
    else if (a == "--out" && k + 1 < argc)
      out = argv[++k];
    else if (a == "--every" && k + 1 < argc)
      every = std::atoi(argv[++k]);
    else if (a == "--dry-run")
      dry = true;
    else if (script.empty() && a[0] != '-')
      script = a;
    else
      die("usage: gb2d_sim SCRIPT [--frames N] [--out DIR] [--every K] [--dry-run]");
  }
  if (script.empty()) die("usage: gb2d_sim SCRIPT [--frames N] [--out DIR] [--every K] [--dry-run]");
  Config c;
  try {
    c = load(script);
  } catch (const std::exception& e) {
    die(e.what());
  }
  if (every >= 0) c.every = every;
  const int last = frames >= 0 ? frames : c.last_frame;
  if (dry) {
    std::printf(
        "{\"grid\": [%d, %d, %.17g, %.17g, %.17g, %.17g], \"dt\": %.17g, \"max_dt\": %.17g, \"CFL\": %.17g, "
        "\"last_frame\": %d, \"water_density\": %.17g, \"air_density\": %.17g, \"surface_tension\": %.17g, "
        "\"weno_epsilon\": %.17g, \"reinit_iterations\": %d, \"reinit_scaling\": %d, \"water_viscosity\": %.17g, "
        "\"air_viscosity\": %.17g, \"gravity\": [%.17g, %.17g], \"cfl_number\": %.17g, \"viscosity\": %d, "
        "\"precision\": %d, \"solver_tolerance\": %.17g, \"max_iteration\": %d, \"bubble\": [%.17g, %.17g, %.17g], "
        "\"bubble_source\": \"%s\", \"output_every\": %d}\n",
        c.grid.ni, c.grid.nj, c.grid.x_min, c.grid.y_min, c.grid.x_max, c.grid.y_max, c.dt, c.max_dt, c.cfl, c.last_frame,
        c.params.water_density, c.params.air_density, c.params.surface_tension, c.params.weno_epsilon,
        c.params.reinit_iterations, c.params.reinit_scaling, c.flow.water_viscosity, c.flow.air_viscosity, c.flow.gravity_x,
        c.flow.gravity_y, c.flow.cfl_number, c.flow.viscosity, c.opts.precision, c.opts.tolerance, c.opts.max_iterations, c.cx,
        c.cy, c.radius, c.bubble.c_str(), c.every);
    return 0;
  }

  gb2d_ctx* ctx = nullptr;
  check(nullptr, gb2d_create(&c.grid, &c.params, &ctx), "gb2d_create");
  check(ctx, gb2d_set_flow_params(ctx, &c.flow), "gb2d_set_flow_params");
  // Initial level set: interior from the bubble, ghosts copied from the second interior
  // line, corners at dx (the level set's initial fill, LEVELSET_2D.h:83).
  const int ni = c.grid.ni, nj = c.grid.nj, W = ni + 4;
  const double dx = (c.grid.x_max - c.grid.x_min) / (ni - 1), dy = (c.grid.y_max - c.grid.y_min) / (nj - 1);
  std::vector<double> phi((size_t)W * (nj + 4), dx);
  auto at = [&](int i, int j) -> double& { return phi[(size_t)(i + 2) + (size_t)(j + 2) * W]; };
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i < ni; ++i) {
      const double x = c.grid.x_min + i * dx, y = c.grid.y_min + j * dy;
      at(i, j) = std::sqrt((x - c.cx) * (x - c.cx) + (y - c.cy) * (y - c.cy)) - c.radius;
    }
  for (int j = 0; j < nj; ++j)
    for (int g = 1; g <= 2; ++g) at(-g, j) = at(1, j), at(ni - 1 + g, j) = at(ni - 2, j);
  for (int i = 0; i < ni; ++i)
    for (int g = 1; g <= 2; ++g) at(i, -g) = at(i, 1), at(i, nj - 1 + g) = at(i, nj - 2);
  check(ctx, gb2d_set_field(ctx, GB2D_FIELD_PHI, phi.data()), "gb2d_set_field");

  mkdir(out.c_str(), 0755);
  double dt = c.dt, accu = 0;
  int frame = 0;
  for (frame = 1; frame <= last; ++frame) {
    // SIMULATION_WORLD::AdvanceOneFrame / AdvanceOneFrameThread / DetermineTimeStep
    check(ctx, gb2d_curvature(ctx), "ComputeCurvatures");
    double cdt = 0, rates[4];
    check(ctx, gb2d_cfl_time_step(ctx, &cdt, rates), "CFLOneTimeStep");
    dt = (cdt == 0 ? dt : cdt) * c.cfl;
    accu += dt;
    if (accu > c.max_dt) {
      std::printf("frame %d: accumulated time %.6g exceeds max_dt %.6g; stopping\n", frame, accu, c.max_dt);
      break;
    }
    gb2d_solve_stats st = {};
    check(ctx, gb2d_advance_time_step(ctx, dt, &c.opts, &st), "AdvanceOneTimeStepThread");
    std::printf("frame %d  dt %.6e  time %.6e  max|u| %.4e  max|v| %.4e  cg %d  res %.2e  c_f %.4g g_f %.4g v_f %.4g s_f %.4g\n",
                frame, dt, accu, st.max_velocity_x, st.max_velocity_y, st.iterations, st.rel_residual, rates[0], rates[1], rates[2],
                rates[3]);
    if (c.every > 0 && frame % c.every == 0) dump(ctx, c, out, frame);
  }
  const int done = frame > last ? last : frame - 1;
  if (done > 0 && !(c.every > 0 && done % c.every == 0)) dump(ctx, c, out, done);
  gb2d_destroy(ctx);
  return 0;
}
