// The stages of SolveForRK around the projection (EULERIAN_FLUID_SOLVER_2D.h:1857-1879)
// and the velocity TVD-RK3 blends (:1753-1794): gravity, DetermineDensity, the
// explicit delta-function viscosity (VISCOSITY_2D.h:460-532) and the wall
// conditions, fused into one pass over the two MAC face grids; and the CFL time
// step (:3517-3637).
// Built with --fmad=false, in the reference's association order, like
// gb2d_exact.cu: the results are the reference's FP64 results bit for bit, except
// where the smeared Heaviside's sine (the only libm call) differs in the last ulp.
#include "gb2d_internal.cuh"
#include "gb2d_schemes.cuh"

namespace gb2d {

namespace {

// lo + (hi - lo) * H(phi): a smeared density or viscosity.  at0 / at1 are its
// values where H is 0 or 1, formed on the host with the same two operations.
struct Smear {
  double lo, d, at0, at1;
};
Smear make_smear(double lo, double hi) {
  Smear s;
  s.lo = lo;
  s.d = hi - lo;
  s.at0 = lo + s.d * 0.0;
  s.at1 = lo + s.d * 1.0;
  return s;
}

struct SmearF {
  float lo, d, at0, at1;
};

struct FlowArgs {
  int ni, nj;
  int grav, bc;        // add dt * gravity to every face; zero the wall faces' normal velocity
  double gx, gy;       // dt * gravity
  double dt, odx, ody;
  double eps, oe;      // smearing width 1.5 dx (EULERIAN_FLUID_SOLVER_2D.h:347) and its reciprocal
  Smear rho, mu;       // face density and viscosity
  double coef0, coef1; // dt * (1 / rho.at0), dt * (1 / rho.at1)
  double air, water;   // node densities of DetermineDensity
  // Non-null: the time step is read here when the kernel runs, and the dt-derived fields
  // above are formed from it as the host forms them (g_x, g_y: gravity; inv_rho0/1 = 1 / rho.at0/1).
  const double* dtp;
  double g_x, g_y, inv_rho0, inv_rho1;
  // FP32 viscous-flux path
  float odx_f, ody_f, eps_f, oe_f, dt_f, coef0_f, coef1_f;
  SmearF rho_f, mu_f;
};

__device__ __forceinline__ double smear(double l, const Smear& s, const FlowArgs& a) {
  if (lt_neg(l, a.eps)) return s.at0;
  if (gt_pos(l, a.eps)) return s.at1;
  return s.lo + s.d * heaviside_band(l, a.oe);
}

// dt / rho of a face: rho takes two values outside the band, whose quotients the
// host formed (FP64 divisions are scarce on this part).
__device__ __forceinline__ double face_coef(double l, const FlowArgs& a) {
  if (lt_neg(l, a.eps)) return a.coef0;
  if (gt_pos(l, a.eps)) return a.coef1;
  return a.dt * (1 / (a.rho.lo + a.rho.d * heaviside_band(l, a.oe)));
}

// FP32 forms for the viscous flux of the mixed path.
__device__ __forceinline__ float heaviside_band_f(float phi, float oe) {
  const float PI_REF = 3.141592f, opi = 1.0f / PI_REF;
  return 0.5f + phi * oe * 0.5f + 0.5f * opi * __sinf(PI_REF * phi * oe);
}
__device__ __forceinline__ float smear_f(float l, const SmearF& s, const FlowArgs& a) {
  if (l < -a.eps_f) return s.at0;
  if (l > a.eps_f) return s.at1;
  return s.lo + s.d * heaviside_band_f(l, a.oe_f);
}
__device__ __forceinline__ float face_coef_f(float l, const FlowArgs& a) {
  if (l < -a.eps_f) return a.coef0_f;
  if (l > a.eps_f) return a.coef1_f;
  return __fdividef(a.dt_f, a.rho_f.lo + a.rho_f.d * heaviside_band_f(l, a.oe_f));
}

// The dt-dependent fields of FlowArgs, as launch_flow forms them on the host.
__host__ __device__ __forceinline__ void with_time_step(FlowArgs& a, double dt) {
  a.gx = dt * a.g_x;
  a.gy = dt * a.g_y;
  a.dt = dt;
  a.coef0 = dt * a.inv_rho0;
  a.coef1 = dt * a.inv_rho1;
  a.dt_f = (float)dt;
  a.coef0_f = (float)a.coef0;
  a.coef1_f = (float)a.coef1;
}

// One pass over the (ni+1) x (nj+1) face index space: x-face (i, j), i <= ni,
// j < nj; y-face (i, j), i < ni, j <= nj; node (i, j) for the density.
//   VISC = false: gravity and wall conditions in place (u_out may equal u_in).
//   VISC = true:  ApplyViscosity from the copies temp_x / temp_y of the faces after
//                 gravity, whose values off the face grids are zero (the reference's
//                 freshly initialised temporaries), written to u_out / v_out.
//   MIXED (with VISC): the viscous flux in FP32 from FP64 velocity differences (the
//                 face values and the update stay FP64).
// density (ghost 2, may be null) receives DetermineDensity (:2162-2180): air where
// phi <= 0, water where phi > 0, unchanged for NaN.
template <bool VISC, bool MIXED>
__global__ void k_flow(const double* __restrict__ phi_a, const double* u_in_a, const double* v_in_a, double* u_out_a,
                       double* v_out_a, double* __restrict__ dens_a, FlowArgs a) {
  if (a.dtp) with_time_step(a, *a.dtp);
  const int ni = a.ni, nj = a.nj;
  const DField phi = dfield((double*)phi_a, 2, ni, nj);
  const DField ui = dfield((double*)u_in_a, 2, ni + 1, nj), vi = dfield((double*)v_in_a, 2, ni, nj + 1);
  const DField uo = dfield(u_out_a, 2, ni + 1, nj), vo = dfield(v_out_a, 2, ni, nj + 1);
  auto tu = [&](int i, int j) -> double {
    if (i < 0 || i > ni || j < 0 || j >= nj) return 0.0;
    const double w = GB_AT(ui, i, j);
    return a.grav ? w + a.gx : w;
  };
  auto tv = [&](int i, int j) -> double {
    if (i < 0 || i >= ni || j < 0 || j > nj) return 0.0;
    const double w = GB_AT(vi, i, j);
    return a.grav ? w + a.gy : w;
  };
  auto P = [&](int i, int j) -> double { return __ldg(&GB_AT(phi, i, j)); };
  // Face values without gravity: off the grids -gravity, so that differences of
  // these equal differences of the temporaries.
  auto ru = [&](int i, int j) -> double {
    if (i < 0 || i > ni || j < 0 || j >= nj) return a.grav ? -a.gx : 0.0;
    return GB_AT(ui, i, j);
  };
  auto rv = [&](int i, int j) -> double {
    if (i < 0 || i >= ni || j < 0 || j > nj) return a.grav ? -a.gy : 0.0;
    return GB_AT(vi, i, j);
  };
  auto Pf = [&](int i, int j) -> float { return narrow(__ldg(&GB_AT(phi, i, j))); };
  GB_FOR_IJ(i, j, ni + 1, nj + 1) {
    if (dens_a && i < ni && j < nj) {
      const double l = P(i, j);
      DField dn = dfield(dens_a, 2, ni, nj);
      if (lez(l))
        GB_AT(dn, i, j) = a.air;
      else if (gtz(l))
        GB_AT(dn, i, j) = a.water;
    }
    if (j < nj) {  // x-face between nodes (i-1, j) and (i, j)
      double w;
      if (VISC && MIXED) {
        const float pl = Pf(i - 1, j), pc = Pf(i, j);
        const float cu = 0.25f * (pl + pc + Pf(i - 1, j + 1) + Pf(i, j + 1));
        const float cd = 0.25f * (Pf(i - 1, j - 1) + Pf(i, j - 1) + pl + pc);
        const float mu_cu = smear_f(cu, a.mu_f, a), mu_cd = smear_f(cd, a.mu_f, a);
        const float mu_r = smear_f(pc, a.mu_f, a), mu_c = smear_f(pl, a.mu_f, a);
        const float coef = face_coef_f(0.5f * (pl + pc), a);
        const double u0 = ru(i, j);
        const float dxp = narrow(ru(i + 1, j) - u0), dxm = narrow(u0 - ru(i - 1, j));
        const float dyp = narrow(ru(i, j + 1) - u0), dym = narrow(u0 - ru(i, j - 1));
        const float dvu = narrow(rv(i, j + 1) - rv(i - 1, j + 1)), dvd = narrow(rv(i, j) - rv(i - 1, j));
        const float first = 2.0f * coef * a.odx_f * (mu_r * a.odx_f * dxp - mu_c * a.odx_f * dxm);
        const float second = coef * a.ody_f * (mu_cu * (a.ody_f * dyp + a.odx_f * dvu) - mu_cd * (a.ody_f * dym + a.odx_f * dvd));
        w = (a.grav ? u0 + a.gx : u0) + widen(first + second);
      } else if (VISC) {
        const double pl = P(i - 1, j), pc = P(i, j);
        const double half = 0.5 * (pl + pc);
        const double cu = 0.25 * (pl + pc + P(i - 1, j + 1) + P(i, j + 1));
        const double cd = 0.25 * (P(i - 1, j - 1) + P(i, j - 1) + pl + pc);
        const double mu_cu = smear(cu, a.mu, a), mu_cd = smear(cd, a.mu, a);
        const double mu_r = smear(pc, a.mu, a), mu_c = smear(pl, a.mu, a);
        const double coef = face_coef(half, a);
        const double t0 = tu(i, j);
        const double first = 2.0 * coef * a.odx * (mu_r * a.odx * (tu(i + 1, j) - t0) - mu_c * a.odx * (t0 - tu(i - 1, j)));
        const double second = coef * a.ody *
                               (mu_cu * (a.ody * (tu(i, j + 1) - t0) + a.odx * (tv(i, j + 1) - tv(i - 1, j + 1))) -
                                mu_cd * (a.ody * (t0 - tu(i, j - 1)) + a.odx * (tv(i, j) - tv(i - 1, j))));
        w = t0 + (first + second);
      } else {
        w = tu(i, j);
      }
      if (a.bc && (i == 0 || i == ni)) w = 0.0;
      GB_AT(uo, i, j) = w;
    }
    if (i < ni) {  // y-face between nodes (i, j-1) and (i, j)
      double w;
      if (VISC && MIXED) {
        const float pb = Pf(i, j - 1), pc = Pf(i, j);
        const float cu = 0.25f * (pb + Pf(i + 1, j - 1) + pc + Pf(i + 1, j));
        const float cl = 0.25f * (Pf(i - 1, j - 1) + pb + Pf(i - 1, j) + pc);
        const float mu_cu = smear_f(cu, a.mu_f, a), mu_cl = smear_f(cl, a.mu_f, a);
        const float mu_u = smear_f(pc, a.mu_f, a), mu_c = smear_f(pb, a.mu_f, a);
        const float coef = face_coef_f(0.5f * (pb + pc), a);
        const double v0 = rv(i, j);
        const float dyp = narrow(rv(i, j + 1) - v0), dym = narrow(v0 - rv(i, j - 1));
        const float dur = narrow(ru(i + 1, j) - ru(i + 1, j - 1)), dul = narrow(ru(i, j) - ru(i, j - 1));
        const float dxp = narrow(rv(i + 1, j) - v0), dxm = narrow(v0 - rv(i - 1, j));
        const float first = 2.0f * coef * a.ody_f * (mu_u * a.ody_f * dyp - mu_c * a.ody_f * dym);
        const float second = coef * a.odx_f * (mu_cu * (a.ody_f * dur + a.odx_f * dxp) - mu_cl * (a.ody_f * dul + a.odx_f * dxm));
        w = (a.grav ? v0 + a.gy : v0) + widen(first + second);
      } else if (VISC) {
        const double pb = P(i, j - 1), pc = P(i, j);
        const double half = 0.5 * (pb + pc);
        const double cu = 0.25 * (pb + P(i + 1, j - 1) + pc + P(i + 1, j));
        const double cl = 0.25 * (P(i - 1, j - 1) + pb + P(i - 1, j) + pc);
        const double mu_cu = smear(cu, a.mu, a), mu_cl = smear(cl, a.mu, a);
        const double mu_u = smear(pc, a.mu, a), mu_c = smear(pb, a.mu, a);
        const double coef = face_coef(half, a);
        const double t0 = tv(i, j);
        const double first = 2.0 * coef * a.ody * (mu_u * a.ody * (tv(i, j + 1) - t0) - mu_c * a.ody * (t0 - tv(i, j - 1)));
        const double second = coef * a.odx *
                              (mu_cu * (a.ody * (tu(i + 1, j) - tu(i + 1, j - 1)) + a.odx * (tv(i + 1, j) - t0)) -
                               mu_cl * (a.ody * (tu(i, j) - tu(i, j - 1)) + a.odx * (t0 - tv(i - 1, j))));
        w = t0 + (first + second);
      } else {
        w = tv(i, j);
      }
      if (a.bc && (j == 0 || j == nj)) w = 0.0;
      GB_AT(vo, i, j) = w;
    }
  }
}

// Velocity TVD-RK3 blend on every MAC face: w = c0 * keep + c1 * w.
__global__ void k_face_blend(const double* __restrict__ ku_a, double* __restrict__ u_a, const double* __restrict__ kv_a,
                             double* __restrict__ v_a, int ni, int nj, double c0, double c1) {
  const DField ku = dfield((double*)ku_a, 2, ni + 1, nj), u = dfield(u_a, 2, ni + 1, nj);
  const DField kv = dfield((double*)kv_a, 2, ni, nj + 1), v = dfield(v_a, 2, ni, nj + 1);
  GB_FOR_IJ(i, j, ni + 1, nj + 1) {
    if (j < nj) GB_AT(u, i, j) = c0 * GB_AT(ku, i, j) + c1 * GB_AT(u, i, j);
    if (i < ni) GB_AT(v, i, j) = c0 * GB_AT(kv, i, j) + c1 * GB_AT(v, i, j);
  }
}

// Largest |u|, |v| over the MAC grids and |kappa| over the nodes (CFLOneTimeStep's loops).
__global__ void k_cfl_max(const double* __restrict__ u_a, const double* __restrict__ v_a, const double* __restrict__ kappa,
                          int ni, int nj, Scalars* sc) {
  const DField u = dfield((double*)u_a, 2, ni + 1, nj), v = dfield((double*)v_a, 2, ni, nj + 1);
  unsigned long long mu = 0, mv = 0, mk = 0;
  GB_FOR_IJ(i, j, ni + 1, nj + 1) {
    if (j < nj) mu = abs_max_bits(GB_AT(u, i, j), mu);
    if (i < ni) mv = abs_max_bits(GB_AT(v, i, j), mv);
    if (i < ni && j < nj) mk = abs_max_bits(kappa[i + (size_t)j * ni], mk);
  }
  block_max_bits(mu, &sc->cfl_bits[0]);
  block_max_bits(mv, &sc->cfl_bits[1]);
  block_max_bits(mk, &sc->cfl_bits[2]);
}

struct CflArgs {
  double xs_odx, ys_ody;          // 1/dx of the x-face grid, 1/dy of the y-face grid
  double ody, odx2, ody2, dx, dy; // base grid
  double water_visc, air_visc, water_rho, air_rho, sigma, cfl_number;
};

// The rest of CFLOneTimeStep for air/water (EULERIAN_FLUID_SOLVER_2D.h:3562-3637),
// in the reference's order; one thread.
__global__ void k_cfl_final(CflArgs a, Scalars* sc) {
  const double u_max = __longlong_as_double((long long)sc->cfl_bits[0]);
  const double v_max = __longlong_as_double((long long)sc->cfl_bits[1]);
  const double k_max = __longlong_as_double((long long)sc->cfl_bits[2]);
  const double c_f = (u_max * a.xs_odx + v_max * a.ys_ody);
  const double g_f = sqrt(9.8 * a.ody);  // the constant 9.8, as the reference writes it
  const double rw = a.water_visc / a.water_rho, ra = a.air_visc / a.air_rho;
  const double v_f = (rw < ra ? ra : rw) * (2 * a.odx2 + 2 * a.ody2);
  const double rmin = a.water_rho > a.air_rho ? a.air_rho : a.water_rho;
  const double hmin = a.dy < a.dx ? a.dy : a.dx;
  const double s_f = sqrt(a.sigma * k_max / (rmin * (hmin * hmin)));
  const double CFL = 0.5 * (c_f + v_f + sqrt((c_f + v_f) * (c_f + v_f) + 4 * (g_f * g_f) + 4 * (s_f * s_f)));
  double dt = a.cfl_number / CFL;
  if (CFL == 0) dt = 0;
  sc->cfl[0] = dt;
  sc->cfl[1] = c_f;
  sc->cfl[2] = g_f;
  sc->cfl[3] = v_f;
  sc->cfl[4] = s_f;
}

// The frame's time step: DetermineTimeStep keeps the previous step when the CFL rate is
// zero (SIMULATION_WORLD.h:1201-1204), then the frame's CFL factor.
__global__ void k_frame_dt(Scalars* sc, double cfl) {
  double d = sc->cfl[0];
  if (d == 0) d = sc->dt_frame;
  sc->dt_frame = d * cfl;
}

}  // namespace

void launch_frame_dt(cudaStream_t s, gb2d_ctx* c, double cfl) {
  k_frame_dt<<<1, 1, 0, s>>>(c->sc, cfl);
  GB_LAUNCHED(1);
}

void launch_cfl(cudaStream_t s, gb2d_ctx* c) {
  const int ni = c->grid.ni, nj = c->grid.nj;
  cudaMemsetAsync(c->sc->cfl_bits, 0, sizeof(c->sc->cfl_bits), s);
  k_cfl_max<<<grid_ij(ni + 1, nj + 1), kThreads, 0, s>>>(c->u, c->v, c->kappa, ni, nj, c->sc);
  CflArgs a;
  a.xs_odx = c->xs.odx;
  a.ys_ody = c->ys.ody;
  a.ody = c->base.ody;
  a.odx2 = c->base.odx2;
  a.ody2 = c->base.ody2;
  a.dx = c->base.dx;
  a.dy = c->base.dy;
  a.water_visc = c->flow.water_viscosity;
  a.air_visc = c->flow.air_viscosity;
  a.water_rho = c->prm.water_density;
  a.air_rho = c->prm.air_density;
  a.sigma = c->prm.surface_tension;
  a.cfl_number = c->flow.cfl_number;
  k_cfl_final<<<1, 1, 0, s>>>(a, c->sc);
  GB_LAUNCHED(2);
}

void launch_flow(cudaStream_t s, gb2d_ctx* c, double dt, int grav, int visc, int bc, double* density) {
  const int ni = c->grid.ni, nj = c->grid.nj;
  FlowArgs a;
  a.ni = ni;
  a.nj = nj;
  a.grav = grav;
  a.bc = bc;
  a.g_x = c->flow.gravity_x;
  a.g_y = c->flow.gravity_y;
  a.odx = c->base.odx;
  a.ody = c->base.ody;
  a.eps = 1.5 * c->base.dx;
  a.oe = 1.0 / a.eps;
  a.rho = make_smear(c->prm.air_density, c->prm.water_density);
  a.mu = make_smear(c->flow.air_viscosity, c->flow.water_viscosity);
  a.inv_rho0 = 1 / a.rho.at0;
  a.inv_rho1 = 1 / a.rho.at1;
  a.dtp = c->dt_dev;
  with_time_step(a, dt);
  a.air = c->prm.air_density;
  a.water = c->prm.water_density;
  a.odx_f = (float)a.odx;
  a.ody_f = (float)a.ody;
  a.eps_f = (float)a.eps;
  a.oe_f = (float)a.oe;
  a.rho_f = SmearF{(float)a.rho.lo, (float)a.rho.d, (float)a.rho.at0, (float)a.rho.at1};
  a.mu_f = SmearF{(float)a.mu.lo, (float)a.mu.d, (float)a.mu.at0, (float)a.mu.at1};
  const double* phi = c->phi_buf[c->phi_cur];
  const bool mixed = c->prm.advection_precision == GB2D_PRECISION_MIXED;
  if (visc) {
    if (mixed)
      k_flow<true, true><<<grid_ij(ni + 1, nj + 1), kThreads, 0, s>>>(phi, c->u, c->v, c->u_alt, c->v_alt, density, a);
    else
      k_flow<true, false><<<grid_ij(ni + 1, nj + 1), kThreads, 0, s>>>(phi, c->u, c->v, c->u_alt, c->v_alt, density, a);
    double* t = c->u;
    c->u = c->u_alt;
    c->u_alt = t;
    t = c->v;
    c->v = c->v_alt;
    c->v_alt = t;
  } else {
    k_flow<false, false><<<grid_ij(ni + 1, nj + 1), kThreads, 0, s>>>(phi, c->u, c->v, c->u, c->v, density, a);
  }
  GB_LAUNCHED(1);
}

void launch_face_blend(cudaStream_t s, gb2d_ctx* c, double c0, double c1) {
  const int ni = c->grid.ni, nj = c->grid.nj;
  k_face_blend<<<grid_ij(ni + 1, nj + 1), kThreads, 0, s>>>(c->u_keep, c->u, c->v_keep, c->v, ni, nj, c0, c1);
  GB_LAUNCHED(1);
}

}  // namespace gb2d
