/*
 * gb2d_oracle.c — CPU restatement of the reference hot path.  TEST INFRASTRUCTURE
 * ONLY (the checker, never the product): see gb2d_oracle.h.
 *
 * Each function names the reference file:line it restates.  Expressions keep
 * the reference's association order so that, built with -ffp-contract=off, the
 * results are bit-identical to the reference's own FP64 output (checked against
 * tests/golden/ fixtures generated from the reference build in oracle/ref/).
 */
#include "gb2d_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* Grid spacing exactly as GRID_STRUCTURE_2D::Initialize (GRID_STRUCTURE_2D.h:88-123). */
typedef struct {
  double dx, dy, odx, ody, o2dx, o2dy, odx2, ody2;
} space_t;

static space_t make_space(int ires, int jres, double x_min, double y_min, double x_max, double y_max) {
  space_t s;
  double diff_x = x_max - x_min, diff_y = y_max - y_min;
  s.dx = diff_x / (ires - 1);
  s.dy = diff_y / (jres - 1);
  double two_dx = 2 * s.dx, two_dy = 2 * s.dy;
  double dx2 = s.dx * s.dx, dy2 = s.dy * s.dy;
  s.odx = 1.0 / s.dx;
  s.ody = 1.0 / s.dy;
  s.o2dx = 1.0 / two_dx;
  s.o2dy = 1.0 / two_dy;
  s.odx2 = 1.0 / dx2;
  s.ody2 = 1.0 / dy2;
  return s;
}
static space_t base_space(const or_grid* g) { return make_space(g->ni, g->nj, g->x_min, g->y_min, g->x_max, g->y_max); }
/* MAC face grids (EULERIAN_FLUID_SOLVER_2D.h:355-363). */
static space_t xface_space(const or_grid* g) {
  space_t b = base_space(g);
  return make_space(g->ni + 1, g->nj, g->x_min - 0.5 * b.dx, g->y_min, g->x_max + 0.5 * b.dx, g->y_max);
}
static space_t yface_space(const or_grid* g) {
  space_t b = base_space(g);
  return make_space(g->ni, g->nj + 1, g->x_min, g->y_min - 0.5 * b.dy, g->x_max, g->y_max + 0.5 * b.dy);
}

/* Ghost-inclusive field view. */
typedef struct {
  double* a;
  int g, nI, nJ, ld;
} fld;
static fld F(double* a, int g, int nI, int nJ) {
  fld f = {a, g, nI, nJ, nI + 2 * g};
  return f;
}
#define AT(f, i, j) ((f).a[((i) + (f).g) + (size_t)((j) + (f).g) * (f).ld])

/* ------------------------------------------------------------------------- */
/* a7: FIELD_STRUCTURE_2D::FillGhostCellsFrom (FIELD_STRUCTURE_2D.h:374-449):
 * interior copied; every ghost layer copies the SECOND interior line
 * (i_start+1, i_end-1, ...); corners are left untouched. */
void or_fill_ghost_copy(double* dst_a, int gd, const double* src_a, int gs, int nI, int nJ, int g) {
  fld d = F(dst_a, gd, nI, nJ), s = F((double*)src_a, gs, nI, nJ);
  for (int j = 0; j < nJ; ++j)
    for (int i = 0; i < nI; ++i) AT(d, i, j) = AT(s, i, j);
  for (int j = 0; j < nJ; ++j)
    for (int i = -g; i <= -1; ++i) AT(d, i, j) = AT(s, 1, j);
  for (int j = 0; j < nJ; ++j)
    for (int i = nI; i <= nI - 1 + g; ++i) AT(d, i, j) = AT(s, nI - 2, j);
  for (int i = 0; i < nI; ++i)
    for (int j = nJ; j <= nJ - 1 + g; ++j) AT(d, i, j) = AT(s, i, nJ - 2);
  for (int i = 0; i < nI; ++i)
    for (int j = -g; j <= -1; ++j) AT(d, i, j) = AT(s, i, 1);
}

/* a7: FillGhostCellsContinuousDerivativesFrom(phi, true, thread_id) applied to the
 * field itself (FIELD_STRUCTURE_2D.h:641-716): linear extrapolation 2f(i+1)-f(i+2).
 * Left and bottom faces run outermost layer first, so the outer layer reads the
 * previous value of the inner one; right and top run innermost first. */
void or_fill_ghost_extrapolate(double* a, int g, int nI, int nJ) {
  fld f = F(a, g, nI, nJ);
  for (int j = 0; j < nJ; ++j)
    for (int i = -g; i <= -1; ++i) AT(f, i, j) = 2.0 * AT(f, i + 1, j) - AT(f, i + 2, j);
  for (int j = 0; j < nJ; ++j)
    for (int i = nI; i <= nI - 1 + g; ++i) AT(f, i, j) = 2.0 * AT(f, i - 1, j) - AT(f, i - 2, j);
  for (int i = 0; i < nI; ++i)
    for (int j = nJ; j <= nJ - 1 + g; ++j) AT(f, i, j) = 2.0 * AT(f, i, j - 1) - AT(f, i, j - 2);
  for (int i = 0; i < nI; ++i)
    for (int j = -g; j <= -1; ++j) AT(f, i, j) = 2.0 * AT(f, i, j + 1) - AT(f, i, j + 2);
}

/* ------------------------------------------------------------------------- */
/* WENO5 one-sided derivative from five first differences a1..a5
 * (ADVECTION_METHOD_2D.h:545-619): smoothness, weights 0.1/0.6/0.3 over
 * (eps+beta)^2, and the three third-order candidate stencils. */
static double weno5_side(double a1, double a2, double a3, double a4, double a5, double eps) {
  const double c13 = 13.0 / 12.0;
  double A1 = a1 - 2 * a2 + a3, B1 = a1 - 4 * a2 + 3 * a3;
  double A2 = a2 - 2 * a3 + a4, B2 = a2 - a4;
  double A3 = a3 - 2 * a4 + a5, B3 = 3 * a3 - 4 * a4 + a5;
  double s1 = c13 * A1 * A1 + 0.25 * B1 * B1;
  double s2 = c13 * A2 * A2 + 0.25 * B2 * B2;
  double s3 = c13 * A3 * A3 + 0.25 * B3 * B3;
  double al1 = (1.0 / 10.0) / ((eps + s1) * (eps + s1));
  double al2 = (6.0 / 10.0) / ((eps + s2) * (eps + s2));
  double al3 = (3.0 / 10.0) / ((eps + s3) * (eps + s3));
  double sum = al1 + al2 + al3;
  double w1 = al1 / sum, w2 = al2 / sum, w3 = al3 / sum;
  const double cm16 = (-1.0) / 6.0;
  return w1 * (a1 / 3.0 - a2 * 7.0 / 6.0 + a3 * 11.0 / 6.0) + w2 * (a2 * cm16 + a3 * 5.0 / 6.0 + a4 / 3.0) +
         w3 * (a3 / 3.0 + a4 * 5.0 / 6.0 - a5 / 6.0);
}

/* q[0..6] = values at offsets -3..+3 along one axis; o = 1/spacing.
 * Minus side uses differences d0..d4, plus side d5..d1 (ADVECTION_METHOD_2D.h:521-543). */
static void weno5_pair(const double q[7], double o, double eps, double* dm, double* dp) {
  double d[6];
  for (int k = 0; k < 6; ++k) d[k] = o * (q[k + 1] - q[k]);
  *dm = weno5_side(d[0], d[1], d[2], d[3], d[4], eps);
  *dp = weno5_side(d[5], d[4], d[3], d[2], d[1], eps);
}

static void gather_x(const fld* f, int i, int j, double q[7]) {
  for (int k = 0; k < 7; ++k) q[k] = AT(*f, i - 3 + k, j);
}
static void gather_y(const fld* f, int i, int j, double q[7]) {
  for (int k = 0; k < 7; ++k) q[k] = AT(*f, i, j - 3 + k);
}

/* a1: ADVECTION_METHOD_2D<T>::WENO5th(..., MT, tid) for a node-grid scalar
 * (ADVECTION_METHOD_2D.h:508-663).  ghost = scratch copy with ghost width 3. */
static void weno5_sweep(const or_grid* gr, double eps, fld* phi, fld* ghost, const fld* ua, const fld* va, double dt) {
  space_t s = base_space(gr);
  or_fill_ghost_copy(ghost->a, 3, phi->a, 2, gr->ni, gr->nj, 3);
  double q[7];
  for (int j = 0; j < gr->nj; ++j)
    for (int i = 0; i < gr->ni; ++i) {
      double mx, px, my, py;
      gather_x(ghost, i, j, q);
      weno5_pair(q, s.odx, eps, &mx, &px);
      gather_y(ghost, i, j, q);
      weno5_pair(q, s.ody, eps, &my, &py);
      double u = (AT(*ua, i + 1, j) + AT(*ua, i, j)) * 0.5;
      double v = (AT(*va, i, j + 1) + AT(*va, i, j)) * 0.5;
      double fx = u > 0 ? mx : px;
      double fy = v > 0 ? my : py;
      AT(*phi, i, j) = AT(*phi, i, j) - dt * (u * fx + v * fy);
    }
}

/* a2: WENO5thReinitialization (ADVECTION_METHOD_2D.h:1401-1658): Godunov
 * selection of the one-sided WENO derivatives, phi <- phi - dtau S (|grad phi| - 1).
 * Selection codes: 0 = minus side, 1 = plus side, 2 = no contribution. */
static void reinit_sweep(const or_grid* gr, double eps, fld* phi, fld* ghost, const double* S, double dtau) {
  space_t s = base_space(gr);
  or_fill_ghost_copy(ghost->a, 3, phi->a, 2, gr->ni, gr->nj, 3);
  double q[7];
  for (int j = 0; j < gr->nj; ++j)
    for (int i = 0; i < gr->ni; ++i) {
      double mx, px, my, py;
      gather_x(ghost, i, j, q);
      weno5_pair(q, s.odx, eps, &mx, &px);
      gather_y(ghost, i, j, q);
      weno5_pair(q, s.ody, eps, &my, &py);
      double sg = S[i + (size_t)j * gr->ni];
      double smx = sg * mx, spx = sg * px, smy = sg * my, spy = sg * py;
      int xs, ys;
      if (spx >= 0 && smx >= 0)
        xs = 0;
      else if (spx <= 0 && smx <= 0)
        xs = 1;
      else if (spx > 0 && smx < 0)
        xs = 2;
      else if (spx < 0 && smx > 0) {
        double sss = sg * (fabs(px) - fabs(mx)) / (px - mx);
        if (sss > 0)
          xs = 0;
        else if (sss < 0)
          xs = 1;
        else
          continue; /* sss == 0 or NaN: the reference leaves phi unchanged */
      } else
        continue;
      if (spy >= 0 && smy >= 0)
        ys = 0;
      else if (spy <= 0 && smy <= 0)
        ys = 1;
      else if (spy > 0 && smy < 0)
        ys = 2;
      else if (spy < 0 && smy > 0) {
        double ss = sg * (fabs(py) - fabs(my)) / (py - my);
        ys = (ss > 0) ? 0 : 1;
      } else
        continue;
      double gx = xs == 0 ? mx : px, gy = ys == 0 ? my : py;
      double h;
      if (xs != 2 && ys != 2)
        h = sqrt(gx * gx + gy * gy) - 1;
      else if (xs != 2)
        h = sqrt(gx * gx) - 1;
      else if (ys != 2)
        h = sqrt(gy * gy) - 1;
      else
        h = (-1);
      AT(*phi, i, j) = AT(*phi, i, j) - dtau * sg * h;
    }
}

static double* zalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

/* a1+a5: EULERIAN_FLUID_SOLVER_2D::Levelset_Advection(dt, tid) (:1896-2045) ->
 * ADVECTION_2D::Solve_Levelset (ADVECTION_2D.cpp:166-201) -> WENO5th, then
 * FillGhostCellsContinuousDerivativesFrom(phi, true, tid).  ComputeNormals()
 * at its start does not feed phi. */
int or_levelset_advection(const or_grid* gr, const or_params* pr, double* phi_a, const double* ua_a, const double* va_a, double dt) {
  if (!gr || !pr || !phi_a || !ua_a || !va_a || gr->ni < 4 || gr->nj < 4) return OR_BAD_ARG;
  int ni = gr->ni, nj = gr->nj;
  double* ghost_a = zalloc((size_t)(ni + 6) * (nj + 6));
  if (!ghost_a) return OR_NO_MEMORY;
  fld phi = F(phi_a, 2, ni, nj), ghost = F(ghost_a, 3, ni, nj);
  fld ua = F((double*)ua_a, 3, ni + 1, nj), va = F((double*)va_a, 3, ni, nj + 1);
  weno5_sweep(gr, pr->weno_epsilon, &phi, &ghost, &ua, &va, dt);
  or_fill_ghost_extrapolate(phi_a, 2, ni, nj);
  free(ghost_a);
  return OR_OK;
}

/* a6: EULERIAN_FLUID_SOLVER_2D::Reinitialization(dt, tid) (:2402-2445):
 * fictitious dt = dx / scaling, S from the current phi, then the sweeps. */
int or_reinitialization(const or_grid* gr, const or_params* pr, double* phi_a) {
  if (!gr || !pr || !phi_a || gr->ni < 4 || gr->nj < 4) return OR_BAD_ARG;
  int ni = gr->ni, nj = gr->nj;
  space_t s = base_space(gr);
  double dtau = s.dx / (double)pr->reinit_scaling;
  double* ghost_a = zalloc((size_t)(ni + 6) * (nj + 6));
  double* S = zalloc((size_t)ni * nj);
  if (!ghost_a || !S) {
    free(ghost_a);
    free(S);
    return OR_NO_MEMORY;
  }
  fld phi = F(phi_a, 2, ni, nj), ghost = F(ghost_a, 3, ni, nj);
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i < ni; ++i) {
      double p = AT(phi, i, j);
      S[i + (size_t)j * ni] = p / sqrt(p * p + s.dx * s.dx);
    }
  for (int it = 0; it < pr->reinit_iterations; ++it) reinit_sweep(gr, pr->weno_epsilon, &phi, &ghost, S, dtau);
  free(ghost_a);
  free(S);
  return OR_OK;
}

/* a4: level-set TVD-RK3 and reinit TVD-RK3 of AdvanceOneTimeStepThread
 * (EULERIAN_FLUID_SOLVER_2D.h:1694-1741): Shu-Osher blends on the interior only. */
int or_levelset_rk3(const or_grid* gr, const or_params* pr, double* phi_a, const double* ua, const double* va, double dt) {
  if (!gr || !pr || !phi_a) return OR_BAD_ARG;
  int ni = gr->ni, nj = gr->nj, rc;
  double* t = zalloc((size_t)ni * nj);
  if (!t) return OR_NO_MEMORY;
  fld phi = F(phi_a, 2, ni, nj);
#define SAVE()                                     \
  for (int j = 0; j < nj; ++j)                     \
    for (int i = 0; i < ni; ++i) t[i + (size_t)j * ni] = AT(phi, i, j);
#define BLEND(c0, c1)                              \
  for (int j = 0; j < nj; ++j)                     \
    for (int i = 0; i < ni; ++i) AT(phi, i, j) = (c0) * t[i + (size_t)j * ni] + (c1) * AT(phi, i, j);
  SAVE();
  if ((rc = or_levelset_advection(gr, pr, phi_a, ua, va, dt))) goto out;
  if ((rc = or_levelset_advection(gr, pr, phi_a, ua, va, dt))) goto out;
  BLEND(0.75, 0.25);
  if ((rc = or_levelset_advection(gr, pr, phi_a, ua, va, dt))) goto out;
  BLEND(1 / 3.0, 2 / 3.0);
  SAVE();
  if ((rc = or_reinitialization(gr, pr, phi_a))) goto out;
  if ((rc = or_reinitialization(gr, pr, phi_a))) goto out;
  BLEND(0.75, 0.25);
  if ((rc = or_reinitialization(gr, pr, phi_a))) goto out;
  BLEND(1 / 3.0, 2 / 3.0);
#undef SAVE
#undef BLEND
out:
  free(t);
  return rc;
}

/* ------------------------------------------------------------------------- */
/* a3: ENO3rd (ADVECTION_METHOD_2D.h:2038-2231): third-order ENO one-sided
 * derivatives by divided-difference selection. */
static void eno3_pair(const double q[7], double o, double o2, double o3, double h, double* dm, double* dp) {
  double d1n3 = o * (q[1] - q[0]), d1n2 = o * (q[2] - q[1]), d1n1 = o * (q[3] - q[2]);
  double d10 = o * (q[4] - q[3]), d1p1 = o * (q[5] - q[4]), d1p2 = o * (q[6] - q[5]);
  double d2n2 = o2 * (d1n2 - d1n3), d2n1 = o2 * (d1n1 - d1n2), d20 = o2 * (d10 - d1n1);
  double d2p1 = o2 * (d1p1 - d10), d2p2 = o2 * (d1p2 - d1p1);
  double d3n2 = o3 * (d2n1 - d2n2), d3n1 = o3 * (d20 - d2n1), d30 = o3 * (d2p1 - d20), d3p1 = o3 * (d2p2 - d2p1);
  if (fabs(d2n1) <= fabs(d20)) {
    if (fabs(d3n2) <= fabs(d3n1))
      *dm = d1n1 + d2n1 * h + 2 * d3n2 * h * h;
    else
      *dm = d1n1 + d2n1 * h + 2 * d3n1 * h * h;
  } else {
    if (fabs(d3n1) <= fabs(d30))
      *dm = d1n1 + d20 * h - d3n1 * h * h;
    else
      *dm = d1n1 + d20 * h - d30 * h * h;
  }
  if (fabs(d20) <= fabs(d2p1)) {
    if (fabs(d3n1) <= fabs(d30))
      *dp = d10 - d20 * h - d3n1 * h * h;
    else
      *dp = d10 - d20 * h - d30 * h * h;
  } else {
    if (fabs(d30) <= fabs(d3p1))
      *dp = d10 - d2p1 * h + 2 * d30 * h * h;
    else
      *dp = d10 - d2p1 * h + 2 * d3p1 * h * h;
  }
}

/* One ENO3rd call on a MAC component.  comp 0: x-faces (rho = u), 1: y-faces. */
static void eno3_component(const or_grid* gr, int comp, fld* rho, fld* ghost, const fld* ua, const fld* va, double dt) {
  space_t s = comp == 0 ? xface_space(gr) : yface_space(gr);
  double o3x = s.odx / 3, o3y = s.ody / 3;
  int nI = rho->nI, nJ = rho->nJ;
  or_fill_ghost_copy(ghost->a, 3, rho->a, 2, nI, nJ, 3);
  double q[7];
  for (int j = 0; j < nJ; ++j)
    for (int i = 0; i < nI; ++i) {
      double mx, px, my, py, u, v;
      gather_x(ghost, i, j, q);
      eno3_pair(q, s.odx, s.o2dx, o3x, s.dx, &mx, &px);
      gather_y(ghost, i, j, q);
      eno3_pair(q, s.ody, s.o2dy, o3y, s.dy, &my, &py);
      if (comp == 0) {
        u = AT(*ua, i, j);
        v = (AT(*va, i, j) + AT(*va, i, j + 1) + AT(*va, i - 1, j) + AT(*va, i - 1, j + 1)) * 0.25;
      } else {
        u = (AT(*ua, i, j - 1) + AT(*ua, i + 1, j - 1) + AT(*ua, i, j) + AT(*ua, i + 1, j)) * 0.25;
        v = AT(*va, i, j);
      }
      double fx = u > 0 ? mx : px;
      double fy = v > 0 ? my : py;
      AT(*rho, i, j) = AT(*rho, i, j) - dt * (u * fx + v * fy);
    }
}

/* ADVECTION_2D::Solve_Velocity(dt, tid) with use_3rd_eno_v (ADVECTION_2D.cpp:83-122):
 * refresh both advecting copies, ENO3 on u (its own refreshed copy advects it),
 * then on v, whose advecting u is the pre-update copy. */
int or_velocity_advection(const or_grid* gr, const or_params* pr, double* u_a, double* v_a, double* ua_a, double* va_a, double dt) {
  (void)pr;
  if (!gr || !u_a || !v_a || !ua_a || !va_a || gr->ni < 4 || gr->nj < 4) return OR_BAD_ARG;
  int ni = gr->ni, nj = gr->nj;
  fld u = F(u_a, 2, ni + 1, nj), v = F(v_a, 2, ni, nj + 1);
  fld ua = F(ua_a, 3, ni + 1, nj), va = F(va_a, 3, ni, nj + 1);
  or_fill_ghost_copy(ua_a, 3, u_a, 2, ni + 1, nj, 3);
  or_fill_ghost_copy(va_a, 3, v_a, 2, ni, nj + 1, 3);
  eno3_component(gr, 0, &u, &ua, &ua, &va, dt);
  eno3_component(gr, 1, &v, &va, &ua, &va, dt);
  return OR_OK;
}

/* ------------------------------------------------------------------------- */
/* a8: LEVELSET_2D::ComputeCurvaturesThread with curvature_by_levelset
 * (LEVELSET_2D.h:898-990): ghost extrapolation of phi, central differences,
 * kappa = -(px^2 pyy - 2 px py pxy + py^2 pxx)/|grad phi|^3 clamped to +-1/min(dx,dy). */
int or_curvature(const or_grid* gr, double* phi_a, double* kappa) {
  if (!gr || !phi_a || !kappa) return OR_BAD_ARG;
  int ni = gr->ni, nj = gr->nj;
  space_t s = base_space(gr);
  double tol = 1.0 / (s.dx < s.dy ? s.dx : s.dy);
  or_fill_ghost_extrapolate(phi_a, 2, ni, nj);
  fld phi = F(phi_a, 2, ni, nj);
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i < ni; ++i) {
      double px = (AT(phi, i + 1, j) - AT(phi, i - 1, j)) * s.o2dx;
      double py = (AT(phi, i, j + 1) - AT(phi, i, j - 1)) * s.o2dy;
      double pxx = (AT(phi, i + 1, j) - 2 * AT(phi, i, j) + AT(phi, i - 1, j)) * s.odx2;
      double pyy = (AT(phi, i, j + 1) - 2 * AT(phi, i, j) + AT(phi, i, j - 1)) * s.ody2;
      double pxy = (AT(phi, i + 1, j + 1) - AT(phi, i + 1, j - 1) - AT(phi, i - 1, j + 1) + AT(phi, i - 1, j - 1)) * s.o2dx * s.o2dy;
      double mag = sqrt(px * px + py * py);
      double deno = mag * mag * mag;
      double curv;
      if (deno != 0) {
        double od = 1.0 / deno;
        curv = -(px * px * pyy - 2.0 * px * py * pxy + py * py * pxx) * od;
      } else {
        px = (AT(phi, i + 1, j) - AT(phi, i, j)) * s.odx;
        py = (AT(phi, i, j + 1) - AT(phi, i, j)) * s.ody;
        mag = sqrt(px * px + py * py);
        deno = mag * mag * mag;
        if (deno == 0) return OR_ZERO_GRADIENT; /* the reference exits here (LEVELSET_2D.h:869-873) */
        double od = 1.0 / deno;
        curv = -(px * px * pyy - 2.0 * px * py * pxy + py * py * pxx) * od;
      }
      double* k = &kappa[i + (size_t)j * ni];
      if (fabs(curv) <= tol)
        *k = curv;
      else if (curv > tol)
        *k = tol;
      else if (curv < -tol)
        *k = -tol;
    }
  return OR_OK;
}

/* ------------------------------------------------------------------------- */
/* Variable-coefficient face weight of POISSON_SOLVER.cpp:743-746 between node c
 * and its neighbour n (v = 1/rho): v_c v_n (|phi_n|+|phi_c|) / (v_c|phi_n| + v_n|phi_c|).
 * The expression is symmetric in IEEE arithmetic, so one value per face serves
 * both rows. */
static double face_beta(double vc, double vn, double pc, double pn) {
  return vc * vn * (fabs(pn) + fabs(pc)) / (vc * fabs(pn) + vn * fabs(pc));
}

/* a9+a10: DetermineProjectionDensity/DetermineDivergence/jump (PROJECTION_2D.h:323-478,
 * 814-835) and BuildLinearSystemNodeJumpConditionVaribleCoefficient
 * (POISSON_SOLVER.cpp:714-976) with Neumann walls (PROJECTION_2D.h:940-971).
 * The derivative-jump terms b_l.. vanish because jc_on_derivative is zeroed
 * (PROJECTION_2D.h:501-504), so they are not formed. */
int or_poisson_assemble(const or_grid* gr, const or_params* pr, const double* phi_a, const double* u_a, const double* v_a, const double* kappa, double dt,
                        double* bx, double* by, double* diag, double* rhs) {
  if (!gr || !pr || !phi_a || !u_a || !v_a || !kappa || !bx || !by || !diag || !rhs) return OR_BAD_ARG;
  int ni = gr->ni, nj = gr->nj;
  space_t s = base_space(gr);
  fld phi = F((double*)phi_a, 2, ni, nj);
  fld u = F((double*)u_a, 2, ni + 1, nj), v = F((double*)v_a, 2, ni, nj + 1);
  double* vv_a = zalloc((size_t)(ni + 4) * (nj + 4)); /* 1/rho, ghost 2 */
  double* jc_a = zalloc((size_t)(ni + 2) * (nj + 2)); /* sigma*kappa, ghost 1 (ghosts stay 0) */
  double* rho = zalloc((size_t)ni * nj);
  if (!vv_a || !jc_a || !rho) {
    free(vv_a);
    free(jc_a);
    free(rho);
    return OR_NO_MEMORY;
  }
  fld vv = F(vv_a, 2, ni, nj), jc = F(jc_a, 1, ni, nj);
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i < ni; ++i) {
      double p = AT(phi, i, j);
      double r = 1.0;
      if (p <= 0)
        r = pr->air_density;
      else if (p > 0)
        r = pr->water_density;
      rho[i + (size_t)j * ni] = r;
      AT(vv, i, j) = 1.0 / r; /* POISSON_SOLVER.cpp:131-136 */
      AT(jc, i, j) = pr->surface_tension * kappa[i + (size_t)j * ni];
    }
  or_fill_ghost_copy(vv_a, 2, vv_a, 2, ni, nj, 2);
  /* Faces: bx[i + j*(ni+1)] between nodes (i-1, j) and (i, j); by[i + j*ni] between (i, j-1) and (i, j). */
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i <= ni; ++i) bx[i + (size_t)j * (ni + 1)] = face_beta(AT(vv, i, j), AT(vv, i - 1, j), AT(phi, i, j), AT(phi, i - 1, j));
  for (int j = 0; j <= nj; ++j)
    for (int i = 0; i < ni; ++i) by[i + (size_t)j * ni] = face_beta(AT(vv, i, j), AT(vv, i, j - 1), AT(phi, i, j), AT(phi, i, j - 1));
  double inv_dxdx = 1.0 / (s.dx * s.dx);
  double one_over_dt = 1.0 / dt;
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i < ni; ++i) {
      double bl = bx[i + (size_t)j * (ni + 1)], br = bx[i + 1 + (size_t)j * (ni + 1)];
      double bb = by[i + (size_t)j * ni], bt = by[i + (size_t)(j + 1) * ni];
      double coef = 0;
      if (i > 0) coef += bl;
      if (i < ni - 1) coef += br;
      if (j > 0) coef += bb;
      if (j < nj - 1) coef += bt;
      if (i == 0 && j == 0) { /* Neumann arms of the first cell pin the null space (POISSON_SOLVER.cpp:789-806) */
        if (i - 1 < 0) coef += bl;
        if (i + 1 > ni - 1) coef += br;
        if (j - 1 < 0) coef += bb;
        if (j + 1 > nj - 1) coef += bt;
      }
      if (coef == 0) coef = 1;
      diag[i + (size_t)j * ni] = inv_dxdx * coef; /* dx^2 only, as the reference (:872) */

      double pc = AT(phi, i, j), ac = fabs(pc);
      double pl = AT(phi, i - 1, j), prr = AT(phi, i + 1, j), pb = AT(phi, i, j - 1), pt = AT(phi, i, j + 1);
      double jcc = AT(jc, i, j);
      double FL = 0, FR = 0, FB = 0, FT = 0;
      if (!((pc <= 0 && pl <= 0) || (pc > 0 && pl > 0))) {
        double a = (jcc * fabs(pl) + AT(jc, i - 1, j) * ac) / (ac + fabs(pl));
        if (pc <= 0 && pl > 0)
          FL = s.odx2 * a * bl;
        else if (pc > 0 && pl <= 0)
          FL = -s.odx2 * a * bl;
      }
      if (!((pc <= 0 && prr <= 0) || (pc > 0 && prr > 0))) {
        double a = (jcc * fabs(prr) + AT(jc, i + 1, j) * ac) / (ac + fabs(prr));
        if (pc <= 0 && prr > 0)
          FR = s.odx2 * a * br;
        else if (pc > 0 && prr <= 0)
          FR = -s.odx2 * a * br;
      }
      if (!((pc <= 0 && pb <= 0) || (pc > 0 && pb > 0))) {
        double a = (jcc * fabs(pb) + AT(jc, i, j - 1) * ac) / (ac + fabs(pb));
        if (pc <= 0 && pb > 0)
          FB = s.ody2 * a * bb;
        else if (pc > 0 && pb <= 0)
          FB = -s.ody2 * a * bb;
      }
      if (!((pc <= 0 && pt <= 0) || (pc > 0 && pt > 0))) {
        double a = (jcc * fabs(pt) + AT(jc, i, j + 1) * ac) / (ac + fabs(pt));
        if (pc <= 0 && pt > 0)
          FT = s.ody2 * a * bt;
        else if (pc > 0 && pt <= 0)
          FT = -s.ody2 * a * bt;
      }
      double div = s.odx * (AT(u, i + 1, j) - AT(u, i, j)) + s.ody * (AT(v, i, j + 1) - AT(v, i, j));
      div *= one_over_dt;
      double FX = FL + FR, FY = FB + FT;
      rhs[i + (size_t)j * ni] = -div - FX - FY;
    }
  free(vv_a);
  free(jc_a);
  free(rho);
  return OR_OK;
}

/* CSR_MATRIX::Multiply (CSR_MATRIX.h:233-250) in the builder's row order:
 * left, right, bottom, top, diagonal. */
void or_poisson_apply(const or_grid* gr, const double* bx, const double* by, const double* diag, const double* x, double* y) {
  int ni = gr->ni, nj = gr->nj;
  space_t s = base_space(gr);
  double idx2 = 1.0 / (s.dx * s.dx), idy2 = 1.0 / (s.dy * s.dy);
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i < ni; ++i) {
      size_t k = i + (size_t)j * ni;
      double acc = 0;
      if (i > 0) acc += -bx[i + (size_t)j * (ni + 1)] * idx2 * x[k - 1];
      if (i < ni - 1) acc += -bx[i + 1 + (size_t)j * (ni + 1)] * idx2 * x[k + 1];
      if (j > 0) acc += -by[i + (size_t)j * ni] * idy2 * x[k - ni];
      if (j < nj - 1) acc += -by[i + (size_t)(j + 1) * ni] * idy2 * x[k + ni];
      acc += diag[k] * x[k];
      y[k] = acc;
    }
}

/* ------------------------------------------------------------------------- */
/* a11: PCG_METHOD::PCGMethod (PCG_METHOD.cpp:176-264) with the IC(0) factor of
 * IncompleteCholeskyDecomposition (CSR_MATRIX.h:535-628) and the triangular
 * solves of MultiplicationByMinverse (PCG_METHOD.cpp:70-118).  L rows hold
 * [down, left, diag] in lexicographic order. */
typedef struct {
  double *ld, *ll, *dg;
  int ni, nj;
} ic0_t;

static void ic0_apply(const ic0_t* L, const double* b, double* x, double* y, double* summ) {
  int ni = L->ni;
  size_t n = (size_t)ni * L->nj;
  y[0] = b[0] * (1 / L->dg[0]);
  for (size_t i = 1; i < n; ++i) {
    double sum = 0;
    if (i >= (size_t)ni) sum += L->ld[i] * y[i - ni];
    if (i % ni != 0) sum += L->ll[i] * y[i - 1];
    double o = 1 / L->dg[i];
    y[i] = (b[i] - sum) * o;
  }
  memset(summ, 0, n * sizeof(double));
  x[n - 1] = y[n - 1] * (1 / L->dg[n - 1]);
  for (size_t i = n - 1; i >= 1; --i) {
    if (i % ni != 0) summ[i - 1] += L->ll[i] * x[i];
    if (i >= (size_t)ni) summ[i - ni] += L->ld[i] * x[i];
    double o = 1 / L->dg[i - 1];
    x[i - 1] = (y[i - 1] - summ[i - 1]) * o;
  }
}

/* The PCG state between calls, so that a solve can run in slices of iterations
 * (the CPU baseline times a full solve split over benchmark steps); the arithmetic
 * and its order are those of one uninterrupted PCGMethod call. */
typedef struct {
  const double *bx, *by, *diag;
  const or_grid* gr;
  double* x;
  double *buf, *r, *p, *Ap, *sv, *y, *summ;
  ic0_t L;
  double res_new, sqr_tol, rel_thr2;
  int it, max_it, done;
} pcg_run;

/* ComputeResidual, IncompleteCholeskyDecomposition, the first M^-1 r and r.z
 * (PCG_METHOD.cpp:192-212). */
static int pcg_begin(pcg_run* R, const or_grid* gr, const or_params* pr, const double* bx, const double* by, const double* diag,
                     const double* rhs, double* x) {
  int ni = gr->ni, nj = gr->nj;
  size_t n = (size_t)ni * nj;
  space_t s = base_space(gr);
  double idx2 = 1.0 / (s.dx * s.dx), idy2 = 1.0 / (s.dy * s.dy);
  memset(R, 0, sizeof(*R));
  R->buf = zalloc(9 * n);
  if (!R->buf) return OR_NO_MEMORY;
  R->gr = gr;
  R->bx = bx;
  R->by = by;
  R->diag = diag;
  R->x = x;
  ic0_t L = {R->buf, R->buf + n, R->buf + 2 * n, ni, nj};
  R->r = R->buf + 3 * n;
  R->p = R->buf + 4 * n;
  R->Ap = R->buf + 5 * n;
  R->sv = R->buf + 6 * n;
  R->y = R->buf + 7 * n;
  R->summ = R->buf + 8 * n;
  for (size_t k = 0; k < n; ++k) {
    int i = (int)(k % ni), j = (int)(k / ni);
    double sum = 0;
    if (k >= (size_t)ni) { /* A(down, k): top entry of row k-ni */
      double a = -by[i + (size_t)j * ni] * idy2;
      L.ld[k] = 1 / L.dg[k - ni] * a;
      sum += L.ld[k] * L.ld[k];
    }
    if (i > 0) { /* A(left, k): right entry of row k-1 */
      double a = -bx[i + (size_t)j * (ni + 1)] * idx2;
      L.ll[k] = 1 / L.dg[k - 1] * a;
      sum += L.ll[k] * L.ll[k];
    }
    L.dg[k] = (k == 0) ? sqrt(diag[k]) : sqrt(diag[k] - sum);
  }
  R->L = L;
  or_poisson_apply(gr, bx, by, diag, x, R->Ap);
  for (size_t k = 0; k < n; ++k) R->r[k] = rhs[k] - R->Ap[k];
  ic0_apply(&R->L, R->r, R->p, R->y, R->summ);
  double res_new = 0;
  for (size_t k = 0; k < n; ++k) res_new += R->r[k] * R->p[k];
  R->res_new = res_new;
  R->sqr_tol = pr->pcg_tolerance * pr->pcg_tolerance;
  R->rel_thr2 = 0;
  if (pr->pcg_rel_residual > 0) {
    double bb = 0;
    for (size_t k = 0; k < n; ++k) bb += rhs[k] * rhs[k];
    R->rel_thr2 = pr->pcg_rel_residual * pr->pcg_rel_residual * bb;
  }
  R->max_it = pr->pcg_max_iterations;
  return OR_OK;
}

/* Up to `count` iterations of the PCGMethod loop (PCG_METHOD.cpp:214-258); sets
 * done once a stop test holds.  Returns the iterations run. */
static int pcg_iterate(pcg_run* R, int count) {
  size_t n = (size_t)R->gr->ni * R->gr->nj;
  double *x = R->x, *r = R->r, *p = R->p, *Ap = R->Ap, *sv = R->sv;
  int k0 = 0;
  for (; k0 < count && !R->done; ++k0) {
    or_poisson_apply(R->gr, R->bx, R->by, R->diag, p, Ap);
    double dot = 0;
    for (size_t k = 0; k < n; ++k) dot += p[k] * Ap[k];
    double alpha = R->res_new / dot;
    for (size_t k = 0; k < n; ++k) {
      x[k] += alpha * p[k];
      r[k] -= alpha * Ap[k];
    }
    ic0_apply(&R->L, r, sv, R->y, R->summ);
    double res_old = R->res_new;
    double res_new = 0;
    for (size_t k = 0; k < n; ++k) res_new += r[k] * sv[k];
    R->res_new = res_new;
    double beta = res_new / res_old;
    for (size_t k = 0; k < n; ++k) {
      p[k] *= beta;
      p[k] += sv[k];
    }
    R->it++;
    if (R->it > R->max_it || res_new < R->sqr_tol) {
      R->done = 1;
    } else if (R->rel_thr2 > 0) {
      double rr = 0;
      for (size_t k = 0; k < n; ++k) rr += r[k] * r[k];
      if (rr <= R->rel_thr2) R->done = 1;
    }
  }
  return k0;
}

static void pcg_end(pcg_run* R, or_stats* st) {
  if (st) {
    st->iterations = R->it;
    st->residual = sqrt(R->res_new);
  }
  free(R->buf);
  R->buf = NULL;
}

int or_pcg_ic0(const or_grid* gr, const or_params* pr, const double* bx, const double* by, const double* diag, const double* rhs, double* x, or_stats* st) {
  if (!gr || !pr || !bx || !by || !diag || !rhs || !x) return OR_BAD_ARG;
  pcg_run R;
  int rc = pcg_begin(&R, gr, pr, bx, by, diag, rhs, x);
  if (rc) return rc;
  while (!R.done) pcg_iterate(&R, 1 << 30);
  pcg_end(&R, st);
  return OR_OK;
}

/* ------------------------------------------------------------------------- */
/* HeavisideFunction (PROJECTION_2D.h:1441-1461) with the reference's PI = 3.141592 (MACROS.h:5). */
static double heaviside(double phi, double eps) {
  const double PI_REF = 3.141592;
  if (phi < -eps) return 0;
  if (phi > eps) return 1;
  double oe = 1.0 / eps, opi = 1.0 / PI_REF;
  return 0.5 + phi * oe * 0.5 + 0.5 * opi * sin(PI_REF * phi * oe);
}

/* a9-a14: PROJECTION_2D::Solve(dt, tid) (PROJECTION_2D.h:244-257) for
 * air_bubble_rising with Neumann walls and use_delta_function_formulation, as
 * three calls: or_projection_begin (curvature, assembly, IC(0) factor),
 * or_projection_iterate (slices of PCG iterations) and or_projection_finish
 * (VectorToGrid, velocity update).  or_projection runs the three in one call. */
struct or_projection_run {
  or_grid gr;
  or_params pr;
  double *phi_a, *u_a, *v_a, *p_a, *kappa;
  double dt;
  double *bx, *by, *dg, *rhs, *x;
  pcg_run pcg;
  int pcg_open;
};

int or_projection_begin(const or_grid* gr, const or_params* pr, double* phi_a, double* u_a, double* v_a, double* p_a, double* kappa,
                        double dt, or_projection_run** out) {
  if (!gr || !pr || !phi_a || !u_a || !v_a || !p_a || !kappa || !out || gr->ni < 4 || gr->nj < 4) return OR_BAD_ARG;
  *out = NULL;
  int ni = gr->ni, nj = gr->nj, rc;
  size_t n = (size_t)ni * nj;
  or_projection_run* P = (or_projection_run*)calloc(1, sizeof(or_projection_run));
  if (!P) return OR_NO_MEMORY;
  P->gr = *gr;
  P->pr = *pr;
  P->phi_a = phi_a;
  P->u_a = u_a;
  P->v_a = v_a;
  P->p_a = p_a;
  P->kappa = kappa;
  P->dt = dt;
  P->bx = zalloc((size_t)(ni + 1) * nj);
  P->by = zalloc((size_t)ni * (nj + 1));
  P->dg = zalloc(n);
  P->rhs = zalloc(n);
  P->x = zalloc(n);
  if (!P->bx || !P->by || !P->dg || !P->rhs || !P->x) {
    rc = OR_NO_MEMORY;
    goto fail;
  }
  /* DetermineJumpConditionField -> ComputeCurvaturesThread fills phi's ghosts first. */
  if ((rc = or_curvature(&P->gr, phi_a, kappa))) goto fail;
  if ((rc = or_poisson_assemble(&P->gr, &P->pr, phi_a, u_a, v_a, kappa, dt, P->bx, P->by, P->dg, P->rhs))) goto fail;
  {
    fld p = F(p_a, 1, ni, nj);
    for (int j = 0; j < nj; ++j)
      for (int i = 0; i < ni; ++i) P->x[i + (size_t)j * ni] = AT(p, i, j); /* warm start (:974) */
  }
  if ((rc = pcg_begin(&P->pcg, &P->gr, &P->pr, P->bx, P->by, P->dg, P->rhs, P->x))) goto fail;
  P->pcg_open = 1;
  *out = P;
  return OR_OK;
fail:
  or_projection_free(P);
  return rc;
}

int or_projection_iterate(or_projection_run* P, int count, int* done) {
  if (!P || !P->pcg_open || count < 0) return OR_BAD_ARG;
  int k = pcg_iterate(&P->pcg, count);
  if (done) *done = P->pcg.done;
  return k;
}

int or_projection_finish(or_projection_run* P, or_stats* st) {
  if (!P || !P->pcg_open) return OR_BAD_ARG;
  while (!P->pcg.done) pcg_iterate(&P->pcg, 1 << 30);
  pcg_end(&P->pcg, st);
  P->pcg_open = 0;
  const or_grid* gr = &P->gr;
  const or_params* pr = &P->pr;
  int ni = gr->ni, nj = gr->nj;
  double dt = P->dt;
  const double* kappa = P->kappa;
  const double* x = P->x;
  space_t s = base_space(gr);
  fld phi = F(P->phi_a, 2, ni, nj), u = F(P->u_a, 2, ni + 1, nj), v = F(P->v_a, 2, ni, nj + 1), p = F(P->p_a, 1, ni, nj);
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i < ni; ++i) AT(p, i, j) = x[i + (size_t)j * ni]; /* VectorToGrid */

  /* a14: UpdateVelocityByPressureGradientVariableDensity (PROJECTION_2D.h:1297-1416).
   * Same-sign faces use the node density on the + side; interface faces use the
   * smeared-Heaviside density of the face-averaged phi (eps = 1.5 dx) and the
   * |phi|-weighted jump.  Pressure ghosts are zero; wall faces i = ni / j = nj
   * (bc < 0) are skipped. */
  {
    double eps_h = 1.5 * s.dx, eps_v = 1.5 * s.dy;
    double odx = 1.0 / s.dx, ody = 1.0 / s.dy;
    double mvx = 0, mvy = 0;
    double rw = pr->water_density, ra = pr->air_density;
#define JC(i, j) (((i) < 0 || (j) < 0 || (i) >= ni || (j) >= nj) ? 0.0 : pr->surface_tension * kappa[(i) + (size_t)(j) * ni])
#define RHO(i, j) (AT(phi, i, j) <= 0 ? ra : rw)
    for (int j = 0; j < nj; ++j)
      for (int i = 0; i < ni; ++i) {
        double rho_ij = RHO(i, j), oor = 1 / rho_ij;
        double l0 = AT(phi, i, j), ll = AT(phi, i - 1, j);
        double dh = ra + (rw - ra) * heaviside(0.5 * (l0 + ll), eps_h);
        double odh = 1 / dh;
        double jcc = JC(i, j), jcl = JC(i - 1, j);
        double gx = (jcl * fabs(l0) + jcc * fabs(ll)) / (fabs(l0) + fabs(ll));
        double pij = AT(p, i, j), pl = AT(p, i - 1, j);
        double* w = &AT(u, i, j);
        if (l0 * ll >= 0)
          *w -= dt * (pij - pl) * oor * odx;
        else if (l0 < 0)
          *w -= dt * (pij - pl + gx) * odh * odx;
        else if (l0 > 0)
          *w -= dt * (pij - pl - gx) * odh * odx;
        if (fabs(*w) > mvx) mvx = fabs(*w);
      }
    for (int j = 0; j < nj; ++j)
      for (int i = 0; i < ni; ++i) {
        double rho_ij = RHO(i, j), oor = 1 / rho_ij;
        double l0 = AT(phi, i, j), lb = AT(phi, i, j - 1);
        double dh = ra + (rw - ra) * heaviside(0.5 * (l0 + lb), eps_v);
        double odh = 1 / dh;
        double jcc = JC(i, j), jcb = JC(i, j - 1);
        double gy = (jcb * fabs(l0) + jcc * fabs(lb)) / (fabs(l0) + fabs(lb));
        double pij = AT(p, i, j), pb = AT(p, i, j - 1);
        double* w = &AT(v, i, j);
        if (l0 * lb >= 0)
          *w -= dt * (pij - pb) * oor * ody;
        else if (l0 < 0)
          *w -= dt * (pij - pb + gy) * odh * ody;
        else if (l0 > 0)
          *w -= dt * (pij - pb - gy) * odh * ody;
        if (fabs(*w) > mvy) mvy = fabs(*w);
      }
#undef JC
#undef RHO
    if (st) {
      st->max_velocity_x = mvx;
      st->max_velocity_y = mvy;
    }
  }
  return OR_OK;
}

void or_projection_free(or_projection_run* P) {
  if (!P) return;
  if (P->pcg_open) pcg_end(&P->pcg, NULL);
  free(P->bx);
  free(P->by);
  free(P->dg);
  free(P->rhs);
  free(P->x);
  free(P);
}

int or_projection(const or_grid* gr, const or_params* pr, double* phi_a, double* u_a, double* v_a, double* p_a, double* kappa, double dt, or_stats* st) {
  or_projection_run* P = NULL;
  int rc = or_projection_begin(gr, pr, phi_a, u_a, v_a, p_a, kappa, dt, &P);
  if (rc) return rc;
  rc = or_projection_finish(P, st);
  or_projection_free(P);
  return rc;
}

/* ------------------------------------------------------------------------- */
/* Rest of SolveForRK (EULERIAN_FLUID_SOLVER_2D.h:1857-1879) for air/water. */

/* ApplyGraivity (EULERIAN_FLUID_SOLVER_2D.h:3249-3268): every face of both MAC
 * grids, walls included, gains dt * gravity. */
int or_apply_gravity(const or_grid* gr, const or_flow* fl, double* u_a, double* v_a, double dt) {
  if (!gr || !fl || !u_a || !v_a) return OR_BAD_ARG;
  int ni = gr->ni, nj = gr->nj;
  double gx = dt * fl->gravity_x, gy = dt * fl->gravity_y;
  fld u = F(u_a, 2, ni + 1, nj), v = F(v_a, 2, ni, nj + 1);
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i <= ni; ++i) AT(u, i, j) += gx;
  for (int j = 0; j <= nj; ++j)
    for (int i = 0; i < ni; ++i) AT(v, i, j) += gy;
  return OR_OK;
}

/* SetupBoundaryConditionForVelocity (EULERIAN_FLUID_SOLVER_2D.h:2227-2263,
 * air_bubble_rising): the normal velocity on the four walls is zero. */
void or_velocity_bc(const or_grid* gr, double* u_a, double* v_a) {
  int ni = gr->ni, nj = gr->nj;
  fld u = F(u_a, 2, ni + 1, nj), v = F(v_a, 2, ni, nj + 1);
  for (int j = 0; j < nj; ++j) AT(u, 0, j) = AT(u, ni, j) = 0.0;
  for (int i = 0; i < ni; ++i) AT(v, i, 0) = AT(v, i, nj) = 0.0;
}

/* Sourcing (EULERIAN_FLUID_SOLVER_2D.h:2082-2097): DetermineDensity (:2162-2180,
 * air_bubble_rising: air where phi <= 0, water where phi > 0; interior nodes of the
 * ghost-2 density field), then, when fl->viscosity is set, the explicit
 * delta-function viscosity of VISCOSITY_2D::ApplyViscosity (VISCOSITY_2D.h:460-532).
 *
 * The viscosity update reads a copy of u and v whose ghosts are zero
 * (FIELD_STRUCTURE_2D::Initialize zero-fills, ARRAY_2D.h:48-72), and smeared
 * densities and viscosities (HeavisideFunction, VISCOSITY_2D.h:688-708, eps = 1.5 dx,
 * EULERIAN_FLUID_SOLVER_2D.h:347) of phi averaged to the face (x_half), to the
 * face's upper/lower corners (cu/cd; for y-faces right/left: cu/cl) and taken at
 * the two nodes beside it (r/c; for y-faces u/c). */
int or_sourcing(const or_grid* gr, const or_params* pr, const or_flow* fl, const double* phi_a, double* u_a, double* v_a,
                double* density_a, double dt) {
  if (!gr || !pr || !fl || !phi_a || !u_a || !v_a) return OR_BAD_ARG;
  int ni = gr->ni, nj = gr->nj;
  fld phi = F((double*)phi_a, 2, ni, nj);
  if (density_a) {
    fld d = F(density_a, 2, ni, nj);
    for (int j = 0; j < nj; ++j)
      for (int i = 0; i < ni; ++i) AT(d, i, j) = AT(phi, i, j) <= 0 ? pr->air_density : pr->water_density;
  }
  if (!fl->viscosity) return OR_OK;
  space_t s = base_space(gr);
  size_t nu = (size_t)(ni + 5) * (nj + 4), nv = (size_t)(ni + 4) * (nj + 5);
  double* tu_a = zalloc(nu);
  double* tv_a = zalloc(nv);
  if (!tu_a || !tv_a) {
    free(tu_a);
    free(tv_a);
    return OR_NO_MEMORY;
  }
  fld u = F(u_a, 2, ni + 1, nj), v = F(v_a, 2, ni, nj + 1);
  fld tu = F(tu_a, 2, ni + 1, nj), tv = F(tv_a, 2, ni, nj + 1);
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i <= ni; ++i) AT(tu, i, j) = AT(u, i, j);
  for (int j = 0; j <= nj; ++j)
    for (int i = 0; i < ni; ++i) AT(tv, i, j) = AT(v, i, j);
  const double eps = 1.5 * s.dx, odx = s.odx, ody = s.ody;
  const double rw = pr->water_density, ra = pr->air_density, mw = fl->water_viscosity, ma = fl->air_viscosity;
#define RHO_H(l) (ra + (rw - ra) * heaviside((l), eps))
#define MU_H(l) (ma + (mw - ma) * heaviside((l), eps))
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i <= ni; ++i) {
      double half = 0.5 * (AT(phi, i - 1, j) + AT(phi, i, j));
      double cu = 0.25 * (AT(phi, i - 1, j) + AT(phi, i, j) + AT(phi, i - 1, j + 1) + AT(phi, i, j + 1));
      double cd = 0.25 * (AT(phi, i - 1, j - 1) + AT(phi, i, j - 1) + AT(phi, i - 1, j) + AT(phi, i, j));
      double mu_cu = MU_H(cu), mu_cd = MU_H(cd), mu_r = MU_H(AT(phi, i, j)), mu_c = MU_H(AT(phi, i - 1, j));
      double coef = dt * (1 / RHO_H(half));
      double first = 2.0 * coef * odx *
                     (mu_r * odx * (AT(tu, i + 1, j) - AT(tu, i, j)) - mu_c * odx * (AT(tu, i, j) - AT(tu, i - 1, j)));
      double second = coef * ody *
                      (mu_cu * (ody * (AT(tu, i, j + 1) - AT(tu, i, j)) + odx * (AT(tv, i, j + 1) - AT(tv, i - 1, j + 1))) -
                       mu_cd * (ody * (AT(tu, i, j) - AT(tu, i, j - 1)) + odx * (AT(tv, i, j) - AT(tv, i - 1, j))));
      AT(u, i, j) += first + second;
    }
  for (int j = 0; j <= nj; ++j)
    for (int i = 0; i < ni; ++i) {
      double half = 0.5 * (AT(phi, i, j - 1) + AT(phi, i, j));
      double cu = 0.25 * (AT(phi, i, j - 1) + AT(phi, i + 1, j - 1) + AT(phi, i, j) + AT(phi, i + 1, j));
      double cl = 0.25 * (AT(phi, i - 1, j - 1) + AT(phi, i, j - 1) + AT(phi, i - 1, j) + AT(phi, i, j));
      double mu_cu = MU_H(cu), mu_cl = MU_H(cl), mu_u = MU_H(AT(phi, i, j)), mu_c = MU_H(AT(phi, i, j - 1));
      double coef = dt * (1 / RHO_H(half));
      double first = 2.0 * coef * ody *
                     (mu_u * ody * (AT(tv, i, j + 1) - AT(tv, i, j)) - mu_c * ody * (AT(tv, i, j) - AT(tv, i, j - 1)));
      double second = coef * odx *
                      (mu_cu * (ody * (AT(tu, i + 1, j) - AT(tu, i + 1, j - 1)) + odx * (AT(tv, i + 1, j) - AT(tv, i, j))) -
                       mu_cl * (ody * (AT(tu, i, j) - AT(tu, i, j - 1)) + odx * (AT(tv, i, j) - AT(tv, i - 1, j))));
      AT(v, i, j) += first + second;
    }
#undef RHO_H
#undef MU_H
  free(tu_a);
  free(tv_a);
  return OR_OK;
}

/* SolveForRK (EULERIAN_FLUID_SOLVER_2D.h:1857-1879): velocity advection,
 * gravity, sourcing, wall conditions, projection. */
int or_solve_for_rk(const or_grid* gr, const or_params* pr, const or_flow* fl, double* phi, double* u, double* v, double* ua,
                    double* va, double* p, double* kappa, double* density, double dt, or_stats* st) {
  int rc;
  if ((rc = or_velocity_advection(gr, pr, u, v, ua, va, dt))) return rc;
  if ((rc = or_apply_gravity(gr, fl, u, v, dt))) return rc;
  if ((rc = or_sourcing(gr, pr, fl, phi, u, v, density, dt))) return rc;
  or_velocity_bc(gr, u, v);
  return or_projection(gr, pr, phi, u, v, p, kappa, dt, st);
}

/* AdvanceOneTimeStepThread, order_for_time_advancing = 3 (EULERIAN_FLUID_SOLVER_2D.h:1694-1794):
 * level-set and reinitialisation TVD-RK3, then the velocity TVD-RK3 over three
 * SolveForRK stages, blended on every MAC face.  st sums the three projections'
 * iterations; its residual and maxima are the last projection's. */
int or_time_step(const or_grid* gr, const or_params* pr, const or_flow* fl, double* phi, double* u_a, double* v_a, double* ua,
                 double* va, double* p, double* kappa, double* density, double dt, or_stats* st) {
  if (!gr || !pr || !fl || !phi || !u_a || !v_a) return OR_BAD_ARG;
  int ni = gr->ni, nj = gr->nj, rc, its = 0;
  or_stats s1;
  memset(&s1, 0, sizeof s1);
  if ((rc = or_levelset_rk3(gr, pr, phi, ua, va, dt))) return rc;
  size_t nu = (size_t)(ni + 5) * (nj + 4), nv = (size_t)(ni + 4) * (nj + 5);
  double* ku_a = zalloc(nu);
  double* kv_a = zalloc(nv);
  if (!ku_a || !kv_a) {
    rc = OR_NO_MEMORY;
    goto out;
  }
  fld u = F(u_a, 2, ni + 1, nj), v = F(v_a, 2, ni, nj + 1), ku = F(ku_a, 2, ni + 1, nj), kv = F(kv_a, 2, ni, nj + 1);
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i <= ni; ++i) AT(ku, i, j) = AT(u, i, j);
  for (int j = 0; j <= nj; ++j)
    for (int i = 0; i < ni; ++i) AT(kv, i, j) = AT(v, i, j);
#define STAGE()                                                                                     \
  do {                                                                                              \
    if ((rc = or_solve_for_rk(gr, pr, fl, phi, u_a, v_a, ua, va, p, kappa, density, dt, &s1))) goto out; \
    its += s1.iterations;                                                                           \
  } while (0)
#define BLEND(c0, c1)                                                                     \
  do {                                                                                    \
    for (int j = 0; j < nj; ++j)                                                          \
      for (int i = 0; i <= ni; ++i) AT(u, i, j) = (c0) * AT(ku, i, j) + (c1) * AT(u, i, j); \
    for (int j = 0; j <= nj; ++j)                                                         \
      for (int i = 0; i < ni; ++i) AT(v, i, j) = (c0) * AT(kv, i, j) + (c1) * AT(v, i, j); \
  } while (0)
  STAGE();
  STAGE();
  BLEND(0.75, 0.25);
  STAGE();
  BLEND(1 / 3.0, 2 / 3.0);
#undef STAGE
#undef BLEND
  rc = OR_OK;
out:
  if (st) {
    *st = s1;
    st->iterations = its;
  }
  free(ku_a);
  free(kv_a);
  return rc;
}

/* CFLOneTimeStep for air/water (EULERIAN_FLUID_SOLVER_2D.h:3517-3637): the
 * advection rate from the largest |u| and |v| over the MAC grids (divided by
 * their own spacings), gravity sqrt(9.8 / dy) (the constant, not the gravity
 * vector), viscosity max(mu_w/rho_w, mu_a/rho_a) (2/dx^2 + 2/dy^2) (whether or not
 * the viscous term is applied) and surface tension from the largest |kappa|;
 * returns cfl_number / CFL, or 0 where CFL is 0.  cf/gf/vf/sf (may be null)
 * receive the four rates as the reference prints them. */
double or_cfl_time_step(const or_grid* gr, const or_params* pr, const or_flow* fl, const double* u_a, const double* v_a,
                        const double* kappa, double cfl_number, double rates[4]) {
  int ni = gr->ni, nj = gr->nj;
  space_t b = base_space(gr), xs = xface_space(gr), ys = yface_space(gr);
  fld u = F((double*)u_a, 2, ni + 1, nj), v = F((double*)v_a, 2, ni, nj + 1);
  double u_max = 0, v_max = 0, k_max = 0;
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i <= ni; ++i)
      if (u_max <= fabs(AT(u, i, j))) u_max = fabs(AT(u, i, j));
  for (int j = 0; j <= nj; ++j)
    for (int i = 0; i < ni; ++i)
      if (v_max <= fabs(AT(v, i, j))) v_max = fabs(AT(v, i, j));
  double c_f = (u_max * xs.odx + v_max * ys.ody);
  double g_f = sqrt(9.8 * b.ody);
  double rw = fl->water_viscosity / pr->water_density, ra = fl->air_viscosity / pr->air_density;
  double v_f = (rw < ra ? ra : rw) * (2 * b.odx2 + 2 * b.ody2);
  for (size_t k = 0; k < (size_t)ni * nj; ++k)
    if (fabs(kappa[k]) >= k_max) k_max = fabs(kappa[k]);
  double rmin = pr->water_density > pr->air_density ? pr->air_density : pr->water_density;
  double hmin = b.dx > b.dy ? b.dy : b.dx;
  double s_f = sqrt(pr->surface_tension * k_max / (rmin * (hmin * hmin)));
  double CFL = 0.5 * (c_f + v_f + sqrt((c_f + v_f) * (c_f + v_f) + 4 * (g_f * g_f) + 4 * (s_f * s_f)));
  double dt = cfl_number / CFL;
  if (CFL == 0) dt = 0;
  if (rates) {
    rates[0] = c_f;
    rates[1] = g_f;
    rates[2] = v_f;
    rates[3] = s_f;
  }
  return dt;
}

/* ------------------------------------------------------------------------- */
/* General jump-condition Poisson problem: POISSON_SOLVER::Solve(pressure, density, bc,
 * div, levelset, jc_on_solution, jc_on_derivative) (POISSON_SOLVER.cpp:127-145) with
 * BuildLinearSystemNodeJumpConditionVaribleCoefficient (:714-976), as POISSON_EQUATION_TEST
 * calls it (POISSON_EQUATION_TEST.h:352-396). */

/* LEVELSET_2D::ComputeNormals(thread_id) (LEVELSET_2D.h:640-662): phi's ghosts refreshed by
 * the copy fill first, then unit central-difference normals (one-sided where the central
 * ones vanish) on the interior nodes; nx, ny have ghost 1 (left untouched there). */
void or_normals(const or_grid* gr, double* phi_a, double* nx_a, double* ny_a) {
  int ni = gr->ni, nj = gr->nj;
  space_t s = base_space(gr);
  fld phi = F(phi_a, 2, ni, nj), nx = F(nx_a, 1, ni, nj), ny = F(ny_a, 1, ni, nj);
  or_fill_ghost_copy(phi_a, 2, phi_a, 2, ni, nj, 2);
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i < ni; ++i) {
      double x = (AT(phi, i + 1, j) - AT(phi, i - 1, j)) * s.o2dx, y = (AT(phi, i, j + 1) - AT(phi, i, j - 1)) * s.o2dy;
      double m = sqrt(x * x + y * y);
      if (!(m != 0)) {
        x = (AT(phi, i + 1, j) - AT(phi, i, j)) * s.odx;
        y = (AT(phi, i, j + 1) - AT(phi, i, j)) * s.ody;
      }
      double mag = sqrt(x * x + y * y), om = 1 / mag; /* VECTOR_2D::MakeThisUnit */
      if (mag != 0) {
        x *= om;
        y *= om;
      }
      AT(nx, i, j) = x;
      AT(ny, i, j) = y;
    }
}

#define OR_BC_DIR (-1)
#define OR_BC_NEUM (-4)

/* The system in the grid layout: rows of full cells (bc >= 0) as the builder writes them,
 * rows of every other node the identity scaled by 1/dx^2 with the node's pressure as its
 * value; faces touching a non-full node carry no coupling.  All node fields have ghost 1
 * (phi ghost 2; normals from or_normals).  bx: (ni+1) x nj, by: ni x (nj+1). */
int or_jump_poisson_assemble(const or_grid* gr, const double* pressure_a, const double* density_a, const int* bc_a,
                             const double* div_a, const double* phi_a, const double* nx_a, const double* ny_a,
                             const double* jcs_a, const double* jcd_a, double* bx, double* by, double* diag, double* rhs) {
  if (!gr || gr->ni < 4 || gr->nj < 4) return OR_BAD_ARG;
  int ni = gr->ni, nj = gr->nj, ld = ni + 2;
  space_t s = base_space(gr);
  const double inv_dxdx = 1 / (s.dx * s.dx), inv_dydy = 1 / (s.dy * s.dy);
  fld P = F((double*)pressure_a, 1, ni, nj), D = F((double*)div_a, 1, ni, nj), phi = F((double*)phi_a, 2, ni, nj);
  fld NX = F((double*)nx_a, 1, ni, nj), NY = F((double*)ny_a, 1, ni, nj);
  fld JS = F((double*)jcs_a, 1, ni, nj), JD = F((double*)jcd_a, 1, ni, nj);
  /* variable = 1/density on the interior, ghosts copied from the second interior line (:131-138) */
  double* v_a = zalloc((size_t)(ni + 4) * (nj + 4));
  if (!v_a) return OR_NO_MEMORY;
  fld V = F(v_a, 2, ni, nj), Dn = F((double*)density_a, 1, ni, nj);
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i < ni; ++i) AT(V, i, j) = 1 / AT(Dn, i, j);
  or_fill_ghost_copy(v_a, 2, v_a, 2, ni, nj, 2);
#define BC(i, j) (bc_a[((i) + 1) + (size_t)((j) + 1) * ld])
  for (size_t k = 0; k < (size_t)(ni + 1) * nj; ++k) bx[k] = 0;
  for (size_t k = 0; k < (size_t)ni * (nj + 1); ++k) by[k] = 0;
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i < ni; ++i) {
      size_t t = i + (size_t)j * ni;
      if (BC(i, j) < 0) {
        diag[t] = inv_dxdx;
        rhs[t] = inv_dxdx * AT(P, i, j);
        continue;
      }
      double lc = AT(phi, i, j), ll = AT(phi, i - 1, j), lr = AT(phi, i + 1, j), lb = AT(phi, i, j - 1), lt = AT(phi, i, j + 1);
      double vc = AT(V, i, j), vl = AT(V, i - 1, j), vr = AT(V, i + 1, j), vb = AT(V, i, j - 1), vt = AT(V, i, j + 1);
      double beta_l = vc * vl * (fabs(ll) + fabs(lc)) / (vc * fabs(ll) + vl * fabs(lc));
      double beta_r = vc * vr * (fabs(lr) + fabs(lc)) / (vr * fabs(lc) + vc * fabs(lr));
      double beta_b = vc * vb * (fabs(lb) + fabs(lc)) / (vc * fabs(lb) + vb * fabs(lc));
      double beta_t = vc * vt * (fabs(lt) + fabs(lc)) / (vt * fabs(lc) + vc * fabs(lt));
      int cl = BC(i - 1, j), cr = BC(i + 1, j), cb = BC(i, j - 1), ct = BC(i, j + 1);
      double coef = 0;
      if (cl > -1) coef += beta_l, bx[i + (size_t)j * (ni + 1)] = beta_l;
      if (cr > -1) coef += beta_r, bx[i + 1 + (size_t)j * (ni + 1)] = beta_r;
      if (cb > -1) coef += beta_b, by[i + (size_t)j * ni] = beta_b;
      if (ct > -1) coef += beta_t, by[i + (size_t)(j + 1) * ni] = beta_t;
      if (cl == OR_BC_DIR) coef += beta_l;
      if (cr == OR_BC_DIR) coef += beta_r;
      if (cb == OR_BC_DIR) coef += beta_b;
      if (ct == OR_BC_DIR) coef += beta_t;
      if (i == 0 && j == 0) {
        if (cl == OR_BC_NEUM) coef += beta_l;
        if (cr == OR_BC_NEUM) coef += beta_r;
        if (cb == OR_BC_NEUM) coef += beta_b;
        if (ct == OR_BC_NEUM) coef += beta_t;
      }
      if (coef == 0) coef = 1;
      diag[t] = inv_dxdx * coef;
      double jc = AT(JS, i, j), jd = AT(JD, i, j), nxc = AT(NX, i, j), nyc = AT(NY, i, j);
#define ARM(ln, jsn, jdn, nn, nc, beta, vn, o, o2, side)                                       \
  do {                                                                                          \
    double sub = fabs(ln) / (fabs(lc) + fabs(ln));                                              \
    double a = (jc * fabs(ln) + (jsn) * fabs(lc)) / (fabs(lc) + fabs(ln));                      \
    double b = (jd * (nc) * fabs(ln) + (jdn) * (nn) * fabs(lc)) / (fabs(lc) + fabs(ln));        \
    if ((lc <= 0 && (ln) <= 0) || (lc > 0 && (ln) > 0))                                         \
      side = 0;                                                                                 \
    else if (lc <= 0 && (ln) > 0)                                                               \
      side = (o2) * a * (beta) + SGN * ((o) * (beta) * b * sub / (vn));                         \
    else if (lc > 0 && (ln) <= 0)                                                               \
      side = -(o2) * a * (beta) - SGN * ((o) * (beta) * b * sub / (vn));                        \
  } while (0)
      double FL = 0, FR = 0, FB = 0, FT = 0;
#define SGN (-1)
      ARM(ll, AT(JS, i - 1, j), AT(JD, i - 1, j), AT(NX, i - 1, j), nxc, beta_l, vl, s.odx, s.odx2, FL);
      ARM(lb, AT(JS, i, j - 1), AT(JD, i, j - 1), AT(NY, i, j - 1), nyc, beta_b, vb, s.ody, s.ody2, FB);
#undef SGN
#define SGN (+1)
      ARM(lr, AT(JS, i + 1, j), AT(JD, i + 1, j), AT(NX, i + 1, j), nxc, beta_r, vr, s.odx, s.odx2, FR);
      ARM(lt, AT(JS, i, j + 1), AT(JD, i, j + 1), AT(NY, i, j + 1), nyc, beta_t, vt, s.ody, s.ody2, FT);
#undef SGN
#undef ARM
      double FX = FL + FR, FY = FB + FT;
      double r = -AT(D, i, j) - FX - FY;
      if (cl == OR_BC_DIR) r += beta_l * inv_dxdx * AT(P, i - 1, j);
      if (cr == OR_BC_DIR) r += beta_r * inv_dxdx * AT(P, i + 1, j);
      if (cb == OR_BC_DIR) r += beta_b * inv_dydy * AT(P, i, j - 1);
      if (ct == OR_BC_DIR) r += beta_t * inv_dydy * AT(P, i, j + 1);
      rhs[t] = r;
    }
#undef BC
  free(v_a);
  return OR_OK;
}

/* ------------------------------------------------------------------------- */
/* LEVELSET_2D::FastSweepingMethodOriginal(sweep_number) (LEVELSET_2D.h:281-384) with
 * Sweep (:507-589): nodes with |phi| < 2 dx stay fixed; phi's ghosts are extrapolated,
 * then sweep_number Gauss-Seidel sweeps (directions ++, -+, --, +- in turn) of Zhao's
 * upwind update, then the ghosts are extrapolated again (the single-threaded fill). */
static void fsm_sweep(fld* phi, const unsigned char* fixed, int ni, int nj, double h, int dir) {
  const double one_over_two = 1.0 / 2.0, hh = h * h, hh2 = hh * 2.0;
  const int ip = (dir == 1 || dir == 2) ? -1 : 1, jp = (dir == 2 || dir == 3) ? -1 : 1;
  for (int jj = 0; jj < nj; ++jj) {
    const int j = jp > 0 ? jj : nj - 1 - jj;
    for (int ii = 0; ii < ni; ++ii) {
      const int i = ip > 0 ? ii : ni - 1 - ii;
      if (fixed[i + (size_t)j * ni]) continue;
      double* pc = &AT(*phi, i, j);
      double a, b, a1, a2, update;
      double l = AT(*phi, i - 1, j), r = AT(*phi, i + 1, j), d = AT(*phi, i, j - 1), u = AT(*phi, i, j + 1);
      if (*pc > 0) {
        a = l > r ? r : l;
        b = d > u ? u : d;
        if (a <= b) a1 = a, a2 = b;
        else a1 = b, a2 = a;
        if (fabs(a1 - a2) >= h)
          update = a1 + h;
        else
          update = one_over_two * (a1 + a2 + sqrt(hh2 - (a1 - a2) * (a1 - a2)));
        *pc = update > *pc ? *pc : update;
      } else if (*pc <= 0) {
        a = l > r ? l : r;
        b = d > u ? d : u;
        if (a <= b) a1 = a, a2 = b;
        else a1 = b, a2 = a;
        if (fabs(a1 - a2) >= h)
          update = a2 - h;
        else
          update = one_over_two * (a2 + a1 - sqrt(hh2 - (a2 - a1) * (a2 - a1)));
        *pc = update > *pc ? update : *pc;
      }
    }
  }
}

/* The single-threaded FillGhostCellsContinuousDerivativesFrom (FIELD_STRUCTURE_2D.h:584-639):
 * every side innermost layer first, so outer layers read the freshly extrapolated inner one. */
static void extrapolate_inner_first(double* a, int g, int nI, int nJ) {
  fld f = F(a, g, nI, nJ);
  for (int j = 0; j < nJ; ++j)
    for (int i = -1; i >= -g; --i) AT(f, i, j) = 2.0 * AT(f, i + 1, j) - AT(f, i + 2, j);
  for (int j = 0; j < nJ; ++j)
    for (int i = nI; i <= nI - 1 + g; ++i) AT(f, i, j) = 2.0 * AT(f, i - 1, j) - AT(f, i - 2, j);
  for (int i = 0; i < nI; ++i)
    for (int j = nJ; j <= nJ - 1 + g; ++j) AT(f, i, j) = 2.0 * AT(f, i, j - 1) - AT(f, i, j - 2);
  for (int i = 0; i < nI; ++i)
    for (int j = -1; j >= -g; --j) AT(f, i, j) = 2.0 * AT(f, i, j + 1) - AT(f, i, j + 2);
}

int or_fast_sweeping(const or_grid* gr, double* phi_a, int sweeps) {
  if (!gr || !phi_a || sweeps < 0) return OR_BAD_ARG;
  int ni = gr->ni, nj = gr->nj;
  space_t s = base_space(gr);
  fld phi = F(phi_a, 2, ni, nj);
  unsigned char* fixed = (unsigned char*)calloc((size_t)ni * nj, 1);
  if (!fixed) return OR_NO_MEMORY;
  const double nb = 2.0 * s.dx;
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i < ni; ++i) fixed[i + (size_t)j * ni] = fabs(AT(phi, i, j)) < nb;
  extrapolate_inner_first(phi_a, 2, ni, nj);
  for (int k = 0; k < sweeps; ++k) fsm_sweep(&phi, fixed, ni, nj, s.dx, k % 4);
  extrapolate_inner_first(phi_a, 2, ni, nj);
  free(fixed);
  return OR_OK;
}
