// Adjoints (vector-Jacobian products) of the level-set WENO5 advection sweep and of
// the projection's velocity map, for gradients of a scalar loss through the step.
// The reference has no derivative code; these differentiate the reference's own
// forward maps as the FP64 kernels compute them:
//   * Levelset_Advection (ADVECTION_METHOD_2D.h:508-663 with the ghost copy of
//     FIELD_STRUCTURE_2D.h:374-449 and the extrapolation of :641-716): WENO5 weights
//     included; the upwind switch on the sign of the face-averaged velocity is held.
//   * PROJECTION_2D::Solve (PROJECTION_2D.h:244-257): u' = u* - dt M p, A p = b(u*),
//     so dL/du* = lam + D^T z with A z = M^T-applied cotangent (A symmetric): the
//     transposed gradient, the same solve, the transposed divergence.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "gb2d_internal.cuh"
#include "gb2d_schemes.cuh"

namespace gb2d {

namespace {

// d f / d a_m of one WENO5 side f(a1..a5) = sum_k w_k P_k (ADVECTION_METHOD_2D.h:545-619):
//   df/da = sum_k w_k dP_k/da + sum_k (P_k - f) / S * dalpha_k/da,
//   alpha_k = c_k / (eps + beta_k)^2, S = sum alpha_k, w_k = alpha_k / S.
__device__ void weno5_side_grad(const double a[5], double eps, double& f, double g[5]) {
  const double A[3] = {a[0] - 2 * a[1] + a[2], a[1] - 2 * a[2] + a[3], a[2] - 2 * a[3] + a[4]};
  const double B[3] = {a[0] - 4 * a[1] + 3 * a[2], a[1] - a[3], 3 * a[2] - 4 * a[3] + a[4]};
  const double dA[3][5] = {{1, -2, 1, 0, 0}, {0, 1, -2, 1, 0}, {0, 0, 1, -2, 1}};
  const double dB[3][5] = {{1, -4, 3, 0, 0}, {0, 1, 0, -1, 0}, {0, 0, 3, -4, 1}};
  const double dP[3][5] = {{1.0 / 3, -7.0 / 6, 11.0 / 6, 0, 0}, {0, -1.0 / 6, 5.0 / 6, 1.0 / 3, 0}, {0, 0, 1.0 / 3, 5.0 / 6, -1.0 / 6}};
  const double c[3] = {0.1, 0.6, 0.3};
  double beta[3], al[3], P[3], S = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    beta[k] = 13.0 / 12.0 * A[k] * A[k] + 0.25 * B[k] * B[k];
    al[k] = c[k] / ((eps + beta[k]) * (eps + beta[k]));
    S += al[k];
    P[k] = 0;
#pragma unroll
    for (int m = 0; m < 5; ++m) P[k] += dP[k][m] * a[m];
  }
  f = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) f += al[k] / S * P[k];
#pragma unroll
  for (int m = 0; m < 5; ++m) g[m] = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double w = al[k] / S, r = (P[k] - f) / S * (-2 * al[k] / (eps + beta[k]));
#pragma unroll
    for (int m = 0; m < 5; ++m) g[m] += w * dP[k][m] + r * (13.0 / 6.0 * A[k] * dA[k][m] + 0.5 * B[k] * dB[k][m]);
  }
}

// Derivative of the upwind WENO5 derivative along one line with respect to its seven
// stencil values q[0..6] (offsets -3..+3): minus side (d0..d4) when up, else plus side
// (d5..d1); d_k = o (q[k+1] - q[k]).  f receives the derivative itself.
__device__ void weno5_line_grad(const double q[7], double o, double eps, bool up, double& f, double J[7]) {
  double d[6], gd[6] = {0, 0, 0, 0, 0, 0}, a[5], g[5];
#pragma unroll
  for (int k = 0; k < 6; ++k) d[k] = o * (q[k + 1] - q[k]);
  if (up) {
#pragma unroll
    for (int t = 0; t < 5; ++t) a[t] = d[t];
    weno5_side_grad(a, eps, f, g);
#pragma unroll
    for (int t = 0; t < 5; ++t) gd[t] = g[t];
  } else {
#pragma unroll
    for (int t = 0; t < 5; ++t) a[t] = d[5 - t];
    weno5_side_grad(a, eps, f, g);
#pragma unroll
    for (int t = 0; t < 5; ++t) gd[5 - t] = g[t];
  }
#pragma unroll
  for (int m = 0; m < 7; ++m) J[m] = o * ((m > 0 ? gd[m - 1] : 0.0) - (m < 6 ? gd[m] : 0.0));
}

// The seven stencil positions of the ghost-filled copy read clamped positions of the
// interior (FillGhostCellsFrom copies the second interior line into every ghost layer).
__device__ __forceinline__ int clamp_line(int k, int n) { return k < 0 ? 1 : (k >= n ? n - 2 : k); }

struct AdjArgs {
  int ni, nj;
  double odx, ody, eps, dt;
};

// Per interior node n: C[m] = -dt u_n lam_n dfx/dq_m (m = 0..6) and the same for y
// (m = 7..13); gv = -dt lam f / 2 per direction (the face-averaged velocity's share).
__global__ void k_weno5_adj_coef(const double* __restrict__ phi_a, const double* __restrict__ ua_a, const double* __restrict__ va_a,
                                 const double* __restrict__ lam_a, double* __restrict__ coef, double* __restrict__ gvel, AdjArgs a) {
  const int ni = a.ni, nj = a.nj;
  const DField phi = dfield((double*)phi_a, 2, ni, nj), lam = dfield((double*)lam_a, 2, ni, nj);
  const DField ua = dfield((double*)ua_a, 3, ni + 1, nj), va = dfield((double*)va_a, 3, ni, nj + 1);
  const size_t n = (size_t)ni * nj;
  GB_FOR_IJ(i, j, ni, nj) {
    const size_t t = (size_t)j * ni + i;
    const double u = (GB_AT(ua, i + 1, j) + GB_AT(ua, i, j)) * 0.5;
    const double v = (GB_AT(va, i, j + 1) + GB_AT(va, i, j)) * 0.5;
    const double l = GB_AT(lam, i, j);
    double q[7], J[7], fx, fy;
#pragma unroll
    for (int m = 0; m < 7; ++m) q[m] = GB_AT(phi, clamp_line(i - 3 + m, ni), j);
    weno5_line_grad(q, a.odx, a.eps, gtz(u), fx, J);
#pragma unroll
    for (int m = 0; m < 7; ++m) coef[m * n + t] = -a.dt * u * l * J[m];
#pragma unroll
    for (int m = 0; m < 7; ++m) q[m] = GB_AT(phi, i, clamp_line(j - 3 + m, nj));
    weno5_line_grad(q, a.ody, a.eps, gtz(v), fy, J);
#pragma unroll
    for (int m = 0; m < 7; ++m) coef[(7 + m) * n + t] = -a.dt * v * l * J[m];
    gvel[t] = -a.dt * l * fx * 0.5;
    gvel[n + t] = -a.dt * l * fy * 0.5;
  }
}

// One reinitialisation sweep (the FP64 form of k_reinit_sweep): phi' = phi - dtau S h on the
// interior where the Godunov selection yields h = |grad phi| - 1 over the chosen one-sided WENO5
// derivatives, phi' = phi elsewhere and on the ghost ring.  With the selections held, per
// interior node: C[m] = -dtau S lam dh/dq_m along x (m = 0..6) and y (7..13), and the
// cotangent of S, -dtau h lam.  Gathered by k_weno5_adj_gather.
__global__ void k_reinit_adj_coef(const double* __restrict__ phi_a, const double* __restrict__ S, const double* __restrict__ lam_a,
                                  double* __restrict__ coef, double* __restrict__ gS, AdjArgs a, double dtau) {
  const int ni = a.ni, nj = a.nj;
  const DField phi = dfield((double*)phi_a, 2, ni, nj), lam = dfield((double*)lam_a, 2, ni, nj);
  const size_t n = (size_t)ni * nj;
  GB_FOR_IJ(i, j, ni, nj) {
    const size_t t = (size_t)j * ni + i;
    double qx[7], qy[7], Jmx[7], Jpx[7], Jmy[7], Jpy[7], mx, px, my, py;
#pragma unroll
    for (int m = 0; m < 7; ++m) qx[m] = GB_AT(phi, clamp_line(i - 3 + m, ni), j);
#pragma unroll
    for (int m = 0; m < 7; ++m) qy[m] = GB_AT(phi, i, clamp_line(j - 3 + m, nj));
    weno5_line_grad(qx, a.odx, a.eps, true, mx, Jmx);
    weno5_line_grad(qx, a.odx, a.eps, false, px, Jpx);
    weno5_line_grad(qy, a.ody, a.eps, true, my, Jmy);
    weno5_line_grad(qy, a.ody, a.eps, false, py, Jpy);
    const double s = S[t], l = GB_AT(lam, i, j);
    double h = 0.0, dgx = 0.0, dgy = 0.0;  // dh / d(chosen x and y derivatives)
    const double* Jx = Jmx;
    const double* Jy = Jmy;
    bool on = false;
    {
      // godunov_h<double>'s choices (ADVECTION_METHOD_2D.h:1505-1655)
      const double smx = s * mx, spx = s * px, smy = s * my, spy = s * py;
      int xs = -1, ys = -1;
      if (gez(spx) && gez(smx))
        xs = 0;
      else if (lez(spx) && lez(smx))
        xs = 1;
      else if (gtz(spx) && ltz(smx))
        xs = 2;
      else if (ltz(spx) && gtz(smx)) {
        const double sss = s * (fabs(px) - fabs(mx)) / (px - mx);
        xs = gtz(sss) ? 0 : (ltz(sss) ? 1 : -1);
      }
      if (xs >= 0) {
        if (gez(spy) && gez(smy))
          ys = 0;
        else if (lez(spy) && lez(smy))
          ys = 1;
        else if (gtz(spy) && ltz(smy))
          ys = 2;
        else if (ltz(spy) && gtz(smy)) {
          const double ss = s * (fabs(py) - fabs(my)) / (py - my);
          ys = gtz(ss) ? 0 : 1;
        }
      }
      if (xs >= 0 && ys >= 0) {
        on = true;
        const double gx = xs == 0 ? mx : px, gy = ys == 0 ? my : py;
        Jx = xs == 0 ? Jmx : Jpx;
        Jy = ys == 0 ? Jmy : Jpy;
        if (xs != 2 && ys != 2) {
          const double r = sqrt(gx * gx + gy * gy);
          h = r - 1.0;
          if (r > 0) dgx = gx / r, dgy = gy / r;
        } else if (xs != 2) {
          const double r = sqrt(gx * gx);
          h = r - 1.0;
          if (r > 0) dgx = gx / r;
        } else if (ys != 2) {
          const double r = sqrt(gy * gy);
          h = r - 1.0;
          if (r > 0) dgy = gy / r;
        } else {
          h = -1.0;
        }
      }
    }
    const double w = on ? -dtau * s * l : 0.0;
#pragma unroll
    for (int m = 0; m < 7; ++m) {
      coef[m * n + t] = w * dgx * Jx[m];
      coef[(7 + m) * n + t] = w * dgy * Jy[m];
    }
    gS[t] = on ? -dtau * h * l : 0.0;
  }
}

// Sum of the stencil coefficients that land on interior position k of one line:
// position p of the ghost-filled copy feeds nodes within 3 of it; k = 1 also owns the
// low ghost positions -1..-3, k = n-2 the high ones n..n+2.
__device__ __forceinline__ double line_gather(const double* __restrict__ coef, size_t n, size_t stride, size_t base, int k, int nk,
                                              int mbase) {
  double acc = 0;
  int ps[4] = {k, 0, 0, 0}, np = 1;
  if (k == 1) {
    ps[1] = -1;
    ps[2] = -2;
    ps[3] = -3;
    np = 4;
  } else if (k == nk - 2) {
    ps[1] = nk;
    ps[2] = nk + 1;
    ps[3] = nk + 2;
    np = 4;
  }
  for (int s = 0; s < np; ++s) {
    const int p = ps[s];
    const int lo = p - 3 < 0 ? 0 : p - 3, hi = p + 3 > nk - 1 ? nk - 1 : p + 3;
    for (int c = lo; c <= hi; ++c) acc += coef[(size_t)(mbase + p - c + 3) * n + base + (size_t)c * stride];
  }
  return acc;
}

// mu = lam (identity part) + the stencil coefficients gathered onto each interior
// node; ghost positions pass lam through (the sweep copies the input's ghost ring).
__global__ void k_weno5_adj_gather(const double* __restrict__ lam_a, const double* __restrict__ coef, double* __restrict__ mu_a, AdjArgs a) {
  const int ni = a.ni, nj = a.nj;
  const DField lam = dfield((double*)lam_a, 2, ni, nj), mu = dfield(mu_a, 2, ni, nj);
  const size_t n = (size_t)ni * nj;
  GB_FOR_IJ(ii, jj, ni + 4, nj + 4) {
    const int i = ii - 2, j = jj - 2;
    double v = GB_AT(lam, i, j);
    if (i >= 0 && i < ni && j >= 0 && j < nj) {
      v += line_gather(coef, n, 1, (size_t)j * ni, i, ni, 0);
      v += line_gather(coef, n, (size_t)ni, (size_t)i, j, nj, 7);
    }
    GB_AT(mu, i, j) = v;
  }
}

// dL/dUA, dL/dVA: each node's velocity share goes to the two faces it averages.
__global__ void k_weno5_adj_vel(const double* __restrict__ gvel, double* __restrict__ mu_ua_a, double* __restrict__ mu_va_a, int ni, int nj) {
  const DField mu_ua = dfield(mu_ua_a, 3, ni + 1, nj), mu_va = dfield(mu_va_a, 3, ni, nj + 1);
  const size_t n = (size_t)ni * nj;
  GB_FOR_IJ(i, j, ni + 1, nj + 1) {
    if (mu_ua_a && j < nj) GB_AT(mu_ua, i, j) = (i > 0 ? gvel[(size_t)j * ni + i - 1] : 0.0) + (i < ni ? gvel[(size_t)j * ni + i] : 0.0);
    if (mu_va_a && i < ni) GB_AT(mu_va, i, j) = (j > 0 ? gvel[n + (size_t)(j - 1) * ni + i] : 0.0) + (j < nj ? gvel[n + (size_t)j * ni + i] : 0.0);
  }
}

// Reverse of the ghost extrapolation (FillGhostCellsContinuousDerivativesFrom, ghost 2):
// each overwrite t <- 2 a - b becomes lam_a += 2 lam_t, lam_b -= lam_t, lam_t = 0, in
// the reverse order of the forward assignments.  What remains on a ghost cell is the
// cotangent of the value it held before the extrapolation.  Rows: left and right sides.
__global__ void k_extrap_adj_rows(double* lam_a, int ni, int nj) {
  const DField L = dfield(lam_a, 2, ni, nj);
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nj; j += gridDim.x * blockDim.x) {
    // right: forward i = ni then ni+1
    double t = GB_AT(L, ni + 1, j);
    GB_AT(L, ni, j) += 2 * t, GB_AT(L, ni - 1, j) -= t, GB_AT(L, ni + 1, j) = 0;
    t = GB_AT(L, ni, j);
    GB_AT(L, ni - 1, j) += 2 * t, GB_AT(L, ni - 2, j) -= t, GB_AT(L, ni, j) = 0;
    // left: forward i = -2 (reading the old -1) then i = -1
    t = GB_AT(L, -1, j);
    GB_AT(L, 0, j) += 2 * t, GB_AT(L, 1, j) -= t, GB_AT(L, -1, j) = 0;
    t = GB_AT(L, -2, j);
    GB_AT(L, -1, j) += 2 * t, GB_AT(L, 0, j) -= t, GB_AT(L, -2, j) = 0;
  }
}
// Columns: top and bottom sides.
__global__ void k_extrap_adj_cols(double* lam_a, int ni, int nj) {
  const DField L = dfield(lam_a, 2, ni, nj);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ni; i += gridDim.x * blockDim.x) {
    double t = GB_AT(L, i, -1);  // bottom: forward j = -2 then j = -1
    GB_AT(L, i, 0) += 2 * t, GB_AT(L, i, 1) -= t, GB_AT(L, i, -1) = 0;
    t = GB_AT(L, i, -2);
    GB_AT(L, i, -1) += 2 * t, GB_AT(L, i, 0) -= t, GB_AT(L, i, -2) = 0;
    t = GB_AT(L, i, nj + 1);  // top: forward j = nj then nj+1
    GB_AT(L, i, nj) += 2 * t, GB_AT(L, i, nj - 1) -= t, GB_AT(L, i, nj + 1) = 0;
    t = GB_AT(L, i, nj);
    GB_AT(L, i, nj - 1) += 2 * t, GB_AT(L, i, nj - 2) -= t, GB_AT(L, i, nj) = 0;
  }
}

struct ProjAdjArgs {
  int ni, nj;
  double dt, odx, ody, odt;
  double inv_water, inv_air, water, air, eps_h, eps_v, oeh, oev;
};

// 1/rho of a velocity-update face (UpdateVelocityByPressureGradientVariableDensity,
// PROJECTION_2D.h:1297-1416): the + side's node density on same-sign faces, the
// smeared density of the face-averaged phi on interface faces, 0 where the forward
// leaves the face alone (NaN).
__device__ __forceinline__ double face_inv_rho(double l0, double ln, bool xc, const ProjAdjArgs& a) {
  if (l0 * ln >= 0) return lez(l0) ? a.inv_air : a.inv_water;
  if (!(ltz(l0) || gtz(l0))) return 0;
  const double dh = a.air + (a.water - a.air) * heaviside(0.5 * (l0 + ln), xc ? a.eps_h : a.eps_v, xc ? a.oeh : a.oev);
  return 1 / dh;
}

// r = dL/dp = (d u'/d p)^T lam + lam_p for u'_f = u*_f - dt c_f od (p_+ - p_-), on the
// faces the forward updates (x-faces i < ni, y-faces j < nj; the pressure ghost is 0).
__global__ void k_proj_adj_rhs(const double* __restrict__ phi_a, const double* __restrict__ lu_a, const double* __restrict__ lv_a,
                               const double* __restrict__ lp_a, double* __restrict__ r, ProjAdjArgs a) {
  const int ni = a.ni, nj = a.nj;
  const DField phi = dfield((double*)phi_a, 2, ni, nj);
  const DField lu = dfield((double*)lu_a, 2, ni + 1, nj), lv = dfield((double*)lv_a, 2, ni, nj + 1);
  const DField lp = dfield((double*)lp_a, 1, ni, nj);
  GB_FOR_IJ(i, j, ni, nj) {
    const double pc = GB_AT(phi, i, j);
    double acc = lp_a ? GB_AT(lp, i, j) : 0.0;
    acc -= a.dt * face_inv_rho(pc, GB_AT(phi, i - 1, j), true, a) * a.odx * GB_AT(lu, i, j);
    acc -= a.dt * face_inv_rho(pc, GB_AT(phi, i, j - 1), false, a) * a.ody * GB_AT(lv, i, j);
    if (i + 1 < ni) acc += a.dt * face_inv_rho(GB_AT(phi, i + 1, j), pc, true, a) * a.odx * GB_AT(lu, i + 1, j);
    if (j + 1 < nj) acc += a.dt * face_inv_rho(GB_AT(phi, i, j + 1), pc, false, a) * a.ody * GB_AT(lv, i, j + 1);
    r[(size_t)j * ni + i] = acc;
  }
}

// mu = lam + (db/du*)^T z with b = -(odx dU + ody dV) / dt - F: z is the padded adjoint
// pressure (zero ghost ring), so wall faces see only their one interior node.
__global__ void k_proj_adj_vel(const double* __restrict__ lu_a, const double* __restrict__ lv_a, const double* __restrict__ z_a,
                               double* __restrict__ mu_u_a, double* __restrict__ mu_v_a, ProjAdjArgs a) {
  const int ni = a.ni, nj = a.nj;
  const DField lu = dfield((double*)lu_a, 2, ni + 1, nj), lv = dfield((double*)lv_a, 2, ni, nj + 1);
  const DField mu = dfield(mu_u_a, 2, ni + 1, nj), mv = dfield(mu_v_a, 2, ni, nj + 1);
  const DField z = dfield((double*)z_a, 1, ni, nj);
  GB_FOR_IJ(ii, jj, ni + 5, nj + 5) {
    const int i = ii - 2, j = jj - 2;
    if (i <= ni + 2 && j <= nj + 1) {
      double w = GB_AT(lu, i, j);
      if (i >= 0 && i <= ni && j >= 0 && j < nj) w += a.odx * a.odt * (GB_AT(z, i, j) - GB_AT(z, i - 1, j));
      GB_AT(mu, i, j) = w;
    }
    if (i <= ni + 1 && j <= nj + 2) {
      double w = GB_AT(lv, i, j);
      if (i >= 0 && i < ni && j >= 0 && j <= nj) w += a.ody * a.odt * (GB_AT(z, i, j) - GB_AT(z, i, j - 1));
      GB_AT(mv, i, j) = w;
    }
  }
}

// d/d(theta) of a projection loss, theta one of the two densities, after the projection
// adjoint (z with A z = dL/dp):
//   dL/dtheta = sum_f lam_f du'_f/dtheta |_p  +  z . (db/dtheta - (dA/dtheta) p).
// The face weights beta = vc vn (|phi_n|+|phi_c|) / (vc |phi_n| + vn |phi_c|), v = 1/rho
// of the node's phase, enter A (off-diagonals and the dx-only diagonal with its corner pin,
// POISSON_SOLVER.cpp:743-872) and the jump fluxes of b (:878-948); the velocity update's
// coefficients are 1/rho of the + node or 1/rho of the smeared face density
// (PROJECTION_2D.h:1297-1416).  One partial sum per block.
struct DensArgs {
  int ni, nj;
  double odx, ody, idx2, idy2, odx2, ody2, dt, sigma;
  double water, air, inv_water, inv_air, eps_h, eps_v, oeh, oev;
  int wrt_water;  // 1: d/d(water density), 0: d/d(air density)
};

__device__ __forceinline__ double v_of(double l, const DensArgs& a) {
  if (lez(l)) return a.inv_air;
  if (gtz(l)) return a.inv_water;
  return 1.0;
}
__device__ __forceinline__ double dv_of(double l, const DensArgs& a) {  // d(1/rho)/d(theta)
  if (lez(l)) return a.wrt_water ? 0.0 : -a.inv_air * a.inv_air;
  if (gtz(l)) return a.wrt_water ? -a.inv_water * a.inv_water : 0.0;
  return 0.0;
}
// d beta / d theta of the face between c and n (phi values lc, ln; ghost-mapped nodes).
__device__ __forceinline__ double dbeta(double lc, double ln, double lvc, double lvn, const DensArgs& a) {
  const double vc = v_of(lvc, a), vn = v_of(lvn, a), dvc = dv_of(lvc, a), dvn = dv_of(lvn, a);
  if (dvc == 0.0 && dvn == 0.0) return 0.0;
  const double ac = fabs(lc), an = fabs(ln), S = an + ac, D = vc * an + vn * ac;
  return (vn * vn * S * ac * dvc + vc * vc * S * an * dvn) / (D * D);
}

__global__ void k_density_grad(const double* __restrict__ phi_a, const double* __restrict__ kappa, const double* __restrict__ p_a,
                               const double* __restrict__ z_a, const double* __restrict__ lu_a, const double* __restrict__ lv_a,
                               double* __restrict__ part, DensArgs a) {
  const int ni = a.ni, nj = a.nj;
  const DField phi = dfield((double*)phi_a, 2, ni, nj), P = dfield((double*)p_a, 1, ni, nj), Z = dfield((double*)z_a, 1, ni, nj);
  const DField lu = dfield((double*)lu_a, 2, ni + 1, nj), lv = dfield((double*)lv_a, 2, ni, nj + 1);
  auto L = [&](int i, int j) { return GB_AT(phi, i, j); };
  // the node whose density a face weight reads (FillGhostCellsFrom mapping, as vnode)
  auto LV = [&](int i, int j) {
    i = i < 0 ? 1 : (i >= ni ? ni - 2 : i);
    j = j < 0 ? 1 : (j >= nj ? nj - 2 : j);
    return GB_AT(phi, i, j);
  };
  auto jc = [&](int i, int j) -> double {
    if (i < 0 || j < 0 || i >= ni || j >= nj) return 0.0;
    return a.sigma * kappa[i + (size_t)j * ni];
  };
  double acc = 0;
  GB_FOR_IJ(i, j, ni, nj) {
    const double lc = L(i, j);
    const double bl = dbeta(lc, L(i - 1, j), LV(i, j), LV(i - 1, j), a), br = dbeta(lc, L(i + 1, j), LV(i, j), LV(i + 1, j), a);
    const double bb = dbeta(lc, L(i, j - 1), LV(i, j), LV(i, j - 1), a), bt = dbeta(lc, L(i, j + 1), LV(i, j), LV(i, j + 1), a);
    double coef = 0;
    if (i > 0) coef += bl;
    if (i < ni - 1) coef += br;
    if (j > 0) coef += bb;
    if (j < nj - 1) coef += bt;
    if (i == 0 && j == 0) coef += bl + bb;  // the Neumann arms of the pinned corner cell
    double Ap = a.idx2 * coef * GB_AT(P, i, j);
    if (i > 0) Ap -= bl * a.idx2 * GB_AT(P, i - 1, j);
    if (i < ni - 1) Ap -= br * a.idx2 * GB_AT(P, i + 1, j);
    if (j > 0) Ap -= bb * a.idy2 * GB_AT(P, i, j - 1);
    if (j < nj - 1) Ap -= bt * a.idy2 * GB_AT(P, i, j + 1);
    // jump fluxes: +/- o2 av beta on arms that cross the interface
    auto dF = [&](double ln, int in, int jn, double db, double o2) -> double {
      const bool cneg = lez(lc), nneg = lez(ln);
      const double ac = fabs(lc), an = fabs(ln);
      if (cneg && !nneg && gtz(ln)) return o2 * ((jc(i, j) * an + jc(in, jn) * ac) / (ac + an)) * db;
      if (!cneg && gtz(lc) && nneg) return -o2 * ((jc(i, j) * an + jc(in, jn) * ac) / (ac + an)) * db;
      return 0.0;
    };
    const double db_node = -(dF(L(i - 1, j), i - 1, j, bl, a.odx2) + dF(L(i + 1, j), i + 1, j, br, a.odx2) +
                             dF(L(i, j - 1), i, j - 1, bb, a.ody2) + dF(L(i, j + 1), i, j + 1, bt, a.ody2));
    acc += GB_AT(Z, i, j) * (db_node - Ap);
    // velocity update of the x-face (i, j) and the y-face (i, j), p fixed
    for (int xc = 1; xc >= 0; --xc) {
      const int in = xc ? i - 1 : i, jn = xc ? j : j - 1;
      const double ln = L(in, jn), dp = GB_AT(P, i, j) - GB_AT(P, in, jn), od = xc ? a.odx : a.ody;
      const double lam = xc ? GB_AT(lu, i, j) : GB_AT(lv, i, j);
      double dc = 0, g = dp;
      if (lc * ln >= 0) {
        dc = dv_of(lc, a);
      } else if (ltz(lc) || gtz(lc)) {
        const double jcc = jc(i, j), jcn = jc(in, jn);
        const double gam = (jcn * fabs(lc) + jcc * fabs(ln)) / (fabs(lc) + fabs(ln));
        const double H = heaviside(0.5 * (lc + ln), xc ? a.eps_h : a.eps_v, xc ? a.oeh : a.oev);
        const double dh = a.air + (a.water - a.air) * H;
        const double ddh = a.wrt_water ? H : 1.0 - H;
        dc = -ddh / (dh * dh);
        g = ltz(lc) ? dp + gam : dp - gam;
      }
      acc += lam * (-a.dt * g * od * dc);
    }
  }
  // block sum: warps by shuffle, then the warp sums in a fixed order
  __shared__ double ws[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  const int lane = threadIdx.x & 31, warp = (threadIdx.x + threadIdx.y * blockDim.x) >> 5;
  if (lane == 0) ws[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    double t = 0;
    for (int w = 0; w < (int)((blockDim.x * blockDim.y + 31) / 32); ++w) t += ws[w];
    part[blockIdx.x + (size_t)blockIdx.y * gridDim.x] = t;
  }
}

// ---- d/d(phi) of a projection loss (after the projection adjoint) -----------------
//
//   dL/dphi = sum_f lam_f du'_f/dphi |_p  +  z . (db/dphi - (dA/dphi) p)
//
// phi enters through the face weights beta (|phi|-weighted harmonic mean of 1/rho, in A's
// off-diagonals and dx-only diagonal with the corner pin and in b's jump fluxes), the jump
// fluxes' |phi|-weighted interpolation of jc = sigma kappa, the curvature kappa(phi) (a
// 9-point stencil, zero slope where it is clamped), and on the velocity update's interface
// faces the |phi|-weighted jump and the smeared Heaviside density.  The phases (signs of
// phi) are piecewise constant: no derivative.  Two passes, both gathers (deterministic):
// per node the cotangent of kappa and from it the coefficients of the curvature's five
// differences; then per node of the ghost-1 ring and interior the direct terms of its four
// faces plus the curvature stencils that read it.  The extrapolation of phi's ghosts that
// the projection starts with is reversed last.
struct PhiArgs {
  int ni, nj;
  double odx, ody, o2dx, o2dy, odx2, ody2, idx2, idy2, dt, sigma, tol;
  double water, air, inv_water, inv_air, eps_h, eps_v, oeh, oev;
};

__device__ __forceinline__ double sgn(double x) { return gtz(x) ? 1.0 : (ltz(x) ? -1.0 : 0.0); }
__device__ __forceinline__ double vphase(double l, const PhiArgs& a) { return lez(l) ? a.inv_air : (gtz(l) ? a.inv_water : 1.0); }
// d H / d x of the smeared Heaviside inside its band (0 outside), PI as the forward's.
__device__ __forceinline__ double dheaviside(double x, double eps, double oe) {
  if (lt_neg(x, eps) || gt_pos(x, eps)) return 0.0;
  const double PI_REF = 3.141592;
  return 0.5 * oe * (1.0 + cos(PI_REF * x * oe));
}
// Jump-flux sign of the arm c -> n: +1 (c <= 0 < n), -1 (c > 0 >= n), 0.
__device__ __forceinline__ double arm_sign(double lc, double ln) {
  if (lez(lc) && !lez(ln) && gtz(ln)) return 1.0;
  if (!lez(lc) && gtz(lc) && lez(ln)) return -1.0;
  return 0.0;
}

struct PhiView {
  DField phi, P, Z, lu, lv;
  const double* kappa;
  int ni, nj;
  __device__ double L(int i, int j) const { return GB_AT(phi, i, j); }
  __device__ double LV(int i, int j) const {  // the node a face weight takes its phase from (as vnode)
    i = i < 0 ? 1 : (i >= ni ? ni - 2 : i);
    j = j < 0 ? 1 : (j >= nj ? nj - 2 : j);
    return GB_AT(phi, i, j);
  }
  __device__ double jc(int i, int j, double sigma) const {
    if (i < 0 || j < 0 || i >= ni || j >= nj) return 0.0;
    return sigma * kappa[i + (size_t)j * ni];
  }
  __device__ bool interior(int i, int j) const { return i >= 0 && j >= 0 && i < ni && j < nj; }
};

// One face between node c (the + side: (i, j)) and node n ((i-1, j) for an x-face, (i, j-1)
// for a y-face): its direct contributions to dL/dphi_c and dL/dphi_n, and to dL/djc_c and
// dL/djc_n (the curvature pass uses the latter).
__device__ void face_terms(const PhiView& v, const PhiArgs& a, bool xc, int i, int j, double& gc, double& gn, double& kc, double& kn) {
  gc = gn = kc = kn = 0.0;
  const int in = xc ? i - 1 : i, jn = xc ? j : j - 1;
  const int nmax = xc ? a.ni : a.nj, f = xc ? i : j;  // the face's index along its axis, 0..nmax
  const double lc = v.L(i, j), ln = v.L(in, jn);
  const double vc = vphase(v.LV(i, j), a), vn = vphase(v.LV(in, jn), a);
  const double ac = fabs(lc), an = fabs(ln), S = ac + an, D = vc * an + vn * ac;
  const double beta = vc * vn * (an + ac) / D;
  const double dbc = sgn(lc) * vc * vn * an * (vc - vn) / (D * D), dbn = sgn(ln) * vc * vn * ac * (vn - vc) / (D * D);
  const bool crow = v.interior(i, j), nrow = v.interior(in, jn);
  const double pc = crow ? GB_AT(v.P, i, j) : 0.0, pn = nrow ? GB_AT(v.P, in, jn) : 0.0;
  const double zc = crow ? GB_AT(v.Z, i, j) : 0.0, zn = nrow ? GB_AT(v.Z, in, jn) : 0.0;
  const double hoff = xc ? a.idx2 : a.idy2, o2 = xc ? a.odx2 : a.ody2;
  // A p: the c row's arm toward n (an interior face, or the pinned corner's wall arm) and
  // the n row's arm toward c (unless it is the far wall)
  double dLdb = 0.0;
  if (crow) {
    if (f > 0)
      dLdb -= zc * (a.idx2 * pc - hoff * pn);
    else if (i == 0 && j == 0)
      dLdb -= zc * a.idx2 * pc;
  }
  if (nrow && f < nmax) dLdb -= zn * (a.idx2 * pn - hoff * pc);
  // jump fluxes F = s o2 av beta, in b as -F: arm c -> n in row c, arm n -> c in row n
  const double jcc = v.jc(i, j, a.sigma), jcn = v.jc(in, jn, a.sigma);
  if (S > 0.0) {
    const double av = (jcc * an + jcn * ac) / S;
    const double scn = crow ? arm_sign(lc, ln) : 0.0, snc = nrow ? arm_sign(ln, lc) : 0.0;
    const double wc = -zc * scn * o2, wn = -zn * snc * o2;  // dL/dF-weights times o2 s
    dLdb += (wc + wn) * av;
    const double dav_ac = an * (jcn - jcc) / (S * S), dav_an = ac * (jcc - jcn) / (S * S);
    gc += (wc + wn) * beta * dav_ac * sgn(lc);
    gn += (wc + wn) * beta * dav_an * sgn(ln);
    kc += (wc + wn) * beta * an / S * a.sigma;
    kn += (wc + wn) * beta * ac / S * a.sigma;
  }
  gc += dLdb * dbc;
  gn += dLdb * dbn;
  // velocity update of this face (updated for i < ni on x-faces, j < nj on y-faces)
  if (crow && lc * ln < 0 && (ltz(lc) || gtz(lc))) {
    const double lam = xc ? GB_AT(v.lu, i, j) : GB_AT(v.lv, i, j);
    const double od = xc ? a.odx : a.ody, eps = xc ? a.eps_h : a.eps_v, oe = xc ? a.oeh : a.oev;
    const double s0 = ltz(lc) ? 1.0 : -1.0;
    const double gam = (jcn * ac + jcc * an) / S;
    const double m = 0.5 * (lc + ln);
    const double dh = a.air + (a.water - a.air) * heaviside(m, eps, oe), odh = 1.0 / dh;
    const double dp = pc - pn;
    const double w_gam = -a.dt * od * s0 * odh * lam;                  // dL/dgam
    const double w_odh = -a.dt * od * (dp + s0 * gam) * lam;            // dL/dodh
    const double dodh_dm = -odh * odh * (a.water - a.air) * dheaviside(m, eps, oe);
    gc += w_gam * sgn(lc) * an * (jcn - jcc) / (S * S) + w_odh * dodh_dm * 0.5;
    gn += w_gam * sgn(ln) * ac * (jcc - jcn) / (S * S) + w_odh * dodh_dm * 0.5;
    kc += w_gam * an / S * a.sigma;
    kn += w_gam * ac / S * a.sigma;
  }
}

// Pass 1, per interior node: dL/dkappa from its faces, then the coefficients of the five
// curvature differences (central: cx, cy; one-sided fallback: fx, fy; cxx, cyy, cxy).
__global__ void k_phi_grad_kappa(PhiView v, PhiArgs a, double* __restrict__ co) {
  const int ni = a.ni, nj = a.nj;
  const size_t n = (size_t)ni * nj;
  GB_FOR_IJ(i, j, ni, nj) {
    double gk = 0.0, t0, t1, kc, kn;
    face_terms(v, a, true, i, j, t0, t1, kc, kn);  // x-face (i, j): this node is c
    gk += kc;
    face_terms(v, a, false, i, j, t0, t1, kc, kn);  // y-face (i, j)
    gk += kc;
    face_terms(v, a, true, i + 1, j, t0, t1, kc, kn);  // x-face (i+1, j): this node is n
    gk += kn;
    face_terms(v, a, false, i, j + 1, t0, t1, kc, kn);  // y-face (i, j+1)
    gk += kn;
    // kappa's partials, as the forward computes kappa (the clamp has zero slope)
    const double c = v.L(i, j), l = v.L(i - 1, j), r = v.L(i + 1, j), b = v.L(i, j - 1), tp = v.L(i, j + 1);
    double px = (r - l) * a.o2dx, py = (tp - b) * a.o2dy;
    const double pxx = (r - 2 * c + l) * a.odx2, pyy = (tp - 2 * c + b) * a.ody2;
    const double pxy = (v.L(i + 1, j + 1) - v.L(i + 1, j - 1) - v.L(i - 1, j + 1) + v.L(i - 1, j - 1)) * a.o2dx * a.o2dy;
    double mag = sqrt(px * px + py * py);
    bool central = mag * mag * mag != 0.0;
    if (!central) {
      px = (r - c) * a.odx;
      py = (tp - c) * a.ody;
      mag = sqrt(px * px + py * py);
    }
    const double deno = mag * mag * mag;
    double e[7] = {0, 0, 0, 0, 0, 0, 0};
    if (deno != 0.0 && gk != 0.0) {
      const double N = px * px * pyy - 2.0 * px * py * pxy + py * py * pxx;
      const double curv = -N / deno;
      if (fabs(curv) <= a.tol) {
        const double dpx = -(2 * px * pyy - 2 * py * pxy) / deno + N * 3 * px * mag / (deno * deno);
        const double dpy = -(2 * py * pxx - 2 * px * pxy) / deno + N * 3 * py * mag / (deno * deno);
        e[central ? 0 : 2] = gk * dpx;
        e[central ? 1 : 3] = gk * dpy;
        e[4] = gk * (-py * py / deno);
        e[5] = gk * (-px * px / deno);
        e[6] = gk * (2 * px * py / deno);
      }
    }
    const size_t t = (size_t)j * ni + i;
#pragma unroll
    for (int k = 0; k < 7; ++k) co[k * n + t] = e[k];
  }
}

// Pass 2, per node of the interior and the ghost-1 ring: the direct terms of its four faces
// and the curvature stencils that read it, into g (phi's layout, ghost 2).
__global__ void k_phi_grad_gather(PhiView v, PhiArgs a, const double* __restrict__ co, double* __restrict__ g_a) {
  const int ni = a.ni, nj = a.nj;
  const size_t n = (size_t)ni * nj;
  DField g = dfield(g_a, 2, ni, nj);
  GB_FOR_IJ(ii, jj, ni + 2, nj + 2) {
    const int i = ii - 1, j = jj - 1;
    double acc = 0.0, gc, gn, kc, kn;
    if (i >= 0 && i <= ni && j >= 0 && j < nj) {  // x-face (i, j): this node is c
      face_terms(v, a, true, i, j, gc, gn, kc, kn);
      acc += gc;
    }
    if (i + 1 >= 0 && i + 1 <= ni && j >= 0 && j < nj) {  // x-face (i+1, j): this node is n
      face_terms(v, a, true, i + 1, j, gc, gn, kc, kn);
      acc += gn;
    }
    if (j >= 0 && j <= nj && i >= 0 && i < ni) {
      face_terms(v, a, false, i, j, gc, gn, kc, kn);
      acc += gc;
    }
    if (j + 1 >= 0 && j + 1 <= nj && i >= 0 && i < ni) {
      face_terms(v, a, false, i, j + 1, gc, gn, kc, kn);
      acc += gn;
    }
    auto C = [&](int k, int mi, int mj) -> double {
      return (mi >= 0 && mj >= 0 && mi < ni && mj < nj) ? co[k * n + (size_t)mj * ni + mi] : 0.0;
    };
    // curvature of (i-1, j), (i+1, j), (i, j-1), (i, j+1), (i, j) and the four diagonal nodes
    acc += C(0, i - 1, j) * a.o2dx + C(2, i - 1, j) * a.odx + C(4, i - 1, j) * a.odx2;
    acc += -C(0, i + 1, j) * a.o2dx + C(4, i + 1, j) * a.odx2;
    acc += C(1, i, j - 1) * a.o2dy + C(3, i, j - 1) * a.ody + C(5, i, j - 1) * a.ody2;
    acc += -C(1, i, j + 1) * a.o2dy + C(5, i, j + 1) * a.ody2;
    acc += -C(2, i, j) * a.odx - C(3, i, j) * a.ody - 2 * C(4, i, j) * a.odx2 - 2 * C(5, i, j) * a.ody2;
    const double oxy = a.o2dx * a.o2dy;
    acc += (C(6, i - 1, j - 1) - C(6, i - 1, j + 1) - C(6, i + 1, j - 1) + C(6, i + 1, j + 1)) * oxy;
    GB_AT(g, i, j) = acc;
  }
}

// ---- ENO3 velocity advection (the FP64 forms of k_eno3) -------------------------------
//
// u'_f = u_f - dt (uu f_x + vv f_y) on every face of both MAC components, f_x the upwind
// ENO3 one-sided derivative of the advected component's copy (UA or VA) along x, f_y along
// y, uu and vv the face's advecting velocities (its own copy value or a 4-face average).  With
// the divided-difference choices and the upwind sides held (piecewise constant), f_x and f_y
// are linear in their seven stencil values.  Per face: its 14 stencil coefficients times
// lam (-dt uu) / lam (-dt vv) and its two velocity shares lam (-dt f_x), lam (-dt f_y); then
// per cell of UA and VA a gather over the faces that read it.
struct EnoAdjArgs {
  int ni, nj;
  Space xs, ys;
  double o3[2][2];
  double dt;
};

// eno3_select's four choices, and its formulas for any d with those choices.
__device__ __forceinline__ void eno3_flags(const double d[6], double o2, double o3, bool f[4]) {
  const double d2n2 = o2 * (d[1] - d[0]), d2n1 = o2 * (d[2] - d[1]), d20 = o2 * (d[3] - d[2]);
  const double d2p1 = o2 * (d[4] - d[3]), d2p2 = o2 * (d[5] - d[4]);
  const double d3n2 = o3 * (d2n1 - d2n2), d3n1 = o3 * (d20 - d2n1), d30 = o3 * (d2p1 - d20), d3p1 = o3 * (d2p2 - d2p1);
  f[0] = mag_le(d2n1, d20);
  f[1] = f[0] ? mag_le(d3n2, d3n1) : mag_le(d3n1, d30);
  f[2] = mag_le(d20, d2p1);
  f[3] = f[2] ? mag_le(d3n1, d30) : mag_le(d30, d3p1);
}
__device__ __forceinline__ void eno3_apply(const double d[6], const bool f[4], double o2, double o3, double h, double& dm, double& dp) {
  const double d1n1 = d[2], d10 = d[3];
  const double d2n2 = o2 * (d[1] - d[0]), d2n1 = o2 * (d[2] - d[1]), d20 = o2 * (d[3] - d[2]);
  const double d2p1 = o2 * (d[4] - d[3]), d2p2 = o2 * (d[5] - d[4]);
  const double d3n2 = o3 * (d2n1 - d2n2), d3n1 = o3 * (d20 - d2n1), d30 = o3 * (d2p1 - d20), d3p1 = o3 * (d2p2 - d2p1);
  if (f[0])
    dm = d1n1 + d2n1 * h + 2.0 * (f[1] ? d3n2 : d3n1) * h * h;
  else
    dm = d1n1 + d20 * h - (f[1] ? d3n1 : d30) * h * h;
  if (f[2])
    dp = d10 - d20 * h - (f[3] ? d3n1 : d30) * h * h;
  else
    dp = d10 - d2p1 * h + 2.0 * (f[3] ? d30 : d3p1) * h * h;
}
// The coefficients of the chosen dm and dp on q[0..6] (d_k = o (q_{k+1} - q_k)).
__device__ void eno3_coef(const double q[7], double o, double o2, double o3, double h, double cm[7], double cp[7]) {
  double d[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) d[k] = o * (q[k + 1] - q[k]);
  bool f[4];
  eno3_flags(d, o2, o3, f);
  double am[6], ap[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    double e[6] = {0, 0, 0, 0, 0, 0};
    e[k] = 1.0;
    eno3_apply(e, f, o2, o3, h, am[k], ap[k]);
  }
#pragma unroll
  for (int m = 0; m < 7; ++m) {
    cm[m] = o * ((m > 0 ? am[m - 1] : 0.0) - (m < 6 ? am[m] : 0.0));
    cp[m] = o * ((m > 0 ? ap[m - 1] : 0.0) - (m < 6 ? ap[m] : 0.0));
  }
}

__global__ void k_eno3_adj_face(const double* __restrict__ ua_a, const double* __restrict__ va_a, const double* __restrict__ lu_a,
                                const double* __restrict__ lv_a, double* __restrict__ co, EnoAdjArgs a) {
  const int ni = a.ni, nj = a.nj;
  const DField ua = dfield((double*)ua_a, 3, ni + 1, nj), va = dfield((double*)va_a, 3, ni, nj + 1);
  const DField lu = dfield((double*)lu_a, 2, ni + 1, nj), lv = dfield((double*)lv_a, 2, ni, nj + 1);
  auto face = [&](bool xc, int i, int j, double* out) {
    const DField& g = xc ? ua : va;
    const Space& s = xc ? a.xs : a.ys;
    double qx[7], qy[7], cmx[7], cpx[7], cmy[7], cpy[7], mx, px, my, py;
    for (int m = 0; m < 7; ++m) qx[m] = GB_AT(g, i - 3 + m, j);
    for (int m = 0; m < 7; ++m) qy[m] = GB_AT(g, i, j - 3 + m);
    eno3_pair(qx, s.odx, s.o2dx, a.o3[xc ? 0 : 1][0], s.dx, mx, px);
    eno3_pair(qy, s.ody, s.o2dy, a.o3[xc ? 0 : 1][1], s.dy, my, py);
    eno3_coef(qx, s.odx, s.o2dx, a.o3[xc ? 0 : 1][0], s.dx, cmx, cpx);
    eno3_coef(qy, s.ody, s.o2dy, a.o3[xc ? 0 : 1][1], s.dy, cmy, cpy);
    double uu, vv;
    if (xc) {
      uu = GB_AT(ua, i, j);
      vv = (GB_AT(va, i, j) + GB_AT(va, i, j + 1) + GB_AT(va, i - 1, j) + GB_AT(va, i - 1, j + 1)) * 0.25;
    } else {
      uu = (GB_AT(ua, i, j - 1) + GB_AT(ua, i + 1, j - 1) + GB_AT(ua, i, j) + GB_AT(ua, i + 1, j)) * 0.25;
      vv = GB_AT(va, i, j);
    }
    const bool ux = gtz(uu), vy = gtz(vv);
    const double lam = xc ? GB_AT(lu, i, j) : GB_AT(lv, i, j), w = -a.dt * lam;
    for (int m = 0; m < 7; ++m) {
      out[m] = w * uu * (ux ? cmx[m] : cpx[m]);
      out[7 + m] = w * vv * (vy ? cmy[m] : cpy[m]);
    }
    out[14] = w * (ux ? mx : px);
    out[15] = w * (vy ? my : py);
  };
  const size_t nu = (size_t)(ni + 1) * nj;
  GB_FOR_IJ(i, j, ni + 1, nj) face(true, i, j, co + 16 * ((size_t)j * (ni + 1) + i));
  GB_FOR_IJ(i, j, ni, nj + 1) face(false, i, j, co + 16 * (nu + (size_t)j * ni + i));
}

__global__ void k_eno3_adj_gather(const double* __restrict__ co, double* __restrict__ mua_a, double* __restrict__ mva_a, EnoAdjArgs a) {
  const int ni = a.ni, nj = a.nj;
  const size_t nu = (size_t)(ni + 1) * nj;
  DField mua = dfield(mua_a, 3, ni + 1, nj), mva = dfield(mva_a, 3, ni, nj + 1);
  auto CU = [&](int i, int j, int k) -> double {  // x-face (i, j): 0 <= i <= ni, 0 <= j < nj
    return (i >= 0 && i <= ni && j >= 0 && j < nj) ? co[16 * ((size_t)j * (ni + 1) + i) + k] : 0.0;
  };
  auto CV = [&](int i, int j, int k) -> double {  // y-face (i, j): 0 <= i < ni, 0 <= j <= nj
    return (i >= 0 && i < ni && j >= 0 && j <= nj) ? co[16 * (nu + (size_t)j * ni + i) + k] : 0.0;
  };
  GB_FOR_IJ(ii, jj, ni + 7, nj + 7) {
    const int i = ii - 3, j = jj - 3;
    if (i <= ni + 3 && j <= nj + 2) {  // UA cell
      double acc = CU(i, j, 14);
      for (int m = 0; m < 7; ++m) acc += CU(i + 3 - m, j, m) + CU(i, j + 3 - m, 7 + m);
      acc += 0.25 * (CV(i, j, 14) + CV(i - 1, j, 14) + CV(i, j + 1, 14) + CV(i - 1, j + 1, 14));
      GB_AT(mua, i, j) = acc;
    }
    if (i <= ni + 2 && j <= nj + 3) {  // VA cell
      double acc = CV(i, j, 15);
      for (int m = 0; m < 7; ++m) acc += CV(i + 3 - m, j, m) + CV(i, j + 3 - m, 7 + m);
      acc += 0.25 * (CU(i, j, 15) + CU(i + 1, j, 15) + CU(i, j - 1, 15) + CU(i + 1, j - 1, 15));
      GB_AT(mva, i, j) = acc;
    }
  }
}

// ---- explicit viscosity adjoint ----
// ApplyViscosity (VISCOSITY_2D.h:460-532) as k_flow's FP64 viscous branch without gravity and
// walls (the Sourcing form): each new face value is t0 + coef * (stencil of the old faces), affine
// in U, V, with coef = dt / rho(H(phi)) and the smeared viscosities mu(H(phi)) depending on phi.
// Pass 1 stores per face of both MAC grids 13 cotangent-weighted numbers: the 7 velocity
// coefficients (x-face: +x, -x, +y, -y neighbours, the two cross-term weights, self), 4 phi
// weights (the two face nodes, the upper / lower (right / left) corner averages' quarter shares)
// and the face's shares of dL / d rho_water and dL / d rho_air (through coef).
// Pass 2 gathers them onto every face and node that each stencil read, in a fixed order.
struct ViscAdjArgs {
  int ni, nj;
  double dt, odx, ody, eps, oe;
  double mu_lo, mu_d, mu_at0, mu_at1, rho_lo, rho_d, coef0, coef1;
};

__device__ __forceinline__ double visc_mu(double l, const ViscAdjArgs& a) {
  if (lt_neg(l, a.eps)) return a.mu_at0;
  if (gt_pos(l, a.eps)) return a.mu_at1;
  return a.mu_lo + a.mu_d * heaviside_band(l, a.oe);
}
// coef = dt / rho(H(l)), its slope in l, and its partials in the water and air densities.
__device__ __forceinline__ double visc_coef(double l, const ViscAdjArgs& a, double& dcoef, double& dw, double& da) {
  const double H = lt_neg(l, a.eps) ? 0.0 : (gt_pos(l, a.eps) ? 1.0 : heaviside_band(l, a.oe));
  const double r = a.rho_lo + a.rho_d * H;
  dw = -a.dt * H / (r * r);
  da = -a.dt * (1.0 - H) / (r * r);
  if (lt_neg(l, a.eps)) return dcoef = 0.0, a.coef0;
  if (gt_pos(l, a.eps)) return dcoef = 0.0, a.coef1;
  dcoef = -a.dt * a.rho_d * dheaviside(l, a.eps, a.oe) / (r * r);
  return a.dt * (1 / r);
}

__global__ void k_visc_adj_coef(const double* __restrict__ phi_a, const double* __restrict__ u_a, const double* __restrict__ v_a,
                                const double* __restrict__ lu_a, const double* __restrict__ lv_a, double* __restrict__ C,
                                ViscAdjArgs a) {
  const int ni = a.ni, nj = a.nj;
  const DField phi = dfield((double*)phi_a, 2, ni, nj);
  const DField u = dfield((double*)u_a, 2, ni + 1, nj), v = dfield((double*)v_a, 2, ni, nj + 1);
  const DField lu = dfield((double*)lu_a, 2, ni + 1, nj), lv = dfield((double*)lv_a, 2, ni, nj + 1);
  const size_t nX = (size_t)(ni + 1) * nj, nY = (size_t)ni * (nj + 1);
  auto tu = [&](int i, int j) -> double { return (i < 0 || i > ni || j < 0 || j >= nj) ? 0.0 : GB_AT(u, i, j); };
  auto tv = [&](int i, int j) -> double { return (i < 0 || i >= ni || j < 0 || j > nj) ? 0.0 : GB_AT(v, i, j); };
  auto P = [&](int i, int j) -> double { return GB_AT(phi, i, j); };
  auto dmu = [&](double l) -> double { return a.mu_d * dheaviside(l, a.eps, a.oe); };
  const double ox2 = a.odx * a.odx, oy2 = a.ody * a.ody, oxy = a.odx * a.ody;
  GB_FOR_IJ(i, j, ni + 1, nj + 1) {
    if (j < nj) {  // x-face (i, j): nodes (i-1, j) and (i, j)
      double* o = C + (size_t)j * (ni + 1) + i;
      const double lam = GB_AT(lu, i, j);
      const double pl = P(i - 1, j), pc = P(i, j);
      const double cu = 0.25 * (pl + pc + P(i - 1, j + 1) + P(i, j + 1));
      const double cd = 0.25 * (P(i - 1, j - 1) + P(i, j - 1) + pl + pc);
      double dcoef, dw, da;
      const double coef = visc_coef(0.5 * (pl + pc), a, dcoef, dw, da);
      const double m_cu = visc_mu(cu, a), m_cd = visc_mu(cd, a), m_r = visc_mu(pc, a), m_c = visc_mu(pl, a);
      const double t0 = tu(i, j);
      const double dxp = tu(i + 1, j) - t0, dxm = t0 - tu(i - 1, j);
      const double gup = a.ody * (tu(i, j + 1) - t0) + a.odx * (tv(i, j + 1) - tv(i - 1, j + 1));
      const double gdn = a.ody * (t0 - tu(i, j - 1)) + a.odx * (tv(i, j) - tv(i - 1, j));
      const double axp = coef * 2.0 * ox2 * m_r, axm = coef * 2.0 * ox2 * m_c, ayp = coef * oy2 * m_cu, aym = coef * oy2 * m_cd;
      o[0] = lam * axp;
      o[nX] = lam * axm;
      o[2 * nX] = lam * ayp;
      o[3 * nX] = lam * aym;
      o[4 * nX] = lam * coef * oxy * m_cu;
      o[5 * nX] = lam * coef * oxy * m_cd;
      o[6 * nX] = lam * (1.0 - (axp + axm + ayp + aym));
      const double F = 2.0 * ox2 * (m_r * dxp - m_c * dxm), G = a.ody * (m_cu * gup - m_cd * gdn);
      const double wco = lam * (F + G) * dcoef;
      o[7 * nX] = -lam * coef * 2.0 * ox2 * dxm * dmu(pl) + 0.5 * wco;  // node (i-1, j)
      o[8 * nX] = lam * coef * 2.0 * ox2 * dxp * dmu(pc) + 0.5 * wco;   // node (i, j)
      o[9 * nX] = 0.25 * lam * coef * a.ody * gup * dmu(cu);
      o[10 * nX] = -0.25 * lam * coef * a.ody * gdn * dmu(cd);
      o[11 * nX] = lam * (F + G) * dw;
      o[12 * nX] = lam * (F + G) * da;
    }
    if (i < ni) {  // y-face (i, j): nodes (i, j-1) and (i, j)
      double* o = C + 13 * nX + (size_t)j * ni + i;
      const double lam = GB_AT(lv, i, j);
      const double pb = P(i, j - 1), pc = P(i, j);
      const double cu = 0.25 * (pb + P(i + 1, j - 1) + pc + P(i + 1, j));
      const double cl = 0.25 * (P(i - 1, j - 1) + pb + P(i - 1, j) + pc);
      double dcoef, dw, da;
      const double coef = visc_coef(0.5 * (pb + pc), a, dcoef, dw, da);
      const double m_cu = visc_mu(cu, a), m_cl = visc_mu(cl, a), m_u = visc_mu(pc, a), m_c = visc_mu(pb, a);
      const double t0 = tv(i, j);
      const double dyp = tv(i, j + 1) - t0, dym = t0 - tv(i, j - 1);
      const double grt = a.ody * (tu(i + 1, j) - tu(i + 1, j - 1)) + a.odx * (tv(i + 1, j) - t0);
      const double glf = a.ody * (tu(i, j) - tu(i, j - 1)) + a.odx * (t0 - tv(i - 1, j));
      const double ayp = coef * 2.0 * oy2 * m_u, aym = coef * 2.0 * oy2 * m_c, axp = coef * ox2 * m_cu, axm = coef * ox2 * m_cl;
      o[0] = lam * ayp;
      o[nY] = lam * aym;
      o[2 * nY] = lam * axp;
      o[3 * nY] = lam * axm;
      o[4 * nY] = lam * coef * oxy * m_cu;
      o[5 * nY] = lam * coef * oxy * m_cl;
      o[6 * nY] = lam * (1.0 - (ayp + aym + axp + axm));
      const double F = 2.0 * oy2 * (m_u * dyp - m_c * dym), G = a.odx * (m_cu * grt - m_cl * glf);
      const double wco = lam * (F + G) * dcoef;
      o[7 * nY] = -lam * coef * 2.0 * oy2 * dym * dmu(pb) + 0.5 * wco;  // node (i, j-1)
      o[8 * nY] = lam * coef * 2.0 * oy2 * dyp * dmu(pc) + 0.5 * wco;   // node (i, j)
      o[9 * nY] = 0.25 * lam * coef * a.odx * grt * dmu(cu);
      o[10 * nY] = -0.25 * lam * coef * a.odx * glf * dmu(cl);
      o[11 * nY] = lam * (F + G) * dw;
      o[12 * nY] = lam * (F + G) * da;
    }
  }
}

// Over the (ni + 2) x (nj + 2) index space (x, y): the x-face and the y-face (x, y) where they
// exist, and the node (x - 1, y - 1) of phi's interior and ghost-1 ring.
__global__ void k_visc_adj_gather(const double* __restrict__ C, double* __restrict__ mu_a, double* __restrict__ mv_a,
                                  double* __restrict__ mp_a, int ni, int nj) {
  const size_t nX = (size_t)(ni + 1) * nj, nY = (size_t)ni * (nj + 1);
  const double* CY = C + 13 * nX;
  auto X = [&](int k, int I, int J) -> double {
    return (I < 0 || I > ni || J < 0 || J >= nj) ? 0.0 : C[k * nX + (size_t)J * (ni + 1) + I];
  };
  auto Y = [&](int k, int I, int J) -> double {
    return (I < 0 || I >= ni || J < 0 || J > nj) ? 0.0 : CY[k * nY + (size_t)J * ni + I];
  };
  DField mu = dfield(mu_a, 2, ni + 1, nj), mv = dfield(mv_a, 2, ni, nj + 1), mp = dfield(mp_a, 2, ni, nj);
  GB_FOR_IJ(x, y, ni + 2, nj + 2) {
    if (x <= ni && y < nj) {
      const int i = x, j = y;
      GB_AT(mu, i, j) = X(6, i, j) + X(0, i - 1, j) + X(1, i + 1, j) + X(2, i, j - 1) + X(3, i, j + 1) + Y(4, i - 1, j) -
                        Y(4, i - 1, j + 1) - Y(5, i, j) + Y(5, i, j + 1);
    }
    if (x < ni && y <= nj) {
      const int i = x, j = y;
      GB_AT(mv, i, j) = Y(6, i, j) + Y(0, i, j - 1) + Y(1, i, j + 1) + Y(2, i - 1, j) + Y(3, i + 1, j) + X(4, i, j - 1) -
                        X(4, i + 1, j - 1) - X(5, i, j) + X(5, i + 1, j);
    }
    const int i = x - 1, j = y - 1;
    GB_AT(mp, i, j) = X(8, i, j) + X(7, i + 1, j) + X(9, i, j) + X(9, i + 1, j) + X(9, i, j - 1) + X(9, i + 1, j - 1) +
                      X(10, i, j) + X(10, i + 1, j) + X(10, i, j + 1) + X(10, i + 1, j + 1) + Y(8, i, j) + Y(7, i, j + 1) +
                      Y(9, i, j) + Y(9, i - 1, j) + Y(9, i, j + 1) + Y(9, i - 1, j + 1) + Y(10, i, j) + Y(10, i + 1, j) +
                      Y(10, i, j + 1) + Y(10, i + 1, j + 1);
  }
}


}  // namespace

int density_gradient(gb2d_ctx* c, double dt, double* d_water, double* d_air) {
  const int ni = c->grid.ni, nj = c->grid.nj;
  const dim3 g = grid_ij(ni, nj);
  const size_t nb = (size_t)g.x * g.y;
  DensArgs a;
  a.ni = ni;
  a.nj = nj;
  a.odx = c->base.odx;
  a.ody = c->base.ody;
  a.idx2 = 1.0 / (c->base.dx * c->base.dx);
  a.idy2 = 1.0 / (c->base.dy * c->base.dy);
  a.odx2 = c->base.odx2;
  a.ody2 = c->base.ody2;
  a.dt = dt;
  a.sigma = c->prm.surface_tension;
  a.water = c->prm.water_density;
  a.air = c->prm.air_density;
  a.inv_water = 1.0 / a.water;
  a.inv_air = 1.0 / a.air;
  a.eps_h = 1.5 * c->base.dx;
  a.eps_v = 1.5 * c->base.dy;
  a.oeh = 1.0 / a.eps_h;
  a.oev = 1.0 / a.eps_v;
  double out[2];
  std::vector<double> host(nb);
  for (int w = 0; w < 2; ++w) {
    a.wrt_water = w == 0;
    k_density_grad<<<g, kThreads, 0, c->stream>>>(c->phi_buf[c->phi_cur], c->kappa, c->p, c->xw, c->adj_lam_u, c->adj_lam_v,
                                                   c->adj_gvel, a);
    GB_LAUNCHED(1);
    cudaError_t e = cudaMemcpyAsync(host.data(), c->adj_gvel, nb * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
      snprintf(c->err, sizeof(c->err), "density gradient: %s", cudaGetErrorString(e));
      return GB2D_ERR_CUDA;
    }
    double sum = 0;
    for (size_t k = 0; k < nb; ++k) sum += host[k];
    out[w] = sum;
  }
  if (d_water) *d_water = out[0];
  if (d_air) *d_air = out[1];
  return GB2D_OK;
}

int adjoint_buffers(gb2d_ctx* c) {
  if (c->adj_coef) return GB2D_OK;
  const size_t ni = c->grid.ni, nj = c->grid.nj;
  struct A {
    double** p;
    size_t n;
  } allocs[] = {
      {&c->adj_coef, 14 * ni * nj},           {&c->adj_gvel, 2 * ni * nj},
      {&c->adj_lam_phi, (ni + 4) * (nj + 4)}, {&c->adj_mu_phi, (ni + 4) * (nj + 4)},
      {&c->adj_lam_u, (ni + 5) * (nj + 4)},   {&c->adj_lam_v, (ni + 4) * (nj + 5)},
      {&c->adj_mu_u, (ni + 7) * (nj + 6)},    {&c->adj_mu_v, (ni + 6) * (nj + 7)},
      {&c->adj_lam_p, (ni + 2) * (nj + 2)},    {&c->adj_eno, 16 * ((ni + 1) * nj + ni * (nj + 1))},
  };
  for (auto& a : allocs) {
    cudaError_t e = cudaMalloc(a.p, a.n * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(*a.p, 0, a.n * sizeof(double));
    if (e != cudaSuccess) {
      snprintf(c->err, sizeof(c->err), "adjoint buffers: %s", cudaGetErrorString(e));
      return GB2D_ERR_CUDA;
    }
  }
  return GB2D_OK;
}

void launch_weno5_adjoint(cudaStream_t s, gb2d_ctx* c, double dt, double* mu_ua, double* mu_va) {
  const int ni = c->grid.ni, nj = c->grid.nj;
  AdjArgs a{ni, nj, c->base.odx, c->base.ody, c->prm.weno_epsilon, dt};
  k_extrap_adj_cols<<<(ni + 127) / 128, 128, 0, s>>>(c->adj_lam_phi, ni, nj);
  k_extrap_adj_rows<<<(nj + 127) / 128, 128, 0, s>>>(c->adj_lam_phi, ni, nj);
  k_weno5_adj_coef<<<grid_ij(ni, nj), kThreads, 0, s>>>(c->phi_buf[c->phi_cur], c->ua, c->va, c->adj_lam_phi, c->adj_coef, c->adj_gvel, a);
  k_weno5_adj_gather<<<grid_ij(ni + 4, nj + 4), kThreads, 0, s>>>(c->adj_lam_phi, c->adj_coef, c->adj_mu_phi, a);
  GB_LAUNCHED(4);
  if (mu_ua || mu_va) {
    k_weno5_adj_vel<<<grid_ij(ni + 1, nj + 1), kThreads, 0, s>>>(c->adj_gvel, mu_ua, mu_va, ni, nj);
    GB_LAUNCHED(1);
  }
}

void launch_projection_adjoint_rhs(cudaStream_t s, gb2d_ctx* c, double dt, int with_lam_p) {
  const int ni = c->grid.ni, nj = c->grid.nj;
  ProjAdjArgs a;
  a.ni = ni;
  a.nj = nj;
  a.dt = dt;
  a.odx = c->base.odx;
  a.ody = c->base.ody;
  a.odt = 1.0 / dt;
  a.water = c->prm.water_density;
  a.air = c->prm.air_density;
  a.inv_water = 1.0 / a.water;
  a.inv_air = 1.0 / a.air;
  a.eps_h = 1.5 * c->base.dx;
  a.eps_v = 1.5 * c->base.dy;
  a.oeh = 1.0 / a.eps_h;
  a.oev = 1.0 / a.eps_v;
  k_proj_adj_rhs<<<grid_ij(ni, nj), kThreads, 0, s>>>(c->phi_buf[c->phi_cur], c->adj_lam_u, c->adj_lam_v,
                                                      with_lam_p ? c->adj_lam_p : nullptr, c->rhs, a);
  GB_LAUNCHED(1);
}

void launch_projection_adjoint_vel(cudaStream_t s, gb2d_ctx* c, double dt, const double* z) {
  const int ni = c->grid.ni, nj = c->grid.nj;
  ProjAdjArgs a;
  memset(&a, 0, sizeof a);
  a.ni = ni;
  a.nj = nj;
  a.odx = c->base.odx;
  a.ody = c->base.ody;
  a.odt = 1.0 / dt;
  k_proj_adj_vel<<<grid_ij(ni + 5, nj + 5), kThreads, 0, s>>>(c->adj_lam_u, c->adj_lam_v, z, c->adj_mu_u, c->adj_mu_v, a);
  GB_LAUNCHED(1);
}

int phi_gradient(gb2d_ctx* c, double dt, double* host_out) {
  const int ni = c->grid.ni, nj = c->grid.nj;
  PhiArgs a;
  a.ni = ni;
  a.nj = nj;
  a.odx = c->base.odx;
  a.ody = c->base.ody;
  a.o2dx = c->base.o2dx;
  a.o2dy = c->base.o2dy;
  a.odx2 = c->base.odx2;
  a.ody2 = c->base.ody2;
  a.idx2 = 1.0 / (c->base.dx * c->base.dx);
  a.idy2 = 1.0 / (c->base.dy * c->base.dy);
  a.dt = dt;
  a.sigma = c->prm.surface_tension;
  a.tol = c->base.dx < c->base.dy ? c->base.odx : c->base.ody;
  a.water = c->prm.water_density;
  a.air = c->prm.air_density;
  a.inv_water = 1.0 / a.water;
  a.inv_air = 1.0 / a.air;
  a.eps_h = 1.5 * c->base.dx;
  a.eps_v = 1.5 * c->base.dy;
  a.oeh = 1.0 / a.eps_h;
  a.oev = 1.0 / a.eps_v;
  PhiView v;
  v.phi = dfield(c->phi_buf[c->phi_cur], 2, ni, nj);
  v.P = dfield(c->p, 1, ni, nj);
  v.Z = dfield(c->xw, 1, ni, nj);
  v.lu = dfield(c->adj_lam_u, 2, ni + 1, nj);
  v.lv = dfield(c->adj_lam_v, 2, ni, nj + 1);
  v.kappa = c->kappa;
  v.ni = ni;
  v.nj = nj;
  const size_t nphi = (size_t)(ni + 4) * (nj + 4);
  GB2D_CUDA_TRY(c, cudaMemsetAsync(c->adj_mu_phi, 0, nphi * sizeof(double), c->stream));
  k_phi_grad_kappa<<<grid_ij(ni, nj), kThreads, 0, c->stream>>>(v, a, c->adj_coef);
  k_phi_grad_gather<<<grid_ij(ni + 2, nj + 2), kThreads, 0, c->stream>>>(v, a, c->adj_coef, c->adj_mu_phi);
  const int m = ni > nj ? ni : nj;
  k_extrap_adj_rows<<<(m + 127) / 128, 128, 0, c->stream>>>(c->adj_mu_phi, ni, nj);
  k_extrap_adj_cols<<<(m + 127) / 128, 128, 0, c->stream>>>(c->adj_mu_phi, ni, nj);
  GB_LAUNCHED(4);
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(host_out, c->adj_mu_phi, nphi * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(c->err, sizeof(c->err), "phi gradient: %s", cudaGetErrorString(e));
    return GB2D_ERR_CUDA;
  }
  return GB2D_OK;
}


int eno3_adjoint(gb2d_ctx* c, double dt) {
  const int ni = c->grid.ni, nj = c->grid.nj;
  EnoAdjArgs a;
  a.ni = ni;
  a.nj = nj;
  a.xs = c->xs;
  a.ys = c->ys;
  a.dt = dt;
  const Space* sp[2] = {&c->xs, &c->ys};
  for (int g = 0; g < 2; ++g) {
    a.o3[g][0] = sp[g]->odx / 3;
    a.o3[g][1] = sp[g]->ody / 3;
  }
  k_eno3_adj_face<<<grid_ij(ni + 1, nj + 1), kThreads, 0, c->stream>>>(c->ua, c->va, c->adj_lam_u, c->adj_lam_v, c->adj_eno, a);
  k_eno3_adj_gather<<<grid_ij(ni + 7, nj + 7), kThreads, 0, c->stream>>>(c->adj_eno, c->adj_mu_u, c->adj_mu_v, a);
  GB_LAUNCHED(2);
  return GB2D_OK;
}


int reinit_sweep_vjp(gb2d_ctx* c, const double* phi_dev, const double* sign_dev, const double* lam_dev, double* mu_dev, double* gs_dev) {
  AdjArgs a;
  a.ni = c->grid.ni;
  a.nj = c->grid.nj;
  a.odx = c->base.odx;
  a.ody = c->base.ody;
  a.eps = c->prm.weno_epsilon;
  a.dt = 0.0;
  const double dtau = c->base.dx / (double)c->prm.reinit_scaling;
  k_reinit_adj_coef<<<grid_ij(a.ni, a.nj), kThreads, 0, c->stream>>>(phi_dev, sign_dev, lam_dev, c->adj_coef, gs_dev, a, dtau);
  k_weno5_adj_gather<<<grid_ij(a.ni + 4, a.nj + 4), kThreads, 0, c->stream>>>(lam_dev, c->adj_coef, mu_dev, a);
  GB_LAUNCHED(2);
  return GB2D_OK;
}


// VJP of the Sourcing viscosity at the context's PHI, U, V: lam_u, lam_v (device, U / V
// layouts) -> mu_u, mu_v (U / V layouts) and mu_phi (PHI's layout, nonzero on the interior and
// the ghost-1 ring); d_density (host, may be null) receives dL / d rho_water, dL / d rho_air, the
// faces' shares added on the host in index order.  The 13 numbers of each face live in adj_eno.
int viscosity_vjp(gb2d_ctx* c, double dt, const double* lu, const double* lv, double* mu, double* mv, double* mp,
                  double* d_density) {
  const int ni = c->grid.ni, nj = c->grid.nj;
  ViscAdjArgs a;
  a.ni = ni;
  a.nj = nj;
  a.dt = dt;
  a.odx = c->base.odx;
  a.ody = c->base.ody;
  a.eps = 1.5 * c->base.dx;
  a.oe = 1.0 / a.eps;
  a.mu_lo = c->flow.air_viscosity;
  a.mu_d = c->flow.water_viscosity - c->flow.air_viscosity;
  a.mu_at0 = a.mu_lo + a.mu_d * 0.0;
  a.mu_at1 = a.mu_lo + a.mu_d * 1.0;
  a.rho_lo = c->prm.air_density;
  a.rho_d = c->prm.water_density - c->prm.air_density;
  a.coef0 = dt * (1 / (a.rho_lo + a.rho_d * 0.0));
  a.coef1 = dt * (1 / (a.rho_lo + a.rho_d * 1.0));
  const size_t nu = (size_t)(ni + 5) * (nj + 4), nv = (size_t)(ni + 4) * (nj + 5), np = (size_t)(ni + 4) * (nj + 4);
  GB2D_CUDA_TRY(c, cudaMemsetAsync(mu, 0, nu * sizeof(double), c->stream));
  GB2D_CUDA_TRY(c, cudaMemsetAsync(mv, 0, nv * sizeof(double), c->stream));
  GB2D_CUDA_TRY(c, cudaMemsetAsync(mp, 0, np * sizeof(double), c->stream));
  k_visc_adj_coef<<<grid_ij(ni + 1, nj + 1), kThreads, 0, c->stream>>>(c->phi_buf[c->phi_cur], c->u, c->v, lu, lv, c->adj_eno, a);
  k_visc_adj_gather<<<grid_ij(ni + 2, nj + 2), kThreads, 0, c->stream>>>(c->adj_eno, mu, mv, mp, ni, nj);
  GB_LAUNCHED(2);
  if (!d_density) return GB2D_OK;
  const size_t nX = (size_t)(ni + 1) * nj, nY = (size_t)ni * (nj + 1);
  std::vector<double> h(2 * (nX + nY));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(h.data(), c->adj_eno + 11 * nX, 2 * nX * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  GB2D_CUDA_TRY(c, cudaMemcpyAsync(h.data() + 2 * nX, c->adj_eno + 13 * nX + 11 * nY, 2 * nY * sizeof(double),
                                   cudaMemcpyDeviceToHost, c->stream));
  GB2D_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  double w = 0.0, a_ = 0.0;
  for (size_t k = 0; k < nX; ++k) w += h[k], a_ += h[nX + k];
  for (size_t k = 0; k < nY; ++k) w += h[2 * nX + k], a_ += h[2 * nX + nY + k];
  d_density[0] = w;
  d_density[1] = a_;
  return GB2D_OK;
}

}  // namespace gb2d
