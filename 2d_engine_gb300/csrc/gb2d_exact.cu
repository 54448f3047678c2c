// FP64 kernels that reproduce the reference's own FP64 CPU arithmetic: ghost
// fills, WENO5 advection and reinitialisation sweeps, ENO3 velocity advection,
// curvature, ghost-fluid Poisson assembly and the GFM velocity update.
// Built with --fmad=false: every multiply and add rounds separately, in the
// reference's association order, so results match it bit for bit (the sine of
// the smeared Heaviside is the only libm call and may differ in the last ulp).
// The "mixed" advection variants (FP32 flux evaluation, FP64 state) live here
// too so that they share the loaders.
#include <cstdio>
#include <cstdlib>

#include "gb2d_internal.cuh"
#include "gb2d_schemes.cuh"

namespace gb2d {

namespace {

inline unsigned blocks_for(size_t n, int threads = kThreads) { return (unsigned)((n + threads - 1) / threads); }

// x * y >= 0 as IEEE evaluates it.  When both are normal and finite and the
// product's exponent keeps it above the subnormal range, only the signs decide;
// zeros, subnormals, infinities, NaN and products that may round to zero take
// the FP64 multiply.
__device__ __forceinline__ bool prod_ge0(double x, double y) {
  const long long bx = __double_as_longlong(x), by = __double_as_longlong(y);
  const int ex = (int)((bx >> 52) & 0x7ff), ey = (int)((by >> 52) & 0x7ff);
  if (ex != 0 && ey != 0 && ex != 0x7ff && ey != 0x7ff && ex + ey >= 972) return (bx ^ by) >= 0;
  return x * y >= 0;
}


// FillGhostCellsFrom (FIELD_STRUCTURE_2D.h:374-449): interior copied, each ghost
// layer copies the second interior line, corners untouched.
__global__ void k_fill_ghost_copy(double* dst_a, int gd, const double* __restrict__ src_a, int gs, int nI, int nJ, int g) {
  DField d = dfield(dst_a, gd, nI, nJ);
  DField s = dfield((double*)src_a, gs, nI, nJ);
  GB_FOR_IJ(ii, jj, nI + 2 * g, nJ + 2 * g) {
    int i = ii - g, j = jj - g;
    bool in_i = i >= 0 && i < nI, in_j = j >= 0 && j < nJ;
    if (in_i && in_j)
      GB_AT(d, i, j) = GB_AT(s, i, j);
    else if (in_j)
      GB_AT(d, i, j) = GB_AT(s, i < 0 ? 1 : nI - 2, j);
    else if (in_i)
      GB_AT(d, i, j) = GB_AT(s, i, j < 0 ? 1 : nJ - 2);
  }
}

// FillGhostCellsContinuousDerivativesFrom(phi, true, tid) on the field itself
// (FIELD_STRUCTURE_2D.h:641-716).  One thread per boundary line keeps the
// reference's layer order: left/bottom outermost first (the outer layer reads
// the previous inner value), right/top innermost first.
__global__ void k_extrapolate(double* a, int g, int nI, int nJ) {
  DField f = dfield(a, g, nI, nJ);
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nJ) {
    int j = t;
    for (int i = -g; i <= -1; ++i) GB_AT(f, i, j) = 2.0 * GB_AT(f, i + 1, j) - GB_AT(f, i + 2, j);
    for (int i = nI; i <= nI - 1 + g; ++i) GB_AT(f, i, j) = 2.0 * GB_AT(f, i - 1, j) - GB_AT(f, i - 2, j);
  }
  if (t < nI) {
    int i = t;
    for (int j = nJ; j <= nJ - 1 + g; ++j) GB_AT(f, i, j) = 2.0 * GB_AT(f, i, j - 1) - GB_AT(f, i, j - 2);
    for (int j = -g; j <= -1; ++j) GB_AT(f, i, j) = 2.0 * GB_AT(f, i, j + 1) - GB_AT(f, i, j + 2);
  }
}

// Reads of the WENO scratch copy (scalar_field_ghost, ghost 3) synthesised from
// phi's interior: ghost layers hold the second interior line.
__device__ __forceinline__ void gather_x(const DField& s, int i, int j, double q[7]) {
  const int nI = s.nI;
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    int ii = i - 3 + k;
    ii = ii < 0 ? 1 : (ii >= nI ? nI - 2 : ii);
    q[k] = __ldg(&GB_AT(s, ii, j));
  }
}
__device__ __forceinline__ void gather_y(const DField& s, int i, int j, double q[7]) {
  const int nJ = s.nJ;
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    int jj = j - 3 + k;
    jj = jj < 0 ? 1 : (jj >= nJ ? nJ - 2 : jj);
    q[k] = __ldg(&GB_AT(s, i, jj));
  }
}

struct LSArgs {
  int ni, nj;
  double odx, ody, eps;
  float odx_f, ody_f, eps_f;  // the same in FP32 for the FP32 flux path
};

// WENO5th (ADVECTION_METHOD_2D.h:508-663) for the node-grid level set: writes
// dst's interior from src, copies src's ghost ring (the sweep leaves phi's own
// ghosts to the caller's extrapolation).
template <bool MIXED>
__global__ void k_weno5_advect(const double* __restrict__ src_a, double* __restrict__ dst_a, const double* __restrict__ ua_a,
                               const double* __restrict__ va_a, LSArgs a, DtArg dt_arg) {
  int ni = a.ni, nj = a.nj;
  const double dt = dt_arg.get();
  int W = ni + 4, H = nj + 4;
  int ix = blockIdx.x * blockDim.x + threadIdx.x, jy = blockIdx.y * blockDim.y + threadIdx.y;
  if (ix >= W || jy >= H) return;
  int i = ix - 2, j = jy - 2;
  DField src = dfield((double*)src_a, 2, ni, nj), dst = dfield(dst_a, 2, ni, nj);
  if (i < 0 || j < 0 || i >= ni || j >= nj) {
    GB_AT(dst, i, j) = GB_AT(src, i, j);
    return;
  }
  DField ua = dfield((double*)ua_a, 3, ni + 1, nj), va = dfield((double*)va_a, 3, ni, nj + 1);
  double q[7];
  double u = (__ldg(&GB_AT(ua, i + 1, j)) + __ldg(&GB_AT(ua, i, j))) * 0.5;
  double v = (__ldg(&GB_AT(va, i, j + 1)) + __ldg(&GB_AT(va, i, j))) * 0.5;
  double fx, fy;
  if (MIXED) {
    float m, p;
    gather_x(src, i, j, q);
    weno5_pair_f32(q, a.odx_f, a.eps_f, m, p);
    fx = gtz(u) ? widen(m) : widen(p);
    gather_y(src, i, j, q);
    weno5_pair_f32(q, a.ody_f, a.eps_f, m, p);
    fy = gtz(v) ? widen(m) : widen(p);
  } else {
    double m, p;
    gather_x(src, i, j, q);
    weno5_pair(q, a.odx, a.eps, m, p);
    fx = gtz(u) ? m : p;
    gather_y(src, i, j, q);
    weno5_pair(q, a.ody, a.eps, m, p);
    fy = gtz(v) ? m : p;
  }
  GB_AT(dst, i, j) = GB_AT(src, i, j) - dt * (u * fx + v * fy);
}

// Sign function of Reinitialization (EULERIAN_FLUID_SOLVER_2D.h:2431-2435).
__global__ void k_reinit_sign(const double* __restrict__ phi_a, double* __restrict__ S, int ni, int nj, double dx) {
  DField phi = dfield((double*)phi_a, 2, ni, nj);
  GB_FOR_IJ(i, j, ni, nj) {
    const size_t t = (size_t)j * ni + i;
    double p = GB_AT(phi, i, j);
    S[t] = p / sqrt(p * p + dx * dx);
  }
}

// WENO5thReinitialization (ADVECTION_METHOD_2D.h:1401-1658).
template <bool MIXED>
__global__ void k_reinit_sweep(const double* __restrict__ src_a, double* __restrict__ dst_a, const double* __restrict__ S, LSArgs a,
                               double dtau) {
  int ni = a.ni, nj = a.nj;
  int W = ni + 4, H = nj + 4;
  int ix = blockIdx.x * blockDim.x + threadIdx.x, jy = blockIdx.y * blockDim.y + threadIdx.y;
  if (ix >= W || jy >= H) return;
  int i = ix - 2, j = jy - 2;
  DField src = dfield((double*)src_a, 2, ni, nj), dst = dfield(dst_a, 2, ni, nj);
  double old = GB_AT(src, i, j);
  if (i < 0 || j < 0 || i >= ni || j >= nj) {
    GB_AT(dst, i, j) = old;
    return;
  }
  double q[7];
  double out = old;
  if (MIXED) {
    float mx, px, my, py, h;
    gather_x(src, i, j, q);
    weno5_pair_f32(q, a.odx_f, a.eps_f, mx, px);
    gather_y(src, i, j, q);
    weno5_pair_f32(q, a.ody_f, a.eps_f, my, py);
    double s = __ldg(&S[i + (size_t)j * ni]);
    if (godunov_h<float>(narrow(s), mx, px, my, py, h)) out = old - dtau * s * widen(h);
  } else {
    double mx, px, my, py, h;
    gather_x(src, i, j, q);
    weno5_pair(q, a.odx, a.eps, mx, px);
    gather_y(src, i, j, q);
    weno5_pair(q, a.ody, a.eps, my, py);
    double s = __ldg(&S[i + (size_t)j * ni]);
    if (godunov_h<double>(s, mx, px, my, py, h)) out = old - dtau * s * h;
  }
  GB_AT(dst, i, j) = out;
}

// The mixed reinit sweep, tiled: the WENO first differences of a node and of its
// neighbours overlap, so one 32 x 8 tile stages phi with a 3-node halo (positions mapped
// as the ghost-filled copy maps them) and forms every FP64 difference once (2.8 per node
// instead of 12; FP64 issue is this kernel's bound), narrowed to FP32 in shared memory.
// Each node then reads its 6 + 6 differences: the same values as the per-node gathers,
// so the results equal k_reinit_sweep<true>'s bit for bit.
constexpr int kRtX = 32, kRtY = 8;
__global__ void __launch_bounds__(kRtX* kRtY) k_reinit_sweep_tiled(const double* __restrict__ src_a, double* __restrict__ dst_a,
                                                                    const double* __restrict__ S, LSArgs a, double dtau) {
  __shared__ double ph[kRtY + 6][kRtX + 6];
  __shared__ float dxs[kRtY][kRtX + 5];
  __shared__ float dys[kRtY + 5][kRtX];
  const int ni = a.ni, nj = a.nj, tx = threadIdx.x, ty = threadIdx.y;
  const int i0 = (int)blockIdx.x * kRtX - 2, j0 = (int)blockIdx.y * kRtY - 2;  // tile origin in node coordinates
  const DField src = dfield((double*)src_a, 2, ni, nj), dst = dfield(dst_a, 2, ni, nj);
  for (int k = ty * kRtX + tx; k < (kRtX + 6) * (kRtY + 6); k += kRtX * kRtY) {
    const int x = k % (kRtX + 6), y = k / (kRtX + 6);
    int ii = i0 - 3 + x, jj = j0 - 3 + y;
    ii = ii < 0 ? 1 : (ii >= ni ? ni - 2 : ii);
    jj = jj < 0 ? 1 : (jj >= nj ? nj - 2 : jj);
    ph[y][x] = __ldg(&GB_AT(src, ii, jj));
  }
  __syncthreads();
  for (int k = ty * kRtX + tx; k < kRtY * (kRtX + 5); k += kRtX * kRtY) {
    const int p = k % (kRtX + 5), r = k / (kRtX + 5);
    dxs[r][p] = narrow(ph[r + 3][p + 1] - ph[r + 3][p]);
  }
  for (int k = ty * kRtX + tx; k < (kRtY + 5) * kRtX; k += kRtX * kRtY) {
    const int c = k % kRtX, p = k / kRtX;
    dys[p][c] = narrow(ph[p + 1][c + 3] - ph[p][c + 3]);
  }
  __syncthreads();
  const int i = i0 + tx, j = j0 + ty;
  if (i > ni + 1 || j > nj + 1) return;
  if (i < 0 || j < 0 || i >= ni || j >= nj) {  // the ghost ring is copied
    GB_AT(dst, i, j) = GB_AT(src, i, j);
    return;
  }
  const double old = ph[ty + 3][tx + 3];
  double out = old;
  float d[6], mx, px, my, py, h;
#pragma unroll
  for (int k = 0; k < 6; ++k) d[k] = dxs[ty][tx + k] * a.odx_f;
  mx = weno5_side<float>(d[0], d[1], d[2], d[3], d[4], a.eps_f);
  px = weno5_side<float>(d[5], d[4], d[3], d[2], d[1], a.eps_f);
#pragma unroll
  for (int k = 0; k < 6; ++k) d[k] = dys[ty + k][tx] * a.ody_f;
  my = weno5_side<float>(d[0], d[1], d[2], d[3], d[4], a.eps_f);
  py = weno5_side<float>(d[5], d[4], d[3], d[2], d[1], a.eps_f);
  const double sv = __ldg(&S[i + (size_t)j * ni]);
  if (godunov_h<float>(narrow(sv), mx, px, my, py, h)) out = old - dtau * sv * widen(h);
  GB_AT(dst, i, j) = out;
}

// Shu-Osher blend of the TVD-RK3 stages (EULERIAN_FLUID_SOLVER_2D.h:1706-1741): interior only.
__global__ void k_blend(const double* __restrict__ keep_a, double* phi_a, int ni, int nj, double c0, double c1) {
  DField keep = dfield((double*)keep_a, 2, ni, nj), phi = dfield(phi_a, 2, ni, nj);
  GB_FOR_IJ(i, j, ni, nj) {
    GB_AT(phi, i, j) = c0 * GB_AT(keep, i, j) + c1 * GB_AT(phi, i, j);
  }
}

struct EnoArgs {
  int ni, nj;
  Space xs, ys;
  double o3[2][2];  // 1/(3h) of x and y for the x-face grid [0] and the y-face grid [1], host IEEE quotients
  // FP32 path, per face grid: 1/h, 1/(2h), 1/(3h), h for x ([0..3]) and y ([4..7])
  float xs_f[8], ys_f[8];
};

// ENO3rd on both MAC components (ADVECTION_METHOD_2D.h:2038-2231) as called by
// Solve_Velocity (ADVECTION_2D.cpp:83-122): both read only the advecting copies
// UA/VA (already refreshed from U/V), so one launch updates U and V.
// MIXED: divided differences and the ENO selection in FP32 (first differences,
// face velocities and the update in FP64).
template <bool MIXED>
__global__ void k_eno3(double* __restrict__ u_a, double* __restrict__ v_a, const double* __restrict__ ua_a, const double* __restrict__ va_a,
                       EnoArgs a, DtArg dt_arg) {
  int ni = a.ni, nj = a.nj;
  const double dt = dt_arg.get();
  DField ua = dfield((double*)ua_a, 3, ni + 1, nj), va = dfield((double*)va_a, 3, ni, nj + 1);
  auto face = [&](bool xc, int i, int j) {
    const DField& g = xc ? ua : va;
    const Space& s = xc ? a.xs : a.ys;
    const float* sf = xc ? a.xs_f : a.ys_f;
    double q[7];
    double mx, px, my, py;
    for (int m = 0; m < 7; ++m) q[m] = __ldg(&GB_AT(g, i - 3 + m, j));
    if (MIXED) {
      float m32, p32;
      eno3_pair_f32(q, sf[0], sf[1], sf[2], sf[3], m32, p32);
      mx = widen(m32);
      px = widen(p32);
    } else {
      eno3_pair(q, s.odx, s.o2dx, a.o3[xc ? 0 : 1][0], s.dx, mx, px);
    }
    for (int m = 0; m < 7; ++m) q[m] = __ldg(&GB_AT(g, i, j - 3 + m));
    if (MIXED) {
      float m32, p32;
      eno3_pair_f32(q, sf[4], sf[5], sf[6], sf[7], m32, p32);
      my = widen(m32);
      py = widen(p32);
    } else {
      eno3_pair(q, s.ody, s.o2dy, a.o3[xc ? 0 : 1][1], s.dy, my, py);
    }
    double uu, vv;
    if (xc) {
      uu = GB_AT(ua, i, j);
      vv = (GB_AT(va, i, j) + GB_AT(va, i, j + 1) + GB_AT(va, i - 1, j) + GB_AT(va, i - 1, j + 1)) * 0.25;
    } else {
      uu = (GB_AT(ua, i, j - 1) + GB_AT(ua, i + 1, j - 1) + GB_AT(ua, i, j) + GB_AT(ua, i + 1, j)) * 0.25;
      vv = GB_AT(va, i, j);
    }
    double fx = gtz(uu) ? mx : px, fy = gtz(vv) ? my : py;
    DField out = xc ? dfield(u_a, 2, ni + 1, nj) : dfield(v_a, 2, ni, nj + 1);
    GB_AT(out, i, j) = GB_AT(out, i, j) - dt * (uu * fx + vv * fy);
  };
  GB_FOR_IJ(i, j, ni + 1, nj) face(true, i, j);
  GB_FOR_IJ(i, j, ni, nj + 1) face(false, i, j);
}

// ComputeCurvaturesThread with curvature_by_levelset (LEVELSET_2D.h:898-990);
// phi's ghosts must already be extrapolated.
__global__ void k_curvature(const double* __restrict__ phi_a, double* __restrict__ kappa, int ni, int nj, Space s, int* flag) {
  DField phi = dfield((double*)phi_a, 2, ni, nj);
  const double tol = s.dx < s.dy ? s.odx : s.ody;  // 1 / min(dx, dy), taken on the host
  GB_FOR_IJ(i, j, ni, nj) {
    const size_t t = (size_t)j * ni + i;
    double c = GB_AT(phi, i, j);
    double l = GB_AT(phi, i - 1, j), r = GB_AT(phi, i + 1, j), b = GB_AT(phi, i, j - 1), tp = GB_AT(phi, i, j + 1);
    double px = (r - l) * s.o2dx;
    double py = (tp - b) * s.o2dy;
    double pxx = (r - 2 * c + l) * s.odx2;
    double pyy = (tp - 2 * c + b) * s.ody2;
    double pxy = (GB_AT(phi, i + 1, j + 1) - GB_AT(phi, i + 1, j - 1) - GB_AT(phi, i - 1, j + 1) + GB_AT(phi, i - 1, j - 1)) * s.o2dx * s.o2dy;
    double mag = sqrt(px * px + py * py);
    double deno = mag * mag * mag;
    double curv;
    if ((__double_as_longlong(deno) & kAbsBits) != 0) {  // deno != 0 (NaN included)
      double od = 1.0 / deno;
      curv = -(px * px * pyy - 2.0 * px * py * pxy + py * py * pxx) * od;
    } else {
      px = (r - c) * s.odx;
      py = (tp - c) * s.ody;
      mag = sqrt(px * px + py * py);
      deno = mag * mag * mag;
      if ((__double_as_longlong(deno) & kAbsBits) == 0) {  // deno == 0
        atomicOr(flag, 2);
        continue;
      }
      double od = 1.0 / deno;
      curv = -(px * px * pyy - 2.0 * px * py * pxy + py * py * pxx) * od;
    }
    // Clamp to [-tol, tol] with IEEE comparisons (tol > 0 finite; a NaN stores nothing)
    const long long cb = __double_as_longlong(curv), cm = cb & kAbsBits, tb = __double_as_longlong(tol);
    if (cm <= tb)
      kappa[t] = curv;
    else if (cm <= kInfBits)
      kappa[t] = cb > 0 ? tol : -tol;
  }
}

struct AsmArgs {
  int ni, nj;
  Space s;
  double water, air, sigma, one_over_dt, inv_dxdx, inv_dydy;
  double inv_water, inv_air;  // 1/water, 1/air: IEEE quotients taken once on the host
  const double* dtp;          // non-null: the time step is read here (one_over_dt = 1 / *dtp, IEEE)
  double oeh, oev;            // 1 / (1.5 dx), 1 / (1.5 dy): smeared-Heaviside scales
};

// 1/rho of a node.  The density takes two values, so the quotient is a select of
// the host's correctly rounded reciprocals (FP64 divides are scarce on this part).
__device__ __forceinline__ double inv_density(double phi, const AsmArgs& a) {
  if (lez(phi)) return a.inv_air;
  if (gtz(phi)) return a.inv_water;
  return 1.0;
}

// 1/rho at a node or at its copied ghost (POISSON_SOLVER.cpp:131-138: the ghost
// layer copies the second interior line).
__device__ __forceinline__ double vnode(const DField& phi, int i, int j, const AsmArgs& a) {
  i = i < 0 ? 1 : (i >= a.ni ? a.ni - 2 : i);
  j = j < 0 ? 1 : (j >= a.nj ? a.nj - 2 : j);
  return inv_density(GB_AT(phi, i, j), a);
}

__device__ __forceinline__ double face_beta(double vc, double vn, double pc, double pn) {
  return vc * vn * (fabs(pn) + fabs(pc)) / (vc * fabs(pn) + vn * fabs(pc));
}

// Face weights of BuildLinearSystemNodeJumpConditionVaribleCoefficient
// (POISSON_SOLVER.cpp:743-746): one value per face, symmetric in IEEE arithmetic.
__global__ void k_faces(const double* __restrict__ phi_a, double* __restrict__ bx, double* __restrict__ by, AsmArgs a) {
  int ni = a.ni, nj = a.nj;
  DField phi = dfield((double*)phi_a, 2, ni, nj);
  GB_FOR_IJ(i, j, ni + 1, nj) {
    bx[(size_t)j * (ni + 1) + i] = face_beta(vnode(phi, i, j, a), vnode(phi, i - 1, j, a), GB_AT(phi, i, j), GB_AT(phi, i - 1, j));
  }
  GB_FOR_IJ(i, j, ni, nj + 1) {
    by[(size_t)j * ni + i] = face_beta(vnode(phi, i, j, a), vnode(phi, i, j - 1, a), GB_AT(phi, i, j), GB_AT(phi, i, j - 1));
  }
}

__device__ __forceinline__ double jc_at(const double* kappa, int i, int j, const AsmArgs& a) {
  if (i < 0 || j < 0 || i >= a.ni || j >= a.nj) return 0.0;  // jc_on_solution ghosts stay zero
  return a.sigma * kappa[i + (size_t)j * a.ni];
}

// Jump flux of one arm (POISSON_SOLVER.cpp:881-948) without the derivative-jump
// part, which vanishes because jc_on_derivative is zeroed (PROJECTION_2D.h:501-504).
// Left/bottom and right/top arms follow the same sign rule.  The jump values are
// read only on arms that cross the interface.
__device__ __forceinline__ double arm_flux(double pc, double pn, double jcc, const double* kappa, int in, int jn, double beta, double o2,
                                           const AsmArgs& a) {
  const bool cneg = lez(pc), nneg = lez(pn);
  if (cneg && !nneg && gtz(pn)) {
    double ac = fabs(pc), an = fabs(pn);
    double av = (jcc * an + jc_at(kappa, in, jn, a) * ac) / (ac + an);
    return o2 * av * beta;
  }
  if (!cneg && gtz(pc) && nneg) {
    double ac = fabs(pc), an = fabs(pn);
    double av = (jcc * an + jc_at(kappa, in, jn, a) * ac) / (ac + an);
    return -o2 * av * beta;
  }
  return 0.0;
}

// Diagonal (dx^2 only, POISSON_SOLVER.cpp:872): the face weights of the FULL arms and
// the first cell's Neumann arms (the corner pin).
__global__ void k_diag(const double* __restrict__ bx, const double* __restrict__ by, double* __restrict__ diag, AsmArgs a) {
  int ni = a.ni, nj = a.nj;
  GB_FOR_IJ(i, j, ni, nj) {
    const size_t t = (size_t)j * ni + i;
    double bl = bx[i + (size_t)j * (ni + 1)], br = bx[i + 1 + (size_t)j * (ni + 1)];
    double bb = by[i + (size_t)j * ni], bt = by[i + (size_t)(j + 1) * ni];
    double coef = 0;
    if (i > 0) coef += bl;
    if (i < ni - 1) coef += br;
    if (j > 0) coef += bb;
    if (j < nj - 1) coef += bt;
    if (i == 0 && j == 0) {  // Neumann arms of the first cell (POISSON_SOLVER.cpp:789-806)
      if (i - 1 < 0) coef += bl;
      if (i + 1 > ni - 1) coef += br;
      if (j - 1 < 0) coef += bb;
      if (j + 1 > nj - 1) coef += bt;
    }
    if ((__double_as_longlong(coef) & kAbsBits) == 0) coef = 1;  // coef == 0
    diag[t] = a.inv_dxdx * coef;
  }
}

// Right-hand side -div - F_X - F_Y (POISSON_SOLVER.cpp:878-948).
__global__ void k_rhs(const double* __restrict__ phi_a, const double* __restrict__ kappa, const double* __restrict__ u_a,
                      const double* __restrict__ v_a, const double* __restrict__ bx, const double* __restrict__ by, double* __restrict__ rhs,
                      AsmArgs a) {
  int ni = a.ni, nj = a.nj;
  const double one_over_dt = a.dtp ? 1.0 / *a.dtp : a.one_over_dt;
  DField phi = dfield((double*)phi_a, 2, ni, nj);
  DField u = dfield((double*)u_a, 2, ni + 1, nj), v = dfield((double*)v_a, 2, ni, nj + 1);
  GB_FOR_IJ(i, j, ni, nj) {
    const size_t t = (size_t)j * ni + i;
    double bl = bx[i + (size_t)j * (ni + 1)], br = bx[i + 1 + (size_t)j * (ni + 1)];
    double bb = by[i + (size_t)j * ni], bt = by[i + (size_t)(j + 1) * ni];
    double pc = GB_AT(phi, i, j);
    double jcc = jc_at(kappa, i, j, a);
    double FL = arm_flux(pc, GB_AT(phi, i - 1, j), jcc, kappa, i - 1, j, bl, a.s.odx2, a);
    double FR = arm_flux(pc, GB_AT(phi, i + 1, j), jcc, kappa, i + 1, j, br, a.s.odx2, a);
    double FB = arm_flux(pc, GB_AT(phi, i, j - 1), jcc, kappa, i, j - 1, bb, a.s.ody2, a);
    double FT = arm_flux(pc, GB_AT(phi, i, j + 1), jcc, kappa, i, j + 1, bt, a.s.ody2, a);
    double div = a.s.odx * (GB_AT(u, i + 1, j) - GB_AT(u, i, j)) + a.s.ody * (GB_AT(v, i, j + 1) - GB_AT(v, i, j));
    div *= one_over_dt;
    double FX = FL + FR, FY = FB + FT;
    rhs[t] = -div - FX - FY;
  }
}

// CSR_MATRIX::Multiply in the builder's row order (left, right, bottom, top, diagonal).
__global__ void k_apply_exact(const double* __restrict__ bx, const double* __restrict__ by, const double* __restrict__ diag,
                              const double* __restrict__ x, double* __restrict__ y, int ni, int nj, double idx2, double idy2) {
  GB_FOR_IJ(i, j, ni, nj) {
    const size_t t = (size_t)j * ni + i;
    double acc = 0;
    if (i > 0) acc += -bx[i + (size_t)j * (ni + 1)] * idx2 * x[t - 1];
    if (i < ni - 1) acc += -bx[i + 1 + (size_t)j * (ni + 1)] * idx2 * x[t + 1];
    if (j > 0) acc += -by[i + (size_t)j * ni] * idy2 * x[t - ni];
    if (j < nj - 1) acc += -by[i + (size_t)(j + 1) * ni] * idy2 * x[t + ni];
    acc += diag[t] * x[t];
    y[t] = acc;
  }
}

// UpdateVelocityByPressureGradientVariableDensity (PROJECTION_2D.h:1297-1416):
// same-sign faces use the node density on the + side, interface faces the
// smeared-Heaviside density of the face-averaged phi (eps = 1.5 dx) and the
// |phi|-weighted jump.  Pressure ghosts are zero; wall faces (bc < 0) are skipped.
__global__ void k_velocity_update(const double* __restrict__ phi_a, const double* __restrict__ p_a, const double* __restrict__ kappa,
                                  double* __restrict__ u_a, double* __restrict__ v_a, AsmArgs a, DtArg dt_arg, Scalars* sc) {
  int ni = a.ni, nj = a.nj;
  const double dt = dt_arg.get();
  DField phi = dfield((double*)phi_a, 2, ni, nj), p = dfield((double*)p_a, 1, ni, nj);
  DField u = dfield(u_a, 2, ni + 1, nj), v = dfield(v_a, 2, ni, nj + 1);
  const double odx = a.s.odx, ody = a.s.ody;  // 1 / dx, 1 / dy, taken on the host
  double eh = 1.5 * a.s.dx, ev = 1.5 * a.s.dy;
  unsigned long long mx = 0, my = 0;  // bits of max |u|, |v| (non-negative doubles order as integers)
  auto face = [&](bool xc, int i, int j) {
    int in = xc ? i - 1 : i, jn = xc ? j : j - 1;
    double l0 = GB_AT(phi, i, j), ln = GB_AT(phi, in, jn);
    double oor = lez(l0) ? a.inv_air : a.inv_water;  // 1 / rho_ij
    double dp = GB_AT(p, i, j) - GB_AT(p, in, jn);
    double od = xc ? odx : ody;
    double* w = xc ? &GB_AT(u, i, j) : &GB_AT(v, i, j);
    if (prod_ge0(l0, ln)) {
      *w -= dt * dp * oor * od;
    } else {
      double jcc = jc_at(kappa, i, j, a), jcn = jc_at(kappa, in, jn, a);
      double gam = (jcn * fabs(l0) + jcc * fabs(ln)) / (fabs(l0) + fabs(ln));
      double dh = a.air + (a.water - a.air) * heaviside(0.5 * (l0 + ln), xc ? eh : ev, xc ? a.oeh : a.oev);
      double odh = 1 / dh;
      if (ltz(l0))
        *w -= dt * (dp + gam) * odh * od;
      else if (gtz(l0))
        *w -= dt * (dp - gam) * odh * od;
    }
    unsigned long long& m = xc ? mx : my;
    m = abs_max_bits(*w, m);
  };
  GB_FOR_IJ(i, j, ni, nj) {
    face(true, i, j);
    face(false, i, j);
  }
  block_max_bits(mx, &sc->maxu_bits);
  block_max_bits(my, &sc->maxv_bits);
}

__global__ void k_copy_interior(const double* __restrict__ src_a, int gs, double* __restrict__ dst_a, int gd, int nI, int nJ) {
  DField s = dfield((double*)src_a, gs, nI, nJ), d = dfield(dst_a, gd, nI, nJ);
  GB_FOR_IJ(i, j, nI, nJ) {
    GB_AT(d, i, j) = GB_AT(s, i, j);
  }
}

// FastSweepingMethodOriginal (LEVELSET_2D.h:281-384): the fixed band |phi| < 2 dx.
__global__ void k_fsm_fixed(const double* __restrict__ phi_a, double* __restrict__ fixed, int ni, int nj, double nb) {
  const DField phi = dfield((double*)phi_a, 2, ni, nj);
  GB_FOR_IJ(i, j, ni, nj) { fixed[(size_t)j * ni + i] = fabs(GB_AT(phi, i, j)) < nb ? 1.0 : 0.0; }
}

// The single-threaded FillGhostCellsContinuousDerivativesFrom (FIELD_STRUCTURE_2D.h:584-639):
// each side innermost layer first.  Thread k extrapolates row k's left and right ghosts and
// column k's top and bottom ghosts (disjoint ghost cells, interior reads only).
__global__ void k_extrapolate_inner_first(double* a, int g, int nI, int nJ) {
  const DField f = dfield(a, g, nI, nJ);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < (nI > nJ ? nI : nJ); k += gridDim.x * blockDim.x) {
    if (k < nJ) {
      for (int i = -1; i >= -g; --i) GB_AT(f, i, k) = 2.0 * GB_AT(f, i + 1, k) - GB_AT(f, i + 2, k);
      for (int i = nI; i <= nI - 1 + g; ++i) GB_AT(f, i, k) = 2.0 * GB_AT(f, i - 1, k) - GB_AT(f, i - 2, k);
    }
    if (k < nI) {
      for (int j = nJ; j <= nJ - 1 + g; ++j) GB_AT(f, k, j) = 2.0 * GB_AT(f, k, j - 1) - GB_AT(f, k, j - 2);
      for (int j = -1; j >= -g; --j) GB_AT(f, k, j) = 2.0 * GB_AT(f, k, j + 1) - GB_AT(f, k, j + 2);
    }
  }
}

// One Gauss-Seidel sweep of LEVELSET_2D::Sweep (LEVELSET_2D.h:507-589) in direction dir
// (0: i+ j+, 1: i- j+, 2: i- j-, 3: i+ j-).  The reference visits rows in order and
// nodes within a row in order; a node reads its two predecessors along i and j (already
// updated) and its two successors (not yet).  Anti-diagonal wavefronts in sweep
// coordinates have the same dependencies, so one block walks them in turn, one barrier
// per wavefront, and produces the reference's values bit for bit.
__global__ void k_fsm_sweep(double* phi_a, const double* __restrict__ fixed, int ni, int nj, double h, int dir) {
  const DField phi = dfield(phi_a, 2, ni, nj);
  const double one_over_two = 1.0 / 2.0, hh = h * h, hh2 = hh * 2.0;
  const bool irev = dir == 1 || dir == 2, jrev = dir == 2 || dir == 3;
  for (int d = 0; d <= ni + nj - 2; ++d) {
    const int lo = d - (nj - 1) > 0 ? d - (nj - 1) : 0, hi = d < ni - 1 ? d : ni - 1;
    for (int a = lo + (int)threadIdx.x; a <= hi; a += blockDim.x) {
      const int i = irev ? ni - 1 - a : a, jj = d - a, j = jrev ? nj - 1 - jj : jj;
      if (fixed[(size_t)j * ni + i] != 0.0) continue;
      double* pc = &GB_AT(phi, i, j);
      const double c = *pc, l = GB_AT(phi, i - 1, j), r = GB_AT(phi, i + 1, j), dn = GB_AT(phi, i, j - 1), up = GB_AT(phi, i, j + 1);
      double av, bv, a1, a2, update;
      if (c > 0) {
        av = l > r ? r : l;
        bv = dn > up ? up : dn;
        if (av <= bv) a1 = av, a2 = bv;
        else a1 = bv, a2 = av;
        update = fabs(a1 - a2) >= h ? a1 + h : one_over_two * (a1 + a2 + sqrt(hh2 - (a1 - a2) * (a1 - a2)));
        *pc = update > c ? c : update;
      } else if (c <= 0) {
        av = l > r ? l : r;
        bv = dn > up ? dn : up;
        if (av <= bv) a1 = av, a2 = bv;
        else a1 = bv, a2 = av;
        update = fabs(a1 - a2) >= h ? a2 - h : one_over_two * (a2 + a1 - sqrt(hh2 - (a2 - a1) * (a2 - a1)));
        *pc = update > c ? update : c;
      }
    }
    __syncthreads();
  }
}

inline dim3 grid2d(int W, int H, dim3 blk) { return dim3((W + blk.x - 1) / blk.x, (H + blk.y - 1) / blk.y); }

LSArgs ls_args(const gb2d_ctx* c) {
  return LSArgs{c->grid.ni, c->grid.nj, c->base.odx, c->base.ody, c->prm.weno_epsilon,
                (float)c->base.odx, (float)c->base.ody, (float)c->prm.weno_epsilon};
}

AsmArgs asm_args(const gb2d_ctx* c, double dt) {
  AsmArgs a;
  a.ni = c->grid.ni;
  a.nj = c->grid.nj;
  a.s = c->base;
  a.water = c->prm.water_density;
  a.air = c->prm.air_density;
  a.sigma = c->prm.surface_tension;
  a.one_over_dt = 1.0 / dt;
  a.dtp = c->dt_dev;
  a.inv_dxdx = 1.0 / (c->base.dx * c->base.dx);
  a.inv_dydy = 1.0 / (c->base.dy * c->base.dy);
  a.inv_water = 1.0 / a.water;
  a.inv_air = 1.0 / a.air;
  a.oeh = 1.0 / (1.5 * c->base.dx);
  a.oev = 1.0 / (1.5 * c->base.dy);
  return a;
}

// Self-check of div_by<3> / div_by<6> against the IEEE division: n pseudo-random
// 64-bit patterns (every exponent, sign, NaN and infinity included) and n more
// with exponents in the range the schemes meet; counts results whose bits differ
// (NaN == NaN).
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}
__global__ void k_check_div_by(unsigned long long n, unsigned long long seed, unsigned long long* bad) {
  unsigned long long local = 0;
  for (unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; t < 2 * n; t += (unsigned long long)gridDim.x * blockDim.x) {
    unsigned long long b = mix64(t * 0x9e3779b97f4a7c15ull + seed);
    if (t >= n) b = (b & 0x800fffffffffffffull) | ((unsigned long long)(1023 - 40 + (int)((b >> 52) % 80)) << 52);  // |a| in [2^-40, 2^40)
    const double a = __longlong_as_double((long long)b);
    const double q3 = div_by<3>(a), r3 = a / 3.0, q6 = div_by<6>(a), r6 = a / 6.0;
    const bool ok3 = __double_as_longlong(q3) == __double_as_longlong(r3) || (isnan(q3) && isnan(r3));
    const bool ok6 = __double_as_longlong(q6) == __double_as_longlong(r6) || (isnan(q6) && isnan(r6));
    local += (ok3 ? 0 : 1) + (ok6 ? 0 : 1);
  }
  if (local) atomicAdd(bad, local);
}

}  // namespace

unsigned long long check_div_by(unsigned long long n, unsigned long long seed, int* cuda_error) {
  unsigned long long* d = nullptr;
  unsigned long long h = ~0ull;
  cudaError_t e = cudaMalloc(&d, sizeof h);
  if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof h);
  if (e == cudaSuccess) {
    k_check_div_by<<<152 * 8, 256>>>(n, seed, d);
    GB_LAUNCHED(1);
    e = cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost);
  }
  if (d) cudaFree(d);
  *cuda_error = e == cudaSuccess ? 0 : 1;
  return h;
}

void launch_fill_ghost_copy(cudaStream_t s, double* dst, int gd, const double* src, int gs, int nI, int nJ, int g) {
  k_fill_ghost_copy<<<grid_ij(nI + 2 * g, nJ + 2 * g), kThreads, 0, s>>>(dst, gd, src, gs, nI, nJ, g);
  GB_LAUNCHED(1);
}

void launch_extrapolate_ghosts(cudaStream_t s, double* f, int g, int nI, int nJ) {
  int n = nI > nJ ? nI : nJ;
  k_extrapolate<<<blocks_for(n, 128), 128, 0, s>>>(f, g, nI, nJ);
  GB_LAUNCHED(1);
}

void launch_weno5_advect(cudaStream_t s, const gb2d_ctx* c, const double* src, double* dst, double dt, int mixed) {
  dim3 blk(32, 8);
  dim3 grd = grid2d(c->grid.ni + 4, c->grid.nj + 4, blk);
  if (mixed)
    k_weno5_advect<true><<<grd, blk, 0, s>>>(src, dst, c->ua, c->va, ls_args(c), DtArg{dt, c->dt_dev});
  else
    k_weno5_advect<false><<<grd, blk, 0, s>>>(src, dst, c->ua, c->va, ls_args(c), DtArg{dt, c->dt_dev});
  GB_LAUNCHED(1);
}

void launch_reinit_sign(cudaStream_t s, const gb2d_ctx* c, const double* phi, double* S) {
  k_reinit_sign<<<grid_ij(c->grid.ni, c->grid.nj), kThreads, 0, s>>>(phi, S, c->grid.ni, c->grid.nj, c->base.dx);
  GB_LAUNCHED(1);
}

void launch_reinit_sweep(cudaStream_t s, const gb2d_ctx* c, const double* src, double* dst, const double* S, double dtau, int mixed) {
  dim3 blk(32, 8);
  dim3 grd = grid2d(c->grid.ni + 4, c->grid.nj + 4, blk);
  // GB2D_REINIT_UNTILED=1 (read once) selects the per-node mixed kernel, which the tiled one
  // must equal bit for bit.
  static const bool untiled = [] {
    const char* e = getenv("GB2D_REINIT_UNTILED");
    return e && e[0] == '1';
  }();
  if (mixed && !untiled)
    k_reinit_sweep_tiled<<<grd, blk, 0, s>>>(src, dst, S, ls_args(c), dtau);
  else if (mixed)
    k_reinit_sweep<true><<<grd, blk, 0, s>>>(src, dst, S, ls_args(c), dtau);
  else
    k_reinit_sweep<false><<<grd, blk, 0, s>>>(src, dst, S, ls_args(c), dtau);
  GB_LAUNCHED(1);
}

void launch_blend(cudaStream_t s, const gb2d_ctx* c, const double* keep, double* phi, double c0, double c1) {
  k_blend<<<grid_ij(c->grid.ni, c->grid.nj), kThreads, 0, s>>>(keep, phi, c->grid.ni, c->grid.nj, c0, c1);
  GB_LAUNCHED(1);
}

void launch_eno3(cudaStream_t s, const gb2d_ctx* c, double dt) {
  EnoArgs a;
  a.ni = c->grid.ni;
  a.nj = c->grid.nj;
  a.xs = c->xs;
  a.ys = c->ys;
  const Space* sp[2] = {&c->xs, &c->ys};
  float* out[2] = {a.xs_f, a.ys_f};
  for (int g = 0; g < 2; ++g) {
    const Space& q = *sp[g];
    const double v[8] = {q.odx, q.o2dx, q.odx / 3, q.dx, q.ody, q.o2dy, q.ody / 3, q.dy};
    for (int k = 0; k < 8; ++k) out[g][k] = (float)v[k];
    a.o3[g][0] = q.odx / 3;
    a.o3[g][1] = q.ody / 3;
  }
  if (c->prm.advection_precision == GB2D_PRECISION_MIXED)
    k_eno3<true><<<grid_ij(c->grid.ni + 1, c->grid.nj + 1), kThreads, 0, s>>>(c->u, c->v, c->ua, c->va, a, DtArg{dt, c->dt_dev});
  else
    k_eno3<false><<<grid_ij(c->grid.ni + 1, c->grid.nj + 1), kThreads, 0, s>>>(c->u, c->v, c->ua, c->va, a, DtArg{dt, c->dt_dev});
  GB_LAUNCHED(1);
}

void launch_curvature(cudaStream_t s, const gb2d_ctx* c, const double* phi, double* kappa, int* flag) {
  k_curvature<<<grid_ij(c->grid.ni, c->grid.nj), kThreads, 0, s>>>(phi, kappa, c->grid.ni, c->grid.nj, c->base, flag);
  GB_LAUNCHED(1);
}

void launch_faces(cudaStream_t s, const gb2d_ctx* c, const double* phi, double dt) {
  AsmArgs a = asm_args(c, dt);
  k_faces<<<grid_ij(c->grid.ni + 1, c->grid.nj + 1), kThreads, 0, s>>>(phi, c->bx, c->by, a);
  GB_LAUNCHED(1);
}

// Needs the face weights.
void launch_diag(cudaStream_t s, const gb2d_ctx* c, double dt) {
  AsmArgs a = asm_args(c, dt);
  k_diag<<<grid_ij(c->grid.ni, c->grid.nj), kThreads, 0, s>>>(c->bx, c->by, c->diag, a);
  GB_LAUNCHED(1);
}

// Needs the face weights and the curvature.
void launch_rhs(cudaStream_t s, const gb2d_ctx* c, const double* phi, double dt) {
  AsmArgs a = asm_args(c, dt);
  k_rhs<<<grid_ij(c->grid.ni, c->grid.nj), kThreads, 0, s>>>(phi, c->kappa, c->u, c->v, c->bx, c->by, c->rhs, a);
  GB_LAUNCHED(1);
}

void launch_poisson_apply_exact(cudaStream_t s, const gb2d_ctx* c, const double* x, double* y) {
  double idx2 = 1.0 / (c->base.dx * c->base.dx), idy2 = 1.0 / (c->base.dy * c->base.dy);
  k_apply_exact<<<grid_ij(c->grid.ni, c->grid.nj), kThreads, 0, s>>>(c->bx, c->by, c->diag, x, y, c->grid.ni, c->grid.nj, idx2, idy2);
  GB_LAUNCHED(1);
}

void launch_velocity_update(cudaStream_t s, const gb2d_ctx* c, const double* phi, double dt, Scalars* sc) {
  AsmArgs a = asm_args(c, dt);
  k_velocity_update<<<grid_ij(c->grid.ni, c->grid.nj), kThreads, 0, s>>>(phi, c->p, c->kappa, c->u, c->v, a, DtArg{dt, c->dt_dev}, sc);
  GB_LAUNCHED(1);
}

void launch_fast_sweeping(cudaStream_t s, gb2d_ctx* c, int sweeps) {
  const int ni = c->grid.ni, nj = c->grid.nj, n = ni > nj ? ni : nj;
  double* phi = c->phi_buf[c->phi_cur];
  k_fsm_fixed<<<grid_ij(ni, nj), kThreads, 0, s>>>(phi, c->tmp_a, ni, nj, 2.0 * c->base.dx);
  k_extrapolate_inner_first<<<(n + 127) / 128, 128, 0, s>>>(phi, 2, ni, nj);
  for (int k = 0; k < sweeps; ++k) k_fsm_sweep<<<1, 1024, 0, s>>>(phi, c->tmp_a, ni, nj, c->base.dx, k % 4);
  k_extrapolate_inner_first<<<(n + 127) / 128, 128, 0, s>>>(phi, 2, ni, nj);
  GB_LAUNCHED(3 + sweeps);
}

void launch_copy_interior(cudaStream_t s, const double* src, int gs, double* dst, int gd, int nI, int nJ) {
  k_copy_interior<<<grid_ij(nI, nJ), kThreads, 0, s>>>(src, gs, dst, gd, nI, nJ);
  GB_LAUNCHED(1);
}

}  // namespace gb2d
