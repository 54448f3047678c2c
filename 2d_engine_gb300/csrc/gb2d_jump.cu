// The general jump-condition Poisson problem of POISSON_SOLVER::Solve(pressure, density,
// bc, div, levelset, jc_on_solution, jc_on_derivative) (POISSON_SOLVER.cpp:127-145) with
// BuildLinearSystemNodeJumpConditionVaribleCoefficient (:714-976) and the level-set
// normals it reads (LEVELSET_2D::ComputeNormals, LEVELSET_2D.h:640-662), as
// POISSON_EQUATION_TEST drives it: Dirichlet / Neumann boundary codes, solution jumps and
// flux jumps.  The system is built in the grid layout the solver uses (full cells as the
// builder writes them; every other node an identity row holding its given value) and
// solved by the same MG-preconditioned CG as the projection.
// Built with --fmad=false in the reference's association order: bit-exact entries.
#include "gb2d_internal.cuh"
#include "gb2d_schemes.cuh"

namespace gb2d {

namespace {

constexpr int kBcDir = -1, kBcNeum = -4;  // MACROS.h:6-12

// Unit normals of the interior nodes; phi's ghosts already copy-filled.
__global__ void k_normals(const double* __restrict__ phi_a, double* __restrict__ nx_a, double* __restrict__ ny_a, int ni, int nj,
                          Space s) {
  const DField phi = dfield((double*)phi_a, 2, ni, nj), nx = dfield(nx_a, 1, ni, nj), ny = dfield(ny_a, 1, ni, nj);
  GB_FOR_IJ(i, j, ni, nj) {
    double x = (GB_AT(phi, i + 1, j) - GB_AT(phi, i - 1, j)) * s.o2dx, y = (GB_AT(phi, i, j + 1) - GB_AT(phi, i, j - 1)) * s.o2dy;
    const double m = sqrt(x * x + y * y);
    if (!(m != 0)) {
      x = (GB_AT(phi, i + 1, j) - GB_AT(phi, i, j)) * s.odx;
      y = (GB_AT(phi, i, j + 1) - GB_AT(phi, i, j)) * s.ody;
    }
    const double mag = sqrt(x * x + y * y), om = 1 / mag;  // VECTOR_2D::MakeThisUnit
    if (mag != 0) {
      x *= om;
      y *= om;
    }
    GB_AT(nx, i, j) = x;
    GB_AT(ny, i, j) = y;
  }
}

struct JumpArgs {
  int ni, nj;
  Space s;
  double inv_dxdx, inv_dydy;
};

struct JumpIn {
  const double *p, *dens, *div, *phi, *nx, *ny, *js, *jd;
  const int* bc;
};

__device__ __forceinline__ double var_at(const JumpIn& in, int i, int j, int ni, int nj) {
  // 1/density on the interior, ghosts copied from the second interior line (POISSON_SOLVER.cpp:131-138)
  const int ii = i < 0 ? 1 : (i >= ni ? ni - 2 : i), jj = j < 0 ? 1 : (j >= nj ? nj - 2 : j);
  return 1 / in.dens[(ii + 1) + (size_t)(jj + 1) * (ni + 2)];
}

// beta of the face between node c and neighbour n in the builder's form for that arm:
// left / bottom arms put the centre's variable first in the denominator, right / top
// arms the neighbour's (the value is the same from either side).
__device__ __forceinline__ double arm_beta(double vc, double vn, double lc, double ln, bool low) {
  return low ? vc * vn * (fabs(ln) + fabs(lc)) / (vc * fabs(ln) + vn * fabs(lc))
             : vc * vn * (fabs(ln) + fabs(lc)) / (vn * fabs(lc) + vc * fabs(ln));
}

// One pass over (ni+1) x (nj+1): face weights bx(i, j) / by(i, j) (zero unless both nodes
// are full cells), and for nodes the diagonal and right-hand side.
__global__ void k_jump_assemble(JumpIn in, double* __restrict__ bx, double* __restrict__ by, double* __restrict__ diag,
                                double* __restrict__ rhs, double* __restrict__ shift, JumpArgs a) {
  const int ni = a.ni, nj = a.nj;
  const DField phi = dfield((double*)in.phi, 2, ni, nj), P = dfield((double*)in.p, 1, ni, nj), D = dfield((double*)in.div, 1, ni, nj);
  const DField NX = dfield((double*)in.nx, 1, ni, nj), NY = dfield((double*)in.ny, 1, ni, nj);
  const DField JS = dfield((double*)in.js, 1, ni, nj), JD = dfield((double*)in.jd, 1, ni, nj);
  auto BC = [&](int i, int j) { return in.bc[(i + 1) + (size_t)(j + 1) * (ni + 2)]; };
  GB_FOR_IJ(i, j, ni + 1, nj + 1) {
    if (j < nj) {  // x-face between (i-1, j) and (i, j)
      double w = 0;
      if (i >= 1 && i < ni && BC(i, j) > -1 && BC(i - 1, j) > -1)
        w = arm_beta(var_at(in, i, j, ni, nj), var_at(in, i - 1, j, ni, nj), GB_AT(phi, i, j), GB_AT(phi, i - 1, j), true);
      bx[i + (size_t)j * (ni + 1)] = w;
    }
    if (i < ni) {  // y-face between (i, j-1) and (i, j)
      double w = 0;
      if (j >= 1 && j < nj && BC(i, j) > -1 && BC(i, j - 1) > -1)
        w = arm_beta(var_at(in, i, j, ni, nj), var_at(in, i, j - 1, ni, nj), GB_AT(phi, i, j), GB_AT(phi, i, j - 1), true);
      by[i + (size_t)j * ni] = w;
    }
    if (i >= ni || j >= nj) continue;
    const size_t t = (size_t)j * ni + i;
    if (BC(i, j) < 0) {
      diag[t] = a.inv_dxdx;
      rhs[t] = a.inv_dxdx * GB_AT(P, i, j);
      shift[t] = a.inv_dxdx;
      continue;
    }
    const double lc = GB_AT(phi, i, j), ll = GB_AT(phi, i - 1, j), lr = GB_AT(phi, i + 1, j), lb = GB_AT(phi, i, j - 1),
                 lt = GB_AT(phi, i, j + 1);
    const double vc = var_at(in, i, j, ni, nj), vl = var_at(in, i - 1, j, ni, nj), vr = var_at(in, i + 1, j, ni, nj),
                 vb = var_at(in, i, j - 1, ni, nj), vt = var_at(in, i, j + 1, ni, nj);
    const double beta_l = arm_beta(vc, vl, lc, ll, true), beta_r = arm_beta(vc, vr, lc, lr, false);
    const double beta_b = arm_beta(vc, vb, lc, lb, true), beta_t = arm_beta(vc, vt, lc, lt, false);
    const int cl = BC(i - 1, j), cr = BC(i + 1, j), cb = BC(i, j - 1), ct = BC(i, j + 1);
    double coef = 0;
    if (cl > -1) coef += beta_l;
    if (cr > -1) coef += beta_r;
    if (cb > -1) coef += beta_b;
    if (ct > -1) coef += beta_t;
    if (cl == kBcDir) coef += beta_l;
    if (cr == kBcDir) coef += beta_r;
    if (cb == kBcDir) coef += beta_b;
    if (ct == kBcDir) coef += beta_t;
    if (i == 0 && j == 0) {
      if (cl == kBcNeum) coef += beta_l;
      if (cr == kBcNeum) coef += beta_r;
      if (cb == kBcNeum) coef += beta_b;
      if (ct == kBcNeum) coef += beta_t;
    }
    // The diagonal beyond the face conductances (for the multigrid levels): Dirichlet arms,
    // the Neumann pin, and the y-faces' 1/dx^2 - 1/dy^2 excess of the dx-only diagonal.
    double extra = 0, yfull = 0;
    if (cl == kBcDir) extra += beta_l;
    if (cr == kBcDir) extra += beta_r;
    if (cb == kBcDir) extra += beta_b;
    if (ct == kBcDir) extra += beta_t;
    if (i == 0 && j == 0) {
      if (cl == kBcNeum) extra += beta_l;
      if (cr == kBcNeum) extra += beta_r;
      if (cb == kBcNeum) extra += beta_b;
      if (ct == kBcNeum) extra += beta_t;
    }
    if (cb > -1) yfull += beta_b;
    if (ct > -1) yfull += beta_t;
    shift[t] = coef == 0 ? a.inv_dxdx : extra * a.inv_dxdx + yfull * (a.inv_dxdx - a.inv_dydy);
    if (coef == 0) coef = 1;
    diag[t] = a.inv_dxdx * coef;
    const double jc = GB_AT(JS, i, j), jd = GB_AT(JD, i, j);
    // One arm of the boundary-capturing stencil; sgn = -1 for left / bottom, +1 for right / top.
    auto arm = [&](double ln, double jsn, double jdn, double nn, double nc, double beta, double vn, double o, double o2,
                   double sgn) -> double {
      const double sub = fabs(ln) / (fabs(lc) + fabs(ln));
      const double av = (jc * fabs(ln) + jsn * fabs(lc)) / (fabs(lc) + fabs(ln));
      const double bv = (jd * nc * fabs(ln) + jdn * nn * fabs(lc)) / (fabs(lc) + fabs(ln));
      if ((lc <= 0 && ln <= 0) || (lc > 0 && ln > 0)) return 0;
      if (lc <= 0 && ln > 0) return o2 * av * beta + sgn * (o * beta * bv * sub / vn);
      if (lc > 0 && ln <= 0) return -o2 * av * beta - sgn * (o * beta * bv * sub / vn);
      return 0;
    };
    const double nxc = GB_AT(NX, i, j), nyc = GB_AT(NY, i, j);
    const double FL = arm(ll, GB_AT(JS, i - 1, j), GB_AT(JD, i - 1, j), GB_AT(NX, i - 1, j), nxc, beta_l, vl, a.s.odx, a.s.odx2, -1.0);
    const double FR = arm(lr, GB_AT(JS, i + 1, j), GB_AT(JD, i + 1, j), GB_AT(NX, i + 1, j), nxc, beta_r, vr, a.s.odx, a.s.odx2, 1.0);
    const double FB = arm(lb, GB_AT(JS, i, j - 1), GB_AT(JD, i, j - 1), GB_AT(NY, i, j - 1), nyc, beta_b, vb, a.s.ody, a.s.ody2, -1.0);
    const double FT = arm(lt, GB_AT(JS, i, j + 1), GB_AT(JD, i, j + 1), GB_AT(NY, i, j + 1), nyc, beta_t, vt, a.s.ody, a.s.ody2, 1.0);
    const double FX = FL + FR, FY = FB + FT;
    double r = -GB_AT(D, i, j) - FX - FY;
    if (cl == kBcDir) r += beta_l * a.inv_dxdx * GB_AT(P, i - 1, j);
    if (cr == kBcDir) r += beta_r * a.inv_dxdx * GB_AT(P, i + 1, j);
    if (cb == kBcDir) r += beta_b * a.inv_dydy * GB_AT(P, i, j - 1);
    if (ct == kBcDir) r += beta_t * a.inv_dydy * GB_AT(P, i, j + 1);
    rhs[t] = r;
  }
}

}  // namespace

int jump_buffers(gb2d_ctx* c) {
  if (c->jmp_dens) return GB2D_OK;
  const size_t ni = c->grid.ni, nj = c->grid.nj, np = (ni + 2) * (nj + 2);
  double** bufs[] = {&c->jmp_dens, &c->jmp_div, &c->jmp_js, &c->jmp_jd, &c->jmp_nx, &c->jmp_ny};
  for (double** b : bufs) {
    cudaError_t e = cudaMalloc(b, np * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(*b, 0, np * sizeof(double));
    if (e != cudaSuccess) return GB2D_ERR_CUDA;
  }
  cudaError_t e = cudaMalloc(&c->jmp_phi, (ni + 4) * (nj + 4) * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&c->jmp_bc, np * sizeof(int));
  return e == cudaSuccess ? GB2D_OK : GB2D_ERR_CUDA;
}

void launch_jump_assemble(cudaStream_t s, gb2d_ctx* c) {
  const int ni = c->grid.ni, nj = c->grid.nj;
  launch_fill_ghost_copy(s, c->jmp_phi, 2, c->jmp_phi, 2, ni, nj, 2);  // ComputeNormals refreshes phi's ghosts first
  k_normals<<<grid_ij(ni, nj), kThreads, 0, s>>>(c->jmp_phi, c->jmp_nx, c->jmp_ny, ni, nj, c->base);
  JumpIn in{c->xw, c->jmp_dens, c->jmp_div, c->jmp_phi, c->jmp_nx, c->jmp_ny, c->jmp_js, c->jmp_jd, c->jmp_bc};
  JumpArgs a{ni, nj, c->base, 1 / (c->base.dx * c->base.dx), 1 / (c->base.dy * c->base.dy)};
  k_jump_assemble<<<grid_ij(ni + 1, nj + 1), kThreads, 0, s>>>(in, c->bx, c->by, c->diag, c->rhs, c->tmp_b, a);
  GB_LAUNCHED(2);
}

}  // namespace gb2d
