// Pressure solver: multigrid-preconditioned CG on the matrix-free 5-point
// ghost-fluid operator, in FP64 or as FP64 iterative refinement around an FP32
// CG + FP32 V-cycle inner solve.
//
// Replaces PCG_METHOD::PCGMethod with IC(0) (PCG_METHOD.cpp:176-264) and the
// reference's constant-coefficient MULTIGRID_METHOD (MULTIGRID_METHOD.cpp:107-332)
// by a new design: cell-centred geometric multigrid on the variable-coefficient
// operator (face conductances averaged along the coarse face, Neumann walls,
// the reference's pin/shift terms carried by a diagonal shift), red-black
// Gauss-Seidel smoothing (red-black before, black-red after: a symmetric
// preconditioner), piecewise-constant prolongation with averaging restriction,
// and a dense inverse on the coarsest level (<= 64 cells).
//
// The FP32 inner CG applies the operator in flux form,
//   (A p)_i = sh_i p_i + sum_faces c_f (p_i - p_nb),
// whose differences of neighbouring values are exact, so FP32 rounding is
// relative to the flux rather than to the diagonal; the solution accumulates in
// FP64 and every dot product accumulates in FP64.  Each FP64 refinement step
// recomputes r = b - A x with the reference's own matrix entries.
//
// All reductions are two-stage and deterministic: blocks write partial sums,
// consumers re-reduce the partials in a fixed order.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "gb2d_internal.cuh"

namespace gb2d {

namespace {

constexpr int kSlots = 4;  // partial-sum slots: 0 = p.Ap, 1 = r.r, 2 = r.z, 3 = b.b

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Deterministic block sum (blockDim.x multiple of 32, <= 1024); result valid in every thread.
__device__ double block_sum(double v) {
  __shared__ double sm[32];
  __shared__ double total;
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sm[w] = v;
  __syncthreads();
  if (w == 0) {
    double x = lane < nw ? sm[lane] : 0.0;
    x = warp_sum(x);
    if (lane == 0) total = x;
  }
  __syncthreads();
  return total;
}

__device__ double sum_partials(const double* part, int n) {
  double v = 0.0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) v += part[k];
  return block_sum(v);
}

template <typename T>
__device__ __forceinline__ size_t cell_index(const Level<T>& L, size_t t, int& i, int& j) {
  i = (int)(t % L.nI);
  j = (int)(t / L.nI);
  return (size_t)(i + 1) + (size_t)(j + 1) * L.ld;
}

// ---- level construction -----------------------------------------------------

// Level 0 from the assembled FP64 system: conductances beta/dx^2 on interior
// faces, zero on walls; diagonal as assembled; shift = pin + (dx != dy) terms.
template <typename T>
__global__ void k_build_level0(const double* __restrict__ bx, const double* __restrict__ by, const double* __restrict__ diag,
                               const double* __restrict__ rhs, Level<T> L, double* __restrict__ b64, double idx2, double idy2) {
  int ni = L.nI, nj = L.nJ;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)ni * nj; t += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    size_t k = cell_index(L, t, i, j);
    double bl = bx[i + (size_t)j * (ni + 1)];
    double bb = by[i + (size_t)j * ni], bt = by[i + (size_t)(j + 1) * ni];
    double cl = i > 0 ? bl * idx2 : 0.0, cb = j > 0 ? bb * idy2 : 0.0;
    L.cx[k] = (T)cl;
    L.cy[k] = (T)cb;
    if (i == ni - 1) L.cx[k + 1] = (T)0;
    if (j == nj - 1) L.cy[k + L.ld] = (T)0;
    double d = diag[t];
    L.dg[k] = (T)d;
    L.idg[k] = (T)(1.0 / d);
    double ybeta = (j > 0 ? bb : 0.0) + (j < nj - 1 ? bt : 0.0);
    double pin = (i == 0 && j == 0) ? (bl + bb) : 0.0;
    L.sh[k] = (T)(pin * idx2 + ybeta * (idx2 - idy2));
    if (b64) b64[k] = rhs[t];
  }
}

// Coarse level: cell (I, J) covers fine cells (2I..2I+1, 2J..2J+1) that exist.
// Face conductances: sum of the two fine faces / 8 (face-averaged weight over
// the doubled spacing); shift: average of the children's shifts.
template <typename T>
__global__ void k_coarsen(Level<T> F, Level<T> C) {
  int cI = C.nI, cJ = C.nJ;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)cI * cJ; t += (size_t)gridDim.x * blockDim.x) {
    int I, J;
    size_t k = cell_index(C, t, I, J);
    auto fx = [&](int fi, int fj) -> double {  // fine x-face fi at fine row fj (0 outside)
      if (fj >= F.nJ) return 0.0;
      return (double)F.cx[(size_t)(fi + 1) + (size_t)(fj + 1) * F.ld];
    };
    auto fy = [&](int fi, int fj) -> double {
      if (fi >= F.nI) return 0.0;
      return (double)F.cy[(size_t)(fi + 1) + (size_t)(fj + 1) * F.ld];
    };
    double cl = I > 0 ? (fx(2 * I, 2 * J) + fx(2 * I, 2 * J + 1)) / 8.0 : 0.0;
    double cr = I < cI - 1 ? (fx(2 * I + 2, 2 * J) + fx(2 * I + 2, 2 * J + 1)) / 8.0 : 0.0;
    double cb = J > 0 ? (fy(2 * I, 2 * J) + fy(2 * I + 1, 2 * J)) / 8.0 : 0.0;
    double ct = J < cJ - 1 ? (fy(2 * I, 2 * J + 2) + fy(2 * I + 1, 2 * J + 2)) / 8.0 : 0.0;
    double s = 0.0;
    for (int b = 0; b < 2; ++b)
      for (int a = 0; a < 2; ++a) {
        int fi = 2 * I + a, fj = 2 * J + b;
        if (fi < F.nI && fj < F.nJ) s += (double)F.sh[(size_t)(fi + 1) + (size_t)(fj + 1) * F.ld];
      }
    s *= 0.25;
    C.cx[k] = (T)cl;
    C.cy[k] = (T)cb;
    if (I == cI - 1) C.cx[k + 1] = (T)0;
    if (J == cJ - 1) C.cy[k + C.ld] = (T)0;
    double d = cl + cr + cb + ct + s;
    C.dg[k] = (T)d;
    C.idg[k] = (T)(1.0 / d);
    C.sh[k] = (T)s;
  }
}

// Dense inverse of the coarsest operator (n <= 64), in-place Gauss-Jordan
// without pivoting (the operator is SPD).  One block, one thread per row.
template <typename T>
__global__ void k_dense_inverse(Level<T> C, double* __restrict__ ainv) {
  __shared__ double A[kCoarseMax][kCoarseMax + 1];
  int n = C.nI * C.nJ;
  int r = threadIdx.x;
  if (r < n) {
    for (int m = 0; m < n; ++m) A[r][m] = 0.0;
    int i = r % C.nI, j = r / C.nI;
    size_t k = (size_t)(i + 1) + (size_t)(j + 1) * C.ld;
    A[r][r] = (double)C.dg[k];
    if (i > 0) A[r][r - 1] = -(double)C.cx[k];
    if (i < C.nI - 1) A[r][r + 1] = -(double)C.cx[k + 1];
    if (j > 0) A[r][r - C.nI] = -(double)C.cy[k];
    if (j < C.nJ - 1) A[r][r + C.nI] = -(double)C.cy[k + C.ld];
  }
  __syncthreads();
  for (int kk = 0; kk < n; ++kk) {
    double piv = A[kk][kk];
    __syncthreads();
    if (r == kk) {
      for (int m = 0; m < n; ++m) A[kk][m] /= piv;
      A[kk][kk] = 1.0 / piv;
    }
    __syncthreads();
    if (r < n && r != kk) {
      double f = A[r][kk];
      for (int m = 0; m < n; ++m) A[r][m] -= f * A[kk][m];
      A[r][kk] = -f / piv;
    }
    __syncthreads();
  }
  if (r < n)
    for (int m = 0; m < n; ++m) ainv[(size_t)r * n + m] = A[r][m];
}

// ---- V-cycle kernels -----------------------------------------------------------

// One red-black Gauss-Seidel half sweep.  zero_init: x was implicitly zero, so the
// sweep writes b/dg on this colour and 0 on the other.
template <typename T>
__global__ void k_smooth(Level<T> L, int color, int zero_init, const int* __restrict__ done) {
  if (*done) return;
  int hw = (L.nI + 1) / 2;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)hw * L.nJ; t += (size_t)gridDim.x * blockDim.x) {
    int j = (int)(t / hw);
    int i = 2 * (int)(t % hw) + ((j + color) & 1);
    size_t k = (size_t)(i + 1) + (size_t)(j + 1) * L.ld;
    if (zero_init) {
      if (i < L.nI) L.x[k] = L.b[k] * L.idg[k];
      int io = i + (((j + color) & 1) ? -1 : 1);  // the other colour's cell in this pair
      if (io >= 0 && io < L.nI) L.x[(size_t)(io + 1) + (size_t)(j + 1) * L.ld] = (T)0;
      continue;
    }
    if (i >= L.nI) continue;
    T s = L.b[k] + L.cx[k] * L.x[k - 1] + L.cx[k + 1] * L.x[k + 1] + L.cy[k] * L.x[k - L.ld] + L.cy[k + L.ld] * L.x[k + L.ld];
    L.x[k] = s * L.idg[k];
  }
}

// Coarse right-hand side = average of the four children's residuals b - A x.
template <typename T>
__global__ void k_residual_restrict(Level<T> F, Level<T> C, const int* __restrict__ done) {
  if (*done) return;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)C.nI * C.nJ; t += (size_t)gridDim.x * blockDim.x) {
    int I, J;
    size_t kc = cell_index(C, t, I, J);
    T acc = 0;
    for (int b = 0; b < 2; ++b)
      for (int a = 0; a < 2; ++a) {
        int i = 2 * I + a, j = 2 * J + b;
        if (i >= F.nI || j >= F.nJ) continue;
        size_t k = (size_t)(i + 1) + (size_t)(j + 1) * F.ld;
        T ax = F.dg[k] * F.x[k] - F.cx[k] * F.x[k - 1] - F.cx[k + 1] * F.x[k + 1] - F.cy[k] * F.x[k - F.ld] - F.cy[k + F.ld] * F.x[k + F.ld];
        acc += F.b[k] - ax;
      }
    C.b[kc] = (T)0.25 * acc;
  }
}

// Piecewise-constant prolongation of the coarse correction.
template <typename T>
__global__ void k_prolong(Level<T> F, Level<T> C, const int* __restrict__ done) {
  if (*done) return;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)F.nI * F.nJ; t += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    size_t k = cell_index(F, t, i, j);
    F.x[k] += C.x[(size_t)(i / 2 + 1) + (size_t)(j / 2 + 1) * C.ld];
  }
}

template <typename T>
__global__ void k_coarse_solve(Level<T> C, const double* __restrict__ ainv, const int* __restrict__ done) {
  if (*done) return;
  int n = C.nI * C.nJ;
  int r = threadIdx.x;
  if (r >= n) return;
  double acc = 0.0;
  for (int m = 0; m < n; ++m) {
    int i = m % C.nI, j = m / C.nI;
    acc += ainv[(size_t)r * n + m] * (double)C.b[(size_t)(i + 1) + (size_t)(j + 1) * C.ld];
  }
  int i = r % C.nI, j = r / C.nI;
  C.x[(size_t)(i + 1) + (size_t)(j + 1) * C.ld] = (T)acc;
}

// ---- CG kernels ----------------------------------------------------------------

// FP64 residual of the refinement loop with the reference's matrix entries:
// r64 = b - A x; optional FP32 copy; partial ||r||^2 and ||b||^2.
template <typename T>
__global__ void k_residual64(Level<double> L, const double* __restrict__ x, const double* __restrict__ b, double* __restrict__ r64,
                             T* __restrict__ rT, double* __restrict__ part_rr, double* __restrict__ part_bb) {
  double rr = 0.0, bb = 0.0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)L.nI * L.nJ; t += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    size_t k = cell_index(L, t, i, j);
    double ax = L.dg[k] * x[k] - L.cx[k] * x[k - 1] - L.cx[k + 1] * x[k + 1] - L.cy[k] * x[k - L.ld] - L.cy[k + L.ld] * x[k + L.ld];
    double r = b[k] - ax;
    if (r64) r64[k] = r;
    if (rT) rT[k] = (T)r;
    rr += r * r;
    bb += b[k] * b[k];
  }
  rr = block_sum(rr);
  bb = block_sum(bb);
  if (threadIdx.x == 0) {
    part_rr[blockIdx.x] = rr;
    part_bb[blockIdx.x] = bb;
  }
}

// Ap = A p in flux form; partial p.Ap.
template <typename T>
__global__ void k_apply_dot(Level<T> L, const T* __restrict__ p, T* __restrict__ ap, double* __restrict__ part, const int* __restrict__ done) {
  if (*done) return;
  double acc = 0.0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)L.nI * L.nJ; t += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    size_t k = cell_index(L, t, i, j);
    T pc = p[k];
    T y = L.sh[k] * pc + L.cx[k] * (pc - p[k - 1]) + L.cx[k + 1] * (pc - p[k + 1]) + L.cy[k] * (pc - p[k - L.ld]) +
          L.cy[k + L.ld] * (pc - p[k + L.ld]);
    ap[k] = y;
    acc += (double)pc * (double)y;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// alpha = r.z / p.Ap;  x (FP64) += scale*alpha p;  r -= alpha Ap;  partial r.r.
template <typename T>
__global__ void k_cg_update(Level<T> L, double* __restrict__ x, T* __restrict__ r, const T* __restrict__ p, const T* __restrict__ ap,
                            const double* __restrict__ part_pap, int nparts, Scalars* sc, int par, double scale, double* __restrict__ part_rr,
                            const int* __restrict__ done) {
  if (*done) return;
  double pap = sum_partials(part_pap, nparts);
  double alpha = sc->rz[par] / pap;
  double acc = 0.0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)L.nI * L.nJ; t += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    size_t k = cell_index(L, t, i, j);
    x[k] += (scale * alpha) * (double)p[k];
    T rn = r[k] - (T)alpha * ap[k];
    r[k] = rn;
    acc += (double)rn * (double)rn;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) part_rr[blockIdx.x] = acc;
}

template <typename T>
__global__ void k_dot(Level<T> L, const T* __restrict__ a, const T* __restrict__ b, double* __restrict__ part, const int* __restrict__ done) {
  if (*done) return;
  double acc = 0.0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)L.nI * L.nJ; t += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    size_t k = cell_index(L, t, i, j);
    acc += (double)a[k] * (double)b[k];
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// beta = rz_new / rz_old;  p = z + beta p  (first: p = z).  Block 0 records rz_new in rz[par].
template <typename T>
__global__ void k_p_update(Level<T> L, T* __restrict__ p, const T* __restrict__ z, const double* __restrict__ part_rz, int nparts, Scalars* sc,
                           int par, int first, const int* __restrict__ done) {
  if (*done) return;
  double rz = sum_partials(part_rz, nparts);
  double beta = first ? 0.0 : rz / sc->rz[par ^ 1];
  if (blockIdx.x == 0 && threadIdx.x == 0) sc->rz[par] = rz;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)L.nI * L.nJ; t += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    size_t k = cell_index(L, t, i, j);
    p[k] = first ? z[k] : z[k] + (T)beta * p[k];
  }
}

// Jacobi preconditioner z = r / dg.
template <typename T>
__global__ void k_jacobi(Level<T> L, const T* __restrict__ r, T* __restrict__ z, const int* __restrict__ done) {
  if (*done) return;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)L.nI * L.nJ; t += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    size_t k = cell_index(L, t, i, j);
    z[k] = r[k] * L.idg[k];
  }
}

// Sum one partial slot into sc->rr, set *done when rr <= thr2 (or non-finite).
__global__ void k_finalize(const double* __restrict__ part, int nparts, Scalars* sc, double thr2, int* done, double* host_rr) {
  double rr = sum_partials(part, nparts);
  if (threadIdx.x == 0) {
    sc->rr = rr;
    if (!(rr <= thr2)) {
      if (!isfinite(rr)) {
        sc->flag |= 1;
        *done = 1;
      }
    } else {
      *done = 1;
    }
    *host_rr = rr;
  }
}

__global__ void k_reduce_two(const double* __restrict__ pa, const double* __restrict__ pb, int nparts, double* out) {
  double a = sum_partials(pa, nparts);
  double b = sum_partials(pb, nparts);
  if (threadIdx.x == 0) {
    out[0] = a;
    out[1] = b;
  }
}

__global__ void k_set_int(int* p, int v) { *p = v; }

template <typename T>
__global__ void k_zero_level(Level<T> L) {
  size_t n = (size_t)(L.nI + 2) * (L.nJ + 2);
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    L.x[t] = 0;
    L.b[t] = 0;
    L.cx[t] = 0;
    L.cy[t] = 0;
  }
}

}  // namespace

// ---- host side -------------------------------------------------------------------

template <typename T>
struct Hierarchy {
  int nlev = 0;
  Level<T> L[kMaxLevels];
  T *p = nullptr, *ap = nullptr, *r = nullptr;  // CG vectors (padded fine layout); z = L[0].x
};

struct Solver {
  int ni, nj;
  Hierarchy<double> h64;
  Hierarchy<float> h32;
  double* ainv64 = nullptr;
  double* ainv32 = nullptr;
  double* b64 = nullptr;   // right-hand side, padded
  double* r64 = nullptr;   // FP64 residual, padded
  double* part = nullptr;  // kSlots x kMaxPartials
  double* host = nullptr;  // pinned: [0] rr, [1] rr (reduce_two), [2] bb
  int* done = nullptr;
  Scalars* sc = nullptr;
  int nparts;
  cudaEvent_t ev[2] = {nullptr, nullptr};
};

namespace {

template <typename T>
cudaError_t alloc_level(Level<T>& L, int nI, int nJ, bool own_b) {
  L.nI = nI;
  L.nJ = nJ;
  L.ld = nI + 2;
  size_t n = (size_t)(nI + 2) * (nJ + 2);
  T** arrs[7] = {&L.cx, &L.cy, &L.dg, &L.idg, &L.sh, &L.x, &L.b};
  for (auto a : arrs) {
    if (a == &L.b && !own_b) continue;
    cudaError_t e = cudaMalloc(a, n * sizeof(T));
    if (e != cudaSuccess) return e;
    e = cudaMemset(*a, 0, n * sizeof(T));
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename T>
void free_level(Level<T>& L, bool own_b) {
  T* arrs[7] = {L.cx, L.cy, L.dg, L.idg, L.sh, L.x, own_b ? L.b : nullptr};
  for (auto a : arrs)
    if (a) cudaFree(a);
}

template <typename T>
cudaError_t alloc_hierarchy(Hierarchy<T>& H, int ni, int nj) {
  size_t n = (size_t)(ni + 2) * (nj + 2);
  T** v[3] = {&H.p, &H.ap, &H.r};
  for (auto a : v) {
    cudaError_t e = cudaMalloc(a, n * sizeof(T));
    if (e != cudaSuccess) return e;
    e = cudaMemset(*a, 0, n * sizeof(T));
    if (e != cudaSuccess) return e;
  }
  int nI = ni, nJ = nj;
  H.nlev = 0;
  while (true) {
    Level<T>& L = H.L[H.nlev];
    cudaError_t e = alloc_level(L, nI, nJ, H.nlev > 0);
    if (H.nlev == 0) L.b = H.r;  // the fine level's right-hand side is the CG residual
    if (e != cudaSuccess) return e;
    H.nlev++;
    if (nI * nJ <= kCoarseMax) break;
    if (H.nlev == kMaxLevels) return cudaErrorInvalidValue;  // aspect ratio too extreme for the dense coarse solve
    nI = (nI + 1) / 2;
    nJ = (nJ + 1) / 2;
  }
  return cudaSuccess;
}

template <typename T>
void free_hierarchy(Hierarchy<T>& H) {
  for (int l = 0; l < H.nlev; ++l) free_level(H.L[l], l > 0);
  if (H.p) cudaFree(H.p);
  if (H.ap) cudaFree(H.ap);
  if (H.r) cudaFree(H.r);
}

inline unsigned nblocks(size_t n, unsigned cap) {
  size_t b = (n + kThreads - 1) / kThreads;
  if (b < 1) b = 1;
  return (unsigned)(b < cap ? b : cap);
}

template <typename T>
void build_hierarchy(cudaStream_t s, Hierarchy<T>& H, const gb2d_ctx* c, double* b64, double* ainv) {
  double idx2 = 1.0 / (c->base.dx * c->base.dx), idy2 = 1.0 / (c->base.dy * c->base.dy);
  Level<T>& L0 = H.L[0];
  k_build_level0<T><<<nblocks((size_t)L0.nI * L0.nJ, 1216), kThreads, 0, s>>>(c->bx, c->by, c->diag, c->rhs, L0, b64, idx2, idy2);
    GB_LAUNCHED(1);
  for (int l = 1; l < H.nlev; ++l)
    k_coarsen<T><<<nblocks((size_t)H.L[l].nI * H.L[l].nJ, 1216), kThreads, 0, s>>>(H.L[l - 1], H.L[l]);
    GB_LAUNCHED(1);
  k_dense_inverse<T><<<1, kCoarseMax, 0, s>>>(H.L[H.nlev - 1], ainv);
    GB_LAUNCHED(1);
}

// z = M r with the fine level's x/b pointing at z/r.
// Bytes one red-black half sweep must move: b, 1/dg and x of the updated colour
// (x read and written), x of the other colour, every face conductance once.
template <typename T>
double half_sweep_bytes(const Level<T>& L) {
  double n = (double)L.nI * L.nJ, faces = (double)(L.nI + 1) * L.nJ + (double)L.nI * (L.nJ + 1);
  return sizeof(T) * (0.5 * n * 4 + 0.5 * n + faces);
}

template <typename T>
void smooth_launch(cudaStream_t s, Level<T>& L, int color, int zero_init, const int* done, Probe* pr) {
  size_t half = (size_t)((L.nI + 1) / 2) * L.nJ;
  unsigned gb = nblocks(half, 1216);
  bool probe = pr && pr->on && pr->n < pr->cap;
  if (probe) cudaEventRecord(pr->ev[2 * pr->n], s);
  k_smooth<T><<<gb, kThreads, 0, s>>>(L, color, zero_init, done);
    GB_LAUNCHED(1);
  if (probe) {
    cudaEventRecord(pr->ev[2 * pr->n + 1], s);
    pr->bytes = half_sweep_bytes(L);
    pr->n++;
  }
}

template <typename T>
void vcycle(cudaStream_t s, Hierarchy<T>& H, const double* ainv, int nu, const int* done, Probe* pr) {
  int nl = H.nlev;
  for (int l = 0; l < nl - 1; ++l) {
    Level<T>& L = H.L[l];
    Probe* p = l == 0 ? pr : nullptr;
    for (int sweep = 0; sweep < nu; ++sweep) {
      smooth_launch<T>(s, L, 0, sweep == 0, done, p);
      smooth_launch<T>(s, L, 1, 0, done, p);
    }
    k_residual_restrict<T><<<nblocks((size_t)H.L[l + 1].nI * H.L[l + 1].nJ, 1216), kThreads, 0, s>>>(L, H.L[l + 1], done);
    GB_LAUNCHED(1);
  }
  k_coarse_solve<T><<<1, kCoarseMax, 0, s>>>(H.L[nl - 1], ainv, done);
    GB_LAUNCHED(1);
  for (int l = nl - 2; l >= 0; --l) {
    Level<T>& L = H.L[l];
    k_prolong<T><<<nblocks((size_t)L.nI * L.nJ, 1216), kThreads, 0, s>>>(L, H.L[l + 1], done);
    GB_LAUNCHED(1);
    Probe* p = l == 0 ? pr : nullptr;
    for (int sweep = 0; sweep < nu; ++sweep) {
      smooth_launch<T>(s, L, 1, 0, done, p);
      smooth_launch<T>(s, L, 0, 0, done, p);
    }
  }
}

// Preconditioned CG on A e = r (r given in H.r, which is also the fine level's b),
// accumulating scale*e into the FP64 x.  Stops when ||r||^2 <= thr2 or after
// max_it iterations; returns the iterations done and the last ||r||^2.
// The host checks iteration k-1's residual while iteration k is queued; kernels
// of an iteration queued after convergence return at entry (device flag).
template <typename T>
int inner_pcg(gb2d_ctx* c, Solver* S, Hierarchy<T>& H, const double* ainv, double* x64, double scale, double thr2, int max_it, int use_mg, int nu,
              double* last_rr) {
  cudaStream_t s = c->stream;
  Level<T> L = H.L[0];
  T* z = L.x;
  unsigned G = (unsigned)S->nparts;
  double* P_pap = S->part;
  double* P_rr = S->part + kMaxPartials;
  double* P_rz = S->part + 2 * kMaxPartials;
  k_set_int<<<1, 1, 0, s>>>(S->done, 0);
    GB_LAUNCHED(1);
  auto precond = [&]() {
    if (use_mg) {
      vcycle<T>(s, H, ainv, nu, S->done, &c->probe);
    } else {
      k_jacobi<T><<<G, kThreads, 0, s>>>(L, H.r, z, S->done);
      GB_LAUNCHED(1);
    }
  };
  precond();
  k_dot<T><<<G, kThreads, 0, s>>>(L, H.r, z, P_rz, S->done);
    GB_LAUNCHED(1);
  k_p_update<T><<<G, kThreads, 0, s>>>(L, H.p, z, P_rz, G, S->sc, 0, 1, S->done);
    GB_LAUNCHED(1);
  int k = 0, iters = -1;
  while (k < max_it) {
    int par = k & 1;
    k_apply_dot<T><<<G, kThreads, 0, s>>>(L, H.p, H.ap, P_pap, S->done);
    GB_LAUNCHED(1);
    k_cg_update<T><<<G, kThreads, 0, s>>>(L, x64, H.r, H.p, H.ap, P_pap, G, S->sc, par, scale, P_rr, S->done);
    GB_LAUNCHED(1);
    k_finalize<<<1, kThreads, 0, s>>>(P_rr, G, S->sc, thr2, S->done, S->host + par);
    GB_LAUNCHED(1);
    cudaEventRecord(S->ev[par], s);
    precond();
    k_dot<T><<<G, kThreads, 0, s>>>(L, H.r, z, P_rz, S->done);
    GB_LAUNCHED(1);
    k_p_update<T><<<G, kThreads, 0, s>>>(L, H.p, z, P_rz, G, S->sc, par ^ 1, 0, S->done);
    GB_LAUNCHED(1);
    if (k >= 1) {
      cudaEventSynchronize(S->ev[(k - 1) & 1]);
      double v = S->host[(k - 1) & 1];
      if (!(v > thr2)) {
        iters = k;
        *last_rr = v;
        break;
      }
    }
    k++;
  }
  cudaStreamSynchronize(s);
  if (iters < 0) {
    iters = k;
    *last_rr = k > 0 ? S->host[(k - 1) & 1] : *last_rr;
  }
  return iters;
}

}  // namespace

Solver* solver_create(int ni, int nj, char* err, size_t errlen) {
  Solver* S = new Solver();
  S->ni = ni;
  S->nj = nj;
  size_t n = (size_t)ni * nj;
  S->nparts = (int)nblocks(n, 1216);
  size_t np = (size_t)(ni + 2) * (nj + 2);
  cudaError_t e = alloc_hierarchy(S->h64, ni, nj);
  if (e == cudaSuccess) e = alloc_hierarchy(S->h32, ni, nj);
  if (e == cudaSuccess) e = cudaMalloc(&S->ainv64, sizeof(double) * kCoarseMax * kCoarseMax);
  if (e == cudaSuccess) e = cudaMalloc(&S->ainv32, sizeof(double) * kCoarseMax * kCoarseMax);
  if (e == cudaSuccess) e = cudaMalloc(&S->b64, np * sizeof(double));
  if (e == cudaSuccess) e = cudaMemset(S->b64, 0, np * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&S->r64, np * sizeof(double));
  if (e == cudaSuccess) e = cudaMemset(S->r64, 0, np * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&S->part, sizeof(double) * kSlots * kMaxPartials);
  if (e == cudaSuccess) e = cudaMalloc(&S->done, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&S->sc, sizeof(Scalars));
  if (e == cudaSuccess) e = cudaMemset(S->sc, 0, sizeof(Scalars));
  if (e == cudaSuccess) e = cudaMallocHost(&S->host, 8 * sizeof(double));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S->ev[0], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S->ev[1], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    snprintf(err, errlen, "solver allocation failed: %s", cudaGetErrorString(e));
    solver_destroy(S);
    return nullptr;
  }
  return S;
}

void solver_destroy(Solver* S) {
  if (!S) return;
  free_hierarchy(S->h64);
  free_hierarchy(S->h32);
  double* d[] = {S->ainv64, S->ainv32, S->b64, S->r64, S->part};
  for (auto p : d)
    if (p) cudaFree(p);
  if (S->done) cudaFree(S->done);
  if (S->sc) cudaFree(S->sc);
  if (S->host) cudaFreeHost(S->host);
  for (auto e : S->ev)
    if (e) cudaEventDestroy(e);
  delete S;
}

// x: padded FP64 solution (warm start in, result out); the system is ctx->bx/by/diag/rhs.
int solver_solve(gb2d_ctx* c, const double* /*rhs*/, double* x, const gb2d_solve_opts* o, gb2d_solve_stats* st) {
  Solver* S = c->solver;
  cudaStream_t s = c->stream;
  int nu = o->mg_smooth > 0 ? o->mg_smooth : 2;
  int use_mg = o->solver == GB2D_SOLVER_MGPCG;
  bool mixed = o->precision == GB2D_PRECISION_MIXED;
  double tol = o->tolerance > 0 ? o->tolerance : 1e-8;
  double tin = o->inner_tolerance > 0 ? o->inner_tolerance : 1e-4;
  int max_it = o->max_iterations > 0 ? o->max_iterations : 10000;
  unsigned G = (unsigned)S->nparts;
  double* P_rr = S->part + kMaxPartials;
  double* P_bb = S->part + 3 * kMaxPartials;

  build_hierarchy<double>(s, S->h64, c, S->b64, S->ainv64);
  if (mixed && use_mg) build_hierarchy<float>(s, S->h32, c, nullptr, S->ainv32);
  if (mixed && !use_mg) {
    // Jacobi needs only the fine FP32 level.
    double idx2 = 1.0 / (c->base.dx * c->base.dx), idy2 = 1.0 / (c->base.dy * c->base.dy);
    k_build_level0<float><<<nblocks((size_t)c->grid.ni * c->grid.nj, 1216), kThreads, 0, s>>>(c->bx, c->by, c->diag, c->rhs, S->h32.L[0], nullptr,
                                                                                                idx2, idy2);
    GB_LAUNCHED(1);
  }
  int total = 0, outer = 0;
  double rr = 0, bb = 0;
  int status = GB2D_OK;
  while (true) {
    // FP64 residual with the reference's entries; FP32 copy for the mixed inner solve.
    if (mixed)
      k_residual64<float><<<G, kThreads, 0, s>>>(S->h64.L[0], x, S->b64, nullptr, S->h32.r, P_rr, P_bb);
    else
      k_residual64<double><<<G, kThreads, 0, s>>>(S->h64.L[0], x, S->b64, nullptr, S->h64.r, P_rr, P_bb);
    GB_LAUNCHED(1);
    k_reduce_two<<<1, kThreads, 0, s>>>(P_rr, P_bb, G, S->host + 4);
    GB_LAUNCHED(1);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      snprintf(c->err, sizeof(c->err), "pressure solve: %s", cudaGetErrorString(e));
      return GB2D_ERR_CUDA;
    }
    rr = S->host[4];
    bb = S->host[5];
    if (!std::isfinite(rr) || !std::isfinite(bb)) {
      snprintf(c->err, sizeof(c->err), "pressure solve: non-finite residual");
      status = GB2D_ERR_NONFINITE;
      break;
    }
    double thr2 = tol * tol * bb;
    if (rr <= thr2 || bb == 0.0) break;
    if (total >= max_it) {
      status = GB2D_ERR_MAX_ITERS;
      break;
    }
    double rr_in = rr;
    int it;
    if (mixed) {
      double thr_in = tin * tin * rr;
      it = inner_pcg<float>(c, S, S->h32, S->ainv32, x, 1.0, thr_in > thr2 ? thr_in : thr2, max_it - total, use_mg, nu, &rr_in);
    } else {
      it = inner_pcg<double>(c, S, S->h64, S->ainv64, x, 1.0, thr2, max_it - total, use_mg, nu, &rr_in);
    }
    total += it;
    outer++;
    if (!std::isfinite(rr_in)) {
      snprintf(c->err, sizeof(c->err), "pressure solve: non-finite inner residual");
      status = GB2D_ERR_NONFINITE;
      break;
    }
    if (outer > 64) {
      status = GB2D_ERR_MAX_ITERS;
      break;
    }
  }
  if (st) {
    st->iterations = total;
    st->outer_iterations = outer;
    st->rel_residual = bb > 0 ? std::sqrt(rr / bb) : 0.0;
  }
  if (status == GB2D_ERR_MAX_ITERS)
    snprintf(c->err, sizeof(c->err), "pressure solve stopped at %d iterations, relative residual %.3e", total, bb > 0 ? std::sqrt(rr / bb) : 0.0);
  return status;
}

}  // namespace gb2d
