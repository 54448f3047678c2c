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
// Kernel structure of one V-cycle: on every level with more than 64^2 cells a
// smoothing sweep is ONE launch over 32x16 tiles (the tile plus a halo is staged
// in shared memory, red and black half sweeps run back to back, halo cells are
// recomputed redundantly); the last pre-sweep also forms the residual and
// restricts it, the first post-sweep also prolongs the coarse correction.  All
// levels from 64^2 down run inside one single-CTA kernel with x and b in shared
// memory.  One CG iteration is two more kernels, and each iteration is replayed
// from a CUDA graph.
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

constexpr int TX = 32, TY = 16;  // smoothing tile (even, so restriction stays inside a tile)
constexpr int kTailCells = 64 * 64;
constexpr int kTailThreads = 1024;

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

// Partials written by other blocks: read through L2 (__ldcg), never a stale L1 line.
__device__ double sum_partials(const double* part, int n) {
  double v = 0.0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) v += __ldcg(&part[k]);
  return block_sum(v);
}

__device__ __forceinline__ unsigned block_linear() { return blockIdx.x + blockIdx.y * gridDim.x; }

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
// without pivoting (the operator is SPD).  One block of 1024 threads; each pivot
// step scales the pivot row and updates all other entries in parallel.
template <typename T>
__global__ void __launch_bounds__(1024) k_dense_inverse(Level<T> C, double* __restrict__ ainv) {
  __shared__ double A[kCoarseMax][kCoarseMax + 1];
  __shared__ double prow[kCoarseMax], fcol[kCoarseMax];
  const int n = C.nI * C.nJ;
  if (n > kCoarseMax) return;  // prevented on the host (alloc_hierarchy)
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
    int r = t / n, m = t % n;
    int i = r % C.nI, j = r / C.nI;
    size_t k = (size_t)(i + 1) + (size_t)(j + 1) * C.ld;
    double v = 0.0;
    if (m == r) v = (double)C.dg[k];
    else if (i > 0 && m == r - 1) v = -(double)C.cx[k];
    else if (i < C.nI - 1 && m == r + 1) v = -(double)C.cx[k + 1];
    else if (j > 0 && m == r - C.nI) v = -(double)C.cy[k];
    else if (j < C.nJ - 1 && m == r + C.nI) v = -(double)C.cy[k + C.ld];
    A[r][m] = v;
  }
  __syncthreads();
  for (int kk = 0; kk < n; ++kk) {
    if ((int)threadIdx.x < n) {
      int t = threadIdx.x;
      double piv = A[kk][kk];
      fcol[t] = A[t][kk];
      prow[t] = (t == kk) ? 1.0 / piv : A[kk][t] / piv;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      int r = t / n, m = t % n;
      if (r == kk)
        A[r][m] = prow[m];
      else if (m == kk)
        A[r][m] = -fcol[r] * prow[kk];
      else
        A[r][m] -= fcol[r] * prow[m];
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) ainv[t] = A[t / n][t % n];
}

// ---- tiled smoothing (levels above the tail) ----------------------------------

// Gauss-Seidel value of cell k from the staged neighbours c[-1], c[+1], c[-W], c[+W].
template <typename T, int W>
__device__ __forceinline__ T relax(const Level<T>& L, const T* c, size_t k) {
  return (L.b[k] + L.cx[k] * c[-1] + L.cx[k + 1] * c[1] + L.cy[k] * c[-W] + L.cy[k + L.ld] * c[W]) * L.idg[k];
}

// Stage x over the tile plus a halo of width H (zero outside the domain).  With a
// coarse level given, the piecewise-constant coarse correction is added first.
template <typename T, int H>
__device__ __forceinline__ void stage_x(const Level<T>& L, const Level<T>* C, T* xs, int i0, int j0, bool zero) {
  constexpr int W = TX + 2 * H, HH = TY + 2 * H;
  for (int idx = threadIdx.x; idx < W * HH; idx += blockDim.x) {
    int ci = i0 - H + idx % W, cj = j0 - H + idx / W;
    T v = 0;
    if (!zero && ci >= 0 && ci < L.nI && cj >= 0 && cj < L.nJ) {
      v = L.x[(size_t)(ci + 1) + (size_t)(cj + 1) * L.ld];
      if (C) v += C->x[(size_t)(ci / 2 + 1) + (size_t)(cj / 2 + 1) * C->ld];
    }
    xs[idx] = v;
  }
}

// Half sweep of one colour over the staged region shrunk by `ring` cells per side.
template <typename T, int H>
__device__ __forceinline__ void half_sweep(const Level<T>& L, T* xs, int i0, int j0, int color, int ring) {
  constexpr int W = TX + 2 * H, HH = TY + 2 * H;
  const int RW = W - 2 * ring, RH = HH - 2 * ring;
  for (int idx = threadIdx.x; idx < RW * RH; idx += blockDim.x) {
    int si = ring + idx % RW, sj = ring + idx / RW;
    int ci = i0 - H + si, cj = j0 - H + sj;
    if (((ci + cj) & 1) != color || ci < 0 || ci >= L.nI || cj < 0 || cj >= L.nJ) continue;
    size_t k = (size_t)(ci + 1) + (size_t)(cj + 1) * L.ld;
    T* c = &xs[si + sj * W];
    *c = relax<T, W>(L, c, k);
  }
}

// Pre-smoothing sweep (red, then black) on one tile; with restrict_to, the sweep
// is followed by the residual b - A x on the tile and its average over 2x2
// children written as the coarse right-hand side (halo 3 makes the black values
// one cell outside the tile available for that residual).
template <typename T, int H>
__global__ void __launch_bounds__(256) k_pre_sweep(Level<T> L, Level<T> C, int zero_init, int restrict_to, const int* __restrict__ done) {
  if (*done) return;
  constexpr int W = TX + 2 * H, HH = TY + 2 * H;
  __shared__ T xs[W * HH];
  __shared__ T rs[TX * TY];
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  stage_x<T, H>(L, nullptr, xs, i0, j0, zero_init != 0);
  __syncthreads();
  half_sweep<T, H>(L, xs, i0, j0, 0, 1);
  __syncthreads();
  half_sweep<T, H>(L, xs, i0, j0, 1, 2);
  __syncthreads();
  for (int idx = threadIdx.x; idx < TX * TY; idx += blockDim.x) {
    int ti = idx % TX, tj = idx / TX;
    int ci = i0 + ti, cj = j0 + tj;
    T r = 0;
    if (ci < L.nI && cj < L.nJ) {
      size_t k = (size_t)(ci + 1) + (size_t)(cj + 1) * L.ld;
      const T* c = &xs[(ti + H) + (tj + H) * W];
      L.x[k] = c[0];
      if (restrict_to) {
        T ax = L.dg[k] * c[0] - L.cx[k] * c[-1] - L.cx[k + 1] * c[1] - L.cy[k] * c[-W] - L.cy[k + L.ld] * c[W];
        r = L.b[k] - ax;
      }
    }
    rs[idx] = r;
  }
  if (!restrict_to) return;
  __syncthreads();
  for (int idx = threadIdx.x; idx < (TX / 2) * (TY / 2); idx += blockDim.x) {
    int a = idx % (TX / 2), b = idx / (TX / 2);
    int I = i0 / 2 + a, J = j0 / 2 + b;
    if (I >= C.nI || J >= C.nJ) continue;
    const T* r = &rs[2 * a + 2 * b * TX];
    T acc = r[0] + r[1] + r[TX] + r[TX + 1];
    C.b[(size_t)(I + 1) + (size_t)(J + 1) * C.ld] = (T)0.25 * acc;
  }
}

// Post-smoothing sweep (black, then red) on one tile; with prolong_from, the
// coarse correction is added to x first.  With part_rz (finest level, last
// sweep), the block's share of r.z (b = r, x = z on that level) is written.
template <typename T>
__global__ void __launch_bounds__(256) k_post_sweep(Level<T> L, Level<T> C, int prolong_from, double* __restrict__ part_rz,
                                                   const int* __restrict__ done) {
  if (*done) return;
  constexpr int H = 2, W = TX + 2 * H, HH = TY + 2 * H;
  __shared__ T xs[W * HH];
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  stage_x<T, H>(L, prolong_from ? &C : nullptr, xs, i0, j0, false);
  __syncthreads();
  half_sweep<T, H>(L, xs, i0, j0, 1, 1);
  __syncthreads();
  half_sweep<T, H>(L, xs, i0, j0, 0, 2);
  __syncthreads();
  double acc = 0.0;
  for (int idx = threadIdx.x; idx < TX * TY; idx += blockDim.x) {
    int ci = i0 + idx % TX, cj = j0 + idx / TX;
    if (ci >= L.nI || cj >= L.nJ) continue;
    size_t k = (size_t)(ci + 1) + (size_t)(cj + 1) * L.ld;
    T z = xs[(idx % TX + H) + (idx / TX + H) * W];
    L.x[k] = z;
    if (part_rz) acc += (double)L.b[k] * (double)z;
  }
  if (part_rz) {
    acc = block_sum(acc);
    if (threadIdx.x == 0) part_rz[block_linear()] = acc;
  }
}

// ---- single-CTA tail: every level from the first with <= 64^2 cells down -------

template <typename T>
struct TailArgs {
  int nlev;
  Level<T> L[kMaxLevels];
  int off[kMaxLevels];  // shared-memory offset (elements) of level l's x; b follows it
  double* part_rz;      // when the tail starts at the finest level: r.z partial (slot 0)
};

template <typename T>
__device__ __forceinline__ void tail_half(const Level<T>& L, T* x, const T* b, int color) {
  int hw = (L.nI + 1) / 2;
  for (int t = threadIdx.x; t < hw * L.nJ; t += blockDim.x) {
    int j = t / hw;
    int i = 2 * (t % hw) + ((j + color) & 1);
    if (i >= L.nI) continue;
    int k = (i + 1) + (j + 1) * L.ld;
    x[k] = (b[k] + L.cx[k] * x[k - 1] + L.cx[k + 1] * x[k + 1] + L.cy[k] * x[k - L.ld] + L.cy[k + L.ld] * x[k + L.ld]) * L.idg[k];
  }
}

template <typename T>
__global__ void __launch_bounds__(kTailThreads) k_tail(TailArgs<T> a, const double* __restrict__ ainv, int nu, const int* __restrict__ done) {
  if (*done) return;
  extern __shared__ unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  const int nl = a.nlev;
  int total = a.off[nl - 1] + 2 * (a.L[nl - 1].nI + 2) * (a.L[nl - 1].nJ + 2);
  for (int t = threadIdx.x; t < total; t += blockDim.x) sm[t] = (T)0;
  __syncthreads();
  {
    const Level<T>& L = a.L[0];
    T* b = sm + a.off[0] + (L.nI + 2) * (L.nJ + 2);
    for (int t = threadIdx.x; t < L.nI * L.nJ; t += blockDim.x) {
      int k = (t % L.nI + 1) + (t / L.nI + 1) * L.ld;
      b[k] = L.b[k];
    }
  }
  __syncthreads();
  for (int l = 0; l < nl - 1; ++l) {
    const Level<T>& L = a.L[l];
    T* x = sm + a.off[l];
    T* b = x + (L.nI + 2) * (L.nJ + 2);
    for (int s = 0; s < nu; ++s) {
      tail_half(L, x, b, 0);
      __syncthreads();
      tail_half(L, x, b, 1);
      __syncthreads();
    }
    const Level<T>& C = a.L[l + 1];
    T* cb = sm + a.off[l + 1] + (C.nI + 2) * (C.nJ + 2);
    for (int t = threadIdx.x; t < C.nI * C.nJ; t += blockDim.x) {
      int I = t % C.nI, J = t / C.nI;
      T acc = 0;
      for (int bb = 0; bb < 2; ++bb)
        for (int aa = 0; aa < 2; ++aa) {
          int i = 2 * I + aa, j = 2 * J + bb;
          if (i >= L.nI || j >= L.nJ) continue;
          int k = (i + 1) + (j + 1) * L.ld;
          T ax = L.dg[k] * x[k] - L.cx[k] * x[k - 1] - L.cx[k + 1] * x[k + 1] - L.cy[k] * x[k - L.ld] - L.cy[k + L.ld] * x[k + L.ld];
          acc += b[k] - ax;
        }
      cb[(I + 1) + (J + 1) * C.ld] = (T)0.25 * acc;
    }
    __syncthreads();
  }
  {
    const Level<T>& C = a.L[nl - 1];
    T* x = sm + a.off[nl - 1];
    T* b = x + (C.nI + 2) * (C.nJ + 2);
    int n = C.nI * C.nJ;
    if ((int)threadIdx.x < n) {
      double acc = 0.0;
      for (int m = 0; m < n; ++m) acc += ainv[(size_t)threadIdx.x * n + m] * (double)b[(m % C.nI + 1) + (m / C.nI + 1) * C.ld];
      x[(threadIdx.x % C.nI + 1) + (threadIdx.x / C.nI + 1) * C.ld] = (T)acc;
    }
    __syncthreads();
  }
  for (int l = nl - 2; l >= 0; --l) {
    const Level<T>& L = a.L[l];
    const Level<T>& C = a.L[l + 1];
    T* x = sm + a.off[l];
    T* b = x + (L.nI + 2) * (L.nJ + 2);
    const T* cx = sm + a.off[l + 1];
    for (int t = threadIdx.x; t < L.nI * L.nJ; t += blockDim.x) {
      int i = t % L.nI, j = t / L.nI;
      x[(i + 1) + (j + 1) * L.ld] += cx[(i / 2 + 1) + (j / 2 + 1) * C.ld];
    }
    __syncthreads();
    for (int s = 0; s < nu; ++s) {
      tail_half(L, x, b, 1);
      __syncthreads();
      tail_half(L, x, b, 0);
      __syncthreads();
    }
  }
  {
    const Level<T>& L = a.L[0];
    const T* x = sm + a.off[0];
    const T* b = x + (L.nI + 2) * (L.nJ + 2);
    double acc = 0.0;
    for (int t = threadIdx.x; t < L.nI * L.nJ; t += blockDim.x) {
      int k = (t % L.nI + 1) + (t / L.nI + 1) * L.ld;
      L.x[k] = x[k];
      acc += (double)b[k] * (double)x[k];
    }
    if (a.part_rz) {
      acc = block_sum(acc);
      if (threadIdx.x == 0) a.part_rz[0] = acc;
    }
  }
}

// ---- CG kernels ------------------------------------------------------------------

// FP64 residual of the refinement loop with the reference's matrix entries:
// r64 = b - A x, its copy in the inner precision; partial ||r||^2 and ||b||^2.
template <typename T>
__global__ void k_residual64(Level<double> L, const double* __restrict__ x, const double* __restrict__ b, T* __restrict__ rT,
                             double* __restrict__ part_rr, double* __restrict__ part_bb) {
  double rr = 0.0, bb = 0.0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)L.nI * L.nJ; t += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    size_t k = cell_index(L, t, i, j);
    double ax = L.dg[k] * x[k] - L.cx[k] * x[k - 1] - L.cx[k + 1] * x[k + 1] - L.cy[k] * x[k - L.ld] - L.cy[k + L.ld] * x[k + L.ld];
    double r = b[k] - ax;
    rT[k] = (T)r;
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

__global__ void k_reduce_two(const double* __restrict__ pa, const double* __restrict__ pb, int nparts, double* out) {
  double a = sum_partials(pa, nparts);
  double b = sum_partials(pb, nparts);
  if (threadIdx.x == 0) {
    out[0] = a;
    out[1] = b;
  }
}

// Search direction and operator: beta = rz_new / rz_old, p_new = z + beta p_old
// (p_new = z when first), Ap = A p_new in flux form, partial p_new.Ap.  The
// neighbours' p_new are formed on the fly from z and p_old.  Block 0 records
// rz_new in rz[par ^ 1] (rz[par] is the value of the previous direction).
template <typename T>
__global__ void k_direction_apply(Level<T> L, const T* __restrict__ z, const T* __restrict__ pold, T* __restrict__ pnew, T* __restrict__ ap,
                                  const double* __restrict__ part_rz, int nrz, Scalars* sc, int par, int first, double* __restrict__ part_pap,
                                  const int* __restrict__ done) {
  if (*done) return;
  double rz = sum_partials(part_rz, nrz);
  double beta = first ? 0.0 : rz / sc->rz[par];
  if (blockIdx.x == 0 && threadIdx.x == 0) sc->rz[par ^ 1] = rz;
  const T bt = (T)beta;
  double acc = 0.0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)L.nI * L.nJ; t += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    size_t k = cell_index(L, t, i, j);
    T pc, pl, pr, pb, pt;
    if (first) {
      pc = z[k], pl = z[k - 1], pr = z[k + 1], pb = z[k - L.ld], pt = z[k + L.ld];
    } else {
      pc = z[k] + bt * pold[k];
      pl = z[k - 1] + bt * pold[k - 1];
      pr = z[k + 1] + bt * pold[k + 1];
      pb = z[k - L.ld] + bt * pold[k - L.ld];
      pt = z[k + L.ld] + bt * pold[k + L.ld];
    }
    T y = L.sh[k] * pc + L.cx[k] * (pc - pl) + L.cx[k + 1] * (pc - pr) + L.cy[k] * (pc - pb) + L.cy[k + L.ld] * (pc - pt);
    pnew[k] = pc;
    ap[k] = y;
    acc += (double)pc * (double)y;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) part_pap[blockIdx.x] = acc;
}

// alpha = r.z / p.Ap;  x (FP64) += alpha p;  r -= alpha Ap;  ||r||^2.  The last
// block to finish sums the partials, stores ||r||^2 for the host and raises the
// done flag at the threshold (or on a non-finite value).
template <typename T>
__global__ void k_cg_update(Level<T> L, double* __restrict__ x, T* __restrict__ r, const T* __restrict__ p, const T* __restrict__ ap,
                            const double* __restrict__ part_pap, int nparts, Scalars* sc, int par, double* __restrict__ part_rr,
                            unsigned* __restrict__ counter, int* __restrict__ done, double* __restrict__ host_rr) {
  if (*done) return;
  double pap = sum_partials(part_pap, nparts);
  double alpha = sc->rz[par] / pap;
  const T at = (T)alpha;
  double acc = 0.0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)L.nI * L.nJ; t += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    size_t k = cell_index(L, t, i, j);
    x[k] += alpha * (double)p[k];
    T rn = r[k] - at * ap[k];
    r[k] = rn;
    acc += (double)rn * (double)rn;
  }
  acc = block_sum(acc);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    part_rr[blockIdx.x] = acc;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  double rr = sum_partials(part_rr, gridDim.x);
  if (threadIdx.x == 0) {
    sc->rr = rr;
    if (!(rr > sc->thr2)) {
      *done = 1;
      if (!isfinite(rr)) sc->flag |= 1;
    }
    *host_rr = rr;
    *counter = 0u;
  }
}

// Jacobi preconditioner z = r / dg with partial r.z.
template <typename T>
__global__ void k_jacobi(Level<T> L, const T* __restrict__ r, T* __restrict__ z, double* __restrict__ part_rz, const int* __restrict__ done) {
  if (*done) return;
  double acc = 0.0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)L.nI * L.nJ; t += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    size_t k = cell_index(L, t, i, j);
    T zv = r[k] * L.idg[k];
    z[k] = zv;
    acc += (double)r[k] * (double)zv;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) part_rz[blockIdx.x] = acc;
}

__global__ void k_begin_inner(Scalars* sc, int* done, double thr2) {
  *done = 0;
  sc->thr2 = thr2;
}

}  // namespace

// ---- host side -------------------------------------------------------------------

template <typename T>
struct Hierarchy {
  int nlev = 0, tail = 0;  // levels [tail, nlev) run in the single-CTA tail kernel
  size_t tail_smem = 0;
  Level<T> L[kMaxLevels];
  T *p[2] = {nullptr, nullptr}, *ap = nullptr, *r = nullptr;  // CG vectors (padded fine layout); z = L[0].x
};

struct GraphSet {
  bool ok = false;
  cudaGraphExec_t init = nullptr, iter[2] = {nullptr, nullptr};
  unsigned long long nodes_init = 0, nodes_iter = 0;
};

struct Solver {
  int ni, nj;
  Hierarchy<double> h64;
  Hierarchy<float> h32;
  double* ainv64 = nullptr;
  double* ainv32 = nullptr;
  double* b64 = nullptr;   // right-hand side, padded
  double* part = nullptr;  // 4 slots x nparts_cap
  int nparts_cap = 0;
  unsigned* counter = nullptr;
  double* host = nullptr;  // pinned: [0..1] per-parity r.r, [4..5] residual / rhs norms
  int* done = nullptr;
  Scalars* sc = nullptr;
  int G = 0;               // blocks of the grid-stride CG kernels
  cudaEvent_t ev[2] = {nullptr, nullptr};
  // Graphs per (precision, solver, smoothing sweeps) and the x they update.
  GraphSet graphs[2][2][3];
  double* graph_x[2][2][3] = {};
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
  T** v[4] = {&H.p[0], &H.p[1], &H.ap, &H.r};
  for (auto a : v) {
    cudaError_t e = cudaMalloc(a, n * sizeof(T));
    if (e != cudaSuccess) return e;
    e = cudaMemset(*a, 0, n * sizeof(T));
    if (e != cudaSuccess) return e;
  }
  int nI = ni, nJ = nj;
  H.nlev = 0;
  H.tail = -1;
  while (true) {
    Level<T>& L = H.L[H.nlev];
    cudaError_t e = alloc_level(L, nI, nJ, H.nlev > 0);
    if (H.nlev == 0) L.b = H.r;  // the fine level's right-hand side is the CG residual
    if (e != cudaSuccess) return e;
    if (H.tail < 0 && nI * nJ <= kTailCells) H.tail = H.nlev;
    H.nlev++;
    if (nI * nJ <= kCoarseMax) break;
    if (H.nlev == kMaxLevels) return cudaErrorInvalidValue;  // aspect ratio too extreme for the dense coarse solve
    nI = (nI + 1) / 2;
    nJ = (nJ + 1) / 2;
  }
  // Shared memory of the tail: x and b of every tail level; start one level lower
  // while it does not fit.
  const size_t kSmemCap = 200 * 1024;
  while (true) {
    size_t elems = 0;
    for (int l = H.tail; l < H.nlev; ++l) elems += 2 * (size_t)(H.L[l].nI + 2) * (H.L[l].nJ + 2);
    H.tail_smem = elems * sizeof(T);
    if (H.tail_smem <= kSmemCap || H.tail == H.nlev - 1) break;
    H.tail++;
  }
  if (H.tail_smem > kSmemCap) return cudaErrorInvalidValue;
  return cudaSuccess;
}

template <typename T>
void free_hierarchy(Hierarchy<T>& H) {
  for (int l = 0; l < H.nlev; ++l) free_level(H.L[l], l > 0);
  T* v[4] = {H.p[0], H.p[1], H.ap, H.r};
  for (auto a : v)
    if (a) cudaFree(a);
}

inline unsigned nblocks(size_t n, unsigned cap) {
  size_t b = (n + kThreads - 1) / kThreads;
  if (b < 1) b = 1;
  return (unsigned)(b < cap ? b : cap);
}

inline dim3 tiles(int nI, int nJ) { return dim3((nI + TX - 1) / TX, (nJ + TY - 1) / TY); }

template <typename T>
void build_hierarchy(cudaStream_t s, Hierarchy<T>& H, const gb2d_ctx* c, double* b64, double* ainv) {
  double idx2 = 1.0 / (c->base.dx * c->base.dx), idy2 = 1.0 / (c->base.dy * c->base.dy);
  Level<T>& L0 = H.L[0];
  k_build_level0<T><<<nblocks((size_t)L0.nI * L0.nJ, 1216), kThreads, 0, s>>>(c->bx, c->by, c->diag, c->rhs, L0, b64, idx2, idy2);
  GB_LAUNCHED(1);
  for (int l = 1; l < H.nlev; ++l) {
    k_coarsen<T><<<nblocks((size_t)H.L[l].nI * H.L[l].nJ, 1216), kThreads, 0, s>>>(H.L[l - 1], H.L[l]);
    GB_LAUNCHED(1);
  }
  k_dense_inverse<T><<<1, 1024, 0, s>>>(H.L[H.nlev - 1], ainv);
  GB_LAUNCHED(1);
}

// Only the finest FP64 level (the refinement residual's operator) and b.
void build_level0_f64(cudaStream_t s, Hierarchy<double>& H, const gb2d_ctx* c, double* b64) {
  double idx2 = 1.0 / (c->base.dx * c->base.dx), idy2 = 1.0 / (c->base.dy * c->base.dy);
  Level<double>& L0 = H.L[0];
  k_build_level0<double><<<nblocks((size_t)L0.nI * L0.nJ, 1216), kThreads, 0, s>>>(c->bx, c->by, c->diag, c->rhs, L0, b64, idx2, idy2);
  GB_LAUNCHED(1);
}

// Algorithmic bytes of one tiled sweep on a level: x read and written, b, 1/dg and
// the two face arrays read once; the restricting sweep also reads dg and writes
// the coarse b, the prolonging sweep also reads the coarse x.
template <typename T>
double sweep_bytes(const Level<T>& L, bool zero_init, bool restrict_to, bool prolong) {
  double n = (double)L.nI * L.nJ;
  double arrays = (zero_init ? 1.0 : 2.0) + 4.0 + (restrict_to ? 1.25 : 0.0) + (prolong ? 0.25 : 0.0);
  return sizeof(T) * n * arrays;
}

inline bool probe_begin(Probe* pr, cudaStream_t s) {
  bool on = pr && pr->on && pr->n < pr->cap;
  if (on) cudaEventRecord(pr->ev[2 * pr->n], s);
  return on;
}
inline void probe_end(Probe* pr, cudaStream_t s, bool on, double bytes) {
  if (!on) return;
  cudaEventRecord(pr->ev[2 * pr->n + 1], s);
  pr->bytes_each[pr->n] = bytes;
  pr->n++;
}

// z = M r: the fine level's x/b are z/r.  part_rz receives r.z partials (one per
// finest-level tile, or one from the tail when it starts at the finest level).
template <typename T>
void vcycle(cudaStream_t s, Hierarchy<T>& H, const double* ainv, int nu, const int* done, double* part_rz, Probe* pr) {
  const int tail = H.tail;
  for (int l = 0; l < tail; ++l) {
    Level<T>& L = H.L[l];
    for (int sweep = 0; sweep < nu; ++sweep) {
      bool last = sweep == nu - 1;
      bool on = l == 0 && probe_begin(pr, s);
      if (last)
        k_pre_sweep<T, 3><<<tiles(L.nI, L.nJ), 256, 0, s>>>(L, H.L[l + 1], sweep == 0, 1, done);
      else
        k_pre_sweep<T, 2><<<tiles(L.nI, L.nJ), 256, 0, s>>>(L, H.L[l + 1], sweep == 0, 0, done);
      GB_LAUNCHED(1);
      probe_end(pr, s, on, sweep_bytes(L, sweep == 0, last, false));
    }
  }
  TailArgs<T> ta;
  memset(&ta, 0, sizeof ta);
  ta.nlev = H.nlev - tail;
  int off = 0;
  for (int l = 0; l < ta.nlev; ++l) {
    ta.L[l] = H.L[tail + l];
    ta.off[l] = off;
    off += 2 * (ta.L[l].nI + 2) * (ta.L[l].nJ + 2);
  }
  ta.part_rz = tail == 0 ? part_rz : nullptr;
  k_tail<T><<<1, kTailThreads, H.tail_smem, s>>>(ta, ainv, nu, done);
  GB_LAUNCHED(1);
  for (int l = tail - 1; l >= 0; --l) {
    Level<T>& L = H.L[l];
    for (int sweep = 0; sweep < nu; ++sweep) {
      bool first = sweep == 0;
      double* prz = (l == 0 && sweep == nu - 1) ? part_rz : nullptr;
      bool on = l == 0 && probe_begin(pr, s);
      k_post_sweep<T><<<tiles(L.nI, L.nJ), 256, 0, s>>>(L, H.L[l + 1], first, prz, done);
      GB_LAUNCHED(1);
      probe_end(pr, s, on, sweep_bytes(L, false, false, first));
    }
  }
}

template <typename T>
int n_rz_parts(const Hierarchy<T>& H, bool use_mg, unsigned G) {
  if (!use_mg) return (int)G;
  if (H.tail == 0) return 1;
  dim3 t = tiles(H.L[0].nI, H.L[0].nJ);
  return (int)(t.x * t.y);
}

// Preconditioner + first direction: z = M r, p[0] = z, Ap, rz[0].
template <typename T>
void enqueue_init(cudaStream_t s, Solver* S, Hierarchy<T>& H, const double* ainv, int use_mg, int nu, Probe* pr) {
  Level<T>& L = H.L[0];
  double* P_pap = S->part;
  double* P_rz = S->part + 2 * (size_t)S->nparts_cap;
  if (use_mg) {
    vcycle<T>(s, H, ainv, nu, S->done, P_rz, pr);
  } else {
    k_jacobi<T><<<S->G, kThreads, 0, s>>>(L, H.r, L.x, P_rz, S->done);
    GB_LAUNCHED(1);
  }
  k_direction_apply<T><<<S->G, kThreads, 0, s>>>(L, L.x, H.p[1], H.p[0], H.ap, P_rz, n_rz_parts(H, use_mg, S->G), S->sc, 1, 1, P_pap, S->done);
  GB_LAUNCHED(1);
}

// One CG iteration with direction p[par]: update x and r, precondition, next direction p[par^1].
template <typename T>
void enqueue_iter(cudaStream_t s, Solver* S, Hierarchy<T>& H, const double* ainv, double* x64, int use_mg, int nu, int par, Probe* pr) {
  Level<T>& L = H.L[0];
  double* P_pap = S->part;
  double* P_rr = S->part + (size_t)S->nparts_cap;
  double* P_rz = S->part + 2 * (size_t)S->nparts_cap;
  k_cg_update<T><<<S->G, kThreads, 0, s>>>(L, x64, H.r, H.p[par], H.ap, P_pap, S->G, S->sc, par, P_rr, S->counter, S->done, S->host + par);
  GB_LAUNCHED(1);
  if (use_mg) {
    vcycle<T>(s, H, ainv, nu, S->done, P_rz, pr);
  } else {
    k_jacobi<T><<<S->G, kThreads, 0, s>>>(L, H.r, L.x, P_rz, S->done);
    GB_LAUNCHED(1);
  }
  k_direction_apply<T><<<S->G, kThreads, 0, s>>>(L, L.x, H.p[par], H.p[par ^ 1], H.ap, P_rz, n_rz_parts(H, use_mg, S->G), S->sc, par, 0, P_pap,
                                                 S->done);
  GB_LAUNCHED(1);
}

// Capture fn's launches on the context's own stream into an executable graph.
template <typename F>
bool capture_graph(gb2d_ctx* c, cudaGraphExec_t* exec, unsigned long long* nodes, F fn) {
  cudaStream_t cs = c->own_stream;
  unsigned long long before = g_launches;
  if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  fn(cs);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(cs, &g);
  *nodes = g_launches - before;
  g_launches = before;  // captured launches are counted when the graph runs
  if (e != cudaSuccess || !g) {
    cudaGetLastError();
    return false;
  }
  e = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *exec = nullptr;
    return false;
  }
  return true;
}

template <typename T>
GraphSet* graphs_for(gb2d_ctx* c, Solver* S, Hierarchy<T>& H, const double* ainv, double* x64, int prec, int use_mg, int nu) {
  int slot = nu - 1;
  GraphSet& gs = S->graphs[prec][use_mg][slot];
  if (gs.ok && S->graph_x[prec][use_mg][slot] == x64) return &gs;
  if (gs.init) cudaGraphExecDestroy(gs.init);
  for (auto& g : gs.iter)
    if (g) cudaGraphExecDestroy(g);
  gs = GraphSet();
  bool ok = capture_graph(c, &gs.init, &gs.nodes_init, [&](cudaStream_t cs) { enqueue_init<T>(cs, S, H, ainv, use_mg, nu, nullptr); });
  for (int par = 0; par < 2 && ok; ++par)
    ok = capture_graph(c, &gs.iter[par], &gs.nodes_iter, [&](cudaStream_t cs) { enqueue_iter<T>(cs, S, H, ainv, x64, use_mg, nu, par, nullptr); });
  gs.ok = ok;
  S->graph_x[prec][use_mg][slot] = x64;
  return ok ? &gs : nullptr;
}

// Preconditioned CG on A e = r (r in H.r, the fine level's b), accumulating e into
// the FP64 x.  Stops when ||r||^2 <= thr2 or after max_it iterations; returns the
// iterations done and the last ||r||^2.  The host checks iteration k-1's residual
// while iteration k is queued; work queued after convergence returns at entry.
template <typename T>
int inner_pcg(gb2d_ctx* c, Solver* S, Hierarchy<T>& H, const double* ainv, double* x64, double thr2, int max_it, int prec, int use_mg, int nu,
              double* last_rr) {
  cudaStream_t s = c->stream;
  Probe* pr = &c->probe;
  GraphSet* gs = pr->on ? nullptr : graphs_for<T>(c, S, H, ainv, x64, prec, use_mg, nu);
  k_begin_inner<<<1, 1, 0, s>>>(S->sc, S->done, thr2);
  GB_LAUNCHED(1);
  if (gs) {
    cudaGraphLaunch(gs->init, s);
    GB_LAUNCHED(gs->nodes_init);
  } else {
    enqueue_init<T>(s, S, H, ainv, use_mg, nu, pr);
  }
  int k = 0, iters = -1;
  while (k < max_it) {
    int par = k & 1;
    if (gs) {
      cudaGraphLaunch(gs->iter[par], s);
      GB_LAUNCHED(gs->nodes_iter);
    } else {
      enqueue_iter<T>(s, S, H, ainv, x64, use_mg, nu, par, pr);
    }
    cudaEventRecord(S->ev[par], s);
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
    if (k > 0) *last_rr = S->host[(k - 1) & 1];
  }
  return iters;
}

}  // namespace

Solver* solver_create(int ni, int nj, char* err, size_t errlen) {
  Solver* S = new Solver();
  S->ni = ni;
  S->nj = nj;
  size_t n = (size_t)ni * nj;
  S->G = (int)nblocks(n, 1216);
  dim3 t = tiles(ni, nj);
  S->nparts_cap = (int)(t.x * t.y) > S->G ? (int)(t.x * t.y) : S->G;
  size_t np = (size_t)(ni + 2) * (nj + 2);
  cudaError_t e = alloc_hierarchy(S->h64, ni, nj);
  if (e == cudaSuccess) e = alloc_hierarchy(S->h32, ni, nj);
  if (e == cudaSuccess) e = cudaMalloc(&S->ainv64, sizeof(double) * kCoarseMax * kCoarseMax);
  if (e == cudaSuccess) e = cudaMalloc(&S->ainv32, sizeof(double) * kCoarseMax * kCoarseMax);
  if (e == cudaSuccess) e = cudaMalloc(&S->b64, np * sizeof(double));
  if (e == cudaSuccess) e = cudaMemset(S->b64, 0, np * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&S->part, sizeof(double) * 4 * (size_t)S->nparts_cap);
  if (e == cudaSuccess) e = cudaMemset(S->part, 0, sizeof(double) * 4 * (size_t)S->nparts_cap);
  if (e == cudaSuccess) e = cudaMalloc(&S->counter, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(S->counter, 0, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&S->done, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(S->done, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&S->sc, sizeof(Scalars));
  if (e == cudaSuccess) e = cudaMemset(S->sc, 0, sizeof(Scalars));
  if (e == cudaSuccess) e = cudaMallocHost(&S->host, 8 * sizeof(double));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S->ev[0], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S->ev[1], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_tail<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S->h64.tail_smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_tail<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S->h32.tail_smem);
  if (e != cudaSuccess) {
    snprintf(err, errlen, "solver allocation failed: %s", cudaGetErrorString(e));
    solver_destroy(S);
    return nullptr;
  }
  return S;
}

void solver_destroy(Solver* S) {
  if (!S) return;
  for (auto& a : S->graphs)
    for (auto& b : a)
      for (auto& g : b) {
        if (g.init) cudaGraphExecDestroy(g.init);
        for (auto& it : g.iter)
          if (it) cudaGraphExecDestroy(it);
      }
  free_hierarchy(S->h64);
  free_hierarchy(S->h32);
  double* d[] = {S->ainv64, S->ainv32, S->b64, S->part};
  for (auto p : d)
    if (p) cudaFree(p);
  if (S->counter) cudaFree(S->counter);
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
  int nu = o->mg_smooth > 0 ? (o->mg_smooth > 3 ? 3 : o->mg_smooth) : 2;
  int use_mg = o->solver == GB2D_SOLVER_MGPCG;
  int prec = o->precision == GB2D_PRECISION_MIXED ? 1 : 0;
  double tol = o->tolerance > 0 ? o->tolerance : 1e-8;
  double tin = o->inner_tolerance > 0 ? o->inner_tolerance : 1e-4;
  int max_it = o->max_iterations > 0 ? o->max_iterations : 10000;
  unsigned G = (unsigned)S->G;
  double* P_rr = S->part + (size_t)S->nparts_cap;
  double* P_bb = S->part + 3 * (size_t)S->nparts_cap;

  if (prec || !use_mg)
    build_level0_f64(s, S->h64, c, S->b64);
  else
    build_hierarchy<double>(s, S->h64, c, S->b64, S->ainv64);
  if (prec && use_mg) build_hierarchy<float>(s, S->h32, c, nullptr, S->ainv32);
  if (prec && !use_mg) {
    double idx2 = 1.0 / (c->base.dx * c->base.dx), idy2 = 1.0 / (c->base.dy * c->base.dy);
    k_build_level0<float><<<nblocks((size_t)c->grid.ni * c->grid.nj, 1216), kThreads, 0, s>>>(c->bx, c->by, c->diag, c->rhs, S->h32.L[0], nullptr,
                                                                                                idx2, idy2);
    GB_LAUNCHED(1);
  }
  int total = 0, outer = 0;
  double rr = 0, bb = 0;
  int status = GB2D_OK;
  while (true) {
    // FP64 residual with the reference's entries, copied into the inner precision.
    if (prec)
      k_residual64<float><<<G, kThreads, 0, s>>>(S->h64.L[0], x, S->b64, S->h32.r, P_rr, P_bb);
    else
      k_residual64<double><<<G, kThreads, 0, s>>>(S->h64.L[0], x, S->b64, S->h64.r, P_rr, P_bb);
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
    if (prec) {
      double thr_in = tin * tin * rr;
      it = inner_pcg<float>(c, S, S->h32, S->ainv32, x, thr_in > thr2 ? thr_in : thr2, max_it - total, prec, use_mg, nu, &rr_in);
    } else {
      it = inner_pcg<double>(c, S, S->h64, S->ainv64, x, thr2, max_it - total, prec, use_mg, nu, &rr_in);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) {
      snprintf(c->err, sizeof(c->err), "pressure solve: %s", cudaGetErrorString(e));
      return GB2D_ERR_CUDA;
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
