// Pressure solver: multigrid-preconditioned CG on the matrix-free 5-point
// ghost-fluid operator.  The CG (x, r, p, A p, every dot product) is FP64 with
// the reference's own matrix entries; the preconditioner (a symmetric V-cycle,
// or Jacobi) runs in FP64, or in FP32 on an FP32 copy of r for
// GB2D_PRECISION_MIXED.
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
// Kernel structure of one V-cycle: every level above the cluster tail does each
// side of its smoothing in ONE tiled launch (the tile plus a halo is staged in
// shared memory, the red and black half sweeps run back to back, halo cells are
// recomputed redundantly); the pre-smoothing launch also forms the residual and
// restricts it, the post-smoothing launch also prolongs the coarse correction.
// The levels from 128^2 down run in one launch of a 16-CTA thread-block cluster
// (gb2d_ctail.cuh), neighbour rows read from the other CTAs' shared memory; a
// single-CTA kernel over the levels from 64^2 down is the fallback.  One CG
// iteration adds three FP64 kernels (direction, operator product with p.Ap,
// update with r.r), and each iteration is replayed from a CUDA graph whose
// kernels use programmatic dependent launch.  The loop around the CG recomputes
// the true FP64 residual and restarts only if the recursive residual drifted.
//
// All reductions are two-stage and deterministic: blocks write partial sums,
// consumers re-reduce the partials in a fixed order.
#include <cooperative_groups.h>

#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <utility>

#include "gb2d_internal.cuh"

namespace gb2d {

namespace {

constexpr int kTailCells = 64 * 64;
constexpr int kTailThreads = 1024;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ int linear_tid() { return threadIdx.x + threadIdx.y * blockDim.x; }
__device__ __forceinline__ int block_threads() { return blockDim.x * blockDim.y; }

// Shared scratch of the block reductions: one array for every reduction helper
// that a kernel uses, so that they add 264 bytes of static shared memory once
// (one byte more can cost a resident block on the smoothing kernels).
__device__ __forceinline__ double* reduce_scratch() {
  __shared__ double buf[33];
  return buf;
}

// Deterministic block sum (block size a multiple of 32, <= 1024); result valid in every thread.
__device__ double block_sum(double v) {
  double* sm = reduce_scratch();
  double& total = sm[32];
  int tid = linear_tid();
  int lane = tid & 31, w = tid >> 5, nw = block_threads() >> 5;
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

// Double-float values (two FP32 words, about 48 significant bits) summed on the
// FP32 pipe: GB300 issues FP64 at a small fraction of its FP32 rate, and an FP64
// shuffle tree in every warp cost as many FP64 instructions as the vector update
// it reduced.  Every operation rounds as written (no contraction), so a sum is
// fixed by the order of its operands.  df_add: Knuth's TwoSum of the leading
// words, the trailing words added to its error, then Dekker's Fast2Sum.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF df_add(DF a, DF b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  const float t = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  const float h = __fadd_rn(s, t);
  return DF{h, __fsub_rn(t, __fsub_rn(h, s))};
}
__device__ __forceinline__ DF warp_sum_df(DF v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = df_add(v, DF{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)});
  return v;
}
// Deterministic block sum of double-float values, as FP64 (valid in every thread).
__device__ double block_sum_df(DF v) {
  double* sm = reduce_scratch();
  float* shi = reinterpret_cast<float*>(sm);
  float* slo = shi + 32;
  double& total = sm[32];
  int tid = linear_tid();
  int lane = tid & 31, w = tid >> 5, nw = block_threads() >> 5;
  v = warp_sum_df(v);
  __syncthreads();
  if (lane == 0) {
    shi[w] = v.hi;
    slo[w] = v.lo;
  }
  __syncthreads();
  if (w == 0) {
    DF x = lane < nw ? DF{shi[lane], slo[lane]} : DF{0.f, 0.f};
    x = warp_sum_df(x);
    if (lane == 0) total = widen(x.hi) + widen(x.lo);
  }
  __syncthreads();
  return total;
}

// Partials written by other blocks: read through L2 (__ldcg), never a stale L1 line.
__device__ double sum_partials(const double* part, int n) {
  double v = 0.0;
  for (int k = linear_tid(); k < n; k += block_threads()) v += __ldcg(&part[k]);
  return block_sum(v);
}

__device__ __forceinline__ unsigned block_linear() { return blockIdx.x + blockIdx.y * gridDim.x; }

// Programmatic dependent launch inside the solver's launch chains: wait until the
// previous kernel in the stream has completed (its writes visible), then let the
// next kernel start launching, so launch latency and block scheduling overlap
// this kernel's tail instead of following it.  Both are no-ops for kernels
// launched without the programmatic-serialization attribute.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// The FP64 inputs in the hierarchy's precision: FP32 levels are built in FP32
// arithmetic from truncated inputs (preconditioner data; FP64 divides and
// conversions would take the scarce FP64 issue slots).
__device__ __forceinline__ float in_prec(double v, float) { return narrow(v); }
__device__ __forceinline__ double in_prec(double v, double) { return v; }

// Level 0 from the assembled FP64 system: conductances beta/dx^2 on interior
// faces, zero on walls; diagonal as assembled; shift = pin + (dx != dy) terms.
template <typename T>
__global__ void k_build_level0(const double* __restrict__ bx, const double* __restrict__ by, const double* __restrict__ diag,
                               const double* __restrict__ rhs, const double* __restrict__ shift, Level<T> L, double* __restrict__ b64,
                               double idx2_, double idy2_) {
  int ni = L.nI, nj = L.nJ;
  const T idx2 = in_prec(idx2_, T()), idy2 = in_prec(idy2_, T()), zero = 0;
  GB_FOR_IJ(i, j, ni, nj) {
    const size_t t = (size_t)j * ni + i;
    const size_t k = (size_t)(i + 1) + (size_t)(j + 1) * L.ld;
    const T bl = in_prec(bx[i + (size_t)j * (ni + 1)], T());
    const T bb = in_prec(by[i + (size_t)j * ni], T()), bt = in_prec(by[i + (size_t)(j + 1) * ni], T());
    L.cx[k] = i > 0 ? bl * idx2 : zero;
    L.cy[k] = j > 0 ? bb * idy2 : zero;
    if (i == ni - 1) L.cx[k + 1] = zero;
    if (j == nj - 1) L.cy[k + L.ld] = zero;
    const T d = in_prec(diag[t], T());
    L.dg[k] = d;
    L.idg[k] = (T)1 / d;
    if (shift) {  // a system that states its diagonal beyond the face conductances itself
      L.sh[k] = in_prec(shift[t], T());
    } else {  // the projection's: the corner pin and the dx-only diagonal's y-face excess
      const T ybeta = (j > 0 ? bb : zero) + (j < nj - 1 ? bt : zero);
      const T pin = (i == 0 && j == 0) ? (bl + bb) : zero;
      L.sh[k] = pin * idx2 + ybeta * (idx2 - idy2);
    }
    if (b64) b64[k] = rhs[t];
  }
}

// Coarse level: cell (I, J) covers fine cells (2I..2I+1, 2J..2J+1) that exist.
// Face conductances: sum of the two fine faces / 8 (face-averaged weight over
// the doubled spacing); shift: average of the children's shifts.  In the
// level's precision.
template <typename T>
__global__ void k_coarsen(Level<T> F, Level<T> C) {
  int cI = C.nI, cJ = C.nJ;
  const T eighth = (T)0.125, zero = 0;
  GB_FOR_IJ(I, J, cI, cJ) {
    const size_t k = (size_t)(I + 1) + (size_t)(J + 1) * C.ld;
    auto fx = [&](int fi, int fj) -> T {  // fine x-face fi at fine row fj (0 outside)
      if (fj >= F.nJ) return zero;
      return F.cx[(size_t)(fi + 1) + (size_t)(fj + 1) * F.ld];
    };
    auto fy = [&](int fi, int fj) -> T {
      if (fi >= F.nI) return zero;
      return F.cy[(size_t)(fi + 1) + (size_t)(fj + 1) * F.ld];
    };
    const T cl = I > 0 ? (fx(2 * I, 2 * J) + fx(2 * I, 2 * J + 1)) * eighth : zero;
    const T cr = I < cI - 1 ? (fx(2 * I + 2, 2 * J) + fx(2 * I + 2, 2 * J + 1)) * eighth : zero;
    const T cb = J > 0 ? (fy(2 * I, 2 * J) + fy(2 * I + 1, 2 * J)) * eighth : zero;
    const T ct = J < cJ - 1 ? (fy(2 * I, 2 * J + 2) + fy(2 * I + 1, 2 * J + 2)) * eighth : zero;
    T s = 0;
    for (int b = 0; b < 2; ++b)
      for (int a = 0; a < 2; ++a) {
        int fi = 2 * I + a, fj = 2 * J + b;
        if (fi < F.nI && fj < F.nJ) s += F.sh[(size_t)(fi + 1) + (size_t)(fj + 1) * F.ld];
      }
    s *= (T)0.25;
    C.cx[k] = cl;
    C.cy[k] = cb;
    if (I == cI - 1) C.cx[k + 1] = zero;
    if (J == cJ - 1) C.cy[k + C.ld] = zero;
    const T d = cl + cr + cb + ct + s;
    C.dg[k] = d;
    C.idg[k] = (T)1 / d;
    C.sh[k] = s;
  }
}

// Dense inverse of the coarsest operator (n <= 64), Gauss-Jordan without
// pivoting (the operator is SPD), computed in the hierarchy's precision (one SM's
// FP64 rate makes the FP64 elimination ~60 us; the FP32 one takes a few).  One
// block of 1024 threads, thread t owning row t/16 and columns t%16 + 16q
// (q = 0..3) in registers; each pivot step publishes the pivot row, the pivot
// column and the pivot's reciprocal through shared memory.
template <typename T>
__global__ void __launch_bounds__(1024) k_dense_inverse(Level<T> C, double* __restrict__ ainv) {
  static_assert(kCoarseMax == 64, "register blocking assumes 64 x 64");
  __shared__ T prow[kCoarseMax], fcol[kCoarseMax];
  __shared__ T s_inv;
  const int n = C.nI * C.nJ;
  if (n > kCoarseMax) return;  // prevented on the host (alloc_hierarchy)
  const int r = threadIdx.x >> 4, m0 = threadIdx.x & 15;
  const bool rok = r < n;
  T a[4];
  {
    int ri = 0, rj = 0;
    size_t k = 0;
    if (rok) {
      ri = r % C.nI;
      rj = r / C.nI;
      k = (size_t)(ri + 1) + (size_t)(rj + 1) * C.ld;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int m = m0 + 16 * q;
      T v = 0;
      if (rok && m < n) {
        if (m == r) v = C.dg[k];
        else if (ri > 0 && m == r - 1) v = -C.cx[k];
        else if (ri < C.nI - 1 && m == r + 1) v = -C.cx[k + 1];
        else if (rj > 0 && m == r - C.nI) v = -C.cy[k];
        else if (rj < C.nJ - 1 && m == r + C.nI) v = -C.cy[k + C.ld];
      }
      a[q] = v;
    }
  }
  for (int kk = 0; kk < n; ++kk) {
    const int qk = kk >> 4;
    const T own_col = qk == 0 ? a[0] : qk == 1 ? a[1] : qk == 2 ? a[2] : a[3];
    if (r == kk) {
#pragma unroll
      for (int q = 0; q < 4; ++q) prow[m0 + 16 * q] = a[q];
      if (m0 == (kk & 15)) s_inv = (T)1 / own_col;
    }
    if (rok && m0 == (kk & 15)) fcol[r] = own_col;
    __syncthreads();
    const T inv = s_inv;
    const T fr = rok ? fcol[r] : (T)0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int m = m0 + 16 * q;
      if (!rok || m >= n) continue;
      const T pm = m == kk ? inv : prow[m] * inv;
      if (r == kk)
        a[q] = pm;
      else if (m == kk)
        a[q] = -fr * inv;
      else
        a[q] -= fr * pm;
    }
    __syncthreads();
  }
  if (rok) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int m = m0 + 16 * q;
      if (m < n) ainv[(size_t)r * n + m] = (double)a[q];
    }
  }
}

// ---- tiled smoothing (levels above the tail) ----------------------------------
//
// A block of 32x8 threads owns a tile of 64x16 cells (shape 0), 32x16 (shape 1),
// 32x8 (shape 2) or 32x32 (shape 3); its 2x2 quads of cells, each one coarse cell,
// are dealt to the threads in order (shapes 0 and 3: one quad per thread).  The
// smaller tiles serve the coarser levels, where a level has fewer large tiles than
// the GPU has SMs and a launch lasts as long as one tile's staging and sweeps:
// a smaller window halves the loads and half-sweep cells per thread.  All NS
// red-black sweeps of one side of the V-cycle run in ONE launch: the block stages
// x and the coefficients (b, 1/dg, cx, cy, and dg when it restricts) for the tile
// plus a halo of 2 NS (+1 to restrict) cells in shared memory with unrolled,
// compile-time-bounded loops, runs the 2 NS half sweeps from shared memory over
// windows shrinking by one cell per side each (the halo is recomputed so that the
// tile's last colour is exact), and writes the tile.  Cells outside the domain
// are staged as zero, which is also the value of every wall-face conductance.
// A launch reads x from one buffer and writes the level's other buffer: blocks
// stage halo cells that neighbouring blocks of the same launch update, so an
// in-place write would let a block read a neighbour's already-smoothed (and,
// when prolonging, already-corrected) value.

constexpr int BXT = 32, BYT = 8;  // threads per block (x, y)
constexpr int kTileShapes = 4;

template <int SH>
struct TileShape {
  static constexpr int X = SH == 0 ? 64 : 32, Y = SH == 2 ? 8 : SH == 3 ? 32 : 16;  // cells of one block's tile
  static constexpr int QX = X / 2, QY = Y / 2;                        // its quads (coarse cells)
};

// The staged window holds W x HH cells per array.  FP64 levels keep it in the
// natural layout (cell (c, r) is element c + r W).  FP32 levels hold it split by
// colour: cell (c, r) is element r WH + c / 2 (WH = W / 2) of plane (c + r) & 1.
// A half sweep then updates one plane and reads its neighbours from the other, so
// consecutive threads touch consecutive elements of each plane; in the natural
// layout the cells of one colour lie two elements apart and every shared-memory
// access of a half sweep takes two bank wavefronts.  FP64 half sweeps are bound by
// the FP64 pipe instead, and the split layout's sweeps run over whole plane rows
// (below), which costs FP64 issue slots.  Where plane 1 starts depends on how the
// window is staged (below): for pair staging at a 128-byte boundary, for cell
// staging 64 bytes past one, so that each warp's staging stores fall in distinct
// banks.
template <typename T, int H, int SH>
struct Win {
  static constexpr bool SPLIT = sizeof(T) == 4, PAIRS = SPLIT && SH == 3;
  static constexpr int W = TileShape<SH>::X + 2 * H, HH = TileShape<SH>::Y + 2 * H, N = W * HH, WH = W / 2;
  static constexpr int E = 128 / (int)sizeof(T), PLANE = HH * WH;
  static constexpr int PO = PAIRS ? (PLANE + E - 1) / E * E : PLANE + (E / 2 - PLANE % E + E) % E;  // plane 1 (elements)
  static constexpr int NA = SPLIT ? 2 * PO : N;  // elements per staged array (a multiple of E when split)
  static_assert(W % 2 == 0, "window rows must hold an even number of cells");
};

template <typename T, int H, bool DG, int SH>
constexpr size_t sweep_smem() {
  return sizeof(T) * (size_t)Win<T, H, SH>::NA * (DG ? 6 : 5);
}

// Element offsets of window cell (c, r) and of its left, right, lower and upper
// neighbours.
struct CellOff {
  int s, l, r, b, t;
};
template <typename T, int H, int SH>
__device__ __forceinline__ CellOff cell_off(int c, int r) {
  using Wn = Win<T, H, SH>;
  if constexpr (Wn::SPLIT) {
    const int m = r * Wn::WH + (c >> 1), pl = (c + r) & 1, o = c & 1, t = (pl ^ 1) * Wn::PO + m;
    return CellOff{pl * Wn::PO + m, t - 1 + o, t + o, t - Wn::WH, t + Wn::WH};
  } else {
    const int e = c + r * Wn::W;
    return CellOff{e, e - 1, e + 1, e - Wn::W, e + Wn::W};
  }
}

template <typename T>
__device__ __forceinline__ void cp_async(T* dst, const T* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(d), "l"(src), "n"((int)sizeof(T)) : "memory");
}
// The same, or zeros when !valid (src-size 0: nothing is read).
template <typename T>
__device__ __forceinline__ void cp_async_zfill(T* dst, const T* src, bool valid) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  const unsigned n = valid ? (unsigned)sizeof(T) : 0u;
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(d), "l"(src), "n"((int)sizeof(T)), "r"(n) : "memory");
}

// Stage the window.  LOAD_X: read x (else zero); PROLONG: add the coarse correction.
// The window is enumerated flat (division by compile-time constants only), so
// every thread of the block has work in every pass.
//   Natural layout: one cell per thread and pass, loaded through registers.
//   Split layout: the coefficients (and x without a correction) are copied with
//   cp.async, so that all of a thread's copies are in flight at once,
//   zero-filled outside the domain by the copy itself.  32x32 tiles (the FP32
//   levels of 1024^2 and more) copy one pair of cells (2m, r), (2m + 1, r) per
//   thread and pass, which land at the same element r WH + m of planes r & 1 and
//   (r + 1) & 1 (half the index arithmetic per cell); the other tiles one cell
//   per thread and pass (one contiguous row segment per warp and copy).
//   Measured on the finest level's two launches, mixed projection: pairs 21.7 /
//   54.0 / 185.8 us against cells 20.7 / 57.5 / 196.0 us at 1024^2 (32x16 tiles),
//   2048^2 and 4096^2 (32x32).
template <typename T, int H, bool LOAD_X, bool PROLONG, bool DG, int SH>
__device__ __forceinline__ void stage_window(const Level<T>& L, const Level<T>& C, T* sm, int i0, int j0) {
  using Wn = Win<T, H, SH>;
  constexpr int W = Wn::W, HH = Wn::HH, N = Wn::N, NA = Wn::NA;
  T *xs = sm, *bs = sm + NA, *is = sm + 2 * NA, *cxs = sm + 3 * NA, *cys = sm + 4 * NA, *ds = sm + 5 * NA;
  const int gi0 = i0 - H, gj0 = j0 - H;
  const bool inner = gi0 >= 0 && gj0 >= 0 && gi0 + W <= L.nI && gj0 + HH <= L.nJ;
  const size_t base = (size_t)(gi0 + 1) + (size_t)(gj0 + 1) * L.ld;
  const int tid = threadIdx.x + threadIdx.y * BXT;
  if constexpr (Wn::SPLIT) {
    if constexpr (Wn::PAIRS) {
      constexpr int WH = Wn::WH, PO = Wn::PO, PLANE = Wn::PLANE;
#pragma unroll
      for (int u0 = 0; u0 < PLANE; u0 += BXT * BYT) {
        const int q = u0 + tid;  // = r WH + m
        if (u0 + BXT * BYT > PLANE && q >= PLANE) continue;
        const int r = q / WH, c = 2 * (q - r * WH);
        const int ea = (r & 1) * PO + q, eb = ((r & 1) ^ 1) * PO + q;
        const int gi = gi0 + c, gj = gj0 + r;
        const bool rok = gj >= 0 && gj < L.nJ;
        const bool ina = inner || (rok && gi >= 0 && gi < L.nI), inb = inner || (rok && gi + 1 >= 0 && gi + 1 < L.nI);
        const size_t k = base + c + (size_t)r * L.ld, ka = ina ? k : 0, kb = inb ? k + 1 : 0;
        if (PROLONG) {
          T xa = 0, xb = 0;
          if (ina) xa = L.x[ka] + C.x[(size_t)(gi / 2 + 1) + (size_t)(gj / 2 + 1) * C.ld];
          if (inb) xb = L.x[kb] + C.x[(size_t)((gi + 1) / 2 + 1) + (size_t)(gj / 2 + 1) * C.ld];
          xs[ea] = xa;
          xs[eb] = xb;
        } else if (LOAD_X) {
          cp_async_zfill(xs + ea, L.x + ka, ina);
          cp_async_zfill(xs + eb, L.x + kb, inb);
        } else {
          xs[ea] = 0;
          xs[eb] = 0;
        }
        if (inner) {
          cp_async(bs + ea, L.b + k);
          cp_async(bs + eb, L.b + k + 1);
          cp_async(is + ea, L.idg + k);
          cp_async(is + eb, L.idg + k + 1);
          cp_async(cxs + ea, L.cx + k);
          cp_async(cxs + eb, L.cx + k + 1);
          cp_async(cys + ea, L.cy + k);
          cp_async(cys + eb, L.cy + k + 1);
          if (DG) {
            cp_async(ds + ea, L.dg + k);
            cp_async(ds + eb, L.dg + k + 1);
          }
        } else {
          cp_async_zfill(bs + ea, L.b + ka, ina);
          cp_async_zfill(bs + eb, L.b + kb, inb);
          cp_async_zfill(is + ea, L.idg + ka, ina);
          cp_async_zfill(is + eb, L.idg + kb, inb);
          cp_async_zfill(cxs + ea, L.cx + ka, ina);
          cp_async_zfill(cxs + eb, L.cx + kb, inb);
          cp_async_zfill(cys + ea, L.cy + ka, ina);
          cp_async_zfill(cys + eb, L.cy + kb, inb);
          if (DG) {
            cp_async_zfill(ds + ea, L.dg + ka, ina);
            cp_async_zfill(ds + eb, L.dg + kb, inb);
          }
        }
      }
    } else {
      constexpr int WH = Wn::WH, PO = Wn::PO;
#pragma unroll
      for (int u0 = 0; u0 < N; u0 += BXT * BYT) {
        const int q = u0 + tid;
        if (u0 + BXT * BYT > N && q >= N) continue;
        const int r = q / W, c = q - r * W;
        const int e = ((c + r) & 1) * PO + r * WH + (c >> 1);
        const int gi = gi0 + c, gj = gj0 + r;
        const bool in = inner || (gi >= 0 && gi < L.nI && gj >= 0 && gj < L.nJ);
        const size_t k = base + c + (size_t)r * L.ld, kz = in ? k : 0;
        if (PROLONG) {
          T x = 0;
          if (in) x = L.x[k] + C.x[(size_t)(gi / 2 + 1) + (size_t)(gj / 2 + 1) * C.ld];
          xs[e] = x;
        } else if (LOAD_X) {
          cp_async_zfill(xs + e, L.x + kz, in);
        } else {
          xs[e] = 0;
        }
        if (inner) {
          cp_async(bs + e, L.b + k);
          cp_async(is + e, L.idg + k);
          cp_async(cxs + e, L.cx + k);
          cp_async(cys + e, L.cy + k);
          if (DG) cp_async(ds + e, L.dg + k);
        } else {
          cp_async_zfill(bs + e, L.b + kz, in);
          cp_async_zfill(is + e, L.idg + kz, in);
          cp_async_zfill(cxs + e, L.cx + kz, in);
          cp_async_zfill(cys + e, L.cy + kz, in);
          if (DG) cp_async_zfill(ds + e, L.dg + kz, in);
        }
      }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
  } else {
#pragma unroll
    for (int u0 = 0; u0 < N; u0 += BXT * BYT) {
      const int q = u0 + tid;
      if (q >= N) continue;
      const int r = q / W, c = q - r * W;
      const int gi = gi0 + c, gj = gj0 + r;
      T x = 0, b = 0, id = 0, cx = 0, cy = 0, dg = 0;
      if (inner || (gi >= 0 && gi < L.nI && gj >= 0 && gj < L.nJ)) {
        const size_t k = base + c + (size_t)r * L.ld;
        if (LOAD_X) {
          x = L.x[k];
          if (PROLONG) x += C.x[(size_t)(gi / 2 + 1) + (size_t)(gj / 2 + 1) * C.ld];
        }
        b = L.b[k];
        id = L.idg[k];
        cx = L.cx[k];
        cy = L.cy[k];
        if (DG) dg = L.dg[k];
      }
      xs[q] = x;
      bs[q] = b;
      is[q] = id;
      cxs[q] = cx;
      cys[q] = cy;
      if (DG) ds[q] = dg;
    }
  }
}

// The smoothers' arithmetic, with every rounding stated: one Gauss-Seidel update
//   x = (b + cxl xl + cxr xr + cyb xb + cyt xt) / dg   (1/dg stored),
// fused multiply-adds in that order, and the residual
//   b - (dg x - cxl xl - cxr xr - cyb xb - cyt xt).
// Written with the rounding intrinsics so that every kernel that smooths a level
// (tiled or streaming) computes each value with the same operations, whatever
// the compiler would contract.
__device__ __forceinline__ float fmad(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmad(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float mulr(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mulr(double a, double b) { return __dmul_rn(a, b); }
template <typename T>
__device__ __forceinline__ T gs_update(T b, T cxl, T xl, T cxr, T xr, T cyb, T xb, T cyt, T xt, T idg) {
  return mulr(fmad(cyt, xt, fmad(cyb, xb, fmad(cxr, xr, fmad(cxl, xl, b)))), idg);
}
template <typename T>
__device__ __forceinline__ T gs_residual(T b, T dg, T x, T cxl, T xl, T cxr, T xr, T cyb, T xb, T cyt, T xt) {
  return b - fmad(-cyt, xt, fmad(-cyb, xb, fmad(-cxr, xr, fmad(-cxl, xl, mulr(dg, x)))));
}

// Half sweep of one colour over the window shrunk by R cells per side.
//   Natural layout: the colour's RH x RW/2 cells are enumerated flat over the
//   block's threads.
//   Split layout: the threads walk the colour's plane element by element over
//   rows R .. HH-R-1, whole rows, so that a warp's accesses to each plane are
//   consecutive elements; with o = c & 1 the left and right neighbours of
//   element e are elements e - 1 + o and e + o of the other plane, the lower and
//   upper ones e - WH and e + WH.  Tile origins are even, so the colour's plane
//   is the colour itself.  The cells of those rows outside the shrunk window,
//   and the cells outside the domain, are updated too, without a test: a cell
//   outside the domain is staged with b, 1/dg and both of its faces' conductances
//   zero (as are the wall faces of the cells next to it), so it stays zero; a
//   cell in the margin (column c < R or c >= W - R) gets a value from its staged
//   neighbours (at the row ends, elements of the adjacent row) that nothing
//   exact reads: after half sweep k the cells of columns k .. W-k-1 hold the
//   exact values, since half sweep k + 1 updates columns k+1 .. W-k-2 from
//   neighbours in columns k .. W-k-1, and the tile with its one-cell ring lies
//   in columns 2 NS .. W-2NS-1.
template <typename T, int H, int R, int SH, int COLOR>
__device__ __forceinline__ void window_half(T* sm, int i0, int j0, int nI, int nJ) {
  using Wn = Win<T, H, SH>;
  constexpr int W = Wn::W, HH = Wn::HH, NA = Wn::NA;
  const int tid = threadIdx.x + threadIdx.y * BXT;
  if constexpr (Wn::SPLIT) {
    constexpr int WH = Wn::WH, PO = Wn::PO, E0 = R * WH, TOT = (HH - 2 * R) * WH;
    constexpr int p = COLOR, pq = COLOR ^ 1;
    T* xp = sm + p * PO;
    const T *xq = sm + pq * PO, *bp = sm + NA + p * PO, *ip = sm + 2 * NA + p * PO;
    const T *cxp = sm + 3 * NA + p * PO, *cxq = sm + 3 * NA + pq * PO, *cyp = sm + 4 * NA + p * PO, *cyq = sm + 4 * NA + pq * PO;
#pragma unroll
    for (int u0 = 0; u0 < TOT; u0 += BXT * BYT) {
      const int e = E0 + u0 + tid;
      if (u0 + BXT * BYT > TOT && e >= E0 + TOT) continue;
      const int o = (p + e / WH) & 1;
      xp[e] = gs_update(bp[e], cxp[e], xq[e - 1 + o], cxq[e + o], xq[e + o], cyp[e], xq[e - WH], cyq[e + WH], xq[e + WH], ip[e]);
    }
  } else {
    constexpr int RW = W - 2 * R, RH = HH - 2 * R, HALF = RW / 2, TOT = RH * HALF;
    T* xs = sm;
    const T *bs = sm + NA, *is = sm + 2 * NA, *cxs = sm + 3 * NA, *cys = sm + 4 * NA;
    const int gi0 = i0 - H, gj0 = j0 - H;
    const bool inner = gi0 + R >= 0 && gj0 + R >= 0 && gi0 + W - R <= nI && gj0 + HH - R <= nJ;
#pragma unroll
    for (int u0 = 0; u0 < TOT; u0 += BXT * BYT) {
      const int u = u0 + tid;
      if (u >= TOT) continue;
      const int rr = u / HALF, m = u - rr * HALF;
      const int r = R + rr, gj = gj0 + r;
      const int c = R + 2 * m + ((COLOR - (gi0 + R) - gj) & 1);
      if (!inner) {
        const int gi = gi0 + c;
        if (gi < 0 || gi >= nI || gj < 0 || gj >= nJ) continue;
      }
      const int s = c + r * W;
      xs[s] = gs_update(bs[s], cxs[s], xs[s - 1], cxs[s + 1], xs[s + 1], cys[s], xs[s - W], cys[s + W], xs[s + W], is[s]);
    }
  }
}

// FP32-friendly accumulation of a few products per thread (Kahan-compensated in
// the vector precision, s - c); the block reduction continues in double-float on
// the FP32 pipe, the grid reduction in FP64.
template <typename T>
struct Acc {
  T s = 0, c = 0;
  __device__ __forceinline__ void add(T v) {
    T y = v - c;
    T t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double block_total() const { return block_sum_df(DF{s, -c}); }
};
template <>
struct Acc<double> {  // FP64 vectors: plain accumulation (FP64 issue slots are scarce)
  double s = 0;
  __device__ __forceinline__ void add(double v) { s += v; }
  __device__ __forceinline__ double block_total() const { return block_sum(s); }
};

// Last-block finalisation of a reduction: every block stores its partial (acc
// already summed over the block), the block that arrives last sums them in a
// fixed order.  Returns true in that block (every thread), with *total set.
__device__ __forceinline__ bool last_block_total(double acc, double* part, unsigned nblocks, unsigned* counter, double* total) {
  __shared__ bool last;
  unsigned bid = block_linear();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    part[bid] = acc;
    __threadfence();
    last = atomicAdd(counter, 1u) == nblocks - 1;
  }
  __syncthreads();
  if (!last) return false;
  *total = sum_partials(part, nblocks);
  if (threadIdx.x == 0 && threadIdx.y == 0) *counter = 0u;
  return true;
}
template <typename T>
__device__ __forceinline__ bool last_block_sum(const Acc<T>& acc, double* part, unsigned nblocks, unsigned* counter, double* total) {
  return last_block_total(acc.block_total(), part, nblocks, counter, total);
}

// z = M r is complete: record r.z and beta = rz_new / rz_cur (Fletcher-Reeves).
// With the FP32 preconditioner, a flexible (Polak-Ribiere) beta and a deflation of
// the pinned operator's near-null constant mode were tried: neither lowered the
// iteration count, and both cost extra traffic per iteration.
__device__ __forceinline__ void publish_rz(Scalars* sc, double rz) {
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    sc->rz_new = rz;
    sc->beta = rz / sc->rz_cur;
  }
}


// Half sweeps R = R0..R1 (window shrunk by R), colour of the first = C0,
// alternating, with a block barrier after each.
template <typename T, int H, int R, int R1, int C0, int SH>
__device__ __forceinline__ void window_halves(T* sm, int i0, int j0, int nI, int nJ) {
  if constexpr (R <= R1) {
    window_half<T, H, R, SH, (C0 + R - 1) & 1>(sm, i0, j0, nI, nJ);
    __syncthreads();
    window_halves<T, H, R + 1, R1, C0, SH>(sm, i0, j0, nI, nJ);
  }
}

template <typename T, int NS, int SH>
constexpr size_t pre_smem() {
  return sweep_smem<T, 2 * NS + 1, false, SH>();
}

// The diagonal from its staged reciprocal (the residual after pre-smoothing;
// keeps dg out of shared memory).
__device__ __forceinline__ float diag_of(float idg) { return __frcp_rn(idg); }
__device__ __forceinline__ double diag_of(double idg) { return __drcp_rn(idg); }
template <typename T, int NS, int SH>
constexpr size_t post_smem() {
  return sweep_smem<T, 2 * NS, false, SH>();
}

// Pre-smoothing: NS red-black sweeps (red first) from x = 0, then the residual
// of the red cells (the black ones are zero after the last black half sweep)
// averaged into the coarse right-hand side, with the diagonal recovered from
// 1/dg.  x is written to xout.
template <typename T, int NS, int SH>
__global__ void __launch_bounds__(BXT* BYT) k_pre_smooth(Level<T> L, Level<T> C, T* __restrict__ xout, const int* __restrict__ done) {
  pdl_enter();
  if (*done) return;
  constexpr int H = 2 * NS + 1;
  using Wn = Win<T, H, SH>;
  using Ts = TileShape<SH>;
  constexpr int NA = Wn::NA;
  extern __shared__ unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  const int i0 = blockIdx.x * Ts::X, j0 = blockIdx.y * Ts::Y;
  stage_window<T, H, false, false, false, SH>(L, C, sm, i0, j0);
  __syncthreads();
  window_halves<T, H, 1, 2 * NS, 0, SH>(sm, i0, j0, L.nI, L.nJ);
  const T *xs = sm, *bs = sm + NA, *is = sm + 2 * NA, *cxs = sm + 3 * NA, *cys = sm + 4 * NA;
  const int tid = threadIdx.x + threadIdx.y * BXT;
#pragma unroll
  for (int q0 = 0; q0 < Ts::QX * Ts::QY; q0 += BXT * BYT) {
    const int q = q0 + tid;
    if (q >= Ts::QX * Ts::QY) continue;
    const int qx = q % Ts::QX, qy = q / Ts::QX;
    T acc = 0;
#pragma unroll
    for (int dr = 0; dr < 2; ++dr)
#pragma unroll
      for (int dc = 0; dc < 2; ++dc) {
        const int ti = 2 * qx + dc, tj = 2 * qy + dr;
        const int gi = i0 + ti, gj = j0 + tj;
        if (gi >= L.nI || gj >= L.nJ) continue;
        const CellOff w = cell_off<T, H, SH>(ti + H, tj + H);
        xout[(size_t)(gi + 1) + (size_t)(gj + 1) * L.ld] = xs[w.s];
        if (!((gi + gj) & 1)) {  // red cells: black residuals are zero after the black half sweep
          acc += gs_residual(bs[w.s], diag_of(is[w.s]), xs[w.s], cxs[w.s], xs[w.l], cxs[w.r], xs[w.r], cys[w.s], xs[w.b], cys[w.t],
                             xs[w.t]);
        }
      }
    const int I = i0 / 2 + qx, J = j0 / 2 + qy;
    if (I < C.nI && J < C.nJ) C.b[(size_t)(I + 1) + (size_t)(J + 1) * C.ld] = (T)0.25 * acc;
  }
}

// Post-smoothing: x (from L.x) plus the prolonged coarse correction, then NS
// black-red sweeps (black first); x to xout.  With part_rz (finest level) r.z
// (b = r, x = z there) is reduced and beta published.
template <typename T, int NS, int SH>
__global__ void __launch_bounds__(BXT* BYT) k_post_smooth(Level<T> L, Level<T> C, T* __restrict__ xout, double* __restrict__ part_rz,
                                                         unsigned* __restrict__ counter, Scalars* sc, const int* __restrict__ done) {
  pdl_enter();
  if (*done) return;
  constexpr int H = 2 * NS;
  using Wn = Win<T, H, SH>;
  using Ts = TileShape<SH>;
  constexpr int NA = Wn::NA;
  extern __shared__ unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  const int i0 = blockIdx.x * Ts::X, j0 = blockIdx.y * Ts::Y;
  stage_window<T, H, true, true, false, SH>(L, C, sm, i0, j0);
  __syncthreads();
  window_halves<T, H, 1, 2 * NS, 1, SH>(sm, i0, j0, L.nI, L.nJ);
  const T *xs = sm, *bs = sm + NA;
  Acc<T> acc;
  const int tid = threadIdx.x + threadIdx.y * BXT;
#pragma unroll
  for (int q0 = 0; q0 < Ts::QX * Ts::QY; q0 += BXT * BYT) {
    const int q = q0 + tid;
    if (q >= Ts::QX * Ts::QY) continue;
    const int qx = q % Ts::QX, qy = q / Ts::QX;
#pragma unroll
    for (int dr = 0; dr < 2; ++dr)
#pragma unroll
      for (int dc = 0; dc < 2; ++dc) {
        const int ti = 2 * qx + dc, tj = 2 * qy + dr;
        const int gi = i0 + ti, gj = j0 + tj;
        if (gi >= L.nI || gj >= L.nJ) continue;
        const int e = cell_off<T, H, SH>(ti + H, tj + H).s;
        xout[(size_t)(gi + 1) + (size_t)(gj + 1) * L.ld] = xs[e];
        if (part_rz) acc.add(bs[e] * xs[e]);
      }
  }
  if (part_rz) {
    double rz;
    if (last_block_sum(acc, part_rz, gridDim.x * gridDim.y, counter, &rz)) publish_rz(sc, rz);
  }
}

#include "gb2d_stream.cuh"

// ---- single-CTA tail: the coarse levels, coefficients resident in shared memory ---

template <typename T>
struct TailArgs {
  int nlev;
  Level<T> L[kMaxLevels];
  int off[kMaxLevels];  // shared-memory offset (elements) of level l's arrays
  Scalars* sc;          // when the tail starts at the finest level: publish r.z / beta
};

// Per tail level, six padded arrays: x, b, cx, cy, 1/dg, dg.
template <typename T>
struct TailLevel {
  T *x, *b, *cx, *cy, *idg, *dg;
};

template <typename T>
__device__ __forceinline__ TailLevel<T> tail_level(T* sm, int off, const Level<T>& L) {
  int n = (L.nI + 2) * (L.nJ + 2);
  T* p = sm + off;
  return TailLevel<T>{p, p + n, p + 2 * n, p + 3 * n, p + 4 * n, p + 5 * n};
}

template <typename T>
__device__ __forceinline__ void tail_half(const Level<T>& L, const TailLevel<T>& t, int color) {
  int hw = (L.nI + 1) / 2;
  for (int u = threadIdx.x; u < hw * L.nJ; u += blockDim.x) {
    int j = u / hw;
    int i = 2 * (u % hw) + ((j + color) & 1);
    if (i >= L.nI) continue;
    int k = (i + 1) + (j + 1) * L.ld;
    t.x[k] = (t.b[k] + t.cx[k] * t.x[k - 1] + t.cx[k + 1] * t.x[k + 1] + t.cy[k] * t.x[k - L.ld] + t.cy[k + L.ld] * t.x[k + L.ld]) * t.idg[k];
  }
}

template <typename T>
__global__ void __launch_bounds__(kTailThreads) k_tail(TailArgs<T> a, const double* __restrict__ ainv, int nu, const int* __restrict__ done) {
  pdl_enter();
  if (*done) return;
  extern __shared__ unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  const int nl = a.nlev;
  // Stage every level's coefficients (padded arrays, so the zero ring comes along),
  // the top level's right-hand side, and zero x / b below.
  for (int l = 0; l < nl; ++l) {
    const Level<T>& L = a.L[l];
    TailLevel<T> t = tail_level(sm, a.off[l], L);
    int n = (L.nI + 2) * (L.nJ + 2);
    for (int u = threadIdx.x; u < n; u += blockDim.x) {
      t.x[u] = (T)0;
      t.b[u] = l == 0 ? L.b[u] : (T)0;
      t.cx[u] = L.cx[u];
      t.cy[u] = L.cy[u];
      t.idg[u] = L.idg[u];
      t.dg[u] = L.dg[u];
    }
  }
  __syncthreads();
  for (int l = 0; l < nl - 1; ++l) {
    const Level<T>& L = a.L[l];
    TailLevel<T> t = tail_level(sm, a.off[l], L);
    for (int s = 0; s < nu; ++s) {
      tail_half(L, t, 0);
      __syncthreads();
      tail_half(L, t, 1);
      __syncthreads();
    }
    const Level<T>& C = a.L[l + 1];
    TailLevel<T> tc = tail_level(sm, a.off[l + 1], C);
    for (int u = threadIdx.x; u < C.nI * C.nJ; u += blockDim.x) {
      int I = u % C.nI, J = u / C.nI;
      T acc = 0;
      for (int bb = 0; bb < 2; ++bb) {  // red cells only: black residuals are zero after the black half sweep
        int j = 2 * J + bb, i = 2 * I + (j & 1);
        if (i >= L.nI || j >= L.nJ) continue;
        int k = (i + 1) + (j + 1) * L.ld;
        T ax = t.dg[k] * t.x[k] - t.cx[k] * t.x[k - 1] - t.cx[k + 1] * t.x[k + 1] - t.cy[k] * t.x[k - L.ld] - t.cy[k + L.ld] * t.x[k + L.ld];
        acc += t.b[k] - ax;
      }
      tc.b[(I + 1) + (J + 1) * C.ld] = (T)0.25 * acc;
    }
    __syncthreads();
  }
  {
    const Level<T>& C = a.L[nl - 1];
    TailLevel<T> t = tail_level(sm, a.off[nl - 1], C);
    int n = C.nI * C.nJ;
    if ((int)threadIdx.x < n) {
      double acc = 0.0;
      for (int m = 0; m < n; ++m) acc += ainv[(size_t)threadIdx.x * n + m] * (double)t.b[(m % C.nI + 1) + (m / C.nI + 1) * C.ld];
      t.x[(threadIdx.x % C.nI + 1) + (threadIdx.x / C.nI + 1) * C.ld] = (T)acc;
    }
    __syncthreads();
  }
  for (int l = nl - 2; l >= 0; --l) {
    const Level<T>& L = a.L[l];
    const Level<T>& C = a.L[l + 1];
    TailLevel<T> t = tail_level(sm, a.off[l], L);
    const T* xc = tail_level(sm, a.off[l + 1], C).x;
    for (int u = threadIdx.x; u < L.nI * L.nJ; u += blockDim.x) {
      int i = u % L.nI, j = u / L.nI;
      t.x[(i + 1) + (j + 1) * L.ld] += xc[(i / 2 + 1) + (j / 2 + 1) * C.ld];
    }
    __syncthreads();
    for (int s = 0; s < nu; ++s) {
      tail_half(L, t, 1);
      __syncthreads();
      tail_half(L, t, 0);
      __syncthreads();
    }
  }
  {
    const Level<T>& L = a.L[0];
    TailLevel<T> t = tail_level(sm, a.off[0], L);
    double acc = 0.0;
    for (int u = threadIdx.x; u < L.nI * L.nJ; u += blockDim.x) {
      int k = (u % L.nI + 1) + (u / L.nI + 1) * L.ld;
      L.x[k] = t.x[k];
      if (a.sc) acc += (double)t.b[k] * (double)t.x[k];
    }
    if (a.sc) {
      acc = block_sum(acc);
      publish_rz(a.sc, acc);
    }
  }
}

#include "gb2d_ctail.cuh"

// ---- CG kernels ------------------------------------------------------------------
//
// The CG itself is FP64 for both precisions: x, r, p and Ap are FP64 and A is
// applied with the reference's matrix entries (standard 5-point form).  Only
// the preconditioner's precision differs: an FP64 or an FP32 V-cycle (or Jacobi)
// maps r to z.  An FP32 preconditioner is only an approximate inverse anyway;
// keeping the Krylov recurrences in FP64 keeps the FP64 iteration count, where
// refinement around an FP32 CG stalls at the FP32 operator's accuracy.
// FP64 issue slots are scarce on this part (about 2 FP64 operations per clock
// per SM), so each kernel does at most a handful per cell; FP32 <-> FP64 moves
// are bit manipulations on the integer pipes.

// The CG kernels below run flat over the padded rows 1..nJ, ghost columns
// included: every vector here is zero on the padding ring and so are the
// padded coefficients (wall conductances are zero), so ghost entries stay zero
// and no per-cell index arithmetic is needed.
#define GB_FLAT_FOR(L, k)                                                                                      \
  for (size_t k = (size_t)(L).ld + blockIdx.x * (size_t)blockDim.x + threadIdx.x, k##_end = (size_t)(L).ld * ((L).nJ + 1); \
       k < k##_end; k += (size_t)gridDim.x * blockDim.x)

// r = b - A x with the reference's matrix entries, in FP64; its copy for the
// preconditioner (rT, FP32 or the FP64 r itself); partial ||r||^2 and ||b||^2.
template <typename T>
__global__ void k_residual64(Level<double> L, const double* __restrict__ x, const double* __restrict__ b, double* __restrict__ r64,
                             T* __restrict__ rT, double* __restrict__ part_rr, double* __restrict__ part_bb) {
  double rr = 0.0, bb = 0.0;
  GB_FLAT_FOR(L, k) {
    double ax = L.dg[k] * x[k] - L.cx[k] * x[k - 1] - L.cx[k + 1] * x[k + 1] - L.cy[k] * x[k - L.ld] - L.cy[k + L.ld] * x[k + L.ld];
    double r = b[k] - ax;
    r64[k] = r;
    if constexpr (sizeof(T) == 4) rT[k] = narrow(r);
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

// Pairs of neighbouring elements of the padded rows 1..nJ, 16-byte aligned:
// the pair loop starts at the even index at or below ld and ends at the even
// index at or above ld (nJ + 1); the extra elements are ghosts (zero).
#define GB_FLAT_PAIRS(L, k)                                                                                   \
  for (size_t k = ((size_t)(L).ld & ~(size_t)1) + 2 * (blockIdx.x * (size_t)blockDim.x + threadIdx.x),        \
              k##_end = ((size_t)(L).ld * ((L).nJ + 1) + 1) & ~(size_t)1;                                    \
       k < k##_end; k += 2 * (size_t)gridDim.x * blockDim.x)

template <typename T>
struct Pair;
template <>
struct Pair<float> {
  using V = float2;
};
template <>
struct Pair<double> {
  using V = double2;
};
template <typename T>
__device__ __forceinline__ typename Pair<T>::V ld2(const T* a, size_t k) {
  return *reinterpret_cast<const typename Pair<T>::V*>(a + k);
}
template <typename T>
__device__ __forceinline__ void st2(T* a, size_t k, T v0, T v1) {
  typename Pair<T>::V v;
  v.x = v0;
  v.y = v1;
  *reinterpret_cast<typename Pair<T>::V*>(a + k) = v;
}

// p = z + beta p (p = z when first).  z is the preconditioner's output in its
// precision; one FP64 operation per cell.
template <typename TZ>
__global__ void k_direction(Level<double> L, const TZ* __restrict__ z, double* __restrict__ p, const Scalars* sc, int first,
                            const int* __restrict__ done) {
  pdl_enter();
  if (*done) return;
  const double bt = first ? 0.0 : sc->beta;
  GB_FLAT_PAIRS(L, k) {
    const auto zv = ld2(z, k);
    if (first) {
      st2(p, k, widen(zv.x), widen(zv.y));
    } else {
      const double2 pv = ld2(p, k);
      st2(p, k, widen(zv.x) + bt * pv.x, widen(zv.y) + bt * pv.y);
    }
  }
}

// Ap = A p (reference entries) and p.Ap; the last block publishes
// alpha = rz_new / p.Ap and rz_cur = rz_new.  With an even row length two
// neighbouring cells per thread (16-byte loads), else one.  With the FP32
// preconditioner (TZ = float, whose r.z and ||r||^2 are FP32 sums already) each
// thread's FP64 partial is split into two FP32 words (one FP64 subtraction) and
// the block sum runs in double-float on the FP32 pipe; with the FP64 one the
// block sum stays FP64.
template <typename TZ>
__global__ void k_apply_pap(Level<double> L, const double* __restrict__ p, double* __restrict__ ap, Scalars* sc, double* __restrict__ part,
                            unsigned* __restrict__ counter, const int* __restrict__ done) {
  pdl_enter();
  if (*done) return;
  double acc = 0.0;
  const size_t ld = L.ld;
  if ((ld & 1) == 0) {
    GB_FLAT_PAIRS(L, k) {
      const double2 pc = ld2(p, k), pb = ld2(p, k - ld), pt = ld2(p, k + ld);
      const double2 dg = ld2(L.dg, k), cx = ld2(L.cx, k), cy = ld2(L.cy, k), cyt = ld2(L.cy, k + ld);
      const double pl = p[k - 1], pr = p[k + 2], cx2 = L.cx[k + 2];
      const double y0 = dg.x * pc.x - cx.x * pl - cx.y * pc.y - cy.x * pb.x - cyt.x * pt.x;
      const double y1 = dg.y * pc.y - cx.y * pc.x - cx2 * pr - cy.y * pb.y - cyt.y * pt.y;
      st2(ap, k, y0, y1);
      acc += pc.x * y0;
      acc += pc.y * y1;
    }
  } else {
    GB_FLAT_FOR(L, k) {
      const double pc = p[k];
      double y = L.dg[k] * pc - L.cx[k] * p[k - 1] - L.cx[k + 1] * p[k + 1] - L.cy[k] * p[k - L.ld] - L.cy[k + L.ld] * p[k + L.ld];
      ap[k] = y;
      acc += pc * y;
    }
  }
  double pap, blk;
  if constexpr (sizeof(TZ) == 4) {
    const float hi = narrow(acc);
    blk = block_sum_df(DF{hi, narrow(acc - widen(hi))});
  } else {
    blk = block_sum(acc);
  }
  if (last_block_total(blk, part, gridDim.x, counter, &pap) && threadIdx.x == 0) {
    double rz = sc->rz_new;
    sc->rz_cur = rz;
    sc->alpha = rz / pap;
  }
}

// x += alpha p;  r -= alpha Ap;  the preconditioner's copy of r (FP32: rT; FP64:
// r is read in place);  ||r||^2 (from the FP32 copy when there is one).  The
// last block stores ||r||^2 for the host and raises the done flag at the
// threshold (or on a non-finite value).  Two neighbouring cells per thread.
template <typename T>
__global__ void k_update(Level<double> L, double* __restrict__ x, double* __restrict__ r, const double* __restrict__ p,
                         const double* __restrict__ ap, T* __restrict__ rT, Scalars* sc, double* __restrict__ part,
                         unsigned* __restrict__ counter, int* __restrict__ done, double* __restrict__ host_rr) {
  pdl_enter();
  if (*done) return;
  const double al = sc->alpha;
  Acc<T> acc;
  GB_FLAT_PAIRS(L, k) {
    const double2 pv = ld2(p, k), av = ld2(ap, k), xv = ld2(x, k), rv = ld2(r, k);
    st2(x, k, xv.x + al * pv.x, xv.y + al * pv.y);
    const double r0 = rv.x - al * av.x, r1 = rv.y - al * av.y;
    st2(r, k, r0, r1);
    if constexpr (sizeof(T) == 4) {
      const float f0 = narrow(r0), f1 = narrow(r1);
      st2(rT, k, f0, f1);
      acc.add(f0 * f0);
      acc.add(f1 * f1);
    } else {
      acc.add(r0 * r0);
      acc.add(r1 * r1);
    }
  }
  double rr;
  if (last_block_sum(acc, part, gridDim.x, counter, &rr) && threadIdx.x == 0) {
    sc->rr = rr;
    if (!(rr > sc->thr2)) {
      *done = 1;
      if (!isfinite(rr)) sc->flag |= 1;
    }
    *host_rr = rr;
  }
}

// Jacobi preconditioner z = r / dg; the last block publishes r.z and beta.
template <typename T>
__global__ void k_jacobi(Level<T> L, const T* __restrict__ r, T* __restrict__ z, Scalars* sc, double* __restrict__ part_rz,
                         unsigned* __restrict__ counter, const int* __restrict__ done) {
  pdl_enter();
  if (*done) return;
  Acc<T> acc;
  for (size_t k = (size_t)L.ld + blockIdx.x * (size_t)blockDim.x + threadIdx.x, k_end = (size_t)L.ld * (L.nJ + 1); k < k_end;
       k += (size_t)gridDim.x * blockDim.x) {  // flat over the padded rows: r and 1/dg are zero on the ring
    T zv = r[k] * L.idg[k];
    z[k] = zv;
    acc.add(r[k] * zv);
  }
  double rz;
  if (last_block_sum(acc, part_rz, gridDim.x, counter, &rz)) publish_rz(sc, rz);
}

__global__ void k_begin_inner(Scalars* sc, int* done, double thr2) {
  *done = 0;
  sc->thr2 = thr2;
  sc->rz_cur = 1.0;
}

// Start of a device-driven CG run (the solve graph's WHILE loop): as k_begin_inner,
// with the iteration count reset and its cap.
__global__ void k_begin_loop(Scalars* sc, int* done, double thr2, int max_it) {
  *done = 0;
  sc->thr2 = thr2;
  sc->rz_cur = 1.0;
  sc->iters = 0;
  sc->max_it = max_it;
}

// Last node of the loop body: counts the iteration, hands the count and the latest
// ||r||^2 to the host, and continues the loop only while the run has not converged
// and is under its cap.  It never returns early: every pass sets the condition, so the
// loop ends after at most max_it passes (and after 1 << 20 in any case).
__global__ void k_loop_cond(cudaGraphConditionalHandle h, Scalars* sc, const int* __restrict__ done, double* host_out) {
  pdl_enter();
  const int n = ++sc->iters;
  host_out[0] = sc->rr;
  host_out[1] = (double)n;
  const bool more = *done == 0 && n < sc->max_it && n < (1 << 20);
  cudaGraphSetConditional(h, more ? 1u : 0u);
}

// Start of one pass of a solve inside a device-driven frame: the pass's threshold and
// done flag from the true residual and ||b||^2 in the frame scalars fs (g_rr, g_bb), as
// solver_solve's host loop decides them (a non-finite norm marks fs->flag bit 4 and ends
// the solve), the pass's iteration cap (what the solve's earlier passes left of max_it),
// and the WHILE node's condition.  first: the solve's first pass.
__global__ void k_begin_device(cudaGraphConditionalHandle h, Scalars* sc, int* done, Scalars* fs, double tol2, int max_it, int first) {
  const double rr = fs->g_rr, bb = fs->g_bb;
  if (first) fs->iters = 0;  // the frame scalars' iters count this solve's iterations
  const double thr2 = tol2 * bb;
  int d = 0;
  if (!isfinite(rr) || !isfinite(bb)) {
    d = 1;
    fs->flag |= 4;
  } else if (rr <= thr2 || bb == 0.0) {
    d = 1;
  }
  const int cap = max_it - fs->iters;
  if (cap <= 0) d = 1;
  *done = d;
  sc->thr2 = thr2;
  sc->rz_cur = 1.0;
  sc->iters = 0;
  sc->max_it = cap;
  cudaGraphSetConditional(h, d ? 0u : 1u);
}

// End of a pass (after the true residual is in fs->g_rr / g_bb): the pass's iterations join
// the solve's and the instance's totals, a non-finite ||r||^2 of the CG marks fs->flag.
// last: the solve's last pass, whose residual is the solve's result.
__global__ void k_end_device(const Scalars* sc, Scalars* fs, int last) {
  fs->iters += sc->iters;
  fs->g_iters += (unsigned long long)sc->iters;
  if (sc->flag & 1) fs->flag |= 4;
  if (!last) return;
  const double rr = fs->g_rr, bb = fs->g_bb;
  if (!isfinite(rr) || !isfinite(bb)) fs->flag |= 4;
  const double rel2 = bb > 0 ? rr / bb : 0.0;
  if (rel2 > fs->g_rel2_max) fs->g_rel2_max = rel2;
  if (!(rr <= sc->thr2) && bb != 0.0) fs->g_capped = 1;
}

}  // namespace

// ---- host side -------------------------------------------------------------------

template <typename T>
struct Hierarchy {
  int nlev = 0, tail = 0;  // levels [tail, nlev) run in the single-CTA tail kernel
  size_t tail_smem = 0;
  int ctail = -1;          // levels [ctail, nlev) run in the cluster tail (-1: not used)
  int ct_P = 0;            // CTAs in that cluster
  size_t ct_smem = 0;
  CtArgs<T> ct;
  Level<T> L[kMaxLevels];
  int shape[kMaxLevels] = {};  // tile shape of each tiled level's smoothing launches
  T* r = nullptr;  // the preconditioner's input (padded fine layout, = L[0].b); z = L[0].x
};

struct GraphSet {
  bool ok = false;
  cudaGraphExec_t init = nullptr, iter[2] = {nullptr, nullptr};
  unsigned long long nodes_init = 0, nodes_iter = 0;
  cudaGraphExec_t loop = nullptr;  // init + a WHILE node over one iteration: the whole CG run
  cudaGraph_t loop_graph = nullptr;  // its source (holds the conditional handle), kept while loop lives
  unsigned long long nodes_body = 0;
};

struct Solver {
  int ni, nj;
  Hierarchy<double> h64;
  Hierarchy<float> h32;
  double* ainv64 = nullptr;
  double* ainv32 = nullptr;
  double* b64 = nullptr;   // right-hand side, padded
  double *p = nullptr, *ap = nullptr;  // FP64 CG direction and A p (padded); r = h64.r
  double* part = nullptr;  // kSlots x nparts_cap block partials (see slot())
  int nparts_cap = 0;
  unsigned* counter = nullptr;  // 4 last-block counters: p.Ap, r.r, r.z (jacobi), r.z (sweep)
  double* host = nullptr;  // pinned: [0..1] per-parity r.r, [4..5] residual / rhs norms
  int* done = nullptr;
  Scalars* sc = nullptr;
  int G = 0;               // blocks of the grid-stride CG kernels
  cudaEvent_t ev[2] = {nullptr, nullptr};
  bool prebuilt = false;  // the hierarchies are building on ctx->side2 (solver_prebuild)
  bool keep = false;      // the levels of the previous solve stand (solver_keep_levels)
  // Graphs per (precision, solver, smoothing sweeps) and the x they update.
  GraphSet graphs[2][2][3];
  double* graph_x[2][2][3] = {};
  unsigned long long body_nodes = 0;  // kernels of one CG iteration in a device-driven frame's loop body
};

// Block-partial slots (nparts_cap doubles each).
constexpr int kSlotPap = 0, kSlotRr = 1, kSlotRz = 2, kSlotBb = 3, kSlots = 4;
inline double* slot(Solver* S, int k) { return S->part + (size_t)k * S->nparts_cap; }

namespace {

template <typename T>
cudaError_t alloc_level(Level<T>& L, int nI, int nJ, bool own_b) {
  L.nI = nI;
  L.nJ = nJ;
  L.ld = nI + 2;
  size_t n = (size_t)(nI + 2) * (nJ + 2);
  T** arrs[8] = {&L.cx, &L.cy, &L.dg, &L.idg, &L.sh, &L.x, &L.xa, &L.b};
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
  T* arrs[8] = {L.cx, L.cy, L.dg, L.idg, L.sh, L.x, L.xa, own_b ? L.b : nullptr};
  for (auto a : arrs)
    if (a) cudaFree(a);
}

template <typename T>
cudaError_t alloc_hierarchy(Hierarchy<T>& H, int ni, int nj) {
  size_t n = (size_t)(ni + 2) * (nj + 2);
  {
    cudaError_t e = cudaMalloc(&H.r, n * sizeof(T));
    if (e != cudaSuccess) return e;
    e = cudaMemset(H.r, 0, n * sizeof(T));
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
  // Shared memory of the tail: six padded arrays per tail level; start one level
  // lower while it does not fit.
  const size_t kSmemCap = 200 * 1024;
  while (true) {
    size_t elems = 0;
    for (int l = H.tail; l < H.nlev; ++l) elems += 6 * (size_t)(H.L[l].nI + 2) * (H.L[l].nJ + 2);
    H.tail_smem = elems * sizeof(T);
    if (H.tail_smem <= kSmemCap || H.tail == H.nlev - 1) break;
    H.tail++;
  }
  if (H.tail_smem > kSmemCap) return cudaErrorInvalidValue;
  return cudaSuccess;
}

inline int ceil_log2(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return l;
}

// Lay out the cluster tail: the finest top level whose levels fit in one CTA's
// shared memory.  Distributed levels have at least P * kCtMinRows rows; the
// coarsest level is always local.  Returns false (single-CTA tail instead) when
// no top level qualifies.
template <typename T>
bool plan_ctail(Hierarchy<T>& H, int P) {
  H.ctail = -1;
  if (P < 2 || P > kClusterMax) return false;
  const int nl = H.nlev;
  const char* env = getenv("GB2D_CTAIL_TOP_CELLS");  // tuning override of kCtMaxTopCells
  const long top_cells = env && atol(env) > 0 ? atol(env) : kCtMaxTopCells;
  const char* env_rows = getenv("GB2D_CTAIL_MIN_ROWS");  // tuning override of kCtMinRows
  const int min_rows = env_rows && atoi(env_rows) > 0 ? atoi(env_rows) : kCtMinRows;
  for (int top = 0; top < nl - 1; ++top) {
    if (nl - top > kCtMaxLevels) continue;
    if ((long)H.L[top].nI * H.L[top].nJ > top_cells) continue;
    int lb = top - 1;
    while (lb + 1 < nl - 1 && H.L[lb + 1].nJ >= P * min_rows) ++lb;
    if (lb < top || H.L[lb].nJ > kCtOwnerRows) continue;
    CtArgs<T> a;
    memset(&a, 0, sizeof a);
    a.nlev = nl - top;
    a.ndist = lb - top + 1;
    for (int c = 0; c <= P; ++c) a.J0[a.ndist - 1][c] = (short)((long)c * H.L[lb].nJ / P);
    for (int l = a.ndist - 2; l >= 0; --l) {
      for (int c = 0; c < P; ++c) a.J0[l][c] = (short)(2 * a.J0[l + 1][c]);
      a.J0[l][P] = (short)H.L[top + l].nJ;
    }
    size_t off = 0;
    bool ok = true;
    for (int l = 0; l < a.nlev; ++l) {
      const Level<T>& L = H.L[top + l];
      CtLevel<T>& C = a.L[l];
      C.nI = L.nI;
      C.nJ = L.nJ;
      C.ld = L.ld;
      int rc = L.nJ;
      if (l < a.ndist) {
        rc = 0;
        for (int c = 0; c < P; ++c) {
          int r = a.J0[l][c + 1] - a.J0[l][c];
          if (r < 1) ok = false;
          rc = r > rc ? r : rc;
        }
      }
      C.rows_cap = rc;
      C.off = (int)off;
      off += 6 * (size_t)(rc + 2) * L.ld;
      int hw = (L.nI + 1) / 2;
      C.half_log2 = ceil_log2(hw < kCtThreads ? hw : kCtThreads);
      C.full_log2 = ceil_log2(L.nI < kCtThreads ? L.nI : kCtThreads);
      C.cx = L.cx;
      C.cy = L.cy;
      C.idg = L.idg;
      C.dg = L.dg;
      C.b = L.b;
      C.x = L.x;
    }
    if (!ok) continue;
    a.res_off = (int)off;
    off += (size_t)(a.L[a.ndist - 1].rows_cap + 2) * a.L[a.ndist - 1].ld;
    a.ainv_off = (int)off;
    const int nc = H.L[nl - 1].nI * H.L[nl - 1].nJ;
    off += (size_t)nc * nc;
    a.bc_off = (int)off;
    off += (size_t)nc;
    const size_t bytes = off * sizeof(T);
    if (bytes > kCtSmemCap) continue;
    H.ctail = top;
    H.ct = a;
    H.ct_P = P;
    H.ct_smem = bytes;
    return true;
  }
  return false;
}

// Cluster size the part can co-schedule for the cluster tail (16, else 8), or 0.
// GB2D_CLUSTER_TAIL=0 in the environment selects the single-CTA tail instead;
// GB2D_CLUSTER_CTAS=P (2-16) asks for P CTAs, for tuning.
int ctail_cluster_size() {
  const char* env = getenv("GB2D_CLUSTER_TAIL");
  if (env && env[0] == '0') return 0;
  static int cached = -1;
  if (cached >= 0) return cached;
  cached = 0;
  bool attr_ok = cudaFuncSetAttribute(k_ctail<float>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
                 cudaFuncSetAttribute(k_ctail<double>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
                 cudaFuncSetAttribute(k_ctail<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCtSmemCap) == cudaSuccess &&
                 cudaFuncSetAttribute(k_ctail<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCtSmemCap) == cudaSuccess;
  if (!attr_ok) {
    cudaGetLastError();
    return cached;
  }
  const char* pe = getenv("GB2D_CLUSTER_CTAS");
  const int want = pe ? atoi(pe) : 0;
  const int sizes[2] = {want >= 2 && want <= kClusterMax ? want : 16, want >= 2 && want <= kClusterMax ? want : 8};
  for (int P : sizes) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = P;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(P);
    cfg.blockDim = dim3(kCtThreads);
    cfg.dynamicSmemBytes = kCtSmemCap;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n32 = 0, n64 = 0;
    bool ok = cudaOccupancyMaxActiveClusters(&n32, k_ctail<float>, &cfg) == cudaSuccess &&
              cudaOccupancyMaxActiveClusters(&n64, k_ctail<double>, &cfg) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      continue;
    }
    if (n32 >= 1 && n64 >= 1) {
      cached = P;
      break;
    }
  }
  return cached;
}

template <typename T>
void launch_ctail(cudaStream_t s, const Hierarchy<T>& H, const double* ainv, int nu, const int* done, Scalars* sc) {
  CtArgs<T> a = H.ct;
  a.sc = H.ctail == 0 ? sc : nullptr;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = H.ct_P;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.gridDim = dim3(H.ct_P);
  cfg.blockDim = dim3(kCtThreads);
  cfg.dynamicSmemBytes = H.ct_smem;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 2;
  cudaLaunchKernelEx(&cfg, k_ctail<T>, a, ainv, nu, done);
}

template <typename T>
void free_hierarchy(Hierarchy<T>& H) {
  for (int l = 0; l < H.nlev; ++l) free_level(H.L[l], l > 0);
  if (H.r) cudaFree(H.r);
}

inline unsigned nblocks(size_t n, unsigned cap) {
  size_t b = (n + kThreads - 1) / kThreads;
  if (b < 1) b = 1;
  return (unsigned)(b < cap ? b : cap);
}

inline dim3 tiles(int nI, int nJ, int sh) {
  const int X = sh == 0 ? TileShape<0>::X : sh == 1 ? TileShape<1>::X : sh == 2 ? TileShape<2>::X : TileShape<3>::X;
  const int Y = sh == 0 ? TileShape<0>::Y : sh == 1 ? TileShape<1>::Y : sh == 2 ? TileShape<2>::Y : TileShape<3>::Y;
  return dim3((nI + X - 1) / X, (nJ + Y - 1) / Y);
}

template <typename T>
void build_coarse(cudaStream_t s, Hierarchy<T>& H, double* ainv) {
  for (int l = 1; l < H.nlev; ++l) {
    k_coarsen<T><<<grid_ij(H.L[l].nI, H.L[l].nJ), kThreads, 0, s>>>(H.L[l - 1], H.L[l]);
    GB_LAUNCHED(1);
  }
  k_dense_inverse<T><<<1, 1024, 0, s>>>(H.L[H.nlev - 1], ainv);
  GB_LAUNCHED(1);
}

template <typename T>
void build_hierarchy(cudaStream_t s, Hierarchy<T>& H, const gb2d_ctx* c, double* b64, double* ainv) {
  double idx2 = 1.0 / (c->base.dx * c->base.dx), idy2 = 1.0 / (c->base.dy * c->base.dy);
  Level<T>& L0 = H.L[0];
  k_build_level0<T><<<grid_ij(L0.nI, L0.nJ), kThreads, 0, s>>>(c->bx, c->by, c->diag, c->rhs, c->sys_shift, L0, b64, idx2, idy2);
  GB_LAUNCHED(1);
  build_coarse<T>(s, H, ainv);
}

// Only the finest FP64 level (the refinement residual's operator) and b.
void build_level0_f64(cudaStream_t s, Hierarchy<double>& H, const gb2d_ctx* c, double* b64) {
  double idx2 = 1.0 / (c->base.dx * c->base.dx), idy2 = 1.0 / (c->base.dy * c->base.dy);
  Level<double>& L0 = H.L[0];
  k_build_level0<double><<<grid_ij(L0.nI, L0.nJ), kThreads, 0, s>>>(c->bx, c->by, c->diag, c->rhs, c->sys_shift, L0, b64, idx2,
                                                                     idy2);
  GB_LAUNCHED(1);
}

// Algorithmic bytes of one tiled smoothing launch on a level (every array read
// or written once): pre-smoothing reads b, 1/dg, cx, cy, writes x and the
// coarse b (5.25 arrays); post-smoothing reads x, b, 1/dg, cx, cy and the coarse
// x, writes x (6.25 arrays).
template <typename T>
double smooth_bytes(const Level<T>& L, bool pre) {
  return sizeof(T) * (double)L.nI * L.nJ * (pre ? 5.25 : 6.25);
}

// Launch with programmatic stream serialization (see pdl_enter).
template <typename... P, typename... A>
void pdl_launch(cudaStream_t s, dim3 grid, dim3 block, size_t smem, void (*k)(P...), A&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k, std::forward<A>(args)...);
}

template <typename T, int NS, int SH>
void launch_pre_sh(cudaStream_t s, const Level<T>& L, const Level<T>& C, T* xo, const int* done) {
  pdl_launch(s, tiles(L.nI, L.nJ, SH), dim3(BXT, BYT), pre_smem<T, NS, SH>(), k_pre_smooth<T, NS, SH>, L, C, xo, done);
}
template <typename T, int NS, int SH>
void launch_post_sh(cudaStream_t s, const Level<T>& L, const Level<T>& C, T* xo, double* prz, Solver* S) {
  pdl_launch(s, tiles(L.nI, L.nJ, SH), dim3(BXT, BYT), post_smem<T, NS, SH>(), k_post_smooth<T, NS, SH>, L, C, xo, prz, S->counter + 3,
             S->sc, (const int*)S->done);
}
template <typename T, int NS>
void launch_pre(cudaStream_t s, int sh, const Level<T>& L, const Level<T>& C, T* xo, const int* done) {
  if (sh == 0)
    launch_pre_sh<T, NS, 0>(s, L, C, xo, done);
  else if (sh == 1)
    launch_pre_sh<T, NS, 1>(s, L, C, xo, done);
  else if (sh == 2)
    launch_pre_sh<T, NS, 2>(s, L, C, xo, done);
  else
    launch_pre_sh<T, NS, 3>(s, L, C, xo, done);
}
template <typename T, int NS>
void launch_post(cudaStream_t s, int sh, const Level<T>& L, const Level<T>& C, T* xo, double* prz, Solver* S) {
  if (sh == 0)
    launch_post_sh<T, NS, 0>(s, L, C, xo, prz, S);
  else if (sh == 1)
    launch_post_sh<T, NS, 1>(s, L, C, xo, prz, S);
  else if (sh == 2)
    launch_post_sh<T, NS, 2>(s, L, C, xo, prz, S);
  else
    launch_post_sh<T, NS, 3>(s, L, C, xo, prz, S);
}

// ---- streaming smoother launches (gb2d_stream.cuh) ----

// Whether the levels above the tail use the streaming smoother (GB2D_SMOOTHER=stream)
// or the tiled one (the default; GB2D_SMOOTHER=tiled).  The test that the two give
// bit-identical V-cycles runs both.
inline bool stream_smoother() {
  static const bool on = [] {
    const char* e = getenv("GB2D_SMOOTHER");
    return e && strcmp(e, "stream") == 0;
  }();
  return on;
}

// Rows per segment: an even S that gives the launch about `target` blocks (one per
// strip and segment), at least 16 rows (below that the vertical halo would exceed
// the work) and at most 256.  A block takes S + 2 EXTRA steps.
struct StreamPlan {
  int S, nsteps, blocks;
};
inline StreamPlan stream_plan(int nI, int nJ, int ns, bool post) {
  static const int target = [] {
    const char* e = getenv("GB2D_STREAM_TARGET_BLOCKS");
    return e && atoi(e) > 0 ? atoi(e) : 3 * 152;
  }();
  const int out = post ? st::W - 4 * ns : st::W - 2 - 4 * ns;
  const int extra = post ? 4 * ns : 4 * ns + 2;
  const int nstrips = post ? (nI + 1 + out - 1) / out : (nI + out - 1) / out;
  const int segs = (target + nstrips - 1) / nstrips;
  int S = (nJ + segs - 1) / segs;
  S += S & 1;
  S = S < 16 ? 16 : S > 256 ? 256 : S;
  StreamPlan p;
  p.S = S;
  p.nsteps = S + 2 * extra;
  p.blocks = nstrips * ((nJ + S - 1) / S);
  return p;
}

template <typename T, int NS, bool POST>
void launch_stream_ns(cudaStream_t s, const Level<T>& L, const Level<T>& C, T* xo, double* prz, Solver* S) {
  const StreamPlan p = stream_plan(L.nI, L.nJ, NS, POST);
  const dim3 grid(p.blocks), block(32 * st::Geo<NS, POST>::WARPS);
  const size_t smem = st::smem_bytes<T, NS, POST>();
  if (L.ld % 2 == 0)
    pdl_launch(s, grid, block, smem, k_stream<T, NS, POST, true>, L, C, xo, p.S, p.nsteps, prz, S->counter + 3, S->sc,
               (const int*)S->done);
  else
    pdl_launch(s, grid, block, smem, k_stream<T, NS, POST, false>, L, C, xo, p.S, p.nsteps, prz, S->counter + 3, S->sc,
               (const int*)S->done);
}
template <typename T, bool POST>
void launch_stream(cudaStream_t s, int nu, const Level<T>& L, const Level<T>& C, T* xo, double* prz, Solver* S) {
  if (nu == 1)
    launch_stream_ns<T, 1, POST>(s, L, C, xo, prz, S);
  else if (nu == 2)
    launch_stream_ns<T, 2, POST>(s, L, C, xo, prz, S);
  else
    launch_stream_ns<T, 3, POST>(s, L, C, xo, prz, S);
}

template <typename T, int NS>
cudaError_t set_stream_smem_ns() {
  const auto a = cudaFuncAttributeMaxDynamicSharedMemorySize;
  cudaError_t e = cudaFuncSetAttribute(k_stream<T, NS, false, true>, a, (int)st::smem_bytes<T, NS, false>());
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_stream<T, NS, false, false>, a, (int)st::smem_bytes<T, NS, false>());
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_stream<T, NS, true, true>, a, (int)st::smem_bytes<T, NS, true>());
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_stream<T, NS, true, false>, a, (int)st::smem_bytes<T, NS, true>());
  return e;
}
template <typename T>
cudaError_t set_stream_smem() {
  cudaError_t e = set_stream_smem_ns<T, 1>();
  if (e == cudaSuccess) e = set_stream_smem_ns<T, 2>();
  if (e == cudaSuccess) e = set_stream_smem_ns<T, 3>();
  return e;
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

// z = M r: the fine level's x/b are z/r.  The last finest-level post-sweep (or the
// tail, when it starts at the finest level) publishes r.z and beta.
template <typename T>
void vcycle(cudaStream_t s, Solver* S, Hierarchy<T>& H, const double* ainv, int nu, Probe* pr) {
  const bool cluster = H.ctail >= 0;
  const int tail = cluster ? H.ctail : H.tail;
  const int* done = S->done;
  double* P_rz = slot(S, kSlotRz);
  // Pre-smoothing writes L.xa, post-smoothing reads it and writes L.x (the
  // buffer the next finer level prolongs from, and z on the finest level).
  for (int l = 0; l < tail; ++l) {
    Level<T>& L = H.L[l];
    const int sh = H.shape[l];
    bool on = l == 0 && probe_begin(pr, s);
    if (stream_smoother())
      launch_stream<T, false>(s, nu, L, H.L[l + 1], L.xa, nullptr, S);
    else if (nu == 1)
      launch_pre<T, 1>(s, sh, L, H.L[l + 1], L.xa, done);
    else if (nu == 2)
      launch_pre<T, 2>(s, sh, L, H.L[l + 1], L.xa, done);
    else
      launch_pre<T, 3>(s, sh, L, H.L[l + 1], L.xa, done);
    GB_LAUNCHED(1);
    probe_end(pr, s, on, smooth_bytes(L, true));
  }
  if (cluster) {
    launch_ctail<T>(s, H, ainv, nu, done, S->sc);
  } else {
    TailArgs<T> ta;
    memset(&ta, 0, sizeof ta);
    ta.nlev = H.nlev - tail;
    int off = 0;
    for (int l = 0; l < ta.nlev; ++l) {
      ta.L[l] = H.L[tail + l];
      ta.off[l] = off;
      off += 6 * (ta.L[l].nI + 2) * (ta.L[l].nJ + 2);
    }
    ta.sc = tail == 0 ? S->sc : nullptr;
    pdl_launch(s, dim3(1), dim3(kTailThreads), H.tail_smem, k_tail<T>, ta, ainv, nu, done);
  }
  GB_LAUNCHED(1);
  for (int l = tail - 1; l >= 0; --l) {
    Level<T>& L = H.L[l];
    const int sh = H.shape[l];
    Level<T> Lin = L;
    Lin.x = L.xa;
    double* prz = l == 0 ? P_rz : nullptr;
    bool on = l == 0 && probe_begin(pr, s);
    if (stream_smoother())
      launch_stream<T, true>(s, nu, Lin, H.L[l + 1], L.x, prz, S);
    else if (nu == 1)
      launch_post<T, 1>(s, sh, Lin, H.L[l + 1], L.x, prz, S);
    else if (nu == 2)
      launch_post<T, 2>(s, sh, Lin, H.L[l + 1], L.x, prz, S);
    else
      launch_post<T, 3>(s, sh, Lin, H.L[l + 1], L.x, prz, S);
    GB_LAUNCHED(1);
    probe_end(pr, s, on, smooth_bytes(L, false));
  }
}

// z = M r with the preconditioner hierarchy H (FP64 or FP32): V-cycle or Jacobi.
template <typename T>
void precondition(cudaStream_t s, Solver* S, Hierarchy<T>& H, const double* ainv, int use_mg, int nu, Probe* pr) {
  if (use_mg) {
    vcycle<T>(s, S, H, ainv, nu, pr);
  } else {
    pdl_launch(s, dim3(S->G), dim3(kThreads), 0, k_jacobi<T>, H.L[0], (const T*)H.r, H.L[0].x, S->sc, slot(S, kSlotRz), S->counter + 2,
               (const int*)S->done);
    GB_LAUNCHED(1);
  }
}

// First direction: z = M r, p = z, Ap, alpha.
template <typename T>
void enqueue_init(cudaStream_t s, Solver* S, Hierarchy<T>& H, const double* ainv, int use_mg, int nu, Probe* pr) {
  const Level<double>& L = S->h64.L[0];
  precondition<T>(s, S, H, ainv, use_mg, nu, pr);
  pdl_launch(s, dim3(S->G), dim3(kThreads), 0, k_direction<T>, L, (const T*)H.L[0].x, S->p, (const Scalars*)S->sc, 1, (const int*)S->done);
  pdl_launch(s, dim3(S->G), dim3(kThreads), 0, k_apply_pap<T>, L, (const double*)S->p, S->ap, S->sc, slot(S, kSlotPap), S->counter,
             (const int*)S->done);
  GB_LAUNCHED(2);
}

// One CG iteration: x += alpha p, r -= alpha Ap (||r||^2 to host slot par),
// z = M r, p = z + beta p, Ap, alpha.
template <typename T>
void enqueue_iter(cudaStream_t s, Solver* S, Hierarchy<T>& H, const double* ainv, double* x64, int use_mg, int nu, int par, Probe* pr) {
  const Level<double>& L = S->h64.L[0];
  T* rT = sizeof(T) == 4 ? H.r : nullptr;
  pdl_launch(s, dim3(S->G), dim3(kThreads), 0, k_update<T>, L, x64, S->h64.r, (const double*)S->p, (const double*)S->ap, rT, S->sc,
             slot(S, kSlotRr), S->counter + 1, S->done, S->host + par);
  GB_LAUNCHED(1);
  precondition<T>(s, S, H, ainv, use_mg, nu, pr);
  pdl_launch(s, dim3(S->G), dim3(kThreads), 0, k_direction<T>, L, (const T*)H.L[0].x, S->p, (const Scalars*)S->sc, 0, (const int*)S->done);
  pdl_launch(s, dim3(S->G), dim3(kThreads), 0, k_apply_pap<T>, L, (const double*)S->p, S->ap, S->sc, slot(S, kSlotPap), S->counter,
             (const int*)S->done);
  GB_LAUNCHED(2);
}

// Capture fn's launches on the context's own stream into an executable graph.
template <typename F>
bool capture_graph(gb2d_ctx* c, cudaGraphExec_t* exec, unsigned long long* nodes, F fn) {
  cudaStream_t cs = c->own_stream;
  if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  unsigned long long captured = 0;
  t_capture_count = &captured;  // captured launches are counted when the graph runs
  fn(cs);
  t_capture_count = nullptr;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(cs, &g);
  *nodes = captured;
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

// The whole CG run as one graph: the init step, then a WHILE node whose body is one
// iteration followed by k_loop_cond.  Built by capturing into the graph (the init),
// adding the conditional node behind the captured work, and capturing the iteration
// into its body.  Returns false (nothing kept) if any step is refused.
template <typename T>
bool capture_loop_graph(gb2d_ctx* c, Solver* S, Hierarchy<T>& H, const double* ainv, double* x64, int use_mg, int nu, GraphSet& gs) {
  cudaStream_t cs = c->own_stream;
  cudaGraph_t g = nullptr;
  cudaGraphConditionalHandle h;
  bool ok = cudaGraphCreate(&g, 0) == cudaSuccess && cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
  unsigned long long captured = 0;
  if (ok && cudaStreamBeginCaptureToGraph(cs, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    t_capture_count = &captured;
    enqueue_init<T>(cs, S, H, ainv, use_mg, nu, nullptr);
    t_capture_count = nullptr;
    cudaStreamCaptureStatus st;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cnode = nullptr;
    ok = cudaStreamGetCaptureInfo(cs, &st, nullptr, nullptr, &deps, nullptr, &nd) == cudaSuccess && st == cudaStreamCaptureStatusActive &&
         cudaGraphAddNode(&cnode, g, deps, nullptr, nd, &cp) == cudaSuccess &&
         cudaStreamUpdateCaptureDependencies(cs, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies) == cudaSuccess;
    cudaGraph_t gout = nullptr;
    ok = cudaStreamEndCapture(cs, &gout) == cudaSuccess && ok;
    if (ok) {
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      unsigned long long nb = 0;
      ok = cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
      if (ok) {
        t_capture_count = &nb;
        enqueue_iter<T>(cs, S, H, ainv, x64, use_mg, nu, 0, nullptr);
        pdl_launch(cs, dim3(1), dim3(1), 0, k_loop_cond, h, S->sc, (const int*)S->done, S->host + 2);
        GB_LAUNCHED(1);
        t_capture_count = nullptr;
        cudaGraph_t bout = nullptr;
        ok = cudaStreamEndCapture(cs, &bout) == cudaSuccess;
      }
      gs.nodes_body = nb;
    }
  } else {
    ok = false;
  }
  if (ok) ok = cudaGraphInstantiate(&gs.loop, g, 0) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    gs.loop = nullptr;
    if (g) cudaGraphDestroy(g);
    return false;
  }
  gs.loop_graph = g;
  return true;
}

// Whether a context runs each CG solve as one graph launch.  A standalone solve does
// not gain from it: the host already checks iteration k-1 while k runs, and the WHILE
// node's pass boundary costs a few microseconds per iteration (1024^2: 2.45 -> 2.49 ms).
// Many contexts driven by contending host threads do (batch of 256 small grids:
// 2.19 -> 2.05 s), so batch instances turn it on.  GB2D_DEVICE_LOOP=0 / =1 forces it.
inline bool device_loop_enabled(const gb2d_ctx* c) {
  static const int forced = [] {
    const char* e = getenv("GB2D_DEVICE_LOOP");
    return e && (e[0] == '0' || e[0] == '1') ? e[0] - '0' : -1;
  }();
  return forced >= 0 ? forced == 1 : c->device_loop != 0;
}

template <typename T>
GraphSet* graphs_for(gb2d_ctx* c, Solver* S, Hierarchy<T>& H, const double* ainv, double* x64, int prec, int use_mg, int nu) {
  int slot = nu - 1;
  GraphSet& gs = S->graphs[prec][use_mg][slot];
  if (gs.ok && S->graph_x[prec][use_mg][slot] == x64) return &gs;
  if (gs.init) cudaGraphExecDestroy(gs.init);
  for (auto& g : gs.iter)
    if (g) cudaGraphExecDestroy(g);
  if (gs.loop) cudaGraphExecDestroy(gs.loop);
  if (gs.loop_graph) cudaGraphDestroy(gs.loop_graph);
  gs = GraphSet();
  bool ok = capture_graph(c, &gs.init, &gs.nodes_init, [&](cudaStream_t cs) { enqueue_init<T>(cs, S, H, ainv, use_mg, nu, nullptr); });
  for (int par = 0; par < 2 && ok; ++par)
    ok = capture_graph(c, &gs.iter[par], &gs.nodes_iter, [&](cudaStream_t cs) { enqueue_iter<T>(cs, S, H, ainv, x64, use_mg, nu, par, nullptr); });
  if (ok && device_loop_enabled(c)) capture_loop_graph<T>(c, S, H, ainv, x64, use_mg, nu, gs);
  gs.ok = ok;
  S->graph_x[prec][use_mg][slot] = x64;
  return ok ? &gs : nullptr;
}

// FP64 preconditioned CG from x64 with r = b - A x64 in h64.r (and its FP32 copy
// in H.r for an FP32 preconditioner), preconditioned by hierarchy H.  Stops when
// ||r||^2 <= thr2 or after max_it iterations; returns the iterations done and the
// last ||r||^2.  The host checks iteration k-1's residual while iteration k is
// queued; work queued after convergence returns at entry.
template <typename T>
int inner_pcg(gb2d_ctx* c, Solver* S, Hierarchy<T>& H, const double* ainv, double* x64, double thr2, int max_it, int prec, int use_mg, int nu,
              double* last_rr) {
  cudaStream_t s = c->stream;
  Probe* pr = &c->probe;
  GraphSet* gs = pr->on ? nullptr : graphs_for<T>(c, S, H, ainv, x64, prec, use_mg, nu);
  if (gs && gs->loop) {  // the whole run on the device: one launch, one wait
    k_begin_loop<<<1, 1, 0, s>>>(S->sc, S->done, thr2, max_it);
    cudaGraphLaunch(gs->loop, s);
    cudaStreamSynchronize(s);
    const int n = (int)S->host[3];
    *last_rr = S->host[2];
    GB_LAUNCHED(1 + gs->nodes_init + (unsigned long long)n * gs->nodes_body);
    return n;
  }
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

template <typename T, int SH>
cudaError_t set_smooth_smem_sh() {
  const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
  cudaError_t e = cudaFuncSetAttribute(k_pre_smooth<T, 1, SH>, a, (int)pre_smem<T, 1, SH>());
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_pre_smooth<T, 2, SH>, a, (int)pre_smem<T, 2, SH>());
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_pre_smooth<T, 3, SH>, a, (int)pre_smem<T, 3, SH>());
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_post_smooth<T, 1, SH>, a, (int)post_smem<T, 1, SH>());
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_post_smooth<T, 2, SH>, a, (int)post_smem<T, 2, SH>());
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_post_smooth<T, 3, SH>, a, (int)post_smem<T, 3, SH>());
  return e;
}
template <typename T>
cudaError_t set_smooth_smem() {
  cudaError_t e = set_smooth_smem_sh<T, 0>();
  if (e == cudaSuccess) e = set_smooth_smem_sh<T, 1>();
  if (e == cudaSuccess) e = set_smooth_smem_sh<T, 2>();
  if (e == cudaSuccess) e = set_smooth_smem_sh<T, 3>();
  return e;
}

// Tile shape per tiled level: 32x16 where that gives at least 8 blocks per SM,
// else 32x8; FP32 levels of 1024^2 cells and more take 32x32.  Measured on GB300
// (MG-PCG projection to 1e-8, 512^2-4096^2): the 32x16 tile beats 64x16 on every
// level size, its 22 KB window (FP32, two sweeps) letting 8 blocks share an SM
// against 5, and the extra warps hide the staging loads' latency better than the
// larger tile saves halo work; below 1024^2 the 32x8 tile's shorter per-block
// pipeline wins; on the large FP32 levels, with the colour-split window staged
// by pairs of cells, the 32x32 tile's smaller halo share wins (mixed projection
// 2.280 -> 2.249 ms at 1024^2, 6.000 -> 5.973 ms at 2048^2 from its 1024^2
// level); not in FP64.  GB2D_TILE_SHAPES="s0,s1,..." (0-3
// per level from the finest) overrides the rule, for tuning.
template <typename T>
void plan_shapes(Hierarchy<T>& H, int nsm) {
  const char* env = getenv("GB2D_TILE_SHAPES");
  for (int l = 0; l < H.nlev; ++l) {
    const dim3 t = tiles(H.L[l].nI, H.L[l].nJ, 1);
    int sh = (long long)t.x * t.y >= 8LL * nsm ? 1 : 2;
    if (sizeof(T) == 4 && (long long)H.L[l].nI * H.L[l].nJ >= 1024LL * 1024) sh = 3;
    H.shape[l] = sh;
  }
  for (int l = 0; env && *env && l < H.nlev; ++l) {
    const int v = *env - '0';
    if (v >= 0 && v < kTileShapes) H.shape[l] = v;
    while (*env && *env != ',') ++env;
    if (*env == ',') ++env;
  }
}

}  // namespace

Solver* solver_create(int ni, int nj, char* err, size_t errlen) {
  // Kernel attributes and the cluster-size probe are process-wide: one creation at a time.
  static std::mutex create_lock;
  std::lock_guard<std::mutex> hold(create_lock);
  Solver* S = new Solver();
  S->ni = ni;
  S->nj = nj;
  size_t n = (size_t)ni * nj;
  S->G = (int)nblocks(n, 1216);
  dim3 t = tiles(ni, nj, 2);  // the most blocks any tile shape launches (32x8)
  S->nparts_cap = (int)(t.x * t.y) > S->G ? (int)(t.x * t.y) : S->G;
  size_t np = (size_t)(ni + 2) * (nj + 2);
  cudaError_t e = alloc_hierarchy(S->h64, ni, nj);
  if (e == cudaSuccess) e = alloc_hierarchy(S->h32, ni, nj);
  if (e == cudaSuccess) {
    int P = ctail_cluster_size();
    plan_ctail(S->h64, P);
    plan_ctail(S->h32, P);
    int dev = 0, nsm = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    plan_shapes(S->h64, nsm);
    plan_shapes(S->h32, nsm);
  }
  if (e == cudaSuccess) e = cudaMalloc(&S->ainv64, sizeof(double) * kCoarseMax * kCoarseMax);
  if (e == cudaSuccess) e = cudaMalloc(&S->ainv32, sizeof(double) * kCoarseMax * kCoarseMax);
  for (double** v : {&S->b64, &S->p, &S->ap}) {
    if (e == cudaSuccess) e = cudaMalloc(v, np * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(*v, 0, np * sizeof(double));
  }
  if (e == cudaSuccess) e = cudaMalloc(&S->part, sizeof(double) * kSlots * (size_t)S->nparts_cap);
  if (e == cudaSuccess) e = cudaMemset(S->part, 0, sizeof(double) * kSlots * (size_t)S->nparts_cap);
  if (e == cudaSuccess) e = cudaMalloc(&S->counter, 4 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(S->counter, 0, 4 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&S->done, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(S->done, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&S->sc, sizeof(Scalars));
  if (e == cudaSuccess) e = cudaMemset(S->sc, 0, sizeof(Scalars));
  if (e == cudaSuccess) e = cudaMallocHost(&S->host, 8 * sizeof(double));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S->ev[0], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S->ev[1], cudaEventDisableTiming);
  if (e == cudaSuccess) e = set_smooth_smem<float>();
  if (e == cudaSuccess) e = set_smooth_smem<double>();
  if (e == cudaSuccess) e = set_stream_smem<float>();
  if (e == cudaSuccess) e = set_stream_smem<double>();
  // The attribute is per kernel for the whole process: only ever raise it.
  static size_t tail_smem_set[2] = {0, 0};
  if (e == cudaSuccess && S->h64.tail_smem > tail_smem_set[0]) {
    e = cudaFuncSetAttribute(k_tail<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S->h64.tail_smem);
    if (e == cudaSuccess) tail_smem_set[0] = S->h64.tail_smem;
  }
  if (e == cudaSuccess && S->h32.tail_smem > tail_smem_set[1]) {
    e = cudaFuncSetAttribute(k_tail<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S->h32.tail_smem);
    if (e == cudaSuccess) tail_smem_set[1] = S->h32.tail_smem;
  }
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
        if (g.loop) cudaGraphExecDestroy(g.loop);
        if (g.loop_graph) cudaGraphDestroy(g.loop_graph);
      }
  free_hierarchy(S->h64);
  free_hierarchy(S->h32);
  double* d[] = {S->ainv64, S->ainv32, S->b64, S->p, S->ap, S->part};
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

void solver_layout(const Solver* S, int mixed, int* levels, int* cluster_top, int* cluster_ctas) {
  if (mixed) {
    *levels = S->h32.nlev;
    *cluster_top = S->h32.ctail;
    *cluster_ctas = S->h32.ctail >= 0 ? S->h32.ct_P : 0;
  } else {
    *levels = S->h64.nlev;
    *cluster_top = S->h64.ctail;
    *cluster_ctas = S->h64.ctail >= 0 ? S->h64.ct_P : 0;
  }
}

// Tile shapes of the tiled smoothing levels: plan < 0 restores the default rule
// (plan_shapes), 0-3 give every tiled level that shape (64x16, 32x16, 32x8, 32x32).  The
// cached CG graphs hold the old launches and are captured again on their next use.
void solver_set_tile_plan(gb2d_ctx* c, int plan) {
  Solver* S = c->solver;
  if (!S) return;
  int dev = 0, nsm = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  plan_shapes(S->h64, nsm);
  plan_shapes(S->h32, nsm);
  if (plan >= 0 && plan < kTileShapes)
    for (int l = 0; l < kMaxLevels; ++l) S->h64.shape[l] = S->h32.shape[l] = plan;
  for (auto& a : S->graphs)
    for (auto& b : a)
      for (auto& g : b) g.ok = false;
}

unsigned long long solver_body_nodes(const gb2d_ctx* c) { return c->solver ? c->solver->body_nodes : 0; }

namespace {
// Padded level layout <- compact FP64 host-order array (the preconditioner's input r,
// narrowed as the solver narrows its FP32 copy of r).
template <typename T>
__global__ void k_load_padded(const double* __restrict__ src, T* __restrict__ dst, int ni, int nj, int ld) {
  GB_FOR_IJ(i, j, ni, nj) dst[(size_t)(i + 1) + (size_t)(j + 1) * ld] = in_prec(src[(size_t)j * ni + i], T());
}
template <typename T>
__global__ void k_store_compact(const T* __restrict__ src, double* __restrict__ dst, int ni, int nj, int ld) {
  GB_FOR_IJ(i, j, ni, nj) dst[(size_t)j * ni + i] = widen(src[(size_t)(i + 1) + (size_t)(j + 1) * ld]);
}

template <typename T>
int precondition_once(gb2d_ctx* c, Hierarchy<T>& H, double* ainv, int nu, const double* r_dev, double* z_dev) {
  Solver* S = c->solver;
  cudaStream_t s = c->stream;
  const int ni = c->grid.ni, nj = c->grid.nj;
  build_hierarchy<T>(s, H, c, sizeof(T) == 8 ? S->b64 : nullptr, ainv);
  k_load_padded<T><<<grid_ij(ni, nj), kThreads, 0, s>>>(r_dev, H.r, ni, nj, H.L[0].ld);
  GB_LAUNCHED(1);
  if (cudaMemsetAsync(S->done, 0, sizeof(int), s) != cudaSuccess) return GB2D_ERR_CUDA;
  vcycle<T>(s, S, H, ainv, nu, nullptr);
  k_store_compact<T><<<grid_ij(ni, nj), kThreads, 0, s>>>(H.L[0].x, z_dev, ni, nj, H.L[0].ld);
  GB_LAUNCHED(1);
  S->keep = false;  // the next solve rebuilds its levels from the system it is given
  return cudaGetLastError() == cudaSuccess ? GB2D_OK : GB2D_ERR_CUDA;
}
}  // namespace

int solver_precondition(gb2d_ctx* c, int prec, int nu, const double* r_dev, double* z_dev) {
  Solver* S = c->solver;
  if (!S) return GB2D_ERR_ARG;
  nu = nu > 0 ? (nu > 3 ? 3 : nu) : 2;
  return prec ? precondition_once<float>(c, S->h32, S->ainv32, nu, r_dev, z_dev)
              : precondition_once<double>(c, S->h64, S->ainv64, nu, r_dev, z_dev);
}

void solver_prebuild(gb2d_ctx* c, const gb2d_solve_opts* o) {
  Solver* S = c->solver;
  if (!S || o->solver != GB2D_SOLVER_MGPCG) return;
  // Below this size the assembly kernels are too short for the overlap to repay the
  // extra fork and join: a batch of 256 rising bubbles of 64^2-512^2 on 16 host threads
  // took 2.25 s with the prebuild and 2.16 s without (GB2D_PREBUILD_MIN_CELLS overrides,
  // for tuning).
  static const long min_cells = [] {
    const char* e = getenv("GB2D_PREBUILD_MIN_CELLS");
    return e && atol(e) >= 0 ? atol(e) : 300000L;
  }();
  if ((long)S->ni * S->nj < min_cells) return;
  cudaEventRecord(c->ev_fork2, c->stream);
  cudaStreamWaitEvent(c->side2, c->ev_fork2, 0);
  if (o->precision == GB2D_PRECISION_MIXED) {
    // The FP32 hierarchy; the FP64 finest level stays on the context stream (it is
    // short, and queued here it would delay the hierarchy the first V-cycle waits for).
    build_hierarchy<float>(c->side2, S->h32, c, nullptr, S->ainv32);
  } else {
    // The FP64 finest level first (the residual waits for it; solver_solve copies its
    // right-hand side once that exists), then the coarse levels and dense inverse.
    build_level0_f64(c->side2, S->h64, c, nullptr);
    cudaEventRecord(c->ev_pre0, c->side2);
    build_coarse<double>(c->side2, S->h64, S->ainv64);
  }
  cudaEventRecord(c->ev_join2, c->side2);
  S->prebuilt = true;
}

void solver_keep_levels(gb2d_ctx* c) {
  if (c->solver) c->solver->keep = true;
}

void solver_drop_prebuild(gb2d_ctx* c) {
  Solver* S = c->solver;
  if (!S || !S->prebuilt) return;
  cudaStreamWaitEvent(c->stream, c->ev_join2, 0);  // later builds on the side stream follow it
  S->prebuilt = false;
}

// Append to the capture running on s a WHILE node whose body (captured on body) is one CG
// iteration followed by k_loop_cond, with the handle h (created on the capturing graph).
template <typename T>
bool append_cg_loop(cudaStream_t s, cudaStream_t body, cudaGraphConditionalHandle h, Solver* S, Hierarchy<T>& H, const double* ainv,
                    double* x64, int use_mg, int nu) {
  cudaStreamCaptureStatus st;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  if (cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd) != cudaSuccess || st != cudaStreamCaptureStatusActive) return false;
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node = nullptr;
  if (cudaGraphAddNode(&node, g, deps, nullptr, nd, &cp) != cudaSuccess) return false;
  if (cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess) return false;
  if (cudaStreamBeginCaptureToGraph(body, cp.conditional.phGraph_out[0], nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) !=
      cudaSuccess)
    return false;
  unsigned long long* outer = t_capture_count;  // the body's launches count per iteration, apart
  unsigned long long nb = 0;
  t_capture_count = &nb;
  enqueue_iter<T>(body, S, H, ainv, x64, use_mg, nu, 0, nullptr);
  pdl_launch(body, dim3(1), dim3(1), 0, k_loop_cond, h, S->sc, (const int*)S->done, S->host + 2);
  GB_LAUNCHED(1);
  t_capture_count = outer;
  S->body_nodes = nb;
  cudaGraph_t out = nullptr;
  return cudaStreamEndCapture(body, &out) == cudaSuccess;
}

// The solve of a device-driven frame (ctx->graph_mode, captured on ctx->stream): the true
// residual and ||b||^2 into the frame scalars, then two passes of [threshold and done flag
// on the device, CG init, WHILE over one iteration, true residual] -- the host loop's first
// pass and the restart it takes when the recursive residual has drifted above the
// tolerance (a pass whose start is converged runs no iteration).  Nothing is read back.
template <typename T>
int solve_on_device(gb2d_ctx* c, Solver* S, Hierarchy<T>& H, const double* ainv, double* x, int use_mg, int nu, double tol,
                    int max_it, cudaEvent_t join_ev, bool joined) {
  cudaStream_t s = c->stream;
  const unsigned G = (unsigned)S->G;
  double* P_rr = slot(S, kSlotRr);
  double* P_bb = slot(S, kSlotBb);
  const bool mixed = sizeof(T) == 4;
  auto residual = [&]() {
    if (mixed)
      k_residual64<float><<<G, kThreads, 0, s>>>(S->h64.L[0], x, S->b64, S->h64.r, S->h32.r, P_rr, P_bb);
    else
      k_residual64<double><<<G, kThreads, 0, s>>>(S->h64.L[0], x, S->b64, S->h64.r, nullptr, P_rr, P_bb);
    k_reduce_two<<<1, kThreads, 0, s>>>(P_rr, P_bb, G, &c->sc->g_rr);
    GB_LAUNCHED(2);
  };
  residual();
  if (!joined) cudaStreamWaitEvent(s, join_ev, 0);
  cudaMemsetAsync(&S->sc->flag, 0, sizeof(int), s);
  for (int pass = 0; pass < 2; ++pass) {
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    if (cudaStreamGetCaptureInfo(s, &st, nullptr, &g, nullptr, nullptr, nullptr) != cudaSuccess || st != cudaStreamCaptureStatusActive) {
      snprintf(c->err, sizeof(c->err), "device-driven solve: the stream is not capturing");
      return GB2D_ERR_CUDA;
    }
    cudaGraphConditionalHandle h;
    if (cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault) != cudaSuccess) {
      cudaGetLastError();
      snprintf(c->err, sizeof(c->err), "device-driven solve: conditional handle refused");
      return GB2D_ERR_CUDA;
    }
    k_begin_device<<<1, 1, 0, s>>>(h, S->sc, S->done, c->sc, tol * tol, max_it, pass == 0);
    GB_LAUNCHED(1);
    enqueue_init<T>(s, S, H, ainv, use_mg, nu, nullptr);
    if (!append_cg_loop<T>(s, c->body_stream, h, S, H, ainv, x, use_mg, nu)) {
      cudaGetLastError();
      snprintf(c->err, sizeof(c->err), "device-driven solve: the CG loop node was refused");
      return GB2D_ERR_CUDA;
    }
    residual();
    k_end_device<<<1, 1, 0, s>>>(S->sc, c->sc, pass == 1);
    GB_LAUNCHED(1);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(c->err, sizeof(c->err), "device-driven solve: %s", cudaGetErrorString(e));
    return GB2D_ERR_CUDA;
  }
  return GB2D_OK;
}

// x: padded FP64 solution (warm start in, result out); the system is ctx->bx/by/diag/rhs.
// FP64 CG throughout; the preconditioner runs in FP64 or, for
// GB2D_PRECISION_MIXED, in FP32.  The loop around the CG recomputes the true
// residual with the reference's entries and restarts only if the recursive
// residual has drifted above the tolerance.
int solver_solve(gb2d_ctx* c, const double* /*rhs*/, double* x, const gb2d_solve_opts* o, gb2d_solve_stats* st) {
  Solver* S = c->solver;
  cudaStream_t s = c->stream;
  int nu = o->mg_smooth > 0 ? (o->mg_smooth > 3 ? 3 : o->mg_smooth) : 2;
  int use_mg = o->solver == GB2D_SOLVER_MGPCG;
  int prec = o->precision == GB2D_PRECISION_MIXED ? 1 : 0;
  double tol = o->tolerance > 0 ? o->tolerance : 1e-8;
  int max_it = o->max_iterations > 0 ? o->max_iterations : 10000;
  unsigned G = (unsigned)S->G;
  double* P_rr = slot(S, kSlotRr);
  double* P_bb = slot(S, kSlotBb);

  cudaEvent_t join_ev = c->ev_join;
  bool joined = !(prec && use_mg);
  const bool keep = S->keep && !S->prebuilt;
  S->keep = false;
  if (keep) {
    // The system's coefficients are those of the previous solve: its levels stand,
    // only b changes.
    launch_copy_interior(s, c->rhs, 0, S->b64, 1, c->grid.ni, c->grid.nj);
    joined = true;
  } else if (use_mg && S->prebuilt) {
    // Started by solver_prebuild during the assembly; joined before the first V-cycle.
    if (prec) {
      build_level0_f64(s, S->h64, c, S->b64);
    } else {  // b here, the finest FP64 level before the residual
      launch_copy_interior(s, c->rhs, 0, S->b64, 1, c->grid.ni, c->grid.nj);
      cudaStreamWaitEvent(s, c->ev_pre0, 0);
    }
    join_ev = c->ev_join2;
    joined = false;
  } else {
    if (prec && use_mg) {
      // The FP32 hierarchy (its dense coarse inverse keeps one SM busy) builds on
      // the side stream while the FP64 residual runs; joined before the first V-cycle.
      cudaEventRecord(c->ev_fork, s);
      cudaStreamWaitEvent(c->side, c->ev_fork, 0);
      build_hierarchy<float>(c->side, S->h32, c, nullptr, S->ainv32);
      cudaEventRecord(c->ev_join, c->side);
    }
    if (prec || !use_mg)
      build_level0_f64(s, S->h64, c, S->b64);
    else
      build_hierarchy<double>(s, S->h64, c, S->b64, S->ainv64);
  }
  S->prebuilt = false;
  if (prec && !use_mg && !keep) {
    double idx2 = 1.0 / (c->base.dx * c->base.dx), idy2 = 1.0 / (c->base.dy * c->base.dy);
    k_build_level0<float><<<grid_ij(c->grid.ni, c->grid.nj), kThreads, 0, s>>>(c->bx, c->by, c->diag, c->rhs, c->sys_shift,
                                                                                                S->h32.L[0], nullptr, idx2, idy2);
    GB_LAUNCHED(1);
  }
  if (c->graph_mode) {
    if (prec)
      return solve_on_device<float>(c, S, S->h32, S->ainv32, x, use_mg, nu, tol, max_it, join_ev, joined);
    return solve_on_device<double>(c, S, S->h64, S->ainv64, x, use_mg, nu, tol, max_it, join_ev, joined);
  }
  int total = 0, outer = 0;
  double rr = 0, bb = 0;
  int status = GB2D_OK;
  while (true) {
    if (prec)
      k_residual64<float><<<G, kThreads, 0, s>>>(S->h64.L[0], x, S->b64, S->h64.r, S->h32.r, P_rr, P_bb);
    else
      k_residual64<double><<<G, kThreads, 0, s>>>(S->h64.L[0], x, S->b64, S->h64.r, nullptr, P_rr, P_bb);
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
    if (total >= max_it || outer >= 64) {
      status = GB2D_ERR_MAX_ITERS;
      break;
    }
    double rr_in = rr;
    int it;
    if (!joined) {
      cudaStreamWaitEvent(s, join_ev, 0);
      joined = true;
    }
    if (prec)
      it = inner_pcg<float>(c, S, S->h32, S->ainv32, x, thr2, max_it - total, prec, use_mg, nu, &rr_in);
    else
      it = inner_pcg<double>(c, S, S->h64, S->ainv64, x, thr2, max_it - total, prec, use_mg, nu, &rr_in);
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
  }
  if (!joined) cudaStreamWaitEvent(s, join_ev, 0);  // later work on the context stream follows the side build
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
