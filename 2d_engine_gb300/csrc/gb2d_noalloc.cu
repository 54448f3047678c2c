// Allocation-free pressure solve: FP64 Jacobi-preconditioned CG on an assembled
// ghost-fluid system, for callers that cannot allocate device memory.
//
// Who needs it: hosts that reserve all device memory up front for their own
// pool and forbid further cudaMalloc/cudaFree (a game or visual-effects engine
// running a fixed memory budget, a solver embedded in another application's
// allocator), and code that must not allocate between frames because an
// allocation can synchronise the device.  They hand in device buffers for the
// system and the solution; the CG vectors and reduction partials live in one
// file-scope device array instead of memory from cudaMalloc.
//
// Limits and rules:
//   * at most GB2D_NOALLOC_MAX_CELLS (65536) unknowns (ni * nj); larger sizes are
//     rejected with GB2D_ERR_TOO_LARGE before any work;
//   * the array (about 2.1 MB) stays resident on every GPU that loads this library
//     until the process exits;
//   * the first call on a device looks up the array's device address with that
//     device current (cudaGetSymbolAddress) and caches it per device ordinal for
//     the life of the process; make that first call before any stream capture.
//     The cached address belongs to the context that was current at that first
//     call (normally the device's primary context): after cudaDeviceReset, or
//     from a different context on the same device, the array lives elsewhere and
//     this entry point must not be called again in that process;
//   * every call shares the one array and keeps the previous call's contents:
//     calls whose work overlaps on the GPU (other streams or threads) race and
//     must be serialised by the caller.
#include <cmath>
#include <cstdio>

#include "gb2d.h"

namespace {

constexpr int kMaxCells = GB2D_NOALLOC_MAX_CELLS;
constexpr int kThreads = 256;
constexpr int kBlocks = 256;  // fixed grid: partial sums per reduction

// Layout: r, z, p, ap (kMaxCells each), then 3 partial-sum slots, then scalars.
constexpr size_t kVec = kMaxCells;
constexpr size_t kPartOff = 4 * kVec;
constexpr size_t kScalOff = kPartOff + 3 * kBlocks;
constexpr size_t kScratchDoubles = kScalOff + 8;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
static double* g_scratch_ptr[kMaxDevices];  // device address per device, set on first use

struct Sys {
  int ni, nj;
  double idx2, idy2;
  const double *bx, *by, *dg, *rhs;
};

__device__ __forceinline__ double apply(const Sys& s, const double* x, int i, int j) {
  size_t t = (size_t)i + (size_t)j * s.ni;
  double acc = s.dg[t] * x[t];
  if (i > 0) acc -= s.bx[i + (size_t)j * (s.ni + 1)] * s.idx2 * x[t - 1];
  if (i < s.ni - 1) acc -= s.bx[i + 1 + (size_t)j * (s.ni + 1)] * s.idx2 * x[t + 1];
  if (j > 0) acc -= s.by[i + (size_t)j * s.ni] * s.idy2 * x[t - s.ni];
  if (j < s.nj - 1) acc -= s.by[i + (size_t)(j + 1) * s.ni] * s.idy2 * x[t + s.ni];
  return acc;
}

__device__ double block_sum(double v) {
  __shared__ double sm[kThreads / 32];
  __shared__ double total;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double x = threadIdx.x < kThreads / 32 ? sm[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (threadIdx.x == 0) total = x;
  }
  __syncthreads();
  return total;
}

__device__ double sum_parts(const double* part) {
  double v = 0;
  for (int k = threadIdx.x; k < kBlocks; k += kThreads) v += part[k];
  return block_sum(v);
}

// r = b - A x, z = r/dg, p = z; partials r.z (slot 0), b.b (slot 1) and r.r (slot 2).
__global__ void k_init(Sys s, const double* __restrict__ x, double* scr) {
  double *r = scr, *z = scr + kVec, *p = scr + 2 * kVec, *part = scr + kPartOff;
  size_t n = (size_t)s.ni * s.nj;
  double rz = 0, bb = 0, rr = 0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(t % s.ni), j = (int)(t / s.ni);
    double rv = s.rhs[t] - apply(s, x, i, j);
    double zv = rv / s.dg[t];
    r[t] = rv;
    z[t] = zv;
    p[t] = zv;
    rz += rv * zv;
    bb += s.rhs[t] * s.rhs[t];
    rr += rv * rv;
  }
  rz = block_sum(rz);
  bb = block_sum(bb);
  rr = block_sum(rr);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = rz;
    part[kBlocks + blockIdx.x] = bb;
    part[2 * kBlocks + blockIdx.x] = rr;
  }
}

// Scalars: [0] r.z, [1] b.b, [2] r.r (of the starting guess, then of the latest update).
__global__ void k_init_scalars(double* scr) {
  double* part = scr + kPartOff;
  double* sc = scr + kScalOff;
  double rz = sum_parts(part), bb = sum_parts(part + kBlocks), rr = sum_parts(part + 2 * kBlocks);
  if (threadIdx.x == 0) {
    sc[0] = rz;
    sc[1] = bb;
    sc[2] = rr;
  }
}

// ap = A p; partial p.ap (slot 2).
__global__ void k_apply(Sys s, double* scr) {
  double *p = scr + 2 * kVec, *ap = scr + 3 * kVec, *part = scr + kPartOff;
  size_t n = (size_t)s.ni * s.nj;
  double acc = 0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(t % s.ni), j = (int)(t / s.ni);
    double y = apply(s, p, i, j);
    ap[t] = y;
    acc += p[t] * y;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) part[2 * kBlocks + blockIdx.x] = acc;
}

// alpha = r.z / p.ap; x += alpha p; r -= alpha ap; z = r/dg; partials r.z (slot 0), r.r (slot 1).
__global__ void k_update(Sys s, double* __restrict__ x, double* scr) {
  double *r = scr, *z = scr + kVec, *p = scr + 2 * kVec, *ap = scr + 3 * kVec, *part = scr + kPartOff;
  const double* sc = scr + kScalOff;
  // p.ap is zero only when p is: r.z was zero too, and the step is none.
  const double pap = sum_parts(part + 2 * kBlocks);
  double alpha = pap != 0.0 ? sc[0] / pap : 0.0;
  size_t n = (size_t)s.ni * s.nj;
  double rz = 0, rr = 0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    x[t] += alpha * p[t];
    double rv = r[t] - alpha * ap[t];
    double zv = rv / s.dg[t];
    r[t] = rv;
    z[t] = zv;
    rz += rv * zv;
    rr += rv * rv;
  }
  rz = block_sum(rz);
  rr = block_sum(rr);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = rz;
    part[kBlocks + blockIdx.x] = rr;
  }
}

// beta = rz_new / rz_old; p = z + beta p; records rz_new and r.r.
__global__ void k_direction(Sys s, double* scr) {
  double *z = scr + kVec, *p = scr + 2 * kVec, *part = scr + kPartOff;
  double* sc = scr + kScalOff;
  double rz_new = sum_parts(part), rr = sum_parts(part + kBlocks);
  double beta = sc[0] != 0.0 ? rz_new / sc[0] : 0.0;
  size_t n = (size_t)s.ni * s.nj;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) p[t] = z[t] + beta * p[t];
  // Other blocks may still be reading the old r.z in sc[0]: the new one goes to
  // sc[3] and k_swap makes it current once this kernel has finished.
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sc[3] = rz_new;
    sc[2] = rr;
  }
}

__global__ void k_swap(double* scr) {
  double* sc = scr + kScalOff;
  sc[0] = sc[3];
}

}  // namespace

extern "C" int gb2d_poisson_solve_noalloc(int ni, int nj, double dx, double dy, const double* bx, const double* by, const double* diag,
                                          const double* rhs, double* x, double tolerance, int max_iterations, void* stream, int* iterations,
                                          double* rel_residual) {
  if (ni < 1 || nj < 1 || !bx || !by || !diag || !rhs || !x || !(dx > 0) || !(dy > 0) || max_iterations < 1) return GB2D_ERR_ARG;
  if ((long long)ni * nj > kMaxCells) return GB2D_ERR_TOO_LARGE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GB2D_ERR_CUDA;
  if (!g_scratch_ptr[dev]) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) {
      cudaGetLastError();
      return GB2D_ERR_CUDA;
    }
    g_scratch_ptr[dev] = (double*)ptr;
  }
  double* scr = g_scratch_ptr[dev];
  cudaStream_t s = (cudaStream_t)stream;
  Sys sys{ni, nj, 1.0 / (dx * dx), 1.0 / (dy * dy), bx, by, diag, rhs};
  k_init<<<kBlocks, kThreads, 0, s>>>(sys, x, scr);
  k_init_scalars<<<1, kThreads, 0, s>>>(scr);
  if (cudaGetLastError() != cudaSuccess) return GB2D_ERR_CUDA;
  double sc[4] = {0, 0, 0, 0};
  if (cudaMemcpyAsync(sc, scr + kScalOff, 3 * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) return GB2D_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return GB2D_ERR_CUDA;
  double bb = sc[1], thr2 = tolerance * tolerance * bb;
  int it = 0;
  double rr = sc[2];
  if (!std::isfinite(bb) || !std::isfinite(rr)) return GB2D_ERR_NONFINITE;
  // A starting guess that already meets the tolerance (a warm start from the
  // solution) is returned unchanged after zero iterations.
  if (bb > 0 && rr > thr2) {
    for (it = 1; it <= max_iterations; ++it) {
      k_apply<<<kBlocks, kThreads, 0, s>>>(sys, scr);
      k_update<<<kBlocks, kThreads, 0, s>>>(sys, x, scr);
      k_direction<<<kBlocks, kThreads, 0, s>>>(sys, scr);
      k_swap<<<1, 1, 0, s>>>(scr);
      if (cudaGetLastError() != cudaSuccess) return GB2D_ERR_CUDA;
      if (cudaMemcpyAsync(sc, scr + kScalOff, 4 * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) return GB2D_ERR_CUDA;
      if (cudaStreamSynchronize(s) != cudaSuccess) return GB2D_ERR_CUDA;
      rr = sc[2];
      if (!std::isfinite(rr)) return GB2D_ERR_NONFINITE;
      if (rr <= thr2) break;
    }
  }
  if (iterations) *iterations = it > max_iterations ? max_iterations : it;
  if (rel_residual) *rel_residual = bb > 0 ? std::sqrt(rr / bb) : 0.0;
  return it > max_iterations ? GB2D_ERR_MAX_ITERS : GB2D_OK;
}
