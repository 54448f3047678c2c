// gb2d_peaks: arithmetic peaks of the device, measured, for the roofline of the
// ALU-bound kernels (the WENO5 / reinitialisation sweeps).  The HBM peak comes from a
// copy benchmark outside this library; the FP64 and FP32 FMA rates come from here.
//
// Every thread runs kChains independent FMA chains (x <- x * m + a) for a fixed
// number of iterations; the grid fills every SM with 2048 resident threads.  m and a
// are kernel arguments, so nothing is folded at compile time, and the chains' sum is
// stored, so nothing is removed.  Flops = 2 per FMA.  Each measurement is the best
// of three timed launches after one warm-up, timed with CUDA events.
#include <cuda_runtime.h>

#include "gb2d_internal.cuh"

namespace {

constexpr int kChains = 8;
constexpr int kPeakThreads = 256;
constexpr int kPeakBlocksPerSm = 8;

template <typename T>
__global__ void __launch_bounds__(kPeakThreads) k_fma_chains(T* __restrict__ out, T m, T a, int iters) {
  T x[kChains];
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll
  for (int k = 0; k < kChains; ++k) x[k] = (T)(tid & 7) * (T)0.125 + (T)k;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) x[k] = fma(x[k], m, a);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += x[k];
  out[tid] = s;
}

template <typename T>
int time_chains(int nsm, int iters, double* tflops) {
  const int blocks = nsm * kPeakBlocksPerSm, threads = blocks * kPeakThreads;
  T* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(T) * threads);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float best = 0.f;
  for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
    cudaEventRecord(e0);
    // m slightly below 1 and a small: the chains stay finite and normal for any iters.
    k_fma_chains<T><<<blocks, kPeakThreads>>>(out, (T)0.999999, (T)1e-3, iters);
    cudaEventRecord(e1);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && (best == 0.f || ms < best)) best = ms;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  if (e != cudaSuccess) return GB2D_ERR_CUDA;
  *tflops = 2.0 * kChains * (double)iters * threads / (best * 1e-3) / 1e12;
  return GB2D_OK;
}

}  // namespace

extern "C" {

int gb2d_alu_peaks(double* fp64_tflops, double* fp32_tflops) {
  if (!fp64_tflops || !fp32_tflops) return GB2D_ERR_ARG;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      nsm <= 0)
    return GB2D_ERR_NO_DEVICE;
  // About 16 ms per FP64 launch and 8 ms per FP32 launch on a GB300 (20 and 650 GFLOP).
  int rc = time_chains<double>(nsm, 1 << 12, fp64_tflops);
  if (rc == GB2D_OK) rc = time_chains<float>(nsm, 1 << 17, fp32_tflops);
  GB_LAUNCHED(8);
  return rc;
}

}  // extern "C"
