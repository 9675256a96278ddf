// gbn_probe.cu -- shared-memory atomic throughput with the spread's access
// pattern, the ceiling the shared-memory spreading kernels are held against.
// A measurement aid of bench.py, built into its own library (libgbnprobe.so)
// and not part of libgbnufft.so.
//
// Each 8-lane group stands for one point: lane gl < w adds into x offset gl
// of w rows of a 32 KB shared tile (row pitch 24 words, random row origin
// per point), exactly the int32 red.shared pattern of the fixed-point spread.
// The result is int32 atomic adds per second over the whole GPU.
#include <cuda_runtime.h>

namespace {

constexpr int kProbeWords = 8192;  // 32 KB of int32 cells

__device__ __forceinline__ unsigned probe_hash(unsigned x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

__global__ void __launch_bounds__(256) smem_atomic_probe_kernel(int iters, int w, int* sink) {
  __shared__ int tile[kProbeWords];
  for (int i = threadIdx.x; i < kProbeWords; i += blockDim.x) tile[i] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, gl = lane & 7;
  const unsigned seed = blockIdx.x * 977u + (threadIdx.x >> 3);
  for (int it = 0; it < iters; ++it) {
    const unsigned base = probe_hash(seed + it * 131u) & (kProbeWords - 1);
    if (gl < w) {
      for (int r = 0; r < w; ++r) atomicAdd(&tile[(base + gl + r * 24) & (kProbeWords - 1)], 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) sink[blockIdx.x] = tile[lane] + tile[100];
}

}  // namespace

// int32 shared-memory atomic adds per second over the whole GPU with the
// access pattern of the fixed-point spread (w lanes x w rows per point,
// 8-lane groups).  Synchronises `stream`.  Returns 0, -1 for bad arguments,
// or the CUDA error code.
extern "C" __attribute__((visibility("default"))) int gbn_probe_smem_atomics(
    void* stream, int w, double* atomics_per_s) {
  if (!atomics_per_s || w < 1 || w > 8) return -1;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = 4 * sms, iters = 2000;
  int* sink = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMallocAsync(&sink, blocks * sizeof(int), s);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float best = 0.f;
  for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
    cudaEventRecord(e0, s);
    smem_atomic_probe_kernel<<<blocks, 256, 0, s>>>(iters, w, sink);
    cudaEventRecord(e1, s);
    e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && (best == 0.f || ms < best)) best = ms;  // first launch is a warm-up
  }
  if (sink) cudaFreeAsync(sink, s);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) return (int)e;
  const double atomics = (double)blocks * (256 / 8) * iters * w * w;
  *atomics_per_s = best > 0.f ? atomics / (best * 1e-3) : 0.0;
  return 0;
}
