// gbn_probe.cu -- shared-memory atomic throughput with the access pattern of
// the row-owned spread (spread_rows_kernel), the ceiling its atomic phase is
// held against.  A measurement aid of bench.py, built into its own library
// (libgbnprobe.so) and not part of libgbnufft.so.
//
// Each warp stands for one point at a time, exactly as the row-owned spread
// adds it: lane (part, r, gl) -- part = lane / 16 the real or imaginary
// word, gl = q % WV an x offset, r = q / WV a row, q = lane % 16, WV = w
// rounded up to even -- adds to word 2 (base + gl + PY (chunk R + r) + PZ iz)
// + part of a fixed-point tile with the spread's pitches (PY = 16 + WV, PZ =
// PY (15 + w)), for ceil(w / R) row chunks times w planes, R = 16 / WV; the
// point's base cell is random.  The adds are int32 red.shared, every lane on
// every instruction, as in the kernel; only the kernel-value arithmetic is
// left out.  The result is the point's w^3 complex cell updates per second
// over the whole GPU.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

constexpr int kProbeWords = 12288;  // 48 KB of int32 cells

__device__ __forceinline__ unsigned probe_hash(unsigned x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

template <int W>
__global__ void __launch_bounds__(256) smem_row_probe_kernel(int iters, int* sink) {
  constexpr int WV = (W + 1) & ~1, R = 16 / WV, NCH = (W + R - 1) / R;
  constexpr int PY = 16 + WV, PZ = PY * (15 + W);
  // highest word: 2 (1023 + PY R NCH + PZ (W - 1) + PY) + 1 < kProbeWords
  static_assert(2 * (1023 + PY * R * NCH + PZ * (W - 1) + PY) + 1 < kProbeWords, "probe tile");
  __shared__ int tile[kProbeWords];
  for (int i = threadIdx.x; i < kProbeWords; i += blockDim.x) tile[i] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, q = lane & 15, hp = lane >> 4;
  const int gl = q % WV, r = q / WV;
  const unsigned tile_addr = (unsigned)__cvta_generic_to_shared(tile);
  const unsigned lane_off = 4u * (2u * (gl + PY * r) + hp);
  const unsigned seed = blockIdx.x * 977u + (threadIdx.x >> 5);
  for (int it = 0; it < iters; ++it) {
    const unsigned base = probe_hash(seed + it * 131u) & 1023u;
    const unsigned a = tile_addr + 8u * base + lane_off;
#pragma unroll
    for (int ch = 0; ch < NCH; ++ch)
#pragma unroll
      for (int iz = 0; iz < W; ++iz)
        asm volatile("red.shared.add.s32 [%0], %1;" ::"r"(a + 8u * (ch * R * PY + iz * PZ)),
                     "r"(1)
                     : "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) sink[blockIdx.x] = tile[lane] + tile[100];
}

template <int W>
cudaError_t run_probe(cudaStream_t s, int blocks, int iters, int* sink, cudaEvent_t e0,
                      cudaEvent_t e1, float* ms) {
  cudaEventRecord(e0, s);
  smem_row_probe_kernel<W><<<blocks, 256, 0, s>>>(iters, sink);
  cudaEventRecord(e1, s);
  cudaError_t e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
  return e;
}

}  // namespace

// Complex cell updates per second over the whole GPU with the access pattern
// of the row-owned spread at kernel width w (4..8): each point's w^3 updates
// as 2 ceil(w / R) w int32 shared-memory atomic instructions.  Synchronises
// `stream`.  Returns 0, -1 for bad arguments, or the CUDA error code.
extern "C" __attribute__((visibility("default"))) int gbn_probe_smem_atomics(
    void* stream, int w, double* updates_per_s) {
  if (!updates_per_s || w < 4 || w > 8) return -1;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = 3 * sms, iters = 2000;  // three 256-thread blocks per SM, as the spread
  int* sink = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMallocAsync(&sink, blocks * sizeof(int), s);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float best = 0.f;
  for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
    float ms = 0.f;
    switch (w) {
      case 4:
        e = run_probe<4>(s, blocks, iters, sink, e0, e1, &ms);
        break;
      case 5:
        e = run_probe<5>(s, blocks, iters, sink, e0, e1, &ms);
        break;
      case 6:
        e = run_probe<6>(s, blocks, iters, sink, e0, e1, &ms);
        break;
      case 7:
        e = run_probe<7>(s, blocks, iters, sink, e0, e1, &ms);
        break;
      default:
        e = run_probe<8>(s, blocks, iters, sink, e0, e1, &ms);
        break;
    }
    if (rep > 0 && (best == 0.f || ms < best)) best = ms;  // first launch is a warm-up
  }
  if (sink) cudaFreeAsync(sink, s);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) return (int)e;
  const double updates = (double)blocks * (256 / 32) * iters * w * w * w;
  *updates_per_s = best > 0.f ? updates / (best * 1e-3) : 0.0;
  return 0;
}
