// gbn_noalloc.cu -- bin-sorting nonuniform points without allocating memory.
//
// Some callers cannot call cudaMalloc: code that runs where the host
// framework owns every device allocation (a plugin handed fixed buffers by
// its host, an embedded or real-time pipeline that reserves all memory up
// front, an allocator-free hook called between other work).  For them
// gbn_binsort_noalloc runs the point fold and bin sort of setpts without any
// allocation: the caller passes the points and the three output arrays, and
// the per-point ranks, folded records and scan partial sums live in one
// fixed array of device memory that belongs to this library.
//
// That array is a file-scope __device__ variable, so every GPU that loads
// the library holds its kNoallocBytes until the process exits.  Host code
// cannot use the array's name as a device address (in host code it names a
// host-side stand-in); every call looks the address up with
// cudaGetSymbolAddress on the current device.  Nothing is cached, so a
// device reset or a new context (the module loads again, possibly at another
// address) leaves no stale pointer; the first lookup after a load loads the
// module, which is why the first call per device goes before stream capture.
// Every call shares the array and it keeps the previous call's contents, so
// whatever must start at zero is cleared by the call itself, and two calls
// whose work overlaps on the GPU (different streams, or the same array on
// the same device concurrently) race on it.
#include <cuda_runtime.h>

#include <string>

#include "../../include/gbnufft.h"
#include "gbn_common.cuh"

namespace gbn {

namespace {

constexpr int64_t kMaxPoints = GBN_NOALLOC_MAX_POINTS;
constexpr int64_t kMaxBins = GBN_NOALLOC_MAX_BINS;
constexpr size_t kRankBytes = kMaxPoints * sizeof(int);
constexpr size_t kRecBytes = kMaxPoints * sizeof(PtRec<double, 3>);  // widest record
constexpr size_t kStartBytes = kMaxBins * sizeof(int);
constexpr size_t kNoallocBytes = (size_t)GBN_NOALLOC_SCRATCH_BYTES;
static_assert(kRankBytes + kRecBytes + kStartBytes + 64 * 1024 <= kNoallocBytes,
              "scratch array too small for the stated limits");

static __device__ __align__(256) unsigned char g_scratch[kNoallocBytes];

// Address of g_scratch in the current device's context.
cudaError_t scratch_on_current_device(void** out) { return cudaGetSymbolAddress(out, g_scratch); }

__global__ void noalloc_scatter_kernel(int64_t M, const int* __restrict__ bins,
                                       const int* __restrict__ rank,
                                       const int* __restrict__ bin_start,
                                       int* __restrict__ perm) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < M) perm[bin_start[bins[j]] + rank[j]] = (int)j;
}

template <typename TX>
cudaError_t binsort(const Geom& g, int64_t M, const TX* x, const TX* y, const TX* z, int* bins,
                    int* counts, int* perm, unsigned char* scratch, cudaStream_t s) {
  SortState st{};
  st.pt_bin = bins;
  st.bin_count = counts;
  st.key_count = counts;  // plain bin order
  st.pt_rank = reinterpret_cast<int*>(scratch);
  st.recs_in = scratch + kRankBytes;
  int* bin_start = reinterpret_cast<int*>(scratch + kRankBytes + kRecBytes);
  int* scan_tmp = reinterpret_cast<int*>(scratch + kRankBytes + kRecBytes + kStartBytes);
  cudaError_t e = cudaMemsetAsync(counts, 0, (size_t)g.nbins * sizeof(int), s);
  if (e != cudaSuccess) return e;
  FoldSpec fs{};
  fs.mode = 0;
  if (sizeof(TX) == 4)
    e = launch_fold<float, float>(g, fs, M, (const float*)x, (const float*)y, (const float*)z,
                                  st, s);
  else
    e = launch_fold<double, double>(g, fs, M, (const double*)x, (const double*)y,
                                    (const double*)z, st, s);
  if (e != cudaSuccess) return e;
  e = launch_scan(counts, bin_start, g.nbins, scan_tmp, s);
  if (e != cudaSuccess) return e;
  if (M > 0) {
    noalloc_scatter_kernel<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(M, bins, st.pt_rank,
                                                                       bin_start, perm);
    note_launch();
  }
  return cudaGetLastError();
}

}  // namespace

}  // namespace gbn

extern "C" int gbn_binsort_noalloc(void* stream, int dim, int single, int64_t M, const void* x,
                                   const void* y, const void* z, const int64_t* nf,
                                   const int* binsize, int w, int* bins, int* counts, int* perm) {
  using namespace gbn;
  if (dim < 1 || dim > 3) return set_error(GBN_ERR_ARGS, "gbn_binsort_noalloc: dim must be 1..3");
  if (!nf || !binsize) return set_error(GBN_ERR_ARGS, "gbn_binsort_noalloc: NULL nf or binsize");
  if (M < 0 || M > kMaxPoints)
    return set_error(GBN_ERR_ARGS, "gbn_binsort_noalloc: M = " + std::to_string(M) +
                                       " exceeds the limit of " + std::to_string(kMaxPoints) +
                                       " points (GBN_NOALLOC_MAX_POINTS)");
  if (w < 2 || w > kMaxW)
    return set_error(GBN_ERR_ARGS, "gbn_binsort_noalloc: kernel width w must be 2..16");
  Geom g{};
  g.dim = dim;
  g.w = w;
  g.nbins = 1;
  g.maxsub = 1;
  for (int d = 0; d < 3; ++d) {
    g.nf[d] = 1;
    g.bs[d] = 1;
    g.nb[d] = 1;
    if (d < dim) {
      if (nf[d] < 2 * w || nf[d] > (int64_t)INT32_MAX || binsize[d] < 1)
        return set_error(GBN_ERR_ARGS, "gbn_binsort_noalloc: need 2w <= nf < 2^31 and binsize >= 1");
      g.nf[d] = nf[d];
      g.bs[d] = binsize[d];
      g.nb[d] = (int)((nf[d] + binsize[d] - 1) / binsize[d]);
      g.nbins *= g.nb[d];
    }
  }
  if (g.nbins > kMaxBins)
    return set_error(GBN_ERR_ARGS, "gbn_binsort_noalloc: " + std::to_string(g.nbins) +
                                       " bins exceed the limit of " + std::to_string(kMaxBins) +
                                       " (GBN_NOALLOC_MAX_BINS)");
  if (M > 0 && (!x || (dim > 1 && !y) || (dim > 2 && !z) || !bins || !perm))
    return set_error(GBN_ERR_ARGS, "gbn_binsort_noalloc: NULL point or output array");
  if (!counts) return set_error(GBN_ERR_ARGS, "gbn_binsort_noalloc: NULL counts");
  void* scratch = nullptr;
  cudaError_t e = scratch_on_current_device(&scratch);
  if (e != cudaSuccess)
    return set_error(GBN_ERR_CUDA, std::string("gbn_binsort_noalloc: scratch lookup failed: ") +
                                       cudaGetErrorString(e));
  cudaStream_t s = (cudaStream_t)stream;
  e = single ? binsort<float>(g, M, (const float*)x, (const float*)y, (const float*)z, bins,
                              counts, perm, (unsigned char*)scratch, s)
             : binsort<double>(g, M, (const double*)x, (const double*)y, (const double*)z,
                               bins, counts, perm, (unsigned char*)scratch, s);
  if (e != cudaSuccess)
    return set_error(GBN_ERR_CUDA, std::string("gbn_binsort_noalloc: ") + cudaGetErrorString(e));
  return GBN_OK;
}
