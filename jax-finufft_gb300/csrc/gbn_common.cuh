// gbn_common.cuh -- types shared by the NUFFT kernels and the host plan code.
//
// Data layout in HBM (all row-major, dimension 0 = "x" fastest, the backend
// order of src/jax_finufft/lowering.py:96-105):
//   fine grid      (batch, nf2, nf1, nf0) complex in the compute precision TC
//   sorted points  PtRec<TC, DIM>[M]: per point the offset delta in [0,1) and
//                  the first grid index i0 of its w-wide support, per axis;
//                  ordered by bin (counting sort), with perm[] mapping sorted
//                  position -> input index
//   bins           bin_count / bin_start over nb0*nb1*nb2 bins of bs0*bs1*bs2
//                  cells; subproblems (sub_bin, sub_off) split each bin into
//                  chunks of at most maxsub points
#pragma once

#include <cuda.h>  // CUtensorMap (a plain struct; the encoder is resolved at run time)
#include <cuda_runtime.h>

#include <cmath>

#include <cstdint>
#include <string>
#include <vector>

namespace gbn {

constexpr int kMaxW = 16;       // widest kernel supported
constexpr int kThreads = 256;   // threads per block of the point kernels

template <typename T>
struct Cplx;
template <>
struct Cplx<float> {
  using type = float2;
};
template <>
struct Cplx<double> {
  using type = double2;
};
template <typename T>
using cplx_t = typename Cplx<T>::type;

// One nonuniform point after folding: offsets and grid starts per axis.
// Aligned to 16 bytes when its natural size is a multiple of 16, or when it
// is 24 bytes (FP32 in 3D, padded to one 32-byte sector: the bin-order
// scatter's random stores then write whole sectors with two 16-byte
// accesses), else to 8, so records move with 8/16-byte accesses instead of
// 4-byte ones.
template <typename T, int DIM>
struct alignas((sizeof(T) * DIM + 4 * DIM) % 16 == 0 || (sizeof(T) * DIM + 4 * DIM) == 24
                   ? 16
                   : 8) PtRec {
  T d[DIM];
  int i[DIM];
};

// Spreading-grid and bin geometry.
struct Geom {
  int dim;
  int w;
  int64_t nf[3];
  int bs[3];
  int nb[3];
  int64_t nbins;
  int maxsub;
  int stash;  // spread: a subproblem's strengths are staged in shared memory after the tile
  int rows;   // sort keys per bin: > 1 orders a bin's points by tile row (y, z), 0/1 by bin
  int coarse_round;  // FP32 fixed-point spread: tolerance >= 1e-5 allows 2^22-bounded rounding
};

// Shared-memory tile of one bin: bs + w - 1 cells per axis from the bin's
// first grid start, except along x, where the tile starts on the even cell at
// or below it and spans an even number of cells (one or two more): a TMA copy
// of a float2 grid needs 16-byte aligned x offsets and extents.
__host__ __device__ inline int tile_x(int bs0, int w) { return (bs0 + w + 1) & ~1; }
__host__ __device__ inline int64_t tile_cells(int dim, const int* bs, int w) {
  int64_t n = tile_x(bs[0], w);
  for (int d = 1; d < dim; ++d) n *= bs[d] + w - 1;
  return n;
}

// Shared memory of one shared-memory spread block: per transform an
// accumulator tile (two 4-byte integers per cell in FP32, two doubles in
// FP64) padded to 128 bytes -- the alignment a bulk tensor copy needs for its
// shared-memory side -- and, with g.stash, the subproblem's strengths in the
// compute precision.
__host__ __device__ inline size_t spread_tile_bytes(int dim, const int* bs, int w, bool single) {
  return ((size_t)tile_cells(dim, bs, w) * 2 * (single ? 4 : 8) + 127) & ~(size_t)127;
}
__host__ __device__ inline size_t spread_smem_bytes(int dim, const int* bs, int w, bool single,
                                                    int maxsub, bool stash) {
  return spread_tile_bytes(dim, bs, w, single) +
         (stash ? (size_t)maxsub * 2 * (single ? 4 : 8) : 0);
}

// Shared memory of one interpolation tile (a complex per cell), padded to 128
// bytes so that consecutive tiles of a multi-grid block stay TMA-aligned.
__host__ __device__ inline size_t interp_tile_bytes(int dim, const int* bs, int w, bool single) {
  return ((size_t)tile_cells(dim, bs, w) * 2 * (single ? 4 : 8) + 127) & ~(size_t)127;
}

// How points map onto the grid: mode 0 folds periodically (types 1/2),
// mode 1 rescales (type-3 sources): X = (x - center)*scale + nf/2.
struct FoldSpec {
  int mode;
  double center[3];
  double scale[3];
  double nf_d[3];  // (double)nf per axis, filled by launch_fold
  double hw;       // w / 2, filled by launch_fold
  // integer fast path of mode 0 (FP32 coordinates), filled by launch_fold:
  // 1/(2 pi) in FP64 as kmant * 2^kexp, and ceil(log2 nf) per axis
  unsigned long long kmant;
  int kexp;
  int lnf[3];
  unsigned bs_mul[3];  // floor(2^32 / bs) per axis (bin index by multiply-high)
};

// Kernel evaluation: piecewise Horner coefficients coef[piece*(deg+1)+n]
// (device memory, compute precision) or the direct formula when meth == 0.
template <typename T>
struct KerSpec {
  const T* coef;
  int deg;
  int meth;
  T beta;
  int shape;   // GBN_KERNEL_ES or GBN_KERNEL_KB (direct formula when meth == 0)
  T inv_i0b;   // 1 / I0(beta) for the Kaiser-Bessel shape
};

// Modified Bessel function I0 by its power series sum_k ((x/2)^2k / (k!)^2):
// every term is positive, so the sum keeps full relative precision (host).
inline double bessel_i0(double x) {
  const double q = 0.25 * x * x;
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 500; ++k) {
    term *= q / ((double)k * (double)k);
    sum += term;
    if (term < 1e-17 * sum) break;
  }
  return sum;
}

// Kernel shape as a function of s = sqrt(1 - z^2) in [0, 1], z = 2t/w
// (host): exp(beta (s - 1)) for the exponential of semicircle, I0(beta s) /
// I0(beta) for Kaiser-Bessel.
inline double kernel_of_s(int shape, double beta, double s) {
  if (shape == 1) return bessel_i0(beta * s) / bessel_i0(beta);
  return std::exp(beta * (s - 1.0));
}

// Device-side sort state produced by setpts.
struct SortState {
  int* pt_bin;     // [M] sort key of each input point: bin * rows + row in bin (rows > 1), or bin
  int* key_count;  // [nbins * rows] points per key (the bin counts themselves when rows <= 1)
  int* key_start;  // [nbins * rows] exclusive scan of key_count
  int* pt_rank;    // [M] rank inside its bin
  int* bin_count;  // [nbins]
  int* bin_start;  // [nbins] exclusive scan of bin_count
  int* perm;       // [M] sorted position -> input index
  int* sub_count;  // [nbins] subproblems per bin
  int* sub_start;  // [nbins] exclusive scan of sub_count
  int* sub_bin;    // [max_sub] bin of each subproblem
  int* sub_off;    // [max_sub] first point (within its bin) of each subproblem
  int* n_sub;      // [1] number of subproblems
  void* recs;      // [M] PtRec in sorted order
  void* recs_in;   // [M] PtRec in input order (scratch)
  int* scan_tmp;   // scan scratch
  int64_t max_sub; // capacity of sub_bin/sub_off
};

// Count of kernels this library has launched (process-wide, all threads);
// every launcher adds the launches it makes.  Read through gbn_launch_count().
void note_launch(int n = 1);

// Record msg as the calling thread's last error (read by gbn_last_error())
// and return code.
int set_error(int code, const std::string& msg);

// ---------------------------------------------------------------------------
// Launchers (defined in the .cu files, called by the host plan code).
// TX = coordinate type as given by the caller, TC = compute precision,
// TD = data precision of strengths / modes.
// ---------------------------------------------------------------------------

// Fold points, count bins, write per-point records in input order.
template <typename TX, typename TC>
cudaError_t launch_fold(const Geom& g, const FoldSpec& fs, int64_t M, const TX* x, const TX* y,
                        const TX* z, SortState& st, cudaStream_t s);

// Exclusive scan of n ints (in may equal out); tmp needs scan_tmp_ints(n).
int64_t scan_tmp_ints(int64_t n);
cudaError_t launch_scan(const int* in, int* out, int64_t n, int* tmp, cudaStream_t s);

// Scatter records into bin order, build the subproblem list.
template <typename TC>
cudaError_t launch_sort_finish(const Geom& g, int64_t M, SortState& st, bool sorted,
                               cudaStream_t s);

// Spread ntr transforms: c (ntr, M) data precision -> fine (ntr, nf) compute precision.
// method 1 = global atomics per update, 2 = shared-memory subproblems.
// tmap (optional, FP32 compute, method 2): a TMA map of the ntr fine grids
// from tile_tensor_map; interior tiles are then added to the grid with one
// bulk tensor reduce-add (spread) or staged with one bulk tensor copy
// (interp) instead of per-cell loops.
template <typename TC, typename TD>
cudaError_t launch_spread(const Geom& g, const KerSpec<TC>& ks, int method, int64_t M,
                          const SortState& st, const void* c, void* fine, int ntr,
                          cudaStream_t s, const CUtensorMap* tmap = nullptr);

// Outputs of the fused gradient gather.
template <typename TD>
struct GradOut {
  const cplx_t<TD>* w;  // mode 0: strengths c (ntr, M); mode 1: cotangent g (ntr, M)
  cplx_t<TD>* out_c;    // mode 0 with base: gathered grid 0 (ntr, M), or null
  TD* gx[3];            // coordinate gradients per axis (M), or null
};

// Shared-memory fused gradient gather over ntr*E grids (the interp kernel's
// block with a gradient epilogue); tmap as for launch_interp over the grids.
template <typename TC, typename TD>
cudaError_t launch_interp_grad_sm(const Geom& g, const KerSpec<TC>& ks, int64_t M,
                                  const SortState& st, const void* grids, int ntr, int E,
                                  int mode, int iflag, int base, const int* dims,
                                  const GradOut<TD>& go, const CUtensorMap* tmap,
                                  cudaStream_t s);

// Encode a TMA map over nb float2 fine grids of geometry g (rank = dim:
// x as 2*nf0 floats, the last axis stacked over the nb grids) whose box is
// one bin tile.  False (and no map) when TMA does not apply: 1D, a box
// extent above 256 elements, or no driver entry point.
bool tile_tensor_map(const Geom& g, const void* grid, int nb, CUtensorMap* out);

// Number of bounded waits in the point kernels that gave up (a wait that
// should take microseconds); 0 in a healthy run.  reset clears the count.
cudaError_t read_wait_timeouts(unsigned* out, bool reset);

// A bounded wait that gave up also raises a word of mapped pinned host
// memory of its device, which the host reads without synchronising.
// wait_flag_setup: allocate and publish that word for the current device
// (once per device; plan and batch creation call it).  wait_flag_take: true
// if it was raised on the current device since the last take, and clears
// it.  wait_flag_raise: raise it from the host (test hook, as a kernel would).
cudaError_t wait_flag_setup();
bool wait_flag_take();
void wait_flag_raise();
// The second word of that memory: type-3 points found outside the extents a
// caller declared (gbn_set_t3_extents).  extent_flag_device: its device
// pointer for the check kernel (null before setup); extent_flag_take: true
// if raised on the current device since the last take, and clears it.
unsigned* extent_flag_device();
bool extent_flag_take();

// Raise *flag (mapped host memory) if any finite coordinate of the n points
// lies outside [lo[d], hi[d]] on an axis d < dim.
template <typename TX>
cudaError_t launch_extent_check(int dim, int64_t n, const TX* const* a, const double* lo,
                                const double* hi, unsigned* flag, cudaStream_t s);

// Type-3 gradient request: the outer gather of the adjoint also
// differentiates along the sources (interp_t3grad_kernel).  c: forward
// strengths (ntr, M, data precision) or null; pre: pre-phase factors (M,
// compute precision); grad_c: strength gradient (ntr, M) or null; gx: per
// backend axis M reals (data precision, accumulated) or null; D, scale: the
// plan's target centres and source scales per backend axis; t0: first
// transform of the launch in the c/grad_c arrays.
struct T3Grad {
  const void* c;
  const void* pre;
  void* grad_c;
  void* gx[3];
  double D[3], scale[3];
  int iflag, t0;
};
template <typename TC, typename TD>
cudaError_t launch_interp_t3grad(const Geom& g, const KerSpec<TC>& ks, int64_t M,
                                 const SortState& st, const void* fine, int nb,
                                 const T3Grad& tg, cudaStream_t s,
                                 const CUtensorMap* tmap = nullptr);

// Interpolate ntr transforms: fine -> c (ntr, M).
template <typename TC, typename TD>
cudaError_t launch_interp(const Geom& g, const KerSpec<TC>& ks, int method, int64_t M,
                          const SortState& st, const void* fine, void* c, int ntr,
                          cudaStream_t s, const CUtensorMap* tmap = nullptr);

// The library's pruned FP32 FFT for power-of-two fine grids (gbn_fft.cu):
// applicability, the twiddle table exp(2 pi i m / n) (n cos/sin pairs), and
// the two directions with the deconvolution fused -- type 2 reads the modes
// (TD) and leaves the transformed fine grid; type 1 reads the fine grid and
// writes the modes.  phi: 1/psihat per axis; tw: twiddles per axis.
bool fft_pow2_supported(int dim, const int64_t* nf, int nb);
// Weighted grids of the fused gradient for launch_fft_type2: E grids per
// transform, grid e the deconvolved modes times 1 (e < base) or times
// (a_re + i a_im) k along axis dims[e] (k the signed integer frequency).
struct FftWeights {
  int E, base;
  int dims[4];
  double a_re, a_im;
};
void fft_pow2_twiddles(int64_t n, std::vector<float>& out);
template <typename TD>
cudaError_t launch_fft_type2(int dim, const int64_t* N, const int64_t* nf, int modeord,
                             const float* const* phi, const float2* const* tw,
                             const void* modes, void* fine, int nb, int sign, cudaStream_t s,
                             const FftWeights* wts = nullptr);
template <typename TD>
cudaError_t launch_fft_type1(int dim, const int64_t* N, const int64_t* nf, int modeord,
                             const float* const* phi, const float2* const* tw, void* fine,
                             void* modes, int nb, int sign, cudaStream_t s);

// Type-1 deconvolution + mode reorder: fine (ntr, nf) -> out (ntr, N).
// phi[d] holds 1/psihat for each output index along axis d.
template <typename TC, typename TD>
cudaError_t launch_deconv1(int dim, const int64_t* N, const int64_t* nf, int modeord,
                           const TC* const* phi, const void* fine, void* out, int ntr,
                           cudaStream_t s);

// Type-2 pre-correction + zero padding: in (ntr, N) -> fine (ntr, nf), every
// fine cell written.
template <typename TC, typename TD>
cudaError_t launch_deconv2(int dim, const int64_t* N, const int64_t* nf, int modeord,
                           const TC* const* phi, const void* in, void* fine, int ntr,
                           cudaStream_t s);

// Type 3: min/max of each coordinate array (out: 2 doubles per array).
template <typename TX>
cudaError_t launch_minmax(const TX* const* arrs, int narr, int64_t n, double* out,
                          cudaStream_t s);

// Type 3: tau = (s - center) / scale per axis into double arrays.
template <typename TX>
cudaError_t launch_t3_targets(int dim, int64_t N, const TX* const* s, const double* center,
                              const double* scale, double* const* tau, cudaStream_t s_);

// Type 3: per-point pre-phase exp(iflag*i*sum_d cs_d*(x_d - cx_d)) (compute precision).
template <typename TX, typename TC>
cudaError_t launch_t3_prephase_factors(int dim, int64_t M, const TX* const* x, const double* cx,
                                       const double* cs, int iflag, void* fac, cudaStream_t s);

// Type 3: per-target post factor exp(iflag*i*sum_d cx_d*s_d) / prod_d psihat(tau_d).
// With tau_max > 0 (a bound on |tau|), psihat comes from a piecewise
// Chebyshev fit checked on the host against the quadrature (relative 1e-14
// in FP64, 1e-9 in FP32), else from the quadrature per target.
// A fitted psihat table kept on the device across setpts calls of a type-3
// plan: refitted on the host and uploaded only when the kernel changes or
// the |tau| bound grows past the one it was fitted for, so that later setpts
// calls skip the fit (and, with declared extents, make no host copy and can
// be captured into a CUDA graph).  dev is freed by the owner (cudaFree).
struct T3PsihatCache {
  double* dev = nullptr;
  size_t cap = 0;  // doubles allocated at dev
  bool fitted = false;
  double tau_max = -1.0, beta = 0.0, h = 0.0;
  int w = 0, shape = -1, single = -1, P = 0;
};

template <typename TX, typename TC>
cudaError_t launch_t3_post_factors(int dim, int64_t N, const TX* const* sx, const double* cx,
                                   const double* const* tau, int iflag, int w, double beta,
                                   int shape,
                                   void* fac, cudaStream_t s, double tau_max = 0.0,
                                   T3PsihatCache* cache = nullptr);

// Gradient grids: for every transform, E fine grids from its modes `in`
// (ntr, N): grid e < base holds mode/psihat, grid e >= base holds
// (a_re + i a_im) * k_{dims[e]} * mode/psihat, with k the integer frequency
// along backend axis dims[e].  Layout (t*E + e)*nftot + cell.
template <typename TC, typename TD>
cudaError_t launch_deconv2w(int dim, const int64_t* N, const int64_t* nf, int modeord,
                            const TC* const* phi, const void* in, void* grids, int ntr, int E,
                            int base, const int* dims, double a_re, double a_im, cudaStream_t s);

// Gather all E grids of every transform at each point with shared kernel
// weights and combine them into gradients (see gbn_grad.cu): mode 0 = the
// type-1 gradient (w = strengths; grid 0 -> out_c when base = 1), mode 1 =
// the type-2 coordinate gradient (w = output cotangent).  gx[d] (M reals,
// may be null, zeroed by the caller) receives the gradient.  tmap: a TMA map
// of the ntr*E grids for the shared-memory gather (or null).
template <typename TC, typename TD>
cudaError_t launch_interp_grad(const Geom& g, const KerSpec<TC>& ks, int64_t M,
                               const SortState& st, const void* grids, int ntr, int E, int mode,
                               int iflag, int base, const int* dims, const void* w, void* out_c,
                               void* const* gx, bool shared, cudaStream_t s,
                               const CUtensorMap* tmap = nullptr);

// One problem of a batched plan, as the work-queue kernels see it: its
// geometry, kernel, sorted points, and where its strengths/values (T, M)
// and its T fine grids live inside the packed arrays.
template <typename TC>
struct BatchProb {
  Geom g;
  KerSpec<TC> ks;
  int64_t M;
  const void* recs;
  const int* sub_bin;
  const int* sub_off;
  const int* n_sub;
  const int* bin_start;
  const int* bin_count;
  const int* perm;
  int64_t c_off;     // element offset of the problem's (T, M) block
  int64_t grid_off;  // element offset of its T grids in the arena
  int64_t nftot;
};

// item_start[k] = T * sum_{i<k} n_sub_i for k = 0..K (device, one block);
// T here is the number of items per subproblem.
template <typename TC>
cudaError_t launch_item_prefix(const BatchProb<TC>* probs, int K, int T, int64_t* item_start,
                               cudaStream_t s);

// Persistent spread/interp over every (problem, subproblem, transform) item
// of a batch, pulled from one atomic counter (reset by the caller).
// group = lanes per point (6, 8 or 16, covering the widest kernel); the
// spread takes tb transforms per item (item_start counted in groups of tb)
// and smem1 = one transform's shared memory.
template <typename TC, typename TD>
cudaError_t launch_spread_queue(int dim, int group, int tb, const BatchProb<TC>* probs, int K,
                                const int64_t* item_start, int* counter, int T, const void* c,
                                void* arena, size_t smem1, cudaStream_t s);
template <typename TC, typename TD>
cudaError_t launch_interp_queue(int dim, int group, const BatchProb<TC>* probs, int K,
                                const int64_t* item_start, int* counter, int T,
                                const void* arena, void* c, size_t smem, cudaStream_t s);

// out[t, j] = in[t, j] * fac[j] (complex; conj(fac[j]) with conj), ntr
// transforms of length n.
template <typename TI, typename TO, typename TF>
cudaError_t launch_cmul(int64_t n, int ntr, const void* in, const void* fac, void* out,
                        cudaStream_t s, bool conj = false);

}  // namespace gbn
