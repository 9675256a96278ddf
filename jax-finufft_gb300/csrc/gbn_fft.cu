// gbn_fft.cu -- pruned FP32 FFTs of power-of-two fine grids with the
// deconvolution fused in.
//
// Replaces, for FP32 plans whose fine-grid axes all have 128, 256, 512 or
// 1024 cells, the cuFFT transform and the separate deconvolution kernels of
// the type-1 and type-2 execute (cuFINUFFT's fft + deconvolve stages, which
// lib/kernels.cc.cu:57-80 reaches through cufinufft_execute).  Each axis is
// one pass over HBM in which a block holds whole lines (a row along x, or
// eight adjacent columns along y or z) and transforms them in registers and
// shared memory: Stockham radix-8 passes (the last one radix 2 or 4 where
// log2 N is not a multiple of 3), twiddles from a per-axis table.
//
// Only the mode region matters on one side of each transform, so
//   type 2 (modes -> grid): x pass reads the modes times 1/psihat and writes
//     the mode rows of the mode planes (no zero padding is stored: loads of
//     cells outside the mode region are skipped and count as zero); y pass
//     over the mode planes reads only mode rows; z pass reads only mode planes
//     and writes every plane.
//   type 1 (grid -> modes): z pass reads every plane and writes only mode
//     planes; y pass over those writes only mode rows; x pass reads the mode
//     rows and writes the modes times 1/psihat straight into the output.
// At 512^3 this moves 2.8 GB per transform against cuFFT's 3D transform plus
// a separate deconvolution (which also writes the zero padding).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "gbn_common.cuh"

namespace gbn {

namespace {

__device__ __forceinline__ float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 c_mul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * (SIGN i)
template <int SIGN>
__device__ __forceinline__ float2 c_muli(float2 a) {
  return SIGN > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// DFT_R in place: A_q = sum_r a_r w^(r q), w = exp(SIGN 2 pi i / R).
template <int SIGN>
__device__ __forceinline__ void dft2(float2* a) {
  const float2 t = a[0];
  a[0] = c_add(t, a[1]);
  a[1] = c_sub(t, a[1]);
}
template <int SIGN>
__device__ __forceinline__ void dft4(float2* z) {
  const float2 p0 = c_add(z[0], z[2]), p1 = c_sub(z[0], z[2]);
  const float2 p2 = c_add(z[1], z[3]), p3 = c_muli<SIGN>(c_sub(z[1], z[3]));
  z[0] = c_add(p0, p2);
  z[2] = c_sub(p0, p2);
  z[1] = c_add(p1, p3);
  z[3] = c_sub(p1, p3);
}
// radix-2 step on stride 4, twiddles w^r, then two DFT_4: X[2q] from the
// sums, X[2q+1] from the twiddled differences.
template <int SIGN>
__device__ __forceinline__ void dft8(float2* a) {
  const float h = 0.70710678118654752440f;
  float2 u[4], v[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    u[r] = c_add(a[r], a[r + 4]);
    v[r] = c_sub(a[r], a[r + 4]);
  }
  v[1] = c_mul(v[1], make_float2(h, SIGN * h));
  v[2] = c_muli<SIGN>(v[2]);
  v[3] = c_mul(v[3], make_float2(-h, SIGN * h));
  dft4<SIGN>(u);
  dft4<SIGN>(v);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    a[2 * q] = u[q];
    a[2 * q + 1] = v[q];
  }
}
template <int R, int SIGN>
__device__ __forceinline__ void dft(float2* a) {
  if constexpr (R == 8)
    dft8<SIGN>(a);
  else if constexpr (R == 4)
    dft4<SIGN>(a);
  else
    dft2<SIGN>(a);
}

// Radix of pass p for a line of N cells; every thread holds 8 elements, so
// a line takes N/8 threads (one radix-8 butterfly, two radix-4 or four
// radix-2 butterflies per thread and pass).
__host__ __device__ constexpr int fft_radix(int N, int p) {
  return N == 128 ? (p < 2 ? 8 : 2) : N == 256 ? (p < 2 ? 8 : 4) : N == 1024 ? (p < 3 ? 8 : 2) : 8;
}
__host__ __device__ constexpr int fft_npass(int N) { return N == 1024 ? 4 : 3; }

// Stockham passes P.. of one line.  Thread t < N/8 holds 8 elements: for
// pass radix R and span LS (product of the earlier radices), butterfly
// j = t + u N/8 (u < 8/R) takes x[j + r N/R], twiddles it by
// w_{LS R}^{r (j mod LS)} and writes y[(j / LS) LS R + j mod LS + q LS].
// Between passes the elements go through shared memory at index si(n).
// On entry a[] holds pass P's inputs; on exit the last pass's outputs, a[u R + q]
// being element t + u N/8 + q N/R of the result.  Every thread of the block
// must call this (it synchronises the block).
template <int N, int SIGN, int P, int LS, typename SIdx>
__device__ __forceinline__ void fft_passes(float2 (&a)[8], int t, float2* sm, const SIdx& si,
                                           const float2* __restrict__ tw) {
  constexpr int R = fft_radix(N, P);
  constexpr int L = LS * R;
#pragma unroll
  for (int u = 0; u < 8 / R; ++u) {
    const int j = t + u * (N / 8);
    if constexpr (LS > 1) {
      const int k = j & (LS - 1);
#pragma unroll
      for (int r = 1; r < R; ++r) {
        float2 w = __ldg(&tw[r * k * (N / L)]);
        if (SIGN < 0) w.y = -w.y;
        a[u * R + r] = c_mul(a[u * R + r], w);
      }
    }
    dft<R, SIGN>(&a[u * R]);
  }
  if constexpr (P + 1 < fft_npass(N)) {
    constexpr int R2 = fft_radix(N, P + 1);
#pragma unroll
    for (int u = 0; u < 8 / R; ++u) {
      const int j = t + u * (N / 8);
      const int base = (j / LS) * L + (j & (LS - 1));
#pragma unroll
      for (int q = 0; q < R; ++q) sm[si(base + q * LS)] = a[u * R + q];
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 8 / R2; ++u)
#pragma unroll
      for (int r = 0; r < R2; ++r) a[u * R2 + r] = sm[si(t + u * (N / 8) + r * (N / R2))];
    __syncthreads();
    fft_passes<N, SIGN, P + 1, L, SIdx>(a, t, sm, si, tw);
  }
}

// Element position of a[e] on entry (first pass inputs) and on exit.
template <int N>
__device__ __forceinline__ int in_pos(int t, int e) {
  constexpr int R = fft_radix(N, 0);
  return t + (e / R) * (N / 8) + (e % R) * (N / R);
}
template <int N>
__device__ __forceinline__ int out_pos(int t, int e) {
  constexpr int R = fft_radix(N, fft_npass(N) - 1);
  return t + (e / R) * (N / 8) + (e % R) * (N / R);
}

// Shared-memory index of element n of row c (x pass: rows contiguous, one
// pad cell per 8) and of column c (strided passes: 8 columns interleaved,
// 8 pad cells per 8 rows); both keep a warp's accesses to the minimum
// number of wavefronts for the two access patterns of the passes.
template <int N>
struct RowIdx {
  int base;
  __device__ __forceinline__ int operator()(int n) const { return base + n + (n >> 3); }
};
struct ColIdx {
  int c;
  __device__ __forceinline__ int operator()(int n) const { return n * 8 + c + (n >> 3) * 8; }
};

// Fine index g <-> mode index along one axis (modeord 0: k = i - N/2 order,
// 1: FFT order); fine_to_mode gives -1 outside the mode region.
__device__ __forceinline__ int mode_to_fine_f(int i, int N, int nf, int modeord) {
  const int k = modeord == 0 ? i - N / 2 : (i < (N + 1) / 2 ? i : i - N);
  return k < 0 ? k + nf : k;
}
__device__ __forceinline__ int fine_to_mode_f(int g, int N, int nf, int modeord) {
  int k;
  if (g <= (N - 1) / 2)
    k = g;
  else if (g >= nf - N / 2)
    k = g - nf;
  else
    return -1;
  if (modeord == 0) return k + N / 2;
  return k >= 0 ? k : k + N;
}

struct AxisSpec {
  int N[3];     // modes per axis
  int nf[3];    // fine cells per axis
  int modeord;
  // type-2 direction with E weighted grids per transform (fused gradient):
  // grid e of transform t is launch grid t*E + e and gets the modes times 1
  // (e < base) or times (a_re + i a_im) k along axis wdim[e]; E = base = 1
  // for a plain transform
  int E, base;
  int wdim[4];
  float a_re, a_im;
};

// Signed integer frequency of mode index i along an axis of N modes.
__device__ __forceinline__ int mode_freq_f(int i, int N, int modeord) {
  return modeord == 0 ? i - N / 2 : (i < (N + 1) / 2 ? i : i - N);
}

// x pass over mode rows.  Row r of the launch (r < M1*M2 per transform,
// blockIdx.y = transform) is mode row (i1, i2) = (r % M1, r / M1), fine row
// (g1, g2).  TO_GRID (type 2): the line is the modes of the row times
// 1/psihat (zero outside the mode region), transformed and stored into the
// fine row.  Otherwise (type 1): the fine row is transformed and its mode
// cells, times 1/psihat, stored into the output row.
template <int N, int SIGN, int DIM, bool TO_GRID, typename TD>
__global__ void __launch_bounds__(256)
    fft_x_kernel(AxisSpec ax, const float* __restrict__ p0, const float* __restrict__ p1,
                 const float* __restrict__ p2, const float2* __restrict__ tw, float2* fine,
                 cplx_t<TD>* modes, int64_t nftot, int64_t Ntot) {
  constexpr int T = N / 8;
  constexpr int B = 256 / T;  // rows per block
  extern __shared__ __align__(16) unsigned char fft_smem[];
  float2* sm = reinterpret_cast<float2*>(fft_smem);
  const int t = threadIdx.x % T, rb = threadIdx.x / T;
  const int M0 = ax.N[0], M1 = DIM > 1 ? ax.N[1] : 1, M2 = DIM > 2 ? ax.N[2] : 1;
  const int nrows = M1 * M2;
  const int row = blockIdx.x * B + rb;
  const bool live = row < nrows;
  const int i1 = live ? row % M1 : 0, i2 = live ? row / M1 : 0;
  const int g1 = DIM > 1 ? mode_to_fine_f(i1, M1, ax.nf[1], ax.modeord) : 0;
  const int g2 = DIM > 2 ? mode_to_fine_f(i2, M2, ax.nf[2], ax.modeord) : 0;
  float f12 = 1.f;
  if (live) {
    if (DIM > 1) f12 *= p1[i1];
    if (DIM > 2) f12 *= p2[i2];
  }
  const int64_t tr = blockIdx.y;
  float2* frow = fine + tr * nftot + ((int64_t)g2 * ax.nf[1] + g1) * N;
  // grid tr holds weighted grid we of transform tm (TO_GRID; E = 1 otherwise)
  const int64_t tm = TO_GRID ? tr / ax.E : tr;
  const int we = TO_GRID ? (int)(tr - tm * ax.E) : 0;
  cplx_t<TD>* mrow = modes + tm * Ntot + ((int64_t)i2 * M1 + i1) * M0;
  const bool weighted = TO_GRID && we >= ax.base;
  const int wd = weighted ? ax.wdim[we] : 0;
  float2 a[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int n = in_pos<N>(t, e);
    if constexpr (TO_GRID) {
      const int i0 = live ? fine_to_mode_f(n, M0, N, ax.modeord) : -1;
      a[e] = make_float2(0.f, 0.f);
      if (i0 >= 0) {
        const cplx_t<TD> v = mrow[i0];
        const float f = p0[i0] * f12;
        a[e] = make_float2((float)v.x * f, (float)v.y * f);
        if (weighted) {
          const float kk = (float)(wd == 0   ? mode_freq_f(i0, M0, ax.modeord)
                                   : wd == 1 ? mode_freq_f(i1, M1, ax.modeord)
                                             : mode_freq_f(i2, M2, ax.modeord));
          a[e] = c_mul(a[e], make_float2(ax.a_re * kk, ax.a_im * kk));
        }
      }
    } else {
      a[e] = live ? frow[n] : make_float2(0.f, 0.f);
    }
  }
  const RowIdx<N> si{rb * (N + N / 8)};
  fft_passes<N, SIGN, 0, 1>(a, t, sm, si, tw);
  if (!live) return;
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int k = out_pos<N>(t, e);
    if constexpr (TO_GRID) {
      frow[k] = a[e];
    } else {
      const int i0 = fine_to_mode_f(k, M0, N, ax.modeord);
      if (i0 >= 0) {
        const float f = p0[i0] * f12;
        cplx_t<TD> o;
        o.x = (TD)(a[e].x * f);
        o.y = (TD)(a[e].y * f);
        mrow[i0] = o;
      }
    }
  }
}

// Strided pass along an axis of N cells with element stride es: block
// (x group of 8 columns, line set p, transform) transforms 8 adjacent lines.
// Line set p selects the plane (z for a y pass, y for a z pass) through the
// pruned enumeration pl(p) = p < pl_lo ? p : p + pl_skip, stride ps.  Inputs
// outside [0, in_lo) u [N - in_hi, N) are zero and not loaded; outputs
// outside [0, out_lo) u [N - out_hi, N) are not stored.
template <int N, int SIGN>
__global__ void __launch_bounds__(8 * (N / 8))
    fft_col_kernel(float2* fine, int64_t nftot, int nx, int64_t es, int64_t ps, int pl_lo,
                   int pl_skip, int in_lo, int in_hi, int out_lo, int out_hi,
                   const float2* __restrict__ tw) {
  extern __shared__ __align__(16) unsigned char fft_smem[];
  float2* sm = reinterpret_cast<float2*>(fft_smem);
  const int c = threadIdx.x & 7, t = threadIdx.x >> 3;
  const int x = blockIdx.x * 8 + c;
  const bool live = x < nx;
  const int p = blockIdx.y;
  const int64_t plane = p < pl_lo ? p : p + pl_skip;
  float2* col = fine + (int64_t)blockIdx.z * nftot + plane * ps + x;
  float2 a[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int n = in_pos<N>(t, e);
    const bool in = live && (n < in_lo || n >= N - in_hi);
    a[e] = in ? col[n * es] : make_float2(0.f, 0.f);
  }
  const ColIdx si{c};
  fft_passes<N, SIGN, 0, 1>(a, t, sm, si, tw);
  if (!live) return;
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int k = out_pos<N>(t, e);
    if (k < out_lo || k >= N - out_hi) col[k * es] = a[e];
  }
}

size_t col_smem(int N) { return (size_t)(8 * N + N) * sizeof(float2); }
size_t row_smem(int N) { return (size_t)(256 / (N / 8)) * (N + N / 8) * sizeof(float2); }

template <int N, int SIGN>
cudaError_t launch_col(float2* fine, int64_t nftot, int nb, int nx, int64_t es, int64_t ps,
                       int nplanes, int pl_lo, int pl_skip, int in_lo, int in_hi, int out_lo,
                       int out_hi, const float2* tw, cudaStream_t s) {
  auto kern = fft_col_kernel<N, SIGN>;
  const size_t smem = col_smem(N);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid((unsigned)((nx + 7) / 8), (unsigned)nplanes, (unsigned)nb);
  kern<<<grid, N, smem, s>>>(fine, nftot, nx, es, ps, pl_lo, pl_skip, in_lo, in_hi, out_lo,
                             out_hi, tw);
  note_launch();
  return cudaGetLastError();
}

template <int SIGN>
cudaError_t launch_col_n(int N, float2* fine, int64_t nftot, int nb, int nx, int64_t es,
                         int64_t ps, int nplanes, int pl_lo, int pl_skip, int in_lo, int in_hi,
                         int out_lo, int out_hi, const float2* tw, cudaStream_t s) {
#define GBN_COL(NN)                                                                          \
  return launch_col<NN, SIGN>(fine, nftot, nb, nx, es, ps, nplanes, pl_lo, pl_skip, in_lo,   \
                              in_hi, out_lo, out_hi, tw, s);
  switch (N) {
    case 128:
      GBN_COL(128)
    case 256:
      GBN_COL(256)
    case 512:
      GBN_COL(512)
    default:
      GBN_COL(1024)
  }
#undef GBN_COL
}

template <int N, int SIGN, int DIM, bool TO_GRID, typename TD>
cudaError_t launch_row(const AxisSpec& ax, const float* const* phi, const float2* tw,
                       float2* fine, void* modes, int64_t nftot, int64_t Ntot, int nb,
                       cudaStream_t s) {
  auto kern = fft_x_kernel<N, SIGN, DIM, TO_GRID, TD>;
  const size_t smem = row_smem(N);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  constexpr int B = 256 / (N / 8);
  const int64_t nrows = (int64_t)(DIM > 1 ? ax.N[1] : 1) * (DIM > 2 ? ax.N[2] : 1);
  dim3 grid((unsigned)((nrows + B - 1) / B), (unsigned)nb);
  kern<<<grid, B * (N / 8), smem, s>>>(ax, phi[0], phi[1], phi[2], tw, fine,
                                       (cplx_t<TD>*)modes, nftot, Ntot);
  note_launch();
  return cudaGetLastError();
}

template <int SIGN, int DIM, bool TO_GRID, typename TD>
cudaError_t launch_row_n(const AxisSpec& ax, const float* const* phi, const float2* tw,
                         float2* fine, void* modes, int64_t nftot, int64_t Ntot, int nb,
                         cudaStream_t s) {
#define GBN_ROW(NN) \
  return launch_row<NN, SIGN, DIM, TO_GRID, TD>(ax, phi, tw, fine, modes, nftot, Ntot, nb, s);
  switch (ax.nf[0]) {
    case 128:
      GBN_ROW(128)
    case 256:
      GBN_ROW(256)
    case 512:
      GBN_ROW(512)
    default:
      GBN_ROW(1024)
  }
#undef GBN_ROW
}

template <bool TO_GRID, typename TD>
cudaError_t launch_row_any(int dim, int sign, const AxisSpec& ax, const float* const* phi,
                           const float2* tw, float2* fine, void* modes, int64_t nftot,
                           int64_t Ntot, int nb, cudaStream_t s) {
  if (sign > 0) {
    if (dim == 1) return launch_row_n<1, 1, TO_GRID, TD>(ax, phi, tw, fine, modes, nftot, Ntot, nb, s);
    if (dim == 2) return launch_row_n<1, 2, TO_GRID, TD>(ax, phi, tw, fine, modes, nftot, Ntot, nb, s);
    return launch_row_n<1, 3, TO_GRID, TD>(ax, phi, tw, fine, modes, nftot, Ntot, nb, s);
  }
  if (dim == 1) return launch_row_n<-1, 1, TO_GRID, TD>(ax, phi, tw, fine, modes, nftot, Ntot, nb, s);
  if (dim == 2) return launch_row_n<-1, 2, TO_GRID, TD>(ax, phi, tw, fine, modes, nftot, Ntot, nb, s);
  return launch_row_n<-1, 3, TO_GRID, TD>(ax, phi, tw, fine, modes, nftot, Ntot, nb, s);
}

cudaError_t launch_col_any(int sign, int N, float2* fine, int64_t nftot, int nb, int nx,
                           int64_t es, int64_t ps, int nplanes, int pl_lo, int pl_skip,
                           int in_lo, int in_hi, int out_lo, int out_hi, const float2* tw,
                           cudaStream_t s) {
  return sign > 0 ? launch_col_n<1>(N, fine, nftot, nb, nx, es, ps, nplanes, pl_lo, pl_skip,
                                     in_lo, in_hi, out_lo, out_hi, tw, s)
                  : launch_col_n<-1>(N, fine, nftot, nb, nx, es, ps, nplanes, pl_lo, pl_skip,
                                      in_lo, in_hi, out_lo, out_hi, tw, s);
}

}  // namespace

bool fft_pow2_supported(int dim, const int64_t* nf, int nb) {
  if (dim < 1 || dim > 3 || nb < 1 || nb > 65535) return false;
  for (int d = 0; d < dim; ++d)
    if (nf[d] != 128 && nf[d] != 256 && nf[d] != 512 && nf[d] != 1024) return false;
  return true;
}

void fft_pow2_twiddles(int64_t n, std::vector<float>& out) {
  out.resize((size_t)(2 * n));
  const double pi = 3.14159265358979323846264338327950288;
  for (int64_t m = 0; m < n; ++m) {
    const double a = 2.0 * pi * (double)m / (double)n;
    out[(size_t)(2 * m)] = (float)std::cos(a);
    out[(size_t)(2 * m + 1)] = (float)std::sin(a);
  }
}

// Mode region along one axis of nf cells with N modes: fine cells [0, lo)
// and [nf - hi, nf).
static void mode_span(int64_t N, int* lo, int* hi) {
  *lo = (int)((N - 1) / 2 + 1);
  *hi = (int)(N / 2);
}

template <typename TD>
cudaError_t launch_fft_type2(int dim, const int64_t* N, const int64_t* nf, int modeord,
                             const float* const* phi, const float2* const* tw,
                             const void* modes, void* fine, int nb, int sign, cudaStream_t s,
                             const FftWeights* wts) {
  AxisSpec ax;
  for (int d = 0; d < 3; ++d) {
    ax.N[d] = (int)N[d];
    ax.nf[d] = (int)nf[d];
  }
  ax.modeord = modeord;
  ax.E = 1;
  ax.base = 1;
  ax.wdim[0] = ax.wdim[1] = ax.wdim[2] = ax.wdim[3] = 0;
  ax.a_re = 1.f;
  ax.a_im = 0.f;
  if (wts) {
    if (wts->E < 1 || wts->E > 4 || wts->base < 0 || wts->base > wts->E) return cudaErrorInvalidValue;
    ax.E = wts->E;
    ax.base = wts->base;
    for (int e = 0; e < 4; ++e) ax.wdim[e] = wts->dims[e];
    ax.a_re = (float)wts->a_re;
    ax.a_im = (float)wts->a_im;
    nb *= wts->E;  // every weighted grid is a transform of its own from here on
  }
  if (nb > 65535) return cudaErrorInvalidValue;
  const int64_t nftot = nf[0] * nf[1] * nf[2], Ntot = N[0] * N[1] * N[2];
  float2* g = (float2*)fine;
  cudaError_t e = launch_row_any<true, TD>(dim, sign, ax, phi, tw[0], g, (void*)modes, nftot,
                                           Ntot, nb, s);
  if (e != cudaSuccess || dim == 1) return e;
  int lo1, hi1, lo2 = 1, hi2 = 0;
  mode_span(N[1], &lo1, &hi1);
  if (dim == 3) mode_span(N[2], &lo2, &hi2);
  // y over the mode planes (every plane in 2D), reading only mode rows
  const int nplanes = dim == 3 ? lo2 + hi2 : 1;
  e = launch_col_any(sign, (int)nf[1], g, nftot, nb, (int)nf[0], nf[0], nf[0] * nf[1], nplanes,
                     lo2, dim == 3 ? (int)nf[2] - lo2 - hi2 : 0, lo1, hi1, (int)nf[1], 0,
                     tw[1], s);
  if (e != cudaSuccess || dim == 2) return e;
  // z over every (y, x) column, reading only mode planes
  return launch_col_any(sign, (int)nf[2], g, nftot, nb, (int)nf[0], nf[0] * nf[1], nf[0],
                        (int)nf[1], (int)nf[1], 0, lo2, hi2, (int)nf[2], 0, tw[2], s);
}

template <typename TD>
cudaError_t launch_fft_type1(int dim, const int64_t* N, const int64_t* nf, int modeord,
                             const float* const* phi, const float2* const* tw, void* fine,
                             void* modes, int nb, int sign, cudaStream_t s) {
  AxisSpec ax;
  for (int d = 0; d < 3; ++d) {
    ax.N[d] = (int)N[d];
    ax.nf[d] = (int)nf[d];
  }
  ax.modeord = modeord;
  ax.E = 1;
  ax.base = 1;
  ax.wdim[0] = ax.wdim[1] = ax.wdim[2] = ax.wdim[3] = 0;
  ax.a_re = 1.f;
  ax.a_im = 0.f;
  const int64_t nftot = nf[0] * nf[1] * nf[2], Ntot = N[0] * N[1] * N[2];
  float2* g = (float2*)fine;
  cudaError_t e = cudaSuccess;
  int lo1 = 0, hi1 = 0, lo2 = 1, hi2 = 0;
  if (dim >= 2) mode_span(N[1], &lo1, &hi1);
  if (dim == 3) {
    mode_span(N[2], &lo2, &hi2);
    // z over every column, storing only mode planes
    e = launch_col_any(sign, (int)nf[2], g, nftot, nb, (int)nf[0], nf[0] * nf[1], nf[0],
                       (int)nf[1], (int)nf[1], 0, (int)nf[2], 0, lo2, hi2, tw[2], s);
    if (e != cudaSuccess) return e;
  }
  if (dim >= 2) {
    // y over the mode planes, storing only mode rows
    const int nplanes = dim == 3 ? lo2 + hi2 : 1;
    e = launch_col_any(sign, (int)nf[1], g, nftot, nb, (int)nf[0], nf[0], nf[0] * nf[1],
                       nplanes, lo2, dim == 3 ? (int)nf[2] - lo2 - hi2 : 0, (int)nf[1], 0, lo1,
                       hi1, tw[1], s);
    if (e != cudaSuccess) return e;
  }
  return launch_row_any<false, TD>(dim, sign, ax, phi, tw[0], g, modes, nftot, Ntot, nb, s);
}

template cudaError_t launch_fft_type2<float>(int, const int64_t*, const int64_t*, int,
                                             const float* const*, const float2* const*,
                                             const void*, void*, int, int, cudaStream_t,
                                             const FftWeights*);
template cudaError_t launch_fft_type2<double>(int, const int64_t*, const int64_t*, int,
                                              const float* const*, const float2* const*,
                                              const void*, void*, int, int, cudaStream_t,
                                              const FftWeights*);
template cudaError_t launch_fft_type1<float>(int, const int64_t*, const int64_t*, int,
                                             const float* const*, const float2* const*, void*,
                                             void*, int, int, cudaStream_t);
template cudaError_t launch_fft_type1<double>(int, const int64_t*, const int64_t*, int,
                                              const float* const*, const float2* const*, void*,
                                              void*, int, int, cudaStream_t);

}  // namespace gbn
