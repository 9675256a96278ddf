// gbn_setpts.cu -- point folding and bin sort (setpts), deconvolution and
// mode reordering, and the type-3 phase kernels.
//
// These kernels replace the setpts stage and the deconvolve stage of the
// vendored cuFINUFFT that lib/cufinufft_wrapper.cc:63-89 calls (per
// lib/kernels.cc.cu:57-80).  All HBM-bound; each reads and writes its arrays
// once with coalesced accesses.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include <cstdint>
#include <cstring>

#include "gbn_common.cuh"
#include "gbn_fold.cuh"

namespace gbn {

namespace {

constexpr double kInv2Pi = 0.159154943091895335768883763372514362;

// Grid coordinate of a point minus w/2, i.e. s = X - w/2 with X the point's
// position in fine-grid cells.  Periodic fold (mode 0): t = x/(2 pi),
// f = t - floor(t) in [0, 1), s = fma(f, nf, -w/2).  Type-3 rescale (mode 1):
// s = fma(x - center, scale, nf/2 - w/2).  FP64 with one rounding per
// operation, the order the CPU restatement uses (bit-identical results).
// Non-finite coordinates are treated as 0 (mode 0) or as the centre (mode 1).
// nf_d = (double)nf and hw = w/2 come from the host (no per-point
// conversions on the FP64 pipe); for 0 <= t < 1 the floor is 0 and for
// -1 <= t < 0 it is -1, so f is t itself or the one rounded sum t + 1 --
// the same operation t - (-1) -- and only other t take the general path.
template <typename TX>
__device__ __forceinline__ double grid_shift(TX xin, int mode, double center, double scale,
                                             double nf_d, double hw) {
  if (mode == 0) {
    const double x = isfinite(xin) ? (double)xin : 0.0;
    const double t = __dmul_rn(x, kInv2Pi);
    const unsigned long long b = (unsigned long long)__double_as_longlong(t);
    const unsigned e = (unsigned)(b >> 52) & 0x7FFu;
    const bool neg = (b >> 63) != 0;
    double f;
    if (e < 0x3FFu && (!neg || (b << 1) == 0))
      f = t;  // 0 <= t < 1 (or -0): t - 0
    else if (neg && (e < 0x3FFu || b == 0xBFF0000000000000ull))
      f = __dadd_rn(t, 1.0);  // -1 <= t < 0: t - (-1)
    else
      f = __dsub_rn(t, floor(t));
    return __fma_rn(f, nf_d, -hw);
  }
  const double d = isfinite(xin) ? __dsub_rn((double)xin, center) : 0.0;
  return __fma_rn(d, scale, __dmul_rn(0.5, nf_d) - hw);
}

// Fold, grid start and bin of every point.  The first grid index a point
// touches is i0 = ceil(s); its offset is delta = i0 - s in [0, 1).  The bin is
// (i0 + w/2) / bs per axis after wrapping i0 + w/2 into [0, nf), so every
// point's support starts inside its bin's tile, which therefore needs only
// bs + w - 1 cells per axis.  With g.rows > 1 the sort key is
// bin * rows + (tile row of the point in its bin: y, or y + z * bs_y), so a
// bin's points come out ordered by row: an interpolation warp then gathers
// for points of the same or neighbouring rows, whose shared-memory reads
// collide on fewer banks.  FP32 coordinates with FP32 offsets take the
// integer fast path of the periodic fold (fold_fast_f32, same results), and
// the FP64 chain only for the points it declines.
// Bin counting is aggregated per block: the block's kFoldPts * kThreads
// points enter their bins into a shared-memory hash table (one slot per
// distinct bin, ranks from shared-memory atomics), and each slot then makes a
// single global atomic for its count.  Clustered points otherwise send one
// global atomic per warp to the same few bins, which serialise in L2.
constexpr int kFoldPts = 4;        // points per thread
constexpr int kFoldSlots = 2048;   // hash slots (twice the block's points)

template <typename TX, typename TC, int DIM>
__global__ void __launch_bounds__(kThreads)
    fold_kernel(Geom g, FoldSpec fs, int64_t M, const TX* __restrict__ x,
                const TX* __restrict__ y, const TX* __restrict__ z, int* __restrict__ pt_bin,
                int* __restrict__ pt_rank, int* __restrict__ bin_count,
                PtRec<TC, DIM>* __restrict__ recs_in, int count_bins) {
  static_assert(kFoldSlots >= 2 * kFoldPts * kThreads, "hash table at most half full");
  __shared__ int s_key[kFoldSlots];
  __shared__ int s_cnt[kFoldSlots];
  if (count_bins) {
    for (int i = threadIdx.x; i < kFoldSlots; i += kThreads) {
      s_key[i] = -1;
      s_cnt[i] = 0;
    }
    __syncthreads();
  }
  const int64_t j0 = (int64_t)blockIdx.x * (kFoldPts * kThreads) + threadIdx.x;
  int slot[kFoldPts], lrank[kFoldPts], binv[kFoldPts];
  const TX* c[3] = {x, y, z};
  const int h = g.w >> 1;
  // all the thread's coordinates in flight at once
  TX cv[kFoldPts][DIM];
#pragma unroll
  for (int k = 0; k < kFoldPts; ++k) {
    const int64_t j = j0 + (int64_t)k * kThreads;
#pragma unroll
    for (int d = 0; d < DIM; ++d) cv[k][d] = j < M ? c[d][j] : TX(0);
  }
#pragma unroll
  for (int k = 0; k < kFoldPts; ++k) {
    const int64_t j = j0 + (int64_t)k * kThreads;
    slot[k] = -1;
    if (j >= M) continue;
    PtRec<TC, DIM> r;
    int bin = 0, stride = 1, row = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const int nf = (int)g.nf[d];
      int i0;
      bool done = false;
      if constexpr (sizeof(TX) == 4 && sizeof(TC) == 4) {
        if (fs.mode == 0) {
          float dl;
          done = fold_fast_f32((float)cv[k][d], nf, g.w, fs.lnf[d], fs.kmant, fs.kexp, i0, dl);
          if (done) r.d[d] = (TC)dl;
        }
      }
      if (!done) {
        const double sh = grid_shift(cv[k][d], fs.mode, fs.center[d], fs.scale[d], fs.nf_d[d],
                                     fs.hw);
        const double cl = ceil(sh);
        i0 = (int)cl;
        r.d[d] = (TC)__dsub_rn(cl, sh);
      }
      int tb = i0 + h;
      if (tb < 0) {
        tb += nf;
        i0 += nf;
      }
      if (tb >= nf) {
        tb -= nf;
        i0 -= nf;
      }
      r.i[d] = i0;
      // tb / bs by multiply-high with floor(2^32 / bs): one correction step
      int bd = tb;
      if (g.bs[d] > 1) {
        bd = (int)__umulhi((unsigned)tb, fs.bs_mul[d]);
        if (tb - bd * g.bs[d] >= g.bs[d]) ++bd;
      }
      bin += bd * stride;
      stride *= g.nb[d];
      if (d == 1) row += tb - bd * g.bs[1];
      if (d == 2) row += (tb - bd * g.bs[2]) * g.bs[1];
    }
    if (g.rows > 1) bin = bin * g.rows + row;  // bin order, then tile row within the bin
    recs_in[j] = r;
    binv[k] = bin;
    if (count_bins) {
      // linear probing; at most kFoldPts * kThreads distinct keys, so a free
      // or matching slot turns up within kFoldSlots probes
      unsigned hs = ((unsigned)bin * 2654435761u) >> 21;
      int sl = -1;
      for (int probe = 0; probe < kFoldSlots; ++probe) {
        const int prev = atomicCAS(&s_key[hs], -1, bin);
        if (prev == -1 || prev == bin) {
          sl = (int)hs;
          break;
        }
        hs = (hs + 1) & (kFoldSlots - 1);
      }
      if (sl >= 0) {
        slot[k] = sl;
        lrank[k] = atomicAdd(&s_cnt[sl], 1);
      } else {  // not reached (the table cannot fill); a direct global rank
        slot[k] = -2;
        lrank[k] = atomicAdd(&bin_count[bin], 1);
      }
    }
  }
  if (!count_bins) return;
  __syncthreads();
  // one global atomic per distinct bin of the block; s_cnt becomes its base
  for (int i = threadIdx.x; i < kFoldSlots; i += kThreads) {
    const int key = s_key[i];
    if (key >= 0) s_cnt[i] = atomicAdd(&bin_count[key], s_cnt[i]);
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kFoldPts; ++k) {
    const int64_t j = j0 + (int64_t)k * kThreads;
    if (j >= M) continue;
    pt_bin[j] = binv[k];
    pt_rank[j] = slot[k] >= 0 ? s_cnt[slot[k]] + lrank[k] : lrank[k];
  }
}

// --- exclusive scan of int32 ------------------------------------------------
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int* total) {
  __shared__ int warp_sums[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int n = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += n;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int ws = warp_sums[lane];
    int wi = ws;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int n = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += n;
    }
    warp_sums[lane] = wi - ws;
    if (lane == 31) *total = wi;
  }
  __syncthreads();
  int r = incl - v + warp_sums[warp];
  __syncthreads();
  return r;
}

__global__ void scan_local_kernel(const int* in, int* out, int64_t n, int* block_sums) {
  __shared__ int total;
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int v[kScanItems];
  int s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (base + i < n) ? in[base + i] : 0;
    s += v[i];
  }
  int ex = block_exclusive_scan(s, &total);
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) out[base + i] = ex;
    ex += v[i];
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void scan_sums_kernel(int* sums, int64_t nb) {
  __shared__ int total;
  int carry = 0;
  for (int64_t b0 = 0; b0 < nb; b0 += kScanThreads) {
    const int64_t i = b0 + threadIdx.x;
    int v = i < nb ? sums[i] : 0;
    int ex = block_exclusive_scan(v, &total);
    if (i < nb) sums[i] = ex + carry;
    carry += total;
    __syncthreads();
  }
}

__global__ void scan_add_kernel(int* out, int64_t n, const int* sums) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += sums[i / kScanTile];
}

// --- bin-order scatter and subproblems ---------------------------------------
// kScatterPts points per thread, each stage's loads issued for all of them
// before the next stage needs them (the bin start depends on the bin).
constexpr int kScatterPts = 4;

template <typename REC>
__global__ void __launch_bounds__(kThreads)
    scatter_kernel(int64_t M, const int* __restrict__ pt_bin, const int* __restrict__ pt_rank,
                   const int* __restrict__ bin_start, const REC* __restrict__ recs_in,
                   REC* __restrict__ recs, int* __restrict__ perm) {
  const int64_t j0 = (int64_t)blockIdx.x * (kScatterPts * kThreads) + threadIdx.x;
  int b[kScatterPts], rk[kScatterPts], pos[kScatterPts];
  REC rv[kScatterPts];
#pragma unroll
  for (int k = 0; k < kScatterPts; ++k) {
    const int64_t j = j0 + (int64_t)k * kThreads;
    if (j < M) {
      b[k] = pt_bin[j];
      rk[k] = pt_rank[j];
      rv[k] = recs_in[j];
    }
  }
#pragma unroll
  for (int k = 0; k < kScatterPts; ++k)
    if (j0 + (int64_t)k * kThreads < M) pos[k] = bin_start[b[k]] + rk[k];
#pragma unroll
  for (int k = 0; k < kScatterPts; ++k) {
    const int64_t j = j0 + (int64_t)k * kThreads;
    if (j < M) {
      perm[pos[k]] = (int)j;
      recs[pos[k]] = rv[k];
    }
  }
}

// Bin b holds keys [b*rows, (b+1)*rows): its range in the sorted order.
__global__ void bin_ranges_kernel(int64_t nbins, int rows, int64_t M,
                                  const int* __restrict__ key_start, int* __restrict__ bin_start,
                                  int* __restrict__ bin_count) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbins) return;
  const int s0 = key_start[b * rows];
  const int s1 = b + 1 < nbins ? key_start[(b + 1) * rows] : (int)M;
  bin_start[b] = s0;
  bin_count[b] = s1 - s0;
}

__global__ void subcount_kernel(int64_t nbins, const int* __restrict__ bin_count, int maxsub,
                                int* __restrict__ sub_count) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nbins) sub_count[b] = (bin_count[b] + maxsub - 1) / maxsub;
}

__global__ void subfill_kernel(int64_t nbins, const int* __restrict__ sub_count,
                               const int* __restrict__ sub_start, int maxsub,
                               int* __restrict__ sub_bin, int* __restrict__ sub_off,
                               int* __restrict__ n_sub) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbins) return;
  const int n = sub_count[b], s0 = sub_start[b];
  for (int s = 0; s < n; ++s) {
    sub_bin[s0 + s] = (int)b;
    sub_off[s0 + s] = s * maxsub;
  }
  if (b == nbins - 1) *n_sub = s0 + n;
}

// --- deconvolution -------------------------------------------------------------
// Mode index i -> fine index along one axis (modeord 0: CMCL order, k = i - N/2;
// 1: FFT order).
__device__ __forceinline__ int mode_to_fine(int i, int N, int nf, int modeord) {
  const int k = modeord == 0 ? i - N / 2 : (i < (N + 1) / 2 ? i : i - N);
  return k < 0 ? k + nf : k;
}

// Deconvolved copy of the fine grid's mode region into the modes (type 1).
// Items are (output row, chunk of blockDim.x cell pairs of the row); each
// block walks a contiguous range of items, advancing the row's y/z indices
// incrementally, and each thread handles pair q = chunk * blockDim.x +
// threadIdx.x of its items, re-deriving that pair's fine indices and factors
// only when the chunk changes (never when a row is one chunk).  Pairs whose
// two fine cells are adjacent and 16-byte aligned move with one 16-byte load
// and, when vec_out, one 16-byte (FP32) store; indexing inside a transform is
// 32-bit (a fine grid has < 2^31 cells).
template <typename TC, typename TD, int DIM>
__global__ void __launch_bounds__(256, sizeof(TC) == 4 && sizeof(TD) == 4 ? 6 : 1)
    deconv1_kernel(int N0, int N1, int N2, int nf0, int nf1, int nf2, int modeord,
                   const TC* __restrict__ p0, const TC* __restrict__ p1,
                   const TC* __restrict__ p2, const cplx_t<TC>* __restrict__ fine,
                   cplx_t<TD>* __restrict__ out, int ntr, int64_t nftot, int64_t Ntot,
                   int vec_out) {
  const int nrows = N1 * N2;
  const int npair = (N0 + 1) >> 1;
  const int nchunk = (npair + blockDim.x - 1) / blockDim.x;
  const int64_t nitem = (int64_t)nrows * nchunk;
  const int64_t per = (nitem + gridDim.x - 1) / gridDim.x;
  const int64_t it0 = blockIdx.x * per, it1 = min(it0 + per, nitem);
  if (it0 >= it1) return;
  int row = (int)(it0 / nchunk), chunk = (int)(it0 - (int64_t)row * nchunk);
  int i1 = DIM > 1 ? row % N1 : 0;
  int i2 = DIM > 2 ? row / N1 : 0;
  int g2 = DIM > 2 ? mode_to_fine(i2, N2, nf2, modeord) : 0;
  TC f2 = DIM > 2 ? p2[i2] : TC(1);
  int q = -1, ga = 0, gb = 0;
  TC fa = TC(0), fb = TC(0);
  bool hasb = false, vin = false;
  for (int64_t item = it0; item < it1; ++item) {
    if (item > it0 && ++chunk == nchunk) {
      chunk = 0;
      ++row;
      if (++i1 == N1) {
        i1 = 0;
        ++i2;
        if (DIM > 2) {
          g2 = mode_to_fine(i2, N2, nf2, modeord);
          f2 = p2[i2];
        }
      }
    }
    const int qn = chunk * blockDim.x + threadIdx.x;
    if (qn >= npair) continue;
    if (qn != q) {  // this thread's pair changed: its x side of the map
      q = qn;
      const int ia = 2 * q, ib = ia + 1;
      hasb = ib < N0;
      ga = mode_to_fine(ia, N0, nf0, modeord);
      gb = hasb ? mode_to_fine(ib, N0, nf0, modeord) : ga;
      fa = p0[ia];
      fb = hasb ? p0[ib] : TC(0);
      vin = sizeof(TC) == 4 && hasb && gb == ga + 1 && (ga & 1) == 0;
    }
    const int g1 = DIM > 1 ? mode_to_fine(i1, N1, nf1, modeord) : 0;
    const TC f12 = DIM > 1 ? f2 * p1[i1] : f2;
    const TC ca = fa * f12, cb = fb * f12;
    const cplx_t<TC>* src = fine + (g2 * nf1 + g1) * nf0;
    cplx_t<TD>* dst = out + row * N0 + 2 * q;
    for (int t = 0; t < ntr; ++t, src += nftot, dst += Ntot) {
      cplx_t<TC> a, b;
      if (vin) {
        const float4 v = *reinterpret_cast<const float4*>(src + ga);
        a.x = v.x;
        a.y = v.y;
        b.x = v.z;
        b.y = v.w;
      } else {
        a = src[ga];
        b = src[gb];
      }
      if constexpr (sizeof(TC) == 4 && sizeof(TD) == 4) {
        if (vec_out && hasb) {
          *reinterpret_cast<float4*>(dst) = make_float4(a.x * ca, a.y * ca, b.x * cb, b.y * cb);
          continue;
        }
      }
      cplx_t<TD> o;
      o.x = (TD)(a.x * ca);
      o.y = (TD)(a.y * ca);
      dst[0] = o;
      if (hasb) {
        o.x = (TD)(b.x * cb);
        o.y = (TD)(b.y * cb);
        dst[1] = o;
      }
    }
  }
}

// Fine index g -> output index along one axis, or -1 when g holds no mode.
__device__ __forceinline__ int fine_to_mode(int g, int N, int nf, int modeord) {
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

// Zero-padded, deconvolved copy of the modes into the fine grid (type 2).
// Items are (fine-grid row, chunk of blockDim.x cell pairs of the row); each
// block walks a contiguous range of items, advancing the row's y/z indices
// incrementally, and each thread writes pair q = chunk * blockDim.x +
// threadIdx.x of its items with one 16-byte store per transform (zeros
// outside the mode region, so the padding needs no memset).  The pair's mode
// indices and factors are re-derived only when the chunk changes (never
// when a row is one chunk), so a row costs a few instructions per store and
// the kernel runs at the HBM write rate.
template <typename TC, typename TD, int DIM>
__global__ void __launch_bounds__(256)
    deconv2_kernel(int N0, int N1, int N2, int nf0, int nf1, int nf2, int modeord,
                   const TC* __restrict__ p0, const TC* __restrict__ p1,
                   const TC* __restrict__ p2, const cplx_t<TD>* __restrict__ in,
                   cplx_t<TC>* __restrict__ fine, int ntr, int64_t nftot, int64_t Ntot) {
  const int nrows = nf1 * nf2;
  const int npair = nf0 >> 1;  // nf0 is even
  const int nchunk = (npair + blockDim.x - 1) / blockDim.x;
  const int64_t nitem = (int64_t)nrows * nchunk;
  const int64_t per = (nitem + gridDim.x - 1) / gridDim.x;
  const int64_t it0 = blockIdx.x * per, it1 = min(it0 + per, nitem);
  if (it0 >= it1) return;
  int row = (int)(it0 / nchunk), chunk = (int)(it0 - (int64_t)row * nchunk);
  int g1 = DIM > 1 ? row % nf1 : 0;
  int g2 = DIM > 2 ? row / nf1 : 0;
  int i2 = DIM > 2 ? fine_to_mode(g2, N2, nf2, modeord) : 0;
  TC f2 = DIM > 2 && i2 >= 0 ? p2[i2] : TC(1);
  int q = -1, ia = -1, ib = -1;
  TC fa = TC(0), fb = TC(0);
  for (int64_t item = it0; item < it1; ++item) {
    if (item > it0 && ++chunk == nchunk) {
      chunk = 0;
      ++row;
      if (++g1 == nf1) {
        g1 = 0;
        ++g2;
        if (DIM > 2) {
          i2 = fine_to_mode(g2, N2, nf2, modeord);
          f2 = i2 >= 0 ? p2[i2] : TC(1);
        }
      }
    }
    const int qn = chunk * blockDim.x + threadIdx.x;
    if (qn >= npair) continue;
    if (qn != q) {  // this thread's pair changed: its x side of the map
      q = qn;
      ia = fine_to_mode(2 * q, N0, nf0, modeord);
      ib = fine_to_mode(2 * q + 1, N0, nf0, modeord);
      fa = ia >= 0 ? p0[ia] : TC(0);
      fb = ib >= 0 ? p0[ib] : TC(0);
    }
    const int i1 = DIM > 1 ? fine_to_mode(g1, N1, nf1, modeord) : 0;
    const bool live = i1 >= 0 && i2 >= 0;
    const TC f12 = live ? (DIM > 1 ? f2 * p1[i1] : f2) : TC(0);
    const int ja = live ? ia : -1, jb = live ? ib : -1;
    const TC ca = fa * f12, cb = fb * f12;
    const cplx_t<TD>* src = in + (live ? (i2 * N1 + i1) * N0 : 0);
    cplx_t<TC>* d = fine + row * nf0 + 2 * q;  // even cell: 16-byte aligned pair
    for (int t = 0; t < ntr; ++t, src += Ntot, d += nftot) {
      cplx_t<TC> a, b;
      a.x = a.y = b.x = b.y = TC(0);
      if (ja >= 0) {
        const cplx_t<TD> v = src[ja];
        a.x = (TC)v.x * ca;
        a.y = (TC)v.y * ca;
      }
      if (jb >= 0) {
        const cplx_t<TD> v = src[jb];
        b.x = (TC)v.x * cb;
        b.y = (TC)v.y * cb;
      }
      if constexpr (sizeof(TC) == 4) {
        *reinterpret_cast<float4*>(d) = make_float4(a.x, a.y, b.x, b.y);
      } else {
        d[0] = a;
        d[1] = b;
      }
    }
  }
}

// --- type 3 -----------------------------------------------------------------------
__device__ __forceinline__ unsigned long long dkey(double v) {
  unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}

template <typename TX>
__global__ void minmax_kernel(const TX* __restrict__ a, int64_t n, unsigned long long* out) {
  unsigned long long lo = ~0ull, hi = 0ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double v = (double)a[i];
    if (!isfinite(v)) continue;
    unsigned long long k = dkey(v);
    lo = k < lo ? k : lo;
    hi = k > hi ? k : hi;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long l2 = __shfl_xor_sync(0xffffffffu, lo, o);
    unsigned long long h2 = __shfl_xor_sync(0xffffffffu, hi, o);
    lo = l2 < lo ? l2 : lo;
    hi = h2 > hi ? h2 : hi;
  }
  // one atomic pair per block (all blocks' atomics meet at one address)
  __shared__ unsigned long long s_lo[32], s_hi[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0) {
    s_lo[warp] = lo;
    s_hi[warp] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < nw; ++i) {
      lo = s_lo[i] < lo ? s_lo[i] : lo;
      hi = s_hi[i] > hi ? s_hi[i] : hi;
    }
    atomicMin(&out[0], lo);
    atomicMax(&out[1], hi);
  }
}

__global__ void minmax_init_kernel(unsigned long long* k, int narr) {
  int i = threadIdx.x;
  if (i < narr) {
    k[2 * i] = ~0ull;
    k[2 * i + 1] = 0ull;
  }
}

__global__ void minmax_decode_kernel(const unsigned long long* k, double* out, int narr) {
  int i = threadIdx.x;
  if (i < 2 * narr) {
    unsigned long long b = k[i];
    if (i % 2 == 0 && b == ~0ull) {
      out[i] = 0.0;  // no finite values
      return;
    }
    if (i % 2 == 1 && b == 0ull) {
      out[i] = 0.0;
      return;
    }
    b = (b & 0x8000000000000000ull) ? (b & 0x7fffffffffffffffull) : ~b;
    out[i] = __longlong_as_double((long long)b);
  }
}

struct Ptrs3 {
  const void* p[3];
};
struct Bounds3 {
  double lo[3], hi[3];
};
struct DPtrs3 {
  double* p[3];
};
struct CDPtrs3 {
  const double* p[3];
};

template <typename TX>
__global__ void t3_targets_kernel(int dim, int64_t N, Ptrs3 s, double c0, double c1, double c2,
                                  double isc0, double isc1, double isc2, DPtrs3 tau) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  // isc: reciprocal scales (a multiply where a division would run on the
  // FP64 pipe's slow path; the result differs by at most an ulp)
  const double c[3] = {c0, c1, c2}, isc[3] = {isc0, isc1, isc2};
  for (int d = 0; d < dim; ++d) {
    double v = (double)((const TX*)s.p[d])[k];
    tau.p[d][k] = isfinite(v) ? (v - c[d]) * isc[d] : 0.0;
  }
}

// e^{i ph} / den into a compute-precision complex.  FP32: the phase is
// reduced to [-pi, pi] in FP64 (|ph| / 2 pi cycles removed exactly enough:
// ph - 2 pi k by one FMA) and its sine and cosine taken in FP32, whose
// rounding matches the FP32 output; FP64 throughout otherwise.
template <typename TC>
__device__ __forceinline__ cplx_t<TC> phase_over(double ph, double den) {
  cplx_t<TC> o;
  if constexpr (sizeof(TC) == 4) {
    const double k = rint(ph * 0.15915494309189535);  // 1 / (2 pi)
    const float pr = (float)fma(-k, 6.283185307179586, ph);
    float sn, cn;
    sincosf(pr, &sn, &cn);
    const float inv = 1.0f / (float)den;
    o.x = cn * inv;
    o.y = sn * inv;
  } else {
    double sn, cn;
    sincos(ph, &sn, &cn);
    o.x = cn / den;
    o.y = sn / den;
  }
  return o;
}

template <typename TX, typename TC>
__global__ void t3_pre_kernel(int dim, int64_t M, Ptrs3 x, double cx0, double cx1, double cx2,
                              double cs0, double cs1, double cs2, int iflag,
                              cplx_t<TC>* __restrict__ fac) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  const double cx[3] = {cx0, cx1, cx2}, cs[3] = {cs0, cs1, cs2};
  double ph = 0.0;
  for (int d = 0; d < dim; ++d) {
    double v = (double)((const TX*)x.p[d])[j];
    if (!isfinite(v)) v = cx[d];
    ph += cs[d] * (v - cx[d]);
  }
  fac[j] = phase_over<TC>((double)iflag * ph, 1.0);
}

constexpr int kMaxQuad = 64;
struct Quad {
  int q;
  double t[kMaxQuad];
  double f[kMaxQuad];
};

template <typename TX, typename TC>
__global__ void t3_post_kernel(int dim, int64_t N, Ptrs3 s, double cx0, double cx1, double cx2,
                               CDPtrs3 tau, int iflag, Quad qd, cplx_t<TC>* __restrict__ fac) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  const double cx[3] = {cx0, cx1, cx2};
  double ph = 0.0, den = 1.0;
  for (int d = 0; d < dim; ++d) {
    double v = (double)((const TX*)s.p[d])[k];
    if (!isfinite(v)) v = 0.0;
    ph += cx[d] * v;
    const double tv = tau.p[d][k];
    double acc = 0.0;
    for (int i = 0; i < qd.q; ++i) acc += qd.f[i] * cos(tv * qd.t[i]);
    den *= acc;
  }
  fac[k] = phase_over<TC>((double)iflag * ph, den);
}

// The same factors with psihat from a piecewise Chebyshev table: piece
// p = min(|tau| / h, P - 1), coefficients tab[p*(D+1) .. ] (the first one
// halved), evaluated by Clenshaw's recurrence.
template <typename TX, typename TC>
__global__ void t3_post_table_kernel(int dim, int64_t N, Ptrs3 s, double cx0, double cx1,
                                     double cx2, CDPtrs3 tau, int iflag,
                                     const double* __restrict__ tab, double h, int P, int D,
                                     cplx_t<TC>* __restrict__ fac) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  const double cx[3] = {cx0, cx1, cx2};
  const double inv_h = 1.0 / h;
  double ph = 0.0, den = 1.0;
  for (int d = 0; d < dim; ++d) {
    double v = (double)((const TX*)s.p[d])[k];
    if (!isfinite(v)) v = 0.0;
    ph += cx[d] * v;
    const double u = fabs(tau.p[d][k]);
    int piece = (int)(u * inv_h);
    piece = piece < 0 ? 0 : (piece >= P ? P - 1 : piece);
    const double x = 2.0 * (u - piece * h) * inv_h - 1.0;
    const double* c = tab + (int64_t)piece * (D + 1);
    double b1 = 0.0, b2 = 0.0;
    for (int n = D; n >= 1; --n) {
      const double b0 = fma(2.0 * x, b1, c[n] - b2);
      b2 = b1;
      b1 = b0;
    }
    den *= fma(x, b1, c[0] - b2);
  }
  fac[k] = phase_over<TC>((double)iflag * ph, den);
}

template <typename TI, typename TO, typename TF>
__global__ void cmul_kernel(int64_t n, int ntr, const cplx_t<TI>* __restrict__ in,
                            const cplx_t<TF>* __restrict__ fac, cplx_t<TO>* __restrict__ out,
                            int conj) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  cplx_t<TF> f = fac[j];
  if (conj) f.y = -f.y;
  for (int t = 0; t < ntr; ++t) {
    const cplx_t<TI> v = in[(int64_t)t * n + j];
    const TF vr = (TF)v.x, vi = (TF)v.y;
    cplx_t<TO> o;
    o.x = (TO)(vr * f.x - vi * f.y);
    o.y = (TO)(vr * f.y + vi * f.x);
    out[(int64_t)t * n + j] = o;
  }
}

// item_start[k] = T * sum_{i<k} n_sub_i, k = 0..K, one block of 1024 threads
// walking the problems in chunks with a running carry.
template <typename TC>
__global__ void item_prefix_kernel(const BatchProb<TC>* __restrict__ probs, int K, int T,
                                   int64_t* __restrict__ out) {
  __shared__ int64_t warp_sums[32];
  __shared__ int64_t carry_s;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k0 = 0; k0 < K; k0 += blockDim.x) {
    const int k = k0 + threadIdx.x;
    const int64_t v = k < K ? (int64_t)(*probs[k].n_sub) * T : 0;
    int64_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t n = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += n;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      const int64_t ws = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
      int64_t wi = ws;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t n = __shfl_up_sync(0xffffffffu, wi, o);
        if (lane >= o) wi += n;
      }
      warp_sums[lane] = wi - ws;
    }
    __syncthreads();
    const int64_t carry = carry_s;
    if (k < K) out[k] = carry + incl - v + warp_sums[warp];
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry_s = carry + incl + warp_sums[warp];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[K] = carry_s;
}

inline unsigned grid1(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

// =============================================================================
// launchers
// =============================================================================

template <typename TX, typename TC>
cudaError_t launch_fold(const Geom& g, const FoldSpec& fs_in, int64_t M, const TX* x, const TX* y,
                        const TX* z, SortState& st, cudaStream_t s) {
  if (M == 0) return cudaSuccess;
  FoldSpec fs = fs_in;
  for (int d = 0; d < 3; ++d) fs.nf_d[d] = (double)g.nf[d];
  fs.hw = 0.5 * (double)g.w;
  uint64_t kb;
  std::memcpy(&kb, &kInv2Pi, 8);
  fs.kmant = (kb & ((1ull << 52) - 1)) | (1ull << 52);
  fs.kexp = (int)((kb >> 52) & 0x7FF) - 1075;
  for (int d = 0; d < 3; ++d) {
    int l = 0;
    while (l < 62 && ((int64_t)1 << l) < g.nf[d]) ++l;
    fs.lnf[d] = l;
    fs.bs_mul[d] = g.bs[d] > 1 ? (unsigned)((1ull << 32) / (unsigned)g.bs[d]) : 0u;
  }
  const unsigned nb = grid1(M, kThreads * kFoldPts);
  const int count = st.key_count != nullptr;
  switch (g.dim) {
    case 1:
      fold_kernel<TX, TC, 1><<<nb, kThreads, 0, s>>>(g, fs, M, x, y, z, st.pt_bin, st.pt_rank,
                                                     st.key_count,
                                                     (PtRec<TC, 1>*)st.recs_in, count);
      note_launch();
      break;
    case 2:
      fold_kernel<TX, TC, 2><<<nb, kThreads, 0, s>>>(g, fs, M, x, y, z, st.pt_bin, st.pt_rank,
                                                     st.key_count,
                                                     (PtRec<TC, 2>*)st.recs_in, count);
      note_launch();
      break;
    default:
      fold_kernel<TX, TC, 3><<<nb, kThreads, 0, s>>>(g, fs, M, x, y, z, st.pt_bin, st.pt_rank,
                                                     st.key_count,
                                                     (PtRec<TC, 3>*)st.recs_in, count);
      note_launch();
      break;
  }
  return cudaGetLastError();
}

int64_t scan_tmp_ints(int64_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

cudaError_t launch_scan(const int* in, int* out, int64_t n, int* tmp, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const int64_t nblk = (n + kScanTile - 1) / kScanTile;
  scan_local_kernel<<<(unsigned)nblk, kScanThreads, 0, s>>>(in, out, n, tmp);
  note_launch();
  if (nblk > 1) {
    scan_sums_kernel<<<1, kScanThreads, 0, s>>>(tmp, nblk);
    note_launch();
    scan_add_kernel<<<grid1(n, 256), 256, 0, s>>>(out, n, tmp);
    note_launch();
  }
  return cudaGetLastError();
}

template <typename TC>
cudaError_t launch_sort_finish(const Geom& g, int64_t M, SortState& st, bool sorted,
                               cudaStream_t s) {
  if (!sorted) return cudaSuccess;
  const int rows = g.rows > 1 ? g.rows : 1;
  cudaError_t e = launch_scan(st.key_count, st.key_start, g.nbins * rows, st.scan_tmp, s);
  if (e != cudaSuccess) return e;
  if (M > 0) {
    const unsigned nb = grid1(M, kThreads * kScatterPts);
    switch (g.dim) {
      case 1:
        scatter_kernel<PtRec<TC, 1>><<<nb, kThreads, 0, s>>>(
            M, st.pt_bin, st.pt_rank, st.key_start, (const PtRec<TC, 1>*)st.recs_in,
            (PtRec<TC, 1>*)st.recs, st.perm);
        note_launch();
        break;
      case 2:
        scatter_kernel<PtRec<TC, 2>><<<nb, kThreads, 0, s>>>(
            M, st.pt_bin, st.pt_rank, st.key_start, (const PtRec<TC, 2>*)st.recs_in,
            (PtRec<TC, 2>*)st.recs, st.perm);
        note_launch();
        break;
      default:
        scatter_kernel<PtRec<TC, 3>><<<nb, kThreads, 0, s>>>(
            M, st.pt_bin, st.pt_rank, st.key_start, (const PtRec<TC, 3>*)st.recs_in,
            (PtRec<TC, 3>*)st.recs, st.perm);
        note_launch();
        break;
    }
  }
  const unsigned nbb = grid1(g.nbins, 256);
  if (rows > 1) {  // per-bin ranges from the key scan
    bin_ranges_kernel<<<nbb, 256, 0, s>>>(g.nbins, rows, M, st.key_start, st.bin_start,
                                          st.bin_count);
    note_launch();
  }
  subcount_kernel<<<nbb, 256, 0, s>>>(g.nbins, st.bin_count, g.maxsub, st.sub_count);
  note_launch();
  e = launch_scan(st.sub_count, st.sub_start, g.nbins, st.scan_tmp, s);
  if (e != cudaSuccess) return e;
  subfill_kernel<<<nbb, 256, 0, s>>>(g.nbins, st.sub_count, st.sub_start, g.maxsub, st.sub_bin,
                                     st.sub_off, st.n_sub);
  note_launch();
  return cudaGetLastError();
}

template <typename TC, typename TD>
cudaError_t launch_deconv1(int dim, const int64_t* N, const int64_t* nf, int modeord,
                           const TC* const* phi, const void* fine, void* out, int ntr,
                           cudaStream_t s) {
  const int64_t nftot = nf[0] * nf[1] * nf[2], Ntot = N[0] * N[1] * N[2];
  // threads per block: the row's pairs, rounded up to whole warps (<= 256)
  const int64_t npair = (N[0] + 1) / 2;
  const int threads = (int)std::min<int64_t>(256, (npair + 31) / 32 * 32);
  const int64_t items = N[1] * N[2] * ((npair + threads - 1) / threads);
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const unsigned grid = (unsigned)std::min<int64_t>(items, (int64_t)nsm * 32);
  // 16-byte stores need an even row length and a 16-byte aligned output
  const int vec_out = N[0] % 2 == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0 &&
                      (Ntot % 2 == 0 || ntr == 1);
  const TC* p1 = dim > 1 ? phi[1] : nullptr;
  const TC* p2 = dim > 2 ? phi[2] : nullptr;
  auto args = [&](auto kern) {
    kern<<<grid, threads, 0, s>>>((int)N[0], (int)N[1], (int)N[2], (int)nf[0], (int)nf[1],
                                  (int)nf[2], modeord, phi[0], p1, p2, (const cplx_t<TC>*)fine,
                                  (cplx_t<TD>*)out, ntr, nftot, Ntot, vec_out);
  };
  switch (dim) {
    case 1:
      args(deconv1_kernel<TC, TD, 1>);
      break;
    case 2:
      args(deconv1_kernel<TC, TD, 2>);
      break;
    default:
      args(deconv1_kernel<TC, TD, 3>);
      break;
  }
  note_launch();
  return cudaGetLastError();
}

template <typename TC, typename TD>
cudaError_t launch_deconv2(int dim, const int64_t* N, const int64_t* nf, int modeord,
                           const TC* const* phi, const void* in, void* fine, int ntr,
                           cudaStream_t s) {
  const int64_t nftot = nf[0] * nf[1] * nf[2], Ntot = N[0] * N[1] * N[2];
  const int64_t npair = nf[0] / 2;
  const int threads = (int)std::min<int64_t>(256, (npair + 31) / 32 * 32);
  const int64_t items = nf[1] * nf[2] * ((npair + threads - 1) / threads);
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const unsigned grid = (unsigned)std::min<int64_t>(items, (int64_t)nsm * 32);
  const TC* p1 = dim > 1 ? phi[1] : nullptr;
  const TC* p2 = dim > 2 ? phi[2] : nullptr;
  auto args = [&](auto kern) {
    kern<<<grid, threads, 0, s>>>((int)N[0], (int)N[1], (int)N[2], (int)nf[0], (int)nf[1],
                                  (int)nf[2], modeord, phi[0], p1, p2, (const cplx_t<TD>*)in,
                                  (cplx_t<TC>*)fine, ntr, nftot, Ntot);
  };
  switch (dim) {
    case 1:
      args(deconv2_kernel<TC, TD, 1>);
      break;
    case 2:
      args(deconv2_kernel<TC, TD, 2>);
      break;
    default:
      args(deconv2_kernel<TC, TD, 3>);
      break;
  }
  note_launch();
  return cudaGetLastError();
}

template <typename TX>
cudaError_t launch_minmax(const TX* const* arrs, int narr, int64_t n, double* out,
                          cudaStream_t s) {
  // out doubles as key scratch: 2*narr unsigned long long then decoded in place
  unsigned long long* keys = (unsigned long long*)out;
  minmax_init_kernel<<<1, 32, 0, s>>>(keys, narr);
  note_launch();
  unsigned nb = grid1(n, 256);
  if (nb > 1024) nb = 1024;
  if (nb == 0) nb = 1;
  for (int a = 0; a < narr; ++a)
    if (n > 0) minmax_kernel<TX><<<nb, 256, 0, s>>>(arrs[a], n, keys + 2 * a);
    note_launch();
  minmax_decode_kernel<<<1, 64, 0, s>>>(keys, out, narr);
  note_launch();
  return cudaGetLastError();
}

// Declared type-3 extents: a warp with a finite coordinate outside its
// axis's [lo, hi] raises the flag word once (system-scope atomic on mapped
// host memory); non-finite coordinates are left to the fold, which treats
// them as the centre.
template <typename TX>
__global__ void extent_check_kernel(int dim, int64_t n, Ptrs3 a, Bounds3 b, unsigned* flag) {
  bool out = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    for (int d = 0; d < dim; ++d) {
      const double v = (double)((const TX*)a.p[d])[i];
      if (isfinite(v) && (v < b.lo[d] || v > b.hi[d])) out = true;
    }
  }
  if (__any_sync(0xffffffffu, out) && (threadIdx.x & 31) == 0) {
    atomicAdd_system(flag, 1u);
    __threadfence_system();
  }
}

template <typename TX>
cudaError_t launch_extent_check(int dim, int64_t n, const TX* const* a, const double* lo,
                                const double* hi, unsigned* flag, cudaStream_t s) {
  if (n == 0 || flag == nullptr) return cudaSuccess;
  Ptrs3 ap{};
  Bounds3 bb{};
  for (int d = 0; d < dim; ++d) {
    ap.p[d] = a[d];
    bb.lo[d] = lo[d];
    bb.hi[d] = hi[d];
  }
  unsigned nb = grid1(n, 256);
  if (nb > 1024) nb = 1024;
  extent_check_kernel<TX><<<nb, 256, 0, s>>>(dim, n, ap, bb, flag);
  note_launch();
  return cudaGetLastError();
}

template <typename TX>
cudaError_t launch_t3_targets(int dim, int64_t N, const TX* const* s, const double* center,
                              const double* scale, double* const* tau, cudaStream_t st) {
  if (N == 0) return cudaSuccess;
  Ptrs3 sp{};
  DPtrs3 tp{};
  double c[3] = {0, 0, 0}, sc[3] = {1, 1, 1};
  for (int d = 0; d < dim; ++d) {
    sp.p[d] = s[d];
    tp.p[d] = tau[d];
    c[d] = center[d];
    sc[d] = 1.0 / scale[d];
  }
  t3_targets_kernel<TX><<<grid1(N, 256), 256, 0, st>>>(dim, N, sp, c[0], c[1], c[2], sc[0],
                                                       sc[1], sc[2], tp);
  note_launch();
  return cudaGetLastError();
}

template <typename TX, typename TC>
cudaError_t launch_t3_prephase_factors(int dim, int64_t M, const TX* const* x, const double* cx,
                                       const double* cs, int iflag, void* fac, cudaStream_t s) {
  if (M == 0) return cudaSuccess;
  Ptrs3 xp{};
  double c[3] = {0, 0, 0}, t[3] = {0, 0, 0};
  for (int d = 0; d < dim; ++d) {
    xp.p[d] = x[d];
    c[d] = cx[d];
    t[d] = cs[d];
  }
  t3_pre_kernel<TX, TC><<<grid1(M, 256), 256, 0, s>>>(dim, M, xp, c[0], c[1], c[2], t[0], t[1],
                                                      t[2], iflag, (cplx_t<TC>*)fac);
  note_launch();
  return cudaGetLastError();
}

// Gauss-Legendre nodes on [-1, 1] (Newton iteration on P_q); host side.
static void gauss_legendre(int q, double* x, double* wt) {
  const double pi = 3.141592653589793238462643383279502884;
  for (int i = 0; i < (q + 1) / 2; ++i) {
    double z = cos(pi * (i + 0.75) / (q + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= q; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = q * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) break;
    }
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= q; ++k) {
      double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = q * (z * p1 - p0) / (z * z - 1.0);
    x[i] = -z;
    x[q - 1 - i] = z;
    wt[i] = wt[q - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

// psihat(tau) = sum_i f_i cos(tau t_i) by the quadrature (FP64, host).
double psihat_quad(const Quad& qd, double tau) {
  double acc = 0.0;
  for (int i = 0; i < qd.q; ++i) acc += qd.f[i] * std::cos(tau * qd.t[i]);
  return acc;
}

// Piecewise Chebyshev fit of psihat on [0, tau_max] (degree D per piece,
// pieces of width h halved until every check point of every piece -- nodes
// off the interpolation nodes, piece ends included -- is within rel_tol of
// the quadrature).  False when 4096 pieces do not reach it.
bool fit_psihat(const Quad& qd, double tau_max, double rel_tol, int D, std::vector<double>& tab,
                double& h, int& P) {
  const double pi = 3.141592653589793238462643383279502884;
  const double t_max = qd.t[qd.q - 1] > qd.t[0] ? qd.t[qd.q - 1] : qd.t[0];
  double hh = t_max > 0.0 ? 2.0 / t_max : tau_max;
  for (int attempt = 0; attempt < 12; ++attempt, hh *= 0.5) {
    const int np = (int)std::ceil(tau_max * (1.0 + 1e-12) / hh) + 1;
    if (np > 4096) return false;
    std::vector<double> c((size_t)np * (D + 1));
    std::vector<double> fv(D + 1);
    for (int p = 0; p < np; ++p) {
      const double a = p * hh;
      for (int j = 0; j <= D; ++j) {
        const double xj = std::cos(pi * (j + 0.5) / (D + 1));
        fv[j] = psihat_quad(qd, a + 0.5 * (xj + 1.0) * hh);
      }
      for (int n = 0; n <= D; ++n) {
        double acc = 0.0;
        for (int j = 0; j <= D; ++j) acc += fv[j] * std::cos(pi * n * (j + 0.5) / (D + 1));
        c[(size_t)p * (D + 1) + n] = (n == 0 ? 1.0 : 2.0) * acc / (D + 1);
      }
    }
    bool ok = true;
    for (int p = 0; p < np && ok; ++p) {
      const double* cp = c.data() + (size_t)p * (D + 1);
      for (int m = 0; m <= 16 && ok; ++m) {
        const double x = -1.0 + 2.0 * m / 16.0;
        double b1 = 0.0, b2 = 0.0;
        for (int n = D; n >= 1; --n) {
          const double b0 = 2.0 * x * b1 - b2 + cp[n];
          b2 = b1;
          b1 = b0;
        }
        const double approx = x * b1 - b2 + cp[0];
        const double exact = psihat_quad(qd, p * hh + 0.5 * (x + 1.0) * hh);
        if (!(std::fabs(approx - exact) <= rel_tol * std::fabs(exact))) ok = false;
      }
    }
    if (ok) {
      tab.swap(c);
      h = hh;
      P = np;
      return true;
    }
  }
  return false;
}

template <typename TX, typename TC>
cudaError_t launch_t3_post_factors(int dim, int64_t N, const TX* const* sx, const double* cx,
                                   const double* const* tau, int iflag, int w, double beta,
                                   int shape, void* fac, cudaStream_t s, double tau_max,
                                   T3PsihatCache* cache) {
  if (N == 0) return cudaSuccess;
  const double pi = 3.141592653589793238462643383279502884;
  Quad qd;
  qd.q = 2 * w + 10;
  double xg[kMaxQuad], wg[kMaxQuad];
  gauss_legendre(qd.q, xg, wg);
  for (int i = 0; i < qd.q; ++i) {
    const double th = (xg[i] + 1.0) * pi / 4.0;
    const double wt = wg[i] * pi / 4.0;
    qd.t[i] = 0.5 * w * sin(th);
    qd.f[i] = 2.0 * wt * kernel_of_s(shape, beta, cos(th)) * 0.5 * w * cos(th);
  }
  Ptrs3 sp{};
  CDPtrs3 tp{};
  double c[3] = {0, 0, 0};
  for (int d = 0; d < dim; ++d) {
    sp.p[d] = sx[d];
    tp.p[d] = tau[d];
    c[d] = cx[d];
  }
  std::vector<double> tab;
  double h = 0.0;
  int P = 0;
  constexpr int D = 20;
  const int single = sizeof(TC) == 4;
  // a table fitted for a larger |tau| bound covers this one (same kernel)
  if (cache && cache->fitted && tau_max <= cache->tau_max && cache->beta == beta &&
      cache->w == w && cache->shape == shape && cache->single == single) {
    t3_post_table_kernel<TX, TC><<<grid1(N, 128), 128, 0, s>>>(
        dim, N, sp, c[0], c[1], c[2], tp, iflag, cache->dev, cache->h, cache->P, D,
        (cplx_t<TC>*)fac);
    note_launch();
    return cudaGetLastError();
  }
  if (cache) cache->fitted = false;
  if (tau_max > 0.0 && fit_psihat(qd, tau_max, single ? 1e-9 : 1e-14, D, tab, h, P)) {
    if (cache) {
      // keep the table: a plan-owned device buffer, grown when needed
      cudaError_t e = cudaSuccess;
      if (cache->cap < tab.size()) {
        if (cache->dev) cudaFree(cache->dev);
        cache->dev = nullptr;
        cache->cap = 0;
        e = cudaMalloc(&cache->dev, tab.size() * sizeof(double));
        if (e != cudaSuccess) return e;
        cache->cap = tab.size();
      }
      // pageable source: the call returns once the host buffer has been consumed
      e = cudaMemcpyAsync(cache->dev, tab.data(), tab.size() * sizeof(double),
                          cudaMemcpyHostToDevice, s);
      if (e != cudaSuccess) return e;
      cache->fitted = true;
      cache->tau_max = tau_max;
      cache->beta = beta;
      cache->w = w;
      cache->shape = shape;
      cache->single = single;
      cache->h = h;
      cache->P = P;
      t3_post_table_kernel<TX, TC><<<grid1(N, 128), 128, 0, s>>>(
          dim, N, sp, c[0], c[1], c[2], tp, iflag, cache->dev, h, P, D, (cplx_t<TC>*)fac);
      note_launch();
      return cudaGetLastError();
    }
    double* dtab = nullptr;
    cudaError_t e = cudaMallocAsync(&dtab, tab.size() * sizeof(double), s);
    if (e != cudaSuccess) return e;
    // pageable source: the call returns once the host buffer has been consumed
    e = cudaMemcpyAsync(dtab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    t3_post_table_kernel<TX, TC><<<grid1(N, 128), 128, 0, s>>>(
        dim, N, sp, c[0], c[1], c[2], tp, iflag, dtab, h, P, D, (cplx_t<TC>*)fac);
    note_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaFreeAsync(dtab, s);
  }
  t3_post_kernel<TX, TC><<<grid1(N, 128), 128, 0, s>>>(dim, N, sp, c[0], c[1], c[2], tp, iflag,
                                                       qd, (cplx_t<TC>*)fac);
  note_launch();
  return cudaGetLastError();
}

template <typename TI, typename TO, typename TF>
cudaError_t launch_cmul(int64_t n, int ntr, const void* in, const void* fac, void* out,
                        cudaStream_t s, bool conj) {
  if (n == 0 || ntr == 0) return cudaSuccess;
  cmul_kernel<TI, TO, TF><<<grid1(n, 256), 256, 0, s>>>(n, ntr, (const cplx_t<TI>*)in,
                                                        (const cplx_t<TF>*)fac,
                                                        (cplx_t<TO>*)out, conj ? 1 : 0);
  note_launch();
  return cudaGetLastError();
}

template <typename TC>
cudaError_t launch_item_prefix(const BatchProb<TC>* probs, int K, int T, int64_t* item_start,
                               cudaStream_t s) {
  item_prefix_kernel<TC><<<1, 1024, 0, s>>>(probs, K, T, item_start);
  note_launch();
  return cudaGetLastError();
}
template cudaError_t launch_item_prefix<float>(const BatchProb<float>*, int, int, int64_t*,
                                               cudaStream_t);
template cudaError_t launch_item_prefix<double>(const BatchProb<double>*, int, int, int64_t*,
                                                cudaStream_t);

// explicit instantiations
#define GBN_INST_FOLD(TX, TC)                                                                 \
  template cudaError_t launch_fold<TX, TC>(const Geom&, const FoldSpec&, int64_t, const TX*, \
                                           const TX*, const TX*, SortState&, cudaStream_t);
GBN_INST_FOLD(float, float)
GBN_INST_FOLD(double, float)
GBN_INST_FOLD(double, double)
template cudaError_t launch_sort_finish<float>(const Geom&, int64_t, SortState&, bool,
                                               cudaStream_t);
template cudaError_t launch_sort_finish<double>(const Geom&, int64_t, SortState&, bool,
                                                cudaStream_t);
#define GBN_INST_DECONV(TC, TD)                                                               \
  template cudaError_t launch_deconv1<TC, TD>(int, const int64_t*, const int64_t*, int,       \
                                              const TC* const*, const void*, void*, int,      \
                                              cudaStream_t);                                  \
  template cudaError_t launch_deconv2<TC, TD>(int, const int64_t*, const int64_t*, int,       \
                                              const TC* const*, const void*, void*, int,      \
                                              cudaStream_t);
GBN_INST_DECONV(float, float)
GBN_INST_DECONV(float, double)
GBN_INST_DECONV(double, double)
template cudaError_t launch_minmax<float>(const float* const*, int, int64_t, double*,
                                          cudaStream_t);
template cudaError_t launch_minmax<double>(const double* const*, int, int64_t, double*,
                                           cudaStream_t);
template cudaError_t launch_extent_check<float>(int, int64_t, const float* const*,
                                                const double*, const double*, unsigned*,
                                                cudaStream_t);
template cudaError_t launch_extent_check<double>(int, int64_t, const double* const*,
                                                 const double*, const double*, unsigned*,
                                                 cudaStream_t);
template cudaError_t launch_t3_targets<float>(int, int64_t, const float* const*, const double*,
                                              const double*, double* const*, cudaStream_t);
template cudaError_t launch_t3_targets<double>(int, int64_t, const double* const*,
                                               const double*, const double*, double* const*,
                                               cudaStream_t);
#define GBN_INST_T3(TX, TC)                                                                    \
  template cudaError_t launch_t3_prephase_factors<TX, TC>(int, int64_t, const TX* const*,      \
                                                          const double*, const double*, int,   \
                                                          void*, cudaStream_t);                \
  template cudaError_t launch_t3_post_factors<TX, TC>(int, int64_t, const TX* const*,          \
                                                      const double*, const double* const*,     \
                                                      int, int, double, int, void*,            \
                                                      cudaStream_t, double, T3PsihatCache*);
GBN_INST_T3(float, float)
GBN_INST_T3(double, float)
GBN_INST_T3(double, double)
#define GBN_INST_CMUL(TI, TO, TF)                                                             \
  template cudaError_t launch_cmul<TI, TO, TF>(int64_t, int, const void*, const void*, void*, \
                                               cudaStream_t, bool);
GBN_INST_CMUL(float, float, float)
GBN_INST_CMUL(double, float, float)
GBN_INST_CMUL(float, double, float)
GBN_INST_CMUL(double, double, double)

}  // namespace gbn
