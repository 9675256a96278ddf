// gbn_grad.cu -- fused gradient kernels (the adjoint of a type-1/type-2 NUFFT
// with respect to its strengths/modes and its point coordinates).
//
// The reference differentiates through separate transforms issued by its JVP
// and transpose rules (src/jax_finufft/ops.py:158-314): for d point
// coordinates, d stacked ik-weighted transforms plus one transform for the
// strengths, each call re-sorting the points.  Here one point set (the
// forward's sort) serves every gradient, the d+1 weighted grids are written
// in a single pass over the modes and transformed by one batched cuFFT, and
// a single interpolation pass gathers, per point, the values of all grids
// with kernel weights evaluated once and combines them into the strength
// gradient and every coordinate gradient at once.  Kernel weights are
// recomputed from the sorted records, never stored.
#include <cuda_runtime.h>

#include "gbn_common.cuh"
#include "gbn_device.cuh"

namespace gbn {

namespace {

__device__ __forceinline__ int64_t mode_freq_d(int64_t i, int64_t N, int modeord) {
  if (modeord == 0) return i - N / 2;
  return i < (N + 1) / 2 ? i : i - N;
}

__device__ __forceinline__ int64_t fine_to_mode_d(int64_t g, int64_t N, int64_t nf, int modeord) {
  int64_t k;
  if (g <= (N - 1) / 2)
    k = g;
  else if (g >= nf - N / 2)
    k = g - nf;
  else
    return -1;
  if (modeord == 0) return k + N / 2;
  return k >= 0 ? k : k + N;
}

// For every fine cell: the mode it holds (or zero padding), divided by the
// kernel's Fourier transform, times E weights: grid e gets factor 1 when
// e < base, else a * k_{dims[e]} (k the integer frequency along that axis,
// a = 1 or i*iflag).  Output grids are (t*E + e)*nftot + cell.  One block
// per item = up to 512 cells of one fine-grid row; each thread writes two
// neighbouring cells of every grid (16-byte stores in FP32).
template <typename TC, typename TD, int DIM, int E>
__global__ void __launch_bounds__(256)
    deconv2w_kernel(int N0, int N1, int N2, int nf0, int nf1, int nf2, int modeord,
                    const TC* __restrict__ p0, const TC* __restrict__ p1,
                    const TC* __restrict__ p2, const cplx_t<TD>* __restrict__ in,
                    cplx_t<TC>* __restrict__ grids, int ntr, int64_t nftot, int64_t Ntot,
                    int base, int4 dims, TC a_re, TC a_im) {
  const int dd[4] = {dims.x, dims.y, dims.z, dims.w};
  const int nrows = nf1 * nf2;
  const int npair = nf0 >> 1;  // nf0 is even
  const int nchunk = (npair + blockDim.x - 1) / blockDim.x;
  for (int item = blockIdx.x; item < nrows * nchunk; item += gridDim.x) {
    const int row = item / nchunk, chunk = item - row * nchunk;
    const int g1 = DIM > 1 ? row % nf1 : 0;
    const int g2 = DIM > 2 ? row / nf1 : 0;
    const int i1 = DIM > 1 ? (int)fine_to_mode_d(g1, N1, nf1, modeord) : 0;
    const int i2 = DIM > 2 ? (int)fine_to_mode_d(g2, N2, nf2, modeord) : 0;
    const bool live = i1 >= 0 && i2 >= 0;
    TC f12 = TC(1), k1 = TC(0), k2 = TC(0);
    if (live) {
      if (DIM > 1) {
        f12 *= p1[i1];
        k1 = (TC)mode_freq_d(i1, N1, modeord);
      }
      if (DIM > 2) {
        f12 *= p2[i2];
        k2 = (TC)mode_freq_d(i2, N2, modeord);
      }
    }
    const int q = chunk * blockDim.x + threadIdx.x;
    if (q >= npair) continue;
    const int g0 = 2 * q;
    int ia[2] = {-1, -1};
    TC fa[2] = {TC(0), TC(0)}, k0[2] = {TC(0), TC(0)};
    if (live) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        ia[h] = (int)fine_to_mode_d(g0 + h, N0, nf0, modeord);
        if (ia[h] >= 0) {
          fa[h] = p0[ia[h]] * f12;
          k0[h] = (TC)mode_freq_d(ia[h], N0, modeord);
        }
      }
    }
    const int64_t src_row = live ? ((int64_t)i2 * N1 + i1) * N0 : 0;
    const int64_t dst = (int64_t)row * nf0 + g0;
    for (int t = 0; t < ntr; ++t) {
      TC vr[2] = {TC(0), TC(0)}, vi[2] = {TC(0), TC(0)};
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (ia[h] >= 0) {
          const cplx_t<TD> v = in[t * Ntot + src_row + ia[h]];
          vr[h] = (TC)v.x * fa[h];
          vi[h] = (TC)v.y * fa[h];
        }
      }
#pragma unroll
      for (int e = 0; e < E; ++e) {
        cplx_t<TC> o[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          if (e < base) {
            o[h].x = vr[h];
            o[h].y = vi[h];
          } else {
            const TC kk = dd[e] == 0 ? k0[h] : dd[e] == 1 ? k1 : k2;
            const TC wr = a_re * kk, wi = a_im * kk;
            o[h].x = vr[h] * wr - vi[h] * wi;
            o[h].y = vr[h] * wi + vi[h] * wr;
          }
        }
        cplx_t<TC>* d = grids + (int64_t)(t * E + e) * nftot + dst;
        if constexpr (sizeof(TC) == 4) {
          *reinterpret_cast<float4*>(d) = make_float4(o[0].x, o[0].y, o[1].x, o[1].y);
        } else {
          d[0] = o[0];
          d[1] = o[1];
        }
      }
    }
  }
}

struct SubArgs {
  const int* sub_bin;
  const int* sub_off;
  const int* n_sub;
  const int* bin_start;
  const int* bin_count;
  const int* perm;
  int sorted;
};

__device__ __forceinline__ bool sub_range(const SubArgs& sa, const Geom& g, int64_t M, int sub,
                                          int& start, int& cnt) {
  if (sa.sorted) {
    if (sub >= *sa.n_sub) return false;
    const int bin = sa.sub_bin[sub];
    const int off = sa.sub_off[sub];
    start = sa.bin_start[bin] + off;
    cnt = min(sa.bin_count[bin] - off, g.maxsub);
  } else {
    const int64_t s0 = (int64_t)sub * g.maxsub;
    if (s0 >= M) return false;
    start = (int)s0;
    cnt = (int)min((int64_t)g.maxsub, M - s0);
  }
  return cnt > 0;
}


// One pass over the points gathering E grids per transform with shared
// kernel weights.  mode 0 (type-1 gradient): grid 0 (when base) is the
// strength gradient, grid e >= base contributes
// iflag*(Re c * Im h - Im c * Re h) to the gradient of axis dims[e];
// mode 1 (type-2 coordinate gradient): Re(conj(g) h).  Summed over the
// transforms; added to gx (which the caller zeroes).
template <typename TC, typename TD, int DIM, int G, int E>
__global__ void __launch_bounds__(kThreads)
    interp_grad_kernel(Geom g, KerSpec<TC> ks, int64_t M, const PtRec<TC, DIM>* __restrict__ recs,
                       SubArgs sa, const cplx_t<TC>* __restrict__ grids, int ntr, int64_t nftot,
                       int mode, int iflag, int base, int4 dims, GradOut<TD> go) {
  constexpr int NCO = GroupCfg<G>::NCO;
  constexpr int PPW = 32 / G;
  constexpr int NWARP = kThreads / 32;
  int start, cnt;
  if (!sub_range(sa, g, M, blockIdx.x, start, cnt)) return;
  const int w = g.w;
  const int lane = threadIdx.x & 31, grp = lane / G, gl = lane % G, warp = threadIdx.x >> 5;
  TC co[NCO];
  load_coef<TC, NCO>(co, ks, gl, w);
  const bool lane_on = gl < w;
  const int nf0 = (int)g.nf[0], nf1 = (int)g.nf[1], nf2 = (int)g.nf[2];
  const int dd[4] = {dims.x, dims.y, dims.z, dims.w};
  for (int pb = warp * PPW; pb < cnt; pb += NWARP * PPW) {
    const int pi = pb + grp;
    const bool valid = pi < cnt && grp < PPW;
    const int js = start + (valid ? pi : 0);
    const PtRec<TC, DIM> r = recs[js];
    const int idx = sa.perm ? sa.perm[js] : js;
    const TC kx = kerval<TC, NCO>(co, ks, r.d[0], gl, w);
    const TC ky = DIM > 1 ? kerval<TC, NCO>(co, ks, r.d[1], gl, w) : TC(1);
    const TC kz = DIM > 2 ? kerval<TC, NCO>(co, ks, r.d[2], gl, w) : TC(1);
    const int gx = wrap_i32(r.i[0] + gl, nf0);
    const int wy = DIM > 1 ? w : 1, wz = DIM > 2 ? w : 1;
    TC acc[3] = {TC(0), TC(0), TC(0)};
    for (int t = 0; t < ntr; ++t) {
      TC hr[E], hi[E];
#pragma unroll
      for (int e = 0; e < E; ++e) hr[e] = hi[e] = TC(0);
      const cplx_t<TC>* gt = grids + (int64_t)t * E * nftot;
      for (int iz = 0; iz < wz; ++iz) {
        const TC kzv = DIM > 2 ? __shfl_sync(0xffffffffu, kz, grp * G + iz) : TC(1);
        const int gz = DIM > 2 ? wrap_i32(r.i[2] + iz, nf2) : 0;
        for (int iy = 0; iy < wy; ++iy) {
          const TC kyv = DIM > 1 ? __shfl_sync(0xffffffffu, ky, grp * G + iy) : TC(1);
          const int gy = DIM > 1 ? wrap_i32(r.i[1] + iy, nf1) : 0;
          if (lane_on) {
            const TC wgt = kyv * kzv;
            const int cell = (gz * nf1 + gy) * nf0 + gx;
#pragma unroll
            for (int e = 0; e < E; ++e) {
              const cplx_t<TC> v = gt[(int64_t)e * nftot + cell];
              hr[e] = fma(v.x, wgt, hr[e]);
              hi[e] = fma(v.y, wgt, hi[e]);
            }
          }
        }
      }
#pragma unroll
      for (int e = 0; e < E; ++e) {
        hr[e] *= kx;
        hi[e] *= kx;
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
          hr[e] += __shfl_xor_sync(0xffffffffu, hr[e], o);
          hi[e] += __shfl_xor_sync(0xffffffffu, hi[e], o);
        }
      }
      if (valid && gl == 0) {
        const cplx_t<TD> wv = go.w[(int64_t)t * M + idx];
        const TC wr = (TC)wv.x, wi = (TC)wv.y;
#pragma unroll
        for (int e = 0; e < E; ++e) {
          if (e < base) {
            if (go.out_c) {
              cplx_t<TD> o;
              o.x = (TD)hr[e];
              o.y = (TD)hi[e];
              go.out_c[(int64_t)t * M + idx] = o;
            }
          } else {
            const TC v = mode == 0 ? (TC)iflag * (wr * hi[e] - wi * hr[e])
                                   : wr * hr[e] + wi * hi[e];
            const int d = dd[e];
            acc[0] += d == 0 ? v : TC(0);
            acc[1] += d == 1 ? v : TC(0);
            acc[2] += d == 2 ? v : TC(0);
          }
        }
      }
    }
    if (valid && gl == 0) {
#pragma unroll
      for (int d = 0; d < 3; ++d)
        if (go.gx[d]) go.gx[d][idx] += (TD)acc[d];
    }
  }
}

template <typename TC, typename TD, int DIM, int G, int E>
cudaError_t run_interp_grad_s(const Geom& g, const KerSpec<TC>& ks, int64_t M,
                              const SortState& st, const void* grids, int ntr, int mode,
                              int iflag, int base, const int* dims, const void* w, void* out_c,
                              void* const* gx, cudaStream_t s) {
  SubArgs sa;
  sa.sub_bin = st.sub_bin;
  sa.sub_off = st.sub_off;
  sa.n_sub = st.n_sub;
  sa.bin_start = st.bin_start;
  sa.bin_count = st.bin_count;
  sa.perm = st.perm;
  sa.sorted = st.perm != nullptr;
  const int64_t nblk = sa.sorted ? st.max_sub : (M + g.maxsub - 1) / g.maxsub;
  if (nblk == 0) return cudaSuccess;
  int64_t nftot = 1;
  for (int d = 0; d < DIM; ++d) nftot *= g.nf[d];
  GradOut<TD> go;
  go.w = (const cplx_t<TD>*)w;
  go.out_c = (cplx_t<TD>*)out_c;
  for (int d = 0; d < 3; ++d) go.gx[d] = gx ? (TD*)gx[d] : nullptr;
  const PtRec<TC, DIM>* recs = (const PtRec<TC, DIM>*)(sa.sorted ? st.recs : st.recs_in);
  interp_grad_kernel<TC, TD, DIM, G, E><<<(unsigned)nblk, kThreads, 0, s>>>(
      g, ks, M, recs, sa, (const cplx_t<TC>*)grids, ntr, nftot, mode, iflag, base,
      make_int4(dims[0], dims[1], dims[2], dims[3]), go);
  return cudaGetLastError();
}

}  // namespace

template <typename TC, typename TD>
cudaError_t launch_deconv2w(int dim, const int64_t* N, const int64_t* nf, int modeord,
                            const TC* const* phi, const void* in, void* grids, int ntr, int E,
                            int base, const int* dims, double a_re, double a_im,
                            cudaStream_t s) {
  const int64_t nftot = nf[0] * nf[1] * nf[2], Ntot = N[0] * N[1] * N[2];
  const int64_t items = nf[1] * nf[2] * ((nf[0] / 2 + 255) / 256);
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const unsigned grid = (unsigned)(items < (int64_t)nsm * 16 ? items : (int64_t)nsm * 16);
  const TC* p1 = dim > 1 ? phi[1] : nullptr;
  const TC* p2 = dim > 2 ? phi[2] : nullptr;
  const int4 dv = make_int4(dims[0], dims[1], dims[2], dims[3]);
  auto go = [&](auto kern) {
    kern<<<grid, 256, 0, s>>>((int)N[0], (int)N[1], (int)N[2], (int)nf[0], (int)nf[1],
                              (int)nf[2], modeord, phi[0], p1, p2, (const cplx_t<TD>*)in,
                              (cplx_t<TC>*)grids, ntr, nftot, Ntot, base, dv, (TC)a_re, (TC)a_im);
  };
#define GBN_D2W(D)                                 \
  switch (E) {                                     \
    case 1: go(deconv2w_kernel<TC, TD, D, 1>); break; \
    case 2: go(deconv2w_kernel<TC, TD, D, 2>); break; \
    case 3: go(deconv2w_kernel<TC, TD, D, 3>); break; \
    default: go(deconv2w_kernel<TC, TD, D, 4>); break; \
  }
  switch (dim) {
    case 1:
      GBN_D2W(1);
      break;
    case 2:
      GBN_D2W(2);
      break;
    default:
      GBN_D2W(3);
      break;
  }
#undef GBN_D2W
  note_launch();
  return cudaGetLastError();
}

template <typename TC, typename TD>
cudaError_t launch_interp_grad(const Geom& g, const KerSpec<TC>& ks, int64_t M,
                               const SortState& st, const void* grids, int ntr, int E, int mode,
                               int iflag, int base, const int* dims, const void* w, void* out_c,
                               void* const* gx, bool shared, cudaStream_t s,
                               const CUtensorMap* tmap) {
  if (M == 0) return cudaSuccess;
  const bool wide = g.w > 8;
  cudaError_t e = cudaSuccess;
  if (shared && st.perm != nullptr && (int64_t)ntr * E <= 65535) {
    GradOut<TD> go;
    go.w = (const cplx_t<TD>*)w;
    go.out_c = (cplx_t<TD>*)out_c;
    for (int d = 0; d < 3; ++d) go.gx[d] = gx ? (TD*)gx[d] : nullptr;
    return launch_interp_grad_sm<TC, TD>(g, ks, M, st, grids, ntr, E, mode, iflag, base, dims,
                                         go, tmap, s);
  }
#define GBN_IG(D, GG)                                                                          \
  switch (E) {                                                                                 \
    case 1: e = run_interp_grad_s<TC, TD, D, GG, 1>(g, ks, M, st, grids, ntr, mode, iflag, base, dims, w, out_c, gx, s); break; \
    case 2: e = run_interp_grad_s<TC, TD, D, GG, 2>(g, ks, M, st, grids, ntr, mode, iflag, base, dims, w, out_c, gx, s); break; \
    case 3: e = run_interp_grad_s<TC, TD, D, GG, 3>(g, ks, M, st, grids, ntr, mode, iflag, base, dims, w, out_c, gx, s); break; \
    default: e = run_interp_grad_s<TC, TD, D, GG, 4>(g, ks, M, st, grids, ntr, mode, iflag, base, dims, w, out_c, gx, s); break; \
  }
  switch (g.dim) {
    case 1:
      if (wide) { GBN_IG(1, 16) } else { GBN_IG(1, 8) }
      break;
    case 2:
      if (wide) { GBN_IG(2, 16) } else { GBN_IG(2, 8) }
      break;
    default:
      if (wide) { GBN_IG(3, 16) } else { GBN_IG(3, 8) }
      break;
  }
#undef GBN_IG
  note_launch();
  return e;
}

#define GBN_INST_GRAD(TC, TD)                                                                  \
  template cudaError_t launch_deconv2w<TC, TD>(int, const int64_t*, const int64_t*, int,       \
                                               const TC* const*, const void*, void*, int, int, \
                                               int, const int*, double, double, cudaStream_t); \
  template cudaError_t launch_interp_grad<TC, TD>(const Geom&, const KerSpec<TC>&, int64_t,    \
                                                  const SortState&, const void*, int, int, int, \
                                                  int, int, const int*, const void*, void*,     \
                                                  void* const*, bool, cudaStream_t,             \
                                                  const CUtensorMap*);
GBN_INST_GRAD(float, float)
GBN_INST_GRAD(float, double)
GBN_INST_GRAD(double, double)

}  // namespace gbn
