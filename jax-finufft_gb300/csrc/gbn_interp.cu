// gbn_interp.cu -- type-2 interpolation (fine grid -> nonuniform values).
//
// Replaces cuFINUFFT's interp stage.  Same work decomposition as the spread:
// G lanes per point, lane gl owning x offset gl; each lane gathers its
// column of w^(d-1) cells weighted by the broadcast y/z kernel values, then
// the G partial sums are reduced with xor shuffles and one lane writes the
// result to the point's original position.
//
//   method 2 (SM): the block first stages its bin's tile from the fine grid
//     into shared memory -- one bulk tensor copy (TMA, FP32) when the tile
//     does not wrap around the grid, else a cell loop with periodic wrap --
//     so the gathers never touch HBM.
//   method 1 (GM): gathers straight from the fine grid through L1/L2.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "gbn_common.cuh"
#include "gbn_device.cuh"

namespace gbn {

namespace {

// Bounded waits that gave up: counted on the device (read_wait_timeouts)
// and raised in a word of mapped pinned host memory (g_wait_host, set up per
// device by wait_flag_setup), which the host reads on every API call without
// synchronising.
__device__ unsigned g_wait_timeouts;
__device__ unsigned* g_wait_host;
constexpr int kWaitPolls = 1 << 20;

// Grids per shared-memory interpolation block: up to four stacked grids share
// each point's record and kernel values (FP32, groups of at most 8 lanes,
// while the block's tiles stay within 100 KB of shared memory).
template <typename TC, int G>
int grids_per_block(int ngrid, size_t tile_bytes) {
  if (sizeof(TC) != 4 || G > 8) return 1;
  if (ngrid >= 3 && 4 * tile_bytes <= 100 * 1024) return 4;
  if (ngrid >= 2 && 2 * tile_bytes <= 100 * 1024) return 2;
  return 1;
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
                                          int& start, int& cnt, int& bin) {
  if (sa.sorted) {
    if (sub >= *sa.n_sub) return false;
    bin = sa.sub_bin[sub];
    const int off = sa.sub_off[sub];
    start = sa.bin_start[bin] + off;
    cnt = min(sa.bin_count[bin] - off, g.maxsub);
  } else {
    const int64_t s0 = (int64_t)sub * g.maxsub;
    if (s0 >= M) return false;
    bin = 0;
    start = (int)s0;
    cnt = (int)min((int64_t)g.maxsub, M - s0);
  }
  return cnt > 0;
}

template <typename TC, int G>
__device__ __forceinline__ void group_reduce(TC& a, TC& b) {
  if constexpr ((G & (G - 1)) == 0) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
  } else {
    // tree towards the group's first lane, skipping partners past the group
    constexpr int P = G > 8 ? 8 : G > 4 ? 4 : G > 2 ? 2 : 1;
    const int gl = (threadIdx.x & 31) % G;
#pragma unroll
    for (int o = P; o > 0; o >>= 1) {
      const TC ta = __shfl_down_sync(0xffffffffu, a, o);
      const TC tb = __shfl_down_sync(0xffffffffu, b, o);
      if (gl + o < G) {
        a += ta;
        b += tb;
      }
    }
  }
}

// Epilogue of the gather: the interpolated value of a point (input index
// idx) from the block's grid slot k goes to transform t0 + k of the output.
template <typename TC, typename TD>
struct StoreOut {
  cplx_t<TD>* c;
  int64_t M;
  int t0;
  __device__ __forceinline__ void operator()(int k, int idx, TC ar, TC ai) const {
    cplx_t<TD> o;
    o.x = (TD)ar;
    o.y = (TD)ai;
    c[(int64_t)(t0 + k) * M + idx] = o;
  }
};

// Epilogue of the fused gradient gather for grid g0 + k = t*E + e (grid e of
// transform t): e < base stores the value as the strength gradient;
// otherwise the coordinate gradient of axis dims[e] gets Re(conj-weighted)
// terms against the weights w (mode 0, type-1 plan: iflag * (w_re*v_im -
// w_im*v_re); mode 1, type-2 plan: w_re*v_re + w_im*v_im), added atomically
// when several transforms share the gradient, else stored.
template <typename TC, typename TD>
struct GradEpi {
  cplx_t<TD>* out[4];      // slot k: strength gradient of its transform, or null
  TD* gx[4];               // slot k: coordinate gradient of its axis, or null
  const cplx_t<TD>* w[4];  // slot k: weights of its transform
  int mode, iflag, atomic;
  __device__ __forceinline__ void operator()(int k, int idx, TC ar, TC ai) const {
    if (out[k]) {
      cplx_t<TD> o;
      o.x = (TD)ar;
      o.y = (TD)ai;
      out[k][idx] = o;
      return;
    }
    if (!gx[k]) return;
    const cplx_t<TD> wv = w[k][idx];
    const TC wr = (TC)wv.x, wi = (TC)wv.y;
    const TC v = mode == 0 ? (TC)iflag * (wr * ai - wi * ar) : wr * ar + wi * ai;
    if (atomic)
      atomicAdd(&gx[k][idx], (TD)v);
    else
      gx[k][idx] = (TD)v;
  }
};

// Stage the bin tile of grids t .. t+ntb-1 into shared memory (tile k at
// tiles + k*tile_c): one bulk tensor copy per grid when the tile does not wrap
// (FP32, 2D/3D, with a map), else a cell loop with periodic wrap.  False when
// a bounded wait gave up and the copies never completed: the block must then
// write no output.
template <typename TC, int DIM>
__device__ __forceinline__ bool stage_tiles(const Geom& g, const Tile<DIM>& tl,
                                            cplx_t<TC>* tiles, int tile_c, int t, int ntb,
                                            const cplx_t<TC>* __restrict__ fine, int64_t nftot,
                                            const CUtensorMap* tmap, int t_map) {
  const int ncell = tl.ncell;
  bool staged = false;
  if constexpr (sizeof(TC) == 4 && DIM > 1) {
    if (tmap != nullptr && tl.interior(g) && (smem_addr(tiles) & 127u) == 0 &&
        ((size_t)tile_c * sizeof(cplx_t<TC>)) % 128 == 0) {
      __shared__ alignas(8) uint64_t s_bar;
      if (threadIdx.x == 0) {
        mbar_init(&s_bar, 1);
        mbar_expect_tx(&s_bar, (uint32_t)(ntb * ncell * sizeof(cplx_t<TC>)));
        for (int k = 0; k < ntb; ++k) {
          if (DIM == 2)
            tma_load_2d(tiles + k * tile_c, tmap, &s_bar, 2 * tl.org[0],
                        tl.org[1] + (t_map + k) * (int)g.nf[1]);
          else
            tma_load_3d(tiles + k * tile_c, tmap, &s_bar, 2 * tl.org[0], tl.org[1],
                        tl.org[2] + (t_map + k) * (int)g.nf[2]);
        }
      }
      __syncthreads();  // the barrier is initialised before anyone polls it
      // block-uniform outcome: if any thread gave up, all take the error path
      if (__syncthreads_or(!mbar_wait_bounded(&s_bar, 0, kWaitPolls))) {
        if (threadIdx.x == 0) {
          atomicAdd(&g_wait_timeouts, 1u);
          if (g_wait_host) {
            atomicAdd_system(g_wait_host, 1u);
            __threadfence_system();
          }
        }
        // wait (bounded again) for the copies in flight; a tile that still
        // has not arrived is never read and the block writes no output
        if (__syncthreads_or(!mbar_wait_bounded(&s_bar, 0, kWaitPolls))) return false;
      }
      staged = true;
    }
  }
  if (!staged) {
    const int nf0 = (int)g.nf[0], nf1 = (int)g.nf[1], nf2 = (int)g.nf[2];
    for (int k = 0; k < ntb; ++k) {
      const cplx_t<TC>* ft = fine + (int64_t)(t + k) * nftot;
      cplx_t<TC>* tile = tiles + k * tile_c;
      CellWalk cw(threadIdx.x, kThreads, tl.T[0], tl.T[1]);
      for (int i = threadIdx.x; i < ncell; i += kThreads, cw.next()) {
        const int g0 = wrap_i32(tl.org[0] + cw.c0, nf0);
        const int g1 = DIM > 1 ? wrap_i32(tl.org[1] + cw.c1, nf1) : 0;
        const int g2 = DIM > 2 ? wrap_i32(tl.org[2] + cw.c2, nf2) : 0;
        tile[i] = ft[(g2 * nf1 + g1) * nf0 + g0];
      }
    }
  }
  return true;
}

// One subproblem of ntb <= TB grids t, t+1, ..., executed by the whole block
// (shared by the per-subproblem kernel, the work-queue kernel of batched
// plans and the fused gradient kernel).  Grid t+k is fine + (t+k)*nftot and
// is staged in tile k (shared memory, each tile padded to 128 bytes); a
// point's record and kernel values are computed once for all its grids, and
// its value from grid slot k goes through epi(k, input index, re, im).
// tmap (or null): TMA map of the grids; t_map = grid t's index in it.
template <typename TC, typename TD, int DIM, int G, int TB, typename Epi>
__device__ __forceinline__ void interp_sm_block(const Geom& g, const KerSpec<TC>& ks, int64_t M,
                                                const PtRec<TC, DIM>* __restrict__ recs,
                                                const SubArgs& sa, int sub, int t, int ntb,
                                                const cplx_t<TC>* __restrict__ fine,
                                                const Epi& epi, int64_t nftot,
                                                unsigned char* smem_raw,
                                                const CUtensorMap* tmap = nullptr,
                                                int t_map = 0) {
  constexpr int NCO = GroupCfg<G>::NCO;
  constexpr int PPW = 32 / G;
  constexpr int NWARP = kThreads / 32;
  int start, cnt, bin;
  if (!sub_range(sa, g, M, sub, start, cnt, bin)) return;
  const int w = g.w;
  const Tile<DIM> tl(g, bin);
  const int ncell = tl.ncell;
  const int tile_c = (int)(interp_tile_bytes(DIM, g.bs, w, sizeof(TC) == 4) / sizeof(cplx_t<TC>));
  cplx_t<TC>* tiles = reinterpret_cast<cplx_t<TC>*>(smem_raw);  // tile k at tiles + k*tile_c
  if (!stage_tiles<TC, DIM>(g, tl, tiles, tile_c, t, ntb, fine, nftot, tmap, t_map)) return;
  const int lane = threadIdx.x & 31, grp = lane / G, gl = lane % G, warp = threadIdx.x >> 5;
  TC co[NCO];
  load_coef<TC, NCO>(co, ks, gl, w);
  __syncthreads();

  const bool lane_on = gl < w;
  constexpr int kStep = NWARP * PPW;
  // each group's next point record and output index are loaded one
  // iteration ahead, so their latency hides behind the current gather
  PtRec<TC, DIM> rn;
  int on_next = 0;
  if (warp * PPW < cnt) {
    const int pn = warp * PPW + grp;
    const int jn = start + (pn < cnt ? pn : 0);
    rn = recs[jn];
    on_next = sa.perm ? sa.perm[jn] : jn;
  }
  const int T0 = tl.T[0];
  const int plane = T0 * tl.T[1];
  for (int pb = warp * PPW; pb < cnt; pb += kStep) {
    const int pi = pb + grp;
    const bool valid = pi < cnt && grp < PPW;
    const PtRec<TC, DIM> r = rn;
    const int out_idx = on_next;
    if (pb + kStep < cnt) {
      const int pn = pb + kStep + grp;
      const int jn = start + (pn < cnt ? pn : 0);
      rn = recs[jn];
      on_next = sa.perm ? sa.perm[jn] : jn;
    }
    const TC kx = kerval<TC, NCO>(co, ks, r.d[0], gl, w);
    const int l0 = r.i[0] - tl.org[0] + gl;
    // the group's y (and z) kernel values, fetched once per point
    TC ky = TC(0), kz = TC(0);
    TC kyr[G];
    if (DIM > 1) {
      ky = kerval<TC, NCO>(co, ks, r.d[1], gl, w);
#pragma unroll
      for (int i = 0; i < G; ++i) kyr[i] = __shfl_sync(0xffffffffu, ky, grp * G + i);
    }
    if (DIM > 2) kz = kerval<TC, NCO>(co, ks, r.d[2], gl, w);
    const int cell0 = DIM == 1 ? l0
                      : DIM == 2 ? (r.i[1] - tl.org[1]) * T0 + l0
                                 : ((r.i[2] - tl.org[2]) * tl.T[1] + (r.i[1] - tl.org[1])) * T0 +
                                       l0;
#pragma unroll
    for (int k = 0; k < TB; ++k) {
      if (k >= ntb) break;
      const cplx_t<TC>* tk = tiles + k * tile_c + cell0;
      TC ar = TC(0), ai = TC(0);
      if (DIM == 1) {
        if (lane_on) {
          const cplx_t<TC> v = tk[0];
          ar = v.x;
          ai = v.y;
        }
      } else if (DIM == 2) {
#pragma unroll
        for (int iy = 0; iy < G; ++iy) {
          if (iy < w && lane_on) {
            const cplx_t<TC> v = tk[iy * T0];
            ar = fma(v.x, kyr[iy], ar);
            ai = fma(v.y, kyr[iy], ai);
          }
        }
      } else {
        const cplx_t<TC>* zrow = tk;
        for (int iz = 0; iz < w; ++iz) {
          const TC kzv = __shfl_sync(0xffffffffu, kz, grp * G + iz);
          TC yr = TC(0), yi = TC(0);
#pragma unroll
          for (int iy = 0; iy < G; ++iy) {
            if (iy < w && lane_on) {
              const cplx_t<TC> v = zrow[iy * T0];
              yr = fma(v.x, kyr[iy], yr);
              yi = fma(v.y, kyr[iy], yi);
            }
          }
          ar = fma(yr, kzv, ar);
          ai = fma(yi, kzv, ai);
          zrow += plane;
        }
      }
      ar *= kx;
      ai *= kx;
      group_reduce<TC, G>(ar, ai);
      if (valid && gl == 0) epi(k, out_idx, ar, ai);
    }
  }
}

// Kernel value and its derivative with respect to delta (the Horner
// polynomial and its derivative together, or the direct formula).
template <typename T, int NCO>
__device__ __forceinline__ T kerval_d(const T (&co)[NCO], const KerSpec<T>& ks, T delta,
                                      int piece, int w, T& dval) {
  if (ks.meth == 0) {
    dval = T(0);
    if (piece >= w) return T(0);
    const T t = (T)piece - T(0.5) * (T)w + delta;
    const T z = t * (T(2) / (T)w);
    const T s2 = T(1) - z * z;
    if (!(s2 > T(0))) return T(0);
    const T sq = sqrt(s2);
    const T dsq = -z / sq * (T(2) / (T)w);  // d sqrt(1 - z^2) / dt, dt/d delta = 1
    if (ks.shape == 1) {
      dval = bessel_i1_dev(ks.beta * sq) * ks.beta * dsq * ks.inv_i0b;
      return bessel_i0_dev(ks.beta * sq) * ks.inv_i0b;
    }
    const T v = exp(ks.beta * (sq - T(1)));
    dval = v * ks.beta * dsq;
    return v;
  }
  const T u = T(2) * delta - T(1);
  T v = T(0), dv = T(0);
#pragma unroll
  for (int n = NCO - 1; n >= 0; --n) {
    dv = fma(dv, u, v);
    v = fma(v, u, co[n]);
  }
  dval = T(2) * dv;  // du / d delta = 2
  return v;
}

// Type-3 gradient gather on the outer grid of the adjoint (see t3_adjoint in
// the plan code): for each source point j and transform t, the value I and
// its derivatives J_a along the grid coordinate X_a of the adjoint grid, then
//   H = conj(pre_j) I                      (the strength gradient, stored)
//   dH_a = conj(pre_j) (-i iflag D_a I + scale_a J_a)
//   grad_x_a[j] += Re(c_tj conj(dH_a))     (atomic: summed over transforms)
// with X_a = (x_a - C_a) scale_a + nf_a/2 and pre_j = exp(i iflag D.(x_j - C)).
template <typename TC, typename TD>
struct T3GradArgs {
  const cplx_t<TD>* c;     // forward strengths (ntr, M), null when no gx is asked
  const cplx_t<TC>* pre;   // pre-phase factor of each source (M)
  cplx_t<TD>* grad_c;      // (ntr, M) or null
  TD* gx[3];               // per backend axis: M reals, accumulated, or null
  TC D[3], scale[3];
  int iflag, t0;
};

template <typename TC, typename TD, int DIM, int G>
__global__ void __launch_bounds__(kThreads)
    interp_t3grad_kernel(Geom g, KerSpec<TC> ks, int64_t M,
                         const PtRec<TC, DIM>* __restrict__ recs, SubArgs sa,
                         const cplx_t<TC>* __restrict__ fine, int64_t nftot,
                         T3GradArgs<TC, TD> ga, const __grid_constant__ CUtensorMap tmap,
                         int use_tma, int t_map0) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  constexpr int NCO = GroupCfg<G>::NCO;
  constexpr int PPW = 32 / G;
  constexpr int NWARP = kThreads / 32;
  int start, cnt, bin;
  if (!sub_range(sa, g, M, blockIdx.x, start, cnt, bin)) return;
  const int t = blockIdx.y;  // transform within this launch
  const int w = g.w;
  const Tile<DIM> tl(g, bin);
  const int tile_c = (int)(interp_tile_bytes(DIM, g.bs, w, sizeof(TC) == 4) / sizeof(cplx_t<TC>));
  cplx_t<TC>* tile = reinterpret_cast<cplx_t<TC>*>(smem_raw);
  if (!stage_tiles<TC, DIM>(g, tl, tile, tile_c, t, 1, fine, nftot, use_tma ? &tmap : nullptr,
                            t_map0 + t))
    return;
  const int lane = threadIdx.x & 31, grp = lane / G, gl = lane % G, warp = threadIdx.x >> 5;
  TC co[NCO];
  load_coef<TC, NCO>(co, ks, gl, w);
  __syncthreads();
  const bool lane_on = gl < w;
  const int T0 = tl.T[0];
  const int plane = T0 * tl.T[1];
  const int tg = ga.t0 + t;  // transform index in the caller's arrays
  for (int pb = warp * PPW; pb < cnt; pb += NWARP * PPW) {
    const int pi = pb + grp;
    const bool valid = pi < cnt && grp < PPW;
    const int js = start + (valid ? pi : 0);
    const PtRec<TC, DIM> r = recs[js];
    const int j = sa.perm ? sa.perm[js] : js;
    TC dkx;
    const TC kx = kerval_d<TC, NCO>(co, ks, r.d[0], gl, w, dkx);
    TC kyr[G], dkyr[G];
    TC kz = TC(0), dkz = TC(0);
    if (DIM > 1) {
      TC dky;
      const TC ky = kerval_d<TC, NCO>(co, ks, r.d[1], gl, w, dky);
#pragma unroll
      for (int i = 0; i < G; ++i) {
        kyr[i] = __shfl_sync(0xffffffffu, ky, grp * G + i);
        dkyr[i] = __shfl_sync(0xffffffffu, dky, grp * G + i);
      }
    }
    if (DIM > 2) kz = kerval_d<TC, NCO>(co, ks, r.d[2], gl, w, dkz);
    const int l0 = r.i[0] - tl.org[0] + gl;
    const int cell0 = DIM == 1 ? l0
                      : DIM == 2 ? (r.i[1] - tl.org[1]) * T0 + l0
                                 : ((r.i[2] - tl.org[2]) * tl.T[1] + (r.i[1] - tl.org[1])) * T0 +
                                       l0;
    // a: sum over the lane's rows weighted by ky kz; b: by dky kz; e: by ky dkz
    TC ar = 0, ai = 0, br = 0, bi = 0, er = 0, ei = 0;
    if (DIM == 1) {
      if (lane_on) {
        const cplx_t<TC> v = tile[cell0];
        ar = v.x;
        ai = v.y;
      }
    } else {
      const cplx_t<TC>* zrow = tile + cell0;
      for (int iz = 0; iz < (DIM > 2 ? w : 1); ++iz) {
        const TC kzv = DIM > 2 ? __shfl_sync(0xffffffffu, kz, grp * G + iz) : TC(1);
        const TC dkzv = DIM > 2 ? __shfl_sync(0xffffffffu, dkz, grp * G + iz) : TC(0);
        TC yr = 0, yi = 0, dyr = 0, dyi = 0;
#pragma unroll
        for (int iy = 0; iy < G; ++iy) {
          if (iy < w && lane_on) {
            const cplx_t<TC> v = zrow[iy * T0];
            yr = fma(v.x, kyr[iy], yr);
            yi = fma(v.y, kyr[iy], yi);
            dyr = fma(v.x, dkyr[iy], dyr);
            dyi = fma(v.y, dkyr[iy], dyi);
          }
        }
        ar = fma(yr, kzv, ar);
        ai = fma(yi, kzv, ai);
        br = fma(dyr, kzv, br);
        bi = fma(dyi, kzv, bi);
        er = fma(yr, dkzv, er);
        ei = fma(yi, dkzv, ei);
        zrow += plane;
      }
    }
    // value and the derivatives along backend axes 0, 1, 2 (w.r.t. delta)
    TC vr = ar * kx, vi = ai * kx;
    TC d0r = ar * dkx, d0i = ai * dkx;
    TC d1r = br * kx, d1i = bi * kx;
    TC d2r = er * kx, d2i = ei * kx;
    group_reduce<TC, G>(vr, vi);
    group_reduce<TC, G>(d0r, d0i);
    if (DIM > 1) group_reduce<TC, G>(d1r, d1i);
    if (DIM > 2) group_reduce<TC, G>(d2r, d2i);
    if (!(valid && gl == 0)) continue;
    const cplx_t<TC> pre = ga.pre[j];
    const TC pr = pre.x, pi_ = -pre.y;  // conj(pre)
    if (ga.grad_c) {
      cplx_t<TD> o;
      o.x = (TD)(pr * vr - pi_ * vi);
      o.y = (TD)(pr * vi + pi_ * vr);
      ga.grad_c[(int64_t)tg * M + j] = o;
    }
    if (!ga.c) continue;
    const cplx_t<TD> cv = ga.c[(int64_t)tg * M + j];
    const TC cr = (TC)cv.x, ci = (TC)cv.y;
    const TC sg = (TC)ga.iflag;
    const TC dr[3] = {d0r, d1r, d2r}, di[3] = {d0i, d1i, d2i};
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      if (!ga.gx[a]) continue;
      // q = -i iflag D_a I + scale_a J_a, J_a = -(derivative w.r.t. delta)
      const TC qr = sg * ga.D[a] * vi - ga.scale[a] * dr[a];
      const TC qi = -sg * ga.D[a] * vr - ga.scale[a] * di[a];
      const TC hr = pr * qr - pi_ * qi, hi = pr * qi + pi_ * qr;  // dH_a
      atomicAdd(&ga.gx[a][j], (TD)(cr * hr + ci * hi));          // Re(c conj(dH_a))
    }
  }
}

// grid (subproblems, ceil(ntr / TB)); block y handles transforms TB*y ...
template <typename TC, typename TD, int DIM, int G, int TB>
__global__ void __launch_bounds__(kThreads)
    interp_sm_kernel(Geom g, KerSpec<TC> ks, int64_t M, const PtRec<TC, DIM>* __restrict__ recs,
                     SubArgs sa, const cplx_t<TC>* __restrict__ fine, cplx_t<TD>* __restrict__ c,
                     int64_t nftot, int ntr, const __grid_constant__ CUtensorMap tmap,
                     int use_tma, int t_base) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int t = TB * (int)blockIdx.y;
  const StoreOut<TC, TD> epi{c, M, t};
  interp_sm_block<TC, TD, DIM, G, TB>(g, ks, M, recs, sa, blockIdx.x, t, min(TB, ntr - t), fine,
                                      epi, nftot, smem_raw, use_tma ? &tmap : nullptr,
                                      t_base + t);
}

// Fused gradient gather: block (subproblem, y) gathers grids TB*y ... of
// the ntr*E grids (grid t*E + e) at the subproblem's points into the
// strength or coordinate gradients, with each point's kernel values shared
// by the block's grids.
template <typename TC, typename TD, int DIM, int G, int TB>
__global__ void __launch_bounds__(kThreads)
    interp_grad_sm_kernel(Geom g, KerSpec<TC> ks, int64_t M,
                          const PtRec<TC, DIM>* __restrict__ recs, SubArgs sa,
                          const cplx_t<TC>* __restrict__ grids, int ngrid, int E, int64_t nftot,
                          int mode, int iflag, int base, int4 dims, GradOut<TD> go, int atomic,
                          const __grid_constant__ CUtensorMap tmap, int use_tma) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int g0 = TB * (int)blockIdx.y;
  GradEpi<TC, TD> epi;
  const int dd[4] = {dims.x, dims.y, dims.z, dims.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int gi = g0 + (k < TB ? k : 0), t = gi / E, e = gi - t * E;
    epi.out[k] = e < base && go.out_c ? go.out_c + (int64_t)t * M : nullptr;
    epi.gx[k] = e >= base ? go.gx[dd[e]] : nullptr;
    epi.w[k] = go.w + (int64_t)t * M;
  }
  epi.mode = mode;
  epi.iflag = iflag;
  epi.atomic = atomic;
  interp_sm_block<TC, TD, DIM, G, TB>(g, ks, M, recs, sa, blockIdx.x, g0, min(TB, ngrid - g0),
                                      grids, epi, nftot, smem_raw, use_tma ? &tmap : nullptr, g0);
}

template <typename TC, typename TD, int DIM, int G>
__global__ void __launch_bounds__(kThreads)
    interp_gm_kernel(Geom g, KerSpec<TC> ks, int64_t M, const PtRec<TC, DIM>* __restrict__ recs,
                     SubArgs sa, const cplx_t<TC>* __restrict__ fine, cplx_t<TD>* __restrict__ c,
                     int64_t nftot) {
  constexpr int NCO = GroupCfg<G>::NCO;
  constexpr int PPW = 32 / G;
  constexpr int NWARP = kThreads / 32;
  int start, cnt, bin;
  if (!sub_range(sa, g, M, blockIdx.x, start, cnt, bin)) return;
  const int t = blockIdx.y;
  const int w = g.w;
  const int lane = threadIdx.x & 31, grp = lane / G, gl = lane % G, warp = threadIdx.x >> 5;
  TC co[NCO];
  load_coef<TC, NCO>(co, ks, gl, w);
  const cplx_t<TC>* ft = fine + (int64_t)t * nftot;
  cplx_t<TD>* ct = c + (int64_t)t * M;
  const bool lane_on = gl < w;
  const int nf0 = (int)g.nf[0], nf1 = (int)g.nf[1], nf2 = (int)g.nf[2];
  for (int pb = warp * PPW; pb < cnt; pb += NWARP * PPW) {
    const int pi = pb + grp;
    const bool valid = pi < cnt && grp < PPW;
    const int js = start + (valid ? pi : 0);
    const PtRec<TC, DIM> r = recs[js];
    const TC kx = kerval<TC, NCO>(co, ks, r.d[0], gl, w);
    const int gx = wrap_i32(r.i[0] + gl, nf0);
    TC ar = TC(0), ai = TC(0);
    if (DIM == 1) {
      if (lane_on) {
        const cplx_t<TC> v = ft[gx];
        ar = v.x;
        ai = v.y;
      }
    } else if (DIM == 2) {
      const TC ky = kerval<TC, NCO>(co, ks, r.d[1], gl, w);
      for (int iy = 0; iy < w; ++iy) {
        const TC kyv = __shfl_sync(0xffffffffu, ky, grp * G + iy);
        const int gy = wrap_i32(r.i[1] + iy, nf1);
        if (lane_on) {
          const cplx_t<TC> v = ft[gy * nf0 + gx];
          ar = fma(v.x, kyv, ar);
          ai = fma(v.y, kyv, ai);
        }
      }
    } else {
      const TC ky = kerval<TC, NCO>(co, ks, r.d[1], gl, w);
      const TC kz = kerval<TC, NCO>(co, ks, r.d[2], gl, w);
      for (int iz = 0; iz < w; ++iz) {
        const TC kzv = __shfl_sync(0xffffffffu, kz, grp * G + iz);
        const int gz = wrap_i32(r.i[2] + iz, nf2);
        TC yr = TC(0), yi = TC(0);
        for (int iy = 0; iy < w; ++iy) {
          const TC kyv = __shfl_sync(0xffffffffu, ky, grp * G + iy);
          const int gy = wrap_i32(r.i[1] + iy, nf1);
          if (lane_on) {
            const cplx_t<TC> v = ft[(gz * nf1 + gy) * nf0 + gx];
            yr = fma(v.x, kyv, yr);
            yi = fma(v.y, kyv, yi);
          }
        }
        ar = fma(yr, kzv, ar);
        ai = fma(yi, kzv, ai);
      }
    }
    ar *= kx;
    ai *= kx;
    group_reduce<TC, G>(ar, ai);
    if (valid && gl == 0) {
      cplx_t<TD> o;
      o.x = (TD)ar;
      o.y = (TD)ai;
      ct[sa.perm ? sa.perm[js] : js] = o;
    }
  }
}


template <typename TC, typename TD, int DIM, int G>
__global__ void __launch_bounds__(kThreads)
    interp_queue_kernel(const BatchProb<TC>* __restrict__ probs, int K,
                        const int64_t* __restrict__ item_start, int* counter, int T,
                        const cplx_t<TC>* __restrict__ arena, cplx_t<TD>* __restrict__ c) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ int s_item;
  const int64_t total = item_start[K];
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int64_t item = s_item;
    if (item >= total) break;
    int lo = 0, hi = K - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (item_start[mid] <= item)
        lo = mid;
      else
        hi = mid - 1;
    }
    const BatchProb<TC> P = probs[lo];
    const int64_t local = item - item_start[lo];
    const int sub = (int)(local / T), t = (int)(local - (int64_t)sub * T);
    SubArgs sa{P.sub_bin, P.sub_off, P.n_sub, P.bin_start, P.bin_count, P.perm, 1};
    const StoreOut<TC, TD> epi{c + P.c_off, P.M, t};
    interp_sm_block<TC, TD, DIM, G, 1>(P.g, P.ks, P.M, (const PtRec<TC, DIM>*)P.recs, sa, sub, t,
                                       1, arena + P.grid_off, epi, P.nftot, smem_raw);
  }
}

template <typename TC, typename TD, int DIM, int G>
cudaError_t run_interp_queue(const BatchProb<TC>* probs, int K, const int64_t* item_start,
                             int* counter, int T, const void* arena, void* c, size_t smem,
                             cudaStream_t s) {
  auto kern = interp_queue_kernel<TC, TD, DIM, G>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
  if (per_sm < 1) per_sm = 1;
  kern<<<nsm * per_sm, kThreads, smem, s>>>(probs, K, item_start, counter, T,
                                            (const cplx_t<TC>*)arena, (cplx_t<TD>*)c);
  note_launch();
  return cudaGetLastError();
}

template <typename TC, typename TD, int DIM, int G>
cudaError_t run_interp(const Geom& g, const KerSpec<TC>& ks, int method, int64_t M,
                       const SortState& st, const void* fine, void* c, int ntr,
                       cudaStream_t s, const CUtensorMap* tmap) {
  SubArgs sa;
  sa.sub_bin = st.sub_bin;
  sa.sub_off = st.sub_off;
  sa.n_sub = st.n_sub;
  sa.bin_start = st.bin_start;
  sa.bin_count = st.bin_count;
  sa.perm = st.perm;
  sa.sorted = st.perm != nullptr;
  const int64_t nblk = sa.sorted ? st.max_sub : (M + g.maxsub - 1) / g.maxsub;
  if (nblk == 0 || ntr == 0) return cudaSuccess;
  int64_t nftot = 1;
  for (int d = 0; d < DIM; ++d) nftot *= g.nf[d];
  const PtRec<TC, DIM>* recs = (const PtRec<TC, DIM>*)(sa.sorted ? st.recs : st.recs_in);
  const bool sm = method == 2 && sa.sorted;
  const size_t tile1 = interp_tile_bytes(DIM, g.bs, g.w, sizeof(TC) == 4);
  const int TB = sm ? grids_per_block<TC, G>(ntr, tile1) : 1;
  for (int t0 = 0; t0 < ntr; t0 += 65535 * TB) {
    const int nt = std::min(ntr - t0, 65535 * TB);
    dim3 grid((unsigned)nblk, (unsigned)((nt + TB - 1) / TB));
    const cplx_t<TC>* ft = (const cplx_t<TC>*)fine + (int64_t)t0 * nftot;
    cplx_t<TD>* ct = (cplx_t<TD>*)c + (int64_t)t0 * M;
    if (sm) {
      CUtensorMap m;
      memset(&m, 0, sizeof(m));
      const int use = tmap != nullptr && sizeof(TC) == 4;
      if (use) m = *tmap;
      auto go = [&](auto kern, int tb) -> cudaError_t {
        const size_t smem = tile1 * tb;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        kern<<<grid, kThreads, smem, s>>>(g, ks, M, recs, sa, ft, ct, nftot, nt, m, use, t0);
        note_launch();
        return cudaSuccess;
      };
      cudaError_t e;
      if constexpr (sizeof(TC) == 4 && G <= 8) {
        e = TB == 4   ? go(interp_sm_kernel<TC, TD, DIM, G, 4>, 4)
            : TB == 2 ? go(interp_sm_kernel<TC, TD, DIM, G, 2>, 2)
                      : go(interp_sm_kernel<TC, TD, DIM, G, 1>, 1);
      } else {
        e = go(interp_sm_kernel<TC, TD, DIM, G, 1>, 1);
      }
      if (e != cudaSuccess) return e;
    } else {
      interp_gm_kernel<TC, TD, DIM, G><<<grid, kThreads, 0, s>>>(g, ks, M, recs, sa, ft, ct,
                                                                  nftot);
      note_launch();
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

template <typename TC, typename TD>
cudaError_t launch_interp(const Geom& g, const KerSpec<TC>& ks, int method, int64_t M,
                          const SortState& st, const void* fine, void* c, int ntr,
                          cudaStream_t s, const CUtensorMap* tmap) {
  if (M == 0) return cudaSuccess;
  // lanes per point: the narrowest group that covers the kernel width
  const int G = g.w > 8 ? 16 : g.w > 6 ? 8 : 6;
#define GBN_DISPATCH(DIM, TM)                                        \
  return G == 16 ? run_interp<TC, TD, DIM, 16>(g, ks, method, M, st, fine, c, ntr, s, TM)      \
         : G == 8 ? run_interp<TC, TD, DIM, 8>(g, ks, method, M, st, fine, c, ntr, s, TM)      \
                  : run_interp<TC, TD, DIM, 6>(g, ks, method, M, st, fine, c, ntr, s, TM);
  switch (g.dim) {
    case 1:
      GBN_DISPATCH(1, nullptr)
    case 2:
      GBN_DISPATCH(2, tmap)
    default:
      GBN_DISPATCH(3, tmap)
  }
#undef GBN_DISPATCH
}

template cudaError_t launch_interp<float, float>(const Geom&, const KerSpec<float>&, int,
                                                 int64_t, const SortState&, const void*, void*,
                                                 int, cudaStream_t, const CUtensorMap*);
template cudaError_t launch_interp<float, double>(const Geom&, const KerSpec<float>&, int,
                                                  int64_t, const SortState&, const void*, void*,
                                                  int, cudaStream_t, const CUtensorMap*);
template cudaError_t launch_interp<double, double>(const Geom&, const KerSpec<double>&, int,
                                                   int64_t, const SortState&, const void*,
                                                   void*, int, cudaStream_t, const CUtensorMap*);

template <typename TC, typename TD>
cudaError_t launch_interp_t3grad(const Geom& g, const KerSpec<TC>& ks, int64_t M,
                                 const SortState& st, const void* fine, int nb,
                                 const T3Grad& tg, cudaStream_t s,
                                 const CUtensorMap* tmap) {
  if (M == 0 || nb == 0) return cudaSuccess;
  SubArgs sa;
  sa.sub_bin = st.sub_bin;
  sa.sub_off = st.sub_off;
  sa.n_sub = st.n_sub;
  sa.bin_start = st.bin_start;
  sa.bin_count = st.bin_count;
  sa.perm = st.perm;
  sa.sorted = st.perm != nullptr;
  const int64_t nblk = sa.sorted ? st.max_sub : (M + g.maxsub - 1) / g.maxsub;
  int64_t nftot = 1;
  for (int d = 0; d < g.dim; ++d) nftot *= g.nf[d];
  T3GradArgs<TC, TD> ga;
  ga.c = (const cplx_t<TD>*)tg.c;
  ga.pre = (const cplx_t<TC>*)tg.pre;
  ga.grad_c = (cplx_t<TD>*)tg.grad_c;
  for (int a = 0; a < 3; ++a) {
    ga.gx[a] = (TD*)tg.gx[a];
    ga.D[a] = (TC)tg.D[a];
    ga.scale[a] = (TC)tg.scale[a];
  }
  ga.iflag = tg.iflag;
  ga.t0 = tg.t0;
  const size_t smem = interp_tile_bytes(g.dim, g.bs, g.w, sizeof(TC) == 4);
  CUtensorMap m;
  memset(&m, 0, sizeof(m));
  const int use = tmap != nullptr && sizeof(TC) == 4;
  if (use) m = *tmap;
  const int G = g.w > 8 ? 16 : g.w > 6 ? 8 : 6;
  for (int t0 = 0; t0 < nb; t0 += 65535) {
    dim3 grid((unsigned)nblk, (unsigned)std::min(nb - t0, 65535));
    const cplx_t<TC>* ft = (const cplx_t<TC>*)fine + (int64_t)t0 * nftot;
    T3GradArgs<TC, TD> gb = ga;
    gb.t0 = ga.t0 + t0;
    cudaError_t e = cudaSuccess;
#define GBN_T3G(DIM, GG)                                                                        \
  {                                                                                             \
    auto kern = interp_t3grad_kernel<TC, TD, DIM, GG>;                                          \
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);     \
    if (e == cudaSuccess) {                                                                     \
      kern<<<grid, kThreads, smem, s>>>(g, ks, M, (const PtRec<TC, DIM>*)st.recs, sa, ft,       \
                                        nftot, gb, m, use, t0);                                 \
      note_launch();                                                                            \
    }                                                                                           \
  }
    if (g.dim == 1) {
      if (G == 16) GBN_T3G(1, 16) else if (G == 8) GBN_T3G(1, 8) else GBN_T3G(1, 6)
    } else if (g.dim == 2) {
      if (G == 16) GBN_T3G(2, 16) else if (G == 8) GBN_T3G(2, 8) else GBN_T3G(2, 6)
    } else {
      if (G == 16) GBN_T3G(3, 16) else if (G == 8) GBN_T3G(3, 8) else GBN_T3G(3, 6)
    }
#undef GBN_T3G
    if (e != cudaSuccess) return e;
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}
template cudaError_t launch_interp_t3grad<float, float>(const Geom&, const KerSpec<float>&,
                                                        int64_t, const SortState&, const void*,
                                                        int, const T3Grad&,
                                                        cudaStream_t, const CUtensorMap*);
template cudaError_t launch_interp_t3grad<float, double>(const Geom&, const KerSpec<float>&,
                                                         int64_t, const SortState&, const void*,
                                                         int, const T3Grad&,
                                                         cudaStream_t, const CUtensorMap*);
template cudaError_t launch_interp_t3grad<double, double>(const Geom&, const KerSpec<double>&,
                                                          int64_t, const SortState&,
                                                          const void*, int,
                                                          const T3Grad&,
                                                          cudaStream_t, const CUtensorMap*);

namespace {

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library); null when unavailable.
EncodeTiledFn tiled_encoder() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

}  // namespace

bool tile_tensor_map(const Geom& g, const void* grid, int nb, CUtensorMap* out) {
  if (g.dim < 2 || g.dim > 3 || nb < 1 || grid == nullptr) return false;
  if ((reinterpret_cast<uintptr_t>(grid) & 15) != 0 || (g.nf[0] & 1) != 0) return false;
  const int64_t tx = tile_x(g.bs[0], g.w);
  const int64_t ty = g.bs[1] + g.w - 1, tz = g.bs[2] + g.w - 1;
  cuuint64_t dims[3] = {0, 0, 0}, strides[2] = {0, 0};
  cuuint32_t box[3] = {1, 1, 1}, es[3] = {1, 1, 1};
  dims[0] = (cuuint64_t)(2 * g.nf[0]);
  box[0] = (cuuint32_t)(2 * tx);
  strides[0] = (cuuint64_t)(8 * g.nf[0]);
  if (g.dim == 2) {
    dims[1] = (cuuint64_t)(g.nf[1] * nb);
    box[1] = (cuuint32_t)ty;
  } else {
    dims[1] = (cuuint64_t)g.nf[1];
    dims[2] = (cuuint64_t)(g.nf[2] * nb);
    strides[1] = (cuuint64_t)(8 * g.nf[0] * g.nf[1]);
    box[1] = (cuuint32_t)ty;
    box[2] = (cuuint32_t)tz;
  }
  for (int d = 0; d < g.dim; ++d) {
    if (box[d] > 256 || box[d] > dims[d] || dims[d] > ((cuuint64_t)1 << 32)) return false;
  }
  EncodeTiledFn fn = tiled_encoder();
  if (!fn) return false;
  const CUresult r = fn(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, (cuuint32_t)g.dim,
                        const_cast<void*>(grid), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

namespace {

template <typename TC, typename TD, int DIM, int G>
cudaError_t run_interp_grad_sm(const Geom& g, const KerSpec<TC>& ks, int64_t M,
                               const SortState& st, const void* grids, int ntr, int E, int mode,
                               int iflag, int base, const int* dims, const GradOut<TD>& go,
                               const CUtensorMap* tmap, cudaStream_t s) {
  SubArgs sa;
  sa.sub_bin = st.sub_bin;
  sa.sub_off = st.sub_off;
  sa.n_sub = st.n_sub;
  sa.bin_start = st.bin_start;
  sa.bin_count = st.bin_count;
  sa.perm = st.perm;
  sa.sorted = 1;
  if (st.max_sub == 0) return cudaSuccess;
  int64_t nftot = 1;
  for (int d = 0; d < DIM; ++d) nftot *= g.nf[d];
  const int ngrid = ntr * E;
  const size_t tile1 = interp_tile_bytes(DIM, g.bs, g.w, sizeof(TC) == 4);
  const int TB = grids_per_block<TC, G>(ngrid, tile1);
  CUtensorMap m;
  memset(&m, 0, sizeof(m));
  const int use = tmap != nullptr && sizeof(TC) == 4;
  if (use) m = *tmap;
  auto launch = [&](auto kern, int tb) -> cudaError_t {
    const size_t smem = tile1 * tb;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<dim3((unsigned)st.max_sub, (unsigned)((ngrid + tb - 1) / tb)), kThreads, smem, s>>>(
        g, ks, M, (const PtRec<TC, DIM>*)st.recs, sa, (const cplx_t<TC>*)grids, ngrid, E, nftot,
        mode, iflag, base, make_int4(dims[0], dims[1], dims[2], dims[3]), go, ntr > 1 ? 1 : 0, m,
        use);
    note_launch();
    return cudaGetLastError();
  };
  if constexpr (sizeof(TC) == 4 && G <= 8) {
    if (TB == 4) return launch(interp_grad_sm_kernel<TC, TD, DIM, G, 4>, 4);
    if (TB == 2) return launch(interp_grad_sm_kernel<TC, TD, DIM, G, 2>, 2);
  }
  return launch(interp_grad_sm_kernel<TC, TD, DIM, G, 1>, 1);
}

}  // namespace

template <typename TC, typename TD>
cudaError_t launch_interp_grad_sm(const Geom& g, const KerSpec<TC>& ks, int64_t M,
                                  const SortState& st, const void* grids, int ntr, int E,
                                  int mode, int iflag, int base, const int* dims,
                                  const GradOut<TD>& go, const CUtensorMap* tmap,
                                  cudaStream_t s) {
  if (M == 0) return cudaSuccess;
  const int G = g.w > 8 ? 16 : g.w > 6 ? 8 : 6;
#define GBN_GDISPATCH(DIM, TM)                                                                 \
  return G == 16 ? run_interp_grad_sm<TC, TD, DIM, 16>(g, ks, M, st, grids, ntr, E, mode,     \
                                                       iflag, base, dims, go, TM, s)          \
         : G == 8 ? run_interp_grad_sm<TC, TD, DIM, 8>(g, ks, M, st, grids, ntr, E, mode,     \
                                                       iflag, base, dims, go, TM, s)          \
                  : run_interp_grad_sm<TC, TD, DIM, 6>(g, ks, M, st, grids, ntr, E, mode,     \
                                                       iflag, base, dims, go, TM, s);
  switch (g.dim) {
    case 1:
      GBN_GDISPATCH(1, nullptr)
    case 2:
      GBN_GDISPATCH(2, tmap)
    default:
      GBN_GDISPATCH(3, tmap)
  }
#undef GBN_GDISPATCH
}

#define GBN_INST_IGS(TC, TD)                                                                   \
  template cudaError_t launch_interp_grad_sm<TC, TD>(                                          \
      const Geom&, const KerSpec<TC>&, int64_t, const SortState&, const void*, int, int, int,  \
      int, int, const int*, const GradOut<TD>&, const CUtensorMap*, cudaStream_t);
GBN_INST_IGS(float, float)
GBN_INST_IGS(float, double)
GBN_INST_IGS(double, double)

namespace {
// Per device: two words of mapped pinned host memory, [0] bounded waits that
// gave up, [1] type-3 points outside declared extents; host and device views.
struct WaitFlag {
  std::once_flag once;
  cudaError_t err = cudaSuccess;
  volatile unsigned* host = nullptr;
  unsigned* dev = nullptr;
};
constexpr int kMaxDevices = 64;
WaitFlag g_flags[kMaxDevices];

WaitFlag* flag_of_current(int* dev_out = nullptr) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
  if (dev_out) *dev_out = dev;
  return &g_flags[dev];
}
}  // namespace

cudaError_t wait_flag_setup() {
  WaitFlag* f = flag_of_current();
  if (!f) return cudaErrorInvalidDevice;
  std::call_once(f->once, [f]() {
    void* h = nullptr;
    f->err = cudaHostAlloc(&h, 2 * sizeof(unsigned), cudaHostAllocMapped | cudaHostAllocPortable);
    if (f->err != cudaSuccess) return;
    ((volatile unsigned*)h)[0] = 0u;
    ((volatile unsigned*)h)[1] = 0u;
    void* d = nullptr;
    f->err = cudaHostGetDevicePointer(&d, h, 0);
    if (f->err == cudaSuccess) f->err = cudaMemcpyToSymbol(g_wait_host, &d, sizeof(d));
    if (f->err != cudaSuccess) {
      cudaFreeHost(h);
      return;
    }
    f->host = (volatile unsigned*)h;
    f->dev = (unsigned*)d;
  });
  return f->err;
}

bool wait_flag_take() {
  WaitFlag* f = flag_of_current();
  if (!f || !f->host || *f->host == 0u) return false;
  *f->host = 0u;
  return true;
}

void wait_flag_raise() {
  WaitFlag* f = flag_of_current();
  if (f && f->host) *f->host += 1u;
}

unsigned* extent_flag_device() {
  WaitFlag* f = flag_of_current();
  return f && f->dev ? f->dev + 1 : nullptr;
}

bool extent_flag_take() {
  WaitFlag* f = flag_of_current();
  if (!f || !f->host || f->host[1] == 0u) return false;
  f->host[1] = 0u;
  return true;
}

cudaError_t read_wait_timeouts(unsigned* out, bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, g_wait_timeouts, sizeof(unsigned));
  if (e == cudaSuccess && reset) {
    const unsigned zero = 0;
    e = cudaMemcpyToSymbol(g_wait_timeouts, &zero, sizeof(unsigned));
  }
  return e;
}

template <typename TC, typename TD>
cudaError_t launch_interp_queue(int dim, int group, const BatchProb<TC>* probs, int K,
                                const int64_t* item_start, int* counter, int T,
                                const void* arena, void* c, size_t smem, cudaStream_t s) {
  if (K == 0) return cudaSuccess;
#define GBN_QDISPATCH(DIM)                                                                     \
  return group == 16 ? run_interp_queue<TC, TD, DIM, 16>(probs, K, item_start, counter, T,     \
                                                         arena, c, smem, s)                    \
         : group == 8 ? run_interp_queue<TC, TD, DIM, 8>(probs, K, item_start, counter, T,     \
                                                         arena, c, smem, s)                    \
                      : run_interp_queue<TC, TD, DIM, 6>(probs, K, item_start, counter, T,     \
                                                         arena, c, smem, s);
  switch (dim) {
    case 1:
      GBN_QDISPATCH(1)
    case 2:
      GBN_QDISPATCH(2)
    default:
      GBN_QDISPATCH(3)
  }
#undef GBN_QDISPATCH
}

#define GBN_INST_IQ(TC, TD)                                                                  \
  template cudaError_t launch_interp_queue<TC, TD>(int, int, const BatchProb<TC>*, int,     \
                                                   const int64_t*, int*, int, const void*,   \
                                                   void*, size_t, cudaStream_t);
GBN_INST_IQ(float, float)
GBN_INST_IQ(float, double)
GBN_INST_IQ(double, double)

}  // namespace gbn
