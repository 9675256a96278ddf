// gbn_spread.cu -- type-1 spreading (nonuniform strengths -> fine grid).
//
// Replaces cuFINUFFT's spread stage (methods 1 "GM-sort" and 2 "SM" that
// options.py:66-79 exposes as gpu_method).  Work unit: one subproblem = up to
// maxsub bin-sorted points of one bin.  Inside a block, G consecutive lanes
// share a point: lane gl evaluates kernel piece gl in every axis (Horner),
// the y/z values are broadcast with warp shuffles, and lane gl applies the
// x offset gl of every (y, z) row.
//
//   method 2 (SM): the block accumulates into a shared-memory tile of the
//     bin (bs+w-1 cells per axis, x widened to an even start and extent),
//     real and imaginary parts interleaved, then adds the tile to the fine
//     grid: a tile that does not wrap around the grid goes back with one
//     bulk tensor reduce-add (TMA, FP32), any other with one vector atomic
//     (float2) per non-zero cell.
//     In FP32 the tile holds 32-bit fixed-point integers: the block scales
//     its points' strengths by s = 2^30 / sum_j max(|Re c_j|, |Im c_j|), so
//     no cell sum can exceed 2^30 in magnitude, rounds every contribution to
//     an integer and adds it with an integer shared-memory atomic (about 3x
//     the throughput of a float shared-memory atomic on sm_103).  The integer
//     sums are exact; the only rounding is the per-contribution 0.5/s =
//     sum|c|/2^31, the size of an FP32 rounding of the contribution itself.
//     FP64 keeps double atomics.
//   method 1 (GM): every update is a global atomic; used when the tile would
//     not fit or when points are not sorted.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "gbn_common.cuh"
#include "gbn_device.cuh"

namespace gbn {

namespace {

struct SubArgs {
  const int* sub_bin;
  const int* sub_off;
  const int* n_sub;
  const int* bin_start;
  const int* bin_count;
  const int* perm;  // null: identity (unsorted points)
  int sorted;
};

// Subproblem -> (first sorted position, point count, bin); false if empty.
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

// Shared-memory accumulators: float/double planes, or int32 fixed point.
template <typename TC>
struct Acc {
  using type = TC;
};
template <>
struct Acc<float> {
  using type = int;
};

__device__ __forceinline__ void acc_add(int* p, float v) { atomicAdd(p, __float2int_rn(v)); }
__device__ __forceinline__ void acc_add(double* p, double v) { atomicAdd(p, v); }

// One subproblem of ntb <= TB transforms t, t+1, ..., executed by the whole
// block (shared by the per-subproblem kernel and the work-queue kernel of
// batched plans).  Each transform has its own tile; a point's record, kernel
// values and shuffles are computed once and applied to every transform.
// Shared memory: TB tiles of spread_tile_bytes, then (g.stash) TB x maxsub
// strengths.  tmap (or null): TMA map of the grids; t_map = transform t's
// index in it.
template <typename TC, typename TD, int DIM, int G, int TB = 1>
__device__ __forceinline__ void spread_sm_block(const Geom& g, const KerSpec<TC>& ks, int64_t M,
                                                const PtRec<TC, DIM>* __restrict__ recs,
                                                const SubArgs& sa, int sub, int t, int ntb,
                                                const cplx_t<TD>* __restrict__ c,
                                                cplx_t<TC>* __restrict__ fine, int64_t nftot,
                                                unsigned char* smem_raw,
                                                const CUtensorMap* tmap = nullptr,
                                                int t_map = 0) {
  using A = typename Acc<TC>::type;
  constexpr bool kFixed = sizeof(A) == 4 && sizeof(TC) == 4;
  constexpr int NCO = GroupCfg<G>::NCO;
  constexpr int PPW = 32 / G;
  constexpr int NWARP = kThreads / 32;
  __shared__ TC s_red[TB][NWARP];
  int start, cnt, bin;
  if (!sub_range(sa, g, M, sub, start, cnt, bin)) return;
  const int w = g.w;
  const Tile<DIM> tl(g, bin);
  const size_t tile_b = spread_tile_bytes(DIM, g.bs, w, sizeof(TC) == 4);
  const int tile_w = (int)(tile_b / sizeof(A));  // accumulator words per tile
  A* sacc = reinterpret_cast<A*>(smem_raw);  // tile k at sacc + k*tile_w; cell i: [2i] re, [2i+1] im
  for (int i = threadIdx.x; i < tile_w * ntb; i += kThreads) sacc[i] = A(0);
  const int lane = threadIdx.x & 31, grp = lane / G, gl = lane % G, warp = threadIdx.x >> 5;

  // one pass over the subproblem's strengths: stage them in shared memory
  // (g.stash) and, in FP32, take each transform's fixed-point scale from them
  cplx_t<TC>* cst = reinterpret_cast<cplx_t<TC>*>(smem_raw + TB * tile_b);
  const bool stash = g.stash != 0;
  TC scale[TB], inv[TB];
#pragma unroll
  for (int k = 0; k < TB; ++k) {
    scale[k] = TC(1);
    inv[k] = TC(1);
    if (k >= ntb) continue;
    const cplx_t<TD>* ct = c + (int64_t)(t + k) * M;
    TC part = TC(0);
    if (kFixed || stash) {
      for (int p = threadIdx.x; p < cnt; p += kThreads) {
        const int js = start + p;
        TC re, im;
        load_c<TD, TC>(ct + (sa.perm ? sa.perm[js] : js), re, im);
        if (stash) {
          cplx_t<TC> v;
          v.x = re;
          v.y = im;
          cst[k * g.maxsub + p] = v;
        }
        part += fmax(fabs(re), fabs(im));
      }
    }
    if (kFixed) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
      if (lane == 0) s_red[k][warp] = part;
    }
  }
  if (kFixed) {
    __syncthreads();
#pragma unroll
    for (int k = 0; k < TB; ++k) {
      if (k >= ntb) continue;
      TC B = TC(0);
#pragma unroll
      for (int i = 0; i < NWARP; ++i) B += s_red[k][i];
      // B == 0 (or denormal): nothing to spread; the tile stays zero
      scale[k] = B > TC(1e-30) ? TC(1073741824.0) / B : TC(0);
      inv[k] = B > TC(1e-30) ? B / TC(1073741824.0) : TC(0);
    }
  }
  TC co[NCO];
  load_coef<TC, NCO>(co, ks, gl, w);
  __syncthreads();  // tiles cleared, strengths staged

  const bool lane_on = gl < w;
  constexpr int kStep = NWARP * PPW;
  // each group's next point record is loaded one iteration ahead
  PtRec<TC, DIM> rn;
  if (warp * PPW < cnt) {
    const int pn = warp * PPW + grp;
    rn = recs[start + (pn < cnt ? pn : 0)];
  }
  for (int pb = warp * PPW; pb < cnt; pb += kStep) {
    const int pi = pb + grp;
    const bool valid = pi < cnt && grp < PPW;
    const int js = start + (valid ? pi : 0);
    const PtRec<TC, DIM> r = rn;
    if (pb + kStep < cnt) {
      const int pn = pb + kStep + grp;
      rn = recs[start + (pn < cnt ? pn : 0)];
    }
    const TC kx = kerval<TC, NCO>(co, ks, r.d[0], gl, w);
    const int l0 = r.i[0] - tl.org[0] + gl;
    const bool on = valid && lane_on;
    // the group's y (and z) kernel values, fetched once per point
    TC ky = TC(0), kz = TC(0);
    TC kyr[G];
    if (DIM > 1) {
      ky = kerval<TC, NCO>(co, ks, r.d[1], gl, w);
#pragma unroll
      for (int i = 0; i < G; ++i) kyr[i] = __shfl_sync(0xffffffffu, ky, grp * G + i);
    }
    if (DIM > 2) kz = kerval<TC, NCO>(co, ks, r.d[2], gl, w);
    const int pitch = 2 * tl.T[0];
    const int plane = pitch * tl.T[1];
    const int cell0 = DIM == 1 ? 2 * l0
                      : DIM == 2
                          ? pitch * (r.i[1] - tl.org[1]) + 2 * l0
                          : plane * (r.i[2] - tl.org[2]) + pitch * (r.i[1] - tl.org[1]) + 2 * l0;
#pragma unroll
    for (int k = 0; k < TB; ++k) {
      if (k >= ntb) break;
      TC cr = TC(0), ci = TC(0);
      if (valid) {
        if (stash) {
          const cplx_t<TC> v = cst[k * g.maxsub + pi];
          cr = v.x;
          ci = v.y;
        } else {
          load_c<TD, TC>(c + (int64_t)(t + k) * M + (sa.perm ? sa.perm[js] : js), cr, ci);
        }
      }
      const TC kxs = kx * scale[k];
      const TC vr = cr * kxs, vi = ci * kxs;
      A* acc = sacc + k * tile_w + cell0;
      if (DIM == 1) {
        if (on) {
          acc_add(&acc[0], vr);
          acc_add(&acc[1], vi);
        }
      } else if (DIM == 2) {
#pragma unroll
        for (int iy = 0; iy < G; ++iy) {
          if (iy < w && on) {
            acc_add(&acc[iy * pitch], vr * kyr[iy]);
            acc_add(&acc[iy * pitch + 1], vi * kyr[iy]);
          }
        }
      } else {
        for (int iz = 0; iz < w; ++iz) {
          const TC kzv = __shfl_sync(0xffffffffu, kz, grp * G + iz);
          const TC zr = vr * kzv, zi = vi * kzv;
#pragma unroll
          for (int iy = 0; iy < G; ++iy) {
            if (iy < w && on) {
              acc_add(&acc[iy * pitch], zr * kyr[iy]);
              acc_add(&acc[iy * pitch + 1], zi * kyr[iy]);
            }
          }
          acc += plane;
        }
      }
    }
  }
  __syncthreads();

  const int nf0 = (int)g.nf[0], nf1 = (int)g.nf[1], nf2 = (int)g.nf[2];
  if constexpr (kFixed && DIM > 1) {
    // every tile must start on a 128-byte boundary of shared memory
    if (tmap != nullptr && tl.interior(g) && (smem_addr(sacc) & 127u) == 0 &&
        (tile_b & 127u) == 0) {
      // fixed point -> float in place, then one bulk reduce-add per tile
      for (int k = 0; k < ntb; ++k) {
        A* tk = sacc + k * tile_w;
        for (int i = threadIdx.x; i < 2 * tl.ncell; i += kThreads)
          tk[i] = __float_as_int((TC)tk[i] * inv[k]);
      }
      fence_async_smem();
      __syncthreads();
      if (threadIdx.x == 0) {
        for (int k = 0; k < ntb; ++k) {
          const A* tk = sacc + k * tile_w;
          if (DIM == 2)
            tma_reduce_add_2d(tmap, tk, 2 * tl.org[0], tl.org[1] + (t_map + k) * nf1);
          else
            tma_reduce_add_3d(tmap, tk, 2 * tl.org[0], tl.org[1], tl.org[2] + (t_map + k) * nf2);
        }
        bulk_commit();
        bulk_wait_read();  // the tiles stay allocated until the copies have read them
      }
      return;
    }
  }
  for (int k = 0; k < ntb; ++k) {
    const A* tk = sacc + k * tile_w;
    cplx_t<TC>* ft = fine + (int64_t)(t + k) * nftot;
    CellWalk cw(threadIdx.x, kThreads, tl.T[0], tl.T[1]);
    for (int i = threadIdx.x; i < tl.ncell; i += kThreads, cw.next()) {
      const A ar = tk[2 * i], ai = tk[2 * i + 1];
      if (ar == A(0) && ai == A(0)) continue;
      const int g0 = wrap_i32(tl.org[0] + cw.c0, nf0);
      const int g1 = DIM > 1 ? wrap_i32(tl.org[1] + cw.c1, nf1) : 0;
      const int g2 = DIM > 2 ? wrap_i32(tl.org[2] + cw.c2, nf2) : 0;
      atomic_add_c(&ft[(g2 * nf1 + g1) * nf0 + g0], (TC)ar * inv[k], (TC)ai * inv[k]);
    }
  }
}

// grid (subproblems, ceil(ntr / TB)); block y handles transforms TB*y ...
template <typename TC, typename TD, int DIM, int G, int TB>
__global__ void __launch_bounds__(kThreads)
    spread_sm_kernel(Geom g, KerSpec<TC> ks, int64_t M, const PtRec<TC, DIM>* __restrict__ recs,
                     SubArgs sa, const cplx_t<TD>* __restrict__ c, cplx_t<TC>* __restrict__ fine,
                     int64_t nftot, int ntr, const __grid_constant__ CUtensorMap tmap,
                     int use_tma, int t_base) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int t = TB * (int)blockIdx.y;
  const int ntb = min(TB, ntr - t);
  spread_sm_block<TC, TD, DIM, G, TB>(g, ks, M, recs, sa, blockIdx.x, t, ntb, c, fine, nftot,
                                      smem_raw, use_tma ? &tmap : nullptr, t_base + t);
}

template <typename TC, typename TD, int DIM, int G>
__global__ void __launch_bounds__(kThreads)
    spread_gm_kernel(Geom g, KerSpec<TC> ks, int64_t M, const PtRec<TC, DIM>* __restrict__ recs,
                     SubArgs sa, const cplx_t<TD>* __restrict__ c, cplx_t<TC>* __restrict__ fine,
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
  const cplx_t<TD>* ct = c + (int64_t)t * M;
  cplx_t<TC>* ft = fine + (int64_t)t * nftot;
  const bool lane_on = gl < w;
  const int nf0 = (int)g.nf[0], nf1 = (int)g.nf[1], nf2 = (int)g.nf[2];
  for (int pb = warp * PPW; pb < cnt; pb += NWARP * PPW) {
    const int pi = pb + grp;
    const bool valid = pi < cnt && grp < PPW;
    const int js = start + (valid ? pi : 0);
    const PtRec<TC, DIM> r = recs[js];
    TC cr = TC(0), ci = TC(0);
    if (valid) load_c<TD, TC>(ct + (sa.perm ? sa.perm[js] : js), cr, ci);
    const TC kx = kerval<TC, NCO>(co, ks, r.d[0], gl, w);
    const int gx = wrap_i32(r.i[0] + gl, nf0);
    const bool on = valid && lane_on;
    const TC vr = cr * kx, vi = ci * kx;
    if (DIM == 1) {
      if (on) atomic_add_c(&ft[gx], vr, vi);
    } else if (DIM == 2) {
      const TC ky = kerval<TC, NCO>(co, ks, r.d[1], gl, w);
      for (int iy = 0; iy < w; ++iy) {
        const TC kyv = __shfl_sync(0xffffffffu, ky, grp * G + iy);
        const int gy = wrap_i32(r.i[1] + iy, nf1);
        if (on) atomic_add_c(&ft[gy * nf0 + gx], vr * kyv, vi * kyv);
      }
    } else {
      const TC ky = kerval<TC, NCO>(co, ks, r.d[1], gl, w);
      const TC kz = kerval<TC, NCO>(co, ks, r.d[2], gl, w);
      for (int iz = 0; iz < w; ++iz) {
        const TC kzv = __shfl_sync(0xffffffffu, kz, grp * G + iz);
        const int gz = wrap_i32(r.i[2] + iz, nf2);
        const TC zr = vr * kzv, zi = vi * kzv;
        for (int iy = 0; iy < w; ++iy) {
          const TC kyv = __shfl_sync(0xffffffffu, ky, grp * G + iy);
          const int gy = wrap_i32(r.i[1] + iy, nf1);
          if (on) atomic_add_c(&ft[(gz * nf1 + gy) * nf0 + gx], zr * kyv, zi * kyv);
        }
      }
    }
  }
}


template <typename TC, typename TD, int DIM, int G, int TB>
__global__ void __launch_bounds__(kThreads)
    spread_queue_kernel(const BatchProb<TC>* __restrict__ probs, int K,
                        const int64_t* __restrict__ item_start, int* counter, int T,
                        const cplx_t<TD>* __restrict__ c, cplx_t<TC>* __restrict__ arena) {
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
    const int Tg = (T + TB - 1) / TB;  // items per subproblem
    const int sub = (int)(local / Tg), tg = (int)(local - (int64_t)sub * Tg);
    const int t = tg * TB;
    SubArgs sa{P.sub_bin, P.sub_off, P.n_sub, P.bin_start, P.bin_count, P.perm, 1};
    spread_sm_block<TC, TD, DIM, G, TB>(P.g, P.ks, P.M, (const PtRec<TC, DIM>*)P.recs, sa, sub,
                                        t, min(TB, T - t), c + P.c_off, arena + P.grid_off,
                                        P.nftot, smem_raw);
  }
}

template <typename TC, typename TD, int DIM, int G, int TB>
cudaError_t run_spread_queue(const BatchProb<TC>* probs, int K, const int64_t* item_start,
                             int* counter, int T, const void* c, void* arena, size_t smem,
                             cudaStream_t s) {
  auto kern = spread_queue_kernel<TC, TD, DIM, G, TB>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
  if (per_sm < 1) per_sm = 1;
  kern<<<nsm * per_sm, kThreads, smem, s>>>(probs, K, item_start, counter, T,
                                            (const cplx_t<TD>*)c, (cplx_t<TC>*)arena);
  note_launch();
  return cudaGetLastError();
}

template <typename TC, typename TD, int DIM, int G>
cudaError_t run_spread(const Geom& g, const KerSpec<TC>& ks, int method, int64_t M,
                       const SortState& st, const void* c, void* fine, int ntr,
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
  // transforms per block: several stacked transforms share each point's
  // record, kernel values and shuffles (FP32 with staged strengths, while
  // the block's shared memory stays within 100 KB)
  const bool sm = method == 2 && sa.sorted;
  const size_t smem1 = spread_smem_bytes(DIM, g.bs, g.w, sizeof(TC) == 4, g.maxsub, g.stash != 0);
  int TB = 1;
  if (sm && sizeof(TC) == 4 && G <= 8 && g.stash) {
    if (ntr >= 4 && 4 * smem1 <= 100 * 1024)
      TB = 4;
    else if (ntr >= 2 && 2 * smem1 <= 100 * 1024)
      TB = 2;
  }
  for (int t0 = 0; t0 < ntr; t0 += 65535 * TB) {
    const int nt = std::min(ntr - t0, 65535 * TB);
    dim3 grid((unsigned)nblk, (unsigned)((nt + TB - 1) / TB));
    const cplx_t<TD>* ct = (const cplx_t<TD>*)c + (int64_t)t0 * M;
    cplx_t<TC>* ft = (cplx_t<TC>*)fine + (int64_t)t0 * nftot;
    if (sm) {
      CUtensorMap m;
      memset(&m, 0, sizeof(m));
      const int use = tmap != nullptr && sizeof(TC) == 4;
      if (use) m = *tmap;
      auto go = [&](auto kern, int tb) -> cudaError_t {
        const size_t smem = smem1 * tb;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        kern<<<grid, kThreads, smem, s>>>(g, ks, M, recs, sa, ct, ft, nftot, nt, m, use, t0);
        note_launch();
        return cudaSuccess;
      };
      cudaError_t e;
      if constexpr (sizeof(TC) == 4 && G <= 8) {
        e = TB == 4   ? go(spread_sm_kernel<TC, TD, DIM, G, 4>, 4)
            : TB == 2 ? go(spread_sm_kernel<TC, TD, DIM, G, 2>, 2)
                      : go(spread_sm_kernel<TC, TD, DIM, G, 1>, 1);
      } else {
        e = go(spread_sm_kernel<TC, TD, DIM, G, 1>, 1);
      }
      if (e != cudaSuccess) return e;
    } else {
      spread_gm_kernel<TC, TD, DIM, G><<<grid, kThreads, 0, s>>>(g, ks, M, recs, sa, ct, ft,
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
cudaError_t launch_spread(const Geom& g, const KerSpec<TC>& ks, int method, int64_t M,
                          const SortState& st, const void* c, void* fine, int ntr,
                          cudaStream_t s, const CUtensorMap* tmap) {
  if (M == 0) return cudaSuccess;
  // lanes per point: the narrowest group that covers the kernel width
  const int G = g.w > 8 ? 16 : g.w > 6 ? 8 : 6;
#define GBN_DISPATCH(DIM, TM)                                        \
  return G == 16 ? run_spread<TC, TD, DIM, 16>(g, ks, method, M, st, c, fine, ntr, s, TM)      \
         : G == 8 ? run_spread<TC, TD, DIM, 8>(g, ks, method, M, st, c, fine, ntr, s, TM)      \
                  : run_spread<TC, TD, DIM, 6>(g, ks, method, M, st, c, fine, ntr, s, TM);
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

template cudaError_t launch_spread<float, float>(const Geom&, const KerSpec<float>&, int,
                                                 int64_t, const SortState&, const void*, void*,
                                                 int, cudaStream_t, const CUtensorMap*);
template cudaError_t launch_spread<float, double>(const Geom&, const KerSpec<float>&, int,
                                                  int64_t, const SortState&, const void*, void*,
                                                  int, cudaStream_t, const CUtensorMap*);
template cudaError_t launch_spread<double, double>(const Geom&, const KerSpec<double>&, int,
                                                   int64_t, const SortState&, const void*,
                                                   void*, int, cudaStream_t, const CUtensorMap*);


template <typename TC, typename TD, int DIM>
cudaError_t spread_queue_dim(int group, int tb, const BatchProb<TC>* probs, int K,
                             const int64_t* item_start, int* counter, int T, const void* c,
                             void* arena, size_t smem1, cudaStream_t s) {
  if (group == 16)
    return run_spread_queue<TC, TD, DIM, 16, 1>(probs, K, item_start, counter, T, c, arena,
                                                smem1, s);
  if constexpr (sizeof(TC) == 4) {
    if (tb == 4)
      return group == 8 ? run_spread_queue<TC, TD, DIM, 8, 4>(probs, K, item_start, counter, T,
                                                              c, arena, 4 * smem1, s)
                        : run_spread_queue<TC, TD, DIM, 6, 4>(probs, K, item_start, counter, T,
                                                              c, arena, 4 * smem1, s);
    if (tb == 2)
      return group == 8 ? run_spread_queue<TC, TD, DIM, 8, 2>(probs, K, item_start, counter, T,
                                                              c, arena, 2 * smem1, s)
                        : run_spread_queue<TC, TD, DIM, 6, 2>(probs, K, item_start, counter, T,
                                                              c, arena, 2 * smem1, s);
  }
  return group == 8 ? run_spread_queue<TC, TD, DIM, 8, 1>(probs, K, item_start, counter, T, c,
                                                          arena, smem1, s)
                    : run_spread_queue<TC, TD, DIM, 6, 1>(probs, K, item_start, counter, T, c,
                                                          arena, smem1, s);
}

template <typename TC, typename TD>
cudaError_t launch_spread_queue(int dim, int group, int tb, const BatchProb<TC>* probs, int K,
                                const int64_t* item_start, int* counter, int T, const void* c,
                                void* arena, size_t smem1, cudaStream_t s) {
  if (K == 0) return cudaSuccess;
  switch (dim) {
    case 1:
      return spread_queue_dim<TC, TD, 1>(group, tb, probs, K, item_start, counter, T, c, arena,
                                         smem1, s);
    case 2:
      return spread_queue_dim<TC, TD, 2>(group, tb, probs, K, item_start, counter, T, c, arena,
                                         smem1, s);
    default:
      return spread_queue_dim<TC, TD, 3>(group, tb, probs, K, item_start, counter, T, c, arena,
                                         smem1, s);
  }
}

#define GBN_INST_SQ(TC, TD)                                                                   \
  template cudaError_t launch_spread_queue<TC, TD>(int, int, int, const BatchProb<TC>*, int,  \
                                                   const int64_t*, int*, int, const void*,    \
                                                   void*, size_t, cudaStream_t);
GBN_INST_SQ(float, float)
GBN_INST_SQ(float, double)
GBN_INST_SQ(double, double)


}  // namespace gbn
