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
//
// 3D FP32 plans with bins 16 x 16 x bz and widths 4..8 take the row-owned
// kernel below (spread_rows_kernel) instead of the G-lane one: the same
// tile, but one point per warp on lanes laid out so that every atomic
// instruction reaches distinct banks, contributions rounded by one FFMA
// where the tolerance allows, and the scale bounded to 0.999 * 2^31 / sum.
// 2D FP32 plans of four or more stacked transforms with bins 16 x 16 or
// 32 x 32 and widths 4..8 take its 2D counterpart (spread_rows2_kernel: four
// transforms per block, two points per warp step, integer-product
// contributions below 1e-5).  Batched plans (the work queue) keep the G-lane
// block.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <utility>

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

// ---------------------------------------------------------------------------
// Row-owned spread: 3D, FP32 compute, bin-sorted points, Horner kernel
// values, kernel widths 4..8, bins 16 x 16 x bz.
//
// Same fixed-point tile as spread_sm_block (int32 re/im pairs, cell (x, y, z)
// at x + PY y + PZ z with PY = tile_x(16, w) = 16 + WV, WV = w rounded up to
// even, PZ = PY (15 + w)), but a warp adds ONE point at a time: lane = (part,
// r, gl) with part = lane / 16 selecting the real or imaginary word, r < R =
// 16 / WV a row of the point's support and gl < WV an x offset.  One atomic
// instruction covers R rows of one z-plane; a point takes ceil(w / R) row
// chunks times w planes of them.  The lane's word is 2 (gl + PY r) + part
// past the point's base, and PY = 16 + WV is congruent to WV modulo 16, so
// gl + PY r is distinct modulo 16 over the active lanes and every instruction
// reaches 32 distinct banks (points spread G lanes at a time collide on most
// of their shared-memory wavefronts).
// Contributions become integers with one FFMA each where the precision
// allows: for |v| < 2^22, fma(a, kz, 1.5 * 2^23) carries round(a kz) in its
// low bits, offset by the bit pattern of 1.5 * 2^23 (the FP32-to-int32
// conversion instruction runs at a quarter of the FMA rate and bounded the
// G-lane kernel).  The block's scale s = 0.999 * 2^31 / sum_j max|c_j| keeps
// every final cell sum inside int32 (partial sums may wrap: two's-complement
// addition is exact modulo 2^32); FFMA rounding also caps it at 0.999 * 2^22
// / max_j max|c_j|.
// Kernel values: the 3w pieces of a point are evaluated once (one Horner
// evaluation per lane) into a per-warp table, from which every lane reads its
// x value, the w z values and the y values of its rows.
// ---------------------------------------------------------------------------
// threads per row-owned spread block (three blocks per SM; 512-thread
// blocks, two per SM, measured slower: 2.07 -> 2.34 ms on the headline)
constexpr int kRowThreads = 256;

constexpr float kRoundMagic = 12582912.0f;   // 1.5 * 2^23
constexpr int kRoundMagicBits = 0x4B400000;  // its bit pattern

// One contribution, rounded as the block's scale requires, added at
// shared-memory byte address a + OFF (OFF a compile-time immediate).
template <int OFF, bool MAGIC>
__device__ __forceinline__ void red_at(uint32_t a, float av, float kz) {
  const int v = MAGIC ? __float_as_int(fmaf(av, kz, kRoundMagic)) - kRoundMagicBits
                      : __float2int_rn(av * kz);
  asm volatile("red.shared.add.s32 [%0+%2], %1;" ::"r"(a), "r"(v), "n"(OFF) : "memory");
}

template <int W, bool MAGIC, int... K>
__device__ __forceinline__ void rows_add_all(uint32_t a, const float (&av)[RowCfg<W>::NCH],
                                             const float (&kz)[8],
                                             std::integer_sequence<int, K...>) {
  using C = RowCfg<W>;
  // instruction k: row chunk k / W, plane k % W
  (red_at<8 * ((K / W) * C::R * C::PY + (K % W) * C::PZ), MAGIC>(a, av[K / W], kz[K % W]), ...);
}

// One point's contributions: R rows per atomic instruction, NCH row chunks
// times W planes, to the point's cells from shared-memory byte address a (the
// lane's word of the point's first cell).  Every lane adds on every
// instruction; a lane without a cell of the point in this chunk (row >= W, x
// offset >= W, or a lane past the R rows) adds an exact zero: its y or x
// kernel value comes from a table slot that holds zero (the table's slots
// past w are never written).  Its cell is the one its lane position names:
// within the tile's rows, or at most two rows past the tile's last plane,
// inside the staged strengths that follow the tile in shared memory (an
// atomic add of zero leaves them unchanged), and still on a bank of its own.
// ty: the lane's first row's y value (rows ch R + r at offsets ch R).
template <int W, bool MAGIC>
__device__ __forceinline__ void rows_add(uint32_t a, float a0, const float* ty,
                                         const float (&kz)[8]) {
  using C = RowCfg<W>;
  float av[C::NCH];
#pragma unroll
  for (int ch = 0; ch < C::NCH; ++ch) av[ch] = a0 * ty[ch * C::R];
  rows_add_all<W, MAGIC>(a, av, kz, std::make_integer_sequence<int, C::NCH * W>{});
}

// Lane roles in the per-warp kernel-value table of rows_points: one Horner
// evaluation per lane and point -- lane (part 0, q < w): z piece q; (part 0,
// w <= q < 2w): x piece q - w; (part 1, q < w): y piece q -- into the
// table [z 0..7 | y 8..15 | x 16..23] of the point.
struct RowTab {
  int axis, slot;
  bool writes;
  __device__ __forceinline__ RowTab(int hp, int q, int W) {
    axis = hp ? 1 : (q < W ? 2 : 0);
    writes = hp ? q < W : q < 2 * W;
    slot = hp ? 8 + q : (q < W ? q : 16 + q - W);
  }
};

// Two points of the warp (p and p + NWARP when `two`): their kernel values
// through one table round trip, then their contributions.
template <int W, bool MAGIC>
__device__ __forceinline__ void rows_pair(const PtRec<float, 3>& ra, const PtRec<float, 3>& rb,
                                          bool two, int p, const float2* cst, float scale,
                                          const float (&co)[RowCfg<W>::NCO], uint32_t lbase,
                                          unsigned org_cell, float (*tb)[24], const RowTab& rt,
                                          int hp, int r, int xs) {
  using C = RowCfg<W>;
  constexpr int NWARP = kRowThreads / 32;
  const float2 ca = cst[p], cb = cst[two ? p + NWARP : p];
  const float da = rt.axis == 0 ? ra.d[0] : rt.axis == 1 ? ra.d[1] : ra.d[2];
  const float db = rt.axis == 0 ? rb.d[0] : rt.axis == 1 ? rb.d[1] : rb.d[2];
  const float tva = horner_piece(co, da);
  const float tvb = horner_piece(co, db);
  const uint32_t aa =
      lbase + 8u * ((unsigned)ra.i[0] + C::PY * (unsigned)ra.i[1] + C::PZ * (unsigned)ra.i[2] -
                    org_cell);
  const uint32_t ab =
      lbase + 8u * ((unsigned)rb.i[0] + C::PY * (unsigned)rb.i[1] + C::PZ * (unsigned)rb.i[2] -
                    org_cell);
  if (rt.writes) {
    tb[0][rt.slot] = tva;
    tb[1][rt.slot] = tvb;
  }
  __syncwarp();
  {
    const float4* t4 = reinterpret_cast<const float4*>(tb[0]);
    const float4 z0 = t4[0], z1 = t4[1];
    const float kz[8] = {z0.x, z0.y, z0.z, z0.w, z1.x, z1.y, z1.z, z1.w};
    rows_add<W, MAGIC>(aa, (hp ? ca.y : ca.x) * scale * tb[0][xs], tb[0] + 8 + r, kz);
  }
  if (two) {
    const float4* t4 = reinterpret_cast<const float4*>(tb[1]);
    const float4 z0 = t4[0], z1 = t4[1];
    const float kz[8] = {z0.x, z0.y, z0.z, z0.w, z1.x, z1.y, z1.z, z1.w};
    rows_add<W, MAGIC>(ab, (hp ? cb.y : cb.x) * scale * tb[1][xs], tb[1] + 8 + r, kz);
  }
}

// The point loop of spread_rows_kernel: this warp's points p = warp,
// warp + NWARP, ... of the subproblem, two per step, with the records of the
// next step loaded during the current one into a second register set (the
// loop body is written out twice, alternating the sets, so no record is
// copied).  MAGIC: contributions rounded by the FFMA above (|v| < 2^22
// guaranteed by the scale); otherwise by the FP32 to int32 conversion
// (|v| < 2^31).
template <int W, bool MAGIC>
__device__ __forceinline__ void rows_points(const PtRec<float, 3>* __restrict__ recs, int start,
                                            int cnt, const float2* cst, float scale,
                                            const float (&co)[RowCfg<W>::NCO], uint32_t lbase,
                                            unsigned org_cell, float (*tab)[2][24], int warp,
                                            int hp, int q, int gl, int r) {
  constexpr int NWARP = kRowThreads / 32;
  constexpr int STEP = 2 * NWARP;
  const RowTab rt(hp, q, W);
  // x slot of the lane's value: slot 23 is a zero for w <= 7 (and no lane
  // needs it at w = 8, where 16 lanes are 2 rows of 8 offsets)
  const int xs = (gl < W && r < RowCfg<W>::R) ? 16 + gl : 23;
  // zero the warp's tables once: the slots past w are never written
  {
    float* t = &tab[0][0][0];
    const int lane = threadIdx.x & 31;
    for (int i = lane; i < 2 * 2 * 24; i += 32) t[i] = 0.f;
    __syncwarp();
  }
  const PtRec<float, 3>* rp = recs + start;
  auto jc = [&](int p) { return p < cnt ? p : cnt - 1; };
  int p = warp;
  if (p >= cnt) return;
  PtRec<float, 3> xa = rp[p], xb = rp[jc(p + NWARP)], ya, yb;
  for (;;) {
    if (p + STEP < cnt) {
      ya = rp[p + STEP];
      yb = rp[jc(p + STEP + NWARP)];
    }
    rows_pair<W, MAGIC>(xa, xb, p + NWARP < cnt, p, cst, scale, co, lbase, org_cell, tab[0], rt,
                        hp, r, xs);
    p += STEP;
    if (p >= cnt) break;
    if (p + STEP < cnt) {
      xa = rp[p + STEP];
      xb = rp[jc(p + STEP + NWARP)];
    }
    rows_pair<W, MAGIC>(ya, yb, p + NWARP < cnt, p, cst, scale, co, lbase, org_cell, tab[1], rt,
                        hp, r, xs);
    p += STEP;
    if (p >= cnt) break;
  }
}

template <typename TD, int W>
__global__ void __launch_bounds__(kRowThreads)
    spread_rows_kernel(Geom g, KerSpec<float> ks, int64_t M,
                       const PtRec<float, 3>* __restrict__ recs, SubArgs sa,
                       const cplx_t<TD>* __restrict__ c, cplx_t<float>* __restrict__ fine,
                       int64_t nftot, const __grid_constant__ CUtensorMap tmap, int use_tma,
                       int t_base) {
  using C = RowCfg<W>;
  constexpr int NWARP = kRowThreads / 32;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ float s_sum[NWARP], s_max[NWARP];
  __shared__ __align__(16) float s_tab[NWARP][2][2][24];  // [warp][buffer][point][z | y | x]
  __shared__ int s_org[3];
  int start, cnt, bin;
  if (!sub_range(sa, g, M, blockIdx.x, start, cnt, bin)) return;
  const int t = blockIdx.y;
  // the tile origin (three integer divisions) by one thread, read after the
  // first barrier; the extents are the same for every bin
  if (threadIdx.x == 0) {
    const Tile<3> t0(g, bin);
    s_org[0] = t0.org[0];
    s_org[1] = t0.org[1];
    s_org[2] = t0.org[2];
  }
  const size_t tile_b = spread_tile_bytes(3, g.bs, W, true);
  int* sacc = reinterpret_cast<int*>(smem_raw);
  {
    int4* z4 = reinterpret_cast<int4*>(smem_raw);
    for (int i = threadIdx.x; i < (int)(tile_b / 16); i += kRowThreads) z4[i] = make_int4(0, 0, 0, 0);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // stage the strengths; sum and maximum of max(|Re c|, |Im c|)
  float2* cst = reinterpret_cast<float2*>(smem_raw + tile_b);
  const cplx_t<TD>* ct = c + (int64_t)t * M;
  float psum = 0.f, pmax = 0.f;
  for (int p = threadIdx.x; p < cnt; p += kRowThreads) {
    float re, im;
    load_c<TD, float>(ct + sa.perm[start + p], re, im);
    cst[p] = make_float2(re, im);
    const float m = fmaxf(fabsf(re), fabsf(im));
    psum += m;
    pmax = fmaxf(pmax, m);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    psum += __shfl_xor_sync(0xffffffffu, psum, o);
    pmax = fmaxf(pmax, __shfl_xor_sync(0xffffffffu, pmax, o));
  }
  if (lane == 0) {
    s_sum[warp] = psum;
    s_max[warp] = pmax;
  }
  const int hp = lane >> 4, q = lane & 15, gl = q % C::WV, r = q / C::WV;
  // coefficients of the piece this lane evaluates (see rows_points)
  float co[C::NCO];
  load_coef<float, C::NCO>(co, ks, q < W ? q : q - W, W);
  __syncthreads();  // tile cleared, strengths staged, partial sums written
  float B = 0.f, Mx = 0.f;
#pragma unroll
  for (int i = 0; i < NWARP; ++i) {
    B += s_sum[i];
    Mx = fmaxf(Mx, s_max[i]);
  }
  // Scale: every final cell sum stays below 2^31 in magnitude; with FFMA
  // rounding also every contribution below 2^22.  The FFMA rounding is used
  // where the tolerance allows its resolution (2^-22 of the largest strength)
  // or where it costs nothing (sum >= 512 x largest: the 2^31 bound is the
  // tighter one).  B == 0 (or denormal): nothing to spread, the tile stays zero.
  const bool magic = g.coarse_round != 0 || B >= 512.f * Mx;
  float scale = 0.f;
  if (B > 1e-30f) {
    scale = 0.999f * 2147483648.f / B;
    if (magic) scale = fminf(scale, 0.999f * 4194304.f / Mx);
  }
  const float inv = scale > 0.f ? 1.f / scale : 0.f;
  const uint32_t lbase = smem_addr(sacc) + 4u * (2 * (gl + C::PY * r) + hp);
  const int org[3] = {s_org[0], s_org[1], s_org[2]};
  const int T2 = g.bs[2] + W - 1, ncell = C::PZ * T2;
  // cell index of the tile origin, modulo 2^32 (the cell offsets of the
  // points from it are small; the absolute indices need not fit an int)
  const unsigned org_cell = (unsigned)org[0] + C::PY * (unsigned)org[1] + C::PZ * (unsigned)org[2];
  if (magic)
    rows_points<W, true>(recs, start, cnt, cst, scale, co, lbase, org_cell, s_tab[warp], warp,
                         hp, q, gl, r);
  else
    rows_points<W, false>(recs, start, cnt, cst, scale, co, lbase, org_cell, s_tab[warp], warp,
                          hp, q, gl, r);
  __syncthreads();

  const int nf0 = (int)g.nf[0], nf1 = (int)g.nf[1], nf2 = (int)g.nf[2];
  const bool interior = org[0] >= 0 && org[0] + C::PY <= nf0 && org[1] >= 0 &&
                        org[1] + 15 + W <= nf1 && org[2] >= 0 && org[2] + T2 <= nf2;
  if (use_tma && interior && (smem_addr(sacc) & 127u) == 0 && (tile_b & 127u) == 0) {
    // fixed point -> float in place (four words per access; the padded tile
    // is a whole number of 16-byte words), then one bulk reduce-add
    int4* s4 = reinterpret_cast<int4*>(sacc);
    for (int i = threadIdx.x; i < (2 * ncell + 3) / 4; i += kRowThreads) {
      const int4 v = s4[i];
      s4[i] = make_int4(__float_as_int((float)v.x * inv), __float_as_int((float)v.y * inv),
                        __float_as_int((float)v.z * inv), __float_as_int((float)v.w * inv));
    }
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      tma_reduce_add_3d(&tmap, sacc, 2 * org[0], org[1], org[2] + (t_base + t) * nf2);
      bulk_commit();
      bulk_wait_read();  // the tile stays allocated until the copy has read it
    }
    return;
  }
  cplx_t<float>* ft = fine + (int64_t)t * nftot;
  CellWalk cw(threadIdx.x, kRowThreads, C::PY, 15 + W);
  for (int i = threadIdx.x; i < ncell; i += kRowThreads, cw.next()) {
    const int ar = sacc[2 * i], ai = sacc[2 * i + 1];
    if (ar == 0 && ai == 0) continue;
    const int g0 = wrap_i32(org[0] + cw.c0, nf0);
    const int g1 = wrap_i32(org[1] + cw.c1, nf1);
    const int g2 = wrap_i32(org[2] + cw.c2, nf2);
    atomic_add_c(&ft[(g2 * nf1 + g1) * nf0 + g0], (float)ar * inv, (float)ai * inv);
  }
}

// ---------------------------------------------------------------------------
// Row-owned 2D spread: FP32 compute, sorted points, Horner values, widths
// 4..8, bins BS x BS (BS = 16 or 32), TB stacked transforms per block (one
// tile each, as spread_sm_block stacks them; run_spread launches TB = 4).  The lane layout of the 3D
// kernel (RowCfg: part, row r, x offset gl; tile row pitch T0 = tile_x(BS, w)
// = BS + WV, congruent to WV modulo 16, so every atomic instruction reaches
// 32 distinct banks), one point per warp at a time: per point and transform
// ceil(w / R) atomic instructions, at compile-time offsets from one address.
// Lanes without a cell add an exact zero to the cell their position names:
// in the tile, at most two rows past its end (inside the next tile or the
// staged strengths that follow the tiles; zero adds change nothing).
// Contributions, for all the block's transforms one of:
//   integer products (RND_IMUL): the staged strengths become int32, a =
//     round(c S) with S = 0.999 min(2^31 / max, 2^33 / sum) per transform
//     (max and sum of max(|Re c|, |Im c|) over the subproblem), the kernel
//     products Q30 fractions, kq = round(2^30 ky kx) (the y pieces' Horner
//     coefficients carry the 2^30), and a contribution is the high word of
//     the 64-bit a kq + 2^31, round(c S ky kx / 4), by one multiply-add.
//     Cell sums stay below 2^31 (S sum / 4 < 2^31); the resolution, 4 / S =
//     max(sum / 2^31, max / 2^29) in strength units, is the FP32-to-int32
//     rounding's sum / 2^31 wherever sum >= 4 max;
//   FFMA rounding (RND_FFMA; tolerance >= 1e-5, or every transform's
//     strengths sum to >= 512 x their largest): fma(c S 2^-30, 2^30 ky kx,
//     1.5 2^23) carries round(c S ky kx) in its low bits, with S = 0.999
//     min(2^31 / sum, 2^22 / max) as in spread_rows_kernel.
// ---------------------------------------------------------------------------
template <int OFF>
__device__ __forceinline__ void red_imm(uint32_t a, int v) {
  asm volatile("red.shared.add.s32 [%0+%2], %1;" ::"r"(a), "r"(v), "n"(OFF) : "memory");
}

// round(a kq / 2^32): the high word of the 64-bit a kq + 2^31
__device__ __forceinline__ int mul_round_hi(int a, int kq) {
  int hi;
  asm("{\n\t.reg .s64 t;\n\t.reg .b32 lo;\n\t"
      "mad.wide.s32 t, %1, %2, 2147483648;\n\t"
      "mov.b64 {lo, %0}, t;\n\t}"
      : "=r"(hi)
      : "r"(a), "r"(kq));
  return hi;
}

template <int W, int BS>
struct Rows2Cfg {
  using C = RowCfg<W>;
  static constexpr int T0 = BS + C::WV;  // = tile_x(BS, W)
  static constexpr int T1 = BS + W - 1;
  static constexpr int TILE_B = (T0 * T1 * 8 + 127) & ~127;  // = spread_tile_bytes
  static constexpr int ROW_B = 8 * C::R * T0;                // one row chunk
};

// One point's contributions: transform k, row chunk ch at byte offset
// k TILE_B + ch ROW_B from a.  RND_IMUL: integer strengths ci times Q30
// kernel products kq; RND_FFMA: float strengths cf (times 2^-30) times the
// same products as floats, rounded by one FFMA each.
enum { RND_IMUL = 0, RND_FFMA = 1 };
template <int W, int BS, int TB, int RND, int... I>
__device__ __forceinline__ void rows2_add(uint32_t a, const int (&ci)[TB], const float (&cf)[TB],
                                          const int (&kq)[RowCfg<W>::NCH],
                                          const float (&kf)[RowCfg<W>::NCH],
                                          std::integer_sequence<int, I...>) {
  using C = RowCfg<W>;
  using Q = Rows2Cfg<W, BS>;
  if constexpr (RND == RND_IMUL)
    (red_imm<(I / C::NCH) * Q::TILE_B + (I % C::NCH) * Q::ROW_B>(
         a, mul_round_hi(ci[I / C::NCH], kq[I % C::NCH])),
     ...);
  else
    (red_imm<(I / C::NCH) * Q::TILE_B + (I % C::NCH) * Q::ROW_B>(
         a, __float_as_int(fmaf(cf[I / C::NCH], kf[I % C::NCH], kRoundMagic)) - kRoundMagicBits),
     ...);
}

// One point: kernel values from the warp's table tb ([y 0..7 | x 8..15], y
// in Q30; the slots past w hold zeros), strengths from the staged ones (word
// (2 p + part) TB + k: int32 for RND_IMUL, float for RND_FFMA).  The lane's
// rows are y slots ch R + r (from its own base tb + r, compile-time offsets),
// its x value slot xs: a lane without a cell (x offset >= w, row >= w, or r
// >= R with slot xs a zero) gets zero products without a select.
template <int W, int BS, int TB, int RND>
__device__ __forceinline__ void rows2_point(const PtRec<float, 2>& rc, int p, const float* tb,
                                            const int* cint, uint32_t lbase, int org0, int org1,
                                            int hp, int r, int xs) {
  using C = RowCfg<W>;
  using Q = Rows2Cfg<W, BS>;
  const float* ty = tb + r;
  const float kx = tb[xs];
  int kq[C::NCH];
  float kf[C::NCH];
#pragma unroll
  for (int ch = 0; ch < C::NCH; ++ch) {
    kf[ch] = ty[ch * C::R] * kx;
    kq[ch] = 0;
    if constexpr (RND == RND_IMUL) kq[ch] = __float2int_rn(kf[ch]);
  }
  int ci[TB];
  float cf[TB];
  const int* cp = cint + (2 * p + hp) * TB;
  if constexpr (TB == 4) {
    const int4 v = *reinterpret_cast<const int4*>(cp);
    ci[0] = v.x;
    ci[1] = v.y;
    ci[2] = v.z;
    ci[3] = v.w;
  } else if constexpr (TB == 2) {
    const int2 v = *reinterpret_cast<const int2*>(cp);
    ci[0] = v.x;
    ci[1] = v.y;
  } else {
#pragma unroll
    for (int k = 0; k < TB; ++k) ci[k] = cp[k];
  }
#pragma unroll
  for (int k = 0; k < TB; ++k) cf[k] = __int_as_float(ci[k]);
  const uint32_t a = lbase + 8u * (uint32_t)((rc.i[0] - org0) + Q::T0 * (rc.i[1] - org1));
  rows2_add<W, BS, TB, RND>(a, ci, cf, kq, kf, std::make_integer_sequence<int, TB * C::NCH>{});
}

// The point loop: this warp's points in pairs (p, p + NWARP), p = warp,
// warp + 2 NWARP, ...; the pair's kernel values by one Horner evaluation per
// lane (part 0 lanes for the first point, part 1 lanes for the second; lane q
// < w: y piece q, w <= q < 2w: x piece q - w) into a double-buffered per-warp
// table, the next pair's records loaded during the current pair.
template <int W, int BS, int TB, int NT, int RND>
__device__ __forceinline__ void rows2_points(const PtRec<float, 2>* __restrict__ recs, int start,
                                             int cnt, const int* cint,
                                             const float (&co)[RowCfg<W>::NCO], uint32_t lbase,
                                             int org0, int org1, float (*tab)[2][16], int warp,
                                             int hp, int q, int gl, int r) {
  using C = RowCfg<W>;
  constexpr int NWARP = NT / 32;
  constexpr int STEP = 2 * NWARP;
  const bool tab_w = q < 2 * W;
  const int slot = q < W ? q : 8 + q - W;
  const int axis = q < W ? 1 : 0;
  // x slot of the lane's value: slot 15 is a zero for w <= 7 (and no lane
  // needs it at w = 8, where 16 lanes are 2 rows of 8 offsets)
  const int xs = (gl < W && r < C::R) ? 8 + gl : 15;
  // zero the warp's tables once: the slots past w are never written
  {
    float* t = &tab[0][0][0];
    const int lane = threadIdx.x & 31;
    for (int i = lane; i < 2 * 2 * 16; i += 32) t[i] = 0.f;
    __syncwarp();
  }
  const PtRec<float, 2>* rp = recs + start;
  auto jc = [&](int i) { return i < cnt ? i : cnt - 1; };
  int buf = 0;
  if (warp >= cnt) return;  // (no record of this subproblem to load)
  PtRec<float, 2> na = rp[warp], nb = rp[jc(warp + NWARP)];
  for (int p = warp; p < cnt; p += STEP) {
    const PtRec<float, 2> ra = na, rb = nb;
    if (p + STEP < cnt) {
      na = rp[p + STEP];
      nb = rp[jc(p + STEP + NWARP)];
    }
    const PtRec<float, 2>& mine = hp ? rb : ra;
    const float tv = horner_piece(co, axis ? mine.d[1] : mine.d[0]);
    if (tab_w) tab[buf][hp][slot] = tv;
    __syncwarp();
    rows2_point<W, BS, TB, RND>(ra, p, tab[buf][0], cint, lbase, org0, org1, hp, r, xs);
    if (p + NWARP < cnt)
      rows2_point<W, BS, TB, RND>(rb, p + NWARP, tab[buf][1], cint, lbase, org0, org1, hp, r,
                                  xs);
    buf ^= 1;
  }
}

// Shared memory: TB tiles of TILE_B bytes, then the staged strengths of up to
// maxsub points (2 TB words each).
template <typename TD, int W, int BS, int TB, int NT>
__global__ void __launch_bounds__(NT, 1024 / NT)
    spread_rows2_kernel(Geom g, KerSpec<float> ks, int64_t M,
                        const PtRec<float, 2>* __restrict__ recs, SubArgs sa,
                        const cplx_t<TD>* __restrict__ c, cplx_t<float>* __restrict__ fine,
                        int64_t nftot, int ntr, const __grid_constant__ CUtensorMap tmap,
                        int use_tma, int t_base) {
  using C = RowCfg<W>;
  using Q = Rows2Cfg<W, BS>;
  constexpr int NWARP = NT / 32;
  static_assert(NT % (2 * TB) == 0, "a thread converts words of one transform");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ float s_sum[TB][NWARP], s_max[TB][NWARP];
  __shared__ __align__(16) float s_tab[NWARP][2][2][16];  // [warp][buffer][point][y | x]
  __shared__ int s_org[2];
  int start, cnt, bin;
  if (!sub_range(sa, g, M, blockIdx.x, start, cnt, bin)) return;
  const int t = TB * (int)blockIdx.y;
  const int ntb = min(TB, ntr - t);
  if (threadIdx.x == 0) {
    const Tile<2> t0(g, bin);
    s_org[0] = t0.org[0];
    s_org[1] = t0.org[1];
  }
  int* sacc = reinterpret_cast<int*>(smem_raw);
  {
    int4* z4 = reinterpret_cast<int4*>(smem_raw);
    for (int i = threadIdx.x; i < TB * Q::TILE_B / 16; i += NT) z4[i] = make_int4(0, 0, 0, 0);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // stage the strengths (a point's TB gathers in flight together; zeros for
  // the transforms past ntr) at word (2 p + part) TB + k; per transform the
  // sum and maximum of max(|Re c|, |Im c|)
  float* cs = reinterpret_cast<float*>(smem_raw + TB * Q::TILE_B);
  {
    float psum[TB], pmax[TB];
#pragma unroll
    for (int k = 0; k < TB; ++k) psum[k] = pmax[k] = 0.f;
    const cplx_t<TD>* ct = c + (int64_t)t * M;
    for (int p = threadIdx.x; p < cnt; p += NT) {
      const int64_t j = sa.perm[start + p];
      float re[TB], im[TB];
#pragma unroll
      for (int k = 0; k < TB; ++k) {
        re[k] = im[k] = 0.f;
        if (k < ntb) load_c<TD, float>(ct + k * M + j, re[k], im[k]);
        const float m = fmaxf(fabsf(re[k]), fabsf(im[k]));
        psum[k] += m;
        pmax[k] = fmaxf(pmax[k], m);
      }
      float* w = cs + 2 * p * TB;
      if constexpr (TB == 4) {
        reinterpret_cast<float4*>(w)[0] = make_float4(re[0], re[1], re[2], re[3]);
        reinterpret_cast<float4*>(w)[1] = make_float4(im[0], im[1], im[2], im[3]);
      } else if constexpr (TB == 2) {
        reinterpret_cast<float4*>(w)[0] = make_float4(re[0], re[1], im[0], im[1]);
      } else {
#pragma unroll
        for (int k = 0; k < TB; ++k) {
          w[k] = re[k];
          w[TB + k] = im[k];
        }
      }
    }
#pragma unroll
    for (int k = 0; k < TB; ++k) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        psum[k] += __shfl_xor_sync(0xffffffffu, psum[k], o);
        pmax[k] = fmaxf(pmax[k], __shfl_xor_sync(0xffffffffu, pmax[k], o));
      }
      if (lane == 0) {
        s_sum[k][warp] = psum[k];
        s_max[k][warp] = pmax[k];
      }
    }
  }
  const int hp = lane >> 4, q = lane & 15, gl = q % C::WV, r = q / C::WV;
  float co[C::NCO];
  load_coef<float, C::NCO>(co, ks, q < W ? q : q - W, W);  // y piece q, or x piece q - w
  if (q < W) {
#pragma unroll
    for (int n = 0; n < C::NCO; ++n) co[n] *= 1073741824.f;  // y values in Q30
  }
  __syncthreads();  // tiles cleared, strengths staged, partial sums written
  // Rounding for all the block's transforms: one FFMA per contribution
  // (RND_FFMA) where the tolerance allows its resolution, 2^-22 of the
  // largest strength, or where every transform's strengths sum to >= 512
  // times their largest (then the 2^31 sum bound is the tighter one and the
  // FFMA rounding costs nothing); integer products (RND_IMUL) otherwise.
  // Per transform: S (strength -> tile units; RND_IMUL: -> int32 strength
  // units, four of which make a tile unit) and inv (tile units -> strength);
  // sum == 0 (or denormal): nothing to spread, the tile stays zero.
  float Bk[TB], Mk[TB];
  bool ffma = g.coarse_round != 0, dense = true;
#pragma unroll
  for (int k = 0; k < TB; ++k) {
    Bk[k] = Mk[k] = 0.f;
#pragma unroll
    for (int i = 0; i < NWARP; ++i) {
      Bk[k] += s_sum[k][i];
      Mk[k] = fmaxf(Mk[k], s_max[k][i]);
    }
    if (k < ntb && !(Bk[k] >= 512.f * Mk[k])) dense = false;
  }
  ffma = ffma || dense;
  float inv[TB], sk = 0.f;
#pragma unroll
  for (int k = 0; k < TB; ++k) {
    float S = 0.f;
    if (Bk[k] > 1e-30f)
      S = ffma ? fminf(0.999f * 2147483648.f / Bk[k], 0.999f * 4194304.f / Mk[k])
               : fminf(0.999f * 2147483648.f / Mk[k], 0.999f * 8589934592.f / Bk[k]);
    inv[k] = S > 0.f ? (ffma ? 1.f : 4.f) / S : 0.f;
    // RND_FFMA: the kernel products carry 2^30 (the y coefficients' Q30)
    if ((int)(threadIdx.x % TB) == k) sk = ffma ? S * (1.f / 1073741824.f) : S;
  }
  {
    int* ci = reinterpret_cast<int*>(cs);
    if (ffma)
      for (int i = threadIdx.x; i < 2 * TB * cnt; i += NT) cs[i] *= sk;
    else
      for (int i = threadIdx.x; i < 2 * TB * cnt; i += NT) ci[i] = __float2int_rn(cs[i] * sk);
  }
  const uint32_t lbase = smem_addr(sacc) + 4u * (2 * (gl + Q::T0 * r) + hp);
  const int org0 = s_org[0], org1 = s_org[1];
  __syncthreads();  // scaled strengths written
  if (ffma)
    rows2_points<W, BS, TB, NT, RND_FFMA>(recs, start, cnt, reinterpret_cast<const int*>(cs), co,
                                          lbase, org0, org1, s_tab[warp], warp, hp, q, gl, r);
  else
    rows2_points<W, BS, TB, NT, RND_IMUL>(recs, start, cnt, reinterpret_cast<const int*>(cs), co,
                                          lbase, org0, org1, s_tab[warp], warp, hp, q, gl, r);
  __syncthreads();

  const int nf0 = (int)g.nf[0], nf1 = (int)g.nf[1];
  const bool interior =
      org0 >= 0 && org0 + Q::T0 <= nf0 && org1 >= 0 && org1 + Q::T1 <= nf1;
  constexpr int ncell = Q::T0 * Q::T1;
  constexpr int tile_w = Q::TILE_B / 4;
  if (use_tma && interior && (smem_addr(sacc) & 127u) == 0) {
    // fixed point -> float in place (four words per access), then one bulk
    // reduce-add per tile
    for (int k = 0; k < ntb; ++k) {
      int4* s4 = reinterpret_cast<int4*>(sacc + k * tile_w);
      for (int i = threadIdx.x; i < (2 * ncell + 3) / 4; i += NT) {
        const int4 v = s4[i];
        s4[i] = make_int4(
            __float_as_int((float)v.x * inv[k]), __float_as_int((float)v.y * inv[k]),
            __float_as_int((float)v.z * inv[k]), __float_as_int((float)v.w * inv[k]));
      }
    }
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int k = 0; k < ntb; ++k)
        tma_reduce_add_2d(&tmap, sacc + k * tile_w, 2 * org0, org1 + (t_base + t + k) * nf1);
      bulk_commit();
      bulk_wait_read();  // the tiles stay allocated until the copies have read them
    }
    return;
  }
  for (int k = 0; k < ntb; ++k) {
    const int* tk = sacc + k * tile_w;
    cplx_t<float>* ft = fine + (int64_t)(t + k) * nftot;
    CellWalk cw(threadIdx.x, NT, Q::T0, Q::T1);
    for (int i = threadIdx.x; i < ncell; i += NT, cw.next()) {
      const int ar = tk[2 * i], ai = tk[2 * i + 1];
      if (ar == 0 && ai == 0) continue;
      const int g0 = wrap_i32(org0 + cw.c0, nf0);
      const int g1 = wrap_i32(org1 + cw.c1, nf1);
      atomic_add_c(&ft[g1 * nf0 + g0], (float)ar * inv[k], (float)ai * inv[k]);
    }
  }
}

// Whether spread_rows2_kernel serves this geometry (2D, FP32 compute, sorted,
// Horner values, widths 4..8, bins 16 x 16 or 32 x 32; the caller checks the
// rest).
inline bool rows2_fit(const Geom& g, int deg) {
  if (g.dim != 2 || g.bs[0] != g.bs[1] || (g.bs[0] != 16 && g.bs[0] != 32) || g.w < 4 ||
      g.w > 8)
    return false;
  if (!rows_reach_fits(g)) return false;
  return deg + 1 <= (g.w <= 6 ? 9 : 11);
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
  // the row-owned kernel (one transform per block) where it applies
  // (GBN_DISABLE_ROW_SPREAD=1: the G-lane kernel everywhere)
  static const bool no_rows = std::getenv("GBN_DISABLE_ROW_SPREAD") != nullptr;
  const bool rows = DIM == 3 && sizeof(TC) == 4 && sm && g.stash && ks.meth == 1 && !no_rows &&
                    rows_fit(g, ks.deg);
  // 2D: the row-owned kernel where four transforms share each block (with
  // fewer the G-lane kernel measured faster: one transform of 4e6 points on
  // a 1024^2 grid, 0.26 against 0.32 ms at eps 1e-6)
  const bool rows2_fits = DIM == 2 && sizeof(TC) == 4 && sm && g.stash && ks.meth == 1 &&
                          !no_rows && rows2_fit(g, ks.deg);
  int TB = 1;
  if (sm && !rows && sizeof(TC) == 4 && G <= 8 && g.stash) {
    if (ntr >= 4 && 4 * smem1 <= 100 * 1024)
      TB = 4;
    else if (ntr >= 2 && 2 * smem1 <= 100 * 1024)
      TB = 2;
  }
  const bool rows2 = rows2_fits && TB == 4;
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
      if constexpr (DIM == 3 && sizeof(TC) == 4) {
        if (rows) {
          auto go_rows = [&](auto kern) -> cudaError_t {
            cudaError_t er = cudaFuncSetAttribute(
                kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
            if (er != cudaSuccess) return er;
            kern<<<grid, kRowThreads, smem1, s>>>(g, ks, M, (const PtRec<float, 3>*)recs, sa, ct,
                                               (cplx_t<float>*)ft, nftot, m, use, t0);
            note_launch();
            return cudaSuccess;
          };
          switch (g.w) {
            case 4:
              e = go_rows(spread_rows_kernel<TD, 4>);
              break;
            case 5:
              e = go_rows(spread_rows_kernel<TD, 5>);
              break;
            case 6:
              e = go_rows(spread_rows_kernel<TD, 6>);
              break;
            case 7:
              e = go_rows(spread_rows_kernel<TD, 7>);
              break;
            default:
              e = go_rows(spread_rows_kernel<TD, 8>);
              break;
          }
          if (e != cudaSuccess) return e;
          e = cudaGetLastError();
          if (e != cudaSuccess) return e;
          continue;
        }
      }
      if constexpr (DIM == 2 && sizeof(TC) == 4) {
        if (rows2) {
          auto go_rows2 = [&](auto kern, int tb, int nth) -> cudaError_t {
            const size_t smem = smem1 * tb;
            cudaError_t er = cudaFuncSetAttribute(
                kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (er != cudaSuccess) return er;
            dim3 gr((unsigned)nblk, (unsigned)((nt + tb - 1) / tb));
            kern<<<gr, nth, smem, s>>>(g, ks, M, (const PtRec<float, 2>*)recs, sa, ct,
                                       (cplx_t<float>*)ft, nftot, nt, m, use, t0);
            note_launch();
            return cudaSuccess;
          };
          // four stacked transforms per 512-thread block (two blocks per SM)
#define GBN_ROWS2(W_)                                                          \
  e = g.bs[0] == 16 ? go_rows2(spread_rows2_kernel<TD, W_, 16, 4, 512>, 4, 512) \
                    : go_rows2(spread_rows2_kernel<TD, W_, 32, 4, 512>, 4, 512);
          switch (g.w) {
            case 4:
              GBN_ROWS2(4)
              break;
            case 5:
              GBN_ROWS2(5)
              break;
            case 6:
              GBN_ROWS2(6)
              break;
            case 7:
              GBN_ROWS2(7)
              break;
            default:
              GBN_ROWS2(8)
              break;
          }
#undef GBN_ROWS2
          if (e != cudaSuccess) return e;
          e = cudaGetLastError();
          if (e != cudaSuccess) return e;
          continue;
        }
      }
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
