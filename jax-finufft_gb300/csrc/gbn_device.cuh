// gbn_device.cuh -- device helpers shared by the spread and interp kernels.
#pragma once

#include "gbn_common.cuh"

namespace gbn {

// Lanes per point: a group of G consecutive lanes handles one point, lane gl
// owning piece gl of the kernel (x offset gl of the w-wide support).
// G = 6 covers w <= 6, G = 8 covers w <= 8, G = 16 covers w <= 16; a warp
// holds 32 / G groups (lanes past the last whole group stay idle).  NCO is the number of Horner
// coefficients held in registers (degree w + 2, zero-padded).
template <int G>
struct GroupCfg;
template <>
struct GroupCfg<6> {
  static constexpr int NCO = 9;  // w <= 6: five groups per warp, lanes 30-31 idle
};
template <>
struct GroupCfg<8> {
  static constexpr int NCO = 11;
};
template <>
struct GroupCfg<16> {
  static constexpr int NCO = 19;
};

// Load this lane's piece of the piecewise polynomial into registers.
template <typename T, int NCO>
__device__ __forceinline__ void load_coef(T (&co)[NCO], const KerSpec<T>& ks, int piece, int w) {
#pragma unroll
  for (int n = 0; n < NCO; ++n)
    co[n] = (piece < w && n <= ks.deg) ? ks.coef[piece * (ks.deg + 1) + n] : T(0);
}

__device__ __forceinline__ float bessel_i0_dev(float x) { return cyl_bessel_i0f(x); }
__device__ __forceinline__ double bessel_i0_dev(double x) { return cyl_bessel_i0(x); }
__device__ __forceinline__ float bessel_i1_dev(float x) { return cyl_bessel_i1f(x); }
__device__ __forceinline__ double bessel_i1_dev(double x) { return cyl_bessel_i1(x); }

// Kernel value of piece `piece` at offset delta in [0, 1): Horner in
// u = 2*delta - 1, or the direct formula: exp(beta*(sqrt(1-z^2)-1)), or
// I0(beta*sqrt(1-z^2)) / I0(beta) for the Kaiser-Bessel shape.
template <typename T, int NCO>
__device__ __forceinline__ T kerval(const T (&co)[NCO], const KerSpec<T>& ks, T delta, int piece,
                                    int w) {
  if (ks.meth == 0) {
    if (piece >= w) return T(0);
    const T t = (T)piece - T(0.5) * (T)w + delta;
    const T z = t * (T(2) / (T)w);
    const T s = T(1) - z * z;
    if (!(s > T(0))) return T(0);
    if (ks.shape == 1) return bessel_i0_dev(ks.beta * sqrt(s)) * ks.inv_i0b;
    return exp(ks.beta * (sqrt(s) - T(1)));
  }
  const T u = T(2) * delta - T(1);
  T v = T(0);
#pragma unroll
  for (int n = NCO - 1; n >= 0; --n) v = fma(v, u, co[n]);
  return v;
}

// Lane layout of the row-owned spread kernel (3D, FP32 compute, bins
// 16 x 16 x bz, kernel widths 4..8).  Sixteen lanes serve one point: lane
// q = (r, gl) with gl = q % WV an x offset and r = q / WV one of R rows, WV =
// w rounded up to even.  The tile's row pitch is PY = tile_x(16, w) = 16 + WV
// cells, congruent to WV modulo 16, so the cells gl + PY r of the sixteen
// lanes fall on distinct 8-byte bank pairs; a point takes NCH = ceil(w / R)
// row chunks times w planes of such accesses.
template <int W>
struct RowCfg {
  static constexpr int WV = (W + 1) & ~1;          // lanes per row
  static constexpr int R = 16 / WV;                 // rows per access
  static constexpr int NCH = (W + R - 1) / R;       // row chunks per z plane
  static constexpr int PY = 16 + WV;                // = tile_x(16, W)
  static constexpr int PZ = PY * (15 + W);          // cells per tile plane
  static constexpr int NCO = W <= 6 ? 9 : 11;       // Horner coefficients held
};


// Horner evaluation of one piece (coefficients in registers) at offset delta.
template <int NCO>
__device__ __forceinline__ float horner_piece(const float (&co)[NCO], float delta) {
  const float u = 2.f * delta - 1.f;
  float v = 0.f;
#pragma unroll
  for (int n = NCO - 1; n >= 0; --n) v = fmaf(v, u, co[n]);
  return v;
}

// Whether the row-owned spread serves this geometry (the caller checks the
// rest: FP32 compute, sorted points, Horner kernel values).  Lanes without a
// cell add zeros up to two tile rows (and one cell) past the last tile; the
// staged strengths that follow the tiles (maxsub complex values) must cover
// that reach, so small subproblem sizes take the G-lane kernel.
inline bool rows_reach_fits(const Geom& g) {
  return (int64_t)g.maxsub >= 2 * (int64_t)tile_x(g.bs[0], g.w) + 2;
}
inline bool rows_fit(const Geom& g, int deg) {
  if (g.dim != 3 || g.bs[0] != 16 || g.bs[1] != 16 || g.w < 4 || g.w > 8) return false;
  if (!rows_reach_fits(g)) return false;
  return deg + 1 <= (g.w <= 6 ? 9 : 11);
}

// Periodic wrap for indices in [-n, 3n).
__device__ __forceinline__ int64_t wrap_idx(int64_t i, int64_t n) {
  if (i < 0) i += n;
  while (i >= n) i -= n;
  return i;
}
__device__ __forceinline__ int wrap_i32(int i, int n) {
  if (i < 0) i += n;
  if (i >= n) i -= n;
  if (i >= n) i -= n;
  return i;
}

// Bin tile of a subproblem: origin (first grid index, may be negative) and
// extent per axis; points of the bin start at grid offsets [0, bs) from the
// bin's first grid start bin*bs - floor(w/2) (the bin rule of the fold
// kernel), so their w-wide supports fit in bs + w - 1 cells.  Along x the
// origin is rounded down to an even cell and the extent is tile_x(bs, w).
template <int DIM>
struct Tile {
  int org[3];
  int T[3];
  int ncell;
  __device__ __forceinline__ Tile(const Geom& g, int bin) {
    int rem = bin;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      org[d] = 0;
      T[d] = 1;
    }
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const int b = rem % g.nb[d];
      rem /= g.nb[d];
      org[d] = b * g.bs[d] - (g.w >> 1);
      T[d] = g.bs[d] + g.w - 1;
    }
    org[0] -= org[0] & 1;  // even start (two's complement: rounds negatives down too)
    T[0] = tile_x(g.bs[0], g.w);
    ncell = T[0] * T[1] * T[2];
  }
  // The tile lies inside one period of the grid on every axis (no wrap).
  __device__ __forceinline__ bool interior(const Geom& g) const {
    bool in = true;
#pragma unroll
    for (int d = 0; d < DIM; ++d) in = in && org[d] >= 0 && org[d] + T[d] <= (int)g.nf[d];
    return in;
  }
};

// ---------------------------------------------------------------------------
// Bulk tensor copies (TMA) and mbarriers, inline PTX for sm_90+ / sm_103a.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// Wait for phase `parity` of bar, giving up after `limit` polls (each poll
// suspends for a hardware-bounded time); false if it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int limit) {
  for (int i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// Copy the box at coordinates c (floats along x) of the map into dst,
// completing `bytes` transactions on bar.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
      : "memory");
}
// Element-wise add of the shared-memory box src into the map's box at c.
__device__ __forceinline__ void tma_reduce_add_2d(const CUtensorMap* map, const void* src, int c0,
                                                  int c1) {
  asm volatile(
      "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group"
      " [%0, {%2, %3}], [%1];" ::"l"(reinterpret_cast<uint64_t>(map)),
      "r"(smem_addr(src)), "r"(c0), "r"(c1)
      : "memory");
}
__device__ __forceinline__ void tma_reduce_add_3d(const CUtensorMap* map, const void* src, int c0,
                                                  int c1, int c2) {
  asm volatile(
      "cp.reduce.async.bulk.tensor.3d.global.shared::cta.add.tile.bulk_group"
      " [%0, {%2, %3, %4}], [%1];" ::"l"(reinterpret_cast<uint64_t>(map)),
      "r"(smem_addr(src)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// Wait until every committed bulk operation of this thread has read its
// shared-memory source.
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// Order this thread's generic-proxy shared-memory writes before later bulk
// (async-proxy) reads of them.
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Walks the cells tid, tid + step, ... of a T0 x T1 x T2 tile keeping the
// coordinates (c0, c1, c2) with additions instead of a division per cell.
struct CellWalk {
  int c0, c1, c2, d0, d1, d2, T0, T1;
  __device__ __forceinline__ CellWalk(int start, int step, int T0_, int T1_) : T0(T0_), T1(T1_) {
    c0 = start % T0;
    const int r = start / T0;
    c1 = r % T1;
    c2 = r / T1;
    d0 = step % T0;
    const int rs = step / T0;
    d1 = rs % T1;
    d2 = rs / T1;
  }
  __device__ __forceinline__ void next() {
    c0 += d0;
    if (c0 >= T0) {
      c0 -= T0;
      ++c1;
    }
    c1 += d1;
    if (c1 >= T1) {
      c1 -= T1;
      ++c2;
    }
    c2 += d2;
  }
};

__device__ __forceinline__ void atomic_add_c(float2* p, float a, float b) {
  atomicAdd(p, make_float2(a, b));
}
__device__ __forceinline__ void atomic_add_c(double2* p, double a, double b) {
  atomicAdd(&p->x, a);
  atomicAdd(&p->y, b);
}

template <typename TD, typename TC>
__device__ __forceinline__ void load_c(const cplx_t<TD>* p, TC& re, TC& im) {
  const cplx_t<TD> v = *p;
  re = (TC)v.x;
  im = (TC)v.y;
}

}  // namespace gbn
