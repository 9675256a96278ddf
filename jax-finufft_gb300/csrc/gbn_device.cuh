// gbn_device.cuh -- device helpers shared by the spread and interp kernels.
#pragma once

#include "gbn_common.cuh"

namespace gbn {

// Lanes per point: a group of G consecutive lanes handles one point, lane gl
// owning piece gl of the kernel (x offset gl of the w-wide support).
// G = 8 covers w <= 8, G = 16 covers w <= 16.  NCO is the number of Horner
// coefficients held in registers (degree w + 2, zero-padded).
template <int G>
struct GroupCfg;
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

// Kernel value of piece `piece` at offset delta in [0, 1): Horner in
// u = 2*delta - 1, or the direct formula exp(beta*(sqrt(1-z^2)-1)).
template <typename T, int NCO>
__device__ __forceinline__ T kerval(const T (&co)[NCO], const KerSpec<T>& ks, T delta, int piece,
                                    int w) {
  if (ks.meth == 0) {
    if (piece >= w) return T(0);
    const T t = (T)piece - T(0.5) * (T)w + delta;
    const T z = t * (T(2) / (T)w);
    const T s = T(1) - z * z;
    return s > T(0) ? exp(ks.beta * (sqrt(s) - T(1))) : T(0);
  }
  const T u = T(2) * delta - T(1);
  T v = T(0);
#pragma unroll
  for (int n = NCO - 1; n >= 0; --n) v = fma(v, u, co[n]);
  return v;
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
// extent bs + w - 1 per axis; points of the bin start at tile offsets
// [0, bs) (the bin rule of the fold kernel), so their supports fit.
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
    ncell = T[0] * T[1] * T[2];
  }
};

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
