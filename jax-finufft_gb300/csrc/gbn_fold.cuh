// gbn_fold.cuh -- integer fast path of the periodic fold for FP32 coordinates.
//
// The FP64 fold (t = RN(x * K) with K = RN(1/(2 pi)), f = t - floor(t),
// s = RN(f*nf - w/2), i0 = ceil(s), delta = RN32(RN(i0 - s))) runs on the
// FP64 pipe, which on this GPU issues a small fraction of the FP32/integer
// rate.  For an FP32 coordinate x = mx * 2^e the product x * K is an exact
// 77-bit integer times a power of two, so the fractional part of x*K, and
// from it s, follow exactly in 64-bit fixed point with integer multiplies.
// The FP64 chain differs from that exact value by its roundings, at most
//   E = nf*ulp(t)/2 + nf*2^-54 + ulp(s)/2 + 2^-54 <= 2^(lnf + max(eT,0) - 50)
// cells (lnf = ceil(log2 nf), |t| < 2^eT).  Whenever no decision of the FP64
// chain lies within E of the exact value -- the floor of t, the ceiling of
// s, the FP32 rounding of delta -- both give the same i0 and delta, and the
// fast path returns them; otherwise it declines and the caller runs the FP64
// chain.  Declined points are those within about 2^(lnf - 25) (relative to an
// FP32 ulp) of a boundary: about 1e-5 of uniformly spread points at nf = 512.
//
// __host__ __device__ so that a host build can check it exhaustively against
// the FP64 chain.
#pragma once

#include <cstdint>
#include <cstring>

#ifndef __CUDACC__
#define GBN_HD
#else
#define GBN_HD __host__ __device__
#endif

namespace gbn {

GBN_HD inline uint64_t fold_mulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

GBN_HD inline int fold_clz(uint64_t v) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)v);
#else
  return v ? __builtin_clzll(v) : 64;
#endif
}

GBN_HD inline uint32_t fold_bits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t b;
  std::memcpy(&b, &x, 4);
  return b;
#endif
}

GBN_HD inline float fold_float(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float x;
  std::memcpy(&x, &b, 4);
  return x;
#endif
}

// The FP64 constant K = kmant * 2^kexp (kmant with its leading bit, 53 bits)
// and ceil(log2 nf), filled on the host.
struct FoldFast {
  uint64_t kmant;
  int kexp;
  int lnf[3];
};

// Periodic fold of x for a grid of nf cells and kernel width w: true with
// the grid start i0 (before wrapping) and the offset delta, equal to what the
// FP64 chain gives; false where the caller must run the FP64 chain (zero,
// subnormal or non-finite x, |x/(2 pi)| >= 2^20, or a boundary within the
// error bound).
GBN_HD inline bool fold_fast_f32(float x, int nf, int w, int lnf, uint64_t kmant, int kexp,
                                 int& i0, float& delta) {
  const uint32_t b = fold_bits(x);
  const uint32_t ex = (b >> 23) & 0xFFu;
  if (ex == 0u || ex == 0xFFu) return false;
  const uint64_t mx = (uint64_t)((b & 0x7FFFFFu) | 0x800000u);
  // |x| * K = P / 2^sh with P = mx * kmant < 2^77
  const int sh = -((int)ex - 150 + kexp);
  if (sh <= 0) return false;
  const uint64_t plo = mx * kmant, phi = fold_mulhi(mx, kmant);
  const int plen = phi ? 128 - fold_clz(phi) : 64 - fold_clz(plo);
  const int eT = plen - sh;  // 2^(eT-1) <= |t| < 2^eT
  if (eT > 20) return false;
  const int eTp = eT > 0 ? eT : 0;
  // fractional part of |t| in units of 2^-64 (truncated when sh > 64)
  uint64_t fa;
  if (sh <= 64) {
    fa = plo << (64 - sh);
  } else {
    const int k = sh - 64;
    fa = k >= 128 ? 0 : k >= 64 ? (phi >> (k - 64)) : ((plo >> k) | (phi << (64 - k)));
  }
  const uint64_t F = (b >> 31) ? (uint64_t)0 - fa : fa;  // frac(t) for negative t
  // the floor of t: F must stay clear of 0 and 1 by ulp(t)-scale margins
  const int efb = 14 + eTp;
  const uint64_t ef = (uint64_t)1 << efb;
  if (F < ef || (uint64_t)0 - F < ef) return false;
  // s + w/2 = F * nf / 2^64 = I + R / 2^64
  uint64_t R = F * (uint64_t)nf;
  int64_t I = (int64_t)fold_mulhi(F, (uint64_t)nf);
  const int h = w >> 1;
  if (w & 1) {  // w/2 = h + 1/2
    if (R >= ((uint64_t)1 << 63)) {
      R -= (uint64_t)1 << 63;
      I -= h;
    } else {
      R += (uint64_t)1 << 63;
      I -= h + 1;
    }
  } else {
    I -= h;
  }
  // s = I + R / 2^64; the error bound in units of 2^-64
  const int edb = lnf + eTp + 15;
  if (edb >= 60) return false;
  const uint64_t ed = (uint64_t)1 << edb;
  if (R < ed || (uint64_t)0 - R < ed) return false;  // ceil(s) undecided
  // delta = 1 - R / 2^64 = D / 2^64, rounded to FP32
  const uint64_t D = (uint64_t)0 - R;
  const int p = 63 - fold_clz(D);
  if (p < 40) return false;
  if (D - ((uint64_t)1 << p) < ed) return false;  // next to the binade below
  const int us = p - 23;
  const uint64_t q = D >> us, rem = D & (((uint64_t)1 << us) - 1);
  const uint64_t half = (uint64_t)1 << (us - 1);
  const uint64_t gap = rem > half ? rem - half : half - rem;
  if (gap <= ed) return false;  // next to a rounding midpoint
  const uint32_t qr = (uint32_t)(q + (rem > half ? 1 : 0));  // <= 2^24, exact in FP32
  const float scale = fold_float((uint32_t)(127 + us - 64) << 23);
  delta = (float)qr * scale;
  i0 = (int)(I + 1);
  return true;
}

}  // namespace gbn
