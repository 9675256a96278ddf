// Host check of the FP32 fold's integer fast path (gbn_fold.cuh) against the
// FP64 chain it stands in for: for every float bit pattern in a stride over
// all 2^32 (non-finite ones included), wherever fold_fast_f32 accepts a
// point, its grid start and FP32 offset must equal those of the FP64 chain.
// Usage: fold_fast_check nf w stride threads [boundary]; prints
// "<accepted> <mismatches>".  With "boundary" the inputs are instead the
// floats within 64 ulps of every grid cell and half cell, x = 2 pi (j + o)/nf
// for j in [-nf, nf) and o in {0, 1/2}: where the ceiling of s and the FP32
// rounding of the offset are closest to a decision.
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "gbn_fold.cuh"

namespace {

const double kInv2Pi = 0.159154943091895335768883763372514362;

// The FP64 chain: t = RN(x K), f = t - floor(t) (t itself on [0, 1), RN(t + 1)
// on [-1, 0)), s = RN(f nf - w/2); non-finite x fold as 0.
double grid_shift(float xin, double nf_d, double hw) {
  const double x = std::isfinite(xin) ? (double)xin : 0.0;
  const double t = x * kInv2Pi;
  uint64_t b;
  std::memcpy(&b, &t, 8);
  const unsigned e = (unsigned)(b >> 52) & 0x7FFu;
  const bool neg = (b >> 63) != 0;
  double f;
  if (e < 0x3FFu && (!neg || (b << 1) == 0))
    f = t;
  else if (neg && (e < 0x3FFu || b == 0xBFF0000000000000ull))
    f = t + 1.0;
  else
    f = t - std::floor(t);
  return std::fma(f, nf_d, -hw);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 5) return 2;
  const int nf = std::atoi(argv[1]), w = std::atoi(argv[2]);
  const uint64_t stride = std::strtoull(argv[3], nullptr, 10);
  const int nt = std::atoi(argv[4]);
  uint64_t kb;
  std::memcpy(&kb, &kInv2Pi, 8);
  const uint64_t kmant = (kb & ((1ull << 52) - 1)) | (1ull << 52);
  const int kexp = (int)((kb >> 52) & 0x7FF) - 1075;
  int lnf = 0;
  while ((1ll << lnf) < nf) ++lnf;
  std::atomic<long long> accepted{0}, bad{0};
  auto check = [&](float x, long long& a, long long& m) {
    int i0 = 0;
    float d = 0.f;
    if (!gbn::fold_fast_f32(x, nf, w, lnf, kmant, kexp, i0, d)) return;
    ++a;
    const double sh = grid_shift(x, nf, 0.5 * w);
    const double cl = std::ceil(sh);
    const float rd = (float)(cl - sh);
    if ((int)cl != i0 || std::memcmp(&d, &rd, 4) != 0) ++m;
  };
  if (argc > 5 && std::strcmp(argv[5], "boundary") == 0) {
    long long a = 0, m = 0;
    const double pi = 3.14159265358979323846;
    for (long long j = -nf; j < nf; ++j) {
      for (int h = 0; h < 2; ++h) {
        const float x0 = (float)(2.0 * pi * ((double)j + 0.5 * h) / nf);
        uint32_t b0;
        std::memcpy(&b0, &x0, 4);
        for (int k = -64; k <= 64; ++k) {
          const uint32_t bk = b0 + (uint32_t)k;
          float x;
          std::memcpy(&x, &bk, 4);
          check(x, a, m);
        }
      }
    }
    std::printf("%lld %lld\n", a, m);
    return 0;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t) {
    th.emplace_back([&, t] {
      long long a = 0, m = 0;
      for (uint64_t u = (uint64_t)t; u < (1ull << 32); u += stride * (uint64_t)nt) {
        const uint32_t bits = (uint32_t)(u * 2654435761ull % (1ull << 32)) ^ (uint32_t)(u & 1);
        float x;
        std::memcpy(&x, &bits, 4);
        int i0 = 0;
        float d = 0.f;
        if (!gbn::fold_fast_f32(x, nf, w, lnf, kmant, kexp, i0, d)) continue;
        ++a;
        const double sh = grid_shift(x, nf, 0.5 * w);
        const double cl = std::ceil(sh);
        const float rd = (float)(cl - sh);
        if ((int)cl != i0 || std::memcmp(&d, &rd, 4) != 0) ++m;
      }
      accepted += a;
      bad += m;
    });
  }
  for (auto& x : th) x.join();
  std::printf("%lld %lld\n", (long long)accepted, (long long)bad);
  return 0;
}
