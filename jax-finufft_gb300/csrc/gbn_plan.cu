// gbn_plan.cu -- host side of the library: plans, setpts/execute
// orchestration, cuFFT, the plan cache and the C ABI (include/gbnufft.h).
//
// Replaces lib/kernels.cc.cu (run_nufft and the nufft{d}d{t}{f}_impl
// functions) and lib/cufinufft_wrapper.cc (makeplan/setpts/execute/destroy).
// Differences from the reference driver, all deliberate:
//   * plans (kernel coefficients, deconvolution factors, cuFFT plan, grids
//     and sort buffers) are cached across one-shot calls instead of being
//     rebuilt per call (kernels.cc.cu:51);
//   * the host is never blocked at the end of a call (kernels.cc.cu:83); all
//     work is stream-ordered and scratch memory is stream-ordered
//     (cudaMallocAsync/cudaFreeAsync);
//   * double-precision 3D does not force global-memory spreading
//     (cufinufft_wrapper.cc:33-35): the shared-memory method is used while
//     its tile fits.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <list>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/gbnufft.h"
#include "gbn_common.cuh"

using namespace gbn;

namespace gbn {
static std::atomic<long long> g_launches{0};
void note_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
}  // namespace gbn

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

// A bounded device-side wait that gave up (a tile copy into shared memory
// that never completed; the kernel then skipped that block's output) turns
// the status of the first API call on that device that observes it into an
// error: the check reads mapped host memory and does not synchronise, so it
// reports work enqueued by this or an earlier call, like CUDA's own
// asynchronous errors.
int check_waits(int r) {
  if (r >= 2) return r;
  if (gbn::wait_flag_take())
    return fail(GBN_ERR_CUDA,
                "a bounded device-side wait gave up (tile copy into shared memory): outputs of "
                "the calls enqueued on this device since the previous check are invalid");
  if (gbn::extent_flag_take())
    return fail(GBN_ERR_ARGS,
                "type-3 points outside the extents given to gbn_set_t3_extents: outputs of the "
                "calls enqueued on this device since the previous check are invalid");
  return r;
}

#define GBN_CUDA(expr)                                                                    \
  do {                                                                                    \
    cudaError_t e_ = (expr);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(GBN_ERR_CUDA, std::string(#expr) + " failed: " + cudaGetErrorString(e_)); \
  } while (0)

#define GBN_TRY(expr)      \
  do {                     \
    int r_ = (expr);       \
    if (r_ >= 2) return r_; \
  } while (0)

constexpr double kPi = 3.141592653589793238462643383279502884;

// ---------------------------------------------------------------------------
// plan-time arithmetic (same rules as the CPU restatement in oracle/)
// ---------------------------------------------------------------------------
int64_t next235even(int64_t n0) {
  if (n0 <= 2) return 2;
  int64_t n = (n0 % 2) ? n0 + 1 : n0;
  for (;; n += 2) {
    int64_t m = n;
    while (m % 2 == 0) m /= 2;
    while (m % 3 == 0) m /= 3;
    while (m % 5 == 0) m /= 5;
    if (m == 1) return n;
  }
}

// Width w and shape parameter beta for tolerance eps; returns 1 when the
// width is clamped at kMaxW.  The width rule is the published one for the
// exponential of semicircle (shape 0) and is kept for Kaiser-Bessel (shape
// 1), whose beta follows Beatty, Nishimura and Pauly (IEEE TMI 2005).
int kernel_params(double eps, double sigma, int shape, int* w_out, double* beta_out) {
  int warn = 0;
  double a = (sigma == 2.0) ? -std::log10(eps / 10.0)
                            : -std::log(eps) / (kPi * std::sqrt(1.0 - 1.0 / sigma));
  // a tolerance given in single precision (1e-5f = 9.99999975e-6) must not
  // gain a kernel width from its rounding: snap to the integer within 1e-5
  if (std::fabs(a - std::round(a)) < 1e-5) a = std::round(a);
  double wd = std::ceil(a);
  if (!(wd >= 2.0)) wd = 2.0;
  if (wd > kMaxW) {
    wd = kMaxW;
    warn = 1;
  }
  const int w = (int)wd;
  double ratio;
  if (sigma == 2.0) {
    ratio = 2.30;
    if (w == 2) ratio = 2.20;
    if (w == 3) ratio = 2.26;
    if (w == 4) ratio = 2.38;
  } else {
    ratio = 0.97 * kPi * (1.0 - 1.0 / (2.0 * sigma));
  }
  *w_out = w;
  *beta_out = ratio * (double)w;
  if (shape == 1) {
    const double a = ((double)w / sigma) * (sigma - 0.5);
    *beta_out = kPi * std::sqrt(std::max(a * a - 0.8, 0.25));
  }
  return warn;
}

int64_t fine_size(int64_t n, double sigma, int w) {
  int64_t m = (int64_t)std::ceil(sigma * (double)n);
  if (m < 2 * (int64_t)w) m = 2 * (int64_t)w;
  return next235even(m);
}

// Upsampling factor of a type-3 plan's inner FP32 type-2 transform: a little
// below 2 where that puts every axis of its fine grid on a power of two
// (128..1024: the library's own pruned FFT with the deconvolution fused,
// against cuFFT on the 2,3,5-smooth sizes of sigma = 2) without widening
// the kernel; sigma = 2 otherwise.  The width and shape parameter follow the
// published rules for the factor chosen, which hold the tolerance.
double inner_sigma_pow2(int dim, const int64_t* n, double eps, int shape) {
  int w2 = 0;
  double b2 = 0.0;
  kernel_params(eps, 2.0, shape, &w2, &b2);
  int64_t P[3] = {1, 1, 1}, nf2[3] = {1, 1, 1};
  double sig = 2.0;
  bool already = true;
  for (int d = 0; d < dim; ++d) {
    nf2[d] = fine_size(n[d], 2.0, w2);
    int64_t q = 1;
    while (q * 2 <= nf2[d]) q *= 2;
    if (q < 128 || q > 1024 || (double)q < 1.5 * (double)n[d]) return 2.0;
    P[d] = q;
    if (q != nf2[d]) already = false;
    sig = std::min(sig, (double)q / (double)n[d]);
  }
  if (already) return 2.0;
  sig *= 1.0 - 1e-12;  // ceil(sig n) stays at the power of two
  int w = 0;
  double b = 0.0;
  kernel_params(eps, sig, shape, &w, &b);
  if (w != w2) return 2.0;
  for (int d = 0; d < dim; ++d)
    if (fine_size(n[d], sig, w) != P[d]) return 2.0;
  return fft_pow2_supported(dim, P, 1) ? sig : 2.0;
}

double kernel_value(double t, int w, double beta, int shape) {
  const double z = 2.0 * t / (double)w;
  const double s = 1.0 - z * z;
  return s < 0.0 ? 0.0 : kernel_of_s(shape, beta, std::sqrt(s));
}

// Chebyshev interpolation of each unit piece at degree deg, as monomials in
// u = 2*delta - 1.
void horner_fit(int w, double beta, int shape, int deg, std::vector<double>& coef) {
  const int n1 = deg + 1;
  std::vector<double> node(n1), val(n1), cheb(n1);
  std::vector<std::vector<double>> tk(n1, std::vector<double>(n1, 0.0));
  for (int i = 0; i < n1; ++i) node[i] = std::cos(kPi * (i + 0.5) / n1);
  tk[0][0] = 1.0;
  if (n1 > 1) tk[1][1] = 1.0;
  for (int k = 2; k < n1; ++k)
    for (int n = 0; n < n1; ++n) tk[k][n] = (n ? 2.0 * tk[k - 1][n - 1] : 0.0) - tk[k - 2][n];
  coef.assign((size_t)w * n1, 0.0);
  for (int j = 0; j < w; ++j) {
    for (int i = 0; i < n1; ++i)
      val[i] = kernel_value(j - 0.5 * w + 0.5 * (node[i] + 1.0), w, beta, shape);
    for (int k = 0; k < n1; ++k) {
      double s = 0.0;
      for (int i = 0; i < n1; ++i) s += val[i] * std::cos(kPi * k * (i + 0.5) / n1);
      cheb[k] = s * (k == 0 ? 1.0 : 2.0) / n1;
    }
    for (int n = 0; n < n1; ++n) {
      double s = 0.0;
      for (int k = 0; k < n1; ++k) s += cheb[k] * tk[k][n];
      coef[(size_t)j * n1 + n] = s;
    }
  }
}

void gauss_legendre(int q, double* x, double* wt) {
  for (int i = 0; i < (q + 1) / 2; ++i) {
    double z = std::cos(kPi * (i + 0.75) / (q + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= q; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = q * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
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

// psihat(omega) = int psi(t) cos(omega t) dt, t = (w/2) sin(theta) substitution.
void kernel_ft(int w, double beta, int shape, const std::vector<double>& omega,
               std::vector<double>& out) {
  const int q = 2 * w + 10;
  double xg[64], wg[64], tq[64], fq[64];
  gauss_legendre(q, xg, wg);
  for (int i = 0; i < q; ++i) {
    const double th = (xg[i] + 1.0) * kPi / 4.0;
    const double wt = wg[i] * kPi / 4.0;
    tq[i] = 0.5 * w * std::sin(th);
    fq[i] = 2.0 * wt * kernel_of_s(shape, beta, std::cos(th)) * 0.5 * w * std::cos(th);
  }
  out.resize(omega.size());
  for (size_t k = 0; k < omega.size(); ++k) {
    double s = 0.0;
    for (int i = 0; i < q; ++i) s += fq[i] * std::cos(omega[k] * tq[i]);
    out[k] = s;
  }
}

int64_t type3_params(double xmin, double xmax, double smin, double smax, double sigma, int w,
                     double* cx, double* cs, double* scale) {
  *cx = 0.5 * (xmax + xmin);
  const double hx = 0.5 * (xmax - xmin);
  *cs = 0.5 * (smax + smin);
  const double hs = 0.5 * (smax - smin);
  double X = hx, S = hs;
  if (X == 0.0) {
    if (S == 0.0) {
      X = 1.0;
      S = 1.0;
    } else if (X < 1.0 / S) {
      X = 1.0 / S;
    }
  } else if (S < 1.0 / X) {
    S = 1.0 / X;
  }
  double nfd = 2.0 * sigma * S * X / kPi + (double)(w + 1);
  if (!std::isfinite(nfd)) nfd = 0.0;
  int64_t nf = (int64_t)nfd;
  if (nf < 2 * (int64_t)w) nf = 2 * (int64_t)w;
  nf = next235even(nf);
  *scale = sigma * S / kPi;
  return nf;
}

int64_t mode_freq(int64_t i, int64_t N, int modeord) {
  if (modeord == 0) return i - N / 2;
  return i < (N + 1) / 2 ? i : i - N;
}

// ---------------------------------------------------------------------------
// stream-ordered device buffer
// ---------------------------------------------------------------------------
struct DevBuf {
  void* p = nullptr;
  size_t n = 0;
  cudaError_t ensure(size_t bytes, cudaStream_t s) {
    if (bytes <= n && p) return cudaSuccess;
    release(s);
    if (bytes == 0) return cudaSuccess;
    cudaError_t e = cudaMallocAsync(&p, bytes, s);
    if (e != cudaSuccess) {
      p = nullptr;
      n = 0;
      return e;
    }
    n = bytes;
    return cudaSuccess;
  }
  void release(cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    n = 0;
  }
  template <typename T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

size_t rec_size(int dim, bool single) {
  if (single) {
    switch (dim) {
      case 1:
        return sizeof(PtRec<float, 1>);
      case 2:
        return sizeof(PtRec<float, 2>);
      default:
        return sizeof(PtRec<float, 3>);
    }
  }
  switch (dim) {
    case 1:
      return sizeof(PtRec<double, 1>);
    case 2:
      return sizeof(PtRec<double, 2>);
    default:
      return sizeof(PtRec<double, 3>);
  }
}

}  // namespace

// =============================================================================
// point sets and plans
// =============================================================================

// Sorted nonuniform points for a plan's geometry.  A plan owns one (the
// classic setpts/execute API); gbn_points_create makes more that outlive an
// execute, so a gradient can reuse the forward's sort.
struct gbn_points_s {
  DevBuf pt_bin, pt_rank, bin_count, bin_start, perm, sub_count, sub_start, sub_bin, sub_off,
      n_sub, recs, recs_in, scan_tmp, key_count, key_start;
  int rows = 1;  // sort keys per bin of the last sort
  SortState st{};
  int64_t M = 0;
  bool set = false;
  // geometry it was sorted for (checked against the plan that uses it)
  int dim = 0;
  bool comp_single = true;
  int64_t nf[3] = {0, 0, 0};
  int w = 0;
  cudaStream_t stream = nullptr;

  void release() {
    DevBuf* bufs[] = {&pt_bin,  &pt_rank, &bin_count, &bin_start, &perm,    &sub_count,
                      &sub_start, &sub_bin, &sub_off, &n_sub,   &recs,      &recs_in,
                      &scan_tmp, &key_count, &key_start};
    for (DevBuf* b : bufs) b->release(stream);
  }
  ~gbn_points_s() { release(); }
};

struct gbn_plan_s {
  int type = 1, dim = 1, iflag = 1, ntransf = 1;
  bool data_single = true, comp_single = true;
  double eps = 1e-6, sigma = 2.0, beta = 0.0;
  int w = 2, deg = 4, warn = 0;
  int64_t N[3] = {1, 1, 1};
  int64_t nf[3] = {1, 1, 1};
  int64_t nftot = 1, Ntot = 1;
  gbn_opts opts{};
  int method = 2;
  bool sorted = true;
  int batch = 1;
  cudaStream_t stream = nullptr;
  int device = 0;
  Geom geom{};

  DevBuf coef, phi[3], fine, gfine;
  gbn_points_s own;  // the point set of setpts/execute

  // cuFFT plans by batch count (fine grids per exec)
  std::vector<std::pair<int, cufftHandle>> ffts;
  // pruned 3D FFT: 2D plans over the low and high planes of the mode region
  // and one strided 1D plan along z, sharing one work area
  cufftHandle fft_lo = 0, fft_hi = 0, fft_z = 0;
  int64_t prune_lo = 0, prune_hi = 0;
  int prune_state = 0;  // 0 not tried, 1 ready, -1 not applicable
  DevBuf fft_work;
  // FP32 power-of-two grids: the library's own pruned FFT with the
  // deconvolution fused (gbn_fft.cu), twiddles exp(2 pi i m / nf) per axis
  bool fft_own = false;
  DevBuf fft_tw[3];

  // type 3
  std::unique_ptr<gbn_plan_s> inner;
  double t3_cx[3] = {0, 0, 0}, t3_cs[3] = {0, 0, 0}, t3_scale[3] = {1, 1, 1};
  // extents declared by gbn_set_t3_extents: x_lo, x_hi, s_lo, s_hi per axis
  bool t3_ext = false;
  double t3_ext_v[4][3] = {};
  T3PsihatCache t3_tab;  // the fitted psihat table, kept on the device across setpts calls
  int64_t Nt = 0;
  DevBuf t3_tau[3], t3_pre, t3_post, t3_cbuf, t3_obuf, t3_minmax;

  // debug timings: 4 events per executed batch (stage boundaries) and 2 per
  // setpts, recorded without host synchronisation and summed by
  // gbn_get_timings, which then resets the pool.
  // per-call driver (gbn_run): the arguments of recent calls and, for
  // arguments that came again, that call's setpts + execute captured as a
  // CUDA graph, replayed by later identical calls (types 1 and 2).  All are
  // for one (n_tot, n_j): a call of other sizes may grow the plan's buffers
  // and drops them first.
  struct OneshotArgs {
    int64_t n_tot, n_j, n_k_total;
    const void* src;
    void* out;
    const void* pts[3];
  };
  static constexpr size_t kOneshotKeep = 4;
  std::vector<OneshotArgs> os_seen;
  std::vector<std::pair<OneshotArgs, cudaGraphExec_t>> os_graphs;
  bool os_nograph = false;  // a capture failed: no graphs for this plan
  // stream the graphs are captured on (the caller's may be the legacy
  // default stream, which cannot be captured; a graph launches on any)
  cudaStream_t os_cap = nullptr;
  void os_clear() {
    for (auto& g : os_graphs) cudaGraphExecDestroy(g.second);
    os_graphs.clear();
    os_seen.clear();
  }

  bool ev_ok = false;
  std::vector<cudaEvent_t> ev_exec, ev_setpts;
  size_t ev_exec_used = 0, ev_setpts_used = 0;

  ~gbn_plan_s() {
    cudaStreamSynchronize(stream);
    DevBuf* bufs[] = {&coef,      &phi[0],    &phi[1],    &phi[2],    &fine,      &gfine,
                      &t3_tau[0], &t3_tau[1], &t3_tau[2], &t3_pre,    &t3_post,   &t3_cbuf,
                      &t3_obuf,   &t3_minmax, &fft_tw[0], &fft_tw[1], &fft_tw[2]};
    for (DevBuf* b : bufs) b->release(stream);
    if (t3_tab.dev) cudaFree(t3_tab.dev);
    own.stream = stream;
    own.release();
    for (auto& h : ffts) cufftDestroy(h.second);
    for (cufftHandle h : {fft_lo, fft_hi, fft_z})
      if (h) cufftDestroy(h);
    fft_work.release(stream);
    for (auto& e : ev_exec) cudaEventDestroy(e);
    for (auto& e : ev_setpts) cudaEventDestroy(e);
    os_clear();
    if (os_cap) cudaStreamDestroy(os_cap);
    cudaStreamSynchronize(stream);
  }
};

namespace {

size_t cplx_size(bool single) { return single ? 8 : 16; }

// Default bin sizes (cells per axis) for the shared-memory method.
void default_bins(int dim, bool single, int* bs) {
  bs[0] = bs[1] = bs[2] = 1;
  if (dim == 1) {
    bs[0] = 1024;
  } else if (dim == 2) {
    bs[0] = 32;
    bs[1] = 32;
  } else if (single) {
    bs[0] = 16;
    bs[1] = 16;
    bs[2] = 8;
  } else {
    bs[0] = 8;
    bs[1] = 8;
    bs[2] = 8;
  }
}

size_t tile_bytes(int dim, const int* bs, int w, bool single) {
  return (size_t)tile_cells(dim, bs, w) * 2 * (single ? 4 : 8);
}

// Fill geometry (bins, nb) for the current nf and options; choose method.
void setup_geom(gbn_plan_s* p) {
  Geom& g = p->geom;
  g.dim = p->dim;
  g.w = p->w;
  int bs[3];
  default_bins(p->dim, p->comp_single, bs);
  // type-1 3D FP32 at w <= 6 (the row-owned spread): bins 12 planes deep
  // halve the per-bin tile overhead of sparse bins for 1.5x the tile
  // (2.19 -> 2.06 ms on 1e7 mixed points, 512^3 grid; interp prefers 8)
  if (p->type == 1 && p->dim == 3 && p->comp_single && p->w <= 6) bs[2] = 12;
  // type-1 2D FP32 at w 4..8 (the 2D row-owned spread): bins 16 x 16
  // (32 stacked transforms, 4e6 points, 1024^2 grid: spread 5.57 -> 5.13 ms
  // and setpts 0.33 -> 0.23 ms against 32 x 32)
  if (p->type == 1 && p->dim == 2 && p->comp_single && p->w >= 4 && p->w <= 8)
    bs[0] = bs[1] = 16;
  const int user[3] = {p->opts.gpu_binsizex, p->opts.gpu_binsizey, p->opts.gpu_binsizez};
  for (int d = 0; d < 3; ++d) {
    if (d < p->dim && user[d] > 0) bs[d] = user[d];
    if (d >= p->dim) bs[d] = 1;
    if (d < p->dim && bs[d] > p->nf[d]) bs[d] = (int)p->nf[d];
    if (bs[d] < 1) bs[d] = 1;
  }
  // method: 1 = global atomics, 2 = shared-memory tiles
  int method = p->opts.gpu_method;
  const size_t smem_limit = 200 * 1024;
  if (!p->sorted) method = 1;
  if (method == 0) {
    method = 2;
    if (!p->comp_single && p->dim == 3 && tile_bytes(3, bs, p->w, false) > 96 * 1024) method = 1;
  }
  if (method == 2) {
    // shrink the largest bin axis until the tile fits
    while (tile_bytes(p->dim, bs, p->w, p->comp_single) > smem_limit) {
      int dmax = 0;
      for (int d = 1; d < p->dim; ++d)
        if (bs[d] > bs[dmax]) dmax = d;
      if (bs[dmax] <= 1) {
        method = 1;
        break;
      }
      bs[dmax] = (bs[dmax] + 1) / 2;
    }
  }
  p->method = method;
  g.nbins = 1;
  for (int d = 0; d < 3; ++d) {
    g.nf[d] = d < p->dim ? p->nf[d] : 1;
    g.bs[d] = bs[d];
    g.nb[d] = d < p->dim ? (int)((p->nf[d] + bs[d] - 1) / bs[d]) : 1;
    g.nbins *= g.nb[d];
  }
  g.maxsub = p->opts.gpu_maxsubprobsize > 0 ? p->opts.gpu_maxsubprobsize : 1024;
  // type-2 plans order a bin's points by tile row, so that the points a warp
  // gathers together read the same or neighbouring rows of the tile
  // (GBN_DISABLE_ROW_ORDER=1: bin order only)
  static const bool no_rows = std::getenv("GBN_DISABLE_ROW_ORDER") != nullptr;
  g.rows = 1;
  if (!no_rows && p->type == 2 && method == 2 && p->sorted && p->dim >= 2) {
    const int64_t r = p->dim == 2 ? bs[1] : (int64_t)bs[1] * bs[2];
    if (r > 1 && g.nbins * r < ((int64_t)1 << 30)) g.rows = (int)r;
  }
  // the FP32 fixed-point spread may round every contribution on the FMA pipe
  // (absolute resolution 2^-22 of the largest strength of a subproblem, a
  // relative error near 1e-6 of the output) where the tolerance leaves room
  // (1e-5 as float32, 9.99999975e-6, counts as 1e-5)
  g.coarse_round = p->eps >= 9.99e-6;
  // stage each subproblem's strengths in shared memory when it still fits
  g.stash = method == 2 && spread_smem_bytes(p->dim, bs, p->w, p->comp_single, g.maxsub, true) <=
                               smem_limit;
}

int upload_doubles_as(const std::vector<double>& v, bool single, DevBuf& buf, cudaStream_t s) {
  const size_t bytes = v.size() * (single ? 4 : 8);
  GBN_CUDA(buf.ensure(bytes, s));
  if (v.empty()) return GBN_OK;
  if (single) {
    std::vector<float> f(v.begin(), v.end());
    GBN_CUDA(cudaMemcpyAsync(buf.p, f.data(), bytes, cudaMemcpyHostToDevice, s));
    // keep host staging alive until the copy ran: pageable copies are staged
    // synchronously by the driver before the call returns
  } else {
    GBN_CUDA(cudaMemcpyAsync(buf.p, v.data(), bytes, cudaMemcpyHostToDevice, s));
  }
  return GBN_OK;
}

// Deconvolution factors 1/psihat(2 pi k / nf) per output index, per axis.
int setup_phi(gbn_plan_s* p) {
  for (int d = 0; d < p->dim; ++d) {
    std::vector<double> om((size_t)p->N[d]);
    for (int64_t i = 0; i < p->N[d]; ++i)
      om[(size_t)i] = 2.0 * kPi * (double)mode_freq(i, p->N[d], p->opts.modeord) / (double)p->nf[d];
    std::vector<double> ph;
    kernel_ft(p->w, p->beta, p->opts.gpu_kernel, om, ph);
    for (auto& v : ph) v = 1.0 / v;
    GBN_TRY(upload_doubles_as(ph, p->comp_single, p->phi[d], p->stream));
  }
  return GBN_OK;
}

// The library's own FFT applies to FP32 type-1/2 plans whose fine-grid axes
// all have 128, 256, 512 or 1024 cells; GBN_DISABLE_OWN_FFT=1 at execute
// time selects cuFFT and the separate deconvolution instead.
int setup_fft_own(gbn_plan_s* p) {
  p->fft_own = p->comp_single && p->type != 3 && fft_pow2_supported(p->dim, p->nf, p->batch);
  if (!p->fft_own) return GBN_OK;
  for (int d = 0; d < p->dim; ++d) {
    std::vector<float> tw;
    fft_pow2_twiddles(p->nf[d], tw);
    std::vector<double> twd(tw.begin(), tw.end());
    GBN_TRY(upload_doubles_as(twd, true, p->fft_tw[d], p->stream));
  }
  return GBN_OK;
}

int setup_kernel_coef(gbn_plan_s* p) {
  std::vector<double> coef;
  horner_fit(p->w, p->beta, p->opts.gpu_kernel, p->deg, coef);
  return upload_doubles_as(coef, p->comp_single, p->coef, p->stream);
}

int make_fft(gbn_plan_s* p, int nbatch, cufftHandle* h) {
  int n[3];
  for (int d = 0; d < p->dim; ++d) n[d] = (int)p->nf[p->dim - 1 - d];
  cufftResult r = cufftPlanMany(h, p->dim, n, nullptr, 1, (int)p->nftot, nullptr, 1,
                                (int)p->nftot, p->comp_single ? CUFFT_C2C : CUFFT_Z2Z, nbatch);
  if (r != CUFFT_SUCCESS) {
    *h = 0;
    return fail(GBN_ERR_CUFFT, "cufftPlanMany failed with code " + std::to_string((int)r));
  }
  return GBN_OK;
}

// Pruned 3D FFT plans (see exec_fft).  The mode region along z holds the
// planes [0, lo) and [nf2 - hi, nf2).
int make_pruned_fft(gbn_plan_s* p) {
  const int nf0 = (int)p->nf[0], nf1 = (int)p->nf[1], nf2 = (int)p->nf[2];
  const int64_t N2 = p->N[2];
  const int64_t lo = (N2 - 1) / 2 + 1, hi = N2 / 2;
  if (p->dim != 3 || lo + hi >= nf2) return GBN_ERR_ARGS;
  const cufftType ty = p->comp_single ? CUFFT_C2C : CUFFT_Z2Z;
  const int plane = nf0 * nf1;
  size_t ws[3] = {0, 0, 0};
  cufftHandle* hs[3] = {&p->fft_lo, &p->fft_hi, &p->fft_z};
  for (cufftHandle* h : hs) {
    if (cufftCreate(h) != CUFFT_SUCCESS || cufftSetAutoAllocation(*h, 0) != CUFFT_SUCCESS)
      return fail(GBN_ERR_CUFFT, "cufftCreate failed");
  }
  int n2[2] = {nf1, nf0};
  cufftResult r = cufftMakePlanMany(p->fft_lo, 2, n2, nullptr, 1, plane, nullptr, 1, plane, ty,
                                    (int)lo, &ws[0]);
  if (r == CUFFT_SUCCESS && hi > 0)
    r = cufftMakePlanMany(p->fft_hi, 2, n2, nullptr, 1, plane, nullptr, 1, plane, ty, (int)hi,
                          &ws[1]);
  int nz[1] = {nf2}, emb[1] = {nf2};
  if (r == CUFFT_SUCCESS)
    r = cufftMakePlanMany(p->fft_z, 1, nz, emb, plane, 1, emb, plane, 1, ty, plane, &ws[2]);
  if (r != CUFFT_SUCCESS)
    return fail(GBN_ERR_CUFFT, "pruned cufftMakePlanMany failed with code " + std::to_string((int)r));
  const size_t work = std::max(ws[0], std::max(ws[1], ws[2]));
  GBN_CUDA(p->fft_work.ensure(std::max<size_t>(work, 256), p->stream));
  for (cufftHandle* h : hs)
    if (cufftSetWorkArea(*h, p->fft_work.p) != CUFFT_SUCCESS)
      return fail(GBN_ERR_CUFFT, "cufftSetWorkArea failed");
  p->prune_lo = lo;
  p->prune_hi = hi;
  return GBN_OK;
}

int fft_exec(gbn_plan_s* p, cufftHandle h, void* data, int dir) {
  cufftSetStream(h, p->stream);
  const cufftResult r =
      p->comp_single ? cufftExecC2C(h, (cufftComplex*)data, (cufftComplex*)data, dir)
                     : cufftExecZ2Z(h, (cufftDoubleComplex*)data, (cufftDoubleComplex*)data, dir);
  if (r != CUFFT_SUCCESS)
    return fail(GBN_ERR_CUFFT, "cufftExec failed with code " + std::to_string((int)r));
  return GBN_OK;
}

// In-place batched FFT of nb fine grids at buf with exponent sign `sign`.
// kind 1: the input is zero outside the mode region (zero-padded modes);
// kind 2: only the mode region of the output is read afterwards.  For a
// large 3D grid either lets the FFT skip the planes outside the mode region
// along z: kind 1 transforms (x, y) on the mode region's planes, then z on
// every column; kind 2 transforms z first, then (x, y) on those planes only
// (the other planes are left partially transformed).  1/sigma of the plane
// work instead of all of it.  kind 0 (or GBN_DISABLE_FFT_PRUNING=1): the
// full transform.
int exec_fft(gbn_plan_s* p, void* buf, int nb, int sign, int kind = 0) {
  const int dir = sign >= 0 ? CUFFT_INVERSE : CUFFT_FORWARD;
  const char* no_prune = std::getenv("GBN_DISABLE_FFT_PRUNING");
  if (no_prune && no_prune[0] == '1') kind = 0;
  if (kind != 0 && p->dim == 3 && nb <= 8 && p->nftot >= ((int64_t)1 << 21)) {
    if (p->prune_state == 0) p->prune_state = make_pruned_fft(p) == GBN_OK ? 1 : -1;
    if (p->prune_state == 1) {
      const size_t csz = cplx_size(p->comp_single);
      const size_t plane = (size_t)p->nf[0] * p->nf[1] * csz;
      for (int t = 0; t < nb; ++t) {
        char* g = (char*)buf + (size_t)t * p->nftot * csz;
        char* g_hi = g + (size_t)(p->nf[2] - p->prune_hi) * plane;
        if (kind == 2) GBN_TRY(fft_exec(p, p->fft_z, g, dir));
        GBN_TRY(fft_exec(p, p->fft_lo, g, dir));
        if (p->prune_hi > 0) GBN_TRY(fft_exec(p, p->fft_hi, g_hi, dir));
        if (kind == 1) GBN_TRY(fft_exec(p, p->fft_z, g, dir));
      }
      return GBN_OK;
    }
  }
  cufftHandle h = 0;
  for (auto& e : p->ffts)
    if (e.first == nb) h = e.second;
  if (!h) {
    GBN_TRY(make_fft(p, nb, &h));
    p->ffts.emplace_back(nb, h);
    if (p->ffts.size() > 4) {  // keep the cache small: drop the oldest
      cufftDestroy(p->ffts.front().second);
      p->ffts.erase(p->ffts.begin());
    }
  }
  return fft_exec(p, h, buf, dir);
}

// Resolve compute precision; returns an error for unsupported combinations.
int resolve_precision(gbn_plan_s* p) {
  switch (p->opts.gpu_precision) {
    case 0:
      p->comp_single = p->data_single;
      break;
    case 1:
      p->comp_single = true;
      break;
    case 2:
      if (p->data_single)
        return fail(GBN_ERR_ARGS, "gpu_precision=2 (FP64 compute) needs complex128 data");
      p->comp_single = false;
      break;
    case 3:
      p->comp_single = p->data_single || p->eps >= 1e-6;
      break;
    default:
      return fail(GBN_ERR_ARGS, "gpu_precision must be 0..3");
  }
  return GBN_OK;
}

int plan_create(int type, int dim, const int64_t* nmodes, int iflag, int ntransf, double eps,
                bool data_single, const gbn_opts* opts_in, void* stream, gbn_plan_s** out) {
  *out = nullptr;
  if (type < 1 || type > 3) return fail(GBN_ERR_ARGS, "type must be 1, 2 or 3");
  if (dim < 1 || dim > 3) return fail(GBN_ERR_ARGS, "dim must be 1, 2 or 3");
  if (ntransf < 1) return fail(GBN_ERR_ARGS, "ntransf must be >= 1");
  if (!(eps > 0.0) || !std::isfinite(eps)) return fail(GBN_ERR_ARGS, "eps must be positive");
  std::unique_ptr<gbn_plan_s> p(new gbn_plan_s());
  if (opts_in)
    p->opts = *opts_in;
  else
    gbn_default_opts(&p->opts);
  p->type = type;
  p->dim = dim;
  p->iflag = iflag >= 0 ? 1 : -1;
  p->ntransf = ntransf;
  p->data_single = data_single;
  p->eps = eps;
  p->stream = (cudaStream_t)stream;
  GBN_CUDA(cudaGetDevice(&p->device));
  GBN_CUDA(wait_flag_setup());
  GBN_TRY(resolve_precision(p.get()));
  p->sigma = p->opts.upsampfac > 0.0 ? p->opts.upsampfac : 2.0;
  if (!(p->sigma > 1.0)) return fail(GBN_ERR_ARGS, "upsampfac must be > 1");
  if (p->opts.modeord != 0 && p->opts.modeord != 1)
    return fail(GBN_ERR_ARGS, "modeord must be 0 or 1");
  p->sorted = p->opts.gpu_sort != 0;
  int warn = 0;
  double e = eps;
  if (p->comp_single && e < 1e-7) {
    e = 1e-7;
    warn = 1;
  }
  if (p->opts.gpu_kernel != 0 && p->opts.gpu_kernel != 1)
    return fail(GBN_ERR_ARGS, "gpu_kernel must be 0 (exponential of semicircle) or 1 (Kaiser-Bessel)");
  warn |= kernel_params(e, p->sigma, p->opts.gpu_kernel, &p->w, &p->beta);
  p->warn = warn;
  p->deg = p->w + 2;
  if (type != 3) {
    for (int d = 0; d < 3; ++d) {
      p->N[d] = d < dim ? nmodes[d] : 1;
      if (p->N[d] < 1) return fail(GBN_ERR_ARGS, "number of modes must be >= 1");
      p->nf[d] = d < dim ? fine_size(p->N[d], p->sigma, p->w) : 1;
    }
    p->nftot = p->nf[0] * p->nf[1] * p->nf[2];
    p->Ntot = p->N[0] * p->N[1] * p->N[2];
    if (p->nftot > (int64_t)INT32_MAX) return fail(GBN_ERR_ARGS, "fine grid too large (> 2^31 cells)");
    setup_geom(p.get());
    GBN_TRY(setup_phi(p.get()));
    GBN_TRY(setup_fft_own(p.get()));
  }
  GBN_TRY(setup_kernel_coef(p.get()));
  // transforms per batch: bounded so the fine grids stay within 8 GiB
  int b = p->opts.gpu_maxbatchsize > 0 ? p->opts.gpu_maxbatchsize : ntransf;
  if (b > ntransf) b = ntransf;
  if (type != 3 && p->opts.gpu_maxbatchsize <= 0) {
    const double grid_bytes = (double)p->nftot * cplx_size(p->comp_single);
    const int cap = (int)std::max(1.0, std::floor(8.0 * (1 << 30) / grid_bytes));
    if (b > cap) b = cap;
  }
  p->batch = b;
  p->ev_ok = p->opts.debug != 0;
  *out = p.release();
  return warn ? GBN_WARN_EPS_TOO_SMALL : GBN_OK;
}

// Next n events of a pool (created on demand); null once the pool is full.
cudaEvent_t* take_events(std::vector<cudaEvent_t>& pool, size_t& used, size_t n) {
  constexpr size_t kMaxEvents = 1 << 14;
  if (used + n > kMaxEvents) return nullptr;
  while (pool.size() < used + n) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    pool.push_back(e);
  }
  cudaEvent_t* r = pool.data() + used;
  used += n;
  return r;
}

void fill_sort_state(gbn_points_s& ps, bool sorted) {
  SortState& st = ps.st;
  st.pt_bin = ps.pt_bin.as<int>();
  st.pt_rank = ps.pt_rank.as<int>();
  st.bin_count = sorted ? ps.bin_count.as<int>() : nullptr;
  st.bin_start = ps.bin_start.as<int>();
  st.key_count = !sorted ? nullptr : ps.rows > 1 ? ps.key_count.as<int>() : st.bin_count;
  st.key_start = ps.rows > 1 ? ps.key_start.as<int>() : st.bin_start;
  st.perm = sorted ? ps.perm.as<int>() : nullptr;
  st.sub_count = ps.sub_count.as<int>();
  st.sub_start = ps.sub_start.as<int>();
  st.sub_bin = ps.sub_bin.as<int>();
  st.sub_off = ps.sub_off.as<int>();
  st.n_sub = ps.n_sub.as<int>();
  st.recs = ps.recs.p;
  st.recs_in = ps.recs_in.p;
  st.scan_tmp = ps.scan_tmp.as<int>();
}

// Fold + sort M points (coordinate type TX) onto the plan's geometry into ps.
template <typename TX>
int sort_points(gbn_plan_s* p, gbn_points_s& ps, int64_t M, const TX* x, const TX* y,
                const TX* z, const FoldSpec& fs) {
  if (M < 0) return fail(GBN_ERR_ARGS, "number of points must be >= 0");
  if (M > (int64_t)INT32_MAX) return fail(GBN_ERR_ARGS, "too many points (> 2^31)");
  if (M > 0 && (!x || (p->dim > 1 && !y) || (p->dim > 2 && !z)))
    return fail(GBN_ERR_ARGS, "missing coordinate array");
  cudaStream_t s = p->stream;
  ps.stream = s;
  const Geom& g = p->geom;
  const size_t rs = rec_size(p->dim, p->comp_single);
  const size_t m = (size_t)std::max<int64_t>(M, 1);
  GBN_CUDA(ps.recs_in.ensure(m * rs, s));
  GBN_CUDA(ps.pt_bin.ensure(m * 4, s));
  GBN_CUDA(ps.pt_rank.ensure(m * 4, s));
  ps.rows = g.rows > 1 ? g.rows : 1;
  const int64_t nkeys = g.nbins * ps.rows;
  if (p->sorted) {
    const int64_t nb = g.nbins;
    ps.st.max_sub = nb + (M + g.maxsub - 1) / g.maxsub;
    if (ps.rows > 1) {
      GBN_CUDA(ps.key_count.ensure((size_t)nkeys * 4, s));
      GBN_CUDA(ps.key_start.ensure((size_t)nkeys * 4, s));
    }
    GBN_CUDA(ps.recs.ensure(m * rs, s));
    GBN_CUDA(ps.perm.ensure(m * 4, s));
    GBN_CUDA(ps.bin_count.ensure((size_t)nb * 4, s));
    GBN_CUDA(ps.bin_start.ensure((size_t)nb * 4, s));
    GBN_CUDA(ps.sub_count.ensure((size_t)nb * 4, s));
    GBN_CUDA(ps.sub_start.ensure((size_t)nb * 4, s));
    GBN_CUDA(ps.sub_bin.ensure((size_t)ps.st.max_sub * 4, s));
    GBN_CUDA(ps.sub_off.ensure((size_t)ps.st.max_sub * 4, s));
    GBN_CUDA(ps.n_sub.ensure(4, s));
    GBN_CUDA(ps.scan_tmp.ensure((size_t)scan_tmp_ints(nkeys) * 4, s));
  }
  fill_sort_state(ps, p->sorted);
  if (p->sorted) GBN_CUDA(cudaMemsetAsync(ps.st.key_count, 0, (size_t)nkeys * 4, s));
  if (p->comp_single) {
    GBN_CUDA((launch_fold<TX, float>(g, fs, M, x, y, z, ps.st, s)));
    GBN_CUDA(launch_sort_finish<float>(g, M, ps.st, p->sorted, s));
  } else {
    if (std::is_same<TX, float>::value)
      return fail(GBN_ERR_ARGS, "FP64 compute with float32 points is not supported");
    GBN_CUDA((launch_fold<double, double>(g, fs, M, (const double*)x, (const double*)y,
                                          (const double*)z, ps.st, s)));
    GBN_CUDA(launch_sort_finish<double>(g, M, ps.st, p->sorted, s));
  }
  ps.M = M;
  ps.set = true;
  ps.dim = p->dim;
  ps.comp_single = p->comp_single;
  ps.w = p->w;
  for (int d = 0; d < 3; ++d) ps.nf[d] = p->nf[d];
  return GBN_OK;
}

// A point set is usable with a plan when it was sorted for the same geometry.
bool points_match(const gbn_plan_s* p, const gbn_points_s& ps) {
  if (!ps.set || ps.dim != p->dim || ps.comp_single != p->comp_single || ps.w != p->w)
    return false;
  for (int d = 0; d < 3; ++d)
    if (ps.nf[d] != p->nf[d]) return false;
  return true;
}

int execute_ntr(gbn_plan_s* p, gbn_points_s& ps, void* c, void* f, int ntr, int dir);

template <typename TX>
int plan_setpts(gbn_plan_s* p, int64_t M, const TX* x, const TX* y, const TX* z, int64_t N,
                const TX* s, const TX* t, const TX* u) {
  cudaStream_t st = p->stream;
  cudaEvent_t* sev = p->ev_ok ? take_events(p->ev_setpts, p->ev_setpts_used, 2) : nullptr;
  if (sev) GBN_CUDA(cudaEventRecord(sev[0], st));
  if (p->type != 3) {
    FoldSpec fs{};
    fs.mode = 0;
    GBN_TRY(sort_points<TX>(p, p->own, M, x, y, z, fs));
  } else {
    if (N < 0) return fail(GBN_ERR_ARGS, "number of targets must be >= 0");
    if (N > (int64_t)INT32_MAX) return fail(GBN_ERR_ARGS, "too many targets (> 2^31)");
    const TX* xs[3] = {x, y, z};
    const TX* ss[3] = {s, t, u};
    for (int d = 0; d < p->dim; ++d)
      if ((M > 0 && !xs[d]) || (N > 0 && !ss[d])) return fail(GBN_ERR_ARGS, "missing coordinate array");
    // extents of sources and targets: declared (gbn_set_t3_extents; checked
    // on the device, no host round trip) or measured (one host round trip)
    double h[12] = {};
    if (p->t3_ext) {
      for (int d = 0; d < p->dim; ++d) {
        h[2 * d] = p->t3_ext_v[0][d];
        h[2 * d + 1] = p->t3_ext_v[1][d];
        h[2 * (p->dim + d)] = p->t3_ext_v[2][d];
        h[2 * (p->dim + d) + 1] = p->t3_ext_v[3][d];
      }
      unsigned* flag = extent_flag_device();
      GBN_CUDA(launch_extent_check<TX>(p->dim, M, xs, p->t3_ext_v[0], p->t3_ext_v[1], flag, st));
      GBN_CUDA(launch_extent_check<TX>(p->dim, N, ss, p->t3_ext_v[2], p->t3_ext_v[3], flag, st));
    } else {
      GBN_CUDA(p->t3_minmax.ensure(sizeof(double) * 12, st));
      const TX* arrs[6];
      for (int d = 0; d < p->dim; ++d) {
        arrs[d] = xs[d];
        arrs[p->dim + d] = ss[d];
      }
      double* mm = p->t3_minmax.as<double>();
      GBN_CUDA(launch_minmax<TX>(arrs, p->dim, M, mm, st));
      GBN_CUDA(launch_minmax<TX>(arrs + p->dim, p->dim, N, mm + 2 * p->dim, st));
      GBN_CUDA(cudaMemcpyAsync(h, mm, sizeof(double) * 4 * p->dim, cudaMemcpyDeviceToHost, st));
      GBN_CUDA(cudaStreamSynchronize(st));
    }
    const bool have_x = M > 0 || p->t3_ext, have_s = N > 0 || p->t3_ext;
    int64_t nmodes_inner[3] = {1, 1, 1};
    for (int d = 0; d < p->dim; ++d) {
      const double xmin = have_x ? h[2 * d] : 0.0, xmax = have_x ? h[2 * d + 1] : 0.0;
      const double smin = have_s ? h[2 * (p->dim + d)] : 0.0;
      const double smax = have_s ? h[2 * (p->dim + d) + 1] : 0.0;
      p->nf[d] = type3_params(xmin, xmax, smin, smax, p->sigma, p->w, &p->t3_cx[d],
                              &p->t3_cs[d], &p->t3_scale[d]);
      nmodes_inner[d] = p->nf[d];
    }
    for (int d = p->dim; d < 3; ++d) p->nf[d] = 1;
    // bound on |tau| = |s - cs| / scale over the targets (for the psihat fit)
    double tau_max = 0.0;
    for (int d = 0; d < p->dim && have_s; ++d) {
      const double smin = h[2 * (p->dim + d)], smax = h[2 * (p->dim + d) + 1];
      const double r = std::max(std::fabs(smin - p->t3_cs[d]), std::fabs(smax - p->t3_cs[d]));
      tau_max = std::max(tau_max, r / p->t3_scale[d]);
    }
    tau_max = tau_max * (1.0 + 1e-9) + 1e-300;
    p->nftot = p->nf[0] * p->nf[1] * p->nf[2];
    if (p->nftot > (int64_t)INT32_MAX) return fail(GBN_ERR_ARGS, "type-3 grid too large (> 2^31 cells)");
    p->Nt = N;
    setup_geom(p);
    // inner type-2 plan on the spreading grid, in the compute precision
    bool remake = !p->inner;
    if (p->inner)
      for (int d = 0; d < p->dim; ++d)
        if (p->inner->N[d] != nmodes_inner[d]) remake = true;
    if (remake) {
      p->inner.reset();
      gbn_opts io = p->opts;
      io.modeord = 0;
      io.gpu_precision = 0;
      io.debug = 0;
      io.gpu_maxbatchsize = p->batch;
      if (p->comp_single && p->sigma == 2.0)
        io.upsampfac = inner_sigma_pow2(p->dim, nmodes_inner, std::max(p->eps, 1e-7),
                                        p->opts.gpu_kernel);
      gbn_plan_s* ip = nullptr;
      int r = plan_create(2, p->dim, nmodes_inner, p->iflag, p->batch, p->eps, p->comp_single,
                          &io, (void*)st, &ip);
      if (r >= 2) return r;
      p->inner.reset(ip);
    }
    // targets -> inner type-2 points (FP64)
    double* taus[3] = {nullptr, nullptr, nullptr};
    for (int d = 0; d < p->dim; ++d) {
      GBN_CUDA(p->t3_tau[d].ensure((size_t)std::max<int64_t>(N, 1) * 8, st));
      taus[d] = p->t3_tau[d].as<double>();
    }
    GBN_CUDA(launch_t3_targets<TX>(p->dim, N, ss, p->t3_cs, p->t3_scale, taus, st));
    {
      FoldSpec fs{};
      fs.mode = 0;
      GBN_TRY(sort_points<double>(p->inner.get(), p->inner->own, N, taus[0], taus[1], taus[2], fs));
    }
    // sources -> spreading grid
    {
      FoldSpec fs{};
      fs.mode = 1;
      for (int d = 0; d < 3; ++d) {
        fs.center[d] = p->t3_cx[d];
        fs.scale[d] = p->t3_scale[d];
      }
      GBN_TRY(sort_points<TX>(p, p->own, M, x, y, z, fs));
    }
    const size_t cs = cplx_size(p->comp_single);
    GBN_CUDA(p->t3_pre.ensure((size_t)std::max<int64_t>(M, 1) * cs, st));
    GBN_CUDA(p->t3_post.ensure((size_t)std::max<int64_t>(N, 1) * cs, st));
    const double* ctaus[3] = {taus[0], taus[1], taus[2]};
    if (p->comp_single) {
      GBN_CUDA((launch_t3_prephase_factors<TX, float>(p->dim, M, xs, p->t3_cx, p->t3_cs,
                                                       p->iflag, p->t3_pre.p, st)));
      GBN_CUDA((launch_t3_post_factors<TX, float>(p->dim, N, ss, p->t3_cx, ctaus, p->iflag,
                                                   p->w, p->beta, p->opts.gpu_kernel,
                                                   p->t3_post.p, st, tau_max,
                                                   &p->t3_tab)));
    } else {
      GBN_CUDA((launch_t3_prephase_factors<double, double>(p->dim, M, (const double* const*)xs,
                                                           p->t3_cx, p->t3_cs, p->iflag,
                                                           p->t3_pre.p, st)));
      GBN_CUDA((launch_t3_post_factors<double, double>(p->dim, N, (const double* const*)ss,
                                                       p->t3_cx, ctaus, p->iflag, p->w,
                                                       p->beta, p->opts.gpu_kernel,
                                                       p->t3_post.p, st, tau_max,
                                                       &p->t3_tab)));
    }
  }
  if (sev) GBN_CUDA(cudaEventRecord(sev[1], st));
  return GBN_OK;
}

template <typename TC>
KerSpec<TC> ker_spec(gbn_plan_s* p) {
  KerSpec<TC> ks;
  ks.coef = p->coef.as<TC>();
  ks.deg = p->deg;
  ks.meth = p->opts.gpu_kerevalmeth != 0 ? 1 : 0;
  ks.beta = (TC)p->beta;
  ks.shape = p->opts.gpu_kernel;
  ks.inv_i0b = (TC)(1.0 / bessel_i0(p->beta));
  return ks;
}

// TMA map of nb FP32 grids for the shared-memory point kernels (null when
// not applicable; GBN_DISABLE_TMA=1 selects the per-cell tile loops).
const CUtensorMap* grid_map(const gbn_plan_s* p, const gbn_points_s& ps, const void* grid,
                            int nb, CUtensorMap* storage) {
  if (!p->comp_single || p->method != 2 || !ps.st.perm) return nullptr;
  const char* off = std::getenv("GBN_DISABLE_TMA");
  if (off && off[0] == '1') return nullptr;
  return tile_tensor_map(p->geom, grid, nb, storage) ? storage : nullptr;
}

int do_spread(gbn_plan_s* p, gbn_points_s& ps, const void* c, int nb, bool c_is_compute,
              void* grid) {
  const Geom& g = p->geom;
  cudaError_t e;
  if (p->comp_single) {
    CUtensorMap map;
    const CUtensorMap* tm = grid_map(p, ps, grid, nb, &map);
    if (p->data_single || c_is_compute)
      e = launch_spread<float, float>(g, ker_spec<float>(p), p->method, ps.M, ps.st, c, grid, nb,
                                      p->stream, tm);
    else
      e = launch_spread<float, double>(g, ker_spec<float>(p), p->method, ps.M, ps.st, c, grid,
                                       nb, p->stream, tm);
  } else {
    e = launch_spread<double, double>(g, ker_spec<double>(p), p->method, ps.M, ps.st, c, grid,
                                      nb, p->stream);
  }
  GBN_CUDA(e);
  return GBN_OK;
}

int do_interp(gbn_plan_s* p, gbn_points_s& ps, void* c, int nb, const void* grid) {
  const Geom& g = p->geom;
  cudaError_t e;
  if (p->comp_single) {
    CUtensorMap map;
    const CUtensorMap* tm = grid_map(p, ps, grid, nb, &map);
    if (p->data_single)
      e = launch_interp<float, float>(g, ker_spec<float>(p), p->method, ps.M, ps.st, grid, c, nb,
                                      p->stream, tm);
    else
      e = launch_interp<float, double>(g, ker_spec<float>(p), p->method, ps.M, ps.st, grid, c,
                                       nb, p->stream, tm);
  } else {
    e = launch_interp<double, double>(g, ker_spec<double>(p), p->method, ps.M, ps.st, grid, c,
                                      nb, p->stream);
  }
  GBN_CUDA(e);
  return GBN_OK;
}

int do_deconv(gbn_plan_s* p, void* modes, int nb, bool to_modes, void* grid) {
  cudaError_t e;
  if (p->comp_single) {
    const float* phi[3] = {p->phi[0].as<float>(), p->phi[1].as<float>(), p->phi[2].as<float>()};
    if (p->data_single)
      e = to_modes ? launch_deconv1<float, float>(p->dim, p->N, p->nf, p->opts.modeord, phi,
                                                  grid, modes, nb, p->stream)
                   : launch_deconv2<float, float>(p->dim, p->N, p->nf, p->opts.modeord, phi,
                                                  modes, grid, nb, p->stream);
    else
      e = to_modes ? launch_deconv1<float, double>(p->dim, p->N, p->nf, p->opts.modeord, phi,
                                                   grid, modes, nb, p->stream)
                   : launch_deconv2<float, double>(p->dim, p->N, p->nf, p->opts.modeord, phi,
                                                   modes, grid, nb, p->stream);
  } else {
    const double* phi[3] = {p->phi[0].as<double>(), p->phi[1].as<double>(),
                            p->phi[2].as<double>()};
    e = to_modes ? launch_deconv1<double, double>(p->dim, p->N, p->nf, p->opts.modeord, phi,
                                                  grid, modes, nb, p->stream)
                 : launch_deconv2<double, double>(p->dim, p->N, p->nf, p->opts.modeord, phi,
                                                  modes, grid, nb, p->stream);
  }
  GBN_CUDA(e);
  return GBN_OK;
}

// The library's pruned FFT between the fine grids and the modes (to_modes:
// type-1 direction, grid -> modes; else modes -> grid), deconvolution fused.
int own_fft(gbn_plan_s* p, void* grid, void* modes, int nb, int sign, bool to_modes) {
  const float* phi[3] = {p->phi[0].as<float>(), p->phi[1].as<float>(), p->phi[2].as<float>()};
  const float2* tw[3] = {p->fft_tw[0].as<float2>(), p->fft_tw[1].as<float2>(),
                         p->fft_tw[2].as<float2>()};
  cudaError_t e;
  if (to_modes)
    e = p->data_single ? launch_fft_type1<float>(p->dim, p->N, p->nf, p->opts.modeord, phi, tw,
                                                 grid, modes, nb, sign, p->stream)
                       : launch_fft_type1<double>(p->dim, p->N, p->nf, p->opts.modeord, phi, tw,
                                                  grid, modes, nb, sign, p->stream);
  else
    e = p->data_single ? launch_fft_type2<float>(p->dim, p->N, p->nf, p->opts.modeord, phi, tw,
                                                 modes, grid, nb, sign, p->stream)
                       : launch_fft_type2<double>(p->dim, p->N, p->nf, p->opts.modeord, phi, tw,
                                                  modes, grid, nb, sign, p->stream);
  GBN_CUDA(e);
  return GBN_OK;
}

void ev_record(cudaEvent_t* ev, int i, cudaStream_t s) {
  if (ev) cudaEventRecord(ev[i], s);
}

// Execute ntr transforms on point set ps.  dir = +1 runs the plan's own
// transform; dir = -1 its adjoint with the opposite exponent sign (a type-1
// plan maps modes f to strengths c like a type-2 transform, a type-2 plan
// maps c to f like a type-1 transform), reusing the same sort.
// Adjoint of a type-3 plan on its current points: the cotangents f (ntr, N
// targets) to c (ntr, M sources); with grad the outer gather also
// differentiates along the sources (interp_t3grad_kernel).
int t3_adjoint(gbn_plan_s* p, void* c, const void* f, int ntr, const T3Grad* grad);

int execute_ntr(gbn_plan_s* p, gbn_points_s& ps, void* c, void* f, int ntr, int dir) {
  if (!ps.set) return fail(GBN_ERR_STATE, "execute called before setpts");
  if (p->type != 3 && !points_match(p, ps))
    return fail(GBN_ERR_ARGS, "point set was sorted for a different plan geometry");
  if (p->type == 3 && dir != 1) return t3_adjoint(p, c, f, ntr, nullptr);
  cudaStream_t s = p->stream;
  const size_t dsz = cplx_size(p->data_single);
  const size_t csz = cplx_size(p->comp_single);
  const int op = dir > 0 ? p->type : (p->type == 1 ? 2 : 1);
  const char* no_own = std::getenv("GBN_DISABLE_OWN_FFT");
  const bool own = p->fft_own && !(no_own && no_own[0] == '1');
  const int sign = dir > 0 ? p->iflag : -p->iflag;
  GBN_CUDA(p->fine.ensure((size_t)p->batch * p->nftot * csz, s));
  for (int t0 = 0; t0 < ntr; t0 += p->batch) {
    const int nb = std::min(p->batch, ntr - t0);
    cudaEvent_t* ev = p->ev_ok ? take_events(p->ev_exec, p->ev_exec_used, 4) : nullptr;
    if (op == 1) {
      const char* cb = (const char*)c + (size_t)t0 * ps.M * dsz;
      char* fb = (char*)f + (size_t)t0 * p->Ntot * dsz;
      ev_record(ev, 0, s);
      GBN_CUDA(cudaMemsetAsync(p->fine.p, 0, (size_t)nb * p->nftot * csz, s));
      GBN_TRY(do_spread(p, ps, cb, nb, false, p->fine.p));
      ev_record(ev, 1, s);
      if (own) {  // pruned FFT with the deconvolution fused (deconv stage empty)
        GBN_TRY(own_fft(p, p->fine.p, fb, nb, sign, true));
        ev_record(ev, 2, s);
      } else {
        GBN_TRY(exec_fft(p, p->fine.p, nb, sign, 2));
        ev_record(ev, 2, s);
        GBN_TRY(do_deconv(p, fb, nb, true, p->fine.p));
      }
      ev_record(ev, 3, s);
    } else if (op == 2) {
      char* cb = (char*)c + (size_t)t0 * ps.M * dsz;
      const char* fb = (const char*)f + (size_t)t0 * p->Ntot * dsz;
      ev_record(ev, 0, s);
      if (own) {  // pruned FFT with the deconvolution fused (deconv stage empty)
        ev_record(ev, 1, s);
        GBN_TRY(own_fft(p, p->fine.p, (void*)fb, nb, sign, false));
      } else {
        GBN_TRY(do_deconv(p, (void*)fb, nb, false, p->fine.p));
        ev_record(ev, 1, s);
        GBN_TRY(exec_fft(p, p->fine.p, nb, sign, 1));
      }
      ev_record(ev, 2, s);
      GBN_TRY(do_interp(p, ps, cb, nb, p->fine.p));
      ev_record(ev, 3, s);
    } else {
      const char* cb = (const char*)c + (size_t)t0 * ps.M * dsz;
      char* fb = (char*)f + (size_t)t0 * p->Nt * dsz;
      GBN_CUDA(p->t3_cbuf.ensure((size_t)p->batch * std::max<int64_t>(ps.M, 1) * csz, s));
      GBN_CUDA(p->t3_obuf.ensure((size_t)p->batch * std::max<int64_t>(p->Nt, 1) * csz, s));
      ev_record(ev, 0, s);
      cudaError_t e;
      if (p->comp_single)
        e = p->data_single ? launch_cmul<float, float, float>(ps.M, nb, cb, p->t3_pre.p,
                                                              p->t3_cbuf.p, s)
                           : launch_cmul<double, float, float>(ps.M, nb, cb, p->t3_pre.p,
                                                               p->t3_cbuf.p, s);
      else
        e = launch_cmul<double, double, double>(ps.M, nb, cb, p->t3_pre.p, p->t3_cbuf.p, s);
      GBN_CUDA(e);
      GBN_CUDA(cudaMemsetAsync(p->fine.p, 0, (size_t)nb * p->nftot * csz, s));
      GBN_TRY(do_spread(p, ps, p->t3_cbuf.p, nb, true, p->fine.p));
      ev_record(ev, 1, s);
      // inner type 2: modes = spread grid (CMCL order), points = rescaled targets
      GBN_TRY(execute_ntr(p->inner.get(), p->inner->own, p->t3_obuf.p, p->fine.p, nb, 1));
      ev_record(ev, 2, s);
      if (p->comp_single)
        e = p->data_single ? launch_cmul<float, float, float>(p->Nt, nb, p->t3_obuf.p,
                                                              p->t3_post.p, fb, s)
                           : launch_cmul<float, double, float>(p->Nt, nb, p->t3_obuf.p,
                                                               p->t3_post.p, fb, s);
      else
        e = launch_cmul<double, double, double>(p->Nt, nb, p->t3_obuf.p, p->t3_post.p, fb, s);
      GBN_CUDA(e);
      ev_record(ev, 3, s);
    }
  }
  GBN_CUDA(cudaGetLastError());
  return GBN_OK;
}

int t3_adjoint(gbn_plan_s* p, void* c, const void* f, int ntr, const T3Grad* grad) {
  gbn_points_s& ps = p->own;
  if (!ps.set) return fail(GBN_ERR_STATE, "adjoint called before setpts");
  if (ntr < 1) return fail(GBN_ERR_ARGS, "ntr must be >= 1");
  cudaStream_t s = p->stream;
  const size_t dsz = cplx_size(p->data_single), csz = cplx_size(p->comp_single);
  GBN_CUDA(p->fine.ensure((size_t)p->batch * p->nftot * csz, s));
  GBN_CUDA(p->t3_obuf.ensure((size_t)p->batch * std::max<int64_t>(p->Nt, 1) * csz, s));
  if (!grad)
    GBN_CUDA(p->t3_cbuf.ensure((size_t)p->batch * std::max<int64_t>(ps.M, 1) * csz, s));
  for (int t0 = 0; t0 < ntr; t0 += p->batch) {
    const int nb = std::min(p->batch, ntr - t0);
    const char* fb = (const char*)f + (size_t)t0 * p->Nt * dsz;
    // cotangents times conj(post): the adjoint of the post-phase/deconvolution
    cudaError_t e;
    if (p->comp_single)
      e = p->data_single
              ? launch_cmul<float, float, float>(p->Nt, nb, fb, p->t3_post.p, p->t3_obuf.p, s, true)
              : launch_cmul<double, float, float>(p->Nt, nb, fb, p->t3_post.p, p->t3_obuf.p, s,
                                                  true);
    else
      e = launch_cmul<double, double, double>(p->Nt, nb, fb, p->t3_post.p, p->t3_obuf.p, s, true);
    GBN_CUDA(e);
    // the inner type 2's adjoint (a type 1 on the rescaled targets) onto the
    // spreading grid, on the forward's sorted targets
    GBN_TRY(execute_ntr(p->inner.get(), p->inner->own, p->t3_obuf.p, p->fine.p, nb, -1));
    CUtensorMap map;
    const CUtensorMap* tm = grid_map(p, ps, p->fine.p, nb, &map);
    if (grad) {  // gather the strength and source gradients on the forward's sort
      T3Grad tg = *grad;
      tg.t0 = t0;
      if (p->comp_single)
        e = p->data_single ? launch_interp_t3grad<float, float>(p->geom, ker_spec<float>(p),
                                                               ps.M, ps.st, p->fine.p, nb, tg, s,
                                                               tm)
                           : launch_interp_t3grad<float, double>(p->geom, ker_spec<float>(p),
                                                                ps.M, ps.st, p->fine.p, nb, tg,
                                                                s, tm);
      else
        e = launch_interp_t3grad<double, double>(p->geom, ker_spec<double>(p), ps.M, ps.st,
                                                 p->fine.p, nb, tg, s);
      GBN_CUDA(e);
      continue;
    }
    // gather on the sources, then times conj(pre)
    char* cb = (char*)c + (size_t)t0 * ps.M * dsz;
    if (p->comp_single) {
      GBN_CUDA((launch_interp<float, float>(p->geom, ker_spec<float>(p), p->method, ps.M, ps.st,
                                            p->fine.p, p->t3_cbuf.p, nb, s, tm)));
      e = p->data_single
              ? launch_cmul<float, float, float>(ps.M, nb, p->t3_cbuf.p, p->t3_pre.p, cb, s, true)
              : launch_cmul<float, double, float>(ps.M, nb, p->t3_cbuf.p, p->t3_pre.p, cb, s,
                                                  true);
    } else {
      GBN_CUDA((launch_interp<double, double>(p->geom, ker_spec<double>(p), p->method, ps.M,
                                              ps.st, p->fine.p, p->t3_cbuf.p, nb, s)));
      e = launch_cmul<double, double, double>(ps.M, nb, p->t3_cbuf.p, p->t3_pre.p, cb, s, true);
    }
    GBN_CUDA(e);
  }
  GBN_CUDA(cudaGetLastError());
  return GBN_OK;
}

// Type-3 gradients on the plan's current points (see gbn_grad): one adjoint
// pass of the ntr cotangents whose outer gather also differentiates along
// the sources.
int t3_grad(gbn_plan_s* p, int ntr, const void* src, const void* g, void* grad_src,
            void* const* gx) {
  const size_t rsz = p->data_single ? 4 : 8;
  T3Grad tg{};
  bool any = false;
  for (int d = 0; d < p->dim; ++d) {
    tg.gx[d] = gx ? gx[d] : nullptr;
    if (tg.gx[d]) {
      any = true;
      if (p->own.M > 0) GBN_CUDA(cudaMemsetAsync(tg.gx[d], 0, (size_t)p->own.M * rsz, p->stream));
    }
    tg.D[d] = p->t3_cs[d];
    tg.scale[d] = p->t3_scale[d];
  }
  if (!any && !grad_src) return GBN_OK;
  tg.c = any ? src : nullptr;
  tg.pre = p->t3_pre.p;
  tg.grad_c = grad_src;
  tg.iflag = p->iflag;
  if (p->own.M == 0) return GBN_OK;
  return t3_adjoint(p, grad_src, g, ntr, &tg);
}

// Gradients of a type-1 or type-2 plan on point set ps (see gbn_grad).
int plan_grad(gbn_plan_s* p, gbn_points_s& ps, int ntr, const void* src, const void* g,
              void* grad_src, void* const* gx) {
  if (p->type == 3) return fail(GBN_ERR_ARGS, "gbn_grad supports type-1 and type-2 plans");
  if (!points_match(p, ps)) return fail(GBN_ERR_ARGS, "point set does not match the plan");
  if (ntr < 1) return fail(GBN_ERR_ARGS, "ntr must be >= 1");
  cudaStream_t s = p->stream;
  const size_t csz = cplx_size(p->comp_single), dsz = cplx_size(p->data_single);
  const size_t rsz = p->data_single ? 4 : 8;
  int req[3], nd = 0;
  for (int d = 0; d < p->dim; ++d)
    if (gx && gx[d]) req[nd++] = d;
  void* gxx[3] = {nullptr, nullptr, nullptr};
  for (int d = 0; d < p->dim; ++d) {
    gxx[d] = gx ? gx[d] : nullptr;
    if (gxx[d] && ps.M > 0) GBN_CUDA(cudaMemsetAsync(gxx[d], 0, (size_t)ps.M * rsz, s));
  }
  if (p->type == 2 && grad_src) GBN_TRY(execute_ntr(p, ps, (void*)g, grad_src, ntr, -1));
  const int base = (p->type == 1 && grad_src) ? 1 : 0;
  const int E = base + nd;
  if (E == 0 || ps.M == 0) return GBN_OK;
  int dims[4] = {0, 0, 0, 0};
  for (int e = base; e < E; ++e) dims[e] = req[e - base];
  const double grid_bytes = (double)p->nftot * csz * E;
  int nbmax = (int)std::max(1.0, std::floor(8.0 * (1 << 30) / grid_bytes));
  if (nbmax > ntr) nbmax = ntr;
  GBN_CUDA(p->gfine.ensure((size_t)nbmax * E * p->nftot * csz, s));
  const int mode = p->type == 1 ? 0 : 1;
  const int sign = p->type == 1 ? -p->iflag : p->iflag;
  const double a_re = p->type == 1 ? 1.0 : 0.0, a_im = p->type == 1 ? 0.0 : (double)p->iflag;
  // modes that feed the grids: the cotangent (type 1) or the forward modes (type 2)
  const char* modes = (const char*)(p->type == 1 ? g : src);
  const char* wsrc = (const char*)(p->type == 1 ? src : g);
  for (int t0 = 0; t0 < ntr; t0 += nbmax) {
    const int nb = std::min(nbmax, ntr - t0);
    const void* min = modes + (size_t)t0 * p->Ntot * dsz;
    const void* win = wsrc + (size_t)t0 * ps.M * dsz;
    void* outc = base ? (void*)((char*)grad_src + (size_t)t0 * ps.M * dsz) : nullptr;
    cudaError_t e;
    const char* no_own = std::getenv("GBN_DISABLE_OWN_FFT");
    if (p->fft_own && !(no_own && no_own[0] == '1') &&
        fft_pow2_supported(p->dim, p->nf, nb * E)) {
      // the library's pruned FFT builds the weighted grids in its x pass
      const float* phi[3] = {p->phi[0].as<float>(), p->phi[1].as<float>(), p->phi[2].as<float>()};
      const float2* tw[3] = {p->fft_tw[0].as<float2>(), p->fft_tw[1].as<float2>(),
                             p->fft_tw[2].as<float2>()};
      FftWeights wts{E, base, {dims[0], dims[1], dims[2], dims[3]}, a_re, a_im};
      e = p->data_single
              ? launch_fft_type2<float>(p->dim, p->N, p->nf, p->opts.modeord, phi, tw, min,
                                        p->gfine.p, nb, sign, s, &wts)
              : launch_fft_type2<double>(p->dim, p->N, p->nf, p->opts.modeord, phi, tw, min,
                                         p->gfine.p, nb, sign, s, &wts);
      GBN_CUDA(e);
    } else {
      if (p->comp_single) {
        const float* phi[3] = {p->phi[0].as<float>(), p->phi[1].as<float>(),
                               p->phi[2].as<float>()};
        e = p->data_single
                ? launch_deconv2w<float, float>(p->dim, p->N, p->nf, p->opts.modeord, phi, min,
                                                p->gfine.p, nb, E, base, dims, a_re, a_im, s)
                : launch_deconv2w<float, double>(p->dim, p->N, p->nf, p->opts.modeord, phi, min,
                                                 p->gfine.p, nb, E, base, dims, a_re, a_im, s);
      } else {
        const double* phi[3] = {p->phi[0].as<double>(), p->phi[1].as<double>(),
                                p->phi[2].as<double>()};
        e = launch_deconv2w<double, double>(p->dim, p->N, p->nf, p->opts.modeord, phi, min,
                                            p->gfine.p, nb, E, base, dims, a_re, a_im, s);
      }
      GBN_CUDA(e);
      GBN_TRY(exec_fft(p, p->gfine.p, nb * E, sign, 1));
    }
    if (p->comp_single) {
      CUtensorMap map;
      const CUtensorMap* tm = grid_map(p, ps, p->gfine.p, nb * E, &map);
      e = p->data_single
              ? launch_interp_grad<float, float>(p->geom, ker_spec<float>(p), ps.M, ps.st,
                                                 p->gfine.p, nb, E, mode, p->iflag, base, dims,
                                                 win, outc, gxx, p->method == 2, s, tm)
              : launch_interp_grad<float, double>(p->geom, ker_spec<float>(p), ps.M, ps.st,
                                                  p->gfine.p, nb, E, mode, p->iflag, base, dims,
                                                  win, outc, gxx, p->method == 2, s, tm);
    } else {
      e = launch_interp_grad<double, double>(p->geom, ker_spec<double>(p), ps.M, ps.st,
                                             p->gfine.p, nb, E, mode, p->iflag, base, dims, win,
                                             outc, gxx, p->method == 2, s);
    }
    GBN_CUDA(e);
  }
  GBN_CUDA(cudaGetLastError());
  return GBN_OK;
}

// ---------------------------------------------------------------------------
// plan cache for the one-shot entry points
// ---------------------------------------------------------------------------
struct CacheKey {
  int type, dim, single, iflag, ntransf, device;
  int64_t nk[3];
  double eps;
  gbn_opts opts;
  void* stream;
  bool operator==(const CacheKey& o) const {
    return type == o.type && dim == o.dim && single == o.single && iflag == o.iflag &&
           ntransf == o.ntransf && device == o.device && nk[0] == o.nk[0] && nk[1] == o.nk[1] &&
           nk[2] == o.nk[2] && eps == o.eps && stream == o.stream && opts_equal(opts, o.opts);
  }
  static bool opts_equal(const gbn_opts& a, const gbn_opts& b) {
    return a.modeord == b.modeord && a.upsampfac == b.upsampfac && a.gpu_method == b.gpu_method &&
           a.gpu_sort == b.gpu_sort && a.gpu_kerevalmeth == b.gpu_kerevalmeth &&
           a.gpu_maxbatchsize == b.gpu_maxbatchsize && a.debug == b.debug &&
           a.gpu_binsizex == b.gpu_binsizex && a.gpu_binsizey == b.gpu_binsizey &&
           a.gpu_binsizez == b.gpu_binsizez && a.gpu_maxsubprobsize == b.gpu_maxsubprobsize &&
           a.gpu_precision == b.gpu_precision && a.gpu_kernel == b.gpu_kernel;
  }
};

struct PlanCache {
  std::mutex mu;
  std::list<std::pair<CacheKey, gbn_plan_s*>> idle;  // most recent first
  size_t capacity = 8;

  gbn_plan_s* take(const CacheKey& k) {
    std::lock_guard<std::mutex> lk(mu);
    for (auto it = idle.begin(); it != idle.end(); ++it)
      if (it->first == k) {
        gbn_plan_s* p = it->second;
        idle.erase(it);
        return p;
      }
    return nullptr;
  }
  void give(const CacheKey& k, gbn_plan_s* p) {
    std::vector<gbn_plan_s*> evict;
    {
      std::lock_guard<std::mutex> lk(mu);
      idle.emplace_front(k, p);
      while (idle.size() > capacity) {
        evict.push_back(idle.back().second);
        idle.pop_back();
      }
    }
    for (auto* q : evict) delete q;
  }
  void clear() {
    std::list<std::pair<CacheKey, gbn_plan_s*>> all;
    {
      std::lock_guard<std::mutex> lk(mu);
      all.swap(idle);
    }
    for (auto& kv : all) delete kv.second;
  }
};

PlanCache& cache() {
  static PlanCache* c = new PlanCache();  // never destroyed: no CUDA calls at exit
  return *c;
}

template <typename TX>
int run_oneshot(int type, int dim, bool single, void* stream, double eps, int iflag,
                int64_t n_tot, int64_t n_transf, int64_t n_j, const int64_t* n_k,
                const gbn_opts* opts, const void* source, const TX* const* pts,
                const TX* const* tgts, void* output) {
  if (n_tot < 0 || n_transf < 0 || n_j < 0) return fail(GBN_ERR_ARGS, "negative size");
  if (n_transf > INT32_MAX) return fail(GBN_ERR_ARGS, "n_transf too large");
  if (n_tot == 0 || n_transf == 0) return GBN_OK;
  int64_t nk[3] = {1, 1, 1};
  int64_t n_k_total = 1;
  if (type != 3) {
    for (int d = 0; d < dim; ++d) {
      nk[d] = n_k[d];
      n_k_total *= n_k[d];
    }
  } else {
    n_k_total = n_k[0];
  }
  CacheKey key;
  std::memset(&key, 0, sizeof(key));
  key.type = type;
  key.dim = dim;
  key.single = single;
  key.iflag = iflag >= 0 ? 1 : -1;
  key.ntransf = (int)n_transf;
  GBN_CUDA(cudaGetDevice(&key.device));
  for (int d = 0; d < 3; ++d) key.nk[d] = nk[d];
  key.eps = eps;
  if (opts)
    key.opts = *opts;
  else
    gbn_default_opts(&key.opts);
  key.stream = stream;
  gbn_plan_s* p = cache().take(key);
  int warn = 0;
  if (!p) {
    int r = plan_create(type, dim, nk, iflag, (int)n_transf, eps, single, &key.opts, stream, &p);
    if (r >= 2) return r;
    warn = r;
  } else {
    warn = p->warn;
  }
  const size_t dsz = cplx_size(single);
  // Identical calls (same plan, sizes and buffers) replay a CUDA graph of
  // the previous one: one launch instead of a dozen, the host time of a
  // small transform.  Buffers of a plan only grow for other sizes, so the
  // graph's addresses stay valid while the arguments repeat.  Not while the
  // caller's stream is being captured (the work joins that capture) or with
  // debug timings; never for type 3 (its setpts may read the host).
  gbn_plan_s::OneshotArgs oa{};
  oa.n_tot = n_tot;
  oa.n_j = n_j;
  oa.n_k_total = n_k_total;
  oa.src = source;
  oa.out = output;
  for (int d = 0; d < dim; ++d) oa.pts[d] = pts[d];
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  GBN_CUDA(cudaStreamIsCapturing((cudaStream_t)stream, &cap));
  const bool graphable = type != 3 && !p->ev_ok && !p->os_nograph &&
                         cap == cudaStreamCaptureStatusNone;
  auto eq = [&](const gbn_plan_s::OneshotArgs& o) {
    return std::memcmp(&o, &oa, sizeof(oa)) == 0;
  };
  // other sizes than the kept calls': their graphs and records go first
  if ((!p->os_seen.empty() &&
       (p->os_seen.front().n_j != n_j || p->os_seen.front().n_tot != n_tot)) ||
      (!p->os_graphs.empty() &&
       (p->os_graphs.front().first.n_j != n_j || p->os_graphs.front().first.n_tot != n_tot)))
    p->os_clear();
  if (graphable) {
    for (auto& g : p->os_graphs) {
      if (!eq(g.first)) continue;
      const cudaError_t e = cudaGraphLaunch(g.second, (cudaStream_t)stream);
      if (e != cudaSuccess) {
        delete p;
        return fail(GBN_ERR_CUDA, std::string("CUDA error: ") + cudaGetErrorString(e));
      }
      cache().give(key, p);
      return warn ? GBN_WARN_EPS_TOO_SMALL : GBN_OK;
    }
  }
  bool same = false;  // seen before, not yet a graph
  for (const auto& o : p->os_seen) same = same || eq(o);
  if (!same) {
    if (p->os_seen.size() >= gbn_plan_s::kOneshotKeep) p->os_seen.erase(p->os_seen.begin());
    p->os_seen.push_back(oa);
  }
  // the setpts + execute of every n_tot slice
  auto run_all = [&]() -> int {
    int r = GBN_OK;
    for (int64_t idx = 0; idx < n_tot && r < 2; ++idx) {
      const int64_t i = idx * n_j;
      const int64_t j = idx * n_j * n_transf;
      const int64_t k = idx * n_k_total * n_transf;
      const TX* xs[3] = {nullptr, nullptr, nullptr};
      const TX* ss[3] = {nullptr, nullptr, nullptr};
      for (int d = 0; d < dim; ++d) {
        xs[d] = pts[d] ? pts[d] + i : nullptr;
        if (type == 3) ss[d] = tgts[d] ? tgts[d] + idx * n_k_total : nullptr;
      }
      r = plan_setpts<TX>(p, n_j, xs[0], xs[1], xs[2], type == 3 ? n_k_total : 0, ss[0], ss[1],
                          ss[2]);
      if (r >= 2) break;
      const char* src = (const char*)source;
      char* out = (char*)output;
      if (type == 2)
        r = execute_ntr(p, p->own, out + (size_t)j * dsz, (void*)(src + (size_t)k * dsz),
                        p->ntransf, 1);
      else
        r = execute_ntr(p, p->own, (void*)(src + (size_t)j * dsz), out + (size_t)k * dsz,
                        p->ntransf, 1);
    }
    return r;
  };
  int ret = GBN_OK;
  bool done = false;
  if (graphable && same && !p->os_cap &&
      cudaStreamCreateWithFlags(&p->os_cap, cudaStreamNonBlocking) != cudaSuccess) {
    p->os_cap = nullptr;
    p->os_nograph = true;
    cudaGetLastError();
  }
  if (graphable && same && p->os_cap &&
      cudaStreamBeginCapture(p->os_cap, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    // the second identical call: capture it on the plan's capture stream,
    // then launch the graph on the caller's (the captured work has not run
    // yet); any failure on the way disables graphs for this plan and the
    // call runs directly
    cudaStream_t user = p->stream;
    p->stream = p->os_cap;
    const int r = run_all();
    p->stream = user;
    p->own.stream = user;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t ex = nullptr;
    const cudaError_t e = cudaStreamEndCapture(p->os_cap, &graph);
    const bool made = r < 2 && e == cudaSuccess && graph &&
                      cudaGraphInstantiate(&ex, graph, 0) == cudaSuccess;
    if (made && cudaGraphLaunch(ex, (cudaStream_t)stream) == cudaSuccess) {
      if (p->os_graphs.size() >= gbn_plan_s::kOneshotKeep) {
        cudaGraphExecDestroy(p->os_graphs.front().second);
        p->os_graphs.erase(p->os_graphs.begin());
      }
      p->os_graphs.emplace_back(oa, ex);
      done = true;
    } else {
      if (made) cudaGraphExecDestroy(ex);
      p->os_nograph = true;
      cudaGetLastError();
    }
    if (graph) cudaGraphDestroy(graph);
  }
  if (graphable && same && !done) cudaGetLastError();  // a refused capture's status
  if (!done) ret = run_all();
  if (ret >= 2) {
    delete p;  // state unknown after a failure: do not cache
    return ret;
  }
  cache().give(key, p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(GBN_ERR_CUDA, std::string("CUDA error: ") + cudaGetErrorString(e));
  return warn ? GBN_WARN_EPS_TOO_SMALL : GBN_OK;
}

}  // namespace

// =============================================================================
// C ABI
// =============================================================================
extern "C" {

void gbn_default_opts(gbn_opts* o) {
  std::memset(o, 0, sizeof(*o));
  o->modeord = 0;
  o->upsampfac = 2.0;
  o->gpu_method = 0;
  o->gpu_sort = 1;
  o->gpu_kerevalmeth = 1;
  o->gpu_maxbatchsize = 0;
  o->debug = 0;
  o->gpu_maxsubprobsize = 1024;
  o->gpu_precision = 0;
  o->gpu_kernel = 0;
}

const char* gbn_last_error(void) { return g_err.c_str(); }

int gbn_makeplan(int type, int dim, const int64_t* nmodes, int iflag, int ntransf, double eps,
                 gbn_plan* plan, const gbn_opts* opts, void* stream) {
  if (!plan) return fail(GBN_ERR_ARGS, "plan pointer is NULL");
  if (type != 3 && !nmodes) return fail(GBN_ERR_ARGS, "nmodes is NULL");
  return plan_create(type, dim, nmodes, iflag, ntransf, eps, false, opts, stream, plan);
}

int gbnf_makeplan(int type, int dim, const int64_t* nmodes, int iflag, int ntransf, float eps,
                  gbn_plan* plan, const gbn_opts* opts, void* stream) {
  if (!plan) return fail(GBN_ERR_ARGS, "plan pointer is NULL");
  if (type != 3 && !nmodes) return fail(GBN_ERR_ARGS, "nmodes is NULL");
  return plan_create(type, dim, nmodes, iflag, ntransf, (double)eps, true, opts, stream, plan);
}

int gbn_setpts(gbn_plan plan, int64_t M, const double* x, const double* y, const double* z,
               int64_t N, const double* s, const double* t, const double* u) {
  if (!plan) return fail(GBN_ERR_ARGS, "plan is NULL");
  if (plan->data_single) return fail(GBN_ERR_ARGS, "complex64 plan: use gbnf_setpts");
  return plan_setpts<double>(plan, M, x, y, z, N, s, t, u);
}

int gbnf_setpts(gbn_plan plan, int64_t M, const float* x, const float* y, const float* z,
                int64_t N, const float* s, const float* t, const float* u) {
  if (!plan) return fail(GBN_ERR_ARGS, "plan is NULL");
  if (!plan->data_single) return fail(GBN_ERR_ARGS, "complex128 plan: use gbn_setpts");
  if (!plan->comp_single) return fail(GBN_ERR_ARGS, "FP64 compute needs float64 points");
  return plan_setpts<float>(plan, M, x, y, z, N, s, t, u);
}

int gbn_execute(gbn_plan plan, void* c, void* f) {
  if (!plan) return fail(GBN_ERR_ARGS, "plan is NULL");
  if (int r = check_waits(GBN_OK)) return r;
  return check_waits(execute_ntr(plan, plan->own, c, f, plan->ntransf, 1));
}

int gbn_set_stream(gbn_plan plan, void* stream) {
  if (!plan) return fail(GBN_ERR_ARGS, "plan is NULL");
  plan->stream = (cudaStream_t)stream;
  if (plan->inner) plan->inner->stream = (cudaStream_t)stream;
  return GBN_OK;
}

int gbn_destroy(gbn_plan plan) {
  delete plan;
  return GBN_OK;
}

int gbn_plan_info(gbn_plan plan, int* w, int64_t* nf3, int* method, int* compute_double) {
  if (!plan) return fail(GBN_ERR_ARGS, "plan is NULL");
  if (w) *w = plan->w;
  if (nf3)
    for (int d = 0; d < 3; ++d) nf3[d] = plan->nf[d];
  if (method) *method = plan->method;
  if (compute_double) *compute_double = plan->comp_single ? 0 : 1;
  return GBN_OK;
}

int gbn_get_timings(gbn_plan plan, float* ms5, int* nbatch) {
  if (!plan || !ms5) return fail(GBN_ERR_ARGS, "NULL argument");
  if (!plan->ev_ok) return fail(GBN_ERR_STATE, "plan was made without opts.debug");
  GBN_CUDA(cudaStreamSynchronize(plan->stream));
  double acc[5] = {0, 0, 0, 0, 0};
  for (size_t i = 0; i + 4 <= plan->ev_exec_used; i += 4) {
    float a = 0, b = 0, c = 0;
    cudaEvent_t* e = plan->ev_exec.data() + i;
    GBN_CUDA(cudaEventElapsedTime(&a, e[0], e[1]));
    GBN_CUDA(cudaEventElapsedTime(&b, e[1], e[2]));
    GBN_CUDA(cudaEventElapsedTime(&c, e[2], e[3]));
    if (plan->type == 3) {
      acc[3] += a + c;
      acc[1] += b;
    } else {
      acc[0] += plan->type == 1 ? a : c;
      acc[1] += b;
      acc[2] += plan->type == 1 ? c : a;
    }
  }
  for (size_t i = 0; i + 2 <= plan->ev_setpts_used; i += 2) {
    float a = 0;
    GBN_CUDA(cudaEventElapsedTime(&a, plan->ev_setpts[i], plan->ev_setpts[i + 1]));
    acc[4] += a;
  }
  for (int i = 0; i < 5; ++i) ms5[i] = (float)acc[i];
  if (nbatch) *nbatch = (int)(plan->ev_exec_used / 4);
  plan->ev_exec_used = 0;
  plan->ev_setpts_used = 0;
  return GBN_OK;
}

int gbn_debug_bins(gbn_plan plan, int64_t* bins_out, int64_t* counts_out, int64_t* nbins) {
  if (!plan) return fail(GBN_ERR_ARGS, "plan is NULL");
  if (nbins) *nbins = plan->geom.nbins;
  if (!plan->own.set || !plan->sorted) return fail(GBN_ERR_STATE, "no sorted points");
  GBN_CUDA(cudaStreamSynchronize(plan->stream));
  if (bins_out && plan->own.M > 0) {
    std::vector<int> b((size_t)plan->own.M);
    GBN_CUDA(cudaMemcpy(b.data(), plan->own.pt_bin.p, b.size() * 4, cudaMemcpyDeviceToHost));
    const int rows = plan->own.rows > 1 ? plan->own.rows : 1;  // sort key -> bin
    for (size_t i = 0; i < b.size(); ++i) bins_out[i] = b[i] / rows;
  }
  if (counts_out) {
    std::vector<int> b((size_t)plan->geom.nbins);
    GBN_CUDA(cudaMemcpy(b.data(), plan->own.bin_count.p, b.size() * 4, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < b.size(); ++i) counts_out[i] = b[i];
  }
  return GBN_OK;
}

int gbn_debug_fold(gbn_plan plan, int64_t* i0_out, double* delta_out) {
  if (!plan) return fail(GBN_ERR_ARGS, "plan is NULL");
  if (!plan->own.set) return fail(GBN_ERR_STATE, "no points");
  GBN_CUDA(cudaStreamSynchronize(plan->stream));
  const int dim = plan->dim;
  const size_t rs = rec_size(dim, plan->comp_single);
  std::vector<unsigned char> raw((size_t)plan->own.M * rs);
  if (plan->own.M > 0)
    GBN_CUDA(cudaMemcpy(raw.data(), plan->own.recs_in.p, raw.size(), cudaMemcpyDeviceToHost));
  for (int64_t j = 0; j < plan->own.M; ++j) {
    const unsigned char* r = raw.data() + (size_t)j * rs;
    for (int d = 0; d < 3; ++d) {
      int64_t iv = 0;
      double dv = 0.0;
      if (d < dim) {
        if (plan->comp_single) {
          float f;
          int ii;
          std::memcpy(&f, r + d * 4, 4);
          std::memcpy(&ii, r + dim * 4 + d * 4, 4);
          dv = f;
          iv = ii;
        } else {
          double f;
          int ii;
          std::memcpy(&f, r + d * 8, 8);
          std::memcpy(&ii, r + dim * 8 + d * 4, 4);
          dv = f;
          iv = ii;
        }
      }
      if (i0_out) i0_out[j * 3 + d] = iv;
      if (delta_out) delta_out[j * 3 + d] = dv;
    }
  }
  return GBN_OK;
}

int gbn_points_create(gbn_plan plan, int64_t M, const void* x, const void* y, const void* z,
                      gbn_points* out) {
  if (!plan || !out) return fail(GBN_ERR_ARGS, "NULL argument");
  *out = nullptr;
  if (plan->type == 3) return fail(GBN_ERR_ARGS, "point sets are for type-1 and type-2 plans");
  std::unique_ptr<gbn_points_s> ps(new gbn_points_s());
  FoldSpec fs{};
  fs.mode = 0;
  int r = plan->data_single
              ? sort_points<float>(plan, *ps, M, (const float*)x, (const float*)y,
                                   (const float*)z, fs)
              : sort_points<double>(plan, *ps, M, (const double*)x, (const double*)y,
                                    (const double*)z, fs);
  if (r >= 2) return r;
  *out = ps.release();
  return GBN_OK;
}

int gbn_points_destroy(gbn_points pts) {
  delete pts;
  return GBN_OK;
}

int gbn_execute_points(gbn_plan plan, gbn_points pts, int ntr, int dir, void* c, void* f) {
  if (!plan) return fail(GBN_ERR_ARGS, "NULL plan");
  if ((plan->type == 3) != (pts == nullptr))
    return fail(GBN_ERR_ARGS, "type-3 plans take their own points (pts = NULL); types 1 and 2 "
                              "a point set");
  if (dir != 1 && dir != -1) return fail(GBN_ERR_ARGS, "dir must be +1 or -1");
  if (ntr < 1) return fail(GBN_ERR_ARGS, "ntr must be >= 1");
  if (int r = check_waits(GBN_OK)) return r;
  return check_waits(execute_ntr(plan, pts ? *pts : plan->own, c, f, ntr, dir));
}

int gbn_grad(gbn_plan plan, gbn_points pts, int ntr, const void* src, const void* g,
             void* grad_src, void* const* grad_x) {
  if (!plan || !src || !g) return fail(GBN_ERR_ARGS, "NULL argument");
  if ((plan->type == 3) != (pts == nullptr))
    return fail(GBN_ERR_ARGS, "type-3 plans take their own points (pts = NULL); types 1 and 2 "
                              "a point set");
  if (ntr < 1) return fail(GBN_ERR_ARGS, "ntr must be >= 1");
  if (int r = check_waits(GBN_OK)) return r;
  if (plan->type == 3) return check_waits(t3_grad(plan, ntr, src, g, grad_src, grad_x));
  return check_waits(plan_grad(plan, *pts, ntr, src, g, grad_src, grad_x));
}

void gbn_clear_cache(void) { cache().clear(); }

long long gbn_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

int gbn_set_t3_extents(gbn_plan plan, const double* x_lo, const double* x_hi,
                       const double* s_lo, const double* s_hi) {
  if (!plan) return fail(GBN_ERR_ARGS, "plan is NULL");
  if (plan->type != 3) return fail(GBN_ERR_ARGS, "extents are for type-3 plans");
  if (!x_lo && !x_hi && !s_lo && !s_hi) {
    plan->t3_ext = false;
    return GBN_OK;
  }
  if (!x_lo || !x_hi || !s_lo || !s_hi)
    return fail(GBN_ERR_ARGS, "give all four extent arrays, or none to measure the extents");
  const double* v[4] = {x_lo, x_hi, s_lo, s_hi};
  for (int d = 0; d < plan->dim; ++d) {
    for (int k = 0; k < 4; ++k)
      if (!std::isfinite(v[k][d])) return fail(GBN_ERR_ARGS, "extents must be finite");
    if (x_lo[d] > x_hi[d] || s_lo[d] > s_hi[d])
      return fail(GBN_ERR_ARGS, "each extent needs lo <= hi");
  }
  GBN_CUDA(wait_flag_setup());
  for (int k = 0; k < 4; ++k)
    for (int d = 0; d < 3; ++d) plan->t3_ext_v[k][d] = d < plan->dim ? v[k][d] : 0.0;
  plan->t3_ext = true;
  return GBN_OK;
}

int gbn_wait_timeouts(long long* count, int reset) {
  if (!count) return fail(GBN_ERR_ARGS, "NULL argument");
  unsigned v = 0;
  GBN_CUDA(read_wait_timeouts(&v, reset != 0));
  if (reset) gbn::wait_flag_take();
  *count = (long long)v;
  return GBN_OK;
}

void gbn_debug_raise_wait_timeout(void) { gbn::wait_flag_raise(); }

int gbn_run(int type, int dim, int single, void* stream, double eps, int iflag, int64_t n_tot,
            int64_t n_transf, int64_t n_j, const int64_t* n_k, const gbn_opts* opts,
            const void* source, const void* const* pts, const void* const* tgts, void* output) {
  if (type < 1 || type > 3 || dim < 1 || dim > 3) return fail(GBN_ERR_ARGS, "bad type or dim");
  if (!n_k || !pts) return fail(GBN_ERR_ARGS, "NULL n_k or points");
  if (type == 3 && !tgts) return fail(GBN_ERR_ARGS, "NULL targets");
  if (int r = check_waits(GBN_OK)) return r;
  if (single) {
    const float* p[3] = {(const float*)pts[0], dim > 1 ? (const float*)pts[1] : nullptr,
                         dim > 2 ? (const float*)pts[2] : nullptr};
    const float* t[3] = {nullptr, nullptr, nullptr};
    if (type == 3)
      for (int d = 0; d < dim; ++d) t[d] = (const float*)tgts[d];
    return check_waits(run_oneshot<float>(type, dim, true, stream, eps, iflag, n_tot,
                                          n_transf, n_j, n_k, opts, source, p, t, output));
  }
  const double* p[3] = {(const double*)pts[0], dim > 1 ? (const double*)pts[1] : nullptr,
                        dim > 2 ? (const double*)pts[2] : nullptr};
  const double* t[3] = {nullptr, nullptr, nullptr};
  if (type == 3)
    for (int d = 0; d < dim; ++d) t[d] = (const double*)tgts[d];
  return check_waits(run_oneshot<double>(type, dim, false, stream, eps, iflag, n_tot, n_transf,
                                         n_j, n_k, opts, source, p, t, output));
}

}  // extern "C"

// ---------------------------------------------------------------------------
// the 18 named one-shot entry points (reference FFI target names)
// ---------------------------------------------------------------------------
namespace {
gbn_opts opts_from_attrs(int64_t modeord, double upsampfac, int64_t gpu_method, int64_t gpu_sort,
                         int64_t gpu_kerevalmeth, int64_t gpu_maxbatchsize, int64_t debug) {
  gbn_opts o;
  gbn_default_opts(&o);
  o.modeord = (int)modeord;
  o.upsampfac = upsampfac;
  o.gpu_method = (int)gpu_method;
  o.gpu_sort = (int)gpu_sort;
  o.gpu_kerevalmeth = (int)gpu_kerevalmeth;
  o.gpu_maxbatchsize = (int)gpu_maxbatchsize;
  o.debug = (int)debug;
  return o;
}
}  // namespace

#define GBN_ONESHOT_BODY(TYPE, DIM, SINGLE, TX, ...)                                             \
  {                                                                                              \
    gbn_opts o = opts_from_attrs(modeord, upsampfac, gpu_method, gpu_sort, gpu_kerevalmeth,      \
                                 gpu_maxbatchsize, debug);                                       \
    const int64_t nk[3] = {n_k_1, n_k_2, n_k_3};                                                 \
    const void* P[6] = {__VA_ARGS__};                                                            \
    const void* pts[3] = {P[0], DIM > 1 ? P[1] : nullptr, DIM > 2 ? P[2] : nullptr};             \
    const void* tg[3] = {TYPE == 3 ? P[DIM] : nullptr, (TYPE == 3 && DIM > 1) ? P[DIM + 1] : nullptr, \
                         (TYPE == 3 && DIM > 2) ? P[DIM + 2] : nullptr};                         \
    return gbn_run(TYPE, DIM, SINGLE, stream, (double)eps, (int)iflag, n_tot, n_transf, n_j, nk, \
                   &o, source, pts, tg, output);                                                 \
  }

extern "C" {
int gbn_nufft1d1f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, void* output)
    GBN_ONESHOT_BODY(1, 1, 1, float, x, nullptr, nullptr, nullptr, nullptr, nullptr)
int gbn_nufft1d1(GBN_ONESHOT_ARGS_D, const void* source, const double* x, void* output)
    GBN_ONESHOT_BODY(1, 1, 0, double, x, nullptr, nullptr, nullptr, nullptr, nullptr)
int gbn_nufft2d1f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, const float* y, void* output)
    GBN_ONESHOT_BODY(1, 2, 1, float, x, y, nullptr, nullptr, nullptr, nullptr)
int gbn_nufft2d1(GBN_ONESHOT_ARGS_D, const void* source, const double* x, const double* y, void* output)
    GBN_ONESHOT_BODY(1, 2, 0, double, x, y, nullptr, nullptr, nullptr, nullptr)
int gbn_nufft3d1f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, const float* y,
                  const float* z, void* output)
    GBN_ONESHOT_BODY(1, 3, 1, float, x, y, z, nullptr, nullptr, nullptr)
int gbn_nufft3d1(GBN_ONESHOT_ARGS_D, const void* source, const double* x, const double* y,
                 const double* z, void* output)
    GBN_ONESHOT_BODY(1, 3, 0, double, x, y, z, nullptr, nullptr, nullptr)
int gbn_nufft1d2f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, void* output)
    GBN_ONESHOT_BODY(2, 1, 1, float, x, nullptr, nullptr, nullptr, nullptr, nullptr)
int gbn_nufft1d2(GBN_ONESHOT_ARGS_D, const void* source, const double* x, void* output)
    GBN_ONESHOT_BODY(2, 1, 0, double, x, nullptr, nullptr, nullptr, nullptr, nullptr)
int gbn_nufft2d2f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, const float* y, void* output)
    GBN_ONESHOT_BODY(2, 2, 1, float, x, y, nullptr, nullptr, nullptr, nullptr)
int gbn_nufft2d2(GBN_ONESHOT_ARGS_D, const void* source, const double* x, const double* y, void* output)
    GBN_ONESHOT_BODY(2, 2, 0, double, x, y, nullptr, nullptr, nullptr, nullptr)
int gbn_nufft3d2f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, const float* y,
                  const float* z, void* output)
    GBN_ONESHOT_BODY(2, 3, 1, float, x, y, z, nullptr, nullptr, nullptr)
int gbn_nufft3d2(GBN_ONESHOT_ARGS_D, const void* source, const double* x, const double* y,
                 const double* z, void* output)
    GBN_ONESHOT_BODY(2, 3, 0, double, x, y, z, nullptr, nullptr, nullptr)
int gbn_nufft1d3f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, const float* s, void* output)
    GBN_ONESHOT_BODY(3, 1, 1, float, x, s, nullptr, nullptr, nullptr, nullptr)
int gbn_nufft1d3(GBN_ONESHOT_ARGS_D, const void* source, const double* x, const double* s, void* output)
    GBN_ONESHOT_BODY(3, 1, 0, double, x, s, nullptr, nullptr, nullptr, nullptr)
int gbn_nufft2d3f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, const float* y,
                  const float* s, const float* t, void* output)
    GBN_ONESHOT_BODY(3, 2, 1, float, x, y, s, t, nullptr, nullptr)
int gbn_nufft2d3(GBN_ONESHOT_ARGS_D, const void* source, const double* x, const double* y,
                 const double* s, const double* t, void* output)
    GBN_ONESHOT_BODY(3, 2, 0, double, x, y, s, t, nullptr, nullptr)
int gbn_nufft3d3f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, const float* y,
                  const float* z, const float* s, const float* t, const float* u, void* output)
    GBN_ONESHOT_BODY(3, 3, 1, float, x, y, z, s, t, u)
int gbn_nufft3d3(GBN_ONESHOT_ARGS_D, const void* source, const double* x, const double* y,
                 const double* z, const double* s, const double* t, const double* u,
                 void* output)
    GBN_ONESHOT_BODY(3, 3, 0, double, x, y, z, s, t, u)
}  // extern "C"

int gbn::set_error(int code, const std::string& msg) { return fail(code, msg); }

// =============================================================================
// batched plans: K independent problems (own points, own mode shape) of one
// type/dimension/precision, T transforms each, in packed arrays.
// =============================================================================
struct gbn_batch_s {
  int type = 1, dim = 1, K = 0, T = 1, iflag = 1;
  bool data_single = true, comp_single = true;
  cudaStream_t user = nullptr;    // the caller's stream
  cudaStream_t stream = nullptr;  // the batch's own stream (capturable; joined to `user`)
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  std::vector<std::unique_ptr<gbn_plan_s>> sub;  // geometry, kernel, deconvolution, points
  std::vector<int64_t> M, pt_off, c_off, f_off, grid_off;
  struct Group {
    int first;  // problem whose plan runs the group's FFT
    int count;  // problems in the group (T grids each)
    int64_t off;
  };
  std::vector<Group> groups;
  DevBuf arena, probs, item_start, counter;
  std::vector<unsigned char> probs_host;  // last uploaded table (stays alive for the copy)
  bool queue = true;
  int group = 6;  // lanes per point of the queue kernels: 6, 8 or 16 (widest kernel)
  int tb = 1;     // transforms per spread item
  size_t smem = 0;  // one transform's shared memory (largest problem)
  cudaGraphExec_t gexec = nullptr;
  const void* gkey[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  // per-problem stages (sorting, FFTs, deconvolution) of different problems
  // run on these streams side by side, forked from and joined back to
  // `stream` (small problems are launch-bound one after another)
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> side_done;
  cudaEvent_t ev_fork = nullptr;

  ~gbn_batch_s() {
    if (stream) cudaStreamSynchronize(stream);
    if (gexec) cudaGraphExecDestroy(gexec);
    DevBuf* bufs[] = {&arena, &probs, &item_start, &counter};
    for (DevBuf* b : bufs) b->release(stream);
    sub.clear();
    if (stream) {
      cudaStreamSynchronize(stream);
      cudaStreamDestroy(stream);
    }
    for (cudaStream_t t : side) cudaStreamDestroy(t);
    for (cudaEvent_t e : side_done) cudaEventDestroy(e);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
  }
};

namespace {

// Problems in flight side by side in a batch's per-problem stages.
constexpr int kBatchSideStreams = 8;

// Runs fn(i) for i = 0..n-1, item i with problem sub(i)'s plan on side
// stream i mod S: the side streams wait for everything already on the
// batch's stream, and the batch's stream waits for all of them before
// anything after (also when an item fails, so that a capture stays joined).
template <typename Sub, typename F>
int batch_fork(gbn_batch_s* b, int n, Sub sub, F fn) {
  const int S = (int)b->side.size();
  if (S == 0 || n < 2) {
    for (int i = 0; i < n; ++i) GBN_TRY(fn(i));
    return GBN_OK;
  }
  GBN_CUDA(cudaEventRecord(b->ev_fork, b->stream));
  const int used = std::min(S, n);
  for (int j = 0; j < used; ++j) GBN_CUDA(cudaStreamWaitEvent(b->side[j], b->ev_fork, 0));
  int r = GBN_OK;
  for (int i = 0; i < n && r < 2; ++i) {
    gbn_plan_s* p = sub(i);
    p->stream = b->side[i % S];
    r = fn(i);
    p->stream = b->stream;
    p->own.stream = b->stream;
  }
  for (int j = 0; j < used; ++j) {
    const cudaError_t e1 = cudaEventRecord(b->side_done[j], b->side[j]);
    const cudaError_t e2 = cudaStreamWaitEvent(b->stream, b->side_done[j], 0);
    if (r < 2 && (e1 != cudaSuccess || e2 != cudaSuccess)) GBN_CUDA(e1 != cudaSuccess ? e1 : e2);
  }
  return r;
}

}  // namespace

namespace {

int batch_create(int type, int dim, bool single, int K, const int64_t* nmodes, const int64_t* M,
                 const double* sigma, int T, int iflag, double eps, const gbn_opts* opts,
                 void* stream, gbn_batch_s** out) {
  *out = nullptr;
  if (type != 1 && type != 2) return fail(GBN_ERR_ARGS, "batched plans support types 1 and 2");
  if (K < 1) return fail(GBN_ERR_ARGS, "K must be >= 1");
  if (T < 1) return fail(GBN_ERR_ARGS, "ntransf must be >= 1");
  std::unique_ptr<gbn_batch_s> b(new gbn_batch_s());
  b->type = type;
  b->dim = dim;
  b->K = K;
  b->T = T;
  b->iflag = iflag >= 0 ? 1 : -1;
  b->data_single = single;
  b->user = (cudaStream_t)stream;
  GBN_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  GBN_CUDA(cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming));
  GBN_CUDA(cudaEventCreateWithFlags(&b->ev_out, cudaEventDisableTiming));
  if (K >= 2) {
    GBN_CUDA(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
    for (int j = 0; j < std::min(K, kBatchSideStreams); ++j) {
      cudaStream_t t = nullptr;
      cudaEvent_t e = nullptr;
      GBN_CUDA(cudaStreamCreateWithFlags(&t, cudaStreamNonBlocking));
      b->side.push_back(t);
      GBN_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      b->side_done.push_back(e);
    }
  }
  gbn_opts base;
  if (opts)
    base = *opts;
  else
    gbn_default_opts(&base);
  int warn = 0;
  int64_t pts = 0, modes = 0;
  for (int k = 0; k < K; ++k) {
    gbn_opts o = base;
    if (sigma && sigma[k] > 0.0) o.upsampfac = sigma[k];
    if ((base.gpu_autotune & GBN_TUNE_ON) && M[k] > 0) {
      // per-problem settings, shared-memory method only so the work queue applies
      gbn_opts q = o;
      q.gpu_autotune = base.gpu_autotune | GBN_TUNE_SM_ONLY;
      if (sigma && sigma[k] > 0.0) q.gpu_autotune |= GBN_TUNE_KEEP_SIGMA;
      const int r = gbn_autotune(type, dim, single ? 1 : 0, nmodes + 3 * k, M[k], T, eps, iflag,
                                 &q, (void*)b->stream, &o, nullptr);
      if (r >= 2) return r;
    }
    o.gpu_autotune = 0;
    o.gpu_maxbatchsize = T;
    o.debug = 0;
    gbn_plan_s* p = nullptr;
    int r = plan_create(type, dim, nmodes + 3 * k, iflag, T, eps, single, &o, (void*)b->stream,
                        &p);
    if (r >= 2) return r;
    warn |= r;
    b->sub.emplace_back(p);
    if (p->method != 2 || !p->sorted) b->queue = false;
    b->comp_single = p->comp_single;
    b->group = std::max(b->group, p->w > 8 ? 16 : p->w > 6 ? 8 : 6);
    const size_t tb = spread_smem_bytes(dim, p->geom.bs, p->w, p->comp_single,
                                        p->geom.maxsub, p->geom.stash != 0);
    b->smem = std::max(b->smem, tb);
    if (M[k] < 0) return fail(GBN_ERR_ARGS, "negative number of points");
    b->M.push_back(M[k]);
    b->pt_off.push_back(pts);
    b->c_off.push_back(pts * T);
    b->f_off.push_back(modes * T);
    pts += M[k];
    modes += p->Ntot;
  }
  // group problems by fine-grid shape: each group's grids are contiguous
  b->grid_off.assign(K, 0);
  std::vector<bool> placed(K, false);
  int64_t off = 0;
  for (int k = 0; k < K; ++k) {
    if (placed[k]) continue;
    gbn_batch_s::Group g{k, 0, off};
    for (int j = k; j < K; ++j) {
      if (placed[j]) continue;
      const gbn_plan_s* a = b->sub[k].get();
      const gbn_plan_s* c = b->sub[j].get();
      if (a->nf[0] != c->nf[0] || a->nf[1] != c->nf[1] || a->nf[2] != c->nf[2]) continue;
      placed[j] = true;
      b->grid_off[j] = off;
      off += (int64_t)T * c->nftot;
      ++g.count;
    }
    b->groups.push_back(g);
  }
  // stacked type-1 transforms share each point's kernel values in the queue
  // kernel (FP32, up to 100 KB of shared memory per block)
  if (type == 1 && b->comp_single && b->group <= 8) {
    if (T >= 4 && 4 * b->smem <= 100 * 1024)
      b->tb = 4;
    else if (T >= 2 && 2 * b->smem <= 100 * 1024)
      b->tb = 2;
  }
  // a single problem gains nothing from the work queue: it runs the plain
  // per-subproblem kernels (stacked transforms per block) on its own grid
  if (K == 1) b->queue = false;
  const size_t csz = cplx_size(b->comp_single);
  cudaStream_t s = b->stream;
  if (b->queue) GBN_CUDA(b->arena.ensure((size_t)off * csz, s));
  GBN_CUDA(b->item_start.ensure((size_t)(K + 1) * sizeof(int64_t), s));
  GBN_CUDA(b->counter.ensure(sizeof(int), s));
  *out = b.release();
  return warn ? GBN_WARN_EPS_TOO_SMALL : GBN_OK;
}

template <typename TC>
void fill_probs(gbn_batch_s* b, std::vector<unsigned char>& host) {
  host.assign(sizeof(BatchProb<TC>) * b->K, 0);
  BatchProb<TC>* pr = reinterpret_cast<BatchProb<TC>*>(host.data());
  for (int k = 0; k < b->K; ++k) {
    gbn_plan_s* p = b->sub[k].get();
    BatchProb<TC>& q = pr[k];
    q.g = p->geom;
    q.ks = ker_spec<TC>(p);
    q.M = p->own.M;
    q.recs = p->own.st.recs;
    q.sub_bin = p->own.st.sub_bin;
    q.sub_off = p->own.st.sub_off;
    q.n_sub = p->own.st.n_sub;
    q.bin_start = p->own.st.bin_start;
    q.bin_count = p->own.st.bin_count;
    q.perm = p->own.st.perm;
    q.c_off = b->c_off[k];
    q.grid_off = b->grid_off[k];
    q.nftot = p->nftot;
  }
}

// Sort every problem's points and refresh the work-queue table.
template <typename TX>
int batch_setpts(gbn_batch_s* b, const TX* x, const TX* y, const TX* z) {
  cudaStream_t s = b->stream;
  FoldSpec fs{};
  fs.mode = 0;
  GBN_TRY(batch_fork(
      b, b->K, [&](int k) { return b->sub[k].get(); },
      [&](int k) {
        const int64_t o = b->pt_off[k];
        return sort_points<TX>(b->sub[k].get(), b->sub[k]->own, b->M[k], x ? x + o : nullptr,
                               y ? y + o : nullptr, z ? z + o : nullptr, fs);
      }));
  if (!b->queue) return GBN_OK;
  std::vector<unsigned char> host;
  if (b->comp_single)
    fill_probs<float>(b, host);
  else
    fill_probs<double>(b, host);
  if (host != b->probs_host) {  // pointers change only when point buffers grow
    cudaStreamCaptureStatus cs;
    GBN_CUDA(cudaStreamIsCapturing(s, &cs));
    if (cs != cudaStreamCaptureStatusNone)
      return fail(GBN_ERR_STATE, "batched point buffers changed during graph capture");
    b->probs_host.swap(host);
    GBN_CUDA(b->probs.ensure(b->probs_host.size(), s));
    GBN_CUDA(cudaMemcpyAsync(b->probs.p, b->probs_host.data(), b->probs_host.size(),
                             cudaMemcpyHostToDevice, s));
  }
  const int per_sub = b->type == 1 ? (b->T + b->tb - 1) / b->tb : b->T;  // items per subproblem
  cudaError_t e = b->comp_single
                      ? launch_item_prefix<float>((const BatchProb<float>*)b->probs.p, b->K,
                                                  per_sub, b->item_start.as<int64_t>(), s)
                      : launch_item_prefix<double>((const BatchProb<double>*)b->probs.p, b->K,
                                                   per_sub, b->item_start.as<int64_t>(), s);
  GBN_CUDA(e);
  return GBN_OK;
}

int batch_execute(gbn_batch_s* b, void* c, void* f) {
  cudaStream_t s = b->stream;
  const size_t dsz = cplx_size(b->data_single), csz = cplx_size(b->comp_single);
  char* arena = (char*)b->arena.p;
  if (!b->queue) {  // a problem needs global-memory atomics: run problems one by one
    for (int k = 0; k < b->K; ++k) {
      gbn_plan_s* p = b->sub[k].get();
      GBN_TRY(execute_ntr(p, p->own, (char*)c + b->c_off[k] * dsz, (char*)f + b->f_off[k] * dsz,
                          b->T, 1));
    }
    return GBN_OK;
  }
  // problems on FP32 power-of-two grids take the library's pruned FFT with
  // the deconvolution fused (per problem); the others the per-group cuFFT
  // and separate deconvolution
  const char* no_own = std::getenv("GBN_DISABLE_OWN_FFT");
  const bool own_off = no_own && no_own[0] == '1';
  auto own_k = [&](int k) { return !own_off && b->sub[k]->fft_own; };
  auto sub_k = [&](int k) { return b->sub[k].get(); };
  // per problem: the own FFT with the deconvolution fused, or the
  // deconvolution alone (type 2: before the group FFTs; type 1: after)
  auto per_problem = [&](int k, bool to_modes) {
    char* fk = (char*)f + b->f_off[k] * dsz;
    char* gk = arena + b->grid_off[k] * csz;
    return own_k(k) ? own_fft(b->sub[k].get(), gk, fk, b->T, b->iflag, to_modes)
                    : do_deconv(b->sub[k].get(), fk, b->T, to_modes, gk);
  };
  // the groups whose problems share one cuFFT pass
  std::vector<const gbn_batch_s::Group*> cu;
  for (const auto& g : b->groups)
    if (!own_k(g.first)) cu.push_back(&g);
  auto per_group = [&](int i) {
    const gbn_batch_s::Group& g = *cu[i];
    return exec_fft(b->sub[g.first].get(), arena + g.off * csz, g.count * b->T, b->iflag);
  };
  auto group_sub = [&](int i) { return b->sub[cu[i]->first].get(); };
  if (b->type == 2) {
    GBN_TRY(batch_fork(b, b->K, sub_k, [&](int k) { return per_problem(k, false); }));
    GBN_TRY(batch_fork(b, (int)cu.size(), group_sub, per_group));
    GBN_CUDA(cudaMemsetAsync(b->counter.p, 0, sizeof(int), s));
    cudaError_t e;
    if (b->comp_single)
      e = b->data_single
              ? launch_interp_queue<float, float>(b->dim, b->group,
                                                  (const BatchProb<float>*)b->probs.p, b->K,
                                                  b->item_start.as<int64_t>(),
                                                  b->counter.as<int>(), b->T, arena, c, b->smem, s)
              : launch_interp_queue<float, double>(b->dim, b->group,
                                                   (const BatchProb<float>*)b->probs.p, b->K,
                                                   b->item_start.as<int64_t>(),
                                                   b->counter.as<int>(), b->T, arena, c, b->smem,
                                                   s);
    else
      e = launch_interp_queue<double, double>(b->dim, b->group,
                                              (const BatchProb<double>*)b->probs.p, b->K,
                                              b->item_start.as<int64_t>(), b->counter.as<int>(),
                                              b->T, arena, c, b->smem, s);
    GBN_CUDA(e);
  } else {
    GBN_CUDA(cudaMemsetAsync(arena, 0, b->arena.n, s));
    GBN_CUDA(cudaMemsetAsync(b->counter.p, 0, sizeof(int), s));
    cudaError_t e;
    if (b->comp_single)
      e = b->data_single
              ? launch_spread_queue<float, float>(b->dim, b->group, b->tb,
                                                  (const BatchProb<float>*)b->probs.p, b->K,
                                                  b->item_start.as<int64_t>(),
                                                  b->counter.as<int>(), b->T, c, arena, b->smem, s)
              : launch_spread_queue<float, double>(b->dim, b->group, b->tb,
                                                   (const BatchProb<float>*)b->probs.p, b->K,
                                                   b->item_start.as<int64_t>(),
                                                   b->counter.as<int>(), b->T, c, arena, b->smem,
                                                   s);
    else
      e = launch_spread_queue<double, double>(b->dim, b->group, b->tb,
                                              (const BatchProb<double>*)b->probs.p, b->K,
                                              b->item_start.as<int64_t>(), b->counter.as<int>(),
                                              b->T, c, arena, b->smem, s);
    GBN_CUDA(e);
    GBN_TRY(batch_fork(b, (int)cu.size(), group_sub, per_group));
    GBN_TRY(batch_fork(b, b->K, sub_k, [&](int k) { return per_problem(k, true); }));
  }
  GBN_CUDA(cudaGetLastError());
  return GBN_OK;
}

int batch_pass(gbn_batch_s* b, const void* x, const void* y, const void* z, void* c, void* f) {
  if (b->data_single) {
    GBN_TRY(batch_setpts<float>(b, (const float*)x, (const float*)y, (const float*)z));
  } else {
    GBN_TRY(batch_setpts<double>(b, (const double*)x, (const double*)y, (const double*)z));
  }
  return batch_execute(b, c, f);
}

int batch_run_on_own(gbn_batch_s* b, const void* x, const void* y, const void* z, void* c,
                     void* f, int use_graph);

// Work runs on the batch's own stream, ordered after everything already on
// the caller's stream and before anything the caller enqueues next.
int batch_run(gbn_batch_s* b, const void* x, const void* y, const void* z, void* c, void* f,
              int use_graph) {
  GBN_CUDA(cudaEventRecord(b->ev_in, b->user));
  GBN_CUDA(cudaStreamWaitEvent(b->stream, b->ev_in, 0));
  const int r = batch_run_on_own(b, x, y, z, c, f, use_graph);
  GBN_CUDA(cudaEventRecord(b->ev_out, b->stream));
  GBN_CUDA(cudaStreamWaitEvent(b->user, b->ev_out, 0));
  return r;
}

int batch_run_on_own(gbn_batch_s* b, const void* x, const void* y, const void* z, void* c,
                     void* f, int use_graph) {
  if (!use_graph) return batch_pass(b, x, y, z, c, f);
  const void* key[5] = {x, y, z, c, f};
  const bool same = b->gexec && std::memcmp(key, b->gkey, sizeof(key)) == 0;
  if (same) {
    GBN_CUDA(cudaGraphLaunch(b->gexec, b->stream));
    return GBN_OK;
  }
  // an eager pass sizes every buffer and creates every cuFFT plan, so the
  // captured pass allocates nothing; its results are the call's results
  GBN_TRY(batch_pass(b, x, y, z, c, f));
  if (b->gexec) {
    cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
  }
  cudaGraph_t graph = nullptr;
  GBN_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  int r = batch_pass(b, x, y, z, c, f);
  cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
  if (r >= 2) {
    if (graph) cudaGraphDestroy(graph);
    return r;
  }
  GBN_CUDA(e);
  e = cudaGraphInstantiate(&b->gexec, graph, 0);
  cudaGraphDestroy(graph);
  GBN_CUDA(e);
  std::memcpy(b->gkey, key, sizeof(key));
  return GBN_OK;
}

}  // namespace

extern "C" {

int gbn_batch_create(int type, int dim, int single, int K, const int64_t* nmodes,
                     const int64_t* M, const double* upsampfac, int ntransf, int iflag,
                     double eps, const gbn_opts* opts, void* stream, gbn_batch* out) {
  if (!out || !nmodes || !M) return fail(GBN_ERR_ARGS, "NULL argument");
  return batch_create(type, dim, single != 0, K, nmodes, M, upsampfac, ntransf, iflag, eps, opts,
                      stream, out);
}

int gbn_batch_run(gbn_batch b, const void* x, const void* y, const void* z, void* c, void* f,
                  int use_graph) {
  if (!b) return fail(GBN_ERR_ARGS, "NULL batch");
  if (int r = check_waits(GBN_OK)) return r;
  return check_waits(batch_run(b, x, y, z, c, f, use_graph));
}

int gbn_batch_info(gbn_batch b, int* ngroups, int* queue, int64_t* arena_bytes) {
  if (!b) return fail(GBN_ERR_ARGS, "NULL batch");
  if (ngroups) *ngroups = (int)b->groups.size();
  if (queue) *queue = b->queue ? 1 : 0;
  if (arena_bytes) *arena_bytes = (int64_t)b->arena.n;
  return GBN_OK;
}

int gbn_batch_destroy(gbn_batch b) {
  delete b;
  return GBN_OK;
}

}  // extern "C"

// =============================================================================
// batch chains: several batches (of either type) run as one pass -- each on
// its own stream, forked from and joined back to the chain's stream, so the
// batches overlap -- and, with use_graph, captured into one CUDA graph.
// =============================================================================
struct gbn_batch_chain_s {
  std::vector<gbn_batch_s*> b;  // not owned
  cudaStream_t user = nullptr, stream = nullptr;
  cudaEvent_t ev_in = nullptr, ev_fork = nullptr, ev_out = nullptr;
  cudaGraphExec_t gexec = nullptr;
  std::vector<const void*> gkey;

  ~gbn_batch_chain_s() {
    if (stream) cudaStreamSynchronize(stream);
    if (gexec) cudaGraphExecDestroy(gexec);
    cudaEvent_t evs[] = {ev_in, ev_fork, ev_out};
    for (cudaEvent_t e : evs)
      if (e) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

using PtrList = std::vector<const void*>;

int chain_pass(gbn_batch_chain_s* ch, const PtrList& key) {
  const size_t n = ch->b.size();
  GBN_CUDA(cudaEventRecord(ch->ev_fork, ch->stream));
  for (size_t i = 0; i < n; ++i) {
    gbn_batch_s* b = ch->b[i];
    const void* const* k = key.data() + 5 * i;
    GBN_CUDA(cudaStreamWaitEvent(b->stream, ch->ev_fork, 0));
    GBN_TRY(batch_pass(b, k[0], k[1], k[2], (void*)k[3], (void*)k[4]));
    GBN_CUDA(cudaEventRecord(b->ev_out, b->stream));
    GBN_CUDA(cudaStreamWaitEvent(ch->stream, b->ev_out, 0));
  }
  return GBN_OK;
}

int chain_run(gbn_batch_chain_s* ch, const PtrList& key, int use_graph) {
  GBN_CUDA(cudaEventRecord(ch->ev_in, ch->user));
  GBN_CUDA(cudaStreamWaitEvent(ch->stream, ch->ev_in, 0));
  int r = GBN_OK;
  if (!use_graph) {
    r = chain_pass(ch, key);
  } else if (ch->gexec && ch->gkey == key) {
    GBN_CUDA(cudaGraphLaunch(ch->gexec, ch->stream));
  } else {
    // an eager pass sizes every buffer and plan, then the same pass is
    // captured (the batches' streams join the capture through the fork event)
    GBN_TRY(chain_pass(ch, key));
    if (ch->gexec) {
      cudaGraphExecDestroy(ch->gexec);
      ch->gexec = nullptr;
    }
    cudaGraph_t graph = nullptr;
    GBN_CUDA(cudaStreamBeginCapture(ch->stream, cudaStreamCaptureModeThreadLocal));
    r = chain_pass(ch, key);
    cudaError_t e = cudaStreamEndCapture(ch->stream, &graph);
    if (r >= 2) {
      if (graph) cudaGraphDestroy(graph);
      return r;
    }
    GBN_CUDA(e);
    e = cudaGraphInstantiate(&ch->gexec, graph, 0);
    cudaGraphDestroy(graph);
    GBN_CUDA(e);
    ch->gkey = key;
  }
  GBN_CUDA(cudaEventRecord(ch->ev_out, ch->stream));
  GBN_CUDA(cudaStreamWaitEvent(ch->user, ch->ev_out, 0));
  return r;
}

}  // namespace

extern "C" {

int gbn_batch_chain_create(const gbn_batch* batches, int n, void* stream, gbn_batch_chain* out) {
  if (!out || !batches || n < 1) return fail(GBN_ERR_ARGS, "NULL argument or no batches");
  *out = nullptr;
  std::unique_ptr<gbn_batch_chain_s> ch(new gbn_batch_chain_s());
  for (int i = 0; i < n; ++i) {
    if (!batches[i]) return fail(GBN_ERR_ARGS, "NULL batch in the chain");
    for (gbn_batch_s* o : ch->b)
      if (o == batches[i]) return fail(GBN_ERR_ARGS, "a batch appears twice in the chain");
    ch->b.push_back(batches[i]);
  }
  ch->user = (cudaStream_t)stream;
  GBN_CUDA(cudaStreamCreateWithFlags(&ch->stream, cudaStreamNonBlocking));
  GBN_CUDA(cudaEventCreateWithFlags(&ch->ev_in, cudaEventDisableTiming));
  GBN_CUDA(cudaEventCreateWithFlags(&ch->ev_fork, cudaEventDisableTiming));
  GBN_CUDA(cudaEventCreateWithFlags(&ch->ev_out, cudaEventDisableTiming));
  *out = ch.release();
  return GBN_OK;
}

int gbn_batch_chain_run(gbn_batch_chain ch, const void* const* x, const void* const* y,
                        const void* const* z, void* const* c, void* const* f, int use_graph) {
  if (!ch || !x || !c || !f) return fail(GBN_ERR_ARGS, "NULL argument");
  if (int r = check_waits(GBN_OK)) return r;
  PtrList key;
  for (size_t i = 0; i < ch->b.size(); ++i) {
    key.push_back(x[i]);
    key.push_back(y ? y[i] : nullptr);
    key.push_back(z ? z[i] : nullptr);
    key.push_back(c[i]);
    key.push_back(f[i]);
  }
  return check_waits(chain_run(ch, key, use_graph));
}

int gbn_batch_chain_destroy(gbn_batch_chain ch) {
  delete ch;
  return GBN_OK;
}

}  // extern "C"
