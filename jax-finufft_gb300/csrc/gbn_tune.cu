// gbn_tune.cu -- autotuner for the type-1/2 execution settings.
//
// For one problem class -- type, dimension, precision, mode shape, point
// count (bucketed to a power of two), transforms per call, tolerance -- the
// tuner times a small set of candidate settings on seeded synthetic inputs
// (points iid uniform in [-pi, pi)^d, values uniform in the unit square) and
// keeps the fastest one whose accuracy holds:
//   * upsampling factor sigma in {2, 1.25} (1.25 halves the FFT size per
//     axis at the price of a wider kernel),
//   * method: shared-memory subproblems (2) or global-memory atomics over
//     bin-sorted points (1),
//   * bin size per axis (three shapes per dimension),
//   * points per subproblem (the work of one thread block): 256 .. 4096.
// Accuracy is measured against an FP64 transform of the same inputs at a
// tolerance 100x tighter; a candidate is admitted when its relative l2 error
// is at most max(eps, 1.5 x the error of the default settings).  This keeps
// sigma = 1.25 out of FP32 runs whose round-off it would amplify.
//
// Results are cached in memory and, unless GBN_AUTOTUNE_CACHE is "off", in a
// text file (GBN_AUTOTUNE_CACHE, else $XDG_CACHE_HOME/gbnufft/autotune.txt,
// else $HOME/.cache/gbnufft/autotune.txt), one line per class, keyed also by
// the GPU's name.  Tuning synchronises the stream and allocates its inputs;
// it is a planning step and must not run inside a stream capture.
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/gbnufft.h"
#include "gbn_common.cuh"

namespace gbn {

namespace {

#define GBN_TRY_CUDA(expr)                                                                     \
  do {                                                                                         \
    cudaError_t e_ = (expr);                                                                   \
    if (e_ != cudaSuccess)                                                                     \
      return set_error(GBN_ERR_CUDA, std::string(#expr) + " failed: " + cudaGetErrorString(e_)); \
  } while (0)

#define GBN_TRY(expr)       \
  do {                      \
    int r_ = (expr);        \
    if (r_ >= 2) return r_; \
  } while (0)

// splitmix64: a counter-based generator, one independent value per index.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// out[i] = lo + (hi - lo) * u_i, u_i uniform in [0, 1) with 53 random bits.
template <typename T>
__global__ void synth_uniform_kernel(T* out, int64_t n, uint64_t seed, double lo, double hi) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double u = (double)(mix64(seed ^ (uint64_t)i * 0x2545f4914f6cdd1dull) >> 11) *
                     (1.0 / 9007199254740992.0);
    out[i] = (T)(lo + (hi - lo) * u);
  }
}

__global__ void widen_kernel(const float* in, double* out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (double)in[i];
}

template <typename T>
cudaError_t synth(T* out, int64_t n, uint64_t seed, double lo, double hi, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
  synth_uniform_kernel<T><<<blocks, 256, 0, s>>>(out, n, seed, lo, hi);
  note_launch();
  return cudaGetLastError();
}

cudaError_t widen(const float* in, double* out, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
  widen_kernel<<<blocks, 256, 0, s>>>(in, out, n);
  note_launch();
  return cudaGetLastError();
}

struct Tuned {
  double sigma = 2.0;
  int method = 2;
  int bs[3] = {0, 0, 0};
  int maxsub = 1024;
  double ms = 0.0;
  double err = 0.0;
};

std::mutex g_mu;
std::map<std::string, Tuned> g_cache;
bool g_loaded = false;

std::string cache_path() {
  const char* env = std::getenv("GBN_AUTOTUNE_CACHE");
  if (env && *env) {
    if (std::strcmp(env, "off") == 0) return std::string();
    return env;
  }
  const char* xdg = std::getenv("XDG_CACHE_HOME");
  if (xdg && *xdg) return std::string(xdg) + "/gbnufft/autotune.txt";
  const char* home = std::getenv("HOME");
  if (home && *home) return std::string(home) + "/.cache/gbnufft/autotune.txt";
  return std::string();
}

void make_parents(const std::string& path) {
  for (size_t i = 1; i < path.size(); ++i)
    if (path[i] == '/') ::mkdir(path.substr(0, i).c_str(), 0755);
}

// File format: one line per class, "<key>|<sigma> <method> <bx> <by> <bz>
// <maxsub> <ms> <err>".  Later lines override earlier ones.
void load_cache_locked() {
  if (g_loaded) return;
  g_loaded = true;
  const std::string path = cache_path();
  if (path.empty()) return;
  std::ifstream in(path);
  std::string line;
  while (std::getline(in, line)) {
    const size_t bar = line.find('|');
    if (bar == std::string::npos) continue;
    Tuned t;
    std::istringstream vs(line.substr(bar + 1));
    if (vs >> t.sigma >> t.method >> t.bs[0] >> t.bs[1] >> t.bs[2] >> t.maxsub >> t.ms >> t.err)
      g_cache[line.substr(0, bar)] = t;
  }
}

void store_locked(const std::string& key, const Tuned& t) {
  g_cache[key] = t;
  const std::string path = cache_path();
  if (path.empty()) return;
  make_parents(path);
  std::ofstream out(path, std::ios::app);
  if (!out) return;  // a read-only cache location leaves the in-memory entry
  char buf[256];
  std::snprintf(buf, sizeof(buf), "%.17g %d %d %d %d %d %.6g %.6g", t.sigma, t.method, t.bs[0],
                t.bs[1], t.bs[2], t.maxsub, t.ms, t.err);
  out << key << '|' << buf << '\n';
}

// The current device's name with blanks replaced (looked up once per device).
std::string device_name() {
  static std::mutex mu;
  static std::map<int, std::string> names;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  auto it = names.find(dev);
  if (it != names.end()) return it->second;
  char buf[256] = "gpu";
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) == cudaSuccess)
    std::snprintf(buf, sizeof(buf), "%s", prop.name);
  std::string gpu = buf;
  for (char& ch : gpu)
    if (ch == ' ' || ch == '|') ch = '_';
  names[dev] = gpu;
  return gpu;
}

std::string class_key(int type, int dim, bool single, const int64_t* nm, int64_t M, int T,
                      double eps, const gbn_opts& base, double sigma_fixed, bool allow_gm) {
  const std::string gpu = device_name();
  int lg = 0;
  while (lg < 62 && ((int64_t)1 << lg) < std::max<int64_t>(M, 1)) ++lg;
  char buf[512];
  std::snprintf(buf, sizeof(buf),
                "v1 %s t%d d%d s%d n%lldx%lldx%lld m2^%d T%d e%.3g p%d k%d sig%.3g gm%d%s",
                gpu.c_str(), type, dim, single ? 1 : 0, (long long)nm[0],
                (long long)(dim > 1 ? nm[1] : 1), (long long)(dim > 2 ? nm[2] : 1), lg, T, eps,
                base.gpu_precision, base.gpu_kerevalmeth, sigma_fixed, allow_gm ? 1 : 0,
                base.gpu_kernel == 1 ? " kb" : "");
  return buf;
}

// Device buffers of one tuning session (cudaMallocAsync on the tuning stream).
struct Scratch {
  cudaStream_t s;
  std::vector<void*> ptrs;
  explicit Scratch(cudaStream_t s_) : s(s_) {}
  ~Scratch() {
    for (void* p : ptrs) cudaFreeAsync(p, s);
    cudaStreamSynchronize(s);
  }
  template <typename T>
  cudaError_t get(T** out, size_t n) {
    void* p = nullptr;
    cudaError_t e = cudaMallocAsync(&p, std::max<size_t>(n, 1) * sizeof(T), s);
    if (e == cudaSuccess) ptrs.push_back(p);
    *out = static_cast<T*>(p);
    return e;
  }
};

// One plan + setpts + execute sequence; optionally timed (median of reps).
struct Problem {
  int type, dim, T, iflag;
  bool single;
  const int64_t* nm;
  int64_t M, Ntot;
  double eps;
  cudaStream_t s;
  const void* x[3];  // points, the candidate's precision
  void* c;           // strengths (type 1 input / type 2 output)
  void* f;           // modes (type 1 output / type 2 input)
};

int run_once(const Problem& pb, const gbn_opts& o, int reps, double* ms_out) {
  gbn_plan plan = nullptr;
  int r = pb.single ? gbnf_makeplan(pb.type, pb.dim, pb.nm, pb.iflag, pb.T, (float)pb.eps, &plan,
                                    &o, (void*)pb.s)
                    : gbn_makeplan(pb.type, pb.dim, pb.nm, pb.iflag, pb.T, pb.eps, &plan, &o,
                                   (void*)pb.s);
  if (r >= 2) return r;
  auto step = [&]() -> int {
    int q = pb.single
                ? gbnf_setpts(plan, pb.M, (const float*)pb.x[0], (const float*)pb.x[1],
                              (const float*)pb.x[2], 0, nullptr, nullptr, nullptr)
                : gbn_setpts(plan, pb.M, (const double*)pb.x[0], (const double*)pb.x[1],
                             (const double*)pb.x[2], 0, nullptr, nullptr, nullptr);
    if (q >= 2) return q;
    return gbn_execute(plan, pb.c, pb.f);
  };
  r = step();  // warm-up (and the result when reps == 0)
  if (r < 2 && reps > 0) {
    std::vector<double> t;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int i = 0; i < reps && r < 2; ++i) {
      cudaEventRecord(e0, pb.s);
      r = step();
      cudaEventRecord(e1, pb.s);
      if (cudaEventSynchronize(e1) != cudaSuccess) r = GBN_ERR_CUDA;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      t.push_back(ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!t.empty()) {
      std::sort(t.begin(), t.end());
      *ms_out = t[t.size() / 2];
    }
  }
  cudaStreamSynchronize(pb.s);
  gbn_destroy(plan);
  return r;
}

// Relative l2 distance of the candidate output (the plan's precision) from
// the FP64 reference, over the first n values (both copied to the host).
template <typename T>
double rel_err_host(const void* cand, const std::complex<double>* ref, int64_t n,
                    cudaStream_t s) {
  std::vector<std::complex<T>> h((size_t)n);
  if (cudaMemcpyAsync(h.data(), cand, n * sizeof(std::complex<T>), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return INFINITY;
  double num = 0.0, den = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    const std::complex<double> d = std::complex<double>(h[i]) - ref[i];
    num += std::norm(d);
    den += std::norm(ref[i]);
  }
  return den > 0.0 ? std::sqrt(num / den) : std::sqrt(num);
}

int tune(int type, int dim, bool single, const int64_t* nm, int64_t M, int T, double eps,
         int iflag, const gbn_opts& base, double sigma_fixed, bool allow_gm, cudaStream_t s,
         Tuned* best_out) {
  int64_t Ntot = 1;
  for (int d = 0; d < dim; ++d) Ntot *= nm[d];
  const int64_t n_out = (type == 1 ? Ntot : M) * T;
  const int64_t n_chk = std::min<int64_t>(n_out, (int64_t)1 << 20);
  Scratch sc(s);
  // inputs in the candidate's precision; FP64 copies for the reference
  void* x[3] = {nullptr, nullptr, nullptr};
  double* xd[3] = {nullptr, nullptr, nullptr};
  void *c = nullptr, *f = nullptr;
  double *cd = nullptr, *fd = nullptr;
  const uint64_t seed = 0x5eedf00d1234ull;
  for (int d = 0; d < dim; ++d) {
    if (single) {
      float* p;
      GBN_TRY_CUDA(sc.get(&p, M));
      GBN_TRY_CUDA(synth(p, M, seed + d, -M_PI, M_PI, s));
      x[d] = p;
      GBN_TRY_CUDA(sc.get(&xd[d], M));
      GBN_TRY_CUDA(widen(p, xd[d], M, s));
    } else {
      GBN_TRY_CUDA(sc.get(&xd[d], M));
      GBN_TRY_CUDA(synth(xd[d], M, seed + d, -M_PI, M_PI, s));
      x[d] = xd[d];
    }
  }
  const int64_t n_in = (type == 1 ? M : Ntot) * T;  // complex values
  if (single) {
    float *ci, *co;
    GBN_TRY_CUDA(sc.get(&ci, 2 * n_in));
    GBN_TRY_CUDA(synth(ci, 2 * n_in, seed + 7, -1.0, 1.0, s));
    GBN_TRY_CUDA(sc.get(&co, 2 * n_out));
    double* cid;
    GBN_TRY_CUDA(sc.get(&cid, 2 * n_in));
    GBN_TRY_CUDA(widen(ci, cid, 2 * n_in, s));
    double* cod;
    GBN_TRY_CUDA(sc.get(&cod, 2 * n_out));
    if (type == 1) {
      c = ci, f = co, cd = cid, fd = cod;
    } else {
      f = ci, c = co, fd = cid, cd = cod;
    }
  } else {
    double *ci, *co;
    GBN_TRY_CUDA(sc.get(&ci, 2 * n_in));
    GBN_TRY_CUDA(synth(ci, 2 * n_in, seed + 7, -1.0, 1.0, s));
    GBN_TRY_CUDA(sc.get(&co, 2 * n_out));
    double* cod;
    GBN_TRY_CUDA(sc.get(&cod, 2 * n_out));
    if (type == 1) {
      c = ci, f = co, cd = ci, fd = cod;
    } else {
      f = ci, c = co, fd = ci, cd = cod;
    }
  }
  // FP64 reference at sigma = 2 and a tolerance 100x tighter
  {
    Problem ref{type, dim, T, iflag, false, nm, M, Ntot, std::max(eps * 1e-2, 1e-14), s,
                {xd[0], xd[1], xd[2]}, cd, fd};
    gbn_opts o = base;
    o.upsampfac = 2.0;
    o.gpu_precision = 0;
    o.debug = 0;
    double ms = 0;
    GBN_TRY(run_once(ref, o, 0, &ms));
  }
  std::vector<std::complex<double>> refh((size_t)n_chk);
  GBN_TRY_CUDA(cudaMemcpyAsync(refh.data(), type == 1 ? fd : cd,
                               n_chk * sizeof(std::complex<double>), cudaMemcpyDeviceToHost, s));
  GBN_TRY_CUDA(cudaStreamSynchronize(s));

  Problem pb{type, dim, T, iflag, single, nm, M, Ntot, eps, s, {x[0], x[1], x[2]}, c, f};
  const void* out = type == 1 ? f : c;
  auto evaluate = [&](const gbn_opts& o, double* ms, double* err) -> int {
    *ms = INFINITY;
    int r = run_once(pb, o, 3, ms);
    if (r >= 2) return r;  // a candidate the plan rejects is skipped
    *err = single ? rel_err_host<float>(out, refh.data(), n_chk, s)
                  : rel_err_host<double>(out, refh.data(), n_chk, s);
    return GBN_OK;
  };

  // candidate bin shapes per dimension (0 = the plan's default)
  std::vector<std::vector<int>> bins;
  if (dim == 1) bins = {{0, 1, 1}, {512, 1, 1}, {2048, 1, 1}};
  if (dim == 2) bins = {{0, 0, 1}, {16, 16, 1}, {64, 64, 1}};
  if (dim == 3) bins = {{0, 0, 0}, {8, 8, 8}, {16, 16, 16}};
  std::vector<double> sigmas;
  if (sigma_fixed > 0.0)
    sigmas = {sigma_fixed};
  else
    sigmas = {2.0, 1.25};

  gbn_opts o0 = base;
  o0.debug = 0;
  o0.gpu_sort = 1;
  o0.upsampfac = sigmas[0];
  o0.gpu_method = 0;
  o0.gpu_binsizex = o0.gpu_binsizey = o0.gpu_binsizez = 0;
  o0.gpu_maxsubprobsize = 0;
  double ms0 = INFINITY, err0 = INFINITY;
  GBN_TRY(evaluate(o0, &ms0, &err0));
  const double err_ok = std::max(eps, 1.5 * err0);
  Tuned best;
  best.sigma = o0.upsampfac;
  best.method = 0;
  best.ms = ms0;
  best.err = err0;
  gbn_opts best_o = o0;
  auto consider = [&](const gbn_opts& o) {
    double ms, err;
    if (evaluate(o, &ms, &err) >= 2) return;
    if (!(err <= err_ok)) return;
    if (ms < best.ms) {
      best.ms = ms;
      best.err = err;
      best.sigma = o.upsampfac;
      best.method = o.gpu_method;
      best.bs[0] = o.gpu_binsizex;
      best.bs[1] = o.gpu_binsizey;
      best.bs[2] = o.gpu_binsizez;
      best.maxsub = o.gpu_maxsubprobsize;
      best_o = o;
    }
  };
  for (double sg : sigmas) {
    for (size_t bi = 0; bi < bins.size(); ++bi) {
      gbn_opts o = o0;
      o.upsampfac = sg;
      o.gpu_method = 2;
      o.gpu_binsizex = bins[bi][0];
      o.gpu_binsizey = bins[bi][1];
      o.gpu_binsizez = bins[bi][2];
      consider(o);
    }
    if (allow_gm) {
      gbn_opts o = o0;
      o.upsampfac = sg;
      o.gpu_method = 1;
      consider(o);
    }
  }
  // points per subproblem for the best shared-memory setting
  if (best_o.gpu_method == 2) {
    const gbn_opts bo = best_o;
    for (int ms : {256, 512, 2048, 4096}) {
      gbn_opts o = bo;
      o.gpu_maxsubprobsize = ms;
      consider(o);
    }
  }
  *best_out = best;
  return GBN_OK;
}

}  // namespace

}  // namespace gbn

extern "C" {

int gbn_autotune(int type, int dim, int single, const int64_t* nmodes, int64_t M, int ntransf,
                 double eps, int iflag, const gbn_opts* base_in, void* stream, gbn_opts* out,
                 double* info) {
  using namespace gbn;
  if (!out || !nmodes) return set_error(GBN_ERR_ARGS, "gbn_autotune: null argument");
  if (type != 1 && type != 2) return set_error(GBN_ERR_ARGS, "gbn_autotune: types 1 and 2 only");
  if (dim < 1 || dim > 3) return set_error(GBN_ERR_ARGS, "gbn_autotune: dim must be 1..3");
  if (M < 1 || ntransf < 1) return set_error(GBN_ERR_ARGS, "gbn_autotune: M and ntransf >= 1");
  gbn_opts base;
  if (base_in)
    base = *base_in;
  else
    gbn_default_opts(&base);
  const bool allow_gm = (base.gpu_autotune & GBN_TUNE_SM_ONLY) == 0;
  const double sigma_fixed =
      (base.gpu_autotune & GBN_TUNE_KEEP_SIGMA) ? (base.upsampfac > 0.0 ? base.upsampfac : 2.0)
                                                : 0.0;
  const std::string key = class_key(type, dim, single != 0, nmodes, M, ntransf, eps, base,
                                    sigma_fixed, allow_gm);
  Tuned t;
  bool hit = false;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    load_cache_locked();
    auto it = g_cache.find(key);
    if (it != g_cache.end()) {
      t = it->second;
      hit = true;
    }
  }
  if (!hit) {
    // tune at the class's representative size: M rounded up to its power of two
    int64_t Mt = 1;
    while (Mt < M) Mt <<= 1;
    int r = tune(type, dim, single != 0, nmodes, Mt, ntransf, eps, iflag, base, sigma_fixed,
                 allow_gm, (cudaStream_t)stream, &t);
    if (r >= 2) return r;
    std::lock_guard<std::mutex> lk(g_mu);
    store_locked(key, t);
  }
  *out = base;
  out->upsampfac = t.sigma;
  out->gpu_method = t.method;
  out->gpu_binsizex = t.bs[0];
  out->gpu_binsizey = t.bs[1];
  out->gpu_binsizez = t.bs[2];
  out->gpu_maxsubprobsize = t.maxsub;
  out->gpu_autotune = 0;
  if (info) {
    info[0] = t.ms;
    info[1] = t.err;
    info[2] = hit ? 1.0 : 0.0;
  }
  return GBN_OK;
}

void gbn_autotune_clear(int forget_file) {
  using namespace gbn;
  std::lock_guard<std::mutex> lk(g_mu);
  g_cache.clear();
  g_loaded = forget_file != 0;  // 1: do not reload the file either
}

}  // extern "C"
