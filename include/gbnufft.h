/*
 * gbnufft.h -- C ABI of the GB300 (sm_103a) NUFFT library.
 *
 * The library replaces the GPU path jax-finufft reaches through
 *   lib/jax_finufft_gpu.cc  ->  lib/kernels.cc.cu  ->  lib/cufinufft_wrapper.cc
 *   ->  vendored cuFINUFFT.
 * Every entry point takes plain pointers and sizes.  Device pointers are
 * expected unless a function says otherwise; work is enqueued on the given
 * CUDA stream and never synchronises the host except where noted
 * (type-3 setpts reads the point extents back to size its grid, unless
 * they were declared with gbn_set_t3_extents).
 *
 * Return codes follow the reference's convention (lib/kernels.cc.cu:52-55,
 * 70-79): 0 success, 1 warning (tolerance not reachable, clamped; results
 * are still produced), >= 2 error.  gbn_last_error() returns a message for
 * the calling thread's most recent non-zero code.
 *
 * Layouts are the reference backend's (lib/kernels.cc.cu:57-69,
 * src/jax_finufft/lowering.py:96-105): row-major, dimension 1 ("x") is the
 * fastest-varying mode axis, transforms stacked as (n_tot, n_transf, ...).
 */
#ifndef GBNUFFT_H
#define GBNUFFT_H

#include <stdint.h>

#if defined(__GNUC__)
#define GBN_API __attribute__((visibility("default")))
#else
#define GBN_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define GBN_OK 0
#define GBN_WARN_EPS_TOO_SMALL 1
#define GBN_ERR_ARGS 2
#define GBN_ERR_CUDA 3
#define GBN_ERR_CUFFT 4
#define GBN_ERR_ALLOC 5
#define GBN_ERR_STATE 6

/*
 * Options.  The first seven fields are the ones the reference forwards to
 * cuFINUFFT (src/jax_finufft/options.py:105-119, attrs at
 * lib/jax_finufft_gpu.cc:28-60); the bin-size and subproblem fields are the
 * GPU fields Opts carries but never forwards (options.py:69-77); the
 * precision field selects the compute precision (0 = automatic split).
 */
typedef struct gbn_opts {
  int modeord;            /* 0: modes -N/2..(N-1)/2; 1: FFT order */
  double upsampfac;       /* sigma: 2.0 (default) or 1.25; 0 picks 2.0 */
  int gpu_method;         /* 0 auto, 1 global-memory atomics over sorted points, 2 shared-memory subproblems */
  int gpu_sort;           /* 1 bin-sort points (default); 0 keep input order (forces method 1) */
  int gpu_kerevalmeth;    /* 1 piecewise Horner polynomials (default); 0 direct exp(sqrt) */
  int gpu_maxbatchsize;   /* transforms per cuFFT batch; 0 = all (bounded by memory) */
  int debug;              /* 1: time each stage with CUDA events (gbn_get_timings) */
  int gpu_binsizex;       /* bin size per axis in fine-grid cells; 0 = default */
  int gpu_binsizey;
  int gpu_binsizez;
  int gpu_maxsubprobsize; /* points per subproblem; 0 = default (1024) */
  int gpu_precision;      /* compute precision: 0 = the data's (complex64 -> FP32, complex128 ->
                             FP64, as cuFINUFFT); 1 = FP32; 2 = FP64 (complex128 only);
                             3 = split rule: FP32 when eps >= 1e-6, FP64 otherwise.  Point
                             folding and binning are FP64 in every mode. */
  int gpu_autotune;       /* batched plans: 0 off; GBN_TUNE_ON (| GBN_TUNE_SM_ONLY,
                             | GBN_TUNE_KEEP_SIGMA) picks each problem's settings with
                             gbn_autotune.  Ignored by the plan and one-shot entry points. */
  int gpu_kernel;         /* spreading kernel shape, same width rule either way:
                             GBN_KERNEL_ES (0, default) the exponential of semicircle of
                             FINUFFT, beta = 2.30 w at sigma = 2;
                             GBN_KERNEL_KB (1) Kaiser-Bessel I0(beta sqrt(1-z^2)) / I0(beta),
                             beta = pi sqrt((w/sigma)^2 (sigma-1/2)^2 - 0.8) (Beatty,
                             Nishimura, Pauly, IEEE TMI 2005): 1.5-2.5x smaller aliasing
                             error at the same width and cost. */
} gbn_opts;

#define GBN_KERNEL_ES 0
#define GBN_KERNEL_KB 1

#define GBN_TUNE_ON 1         /* tune sigma, method, bin size and points per subproblem */
#define GBN_TUNE_SM_ONLY 2    /* only the shared-memory method (keeps batches on the work queue) */
#define GBN_TUNE_KEEP_SIGMA 4 /* keep opts->upsampfac (or a batch's per-problem sigma) */

/* Fill *o with the defaults (cuFINUFFT's, per options.py:66-79). */
GBN_API void gbn_default_opts(gbn_opts* o);

/* Opaque plan. */
typedef struct gbn_plan_s* gbn_plan;

/*
 * Plan API.  Replaces cufinufft[f]_makeplan / _setpts / _execute / _destroy
 * as bound by lib/cufinufft_wrapper.cc:48-99.  The gbn_* functions take
 * complex128 data with float64 points, the gbnf_* functions complex64 data
 * with float32 points.  nmodes is in backend order (x first); for type 3 it
 * is ignored.  stream may be NULL (legacy default stream).
 */
GBN_API int gbn_makeplan(int type, int dim, const int64_t* nmodes, int iflag, int ntransf, double eps,
                 gbn_plan* plan, const gbn_opts* opts, void* stream);
GBN_API int gbnf_makeplan(int type, int dim, const int64_t* nmodes, int iflag, int ntransf, float eps,
                  gbn_plan* plan, const gbn_opts* opts, void* stream);

/* Set nonuniform points (device pointers; y/z may be NULL below their dim).
 * Type 3 also takes N target frequencies s/t/u. */
GBN_API int gbn_setpts(gbn_plan plan, int64_t M, const double* x, const double* y, const double* z,
               int64_t N, const double* s, const double* t, const double* u);
GBN_API int gbnf_setpts(gbn_plan plan, int64_t M, const float* x, const float* y, const float* z,
                int64_t N, const float* s, const float* t, const float* u);

/* Type 3: declare the extents of the sources (x_lo[d] <= x <= x_hi[d]) and
 * targets (s_lo[d] <= s <= s_hi[d]) per backend axis (host arrays of dim
 * doubles) for the following setpts calls.  setpts then sizes the grid from
 * them instead of measuring the points, so it does not synchronise the host
 * and is stream-ordered (with unchanged extents and sizes, the inner plan
 * and buffers are reused, so setpts and execute can be captured into a CUDA
 * graph after a first call).  Wider extents give a larger grid, same
 * accuracy.  A finite coordinate outside its declared extent is detected on
 * the device and makes the next API call on that device return
 * GBN_ERR_ARGS (the outputs since the previous check are invalid).  All four
 * pointers NULL: measure the extents again (the default). */
GBN_API int gbn_set_t3_extents(gbn_plan plan, const double* x_lo, const double* x_hi,
                               const double* s_lo, const double* s_hi);

/* Execute ntransf transforms.  Type 1: c (ntransf, M) -> f (ntransf, N...).
 * Type 2: f -> c.  Type 3: c (ntransf, M) -> f (ntransf, N). */
GBN_API int gbn_execute(gbn_plan plan, void* c, void* f);

/* Change the stream later calls enqueue on. */
GBN_API int gbn_set_stream(gbn_plan plan, void* stream);

/* Release the plan (synchronises its stream first). */
GBN_API int gbn_destroy(gbn_plan plan);

/* Plan introspection: kernel width, fine-grid sizes (backend order) and the
 * method actually used (1 or 2).  Any pointer may be NULL. */
GBN_API int gbn_plan_info(gbn_plan plan, int* w, int64_t* nf3, int* method, int* compute_double);

/* Per-stage device time (ms, CUDA events on the plan's stream) summed over
 * every execute and setpts since the previous call, when the plan was made
 * with opts.debug = 1: [0] spread (type 1) or interp (type 2), [1] FFT,
 * [2] deconvolve, [3] type-3 phasing + spread, [4] setpts.  *nbatch (may be
 * NULL) receives the number of executed batches summed.  Recording adds no
 * host synchronisation; this call synchronises the stream and resets the
 * sums. */
GBN_API int gbn_get_timings(gbn_plan plan, float* ms5, int* nbatch);

/* Copy the sorted per-point bin ids and the bin counts of the last setpts to
 * host memory (test hook for bit-exact comparison with the CPU oracle).
 * bins_out has M entries (bin of each input point, in input order);
 * counts_out has nbins entries.  Returns the number of bins in *nbins.
 * Either output may be NULL to query sizes.  Synchronises the stream. */
GBN_API int gbn_debug_bins(gbn_plan plan, int64_t* bins_out, int64_t* counts_out, int64_t* nbins);

/* Copy per-point grid starts (int64, M x 3, input order) and offsets delta
 * (double, M x 3, input order) computed by setpts (test hook). */
GBN_API int gbn_debug_fold(gbn_plan plan, int64_t* i0_out, double* delta_out);

/*
 * Point sets and fused gradients.  No counterpart in the reference: its
 * plans hold one point set (setpts, lib/kernels.cc.cu:57-80) and its
 * gradients are separate transforms issued by the JVP/transpose rules
 * (src/jax_finufft/ops.py:158-314), each sorting the points again.
 *
 * gbn_points_create sorts M points (device pointers in the plan's point
 * precision, backend order) for a type-1 or type-2 plan's geometry into a
 * point set that lives until gbn_points_destroy, so the forward's sort can
 * serve the backward.  gbn_execute_points runs ntr transforms on it: dir = +1
 * the plan's own transform, dir = -1 its adjoint (opposite exponent sign; a
 * type-1 plan then maps modes f to strengths c, a type-2 plan c to f).
 *
 * gbn_grad: gradients of a real loss through the plan's transform, with
 * g = the output cotangent (2 dL/dconj(out), PyTorch's convention):
 *   type-1 plan (f = A c, src = c (ntr, M), g (ntr, N...)):
 *     grad_src = A^H g (ntr, M) if non-NULL;
 *     grad_x[d][j] = sum_t Re(iflag i c_tj conj((A^H (k_d g_t))_j)).
 *   type-2 plan (c = B f, src = f (ntr, N...), g (ntr, M)):
 *     grad_src = B^H g (ntr, N...) if non-NULL;
 *     grad_x[d][j] = sum_t Re(conj(g_tj) (B (iflag i k_d f_t))_j).
 * grad_x holds dim pointers (backend order, M reals in the point precision,
 * NULL to skip an axis).  The coordinate terms and (type 1) the strength
 * gradient come from one batched cuFFT of the stacked k-weighted grids and
 * one interpolation pass with shared kernel weights, on the given point set.
 *
 * Type-3 plans take pts = NULL: they work on their own points (the last
 * gbn_setpts: sources sorted for the spreading grid, rescaled targets sorted
 * for the inner type 2).  gbn_execute_points with dir = -1 is the adjoint,
 * cotangents f (ntr, N targets) to c (ntr, M sources).  gbn_grad (f = A c,
 * src = c, g (ntr, N)) gives
 *     grad_src = A^H g;
 *     grad_x[d][j] = sum_t Re(c_tj conj(dH_tj / dx_d)),  H_t = A^H g_t,
 * from one adjoint pass whose gather on the sources also differentiates the
 * interpolant (the derivative of the kernel's polynomial pieces) -- one
 * inner FFT per transform where the reference's rules issue d + 1.  The
 * derivative of the interpolant amplifies its aliasing error by a small
 * factor: the source gradients carry a few times eps.  Target gradients are
 * not part of it.
 */
typedef struct gbn_points_s* gbn_points;
GBN_API int gbn_points_create(gbn_plan plan, int64_t M, const void* x, const void* y,
                              const void* z, gbn_points* out);
GBN_API int gbn_points_destroy(gbn_points pts);
GBN_API int gbn_execute_points(gbn_plan plan, gbn_points pts, int ntr, int dir, void* c, void* f);
GBN_API int gbn_grad(gbn_plan plan, gbn_points pts, int ntr, const void* src, const void* g,
                     void* grad_src, void* const* grad_x);

/*
 * Batched plans.  No counterpart in the reference, which loops over n_tot
 * point sets on the host with one plan (lib/kernels.cc.cu:57-80) and needs
 * one FFI call per independent problem of a different shape.  A batch holds K
 * independent type-1 or type-2 problems of one dimension and precision, each
 * with its own points and mode shape (nmodes: K x 3, backend order) and T
 * transforms.  Data are packed problem after problem:
 *   points x/y/z: sum_k M_k values, problem k at offset sum_{i<k} M_i;
 *   strengths/values c: problem k's (T, M_k) block at offset T*sum_{i<k} M_i;
 *   modes f: problem k's (T, N_k...) block at offset T*sum_{i<k} N_i.
 * upsampfac (K entries, or NULL for opts->upsampfac) sets sigma per problem.
 * gbn_batch_run sorts every problem's points and executes all transforms:
 * per-problem deconvolution, one batched cuFFT per group of equal grid
 * shapes over a shared grid arena, and one persistent spread (type 1) or
 * interpolation (type 2) kernel over a work queue of (problem, subproblem,
 * transform) items.  With use_graph = 1 the whole pass is captured into a
 * CUDA graph on the first call (after one eager pass, whose results it
 * returns) and replayed on later calls with the same five pointers.
 * The batch runs on a stream of its own (capture needs a non-legacy stream),
 * ordered by events after the work already on `stream` and before the work
 * queued on `stream` after gbn_batch_run returns.
 */
typedef struct gbn_batch_s* gbn_batch;
GBN_API int gbn_batch_create(int type, int dim, int single, int K, const int64_t* nmodes,
                             const int64_t* M, const double* upsampfac, int ntransf, int iflag,
                             double eps, const gbn_opts* opts, void* stream, gbn_batch* out);
GBN_API int gbn_batch_run(gbn_batch b, const void* x, const void* y, const void* z, void* c,
                          void* f, int use_graph);
GBN_API int gbn_batch_info(gbn_batch b, int* ngroups, int* queue, int64_t* arena_bytes);
GBN_API int gbn_batch_destroy(gbn_batch b);

/*
 * Batch chains (no counterpart in the reference): n batches, of either
 * type and any shapes, run as one pass -- each on its own stream, forked
 * from and joined back to the chain's stream so that they overlap -- and,
 * with use_graph = 1, captured into one CUDA graph on the first call and
 * replayed while the 5n pointers stay the same.  x/y/z/c/f hold one pointer
 * per batch, as gbn_batch_run takes them (y, z may be NULL arrays below
 * 3D).  The chain does not own its batches: destroy it before them, and do
 * not run its batches on their own while the chain is in use.  Ordered
 * after the work already on `stream` and before the work queued on it later.
 */
typedef struct gbn_batch_chain_s* gbn_batch_chain;
GBN_API int gbn_batch_chain_create(const gbn_batch* batches, int n, void* stream,
                                   gbn_batch_chain* out);
GBN_API int gbn_batch_chain_run(gbn_batch_chain ch, const void* const* x, const void* const* y,
                                const void* const* z, void* const* c, void* const* f,
                                int use_graph);
GBN_API int gbn_batch_chain_destroy(gbn_batch_chain ch);

/*
 * Autotuner (no counterpart in the reference, whose settings are fixed
 * per call).  For one problem class -- type (1 or 2), dim, precision, the
 * mode shape nmodes (backend order), M rounded up to a power of two,
 * ntransf, eps and the options' precision/kernel-evaluation fields -- times
 * candidate settings on seeded synthetic uniform points: sigma in {2, 1.25},
 * method 2 or 1, three bin shapes and 256..4096 points per subproblem.  The
 * fastest candidate whose relative l2 error against an FP64 transform at
 * eps/100 is at most max(eps, 1.5 x the default settings' error) is
 * written into *out (a copy of *base with upsampfac, gpu_method, bin sizes
 * and gpu_maxsubprobsize replaced).  base->gpu_autotune's GBN_TUNE_SM_ONLY
 * and GBN_TUNE_KEEP_SIGMA bits narrow the search.  Results are cached per
 * class and GPU model in memory and in a text file: $GBN_AUTOTUNE_CACHE
 * ("off" for none), else $XDG_CACHE_HOME/gbnufft/autotune.txt, else
 * $HOME/.cache/gbnufft/autotune.txt.  A cache miss synchronises `stream`
 * and allocates; do not call it while capturing.  info (NULL or 3
 * doubles): median ms of one setpts + execute, its error, 1 if cached.
 */
GBN_API int gbn_autotune(int type, int dim, int single, const int64_t* nmodes, int64_t M,
                         int ntransf, double eps, int iflag, const gbn_opts* base, void* stream,
                         gbn_opts* out, double* info);
/* Forget the in-memory autotuner cache; forget_file = 1 also stops it from
 * reloading the cache file in this process. */
GBN_API void gbn_autotune_clear(int forget_file);

/* Number of bounded device-side waits (the bulk tensor copy of a tile into
 * shared memory) that gave up on the current device since the last reset;
 * 0 in a healthy run.  reset = 1 clears it.  Synchronous.
 *
 * A wait that gives up skips its block's output, and the first call of
 * gbn_execute, gbn_execute_points, gbn_grad, gbn_run (and the named
 * entry points) or gbn_batch_run on that device that observes it returns
 * GBN_ERR_CUDA -- the reference turns a failed execute into an error the
 * same way (lib/kernels.cc.cu:70-79).  The check reads mapped host memory
 * without synchronising, so it reports work enqueued by that call or an
 * earlier one; synchronise the stream first to attribute it to one call. */
GBN_API int gbn_wait_timeouts(long long* count, int reset);

/* Test hook: mark the current device as if a bounded wait had given up, so
 * the error path above can be exercised without stalling a GPU. */
GBN_API void gbn_debug_raise_wait_timeout(void);


/* Thread-local message describing the last non-zero status. */
GBN_API const char* gbn_last_error(void);

/* Drop every cached plan held by the one-shot entry points. */
GBN_API void gbn_clear_cache(void);

/* Number of CUDA kernels this library has launched in this process (its own
 * kernels only; cuFFT's launches are not counted). */
GBN_API long long gbn_launch_count(void);

/*
 * One-shot entry points, one per XLA FFI target name the reference registers
 * (lib/jax_finufft_gpu.cc:392-420).  Each replaces the matching
 * nufft{D}d{T}{f}_impl of lib/kernels.h:24-180 (implemented at
 * lib/kernels.cc.cu:221-467) with the same scalar attributes in the same
 * order and raw device pointers in place of ffi::AnyBuffer:
 *   source, points (dim arrays, backend order), [targets,] output.
 * Semantics follow run_nufft (lib/kernels.cc.cu:25-92): one plan for the
 * call, a setpts + execute per index of n_tot, offsets index*n_j for points,
 * index*n_j*n_transf for strengths and index*n_k_total*n_transf for modes.
 * Unlike the reference, plans are cached across calls (keyed by shape,
 * options and stream) and the host is not synchronised.
 */
#define GBN_ONESHOT_ARGS_F                                                                     \
  void *stream, float eps, int64_t iflag, int64_t n_tot, int64_t n_transf, int64_t n_j,      \
      int64_t n_k_1, int64_t n_k_2, int64_t n_k_3, int64_t modeord, double upsampfac,         \
      int64_t gpu_method, int64_t gpu_sort, int64_t gpu_kerevalmeth, int64_t gpu_maxbatchsize, \
      int64_t debug
#define GBN_ONESHOT_ARGS_D                                                                     \
  void *stream, double eps, int64_t iflag, int64_t n_tot, int64_t n_transf, int64_t n_j,     \
      int64_t n_k_1, int64_t n_k_2, int64_t n_k_3, int64_t modeord, double upsampfac,         \
      int64_t gpu_method, int64_t gpu_sort, int64_t gpu_kerevalmeth, int64_t gpu_maxbatchsize, \
      int64_t debug

/* Type 1 (replaces nufft{1,2,3}d1{f,}_impl, lib/kernels.h:24-70). */
GBN_API int gbn_nufft1d1f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, void* output);
GBN_API int gbn_nufft1d1(GBN_ONESHOT_ARGS_D, const void* source, const double* x, void* output);
GBN_API int gbn_nufft2d1f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, const float* y,
                  void* output);
GBN_API int gbn_nufft2d1(GBN_ONESHOT_ARGS_D, const void* source, const double* x, const double* y,
                 void* output);
GBN_API int gbn_nufft3d1f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, const float* y,
                  const float* z, void* output);
GBN_API int gbn_nufft3d1(GBN_ONESHOT_ARGS_D, const void* source, const double* x, const double* y,
                 const double* z, void* output);

/* Type 2 (replaces nufft{1,2,3}d2{f,}_impl, lib/kernels.h:76-126). */
GBN_API int gbn_nufft1d2f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, void* output);
GBN_API int gbn_nufft1d2(GBN_ONESHOT_ARGS_D, const void* source, const double* x, void* output);
GBN_API int gbn_nufft2d2f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, const float* y,
                  void* output);
GBN_API int gbn_nufft2d2(GBN_ONESHOT_ARGS_D, const void* source, const double* x, const double* y,
                 void* output);
GBN_API int gbn_nufft3d2f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, const float* y,
                  const float* z, void* output);
GBN_API int gbn_nufft3d2(GBN_ONESHOT_ARGS_D, const void* source, const double* x, const double* y,
                 const double* z, void* output);

/* Type 3 (replaces nufft{1,2,3}d3{f,}_impl, lib/kernels.h:132-180); n_k_1 is
 * the number of targets. */
GBN_API int gbn_nufft1d3f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, const float* s,
                  void* output);
GBN_API int gbn_nufft1d3(GBN_ONESHOT_ARGS_D, const void* source, const double* x, const double* s,
                 void* output);
GBN_API int gbn_nufft2d3f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, const float* y,
                  const float* s, const float* t, void* output);
GBN_API int gbn_nufft2d3(GBN_ONESHOT_ARGS_D, const void* source, const double* x, const double* y,
                 const double* s, const double* t, void* output);
GBN_API int gbn_nufft3d3f(GBN_ONESHOT_ARGS_F, const void* source, const float* x, const float* y,
                  const float* z, const float* s, const float* t, const float* u, void* output);
GBN_API int gbn_nufft3d3(GBN_ONESHOT_ARGS_D, const void* source, const double* x, const double* y,
                 const double* z, const double* s, const double* t, const double* u,
                 void* output);

/*
 * Bin-sort nonuniform points without allocating any memory.  No counterpart
 * in the reference: it serves callers that cannot call cudaMalloc (plugins
 * whose host framework owns all device memory, pipelines that reserve every
 * byte up front, hooks that must not allocate).  It runs the fold (with
 * the FP64 chain's results) and bin sort of setpts on caller-provided
 * points (float32 when single = 1,
 * else float64; device pointers, backend order) for a fine grid of nf[d]
 * cells in bins of binsize[d] cells per axis and kernel width w (2..16; a
 * point belongs to the bin holding the first cell of its w-wide support, as
 * in setpts; gbn_plan_info reports a plan's w), and writes to caller-owned
 * device arrays: bins[M] (bin of each point, same numbering as setpts),
 * counts[nbins] (points per bin, nbins = prod ceil(nf/binsize)) and perm[M]
 * (input index of each point in bin order).
 * Its scratch (per-point ranks and folded records, scan partial sums) is one
 * fixed device array of GBN_NOALLOC_SCRATCH_BYTES inside the library, held
 * by every GPU that loads the library until the process exits; M above
 * GBN_NOALLOC_MAX_POINTS or more than GBN_NOALLOC_MAX_BINS bins is rejected
 * with GBN_ERR_ARGS.  Every call looks up the array's device address in the
 * current context (cudaGetSymbolAddress; nothing is cached, so a device reset
 * or another context leaves no stale address); the first call on each
 * device, and the first after a reset, loads the library's module, so make
 * it before any stream capture.  All calls share the array: calls
 * whose work overlaps on the GPU race.  Enqueued on `stream`; no host sync.
 */
#define GBN_NOALLOC_MAX_POINTS 262144
#define GBN_NOALLOC_MAX_BINS 262144
#define GBN_NOALLOC_SCRATCH_BYTES (16 * 1024 * 1024)
GBN_API int gbn_binsort_noalloc(void* stream, int dim, int single, int64_t M, const void* x,
                                const void* y, const void* z, const int64_t* nf,
                                const int* binsize, int w, int* bins, int* counts, int* perm);

/*
 * Generic one-shot call with full options (bin sizes, precision): the torch
 * binding uses this.  single = 1 for complex64/float32 data.  pts/tgts hold
 * dim device pointers each (tgts only for type 3).  n_k in backend order
 * (type 3: n_k[0] = number of targets).  Same semantics as the named
 * entry points above.
 */
GBN_API int gbn_run(int type, int dim, int single, void* stream, double eps, int iflag, int64_t n_tot,
            int64_t n_transf, int64_t n_j, const int64_t* n_k, const gbn_opts* opts,
            const void* source, const void* const* pts, const void* const* tgts, void* output);

#ifdef __cplusplus
}
#endif

#endif /* GBNUFFT_H */
