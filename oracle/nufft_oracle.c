/*
 * nufft_oracle.c -- CPU restatement of the NUFFT algorithm that jax-finufft
 * reaches through cuFINUFFT / FINUFFT 2.4.1.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA library in
 * jax-finufft_gb300/csrc: only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load it.  The product path never calls into it.
 *
 * The reference repository vendors FINUFFT as an empty git submodule
 * (.gitmodules:1-3, CMakeLists.txt:61), so the arithmetic below restates the
 * published method instead of copying code:
 *   - Barnett, Magland, af Klinteberg, "A parallel non-uniform fast Fourier
 *     transform library based on an exponential of semicircle kernel",
 *     SIAM J. Sci. Comput. 41 (2019): ES kernel, the width/beta rule, the
 *     upsampled-grid size rule, deconvolution by the kernel's Fourier
 *     transform, and the type-3 rescaling.
 *   - Shih et al., "cuFINUFFT: a load-balanced GPU library for general-purpose
 *     nonuniform FFTs", IPDPSW 2021: bin sorting of folded points.
 * The call sites that pin the semantics are lib/kernels.cc.cu:25-92
 * (run_nufft), src/jax_finufft/ops.py:159-170 (transform definitions) and
 * src/jax_finufft/ops.py:114-123 (mode ordering).
 *
 * Everything is double precision.  The fold, bin, grid-start and offset
 * arithmetic uses one rounding per operation in a fixed order (built with
 * -ffp-contract=off) so that the CUDA kernels, which use __dmul_rn/__dadd_rn
 * in the same order, produce bit-identical bin indices and offsets.
 *
 * Conventions (shared with the CUDA library):
 *   - dimension 0 ("x") is the fastest-varying grid axis, as in the backend
 *     order that lowering.py:96-105 produces by reversing the user's axes;
 *   - fine grid index l corresponds to coordinate l * 2*pi / nf;
 *   - kernel psi(t) = exp(beta*(sqrt(1-(2t/w)^2)-1)) for |t| <= w/2 in grid
 *     units, zero outside;
 *   - a point at grid coordinate X touches grid indices i0..i0+w-1 with
 *     i0 = ceil(X - w/2); delta = i0 - (X - w/2) lies in [0, 1).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_W 16
#define ORC_PI 3.141592653589793238462643383279502884
#define ORC_INV2PI 0.159154943091895335768883763372514362

/* ----------------------------------------------------------------------- */
/* Plan-time parameters                                                     */
/* ----------------------------------------------------------------------- */

/* Smallest even n >= n0 with prime factors in {2, 3, 5}. */
int64_t orc_next235even(int64_t n0) {
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

/* Kernel width and shape parameter for a requested tolerance.
 * Width rule (published): sigma == 2 gives w = ceil(log10(10/eps)); other
 * sigma gives w = ceil(-ln(eps) / (pi*sqrt(1-1/sigma))).  Shape: beta =
 * 2.30*w at sigma == 2 (2.20, 2.26, 2.38 for w = 2, 3, 4), else
 * beta = 0.97*pi*(1-1/(2*sigma))*w.
 * Kaiser-Bessel (shape 1, an option of the CUDA library) keeps the width
 * rule with beta = pi*sqrt((w/sigma)^2 (sigma-1/2)^2 - 0.8) (Beatty,
 * Nishimura, Pauly, IEEE TMI 2005).
 * Returns 1 when the width had to be clamped at ORC_MAX_W (tolerance not
 * reachable, the reference's FINUFFT_WARN_EPS_TOO_SMALL), else 0. */
int orc_kernel_params(double eps, double sigma, int shape, int *w_out, double *beta_out) {
  int warn = 0;
  double a;
  if (sigma == 2.0)
    a = -log10(eps / 10.0);
  else
    a = -log(eps) / (ORC_PI * sqrt(1.0 - 1.0 / sigma));
  /* a tolerance given in single precision must not gain a width from its
   * rounding: snap to the integer within 1e-5 */
  if (fabs(a - round(a)) < 1e-5) a = round(a);
  double wd = ceil(a);
  if (!(wd >= 2.0)) wd = 2.0;
  if (wd > ORC_MAX_W) {
    wd = ORC_MAX_W;
    warn = 1;
  }
  int w = (int)wd;
  double ratio;
  if (sigma == 2.0) {
    ratio = 2.30;
    if (w == 2) ratio = 2.20;
    if (w == 3) ratio = 2.26;
    if (w == 4) ratio = 2.38;
  } else {
    ratio = 0.97 * ORC_PI * (1.0 - 1.0 / (2.0 * sigma));
  }
  *w_out = w;
  *beta_out = ratio * (double)w;
  if (shape == 1) {
    double a = ((double)w / sigma) * (sigma - 0.5);
    double r = a * a - 0.8;
    *beta_out = ORC_PI * sqrt(r > 0.25 ? r : 0.25);
  }
  return warn;
}

/* Fine-grid size for n modes: next235even(max(ceil(sigma*n), 2w)). */
int64_t orc_fine_size(int64_t nmodes, double sigma, int w) {
  double a = ceil(sigma * (double)nmodes);
  int64_t n = (int64_t)a;
  if (n < 2 * (int64_t)w) n = 2 * (int64_t)w;
  return orc_next235even(n);
}

/* Modified Bessel function I0 by its power series (positive terms). */
static double orc_bessel_i0(double x) {
  double q = 0.25 * x * x, term = 1.0, sum = 1.0;
  for (int k = 1; k < 500; ++k) {
    term *= q / ((double)k * (double)k);
    sum += term;
    if (term < 1e-17 * sum) break;
  }
  return sum;
}

/* The kernel as a function of s = sqrt(1 - (2t/w)^2): shape 0 the ES kernel
 * exp(beta*(s-1)), shape 1 Kaiser-Bessel I0(beta*s)/I0(beta). */
static double orc_kernel_s(double s, double beta, int shape) {
  if (shape == 1) return orc_bessel_i0(beta * s) / orc_bessel_i0(beta);
  return exp(beta * (s - 1.0));
}

/* The kernel at offset t (grid units). */
double orc_kernel(double t, int w, double beta, int shape) {
  double z = 2.0 * t / (double)w;
  double s = 1.0 - z * z;
  if (s < 0.0) return 0.0;
  return orc_kernel_s(sqrt(s), beta, shape);
}

/* Gauss-Legendre nodes/weights on [-1, 1] by Newton iteration on P_q. */
static void orc_gauss_legendre(int q, double *x, double *wt) {
  for (int i = 0; i < (q + 1) / 2; ++i) {
    double z = cos(ORC_PI * (i + 0.75) / (q + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= q; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (q == 1) {
        p1 = z;
        p0 = 1.0;
      }
      dp = q * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) break;
    }
    /* recompute derivative at the converged node */
    {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= q; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = q * (z * p1 - p0) / (z * z - 1.0);
    }
    x[i] = -z;
    x[q - 1 - i] = z;
    wt[i] = wt[q - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

/* Fourier transform of the kernel, psihat(omega) = int psi(t) cos(omega t) dt,
 * by Gauss-Legendre quadrature after the substitution t = (w/2) sin(theta),
 * which removes the square-root endpoint singularity (q = 2w + 10 nodes on
 * [0, pi/2]). */
void orc_kernel_ft(int w, double beta, int shape, int64_t n, const double *omega, double *out) {
  int q = 2 * w + 10;
  double xg[64], wg[64], tq[64], fq[64];
  orc_gauss_legendre(q, xg, wg);
  for (int i = 0; i < q; ++i) {
    double th = (xg[i] + 1.0) * ORC_PI / 4.0;
    double wt = wg[i] * ORC_PI / 4.0;
    tq[i] = 0.5 * w * sin(th);
    fq[i] = 2.0 * wt * orc_kernel_s(cos(th), beta, shape) * 0.5 * w * cos(th);
  }
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < n; ++k) {
    double s = 0.0;
    for (int i = 0; i < q; ++i) s += fq[i] * cos(omega[k] * tq[i]);
    out[k] = s;
  }
}

/* ----------------------------------------------------------------------- */
/* Fold, grid start, bins                                                   */
/* ----------------------------------------------------------------------- */

/* Periodic fold of x (radians) onto grid coordinate X in [0, nf).
 * Non-finite inputs map to 0. */
double orc_fold(double x, int64_t nf) {
  if (!isfinite(x)) return 0.0;
  double t = x * ORC_INV2PI;
  double f = t - floor(t);
  double X = f * (double)nf;
  if (X >= (double)nf) X = X - (double)nf;
  return X;
}

/* Position of a point in fine-grid cells minus w/2: s = X - w/2.
 * mode 0 (periodic fold): t = x/(2 pi), f = t - floor(t), s = fma(f, nf, -w/2).
 * mode 1 (type-3 rescale): s = fma(x - center, scale, nf/2 - w/2).
 * One rounding per operation (fma is a single rounding), the same sequence
 * the CUDA kernels use.  Non-finite x counts as 0 (mode 0) / the centre. */
static double orc_grid_shift(double x, int mode, double center, double scale, int64_t nf, int w) {
  double hw = 0.5 * (double)w;
  if (mode == 0) {
    if (!isfinite(x)) x = 0.0;
    double t = x * ORC_INV2PI;
    double f = t - floor(t);
    return fma(f, (double)nf, -hw);
  }
  double d = isfinite(x) ? x - center : 0.0;
  return fma(d, scale, 0.5 * (double)nf - hw);
}

/* Per point and axis: grid start i0 = ceil(s) (wrapped so that i0 + w/2 lies
 * in [0, nf)), offset delta = i0 - s in [0, 1), and the bin index
 * sum_d ((i0_d + w/2) / B_d) * prod_{e<d} nb_e with nb_d = ceil(nf_d / B_d).
 * X is the folded coordinate s + w/2 (reported for reference).
 * coords[d] may be NULL for d >= dim; center/scale are read for mode 1 only. */
void orc_fold_points(int dim, int mode, int w, const int64_t *nf, const int *binsize, int64_t M,
                     const double *cx, const double *cy, const double *cz,
                     const double *center, const double *scale, double *X, int64_t *i0,
                     double *delta, int64_t *bin) {
  const double *c[3] = {cx, cy, cz};
  int64_t nb[3];
  int h = w / 2;
  for (int d = 0; d < 3; ++d) nb[d] = (d < dim) ? (nf[d] + binsize[d] - 1) / binsize[d] : 1;
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < M; ++j) {
    int64_t b = 0, stride = 1;
    for (int d = 0; d < dim; ++d) {
      double s = orc_grid_shift(c[d][j], mode, mode ? center[d] : 0.0, mode ? scale[d] : 1.0,
                                nf[d], w);
      double cl = ceil(s);
      int64_t s0 = (int64_t)cl;
      int64_t tb = s0 + h;
      if (tb < 0) {
        tb += nf[d];
        s0 += nf[d];
      }
      if (tb >= nf[d]) {
        tb -= nf[d];
        s0 -= nf[d];
      }
      X[j * 3 + d] = s + 0.5 * (double)w;
      i0[j * 3 + d] = s0;
      delta[j * 3 + d] = cl - s;
      b += (tb / binsize[d]) * stride;
      stride *= nb[d];
    }
    for (int d = dim; d < 3; ++d) {
      X[j * 3 + d] = 0.0;
      i0[j * 3 + d] = 0;
      delta[j * 3 + d] = 0.0;
    }
    bin[j] = b;
  }
}

/* ----------------------------------------------------------------------- */
/* Spread (type 1) and interpolate (type 2)                                 */
/* ----------------------------------------------------------------------- */

static inline int64_t wrapi(int64_t i, int64_t n) {
  i %= n;
  return i < 0 ? i + n : i;
}

static void kernel_values(double delta, int w, double beta, int shape, double *k) {
  for (int j = 0; j < w; ++j) k[j] = orc_kernel((double)j - 0.5 * w + delta, w, beta, shape);
}

/* grid (complex interleaved, nf[0]*nf[1]*nf[2] cells, x fastest) +=
 *   sum_j c_j psi(l - X_j) over the w^dim cells each point touches.
 * Parallel over slabs of the slowest used axis; each thread owns a slab and
 * clips every point's support to it, so the result is deterministic.
 * X/i0/delta are the per-point outputs of orc_fold_points. */
void orc_spread(int dim, const int64_t *nf, int w, double beta, int shape, int64_t M,
                const int64_t *i0,
                const double *delta, const double *c, double *grid) {
  int slow = dim - 1;
  int64_t nslow = nf[slow];
  int64_t plane = 1;
  for (int d = 0; d < slow; ++d) plane *= nf[d];
  int nthr = 1;
#ifdef _OPENMP
  nthr = omp_get_max_threads();
#endif
  int64_t nslab = nthr * 4;
  if (nslab > nslow) nslab = nslow;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t sl = 0; sl < nslab; ++sl) {
    int64_t lo = sl * nslow / nslab, hi = (sl + 1) * nslow / nslab;
    double kv[3][ORC_MAX_W];
    for (int64_t j = 0; j < M; ++j) {
      int64_t s0 = i0[j * 3 + slow];
      /* does [s0, s0+w) mod nslow meet [lo, hi)? */
      int hit = 0;
      for (int q = 0; q < w; ++q) {
        int64_t g = wrapi(s0 + q, nslow);
        if (g >= lo && g < hi) {
          hit = 1;
          break;
        }
      }
      if (!hit) continue;
      for (int d = 0; d < dim; ++d) kernel_values(delta[j * 3 + d], w, beta, shape, kv[d]);
      double cr = c[2 * j], ci = c[2 * j + 1];
      for (int qs = 0; qs < w; ++qs) {
        int64_t gs = wrapi(s0 + qs, nslow);
        if (gs < lo || gs >= hi) continue;
        double ks = kv[slow][qs];
        if (dim == 1) {
          grid[2 * gs] += cr * ks;
          grid[2 * gs + 1] += ci * ks;
        } else if (dim == 2) {
          int64_t base = gs * plane;
          for (int qx = 0; qx < w; ++qx) {
            int64_t gx = wrapi(i0[j * 3 + 0] + qx, nf[0]);
            double kk = ks * kv[0][qx];
            grid[2 * (base + gx)] += cr * kk;
            grid[2 * (base + gx) + 1] += ci * kk;
          }
        } else {
          int64_t base = gs * plane;
          for (int qy = 0; qy < w; ++qy) {
            int64_t gy = wrapi(i0[j * 3 + 1] + qy, nf[1]);
            double kyz = ks * kv[1][qy];
            for (int qx = 0; qx < w; ++qx) {
              int64_t gx = wrapi(i0[j * 3 + 0] + qx, nf[0]);
              double kk = kyz * kv[0][qx];
              int64_t idx = base + gy * nf[0] + gx;
              grid[2 * idx] += cr * kk;
              grid[2 * idx + 1] += ci * kk;
            }
          }
        }
      }
    }
  }
}

/* c_j = sum over the w^dim touched cells of grid(l) psi(l - X_j). */
void orc_interp(int dim, const int64_t *nf, int w, double beta, int shape, int64_t M,
                const int64_t *i0,
                const double *delta, const double *grid, double *c) {
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < M; ++j) {
    double kv[3][ORC_MAX_W];
    for (int d = 0; d < 3; ++d)
      for (int q = 0; q < ORC_MAX_W; ++q) kv[d][q] = (d == 0 || q == 0) ? 1.0 : 0.0;
    for (int d = 0; d < dim; ++d) kernel_values(delta[j * 3 + d], w, beta, shape, kv[d]);
    int wy = dim >= 2 ? w : 1, wz = dim >= 3 ? w : 1;
    double sr = 0.0, si = 0.0;
    for (int qz = 0; qz < wz; ++qz) {
      int64_t gz = dim >= 3 ? wrapi(i0[j * 3 + 2] + qz, nf[2]) : 0;
      for (int qy = 0; qy < wy; ++qy) {
        int64_t gy = dim >= 2 ? wrapi(i0[j * 3 + 1] + qy, nf[1]) : 0;
        double kyz = (dim >= 3 ? kv[2][qz] : 1.0) * (dim >= 2 ? kv[1][qy] : 1.0);
        int64_t base = (gz * nf[1] + gy) * nf[0];
        double rr = 0.0, ri = 0.0;
        for (int qx = 0; qx < w; ++qx) {
          int64_t gx = wrapi(i0[j * 3 + 0] + qx, nf[0]);
          rr += grid[2 * (base + gx)] * kv[0][qx];
          ri += grid[2 * (base + gx) + 1] * kv[0][qx];
        }
        sr += rr * kyz;
        si += ri * kyz;
      }
    }
    c[2 * j] = sr;
    c[2 * j + 1] = si;
  }
}

/* Piecewise-polynomial fit of the kernel, the same scheme the CUDA library
 * uses at plan time (Chebyshev interpolation of each unit piece at degree
 * `deg`, converted to monomials in u = 2*delta - 1).  coef[j*(deg+1)+n] is
 * the coefficient of u^n on piece j.  Exposed so the tests can check the fit
 * error against the exact kernel. */
void orc_horner_fit(int w, double beta, int shape, int deg, double *coef) {
  int n1 = deg + 1;
  double node[32], val[32], cheb[32], mono[32], tk[32][32];
  for (int i = 0; i < n1; ++i) node[i] = cos(ORC_PI * (i + 0.5) / n1);
  /* monomial coefficients of Chebyshev T_k: T_0 = 1, T_1 = u, T_k = 2u T_{k-1} - T_{k-2} */
  memset(tk, 0, sizeof(tk));
  tk[0][0] = 1.0;
  if (n1 > 1) tk[1][1] = 1.0;
  for (int k = 2; k < n1; ++k)
    for (int n = 0; n < n1; ++n) tk[k][n] = (n ? 2.0 * tk[k - 1][n - 1] : 0.0) - tk[k - 2][n];
  for (int j = 0; j < w; ++j) {
    for (int i = 0; i < n1; ++i)
      val[i] = orc_kernel((double)j - 0.5 * w + 0.5 * (node[i] + 1.0), w, beta, shape);
    for (int k = 0; k < n1; ++k) {
      double s = 0.0;
      for (int i = 0; i < n1; ++i) s += val[i] * cos(ORC_PI * k * (i + 0.5) / n1);
      cheb[k] = s * (k == 0 ? 1.0 : 2.0) / n1;
    }
    for (int n = 0; n < n1; ++n) {
      double s = 0.0;
      for (int k = 0; k < n1; ++k) s += cheb[k] * tk[k][n];
      mono[n] = s;
    }
    for (int n = 0; n < n1; ++n) coef[j * n1 + n] = mono[n];
  }
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* Type-3 grid parameters for one dimension (published rescaling).
 * Sources lie in [xmin, xmax], targets in [smin, smax].  With half-widths
 * X = (xmax-xmin)/2, S = (smax-smin)/2 (each kept >= 1/other so X*S >= 1),
 * the spreading grid has nf = next235even(max(floor(2*sigma*S*X/pi + w + 1),
 * 2w)) cells; a source maps to grid coordinate (x - cx)*scale + nf/2 with
 * scale = sigma*S/pi, and a target maps to the inner type-2 point
 * (s - cs)/scale (radians, inside [-pi/sigma, pi/sigma]).
 * out[0] = cx, out[1] = cs, out[2] = scale; returns nf. */
int64_t orc_type3_params(double xmin, double xmax, double smin, double smax, double sigma, int w,
                         double *out) {
  double cx = 0.5 * (xmax + xmin), hx = 0.5 * (xmax - xmin);
  double cs = 0.5 * (smax + smin), hs = 0.5 * (smax - smin);
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
  double nfd = 2.0 * sigma * S * X / ORC_PI + (double)(w + 1);
  if (!isfinite(nfd)) nfd = 0.0;
  int64_t nf = (int64_t)nfd;
  if (nf < 2 * (int64_t)w) nf = 2 * (int64_t)w;
  nf = orc_next235even(nf);
  out[0] = cx;
  out[1] = cs;
  out[2] = sigma * S / ORC_PI;
  return nf;
}

/* ----------------------------------------------------------------------- */
/* Single-precision fast path: the timed CPU baseline                       */
/* ----------------------------------------------------------------------- */
/* Not a checker: the FP64 routines above are the oracle.  These restate
 * the CPU method of the paper cited at the top of this file (section 3 of
 * Barnett, Magland, af Klinteberg 2019) in single precision, as FINUFFT runs
 * complex64 transforms: kernel values from the piecewise polynomials of
 * orc_horner_fit evaluated by Horner's rule, points bin-sorted for locality,
 * each bin spread by one thread into a private padded subgrid that is then
 * added to the fine grid.  Bins are coloured by the parity of their index
 * along every axis; bins of one colour are two bins apart, so their
 * subgrids never overlap when the bin size is at least w - 1 and the adds
 * need no atomics.  The eight colours run one after another. */

typedef struct {
  int dim, w, deg;
  int64_t nf[3], bs[3], nb[3];
  float coef[ORC_MAX_W * 24]; /* coef[n * w + j]: u^n on piece j (j contiguous) */
} orc_f32_geom;

static void f32_geom(orc_f32_geom *g, int dim, const int64_t *nf, int w, int deg,
                     const double *coef) {
  g->dim = dim;
  g->w = w;
  g->deg = deg;
  for (int d = 0; d < 3; ++d) {
    g->nf[d] = d < dim ? nf[d] : 1;
    /* an even number of equal bins of >= max(16, w - 1) cells where the axis
     * allows (equal bins keep the colouring valid across the periodic wrap),
     * else one bin */
    int64_t nb = 1;
    if (d < dim)
      for (int64_t k = g->nf[d] / 16; k >= 2; --k)
        if (k % 2 == 0 && g->nf[d] % k == 0 && g->nf[d] / k >= w - 1) {
          nb = k;
          break;
        }
    g->nb[d] = nb;
    g->bs[d] = g->nf[d] / nb;
  }
  for (int j = 0; j < w; ++j)
    for (int n = 0; n <= deg; ++n) g->coef[n * w + j] = (float)coef[j * (deg + 1) + n];
}

/* All w kernel values of one axis by Horner's rule, the pieces side by
 * side (the inner loop over pieces vectorises). */
static inline void f32_kernel(const orc_f32_geom *g, float delta, float *k) {
  const int w = g->w;
  const float u = 2.0f * delta - 1.0f;
  const float *c = g->coef + g->deg * w;
  for (int j = 0; j < w; ++j) k[j] = c[j];
  for (int n = g->deg - 1; n >= 0; --n) {
    c -= w;
    for (int j = 0; j < w; ++j) k[j] = k[j] * u + c[j];
  }
}

static inline int64_t f32_bin(const orc_f32_geom *g, const int64_t *i0) {
  int64_t b = 0;
  for (int d = g->dim - 1; d >= 0; --d) b = b * g->nb[d] + wrapi(i0[d], g->nf[d]) / g->bs[d];
  return b;
}

/* Counting sort of the points by bin: start[nbins + 1] and perm[M]. */
static void f32_sort(const orc_f32_geom *g, int64_t M, const int64_t *i0, int64_t *start,
                     int64_t *perm) {
  const int64_t nbins = g->nb[0] * g->nb[1] * g->nb[2];
  int64_t *bin = (int64_t *)malloc(sizeof(int64_t) * (M > 0 ? M : 1));
  memset(start, 0, sizeof(int64_t) * (nbins + 1));
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < M; ++j) bin[j] = f32_bin(g, i0 + 3 * j);
  for (int64_t j = 0; j < M; ++j) start[bin[j] + 1]++;
  for (int64_t b = 0; b < nbins; ++b) start[b + 1] += start[b];
  int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (nbins > 0 ? nbins : 1));
  memcpy(fill, start, sizeof(int64_t) * nbins);
  for (int64_t j = 0; j < M; ++j) perm[fill[bin[j]]++] = j;
  free(fill);
  free(bin);
}

/* grid (complex64 interleaved, x fastest) += spread of c (complex64) at the
 * folded points (i0, delta as float). */
void orc_spread_f32(int dim, const int64_t *nf, int w, int deg, const double *coef, int64_t M,
                    const int64_t *i0, const float *delta, const float *c, float *grid) {
  orc_f32_geom g;
  f32_geom(&g, dim, nf, w, deg, coef);
  const int64_t nbins = g.nb[0] * g.nb[1] * g.nb[2];
  int64_t *start = (int64_t *)malloc(sizeof(int64_t) * (nbins + 1));
  int64_t *perm = (int64_t *)malloc(sizeof(int64_t) * (M > 0 ? M : 1));
  f32_sort(&g, M, i0, start, perm);
  int64_t T[3];
  for (int d = 0; d < 3; ++d) T[d] = d < dim ? g.bs[d] + w - 1 : 1;
  const int64_t sub_cells = T[0] * T[1] * T[2];
  const int ncol = (g.nb[0] > 1 ? 2 : 1) * (g.nb[1] > 1 ? 2 : 1) * (g.nb[2] > 1 ? 2 : 1);
#pragma omp parallel
  {
    float *sub = (float *)malloc(sizeof(float) * 2 * sub_cells);
    float kv[3][ORC_MAX_W];
    for (int col = 0; col < ncol; ++col) {
#pragma omp for schedule(dynamic, 4)
      for (int64_t b = 0; b < nbins; ++b) {
        int64_t bc[3] = {b % g.nb[0], (b / g.nb[0]) % g.nb[1], b / (g.nb[0] * g.nb[1])};
        int cb = 0, m = 1;
        for (int d = 0; d < 3; ++d)
          if (g.nb[d] > 1) {
            cb += (int)(bc[d] & 1) * m;
            m *= 2;
          }
        if (cb != col || start[b + 1] == start[b]) continue;
        memset(sub, 0, sizeof(float) * 2 * sub_cells);
        int64_t lo[3];
        for (int d = 0; d < 3; ++d) lo[d] = bc[d] * g.bs[d];
        for (int64_t s = start[b]; s < start[b + 1]; ++s) {
          const int64_t j = perm[s];
          for (int d = 0; d < 3; ++d) {
            kv[d][0] = 1.0f;
            if (d < dim) f32_kernel(&g, delta[3 * j + d], kv[d]);
          }
          int64_t o[3];
          for (int d = 0; d < 3; ++d) o[d] = d < dim ? wrapi(i0[3 * j + d], g.nf[d]) - lo[d] : 0;
          const float cr = c[2 * j], ci = c[2 * j + 1];
          const int wy = dim > 1 ? w : 1, wz = dim > 2 ? w : 1;
          for (int qz = 0; qz < wz; ++qz)
            for (int qy = 0; qy < wy; ++qy) {
              const float kyz = kv[1][qy] * kv[2][qz];
              const float vr = cr * kyz, vi = ci * kyz;
              float *row = sub + 2 * (((o[2] + qz) * T[1] + (o[1] + qy)) * T[0] + o[0]);
              for (int qx = 0; qx < w; ++qx) {
                row[2 * qx] += vr * kv[0][qx];
                row[2 * qx + 1] += vi * kv[0][qx];
              }
            }
        }
        /* x: the part before the wrap, then the wrapped part */
        const int64_t x_run = lo[0] + T[0] <= g.nf[0] ? T[0] : g.nf[0] - lo[0];
        for (int64_t z = 0; z < T[2]; ++z)
          for (int64_t y = 0; y < T[1]; ++y) {
            const int64_t gz = dim > 2 ? wrapi(lo[2] + z, g.nf[2]) : 0;
            const int64_t gy = dim > 1 ? wrapi(lo[1] + y, g.nf[1]) : 0;
            float *dst = grid + 2 * ((gz * g.nf[1] + gy) * g.nf[0]);
            const float *src = sub + 2 * ((z * T[1] + y) * T[0]);
            float *d0 = dst + 2 * lo[0];
            for (int64_t x = 0; x < 2 * x_run; ++x) d0[x] += src[x];
            for (int64_t x = x_run; x < T[0]; ++x) {
              const int64_t gx = wrapi(lo[0] + x, g.nf[0]);
              dst[2 * gx] += src[2 * x];
              dst[2 * gx + 1] += src[2 * x + 1];
            }
          }
      }
    }
    free(sub);
  }
  free(perm);
  free(start);
}

/* c (complex64) = interpolation of grid (complex64) at the folded points,
 * visited in bin order for locality. */
void orc_interp_f32(int dim, const int64_t *nf, int w, int deg, const double *coef, int64_t M,
                    const int64_t *i0, const float *delta, const float *grid, float *c) {
  orc_f32_geom g;
  f32_geom(&g, dim, nf, w, deg, coef);
  const int64_t nbins = g.nb[0] * g.nb[1] * g.nb[2];
  int64_t *start = (int64_t *)malloc(sizeof(int64_t) * (nbins + 1));
  int64_t *perm = (int64_t *)malloc(sizeof(int64_t) * (M > 0 ? M : 1));
  f32_sort(&g, M, i0, start, perm);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t s = 0; s < M; ++s) {
    const int64_t j = perm[s];
    float kv[3][ORC_MAX_W];
    for (int d = 0; d < 3; ++d) {
      kv[d][0] = 1.0f;
      if (d < dim) f32_kernel(&g, delta[3 * j + d], kv[d]);
    }
    const int wy = dim > 1 ? w : 1, wz = dim > 2 ? w : 1;
    int64_t gx[ORC_MAX_W];
    for (int q = 0; q < w; ++q) gx[q] = 2 * wrapi(i0[3 * j] + q, g.nf[0]);
    float sr = 0.0f, si = 0.0f;
    for (int qz = 0; qz < wz; ++qz) {
      const int64_t gz = dim > 2 ? wrapi(i0[3 * j + 2] + qz, g.nf[2]) : 0;
      for (int qy = 0; qy < wy; ++qy) {
        const int64_t gy = dim > 1 ? wrapi(i0[3 * j + 1] + qy, g.nf[1]) : 0;
        const float *row = grid + 2 * ((gz * g.nf[1] + gy) * g.nf[0]);
        float rr = 0.0f, ri = 0.0f;
        for (int qx = 0; qx < w; ++qx) {
          rr += row[gx[qx]] * kv[0][qx];
          ri += row[gx[qx] + 1] * kv[0][qx];
        }
        const float kyz = kv[1][qy] * kv[2][qz];
        sr += rr * kyz;
        si += ri * kyz;
      }
    }
    c[2 * j] = sr;
    c[2 * j + 1] = si;
  }
  free(perm);
  free(start);
}

/* Deconvolution between the modes and the fine grid, single precision.
 * Modes f (complex64, user axis order = backend reversed: x fastest) of
 * n[0] x n[1] x n[2] entries; fine grid of nf[0] x nf[1] x nf[2]; mode k of
 * axis d (storage index i) sits at grid index idx_d[i] and is scaled by
 * fac_d[i].  dir = 1: grid = 0 except grid[idx] = f * fac (type 2);
 * dir = -1: f = grid[idx] * fac (type 1). */
void orc_deconv_f32(int dir, int dim, const int64_t *n, const int64_t *nf, const int64_t *idx0,
                    const int64_t *idx1, const int64_t *idx2, const float *fac0,
                    const float *fac1, const float *fac2, float *f, float *grid) {
  const int64_t n1 = dim > 1 ? n[1] : 1, n2 = dim > 2 ? n[2] : 1;
  const int64_t g1 = dim > 1 ? nf[1] : 1, g2 = dim > 2 ? nf[2] : 1;
  if (dir > 0) {
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < g1 * g2; ++r) memset(grid + 2 * r * nf[0], 0, sizeof(float) * 2 * nf[0]);
  }
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t k2 = 0; k2 < n2; ++k2)
    for (int64_t k1 = 0; k1 < n1; ++k1) {
      const float s = (dim > 2 ? fac2[k2] : 1.0f) * (dim > 1 ? fac1[k1] : 1.0f);
      const int64_t grow = ((dim > 2 ? idx2[k2] : 0) * g1 + (dim > 1 ? idx1[k1] : 0)) * nf[0];
      float *fr = f + 2 * ((k2 * n1 + k1) * n[0]);
      float *gr = grid + 2 * grow;
      for (int64_t k0 = 0; k0 < n[0]; ++k0) {
        const float a = s * fac0[k0];
        const int64_t gi = 2 * idx0[k0];
        if (dir > 0) {
          gr[gi] = fr[2 * k0] * a;
          gr[gi + 1] = fr[2 * k0 + 1] * a;
        } else {
          fr[2 * k0] = gr[gi] * a;
          fr[2 * k0 + 1] = gr[gi + 1] * a;
        }
      }
    }
}
