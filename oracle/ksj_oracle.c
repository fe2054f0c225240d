/*
 * ksj_oracle.c -- CPU restatement of KSpaceJet's non-Cartesian reconstruction
 * arithmetic.  TEST INFRASTRUCTURE ONLY: this file is the parity checker for
 * the CUDA path.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it; nothing in kspacejet_gb300/ links or calls it.
 *
 * Every function names the reference file:line whose algorithm it restates
 * (paths relative to the KSpaceJet source tree).  The single-precision forms
 * follow the reference's operation order and rounding points one for one
 * (compile with -ffp-contract=off, as an ISO C++20 build of the reference
 * does), so on the same host they reproduce the reference's float results
 * bit for bit; tests/test_oracle_golden.py pins that against the compiled
 * reference and against the reference tests' known answers.
 *
 * The Kaiser-Bessel forms have no counterpart in the reference.  They restate
 * the published gridding method (Jackson, Meyer, Nishimura, Macovski, IEEE TMI
 * 1991; Beatty, Nishimura, Pauly, IEEE TMI 2005) in double precision, with the
 * conventions of the CUDA path (tap set, normalisation, half-pixel centring)
 * written out below.  Their parity is unpinned by the reference; they are
 * checked against the exact direct NUDFT instead.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define KSJO_EXPORT __attribute__((visibility("default")))

static const float kPiF = 3.14159265358979323846f; /* std::numbers::pi_v<float> */
static const double kPiD = 3.14159265358979323846;

/* ---------------------------------------------------------------- complex */

typedef struct { float re, im; } cf32;
typedef struct { double re, im; } cf64;

/* std::complex<T>::operator*= for finite operands: (ac - bd) + (ad + bc)i,
 * four products rounded separately (no contraction). */
static inline cf32 cmul_f(cf32 a, cf32 b) {
  const float ac = a.re * b.re, bd = a.im * b.im, ad = a.re * b.im, bc = a.im * b.re;
  cf32 r = {ac - bd, ad + bc};
  return r;
}
static inline cf64 cmul_d(cf64 a, cf64 b) {
  const double ac = a.re * b.re, bd = a.im * b.im, ad = a.re * b.im, bc = a.im * b.re;
  cf64 r = {ac - bd, ad + bc};
  return r;
}
static inline cf32 cscale_f(cf32 a, float s) { cf32 r = {a.re * s, a.im * s}; return r; }
static inline cf64 cscale_d(cf64 a, double s) { cf64 r = {a.re * s, a.im * s}; return r; }
static inline cf32 cadd_f(cf32 a, cf32 b) { cf32 r = {a.re + b.re, a.im + b.im}; return r; }
static inline cf32 csub_f(cf32 a, cf32 b) { cf32 r = {a.re - b.re, a.im - b.im}; return r; }
static inline cf64 cadd_d(cf64 a, cf64 b) { cf64 r = {a.re + b.re, a.im + b.im}; return r; }
static inline cf64 csub_d(cf64 a, cf64 b) { cf64 r = {a.re - b.re, a.im - b.im}; return r; }

static int is_pow2(int64_t n) { return n > 0 && (n & (n - 1)) == 0; }

/* ------------------------------------------------------------ ramp DCF */

/* radial_analytic_ramp_dcf2: w = hypot(k_row, k_col); trajectory must be
 * finite and inside [-pi, pi].
 * libs/numerics/kspacejet-nufft/src/eigen/eigen_radial_gridding.cpp:279-295
 * (validation :106-123).  Returns 0, or -1 when the reference would throw. */
KSJO_EXPORT int ksjo_ramp_dcf2_f32(const float* traj, int64_t m, float* dcf) {
  for (int64_t s = 0; s < m; ++s) {
    const float r = traj[2 * s], c = traj[2 * s + 1];
    if (!isfinite(r) || !isfinite(c) || r < -kPiF || r > kPiF || c < -kPiF || c > kPiF) return -1;
  }
  for (int64_t s = 0; s < m; ++s) dcf[s] = hypotf(traj[2 * s], traj[2 * s + 1]);
  return 0;
}

KSJO_EXPORT int ksjo_ramp_dcf2_f64(const double* traj, int64_t m, double* dcf) {
  for (int64_t s = 0; s < m; ++s) {
    const double r = traj[2 * s], c = traj[2 * s + 1];
    if (!isfinite(r) || !isfinite(c) || r < -kPiD || r > kPiD || c < -kPiD || c > kPiD) return -1;
  }
  for (int64_t s = 0; s < m; ++s) dcf[s] = hypot(traj[2 * s], traj[2 * s + 1]);
  return 0;
}

/* --------------------------------------------------------- grid coordinate */

/* grid_coordinate: x = f * N / (2 pi), wrapped once into [0, N);
 * lower = floor(x), frac = x - lower.
 * eigen_radial_gridding.cpp:262-277.  The integer `lower` is the binning key
 * the CUDA path must reproduce bit for bit. */
KSJO_EXPORT int ksjo_grid_coordinate_f32(float f, int64_t extent, int64_t* lower, float* frac) {
  const float n = (float)extent;
  float x = f * n / (2.0f * kPiF);
  if (x < 0.0f) x += n;
  if (x >= n) x -= n;
  if (!isfinite(x) || x < 0.0f || x >= n) return -1;
  const int64_t lo = (int64_t)floorf(x);
  *lower = lo;
  *frac = x - (float)lo;
  return 0;
}

KSJO_EXPORT int ksjo_grid_coordinate_f64(double f, int64_t extent, int64_t* lower, double* frac) {
  const double n = (double)extent;
  double x = f * n / (2.0 * kPiD);
  if (x < 0.0) x += n;
  if (x >= n) x -= n;
  if (!isfinite(x) || x < 0.0 || x >= n) return -1;
  const int64_t lo = (int64_t)floor(x);
  *lower = lo;
  *frac = x - (double)lo;
  return 0;
}

/* ------------------------------------------------------ line transforms */

static int64_t reversed_radix2_index(int64_t index, int64_t length) {
  int64_t reversed = 0, source = index;
  for (int64_t remaining = length; remaining > 1; remaining >>= 1) {
    reversed = (reversed << 1) | (source & 1);
    source >>= 1;
  }
  return reversed;
}

/* Unnormalised inverse DFT exp(+2 pi i k n / N): radix-2 with a per-stage
 * twiddle recurrence for powers of two, the O(N^2) direct sum with a phase
 * recurrence otherwise.  eigen_radial_gridding.cpp:145-211. */
KSJO_EXPORT void ksjo_inverse_transform_f32(const float* src_in, float* dst_out, int64_t n) {
  const cf32* src = (const cf32*)src_in;
  cf32* dst = (cf32*)dst_out;
  if (is_pow2(n)) {
    if (n == 1) { dst[0] = src[0]; return; }
    for (int64_t i = 0; i < n; ++i) dst[reversed_radix2_index(i, n)] = src[i];
    for (int64_t stage = 2;; stage <<= 1) {
      const float angle = (2.0f * kPiF) / (float)stage;
      const cf32 step = {cosf(angle), sinf(angle)};
      const int64_t half = stage / 2;
      for (int64_t block = 0; block < n; block += stage) {
        cf32 phase = {1.0f, 0.0f};
        for (int64_t off = 0; off < half; ++off) {
          const cf32 even = dst[block + off];
          const cf32 odd = cmul_f(dst[block + off + half], phase);
          dst[block + off] = cadd_f(even, odd);
          dst[block + off + half] = csub_f(even, odd);
          phase = cmul_f(phase, step);
        }
      }
      if (stage == n) return;
    }
  }
  const float len = (float)n;
  for (int64_t k = 0; k < n; ++k) {
    const float angle = (2.0f * kPiF * (float)k) / len;
    const cf32 step = {cosf(angle), sinf(angle)};
    cf32 phase = {1.0f, 0.0f}, sum = {0.0f, 0.0f};
    for (int64_t i = 0; i < n; ++i) {
      sum = cadd_f(sum, cmul_f(src[i], phase));
      phase = cmul_f(phase, step);
    }
    dst[k] = sum;
  }
}

KSJO_EXPORT void ksjo_inverse_transform_f64(const double* src_in, double* dst_out, int64_t n) {
  const cf64* src = (const cf64*)src_in;
  cf64* dst = (cf64*)dst_out;
  if (is_pow2(n)) {
    if (n == 1) { dst[0] = src[0]; return; }
    for (int64_t i = 0; i < n; ++i) dst[reversed_radix2_index(i, n)] = src[i];
    for (int64_t stage = 2;; stage <<= 1) {
      const double angle = (2.0 * kPiD) / (double)stage;
      const cf64 step = {cos(angle), sin(angle)};
      const int64_t half = stage / 2;
      for (int64_t block = 0; block < n; block += stage) {
        cf64 phase = {1.0, 0.0};
        for (int64_t off = 0; off < half; ++off) {
          const cf64 even = dst[block + off];
          const cf64 odd = cmul_d(dst[block + off + half], phase);
          dst[block + off] = cadd_d(even, odd);
          dst[block + off + half] = csub_d(even, odd);
          phase = cmul_d(phase, step);
        }
      }
      if (stage == n) return;
    }
  }
  const double len = (double)n;
  for (int64_t k = 0; k < n; ++k) {
    const double angle = (2.0 * kPiD * (double)k) / len;
    const cf64 step = {cos(angle), sin(angle)};
    cf64 phase = {1.0, 0.0}, sum = {0.0, 0.0};
    for (int64_t i = 0; i < n; ++i) {
      sum = cadd_d(sum, cmul_d(src[i], phase));
      phase = cmul_d(phase, step);
    }
    dst[k] = sum;
  }
}

/* Exact (table-free, recurrence-free) inverse DFT in double for any length:
 * mixed radix 2/3/5 recursion with directly evaluated twiddles, direct sum for
 * other prime factors.  Used by the Kaiser-Bessel oracle, which has no
 * reference transform to follow. */
static void exact_idft_d(const cf64* x, cf64* y, int64_t n, int64_t stride, cf64* scratch) {
  if (n == 1) { y[0] = x[0]; return; }
  int64_t p = 0;
  for (int64_t f = 2; f <= 5; ++f) if (n % f == 0) { p = f; break; }
  if (p == 0) {
    for (int64_t k = 0; k < n; ++k) {
      cf64 sum = {0.0, 0.0};
      for (int64_t i = 0; i < n; ++i) {
        const double a = 2.0 * kPiD * (double)((k * i) % n) / (double)n;
        const cf64 w = {cos(a), sin(a)};
        sum = cadd_d(sum, cmul_d(x[i * stride], w));
      }
      y[k] = sum;
    }
    return;
  }
  const int64_t m = n / p;
  /* sub-transforms of the p decimated sequences, stored in scratch[r*m + k] */
  cf64* sub = scratch;
  cf64* deeper = scratch + n;
  for (int64_t r = 0; r < p; ++r) exact_idft_d(x + r * stride, sub + r * m, m, stride * p, deeper);
  for (int64_t k = 0; k < n; ++k) {
    cf64 sum = {0.0, 0.0};
    for (int64_t r = 0; r < p; ++r) {
      const double a = 2.0 * kPiD * (double)((r * k) % n) / (double)n;
      const cf64 w = {cos(a), sin(a)};
      sum = cadd_d(sum, cmul_d(sub[r * m + (k % m)], w));
    }
    y[k] = sum;
  }
}

KSJO_EXPORT void ksjo_exact_idft_f64(const double* src, double* dst, int64_t n) {
  cf64* scratch = (cf64*)calloc((size_t)(4 * n + 64), sizeof(cf64));
  exact_idft_d((const cf64*)src, (cf64*)dst, n, 1, scratch);
  free(scratch);
}

/* Separable 2-D inverse transform in place: rows, then columns. */
static void idft2_rows_cols_f32(cf32* image, int64_t rows, int64_t cols) {
  const int64_t line = rows > cols ? rows : cols;
  cf32* src = (cf32*)malloc((size_t)line * sizeof(cf32));
  cf32* dst = (cf32*)malloc((size_t)line * sizeof(cf32));
  cf32* inter = (cf32*)malloc((size_t)(rows * cols) * sizeof(cf32));
  for (int64_t r = 0; r < rows; ++r) {
    for (int64_t c = 0; c < cols; ++c) src[c] = image[r * cols + c];
    ksjo_inverse_transform_f32((const float*)src, (float*)dst, cols);
    for (int64_t c = 0; c < cols; ++c) inter[r * cols + c] = dst[c];
  }
  for (int64_t c = 0; c < cols; ++c) {
    for (int64_t r = 0; r < rows; ++r) src[r] = inter[r * cols + c];
    ksjo_inverse_transform_f32((const float*)src, (float*)dst, rows);
    for (int64_t r = 0; r < rows; ++r) image[r * cols + c] = dst[r];
  }
  free(src); free(dst); free(inter);
}

static void idft2_rows_cols_f64(cf64* image, int64_t rows, int64_t cols, int exact) {
  const int64_t line = rows > cols ? rows : cols;
  cf64* src = (cf64*)malloc((size_t)line * sizeof(cf64));
  cf64* dst = (cf64*)malloc((size_t)line * sizeof(cf64));
  cf64* inter = (cf64*)malloc((size_t)(rows * cols) * sizeof(cf64));
  for (int64_t r = 0; r < rows; ++r) {
    for (int64_t c = 0; c < cols; ++c) src[c] = image[r * cols + c];
    if (exact) ksjo_exact_idft_f64((const double*)src, (double*)dst, cols);
    else ksjo_inverse_transform_f64((const double*)src, (double*)dst, cols);
    for (int64_t c = 0; c < cols; ++c) inter[r * cols + c] = dst[c];
  }
  for (int64_t c = 0; c < cols; ++c) {
    for (int64_t r = 0; r < rows; ++r) src[r] = inter[r * cols + c];
    if (exact) ksjo_exact_idft_f64((const double*)src, (double*)dst, rows);
    else ksjo_inverse_transform_f64((const double*)src, (double*)dst, rows);
    for (int64_t r = 0; r < rows; ++r) image[r * cols + c] = dst[r];
  }
  free(src); free(dst); free(inter);
}

/* ------------------------------------------------------- linear gridding */

/* Scatter stage of radial_linear_gridding2_adjoint: clear the grid, then per
 * sample in order: two grid coordinates, origin phase
 * e = (cos p, sin p) with p = -(k_row*row_origin + k_col*col_origin), the
 * weighted sample (y * dcf) * e, and four periodic bilinear adds.
 * eigen_radial_gridding.cpp:297-343 (origins cast to float :320-321).
 * Returns 0, or -1 where the reference throws (non-finite sample, negative or
 * non-finite DCF, unmappable coordinate). */
KSJO_EXPORT int ksjo_linear_grid2_f32(int64_t rows, int64_t cols, double row_origin, double col_origin,
                                      const float* samples_in, const float* traj, const float* dcf, int64_t m,
                                      float* grid_out) {
  const cf32* samples = (const cf32*)samples_in;
  cf32* grid = (cf32*)grid_out;
  for (int64_t s = 0; s < m; ++s) {
    if (!isfinite(samples[s].re) || !isfinite(samples[s].im)) return -1;
    if (!isfinite(dcf[s]) || dcf[s] < 0.0f) return -1;
  }
  memset(grid, 0, (size_t)(rows * cols) * sizeof(cf32));
  const float ro = (float)row_origin, co = (float)col_origin;
  for (int64_t s = 0; s < m; ++s) {
    const float kr = traj[2 * s], kc = traj[2 * s + 1];
    int64_t rl, cl;
    float rf, cfr;
    if (ksjo_grid_coordinate_f32(kr, rows, &rl, &rf) != 0) return -1;
    if (ksjo_grid_coordinate_f32(kc, cols, &cl, &cfr) != 0) return -1;
    const int64_t ru = (rl + 1) % rows, cu = (cl + 1) % cols;
    const float phase = -(kr * ro + kc * co);
    if (!isfinite(phase)) return -1;
    const cf32 e = {cosf(phase), sinf(phase)};
    const cf32 ws = cmul_f(cscale_f(samples[s], dcf[s]), e);
    const float rlw = 1.0f - rf, clw = 1.0f - cfr;
    grid[rl * cols + cl] = cadd_f(grid[rl * cols + cl], cscale_f(ws, rlw * clw));
    grid[rl * cols + cu] = cadd_f(grid[rl * cols + cu], cscale_f(ws, rlw * cfr));
    grid[ru * cols + cl] = cadd_f(grid[ru * cols + cl], cscale_f(ws, rf * clw));
    grid[ru * cols + cu] = cadd_f(grid[ru * cols + cu], cscale_f(ws, rf * cfr));
  }
  return 0;
}

KSJO_EXPORT int ksjo_linear_grid2_f64(int64_t rows, int64_t cols, double row_origin, double col_origin,
                                      const double* samples_in, const double* traj, const double* dcf, int64_t m,
                                      double* grid_out) {
  const cf64* samples = (const cf64*)samples_in;
  cf64* grid = (cf64*)grid_out;
  for (int64_t s = 0; s < m; ++s) {
    if (!isfinite(samples[s].re) || !isfinite(samples[s].im)) return -1;
    if (!isfinite(dcf[s]) || dcf[s] < 0.0) return -1;
  }
  memset(grid, 0, (size_t)(rows * cols) * sizeof(cf64));
  for (int64_t s = 0; s < m; ++s) {
    const double kr = traj[2 * s], kc = traj[2 * s + 1];
    int64_t rl, cl;
    double rf, cfr;
    if (ksjo_grid_coordinate_f64(kr, rows, &rl, &rf) != 0) return -1;
    if (ksjo_grid_coordinate_f64(kc, cols, &cl, &cfr) != 0) return -1;
    const int64_t ru = (rl + 1) % rows, cu = (cl + 1) % cols;
    const double phase = -(kr * row_origin + kc * col_origin);
    const cf64 e = {cos(phase), sin(phase)};
    const cf64 ws = cmul_d(cscale_d(samples[s], dcf[s]), e);
    const double rlw = 1.0 - rf, clw = 1.0 - cfr;
    grid[rl * cols + cl] = cadd_d(grid[rl * cols + cl], cscale_d(ws, rlw * clw));
    grid[rl * cols + cu] = cadd_d(grid[rl * cols + cu], cscale_d(ws, rlw * cfr));
    grid[ru * cols + cl] = cadd_d(grid[ru * cols + cl], cscale_d(ws, rf * clw));
    grid[ru * cols + cu] = cadd_d(grid[ru * cols + cu], cscale_d(ws, rf * cfr));
  }
  return 0;
}

/* radial_linear_gridding2_adjoint (scatter + unnormalised separable inverse
 * transform, rows then columns).  eigen_radial_gridding.cpp:297-363. */
KSJO_EXPORT int ksjo_linear_gridding2_adjoint_f32(int64_t rows, int64_t cols, double row_origin, double col_origin,
                                                  const float* samples, const float* traj, const float* dcf,
                                                  int64_t m, float* image) {
  const int status = ksjo_linear_grid2_f32(rows, cols, row_origin, col_origin, samples, traj, dcf, m, image);
  if (status != 0) return status;
  idft2_rows_cols_f32((cf32*)image, rows, cols);
  return 0;
}

/* Same algorithm through the reference's double overload
 * (radial_gridding.hpp:65-69).  `exact` != 0 swaps the recurrence transform
 * for the directly evaluated one, removing the reference's own O(N eps)
 * twiddle drift from the FP64 oracle. */
KSJO_EXPORT int ksjo_linear_gridding2_adjoint_f64(int64_t rows, int64_t cols, double row_origin, double col_origin,
                                                  const double* samples, const double* traj, const double* dcf,
                                                  int64_t m, double* image, int exact) {
  const int status = ksjo_linear_grid2_f64(rows, cols, row_origin, col_origin, samples, traj, dcf, m, image);
  if (status != 0) return status;
  idft2_rows_cols_f64((cf64*)image, rows, cols, exact);
  return 0;
}

/* ----------------------------------------------------------- direct NUDFT */

/* direct_nudft2_adjoint: img(r,c) = sum_s y_s exp(i(k_r,s (r - r0) + k_c,s (c - c0))).
 * libs/numerics/kspacejet-nufft/src/eigen/eigen_nufft_direct_nudft.cpp:77-97. */
KSJO_EXPORT void ksjo_direct_nudft2_adjoint_f64(int64_t rows, int64_t cols, double row_origin, double col_origin,
                                                const double* samples_in, const double* traj, int64_t m,
                                                double* image_out) {
  const cf64* samples = (const cf64*)samples_in;
  cf64* image = (cf64*)image_out;
  for (int64_t r = 0; r < rows; ++r) {
    const double rp = (double)r - row_origin;
    for (int64_t c = 0; c < cols; ++c) {
      const double cp = (double)c - col_origin;
      cf64 sum = {0.0, 0.0};
      for (int64_t s = 0; s < m; ++s) {
        const double phase = traj[2 * s] * rp + traj[2 * s + 1] * cp;
        const cf64 e = {cos(phase), sin(phase)};
        sum = cadd_d(sum, cmul_d(samples[s], e));
      }
      image[r * cols + c] = sum;
    }
  }
}

/* direct_nudft2_adjoint at selected pixels only (FP64): out[i] is the value
 * the full form above gives at (pixels[2i], pixels[2i+1]).  The sum over
 * samples is the same, in the same order; only pixels nobody asked for are
 * skipped, so the exact NUDFT stays affordable at large images and sample
 * counts. */
KSJO_EXPORT void ksjo_direct_nudft2_adjoint_at_f64(int64_t npix, const int64_t* pixels, double row_origin,
                                                   double col_origin, const double* samples_in, const double* traj,
                                                   int64_t m, double* out) {
  const cf64* samples = (const cf64*)samples_in;
  cf64* o = (cf64*)out;
  for (int64_t i = 0; i < npix; ++i) {
    const double rp = (double)pixels[2 * i] - row_origin;
    const double cp = (double)pixels[2 * i + 1] - col_origin;
    cf64 sum = {0.0, 0.0};
    for (int64_t s = 0; s < m; ++s) {
      const double phase = traj[2 * s] * rp + traj[2 * s + 1] * cp;
      const cf64 e = {cos(phase), sin(phase)};
      sum = cadd_d(sum, cmul_d(samples[s], e));
    }
    o[i] = sum;
  }
}

KSJO_EXPORT void ksjo_direct_nudft2_adjoint_f32(int64_t rows, int64_t cols, double row_origin, double col_origin,
                                                const float* samples_in, const float* traj, int64_t m,
                                                float* image_out) {
  const cf32* samples = (const cf32*)samples_in;
  cf32* image = (cf32*)image_out;
  const float ro = (float)row_origin, co = (float)col_origin;
  for (int64_t r = 0; r < rows; ++r) {
    const float rp = (float)r - ro;
    for (int64_t c = 0; c < cols; ++c) {
      const float cp = (float)c - co;
      cf32 sum = {0.0f, 0.0f};
      for (int64_t s = 0; s < m; ++s) {
        const float phase = traj[2 * s] * rp + traj[2 * s + 1] * cp;
        const cf32 e = {cosf(phase), sinf(phase)};
        sum = cadd_f(sum, cmul_f(samples[s], e));
      }
      image[r * cols + c] = sum;
    }
  }
}

/* direct_nudft2_forward: y_s = sum_{r,c} img(r,c) exp(-i(k_r,s (r - r0) + k_c,s (c - c0))).
 * eigen_nufft_direct_nudft.cpp:52-75.  Used to synthesise k-space from a
 * phantom.  The row and column phases are separable, so this evaluates the
 * same sum as an outer product of per-axis exponentials (O(M N^2), not
 * O(M N^2) sin/cos calls). */
KSJO_EXPORT void ksjo_direct_nudft2_forward_f64(int64_t rows, int64_t cols, double row_origin, double col_origin,
                                                const double* image_in, const double* traj, int64_t m,
                                                double* out_samples) {
  const cf64* image = (const cf64*)image_in;
  cf64* out = (cf64*)out_samples;
  cf64* er = (cf64*)malloc((size_t)rows * sizeof(cf64));
  cf64* ec = (cf64*)malloc((size_t)cols * sizeof(cf64));
  for (int64_t s = 0; s < m; ++s) {
    for (int64_t r = 0; r < rows; ++r) {
      const double a = -traj[2 * s] * ((double)r - row_origin);
      er[r].re = cos(a); er[r].im = sin(a);
    }
    for (int64_t c = 0; c < cols; ++c) {
      const double a = -traj[2 * s + 1] * ((double)c - col_origin);
      ec[c].re = cos(a); ec[c].im = sin(a);
    }
    cf64 sum = {0.0, 0.0};
    for (int64_t r = 0; r < rows; ++r) {
      cf64 row_sum = {0.0, 0.0};
      for (int64_t c = 0; c < cols; ++c) row_sum = cadd_d(row_sum, cmul_d(image[r * cols + c], ec[c]));
      sum = cadd_d(sum, cmul_d(row_sum, er[r]));
    }
    out[s] = sum;
  }
  free(er); free(ec);
}

/* --------------------------------------------------------------------- RSS */

/* root_sum_of_squares_across(cube [P, C], Dim::dim2): per pixel a sequential
 * float sum over channels of re*re + im*im (std::norm), then sqrt.
 * libs/numerics/kspacejet-array/include/kspacejet/array/reductions.hpp:972-982,
 * libs/numerics/kspacejet-stats/src/eigen/eigen_stats_common.hpp:375-380. */
KSJO_EXPORT void ksjo_rss_f32(const float* coil_last, int64_t pixels, int64_t channels, float* out) {
  for (int64_t p = 0; p < pixels; ++p) {
    float total = 0.0f;
    for (int64_t c = 0; c < channels; ++c) {
      const float x = coil_last[2 * (p * channels + c)];
      const float y = coil_last[2 * (p * channels + c) + 1];
      total += x * x + y * y;
    }
    out[p] = sqrtf(total);
  }
}

/* ---------------------------------------------------- Kaiser-Bessel oracle */

/* I0 by its power series, summed until the term no longer changes the sum. */
KSJO_EXPORT double ksjo_bessel_i0(double x) {
  const double q = 0.25 * x * x;
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 500; ++k) {
    term *= q / ((double)k * (double)k);
    const double next = sum + term;
    if (next == sum) break;
    sum = next;
  }
  return sum;
}

/* Beatty et al. 2005, eq. 5: beta = pi sqrt((W/sigma)^2 (sigma - 1/2)^2 - 0.8). */
KSJO_EXPORT double ksjo_kb_beta(int width, double sigma) {
  const double a = ((double)width / sigma) * (sigma - 0.5);
  return kPiD * sqrt(a * a - 0.8);
}

/* Kernel value at offset d (grid cells), normalised to 1 at d = 0:
 * I0(beta sqrt(1 - (2d/W)^2)) / I0(beta) for |d| <= W/2, else 0. */
KSJO_EXPORT double ksjo_kb_kernel(double d, int width, double beta) {
  const double t = 2.0 * d / (double)width;
  if (t * t > 1.0) return 0.0;
  return ksjo_bessel_i0(beta * sqrt(1.0 - t * t)) / ksjo_bessel_i0(beta);
}

/* Continuous Fourier transform of that kernel at image offset x (pixels) on a
 * grid of g cells: W sinh(z)/z / I0(beta), z = sqrt(beta^2 - (pi W x / g)^2)
 * (sin(|z|)/|z| past the zero crossing). */
KSJO_EXPORT double ksjo_kb_deapod(double x, int width, double beta, int64_t g) {
  const double a = kPiD * (double)width * x / (double)g;
  const double z2 = beta * beta - a * a;
  double shape;
  if (z2 > 1e-12) {
    const double z = sqrt(z2);
    shape = sinh(z) / z;
  } else if (z2 < -1e-12) {
    const double z = sqrt(-z2);
    shape = sin(z) / z;
  } else {
    shape = 1.0;
  }
  return (double)width * shape / ksjo_bessel_i0(beta);
}

/* Kaiser-Bessel gridding adjoint (double precision), the algorithm of the
 * CUDA radial_kb_gridding path:
 *   grid size g (oversampled), image n x n, kernel width W, shape beta;
 *   grid coordinate u = k g / (2 pi) (no wrap; indices taken mod g);
 *   taps j = floor(u) - W/2 + 1 ... floor(u) + W/2, weight phi(j - u) per axis;
 *   sample weight v = y * dcf * exp(i k * delta), delta = n/2 - origin
 *     (-1/2 for the reference origin (n-1)/2), which centres the image on
 *     pixel offsets q = p - n/2 in [-n/2, n/2);
 *   unnormalised inverse 2-D DFT of the grid (exact, directly evaluated);
 *   image(p_r, p_c) = grid_idft(q_r mod g, q_c mod g) / (psi(q_r) psi(q_c)),
 *     q = p - n/2, psi the kernel's continuous Fourier transform: by Poisson
 *     summation sum_j phi(j - u) exp(2 pi i j q / g) ~ exp(2 pi i u q / g) psi(q),
 *     and exp(i k (q + delta)) = exp(i k (p - origin)).
 * The result approximates direct_nudft2_adjoint of the dcf-weighted samples
 * with origin (row_origin, col_origin). */
KSJO_EXPORT int ksjo_kb_gridding2_adjoint_f64(int64_t g, int64_t n, int width, double beta, double row_origin,
                                              double col_origin, const double* samples_in, const double* traj,
                                              const double* dcf, int64_t m, double* image_out) {
  if (g < n || g < width || (width % 2) != 0) return -1;
  const cf64* samples = (const cf64*)samples_in;
  cf64* image = (cf64*)image_out;
  cf64* grid = (cf64*)calloc((size_t)(g * g), sizeof(cf64));
  const double half = (double)(n / 2);
  const double dr = half - row_origin, dc = half - col_origin;
  for (int64_t s = 0; s < m; ++s) {
    const double kr = traj[2 * s], kc = traj[2 * s + 1];
    const double ur = kr * (double)g / (2.0 * kPiD), uc = kc * (double)g / (2.0 * kPiD);
    const double ph = kr * dr + kc * dc;
    const cf64 e = {cos(ph), sin(ph)};
    const cf64 v = cmul_d(cscale_d(samples[s], dcf ? dcf[s] : 1.0), e);
    const int64_t r0 = (int64_t)floor(ur) - width / 2 + 1;
    const int64_t c0 = (int64_t)floor(uc) - width / 2 + 1;
    for (int a = 0; a < width; ++a) {
      const double wr = ksjo_kb_kernel((double)(r0 + a) - ur, width, beta);
      const int64_t rr = (((r0 + a) % g) + g) % g;
      for (int b = 0; b < width; ++b) {
        const double wc = ksjo_kb_kernel((double)(c0 + b) - uc, width, beta);
        const int64_t cc = (((c0 + b) % g) + g) % g;
        grid[rr * g + cc] = cadd_d(grid[rr * g + cc], cscale_d(v, wr * wc));
      }
    }
  }
  idft2_rows_cols_f64(grid, g, g, 1);
  for (int64_t pr = 0; pr < n; ++pr) {
    const int64_t qr = pr - n / 2;
    const double ar = ksjo_kb_deapod((double)qr, width, beta, g);
    for (int64_t pc = 0; pc < n; ++pc) {
      const int64_t qc = pc - n / 2;
      const double ac = ksjo_kb_deapod((double)qc, width, beta, g);
      const cf64 x = grid[(((qr % g) + g) % g) * g + (((qc % g) + g) % g)];
      image[pr * n + pc] = cscale_d(x, 1.0 / (ar * ac));
    }
  }
  free(grid);
  return 0;
}

/* ---------------------------------------- Kaiser-Bessel, single precision CPU
 *
 * The same Kaiser-Bessel reconstruction as ksjo_kb_gridding2_adjoint_f64 as a
 * practical single-precision CPU program: float gridding with tap weights
 * from the double kernel rounded once, a mixed-radix (2, 3, 4) decimation-in-
 * time FFT with a twiddle table computed in double, the row transforms over
 * every grid row and the column transforms over the kept columns only, then
 * crop and deapodisation.  It is the timed CPU baseline for the KB forms
 * (which the reference does not have), not a parity target; the tests check
 * it against the FP64 form. */
typedef struct {
  int64_t n;
  cf32* tw; /* exp(2 pi i t / n), t < n */
} fftplan_f;

static int fft_plan_f(fftplan_f* p, int64_t n) {
  int64_t m = n;
  while (m % 4 == 0) m /= 4;
  while (m % 2 == 0) m /= 2;
  while (m % 3 == 0) m /= 3;
  if (m != 1) return -1;
  p->n = n;
  p->tw = (cf32*)malloc((size_t)n * sizeof(cf32));
  if (!p->tw) return -1;
  for (int64_t t = 0; t < n; ++t) {
    const double a = 2.0 * kPiD * (double)t / (double)n;
    p->tw[t].re = (float)cos(a);
    p->tw[t].im = (float)sin(a);
  }
  return 0;
}

/* y[k] = sum_j x[j stride] exp(2 pi i j k / len), len | plan n; scratch >= 2 len */
static void fft_dit_f(const fftplan_f* p, const cf32* x, int64_t stride, cf32* y, int64_t len, cf32* scratch) {
  if (len == 1) { y[0] = x[0]; return; }
  const int64_t r = (len % 4 == 0) ? 4 : (len % 2 == 0) ? 2 : 3;
  const int64_t m = len / r;
  const int64_t step = p->n / len;
  for (int64_t q = 0; q < r; ++q) fft_dit_f(p, x + q * stride, stride * r, scratch + q * m, m, scratch + len);
  for (int64_t k = 0; k < m; ++k) {
    cf32 v[4];
    for (int64_t q = 0; q < r; ++q) {
      const cf32 w = p->tw[(q * k * step) % p->n];
      v[q] = q == 0 ? scratch[k] : cmul_f(scratch[q * m + k], w);
    }
    if (r == 2) {
      y[k] = cadd_f(v[0], v[1]);
      y[k + m] = csub_f(v[0], v[1]);
    } else if (r == 4) {
      const cf32 a = cadd_f(v[0], v[2]), b = csub_f(v[0], v[2]);
      const cf32 c = cadd_f(v[1], v[3]), dd = csub_f(v[1], v[3]);
      const cf32 d = {-dd.im, dd.re}; /* i (v1 - v3) */
      y[k] = cadd_f(a, c);
      y[k + m] = cadd_f(b, d);
      y[k + 2 * m] = csub_f(a, c);
      y[k + 3 * m] = csub_f(b, d);
    } else {
      const float s3 = 0.86602540378443865f;
      const cf32 t1 = cadd_f(v[1], v[2]);
      const cf32 t2 = {v[0].re - 0.5f * t1.re, v[0].im - 0.5f * t1.im};
      const cf32 d = csub_f(v[1], v[2]);
      const cf32 t3 = {-s3 * d.im, s3 * d.re}; /* i sin(2 pi / 3) (v1 - v2) */
      y[k] = cadd_f(v[0], t1);
      y[k + m] = cadd_f(t2, t3);
      y[k + 2 * m] = csub_f(t2, t3);
    }
  }
}

KSJO_EXPORT int ksjo_kb_gridding2_adjoint_f32(int64_t g, int64_t n, int width, double beta, double row_origin,
                                              double col_origin, const float* samples_in, const float* traj,
                                              const float* dcf, int64_t m, float* image_out) {
  if (g < n || g < width || (width % 2) != 0 || width > 8) return -1;
  fftplan_f plan;
  if (fft_plan_f(&plan, g) != 0) return -1;
  const cf32* samples = (const cf32*)samples_in;
  cf32* image = (cf32*)image_out;
  cf32* grid = (cf32*)calloc((size_t)(g * g), sizeof(cf32));
  cf32* line = (cf32*)malloc((size_t)g * sizeof(cf32));
  cf32* out = (cf32*)malloc((size_t)g * sizeof(cf32));
  cf32* scratch = (cf32*)malloc((size_t)(4 * g + 64) * sizeof(cf32));
  float* inv_d = (float*)malloc((size_t)n * sizeof(float));
  if (!grid || !line || !out || !scratch || !inv_d) {
    free(grid); free(line); free(out); free(scratch); free(inv_d); free(plan.tw);
    return -1;
  }
  const double half = (double)(n / 2);
  const double dr = half - row_origin, dc = half - col_origin;
  const double scale = (double)g / (2.0 * kPiD);
  for (int64_t s = 0; s < m; ++s) {
    /* coordinates and phase in double (a float grid coordinate moves the
       taps' weights by ~1e-5 at g = 384), then the sample arithmetic in float */
    const double kr = traj[2 * s], kc = traj[2 * s + 1];
    const double ur = kr * scale, uc = kc * scale;
    const double ph = kr * dr + kc * dc;
    const cf32 e = {(float)cos(ph), (float)sin(ph)};
    const cf32 v = cmul_f(cscale_f(samples[s], dcf ? dcf[s] : 1.0f), e);
    const int64_t r0 = (int64_t)floor(ur) - width / 2 + 1;
    const int64_t c0 = (int64_t)floor(uc) - width / 2 + 1;
    float wr[8], wc[8];
    for (int a = 0; a < width; ++a) {
      wr[a] = (float)ksjo_kb_kernel((double)(r0 + a) - ur, width, beta);
      wc[a] = (float)ksjo_kb_kernel((double)(c0 + a) - uc, width, beta);
    }
    for (int a = 0; a < width; ++a) {
      const int64_t rr = (((r0 + a) % g) + g) % g;
      const cf32 va = cscale_f(v, wr[a]);
      for (int b = 0; b < width; ++b) {
        const int64_t cc = (((c0 + b) % g) + g) % g;
        grid[rr * g + cc] = cadd_f(grid[rr * g + cc], cscale_f(va, wc[b]));
      }
    }
  }
  /* rows: every grid row; keep the n columns of the image (frequency q mod g) */
  for (int64_t r = 0; r < g; ++r) {
    fft_dit_f(&plan, grid + r * g, 1, out, g, scratch);
    for (int64_t pc = 0; pc < n; ++pc) grid[r * g + pc] = out[(((pc - n / 2) % g) + g) % g];
  }
  for (int64_t p = 0; p < n; ++p) inv_d[p] = (float)(1.0 / ksjo_kb_deapod((double)(p - n / 2), width, beta, g));
  /* columns: the n kept ones only, cropped and deapodised */
  for (int64_t pc = 0; pc < n; ++pc) {
    for (int64_t r = 0; r < g; ++r) line[r] = grid[r * g + pc];
    fft_dit_f(&plan, line, 1, out, g, scratch);
    for (int64_t pr = 0; pr < n; ++pr)
      image[pr * n + pc] = cscale_f(out[(((pr - n / 2) % g) + g) % g], inv_d[pr] * inv_d[pc]);
  }
  free(grid); free(line); free(out); free(scratch); free(inv_d); free(plan.tw);
  return 0;
}

/* Kaiser-Bessel forward (double precision): the exact transpose of
 * ksjo_kb_gridding2_adjoint_f64 without density weights.  image n x n ->
 * deapodised (1 / (psi(q_r) psi(q_c))), placed at grid (q_r mod g, q_c mod g),
 * q = p - n/2; forward 2-D DFT exp(-2 pi i (k . j) / g) (exact, directly
 * evaluated); per sample y = conj(exp(i k . delta)) sum over the taps
 * (row-major) of phi(j_r - u_r) phi(j_c - u_c) grid[j_r mod g][j_c mod g]. */
KSJO_EXPORT int ksjo_kb_forward2_f64(int64_t g, int64_t n, int width, double beta, double row_origin,
                                     double col_origin, const double* image_in, const double* traj, int64_t m,
                                     double* samples_out) {
  if (g < n || g < width || (width % 2) != 0) return -1;
  const cf64* image = (const cf64*)image_in;
  cf64* samples = (cf64*)samples_out;
  cf64* grid = (cf64*)calloc((size_t)(g * g), sizeof(cf64));
  for (int64_t pr = 0; pr < n; ++pr) {
    const int64_t qr = pr - n / 2;
    const double ar = ksjo_kb_deapod((double)qr, width, beta, g);
    for (int64_t pc = 0; pc < n; ++pc) {
      const int64_t qc = pc - n / 2;
      const double ac = ksjo_kb_deapod((double)qc, width, beta, g);
      const cf64 x = cscale_d(image[pr * n + pc], 1.0 / (ar * ac));
      grid[(((qr % g) + g) % g) * g + (((qc % g) + g) % g)] = (cf64){x.re, -x.im};  /* conj */
    }
  }
  idft2_rows_cols_f64(grid, g, g, 1);  /* conj(IDFT(conj x)) = DFT x */
  for (int64_t i = 0; i < g * g; ++i) grid[i].im = -grid[i].im;
  const double half = (double)(n / 2);
  const double dr = half - row_origin, dc = half - col_origin;
  for (int64_t s = 0; s < m; ++s) {
    const double kr = traj[2 * s], kc = traj[2 * s + 1];
    const double ur = kr * (double)g / (2.0 * kPiD), uc = kc * (double)g / (2.0 * kPiD);
    const double ph = kr * dr + kc * dc;
    const cf64 e = {cos(ph), -sin(ph)};
    const int64_t r0 = (int64_t)floor(ur) - width / 2 + 1;
    const int64_t c0 = (int64_t)floor(uc) - width / 2 + 1;
    cf64 acc = {0.0, 0.0};
    for (int a = 0; a < width; ++a) {
      const double wr = ksjo_kb_kernel((double)(r0 + a) - ur, width, beta);
      const int64_t rr = (((r0 + a) % g) + g) % g;
      for (int b = 0; b < width; ++b) {
        const double wc = ksjo_kb_kernel((double)(c0 + b) - uc, width, beta);
        const int64_t cc = (((c0 + b) % g) + g) % g;
        acc = cadd_d(acc, cscale_d(grid[rr * g + cc], wr * wc));
      }
    }
    samples[s] = cmul_d(acc, e);
  }
  free(grid);
  return 0;
}

/* ------------------------------------------------------------ Pipe-Menon */

/* Iterative density compensation (Pipe & Menon, MRM 41:179-186, 1999) in
 * its grid-based form, with the Kaiser-Bessel kernel phi of the gridding path
 * (ksjo_kb_kernel, taps floor(u) - W/2 + 1 ... floor(u) + W/2, u = k g / 2 pi,
 * indices mod g).  No reference counterpart.  Starting from w = 1 every
 * iteration
 *   grids w:          c[cell] = sum_s w_s * (phi_r * phi_c), samples in index order,
 *   interpolates back: d_s = sum over the sample's taps (row-major) of c[cell] * (phi_r * phi_c),
 *   and updates        w_s = w_s / d_s (0 when d_s is not positive).
 * Double precision throughout.  traj [m][2] float32; out [m] double. */
KSJO_EXPORT int ksjo_pipe_menon_dcf2_f64(int64_t g_rows, int64_t g_cols, int width, double beta, const float* traj,
                                         int64_t m, int iterations, double* out) {
  if (width < 2 || width > 16 || g_rows < width || g_cols < width) return -1;
  double* grid = (double*)malloc((size_t)(g_rows * g_cols) * sizeof(double));
  int64_t* r0 = (int64_t*)malloc((size_t)m * sizeof(int64_t));
  int64_t* c0 = (int64_t*)malloc((size_t)m * sizeof(int64_t));
  double* wr = (double*)malloc((size_t)(m * width) * sizeof(double));
  double* wc = (double*)malloc((size_t)(m * width) * sizeof(double));
  if (!grid || !r0 || !c0 || !wr || !wc) return -2;
  for (int64_t s = 0; s < m; ++s) {
    const double ur = (double)traj[2 * s] * (double)g_rows / (2.0 * kPiD);
    const double uc = (double)traj[2 * s + 1] * (double)g_cols / (2.0 * kPiD);
    const int64_t tr = (int64_t)floor(ur) - width / 2 + 1;
    const int64_t tc = (int64_t)floor(uc) - width / 2 + 1;
    r0[s] = ((tr % g_rows) + g_rows) % g_rows;
    c0[s] = ((tc % g_cols) + g_cols) % g_cols;
    for (int j = 0; j < width; ++j) {
      wr[s * width + j] = ksjo_kb_kernel((double)(tr + j) - ur, width, beta);
      wc[s * width + j] = ksjo_kb_kernel((double)(tc + j) - uc, width, beta);
    }
    out[s] = 1.0;
  }
  for (int it = 0; it < iterations; ++it) {
    memset(grid, 0, (size_t)(g_rows * g_cols) * sizeof(double));
    for (int64_t s = 0; s < m; ++s)
      for (int a = 0; a < width; ++a) {
        const int64_t rr = (r0[s] + a) % g_rows;
        for (int b = 0; b < width; ++b) {
          const int64_t cc = (c0[s] + b) % g_cols;
          grid[rr * g_cols + cc] += out[s] * (wr[s * width + a] * wc[s * width + b]);
        }
      }
    for (int64_t s = 0; s < m; ++s) {
      double d = 0.0;
      for (int a = 0; a < width; ++a) {
        const int64_t rr = (r0[s] + a) % g_rows;
        for (int b = 0; b < width; ++b) {
          const int64_t cc = (c0[s] + b) % g_cols;
          d += grid[rr * g_cols + cc] * (wr[s * width + a] * wc[s * width + b]);
        }
      }
      out[s] = d > 0.0 ? out[s] / d : 0.0;
    }
  }
  free(grid);
  free(r0);
  free(c0);
  free(wr);
  free(wc);
  return 0;
}

/* ------------------------------------------------------ coil covariance */

/* coil_compression_basis_estimate.cpp:207-227 in float, operation for
 * operation: lower triangle sum over samples of x_row * conj(x_col) (complex
 * float multiply and add, rounded separately), times the float reciprocal of
 * the sample count, upper triangle the conjugate.  x complex64 [c][m];
 * out complex64 [c][c]. */
KSJO_EXPORT void ksjo_coil_covariance_f32(int64_t c, int64_t m, const float* x_in, float* out_raw) {
  const cf32* x = (const cf32*)x_in;
  cf32* out = (cf32*)out_raw;
  for (int64_t i = 0; i < c * c; ++i) out[i] = (cf32){0.0f, 0.0f};
  for (int64_t s = 0; s < m; ++s)
    for (int64_t r = 0; r < c; ++r)
      for (int64_t col = 0; col <= r; ++col) {
        const cf32 a = x[r * m + s], b = x[col * m + s];
        const cf32 p = cmul_f(a, (cf32){b.re, -b.im});
        out[r * c + col] = (cf32){out[r * c + col].re + p.re, out[r * c + col].im + p.im};
      }
  const float inv = 1.0f / (float)m;
  for (int64_t r = 0; r < c; ++r) {
    out[r * c + r] = (cf32){out[r * c + r].re * inv, out[r * c + r].im * inv};
    for (int64_t col = 0; col < r; ++col) {
      out[r * c + col] = (cf32){out[r * c + col].re * inv, out[r * c + col].im * inv};
      out[col * c + r] = (cf32){out[r * c + col].re, -out[r * c + col].im};
    }
  }
}

/* The same covariance in double precision (the accuracy reference). */
KSJO_EXPORT void ksjo_coil_covariance_f64(int64_t c, int64_t m, const float* x_in, double* out_raw) {
  const cf32* x = (const cf32*)x_in;
  cf64* out = (cf64*)out_raw;
  for (int64_t i = 0; i < c * c; ++i) out[i] = (cf64){0.0, 0.0};
  for (int64_t s = 0; s < m; ++s)
    for (int64_t r = 0; r < c; ++r)
      for (int64_t col = 0; col <= r; ++col) {
        const double ar = x[r * m + s].re, ai = x[r * m + s].im, br = x[col * m + s].re, bi = x[col * m + s].im;
        out[r * c + col].re += ar * br + ai * bi;
        out[r * c + col].im += ai * br - ar * bi;
      }
  for (int64_t r = 0; r < c; ++r)
    for (int64_t col = 0; col <= r; ++col) {
      out[r * c + col].re /= (double)m;
      out[r * c + col].im /= (double)m;
      out[col * c + r] = (cf64){out[r * c + col].re, -out[r * c + col].im};
    }
}

/* ------------------------------------------------------- 3-D Kaiser-Bessel */

/* The 2-D Kaiser-Bessel adjoint above extended to a cube (the CUDA 3-D path):
 * grid g^3, image n^3, coordinates u = k g / 2 pi per axis (z, y, x order in
 * the trajectory), taps floor(u) - W/2 + 1 ... floor(u) + W/2 mod g, weight
 * phi_z phi_y phi_x, sample weight y * dcf * exp(i k . delta) with
 * delta = n/2 - origin per axis, exact separable inverse DFT along x, y, z,
 * crop q = p - n/2 and deapodisation 1 / (psi(q_z) psi(q_y) psi(q_x)).
 * samples complex128 [m]; traj double [m][3]; image complex128 [n][n][n]. */
KSJO_EXPORT int ksjo_kb_gridding3_adjoint_f64(int64_t g, int64_t n, int width, double beta, double origin,
                                              const double* samples_in, const double* traj, const double* dcf,
                                              int64_t m, double* image_out) {
  if (g < n || g < width || (width % 2) != 0) return -1;
  const cf64* samples = (const cf64*)samples_in;
  cf64* image = (cf64*)image_out;
  cf64* grid = (cf64*)calloc((size_t)(g * g * g), sizeof(cf64));
  cf64* src = (cf64*)malloc((size_t)g * sizeof(cf64));
  cf64* dst = (cf64*)malloc((size_t)g * sizeof(cf64));
  if (!grid || !src || !dst) return -2;
  const double delta = (double)(n / 2) - origin;
  for (int64_t s = 0; s < m; ++s) {
    double u[3], w[3][16];
    int64_t t0[3];
    double ph = 0.0;
    for (int d = 0; d < 3; ++d) {
      const double k = traj[3 * s + d];
      u[d] = k * (double)g / (2.0 * kPiD);
      ph += k * delta;
      t0[d] = (int64_t)floor(u[d]) - width / 2 + 1;
      for (int j = 0; j < width; ++j) w[d][j] = ksjo_kb_kernel((double)(t0[d] + j) - u[d], width, beta);
    }
    const cf64 e = {cos(ph), sin(ph)};
    const cf64 v = cmul_d(cscale_d(samples[s], dcf ? dcf[s] : 1.0), e);
    for (int a = 0; a < width; ++a) {
      const int64_t zz = (((t0[0] + a) % g) + g) % g;
      for (int b = 0; b < width; ++b) {
        const int64_t yy = (((t0[1] + b) % g) + g) % g;
        const double wzy = w[0][a] * w[1][b];
        for (int c = 0; c < width; ++c) {
          const int64_t xx = (((t0[2] + c) % g) + g) % g;
          const int64_t at = (zz * g + yy) * g + xx;
          grid[at] = cadd_d(grid[at], cscale_d(v, wzy * w[2][c]));
        }
      }
    }
  }
  /* separable exact inverse DFT: x lines, then y lines, then z lines */
  for (int axis = 0; axis < 3; ++axis) {
    const int64_t stride = axis == 0 ? 1 : (axis == 1 ? g : g * g);
    for (int64_t a = 0; a < g; ++a)
      for (int64_t b = 0; b < g; ++b) {
        int64_t base;
        if (axis == 0) base = (a * g + b) * g;
        else if (axis == 1) base = a * g * g + b;
        else base = a * g + b;
        for (int64_t i = 0; i < g; ++i) src[i] = grid[base + i * stride];
        ksjo_exact_idft_f64((const double*)src, (double*)dst, g);
        for (int64_t i = 0; i < g; ++i) grid[base + i * stride] = dst[i];
      }
  }
  for (int64_t pz = 0; pz < n; ++pz) {
    const int64_t qz = pz - n / 2;
    const double az = ksjo_kb_deapod((double)qz, width, beta, g);
    for (int64_t py = 0; py < n; ++py) {
      const int64_t qy = py - n / 2;
      const double ay = ksjo_kb_deapod((double)qy, width, beta, g);
      for (int64_t px = 0; px < n; ++px) {
        const int64_t qx = px - n / 2;
        const double ax = ksjo_kb_deapod((double)qx, width, beta, g);
        const cf64 x = grid[((((qz % g) + g) % g) * g + (((qy % g) + g) % g)) * g + (((qx % g) + g) % g)];
        image[(pz * n + py) * n + px] = cscale_d(x, 1.0 / (az * ay * ax));
      }
    }
  }
  free(grid);
  free(src);
  free(dst);
  return 0;
}

/* Exact 3-D adjoint NUDFT: img(z, y, x) = sum_s y_s exp(i k_s . (p - origin)),
 * the 3-D extension of direct_nudft2_adjoint (eigen_nufft_direct_nudft.cpp:77-97);
 * samples complex128 [m], traj double [m][3] (z, y, x), image complex128 [n][n][n]. */
KSJO_EXPORT void ksjo_direct_nudft3_adjoint_f64(int64_t n, double origin, const double* samples_in,
                                                const double* traj, int64_t m, double* image_out) {
  const cf64* samples = (const cf64*)samples_in;
  cf64* image = (cf64*)image_out;
  for (int64_t p = 0; p < n * n * n; ++p) {
    const double z = (double)(p / (n * n)) - origin, y = (double)((p / n) % n) - origin, x = (double)(p % n) - origin;
    double re = 0.0, im = 0.0;
    for (int64_t s = 0; s < m; ++s) {
      const double ph = traj[3 * s] * z + traj[3 * s + 1] * y + traj[3 * s + 2] * x;
      const double c = cos(ph), sn = sin(ph);
      re += samples[s].re * c - samples[s].im * sn;
      im += samples[s].re * sn + samples[s].im * c;
    }
    image[p] = (cf64){re, im};
  }
}

/* The Pipe-Menon iteration of ksjo_pipe_menon_dcf2_f64 on a g^3 grid (taps
 * per axis as the 3-D gridding; tap product (phi_z phi_y) phi_x, taps in
 * z, y, x order).  traj float32 [m][3]; out double [m]. */
KSJO_EXPORT int ksjo_pipe_menon_dcf3_f64(int64_t g, int width, double beta, const float* traj, int64_t m,
                                         int iterations, double* out) {
  if (width < 2 || width > 16 || g < width) return -1;
  double* grid = (double*)malloc((size_t)(g * g * g) * sizeof(double));
  int64_t* t0 = (int64_t*)malloc((size_t)(3 * m) * sizeof(int64_t));
  double* wt = (double*)malloc((size_t)(3 * m * width) * sizeof(double));
  if (!grid || !t0 || !wt) return -2;
  for (int64_t s = 0; s < m; ++s) {
    for (int d = 0; d < 3; ++d) {
      const double u = (double)traj[3 * s + d] * (double)g / (2.0 * kPiD);
      const int64_t t = (int64_t)floor(u) - width / 2 + 1;
      t0[3 * s + d] = ((t % g) + g) % g;
      for (int j = 0; j < width; ++j) wt[(3 * s + d) * width + j] = ksjo_kb_kernel((double)(t + j) - u, width, beta);
    }
    out[s] = 1.0;
  }
  for (int it = 0; it < iterations; ++it) {
    memset(grid, 0, (size_t)(g * g * g) * sizeof(double));
    for (int pass = 0; pass < 2; ++pass)
      for (int64_t s = 0; s < m; ++s) {
        const double* wz = wt + (3 * s) * width;
        const double* wy = wt + (3 * s + 1) * width;
        const double* wx = wt + (3 * s + 2) * width;
        double d = 0.0;
        for (int a = 0; a < width; ++a) {
          const int64_t zz = (t0[3 * s] + a) % g;
          for (int b = 0; b < width; ++b) {
            const int64_t yy = (t0[3 * s + 1] + b) % g;
            const double wzy = wz[a] * wy[b];
            for (int c = 0; c < width; ++c) {
              const int64_t xx = (t0[3 * s + 2] + c) % g;
              double* cell = grid + (zz * g + yy) * g + xx;
              if (pass == 0) *cell += out[s] * (wzy * wx[c]);
              else d += *cell * (wzy * wx[c]);
            }
          }
        }
        if (pass == 1) out[s] = d > 0.0 ? out[s] / d : 0.0;
      }
  }
  free(grid);
  free(t0);
  free(wt);
  return 0;
}
