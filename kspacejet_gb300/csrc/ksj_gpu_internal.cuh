// ksj_gpu_internal.cuh -- device building blocks shared by the sm_103a kernels
// of the non-Cartesian path: float2 complex arithmetic, error-free-transform
// grid coordinates and origin phases, the Kaiser-Bessel tap weight, and an
// in-place mixed-radix (2/3/4/8) Stockham FFT over lines held in shared
// memory.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include "ksj_gpu.h"

namespace ksj_gpu {

// ------------------------------------------------------------------ launches

ksj_gpu_status check_launch();       // cudaGetLastError -> status

// Brackets one kernel launch: counts it and, while timing is enabled, records
// CUDA events before and after it on its stream.  Construct immediately
// before the launch; the destructor runs after it.
class LaunchScope {
 public:
  LaunchScope(const char* name, cudaStream_t stream);
  ~LaunchScope();
  LaunchScope(const LaunchScope&) = delete;
  LaunchScope& operator=(const LaunchScope&) = delete;

 private:
  const char* name_;
  cudaStream_t stream_;
  cudaEvent_t start_ = nullptr;
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// ------------------------------------------------------------------- complex

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cmul_i(float2 a) { return make_float2(-a.y, a.x); }  // a * i

// ------------------------------------------------- error-free transformations

// A float pair hi + lo carrying about 46 significant bits.
struct dfloat {
  float hi, lo;
};

__device__ __forceinline__ dfloat two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ dfloat fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// fl32(2 pi) and the remainder 2 pi - fl32(2 pi).
constexpr float kTwoPiHi = 6.2831854820251465f;
constexpr float kTwoPiLo = -1.7484555314695172e-07f;
// Three-part Cody-Waite split of 2 pi: C1 has 8 significant bits, so n * C1
// is exact for |n| < 2^16; C1 + C2 + C3 = 2 pi to about 2^-60.
constexpr float kCw1 = 6.28125f;
constexpr float kCw2 = 0.0019353071693331003f;
constexpr float kCw3 = 1.0253376273028358e-11f;
constexpr float kInvTwoPi = 0.15915493667125702f;
constexpr float kPiF = 3.14159265358979323846f;

// The real number f * n / (2 pi) (f, n float; n an exact integer) to about
// 2^-46 relative error.  The reference evaluates fl(fl(f*n) / fl(2 pi)) in
// float (eigen_radial_gridding.cpp:264), whose ~1e-7 relative error moves the
// linear weights by up to 3e-5 on a 512 grid; here the product error is kept
// with an FMA, the quotient remainder is exact (p - q*C for q = fl(p/C)), and
// the low part of 2 pi enters the correction term.
__device__ __forceinline__ dfloat grid_coordinate(float f, float n) {
  const float p = __fmul_rn(f, n);
  const float pe = __fmaf_rn(f, n, -p);
  const float q = __fdiv_rn(p, kTwoPiHi);
  const float r = __fmaf_rn(-q, kTwoPiHi, p);
  const float num = __fmaf_rn(-q, kTwoPiLo, __fadd_rn(r, pe));
  return fast_two_sum(q, __fdiv_rn(num, kTwoPiHi));
}

// floor of hi + lo (|lo| <= ulp(hi)/2), and the fractional part in [0, 1).
// The floor is exact; a fraction within 2^-25 of 1 is not representable and
// rounds to 1.0f, so it is clamped to the largest float below 1 -- the floor
// itself must not move, or the tap window would shift by one cell.
__device__ __forceinline__ int dfloor(dfloat x, float* frac) {
  float l = floorf(x.hi);
  float f;
  if (l == x.hi) {
    if (x.lo < 0.0f) {
      l -= 1.0f;
      f = __fadd_rn(1.0f, x.lo);
    } else {
      f = x.lo;
    }
  } else {
    f = __fadd_rn(__fsub_rn(x.hi, l), x.lo);
  }
  *frac = fminf(f, 0.99999994f);
  return static_cast<int>(l);
}

__device__ __forceinline__ int wrap_index(int i, int n) {
  int r = i % n;
  return r < 0 ? r + n : r;
}

// exp(i * sign * (a1*b1 + a2*b2)) for float a, b with |a1 b1 + a2 b2| < 2^14:
// exact products and sum (FMA error terms, two-sum), Cody-Waite reduction by
// 2 pi (Cody & Waite 1980) with the low parts added after the exact first
// step, then sincosf of an argument in [-pi - 0.5, pi + 0.5].  The reference
// rounds the whole phase to float before cos/sin (eigen_radial_gridding.cpp:
// 330-334), an absolute error up to 6e-5 rad on a 512 grid.
__device__ __forceinline__ float2 exp_i_dot(float a1, float b1, float a2, float b2, float sign) {
  const float p1 = __fmul_rn(a1, b1);
  const float e1 = __fmaf_rn(a1, b1, -p1);
  const float p2 = __fmul_rn(a2, b2);
  const float e2 = __fmaf_rn(a2, b2, -p2);
  const dfloat s = two_sum(p1, p2);
  const float lo = __fadd_rn(s.lo, __fadd_rn(e1, e2));
  const float n = rintf(__fmul_rn(s.hi, kInvTwoPi));
  float r = __fmaf_rn(-n, kCw1, s.hi);
  r = __fmaf_rn(-n, kCw2, r);
  r = __fmaf_rn(-n, kCw3, r);
  r = __fadd_rn(r, lo);
  float sn, cs;
  sincosf(sign * r, &sn, &cs);
  return make_float2(cs, sn);
}

// exp(i (a1 b1 + a2 b2 + a3 b3)): the three-term form of exp_i_dot (sign +1).
__device__ __forceinline__ float2 exp_i_dot3(float a1, float b1, float a2, float b2, float a3, float b3) {
  const float p1 = __fmul_rn(a1, b1);
  const float e1 = __fmaf_rn(a1, b1, -p1);
  const float p2 = __fmul_rn(a2, b2);
  const float e2 = __fmaf_rn(a2, b2, -p2);
  const float p3 = __fmul_rn(a3, b3);
  const float e3 = __fmaf_rn(a3, b3, -p3);
  const dfloat s = two_sum(p1, p2);
  const dfloat t = two_sum(s.hi, p3);
  const float lo = __fadd_rn(__fadd_rn(s.lo, t.lo), __fadd_rn(__fadd_rn(e1, e2), e3));
  const float n = rintf(__fmul_rn(t.hi, kInvTwoPi));
  float r = __fmaf_rn(-n, kCw1, t.hi);
  r = __fmaf_rn(-n, kCw2, r);
  r = __fmaf_rn(-n, kCw3, r);
  r = __fadd_rn(r, lo);
  float sn, cs;
  sincosf(r, &sn, &cs);
  return make_float2(cs, sn);
}

// Kaiser-Bessel tap weight at offset d (grid cells), normalised to 1 at d = 0:
// I0(beta sqrt(1 - (2d/W)^2)) / I0(beta).
__device__ __forceinline__ float kb_weight(float d, float two_over_w, float beta, float inv_i0_beta) {
  const float t = d * two_over_w;
  const float a = fmaxf(fmaf(-t, t, 1.0f), 0.0f);
  return cyl_bessel_i0f(beta * sqrtf(a)) * inv_i0_beta;
}

// 1 / psi(q) for kept pixel p of n (q = p - n/2) on a grid of g: psi the
// continuous Fourier transform of the normalised Kaiser-Bessel kernel,
// W sinh(z)/z / I0(beta), z = sqrt(beta^2 - (pi W q / g)^2) (Jackson et al.
// 1991), evaluated in FP64 and rounded once.
__device__ __forceinline__ float kb_inv_deapod(int p, int n, int g, int width, double beta, double i0_beta) {
  const double q = static_cast<double>(p - n / 2);
  const double a = 3.14159265358979323846 * width * q / g;
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
  return static_cast<float>(i0_beta / (width * shape));
}

// The default Kaiser-Bessel shape for width W and oversampling sigma (Beatty
// et al. 2005): pi sqrt((W / sigma)^2 (sigma - 1/2)^2 - 0.8); 0 when that is
// not real.
inline double kb_default_beta(int width, double sigma) {
  const double a = (static_cast<double>(width) / sigma) * (sigma - 0.5);
  const double arg = a * a - 0.8;
  return arg > 0.0 ? 3.14159265358979323846 * std::sqrt(arg) : 0.0;
}

// ----------------------------------------------------------------- bfloat16

__device__ __forceinline__ float bf16_to_float(uint16_t h) { return __uint_as_float(static_cast<uint32_t>(h) << 16); }

template <uint32_t kFormat>
__device__ __forceinline__ float2 load_sample(const void* base, size_t index);

template <>
__device__ __forceinline__ float2 load_sample<KSJ_GPU_SAMPLES_CF32>(const void* base, size_t index) {
  return __ldg(static_cast<const float2*>(base) + index);
}

template <>
__device__ __forceinline__ float2 load_sample<KSJ_GPU_SAMPLES_BF16>(const void* base, size_t index) {
  const uint32_t packed = __ldg(static_cast<const uint32_t*>(base) + index);
  return make_float2(bf16_to_float(static_cast<uint16_t>(packed & 0xffffu)),
                     bf16_to_float(static_cast<uint16_t>(packed >> 16)));
}

// A sample by row index from a lane's own base: `lane_base` points at this
// lane's coil of sample 0 and `row_bytes` is one sample row (channels x
// element bytes, < 2^32), so the address is one 32 x 32 -> 64-bit
// multiply-add per load.
template <uint32_t kFormat>
struct SampleRows {
  static constexpr uint32_t kBytes = kFormat == KSJ_GPU_SAMPLES_BF16 ? 4u : 8u;
  const unsigned char* lane_base;
  uint32_t row_bytes;
  __device__ __forceinline__ SampleRows(const void* samples, size_t lane_index, int channels)
      : lane_base(static_cast<const unsigned char*>(samples) + lane_index * kBytes),
        row_bytes(static_cast<uint32_t>(channels) * kBytes) {}
  __device__ __forceinline__ float2 operator()(uint32_t row) const {
    return load_sample<kFormat>(lane_base + static_cast<uint64_t>(row) * row_bytes, 0);
  }
};

// -------------------------------------------------------------------- FFT

// In-place R-point inverse DFT (exp(+2 pi i j k / R)) on registers.
template <int R>
__device__ __forceinline__ void dft_inverse(float2* v);

template <>
__device__ __forceinline__ void dft_inverse<2>(float2* v) {
  const float2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <>
__device__ __forceinline__ void dft_inverse<3>(float2* v) {
  constexpr float kS3 = 0.8660254037844386f;  // sin(2 pi / 3)
  const float2 t1 = cadd(v[1], v[2]);
  const float2 t2 = make_float2(fmaf(-0.5f, t1.x, v[0].x), fmaf(-0.5f, t1.y, v[0].y));
  const float2 t3 = cscale(csub(v[1], v[2]), kS3);
  v[0] = cadd(v[0], t1);
  v[1] = make_float2(t2.x - t3.y, t2.y + t3.x);
  v[2] = make_float2(t2.x + t3.y, t2.y - t3.x);
}

template <>
__device__ __forceinline__ void dft_inverse<4>(float2* v) {
  const float2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
  const float2 c = cadd(v[1], v[3]), d = cmul_i(csub(v[1], v[3]));
  v[0] = cadd(a, c);
  v[2] = csub(a, c);
  v[1] = cadd(b, d);
  v[3] = csub(b, d);
}

template <>
__device__ __forceinline__ void dft_inverse<8>(float2* v) {
  constexpr float kC = 0.70710678118654752f;
  float2 e[4] = {v[0], v[2], v[4], v[6]};
  float2 o[4] = {v[1], v[3], v[5], v[7]};
  dft_inverse<4>(e);
  dft_inverse<4>(o);
  // o[k] *= exp(2 pi i k / 8)
  o[1] = make_float2((o[1].x - o[1].y) * kC, (o[1].x + o[1].y) * kC);
  o[2] = cmul_i(o[2]);
  o[3] = make_float2(-(o[3].x + o[3].y) * kC, (o[3].x - o[3].y) * kC);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = cadd(e[k], o[k]);
    v[k + 4] = csub(e[k], o[k]);
  }
}

template <>
__device__ __forceinline__ void dft_inverse<6>(float2* v) {
  // 2-point DFTs of (x_j, x_{j+3}); the sums give the even outputs through a
  // 3-point DFT, the differences times exp(i pi j / 3) the odd ones
  constexpr float kS3 = 0.8660254037844386f;  // sin(pi / 3)
  float2 e[3], o[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    e[j] = cadd(v[j], v[j + 3]);
    o[j] = csub(v[j], v[j + 3]);
  }
  o[1] = make_float2(0.5f * o[1].x - kS3 * o[1].y, kS3 * o[1].x + 0.5f * o[1].y);
  o[2] = make_float2(-0.5f * o[2].x - kS3 * o[2].y, kS3 * o[2].x - 0.5f * o[2].y);
  dft_inverse<3>(e);
  dft_inverse<3>(o);
  v[0] = e[0];
  v[1] = o[0];
  v[2] = e[1];
  v[3] = o[1];
  v[4] = e[2];
  v[5] = o[2];
}

// exp(2 pi i t / 5) and exp(2 pi i t / 7), t = 1 .. R-1 (cos, sin), as
// double literals.
__host__ __device__ constexpr double omega_odd(int r, int t, int part) {
  // r = 5: cos 72, 144 degrees, sin 72, 144; t > R/2 by symmetry
  return r == 5 ? (t == 1   ? (part ? 0.9510565162951535 : 0.30901699437494745)
                   : t == 2 ? (part ? 0.5877852522924731 : -0.8090169943749475)
                   : t == 3 ? (part ? -0.5877852522924731 : -0.8090169943749475)
                            : (part ? -0.9510565162951535 : 0.30901699437494745))
                : (t == 1   ? (part ? 0.7818314824680298 : 0.6234898018587336)
                   : t == 2 ? (part ? 0.9749279121818236 : -0.22252093395631434)
                   : t == 3 ? (part ? 0.4338837391175582 : -0.9009688679024191)
                   : t == 4 ? (part ? -0.4338837391175582 : -0.9009688679024191)
                   : t == 5 ? (part ? -0.9749279121818236 : -0.22252093395631434)
                            : (part ? -0.7818314824680298 : 0.6234898018587336));
}

// R-point inverse DFT for R = 5, 7 by its definition (R^2 complex
// multiply-adds with constant twiddles; the inputs' pairwise sums and
// differences halve the products).
template <int R>
__device__ __forceinline__ void dft_inverse_odd(float2* v) {
  constexpr int H = R / 2;
  float2 sum[H + 1], dif[H + 1];
#pragma unroll
  for (int j = 1; j <= H; ++j) {
    sum[j] = cadd(v[j], v[R - j]);
    dif[j] = csub(v[j], v[R - j]);
  }
  float2 out[R];
  out[0] = v[0];
#pragma unroll
  for (int j = 1; j <= H; ++j) out[0] = cadd(out[0], sum[j]);
#pragma unroll
  for (int k = 1; k <= H; ++k) {
    // X[k] = x0 + sum_j (cos(2 pi jk/R) sum_j + i sin(2 pi jk/R) dif_j); X[R-k] has -i
    float2 re = v[0], im = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int j = 1; j <= H; ++j) {
      const float c = static_cast<float>(omega_odd(R, (j * k) % R, 0));
      const float sn = static_cast<float>(omega_odd(R, (j * k) % R, 1));
      re = make_float2(fmaf(c, sum[j].x, re.x), fmaf(c, sum[j].y, re.y));
      im = make_float2(fmaf(sn, dif[j].x, im.x), fmaf(sn, dif[j].y, im.y));
    }
    // i * im = (-im.y, im.x)
    out[k] = make_float2(re.x - im.y, re.y + im.x);
    out[R - k] = make_float2(re.x + im.y, re.y - im.x);
  }
#pragma unroll
  for (int k = 0; k < R; ++k) v[k] = out[k];
}

template <>
__device__ __forceinline__ void dft_inverse<5>(float2* v) {
  dft_inverse_odd<5>(v);
}

template <>
__device__ __forceinline__ void dft_inverse<7>(float2* v) {
  dft_inverse_odd<7>(v);
}

// cos(2 pi r / 96) for r in [0, 24] (a quarter turn), as double literals.
__host__ __device__ constexpr double cos96(int r) {
  switch (r) {
    case 0: return 1.0;
    case 1: return 0.9978589232386035;
    case 2: return 0.9914448613738104;
    case 3: return 0.9807852804032304;
    case 4: return 0.9659258262890683;
    case 5: return 0.9469301294951057;
    case 6: return 0.9238795325112867;
    case 7: return 0.8968727415326884;
    case 8: return 0.8660254037844387;
    case 9: return 0.8314696123025452;
    case 10: return 0.7933533402912352;
    case 11: return 0.7518398074789774;
    case 12: return 0.7071067811865476;
    case 13: return 0.6593458151000688;
    case 14: return 0.6087614290087207;
    case 15: return 0.5555702330196024;
    case 16: return 0.5;
    case 17: return 0.44228869021900125;
    case 18: return 0.38268343236508984;
    case 19: return 0.3214394653031617;
    case 20: return 0.25881904510252074;
    case 21: return 0.19509032201612833;
    case 22: return 0.1305261922200517;
    case 23: return 0.06540312923014327;
    default: return 0.0;
  }
}

// exp(2 pi i m / 96) for m in [0, 96): a whole number of quarter turns times
// the first-quadrant value.  Called with m known at compile time (unrolled
// loops), it folds to two float constants.
__device__ __forceinline__ float2 omega96(int m) {
  const int q = m / 24, r = m - 24 * (m / 24);
  const float c = static_cast<float>(cos96(r)), s = static_cast<float>(cos96(24 - r));
  switch (q & 3) {
    case 0: return make_float2(c, s);
    case 1: return make_float2(-s, c);
    case 2: return make_float2(-c, -s);
    default: return make_float2(s, -c);
  }
}

// Two-factor split L = P * Q of the in-register DFT lengths above 8.
template <int L>
struct DftSplit;
template <>
struct DftSplit<12> { static constexpr int P = 3, Q = 4; };
template <>
struct DftSplit<16> { static constexpr int P = 4, Q = 4; };
template <>
struct DftSplit<24> { static constexpr int P = 3, Q = 8; };
template <>
struct DftSplit<32> { static constexpr int P = 4, Q = 8; };

// In-place L-point inverse DFT on registers, natural order in and out.  For
// L = P * Q > 8 (Cooley-Tukey, n = Q p + q, k = k1 + P k2): the P-point DFTs
// over p of x[Q p + q], times exp(2 pi i q k1 / L), then the Q-point DFTs over
// q give X[k1 + P k2].
template <int L>
__device__ __forceinline__ void dft_reg(float2* v) {
  if constexpr (L == 2 || L == 3 || L == 4 || L == 6 || L == 8) {
    dft_inverse<L>(v);
  } else {
    constexpr int P = DftSplit<L>::P, Q = DftSplit<L>::Q;
    static_assert(96 % L == 0, "twiddles are multiples of 2 pi / 96");
    float2 t[Q][P];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
#pragma unroll
      for (int p = 0; p < P; ++p) t[q][p] = v[Q * p + q];
      dft_inverse<P>(t[q]);
    }
#pragma unroll
    for (int q = 1; q < Q; ++q) {
#pragma unroll
      for (int k1 = 1; k1 < P; ++k1) t[q][k1] = cmul(t[q][k1], omega96(q * k1 * (96 / L)));
    }
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) {
      float2 u[Q];
#pragma unroll
      for (int q = 0; q < Q; ++q) u[q] = t[q][k1];
      dft_inverse<Q>(u);
#pragma unroll
      for (int k2 = 0; k2 < Q; ++k2) v[k1 + P * k2] = u[k2];
    }
  }
}

// Unnormalised inverse DFT (exp(+2 pi i n k / N)) of every line of a block
// held in shared memory as [column][line] (lines = 1 << lg_lines), in two
// steps for N = N1 * N2 (n = N2 n1 + n2, k = k1 + N1 k2):
//   A  for each (n2, line): the N1-point DFT over n1 of x[N2 n1 + n2], times
//      exp(2 pi i n2 k1 / N), written back in place at column N2 k1 + n2;
//   B  for each (k1, line): the N2-point DFT over n2 of those N2 contiguous
//      columns gives X[k1 + N1 k2], handed to emit(k, line, value) instead of
//      being stored back.
// tw[t] = exp(2 pi i t / N).  Synchronises the block between the steps
// (kBarId 0), or only the nthreads threads of named barrier kBarId; the
// caller synchronises before (the block is complete) as needed after.
template <int N1, int N2, int kBarId = 0, typename Emit>
__device__ __forceinline__ void fft_two_step(float2* smem, int lg_lines, const float2* __restrict__ tw, int tid,
                                             int nthreads, Emit&& emit) {
  const int lines = 1 << lg_lines;
  for (int u = tid; u < N2 * lines; u += nthreads) {
    const int line = u & (lines - 1), n2 = u >> lg_lines;
    float2* e = smem + (n2 << lg_lines) + line;
    float2 v[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) v[n1] = e[(N2 * n1) << lg_lines];
    dft_reg<N1>(v);
#pragma unroll
    for (int k1 = 1; k1 < N1; ++k1) v[k1] = cmul(v[k1], tw[n2 * k1]);
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) e[(N2 * k1) << lg_lines] = v[k1];
  }
  if constexpr (kBarId == 0)
    __syncthreads();
  else
    asm volatile("bar.sync %0, %1;" ::"n"(kBarId), "r"(nthreads) : "memory");
  for (int u = tid; u < N1 * lines; u += nthreads) {
    const int line = u & (lines - 1), k1 = u >> lg_lines;
    const float2* e = smem + ((N2 * k1) << lg_lines) + line;
    float2 v[N2];
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) v[n2] = e[n2 << lg_lines];
    dft_reg<N2>(v);
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) emit(k1 + N1 * k2, line, v[k2]);
  }
}

// The two-step transform above for the sigma = 2 crop: of the N = N1 * N2
// outputs only the N/2 frequencies k in [-N/4, N/4) are kept, i.e. k2 <
// N2/4 (k = k1 + N1 k2 < N/4) and k2 >= 3 N2/4 (k >= 3N/4), which the kept
// index p = (k + N/4) mod N places at k + N/4 and k - 3N/4.  With k2
// unrolled, both the kept set and p are known at compile time: no per-output
// range checks, and the outputs nobody uses are never computed.  live(line)
// false skips a line in both steps (padded coils, columns past the image).
// emit(p, slot, line, v): slot = N2 k1 + k2 is the column step B read the
// output's inputs from (the caller may overwrite it).
template <int N1, int N2, int kBarId = 0, typename Live, typename Emit>
__device__ __forceinline__ void fft_two_step_half(float2* smem, int lg_lines, const float2* __restrict__ tw, int tid,
                                                  int nthreads, Live&& live, Emit&& emit) {
  static_assert(N2 % 4 == 0, "the kept quarter-bands split on k2");
  constexpr int kN = N1 * N2;
  const int lines = 1 << lg_lines;
  for (int u = tid; u < N2 * lines; u += nthreads) {
    const int line = u & (lines - 1), n2 = u >> lg_lines;
    if (!live(line)) continue;
    float2* e = smem + (n2 << lg_lines) + line;
    float2 v[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) v[n1] = e[(N2 * n1) << lg_lines];
    dft_reg<N1>(v);
#pragma unroll
    for (int k1 = 1; k1 < N1; ++k1) v[k1] = cmul(v[k1], tw[n2 * k1]);
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) e[(N2 * k1) << lg_lines] = v[k1];
  }
  if constexpr (kBarId == 0)
    __syncthreads();
  else
    asm volatile("bar.sync %0, %1;" ::"n"(kBarId), "r"(nthreads) : "memory");
  for (int u = tid; u < N1 * lines; u += nthreads) {
    const int line = u & (lines - 1), k1 = u >> lg_lines;
    if (!live(line)) continue;
    const float2* e = smem + ((N2 * k1) << lg_lines) + line;
    float2 v[N2];
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) v[n2] = e[n2 << lg_lines];
    dft_reg<N2>(v);
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) {
      if (k2 < N2 / 4)
        emit(k1 + N1 * k2 + kN / 4, N2 * k1 + k2, line, v[k2]);
      else if (k2 >= 3 * N2 / 4)
        emit(k1 + N1 * k2 - 3 * kN / 4, N2 * k1 + k2, line, v[k2]);
    }
  }
}

// Row lengths up to kMaxN with a two-step form (N1 = 16): false for any other n.
template <int kMaxN, int kBarId = 0, typename Emit>
__device__ __forceinline__ bool fft_two_step_rows(int n, float2* smem, int lg_lines, const float2* tw, int tid,
                                                  int nthreads, Emit&& emit) {
  switch (n) {
    case 128: fft_two_step<16, 8, kBarId>(smem, lg_lines, tw, tid, nthreads, emit); return true;
    case 192: fft_two_step<16, 12, kBarId>(smem, lg_lines, tw, tid, nthreads, emit); return true;
    case 256: fft_two_step<16, 16, kBarId>(smem, lg_lines, tw, tid, nthreads, emit); return true;
    case 384: fft_two_step<16, 24, kBarId>(smem, lg_lines, tw, tid, nthreads, emit); return true;
    case 512:
      if constexpr (kMaxN >= 512) {
        fft_two_step<16, 32, kBarId>(smem, lg_lines, tw, tid, nthreads, emit);
        return true;
      }
      return false;
    default: return false;
  }
}
__host__ __device__ constexpr bool has_two_step_rows(int n) {
  return n == 128 || n == 192 || n == 256 || n == 384 || n == 512;
}
// Column of X[k] when step B stores its outputs in place (over the N2
// columns it read): N2 * (k mod 16) + k / 16.
__host__ __device__ constexpr int two_step_slot(int k, int n) { return (k & 15) * (n >> 4) + (k >> 4); }

// In-place mixed-radix decimation-in-frequency plan for n = 2^a 3^b 5^c 7^d
// (n <= 4096).  For n = 2^a 3^b with b <= 1: a factor 3 first (as radix 6
// when n is even), then radix-8 stages, then a final 4 or 2, so every block
// length after the first stage is a power of two and all indexing is
// shifts.  Otherwise the odd factors come first, one stage each (7s, 5s, 3s),
// then the power of two as above; stages whose sub-block length is not a
// power of two index with divisions (lg_m = -1).  Stage s splits blocks of
// length m[s] * radix[s] into radix[s] sub-blocks of length m[s]; its
// twiddles are exp(2 pi i (i * d * tw_stride[s]) / n).  The output X[k] ends
// at dif_position(k) (digit reversal).
struct DifPlan {
  int n;
  int stages;
  int radix[16];
  int lg_m[16];       // log2 of the sub-block length, or -1 when it is not a power of two
  int m[16];          // sub-block length
  int nbf[16];        // butterflies per line: n / radix
  int tw_stride[16];  // n / block length
};

inline bool make_dif_plan(int n, DifPlan* p) {
  if (n < 2 || n > 4096) return false;
  int m = n, threes = 0, fives = 0, sevens = 0;
  while (m % 7 == 0) {
    m /= 7;
    ++sevens;
  }
  while (m % 5 == 0) {
    m /= 5;
    ++fives;
  }
  while (m % 3 == 0) {
    m /= 3;
    ++threes;
  }
  if ((m & (m - 1)) != 0) return false;
  int rad[16];
  int ns = 0;
  if (threes <= 1 && fives == 0 && sevens == 0) {
    if (threes) {
      if (m >= 2) {
        rad[ns++] = 6;
        m /= 2;
      } else {
        rad[ns++] = 3;
      }
    }
  } else {
    for (int i = 0; i < sevens; ++i) rad[ns++] = 7;
    for (int i = 0; i < fives; ++i) rad[ns++] = 5;
    for (int i = 0; i < threes; ++i) rad[ns++] = 3;
  }
  while (m >= 8) {
    rad[ns++] = 8;
    m /= 8;
  }
  if (m == 4) rad[ns++] = 4;
  if (m == 2) rad[ns++] = 2;
  p->n = n;
  p->stages = ns;
  int len = n;
  for (int s = 0; s < ns; ++s) {
    const int sub = len / rad[s];
    int lg = 0;
    while ((1 << lg) < sub) ++lg;
    p->radix[s] = rad[s];
    p->lg_m[s] = (1 << lg) == sub ? lg : -1;
    p->m[s] = sub;
    p->nbf[s] = n / rad[s];
    p->tw_stride[s] = n / len;
    len = sub;
  }
  return true;
}

// Position of output X[k] after all stages of `p`.
__host__ __device__ inline int dif_position(const DifPlan& p, int k) {
  int pos = 0, len = p.n;
  for (int s = 0; s < p.stages; ++s) {
    const int r = p.radix[s];
    len /= r;
    pos += (k % r) * len;
    k /= r;
  }
  return pos;
}

// One DIF stage over 2^lg_lines lines held line-contiguous in shared memory:
// element (line, index) at smem[(index << lg_lines) + line].  A thread keeps
// one line (tid mod lines) and walks that line's butterflies, two at a time
// so that both sets of loads are in flight together; a butterfly reads and
// writes the same radix elements, so no thread needs another's result
// within the stage.
template <int R>
__device__ __forceinline__ void dif_stage(float2* smem, int lg_lines, int nbf, int lg_m, int tws,
                                          const float2* __restrict__ tw, int tid, int nthreads) {
  const int line = tid & ((1 << lg_lines) - 1);
  const int step = nthreads >> lg_lines;
  const int mmask = (1 << lg_m) - 1;
  auto base_of = [&](int u) { return (((u >> lg_m) * R) << lg_m) + (u & mmask); };
  auto finish = [&](float2* v, int u, int base) {
    dft_inverse<R>(v);
    const int i = u & mmask;
    if (i != 0) {
#pragma unroll
      for (int d = 1; d < R; ++d) v[d] = cmul(v[d], tw[i * d * tws]);
    }
#pragma unroll
    for (int d = 0; d < R; ++d) smem[((base + (d << lg_m)) << lg_lines) + line] = v[d];
  };
  int u = tid >> lg_lines;
  for (; u + step < nbf; u += 2 * step) {
    const int ba = base_of(u), bb = base_of(u + step);
    float2 va[R], vb[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      va[r] = smem[((ba + (r << lg_m)) << lg_lines) + line];
      vb[r] = smem[((bb + (r << lg_m)) << lg_lines) + line];
    }
    finish(va, u, ba);
    finish(vb, u + step, bb);
  }
  if (u < nbf) {
    const int ba = base_of(u);
    float2 va[R];
#pragma unroll
    for (int r = 0; r < R; ++r) va[r] = smem[((ba + (r << lg_m)) << lg_lines) + line];
    finish(va, u, ba);
  }
}

// The same stage with two adjacent lines per thread: one 16-byte access
// moves an element of both lines, and the lines share the twiddle loads and
// the index arithmetic.  Needs an even line count (16-byte aligned smem).
template <int R>
__device__ __forceinline__ void dif_stage_pairs(float2* smem, int lg_lines, int nbf, int lg_m, int tws,
                                                const float2* __restrict__ tw, int tid, int nthreads) {
  const int lg_pairs = lg_lines - 1;
  const int lp = tid & ((1 << lg_pairs) - 1);
  const int step = nthreads >> lg_pairs;
  const int mmask = (1 << lg_m) - 1;
  float4* s4 = reinterpret_cast<float4*>(smem);  // elements (2 lp, 2 lp + 1) of index x at s4[(x << lg_pairs) + lp]
  for (int u = tid >> lg_pairs; u < nbf; u += step) {
    const int base = (((u >> lg_m) * R) << lg_m) + (u & mmask);
    float4* e = s4 + (base << lg_pairs) + lp;
    const int stride = 1 << (lg_m + lg_pairs);
    float2 va[R], vb[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const float4 q = e[r * stride];
      va[r] = make_float2(q.x, q.y);
      vb[r] = make_float2(q.z, q.w);
    }
    dft_inverse<R>(va);
    dft_inverse<R>(vb);
    const int i = u & mmask;
    if (i != 0) {
#pragma unroll
      for (int d = 1; d < R; ++d) {
        const float2 w = tw[i * d * tws];
        va[d] = cmul(va[d], w);
        vb[d] = cmul(vb[d], w);
      }
    }
#pragma unroll
    for (int d = 0; d < R; ++d) e[d * stride] = make_float4(va[d].x, va[d].y, vb[d].x, vb[d].y);
  }
}

// A DIF stage whose sub-block length m is not a power of two (plans with
// several odd factors): the butterfly u of each line starts at
// (u / m) * R * m + u mod m; one line per thread as in dif_stage.
template <int R>
__device__ __forceinline__ void dif_stage_any(float2* smem, int lg_lines, int nbf, int m, int tws,
                                              const float2* __restrict__ tw, int tid, int nthreads) {
  const int line = tid & ((1 << lg_lines) - 1);
  const int step = nthreads >> lg_lines;
  for (int u = tid >> lg_lines; u < nbf; u += step) {
    const int blk = u / m, i = u - blk * m;
    const int base = blk * R * m + i;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = smem[((base + r * m) << lg_lines) + line];
    dft_inverse<R>(v);
    if (i != 0) {
#pragma unroll
      for (int d = 1; d < R; ++d) v[d] = cmul(v[d], tw[i * d * tws]);
    }
#pragma unroll
    for (int d = 0; d < R; ++d) smem[((base + d * m) << lg_lines) + line] = v[d];
  }
}

// Unnormalised inverse FFT (exp(+2 pi i n k / N)) of every line, in place,
// output digit-reversed; tw[t] = exp(2 pi i t / n).  Requires nthreads to be
// a multiple of the line count.  Synchronises the block after each stage.
__device__ __forceinline__ void dif_lines(float2* smem, int lg_lines, const DifPlan& p,
                                          const float2* __restrict__ tw, int tid, int nthreads) {
  for (int s = 0; s < p.stages; ++s) {
    const int nbf = p.nbf[s], lg_m = p.lg_m[s], tws = p.tw_stride[s];
    if (lg_m < 0 || p.radix[s] == 5 || p.radix[s] == 7) {
      switch (p.radix[s]) {
        case 8: dif_stage_any<8>(smem, lg_lines, nbf, p.m[s], tws, tw, tid, nthreads); break;
        case 7: dif_stage_any<7>(smem, lg_lines, nbf, p.m[s], tws, tw, tid, nthreads); break;
        case 5: dif_stage_any<5>(smem, lg_lines, nbf, p.m[s], tws, tw, tid, nthreads); break;
        case 4: dif_stage_any<4>(smem, lg_lines, nbf, p.m[s], tws, tw, tid, nthreads); break;
        case 3: dif_stage_any<3>(smem, lg_lines, nbf, p.m[s], tws, tw, tid, nthreads); break;
        default: dif_stage_any<2>(smem, lg_lines, nbf, p.m[s], tws, tw, tid, nthreads); break;
      }
      __syncthreads();
      continue;
    }
    if (lg_lines >= 1) {
      switch (p.radix[s]) {
        case 8: dif_stage_pairs<8>(smem, lg_lines, nbf, lg_m, tws, tw, tid, nthreads); break;
        case 6: dif_stage_pairs<6>(smem, lg_lines, nbf, lg_m, tws, tw, tid, nthreads); break;
        case 4: dif_stage_pairs<4>(smem, lg_lines, nbf, lg_m, tws, tw, tid, nthreads); break;
        case 3: dif_stage_pairs<3>(smem, lg_lines, nbf, lg_m, tws, tw, tid, nthreads); break;
        default: dif_stage_pairs<2>(smem, lg_lines, nbf, lg_m, tws, tw, tid, nthreads); break;
      }
    } else {
      switch (p.radix[s]) {
        case 8: dif_stage<8>(smem, lg_lines, nbf, lg_m, tws, tw, tid, nthreads); break;
        case 6: dif_stage<6>(smem, lg_lines, nbf, lg_m, tws, tw, tid, nthreads); break;
        case 4: dif_stage<4>(smem, lg_lines, nbf, lg_m, tws, tw, tid, nthreads); break;
        case 3: dif_stage<3>(smem, lg_lines, nbf, lg_m, tws, tw, tid, nthreads); break;
        default: dif_stage<2>(smem, lg_lines, nbf, lg_m, tws, tw, tid, nthreads); break;
      }
    }
    __syncthreads();
  }
}

__host__ __device__ __forceinline__ int ilog2(int v) {
  int r = 0;
  while ((1 << (r + 1)) <= v) ++r;
  return r;
}

// exp(2 pi i t / n) in float.  The angle is split into the nearest quarter
// turn (an exact rotation) and a remainder pi * x with |x| <= 1/4, so the one
// rounding of x = rem / (2n) moves the angle by at most ~5e-8 rad.
__device__ __forceinline__ float2 twiddle(int t, int n) {
  const int t4 = 4 * t;
  const int q = (2 * t4 + n) / (2 * n);  // nearest quarter turn, t >= 0
  const int rem = t4 - q * n;            // in [-n/2, n/2]
  float s, c;
  sincospif(static_cast<float>(rem) / static_cast<float>(2 * n), &s, &c);
  switch (q & 3) {
    case 0: return make_float2(c, s);
    case 1: return make_float2(-s, c);
    case 2: return make_float2(-c, -s);
    default: return make_float2(s, -c);
  }
}

// [frame][a][b] -> [frame][b][a] for 4- or 8-byte elements, 32x32 tiles
// through shared memory (launch with blockDim (32, 8), grid (ceil(nb/32),
// ceil(na/32), frames)).
template <typename T>
__global__ void __launch_bounds__(256) k_transpose(const T* in, T* out, int na, int nb) {
  __shared__ T t[32][33];
  const int f = blockIdx.z;
  const int b0 = blockIdx.x * 32;
  const int a0 = blockIdx.y * 32;
  const T* src = in + static_cast<size_t>(f) * na * nb;
  T* dst = out + static_cast<size_t>(f) * na * nb;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int a = a0 + y, b = b0 + threadIdx.x;
    if (a < na && b < nb) t[y][threadIdx.x] = src[static_cast<size_t>(a) * nb + b];
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int b = b0 + y, a = a0 + threadIdx.x;
    if (a < na && b < nb) dst[static_cast<size_t>(b) * na + a] = t[threadIdx.x][y];
  }
}

// ------------------------------------------------ TMA and mbarrier helpers

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Make mbarrier initialisation visible to the async proxy (TMA unit).
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Order earlier generic-proxy shared-memory accesses before later async-proxy ones.
__device__ __forceinline__ void fence_proxy_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait_parity(uint64_t* bar, uint32_t parity) {
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

// Bounded wait: true when the phase completed, false after `limit` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait_parity(bar, parity)) return true;
  return false;
}

// 3-D tiled TMA load of one box into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_3d(void* dst, const void* tensor_map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(tensor_map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

}  // namespace ksj_gpu
