// ksj_gpu_forward.cu -- Kaiser-Bessel forward NUFFT (coil images -> non-Cartesian
// samples) on sm_103a: the exact transpose of the Kaiser-Bessel gridding
// adjoint of ksj_gpu_gridding.cu without density weights.
//
// The adjoint is A^H = D Crop IDFT_cols IDFT_rows Spread diag(e): spread each
// weighted sample onto the oversampled grid, inverse transforms, keep the
// central n x n, deapodise.  Its transpose, the forward operator, is
//   A = diag(conj e) Interp DFT_rows DFT_cols Pad D:
//   k_fwd_cols    deapodise (the adjoint's factors), place each image column at
//                 the adjoint's crop positions (p - n/2) mod g, forward DFT along
//                 the column (conj -> inverse transform -> conj), write
//                 [frame][grid_row][image_col][coil];
//   k_fwd_rows    place each row's n columns the same way, forward DFT along the
//                 row, write the whole grid [frame][grid_row][grid_col][coil];
//   k_fwd_interp  per sample the W x W taps and phase of the adjoint's k_prepare
//                 (same grid coordinate, floor, Kaiser-Bessel weights and
//                 e = exp(i k . delta)), y = conj(e) sum w_r w_c grid[r][c].
// The reference's own forward (nufft2_forward on its Eigen backend) is the
// direct NUDFT (ksj_gpu_direct_forward); this is the fast approximation of it
// the gridding adjoint pairs with.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "ksj_gpu.h"
#include "ksj_gpu_internal.cuh"

namespace ksj_gpu {
namespace {

constexpr int kFwdThreads = 256;
constexpr int kFwdWarps = kFwdThreads / 32;

struct FwdArgs {
  const float2* tw;     // exp(2 pi i t / g)
  const float* inv_d;   // deapodisation factor of kept pixel p
  const int* pos;       // output position of frequency k after the in-place transform (other lengths)
  DifPlan plan;
  int frames, channels, samples, n, g, cg, cpitch;
};

// Twiddles, deapodisation factors and in-place output positions of one axis.
__global__ void k_fwd_tables(float2* tw, float* inv_d, int* pos, int n, int g, int width, double beta, double i0_beta,
                             DifPlan plan) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < g) {
    tw[i] = twiddle(i, g);
    pos[i] = dif_position(plan, i);
  }
  if (i < n) inv_d[i] = kb_inv_deapod(i, n, g, width, beta, i0_beta);
}

// Forward DFT of the cg lines held [g][line] in shared memory (conj ->
// inverse transform -> conj), each output handed to emit(k, line, value).
template <int kN, typename Emit>
__device__ __forceinline__ void fwd_lines(float2* buf, int lg, const FwdArgs& a, const float2* tw, Emit&& emit) {
  auto conj_emit = [&](int k, int line, float2 v) { emit(k, line, make_float2(v.x, -v.y)); };
  if constexpr (kN != 0) {
    fft_two_step<16, kN / 16>(buf, lg, tw, threadIdx.x, blockDim.x, conj_emit);
  } else {
    dif_lines(buf, lg, a.plan, tw, threadIdx.x, blockDim.x);
    const int line = threadIdx.x & (a.cg - 1);
    for (int k = threadIdx.x >> lg; k < a.g; k += blockDim.x >> lg)
      conj_emit(k, line, buf[(__ldg(a.pos + k) << lg) + line]);
  }
}

// One block per (image column, coil group, frame).
template <int kN>
__global__ void __launch_bounds__(kFwdThreads) k_fwd_cols(const float2* __restrict__ image, float2* t1, FwdArgs a) {
  extern __shared__ __align__(16) float2 fwd_smem[];
  float2* buf = fwd_smem;
  float2* tw = fwd_smem + static_cast<size_t>(a.g) * a.cg;
  const int x = blockIdx.x, cgi = blockIdx.y, f = blockIdx.z;
  const int lg = ilog2(a.cg);
  for (int i = threadIdx.x; i < a.g * a.cg; i += blockDim.x) buf[i] = make_float2(0.0f, 0.0f);
  for (int i = threadIdx.x; i < a.g; i += blockDim.x) tw[i] = a.tw[i];
  __syncthreads();
  const float dx = __ldg(a.inv_d + x);
  for (int i = threadIdx.x; i < a.n * a.cg; i += blockDim.x) {
    const int y = i >> lg, c = i & (a.cg - 1), gc = cgi * a.cg + c;
    if (gc >= a.channels) continue;
    float2 v = __ldg(image + ((static_cast<size_t>(f) * a.n + y) * a.n + x) * a.channels + gc);
    const float sc = __ldg(a.inv_d + y) * dx;
    v.x *= sc;
    v.y *= sc;
    int k = y - a.n / 2;
    if (k < 0) k += a.g;
    buf[(k << lg) + c] = make_float2(v.x, -v.y);
  }
  __syncthreads();
  float2* dst = t1 + static_cast<size_t>(f) * a.g * a.n * a.cpitch + static_cast<size_t>(x) * a.cpitch + cgi * a.cg;
  const int live = min(a.cg, a.channels - cgi * a.cg);
  fwd_lines<kN>(buf, lg, a, tw, [&](int k, int line, float2 v) {
    if (line < live) dst[static_cast<size_t>(k) * a.n * a.cpitch + line] = v;
  });
}

// One block per (grid row, coil group, frame).
template <int kN>
__global__ void __launch_bounds__(kFwdThreads) k_fwd_rows(const float2* __restrict__ t1, float2* grid, FwdArgs a) {
  extern __shared__ __align__(16) float2 fwd_smem[];
  float2* buf = fwd_smem;
  float2* tw = fwd_smem + static_cast<size_t>(a.g) * a.cg;
  const int kr = blockIdx.x, cgi = blockIdx.y, f = blockIdx.z;
  const int lg = ilog2(a.cg);
  for (int i = threadIdx.x; i < a.g * a.cg; i += blockDim.x) buf[i] = make_float2(0.0f, 0.0f);
  for (int i = threadIdx.x; i < a.g; i += blockDim.x) tw[i] = a.tw[i];
  __syncthreads();
  const float2* src = t1 + (static_cast<size_t>(f) * a.g + kr) * a.n * a.cpitch + cgi * a.cg;
  for (int i = threadIdx.x; i < a.n * a.cg; i += blockDim.x) {
    const int x = i >> lg, c = i & (a.cg - 1);
    if (cgi * a.cg + c >= a.channels) continue;
    const float2 v = __ldg(src + static_cast<size_t>(x) * a.cpitch + c);
    int k = x - a.n / 2;
    if (k < 0) k += a.g;
    buf[(k << lg) + c] = make_float2(v.x, -v.y);
  }
  __syncthreads();
  float2* dst = grid + (static_cast<size_t>(f) * a.g + kr) * a.g * a.cpitch + cgi * a.cg;
  const int live = min(a.cg, a.channels - cgi * a.cg);
  fwd_lines<kN>(buf, lg, a, tw, [&](int k, int line, float2 v) {
    if (line < live) dst[static_cast<size_t>(k) * a.cpitch + line] = v;
  });
}

struct InterpArgs {
  const float2* grid;
  const float* traj;
  float2* out;
  uint32_t* flags;
  int frames, channels, samples, g, cpitch;
  float beta, two_over_w, inv_i0_beta, phase_row, phase_col;
};

// One warp per 32 consecutive samples of one frame and one group of 32 coils
// (lane = coil): the taps and phase of k_prepare's Kaiser-Bessel branch, the
// W x W weighted cells summed row by row, times conj(e); results staged in
// shared memory and written channel-major with coalesced stores.
template <int W>
__global__ void __launch_bounds__(kFwdThreads) k_fwd_interp(InterpArgs a) {
  __shared__ float2 tile[kFwdWarps][32][33];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int f = blockIdx.z, cgi = blockIdx.y;
  const int s0 = (blockIdx.x * kFwdWarps + warp) * 32;
  if (s0 >= a.samples) return;
  const int gc = cgi * 32 + lane;
  const bool coil_ok = gc < a.channels;
  const float2* grid = a.grid + static_cast<size_t>(f) * a.g * a.g * a.cpitch + (coil_ok ? gc : 0);
  const int ns = min(32, a.samples - s0);
  for (int i = 0; i < ns; ++i) {
    const size_t idx = static_cast<size_t>(f) * a.samples + s0 + i;
    const float2 k = __ldg(reinterpret_cast<const float2*>(a.traj) + idx);
    float2 y = make_float2(0.0f, 0.0f);
    const bool ok = isfinite(k.x) && isfinite(k.y) && fabsf(k.x) < 1.0e4f && fabsf(k.y) < 1.0e4f;
    if (!ok) {
      if (lane == 0) atomicOr(a.flags, KSJ_GPU_FLAG_BAD_TRAJECTORY);
    } else {
      const dfloat ur = grid_coordinate(k.x, static_cast<float>(a.g));
      const dfloat uc = grid_coordinate(k.y, static_cast<float>(a.g));
      float fr, fc;
      const int sr = dfloor(ur, &fr) - W / 2 + 1;
      const int sc = dfloor(uc, &fc) - W / 2 + 1;
      float wc[W];
#pragma unroll
      for (int j = 0; j < W; ++j)
        wc[j] = kb_weight(__fsub_rn(__fsub_rn(static_cast<float>(sc + j), uc.hi), uc.lo), a.two_over_w, a.beta,
                          a.inv_i0_beta);
      const int r0 = wrap_index(sr, a.g), c0 = wrap_index(sc, a.g);
      float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
      for (int i2 = 0; i2 < W; ++i2) {
        const float wr = kb_weight(__fsub_rn(__fsub_rn(static_cast<float>(sr + i2), ur.hi), ur.lo), a.two_over_w,
                                   a.beta, a.inv_i0_beta);
        int rr = r0 + i2;
        if (rr >= a.g) rr -= a.g;
        const float2* row = grid + static_cast<size_t>(rr) * a.g * a.cpitch;
#pragma unroll
        for (int j = 0; j < W; ++j) {
          int cc = c0 + j;
          if (cc >= a.g) cc -= a.g;
          const float w = wr * wc[j];
          const float2 v = coil_ok ? __ldg(row + static_cast<size_t>(cc) * a.cpitch) : make_float2(0.0f, 0.0f);
          acc.x = fmaf(v.x, w, acc.x);
          acc.y = fmaf(v.y, w, acc.y);
        }
      }
      const float2 e = exp_i_dot(k.x, a.phase_row, k.y, a.phase_col, 1.0f);
      y = cmul(acc, make_float2(e.x, -e.y));
    }
    tile[warp][i][lane] = y;
  }
  __syncwarp();
  float2* out = a.out + static_cast<size_t>(f) * a.channels * a.samples + s0 + lane;
  const int nc = min(32, a.channels - cgi * 32);
  for (int c = 0; c < nc; ++c)
    if (lane < ns) out[static_cast<size_t>(cgi * 32 + c) * a.samples] = tile[warp][lane][c];
}

struct FwdShape {
  int frames, channels, samples, n, g, width, cg, cpitch;
  double beta;
  float phase_row, phase_col;
  DifPlan plan;
  size_t flags, tables, t1, grid, total;
};

ksj_gpu_status make_fwd_shape(const ksj_gpu_gridding_desc* d, FwdShape* s) {
  if (d == nullptr || d->struct_size < sizeof(ksj_gpu_gridding_desc)) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (d->kernel != KSJ_GPU_KERNEL_KAISER_BESSEL || d->sample_format != KSJ_GPU_SAMPLES_CF32)
    return KSJ_GPU_ERROR_UNSUPPORTED;
  if (d->image_rows != d->image_cols || d->grid_rows != d->grid_cols || d->image_rows < 2 ||
      d->grid_rows < d->image_rows || d->channels == 0 || d->channels > 1024 || d->samples == 0 || d->frames == 0)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  const int w = static_cast<int>(d->kernel_width);
  if (w != 2 && w != 4 && w != 6 && w != 8) return KSJ_GPU_ERROR_UNSUPPORTED;
  DifPlan plan;
  if (d->grid_rows > 512 || !make_dif_plan(static_cast<int>(d->grid_rows), &plan)) return KSJ_GPU_ERROR_UNSUPPORTED;
  s->frames = static_cast<int>(d->frames);
  s->channels = static_cast<int>(d->channels);
  s->samples = static_cast<int>(d->samples);
  s->n = static_cast<int>(d->image_rows);
  s->g = static_cast<int>(d->grid_rows);
  s->width = w;
  s->plan = plan;
  s->cg = 2;
  while (s->cg < s->channels && s->cg < 32) s->cg <<= 1;
  s->cpitch = (s->channels + s->cg - 1) / s->cg * s->cg;
  s->beta = d->kb_beta > 0.0f ? static_cast<double>(d->kb_beta)
                              : kb_default_beta(w, static_cast<double>(s->g) / static_cast<double>(s->n));
  if (!(s->beta > 0.0)) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  // exp(i k . delta), delta = n/2 - origin, exact in float as the adjoint requires
  const double pr = static_cast<double>(s->n / 2) - d->row_origin, pc = static_cast<double>(s->n / 2) - d->col_origin;
  s->phase_row = static_cast<float>(pr);
  s->phase_col = static_cast<float>(pc);
  if (static_cast<double>(s->phase_row) != pr || static_cast<double>(s->phase_col) != pc)
    return KSJ_GPU_ERROR_UNSUPPORTED;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off = align_up(off + bytes, 256);
    return at;
  };
  s->flags = take(256);
  s->tables = take(static_cast<size_t>(s->g) * (sizeof(float2) + sizeof(int)) + static_cast<size_t>(s->n) * sizeof(float));
  s->t1 = take(static_cast<size_t>(s->frames) * s->g * s->n * s->cpitch * sizeof(float2));
  s->grid = take(static_cast<size_t>(s->frames) * s->g * s->g * s->cpitch * sizeof(float2));
  s->total = off;
  return KSJ_GPU_OK;
}

using FwdKernel = void (*)(const float2*, float2*, FwdArgs);

template <int kN>
void fwd_kernels(FwdKernel* cols, FwdKernel* rows) {
  *cols = k_fwd_cols<kN>;
  *rows = k_fwd_rows<kN>;
}

void fwd_kernels_for(int g, FwdKernel* cols, FwdKernel* rows) {
  switch (g) {
    case 128: return fwd_kernels<128>(cols, rows);
    case 192: return fwd_kernels<192>(cols, rows);
    case 256: return fwd_kernels<256>(cols, rows);
    case 384: return fwd_kernels<384>(cols, rows);
    case 512: return fwd_kernels<512>(cols, rows);
    default: return fwd_kernels<0>(cols, rows);
  }
}

template <int W>
void launch_interp(const InterpArgs& a, dim3 grid, cudaStream_t st) {
  LaunchScope scope("k_fwd_interp", st);
  k_fwd_interp<W><<<grid, kFwdThreads, 0, st>>>(a);
}

}  // namespace
}  // namespace ksj_gpu

using namespace ksj_gpu;

extern "C" size_t ksj_gpu_kb_forward_workspace_bytes(const ksj_gpu_gridding_desc* desc) {
  FwdShape s{};
  return make_fwd_shape(desc, &s) == KSJ_GPU_OK ? s.total : 0;
}

extern "C" ksj_gpu_status ksj_gpu_kb_forward(const ksj_gpu_gridding_desc* desc, const void* d_image,
                                             const float* d_traj, void* d_samples, void* d_workspace,
                                             size_t workspace_bytes, void* stream) {
  FwdShape s{};
  const ksj_gpu_status st = make_fwd_shape(desc, &s);
  if (st != KSJ_GPU_OK) return st;
  if (d_image == nullptr || d_traj == nullptr || d_samples == nullptr ||
      (reinterpret_cast<uintptr_t>(d_image) & 7u) != 0 || (reinterpret_cast<uintptr_t>(d_traj) & 7u) != 0 ||
      (reinterpret_cast<uintptr_t>(d_samples) & 7u) != 0)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (d_workspace == nullptr || (reinterpret_cast<uintptr_t>(d_workspace) & 255u) != 0 || workspace_bytes < s.total)
    return KSJ_GPU_ERROR_WORKSPACE;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  unsigned char* ws = static_cast<unsigned char*>(d_workspace);
  uint32_t* flags = reinterpret_cast<uint32_t*>(ws + s.flags);
  float2* tw = reinterpret_cast<float2*>(ws + s.tables);
  int* pos = reinterpret_cast<int*>(tw + s.g);
  float* inv_d = reinterpret_cast<float*>(pos + s.g);
  float2* t1 = reinterpret_cast<float2*>(ws + s.t1);
  float2* grid = reinterpret_cast<float2*>(ws + s.grid);
  if (cudaMemsetAsync(flags, 0, 256, cs) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  {
    LaunchScope scope("k_fwd_tables", cs);
    // the adjoint's tables take beta rounded to float (its kernel parameter)
    const double beta_t = static_cast<double>(static_cast<float>(s.beta));
    k_fwd_tables<<<(s.g + 255) / 256, 256, 0, cs>>>(tw, inv_d, pos, s.n, s.g, s.width, beta_t,
                                                    std::cyl_bessel_i(0.0, beta_t), s.plan);
  }
  FwdArgs a{tw, inv_d, pos, s.plan, s.frames, s.channels, s.samples, s.n, s.g, s.cg, s.cpitch};
  FwdKernel cols_k = nullptr, rows_k = nullptr;
  fwd_kernels_for(s.g, &cols_k, &rows_k);
  const size_t smem = (static_cast<size_t>(s.g) * s.cg + s.g) * sizeof(float2);
  if (cudaFuncSetAttribute(cols_k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) != cudaSuccess ||
      cudaFuncSetAttribute(rows_k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) != cudaSuccess)
    return KSJ_GPU_ERROR_CUDA;
  const int groups = (s.channels + s.cg - 1) / s.cg;
  {
    LaunchScope scope("k_fwd_cols", cs);
    cols_k<<<dim3(s.n, groups, s.frames), kFwdThreads, smem, cs>>>(static_cast<const float2*>(d_image), t1, a);
  }
  {
    LaunchScope scope("k_fwd_rows", cs);
    rows_k<<<dim3(s.g, groups, s.frames), kFwdThreads, smem, cs>>>(t1, grid, a);
  }
  InterpArgs ia{grid, d_traj, static_cast<float2*>(d_samples), flags, s.frames, s.channels, s.samples, s.g, s.cpitch,
                static_cast<float>(s.beta), 2.0f / static_cast<float>(s.width),
                static_cast<float>(1.0 / std::cyl_bessel_i(0.0, s.beta)), s.phase_row, s.phase_col};
  const dim3 ig((s.samples + 32 * kFwdWarps - 1) / (32 * kFwdWarps), (s.channels + 31) / 32, s.frames);
  switch (s.width) {
    case 2: launch_interp<2>(ia, ig, cs); break;
    case 4: launch_interp<4>(ia, ig, cs); break;
    case 6: launch_interp<6>(ia, ig, cs); break;
    default: launch_interp<8>(ia, ig, cs); break;
  }
  return check_launch();
}
