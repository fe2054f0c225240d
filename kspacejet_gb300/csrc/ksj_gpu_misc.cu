// ksj_gpu_misc.cu -- direct NUDFT adjoint, root-sum-of-squares combine, the
// device context used by the Provider plug-ins, and library bookkeeping.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>
#include <cstdint>
#include <cstring>
#include <new>

#include "ksj_gpu.h"
#include "ksj_gpu_internal.cuh"

namespace ksj_gpu {

namespace {
std::atomic<uint64_t> g_launches{0};
std::atomic<int> g_timing{0};

struct Pending {
  const char* name;
  cudaEvent_t start, stop;
};
struct Totals {
  std::string name;
  uint64_t launches = 0;
  double ms = 0.0;
};
std::mutex g_timing_mutex;
std::vector<Pending> g_pending;
std::vector<Totals> g_totals;

void settle_locked() {
  for (const Pending& p : g_pending) {
    float ms = 0.0f;
    if (cudaEventSynchronize(p.stop) == cudaSuccess && cudaEventElapsedTime(&ms, p.start, p.stop) == cudaSuccess) {
      Totals* t = nullptr;
      for (Totals& x : g_totals)
        if (x.name == p.name) t = &x;
      if (t == nullptr) {
        g_totals.push_back(Totals{p.name, 0, 0.0});
        t = &g_totals.back();
      }
      t->launches += 1;
      t->ms += ms;
    }
    cudaEventDestroy(p.start);
    cudaEventDestroy(p.stop);
  }
  g_pending.clear();
}
}  // namespace

LaunchScope::LaunchScope(const char* name, cudaStream_t stream) : name_(name), stream_(stream) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  if (g_timing.load(std::memory_order_relaxed) &&
      cudaEventCreateWithFlags(&start_, cudaEventDefault) == cudaSuccess) {
    if (cudaEventRecord(start_, stream_) != cudaSuccess) {
      cudaEventDestroy(start_);
      start_ = nullptr;
    }
  }
}

LaunchScope::~LaunchScope() {
  if (start_ == nullptr) return;
  cudaEvent_t stop = nullptr;
  if (cudaEventCreateWithFlags(&stop, cudaEventDefault) != cudaSuccess || cudaEventRecord(stop, stream_) != cudaSuccess) {
    if (stop) cudaEventDestroy(stop);
    cudaEventDestroy(start_);
    return;
  }
  std::lock_guard<std::mutex> lock(g_timing_mutex);
  g_pending.push_back(Pending{name_, start_, stop});
  if (g_pending.size() > 4096) settle_locked();
}

ksj_gpu_status check_launch() {
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? KSJ_GPU_OK : KSJ_GPU_ERROR_CUDA;
}

namespace {

// ------------------------------------------------------------- direct NUDFT

constexpr int kDirectPixels = 128;  // threads (pixels) per block
constexpr int kDirectTile = 256;    // samples staged per iteration
constexpr int kDirectCoils = 8;     // accumulators per thread
constexpr uint32_t kDirectChannelLimit = 65535u * kDirectCoils;  // grid.y of the launch

// img[c][r][col] = sum_s y[c][s] exp(i (k_r,s (r - r0) + k_c,s (col - c0))),
// summed in sample order in float; the phase of every (pixel, sample) pair
// is formed exactly and reduced by 2 pi before sincosf (the reference rounds
// it to float first, eigen_nufft_direct_nudft.cpp:88-90).
__global__ void __launch_bounds__(kDirectPixels) k_direct_adjoint(const float2* __restrict__ kspace,
                                                                  const float2* __restrict__ traj, float2* out,
                                                                  int rows, int cols, float row_origin,
                                                                  float col_origin, int channels, int samples) {
  __shared__ float2 s_traj[kDirectTile];
  __shared__ float2 s_y[kDirectCoils][kDirectTile];
  const int p = blockIdx.x * kDirectPixels + threadIdx.x;
  const int c0 = blockIdx.y * kDirectCoils;
  const int nc = min(kDirectCoils, channels - c0);
  const bool live = p < rows * cols;
  const int r = live ? p / cols : 0;
  const int col = live ? p - r * cols : 0;
  const float xr = __fsub_rn(static_cast<float>(r), row_origin);
  const float xc = __fsub_rn(static_cast<float>(col), col_origin);
  float2 acc[kDirectCoils];
#pragma unroll
  for (int c = 0; c < kDirectCoils; ++c) acc[c] = make_float2(0.0f, 0.0f);
  for (int s0 = 0; s0 < samples; s0 += kDirectTile) {
    const int ns = min(kDirectTile, samples - s0);
    __syncthreads();
    for (int i = threadIdx.x; i < ns; i += kDirectPixels) s_traj[i] = traj[s0 + i];
    for (int i = threadIdx.x; i < ns * nc; i += kDirectPixels) {
      const int c = i / ns, s = i - c * ns;
      s_y[c][s] = kspace[static_cast<size_t>(c0 + c) * samples + s0 + s];
    }
    __syncthreads();
    for (int s = 0; s < ns; ++s) {
      const float2 k = s_traj[s];
      const float2 e = exp_i_dot(k.x, xr, k.y, xc, 1.0f);
#pragma unroll
      for (int c = 0; c < kDirectCoils; ++c) {
        if (c < nc) acc[c] = cadd(acc[c], cmul(s_y[c][s], e));
      }
    }
  }
  if (live) {
#pragma unroll
    for (int c = 0; c < kDirectCoils; ++c)
      if (c < nc) out[static_cast<size_t>(c0 + c) * rows * cols + p] = acc[c];
  }
}

// y[c][s] = sum_p x[p][c] exp(-i (k_r,s (r - r0) + k_c,s (col - c0))), p = r
// cols + col in pixel order, summed in float in that order as
// direct_forward_impl does (eigen_nufft_direct_nudft.cpp:51-74, the
// reference's nufft2_forward on its Eigen backend, nufft.cpp:29).  One thread
// per sample and a group of kDirectCoils coils per block row; each pixel
// tile's positions and coil values are staged in shared memory.  The phase of
// every (sample, pixel) pair is formed exactly and reduced by 2 pi before
// sincosf (the reference rounds it to float first).
constexpr int kForwardSamples = 128;  // threads (samples) per block
constexpr int kForwardTile = 256;     // pixels staged per iteration
__global__ void __launch_bounds__(kForwardSamples) k_direct_forward(const float2* __restrict__ image,
                                                                   const float2* __restrict__ traj, float2* out,
                                                                   int rows, int cols, float row_origin,
                                                                   float col_origin, int channels, int samples) {
  __shared__ float2 s_pos[kForwardTile];
  __shared__ float2 s_x[kDirectCoils][kForwardTile];
  const int s = blockIdx.x * kForwardSamples + threadIdx.x;
  const int c0 = blockIdx.y * kDirectCoils;
  const int nc = min(kDirectCoils, channels - c0);
  const bool live = s < samples;
  const float2 k = live ? traj[s] : make_float2(0.0f, 0.0f);
  const int pixels = rows * cols;
  float2 acc[kDirectCoils];
#pragma unroll
  for (int c = 0; c < kDirectCoils; ++c) acc[c] = make_float2(0.0f, 0.0f);
  for (int p0 = 0; p0 < pixels; p0 += kForwardTile) {
    const int np = min(kForwardTile, pixels - p0);
    __syncthreads();
    for (int i = threadIdx.x; i < np; i += kForwardSamples) {
      const int r = (p0 + i) / cols, col = p0 + i - ((p0 + i) / cols) * cols;
      s_pos[i] = make_float2(__fsub_rn(static_cast<float>(r), row_origin), __fsub_rn(static_cast<float>(col), col_origin));
    }
    for (int i = threadIdx.x; i < np * nc; i += kForwardSamples) {
      const int q = i / nc, c = i - q * nc;
      s_x[c][q] = image[static_cast<size_t>(p0 + q) * channels + c0 + c];
    }
    __syncthreads();
    for (int q = 0; q < np; ++q) {
      const float2 pos = s_pos[q];
      const float2 e = exp_i_dot(k.x, pos.x, k.y, pos.y, -1.0f);
#pragma unroll
      for (int c = 0; c < kDirectCoils; ++c) {
        if (c < nc) acc[c] = cadd(acc[c], cmul(s_x[c][q], e));
      }
    }
  }
  if (live) {
#pragma unroll
    for (int c = 0; c < kDirectCoils; ++c)
      if (c < nc) out[static_cast<size_t>(c0 + c) * samples + s] = acc[c];
  }
}

// ------------------------------------------------------------- ingress

// ISMRMRD trajectories [kx, ky] -> the reconstruction's [row = ky, column =
// kx] in radians per pixel (noncartesian_rss_hdf5.cpp:776-833): each raw
// coordinate is checked (finite, inside its unit's inclusive Nyquist
// interval) and scaled by its axis's float factor with one rounded multiply,
// as the reference does.  A failing sample raises KSJ_GPU_FLAG_BAD_TRAJECTORY
// in *flags (its output is still written).
__global__ void __launch_bounds__(256) k_normalize_trajectory(const float2* __restrict__ raw, float2* out, int m,
                                                              float row_limit, float col_limit, float row_scale,
                                                              float col_scale, uint32_t* flags) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= m) return;
  const float2 k = raw[s];  // (kx, ky)
  const bool ok = isfinite(k.x) && isfinite(k.y) && fabsf(k.x) <= col_limit && fabsf(k.y) <= row_limit;
  if (!ok) atomicOr(flags, KSJ_GPU_FLAG_BAD_TRAJECTORY);
  out[s] = make_float2(__fmul_rn(k.y, row_scale), __fmul_rn(k.x, col_scale));
}

// Per-acquisition channel-major blocks [acquisition][channel][n] ->
// [channel][acquisition * n] (noncartesian_rss_hdf5.cpp:1077-1083), 16-byte
// vectors where n allows.
__global__ void __launch_bounds__(256) k_aggregate_acquisitions(const float2* __restrict__ in, float2* out,
                                                                int acquisitions, int channels, int n) {
  const size_t total = static_cast<size_t>(acquisitions) * channels * n;
  for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const size_t a = i / (static_cast<size_t>(channels) * n);
    const size_t rem = i - a * channels * n;
    const size_t c = rem / n, j = rem - c * n;
    out[(c * acquisitions + a) * n + j] = in[i];
  }
}

// --------------------------------------------------------------------- RSS

// out[p] = sqrt(sum_c re^2 + im^2), a float sum in channel order with every
// product and sum rounded separately: the order and rounding points of
// squared_norm_across + sqrt (reductions.hpp:972-982), so equal inputs give
// bit-identical outputs.  A warp takes 32 consecutive pixels and stages up to
// 32 of their coils at a time in shared memory with coalesced loads (lanes
// read consecutive coils of one pixel); then lane p adds its pixel's staged
// coils in order.
constexpr int kRssWarps = 8;
__global__ void __launch_bounds__(32 * kRssWarps) k_rss(const float2* __restrict__ in, float* out, uint64_t pixels,
                                                        int channels) {
  __shared__ float2 tile[kRssWarps][32][33];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t p0 = (static_cast<uint64_t>(blockIdx.x) * kRssWarps + warp) * 32;
  if (p0 >= pixels) return;
  const int np = pixels - p0 < 32 ? static_cast<int>(pixels - p0) : 32;
  float total = 0.0f;
  for (int c0 = 0; c0 < channels; c0 += 32) {
    const int cw = min(32, channels - c0);
    for (int i = lane; i < np * cw; i += 32) {
      const int q = i / cw, c = i - q * cw;
      tile[warp][q][c] = __ldg(in + (p0 + q) * channels + c0 + c);
    }
    __syncwarp();
    if (lane < np) {
      for (int c = 0; c < cw; ++c) {
        const float2 x = tile[warp][lane][c];
        total = __fadd_rn(total, __fadd_rn(__fmul_rn(x.x, x.x), __fmul_rn(x.y, x.y)));
      }
    }
    __syncwarp();
  }
  if (lane < np) out[p0 + lane] = __fsqrt_rn(total);
}

}  // namespace
}  // namespace ksj_gpu

using namespace ksj_gpu;

extern "C" size_t ksj_gpu_direct_workspace_bytes(uint32_t rows, uint32_t cols, uint32_t channels) {
  return align_up(static_cast<size_t>(rows) * cols * channels * sizeof(float2), 256);
}

extern "C" ksj_gpu_status ksj_gpu_direct_adjoint(uint32_t rows, uint32_t cols, double row_origin, double col_origin,
                                                 uint32_t channels, uint32_t samples, const void* d_kspace,
                                                 const float* d_traj, void* d_out, void* d_workspace,
                                                 size_t workspace_bytes, void* stream) {
  if (rows == 0 || cols == 0 || channels == 0 || samples == 0 || d_kspace == nullptr || d_traj == nullptr ||
      d_out == nullptr)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (rows > 8192 || cols > 8192 || static_cast<uint64_t>(rows) * cols > (1u << 26))
    return KSJ_GPU_ERROR_UNSUPPORTED;
  if (channels > kDirectChannelLimit) return KSJ_GPU_ERROR_UNSUPPORTED;  // launch grid y = ceil(C / 8) <= 65535
  const float ro = static_cast<float>(row_origin), co = static_cast<float>(col_origin);
  if (static_cast<double>(ro) != row_origin || static_cast<double>(co) != col_origin)
    return KSJ_GPU_ERROR_UNSUPPORTED;
  if (d_workspace == nullptr || workspace_bytes < ksj_gpu_direct_workspace_bytes(rows, cols, channels) ||
      (reinterpret_cast<uintptr_t>(d_workspace) & 255u) != 0)
    return KSJ_GPU_ERROR_WORKSPACE;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  float2* tmp = static_cast<float2*>(d_workspace);
  const int pixels = static_cast<int>(rows * cols);
  const dim3 grid((pixels + kDirectPixels - 1) / kDirectPixels, (channels + kDirectCoils - 1) / kDirectCoils);
  {
  LaunchScope scope("k_direct_adjoint", cs);
  k_direct_adjoint<<<grid, kDirectPixels, 0, cs>>>(static_cast<const float2*>(d_kspace),
                                                   reinterpret_cast<const float2*>(d_traj), tmp,
                                                   static_cast<int>(rows), static_cast<int>(cols), ro, co,
                                                   static_cast<int>(channels), static_cast<int>(samples));
  }
  const dim3 tg((pixels + 31) / 32, (channels + 31) / 32, 1);
  LaunchScope scope("k_images_coil_last", cs);
  k_transpose<unsigned long long><<<tg, dim3(32, 8), 0, cs>>>(reinterpret_cast<const unsigned long long*>(tmp),
                                                              static_cast<unsigned long long*>(d_out),
                                                              static_cast<int>(channels), pixels);
  return check_launch();
}

extern "C" ksj_gpu_status ksj_gpu_direct_forward(uint32_t rows, uint32_t cols, double row_origin, double col_origin,
                                                 uint32_t channels, uint32_t samples, const void* d_image,
                                                 const float* d_traj, void* d_out, void* stream) {
  if (rows == 0 || cols == 0 || channels == 0 || samples == 0 || d_image == nullptr || d_traj == nullptr ||
      d_out == nullptr)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (rows > 8192 || cols > 8192 || static_cast<uint64_t>(rows) * cols > (1u << 26) || samples > (1u << 30))
    return KSJ_GPU_ERROR_UNSUPPORTED;
  const float ro = static_cast<float>(row_origin), co = static_cast<float>(col_origin);
  if (static_cast<double>(ro) != row_origin || static_cast<double>(co) != col_origin)
    return KSJ_GPU_ERROR_UNSUPPORTED;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  const dim3 grid((samples + kForwardSamples - 1) / kForwardSamples, (channels + kDirectCoils - 1) / kDirectCoils);
  LaunchScope scope("k_direct_forward", cs);
  k_direct_forward<<<grid, kForwardSamples, 0, cs>>>(static_cast<const float2*>(d_image),
                                                     reinterpret_cast<const float2*>(d_traj),
                                                     static_cast<float2*>(d_out), static_cast<int>(rows),
                                                     static_cast<int>(cols), ro, co, static_cast<int>(channels),
                                                     static_cast<int>(samples));
  return check_launch();
}

extern "C" ksj_gpu_status ksj_gpu_normalize_trajectory(uint32_t samples, uint32_t units, uint32_t encoded_rows,
                                                       uint32_t encoded_cols, const float* d_raw, float* d_out,
                                                       uint32_t* d_flags, void* stream) {
  if (samples == 0 || d_raw == nullptr || d_out == nullptr || d_flags == nullptr) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  constexpr float kPi = 3.14159265358979323846f;
  const float two_pi = 2.0f * kPi;  // the reference's 2.0F * pi_v<float>, rounded once
  float row_limit, col_limit, row_scale, col_scale;
  switch (units) {
    case KSJ_GPU_TRAJ_CYCLES_PER_FOV:
      row_limit = col_limit = 0.5f;
      row_scale = col_scale = two_pi;
      break;
    case KSJ_GPU_TRAJ_RADIANS_PER_PIXEL:
      row_limit = col_limit = kPi;
      row_scale = col_scale = 1.0f;
      break;
    case KSJ_GPU_TRAJ_ENCODED_MATRIX_INDEX:
      if (encoded_rows < 2 || encoded_cols < 2) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
      row_limit = static_cast<float>(encoded_rows) / 2.0f;
      col_limit = static_cast<float>(encoded_cols) / 2.0f;
      row_scale = two_pi / static_cast<float>(encoded_rows);
      col_scale = two_pi / static_cast<float>(encoded_cols);
      break;
    default:
      return KSJ_GPU_ERROR_INVALID_ARGUMENT;  // unspecified or unknown units
  }
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  LaunchScope scope("k_normalize_trajectory", cs);
  k_normalize_trajectory<<<(samples + 255) / 256, 256, 0, cs>>>(reinterpret_cast<const float2*>(d_raw),
                                                                 reinterpret_cast<float2*>(d_out),
                                                                 static_cast<int>(samples), row_limit, col_limit,
                                                                 row_scale, col_scale, d_flags);
  return check_launch();
}

extern "C" ksj_gpu_status ksj_gpu_aggregate_acquisitions(uint32_t acquisitions, uint32_t channels,
                                                         uint32_t samples_per_acquisition, const void* d_in,
                                                         void* d_out, void* stream) {
  if (acquisitions == 0 || channels == 0 || samples_per_acquisition == 0 || d_in == nullptr || d_out == nullptr)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  const size_t total = static_cast<size_t>(acquisitions) * channels * samples_per_acquisition;
  if (total > (static_cast<size_t>(1) << 34)) return KSJ_GPU_ERROR_UNSUPPORTED;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  const unsigned blocks = static_cast<unsigned>(std::min<size_t>((total + 255) / 256, 152 * 16));
  LaunchScope scope("k_aggregate_acquisitions", cs);
  k_aggregate_acquisitions<<<blocks, 256, 0, cs>>>(static_cast<const float2*>(d_in), static_cast<float2*>(d_out),
                                                   static_cast<int>(acquisitions), static_cast<int>(channels),
                                                   static_cast<int>(samples_per_acquisition));
  return check_launch();
}

extern "C" ksj_gpu_status ksj_gpu_rss_coil_last(uint64_t pixels, uint32_t channels, const void* d_coil_last,
                                                float* d_out, void* stream) {
  if (pixels == 0 || channels == 0 || d_coil_last == nullptr || d_out == nullptr)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  LaunchScope scope("k_rss", cs);
  const uint64_t per_block = 32 * kRssWarps;
  k_rss<<<static_cast<unsigned>((pixels + per_block - 1) / per_block), 32 * kRssWarps, 0, cs>>>(
      static_cast<const float2*>(d_coil_last), d_out, pixels, static_cast<int>(channels));
  return check_launch();
}

// ------------------------------------------------------------------ context

namespace {
// Host-side allocation fault injection (tests): the next N device
// allocations of ksj_gpu_context_buffer report out-of-memory without calling
// cudaMalloc.
std::atomic<uint32_t> g_injected_allocation_failures{0};

bool take_injected_allocation_failure() {
  uint32_t n = g_injected_allocation_failures.load();
  while (n > 0) {
    if (g_injected_allocation_failures.compare_exchange_weak(n, n - 1)) return true;
  }
  return false;
}
}  // namespace

extern "C" void ksj_gpu_inject_allocation_failures(uint32_t count) { g_injected_allocation_failures.store(count); }

struct ksj_gpu_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  void* buffers[8] = {};
  size_t buffer_bytes[8] = {};
  void* pinned[4] = {};
  size_t pinned_bytes[4] = {};
};

extern "C" ksj_gpu_status ksj_gpu_context_create(int device, ksj_gpu_context** out_context) {
  if (out_context == nullptr) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  *out_context = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return KSJ_GPU_ERROR_CUDA;
  if (cudaSetDevice(device) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  auto* ctx = new (std::nothrow) ksj_gpu_context{};
  if (ctx == nullptr) return KSJ_GPU_ERROR_OUT_OF_MEMORY;
  ctx->device = device;
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return KSJ_GPU_ERROR_CUDA;
  }
  *out_context = ctx;
  return KSJ_GPU_OK;
}

extern "C" void ksj_gpu_context_destroy(ksj_gpu_context* ctx) {
  if (ctx == nullptr) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (void* b : ctx->buffers)
    if (b) cudaFree(b);
  for (void* b : ctx->pinned)
    if (b) cudaFreeHost(b);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

extern "C" void* ksj_gpu_context_stream(ksj_gpu_context* ctx) { return ctx ? ctx->stream : nullptr; }

extern "C" ksj_gpu_status ksj_gpu_context_buffer(ksj_gpu_context* ctx, uint32_t slot, size_t bytes,
                                                 void** out_pointer) {
  if (ctx == nullptr || slot >= 8 || out_pointer == nullptr) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (bytes == 0) bytes = 256;
  if (ctx->buffer_bytes[slot] < bytes) {
    if (cudaSetDevice(ctx->device) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
    if (ctx->buffers[slot]) {
      cudaStreamSynchronize(ctx->stream);
      cudaFree(ctx->buffers[slot]);
      ctx->buffers[slot] = nullptr;
      ctx->buffer_bytes[slot] = 0;
    }
    void* p = nullptr;
    if (take_injected_allocation_failure()) return KSJ_GPU_ERROR_OUT_OF_MEMORY;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      return KSJ_GPU_ERROR_OUT_OF_MEMORY;
    }
    ctx->buffers[slot] = p;
    ctx->buffer_bytes[slot] = bytes;
  }
  *out_pointer = ctx->buffers[slot];
  return KSJ_GPU_OK;
}

extern "C" ksj_gpu_status ksj_gpu_context_pinned(ksj_gpu_context* ctx, uint32_t slot, size_t bytes,
                                                 void** out_pointer) {
  if (ctx == nullptr || slot >= 4 || out_pointer == nullptr) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (bytes == 0) bytes = 256;
  if (ctx->pinned_bytes[slot] < bytes) {
    if (ctx->pinned[slot]) {
      cudaStreamSynchronize(ctx->stream);
      cudaFreeHost(ctx->pinned[slot]);
      ctx->pinned[slot] = nullptr;
      ctx->pinned_bytes[slot] = 0;
    }
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      return KSJ_GPU_ERROR_OUT_OF_MEMORY;
    }
    ctx->pinned[slot] = p;
    ctx->pinned_bytes[slot] = bytes;
  }
  *out_pointer = ctx->pinned[slot];
  return KSJ_GPU_OK;
}

extern "C" ksj_gpu_status ksj_gpu_context_copy(ksj_gpu_context* ctx, void* dst, const void* src, size_t bytes,
                                               int kind) {
  if (ctx == nullptr || (bytes && (dst == nullptr || src == nullptr))) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (bytes == 0) return KSJ_GPU_OK;
  const cudaMemcpyKind k = kind == 0 ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
  return cudaMemcpyAsync(dst, src, bytes, k, ctx->stream) == cudaSuccess ? KSJ_GPU_OK : KSJ_GPU_ERROR_CUDA;
}

extern "C" ksj_gpu_status ksj_gpu_context_sync(ksj_gpu_context* ctx) {
  if (ctx == nullptr) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  return cudaStreamSynchronize(ctx->stream) == cudaSuccess ? KSJ_GPU_OK : KSJ_GPU_ERROR_CUDA;
}

extern "C" uint64_t ksj_gpu_context_device_bytes(const ksj_gpu_context* ctx) {
  if (ctx == nullptr) return 0;
  uint64_t total = 0;
  for (size_t b : ctx->buffer_bytes) total += b;
  return total;
}

extern "C" const char* ksj_gpu_status_string(ksj_gpu_status status) {
  switch (status) {
    case KSJ_GPU_OK: return "ok";
    case KSJ_GPU_ERROR_INVALID_ARGUMENT: return "invalid argument";
    case KSJ_GPU_ERROR_UNSUPPORTED: return "unsupported configuration";
    case KSJ_GPU_ERROR_CUDA: return "CUDA runtime error";
    case KSJ_GPU_ERROR_WORKSPACE: return "workspace null, misaligned or too small";
    case KSJ_GPU_ERROR_OUT_OF_MEMORY: return "out of memory";
    case KSJ_GPU_ERROR_NONFINITE_INPUT: return "non-finite or out-of-range input rejected on the device";
    default: return "unknown status";
  }
}

extern "C" uint64_t ksj_gpu_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

extern "C" void ksj_gpu_timing_enable(int enable) { g_timing.store(enable ? 1 : 0); }

extern "C" void ksj_gpu_timing_reset(void) {
  std::lock_guard<std::mutex> lock(g_timing_mutex);
  settle_locked();
  g_totals.clear();
}

extern "C" uint32_t ksj_gpu_timing_read(uint32_t max_entries, char* names, uint64_t* launches, double* total_ms) {
  std::lock_guard<std::mutex> lock(g_timing_mutex);
  settle_locked();
  for (uint32_t i = 0; i < max_entries && i < g_totals.size(); ++i) {
    if (names) {
      std::strncpy(names + 48 * i, g_totals[i].name.c_str(), 47);
      names[48 * i + 47] = 0;
    }
    if (launches) launches[i] = g_totals[i].launches;
    if (total_ms) total_ms[i] = g_totals[i].ms;
  }
  return static_cast<uint32_t>(g_totals.size());
}

// --------------------------------------- direct NUDFT, static device scratch
//
// ksj_gpu_direct_adjoint_static runs the kernels of ksj_gpu_direct_adjoint
// with the coil-major intermediate in a file-scope device array instead of a
// caller workspace, so the call itself allocates nothing.  The array's address
// is looked up once per device context (with that device current) and kept
// with the context it belongs to: after a cudaDeviceReset, or a primary
// context released and created again, the module is loaded anew and the
// array may move, so a changed current context looks the address up again.

namespace ksj_gpu {
namespace {
constexpr size_t kDirectStaticScratchBytes = size_t(8) << 20;  // rows x cols x channels x 8 B at most
__device__ __align__(256) unsigned char g_direct_scratch[kDirectStaticScratchBytes];
constexpr int kStaticScratchDevices = 64;
struct StaticScratch {
  void* context = nullptr;  // the CUcontext the address was taken in
  void* address = nullptr;
};
std::mutex g_direct_scratch_mutex;
StaticScratch g_direct_scratch_at[kStaticScratchDevices];

using CtxGetCurrentFn = int (*)(void**);  // cuCtxGetCurrent(CUcontext*)

CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<CtxGetCurrentFn>(p);
  }();
  return fn;
}

// The direct adjoint's launch grid has ceil(channels / kDirectCoils) blocks
// along y, at most 65 535.
constexpr uint32_t kDirectMaxChannels = kDirectChannelLimit;
}  // namespace
}  // namespace ksj_gpu

extern "C" size_t ksj_gpu_direct_static_scratch_bytes(void) { return kDirectStaticScratchBytes; }

extern "C" ksj_gpu_status ksj_gpu_direct_adjoint_static(uint32_t rows, uint32_t cols, double row_origin,
                                                        double col_origin, uint32_t channels, uint32_t samples,
                                                        const void* d_kspace, const float* d_traj, void* d_out,
                                                        void* stream) {
  if (rows == 0 || cols == 0 || channels == 0 || samples == 0 || d_kspace == nullptr || d_traj == nullptr ||
      d_out == nullptr)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (rows > 8192 || cols > 8192 || static_cast<uint64_t>(rows) * cols > (1u << 26))
    return KSJ_GPU_ERROR_UNSUPPORTED;
  const float ro = static_cast<float>(row_origin), co = static_cast<float>(col_origin);
  if (static_cast<double>(ro) != row_origin || static_cast<double>(co) != col_origin)
    return KSJ_GPU_ERROR_UNSUPPORTED;
  // the intermediate must fit the static array: rejected before any device work
  if (static_cast<uint64_t>(rows) * cols * channels * sizeof(float2) > kDirectStaticScratchBytes)
    return KSJ_GPU_ERROR_WORKSPACE;
  if (channels > kDirectMaxChannels) return KSJ_GPU_ERROR_UNSUPPORTED;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  if (device < 0 || device >= kStaticScratchDevices) return KSJ_GPU_ERROR_UNSUPPORTED;
  const CtxGetCurrentFn get_ctx = ctx_get_current();
  if (get_ctx == nullptr) return KSJ_GPU_ERROR_CUDA;
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_direct_scratch_mutex);
    StaticScratch& at = g_direct_scratch_at[device];
    void* ctx = nullptr;
    // with no context current yet, the symbol lookup creates the primary one
    if (get_ctx(&ctx) != 0) return KSJ_GPU_ERROR_CUDA;
    if (at.address == nullptr || ctx == nullptr || ctx != at.context) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_direct_scratch) != cudaSuccess || p == nullptr) {
        cudaGetLastError();
        return KSJ_GPU_ERROR_CUDA;
      }
      if (get_ctx(&ctx) != 0 || ctx == nullptr) return KSJ_GPU_ERROR_CUDA;
      at.context = ctx;
      at.address = p;
    }
    scratch = at.address;
  }
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  float2* tmp = static_cast<float2*>(scratch);
  const int pixels = static_cast<int>(rows * cols);
  const dim3 grid((pixels + kDirectPixels - 1) / kDirectPixels, (channels + kDirectCoils - 1) / kDirectCoils);
  {
    LaunchScope scope("k_direct_adjoint", cs);
    k_direct_adjoint<<<grid, kDirectPixels, 0, cs>>>(static_cast<const float2*>(d_kspace),
                                                     reinterpret_cast<const float2*>(d_traj), tmp,
                                                     static_cast<int>(rows), static_cast<int>(cols), ro, co,
                                                     static_cast<int>(channels), static_cast<int>(samples));
  }
  const dim3 tg((pixels + 31) / 32, (channels + 31) / 32, 1);
  LaunchScope scope("k_images_coil_last", cs);
  k_transpose<unsigned long long><<<tg, dim3(32, 8), 0, cs>>>(reinterpret_cast<const unsigned long long*>(tmp),
                                                              static_cast<unsigned long long*>(d_out),
                                                              static_cast<int>(channels), pixels);
  return check_launch();
}
