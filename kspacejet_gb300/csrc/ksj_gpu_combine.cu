// ksj_gpu_combine.cu -- adaptive coil combination (Walsh) on coil-last images.
//
//   k_walsh<C>  one thread per pixel over a 16 x 16 tile whose coil values,
//               with a halo of half the window, sit in shared memory: the
//               window's coil covariance R = sum_q x(q) x(q)^H (Hermitian,
//               upper triangle in registers), its dominant eigenvector by
//               power iteration started from the pixel's own coil vector,
//               phase-referenced to coil 0, and the combination v^H x(p).
//
// Walsh, Gmitro and Marcellin, MRM 43:682-690, 2000 (noise covariance taken as
// the identity).  The window is clipped at the image border (samples outside
// the image contribute nothing).  No counterpart in the reference, whose
// adaptive combine is a planned interface only.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <vector>

#include "ksj_gpu.h"
#include "ksj_gpu_internal.cuh"

namespace ksj_gpu {
namespace {

constexpr int kWalshTile = 16;
constexpr int kWalshMaxHalf = 4;  // windows 1, 3, ..., 9

template <int C>
__global__ void __launch_bounds__(kWalshTile * kWalshTile) k_walsh(const float2* __restrict__ in, float2* out,
                                                                    int rows, int cols, int half, int iterations) {
  extern __shared__ float2 walsh_tile[];
  const int span = kWalshTile + 2 * half;
  const int r0 = blockIdx.y * kWalshTile - half;
  const int c0 = blockIdx.x * kWalshTile - half;
  const int tid = threadIdx.x;
  for (int i = tid; i < span * span * C; i += blockDim.x) {
    const int pix = i / C;
    const int c = i - pix * C;
    const int r = r0 + pix / span;
    const int cc = c0 + pix % span;
    walsh_tile[i] = (r >= 0 && r < rows && cc >= 0 && cc < cols)
                        ? in[(static_cast<size_t>(r) * cols + cc) * C + c]
                        : make_float2(0.0f, 0.0f);
  }
  __syncthreads();
  const int ty = tid / kWalshTile, tx = tid - ty * kWalshTile;
  const int r = blockIdx.y * kWalshTile + ty;
  const int cc = blockIdx.x * kWalshTile + tx;
  if (r >= rows || cc >= cols) return;

  // R[i][j], i <= j, packed row by row
  float2 R[C * (C + 1) / 2];
#pragma unroll
  for (int k = 0; k < C * (C + 1) / 2; ++k) R[k] = make_float2(0.0f, 0.0f);
  for (int dy = -half; dy <= half; ++dy) {
    for (int dx = -half; dx <= half; ++dx) {
      const float2* x = walsh_tile + ((ty + half + dy) * span + tx + half + dx) * C;
      float2 xv[C];
#pragma unroll
      for (int c = 0; c < C; ++c) xv[c] = x[c];
      int k = 0;
#pragma unroll
      for (int i = 0; i < C; ++i) {
#pragma unroll
        for (int j = i; j < C; ++j, ++k) {
          // x_i conj(x_j)
          R[k].x = fmaf(xv[i].x, xv[j].x, fmaf(xv[i].y, xv[j].y, R[k].x));
          R[k].y = fmaf(xv[i].y, xv[j].x, fmaf(-xv[i].x, xv[j].y, R[k].y));
        }
      }
    }
  }
  const float2* own = walsh_tile + ((ty + half) * span + tx + half) * C;
  float2 v[C];
  float norm = 0.0f;
#pragma unroll
  for (int c = 0; c < C; ++c) {
    v[c] = own[c];
    norm = fmaf(v[c].x, v[c].x, fmaf(v[c].y, v[c].y, norm));
  }
  if (!(norm > 0.0f)) {
#pragma unroll
    for (int c = 0; c < C; ++c) v[c] = make_float2(c == 0 ? 1.0f : 0.0f, 0.0f);
    norm = 1.0f;
  }
  for (int it = 0; it < iterations; ++it) {
    float2 u[C];
#pragma unroll
    for (int i = 0; i < C; ++i) u[i] = make_float2(0.0f, 0.0f);
    int k = 0;
#pragma unroll
    for (int i = 0; i < C; ++i) {
#pragma unroll
      for (int j = i; j < C; ++j, ++k) {
        u[i] = cadd(u[i], cmul(R[k], v[j]));  // R_ij v_j
        if (j != i) u[j] = cadd(u[j], cmul(make_float2(R[k].x, -R[k].y), v[i]));  // conj(R_ij) v_i
      }
    }
    float n2 = 0.0f;
#pragma unroll
    for (int i = 0; i < C; ++i) n2 = fmaf(u[i].x, u[i].x, fmaf(u[i].y, u[i].y, n2));
    if (!(n2 > 0.0f)) break;
    const float inv = rsqrtf(n2);
#pragma unroll
    for (int i = 0; i < C; ++i) v[i] = cscale(u[i], inv);
  }
  // phase reference: coil 0's weight real and non-negative
  const float m0 = sqrtf(v[0].x * v[0].x + v[0].y * v[0].y);
  float2 ph = m0 > 0.0f ? make_float2(v[0].x / m0, -v[0].y / m0) : make_float2(1.0f, 0.0f);
  float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const float2 w = cmul(v[c], ph);
    // conj(w) x
    acc.x = fmaf(w.x, own[c].x, fmaf(w.y, own[c].y, acc.x));
    acc.y = fmaf(w.x, own[c].y, fmaf(-w.y, own[c].x, acc.y));
  }
  out[static_cast<size_t>(r) * cols + cc] = acc;
}

template <int C>
ksj_gpu_status launch_walsh(uint32_t rows, uint32_t cols, int half, uint32_t iterations, const void* in, void* out,
                            cudaStream_t stream) {
  const int span = kWalshTile + 2 * half;
  const size_t smem = static_cast<size_t>(span) * span * C * sizeof(float2);
  if (cudaFuncSetAttribute(k_walsh<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) !=
      cudaSuccess)
    return KSJ_GPU_ERROR_CUDA;
  const dim3 grid((cols + kWalshTile - 1) / kWalshTile, (rows + kWalshTile - 1) / kWalshTile);
  LaunchScope scope("k_walsh", stream);
  k_walsh<C><<<grid, kWalshTile * kWalshTile, smem, stream>>>(static_cast<const float2*>(in),
                                                              static_cast<float2*>(out), static_cast<int>(rows),
                                                              static_cast<int>(cols), half,
                                                              static_cast<int>(iterations));
  return check_launch();
}

}  // namespace
}  // namespace ksj_gpu

using namespace ksj_gpu;

extern "C" ksj_gpu_status ksj_gpu_walsh_combine(uint32_t rows, uint32_t cols, uint32_t channels, uint32_t window,
                                                uint32_t iterations, const void* d_coil_last, void* d_out,
                                                void* stream) {
  if (rows == 0 || cols == 0 || channels == 0 || d_coil_last == nullptr || d_out == nullptr)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if ((window & 1u) == 0 || window / 2 > static_cast<uint32_t>(kWalshMaxHalf) || iterations > 1000 ||
      rows > 65535u * kWalshTile || cols > 65535u * kWalshTile)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  const int half = static_cast<int>(window / 2);
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  switch (channels) {
    case 1: return launch_walsh<1>(rows, cols, half, iterations, d_coil_last, d_out, cs);
    case 2: return launch_walsh<2>(rows, cols, half, iterations, d_coil_last, d_out, cs);
    case 3: return launch_walsh<3>(rows, cols, half, iterations, d_coil_last, d_out, cs);
    case 4: return launch_walsh<4>(rows, cols, half, iterations, d_coil_last, d_out, cs);
    case 5: return launch_walsh<5>(rows, cols, half, iterations, d_coil_last, d_out, cs);
    case 6: return launch_walsh<6>(rows, cols, half, iterations, d_coil_last, d_out, cs);
    case 7: return launch_walsh<7>(rows, cols, half, iterations, d_coil_last, d_out, cs);
    case 8: return launch_walsh<8>(rows, cols, half, iterations, d_coil_last, d_out, cs);
    default: return KSJ_GPU_ERROR_UNSUPPORTED;
  }
}

// ------------------------------------------------- coil covariance (tcgen05)
//
// R = (1/M) X X^H for X complex64 [C][M] (channel-major k-space), C <= 32,
// the covariance of coil_compression_basis_estimate.cpp:207-227.  As a real
// contraction: with A = [Re X; Im X] (64 x M), G = A A^T holds every term
// (R.re = G[i][j] + G[32+i][32+j], R.im = G[32+i][j] - G[i][32+j]).  Each
// element of A is split as hi + lo (both bf16, hi = bf16(a), lo = bf16(a - hi))
// and G ~= hi hi^T + lo hi^T + (lo hi^T)^T, every product accumulated in FP32
// by the tensor cores:
//   k_cov_split   X -> the operand [hi(Re); hi(Im); lo(Re); lo(Im)] (128 rows of bf16, samples contiguous)
//   k_cov_mma     per block a range of 64-sample tiles: TMA (128-byte swizzle) into a 4-stage ring,
//                 one thread issues tcgen05.mma M=128 (the whole operand), N=64 (its hi rows, the same
//                 shared memory), K=16; the 128 x 64 FP32 accumulator lives in tensor memory and is
//                 read out once by the four warps
//   k_cov_sum / k_cov_form  sum the blocks' accumulators in block order and form R (deterministic)

namespace ksj_gpu {
namespace {

constexpr int kCovRows = 128;
constexpr int kCovKTile = 64;  // samples per stage: 128 bytes of bf16 per operand row
constexpr int kCovStages = 4;
constexpr uint32_t kCovStageBytes = kCovRows * kCovKTile * 2;
constexpr int kCovThreads = 128;
constexpr uint32_t kCovWaitLimit = 1u << 22;
constexpr int kCovMaxBlocks = 304;

// Four consecutive samples of one coil per thread: four 8-byte loads (a
// warp reads 1 KiB contiguous) and one 8-byte store per operand row.
constexpr int kSplitPerThread = 4;
static_assert(kCovKTile % kSplitPerThread == 0, "padded sample count is a multiple of the per-thread samples");

__global__ void __launch_bounds__(256) k_cov_split(const float2* __restrict__ x, uint16_t* a, int channels,
                                                   int samples, int kpad) {
  const size_t idx = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int quads = kpad / kSplitPerThread;
  if (idx >= static_cast<size_t>(32) * quads) return;
  const int c = static_cast<int>(idx / quads);
  const int s0 = static_cast<int>(idx - static_cast<size_t>(c) * quads) * kSplitPerThread;
  uint16_t h[2][kSplitPerThread], l[2][kSplitPerThread];
#pragma unroll
  for (int i = 0; i < kSplitPerThread; ++i) {
    const int sm = s0 + i;
    float2 v = make_float2(0.0f, 0.0f);
    if (c < channels && sm < samples) v = __ldg(x + static_cast<size_t>(c) * samples + sm);
    const __nv_bfloat16 hr = __float2bfloat16_rn(v.x);
    const __nv_bfloat16 hi = __float2bfloat16_rn(v.y);
    h[0][i] = __bfloat16_as_ushort(hr);
    h[1][i] = __bfloat16_as_ushort(hi);
    l[0][i] = __bfloat16_as_ushort(__float2bfloat16_rn(v.x - __bfloat162float(hr)));
    l[1][i] = __bfloat16_as_ushort(__float2bfloat16_rn(v.y - __bfloat162float(hi)));
  }
  auto pack = [](const uint16_t (&v)[kSplitPerThread]) {
    return make_uint2(static_cast<uint32_t>(v[0]) | (static_cast<uint32_t>(v[1]) << 16),
                      static_cast<uint32_t>(v[2]) | (static_cast<uint32_t>(v[3]) << 16));
  };
  const size_t k = static_cast<size_t>(kpad);
  *reinterpret_cast<uint2*>(a + static_cast<size_t>(c) * k + s0) = pack(h[0]);
  *reinterpret_cast<uint2*>(a + static_cast<size_t>(32 + c) * k + s0) = pack(h[1]);
  *reinterpret_cast<uint2*>(a + static_cast<size_t>(64 + c) * k + s0) = pack(l[0]);
  *reinterpret_cast<uint2*>(a + static_cast<size_t>(96 + c) * k + s0) = pack(l[1]);
}

// Shared-memory matrix descriptor of a K-major operand in the 128-byte swizzle
// layout (8-row x 128-byte atoms stacked 1024 bytes apart along M/N).
__device__ __forceinline__ uint64_t sw128_kmajor_desc(uint32_t saddr) {
  uint64_t d = static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);  // start address
  d |= static_cast<uint64_t>(1) << 16;                          // leading byte offset (unused here): 16 B
  d |= static_cast<uint64_t>(1024 >> 4) << 32;                  // stride byte offset: 8 rows x 128 B
  d |= static_cast<uint64_t>(1) << 46;                          // descriptor version
  d |= static_cast<uint64_t>(2) << 61;                          // 128-byte swizzle
  return d;
}

// Instruction descriptor, kind::f16: FP32 accumulator, bf16 A and B, both
// K-major, N = 64, M = 128.
constexpr uint32_t kCovIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void tma_load_2d(void* dst, const void* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct CovArgs {
  float* partials;  // [blocks][128][64]
  uint32_t* flags;
  int ktiles;
};

__global__ void __launch_bounds__(kCovThreads) k_cov_mma(const __grid_constant__ CUtensorMap amap, CovArgs a) {
  extern __shared__ __align__(16) unsigned char cov_smem[];
  // stage buffers on a 1024-byte boundary (128-byte swizzle atoms)
  unsigned char* base = cov_smem + ((1024u - (smem_addr(cov_smem) & 1023u)) & 1023u);
  __shared__ __align__(8) uint64_t full[kCovStages], empty[kCovStages], done;
  __shared__ uint32_t tmem_base;
  __shared__ int failed;
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int t0 = static_cast<int>(static_cast<long long>(a.ktiles) * blockIdx.x / gridDim.x);
  const int t1 = static_cast<int>(static_cast<long long>(a.ktiles) * (blockIdx.x + 1) / gridDim.x);
  const int n = t1 - t0;
  if (tid == 0) {
    for (int s = 0; s < kCovStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&done, 1);
    mbar_init_fence();
    failed = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(smem_addr(&tmem_base))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (tid == 0) {
    int issued = 0;  // tiles whose copy was started
    auto stage_ptr = [&](int s) { return base + static_cast<size_t>(s) * kCovStageBytes; };
    auto load = [&](int j) {
      const int s = j % kCovStages;
      mbar_arrive_expect_tx(&full[s], kCovStageBytes);
      tma_load_2d(stage_ptr(s), &amap, (t0 + j) * kCovKTile, 0, &full[s]);
      ++issued;
    };
    bool ok = true;
    for (int j = 0; j < kCovStages - 1 && j < n; ++j) load(j);
    for (int i = 0; i < n && ok; ++i) {
      const int j = i + kCovStages - 1;
      if (j < n) {
        // the slot's previous tile (j - stages) must have been consumed by its MMAs
        if (j >= kCovStages) ok = mbar_wait_bounded(&empty[j % kCovStages], ((j / kCovStages) - 1) & 1, kCovWaitLimit);
        if (!ok) break;
        load(j);
      }
      const int s = i % kCovStages;
      ok = mbar_wait_bounded(&full[s], (i / kCovStages) & 1, kCovWaitLimit);
      if (!ok) break;
      const uint32_t sa = smem_addr(stage_ptr(s));
#pragma unroll
      for (int k = 0; k < kCovKTile / 16; ++k) {
        const uint64_t d = sw128_kmajor_desc(sa + k * 32);
        umma_bf16(tmem, d, d, kCovIdesc, (i > 0 || k > 0) ? 1u : 0u);
      }
      umma_commit(&empty[s]);
    }
    // every MMA issued so far completes before `done` fires
    umma_commit(&done);
    const bool fin = mbar_wait_bounded(&done, 0, kCovWaitLimit);
    if (!ok || !fin) {
      failed = 1;
      atomicOr(a.flags, KSJ_GPU_FLAG_WAIT_TIMEOUT);
      // let every copy this block started land before its shared memory goes
      for (int j = 0; j < issued; ++j) mbar_wait_bounded(&full[j % kCovStages], (j / kCovStages) & 1, kCovWaitLimit);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!failed) {
    // accumulator row 32*warp + lane, 64 FP32 columns
    const int row = warp * 32 + (tid & 31);
    float* dst = a.partials + (static_cast<size_t>(blockIdx.x) * kCovRows + row) * 64;
#pragma unroll
    for (int c = 0; c < 64; c += 16) {
      float v[16];
      tmem_ld16(tmem + (static_cast<uint32_t>(warp * 32) << 16) + c, v);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (n == 0) {
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = 0.0f;
      }
#pragma unroll
      for (int i = 0; i < 16; i += 4) *reinterpret_cast<float4*>(dst + c + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem) : "memory");
}

// Sum of the blocks' accumulators, one thread per accumulator element (the
// blocks' copies of an element are 32 KiB apart: coalesced across threads),
// in block order.
__global__ void __launch_bounds__(256) k_cov_sum(const float* partials, int blocks, float* sum) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kCovRows * 64) return;
  float s = 0.0f;
#pragma unroll 8
  for (int b = 0; b < blocks; ++b) s += partials[static_cast<size_t>(b) * kCovRows * 64 + e];
  sum[e] = s;
}

// One thread per covariance element: G = hi hi^T + lo hi^T + (lo hi^T)^T from
// the summed accumulator, then R times 1/M (in float, as the reference scales
// its sums).  The lower triangle is computed and the upper mirrored
// (conjugate), as the reference stores it, so R is Hermitian bit for bit.
__global__ void __launch_bounds__(256) k_cov_form(const float* d, int channels, float inv_m, float2* cov) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= channels * channels) return;
  const int i = idx / channels, j = idx - (idx / channels) * channels;
  auto g = [&](int r, int c) { return d[r * 64 + c] + d[(64 + r) * 64 + c] + d[(64 + c) * 64 + r]; };
  const int r = i >= j ? i : j, c = i >= j ? j : i;
  const float re = g(r, c) + g(32 + r, 32 + c);
  const float im = r == c ? 0.0f : g(32 + r, c) - g(r, 32 + c);
  cov[idx] = make_float2(re * inv_m, (i >= j ? im : -im) * inv_m);
}

// Per-channel mean of channel-major X [channels][samples] (one block per
// channel, a fixed-order tree over the block: deterministic), as
// covariance_channel_major_with_workspace forms it (moments.hpp:117-123).
__global__ void __launch_bounds__(256) k_channel_means(const float2* __restrict__ x, int samples, float2* means) {
  __shared__ float2 part[256];
  const float2* row = x + static_cast<size_t>(blockIdx.x) * samples;
  float2 acc = make_float2(0.0f, 0.0f);
  for (int s = threadIdx.x; s < samples; s += blockDim.x) {
    const float2 v = __ldg(row + s);
    acc.x += v.x;
    acc.y += v.y;
  }
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int h = blockDim.x >> 1; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      part[threadIdx.x].x += part[threadIdx.x + h].x;
      part[threadIdx.x].y += part[threadIdx.x + h].y;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const float inv = 1.0f / static_cast<float>(samples);
    means[blockIdx.x] = make_float2(part[0].x * inv, part[0].y * inv);
  }
}

// The noise covariance of noise_model_estimate.cpp:161-162
// (covariance_channel_major_with_workspace, population normalisation,
// moments.hpp:99-140): C(r, c) = (1/M) sum_s conj(x_r - mu_r) (x_c - mu_c)
// = conj(R(r, c) - mu_r conj(mu_c)) with R = (1/M) X X^H as k_cov_form
// forms it.  The lower triangle is computed and the upper mirrored, so C is
// Hermitian bit for bit.
__global__ void __launch_bounds__(256) k_noise_form(const float* d, int channels, float inv_m,
                                                    const float2* __restrict__ means, float2* cov) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= channels * channels) return;
  const int i = idx / channels, j = idx - (idx / channels) * channels;
  auto g = [&](int r, int c) { return d[r * 64 + c] + d[(64 + r) * 64 + c] + d[(64 + c) * 64 + r]; };
  const int r = i >= j ? i : j, c = i >= j ? j : i;
  const float rre = (g(r, c) + g(32 + r, 32 + c)) * inv_m;
  const float rim = r == c ? 0.0f : (g(32 + r, c) - g(r, 32 + c)) * inv_m;
  const float2 mr = means[r], mc = means[c];
  // d = R(r, c) - mu_r conj(mu_c)
  const float dre = rre - (mr.x * mc.x + mr.y * mc.y);
  const float dim = r == c ? 0.0f : rim - (mr.y * mc.x - mr.x * mc.y);
  cov[idx] = make_float2(dre, i >= j ? -dim : dim);  // C(r, c) = conj(d); C(c, r) = d
}

using EncodeTiled2Fn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                    const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled2Fn cov_encode() {
  static EncodeTiled2Fn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<EncodeTiled2Fn>(p);
  }();
  return fn;
}

struct CovLayout {
  size_t flags, operand, partials, sum, means, total;
  int kpad, ktiles, blocks;
};

CovLayout cov_layout(uint32_t samples) {
  CovLayout l{};
  l.kpad = static_cast<int>((samples + kCovKTile - 1) / kCovKTile * kCovKTile);
  l.ktiles = l.kpad / kCovKTile;
  l.blocks = std::min(l.ktiles, kCovMaxBlocks);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off = align_up(off + bytes, 256);
    return at;
  };
  l.flags = take(16);
  l.operand = take(static_cast<size_t>(kCovRows) * l.kpad * 2);
  l.partials = take(static_cast<size_t>(l.blocks) * kCovRows * 64 * sizeof(float));
  l.sum = take(static_cast<size_t>(kCovRows) * 64 * sizeof(float));
  l.means = take(32 * sizeof(float2));
  l.total = off;
  return l;
}

}  // namespace
}  // namespace ksj_gpu

extern "C" size_t ksj_gpu_coil_covariance_workspace_bytes(uint32_t channels, uint32_t samples) {
  if (channels == 0 || channels > 32 || samples == 0 || samples > (1u << 28)) return 0;
  return ksj_gpu::cov_layout(samples).total;
}

namespace ksj_gpu {
namespace {

// X [channels][samples] -> the summed split-BF16 products (tensor cores), then
// either R = (1/M) X X^H (noise = false) or the mean-removed noise covariance
// in the reference's convention (noise = true) into d_cov.
ksj_gpu_status covariance_run(uint32_t channels, uint32_t samples, const void* d_kspace, void* d_cov,
                              void* d_workspace, size_t workspace_bytes, void* stream, bool noise) {
  if (channels == 0 || channels > 32 || samples == 0 || samples > (1u << 28) || d_kspace == nullptr ||
      d_cov == nullptr || (reinterpret_cast<uintptr_t>(d_kspace) & 7u) != 0 ||
      (reinterpret_cast<uintptr_t>(d_cov) & 7u) != 0)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  const CovLayout l = cov_layout(samples);
  if (d_workspace == nullptr || (reinterpret_cast<uintptr_t>(d_workspace) & 255u) != 0 || workspace_bytes < l.total)
    return KSJ_GPU_ERROR_WORKSPACE;
  EncodeTiled2Fn enc = cov_encode();
  if (enc == nullptr) return KSJ_GPU_ERROR_CUDA;
  unsigned char* ws = static_cast<unsigned char*>(d_workspace);
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  uint32_t* flags = reinterpret_cast<uint32_t*>(ws + l.flags);
  uint16_t* operand = reinterpret_cast<uint16_t*>(ws + l.operand);
  float* partials = reinterpret_cast<float*>(ws + l.partials);
  if (cudaMemsetAsync(flags, 0, 16, cs) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  {
    const size_t n = static_cast<size_t>(32) * (l.kpad / kSplitPerThread);
    LaunchScope scope("k_cov_split", cs);
    k_cov_split<<<static_cast<unsigned>((n + 255) / 256), 256, 0, cs>>>(static_cast<const float2*>(d_kspace),
                                                                        operand, static_cast<int>(channels),
                                                                        static_cast<int>(samples), l.kpad);
  }
  CUtensorMap map;
  const cuuint64_t dims[2] = {static_cast<cuuint64_t>(l.kpad), static_cast<cuuint64_t>(kCovRows)};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(l.kpad) * 2};
  const cuuint32_t box[2] = {static_cast<cuuint32_t>(kCovKTile), static_cast<cuuint32_t>(kCovRows)};
  const cuuint32_t estr[2] = {1, 1};
  if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, operand, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
          CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return KSJ_GPU_ERROR_CUDA;
  const size_t smem = 1024 + static_cast<size_t>(kCovStages) * kCovStageBytes;
  if (cudaFuncSetAttribute(k_cov_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) !=
      cudaSuccess)
    return KSJ_GPU_ERROR_CUDA;
  {
    CovArgs args{partials, flags, l.ktiles};
    LaunchScope scope("k_cov_mma", cs);
    k_cov_mma<<<l.blocks, kCovThreads, smem, cs>>>(map, args);
  }
  float* sum = reinterpret_cast<float*>(ws + l.sum);
  {
    LaunchScope scope("k_cov_sum", cs);
    k_cov_sum<<<kCovRows * 64 / 256, 256, 0, cs>>>(partials, l.blocks, sum);
  }
  const int n = static_cast<int>(channels * channels);
  const float inv_m = 1.0f / static_cast<float>(samples);
  if (noise) {
    float2* means = reinterpret_cast<float2*>(ws + l.means);
    {
      LaunchScope scope("k_channel_means", cs);
      k_channel_means<<<channels, 256, 0, cs>>>(static_cast<const float2*>(d_kspace), static_cast<int>(samples),
                                                means);
    }
    LaunchScope scope("k_noise_form", cs);
    k_noise_form<<<(n + 255) / 256, 256, 0, cs>>>(sum, static_cast<int>(channels), inv_m, means,
                                                  static_cast<float2*>(d_cov));
  } else {
    LaunchScope scope("k_cov_form", cs);
    k_cov_form<<<(n + 255) / 256, 256, 0, cs>>>(sum, static_cast<int>(channels), inv_m, static_cast<float2*>(d_cov));
  }
  return check_launch();
}

}  // namespace
}  // namespace ksj_gpu

extern "C" ksj_gpu_status ksj_gpu_coil_covariance(uint32_t channels, uint32_t samples, const void* d_kspace,
                                                  void* d_cov, void* d_workspace, size_t workspace_bytes,
                                                  void* stream) {
  return ksj_gpu::covariance_run(channels, samples, d_kspace, d_cov, d_workspace, workspace_bytes, stream, false);
}

extern "C" ksj_gpu_status ksj_gpu_noise_covariance(uint32_t channels, uint32_t samples, const void* d_noise,
                                                   void* d_cov, void* d_workspace, size_t workspace_bytes,
                                                   void* stream) {
  return ksj_gpu::covariance_run(channels, samples, d_noise, d_cov, d_workspace, workspace_bytes, stream, true);
}

// ------------------------------------------------- coil compression basis and apply

namespace ksj_gpu {
namespace {

// Y[v][s] = sum_c B[v][c] X[c][s] (noncartesian_coil_compress.cpp:143-148): one
// thread per sample, the kV outputs in registers, B in shared memory.
template <int kV>
__global__ void __launch_bounds__(256) k_coil_compress(const float2* __restrict__ basis, const float2* __restrict__ x,
                                                       float2* y, int channels, int samples) {
  __shared__ float2 b[kV * 32];
  for (int i = threadIdx.x; i < kV * channels; i += blockDim.x) b[i] = basis[i];
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= samples) return;
  float2 acc[kV];
#pragma unroll
  for (int v = 0; v < kV; ++v) acc[v] = make_float2(0.0f, 0.0f);
  for (int c = 0; c < channels; ++c) {
    const float2 xv = __ldg(x + static_cast<size_t>(c) * samples + s);
#pragma unroll
    for (int v = 0; v < kV; ++v) {
      const float2 w = b[v * channels + c];
      acc[v].x = fmaf(w.x, xv.x, fmaf(-w.y, xv.y, acc[v].x));
      acc[v].y = fmaf(w.x, xv.y, fmaf(w.y, xv.x, acc[v].y));
    }
  }
#pragma unroll
  for (int v = 0; v < kV; ++v) y[static_cast<size_t>(v) * samples + s] = acc[v];
}

template <int kV>
ksj_gpu_status launch_compress(uint32_t channels, uint32_t samples, const void* basis, const void* x, void* y,
                               cudaStream_t stream) {
  LaunchScope scope("k_coil_compress", stream);
  k_coil_compress<kV><<<(samples + 255) / 256, 256, 0, stream>>>(static_cast<const float2*>(basis),
                                                                 static_cast<const float2*>(x), static_cast<float2*>(y),
                                                                 static_cast<int>(channels),
                                                                 static_cast<int>(samples));
  return check_launch();
}

}  // namespace
}  // namespace ksj_gpu

// Cyclic Jacobi for a Hermitian matrix (host, double precision).  For each
// pair (p, q): a phase on index q makes a_pq real and positive, then a real
// plane rotation zeroes it (the symmetric Jacobi step).  `a` and `vec` are
// row-major n x n; on return the diagonal of `a` holds the eigenvalues and
// the columns of `vec` the eigenvectors.
static void hermitian_jacobi(int n, std::complex<double>* a, std::complex<double>* vec) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) vec[i * n + j] = i == j ? 1.0 : 0.0;
  double total = 0.0;
  for (int i = 0; i < n * n; ++i) total += std::norm(a[i]);
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += std::norm(a[p * n + q]);
    if (off <= 1e-32 * total) break;
    for (int p = 0; p < n; ++p) {
      for (int q = p + 1; q < n; ++q) {
        const double r = std::abs(a[p * n + q]);
        if (r <= 1e-300) continue;
        const std::complex<double> e = a[p * n + q] / r;
        for (int k = 0; k < n; ++k) {
          a[k * n + q] *= std::conj(e);
          vec[k * n + q] *= std::conj(e);
        }
        for (int k = 0; k < n; ++k) a[q * n + k] *= e;
        const double theta = (a[q * n + q].real() - a[p * n + p].real()) / (2.0 * r);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          const std::complex<double> kp = a[k * n + p], kq = a[k * n + q];
          a[k * n + p] = c * kp - s * kq;
          a[k * n + q] = s * kp + c * kq;
        }
        for (int k = 0; k < n; ++k) {
          const std::complex<double> pk = a[p * n + k], qk = a[q * n + k];
          a[p * n + k] = c * pk - s * qk;
          a[q * n + k] = s * pk + c * qk;
        }
        for (int k = 0; k < n; ++k) {
          const std::complex<double> vp = vec[k * n + p], vq = vec[k * n + q];
          vec[k * n + p] = c * vp - s * vq;
          vec[k * n + q] = s * vp + c * vq;
        }
      }
    }
  }
}

using namespace ksj_gpu;

extern "C" ksj_gpu_status ksj_coil_compression_basis(uint32_t channels, uint32_t virtual_channels,
                                                     const void* covariance, void* basis, float* eigenvalues) {
  if (channels == 0 || channels > 64 || virtual_channels == 0 || virtual_channels > channels ||
      covariance == nullptr || basis == nullptr)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  const int n = static_cast<int>(channels);
  const float* cov = static_cast<const float*>(covariance);
  std::vector<std::complex<double>> a(static_cast<size_t>(n) * n), vec(static_cast<size_t>(n) * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      // Hermitian part of the input (the lower triangle mirrored, as the reference stores it)
      const int lo = i >= j ? i * n + j : j * n + i;
      const std::complex<double> v(cov[2 * lo], cov[2 * lo + 1]);
      a[static_cast<size_t>(i) * n + j] = i >= j ? v : std::conj(v);
      if (!std::isfinite(v.real()) || !std::isfinite(v.imag())) return KSJ_GPU_ERROR_NONFINITE_INPUT;
    }
  hermitian_jacobi(n, a.data(), vec.data());
  std::vector<int> order(static_cast<size_t>(n));
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return a[static_cast<size_t>(x) * n + x].real() > a[static_cast<size_t>(y) * n + y].real();
  });
  float* out = static_cast<float*>(basis);
  for (uint32_t v = 0; v < virtual_channels; ++v) {
    const int col = order[v];
    for (int c = 0; c < n; ++c) {
      // basis row v = conj(eigenvector), largest eigenvalue first (coil_compression_basis_estimate.cpp:233-239)
      const std::complex<double> e = std::conj(vec[static_cast<size_t>(c) * n + col]);
      out[2 * (v * n + c)] = static_cast<float>(e.real());
      out[2 * (v * n + c) + 1] = static_cast<float>(e.imag());
    }
  }
  if (eigenvalues != nullptr)
    for (int i = 0; i < n; ++i) eigenvalues[i] = static_cast<float>(a[static_cast<size_t>(order[i]) * n + order[i]].real());
  return KSJ_GPU_OK;
}

extern "C" ksj_gpu_status ksj_gpu_coil_compress(uint32_t channels, uint32_t virtual_channels, uint32_t samples,
                                                const void* d_basis, const void* d_kspace, void* d_out,
                                                void* stream) {
  if (channels == 0 || channels > 32 || virtual_channels == 0 || virtual_channels > 16 ||
      virtual_channels > channels || samples == 0 || d_basis == nullptr || d_kspace == nullptr || d_out == nullptr)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  switch (virtual_channels) {
#define KSJ_COMPRESS_CASE(V) \
  case V: return launch_compress<V>(channels, samples, d_basis, d_kspace, d_out, cs);
    KSJ_COMPRESS_CASE(1) KSJ_COMPRESS_CASE(2) KSJ_COMPRESS_CASE(3) KSJ_COMPRESS_CASE(4)
    KSJ_COMPRESS_CASE(5) KSJ_COMPRESS_CASE(6) KSJ_COMPRESS_CASE(7) KSJ_COMPRESS_CASE(8)
    KSJ_COMPRESS_CASE(9) KSJ_COMPRESS_CASE(10) KSJ_COMPRESS_CASE(11) KSJ_COMPRESS_CASE(12)
    KSJ_COMPRESS_CASE(13) KSJ_COMPRESS_CASE(14) KSJ_COMPRESS_CASE(15) KSJ_COMPRESS_CASE(16)
#undef KSJ_COMPRESS_CASE
    default: return KSJ_GPU_ERROR_UNSUPPORTED;
  }
}

// Whitening matrix of a noise covariance (noise_model_estimate.cpp:163-167,
// whitening.hpp:27-51): W = V diag(1 / sqrt(max(lambda, floor))) V^H over the
// eigenpairs of the Hermitian covariance (double-precision cyclic Jacobi),
// W(r, c) = sum_k V(r, k) / sqrt(max(lambda_k, floor)) conj(V(c, k)).
extern "C" ksj_gpu_status ksj_whitening_matrix(uint32_t channels, const void* covariance, float eigenvalue_floor,
                                               void* whitening) {
  if (channels == 0 || channels > 64 || covariance == nullptr || whitening == nullptr || !(eigenvalue_floor > 0.0f))
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  const int n = static_cast<int>(channels);
  const float* cov = static_cast<const float*>(covariance);
  std::vector<std::complex<double>> a(static_cast<size_t>(n) * n), vec(static_cast<size_t>(n) * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      const int lo = i >= j ? i * n + j : j * n + i;
      const std::complex<double> v(cov[2 * lo], cov[2 * lo + 1]);
      if (!std::isfinite(v.real()) || !std::isfinite(v.imag())) return KSJ_GPU_ERROR_NONFINITE_INPUT;
      a[static_cast<size_t>(i) * n + j] = i >= j ? v : std::conj(v);
    }
  hermitian_jacobi(n, a.data(), vec.data());
  std::vector<double> scale(static_cast<size_t>(n));
  for (int k = 0; k < n; ++k)
    scale[k] = 1.0 / std::sqrt(std::max(a[static_cast<size_t>(k) * n + k].real(), static_cast<double>(eigenvalue_floor)));
  float* out = static_cast<float*>(whitening);
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) {
      std::complex<double> sum = 0.0;
      for (int k = 0; k < n; ++k)
        sum += vec[static_cast<size_t>(r) * n + k] * scale[k] * std::conj(vec[static_cast<size_t>(c) * n + k]);
      out[2 * (r * n + c)] = static_cast<float>(sum.real());
      out[2 * (r * n + c) + 1] = static_cast<float>(sum.imag());
    }
  return KSJ_GPU_OK;
}

// Y = W X (noncartesian_noise_prewhiten.cpp:140-146): the square form of the
// compression apply, W complex64 [channels][channels].
extern "C" ksj_gpu_status ksj_gpu_noise_prewhiten(uint32_t channels, uint32_t samples, const void* d_whitening,
                                                  const void* d_kspace, void* d_out, void* stream) {
  if (channels == 0 || channels > 32 || samples == 0 || d_whitening == nullptr || d_kspace == nullptr ||
      d_out == nullptr)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  switch (channels) {
#define KSJ_WHITEN_CASE(V) \
  case V: return launch_compress<V>(channels, samples, d_whitening, d_kspace, d_out, cs);
    KSJ_WHITEN_CASE(1) KSJ_WHITEN_CASE(2) KSJ_WHITEN_CASE(3) KSJ_WHITEN_CASE(4)
    KSJ_WHITEN_CASE(5) KSJ_WHITEN_CASE(6) KSJ_WHITEN_CASE(7) KSJ_WHITEN_CASE(8)
    KSJ_WHITEN_CASE(9) KSJ_WHITEN_CASE(10) KSJ_WHITEN_CASE(11) KSJ_WHITEN_CASE(12)
    KSJ_WHITEN_CASE(13) KSJ_WHITEN_CASE(14) KSJ_WHITEN_CASE(15) KSJ_WHITEN_CASE(16)
    KSJ_WHITEN_CASE(17) KSJ_WHITEN_CASE(18) KSJ_WHITEN_CASE(19) KSJ_WHITEN_CASE(20)
    KSJ_WHITEN_CASE(21) KSJ_WHITEN_CASE(22) KSJ_WHITEN_CASE(23) KSJ_WHITEN_CASE(24)
    KSJ_WHITEN_CASE(25) KSJ_WHITEN_CASE(26) KSJ_WHITEN_CASE(27) KSJ_WHITEN_CASE(28)
    KSJ_WHITEN_CASE(29) KSJ_WHITEN_CASE(30) KSJ_WHITEN_CASE(31) KSJ_WHITEN_CASE(32)
#undef KSJ_WHITEN_CASE
    default: return KSJ_GPU_ERROR_UNSUPPORTED;
  }
}
