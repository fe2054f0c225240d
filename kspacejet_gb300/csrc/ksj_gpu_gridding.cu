// ksj_gpu_gridding.cu -- adjoint gridding reconstruction on sm_103a.
//
// One call reconstructs `frames` independent frames of `channels` coils:
//
//   k_tables   quarter-turn-reduced FFT twiddles, FP64 Kaiser-Bessel
//              deapodisation factors (per call, tiny)
//   k_prepare  per (frame, sample): error-free grid coordinate, taps and
//              weights (linear or Kaiser-Bessel), accurately reduced origin
//              phase times the DCF, and a count per binning list
//   k_scan     per frame: exclusive scan of the list counts
//   k_scatter  per (frame, sample): append the sample to each list it touches
//   k_sort     per list (one warp): sort by sample index, so every cell later
//              accumulates in sample order -- the reference's order -- and the
//              result is deterministic whatever order the scatter produced
//   k_samples_coil_last  [frame][coil][sample] -> [frame][sample][coil], so a
//              warp reads one sample's coils as one coalesced segment
//   k_rows     per (frame, grid row, coil group): each warp owns one
//              32-column chunk of the row and its sorted list and accumulates
//              lane-per-coil into shared memory with no atomics (a cell is
//              only ever touched by its owning warp, in list order); the block
//              then runs the row inverse FFT of every coil line in place and
//              writes only the columns the image keeps, coil-last
//              ([frame][grid row][column][channel]), so the column pass
//              reads every coil of a column as one tile
//   k_cols     per (frame, column block): one TMA tile of all grid rows x
//              columns x a group of coils, column inverse FFT in place, crop,
//              deapodise, then write coil-last images or sum |x|^2 over coils
//              in channel order (the reference RSS order and rounding)
//   k_images_coil_major  coil-last -> coil-major transpose when asked for
//
// Binning lists are (frame, grid row, 32-column chunk); a sample is listed
// once per row its stencil covers and per chunk its W columns fall into
// (one or two).  The "reference permutation" a list must equal is the
// increasing sequence of sample indices whose stencil touches that row and
// chunk, with the lower tap index floor(k N / 2 pi) of the exact coordinate
// (the value the reference's double-precision grid_coordinate computes,
// eigen_radial_gridding.cpp:262-277).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <map>
#include <tuple>
#include <type_traits>
#include <vector>

#include "ksj_gpu.h"
#include "ksj_gpu_internal.cuh"

namespace ksj_gpu {
namespace {

constexpr int kChunk = 16;        // grid columns per binning list (<= 32 lists per row)
constexpr int kMaxWidth = 8;      // largest Kaiser-Bessel width
constexpr int kMaxGrid = 512;
constexpr int kMaxThreads = 512;
constexpr int kColsThreads = 256;  // k_cols block size
constexpr int kAhead = 8;         // coil loads in flight per warp in k_rows
constexpr int kAheadRegs = 2;     // the same for the register-cell form (its unrolled body grows with it: 2 measured best)
constexpr uint32_t kFlagBytes = 256;

// Per (frame, sample) record written by k_prepare, read by k_rows.
template <int W>
struct alignas(16) SampleRecord {
  int r0;        // first tap row (wrapped)
  int c0;        // first tap column (wrapped)
  float2 scale;  // dcf * exp(i * origin phase)
  float wr[W];
  float wc[W];
};

// Per sample record of the 3-D path: first tap plane/row/column (wrapped),
// dcf * phase, and the W tap weights along z, y and x.
template <int W>
struct alignas(16) SampleRecord3 {
  int z0, r0, c0, pad;
  float2 scale;
  float wz[W];
  float wr[W];
  float wc[W];
};

// k_rows stages, per warp, the list entries of its current batch in shared
// memory: {c0, sample, scale} and the W column weights times the row weight,
// in 16-byte vectors read back as warp-wide broadcasts.
__host__ __device__ constexpr int meta_vecs(int w) { return 1 + (w + 3) / 4; }
__host__ __device__ constexpr int meta_batch(int w) { return w <= 4 ? 32 : 16; }

// Shared memory of one k_rows block: accumulators, twiddles, the list
// offsets of the row and the per-warp entry batches.
inline size_t rows_smem_for(int grid_cols, int cg, int width, int threads) {
  const int nchunks = (grid_cols + kChunk - 1) / kChunk;
  const size_t head = static_cast<size_t>(grid_cols) * (cg + 1) * 8 + static_cast<size_t>(nchunks + 1) * 4;
  return ((head + 15) & ~size_t{15}) + static_cast<size_t>(threads / 32) * meta_batch(width) * meta_vecs(width) * 16;
}
inline int rows_threads_for(int grid_cols) { return std::max(64, (grid_cols + 31) / 32 * 32); }

constexpr uint32_t kWaitLimit = 1u << 22;  // polls before a bounded wait gives up

struct Shape {
  int frames, channels, samples;
  int rows, cols;          // image
  int grid_rows, grid_cols;
  int width;
  int nchunks;             // ceil(grid_cols / 32)
  int lists_per_frame;     // grid_rows * nchunks
  size_t entries_per_frame;
  int out_rows, out_cols;  // kept image region
  int col_group;           // coils per column-pass tile: a power of two >= 2, <= 32
  int cpitch;              // channel pitch of the row-transformed grid: channels rounded up to col_group
  bool kb;
  float beta, inv_i0_beta;
  float row_origin, col_origin;
  float phase_row, phase_col, phase_sign;  // origin-phase coefficients
  int coil_group, column_block, list_capacity, frames_per_pass, rows_blocks, coil_parts;
  uint32_t wait_fault;  // tests only: segment waits that cannot succeed, given up after this many polls
  int column_pass;      // 1 one CTA per tile (k_cols), 2 persistent ring (k_cols_ring)
  DifPlan plan_rows, plan_cols;
  // ragged batches (device arrays, null otherwise): valid coils and samples
  // of each frame, and the addresses of its samples [C_f][M_f] and of its
  // trajectory [M_f][2] (device memory or host memory the device reads)
  const uint32_t* frame_channels = nullptr;
  const uint32_t* frame_samples = nullptr;
  const uint64_t* frame_kspace = nullptr;
  const uint64_t* frame_traj = nullptr;
};

struct Layout {
  size_t flags, frame_flags, records, counts, cursor, offsets, entries, expanded, long_lists, samples_t, inter,
      coil_last, tables, total;
};

size_t record_bytes(int width) {
  switch (width) {
    case 2: return sizeof(SampleRecord<2>);
    case 4: return sizeof(SampleRecord<4>);
    case 6: return sizeof(SampleRecord<6>);
    default: return sizeof(SampleRecord<8>);
  }
}

bool is_fft_size(uint32_t n) {
  DifPlan p;
  return n >= 2 && n <= kMaxGrid && make_dif_plan(static_cast<int>(n), &p);
}

ksj_gpu_status make_shape(const ksj_gpu_gridding_desc* d, const ksj_gpu_gridding_tuning* t, Shape* s) {
  if (d == nullptr || d->struct_size < sizeof(ksj_gpu_gridding_desc)) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (d->channels == 0 || d->samples == 0 || d->frames == 0 || d->image_rows < 2 || d->image_cols < 2)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (d->dcf_mode > KSJ_GPU_DCF_EXTERNAL || d->output > KSJ_GPU_OUTPUT_COIL_MAJOR ||
      d->sample_format > KSJ_GPU_SAMPLES_BF16)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (!std::isfinite(d->row_origin) || !std::isfinite(d->col_origin)) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (d->samples > (1u << 26) || d->channels > 4096 || d->frames > 65535) return KSJ_GPU_ERROR_UNSUPPORTED;
  s->kb = d->kernel == KSJ_GPU_KERNEL_KAISER_BESSEL;
  if (d->kernel == KSJ_GPU_KERNEL_LINEAR) {
    if (d->kernel_width != 2 || d->grid_rows != d->image_rows || d->grid_cols != d->image_cols)
      return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  } else if (s->kb) {
    if (d->kernel_width < 2 || d->kernel_width > kMaxWidth || (d->kernel_width & 1u) != 0)
      return KSJ_GPU_ERROR_INVALID_ARGUMENT;
    if (d->grid_rows < d->image_rows || d->grid_cols < d->image_cols || d->grid_rows < d->kernel_width ||
        d->grid_cols < d->kernel_width)
      return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  } else {
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  }
  if (!is_fft_size(d->grid_rows) || !is_fft_size(d->grid_cols)) return KSJ_GPU_ERROR_UNSUPPORTED;
  s->frames = static_cast<int>(d->frames);
  s->channels = static_cast<int>(d->channels);
  s->samples = static_cast<int>(d->samples);
  s->rows = static_cast<int>(d->image_rows);
  s->cols = static_cast<int>(d->image_cols);
  s->grid_rows = static_cast<int>(d->grid_rows);
  s->grid_cols = static_cast<int>(d->grid_cols);
  s->width = static_cast<int>(d->kernel_width);
  s->nchunks = (s->grid_cols + kChunk - 1) / kChunk;
  s->lists_per_frame = s->grid_rows * s->nchunks;
  s->entries_per_frame = static_cast<size_t>(s->samples) * s->width * 2;
  s->out_rows = s->rows;
  s->out_cols = s->cols;
  s->col_group = 2;
  while (s->col_group < s->channels && s->col_group < 32) s->col_group <<= 1;
  s->cpitch = (s->channels + s->col_group - 1) / s->col_group * s->col_group;
  s->row_origin = static_cast<float>(d->row_origin);
  s->col_origin = static_cast<float>(d->col_origin);
  if (s->kb) {
    const double sigma = static_cast<double>(d->grid_rows) / static_cast<double>(d->image_rows);
    double beta = d->kb_beta;
    if (!(beta > 0.0)) {
      const double a = (static_cast<double>(d->kernel_width) / sigma) * (sigma - 0.5);
      const double arg = a * a - 0.8;
      if (arg <= 0.0) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
      beta = 3.14159265358979323846 * std::sqrt(arg);
    }
    s->beta = static_cast<float>(beta);
    s->inv_i0_beta = static_cast<float>(1.0 / std::cyl_bessel_i(0.0, beta));
    // exp(i k (q + delta)), delta = n/2 - origin: the image is centred on
    // offsets q = p - n/2 so the deapodisation sees |q| <= n/2.
    s->phase_row = static_cast<float>(static_cast<double>(s->rows / 2) - d->row_origin);
    s->phase_col = static_cast<float>(static_cast<double>(s->cols / 2) - d->col_origin);
    s->phase_sign = 1.0f;
    if (static_cast<double>(s->phase_row) != static_cast<double>(s->rows / 2) - d->row_origin ||
        static_cast<double>(s->phase_col) != static_cast<double>(s->cols / 2) - d->col_origin)
      return KSJ_GPU_ERROR_UNSUPPORTED;
  } else {
    s->beta = 0.0f;
    s->inv_i0_beta = 0.0f;
    // exp(-i (k_r r0 + k_c c0)) (eigen_radial_gridding.cpp:330-334)
    s->phase_row = s->row_origin;
    s->phase_col = s->col_origin;
    s->phase_sign = -1.0f;
    if (static_cast<double>(s->row_origin) != d->row_origin || static_cast<double>(s->col_origin) != d->col_origin)
      return KSJ_GPU_ERROR_UNSUPPORTED;  // origins must be exact floats (the reference casts them, :320-321)
  }
  make_dif_plan(s->grid_rows, &s->plan_rows);
  make_dif_plan(s->grid_cols, &s->plan_cols);

  // tuning
  int cg = t && t->coil_group ? static_cast<int>(t->coil_group) : 0;
  int cb = t && t->column_block ? static_cast<int>(t->column_block) : 0;
  int cap = t && t->list_capacity ? static_cast<int>(t->list_capacity) : 0;
  if (cap == 0) cap = 512;
  if (cap < 64 || cap > 2048 || (cap & (cap - 1)) != 0) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  const size_t smem_limit = 200 * 1024;
  auto rows_smem = [&](int g) {
    return rows_smem_for(s->grid_cols, g, s->width, rows_threads_for(s->grid_cols));
  };
  if (cg == 0) {
    int want = 1;
    while (want < s->channels && want < 32) want <<= 1;
    cg = want;
    // two row blocks per SM when they fit: (228 KiB - 2 x 1 KiB reserved) / 2;
    // rows wider than 384 columns run one 512-thread block per SM whatever
    // the group, and there the whole 32-coil register path wins (grid 512,
    // 32 coils: 4.8 against 8.6 ms per 16-frame call with a 16-coil group)
    const size_t per_block = rows_threads_for(s->grid_cols) <= 384 ? 115712 : smem_limit;
    while (cg > 1 && rows_smem(cg) > per_block) cg >>= 1;
  }
  if (cg < 1 || cg > 32 || (cg & (cg - 1)) != 0 || rows_smem(cg) > smem_limit) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  // column pass: cb columns x col_group coils per tile (a power of two
  // number of lines, at most the block's threads), double-buffered when the
  // channels take more than one tile
  const int cgroups = s->cpitch / s->col_group;
  auto cols_tile = [&](int b) {
    return static_cast<size_t>(s->grid_rows) * b * s->col_group * sizeof(float2) * (cgroups > 1 ? 2 : 1);
  };
  if (cb == 0) {
    cb = std::max(1, 32 / s->col_group);
    while (cb > 1 && (cols_tile(cb) > 110 * 1024 || cb > s->out_cols)) cb >>= 1;
  }
  if (cb < 1 || cb > 32 || (cb & (cb - 1)) != 0 || cb > s->out_cols || cb * s->col_group > kColsThreads ||
      cols_tile(cb) > smem_limit)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  s->coil_group = cg;
  s->column_block = cb;
  s->list_capacity = cap;
  // frames per k_rows/k_cols pass: keep one pass's row-transformed grid
  // (channels x grid_rows x out_cols complex) within ~64 MB of L2
  // fields appended to the tuning struct are read only when the caller's
  // struct_size covers them
  auto has = [&](size_t field_end) { return t != nullptr && t->struct_size >= field_end; };
  int fpp = has(offsetof(ksj_gpu_gridding_tuning, frames_per_pass) + 4) ? static_cast<int>(t->frames_per_pass) : 0;
  // default: two passes (on two streams, so one pass's last partial wave
  // overlaps the other) once there are enough frames to split
  if (fpp <= 0) fpp = s->frames >= 4 ? (s->frames + 1) / 2 : s->frames;
  s->frames_per_pass = std::min(fpp, s->frames);
  int rb = has(offsetof(ksj_gpu_gridding_tuning, rows_blocks_per_sm) + 4) ? static_cast<int>(t->rows_blocks_per_sm) : 0;
  // default: two row CTAs per SM wherever the row kernel fits them (384
  // threads; the coil group above was sized for two CTAs' shared memory)
  if (rb == 0) rb = rows_threads_for(s->grid_cols) <= 384 && rows_smem(cg) <= 115712 ? 2 : 1;
  if (rb != 1 && rb != 2) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  s->rows_blocks = rb;
  int parts = has(offsetof(ksj_gpu_gridding_tuning, coil_parts) + 4) ? static_cast<int>(t->coil_parts) : 0;
  if (parts == 0) parts = 1;
  if ((parts != 1 && parts != 2) || parts > cg) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  s->coil_parts = parts;
  s->wait_fault = has(offsetof(ksj_gpu_gridding_tuning, wait_fault_polls) + 4) ? t->wait_fault_polls : 0u;
  int cp = has(offsetof(ksj_gpu_gridding_tuning, column_pass) + 4) ? static_cast<int>(t->column_pass) : 0;
  if (cp < 0 || cp > 2) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  s->column_pass = cp == 0 ? 1 : cp;  // one CTA per tile unless asked (measured faster on the 384 grid)
  return KSJ_GPU_OK;
}

size_t sample_bytes(uint32_t format) { return format == KSJ_GPU_SAMPLES_BF16 ? 4 : 8; }

Layout make_layout(const Shape& s, const ksj_gpu_gridding_desc* d) {
  Layout l{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off = align_up(off + bytes, 256);
    return at;
  };
  const size_t fm = static_cast<size_t>(s.frames) * s.samples;
  const size_t nl = static_cast<size_t>(s.frames) * s.lists_per_frame;
  l.flags = take(kFlagBytes);
  l.frame_flags = take(static_cast<size_t>(s.frames) * 4);
  l.records = take(fm * record_bytes(s.width));
  l.counts = take(nl * 4);
  l.cursor = take(nl * 4);
  l.offsets = take((nl + s.frames) * 4);
  l.entries = take(static_cast<size_t>(s.frames) * s.entries_per_frame * 4);
  l.expanded = take(static_cast<size_t>(s.frames) * s.entries_per_frame * meta_vecs(s.width) * 16);
  l.long_lists = take((2 + static_cast<size_t>(s.frames) * s.entries_per_frame / (s.list_capacity + 1)) * 4);
  l.samples_t = take(fm * s.channels * sample_bytes(d->sample_format));
  l.inter = take(static_cast<size_t>(s.frames) * s.grid_rows * s.out_cols * s.cpitch * sizeof(float2));
  l.coil_last = d->output == KSJ_GPU_OUTPUT_COIL_MAJOR
                    ? take(static_cast<size_t>(s.frames) * s.channels * s.out_rows * s.out_cols * sizeof(float2))
                    : off;
  // tables: twiddles for rows and cols, inverse deapodisation for rows and
  // cols, and the FFT output position of every kept row and column
  l.tables = take((static_cast<size_t>(s.grid_rows) + s.grid_cols) * sizeof(float2) +
                  (static_cast<size_t>(s.out_rows) + s.out_cols) * (sizeof(float) + sizeof(int)));
  l.total = off;
  return l;
}

// ------------------------------------------------------------------ kernels

// Twiddles exp(2 pi i t / n) for both axes and the inverse deapodisation
// factors 1 / psi(q), q = p - n/2, psi the continuous Fourier transform of the
// normalised Kaiser-Bessel kernel: W sinh(z)/z / I0(beta),
// z = sqrt(beta^2 - (pi W q / g)^2) (Jackson et al. 1991).  FP64 here only.
//
// pos_rows[p] / pos_cols[p]: where the in-place DIF leaves the frequency
// index that kept image row / column p takes: p itself for the linear
// operator (no oversampling), (p - n/2) mod g for Kaiser-Bessel (the image is
// centred on q = p - n/2).
__global__ void k_tables(float2* tw_rows, int grid_rows, float2* tw_cols, int grid_cols, float* inv_dr, int out_rows,
                         float* inv_dc, int out_cols, int* pos_rows, int* pos_cols, DifPlan plan_rows,
                         DifPlan plan_cols, int kb, int width, double beta, double i0_beta) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  auto source = [&](int p, int n, int g) { return kb ? (p - n / 2 + g) % g : p; };
  if (i < out_rows) {
    const int k = source(i, out_rows, grid_rows);
    pos_rows[i] = has_two_step_rows(grid_rows) ? two_step_slot(k, grid_rows) : dif_position(plan_rows, k);
  }
  if (i < out_cols) pos_cols[i] = dif_position(plan_cols, source(i, out_cols, grid_cols));
  if (i < grid_rows) tw_rows[i] = twiddle(i, grid_rows);
  if (i < grid_cols) tw_cols[i] = twiddle(i, grid_cols);
  auto inv_psi = [&](int p, int n, int g) -> float { return kb ? kb_inv_deapod(p, n, g, width, beta, i0_beta) : 1.0f; };
  if (i < out_rows) inv_dr[i] = inv_psi(i, out_rows, grid_rows);
  if (i < out_cols) inv_dc[i] = inv_psi(i, out_cols, grid_cols);
}

__global__ void __launch_bounds__(256) k_fill(float* p, int n, float v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

struct PrepareArgs {
  const float* traj;
  const float* dcf;
  const uint32_t* frame_samples;  // ragged batches: valid samples of each frame (null: all)
  const uint64_t* frame_traj;     // ragged batches: address of each frame's trajectory [M_f][2]
  uint32_t* frame_flags;          // per-frame copy of the check flags (null: none)
  uint32_t dcf_mode;
  uint32_t require_nyquist;
  unsigned char* records;
  uint32_t* counts;
  uint32_t* flags;
  int frames, samples, grid_rows, grid_cols, nchunks, lists_per_frame;
  int kb;
  float beta, two_over_w, inv_i0_beta;
  float phase_row, phase_col, phase_sign;
};

template <int W>
__device__ __forceinline__ void list_chunks(int c0, int grid_cols, int* k0, int* k1) {
  const int last = c0 + W - 1 >= grid_cols ? c0 + W - 1 - grid_cols : c0 + W - 1;
  *k0 = c0 / kChunk;
  *k1 = last / kChunk;
}

template <int W>
__global__ void __launch_bounds__(256) k_prepare(PrepareArgs a) {
  const size_t idx = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const size_t total = static_cast<size_t>(a.frames) * a.samples;
  if (idx >= total) return;
  const int f = static_cast<int>(idx / a.samples);
  if (a.frame_samples != nullptr &&
      idx - static_cast<size_t>(f) * a.samples >= static_cast<size_t>(__ldg(a.frame_samples + f))) {
    // a padding sample of a ragged batch: in no list (its trajectory is not read)
    reinterpret_cast<SampleRecord<W>*>(a.records)[idx].r0 = -1;
    return;
  }
  const float2 k =
      a.frame_traj != nullptr
          ? reinterpret_cast<const float2*>(__ldg(a.frame_traj + f))[idx - static_cast<size_t>(f) * a.samples]
          : __ldg(reinterpret_cast<const float2*>(a.traj) + idx);
  bool ok = isfinite(k.x) && isfinite(k.y);
  if (ok && a.require_nyquist) ok = k.x >= -kPiF && k.x <= kPiF && k.y >= -kPiF && k.y <= kPiF;
  // a coordinate far outside the grid would overflow the int tap arithmetic
  if (ok && !a.require_nyquist) ok = fabsf(k.x) < 1.0e4f && fabsf(k.y) < 1.0e4f;
  float w = 1.0f;
  if (a.dcf_mode == KSJ_GPU_DCF_ANALYTIC_RAMP) {
    w = hypotf(k.x, k.y);
  } else if (a.dcf_mode == KSJ_GPU_DCF_EXTERNAL) {
    w = __ldg(a.dcf + idx);
    if (!(isfinite(w) && w >= 0.0f)) {
      atomicOr(a.flags, KSJ_GPU_FLAG_BAD_DCF);
      if (a.frame_flags) atomicOr(a.frame_flags + f, KSJ_GPU_FLAG_BAD_DCF);
      w = 0.0f;
    }
  }
  SampleRecord<W> rec;
  if (!ok) {
    atomicOr(a.flags, KSJ_GPU_FLAG_BAD_TRAJECTORY);
    if (a.frame_flags) atomicOr(a.frame_flags + f, KSJ_GPU_FLAG_BAD_TRAJECTORY);
    rec.r0 = 0;
    rec.c0 = 0;
    rec.scale = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int j = 0; j < W; ++j) {
      rec.wr[j] = 0.0f;
      rec.wc[j] = 0.0f;
    }
  } else {
    const dfloat ur = grid_coordinate(k.x, static_cast<float>(a.grid_rows));
    const dfloat uc = grid_coordinate(k.y, static_cast<float>(a.grid_cols));
    float fr, fc;
    const int lr = dfloor(ur, &fr);
    const int lc = dfloor(uc, &fc);
    if (!a.kb) {
      // periodic 2x2 linear stencil (eigen_radial_gridding.cpp:325-342)
      rec.r0 = wrap_index(lr, a.grid_rows);
      rec.c0 = wrap_index(lc, a.grid_cols);
      rec.wr[0] = 1.0f - fr;
      rec.wr[1] = fr;
      rec.wc[0] = 1.0f - fc;
      rec.wc[1] = fc;
#pragma unroll
      for (int j = 2; j < W; ++j) {
        rec.wr[j] = 0.0f;
        rec.wc[j] = 0.0f;
      }
    } else {
      const int sr = lr - W / 2 + 1;
      const int sc = lc - W / 2 + 1;
      rec.r0 = wrap_index(sr, a.grid_rows);
      rec.c0 = wrap_index(sc, a.grid_cols);
#pragma unroll
      for (int j = 0; j < W; ++j) {
        // offset (tap - u), exact in its high part
        const float dr = __fsub_rn(__fsub_rn(static_cast<float>(sr + j), ur.hi), ur.lo);
        const float dc = __fsub_rn(__fsub_rn(static_cast<float>(sc + j), uc.hi), uc.lo);
        rec.wr[j] = kb_weight(dr, a.two_over_w, a.beta, a.inv_i0_beta);
        rec.wc[j] = kb_weight(dc, a.two_over_w, a.beta, a.inv_i0_beta);
      }
    }
    const float2 e = exp_i_dot(k.x, a.phase_row, k.y, a.phase_col, a.phase_sign);
    rec.scale = cscale(e, w);
  }
  reinterpret_cast<SampleRecord<W>*>(a.records)[idx] = rec;
  int k0, k1;
  list_chunks<W>(rec.c0, a.grid_cols, &k0, &k1);
  uint32_t* counts = a.counts + static_cast<size_t>(f) * a.lists_per_frame;
#pragma unroll
  for (int j = 0; j < W; ++j) {
    int row = rec.r0 + j;
    if (row >= a.grid_rows) row -= a.grid_rows;
    atomicAdd(counts + row * a.nchunks + k0, 1u);
    if (k1 != k0) atomicAdd(counts + row * a.nchunks + k1, 1u);
  }
}

// Exclusive scan of one frame's list counts (one block per frame).
__global__ void __launch_bounds__(1024) k_scan(const uint32_t* counts, uint32_t* offsets, int lists) {
  __shared__ uint32_t warp_sums[32];
  const int f = blockIdx.x;
  const uint32_t* c = counts + static_cast<size_t>(f) * lists;
  uint32_t* o = offsets + static_cast<size_t>(f) * (lists + 1);
  const int per = (lists + blockDim.x - 1) / blockDim.x;
  const int begin = threadIdx.x * per;
  const int end = min(begin + per, lists);
  uint32_t local = 0;
  for (int i = begin; i < end; ++i) local += c[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = local;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += v;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    uint32_t ws = lane < nw ? warp_sums[lane] : 0u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t v = __shfl_up_sync(0xffffffffu, ws, d);
      if (lane >= d) ws += v;
    }
    if (lane < nw) warp_sums[lane] = ws;
  }
  __syncthreads();
  uint32_t run = incl - local + (warp > 0 ? warp_sums[warp - 1] : 0u);
  for (int i = begin; i < end; ++i) {
    o[i] = run;
    run += c[i];
  }
  if (threadIdx.x == blockDim.x - 1) o[lists] = run;
}

template <int W>
__global__ void __launch_bounds__(256) k_scatter(const unsigned char* records, const uint32_t* offsets,
                                                 uint32_t* cursor, uint32_t* entries, int frames, int samples,
                                                 int grid_rows, int grid_cols, int nchunks, size_t entries_per_frame) {
  const size_t idx = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= static_cast<size_t>(frames) * samples) return;
  const int f = static_cast<int>(idx / samples);
  const int s = static_cast<int>(idx - static_cast<size_t>(f) * samples);
  const SampleRecord<W>* rec = reinterpret_cast<const SampleRecord<W>*>(records) + idx;
  const int r0 = rec->r0;
  if (r0 < 0) return;  // padding sample of a ragged batch
  const int c0 = rec->c0;
  int k0, k1;
  list_chunks<W>(c0, grid_cols, &k0, &k1);
  const int lists = grid_rows * nchunks;
  const uint32_t* off = offsets + static_cast<size_t>(f) * (lists + 1);
  uint32_t* cur = cursor + static_cast<size_t>(f) * lists;
  uint32_t* ent = entries + static_cast<size_t>(f) * entries_per_frame;
#pragma unroll
  for (int j = 0; j < W; ++j) {
    int row = r0 + j;
    if (row >= grid_rows) row -= grid_rows;
    const int l0 = row * nchunks + k0;
    ent[off[l0] + atomicAdd(cur + l0, 1u)] = static_cast<uint32_t>(s);
    if (k1 != k0) {
      const int l1 = row * nchunks + k1;
      ent[off[l1] + atomicAdd(cur + l1, 1u)] = static_cast<uint32_t>(s);
    }
  }
}

// Warp-cooperative ascending sort of buf[0, n) (shared or global memory):
// the bitonic network in its all-ascending form (first comparator of each
// merge flipped), so positions >= n behave as +infinity and are never
// touched -- no padding is needed.
__device__ __forceinline__ void warp_sort(uint32_t* buf, int n, int lane) {
  int p = 1;
  while (p < n) p <<= 1;
  for (int k = 2; k <= p; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < p; i += 32) {
        const int partner = (j == (k >> 1)) ? (i ^ (k - 1)) : (i ^ j);
        if (partner > i && partner < n) {
          const uint32_t a = buf[i], b = buf[partner];
          if (a > b) {
            buf[i] = b;
            buf[partner] = a;
          }
        }
      }
      __syncwarp();
    }
  }
}

// One list entry as k_rows consumes it (meta_vecs(W) 16-byte vectors):
//   v0 = {tap word, sample index, scale.re, scale.im}, v1.. = the W column
//   weights times this row's weight (zero padded).
// The tap word holds the mask of taps that land in the list's column chunk
// (bits 0-7) and the column of tap 0 as seen from the chunk (bits 9 up, one
// row-length lower when the taps reaching the chunk wrapped past the last
// column); bit 8 marks a one-chunk row that sees both ends of a wrap, whose
// taps are wrapped one by one.
template <int W>
__device__ __forceinline__ void expand_taps(uint32_t sidx, int c0, float sre, float sim, float wrow, const float* wc,
                                            int col_lo, int col_hi, int grid_cols, float4* out) {
  constexpr int kMV = meta_vecs(W);
  const int cb0 = c0 >= col_hi ? c0 - grid_cols : c0;
  uint32_t in_chunk = 0, straight = 0;
#pragma unroll
  for (int j = 0; j < W; ++j) {
    int col = c0 + j;
    if (col >= grid_cols) col -= grid_cols;
    if (col >= col_lo && col < col_hi) in_chunk |= 1u << j;
    if (cb0 + j >= col_lo && cb0 + j < col_hi) straight |= 1u << j;
  }
  const int word0 = in_chunk == straight ? ((cb0 * 512) | static_cast<int>(in_chunk))
                                         : ((c0 * 512) | 256 | static_cast<int>(in_chunk));
  out[0] = make_float4(__int_as_float(word0), __uint_as_float(sidx), sre, sim);
#pragma unroll
  for (int v = 1; v < kMV; ++v) {
    float t4[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int j = 4 * (v - 1) + u;
      t4[u] = j < W ? wrow * wc[j] : 0.0f;
    }
    out[v] = make_float4(t4[0], t4[1], t4[2], t4[3]);
  }
}

// One list entry as k_rows consumes it (meta_vecs(W) 16-byte vectors):
//   v0 = {tap word, sample index, scale.re, scale.im}, v1.. = the W column
//   weights times this row's weight (zero padded).
// The tap word holds the mask of taps that land in the list's column chunk
// (bits 0-7) and the column of tap 0 as seen from the chunk (bits 9 up, one
// row-length lower when the taps reaching the chunk wrapped past the last
// column); bit 8 marks a one-chunk row that sees both ends of a wrap, whose
// taps are wrapped one by one.
template <int W>
__device__ __forceinline__ void expand_entry(const SampleRecord<W>* recs, uint32_t sidx, int row, int col_lo,
                                             int col_hi, int grid_rows, int grid_cols, float4* out) {
  constexpr int kRV = static_cast<int>(sizeof(SampleRecord<W>) / 16);
  float4 q[kRV];
  const float4* rp = reinterpret_cast<const float4*>(recs + sidx);
#pragma unroll
  for (int v = 0; v < kRV; ++v) q[v] = __ldg(rp + v);
  const float* w = reinterpret_cast<const float*>(q);
  int ta = row - __float_as_int(w[0]);
  if (ta < 0) ta += grid_rows;
  float wr = 0.0f;
#pragma unroll
  for (int j = 0; j < W; ++j)
    if (j == ta) wr = w[4 + j];
  expand_taps<W>(sidx, __float_as_int(w[1]), w[2], w[3], wr, w + 4 + W, col_lo, col_hi, grid_cols, out);
}

// The 3-D form: the list's plane and row weights folded together.
template <int W>
__device__ __forceinline__ void expand_entry3(const SampleRecord3<W>* recs, uint32_t sidx, int plane, int row,
                                              int col_lo, int col_hi, int grid, float4* out) {
  constexpr int kRV = static_cast<int>(sizeof(SampleRecord3<W>) / 16);
  float4 q[kRV];
  const float4* rp = reinterpret_cast<const float4*>(recs + sidx);
#pragma unroll
  for (int v = 0; v < kRV; ++v) q[v] = __ldg(rp + v);
  const float* w = reinterpret_cast<const float*>(q);
  int tz = plane - __float_as_int(w[0]);
  if (tz < 0) tz += grid;
  int ta = row - __float_as_int(w[1]);
  if (ta < 0) ta += grid;
  float wz = 0.0f, wr = 0.0f;
#pragma unroll
  for (int j = 0; j < W; ++j) {
    if (j == tz) wz = w[6 + j];
    if (j == ta) wr = w[6 + W + j];
  }
  expand_taps<W>(sidx, __float_as_int(w[2]), w[4], w[5], wr * wz, w + 6 + 2 * W, col_lo, col_hi, grid, out);
}

struct SortArgs {
  const uint32_t* offsets;
  uint32_t* entries;
  const unsigned char* records;
  float4* expanded;
  uint32_t* long_lists;  // lists longer than `capacity`, left to k_sort_long
  uint32_t* long_count;
  int frames, samples, lists_per_frame, nchunks, grid_rows, grid_cols, capacity;
  size_t entries_per_frame;  // 0 when the offsets are absolute (3-D: one entry array for all planes)
  int dim3;                  // 3-D: frames are grid planes and the records are per sample (SampleRecord3)
};

// Expanded entry i of list l of frame f (sample index sidx).
template <int W>
__device__ __forceinline__ void expand_at(const SortArgs& a, int f, int l, uint32_t begin, int i, uint32_t sidx) {
  constexpr int kMV = meta_vecs(W);
  const int row = l / a.nchunks;
  const int col_lo = (l - row * a.nchunks) * kChunk;
  const int col_hi = min(col_lo + kChunk, a.grid_cols);
  float4* out = a.expanded + (static_cast<size_t>(f) * a.entries_per_frame + begin + i) * kMV;
  float4 e[kMV];
  if (a.dim3)
    expand_entry3<W>(reinterpret_cast<const SampleRecord3<W>*>(a.records), sidx, f, row, col_lo, col_hi, a.grid_cols,
                     e);
  else
    expand_entry<W>(reinterpret_cast<const SampleRecord<W>*>(a.records) + static_cast<size_t>(f) * a.samples, sidx, row,
                    col_lo, col_hi, a.grid_rows, a.grid_cols, e);
#pragma unroll
  for (int v = 0; v < kMV; ++v) out[v] = e[v];
}

// Expanded entries of list l of frame f, entries i = first, first + step, ...
template <int W>
__device__ __forceinline__ void expand_list(const SortArgs& a, int f, int l, uint32_t begin, int n,
                                            const uint32_t* sorted, int first, int step) {
  for (int i = first; i < n; i += step) expand_at<W>(a, f, l, begin, i, sorted[i]);
}

constexpr int kSortGroup = 4;  // consecutive lists per warp in k_sort

// One list (one warp): sort the sample indices ascending, then write every
// entry in its expanded form (the dependent record loads happen here, across
// many lists in flight, not in the row pass).  A list of at most 32 entries
// is ranked on registers: its sample indices are distinct, so the number of
// smaller indices is each entry's sorted position.  Longer lists are sorted
// in the warp's shared buffer; lists longer than the buffer are queued for
// k_sort_long.  The sorted indices themselves are written back only for the
// density-weight path (no expansion), the one reader of them.
template <int W>
__device__ __forceinline__ void sort_list(const SortArgs& a, int f, int l, uint32_t begin, int n, int lane,
                                          uint32_t* buf) {
  if (n == 0) return;
  if (n > a.capacity) {
    if (lane == 0)
      a.long_lists[atomicAdd(a.long_count, 1u)] = static_cast<uint32_t>(static_cast<size_t>(f) * a.lists_per_frame + l);
    return;
  }
  uint32_t* ent = a.entries + static_cast<size_t>(f) * a.entries_per_frame + begin;
  if (n <= 32) {
    const uint32_t key = lane < n ? ent[lane] : 0xffffffffu;
    int rank = 0;
    for (int j = 0; j < n; ++j) rank += __shfl_sync(0xffffffffu, key, j) < key ? 1 : 0;
    if (lane < n) {
      if (a.expanded == nullptr)
        ent[rank] = key;  // every lane read its key before the shuffles
      else
        expand_at<W>(a, f, l, begin, rank, key);
    }
    return;
  }
  for (int i = lane; i < n; i += 32) buf[i] = ent[i];
  __syncwarp();
  warp_sort(buf, n, lane);
  if (a.expanded == nullptr) {
    for (int i = lane; i < n; i += 32) ent[i] = buf[i];
    return;
  }
  expand_list<W>(a, f, l, begin, n, buf, lane, 32);
}

// kSortGroup consecutive lists of one frame per warp.  Their entries are
// contiguous; when there are at most 32 of them, lane i takes entry i of the
// group, finds its list from the list starts and ranks it among that list's
// entries (same order as sort_list), so tiny and empty lists share one warp.
template <int W>
__global__ void __launch_bounds__(256) k_sort(SortArgs a) {
  extern __shared__ uint32_t sort_buf[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int groups = (a.lists_per_frame + kSortGroup - 1) / kSortGroup;
  const size_t gg = static_cast<size_t>(blockIdx.x) * (blockDim.x >> 5) + warp;
  if (gg >= static_cast<size_t>(a.frames) * groups) return;
  const int f = static_cast<int>(gg / groups);
  const int l0 = static_cast<int>(gg - static_cast<size_t>(f) * groups) * kSortGroup;
  const int ng = min(kSortGroup, a.lists_per_frame - l0);
  const uint32_t* off = a.offsets + static_cast<size_t>(f) * (a.lists_per_frame + 1) + l0;
  const uint32_t my_off = lane <= ng ? off[lane] : 0u;  // lane s: start of list l0 + s
  const uint32_t begin = __shfl_sync(0xffffffffu, my_off, 0);
  const int total = static_cast<int>(__shfl_sync(0xffffffffu, my_off, ng) - begin);
  if (total == 0) return;
  if (total > 32) {
    uint32_t* buf = sort_buf + static_cast<size_t>(warp) * a.capacity;
    for (int s = 0; s < ng; ++s) {
      const uint32_t b = __shfl_sync(0xffffffffu, my_off, s);
      const uint32_t e = __shfl_sync(0xffffffffu, my_off, s + 1);
      sort_list<W>(a, f, l0 + s, b, static_cast<int>(e - b), lane, buf);
      __syncwarp();
    }
    return;
  }
  uint32_t* ent = a.entries + static_cast<size_t>(f) * a.entries_per_frame + begin;
  const bool live = lane < total;
  const uint32_t key = live ? ent[lane] : 0xffffffffu;
  int seg = 0;  // list of entry `lane` within the group (empty lists are skipped over)
#pragma unroll
  for (int s = 1; s < kSortGroup; ++s) {
    const uint32_t st = __shfl_sync(0xffffffffu, my_off, s);
    if (s < ng && begin + lane >= st) seg = s;
  }
  int rank = 0;
  for (int j = 0; j < total; ++j) {
    const uint32_t kj = __shfl_sync(0xffffffffu, key, j);
    const int sj = __shfl_sync(0xffffffffu, seg, j);
    rank += (sj == seg && kj < key) ? 1 : 0;
  }
  const uint32_t lbegin = __shfl_sync(0xffffffffu, my_off, seg);
  if (live) {
    if (a.expanded == nullptr)
      ent[lbegin - begin + rank] = key;  // every lane read its key before the shuffles
    else
      expand_at<W>(a, f, l0 + seg, lbegin, rank, key);
  }
}

constexpr int kLongSortThreads = 1024;
constexpr int kLongSortSmem = 16384;  // entries sorted in shared memory; longer lists in place in L2/HBM

// The same bitonic network over a whole block.
__device__ __forceinline__ void block_sort(uint32_t* buf, int n) {
  int p = 1;
  while (p < n) p <<= 1;
  for (int k = 2; k <= p; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < p; i += blockDim.x) {
        const int partner = (j == (k >> 1)) ? (i ^ (k - 1)) : (i ^ j);
        if (partner > i && partner < n) {
          const uint32_t x = buf[i], y = buf[partner];
          if (x > y) {
            buf[i] = y;
            buf[partner] = x;
          }
        }
      }
      __syncthreads();
    }
  }
}

// Stages (k, j) for j = j0, j0 / 2, ..., 1 of that network on the chunk of
// list elements [base, base + kLongSortSmem) held in buf (elements at or
// beyond n are absent).  Every pair of these stages lies inside the chunk:
// j < kLongSortSmem, and the mirrored partner of stage j = k / 2 only when
// k <= kLongSortSmem.
__device__ __forceinline__ void chunk_stages(uint32_t* buf, int base, int n, int k, int j0) {
  for (int j = j0; j > 0; j >>= 1) {
    for (int t = threadIdx.x; t < kLongSortSmem && base + t < n; t += blockDim.x) {
      const int i = base + t;
      const int partner = (j == (k >> 1)) ? (i ^ (k - 1)) : (i ^ j);
      if (partner > i && partner < n) {
        const uint32_t x = buf[t], y = buf[partner - base];
        if (x > y) {
          buf[t] = y;
          buf[partner - base] = x;
        }
      }
    }
    __syncthreads();
  }
}

// The network of block_sort on a list longer than the shared buffer, in
// place in global memory, with every stage whose pairs lie inside one
// kLongSortSmem-entry chunk run on that chunk in shared memory: first each
// chunk sorted whole (k up to the chunk size), then per larger k the stages
// with j >= the chunk size over global memory and the rest chunk by chunk.
// Same comparisons in the same stage order as block_sort: the same result.
__device__ __forceinline__ void chunk_load(uint32_t* buf, const uint32_t* ent, int base, int n) {
  for (int t = threadIdx.x; t < kLongSortSmem && base + t < n; t += blockDim.x) buf[t] = ent[base + t];
  __syncthreads();
}
__device__ __forceinline__ void chunk_store(const uint32_t* buf, uint32_t* ent, int base, int n) {
  for (int t = threadIdx.x; t < kLongSortSmem && base + t < n; t += blockDim.x) ent[base + t] = buf[t];
  __syncthreads();
}
__device__ __forceinline__ void block_sort_chunked(uint32_t* ent, int n, uint32_t* buf) {
  int p = 1;
  while (p < n) p <<= 1;
  for (int base = 0; base < n; base += kLongSortSmem) {
    chunk_load(buf, ent, base, n);
    for (int k = 2; k <= kLongSortSmem; k <<= 1) chunk_stages(buf, base, n, k, k >> 1);
    chunk_store(buf, ent, base, n);
  }
  for (int k = 2 * kLongSortSmem; k <= p; k <<= 1) {
    for (int j = k >> 1; j >= kLongSortSmem; j >>= 1) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int partner = (j == (k >> 1)) ? (i ^ (k - 1)) : (i ^ j);
        if (partner > i && partner < n) {
          const uint32_t x = ent[i], y = ent[partner];
          if (x > y) {
            ent[i] = y;
            ent[partner] = x;
          }
        }
      }
      __syncthreads();
    }
    for (int base = 0; base < n; base += kLongSortSmem) {
      chunk_load(buf, ent, base, n);
      chunk_stages(buf, base, n, k, kLongSortSmem >> 1);
      chunk_store(buf, ent, base, n);
    }
  }
}

template <int W>
__device__ __forceinline__ void sort_long_list(const SortArgs& a, size_t gl, uint32_t* long_buf) {
  const int f = static_cast<int>(gl / a.lists_per_frame);
  const int l = static_cast<int>(gl - static_cast<size_t>(f) * a.lists_per_frame);
  const uint32_t* off = a.offsets + static_cast<size_t>(f) * (a.lists_per_frame + 1);
  const uint32_t begin = off[l];
  const int n = static_cast<int>(off[l + 1] - begin);
  uint32_t* ent = a.entries + static_cast<size_t>(f) * a.entries_per_frame + begin;
  const uint32_t* sorted = ent;
  if (n <= kLongSortSmem) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) long_buf[i] = ent[i];
    __syncthreads();
    block_sort(long_buf, n);
    if (a.expanded == nullptr)
      for (int i = threadIdx.x; i < n; i += blockDim.x) ent[i] = long_buf[i];
    sorted = long_buf;
  } else {
    block_sort_chunked(ent, n, long_buf);
  }
  __syncthreads();
  if (a.expanded != nullptr) expand_list<W>(a, f, l, begin, n, sorted, threadIdx.x, blockDim.x);
}

// Blocks take the queued long lists in turn: sort (in shared memory up to
// kLongSortSmem entries, else in place with chunk-local stages in shared
// memory) and expand.
template <int W>
__global__ void __launch_bounds__(kLongSortThreads, 1) k_sort_long(SortArgs a) {
  extern __shared__ uint32_t long_buf[];
  const uint32_t queued = *a.long_count;
  for (uint32_t q = blockIdx.x; q < queued; q += gridDim.x) {
    sort_long_list<W>(a, a.long_lists[q], long_buf);
    __syncthreads();
  }
}

// Launch k_sort and then k_sort_long for the lists it queued.
template <int W>
ksj_gpu_status launch_sort(SortArgs sa, size_t lists, size_t entries_total, int capacity, cudaStream_t stream) {
  if (cudaMemsetAsync(sa.long_count, 0, sizeof(uint32_t), stream) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  const size_t smem = static_cast<size_t>(8) * capacity * 4;
  if (cudaFuncSetAttribute(k_sort<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) !=
          cudaSuccess ||
      cudaFuncSetAttribute(k_sort_long<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, kLongSortSmem * 4) !=
          cudaSuccess)
    return KSJ_GPU_ERROR_CUDA;
  {
    LaunchScope scope("k_sort", stream);
    const size_t warps = static_cast<size_t>(sa.frames) * ((sa.lists_per_frame + kSortGroup - 1) / kSortGroup);
    k_sort<W><<<static_cast<unsigned>((warps + 7) / 8), 256, smem, stream>>>(sa);
  }
  const size_t most = std::max<size_t>(1, entries_total / (static_cast<size_t>(capacity) + 1));
  LaunchScope scope("k_sort_long", stream);
  k_sort_long<W><<<static_cast<unsigned>(std::min<size_t>(std::min<size_t>(most, lists), 1024)), kLongSortThreads,
                   kLongSortSmem * 4, stream>>>(sa);
  return KSJ_GPU_OK;
}

// [frame][channel][sample] -> [frame][sample][channel] through a 32x33
// shared tile (launch (32, 8) threads, grid (ceil(samples/32),
// ceil(channels/32), frames)), checking every sample on the way: a
// non-finite value (either component; bf16 exponent all ones) raises
// KSJ_GPU_FLAG_NONFINITE_SAMPLE.
//
// Ragged batches (frame_channels / frame_samples / frame_src non-null):
// frame f holds frame_channels[f] coils of frame_samples[f] samples, packed
// [channel][sample] at address frame_src[f] (device memory, or host memory
// the device reads in place); the padding up to the call's channels and
// samples is written as zeros.
template <uint32_t kFormat>
__global__ void __launch_bounds__(256) k_samples_coil_last(const void* in_raw, void* out_raw, int channels,
                                                           int samples, uint32_t* flags,
                                                           const uint32_t* frame_channels,
                                                           const uint32_t* frame_samples,
                                                           const uint64_t* frame_src, int frame0,
                                                           uint32_t* frame_flags) {
  using T = typename std::conditional<kFormat == KSJ_GPU_SAMPLES_BF16, uint32_t, unsigned long long>::type;
  __shared__ T t[32][33];
  const T* in = static_cast<const T*>(in_raw);
  T* out = static_cast<T*>(out_raw);
  const int f = blockIdx.z;
  const int s0 = blockIdx.x * 32;
  const int c0 = blockIdx.y * 32;
  T* dst = out + static_cast<size_t>(f) * channels * samples;
  const int live_c = frame_channels ? min(channels, static_cast<int>(__ldg(frame_channels + frame0 + f))) : channels;
  const int live_s = frame_samples ? min(samples, static_cast<int>(__ldg(frame_samples + frame0 + f))) : samples;
  // ragged frames are packed at their own sample count
  const T* src = frame_src ? reinterpret_cast<const T*>(__ldg(frame_src + frame0 + f))
                           : in + static_cast<size_t>(f) * channels * samples;
  const int pitch = frame_src ? live_s : samples;
  bool bad = false;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int c = c0 + y, sm = s0 + threadIdx.x;
    if (c < channels && sm < samples) {
      if (c >= live_c || sm >= live_s) {
        t[y][threadIdx.x] = T(0);
        continue;
      }
      const T v = src[static_cast<size_t>(c) * pitch + sm];
      if (kFormat == KSJ_GPU_SAMPLES_BF16) {
        const uint32_t u = static_cast<uint32_t>(v);
        bad |= (u & 0x7f80u) == 0x7f80u || (u & 0x7f800000u) == 0x7f800000u;
      } else {
        const uint64_t u = static_cast<uint64_t>(v);
        bad |= (u & 0x7f800000ull) == 0x7f800000ull || (u & 0x7f80000000000000ull) == 0x7f80000000000000ull;
      }
      t[y][threadIdx.x] = v;
    }
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0 && threadIdx.y == 0) {
    atomicOr(flags, KSJ_GPU_FLAG_NONFINITE_SAMPLE);
    if (frame_flags) atomicOr(frame_flags + frame0 + f, KSJ_GPU_FLAG_NONFINITE_SAMPLE);
  }
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int sm = s0 + y, c = c0 + threadIdx.x;
    if (c < channels && sm < samples) dst[static_cast<size_t>(sm) * channels + c] = t[threadIdx.x][y];
  }
}

struct RowsArgs {
  int frame0;             // first frame of this pass
  const void* samples_t;  // [frame][sample][channel]
  size_t sample_frame_stride;  // elements between frames of samples_t (0: one sample set for all frames)
  const uint32_t* offsets;
  const float4* expanded;  // sorted list entries, expanded (meta_vecs(W) vectors each)
  const float2* tw_cols;
  const int* pos_cols;    // DIF output position of each kept column
  float2* inter;          // [frame][grid_row][out_col][cpitch]
  uint32_t* flags;
  int frames, channels, samples, grid_rows, grid_cols, nchunks, lists_per_frame;
  size_t entries_per_frame;
  int coil_group, coil_parts;
  int out_cols, cpitch;
  int col_shift;  // kept column of frequency k: (k + col_shift) mod grid_cols, when below out_cols
  uint32_t wait_limit;   // polls before a segment wait gives up
  int wait_beyond;       // added to every segment wait's target: 0, or unreachable in the wait-fault test mode
  DifPlan plan;
};

// Accumulator layout [column][coil]: gridding, the row FFT and the write-out
// all put consecutive coils on consecutive lanes at one column, so every
// shared-memory access of the block reads or writes contiguous float2s.
struct AccAddr {
  int cg;
  __device__ __forceinline__ int operator()(int coil, int col) const { return col * cg + coil; }
};

// Register form of one column chunk (lane = coil): r[t] is the cell of column
// col_lo + t.  A straight entry's taps are the columns cbase + j, so with the
// warp-uniform d = cbase - col_lo every tap is a compile-time register index
// (one switch case per d).  Taps at t < 0 or t >= kChunk belong to other
// lists' chunks and are dropped; taps at width <= t < kChunk (a partial last
// chunk) land in registers that are never stored.
template <int W, int D, int J = 0>
__device__ __forceinline__ void chunk_taps_at(float2 (&r)[kChunk], float2 v, const float* wt) {
  if constexpr (J < W) {
    if constexpr (D + J >= 0 && D + J < kChunk) {
      r[D + J].x = fmaf(v.x, wt[J], r[D + J].x);
      r[D + J].y = fmaf(v.y, wt[J], r[D + J].y);
    }
    chunk_taps_at<W, D, J + 1>(r, v, wt);
  }
}

template <int W>
__device__ __forceinline__ void chunk_taps(float2 (&r)[kChunk], int d, float2 v, const float* wt) {
  static_assert(W <= 8 && kChunk == 16, "cases cover d in [-7, 15]");
  switch (d) {
#define KSJ_TAPS_CASE(D) \
  case D:                \
    chunk_taps_at<W, D>(r, v, wt); \
    break;
    KSJ_TAPS_CASE(-7) KSJ_TAPS_CASE(-6) KSJ_TAPS_CASE(-5) KSJ_TAPS_CASE(-4) KSJ_TAPS_CASE(-3) KSJ_TAPS_CASE(-2)
    KSJ_TAPS_CASE(-1) KSJ_TAPS_CASE(0) KSJ_TAPS_CASE(1) KSJ_TAPS_CASE(2) KSJ_TAPS_CASE(3) KSJ_TAPS_CASE(4)
    KSJ_TAPS_CASE(5) KSJ_TAPS_CASE(6) KSJ_TAPS_CASE(7) KSJ_TAPS_CASE(8) KSJ_TAPS_CASE(9) KSJ_TAPS_CASE(10)
    KSJ_TAPS_CASE(11) KSJ_TAPS_CASE(12) KSJ_TAPS_CASE(13) KSJ_TAPS_CASE(14) KSJ_TAPS_CASE(15)
#undef KSJ_TAPS_CASE
    default:
      break;
  }
}

// Entries whose taps wrap around the grid inside one chunk (grids of at most
// one chunk): the in-chunk taps of the mask, each at its wrapped column.
template <int W>
__device__ __forceinline__ void chunk_taps_wrapped(float2 (&r)[kChunk], int c0, uint32_t mask, int col_lo,
                                                   int grid_cols, float2 v, const float* wt) {
#pragma unroll
  for (int j = 0; j < W; ++j) {
    if (!((mask >> j) & 1u)) continue;
    int col = c0 + j;
    if (col >= grid_cols) col -= grid_cols;
    const int t = col - col_lo;
#pragma unroll
    for (int u = 0; u < kChunk; ++u) {
      if (u == t) {
        r[u].x = fmaf(v.x, wt[j], r[u].x);
        r[u].y = fmaf(v.y, wt[j], r[u].y);
      }
    }
  }
}

// Lists longer than kSegMin entries are gridded in segments (at most
// kSegMax, all but the last of segment_length entries) that different warps
// take at once, so that a row's long lists do not hold its CTA at the
// barrier after the gridding while one warp works through each; a cell is then
// the sum, in segment order, of its segments' partial sums, each partial sum
// in sample order from zero.  Shorter lists are one segment: the cell is its
// samples' sum in sample order.  Every row kernel uses the same segments.
constexpr int kSegMin = 32;
constexpr int kSegMax = 32;

__host__ __device__ inline int list_segments(int n) {
  return n <= kSegMin ? 1 : ((n + kSegMin - 1) / kSegMin < kSegMax ? (n + kSegMin - 1) / kSegMin : kSegMax);
}
static_assert(kSegMin * kSegMax <= (1 << 22), "segment counts are taken from lengths capped at 2^22");
// First entry (absolute, within the frame's entries) of segment seg of a
// list starting at `begin` with segments of sl entries.
__host__ __device__ inline int seg_start(uint32_t begin, int seg, int sl) { return static_cast<int>(begin) + seg * sl; }

__host__ __device__ inline int segment_length(int n) {
  if (n <= kSegMin) return n;  // one segment (most lists): no division
  const int sg = list_segments(n);
  return (n + sg - 1) / sg;
}

// One column chunk's list entries (or one segment of them) gridded by a
// warp, lane = coil: the chunk's 16 cells stay in registers, summed in entry
// order from zero.  kWrap admits entries whose taps wrap around the grid
// inside the chunk.  `meta` is the warp's staging buffer.
//
// have_sk: lane i's sk_first already holds the sample index of entry i (of
// the first batch), loaded ahead by the caller; the first samples are then
// requested before the batch's entries are staged, so the two loads overlap
// instead of following each other.  Within the task, each batch loads the
// next batch's sample indices the same way (one 4-byte load per lane, which
// also brings the next batch's entries towards L1).
template <int W, uint32_t kFormat, bool kWrap, int kAR>
__device__ __forceinline__ void grid_entries_regs(float2 (&r)[kChunk], const RowsArgs& a, size_t sample_base,
                                                  bool coil_ok, int lane, int col_lo, const float4* xent, int n,
                                                  float4* meta, bool have_sk = false, uint32_t sk_first = 0u) {
  constexpr int kMV = meta_vecs(W);
  constexpr int kBatch = meta_batch(W);
  const SampleRows<kFormat> sample_row(a.samples_t, sample_base, a.channels);
#pragma unroll
  for (int t = 0; t < kChunk; ++t) r[t] = make_float2(0.0f, 0.0f);
  uint32_t sk_batch = sk_first;
  bool sk_ready = have_sk;
  for (int base = 0; base < n; base += kBatch) {
    const int cnt = min(kBatch, n - base);
    float2 yv[kAR];
    const bool pre = sk_ready;
    if (pre) {
#pragma unroll
      for (int k = 0; k < kAR; ++k) {
        const uint32_t sk = __shfl_sync(0xffffffffu, sk_batch, k);
        yv[k] = (coil_ok && k < cnt) ? sample_row(sk) : make_float2(0.0f, 0.0f);
      }
    }
    if (have_sk && base + kBatch < n) {
      const int nb = base + kBatch;
      sk_batch = lane < min(kBatch, n - nb) ? __float_as_uint(__ldg(&xent[static_cast<size_t>(nb + lane) * kMV].y)) : 0u;
      sk_ready = true;
    }
    __syncwarp();  // the previous batch is read by every lane before it is replaced
    if (lane < cnt) {
      const float4* src = xent + static_cast<size_t>(base + lane) * kMV;
      float4* m = meta + lane * kMV;
#pragma unroll
      for (int v = 0; v < kMV; ++v) m[v] = __ldg(src + v);
    }
    __syncwarp();
    auto fetch = [&](int i) { return sample_row(__float_as_uint(meta[i * kMV].y)); };
    if (!pre) {
#pragma unroll
      for (int k = 0; k < kAR; ++k) yv[k] = (coil_ok && k < cnt) ? fetch(k) : make_float2(0.0f, 0.0f);
    }
    for (int i0 = 0; i0 < cnt; i0 += kAR) {
#pragma unroll
      for (int k = 0; k < kAR; ++k) {
        const int i = i0 + k;
        if (i >= cnt) break;
        const float2 y = yv[k];
        yv[k] = (coil_ok && i + kAR < cnt) ? fetch(i + kAR) : make_float2(0.0f, 0.0f);
        const float4 m0 = meta[i * kMV];
        float wt[4 * (kMV - 1)];
#pragma unroll
        for (int v = 1; v < kMV; ++v) {
          const float4 mv = meta[i * kMV + v];
          wt[4 * (v - 1)] = mv.x;
          wt[4 * (v - 1) + 1] = mv.y;
          wt[4 * (v - 1) + 2] = mv.z;
          wt[4 * (v - 1) + 3] = mv.w;
        }
        const int word0 = __float_as_int(m0.x);
        const int cbase = word0 >> 9;  // arithmetic shift: may be negative
        const float2 v = cmul(y, make_float2(m0.z, m0.w));
        if (kWrap && (word0 & 256))
          chunk_taps_wrapped<W>(r, cbase, static_cast<uint32_t>(word0) & 255u, col_lo, a.grid_cols, v, wt);
        else
          chunk_taps<W>(r, cbase - col_lo, v, wt);
      }
    }
  }
}

// The chunk's cells from registers into the accumulator (dst: the chunk's
// first cell of this lane's coil, cells `stride` apart).  A one-segment list
// (counter null) stores them.  For a segmented list each lane works on its
// own coil's cells alone: segment 0 stores, segment seg > 0 waits until the
// list's counter shows all 32 lanes of segments 0 .. seg-1 in, then adds its
// partial sums; every lane then counts itself in.  Lanes wait on the counter
// each for itself (no warp-wide sync), fenced on both sides.  The wait is
// bounded: on a timeout the lane's partial sums are dropped, it still counts
// itself in (the later segments do not wait out the limit as well) and
// KSJ_GPU_FLAG_WAIT_TIMEOUT is raised.
__device__ __forceinline__ void put_chunk(const float2 (&r)[kChunk], float2* dst, int stride, int width, bool live,
                                          int seg, int* counter, uint32_t* flags, uint32_t wait_limit,
                                          int wait_beyond) {
  if (counter == nullptr) {
    if (live) {
      if (width == kChunk) {  // every chunk of the row but a partial last one
#pragma unroll
        for (int t = 0; t < kChunk; ++t) dst[t * stride] = r[t];
      } else {
#pragma unroll
        for (int t = 0; t < kChunk; ++t)
          if (t < width) dst[t * stride] = r[t];
      }
    }
    return;
  }
  // segmented list: every lane of segments 0 .. seg-1 has counted itself in
  bool ok = true;
  if (seg > 0) {
    uint32_t polls = 0;
    while (*reinterpret_cast<volatile int*>(counter) < 32 * seg + wait_beyond) {
      if (++polls >= wait_limit) {
        ok = false;
        atomicOr(flags, KSJ_GPU_FLAG_WAIT_TIMEOUT);
        break;
      }
      __nanosleep(32);
    }
    __threadfence_block();
  }
  if (live && ok) {
#pragma unroll
    for (int t = 0; t < kChunk; ++t) {
      if (t < width) {
        float2 v = r[t];
        if (seg > 0) {
          const float2 c = dst[t * stride];
          v = make_float2(c.x + v.x, c.y + v.y);
        }
        dst[t * stride] = v;
      }
    }
  }
  __threadfence_block();
  atomicAdd(counter, 1);
}

// The row's task table, built by warp 0: rank r is the r-th longest list
// (chunk[r]), cut into list_segments(len) segments of segment_length(len)
// entries; tasks base[r] .. base[r + 1] - 1 are its segments (times the coil
// parts).
struct RowTasks {
  int* chunk;
  int* base;      // nchunks + 1 entries
  int* combined;  // per (chunk, part): lanes of finished segments
  int* next;
};

// (rank, segment) of task q (parts folded out by the caller); a row without
// segmented lists has task q = rank q.
__device__ __forceinline__ void task_of(const RowTasks& t, int nchunks, int q, int lane, int* rank, int* seg) {
  if (t.base[nchunks] == nchunks) {
    *rank = q;
    *seg = 0;
    return;
  }
  const unsigned m = __ballot_sync(0xffffffffu, lane < nchunks && t.base[lane] <= q);
  *rank = __popc(m) - 1;
  *seg = q - t.base[*rank];
}

// Gridding of one row by whole 32-coil warps (lane = coil): warps take the
// row's tasks (list segments, longest lists first) from the shared counter.
// Every chunk is at least one task, so every cell of the row is stored.
template <int W, uint32_t kFormat, bool kWrap, int kAR>
__device__ __forceinline__ void rows_grid_regs(const RowsArgs& a, int f, int cgi, int lane, float2* acc,
                                               const uint32_t* offs, const RowTasks& tasks, float4* meta) {
  constexpr int kMV = meta_vecs(W);
  const int coil_global = cgi * 32 + lane;
  const bool coil_ok = coil_global < a.channels;
  const size_t sample_base = static_cast<size_t>(f) * a.sample_frame_stride + (coil_ok ? coil_global : 0);
  const int ntasks = tasks.base[a.nchunks];
  constexpr int kBatch = meta_batch(W);
  // A warp claims one task at a time and loads its first sample indices
  // before it grids it.  Tasks are claimed in increasing order, so the
  // smallest unfinished task is always some warp's current one: a segment's
  // wait for its predecessors always ends.  (Claiming the next task ahead,
  // to hide that load behind the current task, measured slower: 1.34 vs 1.28
  // ms on 96 radial frames, a claimed-ahead task waits behind its owner's
  // current one while other warps idle.)
  auto claim = [&]() {
    int q = 0;
    if (lane == 0) q = atomicAdd(tasks.next, 1);
    return __shfl_sync(0xffffffffu, q, 0);
  };
  struct Task {
    int chunk, seg, n, e0, e1;
  };
  auto decode = [&](int q) {
    Task t;
    int rank;
    task_of(tasks, a.nchunks, q, lane, &rank, &t.seg);
    t.chunk = tasks.chunk[rank];
    const uint32_t begin = offs[t.chunk];
    t.n = static_cast<int>(offs[t.chunk + 1] - begin);
    const int sl = segment_length(t.n);
    t.e0 = seg_start(begin, t.seg, sl);
    t.e1 = min(static_cast<int>(begin) + t.n, t.e0 + sl);
    return t;
  };
  auto entries_of = [&](const Task& t) {
    return a.expanded + (static_cast<size_t>(f) * a.entries_per_frame + static_cast<size_t>(t.e0)) * meta_vecs(W);
  };
  auto first_sk = [&](const Task& t) {
    return lane < min(kBatch, t.e1 - t.e0) ? __float_as_uint(__ldg(&entries_of(t)[static_cast<size_t>(lane) * kMV].y))
                                           : 0u;
  };
  for (;;) {
    const int q = claim();
    if (q >= ntasks) break;
    const Task cur = decode(q);
    float2 r[kChunk];
    grid_entries_regs<W, kFormat, kWrap, kAR>(r, a, sample_base, coil_ok, lane, cur.chunk * kChunk, entries_of(cur),
                                              cur.e1 - cur.e0, meta, true, first_sk(cur));
    put_chunk(r, acc + static_cast<size_t>(cur.chunk * kChunk) * 32 + lane, 32,
              min(kChunk, a.grid_cols - cur.chunk * kChunk), true, cur.seg,
              list_segments(cur.n) > 1 ? tasks.combined + cur.chunk : nullptr, a.flags, a.wait_limit, a.wait_beyond);
  }
}

// kBlocks CTAs per SM: 2 for rows of up to 384 columns (384 threads), 1
// above; two resident CTAs let one block's FFT overlap another's gridding.
// kCG = 32 fixes a 32-coil group taken whole by one warp (coil_parts 1):
// lane = coil, no tap groups, every tap offset a constant; kCG = 0 reads the
// group and the split from the arguments.
// kHalf: the sigma = 2 crop form of the row transform (out_cols =
// grid_cols / 2, col_shift = out_cols / 2), whose kept columns are known at
// compile time (fft_two_step_half); the same bytes as the general form.
template <int W, uint32_t kFormat, int kThreads, int kBlocks, int kCG, bool kHalf = false>
__global__ void __launch_bounds__(kThreads, kBlocks) k_rows(RowsArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int row = blockIdx.x;
  const int cgi = blockIdx.y;
  const int f = a.frame0 + blockIdx.z;
  const int cg = kCG ? kCG : a.coil_group;
  const int tid = threadIdx.x;
  const int nthreads = blockDim.x;
  const int lane = tid & 31;
  float2* acc = reinterpret_cast<float2*>(smem_raw);
  float2* tw = acc + static_cast<size_t>(a.grid_cols) * cg;
  uint32_t* offs = reinterpret_cast<uint32_t*>(tw + a.grid_cols);  // this row's list offsets
  constexpr int kMV = meta_vecs(W);
  constexpr int kBatch = meta_batch(W);
  const int warp = tid >> 5;
  // offsets from the shared array itself keep every access a shared-memory one
  const size_t meta_off = (static_cast<size_t>(a.grid_cols) * (cg + 1) * sizeof(float2) +
                           static_cast<size_t>(a.nchunks + 1) * sizeof(uint32_t) + 15) & ~static_cast<size_t>(15);
  float4* meta = reinterpret_cast<float4*>(smem_raw + meta_off) + warp * kBatch * kMV;
  const AccAddr addr{cg};

  const uint32_t* off = a.offsets + static_cast<size_t>(f) * (a.lists_per_frame + 1) + row * a.nchunks;
  for (int i = tid; i <= a.nchunks; i += nthreads) offs[i] = __ldg(off + i);
  // task order: the row's lists longest first (a bitonic sort across warp 0,
  // one key per lane: length << 8 | chunk), each cut into its segments, taken
  // from a shared counter
  __shared__ int task_chunk[kMaxGrid / kChunk];
  __shared__ int task_base[kMaxGrid / kChunk + 1];
  __shared__ int task_combined[2 * (kMaxGrid / kChunk)];
  __shared__ int task_next;
  if (warp == 0) {
    int key = -1;
    if (lane < a.nchunks) {
      const uint32_t len = min(__ldg(off + lane + 1) - __ldg(off + lane), 1u << 22);
      key = static_cast<int>(len << 8) | lane;
    }
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
      for (int j = k >> 1; j > 0; j >>= 1) {
        const int other = __shfl_xor_sync(0xffffffffu, key, j);
        const bool lower = (lane & j) == 0;
        const bool desc = (lane & k) == 0;
        key = (lower == desc) ? max(key, other) : min(key, other);
      }
    }
    // segments per rank and their exclusive prefix (from the key's length,
    // capped at 2^22 entries: the same count, since kSegMin * kSegMax entries
    // already take the most segments)
    const int len = lane < a.nchunks ? (key >> 8) : 0;
    const int nseg = lane < a.nchunks ? list_segments(len) : 0;
    int incl = nseg;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += v;
    }
    if (lane < a.nchunks) {
      task_chunk[lane] = key & 255;
      task_base[lane] = incl - nseg;
    }
    if (lane == a.nchunks - 1) task_base[a.nchunks] = incl;
    if (lane == 0) task_next = 0;
  }
  for (int i = tid; i < 2 * (kMaxGrid / kChunk); i += nthreads) task_combined[i] = 0;
  const RowTasks tasks{task_chunk, task_base, task_combined, &task_next};
  // (the 32-coil path stores every cell of the row from registers)
  if (kCG != 32)
    for (int i = tid; i < a.grid_cols * cg; i += nthreads) acc[i] = make_float2(0.0f, 0.0f);
  for (int i = tid; i < a.grid_cols; i += nthreads) tw[i] = a.tw_cols[i];
  __syncthreads();

  if constexpr (kCG == 32) {
    constexpr int kAR = kAheadRegs;  // a deeper prefetch measured slower in both instances (code size)
    // taps wrap around the grid inside one chunk only on grids narrower than
    // kChunk + W - 1 columns; the loop for those keeps a per-tap form
    if (a.grid_cols < kChunk + W - 1)
      rows_grid_regs<W, kFormat, true, kAR>(a, f, cgi, lane, acc, offs, tasks, meta);
    else
      rows_grid_regs<W, kFormat, false, kAR>(a, f, cgi, lane, acc, offs, tasks, meta);
  } else {
  // ---- gridding.  A task is (column chunk, coil part): the chunk's sorted
  // list applied to a subset of the coil group.  Cells of different coils are
  // independent, so parts of one list may run on different warps with every
  // cell still summed in sample order.  Warps take tasks round-robin.
  //
  // Per batch of list entries, lane i loads entry i's sample index and record
  // (vector loads), folds the row weight into the W column weights and stages
  // them in the warp's shared batch; then the warp walks the batch in order
  // with the coil loads of the next kAhead samples always in flight.
  // A list longer than kSegMin entries is gridded in segments like the
  // 32-coil path's (lane = coil of the part, cells in registers, segments
  // combined in order), so that every coil grouping gives the same cells.
  const int parts = kCG ? 1 : a.coil_parts;
  const int cpart = cg / parts;
  const int ntasks = tasks.base[a.nchunks] * parts;
  {
    // lanes: coil = lane % cpp, tap group = lane / cpp
    int cpp = 1;
    while (cpp < cpart) cpp <<= 1;
    const int ngroups = 32 / cpp;
    // taps j this lane applies: j mod ngroups equal to its tap group
    uint32_t my_taps = 0;
#pragma unroll
    for (int j = 0; j < W; ++j)
      if ((j & (ngroups - 1)) == lane / cpp) my_taps |= 1u << j;
    const void* ks = a.samples_t;
    for (;;) {
      int task = 0;
      if (lane == 0) task = atomicAdd(&task_next, 1);
      task = __shfl_sync(0xffffffffu, task, 0);
      if (task >= ntasks) break;
      const int q = task / parts;
      const int part = task - q * parts;
      int rank, seg;
      task_of(tasks, a.nchunks, q, lane, &rank, &seg);
      const int chunk = task_chunk[rank];
      const uint32_t begin = offs[chunk];
      const int n = static_cast<int>(offs[chunk + 1] - begin);
      const float4* xent = a.expanded + (static_cast<size_t>(f) * a.entries_per_frame + begin) * kMV;
      const int col_lo = chunk * kChunk;
      if (list_segments(n) > 1) {
        const int sl = segment_length(n);
        const int e0 = seg * sl, e1 = min(n, e0 + sl);
        const bool lane_coil = lane < cpart;
        const int rc = part * cpart + (lane_coil ? lane : 0);
        const int rg = cgi * cg + rc;
        const bool rok = lane_coil && rg < a.channels;
        const size_t rbase = static_cast<size_t>(f) * a.sample_frame_stride + (rok ? rg : 0);
        float2 r[kChunk];
        grid_entries_regs<W, kFormat, true, kAheadRegs>(r, a, rbase, rok, lane, col_lo,
                                                        xent + static_cast<size_t>(e0) * kMV, e1 - e0, meta);
        put_chunk(r, acc + addr(rc, col_lo), cg, min(kChunk, a.grid_cols - col_lo), lane_coil, seg,
                  tasks.combined + part * a.nchunks + chunk, a.flags, a.wait_limit, a.wait_beyond);
        continue;
      }
      const int col_hi = min(col_lo + kChunk, a.grid_cols);
      const int my_coil = part * cpart + lane % cpp;  // coil index within the group
      const int coil_global = cgi * cg + my_coil;
      const bool coil_ok = (lane % cpp) < cpart && coil_global < a.channels;
      const size_t sample_base = static_cast<size_t>(f) * a.sample_frame_stride + (coil_ok ? coil_global : 0);
      for (int base = 0; base < n; base += kBatch) {
        const int cnt = min(kBatch, n - base);
        __syncwarp();  // the previous batch is read by every lane before it is replaced
        if (lane < cnt) {
          const float4* src = xent + static_cast<size_t>(base + lane) * kMV;
          float4* m = meta + lane * kMV;
#pragma unroll
          for (int v = 0; v < kMV; ++v) m[v] = __ldg(src + v);
        }
        __syncwarp();
        auto fetch = [&](int i) {
          const uint32_t sk = __float_as_uint(meta[i * kMV].y);
          return load_sample<kFormat>(ks, sample_base + static_cast<size_t>(sk) * a.channels);
        };
        float2 yv[kAhead];
#pragma unroll
        for (int k = 0; k < kAhead; ++k) yv[k] = (coil_ok && k < cnt) ? fetch(k) : make_float2(0.0f, 0.0f);
        for (int i0 = 0; i0 < cnt; i0 += kAhead) {
#pragma unroll
          for (int k = 0; k < kAhead; ++k) {
            const int i = i0 + k;
            if (i >= cnt) break;
            const float2 y = yv[k];
            yv[k] = (coil_ok && i + kAhead < cnt) ? fetch(i + kAhead) : make_float2(0.0f, 0.0f);
            const float4 m0 = meta[i * kMV];
            float wt[4 * (kMV - 1)];
#pragma unroll
            for (int v = 1; v < kMV; ++v) {
              const float4 mv = meta[i * kMV + v];
              wt[4 * (v - 1)] = mv.x;
              wt[4 * (v - 1) + 1] = mv.y;
              wt[4 * (v - 1) + 2] = mv.z;
              wt[4 * (v - 1) + 3] = mv.w;
            }
            const int word0 = __float_as_int(m0.x);
            const int cbase = word0 >> 9;  // arithmetic shift: may be negative
            const uint32_t mask = static_cast<uint32_t>(word0) & my_taps;
            if (coil_ok) {
              const float2 v = cmul(y, make_float2(m0.z, m0.w));
              if (!(word0 & 256)) {
                // taps j of the mask are the consecutive cells cbase + j
                const int base = addr(my_coil, cbase);
#pragma unroll
                for (int j = 0; j < W; ++j) {
                  if (!((mask >> j) & 1u)) continue;
                  float2* cell = acc + (base + j * cg);
                  float2 c = *cell;
                  c.x = fmaf(v.x, wt[j], c.x);
                  c.y = fmaf(v.y, wt[j], c.y);
                  *cell = c;
                }
              } else {
#pragma unroll
                for (int j = 0; j < W; ++j) {
                  if (!((mask >> j) & 1u)) continue;
                  int col = cbase + j;
                  if (col >= a.grid_cols) col -= a.grid_cols;
                  float2* cell = acc + addr(my_coil, col);
                  float2 c = *cell;
                  c.x = fmaf(v.x, wt[j], c.x);
                  c.y = fmaf(v.y, wt[j], c.y);
                  *cell = c;
                }
              }
            }
            // tap groups of one lane set may meet in a cell across samples
            if (ngroups > 1) __syncwarp();
          }
        }
      }
    }
  }
  }
  __syncthreads();

  // ---- row inverse FFT of every coil line; the kept columns are written
  // coil-last: [frame][grid_row][out_col][channel]
  const int lg_cg = ilog2(cg);
  float2* dst_row = a.inter + (static_cast<size_t>(f) * a.grid_rows + row) * a.out_cols * a.cpitch + cgi * cg;
  const int live_lines = min(cg, a.channels - cgi * cg);
  auto emit = [&](int k, int line, float2 v) {
    int pc = k + a.col_shift;
    if (pc >= a.grid_cols) pc -= a.grid_cols;
    if (pc < a.out_cols && line < live_lines) dst_row[static_cast<size_t>(pc) * a.cpitch + line] = v;
  };
  if constexpr (kHalf) {
    auto live = [&](int line) { return line < live_lines; };
    auto emit_half = [&](int pc, int, int line, float2 v) { dst_row[static_cast<size_t>(pc) * a.cpitch + line] = v; };
    switch (a.grid_cols) {
      case 128: fft_two_step_half<16, 8>(acc, lg_cg, tw, tid, nthreads, live, emit_half); return;
      case 192: fft_two_step_half<16, 12>(acc, lg_cg, tw, tid, nthreads, live, emit_half); return;
      case 256: fft_two_step_half<16, 16>(acc, lg_cg, tw, tid, nthreads, live, emit_half); return;
      case 384: fft_two_step_half<16, 24>(acc, lg_cg, tw, tid, nthreads, live, emit_half); return;
      default:
        if constexpr (kThreads >= 512) {
          fft_two_step_half<16, 32>(acc, lg_cg, tw, tid, nthreads, live, emit_half);
          return;
        }
        break;
    }
  }
  // (blocks of kThreads threads take rows of up to kThreads columns)
  if (fft_two_step_rows<kThreads>(a.grid_cols, acc, lg_cg, tw, tid, nthreads, emit)) return;

  // other lengths: in place (output digit-reversed), then the kept columns
  dif_lines(acc, lg_cg, a.plan, tw, tid, nthreads);
  const int coil = tid & (cg - 1);
  if (coil < live_lines) {
    for (int pc = tid >> lg_cg; pc < a.out_cols; pc += nthreads >> lg_cg)
      dst_row[static_cast<size_t>(pc) * a.cpitch + coil] = acc[(__ldg(a.pos_cols + pc) << lg_cg) + coil];
  }
}

struct ColsArgs {
  const float2* tw_rows;
  const float* inv_dr;
  const float* inv_dc;
  const int* pos_rows;  // DIF output position of each kept row
  void* out;
  uint32_t* flags;
  int frame0;  // first frame of this pass
  int frames, channels, grid_rows, out_rows, out_cols, kb;
  int column_block, col_group, groups;  // tile: column_block columns x col_group coils; groups tiles per block
  int box_rows, boxes;                  // TMA boxes of box_rows rows cover one tile
  uint32_t output;                      // RSS or COIL_LAST (COIL_MAJOR goes through COIL_LAST + transpose)
  int out_pitch;                        // COIL_LAST: elements between pixels of the output (>= channels)
  int row_shift;                        // kept row of frequency k: (k + row_shift) mod grid_rows, when below out_rows
  DifPlan plan;
  // persistent form (k_cols_ring): tiles of tile_coils coils x (kRingLines /
  // tile_coils) columns; a unit is (frame, column block), tiles_per_unit
  // tiles of consecutive coils each; units = frames of the pass x col_blocks
  int tile_coils, tiles_per_unit, units, col_blocks;
};


// One CTA per (frame, column block).  The row-transformed grid
// [frame][grid_row][out_col][channel] is read one tile (grid_rows x
// column_block columns x col_group coils, coils contiguous) at a time by
// TMA; with more than one coil group the next tile's copy is in flight while
// the block transforms the current one.  Each tile is inverse-transformed
// along rows in place (lines = (column, coil) pairs), cropped and
// deapodised; then either written coil-last or squared in place and summed
// over coils in channel order per pixel.  The channel-order sum runs lane =
// pixel with lane j reading coil t - j at step t, so the 32 lanes read 32
// different coils (distinct banks) while each pixel still adds its coils
// 0, 1, 2, ... in order: the result is bit-identical to the RSS of the coil
// images.
//
// kN is the column length for the two-step transform (128 .. 512, see
// has_two_step_rows), or 0 for the in-place mixed-radix form of any other
// length; one instance per length keeps each kernel's code small.
// kLgL (when nonzero) fixes log2 of the line count (column_block x
// col_group) at compile time; kHalf selects the sigma = 2 crop form of the
// two-step transform (out_rows = grid_rows / 2, row_shift = out_rows / 2,
// Kaiser-Bessel deapodisation), whose kept rows are known at compile time.
// Every form gives the same bytes.
template <int kN, int kLgL = 0, bool kHalf = false>
__global__ void __launch_bounds__(kColsThreads) k_cols(const __grid_constant__ CUtensorMap inter_map, ColsArgs a) {
  extern __shared__ __align__(16) unsigned char smem_cols[];
  unsigned char* smem_raw = smem_cols;
  const int cb = a.column_block;
  const int cgc = a.col_group;
  const int lines = kLgL ? (1 << kLgL) : cb * cgc;
  const int lg_lines = kLgL ? kLgL : ilog2(lines);
  const int lg_cgc = ilog2(cgc);
  const int lg_cb = ilog2(cb);
  const int col0 = blockIdx.x * cb;
  const int fg = a.frame0 + blockIdx.y;
  const int tid = threadIdx.x;
  const int nthreads = blockDim.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const int nbuf = a.groups > 1 ? 2 : 1;
  // each tile buffer starts on a 128-byte boundary (TMA destination)
  const size_t tile_elems = (static_cast<size_t>(a.grid_rows) * lines + 15) & ~static_cast<size_t>(15);
  float2* tiles = reinterpret_cast<float2*>(smem_raw + ((128u - (smem_addr(smem_raw) & 127u)) & 127u));
  float2* tw = tiles + nbuf * tile_elems;
  float* rss = reinterpret_cast<float*>(tw + a.grid_rows);
  const int npix = a.out_rows * cb;
  uint64_t* bars = reinterpret_cast<uint64_t*>(rss + ((npix + 1) & ~1));
  float* inv_dr = reinterpret_cast<float*>(bars + 2);  // row deapodisation, out_rows values
  const uint32_t tile_bytes = static_cast<uint32_t>(static_cast<size_t>(a.grid_rows) * lines * sizeof(float2));
  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init_fence();
  }
  for (int i = tid; i < a.grid_rows; i += nthreads) tw[i] = a.tw_rows[i];
  for (int i = tid; i < npix; i += nthreads) rss[i] = 0.0f;
  if (a.kb)
    for (int i = tid; i < a.out_rows; i += nthreads) inv_dr[i] = __ldg(a.inv_dr + i);
  __syncthreads();
  auto issue = [&](int g, int b) {
    float2* dst = tiles + b * tile_elems;
    mbar_arrive_expect_tx(&bars[b], tile_bytes);
    for (int k = 0; k < a.boxes; ++k)
      tma_load_3d(dst + static_cast<size_t>(k) * a.box_rows * lines, &inter_map, g * cgc, col0,
                  fg * a.grid_rows + k * a.box_rows, &bars[b]);
  };
  if (tid == 0) issue(0, 0);
  const int line = tid & (lines - 1);
  const int lcol = line >> lg_cgc;   // column within the block
  const int lcoil = line & (cgc - 1);
  const bool col_ok = col0 + lcol < a.out_cols;
  bool ok = true;
  int issued = 1;
  for (int g = 0; g < a.groups; ++g) {
    const int b = nbuf > 1 ? (g & 1) : 0;
    const uint32_t parity = static_cast<uint32_t>((nbuf > 1 ? (g >> 1) : g) & 1);
    if (tid == 0 && g + 1 < a.groups) {
      fence_proxy_async_shared();  // this buffer was last written by the generic proxy
      issue(g + 1, b ^ 1);
      ++issued;
    }
    const bool mine = mbar_wait_bounded(&bars[b], parity, kWaitLimit);
    if (!__syncthreads_and(mine)) {
      ok = false;
      break;
    }
    float2* tile = tiles + b * tile_elems;
    // crop and deapodise; coil-last images are written from here, RSS
    // inputs are squared in place at pos_rows[pr]
    auto emit_pixel = [&](int pr, int ln, float2* e, float2 x) {
      const int lc = ln >> lg_cgc;
      if (a.kb) {
        const float sc = inv_dr[pr] * __ldg(a.inv_dc + col0 + lc);
        x.x *= sc;
        x.y *= sc;
      }
      if (a.output == KSJ_GPU_OUTPUT_RSS) {
        e->x = __fadd_rn(__fmul_rn(x.x, x.x), __fmul_rn(x.y, x.y));
      } else {
        float2* o = static_cast<float2*>(a.out);
        o[((static_cast<size_t>(fg) * a.out_rows + pr) * a.out_cols + col0 + lc) * a.out_pitch + g * cgc +
          (ln & (cgc - 1))] = x;
      }
    };
    const int live_coils_g = min(cgc, a.channels - g * cgc);
    auto emit = [&](int k, int ln, float2 v) {
      int pr = k + a.row_shift;
      if (pr >= a.grid_rows) pr -= a.grid_rows;
      if (pr >= a.out_rows || col0 + (ln >> lg_cgc) >= a.out_cols || (ln & (cgc - 1)) >= live_coils_g) return;
      emit_pixel(pr, ln, tile + (two_step_slot(k, a.grid_rows) << lg_lines) + ln, v);
    };
    if constexpr (kN != 0 && kHalf) {
      auto live = [&](int ln) { return col0 + (ln >> lg_cgc) < a.out_cols && (ln & (cgc - 1)) < live_coils_g; };
      auto emit_half = [&](int pr, int slot, int ln, float2 v) {
        const int lc = ln >> lg_cgc;
        const float sc = inv_dr[pr] * __ldg(a.inv_dc + col0 + lc);
        v.x *= sc;
        v.y *= sc;
        if (a.output == KSJ_GPU_OUTPUT_RSS) {
          tile[(slot << lg_lines) + ln].x = __fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y));
        } else {
          float2* o = static_cast<float2*>(a.out);
          o[((static_cast<size_t>(fg) * a.out_rows + pr) * a.out_cols + col0 + lc) * a.out_pitch + g * cgc +
            (ln & (cgc - 1))] = v;
        }
      };
      fft_two_step_half<16, kN / 16>(tile, lg_lines, tw, tid, nthreads, live, emit_half);
    } else if constexpr (kN != 0) {
      fft_two_step<16, kN / 16>(tile, lg_lines, tw, tid, nthreads, emit);
    } else {
      dif_lines(tile, lg_lines, a.plan, tw, tid, nthreads);
      if (col_ok && lcoil < live_coils_g) {
        for (int pr = tid >> lg_lines; pr < a.out_rows; pr += nthreads >> lg_lines) {
          float2* e = tile + (static_cast<size_t>(__ldg(a.pos_rows + pr)) << lg_lines) + line;
          emit_pixel(pr, line, e, *e);
        }
      }
    }
    if (a.output == KSJ_GPU_OUTPUT_RSS) {
      __syncthreads();
      // channel-order sum per pixel (reductions.hpp:972-982)
      const int live_coils = min(cgc, a.channels - g * cgc);
      for (int q0 = warp * 32; q0 < npix; q0 += nthreads) {
        const int q = q0 + lane;
        const bool live = q < npix && col0 + (q & (cb - 1)) < a.out_cols;
        const int pr = q >> lg_cb;
        const int base = live ? (__ldg(a.pos_rows + pr) << lg_lines) + ((q & (cb - 1)) << lg_cgc) : 0;
        float total = live ? rss[q] : 0.0f;
        if (live_coils == 32) {
          // fixed trip count: every load of the walk can be issued ahead of
          // the dependent adds
#pragma unroll
          for (int t = 0; t < 63; ++t) {
            const int c = t - lane;
            if (live && c >= 0 && c < 32) total = __fadd_rn(total, tile[base + c].x);
          }
        } else {
          for (int t = 0; t < live_coils + 31; ++t) {
            const int c = t - lane;
            if (live && c >= 0 && c < live_coils) total = __fadd_rn(total, tile[base + c].x);
          }
        }
        if (live) rss[q] = total;
      }
    }
    __syncthreads();
  }
  if (!ok) {
    // a copy never completed: report, then give every copy this block issued
    // a bounded chance to land before the block's shared memory is released
    if (tid == 0) {
      atomicOr(a.flags, KSJ_GPU_FLAG_WAIT_TIMEOUT);
      for (int u = 0; u < issued; ++u) {
        const int bb = nbuf > 1 ? (u & 1) : 0;
        const uint32_t par = static_cast<uint32_t>((nbuf > 1 ? (u >> 1) : u) & 1);
        mbar_wait_bounded(&bars[bb], par, kWaitLimit);
      }
    }
    return;
  }
  if (a.output == KSJ_GPU_OUTPUT_RSS) {
    float* o = static_cast<float*>(a.out);
    for (int q = tid; q < npix; q += nthreads) {
      const int pr = q >> lg_cb;
      const int l = q & (cb - 1);
      if (col0 + l < a.out_cols) o[(static_cast<size_t>(fg) * a.out_rows + pr) * a.out_cols + col0 + l] = __fsqrt_rn(rss[q]);
    }
  }
}

// Persistent column pass for the two-step column lengths.  Each CTA walks
// its share of the (frame, column block) units -- units blockIdx.x,
// blockIdx.x + gridDim.x, ... -- one tile of kRingLines lines (tile_coils
// coils x kRingLines / tile_coils columns, all grid rows) at a time, through
// a two-stage ring of shared-memory tiles: while the block transforms tile i,
// the TMA copy of tile i + 1 is in flight, and tile i + 2's copy is issued as
// soon as tile i's stage is free.  Per line the arithmetic is the one-shot
// k_cols's (the same transform, crop and deapodisation); the RSS sums a
// pixel's coils in channel order across the unit's tiles (the accumulator
// carries over from tile to tile), so the bytes equal k_cols's.
constexpr int kRingLines = 16;
constexpr int kRingLgLines = 4;

template <int kN>
struct RingCfg;  // block size (step A of the two-step transform has kN / 16 x 16 tasks) and CTAs per SM
template <>
struct RingCfg<128> { static constexpr int kThreads = 256, kBlocks = 2; };
template <>
struct RingCfg<192> { static constexpr int kThreads = 256, kBlocks = 2; };
template <>
struct RingCfg<256> { static constexpr int kThreads = 256, kBlocks = 2; };
template <>
struct RingCfg<384> { static constexpr int kThreads = 384, kBlocks = 2; };
template <>
struct RingCfg<512> { static constexpr int kThreads = 512, kBlocks = 1; };

template <int kN>
__global__ void __launch_bounds__(RingCfg<kN>::kThreads, RingCfg<kN>::kBlocks)
    k_cols_ring(const __grid_constant__ CUtensorMap inter_map, ColsArgs a) {
  constexpr int kT = RingCfg<kN>::kThreads;
  constexpr int kL = kRingLines;
  constexpr int kLgL = kRingLgLines;
  extern __shared__ __align__(16) unsigned char smem_cols[];
  unsigned char* smem_raw = smem_cols;
  const int tc = a.tile_coils;
  const int lg_tc = ilog2(tc);
  const int cb = kL / tc;  // columns per tile
  const int lg_cb = kLgL - lg_tc;
  const int tid = threadIdx.x;
  const int tpu = a.tiles_per_unit;
  constexpr size_t kTileElems = static_cast<size_t>(kN) * kL;
  float2* tiles = reinterpret_cast<float2*>(smem_raw + ((128u - (smem_addr(smem_raw) & 127u)) & 127u));
  float2* tw = tiles + 2 * kTileElems;
  float* rss = reinterpret_cast<float*>(tw + kN);
  const int npix = a.out_rows * cb;
  uint64_t* bars = reinterpret_cast<uint64_t*>(rss + ((npix + 1) & ~1));
  float* inv_dr = reinterpret_cast<float*>(bars + 2);
  constexpr uint32_t kTileBytes = static_cast<uint32_t>(kTileElems * sizeof(float2));
  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init_fence();
  }
  for (int i = tid; i < kN; i += kT) tw[i] = a.tw_rows[i];
  for (int i = tid; i < npix; i += kT) rss[i] = 0.0f;
  if (a.kb)
    for (int i = tid; i < a.out_rows; i += kT) inv_dr[i] = __ldg(a.inv_dr + i);
  __syncthreads();
  const int my_units = a.units > static_cast<int>(blockIdx.x)
                           ? (a.units - 1 - static_cast<int>(blockIdx.x)) / static_cast<int>(gridDim.x) + 1
                           : 0;
  const int ntiles = my_units * tpu;
  auto unit_of = [&](int i) { return static_cast<int>(blockIdx.x) + (i / tpu) * static_cast<int>(gridDim.x); };
  auto issue = [&](int i) {
    const int u = unit_of(i), h = i - (i / tpu) * tpu;
    const int f = a.frame0 + u / a.col_blocks;
    const int col0 = (u - (u / a.col_blocks) * a.col_blocks) * cb;
    float2* dst = tiles + (i & 1) * kTileElems;
    mbar_arrive_expect_tx(&bars[i & 1], kTileBytes);
    for (int k = 0; k < a.boxes; ++k)
      tma_load_3d(dst + static_cast<size_t>(k) * a.box_rows * kL, &inter_map, h * tc, col0,
                  f * kN + k * a.box_rows, &bars[i & 1]);
  };
  if (tid == 0)
    for (int i = 0; i < 2 && i < ntiles; ++i) issue(i);
  int i = 0;
  bool ok = true;
  for (; i < ntiles; ++i) {
    const int b = i & 1;
    const bool mine = mbar_wait_bounded(&bars[b], static_cast<uint32_t>((i >> 1) & 1), kWaitLimit);
    if (!__syncthreads_and(mine)) {
      ok = false;
      break;
    }
    const int u = unit_of(i), h = i - (i / tpu) * tpu;
    const int fg = a.frame0 + u / a.col_blocks;
    const int col0 = (u - (u / a.col_blocks) * a.col_blocks) * cb;
    const int coil0 = h * tc;
    const int live_coils = min(tc, a.channels - coil0);
    float2* tile = tiles + b * kTileElems;
    auto emit = [&](int k, int ln, float2 v) {
      int pr = k + a.row_shift;
      if (pr >= kN) pr -= kN;
      const int lc = ln >> lg_tc;
      if (pr >= a.out_rows || col0 + lc >= a.out_cols || (ln & (tc - 1)) >= live_coils) return;
      if (a.kb) {
        const float sc = inv_dr[pr] * __ldg(a.inv_dc + col0 + lc);
        v.x *= sc;
        v.y *= sc;
      }
      if (a.output == KSJ_GPU_OUTPUT_RSS) {
        float2* e = tile + (two_step_slot(k, kN) << kLgL) + ln;
        e->x = __fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y));
      } else {
        float2* o = static_cast<float2*>(a.out);
        o[((static_cast<size_t>(fg) * a.out_rows + pr) * a.out_cols + col0 + lc) * a.out_pitch + coil0 +
          (ln & (tc - 1))] = v;
      }
    };
    fft_two_step<16, kN / 16>(tile, kLgL, tw, tid, kT, emit);
    if (a.output == KSJ_GPU_OUTPUT_RSS) {
      __syncthreads();
      // channel-order sum per pixel (reductions.hpp:972-982), continued from
      // the unit's previous tiles; thread q owns pixel q in both loops below
      const int lane = tid & 31;
      for (int q0 = tid - lane; q0 < npix; q0 += kT) {
        const int q = q0 + lane;
        const bool live = q < npix && col0 + (q & (cb - 1)) < a.out_cols;
        const int pr = q >> lg_cb;
        const int base = live ? (__ldg(a.pos_rows + pr) << kLgL) + ((q & (cb - 1)) << lg_tc) : 0;
        float total = live ? rss[q] : 0.0f;
        for (int t = 0; t < live_coils + 31; ++t) {
          const int c = t - lane;
          if (live && c >= 0 && c < live_coils) total = __fadd_rn(total, tile[base + c].x);
        }
        if (live) rss[q] = total;
      }
      if (h == tpu - 1) {
        float* o = static_cast<float*>(a.out);
        for (int q = tid; q < npix; q += kT) {
          const int pr = q >> lg_cb;
          const int l = q & (cb - 1);
          if (col0 + l < a.out_cols) o[(static_cast<size_t>(fg) * a.out_rows + pr) * a.out_cols + col0 + l] =
              __fsqrt_rn(rss[q]);
          rss[q] = 0.0f;
        }
      }
    }
    __syncthreads();  // every thread is done with stage b
    if (tid == 0 && i + 2 < ntiles) {
      fence_proxy_async_shared();  // the stage was last written by the generic proxy
      issue(i + 2);
    }
  }
  if (!ok && tid == 0) {
    // a copy never completed: report, then give the copies still in flight
    // (tiles i and i + 1) a bounded chance to land before the block exits
    atomicOr(a.flags, KSJ_GPU_FLAG_WAIT_TIMEOUT);
    for (int t = i; t < i + 2 && t < ntiles; ++t)
      mbar_wait_bounded(&bars[t & 1], static_cast<uint32_t>((t >> 1) & 1), kWaitLimit);
  }
}

// ------------------------------------------------------------------ driver

// The row-pass kernel a shape selects (rows_blocks: k_rows with that many
// CTAs per SM), its launch setup and launch.
struct RowsLauncher {
  void (*kernel)(RowsArgs) = nullptr;
  int threads = 0;
  size_t smem = 0;

  template <int W, uint32_t kFormat>
  bool setup(const Shape& s) {
    smem = rows_smem_for(s.grid_cols, s.coil_group, s.width, rows_threads_for(s.grid_cols));
    threads = rows_threads_for(s.grid_cols);
    const bool whole32 = s.coil_group == 32 && s.coil_parts == 1;
    // the sigma = 2 crop form for the 32-coil register path
    const bool half = whole32 && s.kb && s.out_cols * 2 == s.grid_cols && has_two_step_rows(s.grid_cols);
    if (threads <= 384 && s.rows_blocks == 2)
      kernel = half ? k_rows<W, kFormat, 384, 2, 32, true>
                    : (whole32 ? k_rows<W, kFormat, 384, 2, 32> : k_rows<W, kFormat, 384, 2, 0>);
    else
      kernel = half ? k_rows<W, kFormat, kMaxThreads, 1, 32, true>
                    : (whole32 ? k_rows<W, kFormat, kMaxThreads, 1, 32> : k_rows<W, kFormat, kMaxThreads, 1, 0>);
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) ==
               cudaSuccess &&
           cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100) == cudaSuccess;
  }

  // One pass of nf frames of grid_rows rows and `groups` coil groups.
  void launch(const RowsArgs& r, int grid_rows, int groups, int nf, cudaStream_t stream) const {
    LaunchScope scope("k_rows", stream);
    kernel<<<dim3(grid_rows, groups, nf), threads, smem, stream>>>(r);
  }
};

size_t cols_smem_bytes(const Shape& s) {
  const size_t lines = static_cast<size_t>(s.column_block) * s.col_group;
  const size_t tile = (static_cast<size_t>(s.grid_rows) * lines + 15) & ~static_cast<size_t>(15);
  const int nbuf = s.cpitch / s.col_group > 1 ? 2 : 1;
  const size_t npix = static_cast<size_t>(s.out_rows) * s.column_block;
  return 128 + nbuf * tile * sizeof(float2) + s.grid_rows * sizeof(float2) + ((npix + 1) & ~size_t{1}) * sizeof(float) +
         2 * sizeof(uint64_t) + static_cast<size_t>(s.out_rows) * sizeof(float);
}

using ColsKernel = void (*)(const __grid_constant__ CUtensorMap, ColsArgs);

// The k_cols instance for columns of n grid rows; half: the sigma = 2 crop
// (out_rows = n / 2, row_shift = n / 4, Kaiser-Bessel), lines32: 32 lines per
// tile (the default column block).
template <int kN>
ColsKernel cols_kernel_two_step(bool half, bool lines32) {
  if (half) return lines32 ? k_cols<kN, 5, true> : k_cols<kN, 0, true>;
  return lines32 ? k_cols<kN, 5, false> : k_cols<kN, 0, false>;
}

ColsKernel cols_kernel_for(int n, bool half = false, bool lines32 = false) {
  switch (n) {
    case 128: return cols_kernel_two_step<128>(half, lines32);
    case 192: return cols_kernel_two_step<192>(half, lines32);
    case 256: return cols_kernel_two_step<256>(half, lines32);
    case 384: return cols_kernel_two_step<384>(half, lines32);
    case 512: return cols_kernel_two_step<512>(half, lines32);
    default: return k_cols<0>;
  }
}

// Opt a k_cols instance into its dynamic shared memory.
bool cols_kernel_setup(ColsKernel k, size_t smem) {
  return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) == cudaSuccess &&
         cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100) == cudaSuccess;
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

// Tensor map over the row-transformed grid [frame*grid_row][out_col][cpitch]
// of 8-byte elements, box (col_group coils, column_block columns, box_rows rows).
bool make_inter_map(const Shape& s, void* inter, CUtensorMap* map, int* box_rows, int* boxes) {
  EncodeTiledFn enc = encode_tiled();
  if (enc == nullptr) return false;
  int nb = 1;
  while (s.grid_rows / nb > 256 || s.grid_rows % nb != 0) ++nb;
  *boxes = nb;
  *box_rows = s.grid_rows / nb;
  const cuuint64_t dims[3] = {static_cast<cuuint64_t>(s.cpitch), static_cast<cuuint64_t>(s.out_cols),
                              static_cast<cuuint64_t>(s.frames) * s.grid_rows};
  const cuuint64_t strides[2] = {static_cast<cuuint64_t>(s.cpitch) * 8,
                                 static_cast<cuuint64_t>(s.cpitch) * s.out_cols * 8};
  const cuuint32_t box[3] = {static_cast<cuuint32_t>(s.col_group), static_cast<cuuint32_t>(s.column_block),
                             static_cast<cuuint32_t>(*box_rows)};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, inter, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor map for the persistent column pass: box (tile_coils coils,
// kRingLines / tile_coils columns, box_rows rows).
bool make_ring_map(const Shape& s, void* inter, int tile_coils, CUtensorMap* map, int* box_rows, int* boxes) {
  Shape t = s;
  t.col_group = tile_coils;
  t.column_block = kRingLines / tile_coils;
  return make_inter_map(t, inter, map, box_rows, boxes);
}

using RingKernel = void (*)(const __grid_constant__ CUtensorMap, ColsArgs);

// The column pass of one shape: the persistent ring kernel for the two-step
// column lengths, else one k_cols CTA per (frame, column block).  Both give
// the same bytes.
struct ColsPass {
  bool ring = false;
  ColsKernel kernel = nullptr;
  size_t smem = 0;
  int threads = kColsThreads;
  int ctas = 0;
  int column_block = 1;
  int out_cols = 0;
  CUtensorMap map;

  bool setup(const Shape& s, void* inter, ColsArgs* c) {
    const int tc = std::min(s.col_group, kRingLines);
    const int cb = kRingLines / tc;
    out_cols = s.out_cols;
    ring = s.column_pass == 2 && has_two_step_rows(s.grid_rows) && tc >= 2 && cb <= s.out_cols;
    if (!ring) {
      column_block = s.column_block;
      smem = cols_smem_bytes(s);
      const bool half = c->kb && s.out_rows * 2 == s.grid_rows && c->row_shift == s.out_rows / 2;
      kernel = cols_kernel_for(s.grid_rows, half, s.column_block * s.col_group == 32);
      return cols_kernel_setup(kernel, smem) && make_inter_map(s, inter, &map, &c->box_rows, &c->boxes);
    }
    column_block = cb;
    c->tile_coils = tc;
    c->tiles_per_unit = s.cpitch / tc;
    c->col_blocks = (s.out_cols + cb - 1) / cb;
    int blocks = 2;
    switch (s.grid_rows) {
      case 128: kernel = k_cols_ring<128>; threads = RingCfg<128>::kThreads; blocks = RingCfg<128>::kBlocks; break;
      case 192: kernel = k_cols_ring<192>; threads = RingCfg<192>::kThreads; blocks = RingCfg<192>::kBlocks; break;
      case 256: kernel = k_cols_ring<256>; threads = RingCfg<256>::kThreads; blocks = RingCfg<256>::kBlocks; break;
      case 384: kernel = k_cols_ring<384>; threads = RingCfg<384>::kThreads; blocks = RingCfg<384>::kBlocks; break;
      default: kernel = k_cols_ring<512>; threads = RingCfg<512>::kThreads; blocks = RingCfg<512>::kBlocks; break;
    }
    const size_t npix = static_cast<size_t>(s.out_rows) * cb;
    smem = 128 + 2 * static_cast<size_t>(s.grid_rows) * kRingLines * sizeof(float2) + s.grid_rows * sizeof(float2) +
           ((npix + 1) & ~size_t{1}) * sizeof(float) + 2 * sizeof(uint64_t) + static_cast<size_t>(s.out_rows) * sizeof(float);
    int device = 0, sms = 0;
    if (cudaGetDevice(&device) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0)
      return false;
    ctas = sms * blocks;
    return cols_kernel_setup(kernel, smem) && make_ring_map(s, inter, tc, &map, &c->box_rows, &c->boxes);
  }

  // The column pass over nf frames starting at c.frame0.
  void launch(ColsArgs c, int nf, cudaStream_t stream, const char* name) const {
    LaunchScope scope(name, stream);
    if (ring) {
      c.units = nf * c.col_blocks;
      kernel<<<std::min(ctas, c.units), threads, smem, stream>>>(map, c);
    } else {
      kernel<<<dim3((out_cols + column_block - 1) / column_block, nf), kColsThreads, smem, stream>>>(map, c);
    }
  }
};

// The binning lists of one call: per-sample records, list counts, offsets,
// the scattered entries and their sort (and, when `expanded` is given, the
// expanded entries the row pass reads).  `flags` must already be cleared.
template <int W>
ksj_gpu_status build_lists(const Shape& s, const ksj_gpu_gridding_desc* d, const float* d_traj, const float* d_dcf,
                           uint32_t* flags, unsigned char* records, uint32_t* counts, uint32_t* cursor,
                           uint32_t* offsets, uint32_t* entries, float4* expanded, uint32_t* long_lists,
                           cudaStream_t stream, uint32_t* frame_flags = nullptr) {
  const size_t nl = static_cast<size_t>(s.frames) * s.lists_per_frame;
  if (cudaMemsetAsync(counts, 0, nl * 4, stream) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  if (cudaMemsetAsync(cursor, 0, nl * 4, stream) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  const size_t fm = static_cast<size_t>(s.frames) * s.samples;
  {
    PrepareArgs p{};
    p.traj = d_traj;
    p.dcf = d_dcf;
    p.frame_samples = s.frame_samples;
    p.frame_traj = s.frame_traj;
    p.frame_flags = frame_flags;
    p.dcf_mode = d->dcf_mode;
    p.require_nyquist = d->require_nyquist;
    p.records = records;
    p.counts = counts;
    p.flags = flags;
    p.frames = s.frames;
    p.samples = s.samples;
    p.grid_rows = s.grid_rows;
    p.grid_cols = s.grid_cols;
    p.nchunks = s.nchunks;
    p.lists_per_frame = s.lists_per_frame;
    p.kb = s.kb ? 1 : 0;
    p.beta = s.beta;
    p.two_over_w = 2.0f / static_cast<float>(s.width);
    p.inv_i0_beta = s.inv_i0_beta;
    p.phase_row = s.phase_row;
    p.phase_col = s.phase_col;
    p.phase_sign = s.phase_sign;
    LaunchScope scope("k_prepare", stream);
    k_prepare<W><<<static_cast<unsigned>((fm + 255) / 256), 256, 0, stream>>>(p);
  }
  {
    LaunchScope scope("k_scan", stream);
    k_scan<<<s.frames, 1024, 0, stream>>>(counts, offsets, s.lists_per_frame);
  }
  {
    LaunchScope scope("k_scatter", stream);
    k_scatter<W><<<static_cast<unsigned>((fm + 255) / 256), 256, 0, stream>>>(
        records, offsets, cursor, entries, s.frames, s.samples, s.grid_rows, s.grid_cols, s.nchunks,
        s.entries_per_frame);
  }
  {
    SortArgs sa{};
    sa.offsets = offsets;
    sa.entries = entries;
    sa.records = records;
    sa.expanded = expanded;
    sa.long_count = long_lists;
    sa.long_lists = long_lists + 1;
    sa.frames = s.frames;
    sa.samples = s.samples;
    sa.lists_per_frame = s.lists_per_frame;
    sa.nchunks = s.nchunks;
    sa.grid_rows = s.grid_rows;
    sa.grid_cols = s.grid_cols;
    sa.capacity = s.list_capacity;
    sa.entries_per_frame = s.entries_per_frame;
    sa.dim3 = 0;
    const ksj_gpu_status st = launch_sort<W>(sa, nl, static_cast<size_t>(s.frames) * s.entries_per_frame,
                                             s.list_capacity, stream);
    if (st != KSJ_GPU_OK) return st;
  }
  return KSJ_GPU_OK;
}

// Streams and events of a multi-pass call.  Odd passes run on a second
// compute stream (`alt`, joined after the binning through `ready` and back
// through `alt_done`), so a pass's last, partly filled wave overlaps the
// next pass.  With host buffers (ksj_gpu_gridding_adjoint_host, `copy` set):
// pass p's samples reach device memory on the copy stream (event in[p]); the
// pass waits for them before its transpose, and its images go back to the
// host on the copy stream once the pass is done (event done[p]).
struct HostIo {
  cudaStream_t copy, alt;
  const cudaEvent_t* in;
  const cudaEvent_t* done;
  cudaEvent_t ready, alt_done;
  void* h_out;
  size_t out_frame_bytes;
};

template <int W, uint32_t kFormat>
ksj_gpu_status launch_all(const Shape& s, const Layout& l, const ksj_gpu_gridding_desc* d, const void* d_kspace,
                          const float* d_traj, const float* d_dcf, void* d_out, unsigned char* ws,
                          cudaStream_t stream, const HostIo* io = nullptr) {
  uint32_t* flags = reinterpret_cast<uint32_t*>(ws + l.flags);
  unsigned char* records = ws + l.records;
  uint32_t* counts = reinterpret_cast<uint32_t*>(ws + l.counts);
  uint32_t* cursor = reinterpret_cast<uint32_t*>(ws + l.cursor);
  uint32_t* offsets = reinterpret_cast<uint32_t*>(ws + l.offsets);
  uint32_t* entries = reinterpret_cast<uint32_t*>(ws + l.entries);
  float2* inter = reinterpret_cast<float2*>(ws + l.inter);
  float2* tw_rows = reinterpret_cast<float2*>(ws + l.tables);
  float2* tw_cols = tw_rows + s.grid_rows;
  float* inv_dr = reinterpret_cast<float*>(tw_cols + s.grid_cols);
  float* inv_dc = inv_dr + s.out_rows;
  int* pos_rows = reinterpret_cast<int*>(inv_dc + s.out_cols);
  int* pos_cols = pos_rows + s.out_rows;

  if (cudaMemsetAsync(flags, 0, kFlagBytes, stream) != cudaSuccess ||
      cudaMemsetAsync(ws + l.frame_flags, 0, static_cast<size_t>(s.frames) * 4, stream) != cudaSuccess)
    return KSJ_GPU_ERROR_CUDA;
  {
    const int n = std::max(std::max(s.grid_rows, s.grid_cols), std::max(s.out_rows, s.out_cols));
    const double beta = s.beta;
    LaunchScope scope("k_tables", stream);
    k_tables<<<(n + 255) / 256, 256, 0, stream>>>(tw_rows, s.grid_rows, tw_cols, s.grid_cols, inv_dr, s.out_rows,
                                                  inv_dc, s.out_cols, pos_rows, pos_cols, s.plan_rows, s.plan_cols,
                                                  s.kb ? 1 : 0, s.width, beta,
                                                  s.kb ? std::cyl_bessel_i(0.0, beta) : 1.0);
  }
  {
    const ksj_gpu_status st = build_lists<W>(s, d, d_traj, d_dcf, flags, records, counts, cursor, offsets, entries,
                                             reinterpret_cast<float4*>(ws + l.expanded),
                                             reinterpret_cast<uint32_t*>(ws + l.long_lists), stream,
                                             reinterpret_cast<uint32_t*>(ws + l.frame_flags));
    if (st != KSJ_GPU_OK) return st;
  }
  const size_t frame_samples = static_cast<size_t>(s.samples) * s.channels;  // elements per frame
  auto to_coil_last = [&](int f0, int nf, cudaStream_t st) {
    const size_t eb = sample_bytes(d->sample_format);
    const dim3 tg((s.samples + 31) / 32, (s.channels + 31) / 32, nf);
    LaunchScope scope("k_samples_coil_last", st);
    const unsigned char* in = s.frame_kspace ? nullptr : static_cast<const unsigned char*>(d_kspace) + f0 * frame_samples * eb;
    k_samples_coil_last<kFormat><<<tg, dim3(32, 8), 0, st>>>(
        in, ws + l.samples_t + f0 * frame_samples * eb,
        s.channels, s.samples, flags, s.frame_channels, s.frame_samples, s.frame_kspace, f0,
        reinterpret_cast<uint32_t*>(ws + l.frame_flags));
  };
  if (io == nullptr || io->copy == nullptr) to_coil_last(0, s.frames, stream);
  RowsArgs r{};
  r.samples_t = ws + l.samples_t;
  r.sample_frame_stride = static_cast<size_t>(s.samples) * s.channels;
  r.offsets = offsets;
  r.expanded = reinterpret_cast<const float4*>(ws + l.expanded);
  r.tw_cols = tw_cols;
  r.pos_cols = pos_cols;
  r.inter = inter;
  r.flags = flags;
  r.frames = s.frames;
  r.channels = s.channels;
  r.samples = s.samples;
  r.grid_rows = s.grid_rows;
  r.grid_cols = s.grid_cols;
  r.nchunks = s.nchunks;
  r.lists_per_frame = s.lists_per_frame;
  r.entries_per_frame = s.entries_per_frame;
  r.coil_group = s.coil_group;
  r.coil_parts = s.coil_parts;
  r.wait_limit = s.wait_fault ? s.wait_fault : kWaitLimit;
  r.wait_beyond = s.wait_fault ? (1 << 30) : 0;
  r.out_cols = s.out_cols;
  r.cpitch = s.cpitch;
  r.plan = s.plan_cols;
  r.col_shift = s.kb ? s.out_cols / 2 : 0;
  RowsLauncher rows_launch;
  if (!rows_launch.setup<W, kFormat>(s)) return KSJ_GPU_ERROR_CUDA;

  ColsArgs c{};
  c.tw_rows = tw_rows;
  c.inv_dr = inv_dr;
  c.inv_dc = inv_dc;
  c.pos_rows = pos_rows;
  c.flags = flags;
  c.frames = s.frames;
  c.channels = s.channels;
  c.grid_rows = s.grid_rows;
  c.out_rows = s.out_rows;
  c.out_cols = s.out_cols;
  c.kb = s.kb ? 1 : 0;
  c.row_shift = s.kb ? s.out_rows / 2 : 0;
  c.column_block = s.column_block;
  c.col_group = s.col_group;
  c.groups = s.cpitch / s.col_group;
  c.plan = s.plan_rows;
  const bool coil_major = d->output == KSJ_GPU_OUTPUT_COIL_MAJOR;
  c.output = d->output == KSJ_GPU_OUTPUT_RSS ? KSJ_GPU_OUTPUT_RSS : KSJ_GPU_OUTPUT_COIL_LAST;
  c.out = coil_major ? static_cast<void*>(ws + l.coil_last) : d_out;
  c.out_pitch = s.channels;
  ColsPass cols_pass;
  if (!cols_pass.setup(s, inter, &c)) return KSJ_GPU_ERROR_CUDA;

  // frames in passes sized so one pass's row-transformed grid stays in L2
  const int pixels = s.out_rows * s.out_cols;
  bool alt_used = false;
  if (io != nullptr && s.frames > s.frames_per_pass &&
      (cudaEventRecord(io->ready, stream) != cudaSuccess || cudaStreamWaitEvent(io->alt, io->ready, 0) != cudaSuccess))
    return KSJ_GPU_ERROR_CUDA;
  for (int f0 = 0, pass = 0; f0 < s.frames; f0 += s.frames_per_pass, ++pass) {
    const int nf = std::min(s.frames_per_pass, s.frames - f0);
    cudaStream_t ps = stream;
    if (io != nullptr) {
      if (pass & 1) {
        ps = io->alt;
        alt_used = true;
      }
      if (io->copy != nullptr) {
        if (cudaStreamWaitEvent(ps, io->in[pass], 0) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
        to_coil_last(f0, nf, ps);
      }
    }
    r.frame0 = f0;
    c.frame0 = f0;
    rows_launch.launch(r, s.grid_rows, (s.channels + s.coil_group - 1) / s.coil_group, nf, ps);
    cols_pass.launch(c, nf, ps, "k_cols");
    if (coil_major) {
      // [frame][pixel][channel] -> [frame][channel][pixel], this pass's frames
      const size_t fe = static_cast<size_t>(pixels) * s.channels;
      const dim3 tg((s.channels + 31) / 32, (pixels + 31) / 32, nf);
      LaunchScope scope("k_images_coil_major", ps);
      k_transpose<unsigned long long><<<tg, dim3(32, 8), 0, ps>>>(
          reinterpret_cast<const unsigned long long*>(ws + l.coil_last) + f0 * fe,
          static_cast<unsigned long long*>(d_out) + f0 * fe, pixels, s.channels);
    }
    if (io != nullptr && io->copy != nullptr) {
      const size_t off = static_cast<size_t>(f0) * io->out_frame_bytes;
      if (cudaEventRecord(io->done[pass], ps) != cudaSuccess ||
          cudaStreamWaitEvent(io->copy, io->done[pass], 0) != cudaSuccess ||
          cudaMemcpyAsync(static_cast<unsigned char*>(io->h_out) + off, static_cast<unsigned char*>(d_out) + off,
                          static_cast<size_t>(nf) * io->out_frame_bytes, cudaMemcpyDeviceToHost, io->copy) !=
              cudaSuccess)
        return KSJ_GPU_ERROR_CUDA;
    }
  }
  // the second compute stream joins back before the call's stream goes on
  if (alt_used &&
      (cudaEventRecord(io->alt_done, io->alt) != cudaSuccess || cudaStreamWaitEvent(stream, io->alt_done, 0) != cudaSuccess))
    return KSJ_GPU_ERROR_CUDA;
  return check_launch();
}

// ------------------------------------------------- Pipe-Menon density weights
//
// w <- w / ((w * phi) sampled back through phi), phi the Kaiser-Bessel
// gridding kernel, 10 iterations by default, in double precision (Pipe and
// Menon, MRM 1999; grid-based form).  The binning lists of the gridding path
// give, per (row, 16-column chunk), the samples touching it in increasing
// order, so each grid cell sums its samples in that order: deterministic.

template <int W>
struct PmRecord {
  int r0, c0;  // first tap row and column (wrapped)
  double wr[W];
  double wc[W];
};

__device__ __forceinline__ double kb_weight64(double d, int width, double beta, double inv_i0_beta) {
  const double t = 2.0 * d / static_cast<double>(width);
  if (t * t > 1.0) return 0.0;
  return cyl_bessel_i0(beta * sqrt(1.0 - t * t)) * inv_i0_beta;
}

// Per sample: the double-precision tap weights and w = 1.  The coordinate
// u = k g / (2 pi) is formed in double (an exact product, one rounded
// division); a sample the gridding checks rejected gets w = 0.
template <int W>
__global__ void __launch_bounds__(256) k_pm_prepare(const float* traj, PmRecord<W>* pm, double* w, size_t total,
                                                    int grid_rows, int grid_cols, double beta, double inv_i0_beta,
                                                    int require_nyquist) {
  const size_t idx = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const float2 k = __ldg(reinterpret_cast<const float2*>(traj) + idx);
  bool ok = isfinite(k.x) && isfinite(k.y);
  if (ok && require_nyquist) ok = k.x >= -kPiF && k.x <= kPiF && k.y >= -kPiF && k.y <= kPiF;
  if (ok && !require_nyquist) ok = fabsf(k.x) < 1.0e4f && fabsf(k.y) < 1.0e4f;
  PmRecord<W> r;
  constexpr double kTwoPiD = 6.283185307179586476925286766559;
  if (ok) {
    const double ur = static_cast<double>(k.x) * grid_rows / kTwoPiD;
    const double uc = static_cast<double>(k.y) * grid_cols / kTwoPiD;
    const int tr = static_cast<int>(floor(ur)) - W / 2 + 1;
    const int tc = static_cast<int>(floor(uc)) - W / 2 + 1;
    r.r0 = wrap_index(tr, grid_rows);
    r.c0 = wrap_index(tc, grid_cols);
#pragma unroll
    for (int j = 0; j < W; ++j) {
      r.wr[j] = kb_weight64(static_cast<double>(tr + j) - ur, W, beta, inv_i0_beta);
      r.wc[j] = kb_weight64(static_cast<double>(tc + j) - uc, W, beta, inv_i0_beta);
    }
  } else {
    r.r0 = 0;
    r.c0 = 0;
#pragma unroll
    for (int j = 0; j < W; ++j) {
      r.wr[j] = 0.0;
      r.wc[j] = 0.0;
    }
  }
  pm[idx] = r;
  w[idx] = ok ? 1.0 : 0.0;
}

// The grid step, kPmLanes lanes per list: lane q takes the list's entries q,
// q + kPmLanes, ... in order and, for every column tap of an entry that lands
// in the list's 16-column chunk, adds u * wc[k] (u = w times the entry's row,
// and plane, weights) to its own 16 cells in shared memory (cell t of thread
// i at cells[t * kPmThreads + i]: the lanes of a warp always touch distinct
// banks).  Then lane q sums cells 4q .. 4q+3 over the list's lanes, each cell
// in a fixed order (starting at lane q), and writes them.  Every FP64
// operation a lane issues is one a cell needs; with a lane per column
// instead, 12 of every 16 lanes multiplied by taps outside their column, and
// this step is bound by the FP64 pipe.  Lists are kPmLanes consecutive lanes
// of one warp, so a warp barrier orders the two phases.
constexpr int kPmLanes = 4;
constexpr int kPmThreads = 256;
constexpr int kPmCellsPerLane = kChunk / kPmLanes;
static_assert(kChunk == 16 && (kPmLanes & (kPmLanes - 1)) == 0 && 32 % kPmLanes == 0, "lanes of a list");

// One lane's share of the list's entries [e0, e1) (every `step`-th), added to
// its cells (cell[t * kPmThreads], t = column - lo).  `weight(r, sidx, &u)`
// gives the entry's u, or false when its row (and plane) taps miss the list.
template <int W, class Rec, class Weight>
__device__ __forceinline__ void pm_accumulate(const uint32_t* entries, uint32_t e0, uint32_t e1, uint32_t step,
                                              const Rec* rec, int lo, int grid_cols, double* cell, Weight weight) {
  for (uint32_t e = e0; e < e1; e += step) {
    const uint32_t sidx = __ldg(entries + e);
    const Rec& r = rec[sidx];
    double u;
    if (!weight(r, sidx, &u)) continue;
    int col = r.c0;
#pragma unroll
    for (int k = 0; k < W; ++k) {
      const int t = col - lo;
      if (t >= 0 && t < kChunk) cell[t * kPmThreads] = fma(u, r.wc[k], cell[t * kPmThreads]);
      if (++col == grid_cols) col = 0;
    }
  }
}

// Lane q of a list (its lane 0 is thread `lane0`): cells 4q .. 4q+3 summed
// over the list's lanes, starting at lane q, written to row[lo + t] inside
// the grid.
__device__ __forceinline__ void pm_reduce_store(const double* cells, int lane0, int q, double* row, int lo,
                                                int grid_cols) {
#pragma unroll
  for (int i = 0; i < kPmCellsPerLane; ++i) {
    const int t = q * kPmCellsPerLane + i;
    const double* c = cells + t * kPmThreads + lane0;
    double acc = c[q];
#pragma unroll
    for (int j = 1; j < kPmLanes; ++j) acc += c[(q + j) & (kPmLanes - 1)];
    if (lo + t < grid_cols) row[lo + t] = acc;
  }
}

template <int W>
__global__ void __launch_bounds__(kPmThreads) k_pm_grid(const uint32_t* offsets, const uint32_t* entries,
                                                        const PmRecord<W>* pm, const double* w, double* grid,
                                                        int frames, int samples, int grid_rows, int grid_cols,
                                                        int nchunks, int lists_per_frame, size_t entries_per_frame) {
  __shared__ double cells[kChunk * kPmThreads];
  const size_t list = (static_cast<size_t>(blockIdx.x) * kPmThreads + threadIdx.x) / kPmLanes;
  const int q = threadIdx.x & (kPmLanes - 1);
  double* cell = cells + threadIdx.x;
#pragma unroll
  for (int t = 0; t < kChunk; ++t) cell[t * kPmThreads] = 0.0;
  const bool active = list < static_cast<size_t>(frames) * lists_per_frame;
  int f = 0, row = 0, lo = 0;
  if (active) {
    f = static_cast<int>(list / lists_per_frame);
    const int l = static_cast<int>(list - static_cast<size_t>(f) * lists_per_frame);
    row = l / nchunks;
    lo = (l - row * nchunks) * kChunk;
    const uint32_t* off = offsets + static_cast<size_t>(f) * (lists_per_frame + 1);
    const PmRecord<W>* rec = pm + static_cast<size_t>(f) * samples;
    const double* wf = w + static_cast<size_t>(f) * samples;
    pm_accumulate<W>(entries + static_cast<size_t>(f) * entries_per_frame, off[l] + q, off[l + 1], kPmLanes, rec, lo,
                     grid_cols, cell, [&](const PmRecord<W>& r, uint32_t sidx, double* u) {
                       int dr = row - r.r0;
                       if (dr < 0) dr += grid_rows;
                       if (dr >= W) return false;
                       *u = wf[sidx] * r.wr[dr];
                       return true;
                     });
  }
  __syncwarp();
  if (active)
    pm_reduce_store(cells, threadIdx.x - q, q, grid + (static_cast<size_t>(f) * grid_rows + row) * grid_cols, lo,
                    grid_cols);
}

// Per sample: d = the grid read back through the sample's taps (row-major),
// w = w / d (0 when d is not positive); the last iteration also writes the
// float weights.
template <int W>
__global__ void __launch_bounds__(256) k_pm_update(const PmRecord<W>* pm, const double* grid, double* w, float* out,
                                                   size_t total, int samples, int grid_rows, int grid_cols) {
  const size_t idx = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const size_t f = idx / samples;
  const PmRecord<W> r = pm[idx];
  const double* g = grid + f * grid_rows * grid_cols;
  // separable taps: d = sum_a wr[a] (sum_b wc[b] grid[a][b]), W + 1 FP64
  // operations per row of taps instead of 2W
  int cols[W];
#pragma unroll
  for (int b = 0; b < W; ++b) {
    cols[b] = r.c0 + b;
    if (cols[b] >= grid_cols) cols[b] -= grid_cols;
  }
  double d = 0.0;
#pragma unroll
  for (int a = 0; a < W; ++a) {
    int rr = r.r0 + a;
    if (rr >= grid_rows) rr -= grid_rows;
    const double* line = g + static_cast<size_t>(rr) * grid_cols;
    double t = 0.0;
#pragma unroll
    for (int b = 0; b < W; ++b) t = fma(line[cols[b]], r.wc[b], t);
    d = fma(r.wr[a], t, d);
  }
  const double nw = d > 0.0 ? w[idx] / d : 0.0;
  w[idx] = nw;
  if (out != nullptr) out[idx] = static_cast<float>(nw);
}

struct PmLayout {
  size_t flags, records, counts, cursor, offsets, entries, long_lists, pm, w, grid, total;
};

PmLayout make_pm_layout(const Shape& s) {
  PmLayout l{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off = align_up(off + bytes, 256);
    return at;
  };
  const size_t fm = static_cast<size_t>(s.frames) * s.samples;
  const size_t nl = static_cast<size_t>(s.frames) * s.lists_per_frame;
  l.flags = take(kFlagBytes);
  l.records = take(fm * record_bytes(s.width));
  l.counts = take(nl * 4);
  l.cursor = take(nl * 4);
  l.offsets = take((nl + s.frames) * 4);
  l.entries = take(static_cast<size_t>(s.frames) * s.entries_per_frame * 4);
  l.long_lists = take((2 + static_cast<size_t>(s.frames) * s.entries_per_frame / (s.list_capacity + 1)) * 4);
  l.pm = take(fm * (8 + 16 * static_cast<size_t>(s.width)));
  l.w = take(fm * sizeof(double));
  l.grid = take(static_cast<size_t>(s.frames) * s.grid_rows * s.grid_cols * sizeof(double));
  l.total = off;
  return l;
}

template <int W>
ksj_gpu_status launch_pipe_menon(const Shape& s, const PmLayout& l, const ksj_gpu_gridding_desc* d,
                                 uint32_t iterations, const float* d_traj, float* d_dcf, unsigned char* ws,
                                 cudaStream_t stream) {
  static_assert(sizeof(PmRecord<W>) == 8 + 16 * W, "PmRecord layout");
  uint32_t* flags = reinterpret_cast<uint32_t*>(ws + l.flags);
  if (cudaMemsetAsync(flags, 0, kFlagBytes, stream) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  ksj_gpu_gridding_desc dd = *d;
  dd.dcf_mode = KSJ_GPU_DCF_NONE;
  const ksj_gpu_status st =
      build_lists<W>(s, &dd, d_traj, nullptr, flags, ws + l.records, reinterpret_cast<uint32_t*>(ws + l.counts),
                     reinterpret_cast<uint32_t*>(ws + l.cursor), reinterpret_cast<uint32_t*>(ws + l.offsets),
                     reinterpret_cast<uint32_t*>(ws + l.entries), nullptr,
                     reinterpret_cast<uint32_t*>(ws + l.long_lists), stream);
  if (st != KSJ_GPU_OK) return st;
  const size_t fm = static_cast<size_t>(s.frames) * s.samples;
  PmRecord<W>* pm = reinterpret_cast<PmRecord<W>*>(ws + l.pm);
  double* w = reinterpret_cast<double*>(ws + l.w);
  double* grid = reinterpret_cast<double*>(ws + l.grid);
  const double beta = s.beta;
  {
    LaunchScope scope("k_pm_prepare", stream);
    k_pm_prepare<W><<<static_cast<unsigned>((fm + 255) / 256), 256, 0, stream>>>(
        d_traj, pm, w, fm, s.grid_rows, s.grid_cols, beta, 1.0 / std::cyl_bessel_i(0.0, beta), d->require_nyquist);
  }
  const size_t lists = static_cast<size_t>(s.frames) * s.lists_per_frame;
  for (uint32_t it = 0; it < iterations; ++it) {
    {
      LaunchScope scope("k_pm_grid", stream);
      k_pm_grid<W><<<static_cast<unsigned>((lists * kPmLanes + kPmThreads - 1) / kPmThreads), kPmThreads, 0, stream>>>(
          reinterpret_cast<const uint32_t*>(ws + l.offsets), reinterpret_cast<const uint32_t*>(ws + l.entries), pm,
          w, grid, s.frames, s.samples, s.grid_rows, s.grid_cols, s.nchunks, s.lists_per_frame,
          s.entries_per_frame);
    }
    LaunchScope scope("k_pm_update", stream);
    k_pm_update<W><<<static_cast<unsigned>((fm + 255) / 256), 256, 0, stream>>>(
        pm, grid, w, it + 1 == iterations ? d_dcf : nullptr, fm, s.samples, s.grid_rows, s.grid_cols);
  }
  return check_launch();
}

// ------------------------------------------------------------ 3-D gridding
//
// A g^3 grid is gridded as g z-planes of the 2-D row/column machinery: the
// binning lists are (plane, row, 16-column chunk); an entry's row weight is
// the sample's y weight times its z weight for that plane; every plane reads
// the one coil-last sample array.  After the per-plane row and column passes
// (y and x transformed, cropped, deapodised) the intermediate
// [plane][pixel][coil] takes a third pass along z, which is the column pass
// again with planes as rows and pixels as columns.

struct Prepare3Args {
  const float* traj;  // [M][3] (k_z, k_y, k_x)
  const float* dcf;
  uint32_t dcf_mode;
  unsigned char* records;
  uint32_t* counts;  // [plane][row * nchunks + chunk]
  uint32_t* flags;
  int samples, grid, nchunks, lists_per_plane;
  float beta, two_over_w, inv_i0_beta, phase;
};

template <int W>
__global__ void __launch_bounds__(256) k_prepare3(Prepare3Args a) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= a.samples) return;
  const float kz = __ldg(a.traj + 3 * static_cast<size_t>(idx));
  const float ky = __ldg(a.traj + 3 * static_cast<size_t>(idx) + 1);
  const float kx = __ldg(a.traj + 3 * static_cast<size_t>(idx) + 2);
  bool ok = isfinite(kz) && isfinite(ky) && isfinite(kx) && fabsf(kz) < 1.0e4f && fabsf(ky) < 1.0e4f &&
            fabsf(kx) < 1.0e4f;
  float w = 1.0f;
  if (a.dcf_mode == KSJ_GPU_DCF_ANALYTIC_RAMP) {
    w = fmaf(kz, kz, fmaf(ky, ky, kx * kx));  // 3-D radial density ~ 1 / |k|^2
  } else if (a.dcf_mode == KSJ_GPU_DCF_EXTERNAL) {
    w = __ldg(a.dcf + idx);
    if (!(isfinite(w) && w >= 0.0f)) {
      atomicOr(a.flags, KSJ_GPU_FLAG_BAD_DCF);
      w = 0.0f;
    }
  }
  SampleRecord3<W> rec;
  rec.pad = 0;
  if (!ok) {
    atomicOr(a.flags, KSJ_GPU_FLAG_BAD_TRAJECTORY);
    rec.z0 = rec.r0 = rec.c0 = 0;
    rec.scale = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int j = 0; j < W; ++j) rec.wz[j] = rec.wr[j] = rec.wc[j] = 0.0f;
  } else {
    const float gf = static_cast<float>(a.grid);
    const dfloat uz = grid_coordinate(kz, gf), uy = grid_coordinate(ky, gf), ux = grid_coordinate(kx, gf);
    float f;
    const int sz = dfloor(uz, &f) - W / 2 + 1;
    const int sy = dfloor(uy, &f) - W / 2 + 1;
    const int sx = dfloor(ux, &f) - W / 2 + 1;
    rec.z0 = wrap_index(sz, a.grid);
    rec.r0 = wrap_index(sy, a.grid);
    rec.c0 = wrap_index(sx, a.grid);
#pragma unroll
    for (int j = 0; j < W; ++j) {
      rec.wz[j] = kb_weight(__fsub_rn(__fsub_rn(static_cast<float>(sz + j), uz.hi), uz.lo), a.two_over_w, a.beta,
                            a.inv_i0_beta);
      rec.wr[j] = kb_weight(__fsub_rn(__fsub_rn(static_cast<float>(sy + j), uy.hi), uy.lo), a.two_over_w, a.beta,
                            a.inv_i0_beta);
      rec.wc[j] = kb_weight(__fsub_rn(__fsub_rn(static_cast<float>(sx + j), ux.hi), ux.lo), a.two_over_w, a.beta,
                            a.inv_i0_beta);
    }
    rec.scale = cscale(exp_i_dot3(kz, a.phase, ky, a.phase, kx, a.phase), w);
  }
  reinterpret_cast<SampleRecord3<W>*>(a.records)[idx] = rec;
  int k0, k1;
  list_chunks<W>(rec.c0, a.grid, &k0, &k1);
#pragma unroll
  for (int i = 0; i < W; ++i) {
    int plane = rec.z0 + i;
    if (plane >= a.grid) plane -= a.grid;
    uint32_t* counts = a.counts + static_cast<size_t>(plane) * a.lists_per_plane;
#pragma unroll
    for (int j = 0; j < W; ++j) {
      int row = rec.r0 + j;
      if (row >= a.grid) row -= a.grid;
      atomicAdd(counts + row * a.nchunks + k0, 1u);
      if (k1 != k0) atomicAdd(counts + row * a.nchunks + k1, 1u);
    }
  }
}

// The per-plane scans leave offsets[p][lists] = the plane's total; turn them
// into absolute positions in one entry array (one block: planes <= 512).
__global__ void __launch_bounds__(512) k_plane_bases(uint32_t* offsets, int planes, int lists, uint32_t* bases) {
  __shared__ uint32_t tot[512];
  const int t = threadIdx.x;
  tot[t] = t < planes ? offsets[static_cast<size_t>(t) * (lists + 1) + lists] : 0u;
  __syncthreads();
  if (t == 0) {
    uint32_t run = 0;
    for (int p = 0; p < planes; ++p) {
      const uint32_t v = tot[p];
      tot[p] = run;
      run += v;
    }
  }
  __syncthreads();
  if (t < planes) bases[t] = tot[t];
}

__global__ void __launch_bounds__(256) k_offsets_add(uint32_t* offsets, int planes, int lists, const uint32_t* bases) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= static_cast<size_t>(planes) * (lists + 1)) return;
  offsets[i] += bases[i / (lists + 1)];
}

template <int W>
__global__ void __launch_bounds__(256) k_scatter3(const unsigned char* records, const uint32_t* offsets,
                                                  uint32_t* cursor, uint32_t* entries, int samples, int grid,
                                                  int nchunks, int lists_per_plane) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= samples) return;
  const SampleRecord3<W>& rec = reinterpret_cast<const SampleRecord3<W>*>(records)[idx];
  int k0, k1;
  list_chunks<W>(rec.c0, grid, &k0, &k1);
  for (int i = 0; i < W; ++i) {
    int plane = rec.z0 + i;
    if (plane >= grid) plane -= grid;
    const uint32_t* off = offsets + static_cast<size_t>(plane) * (lists_per_plane + 1);
    uint32_t* cur = cursor + static_cast<size_t>(plane) * lists_per_plane;
    for (int j = 0; j < W; ++j) {
      int row = rec.r0 + j;
      if (row >= grid) row -= grid;
      const int l0 = row * nchunks + k0;
      entries[off[l0] + atomicAdd(cur + l0, 1u)] = static_cast<uint32_t>(idx);
      if (k1 != k0) {
        const int l1 = row * nchunks + k1;
        entries[off[l1] + atomicAdd(cur + l1, 1u)] = static_cast<uint32_t>(idx);
      }
    }
  }
}

struct Layout3 {
  size_t flags, records, counts, cursor, offsets, bases, entries, expanded, long_lists, samples_t, inter, inter2,
      tables, total;
  size_t entries_total;
};

size_t record3_bytes(int width) {
  switch (width) {
    case 2: return sizeof(SampleRecord3<2>);
    case 4: return sizeof(SampleRecord3<4>);
    case 6: return sizeof(SampleRecord3<6>);
    default: return sizeof(SampleRecord3<8>);
  }
}

// s: the 2-D shape of one plane with frames = planes (see make_shape3).
Layout3 make_layout3(const Shape& s, uint32_t sample_format) {
  Layout3 l{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off = align_up(off + bytes, 256);
    return at;
  };
  const size_t g = static_cast<size_t>(s.grid_rows), n = static_cast<size_t>(s.rows);
  const size_t nl = g * s.lists_per_frame;
  l.entries_total = static_cast<size_t>(s.samples) * s.width * s.width * 2;
  l.flags = take(kFlagBytes);
  l.records = take(static_cast<size_t>(s.samples) * record3_bytes(s.width));
  l.counts = take(nl * 4);
  l.cursor = take(nl * 4);
  l.offsets = take((nl + g) * 4);
  l.bases = take(g * 4);
  l.entries = take(l.entries_total * 4);
  l.expanded = take(l.entries_total * meta_vecs(s.width) * 16);
  l.long_lists = take((2 + l.entries_total / (s.list_capacity + 1)) * 4);
  l.samples_t = take(static_cast<size_t>(s.samples) * s.channels * sample_bytes(sample_format));
  l.inter = take(g * g * n * s.cpitch * sizeof(float2));
  l.inter2 = take(g * n * n * s.cpitch * sizeof(float2));
  // twiddles (rows, cols), deapodisation (rows, cols), DIF positions (rows, cols), ones for the pixel axis
  l.tables = take(2 * g * sizeof(float2) + 2 * n * sizeof(float) + 2 * n * sizeof(int) + n * n * sizeof(float));
  l.total = off;
  return l;
}

ksj_gpu_status make_shape3(const ksj_gpu_gridding3_desc* d, const ksj_gpu_gridding_tuning* t, Shape* s) {
  if (d == nullptr || d->struct_size < sizeof(ksj_gpu_gridding3_desc)) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (d->output != KSJ_GPU_OUTPUT_RSS && d->output != KSJ_GPU_OUTPUT_COIL_LAST) return KSJ_GPU_ERROR_UNSUPPORTED;
  if (d->image == 0 || d->grid == 0 || static_cast<uint64_t>(d->image) * d->image > (1u << 24))
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  ksj_gpu_gridding_desc d2{};
  d2.struct_size = sizeof(d2);
  d2.kernel = KSJ_GPU_KERNEL_KAISER_BESSEL;
  d2.image_rows = d2.image_cols = d->image;
  d2.grid_rows = d2.grid_cols = d->grid;
  d2.kernel_width = d->kernel_width;
  d2.kb_beta = d->kb_beta;
  d2.row_origin = d2.col_origin = (static_cast<double>(d->image) - 1.0) / 2.0;
  d2.channels = d->channels;
  d2.samples = d->samples;
  d2.frames = d->grid;  // one frame per z-plane
  d2.dcf_mode = d->dcf_mode;
  d2.output = KSJ_GPU_OUTPUT_COIL_LAST;
  d2.sample_format = d->sample_format;
  const ksj_gpu_status st = make_shape(&d2, t, s);
  if (st != KSJ_GPU_OK) return st;
  s->entries_per_frame = 0;  // absolute offsets into one entry array
  return KSJ_GPU_OK;
}

// The 3-D binning lists: per-sample records, (plane, row, chunk) counts, per-plane
// scans made absolute, the scattered entries, their sort and (when `expanded`
// is given) the expanded entries.  `flags` must already be cleared.
template <int W>
ksj_gpu_status build_lists3(const Shape& s, uint32_t dcf_mode, const float* d_traj, const float* d_dcf,
                            uint32_t* flags, unsigned char* records, uint32_t* counts, uint32_t* cursor,
                            uint32_t* offsets, uint32_t* bases, uint32_t* entries, float4* expanded,
                            uint32_t* long_lists, size_t entries_total, cudaStream_t stream) {
  const int g = s.grid_rows;
  const size_t nl = static_cast<size_t>(g) * s.lists_per_frame;
  if (cudaMemsetAsync(counts, 0, nl * 4, stream) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  if (cudaMemsetAsync(cursor, 0, nl * 4, stream) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  {
    Prepare3Args p{};
    p.traj = d_traj;
    p.dcf = d_dcf;
    p.dcf_mode = dcf_mode;
    p.records = records;
    p.counts = counts;
    p.flags = flags;
    p.samples = s.samples;
    p.grid = g;
    p.nchunks = s.nchunks;
    p.lists_per_plane = s.lists_per_frame;
    p.beta = s.beta;
    p.two_over_w = 2.0f / static_cast<float>(s.width);
    p.inv_i0_beta = s.inv_i0_beta;
    p.phase = s.phase_row;
    LaunchScope scope("k_prepare3", stream);
    k_prepare3<W><<<(s.samples + 255) / 256, 256, 0, stream>>>(p);
  }
  {
    LaunchScope scope("k_scan", stream);
    k_scan<<<g, 1024, 0, stream>>>(counts, offsets, s.lists_per_frame);
  }
  {
        LaunchScope scope("k_plane_offsets", stream);
    k_plane_bases<<<1, 512, 0, stream>>>(offsets, g, s.lists_per_frame, bases);
    const size_t total = static_cast<size_t>(g) * (s.lists_per_frame + 1);
    k_offsets_add<<<static_cast<unsigned>((total + 255) / 256), 256, 0, stream>>>(offsets, g, s.lists_per_frame,
                                                                                bases);
  }
  {
    LaunchScope scope("k_scatter3", stream);
    k_scatter3<W><<<(s.samples + 255) / 256, 256, 0, stream>>>(records, offsets, cursor, entries, s.samples, g,
                                                               s.nchunks, s.lists_per_frame);
  }
  {
    SortArgs sa{};
    sa.offsets = offsets;
    sa.entries = entries;
    sa.records = records;
    sa.expanded = expanded;
    sa.long_count = long_lists;
    sa.long_lists = sa.long_count + 1;
    sa.frames = g;
    sa.samples = s.samples;
    sa.lists_per_frame = s.lists_per_frame;
    sa.nchunks = s.nchunks;
    sa.grid_rows = g;
    sa.grid_cols = g;
    sa.capacity = s.list_capacity;
    sa.entries_per_frame = 0;
    sa.dim3 = 1;
    const ksj_gpu_status st = launch_sort<W>(sa, nl, entries_total, s.list_capacity, stream);
    if (st != KSJ_GPU_OK) return st;
  }
  return KSJ_GPU_OK;
}

template <int W, uint32_t kFormat>
ksj_gpu_status launch_all3(const Shape& s, const Layout3& l, const ksj_gpu_gridding3_desc* d, const void* d_kspace,
                           const float* d_traj, const float* d_dcf, void* d_out, unsigned char* ws,
                           cudaStream_t stream) {
  const int g = s.grid_rows, n = s.rows;
  uint32_t* flags = reinterpret_cast<uint32_t*>(ws + l.flags);
  uint32_t* counts = reinterpret_cast<uint32_t*>(ws + l.counts);
  uint32_t* cursor = reinterpret_cast<uint32_t*>(ws + l.cursor);
  uint32_t* offsets = reinterpret_cast<uint32_t*>(ws + l.offsets);
  uint32_t* entries = reinterpret_cast<uint32_t*>(ws + l.entries);
  float2* inter = reinterpret_cast<float2*>(ws + l.inter);
  float2* inter2 = reinterpret_cast<float2*>(ws + l.inter2);
  float2* tw_rows = reinterpret_cast<float2*>(ws + l.tables);
  float2* tw_cols = tw_rows + g;
  float* inv_dr = reinterpret_cast<float*>(tw_cols + g);
  float* inv_dc = inv_dr + n;
  int* pos_rows = reinterpret_cast<int*>(inv_dc + n);
  int* pos_cols = pos_rows + n;
  float* ones = reinterpret_cast<float*>(pos_cols + n);

  if (cudaMemsetAsync(flags, 0, kFlagBytes, stream) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  {
    const int nt = std::max(g, n);
    LaunchScope scope("k_tables", stream);
    k_tables<<<(nt + 255) / 256, 256, 0, stream>>>(tw_rows, g, tw_cols, g, inv_dr, n, inv_dc, n, pos_rows, pos_cols,
                                                   s.plan_rows, s.plan_cols, 1, s.width, s.beta,
                                                   std::cyl_bessel_i(0.0, static_cast<double>(s.beta)));
  }
  {
    LaunchScope scope("k_fill_ones", stream);
    k_fill<<<(n * n + 255) / 256, 256, 0, stream>>>(ones, n * n, 1.0f);
  }
  {
    const ksj_gpu_status st = build_lists3<W>(s, d->dcf_mode, d_traj, d_dcf, flags, ws + l.records, counts, cursor,
                                              offsets, reinterpret_cast<uint32_t*>(ws + l.bases), entries,
                                              reinterpret_cast<float4*>(ws + l.expanded),
                                              reinterpret_cast<uint32_t*>(ws + l.long_lists), l.entries_total,
                                              stream);
    if (st != KSJ_GPU_OK) return st;
  }
  {
    const dim3 tg((s.samples + 31) / 32, (s.channels + 31) / 32, 1);
    LaunchScope scope("k_samples_coil_last", stream);
    k_samples_coil_last<kFormat><<<tg, dim3(32, 8), 0, stream>>>(d_kspace, ws + l.samples_t, s.channels, s.samples,
                                                                 flags, nullptr, nullptr, nullptr, 0, nullptr);
  }
  // rows of every plane (x transformed, kept columns, coil-last)
  RowsArgs r{};
  r.samples_t = ws + l.samples_t;
  r.sample_frame_stride = 0;
  r.offsets = offsets;
  r.expanded = reinterpret_cast<const float4*>(ws + l.expanded);
  r.tw_cols = tw_cols;
  r.pos_cols = pos_cols;
  r.inter = inter;
  r.flags = flags;
  r.frames = g;
  r.channels = s.channels;
  r.samples = s.samples;
  r.grid_rows = g;
  r.grid_cols = g;
  r.nchunks = s.nchunks;
  r.lists_per_frame = s.lists_per_frame;
  r.entries_per_frame = 0;
  r.coil_group = s.coil_group;
  r.coil_parts = s.coil_parts;
  r.wait_limit = s.wait_fault ? s.wait_fault : kWaitLimit;
  r.wait_beyond = s.wait_fault ? (1 << 30) : 0;
  r.out_cols = n;
  r.cpitch = s.cpitch;
  r.plan = s.plan_cols;
  r.col_shift = n / 2;
  RowsLauncher rows_launch;
  if (!rows_launch.setup<W, kFormat>(s)) return KSJ_GPU_ERROR_CUDA;
  // columns of every plane (y transformed, cropped, y/x deapodised): [plane][pixel][cpitch]
  ColsArgs c{};
  c.tw_rows = tw_rows;
  c.inv_dr = inv_dr;
  c.inv_dc = inv_dc;
  c.pos_rows = pos_rows;
  c.flags = flags;
  c.frames = g;
  c.channels = s.channels;
  c.grid_rows = g;
  c.out_rows = n;
  c.out_cols = n;
  c.kb = 1;
  c.row_shift = n / 2;
  c.column_block = s.column_block;
  c.col_group = s.col_group;
  c.groups = s.cpitch / s.col_group;
  c.plan = s.plan_rows;
  c.output = KSJ_GPU_OUTPUT_COIL_LAST;
  c.out = inter2;
  c.out_pitch = s.cpitch;
  ColsPass cols_pass;
  if (!cols_pass.setup(s, inter, &c)) return KSJ_GPU_ERROR_CUDA;
  for (int f0 = 0; f0 < g; f0 += s.frames_per_pass) {
    const int nf = std::min(s.frames_per_pass, g - f0);
    r.frame0 = f0;
    c.frame0 = f0;
    rows_launch.launch(r, g, (s.channels + s.coil_group - 1) / s.coil_group, nf, stream);
    cols_pass.launch(c, nf, stream, "k_cols");
  }
  // z: the column pass over [plane][pixel][cpitch] with planes as rows and pixels as columns
  Shape z = s;
  z.frames = 1;
  z.out_cols = n * n;
  ColsArgs cz = c;
  cz.frame0 = 0;
  cz.frames = 1;
  cz.out_cols = n * n;
  cz.inv_dc = ones;
  cz.output = d->output;
  cz.out = d_out;
  cz.out_pitch = s.channels;
  ColsPass z_pass;
  if (!z_pass.setup(z, inter2, &cz)) return KSJ_GPU_ERROR_CUDA;
  z_pass.launch(cz, 1, stream, "k_cols_z");
  return check_launch();
}

// ------------------------------------------- 3-D Pipe-Menon density weights

template <int W>
struct PmRecord3 {
  int z0, r0, c0, pad;
  double wz[W];
  double wr[W];
  double wc[W];
};

// The column part of a 3-D record, compact: what the grid step gathers per
// entry after the first iteration (the entry's plane and row weight product
// is kept per entry then).
template <int W>
struct PmCol3 {
  double wc[W];
  int c0, pad;
};

template <int W>
__global__ void __launch_bounds__(256) k_pm_prepare3(const float* traj, PmRecord3<W>* pm, PmCol3<W>* pmc, double* w,
                                                     int samples, int grid, double beta, double inv_i0_beta) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= samples) return;
  float k[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) k[d] = __ldg(traj + 3 * static_cast<size_t>(idx) + d);
  const bool ok = isfinite(k[0]) && isfinite(k[1]) && isfinite(k[2]) && fabsf(k[0]) < 1.0e4f &&
                  fabsf(k[1]) < 1.0e4f && fabsf(k[2]) < 1.0e4f;
  PmRecord3<W> r;
  r.pad = 0;
  constexpr double kTwoPiD = 6.283185307179586476925286766559;
  int t0[3] = {0, 0, 0};
  double u[3] = {0.0, 0.0, 0.0};
  if (ok)
    for (int d = 0; d < 3; ++d) {
      u[d] = static_cast<double>(k[d]) * grid / kTwoPiD;
      t0[d] = static_cast<int>(floor(u[d])) - W / 2 + 1;
    }
  r.z0 = wrap_index(t0[0], grid);
  r.r0 = wrap_index(t0[1], grid);
  r.c0 = wrap_index(t0[2], grid);
#pragma unroll
  for (int j = 0; j < W; ++j) {
    r.wz[j] = ok ? kb_weight64(static_cast<double>(t0[0] + j) - u[0], W, beta, inv_i0_beta) : 0.0;
    r.wr[j] = ok ? kb_weight64(static_cast<double>(t0[1] + j) - u[1], W, beta, inv_i0_beta) : 0.0;
    r.wc[j] = ok ? kb_weight64(static_cast<double>(t0[2] + j) - u[2], W, beta, inv_i0_beta) : 0.0;
  }
  pm[idx] = r;
  PmCol3<W> c;
#pragma unroll
  for (int j = 0; j < W; ++j) c.wc[j] = r.wc[j];
  c.c0 = r.c0;
  c.pad = 0;
  pmc[idx] = c;
  w[idx] = ok ? 1.0 : 0.0;
}

// One lane's share of a 3-D list's entries (as pm_accumulate).  The first
// iteration (kFirst) reads each entry's whole record, forms u = w * (wz[dz] *
// wr[dr]) and keeps the product wz[dz] * wr[dr] per entry (wzr, in entry
// order); the later iterations gather only w and the compact column record
// and read the product back in entry order -- under half the bytes per
// entry, the bound of this step.  The same operations in the same order
// either way: bit-identical cells.
template <int W, bool kFirst>
__device__ __forceinline__ void pm3_accumulate(const uint32_t* entries, uint32_t e0, uint32_t e1, uint32_t step,
                                               const PmRecord3<W>* pm, const PmCol3<W>* pmc, const double* w,
                                               double* wzr, int plane, int row, int lo, int g, double* cell) {
  for (uint32_t e = e0; e < e1; e += step) {
    const uint32_t sidx = __ldg(entries + e);
    double f;
    int col;
    const double* wc;
    if constexpr (kFirst) {
      const PmRecord3<W>& r = pm[sidx];
      int dz = plane - r.z0;
      if (dz < 0) dz += g;
      int dr = row - r.r0;
      if (dr < 0) dr += g;
      f = dz < W && dr < W ? r.wz[dz] * r.wr[dr] : 0.0;
      wzr[e] = f;
      col = r.c0;
      wc = r.wc;
    } else {
      f = wzr[e];
      const PmCol3<W>& c = pmc[sidx];
      col = c.c0;
      wc = c.wc;
    }
    // taps outside the list's plane or row (f >= 0: an integer test keeps
    // the FP64 pipe, the bound of this step, for the arithmetic)
    if (__double_as_longlong(f) == 0) continue;
    const double u = w[sidx] * f;
#pragma unroll
    for (int k = 0; k < W; ++k) {
      const int t = col - lo;
      if (t >= 0 && t < kChunk) cell[t * kPmThreads] = fma(u, wc[k], cell[t * kPmThreads]);
      if (++col == g) col = 0;
    }
  }
}

// The 3-D grid step for lists of at most `capacity` entries: the
// lanes-per-list form of k_pm_grid, with the entry's plane weight in u.
// Longer lists (queued by the list sort) are left to k_pm_long3.
template <int W, bool kFirst>
__global__ void __launch_bounds__(kPmThreads) k_pm_grid3(const uint32_t* offsets, const uint32_t* entries,
                                                         const PmRecord3<W>* pm, const PmCol3<W>* pmc, const double* w,
                                                         double* wzr, double* grid, int g, int nchunks,
                                                         int lists_per_plane, int capacity) {
  __shared__ double cells[kChunk * kPmThreads];
  const size_t list = (static_cast<size_t>(blockIdx.x) * kPmThreads + threadIdx.x) / kPmLanes;
  const int q = threadIdx.x & (kPmLanes - 1);
  double* cell = cells + threadIdx.x;
#pragma unroll
  for (int t = 0; t < kChunk; ++t) cell[t * kPmThreads] = 0.0;
  bool active = list < static_cast<size_t>(g) * lists_per_plane;
  int plane = 0, row = 0, lo = 0;
  if (active) {
    plane = static_cast<int>(list / lists_per_plane);
    const int l = static_cast<int>(list - static_cast<size_t>(plane) * lists_per_plane);
    row = l / nchunks;
    lo = (l - row * nchunks) * kChunk;
    const uint32_t* off = offsets + static_cast<size_t>(plane) * (lists_per_plane + 1);
    const uint32_t begin = off[l], end = off[l + 1];
    active = static_cast<int>(end - begin) <= capacity;
    if (active)
      pm3_accumulate<W, kFirst>(entries, begin + q, end, kPmLanes, pm, pmc, w, wzr, plane, row, lo, g, cell);
  }
  __syncwarp();
  if (active) pm_reduce_store(cells, threadIdx.x - q, q, grid + (static_cast<size_t>(plane) * g + row) * g, lo, g);
}

// The queued long lists (count at long_lists[0], global list ids after it)
// are cut into parts of kPmPart entries: part_base[i] is the first part of
// queued list i (an exclusive scan, the total at part_base[count]).
constexpr uint32_t kPmPart = 512;

__global__ void __launch_bounds__(1024) k_pm_long_parts(const uint32_t* long_lists, const uint32_t* offsets,
                                                        int lists_per_plane, uint32_t* part_base) {
  __shared__ uint32_t warp_sums[32];
  __shared__ uint32_t carry;
  const uint32_t queued = long_lists[0];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t i0 = 0; i0 < queued; i0 += 1024) {
    const uint32_t i = i0 + threadIdx.x;
    uint32_t parts = 0;
    if (i < queued) {
      const uint32_t gl = long_lists[1 + i];
      const uint32_t plane = gl / static_cast<uint32_t>(lists_per_plane);
      const uint32_t l = gl - plane * static_cast<uint32_t>(lists_per_plane);
      const uint32_t* off = offsets + static_cast<size_t>(plane) * (lists_per_plane + 1);
      parts = (off[l + 1] - off[l] + kPmPart - 1) / kPmPart;
    }
    uint32_t incl = parts;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += v;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      uint32_t ws = warp_sums[lane];
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, ws, d);
        if (lane >= d) ws += v;
      }
      warp_sums[lane] = ws;  // inclusive over warps
    }
    __syncthreads();
    const uint32_t before = carry + (warp > 0 ? warp_sums[warp - 1] : 0u) + incl - parts;
    if (i < queued) part_base[i] = before;
    __syncthreads();
    if (threadIdx.x == 1023) carry = before + parts;
    __syncthreads();
  }
  if (threadIdx.x == 0) part_base[queued] = carry;
}

// The long lists' parts, kPmLanes lanes per part (as in k_pm_grid3; every
// part the same work however long its list).  Each part's sums go to
// partial[part]; the part that completes its list's count (the counters grow
// by the list's part count every iteration, zeroed once per call) adds the
// list's parts in part order and writes the cells -- deterministic, and no
// part waits for another.  Groups stride over the parts.
template <int W, bool kFirst>
__global__ void __launch_bounds__(kPmThreads) k_pm_long3(const uint32_t* long_lists, const uint32_t* part_base,
                                                         const uint32_t* offsets, const uint32_t* entries,
                                                         const PmRecord3<W>* pm, const PmCol3<W>* pmc,
                                                         const double* w, double* wzr, double* grid, int g,
                                                         int nchunks, int lists_per_plane, double* partial,
                                                         uint32_t* counters) {
  __shared__ double cells[kChunk * kPmThreads];
  const int q = threadIdx.x & (kPmLanes - 1);
  const int lane0 = (threadIdx.x & 31) & ~(kPmLanes - 1);
  const unsigned gmask = ((1u << kPmLanes) - 1u) << lane0;
  const uint32_t queued = long_lists[0];
  const uint32_t total_parts = part_base[queued];
  const uint32_t groups = gridDim.x * (kPmThreads / kPmLanes);
  double* cell = cells + threadIdx.x;
  for (uint32_t part = (blockIdx.x * kPmThreads + threadIdx.x) / kPmLanes; part < total_parts; part += groups) {
    // the queued list holding this part: the last i with part_base[i] <= part
    uint32_t lo_i = 0, hi_i = queued;  // part_base[lo_i] <= part < part_base[hi_i]
    while (hi_i - lo_i > 1) {
      const uint32_t mid = (lo_i + hi_i) / 2;
      if (__ldg(part_base + mid) <= part)
        lo_i = mid;
      else
        hi_i = mid;
    }
    const uint32_t first = __ldg(part_base + lo_i), parts = __ldg(part_base + lo_i + 1) - first;
    const uint32_t gl = __ldg(long_lists + 1 + lo_i);
    const int plane = static_cast<int>(gl / static_cast<uint32_t>(lists_per_plane));
    const int l = static_cast<int>(gl - static_cast<uint32_t>(plane) * lists_per_plane);
    const int row = l / nchunks;
    const int lo = (l - row * nchunks) * kChunk;
    const uint32_t* off = offsets + static_cast<size_t>(plane) * (lists_per_plane + 1);
    const uint32_t e0 = off[l] + (part - first) * kPmPart, e1 = min(off[l + 1], e0 + kPmPart);
#pragma unroll
    for (int t = 0; t < kChunk; ++t) cell[t * kPmThreads] = 0.0;
    pm3_accumulate<W, kFirst>(entries, e0 + q, e1, kPmLanes, pm, pmc, w, wzr, plane, row, lo, g, cell);
    __syncwarp(gmask);
    // this part's sums (cells 4q .. 4q+3 over the group's lanes)
    double* mine = partial + static_cast<size_t>(part) * kChunk + q * kPmCellsPerLane;
#pragma unroll
    for (int i = 0; i < kPmCellsPerLane; ++i) {
      const double* c = cells + (q * kPmCellsPerLane + i) * kPmThreads + (threadIdx.x - q);
      double acc = c[q];
#pragma unroll
      for (int j = 1; j < kPmLanes; ++j) acc += c[(q + j) & (kPmLanes - 1)];
      mine[i] = acc;
    }
    __threadfence();
    __syncwarp(gmask);
    uint32_t old = 0;
    if (q == 0) old = atomicAdd(counters + lo_i, 1u);
    old = __shfl_sync(gmask, old, lane0);
    if ((old + 1) % parts == 0) {
      __threadfence();
      double acc[kPmCellsPerLane];
#pragma unroll
      for (int i = 0; i < kPmCellsPerLane; ++i) acc[i] = 0.0;
      for (uint32_t p = first; p < first + parts; ++p) {
        const double* src = partial + static_cast<size_t>(p) * kChunk + q * kPmCellsPerLane;
#pragma unroll
        for (int i = 0; i < kPmCellsPerLane; ++i) acc[i] += __ldcg(src + i);
      }
      double* out_row = grid + (static_cast<size_t>(plane) * g + row) * g;
#pragma unroll
      for (int i = 0; i < kPmCellsPerLane; ++i) {
        const int col = lo + q * kPmCellsPerLane + i;
        if (col < g) out_row[col] = acc[i];
      }
    }
    __syncwarp(gmask);  // the cells are read before the next part clears them
  }
}

template <int W>
__global__ void __launch_bounds__(256) k_pm_update3(const PmRecord3<W>* pm, const double* grid, double* w, float* out,
                                                    int samples, int g) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= samples) return;
  const PmRecord3<W> r = pm[idx];
  // separable taps: d = sum_a wz[a] sum_b wr[b] (sum_c wc[c] grid[a][b][c]):
  // W^3 + W^2 + W FP64 operations instead of 2 W^3 + W^2
  int cols[W];
#pragma unroll
  for (int c = 0; c < W; ++c) {
    cols[c] = r.c0 + c;
    if (cols[c] >= g) cols[c] -= g;
  }
  double d = 0.0;
  for (int a = 0; a < W; ++a) {
    int zz = r.z0 + a;
    if (zz >= g) zz -= g;
    double plane = 0.0;
#pragma unroll
    for (int b = 0; b < W; ++b) {
      int yy = r.r0 + b;
      if (yy >= g) yy -= g;
      const double* line = grid + (static_cast<size_t>(zz) * g + yy) * g;
      double t = 0.0;
#pragma unroll
      for (int c = 0; c < W; ++c) t = fma(line[cols[c]], r.wc[c], t);
      plane = fma(r.wr[b], t, plane);
    }
    d = fma(r.wz[a], plane, d);
  }
  const double nw = d > 0.0 ? w[idx] / d : 0.0;
  w[idx] = nw;
  if (out != nullptr) out[idx] = static_cast<float>(nw);
}

struct PmLayout3 {
  size_t flags, records, counts, cursor, offsets, bases, entries, long_lists, pm, pmc, wzr, w, grid, part_base, partial,
      counters, total, entries_total, max_long;
};

PmLayout3 make_pm_layout3(const Shape& s) {
  PmLayout3 l{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off = align_up(off + bytes, 256);
    return at;
  };
  const size_t g = static_cast<size_t>(s.grid_rows);
  const size_t nl = g * s.lists_per_frame;
  l.entries_total = static_cast<size_t>(s.samples) * s.width * s.width * 2;
  l.flags = take(kFlagBytes);
  l.records = take(static_cast<size_t>(s.samples) * record3_bytes(s.width));
  l.counts = take(nl * 4);
  l.cursor = take(nl * 4);
  l.offsets = take((nl + g) * 4);
  l.bases = take(g * 4);
  l.entries = take(l.entries_total * 4);
  l.long_lists = take((2 + l.entries_total / (s.list_capacity + 1)) * 4);
  l.pm = take(static_cast<size_t>(s.samples) * (16 + 24 * static_cast<size_t>(s.width)));
  l.pmc = take(static_cast<size_t>(s.samples) * (8 + 8 * static_cast<size_t>(s.width)));
  l.wzr = take(l.entries_total * sizeof(double));
  l.w = take(static_cast<size_t>(s.samples) * sizeof(double));
  l.grid = take(g * g * g * sizeof(double));
  // the long lists' parts of kPmPart entries: first part of each list, the
  // parts' sums, one counter per list
  l.max_long = l.entries_total / (static_cast<size_t>(s.list_capacity) + 1) + 2;
  l.part_base = take((l.max_long + 1) * 4);
  l.partial = take((l.entries_total / kPmPart + l.max_long) * kChunk * sizeof(double));
  l.counters = take(l.max_long * 4);
  l.total = off;
  return l;
}

template <int W>
ksj_gpu_status launch_pipe_menon3(const Shape& s, const PmLayout3& l, uint32_t iterations, const float* d_traj,
                                  float* d_dcf, unsigned char* ws, cudaStream_t stream) {
  static_assert(sizeof(PmRecord3<W>) == 16 + 24 * W, "PmRecord3 layout");
  const int g = s.grid_rows;
  uint32_t* flags = reinterpret_cast<uint32_t*>(ws + l.flags);
  if (cudaMemsetAsync(flags, 0, kFlagBytes, stream) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  const ksj_gpu_status st = build_lists3<W>(
      s, KSJ_GPU_DCF_NONE, d_traj, nullptr, flags, ws + l.records, reinterpret_cast<uint32_t*>(ws + l.counts),
      reinterpret_cast<uint32_t*>(ws + l.cursor), reinterpret_cast<uint32_t*>(ws + l.offsets),
      reinterpret_cast<uint32_t*>(ws + l.bases), reinterpret_cast<uint32_t*>(ws + l.entries), nullptr,
      reinterpret_cast<uint32_t*>(ws + l.long_lists), l.entries_total, stream);
  if (st != KSJ_GPU_OK) return st;
  static_assert(sizeof(PmCol3<W>) == 8 + 8 * W, "PmCol3 layout");
  PmRecord3<W>* pm = reinterpret_cast<PmRecord3<W>*>(ws + l.pm);
  PmCol3<W>* pmc = reinterpret_cast<PmCol3<W>*>(ws + l.pmc);
  double* wzr = reinterpret_cast<double*>(ws + l.wzr);
  double* w = reinterpret_cast<double*>(ws + l.w);
  double* grid = reinterpret_cast<double*>(ws + l.grid);
  {
    LaunchScope scope("k_pm_prepare3", stream);
    k_pm_prepare3<W><<<(s.samples + 255) / 256, 256, 0, stream>>>(d_traj, pm, pmc, w, s.samples, g, s.beta,
                                                                 1.0 / std::cyl_bessel_i(0.0, static_cast<double>(s.beta)));
  }
  const uint32_t* offsets = reinterpret_cast<const uint32_t*>(ws + l.offsets);
  const uint32_t* entries = reinterpret_cast<const uint32_t*>(ws + l.entries);
  const uint32_t* long_lists = reinterpret_cast<const uint32_t*>(ws + l.long_lists);
  uint32_t* part_base = reinterpret_cast<uint32_t*>(ws + l.part_base);
  uint32_t* counters = reinterpret_cast<uint32_t*>(ws + l.counters);
  double* partial = reinterpret_cast<double*>(ws + l.partial);
  if (cudaMemsetAsync(counters, 0, l.max_long * 4, stream) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  {
    LaunchScope scope("k_pm_long_parts", stream);
    k_pm_long_parts<<<1, 1024, 0, stream>>>(long_lists, offsets, s.lists_per_frame, part_base);
  }
  const size_t lists = static_cast<size_t>(g) * s.lists_per_frame;
  const unsigned grid_blocks = static_cast<unsigned>((lists * kPmLanes + kPmThreads - 1) / kPmThreads);
  // the long-list parts: a grid-stride loop over six 256-thread blocks per SM
  int device = 0, sms = 0;
  if (cudaGetDevice(&device) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0)
    return KSJ_GPU_ERROR_CUDA;
  const unsigned long_blocks = static_cast<unsigned>(sms) * 6;
  for (uint32_t it = 0; it < iterations; ++it) {
    // the first iteration keeps each entry's plane-row weight product
    {
      LaunchScope scope("k_pm_grid3", stream);
      auto kernel = it == 0 ? k_pm_grid3<W, true> : k_pm_grid3<W, false>;
      kernel<<<grid_blocks, kPmThreads, 0, stream>>>(offsets, entries, pm, pmc, w, wzr, grid, g, s.nchunks,
                                                     s.lists_per_frame, s.list_capacity);
    }
    {
      LaunchScope scope("k_pm_long3", stream);
      auto kernel = it == 0 ? k_pm_long3<W, true> : k_pm_long3<W, false>;
      kernel<<<long_blocks, kPmThreads, 0, stream>>>(long_lists, part_base, offsets, entries, pm, pmc, w, wzr, grid, g,
                                                 s.nchunks, s.lists_per_frame, partial, counters);
    }
    LaunchScope scope("k_pm_update3", stream);
    k_pm_update3<W><<<(s.samples + 255) / 256, 256, 0, stream>>>(pm, grid, w, it + 1 == iterations ? d_dcf : nullptr,
                                                                s.samples, g);
  }
  return check_launch();
}

template <int W>
ksj_gpu_status dispatch_format(const Shape& s, const Layout& l, const ksj_gpu_gridding_desc* d, const void* k,
                               const float* t, const float* w, void* o, unsigned char* ws, cudaStream_t st,
                               const HostIo* io = nullptr) {
  if (d->sample_format == KSJ_GPU_SAMPLES_BF16)
    return launch_all<W, KSJ_GPU_SAMPLES_BF16>(s, l, d, k, t, w, o, ws, st, io);
  return launch_all<W, KSJ_GPU_SAMPLES_CF32>(s, l, d, k, t, w, o, ws, st, io);
}

ksj_gpu_status dispatch_width(const Shape& s, const Layout& l, const ksj_gpu_gridding_desc* d, const void* k,
                              const float* t, const float* w, void* o, unsigned char* ws, cudaStream_t st,
                              const HostIo* io = nullptr) {
  switch (s.width) {
    case 2: return dispatch_format<2>(s, l, d, k, t, w, o, ws, st, io);
    case 4: return dispatch_format<4>(s, l, d, k, t, w, o, ws, st, io);
    case 6: return dispatch_format<6>(s, l, d, k, t, w, o, ws, st, io);
    case 8: return dispatch_format<8>(s, l, d, k, t, w, o, ws, st, io);
    default: return KSJ_GPU_ERROR_UNSUPPORTED;
  }
}

// ------------------------------------------------ Cartesian coil images
//
// cartesian_ifft2_coil_images (providers/kspacejet-cartesian-recon/src/
// operators/cartesian_ifft2_coil_images.cpp:372-407): per channel, the
// inverse 2-D DFT normalised by 1 / (rows cols) (fft2_inplace_with_workspace
// with Direction::inverse and Normalization::inverse: 1/cols on the row pass,
// 1/rows on the column pass, libs/numerics/kspacejet-fft/src/eigen/
// eigen_fft_transforms.cpp:148-205), no shift; channel-major k-space in,
// coil-last images out.  Here: [frame][channel][pixel] ->
// [frame][pixel][channel] (k_transpose), the row transform per (frame, row,
// coil group) (k_cart_rows), then the column pass k_cols with its
// deapodisation factors set to 1/rows and 1/cols and no crop or shift.
// An axis whose length has a prime factor above 7 (no mixed-radix plan; the
// reference's transform takes every length 2..512) is transformed by a
// direct DFT instead: the row form of k_cart_rows, and k_cart_cols_direct
// for the columns (coil-last output, then k_rss for the RSS form).

constexpr int kCartThreads = 256;

// Direct inverse DFT of 2^lg lines of length n held line-contiguous in
// shared memory (element (j, line) at x[(j << lg) + line]): output k of a
// line is sum_j x[j] w^(jk), w = exp(2 pi i / n), with jk reduced mod n
// exactly in integers (tw[t] = w^t) and eight interleaved partial sums
// (rounding error ~ sqrt(n / 8) ulp instead of sqrt(n)).  emit(k, line, v).
template <class Emit>
__device__ __forceinline__ void dft_direct_lines(const float2* x, int lg, int n, const float2* tw, int tid,
                                                 int nthreads, Emit emit) {
  const int lines = 1 << lg;
  for (int o = tid; o < n * lines; o += nthreads) {
    const int k = o >> lg, line = o & (lines - 1);
    float2 s[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) s[u] = make_float2(0.0f, 0.0f);
    int e = 0, j = 0;
    for (; j + 8 <= n; j += 8) {
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const float2 v = x[((j + u) << lg) + line];
        const float2 w = tw[e];
        s[u].x = fmaf(v.x, w.x, fmaf(-v.y, w.y, s[u].x));
        s[u].y = fmaf(v.x, w.y, fmaf(v.y, w.x, s[u].y));
        e += k;
        if (e >= n) e -= n;
      }
    }
    for (int u = 0; j < n; ++j, ++u) {
      const float2 v = x[(j << lg) + line];
      const float2 w = tw[e];
      s[u].x = fmaf(v.x, w.x, fmaf(-v.y, w.y, s[u].x));
      s[u].y = fmaf(v.x, w.y, fmaf(v.y, w.x, s[u].y));
      e += k;
      if (e >= n) e -= n;
    }
    const float re = ((s[0].x + s[1].x) + (s[2].x + s[3].x)) + ((s[4].x + s[5].x) + (s[6].x + s[7].x));
    const float im = ((s[0].y + s[1].y) + (s[2].y + s[3].y)) + ((s[4].y + s[5].y) + (s[6].y + s[7].y));
    emit(k, line, make_float2(re, im));
  }
}

// Twiddles, the normalisation factors and the position of output k of each
// axis's transform (two-step slot or digit-reversed position).
__global__ void k_cart_tables(float2* tw_rows, int rows, float2* tw_cols, int cols, float* inv_dr, float* inv_dc,
                              int* pos_rows, int* pos_cols, DifPlan plan_rows, DifPlan plan_cols) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < rows) {
    tw_rows[i] = twiddle(i, rows);
    inv_dr[i] = 1.0f / static_cast<float>(rows);
    pos_rows[i] = has_two_step_rows(rows) ? two_step_slot(i, rows) : dif_position(plan_rows, i);
  }
  if (i < cols) {
    tw_cols[i] = twiddle(i, cols);
    inv_dc[i] = 1.0f / static_cast<float>(cols);
    pos_cols[i] = dif_position(plan_cols, i);
  }
}

// One block per (frame, row, coil group of cg): the row's cg coil lines
// [column][coil] from the coil-last samples, transformed along the row; every
// column written to [frame][row][column][cpitch].  kN > 0: the two-step
// transform of that length; 0: the mixed-radix plan; -1: the direct DFT.
template <int kN>
__global__ void __launch_bounds__(kCartThreads) k_cart_rows(const float2* __restrict__ coil_last, float2* inter,
                                                            const float2* __restrict__ tw_cols,
                                                            const int* __restrict__ pos_cols, DifPlan plan, int rows,
                                                            int cols, int channels, int cg, int cpitch) {
  extern __shared__ __align__(16) float2 cart_smem[];
  float2* acc = cart_smem;
  float2* tw = cart_smem + static_cast<size_t>(cols) * cg;
  const int row = blockIdx.x, cgi = blockIdx.y, f = blockIdx.z;
  const int lg = ilog2(cg);
  const float2* src = coil_last + (static_cast<size_t>(f) * rows + row) * cols * channels;
  for (int i = threadIdx.x; i < cols * cg; i += blockDim.x) {
    const int col = i >> lg, gc = cgi * cg + (i & (cg - 1));
    acc[i] = gc < channels ? __ldg(src + static_cast<size_t>(col) * channels + gc) : make_float2(0.0f, 0.0f);
  }
  for (int i = threadIdx.x; i < cols; i += blockDim.x) tw[i] = tw_cols[i];
  __syncthreads();
  float2* dst = inter + (static_cast<size_t>(f) * rows + row) * cols * cpitch + cgi * cg;
  const int live = min(cg, channels - cgi * cg);
  auto emit = [&](int k, int line, float2 v) {
    if (line < live) dst[static_cast<size_t>(k) * cpitch + line] = v;
  };
  if constexpr (kN > 0) {
    fft_two_step<16, kN / 16>(acc, lg, tw, threadIdx.x, blockDim.x, emit);
  } else if constexpr (kN < 0) {
    dft_direct_lines(acc, lg, cols, tw, threadIdx.x, blockDim.x, emit);
  } else {
    dif_lines(acc, lg, plan, tw, threadIdx.x, blockDim.x);
    const int c = threadIdx.x & (cg - 1);
    if (c < live)
      for (int k = threadIdx.x >> lg; k < cols; k += blockDim.x >> lg)
        dst[static_cast<size_t>(k) * cpitch + c] = acc[(__ldg(pos_cols + k) << lg) + c];
  }
}

using CartRowsKernel = void (*)(const float2*, float2*, const float2*, const int*, DifPlan, int, int, int, int, int);

CartRowsKernel cart_rows_for(int n) {
  if (!is_fft_size(static_cast<uint32_t>(n))) return k_cart_rows<-1>;
  switch (n) {
    case 128: return k_cart_rows<128>;
    case 192: return k_cart_rows<192>;
    case 256: return k_cart_rows<256>;
    case 384: return k_cart_rows<384>;
    case 512: return k_cart_rows<512>;
    default: return k_cart_rows<0>;
  }
}

// Columns of an axis without a mixed-radix plan: one block per (frame,
// column, coil group of cg): the column's rows x cg lines from the
// row-transformed grid [frame][row][column][cpitch] into shared memory, the
// direct DFT along the rows, each output scaled by (1/rows)(1/cols) and
// written coil-last [frame][row][column][channel].
__global__ void __launch_bounds__(kCartThreads) k_cart_cols_direct(const float2* __restrict__ inter, float2* out,
                                                                   const float2* __restrict__ tw_rows, int rows,
                                                                   int cols, int channels, int cg, int cpitch) {
  extern __shared__ __align__(16) float2 cart_smem[];
  float2* acc = cart_smem;
  float2* tw = cart_smem + static_cast<size_t>(rows) * cg;
  const int col = blockIdx.x, cgi = blockIdx.y, f = blockIdx.z;
  const int lg = ilog2(cg);
  const float2* src = inter + (static_cast<size_t>(f) * rows * cols + col) * cpitch + cgi * cg;
  for (int i = threadIdx.x; i < rows * cg; i += blockDim.x)
    acc[i] = __ldg(src + static_cast<size_t>(i >> lg) * cols * cpitch + (i & (cg - 1)));
  for (int i = threadIdx.x; i < rows; i += blockDim.x) tw[i] = tw_rows[i];
  __syncthreads();
  const float scale = (1.0f / static_cast<float>(rows)) * (1.0f / static_cast<float>(cols));
  const int live = min(cg, channels - cgi * cg);
  float2* dst = out + static_cast<size_t>(f) * rows * cols * channels + static_cast<size_t>(col) * channels + cgi * cg;
  dft_direct_lines(acc, lg, rows, tw, threadIdx.x, blockDim.x, [&](int k, int line, float2 v) {
    if (line < live)
      dst[static_cast<size_t>(k) * cols * channels + line] = make_float2(v.x * scale, v.y * scale);
  });
}

// The shape of a Cartesian call as the column pass reads it.
struct CartShape {
  Shape s;
  int cg;  // coils per row block
  size_t flags, coil_last, inter, tables, total;
};

ksj_gpu_status make_cart_shape(uint32_t rows, uint32_t cols, uint32_t channels, uint32_t frames, CartShape* c) {
  if (rows < 2 || cols < 2 || channels == 0 || channels > 64 || frames == 0) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (rows > kMaxGrid || cols > kMaxGrid) return KSJ_GPU_ERROR_UNSUPPORTED;
  Shape& s = c->s;
  s = Shape{};
  s.frames = static_cast<int>(frames);
  s.channels = static_cast<int>(channels);
  s.rows = s.grid_rows = s.out_rows = static_cast<int>(rows);
  s.cols = s.grid_cols = s.out_cols = static_cast<int>(cols);
  s.col_group = 2;
  while (s.col_group < s.channels && s.col_group < 32) s.col_group <<= 1;
  s.cpitch = (s.channels + s.col_group - 1) / s.col_group * s.col_group;
  const int cgroups = s.cpitch / s.col_group;
  auto tile = [&](int b) {
    return static_cast<size_t>(s.grid_rows) * b * s.col_group * sizeof(float2) * (cgroups > 1 ? 2 : 1);
  };
  int cb = std::max(1, 32 / s.col_group);
  if (is_fft_size(rows)) {  // the column pass k_cols and its tile
    while (cb > 1 && (tile(cb) > 110 * 1024 || cb > s.out_cols)) cb >>= 1;
    if (tile(cb) > 200 * 1024) return KSJ_GPU_ERROR_UNSUPPORTED;
  } else {
    cb = 1;
  }
  s.column_block = cb;
  s.frames_per_pass = s.frames;
  // an axis without a mixed-radix plan (direct DFT) keeps an empty plan
  if (!make_dif_plan(s.grid_rows, &s.plan_rows)) s.plan_rows = DifPlan{s.grid_rows, 0, {}, {}, {}, {}, {}};
  if (!make_dif_plan(s.grid_cols, &s.plan_cols)) s.plan_cols = DifPlan{s.grid_cols, 0, {}, {}, {}, {}, {}};
  c->cg = s.col_group;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off = align_up(off + bytes, 256);
    return at;
  };
  const size_t px = static_cast<size_t>(frames) * rows * cols;
  c->flags = take(kFlagBytes);
  c->coil_last = take(px * channels * sizeof(float2));
  c->inter = take(px * s.cpitch * sizeof(float2));
  c->tables = take((static_cast<size_t>(rows) + cols) * (sizeof(float2) + sizeof(float) + sizeof(int)));
  c->total = off;
  return KSJ_GPU_OK;
}

// Workspace of the host-buffer entry point: the device workspace, then the
// device copies of the samples, trajectory, density weights and images.
struct HostLayout {
  Layout dev;
  size_t kspace, traj, dcf, out, total;
};

size_t image_frame_bytes(const Shape& s, const ksj_gpu_gridding_desc* d) {
  const size_t px = static_cast<size_t>(s.out_rows) * s.out_cols;
  return d->output == KSJ_GPU_OUTPUT_RSS ? px * sizeof(float) : px * s.channels * sizeof(float2);
}

HostLayout make_host_layout(const Shape& s, const ksj_gpu_gridding_desc* d) {
  HostLayout h{};
  h.dev = make_layout(s, d);
  size_t off = h.dev.total;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off = align_up(off + bytes, 256);
    return at;
  };
  const size_t fm = static_cast<size_t>(s.frames) * s.samples;
  h.kspace = take(fm * s.channels * sample_bytes(d->sample_format));
  h.traj = take(fm * 2 * sizeof(float));
  h.dcf = d->dcf_mode == KSJ_GPU_DCF_EXTERNAL ? take(fm * sizeof(float)) : off;
  h.out = take(static_cast<size_t>(s.frames) * image_frame_bytes(s, d));
  h.total = off;
  return h;
}

// Non-blocking streams per device for the host-buffer entry point: which 0
// carries the copies, which 1 the odd frame passes.
cudaStream_t side_stream(int device, int which) {
  static std::mutex m;
  static std::map<std::pair<int, int>, cudaStream_t> streams;
  std::lock_guard<std::mutex> lock(m);
  auto it = streams.find({device, which});
  if (it != streams.end()) return it->second;
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
  streams[{device, which}] = st;
  return st;
}

}  // namespace
}  // namespace ksj_gpu

using namespace ksj_gpu;

extern "C" size_t ksj_gpu_gridding_workspace_bytes(const ksj_gpu_gridding_desc* desc) {
  Shape s{};
  if (make_shape(desc, nullptr, &s) != KSJ_GPU_OK) return 0;
  return make_layout(s, desc).total;
}

extern "C" size_t ksj_gpu_gridding_frame_flags_offset(const ksj_gpu_gridding_desc* desc) {
  Shape s{};
  if (make_shape(desc, nullptr, &s) != KSJ_GPU_OK) return 0;
  return make_layout(s, desc).frame_flags;
}

namespace {
// The adjoint of a uniform batch (ragged null) or a ragged one (per-frame
// counts and input addresses; d_kspace and d_traj unused).
struct Ragged {
  const uint32_t* channels;
  const uint32_t* samples;
  const uint64_t* kspace;
  const uint64_t* traj;
};

ksj_gpu_status gridding_adjoint(const ksj_gpu_gridding_desc* desc, const ksj_gpu_gridding_tuning* tuning,
                                const Ragged* ragged, const void* d_kspace, const float* d_traj, const float* d_dcf,
                                void* d_out, void* d_workspace, size_t workspace_bytes, void* stream) {
  Shape s{};
  const ksj_gpu_status st = make_shape(desc, tuning, &s);
  if (st != KSJ_GPU_OK) return st;
  if (ragged != nullptr) {
    s.frame_channels = ragged->channels;
    s.frame_samples = ragged->samples;
    s.frame_kspace = ragged->kspace;
    s.frame_traj = ragged->traj;
  } else if (d_kspace == nullptr || d_traj == nullptr) {
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  }
  if (d_out == nullptr) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (desc->dcf_mode == KSJ_GPU_DCF_EXTERNAL && d_dcf == nullptr) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  const Layout l = make_layout(s, desc);
  if (d_workspace == nullptr || (reinterpret_cast<uintptr_t>(d_workspace) & 255u) != 0 || workspace_bytes < l.total)
    return KSJ_GPU_ERROR_WORKSPACE;
  if ((reinterpret_cast<uintptr_t>(d_kspace) & (sample_bytes(desc->sample_format) - 1)) != 0 ||
      (reinterpret_cast<uintptr_t>(d_traj) & 7u) != 0 || (reinterpret_cast<uintptr_t>(d_out) & 7u) != 0)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  unsigned char* ws = static_cast<unsigned char*>(d_workspace);
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  if (s.frames_per_pass >= s.frames) return dispatch_width(s, l, desc, d_kspace, d_traj, d_dcf, d_out, ws, cs);
  // several passes: odd ones on the second compute stream
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  cudaStream_t alt = side_stream(device, 1);
  cudaEvent_t ready = nullptr, alt_done = nullptr;
  if (alt == nullptr || cudaEventCreateWithFlags(&ready, cudaEventDisableTiming) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  if (cudaEventCreateWithFlags(&alt_done, cudaEventDisableTiming) != cudaSuccess) {
    cudaEventDestroy(ready);
    return KSJ_GPU_ERROR_CUDA;
  }
  const HostIo io{nullptr, alt, nullptr, nullptr, ready, alt_done, nullptr, 0};
  const ksj_gpu_status result = dispatch_width(s, l, desc, d_kspace, d_traj, d_dcf, d_out, ws, cs, &io);
  cudaEventDestroy(ready);
  cudaEventDestroy(alt_done);
  return result;
}
}  // namespace

extern "C" ksj_gpu_status ksj_gpu_gridding_adjoint(const ksj_gpu_gridding_desc* desc,
                                                   const ksj_gpu_gridding_tuning* tuning, const void* d_kspace,
                                                   const float* d_traj, const float* d_dcf, void* d_out,
                                                   void* d_workspace, size_t workspace_bytes, void* stream) {
  return gridding_adjoint(desc, tuning, nullptr, d_kspace, d_traj, d_dcf, d_out, d_workspace, workspace_bytes, stream);
}

extern "C" ksj_gpu_status ksj_gpu_gridding_adjoint_ragged(const ksj_gpu_gridding_desc* desc,
                                                          const ksj_gpu_gridding_tuning* tuning,
                                                          const uint32_t* d_frame_channels,
                                                          const uint32_t* d_frame_samples,
                                                          const uint64_t* d_frame_kspace,
                                                          const uint64_t* d_frame_traj, void* d_out,
                                                          void* d_workspace, size_t workspace_bytes, void* stream) {
  if (d_frame_channels == nullptr || d_frame_samples == nullptr || d_frame_kspace == nullptr ||
      d_frame_traj == nullptr)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (desc == nullptr || desc->struct_size < sizeof(ksj_gpu_gridding_desc) ||
      desc->kernel != KSJ_GPU_KERNEL_KAISER_BESSEL || desc->dcf_mode == KSJ_GPU_DCF_EXTERNAL)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  const Ragged r{d_frame_channels, d_frame_samples, d_frame_kspace, d_frame_traj};
  return gridding_adjoint(desc, tuning, &r, nullptr, nullptr, nullptr, d_out, d_workspace, workspace_bytes, stream);
}

extern "C" size_t ksj_gpu_gridding_host_workspace_bytes(const ksj_gpu_gridding_desc* desc) {
  Shape s{};
  if (make_shape(desc, nullptr, &s) != KSJ_GPU_OK) return 0;
  return make_host_layout(s, desc).total;
}

extern "C" ksj_gpu_status ksj_gpu_gridding_adjoint_host(const ksj_gpu_gridding_desc* desc,
                                                        const ksj_gpu_gridding_tuning* tuning, const void* h_kspace,
                                                        const float* h_traj, const float* h_dcf, void* h_out,
                                                        void* d_workspace, size_t workspace_bytes, void* stream) {
  Shape s{};
  const ksj_gpu_status st = make_shape(desc, tuning, &s);
  if (st != KSJ_GPU_OK) return st;
  if (h_kspace == nullptr || h_traj == nullptr || h_out == nullptr) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (desc->dcf_mode == KSJ_GPU_DCF_EXTERNAL && h_dcf == nullptr) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  // copies and passes overlap: at least 8 passes (fewer leave more of the
  // first copy exposed; with odd passes on a second stream, 8 measured best
  // for 96 frames); a tuning with smaller passes keeps them
  s.frames_per_pass = std::min(s.frames_per_pass, std::max(1, (s.frames + 7) / 8));
  const HostLayout h = make_host_layout(s, desc);
  if (d_workspace == nullptr || (reinterpret_cast<uintptr_t>(d_workspace) & 255u) != 0 || workspace_bytes < h.total)
    return KSJ_GPU_ERROR_WORKSPACE;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  cudaStream_t copy = side_stream(device, 0), alt = side_stream(device, 1);
  if (copy == nullptr || alt == nullptr) return KSJ_GPU_ERROR_CUDA;
  unsigned char* ws = static_cast<unsigned char*>(d_workspace);
  const size_t fm = static_cast<size_t>(s.frames) * s.samples;
  const size_t frame_bytes = static_cast<size_t>(s.samples) * s.channels * sample_bytes(desc->sample_format);
  const int passes = (s.frames + s.frames_per_pass - 1) / s.frames_per_pass;
  std::vector<cudaEvent_t> events(static_cast<size_t>(2 * passes + 4), nullptr);
  auto release = [&]() {
    for (cudaEvent_t e : events)
      if (e != nullptr) cudaEventDestroy(e);
  };
  for (cudaEvent_t& e : events)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      release();
      return KSJ_GPU_ERROR_CUDA;
    }
  cudaEvent_t* in = events.data();
  cudaEvent_t* done = in + passes;
  cudaEvent_t start = done[passes], end = done[passes + 1], ready = done[passes + 2], alt_done = done[passes + 3];
  ksj_gpu_status result = KSJ_GPU_OK;
  // the trajectory (and weights) first, on the stream, for the binning; the
  // copy stream starts after everything already queued on the stream (the
  // staging buffers may still be read by an earlier call)
  if (cudaMemcpyAsync(ws + h.traj, h_traj, fm * 2 * sizeof(float), cudaMemcpyHostToDevice, cs) != cudaSuccess ||
      (desc->dcf_mode == KSJ_GPU_DCF_EXTERNAL &&
       cudaMemcpyAsync(ws + h.dcf, h_dcf, fm * sizeof(float), cudaMemcpyHostToDevice, cs) != cudaSuccess) ||
      cudaEventRecord(start, cs) != cudaSuccess || cudaStreamWaitEvent(copy, start, 0) != cudaSuccess)
    result = KSJ_GPU_ERROR_CUDA;
  for (int p = 0; p < passes && result == KSJ_GPU_OK; ++p) {
    const int f0 = p * s.frames_per_pass, nf = std::min(s.frames_per_pass, s.frames - f0);
    if (cudaMemcpyAsync(ws + h.kspace + f0 * frame_bytes, static_cast<const unsigned char*>(h_kspace) + f0 * frame_bytes,
                        static_cast<size_t>(nf) * frame_bytes, cudaMemcpyHostToDevice, copy) != cudaSuccess ||
        cudaEventRecord(in[p], copy) != cudaSuccess)
      result = KSJ_GPU_ERROR_CUDA;
  }
  if (result == KSJ_GPU_OK) {
    const HostIo io{copy, alt, in, done, ready, alt_done, h_out, image_frame_bytes(s, desc)};
    result = dispatch_width(s, h.dev, desc, ws + h.kspace, reinterpret_cast<const float*>(ws + h.traj),
                            desc->dcf_mode == KSJ_GPU_DCF_EXTERNAL ? reinterpret_cast<const float*>(ws + h.dcf)
                                                                   : nullptr,
                            ws + h.out, ws, cs, &io);
  }
  // the stream completes only after the last image copy
  if (cudaEventRecord(end, copy) != cudaSuccess || cudaStreamWaitEvent(cs, end, 0) != cudaSuccess)
    if (result == KSJ_GPU_OK) result = KSJ_GPU_ERROR_CUDA;
  release();
  return result;
}

extern "C" ksj_gpu_status ksj_gpu_gridding_binning(const ksj_gpu_gridding_desc* desc,
                                                   const ksj_gpu_gridding_tuning* tuning, const void* d_workspace,
                                                   uint32_t* out_chunk_width, uint64_t* out_list_count,
                                                   uint64_t* out_entry_count, uint64_t* out_offsets,
                                                   uint32_t* out_samples) {
  Shape s{};
  const ksj_gpu_status st = make_shape(desc, tuning, &s);
  if (st != KSJ_GPU_OK) return st;
  if (d_workspace == nullptr) return KSJ_GPU_ERROR_WORKSPACE;
  const Layout l = make_layout(s, desc);
  const unsigned char* ws = static_cast<const unsigned char*>(d_workspace);
  const size_t lists = static_cast<size_t>(s.frames) * s.lists_per_frame;
  if (out_chunk_width) *out_chunk_width = kChunk;
  if (out_list_count) *out_list_count = lists;
  std::vector<uint32_t> off(static_cast<size_t>(s.frames) * (s.lists_per_frame + 1));
  if (cudaDeviceSynchronize() != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  if (cudaMemcpy(off.data(), ws + l.offsets, off.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return KSJ_GPU_ERROR_CUDA;
  uint64_t total = 0;
  for (int f = 0; f < s.frames; ++f) total += off[static_cast<size_t>(f) * (s.lists_per_frame + 1) + s.lists_per_frame];
  if (out_entry_count) *out_entry_count = total;
  if (out_offsets == nullptr || out_samples == nullptr) return KSJ_GPU_OK;
  uint64_t base = 0;
  for (int f = 0; f < s.frames; ++f) {
    const uint32_t* fo = off.data() + static_cast<size_t>(f) * (s.lists_per_frame + 1);
    for (int i = 0; i < s.lists_per_frame; ++i)
      out_offsets[static_cast<size_t>(f) * s.lists_per_frame + i] = base + fo[i];
    // the sample index of every expanded entry (second word of its first vector)
    const uint32_t n = fo[s.lists_per_frame];
    const size_t entry_bytes = static_cast<size_t>(meta_vecs(s.width)) * 16;
    if (n && cudaMemcpy2D(out_samples + base, 4, ws + l.expanded + static_cast<size_t>(f) * s.entries_per_frame * entry_bytes + 4,
                          entry_bytes, 4, n, cudaMemcpyDeviceToHost) != cudaSuccess)
      return KSJ_GPU_ERROR_CUDA;
    base += n;
  }
  out_offsets[lists] = base;
  return KSJ_GPU_OK;
}

extern "C" ksj_gpu_status ksj_gpu_read_flags(const void* d_workspace, void* stream, uint32_t* out_flags) {
  if (d_workspace == nullptr || out_flags == nullptr) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  if (cudaStreamSynchronize(cs) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  if (cudaMemcpy(out_flags, d_workspace, sizeof(uint32_t), cudaMemcpyDeviceToHost) != cudaSuccess)
    return KSJ_GPU_ERROR_CUDA;
  return KSJ_GPU_OK;
}

namespace {
std::mutex g_tune_mutex;
// keyed by the shape and the device: a tuning is chosen against one device's
// shared-memory and SM limits
std::map<std::tuple<int, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t, uint32_t,
                    uint32_t, uint32_t>,
         ksj_gpu_gridding_tuning>
    g_tune_cache;
}  // namespace

extern "C" ksj_gpu_status ksj_gpu_gridding_tune(const ksj_gpu_gridding_desc* desc, const void* d_kspace,
                                                const float* d_traj, const float* d_dcf, void* d_out,
                                                void* d_workspace, size_t workspace_bytes, void* stream,
                                                ksj_gpu_gridding_tuning* tuning) {
  if (desc == nullptr || tuning == nullptr) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  const auto key = std::make_tuple(device, desc->kernel, desc->image_rows, desc->image_cols, desc->grid_rows,
                                   desc->grid_cols, desc->kernel_width, desc->channels, desc->samples, desc->frames,
                                   desc->output, desc->sample_format);
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    const auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      *tuning = it->second;
      return KSJ_GPU_OK;
    }
  }
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return KSJ_GPU_ERROR_CUDA;
  }
  ksj_gpu_gridding_tuning best{};
  float best_ms = 1e30f;
  for (uint32_t cg : {32u, 16u, 8u, 4u, 2u, 1u}) {
    if (cg > 1 && cg / 2 >= desc->channels) continue;
    if (cg * 4 < desc->channels && cg < 8) continue;
    for (uint32_t cbm : {1u, 2u})
    for (uint32_t fpp : {0u, 12u, 48u})
    for (uint32_t rb : {1u, 2u})
    for (uint32_t colp : {1u, 2u})
    for (uint32_t parts : {1u, 2u}) {
      if (fpp >= desc->frames) continue;
      if (parts > 1 && cg < 16) continue;
      ksj_gpu_gridding_tuning t{};
      t.struct_size = sizeof(t);
      uint32_t gcols = 2;
      while (gcols < desc->channels && gcols < 32) gcols <<= 1;
      t.coil_group = cg;
      t.column_block = cbm * std::max(1u, 32u / gcols);
      t.frames_per_pass = fpp;
      t.rows_blocks_per_sm = rb;
      t.coil_parts = parts;
      t.column_pass = colp;
      Shape s{};
      if (make_shape(desc, &t, &s) != KSJ_GPU_OK) continue;
      if (workspace_bytes < make_layout(s, desc).total) continue;
      if (ksj_gpu_gridding_adjoint(desc, &t, d_kspace, d_traj, d_dcf, d_out, d_workspace, workspace_bytes, stream) !=
          KSJ_GPU_OK)
        continue;
      cudaEventRecord(e0, cs);
      for (int rep = 0; rep < 2; ++rep)
        ksj_gpu_gridding_adjoint(desc, &t, d_kspace, d_traj, d_dcf, d_out, d_workspace, workspace_bytes, stream);
      cudaEventRecord(e1, cs);
      if (cudaEventSynchronize(e1) != cudaSuccess) break;
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best_ms) {
        best_ms = ms;
        best = t;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best.struct_size == 0) return KSJ_GPU_ERROR_UNSUPPORTED;
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[key] = best;
  }
  *tuning = best;
  return KSJ_GPU_OK;
}

extern "C" size_t ksj_gpu_pipe_menon_workspace_bytes(const ksj_gpu_gridding_desc* desc) {
  Shape s{};
  if (desc == nullptr || desc->kernel != KSJ_GPU_KERNEL_KAISER_BESSEL || make_shape(desc, nullptr, &s) != KSJ_GPU_OK)
    return 0;
  return make_pm_layout(s).total;
}

extern "C" ksj_gpu_status ksj_gpu_pipe_menon_dcf(const ksj_gpu_gridding_desc* desc, uint32_t iterations,
                                                 const float* d_traj, float* d_dcf, void* d_workspace,
                                                 size_t workspace_bytes, void* stream) {
  if (desc == nullptr || desc->kernel != KSJ_GPU_KERNEL_KAISER_BESSEL || iterations == 0 || iterations > 1000)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  Shape s{};
  const ksj_gpu_status st = make_shape(desc, nullptr, &s);
  if (st != KSJ_GPU_OK) return st;
  if (d_traj == nullptr || d_dcf == nullptr || (reinterpret_cast<uintptr_t>(d_traj) & 7u) != 0 ||
      (reinterpret_cast<uintptr_t>(d_dcf) & 3u) != 0)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  const PmLayout l = make_pm_layout(s);
  if (d_workspace == nullptr || (reinterpret_cast<uintptr_t>(d_workspace) & 255u) != 0 || workspace_bytes < l.total)
    return KSJ_GPU_ERROR_WORKSPACE;
  unsigned char* ws = static_cast<unsigned char*>(d_workspace);
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  switch (s.width) {
    case 2: return launch_pipe_menon<2>(s, l, desc, iterations, d_traj, d_dcf, ws, cs);
    case 4: return launch_pipe_menon<4>(s, l, desc, iterations, d_traj, d_dcf, ws, cs);
    case 6: return launch_pipe_menon<6>(s, l, desc, iterations, d_traj, d_dcf, ws, cs);
    case 8: return launch_pipe_menon<8>(s, l, desc, iterations, d_traj, d_dcf, ws, cs);
    default: return KSJ_GPU_ERROR_UNSUPPORTED;
  }
}

extern "C" size_t ksj_gpu_gridding3_workspace_bytes(const ksj_gpu_gridding3_desc* desc) {
  Shape s{};
  if (make_shape3(desc, nullptr, &s) != KSJ_GPU_OK) return 0;
  return make_layout3(s, desc->sample_format).total;
}

extern "C" ksj_gpu_status ksj_gpu_gridding3_adjoint(const ksj_gpu_gridding3_desc* desc,
                                                    const ksj_gpu_gridding_tuning* tuning, const void* d_kspace,
                                                    const float* d_traj, const float* d_dcf, void* d_out,
                                                    void* d_workspace, size_t workspace_bytes, void* stream) {
  Shape s{};
  const ksj_gpu_status st = make_shape3(desc, tuning, &s);
  if (st != KSJ_GPU_OK) return st;
  if (d_kspace == nullptr || d_traj == nullptr || d_out == nullptr) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (desc->dcf_mode == KSJ_GPU_DCF_EXTERNAL && d_dcf == nullptr) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  const Layout3 l = make_layout3(s, desc->sample_format);
  if (l.entries_total > 0xffffffffull) return KSJ_GPU_ERROR_UNSUPPORTED;
  if (d_workspace == nullptr || (reinterpret_cast<uintptr_t>(d_workspace) & 255u) != 0 || workspace_bytes < l.total)
    return KSJ_GPU_ERROR_WORKSPACE;
  if ((reinterpret_cast<uintptr_t>(d_kspace) & (sample_bytes(desc->sample_format) - 1)) != 0 ||
      (reinterpret_cast<uintptr_t>(d_traj) & 3u) != 0 || (reinterpret_cast<uintptr_t>(d_out) & 7u) != 0)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  unsigned char* ws = static_cast<unsigned char*>(d_workspace);
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  const bool bf16 = desc->sample_format == KSJ_GPU_SAMPLES_BF16;
  switch (s.width) {
#define KSJ_G3_CASE(W)                                                                                       \
  case W:                                                                                                    \
    return bf16 ? launch_all3<W, KSJ_GPU_SAMPLES_BF16>(s, l, desc, d_kspace, d_traj, d_dcf, d_out, ws, cs)     \
                : launch_all3<W, KSJ_GPU_SAMPLES_CF32>(s, l, desc, d_kspace, d_traj, d_dcf, d_out, ws, cs);
    KSJ_G3_CASE(2) KSJ_G3_CASE(4) KSJ_G3_CASE(6) KSJ_G3_CASE(8)
#undef KSJ_G3_CASE
    default: return KSJ_GPU_ERROR_UNSUPPORTED;
  }
}

extern "C" size_t ksj_gpu_pipe_menon3_workspace_bytes(const ksj_gpu_gridding3_desc* desc) {
  Shape s{};
  if (make_shape3(desc, nullptr, &s) != KSJ_GPU_OK) return 0;
  return make_pm_layout3(s).total;
}

extern "C" ksj_gpu_status ksj_gpu_pipe_menon_dcf3(const ksj_gpu_gridding3_desc* desc, uint32_t iterations,
                                                  const float* d_traj, float* d_dcf, void* d_workspace,
                                                  size_t workspace_bytes, void* stream) {
  if (iterations == 0 || iterations > 1000) return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  Shape s{};
  const ksj_gpu_status st = make_shape3(desc, nullptr, &s);
  if (st != KSJ_GPU_OK) return st;
  if (d_traj == nullptr || d_dcf == nullptr || (reinterpret_cast<uintptr_t>(d_traj) & 3u) != 0 ||
      (reinterpret_cast<uintptr_t>(d_dcf) & 3u) != 0)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  const PmLayout3 l = make_pm_layout3(s);
  if (l.entries_total > 0xffffffffull) return KSJ_GPU_ERROR_UNSUPPORTED;
  if (d_workspace == nullptr || (reinterpret_cast<uintptr_t>(d_workspace) & 255u) != 0 || workspace_bytes < l.total)
    return KSJ_GPU_ERROR_WORKSPACE;
  unsigned char* ws = static_cast<unsigned char*>(d_workspace);
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  switch (s.width) {
    case 2: return launch_pipe_menon3<2>(s, l, iterations, d_traj, d_dcf, ws, cs);
    case 4: return launch_pipe_menon3<4>(s, l, iterations, d_traj, d_dcf, ws, cs);
    case 6: return launch_pipe_menon3<6>(s, l, iterations, d_traj, d_dcf, ws, cs);
    case 8: return launch_pipe_menon3<8>(s, l, iterations, d_traj, d_dcf, ws, cs);
    default: return KSJ_GPU_ERROR_UNSUPPORTED;
  }
}

extern "C" size_t ksj_gpu_cartesian_workspace_bytes(uint32_t rows, uint32_t cols, uint32_t channels,
                                                    uint32_t frames) {
  CartShape c{};
  return make_cart_shape(rows, cols, channels, frames, &c) == KSJ_GPU_OK ? c.total : 0;
}

extern "C" ksj_gpu_status ksj_gpu_cartesian_ifft2(uint32_t rows, uint32_t cols, uint32_t channels, uint32_t frames,
                                                  uint32_t output, const void* d_kspace, void* d_out,
                                                  void* d_workspace, size_t workspace_bytes, void* stream) {
  CartShape cs{};
  const ksj_gpu_status st = make_cart_shape(rows, cols, channels, frames, &cs);
  if (st != KSJ_GPU_OK) return st;
  if (d_kspace == nullptr || d_out == nullptr || (output != KSJ_GPU_OUTPUT_COIL_LAST && output != KSJ_GPU_OUTPUT_RSS) ||
      (reinterpret_cast<uintptr_t>(d_kspace) & 7u) != 0 || (reinterpret_cast<uintptr_t>(d_out) & 7u) != 0)
    return KSJ_GPU_ERROR_INVALID_ARGUMENT;
  if (d_workspace == nullptr || (reinterpret_cast<uintptr_t>(d_workspace) & 255u) != 0 || workspace_bytes < cs.total)
    return KSJ_GPU_ERROR_WORKSPACE;
  const Shape& s = cs.s;
  cudaStream_t cstream = static_cast<cudaStream_t>(stream);
  unsigned char* ws = static_cast<unsigned char*>(d_workspace);
  uint32_t* flags = reinterpret_cast<uint32_t*>(ws + cs.flags);
  float2* coil_last = reinterpret_cast<float2*>(ws + cs.coil_last);
  float2* inter = reinterpret_cast<float2*>(ws + cs.inter);
  float2* tw_rows = reinterpret_cast<float2*>(ws + cs.tables);
  float2* tw_cols = tw_rows + rows;
  float* inv_dr = reinterpret_cast<float*>(tw_cols + cols);
  float* inv_dc = inv_dr + rows;
  int* pos_rows = reinterpret_cast<int*>(inv_dc + cols);
  int* pos_cols = pos_rows + rows;
  if (cudaMemsetAsync(flags, 0, kFlagBytes, cstream) != cudaSuccess) return KSJ_GPU_ERROR_CUDA;
  {
    const int n = static_cast<int>(std::max(rows, cols));
    LaunchScope scope("k_cart_tables", cstream);
    k_cart_tables<<<(n + 255) / 256, 256, 0, cstream>>>(tw_rows, static_cast<int>(rows), tw_cols,
                                                       static_cast<int>(cols), inv_dr, inv_dc, pos_rows, pos_cols,
                                                       s.plan_rows, s.plan_cols);
  }
  {
    // [frame][channel][pixel] -> [frame][pixel][channel]
    const int pixels = static_cast<int>(rows * cols);
    const dim3 tg((pixels + 31) / 32, (channels + 31) / 32, frames);
    LaunchScope scope("k_kspace_coil_last", cstream);
    k_transpose<unsigned long long><<<tg, dim3(32, 8), 0, cstream>>>(
        static_cast<const unsigned long long*>(d_kspace), reinterpret_cast<unsigned long long*>(coil_last),
        static_cast<int>(channels), pixels);
  }
  {
    const CartRowsKernel rk = cart_rows_for(static_cast<int>(cols));
    const size_t smem = (static_cast<size_t>(cols) * cs.cg + cols) * sizeof(float2);
    if (cudaFuncSetAttribute(rk, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) != cudaSuccess)
      return KSJ_GPU_ERROR_CUDA;
    const dim3 grid(rows, (channels + cs.cg - 1) / cs.cg, frames);
    LaunchScope scope("k_cart_rows", cstream);
    rk<<<grid, kCartThreads, smem, cstream>>>(coil_last, inter, tw_cols, pos_cols, s.plan_cols, static_cast<int>(rows),
                                             static_cast<int>(cols), static_cast<int>(channels), cs.cg, s.cpitch);
  }
  if (!is_fft_size(rows)) {
    // direct DFT along the columns, coil-last into the output (or into the
    // consumed coil-last buffer, then its RSS)
    float2* dst = output == KSJ_GPU_OUTPUT_COIL_LAST ? static_cast<float2*>(d_out) : coil_last;
    const size_t smem = (static_cast<size_t>(rows) * cs.cg + rows) * sizeof(float2);
    if (cudaFuncSetAttribute(k_cart_cols_direct, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem)) != cudaSuccess)
      return KSJ_GPU_ERROR_CUDA;
    {
      const dim3 grid(cols, (channels + cs.cg - 1) / cs.cg, frames);
      LaunchScope scope("k_cart_cols_direct", cstream);
      k_cart_cols_direct<<<grid, kCartThreads, smem, cstream>>>(inter, dst, tw_rows, static_cast<int>(rows),
                                                               static_cast<int>(cols), static_cast<int>(channels),
                                                               cs.cg, s.cpitch);
    }
    if (output == KSJ_GPU_OUTPUT_RSS) {
      const ksj_gpu_status rs = check_launch();
      if (rs != KSJ_GPU_OK) return rs;
      return ksj_gpu_rss_coil_last(static_cast<uint64_t>(frames) * rows * cols, channels, coil_last,
                                   static_cast<float*>(d_out), stream);
    }
    return check_launch();
  }
  ColsArgs c{};
  c.tw_rows = tw_rows;
  c.inv_dr = inv_dr;
  c.inv_dc = inv_dc;
  c.pos_rows = pos_rows;
  c.flags = flags;
  c.frames = s.frames;
  c.channels = s.channels;
  c.grid_rows = s.grid_rows;
  c.out_rows = s.out_rows;
  c.out_cols = s.out_cols;
  c.kb = 1;  // apply the factors: here the normalisation
  c.row_shift = 0;
  c.column_block = s.column_block;
  c.col_group = s.col_group;
  c.groups = s.cpitch / s.col_group;
  c.plan = s.plan_rows;
  c.output = output;
  c.out = d_out;
  c.out_pitch = s.channels;
  c.frame0 = 0;
  ColsPass cols_pass;
  if (!cols_pass.setup(s, inter, &c)) return KSJ_GPU_ERROR_CUDA;
  cols_pass.launch(c, s.frames, cstream, "k_cols");
  return check_launch();
}
