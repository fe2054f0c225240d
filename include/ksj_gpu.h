/*
 * ksj_gpu.h -- the thin C ABI over the sm_103a kernels of the non-Cartesian
 * reconstruction path.  Plain pointers and sizes only; every pointer named
 * `d_*` is device memory of the current CUDA device, `stream` is a
 * cudaStream_t (NULL = legacy default stream).  Nothing here allocates device
 * memory except the ksj_gpu_context helpers, which are a convenience for hosts
 * (the Provider plug-ins) that do not manage their own workspace.
 *
 * Every function returns a ksj_gpu_status.  There is no CPU fallback: a
 * missing or failing device is reported, never emulated.
 *
 * Reference interfaces replaced (paths relative to the KSpaceJet tree):
 *   ksj_gpu_gridding_adjoint with KSJ_GPU_KERNEL_LINEAR
 *       <- ksj::nufft::radial_analytic_ramp_dcf2 +
 *          ksj::nufft::radial_linear_gridding2_adjoint, per channel
 *          (libs/numerics/kspacejet-nufft/include/kspacejet/nufft/radial_gridding.hpp:33-37, 59-70)
 *          and the per-channel loop + coil-last scatter of
 *          providers/kspacejet-noncartesian-recon/src/operators/radial_gridding_reconstruct.cpp:394-413
 *   ksj_gpu_gridding_adjoint with KSJ_GPU_KERNEL_KAISER_BESSEL
 *       <- no reference counterpart (new operator radial_kb_gridding_reconstruct)
 *   ksj_gpu_direct_adjoint
 *       <- ksj::nufft::direct_nudft2_adjoint, per channel
 *          (libs/numerics/kspacejet-nufft/include/kspacejet/nufft/direct_nudft.hpp:62-69) and
 *          providers/kspacejet-noncartesian-recon/src/operators/noncartesian_adjoint_reconstruct.cpp:352-368
 *   ksj_gpu_direct_forward
 *       <- ksj::nufft::direct_nudft2_forward / nufft2_forward on the Eigen backend, per channel
 *          (libs/numerics/kspacejet-nufft/include/kspacejet/nufft/direct_nudft.hpp:14-21, src/nufft.cpp:29)
 *   ksj_gpu_cartesian_ifft2
 *       <- providers/kspacejet-cartesian-recon/src/operators/cartesian_ifft2_coil_images.cpp:372-407
 *   ksj_gpu_normalize_trajectory, ksj_gpu_aggregate_acquisitions
 *       <- libs/recon/kspacejet-recon-runtime/src/noncartesian_rss_hdf5.cpp:776-833, 1077-1103
 *   ksj_gpu_rss_coil_last
 *       <- ksj::stats::root_sum_of_squares_across(cube, image, Dim::dim2)
 *          (libs/numerics/kspacejet-stats/include/kspacejet/stats/norms.hpp:207-218) as called by
 *          providers/kspacejet-coil-combine/src/operators/coil_combine_rss.cpp:303-308
 */
#ifndef KSJ_GPU_H_
#define KSJ_GPU_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define KSJ_GPU_API __attribute__((visibility("default")))
#else
#define KSJ_GPU_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t ksj_gpu_status;
#define KSJ_GPU_OK 0
#define KSJ_GPU_ERROR_INVALID_ARGUMENT 1  /* a size, pointer or mode outside the documented envelope */
#define KSJ_GPU_ERROR_UNSUPPORTED 2       /* a combination this build does not implement */
#define KSJ_GPU_ERROR_CUDA 3              /* a CUDA runtime call or launch failed */
#define KSJ_GPU_ERROR_WORKSPACE 4         /* workspace pointer null, misaligned or too small */
#define KSJ_GPU_ERROR_OUT_OF_MEMORY 5     /* a ksj_gpu_context allocation failed */
#define KSJ_GPU_ERROR_NONFINITE_INPUT 6   /* device check: a sample, trajectory or DCF value was rejected */

/* Device-side input checks, reported through ksj_gpu_read_flags(). */
#define KSJ_GPU_FLAG_NONFINITE_SAMPLE (1u << 0)
#define KSJ_GPU_FLAG_BAD_TRAJECTORY (1u << 1)   /* non-finite, or outside [-pi, pi] where required */
#define KSJ_GPU_FLAG_BAD_DCF (1u << 2)          /* non-finite or negative external weight */
#define KSJ_GPU_FLAG_WAIT_TIMEOUT (1u << 3)     /* a bounded device wait (a tile copy, a long list's segment order) gave up; output invalid */

/* ------------------------------------------------------------- gridding */

#define KSJ_GPU_KERNEL_LINEAR 0u        /* the reference's periodic 2x2 linear stencil, grid == image */
#define KSJ_GPU_KERNEL_KAISER_BESSEL 1u /* W-tap Kaiser-Bessel on an oversampled grid, deapodised and cropped */

#define KSJ_GPU_DCF_NONE 0u           /* weight 1 */
#define KSJ_GPU_DCF_ANALYTIC_RAMP 1u  /* hypot(k_row, k_col), radians per pixel (Ram-Lak) */
#define KSJ_GPU_DCF_EXTERNAL 2u       /* caller weights d_dcf[frame][sample], finite and >= 0 */

#define KSJ_GPU_OUTPUT_COIL_LAST 0u   /* complex64 [frame][row][col][channel] (ksj.coil-image-frame) */
#define KSJ_GPU_OUTPUT_RSS 1u         /* float32 [frame][row][col], root-sum-of-squares over channels */
#define KSJ_GPU_OUTPUT_COIL_MAJOR 2u  /* complex64 [frame][channel][row][col] */

#define KSJ_GPU_SAMPLES_CF32 0u       /* interleaved float32 (re, im) */
#define KSJ_GPU_SAMPLES_BF16 1u       /* interleaved bfloat16 (re, im); arithmetic stays float32 */

typedef struct ksj_gpu_gridding_desc {
  uint32_t struct_size;     /* sizeof(ksj_gpu_gridding_desc) */
  uint32_t kernel;          /* KSJ_GPU_KERNEL_* */
  uint32_t image_rows;      /* output image, 2..512 */
  uint32_t image_cols;
  uint32_t grid_rows;       /* oversampled grid; == image for LINEAR; 2^a 3^b 5^c 7^d, 2..512 */
  uint32_t grid_cols;
  uint32_t kernel_width;    /* LINEAR: 2.  KAISER_BESSEL: even, 2..8 */
  float kb_beta;            /* KAISER_BESSEL shape; <= 0 selects Beatty et al. 2005 for (width, grid/image) */
  double row_origin;        /* image origin in pixels; the reference uses (rows-1)/2 */
  double col_origin;
  uint32_t channels;        /* coils, >= 1 */
  uint32_t samples;         /* samples per frame and channel, >= 1 */
  uint32_t frames;          /* independent frames in this call, >= 1 */
  uint32_t dcf_mode;        /* KSJ_GPU_DCF_* */
  uint32_t output;          /* KSJ_GPU_OUTPUT_* */
  uint32_t sample_format;   /* KSJ_GPU_SAMPLES_* */
  uint32_t require_nyquist; /* nonzero: reject |k| > pi (the reference operator's trajectory contract) */
  uint32_t reserved0;
} ksj_gpu_gridding_desc;

/* Tuning knobs chosen per shape by ksj_gpu_gridding_tune() (or by hand).
 * Zero fields select the built-in heuristic. */
typedef struct ksj_gpu_gridding_tuning {
  uint32_t struct_size;
  uint32_t coil_group;      /* channels accumulated per row CTA: 1, 2, 4, 8, 16 or 32 */
  uint32_t column_block;    /* columns per column-pass tile: a power of two (1..32) */
  uint32_t list_capacity;   /* per-warp sorted-list buffer, entries (power of two, 64..2048) */
  uint32_t frames_per_pass; /* frames per row/column pass; passes alternate between two streams (0: two passes
                                once there are 4 or more frames) */
  uint32_t rows_blocks_per_sm; /* 1 or 2 resident row CTAs per SM (2 caps registers at 80 per thread) */
  uint32_t coil_parts;      /* 1 or 2: a row CTA's coil group is split into this many independent list tasks */
  uint32_t column_pass;     /* 0 heuristic, 1 one CTA per (frame, column block), 2 persistent CTAs with a
                                two-stage TMA ring of 16-line tiles (two-step column lengths only) */
  uint32_t wait_fault_polls; /* tests only; 0 in normal use.  Nonzero: every later segment of a long binning
                                list waits for a count that never comes and gives up after this many polls,
                                raising KSJ_GPU_FLAG_WAIT_TIMEOUT (the output is then invalid): exercises the
                                bounded-wait path of the row pass without a fault */
} ksj_gpu_gridding_tuning;

/* Workspace bytes ksj_gpu_gridding_adjoint needs for `desc` (0 on a bad desc). */
KSJ_GPU_API size_t ksj_gpu_gridding_workspace_bytes(const ksj_gpu_gridding_desc* desc);

/* Adjoint gridding reconstruction of `frames` independent frames.
 *   d_kspace  [frame][channel][sample] samples (channel-major, ksj.noncartesian-kspace-frame per frame)
 *   d_traj    [frame][sample][2] float32, (k_row, k_col) in radians per pixel (ksj.trajectory-frame)
 *   d_dcf     [frame][sample] float32 for KSJ_GPU_DCF_EXTERNAL, else ignored (may be NULL)
 *   d_out     per desc->output
 *   d_workspace >= ksj_gpu_gridding_workspace_bytes(desc) bytes, 256-byte aligned; its
 *               contents need not be initialised and are overwritten.
 * Asynchronous on `stream`.  Input checks run on the device; read them with
 * ksj_gpu_read_flags() after the stream has completed.
 * Deterministic: repeated calls on the same inputs give byte-identical output. */
KSJ_GPU_API ksj_gpu_status ksj_gpu_gridding_adjoint(const ksj_gpu_gridding_desc* desc,
                                                    const ksj_gpu_gridding_tuning* tuning, const void* d_kspace,
                                                    const float* d_traj, const float* d_dcf, void* d_out,
                                                    void* d_workspace, size_t workspace_bytes, void* stream);

/* A ragged batch: frames of different coil and sample counts (and the same
 * grid, image, kernel and DCF mode) in one call, each frame's inputs where
 * they already are.  desc->channels and desc->samples are the maxima (they
 * size the workspace); desc->dcf_mode is NONE or ANALYTIC_RAMP.  Device
 * arrays of `frames` entries give frame f's coils d_frame_channels[f]
 * (1..channels), samples d_frame_samples[f] (1..samples), and the addresses
 * of its samples d_frame_kspace[f] (complex64 [channel][sample], packed at
 * its own counts) and trajectory d_frame_traj[f] (float32 [sample][2]).  An
 * address may be device memory or host memory the device reads in place
 * (page-locked and mapped, e.g. cudaHostAlloc / cudaHostRegister on a
 * unified-addressing system; check with cudaPointerGetAttributes): the
 * samples are then read across the host link by the kernel that reorders
 * them, with no separate copy.  d_out as for ksj_gpu_gridding_adjoint.
 * Frame f's output equals that of ksj_gpu_gridding_adjoint on the frame
 * alone with its own coil and sample counts, byte for byte (coil outputs:
 * its first d_frame_channels[f] coils, the others zero).  Kaiser-Bessel
 * only.  Workspace: ksj_gpu_gridding_workspace_bytes(desc); per-frame check
 * flags at ksj_gpu_gridding_frame_flags_offset(desc).  No counterpart in the
 * reference (the batching behind the request loop of ksj_serve.h). */
KSJ_GPU_API ksj_gpu_status ksj_gpu_gridding_adjoint_ragged(const ksj_gpu_gridding_desc* desc,
                                                           const ksj_gpu_gridding_tuning* tuning,
                                                           const uint32_t* d_frame_channels,
                                                           const uint32_t* d_frame_samples,
                                                           const uint64_t* d_frame_kspace,
                                                           const uint64_t* d_frame_traj, void* d_out,
                                                           void* d_workspace, size_t workspace_bytes, void* stream);

/* The same reconstruction from and to host memory: h_kspace, h_traj, h_dcf
 * and h_out have the layouts of the device form above and should be pinned
 * (page-locked) for the copies to run asynchronously.  The trajectory is
 * copied first and the binning lists are built while the samples stream in on
 * a second stream in passes of frames; each pass is transposed, gridded and
 * transformed as soon as its samples have arrived, and its images are copied
 * back while the next pass computes; odd passes run on a second compute
 * stream so consecutive passes overlap.  The frames are split into at least
 * 8 passes (a tuning's smaller frames_per_pass is kept).  Returns at
 * once; `stream` completes after the last image copy.  The output bytes equal
 * those of ksj_gpu_gridding_adjoint.  The device workspace is
 * ksj_gpu_gridding_host_workspace_bytes(desc) bytes (the device form's
 * workspace plus device copies of the inputs and images), 256-byte aligned.
 * No counterpart in the reference (its Provider copies and computes in turn). */
KSJ_GPU_API size_t ksj_gpu_gridding_host_workspace_bytes(const ksj_gpu_gridding_desc* desc);
KSJ_GPU_API ksj_gpu_status ksj_gpu_gridding_adjoint_host(const ksj_gpu_gridding_desc* desc,
                                                         const ksj_gpu_gridding_tuning* tuning, const void* h_kspace,
                                                         const float* h_traj, const float* h_dcf, void* h_out,
                                                         void* d_workspace, size_t workspace_bytes, void* stream);

/* The sorted binning lists of the last call that used `d_workspace`, copied to
 * host memory: for every frame, list (grid_row, column_chunk) in row-major
 * order, the sample indices that touch it in increasing order (read from the
 * expanded entries the row pass consumes).  out_offsets
 * receives frames * lists + 1 entries (lists = grid_rows * chunks), out_samples
 * the concatenated indices.  Pass NULL arrays to query the sizes. */
KSJ_GPU_API ksj_gpu_status ksj_gpu_gridding_binning(const ksj_gpu_gridding_desc* desc,
                                                    const ksj_gpu_gridding_tuning* tuning, const void* d_workspace,
                                                    uint32_t* out_chunk_width, uint64_t* out_list_count,
                                                    uint64_t* out_entry_count, uint64_t* out_offsets,
                                                    uint32_t* out_samples);

/* Byte offset in the workspace of `desc`'s call of `frames` 32-bit words:
 * frame f's own KSJ_GPU_FLAG_* bits (non-finite sample, bad trajectory, bad
 * DCF) of the last ksj_gpu_gridding_adjoint / _ragged call that used the
 * workspace, for callers that batch independent requests into one call and
 * must fail only the offending one.  0 on a bad desc. */
KSJ_GPU_API size_t ksj_gpu_gridding_frame_flags_offset(const ksj_gpu_gridding_desc* desc);

/* Device-side check flags (KSJ_GPU_FLAG_*) of the last call that used
 * `d_workspace`.  Synchronises `stream`. */
KSJ_GPU_API ksj_gpu_status ksj_gpu_read_flags(const void* d_workspace, void* stream, uint32_t* out_flags);

/* Fill `tuning` with the autotuner's choice for `desc`: every admissible
 * (coil_group, column_block) pair is timed with CUDA events on `stream`, the
 * fastest kept and cached per shape for the life of the process.  The buffers
 * are those a real call would use. */
KSJ_GPU_API ksj_gpu_status ksj_gpu_gridding_tune(const ksj_gpu_gridding_desc* desc, const void* d_kspace,
                                                 const float* d_traj, const float* d_dcf, void* d_out,
                                                 void* d_workspace, size_t workspace_bytes, void* stream,
                                                 ksj_gpu_gridding_tuning* tuning);

/* ------------------------------------------------------ 3-D gridding */

/* 3-D Kaiser-Bessel adjoint gridding on a cube (no counterpart in the
 * reference, which is 2-D only): image n^3, grid g^3 (g = 2^a 3^b 5^c 7^d <= 512,
 * g >= n), origin (n-1)/2 on every axis, taps, weights, crop and
 * deapodisation as the 2-D Kaiser-Bessel path along each axis. */
typedef struct ksj_gpu_gridding3_desc {
  uint32_t struct_size;
  uint32_t image;          /* n */
  uint32_t grid;           /* g */
  uint32_t kernel_width;   /* even, 2..8 */
  double kb_beta;          /* 0: Beatty et al. for sigma = g / n */
  uint32_t channels;
  uint32_t samples;
  uint32_t dcf_mode;       /* NONE, ANALYTIC_RAMP (|k|^2, 3-D radial), EXTERNAL */
  uint32_t output;         /* KSJ_GPU_OUTPUT_RSS (float [n][n][n]) or COIL_LAST (complex [n][n][n][C]) */
  uint32_t sample_format;  /* KSJ_GPU_SAMPLES_CF32 or _BF16 */
  uint32_t reserved0;
} ksj_gpu_gridding3_desc;

/* Workspace bytes for `desc` (0 on a bad desc). */
KSJ_GPU_API size_t ksj_gpu_gridding3_workspace_bytes(const ksj_gpu_gridding3_desc* desc);

/*   d_kspace [channel][sample] samples; d_traj [sample][3] float32 (k_z, k_y, k_x)
 *   radians per voxel; d_dcf [sample] for KSJ_GPU_DCF_EXTERNAL.  The tuning
 *   knobs are those of the 2-D call (a z-plane is one frame). */
KSJ_GPU_API ksj_gpu_status ksj_gpu_gridding3_adjoint(const ksj_gpu_gridding3_desc* desc,
                                                     const ksj_gpu_gridding_tuning* tuning, const void* d_kspace,
                                                     const float* d_traj, const float* d_dcf, void* d_out,
                                                     void* d_workspace, size_t workspace_bytes, void* stream);

/* ------------------------------------------------- Pipe-Menon density weights */

/* Iterative density compensation (Pipe and Menon, MRM 41:179-186, 1999; no
 * counterpart in the reference) for the Kaiser-Bessel gridding of `desc`
 * (kernel KSJ_GPU_KERNEL_KAISER_BESSEL; grid, width, beta, frames and samples
 * are used, channels and output are not):
 *   w = 1; repeat `iterations` times:
 *     c = grid of w through phi (every cell sums its samples in increasing order),
 *     d_s = c read back through sample s's taps, w_s = w_s / d_s (0 if d_s <= 0),
 * phi the same tap set and kernel as the gridding, all in double precision.
 *   d_traj [frame][sample][2] float32 radians per pixel
 *   d_dcf  [frame][sample] float32 out: the final weights, usable as
 *          KSJ_GPU_DCF_EXTERNAL for the same gridding
 * Workspace: ksj_gpu_pipe_menon_workspace_bytes (0 on a bad desc). */
KSJ_GPU_API size_t ksj_gpu_pipe_menon_workspace_bytes(const ksj_gpu_gridding_desc* desc);
KSJ_GPU_API ksj_gpu_status ksj_gpu_pipe_menon_dcf(const ksj_gpu_gridding_desc* desc, uint32_t iterations,
                                                  const float* d_traj, float* d_dcf, void* d_workspace,
                                                  size_t workspace_bytes, void* stream);

/* The same iteration in 3-D, for the kernel and grid of a 3-D gridding
 * descriptor (its channels and output are not used): d_traj [sample][3],
 * d_dcf [sample] float32 out. */
KSJ_GPU_API size_t ksj_gpu_pipe_menon3_workspace_bytes(const ksj_gpu_gridding3_desc* desc);
KSJ_GPU_API ksj_gpu_status ksj_gpu_pipe_menon_dcf3(const ksj_gpu_gridding3_desc* desc, uint32_t iterations,
                                                   const float* d_traj, float* d_dcf, void* d_workspace,
                                                   size_t workspace_bytes, void* stream);

/* ----------------------------------------------------------- direct NUDFT */

/* Exact direct adjoint NUDFT, no DCF:
 *   img(c)(r, col) = sum_s y(c)(s) exp(i (k_row,s (r - row_origin) + k_col,s (col - col_origin)))
 * d_kspace [channel][sample] complex64, d_traj [sample][2], d_out coil-last
 * complex64 [row][col][channel].  channels <= 524,280 (KSJ_GPU_ERROR_UNSUPPORTED
 * above).  Workspace: ksj_gpu_direct_workspace_bytes. */
KSJ_GPU_API size_t ksj_gpu_direct_workspace_bytes(uint32_t rows, uint32_t cols, uint32_t channels);
KSJ_GPU_API ksj_gpu_status ksj_gpu_direct_adjoint(uint32_t rows, uint32_t cols, double row_origin, double col_origin,
                                                  uint32_t channels, uint32_t samples, const void* d_kspace,
                                                  const float* d_traj, void* d_out, void* d_workspace,
                                                  size_t workspace_bytes, void* stream);

/* Kaiser-Bessel forward NUFFT: the exact transpose of ksj_gpu_gridding_adjoint
 * with KSJ_GPU_KERNEL_KAISER_BESSEL and no density weights (the same taps,
 * weights, phase, crop positions and deapodisation), i.e. the fast
 * approximation of ksj_gpu_direct_forward that the gridding adjoint pairs
 * with.  desc: kernel KAISER_BESSEL, square image and grid (grid <= 512,
 * 2^a 3^b 5^c 7^d), width 2/4/6/8, complex64 samples; dcf_mode and output are
 * ignored.  d_image complex64 coil-last [frame][row][col][channel]; d_traj
 * [frame][sample][2]; d_samples complex64 [frame][channel][sample].  A
 * non-finite or far out-of-range coordinate gives 0 and raises
 * KSJ_GPU_FLAG_BAD_TRAJECTORY (ksj_gpu_read_flags on the workspace).
 * Workspace: ksj_gpu_kb_forward_workspace_bytes (the row-transformed image
 * and the transformed grid, frames x grid^2 x channels complex64).  No
 * counterpart in the reference (its forward is the direct NUDFT, or BART). */
KSJ_GPU_API size_t ksj_gpu_kb_forward_workspace_bytes(const ksj_gpu_gridding_desc* desc);
KSJ_GPU_API ksj_gpu_status ksj_gpu_kb_forward(const ksj_gpu_gridding_desc* desc, const void* d_image,
                                              const float* d_traj, void* d_samples, void* d_workspace,
                                              size_t workspace_bytes, void* stream);

/* Exact direct forward NUDFT (the reference's nufft2_forward on its Eigen
 * backend, nufft.cpp:29 -> eigen_nufft_direct_nudft.cpp:51-74), per channel:
 *   y(c)(s) = sum_{r, col} x(c)(r, col) exp(-i (k_row,s (r - row_origin) + k_col,s (col - col_origin)))
 * summed in pixel (row-major) order.  d_image coil-last complex64
 * [row][col][channel] (the layout ksj_gpu_direct_adjoint writes), d_traj
 * [sample][2], d_out [channel][sample] complex64 (the layout it reads): the
 * two are adjoint to each other.  No workspace. */
KSJ_GPU_API ksj_gpu_status ksj_gpu_direct_forward(uint32_t rows, uint32_t cols, double row_origin, double col_origin,
                                                  uint32_t channels, uint32_t samples, const void* d_image,
                                                  const float* d_traj, void* d_out, void* stream);

/* The direct NUDFT adjoint above without a caller workspace and without any
 * allocation.  No counterpart in the reference.  For callers that cannot
 * allocate device memory at call time: hosts that bind only this C ABI and
 * own no device allocator, and latency-bound loops where cudaMalloc/cudaFree
 * would synchronise the device and stall every other stream.  Same kernels
 * and same output as ksj_gpu_direct_adjoint.
 *   - The coil-major intermediate lives in a file-scope device array of
 *     ksj_gpu_direct_static_scratch_bytes() = 8 MiB per device, so
 *     rows * cols * channels <= 1,048,576 (e.g. 128 x 128 x 64, 256 x 256 x 16);
 *     larger requests return KSJ_GPU_ERROR_WORKSPACE before any device work.
 *     channels <= 524,280 as for ksj_gpu_direct_adjoint (UNSUPPORTED above).
 *   - Nothing needs to start at zero: every scratch element the call reads
 *     was written earlier in the same call.
 *   - The first call on each device (with that device current) looks up the
 *     array's address, which may load the module; make that first call before
 *     any stream capture.  The address is kept with the CUDA context it was
 *     taken in and looked up again when the current context changes (after a
 *     cudaDeviceReset, for instance).  The device used is the current device;
 *     `stream` must belong to it.
 *   - All calls on one device share the one array: calls that overlap in time
 *     (different streams, or host threads without ordering) race on it and
 *     give wrong results.  Serialise them, e.g. on one stream. */
KSJ_GPU_API size_t ksj_gpu_direct_static_scratch_bytes(void);
KSJ_GPU_API ksj_gpu_status ksj_gpu_direct_adjoint_static(uint32_t rows, uint32_t cols, double row_origin,
                                                         double col_origin, uint32_t channels, uint32_t samples,
                                                         const void* d_kspace, const float* d_traj, void* d_out,
                                                         void* stream);

/* --------------------------------------------------------------- combine */

/* Root-sum-of-squares over the channel (last) axis:
 *   d_out[p] = sqrt(sum_c re^2 + im^2), summed in channel order in float32,
 * d_coil_last complex64 [pixels][channels] -> d_out float32 [pixels]. */
KSJ_GPU_API ksj_gpu_status ksj_gpu_rss_coil_last(uint64_t pixels, uint32_t channels, const void* d_coil_last,
                                                 float* d_out, void* stream);

/* Adaptive coil combination (Walsh, Gmitro, Marcellin, MRM 2000; no
 * counterpart in the reference): for every pixel, the coil covariance of the
 * window x window neighbourhood (clipped at the image border), its dominant
 * eigenvector v by `iterations` power iterations from the pixel's own coil
 * vector, phase-referenced so that v[0] is real and non-negative; out = v^H x.
 * d_coil_last complex64 [rows][cols][channels] -> d_out complex64 [rows][cols].
 * channels 1..8 (apply after coil compression); window odd, <= 9. */
KSJ_GPU_API ksj_gpu_status ksj_gpu_walsh_combine(uint32_t rows, uint32_t cols, uint32_t channels, uint32_t window,
                                                 uint32_t iterations, const void* d_coil_last, void* d_out,
                                                 void* stream);

/* ----------------------------------------------------- coil compression */

/* Coil covariance R = (1/M) X X^H of channel-major k-space X complex64
 * [channels][samples] (coil_compression_basis_estimate.cpp:207-227; the 1/M
 * is applied in float as there): d_cov complex64 [channels][channels], full
 * Hermitian.  On the tensor cores: each element of [Re X; Im X] is split into
 * bf16 hi + lo and hi hi^T + lo hi^T + (lo hi^T)^T is accumulated in FP32
 * (tcgen05), stated bound 1e-4 relative Frobenius error against FP64.
 * channels <= 32.  Workspace: ksj_gpu_coil_covariance_workspace_bytes. */
KSJ_GPU_API size_t ksj_gpu_coil_covariance_workspace_bytes(uint32_t channels, uint32_t samples);
KSJ_GPU_API ksj_gpu_status ksj_gpu_coil_covariance(uint32_t channels, uint32_t samples, const void* d_kspace,
                                                   void* d_cov, void* d_workspace, size_t workspace_bytes,
                                                   void* stream);

/* Host: the compression basis of a covariance (host complex64 [C][C], lower
 * triangle read and mirrored as the reference does): conj of the eigenvectors
 * of the largest `virtual_channels` eigenvalues, largest first
 * (coil_compression_basis_estimate.cpp:228-239), by double-precision cyclic
 * Jacobi.  basis: host complex64 [virtual_channels][channels]; eigenvalues
 * (optional, host float [channels]) in decreasing order. */
KSJ_GPU_API ksj_gpu_status ksj_coil_compression_basis(uint32_t channels, uint32_t virtual_channels,
                                                      const void* covariance, void* basis, float* eigenvalues);

/* Noise covariance of noise_model_estimate.cpp:161-162 (population
 * normalisation, channel means removed, the reference's convention
 * C(r, c) = (1/M) sum_s conj(x_r - mu_r) (x_c - mu_c), moments.hpp:99-140)
 * of channel-major noise samples complex64 [channels][samples] -> d_cov
 * complex64 [channels][channels], Hermitian.  The product sums run on the
 * tensor cores as in ksj_gpu_coil_covariance (split BF16, FP32 accumulate);
 * the means are removed afterwards as mu_r conj(mu_c).  channels <= 32.
 * Workspace: ksj_gpu_coil_covariance_workspace_bytes. */
KSJ_GPU_API ksj_gpu_status ksj_gpu_noise_covariance(uint32_t channels, uint32_t samples, const void* d_noise,
                                                    void* d_cov, void* d_workspace, size_t workspace_bytes,
                                                    void* stream);

/* Host: the whitening matrix of a noise covariance (host complex64 [C][C],
 * lower triangle read and mirrored), noise_model_estimate.cpp:163-167 and
 * whitening.hpp:27-51: W = V diag(1 / sqrt(max(lambda, floor))) V^H by
 * double-precision cyclic Jacobi; the reference's floor is 1e-6.  whitening:
 * host complex64 [channels][channels].  channels <= 64. */
KSJ_GPU_API ksj_gpu_status ksj_whitening_matrix(uint32_t channels, const void* covariance, float eigenvalue_floor,
                                                void* whitening);

/* Y = W X (noncartesian_noise_prewhiten.cpp:140-146): d_whitening complex64
 * [channels][channels], d_kspace complex64 [channels][samples] -> d_out
 * complex64 [channels][samples].  channels <= 32. */
KSJ_GPU_API ksj_gpu_status ksj_gpu_noise_prewhiten(uint32_t channels, uint32_t samples, const void* d_whitening,
                                                   const void* d_kspace, void* d_out, void* stream);

/* Y = B X (noncartesian_coil_compress.cpp:143-148): d_basis complex64
 * [virtual][channels], d_kspace complex64 [channels][samples] ->
 * d_out complex64 [virtual][samples].  channels <= 32, virtual <= 16. */
KSJ_GPU_API ksj_gpu_status ksj_gpu_coil_compress(uint32_t channels, uint32_t virtual_channels, uint32_t samples,
                                                 const void* d_basis, const void* d_kspace, void* d_out,
                                                 void* stream);

/* -------------------------------------------------------------- ingress */

/* Trajectory units of the ISMRMRD route (RadialHdf5TrajectoryUnits). */
#define KSJ_GPU_TRAJ_CYCLES_PER_FOV 1u       /* |k| <= 0.5, scaled by 2 pi */
#define KSJ_GPU_TRAJ_RADIANS_PER_PIXEL 2u    /* |k| <= pi, unscaled */
#define KSJ_GPU_TRAJ_ENCODED_MATRIX_INDEX 3u /* |k| <= encoded / 2, scaled by 2 pi / encoded */

/* ISMRMRD [kx, ky] float32 pairs -> [row = ky, column = kx] radians per pixel
 * (libs/recon/kspacejet-recon-runtime/src/noncartesian_rss_hdf5.cpp:776-833),
 * on the device so the trajectory stays resident: each raw coordinate checked
 * (finite, inside its unit's inclusive Nyquist interval; a failure ORs
 * KSJ_GPU_FLAG_BAD_TRAJECTORY into *d_flags) and scaled with the reference's
 * float factor in one rounded multiply (bit-identical).  encoded_rows /
 * encoded_cols are the XML encoded dimensions (used by
 * KSJ_GPU_TRAJ_ENCODED_MATRIX_INDEX, >= 2). */
KSJ_GPU_API ksj_gpu_status ksj_gpu_normalize_trajectory(uint32_t samples, uint32_t units, uint32_t encoded_rows,
                                                        uint32_t encoded_cols, const float* d_raw, float* d_out,
                                                        uint32_t* d_flags, void* stream);

/* Per-acquisition channel-major blocks complex64 [acquisition][channel][n] ->
 * one channel-major frame [channel][acquisition * n]
 * (noncartesian_rss_hdf5.cpp:1077-1083, acquisitions of equal length). */
KSJ_GPU_API ksj_gpu_status ksj_gpu_aggregate_acquisitions(uint32_t acquisitions, uint32_t channels,
                                                          uint32_t samples_per_acquisition, const void* d_in,
                                                          void* d_out, void* stream);

/* ------------------------------------------------- Cartesian coil images */

/* cartesian_ifft2_coil_images (providers/kspacejet-cartesian-recon/src/
 * operators/cartesian_ifft2_coil_images.cpp:372-407): per frame and channel
 * the inverse 2-D DFT normalised by 1 / (rows cols), no shift
 * (fft2_inplace_with_workspace, Direction::inverse, Normalization::inverse).
 * d_kspace complex64 [frame][channel][row][col] (channel-major, as the
 * reference's ksj.kspace-frame) -> d_out per `output`: KSJ_GPU_OUTPUT_COIL_LAST
 * complex64 [frame][row][col][channel] (the reference's coil-image frame) or
 * KSJ_GPU_OUTPUT_RSS float32 [frame][row][col].  rows and cols 2..512, every
 * length the reference takes: lengths 2^a 3^b 5^c 7^d by mixed-radix FFTs,
 * lengths with a larger prime factor by a direct DFT along that axis (larger
 * lengths: KSJ_GPU_ERROR_UNSUPPORTED); channels 1..64.  Workspace:
 * ksj_gpu_cartesian_workspace_bytes. */
KSJ_GPU_API size_t ksj_gpu_cartesian_workspace_bytes(uint32_t rows, uint32_t cols, uint32_t channels,
                                                     uint32_t frames);
KSJ_GPU_API ksj_gpu_status ksj_gpu_cartesian_ifft2(uint32_t rows, uint32_t cols, uint32_t channels, uint32_t frames,
                                                   uint32_t output, const void* d_kspace, void* d_out,
                                                   void* d_workspace, size_t workspace_bytes, void* stream);

/* --------------------------------------------------------------- context */

/* A device, a non-blocking stream and a grow-only device workspace; used by
 * the Provider plug-ins.  Not thread-safe: one context per serial instance. */
typedef struct ksj_gpu_context ksj_gpu_context;

KSJ_GPU_API ksj_gpu_status ksj_gpu_context_create(int device, ksj_gpu_context** out_context);
KSJ_GPU_API void ksj_gpu_context_destroy(ksj_gpu_context* context);
KSJ_GPU_API void* ksj_gpu_context_stream(ksj_gpu_context* context);
/* Ensure `bytes` of device memory, keyed by `slot` (0..7); returns the pointer. */
KSJ_GPU_API ksj_gpu_status ksj_gpu_context_buffer(ksj_gpu_context* context, uint32_t slot, size_t bytes,
                                                  void** out_pointer);
/* Host staging: pinned host memory, keyed by slot (0..3). */
KSJ_GPU_API ksj_gpu_status ksj_gpu_context_pinned(ksj_gpu_context* context, uint32_t slot, size_t bytes,
                                                  void** out_pointer);
/* Async copies on the context stream (kind: 0 host->device, 1 device->host). */
KSJ_GPU_API ksj_gpu_status ksj_gpu_context_copy(ksj_gpu_context* context, void* dst, const void* src, size_t bytes,
                                                int kind);
KSJ_GPU_API ksj_gpu_status ksj_gpu_context_sync(ksj_gpu_context* context);
/* Total device bytes and streams the context holds (the Provider declares them). */
KSJ_GPU_API uint64_t ksj_gpu_context_device_bytes(const ksj_gpu_context* context);
/* Host-side fault injection for tests of the plug-ins' failure paths: the
 * next `count` device allocations ksj_gpu_context_buffer would make return
 * KSJ_GPU_ERROR_OUT_OF_MEMORY without calling cudaMalloc (0 clears).  The
 * device is not touched.  No counterpart in the reference (its tests fake a
 * misbehaving Provider instead). */
KSJ_GPU_API void ksj_gpu_inject_allocation_failures(uint32_t count);

/* Per-kernel timing for measurement.  While enabled, every kernel the
 * library launches is bracketed by CUDA events on the stream it is launched
 * on; ksj_gpu_timing_read waits for those events and returns, per kernel
 * name, the launch count and the summed event-to-event milliseconds since the
 * last reset.  names receives max_entries rows of 48 bytes.  Returns the
 * number of distinct kernels (which may exceed max_entries). */
KSJ_GPU_API void ksj_gpu_timing_enable(int enable);
KSJ_GPU_API void ksj_gpu_timing_reset(void);
KSJ_GPU_API uint32_t ksj_gpu_timing_read(uint32_t max_entries, char* names, uint64_t* launches, double* total_ms);

/* Human-readable status text (static storage). */
KSJ_GPU_API const char* ksj_gpu_status_string(ksj_gpu_status status);
/* Number of kernel launches this process issued through the library. */
KSJ_GPU_API uint64_t ksj_gpu_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* KSJ_GPU_H_ */
