/*
 * ksj_serve.h -- a host-scheduled request loop with continuous batching for
 * slice reconstructions of uneven shape (readout, spokes, coils) arriving
 * over time, on one GPU.
 *
 * A scheduler thread keeps up to `slots` batches in flight, each on its own
 * CUDA stream with grow-only device buffers.  Whenever a slot is free, the
 * oldest pending request opens a batch and the later pending requests of its
 * class (grid, image, kernel width, DCF mode, output form, and optionally
 * whether it has at most coil_split coils) join it in
 * arrival order, up to max_batch_frames requests and as long as the device
 * bytes of everything in flight stay within the configured cap.  A batch is
 * ONE ragged multi-frame reconstruction (ksj_gpu_gridding_adjoint_ragged:
 * every request a frame with its own coil and sample counts), so small
 * requests share one launch chain instead of paying for their own.  Requests
 * that arrive while batches are on the GPU are admitted as slots and memory
 * free up; batches on different slots overlap on the device.  Trajectories
 * submitted with an id stay resident on the device and are reused.
 * Per-request caps mirror the reference's target envelope
 * (config/target-envelope.json: max_frame_bytes, max_image_bytes,
 * max_channels_per_acquisition); the device cap plays the role of the machine
 * policy's memory limit for device bytes.
 *
 * Each result is byte-identical to the same ksj_gpu_gridding_adjoint call
 * (Kaiser-Bessel, frames = 1) made alone: a ragged call's frames are
 * independent and each equals its one-frame call.  A request whose own
 * samples or trajectory fail the device checks fails alone.
 * max_batch_frames = 1 with slots = 1 is the plain one-request-at-a-time path.
 *
 * No counterpart in the reference (its executor is synchronous,
 * max_in_flight = 1: libs/recon/kspacejet-recon-runtime/src/synchronous_firing_lease.cpp).
 */
#ifndef KSJ_SERVE_H_
#define KSJ_SERVE_H_

#include <stdint.h>

#include "ksj_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ksj_serve ksj_serve;

typedef struct ksj_serve_config {
  uint32_t struct_size;
  int32_t device;
  uint32_t slots;              /* batches in flight on the device, >= 1 (1 with max_batch_frames 1: the serial path) */
  uint32_t max_channels;       /* per request (target envelope: 32) */
  uint64_t device_memory_cap;  /* bytes of device memory admitted requests may hold */
  uint64_t max_frame_bytes;    /* per-request k-space bytes (target envelope: 256 MiB) */
  uint64_t max_image_bytes;    /* per-request output bytes (target envelope: 128 MiB) */
  uint32_t max_batch_frames;   /* requests per batch (one ragged call); 0 = 32, 1 = no batching */
  uint32_t read_inputs_in_place; /* nonzero: page-locked, mapped inputs are read by the kernels across the
                                    host link where they are, with no copy (pageable ones are staged in
                                    page-locked memory first); 0: inputs are copied to the device */
  uint32_t coil_split;         /* nonzero: requests of at most this many coils form their own batches */
  uint32_t reserved0;
} ksj_serve_config;

#define KSJ_SERVE_OUTPUT_RSS 1u         /* float32 [image][image] */
#define KSJ_SERVE_HOST_PINNED 1u        /* request flag: kspace, trajectory and out are pinned host memory */
#define KSJ_SERVE_OUTPUT_COIL_MAJOR 2u  /* complex64 [channel][image][image] */

typedef struct ksj_serve_request {
  uint32_t struct_size;
  uint32_t image;          /* square image side N */
  uint32_t grid;           /* oversampled grid side G (2^a 3^b, >= N) */
  uint32_t kernel_width;   /* even, 2..8 */
  uint32_t channels;
  uint32_t samples;        /* samples per channel */
  uint32_t output;         /* KSJ_SERVE_OUTPUT_* */
  uint32_t dcf_mode;       /* KSJ_GPU_DCF_NONE or KSJ_GPU_DCF_ANALYTIC_RAMP */
  uint32_t flags;          /* KSJ_SERVE_HOST_PINNED: copy by DMA directly, no staging through the slot */
  uint32_t reserved0;
  uint64_t trajectory_id;  /* nonzero: keep this trajectory resident under the id and reuse it */
  const void* kspace;      /* host complex64 [channels][samples]; valid until the request completes */
  const float* trajectory; /* host float32 [samples][2], radians per pixel */
  void* out;               /* host output, written when the request completes */
} ksj_serve_request;

typedef struct ksj_serve_stats {
  uint64_t submitted, completed, rejected, failed;
  uint64_t gridded_samples;   /* sum over completed requests of channels x samples */
  double wall_seconds;        /* first submit to last completion */
  double latency_p50_ms;      /* submit -> result in host memory */
  double latency_p99_ms;
  double latency_max_ms;
  uint64_t peak_device_bytes; /* high-water mark of admitted request bytes */
  uint32_t peak_in_flight;    /* most requests on the device at once (over all batches) */
  uint32_t reserved0;
  uint64_t batches;           /* ragged calls launched */
  uint64_t batched_frames;    /* requests those calls carried */
  double copy_in_ms;          /* per batch, summed: stream time of the input copies */
  double compute_ms;          /* the ragged reconstruction calls */
  double copy_out_ms;         /* the result copies */
} ksj_serve_stats;

KSJ_GPU_API ksj_gpu_status ksj_serve_create(const ksj_serve_config* config, ksj_serve** out);
/* Queue a request; returns KSJ_GPU_ERROR_INVALID_ARGUMENT (and counts a
 * rejection) when it exceeds a per-request cap or the device cap on its own. */
KSJ_GPU_API ksj_gpu_status ksj_serve_submit(ksj_serve* s, const ksj_serve_request* request, uint64_t* out_ticket);
/* Wait until the ticket completes (timeout_ms 0 = no limit); *out_result is
 * its status.  Returns KSJ_GPU_ERROR_UNSUPPORTED on timeout. */
KSJ_GPU_API ksj_gpu_status ksj_serve_wait(ksj_serve* s, uint64_t ticket, uint32_t timeout_ms,
                                          ksj_gpu_status* out_result);
/* Wait for every submitted request. */
KSJ_GPU_API ksj_gpu_status ksj_serve_drain(ksj_serve* s);
KSJ_GPU_API ksj_gpu_status ksj_serve_get_stats(ksj_serve* s, ksj_serve_stats* out);
KSJ_GPU_API void ksj_serve_reset_stats(ksj_serve* s);
KSJ_GPU_API void ksj_serve_destroy(ksj_serve* s);

#ifdef __cplusplus
}
#endif

#endif /* KSJ_SERVE_H_ */
