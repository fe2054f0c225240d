/*
 * ksj_serve.h -- a device-resident request loop for slice reconstructions of
 * uneven shape (readout, spokes, coils) arriving over time.
 *
 * Requests are admitted in arrival order as soon as a slot (one CUDA stream
 * with its own grow-only device workspace) is free and the device bytes held
 * by admitted requests stay within the configured cap; admitted requests run
 * concurrently on their streams, so a request that arrives while others are
 * on the GPU starts as soon as capacity frees up (continuous batching, not a
 * queue in front of one GPU job).  Trajectories submitted with an id stay
 * resident on the device and are reused.  Per-request caps mirror the
 * reference's target envelope (config/target-envelope.json: max_frame_bytes,
 * max_image_bytes, max_channels_per_acquisition); the device cap plays the
 * role of the machine policy's memory limit for device bytes.
 *
 * Each request is one ksj_gpu_gridding_adjoint call (Kaiser-Bessel, frames = 1)
 * whose result is byte-identical to the same call made alone: the kernels are
 * deterministic and requests share no device state but cached trajectories.
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
  uint32_t slots;              /* requests in flight on the device, >= 1 (1 = the serial path) */
  uint32_t max_channels;       /* per request (target envelope: 32) */
  uint64_t device_memory_cap;  /* bytes of device memory admitted requests may hold */
  uint64_t max_frame_bytes;    /* per-request k-space bytes (target envelope: 256 MiB) */
  uint64_t max_image_bytes;    /* per-request output bytes (target envelope: 128 MiB) */
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
  uint32_t peak_in_flight;
  uint32_t reserved0;
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
