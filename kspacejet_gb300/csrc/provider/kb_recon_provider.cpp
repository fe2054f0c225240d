// kb_recon_provider.cpp -- `org.kspacejet.gb300-noncartesian-recon`: the
// Kaiser-Bessel adjoint reconstruction operators the reference lacks, behind
// the same Provider C ABI, ports and payload types as its
// radial_gridding_reconstruct (providers/kspacejet-noncartesian-recon/src/
// operators/radial_gridding_reconstruct.cpp:228-436):
//
//   radial_kb_gridding_reconstruct  k-space [C, M] + trajectory [M, 2]
//                                   -> ksj.coil-image-frame [N_r, N_c, C]
//   radial_kb_gridding_rss          same inputs -> ksj.image-frame [N_r, N_c]
//                                   (root sum of squares fused on the device)
//
// Canonical config (keys in this order, no whitespace):
//   {"channels":C,"density_compensation":"radial_analytic_ramp"|"none",
//    "grid_cols":G,"grid_rows":G,"image_cols":N,"image_rows":N,
//    "kernel_width":W,"sample_count":M,"trajectory_units":"radians_per_pixel"}
// with C in [1, 64], N in [2, 512], G >= N of the form 2^a 3^b <= 512,
// W even in [2, 8], M in [1, 2^22].  Origin ((N-1)/2, (N-1)/2) as the
// reference operator uses; trajectory finite (any |k|: the grid is periodic).
// No host scratch is needed: the working set lives in HBM in a per-instance
// ksj_gpu_context created at the first valid firing.
#include <cmath>
#include <cstdint>
#include <new>
#include <string_view>

#include "abi_support.hpp"
#include "ksj_gpu.h"
#include "ksj_provider_abi.h"

using namespace ksj_gb300;

namespace {

constexpr char kProviderId[] = "org.kspacejet.gb300-noncartesian-recon";
// SHA-256 of "kspacejet.provider-bundle\0org.kspacejet.gb300-noncartesian-recon\0
// radial_kb_gridding_reconstruct\0radial_kb_gridding_rss\0"
constexpr char kBundleDigestHex[] = "012f974b83357f52844a48c624ba3c47df5b3654baa0f2f1e0c655a4f38c96a2";

constexpr std::string_view kOpCoils = "radial_kb_gridding_reconstruct";
constexpr std::string_view kOpRss = "radial_kb_gridding_rss";
constexpr std::string_view kErrBadAbi = "GB300 Kaiser-Bessel reconstruction Provider received incompatible ABI storage";
constexpr std::string_view kErrInvalidArgument =
    "GB300 Kaiser-Bessel reconstruction Provider received an invalid lifecycle argument";
constexpr std::string_view kErrUnsupportedOperator =
    "GB300 Kaiser-Bessel reconstruction Provider does not expose the requested operator";
constexpr std::string_view kErrConfig =
    "GB300 Kaiser-Bessel reconstruction requires canonical {\"channels\":N,\"density_compensation\":"
    "\"radial_analytic_ramp\"|\"none\",\"grid_cols\":N,\"grid_rows\":N,\"image_cols\":N,\"image_rows\":N,"
    "\"kernel_width\":N,\"sample_count\":N,\"trajectory_units\":\"radians_per_pixel\"} within its envelope";
constexpr std::string_view kErrLease = "GB300 Kaiser-Bessel reconstruction requires two input batches and one output grant";
constexpr std::string_view kErrKspace =
    "GB300 Kaiser-Bessel reconstruction requires one exact ksj.noncartesian-kspace-frame on input port 0";
constexpr std::string_view kErrTrajectory =
    "GB300 Kaiser-Bessel reconstruction requires one exact finite ksj.trajectory-frame on input port 1";
constexpr std::string_view kErrIdentity =
    "GB300 Kaiser-Bessel k-space and trajectory inputs must have equal semantic_key_hash and order_key";
constexpr std::string_view kErrOutput = "GB300 Kaiser-Bessel reconstruction requires one exact output grant of its type";
constexpr std::string_view kErrInternal = "GB300 Kaiser-Bessel reconstruction trapped an unexpected internal exception";
constexpr std::string_view kErrDevice =
    "GB300 Kaiser-Bessel reconstruction could not use its CUDA device (no device, out of memory, or a kernel failure)";

constexpr uint32_t kMaxImage = 512, kMaxGrid = 512, kMaxChannels = 64, kMaxSamples = 1u << 22;
constexpr uint64_t kMaxOutputBytes = uint64_t{kMaxImage} * kMaxImage * kMaxChannels * 8;

bool grid_size_ok(uint32_t g) {
  if (g < 2 || g > kMaxGrid) return false;
  uint32_t m = g;
  if (m % 3 == 0) m /= 3;
  return m % 3 != 0 && pow2(m);
}

}  // namespace

struct ksj_execution_context {
  ksj_provider_operator* owner = nullptr;
};
struct ksj_key_state {
  ksj_provider_operator* owner = nullptr;
};
struct ksj_provider_operator {
  bool rss = false;
  uint32_t channels = 0, grid_rows = 0, grid_cols = 0, image_rows = 0, image_cols = 0, width = 0, samples = 0;
  uint32_t dcf_mode = KSJ_GPU_DCF_ANALYTIC_RAMP;
  ksj_execution_context context{};
  ksj_key_state key_state{};
  bool context_active = false, key_state_active = false;
  ksj_gpu_context* gpu = nullptr;
  uint32_t device = 0;
};

namespace {

bool valid(const ksj_provider_operator& o) {
  return o.channels >= 1 && o.channels <= kMaxChannels && o.image_rows >= 2 && o.image_rows <= kMaxImage &&
         o.image_cols >= 2 && o.image_cols <= kMaxImage && grid_size_ok(o.grid_rows) && grid_size_ok(o.grid_cols) &&
         o.grid_rows >= o.image_rows && o.grid_cols >= o.image_cols && o.width >= 2 && o.width <= 8 &&
         o.width % 2 == 0 && o.grid_rows >= o.width && o.grid_cols >= o.width && o.samples >= 1 &&
         o.samples <= kMaxSamples;
}

bool configure(const ksj_byte_view& config, ksj_provider_operator* o) {
  const std::string_view lit[] = {"{\"channels\":",   ",\"density_compensation\":\"", "\",\"grid_cols\":",
                                  ",\"grid_rows\":",  ",\"image_cols\":",           ",\"image_rows\":",
                                  ",\"kernel_width\":", ",\"sample_count\":",
                                  ",\"trajectory_units\":\"radians_per_pixel\"}"};
  std::string_view v[8];
  if (!split_canonical(config, lit, 9, v)) return false;
  if (v[1] == "radial_analytic_ramp") o->dcf_mode = KSJ_GPU_DCF_ANALYTIC_RAMP;
  else if (v[1] == "none") o->dcf_mode = KSJ_GPU_DCF_NONE;
  else return false;
  return parse_u32(v[0], 1, kMaxChannels, &o->channels) && parse_u32(v[2], 2, kMaxGrid, &o->grid_cols) &&
         parse_u32(v[3], 2, kMaxGrid, &o->grid_rows) && parse_u32(v[4], 2, kMaxImage, &o->image_cols) &&
         parse_u32(v[5], 2, kMaxImage, &o->image_rows) && parse_u32(v[6], 2, 8, &o->width) &&
         parse_u32(v[7], 1, kMaxSamples, &o->samples) && valid(*o);
}

bool is_operator(const ksj_provider_operator* o) { return o != nullptr && valid(*o); }
bool is_context(const ksj_provider_operator* o, const ksj_execution_context* c) {
  return is_operator(o) && c == &o->context && c->owner == o && o->context_active;
}
bool is_key_state(const ksj_provider_operator* o, const ksj_key_state* k) {
  return is_operator(o) && k == &o->key_state && k->owner == o && o->key_state_active;
}

ksj_gpu_gridding_desc make_desc(const ksj_provider_operator& o) {
  ksj_gpu_gridding_desc d{};
  d.struct_size = sizeof(d);
  d.kernel = KSJ_GPU_KERNEL_KAISER_BESSEL;
  d.image_rows = o.image_rows;
  d.image_cols = o.image_cols;
  d.grid_rows = o.grid_rows;
  d.grid_cols = o.grid_cols;
  d.kernel_width = o.width;
  d.row_origin = (o.image_rows - 1) / 2.0;
  d.col_origin = (o.image_cols - 1) / 2.0;
  d.channels = o.channels;
  d.samples = o.samples;
  d.frames = 1;
  d.dcf_mode = o.dcf_mode;
  d.output = o.rss ? KSJ_GPU_OUTPUT_RSS : KSJ_GPU_OUTPUT_COIL_LAST;
  d.sample_format = KSJ_GPU_SAMPLES_CF32;
  return d;
}

ksj_status process(ksj_provider_operator& o, ksj_firing_lease* lease, const ksj_firing_lease_callbacks* cb,
                   ksj_process_result* result, ksj_error_view* err) {
  if (lease == nullptr || !full_header(result)) return fail(err, KSJ_STATUS_INVALID_ARGUMENT, kErrBadAbi);
  if (!lease_callbacks_ok(cb, KSJ_LEASE_CAP_INPUT_BATCHES | KSJ_LEASE_CAP_OUTPUT_GRANTS))
    return fail(err, KSJ_STATUS_BAD_ABI, kErrBadAbi);
  const uint64_t pixels = uint64_t{o.image_rows} * o.image_cols;
  const uint64_t kspace_bytes = uint64_t{o.channels} * o.samples * 8;
  const uint64_t traj_bytes = uint64_t{o.samples} * 8;
  const uint64_t out_bytes = o.rss ? pixels * 4 : pixels * o.channels * 8;
  ksj_firing_lease_info info{};
  info.abi = header(sizeof(info));
  const ksj_status is = cb->get_info(cb->host_context, lease, &info, err);
  if (is != KSJ_STATUS_OK || !full_header(&info) || info.input_batch_count != 2 || info.output_grant_count != 1 ||
      info.reserved_output_bytes < out_bytes)
    return is == KSJ_STATUS_OK ? fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrLease) : is;
  ksj_input_batch_view batches[2]{};
  for (uint32_t i = 0; i < 2; ++i) {
    batches[i].abi = header(sizeof(batches[i]));
    const ksj_status bs = cb->get_input_batch(cb->host_context, lease, i, &batches[i], err);
    if (bs != KSJ_STATUS_OK) return bs;
  }
  const ksj_input_batch_view* kb = nullptr;
  const ksj_input_batch_view* tb = nullptr;
  for (const ksj_input_batch_view* b : {&batches[0], &batches[1]}) {
    if (!full_header(b)) return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrLease);
    if (b->input_port == 0 && kb == nullptr) kb = b;
    else if (b->input_port == 1 && tb == nullptr) tb = b;
    else return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrLease);
  }
  auto exact = [](const ksj_input_batch_view* b) {
    return b != nullptr && b->item_count == 1 && b->items != nullptr && full_header(&b->items[0]);
  };
  if (!exact(kb)) return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrKspace);
  if (!exact(tb)) return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrTrajectory);
  const ksj_input_item_view& k = kb->items[0];
  const ksj_input_item_view& t = tb->items[0];
  if (!full_header(&k.payload) || k.payload.data == nullptr || k.payload.byte_count != kspace_bytes ||
      k.payload.memory_domain != KSJ_PROVIDER_MEMORY_HOST_PAGEABLE ||
      !host_memory_ok(k.payload.data, k.payload.alignment, 64) || !borrowed_ok(k.metadata) ||
      !type_matches(k.payload.type, kNoncartesianKspaceFrame))
    return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrKspace);
  if (!full_header(&t.payload) || t.payload.data == nullptr || t.payload.byte_count != traj_bytes ||
      t.payload.memory_domain != KSJ_PROVIDER_MEMORY_HOST_PAGEABLE ||
      !host_memory_ok(t.payload.data, t.payload.alignment, 64) || !borrowed_ok(t.metadata) ||
      !type_matches(t.payload.type, kTrajectoryFrame))
    return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrTrajectory);
  if (k.semantic_key_hash != t.semantic_key_hash || k.order_key != t.order_key)
    return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrIdentity);
  const float* tv = static_cast<const float*>(t.payload.data);
  for (uint64_t i = 0; i < uint64_t{o.samples} * 2; ++i)
    if (!std::isfinite(tv[i]) || std::fabs(tv[i]) >= 1.0e4f) return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrTrajectory);

  ksj_output_grant* grant = nullptr;
  const ksj_status as = cb->acquire_output_grant(cb->host_context, lease, 0, &grant, err);
  if (as != KSJ_STATUS_OK || grant == nullptr)
    return as == KSJ_STATUS_OK ? fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrOutput) : as;
  GrantGuard guard{cb->output_grants, grant, false};
  ksj_mutable_payload_view out{};
  out.abi = header(sizeof(out));
  const ksj_status ms = cb->output_grants->map_mutable_payload(cb->output_grants->host_context, grant, &out, err);
  if (ms != KSJ_STATUS_OK) return ms;
  if (!full_header(&out) || out.data == nullptr || out.capacity_bytes < out_bytes || out.committed_bytes != 0 ||
      out.memory_domain != KSJ_PROVIDER_MEMORY_HOST_PAGEABLE || !host_memory_ok(out.data, out.alignment, 64) ||
      !type_matches(out.type, o.rss ? kImageFrame : kCoilImageFrame))
    return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrOutput);

  if (o.gpu == nullptr && ksj_gpu_context_create(static_cast<int>(o.device), &o.gpu) != KSJ_GPU_OK)
    return fail(err, KSJ_STATUS_FAILED_PRECONDITION, kErrDevice);
  const ksj_gpu_gridding_desc desc = make_desc(o);
  const size_t ws_bytes = ksj_gpu_gridding_workspace_bytes(&desc);
  void *d_k = nullptr, *d_t = nullptr, *d_o = nullptr, *d_w = nullptr;
  if (ws_bytes == 0 || ksj_gpu_context_buffer(o.gpu, 0, kspace_bytes, &d_k) != KSJ_GPU_OK ||
      ksj_gpu_context_buffer(o.gpu, 1, traj_bytes, &d_t) != KSJ_GPU_OK ||
      ksj_gpu_context_buffer(o.gpu, 2, out_bytes, &d_o) != KSJ_GPU_OK ||
      ksj_gpu_context_buffer(o.gpu, 3, ws_bytes, &d_w) != KSJ_GPU_OK)
    return fail(err, KSJ_STATUS_RESOURCE_EXHAUSTED, kErrDevice);
  void* stream = ksj_gpu_context_stream(o.gpu);
  uint32_t flags = 0;
  if (ksj_gpu_context_copy(o.gpu, d_k, k.payload.data, kspace_bytes, 0) != KSJ_GPU_OK ||
      ksj_gpu_context_copy(o.gpu, d_t, t.payload.data, traj_bytes, 0) != KSJ_GPU_OK ||
      ksj_gpu_gridding_adjoint(&desc, nullptr, d_k, static_cast<const float*>(d_t), nullptr, d_o, d_w, ws_bytes,
                               stream) != KSJ_GPU_OK ||
      ksj_gpu_context_copy(o.gpu, out.data, d_o, out_bytes, 1) != KSJ_GPU_OK ||
      ksj_gpu_read_flags(d_w, stream, &flags) != KSJ_GPU_OK)
    return fail(err, KSJ_STATUS_INTERNAL_ERROR, kErrDevice);
  if (flags != 0) return fail(err, KSJ_STATUS_INTERNAL_ERROR, kErrInternal);

  ksj_output_seal_descriptor seal{};
  seal.abi = header(sizeof(seal));
  seal.output_port = 0;
  seal.produced_item_count = 1;
  seal.produced_byte_count = out_bytes;
  seal.semantic_key_hash = k.semantic_key_hash;
  seal.order_key = k.order_key;
  seal.type = out.type;
  seal.metadata = k.metadata;
  const ksj_status ss = cb->output_grants->seal(cb->output_grants->host_context, grant, &seal, err);
  if (ss != KSJ_STATUS_OK) return ss;
  guard.settled = true;
  done(result, 1, 2, info.terminal_epoch);
  return KSJ_STATUS_OK;
}

ksj_status create(const ksj_operator_create_request* req, ksj_provider_operator** out, ksj_error_view* err) noexcept {
  try {
    if (!full_header(req) || out == nullptr) return fail(err, KSJ_STATUS_INVALID_ARGUMENT, kErrInvalidArgument);
    *out = nullptr;
    ksj_provider_operator o{};
    if (text_is(req->operator_id, kOpCoils)) o.rss = false;
    else if (text_is(req->operator_id, kOpRss)) o.rss = true;
    else return fail(err, KSJ_STATUS_UNSUPPORTED, kErrUnsupportedOperator);
    if (req->host_services != nullptr && !full_header(req->host_services))
      return fail(err, KSJ_STATUS_BAD_ABI, kErrBadAbi);
    if (!configure(req->canonical_config, &o)) return fail(err, KSJ_STATUS_INVALID_ARGUMENT, kErrConfig);
    auto* p = new (std::nothrow) ksj_provider_operator{o};
    if (p == nullptr) return fail(err, KSJ_STATUS_RESOURCE_EXHAUSTED, kErrInternal);
    *out = p;
    return KSJ_STATUS_OK;
  } catch (...) {
    return fail(err, KSJ_STATUS_INTERNAL_ERROR, kErrInternal);
  }
}

ksj_status context_create(ksj_provider_operator* o, const ksj_execution_context_descriptor* d,
                          ksj_execution_context** out, ksj_error_view* err) noexcept {
  if (!is_operator(o) || !full_header(d) || out == nullptr)
    return fail(err, KSJ_STATUS_INVALID_ARGUMENT, kErrInvalidArgument);
  if (d->host_services != nullptr && !full_header(d->host_services)) return fail(err, KSJ_STATUS_BAD_ABI, kErrBadAbi);
  if (o->context_active) return fail(err, KSJ_STATUS_FAILED_PRECONDITION, kErrInvalidArgument);
  o->device = d->device_ordinal;
  o->context.owner = o;
  o->context_active = true;
  *out = &o->context;
  return KSJ_STATUS_OK;
}

ksj_status key_init(ksj_provider_operator* o, ksj_execution_context* c, const ksj_key_state_descriptor* d,
                    ksj_key_state** out, ksj_error_view* err) noexcept {
  if (!is_context(o, c) || !full_header(d) || out == nullptr || !borrowed_ok(d->semantic_key))
    return fail(err, KSJ_STATUS_INVALID_ARGUMENT, kErrInvalidArgument);
  if (o->key_state_active) return fail(err, KSJ_STATUS_FAILED_PRECONDITION, kErrInvalidArgument);
  o->key_state.owner = o;
  o->key_state_active = true;
  *out = &o->key_state;
  return KSJ_STATUS_OK;
}

ksj_status on_start(ksj_provider_operator* o, ksj_execution_context* c, ksj_key_state* k,
                    const ksj_scan_start_descriptor* d, ksj_error_view* err) noexcept {
  if (!is_context(o, c) || !is_key_state(o, k) || !full_header(d))
    return fail(err, KSJ_STATUS_INVALID_ARGUMENT, kErrInvalidArgument);
  return KSJ_STATUS_OK;
}

ksj_status process_batch(ksj_provider_operator* o, ksj_execution_context* c, ksj_key_state* k,
                         ksj_firing_lease* lease, const ksj_firing_lease_callbacks* cb, ksj_process_result* result,
                         ksj_error_view* err) noexcept {
  if (!is_context(o, c) || !is_key_state(o, k) || lease == nullptr || !full_header(result))
    return fail(err, KSJ_STATUS_INVALID_ARGUMENT, kErrInvalidArgument);
  try {
    return process(*o, lease, cb, result, err);
  } catch (...) {
    return fail(err, KSJ_STATUS_INTERNAL_ERROR, kErrInternal);
  }
}

ksj_status on_scan_end(ksj_provider_operator* o, ksj_execution_context* c, ksj_key_state* k,
                       const ksj_scan_end_descriptor* d, ksj_firing_lease* lease, const ksj_firing_lease_callbacks* cb,
                       ksj_process_result* result, ksj_error_view* err) noexcept {
  if (!is_context(o, c) || !is_key_state(o, k) || !full_header(d) || d->kind != KSJ_PROVIDER_SCAN_END_NORMAL ||
      d->reserved0 != 0 || lease == nullptr || !full_header(result) || !full_header(cb))
    return fail(err, KSJ_STATUS_INVALID_ARGUMENT, kErrInvalidArgument);
  done(result, 0, 0, d->terminal_epoch);
  return KSJ_STATUS_OK;
}

ksj_status on_cancel(ksj_provider_operator* o, ksj_execution_context* c, ksj_key_state* k,
                     const ksj_cancel_context* d, ksj_error_view* err) noexcept {
  if (!is_context(o, c) || !is_key_state(o, k) || !full_header(d) || d->reserved0 != 0 ||
      (d->kind != KSJ_PROVIDER_SCAN_END_CANCELLED && d->kind != KSJ_PROVIDER_SCAN_END_FAILED))
    return fail(err, KSJ_STATUS_INVALID_ARGUMENT, kErrInvalidArgument);
  // cancellation emits nothing and only releases provider work
  // (provider.h:676-694): firings finish their device work before they
  // return, so nothing is in flight; the scan's device memory and stream are
  // freed here (a later firing creates them again) -- no allocation, no throw
  if (o->gpu != nullptr) {
    ksj_gpu_context_destroy(o->gpu);
    o->gpu = nullptr;
  }
  return KSJ_STATUS_OK;
}

void key_reset(ksj_provider_operator* o, ksj_execution_context* c, ksj_key_state* k) noexcept {
  if (!is_context(o, c) || !is_key_state(o, k)) return;
  o->key_state.owner = nullptr;
  o->key_state_active = false;
}

void context_destroy(ksj_provider_operator* o, ksj_execution_context* c) noexcept {
  if (!is_context(o, c)) return;
  o->context.owner = nullptr;
  o->context_active = false;
}

void destroy(ksj_provider_operator* o) noexcept {
  if (o == nullptr) return;
  if (o->gpu != nullptr) ksj_gpu_context_destroy(o->gpu);
  delete o;
}

struct Metadata {
  ksj_operator_descriptor ops[2]{};
  ksj_provider_descriptor provider{};
  Metadata() {
    const std::string_view ids[2] = {kOpCoils, kOpRss};
    for (int i = 0; i < 2; ++i) {
      ksj_operator_descriptor& d = ops[i];
      d.abi = header(sizeof(d), KSJ_OPERATOR_CAP_CANCEL_NO_ALLOCATION | KSJ_OPERATOR_CAP_CANCEL_NO_THROW);
      d.operator_id = utf8(ids[i].data(), ids[i].size());
      d.max_in_flight = 1;
      d.thread_safety = KSJ_PROVIDER_SERIAL_INSTANCE;
      d.max_input_items_per_firing = 2;
      d.max_output_items_per_firing = 1;
      d.max_output_bytes_per_firing = i == 0 ? kMaxOutputBytes : uint64_t{kMaxImage} * kMaxImage * 4;
      d.max_scratch_bytes_per_firing = 0;
    }
    provider.abi = header(sizeof(provider), KSJ_PROVIDER_CAP_SYNC_PROCESS | KSJ_PROVIDER_CAP_NO_PRIVATE_THREADS |
                                                KSJ_PROVIDER_CAP_NO_DIRECT_FILE_IO |
                                                KSJ_PROVIDER_CAP_NO_DIRECT_NETWORK_IO);
    provider.provider_id = utf8(kProviderId, sizeof(kProviderId) - 1);
    provider.bundle_digest = digest_from_hex(kBundleDigestHex);
    provider.operator_count = 2;
    provider.operators = ops;
  }
};

const Metadata& metadata() {
  static const Metadata m;
  return m;
}

}  // namespace

KSJ_PROVIDER_ENTRY ksj_status KSJ_PROVIDER_CALL ksj_provider_query(const ksj_provider_query_request* req,
                                                                   ksj_provider_descriptor* out_descriptor,
                                                                   ksj_provider_api* out_api,
                                                                   ksj_error_view* err) {
  try {
    if (!full_header(req) || !full_header(out_descriptor) || !full_header(out_api))
      return fail(err, KSJ_STATUS_BAD_ABI, kErrBadAbi);
    if (!full_header(&req->host_build_id) || (req->host_build_id.size != 0 && req->host_build_id.data == nullptr))
      return fail(err, KSJ_STATUS_BAD_ABI, kErrBadAbi);
    *out_descriptor = metadata().provider;
    *out_api = {};
    out_api->abi = header(sizeof(*out_api));
    out_api->operator_create = &create;
    out_api->execution_context_create = &context_create;
    out_api->key_state_init = &key_init;
    out_api->operator_on_start = &on_start;
    out_api->operator_process_batch = &process_batch;
    out_api->operator_on_scan_end = &on_scan_end;
    out_api->operator_on_cancel = &on_cancel;
    out_api->key_state_reset = &key_reset;
    out_api->execution_context_destroy = &context_destroy;
    out_api->operator_destroy = &destroy;
    return KSJ_STATUS_OK;
  } catch (...) {
    return fail(err, KSJ_STATUS_INTERNAL_ERROR, kErrInternal);
  }
}
