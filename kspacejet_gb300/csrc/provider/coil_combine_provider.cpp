// coil_combine_provider.cpp -- GB300 drop-in for the `org.kspacejet.coil-combine`
// Provider plug-in: operator coil_combine_rss, ksj.coil-image-frame
// [ky, kx, channel] complex64 -> ksj.image-frame [ky, kx] float32, root sum of
// squares over channels.
//
// Descriptor, config grammar {"channels":C,"cols":N,"rows":N}, validation
// order and seal (empty metadata) follow providers/kspacejet-coil-combine
// (src/provider_api.cpp:15-71, src/operators/coil_combine_rss.cpp:28-331).
// The sum runs on the GPU (ksj_gpu_rss_coil_last) in the reference's channel
// order and rounding, so outputs are bit-identical to the reference's float
// arithmetic on the same input.
#include <cstdint>
#include <new>
#include <string_view>

#include "abi_support.hpp"
#include "ksj_gpu.h"
#include "ksj_provider_abi.h"

using namespace ksj_gb300;

namespace {

constexpr char kProviderId[] = "org.kspacejet.coil-combine";
constexpr char kBundleDigestHex[] = "ba4f619047391419c8ffc42220ace7d888f047c9e2fd64aaeb78d9093191aed5";
constexpr std::string_view kOperatorId = "coil_combine_rss";
constexpr std::string_view kErrBadAbi = "Coil-combine Provider received incompatible ABI storage";
constexpr std::string_view kErrInvalidArgument = "Coil-combine Provider received an invalid lifecycle argument";
constexpr std::string_view kErrUnsupportedOperator = "Coil-combine Provider does not expose the requested operator";
constexpr std::string_view kErrUnsupportedConfig =
    "Coil-combine Provider requires canonical {\"channels\":N,\"cols\":N,\"rows\":N} dimensions";
constexpr std::string_view kErrLease = "Coil-combine Provider requires one input frame and one output grant";
constexpr std::string_view kErrInput = "Coil-combine Provider requires one exact ksj.coil-image-frame payload";
constexpr std::string_view kErrOutput = "Coil-combine Provider requires one exact ksj.image-frame output grant";
constexpr std::string_view kErrInternal = "Coil-combine Provider trapped an unexpected internal exception";
constexpr std::string_view kErrDevice =
    "GB300 coil-combine Provider could not use its CUDA device (no device, out of memory, or a kernel failure)";

constexpr uint32_t kMaxDimension = 512;
constexpr uint32_t kMaxChannels = 64;
constexpr uint64_t kMaxPixels = uint64_t{kMaxDimension} * kMaxDimension;
constexpr uint64_t kMaxImageBytes = kMaxPixels * 4;

}  // namespace

struct ksj_execution_context {
  ksj_provider_operator* owner = nullptr;
};
struct ksj_key_state {
  ksj_provider_operator* owner = nullptr;
};
struct ksj_provider_operator {
  uint32_t channels = 0, rows = 0, cols = 0;
  ksj_execution_context context{};
  ksj_key_state key_state{};
  bool context_active = false;
  bool key_state_active = false;
  ksj_gpu_context* gpu = nullptr;
  uint32_t device = 0;
};

namespace {

bool shape(const ksj_provider_operator& o, uint64_t* pixels, uint64_t* coil_bytes) {
  if (o.channels == 0 || o.channels > kMaxChannels || o.rows < 2 || o.rows > kMaxDimension || o.cols < 2 ||
      o.cols > kMaxDimension)
    return false;
  *pixels = uint64_t{o.rows} * o.cols;
  *coil_bytes = *pixels * o.channels * 8;
  return true;
}

bool is_operator(const ksj_provider_operator* o) {
  uint64_t p, b;
  return o != nullptr && shape(*o, &p, &b);
}
bool is_context(const ksj_provider_operator* o, const ksj_execution_context* c) {
  return is_operator(o) && c == &o->context && c->owner == o && o->context_active;
}
bool is_key_state(const ksj_provider_operator* o, const ksj_key_state* k) {
  return is_operator(o) && k == &o->key_state && k->owner == o && o->key_state_active;
}

ksj_status create(const ksj_operator_create_request* req, ksj_provider_operator** out, ksj_error_view* err) noexcept {
  try {
    if (!full_header(req) || out == nullptr) return fail(err, KSJ_STATUS_INVALID_ARGUMENT, kErrInvalidArgument);
    *out = nullptr;
    if (!text_is(req->operator_id, kOperatorId)) return fail(err, KSJ_STATUS_UNSUPPORTED, kErrUnsupportedOperator);
    if (req->host_services != nullptr && !full_header(req->host_services))
      return fail(err, KSJ_STATUS_BAD_ABI, kErrBadAbi);
    const std::string_view lit[] = {"{\"channels\":", ",\"cols\":", ",\"rows\":", "}"};
    std::string_view v[3];
    ksj_provider_operator o{};
    if (!split_canonical(req->canonical_config, lit, 4, v) || !parse_u32(v[0], 1, kMaxChannels, &o.channels) ||
        !parse_u32(v[1], 2, kMaxDimension, &o.cols) || !parse_u32(v[2], 2, kMaxDimension, &o.rows))
      return fail(err, KSJ_STATUS_INVALID_ARGUMENT, kErrUnsupportedConfig);
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

ksj_status process(ksj_provider_operator* o, ksj_execution_context* c, ksj_key_state* k, ksj_firing_lease* lease,
                   const ksj_firing_lease_callbacks* cb, ksj_process_result* result, ksj_error_view* err) noexcept {
  try {
    if (!is_context(o, c) || !is_key_state(o, k) || lease == nullptr || !full_header(result))
      return fail(err, KSJ_STATUS_INVALID_ARGUMENT, kErrInvalidArgument);
    if (!lease_callbacks_ok(cb, KSJ_LEASE_CAP_INPUT_BATCHES | KSJ_LEASE_CAP_OUTPUT_GRANTS))
      return fail(err, KSJ_STATUS_BAD_ABI, kErrBadAbi);
    uint64_t pixels = 0, coil_bytes = 0;
    if (!shape(*o, &pixels, &coil_bytes)) return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrInput);
    const uint64_t image_bytes = pixels * 4;
    ksj_firing_lease_info info{};
    info.abi = header(sizeof(info));
    const ksj_status is = cb->get_info(cb->host_context, lease, &info, err);
    if (is != KSJ_STATUS_OK || !full_header(&info) || info.input_batch_count != 1 || info.output_grant_count != 1 ||
        info.reserved_output_bytes < image_bytes)
      return is == KSJ_STATUS_OK ? fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrLease) : is;
    ksj_input_batch_view batch{};
    batch.abi = header(sizeof(batch));
    const ksj_status bs = cb->get_input_batch(cb->host_context, lease, 0, &batch, err);
    if (bs != KSJ_STATUS_OK) return bs;
    if (!full_header(&batch) || batch.input_port != 0 || batch.item_count != 1 || batch.items == nullptr ||
        !full_header(&batch.items[0]))
      return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrInput);
    const ksj_input_item_view& in = batch.items[0];
    if (!full_header(&in.payload) || in.payload.data == nullptr || in.payload.byte_count != coil_bytes ||
        in.payload.memory_domain != KSJ_PROVIDER_MEMORY_HOST_PAGEABLE ||
        !host_memory_ok(in.payload.data, in.payload.alignment, 64) || !borrowed_ok(in.metadata) ||
        !type_matches(in.payload.type, kCoilImageFrame))
      return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrInput);
    ksj_output_grant* grant = nullptr;
    const ksj_status as = cb->acquire_output_grant(cb->host_context, lease, 0, &grant, err);
    if (as != KSJ_STATUS_OK || grant == nullptr)
      return as == KSJ_STATUS_OK ? fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrOutput) : as;
    GrantGuard guard{cb->output_grants, grant, false};
    ksj_mutable_payload_view out{};
    out.abi = header(sizeof(out));
    const ksj_status ms = cb->output_grants->map_mutable_payload(cb->output_grants->host_context, grant, &out, err);
    if (ms != KSJ_STATUS_OK) return ms;
    if (!full_header(&out) || out.data == nullptr || out.capacity_bytes < image_bytes || out.committed_bytes != 0 ||
        out.memory_domain != KSJ_PROVIDER_MEMORY_HOST_PAGEABLE || !host_memory_ok(out.data, out.alignment, 64) ||
        !type_matches(out.type, kImageFrame))
      return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, kErrOutput);

    if (o->gpu == nullptr && ksj_gpu_context_create(static_cast<int>(o->device), &o->gpu) != KSJ_GPU_OK)
      return fail(err, KSJ_STATUS_FAILED_PRECONDITION, kErrDevice);
    void *d_in = nullptr, *d_out = nullptr;
    if (ksj_gpu_context_buffer(o->gpu, 0, coil_bytes, &d_in) != KSJ_GPU_OK ||
        ksj_gpu_context_buffer(o->gpu, 1, image_bytes, &d_out) != KSJ_GPU_OK)
      return fail(err, KSJ_STATUS_RESOURCE_EXHAUSTED, kErrDevice);
    if (ksj_gpu_context_copy(o->gpu, d_in, in.payload.data, coil_bytes, 0) != KSJ_GPU_OK ||
        ksj_gpu_rss_coil_last(pixels, o->channels, d_in, static_cast<float*>(d_out), ksj_gpu_context_stream(o->gpu)) !=
            KSJ_GPU_OK ||
        ksj_gpu_context_copy(o->gpu, out.data, d_out, image_bytes, 1) != KSJ_GPU_OK ||
        ksj_gpu_context_sync(o->gpu) != KSJ_GPU_OK)
      return fail(err, KSJ_STATUS_INTERNAL_ERROR, kErrDevice);

    ksj_output_seal_descriptor seal{};
    seal.abi = header(sizeof(seal));
    seal.output_port = 0;
    seal.produced_item_count = 1;
    seal.produced_byte_count = image_bytes;
    seal.semantic_key_hash = in.semantic_key_hash;
    seal.order_key = in.order_key;
    seal.type = out.type;
    seal.metadata.abi = header(sizeof(seal.metadata));  // empty metadata (coil_combine_rss.cpp:318)
    const ksj_status ss = cb->output_grants->seal(cb->output_grants->host_context, grant, &seal, err);
    if (ss != KSJ_STATUS_OK) return ss;
    guard.settled = true;
    done(result, 1, 1, info.terminal_epoch);
    return KSJ_STATUS_OK;
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
  ksj_operator_descriptor op{};
  ksj_provider_descriptor provider{};
  Metadata() {
    op.abi = header(sizeof(op), KSJ_OPERATOR_CAP_CANCEL_NO_ALLOCATION | KSJ_OPERATOR_CAP_CANCEL_NO_THROW);
    op.operator_id = utf8(kOperatorId.data(), kOperatorId.size());
    op.max_in_flight = 1;
    op.thread_safety = KSJ_PROVIDER_SERIAL_INSTANCE;
    op.max_input_items_per_firing = 1;
    op.max_output_items_per_firing = 1;
    op.max_output_bytes_per_firing = kMaxImageBytes;
    provider.abi = header(sizeof(provider), KSJ_PROVIDER_CAP_SYNC_PROCESS | KSJ_PROVIDER_CAP_NO_PRIVATE_THREADS |
                                                KSJ_PROVIDER_CAP_NO_DIRECT_FILE_IO |
                                                KSJ_PROVIDER_CAP_NO_DIRECT_NETWORK_IO);
    provider.provider_id = utf8(kProviderId, sizeof(kProviderId) - 1);
    provider.bundle_digest = digest_from_hex(kBundleDigestHex);
    provider.operator_count = 1;
    provider.operators = &op;
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
    out_api->operator_process_batch = &process;
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
