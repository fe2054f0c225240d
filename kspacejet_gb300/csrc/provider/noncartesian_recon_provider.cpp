// noncartesian_recon_provider.cpp -- GB300 drop-in for the
// `org.kspacejet.noncartesian-recon` Provider plug-in.
//
// Same descriptor (provider id, operator ids and order, bounds, capability
// bits, bundle digest), same canonical configs, same port resolution, same
// rejections in the same order, same output payloads as
// providers/kspacejet-noncartesian-recon (src/provider_api.cpp:36-325,
// src/operators/radial_gridding_reconstruct.cpp, src/operators/
// noncartesian_adjoint_reconstruct.cpp).  The arithmetic runs on the GPU
// through ksj_gpu.h; there is no CPU path.  Payloads stay host memory (the
// registry types allow only host_normal), so a firing copies its inputs to
// the device and its output back.
//
// Device resources (declared, not hidden): one ksj_gpu_context per operator
// instance -- one non-blocking stream and a grow-only device workspace sized
// to the configured shape -- created at the first firing that passes
// validation and freed by operator_destroy.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <string_view>

#include "abi_support.hpp"
#include "ksj_gpu.h"
#include "ksj_provider_abi.h"

using namespace ksj_gb300;

namespace {

constexpr char kProviderId[] = "org.kspacejet.noncartesian-recon";
// SHA-256 over the NUL-delimited fields "kspacejet.provider-bundle", the
// Provider id and the operator ids in descriptor order -- unchanged from the
// reference because the operator set is unchanged.
constexpr char kBundleDigestHex[] = "4297da20fe070aae1988f456967aeed82d5bae62f8aad41585e25fe767000ef6";

constexpr std::string_view kErrBadAbi = "Non-Cartesian reconstruction Provider received incompatible ABI storage";
constexpr std::string_view kErrInvalidArgument =
    "Non-Cartesian reconstruction Provider received an invalid lifecycle argument";
constexpr std::string_view kErrUnsupportedOperator =
    "Non-Cartesian reconstruction Provider does not expose the requested operator";
constexpr std::string_view kErrInternal = "Non-Cartesian reconstruction Provider trapped an unexpected internal exception";
constexpr std::string_view kErrDevice =
    "GB300 non-Cartesian reconstruction Provider could not use its CUDA device (no device, out of memory, or a "
    "kernel failure)";
constexpr std::string_view kErrNonfinite =
    "Non-Cartesian reconstruction rejected a non-finite sample, trajectory or density-compensation value";

constexpr uint32_t kMaxDimension = 512;
constexpr uint32_t kMaxChannels = 64;
constexpr uint32_t kMaxSamples = 65536;
constexpr uint64_t kMaxPixels = uint64_t{kMaxDimension} * kMaxDimension;
constexpr uint64_t kMaxKspaceBytes = uint64_t{kMaxChannels} * kMaxSamples * 8;
constexpr uint64_t kMaxTrajectoryBytes = uint64_t{kMaxSamples} * 2 * 4;
constexpr uint64_t kMaxCoilImageBytes = kMaxPixels * kMaxChannels * 8;
constexpr uint64_t kMaxDirectWork = uint64_t{1} << 28;
constexpr uint32_t kAlignment = 64;

enum class Op { kDirectAdjoint = 0, kRadialGridding = 1 };

struct OperatorSpec {
  std::string_view id;
  std::string_view unsupported_config;
  std::string_view lease, kspace, trajectory, identity, output, scratch, internal;
  uint64_t max_output_bytes;
  uint64_t max_scratch_bytes;
};

// noncartesian_adjoint_reconstruct.cpp:33-49 and radial_gridding_reconstruct.cpp:34-55
const OperatorSpec kSpecs[2] = {
    {"noncartesian_adjoint_reconstruct",
     "Non-Cartesian reconstruction Provider requires canonical "
     "{\"channels\":N,\"image_cols\":N,\"image_rows\":N,\"sample_count\":N} within its direct-adjoint bound",
     "Non-Cartesian reconstruction Provider requires two input batches, one output grant, and one bounded image "
     "scratch plane",
     "Non-Cartesian reconstruction Provider requires one exact ksj.noncartesian-kspace-frame on input port 0",
     "Non-Cartesian reconstruction Provider requires one exact finite ksj.trajectory-frame on input port 1",
     "Non-Cartesian k-space and trajectory inputs must have equal semantic_key_hash and order_key",
     "Non-Cartesian reconstruction Provider requires one exact ksj.coil-image-frame output grant",
     "Non-Cartesian reconstruction Provider scratch grant is too small or incompatible",
     "Non-Cartesian reconstruction Provider trapped an unexpected internal exception",
     kMaxCoilImageBytes, kMaxPixels * 8},
    {"radial_gridding_reconstruct",
     "Non-Cartesian reconstruction Provider radial_gridding_reconstruct requires canonical "
     "{\"channels\":N,\"density_compensation\":\"radial_analytic_ramp\",\"image_cols\":N,\"image_rows\":N,"
     "\"sample_count\":N,\"trajectory_units\":\"radians_per_pixel\"} with power-of-two image dimensions within its "
     "bounded radial-gridding envelope",
     "Non-Cartesian radial gridding requires two input batches, one output grant, and bounded caller-owned gridding "
     "workspace",
     "Non-Cartesian radial gridding requires one exact ksj.noncartesian-kspace-frame on input port 0",
     "Non-Cartesian radial gridding requires one exact finite ksj.trajectory-frame on input port 1 in "
     "radians_per_pixel within [-pi, pi]",
     "Non-Cartesian radial k-space and trajectory inputs must have equal semantic_key_hash and order_key",
     "Non-Cartesian radial gridding requires one exact ksj.coil-image-frame output grant",
     "Non-Cartesian radial gridding scratch grant is too small or incompatible",
     "Non-Cartesian radial gridding trapped an unexpected internal exception",
     kMaxCoilImageBytes, (2 * kMaxPixels + 2 * kMaxDimension) * 8 + uint64_t{kMaxSamples} * 4},
};

}  // namespace

struct ksj_execution_context {
  ksj_provider_operator* owner = nullptr;
};
struct ksj_key_state {
  ksj_provider_operator* owner = nullptr;
};
struct ksj_provider_operator {
  Op op = Op::kDirectAdjoint;
  uint32_t channels = 0, image_rows = 0, image_cols = 0, sample_count = 0;
  ksj_execution_context context{};
  ksj_key_state key_state{};
  bool context_active = false;
  bool key_state_active = false;
  ksj_gpu_context* gpu = nullptr;
  uint32_t device = 0;
};

namespace {

struct Shape {
  uint64_t pixels, kspace_bytes, trajectory_bytes, coil_image_bytes, scratch_bytes;
};

// shape_bytes of each operator (radial :146-176, direct :152-170)
bool shape_bytes(const ksj_provider_operator& o, Shape* s) {
  if (o.channels == 0 || o.channels > kMaxChannels || o.image_rows < 2 || o.image_rows > kMaxDimension ||
      o.image_cols < 2 || o.image_cols > kMaxDimension || o.sample_count == 0 || o.sample_count > kMaxSamples)
    return false;
  s->pixels = uint64_t{o.image_rows} * o.image_cols;
  s->kspace_bytes = uint64_t{o.channels} * o.sample_count * 8;
  s->trajectory_bytes = uint64_t{o.sample_count} * 2 * 4;
  s->coil_image_bytes = s->pixels * o.channels * 8;
  if (o.op == Op::kRadialGridding) {
    if (!pow2(o.image_rows) || !pow2(o.image_cols)) return false;
    const uint64_t line = o.image_rows > o.image_cols ? o.image_rows : o.image_cols;
    s->scratch_bytes = (2 * s->pixels + 2 * line) * 8 + uint64_t{o.sample_count} * 4;
    if (s->scratch_bytes > kSpecs[1].max_scratch_bytes) return false;
  } else {
    s->scratch_bytes = s->pixels * 8;
    if (s->pixels * o.channels * o.sample_count > kMaxDirectWork) return false;
  }
  return s->pixels <= kMaxPixels && s->kspace_bytes <= kMaxKspaceBytes &&
         s->trajectory_bytes <= kMaxTrajectoryBytes && s->coil_image_bytes <= kMaxCoilImageBytes;
}

bool configure(Op op, const ksj_byte_view& config, ksj_provider_operator* o) {
  std::string_view v[6];
  o->op = op;
  if (op == Op::kRadialGridding) {
    const std::string_view lit[] = {"{\"channels\":",
                                    ",\"density_compensation\":\"radial_analytic_ramp\"",
                                    ",\"image_cols\":",
                                    ",\"image_rows\":",
                                    ",\"sample_count\":",
                                    ",\"trajectory_units\":\"radians_per_pixel\"}"};
    if (!split_canonical(config, lit, 6, v)) return false;
    // v[1] (between the DCF literal and ",\"image_cols\":") is not a value;
    // the reference searches past it (radial_gridding_reconstruct.cpp:118-121)
    if (!parse_u32(v[0], 1, kMaxChannels, &o->channels) || !parse_u32(v[2], 2, kMaxDimension, &o->image_cols) ||
        !parse_u32(v[3], 2, kMaxDimension, &o->image_rows) || !parse_u32(v[4], 1, kMaxSamples, &o->sample_count))
      return false;
    if (!pow2(o->image_rows) || !pow2(o->image_cols)) return false;
  } else {
    const std::string_view lit[] = {"{\"channels\":", ",\"image_cols\":", ",\"image_rows\":", ",\"sample_count\":",
                                    "}"};
    if (!split_canonical(config, lit, 5, v)) return false;
    if (!parse_u32(v[0], 1, kMaxChannels, &o->channels) || !parse_u32(v[1], 2, kMaxDimension, &o->image_cols) ||
        !parse_u32(v[2], 2, kMaxDimension, &o->image_rows) || !parse_u32(v[3], 1, kMaxSamples, &o->sample_count))
      return false;
    if (uint64_t{o->channels} * o->image_rows * o->image_cols * o->sample_count > kMaxDirectWork) return false;
  }
  Shape s;
  return shape_bytes(*o, &s);
}

bool is_operator(const ksj_provider_operator* o) {
  Shape s;
  return o != nullptr && (o->op == Op::kDirectAdjoint || o->op == Op::kRadialGridding) && shape_bytes(*o, &s);
}
bool is_context(const ksj_provider_operator* o, const ksj_execution_context* c) {
  return is_operator(o) && c == &o->context && c->owner == o && o->context_active;
}
bool is_key_state(const ksj_provider_operator* o, const ksj_key_state* k) {
  return is_operator(o) && k == &o->key_state && k->owner == o && o->key_state_active;
}

bool exact_batch(const ksj_input_batch_view& b, uint32_t port) {
  return full_header(&b) && b.input_port == port && b.item_count == 1 && b.items != nullptr &&
         full_header(&b.items[0]);
}

// GPU work of one firing: inputs already validated; returns a ksj_status.
ksj_status run_gpu(ksj_provider_operator& o, const Shape& s, const void* kspace_host, const void* traj_host,
                   void* out_host, const OperatorSpec& spec, ksj_error_view* err) {
  if (o.gpu == nullptr && ksj_gpu_context_create(static_cast<int>(o.device), &o.gpu) != KSJ_GPU_OK)
    return fail(err, KSJ_STATUS_FAILED_PRECONDITION, kErrDevice);
  void *d_k = nullptr, *d_t = nullptr, *d_o = nullptr, *d_w = nullptr;
  size_t ws_bytes = 0;
  ksj_gpu_gridding_desc desc{};
  if (o.op == Op::kRadialGridding) {
    desc.struct_size = sizeof(desc);
    desc.kernel = KSJ_GPU_KERNEL_LINEAR;
    desc.image_rows = desc.grid_rows = o.image_rows;
    desc.image_cols = desc.grid_cols = o.image_cols;
    desc.kernel_width = 2;
    // Grid2D origin ((N-1)/2, (N-1)/2) (radial_gridding_reconstruct.cpp:383-388)
    desc.row_origin = static_cast<double>(o.image_rows - 1) / 2.0;
    desc.col_origin = static_cast<double>(o.image_cols - 1) / 2.0;
    desc.channels = o.channels;
    desc.samples = o.sample_count;
    desc.frames = 1;
    desc.dcf_mode = KSJ_GPU_DCF_ANALYTIC_RAMP;
    desc.output = KSJ_GPU_OUTPUT_COIL_LAST;
    desc.sample_format = KSJ_GPU_SAMPLES_CF32;
    desc.require_nyquist = 1;
    ws_bytes = ksj_gpu_gridding_workspace_bytes(&desc);
  } else {
    ws_bytes = ksj_gpu_direct_workspace_bytes(o.image_rows, o.image_cols, o.channels);
  }
  if (ws_bytes == 0 || ksj_gpu_context_buffer(o.gpu, 0, s.kspace_bytes, &d_k) != KSJ_GPU_OK ||
      ksj_gpu_context_buffer(o.gpu, 1, s.trajectory_bytes, &d_t) != KSJ_GPU_OK ||
      ksj_gpu_context_buffer(o.gpu, 2, s.coil_image_bytes, &d_o) != KSJ_GPU_OK ||
      ksj_gpu_context_buffer(o.gpu, 3, ws_bytes, &d_w) != KSJ_GPU_OK)
    return fail(err, KSJ_STATUS_RESOURCE_EXHAUSTED, kErrDevice);
  if (ksj_gpu_context_copy(o.gpu, d_k, kspace_host, s.kspace_bytes, 0) != KSJ_GPU_OK ||
      ksj_gpu_context_copy(o.gpu, d_t, traj_host, s.trajectory_bytes, 0) != KSJ_GPU_OK)
    return fail(err, KSJ_STATUS_INTERNAL_ERROR, kErrDevice);
  void* stream = ksj_gpu_context_stream(o.gpu);
  ksj_gpu_status st;
  if (o.op == Op::kRadialGridding) {
    st = ksj_gpu_gridding_adjoint(&desc, nullptr, d_k, static_cast<const float*>(d_t), nullptr, d_o, d_w, ws_bytes,
                                  stream);
  } else {
    st = ksj_gpu_direct_adjoint(o.image_rows, o.image_cols, static_cast<double>(o.image_rows - 1) / 2.0,
                                static_cast<double>(o.image_cols - 1) / 2.0, o.channels, o.sample_count, d_k,
                                static_cast<const float*>(d_t), d_o, d_w, ws_bytes, stream);
  }
  if (st != KSJ_GPU_OK) return fail(err, KSJ_STATUS_INTERNAL_ERROR, kErrDevice);
  if (ksj_gpu_context_copy(o.gpu, out_host, d_o, s.coil_image_bytes, 1) != KSJ_GPU_OK)
    return fail(err, KSJ_STATUS_INTERNAL_ERROR, kErrDevice);
  if (o.op == Op::kRadialGridding) {
    uint32_t flags = 0;
    if (ksj_gpu_read_flags(d_w, stream, &flags) != KSJ_GPU_OK) return fail(err, KSJ_STATUS_INTERNAL_ERROR, kErrDevice);
    // the reference library throws on a non-finite sample and the operator
    // turns that into INTERNAL_ERROR (radial_gridding_reconstruct.cpp:432-435)
    if (flags != 0) return fail(err, KSJ_STATUS_INTERNAL_ERROR, spec.internal);
  } else if (ksj_gpu_context_sync(o.gpu) != KSJ_GPU_OK) {
    return fail(err, KSJ_STATUS_INTERNAL_ERROR, kErrDevice);
  }
  return KSJ_STATUS_OK;
}

ksj_status process(ksj_provider_operator& o, ksj_firing_lease* lease, const ksj_firing_lease_callbacks* cb,
                   ksj_process_result* out_result, ksj_error_view* err) {
  const OperatorSpec& spec = kSpecs[static_cast<int>(o.op)];
  if (lease == nullptr || !full_header(out_result)) return fail(err, KSJ_STATUS_INVALID_ARGUMENT, kErrBadAbi);
  if (!lease_callbacks_ok(cb, KSJ_LEASE_CAP_INPUT_BATCHES | KSJ_LEASE_CAP_OUTPUT_GRANTS | KSJ_LEASE_CAP_SCRATCH))
    return fail(err, KSJ_STATUS_BAD_ABI, kErrBadAbi);
  Shape s;
  if (!shape_bytes(o, &s)) return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, spec.unsupported_config);

  ksj_firing_lease_info info{};
  info.abi = header(sizeof(info));
  const ksj_status info_status = cb->get_info(cb->host_context, lease, &info, err);
  if (info_status != KSJ_STATUS_OK || !full_header(&info) || info.input_batch_count != 2 ||
      info.output_grant_count != 1 || info.reserved_output_bytes < s.coil_image_bytes ||
      info.reserved_scratch_bytes < s.scratch_bytes)
    return info_status == KSJ_STATUS_OK ? fail(err, KSJ_STATUS_CONTRACT_VIOLATION, spec.lease) : info_status;

  ksj_input_batch_view batches[2]{};
  for (uint32_t i = 0; i < 2; ++i) {
    batches[i].abi = header(sizeof(batches[i]));
    const ksj_status bs = cb->get_input_batch(cb->host_context, lease, i, &batches[i], err);
    if (bs != KSJ_STATUS_OK) return bs;
  }
  if (!full_header(&batches[0]) || !full_header(&batches[1]))
    return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, spec.lease);
  // resolve by port id, not batch index (radial_gridding_reconstruct.cpp:278-301)
  const ksj_input_batch_view* kb = nullptr;
  const ksj_input_batch_view* tb = nullptr;
  for (const ksj_input_batch_view* b : {&batches[0], &batches[1]}) {
    if (b->input_port == 0) {
      if (kb != nullptr) return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, spec.kspace);
      kb = b;
    } else if (b->input_port == 1) {
      if (tb != nullptr) return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, spec.trajectory);
      tb = b;
    } else {
      return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, spec.lease);
    }
  }
  if (kb == nullptr || !exact_batch(*kb, 0)) return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, spec.kspace);
  if (tb == nullptr || !exact_batch(*tb, 1)) return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, spec.trajectory);
  const ksj_input_item_view& k = kb->items[0];
  const ksj_input_item_view& t = tb->items[0];
  if (!full_header(&k.payload) || k.payload.data == nullptr || k.payload.byte_count != s.kspace_bytes ||
      k.payload.memory_domain != KSJ_PROVIDER_MEMORY_HOST_PAGEABLE ||
      !host_memory_ok(k.payload.data, k.payload.alignment, kAlignment) || !borrowed_ok(k.metadata) ||
      !type_matches(k.payload.type, kNoncartesianKspaceFrame))
    return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, spec.kspace);
  if (!full_header(&t.payload) || t.payload.data == nullptr || t.payload.byte_count != s.trajectory_bytes ||
      t.payload.memory_domain != KSJ_PROVIDER_MEMORY_HOST_PAGEABLE ||
      !host_memory_ok(t.payload.data, t.payload.alignment, kAlignment) || !borrowed_ok(t.metadata) ||
      !type_matches(t.payload.type, kTrajectoryFrame))
    return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, spec.trajectory);
  if (k.semantic_key_hash != t.semantic_key_hash || k.order_key != t.order_key)
    return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, spec.identity);

  // host trajectory check: finite (and in [-pi, pi] for the radial operator)
  const float* tv = static_cast<const float*>(t.payload.data);
  constexpr float kPi = 3.14159265358979323846f;
  for (uint64_t i = 0; i < uint64_t{o.sample_count} * 2; ++i) {
    const bool finite = std::isfinite(tv[i]);
    if (!finite || (o.op == Op::kRadialGridding && (tv[i] < -kPi || tv[i] > kPi)))
      return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, spec.trajectory);
  }

  ksj_scratch_view scratch{};
  scratch.abi = header(sizeof(scratch));
  const ksj_status ss = cb->get_scratch(cb->host_context, lease, &scratch, err);
  if (ss != KSJ_STATUS_OK) return ss;
  // the scratch grant is validated exactly as the reference does, although
  // the device path keeps its working set in HBM
  // radial: 64 bytes (:336); direct: alignof(std::complex<float>) = 4 (:322)
  const uint32_t scratch_align = o.op == Op::kRadialGridding ? kAlignment : 4u;
  if (!full_header(&scratch) || scratch.data == nullptr || scratch.byte_count < s.scratch_bytes ||
      scratch.memory_domain != KSJ_PROVIDER_MEMORY_HOST_PAGEABLE ||
      !host_memory_ok(scratch.data, scratch.alignment, scratch_align))
    return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, spec.scratch);

  ksj_output_grant* grant = nullptr;
  const ksj_status as = cb->acquire_output_grant(cb->host_context, lease, 0, &grant, err);
  if (as != KSJ_STATUS_OK || grant == nullptr)
    return as == KSJ_STATUS_OK ? fail(err, KSJ_STATUS_CONTRACT_VIOLATION, spec.output) : as;
  GrantGuard guard{cb->output_grants, grant, false};

  ksj_mutable_payload_view out{};
  out.abi = header(sizeof(out));
  const ksj_status ms = cb->output_grants->map_mutable_payload(cb->output_grants->host_context, grant, &out, err);
  if (ms != KSJ_STATUS_OK) return ms;
  if (!full_header(&out) || out.data == nullptr || out.capacity_bytes < s.coil_image_bytes ||
      out.committed_bytes != 0 || out.memory_domain != KSJ_PROVIDER_MEMORY_HOST_PAGEABLE ||
      !host_memory_ok(out.data, out.alignment, kAlignment) || !type_matches(out.type, kCoilImageFrame))
    return fail(err, KSJ_STATUS_CONTRACT_VIOLATION, spec.output);

  const ksj_status gs = run_gpu(o, s, k.payload.data, t.payload.data, out.data, spec, err);
  if (gs != KSJ_STATUS_OK) return gs;

  ksj_output_seal_descriptor seal{};
  seal.abi = header(sizeof(seal));
  seal.output_port = 0;
  seal.produced_item_count = 1;
  seal.produced_byte_count = s.coil_image_bytes;
  seal.semantic_key_hash = k.semantic_key_hash;
  seal.order_key = k.order_key;
  seal.type = out.type;
  seal.metadata = k.metadata;
  const ksj_status sealed = cb->output_grants->seal(cb->output_grants->host_context, grant, &seal, err);
  if (sealed != KSJ_STATUS_OK) return sealed;
  guard.settled = true;
  done(out_result, 1, 2, info.terminal_epoch);
  return KSJ_STATUS_OK;
}

// ----------------------------------------------------------- lifecycle table

ksj_operator_descriptor operator_descriptor(const OperatorSpec& spec) {
  ksj_operator_descriptor d{};
  d.abi = header(sizeof(d), KSJ_OPERATOR_CAP_CANCEL_NO_ALLOCATION | KSJ_OPERATOR_CAP_CANCEL_NO_THROW);
  d.operator_id = utf8(spec.id.data(), spec.id.size());
  d.max_in_flight = 1;
  d.thread_safety = KSJ_PROVIDER_SERIAL_INSTANCE;
  d.max_private_threads = 0;
  d.max_input_items_per_firing = 2;
  d.max_output_items_per_firing = 1;
  d.max_output_bytes_per_firing = spec.max_output_bytes;
  d.max_scratch_bytes_per_firing = spec.max_scratch_bytes;
  return d;
}

struct Metadata {
  ksj_operator_descriptor ops[2];
  ksj_provider_descriptor provider;
  Metadata() {
    ops[0] = operator_descriptor(kSpecs[0]);
    ops[1] = operator_descriptor(kSpecs[1]);
    provider = {};
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

ksj_status operator_create(const ksj_operator_create_request* req, ksj_provider_operator** out,
                           ksj_error_view* err) noexcept {
  try {
    if (!full_header(req) || out == nullptr) return fail(err, KSJ_STATUS_INVALID_ARGUMENT, kErrInvalidArgument);
    *out = nullptr;
    int which = -1;
    for (int i = 0; i < 2; ++i)
      if (text_is(req->operator_id, kSpecs[i].id)) which = i;
    if (which < 0) return fail(err, KSJ_STATUS_UNSUPPORTED, kErrUnsupportedOperator);
    if (req->host_services != nullptr && !full_header(req->host_services))
      return fail(err, KSJ_STATUS_BAD_ABI, kErrBadAbi);
    ksj_provider_operator configured{};
    if (!configure(static_cast<Op>(which), req->canonical_config, &configured))
      return fail(err, KSJ_STATUS_INVALID_ARGUMENT, kSpecs[which].unsupported_config);
    auto* o = new (std::nothrow) ksj_provider_operator{configured};
    if (o == nullptr) return fail(err, KSJ_STATUS_RESOURCE_EXHAUSTED, kErrInternal);
    *out = o;
    return KSJ_STATUS_OK;
  } catch (...) {
    return fail(err, KSJ_STATUS_INTERNAL_ERROR, kErrInternal);
  }
}

ksj_status execution_context_create(ksj_provider_operator* o, const ksj_execution_context_descriptor* d,
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

ksj_status key_state_init(ksj_provider_operator* o, ksj_execution_context* c, const ksj_key_state_descriptor* d,
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
    return fail(err, KSJ_STATUS_INTERNAL_ERROR, kSpecs[static_cast<int>(o->op)].internal);
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

void key_state_reset(ksj_provider_operator* o, ksj_execution_context* c, ksj_key_state* k) noexcept {
  if (!is_context(o, c) || !is_key_state(o, k)) return;
  o->key_state.owner = nullptr;
  o->key_state_active = false;
}

void execution_context_destroy(ksj_provider_operator* o, ksj_execution_context* c) noexcept {
  if (!is_context(o, c)) return;
  o->context.owner = nullptr;
  o->context_active = false;
}

void operator_destroy(ksj_provider_operator* o) noexcept {
  if (o == nullptr) return;
  if (o->gpu != nullptr) ksj_gpu_context_destroy(o->gpu);
  delete o;
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
    out_api->operator_create = &operator_create;
    out_api->execution_context_create = &execution_context_create;
    out_api->key_state_init = &key_state_init;
    out_api->operator_on_start = &on_start;
    out_api->operator_process_batch = &process_batch;
    out_api->operator_on_scan_end = &on_scan_end;
    out_api->operator_on_cancel = &on_cancel;
    out_api->key_state_reset = &key_state_reset;
    out_api->execution_context_destroy = &execution_context_destroy;
    out_api->operator_destroy = &operator_destroy;
    return KSJ_STATUS_OK;
  } catch (...) {
    return fail(err, KSJ_STATUS_INTERNAL_ERROR, kErrInternal);
  }
}
