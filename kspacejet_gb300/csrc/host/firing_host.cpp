// firing_host.cpp -- a minimal synchronous KSpaceJet Provider host: dlopen a
// plug-in, query it, drive one operator instance through its lifecycle and
// fire it with caller-owned host buffers.  It plays the role of the
// reference's firing-lease host (libs/recon/kspacejet-recon-runtime/src/
// synchronous_firing_lease.cpp:805-865) and of the Provider unit tests'
// HostState callback tables (tests/unit/providers/kspacejet-noncartesian-
// recon/noncartesian_recon_provider_tests.cpp:71-280), including their fault
// knobs (reversed batch order, wrong type identity, short scratch, one input
// batch).  Any plug-in that exports ksj_provider_query can be driven: the GB300
// plug-ins and the reference's own.
#include <dlfcn.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../provider/abi_support.hpp"
#include "ksj_provider_abi.h"

using namespace ksj_gb300;

#define KSJH_API extern "C" __attribute__((visibility("default")))

namespace {

const PayloadType* kTypes[4] = {&kNoncartesianKspaceFrame, &kTrajectoryFrame, &kCoilImageFrame, &kImageFrame};

struct TypeStorage {
  ksj_utf8_view dims[4][3];
  ksj_type_descriptor_view desc[4];
  TypeStorage() {
    for (int t = 0; t < 4; ++t) {
      const PayloadType& p = *kTypes[t];
      for (uint32_t i = 0; i < p.rank; ++i) dims[t][i] = utf8(p.dims[i].data(), p.dims[i].size());
      ksj_type_descriptor_view d{};
      d.abi = header(sizeof(d));
      d.type_ref = utf8(p.type_ref.data(), p.type_ref.size());
      d.type_identity_digest = digest_from_hex(p.digest_hex);
      d.payload_kind = KSJ_PAYLOAD_KIND_BUFFER_HANDLE;
      d.element_type = p.element_type;
      d.rank = p.rank;
      d.dimension_names = dims[t];
      d.layout_flags = p.layout_flags;
      d.allowed_memory_domains = KSJ_PROVIDER_MEMORY_HOST_PAGEABLE;
      d.minimum_alignment = 64;
      d.mutability = KSJ_PAYLOAD_MUTABILITY_IMMUTABLE_AFTER_PUBLISH;
      desc[t] = d;
    }
  }
};

const TypeStorage& types() {
  static const TypeStorage t;
  return t;
}

ksj_error_view empty_error() {
  ksj_error_view e{};
  e.abi = header(sizeof(e));
  e.message.abi = header(sizeof(e.message));
  return e;
}

}  // namespace

struct ksjh_module {
  void* handle = nullptr;
  ksj_provider_descriptor descriptor{};
  ksj_provider_api api{};
};

struct ksjh_instance {
  ksjh_module* module = nullptr;
  ksj_provider_operator* op = nullptr;
  ksj_execution_context* context = nullptr;
  ksj_key_state* key = nullptr;
};

// One firing's inputs, fault knobs and observed results.
typedef struct ksjh_firing {
  uint32_t struct_size;
  uint32_t input_count;  // 1 or 2 batches of one item each
  const void* payload[2];
  uint64_t payload_bytes[2];
  uint32_t payload_type[2];  // 0 noncartesian-kspace, 1 trajectory, 2 coil-image, 3 image
  uint32_t payload_port[2];
  uint64_t semantic_key_hash[2];
  uint64_t order_key[2];
  const void* metadata;  // metadata of input 0
  uint64_t metadata_bytes;
  void* output;
  uint64_t output_capacity;
  uint32_t output_type;
  uint32_t reported_input_batch_count;
  void* scratch;
  uint64_t scratch_bytes;
  uint64_t reserved_output_bytes;
  uint64_t reserved_scratch_bytes;
  uint32_t reverse_batch_order;
  uint32_t corrupt_input_type;   // 1 + index of the input whose type digest is replaced, 0 = none
  uint32_t corrupt_output_type;  // nonzero: the output grant carries a wrong type digest
  uint32_t reserved0;
  uint64_t terminal_epoch;
  // results
  uint32_t status;
  uint32_t outcome;
  uint32_t sealed_count;
  uint32_t acquire_calls, map_calls, seal_calls, release_calls, input_batch_requests;
  uint64_t consumed;
  uint64_t sealed_bytes, sealed_key, sealed_order, sealed_metadata_size;
  const void* sealed_metadata;
  char error[512];
} ksjh_firing;

namespace {

struct Host {
  ksjh_firing* f;
  ksj_input_item_view items[2];
  ksj_input_batch_view batches[2];
  bool acquired = false, mapped = false, sealed = false;
  alignas(64) unsigned char grant_token = 0;
  ksj_output_grant* grant() { return reinterpret_cast<ksj_output_grant*>(&grant_token); }
};

ksj_status get_info(void* ctx, const ksj_firing_lease*, ksj_firing_lease_info* out, ksj_error_view*) {
  Host* h = static_cast<Host*>(ctx);
  if (h == nullptr || out == nullptr) return KSJ_STATUS_INVALID_ARGUMENT;
  *out = {};
  out->abi = header(sizeof(*out));
  out->terminal_epoch = h->f->terminal_epoch;
  out->input_batch_count = h->f->reported_input_batch_count;
  out->output_grant_count = 1;
  out->reserved_output_bytes = h->f->reserved_output_bytes;
  out->reserved_scratch_bytes = h->f->reserved_scratch_bytes;
  return KSJ_STATUS_OK;
}

ksj_status get_input_batch(void* ctx, const ksj_firing_lease*, uint32_t index, ksj_input_batch_view* out,
                           ksj_error_view*) {
  Host* h = static_cast<Host*>(ctx);
  if (h == nullptr || out == nullptr || index >= h->f->input_count) return KSJ_STATUS_INVALID_ARGUMENT;
  ++h->f->input_batch_requests;
  const uint32_t src = (h->f->reverse_batch_order && h->f->input_count == 2) ? 1 - index : index;
  *out = h->batches[src];
  return KSJ_STATUS_OK;
}

ksj_status get_scratch(void* ctx, const ksj_firing_lease*, ksj_scratch_view* out, ksj_error_view*) {
  Host* h = static_cast<Host*>(ctx);
  if (h == nullptr || out == nullptr) return KSJ_STATUS_INVALID_ARGUMENT;
  *out = {};
  out->abi = header(sizeof(*out));
  out->data = h->f->scratch;
  out->byte_count = h->f->scratch_bytes;
  out->memory_domain = KSJ_PROVIDER_MEMORY_HOST_PAGEABLE;
  out->alignment = 64;
  return KSJ_STATUS_OK;
}

ksj_status acquire(void* ctx, ksj_firing_lease*, uint32_t slot, ksj_output_grant** out, ksj_error_view*) {
  Host* h = static_cast<Host*>(ctx);
  if (h == nullptr || out == nullptr || slot != 0 || h->acquired) return KSJ_STATUS_CONTRACT_VIOLATION;
  ++h->f->acquire_calls;
  h->acquired = true;
  *out = h->grant();
  return KSJ_STATUS_OK;
}

ksj_status map_output(void* ctx, ksj_output_grant* g, ksj_mutable_payload_view* out, ksj_error_view*) {
  Host* h = static_cast<Host*>(ctx);
  if (h == nullptr || out == nullptr || g != h->grant() || !h->acquired || h->mapped)
    return KSJ_STATUS_CONTRACT_VIOLATION;
  ++h->f->map_calls;
  h->mapped = true;
  *out = {};
  out->abi = header(sizeof(*out));
  out->data = h->f->output;
  out->capacity_bytes = h->f->output_capacity;
  out->memory_domain = KSJ_PROVIDER_MEMORY_HOST_PAGEABLE;
  out->alignment = 64;
  out->type = types().desc[h->f->output_type & 3];
  if (h->f->corrupt_output_type)
    out->type.type_identity_digest = types().desc[(h->f->output_type + 1) & 3].type_identity_digest;
  return KSJ_STATUS_OK;
}

ksj_status seal_output(void* ctx, ksj_output_grant* g, const ksj_output_seal_descriptor* d, ksj_error_view*) {
  Host* h = static_cast<Host*>(ctx);
  if (h == nullptr || d == nullptr || g != h->grant() || !h->mapped || h->sealed || d->output_port != 0 ||
      d->produced_item_count != 1 || d->produced_byte_count > h->f->output_capacity)
    return KSJ_STATUS_CONTRACT_VIOLATION;
  ++h->f->seal_calls;
  h->sealed = true;
  h->f->sealed_bytes = d->produced_byte_count;
  h->f->sealed_key = d->semantic_key_hash;
  h->f->sealed_order = d->order_key;
  h->f->sealed_metadata = d->metadata.data;
  h->f->sealed_metadata_size = d->metadata.size;
  return KSJ_STATUS_OK;
}

ksj_status release_output(void* ctx, ksj_output_grant* g, ksj_error_view*) {
  Host* h = static_cast<Host*>(ctx);
  if (h == nullptr || g != h->grant() || h->sealed) return KSJ_STATUS_CONTRACT_VIOLATION;
  ++h->f->release_calls;
  return KSJ_STATUS_OK;
}

void copy_error(const ksj_error_view& e, char* out) {
  out[0] = 0;
  if (e.message.data != nullptr && e.message.size > 0) {
    const size_t n = e.message.size < 511 ? static_cast<size_t>(e.message.size) : 511;
    std::memcpy(out, e.message.data, n);
    out[n] = 0;
  }
}

}  // namespace

KSJH_API int ksjh_load(const char* path, ksjh_module** out, char* error, size_t error_capacity) {
  if (out == nullptr) return -1;
  *out = nullptr;
  void* handle = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (handle == nullptr) {
    if (error && error_capacity) std::snprintf(error, error_capacity, "%s", dlerror());
    return -1;
  }
  auto query = reinterpret_cast<ksj_provider_query_fn>(dlsym(handle, "ksj_provider_query"));
  if (query == nullptr) {
    if (error && error_capacity) std::snprintf(error, error_capacity, "missing ksj_provider_query");
    dlclose(handle);
    return -2;
  }
  auto* m = new (std::nothrow) ksjh_module{};
  if (m == nullptr) {
    dlclose(handle);
    return -3;
  }
  m->handle = handle;
  ksj_provider_query_request req{};
  req.abi = header(sizeof(req));
  req.host_build_id = utf8("ksj-gb300-firing-host", 21);
  m->descriptor.abi = header(sizeof(m->descriptor));
  m->api.abi = header(sizeof(m->api));
  ksj_error_view e = empty_error();
  const ksj_status st = query(&req, &m->descriptor, &m->api, &e);
  if (st != KSJ_STATUS_OK) {
    if (error && error_capacity) copy_error(e, error);
    dlclose(handle);
    delete m;
    return static_cast<int>(st) + 100;
  }
  *out = m;
  return 0;
}

KSJH_API void ksjh_unload(ksjh_module* m) {
  if (m == nullptr) return;
  if (m->handle) dlclose(m->handle);
  delete m;
}

KSJH_API int ksjh_describe(const ksjh_module* m, char* provider_id, size_t cap, uint8_t* digest,
                           uint32_t* operator_count, uint64_t* capability_bits) {
  if (m == nullptr) return -1;
  const ksj_provider_descriptor& d = m->descriptor;
  if (provider_id && cap) {
    const size_t n = d.provider_id.size < cap - 1 ? static_cast<size_t>(d.provider_id.size) : cap - 1;
    std::memcpy(provider_id, d.provider_id.data, n);
    provider_id[n] = 0;
  }
  if (digest) std::memcpy(digest, d.bundle_digest.bytes, 32);
  if (operator_count) *operator_count = d.operator_count;
  if (capability_bits) *capability_bits = d.abi.capability_bits;
  return 0;
}

// fields: [0] max_in_flight [1] thread_safety [2] max_private_threads [3] max_inputs [4] max_outputs
//         [5] max_output_bytes [6] max_scratch_bytes [7] max_retained [8] max_async_tail [9] capability bits
KSJH_API int ksjh_operator_info(const ksjh_module* m, uint32_t index, char* id, size_t cap, uint64_t* fields) {
  if (m == nullptr || index >= m->descriptor.operator_count) return -1;
  const ksj_operator_descriptor& o = m->descriptor.operators[index];
  if (id && cap) {
    const size_t n = o.operator_id.size < cap - 1 ? static_cast<size_t>(o.operator_id.size) : cap - 1;
    std::memcpy(id, o.operator_id.data, n);
    id[n] = 0;
  }
  if (fields) {
    fields[0] = o.max_in_flight;
    fields[1] = o.thread_safety;
    fields[2] = o.max_private_threads;
    fields[3] = o.max_input_items_per_firing;
    fields[4] = o.max_output_items_per_firing;
    fields[5] = o.max_output_bytes_per_firing;
    fields[6] = o.max_scratch_bytes_per_firing;
    fields[7] = o.max_retained_input_bytes;
    fields[8] = o.max_async_tail_bytes;
    fields[9] = o.abi.capability_bits;
  }
  return 0;
}

// operator_create only; returns the ksj_status and the error text.
KSJH_API uint32_t ksjh_try_create(ksjh_module* m, const char* operator_id, const char* config, size_t config_len,
                                  char* error, size_t error_capacity, int* created) {
  if (created) *created = 0;
  if (m == nullptr) return KSJ_STATUS_INVALID_ARGUMENT;
  ksj_operator_create_request req{};
  req.abi = header(sizeof(req));
  req.operator_id = utf8(operator_id, std::strlen(operator_id));
  req.canonical_config.abi = header(sizeof(req.canonical_config));
  req.canonical_config.data = config;
  req.canonical_config.size = config_len;
  ksj_provider_operator* op = nullptr;
  ksj_error_view e = empty_error();
  const ksj_status st = m->api.operator_create(&req, &op, &e);
  if (error && error_capacity > 511) copy_error(e, error);
  if (op != nullptr) {
    if (created) *created = 1;
    m->api.operator_destroy(op);
  }
  return st;
}

// operator_create + execution_context_create + key_state_init + on_start.
KSJH_API uint32_t ksjh_create(ksjh_module* m, const char* operator_id, const char* config, size_t config_len,
                              uint32_t device, ksjh_instance** out, char* error, size_t error_capacity) {
  if (m == nullptr || out == nullptr) return KSJ_STATUS_INVALID_ARGUMENT;
  *out = nullptr;
  auto* inst = new (std::nothrow) ksjh_instance{};
  if (inst == nullptr) return KSJ_STATUS_RESOURCE_EXHAUSTED;
  inst->module = m;
  ksj_error_view e = empty_error();
  ksj_operator_create_request req{};
  req.abi = header(sizeof(req));
  req.operator_id = utf8(operator_id, std::strlen(operator_id));
  req.canonical_config.abi = header(sizeof(req.canonical_config));
  req.canonical_config.data = config;
  req.canonical_config.size = config_len;
  ksj_status st = m->api.operator_create(&req, &inst->op, &e);
  if (st == KSJ_STATUS_OK) {
    ksj_execution_context_descriptor cd{};
    cd.abi = header(sizeof(cd));
    cd.device_ordinal = device;
    cd.max_backend_concurrency = 1;
    e = empty_error();
    st = m->api.execution_context_create(inst->op, &cd, &inst->context, &e);
  }
  if (st == KSJ_STATUS_OK) {
    ksj_key_state_descriptor kd{};
    kd.abi = header(sizeof(kd));
    kd.semantic_key.abi = header(sizeof(kd.semantic_key));
    e = empty_error();
    st = m->api.key_state_init(inst->op, inst->context, &kd, &inst->key, &e);
  }
  if (st == KSJ_STATUS_OK) {
    ksj_scan_start_descriptor sd{};
    sd.abi = header(sizeof(sd));
    e = empty_error();
    st = m->api.operator_on_start(inst->op, inst->context, inst->key, &sd, &e);
  }
  if (error && error_capacity > 511) copy_error(e, error);
  if (st != KSJ_STATUS_OK) {
    if (inst->key) m->api.key_state_reset(inst->op, inst->context, inst->key);
    if (inst->context) m->api.execution_context_destroy(inst->op, inst->context);
    if (inst->op) m->api.operator_destroy(inst->op);
    delete inst;
    return st;
  }
  *out = inst;
  return KSJ_STATUS_OK;
}

KSJH_API void ksjh_destroy(ksjh_instance* inst) {
  if (inst == nullptr) return;
  const ksj_provider_api& api = inst->module->api;
  if (inst->key) api.key_state_reset(inst->op, inst->context, inst->key);
  if (inst->context) api.execution_context_destroy(inst->op, inst->context);
  if (inst->op) api.operator_destroy(inst->op);
  delete inst;
}

// operator_on_cancel for a cancelled (kind 1) or failed (kind 2) scan: the
// terminal protocol's cancellation path (provider.h:676-694): no lease, no
// output grants.  Returns the provider's status; `error` (512 bytes) gets
// its message.
KSJH_API uint32_t ksjh_cancel(ksjh_instance* inst, uint32_t kind, char* error) {
  if (inst == nullptr) return KSJ_STATUS_INVALID_ARGUMENT;
  ksj_cancel_context cc{};
  cc.abi = header(sizeof(cc));
  cc.kind = kind;
  cc.terminal_epoch = 89;
  cc.cancellation_generation = 1;
  cc.reason.abi = header(sizeof(cc.reason));
  static const char kReason[] = "cancelled by the host";
  cc.reason.data = kReason;
  cc.reason.size = sizeof(kReason) - 1;
  ksj_error_view e = empty_error();
  const ksj_status st = inst->module->api.operator_on_cancel(inst->op, inst->context, inst->key, &cc, &e);
  if (error) copy_error(e, error);
  return st;
}

KSJH_API size_t ksjh_firing_size(void) { return sizeof(ksjh_firing); }

KSJH_API uint32_t ksjh_fire(ksjh_instance* inst, ksjh_firing* f) {
  if (inst == nullptr || f == nullptr || f->struct_size != sizeof(ksjh_firing) || f->input_count < 1 ||
      f->input_count > 2)
    return KSJ_STATUS_INVALID_ARGUMENT;
  Host h{};
  h.f = f;
  f->acquire_calls = f->map_calls = f->seal_calls = f->release_calls = f->input_batch_requests = 0;
  for (uint32_t i = 0; i < f->input_count; ++i) {
    ksj_input_item_view& it = h.items[i];
    it = {};
    it.abi = header(sizeof(it));
    it.payload.abi = header(sizeof(it.payload));
    it.payload.data = f->payload[i];
    it.payload.byte_count = f->payload_bytes[i];
    it.payload.memory_domain = KSJ_PROVIDER_MEMORY_HOST_PAGEABLE;
    it.payload.alignment = 64;
    it.payload.type = types().desc[f->payload_type[i] & 3];
    if (f->corrupt_input_type == i + 1)
      it.payload.type.type_identity_digest = types().desc[(f->payload_type[i] + 2) & 3].type_identity_digest;
    it.metadata.abi = header(sizeof(it.metadata));
    if (i == 0) {
      it.metadata.data = f->metadata;
      it.metadata.size = f->metadata_bytes;
    }
    it.semantic_key_hash = f->semantic_key_hash[i];
    it.order_key = f->order_key[i];
    it.item_ordinal = 79 + i;
    ksj_input_batch_view& b = h.batches[i];
    b = {};
    b.abi = header(sizeof(b));
    b.items = &h.items[i];
    b.item_count = 1;
    b.input_port = f->payload_port[i];
    b.batch_id = 5 + 6 * i;
    b.order_domain = 7 + 6 * i;
  }
  ksj_output_grant_callbacks og{};
  og.abi = header(sizeof(og));
  og.host_context = &h;
  og.map_mutable_payload = &map_output;
  og.seal = &seal_output;
  og.release = &release_output;
  ksj_firing_lease_callbacks cb{};
  cb.abi = header(sizeof(cb), KSJ_LEASE_CAP_INPUT_BATCHES | KSJ_LEASE_CAP_OUTPUT_GRANTS | KSJ_LEASE_CAP_SCRATCH);
  cb.host_context = &h;
  cb.output_grants = &og;
  cb.get_info = &get_info;
  cb.get_input_batch = &get_input_batch;
  cb.get_scratch = &get_scratch;
  cb.acquire_output_grant = &acquire;
  alignas(64) static unsigned char lease_token;
  ksj_process_result result{};
  result.abi = header(sizeof(result));
  ksj_error_view e = empty_error();
  const ksj_status st =
      inst->module->api.operator_process_batch(inst->op, inst->context, inst->key,
                                               reinterpret_cast<ksj_firing_lease*>(&lease_token), &cb, &result, &e);
  f->status = st;
  f->outcome = result.outcome;
  f->sealed_count = result.sealed_output_count;
  f->consumed = result.consumed_input_item_count;
  copy_error(e, f->error);
  return st;
}
