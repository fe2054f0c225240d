/*
 * ksj_provider_abi.h -- the KSpaceJet Provider C ABI, restated so that the
 * GB300 plug-ins build without the reference tree.
 *
 * This is an interface that must stay identical, not a design of this
 * project: every struct below has the field order, types and constant values
 * of libs/recon/kspacejet-provider-sdk/include/kspacejet/provider/provider.h
 * (lines cited per block), so a host built against that header loads these
 * plug-ins unchanged and vice versa.  tests/test_abi_layout.py compiles one
 * offset/size probe against both headers and requires equal output.  Either
 * header may be used by a translation unit, never both.
 *
 * The plug-ins export exactly one symbol, ksj_provider_query (provider.h:667-674).
 */
#ifndef KSPACEJET_PROVIDER_PROVIDER_H_
#define KSPACEJET_PROVIDER_PROVIDER_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__) && defined(KSJ_PROVIDER_BUILDING_PLUGIN)
#define KSJ_PROVIDER_SYMBOL_EXPORT __attribute__((visibility("default")))
#else
#define KSJ_PROVIDER_SYMBOL_EXPORT
#endif
#define KSJ_PROVIDER_CALL
#if defined(__cplusplus)
#define KSJ_PROVIDER_EXTERN_C extern "C"
#else
#define KSJ_PROVIDER_EXTERN_C extern
#endif
#define KSJ_PROVIDER_ENTRY KSJ_PROVIDER_EXTERN_C KSJ_PROVIDER_SYMBOL_EXPORT
#define KSJ_PROVIDER_DIGEST256_SIZE UINT32_C(32)

#ifdef __cplusplus
extern "C" {
#endif

/* provider.h:74-90 -- every ABI struct begins with this header. */
typedef struct ksj_provider_abi_header {
  uint32_t struct_size;
  uint32_t reserved0;
  uint64_t capability_bits;
  uint64_t reserved[2];
} ksj_provider_abi_header;

static inline ksj_provider_abi_header ksj_provider_abi_header_make(const uint32_t struct_size,
                                                                   const uint64_t capability_bits) {
  ksj_provider_abi_header h;
  h.struct_size = struct_size;
  h.reserved0 = 0u;
  h.capability_bits = capability_bits;
  h.reserved[0] = 0u;
  h.reserved[1] = 0u;
  return h;
}

/* provider.h:98-135 -- fixed-width enums. */
typedef uint32_t ksj_status;
#define KSJ_STATUS_OK UINT32_C(0)
#define KSJ_STATUS_BAD_ABI UINT32_C(1)
#define KSJ_STATUS_INVALID_ARGUMENT UINT32_C(2)
#define KSJ_STATUS_UNSUPPORTED UINT32_C(3)
#define KSJ_STATUS_RESOURCE_EXHAUSTED UINT32_C(4)
#define KSJ_STATUS_CANCELLED UINT32_C(5)
#define KSJ_STATUS_FAILED_PRECONDITION UINT32_C(6)
#define KSJ_STATUS_INTERNAL_ERROR UINT32_C(7)
#define KSJ_STATUS_CONTRACT_VIOLATION UINT32_C(8)

typedef uint32_t ksj_provider_process_outcome;
#define KSJ_PROVIDER_PROCESS_DONE UINT32_C(0)
#define KSJ_PROVIDER_PROCESS_YIELD UINT32_C(1)
#define KSJ_PROVIDER_PROCESS_ASYNC_PENDING UINT32_C(2)
#define KSJ_PROVIDER_PROCESS_STRUCTURED_FAILURE UINT32_C(3)
#define KSJ_PROVIDER_PROCESS_CONTRACT_VIOLATION UINT32_C(4)

typedef uint32_t ksj_provider_thread_safety;
#define KSJ_PROVIDER_SERIAL_INSTANCE UINT32_C(0)
#define KSJ_PROVIDER_SERIAL_PER_KEY_REENTRANT_ACROSS_KEYS UINT32_C(1)
#define KSJ_PROVIDER_FULLY_REENTRANT UINT32_C(2)

typedef uint32_t ksj_provider_cancellation_state;
#define KSJ_PROVIDER_NOT_CANCELLED UINT32_C(0)
#define KSJ_PROVIDER_CANCELLATION_REQUESTED UINT32_C(1)
#define KSJ_PROVIDER_CANCELLATION_FORCED UINT32_C(2)

typedef uint32_t ksj_provider_scan_end_kind;
#define KSJ_PROVIDER_SCAN_END_NORMAL UINT32_C(0)
#define KSJ_PROVIDER_SCAN_END_CANCELLED UINT32_C(1)
#define KSJ_PROVIDER_SCAN_END_FAILED UINT32_C(2)

typedef uint32_t ksj_provider_memory_domain;
#define KSJ_PROVIDER_MEMORY_HOST_PAGEABLE UINT32_C(1)
#define KSJ_PROVIDER_MEMORY_HOST_PINNED UINT32_C(2)
#define KSJ_PROVIDER_MEMORY_DEVICE UINT32_C(4)
#define KSJ_PROVIDER_MEMORY_SHARED UINT32_C(8)

/* provider.h:146-177 -- type descriptor enums. */
typedef uint32_t ksj_payload_kind;
#define KSJ_PAYLOAD_KIND_BUFFER_HANDLE UINT32_C(0)
#define KSJ_PAYLOAD_KIND_MESSAGE_HANDLE UINT32_C(1)
#define KSJ_PAYLOAD_KIND_CONTROL_TOKEN UINT32_C(2)
#define KSJ_PAYLOAD_KIND_OPAQUE_HANDLE UINT32_C(3)

typedef uint32_t ksj_element_type;
#define KSJ_ELEMENT_TYPE_NONE UINT32_C(0)
#define KSJ_ELEMENT_TYPE_UINT8 UINT32_C(1)
#define KSJ_ELEMENT_TYPE_INT16 UINT32_C(2)
#define KSJ_ELEMENT_TYPE_UINT16 UINT32_C(3)
#define KSJ_ELEMENT_TYPE_INT32 UINT32_C(4)
#define KSJ_ELEMENT_TYPE_UINT32 UINT32_C(5)
#define KSJ_ELEMENT_TYPE_FLOAT32 UINT32_C(6)
#define KSJ_ELEMENT_TYPE_FLOAT64 UINT32_C(7)
#define KSJ_ELEMENT_TYPE_COMPLEX_INT16 UINT32_C(8)
#define KSJ_ELEMENT_TYPE_COMPLEX_FLOAT32 UINT32_C(9)
#define KSJ_ELEMENT_TYPE_COMPLEX_FLOAT64 UINT32_C(10)

typedef uint32_t ksj_payload_mutability;
#define KSJ_PAYLOAD_MUTABILITY_IMMUTABLE_AFTER_PUBLISH UINT32_C(0)
#define KSJ_PAYLOAD_MUTABILITY_MUTABLE_EXCLUSIVE UINT32_C(1)

typedef uint64_t ksj_type_layout_flags;
#define KSJ_TYPE_LAYOUT_CANONICAL_CONTIGUOUS (UINT64_C(1) << 0)
#define KSJ_TYPE_LAYOUT_CHANNEL_MAJOR_CONTIGUOUS (UINT64_C(1) << 1)
#define KSJ_TYPE_LAYOUT_ROW_MAJOR_CONTIGUOUS (UINT64_C(1) << 2)
#define KSJ_TYPE_LAYOUT_COLUMN_MAJOR_CONTIGUOUS (UINT64_C(1) << 3)
#define KSJ_TYPE_LAYOUT_OPAQUE (UINT64_C(1) << 4)
#define KSJ_TYPE_STRIDES_CANONICAL (UINT64_C(1) << 16)
#define KSJ_TYPE_STRIDES_EXPLICIT_BYTE (UINT64_C(1) << 17)

/* provider.h:180-209 -- capability bits. */
#define KSJ_PROVIDER_CAP_SYNC_PROCESS (UINT64_C(1) << 0)
#define KSJ_PROVIDER_CAP_ASYNC_PROCESS (UINT64_C(1) << 1)
#define KSJ_PROVIDER_CAP_INPUT_RETENTION (UINT64_C(1) << 2)
#define KSJ_PROVIDER_CAP_TERMINAL_OUTPUT (UINT64_C(1) << 3)
#define KSJ_PROVIDER_CAP_HOST_MEMORY_BROKER (UINT64_C(1) << 4)
#define KSJ_PROVIDER_CAP_HOST_BACKEND_EXECUTOR (UINT64_C(1) << 5)
#define KSJ_PROVIDER_CAP_NO_PRIVATE_THREADS (UINT64_C(1) << 6)
#define KSJ_PROVIDER_CAP_NO_DIRECT_FILE_IO (UINT64_C(1) << 7)
#define KSJ_PROVIDER_CAP_NO_DIRECT_NETWORK_IO (UINT64_C(1) << 8)

#define KSJ_OPERATOR_CAP_MAY_YIELD (UINT64_C(1) << 0)
#define KSJ_OPERATOR_CAP_MAY_ASYNC (UINT64_C(1) << 1)
#define KSJ_OPERATOR_CAP_MAY_RETAIN_INPUT (UINT64_C(1) << 2)
#define KSJ_OPERATOR_CAP_MAY_EMIT_TERMINAL_OUTPUT (UINT64_C(1) << 3)
#define KSJ_OPERATOR_CAP_CANCEL_NO_ALLOCATION (UINT64_C(1) << 4)
#define KSJ_OPERATOR_CAP_CANCEL_NO_THROW (UINT64_C(1) << 5)

#define KSJ_LEASE_CAP_INPUT_BATCHES (UINT64_C(1) << 0)
#define KSJ_LEASE_CAP_OUTPUT_GRANTS (UINT64_C(1) << 1)
#define KSJ_LEASE_CAP_SCRATCH (UINT64_C(1) << 2)
#define KSJ_LEASE_CAP_KEY_STATE (UINT64_C(1) << 3)
#define KSJ_LEASE_CAP_RETENTION (UINT64_C(1) << 4)
#define KSJ_LEASE_CAP_ASYNC (UINT64_C(1) << 5)
#define KSJ_LEASE_CAP_CANCELLATION (UINT64_C(1) << 6)

#define KSJ_ASYNC_REGISTRATION_RETAINS_OUTPUT_GRANTS (UINT64_C(1) << 0)
#define KSJ_ASYNC_REGISTRATION_RETAINS_SCRATCH (UINT64_C(1) << 1)

/* provider.h:212-220 -- opaque handles. */
typedef struct ksj_provider_operator ksj_provider_operator;
typedef struct ksj_execution_context ksj_execution_context;
typedef struct ksj_key_state ksj_key_state;
typedef struct ksj_firing_lease ksj_firing_lease;
typedef struct ksj_output_grant ksj_output_grant;
typedef struct ksj_retention_handle ksj_retention_handle;
typedef struct ksj_async_token ksj_async_token;
typedef struct ksj_host_memory_allocation ksj_host_memory_allocation;
typedef struct ksj_backend_executor ksj_backend_executor;

/* provider.h:222-250 */
typedef struct ksj_utf8_view {
  ksj_provider_abi_header abi;
  const char* data;
  uint64_t size;
} ksj_utf8_view;

typedef struct ksj_byte_view {
  ksj_provider_abi_header abi;
  const void* data;
  uint64_t size;
} ksj_byte_view;

typedef struct ksj_digest256 {
  ksj_provider_abi_header abi;
  uint8_t bytes[KSJ_PROVIDER_DIGEST256_SIZE];
} ksj_digest256;

typedef struct ksj_error_view {
  ksj_provider_abi_header abi;
  ksj_status status;
  uint32_t category;
  uint64_t provider_error_code;
  ksj_utf8_view message;
} ksj_error_view;

/* provider.h:264-278 */
typedef struct ksj_type_descriptor_view {
  ksj_provider_abi_header abi;
  ksj_utf8_view type_ref;
  ksj_digest256 type_identity_digest;
  uint32_t payload_kind;
  uint32_t element_type;
  uint32_t rank;
  const ksj_utf8_view* dimension_names;
  uint64_t layout_flags;
  uint64_t stride_bytes[8];
  uint32_t allowed_memory_domains;
  uint32_t minimum_alignment;
  uint32_t mutability;
  uint32_t reserved0;
} ksj_type_descriptor_view;

/* provider.h:280-307 */
typedef struct ksj_operator_descriptor {
  ksj_provider_abi_header abi;
  ksj_utf8_view operator_id;
  uint32_t max_in_flight;
  ksj_provider_thread_safety thread_safety;
  uint32_t max_private_threads;
  uint32_t max_input_items_per_firing;
  uint32_t max_output_items_per_firing;
  uint64_t max_output_bytes_per_firing;
  uint64_t max_scratch_bytes_per_firing;
  uint64_t max_retained_input_bytes;
  uint64_t max_async_tail_bytes;
} ksj_operator_descriptor;

typedef struct ksj_provider_descriptor {
  ksj_provider_abi_header abi;
  ksj_utf8_view provider_id;
  ksj_digest256 bundle_digest;
  uint32_t operator_count;
  uint32_t reserved0;
  const ksj_operator_descriptor* operators;
} ksj_provider_descriptor;

typedef struct ksj_provider_query_request {
  ksj_provider_abi_header abi;
  uint64_t host_capability_bits;
  ksj_utf8_view host_build_id;
} ksj_provider_query_request;

/* provider.h:309-361 */
typedef struct ksj_host_allocation_request {
  ksj_provider_abi_header abi;
  uint64_t byte_count;
  uint32_t alignment;
  uint32_t memory_domain;
  uint64_t resource_occurrence_id;
  uint64_t allocation_flags;
} ksj_host_allocation_request;

typedef struct ksj_mutable_payload_view {
  ksj_provider_abi_header abi;
  void* data;
  uint64_t capacity_bytes;
  uint64_t committed_bytes;
  uint32_t memory_domain;
  uint32_t alignment;
  ksj_type_descriptor_view type;
} ksj_mutable_payload_view;

typedef struct ksj_host_services ksj_host_services;
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_host_allocate_fn)(void* host_context,
                                                            const ksj_host_allocation_request* request,
                                                            ksj_host_memory_allocation** out_allocation,
                                                            ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_host_map_allocation_fn)(void* host_context,
                                                                  ksj_host_memory_allocation* allocation,
                                                                  ksj_mutable_payload_view* out_view,
                                                                  ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_host_release_allocation_fn)(void* host_context,
                                                                      ksj_host_memory_allocation* allocation,
                                                                      ksj_error_view* out_error);
struct ksj_host_services {
  ksj_provider_abi_header abi;
  void* host_context;
  ksj_host_allocate_fn allocate;
  ksj_host_map_allocation_fn map_allocation;
  ksj_host_release_allocation_fn release_allocation;
  ksj_backend_executor* backend_executor;
};

typedef struct ksj_operator_create_request {
  ksj_provider_abi_header abi;
  ksj_utf8_view operator_id;
  ksj_byte_view canonical_config;
  const ksj_host_services* host_services;
} ksj_operator_create_request;

/* provider.h:363-443 */
typedef struct ksj_execution_context_descriptor {
  ksj_provider_abi_header abi;
  uint32_t numa_node;
  uint32_t device_ordinal;
  uint64_t execution_context_id;
  uint64_t resource_domain_id;
  uint64_t max_backend_concurrency;
  const ksj_host_services* host_services;
} ksj_execution_context_descriptor;

typedef struct ksj_key_state_descriptor {
  ksj_provider_abi_header abi;
  ksj_byte_view semantic_key;
  uint64_t placement_key;
  uint64_t key_state_generation;
  uint64_t home_shard;
} ksj_key_state_descriptor;

typedef struct ksj_scan_start_descriptor {
  ksj_provider_abi_header abi;
  ksj_utf8_view run_id;
  ksj_utf8_view scan_id;
  ksj_digest256 normalized_scan_facts_digest;
  ksj_digest256 execution_plan_digest;
  uint64_t terminal_epoch;
} ksj_scan_start_descriptor;

typedef struct ksj_payload_view {
  ksj_provider_abi_header abi;
  const void* data;
  uint64_t byte_count;
  uint32_t memory_domain;
  uint32_t alignment;
  ksj_type_descriptor_view type;
} ksj_payload_view;

typedef struct ksj_input_item_view {
  ksj_provider_abi_header abi;
  ksj_payload_view payload;
  ksj_byte_view metadata;
  uint64_t semantic_key_hash;
  uint64_t order_key;
  uint64_t item_ordinal;
} ksj_input_item_view;

typedef struct ksj_input_batch_view {
  ksj_provider_abi_header abi;
  const ksj_input_item_view* items;
  uint32_t item_count;
  uint32_t input_port;
  uint64_t batch_id;
  uint64_t order_domain;
} ksj_input_batch_view;

typedef struct ksj_scratch_view {
  ksj_provider_abi_header abi;
  void* data;
  uint64_t byte_count;
  uint32_t memory_domain;
  uint32_t alignment;
  uint64_t resource_occurrence_id;
} ksj_scratch_view;

typedef struct ksj_key_state_view {
  ksj_provider_abi_header abi;
  void* data;
  uint64_t byte_count;
  uint64_t key_state_generation;
  uint64_t slot_generation;
} ksj_key_state_view;

typedef struct ksj_firing_lease_info {
  ksj_provider_abi_header abi;
  uint64_t resource_occurrence_id;
  uint64_t slot_generation;
  uint64_t terminal_epoch;
  uint32_t input_batch_count;
  uint32_t output_grant_count;
  uint64_t reserved_output_bytes;
  uint64_t reserved_scratch_bytes;
} ksj_firing_lease_info;

/* provider.h:445-489 */
typedef struct ksj_retention_request {
  ksj_provider_abi_header abi;
  uint64_t requested_bytes;
  uint64_t retention_class;
  uint64_t maximum_lifetime_epoch;
} ksj_retention_request;

typedef struct ksj_async_registration {
  ksj_provider_abi_header abi;
  uint64_t resource_occurrence_id;
  uint64_t slot_generation;
  uint64_t terminal_epoch;
  uint64_t reserved_output_bytes;
  uint64_t reserved_scratch_bytes;
  uint64_t completion_deadline_ns;
  uint32_t maximum_completion_callbacks;
  uint32_t reserved0;
} ksj_async_registration;

typedef struct ksj_async_completion {
  ksj_provider_abi_header abi;
  ksj_provider_process_outcome outcome;
  uint32_t sealed_output_count;
  uint64_t completion_sequence;
  uint64_t terminal_epoch;
} ksj_async_completion;

typedef struct ksj_cancellation_view {
  ksj_provider_abi_header abi;
  ksj_provider_cancellation_state state;
  uint32_t reserved0;
  uint64_t terminal_epoch;
  uint64_t cancellation_generation;
} ksj_cancellation_view;

typedef struct ksj_output_seal_descriptor {
  ksj_provider_abi_header abi;
  uint32_t output_port;
  uint32_t produced_item_count;
  uint64_t produced_byte_count;
  uint64_t semantic_key_hash;
  uint64_t order_key;
  ksj_type_descriptor_view type;
  ksj_byte_view metadata;
} ksj_output_seal_descriptor;

/* provider.h:491-576 -- host callback tables. */
typedef struct ksj_output_grant_callbacks ksj_output_grant_callbacks;
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_output_grant_map_fn)(void* host_context, ksj_output_grant* grant,
                                                               ksj_mutable_payload_view* out_payload,
                                                               ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_output_grant_seal_fn)(void* host_context, ksj_output_grant* grant,
                                                                const ksj_output_seal_descriptor* descriptor,
                                                                ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_output_grant_release_fn)(void* host_context, ksj_output_grant* grant,
                                                                   ksj_error_view* out_error);
struct ksj_output_grant_callbacks {
  ksj_provider_abi_header abi;
  void* host_context;
  ksj_output_grant_map_fn map_mutable_payload;
  ksj_output_grant_seal_fn seal;
  ksj_output_grant_release_fn release;
};

typedef struct ksj_firing_lease_callbacks ksj_firing_lease_callbacks;
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_lease_get_info_fn)(void* host_context, const ksj_firing_lease* lease,
                                                             ksj_firing_lease_info* out_info,
                                                             ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_lease_get_input_batch_fn)(void* host_context, const ksj_firing_lease* lease,
                                                                    uint32_t batch_index,
                                                                    ksj_input_batch_view* out_batch,
                                                                    ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_lease_get_scratch_fn)(void* host_context, const ksj_firing_lease* lease,
                                                                ksj_scratch_view* out_scratch,
                                                                ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_lease_get_key_state_fn)(void* host_context, const ksj_firing_lease* lease,
                                                                  ksj_key_state* key_state,
                                                                  ksj_key_state_view* out_key_state,
                                                                  ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_lease_acquire_output_fn)(void* host_context, ksj_firing_lease* lease,
                                                                   uint32_t output_slot, ksj_output_grant** out_grant,
                                                                   ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_lease_retain_input_fn)(void* host_context, ksj_firing_lease* lease,
                                                                 uint32_t batch_index, uint32_t item_index,
                                                                 const ksj_retention_request* request,
                                                                 ksj_retention_handle** out_retention,
                                                                 ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_lease_release_retention_fn)(void* host_context,
                                                                      ksj_retention_handle* retention,
                                                                      ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_lease_register_async_fn)(void* host_context, ksj_firing_lease* lease,
                                                                   const ksj_async_registration* registration,
                                                                   ksj_async_token** out_token,
                                                                   ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_lease_complete_async_fn)(void* host_context, ksj_async_token* token,
                                                                   const ksj_async_completion* completion,
                                                                   ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_lease_release_async_fn)(void* host_context, ksj_async_token* token,
                                                                  ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_lease_get_cancellation_fn)(void* host_context, const ksj_firing_lease* lease,
                                                                     ksj_cancellation_view* out_cancellation,
                                                                     ksj_error_view* out_error);
struct ksj_firing_lease_callbacks {
  ksj_provider_abi_header abi;
  void* host_context;
  const ksj_output_grant_callbacks* output_grants;
  ksj_lease_get_info_fn get_info;
  ksj_lease_get_input_batch_fn get_input_batch;
  ksj_lease_get_scratch_fn get_scratch;
  ksj_lease_get_key_state_fn get_key_state;
  ksj_lease_acquire_output_fn acquire_output_grant;
  ksj_lease_retain_input_fn retain_input;
  ksj_lease_release_retention_fn release_retention;
  ksj_lease_register_async_fn register_async;
  ksj_lease_complete_async_fn complete_async;
  ksj_lease_release_async_fn release_async;
  ksj_lease_get_cancellation_fn get_cancellation;
};

/* provider.h:578-602 */
typedef struct ksj_process_result {
  ksj_provider_abi_header abi;
  ksj_provider_process_outcome outcome;
  uint32_t sealed_output_count;
  uint64_t consumed_input_item_count;
  uint64_t terminal_epoch;
  ksj_async_token* async_token;
} ksj_process_result;

typedef struct ksj_scan_end_descriptor {
  ksj_provider_abi_header abi;
  ksj_provider_scan_end_kind kind;
  uint32_t reserved0;
  uint64_t terminal_epoch;
  uint64_t completed_input_item_count;
} ksj_scan_end_descriptor;

typedef struct ksj_cancel_context {
  ksj_provider_abi_header abi;
  ksj_provider_scan_end_kind kind;
  uint32_t reserved0;
  uint64_t terminal_epoch;
  uint64_t cancellation_generation;
  ksj_utf8_view reason;
} ksj_cancel_context;

/* provider.h:604-658 -- the Provider's lifecycle table. */
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_operator_create_fn)(const ksj_operator_create_request* request,
                                                              ksj_provider_operator** out_operator,
                                                              ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_execution_context_create_fn)(
    ksj_provider_operator* operator_handle, const ksj_execution_context_descriptor* descriptor,
    ksj_execution_context** out_context, ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_key_state_init_fn)(ksj_provider_operator* operator_handle,
                                                             ksj_execution_context* context,
                                                             const ksj_key_state_descriptor* descriptor,
                                                             ksj_key_state** out_key_state, ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_operator_on_start_fn)(ksj_provider_operator* operator_handle,
                                                                ksj_execution_context* context,
                                                                ksj_key_state* key_state,
                                                                const ksj_scan_start_descriptor* descriptor,
                                                                ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_operator_process_batch_fn)(ksj_provider_operator* operator_handle,
                                                                     ksj_execution_context* context,
                                                                     ksj_key_state* key_state, ksj_firing_lease* lease,
                                                                     const ksj_firing_lease_callbacks* lease_callbacks,
                                                                     ksj_process_result* out_result,
                                                                     ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_operator_on_scan_end_fn)(
    ksj_provider_operator* operator_handle, ksj_execution_context* context, ksj_key_state* key_state,
    const ksj_scan_end_descriptor* descriptor, ksj_firing_lease* terminal_lease,
    const ksj_firing_lease_callbacks* lease_callbacks, ksj_process_result* out_result, ksj_error_view* out_error);
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_operator_on_cancel_fn)(ksj_provider_operator* operator_handle,
                                                                 ksj_execution_context* context,
                                                                 ksj_key_state* key_state,
                                                                 const ksj_cancel_context* context_descriptor,
                                                                 ksj_error_view* out_error);
typedef void(KSJ_PROVIDER_CALL* ksj_key_state_reset_fn)(ksj_provider_operator* operator_handle,
                                                        ksj_execution_context* context, ksj_key_state* key_state);
typedef void(KSJ_PROVIDER_CALL* ksj_execution_context_destroy_fn)(ksj_provider_operator* operator_handle,
                                                                  ksj_execution_context* context);
typedef void(KSJ_PROVIDER_CALL* ksj_operator_destroy_fn)(ksj_provider_operator* operator_handle);

typedef struct ksj_provider_api {
  ksj_provider_abi_header abi;
  ksj_operator_create_fn operator_create;
  ksj_execution_context_create_fn execution_context_create;
  ksj_key_state_init_fn key_state_init;
  ksj_operator_on_start_fn operator_on_start;
  ksj_operator_process_batch_fn operator_process_batch;
  ksj_operator_on_scan_end_fn operator_on_scan_end;
  ksj_operator_on_cancel_fn operator_on_cancel;
  ksj_key_state_reset_fn key_state_reset;
  ksj_execution_context_destroy_fn execution_context_destroy;
  ksj_operator_destroy_fn operator_destroy;
} ksj_provider_api;

/* provider.h:667-674 -- the one exported entry point of every plug-in. */
typedef ksj_status(KSJ_PROVIDER_CALL* ksj_provider_query_fn)(const ksj_provider_query_request* request,
                                                             ksj_provider_descriptor* out_descriptor,
                                                             ksj_provider_api* out_api, ksj_error_view* out_error);

KSJ_PROVIDER_ENTRY ksj_status KSJ_PROVIDER_CALL ksj_provider_query(const ksj_provider_query_request* request,
                                                                   ksj_provider_descriptor* out_descriptor,
                                                                   ksj_provider_api* out_api,
                                                                   ksj_error_view* out_error);

#ifdef __cplusplus
}
#endif

#endif /* KSPACEJET_PROVIDER_PROVIDER_H_ */
