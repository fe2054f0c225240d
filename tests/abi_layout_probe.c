/* Prints sizeof/offsetof of every ABI struct field.  Compiled by
 * tests/test_abi_layout.py once against include/ksj_provider_abi.h and once
 * against the reference's provider.h; the two outputs must be identical. */
#include <stddef.h>
#include <stdio.h>
#include KSJ_ABI_HEADER

#define S(t) printf("%s %zu\n", #t, sizeof(t))
#define F(t, f) printf("%s.%s %zu\n", #t, #f, offsetof(t, f))

int main(void) {
  S(ksj_provider_abi_header); F(ksj_provider_abi_header, capability_bits); F(ksj_provider_abi_header, reserved);
  S(ksj_utf8_view); F(ksj_utf8_view, data); F(ksj_utf8_view, size);
  S(ksj_byte_view); F(ksj_byte_view, data); F(ksj_byte_view, size);
  S(ksj_digest256); F(ksj_digest256, bytes);
  S(ksj_error_view); F(ksj_error_view, status); F(ksj_error_view, category); F(ksj_error_view, provider_error_code);
  F(ksj_error_view, message);
  S(ksj_type_descriptor_view); F(ksj_type_descriptor_view, type_ref); F(ksj_type_descriptor_view, type_identity_digest);
  F(ksj_type_descriptor_view, payload_kind); F(ksj_type_descriptor_view, element_type); F(ksj_type_descriptor_view, rank);
  F(ksj_type_descriptor_view, dimension_names); F(ksj_type_descriptor_view, layout_flags);
  F(ksj_type_descriptor_view, stride_bytes); F(ksj_type_descriptor_view, allowed_memory_domains);
  F(ksj_type_descriptor_view, minimum_alignment); F(ksj_type_descriptor_view, mutability);
  F(ksj_type_descriptor_view, reserved0);
  S(ksj_operator_descriptor); F(ksj_operator_descriptor, operator_id); F(ksj_operator_descriptor, max_in_flight);
  F(ksj_operator_descriptor, thread_safety); F(ksj_operator_descriptor, max_private_threads);
  F(ksj_operator_descriptor, max_input_items_per_firing); F(ksj_operator_descriptor, max_output_items_per_firing);
  F(ksj_operator_descriptor, max_output_bytes_per_firing); F(ksj_operator_descriptor, max_scratch_bytes_per_firing);
  F(ksj_operator_descriptor, max_retained_input_bytes); F(ksj_operator_descriptor, max_async_tail_bytes);
  S(ksj_provider_descriptor); F(ksj_provider_descriptor, provider_id); F(ksj_provider_descriptor, bundle_digest);
  F(ksj_provider_descriptor, operator_count); F(ksj_provider_descriptor, operators);
  S(ksj_provider_query_request); F(ksj_provider_query_request, host_capability_bits);
  F(ksj_provider_query_request, host_build_id);
  S(ksj_host_allocation_request); F(ksj_host_allocation_request, byte_count); F(ksj_host_allocation_request, alignment);
  F(ksj_host_allocation_request, memory_domain); F(ksj_host_allocation_request, resource_occurrence_id);
  F(ksj_host_allocation_request, allocation_flags);
  S(ksj_mutable_payload_view); F(ksj_mutable_payload_view, data); F(ksj_mutable_payload_view, capacity_bytes);
  F(ksj_mutable_payload_view, committed_bytes); F(ksj_mutable_payload_view, memory_domain);
  F(ksj_mutable_payload_view, alignment); F(ksj_mutable_payload_view, type);
  S(ksj_host_services); F(ksj_host_services, host_context); F(ksj_host_services, allocate);
  F(ksj_host_services, map_allocation); F(ksj_host_services, release_allocation); F(ksj_host_services, backend_executor);
  S(ksj_operator_create_request); F(ksj_operator_create_request, operator_id);
  F(ksj_operator_create_request, canonical_config); F(ksj_operator_create_request, host_services);
  S(ksj_execution_context_descriptor); F(ksj_execution_context_descriptor, numa_node);
  F(ksj_execution_context_descriptor, device_ordinal); F(ksj_execution_context_descriptor, execution_context_id);
  F(ksj_execution_context_descriptor, resource_domain_id); F(ksj_execution_context_descriptor, max_backend_concurrency);
  F(ksj_execution_context_descriptor, host_services);
  S(ksj_key_state_descriptor); F(ksj_key_state_descriptor, semantic_key); F(ksj_key_state_descriptor, placement_key);
  F(ksj_key_state_descriptor, key_state_generation); F(ksj_key_state_descriptor, home_shard);
  S(ksj_scan_start_descriptor); F(ksj_scan_start_descriptor, run_id); F(ksj_scan_start_descriptor, scan_id);
  F(ksj_scan_start_descriptor, normalized_scan_facts_digest); F(ksj_scan_start_descriptor, execution_plan_digest);
  F(ksj_scan_start_descriptor, terminal_epoch);
  S(ksj_payload_view); F(ksj_payload_view, data); F(ksj_payload_view, byte_count); F(ksj_payload_view, memory_domain);
  F(ksj_payload_view, alignment); F(ksj_payload_view, type);
  S(ksj_input_item_view); F(ksj_input_item_view, payload); F(ksj_input_item_view, metadata);
  F(ksj_input_item_view, semantic_key_hash); F(ksj_input_item_view, order_key); F(ksj_input_item_view, item_ordinal);
  S(ksj_input_batch_view); F(ksj_input_batch_view, items); F(ksj_input_batch_view, item_count);
  F(ksj_input_batch_view, input_port); F(ksj_input_batch_view, batch_id); F(ksj_input_batch_view, order_domain);
  S(ksj_scratch_view); F(ksj_scratch_view, data); F(ksj_scratch_view, byte_count); F(ksj_scratch_view, memory_domain);
  F(ksj_scratch_view, alignment); F(ksj_scratch_view, resource_occurrence_id);
  S(ksj_key_state_view); F(ksj_key_state_view, data); F(ksj_key_state_view, byte_count);
  F(ksj_key_state_view, key_state_generation); F(ksj_key_state_view, slot_generation);
  S(ksj_firing_lease_info); F(ksj_firing_lease_info, resource_occurrence_id); F(ksj_firing_lease_info, slot_generation);
  F(ksj_firing_lease_info, terminal_epoch); F(ksj_firing_lease_info, input_batch_count);
  F(ksj_firing_lease_info, output_grant_count); F(ksj_firing_lease_info, reserved_output_bytes);
  F(ksj_firing_lease_info, reserved_scratch_bytes);
  S(ksj_retention_request); F(ksj_retention_request, requested_bytes); F(ksj_retention_request, retention_class);
  F(ksj_retention_request, maximum_lifetime_epoch);
  S(ksj_async_registration); F(ksj_async_registration, resource_occurrence_id); F(ksj_async_registration, slot_generation);
  F(ksj_async_registration, terminal_epoch); F(ksj_async_registration, reserved_output_bytes);
  F(ksj_async_registration, reserved_scratch_bytes); F(ksj_async_registration, completion_deadline_ns);
  F(ksj_async_registration, maximum_completion_callbacks); F(ksj_async_registration, reserved0);
  S(ksj_async_completion); F(ksj_async_completion, outcome); F(ksj_async_completion, sealed_output_count);
  F(ksj_async_completion, completion_sequence); F(ksj_async_completion, terminal_epoch);
  S(ksj_cancellation_view); F(ksj_cancellation_view, state); F(ksj_cancellation_view, terminal_epoch);
  F(ksj_cancellation_view, cancellation_generation);
  S(ksj_output_seal_descriptor); F(ksj_output_seal_descriptor, output_port);
  F(ksj_output_seal_descriptor, produced_item_count); F(ksj_output_seal_descriptor, produced_byte_count);
  F(ksj_output_seal_descriptor, semantic_key_hash); F(ksj_output_seal_descriptor, order_key);
  F(ksj_output_seal_descriptor, type); F(ksj_output_seal_descriptor, metadata);
  S(ksj_output_grant_callbacks); F(ksj_output_grant_callbacks, host_context);
  F(ksj_output_grant_callbacks, map_mutable_payload); F(ksj_output_grant_callbacks, seal);
  F(ksj_output_grant_callbacks, release);
  S(ksj_firing_lease_callbacks); F(ksj_firing_lease_callbacks, host_context); F(ksj_firing_lease_callbacks, output_grants);
  F(ksj_firing_lease_callbacks, get_info); F(ksj_firing_lease_callbacks, get_input_batch);
  F(ksj_firing_lease_callbacks, get_scratch); F(ksj_firing_lease_callbacks, get_key_state);
  F(ksj_firing_lease_callbacks, acquire_output_grant); F(ksj_firing_lease_callbacks, retain_input);
  F(ksj_firing_lease_callbacks, release_retention); F(ksj_firing_lease_callbacks, register_async);
  F(ksj_firing_lease_callbacks, complete_async); F(ksj_firing_lease_callbacks, release_async);
  F(ksj_firing_lease_callbacks, get_cancellation);
  S(ksj_process_result); F(ksj_process_result, outcome); F(ksj_process_result, sealed_output_count);
  F(ksj_process_result, consumed_input_item_count); F(ksj_process_result, terminal_epoch);
  F(ksj_process_result, async_token);
  S(ksj_scan_end_descriptor); F(ksj_scan_end_descriptor, kind); F(ksj_scan_end_descriptor, terminal_epoch);
  F(ksj_scan_end_descriptor, completed_input_item_count);
  S(ksj_cancel_context); F(ksj_cancel_context, kind); F(ksj_cancel_context, terminal_epoch);
  F(ksj_cancel_context, cancellation_generation); F(ksj_cancel_context, reason);
  S(ksj_provider_api); F(ksj_provider_api, operator_create); F(ksj_provider_api, execution_context_create);
  F(ksj_provider_api, key_state_init); F(ksj_provider_api, operator_on_start); F(ksj_provider_api, operator_process_batch);
  F(ksj_provider_api, operator_on_scan_end); F(ksj_provider_api, operator_on_cancel); F(ksj_provider_api, key_state_reset);
  F(ksj_provider_api, execution_context_destroy); F(ksj_provider_api, operator_destroy);
  printf("consts %u %u %u %u %u %u %u %u %u\n", (unsigned)KSJ_STATUS_CONTRACT_VIOLATION,
         (unsigned)KSJ_PROVIDER_MEMORY_DEVICE, (unsigned)KSJ_ELEMENT_TYPE_COMPLEX_FLOAT64,
         (unsigned)KSJ_PROVIDER_SCAN_END_FAILED, (unsigned)KSJ_PROVIDER_PROCESS_CONTRACT_VIOLATION,
         (unsigned)(KSJ_TYPE_STRIDES_EXPLICIT_BYTE >> 16), (unsigned)(KSJ_PROVIDER_CAP_NO_DIRECT_NETWORK_IO >> 8),
         (unsigned)(KSJ_OPERATOR_CAP_CANCEL_NO_THROW >> 5), (unsigned)(KSJ_LEASE_CAP_CANCELLATION >> 6));
  return 0;
}
