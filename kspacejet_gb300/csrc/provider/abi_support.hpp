// abi_support.hpp -- Provider-side checks of the KSpaceJet C ABI rules and
// the four payload types of the non-Cartesian path, for the GB300 plug-ins.
//
// The checks implement the normative rules of the ABI header (every struct
// starts with an abi header whose struct_size covers the fields read and
// whose reserved fields are zero; borrowed views are non-null when non-empty;
// errors are Provider-owned static text) -- the same rules the reference
// Provider SDK helpers enforce (libs/recon/kspacejet-provider-sdk/include/
// kspacejet/provider/detail/provider_support.hpp:24-290).
//
// The type table restates the generated registry entries that the plug-ins
// must accept and emit (libs/recon/kspacejet-provider-sdk/include/kspacejet/
// provider/type_registry.h, generated from types/registry.json): a payload
// type matches when every field equals the registry's, including the
// SHA-256 identity digest.  These values are a frozen interface, not a design
// choice; tests/test_abi_layout.py checks them against the reference header.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <string_view>

#include "ksj_provider_abi.h"

namespace ksj_gb300 {

inline ksj_provider_abi_header header(uint32_t size, uint64_t caps = 0) {
  return ksj_provider_abi_header_make(size, caps);
}

template <typename T>
inline bool full_header(const T* v) {
  return v != nullptr && v->abi.struct_size >= sizeof(T) && v->abi.reserved0 == 0 && v->abi.reserved[0] == 0 &&
         v->abi.reserved[1] == 0;
}

inline ksj_utf8_view utf8(const char* data, uint64_t size) {
  ksj_utf8_view v{};
  v.abi = header(sizeof(v));
  v.data = data;
  v.size = size;
  return v;
}

inline bool text_is(const ksj_utf8_view& v, std::string_view s) {
  return full_header(&v) && v.data != nullptr && v.size == s.size() && std::memcmp(v.data, s.data(), s.size()) == 0;
}

inline ksj_status fail(ksj_error_view* err, ksj_status status, std::string_view message) {
  if (full_header(err)) {
    *err = {};
    err->abi = header(sizeof(*err));
    err->status = status;
    err->message = utf8(message.data(), message.size());
  }
  return status;
}

inline bool borrowed_ok(const ksj_byte_view& b) { return full_header(&b) && (b.size == 0 || b.data != nullptr); }

inline bool pow2(uint32_t v) { return v != 0 && (v & (v - 1)) == 0; }

inline bool host_memory_ok(const void* p, uint32_t declared_alignment, uint32_t required) {
  return pow2(required) && declared_alignment >= required && p != nullptr && pow2(declared_alignment) &&
         (reinterpret_cast<uintptr_t>(p) & (static_cast<uintptr_t>(declared_alignment) - 1)) == 0;
}

inline bool lease_callbacks_ok(const ksj_firing_lease_callbacks* cb, uint64_t required) {
  if (!full_header(cb) || cb->get_info == nullptr || (cb->abi.capability_bits & required) != required) return false;
  const uint64_t caps = cb->abi.capability_bits;
  if ((caps & KSJ_LEASE_CAP_INPUT_BATCHES) && cb->get_input_batch == nullptr) return false;
  if (caps & KSJ_LEASE_CAP_OUTPUT_GRANTS) {
    const ksj_output_grant_callbacks* og = cb->output_grants;
    if (cb->acquire_output_grant == nullptr || !full_header(og) || og->map_mutable_payload == nullptr ||
        og->seal == nullptr || og->release == nullptr)
      return false;
  }
  if ((caps & KSJ_LEASE_CAP_SCRATCH) && cb->get_scratch == nullptr) return false;
  if ((caps & KSJ_LEASE_CAP_KEY_STATE) && cb->get_key_state == nullptr) return false;
  if ((caps & KSJ_LEASE_CAP_RETENTION) && (cb->retain_input == nullptr || cb->release_retention == nullptr))
    return false;
  if ((caps & KSJ_LEASE_CAP_ASYNC) &&
      (cb->register_async == nullptr || cb->complete_async == nullptr || cb->release_async == nullptr))
    return false;
  return (caps & KSJ_LEASE_CAP_CANCELLATION) == 0 || cb->get_cancellation != nullptr;
}

inline void done(ksj_process_result* r, uint32_t sealed, uint64_t consumed, uint64_t epoch) {
  if (!full_header(r)) return;
  *r = {};
  r->abi = header(sizeof(*r));
  r->outcome = KSJ_PROVIDER_PROCESS_DONE;
  r->sealed_output_count = sealed;
  r->consumed_input_item_count = consumed;
  r->terminal_epoch = epoch;
}

// Releases an acquired output grant unless it was sealed.
struct GrantGuard {
  const ksj_output_grant_callbacks* cb = nullptr;
  ksj_output_grant* grant = nullptr;
  bool settled = false;
  ~GrantGuard() {
    if (cb == nullptr || grant == nullptr || settled) return;
    ksj_error_view e{};
    e.abi = header(sizeof(e));
    e.message.abi = header(sizeof(e.message));
    (void)cb->release(cb->host_context, grant, &e);
  }
};

inline ksj_digest256 digest_from_hex(std::string_view hex) {
  ksj_digest256 d{};
  if (hex.size() != 64) return d;
  auto nib = [](char c) -> int {
    if (c >= '0' && c <= '9') return c - '0';
    if (c >= 'a' && c <= 'f') return c - 'a' + 10;
    if (c >= 'A' && c <= 'F') return c - 'A' + 10;
    return -1;
  };
  for (int i = 0; i < 32; ++i) {
    const int hi = nib(hex[2 * i]), lo = nib(hex[2 * i + 1]);
    if (hi < 0 || lo < 0) return ksj_digest256{};
    d.bytes[i] = static_cast<uint8_t>(hi * 16 + lo);
  }
  d.abi = header(sizeof(d));
  return d;
}

// ------------------------------------------------------------ payload types

struct PayloadType {
  std::string_view type_ref;
  std::string_view digest_hex;
  uint32_t element_type;
  uint32_t rank;
  uint64_t layout_flags;
  std::string_view dims[3];
};

// types/registry.json entries as generated into type_registry.h.
inline constexpr PayloadType kNoncartesianKspaceFrame{
    "ksj.noncartesian-kspace-frame",
    "c9b88da9074503096e68f8aeb005fdcfa91e5dd6c2b9820e02afd597807e085d",
    KSJ_ELEMENT_TYPE_COMPLEX_FLOAT32,
    2,
    KSJ_TYPE_LAYOUT_CHANNEL_MAJOR_CONTIGUOUS | KSJ_TYPE_STRIDES_CANONICAL,
    {"channel", "sample", ""}};
inline constexpr PayloadType kTrajectoryFrame{
    "ksj.trajectory-frame",
    "10500da95cd005c237c3b5e811573864ce99729e41c15e54697cb473a72d81e7",
    KSJ_ELEMENT_TYPE_FLOAT32,
    2,
    KSJ_TYPE_LAYOUT_ROW_MAJOR_CONTIGUOUS | KSJ_TYPE_STRIDES_CANONICAL,
    {"sample", "coordinate", ""}};
inline constexpr PayloadType kCoilImageFrame{
    "ksj.coil-image-frame",
    "cb9c72b7143769f37f002ecc2983b7f24469c40af95b4fb0bbc8bef2b4741a87",
    KSJ_ELEMENT_TYPE_COMPLEX_FLOAT32,
    3,
    KSJ_TYPE_LAYOUT_ROW_MAJOR_CONTIGUOUS | KSJ_TYPE_STRIDES_CANONICAL,
    {"ky", "kx", "channel"}};
inline constexpr PayloadType kImageFrame{
    "ksj.image-frame",
    "66d13ed43407ba9dd449327f62a752f8137d328bad2620f56b817bf2140b3586",
    KSJ_ELEMENT_TYPE_FLOAT32,
    2,
    KSJ_TYPE_LAYOUT_ROW_MAJOR_CONTIGUOUS | KSJ_TYPE_STRIDES_CANONICAL,
    {"ky", "kx", ""}};

// Structural validity of any type descriptor (the SDK's
// has_valid_type_descriptor, provider_support.hpp:159-180).
inline bool type_descriptor_ok(const ksj_type_descriptor_view& t) {
  if (!full_header(&t) || !full_header(&t.type_ref) || t.type_ref.data == nullptr || t.type_ref.size == 0 ||
      !full_header(&t.type_identity_digest) || t.rank > 8 || t.minimum_alignment == 0 || t.reserved0 != 0 ||
      (t.rank != 0 && t.dimension_names == nullptr) || !pow2(t.minimum_alignment))
    return false;
  for (uint32_t i = 0; i < t.rank; ++i) {
    const ksj_utf8_view& d = t.dimension_names[i];
    if (!full_header(&d) || d.data == nullptr || d.size == 0) return false;
  }
  return true;
}

// Exact match against one registry entry (every field, as the generated
// ksj_type_registry_matches_* functions compare).
inline bool type_matches(const ksj_type_descriptor_view& t, const PayloadType& p) {
  if (!type_descriptor_ok(t)) return false;
  if (!text_is(t.type_ref, p.type_ref) || t.payload_kind != KSJ_PAYLOAD_KIND_BUFFER_HANDLE ||
      t.element_type != p.element_type || t.rank != p.rank || t.layout_flags != p.layout_flags ||
      t.allowed_memory_domains != KSJ_PROVIDER_MEMORY_HOST_PAGEABLE || t.minimum_alignment != 64 ||
      t.mutability != KSJ_PAYLOAD_MUTABILITY_IMMUTABLE_AFTER_PUBLISH)
    return false;
  const ksj_digest256 want = digest_from_hex(p.digest_hex);
  if (std::memcmp(t.type_identity_digest.bytes, want.bytes, 32) != 0) return false;
  for (uint32_t i = 0; i < p.rank; ++i) {
    const ksj_utf8_view& d = t.dimension_names[i];
    if (d.data == nullptr || d.size != p.dims[i].size() || std::memcmp(d.data, p.dims[i].data(), d.size) != 0)
      return false;
  }
  for (int i = 0; i < 8; ++i)
    if (t.stride_bytes[i] != 0) return false;
  return true;
}

// --------------------------------------------------------- canonical config

// Canonical positive decimal without sign or leading zero, in [lo, hi]
// (parse_canonical_positive_u32, provider_support.hpp:189-206).
inline bool parse_u32(std::string_view text, uint32_t lo, uint32_t hi, uint32_t* out) {
  if (text.empty() || text.size() > 10 || text[0] == '0') return false;
  uint64_t v = 0;
  for (char c : text) {
    if (c < '0' || c > '9') return false;
    v = v * 10 + static_cast<uint64_t>(c - '0');
  }
  if (v == 0 || v > 0xffffffffull || v < lo || v > hi) return false;
  *out = static_cast<uint32_t>(v);
  return true;
}

// A canonical config is `{` key-value pairs in a fixed order `}` with no
// whitespace.  `keys` alternates literal separators and value slots: each
// literal must occur in order after the previous match; the text between two
// literals is a value.  Returns false unless the whole string is consumed.
// This is the matching discipline of the reference operators'
// parse_canonical_config (radial_gridding_reconstruct.cpp:99-144).
inline bool split_canonical(const ksj_byte_view& config, const std::string_view* literals, int nliterals,
                            std::string_view* values) {
  if (!full_header(&config) || config.data == nullptr || config.size == 0 || config.size > (1u << 20)) return false;
  const std::string_view s(static_cast<const char*>(config.data), static_cast<size_t>(config.size));
  if (s.substr(0, literals[0].size()) != literals[0]) return false;
  size_t pos = literals[0].size();
  for (int i = 1; i < nliterals; ++i) {
    const bool last = i == nliterals - 1;
    size_t at;
    if (last) {
      if (s.size() < literals[i].size() || s.substr(s.size() - literals[i].size()) != literals[i]) return false;
      at = s.size() - literals[i].size();
      if (at < pos) return false;
    } else {
      at = s.find(literals[i], pos);
      if (at == std::string_view::npos) return false;
    }
    values[i - 1] = s.substr(pos, at - pos);
    pos = at + literals[i].size();
  }
  return pos == s.size();
}

}  // namespace ksj_gb300
