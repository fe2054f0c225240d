"""Python front end of ``libksj_firing_host.so``: load a Provider plug-in,
create an operator instance, fire it with numpy host buffers.  Mirrors the
reference Provider tests' harness (HostState + CallbackTables)."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import FIRING_HOST_LIB, NativeLibraryMissing

TYPE_KSPACE, TYPE_TRAJECTORY, TYPE_COIL_IMAGE, TYPE_IMAGE = 0, 1, 2, 3
STATUS = {0: "OK", 1: "BAD_ABI", 2: "INVALID_ARGUMENT", 3: "UNSUPPORTED", 4: "RESOURCE_EXHAUSTED", 5: "CANCELLED",
          6: "FAILED_PRECONDITION", 7: "INTERNAL_ERROR", 8: "CONTRACT_VIOLATION"}
OK, INVALID_ARGUMENT, UNSUPPORTED, INTERNAL_ERROR, CONTRACT_VIOLATION = 0, 2, 3, 7, 8
RESOURCE_EXHAUSTED, FAILED_PRECONDITION = 4, 6
SCAN_END_NORMAL, SCAN_END_CANCELLED, SCAN_END_FAILED = 0, 1, 2


class Firing(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("input_count", ctypes.c_uint32),
                ("payload", ctypes.c_void_p * 2), ("payload_bytes", ctypes.c_uint64 * 2),
                ("payload_type", ctypes.c_uint32 * 2), ("payload_port", ctypes.c_uint32 * 2),
                ("semantic_key_hash", ctypes.c_uint64 * 2), ("order_key", ctypes.c_uint64 * 2),
                ("metadata", ctypes.c_void_p), ("metadata_bytes", ctypes.c_uint64),
                ("output", ctypes.c_void_p), ("output_capacity", ctypes.c_uint64), ("output_type", ctypes.c_uint32),
                ("reported_input_batch_count", ctypes.c_uint32), ("scratch", ctypes.c_void_p),
                ("scratch_bytes", ctypes.c_uint64), ("reserved_output_bytes", ctypes.c_uint64),
                ("reserved_scratch_bytes", ctypes.c_uint64), ("reverse_batch_order", ctypes.c_uint32),
                ("corrupt_input_type", ctypes.c_uint32), ("corrupt_output_type", ctypes.c_uint32),
                ("reserved0", ctypes.c_uint32), ("terminal_epoch", ctypes.c_uint64),
                ("status", ctypes.c_uint32), ("outcome", ctypes.c_uint32), ("sealed_count", ctypes.c_uint32),
                ("acquire_calls", ctypes.c_uint32), ("map_calls", ctypes.c_uint32), ("seal_calls", ctypes.c_uint32),
                ("release_calls", ctypes.c_uint32), ("input_batch_requests", ctypes.c_uint32),
                ("consumed", ctypes.c_uint64), ("sealed_bytes", ctypes.c_uint64), ("sealed_key", ctypes.c_uint64),
                ("sealed_order", ctypes.c_uint64), ("sealed_metadata_size", ctypes.c_uint64),
                ("sealed_metadata", ctypes.c_void_p), ("error", ctypes.c_char * 512)]


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not FIRING_HOST_LIB.exists():
            raise NativeLibraryMissing(f"{FIRING_HOST_LIB} is not built; run kspacejet_gb300.build()")
        L = ctypes.CDLL(str(FIRING_HOST_LIB))
        vp, cp = ctypes.c_void_p, ctypes.c_char_p
        L.ksjh_load.restype = ctypes.c_int
        L.ksjh_load.argtypes = [cp, ctypes.POINTER(vp), cp, ctypes.c_size_t]
        L.ksjh_unload.argtypes = [vp]
        L.ksjh_describe.restype = ctypes.c_int
        L.ksjh_describe.argtypes = [vp, cp, ctypes.c_size_t, vp, ctypes.POINTER(ctypes.c_uint32),
                                    ctypes.POINTER(ctypes.c_uint64)]
        L.ksjh_operator_info.restype = ctypes.c_int
        L.ksjh_operator_info.argtypes = [vp, ctypes.c_uint32, cp, ctypes.c_size_t, vp]
        L.ksjh_try_create.restype = ctypes.c_uint32
        L.ksjh_try_create.argtypes = [vp, cp, cp, ctypes.c_size_t, cp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_int)]
        L.ksjh_create.restype = ctypes.c_uint32
        L.ksjh_create.argtypes = [vp, cp, cp, ctypes.c_size_t, ctypes.c_uint32, ctypes.POINTER(vp), cp,
                                  ctypes.c_size_t]
        L.ksjh_destroy.argtypes = [vp]
        L.ksjh_firing_size.restype = ctypes.c_size_t
        L.ksjh_fire.restype = ctypes.c_uint32
        L.ksjh_fire.argtypes = [vp, ctypes.POINTER(Firing)]
        L.ksjh_cancel.restype = ctypes.c_uint32
        L.ksjh_cancel.argtypes = [vp, ctypes.c_uint32, cp]
        if L.ksjh_firing_size() != ctypes.sizeof(Firing):
            raise RuntimeError("firing host struct layout mismatch")
        _lib = L
    return _lib


def aligned(shape, dtype, alignment: int = 64) -> np.ndarray:
    """Zeroed numpy array whose data pointer is `alignment`-byte aligned."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape)) * dtype.itemsize
    raw = np.zeros(n + alignment, dtype=np.uint8)
    off = (-raw.ctypes.data) % alignment
    return raw[off:off + n].view(dtype).reshape(shape)


def aligned_copy(a: np.ndarray, alignment: int = 64) -> np.ndarray:
    out = aligned(a.shape, a.dtype, alignment)
    out[...] = a
    return out


@dataclass
class OperatorInfo:
    id: str
    max_in_flight: int
    thread_safety: int
    max_private_threads: int
    max_inputs: int
    max_outputs: int
    max_output_bytes: int
    max_scratch_bytes: int
    max_retained_input_bytes: int
    capability_bits: int


class ProviderModule:
    def __init__(self, path: str | Path):
        L = lib()
        h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(512)
        rc = L.ksjh_load(str(path).encode(), ctypes.byref(h), err, 512)
        if rc != 0:
            raise RuntimeError(f"cannot load Provider {path}: {rc} {err.value.decode(errors='replace')}")
        self._h = h
        pid = ctypes.create_string_buffer(256)
        self.bundle_digest = (ctypes.c_uint8 * 32)()
        n = ctypes.c_uint32()
        caps = ctypes.c_uint64()
        L.ksjh_describe(h, pid, 256, self.bundle_digest, ctypes.byref(n), ctypes.byref(caps))
        self.provider_id = pid.value.decode()
        self.capability_bits = caps.value
        self.digest_hex = bytes(self.bundle_digest).hex()
        self.operators = []
        for i in range(n.value):
            name = ctypes.create_string_buffer(256)
            f = (ctypes.c_uint64 * 10)()
            L.ksjh_operator_info(h, i, name, 256, f)
            self.operators.append(OperatorInfo(name.value.decode(), *[int(x) for x in f[:8]], int(f[9])))

    def try_create(self, operator_id: str, config: str) -> tuple[int, bool, str]:
        err = ctypes.create_string_buffer(512)
        created = ctypes.c_int()
        cfg = config.encode()
        st = lib().ksjh_try_create(self._h, operator_id.encode(), cfg, len(cfg), err, 512, ctypes.byref(created))
        return int(st), bool(created.value), err.value.decode(errors="replace")

    def instance(self, operator_id: str, config: str, device: int = 0) -> "Instance":
        return Instance(self, operator_id, config, device)

    def close(self):
        if self._h:
            lib().ksjh_unload(self._h)
            self._h = None


@dataclass
class FireResult:
    status: int
    outcome: int
    sealed_count: int
    consumed: int
    acquire_calls: int
    map_calls: int
    seal_calls: int
    release_calls: int
    input_batch_requests: int
    sealed_bytes: int
    sealed_key: int
    sealed_order: int
    sealed_metadata: int
    sealed_metadata_size: int
    error: str
    output: np.ndarray | None = field(default=None, repr=False)


class Instance:
    def __init__(self, module: ProviderModule, operator_id: str, config: str, device: int = 0):
        self.module = module
        h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(512)
        cfg = config.encode()
        st = lib().ksjh_create(module._h, operator_id.encode(), cfg, len(cfg), device, ctypes.byref(h), err, 512)
        if st != 0:
            raise RuntimeError(f"operator {operator_id} not created: {STATUS.get(st, st)} {err.value.decode()}")
        self._h = h

    def close(self):
        if self._h:
            lib().ksjh_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def cancel(self, kind: int = SCAN_END_CANCELLED) -> tuple[int, str]:
        """operator_on_cancel (no lease, no grants); returns (status, error message)."""
        err = ctypes.create_string_buffer(512)
        st = lib().ksjh_cancel(self._h, kind, err)
        return int(st), err.value.decode(errors="replace")

    def fire(self, inputs: list[tuple[np.ndarray, int, int]], output: np.ndarray, output_type: int,
             scratch_bytes: int = 0, metadata: bytes = b"\x31\x32\x33", keys=(71, 73), input_keys=None,
             reserved_output_bytes: int | None = None, reserved_scratch_bytes: int | None = None,
             reported_input_batch_count: int | None = None, reverse_batch_order: bool = False,
             corrupt_input_type: int = 0, corrupt_output_type: bool = False,
             terminal_epoch: int = 89) -> FireResult:
        """inputs: [(array, payload type, port)], each 64-byte aligned host memory."""
        f = Firing()
        f.struct_size = ctypes.sizeof(Firing)
        f.input_count = len(inputs)
        for i, (arr, typ, port) in enumerate(inputs):
            if arr.ctypes.data % 64:
                raise ValueError("payloads must be 64-byte aligned (use host.aligned_copy)")
            f.payload[i] = arr.ctypes.data
            f.payload_bytes[i] = arr.nbytes
            f.payload_type[i] = typ
            f.payload_port[i] = port
            k = input_keys[i] if input_keys else keys
            f.semantic_key_hash[i] = k[0]
            f.order_key[i] = k[1]
        self._meta = ctypes.create_string_buffer(metadata, len(metadata)) if metadata else None
        f.metadata = ctypes.addressof(self._meta) if metadata else None
        f.metadata_bytes = len(metadata) if metadata else 0
        f.output = output.ctypes.data
        f.output_capacity = output.nbytes
        f.output_type = output_type
        f.reported_input_batch_count = len(inputs) if reported_input_batch_count is None else reported_input_batch_count
        scratch = aligned((max(1, scratch_bytes),), np.uint8)
        f.scratch = scratch.ctypes.data
        f.scratch_bytes = scratch_bytes
        f.reserved_output_bytes = output.nbytes if reserved_output_bytes is None else reserved_output_bytes
        f.reserved_scratch_bytes = scratch_bytes if reserved_scratch_bytes is None else reserved_scratch_bytes
        f.reverse_batch_order = int(reverse_batch_order)
        f.corrupt_input_type = corrupt_input_type
        f.corrupt_output_type = int(corrupt_output_type)
        f.terminal_epoch = terminal_epoch
        lib().ksjh_fire(self._h, ctypes.byref(f))
        return FireResult(f.status, f.outcome, f.sealed_count, f.consumed, f.acquire_calls, f.map_calls, f.seal_calls,
                          f.release_calls, f.input_batch_requests, f.sealed_bytes, f.sealed_key, f.sealed_order,
                          f.sealed_metadata or 0, f.sealed_metadata_size, f.error.decode(errors="replace"), output)


# ----------------------------------------------------------- config strings

def radial_config(channels: int, rows: int, cols: int, samples: int) -> str:
    return (f'{{"channels":{channels},"density_compensation":"radial_analytic_ramp","image_cols":{cols},'
            f'"image_rows":{rows},"sample_count":{samples},"trajectory_units":"radians_per_pixel"}}')


def direct_config(channels: int, rows: int, cols: int, samples: int) -> str:
    return f'{{"channels":{channels},"image_cols":{cols},"image_rows":{rows},"sample_count":{samples}}}'


def rss_config(channels: int, rows: int, cols: int) -> str:
    return f'{{"channels":{channels},"cols":{cols},"rows":{rows}}}'


def radial_scratch_bytes(rows: int, cols: int, samples: int) -> int:
    """Host scratch the reference radial operator demands (:178-181)."""
    return (2 * rows * cols + 2 * max(rows, cols)) * 8 + samples * 4
