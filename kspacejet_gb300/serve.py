"""Python binding of the request loop in include/ksj_serve.h.

A :class:`Server` owns a scheduler thread and ``slots`` CUDA streams on one
device.  Requests (one Kaiser-Bessel slice reconstruction each, of any
readout/spoke/coil shape within the caps) are queued with :meth:`Server.submit`;
pending requests of one class leave together as one ragged multi-frame call
whenever a slot is free, and batches on different slots overlap, as slots and
the device-byte cap allow.  Each result is byte-identical to the same
``ksj_gpu_gridding_adjoint`` call made alone.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import gpu

OUTPUT_RSS = 1
OUTPUT_COIL_MAJOR = 2
HOST_PINNED = 1


class ServeConfig(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("device", ctypes.c_int32), ("slots", ctypes.c_uint32),
                ("max_channels", ctypes.c_uint32), ("device_memory_cap", ctypes.c_uint64),
                ("max_frame_bytes", ctypes.c_uint64), ("max_image_bytes", ctypes.c_uint64),
                ("max_batch_frames", ctypes.c_uint32), ("read_inputs_in_place", ctypes.c_uint32),
                ("coil_split", ctypes.c_uint32), ("reserved0", ctypes.c_uint32)]


class ServeRequest(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("image", ctypes.c_uint32), ("grid", ctypes.c_uint32),
                ("kernel_width", ctypes.c_uint32), ("channels", ctypes.c_uint32), ("samples", ctypes.c_uint32),
                ("output", ctypes.c_uint32), ("dcf_mode", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("reserved0", ctypes.c_uint32), ("trajectory_id", ctypes.c_uint64), ("kspace", ctypes.c_void_p),
                ("trajectory", ctypes.c_void_p), ("out", ctypes.c_void_p)]


class ServeStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("rejected", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("gridded_samples", ctypes.c_uint64), ("wall_seconds", ctypes.c_double),
                ("latency_p50_ms", ctypes.c_double), ("latency_p99_ms", ctypes.c_double),
                ("latency_max_ms", ctypes.c_double), ("peak_device_bytes", ctypes.c_uint64),
                ("peak_in_flight", ctypes.c_uint32), ("reserved0", ctypes.c_uint32),
                ("batches", ctypes.c_uint64), ("batched_frames", ctypes.c_uint64),
                ("copy_in_ms", ctypes.c_double), ("compute_ms", ctypes.c_double), ("copy_out_ms", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved0"}


_bound = False


def _lib() -> ctypes.CDLL:
    global _bound
    L = gpu.lib()
    if not _bound:
        vp = ctypes.c_void_p
        L.ksj_serve_create.restype = ctypes.c_int32
        L.ksj_serve_create.argtypes = [ctypes.POINTER(ServeConfig), ctypes.POINTER(vp)]
        L.ksj_serve_submit.restype = ctypes.c_int32
        L.ksj_serve_submit.argtypes = [vp, ctypes.POINTER(ServeRequest), ctypes.POINTER(ctypes.c_uint64)]
        L.ksj_serve_wait.restype = ctypes.c_int32
        L.ksj_serve_wait.argtypes = [vp, ctypes.c_uint64, ctypes.c_uint32, ctypes.POINTER(ctypes.c_int32)]
        L.ksj_serve_drain.restype = ctypes.c_int32
        L.ksj_serve_drain.argtypes = [vp]
        L.ksj_serve_get_stats.restype = ctypes.c_int32
        L.ksj_serve_get_stats.argtypes = [vp, ctypes.POINTER(ServeStats)]
        L.ksj_serve_reset_stats.restype = None
        L.ksj_serve_reset_stats.argtypes = [vp]
        L.ksj_serve_destroy.restype = None
        L.ksj_serve_destroy.argtypes = [vp]
        _bound = True
    return L


@dataclass
class Request:
    """One slice: kspace complex64 [channels, samples], trajectory float32 [samples, 2]."""

    image: int
    grid: int
    kspace: np.ndarray
    trajectory: np.ndarray
    width: int = 4
    output: int = OUTPUT_RSS
    dcf: int = gpu.DCF_ANALYTIC_RAMP
    trajectory_id: int = 0
    pinned: bool = False
    out: np.ndarray | None = None

    def output_shape(self) -> tuple[int, ...]:
        if self.output == OUTPUT_RSS:
            return (self.image, self.image)
        return (self.kspace.shape[0], self.image, self.image)


class Server:
    def __init__(self, slots: int = 4, device_memory_cap: int = 16 << 30, max_channels: int = 32,
                 max_frame_bytes: int = 256 << 20, max_image_bytes: int = 128 << 20, device: int = 0,
                 max_batch_frames: int = 0, read_inputs_in_place: bool = False, coil_split: int = 0):
        self._L = _lib()
        cfg = ServeConfig(ctypes.sizeof(ServeConfig), device, slots, max_channels, device_memory_cap,
                          max_frame_bytes, max_image_bytes, max_batch_frames, int(read_inputs_in_place),
                          coil_split, 0)
        h = ctypes.c_void_p()
        gpu._check(self._L.ksj_serve_create(ctypes.byref(cfg), ctypes.byref(h)), "serve_create")
        self._h = h
        self._live: dict[int, Request] = {}

    def submit(self, r: Request) -> int:
        """Queue `r`; its arrays must stay alive until :meth:`wait` returns for it."""
        ks = r.kspace
        tr = r.trajectory
        if not r.pinned:
            ks = np.ascontiguousarray(ks, dtype=np.complex64)
            tr = np.ascontiguousarray(tr, dtype=np.float32)
            r.kspace, r.trajectory = ks, tr
        if r.out is None:
            dt = np.float32 if r.output == OUTPUT_RSS else np.complex64
            r.out = np.empty(r.output_shape(), dtype=dt)
        c, m = ks.shape
        req = ServeRequest(ctypes.sizeof(ServeRequest), r.image, r.grid, r.width, c, m, r.output, r.dcf,
                           HOST_PINNED if r.pinned else 0, 0, r.trajectory_id, ks.ctypes.data, tr.ctypes.data,
                           r.out.ctypes.data)
        t = ctypes.c_uint64()
        gpu._check(self._L.ksj_serve_submit(self._h, ctypes.byref(req), ctypes.byref(t)), "serve_submit")
        self._live[t.value] = r
        return int(t.value)

    def wait(self, ticket: int, timeout_ms: int = 0) -> np.ndarray:
        res = ctypes.c_int32()
        gpu._check(self._L.ksj_serve_wait(self._h, ticket, timeout_ms, ctypes.byref(res)), "serve_wait")
        r = self._live.pop(ticket)
        gpu._check(res.value, "serve request")
        return r.out

    def drain(self) -> None:
        gpu._check(self._L.ksj_serve_drain(self._h), "serve_drain")

    def stats(self) -> dict:
        s = ServeStats()
        gpu._check(self._L.ksj_serve_get_stats(self._h, ctypes.byref(s)), "serve_stats")
        return s.as_dict()

    def reset_stats(self) -> None:
        self._L.ksj_serve_reset_stats(self._h)

    def close(self) -> None:
        if self._h:
            self._L.ksj_serve_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
