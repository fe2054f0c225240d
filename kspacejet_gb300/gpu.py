"""ctypes bindings for ``include/ksj_gpu.h`` over torch CUDA tensors.

torch provides device memory and streams only; all arithmetic happens in
``libksj_gpu.so``.  Loading fails loudly if the library is missing.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import torch

from . import GPU_LIB, NativeLibraryMissing

KERNEL_LINEAR, KERNEL_KAISER_BESSEL = 0, 1
DCF_NONE, DCF_ANALYTIC_RAMP, DCF_EXTERNAL = 0, 1, 2
OUTPUT_COIL_LAST, OUTPUT_RSS, OUTPUT_COIL_MAJOR = 0, 1, 2
SAMPLES_CF32, SAMPLES_BF16 = 0, 1
FLAG_NONFINITE_SAMPLE, FLAG_BAD_TRAJECTORY, FLAG_BAD_DCF, FLAG_WAIT_TIMEOUT = 1, 2, 4, 8

STATUS_TEXT = {0: "ok", 1: "invalid argument", 2: "unsupported", 3: "CUDA error", 4: "workspace",
               5: "out of memory", 6: "non-finite input"}


class GpuError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: ksj_gpu status {status} ({STATUS_TEXT.get(status, '?')})")
        self.status = status


class GriddingDesc(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("kernel", ctypes.c_uint32), ("image_rows", ctypes.c_uint32),
                ("image_cols", ctypes.c_uint32), ("grid_rows", ctypes.c_uint32), ("grid_cols", ctypes.c_uint32),
                ("kernel_width", ctypes.c_uint32), ("kb_beta", ctypes.c_float), ("row_origin", ctypes.c_double),
                ("col_origin", ctypes.c_double), ("channels", ctypes.c_uint32), ("samples", ctypes.c_uint32),
                ("frames", ctypes.c_uint32), ("dcf_mode", ctypes.c_uint32), ("output", ctypes.c_uint32),
                ("sample_format", ctypes.c_uint32), ("require_nyquist", ctypes.c_uint32),
                ("reserved0", ctypes.c_uint32)]


class GriddingTuning(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("coil_group", ctypes.c_uint32),
                ("column_block", ctypes.c_uint32), ("list_capacity", ctypes.c_uint32),
                ("frames_per_pass", ctypes.c_uint32), ("rows_blocks_per_sm", ctypes.c_uint32),
                ("coil_parts", ctypes.c_uint32), ("column_pass", ctypes.c_uint32),
                ("wait_fault_polls", ctypes.c_uint32)]


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not GPU_LIB.exists():
            raise NativeLibraryMissing(f"{GPU_LIB} is not built; run kspacejet_gb300.build()")
        L = ctypes.CDLL(str(GPU_LIB))
        vp, u32, u64, sz = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_size_t
        L.ksj_gpu_gridding_workspace_bytes.restype = sz
        L.ksj_gpu_gridding_workspace_bytes.argtypes = [ctypes.POINTER(GriddingDesc)]
        L.ksj_gpu_gridding_host_workspace_bytes.restype = sz
        L.ksj_gpu_gridding_host_workspace_bytes.argtypes = [ctypes.POINTER(GriddingDesc)]
        L.ksj_gpu_gridding_adjoint_host.restype = ctypes.c_int32
        L.ksj_gpu_gridding_adjoint_host.argtypes = [ctypes.POINTER(GriddingDesc), ctypes.POINTER(GriddingTuning), vp,
                                                    vp, vp, vp, vp, sz, vp]
        L.ksj_gpu_gridding_adjoint.restype = ctypes.c_int32
        L.ksj_gpu_gridding_adjoint.argtypes = [ctypes.POINTER(GriddingDesc), ctypes.POINTER(GriddingTuning), vp, vp,
                                               vp, vp, vp, sz, vp]
        L.ksj_gpu_gridding_binning.restype = ctypes.c_int32
        L.ksj_gpu_gridding_binning.argtypes = [ctypes.POINTER(GriddingDesc), ctypes.POINTER(GriddingTuning), vp,
                                               ctypes.POINTER(u32), ctypes.POINTER(u64), ctypes.POINTER(u64), vp, vp]
        L.ksj_gpu_read_flags.restype = ctypes.c_int32
        L.ksj_gpu_read_flags.argtypes = [vp, vp, ctypes.POINTER(u32)]
        L.ksj_gpu_inject_allocation_failures.restype = None
        L.ksj_gpu_inject_allocation_failures.argtypes = [u32]
        L.ksj_gpu_gridding_tune.restype = ctypes.c_int32
        L.ksj_gpu_gridding_tune.argtypes = [ctypes.POINTER(GriddingDesc), vp, vp, vp, vp, vp, sz, vp,
                                            ctypes.POINTER(GriddingTuning)]
        L.ksj_gpu_direct_workspace_bytes.restype = sz
        L.ksj_gpu_direct_workspace_bytes.argtypes = [u32, u32, u32]
        L.ksj_gpu_normalize_trajectory.restype = ctypes.c_int32
        L.ksj_gpu_normalize_trajectory.argtypes = [u32, u32, u32, u32, vp, vp, vp, vp]
        L.ksj_gpu_aggregate_acquisitions.restype = ctypes.c_int32
        L.ksj_gpu_aggregate_acquisitions.argtypes = [u32, u32, u32, vp, vp, vp]
        L.ksj_gpu_cartesian_workspace_bytes.restype = sz
        L.ksj_gpu_cartesian_workspace_bytes.argtypes = [u32, u32, u32, u32]
        L.ksj_gpu_cartesian_ifft2.restype = ctypes.c_int32
        L.ksj_gpu_cartesian_ifft2.argtypes = [u32, u32, u32, u32, u32, vp, vp, vp, sz, vp]
        L.ksj_gpu_kb_forward_workspace_bytes.restype = sz
        L.ksj_gpu_kb_forward_workspace_bytes.argtypes = [ctypes.POINTER(GriddingDesc)]
        L.ksj_gpu_kb_forward.restype = ctypes.c_int32
        L.ksj_gpu_kb_forward.argtypes = [ctypes.POINTER(GriddingDesc), vp, vp, vp, vp, sz, vp]
        L.ksj_gpu_direct_forward.restype = ctypes.c_int32
        L.ksj_gpu_direct_forward.argtypes = [u32, u32, ctypes.c_double, ctypes.c_double, u32, u32, vp, vp, vp, vp]
        L.ksj_gpu_direct_adjoint.restype = ctypes.c_int32
        L.ksj_gpu_direct_adjoint.argtypes = [u32, u32, ctypes.c_double, ctypes.c_double, u32, u32, vp, vp, vp, vp,
                                             sz, vp]
        L.ksj_gpu_pipe_menon_workspace_bytes.restype = sz
        L.ksj_gpu_pipe_menon_workspace_bytes.argtypes = [ctypes.POINTER(GriddingDesc)]
        L.ksj_gpu_pipe_menon_dcf.restype = ctypes.c_int32
        L.ksj_gpu_pipe_menon_dcf.argtypes = [ctypes.POINTER(GriddingDesc), u32, vp, vp, vp, sz, vp]
        L.ksj_gpu_walsh_combine.restype = ctypes.c_int32
        L.ksj_gpu_walsh_combine.argtypes = [u32, u32, u32, u32, u32, vp, vp, vp]
        L.ksj_gpu_coil_covariance_workspace_bytes.restype = sz
        L.ksj_gpu_coil_covariance_workspace_bytes.argtypes = [u32, u32]
        L.ksj_gpu_coil_covariance.restype = ctypes.c_int32
        L.ksj_gpu_coil_covariance.argtypes = [u32, u32, vp, vp, vp, sz, vp]
        L.ksj_coil_compression_basis.restype = ctypes.c_int32
        L.ksj_coil_compression_basis.argtypes = [u32, u32, vp, vp, vp]
        L.ksj_gpu_coil_compress.restype = ctypes.c_int32
        L.ksj_gpu_coil_compress.argtypes = [u32, u32, u32, vp, vp, vp, vp]
        L.ksj_gpu_noise_covariance.restype = ctypes.c_int32
        L.ksj_gpu_noise_covariance.argtypes = [u32, u32, vp, vp, vp, sz, vp]
        L.ksj_whitening_matrix.restype = ctypes.c_int32
        L.ksj_whitening_matrix.argtypes = [u32, vp, ctypes.c_float, vp]
        L.ksj_gpu_noise_prewhiten.restype = ctypes.c_int32
        L.ksj_gpu_noise_prewhiten.argtypes = [u32, u32, vp, vp, vp, vp]
        L.ksj_gpu_gridding3_workspace_bytes.restype = sz
        L.ksj_gpu_gridding3_workspace_bytes.argtypes = [ctypes.POINTER(Gridding3Desc)]
        L.ksj_gpu_gridding3_adjoint.restype = ctypes.c_int32
        L.ksj_gpu_gridding3_adjoint.argtypes = [ctypes.POINTER(Gridding3Desc), ctypes.POINTER(GriddingTuning), vp, vp,
                                                vp, vp, vp, sz, vp]
        L.ksj_gpu_pipe_menon3_workspace_bytes.restype = sz
        L.ksj_gpu_pipe_menon3_workspace_bytes.argtypes = [ctypes.POINTER(Gridding3Desc)]
        L.ksj_gpu_pipe_menon_dcf3.restype = ctypes.c_int32
        L.ksj_gpu_pipe_menon_dcf3.argtypes = [ctypes.POINTER(Gridding3Desc), u32, vp, vp, vp, sz, vp]
        L.ksj_gpu_rss_coil_last.restype = ctypes.c_int32
        L.ksj_gpu_rss_coil_last.argtypes = [u64, u32, vp, vp, vp]
        L.ksj_gpu_launch_count.restype = u64
        L.ksj_gpu_launch_count.argtypes = []
        L.ksj_gpu_timing_enable.argtypes = [ctypes.c_int]
        L.ksj_gpu_timing_reset.argtypes = []
        L.ksj_gpu_timing_read.restype = u32
        L.ksj_gpu_timing_read.argtypes = [u32, vp, vp, vp]
        L.ksj_gpu_status_string.restype = ctypes.c_char_p
        L.ksj_gpu_status_string.argtypes = [ctypes.c_int32]
        _lib = L
    return _lib


def _check(status: int, what: str) -> None:
    if status != 0:
        raise GpuError(status, what)


def _stream(stream: torch.cuda.Stream | None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def launch_count() -> int:
    return int(lib().ksj_gpu_launch_count())


def timing_enable(on: bool = True) -> None:
    lib().ksj_gpu_timing_enable(1 if on else 0)


def timing_reset() -> None:
    lib().ksj_gpu_timing_reset()


def timing_read() -> list[tuple[str, int, float]]:
    """[(kernel name, launches, total ms)] since the last reset (waits for the events)."""
    L = lib()
    n = int(L.ksj_gpu_timing_read(0, None, None, None))
    names = ctypes.create_string_buffer(48 * max(n, 1))
    launches = (ctypes.c_uint64 * max(n, 1))()
    ms = (ctypes.c_double * max(n, 1))()
    n = int(L.ksj_gpu_timing_read(n, names, launches, ms))
    raw = names.raw
    return [(raw[48 * i:48 * i + 48].split(b"\0")[0].decode(), int(launches[i]), float(ms[i])) for i in range(n)]


@dataclass
class Gridding:
    """One adjoint-gridding shape (see ``ksj_gpu_gridding_desc``)."""

    image: tuple[int, int]
    channels: int
    samples: int
    frames: int = 1
    kernel: int = KERNEL_LINEAR
    grid: tuple[int, int] | None = None
    width: int = 2
    beta: float = 0.0
    origin: tuple[float, float] | None = None
    dcf: int = DCF_ANALYTIC_RAMP
    output: int = OUTPUT_COIL_LAST
    sample_format: int = SAMPLES_CF32
    require_nyquist: bool = True

    def desc(self) -> GriddingDesc:
        rows, cols = self.image
        grid = self.grid if self.grid is not None else self.image
        ro, co = self.origin if self.origin is not None else ((rows - 1) / 2.0, (cols - 1) / 2.0)
        return GriddingDesc(ctypes.sizeof(GriddingDesc), self.kernel, rows, cols, grid[0], grid[1], self.width,
                            self.beta, ro, co, self.channels, self.samples, self.frames, self.dcf, self.output,
                            self.sample_format, int(self.require_nyquist), 0)

    def workspace_bytes(self) -> int:
        d = self.desc()
        n = lib().ksj_gpu_gridding_workspace_bytes(ctypes.byref(d))
        if n == 0:
            raise GpuError(1, "gridding_workspace_bytes")
        return int(n)

    def output_shape(self) -> tuple[int, ...]:
        rows, cols = self.image
        if self.output == OUTPUT_RSS:
            return (self.frames, rows, cols)
        if self.output == OUTPUT_COIL_MAJOR:
            return (self.frames, self.channels, rows, cols)
        return (self.frames, rows, cols, self.channels)

    def output_dtype(self) -> torch.dtype:
        return torch.float32 if self.output == OUTPUT_RSS else torch.complex64

    def new_workspace(self, device="cuda") -> torch.Tensor:
        return torch.empty(self.workspace_bytes(), dtype=torch.uint8, device=device)

    def new_output(self, device="cuda") -> torch.Tensor:
        return torch.empty(self.output_shape(), dtype=self.output_dtype(), device=device)

    def run(self, kspace: torch.Tensor, traj: torch.Tensor, out: torch.Tensor, workspace: torch.Tensor,
            dcf: torch.Tensor | None = None, tuning: GriddingTuning | None = None,
            stream: torch.cuda.Stream | None = None) -> None:
        d = self.desc()
        for t in (kspace, traj, out, workspace):
            if not t.is_cuda or not t.is_contiguous():
                raise ValueError("tensors must be contiguous CUDA tensors")
        st = lib().ksj_gpu_gridding_adjoint(ctypes.byref(d), ctypes.byref(tuning) if tuning else None,
                                            kspace.data_ptr(), traj.data_ptr(),
                                            dcf.data_ptr() if dcf is not None else None, out.data_ptr(),
                                            workspace.data_ptr(), workspace.numel(), _stream(stream))
        _check(st, "gridding_adjoint")

    def host_workspace_bytes(self) -> int:
        d = self.desc()
        n = lib().ksj_gpu_gridding_host_workspace_bytes(ctypes.byref(d))
        if n == 0:
            raise GpuError(1, "gridding_host_workspace_bytes")
        return int(n)

    def new_host_workspace(self, device="cuda") -> torch.Tensor:
        """Device workspace of run_host (the device workspace plus device copies of inputs and images)."""
        return torch.empty(self.host_workspace_bytes(), dtype=torch.uint8, device=device)

    def run_host(self, kspace: torch.Tensor, traj: torch.Tensor, out: torch.Tensor, workspace: torch.Tensor,
                 dcf: torch.Tensor | None = None, tuning: GriddingTuning | None = None,
                 stream: torch.cuda.Stream | None = None) -> None:
        """ksj_gpu_gridding_adjoint_host: kspace, traj, dcf and out are contiguous host (CPU) tensors, pinned for
        the copies to overlap the passes; asynchronous on `stream` (synchronise before reading `out`)."""
        d = self.desc()
        for t in (kspace, traj, out) + ((dcf,) if dcf is not None else ()):
            if t.is_cuda or not t.is_contiguous():
                raise ValueError("kspace, traj, dcf and out must be contiguous host tensors")
        if not workspace.is_cuda:
            raise ValueError("the workspace is device memory")
        st = lib().ksj_gpu_gridding_adjoint_host(ctypes.byref(d), ctypes.byref(tuning) if tuning else None,
                                                 kspace.data_ptr(), traj.data_ptr(),
                                                 dcf.data_ptr() if dcf is not None else None, out.data_ptr(),
                                                 workspace.data_ptr(), workspace.numel(), _stream(stream))
        _check(st, "gridding_adjoint_host")

    def forward_workspace_bytes(self) -> int:
        d = self.desc()
        n = lib().ksj_gpu_kb_forward_workspace_bytes(ctypes.byref(d))
        if n == 0:
            raise GpuError(1, "kb_forward_workspace_bytes")
        return int(n)

    def forward(self, image: torch.Tensor, traj: torch.Tensor, workspace: torch.Tensor | None = None,
                stream: torch.cuda.Stream | None = None) -> torch.Tensor:
        """ksj_gpu_kb_forward: coil-last images [F, rows, cols, C] complex64 (F may be omitted when frames == 1),
        traj [F, M, 2] -> samples [F, C, M] complex64 (the transpose of run() without density weights)."""
        d = self.desc()
        if workspace is None:
            workspace = torch.empty(self.forward_workspace_bytes(), dtype=torch.uint8, device=image.device)
        out = torch.empty((self.frames, self.channels, self.samples), dtype=torch.complex64, device=image.device)
        _check(lib().ksj_gpu_kb_forward(ctypes.byref(d), image.contiguous().data_ptr(), traj.contiguous().data_ptr(),
                                        out.data_ptr(), workspace.data_ptr(), workspace.numel(), _stream(stream)),
               "kb_forward")
        return out

    def flags(self, workspace: torch.Tensor, stream: torch.cuda.Stream | None = None) -> int:
        v = ctypes.c_uint32()
        _check(lib().ksj_gpu_read_flags(workspace.data_ptr(), _stream(stream), ctypes.byref(v)), "read_flags")
        return int(v.value)

    def binning(self, workspace: torch.Tensor, tuning: GriddingTuning | None = None):
        """(chunk_width, offsets[frames*lists+1] int64, samples uint32) of the last call."""
        import numpy as np

        d = self.desc()
        cw, nl, ne = ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_uint64()
        L = lib()
        tp = ctypes.byref(tuning) if tuning else None
        _check(L.ksj_gpu_gridding_binning(ctypes.byref(d), tp, workspace.data_ptr(), ctypes.byref(cw),
                                          ctypes.byref(nl), ctypes.byref(ne), None, None), "binning sizes")
        off = np.zeros(nl.value + 1, dtype=np.uint64)
        smp = np.zeros(max(1, ne.value), dtype=np.uint32)
        _check(L.ksj_gpu_gridding_binning(ctypes.byref(d), tp, workspace.data_ptr(), None, None, None,
                                          off.ctypes.data, smp.ctypes.data), "binning")
        return int(cw.value), off.astype(np.int64), smp[: ne.value]

    def tune(self, kspace, traj, out, workspace, dcf=None, stream=None) -> GriddingTuning:
        d = self.desc()
        t = GriddingTuning()
        _check(lib().ksj_gpu_gridding_tune(ctypes.byref(d), kspace.data_ptr(), traj.data_ptr(),
                                           dcf.data_ptr() if dcf is not None else None, out.data_ptr(),
                                           workspace.data_ptr(), workspace.numel(), _stream(stream),
                                           ctypes.byref(t)), "gridding_tune")
        return t


class Gridding3Desc(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("image", ctypes.c_uint32), ("grid", ctypes.c_uint32),
                ("kernel_width", ctypes.c_uint32), ("kb_beta", ctypes.c_double), ("channels", ctypes.c_uint32),
                ("samples", ctypes.c_uint32), ("dcf_mode", ctypes.c_uint32), ("output", ctypes.c_uint32),
                ("sample_format", ctypes.c_uint32), ("reserved0", ctypes.c_uint32)]


@dataclass
class Gridding3:
    """3-D Kaiser-Bessel adjoint gridding (see ``ksj_gpu_gridding3_desc``)."""

    image: int
    grid: int
    channels: int
    samples: int
    width: int = 4
    beta: float = 0.0
    dcf: int = DCF_NONE
    output: int = OUTPUT_RSS
    sample_format: int = SAMPLES_CF32

    def desc(self) -> Gridding3Desc:
        return Gridding3Desc(ctypes.sizeof(Gridding3Desc), self.image, self.grid, self.width, self.beta,
                             self.channels, self.samples, self.dcf, self.output, self.sample_format, 0)

    def workspace_bytes(self) -> int:
        d = self.desc()
        n = lib().ksj_gpu_gridding3_workspace_bytes(ctypes.byref(d))
        if n == 0:
            raise GpuError(1, "gridding3_workspace_bytes")
        return int(n)

    def output_shape(self) -> tuple[int, ...]:
        n = self.image
        return (n, n, n) if self.output == OUTPUT_RSS else (n, n, n, self.channels)

    def new_output(self, device="cuda") -> torch.Tensor:
        dt = torch.float32 if self.output == OUTPUT_RSS else torch.complex64
        return torch.empty(self.output_shape(), dtype=dt, device=device)

    def new_workspace(self, device="cuda") -> torch.Tensor:
        return torch.empty(self.workspace_bytes(), dtype=torch.uint8, device=device)

    def run(self, kspace: torch.Tensor, traj: torch.Tensor, out: torch.Tensor, workspace: torch.Tensor,
            dcf: torch.Tensor | None = None, tuning: GriddingTuning | None = None, stream=None) -> None:
        d = self.desc()
        st = lib().ksj_gpu_gridding3_adjoint(ctypes.byref(d), ctypes.byref(tuning) if tuning else None,
                                             kspace.data_ptr(), traj.data_ptr(),
                                             dcf.data_ptr() if dcf is not None else None, out.data_ptr(),
                                             workspace.data_ptr(), workspace.numel(), _stream(stream))
        _check(st, "gridding3_adjoint")


def kb_gridding(image: int, grid: int, channels: int, samples: int, frames: int = 1, width: int = 4,
                output: int = OUTPUT_RSS, dcf: int = DCF_ANALYTIC_RAMP, sample_format: int = SAMPLES_CF32) -> Gridding:
    """Kaiser-Bessel shape: square image and grid, beta from Beatty et al. 2005."""
    return Gridding(image=(image, image), channels=channels, samples=samples, frames=frames,
                    kernel=KERNEL_KAISER_BESSEL, grid=(grid, grid), width=width, dcf=dcf, output=output,
                    sample_format=sample_format, require_nyquist=False)


def pipe_menon_dcf(traj: torch.Tensor, image: int, grid: int, width: int = 4, iterations: int = 10,
                   stream=None) -> torch.Tensor:
    """Pipe-Menon density weights for Kaiser-Bessel gridding on a square grid:
    traj [F, M, 2] (or [M, 2]) float32 on the GPU -> float32 [F, M] (or [M])."""
    t = traj if traj.dim() == 3 else traj.unsqueeze(0)
    f, m, _ = t.shape
    g = kb_gridding(image, grid, 1, m, frames=f, width=width)
    d = g.desc()
    L = lib()
    n = int(L.ksj_gpu_pipe_menon_workspace_bytes(ctypes.byref(d)))
    if n == 0:
        raise GpuError(1, "pipe_menon_workspace_bytes")
    ws = torch.empty(n, dtype=torch.uint8, device=t.device)
    out = torch.empty((f, m), dtype=torch.float32, device=t.device)
    _check(L.ksj_gpu_pipe_menon_dcf(ctypes.byref(d), iterations, t.contiguous().data_ptr(), out.data_ptr(),
                                    ws.data_ptr(), ws.numel(), _stream(stream)), "pipe_menon_dcf")
    return out if traj.dim() == 3 else out[0]


def pipe_menon_dcf3(traj: torch.Tensor, image: int, grid: int, width: int = 4, iterations: int = 10,
                    stream=None) -> torch.Tensor:
    """3-D Pipe-Menon weights: traj [M, 3] float32 on the GPU -> float32 [M]."""
    m = traj.shape[0]
    d = Gridding3(image=image, grid=grid, channels=1, samples=m, width=width).desc()
    L = lib()
    n = int(L.ksj_gpu_pipe_menon3_workspace_bytes(ctypes.byref(d)))
    if n == 0:
        raise GpuError(1, "pipe_menon3_workspace_bytes")
    ws = torch.empty(n, dtype=torch.uint8, device=traj.device)
    out = torch.empty(m, dtype=torch.float32, device=traj.device)
    _check(L.ksj_gpu_pipe_menon_dcf3(ctypes.byref(d), iterations, traj.contiguous().data_ptr(), out.data_ptr(),
                                     ws.data_ptr(), ws.numel(), _stream(stream)), "pipe_menon_dcf3")
    return out


def direct_adjoint(kspace: torch.Tensor, traj: torch.Tensor, rows: int, cols: int,
                   origin: tuple[float, float] | None = None, stream=None) -> torch.Tensor:
    """Exact direct NUDFT adjoint: kspace [C, M] complex64, traj [M, 2] -> [rows, cols, C]."""
    c, m = kspace.shape
    ro, co = origin if origin is not None else ((rows - 1) / 2.0, (cols - 1) / 2.0)
    L = lib()
    ws = torch.empty(L.ksj_gpu_direct_workspace_bytes(rows, cols, c), dtype=torch.uint8, device=kspace.device)
    out = torch.empty((rows, cols, c), dtype=torch.complex64, device=kspace.device)
    _check(L.ksj_gpu_direct_adjoint(rows, cols, ro, co, c, m, kspace.data_ptr(), traj.data_ptr(), out.data_ptr(),
                                    ws.data_ptr(), ws.numel(), _stream(stream)), "direct_adjoint")
    return out


def direct_forward(image: torch.Tensor, traj: torch.Tensor, origin: tuple[float, float] | None = None,
                   stream=None) -> torch.Tensor:
    """Exact direct NUDFT forward: image [rows, cols, C] complex64 (coil-last), traj [M, 2] -> [C, M]."""
    rows, cols, c = image.shape
    m = traj.shape[0]
    ro, co = origin if origin is not None else ((rows - 1) / 2.0, (cols - 1) / 2.0)
    out = torch.empty((c, m), dtype=torch.complex64, device=image.device)
    _check(lib().ksj_gpu_direct_forward(rows, cols, ro, co, c, m, image.contiguous().data_ptr(),
                                        traj.contiguous().data_ptr(), out.data_ptr(), _stream(stream)),
           "direct_forward")
    return out


TRAJ_CYCLES_PER_FOV, TRAJ_RADIANS_PER_PIXEL, TRAJ_ENCODED_MATRIX_INDEX = 1, 2, 3


def normalize_trajectory(raw: torch.Tensor, units: int, encoded: tuple[int, int] = (0, 0),
                         stream=None) -> tuple[torch.Tensor, int]:
    """ISMRMRD [M, 2] (kx, ky) float32 on the GPU -> ([M, 2] (row = ky, column = kx) radians per pixel, flags)."""
    m = raw.shape[0]
    out = torch.empty((m, 2), dtype=torch.float32, device=raw.device)
    flags = torch.zeros(1, dtype=torch.int32, device=raw.device)
    _check(lib().ksj_gpu_normalize_trajectory(m, units, encoded[0], encoded[1], raw.contiguous().data_ptr(),
                                              out.data_ptr(), flags.data_ptr(), _stream(stream)),
           "normalize_trajectory")
    return out, int(flags.item())


def aggregate_acquisitions(blocks: torch.Tensor, stream=None) -> torch.Tensor:
    """Per-acquisition channel-major blocks [A, C, n] complex64 -> one channel-major frame [C, A * n]."""
    a, c, n = blocks.shape
    out = torch.empty((c, a * n), dtype=torch.complex64, device=blocks.device)
    _check(lib().ksj_gpu_aggregate_acquisitions(a, c, n, blocks.contiguous().data_ptr(), out.data_ptr(),
                                                _stream(stream)), "aggregate_acquisitions")
    return out


def cartesian_ifft2(kspace: torch.Tensor, output: int = OUTPUT_COIL_LAST, stream=None) -> torch.Tensor:
    """cartesian_ifft2_coil_images: kspace [F, C, rows, cols] (or [C, rows, cols]) complex64 channel-major ->
    coil-last images [F, rows, cols, C] complex64, or RSS [F, rows, cols] float32 (leading F dropped if absent)."""
    k = kspace if kspace.dim() == 4 else kspace.unsqueeze(0)
    f, c, rows, cols = k.shape
    L = lib()
    n = int(L.ksj_gpu_cartesian_workspace_bytes(rows, cols, c, f))
    if n == 0:
        raise GpuError(1, "cartesian_workspace_bytes")
    ws = torch.empty(n, dtype=torch.uint8, device=k.device)
    if output == OUTPUT_RSS:
        out = torch.empty((f, rows, cols), dtype=torch.float32, device=k.device)
    else:
        out = torch.empty((f, rows, cols, c), dtype=torch.complex64, device=k.device)
    _check(L.ksj_gpu_cartesian_ifft2(rows, cols, c, f, output, k.contiguous().data_ptr(), out.data_ptr(),
                                     ws.data_ptr(), ws.numel(), _stream(stream)), "cartesian_ifft2")
    return out if kspace.dim() == 4 else out[0]


def walsh_combine(coil_last: torch.Tensor, window: int = 7, iterations: int = 24, stream=None) -> torch.Tensor:
    """[rows, cols, C] complex64 (C <= 8) -> [rows, cols] complex64 adaptive combination."""
    rows, cols, c = coil_last.shape
    out = torch.empty((rows, cols), dtype=torch.complex64, device=coil_last.device)
    _check(lib().ksj_gpu_walsh_combine(rows, cols, c, window, iterations, coil_last.contiguous().data_ptr(),
                                       out.data_ptr(), _stream(stream)), "walsh_combine")
    return out


def coil_covariance(kspace: torch.Tensor, stream=None) -> torch.Tensor:
    """[C, M] complex64 channel-major k-space -> [C, C] complex64 covariance (tensor cores)."""
    c, m = kspace.shape
    L = lib()
    n = int(L.ksj_gpu_coil_covariance_workspace_bytes(c, m))
    if n == 0:
        raise GpuError(1, "coil_covariance_workspace_bytes")
    ws = torch.empty(n, dtype=torch.uint8, device=kspace.device)
    out = torch.empty((c, c), dtype=torch.complex64, device=kspace.device)
    _check(L.ksj_gpu_coil_covariance(c, m, kspace.contiguous().data_ptr(), out.data_ptr(), ws.data_ptr(), ws.numel(),
                                     _stream(stream)), "coil_covariance")
    return out


def compression_basis(covariance, virtual_channels: int):
    """Host: covariance [C, C] complex64 (numpy) -> (basis [V, C] complex64, eigenvalues [C] float32)."""
    import numpy as np

    cov = np.ascontiguousarray(covariance, dtype=np.complex64)
    c = cov.shape[0]
    basis = np.zeros((virtual_channels, c), dtype=np.complex64)
    ev = np.zeros(c, dtype=np.float32)
    _check(lib().ksj_coil_compression_basis(c, virtual_channels, cov.ctypes.data, basis.ctypes.data, ev.ctypes.data),
           "compression_basis")
    return basis, ev


def coil_compress(basis: torch.Tensor, kspace: torch.Tensor, stream=None) -> torch.Tensor:
    """basis [V, C], kspace [C, M] complex64 on the GPU -> [V, M]."""
    v, c = basis.shape
    _, m = kspace.shape
    out = torch.empty((v, m), dtype=torch.complex64, device=kspace.device)
    _check(lib().ksj_gpu_coil_compress(c, v, m, basis.contiguous().data_ptr(), kspace.contiguous().data_ptr(),
                                       out.data_ptr(), _stream(stream)), "coil_compress")
    return out


NOISE_EIGENVALUE_FLOOR = 1.0e-6  # noise_model_estimate.cpp:38


def noise_covariance(noise: torch.Tensor, stream=None) -> torch.Tensor:
    """[C, M] complex64 channel-major noise samples -> [C, C] complex64 noise
    covariance (means removed, 1/M, conj on the row index as the reference
    forms it); the product sums on the tensor cores."""
    c, m = noise.shape
    L = lib()
    n = int(L.ksj_gpu_coil_covariance_workspace_bytes(c, m))
    if n == 0:
        raise GpuError(1, "noise_covariance workspace")
    ws = torch.empty(n, dtype=torch.uint8, device=noise.device)
    out = torch.empty((c, c), dtype=torch.complex64, device=noise.device)
    _check(L.ksj_gpu_noise_covariance(c, m, noise.contiguous().data_ptr(), out.data_ptr(), ws.data_ptr(), ws.numel(),
                                      _stream(stream)), "noise_covariance")
    return out


def whitening_matrix(covariance, floor: float = NOISE_EIGENVALUE_FLOOR):
    """Host: noise covariance [C, C] complex64 (numpy) -> whitening matrix
    W = V diag(1/sqrt(max(lambda, floor))) V^H, [C, C] complex64."""
    import numpy as np

    cov = np.ascontiguousarray(covariance, dtype=np.complex64)
    w = np.zeros_like(cov)
    _check(lib().ksj_whitening_matrix(cov.shape[0], cov.ctypes.data, floor, w.ctypes.data), "whitening_matrix")
    return w


def noise_model(noise: torch.Tensor, stream=None) -> torch.Tensor:
    """noise_model_estimate: [C, M] noise samples -> the [C, C] whitening
    matrix on the same device (covariance on the GPU, eigensolve on the host)."""
    cov = noise_covariance(noise, stream).cpu().numpy()
    return torch.from_numpy(whitening_matrix(cov)).to(noise.device)


def noise_prewhiten(whitening: torch.Tensor, kspace: torch.Tensor, stream=None) -> torch.Tensor:
    """noncartesian_noise_prewhiten: W [C, C], kspace [C, M] complex64 -> W kspace."""
    c, m = kspace.shape
    if tuple(whitening.shape) != (c, c):
        raise GpuError(1, "noise_prewhiten: whitening must be [C, C]")
    out = torch.empty((c, m), dtype=torch.complex64, device=kspace.device)
    _check(lib().ksj_gpu_noise_prewhiten(c, m, whitening.contiguous().data_ptr(), kspace.contiguous().data_ptr(),
                                         out.data_ptr(), _stream(stream)), "noise_prewhiten")
    return out


def rss_coil_last(coil_last: torch.Tensor, stream=None) -> torch.Tensor:
    """[..., C] complex64 -> [...] float32 root sum of squares."""
    c = coil_last.shape[-1]
    p = coil_last.numel() // c
    out = torch.empty(coil_last.shape[:-1], dtype=torch.float32, device=coil_last.device)
    _check(lib().ksj_gpu_rss_coil_last(p, c, coil_last.data_ptr(), out.data_ptr(), _stream(stream)), "rss")
    return out


def kb_beta(width: int, sigma: float) -> float:
    a = (width / sigma) * (sigma - 0.5)
    return math.pi * math.sqrt(a * a - 0.8)
