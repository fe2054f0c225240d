"""CPU oracle for the non-Cartesian reconstruction path -- TEST INFRASTRUCTURE.

This package is the parity checker, never the thing measured or shipped.
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import it.  The product package ``kspacejet_gb300`` has no import
path to it and fails loudly when its CUDA library is missing.

Two back ends, same signatures:

* ``Oracle`` wraps ``ksj_oracle.c``, the C restatement of the reference's
  arithmetic (built on any host by ``oracle/build.py``);
* ``Reference`` wraps ``oracle/_ref/libksj_ref.so``, the reference's own
  sources compiled where the reference tree exists.  It pins the restatement.

Arrays are numpy: complex samples as complex64/complex128 ``[M]``,
trajectories ``[M, 2]`` float32/float64 in radians per pixel ordered
``(k_row, k_col)``, images ``[rows, cols]``.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import build as _build

_i64 = ctypes.c_int64
_dbl = ctypes.c_double
_ptr = ctypes.c_void_p


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


class OracleError(RuntimeError):
    """The restated function rejected its input where the reference throws."""


class _Base:
    _lib: ctypes.CDLL
    _prefix: str

    def _fn(self, name: str, restype, argtypes):
        f = getattr(self._lib, self._prefix + name)
        f.restype = restype
        f.argtypes = argtypes
        return f

    # --- radial_analytic_ramp_dcf2 -------------------------------------------------
    def ramp_dcf(self, traj: np.ndarray) -> np.ndarray:
        traj = np.ascontiguousarray(traj)
        f64 = traj.dtype == np.float64
        out = np.zeros(traj.shape[0], dtype=traj.dtype)
        fn = self._fn("ramp_dcf2_f64" if f64 else "ramp_dcf2_f32", ctypes.c_int, [_ptr, _i64, _ptr])
        if fn(_p(traj), traj.shape[0], _p(out)) != 0:
            raise OracleError("ramp DCF rejected the trajectory")
        return out

    # --- radial_linear_gridding2_adjoint ------------------------------------------
    def linear_gridding(self, rows: int, cols: int, samples: np.ndarray, traj: np.ndarray, dcf: np.ndarray,
                        row_origin: float | None = None, col_origin: float | None = None,
                        exact: bool = False) -> np.ndarray:
        f64 = samples.dtype == np.complex128
        rdt = np.float64 if f64 else np.float32
        samples = np.ascontiguousarray(samples)
        traj = np.ascontiguousarray(traj, dtype=rdt)
        dcf = np.ascontiguousarray(dcf, dtype=rdt)
        ro = (rows - 1) / 2.0 if row_origin is None else row_origin
        co = (cols - 1) / 2.0 if col_origin is None else col_origin
        out = np.zeros((rows, cols), dtype=samples.dtype)
        args = [_i64, _i64, _dbl, _dbl, _ptr, _ptr, _ptr, _i64, _ptr]
        if f64 and isinstance(self, Oracle):
            fn = self._fn("linear_gridding2_adjoint_f64", ctypes.c_int, args + [ctypes.c_int])
            rc = fn(rows, cols, ro, co, _p(samples), _p(traj), _p(dcf), samples.shape[0], _p(out), int(exact))
        else:
            if exact:
                raise ValueError("exact transforms exist only in the restatement")
            fn = self._fn("linear_gridding2_adjoint_f64" if f64 else "linear_gridding2_adjoint_f32",
                          ctypes.c_int, args)
            rc = fn(rows, cols, ro, co, _p(samples), _p(traj), _p(dcf), samples.shape[0], _p(out))
        if rc != 0:
            raise OracleError("linear gridding rejected its input")
        return out

    # --- direct_nudft2_adjoint ------------------------------------------------------
    def direct_adjoint(self, rows: int, cols: int, samples: np.ndarray, traj: np.ndarray,
                       row_origin: float | None = None, col_origin: float | None = None) -> np.ndarray:
        f64 = samples.dtype == np.complex128
        rdt = np.float64 if f64 else np.float32
        samples = np.ascontiguousarray(samples)
        traj = np.ascontiguousarray(traj, dtype=rdt)
        ro = (rows - 1) / 2.0 if row_origin is None else row_origin
        co = (cols - 1) / 2.0 if col_origin is None else col_origin
        out = np.zeros((rows, cols), dtype=samples.dtype)
        fn = self._fn("direct_nudft2_adjoint_f64" if f64 else "direct_nudft2_adjoint_f32",
                      None if isinstance(self, Oracle) else ctypes.c_int,
                      [_i64, _i64, _dbl, _dbl, _ptr, _ptr, _i64, _ptr])
        fn(rows, cols, ro, co, _p(samples), _p(traj), samples.shape[0], _p(out))
        return out


class Oracle(_Base):
    """The C restatement (``ksj_oracle.c``)."""

    def __init__(self, path: str | Path | None = None):
        lib = Path(path) if path else _build.build_oracle()
        self._lib = ctypes.CDLL(str(lib))
        self._prefix = "ksjo_"

    def grid_coordinate(self, f: float, extent: int, f64: bool = False) -> tuple[int, float]:
        lo = ctypes.c_int64()
        if f64:
            fr = ctypes.c_double()
            fn = self._fn("grid_coordinate_f64", ctypes.c_int,
                          [ctypes.c_double, _i64, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double)])
        else:
            fr = ctypes.c_float()
            fn = self._fn("grid_coordinate_f32", ctypes.c_int,
                          [ctypes.c_float, _i64, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_float)])
        if fn(f, extent, ctypes.byref(lo), ctypes.byref(fr)) != 0:
            raise OracleError("coordinate cannot be mapped")
        return lo.value, fr.value

    def linear_grid_only(self, rows: int, cols: int, samples: np.ndarray, traj: np.ndarray, dcf: np.ndarray,
                         row_origin: float | None = None, col_origin: float | None = None) -> np.ndarray:
        """The scatter stage alone (gridded k-space before the transform)."""
        f64 = samples.dtype == np.complex128
        rdt = np.float64 if f64 else np.float32
        samples = np.ascontiguousarray(samples)
        traj = np.ascontiguousarray(traj, dtype=rdt)
        dcf = np.ascontiguousarray(dcf, dtype=rdt)
        ro = (rows - 1) / 2.0 if row_origin is None else row_origin
        co = (cols - 1) / 2.0 if col_origin is None else col_origin
        out = np.zeros((rows, cols), dtype=samples.dtype)
        fn = self._fn("linear_grid2_f64" if f64 else "linear_grid2_f32", ctypes.c_int,
                      [_i64, _i64, _dbl, _dbl, _ptr, _ptr, _ptr, _i64, _ptr])
        if fn(rows, cols, ro, co, _p(samples), _p(traj), _p(dcf), samples.shape[0], _p(out)) != 0:
            raise OracleError("linear gridding rejected its input")
        return out

    def inverse_transform(self, line: np.ndarray) -> np.ndarray:
        line = np.ascontiguousarray(line)
        f64 = line.dtype == np.complex128
        out = np.zeros_like(line)
        fn = self._fn("inverse_transform_f64" if f64 else "inverse_transform_f32", None, [_ptr, _ptr, _i64])
        fn(_p(line), _p(out), line.shape[0])
        return out

    def direct_forward(self, rows: int, cols: int, image: np.ndarray, traj: np.ndarray,
                       row_origin: float | None = None, col_origin: float | None = None) -> np.ndarray:
        image = np.ascontiguousarray(image, dtype=np.complex128)
        traj = np.ascontiguousarray(traj, dtype=np.float64)
        ro = (rows - 1) / 2.0 if row_origin is None else row_origin
        co = (cols - 1) / 2.0 if col_origin is None else col_origin
        out = np.zeros(traj.shape[0], dtype=np.complex128)
        fn = self._fn("direct_nudft2_forward_f64", None, [_i64, _i64, _dbl, _dbl, _ptr, _ptr, _i64, _ptr])
        fn(rows, cols, ro, co, _p(image), _p(traj), traj.shape[0], _p(out))
        return out

    def rss(self, coil_last: np.ndarray) -> np.ndarray:
        """``coil_last`` complex64 ``[..., C]`` -> float32 ``[...]``."""
        x = np.ascontiguousarray(coil_last, dtype=np.complex64)
        c = x.shape[-1]
        p = x.size // c
        out = np.zeros(x.shape[:-1], dtype=np.float32)
        fn = self._fn("rss_f32", None, [_ptr, _i64, _i64, _ptr])
        fn(_p(x), p, c, _p(out))
        return out

    def kb_beta(self, width: int, sigma: float) -> float:
        return self._fn("kb_beta", ctypes.c_double, [ctypes.c_int, ctypes.c_double])(width, sigma)

    def kb_kernel(self, d: float, width: int, beta: float) -> float:
        return self._fn("kb_kernel", ctypes.c_double, [ctypes.c_double, ctypes.c_int, ctypes.c_double])(d, width, beta)

    def kb_deapod(self, x: float, width: int, beta: float, g: int) -> float:
        return self._fn("kb_deapod", ctypes.c_double,
                        [ctypes.c_double, ctypes.c_int, ctypes.c_double, _i64])(x, width, beta, g)

    def direct_adjoint_at(self, pixels: np.ndarray, samples: np.ndarray, traj: np.ndarray, row_origin: float,
                          col_origin: float) -> np.ndarray:
        """The exact FP64 direct adjoint NUDFT at the (row, col) pairs `pixels` [P, 2] only."""
        pixels = np.ascontiguousarray(pixels, dtype=np.int64).reshape(-1, 2)
        samples = np.ascontiguousarray(samples, dtype=np.complex128)
        traj = np.ascontiguousarray(traj, dtype=np.float64).reshape(-1, 2)
        out = np.zeros(pixels.shape[0], dtype=np.complex128)
        self._fn("direct_nudft2_adjoint_at_f64", None, [_i64, _ptr, _dbl, _dbl, _ptr, _ptr, _i64, _ptr])(
            pixels.shape[0], _p(pixels), row_origin, col_origin, _p(samples), _p(traj), samples.shape[0], _p(out))
        return out

    def kb_gridding(self, grid: int, n: int, samples: np.ndarray, traj: np.ndarray, dcf: np.ndarray | None,
                    width: int = 4, sigma: float | None = None, beta: float | None = None,
                    row_origin: float | None = None, col_origin: float | None = None) -> np.ndarray:
        """Kaiser-Bessel gridding adjoint in double precision (one coil)."""
        samples = np.ascontiguousarray(samples, dtype=np.complex128)
        traj = np.ascontiguousarray(traj, dtype=np.float64)
        if beta is None:
            beta = self.kb_beta(width, sigma if sigma is not None else grid / n)
        ro = (n - 1) / 2.0 if row_origin is None else row_origin
        co = (n - 1) / 2.0 if col_origin is None else col_origin
        d = None if dcf is None else np.ascontiguousarray(dcf, dtype=np.float64)
        out = np.zeros((n, n), dtype=np.complex128)
        fn = self._fn("kb_gridding2_adjoint_f64", ctypes.c_int,
                      [_i64, _i64, ctypes.c_int, _dbl, _dbl, _dbl, _ptr, _ptr, _ptr, _i64, _ptr])
        rc = fn(grid, n, width, beta, ro, co, _p(samples), _p(traj), None if d is None else _p(d),
                samples.shape[0], _p(out))
        if rc != 0:
            raise OracleError("KB gridding rejected its configuration")
        return out


    def kb_gridding_f32(self, grid: int, n: int, samples: np.ndarray, traj: np.ndarray, dcf: np.ndarray | None,
                        width: int = 4, sigma: float | None = None, beta: float | None = None) -> np.ndarray:
        """The same Kaiser-Bessel reconstruction as a single-precision CPU program with an FFT (one coil,
        origin (n-1)/2): the timed CPU baseline of the KB forms, not a parity target."""
        samples = np.ascontiguousarray(samples, dtype=np.complex64)
        traj = np.ascontiguousarray(traj, dtype=np.float32)
        if beta is None:
            beta = self.kb_beta(width, sigma if sigma is not None else grid / n)
        d = None if dcf is None else np.ascontiguousarray(dcf, dtype=np.float32)
        out = np.zeros((n, n), dtype=np.complex64)
        fn = self._fn("kb_gridding2_adjoint_f32", ctypes.c_int,
                      [_i64, _i64, ctypes.c_int, _dbl, _dbl, _dbl, _ptr, _ptr, _ptr, _i64, _ptr])
        rc = fn(grid, n, width, beta, (n - 1) / 2.0, (n - 1) / 2.0, _p(samples), _p(traj),
                None if d is None else _p(d), samples.shape[0], _p(out))
        if rc != 0:
            raise OracleError("single-precision KB gridding rejected its configuration")
        return out

    def kb_forward(self, grid: int, n: int, image: np.ndarray, traj: np.ndarray, width: int = 4,
                   sigma: float | None = None, beta: float | None = None) -> np.ndarray:
        """Kaiser-Bessel forward in double precision (one coil, origin (n-1)/2): the exact transpose of
        kb_gridding without density weights."""
        image = np.ascontiguousarray(image, dtype=np.complex128)
        traj = np.ascontiguousarray(traj, dtype=np.float64)
        if beta is None:
            beta = self.kb_beta(width, sigma if sigma is not None else grid / n)
        out = np.zeros(traj.shape[0], dtype=np.complex128)
        fn = self._fn("kb_forward2_f64", ctypes.c_int,
                      [_i64, _i64, ctypes.c_int, _dbl, _dbl, _dbl, _ptr, _ptr, _i64, _ptr])
        rc = fn(grid, n, width, beta, (n - 1) / 2.0, (n - 1) / 2.0, _p(image), _p(traj), traj.shape[0], _p(out))
        if rc != 0:
            raise OracleError("KB forward rejected its configuration")
        return out

    def pipe_menon_dcf(self, traj: np.ndarray, grid_rows: int, grid_cols: int, width: int = 4,
                       beta: float | None = None, sigma: float = 2.0, iterations: int = 10) -> np.ndarray:
        """Pipe-Menon density compensation, grid-based, double precision (one frame)."""
        traj = np.ascontiguousarray(traj, dtype=np.float32).reshape(-1, 2)
        if beta is None:
            beta = self.kb_beta(width, sigma)
        out = np.zeros(traj.shape[0], dtype=np.float64)
        fn = self._fn("pipe_menon_dcf2_f64", ctypes.c_int, [_i64, _i64, ctypes.c_int, _dbl, _ptr, _i64, ctypes.c_int, _ptr])
        if fn(grid_rows, grid_cols, width, beta, _p(traj), traj.shape[0], iterations, _p(out)) != 0:
            raise OracleError("Pipe-Menon rejected its configuration")
        return out


    def kb_gridding3(self, grid: int, n: int, samples: np.ndarray, traj: np.ndarray, dcf: np.ndarray | None,
                     width: int = 4, sigma: float | None = None, beta: float | None = None) -> np.ndarray:
        """3-D Kaiser-Bessel gridding adjoint in double precision (one coil), origin (n-1)/2."""
        samples = np.ascontiguousarray(samples, dtype=np.complex128)
        traj = np.ascontiguousarray(traj, dtype=np.float64).reshape(-1, 3)
        if beta is None:
            beta = self.kb_beta(width, sigma if sigma is not None else grid / n)
        d = None if dcf is None else np.ascontiguousarray(dcf, dtype=np.float64)
        out = np.zeros((n, n, n), dtype=np.complex128)
        fn = self._fn("kb_gridding3_adjoint_f64", ctypes.c_int,
                      [_i64, _i64, ctypes.c_int, _dbl, _dbl, _ptr, _ptr, _ptr, _i64, _ptr])
        if fn(grid, n, width, beta, (n - 1) / 2.0, _p(samples), _p(traj), None if d is None else _p(d),
              samples.shape[0], _p(out)) != 0:
            raise OracleError("3-D KB gridding rejected its configuration")
        return out

    def direct_adjoint3(self, n: int, samples: np.ndarray, traj: np.ndarray) -> np.ndarray:
        samples = np.ascontiguousarray(samples, dtype=np.complex128)
        traj = np.ascontiguousarray(traj, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((n, n, n), dtype=np.complex128)
        self._fn("direct_nudft3_adjoint_f64", None, [_i64, _dbl, _ptr, _ptr, _i64, _ptr])(
            n, (n - 1) / 2.0, _p(samples), _p(traj), samples.shape[0], _p(out))
        return out

    def pipe_menon_dcf3(self, traj: np.ndarray, grid: int, width: int = 4, beta: float | None = None,
                        sigma: float = 1.5, iterations: int = 10) -> np.ndarray:
        """3-D Pipe-Menon density compensation, grid-based, double precision."""
        traj = np.ascontiguousarray(traj, dtype=np.float32).reshape(-1, 3)
        if beta is None:
            beta = self.kb_beta(width, sigma)
        out = np.zeros(traj.shape[0], dtype=np.float64)
        fn = self._fn("pipe_menon_dcf3_f64", ctypes.c_int, [_i64, ctypes.c_int, _dbl, _ptr, _i64, ctypes.c_int, _ptr])
        if fn(grid, width, beta, _p(traj), traj.shape[0], iterations, _p(out)) != 0:
            raise OracleError("3-D Pipe-Menon rejected its configuration")
        return out

    def coil_covariance(self, x: np.ndarray, double: bool = False) -> np.ndarray:
        """Coil covariance of channel-major k-space x complex64 [C, M]: the
        reference's float arithmetic, or double precision."""
        x = np.ascontiguousarray(x, dtype=np.complex64)
        c, m = x.shape
        out = np.zeros((c, c), dtype=np.complex128 if double else np.complex64)
        name = "coil_covariance_f64" if double else "coil_covariance_f32"
        self._fn(name, None, [_i64, _i64, _ptr, _ptr])(c, m, _p(x), _p(out))
        return out


class Reference(_Base):
    """The reference's own numerics compiled from its sources (``oracle/_ref``).
    Raises ``FileNotFoundError`` where the reference was not built."""

    def __init__(self, path: str | Path | None = None):
        lib = Path(path) if path else _build.REF_NUMERICS_LIB
        if not lib.exists():
            raise FileNotFoundError(f"reference numerics not built: {lib}")
        self._lib = ctypes.CDLL(str(lib))
        self._prefix = "ksjr_"


def reference_available() -> bool:
    return _build.REF_NUMERICS_LIB.exists()


def rel_l2(x: np.ndarray, ref: np.ndarray) -> float:
    """||x - ref||_2 / ||ref||_2 over all elements, in double precision."""
    x = np.asarray(x, dtype=np.complex128)
    ref = np.asarray(ref, dtype=np.complex128)
    den = np.linalg.norm(ref.ravel())
    num = np.linalg.norm((x - ref).ravel())
    return float(num / den) if den > 0 else float(num)
