"""CPU restatement of the ISMRMRD radial ingress conversions.  TEST
INFRASTRUCTURE ONLY: the parity checker for ksj_gpu_normalize_trajectory
and ksj_gpu_aggregate_acquisitions; the product never imports it.

libs/recon/kspacejet-recon-runtime/src/noncartesian_rss_hdf5.cpp:
* normalize_radial_coordinate (:776-811): finite, inside the unit's
  inclusive Nyquist interval (cycles per FOV 0.5, radians per pixel pi,
  encoded matrix index encoded / 2), then one float multiply by 2 pi, 1 or
  2 pi / encoded (factors formed in float as there);
* normalize_radial_coordinate_pair (:822-833): raw [kx, ky] -> [row = ky,
  column = kx], each axis with its own encoded dimension;
* the channel-major aggregation (:1077-1083).
"""
import numpy as np

CYCLES_PER_FOV, RADIANS_PER_PIXEL, ENCODED_MATRIX_INDEX = 1, 2, 3
PI_F = np.float32(np.pi)


def _axis(units: int, encoded: int):
    two_pi = np.float32(np.float32(2.0) * PI_F)
    if units == CYCLES_PER_FOV:
        return np.float32(0.5), two_pi
    if units == RADIANS_PER_PIXEL:
        return PI_F, np.float32(1.0)
    if units == ENCODED_MATRIX_INDEX:
        if encoded < 2:
            raise ValueError("encoded dimension >= 2 required")
        return np.float32(np.float32(encoded) / np.float32(2.0)), np.float32(two_pi / np.float32(encoded))
    raise ValueError("unspecified trajectory units")


def normalize_trajectory(raw: np.ndarray, units: int, encoded_rows: int = 0, encoded_cols: int = 0):
    """[M, 2] (kx, ky) -> ([M, 2] (row, column) float32, per-sample validity)."""
    raw = np.asarray(raw, dtype=np.float32)
    row_limit, row_scale = _axis(units, encoded_rows)
    col_limit, col_scale = _axis(units, encoded_cols)
    kx, ky = raw[:, 0], raw[:, 1]
    ok = np.isfinite(kx) & np.isfinite(ky) & (np.abs(kx) <= col_limit) & (np.abs(ky) <= row_limit)
    with np.errstate(invalid="ignore", over="ignore"):
        out = np.stack([(ky * row_scale).astype(np.float32), (kx * col_scale).astype(np.float32)], axis=1)
    return out, ok


def aggregate_acquisitions(blocks: np.ndarray) -> np.ndarray:
    """[A, C, n] -> [C, A * n]."""
    a, c, n = blocks.shape
    return np.ascontiguousarray(np.moveaxis(blocks, 1, 0).reshape(c, a * n))
