"""CPU restatement of the adaptive (Walsh) coil combination.  TEST
INFRASTRUCTURE ONLY: the parity checker for ksj_gpu_walsh_combine; the
product never imports it.

Walsh, Gmitro and Marcellin, MRM 43:682-690, 2000, with the noise covariance
taken as the identity: per pixel, R = sum over the window (clipped at the
image border) of x x^H, v = the eigenvector of R's largest eigenvalue
(numpy.linalg.eigh, double precision), phase-referenced so that v[0] is real
and non-negative, and the combined value v^H x.  No reference counterpart
(the reference's adaptive combine is a planned interface); parity unpinned.
"""
import numpy as np


def walsh_combine(coil_last: np.ndarray, window: int = 7) -> tuple[np.ndarray, np.ndarray]:
    """coil_last [rows, cols, C] -> (combined [rows, cols] complex128, eigen gap
    lambda_2 / lambda_1 per pixel)."""
    x = np.asarray(coil_last, dtype=np.complex128)
    rows, cols, c = x.shape
    h = window // 2
    outer = x[:, :, :, None] * np.conj(x[:, :, None, :])  # x_i conj(x_j)
    pad = np.zeros((rows + 2 * h, cols + 2 * h, c, c), dtype=np.complex128)
    pad[h:h + rows, h:h + cols] = outer
    cum = pad.cumsum(axis=0).cumsum(axis=1)
    cum = np.pad(cum, ((1, 0), (1, 0), (0, 0), (0, 0)))
    w = window
    R = cum[w:w + rows, w:w + cols] - cum[:rows, w:w + cols] - cum[w:w + rows, :cols] + cum[:rows, :cols]
    vals, vecs = np.linalg.eigh(R)
    v = vecs[:, :, :, -1]
    ref = v[:, :, 0]
    mag = np.abs(ref)
    ph = np.where(mag > 0, np.conj(ref) / np.where(mag > 0, mag, 1.0), 1.0)
    v = v * ph[:, :, None]
    out = np.sum(np.conj(v) * x, axis=2)
    gap = vals[:, :, -2] / np.maximum(vals[:, :, -1], 1e-300) if c > 1 else np.zeros((rows, cols))
    return out, gap
