"""The reference binning permutation, restated in numpy (test helper).

A sample's lower tap index is floor(k * G / (2 pi)) of its exact coordinate,
as the reference's double-precision grid_coordinate computes it
(eigen_radial_gridding.cpp:262-277); the linear stencil starts there, the
W-tap Kaiser-Bessel stencil W/2 - 1 cells earlier.  A list is (frame, grid
row, 32-column chunk); it holds, in increasing order, every sample whose
stencil covers that row and has a column in that chunk.
"""
import math

import numpy as np


def binning(traj: np.ndarray, grid_rows: int, grid_cols: int, width: int, kb: bool, chunk: int = 32):
    """traj [F, M, 2] -> (offsets[F*lists+1], samples) like ksj_gpu_gridding_binning."""
    f_count, m, _ = traj.shape
    nchunks = (grid_cols + chunk - 1) // chunk
    lists = grid_rows * nchunks
    all_off, all_smp = [0], []
    for f in range(f_count):
        t = traj[f].astype(np.float64)
        lr = np.floor(t[:, 0] * grid_rows / (2 * math.pi)).astype(np.int64)
        lc = np.floor(t[:, 1] * grid_cols / (2 * math.pi)).astype(np.int64)
        if kb:
            lr = lr - width // 2 + 1
            lc = lc - width // 2 + 1
        r0 = np.mod(lr, grid_rows)
        c0 = np.mod(lc, grid_cols)
        last = np.mod(c0 + width - 1, grid_cols)
        k0, k1 = c0 // chunk, last // chunk
        ids, smp = [], []
        s = np.arange(m)
        for j in range(width):
            row = np.mod(r0 + j, grid_rows)
            ids.append(row * nchunks + k0)
            smp.append(s)
            two = k1 != k0
            ids.append((row * nchunks + k1)[two])
            smp.append(s[two])
        ids = np.concatenate(ids)
        smp = np.concatenate(smp)
        order = np.lexsort((smp, ids))
        ids, smp = ids[order], smp[order]
        counts = np.bincount(ids, minlength=lists)
        base = all_off[-1]
        all_off.extend((base + np.cumsum(counts)).tolist())
        all_smp.append(smp.astype(np.uint32))
    return np.array(all_off, dtype=np.int64), np.concatenate(all_smp)
