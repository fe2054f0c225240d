"""Pipe-Menon density weights (ksj_gpu_pipe_menon_dcf) against the FP64
oracle restatement of the same grid-based iteration.  Both run in double
precision with the same tap sets; the GPU sums each cell in a fixed order of
its own (a few lanes per list take entries in turn and their sums are added
in lane order; in 3-D, lists split over 512-entry tasks add the tasks' parts
in task order), the oracle in sample order.  They differ in that order, the
Bessel I0 evaluation and fused multiply-adds (~1e-15); the output is float32,
so the bound is 1e-7 relative L2 (float32 rounding of the weights alone is
~3e-8)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-7  # rel L2 of the float32 weights against the FP64 oracle


def _traj(readout, spokes, frames):
    from kspacejet_gb300 import synth

    return np.stack([synth.golden_angle_radial(readout, spokes, first_spoke=spokes * f) for f in range(frames)])


@pytest.mark.parametrize("image,grid,width,iterations", [(32, 64, 4, 10), (48, 96, 6, 10), (32, 64, 4, 1),
                                                         (64, 96, 4, 5)])
def test_pipe_menon_matches_fp64_oracle(native, cuda, orc, image, grid, width, iterations):
    import torch
    from kspacejet_gb300 import gpu

    tr = _traj(grid, 30, 2)
    got = gpu.pipe_menon_dcf(torch.from_numpy(tr).to(cuda), image, grid, width=width,
                             iterations=iterations).cpu().numpy()
    for f in range(tr.shape[0]):
        want = orc.pipe_menon_dcf(tr[f], grid, grid, width, sigma=grid / image, iterations=iterations)
        err = oracle.rel_l2(got[f].astype(np.float64), want)
        print(f"Pipe-Menon {grid} W={width} it={iterations} frame {f}: rel L2 {err:.2e}")
        assert err <= TOL
        assert np.all(got[f] > 0)


def test_pipe_menon_is_deterministic_and_converges(native, cuda, orc):
    """Byte-identical repeats; and at the benchmark's frame shape (34 spokes x
    384, grid 384) the relative change of the weights between iterations falls
    (the fixed point w * (phi conv phi) = 1 is approached)."""
    import torch
    from kspacejet_gb300 import gpu

    tr = torch.from_numpy(_traj(384, 34, 2)).to(cuda)
    a = gpu.pipe_menon_dcf(tr, 192, 384, iterations=10).cpu().numpy()
    b = gpu.pipe_menon_dcf(tr, 192, 384, iterations=10).cpu().numpy()
    assert a.tobytes() == b.tobytes()
    steps = [gpu.pipe_menon_dcf(tr, 192, 384, iterations=i).cpu().numpy().astype(np.float64) for i in (2, 3, 9, 10)]
    early = np.linalg.norm(steps[1] - steps[0]) / np.linalg.norm(steps[0])
    late = np.linalg.norm(steps[3] - steps[2]) / np.linalg.norm(steps[2])
    print(f"relative change: iteration 2->3 {early:.2e}, 9->10 {late:.2e}")
    assert late < early


def _lists3_over(tr, g, width, capacity=512):
    """(longest, count over `capacity`) of the 3-D (plane, row, 16-column
    chunk) lists: a sample is in every list its width^3 taps touch."""
    u = tr.astype(np.float64) * g / (2 * np.pi)
    t0 = np.floor(u).astype(np.int64) - width // 2 + 1
    chunks = np.stack([((t0[:, 2] + c) % g) // 16 for c in range(width)], 1)
    keys = []
    for a in range(width):
        for b in range(width):
            zr = ((t0[:, 0] + a) % g) * g + (t0[:, 1] + b) % g
            for c in range(width):
                first = np.all(chunks[:, :c] != chunks[:, c:c + 1], axis=1)
                keys.append((zr * 64 + chunks[:, c])[first])
    _, cnt = np.unique(np.concatenate(keys), return_counts=True)
    return int(cnt.max()), int((cnt > capacity).sum())


@pytest.mark.parametrize("n,g,width", [(16, 24, 4), (16, 32, 6)])
def test_pipe_menon3_matches_fp64_oracle(native, cuda, orc, n, g, width):
    """3-D Pipe-Menon (the kooshball configuration's density weights) against
    the double-precision restatement, 10 iterations.  The oracle gets the
    float32 kernel shape the GPU path uses.  The centre's lists exceed 1024
    entries, so their cells are split over several 512-entry tasks whose
    parts are added in task order (the oracle sums in sample order, a
    difference of ~1e-16)."""
    import torch
    from kspacejet_gb300 import gpu, synth

    tr = synth.kooshball(g, 300)
    longest, over = _lists3_over(tr, g, width)
    assert longest > 1024 and over > 10
    got = gpu.pipe_menon_dcf3(torch.from_numpy(tr).to(cuda), n, g, width=width).cpu().numpy()
    beta = float(np.float32(orc.kb_beta(width, g / n)))
    want = orc.pipe_menon_dcf3(tr, g, width, beta=beta)
    err = oracle.rel_l2(got.astype(np.float64), want)
    print(f"3-D Pipe-Menon {g}^3 W={width}: rel L2 {err:.2e}")
    assert err <= TOL
    assert np.all(got > 0)
