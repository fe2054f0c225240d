"""Cartesian coil images (ksj_gpu_cartesian_ifft2) against the double-precision
restatement (oracle/cartesian.py) and the reference's known answer; the RSS
output equals the RSS of the coil images bit for bit."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL = 3e-6  # rel L2 per coil against FP64 (float transforms of <= 512 points per axis, FFT or direct DFT)


def test_cartesian_reference_known_answer(native, cuda):
    import torch
    from kspacejet_gb300 import gpu

    k = torch.zeros((2, 2, 2), dtype=torch.complex64)
    k[0, 0, 0] = 4.0
    k[1, 0, 0] = 8.0j
    img = gpu.cartesian_ifft2(k.to(cuda)).cpu().numpy()
    assert np.abs(img[..., 0] - 1.0).max() <= 1e-5 and np.abs(img[..., 1] - 2.0j).max() <= 1e-5


@pytest.mark.parametrize("frames,channels,rows,cols", [(2, 8, 256, 256), (1, 32, 384, 192), (3, 5, 96, 64),
                                                      (1, 40, 128, 512), (1, 64, 48, 24), (2, 1, 2, 12),
                                                      # lengths with factors 5, 7 and 3^2 (matrices such as
                                                      # 160, 240, 320, 448 common in MRI)
                                                      (1, 8, 160, 240), (1, 4, 320, 448), (2, 3, 100, 36),
                                                      (1, 2, 210, 98), (1, 16, 7, 5), (1, 32, 288, 144),
                                                      # lengths with a prime factor above 7 (direct DFT on that
                                                      # axis): 110 = 2 x 5 x 11, 121 = 11^2, 509 and 13 prime
                                                      (1, 8, 110, 121), (2, 3, 509, 13), (1, 40, 127, 64),
                                                      (1, 6, 96, 11), (1, 4, 2, 17)])
def test_cartesian_matches_fp64(native, cuda, orc, frames, channels, rows, cols):
    import torch
    from kspacejet_gb300 import gpu
    from oracle.cartesian import ifft2_coil_images

    rng = np.random.default_rng(rows * cols + channels)
    k = (rng.standard_normal((frames, channels, rows, cols)) +
         1j * rng.standard_normal((frames, channels, rows, cols))).astype(np.complex64)
    kd = torch.from_numpy(k).to(cuda)
    got = gpu.cartesian_ifft2(kd).cpu().numpy()
    want = ifft2_coil_images(k)
    worst = max(oracle.rel_l2(got[f, ..., c], want[f, ..., c]) for f in range(frames) for c in range(channels))
    print(f"cartesian {frames}x{channels}x{rows}x{cols}: worst coil rel L2 {worst:.2e}")
    assert worst <= TOL
    rss = gpu.cartesian_ifft2(kd, output=gpu.OUTPUT_RSS).cpu().numpy()
    assert rss.tobytes() == orc.rss(got).tobytes()


def test_cartesian_rejects(native, cuda):
    import torch
    from kspacejet_gb300 import gpu

    with pytest.raises(gpu.GpuError):
        # an axis above the 512 points of the envelope
        gpu.cartesian_ifft2(torch.zeros((2, 520, 64), dtype=torch.complex64, device=cuda))
    with pytest.raises(gpu.GpuError):
        gpu.cartesian_ifft2(torch.zeros((65, 8, 8), dtype=torch.complex64, device=cuda))
