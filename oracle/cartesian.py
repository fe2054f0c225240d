"""CPU restatement of the Cartesian coil-image operator.  TEST
INFRASTRUCTURE ONLY: the parity checker for ksj_gpu_cartesian_ifft2; the
product never imports it.

cartesian_ifft2_coil_images (providers/kspacejet-cartesian-recon/src/
operators/cartesian_ifft2_coil_images.cpp:372-407): per channel the inverse
2-D DFT with Normalization::inverse (1/cols on the row pass, 1/rows on the
column pass; libs/numerics/kspacejet-fft/src/eigen/eigen_fft_transforms.cpp:
148-205), no shift, channel-major k-space in, coil-last images out.  The
reference computes the DFT through Eigen's FFT module (its bundled kissfft,
a dependency outside the reference tree); the restatement is the exact
normalised inverse DFT in double precision (numpy's ifft2), pinned to the
reference's known-answer test in tests/.
"""
import numpy as np


def ifft2_coil_images(kspace: np.ndarray) -> np.ndarray:
    """[..., C, rows, cols] complex -> [..., rows, cols, C] complex128."""
    x = np.asarray(kspace, dtype=np.complex128)
    img = np.fft.ifft2(x, axes=(-2, -1))
    return np.moveaxis(img, -3, -1)
