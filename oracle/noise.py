"""CPU restatement of the noise model and prewhitening.  TEST INFRASTRUCTURE
ONLY: the parity checker for ksj_gpu_noise_covariance, ksj_whitening_matrix
and ksj_gpu_noise_prewhiten; the product never imports it.

Follows the reference in double precision:
* noise_model_estimate (providers/kspacejet-calibration/src/operators/
  noise_model_estimate.cpp:149-168): channel means, the population
  covariance C(r, c) = (1/M) sum_s conj(x_r,s - mu_r) (x_c,s - mu_c)
  (libs/numerics/kspacejet-stats/include/kspacejet/stats/moments.hpp:99-140),
  its Hermitian eigendecomposition, and the whitening matrix
  W = V diag(1 / sqrt(max(lambda, 1e-6))) V^H (libs/numerics/kspacejet-linalg/
  include/kspacejet/linalg/whitening.hpp:27-51);
* noncartesian_noise_prewhiten (providers/kspacejet-kspace-conditioning/src/
  operators/noncartesian_noise_prewhiten.cpp:140-146): Y = W X.
Pinned to the reference's known-answer tests (calibration_provider_tests.cpp:
464-485, kspace_conditioning_provider_tests.cpp:642-675) in tests/.
"""
import numpy as np

EIGENVALUE_FLOOR = 1.0e-6


def noise_covariance(x: np.ndarray) -> np.ndarray:
    """[C, M] complex -> [C, C] complex128, the reference's convention."""
    x = np.asarray(x, dtype=np.complex128)
    d = x - x.mean(axis=1, keepdims=True)
    return np.conj(d) @ d.T / x.shape[1]


def whitening_matrix(cov: np.ndarray, floor: float = EIGENVALUE_FLOOR) -> np.ndarray:
    lam, v = np.linalg.eigh(np.asarray(cov, dtype=np.complex128))
    return (v * (1.0 / np.sqrt(np.maximum(lam, floor)))) @ np.conj(v).T


def noise_model_estimate(x: np.ndarray) -> np.ndarray:
    return whitening_matrix(noise_covariance(x))


def noise_prewhiten(w: np.ndarray, x: np.ndarray) -> np.ndarray:
    return np.asarray(w, dtype=np.complex128) @ np.asarray(x, dtype=np.complex128)
