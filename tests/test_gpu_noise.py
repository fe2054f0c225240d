"""Noise model (noise_model_estimate) and prewhitening
(noncartesian_noise_prewhiten) on the GPU against the double-precision
restatement (oracle/noise.py) and the reference's known answers.  The noise
covariance's product sums run on the tensor cores in split BF16 (FP32
accumulate): stated bound 1e-4 relative Frobenius error against FP64, as for
the compression covariance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_COV = 1e-4    # noise covariance, relative Frobenius vs FP64
TOL_W = 1e-3      # whitening matrix, relative Frobenius vs FP64 (W = C^-1/2, condition ~50)
TOL_APPLY = 1e-6  # Y = W X, relative L2 vs FP64 with the same W


def _correlated_noise(c, m, seed, mean=0.0):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((c, c)) + 1j * rng.standard_normal((c, c))
    q, _ = np.linalg.qr(a)
    sigma = (q * np.geomspace(1.0, 1.0 / 50.0, c)) @ q.conj().T  # Hermitian, condition 50
    l = np.linalg.cholesky(sigma)
    z = (rng.standard_normal((c, m)) + 1j * rng.standard_normal((c, m))) / np.sqrt(2.0)
    return (l @ z + mean).astype(np.complex64)


@pytest.mark.parametrize("c,m,mean", [(32, 20000, 0.0), (8, 4096, 0.3 - 0.2j), (3, 65, 0.0), (1, 64, 1.0),
                                      (20, 777, 0.05j)])
def test_noise_model_matches_fp64(native, cuda, c, m, mean):
    import torch
    from kspacejet_gb300 import gpu
    from oracle import noise

    x = _correlated_noise(c, m, seed=c * 100 + m, mean=mean)
    xd = torch.from_numpy(x).to(cuda)
    cov = gpu.noise_covariance(xd).cpu().numpy()
    want = noise.noise_covariance(x)
    err = np.linalg.norm(cov - want) / np.linalg.norm(want)
    assert np.abs(cov - cov.conj().T).max() == 0.0
    w = gpu.noise_model(xd).cpu().numpy()
    w_want = noise.noise_model_estimate(x)
    err_w = np.linalg.norm(w - w_want) / np.linalg.norm(w_want)
    print(f"noise model C={c} M={m}: covariance {err:.2e}, whitening {err_w:.2e}")
    assert err <= TOL_COV
    assert err_w <= TOL_W


def test_noise_model_reference_known_answer(native, cuda):
    """calibration_provider_tests.cpp:464-485 through the GPU path."""
    import torch
    from kspacejet_gb300 import gpu

    x = np.array([[-1, 1, -1, 1], [-2, -2, 2, 2]], dtype=np.complex64)
    w = gpu.noise_model(torch.from_numpy(x).to(cuda)).cpu().numpy()
    assert abs(w[0, 0].real - 1.0) <= 2e-4 and abs(w[1, 1].real - 0.5) <= 2e-4
    assert abs(w[0, 1]) <= 2e-4 and abs(w[1, 0]) <= 2e-4


@pytest.mark.parametrize("c,m", [(32, 412160), (8, 13056), (2, 3), (17, 1001)])
def test_prewhiten_matches_fp64(native, cuda, c, m):
    import torch
    from kspacejet_gb300 import gpu
    from oracle import noise

    rng = np.random.default_rng(c + m)
    w = (rng.standard_normal((c, c)) + 1j * rng.standard_normal((c, c))).astype(np.complex64)
    x = (rng.standard_normal((c, m)) + 1j * rng.standard_normal((c, m))).astype(np.complex64)
    y = gpu.noise_prewhiten(torch.from_numpy(w).to(cuda), torch.from_numpy(x).to(cuda)).cpu().numpy()
    want = noise.noise_prewhiten(w, x)
    err = np.linalg.norm(y - want) / np.linalg.norm(want)
    print(f"prewhiten C={c} M={m}: rel L2 {err:.2e}")
    assert err <= TOL_APPLY


def test_prewhiten_reference_known_answer_and_rejects(native, cuda):
    """kspace_conditioning_provider_tests.cpp:642-675 through the GPU path."""
    import torch
    from kspacejet_gb300 import gpu

    x = torch.tensor([[1, 2, 3], [4, 5, 6]], dtype=torch.complex64, device=cuda)
    w = torch.tensor([[2, 0], [0, 3]], dtype=torch.complex64, device=cuda)
    y = gpu.noise_prewhiten(w, x).cpu().numpy()
    assert np.abs(y.real - np.array([[2, 4, 6], [12, 15, 18]])).max() <= 1e-5
    assert np.abs(y.imag).max() <= 1e-5
    with pytest.raises(gpu.GpuError):
        gpu.noise_prewhiten(w, torch.zeros((3, 4), dtype=torch.complex64, device=cuda))
    with pytest.raises(gpu.GpuError):
        gpu.noise_covariance(torch.zeros((33, 64), dtype=torch.complex64, device=cuda))
