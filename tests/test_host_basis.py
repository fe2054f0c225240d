"""Host-side compression basis (ksj_coil_compression_basis, double-precision
cyclic Jacobi) against numpy's eigendecomposition: same eigenvalues, same
top-V subspace, orthonormal rows.  Runs without a GPU (host code of the
library)."""
import numpy as np
import pytest


@pytest.mark.parametrize("n,v", [(32, 8), (8, 3), (4, 4), (1, 1), (17, 5), (64, 16)])
def test_basis_spans_top_eigenvectors(native, n, v):
    from kspacejet_gb300 import gpu

    rng = np.random.default_rng(n * 10 + v)
    x = rng.standard_normal((n, 400)) + 1j * rng.standard_normal((n, 400))
    x[: max(1, n // 4)] *= 4.0
    r = (x @ x.conj().T / 400).astype(np.complex64)
    basis, ev = gpu.compression_basis(r, v)
    w, u = np.linalg.eigh(r.astype(np.complex128))
    top = u[:, ::-1][:, :v]
    assert np.abs(basis.conj().T @ basis - top @ top.conj().T).max() < 1e-5
    assert np.abs(ev - w[::-1]).max() <= 1e-5 * w.max()
    assert np.abs(basis @ basis.conj().T - np.eye(v)).max() < 1e-5


def test_basis_rejects_bad_sizes(native):
    from kspacejet_gb300 import gpu

    with pytest.raises(gpu.GpuError):
        gpu.compression_basis(np.eye(4, dtype=np.complex64), 5)


# ---------------------------------------------------------------- noise model

# Known answers of the reference's own tests: 2 channels x 4 noise samples
# (calibration_provider_tests.cpp:464-485, whitening within 2e-4) and the
# prewhitening of 2 x 3 samples by diag(2, 3) (kspace_conditioning_provider_tests.cpp:642-675).
NOISE_2X4 = np.array([[-1, 1, -1, 1], [-2, -2, 2, 2]], dtype=np.complex64)
PREWHITEN_X = np.array([[1, 2, 3], [4, 5, 6]], dtype=np.complex64)
PREWHITEN_W = np.diag([2.0, 3.0]).astype(np.complex64)
PREWHITEN_Y = np.array([[2, 4, 6], [12, 15, 18]], dtype=np.float64)


def test_noise_oracle_pinned_to_reference_known_answers():
    from oracle import noise

    w = noise.noise_model_estimate(NOISE_2X4)
    assert abs(w[0, 0].real - 1.0) <= 2e-4 and abs(w[1, 1].real - 0.5) <= 2e-4
    assert abs(w[0, 1]) <= 2e-4 and abs(w[1, 0]) <= 2e-4
    y = noise.noise_prewhiten(PREWHITEN_W, PREWHITEN_X)
    assert np.abs(y.real - PREWHITEN_Y).max() <= 1e-5 and np.abs(y.imag).max() <= 1e-5


@pytest.mark.parametrize("n,cond", [(32, 50.0), (8, 5.0), (3, 1.0), (1, 1.0), (64, 20.0)])
def test_host_whitening_matches_oracle(native, n, cond):
    """ksj_whitening_matrix (host Jacobi) against numpy's eigh on the same
    covariance, including eigenvalues under the 1e-6 floor."""
    from kspacejet_gb300 import gpu
    from oracle import noise

    rng = np.random.default_rng(n)
    q, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    lam = np.geomspace(1.0, 1.0 / cond, n)
    if n > 4:
        lam[-1] = 1e-8  # below the floor
    cov = ((q * lam) @ q.conj().T).astype(np.complex64)
    w = gpu.whitening_matrix(cov)
    want = noise.whitening_matrix(cov.astype(np.complex128))
    err = np.linalg.norm(w - want) / np.linalg.norm(want)
    assert err <= 1e-5, err
    assert np.abs(w - w.conj().T).max() <= 1e-5 * np.abs(w).max()


def test_host_whitening_known_answer_and_rejects(native):
    from kspacejet_gb300 import gpu
    from oracle import noise

    w = gpu.whitening_matrix(noise.noise_covariance(NOISE_2X4).astype(np.complex64))
    assert np.allclose(w, np.diag([1.0, 0.5]), atol=2e-4)
    with pytest.raises(gpu.GpuError):
        gpu.whitening_matrix(np.full((2, 2), np.nan, dtype=np.complex64))
    with pytest.raises(gpu.GpuError):
        gpu.whitening_matrix(np.eye(2, dtype=np.complex64), floor=0.0)
