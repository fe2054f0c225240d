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
