"""Adaptive (Walsh) coil combination against the CPU restatement
(oracle/walsh.py: double-precision eigendecomposition per pixel).  The GPU
takes the dominant eigenvector by float32 power iteration, so pixels whose
eigenvalue gap lambda_2 / lambda_1 is close to 1 (background noise) converge
slowly; the bounds are written per region."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_SIGNAL = 2e-4   # rel L2 over pixels with a clear dominant eigenvector (gap < 0.3)
TOL_IMAGE = 5e-3    # rel L2 over the whole image (background pixels: no dominant eigenvector)


def _coil_images(n, c, seed):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:n, 0:n] / n - 0.5
    obj = ((xx ** 2 / 0.16 + yy ** 2 / 0.09) < 1.0) * (1.0 + 0.5 * np.cos(6 * xx)) + 0.0j
    obj *= np.exp(1j * 0.8 * yy)
    maps = []
    for _ in range(c):
        cx, cy = rng.uniform(-0.6, 0.6, 2)
        mag = np.exp(-((xx - cx) ** 2 + (yy - cy) ** 2) / 0.3)
        maps.append(mag * np.exp(1j * (rng.uniform(0, 2 * np.pi) + rng.uniform(-2, 2) * xx + rng.uniform(-2, 2) * yy)))
    x = obj[:, :, None] * np.stack(maps, axis=-1)
    x += 0.01 * (rng.standard_normal(x.shape) + 1j * rng.standard_normal(x.shape))
    return x.astype(np.complex64)


@pytest.mark.parametrize("n,c,window", [(64, 4, 7), (96, 8, 7), (48, 3, 5), (40, 1, 3)])
def test_walsh_matches_eigendecomposition(native, cuda, n, c, window):
    import torch
    from kspacejet_gb300 import gpu
    from oracle.walsh import walsh_combine

    x = _coil_images(n, c, seed=n + c)
    got = gpu.walsh_combine(torch.from_numpy(x).to(cuda), window=window, iterations=32).cpu().numpy()
    want, gap = walsh_combine(x, window)
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    sig = gap < 0.3
    err_sig = np.linalg.norm((got - want)[sig]) / np.linalg.norm(want[sig])
    print(f"Walsh n={n} C={c} window={window}: rel L2 {err:.2e}, signal pixels ({sig.mean():.0%}) {err_sig:.2e}")
    assert err_sig <= TOL_SIGNAL
    assert err <= TOL_IMAGE


def test_walsh_rejects_unsupported(native, cuda):
    import torch
    from kspacejet_gb300 import gpu

    x = torch.zeros((8, 8, 9), dtype=torch.complex64, device=cuda)
    with pytest.raises(gpu.GpuError):
        gpu.walsh_combine(x)
    with pytest.raises(gpu.GpuError):
        gpu.walsh_combine(x[:, :, :4].contiguous(), window=6)


# ------------------------------------------------------------ coil compression

TOL_COV = 1e-4  # split-BF16 covariance: relative Frobenius error against FP64


def _correlated_kspace(c, m, seed):
    rng = np.random.default_rng(seed)
    mix = rng.standard_normal((c, c)) + 1j * rng.standard_normal((c, c))
    mix = mix @ np.diag(np.linspace(3.0, 0.1, c))
    z = rng.standard_normal((c, m)) + 1j * rng.standard_normal((c, m))
    return (mix @ z).astype(np.complex64)


@pytest.mark.parametrize("c,m", [(32, 4096), (32, 412160), (8, 13056), (20, 777), (1, 64), (3, 65)])
def test_coil_covariance_tensor_cores_matches_fp64(native, cuda, orc, c, m):
    import torch
    from kspacejet_gb300 import gpu

    x = _correlated_kspace(c, m, seed=c * 1000 + m)
    got = gpu.coil_covariance(torch.from_numpy(x).to(cuda)).cpu().numpy().astype(np.complex128)
    want = orc.coil_covariance(x, double=True)
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    herm = np.abs(got - got.conj().T).max()
    print(f"covariance C={c} M={m}: rel Frobenius {err:.2e} (reference float path: "
          f"{np.linalg.norm(orc.coil_covariance(x) - want) / np.linalg.norm(want):.2e}), hermitian {herm:.1e}")
    assert err <= TOL_COV
    assert herm == 0.0


def test_compression_end_to_end(native, cuda, orc):
    """32 -> 8: covariance on the tensor cores, basis on the host, Y = B X on
    the GPU; the basis spans the same subspace as the FP64 eigenvectors and Y
    equals B X computed in double."""
    import torch
    from kspacejet_gb300 import gpu

    x = _correlated_kspace(32, 50000, seed=7)
    xd = torch.from_numpy(x).to(cuda)
    cov = gpu.coil_covariance(xd).cpu().numpy()
    basis, ev = gpu.compression_basis(cov, 8)
    w, u = np.linalg.eigh(orc.coil_covariance(x, double=True))
    top = u[:, ::-1][:, :8]
    proj_err = np.abs(basis.conj().T @ basis - top @ top.conj().T).max()
    print(f"compression basis: projector error {proj_err:.2e}")
    assert proj_err < 1e-3
    y = gpu.coil_compress(torch.from_numpy(basis).to(cuda), xd).cpu().numpy()
    want = basis.astype(np.complex128) @ x.astype(np.complex128)
    err = np.linalg.norm(y - want) / np.linalg.norm(want)
    print(f"compression apply: rel L2 {err:.2e}")
    assert err < 1e-6
