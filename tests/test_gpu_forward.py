"""Direct forward NUDFT (ksj_gpu_direct_forward, the reference's
nufft2_forward on its Eigen backend) against the FP64 restatement and the
reference's known answers; adjointness with ksj_gpu_direct_adjoint."""
import math

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-5  # rel L2 per coil against FP64 (float sums over the pixels)


def test_direct_forward_reference_known_answers(native, cuda):
    """nufft_tests.cpp:12-32 and :34-48 through the GPU path."""
    import torch
    from kspacejet_gb300 import gpu

    img = torch.tensor([[1, 2], [3, 4]], dtype=torch.complex64, device=cuda)[:, :, None]
    tr = torch.tensor([[0.0, 0.0], [math.pi, 0.0]], dtype=torch.float32, device=cuda)
    y = gpu.direct_forward(img, tr, origin=(0.0, 0.0)).cpu().numpy()[0]
    assert abs(y[0] - 10.0) <= 1e-5 and abs(y[1] - (-4.0)) <= 1e-5
    img = torch.tensor([[1, 2]], dtype=torch.complex64, device=cuda)[:, :, None]
    tr = torch.zeros((1, 2), dtype=torch.float32, device=cuda)
    y = gpu.direct_forward(img, tr, origin=(0.0, 0.0)).cpu().numpy()[0]
    assert abs(y[0] - 3.0) <= 1e-6


@pytest.mark.parametrize("rows,cols,coils,spokes", [(32, 48, 3, 40), (64, 64, 9, 24), (17, 5, 1, 8)])
def test_direct_forward_matches_fp64(native, cuda, orc, rows, cols, coils, spokes):
    import torch
    from kspacejet_gb300 import gpu, synth

    rng = np.random.default_rng(rows * cols + coils)
    img = (rng.standard_normal((rows, cols, coils)) + 1j * rng.standard_normal((rows, cols, coils))).astype(np.complex64)
    tr = synth.golden_angle_radial(2 * max(rows, cols), spokes)
    got = gpu.direct_forward(torch.from_numpy(img).to(cuda), torch.from_numpy(tr).to(cuda)).cpu().numpy()
    for c in range(coils):
        want = orc.direct_forward(rows, cols, img[:, :, c], tr.astype(np.float64))
        err = oracle.rel_l2(got[c], want)
        assert err <= TOL_FP64, (c, err)
    print(f"direct forward {rows}x{cols} C={coils} M={tr.shape[0]}: last coil rel L2 {err:.2e}")


def test_direct_forward_is_adjoint_of_direct_adjoint(native, cuda):
    """<A x, y> = <x, A^H y> with both operators on the GPU."""
    import torch
    from kspacejet_gb300 import gpu, synth

    rows, cols, coils = 64, 64, 8
    rng = np.random.default_rng(1)
    x = (rng.standard_normal((rows, cols, coils)) + 1j * rng.standard_normal((rows, cols, coils))).astype(np.complex64)
    tr = synth.golden_angle_radial(128, 40)
    y = (rng.standard_normal((coils, tr.shape[0])) + 1j * rng.standard_normal((coils, tr.shape[0]))).astype(np.complex64)
    t = torch.from_numpy(tr).to(cuda)
    ax = gpu.direct_forward(torch.from_numpy(x).to(cuda), t).cpu().numpy().astype(np.complex128)
    ahy = gpu.direct_adjoint(torch.from_numpy(y).to(cuda), t, rows, cols).cpu().numpy().astype(np.complex128)
    lhs = np.vdot(y.astype(np.complex128), ax)   # <A x, y> as y^H (A x)
    rhs = np.vdot(ahy, x.astype(np.complex128))  # (A^H y)^H x
    rel = abs(lhs - rhs) / abs(lhs)
    print(f"adjointness: |<Ax,y> - <x,A^H y>| / |<Ax,y>| = {rel:.2e}")
    assert rel <= 1e-5


def test_direct_forward_rejects(native, cuda):
    import torch
    from kspacejet_gb300 import gpu

    img = torch.zeros((4, 4, 2), dtype=torch.complex64, device=cuda)
    tr = torch.zeros((3, 2), dtype=torch.float32, device=cuda)
    with pytest.raises(gpu.GpuError):
        gpu.direct_forward(img, tr, origin=(0.1, 0.0))  # origin not exact in float
    with pytest.raises(gpu.GpuError):
        gpu.direct_forward(img, torch.zeros((0, 2), dtype=torch.float32, device=cuda))
