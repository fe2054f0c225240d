"""Device ingress conversions against the float32 restatement
(oracle/ingress.py): bit-identical coordinates and validity flags,
bit-identical aggregation."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("units,enc", [(1, (0, 0)), (2, (0, 0)), (3, (256, 192)), (3, (2, 2))])
def test_normalize_trajectory_bit_identical(native, cuda, units, enc):
    import torch
    from kspacejet_gb300 import gpu
    from oracle import ingress

    rng = np.random.default_rng(units * 7 + enc[0])
    lim = {1: (0.5, 0.5), 2: (np.pi, np.pi), 3: (enc[1] / 2.0, enc[0] / 2.0)}[units]
    raw = np.stack([rng.uniform(-lim[0], lim[0], 100000), rng.uniform(-lim[1], lim[1], 100000)], 1).astype(np.float32)
    raw[:4] = [[lim[0], -lim[1]], [-lim[0], lim[1]], [0.0, 0.0], [-0.0, 0.0]]  # interval edges, signed zero
    out, flags = gpu.normalize_trajectory(torch.from_numpy(raw).to(cuda), units, enc)
    want, ok = ingress.normalize_trajectory(raw, units, enc[0], enc[1])
    assert ok.all() and flags == 0
    assert out.cpu().numpy().tobytes() == want.tobytes()


def test_normalize_trajectory_flags_and_rejects(native, cuda):
    import torch
    from kspacejet_gb300 import gpu

    bad = torch.tensor([[0.25, 0.0], [0.5000001, 0.0]], dtype=torch.float32, device=cuda)
    _, flags = gpu.normalize_trajectory(bad, gpu.TRAJ_CYCLES_PER_FOV)
    assert flags & gpu.FLAG_BAD_TRAJECTORY
    nan = torch.tensor([[float("nan"), 0.0]], dtype=torch.float32, device=cuda)
    _, flags = gpu.normalize_trajectory(nan, gpu.TRAJ_RADIANS_PER_PIXEL)
    assert flags & gpu.FLAG_BAD_TRAJECTORY
    with pytest.raises(gpu.GpuError):
        gpu.normalize_trajectory(bad, 0)
    with pytest.raises(gpu.GpuError):
        gpu.normalize_trajectory(bad, gpu.TRAJ_ENCODED_MATRIX_INDEX, (1, 2))


@pytest.mark.parametrize("a,c,n", [(805, 32, 512), (3, 1, 7), (64, 20, 256)])
def test_aggregate_acquisitions_bit_identical(native, cuda, a, c, n):
    import torch
    from kspacejet_gb300 import gpu
    from oracle import ingress

    rng = np.random.default_rng(a + c + n)
    blocks = (rng.standard_normal((a, c, n)) + 1j * rng.standard_normal((a, c, n))).astype(np.complex64)
    got = gpu.aggregate_acquisitions(torch.from_numpy(blocks).to(cuda)).cpu().numpy()
    assert got.tobytes() == ingress.aggregate_acquisitions(blocks).tobytes()
