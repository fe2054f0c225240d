"""Kaiser-Bessel forward NUFFT (ksj_gpu_kb_forward) against the FP64
restatement (the exact transpose of the FP64 gridding adjoint: <= 1e-5 rel
L2 per coil), adjointness with the GPU gridding adjoint, and the
Kaiser-Bessel approximation bound against the exact direct forward."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-5
TOL_EXACT = {4: 3e-3, 6: 2e-4}


def _case(n, g, frames, coils, spokes, seed):
    from kspacejet_gb300 import synth

    rng = np.random.default_rng(seed)
    tr = np.stack([synth.golden_angle_radial(g, spokes, first_spoke=spokes * f) for f in range(frames)])
    img = (rng.standard_normal((frames, n, n, coils)) + 1j * rng.standard_normal((frames, n, n, coils))).astype(np.complex64)
    return tr, img


@pytest.mark.parametrize("n,g,w,frames,coils", [(32, 64, 4, 2, 3), (48, 96, 6, 1, 2), (64, 128, 4, 2, 33),
                                                (96, 192, 4, 1, 8), (24, 48, 8, 1, 1),
                                                # grids with factors 5 and 7 (mixed-radix plans)
                                                (40, 80, 4, 1, 3), (56, 112, 4, 1, 2)])
def test_kb_forward_matches_fp64(native, cuda, orc, n, g, w, frames, coils):
    import torch
    from kspacejet_gb300 import gpu

    tr, img = _case(n, g, frames, coils, spokes=24, seed=n + g + coils)
    fw = gpu.kb_gridding(image=n, grid=g, channels=coils, samples=tr.shape[1], frames=frames, width=w,
                         dcf=gpu.DCF_NONE, output=gpu.OUTPUT_COIL_LAST)
    ws = torch.empty(fw.forward_workspace_bytes(), dtype=torch.uint8, device=cuda)
    got = fw.forward(torch.from_numpy(img).to(cuda), torch.from_numpy(tr).to(cuda), ws).cpu().numpy()
    assert fw.flags(ws) == 0
    worst = 0.0
    for f in range(frames):
        for c in sorted({0, coils - 1}):
            want = orc.kb_forward(g, n, img[f, :, :, c], tr[f].astype(np.float64), width=w)
            worst = max(worst, oracle.rel_l2(got[f, c], want))
    print(f"KB forward n={n} g={g} W={w}: worst rel L2 vs FP64 {worst:.2e}")
    assert worst <= TOL_FP64
    if w in TOL_EXACT:
        exact = orc.direct_forward(n, n, img[0, :, :, 0], tr[0].astype(np.float64))
        e = oracle.rel_l2(got[0, 0], exact)
        print(f"  vs exact direct forward {e:.2e}")
        assert e <= TOL_EXACT[w]


def test_kb_forward_is_adjoint_of_gridding(native, cuda):
    """<A x, y> = <x, A^H y> with A^H the gridding adjoint without density weights."""
    import torch
    from kspacejet_gb300 import gpu

    n, g, frames, coils = 96, 192, 2, 8
    tr, img = _case(n, g, frames, coils, spokes=30, seed=3)
    rng = np.random.default_rng(4)
    y = (rng.standard_normal((frames, coils, tr.shape[1])) + 1j * rng.standard_normal((frames, coils, tr.shape[1]))).astype(np.complex64)
    op = gpu.kb_gridding(image=n, grid=g, channels=coils, samples=tr.shape[1], frames=frames, width=4,
                         dcf=gpu.DCF_NONE, output=gpu.OUTPUT_COIL_LAST)
    t = torch.from_numpy(tr).to(cuda)
    ax = op.forward(torch.from_numpy(img).to(cuda), t).cpu().numpy().astype(np.complex128)
    out = op.new_output(cuda)
    op.run(torch.from_numpy(y).to(cuda), t, out, op.new_workspace(cuda))
    ahy = out.cpu().numpy().astype(np.complex128)
    lhs = np.vdot(y.astype(np.complex128), ax)
    rhs = np.vdot(ahy, img.astype(np.complex128))
    rel = abs(lhs - rhs) / abs(lhs)
    print(f"KB adjointness: {rel:.2e}")
    assert rel <= 1e-5


def test_kb_forward_flags_and_rejects(native, cuda):
    import torch
    from kspacejet_gb300 import gpu

    op = gpu.kb_gridding(image=32, grid=64, channels=2, samples=3, dcf=gpu.DCF_NONE, output=gpu.OUTPUT_COIL_LAST)
    ws = torch.empty(op.forward_workspace_bytes(), dtype=torch.uint8, device=cuda)
    tr = torch.tensor([[[0.1, 0.2], [float("nan"), 0.0], [0.3, -0.1]]], dtype=torch.float32, device=cuda)
    y = op.forward(torch.ones((1, 32, 32, 2), dtype=torch.complex64, device=cuda), tr, ws).cpu().numpy()
    assert op.flags(ws) & gpu.FLAG_BAD_TRAJECTORY
    assert (y[0, :, 1] == 0).all() and np.isfinite(y).all()
    lin = gpu.Gridding(image=(32, 32), channels=2, samples=3)
    with pytest.raises(gpu.GpuError):
        lin.forward_workspace_bytes()
