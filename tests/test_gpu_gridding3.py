"""3-D Kaiser-Bessel gridding (ksj_gpu_gridding3_adjoint) against the FP64
oracle (the same algorithm in double precision: <= 1e-5 rel L2 per coil) and
the exact 3-D NUDFT of the weighted samples (the Kaiser-Bessel approximation
bound, measured on the oracle: W=4 sigma=1.5 2.6e-3, W=6 6.5e-5)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-5
TOL_EXACT = {4: 5e-3, 6: 2e-4}


def _case(n, readout, spokes, coils, seed):
    from kspacejet_gb300 import synth

    tr = synth.kooshball(readout, spokes)
    rng = np.random.default_rng(seed)
    ks = (rng.standard_normal((coils, tr.shape[0])) + 1j * rng.standard_normal((coils, tr.shape[0]))).astype(np.complex64)
    return tr, ks


def _run(cuda, n, g, w, tr, ks, output, dcf_mode=None, sample_format=0, tuning=None):
    import torch
    from kspacejet_gb300 import gpu

    g3 = gpu.Gridding3(image=n, grid=g, channels=ks.shape[0], samples=tr.shape[0], width=w, output=output,
                       dcf=gpu.DCF_ANALYTIC_RAMP if dcf_mode is None else dcf_mode, sample_format=sample_format)
    k = torch.from_numpy(ks).to(cuda)
    if sample_format == gpu.SAMPLES_BF16:
        re = torch.from_numpy(ks.real.copy()).to(cuda).to(torch.bfloat16)
        im = torch.from_numpy(ks.imag.copy()).to(cuda).to(torch.bfloat16)
        k = torch.stack([re, im], dim=-1).contiguous()
    t = torch.from_numpy(np.ascontiguousarray(tr)).to(cuda)
    out = g3.new_output(cuda)
    g3.run(k, t, out, g3.new_workspace(cuda), tuning=tuning)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("n,g,w,readout,spokes,coils", [(16, 24, 4, 24, 400, 3), (16, 32, 6, 32, 300, 2),
                                                        (24, 48, 4, 48, 400, 5), (20, 40, 4, 40, 300, 2)])
def test_gridding3_matches_fp64_oracle_and_nudft(native, cuda, orc, n, g, w, readout, spokes, coils):
    from kspacejet_gb300 import gpu

    tr, ks = _case(n, readout, spokes, coils, seed=n + g)
    got = _run(cuda, n, g, w, tr, ks, gpu.OUTPUT_COIL_LAST)
    tr64 = tr.astype(np.float64)
    dcf = np.sum(tr64.astype(np.float32).astype(np.float64) ** 2, axis=1)
    for c in range(min(coils, 3)):
        ref = orc.kb_gridding3(g, n, ks[c].astype(np.complex128), tr64, dcf, width=w, sigma=g / n)
        e_ref = oracle.rel_l2(got[..., c], ref)
        msg = f"3-D KB n={n} g={g} W={w} coil {c}: vs FP64 KB {e_ref:.2e}"
        if c == 0:
            exact = orc.direct_adjoint3(n, ks[c].astype(np.complex128) * dcf, tr64)
            e_exact = oracle.rel_l2(got[..., c], exact)
            msg += f", vs exact NUDFT {e_exact:.2e}"
            assert e_exact <= TOL_EXACT[w]
        print(msg)
        assert e_ref <= TOL_FP64


def test_gridding3_rss_deterministic_and_bf16(native, cuda, orc):
    from kspacejet_gb300 import gpu

    tr, ks = _case(16, 24, 400, 4, seed=11)
    coil = _run(cuda, 16, 24, 4, tr, ks, gpu.OUTPUT_COIL_LAST)
    rss = _run(cuda, 16, 24, 4, tr, ks, gpu.OUTPUT_RSS)
    rss2 = _run(cuda, 16, 24, 4, tr, ks, gpu.OUTPUT_RSS)
    assert rss.tobytes() == rss2.tobytes()
    assert orc.rss(coil.reshape(16 * 16, 16, 4)).tobytes() == rss.reshape(16 * 16, 16).tobytes()
    bf = _run(cuda, 16, 24, 4, tr, ks, gpu.OUTPUT_COIL_LAST, sample_format=gpu.SAMPLES_BF16)
    e = np.linalg.norm(bf - coil) / np.linalg.norm(coil)
    print(f"3-D BF16 sample storage vs FP32 storage: {e:.2e}")
    assert e < 1e-2


def test_gridding3_tunings_agree(native, cuda):
    import ctypes

    from kspacejet_gb300 import gpu

    tr, ks = _case(16, 24, 300, 3, seed=5)
    base = _run(cuda, 16, 24, 4, tr, ks, gpu.OUTPUT_RSS)
    for cg, parts, rb, fpp in ((4, 1, 1, 0), (4, 2, 2, 5), (32, 1, 2, 7)):
        t = gpu.GriddingTuning(ctypes.sizeof(gpu.GriddingTuning), cg, 0, 0, fpp, rb, parts)
        got = _run(cuda, 16, 24, 4, tr, ks, gpu.OUTPUT_RSS, tuning=t)
        assert got.tobytes() == base.tobytes(), (cg, parts, rb, fpp)


def test_gridding3_two_step_rows_agree(native, cuda):
    """A grid with the two-step transform (128^3): the row kernels with one or
    two CTAs per SM, over one or several plane passes, and the shared-memory
    form of a smaller coil group give the same bytes."""
    import ctypes

    from kspacejet_gb300 import gpu

    tr, ks = _case(64, 128, 300, 3, seed=12)
    base = _run(cuda, 64, 128, 4, tr, ks, gpu.OUTPUT_RSS,
                tuning=gpu.GriddingTuning(ctypes.sizeof(gpu.GriddingTuning), 32, 0, 0, 0, 2, 1))
    for rb, fpp in ((1, 0), (2, 40), (1, 40)):
        t = gpu.GriddingTuning(ctypes.sizeof(gpu.GriddingTuning), 32, 0, 0, fpp, rb, 1)
        got = _run(cuda, 64, 128, 4, tr, ks, gpu.OUTPUT_RSS, tuning=t)
        assert got.tobytes() == base.tobytes(), (rb, fpp)


def test_gridding3_64_cube_subproblem(native, cuda, orc):
    """The kooshball configuration's accuracy check on a 64^3 sub-problem
    (sigma 1.5, W=4, 96 readout x 2000 spokes): against the FP64 Kaiser-Bessel
    restatement on every voxel, and against the exact NUDFT (in double,
    numpy) on 256 seeded voxels."""
    from kspacejet_gb300 import gpu

    n, g = 64, 96
    tr, ks = _case(n, 96, 2000, 2, seed=64)
    got = _run(cuda, n, g, 4, tr, ks, gpu.OUTPUT_COIL_LAST)[..., 0]
    tr64 = tr.astype(np.float64)
    dcf = np.sum(tr64 ** 2, axis=1)
    ref = orc.kb_gridding3(g, n, ks[0].astype(np.complex128), tr64, dcf, width=4, sigma=g / n)
    e_ref = oracle.rel_l2(got, ref)
    rng = np.random.default_rng(3)
    vox = rng.integers(0, n, size=(256, 3))
    y = ks[0].astype(np.complex128) * dcf
    exact = np.empty(256, dtype=np.complex128)
    for i0 in range(0, 256, 32):
        pos = vox[i0:i0 + 32].astype(np.float64) - (n - 1) / 2.0
        exact[i0:i0 + 32] = np.exp(1j * (tr64 @ pos.T)).T @ y
    approx = got[vox[:, 0], vox[:, 1], vox[:, 2]]
    e_exact = np.linalg.norm(approx - exact) / np.linalg.norm(exact)
    print(f"3-D 64^3 sub-problem: vs FP64 KB {e_ref:.2e}, vs exact NUDFT (256 voxels) {e_exact:.2e}")
    assert e_ref <= TOL_FP64
    assert e_exact <= TOL_EXACT[4]
