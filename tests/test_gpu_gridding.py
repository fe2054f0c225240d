"""GPU parity of the adjoint gridding path (ksj_gpu_gridding_adjoint) against
the FP64 oracle, the reference's float outputs and the reference binning
permutation.  Tolerances: rel L2 <= 1e-5 against FP64 for every float32 form
(the bar this path is held to); the reference's own float path sits 1-3e-5
from FP64 (its float coordinate and phase), so GPU-vs-reference-float is
checked at 1e-4."""
import math

import numpy as np
import pytest

import oracle
from binning_reference import binning

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-5
TOL_REF_F32 = 1e-4


def _run_linear(native, cuda, ks, traj, rows, cols, origin=None, output=0):
    import torch
    from kspacejet_gb300 import gpu

    f = 1 if ks.ndim == 2 else ks.shape[0]
    ks3 = ks.reshape(f, -1, ks.shape[-1])
    tr3 = traj.reshape(f, -1, 2)
    g = gpu.Gridding(image=(rows, cols), channels=ks3.shape[1], samples=ks3.shape[2], frames=f, origin=origin,
                     output=output)
    k = torch.from_numpy(np.ascontiguousarray(ks3)).to(cuda)
    t = torch.from_numpy(np.ascontiguousarray(tr3, dtype=np.float32)).to(cuda)
    ws = g.new_workspace(cuda)
    out = g.new_output(cuda)
    g.run(k, t, out, ws)
    torch.cuda.synchronize()
    return g, out.cpu().numpy(), ws, (k, t)


@pytest.mark.parametrize("name", ["med32", "med64", "smallrect"])
def test_linear_matches_fp64_and_reference_float(native, cuda, orc, fixtures, name):
    tr, ks = fixtures[f"{name}_traj"], fixtures[f"{name}_kspace"]
    rows, cols = (int(v) for v in fixtures[f"{name}_shape"])
    _, out, _, _ = _run_linear(native, cuda, ks, tr, rows, cols)
    gpu_img = np.moveaxis(out[0], -1, 0)  # [C, rows, cols]
    d64 = orc.ramp_dcf(tr.astype(np.float64))
    for c in range(ks.shape[0]):
        exact = orc.linear_gridding(rows, cols, ks[c].astype(np.complex128), tr.astype(np.float64), d64, exact=True)
        assert oracle.rel_l2(gpu_img[c], exact) <= TOL_FP64
        assert oracle.rel_l2(gpu_img[c], fixtures[f"{name}_ref_f64"][c]) <= TOL_FP64
        assert oracle.rel_l2(gpu_img[c], fixtures[f"{name}_ref_f32"][c]) <= TOL_REF_F32


def test_reference_unit_fixtures(native, cuda, fixtures):
    # radial_gridding_tests.cpp:92-125 (1, 1, 0, 0) and :31-90 (== weighted direct NUDFT)
    _, out, _, _ = _run_linear(native, cuda, fixtures["offbin_samples"].astype(np.complex64)[None],
                               fixtures["offbin_traj"].astype(np.float32), 2, 2, origin=(0.0, 0.0))
    np.testing.assert_allclose(out[0, ..., 0], [[1, 1], [0, 0]], atol=1e-6)
    _, out, _, _ = _run_linear(native, cuda, fixtures["cartbin_samples"].astype(np.complex64)[None],
                               fixtures["cartbin_traj"].astype(np.float32), 4, 4, origin=(1.5, 0.5))
    np.testing.assert_allclose(out[0, ..., 0], fixtures["cartbin_direct"], atol=2e-5)
    # the 3x4 byte-identity fixture (:127-165): a non-power-of-two axis (radix 3)
    _, out, _, _ = _run_linear(native, cuda, fixtures["repeat_samples"][None], fixtures["repeat_traj"], 3, 4,
                               origin=(0.0, 0.0))
    np.testing.assert_allclose(out[0, ..., 0], fixtures["repeat_out"], atol=2e-5)


def test_large_linear_matches_fp64(native, cuda, orc):
    """N = 256 and 512, M = 65 536 (the reference operator's envelope), 4 coils."""
    from kspacejet_gb300 import synth

    for n in (256, 512):
        tr = synth.golden_angle_radial(512, 128)
        ks = synth.random_kspace(4, tr.shape[0], seed=n)
        _, out, _, _ = _run_linear(native, cuda, ks, tr, n, n)
        # float32(-pi) lies just outside double pi: weight with numpy, not the checked ramp
        d64 = np.hypot(tr[:, 0].astype(np.float64), tr[:, 1].astype(np.float64))
        for c in range(2):
            exact = orc.linear_gridding(n, n, ks[c].astype(np.complex128), tr.astype(np.float64), d64, exact=True)
            err = oracle.rel_l2(out[0, ..., c], exact)
            print(f"linear N={n} coil {c}: rel L2 vs FP64 {err:.3e}")
            assert err <= TOL_FP64, (n, c, err)


def test_deterministic_byte_identical_repeats(native, cuda):
    """radial_gridding_tests.cpp:127-165: repeated executions are byte-identical."""
    import torch
    from kspacejet_gb300 import synth

    tr = synth.golden_angle_radial(256, 64)
    ks = synth.random_kspace(8, tr.shape[0], seed=1)
    g, out1, ws, (k, t) = _run_linear(native, cuda, ks, tr, 128, 128)
    outs = []
    for _ in range(3):
        o = g.new_output(cuda)
        g.run(k, t, o, ws)
        torch.cuda.synchronize()
        outs.append(o.cpu().numpy())
    for o in outs:
        assert o.tobytes() == out1.tobytes()


@pytest.mark.parametrize("kb,grid,width", [(False, 64, 2), (False, 512, 2), (True, 384, 4), (True, 96, 6)])
def test_binning_permutation_is_bit_exact(native, cuda, kb, grid, width):
    import torch
    from kspacejet_gb300 import gpu, synth

    frames = 3
    tr = np.stack([synth.golden_angle_radial(grid, 24, first_spoke=24 * f) for f in range(frames)])
    if kb:
        g = gpu.kb_gridding(image=grid // 2, grid=grid, channels=2, samples=tr.shape[1], frames=frames, width=width)
    else:
        g = gpu.Gridding(image=(grid, grid), channels=2, samples=tr.shape[1], frames=frames)
    k = torch.from_numpy(synth.random_kspace(2, tr.shape[1], 3, frames=frames)).to(cuda)
    t = torch.from_numpy(tr).to(cuda)
    ws = g.new_workspace(cuda)
    g.run(k, t, g.new_output(cuda), ws)
    torch.cuda.synchronize()
    cw, off, smp = g.binning(ws)
    ref_off, ref_smp = binning(tr, grid, grid, width, kb, chunk=cw)
    np.testing.assert_array_equal(off, ref_off)
    np.testing.assert_array_equal(smp, ref_smp)


def test_binning_of_lists_beyond_the_shared_sort_buffer(native, cuda):
    """12 000 spokes through one 64-cell grid: the centre lists hold up to ~9e4
    entries, beyond the long-list sort's 16 K-entry shared buffer, so they are
    sorted in global memory with chunk-local stages in shared memory (several
    merge levels above the chunk size).  The lists match the restatement
    exactly: every entry present, in increasing sample order."""
    import torch
    from kspacejet_gb300 import gpu, synth

    tr = synth.golden_angle_radial(64, 12000)[None]
    g = gpu.kb_gridding(image=32, grid=64, channels=1, samples=tr.shape[1], width=4)
    k = torch.from_numpy(synth.random_kspace(1, tr.shape[1], 5)).to(cuda)[None].contiguous()
    ws = g.new_workspace(cuda)
    g.run(k, torch.from_numpy(tr).to(cuda), g.new_output(cuda), ws)
    torch.cuda.synchronize()
    assert g.flags(ws) == 0
    cw, off, smp = g.binning(ws)
    ref_off, ref_smp = binning(tr, 64, 64, 4, True, chunk=cw)
    lengths = np.diff(ref_off)
    assert lengths.max() > 65536 and (lengths > 16384).sum() > 10
    np.testing.assert_array_equal(off, ref_off)
    np.testing.assert_array_equal(smp, ref_smp)


def test_device_checks_flag_bad_inputs(native, cuda):
    import torch
    from kspacejet_gb300 import gpu, synth

    tr = synth.golden_angle_radial(64, 8)
    ks = synth.random_kspace(2, tr.shape[0], seed=2)
    ks[1, 17] = complex("nan")
    g, _, ws, _ = _run_linear(native, cuda, ks, tr, 32, 32)
    assert g.flags(ws) & gpu.FLAG_NONFINITE_SAMPLE
    tr2 = tr.copy()
    tr2[3, 0] = 3.2  # outside [-pi, pi]
    g, _, ws, _ = _run_linear(native, cuda, synth.random_kspace(2, tr.shape[0], seed=2), tr2, 32, 32)
    assert g.flags(ws) & gpu.FLAG_BAD_TRAJECTORY
    g, _, ws, _ = _run_linear(native, cuda, synth.random_kspace(2, tr.shape[0], seed=2), tr, 32, 32)
    assert g.flags(ws) == 0


def _kb_case(orc, image, grid, width, channels, spokes, seed):
    from kspacejet_gb300 import synth

    tr = synth.golden_angle_radial(grid, spokes, first_spoke=seed)
    ks = synth.multicoil_kspace(tr, image, channels, seed=seed, snr_db=30.0)
    return tr, ks


@pytest.mark.parametrize("image,grid,width,first", [(64, 128, 4, 1), (48, 96, 4, 2), (32, 64, 6, 3), (64, 96, 4, 4),
                                                    (32, 64, 4, 0), (32, 64, 2, 0), (64, 128, 8, 0),
                                                    # grids with factors 5 and 7 (mixed-radix stages of any length)
                                                    (80, 160, 4, 5), (70, 140, 4, 6), (60, 90, 4, 7)])
def test_kaiser_bessel_matches_fp64_oracle(native, cuda, orc, image, grid, width, first):
    """Same algorithm in FP64 (oracle) vs the FP32 GPU path: <= 1e-5; against
    the exact direct NUDFT of the DCF-weighted samples: the KB approximation
    bound (width 4: 3e-3, width 6: 2e-4)."""
    import torch
    from kspacejet_gb300 import gpu

    # first = 0 puts spoke 0 on the column axis: coordinates within 2^-25 of
    # grid integers, where the tap window is decided by the last bit
    tr, ks = _kb_case(orc, image, grid, width, channels=2, spokes=40, seed=first)
    g = gpu.kb_gridding(image=image, grid=grid, channels=2, samples=tr.shape[0], width=width,
                        output=gpu.OUTPUT_COIL_MAJOR)
    out = g.new_output(cuda)
    g.run(torch.from_numpy(ks[None]).to(cuda), torch.from_numpy(tr[None]).to(cuda), out, g.new_workspace(cuda))
    got = out.cpu().numpy()[0]
    d64 = np.hypot(tr[:, 0].astype(np.float64), tr[:, 1].astype(np.float64))
    for c in range(2):
        ref = orc.kb_gridding(grid, image, ks[c].astype(np.complex128), tr.astype(np.float64), d64, width=width)
        exact = orc.direct_adjoint(image, image, ks[c].astype(np.complex128) * d64, tr.astype(np.float64))
        e_ref, e_exact = oracle.rel_l2(got[c], ref), oracle.rel_l2(got[c], exact)
        print(f"KB {image}/{grid} W={width} coil {c}: vs FP64 KB {e_ref:.3e}, vs exact NUDFT {e_exact:.3e}")
        assert e_ref <= TOL_FP64
        assert e_exact <= {2: 5e-2, 4: 3e-3, 6: 2e-4, 8: 2e-5}[width]


def test_rss_epilogue_equals_rss_of_coil_images(native, cuda, orc):
    """The fused RSS output equals the channel-order float RSS of the coil
    images of the same call, bit for bit."""
    import torch
    from kspacejet_gb300 import gpu

    tr, ks = _kb_case(orc, 64, 128, 4, channels=5, spokes=30, seed=4)
    k = torch.from_numpy(ks[None]).to(cuda)
    t = torch.from_numpy(tr[None]).to(cuda)
    outs = {}
    for mode in (gpu.OUTPUT_RSS, gpu.OUTPUT_COIL_LAST):
        g = gpu.kb_gridding(image=64, grid=128, channels=5, samples=tr.shape[0], output=mode)
        o = g.new_output(cuda)
        g.run(k, t, o, g.new_workspace(cuda))
        outs[mode] = o.cpu().numpy()[0]
    assert orc.rss(outs[gpu.OUTPUT_COIL_LAST]).tobytes() == outs[gpu.OUTPUT_RSS].tobytes()


@pytest.mark.parametrize("channels", [1, 3, 40])
def test_tunings_are_byte_identical(native, cuda, orc, channels):
    """Every coil grouping, column block, coil split, occupancy and frame
    pass gives the same bytes: each cell sums in sample order and each line's
    FFT does not depend on which block runs it.  40 channels take two coil
    tiles in the column pass (double-buffered); the RSS still adds them in
    channel order.  The default tuning is also checked against FP64."""
    import ctypes

    import torch
    from kspacejet_gb300 import gpu

    tr, ks = _kb_case(orc, 32, 64, 4, channels=channels, spokes=24, seed=5)
    frames = 2
    k = torch.from_numpy(np.stack([ks, ks[:, ::-1].copy()])).to(cuda)
    t = torch.from_numpy(np.stack([tr, tr[::-1].copy()])).to(cuda)
    outs = {}
    for mode in (gpu.OUTPUT_RSS, gpu.OUTPUT_COIL_LAST, gpu.OUTPUT_COIL_MAJOR):
        g = gpu.kb_gridding(image=32, grid=64, channels=channels, samples=tr.shape[0], frames=frames, output=mode)
        ws = g.new_workspace(cuda)
        base = g.new_output(cuda)
        g.run(k, t, base, ws)
        want = base.cpu().numpy()
        outs[mode] = want
        gcols = 2
        while gcols < channels and gcols < 32:
            gcols *= 2
        for cg in (1, 2, 8, 32):
            for cb in (max(1, 32 // gcols), 2 * max(1, 32 // gcols)):
                for parts, rb, fpp in ((1, 1, 0), (2, 2, 1), (1, 2, 1)):
                    if parts > cg:
                        continue
                    tun = gpu.GriddingTuning(ctypes.sizeof(gpu.GriddingTuning), cg, cb, 0, fpp, rb, parts)
                    try:
                        need = g.workspace_bytes()
                        o = g.new_output(cuda)
                        o.fill_(float("nan")) if o.dtype == torch.float32 else o.real.fill_(float("nan"))
                        g.run(k, t, o, ws, tuning=tun)
                    except gpu.GpuError:
                        continue  # a combination this shape cannot take (shared memory)
                    got = o.cpu().numpy()
                    assert got.tobytes() == want.tobytes(), (mode, cg, cb, parts, rb, fpp, need)
    assert orc.rss(outs[gpu.OUTPUT_COIL_LAST][0]).tobytes() == outs[gpu.OUTPUT_RSS][0].tobytes()
    np.testing.assert_array_equal(outs[gpu.OUTPUT_COIL_MAJOR], np.moveaxis(outs[gpu.OUTPUT_COIL_LAST], -1, 1))
    d64 = np.hypot(tr[:, 0].astype(np.float64), tr[:, 1].astype(np.float64))
    for c in range(min(channels, 3)):
        ref = orc.kb_gridding(64, 32, ks[c].astype(np.complex128), tr.astype(np.float64), d64, width=4)
        assert oracle.rel_l2(outs[gpu.OUTPUT_COIL_MAJOR][0, c], ref) <= TOL_FP64


@pytest.mark.parametrize("channels,grid,width", [(32, 128, 4), (40, 192, 4), (32, 384, 6)])
def test_two_step_rows_byte_identical_across_row_kernels(native, cuda, orc, channels, grid, width):
    """Grid lengths with the two-step transform (128 .. 384): the row pass with
    one or two CTAs per SM, over one or several frame passes (passes of a
    multi-pass call run on two streams), and the shared-memory accumulation of
    smaller coil groups all give the same bytes, for RSS and coil-last output;
    the default is checked against FP64."""
    import ctypes

    import torch
    from kspacejet_gb300 import gpu

    image = grid // 2
    tr, ks = _kb_case(orc, image, grid, width, channels=channels, spokes=20, seed=7)
    frames = 3
    k = torch.from_numpy(np.stack([ks, ks[:, ::-1].copy(), ks])).to(cuda)
    t = torch.from_numpy(np.stack([tr, tr[::-1].copy(), tr[::-1].copy()])).to(cuda)
    for mode in (gpu.OUTPUT_RSS, gpu.OUTPUT_COIL_LAST):
        g = gpu.kb_gridding(image=image, grid=grid, channels=channels, samples=tr.shape[0], frames=frames,
                            width=width, output=mode)
        ws = g.new_workspace(cuda)
        base = g.new_output(cuda)
        g.run(k, t, base, ws)
        want = base.cpu().numpy()
        ran = []
        # column pass 1: one CTA per (frame, column block); 2: the persistent ring
        for cg, rb, fpp, colp in ((32, 1, 0, 1), (32, 2, 0, 2), (32, 2, 1, 1), (32, 1, 2, 2), (16, 2, 0, 1),
                                  (8, 1, 1, 2), (32, 2, 0, 1)):
            tun = gpu.GriddingTuning(ctypes.sizeof(gpu.GriddingTuning), cg, 0, 0, fpp, rb, 1, colp)
            o = g.new_output(cuda)
            o.fill_(float("nan")) if o.dtype == torch.float32 else o.real.fill_(float("nan"))
            g.run(k, t, o, ws, tuning=tun)
            assert g.flags(ws) == 0
            assert o.cpu().numpy().tobytes() == want.tobytes(), (mode, cg, rb, fpp, colp)
            ran.append((cg, rb, fpp))
        assert (32, 2, 1) in ran
        if mode == gpu.OUTPUT_COIL_LAST:
            d64 = np.hypot(tr[:, 0].astype(np.float64), tr[:, 1].astype(np.float64))
            ref = orc.kb_gridding(grid, image, ks[0].astype(np.complex128), tr.astype(np.float64), d64, width=width)
            assert oracle.rel_l2(want[0][..., 0], ref) <= TOL_FP64


@pytest.mark.parametrize("channels,grid,spokes", [(40, 128, 600), (32, 192, 160)])
def test_long_lists_byte_identical(native, cuda, orc, channels, grid, spokes):
    """Dense radial sampling: every spoke crosses the grid centre, so the
    centre rows' lists hold hundreds to thousands of entries (far beyond one
    32-entry staging batch).  Every row kernel (32-coil register path, smaller
    coil groups, coil parts, one or two CTAs per SM, frame passes) sums each
    cell in the same order and gives the same bytes; the result stays within
    1e-5 of FP64."""
    import ctypes

    import torch
    from kspacejet_gb300 import gpu

    image = grid // 2
    tr, ks = _kb_case(orc, image, grid, 4, channels=channels, spokes=spokes, seed=3)
    # every spoke has a sample within one grid unit of the centre, so the
    # centre row's list at the centre column holds at least one entry per spoke
    u = np.hypot(tr[:, 0], tr[:, 1]) * grid / (2 * np.pi)
    assert int((u < 1.0).sum()) >= spokes
    frames = 2
    k = torch.from_numpy(np.stack([ks, ks[:, ::-1].copy()])).to(cuda)
    t = torch.from_numpy(np.stack([tr, tr[::-1].copy()])).to(cuda)
    g = gpu.kb_gridding(image=image, grid=grid, channels=channels, samples=tr.shape[0], frames=frames, width=4,
                        output=gpu.OUTPUT_COIL_LAST)
    ws = g.new_workspace(cuda)
    base = g.new_output(cuda)
    g.run(k, t, base, ws)
    assert g.flags(ws) == 0
    want = base.cpu().numpy()
    for cg, rb, fpp, parts, colp in ((32, 1, 0, 1, 1), (32, 2, 1, 1, 2), (16, 2, 0, 1, 1), (16, 1, 0, 2, 2),
                                     (8, 2, 1, 2, 1), (8, 1, 0, 1, 2)):
        tun = gpu.GriddingTuning(ctypes.sizeof(gpu.GriddingTuning), cg, 0, 0, fpp, rb, parts, colp)
        o = g.new_output(cuda)
        o.real.fill_(float("nan"))
        g.run(k, t, o, ws, tuning=tun)
        assert g.flags(ws) == 0
        assert o.cpu().numpy().tobytes() == want.tobytes(), (cg, rb, fpp, parts, colp)
    d64 = np.hypot(tr[:, 0].astype(np.float64), tr[:, 1].astype(np.float64))
    for c in (0, channels - 1):
        ref = orc.kb_gridding(grid, image, ks[c].astype(np.complex128), tr.astype(np.float64), d64, width=4)
        assert oracle.rel_l2(want[0][..., c], ref) <= TOL_FP64


def test_bf16_sample_storage_bound(native, cuda, orc):
    """BF16 sample storage, FP32 arithmetic: within 2e-3 rel L2 of the
    FP32-storage result (bfloat16 keeps 8 mantissa bits: ~1.6e-3 per sample);
    the bound against the FP64 oracle is tested on the batched shape
    (test_gpu_config_shapes.py)."""
    import torch
    from kspacejet_gb300 import gpu

    tr, ks = _kb_case(orc, 64, 128, 4, channels=3, spokes=40, seed=9)
    k32 = torch.from_numpy(ks[None]).to(cuda)
    kb16 = torch.view_as_real(k32).to(torch.bfloat16).contiguous()
    t = torch.from_numpy(tr[None]).to(cuda)
    res = {}
    for fmt, k in ((gpu.SAMPLES_CF32, k32), (gpu.SAMPLES_BF16, kb16)):
        g = gpu.kb_gridding(image=64, grid=128, channels=3, samples=tr.shape[0], output=gpu.OUTPUT_COIL_MAJOR,
                            sample_format=fmt)
        o = g.new_output(cuda)
        g.run(k, t, o, g.new_workspace(cuda))
        res[fmt] = o.cpu().numpy()
    err = oracle.rel_l2(res[gpu.SAMPLES_BF16], res[gpu.SAMPLES_CF32])
    assert 1e-5 < err < 2e-3


def test_direct_adjoint_matches_fp64(native, cuda, orc, fixtures):
    import torch
    from kspacejet_gb300 import gpu, synth

    tr = synth.golden_angle_radial(64, 16)
    ks = synth.random_kspace(3, tr.shape[0], seed=6)
    out = gpu.direct_adjoint(torch.from_numpy(ks).to(cuda), torch.from_numpy(tr).to(cuda), 32, 48).cpu().numpy()
    for c in range(3):
        ref = orc.direct_adjoint(32, 48, ks[c].astype(np.complex128), tr.astype(np.float64))
        assert oracle.rel_l2(out[..., c], ref) <= TOL_FP64
    k = fixtures["host_kspace"]
    o = gpu.direct_adjoint(torch.from_numpy(k.reshape(2, 2)).to(cuda),
                           torch.from_numpy(fixtures["host_traj"]).to(cuda), 2, 2).cpu().numpy()
    np.testing.assert_allclose(o[..., 0], fixtures["host_direct_ch0"], atol=1e-5)
    np.testing.assert_allclose(o[..., 1], fixtures["host_direct_ch1"], atol=1e-5)


def test_rss_kernel_is_bit_exact(native, cuda, orc, fixtures):
    import torch
    from kspacejet_gb300 import gpu

    x = fixtures["rss_input"]
    out = gpu.rss_coil_last(torch.from_numpy(x).to(cuda)).cpu().numpy()
    assert out.tobytes() == orc.rss(x).tobytes()
    rng = np.random.default_rng(0)
    y = (rng.standard_normal((97, 65, 13)) + 1j * rng.standard_normal((97, 65, 13))).astype(np.complex64)
    out = gpu.rss_coil_last(torch.from_numpy(y).to(cuda)).cpu().numpy()
    assert out.tobytes() == orc.rss(y).tobytes()


@pytest.mark.parametrize("output,fmt,dcf_mode,pinned,fpp", [
    ("rss", "cf32", "ramp", True, 0), ("coil_last", "cf32", "external", True, 0),
    ("coil_major", "bf16", "ramp", False, 0), ("rss", "cf32", "ramp", True, 2)])
def test_host_entry_point_equals_device_entry_point(native, cuda, orc, output, fmt, dcf_mode, pinned, fpp):
    """ksj_gpu_gridding_adjoint_host (host buffers, copies overlapped with the
    frame passes) gives the bytes of ksj_gpu_gridding_adjoint on device copies
    of the same inputs: every output form, both sample formats, external
    weights, pinned and pageable host memory, automatic and fixed passes."""
    import ctypes

    import torch
    from kspacejet_gb300 import gpu

    mode = {"rss": gpu.OUTPUT_RSS, "coil_last": gpu.OUTPUT_COIL_LAST, "coil_major": gpu.OUTPUT_COIL_MAJOR}[output]
    sf = gpu.SAMPLES_BF16 if fmt == "bf16" else gpu.SAMPLES_CF32
    dm = gpu.DCF_EXTERNAL if dcf_mode == "external" else gpu.DCF_ANALYTIC_RAMP
    frames, channels = 5, 6
    trs, kss = [], []
    for f in range(frames):
        tr, ks = _kb_case(orc, 64, 128, 4, channels=channels, spokes=16, seed=20 + f)
        trs.append(tr)
        kss.append(ks)
    tr = np.stack(trs)
    ks = np.stack(kss)
    g = gpu.kb_gridding(image=64, grid=128, channels=channels, samples=tr.shape[1], frames=frames, output=mode,
                        dcf=dm, sample_format=sf)
    kt = torch.from_numpy(ks)
    if sf == gpu.SAMPLES_BF16:
        kt = torch.view_as_real(kt).to(torch.bfloat16).contiguous()
    tt = torch.from_numpy(tr)
    dcf = torch.from_numpy(np.random.default_rng(3).uniform(0.5, 2.0, tr.shape[:2]).astype(np.float32))
    tun = gpu.GriddingTuning(ctypes.sizeof(gpu.GriddingTuning), 0, 0, 0, fpp, 0, 0)
    ws = g.new_workspace(cuda)
    dev_out = g.new_output(cuda)
    g.run(kt.to(cuda), tt.to(cuda), dev_out, ws, dcf=dcf.to(cuda) if dm == gpu.DCF_EXTERNAL else None, tuning=tun)
    want = dev_out.cpu().numpy()
    if pinned:
        kt, tt, dcf = kt.pin_memory(), tt.pin_memory(), dcf.pin_memory()
    host_out = torch.empty(g.output_shape(), dtype=g.output_dtype())
    if pinned:
        host_out = host_out.pin_memory()
    wsh = g.new_host_workspace(cuda)
    for _ in range(2):
        host_out.fill_(float("nan")) if host_out.dtype == torch.float32 else host_out.real.fill_(float("nan"))
        g.run_host(kt, tt, host_out, wsh, dcf=dcf if dm == gpu.DCF_EXTERNAL else None, tuning=tun)
        torch.cuda.synchronize()
        assert host_out.numpy().tobytes() == want.tobytes()
    assert g.flags(wsh) == 0
    with pytest.raises(ValueError):
        g.run_host(kt.to(cuda), tt, host_out, wsh)
