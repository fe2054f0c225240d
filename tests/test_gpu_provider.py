"""The drop-in plug-ins fired end to end on the GPU through the C ABI,
against the reference Provider tests' expectations (tolerance 1e-5 absolute
on the tiny fixtures, as the reference tests use)."""
import math

import numpy as np
import pytest

import oracle

H = pytest.importorskip("kspacejet_gb300.host")
pytestmark = pytest.mark.gpu


def _fire(module, op, cfg, ks, tr, channels, pixels, scratch):
    out = H.aligned((pixels * channels,), np.complex64)
    with module.instance(op, cfg) as inst:
        r = inst.fire([(H.aligned_copy(ks), H.TYPE_KSPACE, 0), (H.aligned_copy(tr), H.TYPE_TRAJECTORY, 1)], out,
                      H.TYPE_COIL_IMAGE, scratch_bytes=scratch)
    return r


@pytest.fixture(scope="module")
def recon(native):
    m = H.ProviderModule(native.NONCARTESIAN_PLUGIN)
    yield m
    m.close()


def test_tiny_radial_channel(recon, fixtures, cuda):
    # provider_tests.cpp:467-502
    k, tr = fixtures["host_kspace"][:2], fixtures["host_traj"].ravel()
    r = _fire(recon, "radial_gridding_reconstruct", H.radial_config(1, 2, 2, 2), k, tr, 1, 4, 104)
    assert r.status == 0 and r.outcome == 0 and r.consumed == 2 and r.sealed_count == 1 and r.seal_calls == 1
    assert (r.sealed_key, r.sealed_order) == (71, 73)
    np.testing.assert_allclose(r.output.reshape(2, 2), fixtures["host_radial_1ch"], atol=1e-5)


def test_tiny_direct_and_coil_last_order(recon, fixtures, cuda):
    # provider_tests.cpp:434-465, 504-530
    k, tr = fixtures["host_kspace"], fixtures["host_traj"].ravel()
    r = _fire(recon, "noncartesian_adjoint_reconstruct", H.direct_config(2, 2, 2, 2), k, tr, 2, 4, 32)
    assert r.status == 0 and r.consumed == 2 and r.sealed_metadata_size == 3
    out = r.output.reshape(2, 2, 2)
    np.testing.assert_allclose(out[..., 0], fixtures["host_direct_ch0"], atol=1e-5)
    np.testing.assert_allclose(out[..., 1], fixtures["host_direct_ch1"], atol=1e-5)


def test_ports_resolved_by_id(recon, fixtures, cuda):
    k, tr = H.aligned_copy(fixtures["host_kspace"]), H.aligned_copy(fixtures["host_traj"].ravel())
    out = H.aligned((8,), np.complex64)
    with recon.instance("noncartesian_adjoint_reconstruct", H.direct_config(2, 2, 2, 2)) as inst:
        r = inst.fire([(k, H.TYPE_KSPACE, 0), (tr, H.TYPE_TRAJECTORY, 1)], out, H.TYPE_COIL_IMAGE,
                      scratch_bytes=32, reverse_batch_order=True)
    assert r.status == 0 and r.consumed == 2 and r.seal_calls == 1


def test_rectangular_route_fixture(recon, fixtures, cuda):
    # radial_rss_hdf5_tests.cpp:187-232, through both plug-ins
    tr = fixtures["rect_traj"].ravel()
    ks = fixtures["rect_coils"]
    r = _fire(recon, "radial_gridding_reconstruct", H.radial_config(2, 2, 4, 2), ks, tr, 2, 8,
              H.radial_scratch_bytes(2, 4, 2))
    assert r.status == 0
    imgs = r.output.reshape(2, 4, 2)
    np.testing.assert_allclose(np.moveaxis(imgs, -1, 0), fixtures["rect_images"], atol=1e-5)
    cc = H.ProviderModule(H.lib and __import__("kspacejet_gb300").COIL_COMBINE_PLUGIN)
    try:
        out = H.aligned((2, 4), np.float32)
        with cc.instance("coil_combine_rss", H.rss_config(2, 4, 2)) as inst:
            rr = inst.fire([(H.aligned_copy(imgs), H.TYPE_COIL_IMAGE, 0)], out, H.TYPE_IMAGE)
        assert rr.status == 0 and rr.sealed_metadata_size == 0
        np.testing.assert_allclose(out, fixtures["rect_rss"], atol=1e-5)
    finally:
        cc.close()


def test_coil_combine_known_answers(native, fixtures, orc, cuda):
    # coil_combine_provider_tests.cpp:299-320
    m = H.ProviderModule(native.COIL_COMBINE_PLUGIN)
    try:
        out = H.aligned((2, 2), np.float32)
        with m.instance("coil_combine_rss", H.rss_config(2, 2, 2)) as inst:
            r = inst.fire([(H.aligned_copy(fixtures["rss_input"]), H.TYPE_COIL_IMAGE, 0)], out, H.TYPE_IMAGE)
        assert r.status == 0 and r.consumed == 1 and r.sealed_count == 1
        np.testing.assert_allclose(out, fixtures["rss_out"], atol=1e-5)
        assert out.tobytes() == orc.rss(fixtures["rss_input"]).tobytes()
    finally:
        m.close()


def test_envelope_maximum_through_the_plugin(recon, orc, cuda):
    """N = 512, M = 65 536, 8 channels through the plug-in, against FP64."""
    from kspacejet_gb300 import synth

    tr = synth.golden_angle_radial(512, 128)
    ks = synth.random_kspace(8, tr.shape[0], seed=3)
    r = _fire(recon, "radial_gridding_reconstruct", H.radial_config(8, 512, 512, 65536), ks, tr.ravel(), 8,
              512 * 512, H.radial_scratch_bytes(512, 512, 65536))
    assert r.status == 0
    out = r.output.reshape(512, 512, 8)
    d64 = np.hypot(tr[:, 0].astype(np.float64), tr[:, 1].astype(np.float64))
    dcf32 = orc.ramp_dcf(tr)
    for c in (0, 7):
        ref = orc.linear_gridding(512, 512, ks[c].astype(np.complex128), tr.astype(np.float64), d64, exact=True)
        assert oracle.rel_l2(out[..., c], ref) <= 1e-5
        # the reference library's own float output (the restatement that is
        # bit-identical to it), as its Provider test compares Provider and
        # library (noncartesian_recon_provider_tests.cpp:434-502); the
        # reference itself sits 1.6-3.2e-5 from FP64 at this size
        lib32 = orc.linear_gridding(512, 512, ks[c], tr, dcf32)
        err32 = oracle.rel_l2(out[..., c], lib32.astype(np.complex128))
        print(f"plug-in vs the reference's float library output, coil {c}: {err32:.3e}")
        assert err32 <= 1e-4


def test_nonfinite_sample_is_an_internal_error_with_released_grant(recon, cuda):
    """The reference library throws on a non-finite sample after the grant is
    acquired; the operator returns INTERNAL_ERROR and its guard releases the
    grant (radial_gridding_reconstruct.cpp:304-312, 432-435)."""
    ks = np.array([1 + 2j, complex("nan")], dtype=np.complex64)
    tr = np.array([0.0, 0.0, math.pi, -0.5 * math.pi], dtype=np.float32)
    r = _fire(recon, "radial_gridding_reconstruct", H.radial_config(1, 2, 2, 2), ks, tr, 1, 4, 104)
    assert r.status == H.INTERNAL_ERROR and r.seal_calls == 0 and r.release_calls == 1


def test_kaiser_bessel_plugin_matches_the_c_abi(native, orc, cuda):
    """radial_kb_gridding_reconstruct / _rss through the plug-in equal the C-ABI
    call on the same inputs (the plug-in adds only copies and validation)."""
    import torch
    from kspacejet_gb300 import gpu, synth

    tr = synth.golden_angle_radial(128, 40, first_spoke=5)
    ks = synth.multicoil_kspace(tr, 64, 3, seed=5)
    cfg = ('{"channels":3,"density_compensation":"radial_analytic_ramp","grid_cols":128,"grid_rows":128,'
           '"image_cols":64,"image_rows":64,"kernel_width":4,"sample_count":%d,'
           '"trajectory_units":"radians_per_pixel"}' % tr.shape[0])
    m = H.ProviderModule(native.KB_PLUGIN)
    try:
        coils = H.aligned((64 * 64 * 3,), np.complex64)
        with m.instance("radial_kb_gridding_reconstruct", cfg) as inst:
            r = inst.fire([(H.aligned_copy(ks), H.TYPE_KSPACE, 0), (H.aligned_copy(tr.ravel()), H.TYPE_TRAJECTORY, 1)],
                          coils, H.TYPE_COIL_IMAGE)
        assert r.status == 0 and r.consumed == 2
        rss = H.aligned((64, 64), np.float32)
        with m.instance("radial_kb_gridding_rss", cfg) as inst:
            r = inst.fire([(H.aligned_copy(ks), H.TYPE_KSPACE, 0), (H.aligned_copy(tr.ravel()), H.TYPE_TRAJECTORY, 1)],
                          rss, H.TYPE_IMAGE)
        assert r.status == 0
    finally:
        m.close()
    g = gpu.kb_gridding(image=64, grid=128, channels=3, samples=tr.shape[0], output=gpu.OUTPUT_COIL_LAST)
    out = g.new_output(cuda)
    g.run(torch.from_numpy(ks[None]).to(cuda), torch.from_numpy(tr[None]).to(cuda), out, g.new_workspace(cuda))
    assert out.cpu().numpy()[0].tobytes() == coils.reshape(64, 64, 3).tobytes()
    assert orc.rss(coils.reshape(64, 64, 3)).tobytes() == rss.tobytes()
