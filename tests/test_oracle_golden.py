"""The CPU oracle pinned against the reference: its own unit-test known
answers, the golden fixtures produced by the compiled reference, and (where
the reference tree exists) the compiled reference itself, live."""
import math

import numpy as np
import pytest

import oracle


def test_ramp_known_answers(orc, fixtures):
    # radial_gridding_tests.cpp:16-29
    out = orc.ramp_dcf(fixtures["ramp_traj"])
    np.testing.assert_array_equal(out, [0.0, 1.0, math.pi])
    np.testing.assert_array_equal(out, fixtures["ramp_out"])


def test_offbin_sample_splits_linearly(orc, fixtures):
    # radial_gridding_tests.cpp:92-125
    tr = fixtures["offbin_traj"]
    out = orc.linear_gridding(2, 2, fixtures["offbin_samples"], tr, orc.ramp_dcf(tr), 0.0, 0.0)
    np.testing.assert_allclose(out, [[1, 1], [0, 0]], atol=1e-12)
    np.testing.assert_array_equal(out, fixtures["offbin_out"])


def test_cartesian_bin_spokes_equal_weighted_direct_nudft(orc, fixtures):
    # radial_gridding_tests.cpp:31-90
    s, tr = fixtures["cartbin_samples"], fixtures["cartbin_traj"]
    d = orc.ramp_dcf(tr)
    out = orc.linear_gridding(4, 4, s, tr, d, 1.5, 0.5)
    direct = orc.direct_adjoint(4, 4, s * d, tr, 1.5, 0.5)
    np.testing.assert_allclose(out, direct, atol=1e-10)
    np.testing.assert_allclose(out, fixtures["cartbin_out"], atol=1e-13)
    np.testing.assert_allclose(direct, fixtures["cartbin_direct"], atol=1e-13)


def test_float_path_matches_reference_fixtures(orc, fixtures):
    s, tr = fixtures["repeat_samples"], fixtures["repeat_traj"]
    out = orc.linear_gridding(3, 4, s, tr, orc.ramp_dcf(tr), 0.0, 0.0)
    np.testing.assert_allclose(out, fixtures["repeat_out"], rtol=0, atol=1e-6)
    again = orc.linear_gridding(3, 4, s, tr, orc.ramp_dcf(tr), 0.0, 0.0)
    assert out.tobytes() == again.tobytes()  # byte-identical repeat (:127-165)


@pytest.mark.parametrize("name", ["med32", "med64", "smallrect"])
def test_seeded_cases_match_reference_overloads(orc, fixtures, name):
    tr, ks = fixtures[f"{name}_traj"], fixtures[f"{name}_kspace"]
    rows, cols = (int(v) for v in fixtures[f"{name}_shape"])
    d32 = orc.ramp_dcf(tr)
    d64 = orc.ramp_dcf(tr.astype(np.float64))
    for c in range(ks.shape[0]):
        f32 = orc.linear_gridding(rows, cols, ks[c], tr, d32)
        f64 = orc.linear_gridding(rows, cols, ks[c].astype(np.complex128), tr.astype(np.float64), d64)
        assert oracle.rel_l2(f32, fixtures[f"{name}_ref_f32"][c]) < 1e-6
        assert oracle.rel_l2(f64, fixtures[f"{name}_ref_f64"][c]) < 1e-13


def test_host_and_rectangular_fixtures(orc, fixtures):
    k, tr = fixtures["host_kspace"], fixtures["host_traj"]
    r = orc.linear_gridding(2, 2, k[:2], tr, orc.ramp_dcf(tr), 0.5, 0.5)
    np.testing.assert_allclose(r, fixtures["host_radial_1ch"], atol=1e-6)
    np.testing.assert_allclose(orc.direct_adjoint(2, 2, k[2:], tr, 0.5, 0.5), fixtures["host_direct_ch1"], atol=1e-5)
    tr = fixtures["rect_traj"]
    imgs = [orc.linear_gridding(2, 4, c, tr, orc.ramp_dcf(tr), 0.5, 1.5) for c in fixtures["rect_coils"]]
    rss = orc.rss(np.stack(imgs, axis=-1))
    np.testing.assert_allclose(rss, fixtures["rect_rss"], rtol=1e-6)


def test_rss_known_answers(orc, fixtures):
    # coil_combine_provider_tests.cpp:299-320
    out = orc.rss(fixtures["rss_input"])
    np.testing.assert_allclose(out, fixtures["rss_out"], atol=1e-5)
    assert out[0, 0] == 5.0 and out[0, 1] == 12.0 and out[1, 0] == 13.0


def test_direct_adjoint_of_dc_sample(orc, fixtures):
    # nufft_tests.cpp:50-68
    out = orc.direct_adjoint(2, 3, np.array([2.0 - 1.0j]), np.array([[0.0, 0.0]]), 0.5, 1.0)
    np.testing.assert_allclose(out, np.full((2, 3), 2.0 - 1.0j), atol=1e-12)
    np.testing.assert_allclose(out, fixtures["dc_out"], atol=1e-12)


def test_forward_known_answer(orc):
    # nufft_tests.cpp:12-32: image [[1,2],[3,4]], origin (0,0): k=0 -> 10, k_row=pi -> -4
    img = np.array([[1, 2], [3, 4]], dtype=np.complex128)
    out = orc.direct_forward(2, 2, img, np.array([[0.0, 0.0], [math.pi, 0.0]]), 0.0, 0.0)
    np.testing.assert_allclose(out, [10.0, -4.0], atol=1e-12)


def test_rejections(orc):
    tr = np.array([[math.pi + 0.001, 0.0]])
    with pytest.raises(oracle.OracleError):
        orc.ramp_dcf(tr)
    with pytest.raises(oracle.OracleError):
        orc.linear_gridding(2, 2, np.array([complex("nan")]), np.zeros((1, 2)), np.ones(1))
    with pytest.raises(oracle.OracleError):
        orc.linear_gridding(2, 2, np.array([1 + 0j]), np.zeros((1, 2)), -np.ones(1))


@pytest.mark.skipif(not oracle.reference_available(), reason="reference tree not compiled on this machine")
def test_restatement_is_bit_identical_to_compiled_reference(orc):
    ref = oracle.Reference()
    rng = np.random.default_rng(5)
    for n, m in [(8, 40), (64, 3000), (256, 20000)]:
        tr = rng.uniform(-math.pi, math.pi, (m, 2)).astype(np.float32)
        y = (rng.standard_normal(m) + 1j * rng.standard_normal(m)).astype(np.complex64)
        d = orc.ramp_dcf(tr)
        np.testing.assert_array_equal(d, ref.ramp_dcf(tr))
        a = orc.linear_gridding(n, n, y, tr, d)
        b = ref.linear_gridding(n, n, y, tr, d)
        assert a.tobytes() == b.tobytes()
        c = orc.direct_adjoint(4, 4, y[:50], tr[:50])
        assert c.tobytes() == ref.direct_adjoint(4, 4, y[:50], tr[:50]).tobytes()
    # a non-power-of-two axis takes the reference's direct-DFT fallback
    tr = rng.uniform(-math.pi, math.pi, (500, 2)).astype(np.float32)
    y = (rng.standard_normal(500) + 1j * rng.standard_normal(500)).astype(np.complex64)
    d = orc.ramp_dcf(tr)
    assert orc.linear_gridding(12, 6, y, tr, d).tobytes() == ref.linear_gridding(12, 6, y, tr, d).tobytes()


def test_binning_rule_matches_double_grid_coordinate(orc):
    """The binning key is the lower index of the reference's double-precision
    grid_coordinate; spot-check the restatement against a numpy evaluation."""
    rng = np.random.default_rng(3)
    for n in (4, 64, 384, 512):
        for f in rng.uniform(-math.pi, math.pi, 200):
            lo, fr = orc.grid_coordinate(float(f), n, f64=True)
            x = f * n / (2 * math.pi)
            x = x + n if x < 0 else x
            x = x - n if x >= n else x
            assert lo == math.floor(x) and abs(fr - (x - math.floor(x))) < 1e-12


def test_kaiser_bessel_oracle_approximates_exact_nudft(orc):
    """KB W=4/6, sigma=2 gridding against the exact direct adjoint of the same
    weighted samples: the approximation error shrinks with the width as the
    published error analysis predicts (about 1e-3 and 1e-5)."""
    rng = np.random.default_rng(8)
    n, g = 16, 32
    tr = rng.uniform(-math.pi, math.pi, (600, 2))
    y = rng.standard_normal(600) + 1j * rng.standard_normal(600)
    exact = orc.direct_adjoint(n, n, y, tr)
    e4 = oracle.rel_l2(orc.kb_gridding(g, n, y, tr, None, width=4), exact)
    e6 = oracle.rel_l2(orc.kb_gridding(g, n, y, tr, None, width=6), exact)
    assert e4 < 5e-3 and e6 < 2e-4 and e6 < e4 / 5
    assert orc.kb_kernel(0.0, 4, orc.kb_beta(4, 2.0)) == 1.0


def test_cartesian_oracle_pinned_to_reference_known_answer():
    """cartesian_recon_provider_tests.cpp:339-366: channels 2, 2 x 2, DC values
    4 and 8i -> coil-last (1, 2i) at every pixel."""
    from oracle.cartesian import ifft2_coil_images

    k = np.zeros((2, 2, 2), dtype=np.complex64)
    k[0, 0, 0] = 4.0
    k[1, 0, 0] = 8.0j
    img = ifft2_coil_images(k)
    assert img.shape == (2, 2, 2)
    assert np.abs(img[..., 0] - 1.0).max() <= 1e-5 and np.abs(img[..., 1] - 2.0j).max() <= 1e-5


def test_ingress_oracle_pinned_to_reference_unit_equivalence():
    """radial_rss_hdf5_tests.cpp:353-390: cycles per FOV 0.5, radians per
    pixel pi and encoded index 1 on a 2 x 2 matrix are the same coordinate
    (float pi), and raw [kx, ky] lands as [row = ky, column = kx]
    (:136-144)."""
    from oracle import ingress

    pi_f = np.float32(np.pi)
    for units, v in ((ingress.CYCLES_PER_FOV, 0.5), (ingress.RADIANS_PER_PIXEL, float(pi_f)),
                     (ingress.ENCODED_MATRIX_INDEX, 1.0)):
        out, ok = ingress.normalize_trajectory(np.array([[v, 0.0], [-v, 0.0]], dtype=np.float32), units, 2, 2)
        assert ok.all()
        assert out[0, 1] == pi_f and out[1, 1] == -pi_f and out[0, 0] == 0.0
    out, ok = ingress.normalize_trajectory(np.array([[-0.25, 0.125]], dtype=np.float32), ingress.CYCLES_PER_FOV)
    assert out[0, 0] == np.float32(0.125) * np.float32(2 * pi_f) and out[0, 1] == np.float32(-0.25) * np.float32(2 * pi_f)
    _, ok = ingress.normalize_trajectory(np.array([[0.5000001, 0.0], [np.nan, 0.0]], dtype=np.float32),
                                         ingress.CYCLES_PER_FOV)
    assert not ok.any()
