"""The drop-in plug-ins' C-ABI contract, checked without a GPU: descriptors,
canonical-config rejections, and every rejection the reference Provider tests
pin that happens before any device work (tests/unit/providers/
kspacejet-noncartesian-recon/noncartesian_recon_provider_tests.cpp:415-705,
kspacejet-coil-combine/coil_combine_provider_tests.cpp:286-353).  Where the
reference tree is compiled, the reference plug-in is driven through the same
host and must answer identically."""
import math

import numpy as np
import pytest

from oracle import build as obuild

H = pytest.importorskip("kspacejet_gb300.host")

RADIAL = "radial_gridding_reconstruct"
DIRECT = "noncartesian_adjoint_reconstruct"


def plugins(native):
    out = [("gb300", native.NONCARTESIAN_PLUGIN)]
    if obuild.REF_PROVIDER_LIB.exists():
        out.append(("reference", obuild.REF_PROVIDER_LIB))
    return out


@pytest.fixture(scope="module")
def modules(native):
    mods = {name: H.ProviderModule(path) for name, path in plugins(native)}
    yield mods
    for m in mods.values():
        m.close()


def test_descriptor_is_the_reference_descriptor(modules):
    m = modules["gb300"]
    assert m.provider_id == "org.kspacejet.noncartesian-recon"
    assert m.digest_hex == "4297da20fe070aae1988f456967aeed82d5bae62f8aad41585e25fe767000ef6"
    assert [o.id for o in m.operators] == [DIRECT, RADIAL]
    d, r = m.operators
    assert d.max_inputs == 2 and d.max_output_bytes == 128 * 1024 * 1024 and d.max_scratch_bytes == 2 * 1024 * 1024
    assert r.max_inputs == 2 and r.max_output_bytes == 128 * 1024 * 1024 and r.max_scratch_bytes == 4464640
    for o in m.operators:
        assert o.max_in_flight == 1 and o.thread_safety == 0 and o.max_private_threads == 0
        assert o.capability_bits == (1 << 4) | (1 << 5)
    assert m.capability_bits == 1 | (1 << 6) | (1 << 7) | (1 << 8)
    if "reference" in modules:
        ref = modules["reference"]
        assert (ref.provider_id, ref.digest_hex, ref.capability_bits) == (m.provider_id, m.digest_hex,
                                                                          m.capability_bits)
        assert ref.operators == m.operators


@pytest.mark.parametrize("op,config", [
    (DIRECT, '{"channels":1,"image_rows":2,"image_cols":2,"sample_count":2}'),          # wrong key order
    (DIRECT, '{"channels":64,"image_cols":512,"image_rows":512,"sample_count":65536}'),  # over the 2^28 bound
    (DIRECT, '{"channels":01,"image_cols":2,"image_rows":2,"sample_count":2}'),         # leading zero
    (DIRECT, '{"channels":1,"image_cols":1,"image_rows":2,"sample_count":2}'),          # axis < 2
    (RADIAL, '{"channels":1,"image_cols":2,"image_rows":2,"sample_count":2,"trajectory_units":"radians_per_pixel"}'),
    (RADIAL, H.radial_config(1, 2, 2, 2).replace("radians_per_pixel", "cycles_per_pixel")),
    (RADIAL, H.radial_config(1, 2, 3, 2)),                                               # non power of two
    (RADIAL, H.radial_config(65, 2, 2, 2)),                                              # channels > 64
    (RADIAL, H.radial_config(1, 2, 2, 65537)),                                           # samples > 65536
    (RADIAL, H.radial_config(1, 1024, 1024, 2)),                                         # axis > 512
])
def test_noncanonical_configs_are_rejected_before_creation(modules, op, config):
    for name, m in modules.items():
        st, created, _ = m.try_create(op, config)
        assert st == H.INVALID_ARGUMENT and not created, name


def test_unknown_operator_is_unsupported(modules):
    for m in modules.values():
        assert m.try_create("radial_kb_gridding_reconstruct", H.radial_config(1, 2, 2, 2))[0] == H.UNSUPPORTED


def test_canonical_configs_create(modules):
    for m in modules.values():
        assert m.try_create(RADIAL, H.radial_config(64, 512, 512, 65536))[:2] == (0, True)
        assert m.try_create(DIRECT, H.direct_config(2, 2, 2, 2))[:2] == (0, True)


def _host_inputs(channels=2, samples=2, traj=None):
    """The reference tests' HostState payloads (provider_tests.cpp:76-78)."""
    ks = np.array([1 + 2j, 3 - 1j, 10 - 4j, -2 + 7j], dtype=np.complex64)[: channels * samples]
    tr = np.array([0.0, 0.0, math.pi, -0.5 * math.pi], dtype=np.float32) if traj is None else traj
    return H.aligned_copy(ks), H.aligned_copy(tr.astype(np.float32))


def _fire(m, op, cfg, scratch, **kw):
    ks, tr = kw.pop("payloads", None) or _host_inputs()
    channels = int(cfg.split('"channels":')[1].split(",")[0])
    out = H.aligned((4 * channels,), np.complex64)
    with m.instance(op, cfg) as inst:
        return inst.fire([(ks, H.TYPE_KSPACE, 0), (tr, H.TYPE_TRAJECTORY, 1)], out, H.TYPE_COIL_IMAGE,
                         scratch_bytes=scratch, **kw)


def _cases():
    direct2 = (DIRECT, H.direct_config(2, 2, 2, 2), 32)
    radial1 = (RADIAL, H.radial_config(1, 2, 2, 2), 104)
    bad_traj = np.array([math.pi + 0.01, 0.0, math.pi, -0.5 * math.pi], dtype=np.float32)
    return {
        "wrong trajectory type": (direct2, dict(corrupt_input_type=2)),
        "wrong kspace type": (direct2, dict(corrupt_input_type=1)),
        "short trajectory": (direct2, dict(payloads=(_host_inputs()[0], H.aligned_copy(np.zeros(3, np.float32))))),
        "identity mismatch": (direct2, dict(input_keys=[(71, 73), (71, 74)])),
        "one input batch": (direct2, dict(reported_input_batch_count=1)),
        "small reserved output": (direct2, dict(reserved_output_bytes=8)),
        "out-of-range radial trajectory": (radial1, dict(payloads=(H.aligned_copy(
            np.array([1 + 2j, 3 - 1j], np.complex64)), H.aligned_copy(bad_traj)))),
        "short radial scratch": ((RADIAL, H.radial_config(1, 2, 2, 2), 103), dict(payloads=(H.aligned_copy(
            np.array([1 + 2j, 3 - 1j], np.complex64)), _host_inputs()[1]))),
    }


@pytest.mark.parametrize("case", list(_cases()))
def test_input_rejections_happen_before_any_output(modules, case):
    (op, cfg, scratch), kw = _cases()[case]
    results = {}
    for name, m in modules.items():
        r = _fire(m, op, cfg, scratch, **dict(kw))
        assert r.status == H.CONTRACT_VIOLATION, (name, r)
        assert r.acquire_calls == 0 and r.seal_calls == 0 and r.release_calls == 0, (name, r)
        assert r.sealed_count == 0
        results[name] = (r.status, r.acquire_calls, r.input_batch_requests)
    assert len(set(results.values())) == 1, results


def test_duplicate_port_rejected(modules):
    direct2 = (DIRECT, H.direct_config(2, 2, 2, 2), 32)
    for name, m in modules.items():
        ks, tr = _host_inputs()
        out = H.aligned((8,), np.complex64)
        with m.instance(direct2[0], direct2[1]) as inst:
            r = inst.fire([(ks, H.TYPE_KSPACE, 0), (tr, H.TYPE_TRAJECTORY, 0)], out, H.TYPE_COIL_IMAGE,
                          scratch_bytes=32)
        assert r.status == H.CONTRACT_VIOLATION and r.acquire_calls == 0, name


def test_invalid_output_grant_is_released_unsealed(modules):
    # provider_tests.cpp:689-705
    for name, m in modules.items():
        r = _fire(m, DIRECT, H.direct_config(2, 2, 2, 2), 32, corrupt_output_type=True)
        assert r.status == H.CONTRACT_VIOLATION, name
        assert (r.acquire_calls, r.map_calls, r.seal_calls, r.release_calls) == (1, 1, 0, 1), name


def test_coil_combine_contract(native):
    m = H.ProviderModule(native.COIL_COMBINE_PLUGIN)
    try:
        assert m.provider_id == "org.kspacejet.coil-combine"
        assert m.digest_hex == "ba4f619047391419c8ffc42220ace7d888f047c9e2fd64aaeb78d9093191aed5"
        assert [o.id for o in m.operators] == ["coil_combine_rss"]
        assert m.operators[0].max_output_bytes == 1024 * 1024 and m.operators[0].max_inputs == 1
        assert m.try_create("coil_combine_rss", H.rss_config(2, 2, 2))[:2] == (0, True)
        for bad in ['{"channels":2,"rows":2,"cols":2}', '{"channels":0,"cols":2,"rows":2}',
                    '{"channels":2,"cols":513,"rows":2}', '{"channels":2,"cols":2,"rows":2} ']:
            assert m.try_create("coil_combine_rss", bad)[0] == H.INVALID_ARGUMENT
        x = H.aligned((2, 2, 2), np.complex64)
        out = H.aligned((2, 2), np.float32)
        with m.instance("coil_combine_rss", H.rss_config(2, 2, 2)) as inst:
            # coil_combine_provider_tests.cpp:322-338: wrong input identity -> no grant
            r = inst.fire([(x, H.TYPE_COIL_IMAGE, 0)], out, H.TYPE_IMAGE, corrupt_input_type=1)
            assert r.status == H.CONTRACT_VIOLATION and r.acquire_calls == 0
        with m.instance("coil_combine_rss", H.rss_config(2, 2, 2)) as inst:
            # :340-353: wrong output identity -> grant acquired, released, unsealed
            r = inst.fire([(x, H.TYPE_COIL_IMAGE, 0)], out, H.TYPE_IMAGE, corrupt_output_type=True)
            assert r.status == H.CONTRACT_VIOLATION and r.acquire_calls == 1 and r.seal_calls == 0
    finally:
        m.close()


def kb_config(channels=2, image=32, grid=64, width=4, samples=64, dcf="radial_analytic_ramp"):
    return (f'{{"channels":{channels},"density_compensation":"{dcf}","grid_cols":{grid},"grid_rows":{grid},'
            f'"image_cols":{image},"image_rows":{image},"kernel_width":{width},"sample_count":{samples},'
            f'"trajectory_units":"radians_per_pixel"}}')


def test_kaiser_bessel_plugin_descriptor_and_configs(native):
    import hashlib

    m = H.ProviderModule(native.KB_PLUGIN)
    try:
        ids = ["radial_kb_gridding_reconstruct", "radial_kb_gridding_rss"]
        assert m.provider_id == "org.kspacejet.gb300-noncartesian-recon"
        fields = ["kspacejet.provider-bundle", m.provider_id] + ids
        assert m.digest_hex == hashlib.sha256(b"".join(f.encode() + b"\0" for f in fields)).hexdigest()
        assert [o.id for o in m.operators] == ids
        assert all(o.max_scratch_bytes == 0 and o.max_in_flight == 1 for o in m.operators)
        for op in ids:
            assert m.try_create(op, kb_config())[:2] == (0, True)
            assert m.try_create(op, kb_config(grid=384, image=192, channels=32, samples=13056))[:2] == (0, True)
            assert m.try_create(op, kb_config(dcf="none"))[:2] == (0, True)
            for bad in [kb_config(width=5), kb_config(width=10), kb_config(grid=20), kb_config(grid=32, image=64),
                        kb_config(dcf="pipe_menon"), kb_config(channels=65), kb_config(grid=1024, image=512),
                        kb_config().replace('"grid_cols"', '"grid_colz"')]:
                assert m.try_create(op, bad)[0] == H.INVALID_ARGUMENT, bad
    finally:
        m.close()
