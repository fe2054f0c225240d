"""Failure paths of the plug-ins and the device waits, in the forms that
fault no GPU: failures are made on the host (a cancelled scan, an allocation
that a host-side hook refuses) or by a device wait on a count that nothing
will ever reach, bounded so that the kernel gives up, raises a status flag
and returns with the context still usable.

The reference pins its Provider fault modes with a fake Provider and a host
harness (tests/unit/libs/recon/kspacejet-recon-runtime/
synchronous_firing_lease_test_provider.cpp:8-59); the terminal protocol is
provider.h:676-694 (on_cancel emits nothing, a failed firing releases its
grants and seals nothing).
"""
import numpy as np
import pytest

H = pytest.importorskip("kspacejet_gb300.host")


@pytest.fixture(scope="module")
def recon(native):
    m = H.ProviderModule(native.NONCARTESIAN_PLUGIN)
    yield m
    m.close()


def _radial_inputs(channels=2, readout=64, spokes=16, seed=3):
    from kspacejet_gb300 import synth

    tr = synth.golden_angle_radial(readout, spokes)
    ks = synth.random_kspace(channels, tr.shape[0], seed=seed)
    return ks, tr


def _fire(inst, ks, tr, n, channels):
    out = H.aligned((n * n * channels,), np.complex64)
    r = inst.fire([(H.aligned_copy(ks), H.TYPE_KSPACE, 0), (H.aligned_copy(tr.ravel()), H.TYPE_TRAJECTORY, 1)], out,
                  H.TYPE_COIL_IMAGE, scratch_bytes=H.radial_scratch_bytes(n, n, tr.shape[0]))
    return r, out


def test_on_cancel_emits_nothing_without_a_device(recon):
    """on_cancel of a scan that never fired: accepted for a cancelled or a
    failed scan, refused for the normal-drain kind (that is on_scan_end's);
    there is no lease, so nothing can be acquired or sealed."""
    ks, tr = _radial_inputs()
    with recon.instance("radial_gridding_reconstruct", H.radial_config(2, 64, 64, tr.shape[0])) as inst:
        assert inst.cancel(H.SCAN_END_CANCELLED)[0] == H.OK
        assert inst.cancel(H.SCAN_END_FAILED)[0] == H.OK
        st, msg = inst.cancel(H.SCAN_END_NORMAL)
        assert st == H.INVALID_ARGUMENT and msg


@pytest.mark.gpu
def test_on_cancel_releases_the_device_memory_of_the_scan(recon, cuda):
    import torch

    ks, tr = _radial_inputs(channels=8, readout=256, spokes=64)
    cfg = H.radial_config(8, 256, 256, tr.shape[0])
    with recon.instance("radial_gridding_reconstruct", cfg) as inst:
        r, first = _fire(inst, ks, tr, 256, 8)
        assert r.status == H.OK
        torch.cuda.synchronize()
        free_before, _ = torch.cuda.mem_get_info()
        st, _ = inst.cancel(H.SCAN_END_CANCELLED)
        assert st == H.OK
        free_after, _ = torch.cuda.mem_get_info()
        # the firing's device buffers (k-space, trajectory, 2 MiB of images,
        # workspace) are freed
        assert free_after - free_before >= 256 * 256 * 8 * 8
        # a later firing of the same instance creates them again: same bytes
        r, again = _fire(inst, ks, tr, 256, 8)
        assert r.status == H.OK and r.seal_calls == 1
        assert again.tobytes() == first.tobytes()


@pytest.mark.gpu
def test_allocation_failure_fails_the_firing_and_releases_the_grant(recon, cuda):
    """A device allocation refused by the host-side hook: the firing fails
    with RESOURCE_EXHAUSTED, its output grant is released and nothing is
    sealed; the next firing (allocation succeeds) is normal."""
    from kspacejet_gb300 import gpu

    ks, tr = _radial_inputs()
    cfg = H.radial_config(2, 64, 64, tr.shape[0])
    with recon.instance("radial_gridding_reconstruct", cfg) as inst:
        gpu.lib().ksj_gpu_inject_allocation_failures(1)
        try:
            r, _ = _fire(inst, ks, tr, 64, 2)
        finally:
            gpu.lib().ksj_gpu_inject_allocation_failures(0)
        assert r.status == H.RESOURCE_EXHAUSTED
        assert r.seal_calls == 0 and r.sealed_count == 0
        assert r.acquire_calls == r.release_calls
        r, out = _fire(inst, ks, tr, 64, 2)
        assert r.status == H.OK and r.seal_calls == 1 and r.release_calls == 0


@pytest.mark.gpu
def test_segment_wait_runs_out_and_the_call_returns(native, cuda):
    """The row pass's per-list segment wait (lists over 32 entries are summed
    in segments that wait for their predecessors) pointed, by the test-only
    tuning field, at a count that never comes: every later segment gives up
    after 256 polls, KSJ_GPU_FLAG_WAIT_TIMEOUT comes back, the call returns,
    and the next normal call on the same workspace is clean and correct."""
    import ctypes

    import torch
    from kspacejet_gb300 import gpu, synth

    tr, ks = synth.dynamic_radial(1, 34, 384, 32, seed=7, image=192)
    g = gpu.kb_gridding(image=192, grid=384, channels=32, samples=tr.shape[1], frames=1, width=4,
                        output=gpu.OUTPUT_RSS)
    k = torch.from_numpy(np.ascontiguousarray(ks)).to(cuda)
    t = torch.from_numpy(np.ascontiguousarray(tr)).to(cuda)
    ws = g.new_workspace(cuda)
    want = g.new_output(cuda)
    g.run(k, t, want, ws)
    assert g.flags(ws) == 0
    for cg in (32, 16):  # the 32-coil register path and the shared-memory path
        tun = gpu.GriddingTuning(ctypes.sizeof(gpu.GriddingTuning), cg, 0, 0, 0, 0, 0, 0, 256)
        out = g.new_output(cuda)
        g.run(k, t, out, ws, tuning=tun)
        torch.cuda.synchronize()
        assert g.flags(ws) & gpu.FLAG_WAIT_TIMEOUT, cg
        again = g.new_output(cuda)
        g.run(k, t, again, ws)
        assert g.flags(ws) == 0
        assert again.cpu().numpy().tobytes() == want.cpu().numpy().tobytes()
