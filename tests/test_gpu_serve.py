"""The request loop (include/ksj_serve.h): requests of uneven shape are
batched by class into ragged multi-frame calls that run concurrently, and
each result equals the same gridding call made alone, byte for byte; a
request with a bad input fails alone; per-request caps reject; the
device-byte cap limits how many requests are in flight."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from kspacejet_gb300 import gpu, serve  # noqa: E402
from kspacejet_gb300.synth import golden_angle_radial  # noqa: E402

pytestmark = pytest.mark.gpu


def _request(readout, spokes, coils, seed, output=serve.OUTPUT_RSS, trajectory_id=0):
    rng = np.random.default_rng(seed)
    traj = golden_angle_radial(readout, spokes).astype(np.float32).reshape(-1, 2)
    m = traj.shape[0]
    ks = (rng.standard_normal((coils, m)) + 1j * rng.standard_normal((coils, m))).astype(np.complex64)
    return serve.Request(image=readout // 2, grid=readout, kspace=ks, trajectory=traj, output=output,
                         trajectory_id=trajectory_id)


def _alone(r: serve.Request) -> np.ndarray:
    c, m = r.kspace.shape
    out_mode = gpu.OUTPUT_RSS if r.output == serve.OUTPUT_RSS else gpu.OUTPUT_COIL_MAJOR
    g = gpu.kb_gridding(r.image, r.grid, c, m, 1, width=r.width, output=out_mode, dcf=r.dcf)
    ks = torch.from_numpy(r.kspace).cuda()
    tr = torch.from_numpy(r.trajectory).cuda()
    out = g.new_output()
    ws = g.new_workspace()
    g.run(ks, tr, out, ws)
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(r.output_shape())


def _mix():
    shapes = [(128, 64, 8), (256, 101, 12), (384, 160, 32), (128, 805, 4), (512, 96, 16), (256, 33, 1),
              (384, 64, 24), (128, 200, 32)]
    reqs = []
    for i, (ro, sp, co) in enumerate(shapes):
        out = serve.OUTPUT_COIL_MAJOR if i % 3 == 2 else serve.OUTPUT_RSS
        reqs.append(_request(ro, sp, co, seed=10 + i, output=out, trajectory_id=(ro * 1000 + sp) if i % 2 else 0))
    return reqs


def test_concurrent_requests_equal_alone():
    reqs = _mix()
    with serve.Server(slots=4) as s:
        tickets = [s.submit(r) for r in reqs]
        outs = [s.wait(t, timeout_ms=60000) for t in tickets]
        st = s.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0 and st["rejected"] == 0
    assert st["peak_in_flight"] >= 1
    for r, got in zip(reqs, outs):
        want = _alone(r)
        assert got.shape == want.shape
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_pinned_requests_and_trajectory_reuse():
    base = _request(256, 120, 8, seed=3, trajectory_id=77)
    reqs = []
    for i in range(6):
        ks = torch.from_numpy(np.roll(base.kspace, i, axis=1)).pin_memory()
        tr = torch.from_numpy(base.trajectory).pin_memory()
        out = torch.empty((128, 128), dtype=torch.float32).pin_memory()
        r = serve.Request(image=128, grid=256, kspace=ks.numpy(), trajectory=tr.numpy(), trajectory_id=77,
                          pinned=True, out=out.numpy())
        r._keep = (ks, tr, out)
        reqs.append(r)
    with serve.Server(slots=3) as s:
        tickets = [s.submit(r) for r in reqs]
        outs = [s.wait(t, timeout_ms=60000).copy() for t in tickets]
    for r, got in zip(reqs, outs):
        assert np.array_equal(got, _alone(r))


def test_caps_reject_and_admission_limits_in_flight():
    big = _request(256, 64, 16, seed=5)
    with serve.Server(slots=4, max_channels=8) as s:
        with pytest.raises(gpu.GpuError):
            s.submit(big)
        assert s.stats()["rejected"] == 1
    # a device cap that holds one request's bytes: requests still all complete,
    # one at a time
    reqs = [_request(256, 64, 4, seed=20 + i) for i in range(4)]
    g = gpu.kb_gridding(128, 256, 4, reqs[0].kspace.shape[1], 1)
    one = g.workspace_bytes() + reqs[0].kspace.nbytes + reqs[0].trajectory.nbytes + 128 * 128 * 4
    with serve.Server(slots=4, device_memory_cap=one + one // 2) as s:
        tickets = [s.submit(r) for r in reqs]
        outs = [s.wait(t, timeout_ms=60000) for t in tickets]
        st = s.stats()
    assert st["completed"] == 4 and st["peak_in_flight"] == 1
    assert st["peak_device_bytes"] <= one + one // 2
    for r, got in zip(reqs, outs):
        assert np.array_equal(got, _alone(r))


def test_requests_batch_into_ragged_calls_and_equal_alone():
    """A burst of one class (grid 256) with uneven spokes and coils leaves in
    a few ragged calls, not one call per request; each result still equals
    its own call made alone, byte for byte; the serial configuration
    (one slot, batches of one) gives the same bytes."""
    shapes = [(256, 64 + 37 * i, 4 + (5 * i) % 29) for i in range(12)]
    reqs = [_request(ro, sp, co, seed=40 + i, output=serve.OUTPUT_COIL_MAJOR if i % 4 == 3 else serve.OUTPUT_RSS)
            for i, (ro, sp, co) in enumerate(shapes)]
    with serve.Server(slots=2, max_batch_frames=8) as s:
        tickets = [s.submit(r) for r in reqs]
        outs = [s.wait(t, timeout_ms=60000).copy() for t in tickets]
        st = s.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["batched_frames"] == len(reqs)
    assert st["batches"] < len(reqs), st
    # the same with page-locked inputs read in place by the kernels (and the
    # pageable ones staged in page-locked memory first)
    pinned = []
    for r in reqs:
        ks = torch.from_numpy(r.kspace).pin_memory()
        tr = torch.from_numpy(r.trajectory).pin_memory()
        dt = torch.float32 if r.output == serve.OUTPUT_RSS else torch.complex64
        out = torch.empty(r.output_shape(), dtype=dt).pin_memory()
        q = serve.Request(image=r.image, grid=r.grid, kspace=ks.numpy(), trajectory=tr.numpy(), output=r.output,
                          pinned=True, out=out.numpy())
        q._keep = (ks, tr, out)
        pinned.append(q)
    with serve.Server(slots=2, max_batch_frames=8, read_inputs_in_place=True) as s:
        tickets = [s.submit(r) for r in pinned + reqs[:3]]
        in_place = [s.wait(t, timeout_ms=60000).copy() for t in tickets]
        assert s.stats()["failed"] == 0
    with serve.Server(slots=1, max_batch_frames=1) as s:
        tickets = [s.submit(r) for r in reqs]
        serial = [s.wait(t, timeout_ms=60000).copy() for t in tickets]
        assert s.stats()["batches"] == len(reqs)
    for i, (r, got, one) in enumerate(zip(reqs, outs, serial)):
        want = _alone(r)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
        assert np.array_equal(one.view(np.uint32), want.view(np.uint32))
        assert np.array_equal(in_place[i].view(np.uint32), want.view(np.uint32))
        if i < 3:
            assert np.array_equal(in_place[len(reqs) + i].view(np.uint32), want.view(np.uint32))


def test_bad_request_fails_alone_in_its_batch():
    """A non-finite sample in one request of a batch fails that request
    (KSJ_GPU_ERROR_NONFINITE_INPUT) and no other."""
    reqs = [_request(128, 64 + 8 * i, 8, seed=70 + i) for i in range(5)]
    reqs[2].kspace[3, 17] = complex(float("nan"), 0.0)
    with serve.Server(slots=1, max_batch_frames=8) as s:
        tickets = [s.submit(r) for r in reqs]
        results = []
        for t in tickets:
            try:
                results.append(s.wait(t, timeout_ms=60000).copy())
            except gpu.GpuError as e:
                results.append(e)
        st = s.stats()
    assert st["failed"] == 1 and st["completed"] == 4
    assert isinstance(results[2], gpu.GpuError)
    for i in (0, 1, 3, 4):
        assert np.array_equal(results[i].view(np.uint32), _alone(reqs[i]).view(np.uint32))
