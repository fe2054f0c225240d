"""ksj_gpu_direct_adjoint_static (direct NUDFT adjoint with static device
scratch, no allocation) through the C ABI, against ksj_gpu_direct_adjoint.

Collected last so it also runs after every other GPU test in one process;
it passes alone in a fresh process as well.  Both entry points launch the same
kernels, so the outputs are expected to agree to the tolerance below (they are
in fact bit-identical).
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

REL_L2_TOL = 1e-6  # relative L2 between the two entry points
OK, ERROR_WORKSPACE = 0, 4


def _lib():
    from kspacejet_gb300 import gpu

    L = gpu.lib()  # raises if the CUDA library is not built
    u32, vp = ctypes.c_uint32, ctypes.c_void_p
    L.ksj_gpu_direct_static_scratch_bytes.restype = ctypes.c_size_t
    L.ksj_gpu_direct_static_scratch_bytes.argtypes = []
    L.ksj_gpu_direct_adjoint_static.restype = ctypes.c_int32
    L.ksj_gpu_direct_adjoint_static.argtypes = [u32, u32, ctypes.c_double, ctypes.c_double, u32, u32, vp, vp, vp,
                                                vp]
    L.ksj_gpu_direct_workspace_bytes.restype = ctypes.c_size_t
    L.ksj_gpu_direct_workspace_bytes.argtypes = [u32, u32, u32]
    L.ksj_gpu_direct_adjoint.restype = ctypes.c_int32
    L.ksj_gpu_direct_adjoint.argtypes = [u32, u32, ctypes.c_double, ctypes.c_double, u32, u32, vp, vp, vp, vp,
                                         ctypes.c_size_t, vp]
    return L


def _inputs(channels, samples, seed):
    rng = np.random.default_rng(seed)
    ks = (rng.standard_normal((channels, samples)) + 1j * rng.standard_normal((channels, samples))).astype(
        np.complex64)
    traj = rng.uniform(-np.pi, np.pi, size=(samples, 2)).astype(np.float32)
    return torch.from_numpy(ks).cuda(), torch.from_numpy(traj).cuda()


def _workspace_call(L, rows, cols, ks, traj, stream):
    c, m = ks.shape
    ws = torch.empty(L.ksj_gpu_direct_workspace_bytes(rows, cols, c), dtype=torch.uint8, device="cuda")
    out = torch.empty((rows, cols, c), dtype=torch.complex64, device="cuda")
    st = L.ksj_gpu_direct_adjoint(rows, cols, (rows - 1) / 2.0, (cols - 1) / 2.0, c, m, ks.data_ptr(),
                                  traj.data_ptr(), out.data_ptr(), ws.data_ptr(), ws.numel(), stream)
    assert st == OK
    return out


def _static_call(L, rows, cols, ks, traj, out, stream):
    c, m = ks.shape
    return L.ksj_gpu_direct_adjoint_static(rows, cols, (rows - 1) / 2.0, (cols - 1) / 2.0, c, m, ks.data_ptr(),
                                           traj.data_ptr(), out.data_ptr(), stream)


def _rel_l2(a, b):
    a = a.cpu().numpy().astype(np.complex128)
    b = b.cpu().numpy().astype(np.complex128)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_static_scratch_matches_workspace_entry_point():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = _lib()
    assert L.ksj_gpu_direct_static_scratch_bytes() == 8 << 20
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row of different shapes (the second reuses the scratch
    # the first left behind), then the largest intermediate the array holds
    cases = [(48, 40, 6, 700, 1), (64, 64, 16, 1200, 2), (128, 128, 64, 96, 3)]
    for rows, cols, channels, samples, seed in cases:
        ks, traj = _inputs(channels, samples, seed)
        want = _workspace_call(L, rows, cols, ks, traj, stream)
        got = torch.full((rows, cols, channels), complex(float("nan"), float("nan")), dtype=torch.complex64,
                         device="cuda")
        assert _static_call(L, rows, cols, ks, traj, got, stream) == OK
        torch.cuda.synchronize()
        err = _rel_l2(got, want)
        assert err <= REL_L2_TOL, (rows, cols, channels, err)


def test_static_scratch_call_allocates_no_device_memory():
    """The property the entry point exists for: after a first call on the
    device, a further call changes the device's free memory by nothing
    (cudaMemGetInfo read around it, no torch allocation in between)."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = _lib()
    stream = torch.cuda.current_stream().cuda_stream
    ks, traj = _inputs(8, 512, 5)
    out = torch.empty((64, 64, 8), dtype=torch.complex64, device="cuda")
    assert _static_call(L, 64, 64, ks, traj, out, stream) == OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _static_call(L, 64, 64, ks, traj, out, stream) == OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_static_scratch_rejects_oversize():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = _lib()
    stream = torch.cuda.current_stream().cuda_stream
    ks, traj = _inputs(65, 8, 4)
    out = torch.zeros((128, 128, 65), dtype=torch.complex64, device="cuda")
    # 128 x 128 x 65 x 8 B is above the 8 MiB array: refused before any device work
    st = _static_call(L, 128, 128, ks, traj, out, stream)
    assert st == ERROR_WORKSPACE
    assert b"workspace" in L.ksj_gpu_status_string(st)
    torch.cuda.synchronize()
    assert not bool(out.abs().amax() > 0)
