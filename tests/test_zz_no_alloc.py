"""The allocation-free single-slice reconstruction.

gnc_reconstruct_device_noalloc serves callers that cannot allocate device
memory inside a call (a fixed device-memory budget owned by the application,
a real-time loop that must not touch the allocator).  It keeps its scratch in
static device arrays instead.  These tests
call it through the C ABI and check it against gnc_reconstruct_device -- the
allocating entry point -- within the FP32 parity tolerance, for two calls in a
row (the second must not see anything the first left in the shared scratch),
and check that requests beyond the static scratch are rejected.

This file runs last (its name sorts last) and also passes alone in a fresh
process: its first call does the per-device set-up.  The cases reach the
advertised limits (a 4096-pixel detector with exactly 4 Mi sinogram floats),
a volume narrower than the detector, and the reference's own recorded
reconstructions.
"""
import ctypes

import numpy as np
import pytest

from conftest import golden, golden_names

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-4


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def env():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from guanaco_gb300 import _lib

    return torch, _lib, _lib.load()


def config(_lib, N, T, D, Z, X, angles, centre, mn=0.0, mx=0.0):
    c = _lib.GncConfig()
    c.device = 1
    c.gpu_index = -1
    c.num_pixels = N
    c.num_angles = T
    c.num_defocus = D
    c.grid_height = Z
    c.grid_width = X
    c.pixel_size = 1.0
    c.centre = centre
    c.min_defocus = mn
    c.max_defocus = mx
    c.angles = angles.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    return c


# (N, T, D, Z, X): the last two reach the limits (4096 pixels, 1024 tilts,
# D * T * N == 4194304 floats); (256, ..., 200) has X != N.
@pytest.mark.parametrize("N,T,D,Z,X", [(256, 41, 3, 128, 256), (100, 21, 1, 100, 100),
                                       (1024, 61, 10, 64, 1024), (256, 31, 4, 90, 200),
                                       (4096, 1024, 1, 24, 4096), (4096, 256, 4, 16, 3000)])
def test_noalloc_matches_allocating_entry_point(env, N, T, D, Z, X):
    torch, _lib, L = env
    ang = np.deg2rad(np.linspace(-60, 60, T)).astype(np.float32)
    rng = np.random.default_rng(N + T)
    mn, mx = (-float(N) / 2, float(N) / 2) if D > 1 else (0.0, 0.0)
    cfg = config(_lib, N, T, D, Z, X, ang, N / 2.0, mn, mx)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):  # two calls in a row, different data
        sino = torch.from_numpy(rng.standard_normal((D, T, N)).astype(np.float32)).cuda()
        ref = torch.empty((Z, X), dtype=torch.float32, device="cuda")
        out = torch.full((Z, X), float("nan"), dtype=torch.float32, device="cuda")
        _lib.check(L.gnc_reconstruct_device(ctypes.byref(cfg), sino.data_ptr(), ref.data_ptr(),
                                            stream))
        _lib.check(L.gnc_reconstruct_device_noalloc(ctypes.byref(cfg), sino.data_ptr(),
                                                    out.data_ptr(), stream))
        torch.cuda.synchronize()
        assert rel_l2(out.cpu().numpy(), ref.cpu().numpy()) < FP32_TOL, f"call {call}"


@pytest.mark.parametrize("name", golden_names("recon_"))
def test_noalloc_matches_reference_goldens(env, name):
    """The reference's own recorded reconstructions (its CPU path compiled
    from source), through the allocation-free entry point."""
    torch, _lib, L = env
    g = golden(name)
    sino = np.ascontiguousarray(g["sino"], np.float32)
    if sino.ndim == 2:
        sino = sino[None]
    D, T, N = sino.shape
    Z, X = g["rec"].shape
    ang = np.ascontiguousarray(g["angles"], np.float32)
    cfg = config(_lib, N, T, D, Z, X, ang, float(g["centre"]), float(g["min_defocus"]),
                 float(g["max_defocus"]))
    cfg.pixel_size = float(g["pixel_size"])
    d_sino = torch.from_numpy(sino).cuda()
    out = torch.full((Z, X), float("nan"), dtype=torch.float32, device="cuda")
    for _ in range(2):
        _lib.check(L.gnc_reconstruct_device_noalloc(ctypes.byref(cfg), d_sino.data_ptr(),
                                                    out.data_ptr(), None))
        torch.cuda.synchronize()
        assert rel_l2(out.cpu().numpy(), g["rec"]) < FP32_TOL


def test_noalloc_rejects_requests_beyond_its_scratch(env):
    torch, _lib, L = env
    T = 1100  # more tilts than the static geometry table holds
    ang = np.zeros(T, np.float32)
    cfg = config(_lib, 64, T, 1, 64, 64, ang, 32.0)
    buf = torch.zeros((T, 64), dtype=torch.float32, device="cuda")
    rec = torch.zeros((64, 64), dtype=torch.float32, device="cuda")
    st = L.gnc_reconstruct_device_noalloc(ctypes.byref(cfg), buf.data_ptr(), rec.data_ptr(), None)
    assert st == _lib.GNC_ERR_INVALID_ARGUMENT
    assert b"static scratch" in L.gnc_last_error()
    cfg = config(_lib, 4096, 61, 20, 64, 64, np.zeros(61, np.float32), 32.0, -1.0, 1.0)
    st = L.gnc_reconstruct_device_noalloc(ctypes.byref(cfg), buf.data_ptr(), rec.data_ptr(), None)
    assert st == _lib.GNC_ERR_INVALID_ARGUMENT  # 20 * 61 * 4096 floats > 4 Mi
    # 2 * num_pixels with a prime factor above 16: unsupported, as for the
    # allocating entry point
    cfg = config(_lib, 34, 8, 1, 34, 34, np.zeros(8, np.float32), 17.0)
    st = L.gnc_reconstruct_device_noalloc(ctypes.byref(cfg), buf.data_ptr(), rec.data_ptr(), None)
    assert st == _lib.GNC_ERR_UNSUPPORTED
    st = L.gnc_reconstruct_device(ctypes.byref(cfg), buf.data_ptr(), rec.data_ptr(), None)
    assert st == _lib.GNC_ERR_UNSUPPORTED
