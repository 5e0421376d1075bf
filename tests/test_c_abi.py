"""The C ABI library on the CPU: it builds, loads, exports every symbol the
header declares, and its host-side CTF physics matches the reference's known
answers.  No compute on a GPU here."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import REPO, golden

HEADER = os.path.join(REPO, "include", "guanaco_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"GNC_API\s+[\w\s\*]+?\b(gnc_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from guanaco_gb300 import _lib

    return _lib.load()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "gnc_reconstruct" in names and "gnc_correct" in names and "gnc_fbp_execute" in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(lib):
    from guanaco_gb300 import _lib

    path = _lib.lib_path()
    handle = ctypes.CDLL(path)
    for name in declared_symbols():
        assert hasattr(handle, name), f"{name} declared in the header but not exported"
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"


def test_ctf_known_answers(lib):
    from guanaco_gb300 import detail

    g = golden("ctf_kat")
    l = detail.get_electron_wavelength(300000)
    assert l == pytest.approx(float(g["wavelength_300kV"]), rel=1e-15)
    assert detail.get_defocus_spread(2.7e7, 1e-6, 1e-6, 1e-6) == pytest.approx(
        float(g["defocus_spread"]), rel=1e-15)
    assert detail.q_to_Q(10, l, 2.7e7) == pytest.approx(float(g["q_to_Q"]), rel=1e-15)
    assert detail.Q_to_q(float(g["q_to_Q"]), l, 2.7e7) == pytest.approx(float(g["Q_to_q"]), rel=1e-15)
    assert detail.df_to_D(20000, l, 2.7e7) == pytest.approx(float(g["df_to_D"]), rel=1e-15)
    assert detail.D_to_df(float(g["df_to_D"]), l, 2.7e7) == pytest.approx(float(g["D_to_df"]), rel=1e-15)
    env = detail.CTF(l, 20000, 2.7e7, 0, 0, 1, 1e-3, 0)
    np.testing.assert_allclose(env.get_Es([10.0], [0.0]), g["Es_q10"], rtol=1e-14)
    np.testing.assert_allclose(env.get_Et([10.0]), g["Et_q10"], rtol=1e-14)
    assert detail.CTF(l, 20000, 2.7e7).get_chi(10, 0) == pytest.approx(float(g["chi_q10"]), rel=1e-15)
    q, a = detail.get_q_and_theta(100, 100, 2)
    np.testing.assert_array_equal(q, g["q_grid"])
    np.testing.assert_array_equal(a, g["theta_grid"])
    full = detail.CTF(l, 20000, 2.7e7, 0, 0, 1, 0.1 / 1e3, 0.1)
    np.testing.assert_allclose(full.get_ctf(100, 100, 2), g["ctf_full"], rtol=0, atol=1e-13)
    simple = detail.CTF(l, 20000, 2.7e7, 0, 0, 0, 0, 0.1)
    np.testing.assert_array_equal(simple.get_ctf_simple(100, 100, 2), g["ctf_simple"])
    np.testing.assert_array_equal(simple.get_ctf_simple_real(100, 100, 2), g["ctf_simple_real"])
    np.testing.assert_array_equal(simple.get_ctf_simple_imag(100, 100, 2), g["ctf_simple_imag"])
    astig = detail.CTF(l, 25000, 2.7e7, 800, 0.3, 0, 0, 0.05)
    np.testing.assert_array_equal(astig.get_ctf_simple(90, 64, 1.5), g["ctf_simple_astig_90x64"])


def test_ctf_reference_test_formulas(lib):
    """The reference's tests/test_ctf.py compares against textbook formulas
    (De Graef eq. 10.9-10.53); restated here from the physics."""
    from guanaco_gb300 import detail
    from scipy.constants import c, e, h, m_e

    V = 300000.0
    l_py = h * c / np.sqrt((e * V) ** 2 + 2 * m_e * e * V * c ** 2) * 1e10
    l = detail.get_electron_wavelength(V)
    assert l == pytest.approx(l_py, rel=1e-6)
    q, Cs, df = 10.0, 2.7e7, 20000.0
    chi = np.pi * (Cs * l ** 3 * q ** 4 / 2 - l * df * q ** 2)
    assert detail.CTF(l, df, Cs).get_chi(q, 0) == pytest.approx(chi, rel=1e-12)
    # FFT-ordered grid equals fftshift of the centred grid
    qg, ag = detail.get_q_and_theta(100, 100, 2)
    y, x = np.mgrid[0:100, 0:100]
    y = ((y - 50) / 100) / 2
    x = ((x - 50) / 100) / 2
    np.testing.assert_allclose(qg, np.fft.fftshift(np.sqrt(x * x + y * y)), atol=1e-12)
    np.testing.assert_allclose(ag, np.fft.fftshift(np.arctan2(y, x)), atol=1e-12)


def test_device_path_is_explicit(lib):
    from guanaco_gb300 import detail

    with pytest.raises(RuntimeError, match="device path only"):
        detail.recon(np.zeros((3, 8), np.float32), np.zeros((8, 8), np.float32),
                     np.zeros(3, np.float32), 4.0)
    with pytest.raises(RuntimeError, match="ASSERT"):
        detail.recon(np.zeros((3, 8), np.float32), np.zeros((8, 7), np.float32),
                     np.zeros(3, np.float32), 4.0, device="gpu")
    with pytest.raises(RuntimeError, match="ASSERT"):
        detail.corr(np.zeros((4, 6), np.float32), np.zeros((2, 4, 5), np.complex64),
                    np.zeros((2, 4, 6), np.float32), "gpu")
    assert detail.eDevice.convert("gpu") == detail.gpu
    assert detail.eDevice.convert(0) == detail.cpu
    with pytest.raises(ValueError):
        detail.eDevice.convert("tpu")


def test_invalid_config_rejected_before_any_device_work(lib):
    from guanaco_gb300 import _lib

    cfg = _lib.GncConfig()
    cfg.device = 1
    cfg.num_pixels = 16
    cfg.num_angles = 3
    cfg.num_defocus = 2
    cfg.grid_height = 16
    cfg.grid_width = 16
    cfg.pixel_size = 1.0
    cfg.min_defocus = 5.0
    cfg.max_defocus = 5.0  # num_defocus > 1 needs max > min (reconstructor.cu:250)
    ang = np.zeros(3, np.float32)
    cfg.angles = ang.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    buf = np.zeros(16 * 3 * 2, np.float32)
    rec = np.zeros((16, 16), np.float32)
    st = lib.gnc_reconstruct(ctypes.byref(cfg), buf.ctypes.data, rec.ctypes.data)
    assert st == _lib.GNC_ERR_INVALID_ARGUMENT
    assert b"max_defocus > c->min_defocus" in lib.gnc_last_error()
    cfg.device = 0
    assert lib.gnc_reconstruct(ctypes.byref(cfg), buf.ctypes.data, rec.ctypes.data) == \
        _lib.GNC_ERR_UNSUPPORTED


def test_unsupported_sizes_reported(lib):
    from guanaco_gb300 import FbpPlan, _lib

    with pytest.raises(_lib.GncError) as ei:  # odd width cannot use the packed real transform
        FbpPlan(3, 8, 17, np.zeros(3, np.float32), correct=True, num_defocus=1,
                slab_defocus=[1e4], energy=300, spherical_aberration=2.7)
    assert ei.value.status == _lib.GNC_ERR_UNSUPPORTED
    with pytest.raises(_lib.GncError) as ei:  # 2 * 4099 has a prime factor > 16
        FbpPlan(3, 8, 4099, np.zeros(3, np.float32), correct=False)
    assert ei.value.status == _lib.GNC_ERR_UNSUPPORTED


# Each argument check of the reference's pybind entry points
# (src/guanaco/detail/ext/reconstruct.h:46-58, correct.h:38-54) raises the same
# "ASSERT (condition) failed" RuntimeError here, before any device work.
_F = np.float32
_RECON_CASES = [
    ((np.zeros(8, _F), np.zeros((8, 8), _F), np.zeros(3, _F)),
     "sinogram.ndim() == 2 || sinogram.ndim() == 3"),
    ((np.zeros((3, 8), _F), np.zeros(64, _F), np.zeros(3, _F)), "reconstruction.ndim() == 2"),
    ((np.zeros((3, 8), _F), np.zeros((8, 8), _F), np.zeros((3, 1), _F)), "angles.ndim() == 1"),
    ((np.zeros((3, 8), _F), np.zeros((8, 8), _F), np.zeros(4, _F)),
     "sinogram.shape()[0] == angles.size()"),
    ((np.zeros((3, 8), _F), np.zeros((7, 8), _F), np.zeros(3, _F)),
     "sinogram.shape()[1] == reconstruction.shape()[0]"),
    ((np.zeros((3, 8), _F), np.zeros((8, 7), _F), np.zeros(3, _F)),
     "sinogram.shape()[1] == reconstruction.shape()[1]"),
    ((np.zeros((2, 3, 8), _F), np.zeros((8, 8), _F), np.zeros(4, _F)),
     "sinogram.shape()[1] == angles.size()"),
    ((np.zeros((2, 3, 8), _F), np.zeros((7, 8), _F), np.zeros(3, _F)),
     "sinogram.shape()[2] == reconstruction.shape()[0]"),
    ((np.zeros((2, 3, 8), _F), np.zeros((8, 7), _F), np.zeros(3, _F)),
     "sinogram.shape()[2] == reconstruction.shape()[1]"),
]


@pytest.mark.parametrize("args,cond", _RECON_CASES)
def test_recon_argument_checks(lib, args, cond):
    from guanaco_gb300 import detail

    sino, rec, ang = args
    with pytest.raises(RuntimeError) as e:
        detail.recon(sino, rec, ang, 4.0, device="gpu")
    assert str(e.value) == f"ASSERT ({cond}) failed"


_C = np.complex64
_CORR_CASES = [
    ((np.zeros(6, _F), np.zeros((4, 6), _C), np.zeros((4, 6), _F)), "image.ndim() == 2"),
    ((np.zeros((4, 6), _F), np.zeros(6, _C), np.zeros((4, 6), _F)),
     "ctf.ndim() == 2 || ctf.ndim() == 3"),
    ((np.zeros((4, 6), _F), np.zeros((2, 4, 6), _C), np.zeros((4, 6), _F)),
     "rec.ndim() == image.ndim() + (ctf.ndim() - 2)"),
    ((np.zeros((4, 6), _F), np.zeros((0, 4, 6), _C), np.zeros((0, 4, 6), _F)), "num_ctf > 0"),
    ((np.zeros((0, 6), _F), np.zeros((0, 6), _C), np.zeros((0, 6), _F)), "ysize > 0"),
    ((np.zeros((4, 0), _F), np.zeros((4, 0), _C), np.zeros((4, 0), _F)), "xsize > 0"),
    ((np.zeros((4, 6), _F), np.zeros((5, 6), _C), np.zeros((4, 6), _F)),
     "ctf.shape()[ctf.ndim() - 2] == ysize"),
    ((np.zeros((4, 6), _F), np.zeros((4, 5), _C), np.zeros((4, 6), _F)),
     "ctf.shape()[ctf.ndim() - 1] == xsize"),
    ((np.zeros((4, 6), _F), np.zeros((4, 6), _C), np.zeros((5, 6), _F)),
     "rec.shape()[rec.ndim() - 2] == ysize"),
    ((np.zeros((4, 6), _F), np.zeros((4, 6), _C), np.zeros((4, 5), _F)),
     "rec.shape()[rec.ndim() - 1] == xsize"),
]


@pytest.mark.parametrize("args,cond", _CORR_CASES)
def test_corr_argument_checks(lib, args, cond):
    from guanaco_gb300 import detail

    image, ctf, rec = args
    with pytest.raises(RuntimeError) as e:
        detail.corr(image, ctf, rec, device="gpu")
    assert str(e.value) == f"ASSERT ({cond}) failed"


def test_host_alloc_argument_checks(lib):
    """gnc_host_alloc rejects a null result pointer and a zero size before any
    CUDA call; gnc_host_free of null is a no-op."""
    import ctypes

    from guanaco_gb300 import _lib

    ptr = ctypes.c_void_p(1234)
    assert lib.gnc_host_alloc(0, ctypes.byref(ptr)) == _lib.GNC_ERR_INVALID_ARGUMENT
    assert "ASSERT" in lib.gnc_last_error().decode()
    assert lib.gnc_host_alloc(16, None) == _lib.GNC_ERR_INVALID_ARGUMENT
    assert lib.gnc_host_free(None) == _lib.GNC_OK


def test_noalloc_limits_are_checked_on_the_host(lib):
    """The allocation-free entry point rejects requests beyond its static
    scratch before any CUDA call, and checks each factor of
    num_defocus * num_angles * num_pixels on its own: a product that wraps
    around 2^64 (here to 0) is still rejected instead of reaching the device."""
    import ctypes

    from guanaco_gb300 import _lib

    ang = np.zeros(1024, np.float32)
    cfg = _lib.GncConfig()
    cfg.device = 1
    cfg.gpu_index = -1
    cfg.num_pixels = 4096
    cfg.num_angles = 1024
    cfg.num_defocus = 1 << 42  # 4096 * 1024 * 2^42 == 2^64
    cfg.grid_height = 16
    cfg.grid_width = 16
    cfg.pixel_size = 1.0
    cfg.centre = 2048.0
    cfg.min_defocus = -1.0
    cfg.max_defocus = 1.0
    cfg.angles = ang.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    fake = ctypes.c_void_p(16)  # never dereferenced: the checks come first
    st = lib.gnc_reconstruct_device_noalloc(ctypes.byref(cfg), fake, fake, None)
    assert st == _lib.GNC_ERR_INVALID_ARGUMENT
    assert b"static scratch" in lib.gnc_last_error()
    cfg.num_defocus = 2  # 2 * 4 Mi floats
    assert lib.gnc_reconstruct_device_noalloc(ctypes.byref(cfg), fake, fake,
                                              None) == _lib.GNC_ERR_INVALID_ARGUMENT
    cfg.num_pixels = 34  # 2 * 34 has the prime factor 17: unsupported, as for
    cfg.num_defocus = 1  # the allocating entry point
    assert lib.gnc_reconstruct_device_noalloc(ctypes.byref(cfg), fake, fake,
                                              None) == _lib.GNC_ERR_UNSUPPORTED
    cfg.device = 0
    assert lib.gnc_reconstruct_device_noalloc(ctypes.byref(cfg), fake, fake,
                                              None) == _lib.GNC_ERR_UNSUPPORTED
