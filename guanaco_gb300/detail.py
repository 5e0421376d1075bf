"""Drop-in for the reference's pybind11 module ``guanaco_ext`` (re-exported by
the reference as ``guanaco.detail``, src/guanaco/detail/__init__.py:21).

Same names, keyword arguments, defaults and argument checks as
src/guanaco/detail/ext/*.h; the work goes through the C ABI of
libguanaco_gb300.so.  Only the device path is implemented: ``device="cpu"``
raises, as there is no CPU fallback behind this package.
"""
from __future__ import annotations

import ctypes
import enum

import numpy as np

from . import _lib

__all__ = [
    "eDevice", "cpu", "gpu", "recon", "corr", "CTF", "get_electron_wavelength",
    "get_defocus_spread", "q_to_Q", "Q_to_q", "df_to_D", "D_to_df", "get_q_and_theta",
]


class eDevice(enum.IntEnum):
    """guanaco::eDevice (include/guanaco/constants.h:41-44); converts from
    "cpu"/"gpu" and int like the reference's enum wrapper
    (src/guanaco/detail/ext/enums.h:35-66)."""

    cpu = 0
    gpu = 1

    @classmethod
    def convert(cls, value):
        if isinstance(value, cls):
            return value
        if isinstance(value, str):
            try:
                return cls[value]
            except KeyError:
                raise ValueError(f'"{value}" is not a valid value for enum type eDevice') from None
        return cls(int(value))


cpu = eDevice.cpu
gpu = eDevice.gpu


def _assert(cond, text):
    if not cond:
        raise RuntimeError(f"ASSERT ({text}) failed")


def _device_only(device):
    if eDevice.convert(device) != eDevice.gpu:
        raise RuntimeError("guanaco_gb300 implements the device path only: pass device='gpu'")


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _write_back(dst, src):
    if dst is not src:
        np.copyto(dst, src, casting="unsafe")


def recon(sinogram, reconstruction, angles, centre, pixel_size=1.0, min_defocus=0.0,
          max_defocus=0.0, device=eDevice.cpu, gpu_index=-1):
    """Filter and backproject one Y slice: src/guanaco/detail/ext/reconstruct.h:35-101.

    ``sinogram`` is (T, N) or (D, T, N) float32, ``reconstruction`` (N, N)
    float32, overwritten.  Unlike the reference (whose py::array_t silently
    writes into a temporary when ``reconstruction`` is not float32 C-contiguous)
    the result always lands in the array passed."""
    _device_only(device)
    sino = np.asarray(sinogram)
    rec = reconstruction if isinstance(reconstruction, np.ndarray) else np.asarray(reconstruction)
    ang = np.asarray(angles)
    _assert(sino.ndim == 2 or sino.ndim == 3, "sinogram.ndim() == 2 || sinogram.ndim() == 3")
    _assert(rec.ndim == 2, "reconstruction.ndim() == 2")
    _assert(ang.ndim == 1, "angles.ndim() == 1")
    if sino.ndim == 2:
        _assert(sino.shape[0] == ang.size, "sinogram.shape()[0] == angles.size()")
        _assert(sino.shape[1] == rec.shape[0], "sinogram.shape()[1] == reconstruction.shape()[0]")
        _assert(sino.shape[1] == rec.shape[1], "sinogram.shape()[1] == reconstruction.shape()[1]")
    else:
        _assert(sino.shape[1] == ang.size, "sinogram.shape()[1] == angles.size()")
        _assert(sino.shape[2] == rec.shape[0], "sinogram.shape()[2] == reconstruction.shape()[0]")
        _assert(sino.shape[2] == rec.shape[1], "sinogram.shape()[2] == reconstruction.shape()[1]")
    recon_grid(sino, rec, ang, centre, pixel_size, min_defocus, max_defocus, gpu_index)


def recon_grid(sinogram, reconstruction, angles, centre, pixel_size=1.0, min_defocus=0.0,
               max_defocus=0.0, gpu_index=-1):
    """``recon`` for any (Z, X) grid, as guanaco::Config allows
    (include/guanaco/config.h:29-76) but the pybind wrapper does not."""
    L = _lib.load()
    sino = _f32(sinogram)
    rec = reconstruction
    out = rec if (rec.dtype == np.float32 and rec.flags.c_contiguous) else np.empty(rec.shape, np.float32)
    ang = _f32(angles)
    cfg = _lib.GncConfig()
    cfg.device = 1
    cfg.gpu_index = int(gpu_index)
    cfg.num_pixels = sino.shape[-1]
    cfg.num_angles = ang.size
    cfg.num_defocus = 1 if sino.ndim == 2 else sino.shape[0]
    cfg.grid_height = rec.shape[0]
    cfg.grid_width = rec.shape[1]
    cfg.pixel_size = float(pixel_size)
    cfg.centre = float(centre)
    cfg.min_defocus = float(min_defocus)
    cfg.max_defocus = float(max_defocus)
    cfg.angles = ang.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    _assert(sino.size == cfg.num_pixels * cfg.num_angles * cfg.num_defocus,
            "sinogram.size == num_pixels * num_angles * num_defocus")
    _lib.check(L.gnc_reconstruct(ctypes.byref(cfg), sino.ctypes.data, out.ctypes.data))
    _write_back(rec, out)


def corr(image, ctf, rec, device=eDevice.cpu):
    """CTF phase flip of one image: src/guanaco/detail/ext/correct.h:32-76."""
    _device_only(device)
    L = _lib.load()
    img = np.asarray(image)
    c = np.asarray(ctf)
    r = rec if isinstance(rec, np.ndarray) else np.asarray(rec)
    _assert(img.ndim == 2, "image.ndim() == 2")
    _assert(c.ndim == 2 or c.ndim == 3, "ctf.ndim() == 2 || ctf.ndim() == 3")
    _assert(r.ndim == img.ndim + (c.ndim - 2), "rec.ndim() == image.ndim() + (ctf.ndim() - 2)")
    num_ctf = 1 if c.ndim == 2 else c.shape[0]
    ysize, xsize = img.shape
    _assert(num_ctf > 0, "num_ctf > 0")
    _assert(ysize > 0, "ysize > 0")
    _assert(xsize > 0, "xsize > 0")
    _assert(c.shape[-2] == ysize, "ctf.shape()[ctf.ndim() - 2] == ysize")
    _assert(c.shape[-1] == xsize, "ctf.shape()[ctf.ndim() - 1] == xsize")
    _assert(r.shape[-2] == ysize, "rec.shape()[rec.ndim() - 2] == ysize")
    _assert(r.shape[-1] == xsize, "rec.shape()[rec.ndim() - 1] == xsize")
    img32 = _f32(img)
    c64 = np.ascontiguousarray(c, dtype=np.complex64)
    out = r if (r.dtype == np.float32 and r.flags.c_contiguous) else np.empty(r.shape, np.float32)
    _lib.check(L.gnc_correct(img32.ctypes.data, c64.ctypes.data, out.ctypes.data, xsize, ysize,
                             num_ctf))
    _write_back(r, out)


# ------------------------------------------------------------------ CTF ---
def get_electron_wavelength(V):
    return _lib.load().gnc_get_electron_wavelength(float(V))


def get_defocus_spread(Cc, dEE, dII, dVV):
    return _lib.load().gnc_get_defocus_spread(float(Cc), float(dEE), float(dII), float(dVV))


def q_to_Q(q, l, Cs):
    return _lib.load().gnc_q_to_Q(float(q), float(l), float(Cs))


def Q_to_q(Q, l, Cs):
    return _lib.load().gnc_Q_to_q(float(Q), float(l), float(Cs))


def df_to_D(df, l, Cs):
    return _lib.load().gnc_df_to_D(float(df), float(l), float(Cs))


def D_to_df(D, l, Cs):
    return _lib.load().gnc_D_to_df(float(D), float(l), float(Cs))


def get_q_and_theta(w, h, ps):
    """FFT-ordered (q, theta) grids (h, w): src/guanaco/detail/ext/ctf.h:41-56."""
    q = np.empty((int(h), int(w)), np.float64)
    a = np.empty((int(h), int(w)), np.float64)
    _lib.check(_lib.load().gnc_q_and_theta(int(w), int(h), float(ps), q.ctypes.data, a.ctypes.data))
    return q, a


class CTF:
    """guanaco::CTF with the methods of src/guanaco/detail/ext/ctf.h:222-279.

    Two-argument calls take (q, theta) arrays; three-argument calls take
    (w, h, ps) and return the FFT-ordered (h, w) grid."""

    def __init__(self, l, df=0, Cs=0, Ca=0, Pa=0, dd=0, theta_c=0, phi=0):
        self.l, self.df, self.Cs, self.Ca, self.Pa = float(l), float(df), float(Cs), float(Ca), float(Pa)
        self.dd, self.theta_c, self.phi = float(dd), float(theta_c), float(phi)

    def _c(self):
        return _lib.GncCtf(self.l, self.df, self.Cs, self.Ca, self.Pa, self.dd, self.theta_c,
                           self.phi)

    def _eval(self, kind, q, theta=None):
        qa = np.ascontiguousarray(q, dtype=np.float64)
        ta = None if theta is None else np.ascontiguousarray(theta, dtype=np.float64)
        cplx = kind in ("full", "simple")
        out = np.empty(qa.shape + ((2,) if cplx else ()), np.float64)
        c = self._c()
        _lib.check(_lib.load().gnc_ctf_eval(ctypes.byref(c), _lib.CTF_KIND[kind], qa.ctypes.data,
                                            None if ta is None else ta.ctypes.data, qa.size,
                                            out.ctypes.data))
        return out[..., 0] + 1j * out[..., 1] if cplx else out

    def _grid(self, kind, w, h, ps):
        cplx = kind in ("full", "simple")
        out = np.empty((int(h), int(w)) + ((2,) if cplx else ()), np.float64)
        c = self._c()
        _lib.check(_lib.load().gnc_ctf_grid(ctypes.byref(c), _lib.CTF_KIND[kind], int(w), int(h),
                                            float(ps), out.ctypes.data))
        return out[..., 0] + 1j * out[..., 1] if cplx else out

    def get_chi(self, q, theta):
        c = self._c()
        return _lib.load().gnc_ctf_chi(ctypes.byref(c), float(q), float(theta))

    def get_Es(self, q, theta):
        return self._eval("Es", q, theta)

    def get_Et(self, q):
        return self._eval("Et", q)

    def _dispatch(self, kind, args):
        if len(args) == 2:
            return self._eval(kind, *args)
        if len(args) == 3:
            return self._grid(kind, *args)
        raise TypeError(f"get_{kind}: expected (q, theta) or (w, h, ps)")

    def get_ctf(self, *args):
        return self._dispatch("full", args)

    def get_ctf_simple(self, *args):
        return self._dispatch("simple", args)

    def get_ctf_simple_real(self, *args):
        return self._dispatch("simple_real", args)

    def get_ctf_simple_imag(self, *args):
        return self._dispatch("simple_imag", args)
