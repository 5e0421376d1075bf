"""Oracle for guanaco's 3D-CTF FBP path -- TEST INFRASTRUCTURE ONLY.

numpy front end over ``libgno_oracle.so`` (the C restatement in
``gno_oracle.c``) plus a numpy restatement of the reference's Python-side
steps that decide the defocus slabs and build the CTF stack.  Only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
module; the product package never does.

Reference anchors (paths relative to the guanaco source tree):
  * ``defocus_steps``      src/guanaco/detail/correct.py:44-93
  * ``ctf_stack``          src/guanaco/detail/correct.py:116-214
  * ``fbp_ctf``            src/guanaco/detail/correct.py:217-318,
                           src/guanaco/detail/reconstruct.py:127-213,
                           src/guanaco/detail/mp.py:106-153
  * C functions            see gno_oracle.h
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libgno_oracle.so")
_lib = None

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_sz = ctypes.c_size_t


class _Config(ctypes.Structure):
    _fields_ = [
        ("num_pixels", ctypes.c_size_t),
        ("num_angles", ctypes.c_size_t),
        ("num_defocus", ctypes.c_size_t),
        ("grid_height", ctypes.c_size_t),
        ("grid_width", ctypes.c_size_t),
        ("pixel_size", ctypes.c_float),
        ("centre", ctypes.c_float),
        ("min_defocus", ctypes.c_float),
        ("max_defocus", ctypes.c_float),
        ("angles", ctypes.POINTER(ctypes.c_float)),
    ]


class _CtfParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("l", "df", "Cs", "Ca", "Pa", "dd", "theta_c", "phi")]


def build():
    """Compile libgno_oracle.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.gno_electron_wavelength.restype = ctypes.c_double
        L.gno_electron_wavelength.argtypes = [ctypes.c_double]
        L.gno_defocus_spread.restype = ctypes.c_double
        L.gno_defocus_spread.argtypes = [ctypes.c_double] * 4
        L.gno_chi.restype = ctypes.c_double
        L.gno_chi.argtypes = [ctypes.POINTER(_CtfParams), ctypes.c_double, ctypes.c_double]
        L.gno_ctf_grid.restype = None
        L.gno_ctf_grid.argtypes = [ctypes.POINTER(_CtfParams), _sz, _sz, ctypes.c_double,
                                   ctypes.c_int, _f64p]
        L.gno_correct_f.argtypes = [_f32p, _f32p, _f32p, _sz, _sz, _sz]
        L.gno_correct_d.argtypes = [_f64p, _f32p, _f64p, _sz, _sz, _sz]
        L.gno_filter_f.argtypes = [_f32p, _sz, _sz]
        L.gno_filter_d.argtypes = [_f64p, _sz, _sz]
        L.gno_project_f.argtypes = [ctypes.POINTER(_Config), _f32p, _f32p]
        L.gno_project_d.argtypes = [ctypes.POINTER(_Config), _f64p, _f64p]
        L.gno_recon_f.argtypes = [ctypes.POINTER(_Config), _f32p, _f32p]
        L.gno_recon_d.argtypes = [ctypes.POINTER(_Config), _f64p, _f64p]
        L.gno_slab_index_map.argtypes = [ctypes.POINTER(_Config), _i32p]
        vp = ctypes.c_void_p
        L.gno_fbp_ctf_f.argtypes = [_f32p, _sz, _sz, _sz, _f32p, _f32p, ctypes.c_float, vp, _sz,
                                    ctypes.c_float, ctypes.c_float, vp, ctypes.c_int, _sz, _f32p,
                                    _sz, _sz, _sz, _sz, ctypes.c_int]
        L.gno_fbp_ctf_d.argtypes = [_f32p, _sz, _sz, _sz, _f32p, _f32p, ctypes.c_float, vp, _sz,
                                    ctypes.c_float, ctypes.c_float, vp, ctypes.c_int, _sz, _f64p,
                                    _sz, _sz, ctypes.c_int]
        _szp = np.ctypeslib.ndpointer(dtype=np.uintp, flags="C_CONTIGUOUS")
        L.gno_fbp_ctf_rows_f.argtypes = [_f32p, _sz, _sz, _sz, _f32p, _f32p, ctypes.c_float, vp,
                                         _sz, ctypes.c_float, ctypes.c_float, vp, ctypes.c_int,
                                         _sz, _szp, _sz, _f32p, _sz, _sz, ctypes.c_int]
        L.gno_fbp_ctf_rows_d.argtypes = [_f32p, _sz, _sz, _sz, _f32p, _f32p, ctypes.c_float, vp,
                                         _sz, ctypes.c_float, ctypes.c_float, vp, ctypes.c_int,
                                         _sz, _szp, _sz, _f64p, ctypes.c_int]
        _lib = L
    return _lib


# ---------------------------------------------------------------- CTF physics
def electron_wavelength(V):
    return lib().gno_electron_wavelength(float(V))


def defocus_spread(Cc, dEE, dII, dVV):
    return lib().gno_defocus_spread(float(Cc), float(dEE), float(dII), float(dVV))


def _params(l, df=0.0, Cs=0.0, Ca=0.0, Pa=0.0, dd=0.0, theta_c=0.0, phi=0.0):
    return _CtfParams(float(l), float(df), float(Cs), float(Ca), float(Pa), float(dd),
                      float(theta_c), float(phi))


def chi(q, theta, **params):
    p = _params(**params)
    return lib().gno_chi(ctypes.byref(p), float(q), float(theta))


def ctf_grid(w, h, ps, simple=True, **params):
    """complex128 (h, w) grid of the CTF in FFT order: ctf.h:466-503."""
    p = _params(**params)
    out = np.empty((h, w, 2), dtype=np.float64)
    lib().gno_ctf_grid(ctypes.byref(p), w, h, float(ps), 1 if simple else 0, out)
    return out[..., 0] + 1j * out[..., 1]


# ------------------------------------------------- correct.py restatements
def defocus_steps(defocus, num_defocus=None, step_defocus=None, width=None, centre=None,
                  pixel_size=None):
    """min, max, step, num as correct.py:44-93 computes them (numpy float32
    arithmetic where the reference's centre array is float32)."""
    if num_defocus is None or num_defocus <= 0:
        num_defocus = 1
    if num_defocus == 1:
        return defocus, defocus, 0, num_defocus
    if step_defocus is not None and step_defocus > 0:
        mn = defocus - 0.5 * (num_defocus - 1) * step_defocus
        mx = defocus + 0.5 * (num_defocus - 1) * step_defocus
        return mn, mx, step_defocus, num_defocus
    centre = np.asarray(centre)
    z = [defocus - centre * pixel_size, defocus + centre * pixel_size,
         defocus - (width - centre) * pixel_size, defocus + (width - centre) * pixel_size]
    mn = min(v.min() for v in z)
    mx = max(v.max() for v in z)
    step = (mx - mn) / (num_defocus - 1)
    return mn, mx, step, num_defocus


def ctf_stack(width, height, pixel_size, energy, min_defocus, num_defocus, step_defocus,
              spherical_aberration=0, astigmatism=0, astigmatism_angle=0, phase_shift=0):
    """complex64 (D, H, W) stack: correct.py:116-214 (keV, mm and degrees in)."""
    out = np.zeros((num_defocus, height, width), dtype=np.complex64)
    l = electron_wavelength(energy * 1000)

    def slab(d):  # the C grid runs without the GIL: slabs in parallel threads
        df = min_defocus + d * step_defocus
        out[d] = ctf_grid(width, height, pixel_size, simple=True, l=l, df=df,
                          Cs=spherical_aberration * 1e7, Ca=astigmatism,
                          Pa=astigmatism_angle * math.pi / 180,
                          phi=phase_shift * math.pi / 180)

    if num_defocus > 1 and width * height >= (1 << 18):
        from concurrent.futures import ThreadPoolExecutor

        with ThreadPoolExecutor(max_workers=min(num_defocus, os.cpu_count() or 1)) as ex:
            list(ex.map(slab, range(num_defocus)))
    else:
        for d in range(num_defocus):
            slab(d)
    return out


# ------------------------------------------------------------ C entry points
def correct(image, ctf, precision="f32"):
    """(D, H, W) corrected images of one (H, W) image: correct.cpp:30-90."""
    ctf = np.ascontiguousarray(ctf, dtype=np.complex64)
    if ctf.ndim == 2:
        ctf = ctf[None]
    D, H, W = ctf.shape
    cv = ctf.view(np.float32).reshape(D, H, W, 2)
    cv = np.ascontiguousarray(cv)
    if precision == "f32":
        img = np.ascontiguousarray(image, dtype=np.float32)
        out = np.empty((D, H, W), dtype=np.float32)
        lib().gno_correct_f(img, cv, out, W, H, D)
    else:
        img = np.ascontiguousarray(image, dtype=np.float64)
        out = np.empty((D, H, W), dtype=np.float64)
        lib().gno_correct_d(img, cv, out, W, H, D)
    return out


def ramp_filter(rows, precision="f32"):
    """Ramp-filtered copy of rows (..., N): filter.cpp:61-97."""
    dt = np.float32 if precision == "f32" else np.float64
    a = np.array(rows, dtype=dt, copy=True, order="C")
    N = a.shape[-1]
    nrows = a.size // N
    if precision == "f32":
        lib().gno_filter_f(a, N, nrows)
    else:
        lib().gno_filter_d(a, N, nrows)
    return a


def _config(sino_shape, grid_shape, angles, centre, pixel_size, min_defocus, max_defocus):
    angles = np.ascontiguousarray(angles, dtype=np.float32)
    D = sino_shape[0] if len(sino_shape) == 3 else 1
    cfg = _Config(sino_shape[-1], angles.size, D, grid_shape[0], grid_shape[1],
                  float(pixel_size), float(centre), float(min_defocus), float(max_defocus),
                  angles.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    return cfg, angles


def project(sino, grid_shape, angles, centre, pixel_size=1.0, min_defocus=0.0,
            max_defocus=0.0, precision="f32"):
    """Backprojection only (no filter), zero initial volume: reconstructor.cpp:14-90."""
    cfg, keep = _config(np.shape(sino), grid_shape, angles, centre, pixel_size, min_defocus,
                        max_defocus)
    if precision == "f32":
        s = np.ascontiguousarray(sino, dtype=np.float32)
        rec = np.zeros(grid_shape, dtype=np.float32)
        lib().gno_project_f(ctypes.byref(cfg), s, rec)
    else:
        s = np.ascontiguousarray(sino, dtype=np.float64)
        rec = np.zeros(grid_shape, dtype=np.float64)
        lib().gno_project_d(ctypes.byref(cfg), s, rec)
    del keep
    return rec


def recon(sino, grid_shape, angles, centre, pixel_size=1.0, min_defocus=0.0,
          max_defocus=0.0, precision="f32"):
    """Filter + backproject one slice: reconstructor.cpp:92-115."""
    cfg, keep = _config(np.shape(sino), grid_shape, angles, centre, pixel_size, min_defocus,
                        max_defocus)
    if precision == "f32":
        s = np.ascontiguousarray(sino, dtype=np.float32)
        rec = np.zeros(grid_shape, dtype=np.float32)
        lib().gno_recon_f(ctypes.byref(cfg), s, rec)
    else:
        s = np.ascontiguousarray(sino, dtype=np.float64)
        rec = np.zeros(grid_shape, dtype=np.float64)
        lib().gno_recon_d(ctypes.byref(cfg), s, rec)
    del keep
    return rec


def slab_index_map(num_pixels, num_defocus, grid_shape, angles, centre, pixel_size,
                   min_defocus, max_defocus):
    """int32 (T, Z, X) defocus-slab index: reconstructor.cpp:28-73."""
    cfg, keep = _config((num_defocus, len(angles), num_pixels), grid_shape, angles, centre,
                        pixel_size, min_defocus, max_defocus)
    out = np.empty((len(angles), grid_shape[0], grid_shape[1]), dtype=np.int32)
    lib().gno_slab_index_map(ctypes.byref(cfg), out)
    del keep
    return out


def fbp_ctf(proj, angles, centre, pixel_size, ctf=None, min_defocus=0.0, max_defocus=0.0,
            weights=None, minus=False, Z=None, precision="f32", rows=None, tilts=None,
            nthreads=0):
    """Whole pipeline on (T, H, W) projections -> (H, Z, W) volume.

    ``ctf`` is the complex64 (D, H, W) stack from :func:`ctf_stack` or None
    (no correction).  ``rows`` restricts the backprojection to a sample of Y
    rows (both precisions); ``tilts`` restricts the float pipeline's
    correction to a sample of tilts (timing only)."""
    proj = np.ascontiguousarray(proj, dtype=np.float32)
    T, H, W = proj.shape
    Z = W if Z is None else Z
    angles = np.ascontiguousarray(angles, dtype=np.float32)
    centre = np.ascontiguousarray(np.broadcast_to(np.asarray(centre, np.float32), (H,)))
    D = 0
    cptr = None
    if ctf is not None:
        ctf = np.ascontiguousarray(ctf, dtype=np.complex64)
        D = ctf.shape[0]
        cptr = ctf.ctypes.data
    wptr = None
    if weights is not None:
        weights = np.ascontiguousarray(weights, dtype=np.float64)
        wptr = weights.ctypes.data
    if precision == "f32":
        vol = np.zeros((H, Z, W), dtype=np.float32)
        y0, y1 = (0, H) if rows is None else rows
        t0, t1 = (0, T) if tilts is None else tilts
        lib().gno_fbp_ctf_f(proj, T, H, W, angles, centre, float(pixel_size), cptr, D,
                            float(min_defocus), float(max_defocus), wptr, int(bool(minus)), Z,
                            vol, y0, y1, t0, t1, int(nthreads))
    else:
        vol = np.zeros((H, Z, W), dtype=np.float64)
        y0, y1 = (0, H) if rows is None else rows
        lib().gno_fbp_ctf_d(proj, T, H, W, angles, centre, float(pixel_size), cptr, D,
                            float(min_defocus), float(max_defocus), wptr, int(bool(minus)), Z,
                            vol, y0, y1, int(nthreads))
    return vol


def fbp_ctf_rows(proj, angles, centre, pixel_size, rows, ctf=None, min_defocus=0.0,
                 max_defocus=0.0, weights=None, minus=False, Z=None, precision="f32",
                 nthreads=0):
    """:func:`fbp_ctf` for a list of Y rows only: returns (len(rows), Z, W), row
    i of it the volume's row rows[i].  One correction pass serves every row,
    and only the listed rows' memory is allocated (bands of a volume too large
    to hold whole)."""
    proj = np.ascontiguousarray(proj, dtype=np.float32)
    T, H, W = proj.shape
    Z = W if Z is None else Z
    rows = np.ascontiguousarray(rows, dtype=np.uintp)
    if rows.size and (rows.min() < 0 or rows.max() >= H):
        raise ValueError("row out of range")
    angles = np.ascontiguousarray(angles, dtype=np.float32)
    centre = np.ascontiguousarray(np.broadcast_to(np.asarray(centre, np.float32), (H,)))
    D = 0
    cptr = None
    if ctf is not None:
        ctf = np.ascontiguousarray(ctf, dtype=np.complex64)
        D = ctf.shape[0]
        cptr = ctf.ctypes.data
    wptr = None
    if weights is not None:
        weights = np.ascontiguousarray(weights, dtype=np.float64)
        wptr = weights.ctypes.data
    if precision == "f32":
        out = np.zeros((rows.size, Z, W), dtype=np.float32)
        lib().gno_fbp_ctf_rows_f(proj, T, H, W, angles, centre, float(pixel_size), cptr, D,
                                 float(min_defocus), float(max_defocus), wptr, int(bool(minus)),
                                 Z, rows, rows.size, out, 0, T, int(nthreads))
    else:
        out = np.zeros((rows.size, Z, W), dtype=np.float64)
        lib().gno_fbp_ctf_rows_d(proj, T, H, W, angles, centre, float(pixel_size), cptr, D,
                                 float(min_defocus), float(max_defocus), wptr, int(bool(minus)),
                                 Z, rows, rows.size, out, int(nthreads))
    return out
