"""Whole-series 3D-CTF filtered backprojection plan over the C ABI.

A plan holds the device workspace and tables of one acquisition geometry
(tilts, image size, volume size, defocus slabs, CTF parameters).  It runs on
device memory (torch CUDA tensors or raw device pointers) with an explicit
stream, or from host numpy arrays with the copies included.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _ptr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    raise TypeError(f"cannot take a pointer of {type(x)!r}")


def _stream(stream):
    if stream is None:
        try:
            import torch

            if torch.cuda.is_available():
                return torch.cuda.current_stream().cuda_stream
        except ImportError:
            pass
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class FbpDesc:
    """A gnc_fbp_desc (one acquisition geometry and its CTF and volume) with
    the arrays it points to kept alive.

    Parameters mirror the reference's ``correct_projections`` and
    ``reconstruct`` (src/guanaco/detail/correct.py:217-318,
    src/guanaco/detail/reconstruct.py:127-213): energy in keV, spherical
    aberration in mm, astigmatism angle and phase shift in degrees,
    ``slab_defocus`` the absolute defocus of every CTF slab and
    ``min_defocus``/``max_defocus`` the relative range the backprojector maps
    onto the slabs.
    """

    def __init__(self, num_angles, height, width, angles, *, grid_height=None, grid_width=None,
                 centre=None, pixel_size=1.0, input="raw", correct=True, num_defocus=1,
                 slab_defocus=None, min_defocus=0.0, max_defocus=0.0, energy=300.0,
                 spherical_aberration=0.0, astigmatism=0.0, astigmatism_angle=0.0,
                 phase_shift=0.0, weights=None, minus=False, staging="f32"):
        self.T, self.H, self.W = int(num_angles), int(height), int(width)
        self.Z = int(grid_height if grid_height is not None else width)
        self.X = int(grid_width if grid_width is not None else width)
        self.D = int(num_defocus)
        self.input = input
        self.staging = staging
        self._angles = np.ascontiguousarray(angles, dtype=np.float32)
        self._centre = None if centre is None else np.ascontiguousarray(
            np.broadcast_to(np.asarray(centre, np.float32), (self.H,)))
        self._slabs = None if slab_defocus is None else np.ascontiguousarray(slab_defocus, np.float64)
        self._weights = None if weights is None else np.ascontiguousarray(weights, np.float64)
        d = _lib.GncFbpDesc()
        d.num_angles, d.height, d.width = self.T, self.H, self.W
        d.grid_height, d.grid_width = self.Z, self.X
        d.angles = self._angles.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        d.centre = (None if self._centre is None
                    else self._centre.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        d.pixel_size = float(pixel_size)
        d.ctf_pixel_size = float(pixel_size)
        d.input = _lib.GNC_INPUT_RAW if input == "raw" else _lib.GNC_INPUT_CORRECTED
        d.correct = 1 if (correct and input == "raw") else 0
        d.num_defocus = self.D
        d.slab_defocus = (None if self._slabs is None
                          else self._slabs.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        d.min_defocus = float(min_defocus)
        d.max_defocus = float(max_defocus)
        d.energy_kev = float(energy)
        d.cs_mm = float(spherical_aberration)
        d.astigmatism = float(astigmatism)
        d.astigmatism_angle_deg = float(astigmatism_angle)
        d.phase_shift_deg = float(phase_shift)
        d.weights = (None if self._weights is None
                     else self._weights.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        d.minus = 1 if minus else 0
        stagings = {"f32": _lib.GNC_STAGE_F32, "f16": _lib.GNC_STAGE_F16,
                    "f16t": _lib.GNC_STAGE_F16T}
        if staging not in stagings:
            raise ValueError(f"staging must be one of {sorted(stagings)}, not {staging!r}")
        d.staging = stagings[staging]
        self.correcting = bool(d.correct)
        self.c = d

    @property
    def input_shape(self):
        if self.input == "raw":
            return (self.T, self.H, self.W)
        return (self.T, self.D, self.H, self.W)

    @property
    def volume_shape(self):
        return (self.H, self.Z, self.X)

    @property
    def voxel_tilts(self):
        return self.H * self.Z * self.X * self.T


class FbpPlan(FbpDesc):
    """3D-CTF FBP of (T, H, W) raw projections or a (T, D, H, W) corrected
    stack into an (H, Z, X) volume, with the device workspace of one
    geometry (parameters as FbpDesc)."""

    def __init__(self, num_angles, height, width, angles, **kw):
        super().__init__(num_angles, height, width, angles, **kw)
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(self._lib.gnc_fbp_plan_create(ctypes.byref(self.c), ctypes.byref(h)))
        self._h = h

    # ---------------------------------------------------------------- sizes
    @property
    def workspace_bytes(self):
        return self._lib.gnc_fbp_workspace_bytes(self._h)

    @property
    def launches_per_execute(self):
        return self._lib.gnc_fbp_launches(self._h)

    def live_slabs(self, stream=None):
        """int32 (T, 2): per tilt the first and last slab any voxel reads; the
        flip and filter skip the other (tilt, slab) pairs."""
        out = np.empty((self.T, 2), np.int32)
        _lib.check(self._lib.gnc_fbp_live_slabs(self._h, out.ctypes.data, _stream(stream)))
        return out

    @property
    def backprojector(self):
        """0: the exact backprojection kernel; 2 or 4: the fast kernel and its
        slab capacity per tile."""
        return self._lib.gnc_fbp_backprojector(self._h)

    # ------------------------------------------------------------- running
    def execute(self, inp, vol, stream=None):
        """Device input -> device volume (overwritten), enqueued on ``stream``."""
        _lib.check(self._lib.gnc_fbp_execute(self._h, _ptr(inp), _ptr(vol), _stream(stream)))

    def execute_host(self, inp, vol=None, stream=None):
        """Host input -> host volume; copies in and out, synchronises."""
        a = np.ascontiguousarray(inp, dtype=np.float32)
        if a.shape != self.input_shape:
            raise ValueError(f"input shape {a.shape} != {self.input_shape}")
        out = vol if vol is not None else np.empty(self.volume_shape, np.float32)
        if out.shape != self.volume_shape or out.dtype != np.float32 or not out.flags.c_contiguous:
            raise ValueError("volume must be a C-contiguous float32 array of volume_shape")
        _lib.check(self._lib.gnc_fbp_execute_host(self._h, _ptr(a), _ptr(out), _stream(stream)))
        return out

    def correct(self, proj, corrected, stream=None):
        """Raw (T, H, W) -> corrected (T, D, H, W), device pointers."""
        _lib.check(self._lib.gnc_fbp_correct(self._h, _ptr(proj), _ptr(corrected), _stream(stream)))

    def stage(self, inp, stream=None):
        _lib.check(self._lib.gnc_fbp_stage(self._h, _ptr(inp), _stream(stream)))

    def backproject(self, vol, exact=False, stream=None):
        _lib.check(self._lib.gnc_fbp_backproject(self._h, _ptr(vol), 1 if exact else 0,
                                                 _stream(stream)))

    def backproject_staged(self, staged, row_exp, vol, exact=False, stream=None):
        """Backproject caller-provided staged rows ((ceil(H/2), D, T, W) pairs)."""
        _lib.check(self._lib.gnc_fbp_backproject_staged(self._h, _ptr(staged), _ptr(row_exp),
                                                        _ptr(vol), 1 if exact else 0,
                                                        _stream(stream)))

    def slab_map(self, out, stream=None):
        _lib.check(self._lib.gnc_fbp_slab_map(self._h, _ptr(out), _stream(stream)))

    def sign_table(self, out, stream=None):
        _lib.check(self._lib.gnc_fbp_sign_table(self._h, _ptr(out), _stream(stream)))

    def check(self, stream=None):
        """Synchronise and raise if a bounded device-side wait gave up."""
        _lib.check(self._lib.gnc_fbp_check(self._h, _stream(stream)))

    def staged(self):
        """(device pointer of the staged rows, device pointer of the F16 exponents)."""
        s = ctypes.c_void_p()
        e = ctypes.c_void_p()
        _lib.check(self._lib.gnc_fbp_staged(self._h, ctypes.byref(s), ctypes.byref(e)))
        return s.value, e.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gnc_fbp_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
