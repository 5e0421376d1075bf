"""CTF images: the image-writing part of the reference's ``guanaco.plot``
(src/guanaco/plot.py).

``generate_ctf`` takes the reference's arguments and writes the same file: the
full CTF (envelopes included) of a defocus series as a complex64 MRC stack
(num_defocus, height, width).  The images are computed on the GPU in double
precision by ``gnc_ctf_image_device``, all defoci in one launch, where the
reference evaluates ``CTF.get_ctf`` once per defocus on the host.  The
reference module's matplotlib plots are not part of this package.
"""
from __future__ import annotations

import ctypes
from math import pi

import numpy as np

from . import _lib, detail, mrc

__all__ = ["ctf_images", "generate_ctf"]


def ctf_images(ctf, defoci, width, height, pixel_size, kind="full", stream=None):
    """CTF images of ``ctf`` (a ``detail.CTF``; its own defocus is not used) at
    each defocus of ``defoci`` on the current CUDA device: a torch tensor
    (len(defoci), height, width), complex64 for the kinds "full" and "simple",
    float32 for "simple_real", "simple_imag", "chi", "Es" and "Et".  Each image
    is the FFT-ordered grid of ``CTF.get_<kind>(width, height, pixel_size)``."""
    import torch

    if kind not in _lib.CTF_KIND:
        raise ValueError(f"unknown CTF kind {kind!r}")
    d = np.ascontiguousarray(np.atleast_1d(defoci), dtype=np.float64)
    cplx = kind in ("full", "simple")
    out = torch.empty((d.size, int(height), int(width)),
                      dtype=torch.complex64 if cplx else torch.float32, device="cuda")
    if stream is None:
        stream = torch.cuda.current_stream().cuda_stream
    c = ctf._c()
    _lib.check(_lib.load().gnc_ctf_image_device(ctypes.byref(c), _lib.CTF_KIND[kind],
                                                d.ctypes.data, d.size, int(width), int(height),
                                                float(pixel_size), out.data_ptr(), stream))
    return out


def generate_ctf(filename=None, image_size=None, pixel_size=1, defocus=0, num_defocus=None,
                 step_defocus=None, spherical_aberration=2.7, astigmatism=0,
                 astigmatism_angle=0, energy=300, defocus_spread=None, source_spread=0.02,
                 chromatic_aberration=2.7, energy_spread=0.33e-6, current_spread=0.33e-6,
                 acceleration_voltage_spread=0.8e-6, phase_shift=0, component="imag",
                 envelope=True, recentre=False):
    """Write the CTF images of a defocus series to ``filename`` (plot.py:175-284).

    Units as the reference: pixel size and defocus in A, Cs and Cc in mm,
    astigmatism angle in degrees, energy in keV, source spread in mrad, phase
    shift in rad.  Defocus i of ``num_defocus`` is
    ``defocus + (i - (num_defocus - 1) / 2) * step_defocus``; the defocus spread
    comes from Cc and the energy, current and voltage fluctuations unless given.
    ``component`` and ``envelope`` are accepted and, as in the reference, not
    used: the file holds the full complex CTF.  ``recentre`` moves the zero
    frequency to the image centre."""
    if filename is None or image_size is None:
        raise ValueError("generate_ctf: filename and image_size are required")
    source_spread = source_spread / 1e3  # mrad -> rad
    spherical_aberration = spherical_aberration * 1e7  # mm -> A
    chromatic_aberration = chromatic_aberration * 1e7  # mm -> A
    astigmatism_angle = astigmatism_angle * pi / 180  # deg -> rad
    energy = energy * 1e3  # keV -> eV
    if defocus_spread is None:
        defocus_spread = detail.get_defocus_spread(
            Cc=chromatic_aberration, dEE=energy_spread, dII=current_spread,
            dVV=acceleration_voltage_spread)
    if defocus is None:
        defocus = 0
    if num_defocus is None or num_defocus == 0:
        num_defocus = 1
    if step_defocus is None:
        step_defocus = 0
    wavelength = detail.get_electron_wavelength(energy)
    defoci = [defocus + (i - 0.5 * (num_defocus - 1)) * step_defocus for i in range(num_defocus)]
    c = detail.CTF(l=wavelength, df=defoci[0], Cs=spherical_aberration, Ca=astigmatism,
                   Pa=astigmatism_angle, dd=defocus_spread, theta_c=source_spread,
                   phi=phase_shift)
    images = ctf_images(c, defoci, image_size[1], image_size[0], pixel_size, "full")
    data = images.cpu().numpy()
    if recentre:
        data = np.fft.fftshift(data, axes=(-2, -1))
    with mrc.new_mrc(filename, (num_defocus, image_size[0], image_size[1]), np.complex64,
                     voxel_size=pixel_size) as f:
        f.data[...] = data
