"""Seeded synthetic tilt series for tests and benchmarks.

The phantom is a set of random 3D Gaussian blobs (centre uniform over the
volume, sigma in [2, 8] px, amplitude in [0.5, 1]).  Each tilt (rotation about
the y axis) is the analytic line projection of the blobs -- a 3D Gaussian
integrates to a 2D Gaussian of the same sigma -- optionally convolved with
the phase-contrast transfer function at each blob's height-dependent
defocus, plus Gaussian noise.  Generation runs on the GPU with torch; it is
input preparation, not part of the reconstruction path.
"""
from __future__ import annotations

import math

import numpy as np


def blob_phantom(num_blobs, width, height, thickness, seed, sigma=(2.0, 8.0), amp=(0.5, 1.0)):
    """(x, y, z, sigma, amplitude) of every blob; x, z centred on the volume,
    y a row index."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(-0.45 * width, 0.45 * width, num_blobs)
    y = rng.uniform(0.0, height - 1.0, num_blobs)
    z = rng.uniform(-0.45 * thickness, 0.45 * thickness, num_blobs)
    s = rng.uniform(sigma[0], sigma[1], num_blobs)
    a = rng.uniform(amp[0], amp[1], num_blobs)
    return np.stack([x, y, z, s, a], axis=1)


def tilt_series(blobs, angles, height, width, *, pixel_size=1.0, defocus=None, energy=300.0,
                cs_mm=2.7, amplitude_contrast=0.1, noise=0.05, seed=0, defocus_bins=16,
                device="cuda"):
    """(T, H, W) float32 torch tensor on ``device``.

    With ``defocus`` (A) each blob is imaged at defocus + depth * pixel_size,
    depth = x sin(theta) + z cos(theta), through
    H(k) = -(sqrt(1 - Q0^2) sin(chi) + Q0 cos(chi)), blobs binned into
    ``defocus_bins`` depth bins per tilt."""
    import torch

    g = torch.Generator(device="cpu").manual_seed(int(seed))
    b = torch.as_tensor(blobs, dtype=torch.float64, device=device)
    T = len(angles)
    out = torch.zeros((T, height, width), dtype=torch.float32, device=device)
    xs = torch.arange(width, dtype=torch.float64, device=device) - width / 2 + 0.5
    ys = torch.arange(height, dtype=torch.float64, device=device)
    r = int(math.ceil(4 * float(b[:, 3].max())))
    off = torch.arange(-r, r + 1, device=device)
    if defocus is not None:
        lam = _wavelength(energy * 1000.0)
        ky = torch.fft.fftfreq(height, d=pixel_size, device=device, dtype=torch.float64)
        kx = torch.fft.fftfreq(width, d=pixel_size, device=device, dtype=torch.float64)
        q2 = ky[:, None] ** 2 + kx[None, :] ** 2
        cs = cs_mm * 1e7
        q0 = amplitude_contrast
    for t, th in enumerate(angles):
        th = float(th)
        u = b[:, 0] * math.cos(th) - b[:, 2] * math.sin(th)
        depth = b[:, 0] * math.sin(th) + b[:, 2] * math.cos(th)
        if defocus is None:
            bins = torch.zeros(len(b), dtype=torch.long, device=device)
            nb = 1
        else:
            lo, hi = float(depth.min()), float(depth.max()) + 1e-9
            nb = defocus_bins
            bins = ((depth - lo) / (hi - lo) * nb).long().clamp(0, nb - 1)
        img = torch.zeros((nb, height, width), dtype=torch.float64, device=device)
        # separable Gaussians in a (2r+1)^2 window around each blob
        cx = torch.round(u + width / 2 - 0.5).long()
        cy = torch.round(b[:, 1]).long()
        px = cx[:, None] + off[None, :]
        py = cy[:, None] + off[None, :]
        gx = torch.exp(-0.5 * ((xs[px.clamp(0, width - 1)] - u[:, None]) / b[:, 3:4]) ** 2)
        gy = torch.exp(-0.5 * ((ys[py.clamp(0, height - 1)] - b[:, 1:2]) / b[:, 3:4]) ** 2)
        gx = gx * ((px >= 0) & (px < width))
        gy = gy * ((py >= 0) & (py < height))
        w = (b[:, 4] * b[:, 3] * math.sqrt(2 * math.pi))[:, None, None] * gy[:, :, None] * gx[:, None, :]
        idx = (bins[:, None, None] * height + py.clamp(0, height - 1)[:, :, None]) * width \
            + px.clamp(0, width - 1)[:, None, :]
        img.view(-1).index_add_(0, idx.reshape(-1), w.reshape(-1))
        if defocus is not None:
            centres = lo + (torch.arange(nb, device=device, dtype=torch.float64) + 0.5) * (hi - lo) / nb
            df = defocus + centres * pixel_size
            chi = math.pi * (cs * lam ** 3 * q2[None] ** 2 / 2 - lam * df[:, None, None] * q2[None])
            h = -(math.sqrt(1 - q0 * q0) * torch.sin(chi) + q0 * torch.cos(chi))
            img = torch.fft.ifft2(torch.fft.fft2(img) * h).real
        out[t] = img.sum(0).float()
    if noise:
        out += noise * torch.randn(out.shape, generator=g).to(device)
    return out


def _wavelength(V):
    c, e, m_e, h = 2.99792458e8, 1.602176634e-19, 9.1093837015e-31, 6.62607004e-34
    eV = e * V
    return h * c / math.sqrt(eV * eV + 2 * m_e * eV * c * c) * 1e10


def request_stream(num_requests, rate_hz, seed, sizes=(128, 256, 384, 512), tilts=(31, 41, 61),
                   defocus=(10000.0, 50000.0), max_ndf=10, f16_fraction=0.5, f16_form="f16t"):
    """A seeded stream of serving requests: Poisson arrivals at ``rate_hz``;
    per request a square projection size from ``sizes``, a tilt count from
    ``tilts`` (over +-60 deg), a defocus uniform in ``defocus`` (A), a slab
    count uniform in 1..max_ndf, FP16 staging (the ``f16_form`` staging name)
    with probability ``f16_fraction``, else FP32, volume thickness size / 2,
    and a phantom seed.  Returns a list of dicts sorted by arrival time (s,
    from 0)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, num_requests)
    arrival = np.cumsum(gaps) - gaps[0]
    out = []
    for i in range(num_requests):
        n = int(rng.choice(sizes))
        out.append({
            "id": i,
            "arrival": float(arrival[i]),
            "size": n,
            "tilts": int(rng.choice(tilts)),
            "defocus": float(rng.uniform(defocus[0], defocus[1])),
            "ndf": int(rng.integers(1, max_ndf + 1)),
            "staging": f16_form if rng.random() < f16_fraction else "f32",
            "thickness": n // 2,
            "seed": int(seed * 1000003 + i),
        })
    return out
