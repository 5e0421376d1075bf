"""Generate the golden fixtures in this directory from the reference itself.

Runs only where the guanaco reference tree is present (the development
container).  It builds the reference's own CPU path into ``oracle/_ref`` with
``oracle/ref/Makefile`` (unmodified reference sources plus an FFT<e_host>
stand-in for FFTW, which is not installed) and then drives:

  * the reference's pybind module ``guanaco_ext`` (CTF functions, ``recon``,
    ``corr``) and
  * the reference's Python package ``guanaco`` (``correct_projections``,
    ``reconstruct``) with ``device="cpu"``,

recording inputs and outputs as small ``.npz`` files.  ``mrcfile`` is not
installed; the reference imports it at module level only, so a stub module
stands in for it (no MRC I/O is exercised).

Usage:  python tests/golden/make_golden.py [/path/to/reference]
"""
from __future__ import annotations

import contextlib
import io
import math
import os
import subprocess
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
# the reference source tree: the first argument, else GUANACO_REFERENCE, else a
# "reference" directory beside the repository
REF = (sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GUANACO_REFERENCE")
       or os.path.join(os.path.dirname(REPO), "reference"))


def load_reference():
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle", "ref"), f"REF={REF}"],
                   check=True)
    sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
    sys.path.insert(0, os.path.join(REF, "src"))
    sys.modules.setdefault("mrcfile", types.ModuleType("mrcfile"))
    import guanaco  # noqa: E402
    import guanaco_ext  # noqa: E402
    return guanaco, guanaco_ext


def quiet():
    return contextlib.redirect_stdout(io.StringIO())


def ctf_kats(ext):
    """The quantities the reference's tests/test_ctf.py checks, as the
    reference computes them (300 kV, Cs 2.7 mm, df 20000 A, q = 10, 100x100
    grids at 2 A/px, phase shift 0.1 rad)."""
    out = {}
    l = ext.get_electron_wavelength(300000)
    out["wavelength_300kV"] = np.float64(l)
    out["defocus_spread"] = np.float64(ext.get_defocus_spread(2.7e7, 1e-6, 1e-6, 1e-6))
    out["q_to_Q"] = np.float64(ext.q_to_Q(10, l, 2.7e7))
    out["Q_to_q"] = np.float64(ext.Q_to_q(out["q_to_Q"], l, 2.7e7))
    out["df_to_D"] = np.float64(ext.df_to_D(20000, l, 2.7e7))
    out["D_to_df"] = np.float64(ext.D_to_df(out["df_to_D"], l, 2.7e7))
    env = ext.CTF(l, 20000, 2.7e7, 0, 0, 1, 1e-3, 0)
    out["Es_q10"] = np.asarray(env.get_Es([10.0], [0.0]))
    out["Et_q10"] = np.asarray(env.get_Et([10.0]))
    out["chi_q10"] = np.float64(ext.CTF(l, 20000, 2.7e7, 0, 0, 0, 0, 0).get_chi(10, 0))
    q, a = ext.get_q_and_theta(100, 100, 2)
    out["q_grid"], out["theta_grid"] = np.asarray(q), np.asarray(a)
    full = ext.CTF(l, 20000, 2.7e7, 0, 0, 1, 0.1 / 1e3, 0.1)
    out["ctf_full"] = np.asarray(full.get_ctf(100, 100, 2))
    simple = ext.CTF(l, 20000, 2.7e7, 0, 0, 0, 0, 0.1)
    out["ctf_simple"] = np.asarray(simple.get_ctf_simple(100, 100, 2))
    out["ctf_simple_real"] = np.asarray(simple.get_ctf_simple_real(100, 100, 2))
    out["ctf_simple_imag"] = np.asarray(simple.get_ctf_simple_imag(100, 100, 2))
    # astigmatic case on a non-square grid (exercises theta and the Ca term)
    astig = ext.CTF(l, 25000, 2.7e7, 800, 0.3, 0, 0, 0.05)
    out["ctf_simple_astig_90x64"] = np.asarray(astig.get_ctf_simple(90, 64, 1.5))
    return out


def ref_capi():
    """ctypes handle on oracle/_ref/libguanaco_ref.so (the reference's C++ API
    through oracle/ref/shim.cpp)."""
    import ctypes
    L = ctypes.CDLL(os.path.join(REPO, "oracle", "_ref", "libguanaco_ref.so"))
    f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
    sz, fl = ctypes.c_size_t, ctypes.c_float
    L.gnr_filter.argtypes = [f32p, sz, sz, sz]
    L.gnr_recon.argtypes = [f32p, f32p, sz, sz, sz, sz, sz, fl, fl, fl, fl, f32p]
    return L


def filter_cases(rng):
    """Reference Filter<e_host> (filter.cpp:47-97) on (D, T, N) stacks."""
    L = ref_capi()
    out = {}
    for d, t, n in ((1, 3, 64), (2, 5, 100), (1, 2, 384)):
        x = rng.standard_normal((d, t, n)).astype(np.float32)
        y = x.copy()
        assert L.gnr_filter(y, n, t, d) == 0
        out[f"in_{d}x{t}x{n}"] = x
        out[f"out_{d}x{t}x{n}"] = y
    return out


def config_recon_cases(rng):
    """guanaco::Reconstructor(Config) on the host with grid_height != grid_width
    (possible through the C++ API only; the pybind wrapper forces Z = X)."""
    L = ref_capi()
    cases = {}
    for name, (n, t, d, z, c, mn, mx) in {
        "z24_n48_t17_d3": (48, 17, 3, 24, 24.0, -30.0, 30.0),
        "z40_n32_t13_d1": (32, 13, 1, 40, 16.0, 0.0, 0.0),
    }.items():
        ang = np.deg2rad(np.linspace(-60, 60, t)).astype(np.float32)
        sino = rng.standard_normal((d, t, n)).astype(np.float32)
        rec = np.zeros((z, n), np.float32)
        assert L.gnr_recon(sino, rec, n, t, d, z, n, 1.0, c, mn, mx, ang) == 0
        cases[name] = dict(sino=sino, angles=ang, centre=np.float32(c),
                           pixel_size=np.float32(1.0), min_defocus=np.float32(mn),
                           max_defocus=np.float32(mx), rec=rec)
    return cases


def recon_cases(ext, rng):
    """Single-slice filter + backprojection through the pybind ``recon``."""
    cases = {}
    specs = [
        # name, N, T, D, angles (deg), centre, pixel_size, min_df, max_df
        ("plain_n64_t31", 64, 31, 1, np.linspace(-60, 60, 31), 32.0, 1.0, 0.0, 0.0),
        ("offcentre_n48_t19", 48, 19, 1, np.linspace(-54, 54, 19), 21.25, 1.0, 0.0, 0.0),
        ("slab3_n64_t21", 64, 21, 3, np.linspace(-60, 60, 21), 32.0, 1.0, -40.0, 40.0),
        ("slab5_n40_t15_ps", 40, 15, 5, np.linspace(-45, 60, 15), 19.5, 1.35, -30.0, 24.0),
        ("slab4_n32_t9_wide", 32, 9, 4, np.linspace(-90, 90, 9), 16.0, 1.0, -16.0, 16.0),
    ]
    for name, n, t, d, deg, c, ps, mn, mx in specs:
        ang = np.deg2rad(deg).astype(np.float32)
        shape = (t, n) if d == 1 else (d, t, n)
        sino = rng.standard_normal(shape).astype(np.float32)
        rec = np.zeros((n, n), np.float32)
        ext.recon(sino, rec, ang, c, ps, mn, mx, "cpu")
        cases[name] = dict(sino=sino, angles=ang, centre=np.float32(c), pixel_size=np.float32(ps),
                           min_defocus=np.float32(mn), max_defocus=np.float32(mx), rec=rec)
    return cases


def corr_cases(ext, rng):
    """Per-image CTF phase flip through the pybind ``corr``."""
    cases = {}
    l = ext.get_electron_wavelength(300000)
    for name, (h, w, ps, dfs, phi) in {
        "one_slab_40x48": (40, 48, 1.35, [20000.0], 0.0),
        "three_slab_32x36": (32, 36, 1.0, [29000.0, 30000.0, 31000.0], 0.0),
        "phase_shift_30x40": (30, 40, 2.0, [15000.0, 16000.0], 0.1),
    }.items():
        image = rng.standard_normal((h, w)).astype(np.float32)
        ctf = np.stack([ext.CTF(l, df, 2.7e7, 0, 0, 0, 0, phi).get_ctf_simple(w, h, ps)
                        for df in dfs]).astype(np.complex64)
        rec = np.zeros((len(dfs), h, w), np.float32)
        ext.corr(image, ctf, rec, "cpu")
        cases[name] = dict(image=image, ctf=ctf, rec=rec)
    return cases


def blob_series(rng, T, H, W, nblob, angles):
    """Tilt series of analytically projected 3D Gaussian blobs (about y)."""
    zc = rng.uniform(-0.25 * W, 0.25 * W, nblob)
    xc = rng.uniform(-0.35 * W, 0.35 * W, nblob)
    yc = rng.uniform(0.1 * H, 0.9 * H, nblob)
    sig = rng.uniform(1.5, 3.0, nblob)
    amp = rng.uniform(0.5, 1.0, nblob)
    xs = np.arange(W) - W / 2 + 0.5
    ys = np.arange(H)
    out = np.zeros((T, H, W))
    for t, th in enumerate(angles):
        u = xc * math.cos(th) - zc * math.sin(th)
        for k in range(nblob):
            gx = np.exp(-0.5 * ((xs - u[k]) / sig[k]) ** 2)
            gy = np.exp(-0.5 * ((ys - yc[k]) / sig[k]) ** 2)
            out[t] += amp[k] * sig[k] * math.sqrt(2 * math.pi) * np.outer(gy, gx)
    return (out + rng.normal(0, 0.05, out.shape)).astype(np.float32)


def pipeline_cases(guanaco, rng):
    """Whole path through the reference's Python API: correct_projections
    (device cpu) then reconstruct (device cpu)."""
    cases = {}
    specs = [
        # name, T, H, W, ndf, sdf, df, weights, transform, phase_shift
        ("ndf4_24x32", 11, 24, 32, 4, None, 20000.0, False, None, 0.0),
        ("ndf1_20x28", 9, 20, 28, 1, None, 15000.0, False, None, 0.0),
        ("ndf3_sdf_weights_minus_18x30", 13, 18, 30, 3, 40, 25000.0, True, "minus", 5.0),
        ("nodefocus_16x24", 7, 16, 24, None, None, None, False, None, 0.0),
    ]
    for name, T, H, W, ndf, sdf, df, aw, tr, ps_deg in specs:
        ang = np.deg2rad(np.linspace(-60, 60, T)).astype(np.float32)
        proj = blob_series(rng, T, H, W, 6, ang)
        centre = np.full(H, W / 2.0, np.float32)
        with quiet():
            cp, mn, mx = guanaco.correct_projections(proj, centre, 1.0, 300, df, ndf, sdf, 2.7,
                                                     0, 0, ps_deg, None, "cpu")
            cp = np.array(cp)
            vol = guanaco.reconstruct(cp, ang, None, centre, 1.0, mn, mx, transform=tr,
                                      angular_weights=aw, device="cpu")
        cases[name] = dict(proj=proj, angles=ang, centre=centre, pixel_size=np.float32(1.0),
                           energy=np.float64(300), defocus=np.float64(df if df else np.nan),
                           num_defocus=np.int64(ndf if ndf else 0),
                           step_defocus=np.float64(sdf if sdf else np.nan),
                           Cs=np.float64(2.7), phase_shift=np.float64(ps_deg),
                           angular_weights=np.bool_(aw), minus=np.bool_(tr == "minus"),
                           min_defocus=np.float64(mn), max_defocus=np.float64(mx),
                           corrected=cp.astype(np.float32), volume=vol)
    return cases


def main():
    guanaco, ext = load_reference()
    rng = np.random.default_rng(20211203)
    np.savez_compressed(os.path.join(HERE, "ctf_kat.npz"), **ctf_kats(ext))
    np.savez_compressed(os.path.join(HERE, "filter.npz"), **filter_cases(rng))
    for group, cases in (("recon", recon_cases(ext, rng)), ("config", config_recon_cases(rng)),
                         ("corr", corr_cases(ext, rng)),
                         ("pipeline", pipeline_cases(guanaco, rng))):
        for name, arrays in cases.items():
            np.savez_compressed(os.path.join(HERE, f"{group}_{name}.npz"), **arrays)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
