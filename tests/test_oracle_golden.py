"""The oracle (C restatement of the reference CPU path) against golden
vectors recorded from the reference itself (tests/golden/make_golden.py)."""
import math

import numpy as np
import pytest

from conftest import golden, golden_names


def test_ctf_known_answers(oracle):
    g = golden("ctf_kat")
    l = oracle.electron_wavelength(300000)
    assert l == pytest.approx(float(g["wavelength_300kV"]), rel=1e-15)
    assert oracle.defocus_spread(2.7e7, 1e-6, 1e-6, 1e-6) == pytest.approx(
        float(g["defocus_spread"]), rel=1e-15)
    assert oracle.chi(10, 0, l=l, df=20000, Cs=2.7e7) == pytest.approx(float(g["chi_q10"]), rel=1e-14)
    simple = oracle.ctf_grid(100, 100, 2, simple=True, l=l, df=20000, Cs=2.7e7, phi=0.1)
    np.testing.assert_allclose(simple, g["ctf_simple"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(simple.real, g["ctf_simple_real"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(simple.imag, g["ctf_simple_imag"], rtol=0, atol=1e-12)
    full = oracle.ctf_grid(100, 100, 2, simple=False, l=l, df=20000, Cs=2.7e7, dd=1,
                           theta_c=0.1 / 1e3, phi=0.1)
    np.testing.assert_allclose(full, g["ctf_full"], rtol=0, atol=1e-12)
    astig = oracle.ctf_grid(90, 64, 1.5, simple=True, l=l, df=25000, Cs=2.7e7, Ca=800, Pa=0.3,
                            phi=0.05)
    np.testing.assert_allclose(astig, g["ctf_simple_astig_90x64"], rtol=0, atol=1e-12)


def test_filter_matches_reference(oracle):
    g = golden("filter")
    for k in g:
        if k.startswith("in_"):
            out = oracle.ramp_filter(g[k], "f32")
            np.testing.assert_array_equal(out, g["out_" + k[3:]])


@pytest.mark.parametrize("name", golden_names("recon_") + golden_names("config_"))
def test_recon_matches_reference(oracle, name):
    g = golden(name)
    rec = oracle.recon(g["sino"], g["rec"].shape, g["angles"], g["centre"], g["pixel_size"],
                       g["min_defocus"], g["max_defocus"], "f32")
    np.testing.assert_array_equal(rec, g["rec"])
    # the FP64 oracle agrees to float rounding
    rd = oracle.recon(g["sino"], g["rec"].shape, g["angles"], g["centre"], g["pixel_size"],
                      g["min_defocus"], g["max_defocus"], "f64")
    assert np.linalg.norm(rd - g["rec"]) / np.linalg.norm(rd) < 1e-5


@pytest.mark.parametrize("name", golden_names("corr_"))
def test_corr_matches_reference(oracle, name):
    g = golden(name)
    out = oracle.correct(g["image"], g["ctf"], "f32")
    np.testing.assert_array_equal(out, g["rec"])
    od = oracle.correct(g["image"], g["ctf"], "f64")
    assert np.linalg.norm(od - g["rec"]) / np.linalg.norm(od) < 1e-6


@pytest.mark.parametrize("name", golden_names("pipeline_"))
def test_pipeline_matches_reference(oracle, name):
    g = golden(name)
    proj, ang, centre = g["proj"], g["angles"], g["centre"]
    T, H, W = proj.shape
    ndf = int(g["num_defocus"])
    ctf = None
    mn = mx = 0.0
    if not math.isnan(float(g["defocus"])):
        df = float(g["defocus"])
        sdf = None if math.isnan(float(g["step_defocus"])) else float(g["step_defocus"])
        lo, hi, step, nd = oracle.defocus_steps(df, ndf, sdf, W, centre, float(g["pixel_size"]))
        ctf = oracle.ctf_stack(W, H, float(g["pixel_size"]), float(g["energy"]), lo, nd, step,
                               float(g["Cs"]), 0, 0, float(g["phase_shift"]))
        mn, mx = lo - df, hi - df
        assert np.float32(mn) == np.float32(g["min_defocus"])
        assert np.float32(mx) == np.float32(g["max_defocus"])
    weights = None
    if bool(g["angular_weights"]):
        weights = angular_weights(ang)
    vol = oracle.fbp_ctf(proj, ang, centre, float(g["pixel_size"]), ctf, mn, mx, weights,
                         bool(g["minus"]), Z=W)
    np.testing.assert_array_equal(vol, g["volume"])


def angular_weights(angles):
    """reconstruct.py:55-105 restated with the same numpy scalar types: the
    interval sums run in float32 because the angles are float32."""
    a = np.asarray(angles)
    idx = np.argsort(a)
    w = np.zeros(a.size)
    mean = abs(a[idx[-1]] - a[idx[0]]) / (a.size - 1) if a.size > 1 else 1.0
    for i in range(a.size):
        si = 0.0
        sw = 0.0
        if i - 2 >= 0:
            sw += 1.0 / 1.5
            si += (1.0 / 1.5) * (a[idx[i - 1]] - a[idx[i - 2]])
        if i - 1 >= 0:
            sw += 2.0
            si += 2.0 * (a[idx[i]] - a[idx[i - 1]])
        if i + 1 < a.size:
            sw += 2.0
            si += 2.0 * (a[idx[i + 1]] - a[idx[i]])
        if i + 2 < a.size:
            sw += 1.0 / 1.5
            si += (1.0 / 1.5) * (a[idx[i + 2]] - a[idx[i + 1]])
        w[idx[i]] = si / sw if sw != 0 else 1.0
    w /= mean
    return w


def test_row_list_oracle_equals_row_range(oracle):
    """fbp_ctf_rows (a list of rows, one correction pass) gives exactly the rows
    fbp_ctf computes for a contiguous range, in both precisions."""
    rng = np.random.default_rng(2)
    T, H, W, Z = 7, 12, 40, 30
    ang = np.deg2rad(np.linspace(-60, 60, T)).astype(np.float32)
    proj = rng.standard_normal((T, H, W)).astype(np.float32)
    c = np.full(H, W / 2, np.float32)
    mn, mx, step, nd = oracle.defocus_steps(25000.0, 3, None, W, c, 1.0)
    ctf = oracle.ctf_stack(W, H, 1.0, 300, mn, nd, step, 2.7)
    rows = np.array([0, 5, 6, 11])
    for prec in ("f32", "f64"):
        full = oracle.fbp_ctf(proj, ang, c, 1.0, ctf, float(mn - 25000.0), float(mx - 25000.0),
                              Z=Z, precision=prec)
        part = oracle.fbp_ctf_rows(proj, ang, c, 1.0, rows, ctf, float(mn - 25000.0),
                                   float(mx - 25000.0), Z=Z, precision=prec)
        np.testing.assert_array_equal(part, full[rows])
