"""CTF images on the device (gnc_ctf_image_device, plot.generate_ctf) against
the CTF known answers recorded from the reference (tests/golden/ctf_kat.npz,
the grids of the reference's tests/test_ctf.py) and against the host CTF
class (double) on defocus series with astigmatism.  The device computes in
double and stores float32, so the tolerance is float rounding: 2e-7 of the
largest magnitude (the CTF is at most 1)."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu
TOL = 2e-7


@pytest.fixture(scope="module")
def G():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    import guanaco_gb300 as G

    return G


def test_known_answers(G):
    g = golden("ctf_kat")
    d = G.detail
    l = d.get_electron_wavelength(300000)
    simple = d.CTF(l=l, df=20000, Cs=2.7e7, phi=0.1)
    full = d.CTF(l=l, df=20000, Cs=2.7e7, dd=1, theta_c=0.1 / 1e3, phi=0.1)
    astig = d.CTF(l=l, df=25000, Cs=2.7e7, Ca=800, Pa=0.3, phi=0.05)
    img = lambda c, kind, w, h, ps: G.plot.ctf_images(c, [c.df], w, h, ps, kind)[0].cpu().numpy()
    np.testing.assert_allclose(img(full, "full", 100, 100, 2), g["ctf_full"], rtol=0, atol=TOL)
    np.testing.assert_allclose(img(simple, "simple", 100, 100, 2), g["ctf_simple"], rtol=0,
                               atol=TOL)
    np.testing.assert_allclose(img(simple, "simple_real", 100, 100, 2), g["ctf_simple_real"],
                               rtol=0, atol=TOL)
    np.testing.assert_allclose(img(simple, "simple_imag", 100, 100, 2), g["ctf_simple_imag"],
                               rtol=0, atol=TOL)
    np.testing.assert_allclose(img(astig, "simple", 90, 64, 1.5), g["ctf_simple_astig_90x64"],
                               rtol=0, atol=TOL)


# more defoci than one launch holds (64), odd sizes, astigmatism and envelopes
@pytest.mark.parametrize("kind", ["full", "simple", "chi", "Es", "Et"])
def test_defocus_series_matches_host(G, kind):
    d = G.detail
    c = d.CTF(l=d.get_electron_wavelength(200000), df=0, Cs=2.0e7, Ca=450, Pa=0.7, dd=35,
              theta_c=2e-5, phi=0.08)
    defoci = 12000.0 + 97.5 * np.arange(70)
    got = G.plot.ctf_images(c, defoci, 37, 26, 1.7, kind).cpu().numpy()
    assert got.shape == (70, 26, 37)
    for i in (0, 33, 63, 64, 69):
        c.df = float(defoci[i])
        want = getattr(c, "get_ctf" if kind == "full" else
                       "get_ctf_simple" if kind == "simple" else "_grid")(
            *((37, 26, 1.7) if kind in ("full", "simple") else (kind, 37, 26, 1.7)))
        want = want.astype(np.complex64 if kind in ("full", "simple") else np.float32)
        scale = max(1.0, float(np.abs(want).max()))
        np.testing.assert_allclose(got[i], want, rtol=0, atol=TOL * scale)


@pytest.mark.parametrize("recentre", [False, True])
def test_generate_ctf_writes_complex_mrc(G, tmp_path, recentre):
    path = str(tmp_path / "ctf.mrc")
    G.plot.generate_ctf(path, image_size=(48, 60), pixel_size=1.3, defocus=20000,
                        num_defocus=5, step_defocus=400, spherical_aberration=2.7,
                        astigmatism=300, astigmatism_angle=25, energy=300, recentre=recentre)
    with G.mrc.open_mrc(path) as f:
        assert int(f.header["mode"]) == 4
        assert f.voxel_size["x"] == pytest.approx(1.3)
        data = np.array(f.data)
    assert data.shape == (5, 48, 60) and data.dtype == np.complex64
    d = G.detail
    dd = d.get_defocus_spread(Cc=2.7e7, dEE=0.33e-6, dII=0.33e-6, dVV=0.8e-6)
    for i in range(5):
        c = d.CTF(l=d.get_electron_wavelength(300e3), df=20000 + (i - 2) * 400, Cs=2.7e7,
                  Ca=300, Pa=25 * np.pi / 180, dd=dd, theta_c=0.02 / 1e3, phi=0)
        want = c.get_ctf(60, 48, 1.3).astype(np.complex64)
        if recentre:
            want = np.fft.fftshift(want)
        np.testing.assert_allclose(data[i], want, rtol=0, atol=TOL)


def test_invalid_arguments_fail_before_any_launch(G):
    from guanaco_gb300 import _lib

    c = G.detail.CTF(l=0.02, df=1000)
    with pytest.raises(_lib.GncError) as e:
        G.plot.ctf_images(c, [1000.0], 16, 16, 0.0)
    assert e.value.status == _lib.GNC_ERR_INVALID_ARGUMENT
    with pytest.raises(ValueError):
        G.plot.ctf_images(c, [1000.0], 16, 16, 1.0, kind="phase")
