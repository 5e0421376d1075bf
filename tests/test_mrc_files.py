"""reconstruct_file / correct_file (reconstruct.py:216-402, correct.py:321-473)
on MRC files: the same volumes as the array entry points, with the angles,
voxel size and defocus carried by the files' headers."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    import guanaco_gb300 as G

    return G


def _write_series(path, proj, angles_deg, pixel_size):
    from guanaco_gb300 import mrc

    with mrc.new_mrc(path, proj.shape, np.float32, pixel_size, fei1=True) as f:
        f.data[...] = proj
        f.extended_header["Alpha tilt"] = angles_deg


def test_reconstruct_file_matches_arrays(G, tmp_path):
    from guanaco_gb300 import mrc

    T, H, W = 17, 12, 48
    rng = np.random.default_rng(4)
    proj = rng.standard_normal((T, H, W)).astype(np.float32)
    deg = np.linspace(-60, 60, T)
    inp, out = str(tmp_path / "tilts.mrc"), str(tmp_path / "rec.mrc")
    _write_series(inp, proj, deg, 1.35)
    kw = dict(energy=300, defocus=25000.0, num_defocus=5, spherical_aberration=2.7)
    vol = G.reconstruct_file(inp, out, device="gpu", **kw)
    want = G.reconstruct_ctf(proj, np.deg2rad(deg).astype(np.float32), pixel_size=1.35, **kw)
    np.testing.assert_array_equal(vol, want)
    g = mrc.open_mrc(out)
    assert g.data.shape == (H, W, W)
    np.testing.assert_array_equal(np.asarray(g.data), want)
    assert abs(g.voxel_size["x"] - 1.35) < 1e-6


def test_correct_file_then_reconstruct_corrected_stack(G, tmp_path):
    from guanaco_gb300 import mrc

    T, H, W = 11, 10, 40
    rng = np.random.default_rng(5)
    proj = rng.standard_normal((T, H, W)).astype(np.float32)
    deg = np.linspace(-60, 60, T)
    inp, corr, out = (str(tmp_path / n) for n in ("tilts.mrc", "corr.mrc", "rec.mrc"))
    _write_series(inp, proj, deg, 1.0)
    kw = dict(energy=300, defocus=20000.0, num_defocus=4, spherical_aberration=2.7)
    G.correct_file(inp, corr, device="gpu", **kw)
    centre = G.get_centre(proj.shape, None, False)  # as correct_file computes it
    c, mn, mx = G.correct_projections(proj, centre, 1.0, device="gpu", **kw)
    g = mrc.open_mrc(corr)
    assert g.data.shape == (T, 4, H, W)
    np.testing.assert_array_equal(np.asarray(g.data), c)
    np.testing.assert_allclose(mrc.fei1_angles_deg(g), deg)
    step = (mx - mn) / 3
    np.testing.assert_allclose(mrc.fei1_defocus(g), mn + step * np.arange(4), rtol=1e-6)
    # the corrected stack through reconstruct_file, defocus range from its records
    vol = G.reconstruct_file(corr, out, device="gpu")
    want = G.reconstruct(c, np.deg2rad(deg).astype(np.float32), None, None, 1.0,
                         float(np.float32(mrc.fei1_defocus(g).min())),
                         float(np.float32(mrc.fei1_defocus(g).max())), device="gpu")
    np.testing.assert_array_equal(vol, want)
