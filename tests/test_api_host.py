"""Host-side mirrors of the reference's Python helpers: they must give the
same numbers (and numpy scalar types) as the reference's code."""
import math

import numpy as np
import pytest

from conftest import golden, golden_names


@pytest.mark.parametrize("name", golden_names("pipeline_"))
def test_defocus_steps_match_reference(oracle, name):
    from guanaco_gb300 import api

    g = golden(name)
    if math.isnan(float(g["defocus"])):
        pytest.skip("no CTF in this fixture")
    T, H, W = g["proj"].shape
    df = float(g["defocus"])
    sdf = None if math.isnan(float(g["step_defocus"])) else float(g["step_defocus"])
    nd = int(g["num_defocus"])
    mine = api.get_defocus_steps(df, nd, sdf, W, g["centre"], float(g["pixel_size"]))
    theirs = oracle.defocus_steps(df, nd, sdf, W, g["centre"], float(g["pixel_size"]))
    assert [type(v) for v in mine] == [type(v) for v in theirs]
    assert mine == theirs
    assert np.float32(mine[0] - df) == np.float32(g["min_defocus"])
    assert np.float32(mine[1] - df) == np.float32(g["max_defocus"])
    slabs = api.slab_defoci(mine[0], mine[3], mine[2])
    ctf = oracle.ctf_stack(W, H, float(g["pixel_size"]), 300, mine[0], mine[3], mine[2], 2.7)
    ctf2 = api.get_ctf_array(W, H, float(g["pixel_size"]), 300, mine[0], mine[3], mine[2], 2.7)
    np.testing.assert_array_equal(ctf, ctf2)
    assert slabs.shape == (mine[3],)


def test_angular_weights_match_numpy_semantics():
    from guanaco_gb300 import api

    from test_oracle_golden import angular_weights

    for ang in (np.deg2rad(np.linspace(-60, 60, 13)).astype(np.float32),
                np.deg2rad(np.array([10, -50, 30, 0, -20, 60, 45], np.float32)),
                np.array([0.3], np.float32)):
        np.testing.assert_array_equal(api.compute_angular_weights(ang), angular_weights(ang))
    np.testing.assert_array_equal(api.get_weights(np.zeros(4, np.float32)), np.ones(4))


def test_get_centre_shapes():
    from guanaco_gb300 import api

    c = api.get_centre((10, 5, 32), None, sinogram_order=False)
    assert c.shape == (5,) and c.dtype == np.float32 and c[0] == 16.0
    c = api.get_centre((5, 10, 32), 12.5)
    assert c.shape == (5,) and np.all(c == 12.5)


def test_public_functions_refuse_the_cpu_path():
    """No CPU fallback behind the public functions: device="cpu" (the
    reference's default) raises instead of computing on the host."""
    import guanaco_gb300 as G

    proj = np.zeros((3, 4, 8), np.float32)
    with pytest.raises(RuntimeError, match="device path only"):
        G.reconstruct(proj, np.zeros(3, np.float32), device="cpu")
    with pytest.raises(RuntimeError, match="device path only"):
        G.correct_projections(proj, device="cpu")


def test_row_bands_split_like_the_reference():
    """The gpu_list split of api.reconstruct: contiguous bands with the
    leftover rows on the first bands (mp.py:9-35)."""
    from guanaco_gb300 import api

    assert api.row_bands(10, 3) == [(0, 4), (4, 7), (7, 10)]
    assert api.row_bands(4, 4) == [(0, 1), (1, 2), (2, 3), (3, 4)]
    assert api.row_bands(2, 3) == [(0, 1), (1, 2), (2, 2)]
    for n, k in [(1024, 7), (5, 2), (0, 1)]:
        b = api.row_bands(n, k)
        assert b[0][0] == 0 and b[-1][1] == n
        assert all(b[i][1] == b[i + 1][0] for i in range(k - 1))
        assert max(y1 - y0 for y0, y1 in b) - min(y1 - y0 for y0, y1 in b) <= 1
