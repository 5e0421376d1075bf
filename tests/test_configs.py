"""Parity at the shapes of the two smaller benchmark configurations, on seeded
blob phantoms (the reference publishes no dataset):

* plain FBP: 61 tilts over +-60 deg (2 deg steps), 256 x 256 projections at
  1.0 A/px, no CTF, volume 256 x 128 x 256 (Y, Z, X);
* single-defocus CTF phase flip: 41 tilts over +-60 deg (3 deg steps),
  512 x 512 projections at 1.35 A/px, 300 kV, Cs 2.7 mm, defocus 20000 A,
  volume 512 x 256 x 512 (the oracle checks a band of 48 rows).

FP32 against the reference CPU path (float oracle) and the FP64 oracle within
1e-4 relative L2; FP16 staging against the FP64 oracle within 1e-3.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-4
FP16_TOL = 1e-3


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def G():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    import guanaco_gb300 as G

    return G


def _series(G, T, n, Z, blobs, seed, defocus=None, pixel_size=1.0):
    from guanaco_gb300 import synthetic

    ang = np.deg2rad(np.linspace(-60, 60, T)).astype(np.float32)
    phantom = synthetic.blob_phantom(blobs, n, n, Z, seed)
    proj = synthetic.tilt_series(phantom, ang, n, n, pixel_size=pixel_size, defocus=defocus,
                                 noise=0.05, seed=seed).cpu().numpy()
    return ang, proj


@pytest.mark.parametrize("staging", ["f32", "f16"])
def test_plain_fbp_256(G, oracle, staging):
    T, n, Z = 61, 256, 128
    ang, proj = _series(G, T, n, Z, 200, seed=0)
    c = G.get_centre((T, n, n), None, False)
    plan = G.FbpPlan(T, n, n, ang, grid_height=Z, grid_width=n, centre=c, input="raw",
                     correct=False, staging=staging)
    vol = plan.execute_host(proj)
    plan.close()
    ref64 = oracle.fbp_ctf(proj, ang, c, 1.0, None, Z=Z, precision="f64")
    if staging == "f32":
        ref32 = oracle.fbp_ctf(proj, ang, c, 1.0, None, Z=Z, precision="f32")
        assert rel_l2(vol, ref32) < FP32_TOL
        assert rel_l2(vol, ref64) < FP32_TOL
    else:
        assert rel_l2(vol, ref64) < FP16_TOL


@pytest.mark.parametrize("staging", ["f32", "f16"])
def test_single_defocus_ctf_512(G, oracle, staging):
    T, n, Z, ps, df = 41, 512, 256, 1.35, 20000.0
    ang, proj = _series(G, T, n, Z, 500, seed=1, defocus=df, pixel_size=ps)
    c = G.get_centre((T, n, n), None, False)
    mn, mx, step, nd = G.get_defocus_steps(df, None, None, n, c, ps)
    assert nd == 1
    plan = G.FbpPlan(T, n, n, ang, grid_height=Z, grid_width=n, centre=c, pixel_size=ps,
                     input="raw", correct=True, num_defocus=1,
                     slab_defocus=G.api.slab_defoci(mn, nd, step), energy=300.0,
                     spherical_aberration=2.7, staging=staging)
    vol = plan.execute_host(proj)
    plan.close()
    ctf = oracle.ctf_stack(n, n, ps, 300, mn, nd, step, 2.7)
    rows = (n // 2 - 24, n // 2 + 24)
    sl = slice(*rows)
    ref64 = oracle.fbp_ctf(proj, ang, c, ps, ctf, Z=Z, rows=rows, precision="f64")[sl]
    if staging == "f32":
        ref32 = oracle.fbp_ctf(proj, ang, c, ps, ctf, Z=Z, rows=rows, precision="f32")[sl]
        assert rel_l2(vol[sl], ref32) < FP32_TOL
        assert rel_l2(vol[sl], ref64) < FP32_TOL
    else:
        assert rel_l2(vol[sl], ref64) < FP16_TOL
