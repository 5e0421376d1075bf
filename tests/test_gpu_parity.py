"""GPU parity: the CUDA path through the C ABI against the oracle and the
golden vectors recorded from the reference.

Tolerances (relative L2 over the whole output):
  * FP32 path vs the reference CPU path (golden / float oracle): 1e-4
  * FP16-staged paths (F16 records, F16T tensor-core rows) vs the FP64 oracle: 1e-3
  * slab indices and phase-flip signs: bit-exact
  * the exact backprojector given the oracle's filtered rows: bit-exact
"""
import math

import numpy as np
import pytest

from conftest import golden, golden_names

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-4
FP16_TOL = 1e-3


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def torch():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from guanaco_gb300 import _lib

    _lib.load()
    return torch


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


# --------------------------------------------------------- reference shapes
def test_filter_matches_reference(torch):
    from guanaco_gb300 import _lib

    g = golden("filter")
    L = _lib.load()
    for k in g:
        if not k.startswith("in_"):
            continue
        x = g[k]
        d, t, n = x.shape
        buf = dev(torch, x)
        _lib.check(L.gnc_filter_device(n, t, d, buf.data_ptr(), None))
        out = buf.cpu().numpy()
        assert rel_l2(out, g["out_" + k[3:]]) < 1e-6


@pytest.mark.parametrize("name", golden_names("recon_"))
def test_recon_matches_reference(torch, name):
    from guanaco_gb300 import detail

    g = golden(name)
    rec = np.zeros_like(g["rec"])
    detail.recon(g["sino"], rec, g["angles"], float(g["centre"]), float(g["pixel_size"]),
                 float(g["min_defocus"]), float(g["max_defocus"]), "gpu")
    assert rel_l2(rec, g["rec"]) < FP32_TOL


@pytest.mark.parametrize("name", golden_names("config_"))
def test_config_grid_matches_reference(torch, name):
    from guanaco_gb300 import detail

    g = golden(name)
    rec = np.zeros_like(g["rec"])
    sino = g["sino"] if g["sino"].shape[0] > 1 else g["sino"][0]
    detail.recon_grid(sino, rec, g["angles"], float(g["centre"]), float(g["pixel_size"]),
                      float(g["min_defocus"]), float(g["max_defocus"]))
    assert rel_l2(rec, g["rec"]) < FP32_TOL


@pytest.mark.parametrize("name", golden_names("corr_"))
def test_corr_matches_reference(torch, name):
    from guanaco_gb300 import detail

    g = golden(name)
    rec = np.zeros_like(g["rec"])
    ctf = g["ctf"] if g["ctf"].shape[0] > 1 else g["ctf"][0]
    out = rec if g["ctf"].shape[0] > 1 else rec[0]
    detail.corr(g["image"], ctf, out, "gpu")
    assert rel_l2(rec, g["rec"]) < 1e-5


@pytest.mark.parametrize("name", golden_names("pipeline_"))
def test_pipeline_matches_reference(torch, name):
    import guanaco_gb300 as G

    g = golden(name)
    proj, ang, centre = g["proj"], g["angles"], g["centre"]
    df = None if math.isnan(float(g["defocus"])) else float(g["defocus"])
    sdf = None if math.isnan(float(g["step_defocus"])) else float(g["step_defocus"])
    ndf = int(g["num_defocus"]) or None
    kw = dict(centre=centre, pixel_size=float(g["pixel_size"]), energy=float(g["energy"]),
              defocus=df, num_defocus=ndf, step_defocus=sdf,
              spherical_aberration=float(g["Cs"]), phase_shift=float(g["phase_shift"]))
    # two calls, as the reference's reconstruct_file makes them
    cp, mn, mx = G.correct_projections(proj, device="gpu", **{k: v for k, v in kw.items()})
    if df is not None:
        assert rel_l2(cp, g["corrected"].reshape(cp.shape)) < 1e-5
        assert np.float32(mn) == np.float32(g["min_defocus"])
    vol = G.reconstruct(cp, ang, None, centre, float(g["pixel_size"]), mn, mx,
                        transform="minus" if bool(g["minus"]) else None,
                        angular_weights=bool(g["angular_weights"]), device="gpu")
    assert rel_l2(vol, g["volume"]) < FP32_TOL
    # one fused device pass
    vol2 = G.reconstruct_ctf(proj, ang, transform="minus" if bool(g["minus"]) else None,
                             angular_weights=bool(g["angular_weights"]), **kw)
    assert rel_l2(vol2, g["volume"]) < FP32_TOL


# ------------------------------------------------------------ bit-exactness
def _plan_case(oracle, T=17, H=12, W=48, Z=40, D=5, ps=1.0, Ca=0.0, phi=0.0, df=25000.0,
               staging="f32", centre=None, weights=None, minus=False, seed=0, angles=None):
    import guanaco_gb300 as G

    rng = np.random.default_rng(seed)
    ang = (np.deg2rad(np.linspace(-60, 60, T)) if angles is None else angles).astype(np.float32)
    c = G.get_centre((T, H, W), centre, False)
    mn, mx, step, nd = G.get_defocus_steps(df, D, None, W, c, ps)
    slabs = G.api.slab_defoci(mn, nd, step)
    plan = G.FbpPlan(T, H, W, ang, grid_height=Z, grid_width=W, centre=c, pixel_size=ps,
                     input="raw", correct=True, num_defocus=nd, slab_defocus=slabs,
                     min_defocus=float(mn - df), max_defocus=float(mx - df), energy=300,
                     spherical_aberration=2.7, astigmatism=Ca, astigmatism_angle=30.0,
                     phase_shift=phi, weights=weights, minus=minus, staging=staging)
    ctf = oracle.ctf_stack(W, H, ps, 300, mn, nd, step, 2.7, Ca, 30.0, phi)
    proj = rng.standard_normal((T, H, W)).astype(np.float32)
    return plan, proj, ang, c, ctf, float(mn - df), float(mx - df)


def _sym_sign(ctf):
    s = -np.sign(ctf.imag.astype(np.float32)).astype(np.int32)
    D, H, W = s.shape
    m = s[:, (-np.arange(H)) % H][:, :, (-np.arange(W)) % W]
    return (s + m)[:, :, : W // 2 + 1].astype(np.int8)


@pytest.mark.parametrize("Ca,phi,ps", [(0.0, 0.0, 1.0), (0.0, 5.0, 1.35), (600.0, 2.0, 0.8)])
def test_sign_table_bit_exact(torch, oracle, Ca, phi, ps):
    plan, proj, *_ , ctf, mn, mx = _plan_case(oracle, H=36, W=40, D=4, ps=ps, Ca=Ca, phi=phi)
    out = torch.empty((plan.D, plan.H, plan.W // 2 + 1), dtype=torch.int8, device="cuda")
    plan.sign_table(out)
    np.testing.assert_array_equal(out.cpu().numpy(), _sym_sign(ctf))


# Full-size tables: millions of signs, many near a sign change, where the float
# screen has to hand over to the FP64 phase.
@pytest.mark.parametrize("H,W,D,Ca,phi,ps,df", [(1024, 1024, 10, 0.0, 0.0, 1.0, 30000.0),
                                                (384, 512, 6, 600.0, 2.0, 0.8, 20000.0),
                                                (243, 500, 5, 300.0, 7.0, 1.3, 40000.0)])
def test_sign_table_bit_exact_large(torch, oracle, H, W, D, Ca, phi, ps, df):
    plan, proj, *_, ctf, mn, mx = _plan_case(oracle, T=3, H=H, W=W, Z=8, D=D, ps=ps, Ca=Ca,
                                             phi=phi, df=df)
    out = torch.empty((plan.D, plan.H, plan.W // 2 + 1), dtype=torch.int8, device="cuda")
    plan.sign_table(out)
    np.testing.assert_array_equal(out.cpu().numpy(), _sym_sign(ctf))


@pytest.mark.parametrize("D,Z", [(5, 40), (10, 33), (3, 64)])
def test_slab_map_bit_exact(torch, oracle, D, Z):
    plan, proj, ang, c, ctf, mn, mx = _plan_case(oracle, D=D, Z=Z)
    out = torch.empty((plan.T, Z, plan.W), dtype=torch.int32, device="cuda")
    plan.slab_map(out)
    ref = oracle.slab_index_map(plan.W, D, (Z, plan.W), ang, float(c[0]), 1.0, mn, mx)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


# The phase flip and the ramp filter run only for the (tilt, slab) pairs some
# voxel reads: per tilt the slab range at the volume's corners, which must be
# exactly the range of the reference's slab index over the whole volume
# (reconstructor.cpp:66-72).  At the 3D-CTF benchmark's shape (1024 px,
# Z = 300, ten slabs) the low tilts read fewer than half of the slabs.
@pytest.mark.parametrize("T,W,Z,D", [(17, 48, 40, 5), (13, 64, 33, 10), (61, 1024, 300, 10),
                                     (9, 256, 256, 4)])
def test_live_slabs_match_slab_map(torch, oracle, T, W, Z, D):
    plan, proj, ang, c, ctf, mn, mx = _plan_case(oracle, T=T, H=4, W=W, Z=Z, D=D)
    live = plan.live_slabs()
    ref = oracle.slab_index_map(W, D, (Z, W), ang, float(c[0]), 1.0, mn, mx).reshape(T, -1)
    np.testing.assert_array_equal(live[:, 0], ref.min(axis=1))
    np.testing.assert_array_equal(live[:, 1], ref.max(axis=1))
    if (W, Z, D) == (1024, 300, 10):
        pairs = int((live[:, 1] - live[:, 0] + 1).sum())
        assert pairs < 0.85 * T * D  # the skipped share this shape relies on
        assert (live[T // 2, 1] - live[T // 2, 0] + 1) <= 4  # the untilted view


def _staged_from_rows(filtered_rows, H):
    """Per-row filtered sinograms (H, D, T, N) -> staged pairs (H2, D, T, N, 2)."""
    Hh, D, T, N = filtered_rows.shape
    H2 = (H + 1) // 2
    st = np.zeros((H2, D, T, N, 2), np.float32)
    for y in range(H):
        st[y // 2, :, :, :, y % 2] = filtered_rows[y]
    return st


def test_exact_backprojector_bit_exact(torch, oracle):
    T, H, W, Z, D = 13, 5, 40, 36, 4
    plan, proj, ang, c, ctf, mn, mx = _plan_case(oracle, T=T, H=H, W=W, Z=Z, D=D, seed=3)
    rng = np.random.default_rng(7)
    rows = rng.standard_normal((H, D, T, W)).astype(np.float32)
    filt = np.stack([oracle.ramp_filter(rows[y], "f32") for y in range(H)])
    staged = dev(torch, _staged_from_rows(filt, H))
    vol = torch.empty((H, Z, W), dtype=torch.float32, device="cuda")
    plan.backproject_staged(staged, None, vol, exact=True)
    got = vol.cpu().numpy()
    for y in range(H):
        ref = oracle.project(filt[y], (Z, W), ang, float(c[y]), 1.0, mn, mx)
        np.testing.assert_array_equal(got[y], ref)


def _f16_records(filt, H, exps):
    """FP16 staged records (H2, D, T, W, 4) = (v_a, v_b, dv_a, dv_b) of rows scaled
    by 2^exps[y, d, t], and the int8 exponents (H2, D, T, 2)."""
    _, D, T, W = filt.shape
    H2 = (H + 1) // 2
    rec = np.zeros((H2, D, T, W, 4), np.float16)
    rexp = np.zeros((H2, D, T, 2), np.int8)
    for y in range(H):
        e = exps[y]
        v = (filt[y] * np.exp2(e).astype(np.float32)[..., None]).astype(np.float16)
        dv = np.zeros_like(v)
        dv[..., :-1] = (v[..., 1:].astype(np.float32) - v[..., :-1].astype(np.float32)).astype(
            np.float16)
        rec[y // 2, ..., y % 2] = v
        rec[y // 2, ..., 2 + y % 2] = dv
        rexp[y // 2, ..., y % 2] = e
    return rec, rexp


# The FP16 backprojector brings every slab of a row pair to one reference
# exponent in shared memory (exact powers of two): the same values staged with
# other per-slab exponents must give the same volume bit for bit, and the
# result must match the exact backprojector on the same FP16 values.
def test_fp16_slab_exponents_are_exact(torch, oracle):
    T, H, W, Z, D = 13, 10, 64, 48, 6
    plan, proj, ang, c, ctf, mn, mx = _plan_case(oracle, T=T, H=H, W=W, Z=Z, D=D, seed=5,
                                                 staging="f16")
    rng = np.random.default_rng(11)
    filt = (rng.uniform(0.5, 1.0, (H, D, T, W)) * rng.choice([-1.0, 1.0], (H, D, T, W)))
    filt = (filt * np.exp2(3.0 * np.arange(D))[None, :, None, None]).astype(np.float32)
    natural = 13 - np.floor(np.log2(np.abs(filt).max(axis=-1))).astype(np.int64)
    shifted = natural - 2 * np.arange(D)[None, :, None]  # slab-dependent, still normal FP16
    vols = []
    for exps in (natural, shifted):
        rec, rexp = _f16_records(filt, H, exps)
        vol = torch.empty((H, Z, W), dtype=torch.float32, device="cuda")
        plan.backproject_staged(dev(torch, rec), dev(torch, rexp), vol, exact=False)
        vols.append(vol.cpu().numpy())
    np.testing.assert_array_equal(vols[1], vols[0])
    rec, rexp = _f16_records(filt, H, natural)
    exact = torch.empty((H, Z, W), dtype=torch.float32, device="cuda")
    plan.backproject_staged(dev(torch, rec), dev(torch, rexp), exact, exact=True)
    assert rel_l2(vols[0], exact.cpu().numpy()) < 5e-4


# ---------------------------------------------------------- whole pipeline
def _oracle_volume(oracle, proj, ang, c, ctf, mn, mx, Z, precision, weights=None, minus=False):
    return oracle.fbp_ctf(proj, ang, c, 1.0, ctf, mn, mx, weights, minus, Z=Z,
                          precision=precision)


@pytest.mark.parametrize("staging", ["f32", "f16", "f16t"])
@pytest.mark.parametrize("shape", [(17, 12, 48, 40, 5), (9, 7, 60, 30, 3), (21, 16, 64, 64, 1)])
def test_pipeline_vs_oracles(torch, oracle, staging, shape):
    T, H, W, Z, D = shape
    plan, proj, ang, c, ctf, mn, mx = _plan_case(oracle, T=T, H=H, W=W, Z=Z, D=D, staging=staging)
    vol = plan.execute_host(proj)
    ref32 = _oracle_volume(oracle, proj, ang, c, ctf, mn, mx, Z, "f32")
    ref64 = _oracle_volume(oracle, proj, ang, c, ctf, mn, mx, Z, "f64")
    if staging == "f32":
        assert rel_l2(vol, ref32) < FP32_TOL
        assert rel_l2(vol, ref64) < FP32_TOL
    else:
        assert rel_l2(vol, ref64) < FP16_TOL


# More tilts than the backprojector holds parameters for at once (128): it
# runs them in chunks.  Tilts of very different magnitude per chunk change the
# FP16 form's common exponent from chunk to chunk, so its accumulators are
# rescaled at each chunk boundary.
@pytest.mark.parametrize("staging", ["f32", "f16", "f16t"])
def test_tilt_chunks_of_different_magnitude(torch, oracle, staging):
    T, H, W, Z, D = 300, 6, 48, 32, 3
    plan, proj, ang, c, ctf, mn, mx = _plan_case(oracle, T=T, H=H, W=W, Z=Z, D=D, staging=staging)
    proj[128:256] *= 40.0
    proj[256:] *= 1.0 / 30.0
    vol = plan.execute_host(proj)
    ref32 = _oracle_volume(oracle, proj, ang, c, ctf, mn, mx, Z, "f32")
    ref64 = _oracle_volume(oracle, proj, ang, c, ctf, mn, mx, Z, "f64")
    if staging == "f32":
        assert rel_l2(vol, ref32) < FP32_TOL
        assert rel_l2(vol, ref64) < FP32_TOL
    else:
        assert rel_l2(vol, ref64) < FP16_TOL


# The same chunk hand-over in the fast backprojector: on a 128-pixel detector
# the tiles span few enough slabs for the fast kernel (4 slabs per tile with 3
# slabs, 2 with 1 slab).  Tilts 128-255 and 256-299 are scaled by different
# magnitudes, so the FP16 form changes its common exponent and rescales its
# accumulators at both chunk boundaries.
@pytest.mark.parametrize("staging", ["f32", "f16"])
@pytest.mark.parametrize("D,variant", [(3, 4), (1, 2)])
def test_fast_backprojector_tilt_chunks(torch, oracle, staging, D, variant):
    T, H, W, Z = 300, 6, 128, 48
    plan, proj, ang, c, ctf, mn, mx = _plan_case(oracle, T=T, H=H, W=W, Z=Z, D=D, staging=staging,
                                                 seed=9)
    assert plan.backprojector == variant
    proj[128:256] *= 40.0
    proj[256:] *= 1.0 / 30.0
    vol = plan.execute_host(proj)
    plan.check()
    ref32 = _oracle_volume(oracle, proj, ang, c, ctf, mn, mx, Z, "f32")
    ref64 = _oracle_volume(oracle, proj, ang, c, ctf, mn, mx, Z, "f64")
    if staging == "f32":
        assert rel_l2(vol, ref32) < FP32_TOL
        assert rel_l2(vol, ref64) < FP32_TOL
    else:
        assert rel_l2(vol, ref64) < FP16_TOL
    exact = torch.empty(plan.volume_shape, dtype=torch.float32, device="cuda")
    plan.stage(dev(torch, proj))
    plan.backproject(exact, exact=True)
    assert rel_l2(vol, exact.cpu().numpy()) < (1e-5 if staging == "f32" else 5e-4)


# F16T staging: FP16 rows with one power-of-two scale per tilt, backprojected
# on the tensor cores (tcgen05.mma, FP32 accumulation in tensor memory).  The
# plan must pick that kernel, match the FP64 oracle within the FP16 tolerance
# and the exact backprojector on the same FP16 rows closely (they differ only
# in the FP16 interpolation weights and the summation order).  Shapes: volume
# edges that cut tiles (X, Z not multiples of 16 and 8, rows not a multiple
# of 128), several slabs per tile, one slab, 300 tilts, a 1024-pixel detector;
# and 1-3 tilts over some 16 tiles per block, where a tile has only one or two
# slab slots, so a group's ring slots were last used several tiles back (the
# wait falls back to the last group two tiles back).
@pytest.mark.parametrize("T,H,W,Z,X,D", [(17, 12, 48, 40, 48, 5), (17, 12, 64, 40, 64, 6),
                                         (9, 130, 64, 37, 64, 3),
                                         (300, 6, 128, 48, 128, 3), (21, 16, 64, 64, 64, 1),
                                         (13, 4, 1024, 300, 1024, 10), (11, 20, 96, 21, 53, 4),
                                         (1, 4, 1024, 300, 1024, 3), (2, 4, 1024, 300, 1024, 3),
                                         (3, 4, 512, 300, 512, 2)])
def test_tensor_core_backprojector(torch, oracle, T, H, W, Z, X, D):
    import guanaco_gb300 as G

    rng = np.random.default_rng(T + W)
    ang = np.deg2rad(np.linspace(-60, 60, T)).astype(np.float32)
    c = G.get_centre((T, H, W), None, False)
    df = 25000.0
    mn, mx, step, nd = G.get_defocus_steps(df, D, None, W, c, 1.0)
    plan = G.FbpPlan(T, H, W, ang, grid_height=Z, grid_width=X, centre=c, correct=True,
                     num_defocus=nd, slab_defocus=G.api.slab_defoci(mn, nd, step),
                     min_defocus=float(mn - df), max_defocus=float(mx - df), energy=300,
                     spherical_aberration=2.7, staging="f16t")
    assert plan.backprojector == 16
    proj = rng.standard_normal((T, H, W)).astype(np.float32)
    inp = dev(torch, proj)
    vol = torch.empty(plan.volume_shape, dtype=torch.float32, device="cuda")
    ref = torch.empty_like(vol)
    plan.stage(inp)
    plan.backproject(vol, exact=False)
    plan.backproject(ref, exact=True)
    plan.check()
    got = vol.cpu().numpy()
    assert rel_l2(got, ref.cpu().numpy()) < 3e-4
    if X == W:  # the oracle's volume is as wide as the detector
        ctf = oracle.ctf_stack(W, H, 1.0, 300, mn, nd, step, 2.7)
        want = oracle.fbp_ctf(proj, ang, c, 1.0, ctf, float(mn - df), float(mx - df), Z=Z,
                              precision="f64")
        assert rel_l2(got, want) < FP16_TOL
    # the whole pipeline through the host-buffer entry point gives the same volume
    np.testing.assert_array_equal(plan.execute_host(proj), got)


def test_tensor_core_staging_falls_back(torch, oracle):
    """Rows with different centres are outside the tensor-core kernel: an F16T
    plan then stages FP16 records for the other backprojectors, within the
    FP16 tolerance of the FP64 oracle."""
    T, H, W, Z = 11, 6, 40, 30
    centre = (W / 2 + np.linspace(-1.5, 2.0, H)).astype(np.float32)
    plan, proj, ang, c, ctf, mn, mx = _plan_case(oracle, T=T, H=H, W=W, Z=Z, D=3, centre=centre,
                                                 staging="f16t")
    assert plan.backprojector == 0
    vol = plan.execute_host(proj)
    ref = _oracle_volume(oracle, proj, ang, c, ctf, mn, mx, Z, "f64")
    assert rel_l2(vol, ref) < FP16_TOL


# The host-buffer entry point overlaps its copies with the kernels (tilt groups
# in, row slabs out; with CTF correction it filters row slab by row slab); it
# must give exactly the device entry point's volume.  Shapes: power-of-two and
# generic rows, an odd row count (a last slab with a single-row pair), and
# 1024-pixel rows: three input groups of at least 8 MB and six volume slabs of
# at least 16 MB, the last split in three.
@pytest.mark.parametrize("staging", ["f32", "f16", "f16t"])
@pytest.mark.parametrize("T,H,W,Z,D,ragged", [(37, 64, 256, 40, 4, False), (19, 90, 128, 30, 3, True),
                                                (9, 22, 64, 48, 1, False), (11, 45, 256, 20, 2, False),
                                                (5, 250, 128, 16, 2, False),
                                                (17, 1024, 1024, 24, 3, False),
                                                (4, 384, 384, 16, 3, False)])
def test_host_pipeline_equals_device_path(torch, oracle, staging, T, H, W, Z, D, ragged):
    centre = None
    if ragged:  # per-row centres: the exact backprojector
        centre = (W / 2 + 0.25 * np.sin(np.arange(H))).astype(np.float32)
    plan, proj, *_ = _plan_case(oracle, T=T, H=H, W=W, Z=Z, D=D, staging=staging, centre=centre)
    want = torch.empty(plan.volume_shape, dtype=torch.float32, device="cuda")
    plan.execute(dev(torch, proj), want)
    torch.cuda.synchronize()
    for _ in range(2):  # the second call reuses the plan's I/O buffers and streams
        got = plan.execute_host(proj)
        np.testing.assert_array_equal(got, want.cpu().numpy())


def test_pipeline_exact_backprojector_equals_fast(torch, oracle):
    plan, proj, ang, c, ctf, mn, mx = _plan_case(oracle, T=15, H=10, W=64, Z=48, D=6)
    inp = dev(torch, proj)
    a = torch.empty(plan.volume_shape, dtype=torch.float32, device="cuda")
    b = torch.empty_like(a)
    plan.stage(inp)
    plan.backproject(a, exact=True)
    plan.backproject(b, exact=False)
    assert rel_l2(b.cpu().numpy(), a.cpu().numpy()) < 1e-5


def test_weights_minus_and_offcentre_rows(torch, oracle):
    T, H, W, Z = 11, 6, 40, 30
    ang = np.deg2rad(np.linspace(-60, 60, T)).astype(np.float32)
    import guanaco_gb300 as G

    w = G.compute_angular_weights(ang)
    centre = (W / 2 + np.linspace(-1.5, 2.0, H)).astype(np.float32)
    plan, proj, ang, c, ctf, mn, mx = _plan_case(oracle, T=T, H=H, W=W, Z=Z, D=3, centre=centre,
                                                 weights=w, minus=True)
    vol = plan.execute_host(proj)
    ref = _oracle_volume(oracle, proj, ang, c, ctf, mn, mx, Z, "f32", weights=w, minus=True)
    assert rel_l2(vol, ref) < FP32_TOL


@pytest.mark.parametrize("H", [1, 3, 8])
def test_odd_and_tiny_heights(torch, oracle, H):
    plan, proj, ang, c, ctf, mn, mx = _plan_case(oracle, T=7, H=H, W=32, Z=20, D=2)
    vol = plan.execute_host(proj)
    ref = _oracle_volume(oracle, proj, ang, c, ctf, mn, mx, 20, "f32")
    assert rel_l2(vol, ref) < FP32_TOL


def test_wide_tilt_range_and_single_tilt(torch, oracle):
    ang = np.deg2rad(np.linspace(-90, 90, 9)).astype(np.float32)
    plan, proj, ang, c, ctf, mn, mx = _plan_case(oracle, T=9, H=4, W=32, Z=32, D=4, angles=ang)
    vol = plan.execute_host(proj)
    ref = _oracle_volume(oracle, proj, ang, c, ctf, mn, mx, 32, "f32")
    assert rel_l2(vol, ref) < FP32_TOL
    one = np.array([0.2], np.float32)
    plan, proj, ang, c, ctf, mn, mx = _plan_case(oracle, T=1, H=2, W=32, Z=16, D=1, angles=one)
    vol = plan.execute_host(proj)
    ref = _oracle_volume(oracle, proj, ang, c, ctf, mn, mx, 16, "f32")
    assert rel_l2(vol, ref) < FP32_TOL


def test_correct_only_matches_oracle(torch, oracle):
    plan, proj, ang, c, ctf, mn, mx = _plan_case(oracle, T=5, H=30, W=40, D=3)
    out = torch.empty((plan.T, plan.D, plan.H, plan.W), dtype=torch.float32, device="cuda")
    plan.correct(dev(torch, proj), out)
    got = out.cpu().numpy()
    for t in range(plan.T):
        assert rel_l2(got[t], oracle.correct(proj[t], ctf)) < 1e-5


def test_linearity_at_full_detector_width(torch, oracle):
    """Size-independent check at the 1024-px detector of the 3D-CTF config:
    the path is linear in the projections."""
    import guanaco_gb300 as G

    T, H, W, Z, D = 9, 4, 1024, 64, 10
    ang = np.deg2rad(np.linspace(-60, 60, T)).astype(np.float32)
    c = G.get_centre((T, H, W), None, False)
    mn, mx, step, nd = G.get_defocus_steps(30000.0, D, None, W, c, 1.0)
    plan = G.FbpPlan(T, H, W, ang, grid_height=Z, centre=c, correct=True, num_defocus=nd,
                     slab_defocus=G.api.slab_defoci(mn, nd, step), min_defocus=float(mn - 30000),
                     max_defocus=float(mx - 30000), energy=300, spherical_aberration=2.7)
    rng = np.random.default_rng(5)
    a = rng.standard_normal((T, H, W)).astype(np.float32)
    b = rng.standard_normal((T, H, W)).astype(np.float32)
    va, vb = plan.execute_host(a), plan.execute_host(b)
    vab = plan.execute_host((2.0 * a - 0.5 * b).astype(np.float32))
    assert rel_l2(vab, 2.0 * va - 0.5 * vb) < 1e-5


# ------------------------------------------- power-of-two transform lengths
@pytest.mark.parametrize("staging", ["f32", "f16", "f16t"])
@pytest.mark.parametrize("shape", [(5, 256, 1024, 48, 3), (7, 512, 256, 64, 4),
                                   (3, 1024, 256, 32, 2), (6, 243, 512, 40, 5),
                                   (3, 2048, 256, 16, 2), (2, 4096, 128, 16, 3),
                                   (2, 16, 4096, 16, 3), (4, 128, 384, 32, 3),
                                   (3, 384, 128, 40, 2), (2, 384, 384, 24, 4)])
def test_pipeline_pow2_sizes_vs_oracles(torch, oracle, staging, shape):
    T, H, W, Z, D = shape
    plan, proj, ang, c, ctf, mn, mx = _plan_case(oracle, T=T, H=H, W=W, Z=Z, D=D, staging=staging,
                                                 seed=11)
    vol = plan.execute_host(proj)
    plan.check()
    if staging == "f32":
        ref = _oracle_volume(oracle, proj, ang, c, ctf, mn, mx, Z, "f32")
        assert rel_l2(vol, ref) < FP32_TOL
    else:
        ref = _oracle_volume(oracle, proj, ang, c, ctf, mn, mx, Z, "f64")
        assert rel_l2(vol, ref) < FP16_TOL


@pytest.mark.parametrize("W", [128, 256, 384, 512, 2048, 4096])
def test_plain_filter_pow2_vs_oracle(torch, oracle, W):
    """No CTF: the projections are ramp filtered and backprojected directly."""
    import guanaco_gb300 as G

    T, H, Z = 9, 6, 40
    rng = np.random.default_rng(W)
    ang = np.deg2rad(np.linspace(-60, 60, T)).astype(np.float32)
    proj = rng.standard_normal((T, H, W)).astype(np.float32)
    c = G.get_centre(proj.shape, None, False)
    plan = G.FbpPlan(T, H, W, ang, grid_height=Z, centre=c, correct=False)
    vol = plan.execute_host(proj)
    ref = oracle.fbp_ctf(proj, ang, c, 1.0, None, Z=Z)
    assert rel_l2(vol, ref) < FP32_TOL
    from guanaco_gb300 import _lib

    rows = rng.standard_normal((3, 4, W)).astype(np.float32)
    buf = dev(torch, rows)
    _lib.check(_lib.load().gnc_filter_device(W, 4, 3, buf.data_ptr(), None))
    assert rel_l2(buf.cpu().numpy(), oracle.ramp_filter(rows)) < 1e-6


@pytest.mark.parametrize("T,H,W,D", [(3, 256, 512, 4), (2, 16, 4096, 3), (1, 4096, 64, 2),
                                     (2, 384, 128, 3), (2, 128, 384, 2)])
def test_correct_only_pow2(torch, oracle, T, H, W, D):
    plan, proj, ang, c, ctf, mn, mx = _plan_case(oracle, T=T, H=H, W=W, D=D, seed=4)
    out = torch.empty((plan.T, plan.D, plan.H, plan.W), dtype=torch.float32, device="cuda")
    plan.correct(dev(torch, proj), out)
    got = out.cpu().numpy()
    for t in range(plan.T):
        assert rel_l2(got[t], oracle.correct(proj[t], ctf)) < 1e-5


# gpu_list: the Y rows split into contiguous bands, one plan per band on its
# listed device, all bands at once (here every band on device 0).  Rows are
# independent, so the FP32 volume equals the unsplit one bit for bit, also
# for a four-dimensional (corrected, several slabs) input with per-row centres.
def test_reconstruct_gpu_list_row_bands(torch):
    import guanaco_gb300 as G

    rng = np.random.default_rng(21)
    T, H, W = 13, 21, 64
    ang = np.deg2rad(np.linspace(-60, 60, T)).astype(np.float32)
    proj = rng.standard_normal((T, H, W)).astype(np.float32)
    whole = G.reconstruct(proj, ang, device="gpu")
    split = G.reconstruct(proj, ang, device="gpu", gpu_list=[0, 0, 0])
    np.testing.assert_array_equal(split, whole)
    stack = rng.standard_normal((T, 3, H, W)).astype(np.float32)
    centre = (W / 2 + 0.3 * np.sin(np.arange(H))).astype(np.float32)
    kw = dict(centre=centre, min_defocus=-40.0, max_defocus=40.0, transform="minus",
              angular_weights=True, device="gpu")
    whole = G.reconstruct(stack, ang, **kw)
    split = G.reconstruct(stack, ang, gpu_list=[0, 0], **kw)
    np.testing.assert_array_equal(split, whole)
