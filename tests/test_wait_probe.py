"""Failure detection of the bounded device waits, without a GPU fault.

Every mbarrier wait in the fast and the tensor-core backprojectors gives up
after a bounded number of polls and records the timeout in the plan's device
error word, which gnc_fbp_check and the request server report.
gnc_debug_wait_probe makes the give-up happen on purpose: each backprojection
launch of a plan created while it is on arms a spare mbarrier for 16 bytes that
no copy ever delivers and waits on it for a short, bounded number of polls.
Nothing is in flight on that barrier, so the kernel ends normally and the
context stays usable; the tests check the reported status, that it clears, that the volume is unchanged
and that plans created after the probe is turned off report nothing.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PROBE_POLLS = 1 << 10


@pytest.fixture(scope="module")
def env():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    import guanaco_gb300 as G
    from guanaco_gb300 import _lib

    L = _lib.load()
    yield torch, G, _lib, L
    L.gnc_debug_wait_probe(0)


def _series(G, T=9, n=128, Z=48, D=2, staging="f32", df=20000.0, seed=3):
    rng = np.random.default_rng(seed)
    ang = np.deg2rad(np.linspace(-60, 60, T)).astype(np.float32)
    c = G.get_centre((T, n, n), None, False)
    mn, mx, step, nd = G.get_defocus_steps(df, D, None, n, c, 1.0)
    desc = dict(grid_height=Z, grid_width=n, centre=c, pixel_size=1.0, input="raw",
                correct=True, num_defocus=nd, slab_defocus=G.api.slab_defoci(mn, nd, step),
                min_defocus=float(mn - df), max_defocus=float(mx - df), energy=300.0,
                spherical_aberration=2.7, staging=staging)
    proj = rng.standard_normal((T, n, n)).astype(np.float32)
    return (T, n, n, ang), desc, proj


@pytest.mark.parametrize("staging", ["f32", "f16", "f16t"])
def test_wait_that_gives_up_is_reported_by_check(env, staging):
    torch, G, _lib, L = env
    args, desc, proj = _series(G, staging=staging)
    clean = G.FbpPlan(*args, **desc)
    # the probe lives in the fast and the tensor-core backprojectors
    assert clean.backprojector > 0
    if staging == "f16t":
        assert clean.backprojector == 16
    want = clean.execute_host(proj)
    clean.check()
    clean.close()

    _lib.check(L.gnc_debug_wait_probe(PROBE_POLLS))
    try:
        plan = G.FbpPlan(*args, **desc)
    finally:
        _lib.check(L.gnc_debug_wait_probe(0))
    d_in = torch.from_numpy(proj).cuda()
    vol = torch.empty(plan.volume_shape, dtype=torch.float32, device="cuda")
    plan.execute(d_in, vol)
    with pytest.raises(_lib.GncError) as e:
        plan.check()
    assert e.value.status == _lib.GNC_ERR_CUDA
    assert "gave up" in str(e.value)
    plan.check()  # the error word was cleared by the report
    # the give-up is reported, not a fault: the context still works and the
    # volume is the one the plan without the probe computed
    np.testing.assert_array_equal(vol.cpu().numpy(), want)
    got = plan.execute_host(proj)  # a second run reports the timeout again
    np.testing.assert_array_equal(got, want)
    with pytest.raises(_lib.GncError):
        plan.check()
    plan.close()
    # plans created after the probe was turned off report nothing
    after = G.FbpPlan(*args, **desc)
    np.testing.assert_array_equal(after.execute_host(proj), want)
    after.check()
    after.close()


def test_server_reports_device_error(env):
    torch, G, _lib, L = env
    from guanaco_gb300 import serve

    args, desc, proj = _series(G, T=11, n=128, Z=64, D=2)
    d = G.FbpDesc(*args, **desc)
    _lib.check(L.gnc_debug_wait_probe(PROBE_POLLS))
    try:
        with serve.Server(budget_bytes=4 << 30, slots=2) as srv:
            ids = [srv.submit(d, proj, serve.pinned_empty(d.volume_shape)) for _ in range(3)]
            for rid in ids:  # direct launches for the first, graph replays after
                with pytest.raises(_lib.GncError) as e:
                    srv.wait(rid)
                assert e.value.status == _lib.GNC_ERR_CUDA
                assert e.value.info["device_error"]
            st = srv.stats()
            assert st["failed"] == 3 and st["completed"] == 0
    finally:
        _lib.check(L.gnc_debug_wait_probe(0))
    # a server whose plans are created without the probe serves normally
    with serve.Server(budget_bytes=4 << 30, slots=2) as srv:
        out = serve.pinned_empty(d.volume_shape)
        info = srv.wait(srv.submit(d, proj, out))
        assert not info["device_error"] and info["status"] == _lib.GNC_OK
    plan = G.FbpPlan(*args, **desc)
    np.testing.assert_array_equal(out, plan.execute_host(proj))
    plan.close()
