"""The request server (gnc_server_*): continuous batching of FBP requests.

Every served result must equal the result of the same request run alone
through its own plan (gnc_fbp_execute_host) bit for bit -- the same kernels on
the same data, whatever else shares the GPU -- which is within any tolerance
the FP32 (1e-4) and FP16 (1e-3) forms state.  Admission must respect the
device-memory budget, releasing idle cached plans when a new shape needs the
memory, and oversize or invalid requests fail at submission.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    import guanaco_gb300 as G
    from guanaco_gb300 import _lib

    _lib.load()
    return G


def _request(G, n, T, D, staging, seed, df=20000.0):
    """Desc and seeded input of one request: n x n projections, volume n x n/2 x n."""
    rng = np.random.default_rng(seed)
    ang = np.deg2rad(np.linspace(-60, 60, T)).astype(np.float32)
    c = G.get_centre((T, n, n), None, False)
    mn, mx, step, nd = G.get_defocus_steps(df, D, None, n, c, 1.0)
    kw = dict(grid_height=n // 2, grid_width=n, centre=c, pixel_size=1.0, input="raw",
              correct=True, num_defocus=nd, slab_defocus=G.api.slab_defoci(mn, nd, step),
              min_defocus=float(mn - df), max_defocus=float(mx - df), energy=300.0,
              spherical_aberration=2.7, staging=staging)
    proj = rng.standard_normal((T, n, n)).astype(np.float32)
    return (T, n, n, ang), kw, proj


def _alone(G, args, kw, proj):
    plan = G.FbpPlan(*args, **kw)
    try:
        return plan.execute_host(proj)
    finally:
        plan.close()


# (size, tilts, ndf, staging): repeated shapes replay a captured graph
MIX = [(64, 11, 3, "f32"), (128, 21, 5, "f16"), (96, 9, 1, "f32"), (64, 11, 3, "f32"),
       (128, 15, 4, "f32"), (64, 11, 3, "f16"), (128, 21, 5, "f16"), (96, 9, 1, "f32"),
       (64, 11, 3, "f32"), (160, 13, 2, "f16"), (128, 15, 4, "f32"), (64, 11, 3, "f32"),
       (128, 13, 3, "f16t"), (128, 13, 3, "f16t")]

# The sizes and parameter ranges of the benchmark's serving stream (256^2,
# 384^2 and 512^2 projections through the 1024-pixel-class register
# transforms, 31-61 tilts, up to ten slabs, FP32, FP16 and F16T staging).
MIX_LARGE = [(256, 31, 7, "f32"), (384, 41, 10, "f16"), (512, 31, 4, "f16t"),
             (256, 31, 7, "f32"), (512, 61, 10, "f32"), (384, 41, 10, "f16t"),
             (256, 41, 2, "f16"), (512, 31, 4, "f16t"), (384, 31, 1, "f32"),
             (256, 31, 7, "f32")]


@pytest.mark.parametrize("mix,slots", [(MIX, 4), (MIX_LARGE, 6)], ids=["small", "large"])
def test_served_results_equal_alone(G, mix, slots):
    from guanaco_gb300 import serve

    reqs = []
    for i, (n, T, D, st) in enumerate(mix):
        args, kw, proj = _request(G, n, T, D, st, seed=i, df=15000.0 + 2500.0 * i)
        reqs.append((args, kw, proj, _alone(G, args, kw, proj)))
    with serve.Server(budget_bytes=16 << 30, slots=slots) as srv:
        ids, outs = [], []
        for args, kw, proj, _ in reqs:  # all in flight together
            desc = G.FbpDesc(*args, **kw)
            inp = serve.pinned_empty(proj.shape)
            inp[...] = proj
            out = serve.pinned_empty(desc.volume_shape)
            out[...] = np.nan
            ids.append(srv.submit(desc, inp, out))
            outs.append(out)
        infos = [srv.wait(i) for i in ids]
        stats = srv.stats()
    for (args, kw, proj, want), got, info in zip(reqs, outs, infos):
        assert info["status"] == 0 and not info["device_error"]
        assert info["t_submit"] <= info["t_start"] <= info["t_done"]
        np.testing.assert_array_equal(got, want)
    assert stats["completed"] == len(mix) and stats["failed"] == 0
    assert stats["graph_launches"] > 0          # repeated shapes replayed their graph
    assert stats["peak_in_flight"] > 1          # requests overlapped on the device
    assert stats["plans_created"] < len(mix)    # shapes shared plans


def test_budget_admission_releases_idle_plans(G):
    from guanaco_gb300 import serve

    shapes = [(128, 21, 5, "f32"), (160, 13, 2, "f16"), (96, 9, 1, "f32"), (128, 15, 4, "f16")]
    descs = []
    for i, (n, T, D, st) in enumerate(shapes):
        args, kw, proj = _request(G, n, T, D, st, seed=100 + i)
        descs.append((G.FbpDesc(*args, **kw), proj, args, kw))
    # room for about the largest plan only: new shapes have to release idle ones
    big = 0
    for d, proj, args, kw in descs:
        plan = G.FbpPlan(*args, **kw)
        big = max(big, plan.workspace_bytes + 4 * (int(np.prod(d.input_shape)) +
                                                   int(np.prod(d.volume_shape))))
        plan.close()
    with serve.Server(budget_bytes=big + (1 << 20), slots=2) as srv:
        ids, outs = [], []
        for d, proj, _, _ in descs * 2:
            out = np.full(d.volume_shape, np.nan, np.float32)
            ids.append(srv.submit(d, proj, out))
            outs.append(out)
        for i in ids:
            srv.wait(i)
        stats = srv.stats()
    assert stats["completed"] == 2 * len(shapes)
    assert stats["plans_evicted"] > 0
    assert stats["bytes_in_use"] <= big + (1 << 20)
    for (d, proj, args, kw), out in zip(descs * 2, outs):
        np.testing.assert_array_equal(out, _alone(G, args, kw, proj))


def test_oversize_and_invalid_requests_fail_at_submit(G):
    from guanaco_gb300 import _lib, serve

    args, kw, proj = _request(G, 128, 21, 5, "f32", seed=7)
    d = G.FbpDesc(*args, **kw)
    out = np.empty(d.volume_shape, np.float32)
    with serve.Server(budget_bytes=1 << 20, slots=2) as srv:
        with pytest.raises(_lib.GncError) as e:
            srv.submit(d, proj, out)
        assert e.value.status == _lib.GNC_ERR_OUT_OF_MEMORY
    kw_bad = dict(kw)
    args_bad = (21, 128, 127, args[3])  # odd width with CTF correction
    d_bad = G.FbpDesc(*args_bad, **kw_bad)
    with serve.Server(budget_bytes=1 << 30, slots=2) as srv:
        with pytest.raises(_lib.GncError) as e:
            srv.submit(d_bad, np.zeros(d_bad.input_shape, np.float32),
                       np.empty(d_bad.volume_shape, np.float32))
        assert e.value.status == _lib.GNC_ERR_UNSUPPORTED


def test_wait_any_reports_each_request_once_in_finishing_order(G):
    from guanaco_gb300 import serve

    shapes = [(64, 11, 3, "f32"), (128, 21, 5, "f16"), (96, 9, 1, "f32"), (64, 11, 3, "f32"),
              (128, 13, 3, "f16t"), (96, 9, 1, "f32")]
    reqs = []
    for i, (n, T, D, st) in enumerate(shapes):
        args, kw, proj = _request(G, n, T, D, st, seed=200 + i)
        reqs.append((G.FbpDesc(*args, **kw), proj, _alone(G, args, kw, proj)))
    with serve.Server(budget_bytes=8 << 30, slots=3) as srv:
        assert srv.wait_any(0.0) is None  # nothing outstanding: no wait
        outs, ids = {}, []
        for d, proj, want in reqs:
            out = np.full(d.volume_shape, np.nan, np.float32)
            rid = srv.submit(d, proj, out)
            ids.append(rid)
            outs[rid] = (out, want)
        # one collected by id first; wait_any then reports each other request once
        first = srv.wait(ids[2])
        seen = []
        while True:
            got = srv.wait_any(None)
            if got is None:
                break
            seen.append(got)
        assert srv.wait_any(None) is None  # all collected: returns at once
    assert sorted(r for r, _ in seen) == sorted(ids[:2] + ids[3:])
    done_times = [info["t_done"] for _, info in seen]
    assert done_times == sorted(done_times)  # in the order the requests finished
    assert first["status"] == 0
    for rid, (out, want) in outs.items():
        np.testing.assert_array_equal(out, want)
