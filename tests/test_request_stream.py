"""The seeded serving request stream (host only): the shapes and parameter
ranges of the mixed serving workload, reproducible from its seed."""
import numpy as np

from guanaco_gb300.synthetic import request_stream


def test_stream_is_seeded_and_sorted():
    a = request_stream(500, 800.0, seed=5)
    b = request_stream(500, 800.0, seed=5)
    assert a == b
    t = [r["arrival"] for r in a]
    assert t[0] == 0.0 and all(x <= y for x, y in zip(t, t[1:]))
    assert request_stream(500, 800.0, seed=6) != a


def test_stream_ranges():
    s = request_stream(4000, 1000.0, seed=1)
    assert {r["size"] for r in s} == {128, 256, 384, 512}
    assert {r["tilts"] for r in s} == {31, 41, 61}
    assert {r["ndf"] for r in s} == set(range(1, 11))
    assert {r["staging"] for r in s} == {"f16t", "f32"}
    assert {r["staging"] for r in request_stream(200, 1000.0, seed=1, f16_form="f16")} == {
        "f16", "f32"}
    assert all(10000.0 <= r["defocus"] <= 50000.0 for r in s)
    assert all(r["thickness"] == r["size"] // 2 for r in s)
    # Poisson arrivals: mean gap 1/rate, coefficient of variation about 1
    gaps = np.diff([r["arrival"] for r in s])
    assert abs(gaps.mean() - 1e-3) < 1e-4
    assert 0.9 < gaps.std() / gaps.mean() < 1.1
