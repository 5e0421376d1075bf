"""MRC2014 files (host only): the main-header and FEI1 record layout at their
byte offsets, data round trips in every supported mode (complex64 for CTF
images included), image stacks, volumes and the 4D corrected stack (stack of
volumes)."""
import numpy as np
import pytest

from guanaco_gb300 import mrc


def test_header_and_fei1_record_offsets(tmp_path):
    p = str(tmp_path / "stack.mrc")
    T, H, W = 5, 6, 8
    with mrc.new_mrc(p, (T, H, W), np.float32, voxel_size=1.35, fei1=True) as f:
        f.data[...] = np.arange(T * H * W, dtype=np.float32).reshape(T, H, W)
        f.extended_header["Alpha tilt"] = np.linspace(-60, 60, T)
        f.extended_header["Defocus"] = 20000.0
    raw = open(p, "rb").read()
    i4 = lambda o: int(np.frombuffer(raw[o:o + 4], "<i4")[0])  # noqa: E731
    f4 = lambda o: float(np.frombuffer(raw[o:o + 4], "<f4")[0])  # noqa: E731
    f8 = lambda o: float(np.frombuffer(raw[o:o + 8], "<f8")[0])  # noqa: E731
    assert (i4(0), i4(4), i4(8), i4(12)) == (W, H, T, 2)      # NX NY NZ MODE
    assert (i4(28), i4(32), i4(36)) == (W, H, 1)              # MX MY MZ (image stack)
    assert abs(f4(40) - 1.35 * W) < 1e-4                      # CELLA X
    assert (i4(64), i4(68), i4(72)) == (1, 2, 3)              # MAPC MAPR MAPS
    assert i4(88) == 0 and i4(92) == T * 768                  # ISPG NSYMBT
    assert raw[104:108] == b"FEI1" and raw[208:212] == b"MAP "
    assert raw[212:214] == b"\x44\x44"                        # little-endian stamp
    rec = 1024 + 2 * 768                                      # third FEI1 record
    assert i4(rec) == 768
    assert f8(rec + 100) == 0.0 and f8(rec + 220) == 20000.0  # Alpha tilt, Defocus
    assert f8(1024 + 100) == -60.0
    data0 = np.frombuffer(raw[1024 + T * 768:1024 + T * 768 + 16], "<f4")
    np.testing.assert_array_equal(data0, [0, 1, 2, 3])


@pytest.mark.parametrize("dtype", [np.float32, np.int16, np.uint16, np.int8, np.float16,
                                   np.complex64])
def test_round_trip_modes(tmp_path, dtype):
    p = str(tmp_path / "v.mrc")
    rng = np.random.default_rng(1)
    a = (rng.standard_normal((4, 5, 7)) * 50).astype(dtype)
    if np.dtype(dtype).kind == "c":
        a = a + 1j * (rng.standard_normal(a.shape) * 50).astype(np.float32)
    with mrc.new_mrc(p, a.shape, dtype, voxel_size=(1.0, 2.0, 3.0)) as f:
        f.data[...] = a
    g = mrc.open_mrc(p)
    assert g.data.dtype == np.dtype(dtype).newbyteorder("<")
    np.testing.assert_array_equal(np.asarray(g.data), a)
    assert g.voxel_size == {"x": 1.0, "y": 2.0, "z": 3.0}
    assert int(g.header["ispg"]) == 1 and g.extended_header is None
    assert int(g.header["mode"]) == {np.float32: 2, np.int16: 1, np.uint16: 6, np.int8: 0,
                                     np.float16: 12, np.complex64: 4}[dtype]


def test_corrected_stack_of_volumes(tmp_path):
    p = str(tmp_path / "corr.mrc")
    T, D, H, W = 3, 4, 5, 6
    a = np.random.default_rng(2).standard_normal((T, D, H, W)).astype(np.float32)
    with mrc.new_mrc(p, a.shape, np.float32, voxel_size=0.8, fei1=True) as f:
        f.data[...] = a
        for t in range(T):
            for d in range(D):
                f.extended_header[t, d]["Alpha tilt"] = 10.0 * t
                f.extended_header[t, d]["Defocus"] = -300.0 + 200.0 * d
    g = mrc.open_mrc(p)
    assert int(g.header["ispg"]) == 401 and int(g.header["nz"]) == T * D
    assert int(g.header["mz"]) == D
    np.testing.assert_array_equal(np.asarray(g.data), a)
    np.testing.assert_array_equal(mrc.fei1_angles_deg(g), [0.0, 10.0, 20.0])
    np.testing.assert_array_equal(mrc.fei1_defocus(g), [-300.0, -100.0, 100.0, 300.0])


def test_rejects_non_mrc(tmp_path):
    p = tmp_path / "x.mrc"
    p.write_bytes(b"\0" * 2048)
    with pytest.raises(ValueError):
        mrc.open_mrc(str(p))


def test_fixture_written_from_the_specification(tmp_path):
    """A file written byte by byte from the MRC2014 specification and the FEI1
    record layout (tests/golden/make_mrc_fixture.py, independent of this
    module): read back field by field, and the same stack written by this
    module gives the same bytes wherever the format fixes them."""
    import os
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_mrc_fixture as fx

    path = os.path.join(os.path.dirname(__file__), "golden", "mrc2014_fei1_stack.mrc")
    with mrc.open_mrc(path) as f:
        np.testing.assert_array_equal(f.data, fx.data())
        assert f.data.shape == (fx.T, fx.NY, fx.NX)
        assert f.voxel_size["x"] == pytest.approx(fx.PIXEL, rel=1e-6)
        assert f.voxel_size["y"] == pytest.approx(fx.PIXEL, rel=1e-6)
        np.testing.assert_array_equal(mrc.fei1_angles_deg(f), fx.TILTS)
        assert np.all(f.extended_header["Defocus"] == fx.DEFOCUS)
        assert int(f.header["nversion"]) == 20140 and int(f.header["ispg"]) == 0
    want = open(path, "rb").read()
    out = str(tmp_path / "written.mrc")
    with mrc.new_mrc(out, (fx.T, fx.NY, fx.NX), np.float32, voxel_size=fx.PIXEL,
                     fei1=True) as f:
        f.data[...] = fx.data()
        f.extended_header["Alpha tilt"] = fx.TILTS
        f.extended_header["Defocus"] = fx.DEFOCUS
        f.extended_header["Metadata version"] = 2
    got = open(out, "rb").read()
    assert len(got) == len(want)
    # every header word the format fixes (all but the labels; statistics equal
    # to float32 rounding), then the extended header and the data, exactly
    fixed = [(0, 76), (88, 96), (104, 112), (196, 220)]
    for a, b in fixed:
        assert got[a:b] == want[a:b], (a, b)
    np.testing.assert_allclose(np.frombuffer(got[76:88], "<f4"), np.frombuffer(want[76:88], "<f4"),
                               rtol=1e-6)
    assert got[1024:] == want[1024:]
