"""The C++ interface (include/guanaco_gb300.hpp) compiles with g++ against the
C ABI header, links against the library and behaves like libguanaco's classes
where no GPU is needed: Config validity, the e_host refusal, the reference's
ASSERT texts, the ramp table of Filter and the CTF unit conversions."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <cmath>
#include <cstdio>
#include <string>
#include "guanaco_gb300.hpp"

static int failures = 0;
#define EXPECT(c) do { if (!(c)) { std::printf("FAILED: %s\n", #c); ++failures; } } while (0)

template <typename F>
static std::string thrown(F f) {
  try { f(); } catch (const guanaco::Error &e) { return e.what(); }
  return "";
}

int main() {
  guanaco::Config c;
  EXPECT(c.device == guanaco::e_host && c.pixel_size == 1.f && !c.is_valid());
  c.device = guanaco::e_device;
  c.num_pixels = 8; c.num_angles = 3; c.num_defocus = 2; c.grid_height = 8; c.grid_width = 8;
  c.angles = {0.f, 0.5f, 1.f};
  EXPECT(c.is_valid() && c.sino_size() == 48 && c.grid_size() == 64);

  // the host path is refused when the reconstructor runs, not when it is made
  guanaco::Config h = c;
  h.device = guanaco::e_host;
  guanaco::Reconstructor rh(h);
  float sino[48] = {0}, rec[64] = {0};
  EXPECT(thrown([&] { rh(sino, rec); }).find("device path only") != std::string::npos);
  EXPECT(thrown([&] { guanaco::Filter<guanaco::e_host> f(8, 3, 2); }).find("device path only") !=
         std::string::npos);
  std::complex<float> ctf[32];
  EXPECT(thrown([&] { guanaco::correct(sino, ctf, rec, 8, 4, 1); }).find("device path only") !=
         std::string::npos);

  // the reference's ASSERT texts
  guanaco::Config bad = c;
  bad.angles.pop_back();
  EXPECT(thrown([&] { guanaco::Reconstructor_t<guanaco::e_device> r(bad); }) ==
         "ASSERT (config_.is_valid()) failed");
  EXPECT(thrown([&] { guanaco::Reconstructor_t<guanaco::e_device> r(h); }) ==
         "ASSERT (config_.device == e_device) failed");
  EXPECT(thrown([&] { guanaco::Filter<guanaco::e_device> f(0, 3, 2); }) ==
         "ASSERT (num_pixels_ > 0) failed");

  // null buffers reach the library's own check, which names the condition
  guanaco::Reconstructor_t<guanaco::e_device> rd(c);
  EXPECT(thrown([&] { rd(nullptr, rec); }).find("ASSERT") != std::string::npos);

  // Filter's ramp table: w_i = i / N for i = 0..N
  guanaco::Filter<guanaco::e_device> f(8, 3, 2);
  EXPECT(f.filter().size() == 9 && f.filter()[0] == 0.f && f.filter()[8] == 1.f &&
         f.filter()[2] == 0.25f);

  // CTF unit conversions go through the library's double-precision physics
  EXPECT(guanaco::get_electron_wavelength(300e3) == gnc_get_electron_wavelength(300e3));
  const double l = guanaco::get_electron_wavelength(300e3);
  EXPECT(std::fabs(l - 0.0196875) < 1e-6);
  const double Cs = 2.7e7, q = 0.2;
  EXPECT(std::fabs(guanaco::Q_to_q(guanaco::q_to_Q(q, l, Cs), l, Cs) - q) < 1e-12);
  EXPECT(std::fabs(guanaco::D_to_df(guanaco::df_to_D(20000.0, l, Cs), l, Cs) - 20000.0) < 1e-6);

  std::printf("%s\n", failures ? "FAIL" : "OK");
  return failures ? 1 : 0;
}
"""


def test_cpp_interface(tmp_path):
    from guanaco_gb300 import _lib

    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    lib = _lib.lib_path()
    if not os.path.exists(lib):
        _lib.load()
    src = tmp_path / "hpp.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "hpp"
    libdir = os.path.dirname(lib)
    subprocess.run([gxx, "-std=c++11", "-Wall", "-Werror", "-I", os.path.join(REPO, "include"),
                    str(src), "-o", str(exe), "-L", libdir, "-lguanaco_gb300",
                    "-Wl,-rpath," + libdir], check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("OK")


DEVICE_PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "guanaco_gb300.hpp"

// argv: sinogram file (9 x 32 floats), output reconstruction file (32 x 32),
// image file (16 x 24 floats), ctf file (2 x 16 x 24 complex), output corrected file
static std::vector<float> read(const char *path, size_t n) {
  std::vector<float> v(n);
  FILE *f = std::fopen(path, "rb");
  if (!f || std::fread(v.data(), sizeof(float), n, f) != n) throw guanaco::Error("read");
  std::fclose(f);
  return v;
}
static void write(const char *path, const std::vector<float> &v) {
  FILE *f = std::fopen(path, "wb");
  std::fwrite(v.data(), sizeof(float), v.size(), f);
  std::fclose(f);
}

int main(int argc, char **argv) {
  if (argc != 6) return 2;
  try {
    guanaco::Config c;
    c.device = guanaco::e_device;
    c.gpu_index = -1;
    c.num_pixels = 32; c.num_angles = 9; c.num_defocus = 1;
    c.grid_height = 32; c.grid_width = 32;
    c.centre = 16.f;
    for (int t = 0; t < 9; ++t) c.angles.push_back(-1.f + 0.25f * t);
    std::vector<float> sino = read(argv[1], 9 * 32), rec(32 * 32, -1.f);
    guanaco::make_reconstructor(c)(sino.data(), rec.data());
    write(argv[2], rec);
    std::vector<float> image = read(argv[3], 16 * 24), ctf = read(argv[4], 2 * 16 * 24 * 2);
    std::vector<float> out(2 * 16 * 24);
    guanaco::correct<float>(image.data(), reinterpret_cast<const std::complex<float> *>(ctf.data()),
                            out.data(), 24, 16, 2, guanaco::e_device);
    write(argv[5], out);
  } catch (const guanaco::Error &e) {
    std::printf("Error: %s\n", e.what());
    return 1;
  }
  return 0;
}
"""


@pytest.mark.gpu
def test_cpp_device_calls_match_python(tmp_path):
    """Reconstructor and correct<float> of the C++ interface give exactly the
    volumes of guanaco_gb300.detail.recon and corr (the same C ABI calls)."""
    import numpy as np
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from guanaco_gb300 import _lib, detail

    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    lib = _lib.lib_path()
    _lib.load()
    src = tmp_path / "dev.cpp"
    src.write_text(DEVICE_PROGRAM)
    exe = tmp_path / "dev"
    libdir = os.path.dirname(lib)
    subprocess.run([gxx, "-std=c++11", "-Wall", "-I", os.path.join(REPO, "include"), str(src),
                    "-o", str(exe), "-L", libdir, "-lguanaco_gb300", "-Wl,-rpath," + libdir],
                   check=True, capture_output=True, text=True)
    rng = np.random.default_rng(3)
    sino = rng.standard_normal((9, 32)).astype(np.float32)
    image = rng.standard_normal((16, 24)).astype(np.float32)
    ctf = (rng.standard_normal((2, 16, 24)) + 1j * rng.standard_normal((2, 16, 24))).astype(
        np.complex64)
    paths = [tmp_path / n for n in ("sino", "rec", "image", "ctf", "corr")]
    sino.tofile(paths[0])
    image.tofile(paths[2])
    ctf.tofile(paths[3])
    r = subprocess.run([str(exe)] + [str(p) for p in paths], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    got_rec = np.fromfile(paths[1], np.float32).reshape(32, 32)
    got_corr = np.fromfile(paths[4], np.float32).reshape(2, 16, 24)
    ang = (-1.0 + 0.25 * np.arange(9)).astype(np.float32)
    want_rec = np.empty((32, 32), np.float32)
    detail.recon(sino, want_rec, ang, 16.0, device="gpu")
    want_corr = np.empty((2, 16, 24), np.float32)
    detail.corr(image, ctf, want_corr, device="gpu")
    np.testing.assert_array_equal(got_rec, want_rec)
    np.testing.assert_array_equal(got_corr, want_corr)
    assert np.abs(want_rec).max() > 0 and np.abs(want_corr).max() > 0


CTF_PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "guanaco_gb300.hpp"

// writes the reference's CTF known answers, evaluated through the C++
// interface, to argv[1] as raw doubles in a fixed order
int main(int argc, char **argv) {
  if (argc != 2) return 2;
  std::vector<double> out;
  const double l = guanaco::get_electron_wavelength(300000);
  guanaco::CTF c;
  c.l = l; c.df = 20000; c.Cs = 2.7e7;
  out.push_back(guanaco::get_chi(c, 10, 0));
  guanaco::CTF env = c;
  env.dd = 1; env.theta_c = 1e-3;
  double q = 10, theta = 0, Es = 0, Et = 0;
  guanaco::get_Es_n(env, &q, &theta, &Es, 1);
  guanaco::get_Et_n(env, &q, &Et, 1);
  out.push_back(Es);
  out.push_back(Et);
  guanaco::CTF full = c;
  full.dd = 1; full.theta_c = 0.1 / 1e3; full.phi = 0.1;
  std::vector<std::complex<double>> g(100 * 100);
  guanaco::get_ctf_n(full, g.data(), 100, 100, 2.0);
  for (auto v : g) { out.push_back(v.real()); out.push_back(v.imag()); }
  guanaco::CTF simple = c;
  simple.phi = 0.1;
  guanaco::get_ctf_n_simple(simple, g.data(), 100, 100, 2.0);
  for (auto v : g) { out.push_back(v.real()); out.push_back(v.imag()); }
  std::vector<double> r(100 * 100);
  guanaco::get_ctf_n_simple_real(simple, r.data(), 100, 100, 2.0);
  out.insert(out.end(), r.begin(), r.end());
  guanaco::get_ctf_n_simple_imag(simple, r.data(), 100, 100, 2.0);
  out.insert(out.end(), r.begin(), r.end());
  guanaco::CTF astig = c;
  astig.df = 25000; astig.Ca = 800; astig.Pa = 0.3; astig.phi = 0.05;
  std::vector<std::complex<double>> a(90 * 64);
  guanaco::get_ctf_n_simple(astig, a.data(), 90, 64, 1.5);
  for (auto v : a) { out.push_back(v.real()); out.push_back(v.imag()); }
  // the scalar forms agree with the grid forms
  const std::complex<double> s = guanaco::get_ctf_simple(simple, 0.05, 0.3);
  out.push_back(s.real() - guanaco::get_ctf_simple_real(simple, 0.05, 0.3));
  out.push_back(s.imag() - guanaco::get_ctf_simple_imag(simple, 0.05, 0.3));
  FILE *f = std::fopen(argv[1], "wb");
  std::fwrite(out.data(), sizeof(double), out.size(), f);
  std::fclose(f);
  return 0;
}
"""


def test_cpp_ctf_known_answers(tmp_path):
    """guanaco::CTF and its evaluation functions reproduce the reference's CTF
    known answers (tests/golden/ctf_kat.npz, recorded from the reference)."""
    import numpy as np

    from conftest import golden
    from guanaco_gb300 import _lib

    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    lib = _lib.lib_path()
    _lib.load()
    src = tmp_path / "ctf.cpp"
    src.write_text(CTF_PROGRAM)
    exe = tmp_path / "ctf"
    libdir = os.path.dirname(lib)
    subprocess.run([gxx, "-std=c++11", "-Wall", "-Werror", "-I", os.path.join(REPO, "include"),
                    str(src), "-o", str(exe), "-L", libdir, "-lguanaco_gb300",
                    "-Wl,-rpath," + libdir], check=True, capture_output=True, text=True)
    out = tmp_path / "ctf.bin"
    r = subprocess.run([str(exe), str(out)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    v = np.fromfile(out, np.float64)
    g = golden("ctf_kat")
    n = 100 * 100
    chi, es, et = v[0], v[1], v[2]
    o = 3
    full = v[o:o + 2 * n].view(np.complex128).reshape(100, 100); o += 2 * n
    simple = v[o:o + 2 * n].view(np.complex128).reshape(100, 100); o += 2 * n
    real = v[o:o + n].reshape(100, 100); o += n
    imag = v[o:o + n].reshape(100, 100); o += n
    astig = v[o:o + 2 * 90 * 64].view(np.complex128).reshape(64, 90); o += 2 * 90 * 64
    assert chi == pytest.approx(float(g["chi_q10"]), rel=1e-15)
    np.testing.assert_allclose([es], g["Es_q10"], rtol=1e-14)
    np.testing.assert_allclose([et], g["Et_q10"], rtol=1e-14)
    np.testing.assert_allclose(full, g["ctf_full"], rtol=0, atol=1e-13)
    np.testing.assert_array_equal(simple, g["ctf_simple"])
    np.testing.assert_array_equal(real, g["ctf_simple_real"])
    np.testing.assert_array_equal(imag, g["ctf_simple_imag"])
    np.testing.assert_array_equal(astig, g["ctf_simple_astig_90x64"])
    assert v[o] == 0.0 and v[o + 1] == 0.0 and o + 2 == v.size
