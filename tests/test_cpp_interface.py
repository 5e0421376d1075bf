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
