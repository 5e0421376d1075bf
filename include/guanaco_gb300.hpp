/*
 * guanaco_gb300.hpp -- libguanaco's C++ interface for the device path, header
 * only, on top of the C ABI in guanaco_gb300.h.
 *
 * A C++ caller of libguanaco keeps its code: the names, constructors, call
 * signatures, defaults and exception type below are those of
 *   guanaco::eDevice          include/guanaco/constants.h:41-44
 *   guanaco::Error            include/guanaco/error.h:31-44
 *   guanaco::Config           include/guanaco/config.h:29-76
 *   guanaco::Reconstructor(_t) include/guanaco/reconstructor.h:26-59
 *   guanaco::Filter           include/guanaco/filter.h:32-54
 *   guanaco::correct          include/guanaco/correct.h:77-95
 *   guanaco::CTF              include/guanaco/ctf.h:167-178, with get_chi,
 *                             get_ctf(_simple(_real|_imag)), get_Es_n,
 *                             get_Et_n, the get_ctf_n* grids and the unit
 *                             conversions of include/guanaco/ctf.h.
 * Only e_device runs:
 * an e_host object or call throws guanaco::Error, as there is no CPU path
 * behind this library (the reference's own host code remains the CPU path).
 * A failed call throws guanaco::Error with gnc_last_error(); argument checks
 * that are GUANACO_ASSERTs in the reference carry the same
 * "ASSERT (condition) failed" text.
 *
 * Link with -lguanaco_gb300.  Requires C++11.
 */
#ifndef GUANACO_GB300_HPP
#define GUANACO_GB300_HPP

#include <complex>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "guanaco_gb300.h"

namespace guanaco {

enum eDevice {
  e_host = 0,   // the CPU: not provided by this library
  e_device = 1  // the GPU
};

class Error : public std::runtime_error {
 public:
  Error(const std::string &what_arg) : std::runtime_error(what_arg) {}
  Error(const char *what_arg) : std::runtime_error(what_arg) {}
  Error(const std::string &file, std::size_t line, const std::string &message)
      : std::runtime_error(file + ":" + std::to_string(line) + " " + message) {}
};

namespace gb300_detail {

// A non-zero status of the C ABI as guanaco::Error.
inline void check(int status) {
  if (status != GNC_OK) throw Error(std::string(gnc_last_error()));
}

inline void require_device(int device, const char *what) {
  if (device != e_device)
    throw Error(std::string(what) +
                ": guanaco_gb300 implements the device path only (eDevice e_device)");
}

}  // namespace gb300_detail

struct Config {
  using size_type = std::size_t;

  eDevice device;             // e_device (e_host is the reference's CPU path)
  int gpu_index;              // GPU to use (negative: the current one)
  size_type num_pixels;       // detector pixels N
  size_type num_angles;       // tilts T
  size_type num_defocus;      // defocus slabs D
  size_type grid_height;      // reconstruction rows Z
  size_type grid_width;       // reconstruction columns X
  float pixel_size;           // A
  float centre;               // rotation centre (px)
  std::vector<float> angles;  // rad
  float min_defocus;          // A
  float max_defocus;          // A

  Config()
      : device(e_host),
        gpu_index(0),
        num_pixels(0),
        num_angles(0),
        num_defocus(0),
        grid_height(0),
        grid_width(0),
        pixel_size(1),
        centre(0),
        min_defocus(0),
        max_defocus(0) {}

  size_type sino_size() const { return num_pixels * num_angles * num_defocus; }
  size_type grid_size() const { return grid_height * grid_width; }

  bool is_valid() const {
    return (device == e_host || device == e_device) && num_pixels > 0 && num_angles > 0 &&
           num_defocus > 0 && grid_height > 0 && grid_width > 0 && pixel_size > 0 &&
           min_defocus <= max_defocus && angles.size() == num_angles;
  }
};

namespace gb300_detail {

inline gnc_config to_c(const Config &c) {
  gnc_config g;
  g.device = (int)c.device;
  g.gpu_index = c.gpu_index;
  g.num_pixels = c.num_pixels;
  g.num_angles = c.num_angles;
  g.num_defocus = c.num_defocus;
  g.grid_height = c.grid_height;
  g.grid_width = c.grid_width;
  g.pixel_size = c.pixel_size;
  g.centre = c.centre;
  g.min_defocus = c.min_defocus;
  g.max_defocus = c.max_defocus;
  g.angles = c.angles.empty() ? nullptr : c.angles.data();
  return g;
}

}  // namespace gb300_detail

// Filtered backprojection of one Y slice: sinogram (D, T, N) and
// reconstruction (Z, X) are host float arrays; the reconstruction is
// overwritten.  Synchronous, like the reference.
template <eDevice device>
class Reconstructor_t {
 public:
  using size_type = std::size_t;

  // src/libguanaco/reconstructor.cu:281-286
  explicit Reconstructor_t(const Config &config) : config_(config) {
    gb300_detail::require_device(device, "Reconstructor_t");
    if (!(config_.device == e_device)) throw Error("ASSERT (config_.device == e_device) failed");
    if (!config_.is_valid()) throw Error("ASSERT (config_.is_valid()) failed");
  }

  void operator()(const float *sinogram, float *reconstruction) const {
    const gnc_config g = gb300_detail::to_c(config_);
    gb300_detail::check(gnc_reconstruct(&g, sinogram, reconstruction));
  }

 protected:
  Config config_;
};

class Reconstructor {
 public:
  using size_type = std::size_t;

  // src/libguanaco/reconstructor.cpp:117-131: the device is chosen per call
  explicit Reconstructor(const Config &config) : config_(config) {}

  void operator()(const float *sinogram, float *reconstruction) const {
    gb300_detail::require_device(config_.device, "Reconstructor");
    const Reconstructor_t<e_device> alg(config_);
    alg(sinogram, reconstruction);
  }

 protected:
  Config config_;
};

inline Reconstructor make_reconstructor(const Config &config) { return Reconstructor(config); }

// Ramp filter of num_defocus * num_angles rows of num_pixels (zero padded to
// 2 num_pixels) in place.  Filter<e_device> takes a device pointer and runs on
// the legacy default stream, so later default-stream work sees the result.
template <eDevice device>
class Filter {
 public:
  using size_type = std::size_t;
  using vector_type = std::vector<float>;

  Filter(size_type num_pixels, size_type num_angles, size_type num_defocus)
      : num_pixels_(num_pixels), num_angles_(num_angles), num_defocus_(num_defocus) {
    gb300_detail::require_device(device, "Filter");
    if (!(num_pixels_ > 0)) throw Error("ASSERT (num_pixels_ > 0) failed");
    if (!(num_angles_ > 0)) throw Error("ASSERT (num_angles_ > 0) failed");
    if (!(num_defocus_ > 0)) throw Error("ASSERT (num_defocus_ > 0) failed");
    // the ramp weights the transform's bins 0..N are multiplied by: w_i = i / N
    // (src/libguanaco/filter.cpp:30-45)
    filter_.resize(num_pixels_ + 1);
    for (size_type i = 0; i <= num_pixels_; ++i)
      filter_[i] = float(i) / float(num_pixels_);
  }

  void operator()(float *data) const {
    gb300_detail::check(gnc_filter_device(num_pixels_, num_angles_, num_defocus_, data, nullptr));
  }

  const vector_type &filter() const { return filter_; }

 protected:
  size_type num_pixels_;
  size_type num_angles_;
  size_type num_defocus_;
  vector_type filter_;
};

// CTF phase flip of one image against num_ctf CTFs: image (ysize, xsize), ctf
// (num_ctf, ysize, xsize), rec (num_ctf, ysize, xsize), host arrays, output
// unnormalised as in the reference.  float only (the device path's type).
template <typename T>
void correct(const T *image, const std::complex<T> *ctf, T *rec, std::size_t xsize,
             std::size_t ysize, std::size_t num_ctf = 1, eDevice device = e_host) {
  static_assert(std::is_same<T, float>::value, "guanaco_gb300 corrects float images");
  gb300_detail::require_device(device, "correct");
  gb300_detail::check(gnc_correct(image, reinterpret_cast<const float *>(ctf), rec, xsize, ysize,
                                  num_ctf));
}

// CTF parameters (include/guanaco/ctf.h:167-178) and their evaluation through
// the library's CTF physics (double precision, as the reference evaluates
// them): chi, the full CTF with envelopes, the simple CTF and its parts, the
// envelopes element-wise, and FFT-ordered grids at pixel size ps.
struct CTF {
  double l;        // wavelength (A)
  double df;       // defocus (A)
  double Cs;       // spherical aberration (A)
  double Ca;       // 2-fold astigmatism (A)
  double Pa;       // angle of 2-fold astigmatism (rad)
  double dd;       // defocus spread (A)
  double theta_c;  // source spread (rad)
  double phi;      // phase shift (rad)

  CTF() : l(0), df(0), Cs(0), Ca(0), Pa(0), dd(0), theta_c(0), phi(0) {}
};

namespace gb300_detail {

inline gnc_ctf to_c(const CTF &c) {
  gnc_ctf g;
  g.l = c.l;
  g.df = c.df;
  g.Cs = c.Cs;
  g.Ca = c.Ca;
  g.Pa = c.Pa;
  g.dd = c.dd;
  g.theta_c = c.theta_c;
  g.phi = c.phi;
  return g;
}

// one (q, theta) of a kind: out[0] (real kinds) or out[0] + i out[1]
inline void eval1(const CTF &c, int kind, double q, double theta, double *out) {
  const gnc_ctf g = to_c(c);
  check(gnc_ctf_eval(&g, kind, &q, &theta, 1, out));
}

// an (h, w) grid of a complex or a real kind, converted to the caller's
// element type
template <typename U>
void grid_complex(const CTF &c, int kind, U *out, std::size_t w, std::size_t h, double ps) {
  std::vector<double> tmp(2 * w * h);
  const gnc_ctf g = to_c(c);
  check(gnc_ctf_grid(&g, kind, w, h, ps, tmp.data()));
  for (std::size_t i = 0; i < w * h; ++i) out[i] = U(tmp[2 * i], tmp[2 * i + 1]);
}

template <typename U>
void grid_real(const CTF &c, int kind, U *out, std::size_t w, std::size_t h, double ps) {
  std::vector<double> tmp(w * h);
  const gnc_ctf g = to_c(c);
  check(gnc_ctf_grid(&g, kind, w, h, ps, tmp.data()));
  for (std::size_t i = 0; i < w * h; ++i) out[i] = U(tmp[i]);
}

}  // namespace gb300_detail

inline double get_chi(const CTF &c, double q, double theta) {
  const gnc_ctf g = gb300_detail::to_c(c);
  return gnc_ctf_chi(&g, q, theta);
}

inline std::complex<double> get_ctf(const CTF &c, double q, double theta) {
  double v[2];
  gb300_detail::eval1(c, GNC_CTF_FULL, q, theta, v);
  return std::complex<double>(v[0], v[1]);
}

inline std::complex<double> get_ctf_simple(const CTF &c, double q, double theta) {
  double v[2];
  gb300_detail::eval1(c, GNC_CTF_SIMPLE, q, theta, v);
  return std::complex<double>(v[0], v[1]);
}

inline double get_ctf_simple_real(const CTF &c, double q, double theta) {
  double v;
  gb300_detail::eval1(c, GNC_CTF_SIMPLE_REAL, q, theta, &v);
  return v;
}

inline double get_ctf_simple_imag(const CTF &c, double q, double theta) {
  double v;
  gb300_detail::eval1(c, GNC_CTF_SIMPLE_IMAG, q, theta, &v);
  return v;
}

// spatial and temporal coherence envelopes of n frequencies
inline void get_Es_n(const CTF &c, const double *q, const double *theta, double *Es,
                     std::size_t n) {
  const gnc_ctf g = gb300_detail::to_c(c);
  gb300_detail::check(gnc_ctf_eval(&g, GNC_CTF_ES, q, theta, n, Es));
}

inline void get_Et_n(const CTF &c, const double *q, double *Et, std::size_t n) {
  const gnc_ctf g = gb300_detail::to_c(c);
  gb300_detail::check(gnc_ctf_eval(&g, GNC_CTF_ET, q, nullptr, n, Et));
}

// FFT-ordered (h, w) grids at pixel size ps (include/guanaco/ctf.h:466-557)
template <typename T, typename U = std::complex<T>>
void get_ctf_n(const CTF &c, U *ctf, std::size_t w, std::size_t h, T ps) {
  gb300_detail::grid_complex(c, GNC_CTF_FULL, ctf, w, h, (double)ps);
}

template <typename T, typename U = std::complex<T>>
void get_ctf_n_simple(const CTF &c, U *ctf, std::size_t w, std::size_t h, T ps) {
  gb300_detail::grid_complex(c, GNC_CTF_SIMPLE, ctf, w, h, (double)ps);
}

template <typename T>
void get_ctf_n_simple_real(const CTF &c, T *ctf, std::size_t w, std::size_t h, T ps) {
  gb300_detail::grid_real(c, GNC_CTF_SIMPLE_REAL, ctf, w, h, (double)ps);
}

template <typename T>
void get_ctf_n_simple_imag(const CTF &c, T *ctf, std::size_t w, std::size_t h, T ps) {
  gb300_detail::grid_real(c, GNC_CTF_SIMPLE_IMAG, ctf, w, h, (double)ps);
}

// CTF unit conversions (include/guanaco/ctf.h), double precision.
inline double get_electron_wavelength(double V) { return gnc_get_electron_wavelength(V); }
inline double get_defocus_spread(double Cc, double dEE, double dII, double dVV) {
  return gnc_get_defocus_spread(Cc, dEE, dII, dVV);
}
inline double q_to_Q(double q, double l, double Cs) { return gnc_q_to_Q(q, l, Cs); }
inline double Q_to_q(double Q, double l, double Cs) { return gnc_Q_to_q(Q, l, Cs); }
inline double df_to_D(double df, double l, double Cs) { return gnc_df_to_D(df, l, Cs); }
inline double D_to_df(double D, double l, double Cs) { return gnc_D_to_df(D, l, Cs); }

}  // namespace guanaco

#endif /* GUANACO_GB300_HPP */
