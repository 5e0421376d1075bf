// FFT<e_host> for the reference build in oracle/_ref (test infrastructure).
//
// The reference CPU path calls FFTW3 single precision through the pimpl class
// guanaco::FFT<e_host> (include/guanaco/fft.h:30-62, src/libguanaco/fft.cpp).
// FFTW is not installed, so this file implements that declared interface over
// the oracle's own Stockham FFT (oracle/gno_fft.c): unnormalised, forward
// exp(-i...), inverse exp(+i...), row-major (ysize, xsize) for 2D -- the
// conventions of fftwf_plan_dft_1d / fftwf_plan_dft_2d(ysize, xsize, ...).
#include <cstring>
#include <guanaco/fft.h>
#include "../gno_fft.h"

namespace guanaco {

template <>
struct FFT<e_host>::Impl {
  size_type nx = 0, ny = 0;
  int dims = 0;
  void run(void *in, void *out, int inverse) const {
    size_type n = nx * (dims == 2 ? ny : 1);
    if (in != out) std::memcpy(out, in, n * 2 * sizeof(float));
    float *d = reinterpret_cast<float *>(out);
    if (dims == 1) gno_fft_c2c_f(d, nx, inverse);
    else if (dims == 2) gno_fft2_c2c_f(d, nx, ny, inverse);
  }
};

template <> FFT<e_host>::FFT() : pimpl(std::make_unique<Impl>()) {}
template <> FFT<e_host>::FFT(const FFT &o) : pimpl(std::make_unique<Impl>(*o.pimpl)) {}
template <> FFT<e_host>::FFT(FFT &&) = default;
template <> FFT<e_host> &FFT<e_host>::operator=(const FFT &o) { *pimpl = *o.pimpl; return *this; }
template <> FFT<e_host> &FFT<e_host>::operator=(FFT &&) = default;
template <> FFT<e_host>::~FFT() = default;

template <> FFT<e_host>::FFT(size_type size) : pimpl(std::make_unique<Impl>()) {
  pimpl->nx = size;
  pimpl->dims = 1;
}

template <> FFT<e_host>::FFT(size_type xsize, size_type ysize) : pimpl(std::make_unique<Impl>()) {
  pimpl->nx = xsize;
  pimpl->ny = ysize;
  pimpl->dims = 2;
}

template <> void FFT<e_host>::forward(void *in, void *out) const { pimpl->run(in, out, 0); }
template <> void FFT<e_host>::inverse(void *in, void *out) const { pimpl->run(in, out, 1); }
template <> void FFT<e_host>::forward(void *data) const { pimpl->run(data, data, 0); }
template <> void FFT<e_host>::inverse(void *data) const { pimpl->run(data, data, 1); }

template <>
FFT<e_host> FFT<e_host>::make_1d(size_type size, size_type nbatch, bool real) {
  GUANACO_ASSERT(nbatch == 1);
  GUANACO_ASSERT(real == false);
  return FFT<e_host>(size);
}

template <>
FFT<e_host> FFT<e_host>::make_2d(size_type xsize, size_type ysize, size_type nbatch, bool real) {
  GUANACO_ASSERT(nbatch == 1);
  GUANACO_ASSERT(real == false);
  return FFT<e_host>(xsize, ysize);
}

}  // namespace guanaco
