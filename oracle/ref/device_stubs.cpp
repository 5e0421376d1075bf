// The reference's device (CUDA) path is not part of the CPU oracle build in
// oracle/_ref.  These definitions satisfy the linker for the symbols that the
// CPU sources reference (Reconstructor dispatch, explicit instantiations) and
// fail loudly if reached.
#include <guanaco/guanaco.h>

namespace guanaco {

[[noreturn]] static void no_device() { throw Error("oracle/_ref is a CPU-only build of the reference"); }

template <>
struct FFT<e_device>::Impl {};

template <> FFT<e_device>::FFT() { no_device(); }
template <> FFT<e_device>::FFT(const FFT &) { no_device(); }
template <> FFT<e_device>::FFT(FFT &&) { no_device(); }
template <> FFT<e_device> &FFT<e_device>::operator=(const FFT &) { no_device(); return *this; }
template <> FFT<e_device> &FFT<e_device>::operator=(FFT &&) { no_device(); return *this; }
template <> FFT<e_device>::~FFT() {}
template <> FFT<e_device> FFT<e_device>::make_1d(size_type, size_type, bool) { no_device(); }
template <> Filter<e_device>::Filter(size_type, size_type, size_type) : fft_(FFT<e_device>::make_1d(0, 0, false)) { no_device(); }
template <> void Filter<e_device>::operator()(float *) const { no_device(); }
template <> Reconstructor_t<e_device>::Reconstructor_t(const Config &c) : config_(c), filter_(0, 0, 0) { no_device(); }
template <> void Reconstructor_t<e_device>::operator()(const float *, float *) const { no_device(); }
template <> void Reconstructor_t<e_device>::project(const float *, float *) const { no_device(); }
namespace detail {
template <> void Corrector<e_device, float>::correct(const float *, const std::complex<float> *, float *,
                                                     std::size_t, std::size_t, std::size_t) { no_device(); }
}

}  // namespace guanaco
