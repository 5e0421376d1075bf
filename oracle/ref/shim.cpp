// extern "C" entry points over the reference's own CPU sources, compiled
// unmodified into oracle/_ref (test infrastructure).  They let tests and the
// fixture generator call guanaco::Reconstructor (e_host),
// guanaco::correct<float> (e_host), guanaco::Filter<e_host> and the CTF grid
// functions of include/guanaco/ctf.h directly from Python (ctypes).
#include <cstring>
#include <guanaco/guanaco.h>

extern "C" {

int gnr_recon(const float *sino, float *rec, size_t num_pixels, size_t num_angles,
              size_t num_defocus, size_t grid_height, size_t grid_width, float pixel_size,
              float centre, float min_defocus, float max_defocus, const float *angles) {
  try {
    guanaco::Config c;
    c.device = guanaco::e_host;
    c.gpu_index = -1;
    c.num_pixels = num_pixels;
    c.num_angles = num_angles;
    c.num_defocus = num_defocus;
    c.grid_height = grid_height;
    c.grid_width = grid_width;
    c.pixel_size = pixel_size;
    c.centre = centre;
    c.min_defocus = min_defocus;
    c.max_defocus = max_defocus;
    c.angles.assign(angles, angles + num_angles);
    guanaco::make_reconstructor(c)(sino, rec);
    return 0;
  } catch (...) {
    return 1;
  }
}

int gnr_correct(const float *image, const float *ctf, float *rec, size_t xsize, size_t ysize,
                size_t num_ctf) {
  try {
    guanaco::correct<float>(image, reinterpret_cast<const std::complex<float> *>(ctf), rec,
                            xsize, ysize, num_ctf, guanaco::e_host);
    return 0;
  } catch (...) {
    return 1;
  }
}

int gnr_filter(float *data, size_t num_pixels, size_t num_angles, size_t num_defocus) {
  try {
    guanaco::Filter<guanaco::e_host> f(num_pixels, num_angles, num_defocus);
    f(data);
    return 0;
  } catch (...) {
    return 1;
  }
}

int gnr_ctf_simple(double l, double df, double Cs, double Ca, double Pa, double phi, size_t w,
                   size_t h, double ps, double *out) {
  guanaco::CTF c;
  c.l = l;
  c.df = df;
  c.Cs = Cs;
  c.Ca = Ca;
  c.Pa = Pa;
  c.phi = phi;
  guanaco::get_ctf_n_simple(c, reinterpret_cast<std::complex<double> *>(out), w, h, ps);
  return 0;
}

}
