/*
 * Oracle restatement of guanaco's CPU path -- TEST INFRASTRUCTURE ONLY.
 * See gno_oracle.h.  Build with -ffp-contract=off: the float functions must
 * evaluate every expression in the reference's order without fused
 * multiply-adds, on x86-64 and on aarch64 alike.
 */
#include "gno_oracle.h"
#include "gno_fft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Physical constants: include/guanaco/constants.h:28-37 */
static const double k_c = 2.99792458e8;
static const double k_e = 1.602176634e-19;
static const double k_m_e = 9.1093837015e-31;
static const double k_h = 6.62607004e-34;
static const double k_m_to_A = 1e10;

/* ctf.h:39-48 */
double gno_electron_wavelength(double V) {
  double eV = k_e * V;
  return (k_h * k_c / sqrt(eV * eV + 2 * k_m_e * eV * k_c * k_c)) * k_m_to_A;
}

/* ctf.h:61-64 */
double gno_defocus_spread(double Cc, double dEE, double dII, double dVV) {
  return Cc * sqrt((dEE) * (dEE) + (2 * dII) * (2 * dII) + (dVV) * (dVV));
}

/* ctf.h:88-101: FFT-ordered frequency of pixel (x, y) */
void gno_r_and_theta(size_t x, size_t y, size_t w, size_t h, double inv_ps, double *r,
                     double *theta) {
  size_t w2 = w / 2, h2 = h / 2;
  double dx = ((double)((x + w2) % w) - (double)w2) / (double)w;
  double dy = ((double)((y + h2) % h) - (double)h2) / (double)h;
  *r = sqrt((dx * dx + dy * dy) * inv_ps * inv_ps);
  *theta = atan2(dy, dx);
}

/* ctf.h:233-238 */
double gno_chi(const gno_ctf_params *c, double q, double theta) {
  double df = c->df + c->Ca * cos(2 * (theta - c->Pa));
  return M_PI * (c->Cs * c->l * c->l * c->l * q * q * q * q / 2 - c->l * df * q * q);
}

/* ctf.h:188-195 */
double gno_log_Es(const gno_ctf_params *c, double q, double theta) {
  double df = c->df + c->Ca * cos(2 * (theta - c->Pa));
  double u = 1 + 2 * M_PI * M_PI * c->theta_c * c->theta_c * c->dd * c->dd * q * q;
  double v = c->Cs * c->l * c->l * c->l * q * q * q - df * c->l * q;
  return -(M_PI * M_PI * c->theta_c * c->theta_c * v * v / (c->l * c->l * u));
}

/* ctf.h:204-209 */
double gno_log_Et(const gno_ctf_params *c, double q) {
  double u = 1 + 2 * M_PI * M_PI * c->theta_c * c->theta_c * c->dd * c->dd * q * q;
  return -(M_PI * M_PI * c->l * c->l * c->dd * c->dd * q * q * q * q / (2 * u));
}

/* ctf.h:218-223 */
double gno_A(const gno_ctf_params *c, double q) {
  double u = 1 + 2 * M_PI * M_PI * c->theta_c * c->theta_c * c->dd * c->dd * q * q;
  return 1 / sqrt(u);
}

/* ctf.h:466-503: simple = exp(-i(chi - phi)); full adds A*exp(logEs+logEt) */
void gno_ctf_grid(const gno_ctf_params *c, size_t w, size_t h, double ps, int simple,
                  double *out) {
  double inv_ps = 1.0 / ps;
  for (size_t j = 0; j < h; ++j) {
    for (size_t i = 0; i < w; ++i) {
      double q, theta;
      gno_r_and_theta(i, j, w, h, inv_ps, &q, &theta);
      double a = -(gno_chi(c, q, theta) - c->phi);
      double mag = 1.0;
      if (!simple) mag = gno_A(c, q) * exp(gno_log_Es(c, q, theta) + gno_log_Et(c, q));
      out[2 * (j * w + i)] = mag * cos(a);
      out[2 * (j * w + i) + 1] = mag * sin(a);
    }
  }
}

/* correct.h:30-39: phase_flip(x, h) = -x * sign(h.imag()), sign(0) = 0.
 * Returns the real factor that multiplies x. */
static inline float flip_factor(float h_imag) {
  int s = (0.0f < h_imag) - (h_imag < 0.0f);
  return (float)(-s);
}

/* correct.cpp:30-90 in float */
void gno_correct_f(const float *image, const float *ctf, float *rec, size_t xsize,
                   size_t ysize, size_t num_ctf) {
  size_t n = xsize * ysize;
  float *img = (float *)malloc(2 * n * sizeof(float));
  float *b = (float *)malloc(2 * n * sizeof(float));
  for (size_t k = 0; k < n; ++k) { img[2 * k] = image[k]; img[2 * k + 1] = 0.0f; }
  gno_fft2_c2c_f(img, xsize, ysize, 0);
  for (size_t j = 0; j < num_ctf; ++j) {
    const float *c = ctf + 2 * j * n;
    for (size_t k = 0; k < n; ++k) {
      float s = flip_factor(c[2 * k + 1]);
      b[2 * k] = img[2 * k] * s;
      b[2 * k + 1] = img[2 * k + 1] * s;
    }
    gno_fft2_c2c_f(b, xsize, ysize, 1);
    float *r = rec + j * n;
    for (size_t k = 0; k < n; ++k) r[k] = b[2 * k];
  }
  free(img);
  free(b);
}

/* correct.cpp:30-90 in double; the flip sign uses the complex64 CTF */
void gno_correct_d(const double *image, const float *ctf, double *rec, size_t xsize,
                   size_t ysize, size_t num_ctf) {
  size_t n = xsize * ysize;
  double *img = (double *)malloc(2 * n * sizeof(double));
  double *b = (double *)malloc(2 * n * sizeof(double));
  for (size_t k = 0; k < n; ++k) { img[2 * k] = image[k]; img[2 * k + 1] = 0.0; }
  gno_fft2_c2c_d(img, xsize, ysize, 0);
  for (size_t j = 0; j < num_ctf; ++j) {
    const float *c = ctf + 2 * j * n;
    for (size_t k = 0; k < n; ++k) {
      double s = (double)flip_factor(c[2 * k + 1]);
      b[2 * k] = img[2 * k] * s;
      b[2 * k + 1] = img[2 * k + 1] * s;
    }
    gno_fft2_c2c_d(b, xsize, ysize, 1);
    double *r = rec + j * n;
    for (size_t k = 0; k < n; ++k) r[k] = b[2 * k];
  }
  free(img);
  free(b);
}

/* filter.cpp:30-45: w_i = i / N for i in [0, N] */
static float ramp_weight_f(size_t i, size_t num_pixels) {
  return (float)i / (float)(num_pixels);
}

/* filter.cpp:61-97 in float */
void gno_filter_f(float *data, size_t num_pixels, size_t num_rows) {
  size_t L = 2 * num_pixels;
  float *row = (float *)malloc(2 * L * sizeof(float));
  float *w = (float *)malloc((num_pixels + 1) * sizeof(float));
  for (size_t j = 0; j <= num_pixels; ++j) w[j] = ramp_weight_f(j, num_pixels);
  for (size_t i = 0; i < num_rows; ++i) {
    float *d = data + i * num_pixels;
    for (size_t j = 0; j < num_pixels; ++j) { row[2 * j] = d[j]; row[2 * j + 1] = 0.0f; }
    for (size_t j = num_pixels; j < L; ++j) { row[2 * j] = 0.0f; row[2 * j + 1] = 0.0f; }
    gno_fft_c2c_f(row, L, 0);
    for (size_t j = 0; j < L; ++j) {
      float f = j <= num_pixels ? w[j] : w[L - j];
      row[2 * j] *= f;
      row[2 * j + 1] *= f;
    }
    gno_fft_c2c_f(row, L, 1);
    for (size_t j = 0; j < num_pixels; ++j) d[j] = row[2 * j] / (float)L;
  }
  free(row);
  free(w);
}

/* filter.cpp:61-97 in double (ramp weights as the float table) */
void gno_filter_d(double *data, size_t num_pixels, size_t num_rows) {
  size_t L = 2 * num_pixels;
  double *row = (double *)malloc(2 * L * sizeof(double));
  double *w = (double *)malloc((num_pixels + 1) * sizeof(double));
  for (size_t j = 0; j <= num_pixels; ++j) w[j] = (double)j / (double)num_pixels;
  for (size_t i = 0; i < num_rows; ++i) {
    double *d = data + i * num_pixels;
    for (size_t j = 0; j < num_pixels; ++j) { row[2 * j] = d[j]; row[2 * j + 1] = 0.0; }
    for (size_t j = num_pixels; j < L; ++j) { row[2 * j] = 0.0; row[2 * j + 1] = 0.0; }
    gno_fft_c2c_d(row, L, 0);
    for (size_t j = 0; j < L; ++j) {
      double f = j <= num_pixels ? w[j] : w[L - j];
      row[2 * j] *= f;
      row[2 * j + 1] *= f;
    }
    gno_fft_c2c_d(row, L, 1);
    for (size_t j = 0; j < num_pixels; ++j) d[j] = row[2 * j] / (double)L;
  }
  free(row);
  free(w);
}

/* Per-tilt geometry exactly as reconstructor.cpp:35-47 (float) */
typedef struct {
  float cos_a, sin_a, offset, scale;
} geom_f;

static geom_f tilt_geometry_f(const gno_config *cfg, size_t angle) {
  double output_scale = M_PI / (double)(2 * cfg->num_angles);
  float theta = cfg->angles[angle];
  float cos_angle = cosf(theta);
  float sin_angle = sinf(theta);
  float det_x0 = -cfg->centre * cos_angle;
  float det_y0 = -cfg->centre * sin_angle;
  float ray_length = sqrtf(cos_angle * cos_angle + sin_angle * sin_angle);
  float d = cos_angle * cos_angle + sin_angle * sin_angle;
  geom_f g;
  g.offset = (det_y0 * (-sin_angle) - det_x0 * cos_angle) / d;
  g.scale = (float)(output_scale * ray_length / fabsf(d));
  g.cos_a = cos_angle / d;
  g.sin_a = sin_angle / d;
  return g;
}

/* reconstructor.cpp:28-32 */
static void defocus_scale_f(const gno_config *cfg, float *dscale, float *doffset) {
  float ds = cfg->num_defocus > 1
               ? (float)cfg->num_defocus * cfg->pixel_size / (cfg->max_defocus - cfg->min_defocus)
               : 0.0f;
  *dscale = ds;
  *doffset = -ds * (cfg->min_defocus / cfg->pixel_size);
}

/* reconstructor.cpp:66-72: the slab index in float, floor in double */
static inline int slab_index_f(float x, float y, float sin_a, float cos_a, float dscale,
                               float doffset, size_t num_defocus) {
  float height = -x * sin_a - y * cos_a;
  float defocus = height * dscale + doffset;
  int k = (int)floor((double)defocus + 0.5);
  if (k < 0) k = 0;
  if (k > (int)num_defocus - 1) k = (int)num_defocus - 1;
  return k;
}

/* reconstructor.cpp:14-90 in float */
void gno_project_f(const gno_config *cfg, const float *sino, float *rec) {
  size_t gw = cfg->grid_width, gh = cfg->grid_height;
  size_t np = cfg->num_pixels, na = cfg->num_angles, nd = cfg->num_defocus;
  float dscale, doffset;
  defocus_scale_f(cfg, &dscale, &doffset);
  for (size_t angle = 0; angle < na; ++angle) {
    geom_f g = tilt_geometry_f(cfg, angle);
    const float *row_angle = sino + angle * np;
    for (size_t j = 0; j < gh; ++j) {
      for (size_t i = 0; i < gw; ++i) {
        const float *row = row_angle;
        float x = (float)((double)i - 0.5 * (double)gw + 0.5);
        float y = (float)((double)j - 0.5 * (double)gh + 0.5);
        size_t index = i + j * gw;
        float pixel = x * g.cos_a - y * g.sin_a + g.offset;
        if (nd > 1) {
          int k = slab_index_f(x, y, g.sin_a, g.cos_a, dscale, doffset, nd);
          row += (size_t)k * np * na;
        }
        pixel = (float)((double)pixel - 0.5);
        int ind = (int)floorf(pixel);
        float t = pixel - (float)ind;
        if (ind >= 0 && (size_t)ind < np - 1) {
          float v0 = row[ind];
          float v1 = row[ind + 1];
          float value = (1 - t) * v0 + t * v1;
          rec[index] += g.scale * value;
        }
      }
    }
  }
}

/* reconstructor.cpp:14-90 in double.  The discrete decisions -- slab index,
 * pixel floor and the edge skip -- follow the reference's float rule exactly;
 * the interpolation weight, the samples and the sum are double. */
void gno_project_d(const gno_config *cfg, const double *sino, double *rec) {
  size_t gw = cfg->grid_width, gh = cfg->grid_height;
  size_t np = cfg->num_pixels, na = cfg->num_angles, nd = cfg->num_defocus;
  float dscale, doffset;
  defocus_scale_f(cfg, &dscale, &doffset);
  double output_scale = M_PI / (double)(2 * na);
  for (size_t angle = 0; angle < na; ++angle) {
    geom_f gf = tilt_geometry_f(cfg, angle);
    double theta = (double)cfg->angles[angle];
    double c = cos(theta), s = sin(theta);
    double d = c * c + s * s;
    double centre = (double)cfg->centre;
    double offset = (centre * s * s + centre * c * c) / d;
    double scale = output_scale * sqrt(d) / fabs(d);
    double cos_a = c / d, sin_a = s / d;
    const double *row_angle = sino + angle * np;
    for (size_t j = 0; j < gh; ++j) {
      for (size_t i = 0; i < gw; ++i) {
        const double *row = row_angle;
        float xf = (float)((double)i - 0.5 * (double)gw + 0.5);
        float yf = (float)((double)j - 0.5 * (double)gh + 0.5);
        size_t index = i + j * gw;
        if (nd > 1) {
          int k = slab_index_f(xf, yf, gf.sin_a, gf.cos_a, dscale, doffset, nd);
          row += (size_t)k * np * na;
        }
        float pf = xf * gf.cos_a - yf * gf.sin_a + gf.offset;
        pf = (float)((double)pf - 0.5);
        int ind = (int)floorf(pf);
        if (ind >= 0 && (size_t)ind < np - 1) {
          double pixel = (double)xf * cos_a - (double)yf * sin_a + offset - 0.5;
          double t = pixel - (double)ind;
          double value = (1 - t) * row[ind] + t * row[ind + 1];
          rec[index] += scale * value;
        }
      }
    }
  }
}

void gno_slab_index_map(const gno_config *cfg, int32_t *out) {
  size_t gw = cfg->grid_width, gh = cfg->grid_height;
  float dscale, doffset;
  defocus_scale_f(cfg, &dscale, &doffset);
  for (size_t angle = 0; angle < cfg->num_angles; ++angle) {
    geom_f g = tilt_geometry_f(cfg, angle);
    for (size_t j = 0; j < gh; ++j) {
      for (size_t i = 0; i < gw; ++i) {
        float x = (float)((double)i - 0.5 * (double)gw + 0.5);
        float y = (float)((double)j - 0.5 * (double)gh + 0.5);
        int k = 0;
        if (cfg->num_defocus > 1)
          k = slab_index_f(x, y, g.sin_a, g.cos_a, dscale, doffset, cfg->num_defocus);
        out[(angle * gh + j) * gw + i] = k;
      }
    }
  }
}

/* reconstructor.cpp:92-115 */
void gno_recon_f(const gno_config *cfg, const float *sino, float *rec) {
  size_t n = cfg->num_pixels * cfg->num_angles * cfg->num_defocus;
  float *filtered = (float *)malloc(n * sizeof(float));
  memcpy(filtered, sino, n * sizeof(float));
  gno_filter_f(filtered, cfg->num_pixels, cfg->num_angles * cfg->num_defocus);
  memset(rec, 0, cfg->grid_width * cfg->grid_height * sizeof(float));
  gno_project_f(cfg, filtered, rec);
  free(filtered);
}

void gno_recon_d(const gno_config *cfg, const double *sino, double *rec) {
  size_t n = cfg->num_pixels * cfg->num_angles * cfg->num_defocus;
  double *filtered = (double *)malloc(n * sizeof(double));
  memcpy(filtered, sino, n * sizeof(double));
  gno_filter_d(filtered, cfg->num_pixels, cfg->num_angles * cfg->num_defocus);
  memset(rec, 0, cfg->grid_width * cfg->grid_height * sizeof(double));
  gno_project_d(cfg, filtered, rec);
  free(filtered);
}

static void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

/* correct.py:291-318 (tilt loop calling corr) then mp.py:124-153 per row */
void gno_fbp_ctf_rows_f(const float *proj, size_t T, size_t H, size_t W, const float *angles,
                        const float *centre, float pixel_size, const float *ctf, size_t D,
                        float min_defocus, float max_defocus, const double *weights, int minus,
                        size_t Z, const size_t *rows, size_t nrows, float *out, size_t t_begin,
                        size_t t_end, int nthreads) {
  set_threads(nthreads);
  size_t nd = D > 0 ? D : 1;
  size_t img = H * W;
  /* corrected stack (T, D, H, W); without CTF the projections themselves */
  float *corr = NULL;
  const float *stack = proj;
  if (D > 0) {
    corr = (float *)calloc(T * nd * img, sizeof(float));
#pragma omp parallel for schedule(dynamic, 1)
    for (long t = (long)t_begin; t < (long)t_end; ++t)
      gno_correct_f(proj + (size_t)t * img, ctf, corr + (size_t)t * nd * img, W, H, nd);
    stack = corr;
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (long i = 0; i < (long)nrows; ++i) {
    size_t y = rows[i];
    /* numpy.swapaxes + ascontiguousarray: sino (D, T, W) for row y */
    float *sino = (float *)malloc(nd * T * W * sizeof(float));
    for (size_t d = 0; d < nd; ++d)
      for (size_t t = 0; t < T; ++t) {
        const float *src = stack + ((t * nd + d) * H + y) * W;
        float *dst = sino + (d * T + t) * W;
        for (size_t x = 0; x < W; ++x) dst[x] = minus ? -src[x] : src[x];
      }
    /* mp.py:135-141: float32 data times a float64 weight, stored as float32 */
    for (size_t d = 0; d < nd; ++d)
      for (size_t t = 0; t < T; ++t) {
        double wt = weights ? (double)weights[t] : 1.0;
        float *r = sino + (d * T + t) * W;
        for (size_t x = 0; x < W; ++x) r[x] = (float)((double)r[x] * wt);
      }
    gno_config cfg;
    cfg.num_pixels = W;
    cfg.num_angles = T;
    cfg.num_defocus = nd;
    cfg.grid_height = Z;
    cfg.grid_width = W;
    cfg.pixel_size = pixel_size;
    cfg.centre = centre[y];
    cfg.min_defocus = D > 1 ? min_defocus : 0.0f;
    cfg.max_defocus = D > 1 ? max_defocus : 0.0f;
    cfg.angles = angles;
    gno_recon_f(&cfg, sino, out + (size_t)i * Z * W);
    free(sino);
  }
  free(corr);
}

static size_t *row_range(size_t y_begin, size_t y_end) {
  size_t n = y_end > y_begin ? y_end - y_begin : 0;
  size_t *rows = (size_t *)malloc((n ? n : 1) * sizeof(size_t));
  for (size_t i = 0; i < n; ++i) rows[i] = y_begin + i;
  return rows;
}

void gno_fbp_ctf_f(const float *proj, size_t T, size_t H, size_t W, const float *angles,
                   const float *centre, float pixel_size, const float *ctf, size_t D,
                   float min_defocus, float max_defocus, const double *weights, int minus,
                   size_t Z, float *vol, size_t y_begin, size_t y_end, size_t t_begin,
                   size_t t_end, int nthreads) {
  size_t *rows = row_range(y_begin, y_end);
  gno_fbp_ctf_rows_f(proj, T, H, W, angles, centre, pixel_size, ctf, D, min_defocus,
                     max_defocus, weights, minus, Z, rows, y_end > y_begin ? y_end - y_begin : 0,
                     vol + y_begin * Z * W, t_begin, t_end, nthreads);
  free(rows);
}

void gno_fbp_ctf_rows_d(const float *proj, size_t T, size_t H, size_t W, const float *angles,
                        const float *centre, float pixel_size, const float *ctf, size_t D,
                        float min_defocus, float max_defocus, const double *weights, int minus,
                        size_t Z, const size_t *rows, size_t nrows, double *out, int nthreads) {
  set_threads(nthreads);
  size_t nd = D > 0 ? D : 1;
  size_t img = H * W;
  double *stack = (double *)malloc(T * nd * img * sizeof(double));
  if (D > 0) {
#pragma omp parallel for schedule(dynamic, 1)
    for (long t = 0; t < (long)T; ++t) {
      double *im = (double *)malloc(img * sizeof(double));
      for (size_t k = 0; k < img; ++k) im[k] = (double)proj[(size_t)t * img + k];
      gno_correct_d(im, ctf, stack + (size_t)t * nd * img, W, H, nd);
      free(im);
    }
  } else {
    for (size_t k = 0; k < T * img; ++k) stack[k] = (double)proj[k];
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (long i = 0; i < (long)nrows; ++i) {
    size_t y = rows[i];
    double *sino = (double *)malloc(nd * T * W * sizeof(double));
    for (size_t d = 0; d < nd; ++d)
      for (size_t t = 0; t < T; ++t) {
        const double *src = stack + ((t * nd + d) * H + y) * W;
        double *dst = sino + (d * T + t) * W;
        double wt = weights ? (double)weights[t] : 1.0;
        for (size_t x = 0; x < W; ++x) dst[x] = (minus ? -src[x] : src[x]) * wt;
      }
    gno_config cfg;
    cfg.num_pixels = W;
    cfg.num_angles = T;
    cfg.num_defocus = nd;
    cfg.grid_height = Z;
    cfg.grid_width = W;
    cfg.pixel_size = pixel_size;
    cfg.centre = centre[y];
    cfg.min_defocus = D > 1 ? min_defocus : 0.0f;
    cfg.max_defocus = D > 1 ? max_defocus : 0.0f;
    cfg.angles = angles;
    gno_recon_d(&cfg, sino, out + (size_t)i * Z * W);
    free(sino);
  }
  free(stack);
}

void gno_fbp_ctf_d(const float *proj, size_t T, size_t H, size_t W, const float *angles,
                   const float *centre, float pixel_size, const float *ctf, size_t D,
                   float min_defocus, float max_defocus, const double *weights, int minus,
                   size_t Z, double *vol, size_t y_begin, size_t y_end, int nthreads) {
  size_t *rows = row_range(y_begin, y_end);
  gno_fbp_ctf_rows_d(proj, T, H, W, angles, centre, pixel_size, ctf, D, min_defocus,
                     max_defocus, weights, minus, Z, rows, y_end > y_begin ? y_end - y_begin : 0,
                     vol + y_begin * Z * W, nthreads);
  free(rows);
}
