/*
 * Oracle for guanaco's 3D-CTF filtered-backprojection path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * CPU path, used as the parity checker by tests/, by __graft_entry__.smoke()
 * and by the CPU-baseline leg of bench.py.  The product (guanaco_gb300) never
 * links or calls it.
 *
 * Two precisions:
 *   *_f : the reference CPU path's own float arithmetic, operation by
 *         operation (built with -ffp-contract=off so no FMA is formed), with
 *         the oracle FFT standing in for FFTW single precision.
 *   *_d : the same algorithm in double precision (the FP64 oracle).  Discrete
 *         decisions that the reference takes in float -- the defocus-slab index
 *         and the CTF phase-flip sign -- are taken with the reference's float
 *         rule so both precisions assign identical slabs and signs.
 *
 * Every function cites the reference file:line it follows (paths relative to
 * the guanaco source tree).
 */
#ifndef GNO_ORACLE_H
#define GNO_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- CTF physics, double (include/guanaco/ctf.h) ---------------------- */
typedef struct {
  double l;       /* wavelength (A) */
  double df;      /* defocus (A) */
  double Cs;      /* spherical aberration (A) */
  double Ca;      /* 2-fold astigmatism (A) */
  double Pa;      /* astigmatism angle (rad) */
  double dd;      /* defocus spread (A) */
  double theta_c; /* source spread (rad) */
  double phi;     /* phase shift (rad) */
} gno_ctf_params;

double gno_electron_wavelength(double V);                              /* ctf.h:39-48 */
double gno_defocus_spread(double Cc, double dEE, double dII, double dVV); /* ctf.h:61-64 */
void gno_r_and_theta(size_t x, size_t y, size_t w, size_t h, double inv_ps,
                     double *r, double *theta);                         /* ctf.h:88-101 */
double gno_chi(const gno_ctf_params *c, double q, double theta);        /* ctf.h:233-238 */
double gno_log_Es(const gno_ctf_params *c, double q, double theta);     /* ctf.h:188-195 */
double gno_log_Et(const gno_ctf_params *c, double q);                   /* ctf.h:204-209 */
double gno_A(const gno_ctf_params *c, double q);                        /* ctf.h:218-223 */
/* (h, w) grids, complex output interleaved re/im: ctf.h:466-503 */
void gno_ctf_grid(const gno_ctf_params *c, size_t w, size_t h, double ps, int simple,
                  double *out);

/* ---- CTF phase-flip correction (src/libguanaco/correct.cpp:30-90) ------ */
/* image (ysize, xsize); ctf (num_ctf, ysize, xsize) complex64 interleaved;
 * rec (num_ctf, ysize, xsize).  Output is unnormalised like the reference. */
void gno_correct_f(const float *image, const float *ctf, float *rec, size_t xsize,
                   size_t ysize, size_t num_ctf);
void gno_correct_d(const double *image, const float *ctf, double *rec, size_t xsize,
                   size_t ysize, size_t num_ctf);

/* ---- Ramp filter (src/libguanaco/filter.cpp:30-97) --------------------- */
/* num_rows rows of num_pixels each, filtered in place. */
void gno_filter_f(float *data, size_t num_pixels, size_t num_rows);
void gno_filter_d(double *data, size_t num_pixels, size_t num_rows);

/* ---- Backprojection (src/libguanaco/reconstructor.cpp:14-115) ---------- */
typedef struct {
  size_t num_pixels;
  size_t num_angles;
  size_t num_defocus;
  size_t grid_height; /* Z */
  size_t grid_width;  /* X */
  float pixel_size;
  float centre;
  float min_defocus;
  float max_defocus;
  const float *angles; /* num_angles, radians */
} gno_config;

/* Accumulates into rec (grid_height, grid_width); reconstructor.cpp:14-90 */
void gno_project_f(const gno_config *cfg, const float *sino, float *rec);
void gno_project_d(const gno_config *cfg, const double *sino, double *rec);
/* copy, filter, zero, project: reconstructor.cpp:92-115 */
void gno_recon_f(const gno_config *cfg, const float *sino, float *rec);
void gno_recon_d(const gno_config *cfg, const double *sino, double *rec);
/* The defocus-slab index the reference assigns to every (tilt, z, x):
 * out[(t*grid_height + z)*grid_width + x]; reconstructor.cpp:28-73. */
void gno_slab_index_map(const gno_config *cfg, int32_t *out);

/* ---- Whole 3D-CTF FBP pipeline ----------------------------------------
 * correct.py:217-318 (per-tilt corr) + reconstruct.py:127-213 and
 * mp.py:106-153 (per-row weights / transform / recon).
 * proj (T, H, W); ctf (D, H, W) complex64 (NULL when D == 0 means "no
 * correction": the projections are reconstructed directly with one slab);
 * centre (H) per row; weights (T, float64 as numpy keeps them) or NULL; vol (H, Z, W) for rows
 * [y_begin, y_end) only (rows outside are left untouched).
 * Correction covers tilts [t_begin, t_end) only when timing a sample; a full
 * run passes 0, T.  nthreads <= 0 uses all OpenMP threads. */
void gno_fbp_ctf_f(const float *proj, size_t T, size_t H, size_t W, const float *angles,
                   const float *centre, float pixel_size, const float *ctf, size_t D,
                   float min_defocus, float max_defocus, const double *weights, int minus,
                   size_t Z, float *vol, size_t y_begin, size_t y_end, size_t t_begin,
                   size_t t_end, int nthreads);
void gno_fbp_ctf_d(const float *proj, size_t T, size_t H, size_t W, const float *angles,
                   const float *centre, float pixel_size, const float *ctf, size_t D,
                   float min_defocus, float max_defocus, const double *weights, int minus,
                   size_t Z, double *vol, size_t y_begin, size_t y_end, int nthreads);
/* The same for an arbitrary list of rows: rows[i] (i < nrows) is written to
 * out + i * Z * W, so a sample of bands of a large volume needs one
 * correction pass and only the sampled rows' memory. */
void gno_fbp_ctf_rows_f(const float *proj, size_t T, size_t H, size_t W, const float *angles,
                        const float *centre, float pixel_size, const float *ctf, size_t D,
                        float min_defocus, float max_defocus, const double *weights, int minus,
                        size_t Z, const size_t *rows, size_t nrows, float *out, size_t t_begin,
                        size_t t_end, int nthreads);
void gno_fbp_ctf_rows_d(const float *proj, size_t T, size_t H, size_t W, const float *angles,
                        const float *centre, float pixel_size, const float *ctf, size_t D,
                        float min_defocus, float max_defocus, const double *weights, int minus,
                        size_t Z, const size_t *rows, size_t nrows, double *out, int nthreads);

#ifdef __cplusplus
}
#endif

#endif
