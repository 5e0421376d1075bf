/*
 * guanaco_gb300 -- C ABI of the GB300 (sm_103a) implementation of guanaco's
 * 3D-CTF filtered-backprojection path.
 *
 * Every entry point returns a gnc_status (0 on success).  On failure
 * gnc_last_error() returns a message for the calling thread; argument checks
 * that correspond to a GUANACO_ASSERT in the reference report
 * GNC_ERR_INVALID_ARGUMENT with the asserted condition in the message, the
 * way guanaco::Error carries "file:line ASSERT (...) failed"
 * (include/guanaco/error.h:31-61).
 *
 * Pointers are plain host or device pointers (as named), sizes are element
 * counts, streams are cudaStream_t passed as void* (NULL = legacy default
 * stream).  No entry point takes ownership of caller memory.
 *
 * Reference paths below are relative to the guanaco source tree.
 */
#ifndef GUANACO_GB300_H
#define GUANACO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define GNC_API __attribute__((visibility("default")))
#else
#define GNC_API
#endif

typedef enum {
  GNC_OK = 0,
  GNC_ERR_INVALID_ARGUMENT = 1, /* a reference GUANACO_ASSERT would fire */
  GNC_ERR_UNSUPPORTED = 2,      /* valid for the reference, not built here (message says why) */
  GNC_ERR_CUDA = 3,             /* CUDA runtime error (message has cudaGetErrorString) */
  GNC_ERR_OUT_OF_MEMORY = 4,
  GNC_ERR_DEVICE = 5,           /* device path requested on a machine without a usable GPU */
  GNC_ERR_PENDING = 6           /* gnc_server_wait: the request has not finished yet */
} gnc_status;

/* Message of the last failed call on this thread ("" if none). */
GNC_API const char *gnc_last_error(void);
/* ABI version: major * 10000 + minor * 100 + patch. */
GNC_API int gnc_version(void);

/* ------------------------------------------------------------------------
 * Configuration: guanaco::Config (include/guanaco/config.h:29-76).
 * device 1 = e_device is the only value this library runs; 0 = e_host is
 * rejected with GNC_ERR_UNSUPPORTED (the CPU path is the reference's).
 * ---------------------------------------------------------------------- */
typedef struct {
  int device;           /* eDevice: 0 e_host, 1 e_device */
  int gpu_index;        /* cudaSetDevice(gpu_index) when >= 0 (reconstructor.cu:321-328) */
  size_t num_pixels;    /* N */
  size_t num_angles;    /* T */
  size_t num_defocus;   /* D */
  size_t grid_height;   /* Z */
  size_t grid_width;    /* X */
  float pixel_size;     /* A */
  float centre;         /* rotation centre (px) */
  float min_defocus;    /* A, relative to the defocus at the tilt axis */
  float max_defocus;    /* A */
  const float *angles;  /* host, num_angles, radians */
} gnc_config;

/* guanaco::Reconstructor(config)(sinogram, reconstruction) on the device path
 * (src/libguanaco/reconstructor.cpp:117-131 -> reconstructor.cu:317-354).
 * Host pointers: sinogram (D, T, N) float32, reconstruction (Z, X) float32,
 * overwritten.  Synchronous.  Bound from Python as guanaco.detail.recon
 * (src/guanaco/detail/ext/reconstruct.h:35-101). */
GNC_API int gnc_reconstruct(const gnc_config *config, const float *sinogram,
                            float *reconstruction);

/* The same on device pointers, enqueued on `stream`. */
GNC_API int gnc_reconstruct_device(const gnc_config *config, const float *d_sinogram,
                                   float *d_reconstruction, void *stream);

/* No counterpart in the reference.  gnc_reconstruct_device without any device
 * allocation, for callers that cannot allocate inside a call: an application
 * that owns a fixed device-memory budget, or a real-time loop that must not
 * touch the allocator.  Its scratch lives
 * in static device arrays (about 16.1 MiB held by every GPU that loads the
 * library until exit).  Limits: num_defocus * num_angles * num_pixels <=
 * 4194304, num_angles <= 1024, num_pixels <= 4096; larger requests return
 * GNC_ERR_INVALID_ARGUMENT (other checks and statuses as for
 * gnc_reconstruct_device).  All calls on a device share the scratch, so calls
 * that overlap on the GPU race; serialise them.  Every call looks up the
 * scratch's device addresses on the current device (cudaGetSymbolAddress,
 * which allocates nothing); the first call on a device is its set-up, which
 * loads the library's device code there, so make it before any stream
 * capture on that device. */
GNC_API int gnc_reconstruct_device_noalloc(const gnc_config *config, const float *d_sinogram,
                                           float *d_reconstruction, void *stream);

/* guanaco::Filter<e_device>(num_pixels, num_angles, num_defocus)(data)
 * (include/guanaco/filter.h:32-54, src/libguanaco/filter.cu:144-202): ramp
 * filter of D*T rows of N pixels in place, device pointer. */
GNC_API int gnc_filter_device(size_t num_pixels, size_t num_angles, size_t num_defocus,
                              float *d_data, void *stream);

/* guanaco::correct<float>(image, ctf, rec, xsize, ysize, num_ctf, e_device)
 * (include/guanaco/correct.h:77-95, src/libguanaco/correct.cu:30-86).
 * Host pointers: image (ysize, xsize) float32, ctf (num_ctf, ysize, xsize)
 * complex64 as interleaved float pairs, rec (num_ctf, ysize, xsize) float32.
 * Output is unnormalised (xsize * ysize times the corrected image), as in the
 * reference.  Bound from Python as guanaco.detail.corr
 * (src/guanaco/detail/ext/correct.h:32-76). */
GNC_API int gnc_correct(const float *image, const float *ctf, float *rec, size_t xsize,
                        size_t ysize, size_t num_ctf);

/* ------------------------------------------------------------------------
 * CTF physics, host, double (include/guanaco/ctf.h).  Bound from Python as
 * the guanaco_ext CTF class and free functions (src/guanaco/detail/ext/ctf.h).
 * ---------------------------------------------------------------------- */
typedef struct {
  double l;       /* wavelength (A) */
  double df;      /* defocus (A) */
  double Cs;      /* spherical aberration (A) */
  double Ca;      /* 2-fold astigmatism (A) */
  double Pa;      /* astigmatism angle (rad) */
  double dd;      /* defocus spread (A) */
  double theta_c; /* source spread (rad) */
  double phi;     /* phase shift (rad) */
} gnc_ctf; /* guanaco::CTF, ctf.h:167-178 */

enum {
  GNC_CTF_FULL = 0,        /* complex: get_ctf, ctf.h:250-257 */
  GNC_CTF_SIMPLE = 1,      /* complex: get_ctf_simple, ctf.h:269-273 */
  GNC_CTF_SIMPLE_REAL = 2, /* ctf.h:285-288 */
  GNC_CTF_SIMPLE_IMAG = 3, /* ctf.h:300-303 */
  GNC_CTF_CHI = 4,         /* get_chi, ctf.h:233-238 */
  GNC_CTF_ES = 5,          /* exp(get_log_Es), ctf.h:314-319 */
  GNC_CTF_ET = 6           /* exp(get_log_Et), ctf.h:329-332 */
};

GNC_API double gnc_get_electron_wavelength(double V);                       /* ctf.h:39-48 */
GNC_API double gnc_get_defocus_spread(double Cc, double dEE, double dII, double dVV); /* :61-64 */
GNC_API double gnc_q_to_Q(double q, double l, double Cs);                   /* ctf.h:114-117 */
GNC_API double gnc_Q_to_q(double Q, double l, double Cs);                   /* ctf.h:129-132 */
GNC_API double gnc_df_to_D(double df, double l, double Cs);                 /* ctf.h:144-147 */
GNC_API double gnc_D_to_df(double D, double l, double Cs);                  /* ctf.h:159-162 */
GNC_API double gnc_ctf_chi(const gnc_ctf *c, double q, double theta);       /* ctf.h:233-238 */
/* Element-wise over n (q, theta) pairs; complex kinds write 2n doubles. */
GNC_API int gnc_ctf_eval(const gnc_ctf *c, int kind, const double *q, const double *theta,
                         size_t n, double *out);
/* (h, w) FFT-ordered grid at pixel size ps: ctf.h:466-557; get_q_and_theta
 * (src/guanaco/detail/ext/ctf.h:41-56). */
GNC_API int gnc_ctf_grid(const gnc_ctf *c, int kind, size_t w, size_t h, double ps, double *out);
GNC_API int gnc_q_and_theta(size_t w, size_t h, double ps, double *q, double *theta);
/* CTF image stack computed on the device: slab d is the (h, w) FFT-ordered grid
 * of `kind` (as gnc_ctf_grid, double arithmetic) with the defocus replaced by
 * defocus[d] (host array of num_defocus values; c->df is not used), written to
 * d_out as complex64 (kinds FULL, SIMPLE) or float32 (the others), shape
 * (num_defocus, h, w), on `stream`.  Replaces the per-slab host loops of
 * generate_ctf (src/guanaco/plot.py:175-284, CTF.get_ctf per defocus) and
 * get_ctf_array (src/guanaco/detail/correct.py:157-214). */
GNC_API int gnc_ctf_image_device(const gnc_ctf *c, int kind, const double *defocus,
                                 int num_defocus, size_t w, size_t h, double ps, void *d_out,
                                 void *stream);

/* ------------------------------------------------------------------------
 * Whole-series 3D-CTF FBP.  One plan replaces the reference's
 * correct_projections (src/guanaco/detail/correct.py:217-318, one corr call
 * per tilt) followed by reconstruct (src/guanaco/detail/reconstruct.py:127-213,
 * one recon call per Y row from src/guanaco/detail/mp.py:106-153): the same
 * arithmetic, for every tilt and row in one device-resident pass.
 * ---------------------------------------------------------------------- */
typedef struct gnc_fbp_plan gnc_fbp_plan;

/* Staging of the filtered rows between the ramp filter and the backprojection:
 * F32; F16 (per-row exponents, CUDA-core backprojection); F16T (FP16 rows
 * with one power-of-two scale per tilt, backprojected on the tensor cores
 * with FP32 accumulation; where that kernel does not take the geometry --
 * rows with different centres, a width not a multiple of 8, more than 512
 * tilts or slabs thinner than about 10 pixels -- a plan uses F16). */
enum { GNC_STAGE_F32 = 0, GNC_STAGE_F16 = 1, GNC_STAGE_F16T = 2 };
enum { GNC_INPUT_RAW = 0, GNC_INPUT_CORRECTED = 1 };

typedef struct {
  size_t num_angles;     /* T */
  size_t height;         /* H: image rows = volume Y */
  size_t width;          /* W: image columns = detector pixels N */
  size_t grid_height;    /* Z (the reference's Python path uses W) */
  size_t grid_width;     /* X (the reference's Python path uses W) */
  const float *angles;   /* host, T radians */
  const float *centre;   /* host, H per-row rotation centres; NULL = W / 2 */
  float pixel_size;      /* A */
  int input;             /* GNC_INPUT_RAW: (T, H, W) projections, corrected here;
                            GNC_INPUT_CORRECTED: (T, D, H, W) already corrected */
  int correct;           /* RAW input only: 1 = CTF phase flip, 0 = none (D must be 1) */
  size_t num_defocus;    /* D >= 1 */
  const double *slab_defocus; /* host, D absolute slab defoci (A) for the CTF (correct.py:195-199) */
  float min_defocus;     /* relative range handed to the backprojector (correct.py:318) */
  float max_defocus;
  double energy_kev;     /* CTF: wavelength from energy * 1000 eV (correct.py:146) */
  double cs_mm;          /* CTF: Cs * 1e7 A (correct.py:148) */
  double astigmatism;    /* A */
  double astigmatism_angle_deg;
  double phase_shift_deg;
  const double *weights; /* host, T per-tilt weights (mp.py:135-141) or NULL */
  int minus;             /* transform == "minus" (mp.py:128-129) */
  int staging;           /* GNC_STAGE_F32, GNC_STAGE_F16 or GNC_STAGE_F16T */
  double ctf_pixel_size; /* A, for the CTF only, in double as the reference's CTF
                            takes it (src/guanaco/detail/ext/ctf.h:142-149);
                            0 = pixel_size */
} gnc_fbp_desc;

/* Allocates the plan's device workspace on the current device. */
GNC_API int gnc_fbp_plan_create(const gnc_fbp_desc *desc, gnc_fbp_plan **plan);
GNC_API int gnc_fbp_plan_destroy(gnc_fbp_plan *plan);
GNC_API size_t gnc_fbp_workspace_bytes(const gnc_fbp_plan *plan);
/* Input (T, H, W) or (T, D, H, W) float32 device; volume (H, Z, X) float32
 * device, overwritten. */
GNC_API int gnc_fbp_execute(gnc_fbp_plan *plan, const float *d_input, float *d_volume,
                            void *stream);
/* The same from host buffers, synchronising before it returns.  The input
 * goes up in tilt groups and the volume comes down in row slabs, overlapped
 * with the kernels on two streams of the plan; the first call creates them
 * and the device input/output buffers (kept until the plan is destroyed, not
 * counted by gnc_fbp_workspace_bytes).  Pinned host memory gives the fastest
 * copies. */
GNC_API int gnc_fbp_execute_host(gnc_fbp_plan *plan, const float *h_input, float *h_volume,
                                 void *stream);
/* No counterpart in the reference.  Page-locked host memory of exactly `bytes`
 * (cudaHostAlloc) for the host buffers of gnc_fbp_execute_host and of the
 * request server: copies from and to it run at the host link's full rate.
 * Release with gnc_host_free. */
GNC_API int gnc_host_alloc(size_t bytes, void **ptr);
GNC_API int gnc_host_free(void *ptr);
/* Correction only: raw (T, H, W) -> corrected stack (T, D, H, W), the output
 * of correct_projections (correct.py:276-303), device pointers. */
GNC_API int gnc_fbp_correct(gnc_fbp_plan *plan, const float *d_proj, float *d_corrected,
                            void *stream);
/* Stage entry points used by tests and benchmarks. */
GNC_API int gnc_fbp_stage(gnc_fbp_plan *plan, const float *d_input, void *stream);
GNC_API int gnc_fbp_backproject(gnc_fbp_plan *plan, float *d_volume, int exact, void *stream);
/* Backprojection of caller-provided staged rows (same layout as
 * gnc_fbp_staged describes) with this plan's geometry. */
GNC_API int gnc_fbp_backproject_staged(gnc_fbp_plan *plan, const void *d_staged,
                                       const int8_t *d_row_exp, float *d_volume, int exact,
                                       void *stream);
/* int32 (T, Z, X) slab index the backprojector assigns (reconstructor.cpp:66-72). */
GNC_API int gnc_fbp_slab_map(gnc_fbp_plan *plan, int32_t *d_out, void *stream);
/* int8 (D, H, W/2 + 1) table of s(k) + s(-k) with s the phase-flip factor. */
GNC_API int gnc_fbp_sign_table(gnc_fbp_plan *plan, int8_t *d_out, void *stream);
/* Number of kernel launches one gnc_fbp_execute enqueues. */
GNC_API int gnc_fbp_launches(const gnc_fbp_plan *plan);
/* Per tilt, the first and last defocus slab any voxel of the volume reads
 * (h_out: 2 * T int32, host), as the plan computes them on the device; the
 * phase flip and ramp filter of gnc_fbp_execute skip the other (tilt, slab)
 * pairs, whose staged rows are then left unwritten.  Synchronises `stream`. */
GNC_API int gnc_fbp_live_slabs(gnc_fbp_plan *plan, int32_t *h_out, void *stream);
/* Which backprojection kernel gnc_fbp_execute runs for this plan: 0 the
 * exact kernel (rows with different centres, an odd detector width or too
 * many slabs per tile), 2 or 4 the CUDA-core fast kernel (its slab capacity
 * per tile), 16 the tensor-core kernel of F16T staging; -1 for a null plan. */
GNC_API int gnc_fbp_backprojector(const gnc_fbp_plan *plan);
/* Test hook of the failure detection, no counterpart in the reference.
 * polls > 0: plans created afterwards (by gnc_fbp_plan_create and by the
 * request server) make every fast backprojection launch arm one spare
 * mbarrier for 16 bytes that no copy delivers and wait on it at most `polls`
 * polls, so the wait gives up and sets the plan's error word exactly as a lost
 * bulk copy would (gnc_fbp_check returns GNC_ERR_CUDA, a served request
 * reports device_error); the volume is still computed, no copy is in flight on
 * that barrier and the kernel ends normally.  polls = 0 (the default) turns it
 * off for plans created afterwards. */
GNC_API int gnc_debug_wait_probe(unsigned polls);
/* Synchronises `stream` and reports (then clears) a device-side error of the
 * plan's kernels: every wait in them is bounded and records a timeout here
 * instead of hanging. */
GNC_API int gnc_fbp_check(gnc_fbp_plan *plan, void *stream);
/* Staged filtered rows, (ceil(H/2), D, T, W) pixels of row pairs (rows 2 y2 and
 * 2 y2 + 1), 8 bytes each:
 *   F32: float (v_a, v_b)
 *   F16: half (v_a, v_b, dv_a, dv_b), dv the difference of the next pixel's FP16
 *        value and this one (0 for the last pixel), value = half * 2^-e;
 *        with the (ceil(H/2), D, T, 2) int8 row exponents e.
 * F16T plans instead stage plain FP16 rows (D, T, H, W), value = half * 2^-e(t),
 * with the (T) int8 tilt exponents in place of the row exponents. */
GNC_API int gnc_fbp_staged(gnc_fbp_plan *plan, const void **d_staged, const int8_t **d_row_exp);

/* ------------------------------------------------------------------------
 * Request server: continuous batching of whole-series FBP requests on one GPU.
 * No counterpart in the reference, which runs one synchronous call at a time
 * (src/guanaco/detail/mp.py:38-153 loops over rows inside one request).
 *
 * Requests (a gnc_fbp_desc plus host input and output buffers) are queued by
 * gnc_server_submit and admitted by a scheduler thread whenever one of the
 * server's slots (CUDA streams) is free and the request's plan fits in the
 * device-memory budget; requests of different sizes and parameters run
 * concurrently on the slots.  Plans are cached by shape (gnc_fbp_desc minus
 * the per-request values: angles, centres, defocus, CTF constants, weights)
 * and the device work of a cached plan is captured once as a CUDA graph; a
 * later request of that shape uploads its parameters and replays the graph.
 * Idle cached plans are released (least recently used first) when a new shape
 * needs the memory.  Page-locked host buffers let the copies run
 * asynchronously; the buffers must stay valid until gnc_server_wait reports
 * the request finished.
 * ---------------------------------------------------------------------- */
typedef struct gnc_server gnc_server;

typedef struct {
  int status;          /* GNC_OK, or the request's error (gnc_server_wait returns it too) */
  int graph;           /* 1: ran as a replay of a captured graph, 0: direct launches */
  int device_error;    /* a bounded wait in a kernel gave up (status GNC_ERR_CUDA) */
  double t_submit;     /* seconds on the server clock (gnc_server_now) */
  double t_start;      /* admitted: parameters, input copy and kernels enqueued */
  double t_done;       /* volume back in the host buffer */
} gnc_request_info;

typedef struct {
  uint64_t submitted, completed, failed;
  uint64_t graph_launches, direct_launches, plans_created, plans_evicted;
  size_t budget_bytes, bytes_in_use;
  int slots, cached_plans, in_flight, peak_in_flight, queued;
} gnc_server_stats;

/* Creates a server on the current device with `slots` concurrent requests
 * (1..64) and a device-memory budget for its plans and request buffers. */
GNC_API int gnc_server_create(size_t budget_bytes, int slots, gnc_server **server);
/* Waits for every admitted request, then frees everything; queued requests
 * that were never admitted finish with GNC_ERR_INVALID_ARGUMENT. */
GNC_API int gnc_server_destroy(gnc_server *server);
/* Queues one request: desc as for gnc_fbp_plan_create (its arrays are copied),
 * h_input (T, H, W) raw or (T, D, H, W) corrected float32, h_volume (H, Z, X)
 * float32 written when the request finishes.  Invalid or unsupported
 * descriptors, and requests larger than the whole budget, fail here. */
GNC_API int gnc_server_submit(gnc_server *server, const gnc_fbp_desc *desc, const float *h_input,
                              float *h_volume, uint64_t *id);
/* Waits up to timeout_s seconds (< 0: forever) for request id.  Returns
 * GNC_ERR_PENDING if it has not finished, else its status, and fills info
 * (may be NULL); a finished request is forgotten after this call. */
GNC_API int gnc_server_wait(gnc_server *server, uint64_t id, double timeout_s,
                            gnc_request_info *info);
/* Waits up to timeout_s seconds (< 0: forever) for any request that has
 * finished and not been collected (by this call or gnc_server_wait), in the
 * order requests finish; sets *id and returns as gnc_server_wait does for it.
 * Returns GNC_ERR_PENDING if none finished in time, at once if no request is
 * outstanding.  A client serving a stream collects each request with one call
 * instead of polling every outstanding id. */
GNC_API int gnc_server_wait_any(gnc_server *server, double timeout_s, uint64_t *id,
                                gnc_request_info *info);
/* Seconds since the server was created (the clock of gnc_request_info). */
GNC_API double gnc_server_now(const gnc_server *server);
GNC_API int gnc_server_get_stats(gnc_server *server, gnc_server_stats *stats);

#ifdef __cplusplus
}
#endif

#endif /* GUANACO_GB300_H */
