// Host side of guanaco_gb300: error state, FFT twiddle cache, the whole-series
// FBP plan and every C ABI entry point declared in include/guanaco_gb300.h.
//
// The host geometry (per-tilt cos/sin/offset/scale, slab scale/offset) is
// computed with the reference's float arithmetic; this file is compiled with
// -ffp-contract=off so the host compiler forms no fused multiply-add on any
// architecture.
#include <math.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/guanaco_gb300.h"
#include "gnc_common.cuh"
#include "gnc_host_geom.h"
#include "gnc_plan_hooks.h"

namespace gnc {

// ---------------------------------------------------------------- errors ---
static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }
const char *last_error() { return g_last_error.c_str(); }

// ----------------------------------------------------------- FFT plans -----
static std::mutex g_fft_lock;
static std::map<std::pair<int, int>, const float2 *> g_roots;

static bool factorize(long n, int *radix, int *nstage) {
  int ns = 0;
  while (n % 8 == 0) { radix[ns++] = 8; n /= 8; }
  while (n % 4 == 0) { radix[ns++] = 4; n /= 4; }
  while (n % 2 == 0) { radix[ns++] = 2; n /= 2; }
  for (long p = 3; n > 1; p += 2) {
    while (n % p == 0) {
      if (p > kMaxRadix || ns >= kMaxStages) return false;
      radix[ns++] = (int)p;
      n /= p;
    }
  }
  *nstage = ns;
  return true;
}

bool fft_length_supported(long n) {
  int r[kMaxStages], ns = 0;
  return n >= 1 && factorize(n, r, &ns);
}

bool make_fft_factors(int n, FftPlan *out) {
  FftPlan p{};
  p.n = n;
  if (!factorize(n, p.radix, &p.nstage)) return false;
  *out = p;
  return true;
}

bool make_fft_plan(int n, FftPlan *out) {
  FftPlan p{};
  p.n = n;
  if (!factorize(n, p.radix, &p.nstage)) {
    set_error("transform length " + std::to_string(n) + " has a prime factor above " +
              std::to_string(kMaxRadix));
    return false;
  }
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_fft_lock);
  auto key = std::make_pair(dev, n);
  auto it = g_roots.find(key);
  if (it == g_roots.end()) {
    std::vector<float2> h(n);
    for (int k = 0; k < n; ++k) {
      double a = 2.0 * M_PI * (double)k / (double)n;
      h[k] = make_float2((float)std::cos(a), (float)-std::sin(a));
    }
    float2 *d = nullptr;
    if (cudaMalloc(&d, n * sizeof(float2)) != cudaSuccess ||
        cudaMemcpy(d, h.data(), n * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess) {
      set_error("cannot allocate FFT twiddles");
      return false;
    }
    it = g_roots.emplace(key, d).first;
  }
  p.roots = it->second;
  *out = p;
  return true;
}

}  // namespace gnc

using namespace gnc;

#define GNC_REQUIRE(cond)                                                   \
  do {                                                                      \
    if (!(cond)) {                                                          \
      set_error(std::string(__func__) + ": ASSERT (" #cond ") failed");     \
      return GNC_ERR_INVALID_ARGUMENT;                                      \
    }                                                                       \
  } while (0)

#define GNC_CUDA(expr)                                                       \
  do {                                                                       \
    cudaError_t e_ = (expr);                                                 \
    if (e_ != cudaSuccess) {                                                 \
      set_error(std::string(__func__) + ": " #expr ": " + cudaGetErrorString(e_)); \
      return e_ == cudaErrorMemoryAllocation ? GNC_ERR_OUT_OF_MEMORY : GNC_ERR_CUDA; \
    }                                                                        \
  } while (0)

// Test hook of the bounded device waits (gnc_debug_wait_probe): plans copy
// the value when they are created.
static std::atomic<unsigned> g_wait_probe{0};

// ------------------------------------------------------------- the plan ----
// Host-buffer pipeline: input copies in up to kIoGroups tilt groups, volume
// copies out in up to kIoSlabs row slabs (eight, the last one split in three
// so the copy that remains after the last kernel is short), plus two events
// for the stream joins.
constexpr int kIoGroups = 32, kIoSlabs = 10, kIoEvents = kIoGroups + kIoSlabs + 2;
// Largest phase-flipped spectrum stack (T, D, H, W/2) the host-buffer path
// keeps whole so that it can filter and backproject row slab by row slab.
constexpr size_t kSlabMajorMaxBytes = (size_t)8 << 30;
// Tilts whose phase-flipped spectra one flip launch produces and one row-stage
// launch consumes (two such chunks in flight): enough tilts for 48 MB, at
// least 4 while that stays within 192 MB (1024^2 x ten slabs: 4 tilts of
// 42 MB; larger launches fill the GPU's last wave better than L2-sized ones
// save in traffic), at least 1.
static size_t flip_chunk(size_t T, size_t per_tilt) {
  const size_t by_l2 = ((size_t)48 << 20) / per_tilt, cap = ((size_t)192 << 20) / per_tilt;
  return std::max<size_t>(1, std::min<size_t>(T, std::min(cap, std::max<size_t>(4, by_l2))));
}

// Per-request parameter block of a plan: the same byte layout on the host and
// on the device, so one copy moves all of it.
struct ParamLayout {
  size_t sign, bp, geom, factor, slab, offset, bytes;
};
static ParamLayout param_layout(int T, int H, int D) {
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  ParamLayout L{};
  size_t o = 0;
  L.sign = o;
  o = up(o + sizeof(SignTableArgs));
  L.bp = o;
  o = up(o + 2 * sizeof(float));
  L.geom = o;
  o = up(o + (size_t)T * sizeof(TiltGeom));
  L.factor = o;
  o = up(o + (size_t)T * sizeof(float));
  L.slab = o;
  o = up(o + (size_t)D * sizeof(double));
  L.offset = o;
  o = up(o + (size_t)H * T * sizeof(float));
  L.bytes = o;
  return L;
}

struct gnc_fbp_plan {
  int device = 0;
  int T = 0, H = 0, W = 0, Z = 0, X = 0, D = 1, Y2 = 0;
  int input = GNC_INPUT_RAW, correct = 0, staging = GNC_STAGE_F32;
  float pixel_size = 1.f, min_def = 0.f, max_def = 0.f, dscale = 0.f, doffset = 0.f;
  bool uniform_centre = true;
  int chunk = 1;
  SignTableArgs sargs{};
  // device memory
  float2 *spec = nullptr;   // (T, H, W/2)
  float2 *gbuf = nullptr;   // 2 x (chunk, D, H, W/2): flips of two chunks in flight
  // side stream for the phase flips, so a chunk's flip overlaps the previous
  // chunk's row stage; events: fork, flip done (per buffer), rows done (per buffer)
  cudaStream_t s_flip = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_flip[2] = {}, ev_rows[2] = {};
  void *staged = nullptr;   // (Y2, D, T, W) pairs, or F16T rows (D, T, H, W)
  int8_t *row_exp = nullptr;
  int8_t *tilt_exp = nullptr;  // F16T: (T) per-tilt exponents
  float *tilt_part = nullptr;  // F16T: (T, kTiltPartsMax) partial sums of squares
  TcMap tc_map{};              // F16T: TMA descriptor of the staged rows
  int8_t *sign = nullptr;   // (D, H, W/2 + 1)
  int2 *live = nullptr;     // (T): first and last slab the volume reads (CTF, D > 1)
  // everything that differs between two requests of the same shape, in one
  // block (ParamLayout): views into it
  unsigned char *params = nullptr;
  ParamLayout pl{};
  SignTableArgs *dyn_sign = nullptr;
  float *dyn_bp = nullptr;  // (dscale, doffset)
  double *slab_df = nullptr;
  TiltGeom *geom = nullptr;
  float *offset = nullptr;  // (H, T)
  float *tilt_factor = nullptr;
  int *err = nullptr;        // device error word of the bounded waits
  unsigned wait_probe = 0;   // gnc_debug_wait_probe's value when the plan was created
  size_t bytes = 0;
  // request-server plans: device memory from this pool, stream-ordered on
  // alloc_stream (null: cudaMalloc / cudaFree)
  cudaMemPool_t pool = nullptr;
  cudaStream_t alloc_stream = nullptr;
  // host-buffer path (gnc_fbp_execute_host), created on its first call
  float *io_in = nullptr, *io_out = nullptr;
  float2 *gfull = nullptr;  // (T, D, H, W/2) flipped spectra (slab-major order)
  bool gfull_tried = false;
  cudaStream_t s_in = nullptr, s_out = nullptr;
  cudaEvent_t ev[kIoEvents] = {};
};

// Device memory of a plan: from cudaMalloc, or -- for plans of the request
// server -- stream-ordered from the server's memory pool (no device-wide
// synchronisation when it is allocated or freed).
static void dfree(gnc_fbp_plan *p, void *ptr) {
  if (!ptr) return;
  if (p->pool)
    cudaFreeAsync(ptr, p->alloc_stream);
  else
    cudaFree(ptr);
}

static void plan_free(gnc_fbp_plan *p) {
  dfree(p, p->spec);
  dfree(p, p->gbuf);
  if (p->ev_fork) cudaEventDestroy(p->ev_fork);
  for (cudaEvent_t e : p->ev_flip)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : p->ev_rows)
    if (e) cudaEventDestroy(e);
  if (p->s_flip) cudaStreamDestroy(p->s_flip);
  dfree(p, p->staged);
  dfree(p, p->row_exp);
  dfree(p, p->tilt_exp);
  dfree(p, p->tilt_part);
  dfree(p, p->sign);
  dfree(p, p->live);
  dfree(p, p->params);
  dfree(p, p->err);
  cudaFree(p->io_in);  // the host-buffer path's buffers (never from the pool)
  cudaFree(p->io_out);
  cudaFree(p->gfull);
  for (cudaEvent_t e : p->ev)
    if (e) cudaEventDestroy(e);
  if (p->s_in) cudaStreamDestroy(p->s_in);
  if (p->s_out) cudaStreamDestroy(p->s_out);
}

template <typename T>
static cudaError_t dalloc(gnc_fbp_plan *p, T **ptr, size_t count) {
  size_t b = std::max<size_t>(count, 1) * sizeof(T);
  p->bytes += b;
  if (p->pool) return cudaMallocFromPoolAsync((void **)ptr, b, p->pool, p->alloc_stream);
  return cudaMalloc((void **)ptr, b);
}

static BpArgs bp_args(const gnc_fbp_plan *p, float *vol) {
  BpArgs a{};
  a.staged = p->staged;
  a.row_exp = p->row_exp;
  a.tilt_exp = p->tilt_exp;
  a.stack_h = p->H;
  a.y_begin = 0;
  a.staging = p->staging;
  a.Y = p->H;
  a.D = p->D;
  a.T = p->T;
  a.N = p->W;
  a.Z = p->Z;
  a.X = p->X;
  a.geom = p->geom;
  a.offset = p->offset;
  a.dscale = p->dscale;
  a.doffset = p->doffset;
  a.uniform_centre = p->uniform_centre ? 1 : 0;
  a.vol = vol;
  a.err = p->err;
  a.dyn = p->dyn_bp;
  a.wait_limit = 0;  // the default bound
  a.wait_probe = p->wait_probe;
  return a;
}

// Fills the parameter block `blk` (layout p->pl) for descriptor d: the tilt
// geometry and per-row detector offsets (reconstructor.cpp:35-47), per-tilt
// factors (weight and sign, mp.py:128-141), slab defoci, the CTF arguments of
// the sign table and the slab map (dscale, doffset).  Also returns whether all
// rows share one centre and the host copies of the by-value arguments.
static void fill_params(const gnc_fbp_plan *p, const gnc_fbp_desc *d, unsigned char *blk,
                        bool *uniform, float *dscale, float *doffset, SignTableArgs *sargs) {
  const ParamLayout &L = p->pl;
  const float min_def = d->num_defocus > 1 ? d->min_defocus : 0.f;
  const float max_def = d->num_defocus > 1 ? d->max_defocus : 0.f;
  defocus_scale(d->num_defocus, d->pixel_size, min_def, max_def, dscale, doffset);
  float *bp = (float *)(blk + L.bp);
  bp[0] = *dscale;
  bp[1] = *doffset;
  TiltGeom *geom = (TiltGeom *)(blk + L.geom);
  float *offset = (float *)(blk + L.offset);
  std::vector<float> centre(p->H);
  for (int y = 0; y < p->H; ++y) centre[y] = d->centre ? d->centre[y] : (float)(p->W * 0.5);
  *uniform = true;
  for (int y = 1; y < p->H; ++y)
    if (centre[y] != centre[0]) *uniform = false;
  for (int y = 0; y < p->H; ++y)
    for (int t = 0; t < p->T; ++t)
      geom[t] = tilt_geometry(d->angles[t], centre[y], d->num_angles, &offset[(size_t)y * p->T + t]);
  float *factor = (float *)(blk + L.factor);
  for (int t = 0; t < p->T; ++t)
    factor[t] = (float)((d->minus ? -1.0 : 1.0) * (d->weights ? d->weights[t] : 1.0));
  double *slab = (double *)(blk + L.slab);
  SignTableArgs sa{};
  if (p->correct) {
    for (int k = 0; k < p->D; ++k) slab[k] = d->slab_defocus[k];
    sa.D = p->D;
    sa.H = p->H;
    sa.W = p->W;
    sa.inv_ps = 1.0 / (d->ctf_pixel_size > 0 ? d->ctf_pixel_size : (double)d->pixel_size);
    sa.l = gnc_get_electron_wavelength(d->energy_kev * 1000);
    sa.Cs = d->cs_mm * 1e7;
    sa.Ca = d->astigmatism;
    sa.Pa = d->astigmatism_angle_deg * M_PI / 180;
    sa.phi = d->phase_shift_deg * M_PI / 180;
    sa.slab_df = p->slab_df;
    fill_sign_screen(&sa);
  }
  std::memcpy(blk + L.sign, &sa, sizeof(sa));  // the device copy has dyn = null
  sa.dyn = p->dyn_sign;
  *sargs = sa;
}

// ------------------------------------------- hooks for the request server --
namespace gnc {

int desc_check(const gnc_fbp_desc *d) {
  GNC_REQUIRE(d != nullptr);
  GNC_REQUIRE(d->num_angles > 0);
  GNC_REQUIRE(d->height > 0);
  GNC_REQUIRE(d->width > 0);
  GNC_REQUIRE(d->grid_height > 0);
  GNC_REQUIRE(d->grid_width > 0);
  GNC_REQUIRE(d->pixel_size > 0);
  GNC_REQUIRE(d->num_defocus > 0);
  GNC_REQUIRE(d->angles != nullptr);
  GNC_REQUIRE(d->min_defocus <= d->max_defocus);
  GNC_REQUIRE(d->num_defocus == 1 || d->max_defocus > d->min_defocus);
  GNC_REQUIRE(d->input == GNC_INPUT_RAW || d->input == GNC_INPUT_CORRECTED);
  GNC_REQUIRE(d->staging == GNC_STAGE_F32 || d->staging == GNC_STAGE_F16 ||
              d->staging == GNC_STAGE_F16T);
  const bool ctf = d->input == GNC_INPUT_RAW && d->correct;
  GNC_REQUIRE(ctf || d->input == GNC_INPUT_CORRECTED || d->num_defocus == 1);
  if (ctf) GNC_REQUIRE(d->slab_defocus != nullptr);
  if (d->width > 6400 || !fft_length_supported(2 * (long)d->width) ||
      (ctf && (d->width % 2 != 0 || d->height > 8192 || !fft_length_supported((long)d->height) ||
               !fft_length_supported((long)d->width)))) {
    set_error("gnc_fbp_plan_create: unsupported size (width <= 6400 with 2*width "
              "factorising into radices <= 16; with CTF correction an even width and a "
              "height <= 8192 that also factorise)");
    return GNC_ERR_UNSUPPORTED;
  }
  return GNC_OK;
}

// The staging a plan for d uses: F16T (FP16 rows, tensor-core backprojection)
// only where that kernel takes the geometry, else the FP16 records.
int effective_staging(const gnc_fbp_desc *d) {
  if (d->staging != GNC_STAGE_F16T) return d->staging;
  float dscale, doffset;
  const float mn = d->num_defocus > 1 ? d->min_defocus : 0.f;
  const float mx = d->num_defocus > 1 ? d->max_defocus : 0.f;
  defocus_scale(d->num_defocus, d->pixel_size, mn, mx, &dscale, &doffset);
  bool uniform = true;
  if (d->centre)
    for (size_t y = 1; y < d->height; ++y)
      if (d->centre[y] != d->centre[0]) uniform = false;
  return backproject_tc_supported((int)d->width, (int)d->num_angles, dscale,
                                  (int)d->num_defocus, uniform)
             ? GNC_STAGE_F16T
             : GNC_STAGE_F16;
}

// Device bytes gnc_fbp_plan_create allocates for d (the same sizes, without
// allocating), plus the input and output buffers of one request.
size_t plan_bytes(const gnc_fbp_desc *d) {
  const size_t T = d->num_angles, H = d->height, W = d->width, D = d->num_defocus;
  const size_t Y2 = (H + 1) / 2, half = W / 2;
  const bool ctf = d->input == GNC_INPUT_RAW && d->correct;
  size_t b = param_layout((int)T, (int)H, (int)D).bytes + sizeof(int);
  if (ctf) {
    const size_t per_tilt = D * H * half * sizeof(float2);
    const size_t chunk = flip_chunk(T, per_tilt);
    b += T * H * half * sizeof(float2) + 2 * chunk * D * H * half * sizeof(float2) +
         sign_table_bytes((int)D, (int)H, (int)W) + (D > 1 ? T * sizeof(int2) : 0);
  }
  const int staging = effective_staging(d);
  if (staging == GNC_STAGE_F16T)
    b += (D * T * H * W + 64) * 2 + T + T * kTiltPartsMax * sizeof(float);
  else
    b += (Y2 * D * T * W + 8) * kStagedPixelBytes;
  if (staging == GNC_STAGE_F16) b += Y2 * D * T * 2;
  const size_t in_elems = T * (d->input == GNC_INPUT_CORRECTED ? D : 1) * H * W;
  b += (in_elems + H * d->grid_height * d->grid_width) * sizeof(float);
  return b;
}

// Everything that fixes a plan's buffers and its sequence of launches; two
// requests with the same key can share one plan and one captured graph.
std::string plan_key(const gnc_fbp_desc *d) {
  float dscale, doffset;
  const float mn = d->num_defocus > 1 ? d->min_defocus : 0.f;
  const float mx = d->num_defocus > 1 ? d->max_defocus : 0.f;
  defocus_scale(d->num_defocus, d->pixel_size, mn, mx, &dscale, &doffset);
  bool uniform = true;
  if (d->centre)
    for (size_t y = 1; y < d->height; ++y)
      if (d->centre[y] != d->centre[0]) uniform = false;
  BpArgs a{};
  a.staging = effective_staging(d);
  a.N = (int)d->width;
  a.D = (int)d->num_defocus;
  a.dscale = dscale;
  a.uniform_centre = uniform ? 1 : 0;
  char buf[256];
  snprintf(buf, sizeof buf, "%zu,%zu,%zu,%zu,%zu,%zu,%d,%d,%d,%d,%d", d->num_angles, d->height,
           d->width, d->grid_height, d->grid_width, d->num_defocus, d->input,
           (d->input == GNC_INPUT_RAW && d->correct) ? 1 : 0, a.staging,
           backproject_fast_variant(a),
           a.staging == GNC_STAGE_F16T ? tc_rows(dscale, (int)d->num_defocus) : 0);
  return buf;
}

size_t plan_param_bytes(const gnc_fbp_plan *p) { return p->pl.bytes; }

// Points the plan at a new request of the same key: fills the parameter block
// in `host_block` (page-locked, plan_param_bytes long, not in use by an
// earlier copy) and enqueues its copy to the device on s.
int plan_set_request(gnc_fbp_plan *p, const gnc_fbp_desc *d, unsigned char *host_block,
                     cudaStream_t s) {
  bool uniform;
  std::memset(host_block, 0, p->pl.bytes);
  fill_params(p, d, host_block, &uniform, &p->dscale, &p->doffset, &p->sargs);
  GNC_REQUIRE(uniform == p->uniform_centre);
  GNC_CUDA(cudaMemcpyAsync(p->params, host_block, p->pl.bytes, cudaMemcpyHostToDevice, s));
  return GNC_OK;
}

int *plan_error_word(gnc_fbp_plan *p) { return p->err; }

}  // namespace gnc

extern "C" {
static int plan_create(const gnc_fbp_desc *d, cudaMemPool_t pool, cudaStream_t alloc,
                       gnc_fbp_plan **out);
}

namespace gnc {
int plan_create_pooled(const gnc_fbp_desc *d, cudaMemPool_t pool, cudaStream_t alloc,
                       gnc_fbp_plan **out) {
  return plan_create(d, pool, alloc, out);
}
}  // namespace gnc

// ------------------------------------------------ shared request checks ---
namespace gnc {

#define GNC_CONFIG_REQUIRE(cond)                                              \
  do {                                                                        \
    if (!(cond)) {                                                            \
      set_error(std::string(who) + ": ASSERT (" #cond ") failed");            \
      return GNC_ERR_INVALID_ARGUMENT;                                        \
    }                                                                         \
  } while (0)

int config_check(const gnc_config *c, const char *who) {
  GNC_CONFIG_REQUIRE(c != nullptr);
  if (c->device != 1) {
    set_error(std::string(who) + ": guanaco_gb300 implements the device path (device = gpu) only");
    return GNC_ERR_UNSUPPORTED;
  }
  // Config::is_valid (config.h:66-75)
  GNC_CONFIG_REQUIRE(c->num_pixels > 0);
  GNC_CONFIG_REQUIRE(c->num_angles > 0);
  GNC_CONFIG_REQUIRE(c->num_defocus > 0);
  GNC_CONFIG_REQUIRE(c->grid_height > 0);
  GNC_CONFIG_REQUIRE(c->grid_width > 0);
  GNC_CONFIG_REQUIRE(c->pixel_size > 0);
  GNC_CONFIG_REQUIRE(c->min_defocus <= c->max_defocus);
  GNC_CONFIG_REQUIRE(c->angles != nullptr);
  // BP::launch (reconstructor.cu:250)
  GNC_CONFIG_REQUIRE(c->num_defocus == 1 || c->max_defocus > c->min_defocus);
  if (c->num_pixels > 6400 || !fft_length_supported(2 * (long)c->num_pixels)) {
    set_error(std::string(who) +
              ": unsupported num_pixels: 2 * num_pixels must factorise into radices <= 16 "
              "and num_pixels <= 6400");
    return GNC_ERR_UNSUPPORTED;
  }
  return GNC_OK;
}

#undef GNC_CONFIG_REQUIRE

}  // namespace gnc

extern "C" {

const char *gnc_last_error(void) { return last_error(); }
int gnc_version(void) { return 100; }

// pool / alloc: null for cudaMalloc'd plans, else the request server's pool and
// the stream its allocations are ordered on
static int plan_create(const gnc_fbp_desc *d, cudaMemPool_t pool, cudaStream_t alloc,
                       gnc_fbp_plan **out) {
  GNC_REQUIRE(d != nullptr && out != nullptr);
  *out = nullptr;
  const int st = gnc::desc_check(d);
  if (st != GNC_OK) return st;
  const bool ctf = d->input == GNC_INPUT_RAW && d->correct;
  auto *p = new gnc_fbp_plan();
  p->pool = pool;
  p->alloc_stream = alloc;
  cudaGetDevice(&p->device);
  p->wait_probe = g_wait_probe.load();
  p->T = (int)d->num_angles;
  p->H = (int)d->height;
  p->W = (int)d->width;
  p->Z = (int)d->grid_height;
  p->X = (int)d->grid_width;
  p->D = (int)d->num_defocus;
  p->Y2 = (p->H + 1) / 2;
  p->input = d->input;
  p->correct = ctf ? 1 : 0;
  p->staging = gnc::effective_staging(d);
  p->pixel_size = d->pixel_size;
  p->min_def = d->num_defocus > 1 ? d->min_defocus : 0.f;
  p->max_def = d->num_defocus > 1 ? d->max_defocus : 0.f;

  const size_t half = (size_t)p->W / 2;
  cudaError_t e = cudaSuccess;
  p->pl = param_layout(p->T, p->H, p->D);
  e = dalloc(p, &p->params, p->pl.bytes);
  if (e == cudaSuccess) {
    p->dyn_sign = (SignTableArgs *)(p->params + p->pl.sign);
    p->dyn_bp = (float *)(p->params + p->pl.bp);
    p->geom = (TiltGeom *)(p->params + p->pl.geom);
    p->tilt_factor = (float *)(p->params + p->pl.factor);
    p->slab_df = (double *)(p->params + p->pl.slab);
    p->offset = (float *)(p->params + p->pl.offset);
    std::vector<unsigned char> blk(p->pl.bytes, 0);
    fill_params(p, d, blk.data(), &p->uniform_centre, &p->dscale, &p->doffset, &p->sargs);
    // pageable source: the call returns once the bytes are staged
    e = pool ? cudaMemcpyAsync(p->params, blk.data(), blk.size(), cudaMemcpyHostToDevice, alloc)
             : cudaMemcpy(p->params, blk.data(), blk.size(), cudaMemcpyHostToDevice);
  }
  if (ctf) {
    size_t per_tilt = (size_t)p->D * p->H * half * sizeof(float2);
    p->chunk = (int)flip_chunk(p->T, per_tilt);
    if (e == cudaSuccess) e = dalloc(p, &p->spec, (size_t)p->T * p->H * half);
    if (e == cudaSuccess) e = dalloc(p, &p->gbuf, 2 * (size_t)p->chunk * p->D * p->H * half);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->s_flip, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming);
    for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
      e = cudaEventCreateWithFlags(&p->ev_flip[b], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_rows[b], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = dalloc(p, &p->sign, sign_table_bytes(p->D, p->H, p->W));
    if (e == cudaSuccess && p->D > 1) e = dalloc(p, &p->live, (size_t)p->T);
  }
  if (p->staging == GNC_STAGE_F16T) {
    // plain FP16 rows (D, T, H, W) read by TMA tiles, and one exponent per tilt
    const size_t elems = (size_t)p->D * p->T * p->H * p->W + 64;
    if (e == cudaSuccess) e = dalloc(p, (__half **)&p->staged, elems);
    if (e == cudaSuccess) e = dalloc(p, &p->tilt_exp, (size_t)p->T);
    if (e == cudaSuccess) e = dalloc(p, &p->tilt_part, (size_t)p->T * kTiltPartsMax);
    if (e == cudaSuccess)
      e = make_tc_map(p->staged, p->D, p->T, p->H, p->W, tc_rows(p->dscale, p->D), &p->tc_map);
  } else {
    // +8 pixels: a 16-byte aligned bulk copy of the last row may run past its end
    const size_t elems = (size_t)p->Y2 * p->D * p->T * p->W + 8;
    if (e == cudaSuccess)
      e = p->staging == GNC_STAGE_F16 ? dalloc(p, (uint2 **)&p->staged, elems)
                                      : dalloc(p, (float2 **)&p->staged, elems);
    if (e == cudaSuccess && p->staging == GNC_STAGE_F16)
      e = dalloc(p, &p->row_exp, (size_t)p->Y2 * p->D * p->T * 2);
  }
  if (e == cudaSuccess) e = dalloc(p, &p->err, 1);
  if (e == cudaSuccess)
    e = pool ? cudaMemsetAsync(p->err, 0, sizeof(int), alloc) : cudaMemset(p->err, 0, sizeof(int));
  if (e != cudaSuccess) {
    set_error(std::string("gnc_fbp_plan_create: ") + cudaGetErrorString(e));
    plan_free(p);
    delete p;
    return e == cudaErrorMemoryAllocation ? GNC_ERR_OUT_OF_MEMORY : GNC_ERR_CUDA;
  }
  *out = p;
  return GNC_OK;
}

int gnc_fbp_plan_create(const gnc_fbp_desc *d, gnc_fbp_plan **out) {
  return plan_create(d, nullptr, nullptr, out);
}

int gnc_fbp_plan_destroy(gnc_fbp_plan *p) {
  if (!p) return GNC_OK;
  plan_free(p);
  delete p;
  return GNC_OK;
}

size_t gnc_fbp_workspace_bytes(const gnc_fbp_plan *p) { return p ? p->bytes : 0; }

int gnc_fbp_sign_table(gnc_fbp_plan *p, int8_t *d_out, void *stream) {
  GNC_REQUIRE(p != nullptr && p->correct);
  cudaStream_t s = (cudaStream_t)stream;
  GNC_CUDA(launch_sign_table(p->sargs, d_out ? d_out : p->sign, s));
  return GNC_OK;
}

// Phase flip and row stage of the tilts [t_begin, t_end), chunk by chunk: the
// flips run on the plan's side stream into two alternating buffers, so chunk
// c + 1 is flipped while chunk c's rows are filtered on s.  out_rows (plain
// corrected rows) or null (the row stage writes r's staged output).
static int flip_rows(gnc_fbp_plan *p, RowStageArgs r, int t_begin, int t_end, float *out_rows,
                     cudaStream_t s) {
  const size_t gsz = (size_t)p->chunk * p->D * p->H * (p->W / 2);
  // everything on s so far (spectra, sign table, earlier row stages) comes first
  GNC_CUDA(cudaEventRecord(p->ev_fork, s));
  GNC_CUDA(cudaStreamWaitEvent(p->s_flip, p->ev_fork, 0));
  int k = 0;
  for (int c0 = t_begin; c0 < t_end; c0 += p->chunk, ++k) {
    const int nt = std::min(p->chunk, t_end - c0);
    const int b = k & 1;
    float2 *g = p->gbuf + b * gsz;
    if (k >= 2) GNC_CUDA(cudaStreamWaitEvent(p->s_flip, p->ev_rows[b], 0));
    GNC_CUDA(launch_column_flip(p->spec, g, p->sign, c0, nt, p->D, p->H, p->W, r.live, p->s_flip));
    GNC_CUDA(cudaEventRecord(p->ev_flip[b], p->s_flip));
    GNC_CUDA(cudaStreamWaitEvent(s, p->ev_flip[b], 0));
    r.g = g;
    r.nt = nt;
    r.t0 = c0;
    if (out_rows) r.out_rows = out_rows + (size_t)c0 * p->D * p->H * p->W;
    GNC_CUDA(launch_row_stage(r, s));
    GNC_CUDA(cudaEventRecord(p->ev_rows[b], s));
  }
  return GNC_OK;  // s has waited for every flip: the side stream is joined
}

// F16T: the per-tilt exponents of input tilts [t0, t0 + nt) (input holds
// every tilt, (T, per_tilt) floats).
static cudaError_t tilt_exponents(gnc_fbp_plan *p, const float *input, int t0, int nt,
                                  cudaStream_t s) {
  if (p->staging != GNC_STAGE_F16T) return cudaSuccess;
  const size_t per_tilt = (size_t)(p->input == GNC_INPUT_CORRECTED ? p->D : 1) * p->H * p->W;
  // the unnormalised correction multiplies the L2 norm by at most H W
  const double gain = p->correct ? (double)p->H * p->W : 1.0;
  return launch_tilt_exponents(input, per_tilt, t0, nt, p->tilt_factor, gain, p->tilt_part,
                               p->tilt_exp, s);
}

// The staged-output arguments of the row stage.
static RowStageArgs stage_args(const gnc_fbp_plan *p) {
  RowStageArgs r{};
  r.D = p->D;
  r.H = p->H;
  r.N = p->W;
  r.T = p->T;
  r.ramp = 1;
  r.tilt_factor = p->tilt_factor;
  r.out_staged = 1;
  r.staging = p->staging;
  r.staged = p->staged;
  r.row_exp = p->row_exp;
  r.tilt_exp = p->tilt_exp;
  return r;
}

// The fast backprojector of the plan's staging (tensor cores for F16T), or
// the exact kernel for rows with different centres or when asked for.
static cudaError_t backproject(const gnc_fbp_plan *p, const BpArgs &a, bool exact,
                               cudaStream_t s, const TcMap *map = nullptr) {
  if (exact || !p->uniform_centre) return launch_backproject_exact(a, s);
  if (a.staging == GNC_STAGE_F16T) return launch_backproject_tc(a, map ? *map : p->tc_map, s);
  return launch_backproject_fast(a, s);
}

// Raw or corrected input -> staged filtered rows (the plan's staging buffer).
int gnc_fbp_stage(gnc_fbp_plan *p, const float *d_input, void *stream) {
  GNC_REQUIRE(p != nullptr && d_input != nullptr);
  cudaStream_t s = (cudaStream_t)stream;
  RowStageArgs r = stage_args(p);
  GNC_CUDA(tilt_exponents(p, d_input, 0, p->T, s));
  if (p->correct) {
    GNC_CUDA(launch_sign_table(p->sargs, p->sign, s));
    GNC_CUDA(launch_sign_pack(p->sign, p->D, p->H, p->W, s));
    if (p->live) GNC_CUDA(launch_live_slabs(bp_args(p, nullptr), p->live, s));
    GNC_CUDA(launch_rfft_rows(d_input, p->spec, p->T, p->H, p->W, s));
    GNC_CUDA(launch_column_fft(p->spec, p->T, p->H, p->W, s));
    r.input_spectra = 1;
    r.live = p->live;  // only the (tilt, slab) pairs some voxel reads
    const int st = flip_rows(p, r, 0, p->T, nullptr, s);
    if (st != GNC_OK) return st;
  } else {
    r.input_spectra = 0;
    r.rows = d_input;
    r.row_stride = p->W;
    r.plane_stride = (long)p->H * p->W;
    r.nt = p->T;
    r.t0 = 0;
    GNC_CUDA(launch_row_stage(r, s));
  }
  return GNC_OK;
}

int gnc_fbp_backproject(gnc_fbp_plan *p, float *d_volume, int exact, void *stream) {
  GNC_REQUIRE(p != nullptr && d_volume != nullptr);
  cudaStream_t s = (cudaStream_t)stream;
  GNC_CUDA(backproject(p, bp_args(p, d_volume), exact != 0, s));
  return GNC_OK;
}

int gnc_fbp_backproject_staged(gnc_fbp_plan *p, const void *d_staged, const int8_t *d_row_exp,
                               float *d_volume, int exact, void *stream) {
  GNC_REQUIRE(p != nullptr && d_staged != nullptr && d_volume != nullptr);
  GNC_REQUIRE(p->staging == GNC_STAGE_F32 || d_row_exp != nullptr);
  cudaStream_t s = (cudaStream_t)stream;
  BpArgs a = bp_args(p, d_volume);
  a.staged = d_staged;
  a.row_exp = d_row_exp;
  if (p->staging == GNC_STAGE_F16T) {  // F16T: the exponents are per tilt
    a.row_exp = nullptr;
    a.tilt_exp = d_row_exp;
    TcMap map;
    GNC_CUDA(make_tc_map(d_staged, p->D, p->T, p->H, p->W, p->tc_map.rows, &map));
    GNC_CUDA(backproject(p, a, exact != 0, s, &map));
    return GNC_OK;
  }
  GNC_CUDA(backproject(p, a, exact != 0, s));
  return GNC_OK;
}

int gnc_fbp_execute(gnc_fbp_plan *p, const float *d_input, float *d_volume, void *stream) {
  int st = gnc_fbp_stage(p, d_input, stream);
  if (st != GNC_OK) return st;
  return gnc_fbp_backproject(p, d_volume, 0, stream);
}

// Host buffers in and out, with the copies overlapped with the kernels: the
// input goes up in tilt groups, each group's transforms start as soon as it
// has arrived; the backprojection runs in row slabs and each finished slab
// goes down while the next one is computed.  Device buffers, streams and
// events are created on the first call and kept with the plan.
static cudaError_t io_setup(gnc_fbp_plan *p, size_t in_elems, size_t out_elems) {
  cudaError_t e = cudaSuccess;
  if (!p->io_in) e = cudaMalloc((void **)&p->io_in, in_elems * sizeof(float));
  if (e == cudaSuccess && !p->io_out) e = cudaMalloc((void **)&p->io_out, out_elems * sizeof(float));
  if (e == cudaSuccess && !p->s_in) e = cudaStreamCreateWithFlags(&p->s_in, cudaStreamNonBlocking);
  if (e == cudaSuccess && !p->s_out) e = cudaStreamCreateWithFlags(&p->s_out, cudaStreamNonBlocking);
  for (int i = 0; e == cudaSuccess && i < kIoEvents; ++i)
    if (!p->ev[i]) e = cudaEventCreateWithFlags(&p->ev[i], cudaEventDisableTiming);
  return e;
}

// Host-buffer execution.  The input goes up in tilt groups on s_in and each
// group's transforms start on arrival; the volume comes down in row slabs on
// s_out while the next slab is computed.  With CTF correction and room for the
// whole flipped stack, the phase flips of every tilt run first and the ramp
// filter then runs slab by slab just ahead of that slab's backprojection, so
// the first slab's copy-out starts after one slab of filtering instead of
// after all of it.  Otherwise every tilt is filtered before the first slab.
static int execute_host_pipelined(gnc_fbp_plan *p, const float *h_input, float *h_volume,
                                  cudaStream_t s) {
  const size_t per_tilt = (size_t)(p->input == GNC_INPUT_CORRECTED ? p->D : 1) * p->H * p->W;
  const size_t plane = (size_t)p->Z * p->X;
  const size_t half = p->W / 2;
  cudaEvent_t *ev_in = p->ev, *ev_bp = p->ev + kIoGroups;
  cudaEvent_t ev_start = p->ev[kIoEvents - 2], ev_done = p->ev[kIoEvents - 1];
  const size_t gfull_bytes = (size_t)p->T * p->D * p->H * half * sizeof(float2);
  if (p->correct && !p->gfull && !p->gfull_tried && gfull_bytes <= kSlabMajorMaxBytes) {
    p->gfull_tried = true;
    if (cudaMalloc((void **)&p->gfull, gfull_bytes) != cudaSuccess) {
      p->gfull = nullptr;
      (void)cudaGetLastError();  // not enough memory: filter every tilt first instead
    }
  }
  const bool slab_major = p->correct && p->gfull != nullptr;
  // the previous call's reads of the I/O buffers are ordered before this one
  GNC_CUDA(cudaEventRecord(ev_start, s));
  GNC_CUDA(cudaStreamWaitEvent(p->s_in, ev_start, 0));
  GNC_CUDA(cudaStreamWaitEvent(p->s_out, ev_start, 0));
  // tilt groups of at least 8 tilts and 8 MB (small series: fewer, larger copies)
  const size_t tilt_bytes = per_tilt * sizeof(float);
  const int group = std::max({8, (p->T + kIoGroups - 1) / kIoGroups,
                              (int)((((size_t)8 << 20) + tilt_bytes - 1) / tilt_bytes)});
  for (int g = 0, t0 = 0; t0 < p->T; ++g, t0 += group) {
    const int n = std::min(group, p->T - t0);
    GNC_CUDA(cudaMemcpyAsync(p->io_in + (size_t)t0 * per_tilt, h_input + (size_t)t0 * per_tilt,
                             n * per_tilt * sizeof(float), cudaMemcpyHostToDevice, p->s_in));
    GNC_CUDA(cudaEventRecord(ev_in[g], p->s_in));
  }
  RowStageArgs r = stage_args(p);
  if (p->correct) {
    GNC_CUDA(launch_sign_table(p->sargs, p->sign, s));
    GNC_CUDA(launch_sign_pack(p->sign, p->D, p->H, p->W, s));
    if (p->live) GNC_CUDA(launch_live_slabs(bp_args(p, nullptr), p->live, s));
    r.input_spectra = 1;
    r.live = p->live;  // only the (tilt, slab) pairs some voxel reads
  } else {
    r.input_spectra = 0;
    r.rows = p->io_in;
    r.row_stride = p->W;
    r.plane_stride = (long)p->H * p->W;
  }
  for (int g = 0, t0 = 0; t0 < p->T; ++g, t0 += group) {
    const int n = std::min(group, p->T - t0);
    GNC_CUDA(cudaStreamWaitEvent(s, ev_in[g], 0));
    GNC_CUDA(tilt_exponents(p, p->io_in, t0, n, s));
    if (p->correct) {
      float2 *spec = p->spec + (size_t)t0 * p->H * half;
      GNC_CUDA(launch_rfft_rows(p->io_in + (size_t)t0 * per_tilt, spec, n, p->H, p->W, s));
      GNC_CUDA(launch_column_fft(spec, n, p->H, p->W, s));
      if (slab_major) {
        GNC_CUDA(launch_column_flip(p->spec, p->gfull + (size_t)t0 * p->D * p->H * half, p->sign,
                                    t0, n, p->D, p->H, p->W, p->live, s));
      } else {
        const int st = flip_rows(p, r, t0, t0 + n, nullptr, s);
        if (st != GNC_OK) return st;
      }
    } else {
      r.nt = n;
      r.t0 = t0;
      GNC_CUDA(launch_row_stage(r, s));
    }
  }
  if (slab_major) {
    r.g = p->gfull;
    r.t0 = 0;
    r.nt = p->T;
  }
  // backprojection in slabs of whole row pairs, each copied out when done: at
  // most 8 slabs of whole block rows and at least 16 MB each, the last one split
  // into 1/2, 1/4, 1/4 when slabs are larger than that
  const size_t row_bytes = plane * sizeof(float);
  const size_t min_slab = (size_t)16 << 20;
  const int rows = std::max(((p->H + 7) / 8 + 7) / 8 * 8,
                            (int)((min_slab / row_bytes + 7) / 8 * 8));
  int slab_y0[kIoSlabs + 1], nslab = 0;
  for (int y0 = 0; y0 < p->H; y0 += rows) slab_y0[nslab++] = y0;
  if (rows >= 32 && (size_t)rows * row_bytes > min_slab) {
    const int last = slab_y0[nslab - 1], n_last = p->H - last;
    const int a = std::min(rows / 2, n_last), b = std::min(rows / 4, n_last - a);
    if (a < n_last) slab_y0[nslab++] = last + a;
    if (b > 0 && a + b < n_last) slab_y0[nslab++] = last + a + b;
  }
  slab_y0[nslab] = p->H;
  const size_t pb = kStagedPixelBytes;
  for (int j = 0; j < nslab; ++j) {
    const int y0 = slab_y0[j], ny = slab_y0[j + 1] - y0;
    if (slab_major) {  // the ramp filter of this slab's rows, every tilt and slab
      r.y2_begin = y0 / 2;
      r.y2_count = (ny + 1) / 2;
      GNC_CUDA(launch_row_stage(r, s));
    }
    BpArgs a = bp_args(p, p->io_out + (size_t)y0 * plane);
    const size_t pair0 = (size_t)(y0 / 2) * p->D * p->T;
    a.Y = ny;
    if (p->staging == GNC_STAGE_F16T) {
      a.y_begin = y0;  // F16T rows stay whole: the launch starts at stack row y0
    } else {
      a.staged = (const unsigned char *)p->staged + pair0 * p->W * pb;
      a.row_exp = p->row_exp ? p->row_exp + 2 * pair0 : nullptr;
    }
    a.offset = p->offset + (size_t)y0 * p->T;
    GNC_CUDA(backproject(p, a, false, s));
    GNC_CUDA(cudaEventRecord(ev_bp[j], s));
    GNC_CUDA(cudaStreamWaitEvent(p->s_out, ev_bp[j], 0));
    GNC_CUDA(cudaMemcpyAsync(h_volume + (size_t)y0 * plane, p->io_out + (size_t)y0 * plane,
                             ny * plane * sizeof(float), cudaMemcpyDeviceToHost, p->s_out));
  }
  GNC_CUDA(cudaEventRecord(ev_done, p->s_out));
  GNC_CUDA(cudaStreamWaitEvent(s, ev_done, 0));
  return GNC_OK;
}

int gnc_host_alloc(size_t bytes, void **ptr) {
  GNC_REQUIRE(ptr != nullptr && bytes > 0);
  *ptr = nullptr;
  GNC_CUDA(cudaHostAlloc(ptr, bytes, cudaHostAllocDefault));
  return GNC_OK;
}

int gnc_host_free(void *ptr) {
  if (ptr) GNC_CUDA(cudaFreeHost(ptr));
  return GNC_OK;
}

int gnc_fbp_execute_host(gnc_fbp_plan *p, const float *h_input, float *h_volume, void *stream) {
  GNC_REQUIRE(p != nullptr && h_input != nullptr && h_volume != nullptr);
  cudaStream_t s = (cudaStream_t)stream;
  size_t in_elems = (size_t)p->T * (p->input == GNC_INPUT_CORRECTED ? p->D : 1) * p->H * p->W;
  size_t out_elems = (size_t)p->H * p->Z * p->X;
  GNC_CUDA(io_setup(p, in_elems, out_elems));
  int st = execute_host_pipelined(p, h_input, h_volume, s);
  // whatever was queued finishes before the host buffers go back to the caller
  cudaError_t e1 = cudaStreamSynchronize(p->s_in);
  cudaError_t e2 = cudaStreamSynchronize(p->s_out);
  cudaError_t e3 = cudaStreamSynchronize(s);
  if (st != GNC_OK) return st;
  GNC_CUDA(e1);
  GNC_CUDA(e2);
  GNC_CUDA(e3);
  return GNC_OK;
}

int gnc_fbp_correct(gnc_fbp_plan *p, const float *d_proj, float *d_corrected, void *stream) {
  GNC_REQUIRE(p != nullptr && p->correct && d_proj != nullptr && d_corrected != nullptr);
  cudaStream_t s = (cudaStream_t)stream;
  GNC_CUDA(launch_sign_table(p->sargs, p->sign, s));
  GNC_CUDA(launch_sign_pack(p->sign, p->D, p->H, p->W, s));
  GNC_CUDA(launch_rfft_rows(d_proj, p->spec, p->T, p->H, p->W, s));
  GNC_CUDA(launch_column_fft(p->spec, p->T, p->H, p->W, s));
  RowStageArgs r{};
  r.input_spectra = 1;
  r.D = p->D;
  r.H = p->H;
  r.N = p->W;
  r.T = p->T;
  r.ramp = 0;
  r.out_staged = 0;
  return flip_rows(p, r, 0, p->T, d_corrected, s);
}

int gnc_fbp_slab_map(gnc_fbp_plan *p, int32_t *d_out, void *stream) {
  GNC_REQUIRE(p != nullptr && d_out != nullptr);
  BpArgs a = bp_args(p, nullptr);
  GNC_CUDA(launch_slab_map(a, d_out, (cudaStream_t)stream));
  return GNC_OK;
}

int gnc_fbp_launches(const gnc_fbp_plan *p) {
  if (!p) return 0;
  const int f16t = p->staging == GNC_STAGE_F16T ? 2 : 0;  // the per-tilt exponents
  if (!p->correct) return 2 + f16t;  // row stage, backprojection
  const int chunks = (p->T + p->chunk - 1) / p->chunk;
  // sign table (+ its packed copy, + the live slab ranges), row and column
  // transforms, per chunk flip + rows, BP
  return 3 + (sign_pack_used(p->H) ? 1 : 0) + (p->live ? 1 : 0) + f16t + 2 * chunks + 1;
}

int gnc_fbp_live_slabs(gnc_fbp_plan *p, int32_t *h_out, void *stream) {
  GNC_REQUIRE(p != nullptr && h_out != nullptr);
  cudaStream_t s = (cudaStream_t)stream;
  if (!p->live) {  // one slab, or no correction: every tilt reads slab 0 only
    for (int t = 0; t < p->T; ++t) h_out[2 * t] = h_out[2 * t + 1] = 0;
    return GNC_OK;
  }
  GNC_CUDA(launch_live_slabs(bp_args(p, nullptr), p->live, s));
  GNC_CUDA(cudaMemcpyAsync(h_out, p->live, (size_t)p->T * sizeof(int2), cudaMemcpyDeviceToHost, s));
  GNC_CUDA(cudaStreamSynchronize(s));
  return GNC_OK;
}

int gnc_fbp_backprojector(const gnc_fbp_plan *p) {
  if (!p) return -1;
  if (!p->uniform_centre) return 0;
  if (p->staging == GNC_STAGE_F16T) return 16;  // the tensor-core kernel
  return backproject_fast_variant(bp_args(p, nullptr));
}

int gnc_debug_wait_probe(unsigned polls) {
  g_wait_probe.store(polls);
  return GNC_OK;
}

int gnc_fbp_check(gnc_fbp_plan *p, void *stream) {
  GNC_REQUIRE(p != nullptr);
  int h = 0;
  cudaStream_t s = (cudaStream_t)stream;
  GNC_CUDA(cudaMemcpyAsync(&h, p->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  GNC_CUDA(cudaStreamSynchronize(s));
  if (h != 0) {
    GNC_CUDA(cudaMemsetAsync(p->err, 0, sizeof(int), s));
    set_error("gnc_fbp_check: a device-side wait gave up (bulk copy never completed)");
    return GNC_ERR_CUDA;
  }
  return GNC_OK;
}

int gnc_fbp_staged(gnc_fbp_plan *p, const void **d_staged, const int8_t **d_row_exp) {
  GNC_REQUIRE(p != nullptr && d_staged != nullptr);
  *d_staged = p->staged;
  if (d_row_exp) *d_row_exp = p->staging == GNC_STAGE_F16T ? p->tilt_exp : p->row_exp;
  return GNC_OK;
}

// ---------------------------------------------- reference-shaped entry points
static int select_device(int gpu_index) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    set_error("no CUDA device is available for the device path");
    return GNC_ERR_DEVICE;
  }
  if (gpu_index >= 0) GNC_CUDA(cudaSetDevice(gpu_index));
  return GNC_OK;
}

int gnc_filter_device(size_t num_pixels, size_t num_angles, size_t num_defocus, float *d_data,
                      void *stream) {
  // Filter<e_device>::Filter asserts (filter.cu:139-141)
  GNC_REQUIRE(num_pixels > 0);
  GNC_REQUIRE(num_angles > 0);
  GNC_REQUIRE(num_defocus > 0);
  GNC_REQUIRE(d_data != nullptr);
  if (num_pixels > 6400 || !fft_length_supported(2 * (long)num_pixels)) {
    set_error("unsupported num_pixels for the ramp filter");
    return GNC_ERR_UNSUPPORTED;
  }
  RowStageArgs r{};
  r.input_spectra = 0;
  r.rows = d_data;
  r.row_stride = (long)num_pixels;
  r.plane_stride = 0;
  r.nt = 1;
  r.t0 = 0;
  r.T = 1;
  r.D = 1;
  r.H = (int)(num_angles * num_defocus);
  r.N = (int)num_pixels;
  r.ramp = 1;
  r.out_staged = 0;
  r.out_rows = d_data;
  GNC_CUDA(launch_row_stage(r, (cudaStream_t)stream));
  return GNC_OK;
}

int gnc_reconstruct_device(const gnc_config *c, const float *d_sino, float *d_rec, void *stream) {
  int st = config_check(c, "gnc_reconstruct_device");
  if (st != GNC_OK) return st;
  GNC_REQUIRE(d_sino != nullptr && d_rec != nullptr);
  cudaStream_t s = (cudaStream_t)stream;
  const size_t sino = c->num_pixels * c->num_angles * c->num_defocus;
  std::vector<TiltGeom> geom(c->num_angles);
  float offset = 0.f;
  for (size_t t = 0; t < c->num_angles; ++t)
    geom[t] = tilt_geometry(c->angles[t], c->centre, c->num_angles, &offset);
  float dscale, doffset;
  defocus_scale(c->num_defocus, c->pixel_size, c->min_defocus, c->max_defocus, &dscale, &doffset);
  float *filtered = nullptr;
  TiltGeom *dgeom = nullptr;
  GNC_CUDA(cudaMallocAsync((void **)&filtered, sino * sizeof(float), s));
  cudaError_t e = cudaMallocAsync((void **)&dgeom, geom.size() * sizeof(TiltGeom), s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dgeom, geom.data(), geom.size() * sizeof(TiltGeom),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(filtered, d_sino, sino * sizeof(float), cudaMemcpyDeviceToDevice, s);
  int rc = GNC_OK;
  if (e == cudaSuccess)
    rc = gnc_filter_device(c->num_pixels, c->num_angles, c->num_defocus, filtered, stream);
  if (e == cudaSuccess && rc == GNC_OK) {
    SliceBpArgs a{};
    a.sino = filtered;
    a.D = (int)c->num_defocus;
    a.T = (int)c->num_angles;
    a.N = (int)c->num_pixels;
    a.Z = (int)c->grid_height;
    a.X = (int)c->grid_width;
    a.geom = dgeom;
    a.offset = offset;
    a.dscale = dscale;
    a.doffset = doffset;
    a.rec = d_rec;
    e = launch_backproject_slice(a, s);
  }
  cudaFreeAsync(filtered, s);
  cudaFreeAsync(dgeom, s);
  if (rc != GNC_OK) return rc;
  GNC_CUDA(e);
  return GNC_OK;
}

int gnc_reconstruct(const gnc_config *c, const float *sinogram, float *reconstruction) {
  int st = config_check(c, "gnc_reconstruct");
  if (st != GNC_OK) return st;
  GNC_REQUIRE(sinogram != nullptr && reconstruction != nullptr);
  st = select_device(c->gpu_index);
  if (st != GNC_OK) return st;
  const size_t sino = c->num_pixels * c->num_angles * c->num_defocus;
  const size_t grid = c->grid_height * c->grid_width;
  cudaStream_t s = nullptr;
  float *ds = nullptr, *dr = nullptr;
  GNC_CUDA(cudaMallocAsync((void **)&ds, sino * sizeof(float), s));
  cudaError_t e = cudaMallocAsync((void **)&dr, grid * sizeof(float), s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ds, sinogram, sino * sizeof(float), cudaMemcpyHostToDevice, s);
  int rc = GNC_OK;
  if (e == cudaSuccess) rc = gnc_reconstruct_device(c, ds, dr, s);
  if (e == cudaSuccess && rc == GNC_OK)
    e = cudaMemcpyAsync(reconstruction, dr, grid * sizeof(float), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(ds, s);
  cudaFreeAsync(dr, s);
  cudaError_t e2 = cudaStreamSynchronize(s);
  if (rc != GNC_OK) return rc;
  GNC_CUDA(e);
  GNC_CUDA(e2);
  return GNC_OK;
}

// Phase-flip table straight from a complex64 CTF stack: s = -sign(imag),
// stored symmetrised as s(k) + s(-k) for kx <= W/2 (correct.h:30-39).
__global__ void k_sign_from_ctf(const float2 *__restrict__ ctf, int D, int H, int W,
                                int8_t *__restrict__ out) {
  const int half = W / 2, sw = half + 1;
  const long total = (long)D * H * sw;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total;
       i += (long)gridDim.x * blockDim.x) {
    int kx = (int)(i % sw);
    long r = i / sw;
    int ky = (int)(r % H);
    int d = (int)(r / H);
    const float2 *c = ctf + (size_t)d * H * W;
    float a = c[(size_t)ky * W + kx].y;
    float b = c[(size_t)((H - ky) % H) * W + (W - kx) % W].y;
    int sa = -((0.0f < a) - (a < 0.0f));
    int sb = -((0.0f < b) - (b < 0.0f));
    out[i] = (int8_t)(sa + sb);
  }
}

int gnc_correct(const float *image, const float *ctf, float *rec, size_t xsize, size_t ysize,
                size_t num_ctf) {
  // Corrector::correct asserts (correct.cu:38-40)
  GNC_REQUIRE(xsize > 0);
  GNC_REQUIRE(ysize > 0);
  GNC_REQUIRE(num_ctf > 0);
  GNC_REQUIRE(image != nullptr && ctf != nullptr && rec != nullptr);
  if (xsize % 2 != 0 || ysize > 8192 || xsize > 16384 || !fft_length_supported((long)xsize) ||
      !fft_length_supported((long)ysize)) {
    set_error("gnc_correct: unsupported image size (even width; width and height must "
              "factorise into radices <= 16; height <= 8192)");
    return GNC_ERR_UNSUPPORTED;
  }
  int st = select_device(-1);
  if (st != GNC_OK) return st;
  const int W = (int)xsize, H = (int)ysize, D = (int)num_ctf;
  const size_t img = xsize * ysize, half = xsize / 2;
  cudaStream_t s = nullptr;
  float *dimg = nullptr, *drec = nullptr;
  float2 *dctf = nullptr, *spec = nullptr, *g = nullptr;
  int8_t *sign = nullptr;
  auto release = [&]() {
    cudaFreeAsync(dimg, s);
    cudaFreeAsync(drec, s);
    cudaFreeAsync(dctf, s);
    cudaFreeAsync(spec, s);
    cudaFreeAsync(g, s);
    cudaFreeAsync(sign, s);
  };
  cudaError_t e = cudaMallocAsync((void **)&dimg, img * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&drec, D * img * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&dctf, D * img * sizeof(float2), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&spec, H * half * sizeof(float2), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&g, D * H * half * sizeof(float2), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&sign, sign_table_bytes(D, H, W), s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dimg, image, img * sizeof(float), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dctf, ctf, D * img * sizeof(float2), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    k_sign_from_ctf<<<std::min<long>(4096, ((long)D * H * (half + 1) + 255) / 256), 256, 0, s>>>(
        dctf, D, H, W, sign);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = launch_sign_pack(sign, D, H, W, s);
  if (e == cudaSuccess) e = launch_rfft_rows(dimg, spec, 1, H, W, s);
  if (e == cudaSuccess) e = launch_column_fft(spec, 1, H, W, s);
  if (e == cudaSuccess) e = launch_column_flip(spec, g, sign, 0, 1, D, H, W, nullptr, s);
  if (e == cudaSuccess) {
    RowStageArgs r{};
    r.input_spectra = 1;
    r.g = g;
    r.nt = 1;
    r.t0 = 0;
    r.T = 1;
    r.D = D;
    r.H = H;
    r.N = W;
    r.ramp = 0;
    r.out_staged = 0;
    r.out_rows = drec;
    e = launch_row_stage(r, s);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(rec, drec, D * img * sizeof(float), cudaMemcpyDeviceToHost, s);
  release();
  cudaError_t e2 = cudaStreamSynchronize(s);
  GNC_CUDA(e);
  GNC_CUDA(e2);
  return GNC_OK;
}

}  // extern "C"
