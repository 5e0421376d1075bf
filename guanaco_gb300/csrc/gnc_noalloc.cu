// Allocation-free variant of the single-slice device reconstruction.
//
// gnc_reconstruct_device filters the caller's sinogram into a temporary
// device buffer and backprojects from it; that temporary comes from
// cudaMallocAsync.  Some callers cannot allow any device allocation inside a
// call: an application that hands this library a fixed device-memory budget
// and owns every allocation itself, a real-time acquisition loop that must not
// touch the allocator (an allocation can block on the device or fail under
// memory pressure at an arbitrary time).  For them this file keeps the
// scratch in statically sized device arrays declared at file scope: every GPU
// that loads the library holds them (about 16.1 MiB) until the process exits,
// and a call uses them instead of allocating.
//
// Consequences for callers:
//  * limits: num_defocus * num_angles * num_pixels <= 4 Mi floats,
//    num_angles <= 1024, num_pixels <= 4096 (the zero-padded row length
//    2 * num_pixels must also factorise into radices <= 16); larger requests
//    are rejected with GNC_ERR_INVALID_ARGUMENT and a message naming the limit;
//  * all calls on one device share the arrays, which keep the last call's
//    contents: calls that may overlap on the GPU (different streams, or host
//    threads racing) race on them and must be serialised by the caller;
//  * the first call on a device looks up the arrays' device addresses
//    (cudaGetSymbolAddress with that device current) and keeps them.
#include <math.h>

#include <mutex>

#include "../../include/guanaco_gb300.h"
#include "gnc_common.cuh"

namespace gnc {
namespace {

constexpr size_t kMaxSino = (size_t)4 << 20;  // floats: D * T * N
constexpr int kMaxTilts = 1024;
constexpr int kMaxPixels = 4096;
constexpr int kMaxFft = 2 * kMaxPixels;       // zero-padded row length

// The scratch.  In host code these names are host-side stand-ins, not device
// addresses: host code must use the addresses looked up per device below.
static __device__ __align__(256) float g_sino[kMaxSino];       // filtered rows
static __device__ __align__(256) TiltGeom g_geom[kMaxTilts];   // per-tilt geometry
static __device__ __align__(256) float2 g_roots[kMaxFft];      // FFT twiddles

struct DeviceScratch {
  float *sino = nullptr;
  TiltGeom *geom = nullptr;
  float2 *roots = nullptr;
  bool ready = false;
};
constexpr int kMaxDevices = 64;
static DeviceScratch g_scratch[kMaxDevices];
static std::mutex g_scratch_lock;

// Device addresses of the scratch arrays on the current device (first call
// per device looks them up).
static int scratch_for_current_device(DeviceScratch *out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error(std::string("gnc_reconstruct_device_noalloc: cudaGetDevice: ") +
              cudaGetErrorString(e));
    return GNC_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("gnc_reconstruct_device_noalloc: device index beyond 64");
    return GNC_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(g_scratch_lock);
  DeviceScratch &s = g_scratch[dev];
  if (!s.ready) {
    void *p = nullptr;
    if ((e = cudaGetSymbolAddress(&p, g_sino)) != cudaSuccess) goto fail;
    s.sino = (float *)p;
    if ((e = cudaGetSymbolAddress(&p, g_geom)) != cudaSuccess) goto fail;
    s.geom = (TiltGeom *)p;
    if ((e = cudaGetSymbolAddress(&p, g_roots)) != cudaSuccess) goto fail;
    s.roots = (float2 *)p;
    s.ready = true;
  }
  *out = s;
  return GNC_OK;
fail:
  set_error(std::string("gnc_reconstruct_device_noalloc: cudaGetSymbolAddress: ") +
            cudaGetErrorString(e));
  return GNC_ERR_CUDA;
}

static bool factor_radices(int n, FftPlan *p) {
  int ns = 0;
  while (n % 8 == 0) { p->radix[ns++] = 8; n /= 8; }
  while (n % 4 == 0) { p->radix[ns++] = 4; n /= 4; }
  while (n % 2 == 0) { p->radix[ns++] = 2; n /= 2; }
  for (int f = 3; n > 1; f += 2) {
    while (n % f == 0) {
      if (f > kMaxRadix || ns >= kMaxStages) return false;
      p->radix[ns++] = f;
      n /= f;
    }
  }
  p->nstage = ns;
  return true;
}

// exp(-2 pi i k / L) in double, rounded to float.
__global__ void k_fill_roots(float2 *roots, int L) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < L) {
    double s, c;
    sincospi(2.0 * (double)k / (double)L, &s, &c);
    roots[k] = make_float2((float)c, (float)-s);
  }
}

// Ramp filter of `nrows` rows of N pixels in place (src/libguanaco/filter.cpp:
// 30-97): two rows per complex row, zero padded to 2N, transformed, multiplied
// by w_k = k / N (mirrored above N), transformed back, first N samples / 2N.
__global__ void k_noalloc_ramp(float *rows, int nrows, int N, FftPlan plan, int rp) {
  extern __shared__ float2 smem_na[];
  const int L = 2 * N;
  const int npair = (nrows + 1) / 2;
  const int p0 = blockIdx.x * rp;
  const int np = min(rp, npair - p0);
  float2 *bufa = smem_na, *bufb = smem_na + rp * L;
  for (int i = threadIdx.x; i < rp * L; i += blockDim.x) {
    const int s = i / L, k = i - s * L;
    float2 z = make_float2(0.f, 0.f);
    if (s < np && k < N) {
      const int ra = 2 * (p0 + s), rb = ra + 1;
      z.x = rows[(size_t)ra * N + k];
      z.y = rb < nrows ? rows[(size_t)rb * N + k] : 0.f;
    }
    bufa[i] = z;
  }
  __syncthreads();
  float2 *f = fft_batch<false, false>(bufa, bufb, plan, 1, rp, L);
  for (int i = threadIdx.x; i < rp * L; i += blockDim.x) {
    const int k = i % L;
    const int kk = k <= N ? k : L - k;
    const float w = (float)kk / (float)N;
    f[i] = make_float2(f[i].x * w, f[i].y * w);
  }
  __syncthreads();
  float2 *o = f == bufa ? bufb : bufa;
  float2 *y = fft_batch<true, false>(f, o, plan, 1, rp, L);
  for (int i = threadIdx.x; i < np * N; i += blockDim.x) {
    const int s = i / N, k = i - s * N;
    const int ra = 2 * (p0 + s), rb = ra + 1;
    const float2 v = y[s * L + k];
    rows[(size_t)ra * N + k] = v.x / (float)L;
    if (rb < nrows) rows[(size_t)rb * N + k] = v.y / (float)L;
  }
}

}  // namespace
}  // namespace gnc

using namespace gnc;

extern "C" int gnc_reconstruct_device_noalloc(const gnc_config *c, const float *d_sino,
                                              float *d_rec, void *stream) {
  if (!c || !d_sino || !d_rec) {
    set_error("gnc_reconstruct_device_noalloc: null config or buffer");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  if (c->device != 1) {
    set_error("gnc_reconstruct_device_noalloc: the device path (device = gpu) only");
    return GNC_ERR_UNSUPPORTED;
  }
  // guanaco::Config::is_valid (config.h:66-75) and BP::launch (reconstructor.cu:250)
  if (!(c->num_pixels > 0 && c->num_angles > 0 && c->num_defocus > 0 && c->grid_height > 0 &&
        c->grid_width > 0 && c->pixel_size > 0 && c->min_defocus <= c->max_defocus &&
        c->angles != nullptr && (c->num_defocus == 1 || c->max_defocus > c->min_defocus))) {
    set_error("gnc_reconstruct_device_noalloc: invalid configuration (guanaco::Config::is_valid)");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  const size_t sino = c->num_pixels * c->num_angles * c->num_defocus;
  if (sino > kMaxSino || c->num_angles > (size_t)kMaxTilts ||
      c->num_pixels > (size_t)kMaxPixels) {
    set_error("gnc_reconstruct_device_noalloc: request exceeds the static scratch "
              "(num_defocus * num_angles * num_pixels <= 4194304, num_angles <= 1024, "
              "num_pixels <= 4096)");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  const int N = (int)c->num_pixels, L = 2 * N;
  FftPlan plan{};
  plan.n = L;
  if (!factor_radices(L, &plan)) {
    set_error("gnc_reconstruct_device_noalloc: 2 * num_pixels must factorise into radices <= 16");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  DeviceScratch s;
  int st = scratch_for_current_device(&s);
  if (st != GNC_OK) return st;
  plan.roots = s.roots;
  cudaStream_t strm = (cudaStream_t)stream;

  // per-tilt geometry with the reference's float arithmetic (reconstructor.cpp:35-47)
  TiltGeom geom[kMaxTilts];
  float offset = 0.f;
  const double output_scale = M_PI / (double)(2 * c->num_angles);
  for (size_t t = 0; t < c->num_angles; ++t) {
    const float theta = c->angles[t];
    const float ca = cosf(theta), sa = sinf(theta);
    const float det_x0 = -c->centre * ca, det_y0 = -c->centre * sa;
    const float ray = sqrtf(ca * ca + sa * sa);
    const float d = ca * ca + sa * sa;
    offset = (det_y0 * (-sa) - det_x0 * ca) / d;
    geom[t].scale = (float)(output_scale * ray / fabsf(d));
    geom[t].cos_a = ca / d;
    geom[t].sin_a = sa / d;
    geom[t].pad = 0.f;
  }
  const float dscale = c->num_defocus > 1
                           ? (float)c->num_defocus * c->pixel_size / (c->max_defocus - c->min_defocus)
                           : 0.0f;
  const float doffset = -dscale * (c->min_defocus / c->pixel_size);

  cudaError_t e = cudaMemcpyAsync(s.geom, geom, c->num_angles * sizeof(TiltGeom),
                                  cudaMemcpyHostToDevice, strm);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s.sino, d_sino, sino * sizeof(float), cudaMemcpyDeviceToDevice, strm);
  if (e == cudaSuccess) {
    k_fill_roots<<<(L + 255) / 256, 256, 0, strm>>>(s.roots, L);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    int rp = L >= 4096 ? 1 : 4096 / L;
    if (rp > 8) rp = 8;
    const int nrows = (int)(c->num_angles * c->num_defocus);
    const int npair = (nrows + 1) / 2;
    if (rp > npair) rp = npair;
    const size_t smem = 2ull * rp * L * sizeof(float2);
    e = ensure_dynamic_smem<k_noalloc_ramp>(200 * 1024);
    if (e == cudaSuccess) {
      k_noalloc_ramp<<<(npair + rp - 1) / rp, 256, smem, strm>>>(s.sino, nrows, N, plan, rp);
      e = cudaGetLastError();
    }
  }
  if (e == cudaSuccess) {
    SliceBpArgs a{};
    a.sino = s.sino;
    a.D = (int)c->num_defocus;
    a.T = (int)c->num_angles;
    a.N = N;
    a.Z = (int)c->grid_height;
    a.X = (int)c->grid_width;
    a.geom = s.geom;
    a.offset = offset;
    a.dscale = dscale;
    a.doffset = doffset;
    a.rec = d_rec;
    e = launch_backproject_slice(a, strm);
  }
  if (e != cudaSuccess) {
    set_error(std::string("gnc_reconstruct_device_noalloc: ") + cudaGetErrorString(e));
    return GNC_ERR_CUDA;
  }
  return GNC_OK;
}
