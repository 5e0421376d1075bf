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
//    num_angles <= 1024, num_pixels <= 4096; larger requests are rejected
//    with GNC_ERR_INVALID_ARGUMENT and a message naming the limit.  Requests
//    the allocating entry point would reject are rejected here with the same
//    status (the same checks, gnc_host_geom.h);
//  * all calls on one device share the arrays, which keep the last call's
//    contents: calls that may overlap on the GPU (different streams, or host
//    threads racing) race on them and must be serialised by the caller;
//  * every call looks up the arrays' device addresses on the current device
//    (cudaGetSymbolAddress, which allocates nothing), so a context torn down
//    and rebuilt (cudaDeviceReset) cannot leave it stale pointers.  The first
//    call on a device is its set-up: that lookup loads this library's device
//    code there, which is when the arrays come into existence, so the first
//    call should come before any stream capture on that device.
#include <math.h>

#include "../../include/guanaco_gb300.h"
#include "gnc_common.cuh"
#include "gnc_host_geom.h"

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
};

// Device addresses of the scratch arrays on the current device, looked up on
// every call (a lookup is a table search in the runtime, not an allocation).
static int scratch_for_current_device(DeviceScratch *out) {
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_sino);
  if (e == cudaSuccess) {
    out->sino = (float *)p;
    e = cudaGetSymbolAddress(&p, g_geom);
  }
  if (e == cudaSuccess) {
    out->geom = (TiltGeom *)p;
    e = cudaGetSymbolAddress(&p, g_roots);
  }
  if (e != cudaSuccess) {
    set_error(std::string("gnc_reconstruct_device_noalloc: cudaGetSymbolAddress: ") +
              cudaGetErrorString(e));
    return GNC_ERR_CUDA;
  }
  out->roots = (float2 *)p;
  return GNC_OK;
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
  // the allocating entry point's checks first, with its statuses
  const int valid = config_check(c, "gnc_reconstruct_device_noalloc");
  if (valid != GNC_OK) return valid;
  if (!d_sino || !d_rec) {
    set_error("gnc_reconstruct_device_noalloc: ASSERT (d_sino != nullptr && d_rec != nullptr) "
              "failed");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  // then the static scratch's limits, each factor on its own so that the
  // product below cannot wrap
  if (c->num_angles > (size_t)kMaxTilts || c->num_pixels > (size_t)kMaxPixels ||
      c->num_defocus > kMaxSino / (c->num_angles * c->num_pixels)) {
    set_error("gnc_reconstruct_device_noalloc: request exceeds the static scratch "
              "(num_defocus * num_angles * num_pixels <= 4194304, num_angles <= 1024, "
              "num_pixels <= 4096)");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  const size_t sino = c->num_pixels * c->num_angles * c->num_defocus;
  const int N = (int)c->num_pixels, L = 2 * N;
  FftPlan plan{};
  if (!make_fft_factors(L, &plan)) {  // config_check has accepted this length
    set_error("gnc_reconstruct_device_noalloc: 2 * num_pixels does not factorise");
    return GNC_ERR_UNSUPPORTED;
  }
  DeviceScratch s;
  int st = scratch_for_current_device(&s);
  if (st != GNC_OK) return st;
  plan.roots = s.roots;
  cudaStream_t strm = (cudaStream_t)stream;

  // per-tilt geometry with the reference's float arithmetic (reconstructor.cpp:35-47)
  TiltGeom geom[kMaxTilts];
  float offset = 0.f;
  for (size_t t = 0; t < c->num_angles; ++t)
    geom[t] = tilt_geometry(c->angles[t], c->centre, c->num_angles, &offset);
  float dscale, doffset;
  defocus_scale(c->num_defocus, c->pixel_size, c->min_defocus, c->max_defocus, &dscale, &doffset);

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
    // set on every call: the attribute belongs to the current context
    e = cudaFuncSetAttribute(k_noalloc_ramp, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             200 * 1024);
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
