// CTF phase-flip correction on the GPU: row transform of the raw projections
// and the fused column transform / per-slab phase flip / inverse column
// transform.
//
// Reference: guanaco::detail::Corrector<e_device, float>::correct
// (src/libguanaco/correct.cu:30-86) -- per tilt one forward 2D transform of
// the image, then per slab a phase flip (include/guanaco/correct.h:30-39), an
// inverse 2D transform and the real part, unnormalised.
//
// Here the image is real, so the forward transform is a real-to-half-spectrum
// transform, and taking the real part of the inverse is the same as inverting
// the Hermitian half spectrum after symmetrising the flip sign:
//   Re(IFFT(F s)) = IFFT(F (s(k) + s(-k)) / 2)   for real images.
// The sign table therefore holds s(k) + s(-k) (in {-2..2}) and the per-slab
// multiply is exact in float, as it is in the reference.
#include "gnc_common.cuh"

namespace gnc {

// ---------------------------------------------------------------------------
// Row transform: two real rows per complex row.
// ---------------------------------------------------------------------------
__global__ void k_rfft_rows(const float *__restrict__ proj, float2 *__restrict__ spec, int H,
                            int W, int pairs_per_block, FftPlan plan) {
  extern __shared__ float2 smem[];
  const int t = blockIdx.y;
  const int npair = (H + 1) / 2;
  const int p0 = blockIdx.x * pairs_per_block;
  const int np = min(pairs_per_block, npair - p0);
  float2 *bufa = smem;
  float2 *bufb = smem + pairs_per_block * W;
  const float *img = proj + (size_t)t * H * W;

  for (int i = threadIdx.x; i < np * W; i += blockDim.x) {
    int s = i / W, n = i - s * W;
    int ya = 2 * (p0 + s), yb = ya + 1;
    float a = __ldg(img + (size_t)ya * W + n);
    float b = yb < H ? __ldg(img + (size_t)yb * W + n) : 0.0f;
    bufa[s * W + n] = make_float2(a, b);
  }
  for (int i = np * W + threadIdx.x; i < pairs_per_block * W; i += blockDim.x)
    bufa[i] = make_float2(0.f, 0.f);
  __syncthreads();
  float2 *z = fft_batch<false, false>(bufa, bufb, plan, 1, pairs_per_block, W);

  // unpack: A[k] = (Z[k] + conj Z[-k]) / 2, B[k] = -i (Z[k] - conj Z[-k]) / 2
  const int half = W / 2;
  float2 *out = spec + (size_t)t * H * half;
  for (int i = threadIdx.x; i < np * half; i += blockDim.x) {
    int s = i / half, k = i - s * half;
    const float2 *zs = z + s * W;
    int ya = 2 * (p0 + s), yb = ya + 1;
    float2 A, B;
    if (k == 0) {
      float2 z0 = zs[0], zn = zs[half];
      A = make_float2(z0.x, zn.x);  // (DC, Nyquist) of row a
      B = make_float2(z0.y, zn.y);  // (DC, Nyquist) of row b
    } else {
      float2 zk = zs[k], zm = zs[W - k];
      A = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
      B = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
    }
    out[(size_t)ya * half + k] = A;
    if (yb < H) out[(size_t)yb * half + k] = B;
  }
}

cudaError_t launch_rfft_rows(const float *proj, float2 *spec, int T, int H, int W,
                             cudaStream_t s) {
  if (W == 1024) return launch_rfft_rows_w1024(proj, spec, T, H, s);
  if (pow2_fast(W)) return launch_rfft_rows_p2(proj, spec, T, H, W, s);
  FftPlan plan;
  if (!make_fft_plan(W, &plan)) return cudaErrorInvalidValue;
  int ppb = W >= 4096 ? 1 : 4096 / W;
  int npair = (H + 1) / 2;
  if (ppb > npair) ppb = npair;
  size_t smem = 2ull * ppb * W * sizeof(float2);
  if (cudaError_t e_attr = ensure_dynamic_smem<k_rfft_rows>(200 * 1024)) return e_attr;
  dim3 grid((npair + ppb - 1) / ppb, T);
  k_rfft_rows<<<grid, 256, smem, s>>>(proj, spec, H, W, ppb, plan);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Column stage.  A block owns C columns of the half spectrum of one tilt
// (H x C complex in shared memory).  Column kx = 0 carries the DC column in
// its real part and the Nyquist column in its imaginary part (both real
// sequences), so its flip needs the mirrored bin:
//   P'(ky) = a(ky) P(ky) + b(ky) conj(P(-ky)),
//   a = (s_dc + s_nyq) / 2, b = (s_dc - s_nyq) / 2.
// ---------------------------------------------------------------------------
static int column_tile(int H) {
  // two H x C buffers within ~128 KB
  int C = (128 * 1024) / (2 * H * (int)sizeof(float2));
  if (C > 16) C = 16;
  if (C < 1) C = 1;
  return C;
}

// Forward column transform of every tilt's half spectrum, in place.
__global__ void k_column_fft(float2 *__restrict__ spec, int H, int W, int C, FftPlan plan) {
  extern __shared__ float2 smem[];
  const int half = W / 2;
  const int t = blockIdx.y;
  const int c0 = blockIdx.x * C;
  float2 *b0 = smem, *b1 = smem + H * C;
  float2 *col = spec + (size_t)t * H * half;
  for (int i = threadIdx.x; i < H * C; i += blockDim.x) {
    int ky = i / C, c = i - ky * C;
    int kx = c0 + c;
    b0[i] = kx < half ? col[(size_t)ky * half + kx] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  float2 *F = fft_batch<false, true>(b0, b1, plan, C, C, 1);
  for (int i = threadIdx.x; i < H * C; i += blockDim.x) {
    int ky = i / C, c = i - ky * C;
    int kx = c0 + c;
    if (kx < half) col[(size_t)ky * half + kx] = F[i];
  }
}

cudaError_t launch_column_fft(float2 *spec, int T, int H, int W, cudaStream_t s) {
  if (H == 1024) return launch_column_fft_w1024(spec, T, W, s);
  if (H == 4096) return launch_column_fft_b4096(spec, T, W, s);
  if (H == 128 || H == 256 || H == 384 || H == 512) return launch_column_fft_w512(spec, T, H, W, s);
  if (pow2_fast(H)) return launch_column_fft_p2(spec, T, H, W, s);
  FftPlan plan;
  if (!make_fft_plan(H, &plan)) return cudaErrorInvalidValue;
  const int half = W / 2;
  int C = column_tile(H);
  if (C > half) C = half;
  size_t smem = 2ull * H * C * sizeof(float2);
  if (cudaError_t e_attr = ensure_dynamic_smem<k_column_fft>(200 * 1024)) return e_attr;
  dim3 grid((half + C - 1) / C, T);
  k_column_fft<<<grid, 256, smem, s>>>(spec, H, W, C, plan);
  return cudaGetLastError();
}

// Per-slab phase flip and inverse column transform: one block per
// (column tile, slab, tilt of the chunk).
__global__ void k_column_flip(const float2 *__restrict__ spec, float2 *__restrict__ g,
                              const int8_t *__restrict__ sign, int t0, int D, int H, int W, int C,
                              FftPlan plan, const int2 *__restrict__ live) {
  extern __shared__ float2 smem[];
  const int half = W / 2;
  const int d = blockIdx.y;
  const int tl = blockIdx.z;
  const int t = t0 + tl;
  if (!slab_live(live, t, d)) return;  // no voxel reads this (tilt, slab)
  const int c0 = blockIdx.x * C;
  float2 *b0 = smem, *b1 = smem + H * C;
  const float2 *F = spec + (size_t)t * H * half;
  const int sw = half + 1;  // sign table row length
  const int8_t *sg = sign + (size_t)d * H * sw;
  for (int i = threadIdx.x; i < H * C; i += blockDim.x) {
    int ky = i / C, c = i - ky * C;
    int kx = c0 + c;
    float2 r = make_float2(0.f, 0.f);
    if (kx == 0) {
      float2 v = F[(size_t)ky * half];
      float2 m = F[(size_t)((H - ky) % H) * half];
      float sdc = 0.5f * (float)sg[(size_t)ky * sw];
      float sny = 0.5f * (float)sg[(size_t)ky * sw + half];
      float a = 0.5f * (sdc + sny), b = 0.5f * (sdc - sny);
      r = make_float2(a * v.x + b * m.x, a * v.y - b * m.y);
    } else if (kx < half) {
      float2 v = F[(size_t)ky * half + kx];
      float f = 0.5f * (float)sg[(size_t)ky * sw + kx];
      r = make_float2(f * v.x, f * v.y);
    }
    b0[i] = r;
  }
  __syncthreads();
  float2 *R = fft_batch<true, true>(b0, b1, plan, C, C, 1);
  float2 *dst = g + ((size_t)tl * D + d) * H * half;
  for (int i = threadIdx.x; i < H * C; i += blockDim.x) {
    int ky = i / C, c = i - ky * C;
    int kx = c0 + c;
    if (kx < half) dst[(size_t)ky * half + kx] = R[i];
  }
}

cudaError_t launch_column_flip(const float2 *spec, float2 *g, const int8_t *sign, int t0, int nt,
                               int D, int H, int W, const int2 *live, cudaStream_t s) {
  if (H == 1024) return launch_column_flip_w1024(spec, g, sign, t0, nt, D, W, live, s);
  if (H == 4096) return launch_column_flip_b4096(spec, g, sign, t0, nt, D, W, live, s);
  if (H == 128 || H == 256 || H == 384 || H == 512)
    return launch_column_flip_w512(spec, g, sign, t0, nt, D, H, W, live, s);
  if (pow2_fast(H)) return launch_column_flip_p2(spec, g, sign, t0, nt, D, H, W, live, s);
  FftPlan plan;
  if (!make_fft_plan(H, &plan)) return cudaErrorInvalidValue;
  const int half = W / 2;
  int C = column_tile(H);
  if (C > half) C = half;
  size_t smem = 2ull * H * C * sizeof(float2);
  if (cudaError_t e_attr = ensure_dynamic_smem<k_column_flip>(200 * 1024)) return e_attr;
  dim3 grid((half + C - 1) / C, D, nt);
  k_column_flip<<<grid, 256, smem, s>>>(spec, g, sign, t0, D, H, W, C, plan, live);
  return cudaGetLastError();
}

}  // namespace gnc
