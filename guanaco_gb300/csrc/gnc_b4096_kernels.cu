// Correction and ramp-filter kernels for 4096-pixel columns and rows, built on
// the register-resident block transform of gnc_fft_block4096.cuh.  They
// compute what the power-of-two kernels of gnc_pow2_kernels.cu compute (same
// phase flip of the packed half spectra, same four-transform form of the
// zero-padded ramp filter, see there), with each transform's data in
// registers: the column kernels load straight into the transform's layout and
// store straight from it, and the row stage chains its four transforms and the
// pointwise products in registers, holding the second path's data in
// registers too.
#include "gnc_common.cuh"
#include "gnc_fft_block4096.cuh"

namespace gnc {

namespace {

constexpr int kN = 4096;

__device__ __forceinline__ float ramp_w4096(int K) {  // filter.cpp:38-41, w_K = K / N
  const int kk = K <= kN ? K : 2 * kN - K;
  return (float)kk / (float)kN;
}

struct BlockSync {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};

__device__ __forceinline__ float2 scale2(float w, float2 v) { return make_float2(w * v.x, w * v.y); }

// Columns per block of the column kernels: four columns make every row piece a
// block reads or writes 32 contiguous bytes (one sector).
constexpr int kColC = 4;

}  // namespace

// ---------------------------------------------------------------------------
// Column transforms of 4096 rows: thread (c, l) = (tid mod C, tid / C) holds
// rows l + 256 m of column c.  FLIP: per-slab phase flip then the inverse
// transform (the packed DC / Nyquist column as in gnc_correct.cu).
// ---------------------------------------------------------------------------
template <bool FLIP, int C>
__global__ void __launch_bounds__(256 * C, 4 / C) k_column_b4096(const float2 *__restrict__ src,
                                                             float2 *__restrict__ dst,
                                                             const unsigned long long *__restrict__ sign,
                                                             int t0, int D, int W,
                                                             const float2 *__restrict__ roots,
                                                             const int2 *__restrict__ live) {
  extern __shared__ float2 smem_cb[];
  const int c = threadIdx.x % C, l = threadIdx.x / C;
  const int half = W / 2;
  const int kx = blockIdx.x * C + c;
  const int d = FLIP ? blockIdx.y : 0;
  const int tl = blockIdx.z;
  const int t = t0 + tl;
  if (FLIP && !slab_live(live, t, d)) return;  // no voxel reads this (tilt, slab)
  const float2 *F = src + (size_t)t * kN * half;
  const int sw = half + 1;
  // the 16 signs of rows l + 256 m: one packed entry (d, l, kx)
  const unsigned long long *sg = FLIP ? sign + ((size_t)d * 256 + l) * sw : nullptr;
  float2 v[16];
  if (kx < half) {
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = F[(size_t)(l + 256 * m) * half + kx];
    if (FLIP && kx == 0) {
      const unsigned long long wd = sg[0], wn = sg[half];
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        const int ky = l + 256 * m;
        const float2 mr = F[(size_t)((kN - ky) & (kN - 1)) * half];
        const float sdc = 0.5f * (float)packed_sign(wd, m);
        const float sny = 0.5f * (float)packed_sign(wn, m);
        const float a = 0.5f * (sdc + sny), b = 0.5f * (sdc - sny);
        v[m] = make_float2(a * v[m].x + b * mr.x, a * v[m].y - b * mr.y);
      }
    } else if (FLIP) {
      const unsigned long long w = sg[kx];
#pragma unroll
      for (int m = 0; m < 16; ++m) v[m] = scale2(0.5f * (float)packed_sign(w, m), v[m]);
    }
  } else {
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = make_float2(0.f, 0.f);
  }
  float2 *buf = smem_cb + c * kB4096Stride;
  bfft4096<FLIP, true>(v, buf, buf, roots, l, BlockSync());
  float2 *out = FLIP ? dst + ((size_t)tl * D + d) * kN * half : dst + (size_t)t * kN * half;
  if (kx < half) {
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) out[(size_t)(l + 256 * k2) * half + kx] = v[k2];
  }
}

// ---------------------------------------------------------------------------
// Row stage for 4096-pixel rows: one block of 256 threads per row pair.
// SPECTRA + RAMP: u = IFFT(w_even Z) is held in registers while the odd path
// c = IFFT(Z), c exp(-i pi n/N), FFT, times w_odd, IFFT runs; then u's
// transform.  Rows + RAMP: the twisted rows are held while the even path runs.
// ---------------------------------------------------------------------------
template <bool SPECTRA, bool RAMP, bool STAGED, bool F16>
__global__ void __launch_bounds__(256, 2) k_row_b4096(RowStageArgs a,
                                                     const float2 *__restrict__ roots,
                                                     const float2 *__restrict__ roots2N) {
  extern __shared__ float2 smem_rb[];
  __shared__ unsigned s_max[2];
  float2 *A = smem_rb, *B = smem_rb + kB4096Slots;
  const BlockSync sync;
  const int l = threadIdx.x;
  const int Y2 = row_pairs(a);  // row pairs of this launch
  const long pair = blockIdx.x;
  const int tl = (int)(pair / ((long)a.D * Y2));
  const int rem = (int)(pair - (long)tl * a.D * Y2);
  const int d = rem / Y2, y2 = a.y2_begin + (rem - d * Y2);
  const int t = a.t0 + tl;
  if (!slab_live(a.live, t, d)) return;  // no voxel reads this (tilt, slab): whole block
  const int ya = 2 * y2;
  const bool hb = ya + 1 < a.H;
  constexpr int half = kN / 2;

  float2 u[16], o[16];  // even and odd paths (the plain result in o)
  if (SPECTRA) {
    // Z[k] of the complex row pair from the two rows' half spectra
    const float2 *ga = a.g + (((size_t)tl * a.D + d) * a.H + ya) * half;
    const float2 *gb = ga + half;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int k = l + 256 * m;
      if (m < 8) {
        const float2 pa = ga[k];
        const float2 pb = hb ? gb[k] : make_float2(0.f, 0.f);
        o[m] = k == 0 ? make_float2(pa.x, pb.x) : make_float2(pa.x - pb.y, pa.y + pb.x);
      } else {
        const int kk = k == half ? 0 : kN - k;
        const float2 pa = ga[kk];
        const float2 pb = hb ? gb[kk] : make_float2(0.f, 0.f);
        o[m] = k == half ? make_float2(pa.y, pb.y) : make_float2(pa.x + pb.y, pb.x - pa.y);
      }
      if (RAMP) u[m] = scale2(ramp_w4096(2 * k), o[m]);
    }
    bfft4096<true, false>(o, A, B, roots, l, sync);  // c = IFFT(Z)
  } else {
    const float *ra = a.rows + ((size_t)(a.t0 + tl) * a.D + d) * a.plane_stride +
                      (size_t)ya * a.row_stride;
    const float *rb = ra + a.row_stride;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int n = l + 256 * m;
      u[m] = make_float2(ra[n], hb ? rb[n] : 0.f);
    }
    if (RAMP) {
#pragma unroll
      for (int m = 0; m < 16; ++m) o[m] = u[m];
      bfft4096<false, false>(u, A, B, roots, l, sync);  // FFT(c)
#pragma unroll
      for (int m = 0; m < 16; ++m) u[m] = scale2(ramp_w4096(2 * (l + 256 * m)), u[m]);
    }
  }
  if (RAMP) {
    // odd bins: FFT(c exp(-i pi n / N)), times w_odd, inverse
#pragma unroll
    for (int m = 0; m < 16; ++m) o[m] = cmul(o[m], __ldg(roots2N + l + 256 * m));
    bfft4096<false, false>(o, A, B, roots, l, sync);
#pragma unroll
    for (int m = 0; m < 16; ++m) o[m] = scale2(ramp_w4096(2 * (l + 256 * m) + 1), o[m]);
    bfft4096<true, false>(o, A, B, roots, l, sync);
    bfft4096<true, false>(u, A, B, roots, l, sync);  // the even path
  }

  // ---- combine and write
  const float f = a.tilt_factor ? a.tilt_factor[t] : 1.0f;
  const float ea = SPECTRA ? 0.5f : 1.0f / (float)(2 * kN);
  const float eo = 1.0f / (float)(2 * kN);
  float2 yv[16];
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    const int n = l + 256 * m;
    float2 y = o[m];
    if (RAMP) {
      const float2 tw = __ldg(roots2N + n);  // exp(-i pi n / N); conjugate below
      const float2 v = cmul(make_float2(tw.x, -tw.y), y);
      y = make_float2(ea * u[m].x + eo * v.x, ea * u[m].y + eo * v.y);
    }
    yv[m] = make_float2(y.x * f, y.y * f);
  }
  if (STAGED && !F16) {
    float2 *dst = (float2 *)a.staged + (((size_t)y2 * a.D + d) * a.T + t) * kN;
#pragma unroll
    for (int m = 0; m < 16; ++m) dst[l + 256 * m] = yv[m];
  } else if (STAGED && F16 && a.staging == kStageF16T) {
    // plain FP16 rows scaled by the tilt's 2^e(t)
    const float sc = f16t_scale(a, t);
    __half *da = f16t_row(a, d, t, ya);
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      da[l + 256 * m] = __float2half_rn(yv[m].x * sc);
      if (hb) da[kN + l + 256 * m] = __float2half_rn(yv[m].y * sc);
    }
  } else if (STAGED && F16) {
    // records need pixel n + 1 (another thread's): exchange through A, which
    // no thread reads any more; and the row maxima for the exponents
    if (l == 0) s_max[0] = s_max[1] = 0u;
#pragma unroll
    for (int m = 0; m < 16; ++m) A[l + 256 * m] = yv[m];
    float ma = 0.f, mb = 0.f;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      ma = fmaxf(ma, fabsf(yv[m].x));
      mb = fmaxf(mb, fabsf(yv[m].y));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      ma = fmaxf(ma, __shfl_xor_sync(0xffffffffu, ma, off));
      mb = fmaxf(mb, __shfl_xor_sync(0xffffffffu, mb, off));
    }
    sync();  // s_max cleared, A written
    if ((l & 31) == 0) {
      atomicMax(&s_max[0], __float_as_uint(ma));
      atomicMax(&s_max[1], __float_as_uint(mb));
    }
    sync();
    // 2^e brings the row maximum into [2^13, 2^14): full FP16 precision with
    // headroom below the FP16 maximum
    const float mxa = __uint_as_float(s_max[0]), mxb = __uint_as_float(s_max[1]);
    int e_a = mxa > 0.f ? 13 - ilogbf(mxa) : 0;
    int e_b = mxb > 0.f ? 13 - ilogbf(mxb) : 0;
    e_a = max(-120, min(120, e_a));
    e_b = max(-120, min(120, e_b));
    const float sa = __int_as_float((127 + e_a) << 23), sb = __int_as_float((127 + e_b) << 23);
    const size_t rowi = ((size_t)y2 * a.D + d) * a.T + t;
    uint2 *dst = (uint2 *)a.staged + rowi * kN;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int n = l + 256 * m;
      const float2 v1 = n + 1 < kN ? A[n + 1] : yv[m];
      dst[n] = staged_record_f16(make_float2(yv[m].x * sa, yv[m].y * sb),
                                 make_float2(v1.x * sa, v1.y * sb));
    }
    if (l == 0) {
      a.row_exp[2 * rowi] = (int8_t)e_a;
      a.row_exp[2 * rowi + 1] = (int8_t)e_b;
    }
  } else {
    float *da = a.out_rows + (((size_t)tl * a.D + d) * a.H + ya) * kN;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int n = l + 256 * m;
      da[n] = yv[m].x;
      if (hb) da[kN + n] = yv[m].y;
    }
  }
}

// ---------------------------------------------------------------- launchers
template <bool FLIP>
static cudaError_t column_b4096(const float2 *src, float2 *dst, const int8_t *sign, int t0,
                                int nt, int D, int W, const int2 *live, cudaStream_t s) {
  FftPlan p;
  if (!make_fft_plan(kN, &p)) return cudaErrorInvalidValue;
  constexpr int C = kColC;
  const size_t smem = (size_t)C * kB4096Stride * sizeof(float2);
  if (cudaError_t e_attr = ensure_dynamic_smem<k_column_b4096<FLIP, C>>((int)smem)) return e_attr;
  const int half = W / 2;
  dim3 grid((half + C - 1) / C, FLIP ? D : 1, nt);
  const unsigned long long *packed = FLIP ? sign_packed(sign, D, kN, W) : nullptr;
  if (((uintptr_t)packed & 7) != 0) return cudaErrorMisalignedAddress;  // 8-byte loads
  k_column_b4096<FLIP, C><<<grid, 256 * C, smem, s>>>(src, dst, packed, t0, D, W, p.roots, live);
  return cudaGetLastError();
}

cudaError_t launch_column_fft_b4096(float2 *spec, int T, int W, cudaStream_t s) {
  return column_b4096<false>(spec, spec, nullptr, 0, T, 1, W, nullptr, s);
}

cudaError_t launch_column_flip_b4096(const float2 *spec, float2 *g, const int8_t *sign, int t0,
                                     int nt, int D, int W, const int2 *live, cudaStream_t s) {
  return column_b4096<true>(spec, g, sign, t0, nt, D, W, live, s);
}

template <bool SPECTRA, bool RAMP, bool STAGED, bool F16>
static cudaError_t row_b4096(const RowStageArgs &a, cudaStream_t s) {
  FftPlan pN, p2N;
  if (!make_fft_plan(kN, &pN) || !make_fft_plan(2 * kN, &p2N)) return cudaErrorInvalidValue;
  const size_t smem = 2 * (size_t)kB4096Slots * sizeof(float2);
  auto kern = k_row_b4096<SPECTRA, RAMP, STAGED, F16>;
  if (cudaError_t e_attr = ensure_dynamic_smem<k_row_b4096<SPECTRA, RAMP, STAGED, F16>>((int)smem)) return e_attr;
  const long npairs = (long)a.nt * a.D * row_pairs(a);
  if (npairs == 0) return cudaSuccess;
  kern<<<(unsigned)npairs, 256, smem, s>>>(a, pN.roots, p2N.roots);
  return cudaGetLastError();
}

cudaError_t launch_row_stage_b4096(const RowStageArgs &a, cudaStream_t s) {
  const bool sp = a.input_spectra != 0, rm = a.ramp != 0, st = a.out_staged != 0;
  const bool h = a.staging != kStageF32;
  if (sp && rm && st && !h) return row_b4096<true, true, true, false>(a, s);
  if (sp && rm && st && h) return row_b4096<true, true, true, true>(a, s);
  if (!sp && rm && st && !h) return row_b4096<false, true, true, false>(a, s);
  if (!sp && rm && st && h) return row_b4096<false, true, true, true>(a, s);
  if (sp && !rm && !st) return row_b4096<true, false, false, false>(a, s);
  if (!sp && rm && !st) return row_b4096<false, true, false, false>(a, s);
  return cudaErrorInvalidValue;
}

}  // namespace gnc
