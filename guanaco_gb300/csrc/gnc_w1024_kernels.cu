// Correction and ramp-filter kernels for 1024-pixel rows and columns, built on
// the one-warp register FFT of gnc_fft_warp.cuh.  They compute what the
// power-of-two kernels of gnc_pow2_kernels.cu compute (same formulation of the
// phase flip and of the zero-padded ramp filter, see there), with each
// 1024-point transform held in one warp's registers: one shared-memory
// transpose per transform instead of three full passes.
#include "gnc_common.cuh"
#include "gnc_fft_warp.cuh"

namespace gnc {

namespace {
constexpr int kN = 1024;
constexpr float kInvN = 1.0f / 1024.0f;  // exact: w_K = K / N = K * 2^-10

__device__ __forceinline__ float ramp_w1024(int K) {  // filter.cpp:38-41, mirrored above N
  const int kk = K <= kN ? K : 2 * kN - K;
  return (float)kk * kInvN;
}
}  // namespace

// ---------------------------------------------------------------------------
// Row transform of the raw projections: one warp per pair of rows.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_rfft_rows_w1024(const float *__restrict__ proj,
                                                         float2 *__restrict__ spec, int H,
                                                         const float2 *__restrict__ roots) {
  extern __shared__ float2 smem_f[];
  float2 *tw = smem_f;
  warp_fft_twiddles(tw, roots);
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float2 *z = smem_f + 1024 + kWarpFftSlots * w;
  const int t = blockIdx.y;
  const int npair = (H + 1) / 2;
  const int pair = blockIdx.x * 8 + w;
  if (pair >= npair) return;
  const int ya = 2 * pair, yb = ya + 1;
  const float *ra = proj + ((size_t)t * H + ya) * kN;
  const float *rb = ra + kN;
  float2 v[32];
#pragma unroll
  for (int m = 0; m < 32; ++m)
    v[m] = make_float2(ra[32 * m + lane], yb < H ? rb[32 * m + lane] : 0.f);
  warp_fft1024<false>(v, z, tw, lane);
  __syncwarp();
#pragma unroll
  for (int m = 0; m < 32; ++m) z[32 * m + lane] = v[m];
  __syncwarp();
  constexpr int half = kN / 2;
  float2 *oa = spec + ((size_t)t * H + ya) * half;
  float2 *ob = oa + half;
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    const int k = 32 * m + lane;
    float2 A, B;
    if (k == 0) {
      const float2 z0 = z[0], zn = z[half];
      A = make_float2(z0.x, zn.x);
      B = make_float2(z0.y, zn.y);
    } else {
      const float2 zk = z[k], zm = z[kN - k];
      A = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
      B = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
    }
    oa[k] = A;
    if (yb < H) ob[k] = B;
  }
}

// ---------------------------------------------------------------------------
// Column transforms of 1024 rows: a block holds 8 adjacent columns (row pitch
// 9 float2, kWarpFftSlots rows), one warp per column; the warp's transpose
// reuses its column's slots.  FLIP: per-slab phase flip then inverse transform (gnc_correct.cu).
// ---------------------------------------------------------------------------
template <bool FLIP>
__global__ void __launch_bounds__(256, 2) k_column_w1024(const float2 *__restrict__ src,
                                                      float2 *__restrict__ dst,
                                                      const ulonglong2 *__restrict__ sign,
                                                      int t0, int D, int W,
                                                      const float2 *__restrict__ roots,
                                                      const int2 *__restrict__ live) {
  constexpr int C = 8, P = 9;
  const int d = FLIP ? blockIdx.y : 0;
  const int tl = blockIdx.z;
  const int t = t0 + tl;
  if (FLIP && !slab_live(live, t, d)) return;  // no voxel reads this (tilt, slab)
  extern __shared__ float2 smem_w[];
  float2 *tw = smem_w;
  float2 *tile = smem_w + 1024;
  warp_fft_twiddles(tw, roots);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int half = W / 2;
  const int c0 = blockIdx.x * C;
  const float2 *F = src + (size_t)t * kN * half;
  const int sw = half + 1;
  // each thread moves one column (c) of rows y0 + 32 j: all 32 loads in flight;
  // their 32 signs are one packed entry (d, y0, kx).  y0 permutes the 32
  // row residues so that the two rows of a half warp are 8 apart: with the
  // 9-float2 pitch their tile slots then fall in bank pairs 0-7 and 8-15.
  const int c = threadIdx.x & (C - 1), r0 = threadIdx.x / C;
  const int y0 = (r0 & 16) + ((r0 >> 1) & 7) + 8 * (r0 & 1);
  const int kx = c0 + c;
  const ulonglong2 *sg = FLIP ? sign + ((size_t)d * 32 + y0) * sw : nullptr;
  {
    float2 r[32];
    if (kx < half) {
#pragma unroll
      for (int j = 0; j < 32; ++j) r[j] = F[(size_t)(y0 + 32 * j) * half + kx];
      if (FLIP && kx == 0) {
        const ulonglong2 wd = sg[0], wn = sg[half];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int ky = y0 + 32 * j;
          const float2 m = F[(size_t)((kN - ky) & (kN - 1)) * half];
          const float sdc = 0.5f * (float)packed_sign(j < 16 ? wd.x : wd.y, j & 15);
          const float sny = 0.5f * (float)packed_sign(j < 16 ? wn.x : wn.y, j & 15);
          const float a = 0.5f * (sdc + sny), b = 0.5f * (sdc - sny);
          r[j] = make_float2(a * r[j].x + b * m.x, a * r[j].y - b * m.y);
        }
      } else if (FLIP) {
        const ulonglong2 w = sg[kx];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const float f = 0.5f * (float)packed_sign(j < 16 ? w.x : w.y, j & 15);
          r[j] = make_float2(f * r[j].x, f * r[j].y);
        }
      }
    } else {
#pragma unroll
      for (int j = 0; j < 32; ++j) r[j] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int j = 0; j < 32; ++j) tile[(y0 + 32 * j) * P + c] = r[j];
  }
  __syncthreads();
  float2 v[32];
  float2 *col = tile + w;
#pragma unroll
  for (int m = 0; m < 32; ++m) v[m] = col[(32 * m + lane) * P];
  warp_fft1024<FLIP, P>(v, col, tw, lane);
  __syncwarp();
#pragma unroll
  for (int m = 0; m < 32; ++m) col[(32 * m + lane) * P] = v[m];
  __syncthreads();
  float2 *out = FLIP ? dst + ((size_t)tl * D + d) * kN * half : dst + (size_t)t * kN * half;
  if (kx < half) {
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int ky = y0 + 32 * j;
      out[(size_t)ky * half + kx] = tile[ky * P + c];
    }
  }
}

// ---------------------------------------------------------------------------
// Row stage for 1024-pixel rows: one warp per row pair.
// The input is parked in shared memory; the odd path (c, twist, FFT, w_odd,
// IFFT, untwist / 2N) runs in registers and trades places with it; then the
// even path runs on the parked input and adds the odd result.  The ramp's
// four transforms are one forward transform run in a loop.
// ---------------------------------------------------------------------------
template <bool SPECTRA, bool RAMP, bool STAGED, bool F16>
__global__ void __launch_bounds__(128, 3) k_row_w1024(RowStageArgs a,
                                                   const float2 *__restrict__ roots,
                                                   const float2 *__restrict__ roots2N) {
  constexpr int WPB = 4;
  extern __shared__ float2 smem_r[];
  float2 *tw = smem_r;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float2 *tb = smem_r + 1024 + w * (kWarpFftSlots + 1024);  // transpose slots
  float2 *vb = tb + kWarpFftSlots;                           // parking slots
  warp_fft_twiddles(tw, roots);
  __syncthreads();
  const int Y2 = row_pairs(a);  // row pairs of this launch
  const long npairs = (long)a.nt * a.D * Y2;
  const long pair = (long)blockIdx.x * WPB + w;
  if (pair >= npairs) return;
  const int tl = (int)(pair / ((long)a.D * Y2));
  const int rem = (int)(pair - (long)tl * a.D * Y2);
  const int d = rem / Y2, y2 = a.y2_begin + (rem - d * Y2);
  const int t = a.t0 + tl;
  if (!slab_live(a.live, t, d)) return;  // no voxel reads this (tilt, slab)
  const int ya = 2 * y2;
  const bool hb = ya + 1 < a.H;
  constexpr int half = kN / 2;
  const float2 *ga = nullptr, *gb = nullptr;
  const float *ra = nullptr, *rb = nullptr;
  if (SPECTRA) {
    ga = a.g + (((size_t)tl * a.D + d) * a.H + ya) * half;
    gb = ga + half;
  } else {
    const float *base = a.rows + ((size_t)(a.t0 + tl) * a.D + d) * a.plane_stride;
    ra = base + (size_t)ya * a.row_stride;
    rb = base + (size_t)(ya + 1) * a.row_stride;
  }
  // the input row pair as one complex row: the spectrum Z (SPECTRA) or c
  float2 v[32];
#pragma unroll
  for (int m = 0; m < 32; ++m) {
    const int k = 32 * m + lane;
    if (SPECTRA) {
      if (m < 16) {
        const float2 pa = ga[k];
        const float2 pb = hb ? gb[k] : make_float2(0.f, 0.f);
        v[m] = k == 0 ? make_float2(pa.x, pb.x) : make_float2(pa.x - pb.y, pa.y + pb.x);
      } else {
        const int km = kN - k;  // 1 .. 512
        const float2 pa = ga[km & (half - 1)];
        const float2 pb = hb ? gb[km & (half - 1)] : make_float2(0.f, 0.f);
        v[m] = km == half ? make_float2(pa.y, pb.y) : make_float2(pa.x + pb.y, pb.x - pa.y);
      }
    } else {
      v[m] = make_float2(ra[k], hb ? rb[k] : 0.f);
    }
  }
  if (RAMP) {
    // park the input; each lane only touches its own elements 32 m + lane
#pragma unroll
    for (int m = 0; m < 32; ++m) vb[32 * m + lane] = v[m];
  }
  if (!RAMP) {
    if (SPECTRA) warp_fft1024<true>(v, tb, tw, lane);  // the corrected rows: IFFT(Z)
  } else {
    // Four transforms, all run as one forward transform in a loop (one copy of
    // its code): IFFT(x) = conj(FFT(conj(x))), the conjugations folded into
    // the pointwise steps between the passes.
    //   spectra in: IFFT(Z) -> c; FFT(c e^{-i pi n/N}) * w_odd; IFFT -> odd term;
    //               IFFT(w_even Z) -> even term
    //   rows in:    FFT(c e^{-i pi n/N}) * w_odd; IFFT -> odd term; FFT(c) * w_even;
    //               IFFT -> even term
    if (SPECTRA) {
#pragma unroll
      for (int m = 0; m < 32; ++m) v[m].y = -v[m].y;
    } else {
#pragma unroll
      for (int m = 0; m < 32; ++m) v[m] = cmul(v[m], __ldg(roots2N + 32 * m + lane));
    }
    const int first_odd = SPECTRA ? 1 : 0;  // pass whose output is FFT(c twist)
#pragma unroll 1
    for (int ps = 0; ps < 4; ++ps) {
      warp_fft1024<false>(v, tb, tw, lane);
      __syncwarp();
      if (ps == 3) {
        // even term: IFFT = conj of this pass; y = ea * even + odd
        const float ea = SPECTRA ? 0.5f : 0.5f * kInvN;
#pragma unroll
        for (int m = 0; m < 32; ++m) {
          const float2 o = vb[32 * m + lane];
          v[m] = make_float2(ea * v[m].x + o.x, o.y - ea * v[m].y);
        }
      } else if (SPECTRA && ps == 0) {
        // c = conj(v); twist: c e^{-i pi n / N}
#pragma unroll
        for (int m = 0; m < 32; ++m)
          v[m] = cmul(make_float2(v[m].x, -v[m].y), __ldg(roots2N + 32 * m + lane));
      } else if (ps == first_odd) {
        // odd bins times w_odd, conjugated for the inverse
#pragma unroll
        for (int m = 0; m < 32; ++m) {
          const float wo = ramp_w1024(2 * (32 * m + lane) + 1);
          v[m] = make_float2(wo * v[m].x, -wo * v[m].y);
        }
      } else if (ps == first_odd + 1) {
        // odd term conj(v) e^{+i pi n / N} / 2N to the parking slots; the input
        // comes back (spectra: Z, then w_even Z conjugated for the inverse)
#pragma unroll
        for (int m = 0; m < 32; ++m) {
          const float2 r2 = __ldg(roots2N + 32 * m + lane);
          const float2 o = cmul(make_float2(r2.x, -r2.y), make_float2(v[m].x, -v[m].y));
          v[m] = vb[32 * m + lane];
          vb[32 * m + lane] = make_float2(o.x * (0.5f * kInvN), o.y * (0.5f * kInvN));
          if (SPECTRA) {
            const float we = ramp_w1024(2 * (32 * m + lane));
            v[m] = make_float2(we * v[m].x, -we * v[m].y);
          }
        }
      } else {
        // rows in, after FFT(c): w_even, conjugated for the inverse
#pragma unroll
        for (int m = 0; m < 32; ++m) {
          const float we = ramp_w1024(2 * (32 * m + lane));
          v[m] = make_float2(we * v[m].x, -we * v[m].y);
        }
      }
    }
  }
  float2 *y = v;
  const float f = a.tilt_factor ? a.tilt_factor[t] : 1.0f;
#pragma unroll
  for (int m = 0; m < 32; ++m) y[m] = make_float2(y[m].x * f, y[m].y * f);
  // pixel 32 m + lane + 1 of the row pair: the next lane's element m, or lane
  // 0's element m + 1 for lane 31 (the last pixel is its own neighbour)
  auto next_px = [&](const float2 *w, int m) {
    const float2 src = (lane == 0 && m < 31) ? w[m < 31 ? m + 1 : m] : w[m];
    float2 nb;
    nb.x = __shfl_sync(0xffffffffu, src.x, (lane + 1) & 31);
    nb.y = __shfl_sync(0xffffffffu, src.y, (lane + 1) & 31);
    return (m == 31 && lane == 31) ? w[m] : nb;
  };
  if (STAGED && !F16) {
    float2 *dst = (float2 *)a.staged + (((size_t)y2 * a.D + d) * a.T + t) * kN;
#pragma unroll
    for (int m = 0; m < 32; ++m) dst[32 * m + lane] = y[m];
  } else if (STAGED && F16 && a.staging == kStageF16T) {
    // plain FP16 rows scaled by the tilt's 2^e(t)
    const float sc = f16t_scale(a, t);
    __half *da = f16t_row(a, d, t, ya);
#pragma unroll
    for (int m = 0; m < 32; ++m) {
      da[32 * m + lane] = __float2half_rn(y[m].x * sc);
      if (hb) da[kN + 32 * m + lane] = __float2half_rn(y[m].y * sc);
    }
  } else if (STAGED && F16) {
    float ma = 0.f, mb = 0.f;
#pragma unroll
    for (int m = 0; m < 32; ++m) {
      ma = fmaxf(ma, fabsf(y[m].x));
      mb = fmaxf(mb, fabsf(y[m].y));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ma = fmaxf(ma, __shfl_xor_sync(0xffffffffu, ma, o));
      mb = fmaxf(mb, __shfl_xor_sync(0xffffffffu, mb, o));
    }
    // 2^e brings the row maximum into [2^13, 2^14): full FP16 precision with
    // headroom below the FP16 maximum
    int e_a = ma > 0.f ? 13 - ilogbf(ma) : 0;
    int e_b = mb > 0.f ? 13 - ilogbf(mb) : 0;
    e_a = max(-120, min(120, e_a));
    e_b = max(-120, min(120, e_b));
    const float sa = __int_as_float((127 + e_a) << 23), sb = __int_as_float((127 + e_b) << 23);
    const size_t rowi = ((size_t)y2 * a.D + d) * a.T + t;
    uint2 *dst = (uint2 *)a.staged + rowi * kN;
#pragma unroll
    for (int m = 0; m < 32; ++m) y[m] = make_float2(y[m].x * sa, y[m].y * sb);
#pragma unroll
    for (int m = 0; m < 32; ++m) dst[32 * m + lane] = staged_record_f16(y[m], next_px(y, m));
    if (lane == 0) {
      a.row_exp[2 * rowi] = (int8_t)e_a;
      a.row_exp[2 * rowi + 1] = (int8_t)e_b;
    }
  } else {
    float *da = a.out_rows + (((size_t)tl * a.D + d) * a.H + ya) * kN;
#pragma unroll
    for (int m = 0; m < 32; ++m) {
      da[32 * m + lane] = y[m].x;
      if (hb) da[kN + 32 * m + lane] = y[m].y;
    }
  }
}

// ---------------------------------------------------------------- launchers
static bool roots_for(int n, const float2 **r) {
  FftPlan p;
  if (!make_fft_plan(n, &p)) return false;
  *r = p.roots;
  return true;
}

cudaError_t launch_rfft_rows_w1024(const float *proj, float2 *spec, int T, int H,
                                   cudaStream_t s) {
  const float2 *roots;
  if (!roots_for(kN, &roots)) return cudaErrorInvalidValue;
  const int npair = (H + 1) / 2;
  const size_t smem = (1024 + 8 * kWarpFftSlots) * sizeof(float2);
  if (cudaError_t e_attr = ensure_dynamic_smem<k_rfft_rows_w1024>((int)smem)) return e_attr;
  dim3 grid((npair + 7) / 8, T);
  k_rfft_rows_w1024<<<grid, 256, smem, s>>>(proj, spec, H, roots);
  return cudaGetLastError();
}

template <bool FLIP>
static cudaError_t column_w1024(const float2 *src, float2 *dst, const int8_t *sign, int t0,
                                int nt, int D, int W, const int2 *live, cudaStream_t s) {
  const float2 *roots;
  if (!roots_for(kN, &roots)) return cudaErrorInvalidValue;
  const size_t smem = (1024 + (size_t)kWarpFftSlots * 9) * sizeof(float2);
  if (cudaError_t e_attr = ensure_dynamic_smem<k_column_w1024<FLIP>>((int)smem)) return e_attr;
  const int half = W / 2;
  const ulonglong2 *packed = FLIP ? (const ulonglong2 *)sign_packed(sign, D, kN, W) : nullptr;
  if (((uintptr_t)packed & 15) != 0) return cudaErrorMisalignedAddress;  // 16-byte loads
  dim3 grid((half + 7) / 8, FLIP ? D : 1, nt);
  k_column_w1024<FLIP><<<grid, 256, smem, s>>>(src, dst, packed, t0, D, W, roots, live);
  return cudaGetLastError();
}

cudaError_t launch_column_fft_w1024(float2 *spec, int T, int W, cudaStream_t s) {
  return column_w1024<false>(spec, spec, nullptr, 0, T, 1, W, nullptr, s);
}

cudaError_t launch_column_flip_w1024(const float2 *spec, float2 *g, const int8_t *sign, int t0,
                                     int nt, int D, int W, const int2 *live, cudaStream_t s) {
  return column_w1024<true>(spec, g, sign, t0, nt, D, W, live, s);
}

template <bool SPECTRA, bool RAMP, bool STAGED, bool F16>
static cudaError_t row_w1024(const RowStageArgs &a, cudaStream_t s) {
  const float2 *roots, *roots2N;
  if (!roots_for(kN, &roots) || !roots_for(2 * kN, &roots2N)) return cudaErrorInvalidValue;
  const size_t smem = (1024 + 4 * (kWarpFftSlots + 1024)) * sizeof(float2);
  auto kern = k_row_w1024<SPECTRA, RAMP, STAGED, F16>;
  if (cudaError_t e_attr = ensure_dynamic_smem<k_row_w1024<SPECTRA, RAMP, STAGED, F16>>((int)smem)) return e_attr;
  const long npairs = (long)a.nt * a.D * row_pairs(a);
  kern<<<(unsigned)((npairs + 3) / 4), 128, smem, s>>>(a, roots, roots2N);
  return cudaGetLastError();
}

cudaError_t launch_row_stage_w1024(const RowStageArgs &a, cudaStream_t s) {
  const bool sp = a.input_spectra != 0, rm = a.ramp != 0, st = a.out_staged != 0;
  const bool h = a.staging != kStageF32;
  if (sp && rm && st && !h) return row_w1024<true, true, true, false>(a, s);
  if (sp && rm && st && h) return row_w1024<true, true, true, true>(a, s);
  if (!sp && rm && st && !h) return row_w1024<false, true, true, false>(a, s);
  if (!sp && rm && st && h) return row_w1024<false, true, true, true>(a, s);
  if (sp && !rm && !st) return row_w1024<true, false, false, false>(a, s);
  if (!sp && rm && !st) return row_w1024<false, true, false, false>(a, s);
  return cudaErrorInvalidValue;
}

}  // namespace gnc
