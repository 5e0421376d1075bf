// Correction and ramp-filter kernels for 128-, 256-, 384- and 512-pixel rows
// and columns, built on the register transforms of gnc_fft_w512.cuh (16
// values per lane; a warp runs one 512- or 384-point transform, two 256-point
// or four 128-point ones).  They compute what the power-of-two kernels of gnc_pow2_kernels.cu
// compute (same phase flip of the packed half spectra, same four-transform
// form of the zero-padded ramp filter, see there): the row stage chains its
// four transforms and the pointwise products in registers and holds the even
// path's data in registers while the odd path runs; the column kernels stage
// a tile of adjacent columns in shared memory so that every global access is
// a full 64- or 128-byte row piece.
#include "gnc_common.cuh"
#include "gnc_fft_w512.cuh"

namespace gnc {

namespace {

template <int N>
__device__ __forceinline__ float ramp_wn(int K) {  // filter.cpp:38-41, w_K = K / N
  const int kk = K <= N ? K : 2 * N - K;
  return (float)kk / (float)N;
}

__device__ __forceinline__ float2 scale2(float w, float2 v) { return make_float2(w * v.x, w * v.y); }

// Column tile of the column kernels: C columns, row pitch P (float2), one
// transform per column.  512 and 384 rows: 8 columns (64-byte row pieces), a
// warp per column, rows of a thread y0 + 32 j with y0 permuting the 32
// residues so that the two rows of a half warp are 8 apart (pitch 9: bank
// pairs 0-7 and 8-15).  256 rows: 16 columns (128-byte row pieces), a half warp
// per column.  128 rows: 32 columns (256-byte row pieces), a quarter warp per
// column, pitch 34 (= 2 mod 16) so that the two columns of a half warp read
// distinct bank pairs.
template <int H>
struct ColW512 {
  static constexpr int C = H >= 384 ? 8 : (H == 256 ? 16 : 32);
  static constexpr int P = H == 128 ? 34 : C + 1;
  static constexpr int RS = 256 / C;  // row residues per pass of the block
  static constexpr int J = H / RS;    // rows per thread
  static constexpr int SLOTS = WarpFftShape<H>::SLOTS;
  static constexpr size_t SMEM = ((size_t)H * P + (size_t)C * SLOTS) * sizeof(float2);
};

}  // namespace

// ---------------------------------------------------------------------------
// Column transforms of 256 or 512 rows; FLIP: per-slab phase flip (signs from
// the packed table: entry (d, residue, kx) holds the 16 signs of a thread's
// rows) then the inverse transform (the packed DC / Nyquist column as in
// gnc_correct.cu).
// ---------------------------------------------------------------------------
template <int H, bool FLIP>
__global__ void __launch_bounds__(256, 3) k_column_w512(const float2 *__restrict__ src,
                                                       float2 *__restrict__ dst,
                                                       const unsigned long long *__restrict__ sign,
                                                       int t0, int D, int W,
                                                       const float2 *__restrict__ roots,
                                                       const int2 *__restrict__ live) {
  using P = ColW512<H>;
  constexpr int C = P::C, L = WarpFftShape<H>::L;
  extern __shared__ float2 smem_c5[];
  float2 *tile = smem_c5;
  const int half = W / 2;
  const int c0 = blockIdx.x * C;
  const int d = FLIP ? blockIdx.y : 0;
  const int tl = blockIdx.z;
  const int t = t0 + tl;
  if (FLIP && !slab_live(live, t, d)) return;  // no voxel reads this (tilt, slab)
  const float2 *F = src + (size_t)t * H * half;
  const int sw = half + 1;
  const int c = threadIdx.x % C, r0 = threadIdx.x / C;
  const int y0 = C == 8 ? (r0 & 16) + ((r0 >> 1) & 7) + 8 * (r0 & 1) : r0;
  const int kx = c0 + c;
  {
    float2 r[P::J];
    if (kx < half) {
#pragma unroll
      for (int j = 0; j < P::J; ++j) r[j] = F[(size_t)(y0 + P::RS * j) * half + kx];
      if (FLIP) {
        const unsigned long long *sg = sign + ((size_t)d * P::RS + y0) * sw;
        if (kx == 0) {
          const unsigned long long wd = sg[0], wn = sg[half];
#pragma unroll
          for (int j = 0; j < P::J; ++j) {
            const int ky = y0 + P::RS * j;
            const float2 m = F[(size_t)(ky == 0 ? 0 : H - ky) * half];  // row -ky mod H
            const float sdc = 0.5f * (float)packed_sign(wd, j);
            const float sny = 0.5f * (float)packed_sign(wn, j);
            const float a = 0.5f * (sdc + sny), b = 0.5f * (sdc - sny);
            r[j] = make_float2(a * r[j].x + b * m.x, a * r[j].y - b * m.y);
          }
        } else {
          const unsigned long long wv = sg[kx];
#pragma unroll
          for (int j = 0; j < P::J; ++j) r[j] = scale2(0.5f * (float)packed_sign(wv, j), r[j]);
        }
      }
    } else {
#pragma unroll
      for (int j = 0; j < P::J; ++j) r[j] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int j = 0; j < P::J; ++j) tile[(y0 + P::RS * j) * P::P + c] = r[j];
  }
  __syncthreads();
  {
    constexpr int TPW = WarpFftShape<H>::TPW;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int sub = lane / L;
    const bool act = sub < TPW;  // 384 rows: lanes 24..31 idle
    const int l = act ? lane % L : lane - TPW * L;
    const int ct = w * TPW + (act ? sub : 0);  // this transform's column
    float2 *slots = tile + (size_t)H * P::P + (size_t)ct * P::SLOTS;
    float2 v[16];
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = act ? tile[(l + L * m) * P::P + ct] : make_float2(0.f, 0.f);
    warp_fft_n<H, FLIP>(v, slots, roots, l, act);
    if (act) {
#pragma unroll
      for (int m = 0; m < 16; ++m) tile[(l + L * m) * P::P + ct] = v[m];
    }
  }
  __syncthreads();
  float2 *out = FLIP ? dst + ((size_t)tl * D + d) * H * half : dst + (size_t)t * H * half;
  if (kx < half) {
#pragma unroll
    for (int j = 0; j < P::J; ++j) {
      const int ky = y0 + P::RS * j;
      out[(size_t)ky * half + kx] = tile[ky * P::P + c];
    }
  }
}

// ---------------------------------------------------------------------------
// Row stage for 128-, 256-, 384- and 512-pixel rows: one transform (a warp for
// 512 and 384, a half or quarter warp for 256 and 128) per row pair, four
// warps per block.
// SPECTRA + RAMP: u = IFFT(w_even Z) is held in registers while the odd path
// c = IFFT(Z), c exp(-i pi n/N), FFT, times w_odd, IFFT runs; then u's
// transform.  Rows + RAMP: the twisted rows are held while the even path runs.
// ---------------------------------------------------------------------------
template <int N, bool SPECTRA, bool RAMP, bool STAGED, bool F16>
__global__ void __launch_bounds__(128) k_row_w512(RowStageArgs a, const float2 *__restrict__ roots,
                                                  const float2 *__restrict__ roots2N) {
  using S = WarpFftShape<N>;
  constexpr int L = S::L, TPW = S::TPW, PPB = 4 * TPW;
  __shared__ float2 slots_all[PPB][S::SLOTS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // 384: lanes 24..31 are idle and shadow lanes 0..7 (same loads, no stores)
  const bool act = lane / L < TPW;
  const int sub = act ? lane / L : 0, l = act ? lane % L : lane - TPW * L;
  float2 *slots = slots_all[w * TPW + sub];
  const int Y2 = row_pairs(a);  // row pairs of this launch
  const long npairs = (long)a.nt * a.D * Y2;
  long pair = (long)blockIdx.x * PPB + w * TPW + sub;
  bool active = act && pair < npairs;
  if (pair >= npairs) pair = npairs - 1;  // the lanes of a warp stay together for its shuffles
  const int tl = (int)(pair / ((long)a.D * Y2));
  const int rem = (int)(pair - (long)tl * a.D * Y2);
  const int d = rem / Y2, y2 = a.y2_begin + (rem - d * Y2);
  const int t = a.t0 + tl;
  // a (tilt, slab) no voxel reads is not stored; a warp with none to store
  // returns (no block barrier follows)
  active = active && slab_live(a.live, t, d);
  if (!__any_sync(0xffffffffu, active)) return;
  const int ya = 2 * y2;
  const bool hb = ya + 1 < a.H;
  constexpr int half = N / 2;

  float2 u[16], o[16];  // even and odd paths (the plain result in o)
  if (SPECTRA) {
    // Z[k] of the complex row pair from the two rows' half spectra
    const float2 *ga = a.g + (((size_t)tl * a.D + d) * a.H + ya) * half;
    const float2 *gb = ga + half;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int k = l + L * m;
      if (m < 8) {
        const float2 pa = ga[k];
        const float2 pb = hb ? gb[k] : make_float2(0.f, 0.f);
        o[m] = k == 0 ? make_float2(pa.x, pb.x) : make_float2(pa.x - pb.y, pa.y + pb.x);
      } else {
        const int kk = k == half ? 0 : N - k;
        const float2 pa = ga[kk];
        const float2 pb = hb ? gb[kk] : make_float2(0.f, 0.f);
        o[m] = k == half ? make_float2(pa.y, pb.y) : make_float2(pa.x + pb.y, pb.x - pa.y);
      }
      if (RAMP) u[m] = scale2(ramp_wn<N>(2 * k), o[m]);
    }
    warp_fft_n<N, true>(o, slots, roots, l, act);  // c = IFFT(Z)
  } else {
    const float *ra = a.rows + ((size_t)(a.t0 + tl) * a.D + d) * a.plane_stride +
                      (size_t)ya * a.row_stride;
    const float *rb = ra + a.row_stride;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int n = l + L * m;
      u[m] = make_float2(ra[n], hb ? rb[n] : 0.f);
    }
    if (RAMP) {
#pragma unroll
      for (int m = 0; m < 16; ++m) o[m] = u[m];
      warp_fft_n<N, false>(u, slots, roots, l, act);  // FFT(c)
#pragma unroll
      for (int m = 0; m < 16; ++m) u[m] = scale2(ramp_wn<N>(2 * (l + L * m)), u[m]);
    }
  }
  if (RAMP) {
    // odd bins: FFT(c exp(-i pi n / N)), times w_odd, inverse
#pragma unroll
    for (int m = 0; m < 16; ++m) o[m] = cmul(o[m], __ldg(roots2N + l + L * m));
    warp_fft_n<N, false>(o, slots, roots, l, act);
#pragma unroll
    for (int m = 0; m < 16; ++m) o[m] = scale2(ramp_wn<N>(2 * (l + L * m) + 1), o[m]);
    warp_fft_n<N, true>(o, slots, roots, l, act);
    warp_fft_n<N, true>(u, slots, roots, l, act);  // the even path
  }

  // ---- combine and write
  const float f = a.tilt_factor ? a.tilt_factor[t] : 1.0f;
  const float ea = SPECTRA ? 0.5f : 1.0f / (float)(2 * N);
  const float eo = 1.0f / (float)(2 * N);
  float2 yv[16];
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    const int n = l + L * m;
    float2 y = o[m];
    if (RAMP) {
      const float2 tw = __ldg(roots2N + n);  // exp(-i pi n / N); conjugate below
      const float2 v = cmul(make_float2(tw.x, -tw.y), y);
      y = make_float2(ea * u[m].x + eo * v.x, ea * u[m].y + eo * v.y);
    }
    yv[m] = make_float2(y.x * f, y.y * f);
  }
  if (STAGED && !F16) {
    if (active) {
      float2 *dst = (float2 *)a.staged + (((size_t)y2 * a.D + d) * a.T + t) * N;
#pragma unroll
      for (int m = 0; m < 16; ++m) dst[l + L * m] = yv[m];
    }
  } else if (STAGED && F16 && a.staging == kStageF16T) {
    // plain FP16 rows scaled by the tilt's 2^e(t)
    if (active) {
      const float sc = f16t_scale(a, t);
      __half *da = f16t_row(a, d, t, ya);
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        da[l + L * m] = __float2half_rn(yv[m].x * sc);
        if (hb) da[N + l + L * m] = __float2half_rn(yv[m].y * sc);
      }
    }
  } else if (STAGED && F16) {
    float ma = 0.f, mb = 0.f;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      ma = fmaxf(ma, fabsf(yv[m].x));
      mb = fmaxf(mb, fabsf(yv[m].y));
    }
    if (!act) ma = mb = 0.f;
    // within the transform's lanes (384: the whole warp, idle lanes at 0)
    constexpr int R0 = (L & (L - 1)) ? 16 : L / 2;
#pragma unroll
    for (int off = R0; off > 0; off >>= 1) {
      ma = fmaxf(ma, __shfl_xor_sync(0xffffffffu, ma, off));
      mb = fmaxf(mb, __shfl_xor_sync(0xffffffffu, mb, off));
    }
    // 2^e brings the row maximum into [2^13, 2^14): full FP16 precision with
    // headroom below the FP16 maximum
    int e_a = ma > 0.f ? 13 - ilogbf(ma) : 0;
    int e_b = mb > 0.f ? 13 - ilogbf(mb) : 0;
    e_a = max(-120, min(120, e_a));
    e_b = max(-120, min(120, e_b));
    const float sa = __int_as_float((127 + e_a) << 23), sb = __int_as_float((127 + e_b) << 23);
#pragma unroll
    for (int m = 0; m < 16; ++m) yv[m] = make_float2(yv[m].x * sa, yv[m].y * sb);
    // pixel n + 1 of n = l + L m: lane l + 1's element m, or lane 0's element
    // m + 1 for l = L - 1 (the last pixel is its own neighbour)
    const int nb_lane = sub * L + (l + 1) % L;
    const size_t rowi = ((size_t)y2 * a.D + d) * a.T + t;
    uint2 *dst = (uint2 *)a.staged + rowi * N;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const float2 src = (l == 0 && m < 15) ? yv[m + 1] : yv[m];
      float2 nb;
      nb.x = __shfl_sync(0xffffffffu, src.x, nb_lane);
      nb.y = __shfl_sync(0xffffffffu, src.y, nb_lane);
      if (m == 15 && l == L - 1) nb = yv[m];
      if (active) dst[l + L * m] = staged_record_f16(yv[m], nb);
    }
    if (active && l == 0) {
      a.row_exp[2 * rowi] = (int8_t)e_a;
      a.row_exp[2 * rowi + 1] = (int8_t)e_b;
    }
  } else if (active) {
    float *da = a.out_rows + (((size_t)tl * a.D + d) * a.H + ya) * N;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int n = l + L * m;
      da[n] = yv[m].x;
      if (hb) da[N + n] = yv[m].y;
    }
  }
}

// ---------------------------------------------------------------- launchers
template <int H, bool FLIP>
static cudaError_t column_w512(const float2 *src, float2 *dst, const int8_t *sign, int t0, int nt,
                               int D, int W, const int2 *live, cudaStream_t s) {
  using P = ColW512<H>;
  FftPlan p;
  if (!make_fft_plan(H, &p)) return cudaErrorInvalidValue;
  if (cudaError_t e_attr = ensure_dynamic_smem<k_column_w512<H, FLIP>>((int)P::SMEM)) return e_attr;
  const unsigned long long *packed = FLIP ? sign_packed(sign, D, H, W) : nullptr;
  if (((uintptr_t)packed & 7) != 0) return cudaErrorMisalignedAddress;  // 8-byte loads
  const int half = W / 2;
  dim3 grid((half + P::C - 1) / P::C, FLIP ? D : 1, nt);
  k_column_w512<H, FLIP><<<grid, 256, P::SMEM, s>>>(src, dst, packed, t0, D, W, p.roots, live);
  return cudaGetLastError();
}

cudaError_t launch_column_fft_w512(float2 *spec, int T, int H, int W, cudaStream_t s) {
  switch (H) {
    case 128: return column_w512<128, false>(spec, spec, nullptr, 0, T, 1, W, nullptr, s);
    case 256: return column_w512<256, false>(spec, spec, nullptr, 0, T, 1, W, nullptr, s);
    case 384: return column_w512<384, false>(spec, spec, nullptr, 0, T, 1, W, nullptr, s);
    case 512: return column_w512<512, false>(spec, spec, nullptr, 0, T, 1, W, nullptr, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_column_flip_w512(const float2 *spec, float2 *g, const int8_t *sign, int t0,
                                    int nt, int D, int H, int W, const int2 *live,
                                    cudaStream_t s) {
  switch (H) {
    case 128: return column_w512<128, true>(spec, g, sign, t0, nt, D, W, live, s);
    case 256: return column_w512<256, true>(spec, g, sign, t0, nt, D, W, live, s);
    case 384: return column_w512<384, true>(spec, g, sign, t0, nt, D, W, live, s);
    case 512: return column_w512<512, true>(spec, g, sign, t0, nt, D, W, live, s);
  }
  return cudaErrorInvalidValue;
}

template <int N, bool SPECTRA, bool RAMP, bool STAGED, bool F16>
static cudaError_t row_w512(const RowStageArgs &a, cudaStream_t s) {
  FftPlan pN, p2N;
  if (!make_fft_plan(N, &pN) || !make_fft_plan(2 * N, &p2N)) return cudaErrorInvalidValue;
  constexpr int PPB = 4 * WarpFftShape<N>::TPW;
  const long npairs = (long)a.nt * a.D * row_pairs(a);
  if (npairs == 0) return cudaSuccess;
  k_row_w512<N, SPECTRA, RAMP, STAGED, F16><<<(unsigned)((npairs + PPB - 1) / PPB), 128, 0, s>>>(
      a, pN.roots, p2N.roots);
  return cudaGetLastError();
}

template <int N>
static cudaError_t row_w512_dispatch(const RowStageArgs &a, cudaStream_t s) {
  const bool sp = a.input_spectra != 0, rm = a.ramp != 0, st = a.out_staged != 0;
  const bool h = a.staging != kStageF32;
  if (sp && rm && st && !h) return row_w512<N, true, true, true, false>(a, s);
  if (sp && rm && st && h) return row_w512<N, true, true, true, true>(a, s);
  if (!sp && rm && st && !h) return row_w512<N, false, true, true, false>(a, s);
  if (!sp && rm && st && h) return row_w512<N, false, true, true, true>(a, s);
  if (sp && !rm && !st) return row_w512<N, true, false, false, false>(a, s);
  if (!sp && rm && !st) return row_w512<N, false, true, false, false>(a, s);
  return cudaErrorInvalidValue;
}

cudaError_t launch_row_stage_w512(const RowStageArgs &a, cudaStream_t s) {
  switch (a.N) {
    case 128: return row_w512_dispatch<128>(a, s);
    case 256: return row_w512_dispatch<256>(a, s);
    case 384: return row_w512_dispatch<384>(a, s);
    case 512: return row_w512_dispatch<512>(a, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace gnc
