// Correction and ramp-filter kernels for power-of-two sizes: the row transform
// of the raw projections for 256 .. 4096, the column and row stages for 2048
// (those of 256, 512, 1024 and 4096 use the register-transform kernels of
// gnc_w512_kernels.cu, gnc_w1024_kernels.cu and gnc_b4096_kernels.cu), built on the shared-memory
// FFT of gnc_fft_pow2.cuh.  Same results as the generic kernels of
// gnc_correct.cu / gnc_ramp.cu (up to float rounding), which keep serving
// every other size.
//
// Ramp filter without 2N-point transforms.  For a row c of N samples (two
// real rows packed as one complex row) the reference zero pads to 2N,
// transforms, multiplies bin K by w_K and keeps the first N samples of the
// inverse divided by 2N (src/libguanaco/filter.cpp:61-97).  The even bins of
// the padded transform are the N-point transform of c, the odd bins the
// N-point transform of c[n] exp(-i pi n / N); splitting the inverse the same
// way gives, for n < N,
//   y[n] = (1/2N) [ IFFT_N(w_even FFT_N(c))[n]
//                   + exp(+i pi n / N) IFFT_N(w_odd FFT_N(c exp(-i pi n/N)))[n] ]
// with w_even[k] = w_{2k}, w_odd[k] = w_{2k+1}: four N-point transforms.  When
// the row arrives as its N-point spectrum Z (c = IFFT_N(Z), so FFT_N(c) = N Z)
// the first term is (1/2) IFFT_N(w_even Z).
#include "gnc_common.cuh"
#include "gnc_fft_pow2.cuh"

namespace gnc {

namespace {

__device__ __forceinline__ float ramp_w(int K, int N) {  // filter.cpp:38-41, w_K = K / N
  const int kk = K <= N ? K : 2 * N - K;
  return (float)kk / (float)N;
}

struct BlockSync {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};

}  // namespace

bool pow2_fast(long n) { return n >= 256 && n <= 4096 && (n & (n - 1)) == 0; }

// ---------------------------------------------------------------------------
// Row transform of the raw projections (pairs of rows as one complex row).
// ---------------------------------------------------------------------------
template <int W>
__global__ void __launch_bounds__(256) k_rfft_rows_p2(const float *__restrict__ proj,
                                                      float2 *__restrict__ spec, int H,
                                                      const float2 *__restrict__ roots) {
  using P = Pow2<W>;
  constexpr int GPB = 256 / P::NT;  // row pairs per block
  __shared__ float2 buf[GPB][P::PADDED];
  const int g = threadIdx.x / P::NT, j = threadIdx.x % P::NT;
  const int t = blockIdx.y;
  const int npair = (H + 1) / 2;
  const int pair = blockIdx.x * GPB + g;
  const bool active = pair < npair;
  const int ya = 2 * min(pair, npair - 1), yb = ya + 1;
  const float *img = proj + (size_t)t * H * W;
  float2 *z = buf[g];
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    const int n = j + m * P::NT;
    const float va = img[(size_t)ya * W + n];
    const float vb = yb < H ? img[(size_t)yb * W + n] : 0.f;
    z[fpad(n)] = make_float2(va, vb);
  }
  __syncthreads();
  fft_pow2<W, false>(z, j, roots, BlockSync());
  // unpack: A[k] = (Z[k] + conj Z[-k]) / 2, B[k] = -i (Z[k] - conj Z[-k]) / 2
  constexpr int half = W / 2;
  float2 *out = spec + (size_t)t * H * half;
  if (active) {
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const int k = j + m * P::NT;
      float2 A, B;
      if (k == 0) {
        const float2 z0 = z[fpad(0)], zn = z[fpad(half)];
        A = make_float2(z0.x, zn.x);
        B = make_float2(z0.y, zn.y);
      } else {
        const float2 zk = z[fpad(k)], zm = z[fpad(W - k)];
        A = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
        B = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
      }
      out[(size_t)ya * half + k] = A;
      if (yb < H) out[(size_t)yb * half + k] = B;
    }
  }
}

// ---------------------------------------------------------------------------
// Column transforms.  A block owns C = 256 / (H/16) adjacent columns; the
// block loads the H x C tile with consecutive threads on consecutive columns,
// then each group of H/16 threads transforms one column.
// FLIP: per-slab phase flip before an inverse transform (see gnc_correct.cu
// for the packed DC/Nyquist column).
// ---------------------------------------------------------------------------
// Columns per block: 256 threads for short columns; tall columns (2048)
// take 1024 threads so that a block still reads 32 or 64 contiguous
// bytes of every row (four or eight columns).
template <int H>
struct ColTile {
  static constexpr int NT = Pow2<H>::NT;
  static constexpr int THREADS = H >= 2048 ? 1024 : 256;
  static constexpr int C = THREADS / NT;
  static constexpr size_t SMEM = (size_t)C * Pow2<H>::PADDED * sizeof(float2);
};

template <int H, bool FLIP>
__global__ void __launch_bounds__(ColTile<H>::THREADS) k_column_p2(
    const float2 *__restrict__ src, float2 *__restrict__ dst, const int8_t *__restrict__ sign,
    int t0, int D, int W, const float2 *__restrict__ roots, const int2 *__restrict__ live) {
  using P = Pow2<H>;
  constexpr int C = ColTile<H>::C;
  constexpr int NTH = ColTile<H>::THREADS;
  extern __shared__ float2 smem_col[];
  float2(*buf)[P::PADDED] = reinterpret_cast<float2(*)[P::PADDED]>(smem_col);
  const int g = threadIdx.x / P::NT, j = threadIdx.x % P::NT;
  const int half = W / 2;
  const int c0 = blockIdx.x * C;
  const int d = FLIP ? blockIdx.y : 0;
  const int tl = blockIdx.z;
  const int t = t0 + tl;
  if (FLIP && !slab_live(live, t, d)) return;  // no voxel reads this (tilt, slab)
  const float2 *F = src + (size_t)t * H * half;
  const int sw = half + 1;
  const int8_t *sg = FLIP ? sign + (size_t)d * H * sw : nullptr;
  for (int i = threadIdx.x; i < H * C; i += NTH) {
    const int ky = i / C, c = i % C;
    const int kx = c0 + c;
    float2 r = make_float2(0.f, 0.f);
    if (kx < half) {
      const float2 v = F[(size_t)ky * half + kx];
      if (!FLIP) {
        r = v;
      } else if (kx == 0) {
        const float2 m = F[(size_t)((H - ky) % H) * half];
        const float sdc = 0.5f * (float)sg[(size_t)ky * sw];
        const float sny = 0.5f * (float)sg[(size_t)ky * sw + half];
        const float a = 0.5f * (sdc + sny), b = 0.5f * (sdc - sny);
        r = make_float2(a * v.x + b * m.x, a * v.y - b * m.y);
      } else {
        const float f = 0.5f * (float)sg[(size_t)ky * sw + kx];
        r = make_float2(f * v.x, f * v.y);
      }
    }
    buf[c][fpad(ky)] = r;
  }
  __syncthreads();
  fft_pow2<H, FLIP>(buf[g], j, roots, BlockSync());
  float2 *out = FLIP ? dst + ((size_t)tl * D + d) * H * half : dst + (size_t)t * H * half;
  for (int i = threadIdx.x; i < H * C; i += NTH) {
    const int ky = i / C, c = i % C;
    const int kx = c0 + c;
    if (kx < half) out[(size_t)ky * half + kx] = buf[c][fpad(ky)];
  }
}

// ---------------------------------------------------------------------------
// Row stage (ramp filter, optional spectra input, staged or plain output).
// One group of N/16 threads per row pair, 256 / (N/16) pairs per block.
// ---------------------------------------------------------------------------
template <int N, bool SPECTRA, bool RAMP, bool STAGED, bool F16>
__global__ void __launch_bounds__(256) k_row_p2(RowStageArgs a, const float2 *__restrict__ rootsN,
                                                const float2 *__restrict__ roots2N) {
  using P = Pow2<N>;
  constexpr int GPB = 256 / P::NT;
  constexpr int NB = RAMP ? 2 : 1;
  extern __shared__ float2 smem_p2[];
  __shared__ unsigned s_max[GPB][2];
  const int g = threadIdx.x / P::NT, j = threadIdx.x % P::NT;
  float2 *zb = smem_p2 + (size_t)(g * NB) * P::PADDED;  // c, then the odd path
  float2 *eb = zb + P::PADDED;                          // the even path
  const int Y2 = row_pairs(a);  // row pairs of this launch
  const long npairs = (long)a.nt * a.D * Y2;
  long pair = (long)blockIdx.x * GPB + g;
  bool active = pair < npairs;
  if (!active) pair = npairs - 1;
  const int tl = (int)(pair / ((long)a.D * Y2));
  const int rem = (int)(pair - (long)tl * a.D * Y2);
  const int d = rem / Y2, y2 = a.y2_begin + (rem - d * Y2);
  const int t = a.t0 + tl;
  // a (tilt, slab) no voxel reads is not stored; a block with none to store
  // returns before its first barrier
  active = active && slab_live(a.live, t, d);
  if (!__syncthreads_or(active)) return;
  const int ya = 2 * y2;
  const bool hb = ya + 1 < a.H;
  constexpr int half = N / 2;

  // ---- load
  if (SPECTRA) {
    const float2 *ga = a.g + (((size_t)tl * a.D + d) * a.H + ya) * half;
    const float2 *gbp = ga + half;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const int k = j + m * P::NT;  // 0 .. N/2 - 1
      const float2 pa = ga[k];
      const float2 pb = hb ? gbp[k] : make_float2(0.f, 0.f);
      if (k == 0) {
        const float2 z0 = make_float2(pa.x, pb.x), zn = make_float2(pa.y, pb.y);
        zb[fpad(0)] = z0;
        zb[fpad(half)] = zn;
        if (RAMP) {
          eb[fpad(0)] = make_float2(0.f, 0.f);  // w_0 = 0
          const float wn = ramp_w(N, N);
          eb[fpad(half)] = make_float2(wn * zn.x, wn * zn.y);
        }
      } else {
        const float2 zk = make_float2(pa.x - pb.y, pa.y + pb.x);
        const float2 zm = make_float2(pa.x + pb.y, pb.x - pa.y);
        zb[fpad(k)] = zk;
        zb[fpad(N - k)] = zm;
        if (RAMP) {
          const float wk = ramp_w(2 * k, N), wm = ramp_w(2 * (N - k), N);
          eb[fpad(k)] = make_float2(wk * zk.x, wk * zk.y);
          eb[fpad(N - k)] = make_float2(wm * zm.x, wm * zm.y);
        }
      }
    }
  } else {
    const float *base = a.rows + ((size_t)(a.t0 + tl) * a.D + d) * a.plane_stride;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int n = j + m * P::NT;
      const float va = base[(size_t)ya * a.row_stride + n];
      const float vb = hb ? base[(size_t)(ya + 1) * a.row_stride + n] : 0.f;
      const float2 c = make_float2(va, vb);
      zb[fpad(n)] = c;
      if (RAMP) eb[fpad(n)] = c;
    }
  }
  __syncthreads();
  const BlockSync sync;
  if (SPECTRA) {
    fft_pow2<N, true>(zb, j, rootsN, sync);             // c = IFFT(Z)
    if (RAMP) fft_pow2<N, true>(eb, j, rootsN, sync);   // u = IFFT(w_even Z)
  } else if (RAMP) {
    fft_pow2<N, false>(eb, j, rootsN, sync);            // FFT(c)
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int k = j + m * P::NT;
      const float w = ramp_w(2 * k, N);
      const float2 v = eb[fpad(k)];
      eb[fpad(k)] = make_float2(w * v.x, w * v.y);
    }
    __syncthreads();
    fft_pow2<N, true>(eb, j, rootsN, sync);             // IFFT(w_even FFT(c))
  }
  if (RAMP) {
    // odd bins: FFT(c exp(-i pi n / N)), times w_odd, inverse
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int n = j + m * P::NT;
      zb[fpad(n)] = cmul(zb[fpad(n)], __ldg(roots2N + n));
    }
    __syncthreads();
    fft_pow2<N, false>(zb, j, rootsN, sync);
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int k = j + m * P::NT;
      const float w = ramp_w(2 * k + 1, N);
      const float2 v = zb[fpad(k)];
      zb[fpad(k)] = make_float2(w * v.x, w * v.y);
    }
    __syncthreads();
    fft_pow2<N, true>(zb, j, rootsN, sync);
  }

  // ---- combine and write
  const float f = a.tilt_factor ? a.tilt_factor[t] : 1.0f;
  const float ea = SPECTRA ? 0.5f : 1.0f / (float)(2 * N);
  const float eo = 1.0f / (float)(2 * N);
  float2 yv[16];
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    const int n = j + m * P::NT;
    float2 y = zb[fpad(n)];
    if (RAMP) {
      const float2 tw = __ldg(roots2N + n);  // exp(-i pi n / N); conjugate below
      const float2 v = cmul(make_float2(tw.x, -tw.y), y);
      const float2 u = eb[fpad(n)];
      y = make_float2(ea * u.x + eo * v.x, ea * u.y + eo * v.y);
    }
    yv[m] = make_float2(y.x * f, y.y * f);
  }
  if (STAGED && !F16) {
    if (active) {
      float2 *dst = (float2 *)a.staged + (((size_t)y2 * a.D + d) * a.T + t) * N;
#pragma unroll
      for (int m = 0; m < 16; ++m) dst[j + m * P::NT] = yv[m];
    }
  } else if (STAGED && F16 && a.staging == kStageF16T) {
    // plain FP16 rows scaled by the tilt's 2^e(t) (the branch is uniform: no
    // barrier below is skipped by part of the block)
    if (active) {
      const float sc = f16t_scale(a, t);
      __half *da = f16t_row(a, d, t, ya);
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        da[j + m * P::NT] = __float2half_rn(yv[m].x * sc);
        if (hb) da[N + j + m * P::NT] = __float2half_rn(yv[m].y * sc);
      }
    }
  } else if (STAGED && F16) {
    // the records need pixel n + 1, held by another thread: exchange the
    // group's row pair through its (no longer needed) transform buffer
    __syncthreads();
#pragma unroll
    for (int m = 0; m < 16; ++m) zb[fpad(j + m * P::NT)] = yv[m];
    __syncthreads();
    float ma = 0.f, mb = 0.f;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      ma = fmaxf(ma, fabsf(yv[m].x));
      mb = fmaxf(mb, fabsf(yv[m].y));
    }
    if (j == 0) s_max[g][0] = s_max[g][1] = 0u;
    __syncthreads();
    // reduce within the group's lanes of this warp (a group is N/16 threads,
    // fewer than a warp for N < 512), then combine the warps of a group
    constexpr int LW = P::NT < 32 ? P::NT : 32;
#pragma unroll
    for (int o = LW / 2; o > 0; o >>= 1) {
      ma = fmaxf(ma, __shfl_xor_sync(0xffffffffu, ma, o));
      mb = fmaxf(mb, __shfl_xor_sync(0xffffffffu, mb, o));
    }
    if ((threadIdx.x & (LW - 1)) == 0) {
      atomicMax(&s_max[g][0], __float_as_uint(ma));
      atomicMax(&s_max[g][1], __float_as_uint(mb));
    }
    __syncthreads();
    // 2^e brings the row maximum into [2^13, 2^14): full FP16 precision with
    // headroom below the FP16 maximum
    const float mxa = __uint_as_float(s_max[g][0]), mxb = __uint_as_float(s_max[g][1]);
    int e_a = mxa > 0.f ? 13 - ilogbf(mxa) : 0;
    int e_b = mxb > 0.f ? 13 - ilogbf(mxb) : 0;
    e_a = max(-120, min(120, e_a));
    e_b = max(-120, min(120, e_b));
    const float sa = __int_as_float((127 + e_a) << 23), sb = __int_as_float((127 + e_b) << 23);
    if (active) {
      const size_t rowi = ((size_t)y2 * a.D + d) * a.T + t;
      uint2 *dst = (uint2 *)a.staged + rowi * N;
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        const int n = j + m * P::NT;
        const float2 v1 = n + 1 < N ? zb[fpad(n + 1)] : yv[m];
        dst[n] = staged_record_f16(make_float2(yv[m].x * sa, yv[m].y * sb),
                                   make_float2(v1.x * sa, v1.y * sb));
      }
      if (j == 0) {
        a.row_exp[2 * rowi] = (int8_t)e_a;
        a.row_exp[2 * rowi + 1] = (int8_t)e_b;
      }
    }
  } else if (active) {
    float *da = a.out_rows + (((size_t)tl * a.D + d) * a.H + ya) * N;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int n = j + m * P::NT;
      da[n] = yv[m].x;
      if (hb) da[N + n] = yv[m].y;
    }
  }
}

// ---------------------------------------------------------------- launchers
template <int W>
static cudaError_t rfft_rows_p2(const float *proj, float2 *spec, int T, int H, cudaStream_t s) {
  FftPlan p;
  if (!make_fft_plan(W, &p)) return cudaErrorInvalidValue;
  constexpr int GPB = 256 / Pow2<W>::NT;
  const int npair = (H + 1) / 2;
  dim3 grid((npair + GPB - 1) / GPB, T);
  k_rfft_rows_p2<W><<<grid, 256, 0, s>>>(proj, spec, H, p.roots);
  return cudaGetLastError();
}

cudaError_t launch_rfft_rows_p2(const float *proj, float2 *spec, int T, int H, int W,
                                cudaStream_t s) {
  switch (W) {
    case 256: return rfft_rows_p2<256>(proj, spec, T, H, s);
    case 512: return rfft_rows_p2<512>(proj, spec, T, H, s);
    case 2048: return rfft_rows_p2<2048>(proj, spec, T, H, s);
    case 4096: return rfft_rows_p2<4096>(proj, spec, T, H, s);
  }
  return cudaErrorInvalidValue;
}

template <int H, bool FLIP>
static cudaError_t column_p2(const float2 *src, float2 *dst, const int8_t *sign, int t0, int nt,
                             int D, int W, const int2 *live, cudaStream_t s) {
  FftPlan p;
  if (!make_fft_plan(H, &p)) return cudaErrorInvalidValue;
  using CT = ColTile<H>;
  if (cudaError_t e_attr = ensure_dynamic_smem<k_column_p2<H, FLIP>>((int)CT::SMEM)) return e_attr;
  const int half = W / 2;
  dim3 grid((half + CT::C - 1) / CT::C, FLIP ? D : 1, nt);
  k_column_p2<H, FLIP><<<grid, CT::THREADS, CT::SMEM, s>>>(src, dst, sign, t0, D, W, p.roots,
                                                            live);
  return cudaGetLastError();
}

cudaError_t launch_column_fft_p2(float2 *spec, int T, int H, int W, cudaStream_t s) {
  switch (H) {
    case 2048: return column_p2<2048, false>(spec, spec, nullptr, 0, T, 1, W, nullptr, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_column_flip_p2(const float2 *spec, float2 *g, const int8_t *sign, int t0,
                                  int nt, int D, int H, int W, const int2 *live, cudaStream_t s) {
  switch (H) {
    case 2048: return column_p2<2048, true>(spec, g, sign, t0, nt, D, W, live, s);
  }
  return cudaErrorInvalidValue;
}

template <int N, bool SPECTRA, bool RAMP, bool STAGED, bool F16>
static cudaError_t row_p2(const RowStageArgs &a, cudaStream_t s) {
  FftPlan pN, p2N;
  if (!make_fft_plan(N, &pN) || !make_fft_plan(2 * N, &p2N)) return cudaErrorInvalidValue;
  constexpr int GPB = 256 / Pow2<N>::NT;
  constexpr int NB = RAMP ? 2 : 1;
  const size_t smem = (size_t)GPB * NB * Pow2<N>::PADDED * sizeof(float2);
  auto kern = k_row_p2<N, SPECTRA, RAMP, STAGED, F16>;
  if (cudaError_t e_attr = ensure_dynamic_smem<k_row_p2<N, SPECTRA, RAMP, STAGED, F16>>((int)smem)) return e_attr;
  const long npairs = (long)a.nt * a.D * row_pairs(a);
  kern<<<(unsigned)((npairs + GPB - 1) / GPB), 256, smem, s>>>(a, pN.roots, p2N.roots);
  return cudaGetLastError();
}

template <int N>
static cudaError_t row_p2_dispatch(const RowStageArgs &a, cudaStream_t s) {
  const bool sp = a.input_spectra != 0, rm = a.ramp != 0, st = a.out_staged != 0;
  const bool h = a.staging != kStageF32;
  if (sp && rm && st && !h) return row_p2<N, true, true, true, false>(a, s);
  if (sp && rm && st && h) return row_p2<N, true, true, true, true>(a, s);
  if (!sp && rm && st && !h) return row_p2<N, false, true, true, false>(a, s);
  if (!sp && rm && st && h) return row_p2<N, false, true, true, true>(a, s);
  if (sp && !rm && !st) return row_p2<N, true, false, false, false>(a, s);
  if (!sp && rm && !st) return row_p2<N, false, true, false, false>(a, s);
  return cudaErrorInvalidValue;
}

cudaError_t launch_row_stage_p2(const RowStageArgs &a, cudaStream_t s) {
  switch (a.N) {
    case 2048: return row_p2_dispatch<2048>(a, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace gnc
