// Row stage: inverse row transform of the corrected half spectra, ramp filter
// and staging for the backprojector.
//
// Ramp filter reference: guanaco::Filter (src/libguanaco/filter.cpp:30-97,
// src/libguanaco/filter.cu:144-202): each row is zero padded from N to 2N,
// transformed, bin k multiplied by w_k = k / N for k <= N and w_{2N-k}
// above, transformed back, and the first N samples divided by 2N are kept.
//
// Two real rows travel as one complex row (row a in the real part, row b in
// the imaginary part).  The ramp is real and even, so it maps the real and
// imaginary parts independently and the pair is filtered exactly as two
// separate rows would be.
#include "gnc_common.cuh"

namespace gnc {

template <bool SPECTRA, bool RAMP, bool STAGED, bool F16>
__global__ void k_row_stage(RowStageArgs a, FftPlan planN, FftPlan plan2N, int rp) {
  extern __shared__ float2 smem[];
  __shared__ unsigned int s_max[2 * 8];
  const int N = a.N;
  const int L = RAMP ? 2 * N : N;
  const int Y2 = row_pairs(a);  // row pairs of this launch
  const long npairs = (long)a.nt * a.D * Y2;
  const long P0 = (long)blockIdx.x * rp;
  const int np = (int)min((long)rp, npairs - P0);
  float2 *bufa = smem;
  float2 *bufb = smem + rp * L;

  // ---- load one complex row per pair --------------------------------------
  for (int i = threadIdx.x; i < rp * N; i += blockDim.x) {
    int s = i / N, k = i - s * N;
    float2 z = make_float2(0.f, 0.f);
    if (s < np) {
      long P = P0 + s;
      int tl = (int)(P / ((long)a.D * Y2));
      int rem = (int)(P - (long)tl * a.D * Y2);
      int d = rem / Y2, y2 = a.y2_begin + (rem - d * Y2);
      int ya = 2 * y2;
      if (!slab_live(a.live, a.t0 + tl, d)) {  // no voxel reads it: zeros, not stored
        bufa[s * L + k] = z;
        continue;
      }
      bool hb = ya + 1 < a.H;
      if (SPECTRA) {
        const int half = N / 2;
        const float2 *ga = a.g + (((size_t)tl * a.D + d) * a.H + ya) * half;
        const float2 *gb = ga + half;
        if (k == 0) {
          float2 pa = ga[0], pb = hb ? gb[0] : make_float2(0.f, 0.f);
          z = make_float2(pa.x, pb.x);
        } else if (k == half) {
          float2 pa = ga[0], pb = hb ? gb[0] : make_float2(0.f, 0.f);
          z = make_float2(pa.y, pb.y);
        } else if (k < half) {
          float2 g1 = ga[k], g2 = hb ? gb[k] : make_float2(0.f, 0.f);
          z = make_float2(g1.x - g2.y, g1.y + g2.x);
        } else {
          float2 g1 = ga[N - k], g2 = hb ? gb[N - k] : make_float2(0.f, 0.f);
          z = make_float2(g1.x + g2.y, g2.x - g1.y);
        }
      } else {
        const float *base = a.rows + ((size_t)(a.t0 + tl) * a.D + d) * a.plane_stride;
        float va = base[(size_t)ya * a.row_stride + k];
        float vb = hb ? base[(size_t)(ya + 1) * a.row_stride + k] : 0.f;
        z = make_float2(va, vb);
      }
    }
    bufa[s * L + k] = z;
  }
  __syncthreads();
  float2 *cur = bufa, *oth = bufb;
  if (SPECTRA) {
    cur = fft_batch<true, false>(bufa, bufb, planN, 1, rp, L);
    oth = cur == bufa ? bufb : bufa;
  }
  float out_scale = 1.0f;
  if (RAMP) {
    for (int i = threadIdx.x; i < rp * N; i += blockDim.x) {
      int s = i / N, k = i - s * N;
      cur[s * L + N + k] = make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 *f = fft_batch<false, false>(cur, oth, plan2N, 1, rp, L);
    const float fN = (float)N;
    for (int i = threadIdx.x; i < rp * L; i += blockDim.x) {
      int k = i % L;
      int kk = k <= N ? k : L - k;
      float w = (float)kk / fN;
      f[i] = make_float2(f[i].x * w, f[i].y * w);
    }
    __syncthreads();
    float2 *o = f == bufa ? bufb : bufa;
    cur = fft_batch<true, false>(f, o, plan2N, 1, rp, L);
    out_scale = (float)L;  // the reference divides by the padded length
  }

  // ---- output --------------------------------------------------------------
  if (STAGED && F16) {
    if (threadIdx.x < 2 * rp) s_max[threadIdx.x] = 0u;
    __syncthreads();
  }
  for (int s = 0; s < np; ++s) {
    long P = P0 + s;
    int tl = (int)(P / ((long)a.D * Y2));
    int rem = (int)(P - (long)tl * a.D * Y2);
    int d = rem / Y2, y2 = a.y2_begin + (rem - d * Y2);
    int t = a.t0 + tl;
    int ya = 2 * y2;
    bool hb = ya + 1 < a.H;
    if (!slab_live(a.live, t, d)) continue;  // the same for every thread of the block
    float f = a.tilt_factor ? a.tilt_factor[t] : 1.0f;
    const float2 *row = cur + s * L;
    if (STAGED && !F16) {
      float2 *dst = (float2 *)a.staged + (((size_t)y2 * a.D + d) * a.T + t) * N;
      for (int n = threadIdx.x; n < N; n += blockDim.x) {
        float2 v = row[n];
        if (RAMP) v = make_float2(v.x / out_scale, v.y / out_scale);
        dst[n] = make_float2(v.x * f, v.y * f);
      }
    } else if (STAGED && F16 && a.staging == kStageF16T) {
      // plain FP16 rows scaled by the tilt's 2^e(t)
      const float sc = f16t_scale(a, t);
      __half *da = f16t_row(a, d, t, ya);
      for (int n = threadIdx.x; n < N; n += blockDim.x) {
        float2 v = row[n];
        if (RAMP) v = make_float2(v.x / out_scale, v.y / out_scale);
        da[n] = __float2half_rn(v.x * f * sc);
        if (hb) da[N + n] = __float2half_rn(v.y * f * sc);
      }
    } else if (STAGED && F16) {
      float ma = 0.f, mb = 0.f;
      for (int n = threadIdx.x; n < N; n += blockDim.x) {
        float2 v = row[n];
        if (RAMP) v = make_float2(v.x / out_scale, v.y / out_scale);
        ma = fmaxf(ma, fabsf(v.x * f));
        mb = fmaxf(mb, fabsf(v.y * f));
      }
      unsigned ua = __reduce_max_sync(0xffffffffu, __float_as_uint(ma));
      unsigned ub = __reduce_max_sync(0xffffffffu, __float_as_uint(mb));
      if ((threadIdx.x & 31) == 0) {
        atomicMax(&s_max[2 * s], ua);
        atomicMax(&s_max[2 * s + 1], ub);
      }
      __syncthreads();
      // 2^e brings the row maximum into [2^13, 2^14): full FP16 precision,
      // four binades of headroom below the FP16 maximum.
      int ea = 0, eb = 0;
      float mxa = __uint_as_float(s_max[2 * s]), mxb = __uint_as_float(s_max[2 * s + 1]);
      if (mxa > 0.f) ea = 13 - ilogbf(mxa);
      if (mxb > 0.f) eb = 13 - ilogbf(mxb);
      ea = max(-120, min(120, ea));
      eb = max(-120, min(120, eb));
      float sa = __int_as_float((127 + ea) << 23), sb = __int_as_float((127 + eb) << 23);
      size_t rowi = ((size_t)y2 * a.D + d) * a.T + t;
      uint2 *dst = (uint2 *)a.staged + rowi * N;
      // the output value of pixel n (n + 1 past the end: the last pixel itself)
      auto value = [&](int n) {
        float2 v = row[n < N ? n : N - 1];
        if (RAMP) v = make_float2(v.x / out_scale, v.y / out_scale);
        return make_float2(v.x * f * sa, v.y * f * sb);
      };
      for (int n = threadIdx.x; n < N; n += blockDim.x)
        dst[n] = staged_record_f16(value(n), value(n + 1));
      if (threadIdx.x == 0) {
        a.row_exp[2 * rowi] = (int8_t)ea;
        a.row_exp[2 * rowi + 1] = (int8_t)eb;
      }
    } else {
      float *da = a.out_rows + (((size_t)tl * a.D + d) * a.H + ya) * N;
      for (int n = threadIdx.x; n < N; n += blockDim.x) {
        float2 v = row[n];
        if (RAMP) v = make_float2(v.x / out_scale, v.y / out_scale);
        da[n] = v.x * f;
        if (hb) da[N + n] = v.y * f;
      }
    }
  }
}

template <bool SPECTRA, bool RAMP, bool STAGED, bool F16>
static cudaError_t launch_variant(const RowStageArgs &a, cudaStream_t s) {
  const int N = a.N;
  const int L = RAMP ? 2 * N : N;
  FftPlan pN{}, p2N{};
  if (SPECTRA && !make_fft_plan(N, &pN)) return cudaErrorInvalidValue;
  if (RAMP && !make_fft_plan(2 * N, &p2N)) return cudaErrorInvalidValue;
  int rp = L >= 4096 ? 1 : 4096 / L;
  if (rp > 8) rp = 8;
  const long npairs = (long)a.nt * a.D * row_pairs(a);
  if (rp > npairs) rp = (int)npairs;
  if (rp < 1) rp = 1;
  size_t smem = 2ull * rp * L * sizeof(float2);
  auto kern = k_row_stage<SPECTRA, RAMP, STAGED, F16>;
  if (cudaError_t e_attr = ensure_dynamic_smem<k_row_stage<SPECTRA, RAMP, STAGED, F16>>(200 * 1024)) return e_attr;
  long blocks = (npairs + rp - 1) / rp;
  kern<<<(unsigned)blocks, 256, smem, s>>>(a, pN, p2N, rp);
  return cudaGetLastError();
}

cudaError_t launch_row_stage(const RowStageArgs &a, cudaStream_t s) {
  if (a.N == 1024) return launch_row_stage_w1024(a, s);
  if (a.N == 4096) return launch_row_stage_b4096(a, s);
  if (a.N == 128 || a.N == 256 || a.N == 384 || a.N == 512) return launch_row_stage_w512(a, s);
  if (pow2_fast(a.N)) return launch_row_stage_p2(a, s);
  const bool sp = a.input_spectra != 0, rm = a.ramp != 0, st = a.out_staged != 0;
  const bool h = a.staging != kStageF32;
  if (sp && rm && st && !h) return launch_variant<true, true, true, false>(a, s);
  if (sp && rm && st && h) return launch_variant<true, true, true, true>(a, s);
  if (!sp && rm && st && !h) return launch_variant<false, true, true, false>(a, s);
  if (!sp && rm && st && h) return launch_variant<false, true, true, true>(a, s);
  if (sp && !rm && !st) return launch_variant<true, false, false, false>(a, s);
  if (!sp && rm && !st) return launch_variant<false, true, false, false>(a, s);
  return cudaErrorInvalidValue;
}

}  // namespace gnc
