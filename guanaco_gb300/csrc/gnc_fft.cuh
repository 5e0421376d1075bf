// Shared-memory mixed-radix FFT engine for the correction and ramp-filter
// kernels (sm_103a).
//
// Formulation: Stockham autosort, decimation in time.  One stage of radix R
// over n points, with Ns the product of the radices already applied:
//   for j in [0, n/R):  v[r] = x[j + r*n/R] * w^(r*(j mod Ns)*n/(Ns*R))
//                       v    = DFT_R(v)
//                       y[(j/Ns)*Ns*R + (j mod Ns) + r*Ns] = v[r]
// The result is in natural order after the last stage.  Forward uses
// exp(-2*pi*i/n), inverse exp(+2*pi*i/n); neither is normalised -- the same
// conventions as the FFTW/cuFFT calls the reference makes
// (src/libguanaco/fft.cpp:38-71, src/libguanaco/fft.cu:40-85).
//
// A batch of sequences lives in shared memory; element e of sequence s is
// at buf[s*seq_stride + e*elem_stride].  Stages ping-pong between two
// buffers of the same layout; the caller gets back the one holding the result.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gnc {

constexpr int kMaxStages = 20;
constexpr int kMaxRadix = 16;

// Factorisation of one transform length, passed to kernels by value.
struct FftPlan {
  int n;
  int nstage;
  int radix[kMaxStages];
  const float2 *roots;  // n values exp(-2*pi*i*k/n), float, in global memory
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }
// multiply by s*i where s = +1 (inverse) or -1 (forward)
template <bool INV>
__device__ __forceinline__ float2 mul_si(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <bool INV>
__device__ __forceinline__ float2 root(const float2 *__restrict__ roots, int k) {
  float2 w = __ldg(roots + k);
  return INV ? make_float2(w.x, -w.y) : w;
}

// ---- DFT kernels of small length, in registers --------------------------
template <int R, bool INV>
struct Dft;

template <bool INV>
struct Dft<2, INV> {
  __device__ __forceinline__ static void run(float2 *v, const float2 *, int) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <bool INV>
struct Dft<3, INV> {
  __device__ __forceinline__ static void run(float2 *v, const float2 *, int) {
    const float h = 0.8660254037844386f;  // sin(2*pi/3)
    float2 t = cadd(v[1], v[2]);
    float2 a = make_float2(v[0].x - 0.5f * t.x, v[0].y - 0.5f * t.y);
    float2 b = mul_si<INV>(cscale(csub(v[1], v[2]), h));
    v[0] = cadd(v[0], t);
    v[1] = cadd(a, b);
    v[2] = csub(a, b);
  }
};

template <bool INV>
struct Dft<4, INV> {
  __device__ __forceinline__ static void run(float2 *v, const float2 *, int) {
    float2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    float2 c = cadd(v[1], v[3]), d = mul_si<INV>(csub(v[1], v[3]));
    v[0] = cadd(a, c);
    v[2] = csub(a, c);
    v[1] = cadd(b, d);
    v[3] = csub(b, d);
  }
};

template <bool INV>
struct Dft<5, INV> {
  __device__ __forceinline__ static void run(float2 *v, const float2 *, int) {
    const float c1 = 0.30901699437494745f, c2 = -0.8090169943749475f;
    const float s1 = 0.9510565162951535f, s2 = 0.5877852522924731f;
    float2 p1 = cadd(v[1], v[4]), m1 = csub(v[1], v[4]);
    float2 p2 = cadd(v[2], v[3]), m2 = csub(v[2], v[3]);
    float2 x0 = v[0];
    float2 a1 = make_float2(x0.x + c1 * p1.x + c2 * p2.x, x0.y + c1 * p1.y + c2 * p2.y);
    float2 a2 = make_float2(x0.x + c2 * p1.x + c1 * p2.x, x0.y + c2 * p1.y + c1 * p2.y);
    float2 b1 = mul_si<INV>(make_float2(s1 * m1.x + s2 * m2.x, s1 * m1.y + s2 * m2.y));
    float2 b2 = mul_si<INV>(make_float2(s2 * m1.x - s1 * m2.x, s2 * m1.y - s1 * m2.y));
    v[0] = cadd(x0, cadd(p1, p2));
    v[1] = cadd(a1, b1);
    v[4] = csub(a1, b1);
    v[2] = cadd(a2, b2);
    v[3] = csub(a2, b2);
  }
};

template <bool INV>
struct Dft<8, INV> {
  __device__ __forceinline__ static void run(float2 *v, const float2 *, int) {
    const float r = 0.7071067811865476f;
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, INV>::run(e, nullptr, 0);
    Dft<4, INV>::run(o, nullptr, 0);
    // w8^q for q = 1..3 with sign s: w8 = r(1 + s i), w8^2 = s i, w8^3 = r(-1 + s i)
    float2 o1 = o[1], o3 = o[3];
    float2 t1 = INV ? make_float2(r * (o1.x - o1.y), r * (o1.x + o1.y))
                    : make_float2(r * (o1.x + o1.y), r * (o1.y - o1.x));
    float2 t2 = mul_si<INV>(o[2]);
    float2 t3 = INV ? make_float2(-r * (o3.x + o3.y), r * (o3.x - o3.y))
                    : make_float2(r * (o3.y - o3.x), -r * (o3.x + o3.y));
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], t1);
    v[5] = csub(e[1], t1);
    v[2] = cadd(e[2], t2);
    v[6] = csub(e[2], t2);
    v[3] = cadd(e[3], t3);
    v[7] = csub(e[3], t3);
  }
};

// Any other radix up to kMaxRadix: direct O(R^2) DFT using the plan's roots
// (exp(-2*pi*i*r*q/R) = roots[((r*q) mod R) * n/R]).
template <bool INV>
__device__ __forceinline__ void dft_generic(float2 *v, int R, const float2 *roots, int n) {
  float2 out[kMaxRadix];
  const int step = n / R;
  for (int q = 0; q < R; ++q) {
    float2 s = v[0];
    for (int r = 1; r < R; ++r) s = cadd(s, cmul(v[r], root<INV>(roots, ((r * q) % R) * step)));
    out[q] = s;
  }
  for (int q = 0; q < R; ++q) v[q] = out[q];
}

// One Stockham stage with a compile-time radix R (R = 0: generic radix).
// SEQ_FAST: consecutive work items walk the sequences first (column tiles,
// elem_stride = tile width); otherwise they walk elements first (rows).
template <int R, bool INV, bool SEQ_FAST>
__device__ __forceinline__ void fft_stage(const float2 *__restrict__ src, float2 *__restrict__ dst,
                                          int n, int rad, int Ns, const float2 *__restrict__ roots,
                                          int elem_stride, int nseq, int seq_stride, int tid,
                                          int nthr) {
  const int RR = R > 0 ? R : rad;
  const int nR = n / RR;
  const int tstep = n / (Ns * RR);
  const int total = nR * nseq;
  for (int w = tid; w < total; w += nthr) {
    int s, j;
    if (SEQ_FAST) {
      s = w % nseq;
      j = w / nseq;
    } else {
      j = w % nR;
      s = w / nR;
    }
    const float2 *in = src + s * seq_stride;
    float2 *out = dst + s * seq_stride;
    float2 v[R > 0 ? R : kMaxRadix];
#pragma unroll
    for (int r = 0; r < (R > 0 ? R : kMaxRadix); ++r) {
      if (R > 0 || r < RR) v[r] = in[(j + r * nR) * elem_stride];
    }
    const int jm = j % Ns;
    if (jm != 0) {
      const int base = jm * tstep;
#pragma unroll
      for (int r = 1; r < (R > 0 ? R : kMaxRadix); ++r) {
        if (R > 0 || r < RR) v[r] = cmul(v[r], root<INV>(roots, r * base));
      }
    }
    if (R > 0)
      Dft<(R > 0 ? R : 2), INV>::run(v, roots, n);
    else
      dft_generic<INV>(v, RR, roots, n);
    const int ob = (j - jm) * RR + jm;
#pragma unroll
    for (int r = 0; r < (R > 0 ? R : kMaxRadix); ++r) {
      if (R > 0 || r < RR) out[(ob + r * Ns) * elem_stride] = v[r];
    }
  }
}

// Full transform of a batch of sequences.  Both buffers must hold the batch
// in the same layout; the result is returned (it is buf_a when the number of
// stages is even).  Contains __syncthreads(): every thread of the block must
// call it with the same arguments.
template <bool INV, bool SEQ_FAST>
__device__ float2 *fft_batch(float2 *buf_a, float2 *buf_b, const FftPlan &p, int elem_stride,
                             int nseq, int seq_stride) {
  const int tid = threadIdx.x, nthr = blockDim.x;
  float2 *src = buf_a, *dst = buf_b;
  int Ns = 1;
  for (int st = 0; st < p.nstage; ++st) {
    const int R = p.radix[st];
    switch (R) {
      case 2: fft_stage<2, INV, SEQ_FAST>(src, dst, p.n, 2, Ns, p.roots, elem_stride, nseq, seq_stride, tid, nthr); break;
      case 3: fft_stage<3, INV, SEQ_FAST>(src, dst, p.n, 3, Ns, p.roots, elem_stride, nseq, seq_stride, tid, nthr); break;
      case 4: fft_stage<4, INV, SEQ_FAST>(src, dst, p.n, 4, Ns, p.roots, elem_stride, nseq, seq_stride, tid, nthr); break;
      case 5: fft_stage<5, INV, SEQ_FAST>(src, dst, p.n, 5, Ns, p.roots, elem_stride, nseq, seq_stride, tid, nthr); break;
      case 8: fft_stage<8, INV, SEQ_FAST>(src, dst, p.n, 8, Ns, p.roots, elem_stride, nseq, seq_stride, tid, nthr); break;
      default: fft_stage<0, INV, SEQ_FAST>(src, dst, p.n, R, Ns, p.roots, elem_stride, nseq, seq_stride, tid, nthr); break;
    }
    __syncthreads();
    float2 *t = src;
    src = dst;
    dst = t;
    Ns *= R;
  }
  return src;
}

}  // namespace gnc
