// Register-resident FFT for power-of-two lengths L = 16^a * r (r in 1, 2, 4, 8),
// L >= 256, used by the correction and ramp-filter kernels on their hot sizes.
//
// A transform is computed in place in shared memory by a group of L / 16
// threads.  Each pass is one Stockham autosort stage of radix 16 (or the final
// radix r): every thread loads 16 elements into registers, applies the stage
// twiddles, does a 16-point DFT (two layers of 4-point DFTs) and stores the
// results to their autosorted positions.  All loads of a pass happen before a
// barrier and all stores after it, so one buffer suffices.  Storage index i is
// padded to i + i / 16, which keeps both the strided reads and the scattered
// writes of every pass free of shared-memory bank conflicts.
//
// Conventions match the reference's FFTW/cuFFT calls: forward exp(-2 pi i/L),
// inverse exp(+2 pi i/L), unnormalised.
#pragma once

#include "gnc_fft.cuh"

namespace gnc {

__device__ __forceinline__ int fpad(int i) { return i + (i >> 4); }

template <int L>
struct Pow2 {
  static_assert(L >= 256 && (L & (L - 1)) == 0, "power of two >= 256");
  static constexpr int NT = L / 16;  // threads per transform
  static constexpr int PADDED = L + L / 16;
  static constexpr int log2(int v) { return v <= 1 ? 0 : 1 + log2(v / 2); }
  static constexpr int LOG = log2(L);
  static constexpr int NP16 = LOG / 4;               // radix-16 passes
  static constexpr int RLAST = 1 << (LOG - 4 * NP16);  // final radix (1: none)
};

// multiply by the 16th root power w16^m (forward sign; conjugated for inverse)
template <bool INV>
__device__ __forceinline__ float2 w16(float2 v, int m) {
  // cos/sin of 2*pi*m/16 for m = 0..9
  const float c[10] = {1.f, 0.92387953251128674f, 0.70710678118654752f, 0.38268343236508977f, 0.f,
                       -0.38268343236508977f, -0.70710678118654752f, -0.92387953251128674f, -1.f,
                       -0.92387953251128674f};
  const float s[10] = {0.f, 0.38268343236508977f, 0.70710678118654752f, 0.92387953251128674f, 1.f,
                       0.92387953251128674f, 0.70710678118654752f, 0.38268343236508977f, 0.f,
                       -0.38268343236508977f};
  // forward root exp(-i a) = (c, -s); inverse (c, s)
  const float cc = c[m], ss = INV ? s[m] : -s[m];
  return make_float2(v.x * cc - v.y * ss, v.x * ss + v.y * cc);
}

// 16-point DFT in registers: x[n] -> X[k] in natural order.
template <bool INV>
__device__ __forceinline__ void dft16(float2 *x) {
  float2 a[16];
  // layer 1: DFT4 over n1 for each n2 (inputs x[4 n1 + n2])
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    float2 v[4] = {x[n2], x[4 + n2], x[8 + n2], x[12 + n2]};
    Dft<4, INV>::run(v, nullptr, 0);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) a[n2 * 4 + k1] = v[k1];
  }
  // twiddles w16^(n2 k1)
#pragma unroll
  for (int n2 = 1; n2 < 4; ++n2)
#pragma unroll
    for (int k1 = 1; k1 < 4; ++k1) a[n2 * 4 + k1] = w16<INV>(a[n2 * 4 + k1], n2 * k1);
  // layer 2: DFT4 over n2 for each k1; X[k1 + 4 k2]
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    float2 v[4] = {a[k1], a[4 + k1], a[8 + k1], a[12 + k1]};
    Dft<4, INV>::run(v, nullptr, 0);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) x[k1 + 4 * k2] = v[k2];
  }
}

// Twiddle w^(k) from the L-point root table (exp(-2 pi i k / L)).
template <bool INV>
__device__ __forceinline__ float2 troot(const float2 *__restrict__ roots, int k) {
  float2 w = __ldg(roots + k);
  return INV ? make_float2(w.x, -w.y) : w;
}

// In-place transform of buf (padded layout) by threads j = 0 .. L/16 - 1 of a
// group.  SYNC() must synchronise (at least) the group; it is called twice
// per pass.  The caller synchronises before the first and after the last pass.
template <int L, bool INV, typename Sync>
__device__ __forceinline__ void fft_pow2(float2 *buf, int j, const float2 *__restrict__ roots,
                                         Sync sync) {
  using P = Pow2<L>;
  constexpr int Q = L / 16;
  int Ns = 1;
#pragma unroll
  for (int pass = 0; pass < P::NP16; ++pass) {
    float2 x[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) x[r] = buf[fpad(j + r * Q)];
    const int jm = j & (Ns - 1);
    if (pass > 0 && jm != 0) {
      // w^(r jm step), step = L / (16 Ns); powers 1..4 from the table, the rest by products
      const int base = jm * (L / (16 * Ns));
      const float2 w1 = troot<INV>(roots, base), w2 = troot<INV>(roots, 2 * base);
      const float2 w3 = troot<INV>(roots, 3 * base), w4 = troot<INV>(roots, 4 * base);
      const float2 w8 = troot<INV>(roots, 8 * base), w12 = troot<INV>(roots, 12 * base);
      float2 w[16];
      w[1] = w1; w[2] = w2; w[3] = w3; w[4] = w4;
      w[8] = w8; w[12] = w12;
      w[5] = cmul(w4, w1); w[6] = cmul(w4, w2); w[7] = cmul(w4, w3);
      w[9] = cmul(w8, w1); w[10] = cmul(w8, w2); w[11] = cmul(w8, w3);
      w[13] = cmul(w12, w1); w[14] = cmul(w12, w2); w[15] = cmul(w12, w3);
#pragma unroll
      for (int r = 1; r < 16; ++r) x[r] = cmul(x[r], w[r]);
    }
    dft16<INV>(x);
    sync();
    const int ob = (j - jm) * 16 + jm;
#pragma unroll
    for (int r = 0; r < 16; ++r) buf[fpad(ob + r * Ns)] = x[r];
    sync();
    Ns *= 16;
  }
  if (P::RLAST > 1) {
    constexpr int R = P::RLAST;
    constexpr int NB = L / R;   // butterflies
    constexpr int PER = 16 / R; // per thread
    float2 x[16];
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int jb = j + u * Q;
#pragma unroll
      for (int r = 0; r < R; ++r) x[u * R + r] = buf[fpad(jb + r * NB)];
    }
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int jb = j + u * Q;
      const int jm = jb & (Ns - 1);
      float2 *v = x + u * R;
      if (jm != 0) {
#pragma unroll
        for (int r = 1; r < R; ++r) v[r] = cmul(v[r], troot<INV>(roots, r * jm * (L / (R * Ns))));
      }
      Dft<(R > 1 ? R : 2), INV>::run(v, roots, L);
    }
    sync();
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int jb = j + u * Q;
      const int jm = jb & (Ns - 1);
      const int ob = (jb - jm) * R + jm;
#pragma unroll
      for (int r = 0; r < R; ++r) buf[fpad(ob + r * Ns)] = x[u * R + r];
    }
    sync();
  }
}

}  // namespace gnc
