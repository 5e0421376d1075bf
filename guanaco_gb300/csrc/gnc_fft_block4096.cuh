// Block-wide 4096-point FFT with the data in registers: 256 threads per
// transform, thread l holding x[l + 256 m] in v[m] (m = 0..15) before and after
// the transform, so transforms and pointwise products chain in registers.
//
// With n = n0 + 16 n1 + 256 n2 and k = k0 + 16 k1 + 256 k2 (digits 0..15):
//   X[k] = sum_n0 W16^(n0 k2) W256^(n0 k1) W4096^(n0 k0)
//            sum_n1 W16^(n1 k1) W256^(n1 k0)  sum_n2 W16^(n2 k0) x[n]
// 1. thread l = n0 + 16 n1: 16-point DFT over its registers (n2 -> k0), times
//    W4096^(l k0);
// 2. exchange: thread l = n0 + 16 k0 gathers n1 = 0..15 from slots
//    A[n0 + 16 n1 + 264 k0]; 16-point DFT (n1 -> k1), times W4096^(16 n0 k1);
// 3. exchange: thread l = k0 + 16 k1 gathers n0 = 0..15 from slots
//    B[k0 + 16 k1 + 257 n0]; 16-point DFT (n0 -> k2): X[l + 256 k2] in v[k2].
// Two shared-memory exchanges per transform (a Stockham radix-16 transform in
// shared memory moves the data three times, plus the load and store).
// Eight-byte shared accesses are served a half warp at a time; in every
// exchange the 16 lanes of a half warp hit 16 distinct 8-byte bank pairs, also
// when the threads of C = 2 or 4 transforms are interleaved (thread = c + C l)
// and transform c's slots start at c * kB4096Stride (= 4 mod 16).
// Conventions: forward exp(-2 pi i/N), inverse exp(+2 pi i/N), unnormalised.
#pragma once

#include "gnc_fft_pow2.cuh"
#include "gnc_fft_warp.cuh"

namespace gnc {

constexpr int kB4096Slots = 4216;   // slots of one transform's exchanges
constexpr int kB4096Stride = 4228;  // slot stride of interleaved transforms (4 mod 16)

// 16-point DFT in registers, natural order, with the radix-4 butterflies on
// packed f32x2 pairs: the operations of dft16 (gnc_fft_pow2.cuh) in the same
// order, so the results are the same.
template <bool INV>
__device__ __forceinline__ void dft16_pk(float2 *x) {
  pk::c64 a[16];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    pk::c64 v0 = pk::pack(x[n2]), v1 = pk::pack(x[4 + n2]), v2 = pk::pack(x[8 + n2]),
            v3 = pk::pack(x[12 + n2]);
    pk::dft4<INV>(v0, v1, v2, v3);
    a[n2 * 4 + 0] = v0;
    a[n2 * 4 + 1] = v1;
    a[n2 * 4 + 2] = v2;
    a[n2 * 4 + 3] = v3;
  }
#pragma unroll
  for (int n2 = 1; n2 < 4; ++n2)
#pragma unroll
    for (int k1 = 1; k1 < 4; ++k1)
      a[n2 * 4 + k1] = pk::pack(w16<INV>(pk::unpack(a[n2 * 4 + k1]), n2 * k1));
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    pk::dft4<INV>(a[k1], a[4 + k1], a[8 + k1], a[12 + k1]);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) x[k1 + 4 * k2] = pk::unpack(a[k1 + 4 * k2]);
  }
}

// v[r] *= w^(r base) for r = 1..15, w = exp(-2 pi i / 4096) (conjugate for the
// inverse): powers 1, 2, 3, 4, 8 and 12 from the table, the others as products
// of two of them, as in fft_pow2.
template <bool INV>
__device__ __forceinline__ void twiddle16(float2 *v, const float2 *__restrict__ roots, int base) {
  const float2 w1 = troot<INV>(roots, base), w2 = troot<INV>(roots, 2 * base);
  const float2 w3 = troot<INV>(roots, 3 * base), w4 = troot<INV>(roots, 4 * base);
  const float2 w8 = troot<INV>(roots, 8 * base), w12 = troot<INV>(roots, 12 * base);
  v[1] = cmul(v[1], w1);
  v[2] = cmul(v[2], w2);
  v[3] = cmul(v[3], w3);
  v[4] = cmul(v[4], w4);
  v[5] = cmul(v[5], cmul(w4, w1));
  v[6] = cmul(v[6], cmul(w4, w2));
  v[7] = cmul(v[7], cmul(w4, w3));
  v[8] = cmul(v[8], w8);
  v[9] = cmul(v[9], cmul(w8, w1));
  v[10] = cmul(v[10], cmul(w8, w2));
  v[11] = cmul(v[11], cmul(w8, w3));
  v[12] = cmul(v[12], w12);
  v[13] = cmul(v[13], cmul(w12, w1));
  v[14] = cmul(v[14], cmul(w12, w2));
  v[15] = cmul(v[15], cmul(w12, w3));
}

// One transform by the 256 threads l of a group; roots is the 4096-point
// table.  sync() synchronises every thread that shares A and B.  With
// SAME = false (A and B distinct), consecutive transforms need no other
// synchronisation; with SAME = true (one buffer) the caller synchronises
// before the slots are used again.
template <bool INV, bool SAME, typename Sync>
__device__ __forceinline__ void bfft4096(float2 *v, float2 *A, float2 *B,
                                         const float2 *__restrict__ roots, int l, Sync sync) {
  dft16_pk<INV>(v);
  twiddle16<INV>(v, roots, l);
#pragma unroll
  for (int k0 = 0; k0 < 16; ++k0) A[l + 264 * k0] = v[k0];
  sync();
  {
    const int n0 = l & 15, k0 = l >> 4;
    const float2 *a = A + n0 + 264 * k0;
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) v[n1] = a[16 * n1];
    dft16_pk<INV>(v);
    twiddle16<INV>(v, roots, 16 * n0);
    if (SAME) sync();
    float2 *b = B + k0 + 257 * n0;
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) b[16 * k1] = v[k1];
  }
  sync();
#pragma unroll
  for (int n0 = 0; n0 < 16; ++n0) v[n0] = B[l + 257 * n0];
  dft16_pk<INV>(v);
}

}  // namespace gnc
