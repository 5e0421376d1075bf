// One-warp 512-point and half-warp 256-point FFTs with the data in registers:
// 16 values per lane, lane l of a transform holding x[l + L m] in v[m]
// (L = 32 lanes for 512 points, 16 for 256) before and after the transform, so
// transforms and pointwise products chain in registers.
//
// 512 points, n = n0 + 16 n1 + 32 n2 and k = ka + 16 kb + 32 kc (n0, ka, n2,
// kc < 16; n1, kb < 2), lane l = n0 + 16 n1 on entry:
//   X[k] = sum_n0 W16^(n0 kc) W32^(n0 kb) W512^(n0 ka)
//            sum_n1 (-1)^(n1 kb) W32^(n1 ka) sum_n2 W16^(n2 ka) x[n]
// 1. each lane: 16-point DFT over its registers (n2 -> ka), times W512^(l ka);
// 2. radix 2 across lanes l and l ^ 16 (shuffles): lane n0 + 16 kb keeps the
//    sum (kb = 0) or the difference (kb = 1), times W32^(n0 kb);
// 3. exchange through shared memory: lane ka + 16 kb gathers n0 = 0..15 from
//    slots n0 + 17 ka + 272 kb, and a 16-point DFT (n0 -> kc) leaves
//    X[l + 32 kc] in v[kc].
// 256 points: steps 1 and 3 with 16 lanes (no radix-2 step), slots n0 + 17 ka.
// The exchange's writes (fixed ka) and reads (fixed n0) give each half warp 16
// distinct 8-byte bank pairs.  Butterflies on packed f32x2 pairs (dft16_pk).
// Conventions: forward exp(-2 pi i/N), inverse exp(+2 pi i/N), unnormalised.
#pragma once

#include "gnc_fft_block4096.cuh"

namespace gnc {

constexpr int kW512Slots = 544;  // exchange slots of one 512-point transform
constexpr int kW256Slots = 272;  // of one 256-point transform

// lanes of one N-point transform (N = 256 or 512)
template <int N>
struct WarpFftShape {
  static_assert(N == 256 || N == 512, "256 or 512 points");
  static constexpr int L = N / 16;                      // lanes per transform
  static constexpr int SLOTS = N == 512 ? kW512Slots : kW256Slots;
};

// One N-point transform by the L lanes of a (half) warp; l = lane within the
// transform, roots = the N-point table, slots = this transform's exchange
// slots.  Contains __syncwarp() only; the caller's other uses of the slots
// need their own __syncwarp().
template <int N, bool INV>
__device__ __forceinline__ void warp_fft_n(float2 *v, float2 *slots,
                                           const float2 *__restrict__ roots, int l) {
  dft16_pk<INV>(v);
  twiddle16<INV>(v, roots, l);
  if (N == 512) {
    const int n0 = l & 15, kb = l >> 4;
    const float sg = kb ? -1.f : 1.f;
    const float2 w = troot<INV>(roots, 16 * n0 * kb);  // W32^(n0 kb); 1 for kb = 0
#pragma unroll
    for (int ka = 0; ka < 16; ++ka) {
      float2 o;
      o.x = __shfl_xor_sync(0xffffffffu, v[ka].x, 16);
      o.y = __shfl_xor_sync(0xffffffffu, v[ka].y, 16);
      v[ka] = cmul(make_float2(o.x + sg * v[ka].x, o.y + sg * v[ka].y), w);
    }
  }
  const int a = l & 15, b = N == 512 ? (l >> 4) : 0;  // (n0, n1) on write, (ka, kb) on read
  __syncwarp();
#pragma unroll
  for (int ka = 0; ka < 16; ++ka) slots[a + 17 * ka + 272 * b] = v[ka];
  __syncwarp();
#pragma unroll
  for (int n0 = 0; n0 < 16; ++n0) v[n0] = slots[n0 + 17 * a + 272 * b];
  dft16_pk<INV>(v);
}

}  // namespace gnc
