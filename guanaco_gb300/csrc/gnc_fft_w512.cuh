// Register FFTs of 128, 256, 384 and 512 points with 16 values per lane: lane
// l of a transform holds x[l + L m] in v[m] (m = 0..15, L = N / 16 lanes)
// before and after the transform, so transforms and pointwise products chain
// in registers.  A warp runs one 512- or 384-point transform (the 384-point one
// on 24 of its lanes), two 256-point or four 128-point ones.
//
// N = 16 B A with n = n0 + A n1 + A B n2 and k = ka + 16 kb + 16 B kc
// (n2, ka < 16; n1, kb < B; n0, kc < A), lane l = n0 + A n1 on entry:
//   X[k] = sum_n0 WA^(n0 kc) W(AB)^(n0 kb) WN^(n0 ka)
//            sum_n1 WB^(n1 kb) W(16B)^(n1 ka) sum_n2 W16^(n2 ka) x[n]
// 1. each lane: 16-point DFT over its registers (n2 -> ka), times WN^(l ka);
// 2. B > 1: radix B across the lanes n0 + A n1 (shuffles): lane n0 + A kb keeps
//    component kb, times W(AB)^(n0 kb)  (512: B = 2, 384: B = 3);
// 3. exchange through shared memory and A-point DFTs over n0.  A = 16 (256,
//    512): lane ka + 16 kb gathers n0 = 0..15, and X[l + L kc] lands in v[kc].
//    A = 8 (128, 384): the DFT of (ka, kb) has outputs ka + 16 kb + 2 L kc, all
//    in lane (ka + 16 kb) mod L, so lane l runs the DFTs of ka + 16 kb = l and
//    l + L and X[l + L m] lands in v[m] with m = 2 kc (first) or 2 kc + 1.
// Exchange slots n0 + P1 ka + P2 kb, one region of SLOTS per transform: every
// half warp's writes and reads hit 16 distinct 8-byte bank pairs, except, for
// 384 points, half of the second read group (two-way).  Butterflies on packed
// f32x2 pairs.  Conventions: forward exp(-2 pi i/N), inverse exp(+2 pi i/N),
// unnormalised.
#pragma once

#include "gnc_fft_block4096.cuh"
#include "gnc_fft_warp.cuh"

namespace gnc {

template <int N>
struct WarpFftShape {
  static_assert(N == 128 || N == 256 || N == 384 || N == 512, "128, 256, 384 or 512 points");
  static constexpr int L = N / 16;                         // lanes per transform
  static constexpr int A = (N == 256 || N == 512) ? 16 : 8;
  static constexpr int B = L / A;
  static constexpr int TPW = 32 / L;                       // transforms per warp
  static constexpr int P1 = A == 16 ? 17 : 9;
  static constexpr int P2 = N == 512 ? 272 : (N == 384 ? 152 : 0);
  static constexpr int SLOTS = N == 512 ? 544 : N == 384 ? 448 : N == 256 ? 272 : 152;
};

// One N-point transform by the L lanes of a transform; l = lane within it,
// act = false for the idle lanes of a warp (384 points: lanes 24..31), which
// take part in the shuffles but touch no shared memory; roots = the N-point
// table, slots = this transform's exchange region.  Contains __syncwarp()
// only; the caller's other uses of the slots need their own __syncwarp().
template <int N, bool INV>
__device__ __forceinline__ void warp_fft_n(float2 *v, float2 *slots,
                                           const float2 *__restrict__ roots, int l,
                                           bool act = true) {
  using S = WarpFftShape<N>;
  constexpr int A = S::A, B = S::B;
  dft16_pk<INV>(v);
  twiddle16<INV>(v, roots, l);
  const int n0 = l % A, n1 = l / A;  // (n0, n1) on entry, (n0, kb = n1) after step 2
  if (B == 2) {
    const float sg = n1 ? -1.f : 1.f;
    const float2 w = troot<INV>(roots, 16 * n0 * n1);  // W32^(n0 kb)
#pragma unroll
    for (int ka = 0; ka < 16; ++ka) {
      float2 o;
      o.x = __shfl_xor_sync(0xffffffffu, v[ka].x, 16);
      o.y = __shfl_xor_sync(0xffffffffu, v[ka].y, 16);
      v[ka] = cmul(make_float2(o.x + sg * v[ka].x, o.y + sg * v[ka].y), w);
    }
  } else if (B == 3) {
    // lane (n0, kb): sum over n1' of W3^(n1' kb) y[n0 + 8 n1'], then W24^(n0 kb)
    const int lane = threadIdx.x & 31;
    const int base = act ? lane - l : 0;  // first lane of this transform (idle lanes: any)
    const int p1 = (n1 + 1) % 3, p2 = (n1 + 2) % 3;
    const float s3 = INV ? 0.86602540378443865f : -0.86602540378443865f;  // sin of -+2 pi/3
    auto w3 = [&](int e) {  // W3^e
      e %= 3;
      return e == 0 ? make_float2(1.f, 0.f) : make_float2(-0.5f, e == 1 ? s3 : -s3);
    };
    const float2 c0 = w3(n1 * n1), c1 = w3(p1 * n1), c2 = w3(p2 * n1);
    const float2 w = troot<INV>(roots, 16 * n0 * n1);  // W24^(n0 kb)
    const int src1 = base + n0 + 8 * p1, src2 = base + n0 + 8 * p2;
#pragma unroll
    for (int ka = 0; ka < 16; ++ka) {
      float2 y1, y2;
      y1.x = __shfl_sync(0xffffffffu, v[ka].x, src1);
      y1.y = __shfl_sync(0xffffffffu, v[ka].y, src1);
      y2.x = __shfl_sync(0xffffffffu, v[ka].x, src2);
      y2.y = __shfl_sync(0xffffffffu, v[ka].y, src2);
      const float2 z = cadd(cadd(cmul(v[ka], c0), cmul(y1, c1)), cmul(y2, c2));
      v[ka] = cmul(z, w);
    }
  }
  __syncwarp();
  if (act) {
#pragma unroll
    for (int ka = 0; ka < 16; ++ka) slots[n0 + S::P1 * ka + S::P2 * n1] = v[ka];
  }
  __syncwarp();
  if (A == 16) {
    if (act) {
#pragma unroll
      for (int j = 0; j < 16; ++j) v[j] = slots[j + S::P1 * n0 + S::P2 * n1];
    }
    dft16_pk<INV>(v);
  } else {
    // the 8-point DFTs of ka + 16 kb = l + s L, s = 0, 1
    pk::c64 t[2][8];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int b = l + s * S::L, ka = b & 15, kb = b >> 4;
#pragma unroll
      for (int j = 0; j < 8; ++j)
        t[s][j] = pk::pack(act ? slots[j + S::P1 * ka + S::P2 * kb] : make_float2(0.f, 0.f));
      pk::dft8<INV>(t[s]);
    }
#pragma unroll
    for (int kc = 0; kc < 8; ++kc) {
      v[2 * kc] = pk::unpack(t[0][kc]);
      v[2 * kc + 1] = pk::unpack(t[1][kc]);
    }
  }
}

}  // namespace gnc
