// One-warp 1024-point FFT with the data in registers.
//
// Layout: lane l holds x[32 m + l] in v[m] (m = 0..31), before and after the
// transform (lane = index mod 32, register = index div 32), so transforms and
// pointwise products chain in registers.  With n = 32 m + l, k = k1 + 32 k2:
//   X[k] = sum_l W32^(l k2) W1024^(l k1) sum_m W32^(m k1) x[32 m + l]
// 1. each lane: 32-point DFT over its registers -> Y[l][k1] in v[k1]
// 2. each lane: twiddle Y[l][k1] *= W1024^(l k1)      (table in shared memory)
// 3. transpose through kWarpFftSlots shared-memory slots: lane k1 gets Y[.][k1]
// 4. each lane: 32-point DFT over its registers -> X[k1 + 32 k2] in v[k2].
// The transpose slot of (k1, l) is 33 k1 + l: the row-wise writes and the
// column-wise reads both hit 16 distinct 8-byte bank pairs per half warp, and
// every slot address is one per-lane base plus a constant, so no per-slot
// address stays live from one transform to the next.
// Conventions: forward exp(-2 pi i/N), inverse exp(+2 pi i/N), unnormalised.
#pragma once

#include "gnc_fft.cuh"

namespace gnc {

// cos and sin of 2 pi m / 32, m = 0..31
struct Roots32 {
  static constexpr float c[32] = {
      1.0f, 0.98078528040323043f, 0.92387953251128674f, 0.83146961230254524f,
      0.70710678118654757f, 0.55557023301960229f, 0.38268343236508984f, 0.19509032201612833f,
      0.0f, -0.19509032201612819f, -0.38268343236508973f, -0.55557023301960196f,
      -0.70710678118654746f, -0.83146961230254535f, -0.92387953251128674f, -0.98078528040323043f,
      -1.0f, -0.98078528040323043f, -0.92387953251128685f, -0.83146961230254546f,
      -0.70710678118654768f, -0.55557023301960218f, -0.38268343236509034f, -0.19509032201612866f,
      0.0f, 0.1950903220161283f, 0.38268343236509f, 0.55557023301960184f,
      0.70710678118654735f, 0.83146961230254524f, 0.92387953251128652f, 0.98078528040323032f};
  static constexpr float s[32] = {
      0.0f, 0.19509032201612825f, 0.38268343236508978f, 0.55557023301960218f,
      0.70710678118654746f, 0.83146961230254524f, 0.92387953251128674f, 0.98078528040323043f,
      1.0f, 0.98078528040323043f, 0.92387953251128674f, 0.83146961230254546f,
      0.70710678118654757f, 0.55557023301960218f, 0.38268343236508989f, 0.19509032201612861f,
      0.0f, -0.19509032201612836f, -0.38268343236508967f, -0.55557023301960196f,
      -0.70710678118654746f, -0.83146961230254524f, -0.92387953251128652f, -0.98078528040323032f,
      -1.0f, -0.98078528040323043f, -0.92387953251128663f, -0.83146961230254546f,
      -0.70710678118654768f, -0.55557023301960218f, -0.38268343236509039f, -0.19509032201612872f};
};

// x * W32^m (forward root exp(-2 pi i m/32); conjugate for the inverse)
template <bool INV, int M>
__device__ __forceinline__ float2 w32(float2 x) {
  constexpr float c = Roots32::c[M];
  constexpr float s = INV ? Roots32::s[M] : -Roots32::s[M];
  return make_float2(x.x * c - x.y * s, x.x * s + x.y * c);
}

// 32-point DFT of v[0..31] in registers, natural order in and out.
// 32 = 8 x 4: n = 4 n1 + n2, k = k1 + 8 k2.
template <bool INV>
__device__ __forceinline__ void dft32(float2 *v) {
  float2 a[32];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    float2 t[8];
#pragma unroll
    for (int n1 = 0; n1 < 8; ++n1) t[n1] = v[4 * n1 + n2];
    Dft<8, INV>::run(t, nullptr, 0);
#pragma unroll
    for (int k1 = 0; k1 < 8; ++k1) a[n2 * 8 + k1] = t[k1];
  }
  // twiddles W32^(n2 k1)
#define GNC_TW(N2, K1) a[N2 * 8 + K1] = w32<INV, N2 * K1>(a[N2 * 8 + K1])
  GNC_TW(1, 1); GNC_TW(1, 2); GNC_TW(1, 3); GNC_TW(1, 4); GNC_TW(1, 5); GNC_TW(1, 6); GNC_TW(1, 7);
  GNC_TW(2, 1); GNC_TW(2, 2); GNC_TW(2, 3); GNC_TW(2, 4); GNC_TW(2, 5); GNC_TW(2, 6); GNC_TW(2, 7);
  GNC_TW(3, 1); GNC_TW(3, 2); GNC_TW(3, 3); GNC_TW(3, 4); GNC_TW(3, 5); GNC_TW(3, 6); GNC_TW(3, 7);
#undef GNC_TW
#pragma unroll
  for (int k1 = 0; k1 < 8; ++k1) {
    float2 t[4] = {a[k1], a[8 + k1], a[16 + k1], a[24 + k1]};
    Dft<4, INV>::run(t, nullptr, 0);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 8 * k2] = t[k2];
  }
}

constexpr int kWarpFftSlots = 33 * 32;
__device__ __forceinline__ int wslot(int k1, int l) { return 33 * k1 + l; }

// Fill the shared twiddle table: tw[k1 * 32 + l] = W1024^(l k1) (forward),
// from the 1024-point root table in global memory.  Call with the whole block,
// then __syncthreads().
__device__ __forceinline__ void warp_fft_twiddles(float2 *tw, const float2 *__restrict__ roots) {
  for (int i = threadIdx.x; i < 1024; i += blockDim.x) {
    const int k1 = i >> 5, l = i & 31;
    tw[i] = __ldg(roots + ((l * k1) & 1023));
  }
}

// In-register 1024-point transform by one warp.  The transpose uses
// kWarpFftSlots shared-memory slots owned by this warp: slot s is
// tbuf[s * STRIDE] (STRIDE odd).  Contains __syncwarp() only; the slots may be reused by the
// caller once it has issued another __syncwarp().
template <bool INV, int STRIDE = 1>
__device__ __forceinline__ void warp_fft1024(float2 *v, float2 *tbuf, const float2 *tw, int lane) {
  dft32<INV>(v);
#pragma unroll
  for (int k1 = 1; k1 < 32; ++k1) {
    float2 w = tw[k1 * 32 + lane];
    if (INV) w.y = -w.y;
    v[k1] = cmul(v[k1], w);
  }
  __syncwarp();
#pragma unroll
  for (int k1 = 0; k1 < 32; ++k1) tbuf[wslot(k1, lane) * STRIDE] = v[k1];
  __syncwarp();
#pragma unroll
  for (int l = 0; l < 32; ++l) v[l] = tbuf[wslot(lane, l) * STRIDE];
  dft32<INV>(v);
}

}  // namespace gnc
