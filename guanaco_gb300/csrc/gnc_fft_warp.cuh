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

// ---- complex numbers as f32x2 pairs (sm_100 packed arithmetic): a complex
// add or subtract is one instruction
namespace pk {
typedef unsigned long long c64;
__device__ __forceinline__ c64 pack(float2 a) {
  c64 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 unpack(c64 a) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(a));
  return r;
}
__device__ __forceinline__ c64 add(c64 a, c64 b) {
  c64 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ c64 sub(c64 a, c64 b) {
  c64 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ c64 mul(c64 a, c64 b) {
  c64 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
// times -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ c64 mul_si(c64 a) {
  const float2 f = unpack(a);
  return pack(INV ? make_float2(-f.y, f.x) : make_float2(f.y, -f.x));
}

// The radix-4 and radix-8 butterflies of Dft<4> / Dft<8> (gnc_fft.cuh), the
// same operations in the same order on packed values.
template <bool INV>
__device__ __forceinline__ void dft4(c64 &v0, c64 &v1, c64 &v2, c64 &v3) {
  const c64 a = add(v0, v2), b = sub(v0, v2), c = add(v1, v3), d = mul_si<INV>(sub(v1, v3));
  v0 = add(a, c);
  v2 = sub(a, c);
  v1 = add(b, d);
  v3 = sub(b, d);
}

template <bool INV>
__device__ __forceinline__ void dft8(c64 *v) {
  const float r = 0.7071067811865476f;
  const c64 rr = pack(make_float2(r, r));
  c64 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  c64 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4<INV>(e0, e1, e2, e3);
  dft4<INV>(o0, o1, o2, o3);
  // w8 = r(1 + s i), w8^2 = s i, w8^3 = r(-1 + s i)
  const c64 t1 = mul(add(o1, mul_si<INV>(o1)), rr);
  const c64 t2 = mul_si<INV>(o2);
  const c64 t3 = mul(sub(mul_si<INV>(o3), o3), rr);
  v[0] = add(e0, o0);
  v[4] = sub(e0, o0);
  v[1] = add(e1, t1);
  v[5] = sub(e1, t1);
  v[2] = add(e2, t2);
  v[6] = sub(e2, t2);
  v[3] = add(e3, t3);
  v[7] = sub(e3, t3);
}
}  // namespace pk

// 32-point DFT of v[0..31] in registers, natural order in and out.
// 32 = 8 x 4: n = 4 n1 + n2, k = k1 + 8 k2.  Butterflies on packed pairs.
template <bool INV>
__device__ __forceinline__ void dft32(float2 *v) {
  pk::c64 a[32];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    pk::c64 t[8];
#pragma unroll
    for (int n1 = 0; n1 < 8; ++n1) t[n1] = pk::pack(v[4 * n1 + n2]);
    pk::dft8<INV>(t);
#pragma unroll
    for (int k1 = 0; k1 < 8; ++k1) a[n2 * 8 + k1] = t[k1];
  }
  // twiddles W32^(n2 k1)
#define GNC_TW(N2, K1) a[N2 * 8 + K1] = pk::pack(w32<INV, N2 * K1>(pk::unpack(a[N2 * 8 + K1])))
  GNC_TW(1, 1); GNC_TW(1, 2); GNC_TW(1, 3); GNC_TW(1, 4); GNC_TW(1, 5); GNC_TW(1, 6); GNC_TW(1, 7);
  GNC_TW(2, 1); GNC_TW(2, 2); GNC_TW(2, 3); GNC_TW(2, 4); GNC_TW(2, 5); GNC_TW(2, 6); GNC_TW(2, 7);
  GNC_TW(3, 1); GNC_TW(3, 2); GNC_TW(3, 3); GNC_TW(3, 4); GNC_TW(3, 5); GNC_TW(3, 6); GNC_TW(3, 7);
#undef GNC_TW
#pragma unroll
  for (int k1 = 0; k1 < 8; ++k1) {
    pk::dft4<INV>(a[k1], a[8 + k1], a[16 + k1], a[24 + k1]);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 8 * k2] = pk::unpack(a[k1 + 8 * k2]);
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
