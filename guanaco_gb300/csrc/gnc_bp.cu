// Backprojection of the filtered, staged rows into the volume.
//
// Reference: guanaco::Reconstructor_t<e_host>::project
// (src/libguanaco/reconstructor.cpp:14-90), the parity target:
//   x = i - X/2 + 1/2,  y = j - Z/2 + 1/2                        (float)
//   pixel  = x cos - y sin + offset;  height = -x sin - y cos    (float)
//   slab   = clamp(floor(height * dscale + doffset + 0.5), 0, D-1)
//   pixel -= 0.5;  ind = floor(pixel);  t = pixel - ind
//   if 0 <= ind < N-1:  rec += scale * ((1 - t) v[ind] + t v[ind+1])
// The exact kernels below evaluate every one of these operations with
// round-to-nearest intrinsics (no contraction) in the reference's order, so
// with identical filtered input they reproduce the reference bit for bit.
#include "gnc_common.cuh"

namespace gnc {

__device__ __forceinline__ float voxel_coord(int i, int n) {
  return (float)((double)i - 0.5 * (double)n + 0.5);
}

// MODE: kStageF32, kStageF16 (records) or kStageF16T (plain FP16 rows, one
// exponent per tilt)
template <int MODE>
__global__ void k_bp_exact(BpArgs a) {
  constexpr bool F16 = MODE == kStageF16;
  if (a.dyn) {
    a.dscale = a.dyn[0];
    a.doffset = a.dyn[1];
  }
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int z = blockIdx.y * blockDim.y + threadIdx.y;
  const int y2 = blockIdx.z;
  if (x >= a.X || z >= a.Z) return;
  const float xf = voxel_coord(x, a.X);
  const float zf = voxel_coord(z, a.Z);
  const int ya = 2 * y2, yb = ya + 1;
  const bool hb = yb < a.Y;
  float acc_a = 0.f, acc_b = 0.f;
  for (int t = 0; t < a.T; ++t) {
    const TiltGeom g = a.geom[t];
    int k = a.D > 1 ? slab_index(xf, zf, g.sin_a, g.cos_a, a.dscale, a.doffset, a.D) : 0;
    const size_t rowi = ((size_t)y2 * a.D + k) * a.T + t;
    float sa = 1.f, sb = 1.f;
    if (F16) {
      sa = __int_as_float((127 - a.row_exp[2 * rowi]) << 23);
      sb = __int_as_float((127 - a.row_exp[2 * rowi + 1]) << 23);
    }
    if (MODE == kStageF16T) sa = sb = __int_as_float((127 - a.tilt_exp[t]) << 23);
    const float xc = __fmul_rn(xf, g.cos_a), zs = __fmul_rn(zf, g.sin_a);
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      if (r == 1 && !hb) break;
      const int yy = r == 0 ? ya : yb;
      float pixel = __fadd_rn(__fsub_rn(xc, zs), a.offset[(size_t)yy * a.T + t]);
      pixel = __fsub_rn(pixel, 0.5f);
      const int ind = (int)floorf(pixel);
      const float tt = __fsub_rn(pixel, (float)ind);
      if (ind >= 0 && ind < a.N - 1) {
        float v0, v1;
        if (MODE == kStageF16T) {
          const __half *row = (const __half *)a.staged +
                              (((size_t)k * a.T + t) * a.stack_h + a.y_begin + yy) * a.N;
          v0 = __half2float(row[ind]) * sa;
          v1 = __half2float(row[ind + 1]) * sa;
        } else if (F16) {  // the values of records ind and ind + 1
          const uint2 *row = (const uint2 *)a.staged + rowi * a.N;
          const unsigned u0 = row[ind].x, u1 = row[ind + 1].x;
          float2 p0 = __half22float2(*(const __half2 *)&u0);
          float2 p1 = __half22float2(*(const __half2 *)&u1);
          v0 = (r == 0 ? p0.x : p0.y) * (r == 0 ? sa : sb);
          v1 = (r == 0 ? p1.x : p1.y) * (r == 0 ? sa : sb);
        } else {
          const float2 *row = (const float2 *)a.staged + rowi * a.N;
          float2 p0 = row[ind], p1 = row[ind + 1];
          v0 = r == 0 ? p0.x : p0.y;
          v1 = r == 0 ? p1.x : p1.y;
        }
        const float value = __fadd_rn(__fmul_rn(__fsub_rn(1.0f, tt), v0), __fmul_rn(tt, v1));
        if (r == 0)
          acc_a = __fadd_rn(acc_a, __fmul_rn(g.scale, value));
        else
          acc_b = __fadd_rn(acc_b, __fmul_rn(g.scale, value));
      }
    }
  }
  a.vol[((size_t)ya * a.Z + z) * a.X + x] = acc_a;
  if (hb) a.vol[((size_t)yb * a.Z + z) * a.X + x] = acc_b;
}

cudaError_t launch_backproject_exact(const BpArgs &a, cudaStream_t s) {
  dim3 block(32, 8);
  dim3 grid((a.X + 31) / 32, (a.Z + 7) / 8, (a.Y + 1) / 2);
  if (a.staging == kStageF16)
    k_bp_exact<kStageF16><<<grid, block, 0, s>>>(a);
  else if (a.staging == kStageF16T)
    k_bp_exact<kStageF16T><<<grid, block, 0, s>>>(a);
  else
    k_bp_exact<kStageF32><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

__global__ void k_slab_map(BpArgs a, int32_t *__restrict__ out) {
  if (a.dyn) {
    a.dscale = a.dyn[0];
    a.doffset = a.dyn[1];
  }
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int z = blockIdx.y * blockDim.y + threadIdx.y;
  const int t = blockIdx.z;
  if (x >= a.X || z >= a.Z) return;
  const TiltGeom g = a.geom[t];
  int k = a.D > 1 ? slab_index(voxel_coord(x, a.X), voxel_coord(z, a.Z), g.sin_a, g.cos_a,
                               a.dscale, a.doffset, a.D)
                  : 0;
  out[((size_t)t * a.Z + z) * a.X + x] = k;
}

// One thread per tilt: the slab index at the volume's four corners (the index
// is monotone in x and in z) gives the slabs any voxel reads.
__global__ void k_live_slabs(BpArgs a, int2 *__restrict__ live) {
  if (a.dyn) {
    a.dscale = a.dyn[0];
    a.doffset = a.dyn[1];
  }
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.T) return;
  int lo = 0, hi = 0;
  if (a.D > 1) {
    const TiltGeom g = a.geom[t];
    const float x0 = voxel_coord(0, a.X), x1 = voxel_coord(a.X - 1, a.X);
    const float z0 = voxel_coord(0, a.Z), z1 = voxel_coord(a.Z - 1, a.Z);
    const int k00 = slab_index(x0, z0, g.sin_a, g.cos_a, a.dscale, a.doffset, a.D);
    const int k01 = slab_index(x0, z1, g.sin_a, g.cos_a, a.dscale, a.doffset, a.D);
    const int k10 = slab_index(x1, z0, g.sin_a, g.cos_a, a.dscale, a.doffset, a.D);
    const int k11 = slab_index(x1, z1, g.sin_a, g.cos_a, a.dscale, a.doffset, a.D);
    lo = min(min(k00, k01), min(k10, k11));
    hi = max(max(k00, k01), max(k10, k11));
  }
  live[t] = make_int2(lo, hi);
}

cudaError_t launch_live_slabs(const BpArgs &a, int2 *live, cudaStream_t s) {
  k_live_slabs<<<(a.T + 127) / 128, 128, 0, s>>>(a, live);
  return cudaGetLastError();
}

cudaError_t launch_slab_map(const BpArgs &a, int32_t *out, cudaStream_t s) {
  dim3 block(32, 8);
  dim3 grid((a.X + 31) / 32, (a.Z + 7) / 8, a.T);
  k_slab_map<<<grid, block, 0, s>>>(a, out);
  return cudaGetLastError();
}

// Single slice from plain rows (D, T, N): guanaco.detail.recon's per-call path.
__global__ void k_bp_slice(SliceBpArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int z = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= a.X || z >= a.Z) return;
  const float xf = voxel_coord(x, a.X);
  const float zf = voxel_coord(z, a.Z);
  float acc = 0.f;
  for (int t = 0; t < a.T; ++t) {
    const TiltGeom g = a.geom[t];
    int k = a.D > 1 ? slab_index(xf, zf, g.sin_a, g.cos_a, a.dscale, a.doffset, a.D) : 0;
    const float *row = a.sino + ((size_t)k * a.T + t) * a.N;
    float pixel = __fadd_rn(__fsub_rn(__fmul_rn(xf, g.cos_a), __fmul_rn(zf, g.sin_a)), a.offset);
    pixel = __fsub_rn(pixel, 0.5f);
    const int ind = (int)floorf(pixel);
    const float tt = __fsub_rn(pixel, (float)ind);
    if (ind >= 0 && ind < a.N - 1) {
      const float value =
          __fadd_rn(__fmul_rn(__fsub_rn(1.0f, tt), row[ind]), __fmul_rn(tt, row[ind + 1]));
      acc = __fadd_rn(acc, __fmul_rn(g.scale, value));
    }
  }
  a.rec[(size_t)z * a.X + x] = acc;
}

cudaError_t launch_backproject_slice(const SliceBpArgs &a, cudaStream_t s) {
  dim3 block(32, 8);
  dim3 grid((a.X + 31) / 32, (a.Z + 7) / 8);
  k_bp_slice<<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace gnc
