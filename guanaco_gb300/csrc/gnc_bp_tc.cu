// Tensor-core backprojection of F16T rows (FP16, one power-of-two scale per
// tilt) with FP32 accumulation in tensor memory.
//
// For one tilt, the backprojection of a set of voxels into a set of Y rows is
// a product V[v, y] += sum_u W[v, u] S[u, y] of the interpolation weights
// (two non-zeros per voxel: (1 - t) at the voxel's pixel floor(p), t at the
// next one, src/libguanaco/reconstructor.cpp:76-86) and the staged rows.  A
// block owns 128 voxels -- a 16 (x) by 8 (z) tile, compact so that for any
// tilt they project onto at most 18 detector pixels -- and 256 Y rows.  Per
// tilt and per defocus slab the tile reaches:
//   * one TMA load brings the 32-pixel window [u0, u0 + 32) of the 256 rows
//     (u0 a multiple of 8) into shared memory, 64-byte swizzled;
//   * 256 builder threads (two per voxel, one per half of the window) compute
//     the voxel's detector coordinate, floor, weight and slab with the
//     reference's float operations, and store its 32 weights (zero outside
//     its own slab, its own pixel pair and the detector edge rule) into a
//     tensor-memory row;
//   * one thread issues two tcgen05.mma (M 128 voxels, N 256 rows, K 16
//     pixels each) accumulating into the 128 x 256 FP32 tile in tensor memory.
// Weights carry the tilt's factor 2^(E0 - e(t)) (E0 the smallest exponent over
// the tilts), so the accumulator counts in units of 2^-E0 for every tilt; the
// store multiplies by the backprojection scale and 2^-E0.
//
// What decides which samples a voxel takes -- its detector coordinate, floor,
// weight t, slab index and edge rule -- is the reference's float arithmetic,
// bit for bit (as in gnc_bp.cu); the products and sums are FP16 x FP16 -> FP32
// on the tensor cores.
//
// Warp roles (320 threads, one block per SM): warps 0-7 build weights
// (warps w and w + 4 the two window halves of voxels 32 (w % 4) ..) and store
// the volume, warp 8 issues the TMA loads, warp 9 owns the tensor memory and
// issues the MMAs.  Tilts go in groups of kG; each of kS group stages holds a
// group's windows in shared memory and its weights in tensor memory, with one
// "full" mbarrier (the builders and the producer arrive, the windows' bytes
// complete it) and one "empty" mbarrier (the MMAs' commit), so a group costs
// one barrier round trip and one commit.  The builders compute a group's
// weights before they wait for its stage, and read the tilts' geometry from a
// shared-memory table filled once per block.  (Prefetching the windows of
// later tilts into L2 was measured and made the kernel 25 % slower: the
// prefetches compete with the loads.)  Every wait is bounded and records a
// timeout in the plan's error word.
#include <cuda.h>

#include <cmath>
#include <cstring>

#include "gnc_common.cuh"

namespace gnc {

namespace {

constexpr int kTX = 16, kTZ = 8;  // voxel tile (x, z): 128 voxels = M
constexpr int kKW = 32;           // window pixels (two K = 16 steps)
constexpr int kG = 2;             // tilts per group: one barrier round trip per group
constexpr int kQ = 2;             // builder threads per voxel (parts of the window)
constexpr int kWords = kKW / 2 / kQ;  // tensor-memory columns one builder thread writes
constexpr int kBuilders = 128 * kQ;       // warps 0 .. 4 kQ - 1
constexpr int kThreads = kBuilders + 64;  // + TMA warp + MMA warp
constexpr int kWarpTma = kBuilders / 32, kWarpMma = kWarpTma + 1;
constexpr unsigned kHintNs = 1000;

// A shape: NR rows, at most KMAX slabs per tile and tilt, S group stages,
// TMEM tensor-memory columns and BLOCKS blocks per SM.
template <int NR, int KMAX, int S, int TMEM, int BLOCKS>
struct TcShape {
  static constexpr int kS = S, kTmemCols = TMEM;
  static constexpr int kSlabBytes = NR * kKW * 2;                // one slab's window
  static constexpr int kStageBytes = kG * KMAX * kSlabBytes;     // one group's windows
  static constexpr int kACols = kG * KMAX * (kKW / 2);           // one group's weights
  static_assert(NR + kS * kACols <= kTmemCols, "tensor memory");
  static constexpr size_t kSmem = 1024 + (size_t)kS * kStageBytes + (size_t)kTcMaxTilts * 32;
  static_assert(kSmem * BLOCKS <= 227 * 1024, "shared memory");
  static_assert(TMEM * BLOCKS <= 512, "tensor memory per SM");
  static constexpr unsigned kIdesc = (1u << 4) | ((unsigned)(NR >> 3) << 17) | ((128u >> 4) << 24);
};

constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;

typedef unsigned long long u64;

struct TcTilt {
  int u0;      // first window pixel (multiple of 8; may be negative)
  int k0, nk;  // first slab and slab count of the tile
  float wfac;  // 2^(E0 - e(t))
  float cos_a, sin_a, off;  // the tilt's geometry (reconstructor.cpp:35-47)
  float pad;
};


__device__ __forceinline__ unsigned sa(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ float voxel_coordf(int i, int n) {
  return (float)((double)i - 0.5 * (double)n + 0.5);
}
__device__ __forceinline__ float detector_coord(float xc, float zs, float off) {
  return __fsub_rn(__fadd_rn(__fsub_rn(xc, zs), off), 0.5f);
}
__device__ __forceinline__ int floor_int(float q) {
  return __float_as_int(__fadd_rd(q, kMagic)) - kMagicBits;
}

__device__ __forceinline__ void bar_init(u64 *b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sa(b)), "r"(count));
}
__device__ __forceinline__ void bar_arrive(u64 *b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(sa(b)) : "memory");
}
__device__ __forceinline__ void bar_expect_tx(u64 *b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sa(b)), "r"(bytes)
               : "memory");
}
// Bounded wait for the phase of the given parity; false (and the error word
// set) if it did not complete within `limit` polls.
__device__ __forceinline__ bool bar_wait(u64 *b, unsigned parity, unsigned limit, int *err) {
  for (unsigned it = 0; it < limit; ++it) {
    unsigned done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3; "
        "selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(sa(b)), "r"(parity), "r"(kHintNs)
        : "memory");
    if (done) return true;
  }
  if (err) atomicOr(err, 1);
  return false;
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Shared-memory operand descriptor: K-major, 64-byte swizzle, rows of 64
// bytes in 8-row atoms of 512 bytes (stride between atoms 512 B).
__device__ __forceinline__ u64 b_desc(unsigned addr) {
  u64 d = (u64)((addr & 0x3FFFFu) >> 4);
  d |= (u64)1 << 16;            // leading offset (unused for this layout)
  d |= (u64)(512 >> 4) << 32;   // stride between 8-row atoms
  d |= (u64)1 << 46;            // descriptor version
  d |= (u64)4 << 61;            // 64-byte swizzle
  return d;
}
// Instruction descriptor: FP16 A and B (K-major), FP32 D, M = 128, N rows
// (TcShape::kIdesc).
__device__ __forceinline__ void mma(unsigned d_tmem, unsigned a_tmem, u64 bdesc, unsigned idesc,
                                    unsigned acc) {
  asm volatile(
      "{ .reg .pred p; setp.ne.u32 p, %4, 0; "
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p; }" ::"r"(d_tmem),
      "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(u64 *b) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   sa(b))
               : "memory");
}

__device__ __forceinline__ void tmem_st16(unsigned taddr, const unsigned (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}
__device__ __forceinline__ void tmem_st8(unsigned taddr, const unsigned (&r)[8]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])
      : "memory");
}
__device__ __forceinline__ void tmem_st(unsigned taddr, const unsigned (&r)[8]) { tmem_st8(taddr, r); }
__device__ __forceinline__ void tmem_st(unsigned taddr, const unsigned (&r)[4]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};" ::"r"(taddr),
               "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3])
               : "memory");
}
__device__ __forceinline__ void tmem_ld32(unsigned taddr, unsigned (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
        "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),
        "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

}  // namespace

template <int NR, int KMAX, int S, int TMEM, int BLOCKS>
__global__ void __launch_bounds__(kThreads, BLOCKS)
k_bp_tc(BpArgs a, const __grid_constant__ CUtensorMap map) {
  using P = TcShape<NR, KMAX, S, TMEM, BLOCKS>;
  constexpr int kS = P::kS, kTmemCols = P::kTmemCols;
  if (a.dyn) {
    a.dscale = a.dyn[0];
    a.doffset = a.dyn[1];
  }
  extern __shared__ unsigned char smem_raw[];
  // full[g]: the 256 builders and the TMA producer arrive (plus the windows'
  // bytes); empty[g]: the MMAs of the group have completed
  __shared__ __align__(8) u64 full[kS], empty[kS], done_bar;
  __shared__ unsigned tmem_base;
  __shared__ int s_e0;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const unsigned limit = a.wait_limit ? a.wait_limit : kBpWaitLimit;
  // 1024-aligned windows (the 64-byte swizzle repeats every 512 bytes), then the tilt table
  unsigned char *win = smem_raw + ((1024u - (sa(smem_raw) & 1023u)) & 1023u);
  TcTilt *tab = (TcTilt *)(win + (size_t)kS * P::kStageBytes);

  const int ntx = (a.X + kTX - 1) / kTX;
  const int x0 = (blockIdx.x % ntx) * kTX, z0 = (blockIdx.x / ntx) * kTZ;
  const int y0 = blockIdx.y * NR;
  const int ngroups = (a.T + kG - 1) / kG;

  if (warp == kWarpMma) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     sa(&tmem_base)),
                 "r"((unsigned)kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int i = 0; i < kS; ++i) {
      bar_init(&full[i], kBuilders + 1);
      bar_init(&empty[i], 1);
    }
    bar_init(&done_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_e0 = 127;
  }
  __syncthreads();
  // the tile's window and slabs per tilt: corners inside the volume (the
  // coordinate and the slab index are monotone in x and in z)
  const float cx0 = voxel_coordf(x0, a.X), cx1 = voxel_coordf(min(x0 + kTX, a.X) - 1, a.X);
  const float cz0 = voxel_coordf(z0, a.Z), cz1 = voxel_coordf(min(z0 + kTZ, a.Z) - 1, a.Z);
  for (int t = tid; t < a.T; t += kThreads) {
    const TiltGeom g = a.geom[t];
    const float off = a.offset[t];
    const float xc0 = __fmul_rn(cx0, g.cos_a), xc1 = __fmul_rn(cx1, g.cos_a);
    const float zs0 = __fmul_rn(cz0, g.sin_a), zs1 = __fmul_rn(cz1, g.sin_a);
    const float q00 = detector_coord(xc0, zs0, off), q01 = detector_coord(xc0, zs1, off);
    const float q10 = detector_coord(xc1, zs0, off), q11 = detector_coord(xc1, zs1, off);
    const int p_lo = floor_int(fminf(fminf(q00, q01), fminf(q10, q11)));
    int k_lo = 0, k_hi = 0;
    if (a.D > 1) {
      const int k00 = slab_index(cx0, cz0, g.sin_a, g.cos_a, a.dscale, a.doffset, a.D);
      const int k01 = slab_index(cx0, cz1, g.sin_a, g.cos_a, a.dscale, a.doffset, a.D);
      const int k10 = slab_index(cx1, cz0, g.sin_a, g.cos_a, a.dscale, a.doffset, a.D);
      const int k11 = slab_index(cx1, cz1, g.sin_a, g.cos_a, a.dscale, a.doffset, a.D);
      k_lo = min(min(k00, k01), min(k10, k11));
      k_hi = max(max(k00, k01), max(k10, k11));
    }
    TcTilt tt;
    tt.u0 = p_lo & ~7;  // round down to a multiple of 8 (also for negative p_lo)
    tt.k0 = k_lo;
    tt.nk = k_hi - k_lo + 1;
    if (tt.nk > KMAX) {  // excluded by the host's choice of shape
      tt.nk = KMAX;
      if (a.err) atomicOr(a.err, 2);
    }
    tt.wfac = 0.f;
    tt.cos_a = g.cos_a;
    tt.sin_a = g.sin_a;
    tt.off = off;
    tt.pad = 0.f;
    tab[t] = tt;
    atomicMin(&s_e0, (int)a.tilt_exp[t]);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const int e0 = s_e0;
  for (int t = tid; t < a.T; t += kThreads) tab[t].wfac = pow2f(max(-126, e0 - (int)a.tilt_exp[t]));
  __syncthreads();
  const unsigned tmem = tmem_base;

  if (warp == kWarpTma) {
    // ---- TMA producer: group g's windows into stage g % kS
    if (lane == 0) {
      const int yrow = a.y_begin + y0;
      for (int g = 0; g < ngroups; ++g) {
        const int st = g % kS;
        bar_wait(&empty[st], ((g / kS) & 1) ^ 1, limit, a.err);
        unsigned bytes = 0;
        for (int j = 0; j < kG && g * kG + j < a.T; ++j) bytes += tab[g * kG + j].nk * P::kSlabBytes;
        bar_expect_tx(&full[st], bytes);  // the producer's arrival, with the bytes to come
        for (int j = 0; j < kG && g * kG + j < a.T; ++j) {
          const int i = g * kG + j;
          const TcTilt tt = tab[i];
          for (int s = 0; s < tt.nk; ++s) {
            const unsigned dst =
                sa(win + (size_t)st * P::kStageBytes + (size_t)(j * KMAX + s) * P::kSlabBytes);
            asm volatile(
                "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes "
                "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
                "l"(&map), "r"(tt.u0), "r"(yrow), "r"((tt.k0 + s) * a.T + i), "r"(sa(&full[st]))
                : "memory");
          }
        }
      }
    }
  } else if (warp == kWarpMma) {
    // ---- MMA issuer: one wait and one commit per group
    if (lane == 0) {
      for (int g = 0; g < ngroups; ++g) {
        const int st = g % kS;
        bar_wait(&full[st], (g / kS) & 1, limit, a.err);
        tc_fence_after();
        const unsigned wbase = sa(win + (size_t)st * P::kStageBytes);
        const unsigned abase = tmem + NR + st * P::kACols;
        for (int j = 0; j < kG && g * kG + j < a.T; ++j) {
          const int nk = tab[g * kG + j].nk;
          for (int s = 0; s < nk; ++s)
            for (int kk = 0; kk < 2; ++kk)
              mma(tmem, abase + (j * KMAX + s) * (kKW / 2) + kk * 8,
                  b_desc(wbase + (j * KMAX + s) * P::kSlabBytes + kk * 32), P::kIdesc,
                  (g | j | s | kk) != 0 ? 1u : 0u);
        }
        mma_commit(&empty[st]);  // the stage is free once these MMAs complete
      }
      mma_commit(&done_bar);
    }
  } else {
    // ---- weight builders: voxel m = (x0 + m % 16, z0 + m / 16) = tensor-memory
    // lane m; this thread writes part h of the window (pixels kKW / kQ h ..,
    // columns kKW / 2 / kQ h .. of each slab's block)
    const int m = 32 * (warp & 3) + lane, h = warp >> 2;
    const int x = x0 + (m & (kTX - 1)), z = z0 + (m >> 4);
    const bool inside = x < a.X && z < a.Z;
    const float xf = voxel_coordf(x, a.X), zf = voxel_coordf(z, a.Z);
    const unsigned lane_addr = (unsigned)(32 * (warp & 3)) << 16;
    for (int g = 0; g < ngroups; ++g) {
      const int st = g % kS;
      // the group's weights first (independent tilts: their arithmetic
      // interleaves), then the wait for the stage
      unsigned lo[kG], hi[kG];
      int idx[kG], blk[kG];
#pragma unroll
      for (int j = 0; j < kG; ++j) {
        const int i = min(g * kG + j, a.T - 1);
        const TcTilt tt = tab[i];
        const float q = detector_coord(__fmul_rn(xf, tt.cos_a), __fmul_rn(zf, tt.sin_a), tt.off);
        const float r = __fadd_rd(q, kMagic);
        const int fl = __float_as_int(r) - kMagicBits;
        const float tw = __fsub_rn(q, __fsub_rn(r, kMagic));
        const int k = tt.nk > 1 ? slab_index(xf, zf, tt.sin_a, tt.cos_a, a.dscale, a.doffset, a.D)
                                : tt.k0;
        const int pos = fl - tt.u0;
        // the reference skips samples unless 0 <= floor <= N - 2
        bool valid = inside && fl >= 0 && fl <= a.N - 2;
        if (valid && (pos < 0 || pos > kKW - 2)) {  // excluded by the tile's window
          valid = false;
          if (a.err) atomicOr(a.err, 4);
        }
        const unsigned h0 =
            __half_as_ushort(__float2half_rn(__fmul_rn(__fsub_rn(1.f, tw), tt.wfac)));
        const unsigned h1 = __half_as_ushort(__float2half_rn(__fmul_rn(tw, tt.wfac)));
        const u64 pair = (u64)(h0 | (h1 << 16)) << ((pos & 1) * 16);
        lo[j] = (unsigned)pair;
        hi[j] = (unsigned)(pair >> 32);
        idx[j] = (pos >> 1) - kWords * h;       // word of this part holding the pixel pair
        blk[j] = valid ? k - tt.k0 : -1;        // the slab block holding the weights
      }
      bar_wait(&empty[st], ((g / kS) & 1) ^ 1, limit, a.err);
      tc_fence_after();
      const unsigned abase = tmem + lane_addr + NR + st * P::kACols + kWords * h;
#pragma unroll
      for (int j = 0; j < kG; ++j) {
        if (g * kG + j >= a.T) break;
        const int nk = tab[g * kG + j].nk;
#pragma unroll
        for (int s = 0; s < KMAX; ++s) {
          if (s < nk) {
            const bool mine = blk[j] == s;
            unsigned w[kWords];
#pragma unroll
            for (int q = 0; q < kWords; ++q)
              w[q] = !mine ? 0u : (q == idx[j] ? lo[j] : (q == idx[j] + 1 ? hi[j] : 0u));
            tmem_st(abase + (j * KMAX + s) * (kKW / 2), w);
          }
        }
      }
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      tc_fence_before();
      bar_arrive(&full[st]);
    }
    // ---- store: the accumulator of voxel m; this thread's half of the rows
    bar_wait(&done_bar, 0, limit, a.err);
    tc_fence_after();
    const float sc = a.geom[0].scale * pow2f(max(-126, min(127, -e0)));
#pragma unroll 1
    for (int c = h * (NR / kQ); c < (h + 1) * (NR / kQ); c += 32) {
      unsigned v[32];
      tmem_ld32(tmem + lane_addr + (unsigned)c, v);
      if (inside) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int y = y0 + c + j;
          if (y < a.Y) a.vol[((size_t)y * a.Z + z) * a.X + x] = __uint_as_float(v[j]) * sc;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kWarpMma)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"((unsigned)kTmemCols));
}

// Sum of squares of each input tilt in kTiltPartsMax partial sums (float: the
// result only bounds the values to within a binade, and FP64 arithmetic is
// slow on this GPU), then one thread per tilt turns them into the exponent.

__global__ void k_tilt_sumsq(const float *__restrict__ in, size_t per_tilt, int t0,
                             float *__restrict__ part) {
  const int t = t0 + blockIdx.x, j = blockIdx.y;
  const float *p = in + (size_t)t * per_tilt;
  const size_t chunk = (per_tilt + kTiltPartsMax - 1) / kTiltPartsMax;
  const size_t b0 = (size_t)j * chunk, b1 = min(per_tilt, b0 + chunk);
  float acc = 0.f;
  size_t i = b0 + threadIdx.x;
  // float4 loads over the 16-byte aligned middle of the chunk
  const size_t a0 = min(b1, (b0 + 3) & ~(size_t)3);
  const bool vec = ((((uintptr_t)p) & 15) == 0);
  if (vec) {
    for (i = b0 + threadIdx.x; i < a0; i += blockDim.x) acc = fmaf(p[i], p[i], acc);
    const float4 *p4 = (const float4 *)(p + a0);
    const size_t n4 = (b1 - a0) / 4;
    for (size_t k = threadIdx.x; k < n4; k += blockDim.x) {
      const float4 v = __ldg(p4 + k);
      acc = fmaf(v.x, v.x, fmaf(v.y, v.y, fmaf(v.z, v.z, fmaf(v.w, v.w, acc))));
    }
    for (i = a0 + 4 * n4 + threadIdx.x; i < b1; i += blockDim.x) acc = fmaf(p[i], p[i], acc);
  } else {
    for (; i < b1; i += blockDim.x) acc = fmaf(p[i], p[i], acc);
  }
  __shared__ float w_sum[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) w_sum[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += w_sum[w];
    part[(size_t)t * kTiltPartsMax + j] = s;
  }
}

__global__ void k_tilt_exp(const float *__restrict__ part, int t0, int nt,
                           const float *__restrict__ factor, double gain,
                           int8_t *__restrict__ exp) {
  const int t = t0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= t0 + nt) return;
  double s = 0.0;
  for (int j = 0; j < kTiltPartsMax; ++j) s += (double)part[(size_t)t * kTiltPartsMax + j];
  // float partial sums are within about 1e-4 of the exact sum: one part in
  // 2^10 more keeps the bound above every value
  exp[t] = (int8_t)f16t_exponent(s * (1.0 + 1.0 / 1024.0), factor ? factor[t] : 1.0f, gain);
}

cudaError_t launch_tilt_exponents(const float *input, size_t per_tilt, int t0, int nt,
                                  const float *factor, double gain, float *part, int8_t *exp,
                                  cudaStream_t s) {
  if (nt <= 0) return cudaSuccess;
  k_tilt_sumsq<<<dim3(nt, kTiltPartsMax), 512, 0, s>>>(input, per_tilt, t0, part);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_tilt_exp<<<(nt + 127) / 128, 128, 0, s>>>(part, t0, nt, factor, gain, exp);
  return cudaGetLastError();
}

// Slabs a 16 x 8 tile can reach for one tilt: the voxel centres span at most
// sqrt(15^2 + 7^2) pixels in height (plus one for rounding); slabs are
// 1 / dscale pixels thick.
static int tc_slabs_per_tile(float dscale, int D) {
  if (D <= 1) return 1;
  const double span =
      std::sqrt((double)(kTX - 1) * (kTX - 1) + (double)(kTZ - 1) * (kTZ - 1)) + 1.0;
  return (int)std::ceil(span * std::fabs((double)dscale)) + 1;
}

bool backproject_tc_supported(int N, int T, float dscale, int D, bool uniform_centre) {
  if (!uniform_centre || N % 8 != 0 || N < 2 || T < 1 || T > kTcMaxTilts) return false;
  return tc_slabs_per_tile(dscale, D) <= 3;
}

// Rows per block of the shape a geometry uses (the TMA box height).
constexpr int kRowsTwoSlabs = 128;
int tc_rows(float dscale, int D) { return tc_slabs_per_tile(dscale, D) <= 2 ? kRowsTwoSlabs : 128; }

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

cudaError_t make_tc_map(const void *staged, int D, int T, int H, int N, int rows, TcMap *out) {
  static_assert(sizeof(CUtensorMap) == sizeof(TcMap::bytes), "tensor map size");
  static EncodeTiledFn encode = nullptr;
  if (!encode) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                     cudaEnableDefault, &q);
    if (e != cudaSuccess) return e;
    if (!fn || q != cudaDriverEntryPointSuccess) return cudaErrorNotSupported;
    encode = (EncodeTiledFn)fn;
  }
  // rows (D T, H, N) of FP16; box: 32 pixels x `rows` rows x 1 (64-byte rows, swizzled)
  cuuint64_t dims[3] = {(cuuint64_t)N, (cuuint64_t)H, (cuuint64_t)D * T};
  cuuint64_t strides[2] = {(cuuint64_t)N * 2, (cuuint64_t)H * N * 2};
  cuuint32_t box[3] = {(cuuint32_t)kKW, (cuuint32_t)rows, 1};
  cuuint32_t es[3] = {1, 1, 1};
  CUtensorMap m;
  std::memset(&m, 0, sizeof m);
  const CUresult r = encode(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, const_cast<void *>(staged),
                            dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
  std::memcpy(out->bytes, &m, sizeof m);
  out->rows = rows;
  return cudaSuccess;
}

template <int NR, int KMAX, int S, int TMEM, int BLOCKS>
static cudaError_t launch_tc(const BpArgs &a, const TcMap &map, cudaStream_t s) {
  using P = TcShape<NR, KMAX, S, TMEM, BLOCKS>;
  auto kern = k_bp_tc<NR, KMAX, S, TMEM, BLOCKS>;
  if (cudaError_t e = ensure_dynamic_smem<k_bp_tc<NR, KMAX, S, TMEM, BLOCKS>>((int)P::kSmem))
    return e;
  const int ntx = (a.X + kTX - 1) / kTX, ntz = (a.Z + kTZ - 1) / kTZ;
  dim3 grid(ntx * ntz, (a.Y + NR - 1) / NR);
  CUtensorMap m;
  std::memcpy(&m, map.bytes, sizeof m);
  kern<<<grid, kThreads, P::kSmem, s>>>(a, m);
  return cudaGetLastError();
}

cudaError_t launch_backproject_tc(const BpArgs &a, const TcMap &map, cudaStream_t s) {
  // the map's box height is the shape's row count
  if (map.rows != tc_rows(a.dscale, a.D)) return cudaErrorInvalidValue;
  // up to two slabs per tile: 256 rows, one block per SM, or 128 rows, two
  // blocks per SM (one block's set-up and volume stores overlap the other's
  // tilt loop); three slabs: 128 rows, one block per SM
  if (tc_slabs_per_tile(a.dscale, a.D) <= 2)
    return map.rows == 256 ? launch_tc<256, 2, 3, 512, 1>(a, map, s)
                           : launch_tc<128, 2, 2, 256, 2>(a, map, s);
  return launch_tc<128, 3, 3, 512, 1>(a, map, s);
}

}  // namespace gnc
