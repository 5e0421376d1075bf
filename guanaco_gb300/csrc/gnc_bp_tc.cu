// Tensor-core backprojection of F16T rows (FP16, one power-of-two scale per
// tilt) with FP32 accumulation in tensor memory.
//
// For one tilt, the backprojection of a set of voxels into a set of Y rows is
// a product V[v, y] += sum_u W[v, u] S[u, y] of the interpolation weights
// (two non-zeros per voxel: (1 - t) at the voxel's pixel floor(p), t at the
// next one, src/libguanaco/reconstructor.cpp:76-86) and the staged rows.  A
// block owns 128 voxels -- a 16 (x) by 8 (z) tile, compact so that for any
// tilt they project onto at most 18 detector pixels -- and NR Y rows (256
// when a tile reaches at most two defocus slabs per tilt, 128 for three).
// Per tilt and per defocus slab the tile reaches, it takes one slot of a ring
// of R slots in shared memory; a slot holds
//   * the 32-pixel window [u0, u0 + 32) of the NR rows (u0 a multiple of 8),
//     brought by one TMA load, 64-byte swizzled (the MMA's B operand);
//   * the 128 x 32 FP16 weights of the slab (the A operand, K-major, no
//     swizzle), written by 256 builder threads -- two per voxel, one per tilt
//     of a group -- that compute the voxel's detector coordinate, floor,
//     weight and slab with the reference's float operations, zero the row
//     and store the voxel's two weights when its slab is the slot's;
// and one thread issues two tcgen05.mma per slot (M 128 voxels, N NR rows,
// K 16 pixels each) accumulating into the 128 x NR FP32 tile in tensor
// memory.  Weights carry the tilt's factor 2^(E0 - e(t)) (E0 the smallest
// exponent over the tilts), so the accumulator counts in units of 2^-E0 for
// every tilt; the store multiplies by the backprojection scale and 2^-E0.
//
// What decides which samples a voxel takes -- its detector coordinate, floor,
// weight t, slab index and edge rule -- is the reference's float arithmetic,
// bit for bit (as in gnc_bp.cu); the products and sums are FP16 x FP16 -> FP32
// on the tensor cores.
//
// The kernel is persistent: one block per SM (its shared memory allows no
// second) takes tiles b, b + gridDim.x, ...; its j-th tile accumulates into
// accumulator j % 2 of tensor memory (2 x NR columns) and reads table buffer
// j % 2, so the next tile's table is built and the last tile's accumulator is
// stored while the current tile runs.  Warp roles (448 threads): warps 0-7
// build weights (warps w and w + 4 the first and second tilt of a group for
// voxels 32 (w % 4) ..), warp 8 issues the TMA loads (one lane per copy of a
// group), warp 9 owns the tensor memory and issues the MMAs, warps 10-13
// build each tile's tilt and group tables and store the accumulators.  Tilts
// go in groups of kG, each with a "full" mbarrier (the builders and the
// producer arrive, the windows' bytes complete it) and an "empty" one (the
// MMAs' commit); group numbers and slot counts run on across a block's tiles.
// A group's slots are consecutive in the ring, so before filling them the
// producer and the builders wait for the one earlier group that last used the
// newest of them, found when the table is built.  The builders compute a
// group's weights before that wait.
//
// Measured on the 61-tilt 1024 x 1024 x 300 ten-slab series (GB300): weights
// in tensor memory (tcgen05.st of all 32 words per voxel) 2.41 ms; weights in
// shared memory, two 16-byte zero stores and two 2-byte weight stores per
// thread and slot, 2.17 ms; persistent with the table and store overlapped
// 1.69 ms; the MMA issuer on 32-bit descriptor halves 1.62 ms; copies issued
// one lane per copy 1.60 ms.  What bounds the group loop is the window copies:
// without them (a timing-only variant, wrong volumes, every wait kept) it
// takes 1.10 ms, without the weight stores 1.61 ms, and clock stamps show the
// MMA thread waiting some 700 of a group's 1400 cycles for windows; a copy
// (one box of 32 pixels x 256 rows) keeps the copy engine busy about 300
// cycles.  Boxes of 128 rows with the same number of copies per group (16 x 16
// tiles, two MMA groups sharing each window: half the bytes per voxel) and a
// deeper window ring (copies four groups ahead) did not change the time, and
// 16-byte cp.async copies from three warps instead of the tensor copies were
// three times slower, so the number of tensor copies per group, not their bytes
// or their latency, is the bound.  Prefetching the windows of later tilts into
// L2 made the kernel 25 % slower (the prefetches compete with the loads).
// Every wait is bounded and records a timeout in the plan's error word; after
// one timeout the block's remaining waits return at once.
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "gnc_common.cuh"

namespace gnc {

namespace {

constexpr int kTX = 16, kTZ = 8;  // voxel tile (x, z): 128 voxels = M
constexpr int kKW = 32;           // window pixels (two K = 16 steps)
constexpr int kG = 2;             // tilts per group: one barrier round trip per group
constexpr int kQ = 2;             // builder threads per voxel (one per tilt of a group)
constexpr int kBuilders = 128 * kQ;       // warps 0-7
constexpr int kEpi = 128;                 // table and store threads: warps 10-13
constexpr int kThreads = kBuilders + 64 + kEpi;
constexpr int kWarpTma = kBuilders / 32, kWarpMma = kWarpTma + 1, kWarpEpi = kWarpMma + 1;
constexpr int kSB = 16;           // group barrier stages (more than the groups in flight)
constexpr unsigned kHintNs = 1000;
constexpr int kABytes = 128 * kKW * 2;  // one slab's weights: 128 voxels x 32 pixels, FP16
constexpr int kAChunk = 128 * 16;       // 8 pixels of all 128 voxels (one K core-matrix column)

// A shape: NR rows, at most KMAX slabs per tile and tilt, R slots (a slot holds
// one slab's window and weights; a tilt takes one per slab it reaches).
template <int NR, int KMAX, int R>
struct TcShape {
  static constexpr int kBBytes = NR * kKW * 2;  // one slab's window: NR rows x 32 pixels
  static constexpr int kTmemCols = 2 * NR;      // two accumulators (tile j in j % 2)
  static_assert(R >= 2 * kG * KMAX, "a slot ring holds two groups");
  // a group waits for a group at most R groups back (every group has a slot)
  static_assert(R < kSB, "waits reach back fewer groups than barrier stages");
  // per tile buffer: the tilt table and the group table
  static constexpr size_t kTabBytes = (size_t)kTcMaxTilts * 16 + (size_t)(kTcMaxTilts / kG) * 16;
  static constexpr size_t kSmem = 1024 + (size_t)R * (kBBytes + kABytes) +
                                  (size_t)kTcMaxTilts * 16 + 2 * kTabBytes;
  static_assert(kSmem <= 227 * 1024, "shared memory");
  static constexpr unsigned kIdesc = (1u << 4) | ((unsigned)(NR >> 3) << 17) | ((128u >> 4) << 24);
};

constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;

typedef unsigned long long u64;

// One tilt over one tile.
struct TcTilt {
  int u0;      // first window pixel (multiple of 8; may be negative)
  int k0, nk;  // first slab and slab count of the tile
  int slot;    // the block's running slot count at its first slab (ring slot slot % R)
};

// One group of kG tilts over one tile; group and slot counts run on over the
// block's tiles.
struct TcGroup {
  int c, n;    // first running slot and slot count of the group
  int w;       // the last earlier group that used one of these slots (-1: none)
  int pad;
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
__device__ __forceinline__ bool bar_try(u64 *b, unsigned parity) {
  unsigned done;
  asm volatile(
      "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3; "
      "selp.u32 %0, 1, 0, p; }"
      : "=r"(done)
      : "r"(sa(b)), "r"(parity), "r"(kHintNs)
      : "memory");
  return done != 0;
}
// Bounded wait for the phase of the given parity.  If it does not complete
// within `limit` polls the error word and the block's abort flag are set and
// it returns false; once the flag is set every wait returns at once, so a
// broken pipeline ends the kernel after one timeout instead of one per wait.
__device__ __forceinline__ bool bar_wait(u64 *b, unsigned parity, unsigned limit, int *err,
                                         volatile int *abort) {
  for (unsigned it = 0; it < limit; ++it) {
    if (bar_try(b, parity)) return true;
    if (*abort) return false;
  }
  *abort = 1;
  if (err) atomicOr(err, 1);
  return false;
}
// Bounded wait that ignores the abort flag (for the block's final drain).
__device__ __forceinline__ void bar_wait_plain(u64 *b, unsigned parity, unsigned limit) {
  for (unsigned it = 0; it < limit && !bar_try(b, parity); ++it) {
  }
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Shared-memory matrix descriptors, as two 32-bit halves: bits 0-13 the
// address / 16, 16-29 the leading offset / 16, 32-45 the stride offset / 16,
// bit 46 the descriptor version (1), 61-63 the swizzle mode.
//   A, a weight block: K-major, no swizzle, 8 x 16-byte core matrices;
//      8-voxel groups 128 bytes apart (stride), 8-pixel groups kAChunk apart
//      (leading offset).
//   B, a window: K-major, 64-byte swizzle, rows of 64 bytes in 8-row atoms
//      of 512 bytes (stride 512 B; the leading offset is unused).
// The high halves are constants; the low halves are address / 16 plus
// kALo / kBLo (the address never exceeds 14 bits after the shift).
constexpr unsigned kALo = (unsigned)(kAChunk >> 4) << 16;
constexpr unsigned kBLo = 1u << 16;
constexpr unsigned kAHi = (128u >> 4) | (1u << 14);
constexpr unsigned kBHi = (512u >> 4) | (1u << 14) | (4u << 29);
// D[tmem] (+)= A * B^T, FP16 inputs, FP32 accumulator; acc = 0 overwrites.
// Instruction descriptor: FP16 A and B (K-major), FP32 D, M = 128, N rows
// (TcShape::kIdesc).
__device__ __forceinline__ void mma(unsigned d_tmem, unsigned a_lo, unsigned b_lo, unsigned idesc,
                                    unsigned acc) {
  asm volatile(
      "{ .reg .pred p; .reg .b64 ad, bd; setp.ne.u32 p, %6, 0; mov.b64 ad, {%1, %2}; "
      "mov.b64 bd, {%3, %4}; tcgen05.mma.cta_group::1.kind::f16 [%0], ad, bd, %5, p; }" ::"r"(d_tmem),
      "r"(a_lo), "r"(kAHi), "r"(b_lo), "r"(kBHi), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(u64 *b) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   sa(b))
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

__device__ __forceinline__ void epi_sync() {  // the kEpi table and store threads
  asm volatile("bar.sync 1, %0;" ::"n"(kEpi) : "memory");
}

// Largest index i in [lo, hi] with gt[i].c <= target (gt[lo].c <= target).
__device__ __forceinline__ int last_group_at(const TcGroup *gt, int lo, int hi, int target) {
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (gt[mid].c <= target) lo = mid; else hi = mid - 1;
  }
  return lo;
}

struct TcTile {
  int x0, z0, y0;
};
__device__ __forceinline__ TcTile tc_tile(int tile, int ntx, int ntz, int nr) {
  TcTile t;
  t.x0 = (tile % ntx) * kTX;
  t.z0 = ((tile / ntx) % ntz) * kTZ;
  t.y0 = (tile / (ntx * ntz)) * nr;
  return t;
}

// Persistent: block b takes tiles b, b + gridDim.x, ...  Its j-th tile uses
// accumulator j % 2 and table buffer j % 2; group barriers run on across the
// tiles (the j-th tile's group g is the block's group j * ngroups + g).
template <int NR, int KMAX, int R>
__global__ void __launch_bounds__(kThreads, 1)
k_bp_tc(BpArgs a, const __grid_constant__ CUtensorMap map) {
  using P = TcShape<NR, KMAX, R>;
  if (a.dyn) {
    a.dscale = a.dyn[0];
    a.doffset = a.dyn[1];
  }
  extern __shared__ unsigned char smem_raw[];
  // full[G % kSB]: the builders and the TMA producer arrive (plus the windows'
  // bytes); empty[G % kSB]: the MMAs of group G have completed.  acc_full[b]:
  // a tile's MMAs into accumulator b have completed; acc_empty[b]: the store
  // threads have read it.  tab_full[b]: table buffer b is written; tab_empty[b]:
  // the producer, the MMA issuer and the builders are done with it.
  __shared__ __align__(8) u64 full[kSB], empty[kSB], acc_full[2], acc_empty[2], tab_full[2],
      tab_empty[2], done_bar, probe_bar;
  __shared__ unsigned tmem_base;
  __shared__ int s_e0;
  __shared__ volatile int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const unsigned limit = a.wait_limit ? a.wait_limit : kBpWaitLimit;
  // 1024-aligned windows (the 64-byte swizzle repeats every 512 bytes), then
  // the weight blocks, the tilts' constants and the two table buffers
  unsigned char *bwin = smem_raw + ((1024u - (sa(smem_raw) & 1023u)) & 1023u);
  unsigned char *awts = bwin + (size_t)R * P::kBBytes;
  float4 *tconst = (float4 *)(awts + (size_t)R * kABytes);  // cos, sin, offset, 2^(E0 - e(t))
  unsigned char *tabs = (unsigned char *)(tconst + kTcMaxTilts);
  auto tilt_tab = [&](int b) { return (TcTilt *)(tabs + b * P::kTabBytes); };
  auto group_tab = [&](int b) {
    return (TcGroup *)(tabs + b * P::kTabBytes + (size_t)kTcMaxTilts * 16);
  };

  const int ntx = (a.X + kTX - 1) / kTX, ntz = (a.Z + kTZ - 1) / kTZ;
  const int ntiles = ntx * ntz * ((a.Y + NR - 1) / NR);
  const int ngroups = (a.T + kG - 1) / kG;

  if (warp == kWarpMma) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     sa(&tmem_base)),
                 "r"((unsigned)P::kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int i = 0; i < kSB; ++i) {
      bar_init(&full[i], kBuilders + 1);
      bar_init(&empty[i], 1);
    }
    for (int b = 0; b < 2; ++b) {
      bar_init(&acc_full[b], 1);
      bar_init(&acc_empty[b], kEpi);
      bar_init(&tab_full[b], kEpi);
      bar_init(&tab_empty[b], kBuilders + 2);
    }
    bar_init(&done_bar, 1);
    bar_init(&probe_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_e0 = 127;
    s_abort = 0;
  }
  __syncthreads();
  for (int t = tid; t < a.T; t += kThreads) atomicMin(&s_e0, (int)a.tilt_exp[t]);
  __syncthreads();
  const int e0 = s_e0;
  for (int t = tid; t < a.T; t += kThreads) {
    const TiltGeom g = a.geom[t];
    tconst[t] = make_float4(g.cos_a, g.sin_a, a.offset[t],
                            pow2f(max(-126, e0 - (int)a.tilt_exp[t])));
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = tmem_base;

  if (warp == kWarpTma) {
    // ---- TMA producer: each slab's window into its slot.  Issuing one copy
    // takes a thread some 300 cycles, so lane l issues the group's l-th copy
    // (after lane 0 has armed the group's barrier for all of them).
    for (int j = 0, tile = blockIdx.x; tile < ntiles; ++j, tile += gridDim.x) {
      const int b = j & 1;
      if (lane == 0) bar_wait(&tab_full[b], (j >> 1) & 1, limit, a.err, &s_abort);
      __syncwarp();
      const TcTilt *tab = tilt_tab(b);
      const TcGroup *gtab = group_tab(b);
      const int yrow = a.y_begin + tc_tile(tile, ntx, ntz, NR).y0;
      for (int g = 0; g < ngroups; ++g) {
        const int G = j * ngroups + g;
        const TcGroup gr = gtab[g];
        if (lane == 0) {
          if (gr.w >= 0) bar_wait(&empty[gr.w % kSB], (gr.w / kSB) & 1, limit, a.err, &s_abort);
          bar_expect_tx(&full[G % kSB], (unsigned)(gr.n * P::kBBytes));
        }
        __syncwarp();
        if (lane < gr.n) {
          // copy `lane` of the group: the tilts' slabs in order
          const int i0 = g * kG;
          const int n0 = tab[i0].nk;
          const int i = lane < n0 ? i0 : i0 + 1;
          const int sl = lane < n0 ? lane : lane - n0;
          const TcTilt tt = tab[i];
          const int slot = (gr.c + lane) % R;
          asm volatile(
              "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes "
              "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(sa(bwin + (size_t)slot * P::kBBytes)),
              "l"(&map), "r"(tt.u0), "r"(yrow), "r"((tt.k0 + sl) * a.T + i),
              "r"(sa(&full[G % kSB]))
              : "memory");
        }
      }
      __syncwarp();
      if (lane == 0) bar_arrive(&tab_empty[b]);
    }
  } else if (warp == kWarpMma) {
    // ---- MMA issuer: one wait and one commit per group, accumulator j % 2
    if (lane == 0) {
      for (int j = 0, tile = blockIdx.x; tile < ntiles; ++j, tile += gridDim.x) {
        const int b = j & 1;
        bar_wait(&tab_full[b], (j >> 1) & 1, limit, a.err, &s_abort);
        if (j >= 2) bar_wait(&acc_empty[b], ((j >> 1) - 1) & 1, limit, a.err, &s_abort);
        tc_fence_after();
        const TcGroup *gtab = group_tab(b);
        const unsigned d = tmem + (unsigned)(b * NR);
        // descriptors' low halves at slot 0
        const unsigned a_lo0 = (sa(awts) >> 4) | kALo;
        const unsigned b_lo0 = (sa(bwin) >> 4) | kBLo;
        unsigned acc = 0;  // the tile's first MMA overwrites the accumulator
        for (int g = 0; g < ngroups; ++g) {
          const int G = j * ngroups + g;
          bar_wait(&full[G % kSB], (G / kSB) & 1, limit, a.err, &s_abort);
          tc_fence_after();
          // a group's slots are consecutive: running slots c .. c + n - 1,
          // tilt by tilt and slab by slab
          const TcGroup gr = gtab[g];
          int slot = gr.c % R;
          for (int i = 0; i < gr.n; ++i) {
            const unsigned a_lo = a_lo0 + (unsigned)slot * (kABytes >> 4);
            const unsigned b_lo = b_lo0 + (unsigned)slot * (P::kBBytes >> 4);
            mma(d, a_lo, b_lo, P::kIdesc, acc);  // pixels 0-15, then 16-31
            mma(d, a_lo + (2 * kAChunk >> 4), b_lo + (32 >> 4), P::kIdesc, 1);
            acc = 1;
            slot = slot + 1 == R ? 0 : slot + 1;
          }
          mma_commit(&empty[G % kSB]);  // the group's slots are free once these complete
        }
        mma_commit(&acc_full[b]);
        bar_arrive(&tab_empty[b]);
      }
      // nothing of this block's runs on the tensor cores past this point
      mma_commit(&done_bar);
      bar_wait_plain(&done_bar, 0, limit);
    }
  } else if (warp < kWarpTma) {
    // ---- weight builders: voxel m = (x0 + m % 16, z0 + m / 16) = MMA row m;
    // warps w and w + 4 write the weight rows of voxels 32 (w % 4) .. for the
    // group's first and second tilt
    static_assert(kQ == kG, "one builder thread per voxel and tilt of a group");
    const int m = 32 * (warp & 3) + lane, h = warp >> 2;
    // byte offset of (voxel m, pixel 8 c) in a weight block: 8 x 16-byte core matrices
    const unsigned roff = (unsigned)((m >> 3) * 128 + (m & 7) * 16);
    for (int j = 0, tile = blockIdx.x; tile < ntiles; ++j, tile += gridDim.x) {
      const int b = j & 1;
      const TcTile tl = tc_tile(tile, ntx, ntz, NR);
      const int x = tl.x0 + (m & (kTX - 1)), z = tl.z0 + (m >> 4);
      const bool inside = x < a.X && z < a.Z;
      const float xf = voxel_coordf(x, a.X), zf = voxel_coordf(z, a.Z);
      bar_wait(&tab_full[b], (j >> 1) & 1, limit, a.err, &s_abort);
      const TcTilt *tab = tilt_tab(b);
      const TcGroup *gtab = group_tab(b);
      for (int g = 0; g < ngroups; ++g) {
        const int G = j * ngroups + g;
        // the weights first, then the wait for the group's slots
        const int i = g * kG + h;
        const bool has = i < a.T;  // the last group of an odd tilt count has one tilt
        const TcTilt tt = tab[min(i, a.T - 1)];
        int pos = 0, blk = -1;
        unsigned short h0 = 0, h1 = 0;
        if (has) {
          const float4 tc = tconst[i];
          const float q = detector_coord(__fmul_rn(xf, tc.x), __fmul_rn(zf, tc.y), tc.z);
          const float r = __fadd_rd(q, kMagic);
          const int fl = __float_as_int(r) - kMagicBits;
          const float tw = __fsub_rn(q, __fsub_rn(r, kMagic));
          const int k = tt.nk > 1 ? slab_index(xf, zf, tc.y, tc.x, a.dscale, a.doffset, a.D)
                                  : tt.k0;
          pos = fl - tt.u0;
          // the reference skips samples unless 0 <= floor <= N - 2
          bool valid = inside && fl >= 0 && fl <= a.N - 2;
          if (valid && (pos < 0 || pos > kKW - 2)) {  // excluded by the tile's window
            valid = false;
            if (a.err) atomicOr(a.err, 4);
          }
          h0 = __half_as_ushort(__float2half_rn(__fmul_rn(__fsub_rn(1.f, tw), tc.w)));
          h1 = __half_as_ushort(__float2half_rn(__fmul_rn(tw, tc.w)));
          blk = valid ? k - tt.k0 : -1;  // the slab block holding the weights
        }
        const TcGroup gr = gtab[g];
        if (gr.w >= 0) bar_wait(&empty[gr.w % kSB], (gr.w / kSB) & 1, limit, a.err, &s_abort);
        if (has) {
#pragma unroll
          for (int sl = 0; sl < KMAX; ++sl) {
            if (sl < tt.nk) {
              unsigned char *blkp = awts + (size_t)((tt.slot + sl) % R) * kABytes + roff;
              // the row to zero, then the voxel's two weights
#pragma unroll
              for (int c = 0; c < kKW / 8; ++c)
                *(uint4 *)(blkp + c * kAChunk) = make_uint4(0, 0, 0, 0);
              if (blk == sl) {
                *(unsigned short *)(blkp + (pos >> 3) * kAChunk + (pos & 7) * 2) = h0;
                *(unsigned short *)(blkp + ((pos + 1) >> 3) * kAChunk + ((pos + 1) & 7) * 2) = h1;
              }
            }
          }
        }
        // the tensor cores read the weights through the async proxy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        bar_arrive(&full[G % kSB]);
      }
      bar_arrive(&tab_empty[b]);
    }
  } else {
    // ---- table and store threads: the table of tile j + 1 while tile j is
    // computed, then tile j's accumulator into the volume
    const int e = tid - kWarpEpi * 32;
    const int q = warp & 3, m = 32 * q + lane;
    const unsigned lane_addr = (unsigned)(32 * q) << 16;
    const float sc = a.geom[0].scale * pow2f(max(-126, min(127, -e0)));
    int slot_base = 0;  // the block's running slot count at the next tile's start
    // the j-th tile's window and slabs per tilt, running slots and group table
    auto build = [&](int j, int tile) {
      const int b = j & 1;
      if (j >= 2) bar_wait(&tab_empty[b], ((j >> 1) - 1) & 1, limit, a.err, &s_abort);
      TcTilt *tab = tilt_tab(b);
      TcGroup *gtab = group_tab(b);
      const TcGroup *prev = group_tab(b ^ 1);
      const TcTile tl = tc_tile(tile, ntx, ntz, NR);
      // corners inside the volume (the coordinate and the slab index are
      // monotone in x and in z)
      const float cx0 = voxel_coordf(tl.x0, a.X), cx1 = voxel_coordf(min(tl.x0 + kTX, a.X) - 1, a.X);
      const float cz0 = voxel_coordf(tl.z0, a.Z), cz1 = voxel_coordf(min(tl.z0 + kTZ, a.Z) - 1, a.Z);
      for (int t = e; t < a.T; t += kEpi) {
        const float4 tc = tconst[t];
        const float xc0 = __fmul_rn(cx0, tc.x), xc1 = __fmul_rn(cx1, tc.x);
        const float zs0 = __fmul_rn(cz0, tc.y), zs1 = __fmul_rn(cz1, tc.y);
        const float q00 = detector_coord(xc0, zs0, tc.z), q01 = detector_coord(xc0, zs1, tc.z);
        const float q10 = detector_coord(xc1, zs0, tc.z), q11 = detector_coord(xc1, zs1, tc.z);
        const int p_lo = floor_int(fminf(fminf(q00, q01), fminf(q10, q11)));
        int k_lo = 0, k_hi = 0;
        if (a.D > 1) {
          const int k00 = slab_index(cx0, cz0, tc.y, tc.x, a.dscale, a.doffset, a.D);
          const int k01 = slab_index(cx0, cz1, tc.y, tc.x, a.dscale, a.doffset, a.D);
          const int k10 = slab_index(cx1, cz0, tc.y, tc.x, a.dscale, a.doffset, a.D);
          const int k11 = slab_index(cx1, cz1, tc.y, tc.x, a.dscale, a.doffset, a.D);
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
        tt.slot = 0;
        tab[t] = tt;
      }
      epi_sync();
      if (e < 32) {  // running slot counts: a prefix sum of nk over the tilts
        const int chunk = (a.T + 31) / 32, t0 = e * chunk, t1 = min(a.T, t0 + chunk);
        int local = 0;
        for (int t = t0; t < t1; ++t) local += tab[t].nk;
        int incl = local;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, incl, o);
          if (e >= o) incl += v;
        }
        int run = slot_base + incl - local;
        for (int t = t0; t < t1; ++t) {
          tab[t].slot = run;
          run += tab[t].nk;
        }
        slot_base += __shfl_sync(0xffffffffu, incl, 31);
      }
      epi_sync();
      for (int g = e; g < ngroups; g += kEpi) {
        int n = 0;
        for (int jj = 0; jj < kG && g * kG + jj < a.T; ++jj) n += tab[g * kG + jj].nk;
        gtab[g].c = tab[g * kG].slot;
        gtab[g].n = n;
      }
      epi_sync();
      // the group that last used a slot of group g: the one holding running
      // slot c + n - 1 - R (groups' slots are consecutive).  It lies in this
      // tile or the one before; for an earlier tile (few slots per tile) the
      // last group of the tile before that stands in for it (a later group,
      // so a longer wait, never a shorter one).
      const int base = gtab[0].c;
      for (int g = e; g < ngroups; g += kEpi) {
        const int target = gtab[g].c + gtab[g].n - 1 - R;
        int w;
        if (target < 0) w = -1;
        else if (target >= base) w = j * ngroups + last_group_at(gtab, 0, g - 1, target);
        else if (target >= prev[0].c) w = (j - 1) * ngroups + last_group_at(prev, 0, ngroups - 1, target);
        else w = (j - 1) * ngroups - 1;
        gtab[g].w = w;
      }
      bar_arrive(&tab_full[b]);
    };
    if (blockIdx.x < ntiles) build(0, blockIdx.x);
    for (int j = 0, tile = blockIdx.x; tile < ntiles; ++j, tile += gridDim.x) {
      if (tile + (int)gridDim.x < ntiles) build(j + 1, tile + gridDim.x);
      const int b = j & 1;
      const TcTile tl = tc_tile(tile, ntx, ntz, NR);
      const int x = tl.x0 + (m & (kTX - 1)), z = tl.z0 + (m >> 4);
      const bool inside = x < a.X && z < a.Z;
      bar_wait(&acc_full[b], (j >> 1) & 1, limit, a.err, &s_abort);
      tc_fence_after();
#pragma unroll 1
      for (int c = 0; c < NR; c += 32) {
        unsigned v[32];
        tmem_ld32(tmem + lane_addr + (unsigned)(b * NR + c), v);
        if (inside) {
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            const int y = tl.y0 + c + i;
            if (y < a.Y) a.vol[((size_t)y * a.Z + z) * a.X + x] = __uint_as_float(v[i]) * sc;
          }
        }
      }
      tc_fence_before();
      bar_arrive(&acc_empty[b]);
    }
  }
  // after a timeout, the producer waits (boundedly, once more) for the copies
  // it issued in the last kSB groups, so none lands after the block ends
  if (s_abort && warp == kWarpTma && lane == 0) {
    int nt = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) ++nt;
    const int G1 = nt * ngroups;
    for (int G = max(0, G1 - kSB); G < G1; ++G) bar_wait_plain(&full[G % kSB], (G / kSB) & 1, limit);
  }
  tc_fence_before();
  __syncthreads();
  // Test hook (gnc_debug_wait_probe): after the block's work, one thread arms
  // a spare barrier for 16 bytes that no copy delivers and waits on it with the
  // probe's poll limit, so the wait gives up and sets the error word as a lost
  // copy would; nothing is in flight on that barrier.
  if (a.wait_probe && tid == 0 && blockIdx.x == 0) {
    bar_expect_tx(&probe_bar, 16);
    bar_wait(&probe_bar, 0, a.wait_probe, a.err, &s_abort);
  }
  if (warp == kWarpMma)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"((unsigned)P::kTmemCols));
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
constexpr int kRowsTwoSlabs = 256;
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

template <int NR, int KMAX, int R>
static cudaError_t launch_tc(const BpArgs &a, const TcMap &map, cudaStream_t s) {
  using P = TcShape<NR, KMAX, R>;
  auto kern = k_bp_tc<NR, KMAX, R>;
  if (cudaError_t e = ensure_dynamic_smem<k_bp_tc<NR, KMAX, R>>((int)P::kSmem)) return e;
  int dev = 0, sms = 0;
  if (cudaError_t e = cudaGetDevice(&dev)) return e;
  if (cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) return e;
  const int ntx = (a.X + kTX - 1) / kTX, ntz = (a.Z + kTZ - 1) / kTZ;
  const int ntiles = ntx * ntz * ((a.Y + NR - 1) / NR);
  CUtensorMap m;
  std::memcpy(&m, map.bytes, sizeof m);
  // one block per SM (the shared memory allows no second), each looping over tiles
  kern<<<std::min(ntiles, sms), kThreads, P::kSmem, s>>>(a, m);
  return cudaGetLastError();
}

cudaError_t launch_backproject_tc(const BpArgs &a, const TcMap &map, cudaStream_t s) {
  // the map's box height is the shape's row count
  if (map.rows != tc_rows(a.dscale, a.D)) return cudaErrorInvalidValue;
  // up to two slabs per tile: 256 rows, 8 slots; three: 128 rows, 12 slots
  return map.rows == 256 ? launch_tc<256, 2, 8>(a, map, s) : launch_tc<128, 3, 12>(a, map, s);
}

}  // namespace gnc
