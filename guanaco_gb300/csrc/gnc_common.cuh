// Internal interfaces shared by the guanaco_gb300 CUDA translation units.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "gnc_fft.cuh"

namespace gnc {

// ---- errors -------------------------------------------------------------
void set_error(const std::string &msg);
const char *last_error();

// ---- FFT plans: factorisation + device twiddles, cached per (device, n) ---
// Returns false (and sets the error) when n has a prime factor > kMaxRadix.
bool make_fft_plan(int n, FftPlan *out);
bool fft_length_supported(long n);
// The factorisation only (roots left null, nothing allocated); false when n
// has a prime factor > kMaxRadix.
bool make_fft_factors(int n, FftPlan *out);

// ---- staging element types ------------------------------------------------
enum Staging : int { kStageF32 = 0, kStageF16 = 1, kStageF16T = 2 };

// One staged detector pixel n of a row pair (rows a = 2 y2, b = 2 y2 + 1):
//   F32: float2 (v_a, v_b)                                              8 bytes
//   F16: half2 (v_a, v_b) and half2 (v_a[n+1] - v_a[n], v_b[n+1] - v_b[n]),
//        each row scaled by its 2^e, the difference taken between the two
//        rounded FP16 values (0 for the last pixel), so the backprojector's
//        interpolation is one load and one half2 FMA                    8 bytes
constexpr int kStagedPixelBytes = 8;
// v0, v1: pixels n and n + 1 already multiplied by the rows' 2^e
__device__ __forceinline__ uint2 staged_record_f16(float2 v0, float2 v1) {
  const __half2 h0 = __floats2half2_rn(v0.x, v0.y), h1 = __floats2half2_rn(v1.x, v1.y);
  const float2 f0 = __half22float2(h0), f1 = __half22float2(h1);
  const __half2 dv = __floats2half2_rn(f1.x - f0.x, f1.y - f0.y);
  uint2 r;
  r.x = *(const unsigned *)&h0;
  r.y = *(const unsigned *)&dv;
  return r;
}

// F16T staging (the tensor-core backprojector): plain FP16 rows (D, T, H, N),
// row y of slab d and tilt t at ((d T + t) H + y) N, every value of tilt t
// multiplied by 2^e(t) with one exponent per tilt (int8, T).  e(t) comes from
// a bound on every filtered value of the tilt: |factor_t| * gain * ||input_t||_2
// (gain = H W for the unnormalised CTF correction, 1 otherwise; the phase flip
// and the ramp filter do not increase the L2 norm, and no value of a vector
// exceeds its L2 norm), brought just below 2^14, so no value overflows FP16
// and the largest keeps full precision unless the bound is more than 2^16 loose.
__host__ __device__ __forceinline__ int f16t_exponent(double norm2, float factor, double gain) {
  const double b = fabs((double)factor) * gain * sqrt(norm2);
  if (!(b > 0.0) || !(b < 1e300)) return 0;  // zero, NaN or inf: nothing to scale
  int ex = 0;
  frexp(b, &ex);  // b = m 2^ex, m in [0.5, 1): b 2^(14 - ex) < 2^14
  const int e = 14 - ex;
  return e < -100 ? -100 : (e > 100 ? 100 : e);
}
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + e) << 23); }

// Per-tilt backprojection geometry, computed on the host with the reference's
// float arithmetic (src/libguanaco/reconstructor.cpp:35-47).
struct TiltGeom {
  float cos_a;  // cos(theta) / d
  float sin_a;  // sin(theta) / d
  float scale;  // pi / (2 T) * ray_length / |d|
  float pad;
};

// ---- kernels (launchers return the launch error) ---------------------------

// Row transform of the raw projections: rows (t, 2p) and (t, 2p+1) are packed
// as one complex row, transformed and unpacked into two half spectra of W/2
// bins with the DC and Nyquist real parts packed in bin 0.
// proj (T, H, W) -> spec (T, H, W/2).
cudaError_t launch_rfft_rows(const float *proj, float2 *spec, int T, int H, int W,
                             cudaStream_t s);

// Forward column transform of every tilt's half spectrum, in place.
cudaError_t launch_column_fft(float2 *spec, int T, int H, int W, cudaStream_t s);

// Per-slab phase flip and inverse column transform for the tilts
// [t0, t0 + nt) of the column-transformed spectra: spec (T, H, W/2) ->
// g (nt, D, H, W/2).
// sign: (D, H, W/2 + 1) int8 holding 2 * (s(k) + s(-k)) / 2.
// Bytes of a sign table allocation for (D, H, W): the int8 table (D, H, W/2+1)
// and, for 128, 256, 384, 512, 1024 and 4096 rows, the packed copy the column kernels of those
// sizes read (written by launch_sign_pack after launch_sign_table).
size_t sign_table_bytes(int D, int H, int W);
bool sign_pack_used(int H);
const unsigned long long *sign_packed(const int8_t *sign, int D, int H, int W);
cudaError_t launch_sign_pack(int8_t *sign, int D, int H, int W, cudaStream_t s);
// Sign m (0..15) of a packed word.
__device__ __forceinline__ int packed_sign(unsigned long long w, int m) {
  return (int)((w >> (3 * m)) & 7ull) - 2;
}
// live: per tilt, the first and last slab any voxel of the volume reads (the
// flip and the row stage skip the other (tilt, slab) pairs), or null: all.
cudaError_t launch_column_flip(const float2 *spec, float2 *g, const int8_t *sign, int t0, int nt,
                               int D, int H, int W, const int2 *live, cudaStream_t s);
// Whether slab d of tilt t is read by any voxel (live as above).
__device__ __forceinline__ bool slab_live(const int2 *live, int t, int d) {
  if (!live) return true;
  const int2 r = live[t];
  return d >= r.x && d <= r.y;
}

// The 2 * symmetrised phase-flip sign for every (slab, ky, kx <= W/2), from the
// FP64 CTF phase (include/guanaco/ctf.h:88-101, 233-273; correct.h:30-39).
// The kernel first screens each sign in float (fill_sign_screen sets the f_*
// fields) and evaluates the FP64 phase only where the screen cannot decide.
struct SignTableArgs {
  int D, H, W;
  double inv_ps;
  double l, Cs, Ca, Pa, phi;
  const double *slab_df;  // device, D
  float f_a4, f_phipi, f_c2p, f_s2p, f_ips2, f_lca;
  // device copy of these arguments, or null: when set the kernel reads its
  // arguments there (a captured launch then serves every request of a plan)
  const SignTableArgs *dyn;
};
void fill_sign_screen(SignTableArgs *a);
cudaError_t launch_sign_table(const SignTableArgs &a, int8_t *out, cudaStream_t s);

// Row stage.  Input rows come either from the column stage (packed half
// spectra, INPUT_SPECTRA) or from real rows.  Each pair of rows is one complex
// row.  With RAMP the rows are zero padded to 2N, ramp filtered
// (src/libguanaco/filter.cpp:30-97) and divided by 2N; without it they are the
// corrected rows (correct.cpp:78-84).  Output is either the staged pair layout
// for the backprojector or plain real rows.
struct RowStageArgs {
  // input
  int input_spectra;     // 1: packed half spectra (G), 0: real rows
  const float2 *g;       // (nt, D, H, W/2) when input_spectra
  const float *rows;     // real rows when !input_spectra
  long row_stride;       // floats between consecutive input rows (y)
  long plane_stride;     // floats between consecutive (t, d) planes of rows
  // geometry
  int nt, D, H, N;       // tilts in this launch, slabs, rows per image, row length
  int t0;                // first tilt of this launch (into weights/output)
  int T;                 // total tilts (output layout)
  int y2_begin;          // first row pair of this launch
  int y2_count;          // row pairs in this launch; 0: all (H + 1) / 2
  int ramp;              // apply the ramp filter
  // per-tilt factor (weight * sign) or null
  const float *tilt_factor;
  // output
  int out_staged;        // 1: staged pairs (Y2, D, T, N), 0: plain rows
  int staging;           // kStageF32 / kStageF16 / kStageF16T when out_staged
  void *staged;          // float2 pairs, FP16 records, or F16T rows
  int8_t *row_exp;       // (Y2, D, T, 2) FP16 exponents when staging == F16
  const int8_t *tilt_exp;  // (T) exponents e(t) when staging == F16T
  float *out_rows;       // plain rows: (nt, D, H, N) at [t][d][y][n]
  const int2 *live;      // per tilt (first, last) slab the volume reads; others are
                         // skipped (staged output only), or null: all slabs
};
cudaError_t launch_row_stage(const RowStageArgs &a, cudaStream_t s);

// Raises a kernel's dynamic shared-memory limit on the current device.  The
// attribute belongs to the device's context, so it is set before every launch
// (a cheap host call): a process that launches on several GPUs, or whose
// context was torn down and rebuilt, gets it on the context it launches in.
template <auto KERNEL>
inline cudaError_t ensure_dynamic_smem(int bytes) {
  return cudaFuncSetAttribute(KERNEL, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}
// F16T: row y of slab d and tilt t in the staged stack, and the tilt's scale.
__device__ __forceinline__ __half *f16t_row(const RowStageArgs &a, int d, int t, int y) {
  return (__half *)a.staged + (((size_t)d * a.T + t) * a.H + y) * (size_t)a.N;
}
__device__ __forceinline__ float f16t_scale(const RowStageArgs &a, int t) {
  return __int_as_float((127 + (int)a.tilt_exp[t]) << 23);
}
// Row pairs a row-stage launch covers: rows 2 y2_begin .. of every (tilt, slab).
__host__ __device__ inline int row_pairs(const RowStageArgs &a) {
  return a.y2_count > 0 ? a.y2_count : (a.H + 1) / 2;
}

// Backprojection of the staged pairs into the volume (Y, Z, X).
struct BpArgs {
  const void *staged;     // (Y2, D, T, N) float2 pairs / FP16 records
  const int8_t *row_exp;  // F16 exponents or null
  int staging;
  int Y, D, T, N, Z, X;
  const TiltGeom *geom;   // T
  const float *offset;    // (Y, T): detector offset of each row (depends on its centre)
  float dscale, doffset;  // slab map (reconstructor.cpp:28-32)
  int uniform_centre;     // all rows share one centre
  float *vol;             // (Y, Z, X)
  int *err;               // device error word (bounded waits that gave up), or null
  const float *dyn;       // device (dscale, doffset) overriding the two above, or null
  unsigned wait_limit;    // polls before a bulk-copy wait gives up (0: kBpWaitLimit)
  unsigned wait_probe;    // test hook, 0 = off: see gnc_debug_wait_probe
  const int8_t *tilt_exp; // F16T: (T) per-tilt exponents (staged = F16T rows)
  int y_begin;            // F16T: stack row of this launch's first volume row
  int stack_h;            // F16T: rows of each (slab, tilt) plane of the staged stack
};
// Default poll limit of the backprojector's bounded mbarrier waits (each poll
// suspends for at most about 2 us, so about 2 s in all).
constexpr unsigned kBpWaitLimit = 1u << 20;
// The fast kernel's requirements (shared centre, 16-byte aligned rows, at most
// four slabs per tile); launch_backproject_fast falls back to the exact kernel.
bool backproject_fast_supported(const BpArgs &a);
// Which backprojection kernel a launch with these arguments uses: 0 the exact
// kernel, else the fast kernel's slab capacity per tile (2 or 4).
int backproject_fast_variant(const BpArgs &a);
cudaError_t launch_backproject_exact(const BpArgs &a, cudaStream_t s);
cudaError_t launch_backproject_fast(const BpArgs &a, cudaStream_t s);
cudaError_t launch_slab_map(const BpArgs &a, int32_t *out, cudaStream_t s);
// Per tilt, the first and last slab any voxel of the (Z, X) volume reads:
// the slab index is monotone in x and in z, so the extremes lie at the
// volume's corners (the same float expression as the backprojectors).
cudaError_t launch_live_slabs(const BpArgs &a, int2 *live, cudaStream_t s);

// ---- tensor-core backprojection of F16T rows (gnc_bp_tc.cu) -----------------
// Whether the tensor-core kernel takes this geometry (shared centre, width a
// multiple of 8, at most kTcMaxTilts tilts, at most kTcMaxSlabs slabs per tile).
constexpr int kTcMaxTilts = 512;
bool backproject_tc_supported(int N, int T, float dscale, int D, bool uniform_centre);
// The TMA descriptor of F16T rows at `staged` for (D, T, H, N); 128 bytes,
// passed to the kernel by value.
struct TcMap {
  alignas(64) unsigned char bytes[128];
  int rows;  // Y rows of one tile (the kernel shape it serves)
};
// Rows per block of the kernel shape for this slab map: 256 (at most two slabs
// per tile and tilt) or 128 (three).
int tc_rows(float dscale, int D);
cudaError_t make_tc_map(const void *staged, int D, int T, int H, int N, int rows, TcMap *out);
cudaError_t launch_backproject_tc(const BpArgs &a, const TcMap &map, cudaStream_t s);
// Per-tilt F16T exponents of the input (T tilts of `per_tilt` floats, tilts
// [t0, t0 + nt)): exp[t] = f16t_exponent(||input_t||^2, factor[t], gain);
// `part` holds kTiltPartsMax floats per tilt of scratch.
constexpr int kTiltPartsMax = 16;
cudaError_t launch_tilt_exponents(const float *input, size_t per_tilt, int t0, int nt,
                                  const float *factor, double gain, float *part, int8_t *exp,
                                  cudaStream_t s);

// Single-slice backprojection of plain filtered rows (D, T, N) into (Z, X):
// the per-call path of guanaco.detail.recon.
struct SliceBpArgs {
  const float *sino;  // (D, T, N)
  int D, T, N, Z, X;
  const TiltGeom *geom;
  float offset;
  float dscale, doffset;
  float *rec;          // (Z, X)
};
cudaError_t launch_backproject_slice(const SliceBpArgs &a, cudaStream_t s);

// Register-resident FFT kernels for power-of-two lengths 256 .. 4096
// (gnc_pow2_kernels.cu); the launchers above use them when pow2_fast(size).
bool pow2_fast(long n);
cudaError_t launch_rfft_rows_p2(const float *proj, float2 *spec, int T, int H, int W,
                                cudaStream_t s);
cudaError_t launch_column_fft_p2(float2 *spec, int T, int H, int W, cudaStream_t s);
cudaError_t launch_column_flip_p2(const float2 *spec, float2 *g, const int8_t *sign, int t0,
                                  int nt, int D, int H, int W, const int2 *live, cudaStream_t s);
cudaError_t launch_row_stage_p2(const RowStageArgs &a, cudaStream_t s);

// One-warp register FFT kernels for 1024-point rows / columns
// (gnc_w1024_kernels.cu); the launchers above prefer them for that size.
cudaError_t launch_rfft_rows_w1024(const float *proj, float2 *spec, int T, int H, cudaStream_t s);
cudaError_t launch_column_fft_w1024(float2 *spec, int T, int W, cudaStream_t s);
cudaError_t launch_column_flip_w1024(const float2 *spec, float2 *g, const int8_t *sign, int t0,
                                     int nt, int D, int W, const int2 *live, cudaStream_t s);
cudaError_t launch_row_stage_w1024(const RowStageArgs &a, cudaStream_t s);
// Register-transform kernels for 128-, 256-, 384- and 512-pixel columns and rows
// (gnc_w512_kernels.cu); the launchers above prefer them for those sizes.
cudaError_t launch_column_fft_w512(float2 *spec, int T, int H, int W, cudaStream_t s);
cudaError_t launch_column_flip_w512(const float2 *spec, float2 *g, const int8_t *sign, int t0,
                                    int nt, int D, int H, int W, const int2 *live,
                                    cudaStream_t s);
cudaError_t launch_row_stage_w512(const RowStageArgs &a, cudaStream_t s);
// Block-transform kernels for 4096-pixel columns and rows
// (gnc_b4096_kernels.cu); the launchers above prefer them for that size.
cudaError_t launch_column_fft_b4096(float2 *spec, int T, int W, cudaStream_t s);
cudaError_t launch_column_flip_b4096(const float2 *spec, float2 *g, const int8_t *sign, int t0,
                                     int nt, int D, int W, const int2 *live, cudaStream_t s);
cudaError_t launch_row_stage_b4096(const RowStageArgs &a, cudaStream_t s);

// Exact slab index of the reference (reconstructor.cpp:66-72): the height and
// defocus coordinate in float without contraction, then
// floor((double)defocus + 0.5) clamped to [0, D-1].  floor(d + 0.5) equals
// floor(d) + (d - floor(d) >= 0.5); d - floor(d) is exact for d >= 0 (Sterbenz)
// and any rounding for d in (-1, 0) only moves the result between -1 and 0,
// which the clamp maps to 0 alike.
__device__ __forceinline__ int slab_index(float x, float y, float sin_a, float cos_a,
                                          float dscale, float doffset, int D) {
  float height = __fsub_rn(__fmul_rn(-x, sin_a), __fmul_rn(y, cos_a));
  float defocus = __fadd_rn(__fmul_rn(height, dscale), doffset);
  float fl = floorf(defocus);
  float fr = __fsub_rn(defocus, fl);
  int k = (int)fl + (fr >= 0.5f ? 1 : 0);
  k = k < 0 ? 0 : k;
  return k > D - 1 ? D - 1 : k;
}

}  // namespace gnc
