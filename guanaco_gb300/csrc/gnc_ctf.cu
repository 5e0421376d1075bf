// CTF physics: the device sign table used by the phase flip and the host
// functions behind the CTF entry points.  This file is compiled with
// -fmad=false so that double expressions keep the reference's evaluation order
// (include/guanaco/ctf.h), without fused multiply-adds.
#include <math.h>

#include <algorithm>

#include "../../include/guanaco_gb300.h"
#include "gnc_common.cuh"

namespace gnc {

// FFT-ordered spatial frequency of bin (x, y): include/guanaco/ctf.h:88-101.
__host__ __device__ inline void r_and_theta(long x, long y, long w, long h, double inv_ps,
                                            bool need_theta, double *r, double *theta) {
  long w2 = w / 2, h2 = h / 2;
  double dx = ((double)((x + w2) % w) - (double)w2) / (double)w;
  double dy = ((double)((y + h2) % h) - (double)h2) / (double)h;
  *r = sqrt((dx * dx + dy * dy) * inv_ps * inv_ps);
  *theta = need_theta ? atan2(dy, dx) : 0.0;
}

// chi: include/guanaco/ctf.h:233-238.
__host__ __device__ inline double chi(double l, double df0, double Cs, double Ca, double Pa,
                                      double q, double theta) {
  double df = df0 + Ca * cos(2 * (theta - Pa));
  return M_PI * (Cs * l * l * l * q * q * q * q / 2 - l * df * q * q);
}

// The reference stores exp(-i(chi - phi)) as complex64 (correct.py:192-211)
// and phase_flip multiplies by -sign(imag) (correct.h:30-39).
__host__ __device__ inline int flip_sign(double l, double df, double Cs, double Ca, double Pa, double phi,
                                long x, long y, long w, long h, double inv_ps) {
  double q, theta;
  r_and_theta(x, y, w, h, inv_ps, Ca != 0.0, &q, &theta);
  double a = -(chi(l, df, Cs, Ca, Pa, q, theta) - phi);
  float im = (float)sin(a);
  return -((0.0f < im) - (im < 0.0f));
}

// Float screen for the sign.  With u = a / pi,
//   u = l df q^2 - (Cs l^3 / 2) q^4 + phi / pi,
//   l df q^2 = l df0 q^2 + l Ca inv_ps^2 (cos 2Pa (dx^2 - dy^2) + sin 2Pa 2 dx dy)
// (cos(2 (theta - Pa)) expanded with cos 2theta = (dx^2 - dy^2) / r^2 and
// sin 2theta = 2 dx dy / r^2, so no transcendental is needed), and
// -sign(sin(pi u)) is +1 when floor(u) is odd and -1 when it is even.  The
// float value of u carries at most a few ulps of each term; when it lies within
// kScreen * (sum of the terms' magnitudes) + kScreenAbs of an integer the FP64
// evaluation above decides instead, so every sign equals the FP64 one.
constexpr float kScreen = 4e-6f, kScreenAbs = 1e-6f;

// FFT-ordered frequency coordinate of bin x (0 <= x < w) in float.
__host__ __device__ inline float fft_coord(int x, int w) {
  const int w2 = w / 2;
  int c = x + w2;
  c -= c >= w ? w : 0;
  return (float)(c - w2) / (float)w;
}

__host__ __device__ inline int screened_sign(const SignTableArgs &p, float ldf, int x, int y, bool *sure) {
  const float dx = fft_coord(x, p.W), dy = fft_coord(y, p.H);
  const float xx = dx * dx, yy = dy * dy, xy = 2.0f * dx * dy;
  const float q2 = (xx + yy) * p.f_ips2;
  const float t0 = ldf * q2;
  const float ta = p.f_lca * (p.f_c2p * (xx - yy) + p.f_s2p * xy);
  const float t4 = p.f_a4 * q2 * q2;
  const float u = t0 + ta - t4 + p.f_phipi;
  const float mag = fabsf(t0) + fabsf(p.f_lca) * (fabsf(xx - yy) + fabsf(xy)) + fabsf(t4) +
                    fabsf(p.f_phipi);
  const float fl = floorf(u);
  // within an ulp of 1 of the exact fraction (exact for u >= 0), far below the margin
  const float fr = u - fl;
  const float margin = kScreen * mag + kScreenAbs;
  *sure = fr > margin && fr < 1.0f - margin && fabsf(u) < 4.0e6f;
  return ((int)fl & 1) ? 1 : -1;
}

// One block per (slab, ky) row of the table at a time.
__global__ void k_sign_table(SignTableArgs a0, int8_t *__restrict__ out) {
  const SignTableArgs a = a0.dyn ? *a0.dyn : a0;
  const int sw = a.W / 2 + 1;
  const long rows = (long)a.D * a.H;
  for (long row = blockIdx.x; row < rows; row += gridDim.x) {
    const int d = (int)(row / a.H);
    const int ky = (int)(row - (long)d * a.H);
    const double df = a.slab_df[d];
    const float ldf = (float)(a.l * df);
    int8_t *o = out + row * sw;
    for (int kx = threadIdx.x; kx < sw; kx += blockDim.x) {
      bool sure;
      int s0 = screened_sign(a, ldf, kx, ky, &sure);
      if (!sure) s0 = flip_sign(a.l, df, a.Cs, a.Ca, a.Pa, a.phi, kx, ky, a.W, a.H, a.inv_ps);
      int s1;
      if (a.Ca == 0.0) {
        // without astigmatism q(-k) == q(k) bit for bit, so s(-k) == s(k)
        s1 = s0;
      } else {
        const int mx = kx == 0 ? 0 : a.W - kx, my = ky == 0 ? 0 : a.H - ky;
        s1 = screened_sign(a, ldf, mx, my, &sure);
        if (!sure) s1 = flip_sign(a.l, df, a.Cs, a.Ca, a.Pa, a.phi, mx, my, a.W, a.H, a.inv_ps);
      }
      o[kx] = (int8_t)(s0 + s1);
    }
  }
}

void fill_sign_screen(SignTableArgs *a) {
  a->f_a4 = (float)(a->Cs * a->l * a->l * a->l / 2);
  a->f_phipi = (float)(a->phi / M_PI);
  a->f_c2p = (float)cos(2 * a->Pa);
  a->f_s2p = (float)sin(2 * a->Pa);
  a->f_ips2 = (float)(a->inv_ps * a->inv_ps);
  a->f_lca = (float)(a->l * a->Ca * a->inv_ps * a->inv_ps);
}

// Packed signs for the column kernels of 128, 256, 384, 512, 1024 and 4096 rows, whose threads
// each phase-flip rows r + R m (m < M) of one column: those M signs sit
// together, 3 bits each (s + 2 for s in -2..2), 16 to a 64-bit word, entry
// (d, r, kx) = ceil(M / 16) words at ((d R + r) (W/2 + 1) + kx) ceil(M / 16).  The packed
// table follows the int8 table in the same allocation, 256-byte aligned.
static bool sign_pack_shape(int H, int *R, int *M) {
  if (H == 128 || H == 256 || H == 384 || H == 512) {  // the tiles of gnc_w512_kernels.cu
    *R = H >= 384 ? 32 : (H == 256 ? 16 : 8);
    *M = H / *R;
    return true;
  }
  if (H == 1024) {
    *R = 32;
    *M = 32;
    return true;
  }
  if (H == 4096) {
    *R = 256;
    *M = 16;
    return true;
  }
  return false;
}

bool sign_pack_used(int H) {
  int R, M;
  return sign_pack_shape(H, &R, &M);
}

static size_t sign_int8_bytes(int D, int H, int W) {
  return ((size_t)D * H * (W / 2 + 1) + 255) / 256 * 256;
}

size_t sign_table_bytes(int D, int H, int W) {
  int R, M;
  if (!sign_pack_shape(H, &R, &M)) return (size_t)D * H * (W / 2 + 1);
  return sign_int8_bytes(D, H, W) + (size_t)D * R * (W / 2 + 1) * ((M + 15) / 16) * 8;
}

const unsigned long long *sign_packed(const int8_t *sign, int D, int H, int W) {
  return (const unsigned long long *)(sign + sign_int8_bytes(D, H, W));
}

template <int R, int M>
__global__ void k_sign_pack(const int8_t *__restrict__ sign, int D, int W,
                            unsigned long long *__restrict__ out) {
  constexpr int H = R * M, NW = (M + 15) / 16;
  const int sw = W / 2 + 1;
  const long n = (long)D * R * sw;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const int kx = (int)(i % sw);
    const long dr = i / sw;
    const int r = (int)(dr % R), d = (int)(dr / R);
    const int8_t *src = sign + ((size_t)d * H + r) * sw + kx;
    unsigned long long w[NW];
#pragma unroll
    for (int j = 0; j < NW; ++j) w[j] = 0ull;
#pragma unroll
    for (int m = 0; m < M; ++m)
      w[m >> 4] |= (unsigned long long)((src[(size_t)R * m * sw] + 2) & 7) << (3 * (m & 15));
#pragma unroll
    for (int j = 0; j < NW; ++j) out[i * NW + j] = w[j];
  }
}

cudaError_t launch_sign_pack(int8_t *sign, int D, int H, int W, cudaStream_t s) {
  int R, M;
  if (!sign_pack_shape(H, &R, &M)) return cudaSuccess;
  unsigned long long *out = (unsigned long long *)(sign + sign_int8_bytes(D, H, W));
  const long n = (long)D * R * (W / 2 + 1);
  const int blocks = (int)std::min<long>((n + 255) / 256, 152 * 8);
  if (H == 128)
    k_sign_pack<8, 16><<<blocks, 256, 0, s>>>(sign, D, W, out);
  else if (H == 384)
    k_sign_pack<32, 12><<<blocks, 256, 0, s>>>(sign, D, W, out);
  else if (H == 256)
    k_sign_pack<16, 16><<<blocks, 256, 0, s>>>(sign, D, W, out);
  else if (H == 512)
    k_sign_pack<32, 16><<<blocks, 256, 0, s>>>(sign, D, W, out);
  else if (H == 1024)
    k_sign_pack<32, 32><<<blocks, 256, 0, s>>>(sign, D, W, out);
  else
    k_sign_pack<256, 16><<<blocks, 256, 0, s>>>(sign, D, W, out);
  return cudaGetLastError();
}

cudaError_t launch_sign_table(const SignTableArgs &a, int8_t *out, cudaStream_t s) {
  const long rows = (long)a.D * a.H;
  const int threads = a.W / 2 + 1 >= 256 ? 256 : 128;
  const int blocks = (int)(rows < 152 * 16 ? rows : 152 * 16);
  k_sign_table<<<blocks, threads, 0, s>>>(a, out);
  return cudaGetLastError();
}

}  // namespace gnc

// ---------------------------------------------------------------------------
// Host CTF functions (include/guanaco/ctf.h), exported through the C ABI.
// ---------------------------------------------------------------------------

namespace {
const double kC = 2.99792458e8;        // constants.h:31
const double kE = 1.602176634e-19;     // constants.h:32
const double kMe = 9.1093837015e-31;   // constants.h:33
const double kH = 6.62607004e-34;      // constants.h:34
const double kMtoA = 1e10;             // constants.h:35
}  // namespace

namespace gnc {

__host__ __device__ inline double log_Es(const gnc_ctf &c, double q, double theta) {  // ctf.h:188-195
  double df = c.df + c.Ca * cos(2 * (theta - c.Pa));
  double u = 1 + 2 * M_PI * M_PI * c.theta_c * c.theta_c * c.dd * c.dd * q * q;
  double v = c.Cs * c.l * c.l * c.l * q * q * q - df * c.l * q;
  return -(M_PI * M_PI * c.theta_c * c.theta_c * v * v / (c.l * c.l * u));
}
__host__ __device__ inline double log_Et(const gnc_ctf &c, double q) {  // ctf.h:204-209
  double u = 1 + 2 * M_PI * M_PI * c.theta_c * c.theta_c * c.dd * c.dd * q * q;
  return -(M_PI * M_PI * c.l * c.l * c.dd * c.dd * q * q * q * q / (2 * u));
}
__host__ __device__ inline double env_A(const gnc_ctf &c, double q) {  // ctf.h:218-223
  double u = 1 + 2 * M_PI * M_PI * c.theta_c * c.theta_c * c.dd * c.dd * q * q;
  return 1 / sqrt(u);
}

// One CTF quantity at (q, theta); complex kinds fill re and im, the others re.
// False for an unknown kind.  The same code runs on the host (gnc_ctf_eval)
// and in k_ctf_image.
__host__ __device__ inline bool ctf_value(const gnc_ctf &c, int kind, double q, double t,
                                          double *re, double *im) {
  switch (kind) {
    case GNC_CTF_FULL: {  // ctf.h:250-257
      double x = chi(c.l, c.df, c.Cs, c.Ca, c.Pa, q, t);
      double mag = env_A(c, q) * exp(log_Es(c, q, t) + log_Et(c, q));
      *re = mag * cos(-(x - c.phi));
      *im = mag * sin(-(x - c.phi));
      return true;
    }
    case GNC_CTF_SIMPLE: {  // ctf.h:269-273
      double x = chi(c.l, c.df, c.Cs, c.Ca, c.Pa, q, t);
      *re = cos(-(x - c.phi));
      *im = sin(-(x - c.phi));
      return true;
    }
    case GNC_CTF_SIMPLE_REAL:  // ctf.h:285-288
      *re = cos(-(chi(c.l, c.df, c.Cs, c.Ca, c.Pa, q, t) - c.phi));
      return true;
    case GNC_CTF_SIMPLE_IMAG:  // ctf.h:300-303
      *re = sin(-(chi(c.l, c.df, c.Cs, c.Ca, c.Pa, q, t) - c.phi));
      return true;
    case GNC_CTF_CHI:
      *re = chi(c.l, c.df, c.Cs, c.Ca, c.Pa, q, t);
      return true;
    case GNC_CTF_ES:  // ctf.h:314-319
      *re = exp(log_Es(c, q, t));
      return true;
    case GNC_CTF_ET:  // ctf.h:329-332
      *re = exp(log_Et(c, q));
      return true;
  }
  return false;
}

__host__ __device__ inline bool ctf_kind_complex(int kind) {
  return kind == GNC_CTF_FULL || kind == GNC_CTF_SIMPLE;
}

// CTF images of up to kCtfImageSlabs defoci per launch: slab d of the launch is
// the (h, w) FFT-ordered grid (ctf.h:466-557) at defocus df[d], written as
// float32 (complex64 for the complex kinds), (nd, h, w).
constexpr int kCtfImageSlabs = 64;
struct CtfImageArgs {
  gnc_ctf c;
  int kind, nd;
  long w, h;
  double inv_ps;
  double df[kCtfImageSlabs];
};

__global__ void k_ctf_image(CtfImageArgs a, float *__restrict__ out) {
  const long plane = a.w * a.h, n = plane * a.nd;
  const bool cplx = ctf_kind_complex(a.kind);
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const int d = (int)(i / plane);
    const long p = i - (long)d * plane;
    const long y = p / a.w, x = p - y * a.w;
    double q, theta;
    r_and_theta(x, y, a.w, a.h, a.inv_ps, true, &q, &theta);
    gnc_ctf c = a.c;
    c.df = a.df[d];
    double re = 0.0, im = 0.0;
    ctf_value(c, a.kind, q, theta, &re, &im);
    if (cplx) {
      out[2 * i] = (float)re;
      out[2 * i + 1] = (float)im;
    } else {
      out[i] = (float)re;
    }
  }
}

}  // namespace gnc

extern "C" {

double gnc_get_electron_wavelength(double V) {  // ctf.h:39-48
  double eV = kE * V;
  return (kH * kC / sqrt(eV * eV + 2 * kMe * eV * kC * kC)) * kMtoA;
}

double gnc_get_defocus_spread(double Cc, double dEE, double dII, double dVV) {  // ctf.h:61-64
  return Cc * sqrt((dEE) * (dEE) + (2 * dII) * (2 * dII) + (dVV) * (dVV));
}

double gnc_q_to_Q(double q, double l, double Cs) { return q * pow(Cs * l * l * l, 1.0 / 4.0); }
double gnc_Q_to_q(double Q, double l, double Cs) { return Q / pow(Cs * l * l * l, 1.0 / 4.0); }
double gnc_df_to_D(double df, double l, double Cs) { return df / sqrt(Cs * l); }
double gnc_D_to_df(double D, double l, double Cs) { return D * sqrt(Cs * l); }

double gnc_ctf_chi(const gnc_ctf *c, double q, double theta) {
  return gnc::chi(c->l, c->df, c->Cs, c->Ca, c->Pa, q, theta);
}

int gnc_ctf_eval(const gnc_ctf *c, int kind, const double *q, const double *theta, size_t n,
                 double *out) {
  if (!c || !q || !out || (!theta && kind != GNC_CTF_ET)) {
    gnc::set_error("gnc_ctf_eval: null pointer");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  if (kind < GNC_CTF_FULL || kind > GNC_CTF_ET) {
    gnc::set_error("gnc_ctf_eval: unknown kind");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  const int cplx = gnc::ctf_kind_complex(kind) ? 2 : 1;
  for (size_t i = 0; i < n; ++i) {
    double re = 0.0, im = 0.0;
    gnc::ctf_value(*c, kind, q[i], theta ? theta[i] : 0.0, &re, &im);
    out[cplx * i] = re;
    if (cplx == 2) out[2 * i + 1] = im;
  }
  return GNC_OK;
}

int gnc_q_and_theta(size_t w, size_t h, double ps, double *q, double *theta) {
  if (!(ps > 0) || !q || !theta) {
    gnc::set_error("gnc_q_and_theta: ps must be > 0 and outputs non-null");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  double inv_ps = 1.0 / ps;
  for (size_t j = 0; j < h; ++j)
    for (size_t i = 0; i < w; ++i)
      gnc::r_and_theta((long)i, (long)j, (long)w, (long)h, inv_ps, true, &q[j * w + i],
                       &theta[j * w + i]);
  return GNC_OK;
}

int gnc_ctf_image_device(const gnc_ctf *c, int kind, const double *defocus, int num_defocus,
                         size_t w, size_t h, double ps, void *d_out, void *stream) {
  if (!c || !defocus || !d_out || !(ps > 0) || num_defocus < 1 || w < 1 || h < 1 ||
      kind < GNC_CTF_FULL || kind > GNC_CTF_ET) {
    gnc::set_error("gnc_ctf_image_device: null pointer, ps <= 0, no defocus, empty image or "
                   "unknown kind");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  const size_t plane = w * h * (gnc::ctf_kind_complex(kind) ? 2 : 1);
  cudaStream_t s = (cudaStream_t)stream;
  for (int d0 = 0; d0 < num_defocus; d0 += gnc::kCtfImageSlabs) {
    gnc::CtfImageArgs a{};
    a.c = *c;
    a.kind = kind;
    a.nd = std::min(gnc::kCtfImageSlabs, num_defocus - d0);
    a.w = (long)w;
    a.h = (long)h;
    a.inv_ps = 1.0 / ps;
    for (int d = 0; d < a.nd; ++d) a.df[d] = defocus[d0 + d];
    const long n = (long)(w * h) * a.nd;
    const int blocks = (int)std::min<long>((n + 255) / 256, 152 * 16);
    gnc::k_ctf_image<<<blocks, 256, 0, s>>>(a, (float *)d_out + (size_t)d0 * plane);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      gnc::set_error(std::string("gnc_ctf_image_device: ") + cudaGetErrorString(e));
      return GNC_ERR_CUDA;
    }
  }
  return GNC_OK;
}

int gnc_ctf_grid(const gnc_ctf *c, int kind, size_t w, size_t h, double ps, double *out) {
  if (!c || !out || !(ps > 0)) {  // ctf.h:466-557 assert ps > 0
    gnc::set_error("gnc_ctf_grid: ps must be > 0 and pointers non-null");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  double inv_ps = 1.0 / ps;
  int cplx = (kind == GNC_CTF_FULL || kind == GNC_CTF_SIMPLE) ? 2 : 1;
  for (size_t j = 0; j < h; ++j) {
    for (size_t i = 0; i < w; ++i) {
      double q, theta;
      gnc::r_and_theta((long)i, (long)j, (long)w, (long)h, inv_ps, true, &q, &theta);
      int st = gnc_ctf_eval(c, kind, &q, &theta, 1, out + cplx * (j * w + i));
      if (st != GNC_OK) return st;
    }
  }
  return GNC_OK;
}

}  // extern "C"
