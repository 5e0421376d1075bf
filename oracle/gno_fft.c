/*
 * Oracle FFT (test infrastructure only): see gno_fft.h.
 */
#include "gno_fft.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef struct gno_plan {
  size_t n;
  int nstage;
  int max_radix;
  int radix[64];
  double *wd; /* 2n doubles: re[0..n), im[0..n) of exp(-2*pi*i*k/n) */
  float *wf;  /* the same rounded to float */
  struct gno_plan *next;
} gno_plan;

static gno_plan *g_plans = NULL;
static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;

/* Radix order: 4s first, then 2, then odd primes ascending. */
static int factorize(size_t n, int *radix, int *max_radix) {
  int ns = 0;
  *max_radix = 1;
  while (n % 4 == 0) { radix[ns++] = 4; n /= 4; }
  while (n % 2 == 0) { radix[ns++] = 2; n /= 2; }
  for (size_t p = 3; n > 1; p += 2) {
    while (n % p == 0) { radix[ns++] = (int)p; n /= p; }
  }
  for (int i = 0; i < ns; ++i)
    if (radix[i] > *max_radix) *max_radix = radix[i];
  return ns;
}

static const gno_plan *get_plan(size_t n) {
  pthread_mutex_lock(&g_lock);
  for (gno_plan *p = g_plans; p; p = p->next) {
    if (p->n == n) { pthread_mutex_unlock(&g_lock); return p; }
  }
  gno_plan *p = (gno_plan *)calloc(1, sizeof(gno_plan));
  p->n = n;
  p->nstage = factorize(n, p->radix, &p->max_radix);
  p->wd = (double *)malloc(2 * n * sizeof(double));
  p->wf = (float *)malloc(2 * n * sizeof(float));
  for (size_t k = 0; k < n; ++k) {
    /* angle reduced to the first half turn keeps sin/cos accurate */
    double a = 2.0 * M_PI * (double)k / (double)n;
    p->wd[k] = cos(a);
    p->wd[n + k] = -sin(a);
    p->wf[k] = (float)p->wd[k];
    p->wf[n + k] = (float)p->wd[n + k];
  }
  p->next = g_plans;
  g_plans = p;
  pthread_mutex_unlock(&g_lock);
  return p;
}

static const double *roots_re_d(const gno_plan *p) { return p->wd; }
static const double *roots_im_d(const gno_plan *p) { return p->wd + p->n; }
static const float *roots_re_f(const gno_plan *p) { return p->wf; }
static const float *roots_im_f(const gno_plan *p) { return p->wf + p->n; }

#define GNO_T double
#define GNO_SFX d
#include "gno_fft_impl.inc"
#undef GNO_T
#undef GNO_SFX

#define GNO_T float
#define GNO_SFX f
#include "gno_fft_impl.inc"
#undef GNO_T
#undef GNO_SFX
