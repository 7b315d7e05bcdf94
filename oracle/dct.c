/*
 * DCT-II / DCT-III (FFTW REDFT10 / REDFT01 scaling) for the CPU oracle.
 *
 * Algorithm (Makhoul, "A fast cosine transform in one and two dimensions",
 * IEEE TASSP 28(1), 1980), n a power of two:
 *   DCT-II : v[k] = x[2k], v[n-1-k] = x[2k+1];  V = FFT(v);
 *            Y[k] = 2 Re(exp(-i pi k / 2n) V[k])
 *   DCT-III: W[k] = exp(+i pi k / 2n) (X[k] - i X[n-k]),  X[n] = 0;
 *            v = sum_k W[k] exp(+2 pi i k m / n)  (unnormalised inverse FFT);
 *            y[2m] = Re v[m], y[2m+1] = Re v[n-1-m]
 * Other n: the defining sums directly.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "dct.h"

struct sbfs_dct_plan_s {
  int n;
  int pow2;
  double *fft_c, *fft_s;   /* exp(-2 pi i k / n), k < n/2 */
  int *rev;                /* bit reversal permutation */
  double *tw_c, *tw_s;     /* exp(-i pi k / 2n), k < n */
  double *cos_tab;         /* direct-sum table, n*n (non power of two only) */
};

static const double sbfs_pi = 3.14159265358979323846264338327950288;

sbfs_dct_plan *sbfs_dct_plan_create(int n) {
  if (n <= 0) return NULL;
  sbfs_dct_plan *p = (sbfs_dct_plan *)calloc(1, sizeof(*p));
  if (!p) return NULL;
  p->n = n;
  p->pow2 = (n & (n - 1)) == 0;
  p->tw_c = (double *)malloc(sizeof(double) * n);
  p->tw_s = (double *)malloc(sizeof(double) * n);
  for (int k = 0; k < n; k++) {
    const double a = sbfs_pi * k / (2.0 * n);
    p->tw_c[k] = cos(a);
    p->tw_s[k] = -sin(a);
  }
  if (p->pow2) {
    int half = n / 2 > 0 ? n / 2 : 1;
    p->fft_c = (double *)malloc(sizeof(double) * half);
    p->fft_s = (double *)malloc(sizeof(double) * half);
    for (int k = 0; k < half; k++) {
      const double a = 2.0 * sbfs_pi * k / n;
      p->fft_c[k] = cos(a);
      p->fft_s[k] = -sin(a);
    }
    p->rev = (int *)malloc(sizeof(int) * n);
    int bits = 0;
    while ((1 << bits) < n) bits++;
    for (int i = 0; i < n; i++) {
      int r = 0;
      for (int b = 0; b < bits; b++) if (i & (1 << b)) r |= 1 << (bits - 1 - b);
      p->rev[i] = r;
    }
  } else {
    p->cos_tab = (double *)malloc(sizeof(double) * (size_t)n * n);
    for (int k = 0; k < n; k++)
      for (int j = 0; j < n; j++)
        p->cos_tab[(size_t)k * n + j] = cos(sbfs_pi * (j + 0.5) * k / n);
  }
  return p;
}

void sbfs_dct_plan_destroy(sbfs_dct_plan *p) {
  if (!p) return;
  free(p->fft_c); free(p->fft_s); free(p->rev);
  free(p->tw_c); free(p->tw_s); free(p->cos_tab);
  free(p);
}

int sbfs_dct_plan_size(const sbfs_dct_plan *p) { return p ? p->n : 0; }

/* in-place radix-2 FFT of (re, im); sign = -1 forward, +1 inverse (unnormalised) */
static void fft_inplace(const sbfs_dct_plan *p, double *re, double *im, int sign) {
  const int n = p->n;
  for (int i = 0; i < n; i++) {
    const int r = p->rev[i];
    if (r > i) {
      double t = re[i]; re[i] = re[r]; re[r] = t;
      t = im[i]; im[i] = im[r]; im[r] = t;
    }
  }
  for (int len = 2; len <= n; len <<= 1) {
    const int h = len >> 1;
    const int stride = n / len;
    for (int s = 0; s < n; s += len) {
      for (int k = 0; k < h; k++) {
        const double wc = p->fft_c[k * stride];
        const double ws = sign < 0 ? p->fft_s[k * stride] : -p->fft_s[k * stride];
        const int a = s + k, b = s + k + h;
        const double tr = re[b] * wc - im[b] * ws;
        const double ti = re[b] * ws + im[b] * wc;
        re[b] = re[a] - tr; im[b] = im[a] - ti;
        re[a] = re[a] + tr; im[a] = im[a] + ti;
      }
    }
  }
}

void sbfs_dct2(const sbfs_dct_plan *p, const double *x, double *y, double *work) {
  const int n = p->n;
  if (!p->pow2) {
    double *t = work;
    for (int k = 0; k < n; k++) {
      double s = 0.0;
      for (int j = 0; j < n; j++) s += x[j] * p->cos_tab[(size_t)k * n + j];
      t[k] = 2.0 * s;
    }
    memcpy(y, t, sizeof(double) * n);
    return;
  }
  double *re = work, *im = work + n;
  for (int k = 0; k < n / 2; k++) {
    re[k] = x[2 * k];
    re[n - 1 - k] = x[2 * k + 1];
  }
  if (n == 1) re[0] = x[0];
  for (int k = 0; k < n; k++) im[k] = 0.0;
  fft_inplace(p, re, im, -1);
  for (int k = 0; k < n; k++)
    y[k] = 2.0 * (p->tw_c[k] * re[k] - p->tw_s[k] * im[k]);
}

void sbfs_dct3(const sbfs_dct_plan *p, const double *x, double *y, double *work) {
  const int n = p->n;
  if (!p->pow2) {
    double *t = work;
    for (int m = 0; m < n; m++) {
      double s = 0.0;
      for (int k = 1; k < n; k++) s += x[k] * p->cos_tab[(size_t)k * n + m];
      t[m] = x[0] + 2.0 * s;
    }
    memcpy(y, t, sizeof(double) * n);
    return;
  }
  double *re = work, *im = work + n;
  for (int k = 0; k < n; k++) {
    const double a = x[k];
    const double b = k == 0 ? 0.0 : -x[n - k];
    /* exp(+i pi k/2n) = (tw_c, -tw_s) */
    const double c = p->tw_c[k], s = -p->tw_s[k];
    re[k] = c * a - s * b;
    im[k] = c * b + s * a;
  }
  fft_inplace(p, re, im, +1);
  for (int m = 0; m < n / 2; m++) {
    y[2 * m] = re[m];
    y[2 * m + 1] = re[n - 1 - m];
  }
  if (n == 1) y[0] = re[0];
}
