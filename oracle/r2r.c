/*
 * CPU reference transforms — TEST INFRASTRUCTURE ONLY (oracle). See r2r.h for
 * the definitions restated here and the reference call sites they replace.
 */
#include "r2r.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  double re, im;
} cplx;

/* exp(sign * 2 pi i k / L), evaluated in long double and rounded once. */
static cplx unit_root(long k, long L, int sign) {
  const long double ang = 2.0L * 3.14159265358979323846264338327950288L * (long double)k / (long double)L;
  cplx w;
  w.re = (double)cosl(ang);
  w.im = (double)(sign * sinl(ang));
  return w;
}

static int smallest_factor(int n) {
  if (n % 4 == 0) return 4;
  for (int p = 2; (long)p * p <= n; ++p)
    if (n % p == 0) return p;
  return n;
}

/* Recursive mixed-radix decimation in time: y[0..n) = DFT_n of x[0], x[s], ...
 * tw holds exp(sign 2 pi i e / L) for e in [0, L); n divides L. */
static void fft_rec(const cplx *x, long s, cplx *y, int n, const cplx *tw, long L, cplx *tmp) {
  if (n == 1) {
    y[0] = x[0];
    return;
  }
  const int p = smallest_factor(n);
  const int m = n / p;
  for (int q = 0; q < p; ++q) fft_rec(x + q * s, s * p, y + (long)q * m, m, tw, L, tmp);
  const long step = L / n; /* W_n^e = tw[e * step] */
  for (int k = 0; k < m; ++k) {
    for (int q = 0; q < p; ++q) {
      const cplx a = y[(long)q * m + k];
      const cplx w = tw[((long)q * k * step) % L];
      tmp[q].re = a.re * w.re - a.im * w.im;
      tmp[q].im = a.re * w.im + a.im * w.re;
    }
    for (int r = 0; r < p; ++r) {
      double sr = 0.0, si = 0.0;
      for (int q = 0; q < p; ++q) {
        const cplx w = tw[((long)q * r * m * step) % L];
        sr += tmp[q].re * w.re - tmp[q].im * w.im;
        si += tmp[q].re * w.im + tmp[q].im * w.re;
      }
      y[k + (long)r * m].re = sr;
      y[k + (long)r * m].im = si;
    }
  }
}

/* Twiddle tables are cached per (length, sign): a solve transforms thousands
 * of lines of the same length. Not thread-safe (the oracle is single-threaded;
 * parallel CPU runs use separate processes). */
enum { kCacheSlots = 8 };
static struct {
  int L, sign;
  cplx *tw;
} tw_cache[kCacheSlots];
static int tw_next;
static cplx *tmp_buf;
static long tmp_cap;

static const cplx *twiddles(int L, int sign) {
  for (int q = 0; q < kCacheSlots; ++q)
    if (tw_cache[q].tw && tw_cache[q].L == L && tw_cache[q].sign == sign) return tw_cache[q].tw;
  const int q = tw_next;
  tw_next = (tw_next + 1) % kCacheSlots;
  free(tw_cache[q].tw);
  tw_cache[q].tw = (cplx *)malloc(sizeof(cplx) * (size_t)L);
  tw_cache[q].L = L;
  tw_cache[q].sign = sign;
  for (long e = 0; e < L; ++e) tw_cache[q].tw[e] = unit_root(e, L, sign);
  return tw_cache[q].tw;
}

static void fft(const cplx *x, cplx *y, int L, int sign) {
  const cplx *tw = twiddles(L, sign);
  if (tmp_cap < L) {
    free(tmp_buf);
    tmp_buf = (cplx *)malloc(sizeof(cplx) * (size_t)L);
    tmp_cap = L;
  }
  fft_rec(x, 1, y, L, tw, L, tmp_buf);
}

int oracle_r2r_1d(int n, int kind, const double *in, double *out) {
  if (n < 1) return -1;
  if (kind == ORACLE_REDFT00) {
    if (n < 2) return -1;
    const int L = 2 * (n - 1);
    cplx *x = (cplx *)malloc(sizeof(cplx) * (size_t)L);
    cplx *y = (cplx *)malloc(sizeof(cplx) * (size_t)L);
    for (int j = 0; j < n; ++j) x[j].re = in[j], x[j].im = 0.0;
    for (int j = n; j < L; ++j) x[j].re = in[L - j], x[j].im = 0.0;
    fft(x, y, L, -1);
    for (int k = 0; k < n; ++k) out[k] = y[k].re;
    free(x);
    free(y);
    return 0;
  }
  if (kind == ORACLE_R2HC) {
    cplx *x = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    cplx *y = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    for (int j = 0; j < n; ++j) x[j].re = in[j], x[j].im = 0.0;
    fft(x, y, n, -1);
    for (int k = 0; k <= n / 2; ++k) out[k] = y[k].re;
    for (int k = 1; k < (n + 1) / 2; ++k) out[n - k] = y[k].im;
    free(x);
    free(y);
    return 0;
  }
  if (kind == ORACLE_HC2R) {
    cplx *x = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    cplx *y = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    x[0].re = in[0], x[0].im = 0.0;
    for (int k = 1; k < (n + 1) / 2; ++k) {
      x[k].re = in[k], x[k].im = in[n - k];
      x[n - k].re = in[k], x[n - k].im = -in[n - k];
    }
    if (n % 2 == 0) x[n / 2].re = in[n / 2], x[n / 2].im = 0.0;
    fft(x, y, n, +1);
    for (int j = 0; j < n; ++j) out[j] = y[j].re;
    free(x);
    free(y);
    return 0;
  }
  return -1;
}

int oracle_r2r_1d_direct(int n, int kind, const double *in, double *out) {
  if (n < 1) return -1;
  double *res = (double *)malloc(sizeof(double) * (size_t)n);
  if (kind == ORACLE_REDFT00) {
    if (n < 2) { free(res); return -1; }
    for (int k = 0; k < n; ++k) {
      long double s = (long double)in[0] + ((k % 2) ? -(long double)in[n - 1] : (long double)in[n - 1]);
      for (int j = 1; j < n - 1; ++j)
        s += 2.0L * in[j] * cosl(3.14159265358979323846264338327950288L * (long double)((long)j * k % (2 * (n - 1))) / (long double)(n - 1));
      res[k] = (double)s;
    }
  } else if (kind == ORACLE_R2HC) {
    for (int k = 0; k <= n / 2; ++k) {
      long double s = 0;
      for (int j = 0; j < n; ++j) s += in[j] * (long double)unit_root((long)j * k % n, n, -1).re;
      res[k] = (double)s;
    }
    for (int k = 1; k < (n + 1) / 2; ++k) {
      long double s = 0;
      for (int j = 0; j < n; ++j) s += in[j] * (long double)unit_root((long)j * k % n, n, -1).im;
      res[n - k] = (double)s;
    }
  } else if (kind == ORACLE_HC2R) {
    for (int j = 0; j < n; ++j) {
      long double s = in[0];
      for (int k = 1; k < (n + 1) / 2; ++k) {
        const cplx w = unit_root((long)j * k % n, n, +1);
        s += 2.0L * ((long double)in[k] * w.re - (long double)in[n - k] * w.im);
      }
      if (n % 2 == 0) s += (j % 2 ? -1.0L : 1.0L) * in[n / 2];
      res[j] = (double)s;
    }
  } else {
    free(res);
    return -1;
  }
  memcpy(out, res, sizeof(double) * (size_t)n);
  free(res);
  return 0;
}
