/*
 * oracle_fft.c — TEST INFRASTRUCTURE ONLY: the oracle's own FFT.
 *
 * The reference calls FFTW 3.3.4 (not vendored; configure.sh:131-139 fetches
 * fftw-3.3.4.tar.gz) through fftw_plan_dft_r2c_3d / fftw_plan_dft_c2r_3d with
 * the dimensions reversed (energy.F90:6931-6932), i.e. a real mesh Q(x,y,z)
 * with x fastest is transformed to FQ(0:n/2, y, z).  FFTW's published
 * conventions: forward = sum_j x_j exp(-2 pi i jk/n), backward = exp(+...),
 * both unnormalised; c2r assumes Hermitian input.  This file restates those
 * conventions: power-of-two lengths (every mesh here) by an iterative
 * radix-2 FFT with two real lines packed into one complex transform, other
 * lengths by a plain recursive mixed-radix (2, 3, 5, generic) DFT, all in
 * double precision with long-double twiddles; it is checked against
 * numpy.fft in tests.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "molsim_oracle.h"
#include "oracle_par.h"

typedef struct { double re, im; } cpx;

static const double ORC_PI = 3.14159265358979323846264338327950288;

/* Twiddle table of the top-level length N: w[j] = exp(-2 pi i j/N), computed
   once per length in long double and rounded to double. */
typedef struct { int n; cpx *w; } twiddles;
static twiddles tw_cache[8];

static const cpx *get_twiddles(int n) {
    for (int i = 0; i < 8; ++i) if (tw_cache[i].n == n) return tw_cache[i].w;
    int slot = 0;
    for (int i = 0; i < 8; ++i) if (tw_cache[i].n == 0) { slot = i; break; }
    free(tw_cache[slot].w);
    cpx *w = malloc(sizeof(cpx) * n);
    for (int j = 0; j < n; ++j) {
        long double a = -2.0L * (long double)ORC_PI * (long double)j / (long double)n;
        w[j].re = (double)cosl(a); w[j].im = (double)sinl(a);
    }
    tw_cache[slot].n = n; tw_cache[slot].w = w;
    return w;
}

static inline cpx tw(const cpx *w, int N, long idx, int sign) {
    cpx t = w[idx % N];
    if (sign > 0) t.im = -t.im;
    return t;
}

/* out[k] = sum_j in[j*stride] exp(sign*2 pi i jk/n); recursive decimation in
   time; w is the table of the top-level length N (N a multiple of n). */
static void dft_rec(int n, const cpx *in, int stride, cpx *out, int sign, cpx *tmp,
                    const cpx *w, int N) {
    if (n == 1) { out[0] = in[0]; return; }
    int r = 0;
    if (n % 4 == 0) r = 4; else if (n % 2 == 0) r = 2; else if (n % 3 == 0) r = 3;
    else if (n % 5 == 0) r = 5;
    long f = N / n;
    if (r == 0) {   /* plain DFT for other prime factors */
        for (int k = 0; k < n; ++k) {
            double sr = 0, si = 0;
            for (int j = 0; j < n; ++j) {
                cpx t = tw(w, N, (long)j * k % n * f, sign);
                sr += in[j * stride].re * t.re - in[j * stride].im * t.im;
                si += in[j * stride].re * t.im + in[j * stride].im * t.re;
            }
            tmp[k].re = sr; tmp[k].im = si;
        }
        memcpy(out, tmp, sizeof(cpx) * n);
        return;
    }
    int m = n / r;
    for (int q = 0; q < r; ++q) dft_rec(m, in + q * stride, stride * r, out + q * m, sign, tmp, w, N);
    for (int k = 0; k < m; ++k) {
        cpx v[5];
        for (int q = 0; q < r; ++q) {
            cpx t = tw(w, N, (long)q * k * f, sign);
            cpx x = out[q * m + k];
            v[q].re = x.re * t.re - x.im * t.im;
            v[q].im = x.re * t.im + x.im * t.re;
        }
        for (int t = 0; t < r; ++t) {
            double sr = 0, si = 0;
            for (int q = 0; q < r; ++q) {
                cpx c = tw(w, N, (long)((q * t) % r) * (N / r), sign);
                sr += v[q].re * c.re - v[q].im * c.im;
                si += v[q].re * c.im + v[q].im * c.re;
            }
            tmp[t * m + k].re = sr; tmp[t * m + k].im = si;
        }
    }
    memcpy(out, tmp, sizeof(cpx) * n);
}

/* ---- power-of-two lengths: iterative radix-2 (decimation in time) ------- */

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

/* in-place FFT of a power-of-two length n with the table w of length n
   (w[j] = exp(-2 pi i j / n)); sign -1 forward, +1 backward */
static void fft_pow2(int n, cpx *a, int sign, const cpx *w) {
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) { cpx t = a[i]; a[i] = a[j]; a[j] = t; }
    }
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1, step = n / len;
        for (int i = 0; i < n; i += len)
            for (int k = 0; k < half; ++k) {
                cpx t = w[k * step];
                if (sign > 0) t.im = -t.im;
                cpx u = a[i + k], v = a[i + k + half];
                cpx x = {v.re * t.re - v.im * t.im, v.re * t.im + v.im * t.re};
                a[i + k].re = u.re + x.re; a[i + k].im = u.im + x.im;
                a[i + k + half].re = u.re - x.re; a[i + k + half].im = u.im - x.im;
            }
    }
}

static void dft_line(int n, cpx *line, int sign, cpx *work) {
    if (is_pow2(n)) { fft_pow2(n, line, sign, get_twiddles(n)); return; }
    cpx *in = work, *tmp = work + n;
    memcpy(in, line, sizeof(cpx) * n);
    dft_rec(n, in, 1, line, sign, tmp, get_twiddles(n), n);
}

/* complex FFTs of the columns c of a (n, ncol) array of stride `stride`
   between rows, in blocks of adjacent columns for cache locality */
#define COLBLK 8
static void fft_columns(int n, cpx *base, size_t stride, int ncol, int sign, cpx *buf, cpx *work) {
    for (int c0 = 0; c0 < ncol; c0 += COLBLK) {
        int nc = ncol - c0 < COLBLK ? ncol - c0 : COLBLK;
        for (int t = 0; t < n; ++t)
            for (int c = 0; c < nc; ++c) buf[(size_t)c * n + t] = base[(size_t)t * stride + c0 + c];
        for (int c = 0; c < nc; ++c) dft_line(n, buf + (size_t)c * n, sign, work);
        for (int t = 0; t < n; ++t)
            for (int c = 0; c < nc; ++c) base[(size_t)t * stride + c0 + c] = buf[(size_t)c * n + t];
    }
}

/* The 3D transforms split their independent lines among the oracle's threads
   (oracle_par.h); every line is transformed the same way, so the result does
   not depend on the thread count. */
typedef struct {
    int n, sign, pass;   /* pass 0: x lines, 1: columns per z plane, 2: columns per y row */
    const double *q;     /* r2c input */
    double *qo;          /* c2r output */
    cpx *fq;
    int err;
} fft_task;

static void fft_x_r2c(fft_task *k, long p0, long p1, cpx *line, cpx *work) {
    int n = k->n, nh = n / 2 + 1;
    size_t nl = (size_t)n * n;
    for (long pr = p0; pr < p1; ++pr) {
        size_t l = 2 * (size_t)pr;
        const double *a = k->q + l * n, *b = (l + 1 < nl) ? k->q + (l + 1) * n : NULL;
        for (int x = 0; x < n; ++x) { line[x].re = a[x]; line[x].im = b ? b[x] : 0.0; }
        dft_line(n, line, -1, work);
        cpx *fa = k->fq + l * nh, *fb = k->fq + (l + 1) * nh;
        for (int kk = 0; kk < nh; ++kk) {
            cpx z = line[kk], zc = line[(n - kk) % n];
            fa[kk].re = 0.5 * (z.re + zc.re);
            fa[kk].im = 0.5 * (z.im - zc.im);
            if (b) {
                fb[kk].re = 0.5 * (z.im + zc.im);
                fb[kk].im = -0.5 * (z.re - zc.re);
            }
        }
    }
}

static void fft_x_c2r(fft_task *k, long p0, long p1, cpx *line, cpx *work) {
    int n = k->n, nh = n / 2 + 1;
    size_t nl = (size_t)n * n;
    for (long pr = p0; pr < p1; ++pr) {
        size_t l = 2 * (size_t)pr;
        const cpx *ha = k->fq + l * nh, *hb = (l + 1 < nl) ? k->fq + (l + 1) * nh : NULL;
        for (int kq = 0; kq < n; ++kq) {
            cpx xa, xb = {0.0, 0.0};
            int kk = kq < nh ? kq : n - kq;
            double sg = kq < nh ? 1.0 : -1.0;
            xa.re = ha[kk].re; xa.im = sg * ha[kk].im;
            if (hb) { xb.re = hb[kk].re; xb.im = sg * hb[kk].im; }
            if (kk == 0 || 2 * kk == n) { xa.im = 0.0; xb.im = 0.0; }
            line[kq].re = xa.re - xb.im;
            line[kq].im = xa.im + xb.re;
        }
        dft_line(n, line, +1, work);
        double *qa = k->qo + l * n, *qb = hb ? k->qo + (l + 1) * n : NULL;
        for (int x = 0; x < n; ++x) {
            qa[x] = line[x].re;
            if (qb) qb[x] = line[x].im;
        }
    }
}

static void fft_task_run(void *ctx, int t, int nt) {
    fft_task *k = (fft_task *)ctx;
    int n = k->n, nh = n / 2 + 1;
    cpx *line = malloc(sizeof(cpx) * n), *work = malloc(sizeof(cpx) * 2 * n);
    cpx *buf = malloc(sizeof(cpx) * COLBLK * (size_t)n);
    if (!line || !work || !buf) {
        k->err = 1;
        free(line); free(work); free(buf);
        return;
    }
    long lo, hi;
    if (k->pass == 0) {
        long npair = ((long)n * n + 1) / 2;
        orc_range(npair, t, nt, &lo, &hi);
        if (k->q) fft_x_r2c(k, lo, hi, line, work);
        else fft_x_c2r(k, lo, hi, line, work);
    } else {
        orc_range(n, t, nt, &lo, &hi);
        for (long i = lo; i < hi; ++i) {
            if (k->pass == 1) fft_columns(n, k->fq + (size_t)i * n * nh, nh, nh, k->sign, buf, work);
            else fft_columns(n, k->fq + (size_t)i * nh, (size_t)n * nh, nh, k->sign, buf, work);
        }
    }
    free(line); free(work); free(buf);
}

static int fft_pass(fft_task *k, int pass, int sign) {
    k->pass = pass;
    k->sign = sign;
    int nt = orc_threads();
    if (nt > k->n) nt = k->n;
    orc_par_run(fft_task_run, k, nt);
    return k->err ? -1 : 0;
}

int orc_fft_r2c_3d(int n, const double *q, double *fqd) {
    (void)get_twiddles(n);   /* fill the table cache before any thread reads it */
    fft_task k = {n, -1, 0, q, NULL, (cpx *)fqd, 0};
    /* x: real -> half spectrum, two real lines per complex transform
       (A + iB; X_A = (Z_k + conj Z_{n-k})/2, X_B = (Z_k - conj Z_{n-k})/2i);
       then y and z: columns of the half spectrum */
    if (fft_pass(&k, 0, -1) || fft_pass(&k, 1, -1) || fft_pass(&k, 2, -1)) return -1;
    return 0;
}

int orc_fft_c2r_3d(int n, const double *fqd, double *q) {
    int nh = n / 2 + 1;
    size_t nc = (size_t)nh * n * n;
    cpx *fq = malloc(sizeof(cpx) * nc);
    if (!fq) return -1;
    memcpy(fq, fqd, sizeof(cpx) * nc);
    (void)get_twiddles(n);
    fft_task k = {n, +1, 0, NULL, q, fq, 0};
    /* z, then y: complex backward; then x: two Hermitian lines per complex
       transform, Z = X_A + i X_B over the completed spectra; the imaginary
       parts of the k = 0 and k = n/2 terms are dropped, as a Hermitian-input
       c2r does */
    int st = (fft_pass(&k, 2, +1) || fft_pass(&k, 1, +1) || fft_pass(&k, 0, +1)) ? -1 : 0;
    free(fq);
    return st;
}
