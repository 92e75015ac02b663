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

int orc_fft_r2c_3d(int n, const double *q, double *fqd) {
    int nh = n / 2 + 1;
    cpx *fq = (cpx *)fqd;
    cpx *line = malloc(sizeof(cpx) * n), *work = malloc(sizeof(cpx) * 2 * n);
    cpx *buf = malloc(sizeof(cpx) * COLBLK * (size_t)n);
    if (!line || !work || !buf) { free(line); free(work); free(buf); return -1; }
    /* x: real -> half spectrum, two real lines per complex transform
       (A + iB; X_A = (Z_k + conj Z_{n-k})/2, X_B = (Z_k - conj Z_{n-k})/2i) */
    size_t nl = (size_t)n * n;
    for (size_t l = 0; l < nl; l += 2) {
        const double *a = q + l * n, *b = (l + 1 < nl) ? q + (l + 1) * n : NULL;
        for (int x = 0; x < n; ++x) { line[x].re = a[x]; line[x].im = b ? b[x] : 0.0; }
        dft_line(n, line, -1, work);
        cpx *fa = fq + l * nh, *fb = fq + (l + 1) * nh;
        for (int k = 0; k < nh; ++k) {
            cpx z = line[k], zc = line[(n - k) % n];
            fa[k].re = 0.5 * (z.re + zc.re);
            fa[k].im = 0.5 * (z.im - zc.im);
            if (b) {
                fb[k].re = 0.5 * (z.im + zc.im);
                fb[k].im = -0.5 * (z.re - zc.re);
            }
        }
    }
    /* y and z: columns of the half spectrum */
    for (int z = 0; z < n; ++z) fft_columns(n, fq + (size_t)z * n * nh, nh, nh, -1, buf, work);
    for (int y = 0; y < n; ++y) fft_columns(n, fq + (size_t)y * nh, (size_t)n * nh, nh, -1, buf, work);
    free(line); free(work); free(buf);
    return 0;
}

int orc_fft_c2r_3d(int n, const double *fqd, double *q) {
    int nh = n / 2 + 1;
    size_t nc = (size_t)nh * n * n;
    cpx *fq = malloc(sizeof(cpx) * nc);
    cpx *line = malloc(sizeof(cpx) * n), *work = malloc(sizeof(cpx) * 2 * n);
    cpx *buf = malloc(sizeof(cpx) * COLBLK * (size_t)n);
    if (!fq || !line || !work || !buf) { free(fq); free(line); free(work); free(buf); return -1; }
    memcpy(fq, fqd, sizeof(cpx) * nc);
    /* z, then y: complex backward */
    for (int y = 0; y < n; ++y) fft_columns(n, fq + (size_t)y * nh, (size_t)n * nh, nh, +1, buf, work);
    for (int z = 0; z < n; ++z) fft_columns(n, fq + (size_t)z * n * nh, nh, nh, +1, buf, work);
    /* x: two Hermitian lines per complex transform, Z = X_A + i X_B over the
       completed spectra; the imaginary parts of the k = 0 and k = n/2 terms
       are dropped, as a Hermitian-input c2r does */
    size_t nl = (size_t)n * n;
    for (size_t l = 0; l < nl; l += 2) {
        const cpx *ha = fq + l * nh, *hb = (l + 1 < nl) ? fq + (l + 1) * nh : NULL;
        for (int k = 0; k < n; ++k) {
            cpx xa, xb = {0.0, 0.0};
            int kk = k < nh ? k : n - k;
            double sg = k < nh ? 1.0 : -1.0;
            xa.re = ha[kk].re; xa.im = sg * ha[kk].im;
            if (hb) { xb.re = hb[kk].re; xb.im = sg * hb[kk].im; }
            if (kk == 0 || 2 * kk == n) { xa.im = 0.0; xb.im = 0.0; }
            line[k].re = xa.re - xb.im;
            line[k].im = xa.im + xb.re;
        }
        dft_line(n, line, +1, work);
        double *qa = q + l * n, *qb = hb ? q + (l + 1) * n : NULL;
        for (int x = 0; x < n; ++x) {
            qa[x] = line[x].re;
            if (qb) qb[x] = line[x].im;
        }
    }
    free(fq); free(line); free(work); free(buf);
    return 0;
}
