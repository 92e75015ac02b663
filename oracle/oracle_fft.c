/*
 * oracle_fft.c — TEST INFRASTRUCTURE ONLY: the oracle's own FFT.
 *
 * The reference calls FFTW 3.3.4 (not vendored; configure.sh:131-139 fetches
 * fftw-3.3.4.tar.gz) through fftw_plan_dft_r2c_3d / fftw_plan_dft_c2r_3d with
 * the dimensions reversed (energy.F90:6931-6932), i.e. a real mesh Q(x,y,z)
 * with x fastest is transformed to FQ(0:n/2, y, z).  FFTW's published
 * conventions: forward = sum_j x_j exp(-2 pi i jk/n), backward = exp(+...),
 * both unnormalised; c2r assumes Hermitian input.  This file restates those
 * conventions with a plain recursive mixed-radix (2, 3, 5, generic) DFT in
 * double precision; it is checked against numpy.fft in tests.
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

static void dft_line(int n, cpx *line, int sign, cpx *work) {
    cpx *in = work, *tmp = work + n;
    memcpy(in, line, sizeof(cpx) * n);
    dft_rec(n, in, 1, line, sign, tmp, get_twiddles(n), n);
}

int orc_fft_r2c_3d(int n, const double *q, double *fqd) {
    int nh = n / 2 + 1;
    cpx *fq = (cpx *)fqd;
    cpx *line = malloc(sizeof(cpx) * n), *work = malloc(sizeof(cpx) * 2 * n);
    if (!line || !work) { free(line); free(work); return -1; }
    /* x: real -> half spectrum */
    for (int z = 0; z < n; ++z)
        for (int y = 0; y < n; ++y) {
            for (int x = 0; x < n; ++x) { line[x].re = q[((size_t)z * n + y) * n + x]; line[x].im = 0; }
            dft_line(n, line, -1, work);
            for (int kx = 0; kx < nh; ++kx) fq[((size_t)z * n + y) * nh + kx] = line[kx];
        }
    /* y */
    for (int z = 0; z < n; ++z)
        for (int kx = 0; kx < nh; ++kx) {
            for (int y = 0; y < n; ++y) line[y] = fq[((size_t)z * n + y) * nh + kx];
            dft_line(n, line, -1, work);
            for (int y = 0; y < n; ++y) fq[((size_t)z * n + y) * nh + kx] = line[y];
        }
    /* z */
    for (int y = 0; y < n; ++y)
        for (int kx = 0; kx < nh; ++kx) {
            for (int z = 0; z < n; ++z) line[z] = fq[((size_t)z * n + y) * nh + kx];
            dft_line(n, line, -1, work);
            for (int z = 0; z < n; ++z) fq[((size_t)z * n + y) * nh + kx] = line[z];
        }
    free(line); free(work);
    return 0;
}

int orc_fft_c2r_3d(int n, const double *fqd, double *q) {
    int nh = n / 2 + 1;
    size_t nc = (size_t)nh * n * n;
    cpx *fq = malloc(sizeof(cpx) * nc);
    cpx *line = malloc(sizeof(cpx) * n), *work = malloc(sizeof(cpx) * 2 * n);
    if (!fq || !line || !work) { free(fq); free(line); free(work); return -1; }
    memcpy(fq, fqd, sizeof(cpx) * nc);
    /* z, then y: complex backward */
    for (int y = 0; y < n; ++y)
        for (int kx = 0; kx < nh; ++kx) {
            for (int z = 0; z < n; ++z) line[z] = fq[((size_t)z * n + y) * nh + kx];
            dft_line(n, line, +1, work);
            for (int z = 0; z < n; ++z) fq[((size_t)z * n + y) * nh + kx] = line[z];
        }
    for (int z = 0; z < n; ++z)
        for (int kx = 0; kx < nh; ++kx) {
            for (int y = 0; y < n; ++y) line[y] = fq[((size_t)z * n + y) * nh + kx];
            dft_line(n, line, +1, work);
            for (int y = 0; y < n; ++y) fq[((size_t)z * n + y) * nh + kx] = line[y];
        }
    /* x: Hermitian completion, backward, real part (the imaginary parts of
       the k=0 and k=n/2 terms drop out, as for a Hermitian-input c2r) */
    for (int z = 0; z < n; ++z)
        for (int y = 0; y < n; ++y) {
            const cpx *h = fq + ((size_t)z * n + y) * nh;
            for (int k = 0; k < nh; ++k) line[k] = h[k];
            for (int k = nh; k < n; ++k) { line[k].re = h[n - k].re; line[k].im = -h[n - k].im; }
            dft_line(n, line, +1, work);
            for (int x = 0; x < n; ++x) q[((size_t)z * n + y) * n + x] = line[x].re;
        }
    free(fq); free(line); free(work);
    return 0;
}
