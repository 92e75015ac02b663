// spme.cu — smooth particle-mesh Ewald on the device (rows A10-A12).
//
// Reference: UEwaldRecSPM (energy.F90:1207-1297), SPMFFTRec (energy.F90:6525-
// 6587), CardinalBSpline (mollib.F90:1629-1685), EwaldSetup's SPM branch
// (energy.F90:6855-7018).  The reference calls FFTW's r2c/c2r 3D plans; this
// file has its own FFT.
//
// Pipeline per UTotal (mesh Q[z][y][x], half spectrum F[z][y][kx], kx<=n/2):
//   splines  B-spline values and derivatives per particle; the particle's
//            brick (B^3 mesh points holding the upper corner of its stamp)
//            and its rank in that brick (atomic count)
//   bricks   prefix of the brick counts and of the work items (at most 32
//            particles of one brick each); particles scattered in brick order
//   spread   one warp per work item adds its particles' stamps into a
//            fixed-point tile (the brick plus an order-1 halo) in shared
//            memory, then adds the tile into the 64-bit fixed-point mesh with
//            integer atomics (exact, so independent of the order)
//   x pass   r2c along x from the fixed-point mesh; two real lines are
//            packed into one complex line; the mesh is then cleared
//   y pass   complex FFT along y, tiles of TX consecutive kx columns
//   z pass   complex FFT along z, then the influence function (energy, virial,
//            multiply by meshfac) and the inverse z FFT while the column is
//            still in shared memory
//   y pass   inverse; x pass c2r inverse (FFTW's unnormalised convention)
//   gather   a group of lanes per particle (lane = stamp plane), separable
//            B-spline sums over the potential mesh
// The FFTs are radix-4 Stockham (one radix-2 stage when log2 n is odd) in
// shared memory; twiddles come from a host table computed in long double.
#include <algorithm>
#include <cmath>

#include <type_traits>

#include "mg_internal.cuh"

namespace {

template <typename T> using V2 = typename mg_cplx<T>::type;

template <typename V> __device__ __forceinline__ V cmul(V a, V b) {
    V r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
template <typename V> __device__ __forceinline__ V cadd(V a, V b) { V r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename V> __device__ __forceinline__ V csub(V a, V b) { V r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }

// Unsigned division by a divisor fixed for a whole launch (the half-spectrum
// width n/2+1, the column-tile width) by one multiply-high and two shifts:
// Granlund and Montgomery, "Division by invariant integers using
// multiplication" (1994), the round-up method; exact for every 32-bit n.
struct FastDiv {
    unsigned d, m, s1, s2;
};

static FastDiv make_fastdiv(unsigned d) {
    unsigned l = 0;
    while ((1ull << l) < d) ++l;
    FastDiv f;
    f.d = d;
    f.m = (unsigned)(((((unsigned long long)1 << l) - d) << 32) / d + 1);
    f.s1 = l < 1 ? l : 1;
    f.s2 = l > 0 ? l - 1 : 0;
    return f;
}

__device__ __forceinline__ unsigned fdiv(unsigned n, const FastDiv &f) {
    unsigned t = __umulhi(n, f.m);
    return (t + ((n - t) >> f.s1)) >> f.s2;
}

// The line length of the FFT passes: a power of two (logn >= 0) or a
// product 2^a 3^b 5^c (logn < 0), transformed by Stockham passes of the
// radices r[0..nf) in that order; fn divides by n.
struct FftPlan {
    int logn, nf;
    int r[12];
    FastDiv fn;
};

static FftPlan make_plan(int n) {
    FftPlan p = {};
    p.fn = make_fastdiv((unsigned)n);
    if ((n & (n - 1)) == 0) {
        int l = 0;
        while ((1 << l) < n) ++l;
        p.logn = l;
        return p;
    }
    p.logn = -1;
    int m = n;
    while (m % 4 == 0 && p.nf < 12) { p.r[p.nf++] = 4; m /= 4; }
    while (m % 2 == 0 && p.nf < 12) { p.r[p.nf++] = 2; m /= 2; }
    while (m % 3 == 0 && p.nf < 12) { p.r[p.nf++] = 3; m /= 3; }
    while (m % 5 == 0 && p.nf < 12) { p.r[p.nf++] = 5; m /= 5; }
    if (m != 1) p.nf = 0;   // not 2^a 3^b 5^c: rejected by the caller
    return p;
}

// radix-R butterflies (R = 2, 3, 4, 5) on v[0..R), in place; sign -1
// forward (w = exp(-2 pi i / R)), +1 backward
template <typename T> __device__ __forceinline__ V2<T> mul_i(V2<T> a, T s) {   // s * i * a
    V2<T> r;
    r.x = -s * a.y;
    r.y = s * a.x;
    return r;
}

template <typename T> __device__ __forceinline__ void dft_small(V2<T> *v, int R, int sign) {
    typedef V2<T> V;
    const T sg = (T)sign;
    if (R == 2) {
        V a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else if (R == 4) {
        V a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]), a2 = cadd(v[1], v[3]), a3 = csub(v[1], v[3]);
        v[0] = cadd(a0, a2);
        v[2] = csub(a0, a2);
        V t = mul_i<T>(a3, sg);   // sign * i * (v1 - v3)
        v[1] = cadd(a1, t);
        v[3] = csub(a1, t);
    } else if (R == 3) {
        const T h = (T)0.86602540378443864676;   // sqrt(3)/2
        V t1 = cadd(v[1], v[2]), d = csub(v[1], v[2]);
        V t2;
        t2.x = v[0].x - (T)0.5 * t1.x;
        t2.y = v[0].y - (T)0.5 * t1.y;
        V t3 = mul_i<T>(d, sg * h);
        v[0] = cadd(v[0], t1);
        v[1] = cadd(t2, t3);
        v[2] = csub(t2, t3);
    } else {   // R == 5
        const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;   // cos(2 pi/5), cos(4 pi/5)
        const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;    // sin(2 pi/5), sin(4 pi/5)
        V a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]), a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
        V x0 = v[0], r1, r2, i1, i2;
        r1.x = x0.x + c1 * a1.x + c2 * a2.x;
        r1.y = x0.y + c1 * a1.y + c2 * a2.y;
        r2.x = x0.x + c2 * a1.x + c1 * a2.x;
        r2.y = x0.y + c2 * a1.y + c1 * a2.y;
        i1.x = s1 * b1.x + s2 * b2.x;
        i1.y = s1 * b1.y + s2 * b2.y;
        i2.x = s2 * b1.x - s1 * b2.x;
        i2.y = s2 * b1.y - s1 * b2.y;
        V j1 = mul_i<T>(i1, sg), j2 = mul_i<T>(i2, sg);
        v[0] = cadd(x0, cadd(a1, a2));
        v[1] = cadd(r1, j1);
        v[4] = csub(r1, j1);
        v[2] = cadd(r2, j2);
        v[3] = csub(r2, j2);
    }
}

// Stockham passes for n = 2^a 3^b 5^c (the radices of the plan): pass of
// radix R at span Ns reads x[j + r n/R], twiddles by w^(r k n/(R Ns)) with
// k = j mod Ns, and writes y[(j - k) R + k + r Ns]
template <typename T, bool LINE_MAJOR>
__device__ V2<T> *smem_fft_gen(V2<T> *A, V2<T> *B, int n, const FftPlan &pl, int nl, int cs, int ts, int sign,
                               const V2<T> *__restrict__ tw, const FastDiv &fnl) {
    typedef V2<T> V;
    V *in = A, *out = B;
    int tid = threadIdx.x, nthr = blockDim.x;
    int Ns = 1;
    for (int f = 0; f < pl.nf; ++f) {
        int R = pl.r[f], m = n / R, stride = n / (R * Ns);
        for (int b = tid; b < nl * m; b += nthr) {
            int c, j;
            if (LINE_MAJOR) { c = b / m; j = b - c * m; }
            else { j = (int)fdiv((unsigned)b, fnl); c = b - j * nl; }
            int k = j % Ns;
            const V *src = in + c * cs;
            V v[5];
            for (int r = 0; r < R; ++r) {
                v[r] = src[(j + r * m) * ts];
                if (k && r) {
                    V t = tw[r * k * stride];
                    if (sign > 0) t.y = -t.y;
                    v[r] = cmul(v[r], t);
                }
            }
            dft_small<T>(v, R, sign);
            int d = (j - k) * R + k;
            V *dst = out + c * cs;
            for (int r = 0; r < R; ++r) dst[(d + r * Ns) * ts] = v[r];
        }
        __syncthreads();
        V *t = in; in = out; out = t;
        Ns *= R;
    }
    return in;
}

// Stockham FFT of nl lines of length n = 2^logn held in shared memory.  Element
// (line c, index t) is at buf[c*cs + t*ts].  LINE_MAJOR (ts == 1): threads run
// along t; otherwise (cs == 1) threads run along c.  Returns the buffer that
// holds the result.  sign = -1 forward, +1 backward (unnormalised).  Other
// lengths (2^a 3^b 5^c) go to smem_fft_gen.
template <typename T, bool LINE_MAJOR>
__device__ V2<T> *smem_fft(V2<T> *A, V2<T> *B, int n, const FftPlan &pl, int nl, int cs, int ts, int sign,
                           const V2<T> *__restrict__ tw, const FastDiv &fnl) {
    typedef V2<T> V;
    if (pl.logn < 0) return smem_fft_gen<T, LINE_MAJOR>(A, B, n, pl, nl, cs, ts, sign, tw, fnl);
    const int logn = pl.logn;
    V *in = A, *out = B;
    int tid = threadIdx.x, nthr = blockDim.x;
    int Ns = 1, logNs = 0;
    // (line c, index j) of work item b: shifts along a line, the invariant
    // divider across lines
    if (logn & 1) {
        int nb = n >> 1;
        for (int b = tid; b < nl * nb; b += nthr) {
            int c, j;
            if (LINE_MAJOR) { c = b >> (logn - 1); j = b & (nb - 1); }
            else { j = (int)fdiv((unsigned)b, fnl); c = b - j * nl; }
            V v0 = in[c * cs + j * ts], v1 = in[c * cs + (j + nb) * ts];
            out[c * cs + (2 * j) * ts] = cadd(v0, v1);
            out[c * cs + (2 * j + 1) * ts] = csub(v0, v1);
        }
        __syncthreads();
        V *t = in; in = out; out = t;
        Ns = 2;
        logNs = 1;
    }
    int nq = n >> 2;
    while (Ns < n) {
        int stride = nq >> logNs;   // n / (4 Ns)
        for (int b = tid; b < nl * nq; b += nthr) {
            int c, j;
            if (LINE_MAJOR) { c = b >> (logn - 2); j = b & (nq - 1); }
            else { j = (int)fdiv((unsigned)b, fnl); c = b - j * nl; }
            int k = j & (Ns - 1);
            const V *src = in + c * cs;
            V v0 = src[j * ts], v1 = src[(j + nq) * ts], v2 = src[(j + 2 * nq) * ts],
              v3 = src[(j + 3 * nq) * ts];
            if (k) {
                V t1 = tw[k * stride], t2 = tw[2 * k * stride], t3 = tw[3 * k * stride];
                if (sign > 0) { t1.y = -t1.y; t2.y = -t2.y; t3.y = -t3.y; }
                v1 = cmul(v1, t1);
                v2 = cmul(v2, t2);
                v3 = cmul(v3, t3);
            }
            V a0 = cadd(v0, v2), a1 = csub(v0, v2), a2 = cadd(v1, v3), a3 = csub(v1, v3);
            V y0 = cadd(a0, a2), y2 = csub(a0, a2), y1, y3;
            if (sign < 0) {
                y1.x = a1.x + a3.y; y1.y = a1.y - a3.x;
                y3.x = a1.x - a3.y; y3.y = a1.y + a3.x;
            } else {
                y1.x = a1.x - a3.y; y1.y = a1.y + a3.x;
                y3.x = a1.x + a3.y; y3.y = a1.y - a3.x;
            }
            int d = (j - k) * 4 + k;
            V *dst = out + c * cs;
            dst[d * ts] = y0;
            dst[(d + Ns) * ts] = y1;
            dst[(d + 2 * Ns) * ts] = y2;
            dst[(d + 3 * Ns) * ts] = y3;
        }
        __syncthreads();
        V *t = in; in = out; out = t;
        Ns <<= 2;
        logNs += 2;
    }
    return in;
}

template <typename T>
__device__ __forceinline__ void load_tw(V2<T> *s_tw, const V2<T> *__restrict__ tw, int n) {
    for (int m = threadIdx.x; m < n; m += blockDim.x) s_tw[m] = tw[m];
}

// ---- x pass: r2c, two real lines per complex line ---------------------------
// 64-bit fixed point to the mesh type: double directly; float through two
// 32-bit halves so that the mixed form stays off the FP64 pipe
template <typename T> __device__ __forceinline__ T fx_to_real(long long x);
template <> __device__ __forceinline__ double fx_to_real<double>(long long x) { return (double)x; }
template <> __device__ __forceinline__ float fx_to_real<float>(long long x) {
    // x = hi 2^32 + lo with lo the signed low word, so that a small negative
    // x converts as exactly as a small positive one (an unsigned low word
    // would cancel 2^32 - |x| against -2^32 in single precision)
    int lo = (int)(unsigned)(x & 0xffffffffll);
    int hi = (int)((x - lo) >> 32);
    return (float)hi * 4294967296.0f + (float)lo;
}

template <typename T>
__global__ void k_fft_x_r2c(const long long *__restrict__ Qfx, T fx_inv, V2<T> *__restrict__ F, int n, FftPlan pl,
                            int lp, const V2<T> *__restrict__ tw, FastDiv fnh) {
    typedef V2<T> V;
    extern __shared__ unsigned char smem_raw[];
    V *s_tw = reinterpret_cast<V *>(smem_raw);
    V *A = s_tw + n, *B = A + lp * n;
    int nh = n / 2 + 1;
    load_tw<T>(s_tw, tw, n);
    size_t line0 = (size_t)blockIdx.x * 2 * lp;
    for (int e = threadIdx.x; e < lp * n; e += blockDim.x) {
        int c = (int)fdiv((unsigned)e, pl.fn), t = e - c * n;
        // the spread's fixed-point mesh (cleared after this pass)
        long long q0 = Qfx[(line0 + 2 * c) * n + t], q1 = Qfx[(line0 + 2 * c + 1) * n + t];
        V v;
        v.x = fx_to_real<T>(q0) * fx_inv;
        v.y = fx_to_real<T>(q1) * fx_inv;
        A[c * n + t] = v;
    }
    __syncthreads();
    V *Z = smem_fft<T, true>(A, B, n, pl, lp, n, 1, -1, s_tw, fnh);
    for (int e = threadIdx.x; e < lp * nh; e += blockDim.x) {
        int c = (int)fdiv((unsigned)e, fnh), k = e - c * nh;
        V z = Z[c * n + k], zc = Z[c * n + (k ? n - k : 0)];
        V a, b;
        // X_A = (Z_k + conj Z_{n-k})/2,  X_B = (Z_k - conj Z_{n-k})/(2i)
        a.x = (T)0.5 * (z.x + zc.x);
        a.y = (T)0.5 * (z.y - zc.y);
        b.x = (T)0.5 * (z.y + zc.y);
        b.y = (T)-0.5 * (z.x - zc.x);
        F[(line0 + 2 * c) * nh + k] = a;
        F[(line0 + 2 * c + 1) * nh + k] = b;
    }
}

// ---- x pass: c2r (Hermitian input; imaginary parts of k=0, n/2 dropped) ----
template <typename T>
__global__ void k_fft_x_c2r(const V2<T> *__restrict__ F, T *__restrict__ Q, int n, FftPlan pl,
                            int lp, const V2<T> *__restrict__ tw) {
    typedef V2<T> V;
    extern __shared__ unsigned char smem_raw[];
    V *s_tw = reinterpret_cast<V *>(smem_raw);
    V *A = s_tw + n, *B = A + lp * n;
    int nh = n / 2 + 1;
    load_tw<T>(s_tw, tw, n);
    size_t line0 = (size_t)blockIdx.x * 2 * lp;
    for (int e = threadIdx.x; e < lp * n; e += blockDim.x) {
        int c = (int)fdiv((unsigned)e, pl.fn), k = e - c * n;
        int kk = (k < nh) ? k : n - k;
        V a = F[(line0 + 2 * c) * nh + kk], b = F[(line0 + 2 * c + 1) * nh + kk];
        if (kk == 0 || 2 * kk == n) { a.y = (T)0; b.y = (T)0; }
        if (k >= nh) { a.y = -a.y; b.y = -b.y; }
        V z;
        z.x = a.x - b.y;
        z.y = a.y + b.x;
        A[c * n + k] = z;
    }
    __syncthreads();
    V *Z = smem_fft<T, true>(A, B, n, pl, lp, n, 1, +1, s_tw, FastDiv{});
    for (int e = threadIdx.x; e < lp * n; e += blockDim.x) {
        int c = (int)fdiv((unsigned)e, pl.fn), t = e - c * n;
        V z = Z[c * n + t];
        Q[(line0 + 2 * c) * n + t] = z.x;
        Q[(line0 + 2 * c + 1) * n + t] = z.y;
    }
}

struct ConvArgs {
    const void *mf, *ew, *vw;   // octant tables, T
    double *part;               // per-block (energy, virial)
};

// ---- column passes (y or z); with CONV the influence function and the
//      inverse transform follow the forward one -------------------------------
template <typename T, bool CONV>
__global__ void k_fft_col(V2<T> *__restrict__ F, int n, FftPlan pl, int nh, int tx, size_t tstride,
                          size_t ostride, int sign, const V2<T> *__restrict__ tw, ConvArgs cv, FastDiv ftx) {
    typedef V2<T> V;
    extern __shared__ unsigned char smem_raw[];
    __shared__ double red[2 * 32];
    V *s_tw = reinterpret_cast<V *>(smem_raw);
    V *A = s_tw + n, *B = A + tx * n;
    load_tw<T>(s_tw, tw, n);
    int kx0 = blockIdx.x * tx;
    size_t base = (size_t)blockIdx.y * ostride;
    for (int e = threadIdx.x; e < tx * n; e += blockDim.x) {
        int t = (int)fdiv((unsigned)e, ftx), c = e - t * tx;
        int kx = kx0 + c;
        V v;
        v.x = (T)0;
        v.y = (T)0;
        if (kx < nh) v = F[base + t * tstride + kx];
        A[t * tx + c] = v;
    }
    __syncthreads();
    V *R = smem_fft<T, false>(A, B, n, pl, tx, 1, tx, sign, s_tw, ftx);
    if (CONV) {
        const T *mf = (const T *)cv.mf, *ew = (const T *)cv.ew, *vw = (const T *)cv.vw;
        int ky = blockIdx.y;
        int fy = min(ky, n - ky);
        double e_t = 0, v_t = 0;   // per-element products in the mesh type, sums in FP64
        for (int e = threadIdx.x; e < tx * n; e += blockDim.x) {
            int t = (int)fdiv((unsigned)e, ftx), c = e - t * tx;
            int kx = kx0 + c;
            if (kx >= nh) continue;
            int fz = min(t, n - t);
            size_t id = ((size_t)fz * nh + fy) * nh + kx;
            V f = R[t * tx + c];
            T p2 = f.x * f.x + f.y * f.y;
            e_t += (double)(p2 * ew[id]);
            v_t -= (double)(p2 * vw[id]);
            T m = mf[id];
            f.x *= m;
            f.y *= m;
            R[t * tx + c] = f;
        }
        int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
        for (int o = 16; o > 0; o >>= 1) {
            e_t += __shfl_down_sync(0xffffffffu, e_t, o);
            v_t += __shfl_down_sync(0xffffffffu, v_t, o);
        }
        if (lane == 0) { red[w] = e_t; red[32 + w] = v_t; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double se = 0.0, sv = 0.0;
            for (int k = 0; k < nw; ++k) { se += red[k]; sv += red[32 + k]; }
            size_t blk = (size_t)blockIdx.y * gridDim.x + blockIdx.x;
            cv.part[2 * blk] = se;
            cv.part[2 * blk + 1] = sv;
        }
        V *other = (R == A) ? B : A;
        R = smem_fft<T, false>(R, other, n, pl, tx, 1, tx, +1, s_tw, ftx);
    }
    for (int e = threadIdx.x; e < tx * n; e += blockDim.x) {
        int t = (int)fdiv((unsigned)e, ftx), c = e - t * tx;
        int kx = kx0 + c;
        if (kx < nh) F[base + t * tstride + kx] = R[t * tx + c];
    }
}

// ---- B-spline (CardinalBSpline, mollib.F90:1629-1685) -----------------------
// values v[i] = M(x + i) ... in the reference's order (v[0] = x for order 2)
// and first derivatives dv, for the fractional mesh coordinate x
template <typename T, int ORDER>
__device__ __forceinline__ void bspline_o(T x, T *v, T *dv) {
    T last[ORDER];
    v[0] = x;
    v[1] = (T)1 - x;
#pragma unroll
    for (int i = 2; i < ORDER; ++i) v[i] = (T)0;
#pragma unroll
    for (int i = 0; i < ORDER; ++i) last[i] = (T)0;
#pragma unroll
    for (int nn = 3; nn <= ORDER; ++nn) {
#pragma unroll
        for (int i = 0; i < nn - 1; ++i) last[i] = v[i];
        const T inv = (T)1 / (T)(nn - 1);
        v[0] = x * last[0] * inv;
#pragma unroll
        for (int i = 1; i <= nn - 2; ++i) {
            T aa = (T)i + x;
            v[i] = (aa * last[i] + ((T)nn - aa) * last[i - 1]) * inv;
        }
        v[nn - 1] = ((T)1 - x) * last[nn - 2] * inv;
    }
    dv[0] = last[0];
#pragma unroll
    for (int i = 1; i <= ORDER - 2; ++i) dv[i] = last[i] - last[i - 1];
    dv[ORDER - 1] = -last[ORDER - 2];
}

struct SplineArgs {
    const double *ro, *az;
    // records in the cell order of the last list build: record i is the
    // particle perm[i] (nullptr: record p is particle p)
    const int *perm;
    int np, order, n, n_log;
    double dkdr[3];
    // brick sort, first pass: brick of each particle and its rank among the
    // brick's particles (log2 of the brick edge and of the bricks per edge)
    int lB, lnb;
    int plane;             // sort by the z plane of the stamp corner instead of by brick
    int nosort;            // records only (meshes that are not powers of two: no bricks)
    int *count, *rank, *brick;
    int assign;            // gather: the first writer of the force accumulator
    // gather, forked UTotal without a surface term: forceo = (mesh force +
    // the short-range accumulator) * fac, as the epilogue would write it
    int final_;
    const long long *ffx2;
    const double *force2;
    double *forceo;
    double fac;
};

// The spline record of a particle: a head of two values (the stamp's
// upper corner, 10 bits per axis, stored in the bits of the first value;
// the charge), then order values each of the B-spline values along z, x
// and y, and of their derivatives along x, y and z, padded to a multiple of
// four values so that records start on 16-byte boundaries.  The spreads
// read the head and the values (the first SB values) as one block, the
// gather the values and derivatives.
constexpr int kRecHead = 2;
__host__ __device__ constexpr int spl_rec(int order) { return (kRecHead + 6 * order + 3) & ~3; }
template <int ORDER> struct RecIx {
    static constexpr int VZ = kRecHead, VX = kRecHead + ORDER, VY = kRecHead + 2 * ORDER,
                         DX = kRecHead + 3 * ORDER, DY = kRecHead + 4 * ORDER, DZ = kRecHead + 5 * ORDER,
                         SB = kRecHead + 3 * ORDER;
};

template <typename T> __device__ __forceinline__ T rec_put_corner(int c);
template <> __device__ __forceinline__ float rec_put_corner<float>(int c) { return __int_as_float(c); }
template <> __device__ __forceinline__ double rec_put_corner<double>(int c) {
    return __longlong_as_double((long long)c);
}
__device__ __forceinline__ int rec_corner(float v) { return __float_as_int(v); }
__device__ __forceinline__ int rec_corner(double v) { return (int)__double_as_longlong(v); }

template <typename T, int N> __device__ __forceinline__ void store_rec(T *__restrict__ dst, const T (&r)[N]) {
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int k = 0; k < N / 4; ++k)
            reinterpret_cast<float4 *>(dst)[k] = make_float4(r[4 * k], r[4 * k + 1], r[4 * k + 2], r[4 * k + 3]);
    } else {
#pragma unroll
        for (int k = 0; k < N / 2; ++k) reinterpret_cast<double2 *>(dst)[k] = make_double2(r[2 * k], r[2 * k + 1]);
    }
}

// the first N values of a record (16-byte aligned)
template <typename T, int N> __device__ __forceinline__ void load_rec(const T *__restrict__ src, T (&r)[N]) {
    constexpr int VW = 16 / sizeof(T), NV = N / VW;
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            float4 v = reinterpret_cast<const float4 *>(src)[k];
            r[4 * k] = v.x;
            r[4 * k + 1] = v.y;
            r[4 * k + 2] = v.z;
            r[4 * k + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double2 v = reinterpret_cast<const double2 *>(src)[k];
            r[2 * k] = v.x;
            r[2 * k + 1] = v.y;
        }
    }
#pragma unroll
    for (int k = NV * VW; k < N; ++k) r[k] = src[k];
}

// Spline data of every particle, once per call (the only FP64 of the mesh
// path: position -> mesh coordinate): the record of particle p at
// w[p * spl_rec(ORDER)], its corner the meshmax of the reference.
template <typename T, int ORDER>
__global__ void __launch_bounds__(256) k_spline_prepare(SplineArgs a, T *__restrict__ w) {
    mg_pdl_begin();
    int i = blockIdx.x * blockDim.x + threadIdx.x;   // the record
    bool valid = i < a.np;
    if (!valid) i = a.np - 1;   // a tail lane recomputes the last record and stores nothing
    const int p = a.perm ? a.perm[i] : i;
    int c[3];
    constexpr int S = spl_rec(ORDER);
    typedef RecIx<ORDER> RI;
    T r[S];
#pragma unroll
    for (int k = kRecHead + 6 * ORDER; k < S; ++k) r[k] = (T)0;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        double pos = a.dkdr[m] * a.ro[3 * p + m];
        double fl = floor(pos);
        int mm = (int)fl % a.n;
        c[m] = mm < 0 ? mm + a.n : mm;
        T v[ORDER], d[ORDER];
        bspline_o<T, ORDER>((T)(pos - fl), v, d);
        const int vo = m == 0 ? RI::VX : m == 1 ? RI::VY : RI::VZ;
        const int dof = m == 0 ? RI::DX : m == 1 ? RI::DY : RI::DZ;
#pragma unroll
        for (int k = 0; k < ORDER; ++k) {
            r[vo + k] = v[k];
            r[dof + k] = d[k];
        }
    }
    r[0] = rec_put_corner<T>(c[0] | (c[1] << 10) | (c[2] << 20));
    r[1] = (T)a.az[p];
    int lane = threadIdx.x & 31;
    if constexpr (sizeof(T) == 4 && S <= 48) {
        // the warp's 32 records are contiguous in memory: staged in shared
        // memory (at most 48 KB per block), then written as coalesced
        // 16-byte stores
        __shared__ float4 st[8][32 * S / 4];
        float4 *sw = st[threadIdx.x >> 5];
        store_rec<T, S>(reinterpret_cast<T *>(sw) + lane * S, r);
        __syncwarp();
        int i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31), nv = min(32, a.np - i0);   // i is clamped in the tail
        float4 *dst = reinterpret_cast<float4 *>(w + (size_t)i0 * S);
        for (int k = lane; k < nv * S / 4; k += 32) dst[k] = sw[k];
    } else if (valid) {
        store_rec<T, S>(w + (size_t)i * S, r);
    }
    if (a.plane) {
        // sort by the corner's z plane (at most 128 planes): the block's
        // counts in shared memory, one global atomic per plane and block
        __shared__ int hcnt[128], hbase[128];
        for (int k = threadIdx.x; k < a.n; k += blockDim.x) hcnt[k] = 0;
        __syncthreads();
        int lr = valid ? atomicAdd(&hcnt[c[2]], 1) : 0;
        __syncthreads();
        for (int k = threadIdx.x; k < a.n; k += blockDim.x)
            if (hcnt[k]) hbase[k] = atomicAdd(&a.count[k], hcnt[k]);
        __syncthreads();
        if (valid) {   // of the record
            a.brick[i] = c[2];
            a.rank[i] = hbase[c[2]] + lr;
        }
        return;
    }
    if (a.nosort) return;
    int id = ((((c[2] >> a.lB) << a.lnb) + (c[1] >> a.lB)) << a.lnb) + (c[0] >> a.lB);
    unsigned vm = __ballot_sync(0xffffffffu, valid);
    if (!valid) return;
    a.brick[i] = id;
    // rank among the brick's particles: one atomic per brick and warp (chain
    // beads, numbered along the chain, share bricks within a warp)
    unsigned peers = __match_any_sync(vm, id);
    int leader = __ffs(peers) - 1, base = 0;
    if (lane == leader) base = atomicAdd(&a.count[id], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    a.rank[i] = base + __popc(peers & ((1u << lane) - 1u));
}

// ---- brick-sorted spread -------------------------------------------------------
// The mesh is cut into bricks of B^3 points.  A particle belongs to the brick
// holding the upper corner of its stamp; the stamp then lies in that brick's
// tile (the brick extended by order-1 points towards lower indices).
struct BrickArgs {
    int n, B, nb;          // mesh edge, brick edge, bricks per edge (powers of 2)
    int ln, lB, lnb;       // their log2
    int tile;              // B + order - 1
    int nbricks;
    float fx_scale;        // mixed form: stamp weights to 32-bit integers (2^k)
    float fx_inv;
    double fx_scale64;     // FP64 form: stamp weights to 64-bit integers
    int M;                 // particles per spread work item
    int *count, *start, *perm, *rank, *brick;
    int *istart;           // first work item of each brick (nbricks + 1)
    int *item_brick;       // brick of each work item
};


// exclusive prefixes of the brick counts and of the work items per brick
// (ceil(count / M)), one block of 1024 threads; the item -> brick map is
// filled and the counts are cleared for the next call
__global__ void __launch_bounds__(1024) k_brick_prefix(BrickArgs b) {
    mg_pdl_begin();
    __shared__ int wsum[2][32];
    constexpr int KMAX = 8;   // counts held in registers (one memory round trip) up to 8192 bricks
    int nb = b.nbricks, per = (nb + 1023) / 1024;
    int lo = threadIdx.x * per, hi = min(nb, lo + per);
    int cnt[KMAX];
#pragma unroll
    for (int k = 0; k < KMAX; ++k) cnt[k] = (lo + k < hi) ? b.count[lo + k] : 0;
    int s = 0, si = 0;
#pragma unroll
    for (int k = 0; k < KMAX; ++k) {
        s += cnt[k];
        si += (cnt[k] + b.M - 1) / b.M;
    }
    for (int i = lo + KMAX; i < hi; ++i) {   // meshes above 8192 bricks
        int c = b.count[i];
        s += c;
        si += (c + b.M - 1) / b.M;
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int v = s, vi = si;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, v, o), yi = __shfl_up_sync(0xffffffffu, vi, o);
        if (lane >= o) { v += y; vi += yi; }
    }
    if (lane == 31) { wsum[0][w] = v; wsum[1][w] = vi; }
    __syncthreads();
    if (w < 2) {
        int x = wsum[w][lane];
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        wsum[w][lane] = x;
    }
    __syncthreads();
    int run = v - s + (w ? wsum[0][w - 1] : 0);
    int irun = vi - si + (w ? wsum[1][w - 1] : 0);
    for (int i = lo; i < hi; ++i) {
        int c = (i - lo < KMAX) ? cnt[i - lo] : b.count[i], ni = (c + b.M - 1) / b.M;
        b.start[i] = run;
        b.istart[i] = irun;
        for (int k = 0; k < ni; ++k) b.item_brick[irun + k] = i;
        run += c;
        irun += ni;
        b.count[i] = 0;
    }
    if (threadIdx.x == 1023) { b.start[nb] = run; b.istart[nb] = irun; }
}

__global__ void k_brick_scatter(int np, BrickArgs b) {
    mg_pdl_begin();
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < np) b.perm[b.start[b.brick[p]] + b.rank[p]] = p;
}

// The spread record of a particle in plane order: the first SB values of
// its spline record (head, z, x and y values), padded to a multiple of four
template <int ORDER> __host__ __device__ constexpr int spread_rec() { return (RecIx<ORDER>::SB + 3) & ~3; }

// plane sort, second pass: each spline record's spread part to its place
// in the plane order.  Every block scans the plane counts (at most 128)
// itself; block 0 also stores the plane starts for the spread, which
// clears the counts.
template <int ORDER>
__global__ void k_plane_scatter(int np, BrickArgs b, const float *__restrict__ w, float *__restrict__ ws) {
    mg_pdl_begin();
    typedef RecIx<ORDER> RI;
    constexpr int SR = spread_rec<ORDER>();
    __shared__ int s_start[129];
    const int nb = b.nbricks;   // planes
    int i = blockIdx.x * blockDim.x + threadIdx.x;   // the record
    // the record and its plane and rank first: they do not wait for the prefix
    float v[RI::SB];
    int pl = 0, rk = 0;
    if (i < np) {
        load_rec<float, RI::SB>(w + (size_t)i * spl_rec(ORDER), v);
        pl = b.brick[i];
        rk = b.rank[i];
    }
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        int v[4], tot = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            int idx = 4 * lane + k;
            v[k] = idx < nb ? b.count[idx] : 0;
            tot += v[k];
        }
        int x = tot;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        int run = x - tot;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            int idx = 4 * lane + k;
            if (idx < nb) s_start[idx] = run;
            run += v[k];
        }
        if (lane == 31) s_start[nb] = x;
    }
    __syncthreads();
    if (blockIdx.x == 0)
        for (int k = threadIdx.x; k <= nb; k += blockDim.x) b.start[k] = s_start[k];
    if (i >= np) return;
    int dst = s_start[pl] + rk;
    float r[SR];
#pragma unroll
    for (int k = 0; k < SR; ++k) r[k] = k < RI::SB ? v[k] : 0.f;
    store_rec<float, SR>(ws + (size_t)dst * SR, r);
}

constexpr int kSpreadWarps = 8;   // most work items (warps) per block
constexpr int kSpreadItem = 32;   // most particles per spread work item

// spread: one warp per work item (up to M particles of one brick, so that a
// brick crowded by a polymer coil does not hold up the grid) owns a tile of
// the brick plus its halo in shared memory and adds the particles one after
// another, its lanes covering the order^3 points of a stamp (all distinct),
// so plain read-modify-writes are race free.  ACC is fixed point: 32-bit in
// the mixed form (the scale keeps M stamps below 2^31), 64-bit in the FP64
// form (scale 2^48 or finer, far below FP64 rounding of the energies).  The
// tile is then added into the 64-bit fixed-point mesh with integer atomics:
// exact, so the mesh does not depend on how particles fall into items or on
// the order in which items run.
template <typename T, typename ACC, int ORDER, int B>
__global__ void __launch_bounds__(32 * kSpreadWarps) k_spread_warp(BrickArgs b, const T *__restrict__ w,
                                                                   long long *__restrict__ Qfx) {
    constexpr int t = B + ORDER - 1, t3 = t * t * t, O3 = ORDER * ORDER * ORDER;
    constexpr int NPASS = (O3 + 31) / 32;
    constexpr int REC = 3 * ORDER + 1;   // odd record length: lanes reading one record hit distinct banks
    // per warp: the tile, then a staging area of 32 particles (corner
    // offsets packed in one int; per particle the charge-weighted x weights,
    // then the y and z weights)
    struct Stage {
        int off[32];
        T w[32][REC];
    };
    extern __shared__ __align__(16) unsigned char smem_sw[];
    int wib = threadIdx.x >> 5, lane = threadIdx.x & 31, nwb = blockDim.x >> 5;
    ACC *tile = reinterpret_cast<ACC *>(smem_sw) + (size_t)wib * t3;
    Stage *stg = reinterpret_cast<Stage *>(smem_sw + (((size_t)nwb * t3 * sizeof(ACC) + 15) & ~(size_t)15)) + wib;
    int item = blockIdx.x * nwb + wib;
    if (item >= b.istart[b.nbricks]) return;
    int brick = b.item_brick[item];
    for (int k = lane; k < t3; k += 32) tile[k] = (ACC)0;
    int mnb = b.nb - 1;
    int bx = brick & mnb, by = (brick >> b.lnb) & mnb, bz = brick >> (2 * b.lnb);
    int ox = bx * B - (ORDER - 1), oy = by * B - (ORDER - 1), oz = bz * B - (ORDER - 1);
    int first = b.start[brick] + (item - b.istart[brick]) * b.M;
    int last = min(first + b.M, b.start[brick + 1]);
    // this lane's stamp points, one per pass: tile offset relative to the
    // particle's corner and the packed (ix, iy, iz) weight indices
    int rel[NPASS], wix[NPASS];
#pragma unroll
    for (int pass = 0; pass < NPASS; ++pass) {
        int k = min(lane + 32 * pass, O3 - 1);
        int ix = k % ORDER, iy = (k / ORDER) % ORDER, iz = k / (ORDER * ORDER);
        rel[pass] = -((iz * t + iy) * t + ix);
        wix[pass] = ix | ((ORDER + iy) << 8) | ((2 * ORDER + iz) << 16);
    }
    for (int q0 = first; q0 < last; q0 += 32) {
        int cnt = min(32, last - q0);
        __syncwarp();
        if (lane < cnt) {   // stage one particle per lane
            int p = b.perm[q0 + lane];
            const T *src = w + (size_t)p * spl_rec(ORDER);
            T r[RecIx<ORDER>::SB];
            load_rec<T, RecIx<ORDER>::SB>(src, r);
            int c = rec_corner(r[0]);
            int cx = (c & 1023) - ox, cy = ((c >> 10) & 1023) - oy, cz = (c >> 20) - oz;
            stg->off[lane] = cx | (cy << 8) | (cz << 16);
            T qp = r[1];
            T *rec = stg->w[lane];
#pragma unroll
            for (int i = 0; i < ORDER; ++i) {
                rec[i] = qp * r[RecIx<ORDER>::VX + i];
                rec[ORDER + i] = r[RecIx<ORDER>::VY + i];
                rec[2 * ORDER + i] = r[RecIx<ORDER>::VZ + i];
            }
        }
        __syncwarp();
        for (int e = 0; e < cnt; ++e) {
            int off = stg->off[e];
            int base = ((off >> 16) * t + ((off >> 8) & 255)) * t + (off & 255);
            const T *rec = stg->w[e];
            // the order^3 points of one stamp are distinct: every lane issues
            // all of its loads before any store
            ACC old[NPASS];
            T val[NPASS];
#pragma unroll
            for (int pass = 0; pass < NPASS; ++pass) {
                if (lane + 32 * pass < O3) {
                    int q = wix[pass];
                    val[pass] = rec[q & 255] * rec[(q >> 8) & 255] * rec[q >> 16];
                    old[pass] = tile[base + rel[pass]];
                }
            }
#pragma unroll
            for (int pass = 0; pass < NPASS; ++pass) {
                if (lane + 32 * pass < O3) {
                    if (sizeof(T) == 4)   // |sum of M stamps * fx_scale| < 2^31 by choice of scale
                        tile[base + rel[pass]] = old[pass] + __float2int_rn((float)val[pass] * b.fx_scale);
                    else
                        tile[base + rel[pass]] = old[pass] + __double2ll_rn((double)val[pass] * b.fx_scale64);
                }
            }
            __syncwarp();
        }
    }
    // add the tile into the mesh, row by row: 64-bit integer adds are exact,
    // so the result does not depend on the order in which items arrive
    constexpr int XL = t <= 16 ? 16 : 32, RPI = 32 / XL;
    int mn = b.n - 1, cx = lane & (XL - 1);
    if (cx < t) {
        unsigned long long *qx = reinterpret_cast<unsigned long long *>(Qfx) + ((ox + cx) & mn);
        const ACC *tz = tile + cx;
        for (int cz = 0; cz < t; ++cz, tz += t * t) {
            unsigned long long *qz = qx + ((size_t)((oz + cz) & mn) << (2 * b.ln));
            for (int cy = lane / XL; cy < t; cy += RPI) {
                long long v = (long long)tz[cy * t];
                if (v != 0) atomicAdd(qz + ((size_t)((oy + cy) & mn) << b.ln), (unsigned long long)v);
            }
        }
    }
}

// spread, mixed form: one warp per work item (up to 32 particles of one
// brick), one lane per particle.  The lane holds its particle's B-spline
// weights in registers (the x weights times charge and scale) and adds the
// order^3 stamp values into the warp's 32-bit fixed-point tile with
// shared-memory integer atomics (exact, so the tile does not depend on the
// order of the adds; the scale keeps 32 stamps below 2^31).  The tile is then
// added into the 64-bit fixed-point mesh with integer atomics, as in
// k_spread_warp.
template <int ORDER, int B>
__global__ void __launch_bounds__(32 * kSpreadWarps) k_spread_lane(BrickArgs b, const float *__restrict__ w,
                                                                   long long *__restrict__ Qfx) {
    mg_pdl_begin();
    constexpr int t = B + ORDER - 1, t3 = t * t * t;
    extern __shared__ __align__(16) int tile_l[];
    int wib = threadIdx.x >> 5, lane = threadIdx.x & 31, nwb = blockDim.x >> 5;
    int *tile = tile_l + (size_t)wib * t3;
    int item = blockIdx.x * nwb + wib;
    if (item >= b.istart[b.nbricks]) return;
    int brick = b.item_brick[item];
    for (int k = lane; k < t3; k += 32) tile[k] = 0;
    int mnb = b.nb - 1;
    int bx = brick & mnb, by = (brick >> b.lnb) & mnb, bz = brick >> (2 * b.lnb);
    int ox = bx * B - (ORDER - 1), oy = by * B - (ORDER - 1), oz = bz * B - (ORDER - 1);
    int first = b.start[brick] + (item - b.istart[brick]) * b.M;
    int last = min(first + b.M, b.start[brick + 1]);
    int q = first + lane;
    bool act = q < last;
    float wx[ORDER], wy[ORDER], wz[ORDER];
    int base = 0;
    if (act) {
        int p = b.perm[q];
        const float *src = w + (size_t)p * spl_rec(ORDER);
        float r[RecIx<ORDER>::SB];
        load_rec<float, RecIx<ORDER>::SB>(src, r);
        int c = rec_corner(r[0]);
        int cx = (c & 1023) - ox, cy = ((c >> 10) & 1023) - oy, cz = (c >> 20) - oz;
        base = (cz * t + cy) * t + cx;
        float qs = r[1] * b.fx_scale;
#pragma unroll
        for (int i = 0; i < ORDER; ++i) {
            wx[i] = qs * r[RecIx<ORDER>::VX + i];
            wy[i] = r[RecIx<ORDER>::VY + i];
            wz[i] = r[RecIx<ORDER>::VZ + i];
        }
    }
    __syncwarp();
    if (act) {
#pragma unroll
        for (int iz = 0; iz < ORDER; ++iz) {
#pragma unroll
            for (int iy = 0; iy < ORDER; ++iy) {
                float wyz = wy[iy] * wz[iz];
                int *row = tile + base - (iz * t + iy) * t;
#pragma unroll
                for (int ix = 0; ix < ORDER; ++ix) atomicAdd(row - ix, __float2int_rn(wx[ix] * wyz));
            }
        }
    }
    __syncwarp();
    constexpr int XL = t <= 16 ? 16 : 32, RPI = 32 / XL;
    int mn = b.n - 1, cx = lane & (XL - 1);
    if (cx < t) {
        unsigned long long *qx = reinterpret_cast<unsigned long long *>(Qfx) + ((ox + cx) & mn);
        const int *tz = tile + cx;
        for (int cz = 0; cz < t; ++cz, tz += t * t) {
            unsigned long long *qz = qx + ((size_t)((oz + cz) & mn) << (2 * b.ln));
            for (int cy = lane / XL; cy < t; cy += RPI) {
                long long v = (long long)tz[cy * t];
                if (v != 0) atomicAdd(qz + ((size_t)((oy + cy) & mn) << b.ln), (unsigned long long)v);
            }
        }
    }
}

template <int ORDER> void spread_lane_attr() {
    cudaFuncSetAttribute(k_spread_lane<ORDER, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_spread_lane<ORDER, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

// gather: a group of G lanes per particle (G = 8 for orders up to 8, else
// 16; particles in cell-sorted order for mesh locality).  Lane j < ORDER of a
// group owns the stamp column ix = j, so that the group reads each mesh row
// segment of its stamp as ORDER consecutive values: per plane iz it sums
// M_y*phi and dM_y*phi over the rows, then weights them by M_z and dM_z; the
// x weight of the lane's column and the group sum follow.  E = sum
// dM*M*M*phi (energy.F90:1255-1285); force -= q*E*dkdr*EpsiFourPi.
template <typename T, bool MIXED>
__device__ __forceinline__ void gather_store(const SplineArgs &a, int p, T qk, T kx, T ky, T kz, T e0, T e1, T e2,
                                             double *__restrict__ force, long long *__restrict__ ffx);

template <typename T, bool MIXED, int ORDER>
__global__ void __launch_bounds__(256, MIXED ? 4 : 2) k_gather_grp(SplineArgs a, const int *__restrict__ perm,
                                                    const T *__restrict__ w, const T *__restrict__ Q,
                                                    T kx, T ky, T kz, double *__restrict__ force,
                                                    long long *__restrict__ ffx) {
    mg_pdl_begin();
    constexpr int G = ORDER <= 8 ? 8 : 16;
    int g = (int)((blockIdx.x * blockDim.x + threadIdx.x) / G);
    int j = threadIdx.x & (G - 1);
    bool valid = g < a.np;
    bool act = valid && j < ORDER;
    int p = valid ? perm[g] : 0;
    int n = a.n, mn = n - 1;
    T e0 = 0, e1 = 0, e2 = 0;
    const T *rec = w + (size_t)(a.perm ? (valid ? g : 0) : p) * spl_rec(ORDER);
    typedef RecIx<ORDER> RI;
    if (act) {
        T vy[ORDER], dy[ORDER];
#pragma unroll
        for (int i = 0; i < ORDER; ++i) {
            vy[i] = rec[RI::VY + i];
            dy[i] = rec[RI::DY + i];
        }
        T vx = rec[RI::VX + j], dx = rec[RI::DX + j];
        int c = rec_corner(rec[0]);
        int c0 = c & 1023, c1 = (c >> 10) & 1023, c2 = c >> 20;
        const T *col = Q + ((c0 - j) & mn);
        T A = 0, B = 0, C = 0;
#pragma unroll
        for (int iz = 0; iz < ORDER; ++iz) {
            T vz = rec[RI::VZ + iz], dz = rec[RI::DZ + iz];
            const T *pl = col + ((size_t)((c2 - iz) & mn) << (2 * a.n_log));
            T r0 = 0, r1 = 0;
#pragma unroll
            for (int iy = 0; iy < ORDER; ++iy) {
                T q = pl[(size_t)((c1 - iy) & mn) * n];
                r0 += vy[iy] * q;
                r1 += dy[iy] * q;
            }
            A += vz * r0;
            B += vz * r1;
            C += dz * r0;
        }
        e0 = dx * A;
        e1 = vx * B;
        e2 = vx * C;
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        e0 += __shfl_xor_sync(0xffffffffu, e0, o, G);
        e1 += __shfl_xor_sync(0xffffffffu, e1, o, G);
        e2 += __shfl_xor_sync(0xffffffffu, e2, o, G);
    }
    if (j != 0 || !valid) return;
    gather_store<T, MIXED>(a, p, -rec[1], kx, ky, kz, e0, e1, e2, force, ffx);
}

// the mesh force of particle p (qk = -charge; kx, ky, kz = dkdr *
// EpsiFourPi) into the form's accumulator: added, assigned, or with the
// short-range accumulator straight into forceo (the epilogue's arithmetic)
template <typename T, bool MIXED>
__device__ __forceinline__ void gather_store(const SplineArgs &a, int p, T qk, T kx, T ky, T kz, T e0, T e1, T e2,
                                             double *__restrict__ force, long long *__restrict__ ffx) {
    if (MIXED) {
        long long f0 = mg_f2fx((float)(qk * kx * e0)), f1 = mg_f2fx((float)(qk * ky * e1)),
                  f2 = mg_f2fx((float)(qk * kz * e2));
        if (a.final_) {   // the epilogue's arithmetic (k_epilogue)
            double g0 = (double)(f0 + a.ffx2[3 * p + 0]) * MG_FX_INV;
            double g1 = (double)(f1 + a.ffx2[3 * p + 1]) * MG_FX_INV;
            double g2 = (double)(f2 + a.ffx2[3 * p + 2]) * MG_FX_INV;
            a.forceo[3 * p + 0] = g0 * a.fac;
            a.forceo[3 * p + 1] = g1 * a.fac;
            a.forceo[3 * p + 2] = g2 * a.fac;
        } else if (a.assign) {   // the short-range forces went to their own accumulator
            ffx[3 * p + 0] = f0;
            ffx[3 * p + 1] = f1;
            ffx[3 * p + 2] = f2;
        } else {
            ffx[3 * p + 0] += f0;
            ffx[3 * p + 1] += f1;
            ffx[3 * p + 2] += f2;
        }
    } else {
        double f0 = (double)qk * (double)e0 * (double)kx, f1 = (double)qk * (double)e1 * (double)ky,
               f2 = (double)qk * (double)e2 * (double)kz;
        if (a.final_) {   // the epilogue's arithmetic (k_epilogue)
            a.forceo[3 * p + 0] = __dadd_rn(f0, a.force2[3 * p + 0]) * a.fac;
            a.forceo[3 * p + 1] = __dadd_rn(f1, a.force2[3 * p + 1]) * a.fac;
            a.forceo[3 * p + 2] = __dadd_rn(f2, a.force2[3 * p + 2]) * a.fac;
        } else if (a.assign) {
            force[3 * p + 0] = f0;
            force[3 * p + 1] = f1;
            force[3 * p + 2] = f2;
        } else {
            force[3 * p + 0] += f0;
            force[3 * p + 1] += f1;
            force[3 * p + 2] += f2;
        }
    }
}

// ---- meshes 2^a 3^b 5^c that are not powers of two ------------------------------
// one thread per particle: its record's stamp into the fixed-point mesh
// (64-bit integer atomics at the form's scale); indices wrap by remainders
template <typename T, int ORDER>
__global__ void __launch_bounds__(128) k_spread_gen(int np, int n, const T *__restrict__ w, double scale,
                                                    unsigned long long *__restrict__ Qfx) {
    mg_pdl_begin();
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    typedef RecIx<ORDER> RI;
    const T *rec = w + (size_t)p * spl_rec(ORDER);
    int c = rec_corner(rec[0]);
    int c0 = c & 1023, c1 = (c >> 10) & 1023, c2 = c >> 20;
    T q = rec[1];
    for (int iz = 0; iz < ORDER; ++iz) {
        int nz = c2 - iz < 0 ? c2 - iz + n : c2 - iz;   // ORDER <= n: one wrap at most
        T wz = q * rec[RI::VZ + iz];
        for (int iy = 0; iy < ORDER; ++iy) {
            int ny = c1 - iy < 0 ? c1 - iy + n : c1 - iy;
            T wyz = wz * rec[RI::VY + iy];
            size_t row = ((size_t)nz * n + ny) * n;
            for (int ix = 0; ix < ORDER; ++ix) {
                int nx = c0 - ix < 0 ? c0 - ix + n : c0 - ix;
                atomicAdd(&Qfx[row + nx], (unsigned long long)__double2ll_rn((double)(wyz * rec[RI::VX + ix]) * scale));
            }
        }
    }
}

// one warp per particle, lanes over the (iy, iz) rows of its stamp, the
// three field sums combined by shuffles; the force as k_gather_grp stores it
template <typename T, bool MIXED, int ORDER>
__global__ void __launch_bounds__(128) k_gather_gen(SplineArgs a, const T *__restrict__ w, const T *__restrict__ Q,
                                                    T kx, T ky, T kz, double *__restrict__ force,
                                                    long long *__restrict__ ffx) {
    mg_pdl_begin();
    int p = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (p >= a.np) return;
    typedef RecIx<ORDER> RI;
    const int n = a.n;
    const T *rec = w + (size_t)p * spl_rec(ORDER);
    int c = rec_corner(rec[0]);
    int c0 = c & 1023, c1 = (c >> 10) & 1023, c2 = c >> 20;
    T e0 = 0, e1 = 0, e2 = 0;
    for (int t = lane; t < ORDER * ORDER; t += 32) {
        int iz = t / ORDER, iy = t - iz * ORDER;
        int nz = c2 - iz < 0 ? c2 - iz + n : c2 - iz, ny = c1 - iy < 0 ? c1 - iy + n : c1 - iy;
        T vz = rec[RI::VZ + iz], dz = rec[RI::DZ + iz], vy = rec[RI::VY + iy], dy = rec[RI::DY + iy];
        const T *row = Q + ((size_t)nz * n + ny) * n;
        T r0 = 0, r1 = 0;
        for (int ix = 0; ix < ORDER; ++ix) {
            int nx = c0 - ix < 0 ? c0 - ix + n : c0 - ix;
            T qv = row[nx];
            r0 += rec[RI::DX + ix] * qv;
            r1 += rec[RI::VX + ix] * qv;
        }
        e0 += vy * vz * r0;
        e1 += dy * vz * r1;
        e2 += vy * dz * r1;
    }
    for (int o = 16; o > 0; o >>= 1) {
        e0 += __shfl_xor_sync(0xffffffffu, e0, o);
        e1 += __shfl_xor_sync(0xffffffffu, e1, o);
        e2 += __shfl_xor_sync(0xffffffffu, e2, o);
    }
    if (lane == 0) gather_store<T, MIXED>(a, p, -rec[1], kx, ky, kz, e0, e1, e2, force, ffx);
}

// ---- conversions between the fixed-point, FP64 and mesh-type meshes (MC) ----
__global__ void k_fx_to_f64(const long long *__restrict__ fx, double *__restrict__ q, size_t n, double inv) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) q[i] = (double)fx[i] * inv;
}

__global__ void k_f64_to_fx(const double *__restrict__ q, long long *__restrict__ fx, size_t n, double scale) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) fx[i] = __double2ll_rn(q[i] * scale);
}

template <typename T>
__global__ void k_mesh_to_f64(const T *__restrict__ Q, double *__restrict__ out, size_t n, double mul) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (double)Q[i] * mul;
}

// launch one of the order-templated mesh kernels: 0 = splines, 1 = spread, 2 = gather
template <typename T, typename ACC, int ORDER>
void launch_mesh_kernel(mg_handle *h, int which, const SplineArgs &sa, const BrickArgs &bk) {
    int np = h->np;
    T *w = (T *)h->d_spl_w;
    if (which == 0) {
        mg_launch_pdl(k_spline_prepare<T, ORDER>, (np + 255) / 256, 256, 0, h->st, sa, w);
    } else if (which == 1 && h->gen_mesh) {
        mg_launch_pdl(k_spread_gen<T, ORDER>, (np + 127) / 128, 128, 0, h->st, np, h->nmesh, (const T *)w,
                      mg_spme_fx_scale(h), (unsigned long long *)h->d_Qfx);
    } else if (which == 2 && h->gen_mesh) {
        T kx = (T)(h->dkdr[0] * h->EpsiFourPi), ky = (T)(h->dkdr[1] * h->EpsiFourPi),
          kz = (T)(h->dkdr[2] * h->EpsiFourPi);
        mg_launch_pdl(k_gather_gen<T, sizeof(T) == 4, ORDER>, (unsigned)(((long)np * 32 + 127) / 128), 128, 0,
                      h->st, sa, (const T *)w, (const T *)h->d_Q, kx, ky, kz, h->d_force, h->d_ffx);
    } else if (which == 1 && sizeof(T) == 4) {   // mixed form
        int wpb = h->spread_wpb_lane;
        int grid = (h->max_items + wpb - 1) / wpb;
        const float *wf = (const float *)w;
        if (h->brick == 8)
            mg_launch_pdl(k_spread_lane<ORDER, 8>, grid, 32 * wpb, h->spread_smem_lane, h->st, bk, wf,
                          (long long *)h->d_Qfx);
        else
            mg_launch_pdl(k_spread_lane<ORDER, 16>, grid, 32 * wpb, h->spread_smem_lane, h->st, bk, wf,
                          (long long *)h->d_Qfx);
    } else if (which == 1) {
        int wpb = h->spread_wpb;
        int grid = (h->max_items + wpb - 1) / wpb;
        if (h->brick == 8)
            k_spread_warp<T, ACC, ORDER, 8><<<grid, 32 * wpb, h->spread_smem, h->st>>>(
                bk, w, (long long *)h->d_Qfx);
        else
            k_spread_warp<T, ACC, ORDER, 16><<<grid, 32 * wpb, h->spread_smem, h->st>>>(
                bk, w, (long long *)h->d_Qfx);
    } else {
        // force factors dkdr * EpsiFourPi per direction
        T kx = (T)(h->dkdr[0] * h->EpsiFourPi), ky = (T)(h->dkdr[1] * h->EpsiFourPi),
          kz = (T)(h->dkdr[2] * h->EpsiFourPi);
        constexpr int G = ORDER <= 8 ? 8 : 16;
        mg_launch_pdl(k_gather_grp<T, sizeof(T) == 4, ORDER>, (unsigned)(((long)np * G + 255) / 256), 256, 0,
                      h->st, sa, h->d_perm, w, (const T *)h->d_Q, kx, ky, kz,
                      h->d_force, h->d_ffx);
    }
}

template <typename T, typename ACC>
int mesh_kernel(mg_handle *h, int which, const SplineArgs &sa, const BrickArgs &bk) {
    switch (h->order) {
    case 4: launch_mesh_kernel<T, ACC, 4>(h, which, sa, bk); break;
    case 5: launch_mesh_kernel<T, ACC, 5>(h, which, sa, bk); break;
    case 6: launch_mesh_kernel<T, ACC, 6>(h, which, sa, bk); break;
    case 7: launch_mesh_kernel<T, ACC, 7>(h, which, sa, bk); break;
    case 8: launch_mesh_kernel<T, ACC, 8>(h, which, sa, bk); break;
    case 9: launch_mesh_kernel<T, ACC, 9>(h, which, sa, bk); break;
    case 10: launch_mesh_kernel<T, ACC, 10>(h, which, sa, bk); break;
    case 11: launch_mesh_kernel<T, ACC, 11>(h, which, sa, bk); break;
    case 12: launch_mesh_kernel<T, ACC, 12>(h, which, sa, bk); break;
    default: return mg_fail(h, MG_ERR_UNSUPPORTED, "SPME order %d (supported: 4..12)", h->order);
    }
    h->launches++;
    return MG_OK;
}

template <typename T, typename ACC, int ORDER> void spread_attr_o() {
    cudaFuncSetAttribute(k_spread_warp<T, ACC, ORDER, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    cudaFuncSetAttribute(k_spread_warp<T, ACC, ORDER, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
}

template <typename T, typename ACC> void spread_attrs() {
    spread_attr_o<T, ACC, 4>(); spread_attr_o<T, ACC, 5>(); spread_attr_o<T, ACC, 6>();
    spread_attr_o<T, ACC, 7>(); spread_attr_o<T, ACC, 8>(); spread_attr_o<T, ACC, 9>();
    spread_attr_o<T, ACC, 10>(); spread_attr_o<T, ACC, 11>(); spread_attr_o<T, ACC, 12>();
}

int ilog2(int n) {
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}

// ---- plane passes (mixed form, n = 32 P for P = 1, 2, 4) --------------------
// Three kernels replace the five line passes when a whole mesh plane fits in
// shared memory: one CTA per z plane does the x r2c and the forward y FFT
// (and clears the fixed-point mesh it read); one CTA per ky slab does the
// forward z FFT, the influence function and the inverse z FFT; one CTA per
// z plane does the inverse y FFT and the x c2r.  Each line is transformed
// by one warp in registers:
//   lane l holds elements x[l + 32 j], j < P.  Forward: a P-point DFT in the
//   lane's registers, the twiddle w_n^(l k1), then a 32-point transform
//   across the lanes by decimation in frequency (shuffles), after which lane
//   l holds X[k1 + P bitrev5(l)].  The backward transform starts from that
//   layout (decimation in time across the lanes, conjugate twiddle, P-point
//   DFT) and ends with x[l + 32 j], unnormalised.
// Twiddles come from the table w_n^m = exp(-2 pi i m / n) in shared memory.

template <typename T> __device__ __forceinline__ V2<T> shfl_xor_c(V2<T> v, int m) {
    v.x = __shfl_xor_sync(0xffffffffu, v.x, m);
    v.y = __shfl_xor_sync(0xffffffffu, v.y, m);
    return v;
}

template <typename T> __device__ __forceinline__ V2<T> conj_c(V2<T> t) {
    t.y = -t.y;
    return t;
}

__device__ __forceinline__ int brev5(int l) { return (int)(__brev((unsigned)l) >> 27); }

// in-place P-point DFT in registers (natural order in and out): iterative
// radix-2 with the bit reversal as compile-time register renaming
// times -i (forward quarter turn) or +i (backward)
template <typename T, bool INV> __device__ __forceinline__ V2<T> quarter(V2<T> t) {
    V2<T> r;
    if (INV) { r.x = -t.y; r.y = t.x; }
    else { r.x = t.y; r.y = -t.x; }
    return r;
}

template <typename T, int P, bool INV>
__device__ __forceinline__ void reg_dft(V2<T> *v, const V2<T> *tw, int) {
    typedef V2<T> V;
    constexpr int n = 32 * P;
#pragma unroll
    for (int i = 0; i < P; ++i) {
        int r = 0;
#pragma unroll
        for (int b = 1, x = i; b < P; b <<= 1, x >>= 1) r = (r << 1) | (x & 1);
        if (r > i) { V t = v[i]; v[i] = v[r]; v[r] = t; }
    }
#pragma unroll
    for (int len = 2; len <= P; len <<= 1) {
        const int half = len >> 1;
#pragma unroll
        for (int i = 0; i < P; i += len) {
#pragma unroll
            for (int e = 0; e < half; ++e) {
                V u = v[i + e], t = v[i + e + half];
                if (e && 4 * e == len) {   // w_n^(n/4): a quarter turn
                    t = quarter<T, INV>(t);
                } else if (e) {
                    V w = tw[e * (n / len)];
                    t = cmul(t, INV ? conj_c<T>(w) : w);
                }
                v[i + e] = cadd(u, t);
                v[i + e + half] = csub(u, t);
            }
        }
    }
}

// Per-lane twiddle tables (bank-conflict free): tl[h - 1 + e] = w_2h^e for the
// cross-lane stage h (e < h), tk[32 (k1 - 1) + l] = w_n^(l k1).
template <typename T, int P>
__device__ __forceinline__ void load_lane_tw(V2<T> *tl, V2<T> *tk, const V2<T> *__restrict__ tw) {
    constexpr int n = 32 * P;
    for (int m = threadIdx.x; m < 32 + 32 * (P - 1); m += blockDim.x) {
        if (m < 31) {
            int h = 1;
            while (2 * h - 1 <= m) h <<= 1;
            tl[m] = tw[(m - (h - 1)) * (n / (2 * h))];
        } else if (m >= 32) {
            int mm = m - 32, k1 = mm / 32 + 1, l = mm & 31;
            tk[mm] = tw[(l * k1) & (n - 1)];
        }
    }
}

template <typename T, int P>
__device__ __forceinline__ void warp_fft_fwd(V2<T> *v, const V2<T> *tw, const V2<T> *tl, const V2<T> *tk,
                                             int lane) {
    constexpr int n = 32 * P;
    reg_dft<T, P, false>(v, tw, n);
#pragma unroll
    for (int k1 = 1; k1 < P; ++k1) v[k1] = cmul(v[k1], tk[32 * (k1 - 1) + lane]);
#pragma unroll
    for (int h = 16; h > 0; h >>= 1) {
        const T s = (lane & h) ? (T)-1 : (T)1;   // lower lane: a + b, upper lane: (a - b) w
        if (h >= 4) {
            V2<T> w = tl[h - 1 + (lane & (h - 1))];
            if (!(lane & h)) { w.x = (T)1; w.y = (T)0; }
#pragma unroll
            for (int k1 = 0; k1 < P; ++k1) {
                V2<T> p = shfl_xor_c<T>(v[k1], h), t;
                t.x = p.x + s * v[k1].x;
                t.y = p.y + s * v[k1].y;
                v[k1] = cmul(t, w);
            }
        } else {   // h = 2: w = 1 or -i (upper lanes with e = 1); h = 1: w = 1
            const bool rot = (h == 2) && (lane & 3) == 3;
#pragma unroll
            for (int k1 = 0; k1 < P; ++k1) {
                V2<T> p = shfl_xor_c<T>(v[k1], h), t;
                t.x = p.x + s * v[k1].x;
                t.y = p.y + s * v[k1].y;
                v[k1] = rot ? quarter<T, false>(t) : t;
            }
        }
    }
}

template <typename T, int P>
__device__ __forceinline__ void warp_fft_inv(V2<T> *v, const V2<T> *tw, const V2<T> *tl, const V2<T> *tk,
                                             int lane) {
    constexpr int n = 32 * P;
#pragma unroll
    for (int h = 1; h <= 16; h <<= 1) {
        const bool up = lane & h;   // lower lane: a + w b, upper lane: a - w b
        const T s = up ? (T)-1 : (T)1;
        // h = 1: w = 1; h = 2: w = 1 or +i (e = 1)
        const bool rot = (h == 2) && (lane & 1);
        V2<T> w;
        if (h >= 4) w = conj_c<T>(tl[h - 1 + (lane & (h - 1))]);
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) {
            V2<T> p = shfl_xor_c<T>(v[k1], h);
            V2<T> a = up ? p : v[k1], b = up ? v[k1] : p;
            if (h >= 4) b = cmul(b, w);
            else if (h == 2) b = rot ? quarter<T, true>(b) : b;
            v[k1].x = a.x + s * b.x;
            v[k1].y = a.y + s * b.y;
        }
    }
#pragma unroll
    for (int k1 = 1; k1 < P; ++k1) v[k1] = cmul(v[k1], conj_c<T>(tk[32 * (k1 - 1) + lane]));
    reg_dft<T, P, true>(v, tw, n);
}

// shared-memory row of wave number ky after the forward y pass: lane l's
// register k1 holds ky = k1 + P bitrev5(l) and is kept in row 32 k1 + l
template <int P> __device__ __forceinline__ int perm_row(int ky) { return (ky % P) * 32 + brev5(ky / P); }

// skewed index into a warp's line buffer: one pad entry per 16, so that the
// strided writes k1 + P bitrev5(l) and the natural reads are conflict free
__device__ __forceinline__ int zsk(int i) { return i + (i >> 4); }

// twiddle part of the plane kernels' shared memory: tw[n] | tl[32] | tk[32 (P - 1)]
template <int P> __host__ __device__ constexpr int plane_tw_entries() { return 32 * P + 32 + 32 * (P - 1); }

// x r2c + forward y FFT of plane z; clears the fixed-point plane it reads.
// Shared memory: twiddles | S[n][nh] (plane, row = y) | Zs[warps][n + n/16]
template <typename T, int P>
__global__ void __launch_bounds__(1024) k_plane_fwd(unsigned long long *__restrict__ Qfx, T fx_inv,
                                                    V2<T> *__restrict__ F, const V2<T> *__restrict__ tw,
                                                    FastDiv fnh) {
    mg_pdl_begin();
    typedef V2<T> V;
    constexpr int n = 32 * P, nh = n / 2 + 1;
    extern __shared__ unsigned char smem_raw[];
    V *s_tw = reinterpret_cast<V *>(smem_raw), *s_tl = s_tw + n, *s_tk = s_tl + 32;
    V *S = s_tw + plane_tw_entries<P>();
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    V *Zs = S + n * nh + w * (n + n / 16);
    load_tw<T>(s_tw, tw, n);
    load_lane_tw<T, P>(s_tl, s_tk, tw);
    __syncthreads();
    const size_t z = blockIdx.x;
    const int bl = brev5(lane);
    long long *Qp = reinterpret_cast<long long *>(Qfx) + z * n * n;
    // every line pair of this warp is loaded before the first transform
    constexpr int MP = (P + 1) / 2;   // pairs per warp at 32 warps
    long long raw[MP][2 * P];
#pragma unroll
    for (int r = 0; r < MP; ++r) {
        int pr = w + 32 * r;
        if (pr < n / 2) {
            long long *qa = Qp + (size_t)(2 * pr) * n, *qb = qa + n;
#pragma unroll
            for (int j = 0; j < P; ++j) {
                raw[r][2 * j] = qa[lane + 32 * j];
                raw[r][2 * j + 1] = qb[lane + 32 * j];
            }
#pragma unroll
            for (int j = 0; j < P; ++j) {   // the next spread accumulates into a cleared mesh
                qa[lane + 32 * j] = 0;
                qb[lane + 32 * j] = 0;
            }
        }
    }
#pragma unroll
    for (int r = 0; r < MP; ++r) {
        int pr = w + 32 * r;
        if (pr >= n / 2) break;
        V v[P];
#pragma unroll
        for (int j = 0; j < P; ++j) {
            v[j].x = fx_to_real<T>(raw[r][2 * j]) * fx_inv;
            v[j].y = fx_to_real<T>(raw[r][2 * j + 1]) * fx_inv;
        }
        warp_fft_fwd<T, P>(v, s_tw, s_tl, s_tk, lane);
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) Zs[zsk(k1 + P * bl)] = v[k1];
        __syncwarp();
        V *Sa = S + (2 * pr) * nh, *Sb = Sa + nh;
        for (int k = lane; k < nh; k += 32) {
            V zk = Zs[zsk(k)], zc = Zs[zsk((n - k) & (n - 1))];
            V a, b;
            // X_A = (Z_k + conj Z_{n-k})/2,  X_B = (Z_k - conj Z_{n-k})/(2i)
            a.x = (T)0.5 * (zk.x + zc.x);
            a.y = (T)0.5 * (zk.y - zc.y);
            b.x = (T)0.5 * (zk.y + zc.y);
            b.y = (T)-0.5 * (zk.x - zc.x);
            Sa[k] = a;
            Sb[k] = b;
        }
        __syncwarp();
    }
    __syncthreads();
    for (int c = w; c < nh; c += nw) {   // forward y FFT of column kx = c
        V v[P];
#pragma unroll
        for (int j = 0; j < P; ++j) v[j] = S[(lane + 32 * j) * nh + c];
        warp_fft_fwd<T, P>(v, s_tw, s_tl, s_tk, lane);
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) S[(32 * k1 + lane) * nh + c] = v[k1];
    }
    __syncthreads();
    V *Fp = F + z * n * nh;
    for (int e = threadIdx.x; e < n * nh; e += blockDim.x) {
        int ky = (int)fdiv((unsigned)e, fnh), kx = e - ky * nh;
        Fp[e] = S[perm_row<P>(ky) * nh + kx];
    }
}

// forward z FFT, influence function (energy and virial partial sums, times
// meshfac) and inverse z FFT of the slab ky.  Shared memory: twiddles |
// S[n][nh] (row = z) | mf, ew, vw of the octant row fy, [nh][nh] each
template <typename T, int P>
__global__ void __launch_bounds__(1024) k_slab_conv(V2<T> *__restrict__ F, const V2<T> *__restrict__ tw,
                                                    ConvArgs cv, FastDiv fnh) {
    typedef V2<T> V;
    constexpr int n = 32 * P, nh = n / 2 + 1;
    extern __shared__ unsigned char smem_raw[];
    __shared__ double red[2 * 32];
    V *s_tw = reinterpret_cast<V *>(smem_raw), *s_tl = s_tw + n, *s_tk = s_tl + 32;
    V *S = s_tw + plane_tw_entries<P>();
    T *s_mf = reinterpret_cast<T *>(S + n * nh), *s_ew = s_mf + nh * nh, *s_vw = s_ew + nh * nh;
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    load_tw<T>(s_tw, tw, n);
    load_lane_tw<T, P>(s_tl, s_tk, tw);
    const int ky = blockIdx.x, fy = min(ky, n - ky);
    const T *mf = (const T *)cv.mf, *ew = (const T *)cv.ew, *vw = (const T *)cv.vw;
    for (int e = threadIdx.x; e < nh * nh; e += blockDim.x) {   // constant tables: before the wait
        int fz = (int)fdiv((unsigned)e, fnh), kx = e - fz * nh;
        size_t id = ((size_t)fz * nh + fy) * nh + kx;
        s_mf[e] = mf[id];
        s_ew[e] = ew[id];
        s_vw[e] = vw[id];
    }
    mg_pdl_begin();
    for (int e = threadIdx.x; e < n * nh; e += blockDim.x) {
        int zz = (int)fdiv((unsigned)e, fnh), kx = e - zz * nh;
        S[e] = F[((size_t)zz * n + ky) * nh + kx];
    }
    __syncthreads();
    const int bl = brev5(lane);
    T e_t = 0, v_t = 0;
    for (int c = w; c < nh; c += nw) {
        V v[P];
#pragma unroll
        for (int j = 0; j < P; ++j) v[j] = S[(lane + 32 * j) * nh + c];
        warp_fft_fwd<T, P>(v, s_tw, s_tl, s_tk, lane);
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) {
            int kz = k1 + P * bl;
            int id = min(kz, n - kz) * nh + c;
            T p2 = v[k1].x * v[k1].x + v[k1].y * v[k1].y;
            e_t += p2 * s_ew[id];
            v_t -= p2 * s_vw[id];
            T m = s_mf[id];
            v[k1].x *= m;
            v[k1].y *= m;
        }
        warp_fft_inv<T, P>(v, s_tw, s_tl, s_tk, lane);
#pragma unroll
        for (int j = 0; j < P; ++j) S[(lane + 32 * j) * nh + c] = v[j];
    }
    for (int o = 16; o > 0; o >>= 1) {   // warp sums in the mesh type, FP64 across warps
        e_t += __shfl_down_sync(0xffffffffu, e_t, o);
        v_t += __shfl_down_sync(0xffffffffu, v_t, o);
    }
    if (lane == 0) { red[w] = (double)e_t; red[32 + w] = (double)v_t; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double se = 0.0, sv = 0.0;
        for (int k = 0; k < nw; ++k) { se += red[k]; sv += red[32 + k]; }
        cv.part[2 * blockIdx.x] = se;
        cv.part[2 * blockIdx.x + 1] = sv;
    }
    for (int e = threadIdx.x; e < n * nh; e += blockDim.x) {
        int zz = (int)fdiv((unsigned)e, fnh), kx = e - zz * nh;
        F[((size_t)zz * n + ky) * nh + kx] = S[e];
    }
}

// inverse y FFT + x c2r of plane z (Hermitian input: imaginary parts of
// kx = 0 and n/2 dropped).  Shared memory as k_plane_fwd.
template <typename T, int P>
__global__ void __launch_bounds__(1024) k_plane_inv(const V2<T> *__restrict__ F, T *__restrict__ Q,
                                                    const V2<T> *__restrict__ tw, FastDiv fnh) {
    typedef V2<T> V;
    constexpr int n = 32 * P, nh = n / 2 + 1;
    extern __shared__ unsigned char smem_raw[];
    V *s_tw = reinterpret_cast<V *>(smem_raw), *s_tl = s_tw + n, *s_tk = s_tl + 32;
    V *S = s_tw + plane_tw_entries<P>();
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    V *Zs = S + n * nh + w * (n + n / 16);
    load_tw<T>(s_tw, tw, n);
    load_lane_tw<T, P>(s_tl, s_tk, tw);
    mg_pdl_begin();   // the twiddles need nothing from before
    const size_t z = blockIdx.x;
    const V *Fp = F + z * n * nh;
    for (int e = threadIdx.x; e < n * nh; e += blockDim.x) {
        int ky = (int)fdiv((unsigned)e, fnh), kx = e - ky * nh;
        S[perm_row<P>(ky) * nh + kx] = Fp[e];
    }
    __syncthreads();
    for (int c = w; c < nh; c += nw) {   // inverse y FFT of column kx = c
        V v[P];
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) v[k1] = S[(32 * k1 + lane) * nh + c];
        warp_fft_inv<T, P>(v, s_tw, s_tl, s_tk, lane);
#pragma unroll
        for (int j = 0; j < P; ++j) S[(lane + 32 * j) * nh + c] = v[j];
    }
    __syncthreads();
    const int bl = brev5(lane);
    T *Qp = Q + z * n * n;
    for (int pr = w; pr < n / 2; pr += nw) {
        const V *Sa = S + (2 * pr) * nh, *Sb = Sa + nh;
        for (int k = lane; k < n; k += 32) {
            int kk = (k < nh) ? k : n - k;
            V a = Sa[kk], b = Sb[kk];
            if (kk == 0 || 2 * kk == n) { a.y = (T)0; b.y = (T)0; }
            if (k >= nh) { a.y = -a.y; b.y = -b.y; }
            V zz;
            zz.x = a.x - b.y;
            zz.y = a.y + b.x;
            Zs[zsk(k)] = zz;
        }
        __syncwarp();
        V v[P];
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) v[k1] = Zs[zsk(k1 + P * bl)];
        __syncwarp();
        warp_fft_inv<T, P>(v, s_tw, s_tl, s_tk, lane);
        T *qa = Qp + (size_t)(2 * pr) * n, *qb = qa + n;
#pragma unroll
        for (int j = 0; j < P; ++j) {
            qa[lane + 32 * j] = v[j].x;
            qb[lane + 32 * j] = v[j].y;
        }
    }
}

// ---- fused spread and forward plane pass ---------------------------------------
// Particles are counting-sorted by the z plane c2 of their stamp corner
// (start[c2] .. start[c2+1]), their spread records copied into that order.
// Stamp point iz of a particle lies on plane (c2 - iz) mod n, so the
// particles reaching plane z are those with c2 = z + iz (mod n), iz < ORDER:
// ORDER ranges of the plane order, the plane's window.  One CTA per plane
// spreads its window's (particle, plane) items into the plane in shared
// memory and transforms it: the charge mesh never goes to global memory.
struct PlaneArgs {
    const int *start;
    int *count;                // plane counts of the sort, cleared here for the next call
    const float *srec;         // spread records in plane order (spread_rec values each)
    float mmax2;               // (largest B-spline value)^2
    int *err;
};

// the window of plane z in shared memory: ws[iz] = items before range iz,
// wb[iz] = its first index into the plane order; ws[ORDER] = the item count
template <int ORDER>
__device__ __forceinline__ void plane_window(const PlaneArgs &a, int z, int n, int *wb, int *ws) {
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int iz = 0; iz < ORDER; ++iz) {
            int c2 = (z + iz) & (n - 1);
            wb[iz] = a.start[c2];
            ws[iz] = acc;
            acc += a.start[c2 + 1] - a.start[c2];
        }
        ws[ORDER] = acc;
    }
}

template <int ORDER> __device__ __forceinline__ int window_iz(const int *ws, int t) {
    int iz = 0;
#pragma unroll
    for (int k = 1; k < ORDER; ++k) iz += (t >= ws[k]) ? 1 : 0;
    return iz;
}

// Spread of the plane's window into the plane, then x r2c + forward y FFT
// as k_plane_fwd.  One lane per item; rows are padded to n + 1 points so
// that the lanes' stamp rows spread over the banks.  Stamp values are added
// as 32-bit integers v = round(q Mx My Mz 2^s) with one shared-memory
// atomic each.  The plane's scale 2^s comes from a bound of its largest
// point sum: an item adds at most |q| Mz(plane) mmax^2 to any point of the
// ORDER rows its stamp covers, so the largest of the rows' sums of those
// terms (fixed point, rounded up, integer atomics) bounds every point, and
// B 2^s < 2^30 keeps the integer sums clear of overflow.  Integer sums do
// not depend on the order of the adds, so the plane is bit-reproducible.  The integer plane shares memory with the FFT's plane
// and line buffers, which are used only after every line has been read
// into registers.
template <int P, int ORDER>
__global__ void __launch_bounds__(1024) k_plane_spread_fwd(PlaneArgs a, float2 *__restrict__ F,
                                                           const float2 *__restrict__ tw, FastDiv fnh) {
    typedef float2 V;
    typedef float T;
    constexpr int n = 32 * P, nh = n / 2 + 1, RS = n + 1, n2 = n * RS;
    constexpr int SR = spread_rec<ORDER>();
    typedef RecIx<ORDER> RI;
    extern __shared__ unsigned char smem_raw[];
    __shared__ int wb[ORDER], ws[ORDER + 1];
    V *s_tw = reinterpret_cast<V *>(smem_raw), *s_tl = s_tw + n, *s_tk = s_tl + 32;
    V *S = s_tw + plane_tw_entries<P>();
    int *tacc = reinterpret_cast<int *>(S);
    __shared__ int rowb[n], bmax[32];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    V *Zs = S + n * nh + w * (n + n / 16);
    load_tw<T>(s_tw, tw, n);
    load_lane_tw<T, P>(s_tl, s_tk, tw);
    for (int k = threadIdx.x; k < n2; k += blockDim.x) tacc[k] = 0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) rowb[k] = 0;
    const int z = blockIdx.x;
    mg_pdl_begin();   // the twiddles and the cleared planes above need nothing from before
    plane_window<ORDER>(a, z, n, wb, ws);
    if (threadIdx.x == 0) a.count[z] = 0;   // read by the scatter, which has finished
    __syncthreads();
    const int total = ws[ORDER];
    // per row of the plane: the sum of |q| Mz mmax^2 over the items whose
    // stamp covers it, in units of 2^-12, each term rounded up
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int iz = window_iz<ORDER>(ws, t);
        const float *rec = a.srec + (size_t)(wb[iz] + t - ws[iz]) * SR;
        int bt = (int)ceilf(fabsf(rec[1]) * rec[RI::VZ + iz] * a.mmax2 * 4096.0f) + 1;
        int c1 = (rec_corner(rec[0]) >> 10) & 1023;
#pragma unroll
        for (int iy = 0; iy < ORDER; ++iy) atomicAdd(&rowb[(c1 - iy) & (n - 1)], bt);
    }
    __syncthreads();
    int m = 0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) m = max(m, rowb[k]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) bmax[w] = m;
    __syncthreads();
    int mb = 0;
    for (int k = 0; k < nw; ++k) mb = max(mb, bmax[k]);
    // B 2^s < 2^30 with B < 2^e
    int e;
    frexpf((float)mb * (1.0f / 4096.0f), &e);
    const int sh = min(30 - e, 60);
    const float scale = ldexpf(1.0f, sh), inv = ldexpf(1.0f, -sh);
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int iz = window_iz<ORDER>(ws, t);
        const float *rec = a.srec + (size_t)(wb[iz] + t - ws[iz]) * SR;
        float r[RI::SB];
        load_rec<float, RI::SB>(rec, r);   // head, z, x and y values
        float mz = r[RI::VZ];
#pragma unroll
        for (int k = 1; k < ORDER; ++k)
            if (k == iz) mz = r[RI::VZ + k];
        float qz = r[1] * mz * scale;
        int c = rec_corner(r[0]);
        int c0 = c & 1023, c1 = (c >> 10) & 1023;
#pragma unroll
        for (int iy = 0; iy < ORDER; ++iy) {
            float wyz = r[RI::VY + iy] * qz;
            int row = ((c1 - iy) & (n - 1)) * RS;
#pragma unroll
            for (int ix = 0; ix < ORDER; ++ix) {
                int v = __float2int_rn(r[RI::VX + ix] * wyz);
                atomicAdd(&tacc[row + ((c0 - ix) & (n - 1))], v);
            }
        }
    }
    __syncthreads();
    constexpr int MP = (P + 1) / 2;   // line pairs per warp at 32 warps
    T val[MP][2 * P];
#pragma unroll
    for (int r = 0; r < MP; ++r) {
        int pr = w + 32 * r;
        if (pr < n / 2) {
#pragma unroll
            for (int j = 0; j < P; ++j) {
                int ka = (2 * pr) * RS + lane + 32 * j, kb = ka + RS;
                val[r][2 * j] = (float)tacc[ka] * inv;
                val[r][2 * j + 1] = (float)tacc[kb] * inv;
            }
        }
    }
    __syncthreads();   // the integer planes are dead: S and Zs take their place
    const int bl = brev5(lane);
#pragma unroll
    for (int r = 0; r < MP; ++r) {
        int pr = w + 32 * r;
        if (pr >= n / 2) break;
        V v[P];
#pragma unroll
        for (int j = 0; j < P; ++j) {
            v[j].x = val[r][2 * j];
            v[j].y = val[r][2 * j + 1];
        }
        warp_fft_fwd<T, P>(v, s_tw, s_tl, s_tk, lane);
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) Zs[zsk(k1 + P * bl)] = v[k1];
        __syncwarp();
        V *Sa = S + (2 * pr) * nh, *Sb = Sa + nh;
        for (int k = lane; k < nh; k += 32) {
            V zk = Zs[zsk(k)], zc = Zs[zsk((n - k) & (n - 1))];
            V aa, bb;
            aa.x = (T)0.5 * (zk.x + zc.x);
            aa.y = (T)0.5 * (zk.y - zc.y);
            bb.x = (T)0.5 * (zk.y + zc.y);
            bb.y = (T)-0.5 * (zk.x - zc.x);
            Sa[k] = aa;
            Sb[k] = bb;
        }
        __syncwarp();
    }
    __syncthreads();
    for (int c = w; c < nh; c += nw) {   // forward y FFT of column kx = c
        V v[P];
#pragma unroll
        for (int j = 0; j < P; ++j) v[j] = S[(lane + 32 * j) * nh + c];
        warp_fft_fwd<T, P>(v, s_tw, s_tl, s_tk, lane);
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) S[(32 * k1 + lane) * nh + c] = v[k1];
    }
    __syncthreads();
    V *Fp = F + (size_t)z * n * nh;
    for (int e = threadIdx.x; e < n * nh; e += blockDim.x) {
        int ky = (int)fdiv((unsigned)e, fnh), kx = e - ky * nh;
        Fp[e] = S[perm_row<P>(ky) * nh + kx];
    }
}

template <int P> static size_t fused_fwd_smem() {
    const int n = 32 * P, nh = n / 2 + 1;
    size_t fft = sizeof(float2) * ((size_t)n * nh + (size_t)32 * (n + n / 16));
    size_t tiles = sizeof(int) * (size_t)n * (n + 1);
    return sizeof(float2) * (size_t)plane_tw_entries<P>() + std::max(fft, tiles);
}

template <int P> static size_t plane_smem(int warps) {
    const int n = 32 * P, nh = n / 2 + 1;
    return sizeof(float2) * ((size_t)plane_tw_entries<P>() + (size_t)n * nh + (size_t)warps * (n + n / 16));
}
template <int P> static size_t slab_smem() {
    const int n = 32 * P, nh = n / 2 + 1;
    return sizeof(float2) * ((size_t)plane_tw_entries<P>() + (size_t)n * nh) + 3 * sizeof(float) * (size_t)nh * nh;
}

template <int P>
static int plane_passes(mg_handle *h, float *Q, float2 *F, const float2 *tw, ConvArgs cv, float fx_inv) {
    const int n = 32 * P, thr = 32 * h->fft_warps;
    FastDiv fnh = make_fastdiv((unsigned)h->nh);
    MG_TRY(mg_phase_begin(h, "fft_xy_fwd"));
    mg_launch_pdl(k_plane_fwd<float, P>, n, thr, plane_smem<P>(h->fft_warps), h->st, h->d_Qfx, fx_inv, F, tw, fnh);
    MG_TRY(mg_phase_end(h, "fft_xy_fwd"));
    MG_TRY(mg_phase_begin(h, "fft_z_conv"));
    mg_launch_pdl(k_slab_conv<float, P>, n, thr, slab_smem<P>(), h->st, F, tw, cv, fnh);
    if (h->par_forces) MG_CUDA(h, cudaEventRecord(h->ev_rec, h->st));   // reciprocal partials complete
    MG_TRY(mg_phase_end(h, "fft_z_conv"));
    MG_TRY(mg_phase_begin(h, "fft_yx_inv"));
    mg_launch_pdl(k_plane_inv<float, P>, n, thr, plane_smem<P>(h->fft_warps), h->st, (const float2 *)F, Q, tw, fnh);
    MG_TRY(mg_phase_end(h, "fft_yx_inv"));
    h->launches += 3;
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

static int plane_dispatch(mg_handle *h, float *Q, float2 *F, const float2 *tw, ConvArgs cv, float fx_inv) {
    switch (h->nmesh) {
    case 32: return plane_passes<1>(h, Q, F, tw, cv, fx_inv);
    case 64: return plane_passes<2>(h, Q, F, tw, cv, fx_inv);
    case 128: return plane_passes<4>(h, Q, F, tw, cv, fx_inv);
    default: return mg_fail(h, MG_ERR_UNSUPPORTED, "plane FFT for nmesh = %d", h->nmesh);
    }
}

// the plane passes with the spread fused into the forward one: spread +
// x/y forward per plane, the z pass with the influence function per ky
// slab, y/x inverse per plane (the potential mesh, for the gather)
template <int P, int ORDER> static int fused_passes_o(mg_handle *h, const PlaneArgs &pa) {
    const int n = 32 * P, thr = 32 * h->fft_warps;
    float2 *F = (float2 *)h->d_F;
    const float2 *tw = (const float2 *)h->d_tw;
    FastDiv fnh = make_fastdiv((unsigned)h->nh);
    ConvArgs cv;
    cv.part = h->d_part + h->part_rec;
    cv.mf = h->d_mf_f;
    cv.ew = h->d_ew_f;
    cv.vw = h->d_vw_f;
    MG_TRY(mg_phase_begin(h, "spread+fft_xy"));
    mg_launch_pdl(k_plane_spread_fwd<P, ORDER>, n, thr, fused_fwd_smem<P>(), h->st, pa, F, tw, fnh);
    MG_TRY(mg_phase_end(h, "spread+fft_xy"));
    MG_TRY(mg_phase_begin(h, "fft_z_conv"));
    mg_launch_pdl(k_slab_conv<float, P>, n, thr, slab_smem<P>(), h->st, F, tw, cv, fnh);
    if (h->par_forces) MG_CUDA(h, cudaEventRecord(h->ev_rec, h->st));   // reciprocal partials complete
    MG_TRY(mg_phase_end(h, "fft_z_conv"));
    MG_TRY(mg_phase_begin(h, "fft_yx_inv"));
    mg_launch_pdl(k_plane_inv<float, P>, n, thr, plane_smem<P>(h->fft_warps), h->st, (const float2 *)F,
                  (float *)h->d_Q, tw, fnh);
    MG_TRY(mg_phase_end(h, "fft_yx_inv"));
    h->launches += 3;
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

template <int P> static int fused_passes(mg_handle *h, const PlaneArgs &pa) {
    switch (h->order) {
    case 4: return fused_passes_o<P, 4>(h, pa);
    case 5: return fused_passes_o<P, 5>(h, pa);
    case 6: return fused_passes_o<P, 6>(h, pa);
    case 7: return fused_passes_o<P, 7>(h, pa);
    case 8: return fused_passes_o<P, 8>(h, pa);
    default: return mg_fail(h, MG_ERR_UNSUPPORTED, "fused plane passes for order %d", h->order);
    }
}

template <int P> static void set_plane_limits() {
    cudaFuncSetAttribute(k_plane_fwd<float, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_slab_conv<float, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_plane_inv<float, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_plane_spread_fwd<P, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_plane_spread_fwd<P, 5>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_plane_spread_fwd<P, 6>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_plane_spread_fwd<P, 7>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_plane_spread_fwd<P, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

template <typename T>
int fft_launch(mg_handle *h, T *Q, V2<T> *F, const V2<T> *tw, ConvArgs cv, T fx_inv) {
    if constexpr (std::is_same<T, float>::value) {
        if (h->fft_plane) return plane_dispatch(h, Q, F, tw, cv, fx_inv);
    }
    int n = h->nmesh, nh = h->nh;
    FftPlan pl = make_plan(n);
    // line pairs per CTA in the x passes: the n^2 lines in groups of 2 lp
    int lp = n % 4 == 0 ? 4 : 1;
    size_t vsz = sizeof(V2<T>);
    size_t smx = vsz * (n + 2 * (size_t)lp * n);
    int thx = max(32, min(1024, lp * n / 4));
    int gx = n * n / (2 * lp);
    size_t smc = vsz * (n + 2 * (size_t)h->fft_tx * n);
    int thc = max(32, min(1024, ((h->fft_tx * n / 4) + 31) / 32 * 32));
    dim3 gc(h->fft_tiles, n);
    size_t ystride = nh, yother = (size_t)n * nh;   // y pass: t -> y, other -> z
    size_t zstride = (size_t)n * nh, zother = nh;   // z pass: t -> z, other -> y
    MG_TRY(mg_phase_begin(h, "fft_x_r2c"));
    FastDiv fnh = make_fastdiv((unsigned)nh), ftx = make_fastdiv((unsigned)h->fft_tx);
    k_fft_x_r2c<T><<<gx, thx, smx, h->st>>>((const long long *)h->d_Qfx, fx_inv, F, n, pl, lp, tw, fnh);
    // the next spread accumulates into a cleared mesh
    MG_CUDA(h, cudaMemsetAsync(h->d_Qfx, 0, sizeof(long long) * (size_t)n * n * n, h->st));
    MG_TRY(mg_phase_end(h, "fft_x_r2c"));
    MG_TRY(mg_phase_begin(h, "fft_y_fwd"));
    k_fft_col<T, false><<<gc, thc, smc, h->st>>>(F, n, pl, nh, h->fft_tx, ystride, yother, -1, tw, cv, ftx);
    MG_TRY(mg_phase_end(h, "fft_y_fwd"));
    MG_TRY(mg_phase_begin(h, "fft_z_conv"));
    k_fft_col<T, true><<<gc, thc, smc, h->st>>>(F, n, pl, nh, h->fft_tx, zstride, zother, -1, tw, cv, ftx);
    if (h->par_forces) MG_CUDA(h, cudaEventRecord(h->ev_rec, h->st));   // reciprocal partials complete
    MG_TRY(mg_phase_end(h, "fft_z_conv"));
    MG_TRY(mg_phase_begin(h, "fft_y_inv"));
    k_fft_col<T, false><<<gc, thc, smc, h->st>>>(F, n, pl, nh, h->fft_tx, ystride, yother, +1, tw, cv, ftx);
    MG_TRY(mg_phase_end(h, "fft_y_inv"));
    MG_TRY(mg_phase_begin(h, "fft_x_c2r"));
    k_fft_x_c2r<T><<<gx, thx, smx, h->st>>>(F, Q, n, pl, lp, tw);
    MG_TRY(mg_phase_end(h, "fft_x_c2r"));
    h->launches += 5;
    return MG_OK;
}

// ---- UDipoleEwaldRecSPM (energy.F90:2046-2170) ---------------------------------
// CardinalBSpline (mollib.F90:1629-1685) with first and second derivatives,
// the recursion and divisions as there; the second derivatives come from
// the values of order-2 (zero for order 3 and below, as there)
__device__ void dip_bspline(int order, double pos, int &kmax, double *v, double *d, double *d2) {
    double last[MG_MAX_ORDER], last2[MG_MAX_ORDER];
    int iv = (int)floor(pos);
    double x = pos - iv;
    kmax = iv;
    for (int i = 0; i < order; ++i) { last[i] = 0.0; last2[i] = 0.0; v[i] = 0.0; }
    v[0] = x;
    v[1] = 1.0 - x;
    for (int n = 3; n <= order; ++n) {
        for (int i = 0; i < order; ++i) last[i] = v[i];
        if (n == order - 1)
            for (int i = 0; i < order; ++i) last2[i] = v[i];
        v[0] = x * last[0] / (n - 1);
        for (int i = 1; i <= n - 2; ++i) {
            double a = i + x;
            v[i] = (a * last[i] + (n - a) * last[i - 1]) / (n - 1);
        }
        v[n - 1] = (1 - x) * last[n - 2] / (n - 1);
    }
    d[0] = last[0];
    for (int i = 1; i <= order - 2; ++i) d[i] = last[i] - last[i - 1];
    d[order - 1] = -last[order - 2];
    d2[0] = last2[0];
    d2[1] = last2[1] - 2 * last2[0];
    for (int i = 2; i <= order - 3; ++i) d2[i] = last2[i] - 2 * last2[i - 1] + last2[i - 2];
    if (order > 3) d2[order - 2] = -2 * last2[order - 3] + last2[order - 4];
    if (order > 2) d2[order - 1] = last2[order - 3];
}

struct DipMeshArgs {
    const double *ro, *az, *dip;
    int np, order, n;
    double dkdr[3];
};

// the generalized charge mesh: one thread per particle, q M_x M_y M_z +
// dkdr . dip (derivative products) at each stamp point, added to the
// fixed-point mesh with 64-bit integer atomics (scale 2^k)
__global__ void __launch_bounds__(128) k_dip_spread(DipMeshArgs a, double scale, unsigned long long *__restrict__ Qfx) {
    int ia = blockIdx.x * blockDim.x + threadIdx.x;
    if (ia >= a.np) return;
    const int order = a.order, n = a.n;
    double sp[3][MG_MAX_ORDER], dr[3][MG_MAX_ORDER], d2[MG_MAX_ORDER];
    int mm[3];
    for (int m = 0; m < 3; ++m) {
        int kmax;
        dip_bspline(order, a.dkdr[m] * a.ro[3 * ia + m], kmax, sp[m], dr[m], d2);
        mm[m] = ((kmax % n) + n) % n;
    }
    double dx2 = a.dip[3 * ia] * a.dkdr[0], dy2 = a.dip[3 * ia + 1] * a.dkdr[1], dz2 = a.dip[3 * ia + 2] * a.dkdr[2];
    double q0 = a.az[ia];
    for (int iz = 0; iz < order; ++iz) {
        int nz = (n + mm[2] - iz) % n;
        double splz = sp[2][iz], dsdz = dr[2][iz];
        for (int iy = 0; iy < order; ++iy) {
            int ny = (n + mm[1] - iy) % n;
            double sply = sp[1][iy];
            double q1 = q0 * sply * splz;
            double dipx1 = dx2 * sply * splz;
            double dipy1 = dy2 * dr[1][iy] * splz;
            double dipz1 = dz2 * sply * dsdz;
            size_t row = ((size_t)nz * n + ny) * n;
            for (int ix = 0; ix < order; ++ix) {
                int nx = (n + mm[0] - ix) % n;
                double splx = sp[0][ix];
                double val = q1 * splx + dipx1 * dr[0][ix] + dipy1 * splx + dipz1 * splx;
                atomicAdd(&Qfx[row + nx], (unsigned long long)__double2ll_rn(val * scale));
            }
        }
    }
}

// potential, field, field gradient (second derivatives) at each particle
// from the potential mesh, and the dipole term of the virial: one warp per
// particle, lanes over the (iy, iz) rows, the sums combined by shuffles in
// a fixed order
__global__ void __launch_bounds__(128) k_dip_gather(DipMeshArgs a, const double *__restrict__ Q,
                                                    double *__restrict__ pot, double *__restrict__ est,
                                                    double *__restrict__ efg, double *__restrict__ vir) {
    int ia = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (ia >= a.np) return;
    const int order = a.order, n = a.n;
    double sp[3][MG_MAX_ORDER], dr[3][MG_MAX_ORDER], dd[3][MG_MAX_ORDER];
    int mm[3];
    for (int m = 0; m < 3; ++m) {
        int kmax;
        dip_bspline(order, a.dkdr[m] * a.ro[3 * ia + m], kmax, sp[m], dr[m], dd[m]);
        mm[m] = ((kmax % n) + n) % n;
    }
    double dx2 = a.dip[3 * ia] * a.dkdr[0], dy2 = a.dip[3 * ia + 1] * a.dkdr[1], dz2 = a.dip[3 * ia + 2] * a.dkdr[2];
    double acc[11];
    for (int k = 0; k < 11; ++k) acc[k] = 0.0;
    for (int t = lane; t < order * order; t += 32) {
        int iz = t / order, iy = t - iz * order;
        int nz = (n + mm[2] - iz) % n, ny = (n + mm[1] - iy) % n;
        double splz = sp[2][iz], dsdz = dr[2][iz], d2sdz = dd[2][iz];
        double sply = sp[1][iy], dsdy = dr[1][iy], d2sdy = dd[1][iy];
        const double *row = Q + ((size_t)nz * n + ny) * n;
        for (int ix = 0; ix < order; ++ix) {
            int nx = (n + mm[0] - ix) % n;
            double splx = sp[0][ix], dsdx = dr[0][ix], d2sdx = dd[0][ix];
            double qv = row[nx];
            acc[0] += splx * sply * splz * qv;
            acc[1] += dsdx * sply * splz * qv;
            acc[2] += splx * dsdy * splz * qv;
            acc[3] += splx * sply * dsdz * qv;
            acc[4] += d2sdx * sply * splz * qv;
            acc[5] += splx * d2sdy * splz * qv;
            acc[6] += splx * sply * d2sdz * qv;
            acc[7] += dsdx * dsdy * splz * qv;
            acc[8] += dsdx * sply * dsdz * qv;
            acc[9] += splx * dsdy * dsdz * qv;
            double qdip = dx2 * dsdx * sply * splz + dy2 * splx * dsdy * splz + dz2 * splx * sply * dsdz;
            acc[10] -= qdip * qv;
        }
    }
    for (int k = 0; k < 11; ++k)
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
    if (lane != 0) return;
    const double *dk = a.dkdr;
    double d2k[6] = {dk[0] * dk[0], dk[1] * dk[1], dk[2] * dk[2], dk[0] * dk[1], dk[0] * dk[2], dk[1] * dk[2]};
    pot[ia] += acc[0];
    for (int m = 0; m < 3; ++m) est[3 * ia + m] -= acc[1 + m] * dk[m];   // E = -dU/dr
    for (int m = 0; m < 6; ++m) efg[6 * ia + m] -= acc[4 + m] * d2k[m];
    vir[ia] = acc[10];
}

template <typename T> void set_smem_limits() {
    cudaFuncSetAttribute(k_fft_x_r2c<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_fft_x_c2r<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_fft_col<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_fft_col<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if constexpr (std::is_same<T, float>::value) {
        set_plane_limits<1>();
        set_plane_limits<2>();
        set_plane_limits<4>();
    }
}

}  // namespace

int mg_spme_init(mg_handle *h) {
    int n = h->nmesh;
    bool pow2 = n >= 8 && (n & (n - 1)) == 0;
    if (n < 8 || n > 512 || n % 2 != 0 || (!pow2 && make_plan(n).nf == 0))
        return mg_fail(h, MG_ERR_UNSUPPORTED,
                       "nmesh = %d: the device FFT supports even meshes 2^a 3^b 5^c from 8 to 512", n);
    h->gen_mesh = pow2 ? 0 : 1;
    if (h->order > n) return mg_fail(h, MG_ERR_UNSUPPORTED, "SPME order %d > nmesh %d", h->order, n);
    if (h->order < 2 || h->order > MG_MAX_ORDER)
        return mg_fail(h, MG_ERR_UNSUPPORTED, "SPME order %d outside 2..%d", h->order, MG_MAX_ORDER);
    h->nh = n / 2 + 1;
    for (int m = 0; m < 3; ++m) h->dkdr[m] = n / h->boxlen[m];
    // column tiles: at most 16 columns, as few tiles as possible
    int tiles = (h->nh + 15) / 16;
    h->fft_tiles = tiles;
    h->fft_tx = (h->nh + tiles - 1) / tiles;
    h->nblk_rec = tiles * n;
    // mixed form, 32 <= n <= 128: plane passes, 32 warps per plane, one
    // partial sum per ky slab
    h->fft_plane = (h->form == MG_MIXED && pow2 && n >= 32 && n <= 128) ? 1 : 0;
    if (h->fft_plane) {
        h->fft_warps = 32;
        h->nblk_rec = n;
    }
    // the spread fused into the forward plane pass: MD and BD (MC keeps the
    // charge mesh of the accepted state), orders up to 8
    h->plane_fused = (h->fft_plane && h->mode != MG_MC && h->order >= 4 && h->order <= 8) ? 1 : 0;
    // bricks of 8^3 points (16^3 for orders above 9, whose halo would
    // otherwise reach beyond the next brick)
    if (h->order < 4) return mg_fail(h, MG_ERR_UNSUPPORTED, "SPME order %d (supported: 4..12)", h->order);
    h->brick = (h->order - 1 > 8) ? 16 : 8;
    if (h->brick > n) h->brick = n;
    if (h->order - 1 > h->brick)
        return mg_fail(h, MG_ERR_UNSUPPORTED, "SPME order %d too large for mesh %d", h->order, n);
    h->nbrick_edge = n / h->brick;
    h->nbricks = h->nbrick_edge * h->nbrick_edge * h->nbrick_edge;
    int tile = h->brick + h->order - 1;
    size_t acc = (h->form == MG_MIXED) ? sizeof(int) : sizeof(double);
    size_t tsz = (h->form == MG_MIXED) ? sizeof(float) : sizeof(double);
    size_t t3 = (size_t)tile * tile * tile;
    // warps (work items) per block: the count that keeps the most warps
    // resident per SM (228 KB of shared memory, 1 KB reserved per block)
    size_t stage = 32 * sizeof(int) + 32 * (3 * (size_t)h->order + 1) * tsz;   // per-warp particle staging
    int best = 0;
    h->spread_wpb = 0;
    for (int wpb = 1; wpb <= kSpreadWarps; ++wpb) {
        size_t blk = ((wpb * acc * t3 + 15) & ~(size_t)15) + wpb * stage;
        if (blk > (size_t)200 * 1024) break;
        int blocks = std::min<int>(32, (int)((size_t)228 * 1024 / (blk + 1024)));
        if (blocks * wpb >= best) { best = blocks * wpb; h->spread_wpb = wpb; }
    }
    if (h->spread_wpb < 1)
        return mg_fail(h, MG_ERR_UNSUPPORTED, "SPME spread tile does not fit in shared memory");
    h->spread_smem = ((h->spread_wpb * acc * t3 + 15) & ~(size_t)15) + h->spread_wpb * stage;
    // lane-per-particle spread (mixed form): a 32-bit tile per warp, no staging
    {
        int bestl = 0;
        h->spread_wpb_lane = 1;
        for (int wpb = 1; wpb <= kSpreadWarps; ++wpb) {
            size_t blk = wpb * sizeof(int) * t3;
            if (blk > (size_t)200 * 1024) break;
            int blocks = std::min<int>(32, (int)((size_t)228 * 1024 / (blk + 1024)));
            if (blocks * wpb >= bestl) { bestl = blocks * wpb; h->spread_wpb_lane = wpb; }
        }
        h->spread_smem_lane = h->spread_wpb_lane * sizeof(int) * t3;
    }
    h->spread_m = kSpreadItem;
    h->max_items = h->nbricks + (h->np + kSpreadItem - 1) / kSpreadItem;
    MG_CUDA(h, cudaMalloc(&h->d_brick_count, sizeof(int) * h->nbricks));
    MG_CUDA(h, cudaMemset(h->d_brick_count, 0, sizeof(int) * h->nbricks));
    MG_CUDA(h, cudaMalloc(&h->d_brick_start, sizeof(int) * (h->nbricks + 1)));
    MG_CUDA(h, cudaMalloc(&h->d_brick_perm, sizeof(int) * h->np));
    MG_CUDA(h, cudaMalloc(&h->d_brick_rank, sizeof(int) * h->np));
    MG_CUDA(h, cudaMalloc(&h->d_brick_of, sizeof(int) * h->np));
    MG_CUDA(h, cudaMalloc(&h->d_brick_istart, sizeof(int) * (h->nbricks + 1)));
    MG_CUDA(h, cudaMalloc(&h->d_item_brick, sizeof(int) * h->max_items));
    MG_CUDA(h, cudaMalloc(&h->d_Qfx, sizeof(long long) * (size_t)n * n * n));
    MG_CUDA(h, cudaMemset(h->d_Qfx, 0, sizeof(long long) * (size_t)n * n * n));
    MG_CUDA(h, cudaMalloc(&h->d_spl_w, tsz * spl_rec(h->order) * (size_t)h->np));   // spline records
    if (h->plane_fused)   // spread records in plane order (at most order 8)
        MG_CUDA(h, cudaMalloc(&h->d_spl_plane, sizeof(float) * spread_rec<8>() * (size_t)h->np));
    spread_attrs<float, int>();
    spread_attrs<double, long long>();
    spread_lane_attr<4>(); spread_lane_attr<5>(); spread_lane_attr<6>(); spread_lane_attr<7>(); spread_lane_attr<8>();
    spread_lane_attr<9>(); spread_lane_attr<10>(); spread_lane_attr<11>(); spread_lane_attr<12>();
    // stamp weights q*Mx*My*Mz are below max|q| in magnitude (cardinal
    // B-spline values are < 1); the integer scale keeps them below 2^31
    double qmax = 1.0;
    for (double q : h->h_az) qmax = std::max(qmax, std::fabs(q));
    // The mixed spread sums up to kSpreadItem stamps per tile point in int32:
    // the scale keeps kSpreadItem * max|q| * (max B-spline value)^3 below 2^31.
    double mmax = 0.0;
    {
        std::vector<double> v(h->order), d(h->order);
        int km;
        mg_host_bspline(h->order, 0.5 * h->order + 0.5, &km, v.data(), d.data());
        for (double x : v) mmax = std::max(mmax, x);
        mg_host_bspline(h->order, 0.5 * h->order, &km, v.data(), d.data());
        for (double x : v) mmax = std::max(mmax, x);
    }
    double bound = kSpreadItem * qmax * mmax * mmax * mmax * 1.01;
    int k = 30;
    while (k > 4 && std::ldexp(bound, k) >= 2147483648.0 * 0.99) --k;
    h->fx_shift = k;
    // fused spread: its per-plane scale bounds point sums with mmax
    h->spl_mmax = mmax;
    // FP64 form: the whole mesh sums in 64 bits; no point can hold more than
    // np * max|q| * (max B-spline value)^3
    double bound64 = (double)h->np * qmax * mmax * mmax * mmax * 1.01;
    int k64 = 52;
    while (k64 > 20 && std::ldexp(bound64, k64) >= 9.2e18 * 0.5) --k64;
    h->fx_shift64 = k64;
    bool mixed = h->form == MG_MIXED;
    size_t n3 = (size_t)n * n * n, nc = (size_t)h->nh * n * n, no = (size_t)h->nh * h->nh * h->nh;
    std::vector<double> mf, ew, vw;
    mg_host_spme_tables(n, h->order, h->boxlen, h->TwoPiBoxi, h->vol, h->ualpha, mf, ew, vw);
    // twiddles exp(-2 pi i m / n), long double on the host
    std::vector<double2> tw(n);
    std::vector<float2> twf(n);
    for (int m = 0; m < n; ++m) {
        long double ang = -2.0L * 3.14159265358979323846264338327950288L * m / n;
        tw[m] = make_double2((double)cosl(ang), (double)sinl(ang));
        twf[m] = make_float2((float)cosl(ang), (float)sinl(ang));
    }
    if (mixed) {
        MG_CUDA(h, cudaMalloc(&h->d_Q, sizeof(float) * n3));
        MG_CUDA(h, cudaMalloc(&h->d_F, sizeof(float2) * nc));
        std::vector<float> a(no), b(no), c(no);
        for (size_t i = 0; i < no; ++i) { a[i] = (float)mf[i]; b[i] = (float)ew[i]; c[i] = (float)vw[i]; }
        MG_CUDA(h, cudaMalloc(&h->d_mf_f, sizeof(float) * no));
        MG_CUDA(h, cudaMalloc(&h->d_ew_f, sizeof(float) * no));
        MG_CUDA(h, cudaMalloc(&h->d_vw_f, sizeof(float) * no));
        MG_CUDA(h, cudaMemcpy(h->d_mf_f, a.data(), sizeof(float) * no, cudaMemcpyHostToDevice));
        MG_CUDA(h, cudaMemcpy(h->d_ew_f, b.data(), sizeof(float) * no, cudaMemcpyHostToDevice));
        MG_CUDA(h, cudaMemcpy(h->d_vw_f, c.data(), sizeof(float) * no, cudaMemcpyHostToDevice));
        MG_CUDA(h, cudaMalloc(&h->d_tw, sizeof(float2) * n));
        MG_CUDA(h, cudaMemcpy(h->d_tw, twf.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
        set_smem_limits<float>();
    } else {
        MG_CUDA(h, cudaMalloc(&h->d_Q, sizeof(double) * n3));
        MG_CUDA(h, cudaMalloc(&h->d_F, sizeof(double2) * nc));
        MG_CUDA(h, cudaMalloc(&h->d_tw, sizeof(double2) * n));
        MG_CUDA(h, cudaMemcpy(h->d_tw, tw.data(), sizeof(double2) * n, cudaMemcpyHostToDevice));
        set_smem_limits<double>();
    }
    MG_CUDA(h, cudaMalloc(&h->d_mf, sizeof(double) * no));
    MG_CUDA(h, cudaMalloc(&h->d_ew, sizeof(double) * no));
    MG_CUDA(h, cudaMalloc(&h->d_vw, sizeof(double) * no));
    MG_CUDA(h, cudaMemcpy(h->d_mf, mf.data(), sizeof(double) * no, cudaMemcpyHostToDevice));
    MG_CUDA(h, cudaMemcpy(h->d_ew, ew.data(), sizeof(double) * no, cudaMemcpyHostToDevice));
    MG_CUDA(h, cudaMemcpy(h->d_vw, vw.data(), sizeof(double) * no, cudaMemcpyHostToDevice));
    return MG_OK;
}

double mg_spme_fx_scale(const mg_handle *h) {
    return std::ldexp(1.0, h->form == MG_MIXED ? h->fx_shift : h->fx_shift64);
}

// The fixed-point charge mesh (d_Qfx) -> forward FFT, energy and virial
// partial sums, influence function, inverse FFT -> potential mesh in d_Q
// (the derivative of the reciprocal energy by the mesh charges).  d_Qfx is
// cleared for the next spread.
int mg_spme_potential(mg_handle *h) {
    ConvArgs cv;
    cv.part = h->d_part + h->part_rec;
    if (h->form == MG_MIXED) {
        cv.mf = h->d_mf_f;
        cv.ew = h->d_ew_f;
        cv.vw = h->d_vw_f;
        return fft_launch<float>(h, (float *)h->d_Q, (float2 *)h->d_F, (const float2 *)h->d_tw, cv,
                                 (float)(1.0 / mg_spme_fx_scale(h)));
    }
    cv.mf = h->d_mf;
    cv.ew = h->d_ew;
    cv.vw = h->d_vw;
    return fft_launch<double>(h, (double *)h->d_Q, (double2 *)h->d_F, (const double2 *)h->d_tw, cv,
                              1.0 / mg_spme_fx_scale(h));
}

// the reciprocal part of UDipoleEwald, SPME (FP64 form): device arrays az
// (charges), dip, pot, est, efg of the handle's particles (the last three
// added to); vir[np] the per-particle
// dipole terms of the virial, then the FFT blocks' (energy, virial) partial
// pairs, vir[np + 2 b + 1] summing to SPMFFTRec's virloc (nblk_rec blocks).  The fixed-point scale is
// chosen for the generalized charges: no mesh point can exceed np (max|q| +
// 3 max|dkdr . dip|) with B-spline values and derivatives at most 1.
int mg_spme_dipole(mg_handle *h, const double *az, const double *dip, double bound, double *pot, double *est,
                   double *efg, double *vir) {
    if (h->form != MG_FP64) return mg_fail(h, MG_ERR_UNSUPPORTED, "dipole electrostatics need the FP64 form");
    int k = 52;
    while (k > 8 && std::ldexp(bound, k) >= 9.2e18 * 0.5) --k;
    double scale = std::ldexp(1.0, k);
    DipMeshArgs a;
    a.ro = h->d_ro;
    a.az = az;
    a.dip = dip;
    a.np = h->np;
    a.order = h->order;
    a.n = h->nmesh;
    for (int m = 0; m < 3; ++m) a.dkdr[m] = h->dkdr[m];
    // the FFT pass that read the last mesh cleared it; clear again in case
    // a spread was left unconsumed
    MG_CUDA(h, cudaMemsetAsync(h->d_Qfx, 0, sizeof(long long) * (size_t)a.n * a.n * a.n, h->st));
    k_dip_spread<<<(a.np + 127) / 128, 128, 0, h->st>>>(a, scale, (unsigned long long *)h->d_Qfx);
    ConvArgs cv;
    cv.part = h->d_part + h->part_rec;
    cv.mf = h->d_mf;
    cv.ew = h->d_ew;
    cv.vw = h->d_vw;
    MG_TRY(fft_launch<double>(h, (double *)h->d_Q, (double2 *)h->d_F, (const double2 *)h->d_tw, cv, 1.0 / scale));
    k_dip_gather<<<(a.np * 32 + 127) / 128, 128, 0, h->st>>>(a, (const double *)h->d_Q, pot, est, efg, vir);
    // the FFT blocks' (energy, virial) partial pairs after the per-particle terms
    MG_CUDA(h, cudaMemcpyAsync(vir + a.np, h->d_part + h->part_rec, sizeof(double) * 2 * h->nblk_rec,
                               cudaMemcpyDeviceToDevice, h->st));
    h->launches += 2;
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

// The device FFT on a given mesh, for checking it against another FFT: the
// FP64 mesh q (n^3, x fastest) is loaded as the spread would leave it, the
// form's forward transform, the multiplier `mult` (the place of meshfac) and
// the inverse transform run as in UTotal, and phi = c2r(mult * r2c(q))
// (unnormalised, FFTW's conventions) and esum = sum of ew |r2c(q)|^2 over the
// half spectrum come back.  mult and ew are octant tables [fz][fy][kx] of
// (n/2+1)^3 values, looked up at fz = min(kz, n-kz), fy = min(ky, n-ky).
// The handle's meshes are overwritten (the next UTotal rebuilds them).
int mg_spme_fft_check(mg_handle *h, const double *q, const double *mult, const double *ew, double *phi,
                      double *esum) {
    const int n = h->nmesh, nh = h->nh;
    const size_t n3 = (size_t)n * n * n, o3 = (size_t)nh * nh * nh;
    const bool mixed = h->form == MG_MIXED;
    const size_t esz = mixed ? sizeof(float) : sizeof(double);
    double *d_q = nullptr;
    void *d_tab = nullptr;
    std::vector<unsigned char> tab(3 * o3 * esz, 0);   // mult, ew, vw = 0
    for (size_t i = 0; i < o3; ++i) {
        if (mixed) {
            ((float *)tab.data())[i] = (float)mult[i];
            ((float *)tab.data())[o3 + i] = (float)ew[i];
        } else {
            ((double *)tab.data())[i] = mult[i];
            ((double *)tab.data())[o3 + i] = ew[i];
        }
    }
    int st = MG_OK;
    std::vector<double> part(2 * (size_t)h->nblk_rec);
    cudaError_t ce = cudaMalloc(&d_q, sizeof(double) * n3);
    if (ce == cudaSuccess) ce = cudaMalloc(&d_tab, tab.size());
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_q, q, sizeof(double) * n3, cudaMemcpyHostToDevice, h->st);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_tab, tab.data(), tab.size(), cudaMemcpyHostToDevice, h->st);
    if (ce == cudaSuccess) {
        st = mg_spme_load_mesh(h, d_q);
        ConvArgs cv;
        cv.part = h->d_part + h->part_rec;
        cv.mf = d_tab;
        cv.ew = (const unsigned char *)d_tab + o3 * esz;
        cv.vw = (const unsigned char *)d_tab + 2 * o3 * esz;
        if (st == MG_OK) {
            st = mixed ? fft_launch<float>(h, (float *)h->d_Q, (float2 *)h->d_F, (const float2 *)h->d_tw, cv,
                                           (float)(1.0 / mg_spme_fx_scale(h)))
                       : fft_launch<double>(h, (double *)h->d_Q, (double2 *)h->d_F, (const double2 *)h->d_tw,
                                            cv, 1.0 / mg_spme_fx_scale(h));
        }
        if (st == MG_OK) st = mg_spme_mesh_to_f64(h, d_q, 1.0);
        if (st == MG_OK) {
            ce = cudaMemcpyAsync(phi, d_q, sizeof(double) * n3, cudaMemcpyDeviceToHost, h->st);
            if (ce == cudaSuccess)
                ce = cudaMemcpyAsync(part.data(), h->d_part + h->part_rec, sizeof(double) * part.size(),
                                     cudaMemcpyDeviceToHost, h->st);
            if (ce == cudaSuccess) ce = cudaStreamSynchronize(h->st);
        }
    }
    if (d_q) cudaFree(d_q);
    if (d_tab) cudaFree(d_tab);
    if (st != MG_OK) return st;
    if (ce != cudaSuccess) return mg_fail(h, MG_ERR_CUDA, "fft check: %s", cudaGetErrorString(ce));
    double e = 0.0;
    for (int b = 0; b < h->nblk_rec; ++b) e += part[2 * b];
    *esum = e;
    return MG_OK;
}

// FP64 charge mesh -> the fixed-point mesh the FFT reads
int mg_spme_load_mesh(mg_handle *h, const double *q) {
    size_t n3 = (size_t)h->nmesh * h->nmesh * h->nmesh;
    k_f64_to_fx<<<(unsigned)((n3 + 255) / 256), 256, 0, h->st>>>(q, (long long *)h->d_Qfx, n3, mg_spme_fx_scale(h));
    h->launches++;
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

// potential mesh d_Q (mesh type) -> FP64 copy scaled by mul
int mg_spme_mesh_to_f64(mg_handle *h, double *out, double mul) {
    size_t n3 = (size_t)h->nmesh * h->nmesh * h->nmesh;
    unsigned g = (unsigned)((n3 + 255) / 256);
    if (h->form == MG_MIXED) k_mesh_to_f64<float><<<g, 256, 0, h->st>>>((const float *)h->d_Q, out, n3, mul);
    else k_mesh_to_f64<double><<<g, 256, 0, h->st>>>((const double *)h->d_Q, out, n3, mul);
    h->launches++;
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

static void spme_args(mg_handle *h, SplineArgs &sa, BrickArgs &bk) {
    int n = h->nmesh;
    sa.ro = h->d_ro;
    sa.az = h->d_az;
    sa.perm = nullptr;
    sa.np = h->np;
    sa.order = h->order;
    sa.n = n;
    sa.n_log = ilog2(n);
    for (int m = 0; m < 3; ++m) sa.dkdr[m] = h->dkdr[m];
    sa.lB = ilog2(h->brick);
    sa.lnb = ilog2(h->nbrick_edge);
    sa.plane = 0;
    sa.nosort = h->gen_mesh;
    sa.count = h->d_brick_count;
    sa.rank = h->d_brick_rank;
    sa.brick = h->d_brick_of;
    sa.assign = h->par_forces ? 1 : 0;
    sa.final_ = h->par_final ? 1 : 0;
    sa.ffx2 = h->d_ffx2;
    sa.force2 = h->d_force2;
    sa.forceo = h->d_forceo;
    sa.fac = h->force_fac;
    bk.n = n;
    bk.B = h->brick;
    bk.nb = h->nbrick_edge;
    bk.ln = ilog2(n);
    bk.lB = ilog2(h->brick);
    bk.lnb = ilog2(h->nbrick_edge);
    bk.fx_scale = std::ldexp(1.0f, h->fx_shift);
    bk.fx_inv = std::ldexp(1.0f, -h->fx_shift);
    bk.fx_scale64 = std::ldexp(1.0, h->fx_shift64);
    bk.tile = h->brick + h->order - 1;
    bk.nbricks = h->nbricks;
    bk.count = h->d_brick_count;
    bk.perm = h->d_brick_perm;
    bk.rank = h->d_brick_rank;
    bk.brick = h->d_brick_of;
    bk.start = h->d_brick_start;
    bk.M = h->spread_m;
    bk.istart = h->d_brick_istart;
    bk.item_brick = h->d_item_brick;
}

// splines, brick sort and spread: the charge mesh in d_Qfx
static int spme_spread(mg_handle *h, const SplineArgs &sa, const BrickArgs &bk) {
    int np = h->np, tb = 256, gb = (np + tb - 1) / tb;
    bool mixed = h->form == MG_MIXED;
    MG_TRY(mg_phase_begin(h, "splines"));
    if (mixed) MG_TRY((mesh_kernel<float, int>(h, 0, sa, bk)));
    else MG_TRY((mesh_kernel<double, long long>(h, 0, sa, bk)));
    MG_TRY(mg_phase_end(h, "splines"));
    if (!h->gen_mesh) {
        MG_TRY(mg_phase_begin(h, "brick_sort"));
        mg_launch_pdl(k_brick_prefix, 1, 1024, 0, h->st, bk);   // the counts come from the spline kernel
        mg_launch_pdl(k_brick_scatter, gb, tb, 0, h->st, np, bk);
        h->launches += 2;
        MG_TRY(mg_phase_end(h, "brick_sort"));
    }
    MG_TRY(mg_phase_begin(h, "spread"));
    if (mixed) MG_TRY((mesh_kernel<float, int>(h, 1, sa, bk)));
    else MG_TRY((mesh_kernel<double, long long>(h, 1, sa, bk)));
    MG_TRY(mg_phase_end(h, "spread"));
    return MG_OK;
}

// d(E_rec)/deps_ab for an affine strain of the box (positions strained with
// it, so the mesh charges do not change): sum over the half spectrum of
// |F|^2 ew(k) (-delta_ab + 2 m_a m_b (1/(4 alpha^2) + 1/m^2)), the
// derivative of meshfac = 4 pi/V exp(-m^2/4alpha^2)/m^2 b2 by the strain
// (m -> (1 - eps^T) m, V -> (1 + tr eps) V), with the signed wave vector m
// of the spectrum entry (ky, kz above n/2 are negative); components xx, yy,
// zz, xy, xz, yz.
template <typename T>
__global__ void __launch_bounds__(256) k_box_grad(const V2<T> *__restrict__ F, const T *__restrict__ ew, int n,
                                                  double3 tpbi, double ia2, double *__restrict__ part) {
    __shared__ double red[6][8];
    int nh = n / 2 + 1;
    size_t total = (size_t)nh * n * n;
    double g[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        int kx = (int)(e % nh), ky = (int)((e / nh) % n), kz = (int)(e / ((size_t)nh * n));
        int fy = min(ky, n - ky), fz = min(kz, n - kz);
        if (kx == 0 && fy == 0 && fz == 0) continue;
        double w = (double)ew[((size_t)fz * nh + fy) * nh + kx];
        if (w == 0.0) continue;
        V2<T> f = F[e];
        double p2 = (double)f.x * f.x + (double)f.y * f.y;
        double mx = kx * tpbi.x, my = (ky <= n / 2 ? ky : ky - n) * tpbi.y, mz = (kz <= n / 2 ? kz : kz - n) * tpbi.z;
        double c = ia2 + 1.0 / (mx * mx + my * my + mz * mz), pw = p2 * w;
        g[0] += pw * (-1.0 + 2.0 * mx * mx * c);
        g[1] += pw * (-1.0 + 2.0 * my * my * c);
        g[2] += pw * (-1.0 + 2.0 * mz * mz * c);
        g[3] += pw * (2.0 * mx * my * c);
        g[4] += pw * (2.0 * mx * mz * c);
        g[5] += pw * (2.0 * my * mz * c);
    }
    int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    for (int v = 0; v < 6; ++v) {
        double x = g[v];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[v][wp] = x;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double x = 0.0;
        for (int k = 0; k < 8; ++k) x += red[threadIdx.x][k];
        part[6 * blockIdx.x + threadIdx.x] = x;
    }
}

__global__ void k_sum6(const double *__restrict__ part, int nblk, double *__restrict__ out) {
    if (threadIdx.x >= 6) return;
    double x = 0.0;
    for (int b = 0; b < nblk; ++b) x += part[6 * b + threadIdx.x];
    out[threadIdx.x] = x;
}

template <typename T> static int box_grad_t(mg_handle *h, double *out6, double *scratch, int nblk) {
    int n = h->nmesh, nh = h->nh;
    FftPlan pl = make_plan(n);
    int lp = n % 4 == 0 ? 4 : 1;
    size_t vsz = sizeof(V2<T>);
    size_t smx = vsz * (n + 2 * (size_t)lp * n);
    int thx = max(32, min(1024, lp * n / 4));
    int gx = n * n / (2 * lp);
    size_t smc = vsz * (n + 2 * (size_t)h->fft_tx * n);
    int thc = max(32, min(1024, ((h->fft_tx * n / 4) + 31) / 32 * 32));
    dim3 gc(h->fft_tiles, n);
    ConvArgs cv = {};
    V2<T> *F = (V2<T> *)h->d_F;
    const V2<T> *tw = (const V2<T> *)h->d_tw;
    FastDiv fnh = make_fastdiv((unsigned)nh), ftx = make_fastdiv((unsigned)h->fft_tx);
    k_fft_x_r2c<T><<<gx, thx, smx, h->st>>>((const long long *)h->d_Qfx, (T)(1.0 / mg_spme_fx_scale(h)), F, n,
                                            pl, lp, tw, fnh);
    MG_CUDA(h, cudaMemsetAsync(h->d_Qfx, 0, sizeof(long long) * (size_t)n * n * n, h->st));
    k_fft_col<T, false><<<gc, thc, smc, h->st>>>(F, n, pl, nh, h->fft_tx, nh, (size_t)n * nh, -1, tw, cv, ftx);
    k_fft_col<T, false><<<gc, thc, smc, h->st>>>(F, n, pl, nh, h->fft_tx, (size_t)n * nh, nh, -1, tw, cv, ftx);
    const T *ew = (const T *)(h->form == MG_MIXED ? (const void *)h->d_ew_f : (const void *)h->d_ew);
    double3 tpbi = make_double3(h->TwoPiBoxi[0], h->TwoPiBoxi[1], h->TwoPiBoxi[2]);
    k_box_grad<T><<<nblk, 256, 0, h->st>>>(F, ew, n, tpbi, 1.0 / (4.0 * h->ualpha * h->ualpha), scratch);
    k_sum6<<<1, 32, 0, h->st>>>(scratch, nblk, out6);
    h->launches += 6;
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

// d(E_rec)/deps (before EpsiFourPi; xx, yy, zz, xy, xz, yz) into the device
// array out6; scratch holds 6 * 304 doubles
int mg_spme_box_grad(mg_handle *h, double *out6, double *scratch) {
    SplineArgs sa;
    BrickArgs bk;
    spme_args(h, sa, bk);
    MG_TRY(spme_spread(h, sa, bk));
    if (h->form == MG_MIXED) return box_grad_t<float>(h, out6, scratch, 304);
    return box_grad_t<double>(h, out6, scratch, 304);
}

// UTotal's mesh part with the spread fused into the forward plane pass:
// splines and the plane sort, spread + forward, z + influence function,
// inverse, gather.
static int spme_fused(mg_handle *h, SplineArgs sa, BrickArgs bk) {
    int np = h->np, n = h->nmesh, tb = 256, gb = (np + tb - 1) / tb;
    sa.plane = 1;
    // the records in the cell order of the last list build: the gather walks
    // the particles in that order for the locality of its mesh reads, and
    // reads the records in order too
    sa.perm = h->d_perm;
    bk.nbricks = n;          // one bucket per z plane
    bk.M = 1 << 30;          // one (unused) work item per bucket
    MG_TRY(mg_phase_begin(h, "splines"));
    MG_TRY((mesh_kernel<float, int>(h, 0, sa, bk)));
    MG_TRY(mg_phase_end(h, "splines"));
    MG_TRY(mg_phase_begin(h, "plane_sort"));
    const float *w = (const float *)h->d_spl_w;
    switch (h->order) {
    case 4: mg_launch_pdl(k_plane_scatter<4>, gb, tb, 0, h->st, np, bk, w, h->d_spl_plane); break;
    case 5: mg_launch_pdl(k_plane_scatter<5>, gb, tb, 0, h->st, np, bk, w, h->d_spl_plane); break;
    case 6: mg_launch_pdl(k_plane_scatter<6>, gb, tb, 0, h->st, np, bk, w, h->d_spl_plane); break;
    case 7: mg_launch_pdl(k_plane_scatter<7>, gb, tb, 0, h->st, np, bk, w, h->d_spl_plane); break;
    default: mg_launch_pdl(k_plane_scatter<8>, gb, tb, 0, h->st, np, bk, w, h->d_spl_plane); break;
    }
    h->launches += 1;
    MG_TRY(mg_phase_end(h, "plane_sort"));
    PlaneArgs pa;
    pa.start = h->d_brick_start;
    pa.count = h->d_brick_count;
    pa.srec = h->d_spl_plane;
    pa.mmax2 = (float)(h->spl_mmax * h->spl_mmax);
    pa.err = h->d_err;
    int st;
    switch (n) {
    case 32: st = fused_passes<1>(h, pa); break;
    case 64: st = fused_passes<2>(h, pa); break;
    case 128: st = fused_passes<4>(h, pa); break;
    default: st = mg_fail(h, MG_ERR_UNSUPPORTED, "fused plane passes for nmesh = %d", n);
    }
    MG_TRY(st);
    if (h->par_forces) MG_CUDA(h, cudaStreamWaitEvent(h->st, h->ev_sr, 0));   // the short-range forces
    MG_TRY(mg_phase_begin(h, "gather"));
    MG_TRY((mesh_kernel<float, int>(h, 2, sa, bk)));
    MG_TRY(mg_phase_end(h, "gather"));
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

int mg_spme_launch(mg_handle *h) {
    int n = h->nmesh;
    size_t n3 = (size_t)n * n * n;
    SplineArgs sa;
    BrickArgs bk;
    spme_args(h, sa, bk);
    if (h->plane_fused && !h->d_Qref) return spme_fused(h, sa, bk);
    bool mixed = h->form == MG_MIXED;
    MG_TRY(spme_spread(h, sa, bk));
    if (h->d_Qref) {   // MC: keep the charge mesh of the accepted state in FP64
        k_fx_to_f64<<<(unsigned)((n3 + 255) / 256), 256, 0, h->st>>>((const long long *)h->d_Qfx, h->d_Qref, n3,
                                                                    1.0 / mg_spme_fx_scale(h));
        h->launches++;
    }
    MG_TRY(mg_spme_potential(h));
    if (h->par_forces) MG_CUDA(h, cudaStreamWaitEvent(h->st, h->ev_sr, 0));   // the short-range forces
    MG_TRY(mg_phase_begin(h, "gather"));
    if (mixed) MG_TRY((mesh_kernel<float, int>(h, 2, sa, bk)));
    else MG_TRY((mesh_kernel<double, long long>(h, 2, sa, bk)));
    MG_TRY(mg_phase_end(h, "gather"));
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}
