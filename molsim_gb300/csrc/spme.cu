// spme.cu — smooth particle-mesh Ewald on the device (rows A10-A12).
//
// Reference: UEwaldRecSPM (energy.F90:1207-1297), SPMFFTRec (energy.F90:6525-
// 6587), CardinalBSpline (mollib.F90:1629-1685), EwaldSetup's SPM branch
// (energy.F90:6855-7018).  The reference calls FFTW's r2c/c2r 3D plans; this
// file has its own FFT.
//
// Pipeline per UTotal (mesh Q[z][y][x], half spectrum F[z][y][kx], kx<=n/2):
//   spread   B-spline stamp of every charge into Q (FP64 atomics, or 64-bit
//            fixed point in the mixed form, which makes the mesh and
//            everything after it bit-reproducible)
//   x pass   r2c along x; two real lines are packed into one complex line
//   y pass   complex FFT along y, tiles of TX consecutive kx columns
//   z pass   complex FFT along z, then the influence function (energy, virial,
//            multiply by meshfac) and the inverse z FFT while the column is
//            still in shared memory
//   y pass   inverse; x pass c2r inverse (FFTW's unnormalised convention)
//   gather   force from the potential mesh with separable B-spline sums
// The FFTs are radix-4 Stockham (one radix-2 stage when log2 n is odd) in
// shared memory; twiddles come from a host table computed in long double.
#include <cmath>

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

// Stockham FFT of nl lines of length n = 2^logn held in shared memory.  Element
// (line c, index t) is at buf[c*cs + t*ts].  LINE_MAJOR (ts == 1): threads run
// along t; otherwise (cs == 1) threads run along c.  Returns the buffer that
// holds the result.  sign = -1 forward, +1 backward (unnormalised).
template <typename T, bool LINE_MAJOR>
__device__ V2<T> *smem_fft(V2<T> *A, V2<T> *B, int n, int logn, int nl, int cs, int ts, int sign,
                           const V2<T> *__restrict__ tw) {
    typedef V2<T> V;
    V *in = A, *out = B;
    int tid = threadIdx.x, nthr = blockDim.x;
    int Ns = 1;
    if (logn & 1) {
        int nb = n >> 1;
        for (int b = tid; b < nl * nb; b += nthr) {
            int c = LINE_MAJOR ? b / nb : b % nl;
            int j = LINE_MAJOR ? b % nb : b / nl;
            V v0 = in[c * cs + j * ts], v1 = in[c * cs + (j + nb) * ts];
            out[c * cs + (2 * j) * ts] = cadd(v0, v1);
            out[c * cs + (2 * j + 1) * ts] = csub(v0, v1);
        }
        __syncthreads();
        V *t = in; in = out; out = t;
        Ns = 2;
    }
    int nq = n >> 2;
    while (Ns < n) {
        int stride = n / (4 * Ns);
        for (int b = tid; b < nl * nq; b += nthr) {
            int c = LINE_MAJOR ? b / nq : b % nl;
            int j = LINE_MAJOR ? b % nq : b / nl;
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
    }
    return in;
}

template <typename T>
__device__ __forceinline__ void load_tw(V2<T> *s_tw, const V2<T> *__restrict__ tw, int n) {
    for (int m = threadIdx.x; m < n; m += blockDim.x) s_tw[m] = tw[m];
}

// ---- x pass: r2c, two real lines per complex line ---------------------------
template <typename T>
__global__ void k_fft_x_r2c(const T *__restrict__ Q, V2<T> *__restrict__ F, int n, int logn,
                            int lp, const V2<T> *__restrict__ tw) {
    typedef V2<T> V;
    extern __shared__ unsigned char smem_raw[];
    V *s_tw = reinterpret_cast<V *>(smem_raw);
    V *A = s_tw + n, *B = A + lp * n;
    int nh = n / 2 + 1;
    load_tw<T>(s_tw, tw, n);
    size_t line0 = (size_t)blockIdx.x * 2 * lp;
    for (int e = threadIdx.x; e < lp * n; e += blockDim.x) {
        int c = e / n, t = e % n;
        V v;
        v.x = Q[(line0 + 2 * c) * n + t];
        v.y = Q[(line0 + 2 * c + 1) * n + t];
        A[c * n + t] = v;
    }
    __syncthreads();
    V *Z = smem_fft<T, true>(A, B, n, logn, lp, n, 1, -1, s_tw);
    for (int e = threadIdx.x; e < lp * nh; e += blockDim.x) {
        int c = e / nh, k = e % nh;
        V z = Z[c * n + k], zc = Z[c * n + ((n - k) & (n - 1))];
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
__global__ void k_fft_x_c2r(const V2<T> *__restrict__ F, T *__restrict__ Q, int n, int logn,
                            int lp, const V2<T> *__restrict__ tw) {
    typedef V2<T> V;
    extern __shared__ unsigned char smem_raw[];
    V *s_tw = reinterpret_cast<V *>(smem_raw);
    V *A = s_tw + n, *B = A + lp * n;
    int nh = n / 2 + 1;
    load_tw<T>(s_tw, tw, n);
    size_t line0 = (size_t)blockIdx.x * 2 * lp;
    for (int e = threadIdx.x; e < lp * n; e += blockDim.x) {
        int c = e / n, k = e % n;
        int kk = (k < nh) ? k : n - k;
        V a = F[(line0 + 2 * c) * nh + kk], b = F[(line0 + 2 * c + 1) * nh + kk];
        if (kk == 0 || kk == n / 2) { a.y = (T)0; b.y = (T)0; }
        if (k >= nh) { a.y = -a.y; b.y = -b.y; }
        V z;
        z.x = a.x - b.y;
        z.y = a.y + b.x;
        A[c * n + k] = z;
    }
    __syncthreads();
    V *Z = smem_fft<T, true>(A, B, n, logn, lp, n, 1, +1, s_tw);
    for (int e = threadIdx.x; e < lp * n; e += blockDim.x) {
        int c = e / n, t = e % n;
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
__global__ void k_fft_col(V2<T> *__restrict__ F, int n, int logn, int nh, int tx, size_t tstride,
                          size_t ostride, int sign, const V2<T> *__restrict__ tw, ConvArgs cv) {
    typedef V2<T> V;
    extern __shared__ unsigned char smem_raw[];
    __shared__ double red[2 * 32];
    V *s_tw = reinterpret_cast<V *>(smem_raw);
    V *A = s_tw + n, *B = A + tx * n;
    load_tw<T>(s_tw, tw, n);
    int kx0 = blockIdx.x * tx;
    size_t base = (size_t)blockIdx.y * ostride;
    for (int e = threadIdx.x; e < tx * n; e += blockDim.x) {
        int t = e / tx, c = e % tx;
        int kx = kx0 + c;
        V v;
        v.x = (T)0;
        v.y = (T)0;
        if (kx < nh) v = F[base + t * tstride + kx];
        A[t * tx + c] = v;
    }
    __syncthreads();
    V *R = smem_fft<T, false>(A, B, n, logn, tx, 1, tx, sign, s_tw);
    if (CONV) {
        const T *mf = (const T *)cv.mf, *ew = (const T *)cv.ew, *vw = (const T *)cv.vw;
        int ky = blockIdx.y;
        int fy = min(ky, n - ky);
        double e_acc = 0.0, v_acc = 0.0;
        for (int e = threadIdx.x; e < tx * n; e += blockDim.x) {
            int t = e / tx, c = e % tx;
            int kx = kx0 + c;
            if (kx >= nh) continue;
            int fz = min(t, n - t);
            size_t id = ((size_t)fz * nh + fy) * nh + kx;
            V f = R[t * tx + c];
            T p2 = f.x * f.x + f.y * f.y;
            e_acc += (double)(p2 * ew[id]);
            v_acc -= (double)(p2 * vw[id]);
            T m = mf[id];
            f.x *= m;
            f.y *= m;
            R[t * tx + c] = f;
        }
        int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
        for (int o = 16; o > 0; o >>= 1) {
            e_acc += __shfl_down_sync(0xffffffffu, e_acc, o);
            v_acc += __shfl_down_sync(0xffffffffu, v_acc, o);
        }
        if (lane == 0) { red[w] = e_acc; red[32 + w] = v_acc; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double se = 0.0, sv = 0.0;
            for (int k = 0; k < nw; ++k) { se += red[k]; sv += red[32 + k]; }
            size_t blk = (size_t)blockIdx.y * gridDim.x + blockIdx.x;
            cv.part[2 * blk] = se;
            cv.part[2 * blk + 1] = sv;
        }
        V *other = (R == A) ? B : A;
        R = smem_fft<T, false>(R, other, n, logn, tx, 1, tx, +1, s_tw);
    }
    for (int e = threadIdx.x; e < tx * n; e += blockDim.x) {
        int t = e / tx, c = e % tx;
        int kx = kx0 + c;
        if (kx < nh) F[base + t * tstride + kx] = R[t * tx + c];
    }
}

// ---- B-spline (CardinalBSpline, mollib.F90:1629-1685) -----------------------
template <typename T>
__device__ __forceinline__ int bspline(int order, T pos_frac, int kmax_in, T *v, T *dv) {
    T x = pos_frac;
    T last[MG_MAX_ORDER];
    v[0] = x;
    v[1] = (T)1 - x;
    for (int i = 2; i < order; ++i) v[i] = (T)0;
    for (int i = 0; i < order; ++i) last[i] = (T)0;
    for (int nn = 3; nn <= order; ++nn) {
        for (int i = 0; i < nn - 1; ++i) last[i] = v[i];
        T inv = (T)1 / (T)(nn - 1);
        v[0] = x * last[0] * inv;
        for (int i = 1; i <= nn - 2; ++i) {
            T a = (T)i + x;
            v[i] = (a * last[i] + ((T)nn - a) * last[i - 1]) * inv;
        }
        v[nn - 1] = ((T)1 - x) * last[nn - 2] * inv;
    }
    dv[0] = last[0];
    for (int i = 1; i <= order - 2; ++i) dv[i] = last[i] - last[i - 1];
    dv[order - 1] = -last[order - 2];
    return kmax_in;
}

struct SplineArgs {
    const double *ro, *az;
    int np, order, n;
    double dkdr[3];
};

// stamp origin and spline weights of particle p in dimension m
template <typename T>
__device__ __forceinline__ int particle_spline(const SplineArgs &a, int p, int m, T *v, T *dv) {
    double pos = a.dkdr[m] * a.ro[3 * p + m];
    double fl = floor(pos);
    int kmax = (int)fl;
    T x = (T)(pos - fl);
    bspline<T>(a.order, x, kmax, v, dv);
    int mm = kmax % a.n;
    return mm < 0 ? mm + a.n : mm;
}

__global__ void k_spread_f64(SplineArgs a, double *__restrict__ Q) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.np) return;
    double v[3][MG_MAX_ORDER], dv[MG_MAX_ORDER];
    int mm[3];
    for (int m = 0; m < 3; ++m) mm[m] = particle_spline<double>(a, p, m, v[m], dv);
    int n = a.n, o = a.order;
    double q = a.az[p];
    for (int iz = 0; iz < o; ++iz) {
        int nz = mm[2] - iz;
        nz += (nz < 0) ? n : 0;
        double qz = q * v[2][iz];
        for (int iy = 0; iy < o; ++iy) {
            int ny = mm[1] - iy;
            ny += (ny < 0) ? n : 0;
            double qyz = qz * v[1][iy];
            double *row = Q + ((size_t)nz * n + ny) * n;
            for (int ix = 0; ix < o; ++ix) {
                int nx = mm[0] - ix;
                nx += (nx < 0) ? n : 0;
                atomicAdd(row + nx, qyz * v[0][ix]);
            }
        }
    }
}

__global__ void k_spread_fx(SplineArgs a, unsigned long long *__restrict__ Q) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.np) return;
    float v[3][MG_MAX_ORDER], dv[MG_MAX_ORDER];
    int mm[3];
    for (int m = 0; m < 3; ++m) mm[m] = particle_spline<float>(a, p, m, v[m], dv);
    int n = a.n, o = a.order;
    float q = (float)a.az[p];
    for (int iz = 0; iz < o; ++iz) {
        int nz = mm[2] - iz;
        nz += (nz < 0) ? n : 0;
        float qz = q * v[2][iz];
        for (int iy = 0; iy < o; ++iy) {
            int ny = mm[1] - iy;
            ny += (ny < 0) ? n : 0;
            float qyz = qz * v[1][iy];
            unsigned long long *row = Q + ((size_t)nz * n + ny) * n;
            for (int ix = 0; ix < o; ++ix) {
                int nx = mm[0] - ix;
                nx += (nx < 0) ? n : 0;
                long long fx = __float2ll_rn(qyz * v[0][ix] * 4294967296.0f);
                atomicAdd(row + nx, (unsigned long long)fx);
            }
        }
    }
}

// fixed-point mesh -> float mesh, clearing the accumulator for the next call
__global__ void k_fx_to_float(unsigned long long *__restrict__ Qfx, float *__restrict__ Q, size_t n3) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n3) return;
    long long v = (long long)Qfx[i];
    Q[i] = (float)((double)v * MG_FX_INV);
    Qfx[i] = 0ull;
}

// gather: esum = sum dM*M*M*phi over the stamp (energy.F90:1255-1285),
// evaluated as separable row sums; force -= q*esum*dkdr*EpsiFourPi
template <typename T, bool MIXED>
__global__ void k_gather(SplineArgs a, const T *__restrict__ Q, double efp,
                         double *__restrict__ force, long long *__restrict__ ffx) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.np) return;
    T v[3][MG_MAX_ORDER], d[3][MG_MAX_ORDER];
    int mm[3];
    for (int m = 0; m < 3; ++m) mm[m] = particle_spline<T>(a, p, m, v[m], d[m]);
    int n = a.n, o = a.order;
    int xs[MG_MAX_ORDER];
    for (int ix = 0; ix < o; ++ix) {
        int nx = mm[0] - ix;
        xs[ix] = nx + ((nx < 0) ? n : 0);
    }
    T e0 = 0, e1 = 0, e2 = 0;
    for (int iz = 0; iz < o; ++iz) {
        int nz = mm[2] - iz;
        nz += (nz < 0) ? n : 0;
        T e0z = 0, e1z = 0, e2z = 0;
        for (int iy = 0; iy < o; ++iy) {
            int ny = mm[1] - iy;
            ny += (ny < 0) ? n : 0;
            const T *row = Q + ((size_t)nz * n + ny) * n;
            T sx = 0, s0 = 0;
            for (int ix = 0; ix < o; ++ix) {
                T q = row[xs[ix]];
                sx += d[0][ix] * q;
                s0 += v[0][ix] * q;
            }
            e0z += v[1][iy] * sx;
            e1z += d[1][iy] * s0;
            e2z += v[1][iy] * s0;
        }
        e0 += v[2][iz] * e0z;
        e1 += v[2][iz] * e1z;
        e2 += d[2][iz] * e2z;
    }
    double q = a.az[p];
    double f0 = -q * (double)e0 * a.dkdr[0] * efp;
    double f1 = -q * (double)e1 * a.dkdr[1] * efp;
    double f2 = -q * (double)e2 * a.dkdr[2] * efp;
    if (MIXED) {
        ffx[3 * p + 0] += __double2ll_rn(f0 * MG_FX_SCALE);
        ffx[3 * p + 1] += __double2ll_rn(f1 * MG_FX_SCALE);
        ffx[3 * p + 2] += __double2ll_rn(f2 * MG_FX_SCALE);
    } else {
        force[3 * p + 0] += f0;
        force[3 * p + 1] += f1;
        force[3 * p + 2] += f2;
    }
}

int ilog2(int n) {
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}

template <typename T>
int fft_launch(mg_handle *h, T *Q, V2<T> *F, const V2<T> *tw, ConvArgs cv) {
    int n = h->nmesh, logn = ilog2(n), nh = h->nh;
    int lp = 4;                                  // line pairs per CTA in the x passes
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
    k_fft_x_r2c<T><<<gx, thx, smx, h->st>>>(Q, F, n, logn, lp, tw);
    MG_TRY(mg_phase_end(h, "fft_x_r2c"));
    MG_TRY(mg_phase_begin(h, "fft_y_fwd"));
    k_fft_col<T, false><<<gc, thc, smc, h->st>>>(F, n, logn, nh, h->fft_tx, ystride, yother, -1, tw, cv);
    MG_TRY(mg_phase_end(h, "fft_y_fwd"));
    MG_TRY(mg_phase_begin(h, "fft_z_conv"));
    k_fft_col<T, true><<<gc, thc, smc, h->st>>>(F, n, logn, nh, h->fft_tx, zstride, zother, -1, tw, cv);
    MG_TRY(mg_phase_end(h, "fft_z_conv"));
    MG_TRY(mg_phase_begin(h, "fft_y_inv"));
    k_fft_col<T, false><<<gc, thc, smc, h->st>>>(F, n, logn, nh, h->fft_tx, ystride, yother, +1, tw, cv);
    MG_TRY(mg_phase_end(h, "fft_y_inv"));
    MG_TRY(mg_phase_begin(h, "fft_x_c2r"));
    k_fft_x_c2r<T><<<gx, thx, smx, h->st>>>(F, Q, n, logn, lp, tw);
    MG_TRY(mg_phase_end(h, "fft_x_c2r"));
    h->launches += 5;
    return MG_OK;
}

template <typename T> void set_smem_limits() {
    cudaFuncSetAttribute(k_fft_x_r2c<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_fft_x_c2r<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_fft_col<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_fft_col<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

}  // namespace

int mg_spme_init(mg_handle *h) {
    int n = h->nmesh;
    if (n < 8 || (n & (n - 1)) != 0)
        return mg_fail(h, MG_ERR_UNSUPPORTED, "nmesh = %d: the device FFT supports powers of two >= 8", n);
    if (n > 512) return mg_fail(h, MG_ERR_UNSUPPORTED, "nmesh = %d > 512", n);
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
        MG_CUDA(h, cudaMalloc(&h->d_Qfx, sizeof(unsigned long long) * n3));
        MG_CUDA(h, cudaMemsetAsync(h->d_Qfx, 0, sizeof(unsigned long long) * n3, h->st));
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

int mg_spme_launch(mg_handle *h) {
    int n = h->nmesh, np = h->np;
    size_t n3 = (size_t)n * n * n;
    SplineArgs sa;
    sa.ro = h->d_ro;
    sa.az = h->d_az;
    sa.np = np;
    sa.order = h->order;
    sa.n = n;
    for (int m = 0; m < 3; ++m) sa.dkdr[m] = h->dkdr[m];
    ConvArgs cv;
    cv.part = h->d_part + h->part_rec;
    int tb = 128, gb = (np + tb - 1) / tb;
    if (h->form == MG_MIXED) {
        MG_TRY(mg_phase_begin(h, "spread"));
        k_spread_fx<<<gb, tb, 0, h->st>>>(sa, h->d_Qfx);
        MG_TRY(mg_phase_end(h, "spread"));
        MG_TRY(mg_phase_begin(h, "mesh_convert"));
        k_fx_to_float<<<(unsigned)((n3 + 255) / 256), 256, 0, h->st>>>(h->d_Qfx, (float *)h->d_Q, n3);
        MG_TRY(mg_phase_end(h, "mesh_convert"));
        h->launches += 2;
        cv.mf = h->d_mf_f;
        cv.ew = h->d_ew_f;
        cv.vw = h->d_vw_f;
        MG_TRY(fft_launch<float>(h, (float *)h->d_Q, (float2 *)h->d_F, (const float2 *)h->d_tw, cv));
        MG_TRY(mg_phase_begin(h, "gather"));
        k_gather<float, true><<<gb, tb, 0, h->st>>>(sa, (const float *)h->d_Q, h->EpsiFourPi,
                                                    h->d_force, h->d_ffx);
        h->launches++;
        MG_TRY(mg_phase_end(h, "gather"));
    } else {
        MG_TRY(mg_phase_begin(h, "mesh_clear"));
        MG_CUDA(h, cudaMemsetAsync(h->d_Q, 0, sizeof(double) * n3, h->st));
        MG_TRY(mg_phase_end(h, "mesh_clear"));
        MG_TRY(mg_phase_begin(h, "spread"));
        k_spread_f64<<<gb, tb, 0, h->st>>>(sa, (double *)h->d_Q);
        h->launches++;
        MG_TRY(mg_phase_end(h, "spread"));
        cv.mf = h->d_mf;
        cv.ew = h->d_ew;
        cv.vw = h->d_vw;
        MG_TRY(fft_launch<double>(h, (double *)h->d_Q, (double2 *)h->d_F, (const double2 *)h->d_tw, cv));
        MG_TRY(mg_phase_begin(h, "gather"));
        k_gather<double, false><<<gb, tb, 0, h->st>>>(sa, (const double *)h->d_Q, h->EpsiFourPi,
                                                      h->d_force, h->d_ffx);
        h->launches++;
        MG_TRY(mg_phase_end(h, "gather"));
    }
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}
