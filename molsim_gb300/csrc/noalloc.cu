// noalloc.cu — standard Ewald reciprocal sum with no device allocation.
//
// Some callers cannot call cudaMalloc: a host code that has handed all of its
// device memory to its own pool allocator, a code that must not block the
// device in the middle of its step (cudaMalloc and cudaFree may synchronise
// the whole device), or a caller with device pointers but no licence to
// create library state (no mg_create handle, whose set-up allocates).  For
// them, mg_ewald_rec_std_noalloc computes the same quantity as the
// reciprocal part of mg_utotal for a standard Ewald system (energy.F90
// UEwaldRecStd + UEwaldSelf, no surface term) from caller-owned device
// buffers.  Its one piece of working memory -- the four structure factors
// and the energy and virial terms of every k-vector -- lives in a fixed,
// file-scope device array instead of an allocation.
//
// The array is sized for ncut <= MG_NOALLOC_MAX_NCUT (a cube of (ncut+1)^3
// k-vector slots); every GPU that loads this library holds it (about 1.2 MB)
// until the process exits.  Every call shares it: two calls whose kernels
// overlap on the GPU (different streams, or different host threads) race on
// it and give wrong results.  Each call writes every slot before reading it,
// so nothing has to start at zero.
//
// Kernels, in stream order:
//   k_na_sk      one block per k-vector of the cube: S(k) for the four sign
//                combinations, kfac |S|^2 and its virial -> scratch slot
//   k_na_force   one thread per particle: force += the k-sum, S from scratch
//   k_na_reduce  one block: fixed-order sums of the slots and of q^2 ->
//                uout = {EpsiFourPi (Urec + Uself), EpsiFourPi Virrec}
// e^{i k.r} comes from sincos of the full phase rather than the reference's
// recurrence over n; the two agree to rounding.
#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "mg_internal.cuh"

namespace {

constexpr int kNaMaxNcut = MG_NOALLOC_MAX_NCUT;
constexpr int kNaSlots = (kNaMaxNcut + 1) * (kNaMaxNcut + 1) * (kNaMaxNcut + 1);
constexpr int kNaSlotWords = 5;   // S for the four sign combinations, then (energy, virial)
constexpr int kNaMaxDevices = 64;

// The working memory.  Host code must not pass this name to a kernel: on the
// host it is only a stand-in symbol, not a device address.  The address comes
// from cudaGetSymbolAddress, once per device (scratch_address below).
static __device__ __align__(256) double2 g_na_scratch[(size_t)kNaSlots * kNaSlotWords];

std::mutex g_na_mutex;
double2 *g_na_addr[kNaMaxDevices] = {};

struct NaArgs {
    int np, ncut, ncut2, nside;
    double3 tpbi;       // 2 pi / boxlen
    double fac0;        // 2 pi / volume
    double ualpha2;
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// k-vector of slot s: nx fastest; false for n = 0 and outside the region
__device__ __forceinline__ bool slot_k(const NaArgs &a, int s, int &nx, int &ny, int &nz) {
    nx = s % a.nside;
    ny = (s / a.nside) % a.nside;
    nz = s / (a.nside * a.nside);
    if (nx == 0 && ny == 0 && nz == 0) return false;
    return nx * nx + ny * ny + nz * nz <= a.ncut2;
}

// energy factor of one k-vector (energy.F90:6765-6782 weights 1/2 on nx = 0
// and ny = 0, 2 on nz > 0 for the half-space sum)
__device__ __forceinline__ double slot_kfac(const NaArgs &a, int nx, int ny, int nz, double &k2) {
    double kx = nx * a.tpbi.x, ky = ny * a.tpbi.y, kz = nz * a.tpbi.z;
    k2 = kx * kx + ky * ky + kz * kz;
    double f = a.fac0 * (nz == 0 ? 1.0 : 2.0) * (ny == 0 ? 0.5 : 1.0) * (nx == 0 ? 0.5 : 1.0);
    return f * exp(-k2 / (4.0 * a.ualpha2)) / k2;
}

// q e^{i(+-kx x +-ky y + kz z)} in the order (-,-), (-,+), (+,-), (+,+) of
// (x sign, y sign) used by the structure factors (energy.F90:1056-1061)
__device__ __forceinline__ void phase4(const NaArgs &a, const double *__restrict__ ro, int p, int nx,
                                       int ny, int nz, double q, double2 *er) {
    double sx, cx, sy, cy, sz, cz;
    sincos(nx * a.tpbi.x * ro[3 * p + 0], &sx, &cx);
    sincos(ny * a.tpbi.y * ro[3 * p + 1], &sy, &cy);
    sincos(nz * a.tpbi.z * ro[3 * p + 2], &sz, &cz);
    double2 ey = make_double2(cy, sy), ez = make_double2(cz, sz);
    double2 yzm = cmul(make_double2(cy, -sy), ez), yzp = cmul(ey, ez);
    double2 qxc = make_double2(q * cx, -(q * sx)), qx = make_double2(q * cx, q * sx);
    er[0] = cmul(qxc, yzm);
    er[1] = cmul(qxc, yzp);
    er[2] = cmul(qx, yzm);
    er[3] = cmul(qx, yzp);
}

__global__ void __launch_bounds__(256) k_na_sk(NaArgs a, const double *__restrict__ ro,
                                               const double *__restrict__ az,
                                               double2 *__restrict__ scratch) {
    __shared__ double sh[8][8];
    int s = blockIdx.x, nx, ny, nz;
    double2 *slot = scratch + (size_t)s * kNaSlotWords;
    if (!slot_k(a, s, nx, ny, nz)) {   // unused slot: zeros, read by nobody but written all the same
        if (threadIdx.x < kNaSlotWords) slot[threadIdx.x] = make_double2(0.0, 0.0);
        return;
    }
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int p = threadIdx.x; p < a.np; p += blockDim.x) {
        double2 er[4];
        phase4(a, ro, p, nx, ny, nz, az[p], er);
        for (int c = 0; c < 4; ++c) { acc[2 * c] += er[c].x; acc[2 * c + 1] += er[c].y; }
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int v = 0; v < 8; ++v) {
        double x = acc[v];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sh[v][w] = x;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    int nw = blockDim.x >> 5;
    double term = 0.0;
    for (int c = 0; c < 4; ++c) {
        double re = 0.0, im = 0.0;
        for (int q = 0; q < nw; ++q) { re += sh[2 * c][q]; im += sh[2 * c + 1][q]; }
        slot[c] = make_double2(re, im);
        term = term + (re * re + im * im);
    }
    double k2;
    term = slot_kfac(a, nx, ny, nz, k2) * term;
    slot[4] = make_double2(term, -(1.0 - k2 / (2.0 * a.ualpha2)) * term);
}

__global__ void __launch_bounds__(128) k_na_force(NaArgs a, const double *__restrict__ ro,
                                                  const double *__restrict__ az, double efp,
                                                  const double2 *__restrict__ scratch,
                                                  double *__restrict__ force) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.np) return;
    double q = az[p], f0 = 0.0, f1 = 0.0, f2 = 0.0;
    int nslot = a.nside * a.nside * a.nside;
    for (int s = 0; s < nslot; ++s) {
        int nx, ny, nz;
        if (!slot_k(a, s, nx, ny, nz)) continue;
        const double2 *S = scratch + (size_t)s * kNaSlotWords;
        double2 er[4];
        phase4(a, ro, p, nx, ny, nz, q, er);
        double fmm = -er[0].x * S[0].y + er[0].y * S[0].x;
        double fmp = -er[1].x * S[1].y + er[1].y * S[1].x;
        double fpm = -er[2].x * S[2].y + er[2].y * S[2].x;
        double fpp = -er[3].x * S[3].y + er[3].y * S[3].x;
        double k2;
        double kfac2 = efp * 2.0 * slot_kfac(a, nx, ny, nz, k2);
        f0 += kfac2 * nx * a.tpbi.x * (-fmm - fmp + fpm + fpp);
        f1 += kfac2 * ny * a.tpbi.y * (-fmm + fmp - fpm + fpp);
        f2 += kfac2 * nz * a.tpbi.z * (+fmm + fmp + fpm + fpp);
    }
    force[3 * p + 0] += f0;
    force[3 * p + 1] += f1;
    force[3 * p + 2] += f2;
}

__global__ void __launch_bounds__(256) k_na_reduce(NaArgs a, const double *__restrict__ az,
                                                   double ualpha, double efp,
                                                   const double2 *__restrict__ scratch,
                                                   double *__restrict__ uout) {
    __shared__ double sh[3][8];
    int nslot = a.nside * a.nside * a.nside;
    double e = 0.0, v = 0.0, q2 = 0.0;
    for (int s = threadIdx.x; s < nslot; s += blockDim.x) {
        double2 ev = scratch[(size_t)s * kNaSlotWords + 4];
        e += ev.x;
        v += ev.y;
    }
    for (int p = threadIdx.x; p < a.np; p += blockDim.x) q2 += az[p] * az[p];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        e += __shfl_down_sync(0xffffffffu, e, o);
        v += __shfl_down_sync(0xffffffffu, v, o);
        q2 += __shfl_down_sync(0xffffffffu, q2, o);
    }
    if (lane == 0) { sh[0][w] = e; sh[1][w] = v; sh[2][w] = q2; }
    __syncthreads();
    if (threadIdx.x != 0) return;
    double se = 0.0, sv = 0.0, sq = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { se += sh[0][k]; sv += sh[1][k]; sq += sh[2][k]; }
    double uself = -((ualpha / sqrt(3.1415926535897932)) * sq);   // UEwaldSelf
    uout[0] = efp * (se + uself);
    uout[1] = efp * sv;
}

int na_fail(char *err, size_t err_len, int code, const char *fmt, ...) {
    if (err && err_len) {
        va_list ap;
        va_start(ap, fmt);
        std::vsnprintf(err, err_len, fmt, ap);
        va_end(ap);
    }
    return code;
}

// Device address of the scratch array on the current device.  A call made
// outside stream capture looks it up again (cheap), so that a device reset
// between calls, after which the library's module and its array are loaded
// anew, cannot leave a stale address behind; a call made while `s` is being
// captured uses the address kept by the last call outside capture.
int scratch_address(cudaStream_t s, double2 **out, char *err, size_t err_len) {
    int dev = -1;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess)
        return na_fail(err, err_len, MG_ERR_CUDA, "cudaGetDevice failed: %s", cudaGetErrorString(ce));
    if (dev < 0 || dev >= kNaMaxDevices)
        return na_fail(err, err_len, MG_ERR_UNSUPPORTED, "device ordinal %d is beyond the %d supported",
                       dev, kNaMaxDevices);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
        cudaGetLastError();   // cannot tell: treat the call as one under capture
        cs = cudaStreamCaptureStatusActive;
    }
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (cs == cudaStreamCaptureStatusNone || !g_na_addr[dev]) {
        void *p = nullptr;
        ce = cudaGetSymbolAddress(&p, g_na_scratch);
        if (ce != cudaSuccess || !p)
            return na_fail(err, err_len, MG_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed: %s",
                           cudaGetErrorString(ce));
        g_na_addr[dev] = static_cast<double2 *>(p);
    }
    *out = g_na_addr[dev];
    return MG_OK;
}

}  // namespace

extern "C" int mg_ewald_rec_std_noalloc(int32_t np, const double *d_ro, const double *d_az,
                                        const double boxlen[3], double ualpha, int32_t ncut,
                                        int32_t ncutregion_cube, double epsi_four_pi, double *d_force,
                                        double *d_uout, void *stream, char *err, size_t err_len) {
    if (err && err_len) err[0] = '\0';
    if (np < 1 || !d_ro || !d_az || !boxlen || !d_force || !d_uout)
        return na_fail(err, err_len, MG_ERR_ARG, "np must be >= 1 and every buffer non-NULL");
    if (!(boxlen[0] > 0.0 && boxlen[1] > 0.0 && boxlen[2] > 0.0) || !(ualpha > 0.0))
        return na_fail(err, err_len, MG_ERR_ARG, "box lengths and alpha must be positive");
    if (ncut < 1)
        return na_fail(err, err_len, MG_ERR_ARG, "ncut = %d: must be >= 1", ncut);
    if (ncut > kNaMaxNcut)
        return na_fail(err, err_len, MG_ERR_ARG,
                       "ncut = %d exceeds the %d that the fixed scratch array of %zu bytes holds",
                       ncut, kNaMaxNcut, sizeof(g_na_scratch));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double2 *scratch = nullptr;
    int st = scratch_address(s, &scratch, err, err_len);
    if (st != MG_OK) return st;

    const double tp = 2.0 * 3.1415926535897932;
    NaArgs a;
    a.np = np;
    a.ncut = ncut;
    a.ncut2 = ncutregion_cube ? 3 * ncut * ncut : ncut * ncut;
    a.nside = ncut + 1;
    a.tpbi = make_double3(tp / boxlen[0], tp / boxlen[1], tp / boxlen[2]);
    a.fac0 = tp / (boxlen[0] * boxlen[1] * boxlen[2]);
    a.ualpha2 = ualpha * ualpha;
    int nslot = a.nside * a.nside * a.nside;
    k_na_sk<<<nslot, 256, 0, s>>>(a, d_ro, d_az, scratch);
    k_na_force<<<(np + 127) / 128, 128, 0, s>>>(a, d_ro, d_az, epsi_four_pi, scratch, d_force);
    k_na_reduce<<<1, 256, 0, s>>>(a, d_az, ualpha, epsi_four_pi, scratch, d_uout);
    cudaError_t ce = cudaGetLastError();
    if (ce != cudaSuccess)
        return na_fail(err, err_len, MG_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(ce));
    return MG_OK;
}
