// forces.cu — UTotal on the device (rows A6, A7, A9, A15 and UBond).
//
// Reference: UTotal (energy.F90:280-430), UTwoBodyA / UTwoBodyACellList
// (energy.F90:445-544, 669-777), UEwaldSelf / UEwaldSurf (energy.F90:1301-
// 1371), UBond (energy.F90:5335-5386).
//
// Pair kernel: one thread per cell-sorted slot walks its full Verlet list and
// owns the force of its particle, so no atomics are needed and the result does
// not depend on scheduling.  The table interval is found by binary search over
// the descending lower ends z_low (the same interval the reference's linear
// search from iubuflow stops at, because z_low strictly decreases); r^2 is
// formed without FMA so cutoff, hard-core and interval decisions match the
// reference bit for bit.  Energies and virial go to per-block partial sums that
// one reduction kernel adds in a fixed order (deterministic).
//
// Mixed form: the cutoff decision stays FP64; table arithmetic is FP32 and each
// particle's force is stored as 64-bit fixed point (scale 2^32).
#include <algorithm>

#include "mg_internal.cuh"

namespace {

constexpr int kPairThreads = 128;
constexpr int kThreads = 256;
// bonds: the chain beads come first in the particle order, so small blocks
// spread their FP64 bond work over many SMs
constexpr int kBondThreads = 64;

// block reduction of nv doubles per thread into out[0..nv) (thread 0 writes)
template <int BS>
__device__ void block_sum(double *vals, int nv, double *out, double *sh) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    constexpr int NW = BS / 32;
    for (int v = 0; v < nv; ++v) {
        double x = vals[v];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sh[v * NW + w] = x;
    }
    __syncthreads();
    if (threadIdx.x < nv) {
        double s = 0.0;
        for (int k = 0; k < NW; ++k) s += sh[threadIdx.x * NW + k];
        out[threadIdx.x] = s;
    }
}

__global__ void k_prepare(const double *__restrict__ ro, const int *__restrict__ perm,
                          const int *__restrict__ type, int np, double4 *__restrict__ pos_s) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= np) return;
    int p = perm[s];
    pos_s[s] = make_double4(ro[3 * p], ro[3 * p + 1], ro[3 * p + 2], (double)type[p]);
}

// mixed form: FP32 offset from the centre of the particle's cell (the cell
// of the last list build) and the cell's coordinates packed in 10-bit
// fields, so pair distances need no FP64 arithmetic
struct CellGeom {
    int nc[3];
    double size[3], half[3];
    float sizef[3], lenf[3], halff[3];
};

__global__ void k_prepare_f32(const double *__restrict__ ro, const int *__restrict__ perm,
                              const int *__restrict__ type, const int *__restrict__ cellof, int np,
                              CellGeom g, float4 *__restrict__ pos_f, int *__restrict__ cell_s) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= np) return;
    int p = perm[s];
    int c = cellof[p];
    int cx = c % g.nc[0], cy = (c / g.nc[0]) % g.nc[1], cz = c / (g.nc[0] * g.nc[1]);
    // offsets wrapped to the nearest image, so a particle that crossed the
    // box since the list build keeps a small offset
    double d[3];
    int cc[3] = {cx, cy, cz};
    for (int m = 0; m < 3; ++m) {
        d[m] = ro[3 * p + m] - ((cc[m] + 0.5) * g.size[m] - g.half[m]);
        if (fabs(d[m]) > g.half[m]) d[m] -= copysign(2.0 * g.half[m], d[m]);
    }
    float ox = (float)d[0], oy = (float)d[1], oz = (float)d[2];
    pos_f[s] = make_float4(ox, oy, oz, __int_as_float(type[p]));
    cell_s[s] = cx | (cy << 10) | (cz << 20);
}

struct PairArgs {
    const double4 *pos_s;
    const int *perm, *nnb, *nbr;
    int np, npt, nptpt, nrec, nbins;
    const int *pairidx;          // [npt*npt] 1-based, column-major
    const double *zlow;          // [nrec] lower end (r^2) of every table interval
    const double *coef;          // [nrec*11] FP64 coefficients (usum 6, fsum 5)
    const float *coef_f;         // [nrec*11] FP32 coefficients (mixed form)
    const int *tab_start, *tab_n;
    const double *r2umin, *r2atat, *bin_z0, *bin_inv;
    const unsigned short *bin_kstart;   // [nptpt*nbins] first interval to scan from
    int tab_in_smem;             // coefficient table staged in shared memory
    mg_box box;
    double rcut2;
    int cellcut;                 // 1: r2 < rcut2 (cell list), 0: r2 <= rcut2 (Verlet list)
    double *force;
    long long *ffx;
    double *part;
    int *err;
};

// shared-memory image of the small per-pair data and (optionally) the table
struct PairShared {
    int *pairidx, *start, *n;
    double *r2atat, *r2umin, *z0, *inv, *zlow;
    unsigned short *kstart;
    void *coef;
    double *u;   // per-thread energy slots [nptpt][blockDim]
};

template <bool MIXED>
__host__ __device__ size_t pair_smem_layout(const PairArgs &a, unsigned char *base, PairShared &s, int nthr) {
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t r = o;
        o = (o + bytes + 15) & ~(size_t)15;
        return base ? (void *)(base + r) : nullptr;
    };
    s.r2atat = (double *)take(sizeof(double) * a.nptpt);
    s.r2umin = (double *)take(sizeof(double) * a.nptpt);
    s.z0 = (double *)take(sizeof(double) * a.nptpt);
    s.inv = (double *)take(sizeof(double) * a.nptpt);
    s.u = (double *)take(sizeof(double) * a.nptpt * nthr);
    s.zlow = (double *)take(sizeof(double) * a.nrec);
    s.pairidx = (int *)take(sizeof(int) * a.npt * a.npt);
    s.start = (int *)take(sizeof(int) * a.nptpt);
    s.n = (int *)take(sizeof(int) * a.nptpt);
    s.kstart = (unsigned short *)take(sizeof(unsigned short) * a.nptpt * a.nbins);
    s.coef = a.tab_in_smem ? take((MIXED ? sizeof(float) : sizeof(double)) * 11 * a.nrec) : nullptr;
    return o;
}

// table interval containing r2 (first k with zlow(k) <= r2, as the reference's
// linear search from iubuflow finds it): start from the bin's first
// candidate and step forward; exact by construction of kstart
__device__ __forceinline__ int find_interval(const PairShared &s, int pair, double r2, int nbins) {
    int b = (int)((r2 - s.z0[pair]) * s.inv[pair]);
    b = min(max(b, 0), nbins - 1);
    int k = s.kstart[pair * nbins + b];
    int last = s.n[pair] - 1;
    const double *z = s.zlow + s.start[pair];
    while (k < last && z[k] > r2) ++k;
    return s.start[pair] + k;
}

// One pair (i, j) of the Verlet list; returns false when it is beyond rcut.
template <bool MIXED>
__device__ __forceinline__ void pair_term(const PairArgs &a, const PairShared &s, double4 pi, int ti,
                                          double4 pj, int p, int j, double &fx, double &fy, double &fz,
                                          float &gx, float &gy, float &gz, double *u, double &vir) {
    double dx = mg_pbc1(__dsub_rn(pi.x, pj.x), a.box.half[0], a.box.len[0]);
    double dy = mg_pbc1(__dsub_rn(pi.y, pj.y), a.box.half[1], a.box.len[1]);
    double dz = mg_pbc1(__dsub_rn(pi.z, pj.z), a.box.half[2], a.box.len[2]);
    double r2 = mg_r2_exact(dx, dy, dz);
    if (a.cellcut ? !(r2 < a.rcut2) : (r2 > a.rcut2)) return;
    int tj = (int)pj.w;
    int pair = s.pairidx[tj * a.npt + ti] - 1;   // iptpt(ipt,jpt) - 1
    if (r2 < s.r2atat[pair]) {
        // hard-core overlap: u = 1e10 (the cell-list routine also sets
        // fsum = 1e10; the Verlet-list routine keeps a stale value)
        u[pair * blockDim.x] += 0.5 * 1e10;
        if (MIXED) { gx += 1e10f * (float)dx; gy += 1e10f * (float)dy; gz += 1e10f * (float)dz; }
        else { fx += 1e10 * dx; fy += 1e10 * dy; fz += 1e10 * dz; }
        vir -= 0.5 * (1e10 * r2);
        return;
    }
    if (r2 < s.r2umin[pair]) {
        mg_dev_error(a.err, MG_ERR_TABLE_UNDERRUN, p + 1, a.perm[j] + 1, pair + 1);
        return;
    }
    int rec = find_interval(s, pair, r2, a.nbins);
    double d = r2 - s.zlow[rec];
    if (MIXED) {
        const float *c = a.tab_in_smem ? (const float *)s.coef + (size_t)rec * 11 : a.coef_f + (size_t)rec * 11;
        float df = (float)d;
        float us = c[0] + df * (c[1] + df * (c[2] + df * (c[3] + df * (c[4] + df * c[5]))));
        float fs = c[6] + df * (c[7] + df * (c[8] + df * (c[9] + df * c[10])));
        gx += fs * (float)dx;
        gy += fs * (float)dy;
        gz += fs * (float)dz;
        u[pair * blockDim.x] += 0.5 * (double)us;
        vir -= 0.5 * (double)fs * r2;
    } else {
        const double *c = a.tab_in_smem ? (const double *)s.coef + (size_t)rec * 11 : a.coef + (size_t)rec * 11;
        double us = c[0] + d * (c[1] + d * (c[2] + d * (c[3] + d * (c[4] + d * c[5]))));
        double fs = c[6] + d * (c[7] + d * (c[8] + d * (c[9] + d * c[10])));
        fx += fs * dx;
        fy += fs * dy;
        fz += fs * dz;
        u[pair * blockDim.x] += 0.5 * us;
        vir -= 0.5 * (fs * r2);
    }
}

// WARP: one warp per slot (dense systems); otherwise one thread per slot.
template <bool MIXED, bool WARP>
__global__ void __launch_bounds__(kPairThreads) k_pair(PairArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double red[(MG_MAX_NPTPT + 1) * (kPairThreads / 32)];
    PairShared s;
    pair_smem_layout<MIXED>(a, smem, s, blockDim.x);
    for (int k = threadIdx.x; k < a.npt * a.npt; k += blockDim.x) s.pairidx[k] = a.pairidx[k];
    for (int k = threadIdx.x; k < a.nptpt; k += blockDim.x) {
        s.r2atat[k] = a.r2atat[k];
        s.r2umin[k] = a.r2umin[k];
        s.z0[k] = a.bin_z0[k];
        s.inv[k] = a.bin_inv[k];
        s.start[k] = a.tab_start[k];
        s.n[k] = a.tab_n[k];
    }
    for (int k = threadIdx.x; k < a.nptpt * (int)blockDim.x; k += blockDim.x) s.u[k] = 0.0;
    for (int k = threadIdx.x; k < a.nrec; k += blockDim.x) s.zlow[k] = a.zlow[k];
    {
        const uint4 *src = reinterpret_cast<const uint4 *>(a.bin_kstart);
        uint4 *dst = reinterpret_cast<uint4 *>(s.kstart);
        int nv = (a.nptpt * a.nbins * 2) / 16;
        for (int k = threadIdx.x; k < nv; k += blockDim.x) dst[k] = src[k];
    }
    if (a.tab_in_smem) {
        if (MIXED) {
            float *dst = (float *)s.coef;
            for (int k = threadIdx.x; k < 11 * a.nrec; k += blockDim.x) dst[k] = a.coef_f[k];
        } else {
            double *dst = (double *)s.coef;
            for (int k = threadIdx.x; k < 11 * a.nrec; k += blockDim.x) dst[k] = a.coef[k];
        }
    }
    __syncthreads();
    double *u = s.u + threadIdx.x;
    double vir = 0.0;
    int lane = threadIdx.x & 31;
    int i = WARP ? (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5)
                 : (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i < a.np) {
        double4 pi = a.pos_s[i];
        int ti = (int)pi.w;
        int p = a.perm[i];
        double fx = 0.0, fy = 0.0, fz = 0.0;
        float gx = 0.f, gy = 0.f, gz = 0.f;
        int nn = a.nnb[i];
        int k0 = WARP ? lane : 0, ks = WARP ? 32 : 1;
        // software pipelining: the next neighbour's index and position are
        // requested before the current pair is evaluated
        int k = k0;
        int jn = (k < nn) ? a.nbr[(size_t)k * a.np + i] : 0;
        double4 pn = (k < nn) ? a.pos_s[jn] : make_double4(0, 0, 0, 0);
        for (; k < nn; k += ks) {
            int j = jn;
            double4 pj = pn;
            if (k + ks < nn) {
                jn = a.nbr[(size_t)(k + ks) * a.np + i];
                pn = a.pos_s[jn];
            }
            pair_term<MIXED>(a, s, pi, ti, pj, p, j, fx, fy, fz, gx, gy, gz, u, vir);
        }
        if (WARP) {
            for (int o = 16; o > 0; o >>= 1) {
                fx += __shfl_down_sync(0xffffffffu, fx, o);
                fy += __shfl_down_sync(0xffffffffu, fy, o);
                fz += __shfl_down_sync(0xffffffffu, fz, o);
                gx += __shfl_down_sync(0xffffffffu, gx, o);
                gy += __shfl_down_sync(0xffffffffu, gy, o);
                gz += __shfl_down_sync(0xffffffffu, gz, o);
            }
        }
        if (!WARP || lane == 0) {
            if (MIXED) {
                a.ffx[3 * p + 0] = __double2ll_rn((double)gx * MG_FX_SCALE);
                a.ffx[3 * p + 1] = __double2ll_rn((double)gy * MG_FX_SCALE);
                a.ffx[3 * p + 2] = __double2ll_rn((double)gz * MG_FX_SCALE);
            } else {
                a.force[3 * p + 0] = fx;
                a.force[3 * p + 1] = fy;
                a.force[3 * p + 2] = fz;
            }
        }
    }
    double acc[MG_MAX_NPTPT + 1];
    for (int v = 0; v < a.nptpt; ++v) acc[v] = u[v * blockDim.x];
    acc[a.nptpt] = vir;
    block_sum<kPairThreads>(acc, a.nptpt + 1, a.part + (size_t)blockIdx.x * (a.nptpt + 1), red);
}

// ---- mixed-form pair kernel: FP32 only ------------------------------------------
struct PairArgsF {
    const float4 *pos_f;
    const int *cell_s, *perm, *nnb, *nbr;
    int np, npt, nptpt, nrec, nbins;
    const int *pairidx, *tab_start, *tab_n;
    const float *zlow_f, *coef_f, *r2umin_f, *r2atat_f, *bin_z0_f, *bin_inv_f;
    const unsigned short *bin_kstart;
    int tab_in_smem;
    CellGeom g;
    float rcut2;
    int cellcut;
    long long *ffx;
    double *part;
    int *err;
};

struct PairSharedF {
    int *pairidx, *start, *n;
    float *r2atat, *r2umin, *z0, *inv, *zlow, *coef, *u;
    unsigned short *kstart;
};

__host__ __device__ size_t pair_smem_layout_f(const PairArgsF &a, unsigned char *base, PairSharedF &s, int nthr) {
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t r = o;
        o = (o + bytes + 15) & ~(size_t)15;
        return base ? (void *)(base + r) : nullptr;
    };
    s.r2atat = (float *)take(sizeof(float) * a.nptpt);
    s.r2umin = (float *)take(sizeof(float) * a.nptpt);
    s.z0 = (float *)take(sizeof(float) * a.nptpt);
    s.inv = (float *)take(sizeof(float) * a.nptpt);
    s.u = (float *)take(sizeof(float) * a.nptpt * nthr);
    s.zlow = (float *)take(sizeof(float) * a.nrec);
    s.pairidx = (int *)take(sizeof(int) * a.npt * a.npt);
    s.start = (int *)take(sizeof(int) * a.nptpt);
    s.n = (int *)take(sizeof(int) * a.nptpt);
    s.kstart = (unsigned short *)take(sizeof(unsigned short) * a.nptpt * a.nbins);
    s.coef = a.tab_in_smem ? (float *)take(sizeof(float) * 11 * a.nrec) : nullptr;
    return o;
}

__device__ __forceinline__ int wrap_cell(int d, int n) {
    int h = n >> 1;
    d += (d < -h) ? n : 0;
    d -= (d > h) ? n : 0;
    return d;
}

// A team of TEAM lanes per slot walks the slot's Verlet list with stride
// TEAM; the team's force is combined with shuffles.  Tables are read through
// the read-only path (they stay in L1); per-lane energies sit in shared slots.
template <int TEAM>
__global__ void __launch_bounds__(kPairThreads) k_pair_f32(PairArgsF a) {
    __shared__ float su[MG_MAX_NPTPT * kPairThreads];
    __shared__ double red[(MG_MAX_NPTPT + 1) * (kPairThreads / 32)];
    for (int k = threadIdx.x; k < a.nptpt * kPairThreads; k += kPairThreads) su[k] = 0.f;
    __syncthreads();
    float *u = su + threadIdx.x;
    float vir = 0.f;
    int j0 = threadIdx.x & (TEAM - 1);
    int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) / TEAM);
    float gx = 0.f, gy = 0.f, gz = 0.f;
    if (i < a.np) {
        float4 pi = __ldg(&a.pos_f[i]);
        int ci = __ldg(&a.cell_s[i]);
        int ti = __float_as_int(pi.w);
        int nn = __ldg(&a.nnb[i]);
        for (int k = j0; k < nn; k += TEAM) {
            int j = __ldg(&a.nbr[(size_t)k * a.np + i]);
            float4 pj = __ldg(&a.pos_f[j]);
            int cj = __ldg(&a.cell_s[j]);
            int dcx = wrap_cell((ci & 1023) - (cj & 1023), a.g.nc[0]);
            int dcy = wrap_cell(((ci >> 10) & 1023) - ((cj >> 10) & 1023), a.g.nc[1]);
            int dcz = wrap_cell((ci >> 20) - (cj >> 20), a.g.nc[2]);
            float dx = (float)dcx * a.g.sizef[0] + (pi.x - pj.x);
            float dy = (float)dcy * a.g.sizef[1] + (pi.y - pj.y);
            float dz = (float)dcz * a.g.sizef[2] + (pi.z - pj.z);
            if (fabsf(dx) > a.g.halff[0]) dx -= copysignf(a.g.lenf[0], dx);
            if (fabsf(dy) > a.g.halff[1]) dy -= copysignf(a.g.lenf[1], dy);
            if (fabsf(dz) > a.g.halff[2]) dz -= copysignf(a.g.lenf[2], dz);
            float r2 = dx * dx + dy * dy + dz * dz;
            if (a.cellcut ? !(r2 < a.rcut2) : (r2 > a.rcut2)) continue;
            int pair = __ldg(&a.pairidx[__float_as_int(pj.w) * a.npt + ti]) - 1;
            if (r2 < __ldg(&a.r2atat_f[pair])) {
                u[pair * kPairThreads] += 0.5e10f;
                gx += 1e10f * dx; gy += 1e10f * dy; gz += 1e10f * dz;
                vir -= 0.5e10f * r2;
                continue;
            }
            if (r2 < __ldg(&a.r2umin_f[pair])) {
                mg_dev_error(a.err, MG_ERR_TABLE_UNDERRUN, a.perm[i] + 1, a.perm[j] + 1, pair + 1);
                continue;
            }
            int b = (int)((r2 - __ldg(&a.bin_z0_f[pair])) * __ldg(&a.bin_inv_f[pair]));
            b = min(max(b, 0), a.nbins - 1);
            int start = __ldg(&a.tab_start[pair]);
            int kk = __ldg(&a.bin_kstart[pair * a.nbins + b]), last = __ldg(&a.tab_n[pair]) - 1;
            const float *z = a.zlow_f + start;
            while (kk < last && __ldg(&z[kk]) > r2) ++kk;
            int rec = start + kk;
            const float *c = a.coef_f + (size_t)rec * 11;
            float d = r2 - __ldg(&z[kk]);
            float us = __ldg(&c[0]) + d * (__ldg(&c[1]) + d * (__ldg(&c[2]) + d * (__ldg(&c[3]) + d * (__ldg(&c[4]) + d * __ldg(&c[5])))));
            float fs = __ldg(&c[6]) + d * (__ldg(&c[7]) + d * (__ldg(&c[8]) + d * (__ldg(&c[9]) + d * __ldg(&c[10]))));
            gx += fs * dx;
            gy += fs * dy;
            gz += fs * dz;
            u[pair * kPairThreads] += 0.5f * us;
            vir -= 0.5f * fs * r2;
        }
    }
    // every lane takes part (teams past np hold zeros)
#pragma unroll
    for (int o = TEAM / 2; o > 0; o >>= 1) {
        gx += __shfl_xor_sync(0xffffffffu, gx, o, TEAM);
        gy += __shfl_xor_sync(0xffffffffu, gy, o, TEAM);
        gz += __shfl_xor_sync(0xffffffffu, gz, o, TEAM);
    }
    if (i < a.np && j0 == 0) {
        int p = a.perm[i];
        a.ffx[3 * p + 0] = mg_f2fx(gx);
        a.ffx[3 * p + 1] = mg_f2fx(gy);
        a.ffx[3 * p + 2] = mg_f2fx(gz);
    }
    __syncthreads();
    // warp sums in FP32, FP64 across the block's warps
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    constexpr int NW = kPairThreads / 32;
    for (int v = 0; v <= a.nptpt; ++v) {
        float x = (v < a.nptpt) ? u[v * kPairThreads] : vir;
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[v * NW + wid] = (double)x;
    }
    __syncthreads();
    if (threadIdx.x <= a.nptpt) {
        double sum = 0.0;
        for (int k = 0; k < NW; ++k) sum += red[threadIdx.x * NW + k];
        a.part[(size_t)blockIdx.x * (a.nptpt + 1) + threadIdx.x] = sum;
    }
}

// UBond: every particle adds the forces of its (at most a few) bonds; the
// bond's first particle counts its energy and virial.
struct BondArgs {
    const double *ro;
    int np;
    // bonds: per-particle CSR (bond*2 + role), pairs, parameters
    const int *off, *list, *ij;
    const double *bk, *beq;
    const int *bp;
    // angles: per-particle CSR (angle*4 + role: 0 jm, 1 ip, 2 jp), triples, parameters
    const int *aoff, *alist, *aijk;
    const double *ak, *aeq;
    const int *ap;
    int nangle;
    mg_box box;
    double *force;
    long long *ffx;
    double *part;   // per block: u%bond, bond virial, u%angle
};

// x**n as the oracle's powi (gfortran's expansion of an integer power)
__device__ __forceinline__ double powi_d(double x, int n) {
    switch (n) {
    case 0: return 1.0;
    case 1: return x;
    case 2: return __dmul_rn(x, x);
    case 3: return __dmul_rn(__dmul_rn(x, x), x);
    case 4: { double x2 = __dmul_rn(x, x); return __dmul_rn(x2, x2); }
    default: { double r = 1.0; for (int i = 0; i < n; ++i) r = __dmul_rn(r, x); return r; }
    }
}

// PBC (molaux.F90:104-146, box): d - L*anint(d/L) when |d| > L/2
__device__ __forceinline__ double pbc_anint(double d, double half, double len, double inv) {
    if (fabs(d) > half) d = __dsub_rn(d, __dmul_rn(len, round(__dmul_rn(d, inv))));
    return d;
}

// UBond (energy.F90:5335-5400) and UAngle (energy.F90:5409-5506), one
// thread per particle: the force of every bond and angle the particle takes
// part in (its role in it), summed in a fixed order; each bond's energy and
// virial counted by its first particle, each angle's energy by its vertex.
template <bool MIXED>
__global__ void __launch_bounds__(kBondThreads) k_bond(BondArgs a) {
    __shared__ double sh[3 * (kBondThreads / 32)];
    double acc[3] = {0.0, 0.0, 0.0};
    const double *ro = a.ro;
    const mg_box &box = a.box;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < a.np) {
        double f[3] = {0.0, 0.0, 0.0};
        bool any = false;
        if (a.off) {
            for (int e = a.off[p]; e < a.off[p + 1]; ++e) {
                int b = a.list[e] >> 1, role = a.list[e] & 1;
                int ip = a.ij[2 * b], jp = a.ij[2 * b + 1];
                double dx = mg_pbc1(__dsub_rn(ro[3 * ip], ro[3 * jp]), box.half[0], box.len[0]);
                double dy = mg_pbc1(__dsub_rn(ro[3 * ip + 1], ro[3 * jp + 1]), box.half[1], box.len[1]);
                double dz = mg_pbc1(__dsub_rn(ro[3 * ip + 2], ro[3 * jp + 2]), box.half[2], box.len[2]);
                double r2 = dx * dx + dy * dy + dz * dz;
                double r1 = sqrt(r2);
                double term = r1 - a.beq[b];
                double pw = 1.0;
                for (int k = 0; k < a.bp[b] - 1; ++k) pw *= term;
                double fac = a.bk[b] * pw;
                double u = fac * term;
                fac = -a.bp[b] * fac / r1;
                double sgn = role ? -1.0 : 1.0;
                f[0] += sgn * (fac * dx);
                f[1] += sgn * (fac * dy);
                f[2] += sgn * (fac * dz);
                if (!role) {
                    acc[0] += u;
                    acc[1] -= fac * r2;
                }
                any = true;
            }
        }
        if (a.aoff) {
            for (int e = a.aoff[p]; e < a.aoff[p + 1]; ++e) {
                int an = a.alist[e] >> 2, role = a.alist[e] & 3;
                int jm = a.aijk[3 * an], ip = a.aijk[3 * an + 1], jp = a.aijk[3 * an + 2];
                double dm[3], dq[3];
#pragma unroll
                for (int m = 0; m < 3; ++m) {
                    dm[m] = pbc_anint(__dsub_rn(ro[3 * ip + m], ro[3 * jm + m]), box.half[m], box.len[m], box.inv[m]);
                    dq[m] = pbc_anint(__dsub_rn(ro[3 * ip + m], ro[3 * jp + m]), box.half[m], box.len[m], box.inv[m]);
                }
                double dmi = 1.0 / sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dm[0], dm[0]), __dmul_rn(dm[1], dm[1])),
                                                  __dmul_rn(dm[2], dm[2])));
                double dpi = 1.0 / sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dq[0], dq[0]), __dmul_rn(dq[1], dq[1])),
                                                  __dmul_rn(dq[2], dq[2])));
#pragma unroll
                for (int m = 0; m < 3; ++m) {
                    dm[m] = __dmul_rn(dm[m], dmi);
                    dq[m] = __dmul_rn(dq[m], dpi);
                }
                double cosine = __dadd_rn(__dadd_rn(__dmul_rn(dm[0], dq[0]), __dmul_rn(dm[1], dq[1])),
                                          __dmul_rn(dm[2], dq[2]));
                double theta = acos(fmax(-1.0, fmin(cosine, 1.0)));
                double term = __dsub_rn(theta, a.aeq[an]);
                double fac = __dmul_rn(a.ak[an], powi_d(term, a.ap[an] - 1));
                if (role == 1) acc[2] += __dmul_rn(fac, term);
                fac = __dmul_rn((double)(-a.ap[an]), fac) / sin(theta);
                double fm = __dmul_rn(fac, dmi), fp = __dmul_rn(fac, dpi);
#pragma unroll
                for (int m = 0; m < 3; ++m) {
                    double gm = __dmul_rn(fm, __dsub_rn(dq[m], __dmul_rn(cosine, dm[m])));   // on jm
                    double gp = __dmul_rn(fp, __dsub_rn(dm[m], __dmul_rn(cosine, dq[m])));   // on jp
                    f[m] += role == 0 ? gm : role == 2 ? gp : -__dadd_rn(gm, gp);
                }
                any = true;
            }
        }
        if (any) {
            if (MIXED) {
                for (int m = 0; m < 3; ++m) a.ffx[3 * p + m] += __double2ll_rn(f[m] * MG_FX_SCALE);
            } else {
                for (int m = 0; m < 3; ++m) a.force[3 * p + m] += f[m];
            }
        }
    }
    block_sum<kBondThreads>(acc, 3, a.part + (size_t)blockIdx.x * 3, sh);
}

// the bond/angle kernel's arguments for the handle, forces into force / ffx
static BondArgs bond_args(mg_handle *h, double *force, long long *ffx) {
    BondArgs b;
    b.ro = h->d_ro;
    b.np = h->np;
    b.off = h->nbond > 0 ? h->d_bond_off : nullptr;
    b.list = h->d_bond_list;
    b.ij = h->d_bond_ij;
    b.bk = h->d_bond_k;
    b.beq = h->d_bond_eq;
    b.bp = h->d_bond_p;
    b.aoff = h->nangle > 0 ? h->d_angle_off : nullptr;
    b.alist = h->d_angle_list;
    b.aijk = h->d_angle_ijk;
    b.ak = h->d_angle_k;
    b.aeq = h->d_angle_eq;
    b.ap = h->d_angle_p;
    b.nangle = h->nangle;
    for (int m = 0; m < 3; ++m) {
        b.box.len[m] = h->boxlen[m];
        b.box.half[m] = h->boxlen2[m];
        b.box.inv[m] = h->boxleni[m];
    }
    b.force = force;
    b.ffx = ffx;
    b.part = h->d_part + h->part_bond;
    return b;
}

// sum of az*r per block (UEwaldSurf, energy.F90:1352-1355)
__global__ void __launch_bounds__(kThreads) k_surf_sums(const double *__restrict__ ro,
                                                        const double *__restrict__ az, int np,
                                                        double *__restrict__ part) {
    __shared__ double sh[3 * (kThreads / 32)];
    double acc[3] = {0.0, 0.0, 0.0};
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < np) {
        acc[0] = az[p] * ro[3 * p];
        acc[1] = az[p] * ro[3 * p + 1];
        acc[2] = az[p] * ro[3 * p + 2];
    }
    block_sum<kThreads>(acc, 3, part + (size_t)blockIdx.x * 3, sh);
}

struct ReduceArgs {
    const double *part;
    int nptpt;
    int off[4], nblk[4];    // partial arrays: pair, reciprocal, bonds, surface
    int blk0[5];            // first stage-1 block of each array (blk0[4] = grid)
    int row0[4];            // first scratch entry of each array
    int ewald, lsurf;
    double EpsiFourPi, u_self, surf_fac;
    double *uout;
    double *rows;           // stage-1 sums, one row per block
    unsigned *ticket;       // blocks finished (zero between launches)
};

// Partial sums of the energies and virials -> the UTotal outputs.  The
// partials are four arrays of rows (pair: nptpt + 1 values per row,
// reciprocal 2, bonds 2, surface 3).  Stage 1: each block sums
// kRedThreads / stride consecutive rows of one array (one load per thread)
// into a scratch row.  Stage 2, in the block that finishes last (a ticket
// counter): the scratch rows of each array, by its own warps.  Thread t of a
// group sums the entries t, t + S, ... of its array, S a multiple of the row
// length, so that one thread always meets the same component; per-thread
// sums are combined per component by one warp.  Every sum runs in a fixed
// order.
constexpr int kRedThreads = 256;

__host__ __device__ __forceinline__ int red_stride(int g, int nv_pair) {
    return g == 0 ? nv_pair : g == 1 ? 2 : 3;   // pair, reciprocal, bond (+ angle), surface
}

// sum of component comp over the per-thread sums tsum[t0 + i], i < S
__device__ __forceinline__ double red_comp(const double *tsum, int t0, int S, int stride, int comp, int lane) {
    double sv = 0.0;
    for (int i = comp + stride * lane; i < S; i += 32 * stride) sv += tsum[t0 + i];
    for (int o = 16; o > 0; o >>= 1) sv += __shfl_down_sync(0xffffffffu, sv, o);
    return sv;
}

__global__ void __launch_bounds__(kRedThreads) k_reduce(ReduceArgs a) {
    mg_pdl_begin();
    __shared__ double tsum[kRedThreads];
    __shared__ double vals[MG_MAX_NPTPT + 1 + 2 + 3 + 3];
    __shared__ int is_last;
    int t = threadIdx.x, lane = t & 31, w = t >> 5;
    constexpr int nwarp = kRedThreads / 32;
    int nv_pair = a.nptpt + 1;
    {   // stage 1: block -> (array g, its block index within g)
        int b = blockIdx.x, g = 0;
        while (g < 3 && b >= a.blk0[g + 1]) ++g;
        int stride = red_stride(g, nv_pair), rows = kRedThreads / stride, S = rows * stride;
        const double *src = a.part + a.off[g];
        size_t r0 = (size_t)(b - a.blk0[g]) * rows, r1 = min(r0 + rows, (size_t)a.nblk[g]);
        size_t f = r0 * stride + t;
        tsum[t] = (t < S && f < r1 * stride) ? src[f] : 0.0;
        __syncthreads();
        for (int c = w; c < stride; c += nwarp) {
            double sv = red_comp(tsum, 0, S, stride, c, lane);
            if (lane == 0) a.rows[a.row0[g] + (size_t)(b - a.blk0[g]) * stride + c] = sv;
        }
    }
    __threadfence();
    __syncthreads();
    if (t == 0) is_last = atomicAdd(a.ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    // stage 2: warps 0-3 the pair rows, 4-5 reciprocal, 6 bonds, 7 surface
    const int t0s[4] = {0, 128, 192, 224}, nts[4] = {128, 64, 32, 32};
    int g = w < 4 ? 0 : w < 6 ? 1 : w < 7 ? 2 : 3;
    int stride = red_stride(g, nv_pair);
    int S = stride * (nts[g] / stride), tl = t - t0s[g];
    size_t total = (size_t)(a.blk0[g + 1] - a.blk0[g]) * stride;
    const double *src = a.rows + a.row0[g];
    double s0 = 0.0, s1 = 0.0;
    if (tl < S) {
        size_t f = tl;
        for (; f + S < total; f += 2 * (size_t)S) {
            s0 += __ldcg(src + f);
            s1 += __ldcg(src + f + S);
        }
        if (f < total) s0 += __ldcg(src + f);
    }
    tsum[t] = s0 + s1;
    __syncthreads();
    int nv = nv_pair + 2 + 3 + 3;
    for (int v = w; v < nv; v += nwarp) {
        int gv = v < nv_pair ? 0 : v < nv_pair + 2 ? 1 : v < nv_pair + 5 ? 2 : 3;
        int comp = gv == 0 ? v : gv == 1 ? v - nv_pair : gv == 2 ? v - nv_pair - 2 : v - nv_pair - 5;
        int sg = red_stride(gv, nv_pair);
        double sv = red_comp(tsum, t0s[gv], sg * (nts[gv] / sg), sg, comp, lane);
        if (lane == 0) vals[v] = sv;
    }
    if (t == 0) *a.ticket = 0u;   // for the next launch (graph replays)
    __syncthreads();
    if (threadIdx.x != 0) return;
    double *u = a.uout;
    double twob0 = 0.0;
    for (int k = 1; k <= a.nptpt; ++k) {
        u[k] = vals[k - 1];
        twob0 = twob0 + u[k];
    }
    u[0] = twob0;
    double virtwob = vals[a.nptpt];
    double urec = 0.0, virrec = 0.0;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    if (a.ewald != MG_EWALD_NONE) {
        urec = vals[nv_pair];
        virrec = vals[nv_pair + 1];
        urec = urec + a.u_self;
        if (a.lsurf) {
            sx = vals[nv_pair + 5];
            sy = vals[nv_pair + 6];
            sz = vals[nv_pair + 7];
            double term = a.surf_fac * (sx * sx + sy * sy + sz * sz);
            urec = urec + term;
            virrec = virrec - term;
        }
        urec = a.EpsiFourPi * urec;
    }
    double ubond = vals[nv_pair + 2], virbond = vals[nv_pair + 3], uangle = vals[nv_pair + 4];
    int o = a.nptpt + 1;
    u[o + 0] = twob0 + urec + ubond + uangle;                 // u%tot
    u[o + 1] = urec;                                          // u%rec
    u[o + 2] = ubond;                                         // u%bond
    u[o + 3] = virtwob + a.EpsiFourPi * virrec + virbond;     // virial (angles contribute none)
    u[o + 4] = sx;
    u[o + 5] = sy;
    u[o + 6] = sz;
    u[o + 7] = uangle;                                        // u%angle
}

// force -> forceo with the surface force and the unit factor (energy.F90:405-424)
template <bool MIXED>
__global__ void k_epilogue(const double *__restrict__ force, const double *__restrict__ force2,
                           const long long *__restrict__ ffx, const long long *__restrict__ ffx2,
                           const double *__restrict__ az,
                           const double *__restrict__ uout, int o,
                           int np, int lsurf, double surf_k, double fac,
                           double *__restrict__ forceo) {
    mg_pdl_begin();
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    for (int m = 0; m < 3; ++m) {
        double f = MIXED ? (double)(ffx[3 * p + m] + (ffx2 ? ffx2[3 * p + m] : 0ll)) * MG_FX_INV
                         : (force2 ? __dadd_rn(force[3 * p + m], force2[3 * p + m]) : force[3 * p + m]);
        if (lsurf) f = f - surf_k * az[p] * uout[o + 4 + m];
        forceo[3 * p + m] = f * fac;
    }
}

}  // namespace

// Direct-index table lookup: per type pair a uniform grid of nbins bins over
// [r2umin, max(rcut^2, z_low(1))]; kstart(bin) is the first interval whose
// lower end lies at or below the bin's upper edge (with a margin), so a
// forward scan from it stops at the reference's interval.
static int pair_tables(mg_handle *h, const double *ubuf, const int *start, const int *count) {
    int nptpt = h->nptpt;
    h->nrec = h->nbuf / 12;
    h->nbins = 1024;
    std::vector<double> zlow(h->nrec), coef(11 * (size_t)h->nrec), z0(nptpt), inv(nptpt);
    std::vector<float> coef_f(11 * (size_t)h->nrec);
    std::vector<unsigned short> kst((size_t)nptpt * h->nbins);
    for (int r = 0; r < h->nrec; ++r) {
        zlow[r] = ubuf[12 * (size_t)r];
        for (int c = 0; c < 11; ++c) {
            coef[11 * (size_t)r + c] = ubuf[12 * (size_t)r + 1 + c];
            coef_f[11 * (size_t)r + c] = (float)ubuf[12 * (size_t)r + 1 + c];
        }
    }
    for (int p = 0; p < nptpt; ++p) {
        const double *z = zlow.data() + start[p];
        int n = count[p];
        if (n > 65535) return mg_fail(h, MG_ERR_UNSUPPORTED, "table of pair %d has %d intervals", p + 1, n);
        double lo = z[n - 1], hi = std::max(h->rcut2, z[0]);
        double width = (hi - lo) / h->nbins;
        if (!(width > 0)) width = 1.0;
        z0[p] = lo;
        inv[p] = 1.0 / width;
        for (int b = 0; b < h->nbins; ++b) {
            int k = 0;
            if (b < h->nbins - 1) {
                double upper = lo + (b + 1.001) * width;
                while (k < n - 1 && z[k] > upper) ++k;
            }
            kst[(size_t)p * h->nbins + b] = (unsigned short)k;
        }
    }
    MG_CUDA(h, cudaMalloc(&h->d_zlow, sizeof(double) * h->nrec));
    MG_CUDA(h, cudaMalloc(&h->d_coef, sizeof(double) * coef.size()));
    MG_CUDA(h, cudaMalloc(&h->d_coef_f, sizeof(float) * coef_f.size()));
    MG_CUDA(h, cudaMalloc(&h->d_bin_z0, sizeof(double) * nptpt));
    MG_CUDA(h, cudaMalloc(&h->d_bin_inv, sizeof(double) * nptpt));
    MG_CUDA(h, cudaMalloc(&h->d_bin_kstart, sizeof(unsigned short) * kst.size()));
    MG_CUDA(h, cudaMemcpy(h->d_zlow, zlow.data(), sizeof(double) * h->nrec, cudaMemcpyHostToDevice));
    MG_CUDA(h, cudaMemcpy(h->d_coef, coef.data(), sizeof(double) * coef.size(), cudaMemcpyHostToDevice));
    MG_CUDA(h, cudaMemcpy(h->d_coef_f, coef_f.data(), sizeof(float) * coef_f.size(), cudaMemcpyHostToDevice));
    MG_CUDA(h, cudaMemcpy(h->d_bin_z0, z0.data(), sizeof(double) * nptpt, cudaMemcpyHostToDevice));
    MG_CUDA(h, cudaMemcpy(h->d_bin_inv, inv.data(), sizeof(double) * nptpt, cudaMemcpyHostToDevice));
    MG_CUDA(h, cudaMemcpy(h->d_bin_kstart, kst.data(), sizeof(unsigned short) * kst.size(), cudaMemcpyHostToDevice));
    {   // FP32 copies for the mixed form (interval lower ends, bins, limits)
        std::vector<float> zf(h->nrec), r2u(nptpt), r2a(nptpt), z0f(nptpt), invf(nptpt);
        for (int r = 0; r < h->nrec; ++r) zf[r] = (float)zlow[r];
        for (int p = 0; p < nptpt; ++p) {
            z0f[p] = (float)z0[p];
            invf[p] = (float)inv[p];
        }
        std::vector<double> r2u_d(nptpt), r2a_d(nptpt);
        MG_CUDA(h, cudaMemcpy(r2u_d.data(), h->d_r2umin, sizeof(double) * nptpt, cudaMemcpyDeviceToHost));
        MG_CUDA(h, cudaMemcpy(r2a_d.data(), h->d_r2atat, sizeof(double) * nptpt, cudaMemcpyDeviceToHost));
        for (int p = 0; p < nptpt; ++p) {
            r2u[p] = (float)r2u_d[p];
            r2a[p] = (float)r2a_d[p];
        }
        MG_CUDA(h, cudaMalloc(&h->d_f32_tabs, sizeof(float) * (h->nrec + 4 * nptpt)));
        float *d = h->d_f32_tabs;
        MG_CUDA(h, cudaMemcpy(d, zf.data(), sizeof(float) * h->nrec, cudaMemcpyHostToDevice));
        MG_CUDA(h, cudaMemcpy(d + h->nrec, r2u.data(), sizeof(float) * nptpt, cudaMemcpyHostToDevice));
        MG_CUDA(h, cudaMemcpy(d + h->nrec + nptpt, r2a.data(), sizeof(float) * nptpt, cudaMemcpyHostToDevice));
        MG_CUDA(h, cudaMemcpy(d + h->nrec + 2 * nptpt, z0f.data(), sizeof(float) * nptpt, cudaMemcpyHostToDevice));
        MG_CUDA(h, cudaMemcpy(d + h->nrec + 3 * nptpt, invf.data(), sizeof(float) * nptpt, cudaMemcpyHostToDevice));
    }
    // shared-memory budget: stage the coefficient table when it is small
    PairArgs a{};
    a.nptpt = nptpt;
    a.npt = h->npt;
    a.nrec = h->nrec;
    a.nbins = h->nbins;
    bool mixed = h->form == MG_MIXED;
    size_t base, full;
    if (mixed) {
        PairArgsF af{};
        af.nptpt = nptpt;
        af.npt = h->npt;
        af.nrec = h->nrec;
        af.nbins = h->nbins;
        PairSharedF sf;
        af.tab_in_smem = 0;
        base = pair_smem_layout_f(af, nullptr, sf, kPairThreads);
        af.tab_in_smem = 1;
        full = pair_smem_layout_f(af, nullptr, sf, kPairThreads);
    } else {
        PairShared s;
        a.tab_in_smem = 0;
        base = pair_smem_layout<false>(a, nullptr, s, kPairThreads);
        a.tab_in_smem = 1;
        full = pair_smem_layout<false>(a, nullptr, s, kPairThreads);
    }
    h->pair_tab_smem = (full <= 64 * 1024) ? 1 : 0;
    h->pair_smem = h->pair_tab_smem ? full : base;
    if (h->pair_smem > 200 * 1024) return mg_fail(h, MG_ERR_UNSUPPORTED, "pair tables need %zu bytes of shared memory", h->pair_smem);
    cudaFuncSetAttribute(k_pair<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_pair<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    return MG_OK;
}

int mg_forces_init(mg_handle *h, const double *ubuf, const int *start, const int *count) {
    int np = h->np;
    MG_TRY(pair_tables(h, ubuf, start, count));
    // warp per particle when the expected list is long (dense systems)
    double dens = np / h->vol, rc = h->rcut + h->drnlist;
    double expect = 4.0 / 3.0 * 3.141592653589793 * rc * rc * rc * dens;
    h->pair_warp = expect > 24.0 ? 1 : 0;
    // mixed form: a team of lanes per slot sized to the expected full list
    // (~2x the half-sphere count), so short lists still fill the GPU
    // lanes per particle: at sparse densities the per-particle latency chain
    // (list index, neighbour slot, table) dominates, and more lanes per
    // particle hide it (measured at ~2 neighbours: 1 lane 52 us, 2 lanes
    // 34 us, 4 lanes 26 us for 65 600 particles)
    h->pair_team = expect < 1.0 ? 2 : expect < 10.0 ? 4 : expect < 20.0 ? 8 : expect < 40.0 ? 16 : 32;
    int per_block = h->pair_warp ? kPairThreads / 32 : kPairThreads;
    h->nblk_pair = (np + per_block - 1) / per_block;
    if (h->form == MG_MIXED) h->nblk_pair = (int)(((long)np * h->pair_team + kPairThreads - 1) / kPairThreads);
    h->nblk_bond = (np + kBondThreads - 1) / kBondThreads;
    h->nblk_surf = (np + kThreads - 1) / kThreads;
    // rec partials: SPME z-pass blocks or std k-vectors; sized by the caller
    // of mg_forces_init (nblk_rec set before)
    h->part_pair = 0;
    h->part_rec = h->part_pair + h->nblk_pair * (h->nptpt + 1);
    h->part_bond = h->part_rec + 2 * (h->nblk_rec > 0 ? h->nblk_rec : 1);
    h->part_surf = h->part_bond + 3 * h->nblk_bond;
    // k_reduce: its stage-1 rows (at most one per partial row) and its ticket
    h->part_red = h->part_surf + 3 * h->nblk_surf;
    size_t npart = 2 * (size_t)h->part_red + 1;
    MG_CUDA(h, cudaMalloc(&h->d_part, sizeof(double) * npart));
    MG_CUDA(h, cudaMemsetAsync(h->d_part, 0, sizeof(double) * npart, h->st));
    MG_CUDA(h, cudaMalloc(&h->d_uout, sizeof(double) * (h->nptpt + 1 + 8)));
    MG_CUDA(h, cudaMemsetAsync(h->d_uout, 0, sizeof(double) * (h->nptpt + 1 + 8), h->st));
    MG_CUDA(h, cudaMalloc(&h->d_forceo, sizeof(double) * 3 * np));
    if (h->form == MG_MIXED) {
        for (int m = 0; m < 3; ++m)
            if (h->ncell[m] >= 1024) return mg_fail(h, MG_ERR_UNSUPPORTED, "more than 1023 cells per edge");
        MG_CUDA(h, cudaMalloc(&h->d_pos_f, sizeof(float4) * np));
        MG_CUDA(h, cudaMalloc(&h->d_cell_s, sizeof(int) * np));
        MG_CUDA(h, cudaMalloc(&h->d_ffx, sizeof(long long) * 3 * np));
        if (h->ewald == MG_EWALD_SPM) MG_CUDA(h, cudaMalloc(&h->d_ffx2, sizeof(long long) * 3 * np));
    } else {
        MG_CUDA(h, cudaMalloc(&h->d_force, sizeof(double) * 3 * np));
        if (h->ewald == MG_EWALD_SPM) MG_CUDA(h, cudaMalloc(&h->d_force2, sizeof(double) * 3 * np));
    }
    return MG_OK;
}

static int utotal_reduce(mg_handle *h, bool mixed, bool par);
static int utotal_epilogue(mg_handle *h, bool mixed, bool par);

// Queue one UTotal on the handle's stream.
int mg_utotal_launch(mg_handle *h) {
    int np = h->np;
    bool mixed = h->form == MG_MIXED;
    CellGeom cg;
    for (int m = 0; m < 3; ++m) {
        cg.nc[m] = h->ncell[m];
        cg.size[m] = h->cellSize[m];
        cg.half[m] = h->boxlen2[m];
        cg.sizef[m] = (float)h->cellSize[m];
        cg.lenf[m] = (float)h->boxlen[m];
        cg.halff[m] = (float)h->boxlen2[m];
    }
    // SPME (uncaptured phase timing aside): the short-range forces run on the
    // second stream into their own accumulator while the mesh path runs here
    bool par = h->ewald == MG_EWALD_SPM && (mixed ? h->d_ffx2 != nullptr : h->d_force2 != nullptr) &&
               !h->timing;
    cudaStream_t ss = h->st;
    long long *ffx_sr = h->d_ffx;
    double *force_sr = h->d_force;
    if (par) {
        MG_CUDA(h, cudaEventRecord(h->ev_fork, h->st));
        MG_CUDA(h, cudaStreamWaitEvent(h->st2, h->ev_fork, 0));
        ss = h->st2;
        ffx_sr = h->d_ffx2;
        force_sr = h->d_force2;
    }
    MG_TRY(mg_phase_begin(h, "prepare"));
    if (mixed)
        k_prepare_f32<<<(np + kThreads - 1) / kThreads, kThreads, 0, ss>>>(
            h->d_ro, h->d_perm, h->d_type, h->d_cellof, np, cg, h->d_pos_f, h->d_cell_s);
    else
        k_prepare<<<(np + kThreads - 1) / kThreads, kThreads, 0, ss>>>(h->d_ro, h->d_perm, h->d_type,
                                                                      np, h->d_pos_s);
    MG_TRY(mg_phase_end(h, "prepare"));
    MG_TRY(mg_phase_begin(h, "pair"));
    PairArgs a;
    a.pos_s = h->d_pos_s;
    a.perm = h->d_perm;
    a.nnb = h->d_nnb;
    a.nbr = h->d_nbr;
    a.np = np;
    a.npt = h->npt;
    a.nptpt = h->nptpt;
    a.nrec = h->nrec;
    a.nbins = h->nbins;
    a.pairidx = h->d_pairidx;
    a.zlow = h->d_zlow;
    a.coef = h->d_coef;
    a.coef_f = h->d_coef_f;
    a.tab_start = h->d_tab_start;
    a.tab_n = h->d_tab_n;
    a.r2umin = h->d_r2umin;
    a.r2atat = h->d_r2atat;
    a.bin_z0 = h->d_bin_z0;
    a.bin_inv = h->d_bin_inv;
    a.bin_kstart = h->d_bin_kstart;
    for (int m = 0; m < 3; ++m) {
        a.box.len[m] = h->boxlen[m];
        a.box.half[m] = h->boxlen2[m];
        a.box.inv[m] = h->boxleni[m];
    }
    a.rcut2 = h->rcut2;
    a.cellcut = (h->txintlist == MG_CELLLIST) ? 1 : 0;
    a.force = force_sr;
    a.ffx = h->d_ffx;
    a.part = h->d_part + h->part_pair;
    a.err = h->d_err;
    a.tab_in_smem = h->pair_tab_smem;
    size_t sm = h->pair_smem;
    int nb = h->nblk_pair;
    if (mixed) {
        PairArgsF f;
        f.pos_f = h->d_pos_f;
        f.cell_s = h->d_cell_s;
        f.perm = h->d_perm;
        f.nnb = h->d_nnb;
        f.nbr = h->d_nbr;
        f.np = np;
        f.npt = h->npt;
        f.nptpt = h->nptpt;
        f.nrec = h->nrec;
        f.nbins = h->nbins;
        f.pairidx = h->d_pairidx;
        f.tab_start = h->d_tab_start;
        f.tab_n = h->d_tab_n;
        f.zlow_f = h->d_f32_tabs;
        f.r2umin_f = h->d_f32_tabs + h->nrec;
        f.r2atat_f = h->d_f32_tabs + h->nrec + h->nptpt;
        f.bin_z0_f = h->d_f32_tabs + h->nrec + 2 * h->nptpt;
        f.bin_inv_f = h->d_f32_tabs + h->nrec + 3 * h->nptpt;
        f.coef_f = h->d_coef_f;
        f.bin_kstart = h->d_bin_kstart;
        f.tab_in_smem = h->pair_tab_smem;
        f.g = cg;
        f.rcut2 = (float)h->rcut2;
        f.cellcut = a.cellcut;
        f.ffx = ffx_sr;
        f.part = h->d_part + h->part_pair;
        f.err = h->d_err;
        int team = h->pair_team, nbt = (int)(((long)np * team + kPairThreads - 1) / kPairThreads);
        switch (team) {
        case 1: k_pair_f32<1><<<nbt, kPairThreads, 0, ss>>>(f); break;
        case 2: k_pair_f32<2><<<nbt, kPairThreads, 0, ss>>>(f); break;
        case 4: k_pair_f32<4><<<nbt, kPairThreads, 0, ss>>>(f); break;
        case 8: k_pair_f32<8><<<nbt, kPairThreads, 0, ss>>>(f); break;
        case 16: k_pair_f32<16><<<nbt, kPairThreads, 0, ss>>>(f); break;
        default: k_pair_f32<32><<<nbt, kPairThreads, 0, ss>>>(f); break;
        }
    } else {
        if (h->pair_warp) k_pair<false, true><<<nb, kPairThreads, sm, ss>>>(a);
        else k_pair<false, false><<<nb, kPairThreads, sm, ss>>>(a);
    }
    if (par && (h->nbond > 0 || h->nangle > 0)) {   // bonds and angles follow the pairs on the second stream
        BondArgs ba = bond_args(h, force_sr, ffx_sr);
        if (mixed) k_bond<true><<<h->nblk_bond, kBondThreads, 0, ss>>>(ba);
        else k_bond<false><<<h->nblk_bond, kBondThreads, 0, ss>>>(ba);
        h->launches++;
    }
    if (par) MG_CUDA(h, cudaEventRecord(h->ev_sr, ss));   // the short-range forces are in d_ffx2 / d_force2
    h->chk_queued = false;
    h->cand_queued = false;
    if (par && h->cand_side) {   // the next BD step's candidates (after this step's move)
        cudaStream_t keep = h->st;
        h->st = ss;
        int cst = mg_integrate_bd_cand(h);
        h->st = keep;
        MG_TRY(cst);
        h->cand_queued = true;
    }
    if (par && h->chk_side) {   // the list check overlaps the mesh path too
        cudaStream_t keep = h->st;
        h->st = ss;
        int cst = mg_lists_check(h, true);
        h->st = keep;
        MG_TRY(cst);
        h->chk_queued = true;
    }
    h->launches += 2;
    MG_TRY(mg_phase_end(h, "pair"));

    // forked: the mesh path waits for ev_sr (the short-range forces) before
    // its gather, which then writes forceo itself when there is no surface
    // term; it records ev_rec once the reciprocal energy partials are summed,
    // for the reduction on the second stream
    bool fused = par && !(h->ewald != MG_EWALD_NONE && h->lsurf);
    h->par_forces = par;
    h->par_final = fused;
    int spst = MG_OK;
    if (h->ewald == MG_EWALD_SPM) spst = mg_spme_launch(h);
    else if (h->ewald == MG_EWALD_STD) spst = mg_ewald_std_launch(h);
    h->par_forces = false;
    h->par_final = false;
    if (par && spst == MG_OK) {
        cudaError_t ce = cudaStreamWaitEvent(ss, h->ev_rec, 0);
        if (ce == cudaSuccess) {
            cudaStream_t keep = h->st;
            h->st = ss;
            spst = utotal_reduce(h, mixed, par);
            h->st = keep;
        } else {
            spst = mg_fail(h, MG_ERR_CUDA, "stream wait: %s", cudaGetErrorString(ce));
        }
    }
    if (par) {   // join before any return
        MG_CUDA(h, cudaEventRecord(h->ev_join, ss));
        MG_CUDA(h, cudaStreamWaitEvent(h->st, h->ev_join, 0));
    }
    MG_TRY(spst);
    if (!par) MG_TRY(utotal_reduce(h, mixed, par));
    else if (!fused) MG_TRY(utotal_epilogue(h, mixed, par));
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

// bonds (unforked), surface sums and the energy reduction, queued on h->st;
// unforked also the force epilogue
static int utotal_reduce(mg_handle *h, bool mixed, bool par) {
    int np = h->np;
    mg_box box;
    for (int m = 0; m < 3; ++m) {
        box.len[m] = h->boxlen[m];
        box.half[m] = h->boxlen2[m];
        box.inv[m] = h->boxleni[m];
    }
    MG_TRY(mg_phase_begin(h, "bond+reduce"));
    if ((h->nbond > 0 || h->nangle > 0) && !par) {
        BondArgs ba = bond_args(h, h->d_force, h->d_ffx);
        if (mixed) k_bond<true><<<h->nblk_bond, kBondThreads, 0, h->st>>>(ba);
        else k_bond<false><<<h->nblk_bond, kBondThreads, 0, h->st>>>(ba);
        h->launches++;
    }
    if (h->ewald != MG_EWALD_NONE && h->lsurf) {
        k_surf_sums<<<h->nblk_surf, kThreads, 0, h->st>>>(h->d_ro, h->d_az, np, h->d_part + h->part_surf);
        h->launches++;
    }
    ReduceArgs r;
    r.part = h->d_part;
    r.nptpt = h->nptpt;
    r.off[0] = h->part_pair;
    r.nblk[0] = h->nblk_pair;
    r.off[1] = h->part_rec;
    r.nblk[1] = (h->ewald != MG_EWALD_NONE) ? h->nblk_rec : 0;
    r.off[2] = h->part_bond;
    r.nblk[2] = (h->nbond > 0 || h->nangle > 0) ? h->nblk_bond : 0;
    r.off[3] = h->part_surf;
    r.nblk[3] = (h->ewald != MG_EWALD_NONE && h->lsurf) ? h->nblk_surf : 0;
    r.blk0[0] = 0;
    r.row0[0] = 0;
    for (int g = 0; g < 4; ++g) {
        int stride = red_stride(g, h->nptpt + 1), rows = kRedThreads / stride;
        int nb = (r.nblk[g] + rows - 1) / rows;
        r.blk0[g + 1] = r.blk0[g] + nb;
        if (g < 3) r.row0[g + 1] = r.row0[g] + nb * stride;
    }
    if (r.blk0[4] == 0) r.blk0[4] = r.blk0[3] = r.blk0[2] = r.blk0[1] = 1;   // one (empty) pair block
    r.ewald = h->ewald;
    r.lsurf = h->lsurf;
    r.EpsiFourPi = h->EpsiFourPi;
    r.u_self = h->u_self;
    r.surf_fac = 2.0 * 3.1415926535897932 / (3.0 * h->vol);
    r.uout = h->d_uout;
    r.rows = h->d_part + h->part_red;
    r.ticket = reinterpret_cast<unsigned *>(h->d_part + 2 * (size_t)h->part_red);
    mg_launch_pdl(k_reduce, r.blk0[4], kRedThreads, 0, h->st, r);
    h->launches++;
    MG_TRY(mg_phase_end(h, "bond+reduce"));
    if (!par) MG_TRY(utotal_epilogue(h, mixed, par));
    return MG_OK;
}

// forceo from the force accumulators (and the surface force), on h->st
static int utotal_epilogue(mg_handle *h, bool mixed, bool par) {
    int np = h->np;
    double surf_fac = 2.0 * 3.1415926535897932 / (3.0 * h->vol);
    double surf_k = h->EpsiFourPi * (2.0 * surf_fac);
    int lsurf = (h->ewald != MG_EWALD_NONE && h->lsurf) ? 1 : 0;
    if (mixed)
        mg_launch_pdl(k_epilogue<true>, (np + kThreads - 1) / kThreads, kThreads, 0, h->st, (const double *)h->d_force,
                      (const double *)nullptr, (const long long *)h->d_ffx,
                      (const long long *)(par ? h->d_ffx2 : nullptr), (const double *)h->d_az,
                      (const double *)h->d_uout, h->nptpt + 1, np, lsurf, surf_k, h->force_fac, h->d_forceo);
    else
        k_epilogue<false><<<(np + kThreads - 1) / kThreads, kThreads, 0, h->st>>>(
            h->d_force, par ? h->d_force2 : nullptr, h->d_ffx, nullptr, h->d_az, h->d_uout, h->nptpt + 1, np,
            lsurf, surf_k, h->force_fac, h->d_forceo);
    h->launches++;
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

// energies and forces to the host: the copies and the device error word are
// queued together behind the step, and the host waits once
int mg_utotal_fetch(mg_handle *h, double *forceo, double *u_twob, double *uout) {
    int n = h->nptpt + 1 + 4;
    double *u = h->h_stage;
    int *err = reinterpret_cast<int *>(h->h_stage + n);
    MG_CUDA(h, cudaMemcpyAsync(u, h->d_uout, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
    if (forceo)
        MG_CUDA(h, cudaMemcpyAsync(forceo, h->d_forceo, sizeof(double) * 3 * h->np,
                                   cudaMemcpyDeviceToHost, h->st));
    MG_CUDA(h, cudaMemcpyAsync(err, h->d_err, sizeof(int) * 4, cudaMemcpyDeviceToHost, h->st));
    MG_CUDA(h, cudaStreamSynchronize(h->st));
    return mg_utotal_staged(h, u_twob, uout);
}

// the energies and the device error word already in h_stage
int mg_utotal_staged(mg_handle *h, double *u_twob, double *uout) {
    int n = h->nptpt + 1 + 4;
    const double *u = h->h_stage;
    const int *err = reinterpret_cast<const int *>(h->h_stage + n);
    int e[4] = {err[0], err[1], err[2], err[3]};
    MG_TRY(mg_device_error_status(h, e));
    if (u_twob)
        for (int k = 0; k <= h->nptpt; ++k) u_twob[k] = u[k];
    if (uout)
        for (int k = 0; k < 4; ++k) uout[k] = u[h->nptpt + 1 + k];
    for (int k = 0; k < 4; ++k)
        if (!std::isfinite(u[h->nptpt + 1 + k]))
            return mg_fail(h, MG_ERR_NAN, "non-finite energy or virial (component %d)", k);
    return MG_OK;
}
