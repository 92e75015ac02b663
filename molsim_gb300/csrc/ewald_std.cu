// ewald_std.cu — standard Ewald reciprocal sum on the device (row A8).
//
// Reference: UEwaldRecStd (energy.F90:964-1102, serial branch :1046-1096),
// EwaldSetArray (energy.F90:1401-1425), kfac from EwaldSetup
// (energy.F90:6765-6782).
//
//   k_eik     e^{i k.r} for every particle and |n| <= ncut per dimension, by
//             the reference's recurrence eik(n) = eik(n-1) * eik(1)
//   k_sk      one block per k-vector: the four sign combinations of the
//             structure factor (sumeikr), the energy term and its virial
//   k_fk      one thread per particle: force from all k-vectors, with S(k)
//             staged through shared memory in chunks
// The arithmetic is FP64 in both forms (this sum is O(N nk) and small); the
// mixed form adds the force into its fixed-point accumulator.
#include "mg_internal.cuh"

namespace {

__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zconj(double2 a) { return make_double2(a.x, -a.y); }

__global__ void k_eik(const double *__restrict__ ro, int np, int ncut, double3 tpbi,
                      double2 *__restrict__ eik) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    double t[3] = {tpbi.x, tpbi.y, tpbi.z};
    for (int m = 0; m < 3; ++m) {
        double2 *e = eik + (size_t)m * (ncut + 1) * np + p;
        double a = t[m] * ro[3 * p + m];
        double2 e1 = make_double2(cos(a), sin(a));
        double2 cur = make_double2(1.0, 0.0);
        e[0] = cur;
        if (ncut >= 1) { cur = e1; e[(size_t)np] = cur; }
        for (int n = 2; n <= ncut; ++n) {
            cur = zmul(cur, e1);
            e[(size_t)n * np] = cur;
        }
    }
}

// four combinations for particle p and k = (nx, ny, nz) (energy.F90:1056-1061)
__device__ __forceinline__ void eikr4(const double2 *__restrict__ eik, int np, int ncut, int p,
                                      int nx, int ny, int nz, double q, double2 *er) {
    size_t plane = (size_t)(ncut + 1) * np;
    double2 ex = eik[(size_t)nx * np + p];
    double2 ey = eik[plane + (size_t)ny * np + p];
    double2 ez = eik[2 * plane + (size_t)nz * np + p];
    double2 yzm = zmul(zconj(ey), ez), yzp = zmul(ey, ez);
    double2 qxc = make_double2(q * ex.x, -(q * ex.y)), qx = make_double2(q * ex.x, q * ex.y);
    er[0] = zmul(qxc, yzm);
    er[1] = zmul(qxc, yzp);
    er[2] = zmul(qx, yzm);
    er[3] = zmul(qx, yzp);
}

__global__ void __launch_bounds__(256) k_sk(const double2 *__restrict__ eik,
                                            const double *__restrict__ az, int np, int ncut,
                                            const int4 *__restrict__ kv,
                                            const double *__restrict__ kfac, double3 tpbi,
                                            double ualpha2, double2 *__restrict__ S,
                                            double *__restrict__ part) {
    __shared__ double sh[8][8];
    int k = blockIdx.x;
    int4 n = kv[k];
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int p = threadIdx.x; p < np; p += blockDim.x) {
        double2 er[4];
        eikr4(eik, np, ncut, p, n.x, n.y, n.z, az[p], er);
        for (int c = 0; c < 4; ++c) { acc[2 * c] += er[c].x; acc[2 * c + 1] += er[c].y; }
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int v = 0; v < 8; ++v) {
        double x = acc[v];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sh[v][w] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int nw = blockDim.x >> 5;
        double s[8];
        for (int v = 0; v < 8; ++v) {
            double x = 0.0;
            for (int q = 0; q < nw; ++q) x += sh[v][q];
            s[v] = x;
        }
        double term = 0.0;
        for (int c = 0; c < 4; ++c) {
            S[4 * k + c] = make_double2(s[2 * c], s[2 * c + 1]);
            term = term + (s[2 * c] * s[2 * c] + s[2 * c + 1] * s[2 * c + 1]);
        }
        term = kfac[k] * term;
        double kx = n.x * tpbi.x, ky = n.y * tpbi.y, kz = n.z * tpbi.z;
        double k2 = kx * kx + ky * ky + kz * kz;
        part[2 * k] = term;
        part[2 * k + 1] = -(1.0 - k2 / (2.0 * ualpha2)) * term;
    }
}

template <bool MIXED>
__global__ void __launch_bounds__(128) k_fk(const double2 *__restrict__ eik,
                                            const double *__restrict__ az, int np, int ncut,
                                            const int4 *__restrict__ kv,
                                            const double *__restrict__ kfac,
                                            const double2 *__restrict__ S, int nk, double3 tpbi,
                                            double efp, double *__restrict__ force,
                                            long long *__restrict__ ffx) {
    constexpr int CH = 128;
    __shared__ double2 sS[CH][4];
    __shared__ int4 sK[CH];
    __shared__ double sF[CH];
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    double q = (p < np) ? az[p] : 0.0;
    double f0 = 0.0, f1 = 0.0, f2 = 0.0;
    for (int k0 = 0; k0 < nk; k0 += CH) {
        int cnt = min(CH, nk - k0);
        __syncthreads();
        for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
            sK[e] = kv[k0 + e];
            sF[e] = kfac[k0 + e];
            for (int c = 0; c < 4; ++c) sS[e][c] = S[4 * (k0 + e) + c];
        }
        __syncthreads();
        if (p < np) {
            for (int e = 0; e < cnt; ++e) {
                int4 n = sK[e];
                double2 er[4];
                eikr4(eik, np, ncut, p, n.x, n.y, n.z, q, er);
                double fmm = -er[0].x * sS[e][0].y + er[0].y * sS[e][0].x;
                double fmp = -er[1].x * sS[e][1].y + er[1].y * sS[e][1].x;
                double fpm = -er[2].x * sS[e][2].y + er[2].y * sS[e][2].x;
                double fpp = -er[3].x * sS[e][3].y + er[3].y * sS[e][3].x;
                double kfac2 = efp * 2.0 * sF[e];
                f0 += kfac2 * n.x * tpbi.x * (-fmm - fmp + fpm + fpp);
                f1 += kfac2 * n.y * tpbi.y * (-fmm + fmp - fpm + fpp);
                f2 += kfac2 * n.z * tpbi.z * (+fmm + fmp + fpm + fpp);
            }
        }
    }
    if (p >= np) return;
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

// UDipoleEwaldRecStd (energy.F90:1830-2040, serial branch :1960-2036), one
// block per k-vector: the structure factors of charges and dipoles, S with
// (q + i k.dip) and Sd with i k.dip in the four sign combinations, and the
// k-vector's virial term -kfac (2 sum(Re Sd Re S + Im Sd Im S) + |S|^2 (1 -
// k^2 / (2 alpha^2)))
__global__ void __launch_bounds__(256) k_dip_sk(const double2 *__restrict__ eik, const double *__restrict__ az,
                                                const double *__restrict__ dip, int np, int ncut,
                                                const int4 *__restrict__ kv, const double *__restrict__ kfac,
                                                double3 tpbi, double ualpha2, double2 *__restrict__ S,
                                                double *__restrict__ vir) {
    __shared__ double sh[16][8];
    int k = blockIdx.x;
    int4 n = kv[k];
    double kx = n.x * tpbi.x, ky = n.y * tpbi.y, kz = n.z * tpbi.z;
    double acc[16];
#pragma unroll
    for (int v = 0; v < 16; ++v) acc[v] = 0.0;
    for (int p = threadIdx.x; p < np; p += blockDim.x) {
        double2 er[4];
        eikr4(eik, np, ncut, p, n.x, n.y, n.z, 1.0, er);
        double tx = kx * dip[3 * p], ty = ky * dip[3 * p + 1], tz = kz * dip[3 * p + 2];
        double fac[4] = {-tx - ty + tz, -tx + ty + tz, +tx - ty + tz, +tx + ty + tz};
        double q = az[p];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            // (q + i f) e and (i f) e
            acc[2 * c] += q * er[c].x - fac[c] * er[c].y;
            acc[2 * c + 1] += q * er[c].y + fac[c] * er[c].x;
            acc[8 + 2 * c] += -fac[c] * er[c].y;
            acc[8 + 2 * c + 1] += fac[c] * er[c].x;
        }
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int v = 0; v < 16; ++v) {
        double x = acc[v];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sh[v][w] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int nw = blockDim.x >> 5;
        double t[16];
        for (int v = 0; v < 16; ++v) {
            double x = 0.0;
            for (int q = 0; q < nw; ++q) x += sh[v][q];
            t[v] = x;
        }
        double termx = 0.0, termy = 0.0;
        for (int c = 0; c < 4; ++c) {
            S[4 * k + c] = make_double2(t[2 * c], t[2 * c + 1]);
            termx = termx + (t[8 + 2 * c] * t[2 * c] + t[8 + 2 * c + 1] * t[2 * c + 1]);
            termy = termy + (t[2 * c] * t[2 * c] + t[2 * c + 1] * t[2 * c + 1]);
        }
        double termz = 1.0 - (kx * kx + ky * ky + kz * kz) / (2.0 * ualpha2);
        vir[k] = -(kfac[k] * (2.0 * termx + termy * termz));
    }
}

// the potential, field and field gradient of every k-vector at each atom
// (one thread per atom, the k-vectors in order, S staged in shared memory);
// added to pot[np], est[3 np], efg[6 np]
__global__ void __launch_bounds__(128) k_dip_fk(const double2 *__restrict__ eik, int np, int ncut,
                                                const int4 *__restrict__ kv, const double *__restrict__ kfac,
                                                const double2 *__restrict__ S, int nk, double3 tpbi,
                                                double *__restrict__ pot, double *__restrict__ est,
                                                double *__restrict__ efg) {
    constexpr int CH = 128;
    __shared__ double2 sS[CH][4];
    __shared__ int4 sK[CH];
    __shared__ double sF[CH];
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    double ps = 0.0, e0 = 0.0, e1 = 0.0, e2 = 0.0, g[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int k0 = 0; k0 < nk; k0 += CH) {
        int cnt = min(CH, nk - k0);
        __syncthreads();
        for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
            sK[e] = kv[k0 + e];
            sF[e] = kfac[k0 + e];
            for (int c = 0; c < 4; ++c) sS[e][c] = S[4 * (k0 + e) + c];
        }
        __syncthreads();
        if (p < np) {
            for (int e = 0; e < cnt; ++e) {
                int4 n = sK[e];
                double2 er[4];
                eikr4(eik, np, ncut, p, n.x, n.y, n.z, 1.0, er);
                // c = e_c conj(S_c)
                double2 cc[4];
#pragma unroll
                for (int c = 0; c < 4; ++c) cc[c] = zmul(er[c], zconj(sS[e][c]));
                double kfac2 = 2.0 * sF[e];
                double kx = n.x * tpbi.x, ky = n.y * tpbi.y, kz = n.z * tpbi.z;
                double rsum = cc[0].x + cc[1].x + cc[2].x + cc[3].x;
                ps += kfac2 * rsum;
                e0 += kfac2 * kx * (-cc[0].y - cc[1].y + cc[2].y + cc[3].y);
                e1 += kfac2 * ky * (-cc[0].y + cc[1].y - cc[2].y + cc[3].y);
                e2 += kfac2 * kz * (+cc[0].y + cc[1].y + cc[2].y + cc[3].y);
                g[0] += (kfac2 * kx * kx) * rsum;
                g[1] += (kfac2 * ky * ky) * rsum;
                g[2] += (kfac2 * kz * kz) * rsum;
                g[3] += (kfac2 * kx * ky) * (+cc[0].x - cc[1].x - cc[2].x + cc[3].x);
                g[4] += (kfac2 * kx * kz) * (-cc[0].x - cc[1].x + cc[2].x + cc[3].x);
                g[5] += (kfac2 * ky * kz) * (-cc[0].x + cc[1].x - cc[2].x + cc[3].x);
            }
        }
    }
    if (p >= np) return;
    pot[p] += ps;
    est[3 * p] += e0;
    est[3 * p + 1] += e1;
    est[3 * p + 2] += e2;
    for (int m = 0; m < 6; ++m) efg[6 * p + m] += g[m];
}

}  // namespace

// the reciprocal part of UDipoleEwald, standard Ewald: device arrays az
// (charges), dip, pot, est, efg of the handle's particles (pot, est, efg
// added to), vir[nkvec] per k-vector virial terms
int mg_ewald_std_dipole(mg_handle *h, const double *az, const double *dip, double *pot, double *est, double *efg,
                        double *vir) {
    int np = h->np;
    double3 tpbi = make_double3(h->TwoPiBoxi[0], h->TwoPiBoxi[1], h->TwoPiBoxi[2]);
    k_eik<<<(np + 127) / 128, 128, 0, h->st>>>(h->d_ro, np, h->ncut, tpbi, h->d_eik);
    k_dip_sk<<<h->nkvec, 256, 0, h->st>>>(h->d_eik, az, dip, np, h->ncut, h->d_kvec, h->d_kfac, tpbi,
                                          h->ualpha * h->ualpha, h->d_S, vir);
    k_dip_fk<<<(np + 127) / 128, 128, 0, h->st>>>(h->d_eik, np, h->ncut, h->d_kvec, h->d_kfac, h->d_S, h->nkvec,
                                                  tpbi, pot, est, efg);
    h->launches += 3;
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

int mg_ewald_std_init(mg_handle *h) {
    std::vector<int> kv;
    std::vector<double> kfac;
    mg_host_kvectors(h->ncut, h->ncut2, h->TwoPiBoxi, h->vol, h->ualpha, kv, kfac);
    h->nkvec = (int)kfac.size();
    if (h->nkvec < 1) return mg_fail(h, MG_ERR_ARG, "no k-vectors for ncut = %d", h->ncut);
    h->nblk_rec = h->nkvec;
    MG_CUDA(h, cudaMalloc(&h->d_kvec, sizeof(int4) * h->nkvec));
    MG_CUDA(h, cudaMemcpy(h->d_kvec, kv.data(), sizeof(int4) * h->nkvec, cudaMemcpyHostToDevice));
    MG_CUDA(h, cudaMalloc(&h->d_kfac, sizeof(double) * h->nkvec));
    MG_CUDA(h, cudaMemcpy(h->d_kfac, kfac.data(), sizeof(double) * h->nkvec, cudaMemcpyHostToDevice));
    MG_CUDA(h, cudaMalloc(&h->d_eik, sizeof(double2) * 3 * (size_t)(h->ncut + 1) * h->np));
    MG_CUDA(h, cudaMalloc(&h->d_S, sizeof(double2) * 4 * (size_t)h->nkvec));
    MG_CUDA(h, cudaMalloc(&h->d_Stm, sizeof(double2) * 4 * (size_t)h->nkvec));
    return MG_OK;
}

int mg_ewald_std_launch(mg_handle *h) {
    int np = h->np;
    double3 tpbi = make_double3(h->TwoPiBoxi[0], h->TwoPiBoxi[1], h->TwoPiBoxi[2]);
    MG_TRY(mg_phase_begin(h, "ewald_std"));
    k_eik<<<(np + 127) / 128, 128, 0, h->st>>>(h->d_ro, np, h->ncut, tpbi, h->d_eik);
    k_sk<<<h->nkvec, 256, 0, h->st>>>(h->d_eik, h->d_az, np, h->ncut, h->d_kvec, h->d_kfac, tpbi,
                                      h->ualpha * h->ualpha, h->d_S, h->d_part + h->part_rec);
    if (h->form == MG_MIXED)
        k_fk<true><<<(np + 127) / 128, 128, 0, h->st>>>(h->d_eik, h->d_az, np, h->ncut, h->d_kvec,
                                                        h->d_kfac, h->d_S, h->nkvec, tpbi,
                                                        h->EpsiFourPi, h->d_force, h->d_ffx);
    else
        k_fk<false><<<(np + 127) / 128, 128, 0, h->st>>>(h->d_eik, h->d_az, np, h->ncut, h->d_kvec,
                                                         h->d_kfac, h->d_S, h->nkvec, tpbi,
                                                         h->EpsiFourPi, h->d_force, h->d_ffx);
    h->launches += 3;
    MG_TRY(mg_phase_end(h, "ewald_std"));
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}
