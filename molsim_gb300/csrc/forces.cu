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
#include "mg_internal.cuh"

namespace {

constexpr int kPairThreads = 128;
constexpr int kThreads = 256;

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

struct PairArgs {
    const double4 *pos_s;
    const int *perm, *nnb, *nbr;
    int np, npt, nptpt;
    const int *pairidx;          // [npt*npt] 1-based, column-major
    const double *ubuf;
    const float *ubuf_f;
    const int *tab_start, *tab_n;
    const double *r2umin, *r2atat;
    mg_box box;
    double rcut2;
    int cellcut;                 // 1: r2 < rcut2 (cell list), 0: r2 <= rcut2 (Verlet list)
    double *force;
    long long *ffx;
    double *part;
    int *err;
};

__device__ __forceinline__ int table_interval(const double *__restrict__ ubuf, int start, int n,
                                              double r2) {
    // smallest k with z_low(k) <= r2; z_low strictly decreasing in k
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (r2 >= ubuf[(size_t)(start + mid) * 12]) hi = mid;
        else lo = mid + 1;
    }
    return start + lo;
}

__device__ __forceinline__ int table_interval_f(const float *__restrict__ ubuf, int start, int n,
                                                float r2) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (r2 >= ubuf[(size_t)(start + mid) * 12]) hi = mid;
        else lo = mid + 1;
    }
    return start + lo;
}

template <bool MIXED>
__global__ void __launch_bounds__(kPairThreads) k_pair(PairArgs a) {
    __shared__ double sh[(MG_MAX_NPTPT + 1) * (kPairThreads / 32)];
    double acc[MG_MAX_NPTPT + 1];
    for (int v = 0; v <= a.nptpt; ++v) acc[v] = 0.0;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.np) {
        double4 pi = a.pos_s[i];
        int ti = (int)pi.w;
        int p = a.perm[i];
        double fx = 0.0, fy = 0.0, fz = 0.0;
        float gx = 0.f, gy = 0.f, gz = 0.f;
        double fsum = 0.0;
        int nn = a.nnb[i];
        for (int k = 0; k < nn; ++k) {
            int j = a.nbr[(size_t)k * a.np + i];
            double4 pj = a.pos_s[j];
            double dx = mg_pbc1(__dsub_rn(pi.x, pj.x), a.box.half[0], a.box.len[0]);
            double dy = mg_pbc1(__dsub_rn(pi.y, pj.y), a.box.half[1], a.box.len[1]);
            double dz = mg_pbc1(__dsub_rn(pi.z, pj.z), a.box.half[2], a.box.len[2]);
            double r2 = mg_r2_exact(dx, dy, dz);
            if (a.cellcut ? !(r2 < a.rcut2) : (r2 > a.rcut2)) continue;
            int tj = (int)pj.w;
            int pair = a.pairidx[tj * a.npt + ti];   // iptpt(ipt,jpt), 1-based
            if (r2 < a.r2atat[pair - 1]) {
                // hard-core overlap: u = 1e10 (the cell-list routine also sets
                // fsum = 1e10; the Verlet-list routine keeps a stale value)
                acc[pair - 1] += 0.5 * 1e10;
                if (MIXED) {
                    gx += 1e10f * (float)dx; gy += 1e10f * (float)dy; gz += 1e10f * (float)dz;
                } else {
                    fx += 1e10 * dx; fy += 1e10 * dy; fz += 1e10 * dz;
                }
                acc[a.nptpt] -= 0.5 * (1e10 * r2);
                continue;
            }
            if (r2 < a.r2umin[pair - 1]) {
                mg_dev_error(a.err, MG_ERR_TABLE_UNDERRUN, p + 1, a.perm[j] + 1, pair);
                continue;
            }
            int st = a.tab_start[pair - 1], n = a.tab_n[pair - 1];
            if (MIXED) {
                float r2f = (float)r2;
                int rec = table_interval_f(a.ubuf_f, st, n, r2f);
                const float *c = a.ubuf_f + (size_t)rec * 12;
                float d = r2f - c[0];
                float us = c[1] + d * (c[2] + d * (c[3] + d * (c[4] + d * (c[5] + d * c[6]))));
                float fs = c[7] + d * (c[8] + d * (c[9] + d * (c[10] + d * c[11])));
                gx += fs * (float)dx;
                gy += fs * (float)dy;
                gz += fs * (float)dz;
                acc[pair - 1] += 0.5 * (double)us;
                acc[a.nptpt] -= 0.5 * (double)(fs * r2f);
            } else {
                int rec = table_interval(a.ubuf, st, n, r2);
                const double *c = a.ubuf + (size_t)rec * 12;
                double d = r2 - c[0];
                double us = c[1] + d * (c[2] + d * (c[3] + d * (c[4] + d * (c[5] + d * c[6]))));
                fsum = c[7] + d * (c[8] + d * (c[9] + d * (c[10] + d * c[11])));
                fx += fsum * dx;
                fy += fsum * dy;
                fz += fsum * dz;
                acc[pair - 1] += 0.5 * us;
                acc[a.nptpt] -= 0.5 * (fsum * r2);
            }
        }
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
    block_sum<kPairThreads>(acc, a.nptpt + 1, a.part + (size_t)blockIdx.x * (a.nptpt + 1), sh);
}

// UBond: every particle adds the forces of its (at most a few) bonds; the
// bond's first particle counts its energy and virial.
template <bool MIXED>
__global__ void __launch_bounds__(kThreads) k_bond(const double *__restrict__ ro, int np,
                                                   const int *__restrict__ off,
                                                   const int *__restrict__ list,
                                                   const int *__restrict__ ij,
                                                   const double *__restrict__ bk,
                                                   const double *__restrict__ beq,
                                                   const int *__restrict__ bp, mg_box box,
                                                   double *__restrict__ force,
                                                   long long *__restrict__ ffx,
                                                   double *__restrict__ part) {
    __shared__ double sh[2 * (kThreads / 32)];
    double acc[2] = {0.0, 0.0};
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < np) {
        double f[3] = {0.0, 0.0, 0.0};
        for (int e = off[p]; e < off[p + 1]; ++e) {
            int b = list[e] >> 1, role = list[e] & 1;
            int ip = ij[2 * b], jp = ij[2 * b + 1];
            double dx = mg_pbc1(__dsub_rn(ro[3 * ip], ro[3 * jp]), box.half[0], box.len[0]);
            double dy = mg_pbc1(__dsub_rn(ro[3 * ip + 1], ro[3 * jp + 1]), box.half[1], box.len[1]);
            double dz = mg_pbc1(__dsub_rn(ro[3 * ip + 2], ro[3 * jp + 2]), box.half[2], box.len[2]);
            double r2 = dx * dx + dy * dy + dz * dz;
            double r1 = sqrt(r2);
            double term = r1 - beq[b];
            double pw = 1.0;
            for (int k = 0; k < bp[b] - 1; ++k) pw *= term;
            double fac = bk[b] * pw;
            double u = fac * term;
            fac = -bp[b] * fac / r1;
            double sgn = role ? -1.0 : 1.0;
            f[0] += sgn * (fac * dx);
            f[1] += sgn * (fac * dy);
            f[2] += sgn * (fac * dz);
            if (!role) {
                acc[0] += u;
                acc[1] -= fac * r2;
            }
        }
        if (off[p + 1] > off[p]) {
            if (MIXED) {
                for (int m = 0; m < 3; ++m) ffx[3 * p + m] += __double2ll_rn(f[m] * MG_FX_SCALE);
            } else {
                for (int m = 0; m < 3; ++m) force[3 * p + m] += f[m];
            }
        }
    }
    block_sum<kThreads>(acc, 2, part + (size_t)blockIdx.x * 2, sh);
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
    int off_pair, nblk_pair;
    int off_rec, nblk_rec;
    int off_bond, nblk_bond;
    int off_surf, nblk_surf;
    int ewald, lsurf;
    double EpsiFourPi, u_self, surf_fac;
    double *uout;
};

// one warp per value, lane-strided sums combined by a fixed shuffle tree
__global__ void k_reduce(ReduceArgs a) {
    __shared__ double vals[MG_MAX_NPTPT + 1 + 2 + 2 + 3];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int nv_pair = a.nptpt + 1;
    int nv = nv_pair + 2 + 2 + 3;
    for (int v = w; v < nv; v += nw) {
        const double *src;
        int stride, nblk, comp;
        if (v < nv_pair) { src = a.part + a.off_pair; stride = nv_pair; nblk = a.nblk_pair; comp = v; }
        else if (v < nv_pair + 2) { src = a.part + a.off_rec; stride = 2; nblk = a.nblk_rec; comp = v - nv_pair; }
        else if (v < nv_pair + 4) { src = a.part + a.off_bond; stride = 2; nblk = a.nblk_bond; comp = v - nv_pair - 2; }
        else { src = a.part + a.off_surf; stride = 3; nblk = a.nblk_surf; comp = v - nv_pair - 4; }
        double s = 0.0;
        for (int b = lane; b < nblk; b += 32) s += src[(size_t)b * stride + comp];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) vals[v] = s;
    }
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
            sx = vals[nv_pair + 4];
            sy = vals[nv_pair + 5];
            sz = vals[nv_pair + 6];
            double term = a.surf_fac * (sx * sx + sy * sy + sz * sz);
            urec = urec + term;
            virrec = virrec - term;
        }
        urec = a.EpsiFourPi * urec;
    }
    double ubond = vals[nv_pair + 2], virbond = vals[nv_pair + 3];
    int o = a.nptpt + 1;
    u[o + 0] = twob0 + urec + ubond;                          // u%tot
    u[o + 1] = urec;                                          // u%rec
    u[o + 2] = ubond;                                         // u%bond
    u[o + 3] = virtwob + a.EpsiFourPi * virrec + virbond;     // virial
    u[o + 4] = sx;
    u[o + 5] = sy;
    u[o + 6] = sz;
}

// force -> forceo with the surface force and the unit factor (energy.F90:405-424)
template <bool MIXED>
__global__ void k_epilogue(const double *__restrict__ force, const long long *__restrict__ ffx,
                           const double *__restrict__ az, const double *__restrict__ uout, int o,
                           int np, int lsurf, double surf_k, double fac,
                           double *__restrict__ forceo) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    for (int m = 0; m < 3; ++m) {
        double f = MIXED ? (double)ffx[3 * p + m] * MG_FX_INV : force[3 * p + m];
        if (lsurf) f = f - surf_k * az[p] * uout[o + 4 + m];
        forceo[3 * p + m] = f * fac;
    }
}

}  // namespace

int mg_forces_init(mg_handle *h) {
    int np = h->np;
    h->nblk_pair = (np + kPairThreads - 1) / kPairThreads;
    h->nblk_bond = (np + kThreads - 1) / kThreads;
    h->nblk_surf = (np + kThreads - 1) / kThreads;
    // rec partials: SPME z-pass blocks or std k-vectors; sized by the caller
    // of mg_forces_init (nblk_rec set before)
    h->part_pair = 0;
    h->part_rec = h->part_pair + h->nblk_pair * (h->nptpt + 1);
    h->part_bond = h->part_rec + 2 * (h->nblk_rec > 0 ? h->nblk_rec : 1);
    h->part_surf = h->part_bond + 2 * h->nblk_bond;
    size_t npart = (size_t)h->part_surf + 3 * h->nblk_surf;
    MG_CUDA(h, cudaMalloc(&h->d_part, sizeof(double) * npart));
    MG_CUDA(h, cudaMemsetAsync(h->d_part, 0, sizeof(double) * npart, h->st));
    MG_CUDA(h, cudaMalloc(&h->d_uout, sizeof(double) * (h->nptpt + 1 + 8)));
    MG_CUDA(h, cudaMemsetAsync(h->d_uout, 0, sizeof(double) * (h->nptpt + 1 + 8), h->st));
    MG_CUDA(h, cudaMalloc(&h->d_forceo, sizeof(double) * 3 * np));
    if (h->form == MG_MIXED) {
        MG_CUDA(h, cudaMalloc(&h->d_ffx, sizeof(long long) * 3 * np));
    } else {
        MG_CUDA(h, cudaMalloc(&h->d_force, sizeof(double) * 3 * np));
    }
    return MG_OK;
}

// Queue one UTotal on the handle's stream.
int mg_utotal_launch(mg_handle *h) {
    int np = h->np;
    bool mixed = h->form == MG_MIXED;
    MG_TRY(mg_phase_begin(h, "prepare"));
    k_prepare<<<(np + kThreads - 1) / kThreads, kThreads, 0, h->st>>>(h->d_ro, h->d_perm, h->d_type,
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
    a.pairidx = h->d_pairidx;
    a.ubuf = h->d_ubuf;
    a.ubuf_f = h->d_ubuf_f;
    a.tab_start = h->d_tab_start;
    a.tab_n = h->d_tab_n;
    a.r2umin = h->d_r2umin;
    a.r2atat = h->d_r2atat;
    for (int m = 0; m < 3; ++m) {
        a.box.len[m] = h->boxlen[m];
        a.box.half[m] = h->boxlen2[m];
        a.box.inv[m] = h->boxleni[m];
    }
    a.rcut2 = h->rcut2;
    a.cellcut = (h->txintlist == MG_CELLLIST) ? 1 : 0;
    a.force = h->d_force;
    a.ffx = h->d_ffx;
    a.part = h->d_part + h->part_pair;
    a.err = h->d_err;
    if (mixed) k_pair<true><<<h->nblk_pair, kPairThreads, 0, h->st>>>(a);
    else k_pair<false><<<h->nblk_pair, kPairThreads, 0, h->st>>>(a);
    h->launches += 2;
    MG_TRY(mg_phase_end(h, "pair"));

    if (h->ewald == MG_EWALD_SPM) MG_TRY(mg_spme_launch(h));
    else if (h->ewald == MG_EWALD_STD) MG_TRY(mg_ewald_std_launch(h));

    MG_TRY(mg_phase_begin(h, "bond+reduce"));
    if (h->nbond > 0) {
        if (mixed)
            k_bond<true><<<h->nblk_bond, kThreads, 0, h->st>>>(h->d_ro, np, h->d_bond_off, h->d_bond_list,
                                                               h->d_bond_ij, h->d_bond_k, h->d_bond_eq,
                                                               h->d_bond_p, a.box, h->d_force, h->d_ffx,
                                                               h->d_part + h->part_bond);
        else
            k_bond<false><<<h->nblk_bond, kThreads, 0, h->st>>>(h->d_ro, np, h->d_bond_off, h->d_bond_list,
                                                                h->d_bond_ij, h->d_bond_k, h->d_bond_eq,
                                                                h->d_bond_p, a.box, h->d_force, h->d_ffx,
                                                                h->d_part + h->part_bond);
        h->launches++;
    }
    if (h->ewald != MG_EWALD_NONE && h->lsurf) {
        k_surf_sums<<<h->nblk_surf, kThreads, 0, h->st>>>(h->d_ro, h->d_az, np, h->d_part + h->part_surf);
        h->launches++;
    }
    ReduceArgs r;
    r.part = h->d_part;
    r.nptpt = h->nptpt;
    r.off_pair = h->part_pair;
    r.nblk_pair = h->nblk_pair;
    r.off_rec = h->part_rec;
    r.nblk_rec = (h->ewald != MG_EWALD_NONE) ? h->nblk_rec : 0;
    r.off_bond = h->part_bond;
    r.nblk_bond = (h->nbond > 0) ? h->nblk_bond : 0;
    r.off_surf = h->part_surf;
    r.nblk_surf = (h->ewald != MG_EWALD_NONE && h->lsurf) ? h->nblk_surf : 0;
    r.ewald = h->ewald;
    r.lsurf = h->lsurf;
    r.EpsiFourPi = h->EpsiFourPi;
    r.u_self = h->u_self;
    r.surf_fac = 2.0 * 3.1415926535897932 / (3.0 * h->vol);
    r.uout = h->d_uout;
    k_reduce<<<1, 256, 0, h->st>>>(r);
    double surf_k = h->EpsiFourPi * (2.0 * r.surf_fac);
    int lsurf = (h->ewald != MG_EWALD_NONE && h->lsurf) ? 1 : 0;
    if (mixed)
        k_epilogue<true><<<(np + kThreads - 1) / kThreads, kThreads, 0, h->st>>>(
            h->d_force, h->d_ffx, h->d_az, h->d_uout, h->nptpt + 1, np, lsurf, surf_k, h->force_fac,
            h->d_forceo);
    else
        k_epilogue<false><<<(np + kThreads - 1) / kThreads, kThreads, 0, h->st>>>(
            h->d_force, h->d_ffx, h->d_az, h->d_uout, h->nptpt + 1, np, lsurf, surf_k, h->force_fac,
            h->d_forceo);
    h->launches += 2;
    MG_TRY(mg_phase_end(h, "bond+reduce"));
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

int mg_utotal_fetch(mg_handle *h, double *forceo, double *u_twob, double *uout) {
    int n = h->nptpt + 1 + 4;
    std::vector<double> u(n);
    MG_CUDA(h, cudaMemcpyAsync(u.data(), h->d_uout, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
    if (forceo)
        MG_CUDA(h, cudaMemcpyAsync(forceo, h->d_forceo, sizeof(double) * 3 * h->np,
                                   cudaMemcpyDeviceToHost, h->st));
    MG_TRY(mg_check_device_error(h));
    if (u_twob)
        for (int k = 0; k <= h->nptpt; ++k) u_twob[k] = u[k];
    if (uout)
        for (int k = 0; k < 4; ++k) uout[k] = u[h->nptpt + 1 + k];
    for (int k = 0; k < 4; ++k)
        if (!std::isfinite(u[h->nptpt + 1 + k]))
            return mg_fail(h, MG_ERR_NAN, "non-finite energy or virial (component %d)", k);
    return MG_OK;
}
