// poly.cu — the two-body energy of polyatomic particles (UTwoBodyP,
// energy.F90:786-896).
//
// For every particle pair of the neighbour list whose centres lie within
// rcut (minimum image by PBC2, molaux.F90:193-248: the shift of the centre
// separation is applied to every atom pair of the two particles), every atom
// pair adds the tabulated energy (the linear interval search from iubuflow
// of its atom-type pair and the quintic in d = r^2 - z_low) to u%twob of the
// particle-type pair, fsum*dr to the first atom's force and -fsum*dr to the
// second's, and -fsum*r^2 to the virial.  FP64 arithmetic.
//
// One warp per particle walks its list row; the neighbours' atom forces are
// added as 64-bit fixed-point integers (the same bits on every call; they
// agree with the reference's sequential FP64 sums to the fixed-point
// resolution), the energies and the virial are summed per block and the
// blocks in order on the host.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <new>
#include <string>
#include <vector>

#include "mg_erf.cuh"
#include "mg_internal.cuh"

namespace {

constexpr int kPolyThreads = 128;
constexpr int kPolyMaxAtoms = 16;   // atoms per particle that the pair loop accepts
constexpr int kPolyBins = 1024;     // table-search start bins per atom-type pair


struct PolyArgs {
    int np, nptpt, maxnneigh, lmc, nbuf;
    const int *iptpn, *iptpt, *napt, *ianpn, *iatan, *iatat, *iubuflow;
    int npt, nat;
    const double *ubuf, *r2umin, *r2atat;
    // where the table search of each atom-type pair starts: r2 in bin b
    // (bin_z0 + b/bin_inv) starts at record bin_k[pair*kPolyBins + b], the
    // first record below the bin's upper edge, so the linear search of the
    // reference finds the same record in a few steps
    const double *bin_z0, *bin_inv;
    const int *bin_k;
    const double *ro, *r;
    const int *nneighpn, *jpnlist;
    double len[3], half[3], rcut2;
    double *force;
    long long *ffx;   // k_twobody_p: atom forces in 64-bit fixed point (kPolyFx), converted after the pass
    double *part;   // [nblk][nptpt + 2]: u%twob(1:nptpt), virial
    int *err;
};

// The host-list atom-pair pass adds the atom forces of a particle's
// neighbours from many warps.  It adds them as 64-bit integers at the scale
// 2^36 (a resolution of 1.5e-11 in force units, a range of 1.3e8), so that
// the sums do not depend on the order of the adds and every call gives the
// same bits; a force beyond the range flags MG_ERR_NAN.
constexpr double kPolyFx = 68719476736.0;   // 2^36
__device__ __forceinline__ void poly_fx_add(long long *p, double v, int *err) {
    double s = v * kPolyFx;
    if (!(fabs(s) < 9.0e18)) {
        mg_dev_error(err, MG_ERR_NAN, 0, 0, 0);
        return;
    }
    atomicAdd(reinterpret_cast<unsigned long long *>(p), (unsigned long long)__double2ll_rn(s));
}

__global__ void k_poly_fx_out(const long long *__restrict__ ffx, size_t n, double *__restrict__ force) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) force[i] = (double)ffx[i] * (1.0 / kPolyFx);
}

// the record (0-based index into ubuf) where the search for r2 starts
__device__ __forceinline__ int poly_search_start(const PolyArgs &a, int iatjat, double r2) {
    double x = (r2 - a.bin_z0[iatjat - 1]) * a.bin_inv[iatjat - 1];
    int b = x < 0.0 ? 0 : (x >= (double)(kPolyBins - 1) ? kPolyBins - 1 : (int)x);
    return a.bin_k[(size_t)(iatjat - 1) * kPolyBins + b];
}

__global__ void __launch_bounds__(kPolyThreads) k_twobody_p(PolyArgs a) {
    extern __shared__ double red[];   // [nptpt + 1][kPolyThreads]
    const int nv = a.nptpt + 1;
    double acc[MG_MAX_NPTPT], vir = 0.0;   // u%twob(1:nptpt) and the virial of this thread
#pragma unroll
    for (int k = 0; k < MG_MAX_NPTPT; ++k) acc[k] = 0.0;
    // one warp per particle, its lanes over the list row
    int ip = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (ip < a.np) {
        int ipt = a.iptpn[ip];
        int ialow = a.ianpn[ip] - 1, iaupp = ialow + a.napt[ipt - 1];
        int nn = a.nneighpn[ip];
        double fi[3 * kPolyMaxAtoms];   // forces on ip's atoms from this lane's neighbours
        for (int k = 0; k < 3 * (iaupp - ialow); ++k) fi[k] = 0.0;
        for (int jploc = lane; jploc < nn; jploc += 32) {
            int jp = a.jpnlist[(size_t)ip * a.maxnneigh + jploc] - 1;
            if (a.lmc && jp < ip) continue;
            int jpt = a.iptpn[jp];
            int iptjpt = a.iptpt[(jpt - 1) * a.npt + (ipt - 1)];
            double d[3], sh[3];
            for (int m = 0; m < 3; ++m) {
                d[m] = __dsub_rn(a.ro[3 * ip + m], a.ro[3 * jp + m]);
                sh[m] = fabs(d[m]) > a.half[m] ? copysign(a.len[m], d[m]) : 0.0;   // PBC2
                d[m] = __dsub_rn(d[m], sh[m]);
            }
            double r2 = mg_r2_exact(d[0], d[1], d[2]);
            if (r2 > a.rcut2) continue;
            double usum = 0.0;
            int jalow = a.ianpn[jp] - 1, jaupp = jalow + a.napt[jpt - 1];
            // the atoms of jp outer, so that each of its forces takes one
            // atomic add per particle pair; ip's atom forces stay in fi
            for (int ja = jalow; ja < jaupp; ++ja) {
                int jat = a.iatan[ja];
                double fj0 = 0.0, fj1 = 0.0, fj2 = 0.0;
                for (int ia = ialow; ia < iaupp; ++ia) {
                    int iat = a.iatan[ia];
                    int iatjat = a.iatat[(jat - 1) * a.nat + (iat - 1)];
                    double dx = __dsub_rn(__dsub_rn(a.r[3 * ia], a.r[3 * ja]), sh[0]);
                    double dy = __dsub_rn(__dsub_rn(a.r[3 * ia + 1], a.r[3 * ja + 1]), sh[1]);
                    double dz = __dsub_rn(__dsub_rn(a.r[3 * ia + 2], a.r[3 * ja + 2]), sh[2]);
                    double ar2 = mg_r2_exact(dx, dy, dz);
                    if (ar2 < a.r2umin[iatjat - 1]) {
                        mg_dev_error(a.err, MG_ERR_TABLE_UNDERRUN, ia + 1, ja + 1, iatjat);
                        continue;
                    }
                    int ibuf = poly_search_start(a, iatjat, ar2);   // 0-based start of the search
                    while (!(ar2 >= a.ubuf[ibuf])) {
                        ibuf += 12;
                        if (ibuf >= a.nbuf) break;
                    }
                    if (ibuf >= a.nbuf) {
                        mg_dev_error(a.err, MG_ERR_IBUF, iatjat, ia + 1, ja + 1);
                        continue;
                    }
                    const double *c = a.ubuf + ibuf;
                    double dd = __dsub_rn(ar2, c[0]);
                    // usum = usum + ubuf(ibuf+1) + d*(...): Fortran adds left to right
                    usum = __dadd_rn(__dadd_rn(usum, c[1]), __dmul_rn(dd, __dadd_rn(c[2], __dmul_rn(dd, __dadd_rn(c[3],
                                     __dmul_rn(dd, __dadd_rn(c[4], __dmul_rn(dd, __dadd_rn(c[5], __dmul_rn(dd, c[6]))))))))));
                    double fsum = __dadd_rn(c[7], __dmul_rn(dd, __dadd_rn(c[8], __dmul_rn(dd, __dadd_rn(c[9],
                                  __dmul_rn(dd, __dadd_rn(c[10], __dmul_rn(dd, c[11]))))))));
                    double fx = __dmul_rn(fsum, dx), fy = __dmul_rn(fsum, dy), fz = __dmul_rn(fsum, dz);
                    int k = ia - ialow;
                    fi[3 * k] = __dadd_rn(fi[3 * k], fx);
                    fi[3 * k + 1] = __dadd_rn(fi[3 * k + 1], fy);
                    fi[3 * k + 2] = __dadd_rn(fi[3 * k + 2], fz);
                    fj0 = __dsub_rn(fj0, fx);
                    fj1 = __dsub_rn(fj1, fy);
                    fj2 = __dsub_rn(fj2, fz);
                    vir = __dsub_rn(vir, __dmul_rn(fsum, ar2));
                }
                poly_fx_add(&a.ffx[3 * ja], fj0, a.err);
                poly_fx_add(&a.ffx[3 * ja + 1], fj1, a.err);
                poly_fx_add(&a.ffx[3 * ja + 2], fj2, a.err);
            }
#pragma unroll
            for (int k = 0; k < MG_MAX_NPTPT; ++k)   // static indices keep acc in registers
                if (k == iptjpt - 1) acc[k] = __dadd_rn(acc[k], usum);
        }
        for (int k = 0; k < 3 * (iaupp - ialow); ++k) {
            double v = fi[k];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) poly_fx_add(&a.ffx[3 * ialow + k], v, a.err);
        }
    }
    // block sums in a fixed order (thread 0 adds the block's values in turn)
#pragma unroll
    for (int k = 0; k <= MG_MAX_NPTPT; ++k)
        if (k < nv) red[k * blockDim.x + threadIdx.x] = (k == a.nptpt) ? vir : acc[k < MG_MAX_NPTPT ? k : 0];
    __syncthreads();
    if (threadIdx.x < nv) {
        double s = 0.0;
        for (int t = 0; t < (int)blockDim.x; ++t) s = __dadd_rn(s, red[threadIdx.x * blockDim.x + t]);
        a.part[(size_t)blockIdx.x * nv + threadIdx.x] = s;
    }
}

// the molecular part of UEwaldSelf: one thread per particle, its atom pairs
// ia < ja in order; the thread owns its atoms' forces
__global__ void __launch_bounds__(kPolyThreads) k_ewald_intra(PolyArgs a, const double *__restrict__ aza,
                                                              double ualpha, double ualpha2, double ewaldfac1,
                                                              double efp, int accumulate) {
    __shared__ double red[kPolyThreads];
    double u = 0.0;
    int ip = blockIdx.x * blockDim.x + threadIdx.x;
    if (ip < a.np) {
        int ialow = a.ianpn[ip] - 1, iaupp = ialow + a.napt[a.iptpn[ip] - 1];
        if (!accumulate)
            for (int ia = ialow; ia < iaupp; ++ia)
                for (int k = 0; k < 3; ++k) a.force[3 * ia + k] = 0.0;
        for (int ia = ialow; ia < iaupp; ++ia) {
            for (int ja = ia + 1; ja < iaupp; ++ja) {
                double dx = __dsub_rn(a.r[3 * ia], a.r[3 * ja]);
                double dy = __dsub_rn(a.r[3 * ia + 1], a.r[3 * ja + 1]);
                double dz = __dsub_rn(a.r[3 * ia + 2], a.r[3 * ja + 2]);
                double r2 = mg_r2_exact(dx, dy, dz);
                double r1 = sqrt(r2);
                double r1i = 1.0 / r1;
                double r2i = __dmul_rn(r1i, r1i);
                double ex = exp(-__dmul_rn(ualpha2, r2));
                r1i = __dmul_rn(r1i, mg_erf2(__dmul_rn(ualpha, r1)));
                double r3i = __dmul_rn(r2i, __dsub_rn(r1i, __dmul_rn(ewaldfac1, ex)));
                u = __dsub_rn(u, __dmul_rn(__dmul_rn(aza[ia], aza[ja]), r1i));
                double fac = __dmul_rn(__dmul_rn(__dmul_rn(efp, aza[ia]), aza[ja]), r3i);
                double fx = __dmul_rn(fac, dx), fy = __dmul_rn(fac, dy), fz = __dmul_rn(fac, dz);
                a.force[3 * ia] = __dsub_rn(a.force[3 * ia], fx);
                a.force[3 * ia + 1] = __dsub_rn(a.force[3 * ia + 1], fy);
                a.force[3 * ia + 2] = __dsub_rn(a.force[3 * ia + 2], fz);
                a.force[3 * ja] = __dadd_rn(a.force[3 * ja], fx);
                a.force[3 * ja + 1] = __dadd_rn(a.force[3 * ja + 1], fy);
                a.force[3 * ja + 2] = __dadd_rn(a.force[3 * ja + 2], fz);
            }
        }
    }
    red[threadIdx.x] = u;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int t = 0; t < (int)blockDim.x; ++t) s = __dadd_rn(s, red[t]);
        a.part[blockIdx.x] = s;
    }
}

// the tabulated energy of one atom pair (UTwoBodyA's search and Horner
// sums); 0: ok, MG_ERR_IBUF past the table
__device__ __forceinline__ int poly_pair_u(const PolyArgs &a, int iatjat, double r2, double *u) {
    int ibuf = poly_search_start(a, iatjat, r2);
    while (!(r2 >= a.ubuf[ibuf])) {
        ibuf += 12;
        if (ibuf >= a.nbuf) return MG_ERR_IBUF;
    }
    const double *c = a.ubuf + ibuf;
    double d = __dsub_rn(r2, c[0]);
    *u = __dadd_rn(c[1], __dmul_rn(d, __dadd_rn(c[2], __dmul_rn(d, __dadd_rn(c[3], __dmul_rn(d,
         __dadd_rn(c[4], __dmul_rn(d, __dadd_rn(c[5], __dmul_rn(d, c[6]))))))))));
    return 0;
}

// Single-particle trials (UTwoBodyPNew minus UTwoBodyPOld, nptm = 1): one
// warp per trial, lanes over the moving particle's list row; the energy of
// each neighbour with the trial centre and atoms (a hard core or a pair
// below its table rejects the trial, lhsoverlap) minus that with the
// current ones.
__global__ void k_poly_dutwobody(PolyArgs a, int ntrial, const int *__restrict__ tip,
                                 const double *__restrict__ trotm, const double *__restrict__ trtm,
                                 const int *__restrict__ tatom0, double *__restrict__ du,
                                 int *__restrict__ ovl) {
    int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (t >= ntrial) return;
    int ip = tip[t] - 1, ipt = a.iptpn[ip];
    int ialow = a.ianpn[ip] - 1, nai = a.napt[ipt - 1];
    const double *rn = trotm + 3 * t, *rt = trtm + 3 * (size_t)tatom0[t];
    double dnew = 0.0, dold = 0.0;
    int bad = 0;
    int nn = a.nneighpn[ip];
    for (int jploc = lane; jploc < nn; jploc += 32) {
        int jp = a.jpnlist[(size_t)ip * a.maxnneigh + jploc] - 1;
        if (jp == ip) continue;
        int jpt = a.iptpn[jp];
        int jalow = a.ianpn[jp] - 1, naj = a.napt[jpt - 1];
        for (int pass = 0; pass < 2; ++pass) {   // 0: trial (new), 1: current (old)
            const double *ci = pass ? a.ro + 3 * ip : rn;
            double sh[3], r2 = 0.0;
            {
                double d[3];
                for (int m = 0; m < 3; ++m) {
                    d[m] = __dsub_rn(ci[m], a.ro[3 * jp + m]);
                    sh[m] = fabs(d[m]) > a.half[m] ? copysign(a.len[m], d[m]) : 0.0;
                    d[m] = __dsub_rn(d[m], sh[m]);
                }
                r2 = mg_r2_exact(d[0], d[1], d[2]);
            }
            if (r2 > a.rcut2) continue;
            double usum = 0.0;
            for (int k = 0; k < nai; ++k) {
                const double *ra = pass ? a.r + 3 * (size_t)(ialow + k) : rt + 3 * k;
                int iat = a.iatan[ialow + k];
                for (int l = 0; l < naj; ++l) {
                    int ja = jalow + l, jat = a.iatan[ja];
                    int iatjat = a.iatat[(jat - 1) * a.nat + (iat - 1)];
                    double dx = __dsub_rn(__dsub_rn(ra[0], a.r[3 * ja]), sh[0]);
                    double dy = __dsub_rn(__dsub_rn(ra[1], a.r[3 * ja + 1]), sh[1]);
                    double dz = __dsub_rn(__dsub_rn(ra[2], a.r[3 * ja + 2]), sh[2]);
                    double ar2 = mg_r2_exact(dx, dy, dz);
                    if (pass == 0 && (ar2 < a.r2atat[iatjat - 1] || ar2 < a.r2umin[iatjat - 1])) {
                        bad = 1;
                        continue;
                    }
                    if (pass == 1 && ar2 < a.r2umin[iatjat - 1]) {
                        mg_dev_error(a.err, MG_ERR_TABLE_UNDERRUN, ialow + k + 1, ja + 1, iatjat);
                        continue;
                    }
                    double u;
                    int st = poly_pair_u(a, iatjat, ar2, &u);
                    if (st) {
                        mg_dev_error(a.err, st, iatjat, ialow + k + 1, ja + 1);
                        continue;
                    }
                    usum = __dadd_rn(usum, u);
                }
            }
            if (pass == 0) dnew = __dadd_rn(dnew, usum);
            else dold = __dadd_rn(dold, usum);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dnew += __shfl_xor_sync(0xffffffffu, dnew, o);
        dold += __shfl_xor_sync(0xffffffffu, dold, o);
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if (lane == 0) {
        ovl[t] = bad;
        du[t] = bad ? 0.0 : __dsub_rn(dnew, dold);
    }
}

// the end of UTotal: one thread per particle over its atoms in order
__global__ void __launch_bounds__(kPolyThreads) k_poly_epilogue(PolyArgs a, double fac, double *__restrict__ fo,
                                                                double *__restrict__ to,
                                                                const double *__restrict__ tqa) {
    __shared__ double red[kPolyThreads];
    double vir = 0.0;
    int ip = blockIdx.x * blockDim.x + threadIdx.x;
    if (ip < a.np) {
        int ialow = a.ianpn[ip] - 1, iaupp = ialow + a.napt[a.iptpn[ip] - 1];
        double f[3] = {0.0, 0.0, 0.0}, tq[3] = {0.0, 0.0, 0.0};
        for (int ia = ialow; ia < iaupp; ++ia) {
            double dx = __dsub_rn(a.r[3 * ia], a.ro[3 * ip]);
            double dy = __dsub_rn(a.r[3 * ia + 1], a.ro[3 * ip + 1]);
            double dz = __dsub_rn(a.r[3 * ia + 2], a.ro[3 * ip + 2]);
            const double *fa = a.force + 3 * ia;
            vir = __dadd_rn(__dadd_rn(__dadd_rn(vir, __dmul_rn(dx, fa[0])), __dmul_rn(dy, fa[1])), __dmul_rn(dz, fa[2]));
            double gx = __dmul_rn(fa[0], fac), gy = __dmul_rn(fa[1], fac), gz = __dmul_rn(fa[2], fac);
            f[0] = __dadd_rn(f[0], gx);
            f[1] = __dadd_rn(f[1], gy);
            f[2] = __dadd_rn(f[2], gz);
            tq[0] = __dadd_rn(tq[0], __dsub_rn(__dmul_rn(dy, gz), __dmul_rn(dz, gy)));
            tq[1] = __dadd_rn(tq[1], __dsub_rn(__dmul_rn(dz, gx), __dmul_rn(dx, gz)));
            tq[2] = __dadd_rn(tq[2], __dsub_rn(__dmul_rn(dx, gy), __dmul_rn(dy, gx)));
            if (tqa)   // the atom's own torque (dipoles), scaled like the forces
                for (int m = 0; m < 3; ++m) tq[m] = __dadd_rn(tq[m], __dmul_rn(tqa[3 * ia + m], fac));
        }
        for (int m = 0; m < 3; ++m) {
            fo[3 * ip + m] = f[m];
            to[3 * ip + m] = tq[m];
        }
    }
    red[threadIdx.x] = vir;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int t = 0; t < (int)blockDim.x; ++t) sum = __dadd_rn(sum, red[t]);
        a.part[blockIdx.x] = sum;
    }
}

// the atom-pair loop over the handle's full list (slot space: nbr[k*np +
// slot] holds neighbour slots, perm maps a slot to its particle): every
// thread computes its particle's atom forces from both members of each
// pair; the energy and virial of a pair are taken once, from the particle
// with the lower number
__global__ void __launch_bounds__(kPolyThreads) k_twobody_p_list(PolyArgs a, const int *__restrict__ perm,
                                                                 const int *__restrict__ nnb,
                                                                 const int *__restrict__ nbr) {
    extern __shared__ double red[];   // [nptpt + 1][kPolyThreads]
    const int nv = a.nptpt + 1;
    double acc[MG_MAX_NPTPT], vir = 0.0;
#pragma unroll
    for (int k = 0; k < MG_MAX_NPTPT; ++k) acc[k] = 0.0;
    // one warp per particle (slot), its lanes over the list row
    int slot = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (slot < a.np) {
        int ip = perm[slot];
        int ipt = a.iptpn[ip];
        int ialow = a.ianpn[ip] - 1, nai = a.napt[ipt - 1];
        double fi[3 * kPolyMaxAtoms];
        for (int k = 0; k < 3 * nai; ++k) fi[k] = 0.0;
        int nn = nnb[slot];
        for (int kk = lane; kk < nn; kk += 32) {
            int jp = perm[nbr[(size_t)kk * a.np + slot]];
            int jpt = a.iptpn[jp];
            int iptjpt = a.iptpt[(jpt - 1) * a.npt + (ipt - 1)];
            double sh[3], r2;
            {
                double d[3];
                for (int m = 0; m < 3; ++m) {
                    d[m] = __dsub_rn(a.ro[3 * ip + m], a.ro[3 * jp + m]);
                    sh[m] = fabs(d[m]) > a.half[m] ? copysign(a.len[m], d[m]) : 0.0;   // PBC2
                    d[m] = __dsub_rn(d[m], sh[m]);
                }
                r2 = mg_r2_exact(d[0], d[1], d[2]);
            }
            if (r2 > a.rcut2) continue;
            bool own = ip < jp;   // the pair's energy is counted from its lower-numbered particle
            double usum = 0.0;
            int jalow = a.ianpn[jp] - 1, naj = a.napt[jpt - 1];
            for (int k = 0; k < nai; ++k) {
                int ia = ialow + k, iat = a.iatan[ia];
                for (int l = 0; l < naj; ++l) {
                    int ja = jalow + l, jat = a.iatan[ja];
                    int iatjat = a.iatat[(jat - 1) * a.nat + (iat - 1)];
                    double dx = __dsub_rn(__dsub_rn(a.r[3 * ia], a.r[3 * ja]), sh[0]);
                    double dy = __dsub_rn(__dsub_rn(a.r[3 * ia + 1], a.r[3 * ja + 1]), sh[1]);
                    double dz = __dsub_rn(__dsub_rn(a.r[3 * ia + 2], a.r[3 * ja + 2]), sh[2]);
                    double ar2 = mg_r2_exact(dx, dy, dz);
                    if (ar2 < a.r2umin[iatjat - 1]) {
                        mg_dev_error(a.err, MG_ERR_TABLE_UNDERRUN, ia + 1, ja + 1, iatjat);
                        continue;
                    }
                    int ibuf = poly_search_start(a, iatjat, ar2);
                    while (!(ar2 >= a.ubuf[ibuf])) {
                        ibuf += 12;
                        if (ibuf >= a.nbuf) break;
                    }
                    if (ibuf >= a.nbuf) {
                        mg_dev_error(a.err, MG_ERR_IBUF, iatjat, ia + 1, ja + 1);
                        continue;
                    }
                    const double *c = a.ubuf + ibuf;
                    double dd = __dsub_rn(ar2, c[0]);
                    double fsum = __dadd_rn(c[7], __dmul_rn(dd, __dadd_rn(c[8], __dmul_rn(dd, __dadd_rn(c[9],
                                  __dmul_rn(dd, __dadd_rn(c[10], __dmul_rn(dd, c[11]))))))));
                    fi[3 * k] = __dadd_rn(fi[3 * k], __dmul_rn(fsum, dx));
                    fi[3 * k + 1] = __dadd_rn(fi[3 * k + 1], __dmul_rn(fsum, dy));
                    fi[3 * k + 2] = __dadd_rn(fi[3 * k + 2], __dmul_rn(fsum, dz));
                    if (own) {
                        usum = __dadd_rn(__dadd_rn(usum, c[1]), __dmul_rn(dd, __dadd_rn(c[2], __dmul_rn(dd,
                               __dadd_rn(c[3], __dmul_rn(dd, __dadd_rn(c[4], __dmul_rn(dd, __dadd_rn(c[5],
                               __dmul_rn(dd, c[6]))))))))));
                        vir = __dsub_rn(vir, __dmul_rn(fsum, ar2));
                    }
                }
            }
            if (own) {
#pragma unroll
                for (int k = 0; k < MG_MAX_NPTPT; ++k)
                    if (k == iptjpt - 1) acc[k] = __dadd_rn(acc[k], usum);
            }
        }
        for (int k = 0; k < 3 * nai; ++k) {
            double v = fi[k];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) a.force[3 * ialow + k] = v;
        }
    }
#pragma unroll
    for (int k = 0; k <= MG_MAX_NPTPT; ++k)
        if (k < nv) red[k * blockDim.x + threadIdx.x] = (k == a.nptpt) ? vir : acc[k < MG_MAX_NPTPT ? k : 0];
    __syncthreads();
    if (threadIdx.x < nv) {
        double sum = 0.0;
        for (int t = 0; t < (int)blockDim.x; ++t) sum = __dadd_rn(sum, red[threadIdx.x * blockDim.x + t]);
        a.part[(size_t)blockIdx.x * nv + threadIdx.x] = sum;
    }
}

// ---- charges and point dipoles (UDipoleP energy.F90:1588-1798, UDipoleEwaldSelf
// :2175-2268, UDipoleEwaldSurf :2272-2295, UDipole's loop :1510-1545) ----------
// potstat, estat (3), efg (6: xx, yy, zz, xy, xz, yz) per atom, FP64.

struct DipTerms {
    double p, e[3], g[6];
};

// the potential, field and field gradient at atom i from atom j (charge qj,
// dipole dj) and at j from i, for d = r_i - r_j and the radial kernels
// r1i .. r7i; vv is the pair's virial term (-q_i e_i . d - dip_i . efg_i . d)
__device__ __forceinline__ void dip_pair_terms(const double d[3], double qi, const double *di, double qj,
                                               const double *dj, double r1i, double r3i, double r5i, double r7i,
                                               DipTerms &oi, DipTerms &oj, double &vv) {
    double threer5i = 3.0 * r5i;
    double doti = di[0] * d[0] + di[1] * d[1] + di[2] * d[2];
    double dotj = dj[0] * d[0] + dj[1] * d[1] + dj[2] * d[2];
    double dotir5i = 3.0 * r5i * doti, dotjr5i = 3.0 * r5i * dotj;
    double dotir7i = 15.0 * r7i * doti, dotjr7i = 15.0 * r7i * dotj;
    oi.p = qj * r1i + dotj * r3i;
    oj.p = qi * r1i - doti * r3i;
    for (int m = 0; m < 3; ++m) {
        oi.e[m] = (qj * d[m] - dj[m]) * r3i + dotjr5i * d[m];
        oj.e[m] = (-qi * d[m] - di[m]) * r3i + dotir5i * d[m];
    }
    vv = -qi * (oi.e[0] * d[0] + oi.e[1] * d[1] + oi.e[2] * d[2]);
    for (int m = 0; m < 3; ++m) {
        double dm2 = d[m] * d[m];
        oi.g[m] = qj * r3i + (-qj * dm2 + 2.0 * dj[m] * d[m] + dotj) * threer5i - dotjr7i * dm2;
        oj.g[m] = qi * r3i + (-qi * dm2 - 2.0 * di[m] * d[m] - doti) * threer5i + dotir7i * dm2;
    }
    const int A[3] = {0, 0, 1}, B[3] = {1, 2, 2};
    for (int k = 0; k < 3; ++k) {
        int x = A[k], y = B[k];
        double dxy = d[x] * d[y];
        oi.g[3 + k] = (-qj * dxy + dj[x] * d[y] + dj[y] * d[x]) * threer5i - dotjr7i * dxy;
        oj.g[3 + k] = (-qi * dxy - di[x] * d[y] - di[y] * d[x]) * threer5i + dotir7i * dxy;
    }
    // dip_i . efg_i . d with efg symmetric (xx yy zz xy xz yz)
    const double *g = oi.g;
    double gd0 = g[0] * d[0] + g[3] * d[1] + g[4] * d[2];
    double gd1 = g[3] * d[0] + g[1] * d[1] + g[5] * d[2];
    double gd2 = g[4] * d[0] + g[5] * d[1] + g[2] * d[2];
    vv -= di[0] * gd0 + di[1] * gd1 + di[2] * gd2;
}

struct DipArgs {
    const double *az, *dip;
    double *pot, *est, *efg;
    // k_dipole_real: pot, est, efg (the same layout, 10 na values) in 64-bit
    // fixed point at kDipFx, converted after the pass
    long long *fx;
    int na;
    int *err;
    double ualpha, ualpha2, f1, f2, f3;
    int lewald;
};

// The real-space dipole pass adds the atoms' potentials, fields and field
// gradients (charge units per A^k, k = 1, 2, 3) from many warps as 64-bit
// integers at the scale 2^40 (resolution 9.1e-13, range 8.4e6), so that the
// sums do not depend on the order of the adds; a value beyond the range
// flags MG_ERR_NAN.
constexpr double kDipFx = 1099511627776.0;   // 2^40
__device__ __forceinline__ void dip_fx_add(long long *p, double v, int *err) {
    double s = v * kDipFx;
    if (!(fabs(s) < 9.0e18)) {
        mg_dev_error(err, MG_ERR_NAN, 0, 0, 0);
        return;
    }
    atomicAdd(reinterpret_cast<unsigned long long *>(p), (unsigned long long)__double2ll_rn(s));
}

__device__ __forceinline__ void dip_add_fx(const DipArgs &q, int ia, const DipTerms &t) {
    dip_fx_add(&q.fx[ia], t.p, q.err);
    for (int m = 0; m < 3; ++m) dip_fx_add(&q.fx[q.na + 3 * ia + m], t.e[m], q.err);
    for (int m = 0; m < 6; ++m) dip_fx_add(&q.fx[4 * q.na + 6 * ia + m], t.g[m], q.err);
}

__global__ void k_dip_fx_out(const long long *__restrict__ fx, size_t n, double *__restrict__ out) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (double)fx[i] * (1.0 / kDipFx);
}

// UDipoleP: one warp per particle, lanes over its list row; for each of the
// particle's atoms the lanes' sums are combined by shuffles, the partner
// atoms' terms added as fixed-point integers; the virial per block
__global__ void __launch_bounds__(kPolyThreads) k_dipole_real(PolyArgs a, DipArgs q) {
    __shared__ double red[kPolyThreads];
    double vir = 0.0;
    int ip = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (ip < a.np) {
        int ipt = a.iptpn[ip];
        int ialow = a.ianpn[ip] - 1, iaupp = ialow + a.napt[ipt - 1];
        int nn = a.nneighpn[ip];
        for (int ia = ialow; ia < iaupp; ++ia) {
            DipTerms acc = {};
            double qi = q.az[ia];
            const double *di = q.dip + 3 * ia;
            for (int jploc = lane; jploc < nn; jploc += 32) {
                int jp = a.jpnlist[(size_t)ip * a.maxnneigh + jploc] - 1;
                if (a.lmc && jp < ip) continue;
                int jpt = a.iptpn[jp];
                double dc[3], sh[3];
                for (int m = 0; m < 3; ++m) {
                    dc[m] = a.ro[3 * ip + m] - a.ro[3 * jp + m];
                    sh[m] = fabs(dc[m]) > a.half[m] ? copysign(a.len[m], dc[m]) : 0.0;   // PBC2
                    dc[m] = dc[m] - sh[m];
                }
                if (dc[0] * dc[0] + dc[1] * dc[1] + dc[2] * dc[2] > a.rcut2) continue;
                int jalow = a.ianpn[jp] - 1, jaupp = jalow + a.napt[jpt - 1];
                for (int ja = jalow; ja < jaupp; ++ja) {
                    double d[3];
                    for (int m = 0; m < 3; ++m) d[m] = a.r[3 * ia + m] - a.r[3 * ja + m] - sh[m];
                    double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                    double r1 = sqrt(r2), r1i = 1.0 / r1, r2i = r1i * r1i, r3i, r5i, r7i;
                    if (q.lewald) {
                        double ex = exp(-q.ualpha2 * r2);
                        r1i = r1i * (1.0 - mg_erf2(q.ualpha * r1));
                        r3i = r2i * (r1i + q.f1 * ex);
                        r5i = r2i * (r3i + q.f2 * ex);
                        r7i = r2i * (r5i + q.f3 * ex);
                    } else {
                        r3i = r2i * r1i;
                        r5i = r2i * r3i;
                        r7i = r2i * r5i;
                    }
                    DipTerms oi, oj;
                    double vv;
                    dip_pair_terms(d, qi, di, q.az[ja], q.dip + 3 * ja, r1i, r3i, r5i, r7i, oi, oj, vv);
                    acc.p += oi.p;
                    for (int m = 0; m < 3; ++m) acc.e[m] += oi.e[m];
                    for (int m = 0; m < 6; ++m) acc.g[m] += oi.g[m];
                    vir += vv;
                    dip_add_fx(q, ja, oj);
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                acc.p += __shfl_xor_sync(0xffffffffu, acc.p, o);
                for (int m = 0; m < 3; ++m) acc.e[m] += __shfl_xor_sync(0xffffffffu, acc.e[m], o);
                for (int m = 0; m < 6; ++m) acc.g[m] += __shfl_xor_sync(0xffffffffu, acc.g[m], o);
            }
            if (lane == 0) dip_add_fx(q, ia, acc);
        }
    }
    red[threadIdx.x] = vir;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int t = 0; t < (int)blockDim.x; ++t) sum += red[t];
        a.part[blockIdx.x] = sum;
    }
}

// the molecular part of UDipoleEwaldSelf: one thread per particle, its atom
// pairs ia < ja in order with the erf kernels, every term negated; the
// thread owns its atoms
__global__ void __launch_bounds__(kPolyThreads) k_dipole_intra(PolyArgs a, DipArgs q) {
    __shared__ double red[kPolyThreads];
    double vir = 0.0;
    int ip = blockIdx.x * blockDim.x + threadIdx.x;
    if (ip < a.np) {
        int ialow = a.ianpn[ip] - 1, iaupp = ialow + a.napt[a.iptpn[ip] - 1];
        for (int ia = ialow; ia < iaupp; ++ia) {
            for (int ja = ia + 1; ja < iaupp; ++ja) {
                double d[3];
                for (int m = 0; m < 3; ++m) d[m] = a.r[3 * ia + m] - a.r[3 * ja + m];
                double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                double r1 = sqrt(r2), r1i = 1.0 / r1, r2i = r1i * r1i;
                double ex = exp(-q.ualpha2 * r2);
                r1i = r1i * mg_erf2(q.ualpha * r1);
                double r3i = r2i * (r1i - q.f1 * ex);
                double r5i = r2i * (r3i - q.f2 * ex);
                double r7i = r2i * (r5i - q.f3 * ex);
                DipTerms oi, oj;
                double vv;
                dip_pair_terms(d, q.az[ia], q.dip + 3 * ia, q.az[ja], q.dip + 3 * ja, r1i, r3i, r5i, r7i, oi, oj, vv);
                q.pot[ia] -= oi.p;
                q.pot[ja] -= oj.p;
                for (int m = 0; m < 3; ++m) { q.est[3 * ia + m] -= oi.e[m]; q.est[3 * ja + m] -= oj.e[m]; }
                for (int m = 0; m < 6; ++m) { q.efg[6 * ia + m] -= oi.g[m]; q.efg[6 * ja + m] -= oj.g[m]; }
                vir -= vv;
            }
        }
    }
    red[threadIdx.x] = vir;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int t = 0; t < (int)blockDim.x; ++t) sum += red[t];
        a.part[blockIdx.x] = sum;
    }
}

// UDipoleEwaldSurf's sums (q r and dip over all atoms), one block of 1024
// threads, strided per-thread sums combined in a fixed order
__global__ void __launch_bounds__(1024) k_dipole_surf_sums(int na, DipArgs q, const double *__restrict__ r,
                                                           double *__restrict__ out6) {
    __shared__ double red[6][32];
    double s[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int ia = threadIdx.x; ia < na; ia += blockDim.x) {
        for (int m = 0; m < 3; ++m) s[m] += q.az[ia] * r[3 * ia + m];
        for (int m = 0; m < 3; ++m) s[3 + m] += q.dip[3 * ia + m];
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = 0; k < 6; ++k) {
        for (int o = 16; o > 0; o >>= 1) s[k] += __shfl_down_sync(0xffffffffu, s[k], o);
        if (lane == 0) red[k][w] = s[k];
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[threadIdx.x][k];
        out6[threadIdx.x] = t;
    }
}

__global__ void k_dipole_surf_apply(int na, DipArgs q, const double *__restrict__ r, const double *__restrict__ s6,
                                    double fac) {
    int ia = blockIdx.x * blockDim.x + threadIdx.x;
    if (ia >= na) return;
    double tx = s6[0] + s6[3], ty = s6[1] + s6[4], tz = s6[2] + s6[5];
    q.pot[ia] += fac * (r[3 * ia] * tx + r[3 * ia + 1] * ty + r[3 * ia + 2] * tz);
    q.est[3 * ia] -= fac * tx;
    q.est[3 * ia + 1] -= fac * ty;
    q.est[3 * ia + 2] -= fac * tz;
}

// the UDipole loop: force += EpsiFourPi (q e + dip . efg), torque +=
// EpsiFourPi dip x e, and per block the sum of q pot - dip . e
__global__ void __launch_bounds__(kPolyThreads) k_dipole_finish(int na, DipArgs q, double efp,
                                                                double *__restrict__ force,
                                                                double *__restrict__ torque,
                                                                double *__restrict__ part) {
    __shared__ double red[kPolyThreads];
    double u = 0.0;
    int ia = blockIdx.x * blockDim.x + threadIdx.x;
    if (ia < na) {
        const double *d = q.dip + 3 * ia, *e = q.est + 3 * ia, *g = q.efg + 6 * ia;
        double qa = q.az[ia];
        u = qa * q.pot[ia] - (d[0] * e[0] + d[1] * e[1] + d[2] * e[2]);
        if (force) {
            force[3 * ia] += efp * (qa * e[0] + (d[0] * g[0] + d[1] * g[3] + d[2] * g[4]));
            force[3 * ia + 1] += efp * (qa * e[1] + (d[0] * g[3] + d[1] * g[1] + d[2] * g[5]));
            force[3 * ia + 2] += efp * (qa * e[2] + (d[0] * g[4] + d[1] * g[5] + d[2] * g[2]));
            torque[3 * ia] += efp * (d[1] * e[2] - d[2] * e[1]);
            torque[3 * ia + 1] += efp * (d[2] * e[0] - d[0] * e[2]);
            torque[3 * ia + 2] += efp * (d[0] * e[1] - d[1] * e[0]);
        }
    }
    red[threadIdx.x] = u;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int t = 0; t < (int)blockDim.x; ++t) sum += red[t];
        part[blockIdx.x] = sum;
    }
}

}  // namespace

struct mg_poly {
    mg_poly_params p{};
    int maxnneigh = 0, nblk = 0, nblk_w = 0;   // blocks of the thread- and warp-per-particle kernels
    std::string err;
    int *d_iptpn = nullptr, *d_iptpt = nullptr, *d_napt = nullptr, *d_ianpn = nullptr, *d_iatan = nullptr,
        *d_iatat = nullptr, *d_iubuflow = nullptr, *d_nneigh = nullptr, *d_jpnlist = nullptr, *d_err = nullptr,
        *d_tip = nullptr, *d_tatom0 = nullptr, *d_tovl = nullptr;
    double *d_r2atat = nullptr, *d_trotm = nullptr, *d_trtm = nullptr, *d_tdu = nullptr;
    int tcap = 0, tacap = 0;
    double *d_fo = nullptr, *d_to = nullptr;
    double *d_bin_z0 = nullptr, *d_bin_inv = nullptr;
    int *d_bin_k = nullptr;
    double *d_ubuf = nullptr, *d_r2umin = nullptr, *d_ro = nullptr, *d_r = nullptr, *d_force = nullptr,
           *d_part = nullptr, *d_aza = nullptr;
    long long *d_ffx = nullptr;   // the host-list pair pass's fixed-point atom forces
    long long *d_dfx = nullptr;   // the real-space dipole pass's fixed-point pot, est, efg
    std::vector<double> h_part;
    // rigid-body velocity Verlet (mg_poly_rigid_*): per particle
    // [0,3) ro, [3,7) qua, [7,10) rod, [10,13) rodd, [13,17) quad,
    // [17,21) quadd, [21,24) massip (repeated), [24,27) momp, [27,30) momip
    double *d_rig = nullptr;
    double rig_tstep = 0.0, rig_tvvite = 0.0;
    int rig_nvvite = 0;
    double *d_rig_io = nullptr;   // staging: ro, ori, drostep out; forceo, torqueo in; rod, angvelo out
    // dipole electrostatics (mg_poly_udipole_*): dip, pot, est, efg, force,
    // torque per atom and the surface sums
    double *d_dscr = nullptr;
};

static int poly_fail(mg_poly *c, int code, const char *fmt, ...) {
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return code;
}

#define POLY_CUDA(c, call)                                                                                \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) return poly_fail((c), MG_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

template <typename T> static int poly_upload(mg_poly *c, T **d, const T *h, size_t n) {
    POLY_CUDA(c, cudaMalloc(d, sizeof(T) * std::max<size_t>(n, 1)));
    if (n) POLY_CUDA(c, cudaMemcpy(*d, h, sizeof(T) * n, cudaMemcpyHostToDevice));
    return MG_OK;
}

extern "C" int mg_poly_destroy(mg_poly *c) {
    if (!c) return MG_OK;
    void *ptrs[] = {c->d_iptpn, c->d_iptpt, c->d_napt, c->d_ianpn, c->d_iatan, c->d_iatat, c->d_iubuflow,
                    c->d_nneigh, c->d_jpnlist, c->d_err, c->d_ubuf, c->d_r2umin, c->d_ro, c->d_r,
                    c->d_force, c->d_ffx, c->d_part, c->d_aza, c->d_r2atat, c->d_tip, c->d_tatom0, c->d_tovl,
                    c->d_trotm, c->d_trtm, c->d_tdu, c->d_fo, c->d_to, c->d_bin_z0, c->d_bin_inv, c->d_bin_k,
                    c->d_rig, c->d_rig_io, c->d_dscr, c->d_dfx};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    delete c;
    return MG_OK;
}

extern "C" int mg_poly_last_error(const mg_poly *c, char *buf, size_t n) {
    if (!buf || !n) return MG_ERR_ARG;
    std::snprintf(buf, n, "%s", c ? c->err.c_str() : "");
    return MG_OK;
}

static int poly_check_params(const mg_poly_params *p, int maxnneigh) {
    if (p->abi_version != MG_ABI_VERSION || p->np < 1 || p->npt < 1 || p->nptpt != p->npt * (p->npt + 1) / 2 ||
        p->nptpt > MG_MAX_NPTPT || p->na < 1 || p->nat < 1 || p->natat < 1 || p->nbuf < 12 || maxnneigh < 1)
        return MG_ERR_ARG;
    if (!p->iptpn || !p->iptpt || !p->napt || !p->ianpn || !p->iatan || !p->iatat || !p->ubuf || !p->iubuflow ||
        !p->r2umin)
        return MG_ERR_ARG;
    for (int i = 0; i < p->np; ++i) {
        int t = p->iptpn[i];
        if (t < 1 || t > p->npt) return MG_ERR_ARG;
        int a0 = p->ianpn[i], na = p->napt[t - 1];
        if (a0 < 1 || na < 1 || na > kPolyMaxAtoms || a0 - 1 + na > p->na) return MG_ERR_ARG;
    }
    for (int a = 0; a < p->na; ++a)
        if (p->iatan[a] < 1 || p->iatan[a] > p->nat) return MG_ERR_ARG;
    for (int k = 0; k < p->nat * p->nat; ++k)
        if (p->iatat[k] < 1 || p->iatat[k] > p->natat) return MG_ERR_ARG;
    for (int k = 0; k < p->npt * p->npt; ++k)
        if (p->iptpt[k] < 1 || p->iptpt[k] > p->nptpt) return MG_ERR_ARG;
    for (int k = 0; k < p->natat; ++k)
        if (p->iubuflow[k] < 1 || p->iubuflow[k] + 11 > p->nbuf) return MG_ERR_ARG;
    return MG_OK;
}

extern "C" int mg_poly_create(const mg_poly_params *p, int32_t maxnneigh, mg_poly **out) {
    if (!p || !out) return MG_ERR_ARG;
    *out = nullptr;
    int st = poly_check_params(p, maxnneigh);
    if (st) return st;
    mg_poly *c = new (std::nothrow) mg_poly();
    if (!c) return MG_ERR_ALLOC;
    c->p = *p;
    c->maxnneigh = maxnneigh;
    c->nblk = (p->np + kPolyThreads - 1) / kPolyThreads;
    c->nblk_w = (int)(((long)p->np * 32 + kPolyThreads - 1) / kPolyThreads);
    int np = p->np, na = p->na;
    if ((st = poly_upload(c, &c->d_iptpn, p->iptpn, np)) || (st = poly_upload(c, &c->d_iptpt, p->iptpt, (size_t)p->npt * p->npt)) ||
        (st = poly_upload(c, &c->d_napt, p->napt, p->npt)) || (st = poly_upload(c, &c->d_ianpn, p->ianpn, np)) ||
        (st = poly_upload(c, &c->d_iatan, p->iatan, na)) ||
        (st = poly_upload(c, &c->d_iatat, p->iatat, (size_t)p->nat * p->nat)) ||
        (st = poly_upload(c, &c->d_iubuflow, p->iubuflow, p->natat)) ||
        (st = poly_upload(c, &c->d_ubuf, p->ubuf, p->nbuf)) || (st = poly_upload(c, &c->d_r2umin, p->r2umin, p->natat)) ||
        (p->aza && (st = poly_upload(c, &c->d_aza, p->aza, na))) ||
        (p->r2atat && (st = poly_upload(c, &c->d_r2atat, p->r2atat, p->natat)))) {
        mg_poly_destroy(c);
        return st;
    }
    cudaError_t e = cudaMalloc(&c->d_ro, sizeof(double) * 3 * np);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_r, sizeof(double) * 3 * na);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_force, sizeof(double) * 3 * na);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_ffx, sizeof(long long) * 3 * na);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_nneigh, sizeof(int) * np);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_jpnlist, sizeof(int) * (size_t)maxnneigh * np);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_err, sizeof(int) * 4);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_part, sizeof(double) * (size_t)c->nblk_w * (p->nptpt + 1));
    if (e != cudaSuccess) {
        mg_poly_destroy(c);
        return MG_ERR_CUDA;
    }
    c->h_part.resize((size_t)c->nblk_w * (p->nptpt + 1));
    // search-start bins per atom-type pair over [r2umin, z_low of the first
    // record]: bin b starts at the first record whose z_low is at or below
    // the upper edge of bin b+1 (records run from large to small z_low).
    // The device rounds the bin of an r2 independently of this edge, so an
    // r2 a few ulps past bin b's own upper edge can land in bin b; the
    // margin of one bin keeps such an r2 below the edge used here, and the
    // search never starts past the reference's record.
    {
        std::vector<double> z0(p->natat), inv(p->natat);
        std::vector<int> kk((size_t)p->natat * kPolyBins);
        for (int q = 0; q < p->natat; ++q) {
            int r0 = p->iubuflow[q] - 1;
            double lo = p->r2umin[q], hi = p->ubuf[r0];
            if (!(hi > lo)) hi = lo + 1.0;
            z0[q] = lo;
            inv[q] = kPolyBins / (hi - lo);
            for (int b = 0; b < kPolyBins; ++b) {
                double upper = lo + (b + 2) / inv[q];
                int rr = r0;
                while (rr + 12 < p->nbuf && p->ubuf[rr] > upper) rr += 12;
                kk[(size_t)q * kPolyBins + b] = b == kPolyBins - 1 ? r0 : rr;
            }
        }
        if ((st = poly_upload(c, &c->d_bin_z0, z0.data(), z0.size())) ||
            (st = poly_upload(c, &c->d_bin_inv, inv.data(), inv.size())) ||
            (st = poly_upload(c, &c->d_bin_k, kk.data(), kk.size()))) {
            mg_poly_destroy(c);
            return st;
        }
    }
    *out = c;
    return MG_OK;
}

extern "C" int mg_poly_utwobody(mg_poly *c, const double *ro, const double *r, const int32_t *nneighpn,
                                const int32_t *jpnlist, double *force, double *u_twob, double *virial) {
    if (!c || !ro || !r || !nneighpn || !jpnlist || !force || !u_twob || !virial) return MG_ERR_ARG;
    const mg_poly_params &p = c->p;
    int np = p.np, na = p.na;
    for (int i = 0; i < np; ++i) {
        if (nneighpn[i] < 0 || nneighpn[i] > c->maxnneigh)
            return poly_fail(c, MG_ERR_NEIGH_OVERFLOW, "nneighpn(%d) = %d > maxnneigh %d", i + 1, nneighpn[i],
                             c->maxnneigh);
        for (int k = 0; k < nneighpn[i]; ++k) {
            int j = jpnlist[(size_t)i * c->maxnneigh + k];
            if (j < 1 || j > np || j == i + 1) return poly_fail(c, MG_ERR_ARG, "jpnlist(%d,%d) = %d", k + 1, i + 1, j);
        }
    }
    POLY_CUDA(c, cudaMemcpy(c->d_ro, ro, sizeof(double) * 3 * np, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_r, r, sizeof(double) * 3 * na, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_nneigh, nneighpn, sizeof(int) * np, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_jpnlist, jpnlist, sizeof(int) * (size_t)c->maxnneigh * np, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemset(c->d_ffx, 0, sizeof(long long) * 3 * na));
    POLY_CUDA(c, cudaMemset(c->d_err, 0, sizeof(int) * 4));
    PolyArgs a;
    a.np = np;
    a.nptpt = p.nptpt;
    a.maxnneigh = c->maxnneigh;
    a.lmc = p.lmc;
    a.nbuf = p.nbuf;
    a.iptpn = c->d_iptpn;
    a.iptpt = c->d_iptpt;
    a.napt = c->d_napt;
    a.ianpn = c->d_ianpn;
    a.iatan = c->d_iatan;
    a.iatat = c->d_iatat;
    a.iubuflow = c->d_iubuflow;
    a.npt = p.npt;
    a.nat = p.nat;
    a.ubuf = c->d_ubuf;
    a.r2umin = c->d_r2umin;
    a.r2atat = c->d_r2atat;
    a.bin_z0 = c->d_bin_z0;
    a.bin_inv = c->d_bin_inv;
    a.bin_k = c->d_bin_k;
    a.ro = c->d_ro;
    a.r = c->d_r;
    a.nneighpn = c->d_nneigh;
    a.jpnlist = c->d_jpnlist;
    for (int m = 0; m < 3; ++m) {
        a.len[m] = p.boxlen[m];
        a.half[m] = 0.5 * p.boxlen[m];
    }
    a.rcut2 = p.rcut * p.rcut;
    a.force = c->d_force;
    a.ffx = c->d_ffx;
    a.part = c->d_part;
    a.err = c->d_err;
    size_t sm = sizeof(double) * (p.nptpt + 1) * kPolyThreads;
    k_twobody_p<<<c->nblk_w, kPolyThreads, sm>>>(a);
    k_poly_fx_out<<<(unsigned)((3 * (size_t)na + 255) / 256), 256>>>(c->d_ffx, 3 * (size_t)na, c->d_force);
    POLY_CUDA(c, cudaGetLastError());
    int herr[4];
    POLY_CUDA(c, cudaMemcpy(herr, c->d_err, sizeof herr, cudaMemcpyDeviceToHost));
    if (herr[0] == MG_ERR_TABLE_UNDERRUN)
        return poly_fail(c, herr[0], "r2 < r2umin for atoms %d and %d (atom-type pair %d)", herr[1], herr[2], herr[3]);
    if (herr[0] == MG_ERR_NAN) return poly_fail(c, herr[0], "an atom force beyond the fixed-point range (|f| >= 1.3e8)");
    if (herr[0]) return poly_fail(c, herr[0], "ibuf > nbuf for atom-type pair %d", herr[1]);
    POLY_CUDA(c, cudaMemcpy(force, c->d_force, sizeof(double) * 3 * na, cudaMemcpyDeviceToHost));
    POLY_CUDA(c, cudaMemcpy(c->h_part.data(), c->d_part, sizeof(double) * c->h_part.size(), cudaMemcpyDeviceToHost));
    int nv = p.nptpt + 1;
    double tot = 0.0, vir = 0.0;
    for (int k = 0; k < p.nptpt; ++k) {
        double s = 0.0;
        for (int b = 0; b < c->nblk_w; ++b) s += c->h_part[(size_t)b * nv + k];
        u_twob[k + 1] = s;
    }
    for (int k = 1; k <= p.nptpt; ++k) tot += u_twob[k];   // u%twob(0) = sum(u%twob(1:nptpt))
    u_twob[0] = tot;
    for (int b = 0; b < c->nblk_w; ++b) vir += c->h_part[(size_t)b * nv + p.nptpt];
    *virial = vir;
    return MG_OK;
}

extern "C" int mg_poly_ewald_intra(mg_poly *c, const double *r, double *force, double *u_rec) {
    if (!c || !r || !force || !u_rec) return MG_ERR_ARG;
    if (!c->d_aza) return poly_fail(c, MG_ERR_STATE, "mg_poly_params.aza (atom charges) was not given");
    const mg_poly_params &p = c->p;
    POLY_CUDA(c, cudaMemcpy(c->d_r, r, sizeof(double) * 3 * p.na, cudaMemcpyHostToDevice));
    PolyArgs a = {};
    a.np = p.np;
    a.iptpn = c->d_iptpn;
    a.napt = c->d_napt;
    a.ianpn = c->d_ianpn;
    a.r = c->d_r;
    a.force = c->d_force;
    a.part = c->d_part;
    // UEwaldSelf's constants (EwaldSetup, energy.F90:7040-7042)
    double ualpha2 = p.ualpha * p.ualpha;
    double fac = 1.0 / (std::sqrt(3.1415926535897932) * p.ualpha);
    double ewaldfac1 = fac * 2.0 * ualpha2;
    k_ewald_intra<<<c->nblk, kPolyThreads>>>(a, c->d_aza, p.ualpha, ualpha2, ewaldfac1, p.epsi_four_pi, 0);
    POLY_CUDA(c, cudaGetLastError());
    POLY_CUDA(c, cudaMemcpy(force, c->d_force, sizeof(double) * 3 * p.na, cudaMemcpyDeviceToHost));
    POLY_CUDA(c, cudaMemcpy(c->h_part.data(), c->d_part, sizeof(double) * c->nblk, cudaMemcpyDeviceToHost));
    double u = 0.0;
    for (int b = 0; b < c->nblk; ++b) u += c->h_part[b];
    *u_rec = p.epsi_four_pi * u;   // u%rec = EpsiFourPi*u%rec (UEwald, energy.F90:950)
    return MG_OK;
}

static PolyArgs poly_args(mg_poly *c) {
    const mg_poly_params &p = c->p;
    PolyArgs a = {};
    a.np = p.np;
    a.nptpt = p.nptpt;
    a.maxnneigh = c->maxnneigh;
    a.lmc = p.lmc;
    a.nbuf = p.nbuf;
    a.iptpn = c->d_iptpn;
    a.iptpt = c->d_iptpt;
    a.napt = c->d_napt;
    a.ianpn = c->d_ianpn;
    a.iatan = c->d_iatan;
    a.iatat = c->d_iatat;
    a.iubuflow = c->d_iubuflow;
    a.npt = p.npt;
    a.nat = p.nat;
    a.ubuf = c->d_ubuf;
    a.r2umin = c->d_r2umin;
    a.r2atat = c->d_r2atat;
    a.bin_z0 = c->d_bin_z0;
    a.bin_inv = c->d_bin_inv;
    a.bin_k = c->d_bin_k;
    a.ro = c->d_ro;
    a.r = c->d_r;
    a.nneighpn = c->d_nneigh;
    a.jpnlist = c->d_jpnlist;
    for (int m = 0; m < 3; ++m) {
        a.len[m] = p.boxlen[m];
        a.half[m] = 0.5 * p.boxlen[m];
    }
    a.rcut2 = p.rcut * p.rcut;
    a.force = c->d_force;
    a.part = c->d_part;
    a.err = c->d_err;
    return a;
}

extern "C" int mg_poly_dutwobody_batch(mg_poly *c, const double *ro, const double *r, const int32_t *nneighpn,
                                       const int32_t *jpnlist, int32_t ntrial, const int32_t *ip,
                                       const double *rotm, const double *rtm, double *du_twob,
                                       int32_t *lhsoverlap) {
    if (!c || !ro || !r || !nneighpn || !jpnlist || ntrial < 0 || (ntrial && (!ip || !rotm || !rtm || !du_twob ||
                                                                               !lhsoverlap)))
        return MG_ERR_ARG;
    if (ntrial == 0) return MG_OK;
    if (!c->d_r2atat) return poly_fail(c, MG_ERR_STATE, "mg_poly_params.r2atat was not given");
    const mg_poly_params &p = c->p;
    int np = p.np;
    std::vector<int> atom0(ntrial);
    int tot = 0;
    for (int t = 0; t < ntrial; ++t) {
        if (ip[t] < 1 || ip[t] > np) return poly_fail(c, MG_ERR_ARG, "ip(%d) = %d", t + 1, ip[t]);
        atom0[t] = tot;
        tot += p.napt[p.iptpn[ip[t] - 1] - 1];
    }
    for (int i = 0; i < np; ++i)
        if (nneighpn[i] < 0 || nneighpn[i] > c->maxnneigh)
            return poly_fail(c, MG_ERR_NEIGH_OVERFLOW, "nneighpn(%d) = %d > maxnneigh %d", i + 1, nneighpn[i],
                             c->maxnneigh);
    if (ntrial > c->tcap) {
        void *q[] = {c->d_tip, c->d_tatom0, c->d_tovl, c->d_trotm, c->d_tdu};
        for (void *x : q)
            if (x) cudaFree(x);
        c->d_tip = c->d_tatom0 = c->d_tovl = nullptr;
        c->d_trotm = c->d_tdu = nullptr;
        POLY_CUDA(c, cudaMalloc(&c->d_tip, sizeof(int) * ntrial));
        POLY_CUDA(c, cudaMalloc(&c->d_tatom0, sizeof(int) * ntrial));
        POLY_CUDA(c, cudaMalloc(&c->d_tovl, sizeof(int) * ntrial));
        POLY_CUDA(c, cudaMalloc(&c->d_trotm, sizeof(double) * 3 * ntrial));
        POLY_CUDA(c, cudaMalloc(&c->d_tdu, sizeof(double) * ntrial));
        c->tcap = ntrial;
    }
    if (tot > c->tacap) {
        if (c->d_trtm) cudaFree(c->d_trtm);
        c->d_trtm = nullptr;
        POLY_CUDA(c, cudaMalloc(&c->d_trtm, sizeof(double) * 3 * tot));
        c->tacap = tot;
    }
    POLY_CUDA(c, cudaMemcpy(c->d_ro, ro, sizeof(double) * 3 * np, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_r, r, sizeof(double) * 3 * p.na, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_nneigh, nneighpn, sizeof(int) * np, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_jpnlist, jpnlist, sizeof(int) * (size_t)c->maxnneigh * np, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_tip, ip, sizeof(int) * ntrial, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_tatom0, atom0.data(), sizeof(int) * ntrial, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_trotm, rotm, sizeof(double) * 3 * ntrial, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_trtm, rtm, sizeof(double) * 3 * tot, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemset(c->d_err, 0, sizeof(int) * 4));
    PolyArgs a = poly_args(c);
    int threads = 128, blocks = (int)(((long)ntrial * 32 + threads - 1) / threads);
    k_poly_dutwobody<<<blocks, threads>>>(a, ntrial, c->d_tip, c->d_trotm, c->d_trtm, c->d_tatom0, c->d_tdu,
                                          c->d_tovl);
    POLY_CUDA(c, cudaGetLastError());
    int herr[4];
    POLY_CUDA(c, cudaMemcpy(herr, c->d_err, sizeof herr, cudaMemcpyDeviceToHost));
    if (herr[0] == MG_ERR_TABLE_UNDERRUN)
        return poly_fail(c, herr[0], "current state: r2 < r2umin for atoms %d and %d", herr[1], herr[2]);
    if (herr[0]) return poly_fail(c, herr[0], "ibuf > nbuf for atom-type pair %d", herr[1]);
    POLY_CUDA(c, cudaMemcpy(du_twob, c->d_tdu, sizeof(double) * ntrial, cudaMemcpyDeviceToHost));
    POLY_CUDA(c, cudaMemcpy(lhsoverlap, c->d_tovl, sizeof(int) * ntrial, cudaMemcpyDeviceToHost));
    return MG_OK;
}

namespace {
int dip_scratch(mg_poly *c);
}

extern "C" int mg_poly_epilogue(mg_poly *c, const double *ro, const double *r, const double *force,
                                const double *torque, double force_fac, double *forceo, double *torqueo,
                                double *virmolecule) {
    if (!c || !ro || !r || !force || !forceo || !torqueo || !virmolecule) return MG_ERR_ARG;
    const mg_poly_params &p = c->p;
    if (!c->d_fo) {
        POLY_CUDA(c, cudaMalloc(&c->d_fo, sizeof(double) * 3 * p.np));
        POLY_CUDA(c, cudaMalloc(&c->d_to, sizeof(double) * 3 * p.np));
    }
    POLY_CUDA(c, cudaMemcpy(c->d_ro, ro, sizeof(double) * 3 * p.np, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_r, r, sizeof(double) * 3 * p.na, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_force, force, sizeof(double) * 3 * p.na, cudaMemcpyHostToDevice));
    double *d_tqa = nullptr;
    if (torque) {   // the atom torques go through the dipole scratch's torque slot
        MG_TRY(dip_scratch(c));
        d_tqa = c->d_dscr + 16 * (size_t)p.na;
        POLY_CUDA(c, cudaMemcpy(d_tqa, torque, sizeof(double) * 3 * p.na, cudaMemcpyHostToDevice));
    }
    PolyArgs a = poly_args(c);
    k_poly_epilogue<<<c->nblk, kPolyThreads>>>(a, force_fac, c->d_fo, c->d_to, d_tqa);
    POLY_CUDA(c, cudaGetLastError());
    POLY_CUDA(c, cudaMemcpy(forceo, c->d_fo, sizeof(double) * 3 * p.np, cudaMemcpyDeviceToHost));
    POLY_CUDA(c, cudaMemcpy(torqueo, c->d_to, sizeof(double) * 3 * p.np, cudaMemcpyDeviceToHost));
    POLY_CUDA(c, cudaMemcpy(c->h_part.data(), c->d_part, sizeof(double) * c->nblk, cudaMemcpyDeviceToHost));
    double v = 0.0;
    for (int b = 0; b < c->nblk; ++b) v += c->h_part[b];
    *virmolecule = v;
    return MG_OK;
}

extern "C" int mg_poly_utwobody_list(mg_poly *c, mg_handle *h, const double *r, double *force, double *u_twob,
                                     double *virial) {
    if (!c || !h || !r || !force || !u_twob || !virial) return MG_ERR_ARG;
    const mg_poly_params &p = c->p;
    if (h->np != p.np) return poly_fail(c, MG_ERR_ARG, "the centres handle holds %d particles, not %d", h->np, p.np);
    if (!h->list_valid) return poly_fail(c, MG_ERR_STATE, "the centres handle has no list (mg_nlist_set)");
    // after mg_nlist_update the list holds every pair within the handle's
    // rcut (pairs beyond it may have moved in unnoticed within the skin)
    if (!(h->rcut >= p.rcut))
        return poly_fail(c, MG_ERR_ARG, "the centres handle's rcut %g is below the pair cutoff %g", h->rcut, p.rcut);
    // a pending device error of the handle (mg_nlist_set and mg_nlist_update
    // drop a list whose build failed, so an overflowed list never gets here)
    if (mg_check_device_error(h) != MG_OK)
        return poly_fail(c, MG_ERR_STATE, "the centres handle reports an error: %s", h->err.c_str());
    for (int m = 0; m < 3; ++m)
        if (h->boxlen[m] != p.boxlen[m]) return poly_fail(c, MG_ERR_ARG, "the centres handle has another box");
    POLY_CUDA(c, cudaStreamSynchronize(h->st));
    POLY_CUDA(c, cudaMemcpy(c->d_r, r, sizeof(double) * 3 * p.na, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemset(c->d_err, 0, sizeof(int) * 4));
    PolyArgs a = poly_args(c);
    a.ro = h->d_ro;
    size_t sm = sizeof(double) * (p.nptpt + 1) * kPolyThreads;
    k_twobody_p_list<<<c->nblk_w, kPolyThreads, sm>>>(a, h->d_perm, h->d_nnb, h->d_nbr);
    POLY_CUDA(c, cudaGetLastError());
    int herr[4];
    POLY_CUDA(c, cudaMemcpy(herr, c->d_err, sizeof herr, cudaMemcpyDeviceToHost));
    if (herr[0] == MG_ERR_TABLE_UNDERRUN)
        return poly_fail(c, herr[0], "r2 < r2umin for atoms %d and %d (atom-type pair %d)", herr[1], herr[2], herr[3]);
    if (herr[0]) return poly_fail(c, herr[0], "ibuf > nbuf for atom-type pair %d", herr[1]);
    POLY_CUDA(c, cudaMemcpy(force, c->d_force, sizeof(double) * 3 * p.na, cudaMemcpyDeviceToHost));
    POLY_CUDA(c, cudaMemcpy(c->h_part.data(), c->d_part, sizeof(double) * c->h_part.size(), cudaMemcpyDeviceToHost));
    int nv = p.nptpt + 1;
    double tot = 0.0, vir = 0.0;
    for (int k = 0; k < p.nptpt; ++k) {
        double sum = 0.0;
        for (int b = 0; b < c->nblk_w; ++b) sum += c->h_part[(size_t)b * nv + k];
        u_twob[k + 1] = sum;
    }
    for (int k = 1; k <= p.nptpt; ++k) tot += u_twob[k];
    u_twob[0] = tot;
    for (int b = 0; b < c->nblk_w; ++b) vir += c->h_part[(size_t)b * nv + p.nptpt];
    *virial = vir;
    return MG_OK;
}

// ---- rigid-body velocity Verlet (VelVer, md.F90:252-420, lpolyatom) -------------
// Positions and quaternions advance from the velocities and accelerations
// of the last step; after UTotal the linear velocities take the new forces
// (GetLinAcc, md.F90:601-617) and the quaternion velocities are iterated
// nvvite times from a trial tvvite * tstep * the old acceleration
// (QuaVelToAngVel mollib.F90:2651-2669, GetAngAcc md.F90:628-663).  The
// arithmetic follows the reference's expressions.
namespace {

// rigid-body state per particle: [0,3) ro, [3,7) qua, [7,10) rod, [10,13) rodd,
// [13,17) quad, [17,21) quadd, [21,24) massip, [24,27) momp, [27,30) momip,
// [30,33) angvelo
constexpr int kRig = 33;

__device__ void rig_qua_to_ori(const double *q, double *ori) {   // QuaToOri, ori(3,3) column-major
    double q00 = q[0] * q[0], q11 = q[1] * q[1], q22 = q[2] * q[2], q33 = q[3] * q[3];
    double q01 = q[0] * q[1], q02 = q[0] * q[2], q03 = q[0] * q[3];
    double q12 = q[1] * q[2], q13 = q[1] * q[3], q23 = q[2] * q[3];
    ori[0] = -q22 + q11 - q33 + q00;
    ori[1] = 2.0 * (q03 - q12);
    ori[2] = 2.0 * (q13 + q02);
    ori[3] = -2.0 * (q12 + q03);
    ori[4] = q22 - q11 - q33 + q00;
    ori[5] = 2.0 * (q01 - q23);
    ori[6] = 2.0 * (q13 - q02);
    ori[7] = -2.0 * (q23 + q01);
    ori[8] = -q22 - q11 + q33 + q00;
}

// GetAngAcc for one particle: quaternion acceleration from the torque
// (lab frame) and the angular velocity (principal frame)
__device__ void rig_ang_acc(const double *q, const double *qd, const double *tq, const double *w,
                            const double *momp, const double *momip, double *qdd) {
    double ori[9];
    rig_qua_to_ori(q, ori);
    double t1 = tq[0] * ori[0] + tq[1] * ori[1] + tq[2] * ori[2];
    double t2 = tq[0] * ori[3] + tq[1] * ori[4] + tq[2] * ori[5];
    double t3 = tq[0] * ori[6] + tq[1] * ori[7] + tq[2] * ori[8];
    double a1 = (t1 + w[1] * w[2] * (momp[1] - momp[2])) * momip[0];
    double a2 = (t2 + w[2] * w[0] * (momp[2] - momp[0])) * momip[1];
    double a3 = (t3 + w[0] * w[1] * (momp[0] - momp[1])) * momip[2];
    double fac = -2.0 * (qd[2] * qd[2] + qd[1] * qd[1] + qd[3] * qd[3] + qd[0] * qd[0]);
    qdd[0] = 0.5 * (-q[1] * a1 + q[2] * a2 - q[3] * a3 + q[0] * fac);
    qdd[1] = 0.5 * (+q[0] * a1 - q[3] * a2 - q[2] * a3 + q[1] * fac);
    qdd[2] = 0.5 * (-q[3] * a1 - q[0] * a2 + q[1] * a3 + q[2] * fac);
    qdd[3] = 0.5 * (+q[2] * a1 + q[1] * a2 + q[0] * a3 + q[3] * fac);
}

__device__ void rig_angvel(const double *q, const double *qd, double *w) {   // QuaVelToAngVel
    w[0] = 2.0 * (-q[3] * qd[2] + q[0] * qd[1] + q[2] * qd[3] - q[1] * qd[0]);
    w[1] = 2.0 * (-q[0] * qd[2] - q[3] * qd[1] + q[1] * qd[3] + q[2] * qd[0]);
    w[2] = 2.0 * (+q[1] * qd[2] - q[2] * qd[1] + q[0] * qd[3] - q[3] * qd[0]);
}

// set-up: quaternion velocities from the angular velocities
// (AngVelToQuaVel mollib.F90:2621-2642)
__global__ void k_rigid_setup(int np, double *__restrict__ rig) {
    int ip = blockIdx.x * blockDim.x + threadIdx.x;
    if (ip >= np) return;
    double *g = rig + (size_t)kRig * ip;
    const double *q = g + 3, *w = g + 30;
    double *qd = g + 13;
    qd[0] = 0.5 * (-q[1] * w[0] + q[2] * w[1] - q[3] * w[2]);
    qd[1] = 0.5 * (+q[0] * w[0] - q[3] * w[1] - q[2] * w[2]);
    qd[2] = 0.5 * (-q[3] * w[0] - q[0] * w[1] + q[1] * w[2]);
    qd[3] = 0.5 * (+q[2] * w[0] + q[1] * w[1] + q[0] * w[2]);
}

// VelVer's first part: new positions (PBC) and quaternions (QuaNorm), the
// orientation matrices (QuaToOri) and drostep
__global__ void k_rigid_move(int np, double tstep, mg_box box, double *__restrict__ rig, double *__restrict__ ro,
                             double *__restrict__ ori, double *__restrict__ drostep) {
    int ip = blockIdx.x * blockDim.x + threadIdx.x;
    if (ip >= np) return;
    double *g = rig + (size_t)kRig * ip;
    double fac = 0.5 * (tstep * tstep);
    for (int m = 0; m < 3; ++m) {
        double d = tstep * g[7 + m] + fac * g[10 + m];
        double x = g[m] + d;
        if (fabs(x) > box.half[m]) x = x - box.len[m] * round(x * box.inv[m]);   // PBC (anint)
        g[m] = x;
        ro[3 * ip + m] = x;
        drostep[3 * ip + m] = d;
    }
    double *q = g + 3;
    for (int k = 0; k < 4; ++k) q[k] = q[k] + tstep * g[13 + k] + fac * g[17 + k];
    double norm = 1.0 / sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    for (int k = 0; k < 4; ++k) q[k] = q[k] * norm;
    rig_qua_to_ori(q, ori + 9 * (size_t)ip);
}

// VelVer's second part, after UTotal
__global__ void k_rigid_kick(int np, double tstep, double tvvite, int nvvite, double *__restrict__ rig,
                             const double *__restrict__ forceo, const double *__restrict__ torqueo,
                             double *__restrict__ rod, double *__restrict__ angvelo) {
    int ip = blockIdx.x * blockDim.x + threadIdx.x;
    if (ip >= np) return;
    double *g = rig + (size_t)kRig * ip;
    for (int m = 0; m < 3; ++m) {
        double roddo = g[10 + m];
        g[10 + m] = g[21] * forceo[3 * ip + m];
        g[7 + m] = g[7 + m] + (0.5 * tstep) * (g[10 + m] + roddo);
        rod[3 * ip + m] = g[7 + m];
    }
    double *q = g + 3, *qd = g + 13, *qdd = g + 17, *w = g + 30;
    double qddo[4], qdo[4];
    for (int k = 0; k < 4; ++k) {
        qddo[k] = qdd[k];
        qdo[k] = qd[k];
        qd[k] = qdo[k] + (tvvite * tstep) * qddo[k];
    }
    // angvelo is that of the last iteration's trial quad, as in the
    // reference (QuaVelToAngVel precedes each GetAngAcc)
    for (int it = 0; it < nvvite; ++it) {
        rig_angvel(q, qd, w);
        rig_ang_acc(q, qd, torqueo + 3 * ip, w, g + 24, g + 27, qdd);
        for (int k = 0; k < 4; ++k) qd[k] = qdo[k] + (0.5 * tstep) * (qdd[k] + qddo[k]);
    }
    for (int m = 0; m < 3; ++m) angvelo[3 * ip + m] = w[m];
}

}  // namespace

extern "C" int mg_poly_rigid_setup(mg_poly *c, double tstep, double tvvite, int32_t nvvite, const double *massip,
                                   const double *momp, const double *ro, const double *qua, const double *rod,
                                   const double *angvelo, const double *rodd, const double *quadd) {
    if (!c || !massip || !momp || !ro || !qua || !rod || !angvelo || !rodd || !quadd) return MG_ERR_ARG;
    if (!(tstep > 0.0) || nvvite < 0) return poly_fail(c, MG_ERR_ARG, "tstep must be > 0 and nvvite >= 0");
    int np = c->p.np;
    std::vector<double> h((size_t)kRig * np, 0.0);
    for (int ip = 0; ip < np; ++ip) {
        double *g = h.data() + (size_t)kRig * ip;
        for (int m = 0; m < 3; ++m) {
            g[m] = ro[3 * ip + m];
            g[7 + m] = rod[3 * ip + m];
            g[10 + m] = rodd[3 * ip + m];
            g[21 + m] = massip[ip];
            g[24 + m] = momp[3 * ip + m];
            g[27 + m] = momp[3 * ip + m] > 0.0 ? 1.0 / momp[3 * ip + m] : 0.0;   // InvFlt
            g[30 + m] = angvelo[3 * ip + m];
        }
        for (int k = 0; k < 4; ++k) {
            g[3 + k] = qua[4 * ip + k];
            g[17 + k] = quadd[4 * ip + k];
        }
    }
    if (!c->d_rig) POLY_CUDA(c, cudaMalloc(&c->d_rig, sizeof(double) * h.size()));
    if (!c->d_rig_io) POLY_CUDA(c, cudaMalloc(&c->d_rig_io, sizeof(double) * 15 * (size_t)np));
    POLY_CUDA(c, cudaMemcpy(c->d_rig, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice));
    k_rigid_setup<<<(np + 127) / 128, 128>>>(np, c->d_rig);
    POLY_CUDA(c, cudaGetLastError());
    POLY_CUDA(c, cudaDeviceSynchronize());
    c->rig_tstep = tstep;
    c->rig_tvvite = tvvite;
    c->rig_nvvite = nvvite;
    return MG_OK;
}

extern "C" int mg_poly_rigid_move(mg_poly *c, double *ro, double *ori, double *drostep) {
    if (!c || !ro || !ori || !drostep) return MG_ERR_ARG;
    if (!c->d_rig) return poly_fail(c, MG_ERR_STATE, "mg_poly_rigid_setup has not been called");
    int np = c->p.np;
    mg_box box;
    for (int m = 0; m < 3; ++m) {
        box.len[m] = c->p.boxlen[m];
        box.half[m] = 0.5 * c->p.boxlen[m];
        box.inv[m] = 1.0 / c->p.boxlen[m];
    }
    double *io = c->d_rig_io;   // ro, ori, drostep
    k_rigid_move<<<(np + 127) / 128, 128>>>(np, c->rig_tstep, box, c->d_rig, io, io + 3 * np, io + 12 * np);
    POLY_CUDA(c, cudaGetLastError());
    POLY_CUDA(c, cudaMemcpy(ro, io, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost));
    POLY_CUDA(c, cudaMemcpy(ori, io + 3 * np, sizeof(double) * 9 * np, cudaMemcpyDeviceToHost));
    POLY_CUDA(c, cudaMemcpy(drostep, io + 12 * np, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost));
    return MG_OK;
}

extern "C" int mg_poly_rigid_kick(mg_poly *c, const double *forceo, const double *torqueo, double *rod,
                                  double *angvelo) {
    if (!c || !forceo || !torqueo || !rod || !angvelo) return MG_ERR_ARG;
    if (!c->d_rig) return poly_fail(c, MG_ERR_STATE, "mg_poly_rigid_setup has not been called");
    int np = c->p.np;
    double *io = c->d_rig_io;   // forceo, torqueo, rod, angvelo
    POLY_CUDA(c, cudaMemcpy(io, forceo, sizeof(double) * 3 * np, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(io + 3 * np, torqueo, sizeof(double) * 3 * np, cudaMemcpyHostToDevice));
    k_rigid_kick<<<(np + 127) / 128, 128>>>(np, c->rig_tstep, c->rig_tvvite, c->rig_nvvite, c->d_rig, io,
                                           io + 3 * np, io + 6 * np, io + 9 * np);
    POLY_CUDA(c, cudaGetLastError());
    POLY_CUDA(c, cudaMemcpy(rod, io + 6 * np, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost));
    POLY_CUDA(c, cudaMemcpy(angvelo, io + 9 * np, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost));
    return MG_OK;
}

extern "C" int mg_poly_rigid_prime(mg_poly *c, const double *forceo, const double *torqueo) {
    if (!c || !forceo || !torqueo) return MG_ERR_ARG;
    if (!c->d_rig) return poly_fail(c, MG_ERR_STATE, "mg_poly_rigid_setup has not been called");
    int np = c->p.np;
    double *io = c->d_rig_io;   // forceo, torqueo; rod, angvelo are written and not read back
    POLY_CUDA(c, cudaMemcpy(io, forceo, sizeof(double) * 3 * np, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(io + 3 * np, torqueo, sizeof(double) * 3 * np, cudaMemcpyHostToDevice));
    // a kick of zero length: rod and quad stay, rodd and quadd are those of
    // the current state
    k_rigid_kick<<<(np + 127) / 128, 128>>>(np, 0.0, 0.0, c->rig_nvvite > 0 ? c->rig_nvvite : 1, c->d_rig, io,
                                           io + 3 * np, io + 6 * np, io + 9 * np);
    POLY_CUDA(c, cudaGetLastError());
    POLY_CUDA(c, cudaDeviceSynchronize());
    return MG_OK;
}

extern "C" int mg_poly_rigid_get(mg_poly *c, double *qua, double *quad) {
    if (!c || !qua || !quad) return MG_ERR_ARG;
    if (!c->d_rig) return poly_fail(c, MG_ERR_STATE, "mg_poly_rigid_setup has not been called");
    int np = c->p.np;
    std::vector<double> h((size_t)kRig * np);
    POLY_CUDA(c, cudaMemcpy(h.data(), c->d_rig, sizeof(double) * h.size(), cudaMemcpyDeviceToHost));
    for (int ip = 0; ip < np; ++ip)
        for (int k = 0; k < 4; ++k) {
            qua[4 * ip + k] = h[(size_t)kRig * ip + 3 + k];
            quad[4 * ip + k] = h[(size_t)kRig * ip + 13 + k];
        }
    return MG_OK;
}

// ---- charges and point dipoles ---------------------------------------------------
// The arrays potstat[na], estat[3 na], efg[6 na] travel with every call, as
// the reference's module arrays; the device keeps no state between calls.
namespace {

int dip_scratch(mg_poly *c) {
    if (c->d_dscr) return MG_OK;
    POLY_CUDA(c, cudaMalloc(&c->d_dscr, sizeof(double) * (19 * (size_t)c->p.na + 8)));
    POLY_CUDA(c, cudaMalloc(&c->d_dfx, sizeof(long long) * 10 * (size_t)c->p.na));
    return MG_OK;
}

DipArgs dip_args(mg_poly *c) {
    const mg_poly_params &p = c->p;
    size_t na = (size_t)p.na;
    DipArgs q = {};
    q.az = c->d_aza;
    q.dip = c->d_dscr;
    q.pot = c->d_dscr + 3 * na;
    q.est = q.pot + na;
    q.efg = q.est + 3 * na;
    q.fx = c->d_dfx;
    q.na = p.na;
    q.err = c->d_err;
    q.ualpha = p.ualpha;
    q.ualpha2 = p.ualpha * p.ualpha;
    q.lewald = p.ualpha > 0.0;
    if (q.lewald) {   // EwaldSetup, energy.F90:7040-7044
        double fac = 1.0 / (std::sqrt(3.1415926535897932) * p.ualpha);
        q.f1 = fac * 2.0 * q.ualpha2;
        q.f2 = fac * (2.0 * q.ualpha2) * (2.0 * q.ualpha2) / 3.0;
        q.f3 = fac * (2.0 * q.ualpha2) * (2.0 * q.ualpha2) * (2.0 * q.ualpha2) / 15.0;
    }
    return q;
}

int dip_copy(mg_poly *c, const DipArgs &q, const double *pot, const double *est, const double *efg,
             cudaMemcpyKind kind, double *hpot, double *hest, double *hefg) {
    size_t na = (size_t)c->p.na;
    if (kind == cudaMemcpyHostToDevice) {
        POLY_CUDA(c, cudaMemcpy(q.pot, pot, sizeof(double) * na, kind));
        POLY_CUDA(c, cudaMemcpy(q.est, est, sizeof(double) * 3 * na, kind));
        POLY_CUDA(c, cudaMemcpy(q.efg, efg, sizeof(double) * 6 * na, kind));
    } else {
        POLY_CUDA(c, cudaMemcpy(hpot, q.pot, sizeof(double) * na, kind));
        POLY_CUDA(c, cudaMemcpy(hest, q.est, sizeof(double) * 3 * na, kind));
        POLY_CUDA(c, cudaMemcpy(hefg, q.efg, sizeof(double) * 6 * na, kind));
    }
    return MG_OK;
}

// sum of q pot - dip . e over the atoms (block partials in order)
int dip_usum(mg_poly *c, const DipArgs &q, double *out) {
    int na = c->p.na, nb = (na + kPolyThreads - 1) / kPolyThreads;
    k_dipole_finish<<<nb, kPolyThreads>>>(na, q, 0.0, nullptr, nullptr, c->d_part);
    POLY_CUDA(c, cudaGetLastError());
    POLY_CUDA(c, cudaMemcpy(c->h_part.data(), c->d_part, sizeof(double) * nb, cudaMemcpyDeviceToHost));
    double u = 0.0;
    for (int b = 0; b < nb; ++b) u += c->h_part[b];
    *out = u;
    return MG_OK;
}

}  // namespace

extern "C" int mg_poly_udipole_real(mg_poly *c, const double *ro, const double *r, const double *dip,
                                    const int32_t *nneighpn, const int32_t *jpnlist, double *potstat, double *estat,
                                    double *efg, double *virelec, double *u_real) {
    if (!c || !ro || !r || !dip || !nneighpn || !jpnlist || !potstat || !estat || !efg || !virelec || !u_real)
        return MG_ERR_ARG;
    if (!c->d_aza) return poly_fail(c, MG_ERR_STATE, "mg_poly_params.aza (atom charges) was not given");
    const mg_poly_params &p = c->p;
    for (int i = 0; i < p.np; ++i)
        if (nneighpn[i] < 0 || nneighpn[i] > c->maxnneigh)
            return poly_fail(c, MG_ERR_NEIGH_OVERFLOW, "nneighpn(%d) = %d > maxnneigh %d", i + 1, nneighpn[i],
                             c->maxnneigh);
    MG_TRY(dip_scratch(c));
    DipArgs q = dip_args(c);
    size_t na = (size_t)p.na;
    POLY_CUDA(c, cudaMemcpy(c->d_ro, ro, sizeof(double) * 3 * p.np, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_r, r, sizeof(double) * 3 * na, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_dscr, dip, sizeof(double) * 3 * na, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_nneigh, nneighpn, sizeof(int) * p.np, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_jpnlist, jpnlist, sizeof(int) * (size_t)c->maxnneigh * p.np, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemset(q.fx, 0, sizeof(long long) * 10 * na));   // pot, est, efg
    POLY_CUDA(c, cudaMemset(c->d_err, 0, sizeof(int) * 4));
    PolyArgs a = poly_args(c);
    k_dipole_real<<<c->nblk_w, kPolyThreads>>>(a, q);
    k_dip_fx_out<<<(unsigned)((10 * na + 255) / 256), 256>>>(q.fx, 10 * na, q.pot);
    POLY_CUDA(c, cudaGetLastError());
    int herr[4];
    POLY_CUDA(c, cudaMemcpy(herr, c->d_err, sizeof herr, cudaMemcpyDeviceToHost));
    if (herr[0])
        return poly_fail(c, herr[0], "an atom potential, field or field gradient beyond the fixed-point range (8.4e6)");
    POLY_CUDA(c, cudaMemcpy(c->h_part.data(), c->d_part, sizeof(double) * c->nblk_w, cudaMemcpyDeviceToHost));
    double vir = 0.0;
    for (int b = 0; b < c->nblk_w; ++b) vir += c->h_part[b];
    double u = 0.0;
    MG_TRY(dip_usum(c, q, &u));
    MG_TRY(dip_copy(c, q, nullptr, nullptr, nullptr, cudaMemcpyDeviceToHost, potstat, estat, efg));
    *virelec = vir;
    *u_real = p.epsi_four_pi * 0.5 * u;
    return MG_OK;
}

extern "C" int mg_poly_udipole_self(mg_poly *c, const double *r, const double *dip, int32_t lsurf, double *potstat,
                                    double *estat, double *efg, double *virelec) {
    if (!c || !r || !dip || !potstat || !estat || !efg || !virelec) return MG_ERR_ARG;
    if (!c->d_aza) return poly_fail(c, MG_ERR_STATE, "mg_poly_params.aza (atom charges) was not given");
    const mg_poly_params &p = c->p;
    if (!(p.ualpha > 0.0)) return poly_fail(c, MG_ERR_STATE, "the Ewald self terms need ualpha > 0");
    MG_TRY(dip_scratch(c));
    DipArgs q = dip_args(c);
    size_t na = (size_t)p.na;
    POLY_CUDA(c, cudaMemcpy(c->d_r, r, sizeof(double) * 3 * na, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(c->d_dscr, dip, sizeof(double) * 3 * na, cudaMemcpyHostToDevice));
    MG_TRY(dip_copy(c, q, potstat, estat, efg, cudaMemcpyHostToDevice, nullptr, nullptr, nullptr));
    PolyArgs a = poly_args(c);
    k_dipole_intra<<<c->nblk, kPolyThreads>>>(a, q);
    POLY_CUDA(c, cudaGetLastError());
    POLY_CUDA(c, cudaMemcpy(c->h_part.data(), c->d_part, sizeof(double) * c->nblk, cudaMemcpyDeviceToHost));
    double vir = *virelec;
    for (int b = 0; b < c->nblk; ++b) vir += c->h_part[b];
    if (lsurf) {
        double *s6 = c->d_dscr + 19 * na;
        double vol = p.boxlen[0] * p.boxlen[1] * p.boxlen[2];
        double fac = (4.0 * 3.1415926535897932 / 3.0) / vol;
        k_dipole_surf_sums<<<1, 1024>>>(p.na, q, c->d_r, s6);
        k_dipole_surf_apply<<<(p.na + 127) / 128, 128>>>(p.na, q, c->d_r, s6, fac);
        POLY_CUDA(c, cudaGetLastError());
        double h6[6];
        POLY_CUDA(c, cudaMemcpy(h6, s6, sizeof h6, cudaMemcpyDeviceToHost));
        double qq = h6[0] * h6[0] + h6[1] * h6[1] + h6[2] * h6[2];
        double qd = h6[0] * h6[3] + h6[1] * h6[4] + h6[2] * h6[5];
        double dd = h6[3] * h6[3] + h6[4] * h6[4] + h6[5] * h6[5];
        vir = vir - 2.0 * 3.1415926535897932 / (3.0 * vol) * (qq + 2.0 * (2.0 * qd) + 3.0 * dd);
    }
    MG_TRY(dip_copy(c, q, nullptr, nullptr, nullptr, cudaMemcpyDeviceToHost, potstat, estat, efg));
    *virelec = vir;
    return MG_OK;
}

extern "C" int mg_poly_udipole_finish(mg_poly *c, const double *dip, const double *potstat, const double *estat,
                                      const double *efg, double *force, double *torque, double *u_stat) {
    if (!c || !dip || !potstat || !estat || !efg || !force || !torque || !u_stat) return MG_ERR_ARG;
    if (!c->d_aza) return poly_fail(c, MG_ERR_STATE, "mg_poly_params.aza (atom charges) was not given");
    const mg_poly_params &p = c->p;
    MG_TRY(dip_scratch(c));
    DipArgs q = dip_args(c);
    size_t na = (size_t)p.na;
    double *d_f = q.efg + 6 * na, *d_t = d_f + 3 * na;
    POLY_CUDA(c, cudaMemcpy(c->d_dscr, dip, sizeof(double) * 3 * na, cudaMemcpyHostToDevice));
    MG_TRY(dip_copy(c, q, potstat, estat, efg, cudaMemcpyHostToDevice, nullptr, nullptr, nullptr));
    POLY_CUDA(c, cudaMemcpy(d_f, force, sizeof(double) * 3 * na, cudaMemcpyHostToDevice));
    POLY_CUDA(c, cudaMemcpy(d_t, torque, sizeof(double) * 3 * na, cudaMemcpyHostToDevice));
    int nb = (p.na + kPolyThreads - 1) / kPolyThreads;
    k_dipole_finish<<<nb, kPolyThreads>>>(p.na, q, p.epsi_four_pi, d_f, d_t, c->d_part);
    POLY_CUDA(c, cudaGetLastError());
    POLY_CUDA(c, cudaMemcpy(c->h_part.data(), c->d_part, sizeof(double) * nb, cudaMemcpyDeviceToHost));
    double u = 0.0;
    for (int b = 0; b < nb; ++b) u += c->h_part[b];
    POLY_CUDA(c, cudaMemcpy(force, d_f, sizeof(double) * 3 * na, cudaMemcpyDeviceToHost));
    POLY_CUDA(c, cudaMemcpy(torque, d_t, sizeof(double) * 3 * na, cudaMemcpyDeviceToHost));
    *u_stat = p.epsi_four_pi * 0.5 * u;
    return MG_OK;
}

// ---- rigid-body MD of polyatomic particles on the device ------------------------
// VelVer with lpolyatom (md.F90:252-420) step after step without the host:
// move (centres, quaternions, orientations), atom placement (SetAtomProp:
// r = ro + ori ra, molaux.F90:540-560), the centres' list rebuilt, the atom
// pairs over it (UTwoBodyP), with Ewald the atoms' reciprocal sum and
// atomic self term through the atom handle and the molecular self term,
// UTotal's end (forces and torques of the particles), kick.
namespace {

// r = ro + ori ra for every atom (ori(3,3,np) column-major, ra the local
// positions by particle type, atoms of a type consecutive from ra_off[type])
__global__ void k_place_atoms(int np, const int *__restrict__ iptpn, const int *__restrict__ ianpn,
                              const int *__restrict__ napt, const int *__restrict__ ra_off,
                              const double *__restrict__ ra, const double *__restrict__ ro,
                              const double *__restrict__ ori, double *__restrict__ r) {
    int ip = blockIdx.x * blockDim.x + threadIdx.x;
    if (ip >= np) return;
    int t = iptpn[ip] - 1, a0 = ianpn[ip] - 1, na = napt[t];
    const double *o = ori + 9 * (size_t)ip, *c = ro + 3 * (size_t)ip;
    for (int k = 0; k < na; ++k) {
        const double *x = ra + 3 * (size_t)(ra_off[t] + k);
        for (int m = 0; m < 3; ++m)
            r[3 * (size_t)(a0 + k) + m] = c[m] + o[m] * x[0] + o[m + 3] * x[1] + o[m + 6] * x[2];
    }
}

// the atom positions folded into the box for the atom handle (PBC: ANINT)
__global__ void k_fold_atoms(int na, const double *__restrict__ r, mg_box box, double *__restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * na) return;
    int m = i % 3;
    double x = r[i];
    if (fabs(x) > box.half[m]) x -= box.len[m] * round(x * box.inv[m]);
    out[i] = x;
}

__global__ void k_add_scaled(size_t n, const double *__restrict__ x, double f, double *__restrict__ y) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] += f * x[i];
}

}  // namespace

extern "C" int mg_poly_md_run(mg_poly *c, mg_handle *hc, mg_handle *ha, const double *ra, int32_t nstep,
                              double *ro, double *ori, double *rod, double *angvelo, double *uout) {
    if (!c || !hc || !ra || nstep < 1 || !ro || !ori || !rod || !angvelo || !uout) return MG_ERR_ARG;
    const mg_poly_params &p = c->p;
    if (!c->d_rig) return poly_fail(c, MG_ERR_STATE, "mg_poly_rigid_setup has not been called");
    if (hc->np != p.np) return poly_fail(c, MG_ERR_ARG, "the centres handle holds %d particles, not %d", hc->np, p.np);
    if (!hc->list_valid) return poly_fail(c, MG_ERR_STATE, "the centres handle has no list (mg_nlist_set)");
    if (!(hc->rcut >= p.rcut))
        return poly_fail(c, MG_ERR_ARG, "the centres handle's rcut %g is below the pair cutoff %g", hc->rcut, p.rcut);
    for (int m = 0; m < 3; ++m)
        if (hc->boxlen[m] != p.boxlen[m]) return poly_fail(c, MG_ERR_ARG, "the centres handle has another box");
    bool ewald = p.ualpha > 0.0;
    if (ewald) {
        if (!ha || ha->np != p.na || ha->form != MG_FP64 || ha->ewald == MG_EWALD_NONE)
            return poly_fail(c, MG_ERR_ARG, "Ewald needs an FP64 Ewald handle of the %d atoms", p.na);
        if (!c->d_aza) return poly_fail(c, MG_ERR_STATE, "mg_poly_params.aza (atom charges) was not given");
    }
    const int np = p.np, na = p.na;
    // local positions by type, the type offsets
    std::vector<int> off(p.npt + 1, 0);
    for (int t = 0; t < p.npt; ++t) off[t + 1] = off[t] + p.napt[t];
    // scratch: ori 9np, drostep 3np, ra, offsets, per-block partials (intra, epilogue)
    size_t nra = 3 * (size_t)off[p.npt];
    size_t need = 12 * (size_t)np + nra + (size_t)p.npt + 2 * (size_t)c->nblk + 8;
    double *d = nullptr;
    POLY_CUDA(c, cudaMalloc(&d, sizeof(double) * need));
    double *d_ori = d, *d_dro = d_ori + 9 * (size_t)np, *d_ra = d_dro + 3 * (size_t)np;
    int *d_off = reinterpret_cast<int *>(d_ra + nra);
    double *d_pi = d_ra + nra + p.npt, *d_pe = d_pi + c->nblk;
    cudaStream_t S = hc->st;
    cudaEvent_t e1 = nullptr, e2 = nullptr;
    cudaGraphExec_t ge = nullptr;
    int st = MG_OK;
    auto ok = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && st == MG_OK) st = poly_fail(c, MG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
        return st == MG_OK;
    };
    do {
        if (!ok(cudaEventCreateWithFlags(&e1, cudaEventDisableTiming), "event") ||
            !ok(cudaEventCreateWithFlags(&e2, cudaEventDisableTiming), "event") ||
            !ok(cudaMemcpyAsync(d_ra, ra, sizeof(double) * nra, cudaMemcpyHostToDevice, S), "copy ra") ||
            !ok(cudaMemcpyAsync(d_off, off.data(), sizeof(int) * p.npt, cudaMemcpyHostToDevice, S), "copy offsets") ||
            !ok(cudaMemsetAsync(c->d_err, 0, sizeof(int) * 4, S), "clear error"))
            break;
        mg_box box;
        for (int m = 0; m < 3; ++m) {
            box.len[m] = p.boxlen[m];
            box.half[m] = 0.5 * p.boxlen[m];
            box.inv[m] = 1.0 / p.boxlen[m];
        }
        PolyArgs a = poly_args(c);
        a.ro = hc->d_ro;
        size_t sm = sizeof(double) * (p.nptpt + 1) * kPolyThreads;
        double ualpha2 = p.ualpha * p.ualpha;
        double ewaldfac1 = ewald ? (1.0 / (std::sqrt(3.1415926535897932) * p.ualpha)) * 2.0 * ualpha2 : 0.0;
        // one step's launches on S (the atom handle's streams joined by events)
        auto step_launch = [&]() -> bool {
            k_rigid_move<<<(np + 127) / 128, 128, 0, S>>>(np, c->rig_tstep, box, c->d_rig, hc->d_ro, d_ori, d_dro);
            k_place_atoms<<<(np + 127) / 128, 128, 0, S>>>(np, c->d_iptpn, c->d_ianpn, c->d_napt, d_off, d_ra,
                                                         hc->d_ro, d_ori, c->d_r);
            if (!ok(cudaGetLastError(), "move") || mg_lists_build(hc, false) != MG_OK) {
                if (st == MG_OK) st = poly_fail(c, MG_ERR_STATE, "centres list: %s", hc->err.c_str());
                return false;
            }
            k_twobody_p_list<<<c->nblk_w, kPolyThreads, sm, S>>>(a, hc->d_perm, hc->d_nnb, hc->d_nbr);
            if (ewald) {
                k_fold_atoms<<<(3 * na + 255) / 256, 256, 0, S>>>(na, c->d_r, box, ha->d_ro);
                if (!ok(cudaEventRecord(e1, S), "event") || !ok(cudaStreamWaitEvent(ha->st, e1, 0), "wait"))
                    return false;
                if (mg_utotal_launch(ha) != MG_OK) {
                    st = poly_fail(c, MG_ERR_STATE, "atom handle: %s", ha->err.c_str());
                    return false;
                }
                if (!ok(cudaEventRecord(e2, ha->st), "event") || !ok(cudaStreamWaitEvent(S, e2, 0), "wait"))
                    return false;
                k_add_scaled<<<(unsigned)((3 * (size_t)na + 255) / 256), 256, 0, S>>>(
                    3 * (size_t)na, ha->d_forceo, 1.0 / ha->force_fac, c->d_force);
                PolyArgs ai = a;
                ai.part = d_pi;
                k_ewald_intra<<<c->nblk, kPolyThreads, 0, S>>>(ai, c->d_aza, p.ualpha, ualpha2, ewaldfac1,
                                                              p.epsi_four_pi, 1);
            }
            PolyArgs ae = a;
            ae.part = d_pe;
            k_poly_epilogue<<<c->nblk, kPolyThreads, 0, S>>>(ae, hc->force_fac, c->d_fo, c->d_to, nullptr);
            double *io = c->d_rig_io;
            k_rigid_kick<<<(np + 127) / 128, 128, 0, S>>>(np, c->rig_tstep, c->rig_tvvite, c->rig_nvvite, c->d_rig,
                                                         c->d_fo, c->d_to, io, io + 3 * np);
            return ok(cudaGetLastError(), "step kernels");
        };
        // the first step as launched (it also makes any allocation the
        // handles' passes do on first use); the others replay one captured
        // step, so that a step costs one graph launch.  With phase timing on
        // a handle, every step is launched as the first.
        if (!step_launch()) break;
        bool capture = nstep > 1 && !hc->timing && !(ha && ha->timing);
        for (int step = 1; step < nstep && !capture && st == MG_OK; ++step)
            if (!step_launch()) break;
        if (st != MG_OK) break;
        if (capture) {
            cudaGraph_t g = nullptr;
            if (!ok(cudaStreamBeginCapture(S, cudaStreamCaptureModeThreadLocal), "capture")) break;
            bool launched = step_launch();
            cudaError_t ce = cudaStreamEndCapture(S, &g);
            if (!launched || !ok(ce, "capture")) {
                if (g) cudaGraphDestroy(g);
                break;
            }
            ce = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
            if (!ok(ce, "graph instantiate")) break;
            for (int step = 1; step < nstep; ++step)
                if (!ok(cudaGraphLaunch(ge, S), "graph launch")) break;
        }
        if (st != MG_OK) break;
        // the last step's state and energies
        std::vector<double> hp((size_t)c->nblk_w * (p.nptpt + 1)), hi(c->nblk), he(c->nblk),
            hu(ha ? (size_t)ha->nptpt + 5 : 1);
        int herr[4];
        double *io = c->d_rig_io;
        if (!ok(cudaMemcpyAsync(ro, hc->d_ro, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, S), "ro") ||
            !ok(cudaMemcpyAsync(ori, d_ori, sizeof(double) * 9 * np, cudaMemcpyDeviceToHost, S), "ori") ||
            !ok(cudaMemcpyAsync(rod, io, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, S), "rod") ||
            !ok(cudaMemcpyAsync(angvelo, io + 3 * np, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, S), "angvelo") ||
            !ok(cudaMemcpyAsync(hp.data(), c->d_part, sizeof(double) * hp.size(), cudaMemcpyDeviceToHost, S), "part") ||
            !ok(cudaMemcpyAsync(hi.data(), d_pi, sizeof(double) * hi.size(), cudaMemcpyDeviceToHost, S), "part") ||
            !ok(cudaMemcpyAsync(he.data(), d_pe, sizeof(double) * he.size(), cudaMemcpyDeviceToHost, S), "part") ||
            !ok(cudaMemcpyAsync(herr, c->d_err, sizeof herr, cudaMemcpyDeviceToHost, S), "error word"))
            break;
        if (ewald && !ok(cudaMemcpyAsync(hu.data(), ha->d_uout, sizeof(double) * (ha->nptpt + 5),
                                         cudaMemcpyDeviceToHost, S), "energies"))
            break;
        if (!ok(cudaStreamSynchronize(S), "sync")) break;
        if (herr[0] == MG_ERR_TABLE_UNDERRUN) {
            st = poly_fail(c, herr[0], "r2 < r2umin for atoms %d and %d (atom-type pair %d)", herr[1], herr[2], herr[3]);
            break;
        }
        if (herr[0]) {
            st = poly_fail(c, herr[0], "ibuf > nbuf for atom-type pair %d", herr[1]);
            break;
        }
        int nv = p.nptpt + 1;
        double utw = 0.0, vir = 0.0, uin = 0.0, vmol = 0.0;
        for (int k = 0; k < p.nptpt; ++k)
            for (int b = 0; b < c->nblk_w; ++b) utw += hp[(size_t)b * nv + k];
        for (int b = 0; b < c->nblk_w; ++b) vir += hp[(size_t)b * nv + p.nptpt];
        for (int b = 0; b < c->nblk; ++b) vmol += he[b];
        double urec = 0.0;
        if (ewald) {
            for (int b = 0; b < c->nblk; ++b) uin += hi[b];
            int o = ha->nptpt + 1;   // u_tot, u_rec, u_bond, virial of the atom handle
            urec = hu[o + 1] + p.epsi_four_pi * uin;
            vir += hu[o + 3];
        }
        uout[0] = utw + urec;     // u%tot
        uout[1] = utw;            // u%twob(0)
        uout[2] = urec;           // u%rec (atoms' reciprocal and self terms, molecular self term)
        uout[3] = vir + vmol;     // virial (with the molecular term)
    } while (false);
    if (ge) cudaGraphExecDestroy(ge);
    if (e1) cudaEventDestroy(e1);
    if (e2) cudaEventDestroy(e2);
    cudaFree(d);
    return st;
}

// ---- multi-particle polyatomic trials (UTwoBodyPNew/Old, nptm > 1) ------------
namespace {

struct MultiArgs {
    int nptm, nitem_a, npair;
    const int *ipm;       // moving particles (0-based)
    const int *atom0;     // first trial atom of each moving particle in rtm
    const int *item0;     // [nptm + 1] prefix of the moving particles' list lengths
    const int *moving;    // [np] 1 for a moving particle
    const double *rotm, *rtm;
    double *out;          // [2 nptpt + 1]: new sums, old sums (per type pair), the overlap flag
};

// the atom-pair energy of particles ip (centre ci, atoms ra) and jp (centre
// cj, atoms rb); 1: a hard core or a pair below its table, -1 past the
// table; *inr when the centres are within rcut
__device__ int multi_pair(const PolyArgs &a, int ip, const double *ci, const double *ra, int jp, const double *cj,
                          const double *rb, double *usum, int *inr) {
    double sh[3], d[3];
    for (int m = 0; m < 3; ++m) {
        d[m] = __dsub_rn(ci[m], cj[m]);
        sh[m] = fabs(d[m]) > a.half[m] ? copysign(a.len[m], d[m]) : 0.0;
        d[m] = __dsub_rn(d[m], sh[m]);
    }
    *inr = 0;
    if (mg_r2_exact(d[0], d[1], d[2]) > a.rcut2) return 0;
    *inr = 1;
    int ipt = a.iptpn[ip], jpt = a.iptpn[jp];
    int ialow = a.ianpn[ip] - 1, jalow = a.ianpn[jp] - 1;
    double s = 0.0;
    for (int k = 0; k < a.napt[ipt - 1]; ++k) {
        int iat = a.iatan[ialow + k];
        for (int l = 0; l < a.napt[jpt - 1]; ++l) {
            int jat = a.iatan[jalow + l];
            int iatjat = a.iatat[(jat - 1) * a.nat + (iat - 1)];
            double dx = __dsub_rn(__dsub_rn(ra[3 * k], rb[3 * l]), sh[0]);
            double dy = __dsub_rn(__dsub_rn(ra[3 * k + 1], rb[3 * l + 1]), sh[1]);
            double dz = __dsub_rn(__dsub_rn(ra[3 * k + 2], rb[3 * l + 2]), sh[2]);
            double ar2 = mg_r2_exact(dx, dy, dz);
            if (ar2 < a.r2atat[iatjat - 1] || ar2 < a.r2umin[iatjat - 1]) return 1;
            double u;
            if (poly_pair_u(a, iatjat, ar2, &u)) return -1;
            s = __dadd_rn(s, u);
        }
    }
    *usum = s;
    return 0;
}

__global__ void __launch_bounds__(256) k_poly_dutwobody_multi(PolyArgs a, MultiArgs m) {
    __shared__ double red[2 * MG_MAX_NPTPT][8];
    __shared__ int sbad[8];
    double an[MG_MAX_NPTPT], ao[MG_MAX_NPTPT];
#pragma unroll
    for (int k = 0; k < MG_MAX_NPTPT; ++k) an[k] = ao[k] = 0.0;
    int bad = 0;
    const int total = m.nitem_a + m.npair;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int il, jp, jl = -1;
        if (t < m.nitem_a) {   // a moving particle and a list neighbour that stays
            il = 0;
            while (m.item0[il + 1] <= t) ++il;
            int ip = m.ipm[il];
            jp = a.jpnlist[(size_t)ip * a.maxnneigh + (t - m.item0[il])] - 1;
            if (m.moving[jp]) continue;
        } else {               // two moving particles, il < jl
            int q = t - m.nitem_a;
            il = 0;
            while (q >= m.nptm - 1 - il) { q -= m.nptm - 1 - il; ++il; }
            jl = il + 1 + q;
            jp = m.ipm[jl];
        }
        int ip = m.ipm[il];
        int ipt = a.iptpn[ip], jpt = a.iptpn[jp];
        int iptjpt = a.iptpt[(jpt - 1) * a.npt + (ipt - 1)];
        for (int pass = 0; pass < 2; ++pass) {   // 0: trial, 1: current
            const double *ci = pass ? a.ro + 3 * ip : m.rotm + 3 * il;
            const double *ra = pass ? a.r + 3 * (size_t)(a.ianpn[ip] - 1) : m.rtm + 3 * (size_t)m.atom0[il];
            const double *cj, *rb;
            if (jl >= 0 && pass == 0) {
                cj = m.rotm + 3 * jl;
                rb = m.rtm + 3 * (size_t)m.atom0[jl];
            } else {
                cj = a.ro + 3 * jp;
                rb = a.r + 3 * (size_t)(a.ianpn[jp] - 1);
            }
            double u = 0.0;
            int inr, st = multi_pair(a, ip, ci, ra, jp, cj, rb, &u, &inr);
            if (st > 0) {
                if (pass == 0) bad = 1;
                else mg_dev_error(a.err, MG_ERR_TABLE_UNDERRUN, ip + 1, jp + 1, iptjpt);
                continue;
            }
            if (st < 0) {
                mg_dev_error(a.err, MG_ERR_IBUF, iptjpt, ip + 1, jp + 1);
                continue;
            }
            if (!inr) continue;
#pragma unroll
            for (int k = 0; k < MG_MAX_NPTPT; ++k)
                if (k == iptjpt - 1) {
                    if (pass == 0) an[k] = __dadd_rn(an[k], u);
                    else ao[k] = __dadd_rn(ao[k], u);
                }
        }
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < MG_MAX_NPTPT; ++k) {
        double x = an[k], y = ao[k];
        for (int o = 16; o > 0; o >>= 1) {
            x += __shfl_down_sync(0xffffffffu, x, o);
            y += __shfl_down_sync(0xffffffffu, y, o);
        }
        if (lane == 0 && k < a.nptpt) { red[k][w] = x; red[MG_MAX_NPTPT + k][w] = y; }
    }
    for (int o = 16; o > 0; o >>= 1) bad |= __shfl_down_sync(0xffffffffu, bad, o);
    if (lane == 0) sbad[w] = bad;
    __syncthreads();
    if (threadIdx.x < a.nptpt) {
        double x = 0.0, y = 0.0;
        for (int k = 0; k < nw; ++k) { x += red[threadIdx.x][k]; y += red[MG_MAX_NPTPT + threadIdx.x][k]; }
        m.out[threadIdx.x] = x;
        m.out[a.nptpt + threadIdx.x] = y;
    }
    if (threadIdx.x == 0) {
        int b = 0;
        for (int k = 0; k < nw; ++k) b |= sbad[k];
        m.out[2 * a.nptpt] = b;
    }
}

}  // namespace

extern "C" int mg_poly_dutwobody_multi(mg_poly *c, const double *ro, const double *r, const int32_t *nneighpn,
                                       const int32_t *jpnlist, int32_t nptm, const int32_t *ipnptm,
                                       const double *rotm, const double *rtm, double *du_twob, int32_t *lhsoverlap) {
    if (!c || !ro || !r || !nneighpn || !jpnlist || nptm < 1 || !ipnptm || !rotm || !rtm || !du_twob || !lhsoverlap)
        return MG_ERR_ARG;
    if (!c->d_r2atat) return poly_fail(c, MG_ERR_STATE, "mg_poly_params.r2atat was not given");
    const mg_poly_params &p = c->p;
    const int np = p.np, nptpt = p.nptpt;
    if (nptpt > MG_MAX_NPTPT) return poly_fail(c, MG_ERR_UNSUPPORTED, "%d particle-type pairs", nptpt);
    std::vector<int> ipm(nptm), atom0(nptm), item0(nptm + 1, 0), moving(np, 0);
    int tot = 0;
    for (int k = 0; k < nptm; ++k) {
        int ip = ipnptm[k];
        if (ip < 1 || ip > np) return poly_fail(c, MG_ERR_ARG, "ipnptm(%d) = %d", k + 1, ip);
        if (moving[ip - 1]) return poly_fail(c, MG_ERR_ARG, "particle %d moves twice", ip);
        moving[ip - 1] = 1;
        ipm[k] = ip - 1;
        atom0[k] = tot;
        tot += p.napt[p.iptpn[ip - 1] - 1];
        if (nneighpn[ip - 1] < 0 || nneighpn[ip - 1] > c->maxnneigh)
            return poly_fail(c, MG_ERR_NEIGH_OVERFLOW, "nneighpn(%d) = %d > maxnneigh %d", ip, nneighpn[ip - 1],
                             c->maxnneigh);
        item0[k + 1] = item0[k] + nneighpn[ip - 1];
    }
    // scratch: ints (ipm, atom0, item0, moving), doubles (rotm, rtm, out)
    size_t ni = 3 * (size_t)nptm + 1 + np, nd = 3 * (size_t)nptm + 3 * (size_t)tot + 2 * (size_t)nptpt + 1;
    void *d = nullptr;
    POLY_CUDA(c, cudaMalloc(&d, sizeof(double) * nd + sizeof(int) * ni));
    double *d_rotm = (double *)d, *d_rtm = d_rotm + 3 * nptm, *d_out = d_rtm + 3 * (size_t)tot;
    int *d_ipm = (int *)(d_out + 2 * nptpt + 1), *d_atom0 = d_ipm + nptm, *d_item0 = d_atom0 + nptm,
        *d_moving = d_item0 + nptm + 1;
    int st = MG_OK;
    auto cp = [&](void *dst, const void *src, size_t bytes) {
        if (st == MG_OK && cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess)
            st = poly_fail(c, MG_ERR_CUDA, "mg_poly_dutwobody_multi: copy failed");
    };
    cp(c->d_ro, ro, sizeof(double) * 3 * np);
    cp(c->d_r, r, sizeof(double) * 3 * p.na);
    cp(c->d_nneigh, nneighpn, sizeof(int) * np);
    cp(c->d_jpnlist, jpnlist, sizeof(int) * (size_t)c->maxnneigh * np);
    cp(d_rotm, rotm, sizeof(double) * 3 * nptm);
    cp(d_rtm, rtm, sizeof(double) * 3 * tot);
    cp(d_ipm, ipm.data(), sizeof(int) * nptm);
    cp(d_atom0, atom0.data(), sizeof(int) * nptm);
    cp(d_item0, item0.data(), sizeof(int) * (nptm + 1));
    cp(d_moving, moving.data(), sizeof(int) * np);
    std::vector<double> out(2 * (size_t)nptpt + 1);
    int herr[4] = {0, 0, 0, 0};
    if (st == MG_OK) {
        cudaMemset(c->d_err, 0, sizeof(int) * 4);
        PolyArgs a = poly_args(c);
        MultiArgs m;
        m.nptm = nptm;
        m.nitem_a = item0[nptm];
        m.npair = nptm * (nptm - 1) / 2;
        m.ipm = d_ipm;
        m.atom0 = d_atom0;
        m.item0 = d_item0;
        m.moving = d_moving;
        m.rotm = d_rotm;
        m.rtm = d_rtm;
        m.out = d_out;
        k_poly_dutwobody_multi<<<1, 256>>>(a, m);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpy(out.data(), d_out, sizeof(double) * out.size(), cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(herr, c->d_err, sizeof herr, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = poly_fail(c, MG_ERR_CUDA, "mg_poly_dutwobody_multi: kernel failed");
    }
    cudaFree(d);
    if (st != MG_OK) return st;
    for (int k = 0; k <= nptpt; ++k) du_twob[k] = 0.0;
    // a hard core in the trial configuration rejects the move before the
    // current configuration is summed, as UTwoBodyPNew returns before
    // UTwoBodyPOld runs
    *lhsoverlap = out[2 * nptpt] != 0.0 ? 1 : 0;
    if (*lhsoverlap) return MG_OK;
    if (herr[0] == MG_ERR_TABLE_UNDERRUN)
        return poly_fail(c, herr[0], "current state: r2 < r2umin for particles %d and %d", herr[1], herr[2]);
    if (herr[0]) return poly_fail(c, herr[0], "ibuf > nbuf for particle-type pair %d", herr[1]);
    double s = 0.0;
    for (int k = 0; k < nptpt; ++k) {
        du_twob[k + 1] = out[k] - out[nptpt + k];
        s += du_twob[k + 1];
    }
    du_twob[0] = s;
    return MG_OK;
}
