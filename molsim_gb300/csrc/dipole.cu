// dipole.cu — the reciprocal part of the electrostatics of charges and point
// dipoles (UDipoleEwald, energy.F90:1807-1830) on a handle whose particles
// are the atoms: UDipoleEwaldRecStd or UDipoleEwaldRecSPM by the handle's
// Ewald method (ewald_std.cu k_dip_sk/k_dip_fk; spme.cu k_dip_spread, the
// FP64 FFT passes with the handle's influence function, k_dip_gather), then
// the atomic part of UDipoleEwaldSelf (energy.F90:2183-2191).  FP64.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mg_internal.cuh"

namespace {

// potstat -= (2 alpha / sqrt(pi)) q; estat += (4 alpha^3 / (3 sqrt(pi))) dip;
// efg(xx, yy, zz) -= (4 alpha^3 / (3 sqrt(pi))) q
__global__ void k_dip_self_atomic(int np, const double *__restrict__ az, const double *__restrict__ dip, double s1,
                                  double s2, double *__restrict__ pot, double *__restrict__ est,
                                  double *__restrict__ efg) {
    int ia = blockIdx.x * blockDim.x + threadIdx.x;
    if (ia >= np) return;
    double q = az[ia];
    pot[ia] = pot[ia] - s1 * q;
    for (int m = 0; m < 3; ++m) est[3 * ia + m] = est[3 * ia + m] + s2 * dip[3 * ia + m];
    for (int m = 0; m < 3; ++m) efg[6 * ia + m] = efg[6 * ia + m] - s2 * q;
}

// p = q u (the dipoles of the charges displaced along u)
__global__ void k_jvp_dipoles(int np, const double *__restrict__ az, const double *__restrict__ u,
                              double *__restrict__ p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * np) return;
    p[i] = az[i / 3] * u[i];
}

// jv_i += EpsiFourPi q_i (e_p(r_i) + efg_q(r_i) . u_i): the field of the
// displaced charges' dipoles and the field gradient of the charges moved
// along u_i; with the surface term -2 (2 pi / 3V) EpsiFourPi q_i sum_j q_j u_j
__global__ void k_jvp_rec_combine(int np, const double *__restrict__ az, const double *__restrict__ u,
                                  const double *__restrict__ est, const double *__restrict__ efg,
                                  const double *__restrict__ s3, double surf, double efp, double *__restrict__ jv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const double *g = efg + 6 * i, *ui = u + 3 * i;
    double gu[3] = {g[0] * ui[0] + g[3] * ui[1] + g[4] * ui[2], g[3] * ui[0] + g[1] * ui[1] + g[5] * ui[2],
                    g[4] * ui[0] + g[5] * ui[1] + g[2] * ui[2]};
    double q = az[i];
    for (int m = 0; m < 3; ++m) {
        double v = est[3 * i + m] + gu[m];
        if (s3) v -= surf * s3[m];
        jv[3 * i + m] += efp * q * v;
    }
}

// sum_j q_j u_j, one block of 1024 threads, a fixed order
__global__ void __launch_bounds__(1024) k_jvp_qu_sum(int np, const double *__restrict__ az,
                                                     const double *__restrict__ u, double *__restrict__ s3) {
    __shared__ double red[3][32];
    double s[3] = {0.0, 0.0, 0.0};
    for (int i = threadIdx.x; i < np; i += blockDim.x)
        for (int m = 0; m < 3; ++m) s[m] += az[i] * u[3 * i + m];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int m = 0; m < 3; ++m) {
        for (int o = 16; o > 0; o >>= 1) s[m] += __shfl_down_sync(0xffffffffu, s[m], o);
        if (lane == 0) red[m][w] = s[m];
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[threadIdx.x][k];
        s3[threadIdx.x] = t;
    }
}

}  // namespace

// the reciprocal and surface parts of d(force)/dx . u (force units before
// force_fac, added to jv; device arrays; u scaled to a largest component
// of 1): moving charge j by u_j adds the
// dipole q_j u_j, and charge i sees the field gradient of the others along
// u_i, so d(force_i) = EpsiFourPi q_i (e_p(r_i) + efg_q(r_i) . u_i).  Both
// come from the dipole kernels (charges off with dipoles p, then dipoles off
// with the charges) with their atomic self terms, which remove each
// particle's own contribution.
int mg_force_jvp_rec(mg_handle *h, const double *u, double *jv) {
    const int np = h->np;
    const size_t nvir = std::max((size_t)h->nkvec, (size_t)np + 2 * (size_t)std::max(h->nblk_rec, 1));
    const size_t need = 26 * (size_t)np + nvir + 3;   // p, zero, (pot, est, efg) twice, vir, sums
    if (h->dip_scr_n < need) {
        if (h->d_dip_scr) cudaFree(h->d_dip_scr);
        h->d_dip_scr = nullptr;
        h->dip_scr_n = 0;
        MG_CUDA(h, cudaMalloc(&h->d_dip_scr, sizeof(double) * need));
        h->dip_scr_n = need;
    }
    double *p = h->d_dip_scr, *zero = p + 3 * (size_t)np, *pot = zero + 3 * (size_t)np, *est = pot + np,
           *efg = est + 3 * (size_t)np, *pot2 = efg + 6 * (size_t)np, *est2 = pot2 + np,
           *efg2 = est2 + 3 * (size_t)np, *vir = efg2 + 6 * (size_t)np, *s3 = vir + nvir;
    MG_CUDA(h, cudaMemsetAsync(zero, 0, sizeof(double) * 23 * (size_t)np, h->st));   // zero .. efg2
    k_jvp_dipoles<<<(3 * np + 255) / 256, 256, 0, h->st>>>(np, h->d_az, u, p);
    const double ualpha = h->ualpha;
    const double s2 = (4.0 * ualpha * ualpha * ualpha) / (3.0 * std::sqrt(3.14159265358979323846));
    // the dipoles' field (charges off) and the charges' field gradient (dipoles off)
    if (h->ewald == MG_EWALD_STD) {
        MG_TRY(mg_ewald_std_dipole(h, zero, p, pot, est, efg, vir));
        MG_TRY(mg_ewald_std_dipole(h, h->d_az, zero, pot2, est2, efg2, vir));
    } else {
        // u is scaled to a largest component of 1 by the caller
        double kmax = std::max(h->dkdr[0], std::max(h->dkdr[1], h->dkdr[2]));
        double b1 = (double)np * (3.0 * kmax * h->az_absmax) * 1.01 + 1.0;
        double b2 = (double)np * h->az_absmax * 1.01 + 1.0;
        MG_TRY(mg_spme_dipole(h, zero, p, b1, pot, est, efg, vir));
        MG_TRY(mg_spme_dipole(h, h->d_az, zero, b2, pot2, est2, efg2, vir));
    }
    k_dip_self_atomic<<<(np + 127) / 128, 128, 0, h->st>>>(np, zero, p, 0.0, s2, pot, est, efg);
    k_dip_self_atomic<<<(np + 127) / 128, 128, 0, h->st>>>(np, h->d_az, zero, 0.0, s2, pot2, est2, efg2);
    const double *sums = nullptr;
    double surf = 0.0;
    if (h->lsurf) {
        k_jvp_qu_sum<<<1, 1024, 0, h->st>>>(np, h->d_az, u, s3);
        sums = s3;
        surf = 2.0 * (2.0 * 3.14159265358979323846 / (3.0 * h->vol));
    }
    k_jvp_rec_combine<<<(np + 127) / 128, 128, 0, h->st>>>(np, h->d_az, u, est, efg2, sums, surf, h->EpsiFourPi,
                                                           jv);
    h->launches += 5 + (h->lsurf ? 1 : 0);
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

// dq_k += EpsiFourPi (u_k . e_q(r_k) - phi_p(r_k)) - 2 (2 pi / 3V) EpsiFourPi
// (u_k . M + S . r_k): the reciprocal field of the charges at k, minus the
// reciprocal potential at k of the dipoles q_i u_i, and the surface term's
// charge derivative (M = sum q r, S = sum q u)
__global__ void k_pvjp_rec_combine(int np, const double *__restrict__ ro, const double *__restrict__ u,
                                   const double *__restrict__ est, const double *__restrict__ pot,
                                   const double *__restrict__ m3, const double *__restrict__ s3, double surf,
                                   double efp, double *__restrict__ dq) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= np) return;
    const double *uk = u + 3 * k, *ek = est + 3 * k, *rk = ro + 3 * k;
    double v = uk[0] * ek[0] + uk[1] * ek[1] + uk[2] * ek[2] - pot[k];
    if (m3)
        v -= surf * (uk[0] * m3[0] + uk[1] * m3[1] + uk[2] * m3[2] + s3[0] * rk[0] + s3[1] * rk[1] + s3[2] * rk[2]);
    dq[k] += efp * v;
}

// the reciprocal and surface parts of u . d(force)/dq (force units before
// force_fac, added to dq; device arrays; u scaled to a largest component
// of 1; after a UTotal of these positions, whose surface sums it reads):
// force_i = EpsiFourPi q_i e_i with e_i linear in the charges, so
// u . d(force)/dq_k = EpsiFourPi (u_k . e_k + sum_i q_i u_i . K(r_i, r_k)),
// and the sum is minus the potential at r_k of the dipoles q_i u_i.  Each
// particle's own contributions vanish (its field and its dipole's
// potential at its own site are zero by symmetry).
int mg_force_pvjp_rec(mg_handle *h, const double *u, double *dq) {
    const int np = h->np;
    const size_t nvir = std::max((size_t)h->nkvec, (size_t)np + 2 * (size_t)std::max(h->nblk_rec, 1));
    const size_t need = 26 * (size_t)np + nvir + 3;
    if (h->dip_scr_n < need) {
        if (h->d_dip_scr) cudaFree(h->d_dip_scr);
        h->d_dip_scr = nullptr;
        h->dip_scr_n = 0;
        MG_CUDA(h, cudaMalloc(&h->d_dip_scr, sizeof(double) * need));
        h->dip_scr_n = need;
    }
    double *p = h->d_dip_scr, *zero = p + 3 * (size_t)np, *pot = zero + 3 * (size_t)np, *est = pot + np,
           *efg = est + 3 * (size_t)np, *pot2 = efg + 6 * (size_t)np, *est2 = pot2 + np,
           *efg2 = est2 + 3 * (size_t)np, *vir = efg2 + 6 * (size_t)np, *s3 = vir + nvir;
    MG_CUDA(h, cudaMemsetAsync(zero, 0, sizeof(double) * 23 * (size_t)np, h->st));   // zero .. efg2
    k_jvp_dipoles<<<(3 * np + 255) / 256, 256, 0, h->st>>>(np, h->d_az, u, p);
    if (h->ewald == MG_EWALD_STD) {
        MG_TRY(mg_ewald_std_dipole(h, h->d_az, zero, pot, est, efg, vir));   // the charges' field
        MG_TRY(mg_ewald_std_dipole(h, zero, p, pot2, est2, efg2, vir));      // the dipoles' potential
    } else {
        double kmax = std::max(h->dkdr[0], std::max(h->dkdr[1], h->dkdr[2]));
        double b1 = (double)np * h->az_absmax * 1.01 + 1.0;
        double b2 = (double)np * (3.0 * kmax * h->az_absmax) * 1.01 + 1.0;
        MG_TRY(mg_spme_dipole(h, h->d_az, zero, b1, pot, est, efg, vir));
        MG_TRY(mg_spme_dipole(h, zero, p, b2, pot2, est2, efg2, vir));
    }
    const double *m3 = nullptr;
    double surf = 0.0;
    if (h->lsurf) {
        k_jvp_qu_sum<<<1, 1024, 0, h->st>>>(np, h->d_az, u, s3);
        m3 = h->d_uout + h->nptpt + 1 + 4;   // sum q r of the last UTotal
        surf = 2.0 * (2.0 * 3.14159265358979323846 / (3.0 * h->vol));
    }
    k_pvjp_rec_combine<<<(np + 127) / 128, 128, 0, h->st>>>(np, h->d_ro, u, est, pot2, m3, s3, surf, h->EpsiFourPi,
                                                            dq);
    h->launches += 3 + (h->lsurf ? 1 : 0);
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

extern "C" int mg_dipole_ewald(mg_handle *h, const double *dip, double *potstat, double *estat, double *efg,
                               double *virelec) {
    if (!h || !dip || !potstat || !estat || !efg || !virelec) return MG_ERR_ARG;
    if (h->ewald != MG_EWALD_STD && h->ewald != MG_EWALD_SPM)
        return mg_fail(h, MG_ERR_STATE, "mg_dipole_ewald needs a handle with Ewald summation");
    if (h->form != MG_FP64) return mg_fail(h, MG_ERR_UNSUPPORTED, "dipole electrostatics need the FP64 form");
    if (h->mode == MG_MC)   // the structure factors and meshes of the accepted MC state stay untouched
        return mg_fail(h, MG_ERR_UNSUPPORTED, "mg_dipole_ewald needs an MD or BD handle");
    const int np = h->np;
    const size_t nvir = std::max((size_t)h->nkvec, (size_t)np + 2 * (size_t)std::max(h->nblk_rec, 1));
    const size_t need = 13 * (size_t)np + nvir;
    if (h->dip_scr_n < need) {
        if (h->d_dip_scr) cudaFree(h->d_dip_scr);
        h->d_dip_scr = nullptr;
        h->dip_scr_n = 0;
        MG_CUDA(h, cudaMalloc(&h->d_dip_scr, sizeof(double) * need));
        h->dip_scr_n = need;
    }
    double *d_dip = h->d_dip_scr, *d_pot = d_dip + 3 * (size_t)np, *d_est = d_pot + np, *d_efg = d_est + 3 * (size_t)np,
           *d_vir = d_efg + 6 * (size_t)np;
    MG_CUDA(h, cudaMemcpyAsync(d_dip, dip, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, h->st));
    MG_CUDA(h, cudaMemcpyAsync(d_pot, potstat, sizeof(double) * np, cudaMemcpyHostToDevice, h->st));
    MG_CUDA(h, cudaMemcpyAsync(d_est, estat, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, h->st));
    MG_CUDA(h, cudaMemcpyAsync(d_efg, efg, sizeof(double) * 6 * np, cudaMemcpyHostToDevice, h->st));
    std::vector<double> vir;
    if (h->ewald == MG_EWALD_STD) {
        MG_TRY(mg_ewald_std_dipole(h, h->d_az, d_dip, d_pot, d_est, d_efg, d_vir));
        vir.resize(h->nkvec);
    } else {
        double dmax = 0.0, kmax = std::max(h->dkdr[0], std::max(h->dkdr[1], h->dkdr[2]));
        for (int i = 0; i < 3 * np; ++i) dmax = std::max(dmax, std::fabs(dip[i]));
        double bound = (double)np * (h->az_absmax + 3.0 * kmax * dmax) * 1.01 + 1.0;
        MG_TRY(mg_spme_dipole(h, h->d_az, d_dip, bound, d_pot, d_est, d_efg, d_vir));
        vir.resize((size_t)np + 2 * (size_t)h->nblk_rec);
    }
    const double ualpha = h->ualpha;
    const double s1 = (2.0 * ualpha) / std::sqrt(3.14159265358979323846);
    const double s2 = (4.0 * ualpha * ualpha * ualpha) / (3.0 * std::sqrt(3.14159265358979323846));
    k_dip_self_atomic<<<(np + 127) / 128, 128, 0, h->st>>>(np, h->d_az, d_dip, s1, s2, d_pot, d_est, d_efg);
    h->launches++;
    MG_CUDA(h, cudaGetLastError());
    MG_CUDA(h, cudaMemcpyAsync(potstat, d_pot, sizeof(double) * np, cudaMemcpyDeviceToHost, h->st));
    MG_CUDA(h, cudaMemcpyAsync(estat, d_est, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, h->st));
    MG_CUDA(h, cudaMemcpyAsync(efg, d_efg, sizeof(double) * 6 * np, cudaMemcpyDeviceToHost, h->st));
    MG_CUDA(h, cudaMemcpyAsync(vir.data(), d_vir, sizeof(double) * vir.size(), cudaMemcpyDeviceToHost, h->st));
    MG_CUDA(h, cudaStreamSynchronize(h->st));
    double v = *virelec;
    if (h->ewald == MG_EWALD_STD) {
        for (double x : vir) v = v + x;   // the k-vectors in order
    } else {
        for (int b = 0; b < h->nblk_rec; ++b) v = v + vir[(size_t)np + 2 * b + 1];   // SPMFFTRec's virloc
        for (int ia = 0; ia < np; ++ia) v = v + vir[ia];                             // the dipole terms
    }
    *virelec = v;
    return MG_OK;
}
