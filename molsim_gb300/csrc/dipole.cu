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

}  // namespace

extern "C" int mg_dipole_ewald(mg_handle *h, const double *dip, double *potstat, double *estat, double *efg,
                               double *virelec) {
    if (!h || !dip || !potstat || !estat || !efg || !virelec) return MG_ERR_ARG;
    if (h->ewald != MG_EWALD_STD && h->ewald != MG_EWALD_SPM)
        return mg_fail(h, MG_ERR_STATE, "mg_dipole_ewald needs a handle with Ewald summation");
    if (h->form != MG_FP64) return mg_fail(h, MG_ERR_UNSUPPORTED, "dipole electrostatics need the FP64 form");
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
        MG_TRY(mg_ewald_std_dipole(h, d_dip, d_pot, d_est, d_efg, d_vir));
        vir.resize(h->nkvec);
    } else {
        double dmax = 0.0, kmax = std::max(h->dkdr[0], std::max(h->dkdr[1], h->dkdr[2]));
        for (int i = 0; i < 3 * np; ++i) dmax = std::max(dmax, std::fabs(dip[i]));
        double bound = (double)np * (h->az_absmax + 3.0 * kmax * dmax) * 1.01 + 1.0;
        MG_TRY(mg_spme_dipole(h, d_dip, bound, d_pot, d_est, d_efg, d_vir));
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
