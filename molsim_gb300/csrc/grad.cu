// grad.cu — gradients of UTotal with respect to its parameters (row A16 and
// the adjoint form).
//
//   phi(i)     = dU/dq_i, the site potential: real-space Coulomb over the
//                Verlet list (erfc(alpha r)/r with Ewald, 1/r without), the
//                reciprocal potential at the site (SPME: the B-spline gather
//                of the potential mesh with spline values, as
//                FieldStatEwaldRecSPM, energy.F90:2845-2940, does for
//                fields; standard Ewald: the k-sum with the structure
//                factors), the self term and the surface term
//   dU/deps_ab, dU/dsig_ab
//                for the (1,6,12) pair parameters of every type pair
//                (Pot_1_6_12, potential.F90:1349-1434: sig_ab = (sig_a +
//                sig_b)/2, eps_ab = sqrt(eps_a eps_b), with lljcut's cut and
//                shift) from the analytic Lennard-Jones form
//   dU/deps_ab for an affine strain of the box and the positions,
//                r -> (1 + eps) r (components xx, yy, zz, xy, xz, yz; the
//                tensor is symmetric): pairs and bonds through their radial
//                derivative, angles through their arms, the reciprocal sum
//                through the k-dependence of meshfac / kfac (k -> (1 -
//                eps^T) k, V -> (1 + tr eps) V), the surface term through
//                its volume and dipole.  Its trace is the reference's scalar
//                virial; dU/dL_a = dU/deps_aa / L_a.
// All arithmetic is FP64 in both forms (the mixed form reads its FP32
// potential mesh).
#include <algorithm>
#include <cmath>
#include <vector>

#include "mg_internal.cuh"

namespace {

constexpr int kGradThreads = 128;

struct GradArgs {
    const double *ro, *az;
    const int *type, *pairidx, *perm, *nnb, *nbr;
    int np, npt, nptpt, cellcut, ewald;
    const double *ubuf, *r2atat, *r2umin;
    const int *tab_start, *tab_n;
    mg_box box;
    double rcut2, efp, alpha;
    const double *sig, *eps, *ljrc;   // per pair type: sigma_ab, eps_ab, ljrcut * sigma_ab
    int lljcut;
    double ljushift;
    double *phi;                      // [np]
    double *part;                     // per block: deps[nptpt], dsig[nptpt], strain[6]
};

// strain components: xx, yy, zz, xy, xz, yz
__device__ __forceinline__ void strain_add(double *w, double f, double dx, double dy, double dz) {
    w[0] += f * dx * dx;
    w[1] += f * dy * dy;
    w[2] += f * dz * dz;
    w[3] += f * dx * dy;
    w[4] += f * dx * dz;
    w[5] += f * dy * dz;
}

__global__ void __launch_bounds__(kGradThreads) k_grad_pairs(GradArgs a) {
    __shared__ double red[2 * MG_MAX_NPTPT + 6][kGradThreads / 32];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double de[MG_MAX_NPTPT], ds[MG_MAX_NPTPT], wv[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int k = 0; k < a.nptpt; ++k) { de[k] = 0.0; ds[k] = 0.0; }
    if (i < a.np) {
        int p = a.perm[i], ti = a.type[p];
        const double *ri = a.ro + 3 * (size_t)p;
        double site = 0.0;
        int nn = a.nnb[i];
        for (int k = 0; k < nn; ++k) {
            int q = a.perm[a.nbr[(size_t)k * a.np + i]];
            const double *rj = a.ro + 3 * (size_t)q;
            double dx = mg_pbc1(__dsub_rn(ri[0], rj[0]), a.box.half[0], a.box.len[0]);
            double dy = mg_pbc1(__dsub_rn(ri[1], rj[1]), a.box.half[1], a.box.len[1]);
            double dz = mg_pbc1(__dsub_rn(ri[2], rj[2]), a.box.half[2], a.box.len[2]);
            double r2 = mg_r2_exact(dx, dy, dz);
            if (a.cellcut ? !(r2 < a.rcut2) : (r2 > a.rcut2)) continue;
            int pair = a.pairidx[a.type[q] * a.npt + ti] - 1;
            if (r2 < a.r2atat[pair] || r2 < a.r2umin[pair]) continue;   // constant 1e10 / outside the table
            double r = sqrt(r2);
            // real-space Coulomb kernel at the site
            site += a.az[q] * a.efp * (a.ewald != MG_EWALD_NONE ? erfc(a.alpha * r) / r : 1.0 / r);
            // Lennard-Jones parameter derivatives (each pair is met twice)
            double sg = a.sig[pair], x = sg * sg / r2;
            x = x * x * x;
            bool lj = a.sig && (!a.lljcut || r < a.ljrc[pair]);
            if (lj) {
                de[pair] += 0.5 * (4.0 * (x * x - x) + (a.lljcut ? a.ljushift : 0.0));
                ds[pair] += 0.5 * (24.0 * a.eps[pair] / sg) * (2.0 * x * x - x);
            }
            // table force: dU/deps_ab = -sum fsum dx_a dx_b
            int rr = a.tab_start[pair], nr = a.tab_n[pair], kk = 0;
            while (kk + 1 < nr && r2 < a.ubuf[12 * (size_t)(rr + kk)]) ++kk;
            const double *c = a.ubuf + 12 * (size_t)(rr + kk);
            double d = r2 - c[0];
            double fsum = c[7] + d * (c[8] + d * (c[9] + d * (c[10] + d * c[11])));
            strain_add(wv, -0.5 * fsum, dx, dy, dz);
        }
        a.phi[p] = site;
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int nv = 2 * a.nptpt + 6;
    for (int v = 0; v < nv; ++v) {
        double x = v < a.nptpt ? de[v] : v < 2 * a.nptpt ? ds[v - a.nptpt] : wv[v - 2 * a.nptpt];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[v][w] = x;
    }
    __syncthreads();
    if (threadIdx.x < nv) {
        double s = 0.0;
        for (int k = 0; k < kGradThreads / 32; ++k) s += red[threadIdx.x][k];
        a.part[(size_t)blockIdx.x * nv + threadIdx.x] = s;
    }
}

// bonds: dU/deps_ab = sum du/dr dx_a dx_b / r; angles (UAngle): sum over
// the two arms d = r_ip - r_j of (dU/dd)_a d_b
__global__ void k_grad_bonds(const double *__restrict__ ro, const int *__restrict__ ij,
                             const double *__restrict__ bk, const double *__restrict__ beq,
                             const int *__restrict__ bp, int nbond, const int *__restrict__ aijk,
                             const double *__restrict__ ak, const double *__restrict__ aeq,
                             const int *__restrict__ ap, int nangle, mg_box box, double *__restrict__ part) {
    __shared__ double red[6][8];
    double wv[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int an = blockIdx.x * blockDim.x + threadIdx.x; an < nangle; an += gridDim.x * blockDim.x) {
        int jm = aijk[3 * an], ip = aijk[3 * an + 1], jp = aijk[3 * an + 2];
        double dm[3], dq[3], um[3], uq[3];
        for (int m = 0; m < 3; ++m) {
            double x = ro[3 * (size_t)ip + m] - ro[3 * (size_t)jm + m];
            double y = ro[3 * (size_t)ip + m] - ro[3 * (size_t)jp + m];
            if (fabs(x) > box.half[m]) x -= box.len[m] * round(x * box.inv[m]);
            if (fabs(y) > box.half[m]) y -= box.len[m] * round(y * box.inv[m]);
            dm[m] = x;
            dq[m] = y;
        }
        double dmi = 1.0 / sqrt(dm[0] * dm[0] + dm[1] * dm[1] + dm[2] * dm[2]);
        double dpi = 1.0 / sqrt(dq[0] * dq[0] + dq[1] * dq[1] + dq[2] * dq[2]);
        for (int m = 0; m < 3; ++m) {
            um[m] = dm[m] * dmi;
            uq[m] = dq[m] * dpi;
        }
        double c = um[0] * uq[0] + um[1] * uq[1] + um[2] * uq[2];
        double theta = acos(fmax(-1.0, fmin(c, 1.0)));
        double term = theta - aeq[an];
        int pw = ap[an];
        double fac = -pw * ak[an] * pow(term, pw - 1) / sin(theta);
        double gm[3], gq[3];   // dU/d(arm) for the two arms
        for (int m = 0; m < 3; ++m) {
            gm[m] = (fac * dmi) * (uq[m] - c * um[m]);
            gq[m] = (fac * dpi) * (um[m] - c * uq[m]);
        }
        const int ca[6] = {0, 1, 2, 0, 0, 1}, cb[6] = {0, 1, 2, 1, 2, 2};
        for (int v = 0; v < 6; ++v) wv[v] += gm[ca[v]] * dm[cb[v]] + gq[ca[v]] * dq[cb[v]];
    }
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nbond; b += gridDim.x * blockDim.x) {
        int i = ij[2 * b], j = ij[2 * b + 1];
        double dx = mg_pbc1(ro[3 * (size_t)i] - ro[3 * (size_t)j], box.half[0], box.len[0]);
        double dy = mg_pbc1(ro[3 * (size_t)i + 1] - ro[3 * (size_t)j + 1], box.half[1], box.len[1]);
        double dz = mg_pbc1(ro[3 * (size_t)i + 2] - ro[3 * (size_t)j + 2], box.half[2], box.len[2]);
        double r = sqrt(dx * dx + dy * dy + dz * dz);
        int pw = bp[b];
        double du = bk[b] * pw * pow(r - beq[b], pw - 1) / r;
        strain_add(wv, du, dx, dy, dz);
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int v = 0; v < 6; ++v) {
        double x = wv[v];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[v][w] = x;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double x = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) x += red[threadIdx.x][k];
        part[6 * blockIdx.x + threadIdx.x] = x;
    }
}

// CardinalBSpline values (mollib.F90:1625-1687)
__device__ void grad_bspline(int order, double x, double *v) {
    double last[MG_MAX_ORDER];
    v[0] = x;
    v[1] = 1.0 - x;
    for (int i = 2; i < order; ++i) v[i] = 0.0;
    for (int nn = 3; nn <= order; ++nn) {
        for (int i = 0; i < nn - 1; ++i) last[i] = v[i];
        v[0] = x * last[0] / (nn - 1);
        for (int i = 1; i <= nn - 2; ++i) {
            double aa = i + x;
            v[i] = (aa * last[i] + (nn - aa) * last[i - 1]) / (nn - 1);
        }
        v[nn - 1] = (1.0 - x) * last[nn - 2] / (nn - 1);
    }
}

// reciprocal, self and surface parts of the site potentials
struct SiteArgs {
    const double *ro, *az;
    int np, ewald, lsurf;
    double efp, alpha, surf2;          // surf2 = 2 * 2 pi / (3 V)
    const double *dip;                 // [3] sum q r (UTotal's surface sums)
    // SPME
    int n, order, mixed;
    double dkdr[3];
    const void *mesh;                  // potential mesh dE/dQ (mesh type)
    // standard Ewald
    const int4 *kv;
    const double *kfac;
    const double2 *S;
    int nk;
    double3 tpbi;
    double *phi;
};

__global__ void k_grad_site(SiteArgs a) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.np || a.ewald == MG_EWALD_NONE) return;
    const double *r = a.ro + 3 * (size_t)p;
    double rec = 0.0;
    if (a.ewald == MG_EWALD_SPM) {
        double w[3][MG_MAX_ORDER];
        int c[3];
        for (int d = 0; d < 3; ++d) {
            double pos = a.dkdr[d] * r[d], fl = floor(pos);
            int mm = (int)fl % a.n;
            c[d] = mm < 0 ? mm + a.n : mm;
            grad_bspline(a.order, pos - fl, w[d]);
        }
        int mn = mg_mesh_mask(a.n);
        for (int iz = 0; iz < a.order; ++iz)
            for (int iy = 0; iy < a.order; ++iy) {
                size_t row = ((size_t)mg_wrapm(c[2] - iz, a.n, mn) * a.n + mg_wrapm(c[1] - iy, a.n, mn)) * a.n;
                double wyz = w[2][iz] * w[1][iy], s = 0.0;
                for (int ix = 0; ix < a.order; ++ix) {
                    size_t idx = row + mg_wrapm(c[0] - ix, a.n, mn);
                    double v = a.mixed ? (double)((const float *)a.mesh)[idx] : ((const double *)a.mesh)[idx];
                    s += w[0][ix] * v;
                }
                rec += wyz * s;
            }
    } else {
        // d/dq_i sum_k kfac sum_c |S_c|^2 = sum_k kfac sum_c 2 Re(conj(S_c) e_c)
        for (int k = 0; k < a.nk; ++k) {
            int4 n = a.kv[k];
            double sx, cx, sy, cy, sz, cz;
            sincos(n.x * a.tpbi.x * r[0], &sx, &cx);
            sincos(n.y * a.tpbi.y * r[1], &sy, &cy);
            sincos(n.z * a.tpbi.z * r[2], &sz, &cz);
            // e_c = e^{i(sx kx x + sy ky y + kz z)} for (sx, sy) = (-,-), (-,+), (+,-), (+,+)
            double acc = 0.0;
            for (int cmb = 0; cmb < 4; ++cmb) {
                double ax = (cmb & 2) ? sx : -sx, ay = (cmb & 1) ? sy : -sy;
                // (cx + i ax)(cy + i ay)(cz + i sz)
                double re1 = cx * cy - ax * ay, im1 = cx * ay + ax * cy;
                double re = re1 * cz - im1 * sz, im = re1 * sz + im1 * cz;
                double2 S = a.S[4 * k + cmb];
                acc += S.x * re + S.y * im;
            }
            rec += 2.0 * a.kfac[k] * acc;
        }
    }
    double q = a.az[p];
    double v = rec - 2.0 * a.alpha / sqrt(3.1415926535897932) * q;   // UEwaldSelf
    if (a.lsurf) v += a.surf2 * (a.dip[0] * r[0] + a.dip[1] * r[1] + a.dip[2] * r[2]);
    a.phi[p] += a.efp * v;
}

// standard Ewald: dE/deps_ab = sum_k kfac sum_c |S_c|^2 (-delta_ab + 2 k_a
// k_b (1/(4 alpha^2) + 1/k^2)), the sign combination c = (sx, sy) giving
// k = (sx kx, sy ky, kz)
__global__ void k_grad_box_std(const int4 *__restrict__ kv, const double *__restrict__ kfac,
                               const double2 *__restrict__ S, int nk, double3 tpbi, double ia2,
                               double *__restrict__ out6) {
    __shared__ double red[6][8];
    double g[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int k = threadIdx.x; k < nk; k += blockDim.x) {
        int4 n = kv[k];
        double mx = n.x * tpbi.x, my = n.y * tpbi.y, mz = n.z * tpbi.z;
        double c = ia2 + 1.0 / (mx * mx + my * my + mz * mz);
        for (int cmb = 0; cmb < 4; ++cmb) {
            double sx = (cmb & 2) ? 1.0 : -1.0, sy = (cmb & 1) ? 1.0 : -1.0;
            double e = kfac[k] * (S[4 * k + cmb].x * S[4 * k + cmb].x + S[4 * k + cmb].y * S[4 * k + cmb].y);
            double kx = sx * mx, ky = sy * my, kz = mz;
            g[0] += e * (-1.0 + 2.0 * kx * kx * c);
            g[1] += e * (-1.0 + 2.0 * ky * ky * c);
            g[2] += e * (-1.0 + 2.0 * kz * kz * c);
            g[3] += e * (2.0 * kx * ky * c);
            g[4] += e * (2.0 * kx * kz * c);
            g[5] += e * (2.0 * ky * kz * c);
        }
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int v = 0; v < 6; ++v) {
        double x = g[v];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[v][w] = x;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double x = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) x += red[threadIdx.x][k];
        out6[threadIdx.x] = x;
    }
}

// fixed-order totals: out = [deps(nptpt), dsig(nptpt), strain(6)]
struct FinalGrad {
    const double *pair_part;
    int nblk_pair, nptpt;
    const double *bond_part;
    int nblk_bond;
    const double *rec6;      // dE_rec/deps (before EpsiFourPi) or null
    const double *dip;       // surface sums or null
    double efp, surf_fac;
    double *out;
};

__global__ void k_grad_final(FinalGrad f) {
    int v = threadIdx.x, nv = 2 * f.nptpt + 6;
    if (v >= nv) return;
    double s = 0.0;
    for (int b = 0; b < f.nblk_pair; ++b) s += f.pair_part[(size_t)b * nv + v];
    if (v >= 2 * f.nptpt) {
        const int ca[6] = {0, 1, 2, 0, 0, 1}, cb[6] = {0, 1, 2, 1, 2, 2};
        int d = v - 2 * f.nptpt;
        for (int b = 0; b < f.nblk_bond; ++b) s += f.bond_part[6 * b + d];
        double r = f.rec6 ? f.rec6[d] : 0.0;
        if (f.dip) {   // E_surf = surf_fac |M|^2, M -> (1 + eps) M, V -> (1 + tr eps) V
            double m2 = f.dip[0] * f.dip[0] + f.dip[1] * f.dip[1] + f.dip[2] * f.dip[2];
            r += f.surf_fac * (2.0 * f.dip[ca[d]] * f.dip[cb[d]] - (d < 3 ? m2 : 0.0));
        }
        s += f.efp * r;
    }
    f.out[v] = s;
}

}  // namespace

int mg_spme_box_grad(mg_handle *h, double *out6, double *scratch);

namespace {

// UTotal at the current positions and its gradients: phi (dU/dq_i) into
// phi (if non-null), and out = [deps(nptpt), dsig(nptpt), strain(6)]; with
// pp null the Lennard-Jones parameter derivatives are zero
int grad_run(mg_handle *h, const mg_pot_params *pp, double *phi, std::vector<double> &out) {
    if (pp && (!pp->sigat || !pp->epsat)) return MG_ERR_ARG;
    if (pp && pp->npt != h->npt) return mg_fail(h, MG_ERR_ARG, "pot params npt %d != %d", pp->npt, h->npt);
    if (!h->list_valid) return mg_fail(h, MG_ERR_STATE, "mg_nlist_set has not been called");
    int np = h->np, nptpt = h->nptpt, npt = h->npt;
    // per pair type: Lorentz-Berthelot sigma_ab, eps_ab and the LJ cut
    std::vector<double> ab(3 * (size_t)nptpt, 0.0);
    if (pp)
        for (int a = 0; a < npt; ++a)
            for (int b = 0; b < npt; ++b) {
                int pair = h->h_pairidx[b * npt + a] - 1;
                double sg = 0.5 * (pp->sigat[a] + pp->sigat[b]);
                ab[pair] = sg;
                ab[nptpt + pair] = std::sqrt(pp->epsat[a] * pp->epsat[b]);
                ab[2 * nptpt + pair] = pp->ljrcut * sg;
            }
    if (h->list_stale) {
        MG_TRY(mg_lists_build(h, false));
        h->list_stale = false;
    }
    MG_TRY(mg_utotal_launch(h));   // energies, structure factors / potential mesh, surface sums
    int nblk_pair = (np + kGradThreads - 1) / kGradThreads, nv = 2 * nptpt + 6;
    int nbonded = std::max(h->nbond, h->nangle);
    int nblk_bond = nbonded > 0 ? std::min(304, (nbonded + 255) / 256) : 0;
    size_t need = (size_t)np + 3 * nptpt + (size_t)nblk_pair * nv + 6 * (size_t)std::max(nblk_bond, 1) + 6 +
                  6 * 304 + (size_t)nv;
    if (need > h->grad_cap) {
        if (h->d_grad) cudaFree(h->d_grad);
        h->d_grad = nullptr;
        MG_CUDA(h, cudaMalloc(&h->d_grad, sizeof(double) * need));
        h->grad_cap = need;
    }
    double *d_phi = h->d_grad, *d_ab = d_phi + np, *d_pp = d_ab + 3 * nptpt;
    double *d_bp = d_pp + (size_t)nblk_pair * nv, *d_rec6 = d_bp + 6 * (size_t)std::max(nblk_bond, 1);
    double *d_scr = d_rec6 + 6, *d_out = d_scr + 6 * 304;
    MG_CUDA(h, cudaMemcpyAsync(d_ab, ab.data(), sizeof(double) * 3 * nptpt, cudaMemcpyHostToDevice, h->st));
    GradArgs a;
    a.ro = h->d_ro;
    a.az = h->d_az;
    a.type = h->d_type;
    a.pairidx = h->d_pairidx;
    a.perm = h->d_perm;
    a.nnb = h->d_nnb;
    a.nbr = h->d_nbr;
    a.np = np;
    a.npt = npt;
    a.nptpt = nptpt;
    a.cellcut = h->txintlist == MG_CELLLIST ? 1 : 0;
    a.ewald = h->ewald;
    a.ubuf = h->d_ubuf;
    a.r2atat = h->d_r2atat;
    a.r2umin = h->d_r2umin;
    a.tab_start = h->d_tab_start;
    a.tab_n = h->d_tab_n;
    for (int d = 0; d < 3; ++d) {
        a.box.len[d] = h->boxlen[d];
        a.box.half[d] = h->boxlen2[d];
        a.box.inv[d] = h->boxleni[d];
    }
    a.rcut2 = h->rcut2;
    a.efp = h->EpsiFourPi;
    a.alpha = h->ualpha;
    a.sig = pp ? d_ab : nullptr;
    a.eps = d_ab + nptpt;
    a.ljrc = d_ab + 2 * nptpt;
    a.lljcut = pp ? pp->lljcut : 0;
    a.ljushift = pp ? pp->ljushift : 0.0;
    a.phi = d_phi;
    a.part = d_pp;
    k_grad_pairs<<<nblk_pair, kGradThreads, 0, h->st>>>(a);
    h->launches++;
    bool surf = h->lsurf && h->ewald != MG_EWALD_NONE;
    const double *d_dip = surf ? h->d_uout + nptpt + 1 + 4 : nullptr;
    if (h->ewald != MG_EWALD_NONE) {
        SiteArgs s = {};
        s.ro = h->d_ro;
        s.az = h->d_az;
        s.np = np;
        s.ewald = h->ewald;
        s.lsurf = surf ? 1 : 0;
        s.efp = h->EpsiFourPi;
        s.alpha = h->ualpha;
        s.surf2 = 2.0 * (2.0 * 3.1415926535897932 / (3.0 * h->vol));
        s.dip = d_dip;
        s.n = h->nmesh;
        s.order = h->order;
        s.mixed = h->form == MG_MIXED;
        for (int d = 0; d < 3; ++d) s.dkdr[d] = h->dkdr[d];
        s.mesh = h->d_Q;
        s.kv = h->d_kvec;
        s.kfac = h->d_kfac;
        s.S = h->d_S;
        s.nk = h->nkvec;
        s.tpbi = make_double3(h->TwoPiBoxi[0], h->TwoPiBoxi[1], h->TwoPiBoxi[2]);
        s.phi = d_phi;
        k_grad_site<<<(np + 127) / 128, 128, 0, h->st>>>(s);
        h->launches++;
    }
    if (nblk_bond > 0) {
        mg_box box = a.box;
        k_grad_bonds<<<nblk_bond, 256, 0, h->st>>>(h->d_ro, h->d_bond_ij, h->d_bond_k, h->d_bond_eq, h->d_bond_p,
                                                    h->nbond, h->d_angle_ijk, h->d_angle_k, h->d_angle_eq,
                                                    h->d_angle_p, h->nangle, box, d_bp);
        h->launches++;
    }
    const double *rec6 = nullptr;
    if (h->ewald == MG_EWALD_STD) {
        k_grad_box_std<<<1, 256, 0, h->st>>>(h->d_kvec, h->d_kfac, h->d_S, h->nkvec,
                                             make_double3(h->TwoPiBoxi[0], h->TwoPiBoxi[1], h->TwoPiBoxi[2]),
                                             1.0 / (4.0 * h->ualpha * h->ualpha), d_rec6);
        h->launches++;
        rec6 = d_rec6;
    } else if (h->ewald == MG_EWALD_SPM) {
        MG_TRY(mg_spme_box_grad(h, d_rec6, d_scr));
        rec6 = d_rec6;
    }
    FinalGrad f;
    f.pair_part = d_pp;
    f.nblk_pair = nblk_pair;
    f.nptpt = nptpt;
    f.bond_part = d_bp;
    f.nblk_bond = nblk_bond;
    f.rec6 = rec6;
    f.dip = d_dip;
    f.efp = h->EpsiFourPi;
    f.surf_fac = 2.0 * 3.1415926535897932 / (3.0 * h->vol);
    f.out = d_out;
    k_grad_final<<<1, 32, 0, h->st>>>(f);
    h->launches++;
    MG_CUDA(h, cudaGetLastError());
    out.assign(nv, 0.0);
    if (phi) MG_CUDA(h, cudaMemcpyAsync(phi, d_phi, sizeof(double) * np, cudaMemcpyDeviceToHost, h->st));
    MG_CUDA(h, cudaMemcpyAsync(out.data(), d_out, sizeof(double) * nv, cudaMemcpyDeviceToHost, h->st));
    return mg_check_device_error(h);
}

}  // namespace

// ---- force Jacobian-vector products (Hessian-vector products of U) -------------
namespace {

struct JvpArgs {
    const double4 *pos_s;
    const int *perm, *nnb, *nbr;
    int np, npt, nbins;
    const int *pairidx, *tab_start, *tab_n;
    const double *zlow, *coef, *bin_z0, *bin_inv, *r2umin;
    const unsigned short *bin_kstart;
    mg_box box;
    double rcut2;
    const double *u;
    double *jv;
};

// d(force_i)/dx . u over the full Verlet list (one thread per slot): for
// the tabulated pair force fsum(r^2) d, the change along w = u_i - u_j is
// fsum w + 2 fsum'(r^2) (d . w) d, fsum' the derivative of the table's
// quartic in r^2 - zlow
__global__ void __launch_bounds__(128) k_jvp_pairs(JvpArgs a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.np) return;
    double4 pi = a.pos_s[i];
    int ti = (int)pi.w, p = a.perm[i];
    double ui[3] = {a.u[3 * p], a.u[3 * p + 1], a.u[3 * p + 2]};
    double g[3] = {0.0, 0.0, 0.0};
    int nn = a.nnb[i];
    for (int k = 0; k < nn; ++k) {
        int j = a.nbr[(size_t)k * a.np + i];
        double4 pj = a.pos_s[j];
        double d[3] = {mg_pbc1(pi.x - pj.x, a.box.half[0], a.box.len[0]),
                       mg_pbc1(pi.y - pj.y, a.box.half[1], a.box.len[1]),
                       mg_pbc1(pi.z - pj.z, a.box.half[2], a.box.len[2])};
        double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (r2 > a.rcut2) continue;
        int tj = (int)pj.w;
        int pair = a.pairidx[tj * a.npt + ti] - 1;
        if (r2 < a.r2umin[pair]) continue;   // below the table: UTotal reports it
        int b = (int)((r2 - a.bin_z0[pair]) * a.bin_inv[pair]);
        b = min(max(b, 0), a.nbins - 1);
        int kk = a.bin_kstart[pair * a.nbins + b], last = a.tab_n[pair] - 1;
        const double *z = a.zlow + a.tab_start[pair];
        while (kk < last && z[kk] > r2) ++kk;
        int rec = a.tab_start[pair] + kk;
        const double *c = a.coef + (size_t)rec * 11;
        double dd = r2 - a.zlow[rec];
        double fs = c[6] + dd * (c[7] + dd * (c[8] + dd * (c[9] + dd * c[10])));
        double dfs = c[7] + dd * (2.0 * c[8] + dd * (3.0 * c[9] + dd * 4.0 * c[10]));
        int q = a.perm[j];
        double w[3] = {ui[0] - a.u[3 * q], ui[1] - a.u[3 * q + 1], ui[2] - a.u[3 * q + 2]};
        double dw = 2.0 * dfs * (d[0] * w[0] + d[1] * w[1] + d[2] * w[2]);
        for (int m = 0; m < 3; ++m) g[m] += fs * w[m] + dw * d[m];
    }
    for (int m = 0; m < 3; ++m) a.jv[3 * p + m] += g[m];
}

// bonds u = k (r - r0)^p: d(force_ip)/dx . u = -k p [(p-1)(r-r0)^(p-2)
// (dh . w) dh + (r-r0)^(p-1) (w - dh (dh . w)) / r], dh = d/r, w = u_ip - u_jp;
// force_jp the opposite (FP64 atomics)
__global__ void k_jvp_bonds(int nbond, const int *__restrict__ ij, const double *__restrict__ bk,
                            const double *__restrict__ beq, const int *__restrict__ bp, const double *__restrict__ ro,
                            mg_box box, const double *__restrict__ u, double *__restrict__ jv) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbond) return;
    int ip = ij[2 * b], jp = ij[2 * b + 1];
    double d[3], w[3];
    for (int m = 0; m < 3; ++m) {
        d[m] = mg_pbc1(ro[3 * ip + m] - ro[3 * jp + m], box.half[m], box.len[m]);
        w[m] = u[3 * ip + m] - u[3 * jp + m];
    }
    double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    double dh[3] = {d[0] / r, d[1] / r, d[2] / r};
    double t = r - beq[b];
    int pw = bp[b];
    double t1 = 1.0, t2 = 1.0;   // t^(p-1), t^(p-2)
    for (int k = 0; k < pw - 1; ++k) t1 *= t;
    for (int k = 0; k < pw - 2; ++k) t2 *= t;
    double a1 = pw >= 2 ? (pw - 1) * t2 : 0.0;
    double hw = dh[0] * w[0] + dh[1] * w[1] + dh[2] * w[2];
    for (int m = 0; m < 3; ++m) {
        double g = -bk[b] * pw * (a1 * hw * dh[m] + t1 * (w[m] - dh[m] * hw) / r);
        atomicAdd(&jv[3 * ip + m], g);
        atomicAdd(&jv[3 * jp + m], -g);
    }
}

// forward-mode dual numbers (value, derivative along u) for the angle term
struct Dd {
    double v, d;
};
__device__ __forceinline__ Dd dd_add(Dd a, Dd b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dd dd_sub(Dd a, Dd b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dd dd_mul(Dd a, Dd b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dd dd_scale(double s, Dd a) { return {s * a.v, s * a.d}; }
__device__ __forceinline__ Dd dd_rsqrt(Dd a) {   // a^(-1/2)
    double r = 1.0 / sqrt(a.v);
    return {r, -0.5 * r * r * r * a.d};
}

// angles k (theta - theta0)^p (UAngle, energy.F90:5409-5506): the forces
// of the angle on its three particles, as the angle kernel writes them,
// evaluated in dual numbers along u, so that the derivative parts are
// d(force)/dx . u.  One thread per angle (FP64 atomics).
__global__ void k_jvp_angles(int nangle, const int *__restrict__ ijk, const double *__restrict__ ak,
                             const double *__restrict__ aeq, const int *__restrict__ ap,
                             const double *__restrict__ ro, mg_box box, const double *__restrict__ u,
                             double *__restrict__ jv) {
    int an = blockIdx.x * blockDim.x + threadIdx.x;
    if (an >= nangle) return;
    int jm = ijk[3 * an], ip = ijk[3 * an + 1], jp = ijk[3 * an + 2];
    Dd dm[3], dq[3];
    for (int m = 0; m < 3; ++m) {
        double x = ro[3 * ip + m] - ro[3 * jm + m], y = ro[3 * ip + m] - ro[3 * jp + m];
        if (fabs(x) > box.half[m]) x -= box.len[m] * round(x * box.inv[m]);   // PBC, anint
        if (fabs(y) > box.half[m]) y -= box.len[m] * round(y * box.inv[m]);
        dm[m] = {x, u[3 * ip + m] - u[3 * jm + m]};
        dq[m] = {y, u[3 * ip + m] - u[3 * jp + m]};
    }
    Dd dmi = dd_rsqrt(dd_add(dd_add(dd_mul(dm[0], dm[0]), dd_mul(dm[1], dm[1])), dd_mul(dm[2], dm[2])));
    Dd dpi = dd_rsqrt(dd_add(dd_add(dd_mul(dq[0], dq[0]), dd_mul(dq[1], dq[1])), dd_mul(dq[2], dq[2])));
    for (int m = 0; m < 3; ++m) {
        dm[m] = dd_mul(dm[m], dmi);
        dq[m] = dd_mul(dq[m], dpi);
    }
    Dd c = dd_add(dd_add(dd_mul(dm[0], dq[0]), dd_mul(dm[1], dq[1])), dd_mul(dm[2], dq[2]));
    double cv = fmax(-1.0, fmin(c.v, 1.0));
    double th = acos(cv), sn = sin(th);
    Dd theta = {th, -c.d / sn};                       // d acos(c) = -dc / sin(theta)
    Dd term = {th - aeq[an], theta.d};
    int pw = ap[an];
    Dd tp = {1.0, 0.0};                               // term^(p-1)
    for (int k = 0; k < pw - 1; ++k) tp = dd_mul(tp, term);
    Dd rsin = {1.0 / sn, -cos(th) * theta.d / (sn * sn)};   // 1 / sin(theta)
    Dd fac = dd_mul(dd_scale(-(double)pw * ak[an], tp), rsin);
    Dd fm = dd_mul(fac, dmi), fp = dd_mul(fac, dpi);
    for (int m = 0; m < 3; ++m) {
        Dd gm = dd_mul(fm, dd_sub(dq[m], dd_mul(c, dm[m])));   // on jm
        Dd gp = dd_mul(fp, dd_sub(dm[m], dd_mul(c, dq[m])));   // on jp
        atomicAdd(&jv[3 * jm + m], gm.d);
        atomicAdd(&jv[3 * jp + m], gp.d);
        atomicAdd(&jv[3 * ip + m], -(gm.d + gp.d));
    }
}

// u . d(force)/d(parameter) over the full Verlet list (one thread per slot,
// each unordered pair met twice): the Lennard-Jones force fsum = (24 eps /
// r^2)(2 x^2 - x), x = (sigma/r)^6, differentiated by eps_ab and sigma_ab
// (with lljcut only inside the cut), and the real-space Coulomb force
// EpsiFourPi q_i q_j g(r) d by the particle's own charge, g = (erfc(a r)/r +
// 2a/sqrt(pi) exp(-a^2 r^2)) / r^2 with Ewald, 1/r^3 without; all along
// w = u_i - u_j.  dq[p] is the particle's charge derivative, the per-pair
// parameter sums go to per-block partials [deps(nptpt), dsig(nptpt)].
struct PvjpArgs {
    const double *ro, *az;
    const int *type, *pairidx, *perm, *nnb, *nbr;
    int np, npt, nptpt, ewald, lljcut;
    mg_box box;
    double rcut2, efp, alpha;
    const double *sig, *eps, *ljrc, *r2atat, *r2umin;
    const double *u;
    double *dq, *part;
};

__global__ void __launch_bounds__(kGradThreads) k_pvjp_pairs(PvjpArgs a) {
    __shared__ double red[2 * MG_MAX_NPTPT][kGradThreads / 32];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double de[MG_MAX_NPTPT], ds[MG_MAX_NPTPT];
    for (int k = 0; k < a.nptpt; ++k) { de[k] = 0.0; ds[k] = 0.0; }
    if (i < a.np) {
        int p = a.perm[i], ti = a.type[p];
        const double *ri = a.ro + 3 * (size_t)p;
        const double *ui = a.u + 3 * (size_t)p;
        double dq = 0.0;
        int nn = a.nnb[i];
        for (int k = 0; k < nn; ++k) {
            int q = a.perm[a.nbr[(size_t)k * a.np + i]];
            const double *rj = a.ro + 3 * (size_t)q;
            double d[3] = {mg_pbc1(ri[0] - rj[0], a.box.half[0], a.box.len[0]),
                           mg_pbc1(ri[1] - rj[1], a.box.half[1], a.box.len[1]),
                           mg_pbc1(ri[2] - rj[2], a.box.half[2], a.box.len[2])};
            double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (r2 > a.rcut2) continue;
            int pair = a.pairidx[a.type[q] * a.npt + ti] - 1;
            if (r2 < a.r2atat[pair] || r2 < a.r2umin[pair]) continue;
            const double *uj = a.u + 3 * (size_t)q;
            double dw = d[0] * (ui[0] - uj[0]) + d[1] * (ui[1] - uj[1]) + d[2] * (ui[2] - uj[2]);
            double r = sqrt(r2);
            double g = a.ewald != MG_EWALD_NONE
                           ? (erfc(a.alpha * r) / r + 1.1283791670955126 * a.alpha * exp(-a.alpha * a.alpha * r2)) / r2
                           : 1.0 / (r2 * r);
            dq += a.efp * a.az[q] * g * dw;
            if (a.sig && (!a.lljcut || r < a.ljrc[pair])) {
                double sg = a.sig[pair], x = sg * sg / r2;
                x = x * x * x;
                de[pair] += 0.5 * (24.0 / r2) * (2.0 * x * x - x) * dw;
                ds[pair] += 0.5 * (144.0 * a.eps[pair] * x * (4.0 * x - 1.0) / (sg * r2)) * dw;
            }
        }
        a.dq[p] += dq;
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int nv = 2 * a.nptpt;
    for (int v = 0; v < nv; ++v) {
        double x = v < a.nptpt ? de[v] : ds[v - a.nptpt];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[v][w] = x;
    }
    __syncthreads();
    if (threadIdx.x < nv) {
        double t = 0.0;
        for (int k = 0; k < kGradThreads / 32; ++k) t += red[threadIdx.x][k];
        a.part[(size_t)blockIdx.x * nv + threadIdx.x] = t;
    }
}

__global__ void k_scale(double *__restrict__ x, size_t n, double f) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] *= f;
}

}  // namespace

// d(forceo)/dx . u at the handle's positions (FP64 form, Verlet list, MD
// or BD): a UTotal first (the slot positions and the list the pair part
// reads), then the tabulated pairs (LJ and the real-space Ewald part), the
// bonds, the angles, and the reciprocal and surface parts through the
// dipole kernels
extern "C" int mg_force_jvp(mg_handle *h, const double *u, double *jv) {
    if (!h || !u || !jv) return MG_ERR_ARG;
    if (h->form != MG_FP64) return mg_fail(h, MG_ERR_UNSUPPORTED, "mg_force_jvp needs the FP64 form");
    if (h->txintlist != MG_VLIST) return mg_fail(h, MG_ERR_UNSUPPORTED, "mg_force_jvp needs the Verlet list");
    if (h->mode == MG_MC) return mg_fail(h, MG_ERR_UNSUPPORTED, "mg_force_jvp needs an MD or BD handle");
    if (!h->list_valid) return mg_fail(h, MG_ERR_STATE, "mg_force_jvp needs a neighbour list (NList)");
    MG_TRY(mg_utotal_launch(h));
    const int np = h->np;
    // the product is linear in u: computed for u / max|u| (a fixed-point
    // scale for the reciprocal mesh independent of the size of u), then scaled
    double umax = 0.0;
    for (int i = 0; i < 3 * np; ++i) umax = std::max(umax, std::fabs(u[i]));
    if (umax == 0.0) {
        for (int i = 0; i < 3 * np; ++i) jv[i] = 0.0;
        return MG_OK;
    }
    std::vector<double> us(u, u + 3 * (size_t)np);
    for (double &x : us) x /= umax;
    double *d_u = nullptr, *d_jv = nullptr;
    MG_CUDA(h, cudaMalloc(&d_u, sizeof(double) * 6 * (size_t)np));
    d_jv = d_u + 3 * (size_t)np;
    int st = MG_OK;
    do {
        if (cudaMemcpyAsync(d_u, us.data(), sizeof(double) * 3 * np, cudaMemcpyHostToDevice, h->st) != cudaSuccess ||
            cudaMemsetAsync(d_jv, 0, sizeof(double) * 3 * np, h->st) != cudaSuccess) {
            st = mg_fail(h, MG_ERR_CUDA, "mg_force_jvp: copy failed");
            break;
        }
        JvpArgs a;
        a.pos_s = h->d_pos_s;
        a.perm = h->d_perm;
        a.nnb = h->d_nnb;
        a.nbr = h->d_nbr;
        a.np = np;
        a.npt = h->npt;
        a.nbins = h->nbins;
        a.pairidx = h->d_pairidx;
        a.tab_start = h->d_tab_start;
        a.tab_n = h->d_tab_n;
        a.zlow = h->d_zlow;
        a.coef = h->d_coef;
        a.bin_z0 = h->d_bin_z0;
        a.bin_inv = h->d_bin_inv;
        a.r2umin = h->d_r2umin;
        a.bin_kstart = h->d_bin_kstart;
        for (int m = 0; m < 3; ++m) {
            a.box.len[m] = h->boxlen[m];
            a.box.half[m] = h->boxlen2[m];
            a.box.inv[m] = h->boxleni[m];
        }
        a.rcut2 = h->rcut2;
        a.u = d_u;
        a.jv = d_jv;
        k_jvp_pairs<<<(np + 127) / 128, 128, 0, h->st>>>(a);
        h->launches++;
        if (h->nbond > 0) {
            k_jvp_bonds<<<(h->nbond + 127) / 128, 128, 0, h->st>>>(h->nbond, h->d_bond_ij, h->d_bond_k,
                                                                  h->d_bond_eq, h->d_bond_p, h->d_ro, a.box, d_u,
                                                                  d_jv);
            h->launches++;
        }
        if (h->nangle > 0) {
            k_jvp_angles<<<(h->nangle + 127) / 128, 128, 0, h->st>>>(h->nangle, h->d_angle_ijk, h->d_angle_k,
                                                                     h->d_angle_eq, h->d_angle_p, h->d_ro, a.box,
                                                                     d_u, d_jv);
            h->launches++;
        }
        if (h->ewald != MG_EWALD_NONE && (st = mg_force_jvp_rec(h, d_u, d_jv)) != MG_OK) break;
        size_t n3 = 3 * (size_t)np;
        k_scale<<<(unsigned)((n3 + 255) / 256), 256, 0, h->st>>>(d_jv, n3, h->force_fac * umax);
        h->launches++;
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(jv, d_jv, sizeof(double) * n3, cudaMemcpyDeviceToHost, h->st) != cudaSuccess ||
            cudaStreamSynchronize(h->st) != cudaSuccess)
            st = mg_fail(h, MG_ERR_CUDA, "mg_force_jvp: kernels or copy failed");
    } while (false);
    cudaFree(d_u);
    return st;
}

// u . d(forceo)/d(parameter) at the handle's positions: dq[np] for the
// particles' charges, deps and dsig[nptpt] for the pair types' LJ epsilon
// and sigma (Lorentz-Berthelot from pp as in mg_grad); forceo units
extern "C" int mg_force_pvjp(mg_handle *h, const mg_pot_params *pp, const double *u, double *dq, double *deps,
                             double *dsig) {
    if (!h || !pp || !pp->sigat || !pp->epsat || !u || !dq || !deps || !dsig) return MG_ERR_ARG;
    if (pp->npt != h->npt) return mg_fail(h, MG_ERR_ARG, "pot params npt %d != %d", pp->npt, h->npt);
    if (h->form != MG_FP64) return mg_fail(h, MG_ERR_UNSUPPORTED, "mg_force_pvjp needs the FP64 form");
    if (h->txintlist != MG_VLIST) return mg_fail(h, MG_ERR_UNSUPPORTED, "mg_force_pvjp needs the Verlet list");
    if (h->mode == MG_MC) return mg_fail(h, MG_ERR_UNSUPPORTED, "mg_force_pvjp needs an MD or BD handle");
    if (!h->list_valid) return mg_fail(h, MG_ERR_STATE, "mg_force_pvjp needs a neighbour list (NList)");
    const int np = h->np, npt = h->npt, nptpt = h->nptpt;
    double umax = 0.0;
    for (int i = 0; i < 3 * np; ++i) umax = std::max(umax, std::fabs(u[i]));
    if (umax == 0.0) {
        for (int i = 0; i < np; ++i) dq[i] = 0.0;
        for (int k = 0; k < nptpt; ++k) deps[k] = dsig[k] = 0.0;
        return MG_OK;
    }
    std::vector<double> us(u, u + 3 * (size_t)np);
    for (double &x : us) x /= umax;
    std::vector<double> ab(3 * (size_t)nptpt, 0.0);
    for (int a = 0; a < npt; ++a)
        for (int b = 0; b < npt; ++b) {
            int pair = h->h_pairidx[b * npt + a] - 1;
            double sg = 0.5 * (pp->sigat[a] + pp->sigat[b]);
            ab[pair] = sg;
            ab[nptpt + pair] = std::sqrt(pp->epsat[a] * pp->epsat[b]);
            ab[2 * nptpt + pair] = pp->ljrcut * sg;
        }
    MG_TRY(mg_utotal_launch(h));   // the reciprocal state and the surface sums of these positions
    int nblk = (np + kGradThreads - 1) / kGradThreads, nv = 2 * nptpt;
    size_t need = 4 * (size_t)np + 3 * nptpt + (size_t)nblk * nv;
    double *d = nullptr;
    MG_CUDA(h, cudaMalloc(&d, sizeof(double) * need));
    double *d_u = d, *d_dq = d_u + 3 * (size_t)np, *d_ab = d_dq + np, *d_part = d_ab + 3 * nptpt;
    int st = MG_OK;
    std::vector<double> part((size_t)nblk * nv);
    do {
        if (cudaMemcpyAsync(d_u, us.data(), sizeof(double) * 3 * np, cudaMemcpyHostToDevice, h->st) != cudaSuccess ||
            cudaMemcpyAsync(d_ab, ab.data(), sizeof(double) * 3 * nptpt, cudaMemcpyHostToDevice, h->st) !=
                cudaSuccess ||
            cudaMemsetAsync(d_dq, 0, sizeof(double) * np, h->st) != cudaSuccess) {
            st = mg_fail(h, MG_ERR_CUDA, "mg_force_pvjp: copy failed");
            break;
        }
        PvjpArgs a;
        a.ro = h->d_ro;
        a.az = h->d_az;
        a.type = h->d_type;
        a.pairidx = h->d_pairidx;
        a.perm = h->d_perm;
        a.nnb = h->d_nnb;
        a.nbr = h->d_nbr;
        a.np = np;
        a.npt = npt;
        a.nptpt = nptpt;
        a.ewald = h->ewald;
        a.lljcut = pp->lljcut;
        for (int m = 0; m < 3; ++m) {
            a.box.len[m] = h->boxlen[m];
            a.box.half[m] = h->boxlen2[m];
            a.box.inv[m] = h->boxleni[m];
        }
        a.rcut2 = h->rcut2;
        a.efp = h->EpsiFourPi;
        a.alpha = h->ualpha;
        a.sig = d_ab;
        a.eps = d_ab + nptpt;
        a.ljrc = d_ab + 2 * nptpt;
        a.r2atat = h->d_r2atat;
        a.r2umin = h->d_r2umin;
        a.u = d_u;
        a.dq = d_dq;
        a.part = d_part;
        k_pvjp_pairs<<<nblk, kGradThreads, 0, h->st>>>(a);
        h->launches++;
        if (h->ewald != MG_EWALD_NONE && (st = mg_force_pvjp_rec(h, d_u, d_dq)) != MG_OK) break;
        k_scale<<<(np + 255) / 256, 256, 0, h->st>>>(d_dq, (size_t)np, h->force_fac * umax);
        h->launches++;
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(dq, d_dq, sizeof(double) * np, cudaMemcpyDeviceToHost, h->st) != cudaSuccess ||
            cudaMemcpyAsync(part.data(), d_part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, h->st) !=
                cudaSuccess ||
            cudaStreamSynchronize(h->st) != cudaSuccess) {
            st = mg_fail(h, MG_ERR_CUDA, "mg_force_pvjp: kernels or copy failed");
            break;
        }
        for (int k = 0; k < nptpt; ++k) {
            double e = 0.0, g = 0.0;
            for (int b = 0; b < nblk; ++b) {
                e += part[(size_t)b * nv + k];
                g += part[(size_t)b * nv + nptpt + k];
            }
            deps[k] = e * h->force_fac * umax;
            dsig[k] = g * h->force_fac * umax;
        }
    } while (false);
    cudaFree(d);
    return st;
}

extern "C" int mg_grad(mg_handle *h, const mg_pot_params *pp, double *phi, double *du_deps, double *du_dsig,
                       double *du_dbox) {
    if (!h || !pp || !pp->sigat || !pp->epsat) return MG_ERR_ARG;
    std::vector<double> out;
    MG_TRY(grad_run(h, pp, phi, out));
    int nptpt = h->nptpt;
    if (du_deps)
        for (int k = 0; k < nptpt; ++k) du_deps[k] = out[k];
    if (du_dsig)
        for (int k = 0; k < nptpt; ++k) du_dsig[k] = out[nptpt + k];
    if (du_dbox)
        for (int d = 0; d < 3; ++d) du_dbox[d] = out[2 * nptpt + d] / h->boxlen[d];
    return MG_OK;
}

extern "C" int mg_virial_tensor(mg_handle *h, double *w) {
    if (!h || !w) return MG_ERR_ARG;
    std::vector<double> out;
    MG_TRY(grad_run(h, nullptr, nullptr, out));
    const double *e = out.data() + 2 * h->nptpt;   // xx, yy, zz, xy, xz, yz
    const int ix[9] = {0, 3, 4, 3, 1, 5, 4, 5, 2};
    for (int k = 0; k < 9; ++k) w[k] = e[ix[k]];
    return MG_OK;
}
