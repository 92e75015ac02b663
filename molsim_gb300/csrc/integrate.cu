// integrate.cu — device integrators around UTotal.
//
// Reference: VelVer (md.F90:252-420) with GetLinAcc (md.F90:601-625);
// BDStep (bd.F90:120-155) with GauRandom (mollib.F90:2739-2766); PBC
// (molaux.F90:104-146).
//
// GauRandom is a serial generator: a 31-bit LCG (iseed = iseed*16087 mod 2^31)
// drawn in pairs with polar Box-Muller rejection, so the position of a
// particle's deviate in the stream depends on every rejection before it.  The
// device reproduces the stream exactly in parallel: candidate pair c uses LCG
// states 2c+1 and 2c+2, reached by jump-ahead (16087^k mod 2^31); an
// exclusive scan of the acceptance flags gives each accepted pair its rank,
// and particle p takes deviates 3(p-1)+m (offset by a pending saved value).
#include <cmath>

#include "mg_internal.cuh"

namespace {

constexpr unsigned kLcgA = 16087u;
constexpr unsigned kMask31 = 0x7fffffffu;

__device__ __forceinline__ unsigned lcg_pow(unsigned long long k) {
    // 16087^k mod 2^31
    unsigned long long r = 1, b = kLcgA;
    while (k) {
        if (k & 1) r = (r * b) & kMask31;
        b = (b * b) & kMask31;
        k >>= 1;
    }
    return (unsigned)r;
}

// PBC (lbcbox): if |d| > L/2: d = d - L*anint(d/L)   (round half away from 0)
__device__ __forceinline__ double pbc_wrap(double d, double half, double len, double inv) {
    if (fabs(d) > half) d = __dsub_rn(d, __dmul_rn(len, round(__dmul_rn(d, inv))));
    return d;
}

// candidate pairs: flag, rx, ry (state of the stream is rng[0])
__global__ void k_bd_cand(const int *__restrict__ rng, int ncand, unsigned *__restrict__ flag,
                          double2 *__restrict__ val) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncand) return;
    const double f = 1.0 / 2147483648.0;
    unsigned s0 = (unsigned)rng[0];
    unsigned s1 = (unsigned)(((unsigned long long)s0 * lcg_pow(2ull * c + 1)) & kMask31);
    unsigned s2 = (s1 * kLcgA) & kMask31;
    double rx = 2.0 * (f * (double)s1 - 0.5);
    double ry = 2.0 * (f * (double)s2 - 0.5);
    double r = __dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry));
    flag[c] = (r < 1.0) ? 1u : 0u;
    val[c] = make_double2(rx, ry);
}

__global__ void k_bd_compact(const unsigned *__restrict__ flag, const int *__restrict__ rank,
                             int ncand, int *__restrict__ cidx) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < ncand && flag[c]) cidx[rank[c]] = c;
}

__device__ __forceinline__ double gauss_of_pair(const double2 *__restrict__ val, int c, int comp) {
    double2 v = val[c];
    double r = __dadd_rn(__dmul_rn(v.x, v.x), __dmul_rn(v.y, v.y));
    double fac = sqrt(-2.0 * log(r) / r);
    return (comp == 0 ? v.x : v.y) * fac;
}

struct BdArgs {
    double *ro, *drostep;
    const double *forceo, *fac1, *fac2;
    const int *type;
    int np;
    int *rng;               // [0] iseed, [1] flag
    double *save;
    const int *cidx, *rank_total;   // rank_total = scan out[ncand]
    const double2 *val;
    int ncand;
    mg_box box;
    int *err;
};

// BDStep: drostep = fac1*forceo + fac2*GauRandom; ro += drostep; PBC
__global__ void k_bd_move(BdArgs a) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.np) return;
    int off = (a.rng[1] == 0) ? 1 : 0;   // a saved deviate is pending
    int naccept = *a.rank_total;
    int t = a.type[p];
    double f1 = a.fac1[t], f2 = a.fac2[t];
    for (int m = 0; m < 3; ++m) {
        int g = 3 * p + m;
        double dev;
        if (off && g == 0) {
            dev = *a.save;
        } else {
            int hh = g - off, j = hh >> 1;
            if (j >= naccept) {
                mg_dev_error(a.err, MG_ERR_TIMEOUT, p + 1, j, naccept);
                dev = 0.0;
            } else {
                dev = gauss_of_pair(a.val, a.cidx[j], hh & 1);
            }
        }
        double d = __dadd_rn(__dmul_rn(f1, a.forceo[3 * p + m]), __dmul_rn(f2, dev));
        a.drostep[3 * p + m] = d;
        double r = __dadd_rn(a.ro[3 * p + m], d);
        a.ro[3 * p + m] = pbc_wrap(r, a.box.half[m], a.box.len[m], a.box.inv[m]);
    }
}

// advance the GauRandom state past this step's deviates (one thread)
__global__ void k_bd_state(BdArgs a) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int off = (a.rng[1] == 0) ? 1 : 0;
    int G = 3 * a.np, need = G - off;
    int J = (need + 1) / 2;
    int naccept = *a.rank_total;
    if (J > naccept) return;   // k_bd_move has flagged the error
    int clast = a.cidx[J - 1];
    unsigned s0 = (unsigned)a.rng[0];
    unsigned sn = (unsigned)(((unsigned long long)s0 * lcg_pow(2ull * (clast + 1))) & kMask31);
    a.rng[0] = (int)sn;
    if (need & 1) {
        *a.save = gauss_of_pair(a.val, clast, 1);
        a.rng[1] = 0;
    } else {
        a.rng[1] = 1;
    }
}

struct MdArgs {
    double *ro, *drostep, *rod, *rodd;
    const double *forceo, *massip;
    int np;
    double tstep, fac;
    mg_box box;
};

// VelVer positions: drostep = tstep*rod + fac*rodd; ro += drostep; PBC
__global__ void k_md_pos(MdArgs a) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.np) return;
    for (int m = 0; m < 3; ++m) {
        int i = 3 * p + m;
        double d = __dadd_rn(__dmul_rn(a.tstep, a.rod[i]), __dmul_rn(a.fac, a.rodd[i]));
        a.drostep[i] = d;
        double r = __dadd_rn(a.ro[i], d);
        a.ro[i] = pbc_wrap(r, a.box.half[m], a.box.len[m], a.box.inv[m]);
    }
}

// GetLinAcc and the velocity half-kick: rodd = massip*forceo;
// rod = rod + Half*tstep*(rodd + roddo)
__global__ void k_md_vel(MdArgs a) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.np) return;
    double mi = a.massip[p];
    for (int m = 0; m < 3; ++m) {
        int i = 3 * p + m;
        double old = a.rodd[i];
        double acc = __dmul_rn(mi, a.forceo[i]);
        a.rodd[i] = acc;
        a.rod[i] = __dadd_rn(a.rod[i], __dmul_rn(0.5 * a.tstep, __dadd_rn(acc, old)));
    }
}

mg_box box_of(const mg_handle *h) {
    mg_box b;
    for (int m = 0; m < 3; ++m) {
        b.len[m] = h->boxlen[m];
        b.half[m] = h->boxlen2[m];
        b.inv[m] = h->boxleni[m];
    }
    return b;
}

}  // namespace

int mg_integrate_bd_setup(mg_handle *h, const double *fac1, const double *fac2, int32_t iseed) {
    int npt = h->npt, np = h->np;
    if (!h->d_fac1) {
        MG_CUDA(h, cudaMalloc(&h->d_fac1, sizeof(double) * npt));
        MG_CUDA(h, cudaMalloc(&h->d_fac2, sizeof(double) * npt));
        MG_CUDA(h, cudaMalloc(&h->d_rng, sizeof(int) * 4));
        MG_CUDA(h, cudaMalloc(&h->d_rng_save, sizeof(double)));
        int J = (3 * np + 1) / 2 + 1;
        h->ncand = (int)(J * 1.35) + 4096;
        MG_CUDA(h, cudaMalloc(&h->d_cflag, sizeof(unsigned) * h->ncand));
        MG_CUDA(h, cudaMalloc(&h->d_cval, sizeof(double2) * h->ncand));
        MG_CUDA(h, cudaMalloc(&h->d_cidx, sizeof(int) * h->ncand));
        MG_CUDA(h, cudaMalloc(&h->d_scan_tmp, sizeof(int) * (h->ncand + 1)));
    }
    MG_CUDA(h, cudaMemcpy(h->d_fac1, fac1, sizeof(double) * npt, cudaMemcpyHostToDevice));
    MG_CUDA(h, cudaMemcpy(h->d_fac2, fac2, sizeof(double) * npt, cudaMemcpyHostToDevice));
    int st[4] = {iseed, 1, 0, 0};
    double zero = 0.0;
    MG_CUDA(h, cudaMemcpy(h->d_rng, st, sizeof(st), cudaMemcpyHostToDevice));
    MG_CUDA(h, cudaMemcpy(h->d_rng_save, &zero, sizeof(double), cudaMemcpyHostToDevice));
    h->bd_ready = true;
    h->have_force = false;
    return MG_OK;
}

int mg_integrate_md_setup(mg_handle *h, double tstep, const double *massip, const double *rod,
                          const double *rodd) {
    int np = h->np;
    if (!h->d_massip) {
        MG_CUDA(h, cudaMalloc(&h->d_massip, sizeof(double) * np));
        MG_CUDA(h, cudaMalloc(&h->d_rod, sizeof(double) * 3 * np));
        MG_CUDA(h, cudaMalloc(&h->d_rodd, sizeof(double) * 3 * np));
    }
    h->tstep = tstep;
    MG_CUDA(h, cudaMemcpy(h->d_massip, massip, sizeof(double) * np, cudaMemcpyHostToDevice));
    MG_CUDA(h, cudaMemcpy(h->d_rod, rod, sizeof(double) * 3 * np, cudaMemcpyHostToDevice));
    MG_CUDA(h, cudaMemcpy(h->d_rodd, rodd, sizeof(double) * 3 * np, cudaMemcpyHostToDevice));
    h->md_ready = true;
    return MG_OK;
}

// one BD step (BDStep, UTotal, list check) queued on the stream
int mg_integrate_bd_step_launch(mg_handle *h) {
    int np = h->np, nc = h->ncand;
    BdArgs a;
    a.ro = h->d_ro;
    a.drostep = h->d_drostep;
    a.forceo = h->d_forceo;
    a.fac1 = h->d_fac1;
    a.fac2 = h->d_fac2;
    a.type = h->d_type;
    a.np = np;
    a.rng = h->d_rng;
    a.save = h->d_rng_save;
    a.cidx = h->d_cidx;
    a.rank_total = h->d_scan_tmp + nc;
    a.val = (const double2 *)h->d_cval;
    a.ncand = nc;
    a.box = box_of(h);
    a.err = h->d_err;
    MG_TRY(mg_phase_begin(h, "bd_move"));
    k_bd_cand<<<(nc + 255) / 256, 256, 0, h->st>>>(h->d_rng, nc, h->d_cflag, (double2 *)h->d_cval);
    mg_scan_exclusive(h, (const int *)h->d_cflag, h->d_scan_tmp, nc, nullptr);
    k_bd_compact<<<(nc + 255) / 256, 256, 0, h->st>>>(h->d_cflag, h->d_scan_tmp, nc, h->d_cidx);
    k_bd_move<<<(np + 255) / 256, 256, 0, h->st>>>(a);
    k_bd_state<<<1, 32, 0, h->st>>>(a);
    h->launches += 4;
    MG_TRY(mg_phase_end(h, "bd_move"));
    MG_TRY(mg_utotal_launch(h));
    MG_TRY(mg_phase_begin(h, "list"));
    MG_TRY(mg_lists_check(h));
    MG_TRY(mg_lists_build(h, true));
    MG_TRY(mg_phase_end(h, "list"));
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

// one velocity-Verlet step queued on the stream
int mg_integrate_md_step_launch(mg_handle *h) {
    MdArgs a;
    a.ro = h->d_ro;
    a.drostep = h->d_drostep;
    a.rod = h->d_rod;
    a.rodd = h->d_rodd;
    a.forceo = h->d_forceo;
    a.massip = h->d_massip;
    a.np = h->np;
    a.tstep = h->tstep;
    a.fac = 0.5 * (h->tstep * h->tstep);
    a.box = box_of(h);
    int gb = (h->np + 255) / 256;
    MG_TRY(mg_phase_begin(h, "md_pos"));
    k_md_pos<<<gb, 256, 0, h->st>>>(a);
    h->launches++;
    MG_TRY(mg_phase_end(h, "md_pos"));
    MG_TRY(mg_utotal_launch(h));
    k_md_vel<<<gb, 256, 0, h->st>>>(a);
    h->launches++;
    MG_TRY(mg_phase_begin(h, "list"));
    MG_TRY(mg_lists_check(h));
    MG_TRY(mg_lists_build(h, true));
    MG_TRY(mg_phase_end(h, "list"));
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}
