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

constexpr int kCandBlock = 1024;   // candidates per block

// Candidate pairs c = blockIdx.x*1024 + threadIdx.x use LCG states 2c+1, 2c+2
// after rng[0].  Each block compacts its accepted pairs in candidate order
// and stores the two deviates (rx*fac, ry*fac) of each, its accepted count
// in blkcnt and the candidate index of each accepted pair in cidx.
template <bool F32>
__global__ void __launch_bounds__(kCandBlock) k_bd_cand(const int *__restrict__ rng, int ncand,
                                                         double2 *__restrict__ gval,
                                                         int *__restrict__ cidx,
                                                         int *__restrict__ blkcnt) {
    __shared__ int wcount[kCandBlock / 32];
    int c = blockIdx.x * kCandBlock + threadIdx.x;
    const double f = 1.0 / 2147483648.0;
    bool acc = false;
    double rx = 0.0, ry = 0.0, r = 2.0;
    if (c < ncand) {
        unsigned s0 = (unsigned)rng[0];
        unsigned s1 = (unsigned)(((unsigned long long)s0 * lcg_pow(2ull * c + 1)) & kMask31);
        unsigned s2 = (s1 * kLcgA) & kMask31;
        rx = 2.0 * (f * (double)s1 - 0.5);
        ry = 2.0 * (f * (double)s2 - 0.5);
        r = __dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry));
        acc = r < 1.0;
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned ball = __ballot_sync(0xffffffffu, acc);
    if (lane == 0) wcount[w] = __popc(ball);
    __syncthreads();
    if (w == 0) {
        int x = wcount[lane];
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        wcount[lane] = x;   // inclusive prefix over warps
        if (lane == 31) blkcnt[blockIdx.x] = x;
    }
    __syncthreads();
    if (acc) {
        int rank = (w ? wcount[w - 1] : 0) + __popc(ball & ((1u << lane) - 1u));
        size_t o = (size_t)blockIdx.x * kCandBlock + rank;
        double2 g;
        if (F32) {   // mixed form: the Box-Muller transform in FP32
            float rf = (float)r;
            float fac = sqrtf(-2.0f * __logf(rf) / rf);
            g = make_double2((double)((float)rx * fac), (double)((float)ry * fac));
        } else {     // GauRandom: fac = sqrt(-two*log(r)/r)
            double fac = sqrt(-2.0 * log(r) / r);
            g = make_double2(rx * fac, ry * fac);
        }
        gval[o] = g;
        cidx[o] = c;
    }
}

struct BdArgs {
    double *ro, *drostep;
    const double *forceo, *fac1, *fac2;
    const int *type;
    int np;
    int *rng;               // [0] iseed, [1] flag (1: next call draws a new pair), [3] block counter
    double *save;
    const double2 *gval;
    const int *cidx, *blkcnt;
    int nblk;
    mg_box box;
    int *err;
    mg_chk_args chk;        // the list check's first pass runs here
    const mg_hostio *io;    // host positions in and out (nullptr: device only)
};

// prefix of the per-block accepted counts in shared memory (inclusive): all
// threads load (one memory round trip per blockDim counts), warps scan, the
// warp totals are scanned by warp 0
__device__ __forceinline__ void load_block_prefix(const int *__restrict__ blkcnt, int nblk, int *sp) {
    __shared__ int wtot[32];
    __shared__ int carry_s;
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    for (int base = 0; base < nblk; base += blockDim.x) {
        int i = base + threadIdx.x;
        int x = (i < nblk) ? blkcnt[i] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wtot[w] = x;
        __syncthreads();
        if (w == 0) {
            int t = (lane < nw) ? wtot[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            if (lane < nw) wtot[lane] = t;
        }
        __syncthreads();
        int c = carry_s;
        if (i < nblk) sp[i] = c + x + (w ? wtot[w - 1] : 0);
        __syncthreads();
        if (threadIdx.x == 0) carry_s = c + wtot[nw - 1];
        __syncthreads();
    }
}

// accepted pair j -> offset of its stored deviates (-1 if the stream ran short)
__device__ __forceinline__ long pair_slot(const int *sp, int nblk, int j) {
    if (nblk == 0 || j >= sp[nblk - 1]) return -1;
    int lo = 0, hi = nblk - 1;   // first block with inclusive prefix > j
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (sp[mid] > j) hi = mid;
        else lo = mid + 1;
    }
    int before = lo ? sp[lo - 1] : 0;
    return (long)lo * kCandBlock + (j - before);
}

// BDStep: drostep = fac1*forceo + fac2*GauRandom; ro += drostep; PBC; then
// the first pass of the list check on drostep.  The last block to finish
// also advances the GauRandom state past this step's deviates (every block
// has read the old state by then).
__global__ void __launch_bounds__(kChkThreads) k_bd_move(BdArgs a) {
    extern __shared__ int sp[];
    __shared__ bool last;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    bool reset = (*a.chk.flag != 0);
    double *hro = a.io ? a.io->ro : nullptr;   // host positions, read then written
    // the particle's own data first: none of it waits for the block prefix
    double fo[3] = {0.0, 0.0, 0.0}, r0[3] = {0.0, 0.0, 0.0}, sum0[3] = {0.0, 0.0, 0.0}, f1 = 0.0, f2 = 0.0;
    if (p < a.np) {
        int t = a.type[p];
        f1 = a.fac1[t];
        f2 = a.fac2[t];
        for (int m = 0; m < 3; ++m) {
            fo[m] = a.forceo[3 * p + m];
            r0[m] = hro ? hro[3 * p + m] : a.ro[3 * p + m];
            if (!reset) sum0[m] = a.chk.drosum[3 * p + m];
        }
    }
    load_block_prefix(a.blkcnt, a.nblk, sp);
    int off = (a.rng[1] == 0) ? 1 : 0;   // a saved deviate is pending
    double dd[3] = {0.0, 0.0, 0.0};
    if (p < a.np) {
        for (int m = 0; m < 3; ++m) {
            int g = 3 * p + m;
            double dev;
            if (off && g == 0) {
                dev = *a.save;
            } else {
                int hh = g - off;
                long slot = pair_slot(sp, a.nblk, hh >> 1);
                if (slot < 0) {
                    mg_dev_error(a.err, MG_ERR_TIMEOUT, p + 1, hh >> 1, a.nblk);
                    dev = 0.0;
                } else {
                    double2 v = a.gval[slot];
                    dev = (hh & 1) ? v.y : v.x;
                }
            }
            double d = __dadd_rn(__dmul_rn(f1, fo[m]), __dmul_rn(f2, dev));
            a.drostep[3 * p + m] = d;
            dd[m] = d;
            double r = __dadd_rn(r0[m], d);
            r = pbc_wrap(r, a.box.half[m], a.box.len[m], a.box.inv[m]);
            a.ro[3 * p + m] = r;
            if (hro) hro[3 * p + m] = r;
        }
    }
    mg_chk_accum_from(p, a.np, dd[0], dd[1], dd[2], reset, sum0, a.chk.drosum, a.chk.r2out, a.chk.blkmax);
    __syncthreads();   // this block has read the state (rng, save)
    if (threadIdx.x == 0) {
        __threadfence();
        last = (atomicAdd(&a.rng[3], 1) == (int)gridDim.x - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    a.rng[3] = 0;
    int need = 3 * a.np - off;
    int J = (need + 1) / 2;
    long slot = pair_slot(sp, a.nblk, J - 1);
    if (slot < 0) return;   // the move has flagged the error
    int clast = a.cidx[slot];
    unsigned s0 = (unsigned)a.rng[0];
    unsigned sn = (unsigned)(((unsigned long long)s0 * lcg_pow(2ull * (clast + 1))) & kMask31);
    a.rng[0] = (int)sn;
    if (need & 1) {
        *a.save = a.gval[slot].y;
        a.rng[1] = 0;
    } else {
        a.rng[1] = 1;
    }
}

// the step's results to the host buffers of a host-I/O step: forceo
// (coalesced writes), the energies and the device error word
__global__ void k_forces_to_host(const double *__restrict__ forceo, const mg_hostio *io, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) io->forceo[i] = forceo[i];
    if (blockIdx.x == 0) {
        if (threadIdx.x < io->nu) io->stage[threadIdx.x] = io->uout[threadIdx.x];
        if (threadIdx.x < 4) reinterpret_cast<int *>(io->stage + io->nu)[threadIdx.x] = io->err[threadIdx.x];
    }
}

struct MdArgs {
    double *ro, *drostep, *rod, *rodd;
    const double *forceo, *massip;
    int np;
    double tstep, fac;
    mg_box box;
    mg_chk_args chk;        // the list check's first pass runs in k_md_pos
};

// VelVer positions: drostep = tstep*rod + fac*rodd; ro += drostep; PBC; then
// the first pass of the list check on drostep
__global__ void __launch_bounds__(kChkThreads) k_md_pos(MdArgs a) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    bool reset = (*a.chk.flag != 0);
    double dd[3] = {0.0, 0.0, 0.0};
    if (p < a.np) {
        for (int m = 0; m < 3; ++m) {
            int i = 3 * p + m;
            double d = __dadd_rn(__dmul_rn(a.tstep, a.rod[i]), __dmul_rn(a.fac, a.rodd[i]));
            a.drostep[i] = d;
            dd[m] = d;
            double r = __dadd_rn(a.ro[i], d);
            a.ro[i] = pbc_wrap(r, a.box.half[m], a.box.len[m], a.box.inv[m]);
        }
    }
    mg_chk_accum(p, a.np, dd[0], dd[1], dd[2], reset, a.chk.drosum, a.chk.r2out, a.chk.blkmax);
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
        // acceptance is pi/4: 1.35 J + 4096 candidates leave a margin of
        // hundreds of standard deviations
        int nblk = ((int)(J * 1.35) + 4096 + kCandBlock - 1) / kCandBlock;
        h->ncand = nblk * kCandBlock;
        MG_CUDA(h, cudaMalloc(&h->d_cval, sizeof(double2) * h->ncand));
        MG_CUDA(h, cudaMalloc(&h->d_cidx, sizeof(int) * h->ncand));
        MG_CUDA(h, cudaMalloc(&h->d_scan_tmp, sizeof(int) * nblk));
    }
    MG_CUDA(h, cudaMemcpy(h->d_fac1, fac1, sizeof(double) * npt, cudaMemcpyHostToDevice));
    MG_CUDA(h, cudaMemcpy(h->d_fac2, fac2, sizeof(double) * npt, cudaMemcpyHostToDevice));
    int st[4] = {iseed, 1, 0, 0};
    double zero = 0.0;
    MG_CUDA(h, cudaMemcpy(h->d_rng, st, sizeof(st), cudaMemcpyHostToDevice));
    MG_CUDA(h, cudaMemcpy(h->d_rng_save, &zero, sizeof(double), cudaMemcpyHostToDevice));
    h->bd_ready = true;
    h->have_force = false;
    h->cand_ready = false;
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

static int list_step(mg_handle *h, bool accum_done);

// GauRandom candidate pairs from the generator state in d_rng, on h->st
int mg_integrate_bd_cand(mg_handle *h) {
    int nc = h->ncand, nblk = nc / kCandBlock;
    if (h->form == MG_MIXED)
        k_bd_cand<true><<<nblk, kCandBlock, 0, h->st>>>(h->d_rng, nc, (double2 *)h->d_cval, h->d_cidx, h->d_scan_tmp);
    else
        k_bd_cand<false><<<nblk, kCandBlock, 0, h->st>>>(h->d_rng, nc, (double2 *)h->d_cval, h->d_cidx, h->d_scan_tmp);
    h->launches++;
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

int mg_integrate_bd_prime(mg_handle *h) {
    if (!h->cand_ready) MG_TRY(mg_integrate_bd_cand(h));
    h->cand_ready = true;
    return MG_OK;
}

// one BD step (BDStep, UTotal, list check) queued on the stream.  Uncaptured,
// the step draws its own candidates first; captured into a graph (use_cond),
// it finds them drawn (mg_integrate_bd_prime, or the previous step) and
// draws the next step's after its move, beside the UTotal where it can.
int mg_integrate_bd_step_launch(mg_handle *h) {
    bool prefetch = h->use_cond;
    int np = h->np, nc = h->ncand, nblk = nc / kCandBlock;
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
    a.gval = (const double2 *)h->d_cval;
    a.cidx = h->d_cidx;
    a.blkcnt = h->d_scan_tmp;
    a.nblk = nblk;
    a.box = box_of(h);
    a.err = h->d_err;
    a.chk = mg_lists_chk_args(h);
    a.io = h->hostio ? h->d_hostio : nullptr;
    size_t sm = sizeof(int) * nblk;
    if (!prefetch) {
        MG_TRY(mg_phase_begin(h, "bd_rng"));
        MG_TRY(mg_integrate_bd_cand(h));
        MG_TRY(mg_phase_end(h, "bd_rng"));
    }
    MG_TRY(mg_phase_begin(h, "bd_move"));
    k_bd_move<<<(np + kChkThreads - 1) / kChkThreads, kChkThreads, sm, h->st>>>(a);   // advances the GauRandom state too
    h->launches += 1;
    MG_TRY(mg_phase_end(h, "bd_move"));
    h->chk_side = true;
    h->cand_side = prefetch;
    int ust = mg_utotal_launch(h);
    h->chk_side = false;
    h->cand_side = false;
    MG_TRY(ust);
    if (prefetch && !h->cand_queued) MG_TRY(mg_integrate_bd_cand(h));   // UTotal did not fork
    h->cand_queued = false;
    if (!prefetch) h->cand_ready = false;   // consumed, none drawn ahead
    if (h->hostio) {   // the forces straight into the host buffer
        k_forces_to_host<<<(3 * np + 255) / 256, 256, 0, h->st>>>(h->d_forceo, h->d_hostio, 3 * np);
        h->launches++;
    }
    MG_TRY(list_step(h, true));
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

// NList(iSimulationStep) inside a device step.  In a captured step the
// rebuild sits in the graph's conditional node.  Uncaptured (phase timing,
// profiling) the host reads the rebuild flag after the check and launches the
// build only when it is due, so that uncaptured steps run the same kernels as
// the graph does.
static int list_step(mg_handle *h, bool accum_done) {
    if (!h->chk_queued) {   // else UTotal queued it beside the mesh path
        MG_TRY(mg_phase_begin(h, "list"));
        MG_TRY(mg_lists_check(h, accum_done));
        MG_TRY(mg_phase_end(h, "list"));
    }
    h->chk_queued = false;
    if (h->use_cond) return MG_OK;
    int flag = 0;
    MG_CUDA(h, cudaMemcpyAsync(&flag, h->d_rebuild, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    MG_CUDA(h, cudaStreamSynchronize(h->st));
    if (flag) {
        MG_TRY(mg_phase_begin(h, "list_build"));
        MG_TRY(mg_lists_build(h, false));
        MG_TRY(mg_phase_end(h, "list_build"));
    }
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
    a.chk = mg_lists_chk_args(h);
    int gb = (h->np + kChkThreads - 1) / kChkThreads;
    MG_TRY(mg_phase_begin(h, "md_pos"));
    k_md_pos<<<gb, kChkThreads, 0, h->st>>>(a);
    h->launches++;
    MG_TRY(mg_phase_end(h, "md_pos"));
    h->chk_side = true;
    int ust = mg_utotal_launch(h);
    h->chk_side = false;
    MG_TRY(ust);
    k_md_vel<<<gb, kChkThreads, 0, h->st>>>(a);
    h->launches++;
    MG_TRY(list_step(h, true));
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}
