// mc.cu — Monte Carlo trial-move energy differences (rows A13, A14).
//
// Reference: DUTotal (denergy.F90:98-215) with DUTwoBody (:246-286),
// UTwoBodyANew/Old (:289-504) and their cell-list versions (:728-935),
// DUTwoBodyEwaldRecStd (:1275-1337), DUTwoBodyEwaldRecSPM (:1413-1495),
// DUTwoBodyEwaldSurf (:1504-1548); MCUpdate (mc.F90:5203-5235) with
// EwaldUpdateArray (denergy.F90:1776-1820) and UpdateCellIp
// (celllist.F90:366-382).
//
// A trial moves nptm particles ipnptm(1:nptm) to rotm(3,nptm).  Every
// difference is evaluated in FP64 (both forms), one thread block per trial,
// so that many independent trials (mg_dutotal_batch) run in one launch:
//
//   k_mc_pairs   new and old two-body energies per pair type over the
//                Verlet list (or the 27 neighbour cells' linked lists) of
//                the moving particles, plus the pairs that both move; a
//                hard-core overlap or r^2 < r2umin at the trial position
//                ends the trial as the reference does (lhsoverlap)
//   k_mc_std     standard Ewald: dS(k) = sum_m q_m (e^{ik.r_new} - e^{ik.r_old})
//                for the four sign combinations of every k-vector, and
//                kfac (|S + dS|^2 - |S|^2)
//   k_mc_stamps, k_mc_spm
//                SPME without an FFT per trial.  The reciprocal energy is
//                a quadratic form of the mesh charges, E(Q) = Q.G.Q with
//                G = c2r(meshfac)/2, and the potential mesh that UTotal
//                already computes for the forces is phi = dE/dQ = 2 G.Q.
//                The charge change of a trial, d (the old stamps removed,
//                the new ones added: 2 order^3 points per moving particle),
//                therefore changes the energy by exactly
//                     dE = d.phi + d.G.d,
//                the same number the reference gets by spreading QmeshTM and
//                transforming it (denergy.F90:1413-1495), up to rounding.
//   k_mc_final   du%rec = EpsiFourPi (dE_rec + dE_surf), du%bond and
//                du%angle of the moving chain segments (DUBond, DUAngle:
//                denergy.F90:2893-3077), du%tot, overlap
//
// On accept the moving particles take their trial positions, the mesh
// charges Q += d, the potential phi is recomputed from Q by one FFT round
// trip, S(k) takes the trial values, and the cell lists are patched.
#include <algorithm>
#include <cmath>
#include <new>

#include "mg_internal.cuh"

namespace {

constexpr int kMcThreads = 256;

struct McArgs {
    const double *ro, *az;
    const int *type, *pairidx;
    int np, npt, nptpt;
    const double *ubuf, *r2umin, *r2atat;
    const int *tab_start, *tab_n;
    mg_box box;
    double rcut2;
    int txintlist;
    // Verlet list (slot space, column-major) or MC linked cells
    const int *slot, *perm, *nnb, *nbr;
    const int *iphead, *npart, *ipnext, *cellof;
    int3 nc;
    double3 half, csi;
    int lo[3], hi[3];
    // trials: ntrial x nptm moving particles (1-based ids) and positions
    int nptm;
    const int *ip;
    const double *rt;
    const unsigned char *lptm;   // per-particle moving flags (single trial) or null
    int *err;
};

__device__ __forceinline__ bool is_moving(const McArgs &a, int t, int jp) {
    if (a.lptm) return a.lptm[jp - 1] != 0;
    return jp == a.ip[t];   // batch: one moving particle per trial
}

// table lookup as the reference's linear search from iubuflow (ubuf records
// of 12: z_low, 6 energy coefficients, 5 force coefficients)
__device__ __forceinline__ int mc_table(const McArgs &a, int pair, double r2, double *u) {
    int r = a.tab_start[pair], n = a.tab_n[pair];
    int k = 0;
    while (r2 < a.ubuf[12 * (size_t)(r + k)]) {
        if (++k >= n) return MG_ERR_IBUF;
    }
    const double *c = a.ubuf + 12 * (size_t)(r + k);
    double d = r2 - c[0];
    *u = c[1] + d * (c[2] + d * (c[3] + d * (c[4] + d * (c[5] + d * c[6]))));
    return 0;
}

__device__ __forceinline__ double mc_r2(const McArgs &a, const double *ri, const double *rj) {
    double dx = mg_pbc1(__dsub_rn(ri[0], rj[0]), a.box.half[0], a.box.len[0]);
    double dy = mg_pbc1(__dsub_rn(ri[1], rj[1]), a.box.half[1], a.box.len[1]);
    double dz = mg_pbc1(__dsub_rn(ri[2], rj[2]), a.box.half[2], a.box.len[2]);
    return mg_r2_exact(dx, dy, dz);
}

// one pair for the new (trial) configuration: 1 = overlap, <0 error
__device__ __forceinline__ int pair_new(const McArgs &a, int pair, double r2, bool cellcut, double *un) {
    if (cellcut ? !(r2 < a.rcut2) : (r2 > a.rcut2)) return 0;
    if (r2 < a.r2atat[pair]) return 1;
    if (r2 < a.r2umin[pair]) return 1;
    double u;
    int st = mc_table(a, pair, r2, &u);
    if (st) return st;
    un[pair] += u;
    return 0;
}

__device__ __forceinline__ int pair_old(const McArgs &a, int pair, double r2, bool cellcut, double *uo) {
    if (cellcut ? !(r2 < a.rcut2) : (r2 > a.rcut2)) return 0;
    if (r2 < a.r2umin[pair]) return MG_ERR_TABLE_UNDERRUN;
    double u;
    int st = mc_table(a, pair, r2, &u);
    if (st) return st;
    uo[pair] += u;
    return 0;
}

__device__ __forceinline__ int cell_of(const McArgs &a, const double *r) {
    int ix = (int)floor(__dmul_rn(__dadd_rn(r[0], a.half.x), a.csi.x));
    int iy = (int)floor(__dmul_rn(__dadd_rn(r[1], a.half.y), a.csi.y));
    int iz = (int)floor(__dmul_rn(__dadd_rn(r[2], a.half.z), a.csi.z));
    if (ix < 0 || ix >= a.nc.x || iy < 0 || iy >= a.nc.y || iz < 0 || iz >= a.nc.z) return -1;
    return ix + iy * a.nc.x + iz * a.nc.x * a.nc.y;
}

__device__ __forceinline__ int neigh_cell(const McArgs &a, int c, int k) {
    int cx = c % a.nc.x, cy = (c / a.nc.x) % a.nc.y, cz = c / (a.nc.x * a.nc.y);
    int nx = a.hi[0] - a.lo[0] + 1, ny = a.hi[1] - a.lo[1] + 1;
    int dx = a.lo[0] + k % nx, dy = a.lo[1] + (k / nx) % ny, dz = a.lo[2] + k / (nx * ny);
    int x = (cx + dx + a.nc.x) % a.nc.x, y = (cy + dy + a.nc.y) % a.nc.y, z = (cz + dz + a.nc.z) % a.nc.z;
    return x + y * a.nc.x + z * a.nc.x * a.nc.y;
}

// out per trial: [0, nptpt) new energies, [nptpt, 2 nptpt) old; flag[t]:
// 1 overlap at the trial position
__global__ void __launch_bounds__(kMcThreads) k_mc_pairs(McArgs a, double *__restrict__ out,
                                                         int *__restrict__ flag) {
    __shared__ double red[2 * MG_MAX_NPTPT][kMcThreads / 32];
    __shared__ int s_ovl, s_err;
    int t = blockIdx.x;
    const int *ipt = a.ip + (size_t)t * a.nptm;
    const double *rtt = a.rt + 3 * (size_t)t * a.nptm;
    if (threadIdx.x == 0) { s_ovl = 0; s_err = 0; }
    __syncthreads();
    double un[MG_MAX_NPTPT], uo[MG_MAX_NPTPT];
    for (int k = 0; k < a.nptpt; ++k) { un[k] = 0.0; uo[k] = 0.0; }
    int ovl = 0, err = 0;
    bool vl = a.txintlist == MG_VLIST;
    int nstencil = (a.hi[0] - a.lo[0] + 1) * (a.hi[1] - a.lo[1] + 1) * (a.hi[2] - a.lo[2] + 1);
    for (int m = 0; m < a.nptm && !ovl && !err; ++m) {
        int ip = ipt[m], ti = a.type[ip - 1];
        const double *rn = rtt + 3 * m, *ro = a.ro + 3 * (size_t)(ip - 1);
        if (vl) {
            int si = a.slot[ip - 1], nn = a.nnb[si];
            for (int k = threadIdx.x; k < nn; k += blockDim.x) {
                int jp = a.perm[a.nbr[(size_t)k * a.np + si]] + 1;
                if (is_moving(a, t, jp)) continue;
                int pair = a.pairidx[a.type[jp - 1] * a.npt + ti] - 1;
                const double *rj = a.ro + 3 * (size_t)(jp - 1);
                int st = pair_new(a, pair, mc_r2(a, rn, rj), false, un);
                if (st == 1) { ovl = 1; break; }
                if (st) { err = st; break; }
                st = pair_old(a, pair, mc_r2(a, ro, rj), false, uo);
                if (st) { err = st; break; }
            }
        } else {
            int cn = cell_of(a, rn), co = a.cellof[ip - 1];
            if (cn < 0) { err = MG_ERR_CELL; break; }
            for (int k = threadIdx.x; k < 2 * nstencil; k += blockDim.x) {
                bool isnew = k < nstencil;
                int c = neigh_cell(a, isnew ? cn : co, isnew ? k : k - nstencil);
                int jp = a.iphead[c];
                for (int q = 0; q < a.npart[c] && jp > 0; ++q, jp = a.ipnext[jp - 1]) {
                    if (is_moving(a, t, jp)) continue;
                    int pair = a.pairidx[a.type[jp - 1] * a.npt + ti] - 1;
                    const double *rj = a.ro + 3 * (size_t)(jp - 1);
                    int st = isnew ? pair_new(a, pair, mc_r2(a, rn, rj), true, un)
                                   : pair_old(a, pair, mc_r2(a, ro, rj), true, uo);
                    if (st == 1) { ovl = 1; break; }
                    if (st) { err = st; break; }
                }
                if (ovl || err) break;
            }
        }
    }
    // pairs in which both particles move
    long long n2 = (long long)a.nptm * a.nptm;
    for (long long k = threadIdx.x; k < n2 && !ovl && !err; k += blockDim.x) {
        int i = (int)(k / a.nptm), j = (int)(k % a.nptm);
        if (j <= i) continue;
        int ip = ipt[i], jp = ipt[j];
        int pair = a.pairidx[a.type[jp - 1] * a.npt + a.type[ip - 1]] - 1;
        int st = pair_new(a, pair, mc_r2(a, rtt + 3 * i, rtt + 3 * j), !vl, un);
        if (st == 1) { ovl = 1; break; }
        if (st) { err = st; break; }
        st = pair_old(a, pair, mc_r2(a, a.ro + 3 * (size_t)(ip - 1), a.ro + 3 * (size_t)(jp - 1)), !vl, uo);
        if (st) { err = st; break; }
    }
    if (ovl) atomicOr(&s_ovl, 1);
    if (err) atomicCAS(&s_err, 0, err);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = 0; k < 2 * a.nptpt; ++k) {
        double x = (k < a.nptpt) ? un[k] : uo[k - a.nptpt];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[k][w] = x;
    }
    __syncthreads();
    if (threadIdx.x < 2 * a.nptpt) {
        double s = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[threadIdx.x][q];
        out[(size_t)t * 2 * a.nptpt + threadIdx.x] = s;
    }
    if (threadIdx.x == 0) {
        flag[t] = s_ovl;
        // errors at the trial position count only when there is no overlap,
        // as the reference returns at the first overlap it meets
        if (s_err && !s_ovl) mg_dev_error(a.err, s_err, ipt[0], t, 0);
    }
}

// ---- standard Ewald ---------------------------------------------------------
struct StdArgs {
    const int4 *kv;
    const double *kfac;
    const double2 *S;
    int nk;
    double3 tpbi;
    double2 *Stm;   // single trial: S + dS for the accept, or null
};

__device__ __forceinline__ double2 cm(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// q e^{i k.r} for the four sign combinations (-x-y, -x+y, +x-y, +x+y; +z)
__device__ __forceinline__ void eikr4(double3 tpbi, int4 n, const double *r, double q, double2 *e) {
    double sx, cx, sy, cy, sz, cz;
    sincos(n.x * tpbi.x * r[0], &sx, &cx);
    sincos(n.y * tpbi.y * r[1], &sy, &cy);
    sincos(n.z * tpbi.z * r[2], &sz, &cz);
    double2 ez = make_double2(cz, sz);
    double2 yzm = cm(make_double2(cy, -sy), ez), yzp = cm(make_double2(cy, sy), ez);
    double2 qxc = make_double2(q * cx, -(q * sx)), qx = make_double2(q * cx, q * sx);
    e[0] = cm(qxc, yzm);
    e[1] = cm(qxc, yzp);
    e[2] = cm(qx, yzm);
    e[3] = cm(qx, yzp);
}

__global__ void __launch_bounds__(kMcThreads) k_mc_std(McArgs a, StdArgs s, double *__restrict__ du) {
    __shared__ double red[kMcThreads / 32];
    int t = blockIdx.x;
    const int *ipt = a.ip + (size_t)t * a.nptm;
    const double *rtt = a.rt + 3 * (size_t)t * a.nptm;
    double acc = 0.0;
    for (int k = threadIdx.x; k < s.nk; k += blockDim.x) {
        int4 n = s.kv[k];
        double2 St[4];
        for (int c = 0; c < 4; ++c) St[c] = s.S[4 * k + c];
        for (int m = 0; m < a.nptm; ++m) {
            int ip = ipt[m];
            double q = a.az[ip - 1];
            double2 en[4], eo[4];
            eikr4(s.tpbi, n, rtt + 3 * m, q, en);
            eikr4(s.tpbi, n, a.ro + 3 * (size_t)(ip - 1), q, eo);
            for (int c = 0; c < 4; ++c) {
                St[c].x += en[c].x - eo[c].x;
                St[c].y += en[c].y - eo[c].y;
            }
        }
        double tn = 0.0, to = 0.0;
        for (int c = 0; c < 4; ++c) {
            double2 S0 = s.S[4 * k + c];
            tn = tn + (St[c].x * St[c].x + St[c].y * St[c].y);
            to = to + (S0.x * S0.x + S0.y * S0.y);
        }
        acc += s.kfac[k] * (tn - to);
        if (s.Stm)
            for (int c = 0; c < 4; ++c) s.Stm[4 * k + c] = St[c];
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) red[w] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) x += red[q];
        du[t] = x;
    }
}

// ---- SPME ---------------------------------------------------------------------
struct SpmArgs {
    int n, order, nblk;          // mesh edge, spline order, blocks per trial
    double dkdr[3];
    const double *phi, *g;       // potential mesh dE/dQ and kernel G (FP64)
    int *corner;                 // [trial][set][3]      stamp upper corner
    double *w;                   // [trial][set][3][order] weights
    double *qs;                  // [trial][set]         +q (new) or -q (old)
    double *part;                // [trial][nblk][2]     d.phi, d.G.d partial sums
};

// CardinalBSpline (mollib.F90:1625-1687) values only
__device__ void bspline_values(int order, double x, double *v) {
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

// set 2m: moving particle m at its current position (charge removed),
// set 2m+1: at its trial position (charge added)
__global__ void k_mc_stamps(McArgs a, SpmArgs s, int ntrial) {
    int nsets = 2 * a.nptm;
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= ntrial * nsets * 3) return;
    int d = id % 3, set = (id / 3) % nsets, t = id / (3 * nsets);
    int m = set >> 1;
    int ip = a.ip[(size_t)t * a.nptm + m];
    const double *r = (set & 1) ? a.rt + 3 * ((size_t)t * a.nptm + m) : a.ro + 3 * (size_t)(ip - 1);
    double pos = s.dkdr[d] * r[d];
    double fl = floor(pos);
    int mm = (int)fl % s.n;
    size_t so = (size_t)t * nsets + set;
    s.corner[so * 3 + d] = mm < 0 ? mm + s.n : mm;
    bspline_values(s.order, pos - fl, s.w + (so * 3 + d) * s.order);
    if (d == 0) s.qs[so] = (set & 1) ? a.az[ip - 1] : -a.az[ip - 1];
}

__global__ void __launch_bounds__(kMcThreads) k_mc_spm(McArgs a, SpmArgs s) {
    __shared__ double red[2][kMcThreads / 32];
    int t = blockIdx.y, nsets = 2 * a.nptm, p = s.order, p3 = p * p * p;
    int S = nsets * p3, n = s.n, mn = mg_mesh_mask(n);
    const int *cor = s.corner + (size_t)t * nsets * 3;
    const double *wt = s.w + (size_t)t * nsets * 3 * p;
    const double *qs = s.qs + (size_t)t * nsets;
    double e1 = 0.0, e2 = 0.0;
    for (int ia = blockIdx.x * blockDim.x + threadIdx.x; ia < S; ia += s.nblk * blockDim.x) {
        int sa = ia / p3, r = ia % p3, ix = r % p, iy = (r / p) % p, iz = r / (p * p);
        const double *wa = wt + (size_t)sa * 3 * p;
        double da = qs[sa] * wa[ix] * wa[p + iy] * wa[2 * p + iz];
        int xa = mg_wrapm(cor[3 * sa] - ix, n, mn), ya = mg_wrapm(cor[3 * sa + 1] - iy, n, mn),
            za = mg_wrapm(cor[3 * sa + 2] - iz, n, mn);
        e1 += da * s.phi[((size_t)za * n + ya) * n + xa];
        double inner = 0.0;
        for (int sb = 0; sb < nsets; ++sb) {
            const double *wb = wt + (size_t)sb * 3 * p;
            double qb = qs[sb];
            int cbx = cor[3 * sb], cby = cor[3 * sb + 1], cbz = cor[3 * sb + 2];
            for (int jz = 0; jz < p; ++jz) {
                int dz = mg_wrapm(za - cbz + jz, n, mn);   // za - (cbz - jz)
                double wz = qb * wb[2 * p + jz];
                for (int jy = 0; jy < p; ++jy) {
                    int dy = mg_wrapm(ya - cby + jy, n, mn);
                    double wyz = wz * wb[p + jy];
                    const double *grow = s.g + ((size_t)dz * n + dy) * n;
                    for (int jx = 0; jx < p; ++jx) inner += wyz * wb[jx] * grow[mg_wrapm(xa - cbx + jx, n, mn)];
                }
            }
        }
        e2 += da * inner;
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        e1 += __shfl_down_sync(0xffffffffu, e1, o);
        e2 += __shfl_down_sync(0xffffffffu, e2, o);
    }
    if (lane == 0) { red[0][w] = e1; red[1][w] = e2; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x1 = 0.0, x2 = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { x1 += red[0][q]; x2 += red[1][q]; }
        s.part[((size_t)t * s.nblk + blockIdx.x) * 2] = x1;
        s.part[((size_t)t * s.nblk + blockIdx.x) * 2 + 1] = x2;
    }
}

// accept: Q += d, one thread in stamp order (deterministic)
__global__ void k_mc_spm_accept(McArgs a, SpmArgs s, double *__restrict__ Q) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    int nsets = 2 * a.nptm, p = s.order, n = s.n, mn = mg_mesh_mask(n);
    for (int sa = 0; sa < nsets; ++sa) {
        const int *c = s.corner + 3 * sa;
        const double *wa = s.w + (size_t)sa * 3 * p;
        for (int iz = 0; iz < p; ++iz)
            for (int iy = 0; iy < p; ++iy)
                for (int ix = 0; ix < p; ++ix) {
                    size_t idx = ((size_t)mg_wrapm(c[2] - iz, n, mn) * n + mg_wrapm(c[1] - iy, n, mn)) * n +
                                 mg_wrapm(c[0] - ix, n, mn);
                    Q[idx] += s.qs[sa] * wa[ix] * wa[p + iy] * wa[2 * p + iz];
                }
    }
}

// ---- bonds and angles of the moving chain segments ---------------------------------
struct ChainArgs {
    const int *nn;           // [5 np]: lower, upper neighbour (1-based, 0 none), bond to
                             // each (-1 none), angle at the particle as vertex (-1 none);
                             // null: no chains
    const double *bk, *beq, *ak, *aeq;
    const int *bp, *ap;
    int angles;              // some angle has k != 0
};

// x**n with the integer power expanded as products (gfortran's **)
__device__ __forceinline__ double mc_powi(double x, int n) {
    if (n == 2) return __dmul_rn(x, x);
    double r = x;
    for (int i = 1; i < n; ++i) r = __dmul_rn(r, x);
    return n == 0 ? 1.0 : r;
}

// PBC with anint (molaux.F90:104-146)
__device__ __forceinline__ double mc_pbc_anint(const McArgs &a, double d, int m) {
    if (fabs(d) > a.box.half[m]) d = __dsub_rn(d, __dmul_rn(a.box.len[m], round(__dmul_rn(d, a.box.inv[m]))));
    return d;
}

// angle_rad(-(r0 - rm), r+ - r0) (molaux.F90:836-846) with PBC on both arms
__device__ double mc_angle(const McArgs &a, const double *rm, const double *r0, const double *rp) {
    double x1[3], x2[3];
    for (int m = 0; m < 3; ++m) {
        x1[m] = -mc_pbc_anint(a, __dsub_rn(r0[m], rm[m]), m);
        x2[m] = mc_pbc_anint(a, __dsub_rn(rp[m], r0[m]), m);
    }
    double t1 = __dadd_rn(__dadd_rn(__dmul_rn(x1[0], x2[0]), __dmul_rn(x1[1], x2[1])), __dmul_rn(x1[2], x2[2]));
    double t2 = mg_r2_exact(x1[0], x1[1], x1[2]);
    double t3 = mg_r2_exact(x2[0], x2[1], x2[2]);
    double t = __ddiv_rn(t1, sqrt(__dmul_rn(t2, t3)));
    return acos(fmax(-1.0, fmin(t, 1.0)));
}

// DUBond and DUAngle of trial t: the moving list in order, a moved
// neighbour's new position from the previous / next list entry inside the
// list and from its own entry at the ends (the reference's routines assume
// that the moving segments form one string)
__device__ void mc_bonded(const McArgs &a, const ChainArgs &c, int t, double *dub, double *dua) {
    const int *ipl = a.ip + (size_t)t * a.nptm;
    const double *rtl = a.rt + 3 * (size_t)t * a.nptm;
    auto rtm = [&](int k) { return rtl + 3 * k; };
    auto rold = [&](int jp) { return a.ro + 3 * (size_t)(jp - 1); };
    auto loc = [&](int jp) {
        for (int k = 0; k < a.nptm; ++k)
            if (ipl[k] == jp) return k;
        return 0;
    };
    int last = a.nptm - 1;
    double ub = 0.0;
    for (int k = 0; k < a.nptm; ++k) {
        int ip = ipl[k];
        const int *e = c.nn + 5 * (size_t)(ip - 1);
        int jm = e[0], jp = e[1];
        for (int side = 0; side < 2; ++side) {
            int jn = side ? jp : jm;
            if (jn == 0) continue;
            const double *rn;
            if (!is_moving(a, t, jn)) rn = rold(jn);
            else if (side) continue;   // the upper bond is counted by the upper segment
            else rn = k > 0 ? rtm(k - 1) : rtm(loc(jm));
            int b = e[2 + side];
            double r2n = mc_r2(a, rtm(k), rn), r2o = mc_r2(a, rold(ip), rold(jn));
            ub = __dadd_rn(ub, __dmul_rn(c.bk[b], __dsub_rn(mc_powi(__dsub_rn(sqrt(r2n), c.beq[b]), c.bp[b]),
                                                             mc_powi(__dsub_rn(sqrt(r2o), c.beq[b]), c.bp[b]))));
        }
    }
    *dub = ub;
    double ua = 0.0;
    if (c.angles) {
        auto term = [&](int an, const double *nm, const double *n0, const double *np_, const double *om,
                        const double *o0, const double *op) {
            double tn = mc_angle(a, nm, n0, np_), to = mc_angle(a, om, o0, op);
            ua = __dadd_rn(ua, __dmul_rn(c.ak[an], __dsub_rn(mc_powi(__dsub_rn(tn, c.aeq[an]), c.ap[an]),
                                                             mc_powi(__dsub_rn(to, c.aeq[an]), c.ap[an]))));
        };
        for (int k = 0; k < a.nptm; ++k) {
            int ip = ipl[k];
            const int *e = c.nn + 5 * (size_t)(ip - 1);
            int jm = e[0], jp = e[1];
            if (jm != 0 && jp != 0 && e[4] >= 0) {
                bool mm = is_moving(a, t, jm), mp = is_moving(a, t, jp);
                const double *nm, *np_;
                if (mm && mp) {
                    bool inner = k > 0 && k < last;
                    nm = inner ? rtm(k - 1) : rtm(loc(jm));
                    np_ = inner ? rtm(k + 1) : rtm(loc(jp));
                } else if (mm) {
                    nm = k > 0 ? rtm(k - 1) : rtm(loc(jm));
                    np_ = rold(jp);
                } else {
                    nm = rold(jm);
                    np_ = mp ? (k < last ? rtm(k + 1) : rtm(loc(jp))) : rold(jp);
                }
                term(e[4], nm, rtm(k), np_, rold(jm), rold(ip), rold(jp));
            }
            if (jm != 0) {
                const int *em = c.nn + 5 * (size_t)(jm - 1);
                if (em[0] != 0 && !is_moving(a, t, jm) && em[4] >= 0)
                    term(em[4], rold(em[0]), rold(jm), rtm(k), rold(em[0]), rold(jm), rold(ip));
            }
            if (jp != 0) {
                const int *ep = c.nn + 5 * (size_t)(jp - 1);
                if (ep[1] != 0 && !is_moving(a, t, jp) && ep[4] >= 0)
                    term(ep[4], rtm(k), rold(jp), rold(ep[1]), rold(ip), rold(jp), rold(ep[1]));
            }
        }
    }
    *dua = ua;
}

// ---- combine --------------------------------------------------------------------
struct FinalArgs {
    int ntrial, nptpt, ewald, lsurf, nblk;
    double efp, surf_fac;
    const double *tw;        // k_mc_pairs output
    const int *flag;
    const double *rec_std;   // [ntrial] or null
    const double *spm_part;  // [ntrial][nblk][2] or null
    const double *dip;       // [3] sum q r of the accepted state
    ChainArgs chain;
    double *out;             // [ntrial][nptpt + 6]: du_twob(0:nptpt), du_rec, du_tot, overlap,
                             // du_bond, du_angle
};

__global__ void k_mc_final(McArgs a, FinalArgs f) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= f.ntrial) return;
    double *o = f.out + (size_t)t * (f.nptpt + 6);
    int ovl = f.flag[t];
    const double *un = f.tw + (size_t)t * 2 * f.nptpt, *uo = un + f.nptpt;
    double tn = 0.0, to = 0.0;
    for (int k = 0; k < f.nptpt; ++k) { tn = tn + un[k]; to = to + uo[k]; }
    double du_rec = 0.0, du_tot = 0.0;
    o[0] = ovl ? 0.0 : tn - to;
    for (int k = 0; k < f.nptpt; ++k) o[1 + k] = ovl ? 0.0 : un[k] - uo[k];
    if (!ovl) {
        du_tot = tn - to;
        if (f.ewald != MG_EWALD_NONE) {
            double r = 0.0;
            if (f.ewald == MG_EWALD_STD) {
                r = f.rec_std[t];
            } else {
                double x1 = 0.0, x2 = 0.0;
                for (int b = 0; b < f.nblk; ++b) {
                    x1 += f.spm_part[((size_t)t * f.nblk + b) * 2];
                    x2 += f.spm_part[((size_t)t * f.nblk + b) * 2 + 1];
                }
                r = x1 + x2;
            }
            if (f.lsurf) {
                double sx = f.dip[0], sy = f.dip[1], sz = f.dip[2];
                double tx = sx, ty = sy, tz = sz;
                for (int m = 0; m < a.nptm; ++m) {
                    int ip = a.ip[(size_t)t * a.nptm + m];
                    const double *rn = a.rt + 3 * ((size_t)t * a.nptm + m), *ro = a.ro + 3 * (size_t)(ip - 1);
                    double q = a.az[ip - 1];
                    tx = tx + q * (rn[0] - ro[0]);
                    ty = ty + q * (rn[1] - ro[1]);
                    tz = tz + q * (rn[2] - ro[2]);
                }
                r = r + f.surf_fac * ((tx * tx + ty * ty + tz * tz) - (sx * sx + sy * sy + sz * sz));
            }
            du_rec = f.efp * r;
            du_tot = du_tot + du_rec;
        }
    }
    double du_bond = 0.0, du_angle = 0.0;
    if (!ovl && f.chain.nn) {
        mc_bonded(a, f.chain, t, &du_bond, &du_angle);
        du_tot = __dadd_rn(du_tot, du_bond);
        if (f.chain.angles) du_tot = __dadd_rn(du_tot, du_angle);
    }
    o[f.nptpt + 1] = du_rec;
    o[f.nptpt + 2] = du_tot;
    o[f.nptpt + 3] = ovl;
    o[f.nptpt + 4] = du_bond;
    o[f.nptpt + 5] = du_angle;
}

__global__ void k_mc_flags(const int *__restrict__ ip, int n, unsigned char *__restrict__ lptm, unsigned char v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) lptm[ip[i] - 1] = v;
}

// accept: dipole and positions (one thread, in order)
__global__ void k_mc_move(McArgs a, double *__restrict__ ro, double *__restrict__ dip) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int m = 0; m < a.nptm; ++m) {
        int ip = a.ip[m];
        double q = a.az[ip - 1];
        for (int d = 0; d < 3; ++d) {
            if (dip) dip[d] = dip[d] + q * (a.rt[3 * m + d] - ro[3 * (size_t)(ip - 1) + d]);
            ro[3 * (size_t)(ip - 1) + d] = a.rt[3 * m + d];
        }
    }
}

__global__ void k_mc_impulse(long long *__restrict__ fx, long long v) { fx[0] = v; }

}  // namespace

// ---- host side -------------------------------------------------------------------

struct mg_mc_state {
    int cap_trial = 0;     // trials per launch
    size_t cap_tm = 0;     // moving particles over all trials of a launch
    int *d_ip = nullptr;
    double *d_rt = nullptr;
    unsigned char *d_lptm = nullptr;
    double *d_tw = nullptr, *d_rec = nullptr, *d_out = nullptr, *d_dip = nullptr;
    int *d_flag = nullptr;
    int *d_corner = nullptr;
    double *d_w = nullptr, *d_qs = nullptr, *d_spm = nullptr;
    std::vector<double> h_out;
};

constexpr int kMcMaxSpmBlocks = 64;

static mg_mc_state *mc_of(mg_handle *h) { return reinterpret_cast<mg_mc_state *>(h->mc); }

// grow the trial buffers to ntrial trials of nptm moving particles
static int mc_reserve(mg_handle *h, int ntrial, int nptm) {
    mg_mc_state *m = mc_of(h);
    size_t tm = (size_t)ntrial * nptm;
    if (ntrial > m->cap_trial) {
        int ct = std::max(ntrial, 2 * m->cap_trial);
        void *ptrs[] = {m->d_tw, m->d_rec, m->d_out, m->d_flag, m->d_spm};
        for (void *p : ptrs)
            if (p) cudaFree(p);
        m->d_spm = nullptr;
        MG_CUDA(h, cudaMalloc(&m->d_tw, sizeof(double) * 2 * MG_MAX_NPTPT * (size_t)ct));
        MG_CUDA(h, cudaMalloc(&m->d_rec, sizeof(double) * (size_t)ct));
        MG_CUDA(h, cudaMalloc(&m->d_out, sizeof(double) * (MG_MAX_NPTPT + 7) * (size_t)ct));
        MG_CUDA(h, cudaMalloc(&m->d_flag, sizeof(int) * (size_t)ct));
        if (h->ewald == MG_EWALD_SPM)
            MG_CUDA(h, cudaMalloc(&m->d_spm, sizeof(double) * 2 * kMcMaxSpmBlocks * (size_t)ct));
        m->cap_trial = ct;
        m->h_out.resize((size_t)(MG_MAX_NPTPT + 7) * ct);
    }
    if (tm > m->cap_tm) {
        size_t c = std::max(tm, 2 * m->cap_tm);
        void *ptrs[] = {m->d_ip, m->d_rt, m->d_corner, m->d_w, m->d_qs};
        for (void *p : ptrs)
            if (p) cudaFree(p);
        m->d_corner = nullptr;
        m->d_w = m->d_qs = nullptr;
        MG_CUDA(h, cudaMalloc(&m->d_ip, sizeof(int) * c));
        MG_CUDA(h, cudaMalloc(&m->d_rt, sizeof(double) * 3 * c));
        if (h->ewald == MG_EWALD_SPM) {
            MG_CUDA(h, cudaMalloc(&m->d_corner, sizeof(int) * 3 * 2 * c));
            MG_CUDA(h, cudaMalloc(&m->d_w, sizeof(double) * 3 * 2 * c * h->order));
            MG_CUDA(h, cudaMalloc(&m->d_qs, sizeof(double) * 2 * c));
        }
        m->cap_tm = c;
    }
    return MG_OK;
}

int mg_mc_init(mg_handle *h) {
    mg_mc_state *m = new (std::nothrow) mg_mc_state();
    if (!m) return mg_fail(h, MG_ERR_ALLOC, "MC state");
    h->mc = m;
    MG_CUDA(h, cudaMalloc(&m->d_lptm, h->np));
    MG_CUDA(h, cudaMemset(m->d_lptm, 0, h->np));
    MG_CUDA(h, cudaMalloc(&m->d_dip, sizeof(double) * 3));
    MG_CUDA(h, cudaMemset(m->d_dip, 0, sizeof(double) * 3));
    MG_TRY(mc_reserve(h, 1, 1));
    if (h->ewald == MG_EWALD_SPM) {
        size_t n3 = (size_t)h->nmesh * h->nmesh * h->nmesh;
        MG_CUDA(h, cudaMalloc(&h->d_Qref, sizeof(double) * n3));
        MG_CUDA(h, cudaMalloc(&h->d_phi, sizeof(double) * n3));
        MG_CUDA(h, cudaMalloc(&h->d_gker, sizeof(double) * n3));
        // G = c2r(meshfac)/2: the potential of a unit charge at mesh point 0
        k_mc_impulse<<<1, 1, 0, h->st>>>((long long *)h->d_Qfx, (long long)llround(mg_spme_fx_scale(h)));
        h->launches++;
        MG_TRY(mg_spme_potential(h));
        MG_TRY(mg_spme_mesh_to_f64(h, h->d_gker, 0.5));
        MG_CUDA(h, cudaStreamSynchronize(h->st));
    }
    return MG_OK;
}

void mg_mc_free(mg_handle *h) {
    mg_mc_state *m = mc_of(h);
    if (!m) return;
    void *ptrs[] = {m->d_ip, m->d_rt, m->d_lptm, m->d_tw, m->d_rec, m->d_out, m->d_dip, m->d_flag,
                    m->d_corner, m->d_w, m->d_qs, m->d_spm};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete m;
    h->mc = nullptr;
}

// after UTotal: the potential mesh and the dipole of the accepted state
int mg_mc_after_utotal(mg_handle *h) {
    mg_mc_state *m = mc_of(h);
    if (h->ewald == MG_EWALD_SPM) MG_TRY(mg_spme_mesh_to_f64(h, h->d_phi, 1.0));
    if (h->lsurf && h->ewald != MG_EWALD_NONE)
        MG_CUDA(h, cudaMemcpyAsync(m->d_dip, h->d_uout + h->nptpt + 1 + 4, sizeof(double) * 3,
                                   cudaMemcpyDeviceToDevice, h->st));
    MG_CUDA(h, cudaStreamSynchronize(h->st));
    return MG_OK;
}

static McArgs mc_args(mg_handle *h, int nptm, bool flags) {
    mg_mc_state *m = mc_of(h);
    McArgs a;
    a.ro = h->d_ro;
    a.az = h->d_az;
    a.type = h->d_type;
    a.pairidx = h->d_pairidx;
    a.np = h->np;
    a.npt = h->npt;
    a.nptpt = h->nptpt;
    a.ubuf = h->d_ubuf;
    a.r2umin = h->d_r2umin;
    a.r2atat = h->d_r2atat;
    a.tab_start = h->d_tab_start;
    a.tab_n = h->d_tab_n;
    for (int d = 0; d < 3; ++d) {
        a.box.len[d] = h->boxlen[d];
        a.box.half[d] = h->boxlen2[d];
        a.box.inv[d] = h->boxleni[d];
    }
    a.rcut2 = h->rcut2;
    a.txintlist = h->txintlist;
    a.slot = h->d_slot;
    a.perm = h->d_perm;
    a.nnb = h->d_nnb;
    a.nbr = h->d_nbr;
    a.iphead = h->d_iphead;
    a.npart = h->d_npart;
    a.ipnext = h->d_ipnext;
    a.cellof = h->d_cellof;
    a.nc = make_int3(h->ncell[0], h->ncell[1], h->ncell[2]);
    a.half = make_double3(h->boxlen2[0], h->boxlen2[1], h->boxlen2[2]);
    a.csi = make_double3(h->cellSizei[0], h->cellSizei[1], h->cellSizei[2]);
    for (int d = 0; d < 3; ++d) {
        a.lo[d] = (h->ncell[d] >= 3) ? -1 : 0;
        a.hi[d] = (h->ncell[d] >= 3) ? 1 : 0;
    }
    a.nptm = nptm;
    a.ip = m->d_ip;
    a.rt = m->d_rt;
    a.lptm = flags ? m->d_lptm : nullptr;
    a.err = h->d_err;
    return a;
}

static SpmArgs spm_args(mg_handle *h, int nsets_total) {
    mg_mc_state *m = mc_of(h);
    SpmArgs s;
    s.n = h->nmesh;
    s.order = h->order;
    int S = nsets_total * h->order * h->order * h->order;
    s.nblk = std::max(1, std::min(kMcMaxSpmBlocks, (S + kMcThreads - 1) / kMcThreads));
    for (int d = 0; d < 3; ++d) s.dkdr[d] = h->dkdr[d];
    s.phi = h->d_phi;
    s.g = h->d_gker;
    s.corner = m->d_corner;
    s.w = m->d_w;
    s.qs = m->d_qs;
    s.part = m->d_spm;
    return s;
}

// queue the kernels of ntrial trials of nptm moving particles each
static int mc_launch(mg_handle *h, int ntrial, int nptm, bool flags, bool store_stm) {
    mg_mc_state *m = mc_of(h);
    McArgs a = mc_args(h, nptm, flags);
    k_mc_pairs<<<ntrial, kMcThreads, 0, h->st>>>(a, m->d_tw, m->d_flag);
    FinalArgs f;
    f.ntrial = ntrial;
    f.nptpt = h->nptpt;
    f.ewald = h->ewald;
    f.lsurf = h->lsurf;
    f.efp = h->EpsiFourPi;
    f.surf_fac = 2.0 * 3.1415926535897932 / (3.0 * h->vol);
    f.tw = m->d_tw;
    f.flag = m->d_flag;
    f.rec_std = nullptr;
    f.spm_part = nullptr;
    f.dip = m->d_dip;
    f.out = m->d_out;
    f.nblk = 1;
    f.chain.nn = h->d_chain;
    f.chain.bk = h->d_bond_k;
    f.chain.beq = h->d_bond_eq;
    f.chain.bp = h->d_bond_p;
    f.chain.ak = h->d_angle_k;
    f.chain.aeq = h->d_angle_eq;
    f.chain.ap = h->d_angle_p;
    f.chain.angles = h->chain_angles;
    int nl = 2;
    if (h->ewald == MG_EWALD_STD) {
        StdArgs s;
        s.kv = h->d_kvec;
        s.kfac = h->d_kfac;
        s.S = h->d_S;
        s.nk = h->nkvec;
        s.tpbi = make_double3(h->TwoPiBoxi[0], h->TwoPiBoxi[1], h->TwoPiBoxi[2]);
        s.Stm = store_stm ? h->d_Stm : nullptr;
        k_mc_std<<<ntrial, kMcThreads, 0, h->st>>>(a, s, m->d_rec);
        f.rec_std = m->d_rec;
        ++nl;
    } else if (h->ewald == MG_EWALD_SPM) {
        SpmArgs s = spm_args(h, 2 * nptm);
        int nthr = ntrial * 2 * nptm * 3;
        k_mc_stamps<<<(nthr + 127) / 128, 128, 0, h->st>>>(a, s, ntrial);
        k_mc_spm<<<dim3(s.nblk, ntrial), kMcThreads, 0, h->st>>>(a, s);
        f.spm_part = m->d_spm;
        f.nblk = s.nblk;
        nl += 2;
    }
    k_mc_final<<<(ntrial + 127) / 128, 128, 0, h->st>>>(a, f);
    h->launches += nl;
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

static int mc_check_ready(mg_handle *h) {
    if (!h->list_valid) return mg_fail(h, MG_ERR_STATE, "mg_nlist_set has not been called");
    if (h->ewald != MG_EWALD_NONE && !h->have_rec)
        return mg_fail(h, MG_ERR_STATE, "DUTotal needs a preceding mg_utotal (Ewald arrays)");
    return MG_OK;
}

int mg_mc_dutotal(mg_handle *h, int nptm, const int32_t *ipnptm, const double *rotm, double *du_twob,
                  double *du_rec, double *du_tot, int32_t *lhsoverlap) {
    MG_TRY(mc_check_ready(h));
    for (int i = 0; i < nptm; ++i)
        if (ipnptm[i] < 1 || ipnptm[i] > h->np) return mg_fail(h, MG_ERR_ARG, "ipnptm(%d) = %d", i + 1, ipnptm[i]);
    mg_mc_state *m = mc_of(h);
    MG_TRY(mc_reserve(h, 1, nptm));
    MG_CUDA(h, cudaMemcpyAsync(m->d_ip, ipnptm, sizeof(int) * nptm, cudaMemcpyHostToDevice, h->st));
    MG_CUDA(h, cudaMemcpyAsync(m->d_rt, rotm, sizeof(double) * 3 * nptm, cudaMemcpyHostToDevice, h->st));
    bool flags = nptm > 1;
    if (flags) k_mc_flags<<<(nptm + 255) / 256, 256, 0, h->st>>>(m->d_ip, nptm, m->d_lptm, 1);
    MG_TRY(mc_launch(h, 1, nptm, flags, true));
    if (flags) k_mc_flags<<<(nptm + 255) / 256, 256, 0, h->st>>>(m->d_ip, nptm, m->d_lptm, 0);
    int nv = h->nptpt + 6;
    MG_CUDA(h, cudaMemcpyAsync(m->h_out.data(), m->d_out, sizeof(double) * nv, cudaMemcpyDeviceToHost, h->st));
    MG_TRY(mg_check_device_error(h));
    const double *o = m->h_out.data();
    bool ovl = o[h->nptpt + 3] != 0.0;
    if (du_twob)
        for (int k = 0; k <= h->nptpt; ++k) du_twob[k] = o[k];
    if (du_rec) *du_rec = o[h->nptpt + 1];
    if (du_tot) *du_tot = o[h->nptpt + 2];
    if (lhsoverlap) *lhsoverlap = ovl ? 1 : 0;
    h->nptm = nptm;
    h->trial_ok = !ovl;
    h->h_du_tot = o[h->nptpt + 2];
    return MG_OK;
}

int mg_mc_accept(mg_handle *h) {
    if (!h->trial_ok) return mg_fail(h, MG_ERR_STATE, "no accepted-able trial (mg_dutotal without overlap)");
    mg_mc_state *m = mc_of(h);
    McArgs a = mc_args(h, h->nptm, false);
    if (h->ewald == MG_EWALD_SPM) {
        // the trial's stamps are still in place: Q += d, then phi from Q
        SpmArgs s = spm_args(h, 2 * h->nptm);
        k_mc_spm_accept<<<1, 32, 0, h->st>>>(a, s, h->d_Qref);
        h->launches++;
    }
    k_mc_move<<<1, 32, 0, h->st>>>(a, h->d_ro, (h->lsurf && h->ewald != MG_EWALD_NONE) ? m->d_dip : nullptr);
    h->launches++;
    if (h->ewald == MG_EWALD_STD)
        MG_CUDA(h, cudaMemcpyAsync(h->d_S, h->d_Stm, sizeof(double2) * 4 * (size_t)h->nkvec,
                                   cudaMemcpyDeviceToDevice, h->st));
    if (h->ewald == MG_EWALD_SPM) {
        MG_TRY(mg_spme_load_mesh(h, h->d_Qref));
        MG_TRY(mg_spme_potential(h));
        MG_TRY(mg_spme_mesh_to_f64(h, h->d_phi, 1.0));
    }
    if (h->txintlist == MG_CELLLIST) {
        std::vector<int> ip(h->nptm);
        MG_CUDA(h, cudaMemcpyAsync(ip.data(), m->d_ip, sizeof(int) * h->nptm, cudaMemcpyDeviceToHost, h->st));
        MG_CUDA(h, cudaStreamSynchronize(h->st));
        for (int i = 0; i < h->nptm; ++i) MG_TRY(mg_mc_cells_update(h, ip[i]));
        h->list_stale = true;
    }
    h->have_force = false;
    h->trial_ok = false;
    return mg_check_device_error(h);
}

int mg_mc_batch(mg_handle *h, int ntrial, const int32_t *ip, const double *rt, double *du, int32_t *ovl) {
    if (ntrial == 0) return MG_OK;
    MG_TRY(mc_check_ready(h));
    for (int i = 0; i < ntrial; ++i)
        if (ip[i] < 1 || ip[i] > h->np) return mg_fail(h, MG_ERR_ARG, "ip(%d) = %d", i + 1, ip[i]);
    mg_mc_state *m = mc_of(h);
    MG_TRY(mc_reserve(h, ntrial, 1));
    MG_CUDA(h, cudaMemcpyAsync(m->d_ip, ip, sizeof(int) * ntrial, cudaMemcpyHostToDevice, h->st));
    MG_CUDA(h, cudaMemcpyAsync(m->d_rt, rt, sizeof(double) * 3 * ntrial, cudaMemcpyHostToDevice, h->st));
    MG_TRY(mc_launch(h, ntrial, 1, false, false));
    int nv = h->nptpt + 6;
    MG_CUDA(h, cudaMemcpyAsync(m->h_out.data(), m->d_out, sizeof(double) * nv * (size_t)ntrial,
                               cudaMemcpyDeviceToHost, h->st));
    MG_TRY(mg_check_device_error(h));
    for (int t = 0; t < ntrial; ++t) {
        du[t] = m->h_out[(size_t)t * nv + h->nptpt + 2];
        ovl[t] = m->h_out[(size_t)t * nv + h->nptpt + 3] != 0.0 ? 1 : 0;
    }
    h->trial_ok = false;   // a batch leaves no trial to accept
    return MG_OK;
}
