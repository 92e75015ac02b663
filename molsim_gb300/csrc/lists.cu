// lists.cu — cell list and Verlet list on the device (rows A1-A5).
//
// Reference: InitCellList / pcellro / SetCellList (celllist.F90:76-410),
// SetVListMD / SetVListMC (nlist.F90:724-890), the rebuild rule of
// NList(iSimulationStep) (nlist.F90:598-621) and PBCr2 (molaux.F90:149-184).
//
// GB300 form: the reference's per-cell linked lists become a counting sort of
// particles into cell order (slot space); the Verlet list is built per slot
// from the 27 neighbour cells and stored column-major (nbr[k*np+slot]) so a
// warp reading neighbour k of 32 consecutive slots touches one 128-byte line.
// Inside a cell particles are ordered by index, so lists are deterministic.
// Membership decisions (cell index, r^2 < (rcut+drnlist)^2) use round-to-
// nearest FP64 without contraction, giving the reference's sets bit-exactly.
#include <algorithm>
#include <cstdio>

#include "mg_internal.cuh"

namespace {



__global__ void k_cell_assign(const double *__restrict__ ro, int np, double3 half, double3 csi,
                              int3 nc, int *__restrict__ cellof, int *__restrict__ count,
                              int *__restrict__ err, const int *__restrict__ gate) {
    if (gate && *gate == 0) return;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    // i = floor((ro + boxlen2) * cellSizei)   (celllist.F90:303)
    int ix = (int)floor(__dmul_rn(__dadd_rn(ro[3 * p + 0], half.x), csi.x));
    int iy = (int)floor(__dmul_rn(__dadd_rn(ro[3 * p + 1], half.y), csi.y));
    int iz = (int)floor(__dmul_rn(__dadd_rn(ro[3 * p + 2], half.z), csi.z));
    if (ix < 0 || ix >= nc.x || iy < 0 || iy >= nc.y || iz < 0 || iz >= nc.z) {
        // outside the grid (the reference indexes out of bounds here): report
        // it and clamp so the sort below stays a permutation
        mg_dev_error(err, MG_ERR_CELL, p + 1, 0, 0);
        ix = min(max(ix, 0), nc.x - 1);
        iy = min(max(iy, 0), nc.y - 1);
        iz = min(max(iz, 0), nc.z - 1);
    }
    int c = ix + iy * nc.x + iz * nc.x * nc.y;
    cellof[p] = c;
    atomicAdd(&count[c], 1);
}

// Exclusive scan of the cell counts in two passes over tiles of kScanTile
// cells: k_scan_tiles scans each tile (coalesced loads, a block per tile) and
// records the tile total; k_scan_fix adds the sum of the earlier tiles' totals
// and writes out[n] = total.  out[i] = sum(in[0..i)).
__device__ __forceinline__ int block_excl_scan(int s, int *warp_sums, int *total) {
    int t = threadIdx.x, lane = t & 31, w = t >> 5, nw = blockDim.x >> 5;
    int v = s;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31) warp_sums[w] = v;
    __syncthreads();
    if (w == 0) {
        int x = (lane < nw) ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane < nw) warp_sums[lane] = x;
    }
    __syncthreads();
    if (total) *total = warp_sums[nw - 1];
    return v - s + (w > 0 ? warp_sums[w - 1] : 0);
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int *__restrict__ in, int *__restrict__ out,
                                                             int n, int *__restrict__ tilesum,
                                                             const int *__restrict__ gate) {
    if (gate && *gate == 0) return;
    __shared__ int warp_sums[32];
    constexpr int per = kScanTile / kScanThreads;
    int base = blockIdx.x * kScanTile + threadIdx.x * per;
    int v[per], s = 0;
#pragma unroll
    for (int k = 0; k < per; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        s += v[k];
    }
    int tot;
    int excl = block_excl_scan(s, warp_sums, &tot);
#pragma unroll
    for (int k = 0; k < per; ++k) {
        if (base + k < n) out[base + k] = excl;
        excl += v[k];
    }
    if (threadIdx.x == 0) tilesum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_fix(int *__restrict__ out, int n,
                                                           const int *__restrict__ tilesum, int ntile,
                                                           const int *__restrict__ gate) {
    if (gate && *gate == 0) return;
    __shared__ int warp_sums[32];
    __shared__ int off;
    int b = blockIdx.x;
    int s = 0;
    for (int k = threadIdx.x; k < b; k += blockDim.x) s += tilesum[k];
    int tot;
    block_excl_scan(s, warp_sums, &tot);
    if (threadIdx.x == 0) off = tot;
    __syncthreads();
    int o = off;
    if (o != 0) {
        for (int i = b * kScanTile + threadIdx.x; i < min(n, (b + 1) * kScanTile); i += blockDim.x) out[i] += o;
    }
    if (b == ntile - 1 && threadIdx.x == 0) out[n] = o + tilesum[b];
}

__global__ void k_cell_scatter(const int *__restrict__ cellof, int np, const int *__restrict__ start,
                               int *__restrict__ fill, int *__restrict__ perm,
                               const int *__restrict__ gate) {
    if (gate && *gate == 0) return;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    int c = cellof[p];
    int slot = start[c] + atomicAdd(&fill[c], 1);
    perm[slot] = p;
}

// order each cell's particles by index (insertion sort; cells are small)
__global__ void k_cell_sort(int ncell, const int *__restrict__ start, int *__restrict__ perm,
                            const int *__restrict__ gate) {
    if (gate && *gate == 0) return;
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    int b = start[c], e = start[c + 1];
    for (int i = b + 1; i < e; ++i) {
        int v = perm[i], j = i - 1;
        while (j >= b && perm[j] > v) {
            perm[j + 1] = perm[j];
            --j;
        }
        perm[j + 1] = v;
    }
}

// slot of each particle, and the positions in slot order with the cell
// index in .w (exact: cell indices are far below 2^53)
__global__ void k_slot_of(const int *__restrict__ perm, const double *__restrict__ ro,
                          const int *__restrict__ cellof, int np, int *__restrict__ slot,
                          double4 *__restrict__ ro_slot, float4 *__restrict__ ro_f,
                          const int *__restrict__ gate) {
    if (gate && *gate == 0) return;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= np) return;
    int p = perm[s];
    slot[p] = s;
    double x = ro[3 * p], y = ro[3 * p + 1], z = ro[3 * p + 2];
    ro_slot[s] = make_double4(x, y, z, (double)cellof[p]);
    ro_f[s] = make_float4((float)x, (float)y, (float)z, 0.0f);
}

struct StencilArgs {
    int3 nc;
    int lo[3], hi[3];   // neighbour offset range per dimension ({-1..1} or {0..0})
};

// Verlet list of slot i: all slots j != i in the neighbour cells with
// r^2 < rs2cut (SetVListMD/MC membership; the half-list ownership rule is
// applied only when the list is exported in the reference layout).
// Positions are read in slot order (ro_slot), so the candidates of a cell
// are consecutive.  The three cells x-1, x, x+1 of a stencil row are
// consecutive cells too, so a row that does not wrap around the box is one
// slot range; the nine rows' ranges are loaded before the distance loop.
// Neighbours are listed by cell (dz, dy, dx order) and by slot within a
// cell, as cell-by-cell scanning would list them.
// Membership is decided by the reference's FP64 arithmetic, but GB300 issues
// FP64 at 1/64 of the FP32 rate, so every candidate first gets an FP32
// distance from FP32 copies of the positions (ro_f).  Its error is far below
// `band` (see vlist_band); only candidates within `band` of the cutoff are
// decided in FP64, which gives the same set as testing every candidate so.
__device__ __forceinline__ float pbc1f(float d, float half, float len) {
    return (fabsf(d) > half) ? d - copysignf(len, d) : d;
}
__device__ __forceinline__ int wrap_cell(int x, int n) {
    x += (x < 0) ? n : 0;
    return x - ((x >= n) ? n : 0);
}

struct VlistBand {
    float lo, hi;        // FP32 r^2 below lo: inside; at or above hi: outside
    float half[3], len[3];
};

__global__ void __launch_bounds__(128) k_vlist(const double4 *__restrict__ ro_slot,
                                               const float4 *__restrict__ ro_f,
                                               const int *__restrict__ start, int np, StencilArgs sa,
                                               mg_box box, VlistBand band, double rs2cut, int maxnb,
                                               int *__restrict__ nnb, int *__restrict__ nbr,
                                               const int *__restrict__ perm, int *__restrict__ err,
                                               const int *__restrict__ gate) {
    if (gate && *gate == 0) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    double4 me = ro_slot[i];
    float4 mf = ro_f[i];
    int c = (int)me.w;
    int cx = c % sa.nc.x, cy = (c / sa.nc.x) % sa.nc.y, cz = c / (sa.nc.x * sa.nc.y);
    // a row is one range when it spans three distinct cells without wrapping
    // (or is a collapsed dimension's single cell)
    bool one = (sa.lo[0] == sa.hi[0]) || (cx >= 1 && cx + 1 < sa.nc.x);
    // the nine rows (dz, dy in -1..1; the offsets a collapsed dimension does
    // not have are empty), their slot ranges loaded up front
    int rb[9], re[9];
    unsigned rows = 0;   // bit r: row r exists
#pragma unroll
    for (int r = 0; r < 9; ++r) {
        int dz = r / 3 - 1, dy = r % 3 - 1;
        rb[r] = 0;
        re[r] = 0;
        if (dz < sa.lo[2] || dz > sa.hi[2] || dy < sa.lo[1] || dy > sa.hi[1]) continue;
        rows |= 1u << r;
        int z = wrap_cell(cz + dz, sa.nc.z);
        int y = wrap_cell(cy + dy, sa.nc.y);
        int row = (y + z * sa.nc.y) * sa.nc.x;
        if (one) {
            rb[r] = start[row + cx + sa.lo[0]];
            re[r] = start[row + cx + sa.hi[0] + 1];
        } else {
            rb[r] = row;   // a wrapping row: its three cells are visited one by one below
            re[r] = -1;
        }
    }
    int cnt = 0;
#pragma unroll
    for (int r = 0; r < 9; ++r) {
        if (!(rows >> r & 1u)) continue;   // an offset of a collapsed dimension
        for (int d = 0; d < (one ? 1 : 3); ++d) {
            int b, e;
            if (one) {
                b = rb[r];
                e = re[r];
            } else {
                int cc = rb[r] + wrap_cell(cx + d - 1, sa.nc.x);
                b = start[cc];
                e = start[cc + 1];
            }
            for (int j = b; j < e; ++j) {
                if (j == i) continue;
                float4 qf = ro_f[j];
                float fx = pbc1f(mf.x - qf.x, band.half[0], band.len[0]);
                float fy = pbc1f(mf.y - qf.y, band.half[1], band.len[1]);
                float fz = pbc1f(mf.z - qf.z, band.half[2], band.len[2]);
                float r2f = fx * fx + fy * fy + fz * fz;
                bool in = r2f < band.lo;
                if (!in && r2f < band.hi) {   // near the cutoff: the reference's FP64 test
                    double4 q = ro_slot[j];
                    double ddx = mg_pbc1(__dsub_rn(me.x, q.x), box.half[0], box.len[0]);
                    double ddy = mg_pbc1(__dsub_rn(me.y, q.y), box.half[1], box.len[1]);
                    double ddz = mg_pbc1(__dsub_rn(me.z, q.z), box.half[2], box.len[2]);
                    in = mg_r2_exact(ddx, ddy, ddz) < rs2cut;
                }
                if (in) {
                    if (cnt < maxnb) nbr[(size_t)cnt * np + i] = j;
                    ++cnt;
                }
            }
        }
    }
    int p = perm[i];
    if (cnt > maxnb) {
        mg_dev_error(err, MG_ERR_NEIGH_OVERFLOW, p + 1, cnt, maxnb);
        cnt = maxnb;
    }
    nnb[i] = cnt;
}

// ---- NList(iSimulationStep) rebuild rule (nlist.F90:598-621) ---------------
// The reference scans particles in order keeping r2max1 (running maximum) and
// r2max2 (largest value that was not a new running maximum when met).  The
// device reproduces that exactly: pass 1 accumulates drosum and block maxima,
// pass 2 finds per block the non-record values given the maximum of all
// earlier blocks, pass 3 combines.
// r^2 >= 0, and non-negative doubles order as their 64-bit patterns, so the
// maxima and the prefix maximum below run on integers (no FP64 pipe)
__device__ __forceinline__ long long chk_max(long long a, long long b) { return a > b ? a : b; }

__global__ void __launch_bounds__(kChkThreads) k_chk_accum(const double *__restrict__ drostep,
                                                           double *__restrict__ drosum, double *__restrict__ r2out,
                                                           double *__restrict__ blkmax, int np,
                                                           const int *__restrict__ flag) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    bool reset = (*flag != 0);   // a rebuild happened at the previous check
    double d0 = 0.0, d1 = 0.0, d2 = 0.0;
    if (p < np) {
        d0 = drostep[3 * p];
        d1 = drostep[3 * p + 1];
        d2 = drostep[3 * p + 2];
    }
    mg_chk_accum(p, np, d0, d1, d2, reset, drosum, r2out, blkmax);
}

// Pass 2 per block: the largest value that was not a new running maximum,
// given the maximum of all earlier blocks.  The last block to finish
// combines the blocks (threadfence + counter) and sets the rebuild flag and,
// inside a captured step, the graph condition that runs the rebuild.
__global__ void __launch_bounds__(kChkThreads) k_chk_second(const double *__restrict__ r2in,
                                                            const double *__restrict__ blkmax,
                                                            double *__restrict__ blk2, int np, int nblk,
                                                            double drnlist, int *__restrict__ flag,
                                                            int *__restrict__ counter, int use_cond,
                                                            cudaGraphConditionalHandle cond) {
    __shared__ long long wmax[32], red[32];
    __shared__ long long pb;
    __shared__ bool last;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (w == 0) {   // maximum over all earlier blocks, one warp
        long long m = 0;
        for (int b = lane; b < (int)blockIdx.x; b += 32) m = chk_max(m, __double_as_longlong(blkmax[b]));
        for (int o = 16; o > 0; o >>= 1) m = chk_max(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) pb = m;
    }
    long long r2 = (p < np) ? __double_as_longlong(r2in[p]) : 0;
    // inclusive prefix max within the warp
    long long v = r2;
    for (int o = 1; o < 32; o <<= 1) {
        long long y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v = chk_max(v, y);
    }
    if (lane == 31) wmax[w] = v;
    __syncthreads();
    if (w == 0) {
        int nw = blockDim.x >> 5;
        long long x = (lane < nw) ? wmax[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x = chk_max(x, y);
        }
        if (lane < nw) wmax[lane] = x;
    }
    __syncthreads();
    long long excl = __shfl_up_sync(0xffffffffu, v, 1);
    if (lane == 0) excl = 0;
    if (w > 0) excl = chk_max(excl, wmax[w - 1]);
    long long prev = chk_max(pb, excl);   // running maximum before this particle
    long long cand = (p < np && !(r2 > prev)) ? r2 : 0;
    for (int o = 16; o > 0; o >>= 1) cand = chk_max(cand, __shfl_xor_sync(0xffffffffu, cand, o));
    if (lane == 0) red[w] = cand;
    __syncthreads();
    if (threadIdx.x == 0) {
        int nw = blockDim.x >> 5;
        long long x = 0;
        for (int k = 0; k < nw; ++k) x = chk_max(x, red[k]);
        blk2[blockIdx.x] = __longlong_as_double(x);
        __threadfence();
        last = (atomicAdd(counter, 1) == nblk - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x >= 32) return;
    __threadfence();
    long long m1 = 0, m2 = 0;
    for (int b = lane; b < nblk; b += 32) {
        m1 = chk_max(m1, __double_as_longlong(((volatile const double *)blkmax)[b]));
        m2 = chk_max(m2, __double_as_longlong(((volatile const double *)blk2)[b]));
    }
    for (int o = 16; o > 0; o >>= 1) {
        m1 = chk_max(m1, __shfl_xor_sync(0xffffffffu, m1, o));
        m2 = chk_max(m2, __shfl_xor_sync(0xffffffffu, m2, o));
    }
    if (lane == 0) {
        int f = (sqrt(__longlong_as_double(m1)) + sqrt(__longlong_as_double(m2)) > drnlist) ? 1 : 0;
        flag[0] = f;
        flag[2] += f;   // list builds (the rebuild follows this check)
        *counter = 0;
        if (use_cond) cudaGraphSetConditional(cond, (unsigned)f);
    }
}

__global__ void k_set_int(int *p, int v) { *p = v; }

// ---- MC cell list: the reference's doubly linked lists on the device -------
__global__ void k_mc_cells_set(const double *__restrict__ ro, int np, double3 half, double3 csi,
                               int3 nc, int *__restrict__ iphead, int *__restrict__ npart,
                               int *__restrict__ ipnext, int *__restrict__ ipprev,
                               int *__restrict__ cellof, int *__restrict__ err) {
    // SetCellList: add ip = 1..np in order (head insertion); one thread keeps
    // the reference's list order
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int p = 0; p < np; ++p) {
        int ix = (int)floor(__dmul_rn(__dadd_rn(ro[3 * p + 0], half.x), csi.x));
        int iy = (int)floor(__dmul_rn(__dadd_rn(ro[3 * p + 1], half.y), csi.y));
        int iz = (int)floor(__dmul_rn(__dadd_rn(ro[3 * p + 2], half.z), csi.z));
        if (ix < 0 || ix >= nc.x || iy < 0 || iy >= nc.y || iz < 0 || iz >= nc.z) {
            mg_dev_error(err, MG_ERR_CELL, p + 1, 0, 0);
            return;
        }
        int c = ix + iy * nc.x + iz * nc.x * nc.y;
        int ip = p + 1;
        npart[c] += 1;
        int jp = iphead[c];
        iphead[c] = ip;
        if (jp != 0) {
            ipprev[jp - 1] = ip;
            ipnext[ip - 1] = jp;
        } else {
            ipnext[ip - 1] = 0;
        }
        ipprev[ip - 1] = 0;
        cellof[p] = c;
    }
}

// UpdateCellIp (celllist.F90:366-382) for one particle (1-based ip)
__global__ void k_mc_cells_update(const double *__restrict__ ro, int ip, double3 half, double3 csi,
                                  int3 nc, int *__restrict__ iphead, int *__restrict__ npart,
                                  int *__restrict__ ipnext, int *__restrict__ ipprev,
                                  int *__restrict__ cellof, int *__restrict__ err) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int p = ip - 1;
    int ix = (int)floor(__dmul_rn(__dadd_rn(ro[3 * p + 0], half.x), csi.x));
    int iy = (int)floor(__dmul_rn(__dadd_rn(ro[3 * p + 1], half.y), csi.y));
    int iz = (int)floor(__dmul_rn(__dadd_rn(ro[3 * p + 2], half.z), csi.z));
    if (ix < 0 || ix >= nc.x || iy < 0 || iy >= nc.y || iz < 0 || iz >= nc.z) {
        mg_dev_error(err, MG_ERR_CELL, ip, 0, 0);
        return;
    }
    int cnew = ix + iy * nc.x + iz * nc.x * nc.y, cold = cellof[p];
    if (cnew == cold) return;
    // RmIpFromCell
    npart[cold] -= 1;
    int nextp = ipnext[p], prevp = ipprev[p];
    if (nextp == 0) {
        if (iphead[cold] == ip) iphead[cold] = 0;
        else ipnext[prevp - 1] = 0;
    } else {
        if (iphead[cold] == ip) {
            iphead[cold] = nextp;
            ipprev[nextp - 1] = 0;
        } else {
            ipprev[nextp - 1] = prevp;
            ipnext[prevp - 1] = nextp;
        }
    }
    ipprev[p] = 0;
    ipnext[p] = 0;
    // AddIpToCell
    npart[cnew] += 1;
    int jp = iphead[cnew];
    iphead[cnew] = ip;
    if (jp != 0) {
        ipprev[jp - 1] = ip;
        ipnext[p] = jp;
    } else {
        ipnext[p] = 0;
    }
    ipprev[p] = 0;
    cellof[p] = cnew;
}

StencilArgs make_stencil(const mg_handle *h) {
    StencilArgs sa;
    sa.nc = make_int3(h->ncell[0], h->ncell[1], h->ncell[2]);
    for (int m = 0; m < 3; ++m) {
        // a collapsed dimension (one cell) has only the cell itself;
        // otherwise there are >= 3 cells and -1, 0, +1 are distinct
        sa.lo[m] = (h->ncell[m] >= 3) ? -1 : 0;
        sa.hi[m] = (h->ncell[m] >= 3) ? 1 : 0;
    }
    return sa;
}

// The FP32 filter's band around the cutoff.  With |x| <= L/2 + rcell, the
// FP32 copy of a coordinate is off by at most ulp(L)/2, the difference and the
// periodic shift round once each, so a component is off by at most
// e = 2 ulp(Lmax) (ulp(v) = v 2^-23); r^2 <= rs2cut + band then is off by at
// most about 6 e sqrt(rs2cut) plus its own rounding, 4 ulp(rs2cut).  The band
// takes ten times that and 1e-4 rs2cut more.  (Where |dx| is near L/2 the
// FP32 and FP64 forms may shift differently, but the two shifted values have
// the same magnitude, so r^2 does not jump.)
VlistBand make_band(const mg_handle *h) {
    VlistBand b;
    double lmax = 0;
    for (int m = 0; m < 3; ++m) {
        b.half[m] = (float)h->boxlen2[m];
        b.len[m] = (float)h->boxlen[m];
        lmax = fmax(lmax, h->boxlen[m]);
    }
    double ulp = ldexp(1.0, -23);
    double e = 2.0 * (lmax + h->rcut + h->drnlist) * ulp;
    double band = 10.0 * (6.0 * e * sqrt(h->rs2cut) + 4.0 * h->rs2cut * ulp) + 1e-4 * h->rs2cut;
    b.lo = (float)(h->rs2cut - band);
    b.hi = (float)(h->rs2cut + band);
    return b;
}

mg_box make_box(const mg_handle *h) {
    mg_box b;
    for (int m = 0; m < 3; ++m) {
        b.len[m] = h->boxlen[m];
        b.half[m] = h->boxlen2[m];
        b.inv[m] = h->boxleni[m];
    }
    return b;
}

}  // namespace

void mg_scan_exclusive(mg_handle *h, const int *in, int *out, int n, const int *gate) {
    int ntile = (n + kScanTile - 1) / kScanTile;
    k_scan_tiles<<<ntile, kScanThreads, 0, h->st>>>(in, out, n, h->d_scan_tiles, gate);
    k_scan_fix<<<ntile, kScanThreads, 0, h->st>>>(out, n, h->d_scan_tiles, ntile, gate);
    h->launches += 2;
}

// InitCellList(rcut + drnlist) (celllist.F90:76-152): grid and stencil range
int mg_lists_init(mg_handle *h) {
    double rcell = h->rcut + h->drnlist;
    if (!(rcell > 0)) return mg_fail(h, MG_ERR_ARG, "rcut + drnlist must be > 0");
    double ircell = 1.0 / rcell;
    for (int m = 0; m < 3; ++m) {
        int n = (int)floor(h->boxlen[m] * ircell);
        if (n < 1) n = 1;
        h->ncell[m] = n;
        h->cellSize[m] = h->boxlen[m] / n;
        h->cellSizei[m] = 1.0 / h->cellSize[m];
    }
    for (int m = 0; m < 3; ++m) {
        int dir = (int)ceil(h->rcut * h->cellSizei[m]);
        if (2 * dir + 1 > h->ncell[m]) {
            h->ncell[m] = 1;
            h->cellSize[m] = h->boxlen[m];
            h->cellSizei[m] = h->boxleni[m];
        }
    }
    h->ncelltot = h->ncell[0] * h->ncell[1] * h->ncell[2];
    int np = h->np;
    if (h->maxnb <= 0) {
        // automatic capacity: twice the expected number within rcut+drnlist,
        // at least 64, at most np-1 (the reference's own maxnneigh is >= np-1)
        double dens = np / h->vol;
        double expect = 4.0 / 3.0 * 3.141592653589793 * rcell * rcell * rcell * dens;
        int cap = (int)(2.0 * expect + 64);
        if (cap > np - 1) cap = np - 1;
        if (cap < 1) cap = 1;
        h->maxnb = cap;
    }
    size_t nc = (size_t)h->ncelltot;
    MG_CUDA(h, cudaMalloc(&h->d_cellof, sizeof(int) * np));
    MG_CUDA(h, cudaMalloc(&h->d_cellcount, sizeof(int) * nc));
    MG_CUDA(h, cudaMalloc(&h->d_cellfill, sizeof(int) * nc));
    MG_CUDA(h, cudaMalloc(&h->d_cellstart, sizeof(int) * (nc + 1)));
    MG_CUDA(h, cudaMalloc(&h->d_perm, sizeof(int) * np));
    MG_CUDA(h, cudaMalloc(&h->d_slot, sizeof(int) * np));
    MG_CUDA(h, cudaMalloc(&h->d_nnb, sizeof(int) * np));
    MG_CUDA(h, cudaMalloc(&h->d_nbr, sizeof(int) * (size_t)h->maxnb * np));
    MG_CUDA(h, cudaMalloc(&h->d_pos_s, sizeof(double4) * np));
    MG_CUDA(h, cudaMalloc(&h->d_ro_slot, sizeof(double4) * np));
    MG_CUDA(h, cudaMalloc(&h->d_ro_slot_f, sizeof(float4) * np));
    MG_CUDA(h, cudaMalloc(&h->d_scan_tiles, sizeof(int) * ((nc + kScanTile - 1) / kScanTile)));
    h->nblk_chk = (np + kChkThreads - 1) / kChkThreads;
    MG_CUDA(h, cudaMalloc(&h->d_drostep, sizeof(double) * 3 * np));
    MG_CUDA(h, cudaMalloc(&h->d_drosum, sizeof(double) * 3 * np));
    MG_CUDA(h, cudaMalloc(&h->d_blkmax, sizeof(double) * (2 * h->nblk_chk + np)));
    MG_CUDA(h, cudaMalloc(&h->d_rebuild, sizeof(int) * 3));
    MG_CUDA(h, cudaMemsetAsync(h->d_drosum, 0, sizeof(double) * 3 * np, h->st));
    MG_CUDA(h, cudaMemsetAsync(h->d_drostep, 0, sizeof(double) * 3 * np, h->st));
    MG_CUDA(h, cudaMemsetAsync(h->d_rebuild, 0, sizeof(int) * 3, h->st));
    if (h->mode == MG_MC && h->txintlist == MG_CELLLIST) {
        MG_CUDA(h, cudaMalloc(&h->d_iphead, sizeof(int) * nc));
        MG_CUDA(h, cudaMalloc(&h->d_npart, sizeof(int) * nc));
        MG_CUDA(h, cudaMalloc(&h->d_ipnext, sizeof(int) * np));
        MG_CUDA(h, cudaMalloc(&h->d_ipprev, sizeof(int) * np));
    }
    return MG_OK;
}

// Cell sort + Verlet list.  With `conditional`, every kernel first reads the
// device rebuild flag and returns when it is 0 (graph-friendly rebuild).
int mg_lists_build(mg_handle *h, bool conditional) {
    int np = h->np;
    const int *gate = conditional ? h->d_rebuild : nullptr;
    double3 half = make_double3(h->boxlen2[0], h->boxlen2[1], h->boxlen2[2]);
    double3 csi = make_double3(h->cellSizei[0], h->cellSizei[1], h->cellSizei[2]);
    int3 nc = make_int3(h->ncell[0], h->ncell[1], h->ncell[2]);
    int tb = 256, gb = (np + tb - 1) / tb;
    MG_CUDA(h, cudaMemsetAsync(h->d_cellcount, 0, sizeof(int) * h->ncelltot, h->st));
    MG_CUDA(h, cudaMemsetAsync(h->d_cellfill, 0, sizeof(int) * h->ncelltot, h->st));
    k_cell_assign<<<gb, tb, 0, h->st>>>(h->d_ro, np, half, csi, nc, h->d_cellof, h->d_cellcount,
                                        h->d_err, gate);
    mg_scan_exclusive(h, h->d_cellcount, h->d_cellstart, h->ncelltot, gate);
    k_cell_scatter<<<gb, tb, 0, h->st>>>(h->d_cellof, np, h->d_cellstart, h->d_cellfill, h->d_perm,
                                         gate);
    k_cell_sort<<<(h->ncelltot + tb - 1) / tb, tb, 0, h->st>>>(h->ncelltot, h->d_cellstart,
                                                               h->d_perm, gate);
    k_slot_of<<<gb, tb, 0, h->st>>>(h->d_perm, h->d_ro, h->d_cellof, np, h->d_slot, h->d_ro_slot,
                                    h->d_ro_slot_f, gate);
    k_vlist<<<(np + 127) / 128, 128, 0, h->st>>>(h->d_ro_slot, h->d_ro_slot_f, h->d_cellstart, np,
                                                 make_stencil(h), make_box(h), make_band(h), h->rs2cut,
                                                 h->maxnb, h->d_nnb, h->d_nbr, h->d_perm, h->d_err, gate);
    h->launches += 5;
    MG_CUDA(h, cudaGetLastError());
    h->list_valid = true;
    return MG_OK;
}

// the list-build count of VListAver (nlist.F90:953-986): 1 after the
// initial build, then one more per rebuild (counted by k_chk_second)
int mg_lists_reset_calls(mg_handle *h) {
    k_set_int<<<1, 1, 0, h->st>>>(h->d_rebuild + 2, 1);
    h->launches++;
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

// NList(iSimulationStep): accumulate drostep (already on the device in
// d_drostep) and set the rebuild flag; the caller then runs a conditional build.
mg_chk_args mg_lists_chk_args(mg_handle *h) {
    mg_chk_args c;
    c.drosum = h->d_drosum;
    c.r2out = h->d_blkmax + 2 * h->nblk_chk;
    c.blkmax = h->d_blkmax;
    c.flag = h->d_rebuild;
    return c;
}

// accum_done: the move kernel of this step ran the first pass (blocks of
// kChkThreads particles)
int mg_lists_check(mg_handle *h, bool accum_done) {
    int np = h->np, nb = h->nblk_chk;
    double *r2 = h->d_blkmax + 2 * nb;
    if (!accum_done) {
        k_chk_accum<<<nb, kChkThreads, 0, h->st>>>(h->d_drostep, h->d_drosum, r2, h->d_blkmax, np,
                                                   h->d_rebuild);
        h->launches++;
    }
    k_chk_second<<<nb, kChkThreads, 0, h->st>>>(r2, h->d_blkmax, h->d_blkmax + nb, np, nb, h->drnlist,
                                         h->d_rebuild, h->d_rebuild + 1, h->use_cond ? 1 : 0,
                                         h->cond);
    h->launches += 1;
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

int mg_mc_cells_set(mg_handle *h) {
    double3 half = make_double3(h->boxlen2[0], h->boxlen2[1], h->boxlen2[2]);
    double3 csi = make_double3(h->cellSizei[0], h->cellSizei[1], h->cellSizei[2]);
    int3 nc = make_int3(h->ncell[0], h->ncell[1], h->ncell[2]);
    MG_CUDA(h, cudaMemsetAsync(h->d_iphead, 0, sizeof(int) * h->ncelltot, h->st));
    MG_CUDA(h, cudaMemsetAsync(h->d_npart, 0, sizeof(int) * h->ncelltot, h->st));
    MG_CUDA(h, cudaMemsetAsync(h->d_ipnext, 0, sizeof(int) * h->np, h->st));
    MG_CUDA(h, cudaMemsetAsync(h->d_ipprev, 0, sizeof(int) * h->np, h->st));
    k_mc_cells_set<<<1, 32, 0, h->st>>>(h->d_ro, h->np, half, csi, nc, h->d_iphead, h->d_npart,
                                        h->d_ipnext, h->d_ipprev, h->d_cellof, h->d_err);
    h->launches++;
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

int mg_mc_cells_update(mg_handle *h, int ip) {
    double3 half = make_double3(h->boxlen2[0], h->boxlen2[1], h->boxlen2[2]);
    double3 csi = make_double3(h->cellSizei[0], h->cellSizei[1], h->cellSizei[2]);
    int3 nc = make_int3(h->ncell[0], h->ncell[1], h->ncell[2]);
    k_mc_cells_update<<<1, 32, 0, h->st>>>(h->d_ro, ip, half, csi, nc, h->d_iphead, h->d_npart,
                                           h->d_ipnext, h->d_ipprev, h->d_cellof, h->d_err);
    h->launches++;
    MG_CUDA(h, cudaGetLastError());
    return MG_OK;
}

// Export the Verlet list in the reference layout (1-based, column-major
// jpnlist(maxnneigh, np)).  MD/BD: SetVListMD's ownership rule (pair (i<j)
// listed under i when i+j is odd, under j when even, 1-based); MC: full list.
// Neighbours are listed in increasing particle order, as the reference's jp
// loops produce them.
int mg_lists_export(mg_handle *h, int32_t *nneighpn, int32_t *jpnlist, int32_t maxnneigh) {
    if (!h->list_valid) return mg_fail(h, MG_ERR_STATE, "no Verlet list has been built");
    MG_TRY(mg_check_device_error(h));
    int np = h->np;
    std::vector<int> nnb(np), perm(np), nbr((size_t)h->maxnb * np);
    MG_CUDA(h, cudaMemcpy(nnb.data(), h->d_nnb, sizeof(int) * np, cudaMemcpyDeviceToHost));
    MG_CUDA(h, cudaMemcpy(perm.data(), h->d_perm, sizeof(int) * np, cudaMemcpyDeviceToHost));
    MG_CUDA(h, cudaMemcpy(nbr.data(), h->d_nbr, sizeof(int) * nbr.size(), cudaMemcpyDeviceToHost));
    std::vector<std::vector<int>> out(np);
    for (int i = 0; i < np; ++i) {
        int ip = perm[i] + 1;
        for (int k = 0; k < nnb[i]; ++k) {
            int jp = perm[nbr[(size_t)k * np + i]] + 1;
            bool keep;
            if (h->mode == MG_MC) keep = true;
            else {
                int odd = (ip + jp) % 2;
                keep = (ip < jp) ? (odd != 0) : (odd == 0);
            }
            if (keep) out[ip - 1].push_back(jp);
        }
    }
    for (int p = 0; p < np; ++p) {
        std::vector<int> &v = out[p];
        std::sort(v.begin(), v.end());
        nneighpn[p] = (int32_t)v.size();
        if ((int)v.size() > maxnneigh)
            return mg_fail(h, MG_ERR_NEIGH_OVERFLOW, "particle %d has %d neighbours > %d", p + 1,
                           (int)v.size(), maxnneigh);
        for (size_t k = 0; k < v.size(); ++k) jpnlist[(size_t)p * maxnneigh + k] = v[k];
    }
    return MG_OK;
}

int mg_cells_export(mg_handle *h, int32_t *ncell, int32_t *cellip) {
    if (!h->list_valid && !h->d_iphead) return mg_fail(h, MG_ERR_STATE, "no cell list");
    MG_TRY(mg_check_device_error(h));
    for (int m = 0; m < 3; ++m) ncell[m] = h->ncell[m];
    MG_CUDA(h, cudaMemcpy(cellip, h->d_cellof, sizeof(int) * h->np, cudaMemcpyDeviceToHost));
    return MG_OK;
}
