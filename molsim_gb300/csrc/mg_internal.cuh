// mg_internal.cuh — internal declarations of the GB300 hot-path library.
//
// Device data layout (one handle = one system on one GPU):
//   ro        double[3*np]   positions, reference layout ro(3,np)
//   perm      int[np]        cell-sorted slot -> particle (0-based)
//   pos_s     double4[np]    (x,y,z,charge) in slot order, refreshed per call
//   nbr       int[maxnb*np]  Verlet list in slot space, column-major
//                            (neighbour k of slot i at nbr[k*np+i])
//   force     double[3*np]   FP64 accumulator (plain form), reference layout
//   ffx       long long[3*np] 64-bit fixed-point accumulator (mixed form)
//   mesh      SPME real mesh Q[z][y][x] and half spectrum F[z][y][kx]
//   part      double[]       per-block partial sums, reduced in fixed order
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/molsim_gb300.h"

#define MG_MAX_ORDER 12
#define MG_MAX_NPTPT 10
#define MG_FX_SCALE 4294967296.0          // 2^32: fixed-point force / mesh scale
#define MG_FX_INV (1.0 / 4294967296.0)

struct mg_phase {
    std::string name;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    double total_ms = 0;
    long count = 0;
    bool pending = false;
};

// host buffers that a step reads and writes directly (pinned, mapped into
// the device address space): positions in and out, forces out
struct mg_hostio {
    double *ro;      // 3 np: read before the move, written after it
    double *forceo;  // 3 np: written at the end of the step
    double *stage;   // the energies (nu values) and then the device error word
    const double *uout;
    const int *err;
    int nu;
};

struct mg_handle {
    int dev = 0;
    cudaStream_t st = nullptr;
    // SPME: the short-range forces (prepare, pair, bonds) run on st2 beside
    // the mesh path on st, into their own accumulator (d_ffx2 in the mixed
    // form, d_force2 in the FP64 form)
    cudaStream_t st2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev_sr = nullptr, ev_rec = nullptr;   // short-range forces done; reciprocal partials done
    bool par_final = false;         // the gather writes forceo (forked, no surface term)
    long long *d_ffx2 = nullptr;
    double *d_force2 = nullptr;
    bool par_forces = false;        // set while a forked UTotal queues its mesh path
    // a device step asks UTotal to queue the list check's second pass on st2
    // (it needs only the move's displacements); chk_queued reports that it did
    bool chk_side = false, chk_queued = false;
    std::string err;

    // ---- parameters ---------------------------------------------------
    int np = 0, npt = 0, nptpt = 0, form = 0, mode = 0, txintlist = 0;
    int ewald = 0, ncut = 0, ncut2 = 0, order = 0, nmesh = 0, lsurf = 0, nbond = 0;
    int maxnb = 0;
    double boxlen[3], boxlen2[3], boxleni[3], TwoPiBoxi[3], vol = 0;
    double rcut = 0, rcut2 = 0, drnlist = 0, rs2cut = 0, ualpha = 0, EpsiFourPi = 0;
    double force_fac = 0, u_self = 0;
    std::vector<int> h_type;          // 0-based particle types
    std::vector<int> h_pairidx;       // [npt*npt] 1-based pair index
    std::vector<double> h_az;

    // ---- device: system ------------------------------------------------
    double *d_ro = nullptr, *d_az = nullptr;
    int *d_type = nullptr, *d_pairidx = nullptr;
    double *d_ubuf = nullptr, *d_r2umin = nullptr, *d_r2atat = nullptr;
    float *d_ubuf_f = nullptr;
    int *d_tab_start = nullptr, *d_tab_n = nullptr;   // per pair: first record (0-based double offset / 12), count
    int nbuf = 0;
    // pair kernel tables: interval lower ends, coefficients, direct-index bins
    int nrec = 0, nbins = 0, pair_tab_smem = 0, pair_warp = 0, pair_team = 1;
    size_t pair_smem = 0;
    double *d_zlow = nullptr, *d_coef = nullptr, *d_bin_z0 = nullptr, *d_bin_inv = nullptr;
    float *d_coef_f = nullptr;
    unsigned short *d_bin_kstart = nullptr;
    float *d_f32_tabs = nullptr;     // mixed: zlow, r2umin, r2atat, bin z0, bin inverse width
    float4 *d_pos_f = nullptr;       // mixed: cell-relative FP32 positions in slot order
    int *d_cell_s = nullptr;         // mixed: packed cell coordinates in slot order

    // ---- cells and Verlet list -----------------------------------------
    int ncell[3] = {1, 1, 1}, ncelltot = 1;
    double cellSize[3], cellSizei[3];
    int *d_cellof = nullptr, *d_cellcount = nullptr, *d_cellstart = nullptr, *d_cellfill = nullptr;
    int *d_perm = nullptr, *d_slot = nullptr;
    int *d_nnb = nullptr, *d_nbr = nullptr;
    double4 *d_pos_s = nullptr;
    double4 *d_ro_slot = nullptr;   // list build: positions in slot order, cell index in .w
    float4 *d_ro_slot_f = nullptr;  // list build: their FP32 copies (the distance filter)
    int *d_scan_tiles = nullptr;    // list build: per-tile totals of the cell-count scan
    bool list_valid = false;
    bool list_stale = false;        // MC + cell list: particles moved since the last build
    // MC cell list (doubly linked lists, reference layout; 1-based, 0 = none)
    int *d_iphead = nullptr, *d_npart = nullptr, *d_ipnext = nullptr, *d_ipprev = nullptr;
    int *d_neighcells = nullptr, nneighcell_max = 0;   // [ncelltot * 27]
    int *d_nneighcell = nullptr;

    // ---- forces and reductions ----------------------------------------
    double *d_force = nullptr, *d_forceo = nullptr;
    long long *d_ffx = nullptr;
    double *d_part = nullptr;      // partial sums
    int part_pair = 0, part_rec = 0, part_bond = 0, part_surf = 0;   // offsets
    int nblk_pair = 0, nblk_rec = 0, nblk_bond = 0, nblk_surf = 0;
    int part_red = 0;                   // energy reduction: its scratch rows in d_part
    double *d_uout = nullptr;      // [nptpt+1] u_twob, then u_tot,u_rec,u_bond,virial, then surf sums (3)
    int *d_err = nullptr;          // [4] code, info1, info2, info3
    double *h_pinned = nullptr;    // pinned staging for outputs
    double *h_stage = nullptr;     // pinned: the energies of a fetch, then the device error word
    size_t h_pinned_bytes = 0;

    // ---- bonds -----------------------------------------------------------
    int *d_bond_ij = nullptr, *d_bond_p = nullptr;   // [2*nbond] (0-based), [nbond]
    double *d_bond_k = nullptr, *d_bond_eq = nullptr;
    int *d_bond_off = nullptr, *d_bond_list = nullptr;  // CSR per particle: entries b*2 + (0 first, 1 second)
    // angles jm-ip-jp (UAngle): 0-based triples, parameters, and a CSR per
    // particle of entries a*4 + role (0 jm, 1 ip, 2 jp)
    int nangle = 0;
    int *d_angle_ijk = nullptr, *d_angle_p = nullptr, *d_angle_off = nullptr, *d_angle_list = nullptr;
    double *d_angle_k = nullptr, *d_angle_eq = nullptr;
    // chain table for MC trial moves (DUBond/DUAngle), 5 ints per particle:
    // lower and upper neighbour (1-based, 0 none; bond b joins lower bond_ip
    // and upper bond_jp), the bond to each (-1 none), the angle with the
    // particle as vertex (-1 none); chain_angles: some angle has k != 0
    int *d_chain = nullptr;
    int chain_angles = 0;

    // ---- standard Ewald ----------------------------------------------------
    int nkvec = 0;
    int4 *d_kvec = nullptr;         // (nx, ny, nz, -)
    double *d_kfac = nullptr;
    double2 *d_eik = nullptr;       // [3][ncut+1][np]
    double2 *d_S = nullptr;         // [nkvec][4]
    double2 *d_Stm = nullptr;

    // ---- SPME ------------------------------------------------------------
    int nh = 0;                     // nmesh/2 + 1
    double dkdr[3];
    void *d_Q = nullptr;            // real mesh (double or float)
    void *d_F = nullptr;            // half spectrum (double2 or float2)
    unsigned long long *d_Qfx = nullptr;  // spread mesh in 64-bit fixed point (cleared by the FFT x pass)
    double *d_mf = nullptr, *d_ew = nullptr, *d_vw = nullptr;   // octant tables [nh^3]
    float *d_mf_f = nullptr, *d_ew_f = nullptr, *d_vw_f = nullptr;
    void *d_tw = nullptr;           // twiddles exp(-2 pi i m/n), m < n
    int fft_tx = 0, fft_tiles = 0;
    int fft_plane = 0, fft_warps = 0;   // mixed form, 32 <= nmesh <= 128: three plane/slab passes
    int gen_mesh = 0;                   // nmesh 2^a 3^b 5^c, not a power of two: generic spread and gather
    // mixed form with plane passes, MD/BD: the spread runs inside the forward
    // plane pass (particles sorted by the z plane of their stamp corner), so
    // the charge mesh never leaves shared memory
    int plane_fused = 0;
    float *d_spl_plane = nullptr;   // fused spread: the spread records in plane order
    // dipole electrostatics (mg_dipole_ewald): dip, pot, est, efg, virial terms
    double *d_dip_scr = nullptr;
    size_t dip_scr_n = 0;
    double az_absmax = 0.0;          // max |q| of the particles
    double spl_mmax = 1.0;           // largest cardinal B-spline value at the SPME order
    int brick = 0, nbrick_edge = 0, nbricks = 0;
    size_t spread_smem = 0, gather_smem = 0;
    int fx_shift = 30, fx_shift64 = 48;
    int spread_wpb = 4;             // spread: bricks (warps) per block
    int spread_wpb_lane = 4;        // the same for the lane-per-particle spread
    size_t spread_smem_lane = 0;
    int spread_chunk = 256;         // particles staged per pass of the spread              // mixed spread: weights scaled by 2^fx_shift into int32
    int *d_brick_count = nullptr, *d_brick_perm = nullptr, *d_brick_rank = nullptr, *d_brick_of = nullptr;
    int *d_brick_start = nullptr;
    int *d_brick_istart = nullptr, *d_item_brick = nullptr;   // spread work items per brick
    int spread_m = 32, max_items = 0;
    void *d_tiles = nullptr;        // per-brick spread tiles (mesh type)
    void *d_spl_w = nullptr;   // per particle: B-spline values x, y, z, derivatives x, y, z (padded to 4)
    double *d_Qref = nullptr;       // MC: charge mesh of the accepted state (FP64)
    double *d_phi = nullptr;        // MC: potential mesh of the accepted state
    double *d_gker = nullptr;       // MC: real-space kernel g (nmesh^3)
    double urecold = 0;

    // ---- gradients (grad.cu) ----------------------------------------------
    double *d_grad = nullptr;       // site potentials, pair parameters, partial sums
    size_t grad_cap = 0;

    // ---- MC trial ------------------------------------------------------------
    void *mc = nullptr;             // trial buffers (mc.cu)
    int nptm = 0;
    int *d_ipnptm = nullptr;
    double *d_rotm = nullptr, *d_du = nullptr;
    std::vector<int> h_ipnptm;
    std::vector<double> h_rotm;
    bool trial_ok = false;
    bool have_rec = false;
    double h_du_tot = 0, h_du_rec = 0;

    // ---- list check ---------------------------------------------------------
    double *d_drostep = nullptr, *d_drosum = nullptr, *d_blkmax = nullptr;
    // [3]: current flag, the list check's block counter, number of list
    // builds since mg_nlist_set (counting that one: VListAver's ncall)
    int *d_rebuild = nullptr;
    int nblk_chk = 0;

    // ---- MD / BD ----------------------------------------------------------------
    double tstep = 0;
    double *d_massip = nullptr, *d_rod = nullptr, *d_rodd = nullptr;
    bool md_ready = false, bd_ready = false, have_force = false;
    // BD deviates: a captured step draws the next step's GauRandom candidates
    // beside its UTotal (they depend only on the generator state after the
    // move); cand_ready: the candidate buffers hold those of the next step
    bool cand_ready = false, cand_side = false, cand_queued = false;
    double *d_fac1 = nullptr, *d_fac2 = nullptr;
    int *d_rng = nullptr;            // [4] iseed, flag, ncand_short, -
    double *d_rng_save = nullptr;    // [1]
    int ncand = 0;
    unsigned *d_cflag = nullptr;     // candidate acceptance scan
    int *d_cidx = nullptr;           // accepted candidate index by rank
    double *d_cval = nullptr;        // [2*ncand] rx, ry per candidate
    int *d_scan_tmp = nullptr;
    int scan_cap = 0;

    // ---- graphs and timing -----------------------------------------------------
    cudaGraphExec_t g_bd = nullptr, g_md = nullptr;
    // mg_bd_step_host with pinned (device-mapped) host buffers: a second BD
    // graph whose move kernel reads and writes the host positions and whose
    // last kernel writes the host forces; the pointers live in d_hostio
    cudaGraphExec_t g_bd_io = nullptr;
    mg_hostio *d_hostio = nullptr;
    mg_hostio hostio_last = {nullptr, nullptr, nullptr, nullptr, nullptr, 0};
    bool hostio = false;            // set while the host-I/O graph is captured
    // while a step is captured, the list check sets a graph condition that
    // runs the (otherwise skipped) rebuild body
    bool use_cond = false;
    cudaGraphConditionalHandle cond = 0;
    int kernels_bd = 0, kernels_md = 0;
    bool timing = false;
    std::vector<mg_phase> phases;
    long launches = 0;
};

// ---- error helpers ----------------------------------------------------------
int mg_fail(mg_handle *h, int code, const char *fmt, ...);
#define MG_CUDA(h, call)                                                                   \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return mg_fail((h), MG_ERR_CUDA, "%s failed: %s (%s:%d)", #call,              \
                           cudaGetErrorString(e_), __FILE__, __LINE__);                    \
    } while (0)
// x mod n in [0, n) for any int x: a mask when n is a power of two
// (mn = n - 1), the remainder otherwise (mn < 0: meshes 2^a 3^b 5^c)
__host__ __device__ __forceinline__ int mg_mesh_mask(int n) { return (n & (n - 1)) == 0 ? n - 1 : -1; }
__host__ __device__ __forceinline__ int mg_wrapm(int x, int n, int mn) {
    if (mn >= 0) return x & mn;
    int r = x % n;
    return r < 0 ? r + n : r;
}

#define MG_TRY(x)                  \
    do {                           \
        int s_ = (x);              \
        if (s_ != MG_OK) return s_; \
    } while (0)

// device error word: first error wins
__device__ __forceinline__ void mg_dev_error(int *err, int code, int a, int b, int c) {
    if (atomicCAS(err, 0, code) == 0) {
        err[1] = a;
        err[2] = b;
        err[3] = c;
    }
}

// ---- exact FP64 helpers (no FMA contraction where the result decides a
//      branch: list membership, table interval, cell index) -------------------
__device__ __forceinline__ double mg_r2_exact(double dx, double dy, double dz) {
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}
// Programmatic dependent launch.  A kernel launched by mg_launch_pdl may
// start while the kernel before it in the stream drains (its blocks take the
// places that the finished blocks of the predecessor free); it waits for the
// completion and memory of its predecessor (griddepcontrol.wait) before it
// reads anything.  Launched without the attribute, the wait is a no-op.
__device__ __forceinline__ void mg_pdl_begin() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t mg_launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                 Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

// First pass of the NList(iSimulationStep) rebuild rule (nlist.F90:598-621)
// for particle p of a block of kChkThreads threads: drosum += d (drosum
// restarts after a rebuild), r2 = |drosum|^2 into r2out[p], the block's
// largest r2 into blkmax[blockIdx.x].  r2 >= 0, and non-negative doubles
// order as their 64-bit patterns, so the maximum runs on integers.  Every
// thread of the block calls it (it holds a barrier).
constexpr int kChkThreads = 256;
// cell-count scan: tiles of kScanTile cells, a block of kScanThreads per tile
constexpr int kScanThreads = 512;
constexpr int kScanTile = 4096;
// as mg_chk_accum, with the particle's previous drosum already loaded into
// s (not read on a reset), so that a move kernel can issue that load with
// its other loads
__device__ __forceinline__ void mg_chk_accum_from(int p, int np, double d0, double d1, double d2, bool reset,
                                                  const double *s, double *__restrict__ drosum,
                                                  double *__restrict__ r2out, double *__restrict__ blkmax) {
    __shared__ long long chk_red[kChkThreads / 32];
    double r2 = 0.0;
    if (p < np) {
        double s0, s1, s2;
        if (reset) {
            s0 = 0.0 + d0;
            s1 = 0.0 + d1;
            s2 = 0.0 + d2;
        } else {
            s0 = __dadd_rn(s[0], d0);
            s1 = __dadd_rn(s[1], d1);
            s2 = __dadd_rn(s[2], d2);
        }
        drosum[3 * p] = s0;
        drosum[3 * p + 1] = s1;
        drosum[3 * p + 2] = s2;
        r2 = __dadd_rn(__dadd_rn(__dmul_rn(s0, s0), __dmul_rn(s1, s1)), __dmul_rn(s2, s2));
        r2out[p] = r2;
    }
    long long m = __double_as_longlong(r2);
    for (int o = 16; o > 0; o >>= 1) {
        long long y = __shfl_xor_sync(0xffffffffu, m, o);
        m = y > m ? y : m;
    }
    if ((threadIdx.x & 31) == 0) chk_red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        long long x = (threadIdx.x < kChkThreads / 32) ? chk_red[threadIdx.x] : 0;
        for (int o = 16; o > 0; o >>= 1) {
            long long y = __shfl_xor_sync(0xffffffffu, x, o);
            x = y > x ? y : x;
        }
        if (threadIdx.x == 0) blkmax[blockIdx.x] = __longlong_as_double(x);
    }
}

__device__ __forceinline__ void mg_chk_accum(int p, int np, double d0, double d1, double d2, bool reset,
                                             double *__restrict__ drosum, double *__restrict__ r2out,
                                             double *__restrict__ blkmax) {
    double s[3] = {0.0, 0.0, 0.0};
    if (p < np && !reset) {
        s[0] = drosum[3 * p];
        s[1] = drosum[3 * p + 1];
        s[2] = drosum[3 * p + 2];
    }
    mg_chk_accum_from(p, np, d0, d1, d2, reset, s, drosum, r2out, blkmax);
}

// the list check's device arrays, for move kernels that run its first pass
struct mg_chk_args {
    double *drosum, *r2out, *blkmax;
    const int *flag;   // nonzero: a rebuild happened at the previous check
};

// PBCr2 (molaux.F90:159-162) for a box: single conditional image shift
__device__ __forceinline__ double mg_pbc1(double d, double half, double len) {
    return (fabs(d) > half) ? __dsub_rn(d, copysign(len, d)) : d;
}

// round(v * 2^32) as a 64-bit integer without the FP64 pipe (the mixed
// form's fixed-point forces): integer part and fraction are converted
// separately, both exactly.  |v| >= 2^31 (only the 1e10 hard-core overlap
// force reaches it) saturates.
__device__ __forceinline__ long long mg_f2fx(float v) {
    v = fminf(fmaxf(v, -2147483648.0f), 2147483520.0f);
    float hi = floorf(v);
    float fr = v - hi;                                    // exact, in [0, 1)
    unsigned lo = __float2uint_rn(fr * 4294967296.0f);   // fr * 2^32 < 2^32, exact scaling
    return ((long long)(int)hi << 32) + (long long)lo;
}

struct mg_box {
    double len[3], half[3], inv[3];
};

// ---- phase timing -------------------------------------------------------------
int mg_phase_begin(mg_handle *h, const char *name);
int mg_phase_end(mg_handle *h, const char *name);
void mg_phase_collect(mg_handle *h);

// ---- module entry points (host side) ----------------------------------------------
int mg_lists_init(mg_handle *h);
int mg_lists_build(mg_handle *h, bool conditional);   // cell sort + Verlet list
int mg_lists_check(mg_handle *h, bool accum_done = false);   // NList(iSimulationStep) rule on device
int mg_integrate_bd_cand(mg_handle *h);              // GauRandom candidates from the current state (h->st)
int mg_integrate_bd_prime(mg_handle *h);             // candidates for a captured step, if not ready
mg_chk_args mg_lists_chk_args(mg_handle *h);          // arrays for a move kernel's first pass
int mg_lists_export(mg_handle *h, int32_t *nneighpn, int32_t *jpnlist, int32_t maxnneigh);
int mg_cells_export(mg_handle *h, int32_t *ncell, int32_t *cellip);
int mg_mc_cells_set(mg_handle *h);
int mg_mc_cells_update(mg_handle *h, int ip);

int mg_forces_init(mg_handle *h, const double *ubuf, const int *start, const int *count);
int mg_utotal_launch(mg_handle *h);                    // queue a full UTotal on the stream
int mg_utotal_fetch(mg_handle *h, double *forceo, double *u_twob, double *uout);

int mg_spme_init(mg_handle *h);
int mg_spme_launch(mg_handle *h);                      // spread, FFT, influence, gather
int mg_ewald_std_init(mg_handle *h);
int mg_ewald_std_launch(mg_handle *h);

double mg_spme_fx_scale(const mg_handle *h);
int mg_spme_potential(mg_handle *h);
int mg_spme_dipole(mg_handle *h, const double *az, const double *dip, double bound, double *pot, double *est,
                   double *efg, double *vir);
int mg_ewald_std_dipole(mg_handle *h, const double *az, const double *dip, double *pot, double *est, double *efg,
                        double *vir);
int mg_force_jvp_rec(mg_handle *h, const double *u, double *jv);
int mg_force_pvjp_rec(mg_handle *h, const double *u, double *dq);
int mg_spme_load_mesh(mg_handle *h, const double *q);
int mg_spme_mesh_to_f64(mg_handle *h, double *out, double mul);
int mg_spme_fft_check(mg_handle *h, const double *q, const double *mult, const double *ew, double *phi,
                      double *esum);
int mg_mc_init(mg_handle *h);
void mg_mc_free(mg_handle *h);
int mg_mc_dutotal(mg_handle *h, int nptm, const int32_t *ipnptm, const double *rotm,
                  double *du_twob, double *du_rec, double *du_tot, int32_t *lhsoverlap);
int mg_mc_accept(mg_handle *h);
int mg_mc_after_utotal(mg_handle *h);
int mg_mc_batch(mg_handle *h, int ntrial, const int32_t *ip, const double *rt, double *du,
                int32_t *ovl);

int mg_integrate_bd_step_launch(mg_handle *h);
int mg_integrate_md_step_launch(mg_handle *h);
int mg_integrate_bd_setup(mg_handle *h, const double *fac1, const double *fac2, int32_t iseed);
int mg_integrate_md_setup(mg_handle *h, double tstep, const double *massip, const double *rod,
                          const double *rodd);

int mg_check_device_error(mg_handle *h);               // sync + read the device error word
int mg_device_error_status(mg_handle *h, const int *e);  // status of an error word already read
int mg_utotal_staged(mg_handle *h, double *u_twob, double *uout);   // energies and status from h_stage (after a sync)
constexpr int kStageDoubles = MG_MAX_NPTPT + 1 + 8 + 2;  // energies (nptpt + 1 + 4) and the error word

// host set-up (host_setup.cu)
int mg_host_table(const mg_pot_params *pp, double *ubuf, int32_t nbuf_cap, int32_t *nbuf_used,
                  int32_t *iubuflow, double *r2umin, int32_t *nugrid);
int mg_host_rcut_to_alpha(double uewaldtol, double rcut, double q2sum, double boxlenshort,
                          double epsi_four_pi, double *ualpha);
void mg_host_spme_tables(int n, int order, const double boxlen[3], const double TwoPiBoxi[3],
                         double vol, double ualpha, std::vector<double> &mf,
                         std::vector<double> &ew, std::vector<double> &vw);
void mg_host_kvectors(int ncut, int ncut2, const double TwoPiBoxi[3], double vol, double ualpha,
                      std::vector<int> &kv, std::vector<double> &kfac);
int mg_host_bspline(int order, double pos, int *kmax, double *values, double *derivs);

// kernels shared between modules
void mg_scan_exclusive(mg_handle *h, const int *in, int *out, int n, const int *gate);
int mg_lists_reset_calls(mg_handle *h);

template <typename T> struct mg_cplx;
template <> struct mg_cplx<double> { typedef double2 type; };
template <> struct mg_cplx<float> { typedef float2 type; };
