// api.cu — the C ABI (include/molsim_gb300.h): handle life cycle, data
// movement, and the reference-shaped entry points UTotal / NList / DUTotal /
// VelVer / BDStep that the Fortran drivers call (md.F90:340, bd.F90:57,
// mc.F90:1714, nlist.F90:124-180).
//
// A handle owns one CUDA stream; every call queues its kernels on it and
// returns after a synchronisation that also reads the device error word.  The
// multi-step MD/BD entry points capture one step as a CUDA graph and replay it.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "mg_internal.cuh"

int mg_fail(mg_handle *h, int code, const char *fmt, ...) {
    if (h) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        h->err = buf;
    }
    return code;
}

int mg_check_device_error(mg_handle *h) {
    MG_CUDA(h, cudaStreamSynchronize(h->st));
    int e[4];
    MG_CUDA(h, cudaMemcpy(e, h->d_err, sizeof(e), cudaMemcpyDeviceToHost));
    return mg_device_error_status(h, e);
}

// the status of a device error word read to the host (and the word cleared)
int mg_device_error_status(mg_handle *h, const int *e) {
    mg_phase_collect(h);
    if (e[0] == 0) return MG_OK;
    int zero[4] = {0, 0, 0, 0};
    MG_CUDA(h, cudaMemcpy(h->d_err, zero, sizeof(zero), cudaMemcpyHostToDevice));
    switch (e[0]) {
    case MG_ERR_TABLE_UNDERRUN:
        return mg_fail(h, e[0], "r2 < r2umin for particles ip=%d jp=%d (pair %d)", e[1], e[2], e[3]);
    case MG_ERR_NEIGH_OVERFLOW:
        return mg_fail(h, e[0], "particle %d has %d neighbours > capacity %d", e[1], e[2], e[3]);
    case MG_ERR_CELL:
        return mg_fail(h, e[0], "particle %d lies outside the cell grid", e[1]);
    case MG_ERR_TIMEOUT:
        return mg_fail(h, e[0], "random stream ran short: particle %d needs pair %d of %d", e[1], e[2], e[3]);
    default:
        return mg_fail(h, e[0], "device error %d (%d %d %d)", e[0], e[1], e[2], e[3]);
    }
}

// ---- phase timing (CUDA events on the handle's stream) ------------------------
static mg_phase *find_phase(mg_handle *h, const char *name) {
    for (auto &p : h->phases)
        if (p.name == name) return &p;
    h->phases.emplace_back();
    mg_phase &p = h->phases.back();
    p.name = name;
    cudaEventCreate(&p.e0);
    cudaEventCreate(&p.e1);
    return &p;
}

int mg_phase_begin(mg_handle *h, const char *name) {
    if (!h->timing) return MG_OK;
    mg_phase *p = find_phase(h, name);
    if (p->pending) {   // collect the previous measurement first
        MG_CUDA(h, cudaEventSynchronize(p->e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, p->e0, p->e1);
        p->total_ms += ms;
        p->count++;
        p->pending = false;
    }
    MG_CUDA(h, cudaEventRecord(p->e0, h->st));
    return MG_OK;
}

int mg_phase_end(mg_handle *h, const char *name) {
    if (!h->timing) return MG_OK;
    mg_phase *p = find_phase(h, name);
    MG_CUDA(h, cudaEventRecord(p->e1, h->st));
    p->pending = true;
    return MG_OK;
}

void mg_phase_collect(mg_handle *h) {
    for (auto &p : h->phases) {
        if (!p.pending) continue;
        float ms = 0;
        if (cudaEventElapsedTime(&ms, p.e0, p.e1) == cudaSuccess) {
            p.total_ms += ms;
            p.count++;
        }
        p.pending = false;
    }
}

// ---- handle ------------------------------------------------------------------
static void free_all(mg_handle *h) {
    mg_mc_free(h);
    void *ptrs[] = {h->d_ro, h->d_az, h->d_type, h->d_pairidx, h->d_ubuf, h->d_r2umin, h->d_r2atat,
                    h->d_ubuf_f, h->d_tab_start, h->d_tab_n, h->d_cellof, h->d_cellcount,
                    h->d_cellstart, h->d_cellfill, h->d_perm, h->d_slot, h->d_nnb, h->d_nbr,
                    h->d_pos_s, h->d_iphead, h->d_npart, h->d_ipnext, h->d_ipprev, h->d_neighcells,
                    h->d_nneighcell, h->d_force, h->d_forceo, h->d_ffx, h->d_part, h->d_uout, h->d_err,
                    h->d_bond_ij, h->d_bond_p, h->d_bond_k, h->d_bond_eq, h->d_bond_off,
                    h->d_bond_list, h->d_angle_ijk, h->d_angle_p, h->d_angle_off, h->d_angle_list, h->d_angle_k,
                    h->d_angle_eq, h->d_chain, h->d_kvec, h->d_kfac, h->d_eik, h->d_S, h->d_Stm, h->d_Q, h->d_F,
                    h->d_Qfx, h->d_mf, h->d_ew, h->d_vw, h->d_mf_f, h->d_ew_f, h->d_vw_f, h->d_tw,
                    h->d_Qref, h->d_phi, h->d_gker, h->d_ipnptm, h->d_rotm, h->d_du, h->d_drostep,
                    h->d_drosum, h->d_blkmax, h->d_rebuild, h->d_massip, h->d_rod, h->d_rodd,
                    h->d_fac1, h->d_fac2, h->d_rng, h->d_rng_save, h->d_cflag, h->d_cidx, h->d_cval,
                    h->d_scan_tmp, h->d_zlow, h->d_coef, h->d_coef_f, h->d_bin_z0, h->d_bin_inv,
                    h->d_bin_kstart, h->d_brick_count, h->d_brick_perm, h->d_brick_rank,
                    h->d_brick_of, h->d_brick_start, h->d_brick_istart, h->d_item_brick, h->d_tiles, h->d_grad, h->d_f32_tabs, h->d_pos_f,
                    h->d_cell_s, h->d_spl_w, h->d_ffx2, h->d_force2, h->d_ro_slot, h->d_ro_slot_f, h->d_scan_tiles,
                    h->d_spl_plane, h->d_dip_scr};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (h->h_pinned) cudaFreeHost(h->h_pinned);
    if (h->h_stage) cudaFreeHost(h->h_stage);
    if (h->g_bd) cudaGraphExecDestroy(h->g_bd);
    if (h->g_bd_io) cudaGraphExecDestroy(h->g_bd_io);
    if (h->d_hostio) cudaFree(h->d_hostio);
    if (h->g_md) cudaGraphExecDestroy(h->g_md);
    for (auto &p : h->phases) {
        cudaEventDestroy(p.e0);
        cudaEventDestroy(p.e1);
    }
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->ev_sr) cudaEventDestroy(h->ev_sr);
    if (h->ev_rec) cudaEventDestroy(h->ev_rec);
    if (h->st2) cudaStreamDestroy(h->st2);
    if (h->st) cudaStreamDestroy(h->st);
}

template <typename T> static int upload(mg_handle *h, T **dst, const T *src, size_t n) {
    MG_CUDA(h, cudaMalloc(dst, sizeof(T) * (n ? n : 1)));
    if (n) MG_CUDA(h, cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice));
    return MG_OK;
}

static int create_impl(const mg_params *p, mg_handle *h) {
    if (p->abi_version != MG_ABI_VERSION) return mg_fail(h, MG_ERR_ARG, "ABI version %d != %d", p->abi_version, MG_ABI_VERSION);
    if (p->np < 2 || p->npt < 1) return mg_fail(h, MG_ERR_ARG, "np = %d, npt = %d", p->np, p->npt);
    if (p->nptpt != p->npt * (p->npt + 1) / 2 || p->nptpt > MG_MAX_NPTPT)
        return mg_fail(h, MG_ERR_UNSUPPORTED, "nptpt = %d (at most %d type pairs)", p->nptpt, MG_MAX_NPTPT);
    if (!p->iptpn || !p->iptpt || !p->az || !p->ubuf || !p->iubuflow || !p->r2umin || !p->r2atat || p->nbuf < 12)
        return mg_fail(h, MG_ERR_ARG, "missing system arrays");
    if (p->form != MG_FP64 && p->form != MG_MIXED) return mg_fail(h, MG_ERR_ARG, "form %d", p->form);
    if (p->mode < MG_MD || p->mode > MG_BD) return mg_fail(h, MG_ERR_ARG, "mode %d", p->mode);
    if (p->txintlist != MG_VLIST && p->txintlist != MG_CELLLIST) return mg_fail(h, MG_ERR_ARG, "txintlist %d", p->txintlist);
    for (int m = 0; m < 3; ++m)
        if (!(p->boxlen[m] > 0)) return mg_fail(h, MG_ERR_ARG, "boxlen(%d) <= 0", m + 1);
    if (!(p->rcut > 0) || p->drnlist < 0) return mg_fail(h, MG_ERR_ARG, "rcut/drnlist");
    h->np = p->np;
    h->npt = p->npt;
    h->nptpt = p->nptpt;
    h->form = p->form;
    h->mode = p->mode;
    h->txintlist = p->txintlist;
    h->ewald = p->ewald;
    h->ncut = p->ncut;
    h->ncut2 = p->ncutregion_cube ? 3 * p->ncut * p->ncut : p->ncut * p->ncut;
    h->order = p->order;
    h->nmesh = p->nmesh;
    h->lsurf = p->lsurf ? 1 : 0;
    h->maxnb = p->maxnneigh;
    h->ualpha = p->ualpha;
    h->EpsiFourPi = p->epsi_four_pi;
    h->force_fac = p->force_fac;
    const double two_pi = 2.0 * 3.1415926535897932;
    for (int m = 0; m < 3; ++m) {
        h->boxlen[m] = p->boxlen[m];
        h->boxlen2[m] = p->boxlen[m] / 2.0;
        h->boxleni[m] = 1.0 / p->boxlen[m];
        h->TwoPiBoxi[m] = two_pi * h->boxleni[m];
    }
    h->vol = p->boxlen[0] * p->boxlen[1] * p->boxlen[2];
    h->rcut = p->rcut;
    h->rcut2 = p->rcut * p->rcut;
    h->drnlist = p->drnlist;
    h->rs2cut = (p->rcut + p->drnlist) * (p->rcut + p->drnlist);
    int np = h->np;

    // types, charges and the self energy (UEwaldSelf, energy.F90:1306-1307)
    h->h_type.resize(np);
    h->h_az.assign(p->az, p->az + np);
    for (int i = 0; i < np; ++i) {
        if (p->iptpn[i] < 1 || p->iptpn[i] > p->npt) return mg_fail(h, MG_ERR_ARG, "iptpn(%d) = %d", i + 1, p->iptpn[i]);
        h->h_type[i] = p->iptpn[i] - 1;
    }
    h->h_pairidx.assign(p->iptpt, p->iptpt + p->npt * p->npt);
    for (int v : h->h_pairidx)
        if (v < 1 || v > p->nptpt) return mg_fail(h, MG_ERR_ARG, "iptpt entry %d", v);
    if (h->ewald != MG_EWALD_NONE) {
        double q2 = 0.0;
        for (int i = 0; i < np; ++i) q2 = q2 + p->az[i] * p->az[i];
        h->u_self = -((h->ualpha / std::sqrt(3.1415926535897932)) * q2);
    }

    // table: record ranges per pair
    std::vector<int> start(p->nptpt), count(p->nptpt);
    for (int k = 0; k < p->nptpt; ++k) {
        int lo = p->iubuflow[k];
        if (lo < 1 || (lo - 1) % 12 != 0 || lo > p->nbuf) return mg_fail(h, MG_ERR_ARG, "iubuflow(%d) = %d", k + 1, lo);
        int hi = p->nbuf + 1;
        for (int q = 0; q < p->nptpt; ++q)
            if (p->iubuflow[q] > lo && p->iubuflow[q] < hi) hi = p->iubuflow[q];
        start[k] = (lo - 1) / 12;
        count[k] = (hi - lo) / 12;
        if (count[k] < 1) return mg_fail(h, MG_ERR_ARG, "empty table for pair %d", k + 1);
    }
    h->nbuf = p->nbuf;
    std::vector<float> ubf(p->nbuf);
    for (int i = 0; i < p->nbuf; ++i) ubf[i] = (float)p->ubuf[i];

    MG_CUDA(h, cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
    MG_CUDA(h, cudaStreamCreateWithFlags(&h->st2, cudaStreamNonBlocking));
    MG_CUDA(h, cudaMallocHost(&h->h_stage, sizeof(double) * kStageDoubles));
    MG_CUDA(h, cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
    MG_CUDA(h, cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));
    MG_CUDA(h, cudaEventCreateWithFlags(&h->ev_sr, cudaEventDisableTiming));
    MG_CUDA(h, cudaEventCreateWithFlags(&h->ev_rec, cudaEventDisableTiming));
    MG_CUDA(h, cudaMalloc(&h->d_ro, sizeof(double) * 3 * np));
    MG_CUDA(h, cudaMemset(h->d_ro, 0, sizeof(double) * 3 * np));
    MG_TRY(upload(h, &h->d_az, p->az, np));
    for (int i = 0; i < np; ++i) h->az_absmax = std::max(h->az_absmax, std::fabs(p->az[i]));
    MG_TRY(upload(h, &h->d_type, h->h_type.data(), np));
    MG_TRY(upload(h, &h->d_pairidx, h->h_pairidx.data(), h->h_pairidx.size()));
    MG_TRY(upload(h, &h->d_ubuf, p->ubuf, p->nbuf));
    MG_TRY(upload(h, &h->d_ubuf_f, ubf.data(), ubf.size()));
    MG_TRY(upload(h, &h->d_r2umin, p->r2umin, p->nptpt));
    MG_TRY(upload(h, &h->d_r2atat, p->r2atat, p->nptpt));
    MG_TRY(upload(h, &h->d_tab_start, start.data(), start.size()));
    MG_TRY(upload(h, &h->d_tab_n, count.data(), count.size()));
    MG_CUDA(h, cudaMalloc(&h->d_err, sizeof(int) * 4));
    MG_CUDA(h, cudaMemset(h->d_err, 0, sizeof(int) * 4));

    // bonds: pairs (0-based) and per-particle CSR of (bond, role)
    h->nbond = p->nbond;
    if (p->nbond > 0) {
        if (!p->bond_ip || !p->bond_jp || !p->bond_k || !p->bond_eq || !p->bond_p) return mg_fail(h, MG_ERR_ARG, "missing bond arrays");
        std::vector<int> ij(2 * p->nbond), deg(np + 1, 0), off(np + 1, 0), list(2 * p->nbond);
        for (int b = 0; b < p->nbond; ++b) {
            int i = p->bond_ip[b] - 1, j = p->bond_jp[b] - 1;
            if (i < 0 || i >= np || j < 0 || j >= np || i == j) return mg_fail(h, MG_ERR_ARG, "bond %d", b + 1);
            if (p->bond_p[b] < 1) return mg_fail(h, MG_ERR_ARG, "bond power %d", p->bond_p[b]);
            ij[2 * b] = i;
            ij[2 * b + 1] = j;
            deg[i]++;
            deg[j]++;
        }
        for (int i = 0; i < np; ++i) off[i + 1] = off[i] + deg[i];
        std::vector<int> fill(off.begin(), off.end() - 1);
        for (int b = 0; b < p->nbond; ++b) {
            list[fill[ij[2 * b]]++] = 2 * b;
            list[fill[ij[2 * b + 1]]++] = 2 * b + 1;
        }
        MG_TRY(upload(h, &h->d_bond_ij, ij.data(), ij.size()));
        MG_TRY(upload(h, &h->d_bond_p, p->bond_p, p->nbond));
        MG_TRY(upload(h, &h->d_bond_k, p->bond_k, p->nbond));
        MG_TRY(upload(h, &h->d_bond_eq, p->bond_eq, p->nbond));
        MG_TRY(upload(h, &h->d_bond_off, off.data(), off.size()));
        MG_TRY(upload(h, &h->d_bond_list, list.data(), list.size()));
    }

    // angles: triples (0-based) and per-particle CSR of (angle, role)
    h->nangle = p->nangle;
    if (p->nangle > 0) {
        if (!p->angle_jm || !p->angle_ip || !p->angle_jp || !p->angle_k || !p->angle_eq || !p->angle_p)
            return mg_fail(h, MG_ERR_ARG, "missing angle arrays");
        int na = p->nangle;
        std::vector<int> ijk(3 * na), deg(np + 1, 0), off(np + 1, 0), list(3 * na);
        for (int a = 0; a < na; ++a) {
            int t[3] = {p->angle_jm[a] - 1, p->angle_ip[a] - 1, p->angle_jp[a] - 1};
            for (int r = 0; r < 3; ++r) {
                if (t[r] < 0 || t[r] >= np) return mg_fail(h, MG_ERR_ARG, "angle %d", a + 1);
                ijk[3 * a + r] = t[r];
                deg[t[r]]++;
            }
            if (t[0] == t[1] || t[1] == t[2] || t[0] == t[2]) return mg_fail(h, MG_ERR_ARG, "angle %d", a + 1);
            if (p->angle_p[a] < 1) return mg_fail(h, MG_ERR_ARG, "angle power %d", p->angle_p[a]);
        }
        for (int i = 0; i < np; ++i) off[i + 1] = off[i] + deg[i];
        std::vector<int> fill(off.begin(), off.end() - 1);
        for (int a = 0; a < na; ++a)
            for (int r = 0; r < 3; ++r) list[fill[ijk[3 * a + r]]++] = 4 * a + r;
        MG_TRY(upload(h, &h->d_angle_ijk, ijk.data(), ijk.size()));
        MG_TRY(upload(h, &h->d_angle_p, p->angle_p, na));
        MG_TRY(upload(h, &h->d_angle_k, p->angle_k, na));
        MG_TRY(upload(h, &h->d_angle_eq, p->angle_eq, na));
        MG_TRY(upload(h, &h->d_angle_off, off.data(), off.size()));
        MG_TRY(upload(h, &h->d_angle_list, list.data(), list.size()));
    }
    if (p->nbond > 0) {
        std::vector<int> chain(5 * (size_t)np, 0);
        for (int i = 0; i < np; ++i) chain[5 * i + 2] = chain[5 * i + 3] = chain[5 * i + 4] = -1;
        for (int b = 0; b < p->nbond; ++b) {
            int i = p->bond_ip[b] - 1, j = p->bond_jp[b] - 1;
            chain[5 * i + 1] = j + 1;
            chain[5 * i + 3] = b;
            chain[5 * j + 0] = i + 1;
            chain[5 * j + 2] = b;
        }
        h->chain_angles = 0;
        for (int a = 0; a < p->nangle; ++a) {
            chain[5 * (p->angle_ip[a] - 1) + 4] = a;
            if (p->angle_k[a] != 0.0) h->chain_angles = 1;
        }
        MG_TRY(upload(h, &h->d_chain, chain.data(), chain.size()));
    }

    if (h->ewald == MG_EWALD_SPM) MG_TRY(mg_spme_init(h));
    else if (h->ewald == MG_EWALD_STD) MG_TRY(mg_ewald_std_init(h));
    else if (h->ewald != MG_EWALD_NONE) return mg_fail(h, MG_ERR_ARG, "ewald = %d", h->ewald);
    MG_TRY(mg_lists_init(h));
    MG_TRY(mg_forces_init(h, p->ubuf, start.data(), count.data()));
    if (h->mode == MG_MC) MG_TRY(mg_mc_init(h));
    MG_CUDA(h, cudaStreamSynchronize(h->st));
    return MG_OK;
}

static thread_local std::string g_create_error;

extern "C" {

int mg_abi_version(void) { return MG_ABI_VERSION; }

const char *mg_status_string(int s) {
    switch (s) {
    case MG_OK: return "MG_OK";
    case MG_ERR_ARG: return "MG_ERR_ARG";
    case MG_ERR_CUDA: return "MG_ERR_CUDA";
    case MG_ERR_TABLE_UNDERRUN: return "MG_ERR_TABLE_UNDERRUN";
    case MG_ERR_NEIGH_OVERFLOW: return "MG_ERR_NEIGH_OVERFLOW";
    case MG_ERR_NAN: return "MG_ERR_NAN";
    case MG_ERR_TIMEOUT: return "MG_ERR_TIMEOUT";
    case MG_ERR_IBUF: return "MG_ERR_IBUF";
    case MG_ERR_TABLE: return "MG_ERR_TABLE";
    case MG_ERR_STATE: return "MG_ERR_STATE";
    case MG_ERR_ALLOC: return "MG_ERR_ALLOC";
    case MG_ERR_UNSUPPORTED: return "MG_ERR_UNSUPPORTED";
    case MG_ERR_CELL: return "MG_ERR_CELL";
    default: return "unknown status";
    }
}

int mg_last_error(const mg_handle *h, char *buf, size_t n) {
    if (!buf || n == 0) return MG_ERR_ARG;
    const std::string &s = h ? h->err : g_create_error;
    std::snprintf(buf, n, "%s", s.c_str());
    return MG_OK;
}

int mg_create(const mg_params *p, mg_handle **out) {
    if (!p || !out) return MG_ERR_ARG;
    *out = nullptr;
    mg_handle *h = new mg_handle();
    cudaGetDevice(&h->dev);
    int st = create_impl(p, h);
    if (st != MG_OK) {
        g_create_error = h->err;
        free_all(h);
        delete h;
        return st;
    }
    *out = h;
    return MG_OK;
}

int mg_destroy(mg_handle *h) {
    if (!h) return MG_ERR_ARG;
    cudaStreamSynchronize(h->st);
    free_all(h);
    delete h;
    return MG_OK;
}

int mg_set_positions(mg_handle *h, const double *ro) {
    if (!h || !ro) return MG_ERR_ARG;
    MG_CUDA(h, cudaMemcpyAsync(h->d_ro, ro, sizeof(double) * 3 * h->np, cudaMemcpyHostToDevice, h->st));
    MG_CUDA(h, cudaStreamSynchronize(h->st));
    h->have_force = false;
    return MG_OK;
}

int mg_get_positions(mg_handle *h, double *ro) {
    if (!h || !ro) return MG_ERR_ARG;
    MG_CUDA(h, cudaMemcpyAsync(ro, h->d_ro, sizeof(double) * 3 * h->np, cudaMemcpyDeviceToHost, h->st));
    MG_CUDA(h, cudaStreamSynchronize(h->st));
    return MG_OK;
}

int mg_nlist_set(mg_handle *h) {
    if (!h) return MG_ERR_ARG;
    MG_TRY(mg_lists_build(h, false));
    if (h->mode == MG_MC && h->txintlist == MG_CELLLIST) MG_TRY(mg_mc_cells_set(h));
    MG_CUDA(h, cudaMemsetAsync(h->d_drosum, 0, sizeof(double) * 3 * h->np, h->st));
    MG_CUDA(h, cudaMemsetAsync(h->d_rebuild, 0, sizeof(int) * 2, h->st));
    MG_TRY(mg_lists_reset_calls(h));
    int st = mg_check_device_error(h);
    if (st != MG_OK) h->list_valid = false;   // an overflowed or failed build is no list
    return st;
}

int mg_nlist_update(mg_handle *h, const double *drostep, int32_t *rebuilt) {
    if (!h || !rebuilt) return MG_ERR_ARG;
    *rebuilt = 0;
    if (!h->list_valid) return mg_fail(h, MG_ERR_STATE, "mg_nlist_set has not been called");
    if (h->txintlist == MG_CELLLIST && h->mode == MG_MC) return MG_OK;   // UpdateCellIp keeps cells
    if (drostep)
        MG_CUDA(h, cudaMemcpyAsync(h->d_drostep, drostep, sizeof(double) * 3 * h->np, cudaMemcpyHostToDevice, h->st));
    MG_TRY(mg_lists_check(h));
    MG_TRY(mg_lists_build(h, true));
    int flag = 0;
    MG_CUDA(h, cudaMemcpyAsync(&flag, h->d_rebuild, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    int st = mg_check_device_error(h);
    if (st != MG_OK) {
        h->list_valid = false;   // an overflowed or failed rebuild is no list
        return st;
    }
    *rebuilt = flag;
    return MG_OK;
}

int mg_fft_check(mg_handle *h, const double *q, const double *mult, const double *ew, double *phi,
                 double *esum) {
    if (!h || !q || !mult || !ew || !phi || !esum) return MG_ERR_ARG;
    if (h->ewald != MG_EWALD_SPM) return mg_fail(h, MG_ERR_STATE, "the handle has no SPME mesh");
    MG_CUDA(h, cudaStreamSynchronize(h->st));
    MG_TRY(mg_spme_fft_check(h, q, mult, ew, phi, esum));
    h->have_force = false;
    h->have_rec = false;
    return MG_OK;
}

int mg_nlist_calls(mg_handle *h, int32_t *ncall) {
    if (!h || !ncall) return MG_ERR_ARG;
    if (!h->list_valid) return mg_fail(h, MG_ERR_STATE, "mg_nlist_set has not been called");
    int v[3];
    MG_CUDA(h, cudaMemcpyAsync(v, h->d_rebuild, sizeof(int) * 3, cudaMemcpyDeviceToHost, h->st));
    MG_CUDA(h, cudaStreamSynchronize(h->st));
    *ncall = v[2];
    return MG_OK;
}

int mg_nlist_get(mg_handle *h, int32_t *nneighpn, int32_t *jpnlist, int32_t maxnneigh) {
    if (!h || !nneighpn || !jpnlist || maxnneigh < 1) return MG_ERR_ARG;
    return mg_lists_export(h, nneighpn, jpnlist, maxnneigh);
}

int mg_celllist_get(mg_handle *h, int32_t *ncell, int32_t *cellip) {
    if (!h || !ncell || !cellip) return MG_ERR_ARG;
    return mg_cells_export(h, ncell, cellip);
}

int mg_energy_terms(mg_handle *h, double *terms) {
    if (!h || !terms) return MG_ERR_ARG;
    int n = h->nptpt + 1 + 8;
    std::vector<double> u(n);
    MG_CUDA(h, cudaStreamSynchronize(h->st));
    MG_CUDA(h, cudaMemcpy(u.data(), h->d_uout, sizeof(double) * n, cudaMemcpyDeviceToHost));
    int o = h->nptpt + 1;
    terms[0] = u[o + 0];   // u%tot
    terms[1] = u[0];       // u%twob(0)
    terms[2] = u[o + 1];   // u%rec
    terms[3] = u[o + 2];   // u%bond
    terms[4] = u[o + 7];   // u%angle
    terms[5] = u[o + 3];   // virial
    return MG_OK;
}

int mg_utotal(mg_handle *h, double *forceo, double *u_twob, double *uout) {
    if (!h) return MG_ERR_ARG;
    if (!h->list_valid) return mg_fail(h, MG_ERR_STATE, "mg_nlist_set has not been called");
    if (h->list_stale) {   // MC with a cell list: the reference's pair sum sees the current cells
        MG_TRY(mg_lists_build(h, false));
        h->list_stale = false;
    }
    MG_TRY(mg_utotal_launch(h));
    MG_TRY(mg_utotal_fetch(h, forceo, u_twob, uout));
    h->have_force = true;
    h->have_rec = true;
    if (h->mode == MG_MC && h->ewald != MG_EWALD_NONE) MG_TRY(mg_mc_after_utotal(h));
    return MG_OK;
}

int mg_dutotal(mg_handle *h, int32_t nptm, const int32_t *ipnptm, const double *rotm,
               double *du_twob, double *du_rec, double *du_tot, int32_t *lhsoverlap) {
    if (!h || !ipnptm || !rotm || nptm < 1 || nptm > h->np) return MG_ERR_ARG;
    if (h->mode != MG_MC) return mg_fail(h, MG_ERR_STATE, "DUTotal needs mode MG_MC");
    return mg_mc_dutotal(h, nptm, ipnptm, rotm, du_twob, du_rec, du_tot, lhsoverlap);
}

int mg_accept(mg_handle *h) {
    if (!h) return MG_ERR_ARG;
    return mg_mc_accept(h);
}

int mg_dutotal_batch(mg_handle *h, int32_t ntrial, const int32_t *ip, const double *rtrial,
                     double *du_tot, int32_t *lhsoverlap) {
    if (!h || ntrial < 0 || (ntrial > 0 && (!ip || !rtrial || !du_tot || !lhsoverlap))) return MG_ERR_ARG;
    if (h->mode != MG_MC) return mg_fail(h, MG_ERR_STATE, "DUTotal needs mode MG_MC");
    return mg_mc_batch(h, ntrial, ip, rtrial, du_tot, lhsoverlap);
}

int mg_md_setup(mg_handle *h, double tstep, const double *massip, const double *rod, const double *rodd) {
    if (!h || !massip || !rod || !rodd || !(tstep > 0)) return MG_ERR_ARG;
    return mg_integrate_md_setup(h, tstep, massip, rod, rodd);
}

// Append one device step of handle h to the graph that h->st is being
// captured into.  The Verlet-list rebuild goes into the body of a
// conditional (IF) node whose condition the list check sets on the device,
// so steps without a rebuild launch none of its kernels.
static int capture_step_body(mg_handle *h, bool bd) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg = nullptr;
    cudaError_t ce = cudaStreamGetCaptureInfo(h->st, &cs, nullptr, &cg, nullptr, nullptr, nullptr);
    if (ce == cudaSuccess) ce = cudaGraphConditionalHandleCreate(&h->cond, cg, 0, cudaGraphCondAssignDefault);
    int st = MG_OK;
    if (ce == cudaSuccess) {
        h->use_cond = true;
        st = bd ? mg_integrate_bd_step_launch(h) : mg_integrate_md_step_launch(h);
        h->use_cond = false;
    }
    if (ce == cudaSuccess && st == MG_OK) {
        const cudaGraphNode_t *deps = nullptr;
        const cudaGraphEdgeData *edges = nullptr;
        size_t ndeps = 0;
        ce = cudaStreamGetCaptureInfo(h->st, &cs, nullptr, &cg, &deps, &edges, &ndeps);
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h->cond;
        cp.conditional.type = cudaGraphCondTypeIf;
        cp.conditional.size = 1;
        cudaGraphNode_t cn = nullptr;
        if (ce == cudaSuccess) ce = cudaGraphAddNode(&cn, cg, deps, edges, ndeps, &cp);
        if (ce == cudaSuccess) ce = cudaStreamUpdateCaptureDependencies(h->st, &cn, nullptr, 1, cudaStreamSetCaptureDependencies);
        if (ce == cudaSuccess) {
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            cudaStream_t side = nullptr;
            ce = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
            if (ce == cudaSuccess) ce = cudaStreamBeginCaptureToGraph(side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
            if (ce == cudaSuccess) {
                cudaStream_t keep = h->st;
                h->st = side;
                st = mg_lists_build(h, false);
                h->st = keep;
                cudaGraph_t b2 = nullptr;
                cudaError_t ce2 = cudaStreamEndCapture(side, &b2);
                if (ce2 != cudaSuccess) ce = ce2;
            }
            if (side) cudaStreamDestroy(side);
        }
    }
    if (st != MG_OK) return st;
    if (ce != cudaSuccess) return mg_fail(h, MG_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
    return MG_OK;
}

static int count_kernels(cudaGraph_t graph) {
    size_t nn = 0;
    cudaGraphGetNodes(graph, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (nn) cudaGraphGetNodes(graph, nodes.data(), &nn);
    int nk = 0;
    for (auto &n : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(n, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++nk;
    }
    return nk;
}

static int capture_step(mg_handle *h, bool bd, bool io = false) {
    cudaGraphExec_t &g = io ? h->g_bd_io : bd ? h->g_bd : h->g_md;
    if (g) return MG_OK;
    cudaGraph_t graph = nullptr;
    MG_CUDA(h, cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    h->hostio = io;
    int st = capture_step_body(h, bd);
    h->hostio = false;
    cudaError_t ce = cudaStreamEndCapture(h->st, &graph);
    if (st != MG_OK || ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        if (st != MG_OK) return st;
        return mg_fail(h, MG_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
    }
    if (!io) (bd ? h->kernels_bd : h->kernels_md) = count_kernels(graph);
    ce = cudaGraphInstantiate(&g, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return mg_fail(h, MG_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
    return MG_OK;
}

static int run_steps(mg_handle *h, int nstep, bool bd) {
    cudaGraphExec_t &g = bd ? h->g_bd : h->g_md;
    if (h->timing) {   // uncaptured launches so every phase can be timed
        for (int s = 0; s < nstep; ++s) {
            MG_TRY(bd ? mg_integrate_bd_step_launch(h) : mg_integrate_md_step_launch(h));
            MG_TRY(mg_check_device_error(h));
        }
        return MG_OK;
    }
    MG_TRY(capture_step(h, bd));
    if (bd && nstep > 0) MG_TRY(mg_integrate_bd_prime(h));
    for (int s = 0; s < nstep; ++s) MG_CUDA(h, cudaGraphLaunch(g, h->st));
    return MG_OK;
}

int mg_md_run(mg_handle *h, int32_t nstep, double *forceo, double *uout, double *rod, double *rodd) {
    if (!h || nstep < 0) return MG_ERR_ARG;
    if (!h->md_ready) return mg_fail(h, MG_ERR_STATE, "mg_md_setup has not been called");
    if (!h->list_valid) return mg_fail(h, MG_ERR_STATE, "mg_nlist_set has not been called");
    MG_TRY(run_steps(h, nstep, false));
    MG_TRY(mg_utotal_fetch(h, forceo, nullptr, uout));
    if (rod) MG_CUDA(h, cudaMemcpy(rod, h->d_rod, sizeof(double) * 3 * h->np, cudaMemcpyDeviceToHost));
    if (rodd) MG_CUDA(h, cudaMemcpy(rodd, h->d_rodd, sizeof(double) * 3 * h->np, cudaMemcpyDeviceToHost));
    h->have_force = true;
    return MG_OK;
}

int mg_bd_setup(mg_handle *h, const double *fac1, const double *fac2, int32_t iseed) {
    if (!h || !fac1 || !fac2) return MG_ERR_ARG;
    // GauRandom's LCG stays at 0 from a seed that is 0 modulo 2^31
    if (((uint32_t)iseed & 0x7fffffffu) == 0) return mg_fail(h, MG_ERR_ARG, "iseed must be nonzero modulo 2^31");
    return mg_integrate_bd_setup(h, fac1, fac2, iseed);
}

int mg_bd_run(mg_handle *h, int32_t nstep, double *forceo, double *uout) {
    if (!h || nstep < 0) return MG_ERR_ARG;
    if (!h->bd_ready) return mg_fail(h, MG_ERR_STATE, "mg_bd_setup has not been called");
    if (!h->list_valid) return mg_fail(h, MG_ERR_STATE, "mg_nlist_set has not been called");
    if (!h->have_force) {   // initial forces (UTotal before the first BDStep)
        MG_TRY(mg_utotal_launch(h));
        MG_TRY(mg_check_device_error(h));
        h->have_force = true;
    }
    MG_TRY(run_steps(h, nstep, true));
    return mg_utotal_fetch(h, forceo, nullptr, uout);
}

// true when the device can read and write p in place (pinned host memory
// mapped into the device address space, the pointer valid on the device)
static bool device_mapped_host(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost && at.devicePointer == p;
}

int mg_bd_step_host(mg_handle *h, double *ro_io, double *forceo, double *uout) {
    if (!h || !ro_io) return MG_ERR_ARG;
    if (!h->bd_ready || !h->list_valid) return mg_fail(h, MG_ERR_STATE, "BD not set up");
    // pinned, mapped buffers: the step's kernels read and write them in place
    // (positions in the move kernel, forces in the step's last kernel)
    bool cached = h->hostio_last.ro == ro_io && h->hostio_last.forceo == forceo;   // checked before
    if (!h->timing && h->have_force && forceo &&
        (cached || (device_mapped_host(ro_io) && device_mapped_host(forceo) && device_mapped_host(h->h_stage)))) {
        if (!h->d_hostio) MG_CUDA(h, cudaMalloc(&h->d_hostio, sizeof(mg_hostio)));
        if (h->hostio_last.ro != ro_io || h->hostio_last.forceo != forceo) {
            mg_hostio io = {ro_io, forceo, h->h_stage, h->d_uout, h->d_err, h->nptpt + 1 + 4};
            MG_CUDA(h, cudaMemcpy(h->d_hostio, &io, sizeof(io), cudaMemcpyHostToDevice));
            h->hostio_last = io;
        }
        MG_TRY(capture_step(h, true, true));
        MG_TRY(mg_integrate_bd_prime(h));
        MG_CUDA(h, cudaGraphLaunch(h->g_bd_io, h->st));
        MG_CUDA(h, cudaStreamSynchronize(h->st));
        return mg_utotal_staged(h, nullptr, uout);
    }
    MG_CUDA(h, cudaMemcpyAsync(h->d_ro, ro_io, sizeof(double) * 3 * h->np, cudaMemcpyHostToDevice, h->st));
    if (!h->have_force) {
        MG_TRY(mg_utotal_launch(h));
        h->have_force = true;
    }
    MG_TRY(run_steps(h, 1, true));
    MG_CUDA(h, cudaMemcpyAsync(ro_io, h->d_ro, sizeof(double) * 3 * h->np, cudaMemcpyDeviceToHost, h->st));
    return mg_utotal_fetch(h, forceo, nullptr, uout);
}

int mg_bd_get_seed(mg_handle *h, int32_t *iseed) {
    if (!h || !iseed || !h->bd_ready) return MG_ERR_ARG;
    int st[4];
    MG_CUDA(h, cudaStreamSynchronize(h->st));
    MG_CUDA(h, cudaMemcpy(st, h->d_rng, sizeof(st), cudaMemcpyDeviceToHost));
    *iseed = st[0];
    return MG_OK;
}

int mg_phase_times(mg_handle *h, double *ms, int32_t nmax, int32_t *nphase, char *names, size_t names_len) {
    if (!h || !nphase) return MG_ERR_ARG;
    MG_CUDA(h, cudaStreamSynchronize(h->st));
    mg_phase_collect(h);
    std::string all;
    int k = 0;
    for (auto &p : h->phases) {
        if (k < nmax && ms) ms[k] = p.count ? p.total_ms / p.count : 0.0;
        if (k) all += ",";
        all += p.name;
        ++k;
    }
    *nphase = k;
    if (names && names_len) std::snprintf(names, names_len, "%s", all.c_str());
    return MG_OK;
}

// Reads the L2 flush buffer back after it was written: the write leaves up
// to the whole L2 dirty, and the read makes those lines be written back
// before the timed step instead of during it.  The sum is stored only when
// it equals an arbitrary constant, which keeps the loads.
__global__ void k_l2_sweep(const uint4 *__restrict__ p, size_t n16, unsigned *sink) {
    unsigned x = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x) {
        uint4 v = p[i];
        x ^= v.x ^ v.y ^ v.z ^ v.w;
    }
    if (x == 0x9e3779b9u) *sink = x;
}

int mg_bench_steps(mg_handle *h, int32_t kind, int32_t nstep, int64_t flush_bytes, double *ms_sum) {
    if (!h || !ms_sum || nstep < 0 || flush_bytes < 0) return MG_ERR_ARG;
    bool bd = kind == 1;
    if (bd ? !h->bd_ready : !h->md_ready) return mg_fail(h, MG_ERR_STATE, "integrator not set up");
    if (!h->list_valid) return mg_fail(h, MG_ERR_STATE, "mg_nlist_set has not been called");
    if (bd && !h->have_force) {
        MG_TRY(mg_utotal_launch(h));
        MG_TRY(mg_check_device_error(h));
        h->have_force = true;
    }
    void *flush = nullptr;
    if (flush_bytes) MG_CUDA(h, cudaMalloc(&flush, (size_t)flush_bytes));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double total = 0.0;
    int st = MG_OK;
    if (!h->timing) st = capture_step(h, bd);
    if (st == MG_OK && bd && !h->timing) st = mg_integrate_bd_prime(h);
    for (int s = 0; s < nstep && st == MG_OK; ++s) {
        if (flush) {   // L2 flushed: written, then read back (clean lines)
            cudaMemsetAsync(flush, s & 0xff, (size_t)flush_bytes, h->st);
            k_l2_sweep<<<8 * 152, 256, 0, h->st>>>((const uint4 *)flush, (size_t)flush_bytes / 16,
                                                   (unsigned *)flush);
        }
        cudaEventRecord(e0, h->st);
        if (h->timing) st = bd ? mg_integrate_bd_step_launch(h) : mg_integrate_md_step_launch(h);
        else if (cudaGraphLaunch(bd ? h->g_bd : h->g_md, h->st) != cudaSuccess)
            st = mg_fail(h, MG_ERR_CUDA, "graph launch failed");
        cudaEventRecord(e1, h->st);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            st = mg_fail(h, MG_ERR_CUDA, "step %d failed: %s", s, cudaGetErrorString(cudaGetLastError()));
            break;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        total += ms;
        if (h->timing) mg_phase_collect(h);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (flush) cudaFree(flush);
    if (st != MG_OK) return st;
    *ms_sum = total;
    return mg_check_device_error(h);
}

int mg_step_kernels(mg_handle *h, int32_t kind, int32_t *nkernels) {
    if (!h || !nkernels) return MG_ERR_ARG;
    *nkernels = (kind == 1) ? h->kernels_bd : h->kernels_md;
    return MG_OK;
}

int mg_phase_reset(mg_handle *h, int32_t enable) {
    if (!h) return MG_ERR_ARG;
    MG_CUDA(h, cudaStreamSynchronize(h->st));
    mg_phase_collect(h);
    for (auto &p : h->phases) {
        p.total_ms = 0;
        p.count = 0;
        p.pending = false;
    }
    h->timing = enable != 0;
    return MG_OK;
}

}  // extern "C"

// ---- ensembles of independent systems --------------------------------------
//
// Every replica keeps its own handle (arrays, stream, lists); the ensemble
// captures one step of all of them into a single CUDA graph -- one branch per
// replica, forked from and joined to the ensemble's stream -- so one graph
// launch advances every replica by one step and the replicas' small kernels
// run side by side.  Each branch is the replica's own step, so a replica in
// an ensemble follows the same trajectory as when it runs alone.

struct mg_ensemble {
    std::vector<mg_handle *> hs;
    cudaStream_t st = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    cudaGraphExec_t g[2] = {nullptr, nullptr};
    int kernels[2] = {0, 0};
    std::string err;
};

#define MG_TRY_E(e, x)                  \
    do {                                \
        int _s = (x);                   \
        if (_s != MG_OK) return _s;     \
    } while (0)

static int ens_fail(mg_ensemble *e, int code, const char *msg) {
    if (e) e->err = msg;
    return code;
}

int mg_ensemble_create(int32_t nrep, mg_handle *const *handles, mg_ensemble **out) {
    if (nrep < 1 || !handles || !out) return MG_ERR_ARG;
    *out = nullptr;
    mg_ensemble *e = new (std::nothrow) mg_ensemble();
    if (!e) return MG_ERR_ALLOC;
    int dev = handles[0] ? handles[0]->dev : 0;
    for (int r = 0; r < nrep; ++r) {
        if (!handles[r] || handles[r]->dev != dev) {
            delete e;
            return MG_ERR_ARG;
        }
        e->hs.push_back(handles[r]);
    }
    cudaSetDevice(dev);
    if (cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming) != cudaSuccess) {
        mg_ensemble_destroy(e);
        return MG_ERR_CUDA;
    }
    e->join.resize(nrep, nullptr);
    for (int r = 0; r < nrep; ++r)
        if (cudaEventCreateWithFlags(&e->join[r], cudaEventDisableTiming) != cudaSuccess) {
            mg_ensemble_destroy(e);
            return MG_ERR_CUDA;
        }
    *out = e;
    return MG_OK;
}

int mg_ensemble_destroy(mg_ensemble *e) {
    if (!e) return MG_OK;
    for (int k = 0; k < 2; ++k)
        if (e->g[k]) cudaGraphExecDestroy(e->g[k]);
    for (cudaEvent_t ev : e->join)
        if (ev) cudaEventDestroy(ev);
    if (e->fork) cudaEventDestroy(e->fork);
    if (e->st) cudaStreamDestroy(e->st);
    delete e;
    return MG_OK;
}

static int ens_capture(mg_ensemble *e, int kind) {
    if (e->g[kind]) return MG_OK;
    bool bd = kind == 1;
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return ens_fail(e, MG_ERR_CUDA, "ensemble: begin capture failed");
    cudaError_t ce = cudaEventRecord(e->fork, e->st);
    int st = MG_OK;
    for (size_t r = 0; r < e->hs.size() && ce == cudaSuccess && st == MG_OK; ++r) {
        mg_handle *h = e->hs[r];
        ce = cudaStreamWaitEvent(h->st, e->fork, 0);   // the replica's stream joins the capture
        if (ce == cudaSuccess) st = capture_step_body(h, bd);
        if (ce == cudaSuccess && st == MG_OK) ce = cudaEventRecord(e->join[r], h->st);
        if (ce == cudaSuccess && st == MG_OK) ce = cudaStreamWaitEvent(e->st, e->join[r], 0);
        if (st != MG_OK) e->err = "replica " + std::to_string(r) + ": " + h->err;
    }
    cudaError_t ce2 = cudaStreamEndCapture(e->st, &graph);
    if (st != MG_OK || ce != cudaSuccess || ce2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        if (st != MG_OK) return st;
        e->err = std::string("ensemble capture: ") + cudaGetErrorString(ce != cudaSuccess ? ce : ce2);
        return MG_ERR_CUDA;
    }
    e->kernels[kind] = count_kernels(graph);
    ce = cudaGraphInstantiate(&e->g[kind], graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return ens_fail(e, MG_ERR_CUDA, "ensemble: graph instantiate failed");
    return MG_OK;
}

int mg_ensemble_run(mg_ensemble *e, int32_t kind, int32_t nstep, double *ms) {
    if (!e || nstep < 0 || (kind != 0 && kind != 1)) return MG_ERR_ARG;
    for (size_t r = 0; r < e->hs.size(); ++r) {
        mg_handle *h = e->hs[r];
        if (!(kind ? h->bd_ready : h->md_ready) || !h->list_valid)
            return ens_fail(e, MG_ERR_STATE, "every replica needs mg_md_setup / mg_bd_setup and mg_nlist_set");
        if (h->timing) return ens_fail(e, MG_ERR_STATE, "phase timing must be off in an ensemble");
        if (kind == 1 && !h->have_force) {   // BD: forces of the starting configuration, as mg_bd_run
            MG_TRY(mg_utotal_launch(h));
            h->have_force = true;
        }
        if (kind == 1) MG_TRY(mg_integrate_bd_prime(h));
        if (cudaStreamSynchronize(h->st) != cudaSuccess) return ens_fail(e, MG_ERR_CUDA, "replica stream");
    }
    MG_TRY_E(e, ens_capture(e, kind));
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (ms) {
        cudaEventCreate(&t0);
        cudaEventCreate(&t1);
        cudaEventRecord(t0, e->st);
    }
    for (int s = 0; s < nstep; ++s)
        if (cudaGraphLaunch(e->g[kind], e->st) != cudaSuccess) return ens_fail(e, MG_ERR_CUDA, "graph launch");
    if (ms) cudaEventRecord(t1, e->st);
    if (cudaStreamSynchronize(e->st) != cudaSuccess) return ens_fail(e, MG_ERR_CUDA, "ensemble step failed");
    if (ms) {
        float f = 0.0f;
        cudaEventElapsedTime(&f, t0, t1);
        *ms = f;
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
    }
    for (size_t r = 0; r < e->hs.size(); ++r) {
        int st = mg_check_device_error(e->hs[r]);
        if (st != MG_OK) {
            e->err = "replica " + std::to_string(r) + ": " + e->hs[r]->err;
            return st;
        }
    }
    return MG_OK;
}

int mg_ensemble_kernels(mg_ensemble *e, int32_t kind, int32_t *nkernels) {
    if (!e || !nkernels || (kind != 0 && kind != 1)) return MG_ERR_ARG;
    *nkernels = e->kernels[kind];
    return MG_OK;
}

int mg_ensemble_last_error(const mg_ensemble *e, char *buf, size_t n) {
    if (!e || !buf || n == 0) return MG_ERR_ARG;
    std::snprintf(buf, n, "%s", e->err.c_str());
    return MG_OK;
}
