"""Shared helpers for parity tests: systems, comparisons, tolerances."""
import dataclasses

import numpy as np

from molsim_gb300 import Engine, abi, configs

# Tolerances.  Plain FP64 form against the oracle: energies and virial within
# 1e-10 relative; forces within 1e-10 of the largest force magnitude (a
# per-component relative test is meaningless for components near zero).
# Mixed form: force RMS error <= 1e-5 of the RMS force.
TOL_FP64 = 1e-10
TOL_MIXED_RMS = 1e-5


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def force_err(f, fref):
    d = np.asarray(f) - np.asarray(fref)
    return np.abs(d).max() / np.abs(fref).max()


def force_rms_err(f, fref):
    d = np.asarray(f) - np.asarray(fref)
    return np.sqrt((d * d).sum() / (np.asarray(fref) ** 2).sum())


def prepared(system, orc):
    """System with its table built by the oracle (the library's own table
    builder is checked against this one separately)."""
    system.build_table(orc.orc_pot_twobody_tab)
    return system


def run_pair(system, orc, form=abi.MG_FP64):
    """UTotal from the oracle and from the GPU for the same system."""
    ref = Engine(system, lib=orc, prefix="orc_")
    ref.SetPositions(system.ro_flat())
    ref.NList("write")
    r = ref.UTotal()
    gpu = Engine(system, form=form)
    gpu.SetPositions(system.ro_flat())
    gpu.NList("write")
    g = gpu.UTotal()
    return r, g, ref, gpu


def small_cases():
    """(name, factory) for the UTotal parity matrix."""
    return [
        ("spme_vlist_md", lambda: configs.small_system(seed=11)),
        ("spme_cell_md", lambda: configs.small_system(seed=12, txintlist=abi.MG_CELLLIST)),
        ("spme_surf", lambda: configs.small_system(seed=13, lsurf=1)),
        ("spme_bonds", lambda: configs.small_system(seed=14, chains=4, nseg=12)),
        ("spme_order4_n32", lambda: configs.small_system(seed=15, nmesh=32, order=4, n=600, L=50.0)),
        ("std_vlist", lambda: configs.small_system(seed=16, ewald=abi.MG_EWALD_STD, ncut=6)),
        ("std_cell_surf", lambda: configs.small_system(seed=17, ewald=abi.MG_EWALD_STD, ncut=5,
                                                       txintlist=abi.MG_CELLLIST, lsurf=1)),
        ("no_ewald", lambda: configs.small_system(seed=18, ewald=abi.MG_EWALD_NONE)),
        ("wca_lljcut", lambda: configs.small_system(seed=19, lljcut=1)),
        ("mc_mode", lambda: configs.small_system(seed=20, mode=abi.MG_MC)),
        ("spme_order8_n64", lambda: configs.small_system(seed=21, nmesh=64, order=8)),
        ("spme_order10_n128", lambda: configs.small_system(seed=22, nmesh=128, order=10, n=500, L=45.0)),
        ("spme_order4_n128", lambda: configs.small_system(seed=23, nmesh=128, order=4, n=600, L=50.0)),
        ("spme_order6_n256", lambda: configs.small_system(seed=24, nmesh=256, order=6, n=500, L=45.0)),
        ("spme_bonds_angles", lambda: configs.small_system(seed=25, chains=4, nseg=12, angle_kt=1.0)),
        # meshes 2^a 3^b 5^c that are not powers of two (generic spread, gather, FFT radices 3 and 5)
        ("spme_n40", lambda: configs.small_system(seed=26, nmesh=40)),
        ("spme_n24_order4", lambda: configs.small_system(seed=27, nmesh=24, order=4)),
        ("spme_n60_order8_surf", lambda: configs.small_system(seed=28, nmesh=60, order=8, lsurf=1)),
        ("spme_n120_cell", lambda: configs.small_system(seed=29, nmesh=120, n=500, L=45.0,
                                                        txintlist=abi.MG_CELLLIST)),
    ]


def utotal_errors(g, r, nptpt):
    """Relative errors of every UTotal output (energies against their own
    magnitude, forces against the largest force)."""
    e = {}
    for k in range(nptpt + 1):
        e[f"u_twob[{k}]"] = abs(g["u_twob"][k] - r["u_twob"][k]) / max(abs(r["u_twob"][k]), 1e-12)
    e["u_rec"] = abs(g["u_rec"] - r["u_rec"]) / max(abs(r["u_rec"]), 1.0)
    e["u_bond"] = abs(g["u_bond"] - r["u_bond"]) / max(abs(r["u_bond"]), 1e-12)
    e["u_tot"] = rel(g["u_tot"], r["u_tot"])
    e["virial"] = rel(g["virial"], r["virial"])
    e["force_max"] = force_err(g["forceo"], r["forceo"])
    e["force_rms"] = force_rms_err(g["forceo"], r["forceo"])
    return e


def chain_trial(rng, s, ro, chains, nseg, step=1.0):
    """A trial on the chain beads (particles 1 .. chains*nseg, nseg per
    chain): one bead, or a string of 2-4 consecutive beads of one chain in
    chain order, each displaced by up to step."""
    c = int(rng.integers(chains))
    n = 1 if rng.random() < 0.4 else int(rng.integers(2, 5))
    i0 = int(rng.integers(nseg - n + 1))
    ips = c * nseg + i0 + np.arange(n)
    L = s.boxlen[0]
    new = ro[ips] + rng.uniform(-step, step, (n, 3))
    new -= L * np.round(new / L)
    return ips + 1, new


def chain_system(seed=71, chains=4, nseg=10, **kw):
    """small_system with the chain beads as a fourth particle type (a copy
    of their ion type), as the reference gives chain particles their own
    types."""
    s = configs.small_system(seed=seed, mode=abi.MG_MC, chains=chains, nseg=nseg, angle_kt=0.5, **kw)
    t = int(s.iptpn[0]) - 1
    s.species = list(s.species) + [dataclasses.replace(s.species[t], name="bead")]
    s.iptpn = s.iptpn.copy()
    s.iptpn[:chains * nseg] = len(s.species)
    return s


def brush_system(seed=74, ngraft=6, chains=12, nseg=5, n=400, L=40.0, **kw):
    """A brush for BrushCl2Move: ngraft grafting particles (a fourth type, a
    copy of the divalent ion type) numbered first, then `chains` bonded
    chains of nseg beads (chain ic grafted cyclically on particle
    ((ic - 1) mod ngraft) + 1, as the reference's brush loop reads it), then
    the other ions.  Built from small_system by moving the first ngraft
    divalent ions to the front."""
    s = configs.small_system(seed=seed, mode=abi.MG_MC, chains=chains, nseg=nseg, n=n, L=L, angle_kt=0.0, **kw)
    nbead = chains * nseg
    types = np.asarray(s.iptpn)
    div = [i for i in range(nbead, s.np_) if types[i] == 3][:ngraft]
    if len(div) < ngraft:
        raise ValueError("not enough divalent ions to graft on")
    rest = [i for i in range(nbead, s.np_) if i not in set(div)]
    order = np.array(div + list(range(nbead)) + rest)
    new_of = np.empty(s.np_, dtype=np.int64)
    new_of[order] = np.arange(s.np_)
    s.ro = np.asarray(s.ro)[order].copy()
    s.iptpn = types[order].astype(np.int32)
    s.species = list(s.species) + [dataclasses.replace(s.species[2], name="graft")]
    s.iptpn[:ngraft] = len(s.species)
    s.bond_ip = (new_of[np.asarray(s.bond_ip) - 1] + 1).astype(np.int32)
    s.bond_jp = (new_of[np.asarray(s.bond_jp) - 1] + 1).astype(np.int32)
    return s


def centre_lists(ro, L, rlist, full=False):
    """A Verlet list of particle centres (nneighpn, jpnlist as NList stores
    it: 1-based, maxnneigh entries per particle): every pair within rlist
    (minimum image) once, on its lower-numbered particle, or (full, the MC
    list) on both."""
    ro = np.asarray(ro)
    d = ro[:, None, :] - ro[None, :, :]
    d -= L * np.round(d / L)
    r2 = (d * d).sum(-1)
    n = len(ro)
    near = (r2 <= rlist * rlist) & ~np.eye(n, dtype=bool)
    if not full:
        near &= np.triu(np.ones((n, n), dtype=bool), 1)
    nn = near.sum(1).astype(np.int32)
    maxn = max(1, int(nn.max()))
    jl = np.zeros((n, maxn), dtype=np.int32)
    for i in range(n):
        js = np.flatnonzero(near[i]) + 1
        jl[i, :len(js)] = js
    return nn, jl, maxn
