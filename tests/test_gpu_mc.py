"""MC trial-move energy differences on the GPU against the oracle.

DUTotal (denergy.F90:98-215) and MCUpdate (mc.F90:5203-5235): the same
sequence of trials -- single and multi-particle moves, some of them
overlapping -- runs on the oracle and on the GPU, and every accepted trial
is accepted on both.  Tolerances (plain FP64 form): the two-body and
reciprocal differences within 1e-10 of the corresponding total energies
(the reference forms them as differences of such sums, so its own rounding
floor is ~1e-16 of them); overlap flags equal; positions after the sequence
bit for bit.  The ucheck invariant of the reference (molsim.F90:1728-1745)
then holds on the GPU: UTotal after the moves equals UTotal before plus the
accepted du%tot.
"""
import numpy as np
import pytest

from molsim_gb300 import Engine, abi, configs
from tests.helpers import chain_trial, prepared, rel

pytestmark = pytest.mark.gpu

MC = abi.MG_MC
CASES = [
    ("spme_vlist", dict(seed=61)),
    ("spme_cell", dict(seed=62, txintlist=abi.MG_CELLLIST)),
    ("spme_order8_surf", dict(seed=63, nmesh=32, order=8, lsurf=1)),
    ("std_vlist_surf", dict(seed=64, ewald=abi.MG_EWALD_STD, ncut=5, lsurf=1)),
    ("std_cell", dict(seed=65, ewald=abi.MG_EWALD_STD, ncut=5, txintlist=abi.MG_CELLLIST)),
    ("no_ewald_cell", dict(seed=66, ewald=abi.MG_EWALD_NONE, txintlist=abi.MG_CELLLIST)),
    ("spme_bonds_vlist", dict(seed=67, chains=3, nseg=8)),
    ("spme_angles_cell", dict(seed=68, chains=4, nseg=8, angle_kt=0.6, txintlist=abi.MG_CELLLIST)),
    ("spme_n40_cell", dict(seed=69, nmesh=40, txintlist=abi.MG_CELLLIST)),
    ("spme_n30_order5", dict(seed=70, nmesh=30, order=5)),
]


def _pair(s, orc, form=abi.MG_FP64):
    ref = Engine(s, lib=orc, prefix="orc_")
    gpu = Engine(s, form=form)
    out = []
    for e in (ref, gpu):
        e.SetPositions(s.ro_flat())
        e.NList("write")
        out.append(e.UTotal())
    return ref, gpu, out[0], out[1]


def _trial(rng, s, ro, nptm, step):
    ips = rng.choice(s.np_, size=nptm, replace=False)
    L = s.boxlen[0]
    new = ro[ips] + rng.uniform(-step, step, (nptm, 3))
    new -= L * np.round(new / L)
    return ips + 1, new


@pytest.mark.parametrize("name,kw", CASES, ids=[c[0] for c in CASES])
def test_dutotal_and_accept_match_oracle(name, kw, orc, gpu_lib):
    s = prepared(configs.small_system(mode=MC, **kw), orc)
    ref, gpu, u_ref, u_gpu = _pair(s, orc)
    scale_tw = max(abs(u_ref["u_twob"][0]), 1.0)
    scale_rec = max(abs(u_ref["u_rec"]), 1.0)
    rng = np.random.default_rng(kw["seed"])
    ro = s.ro.copy()
    acc, nacc, novl = 0.0, 0, 0
    for it in range(40):
        nptm = 3 if it % 5 == 4 else 1
        ips, new = _trial(rng, s, ro, nptm, 2.5)
        r, ovl_r = ref.DUTotal(ips, new)
        g, ovl_g = gpu.DUTotal(ips, new)
        assert ovl_g == ovl_r, it
        if ovl_r:
            novl += 1
            continue
        for k in range(s.nptpt + 1):
            assert abs(g["du_twob"][k] - r["du_twob"][k]) <= 1e-10 * scale_tw, (it, k)
        assert abs(g["du_rec"] - r["du_rec"]) <= 1e-10 * scale_rec, it
        assert abs(g["du_tot"] - r["du_tot"]) <= 1e-10 * (scale_tw + scale_rec), it
        if rng.random() < 0.6:
            ref.MCUpdate()
            gpu.MCUpdate()
            ro[ips - 1] = new
            acc += g["du_tot"]
            nacc += 1
    assert nacc >= 10
    assert np.array_equal(gpu.GetPositions(), ref.GetPositions())
    # ucheck on the GPU: a fresh UTotal of the moved configuration
    u1 = gpu.UTotal()
    assert abs((u_gpu["u_tot"] + acc) - u1["u_tot"]) <= 1e-9 * (scale_tw + scale_rec)
    u1_ref = ref.UTotal()
    assert rel(u1["u_tot"], u1_ref["u_tot"]) <= 1e-10


@pytest.mark.parametrize("name,kw", [CASES[0], CASES[1], CASES[3], CASES[5]], ids=lambda x: str(x)[:12])
def test_batch_trials_match_single_oracle_trials(name, kw, orc, gpu_lib):
    s = prepared(configs.small_system(mode=MC, **kw), orc)
    ref, gpu, u_ref, _ = _pair(s, orc)
    scale = max(abs(u_ref["u_twob"][0]), 1.0) + max(abs(u_ref["u_rec"]), 1.0)
    rng = np.random.default_rng(kw["seed"] + 100)
    n = 64
    ips = rng.integers(s.np_, size=n) + 1
    L = s.boxlen[0]
    new = s.ro[ips - 1] + rng.uniform(-2.5, 2.5, (n, 3))
    new -= L * np.round(new / L)
    du, ovl = gpu.DUTotalBatch(ips, new)
    for t in range(n):
        r, o = ref.DUTotal([ips[t]], new[t:t + 1])
        assert bool(ovl[t]) == o, t
        if not o:
            assert abs(du[t] - r["du_tot"]) <= 1e-10 * scale, t
    assert ovl.sum() < n


def test_batch_leaves_state_unchanged(orc, gpu_lib):
    s = prepared(configs.small_system(mode=MC, seed=68), orc)
    _, gpu, _, u0 = _pair(s, orc)
    rng = np.random.default_rng(68)
    ips = rng.integers(s.np_, size=200) + 1
    new = s.ro[ips - 1] + rng.uniform(-1.0, 1.0, (200, 3))
    new -= s.boxlen[0] * np.round(new / s.boxlen[0])
    du1, o1 = gpu.DUTotalBatch(ips, new)
    du2, o2 = gpu.DUTotalBatch(ips, new)
    assert np.array_equal(du1, du2) and np.array_equal(o1, o2)
    assert np.array_equal(gpu.GetPositions(), s.ro)
    with pytest.raises(Exception):
        gpu.MCUpdate()            # a batch leaves no trial to accept


def test_mixed_form_trials_near_fp64(orc, gpu_lib):
    s = prepared(configs.small_system(mode=MC, seed=69), orc)
    g64 = Engine(s)
    gmx = Engine(s, form=abi.MG_MIXED)
    for e in (g64, gmx):
        e.SetPositions(s.ro_flat())
        e.NList("write")
        e.UTotal()
    rng = np.random.default_rng(69)
    ips = rng.integers(s.np_, size=128) + 1
    new = s.ro[ips - 1] + rng.uniform(-1.0, 1.0, (128, 3))
    new -= s.boxlen[0] * np.round(new / s.boxlen[0])
    d64, o64 = g64.DUTotalBatch(ips, new)
    dmx, omx = gmx.DUTotalBatch(ips, new)
    assert np.array_equal(o64, omx)
    ok = ~o64
    err = np.abs(dmx[ok] - d64[ok])
    assert np.sqrt((err ** 2).mean()) <= 1e-5 * np.sqrt((d64[ok] ** 2).mean())


@pytest.mark.parametrize("txintlist", [abi.MG_CELLLIST, abi.MG_VLIST], ids=["cell", "vlist"])
def test_chain_string_trials_match_oracle(txintlist, orc, gpu_lib):
    """DUBond and DUAngle (denergy.F90:2893-3077) on the GPU: single chain
    beads and strings of 2-4 consecutive beads of one chain, against the
    oracle trial by trial (du%tot within 1e-10 of the energy scale), then
    the same moves accepted on both and the GPU's ucheck."""
    chains, nseg = 4, 8
    s = prepared(configs.small_system(seed=69, mode=MC, chains=chains, nseg=nseg, angle_kt=0.6,
                                      txintlist=txintlist), orc)
    ref, gpu, u_ref, u_gpu = _pair(s, orc)
    t0 = ref.EnergyTerms()
    scale = abs(t0["u_twob0"]) + abs(t0["u_rec"]) + abs(t0["u_bond"]) + abs(t0["u_angle"]) + 1.0
    rng = np.random.default_rng(69)
    ro = s.ro.copy()
    acc, nacc, nstr = 0.0, 0, 0
    step = 1.0 if txintlist == abi.MG_CELLLIST else 0.15   # Verlet list: stay inside drnlist
    for it in range(30):
        ips, new = chain_trial(rng, s, ro, chains, nseg, step)
        r, ovl_r = ref.DUTotal(ips, new)
        g, ovl_g = gpu.DUTotal(ips, new)
        assert ovl_g == ovl_r, it
        if ovl_r:
            continue
        assert abs(g["du_tot"] - r["du_tot"]) <= 1e-10 * scale, (it, g["du_tot"], r["du_tot"])
        bonded_g = g["du_tot"] - g["du_twob"][0] - g["du_rec"]
        bonded_r = r["du_tot"] - r["du_twob"][0] - r["du_rec"]
        assert abs(bonded_g - bonded_r) <= 1e-10 * scale, it
        if it < 8 or rng.random() < 0.5:
            ref.MCUpdate()
            gpu.MCUpdate()
            ro[ips - 1] = new
            acc += g["du_tot"]
            nacc += 1
            nstr += len(ips) > 1
    assert nacc >= 8 and nstr >= 3
    assert np.array_equal(gpu.GetPositions(), ref.GetPositions())
    u1 = gpu.UTotal()
    assert abs((u_gpu["u_tot"] + acc) - u1["u_tot"]) <= 1e-9 * scale
    # batched single-bead trials on the chain beads
    n = 48
    ips = rng.integers(chains * nseg, size=n) + 1
    L = s.boxlen[0]
    new = ro[ips - 1] + rng.uniform(-step, step, (n, 3))
    new -= L * np.round(new / L)
    du, ovl = gpu.DUTotalBatch(ips, new)
    for t in range(n):
        r, o = ref.DUTotal([ips[t]], new[t:t + 1])
        assert bool(ovl[t]) == o, t
        if not o:
            assert abs(du[t] - r["du_tot"]) <= 1e-10 * scale, t


@pytest.mark.parametrize("mode", [1, 3])
def test_mc_passes_match_oracle(mode, orc, gpu_lib):
    """MC passes of single-particle, pivot and chain moves (molsim_gb300.mc,
    restating mc.F90's SPartMove, PivotMove and ChainMove) driven by the same
    Random stream through the oracle and through the GPU: the same trials
    are accepted, the positions agree bit for bit, and the accepted du%tot
    add up to the GPU's UTotal."""
    from molsim_gb300.mc import MCPass, MoveParams
    from tests.helpers import chain_system
    s = prepared(chain_system(seed=72, txintlist=abi.MG_CELLLIST), orc)
    ref, gpu, u_ref, u_gpu = _pair(s, orc)
    chain_p = MoveParams(pspart=0.3, dtran=1.0, ppivot=0.4, ipivotrotmode=mode, drotpivot=60.0,
                         pchain=0.3, dtranchain=1.0)
    ion_p = MoveParams(pspart=1.0, dtran=2.0)
    params = [ion_p, ion_p, ion_p, chain_p]
    runs = [MCPass(e, s, iseed=11, params=params, record=True) for e in (ref, gpu)]
    for mc in runs:
        for _ in range(2):
            mc.run_pass()
    a, b = runs
    assert a.stats.events == b.stats.events
    assert b.stats.accepted["pivot"] > 3 and b.stats.accepted["chain"] > 0
    assert np.array_equal(a.ro, b.ro)
    assert np.array_equal(gpu.GetPositions(), b.ro)
    scale = abs(u_ref["u_tot"]) + abs(u_ref["u_rec"]) + 1.0
    assert abs(a.du_acc - b.du_acc) <= 1e-9 * scale
    u1 = gpu.UTotal()
    assert abs((u_gpu["u_tot"] + b.du_acc) - u1["u_tot"]) <= 1e-9 * scale


@pytest.mark.parametrize("memb", ["ipt", "all"])
def test_cluster_passes_match_oracle(memb, orc, gpu_lib):
    """MC passes with the cluster move SPartCl2Move (mc.F90:1818-1945) beside
    single-particle moves, through the oracle and through the GPU with the
    same Random stream: the same clusters are tried and accepted or
    rejected, positions agree bit for bit, and the accepted du%tot add up to
    the GPU's UTotal."""
    from molsim_gb300.mc import MCPass, MoveParams
    from tests.helpers import chain_system
    s = prepared(chain_system(seed=73, txintlist=abi.MG_CELLLIST), orc)
    ref, gpu, u_ref, u_gpu = _pair(s, orc)
    ion_p = MoveParams(pspart=0.5, dtran=2.0, pspartcl2=0.5, txmembcl2=memb, radcl2=6.0, dtrancl2=3.0)
    chain_p = MoveParams(pspart=1.0, dtran=1.0)
    params = [ion_p, ion_p, ion_p, chain_p]
    runs = [MCPass(e, s, iseed=19, params=params, record=True) for e in (ref, gpu)]
    for mc in runs:
        for _ in range(2):
            mc.run_pass()
    a, b = runs
    assert a.stats.events == b.stats.events
    assert b.stats.accepted["cl2"] > 5
    assert np.array_equal(a.ro, b.ro)
    assert np.array_equal(gpu.GetPositions(), b.ro)
    scale = abs(u_ref["u_tot"]) + abs(u_ref["u_rec"]) + 1.0
    assert abs(a.du_acc - b.du_acc) <= 1e-9 * scale
    u1 = gpu.UTotal()
    assert abs((u_gpu["u_tot"] + b.du_acc) - u1["u_tot"]) <= 1e-9 * scale


def test_brush_passes_match_oracle(orc, gpu_lib):
    """MC passes with the brush cluster move BrushCl2Move (mc.F90:3028-3158):
    grafting particles, clustered within radcl2, move together with every
    chain grafted on them, beside single-particle moves of the ions, through
    the oracle and through the GPU with the same Random stream: the same
    moves are tried and accepted or rejected, positions agree bit for bit,
    and the accepted du%tot add up to the GPU's UTotal."""
    from molsim_gb300.mc import MCPass, MoveParams
    from tests.helpers import brush_system
    s = prepared(brush_system(txintlist=abi.MG_CELLLIST), orc)
    ref, gpu, u_ref, u_gpu = _pair(s, orc)
    ion_p = MoveParams(pspart=1.0, dtran=2.0)
    still = MoveParams(pspart=0.0)   # type 2 holds the chain beads: they move only with their brush
    graft_p = MoveParams(pspart=0.2, dtran=1.0, pbrushcl2=0.8, radcl2=14.0, dtranbrush=2.0)
    runs = [MCPass(e, s, iseed=23, params=[ion_p, still, ion_p, graft_p], record=True) for e in (ref, gpu)]
    for mc in runs:
        for _ in range(3):
            mc.run_pass()
    a, b = runs
    assert a.stats.events == b.stats.events
    assert b.stats.trials["brushcl2"] > 5 and b.stats.accepted["brushcl2"] > 0
    assert np.array_equal(a.ro, b.ro)
    assert np.array_equal(gpu.GetPositions(), b.ro)
    scale = abs(u_ref["u_tot"]) + abs(u_ref["u_rec"]) + 1.0
    assert abs(a.du_acc - b.du_acc) <= 1e-9 * scale
    u1 = gpu.UTotal()
    assert abs((u_gpu["u_tot"] + b.du_acc) - u1["u_tot"]) <= 1e-9 * scale


def test_brush_rotation_passes_match_oracle(orc, gpu_lib):
    """MC passes with BrushMove (mc.F90:2850-3019): a grafting particle and
    the chains grafted on it translated and rotated about the particle,
    through the oracle and through the GPU with the same Random stream: the
    same moves are accepted, positions agree bit for bit, and the accepted
    du%tot add up to the GPU's UTotal."""
    from molsim_gb300.mc import MCPass, MoveParams
    from tests.helpers import brush_system
    s = prepared(brush_system(txintlist=abi.MG_CELLLIST), orc)
    ref, gpu, u_ref, u_gpu = _pair(s, orc)
    ion_p = MoveParams(pspart=1.0, dtran=2.0)
    still = MoveParams(pspart=0.0)   # type 2 holds the chain beads: they move only with their brush
    graft_p = MoveParams(pspart=0.2, dtran=1.0, pbrush=0.8, dtranbrush=1.0, drotbrush=10.0)
    runs = [MCPass(e, s, iseed=31, params=[ion_p, still, ion_p, graft_p], record=True) for e in (ref, gpu)]
    for mc in runs:
        for _ in range(3):
            mc.run_pass()
    a, b = runs
    assert a.stats.events == b.stats.events
    assert b.stats.accepted["brush"] > 1
    assert np.array_equal(a.ro, b.ro)
    assert np.array_equal(gpu.GetPositions(), b.ro)
    scale = abs(u_ref["u_tot"]) + abs(u_ref["u_rec"]) + 1.0
    assert abs(a.du_acc - b.du_acc) <= 1e-9 * scale
    u1 = gpu.UTotal()
    assert abs((u_gpu["u_tot"] + b.du_acc) - u1["u_tot"]) <= 1e-9 * scale
