"""UTwoBodyP on the GPU (mg_poly_utwobody) against the oracle.

Rigid three-site waters and one-atom ions: u%twob per particle-type pair and
the virial within 1e-10 relative, atom forces within 1e-10 of the largest
(the GPU adds the neighbours' atom forces as 64-bit fixed-point integers,
the same bits on every call), for the MD half list and the MC full list; an
atom pair below its table reports MG_ERR_TABLE_UNDERRUN as the reference's
Stop does.
"""
import numpy as np
import pytest

from molsim_gb300 import abi, configs
from molsim_gb300.engine import MolsimError
from molsim_gb300.poly import PolyEngine
from tests.helpers import centre_lists
from tests.test_cpu_poly import oracle_poly

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("full", [False, True], ids=["half", "mc_full"])
@pytest.mark.parametrize("seed,nw,ns,L", [(9, 120, 10, 18.0), (10, 400, 30, 30.0)])
def test_poly_utwobody_matches_oracle(seed, nw, ns, L, full, orc, gpu_lib):
    s = configs.water_ions(seed=seed, nwater=nw, nsalt=ns, L=L)
    s.build_table(orc.orc_pot_twobody_tab)
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 1.0, full=full)
    s.lmc = 1 if full else 0
    ref = oracle_poly(orc, s, nn, jl, maxn, lmc=s.lmc)
    e = PolyEngine(s, maxn)
    g = e.UTwoBodyP(nn, jl)
    for k in range(len(ref["u_twob"])):
        assert abs(g["u_twob"][k] - ref["u_twob"][k]) <= 1e-10 * abs(ref["u_twob"][0]), k
    assert abs(g["virial"] - ref["virial"]) <= 1e-10 * abs(ref["virial"])
    assert np.abs(g["force"] - ref["force"]).max() <= 1e-10 * np.abs(ref["force"]).max()
    g2 = e.UTwoBodyP(nn, jl)   # integer sums: the same bits on every call
    assert np.array_equal(g["force"], g2["force"]) and g["virial"] == g2["virial"]
    assert np.array_equal(g["u_twob"], g2["u_twob"])
    e.close()


def test_poly_underrun_is_reported(orc, gpu_lib):
    s = configs.water_ions(seed=11, nwater=60, nsalt=4, L=14.0)
    s.build_table(orc.orc_pot_twobody_tab)
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 1.0)
    r = s.atom_positions()
    # put an atom of particle 2 onto an atom of particle 1 (r2 below every table)
    j = int(jl[0, 0])   # a neighbour of particle 1
    ia, ja = 0, int(s.ianpn()[j - 1]) - 1
    r[ja] = r[ia] + 1e-3
    e = PolyEngine(s, maxn)
    with pytest.raises(MolsimError) as ex:
        e.UTwoBodyP(nn, jl, r=r)
    assert abi.STATUS[ex.value.status] == "MG_ERR_TABLE_UNDERRUN"
    e.close()


@pytest.mark.parametrize("ewald", ["spm", "std"])
def test_poly_utotal_with_ewald_matches_oracle(ewald, orc, gpu_lib):
    """UTwoBodyP with the real-space Ewald table, the reciprocal sum and self
    term over the atoms, and the molecular self term: the GPU against the
    oracle, u%tot and u%rec within 1e-10, atom forces within 1e-10 of the
    largest."""
    from tests.test_cpu_poly import oracle_poly_utotal
    s = configs.water_ions(seed=12, nwater=150, nsalt=10, L=20.0)
    s.relpermitt = 78.0
    if ewald == "spm":
        s.ewald, s.ualpha, s.order, s.nmesh = abi.MG_EWALD_SPM, 0.4, 6, 32
    else:
        s.ewald, s.ualpha, s.ncut = abi.MG_EWALD_STD, 0.4, 10
    s.build_table(orc.orc_pot_twobody_tab)
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 1.0)
    ref = oracle_poly_utotal(orc, s, nn, jl, maxn)
    e = PolyEngine(s, maxn)
    g = e.UTotal(nn, jl)
    scale = abs(ref["parts"][0]) + abs(ref["parts"][1]) + abs(ref["parts"][2])
    assert abs(g["u_tot"] - ref["u_tot"]) <= 1e-10 * scale
    assert abs(g["u_rec"] - ref["u_rec"]) <= 1e-10 * scale
    assert np.abs(g["force"] - ref["force"]).max() <= 1e-10 * np.abs(ref["force"]).max()
    e.close()


def test_poly_trial_batch_matches_oracle(orc, gpu_lib):
    """Independent single-particle trials of rigid waters and ions in one
    launch: the same overlap flags as the oracle's UTwoBodyPNew/Old, and
    du%twob within 1e-10 of the two-body energy."""
    from tests.test_cpu_poly import oracle_trial, poly_trials
    s = configs.water_ions(seed=13, nwater=200, nsalt=12, L=22.0)
    s.lmc = 1
    s.build_table(orc.orc_pot_twobody_tab)
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 2.0, full=True)
    ref_u0 = oracle_poly(orc, s, nn, jl, maxn, lmc=1)["u_twob"][0]
    rng = np.random.default_rng(5)
    ips, rotm, atoms = poly_trials(s, rng, 96, step=1.2, angle=0.8)
    e = PolyEngine(s, maxn)
    du, ovl = e.DUTwoBodyBatch(nn, jl, ips, rotm, np.concatenate(atoms))
    n_ok = 0
    for t in range(len(ips)):
        r_du, r_ovl = oracle_trial(orc, s, nn, jl, maxn, ips[t], rotm[t], atoms[t])
        assert bool(ovl[t]) == r_ovl, t
        if not r_ovl:
            assert abs(du[t] - r_du[0]) <= 1e-10 * abs(ref_u0), (t, du[t], r_du[0])
            n_ok += 1
    assert n_ok > 60
    e.close()


def test_poly_epilogue_matches_oracle(orc, gpu_lib):
    """UTotal's end for polyatomic particles: particle forces and torques
    from the atom forces, summed atom by atom in order per particle as the
    reference does (the same bits), and the molecular virial."""
    import ctypes as C
    from molsim_gb300 import units
    s = configs.water_ions(seed=14, nwater=150, nsalt=10, L=20.0)
    s.build_table(orc.orc_pot_twobody_tab)
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 1.0)
    e = PolyEngine(s, maxn)
    g = e.UTotal(nn, jl)
    p = s.params()
    r = s.atom_positions()
    fo, to, vm = np.zeros(3 * s.np_), np.zeros(3 * s.np_), np.zeros(1)
    assert orc.orc_poly_epilogue(C.byref(p), abi.f64(abi.as_f64(s.ro.reshape(-1))), abi.f64(r.reshape(-1)),
                                 abi.f64(np.ascontiguousarray(g["force"].reshape(-1))), None, units.FORCE_FAC,
                                 abi.f64(fo), abi.f64(to), abi.f64(vm)) == 0
    assert np.array_equal(g["forceo"].reshape(-1), fo)
    assert np.array_equal(g["torqueo"].reshape(-1), to)
    assert abs((g["virial"] - e.UTwoBodyP(nn, jl)["virial"]) - vm[0]) <= 1e-10 * abs(vm[0])
    # the particle forces add up to the atom forces
    assert np.allclose(g["forceo"].sum(0), g["force"].sum(0) * units.FORCE_FAC, rtol=0,
                       atol=1e-9 * np.abs(g["forceo"]).max())
    e.close()


@pytest.mark.parametrize("ewald", [False, True])
def test_poly_device_list_matches_host_list(ewald, orc, gpu_lib):
    """The atom-pair loop over the device-resident list of a centres handle
    (full list, every thread its own atoms' forces) against the oracle with
    the host list: energies and virial within 1e-10, atom forces within 1e-10
    of the largest."""
    s = configs.water_ions(seed=15, nwater=200, nsalt=12, L=22.0)
    if ewald:
        s.relpermitt = 78.0
        s.ewald, s.ualpha, s.order, s.nmesh = abi.MG_EWALD_SPM, 0.4, 6, 32
    s.build_table(orc.orc_pot_twobody_tab)
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 1.0)
    ref = oracle_poly(orc, s, nn, jl, maxn)
    e = PolyEngine(s, maxn)
    g = e.UTwoBodyPList()
    for k in range(len(ref["u_twob"])):
        assert abs(g["u_twob"][k] - ref["u_twob"][k]) <= 1e-10 * abs(ref["u_twob"][0]), k
    assert abs(g["virial"] - ref["virial"]) <= 1e-10 * abs(ref["virial"])
    assert np.abs(g["force"] - ref["force"]).max() <= 1e-10 * np.abs(ref["force"]).max()
    g2 = e.UTwoBodyPList()                     # reproducible: no atomics
    assert np.array_equal(g["force"], g2["force"])
    a, b = e.UTotal(nn, jl), e.UTotal()
    assert abs(a["u_tot"] - b["u_tot"]) <= 1e-10 * abs(a["u_tot"])
    e.close()


def test_poly_device_list_needs_the_pair_cutoff(orc, gpu_lib):
    """A centres handle whose rcut is below the pair cutoff is refused even
    when rcut + drnlist reaches it: after mg_nlist_update its list holds only
    the pairs within its rcut.  A handle whose list build failed has no list."""
    from molsim_gb300 import Engine
    s = configs.water_ions(seed=16, nwater=120, nsalt=8, L=20.0)
    s.build_table(orc.orc_pot_twobody_tab)
    e = PolyEngine(s, 64)
    c = s.centre_system(skin=2.0)
    c.rcut = s.rcut - 1.0                     # rcut + skin > pair cutoff > rcut
    short = Engine(c)
    short.SetPositions(abi.as_f64(s.ro.reshape(-1)))
    short.NList("write")
    r = s.atom_positions()
    force = np.zeros(3 * len(r))
    ut = np.zeros(e.p.nptpt + 1)
    vir = np.zeros(1)
    st = gpu_lib.mg_poly_utwobody_list(e.h, short.h, abi.f64(r.reshape(-1)), abi.f64(force), abi.f64(ut),
                                       abi.f64(vir))
    assert abi.STATUS[st] == "MG_ERR_ARG"
    # a list that overflows its capacity is dropped, and the poly call refuses it
    c2 = s.centre_system(skin=1.0)
    c2.maxnneigh = 1
    tiny = Engine(c2)
    tiny.SetPositions(abi.as_f64(s.ro.reshape(-1)))
    with pytest.raises(MolsimError):
        tiny.NList("write")
    st = gpu_lib.mg_poly_utwobody_list(e.h, tiny.h, abi.f64(r.reshape(-1)), abi.f64(force), abi.f64(ut),
                                       abi.f64(vir))
    assert abi.STATUS[st] == "MG_ERR_STATE"
    for x in (short, tiny, e):
        x.close()


@pytest.mark.parametrize("nptm", [1, 2, 3, 6])
def test_poly_multi_trial_matches_oracle(nptm, orc, gpu_lib):
    """Trials moving nptm neighbouring waters and ions together (one block
    per trial): the oracle's overlap flag, and du%twob per particle-type pair
    within 1e-10 of the two-body energy; nptm = 1 also gives the single-trial
    kernel's du%twob."""
    from tests.test_cpu_poly import multi_trial, oracle_multi
    s = configs.water_ions(seed=16, nwater=200, nsalt=12, L=22.0)
    s.lmc = 1
    s.build_table(orc.orc_pot_twobody_tab)
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 2.0, full=True)
    u0 = abs(oracle_poly(orc, s, nn, jl, maxn, lmc=1)["u_twob"][0])
    rng = np.random.default_rng(70 + nptm)
    e = PolyEngine(s, maxn)
    n_ok = 0
    for _ in range(24):
        ips, rotm, atoms = multi_trial(s, rng, nn, jl, nptm, step=0.5, angle=0.5)
        r_du, r_ovl = oracle_multi(orc, s, nn, jl, maxn, ips, rotm, atoms)
        du, ovl = e.DUTwoBodyMulti(nn, jl, ips, rotm, atoms)
        assert ovl == r_ovl
        if r_ovl:
            continue
        assert np.abs(du - r_du).max() <= 1e-10 * u0, (ips, du, r_du)
        if nptm == 1:
            db, ob = e.DUTwoBodyBatch(nn, jl, ips, rotm, atoms)
            assert not ob[0] and abs(db[0] - du[0]) <= 1e-10 * u0
        n_ok += 1
    assert n_ok >= 12
    e.close()


def test_poly_multi_trial_refuses_a_repeated_particle(orc, gpu_lib):
    s = configs.water_ions(seed=17, nwater=60, nsalt=4, L=14.0)
    s.lmc = 1
    s.build_table(orc.orc_pot_twobody_tab)
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 2.0, full=True)
    e = PolyEngine(s, maxn)
    a = s.atom_positions()[:3]
    with pytest.raises(MolsimError) as ex:
        e.DUTwoBodyMulti(nn, jl, [1, 1], np.vstack([s.ro[0], s.ro[0]]), np.vstack([a, a]))
    assert abi.STATUS[ex.value.status] == "MG_ERR_ARG"
    e.close()
