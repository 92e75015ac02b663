"""Known-answer tests that pin the CPU oracle.

The reference ships no golden numbers for this path, so the oracle is pinned
by answers that do not depend on it: math.erf, numpy's FFT, closed-form
B-splines, the NaCl Madelung constant, brute-force neighbour sets, finite
differences of its own energy, and the DUTotal/UTotal consistency that the
reference itself checks (molsim.F90:1728-1745).
"""
import ctypes as C
import math

import numpy as np
import pytest

from molsim_gb300 import Engine, abi, configs, units
from molsim_gb300.system import Species, System, iptpt_matrix
from tests.helpers import chain_trial

MADELUNG_NACL = 1.747564594633182


def test_erf2_matches_math_erf(orc):
    xs = np.linspace(-7.0, 7.0, 14001)
    err = max(abs(orc.orc_erf2(float(x)) - math.erf(x)) for x in xs)
    assert err < 2e-15


@pytest.mark.parametrize("n", [8, 16, 32])
def test_oracle_fft_matches_numpy(orc, n):
    rng = np.random.default_rng(n)
    q = rng.standard_normal(n ** 3)
    fq = np.zeros(2 * (n // 2 + 1) * n * n)
    assert orc.orc_fft_r2c_3d(n, abi.f64(q), abi.f64(fq)) == 0
    ref = np.fft.rfftn(q.reshape(n, n, n))            # [z][y][kx], kx fastest
    got = fq.view(np.complex128).reshape(n, n, n // 2 + 1)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    back = np.zeros(n ** 3)
    assert orc.orc_fft_c2r_3d(n, abi.f64(fq), abi.f64(back)) == 0
    assert np.abs(back / n ** 3 - q).max() < 1e-13       # unnormalised, as FFTW


@pytest.mark.parametrize("order", [4, 6, 8, 11])
def test_cardinal_bspline_partition_of_unity(orc, order):
    rng = np.random.default_rng(order)
    for pos in rng.uniform(0.0, 100.0, 50):
        kmax = C.c_int()
        v, d = np.zeros(order), np.zeros(order)
        assert orc.orc_cardinal_bspline(order, float(pos), C.byref(kmax), abi.f64(v), abi.f64(d)) == 0
        assert kmax.value == math.floor(pos)
        assert abs(v.sum() - 1.0) < 1e-14
        assert abs(d.sum()) < 1e-13
        assert (v >= 0).all()


def test_cardinal_bspline_order4_closed_form(orc):
    for u in (0.0, 0.1, 0.37, 0.5, 0.999):
        kmax = C.c_int()
        v, d = np.zeros(4), np.zeros(4)
        orc.orc_cardinal_bspline(4, 10.0 + u, C.byref(kmax), abi.f64(v), abi.f64(d))
        ref = [u ** 3 / 6, (-3 * u ** 3 + 3 * u ** 2 + 3 * u + 1) / 6, (3 * u ** 3 - 6 * u ** 2 + 4) / 6,
               (1 - u) ** 3 / 6]
        assert np.allclose(sorted(v), sorted(ref), rtol=0, atol=1e-15)


def test_gau_random_lcg_and_statistics(orc):
    # the LCG behind GauRandom: iseed <- (iseed * 16087) mod 2^31 (32-bit wrap)
    seed, flag, save = C.c_int32(12345), C.c_int32(1), C.c_double(0.0)
    x = [orc.orc_gau_random(C.byref(seed), C.byref(flag), C.byref(save)) for _ in range(200000)]
    x = np.array(x)
    assert abs(x.mean()) < 0.01 and abs(x.var() - 1.0) < 0.01
    # one GauRandom call from a fresh pair advances the LCG an even number
    # of times (one pair per polar-method trial)
    seed2, flag2 = C.c_int32(12345), C.c_int32(1)
    orc.orc_gau_random(C.byref(seed2), C.byref(flag2), C.byref(save))
    s, states = 12345, []
    for _ in range(40):
        s = (s * 16087) & 0x7FFFFFFF
        states.append(s)
    assert seed2.value in states[1::2]


def _rocksalt(ncell, r0):
    idx = np.arange(2 * ncell)
    g = np.stack(np.meshgrid(idx, idx, idx, indexing="ij"), -1).reshape(-1, 3)
    L = 2 * ncell * r0
    typ = np.where(g.sum(1) % 2 == 0, 1, 2).astype(np.int32)
    return g * r0 - L / 2 + 0.25 * r0, typ, L


@pytest.mark.parametrize("ewald", [abi.MG_EWALD_STD, abi.MG_EWALD_SPM])
def test_nacl_madelung_constant(orc, ewald):
    r0 = 2.8
    pos, typ, L = _rocksalt(3, r0)
    rcut = 0.999 * L / 2
    sp = [Species("Na", 1.0, 2.0, 0.0), Species("Cl", -1.0, 2.0, 0.0)]
    s = System(species=sp, iptpn=typ, ro=pos, boxlen=np.array([L, L, L]), relpermitt=1.0, rcut=rcut,
               ewald=ewald, ualpha=configs.alpha_for_erfc(1e-12, rcut), ncut=12, order=10, nmesh=64,
               utoltab=1e-9, ftoltab=1e-7)
    s.build_table(orc.orc_pot_twobody_tab)
    e = Engine(s, lib=orc, prefix="orc_")
    e.SetPositions(s.ro_flat())
    e.NList("write")
    r = e.UTotal()
    m = -r["u_tot"] * 2 * r0 / (len(typ) * s.epsi_four_pi)
    assert abs(m - MADELUNG_NACL) < 1e-6 * MADELUNG_NACL
    # perfect lattice: no net force (relative to one ion pair's force at r0)
    f_pair = units.FORCE_FAC * s.epsi_four_pi / r0 ** 2
    assert np.abs(r["forceo"]).max() < 1e-8 * f_pair


def test_table_accuracy_between_check_points(orc):
    s = configs.small_system(seed=5)
    s.build_table(orc.orc_pot_twobody_tab)
    pp, keep = s.pot_params()
    orc.orc_pot_1_6_12.argtypes = [C.POINTER(abi.MgPotParams), C.c_int, C.c_int, C.c_double,
                                   abi.PF64, abi.PF64, abi.PF64]
    orc.orc_pot_1_6_12.restype = None
    rng = np.random.default_rng(5)
    iptpt = iptpt_matrix(s.npt).reshape(s.npt, s.npt)
    u0, u1, u2 = (C.c_double() for _ in range(3))
    for it in range(1, s.npt + 1):
        for jt in range(it, s.npt + 1):
            pair = iptpt[jt - 1, it - 1]
            rmin = math.sqrt(s.r2umin[pair - 1]) * 1.05
            for r in rng.uniform(rmin, s.rcut, 300):
                ib = s.iubuflow[pair - 1] - 1
                while r * r < s.ubuf[ib]:
                    ib += 12
                d = r * r - s.ubuf[ib]
                c = s.ubuf[ib + 1: ib + 12]
                usum = c[0] + d * (c[1] + d * (c[2] + d * (c[3] + d * (c[4] + d * c[5]))))
                fsum = c[6] + d * (c[7] + d * (c[8] + d * (c[9] + d * c[10])))
                orc.orc_pot_1_6_12(C.byref(pp), it, jt, float(r), C.byref(u0), C.byref(u1), C.byref(u2))
                assert abs(usum - u0.value) <= 2 * s.utoltab
                assert abs(r * fsum + u1.value) <= 2 * s.ftoltab


def _brute_pairs(ro, L, rlist):
    d = ro[:, None, :] - ro[None, :, :]
    d -= L * np.round(d / L)
    r2 = (d * d).sum(-1)
    i, j = np.nonzero(np.triu(r2 <= rlist * rlist, 1))
    return set(zip(i.tolist(), j.tolist()))


@pytest.mark.parametrize("mode", [abi.MG_MD, abi.MG_MC])
def test_verlet_list_equals_brute_force(orc, mode):
    s = configs.small_system(seed=8, mode=mode)
    s.build_table(orc.orc_pot_twobody_tab)
    e = Engine(s, lib=orc, prefix="orc_")
    e.SetPositions(s.ro_flat())
    e.NList("write")
    nn, lists = e.VList()
    got = set()
    for i, js in enumerate(lists):
        for j in js:
            a, b = sorted((i, int(j) - 1))
            if mode == abi.MG_MD:
                assert (a, b) not in got       # half list: each pair once
            got.add((a, b))
    assert got == _brute_pairs(s.ro, s.boxlen[0], s.rcut + s.drnlist)


def test_cell_list_is_complete(orc):
    s = configs.small_system(seed=9, txintlist=abi.MG_CELLLIST)
    s.build_table(orc.orc_pot_twobody_tab)
    e = Engine(s, lib=orc, prefix="orc_")
    e.SetPositions(s.ro_flat())
    e.NList("write")
    assert orc.orc_celllist_test(e.h) == 0
    nc, cell = e.CellList()
    h = s.boxlen / nc
    idx = np.floor((s.ro + s.boxlen / 2) / h).astype(int)
    assert np.array_equal(cell, idx[:, 0] + idx[:, 1] * nc[0] + idx[:, 2] * nc[0] * nc[1])


@pytest.mark.parametrize("ewald", [abi.MG_EWALD_SPM, abi.MG_EWALD_STD])
def test_forces_are_minus_energy_gradient(orc, ewald):
    s = configs.small_system(seed=10, ewald=ewald, chains=2, nseg=6)
    s.utoltab, s.ftoltab = 1e-8, 1e-7
    s.build_table(orc.orc_pot_twobody_tab)
    e = Engine(s, lib=orc, prefix="orc_")
    ro = s.ro_flat().copy()
    e.SetPositions(ro)
    e.NList("write")
    f = e.UTotal()["forceo"].reshape(-1)
    h = 1e-4
    for k in (0, 4, 17, 3 * 11 + 2, 3 * (s.np_ - 1) + 1):
        up, dn = ro.copy(), ro.copy()
        up[k] += h
        dn[k] -= h
        e.SetPositions(up)
        e.NList("write")
        uu = e.UTotal()["u_tot"]
        e.SetPositions(dn)
        e.NList("write")
        ud = e.UTotal()["u_tot"]
        fd = -units.FORCE_FAC * (uu - ud) / (2 * h)
        assert abs(fd - f[k]) < 1e-5 * np.abs(f).max(), (k, fd, f[k])


@pytest.mark.parametrize("kw", [
    dict(ewald=abi.MG_EWALD_SPM),
    dict(ewald=abi.MG_EWALD_STD, ncut=5, lsurf=1),
    dict(ewald=abi.MG_EWALD_SPM, txintlist=abi.MG_CELLLIST),
    dict(ewald=abi.MG_EWALD_SPM, chains=4, nseg=8, angle_kt=0.5),
])
def test_dutotal_accumulates_to_utotal(orc, kw):
    """u%tot after n accepted moves equals u%tot before plus the sum of the
    accepted du%tot (the reference's ucheck, molsim.F90:1728-1745)."""
    s = configs.small_system(seed=12, mode=abi.MG_MC, **kw)
    s.build_table(orc.orc_pot_twobody_tab)
    e = Engine(s, lib=orc, prefix="orc_")
    e.SetPositions(s.ro_flat())
    e.NList("write")
    u0 = e.UTotal()["u_tot"]
    rng = np.random.default_rng(12)
    acc, nacc = 0.0, 0
    ro = s.ro.copy()
    L = s.boxlen[0]
    for _ in range(40):
        ip = int(rng.integers(s.np_))
        new = ro[ip] + rng.uniform(-1.0, 1.0, 3)
        new -= L * np.round(new / L)
        du, ovl = e.DUTotal([ip + 1], new.reshape(1, 3))
        if ovl:
            continue
        e.MCUpdate()
        ro[ip] = new
        acc += du["du_tot"]
        nacc += 1
    assert nacc > 20
    e2 = Engine(s, lib=orc, prefix="orc_")
    e2.SetPositions(ro.reshape(-1))
    e2.NList("write")
    u1 = e2.UTotal()["u_tot"]
    assert abs((u0 + acc) - u1) < 1e-9 * abs(u1)


def test_dutotal_bonded_terms_match_fresh_energies(orc):
    """DUBond and DUAngle (denergy.F90:2893-3077): for single beads and
    strings of beads of a chain, du%tot - du%twob(0) - du%rec equals the
    change of u%bond + u%angle evaluated from scratch (UBond, UAngle), and
    the accepted du%tot add up to the final UTotal (ucheck)."""
    chains, nseg = 4, 8
    # the linked cells stay exact however far the beads wander (a Verlet
    # list would need its displacement check)
    s = configs.small_system(seed=14, mode=abi.MG_MC, chains=chains, nseg=nseg, angle_kt=0.7,
                             txintlist=abi.MG_CELLLIST)
    s.build_table(orc.orc_pot_twobody_tab)

    def fresh(ro):
        e = Engine(s, lib=orc, prefix="orc_")
        e.SetPositions(ro.reshape(-1))
        e.NList("write")
        e.UTotal()
        return e.EnergyTerms()

    e = Engine(s, lib=orc, prefix="orc_")
    e.SetPositions(s.ro_flat())
    e.NList("write")
    u0 = e.UTotal()["u_tot"]
    t_old = fresh(s.ro)
    rng = np.random.default_rng(14)
    ro = s.ro.copy()
    acc, nacc, nstr = 0.0, 0, 0
    for it in range(40):
        ips, new = chain_trial(rng, s, ro, chains, nseg)
        du, ovl = e.DUTotal(ips, new)
        if ovl:
            continue
        ro_new = ro.copy()
        ro_new[ips - 1] = new
        t_new = fresh(ro_new)
        dub = du["du_tot"] - du["du_twob"][0] - du["du_rec"]
        ref = (t_new["u_bond"] + t_new["u_angle"]) - (t_old["u_bond"] + t_old["u_angle"])
        scale = abs(t_old["u_bond"]) + abs(t_old["u_angle"]) + abs(t_old["u_tot"])
        assert abs(dub - ref) <= 1e-10 * scale, (it, dub, ref)
        if rng.random() < 0.7:
            e.MCUpdate()
            ro, t_old = ro_new, t_new
            acc += du["du_tot"]
            nacc += 1
            nstr += len(ips) > 1
    assert nacc >= 15 and nstr >= 5
    u1 = fresh(ro)["u_tot"]
    assert abs((u0 + acc) - u1) < 1e-9 * abs(u1)
    t = e.EnergyTerms()
    assert abs(t["u_bond"] - fresh(ro)["u_bond"]) < 1e-9 * abs(u1)


def test_angle_forces_are_minus_energy_gradient(orc):
    """UAngle (energy.F90:5409-5506): forces on the three beads of every angle
    against central differences of the oracle's energy; u%angle in the total."""
    s = configs.small_system(seed=41, ewald=abi.MG_EWALD_NONE, chains=3, nseg=8, angle_kt=0.8, eps_kt=0.0)
    s.utoltab, s.ftoltab = 1e-8, 1e-7
    s.build_table(orc.orc_pot_twobody_tab)
    e = Engine(s, lib=orc, prefix="orc_")
    ro = s.ro_flat().copy()
    e.SetPositions(ro)
    e.NList("write")
    r = e.UTotal()
    t = e.EnergyTerms()
    assert t["u_angle"] > 0
    assert abs(t["u_tot"] - (t["u_twob0"] + t["u_rec"] + t["u_bond"] + t["u_angle"])) <= 1e-12 * abs(t["u_tot"])
    f = r["forceo"].reshape(-1)
    h = 1e-5
    for k in (0, 5, 3 * 3 + 1, 3 * 7 + 2, 3 * 12):   # chain beads (ends and interior)
        up, dn = ro.copy(), ro.copy()
        up[k] += h
        dn[k] -= h
        e.SetPositions(up)
        e.NList("write")
        uu = e.UTotal()["u_tot"]
        e.SetPositions(dn)
        e.NList("write")
        ud = e.UTotal()["u_tot"]
        fd = -units.FORCE_FAC * (uu - ud) / (2 * h)
        assert abs(fd - f[k]) < 1e-6 * np.abs(f).max(), (k, fd, f[k])
    e.close()
