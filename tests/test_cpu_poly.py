"""UTwoBodyP (energy.F90:786-896) in the oracle: atom forces are minus the
gradient of its energy, the MC full list gives the half list's sums, and
the atom-pair table is the library's (bit for bit)."""
import ctypes as C

import numpy as np
import pytest

from molsim_gb300 import abi, configs
from tests.helpers import centre_lists


def oracle_poly(orc, s, nn, jl, maxn, r=None, lmc=0):
    s.lmc = lmc
    p = s.params()
    r = s.atom_positions() if r is None else r
    force = np.zeros(r.size)
    ut = np.zeros(p.nptpt + 1)
    vir = np.zeros(1)
    st = orc.orc_poly_utwobody(C.byref(p), maxn, abi.f64(abi.as_f64(s.ro.reshape(-1))),
                               abi.f64(np.ascontiguousarray(r.reshape(-1))), abi.i32(abi.as_i32(nn)),
                               abi.i32(abi.as_i32(jl.reshape(-1))), abi.f64(force), abi.f64(ut), abi.f64(vir))
    assert st == 0, abi.STATUS.get(st, st)
    return dict(force=force.reshape(-1, 3), u_twob=ut, virial=vir[0])


@pytest.fixture(scope="module")
def lib():
    """The library's host-side table builder (no GPU needed)."""
    import molsim_gb300
    molsim_gb300.build()
    return abi.load_library()


@pytest.fixture(scope="module")
def water(orc):
    s = configs.water_ions(seed=9, nwater=120, nsalt=10, L=18.0)
    s.build_table(orc.orc_pot_twobody_tab)
    return s


def test_atom_forces_are_minus_the_energy_gradient(water, orc):
    s = water
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 1.0)
    r = s.atom_positions()
    out = oracle_poly(orc, s, nn, jl, maxn, r)
    f = out["force"]
    rng = np.random.default_rng(1)
    h = 1e-5
    for ia in rng.choice(len(r), 12, replace=False):
        for m in range(3):
            up, dn = r.copy(), r.copy()
            up[ia, m] += h
            dn[ia, m] -= h
            uu = oracle_poly(orc, s, nn, jl, maxn, up)["u_twob"][0]
            ud = oracle_poly(orc, s, nn, jl, maxn, dn)["u_twob"][0]
            fd = -(uu - ud) / (2 * h)
            assert abs(fd - f[ia, m]) < 2e-4 * np.abs(f).max(), (ia, m, fd, f[ia, m])


def test_full_list_with_lmc_gives_the_half_list_sums(water, orc):
    s = water
    a = oracle_poly(orc, s, *centre_lists(s.ro, s.boxlen[0], s.rcut + 1.0), lmc=0)
    b = oracle_poly(orc, s, *centre_lists(s.ro, s.boxlen[0], s.rcut + 1.0, full=True), lmc=1)
    assert np.allclose(a["u_twob"], b["u_twob"], rtol=1e-12, atol=0)
    assert np.allclose(a["force"], b["force"], rtol=0, atol=1e-10 * np.abs(a["force"]).max())
    assert abs(a["virial"] - b["virial"]) <= 1e-12 * abs(a["virial"])
    # u%twob(0) is the sum of the type-pair energies; water-water dominates
    assert abs(a["u_twob"][0] - a["u_twob"][1:].sum()) <= 1e-12 * abs(a["u_twob"][0])


def test_atom_table_is_the_library_table(water, lib, orc):
    from molsim_gb300.configs import water_ions
    t = water_ions(seed=9, nwater=120, nsalt=10, L=18.0)
    t.build_table(lib.mg_pot_twobody_tab)
    assert np.array_equal(t.ubuf, water.ubuf) and np.array_equal(t.iubuflow, water.iubuflow)


def oracle_poly_utotal(orc, s, nn, jl, maxn):
    """The polyatomic UTotal with Ewald on the oracle: UTwoBodyP with the
    real-space table, the atoms' reciprocal sum and self term (a handle of
    the atoms with a zero pair table), the molecular self term."""
    from molsim_gb300 import Engine, units
    p = s.params()
    r = s.atom_positions()
    tw = oracle_poly(orc, s, nn, jl, maxn, r, lmc=s.lmc)
    a = s.atom_system()
    e = Engine(a, lib=orc, prefix="orc_")
    e.SetPositions(s.atoms_in_box(r).reshape(-1))
    e.NList("write")
    rec = e.UTotal()
    fi = np.zeros(r.size)
    ui = np.zeros(1)
    assert orc.orc_poly_ewald_intra(C.byref(p), abi.f64(np.ascontiguousarray(r.reshape(-1))), abi.f64(fi),
                                    abi.f64(ui)) == 0
    force = tw["force"] + rec["forceo"] / units.FORCE_FAC + fi.reshape(-1, 3)
    u_rec = rec["u_rec"] + ui[0]
    return dict(u_twob=tw["u_twob"], u_rec=u_rec, u_tot=tw["u_twob"][0] + u_rec, force=force,
                parts=(tw["u_twob"][0], rec["u_rec"], ui[0]))


def test_ewald_splitting_does_not_change_the_energy(orc):
    """With the molecular self term, the total energy does not depend on the
    Ewald split: alpha 0.45 and 0.55 agree to the table tolerance while the
    reciprocal and molecular terms each change by about a hundred kJ/mol."""
    tot, parts = [], []
    for alpha, ncut in ((0.45, 14), (0.55, 18)):
        s = configs.water_ions(seed=9, nwater=120, nsalt=10, L=18.0)
        s.ewald, s.ualpha, s.ncut, s.relpermitt = abi.MG_EWALD_STD, alpha, ncut, 78.0
        s.build_table(orc.orc_pot_twobody_tab)
        out = oracle_poly_utotal(orc, s, *centre_lists(s.ro, s.boxlen[0], s.rcut + 1.0))
        tot.append(out["u_tot"])
        parts.append(out["parts"])
    scale = abs(parts[0][1]) + abs(parts[0][2])
    assert abs(parts[0][2] - parts[1][2]) > 50.0        # the split moves energy between the terms
    assert abs(tot[0] - tot[1]) <= 1e-4 * scale, (tot, parts)


def poly_trials(s, rng, n, step=0.8, angle=0.4):
    """n single-particle trials: a random particle displaced by up to step
    and turned by up to angle radians about a random axis; returns ips
    (1-based), trial centres, the trials' atoms, and per trial its atoms."""
    from molsim_gb300.mc import axis_angle_matrix
    L = s.boxlen[0]
    ips = rng.integers(s.np_, size=n) + 1
    rotm = np.empty((n, 3))
    atoms = []
    for t, ip in enumerate(ips):
        c = s.ro[ip - 1] + rng.uniform(-step, step, 3)
        c -= L * np.round(c / L)
        rotm[t] = c
        R = axis_angle_matrix(rng.normal(size=3), rng.uniform(-angle, angle)) @ s.ori[ip - 1]
        loc = np.array([x for _, x in s.particle_types[s.iptpn[ip - 1] - 1].atoms])
        atoms.append(c + loc @ R.T)
    return ips, rotm, atoms


def oracle_trial(orc, s, nn, jl, maxn, ip, c, atoms):
    p = s.params()
    du = np.zeros(p.nptpt + 1)
    ovl = np.zeros(1, dtype=np.int32)
    st = orc.orc_poly_dutwobody(C.byref(p), maxn, abi.f64(abi.as_f64(s.ro.reshape(-1))),
                                abi.f64(np.ascontiguousarray(s.atom_positions().reshape(-1))),
                                abi.i32(abi.as_i32(nn)), abi.i32(abi.as_i32(jl.reshape(-1))), int(ip),
                                abi.f64(abi.as_f64(c)), abi.f64(np.ascontiguousarray(atoms.reshape(-1))),
                                abi.f64(du), abi.i32(ovl))
    assert st == 0, abi.STATUS.get(st, st)
    return du, bool(ovl[0])


def test_trial_differences_match_full_energies(water, orc):
    """du%twob of a trial (UTwoBodyPNew minus UTwoBodyPOld) equals UTwoBodyP
    of the moved configuration minus that of the current one."""
    s = water
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 2.0, full=True)
    hn, hl, hmax = centre_lists(s.ro, s.boxlen[0], s.rcut + 2.0)
    u0 = oracle_poly(orc, s, hn, hl, hmax)["u_twob"][0]
    rng = np.random.default_rng(4)
    ips, rotm, atoms = poly_trials(s, rng, 12)
    nchecked = 0
    for ip, c, a in zip(ips, rotm, atoms):
        du, ovl = oracle_trial(orc, s, nn, jl, maxn, ip, c, a)
        if ovl:
            continue
        r = s.atom_positions()
        a0 = int(s.ianpn()[ip - 1]) - 1
        r[a0:a0 + len(a)] = a
        ro = s.ro.copy()
        ro[ip - 1] = c
        keep = s.ro
        s.ro = ro
        try:
            u1 = oracle_poly(orc, s, hn, hl, hmax, r)["u_twob"][0]
        finally:
            s.ro = keep
        assert abs(du[0] - (u1 - u0)) <= 1e-9 * abs(u0), (ip, du[0], u1 - u0)
        nchecked += 1
    assert nchecked >= 8


def multi_trial(s, rng, nn, jl, nptm, step=0.6, angle=0.4):
    """One trial moving nptm particles together: a random particle and up to
    nptm - 1 of its list neighbours, each displaced by up to step and turned
    by up to angle radians.  Returns ips (1-based), centres, atoms."""
    from molsim_gb300.mc import axis_angle_matrix
    L = s.boxlen[0]
    ip = int(rng.integers(s.np_)) + 1
    neigh = [int(j) for j in jl[ip - 1, :nn[ip - 1]]]
    rng.shuffle(neigh)
    ips = np.array([ip] + neigh[:nptm - 1], dtype=np.int32)
    rotm = np.empty((len(ips), 3))
    atoms = []
    for t, jp in enumerate(ips):
        c = s.ro[jp - 1] + rng.uniform(-step, step, 3)
        c -= L * np.round(c / L)
        rotm[t] = c
        R = axis_angle_matrix(rng.normal(size=3), rng.uniform(-angle, angle)) @ s.ori[jp - 1]
        loc = np.array([x for _, x in s.particle_types[s.iptpn[jp - 1] - 1].atoms])
        atoms.append(c + loc @ R.T)
    return ips, rotm, np.concatenate(atoms)


def oracle_multi(orc, s, nn, jl, maxn, ips, rotm, atoms):
    p = s.params()
    du = np.zeros(p.nptpt + 1)
    ovl = np.zeros(1, dtype=np.int32)
    st = orc.orc_poly_dutwobody_multi(C.byref(p), maxn, abi.f64(abi.as_f64(s.ro.reshape(-1))),
                                      abi.f64(np.ascontiguousarray(s.atom_positions().reshape(-1))),
                                      abi.i32(abi.as_i32(nn)), abi.i32(abi.as_i32(jl.reshape(-1))), len(ips),
                                      abi.i32(abi.as_i32(ips)), abi.f64(abi.as_f64(rotm.reshape(-1))),
                                      abi.f64(abi.as_f64(atoms.reshape(-1))), abi.f64(du), abi.i32(ovl))
    assert st == 0, abi.STATUS.get(st, st)
    return du, bool(ovl[0])


def test_multi_trial_of_one_particle_is_the_single_trial(water, orc):
    s = water
    s.lmc = 1
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 2.0, full=True)
    rng = np.random.default_rng(6)
    ips, rotm, atoms = poly_trials(s, rng, 16)
    for ip, c, a in zip(ips, rotm, atoms):
        d1, o1 = oracle_trial(orc, s, nn, jl, maxn, ip, c, a)
        dm, om = oracle_multi(orc, s, nn, jl, maxn, np.array([ip]), c.reshape(1, 3), a)
        assert o1 == om
        if not o1:
            assert np.abs(dm - d1).max() <= 1e-12 * np.abs(d1).max() + 1e-12


@pytest.mark.parametrize("nptm", [2, 3, 5])
def test_multi_trial_is_the_full_energy_difference(nptm, water, orc):
    """du%twob per particle-type pair of a trial moving nptm neighbouring
    particles (the moving pairs counted once, at their new separations) is
    UTwoBodyP of the moved configuration minus that of the current one."""
    s = water
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 2.0, full=True)
    hn, hl, hmax = centre_lists(s.ro, s.boxlen[0], s.rcut + 2.0)
    u0 = oracle_poly(orc, s, hn, hl, hmax)["u_twob"]
    s.lmc = 1
    rng = np.random.default_rng(40 + nptm)
    nchecked = 0
    for _ in range(10):
        ips, rotm, atoms = multi_trial(s, rng, nn, jl, nptm)
        du, ovl = oracle_multi(orc, s, nn, jl, maxn, ips, rotm, atoms)
        if ovl:
            continue
        r = s.atom_positions()
        ro = s.ro.copy()
        k = 0
        for t, ip in enumerate(ips):
            a0 = int(s.ianpn()[ip - 1]) - 1
            na = len(s.particle_types[s.iptpn[ip - 1] - 1].atoms)
            r[a0:a0 + na] = atoms[k:k + na]
            k += na
            ro[ip - 1] = rotm[t]
        keep = s.ro
        s.ro = ro
        try:
            u1 = oracle_poly(orc, s, hn, hl, hmax, r)["u_twob"]
        finally:
            s.ro = keep
        assert np.abs(du - (u1 - u0)).max() <= 1e-9 * abs(u0[0]), (ips, du, u1 - u0)
        nchecked += 1
    s.lmc = 0
    assert nchecked >= 5
