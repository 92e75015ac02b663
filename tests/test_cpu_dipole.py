"""Charges and point dipoles with Ewald (UDipole, energy.F90:1476-2295) on
the oracle, pinned without it.

The reference's tests hold no expected numbers for dipoles, so the oracle's
u%stat is checked against an Ewald sum of point charges written in numpy
(tests/test_cpu_ewald_known.py): every point dipole becomes a pair of
charges +-|dip|/d at +-d/2 along it, beside its atom's charge, the
intramolecular Coulomb pairs are taken out (the reference excludes them),
and Richardson's extrapolation of d = 0.04 and 0.02 A removes the O(d^2)
error (what remains, a few 1e-8 of u%stat, is the rounding of the large
dumbbell charges).  The oracle's own derivatives must then hold: dU/d(dip_a) =
-EpsiFourPi e_a, the atom forces are -dU/dr_a at fixed dipoles, the
torques dip x e.  SPME (order 8) agrees with standard Ewald.
"""
import ctypes as C

import numpy as np
import pytest

from molsim_gb300 import Engine, abi, units
from molsim_gb300.poly import AtomType, ParticleType, PolySystem
from tests.helpers import centre_lists

pytest.importorskip("scipy.special")
from tests.test_cpu_ewald_known import ewald_exact   # noqa: E402


def _rot(rng):
    q, r = np.linalg.qr(rng.standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def dipole_system(ewald=abi.MG_EWALD_STD, lsurf=0, seed=3, L=9.0, n=3, alpha=1.4, ncut=20, order=8, nmesh=64):
    """n two-atom neutral particles with charges and dipoles in a cubic box;
    no LJ."""
    rng = np.random.default_rng(seed)
    at = [AtomType("A", 0.6, 0.0, 0.0, 10.0), AtomType("B", -0.6, 0.0, 0.0, 12.0)]
    pt = ParticleType("ab", [(0, (0.0, 0.0, -0.5)), (1, (0.0, 0.0, 0.5))],
                      dipoles=[(0.25, 0.0, 0.3), (0.0, -0.3, 0.1)])
    ro = []
    while len(ro) < n:
        x = rng.uniform(-L / 2, L / 2, 3)
        if all(np.linalg.norm((x - y) - L * np.round((x - y) / L)) > 2.5 for y in ro):
            ro.append(x)
    s = PolySystem(atom_types=at, particle_types=[pt], iptpn=np.ones(n, dtype=np.int32), ro=np.array(ro),
                   ori=np.array([_rot(rng) for _ in range(n)]), boxlen=np.array([L, L, L]), rcut=L / 2 - 0.05,
                   relpermitt=1.0, txelec="dip", lsurf=lsurf, ewald=ewald, ualpha=alpha, ncut=ncut, order=order,
                   nmesh=nmesh, r2uminin=1e-4)
    return s


def oracle_udipole(orc, s, dip=None, r=None):
    """UDipole on the oracle: u_stat, u_real, potstat, estat, efg, atom
    forces and torques, virelec."""
    p = s.params()
    r = s.atom_positions() if r is None else np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
    dip = s.atom_dipoles() if dip is None else np.ascontiguousarray(dip, dtype=np.float64).reshape(-1, 3)
    na = len(r)
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 0.5)
    pot, est, efg = np.zeros(na), np.zeros(3 * na), np.zeros(6 * na)
    vir, ureal = np.zeros(1), np.zeros(1)
    ro = abi.as_f64(np.asarray(s.ro).reshape(-1))
    assert orc.orc_poly_udipole_real(C.byref(p), maxn, abi.f64(ro), abi.f64(r.reshape(-1)), abi.f64(dip.reshape(-1)),
                                     abi.i32(nn), abi.i32(jl.reshape(-1)), abi.f64(pot), abi.f64(est),
                                     abi.f64(efg), abi.f64(vir), abi.f64(ureal)) == 0
    if s.ewald != abi.MG_EWALD_NONE:
        e = Engine(s.atom_system(), lib=orc, prefix="orc_")
        e.SetPositions(s.atoms_in_box(r).reshape(-1))
        assert orc.orc_dipole_ewald(e.h, abi.f64(dip.reshape(-1)), abi.f64(pot), abi.f64(est), abi.f64(efg),
                                    abi.f64(vir)) == 0
        e.close()
        assert orc.orc_poly_udipole_self(C.byref(p), abi.f64(r.reshape(-1)), abi.f64(dip.reshape(-1)), int(s.lsurf),
                                         abi.f64(pot), abi.f64(est), abi.f64(efg), abi.f64(vir)) == 0
    force, torque, ustat = np.zeros(3 * na), np.zeros(3 * na), np.zeros(1)
    assert orc.orc_poly_udipole_finish(C.byref(p), abi.f64(dip.reshape(-1)), abi.f64(pot), abi.f64(est),
                                       abi.f64(efg), abi.f64(force), abi.f64(torque), abi.f64(ustat)) == 0
    return dict(u_stat=float(ustat[0]), u_real=float(ureal[0]), potstat=pot, estat=est.reshape(-1, 3),
                efg=efg.reshape(-1, 6), force=force.reshape(-1, 3), torque=torque.reshape(-1, 3),
                virelec=float(vir[0]))


def _setup(s, orc):
    s.build_table(orc.orc_pot_twobody_tab)
    return s


def dumbbell_energy(s, d, surf, beta):
    """Energy (e^2/A) of the system with each dipole as +-|dip|/d at +-d/2,
    intramolecular pairs excluded."""
    r = s.atom_positions()
    dip = s.atom_dipoles()
    q = s.aza()
    pos, chg, mol = [], [], []
    first = s.ianpn() - 1
    napt = s.napt()[s.iptpn - 1]
    molof = np.repeat(np.arange(s.np_), napt)
    for a in range(len(r)):
        mu = np.linalg.norm(dip[a])
        u = dip[a] / mu
        pos += [r[a], r[a] + 0.5 * d * u, r[a] - 0.5 * d * u]
        chg += [q[a], mu / d, -mu / d]
        mol += [molof[a]] * 3
    pos, chg, mol = np.array(pos), np.array(chg), np.array(mol)
    e = ewald_exact(pos, chg, s.boxlen, surf, beta, nreal=3, kmax=26)
    for i in range(len(chg)):
        for j in range(i + 1, len(chg)):
            if mol[i] == mol[j]:
                e -= chg[i] * chg[j] / np.linalg.norm(pos[i] - pos[j])
    return e


@pytest.mark.parametrize("surf", [0, 1])
def test_dipole_energy_matches_point_charge_limit(surf, orc):
    s = _setup(dipole_system(lsurf=surf), orc)
    beta = 1.2
    e1 = dumbbell_energy(s, 4e-2, surf, beta)
    e2 = dumbbell_energy(s, 2e-2, surf, beta)
    e0 = (4.0 * e2 - e1) / 3.0
    assert abs(e1 - e2) > 1e-7 * abs(e0)               # the extrapolation has something to remove
    # the sum has converged: another splitting parameter gives the same
    e0b = (4.0 * dumbbell_energy(s, 2e-2, surf, 1.5) - dumbbell_energy(s, 4e-2, surf, 1.5)) / 3.0
    assert abs(e0 - e0b) <= 1e-7 * abs(e0)
    o = oracle_udipole(orc, s)
    u = o["u_stat"] / s.epsi_four_pi
    assert abs(u - e0) <= 1e-7 * abs(e0), (u, e0)


def test_dipole_derivatives(orc):
    """-dU/d(dip_a) = EpsiFourPi e_a, -dU/dr_a = force_a, and the torque of
    a small turn of dip_a is dip_a x e_a."""
    s = _setup(dipole_system(seed=5), orc)
    o = oracle_udipole(orc, s)
    dip = s.atom_dipoles()
    r = s.atom_positions()
    h = 1e-5
    efp = s.epsi_four_pi
    for a in (0, 3, 5):
        for m in range(3):
            d1, d2 = dip.copy(), dip.copy()
            d1[a, m] += h
            d2[a, m] -= h
            g = (oracle_udipole(orc, s, dip=d1)["u_stat"] - oracle_udipole(orc, s, dip=d2)["u_stat"]) / (2 * h)
            assert abs(-g - efp * o["estat"][a, m]) <= 1e-6 * efp * np.abs(o["estat"]).max()
            r1, r2 = r.copy(), r.copy()
            r1[a, m] += h
            r2[a, m] -= h
            g = (oracle_udipole(orc, s, r=r1)["u_stat"] - oracle_udipole(orc, s, r=r2)["u_stat"]) / (2 * h)
            assert abs(-g - o["force"][a, m]) <= 1e-6 * np.abs(o["force"]).max()
    assert np.allclose(o["torque"], efp * np.cross(dip, o["estat"]), rtol=0, atol=1e-13 * np.abs(o["torque"]).max())
    # the field gradient at an atom comes from the other charges and dipoles
    # only (the self terms take the atom's own Gaussian out), so it obeys
    # Laplace's equation: traceless
    tr = o["efg"][:, 0] + o["efg"][:, 1] + o["efg"][:, 2]
    assert np.abs(tr).max() <= 1e-7 * np.abs(o["efg"]).max()


def test_dipole_spme_matches_std(orc):
    """Order 10 on 128^3 against standard Ewald: energies within 1e-7 of the
    atomic self term that the reciprocal sum cancels (the reference's
    single-precision b^2 factors bound SPME near 1e-8 of it), fields and
    forces within 1e-5 of their largest values."""
    s_std = _setup(dipole_system(seed=7), orc)
    s_spm = _setup(dipole_system(seed=7, ewald=abi.MG_EWALD_SPM, order=10, nmesh=128), orc)
    a, b = oracle_udipole(orc, s_std), oracle_udipole(orc, s_spm)
    al = s_std.ualpha
    s1, s2 = 2.0 * al / np.sqrt(np.pi), 4.0 * al ** 3 / (3.0 * np.sqrt(np.pi))
    scale = 0.5 * s_std.epsi_four_pi * (s1 * (s_std.aza() ** 2).sum() + s2 * (s_std.atom_dipoles() ** 2).sum())
    assert abs(a["u_stat"] - b["u_stat"]) <= 1e-7 * scale
    assert np.abs(a["efg"] - b["efg"]).max() <= 1e-5 * np.abs(a["efg"]).max()
    assert np.abs(a["force"] - b["force"]).max() <= 1e-5 * np.abs(a["force"]).max()
    assert np.abs(a["torque"] - b["torque"]).max() <= 1e-5 * np.abs(a["torque"]).max()
    assert abs(a["virelec"] - b["virelec"]) <= 1e-5 * abs(a["virelec"])


def oracle_dip_utotal(orc, s, ro, ori):
    """UTotal of a dipole system on the oracle (UTwoBodyP with the LJ-only
    table, UDipole, the epilogue with the atom torques): u%tot, forceo,
    torqueo."""
    from tests.test_cpu_poly import oracle_poly
    s.ro, s.ori = np.ascontiguousarray(ro), np.ascontiguousarray(ori)
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 0.5)
    tw = oracle_poly(orc, s, nn, jl, maxn)
    d = oracle_udipole(orc, s)
    force = tw["force"] + d["force"]
    p = s.params()
    r = s.atom_positions()
    fo, to, vm = np.zeros(3 * s.np_), np.zeros(3 * s.np_), np.zeros(1)
    assert orc.orc_poly_epilogue(C.byref(p), abi.f64(abi.as_f64(s.ro.reshape(-1))), abi.f64(r.reshape(-1)),
                                 abi.f64(abi.as_f64(force.reshape(-1))), abi.f64(abi.as_f64(d["torque"].reshape(-1))),
                                 units.FORCE_FAC, abi.f64(fo), abi.f64(to), abi.f64(vm)) == 0
    return tw["u_twob"][0] + d["u_stat"], fo.reshape(-1, 3), to.reshape(-1, 3)


def test_dipole_particle_forces_and_torques_are_gradients(orc):
    """forceo and torqueo of a dipole system (UTwoBodyP's LJ, UDipole's
    charges and dipoles, the atom torques dip x e in the epilogue) against
    central differences of u%tot under translations of a particle and
    rotations about its centre: -dU/dx = forceo / force_fac and -dU/dtheta
    (about a lab axis n) = torqueo . n / force_fac."""
    from molsim_gb300 import configs
    from molsim_gb300.mc import axis_angle_matrix
    s = _setup(configs.dipolar_waters(seed=23, nwater=30, nsalt=3, L=12.0, rcut=5.5, ewald=abi.MG_EWALD_STD,
                                      ualpha=0.55, ncut=9), orc)
    ro0, ori0 = s.ro.copy(), s.ori.copy()
    u0, fo, to = oracle_dip_utotal(orc, s, ro0, ori0)
    ff = units.FORCE_FAC
    # the atoms' own torques dip x e are a sizeable part of the particle torques
    d = oracle_udipole(orc, s)
    dip_part = np.zeros_like(to)
    np.add.at(dip_part, np.repeat(np.arange(s.np_), s.napt()[s.iptpn - 1]), d["torque"] * ff)
    assert np.abs(dip_part).max() > 0.05 * np.abs(to).max()
    h = 1e-5
    for p in (0, 7, 31):
        for m in range(3):
            r1, r2 = ro0.copy(), ro0.copy()
            r1[p, m] += h
            r2[p, m] -= h
            g = (oracle_dip_utotal(orc, s, r1, ori0)[0] - oracle_dip_utotal(orc, s, r2, ori0)[0]) / (2 * h)
            assert abs(-g - fo[p, m] / ff) <= 1e-6 * np.abs(fo).max() / ff, (p, m, -g, fo[p, m] / ff)
            n = np.zeros(3)
            n[m] = 1.0
            o1, o2 = ori0.copy(), ori0.copy()
            # a turn by +h about n: the reference's matrix of angle a turns by -a
            o1[p] = axis_angle_matrix(n, -h) @ ori0[p]
            o2[p] = axis_angle_matrix(n, h) @ ori0[p]
            g = (oracle_dip_utotal(orc, s, ro0, o1)[0] - oracle_dip_utotal(orc, s, ro0, o2)[0]) / (2 * h)
            assert abs(-g - to[p, m] / ff) <= 1e-6 * np.abs(to).max() / ff, (p, m, -g, to[p, m] / ff)
