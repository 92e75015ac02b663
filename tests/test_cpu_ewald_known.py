"""Known answers for the oracle's Ewald sums from the reference's two-charge
test inputs, computed without the oracle.

The reference's test set holds two-charge Ewald cases (Testin/in/holm.ew1.in:
+1 and -1 e, 0.1 A apart along x in a 1 x 1 x 2 A box, rcut 0.5 A,
ualphared 3 (alpha = 6/A), ncut 15 in the cube region, surface term on;
Testin/in/qq.ew.surf.in and qq.ew.nosurf.in: 1 A apart in a 10 A cube, rcut
5 A, ualphared 4 (alpha = 0.8/A), with and without the surface term) but no
expected numbers.  Here the expected energies come from an Ewald sum written
in numpy (real-space images to |n| <= 4, the full k-space sum, self and
surface terms) at three other splitting parameters, whose agreement shows
that the sum has converged; the forces are central differences of that
energy.  The oracle's UTotal (tabulated real-space part, UEwaldRecStd or
UEwaldRecSPM, UEwaldSelf, UEwaldSurf: energy.F90:280-430, 964-1102,
1207-1371) must agree: standard Ewald within 1e-9 relative, SPME within 1e-8
(its b^2 factors are computed in single-precision complex, as the reference
does, which limits SPME to a few 1e-9 however fine the mesh).
"""
import itertools
import math

import numpy as np
import pytest

from molsim_gb300 import Engine, abi, units
from molsim_gb300.system import Species, System

scipy_special = pytest.importorskip("scipy.special")


def ewald_exact(pos, q, box, surf, beta, nreal=4, kmax=30):
    """Coulomb energy (units of e^2/(4 pi eps0 A)) of the periodic system by
    an Ewald sum with splitting parameter beta."""
    box = np.asarray(box, dtype=float)
    vol = float(box.prod())
    e_real = 0.0
    images = [np.array(n) * box for n in itertools.product(range(-nreal, nreal + 1), repeat=3)]
    for i in range(len(q)):
        for j in range(len(q)):
            for t in images:
                if i == j and not t.any():
                    continue
                r = float(np.linalg.norm(pos[i] - pos[j] + t))
                e_real += 0.5 * q[i] * q[j] * scipy_special.erfc(beta * r) / r
    m = np.arange(-kmax, kmax + 1)
    mx, my, mz = np.meshgrid(m, m, m, indexing="ij")
    k = 2 * np.pi * np.stack([mx / box[0], my / box[1], mz / box[2]], -1).reshape(-1, 3)
    k2 = (k * k).sum(1)
    k, k2 = k[k2 > 0], k2[k2 > 0]
    s = (q[None, :] * np.exp(1j * (k @ pos.T))).sum(1)
    e_rec = float((2 * np.pi / vol * np.exp(-k2 / (4 * beta * beta)) / k2 * np.abs(s) ** 2).sum())
    e_self = -beta / math.sqrt(math.pi) * float((q * q).sum())
    dip = (q[:, None] * pos).sum(0)
    e_surf = 2 * math.pi / (3 * vol) * float(dip @ dip) if surf else 0.0
    return e_real + e_rec + e_self + e_surf


def exact_answer(pos, q, box, surf, betas, h=1e-5, **kw):
    """Energy (checked to agree at every beta) and central-difference forces."""
    es = [ewald_exact(pos, q, box, surf, b, **kw) for b in betas]
    assert max(es) - min(es) <= 1e-13 * abs(es[0]), es
    f = np.zeros_like(pos)
    for i in range(len(q)):
        for m in range(3):
            p1, p2 = pos.copy(), pos.copy()
            p1[i, m] += h
            p2[i, m] -= h
            f[i, m] = -(ewald_exact(p1, q, box, surf, betas[0], **kw)
                        - ewald_exact(p2, q, box, surf, betas[0], **kw)) / (2 * h)
    return es[0], f


def oracle_utotal(orc, pos, box, rcut, alpha, surf, ewald, ncut=12, cube=0, order=10, nmesh=64, **kw):
    sp = [Species("p", 1.0, 2.0, 0.0, radat=0.01), Species("m", -1.0, 2.0, 0.0, radat=0.01)]
    s = System(species=sp, iptpn=np.array([1, 2], dtype=np.int32), ro=pos, boxlen=np.array(box, dtype=float),
               relpermitt=1.0, rcut=rcut, ewald=ewald, ualpha=alpha, ncut=ncut, ncutregion_cube=cube,
               lsurf=surf, order=order, nmesh=nmesh, **kw)
    s.build_table(orc.orc_pot_twobody_tab)
    e = Engine(s, lib=orc, prefix="orc_")
    e.SetPositions(s.ro_flat())
    e.NList("write")
    r = e.UTotal()
    e.close()
    # back to e^2/(4 pi eps0 A) and e^2/(4 pi eps0 A^2)
    return r["u_tot"] / s.epsi_four_pi, r["forceo"] / (units.FORCE_FAC * s.epsi_four_pi)


Q = np.array([1.0, -1.0])
# (name, positions, box, rcut, alpha, surface term, extra table settings, ncut, region)
CASES = [
    ("holm_ew1", np.array([[0.0, 0.0, 0.0], [0.1, 0.0, 0.0]]), [1.0, 1.0, 2.0], 0.5, 3.0 / 0.5, 1,
     dict(r2uminin=1e-8, umaxtab=1e6, fmaxtab=1e6), 15, 1),
    ("qq_ew_surf", np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]]), [10.0] * 3, 5.0, 4.0 / 5.0, 1, {}, 12, 0),
    ("qq_ew_nosurf", np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]]), [10.0] * 3, 5.0, 4.0 / 5.0, 0, {}, 12, 0),
]


@pytest.mark.parametrize("name,pos,box,rcut,alpha,surf,tab,ncut,cube", CASES, ids=[c[0] for c in CASES])
def test_two_charge_ewald_known_answer(name, pos, box, rcut, alpha, surf, tab, ncut, cube, orc):
    bmin = min(box)
    u_ref, f_ref = exact_answer(pos, Q, box, surf, betas=[3.0 / bmin, 4.0 / bmin, 5.0 / bmin])
    # the finite-difference forces are those of the energy: they sum to zero
    assert np.abs(f_ref.sum(0)).max() <= 1e-6 * np.abs(f_ref).max()
    u, f = oracle_utotal(orc, pos, box, rcut, alpha, surf, abi.MG_EWALD_STD, ncut=ncut, cube=cube, **tab)
    assert abs(u - u_ref) <= 1e-9 * abs(u_ref), (u, u_ref)
    assert np.abs(f - f_ref).max() <= 1e-7 * np.abs(f_ref).max(), (f, f_ref)
    if box[0] == box[1] == box[2]:   # the reference's SPME mesh is cubic
        u, f = oracle_utotal(orc, pos, box, rcut, alpha, surf, abi.MG_EWALD_SPM, order=11, nmesh=128, **tab)
        assert abs(u - u_ref) <= 1e-8 * abs(u_ref), (u, u_ref)
        assert np.abs(f - f_ref).max() <= 1e-7 * np.abs(f_ref).max(), (f, f_ref)


def test_two_charges_far_apart_approach_coulomb(orc):
    """In a box much larger than their distance two charges feel their bare
    Coulomb attraction, -1/d, up to the box's small correction."""
    d, L = 1.0, 200.0
    pos = np.array([[0.0, 0.0, 0.0], [d, 0.0, 0.0]])
    u, f = oracle_utotal(orc, pos, [L] * 3, 30.0, 3.0 / 30.0, 0, abi.MG_EWALD_STD, ncut=20)
    assert abs(u - (-1.0 / d)) <= 1e-4
    assert abs(f[0, 0] - 1.0 / d ** 2) <= 1e-4 and abs(f[1, 0] + 1.0 / d ** 2) <= 1e-4
