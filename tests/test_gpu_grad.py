"""Gradients of UTotal (mg_grad, the adjoint form) against finite differences.

The finite differences are central, with the step the gradient configuration
states (1e-4 relative for the species parameters, 1e-5 for the box), taken
on the oracle's UTotal.  The tables are built to a tight tolerance
(utoltab 1e-9), so that the tabulated energy and the analytic derivatives
agree to far below the 1e-6 relative bar.  The identities
sum_a L_a dU/dL_a = virial and (Coulomb only) sum_i q_i phi_i = 2 U tie the
gradients to UTotal's own outputs.
"""
import dataclasses

import numpy as np
import pytest

from molsim_gb300 import Engine, abi, configs, units
from molsim_gb300.system import Species

pytestmark = pytest.mark.gpu

TOL_FD = 1e-6


def _tight(s):
    # a cut-and-shifted LJ (lljcut) keeps a small force step at its cut, so
    # its force table is held to 1e-7
    s.utoltab, s.ftoltab = 1e-9, (1e-7 if s.lljcut else 1e-8)
    return s


def _u_oracle(s, orc):
    s = dataclasses.replace(s, ubuf=None, iubuflow=None, r2umin=None, nugrid=None)
    s.build_table(orc.orc_pot_twobody_tab)
    e = Engine(s, lib=orc, prefix="orc_")
    e.SetPositions(s.ro_flat())
    e.NList("write")
    u = e.UTotal()["u_tot"]
    e.close()
    return u


def _gpu(s, form=abi.MG_FP64):
    s = dataclasses.replace(s, ubuf=None, iubuflow=None, r2umin=None, nugrid=None)
    s.build_table()
    e = Engine(s, form=form)
    e.SetPositions(s.ro_flat())
    e.NList("write")
    return e, e.UTotal(), e.Grad()


SYSTEMS = {
    "spme": lambda: configs.small_system(seed=81),
    "spme_surf_bonds": lambda: configs.small_system(seed=82, lsurf=1, chains=3, nseg=8),
    "std_cell": lambda: configs.small_system(seed=83, ewald=abi.MG_EWALD_STD, ncut=5,
                                             txintlist=abi.MG_CELLLIST),
    "no_ewald_wca": lambda: configs.small_system(seed=84, ewald=abi.MG_EWALD_NONE, lljcut=1),
    "spme_angles": lambda: configs.small_system(seed=89, chains=3, nseg=8, angle_kt=0.8),
}


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_box_gradient_sums_to_virial(name, gpu_lib):
    s = _tight(SYSTEMS[name]())
    _, u, g = _gpu(s)
    lhs = float(np.dot(s.boxlen, g["du_dbox"]))
    assert abs(lhs - u["virial"]) <= 1e-10 * abs(u["virial"]), (lhs, u["virial"])


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_box_gradient_finite_differences(name, orc, gpu_lib):
    s = _tight(SYSTEMS[name]())
    _, _, g = _gpu(s)
    h = 1e-5
    norm = np.abs(g["du_dbox"]).max()
    for a in range(3):
        fd = 0.0
        us = []
        for sgn in (+1, -1):
            f = np.ones(3)
            f[a] += sgn * h
            s2 = dataclasses.replace(s, boxlen=s.boxlen * f, ro=s.ro * f)
            us.append(_u_oracle(s2, orc))
        fd = (us[0] - us[1]) / (2 * h * s.boxlen[a])
        assert abs(fd - g["du_dbox"][a]) <= TOL_FD * norm, (a, fd, g["du_dbox"][a])


def _species_fd(s, orc, a, field, h):
    us = []
    for sgn in (+1, -1):
        sp = list(s.species)
        v = getattr(sp[a], field)
        sp[a] = dataclasses.replace(sp[a], **{field: v * (1 + sgn * h)})
        us.append(_u_oracle(dataclasses.replace(s, species=sp), orc))
    return (us[0] - us[1]) / (2 * h * getattr(s.species[a], field))


@pytest.mark.parametrize("name", ["spme", "spme_surf_bonds", "std_cell"])
def test_species_gradients_finite_differences(name, orc, gpu_lib):
    from molsim_gb300.autograd import _species_grads
    s = _tight(SYSTEMS[name]())
    _, _, g = _gpu(s)
    dz, dsig, deps = _species_grads(s, g)
    for a in range(s.npt):
        for field, val in (("charge", dz[a]), ("sigma", dsig[a]), ("eps", deps[a])):
            fd = _species_fd(s, orc, a, field, 1e-4)
            assert abs(fd - val) <= TOL_FD * max(abs(fd), 1e-3), (a, field, fd, val)


def test_site_potential_of_one_particle(orc, gpu_lib):
    """A probe species with a single member: dU/dz_probe is that particle's
    site potential."""
    s = _tight(configs.small_system(seed=85))
    kt = units.kT(s.temp)
    sp = list(s.species) + [Species("probe", +1.0, 3.5, 0.1 * kt, mass=23.0)]
    iptpn = s.iptpn.copy()
    iptpn[17] = 4
    s = dataclasses.replace(s, species=sp, iptpn=iptpn)
    _, _, g = _gpu(s)
    fd = _species_fd(s, orc, 3, "charge", 1e-4)
    assert abs(fd - g["phi"][17]) <= TOL_FD * abs(fd)


@pytest.mark.parametrize("ewald,lsurf", [(abi.MG_EWALD_SPM, 0), (abi.MG_EWALD_SPM, 1), (abi.MG_EWALD_STD, 1),
                                         (abi.MG_EWALD_NONE, 0)])
def test_site_potentials_euler_identity(ewald, lsurf, gpu_lib):
    """Coulomb energy is homogeneous of degree 2 in the charges."""
    s = _tight(configs.small_system(seed=86, ewald=ewald, lsurf=lsurf, ncut=5, eps_kt=0.0))
    _, u, g = _gpu(s)
    lhs = float(np.dot(s.az, g["phi"]))
    assert abs(lhs - 2 * u["u_tot"]) <= 1e-7 * abs(u["u_tot"])


def test_mixed_site_potentials_near_fp64(gpu_lib):
    s = configs.small_system(seed=87)
    _, _, g64 = _gpu(s)
    _, _, gmx = _gpu(s, abi.MG_MIXED)
    d = gmx["phi"] - g64["phi"]
    assert np.sqrt((d * d).mean()) <= 1e-5 * np.sqrt((g64["phi"] ** 2).mean())
    assert np.allclose(gmx["du_dbox"], g64["du_dbox"], rtol=1e-5, atol=1e-6 * np.abs(g64["du_dbox"]).max())


def test_autograd_function(gpu_lib):
    torch = pytest.importorskip("torch")
    from molsim_gb300.autograd import Model, utotal
    s = _tight(configs.small_system(seed=88))
    model = Model(s)
    dt = torch.float64
    ro = torch.tensor(s.ro, dtype=dt, requires_grad=True)
    z = torch.tensor([sp.charge for sp in s.species], dtype=dt, requires_grad=True)
    sig = torch.tensor([sp.sigma for sp in s.species], dtype=dt, requires_grad=True)
    eps = torch.tensor([sp.eps for sp in s.species], dtype=dt, requires_grad=True)
    box = torch.tensor(s.boxlen, dtype=dt, requires_grad=True)
    u = utotal(ro, z, sig, eps, box, model)
    u.backward()
    e, ref, _ = _gpu(s)
    assert float(u.detach()) == pytest.approx(ref["u_tot"], rel=1e-12)
    assert np.allclose(ro.grad.numpy(), -ref["forceo"] / units.FORCE_FAC, rtol=0, atol=1e-12)
    # the autograd gradient of sigma_1 against a finite difference of the function itself
    h = 1e-4 * float(sig[1])
    with torch.no_grad():
        up = utotal(ro, z, sig + torch.tensor([0, h, 0], dtype=dt), eps, box, model)
        dn = utotal(ro, z, sig - torch.tensor([0, h, 0], dtype=dt), eps, box, model)
    fd = float(up - dn) / (2 * h)
    assert abs(fd - float(sig.grad[1])) <= TOL_FD * abs(fd)
