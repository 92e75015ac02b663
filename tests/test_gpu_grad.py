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
    h = 1e-4 * float(sig.detach()[1])
    with torch.no_grad():
        up = utotal(ro, z, sig + torch.tensor([0, h, 0], dtype=dt), eps, box, model)
        dn = utotal(ro, z, sig - torch.tensor([0, h, 0], dtype=dt), eps, box, model)
    fd = float(up - dn) / (2 * h)
    assert abs(fd - float(sig.grad[1])) <= TOL_FD * abs(fd)


# ---- the virial tensor (dU/deps for an affine strain r -> (1 + eps) r) ---------

def _strained_energy(s, eps, ncut, alpha, rcut, lsurf):
    """UTotal of a Coulomb-only system with standard Ewald, bonds and angles
    after the strain r -> (1 + eps) r of the box and the positions, in
    numpy: real-space erfc pairs of the unstrained minimum-image set within
    rcut, the reciprocal sum over the integer vectors |n| <= ncut (the
    handle's set), the self term, the surface term and the chain terms."""
    from scipy.special import erfc
    pos = np.asarray(s.ro, dtype=float)
    q = s.az
    L = np.asarray(s.boxlen, dtype=float)
    A = np.eye(3) + eps
    H = A @ np.diag(L)
    vol = abs(np.linalg.det(H))
    d = pos[:, None, :] - pos[None, :, :]
    d -= L * np.round(d / L)
    r0 = np.sqrt((d * d).sum(-1))
    mask = (r0 < rcut) & ~np.eye(len(q), dtype=bool)
    ds = d @ A.T
    r = np.sqrt((ds * ds).sum(-1))
    qq = q[:, None] * q[None, :]
    e_real = 0.5 * (qq * erfc(alpha * r) / np.where(mask, r, 1.0))[mask].sum()
    m = np.arange(-ncut, ncut + 1)
    n = np.stack(np.meshgrid(m, m, m, indexing="ij"), -1).reshape(-1, 3)
    n2 = (n * n).sum(1)
    n = n[(n2 > 0) & (n2 <= ncut * ncut)]
    k = 2 * np.pi * n @ np.linalg.inv(H)
    k2 = (k * k).sum(1)
    rs = pos @ A.T
    S = (q[None, :] * np.exp(1j * (k @ rs.T))).sum(1)
    e_rec = (2 * np.pi / vol * np.exp(-k2 / (4 * alpha ** 2)) / k2 * np.abs(S) ** 2).sum()
    e_self = -alpha / np.sqrt(np.pi) * (q * q).sum()
    M = (q[:, None] * rs).sum(0)
    e_surf = 2 * np.pi / (3 * vol) * (M @ M) if lsurf else 0.0
    u = s.epsi_four_pi * (e_real + e_rec + e_self + e_surf)

    def vec(i, j):
        v = pos[i - 1] - pos[j - 1]
        v -= L * np.round(v / L)
        return A @ v
    for i, j, kb, eq, p in zip(s.bond_ip, s.bond_jp, s.bond_k, s.bond_eq, s.bond_p):
        u += kb * (np.linalg.norm(vec(i, j)) - eq) ** p
    for jm, ip, jp, ka, eq, p in zip(s.angle_jm, s.angle_ip, s.angle_jp, s.angle_k, s.angle_eq, s.angle_p):
        a, b = vec(ip, jm), vec(ip, jp)
        c = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
        u += ka * (np.arccos(np.clip(c, -1, 1)) - eq) ** p
    return u


def _tensor_system(lsurf):
    return _tight(configs.small_system(seed=90, n=240, L=34.0, rcut=11.0, ewald=abi.MG_EWALD_STD, ncut=9,
                                       eps_kt=0.0, chains=3, nseg=8, angle_kt=0.8, lsurf=lsurf))


@pytest.mark.parametrize("lsurf", [0, 1])
def test_virial_tensor_against_strained_energy(lsurf, gpu_lib):
    """All nine components against central differences (step 1e-6) of the
    strained energy computed in numpy; the tensor is symmetric, its trace is
    UTotal's virial and its diagonal is L_a dU/dL_a of mg_grad."""
    s = _tensor_system(lsurf)
    e, u, g = _gpu(s)
    w = e.VirialTensor()
    assert abs(np.trace(w) - u["virial"]) <= 1e-10 * abs(u["virial"])
    assert np.abs(np.diag(w) - s.boxlen * g["du_dbox"]).max() <= 1e-10 * np.abs(w).max()
    assert np.abs(w - w.T).max() <= 1e-10 * np.abs(w).max()
    u0 = _strained_energy(s, np.zeros((3, 3)), s.ncut, s.ualpha, s.rcut, lsurf)
    assert abs(u0 - u["u_tot"]) <= 1e-7 * abs(u["u_tot"]), (u0, u["u_tot"])
    h = 1e-6
    for a in range(3):
        for b in range(3):
            ep = np.zeros((3, 3))
            ep[a, b] = h
            fd = (_strained_energy(s, ep, s.ncut, s.ualpha, s.rcut, lsurf)
                  - _strained_energy(s, -ep, s.ncut, s.ualpha, s.rcut, lsurf)) / (2 * h)
            assert abs(fd - w[a, b]) <= TOL_FD * np.abs(w).max(), (a, b, fd, w[a, b])


@pytest.mark.parametrize("form", [abi.MG_FP64, abi.MG_MIXED])
def test_virial_tensor_spme_matches_standard_ewald(form, gpu_lib):
    """The SPME tensor (k-space part through the mesh's signed wave vectors)
    against the standard-Ewald tensor of the same system with a converged
    k-sum: equal to the SPME accuracy."""
    s = _tensor_system(0)
    s_std = dataclasses.replace(s, ncut=16)
    s_spm = dataclasses.replace(s, ewald=abi.MG_EWALD_SPM, order=8, nmesh=64)
    w_std = _gpu(s_std)[0].VirialTensor()
    w_spm = _gpu(s_spm, form)[0].VirialTensor()
    assert np.abs(w_spm - w_std).max() <= 1e-5 * np.abs(w_std).max(), (w_spm, w_std)


def test_gradients_at_the_32768_ion_electrolyte_mixed(orc, gpu_lib):
    """The gradient configuration in full: the 32 768-ion SPME electrolyte
    (64^3, order 6, r_c = 12 A) with the mixed (FP32) forward pass.  dU/deps
    and dU/dsig of both species (all three type pairs through the mixing
    rules) and dU/dq at three sites against central differences (1e-4
    relative) of the oracle's FP64 UTotal; the LJ parameter gradients are
    FP64 sums in both forms and agree to 1e-6, the site potentials carry the
    FP32 potential mesh and agree to 1e-5 of the RMS site potential."""
    from molsim_gb300.autograd import _species_grads
    orc.orc_set_threads(max(1, min(16, __import__("os").cpu_count() or 1)))
    try:
        s = _tight(configs.electrolyte_spme())
        s.txintlist = abi.MG_CELLLIST
        _, _, g = _gpu(s, abi.MG_MIXED)
        dz, dsig, deps = _species_grads(s, g)
        for a in range(s.npt):
            for field, val in (("sigma", dsig[a]), ("eps", deps[a])):
                fd = _species_fd(s, orc, a, field, 1e-4)
                assert abs(fd - val) <= TOL_FD * max(abs(fd), 1e-3), (a, field, fd, val)
        phi_rms = float(np.sqrt((g["phi"] ** 2).mean()))
        for site in (0, 12345, 32767):
            t = int(s.iptpn[site]) - 1
            sp = list(s.species) + [dataclasses.replace(s.species[t], name="probe")]
            iptpn = s.iptpn.copy()
            iptpn[site] = len(sp)
            sp_sys = dataclasses.replace(s, species=sp, iptpn=iptpn)
            fd = _species_fd(sp_sys, orc, len(sp) - 1, "charge", 1e-4)
            assert abs(fd - g["phi"][site]) <= 1e-5 * phi_rms, (site, fd, g["phi"][site])
    finally:
        orc.orc_set_threads(1)
