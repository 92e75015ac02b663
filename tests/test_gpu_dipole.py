"""Charges and point dipoles on the GPU (mg_poly_udipole_*, mg_dipole_ewald)
against the oracle: UDipole with standard Ewald (with and without the
surface term) and SPME, UTotal of a dipole system, and rigid-body steps
driven by it.

FP64 arithmetic; the real-space pair loop adds the partner atoms' terms
as 64-bit fixed-point integers (the same bits on every call), so the
order and rounding of the additions differ from the oracle's: potentials,
fields, field gradients, forces and torques within 1e-10 of their largest
values, energies within 1e-10 of the atomic self term that the reciprocal
sum cancels.
"""
import numpy as np
import pytest

from molsim_gb300 import abi, configs
from molsim_gb300.poly import PolyEngine, ori_to_qua
from tests.helpers import centre_lists
from tests.test_cpu_dipole import _setup, oracle_dip_utotal, oracle_udipole

pytestmark = pytest.mark.gpu


def _system(orc, ewald, lsurf=0, seed=41):
    s = configs.dipolar_waters(seed=seed, nwater=150, nsalt=8, L=20.0, rcut=9.0, ewald=ewald, ualpha=0.35,
                               order=6, nmesh=32, ncut=8)
    s.lsurf = lsurf
    return _setup(s, orc)


def _scale(s):
    al = s.ualpha
    s1, s2 = 2.0 * al / np.sqrt(np.pi), 4.0 * al ** 3 / (3.0 * np.sqrt(np.pi))
    return 0.5 * s.epsi_four_pi * (s1 * (s.aza() ** 2).sum() + s2 * (s.atom_dipoles() ** 2).sum())


def _close(a, b, tol=1e-10):
    return np.abs(np.asarray(a) - np.asarray(b)).max() <= tol * max(np.abs(np.asarray(b)).max(), 1e-300)


@pytest.mark.parametrize("ewald,lsurf", [(abi.MG_EWALD_STD, 0), (abi.MG_EWALD_STD, 1), (abi.MG_EWALD_SPM, 0)],
                         ids=["std", "std_surf", "spm"])
def test_udipole_matches_oracle(ewald, lsurf, orc, gpu_lib):
    s = _system(orc, ewald, lsurf)
    ref = oracle_udipole(orc, s)
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 0.5)
    e = PolyEngine(s, maxn)
    g = e.UDipole(nn, jl)
    for k in ("potstat", "estat", "efg", "force", "torque"):
        assert _close(g[k], ref[k]), k
    sc = _scale(s)
    assert abs(g["u_stat"] - ref["u_stat"]) <= 1e-10 * sc
    assert abs(g["virial"] - s.epsi_four_pi * ref["virelec"]) <= 1e-10 * sc
    g2 = e.UDipole(nn, jl)   # integer sums in the pair loop: the same bits on every call
    for k in ("potstat", "estat", "efg", "force", "torque"):
        assert np.array_equal(g[k], g2[k]), k
    assert g["u_stat"] == g2["u_stat"]
    e.close()


def test_udipole_without_ewald_matches_oracle(orc, gpu_lib):
    """Bare Coulomb kernels (no Ewald): UDipoleP and UDipole's loop only."""
    s = _system(orc, abi.MG_EWALD_NONE)
    s.ualpha = 0.0
    s.build_table(orc.orc_pot_twobody_tab)
    ref = oracle_udipole(orc, s)
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 0.5)
    e = PolyEngine(s, maxn)
    g = e.UDipole(nn, jl)
    for k in ("potstat", "estat", "efg", "force", "torque"):
        assert _close(g[k], ref[k]), k
    assert abs(g["u_stat"] - ref["u_stat"]) <= 1e-10 * abs(ref["u_stat"])
    e.close()


def test_dipole_utotal_matches_oracle(orc, gpu_lib):
    """UTotal of a dipole system (UTwoBodyP with the LJ-only table, UDipole,
    the epilogue with the atom torques) against the oracle."""
    s = _system(orc, abi.MG_EWALD_SPM)
    u_ref, fo_ref, to_ref = oracle_dip_utotal(orc, s, s.ro.copy(), s.ori.copy())
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 0.5)
    e = PolyEngine(s, maxn)
    g = e.UTotal(nn, jl)
    assert abs(g["u_tot"] - u_ref) <= 1e-10 * _scale(s)
    assert _close(g["forceo"], fo_ref) and _close(g["torqueo"], to_ref)
    # the device-resident centre list gives the same
    h = e.UTotal()
    assert abs(h["u_tot"] - u_ref) <= 1e-10 * _scale(s)
    assert _close(h["forceo"], fo_ref, 1e-9) and _close(h["torqueo"], to_ref, 1e-9)
    e.close()


def test_dipole_rigid_steps_match_oracle(orc, gpu_lib):
    """Ten rigid-body steps of dipolar waters (device VelVer, device UTotal
    with dipoles) against ten oracle steps: centres and orientations within
    1e-9."""
    from tests.test_cpu_rigid import OracleRigid, _initial_velocities

    def system():
        s = configs.dipolar_waters(seed=43, nwater=60, nsalt=4, L=15.0, rcut=7.0, ewald=abi.MG_EWALD_SPM,
                                   ualpha=0.45, order=6, nmesh=32).principal_axes()
        return _setup(s, orc)

    dt = 0.0005
    s = system()
    v, w = _initial_velocities(s, seed=3)
    massip, momp = s.rigid_props()
    st = OracleRigid(orc, dt, s.boxlen, massip, momp, s.ro, ori_to_qua(s.ori), v, w)
    u, fo, to = oracle_dip_utotal(orc, s, s.ro.copy(), s.ori.copy())
    st.prime(fo, to)
    for _ in range(10):
        st.move()
        u, fo, to = oracle_dip_utotal(orc, s, st.ro.reshape(-1, 3), st.ori_np())
        st.kick(fo, to)
    g = system()
    e = PolyEngine(g, maxnneigh=256)
    e.RigidSetup(dt, v, w, prime=True)
    out = e.VelVer(10)
    assert np.abs(g.ro.reshape(-1) - st.ro).max() < 1e-9
    assert np.abs(g.ori - st.ori_np()).max() < 1e-9
    assert abs(out["u_tot"] - u) <= 1e-9 * _scale(g)
    e.close()
