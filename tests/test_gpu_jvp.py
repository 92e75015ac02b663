"""Force Jacobian-vector products (mg_force_jvp) against differences of the
forces.

jv = d(forceo)/dx . u from the derivative kernels (the tabulated pair
force's derivative, bonds, angles, the reciprocal part through the dipole
kernels)
against fourth-order central differences of the device's FP64 forces and
of the oracle's forces, (8 (F(+h) - F(-h)) - (F(+2h) - F(-2h))) / 12h along
u, within 1e-6 of the largest component (particles with a pair within
reach of the cutoff, where the truncated force jumps, left out); and the
product is linear and symmetric: v . (J u) = u . (J v).
"""
import numpy as np
import pytest

from molsim_gb300 import Engine, abi, configs
from molsim_gb300.engine import MolsimError
from tests.helpers import prepared

pytestmark = pytest.mark.gpu

CASES = [
    ("spme", dict(seed=81)),
    ("spme_surf", dict(seed=82, lsurf=1)),
    ("spme_n40", dict(seed=83, nmesh=40)),
    ("std_surf", dict(seed=84, ewald=abi.MG_EWALD_STD, ncut=6, lsurf=1)),
    ("no_ewald", dict(seed=85, ewald=abi.MG_EWALD_NONE)),
    ("bonds", dict(seed=86, chains=4, nseg=10)),
    ("bonds_angles", dict(seed=86, chains=4, nseg=10, angle_kt=1.0)),
    ("angles_p3", dict(seed=92, chains=3, nseg=8, angle_kt=0.6, angle_p=3, angle_eq=2.2)),
]


def _forces(e, s, x):
    L = s.boxlen
    e.SetPositions((x - L * np.round(x / L)).reshape(-1))
    e.NList("write")
    return e.UTotal()["forceo"]


def _near_cutoff(s, x, u, h):
    """Particles with a pair whose distance comes within 2 h |u| of rcut
    along the differences: the truncated force jumps there, so differences
    across it measure the jump, not the derivative."""
    L = s.boxlen
    d = x[:, None, :] - x[None, :, :]
    d -= L * np.round(d / L)
    r = np.sqrt((d * d).sum(-1))
    reach = 2.0 * h * (np.linalg.norm(u, axis=1)[:, None] + np.linalg.norm(u, axis=1)[None, :])
    close = np.abs(r - s.rcut) <= reach
    np.fill_diagonal(close, False)
    return close.any(1)


def _fd(e, s, x, u, h):
    f = lambda t: _forces(e, s, x + t * u)
    return (8.0 * (f(h) - f(-h)) - (f(2 * h) - f(-2 * h))) / (12.0 * h)


@pytest.mark.parametrize("name,kw", CASES, ids=[c[0] for c in CASES])
def test_jvp_matches_force_differences(name, kw, orc, gpu_lib):
    s = configs.small_system(**kw)
    s.utoltab, s.ftoltab = 1e-9, 1e-8   # tabulated forces the derivatives of the tabulated energy
    s = prepared(s, orc)
    x = s.ro.copy()
    rng = np.random.default_rng(kw["seed"])
    u = rng.normal(size=x.shape)
    g = Engine(s)
    _forces(g, s, x)
    jv = g.ForceJVP(u)
    h = 1e-4
    fd = _fd(g, s, x, u, h)
    scale = np.abs(jv).max()
    ok = ~_near_cutoff(s, x, u, h)
    assert ok.sum() >= len(ok) - 4
    assert np.abs(jv - fd)[ok].max() <= 1e-6 * scale, (name, np.abs(jv - fd)[ok].max() / scale)
    ref = Engine(s, lib=orc, prefix="orc_")
    fo = _fd(ref, s, x, u, h)
    assert np.abs(jv - fo)[ok].max() <= 1e-6 * scale, (name, np.abs(jv - fo)[ok].max() / scale)
    # symmetric (a Hessian) and linear
    v = rng.normal(size=x.shape)
    _forces(g, s, x)
    jw = g.ForceJVP(v)
    assert abs((v * jv).sum() - (u * jw).sum()) <= 1e-9 * np.abs(u * jw).sum()
    j2 = g.ForceJVP(2.5 * u - v)
    assert np.abs(j2 - (2.5 * jv - jw)).max() <= 1e-9 * scale
    g.close()
    ref.close()


def test_jvp_refuses_what_it_does_not_differentiate(orc, gpu_lib):
    cases = [(configs.small_system(seed=88, mode=abi.MG_MC), abi.MG_FP64),
             (configs.small_system(seed=89), abi.MG_MIXED),
             (configs.small_system(seed=90, txintlist=abi.MG_CELLLIST), abi.MG_FP64)]
    for s, form in cases:
        s = prepared(s, orc)
        e = Engine(s, form=form)
        e.SetPositions(s.ro_flat())
        e.NList("write")
        e.UTotal()
        with pytest.raises(MolsimError) as ex:
            e.ForceJVP(np.ones(s.ro.shape))
        assert abi.STATUS[ex.value.status] == "MG_ERR_UNSUPPORTED"
        e.close()
