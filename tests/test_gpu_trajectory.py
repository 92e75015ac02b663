"""Backward pass through a 50-step velocity-Verlet trajectory.

L = mean potential energy over the 51 states of a trajectory from (x0, v0);
its gradient by the checkpointed adjoint (checkpoints every 10 steps) is
compared with central finite differences of the whole trajectory, with
steps of 1e-4 A for positions and 1e-4 of the RMS speed for velocities, to
1e-6 of the gradient's largest component.  The table is built to 1e-9 so
that the tabulated forces are the derivatives of the tabulated energy.
The Hessian-vector products come from the derivative kernels
(mg_force_jvp) or from differences of the forces.
"""
import numpy as np
import pytest

from molsim_gb300 import abi, configs
from molsim_gb300.trajectory import Trajectory, trajectory_function

pytestmark = pytest.mark.gpu


def _setup(**kw):
    s = configs.small_system(seed=91, n=240, L=32.0, ewald=abi.MG_EWALD_SPM, nmesh=32, order=6, **kw)
    s.utoltab, s.ftoltab = 1e-9, 1e-8
    s.build_table()
    v0 = s.maxwell_velocities(seed=3)
    return s, s.ro_flat().copy(), v0


@pytest.mark.parametrize("hvp,kw", [("analytic", {}), ("fd", {}),
                                    ("analytic", dict(chains=3, nseg=8, angle_kt=0.8))],
                         ids=["analytic", "fd", "analytic_bonds_angles"])
def test_trajectory_gradient_matches_finite_differences(hvp, kw, gpu_lib):
    """The backward pass with the Hessian-vector products of the derivative
    kernels (mg_force_jvp) or of central differences of the forces; also
    through chains with bonds and angles."""
    s, x0, v0 = _setup(**kw)
    tr = Trajectory(s, dt=0.002, nsteps=50, checkpoint=10, hvp=hvp)
    L, cks = tr.forward(x0, v0)
    gx, gv = tr.backward(cks)
    rng = np.random.default_rng(5)
    hv = 1e-4 * np.sqrt((v0 ** 2).mean())
    for k in rng.choice(x0.size, 4, replace=False):
        e = np.zeros_like(x0)
        e[k] = 1e-4
        fd = (tr.forward(x0 + e, v0)[0] - tr.forward(x0 - e, v0)[0]) / 2e-4
        assert abs(fd - gx[k]) <= 1e-6 * np.abs(gx).max(), (k, fd, gx[k])
    for k in rng.choice(v0.size, 2, replace=False):
        e = np.zeros_like(v0)
        e[k] = hv
        fd = (tr.forward(x0, v0 + e)[0] - tr.forward(x0, v0 - e)[0]) / (2 * hv)
        assert abs(fd - gv[k]) <= 1e-6 * np.abs(gv).max(), (k, fd, gv[k])
    tr.close()


def test_trajectory_autograd_and_checkpointing(gpu_lib):
    torch = pytest.importorskip("torch")
    s, x0, v0 = _setup()
    tr = Trajectory(s, dt=0.002, nsteps=50, checkpoint=10)
    fn = trajectory_function()
    x = torch.tensor(x0, dtype=torch.float64, requires_grad=True)
    v = torch.tensor(v0, dtype=torch.float64, requires_grad=True)
    L = fn.apply(x, v, tr)
    L.backward()
    # the same gradient with every state kept (one checkpoint per step)
    full = Trajectory(s, dt=0.002, nsteps=50, checkpoint=1)
    _, cks = full.forward(x0, v0)
    gx, gv = full.backward(cks)
    assert np.allclose(x.grad.numpy(), gx, rtol=0, atol=1e-12 * np.abs(gx).max())
    assert np.allclose(v.grad.numpy(), gv, rtol=0, atol=1e-12 * np.abs(gv).max())
    tr.close()
    full.close()


def _with_params(s, dz=None, dsig=None, deps=None):
    """The system with one species parameter changed and its table rebuilt."""
    import dataclasses
    sp = list(s.species)
    for k, d in ((0, dz), (1, dsig), (2, deps)):
        if d is not None:
            a, h = d
            f = ("charge", "sigma", "eps")[k]
            sp[a] = dataclasses.replace(sp[a], **{f: getattr(sp[a], f) + h})
    t = dataclasses.replace(s, species=sp, ubuf=None, iubuflow=None, r2umin=None, nugrid=None)
    t.utoltab, t.ftoltab = s.utoltab, s.ftoltab
    t.build_table()
    return t


def test_trajectory_parameter_gradients(gpu_lib):
    """dL/d(sigma, epsilon) of each species through a 20-step trajectory
    (dU/dtheta at every state from mg_grad, the acceleration adjoints times
    d(force)/dtheta from mg_force_pvjp) against central differences of L
    with the species parameter changed by 1e-4 of itself (tables rebuilt),
    within 1e-6 of the largest gradient of each kind.  The charges are
    checked along a direction that keeps the system neutral, all of them
    scaled by (1 + t): dL/dt = sum_a z_a dL/dz_a."""
    s, x0, v0 = _setup()
    tr = Trajectory(s, dt=0.002, nsteps=20, checkpoint=5)
    L0, cks = tr.forward(x0, v0)
    _, _, gp = tr.backward(cks, params=True)
    tr.close()

    def L_of(t):
        tt = Trajectory(t, dt=0.002, nsteps=20, checkpoint=5)
        val = tt.forward(x0, v0)[0]
        tt.close()
        return val

    for a in range(s.npt):
        h = 1e-4 * s.species[a].sigma
        fd = (L_of(_with_params(s, dsig=(a, h))) - L_of(_with_params(s, dsig=(a, -h)))) / (2 * h)
        assert abs(fd - gp["dsig_species"][a]) <= 1e-6 * np.abs(gp["dsig_species"]).max(), (a, fd, gp["dsig_species"])
        h = 1e-4 * s.species[a].eps
        fd = (L_of(_with_params(s, deps=(a, h))) - L_of(_with_params(s, deps=(a, -h)))) / (2 * h)
        assert abs(fd - gp["deps_species"][a]) <= 1e-6 * np.abs(gp["deps_species"]).max(), (a, fd, gp["deps_species"])
    # charges: every species scaled by (1 + t), d L / dt = sum_a z_a dL/dz_a
    def scaled(t):
        import dataclasses
        sp = [dataclasses.replace(x, charge=x.charge * (1.0 + t)) for x in s.species]
        u = dataclasses.replace(s, species=sp, ubuf=None, iubuflow=None, r2umin=None, nugrid=None)
        u.utoltab, u.ftoltab = s.utoltab, s.ftoltab
        u.build_table()
        return u
    h = 1e-4
    fd = (L_of(scaled(h)) - L_of(scaled(-h))) / (2 * h)
    an = sum(s.species[a].charge * gp["dz"][a] for a in range(s.npt))
    assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)
