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


def _setup():
    s = configs.small_system(seed=91, n=240, L=32.0, ewald=abi.MG_EWALD_SPM, nmesh=32, order=6)
    s.utoltab, s.ftoltab = 1e-9, 1e-8
    s.build_table()
    v0 = s.maxwell_velocities(seed=3)
    return s, s.ro_flat().copy(), v0


@pytest.mark.parametrize("hvp", ["analytic", "fd"])
def test_trajectory_gradient_matches_finite_differences(hvp, gpu_lib):
    """The backward pass with the Hessian-vector products of the derivative
    kernels (mg_force_jvp) or of central differences of the forces."""
    s, x0, v0 = _setup()
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
