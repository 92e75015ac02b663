"""Gradient of the mean potential energy of a velocity-Verlet trajectory.

L(x0, v0) = 1/(n+1) sum_{k=0..n} U(x_k), where x_k follows the reference's
velocity Verlet (VelVer, md.F90:252-357) from positions x0 and velocities v0:

    x' = x + dt v + dt^2/2 a,   a' = forceo(x') / m,   v' = v + dt/2 (a + a')

The backward pass is the adjoint of these updates, run from the last step to
the first.  It needs the forces at every step and Hessian-vector products:
- The states (x, v, a) are stored every `checkpoint` steps on the forward
  pass. The backward pass recomputes one segment at a time from its
  checkpoint, so memory holds one segment, not the whole trajectory.
- The Hessian-vector products come from the device's derivative kernels
  (mg_force_jvp: the tabulated pair force's derivative, the bonds, the
  reciprocal part through the dipole kernels), hvp="analytic"; or, with
  hvp="fd", from central differences of the device forces,
  (forceo(x + eps u) - forceo(x - eps u)) / 2 eps, with eps scaled so that
  the largest displacement is 1e-5 A.

`TrajectoryFunction` exposes this to torch.autograd; its gradients are
dL/dx0 and dL/dv0.  `backward(cks, params=True)` also returns the gradients
with respect to the species' charges, sigma and epsilon: each state's
dU/dtheta (mg_grad) plus, at each force evaluation, the adjoint of the
acceleration times d(forceo)/dtheta (mg_force_pvjp).
"""
import numpy as np

from . import abi, units
from .engine import Engine


class Trajectory:
    """Velocity Verlet of a System through the GPU forces (FP64 form)."""

    def __init__(self, system, dt=0.002, nsteps=50, checkpoint=10, hvp_disp=1e-5, hvp="analytic"):
        if system.ubuf is None:
            system.build_table()
        if hvp not in ("analytic", "fd"):
            raise ValueError(f"hvp = {hvp!r}: 'analytic' or 'fd'")
        self.s = system
        self.dt, self.n, self.ck, self.hvp_disp, self.hvp = dt, nsteps, checkpoint, hvp_disp, hvp
        self.e = Engine(system, form=abi.MG_FP64)
        self.im = np.repeat(system.massip(), 3)          # inverse masses per coordinate
        self.L = system.boxlen

    def _wrap(self, x):
        x = x.reshape(-1, 3)
        return (x - self.L * np.round(x / self.L)).reshape(-1)

    def forces(self, x):
        """forceo (reference force scale) and U at positions x (flat)."""
        self.e.SetPositions(self._wrap(x))
        self.e.NList("write")
        r = self.e.UTotal()
        return r["forceo"].reshape(-1), r["u_tot"]

    def _step(self, x, v, a):
        dt = self.dt
        x1 = x + dt * v + 0.5 * dt * dt * a
        f1, u1 = self.forces(x1)
        a1 = f1 * self.im
        v1 = v + 0.5 * dt * (a + a1)
        return x1, v1, a1, u1

    def forward(self, x0, v0):
        """L and the checkpoints (x, v, a) every `checkpoint` steps."""
        f0, u0 = self.forces(x0)
        x, v, a = x0.copy(), v0.copy(), f0 * self.im
        usum, cks = u0, {0: (x.copy(), v.copy(), a.copy())}
        for k in range(1, self.n + 1):
            x, v, a, u = self._step(x, v, a)
            usum += u
            if k % self.ck == 0 and k < self.n:
                cks[k] = (x.copy(), v.copy(), a.copy())
        return usum / (self.n + 1), cks

    def _jtv(self, x, lam):
        """(d acc / dx)^T lam at x: acc = forceo * im and d forceo/dx is
        symmetric, so this is the force derivative along im * lam."""
        u = self.im * lam
        nrm = np.abs(u).max()
        if nrm == 0.0:
            return np.zeros_like(lam)
        if self.hvp == "analytic":
            self.e.SetPositions(self._wrap(x))
            self.e.NList("write")
            return self.e.ForceJVP(u).reshape(-1)
        eps = self.hvp_disp / nrm
        fp, _ = self.forces(x + eps * u)
        fm, _ = self.forces(x - eps * u)
        return (fp - fm) / (2.0 * eps)

    def _param_terms(self, x, w, lam):
        """At x: w dU/dtheta + (d acc / dtheta)^T lam, as dq (per
        particle), deps and dsig (per pair type)."""
        self.e.SetPositions(self._wrap(x))
        self.e.NList("write")
        g = self.e.Grad()
        out = dict(dq=w * g["phi"], deps=w * g["du_deps"], dsig=w * g["du_dsig"])
        u = self.im * lam
        if np.abs(u).max() > 0.0:
            pv = self.e.ForcePVJP(u)
            for k in out:
                out[k] = out[k] + pv[k]
        return out

    def backward(self, cks, params=False):
        """dL/dx0 and dL/dv0 by the adjoint of velocity Verlet; with params
        also the gradients with respect to the species' charges (dz),
        sigma (dsig) and epsilon (deps), and their per-particle and
        per-pair-type forms."""
        dt, w = self.dt, 1.0 / (self.n + 1)
        gp = None
        if params:
            gp = dict(dq=np.zeros(self.s.np_), deps=np.zeros(self.s.nptpt), dsig=np.zeros(self.s.nptpt))
        gx = np.zeros_like(cks[0][0])   # adjoints of x, v, a after the step being undone
        gv = np.zeros_like(gx)
        ga = np.zeros_like(gx)
        starts = sorted(cks)
        for si in range(len(starts) - 1, -1, -1):
            k0 = starts[si]
            k1 = starts[si + 1] if si + 1 < len(starts) else self.n
            # the segment's states, recomputed from its checkpoint
            xs, vs, as_ = [cks[k0][0]], [cks[k0][1]], [cks[k0][2]]
            for _ in range(k0, k1):
                x, v, a, _u = self._step(xs[-1], vs[-1], as_[-1])
                xs.append(x)
                vs.append(v)
                as_.append(a)
            for j in range(k1 - k0, 0, -1):
                xk = xs[j]
                # the loss term U(x_k): dU/dx = -forceo / FORCE_FAC
                f, _ = self.forces(xk)
                gx = gx - w * f / units.FORCE_FAC
                # v' = v + dt/2 a + dt/2 a'
                ga_tot = ga + 0.5 * dt * gv
                if params:   # U(x_k) and a' = acc(x_k; theta)
                    for key, val in self._param_terms(xk, w, ga_tot).items():
                        gp[key] += val
                gv_prev = gv.copy()
                ga_prev = 0.5 * dt * gv
                # a' = acc(x')
                gx = gx + self._jtv(xk, ga_tot)
                # x' = x + dt v + dt^2/2 a
                gv_prev = gv_prev + dt * gx
                ga_prev = ga_prev + 0.5 * dt * dt * gx
                gv, ga = gv_prev, ga_prev
                # gx carries over unchanged (dx'/dx = I)
        # step 0: the loss term U(x0) and a0 = acc(x0)
        x0 = cks[0][0]
        f0, _ = self.forces(x0)
        gx = gx - w * f0 / units.FORCE_FAC + self._jtv(x0, ga)
        if not params:
            return gx, gv
        for key, val in self._param_terms(x0, w, ga).items():
            gp[key] += val
        from .autograd import _species_grads
        dz, dsig, deps = _species_grads(self.s, dict(phi=gp["dq"], du_dsig=gp["dsig"], du_deps=gp["deps"]))
        gp.update(dz=dz, dsig_species=dsig, deps_species=deps)
        return gx, gv, gp

    def close(self):
        self.e.close()


def trajectory_function():
    """torch.autograd.Function over (x0, v0) for a Trajectory (imports torch
    lazily: only the Python side uses it)."""
    import torch

    class TrajectoryFunction(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x0, v0, traj):
            L, cks = traj.forward(x0.detach().cpu().numpy().reshape(-1).copy(),
                                  v0.detach().cpu().numpy().reshape(-1).copy())
            ctx.traj, ctx.cks, ctx.shape = traj, cks, x0.shape
            return torch.as_tensor(L, dtype=x0.dtype, device=x0.device)

        @staticmethod
        def backward(ctx, gout):
            gx, gv = ctx.traj.backward(ctx.cks)
            t = lambda g: torch.as_tensor(g, dtype=gout.dtype, device=gout.device).reshape(ctx.shape)
            return gout * t(gx), gout * t(gv), None

    return TrajectoryFunction
