"""PyTorch binding of UTotal and its gradients (the adjoint form).

`UTotalFunction.apply(ro, zat, sigat, epsat, boxlen, model)` returns the total
potential energy U of a System through the GPU path; its backward gives

    dU/dro     = -force                        (mg_utotal)
    dU/dzat_a  = sum over particles of type a of the site potential dU/dq_i
    dU/dsig_a  = sum_b dU/dsig_ab dsig_ab/dsig_a,  sig_ab = (sig_a + sig_b)/2
    dU/deps_a  = sum_b dU/deps_ab deps_ab/deps_a,  eps_ab = sqrt(eps_a eps_b)
    dU/dL_a    = the box gradient for an affine stretch        (mg_grad)

The species parameters enter the tabulated potential, so `Model` rebuilds
the table and the handle whenever they change; positions only move the
particles.  Only the Python side uses torch; the library API is the C ABI.
"""
import dataclasses

import numpy as np
import torch

from . import abi, units
from .engine import Engine
from .system import iptpt_matrix


class Model:
    """A System whose species parameters and box may be changed from torch."""

    def __init__(self, system, form=abi.MG_FP64):
        self.base = system
        self.form = form
        self._key = None
        self.engine = None
        self.system = None

    def engine_for(self, zat, sigat, epsat, boxlen):
        key = (tuple(zat), tuple(sigat), tuple(epsat), tuple(boxlen))
        if key != self._key:
            sp = [dataclasses.replace(s, charge=float(z), sigma=float(sg), eps=float(ep))
                  for s, z, sg, ep in zip(self.base.species, zat, sigat, epsat)]
            s = dataclasses.replace(self.base, species=sp, boxlen=np.asarray(boxlen, dtype=np.float64),
                                    ubuf=None, iubuflow=None, r2umin=None, nugrid=None)
            s.build_table()
            if self.engine is not None:
                self.engine.close()
            self.system = s
            self.engine = Engine(s, form=self.form)
            self._key = key
        return self.engine


def _species_grads(system, g):
    """Pair-type and per-particle gradients -> per-species gradients."""
    npt = system.npt
    pidx = iptpt_matrix(npt).reshape(npt, npt)
    sig = np.array([s.sigma for s in system.species])
    eps = np.array([s.eps for s in system.species])
    dz = np.array([g["phi"][system.iptpn == a + 1].sum() for a in range(npt)])
    dsig, deps = np.zeros(npt), np.zeros(npt)
    for a in range(npt):
        for b in range(npt):
            k = pidx[b, a] - 1
            dsig[a] += g["du_dsig"][k] * (1.0 if a == b else 0.5)
            deps[a] += g["du_deps"][k] * (1.0 if a == b else 0.5 * np.sqrt(eps[b] / eps[a]))
    return dz, dsig, deps


class UTotalFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, ro, zat, sigat, epsat, boxlen, model):
        e = model.engine_for(zat.detach().cpu().numpy(), sigat.detach().cpu().numpy(),
                             epsat.detach().cpu().numpy(), boxlen.detach().cpu().numpy())
        e.SetPositions(ro.detach().cpu().numpy().reshape(-1))
        e.NList("write")
        u = e.UTotal()
        g = e.Grad()
        dz, dsig, deps = _species_grads(model.system, g)
        dro = -u["forceo"] / units.FORCE_FAC
        dev, dt = ro.device, ro.dtype
        ctx.save_for_backward(torch.as_tensor(dro, dtype=dt, device=dev).reshape(ro.shape),
                              torch.as_tensor(dz, dtype=dt, device=dev),
                              torch.as_tensor(dsig, dtype=dt, device=dev),
                              torch.as_tensor(deps, dtype=dt, device=dev),
                              torch.as_tensor(g["du_dbox"], dtype=dt, device=dev))
        return torch.as_tensor(u["u_tot"], dtype=dt, device=dev)

    @staticmethod
    def backward(ctx, gout):
        dro, dz, dsig, deps, dbox = ctx.saved_tensors
        return gout * dro, gout * dz, gout * dsig, gout * deps, gout * dbox, None


def utotal(ro, zat, sigat, epsat, boxlen, model):
    """Differentiable total potential energy (see UTotalFunction)."""
    return UTotalFunction.apply(ro, zat, sigat, epsat, boxlen, model)
