"""Accuracy-driven choice of the SPME parameters.

`tune_spme(system, target)` picks the B-spline order and mesh of a System so
that the force RMS error of the chosen form, against a converged FP64
reference, stays at or below `target` (relative to the RMS force), and among
the settings that meet it takes the one whose UTotal runs fastest on this
GPU.  The real-space split stays the System's (alpha from erfc(alpha r_c)).

The reference is the same system at order 10 on a mesh twice the largest
candidate (capped at 256 per edge); candidates are orders 4-6 on power-of-two
meshes from 16 up to the reference's half.  Every candidate is measured, not
modelled: the error is the measured force difference and the cost the
measured device time of its UTotal.
"""
import dataclasses
import time

import numpy as np

from . import abi
from .engine import Engine


def _forces(s, form):
    e = Engine(s, form=form)
    e.SetPositions(s.ro_flat())
    e.NList("write")
    f = e.UTotal()["forceo"]
    return e, f


def _time_utotal(e, reps=5):
    e.UTotal()
    t = time.perf_counter()
    for _ in range(reps):
        e.UTotal()
    return 1e3 * (time.perf_counter() - t) / reps


def tune_spme(system, target=1e-5, form=abi.MG_MIXED, orders=(4, 5, 6), kmax=128):
    """Returns dict(order, nmesh, err, ms, candidates=[...])."""
    if system.ubuf is None:
        system.build_table()
    L = float(np.min(system.boxlen))
    kmin = 16
    # the coarsest mesh worth trying has a spacing of about 4 A
    k = kmin
    while k * 4.0 < L and k < kmax:
        k *= 2
    kref = min(256, 2 * kmax)
    ref = dataclasses.replace(system, order=10, nmesh=kref, ewald=abi.MG_EWALD_SPM)
    eref, fref = _forces(ref, abi.MG_FP64)
    eref.close()
    frms = np.sqrt((fref ** 2).mean())
    cands = []
    for order in orders:
        kk = max(kmin, k // 2)
        while kk <= min(kmax, kref // 2):
            if kk >= order:
                s = dataclasses.replace(system, order=order, nmesh=kk, ewald=abi.MG_EWALD_SPM)
                e, f = _forces(s, form)
                err = float(np.sqrt(((f - fref) ** 2).mean()) / frms)
                ms = _time_utotal(e) if err <= target else None
                e.close()
                cands.append(dict(order=order, nmesh=kk, err=err, ms=ms))
                if err <= target:
                    break      # finer meshes of this order only cost more
            kk *= 2
    ok = [c for c in cands if c["ms"] is not None]
    if not ok:
        raise RuntimeError(f"no SPME setting up to mesh {kmax} reaches force RMS {target:g}: "
                           + ", ".join(f"p{c['order']}/K{c['nmesh']}: {c['err']:.2e}" for c in cands))
    best = min(ok, key=lambda c: c["ms"])
    return dict(best, candidates=cands)


# ---- fast choice for many replicas ---------------------------------------------
# The SPME force error at order 6 with alpha from erfc(alpha r_c) = 1e-5
# follows err ~ A (alpha h)^6 (h the mesh spacing), with A growing as the
# salt concentration c falls (weaker forces, the same absolute error): the
# oracle's FP64 SPME against order 10 on a 256^3 mesh, 1 000 ions, measured
# A = 0.033 at 1 M, 0.092 at 0.1 M and 0.33 at 0.01 M, i.e. about
# 0.033 c^-0.5 (c in mol/L).
_ERR_A0 = 0.033
_ORDER = 6
_SAFETY = 0.85


def alpha_h_max(target, conc):
    """The largest alpha*h (order 6) for a force RMS error below target at
    salt concentration conc (mol/L), with a safety factor."""
    a = _ERR_A0 * max(conc, 1e-4) ** -0.5
    return _SAFETY * (target / a) ** (1.0 / _ORDER)


def choose_spme(system, conc, target=1e-5, kmax=256, rcuts=(12.0, 16.0, 24.0, 32.0, 48.0, 64.0, 96.0),
                ns_per_pair=0.25, ns_per_point=0.01):
    """Order 6 SPME settings for one replica without measuring it: for each
    real-space cutoff r_c (<= L/2; alpha from erfc(alpha r_c) = 1e-5) the
    smallest power-of-two mesh (16 to kmax) whose spacing meets
    alpha_h_max; among those, the one with the least modelled cost (pairs
    within r_c + skin against mesh points, meshes above 128 at 1.5x the cost
    per point for the line-pass FFT).  The default cost weights are the
    ones that gave the most box-steps per second over the 256-box replica
    set on a GB300 (0.01 ns per mesh point against 0.03, 0.1, 0.3, 1 and
    0.003, 0.001).  Returns dict(rcut, ualpha, order, nmesh, cost_ns)."""
    from .configs import alpha_for_erfc
    L = float(np.min(system.boxlen))
    vol = float(np.prod(system.boxlen))
    rho = system.np_ / vol
    ah = alpha_h_max(target, conc)
    best = None
    for rc in rcuts:
        if rc > 0.5 * L:
            break
        alpha = alpha_for_erfc(1e-5, rc)
        k = 16
        while k < kmax and L / k > ah / alpha:
            k *= 2
        if L / k > ah / alpha:
            continue
        pairs = system.np_ * rho * 4.0 / 3.0 * np.pi * (rc + system.drnlist) ** 3 / 2.0
        cost = pairs * ns_per_pair + k ** 3 * ns_per_point * (1.5 if k > 128 else 1.0)
        if best is None or cost < best["cost_ns"]:
            best = dict(rcut=rc, ualpha=alpha, order=_ORDER, nmesh=k, cost_ns=float(cost))
    if best is None:
        raise RuntimeError(f"no order-6 setting up to mesh {kmax} meets {target:g} for L = {L:.0f} A")
    return best
