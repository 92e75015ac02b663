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
