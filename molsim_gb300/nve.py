"""Energy conservation of velocity-Verlet MD (NVE drift) for a System.

`nve_drift(system, form)` starts from Maxwell velocities and the
accelerations of the initial forces (GetLinAcc, md.F90:601-625), runs the
device integrator (VelVer, md.F90:252-357) and samples the total energy
U + K every `every` steps.  The drift is the least-squares slope of the total
energy over time, reported in kJ/mol per ns and in kT per particle per ns.
Units: velocities in A/ps and masses in g/mol give K = 0.005 sum m v^2 kJ/mol;
forceo carries the reference's force scale, so acceleration = forceo / m.
"""
import numpy as np

from . import abi, units
from .engine import Engine


def nve_drift(system, form=abi.MG_FP64, nsteps=1000, dt=0.002, every=10, seed=1):
    if system.ubuf is None:
        system.build_table()
    e = Engine(system, form=form)
    e.SetPositions(system.ro_flat())
    e.NList("write")
    u = e.UTotal()
    m = 1.0 / system.massip()
    v = system.maxwell_velocities(seed=seed)
    acc = (u["forceo"] * system.massip()[:, None]).reshape(-1)
    e.MDSetup(dt, v, acc)
    t, etot = [0.0], [u["u_tot"] + 0.005 * float((m[:, None] * v.reshape(-1, 3) ** 2).sum())]
    for k in range(nsteps // every):
        r = e.VelVer(every)
        kin = 0.005 * float((m[:, None] * r["rod"] ** 2).sum())
        t.append((k + 1) * every * dt)
        etot.append(r["u_tot"] + kin)
    e.close()
    t, etot = np.array(t), np.array(etot)
    slope = np.polyfit(t, etot, 1)[0]                 # kJ/mol per ps
    kt = units.kT(system.temp)
    return dict(drift_kj_per_ns=1e3 * slope, drift_kt_per_particle_per_ns=1e3 * slope / (system.np_ * kt),
                e_std_kt_per_particle=float(np.std(etot)) / (system.np_ * kt), nsteps=nsteps, dt=dt,
                e_first=float(etot[0]), e_last=float(etot[-1]))
