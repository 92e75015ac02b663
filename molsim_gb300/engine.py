"""Python host mirror of the reference's hot-path subroutines.

`Engine` wraps one handle of the C ABI and exposes the reference's entry
points under their own names:

    NList('write')        NList(iWriteInput)      nlist.F90:553
    NList('step', dro)    NList(iSimulationStep)  nlist.F90:598-621
    UTotal()              UTotal                  energy.F90:280
    DUTotal(ip, rotm)     DUTotal                 denergy.F90:98
    MCUpdate()            MCUpdate                mc.F90:5203
    VelVer(n)             VelVer                  md.F90:252
    BDRun(n)              BDDriver step           bd.F90:53-59

Errors come back as the reference's Stop() conditions, raised as
`MolsimError` with the status name and the library's message.
"""
import ctypes as C

import numpy as np

from . import abi


class MolsimError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{abi.STATUS.get(status, status)}: {msg}")
        self.status = status


class Engine:
    """One system on one GPU (or, with lib/prefix, on a library exporting the
    same entry points)."""

    def __init__(self, system, form=abi.MG_FP64, lib=None, prefix="mg_"):
        self.system = system
        self.form = form
        self.lib = lib if lib is not None else abi.load_library()
        self.prefix = prefix
        self._params, self._keep = system.params(form)
        self.h = C.c_void_p()
        st = self._fn("create")(C.byref(self._params), C.byref(self.h))
        self._check(st, "create")
        self.np = system.np_
        self.nptpt = system.nptpt

    # ---- plumbing -----------------------------------------------------------
    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    def _check(self, st, what):
        if st == 0:
            return
        msg = ""
        if hasattr(self.lib, "mg_last_error") and self.prefix == "mg_":
            buf = C.create_string_buffer(512)
            self.lib.mg_last_error(self.h if self.h else None, buf, 512)
            msg = buf.value.decode(errors="replace")
        raise MolsimError(st, f"{what}: {msg}")

    def close(self):
        if self.h:
            if self.prefix == "mg_":
                self.lib.mg_destroy(self.h)
            else:
                fn = getattr(self.lib, self.prefix + "destroy")
                fn.argtypes = [C.c_void_p]
                fn.restype = None
                fn(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- state --------------------------------------------------------------
    def SetPositions(self, ro):
        ro = abi.as_f64(np.asarray(ro).reshape(-1))
        self._check(self._fn("set_positions")(self.h, abi.f64(ro)), "set_positions")

    def GetPositions(self):
        ro = np.zeros(3 * self.np)
        self._check(self._fn("get_positions")(self.h, abi.f64(ro)), "get_positions")
        return ro.reshape(self.np, 3)

    # ---- lists ---------------------------------------------------------------
    def NList(self, stage="write", drostep=None):
        """'write': build the Verlet or cell list from the current positions;
        'step': accumulate drostep and rebuild on the skin rule.  Returns
        whether the list was rebuilt."""
        if stage == "write":
            self._check(self._fn("nlist_set")(self.h), "nlist_set")
            return True
        reb = np.zeros(1, dtype=np.int32)
        d = None if drostep is None else abi.as_f64(np.asarray(drostep).reshape(-1))
        self._check(self._fn("nlist_update")(self.h, abi.f64(d), abi.i32(reb)), "nlist_update")
        return bool(reb[0])

    def NListCalls(self):
        """Verlet-list builds since NList('write'), counting it (VListAver's
        ncall, nlist.F90:953-986)."""
        n = np.zeros(1, dtype=np.int32)
        self._check(self.lib.mg_nlist_calls(self.h, abi.i32(n)), "nlist_calls")
        return int(n[0])

    def VList(self, maxnneigh=None):
        """nneighpn(np), jpnlist as a list of neighbour arrays (1-based)."""
        maxn = maxnneigh or self.np
        nn = np.zeros(self.np, dtype=np.int32)
        jl = np.zeros(self.np * maxn, dtype=np.int32)
        self._check(self._fn("nlist_get")(self.h, abi.i32(nn), abi.i32(jl), maxn), "nlist_get")
        jl = jl.reshape(self.np, maxn)
        return nn, [jl[i, : nn[i]].copy() for i in range(self.np)]

    def CellList(self):
        nc = np.zeros(3, dtype=np.int32)
        cell = np.zeros(self.np, dtype=np.int32)
        self._check(self._fn("celllist_get")(self.h, abi.i32(nc), abi.i32(cell)), "celllist_get")
        return nc, cell

    # ---- energies -------------------------------------------------------------
    def UTotal(self):
        forceo = np.zeros(3 * self.np)
        ut = np.zeros(self.nptpt + 1)
        uo = np.zeros(4)
        self._check(self._fn("utotal")(self.h, abi.f64(forceo), abi.f64(ut), abi.f64(uo)), "utotal")
        return dict(forceo=forceo.reshape(self.np, 3), u_twob=ut, u_tot=uo[0], u_rec=uo[1],
                    u_bond=uo[2], virial=uo[3])

    def DUTotal(self, ipnptm, rotm):
        ip = abi.as_i32(np.atleast_1d(ipnptm))
        rt = abi.as_f64(np.asarray(rotm).reshape(-1))
        dtw = np.zeros(self.nptpt + 1)
        drec = np.zeros(1)
        dtot = np.zeros(1)
        ovl = np.zeros(1, dtype=np.int32)
        self._check(self._fn("dutotal")(self.h, len(ip), abi.i32(ip), abi.f64(rt), abi.f64(dtw),
                                        abi.f64(drec), abi.f64(dtot), abi.i32(ovl)), "dutotal")
        return dict(du_twob=dtw, du_rec=drec[0], du_tot=dtot[0]), bool(ovl[0])

    def MCUpdate(self):
        self._check(self._fn("accept")(self.h), "accept")

    def DUTotalBatch(self, ip, rtrial):
        ip = abi.as_i32(np.atleast_1d(ip))
        rt = abi.as_f64(np.asarray(rtrial).reshape(-1))
        du = np.zeros(len(ip))
        ovl = np.zeros(len(ip), dtype=np.int32)
        self._check(self.lib.mg_dutotal_batch(self.h, len(ip), abi.i32(ip), abi.f64(rt), abi.f64(du),
                                              abi.i32(ovl)), "dutotal_batch")
        return du, ovl.astype(bool)

    def Grad(self):
        """UTotal at the current positions with its parameter gradients:
        phi (dU/dq_i), du_deps and du_dsig per type pair, du_dbox (dU/dL_a
        for an affine stretch of the box)."""
        pp, keep = self.system.pot_params()
        phi = np.zeros(self.np)
        de = np.zeros(self.nptpt)
        ds = np.zeros(self.nptpt)
        db = np.zeros(3)
        self._check(self.lib.mg_grad(self.h, C.byref(pp), abi.f64(phi), abi.f64(de), abi.f64(ds), abi.f64(db)),
                    "grad")
        return dict(phi=phi, du_deps=de, du_dsig=ds, du_dbox=db)

    def ForceJVP(self, u):
        """d(forceo)/dx . u at the current positions (forceo units per A; the
        Hessian of UTotal times u, negated and scaled by force_fac), by
        hand-written derivative kernels (mg_force_jvp)."""
        u = abi.as_f64(np.asarray(u, dtype=np.float64).reshape(-1))
        jv = np.zeros(3 * self.np)
        self._check(self.lib.mg_force_jvp(self.h, abi.f64(u), abi.f64(jv)), "force_jvp")
        return jv.reshape(self.np, 3)

    def ForcePVJP(self, u):
        """u . d(forceo)/d(parameter) at the current positions: dq per
        particle charge, deps and dsig per pair type (Lorentz-Berthelot from
        the species), by hand-written kernels (mg_force_pvjp)."""
        pp, keep = self.system.pot_params()
        u = abi.as_f64(np.asarray(u, dtype=np.float64).reshape(-1))
        dq = np.zeros(self.np)
        de = np.zeros(self.nptpt)
        ds = np.zeros(self.nptpt)
        self._check(self.lib.mg_force_pvjp(self.h, C.byref(pp), abi.f64(u), abi.f64(dq), abi.f64(de),
                                           abi.f64(ds)), "force_pvjp")
        return dict(dq=dq, deps=de, dsig=ds)

    def VirialTensor(self):
        """dU/deps_ab (3x3) for an affine strain of the box and positions;
        its trace is UTotal's virial."""
        w = np.zeros(9)
        self._check(self.lib.mg_virial_tensor(self.h, abi.f64(w)), "virial_tensor")
        return w.reshape(3, 3)

    # ---- integrators ------------------------------------------------------------
    def MDSetup(self, tstep, rod, rodd=None):
        massip = self.system.massip()
        rod = abi.as_f64(np.asarray(rod).reshape(-1))
        rodd = abi.as_f64(np.zeros(3 * self.np) if rodd is None else np.asarray(rodd).reshape(-1))
        self._check(self._fn("md_setup")(self.h, tstep, abi.f64(massip), abi.f64(rod), abi.f64(rodd)),
                    "md_setup")

    def VelVer(self, nstep):
        forceo = np.zeros(3 * self.np)
        uo = np.zeros(4)
        rod = np.zeros(3 * self.np)
        rodd = np.zeros(3 * self.np)
        self._check(self._fn("md_run")(self.h, nstep, abi.f64(forceo), abi.f64(uo), abi.f64(rod),
                                       abi.f64(rodd)), "md_run")
        return dict(forceo=forceo.reshape(self.np, 3), u_tot=uo[0], u_rec=uo[1], u_bond=uo[2],
                    virial=uo[3], rod=rod.reshape(self.np, 3), rodd=rodd.reshape(self.np, 3))

    def BDSetup(self, tstep, iseed):
        f1, f2 = self.system.bd_factors(tstep)
        self._check(self._fn("bd_setup")(self.h, abi.f64(f1), abi.f64(f2), int(iseed)), "bd_setup")

    def EnergyTerms(self):
        """u%tot, u%twob(0), u%rec, u%bond, u%angle and the virial of the last
        UTotal or step."""
        t = np.zeros(6)
        self._check(self._fn("energy_terms")(self.h, abi.f64(t)), "energy_terms")
        return dict(u_tot=t[0], u_twob0=t[1], u_rec=t[2], u_bond=t[3], u_angle=t[4], virial=t[5])

    def BDRun(self, nstep):
        forceo = np.zeros(3 * self.np)
        uo = np.zeros(4)
        self._check(self._fn("bd_run")(self.h, nstep, abi.f64(forceo), abi.f64(uo)), "bd_run")
        return dict(forceo=forceo.reshape(self.np, 3), u_tot=uo[0], u_rec=uo[1], u_bond=uo[2],
                    virial=uo[3])

    def BDSeed(self):
        s = np.zeros(1, dtype=np.int32)
        self._check(self._fn("bd_get_seed")(self.h, abi.i32(s)), "bd_get_seed")
        return int(s[0])

    def BenchSteps(self, kind, nstep, flush_bytes=0):
        """Summed device ms of nstep integrator steps (kind 0 = MD, 1 = BD),
        L2 flushed before each step when flush_bytes > 0."""
        ms = np.zeros(1)
        self._check(self.lib.mg_bench_steps(self.h, int(kind), int(nstep), int(flush_bytes),
                                            abi.f64(ms)), "bench_steps")
        return float(ms[0])

    def StepKernels(self, kind):
        n = np.zeros(1, dtype=np.int32)
        self._check(self.lib.mg_step_kernels(self.h, int(kind), abi.i32(n)), "step_kernels")
        return int(n[0])

    # ---- timing ---------------------------------------------------------------------
    def PhaseReset(self, enable=True):
        self._check(self.lib.mg_phase_reset(self.h, int(enable)), "phase_reset")

    def PhaseTimes(self):
        ms = np.zeros(32)
        n = np.zeros(1, dtype=np.int32)
        names = C.create_string_buffer(1024)
        self._check(self.lib.mg_phase_times(self.h, abi.f64(ms), 32, abi.i32(n), names, 1024),
                    "phase_times")
        keys = names.value.decode().split(",") if n[0] else []
        return {k: float(ms[i]) for i, k in enumerate(keys)}
