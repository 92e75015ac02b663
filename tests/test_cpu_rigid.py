"""Rigid-body velocity Verlet (VelVer with lpolyatom, md.F90:252-420) on the
oracle (orc_rigid_move / orc_rigid_kick, orc_angvel_to_quavel) and the host
helpers of molsim_gb300/poly.py.

The reference's tests hold no rigid-body trajectories, so the oracle's
conventions are pinned by mechanics computed without it: a spherical top
without torque turns as ori(t) = ori(0) expm(t [w]x) (angular velocity in
the principal frame, atoms at ro + ori . ra), an asymmetric top keeps its
lab angular momentum ori . (I w) and its kinetic energy, a constant lab
torque spins a spherical top up as L = torque t, and rigid waters with
ions keep U + K over a run of UTotal forces.
"""
import ctypes as C

import numpy as np
import pytest

from molsim_gb300 import abi, configs, units
from molsim_gb300.poly import ori_to_qua, qua_to_ori
from tests.helpers import centre_lists

scipy_linalg = pytest.importorskip("scipy.linalg")


def skew(w):
    return np.array([[0.0, -w[2], w[1]], [w[2], 0.0, -w[0]], [-w[1], w[0], 0.0]])


class OracleRigid:
    """The VelVer state of np rigid particles on the oracle."""

    def __init__(self, orc, tstep, boxlen, massip, momp, ro, qua, rod, angvelo, tvvite=0.0, nvvite=2):
        self.orc, self.tstep, self.tvvite, self.nvvite = orc, tstep, tvvite, nvvite
        self.np = n = len(massip)
        self.boxlen = abi.as_f64(boxlen)
        self.massip, self.momp = abi.as_f64(massip), abi.as_f64(np.asarray(momp).reshape(-1))
        self.ro = abi.as_f64(np.array(ro, dtype=np.float64).reshape(-1)).copy()
        self.qua = abi.as_f64(np.array(qua, dtype=np.float64).reshape(-1)).copy()
        self.rod = abi.as_f64(np.array(rod, dtype=np.float64).reshape(-1)).copy()
        self.angvelo = abi.as_f64(np.array(angvelo, dtype=np.float64).reshape(-1)).copy()
        self.rodd = np.zeros(3 * n)
        self.quad = np.zeros(4 * n)
        self.quadd = np.zeros(4 * n)
        self.drostep = np.zeros(3 * n)
        self.ori = np.zeros(9 * n)
        assert orc.orc_angvel_to_quavel(n, abi.f64(self.qua), abi.f64(self.angvelo), abi.f64(self.quad)) == 0

    def move(self):
        assert self.orc.orc_rigid_move(self.np, self.tstep, abi.f64(self.boxlen), abi.f64(self.ro), abi.f64(self.qua),
                                       abi.f64(self.rod), abi.f64(self.rodd), abi.f64(self.quad),
                                       abi.f64(self.quadd), abi.f64(self.drostep), abi.f64(self.ori)) == 0

    def kick(self, forceo, torqueo):
        fo = abi.as_f64(np.asarray(forceo).reshape(-1))
        to = abi.as_f64(np.asarray(torqueo).reshape(-1))
        assert self.orc.orc_rigid_kick(self.np, self.tstep, self.tvvite, self.nvvite, abi.f64(self.massip),
                                       abi.f64(self.momp), abi.f64(self.qua), abi.f64(fo), abi.f64(to),
                                       abi.f64(self.rod), abi.f64(self.rodd), abi.f64(self.quad),
                                       abi.f64(self.quadd), abi.f64(self.angvelo)) == 0

    def prime(self, forceo, torqueo):
        """The accelerations of the current state: a kick of zero length
        (quad stays, GetLinAcc and GetAngAcc run)."""
        t, self.tstep = self.tstep, 0.0
        self.kick(forceo, torqueo)
        self.tstep = t

    def ori_np(self):
        """ori(3,3,np) column-major as (np, 3, 3) with atom = ro + ori @ ra."""
        return self.ori.reshape(-1, 3, 3).transpose(0, 2, 1)

    def angvel_now(self):
        """QuaVelToAngVel of the current quad (mollib.F90:2651-2669)."""
        q, d = self.qua.reshape(-1, 4), self.quad.reshape(-1, 4)
        return 2.0 * np.stack([-q[:, 3] * d[:, 2] + q[:, 0] * d[:, 1] + q[:, 2] * d[:, 3] - q[:, 1] * d[:, 0],
                               -q[:, 0] * d[:, 2] - q[:, 3] * d[:, 1] + q[:, 1] * d[:, 3] + q[:, 2] * d[:, 0],
                               q[:, 1] * d[:, 2] - q[:, 2] * d[:, 1] + q[:, 0] * d[:, 3] - q[:, 3] * d[:, 0]], 1)


def _rot(seed):
    q, r = np.linalg.qr(np.random.default_rng(seed).standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def test_quaternion_round_trip():
    for seed in range(20):
        o = _rot(seed)
        q = ori_to_qua(o[None])
        assert abs(np.linalg.norm(q) - 1.0) < 1e-14
        assert np.abs(qua_to_ori(q)[0] - o).max() < 1e-14


def test_oracle_qua_to_ori_matches_host(orc):
    rng = np.random.default_rng(4)
    q = rng.standard_normal((5, 4))
    q /= np.linalg.norm(q, axis=1)[:, None]
    st = OracleRigid(orc, 1e-3, [100.0] * 3, np.ones(5), np.ones((5, 3)), np.zeros((5, 3)), q, np.zeros((5, 3)),
                     np.zeros((5, 3)))
    st.move()   # no velocities: the quaternions only renormalise
    assert np.abs(st.ori_np() - qua_to_ori(q)).max() < 1e-15


def test_spherical_top_turns_about_its_body_axis(orc):
    """No torque, I = 1: w stays constant and ori(t) = ori(0) expm(t [w]x).
    The runs start from the accelerations of the initial state (GetAngAcc
    without torque: -|quad|^2 qua) rather than from zero as a simulation
    does, so that the error is that of the steps alone."""
    o0, w = _rot(1), np.array([0.7, -1.1, 0.4])
    dt, n = 1e-3, 2000
    st = OracleRigid(orc, dt, [100.0] * 3, [1.0], [[1.0, 1.0, 1.0]], [[0.0, 0.0, 0.0]], ori_to_qua(o0[None]),
                     [[0.0, 0.0, 0.0]], [w])
    st.prime(np.zeros(3), np.zeros(3))
    assert np.abs(st.quadd + float((st.quad ** 2).sum()) * st.qua).max() < 1e-15
    for _ in range(n):
        st.move()
        st.kick(np.zeros(3), np.zeros(3))
    exact = o0 @ scipy_linalg.expm(n * dt * skew(w))
    assert np.abs(st.ori_np()[0] - exact).max() < 1e-5
    assert np.abs(st.angvel_now()[0] - w).max() < 1e-6


def test_asymmetric_top_keeps_angular_momentum_and_energy(orc):
    """No torque, I = (1, 2, 3.5), w about no principal axis: the lab
    angular momentum ori . (I w) and 1/2 sum I w^2 stay constant while w
    itself precesses."""
    I = np.array([1.0, 2.0, 3.5])
    o0, w0 = _rot(2), np.array([0.9, 0.2, -0.6])
    dt = 5e-4
    st = OracleRigid(orc, dt, [100.0] * 3, [1.0], [I], [[0.0, 0.0, 0.0]], ori_to_qua(o0[None]), [[0.0, 0.0, 0.0]],
                     [w0])
    st.prime(np.zeros(3), np.zeros(3))
    L0 = o0 @ (I * w0)
    e0 = 0.5 * float((I * w0 * w0).sum())
    ws = []
    for k in range(8000):
        st.move()
        st.kick(np.zeros(3), np.zeros(3))
        if k % 400 == 399:
            w = st.angvel_now()[0]
            ws.append(w)
            assert np.abs(st.ori_np()[0] @ (I * w) - L0).max() < 2e-5 * np.linalg.norm(L0)
            assert abs(0.5 * float((I * w * w).sum()) - e0) < 2e-5 * e0
    assert np.ptp(np.array(ws), axis=0).max() > 0.1    # w precesses in the body frame


def test_constant_torque_spins_up_a_spherical_top(orc):
    """A constant lab torque on a top at rest: L(t) = torque t."""
    I, tq = 2.5, np.array([0.3, -0.2, 0.5])
    o0 = _rot(3)
    dt, n = 1e-3, 1500
    st = OracleRigid(orc, dt, [100.0] * 3, [1.0], [[I, I, I]], [[0.0, 0.0, 0.0]], ori_to_qua(o0[None]),
                     [[0.0, 0.0, 0.0]], [[0.0, 0.0, 0.0]], nvvite=3)
    for _ in range(n):
        st.move()
        st.kick(np.zeros(3), tq)
    w_lab = st.ori_np()[0] @ st.angvel_now()[0]
    assert np.abs(I * w_lab - tq * n * dt).max() < 1e-3 * np.linalg.norm(tq * n * dt)


def test_linear_motion_and_pbc(orc):
    """Constant force: after the first step (rodd starts at zero, as MDDriver
    sets it) the velocity grows by a dt per step; centres stay in the box."""
    L, dt = 10.0, 0.01
    a = np.array([1.0, -2.0, 0.5])
    st = OracleRigid(orc, dt, [L] * 3, [0.5], [[0.0, 0.0, 0.0]], [[4.9, -4.9, 0.0]], [[1.0, 0.0, 0.0, 0.0]],
                     [[30.0, -20.0, 5.0]], [[0.0, 0.0, 0.0]])
    f = a / 0.5
    x = np.array([4.9, -4.9, 0.0])
    v = np.array([30.0, -20.0, 5.0])
    acc = np.zeros(3)
    for _ in range(300):
        st.move()
        x = x + dt * v + 0.5 * dt * dt * acc
        st.kick(f, np.zeros(3))
        v = v + 0.5 * dt * (a + acc)
        acc = a
        assert np.all(np.abs(st.ro) <= 0.5 * L)
    d = st.ro - x
    assert np.abs(d - L * np.round(d / L)).max() < 1e-10
    assert np.abs(st.rod - v).max() < 1e-10


def _water_system(orc, nw=40, ns=4, L=13.0):
    s = configs.water_ions(seed=21, nwater=nw, nsalt=ns, L=L, rcut=6.0)
    s.relpermitt = 78.0
    s.ewald, s.ualpha, s.ncut = abi.MG_EWALD_STD, 0.5, 8
    s = s.principal_axes()
    s.build_table(orc.orc_pot_twobody_tab)
    return s


def _initial_velocities(s, temp=298.0, seed=5):
    """Maxwell velocities and principal-frame angular velocities at temp."""
    rng = np.random.default_rng(seed)
    massip, momp = s.rigid_props()
    kt = units.GasConstant * temp * 1e-3                      # kJ/mol
    v = rng.standard_normal((s.np_, 3)) * np.sqrt(kt * massip / 0.01)[:, None]
    w = np.where(momp > 0.0, rng.standard_normal(momp.shape) * np.sqrt(kt / (0.01 * np.maximum(momp, 1e-300))), 0.0)
    return v, w


def oracle_rigid_utotal(orc, s, ro, ori):
    """UTotal of the polyatomic system at centres ro and orientations ori
    on the oracle, forces and torques by the epilogue."""
    from tests.test_cpu_poly import oracle_poly_utotal
    s.ro, s.ori = np.ascontiguousarray(ro), np.ascontiguousarray(ori)
    nn, jl, maxn = centre_lists(s.ro, s.boxlen[0], s.rcut + 1.0)
    out = oracle_poly_utotal(orc, s, nn, jl, maxn)
    p = s.params()
    fo = np.zeros(3 * s.np_)
    to = np.zeros(3 * s.np_)
    vm = np.zeros(1)
    r = s.atom_positions()
    assert orc.orc_poly_epilogue(C.byref(p), abi.f64(abi.as_f64(s.ro.reshape(-1))), abi.f64(r.reshape(-1)),
                                 abi.f64(abi.as_f64(out["force"].reshape(-1))), None, units.FORCE_FAC, abi.f64(fo),
                                 abi.f64(to), abi.f64(vm)) == 0
    return out["u_tot"], fo.reshape(-1, 3), to.reshape(-1, 3)


def oracle_rigid_run(orc, s, v, w, dt, nsteps, prime=True):
    """nsteps of VelVer on the oracle from centres s.ro, orientations s.ori,
    velocities v and angular velocities w; prime starts from the
    accelerations of the initial forces instead of zero.  Returns the state
    and per step (u, translational K, rotational K)."""
    massip, momp = s.rigid_props()
    st = OracleRigid(orc, dt, s.boxlen, massip, momp, s.ro, ori_to_qua(s.ori), v, w)
    if prime:
        u, fo, to = oracle_rigid_utotal(orc, s, s.ro.copy(), s.ori.copy())
        st.prime(fo, to)
    e = []
    for _ in range(nsteps):
        st.move()
        u, fo, to = oracle_rigid_utotal(orc, s, st.ro.reshape(-1, 3), st.ori_np())
        st.kick(fo, to)
        e.append((u, *s.kinetic_energy(st.rod, st.angvel_now())))
    return st, np.array(e)


def test_waters_conserve_energy(orc):
    """40 rigid waters and 8 ions (Ewald, eps_r 78) relaxing from random
    placements (U falls by 85 kJ/mol in 0.1 ps): with 0.5 fs steps U + K
    stays within 0.3 % of K, and halving the step changes it by less than
    0.01 kJ/mol (what moves it, steps of about 0.05 kJ/mol, is the LJ
    energy of particle pairs crossing the centre cutoff).  Started from zero
    accelerations, as the reference starts, the first half-kick costs an
    offset of order tstep instead."""
    s = _water_system(orc)
    v, w = _initial_velocities(s)
    k0 = sum(s.kinetic_energy(v, w))
    _, e1 = oracle_rigid_run(orc, s, v, w, 0.0005, 200)
    s = _water_system(orc)
    _, e2 = oracle_rigid_run(orc, s, v, w, 0.00025, 400)
    t1, t2 = e1.sum(1), e2.sum(1)[1::2]
    assert e1[-1, 0] < e1[0, 0] - 50.0
    assert np.abs(t1 - t1[0]).max() < 3e-3 * k0, (np.abs(t1 - t1[0]).max(), k0)
    assert np.abs(t1 - t2).max() < 1e-2, np.abs(t1 - t2).max()
    s = _water_system(orc)
    _, e0 = oracle_rigid_run(orc, s, v, w, 0.0005, 40, prime=False)
    assert e0.sum(1)[0] < t1[0] - 0.05
