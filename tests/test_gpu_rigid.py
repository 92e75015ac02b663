"""Rigid-body velocity Verlet on the GPU (mg_poly_rigid_*) against the oracle
(orc_rigid_move / orc_rigid_kick), VelVer with lpolyatom (md.F90:252-420).

Step by step with the same forces and torques: centres, orientation
matrices, drostep, velocities, angular velocities, quaternions and their
velocities within 1e-12 (the kernels contract products into fused
multiply-adds, the oracle does not).  Whole runs through PolyEngine.VelVer
(device UTotal each step) against oracle runs (oracle UTotal) over 20 steps
within 1e-9; a larger system keeps U + K over 400 steps.
"""
import numpy as np
import pytest

from molsim_gb300 import abi, configs
from molsim_gb300.poly import PolyEngine, ori_to_qua
from tests.test_cpu_rigid import OracleRigid, _initial_velocities, _water_system, oracle_rigid_run

pytestmark = pytest.mark.gpu


def _engine(s):
    return PolyEngine(s, maxnneigh=256)


@pytest.mark.parametrize("nvvite,tvvite", [(2, 0.0), (4, 0.5)])
def test_rigid_steps_match_oracle(nvvite, tvvite, orc, gpu_lib):
    s = _water_system(orc)
    v, w = _initial_velocities(s, seed=7)
    massip, momp = s.rigid_props()
    dt = 0.0005
    e = _engine(s)
    e.RigidSetup(dt, v, w, tvvite=tvvite, nvvite=nvvite, prime=False)
    u0 = e.UTotal()
    assert gpu_lib.mg_poly_rigid_prime(e.h, abi.f64(abi.as_f64(u0["forceo"].reshape(-1))),
                                       abi.f64(abi.as_f64(u0["torqueo"].reshape(-1)))) == 0
    st = OracleRigid(orc, dt, s.boxlen, massip, momp, s.ro, ori_to_qua(s.ori), v, w, tvvite=tvvite, nvvite=nvvite)
    st.prime(u0["forceo"], u0["torqueo"])
    n = s.np_
    ro, ori, dro = np.zeros(3 * n), np.zeros(9 * n), np.zeros(3 * n)
    rod, angv = np.zeros(3 * n), np.zeros(3 * n)
    for _ in range(15):
        assert gpu_lib.mg_poly_rigid_move(e.h, abi.f64(ro), abi.f64(ori), abi.f64(dro)) == 0
        st.move()
        assert np.abs(ro - st.ro).max() < 1e-12
        assert np.abs(ori - st.ori).max() < 1e-12
        assert np.abs(dro - st.drostep).max() < 1e-12
        s.ro = ro.reshape(n, 3).copy()
        s.ori = np.ascontiguousarray(ori.reshape(n, 3, 3).transpose(0, 2, 1))
        u = e.UTotal()
        fo = abi.as_f64(u["forceo"].reshape(-1))
        to = abi.as_f64(u["torqueo"].reshape(-1))
        assert gpu_lib.mg_poly_rigid_kick(e.h, abi.f64(fo), abi.f64(to), abi.f64(rod), abi.f64(angv)) == 0
        st.kick(fo, to)
        assert np.abs(rod - st.rod).max() < 1e-12 * max(1.0, np.abs(st.rod).max())
        assert np.abs(angv - st.angvelo).max() < 1e-12 * max(1.0, np.abs(st.angvelo).max())
        q, qd = e.RigidState()
        assert np.abs(q.reshape(-1) - st.qua).max() < 1e-12
        assert np.abs(qd.reshape(-1) - st.quad).max() < 1e-12 * max(1.0, np.abs(st.quad).max())
    e.close()


def test_rigid_velver_run_matches_oracle_run(orc, gpu_lib):
    """20 steps of PolyEngine.VelVer (device UTotal, device centre list)
    against 20 oracle steps (oracle UTotal): centres and orientations within
    1e-9, the last step's energy within 1e-9 relative."""
    s = _water_system(orc)
    v, w = _initial_velocities(s, seed=8)
    ref_sys = _water_system(orc)
    st, eo = oracle_rigid_run(orc, ref_sys, v, w, 0.0005, 20, prime=True)
    e = _engine(s)
    e.RigidSetup(0.0005, v, w, prime=True)
    out = e.VelVer(20)
    assert np.abs(s.ro.reshape(-1) - st.ro).max() < 1e-9
    assert np.abs(s.ori - st.ori_np()).max() < 1e-9
    assert abs(out["u_tot"] - eo[-1, 0]) <= 1e-9 * abs(eo[-1, 0]) + 1e-9
    assert np.abs(out["rod"].reshape(-1) - st.rod).max() < 1e-8
    e.close()


def test_rigid_waters_keep_energy(gpu_lib):
    """300 waters and 20 ions, SPME, 0.5 fs steps from the accelerations of
    the initial forces: U + K over 400 steps stays within 0.5 % of K."""
    s = configs.water_ions(seed=31, nwater=300, nsalt=10, L=24.0, rcut=9.0)
    s.relpermitt = 78.0
    s.ewald, s.ualpha, s.order, s.nmesh = abi.MG_EWALD_SPM, 0.35, 6, 32
    s = s.principal_axes()
    s.build_table(gpu_lib.mg_pot_twobody_tab)
    v, w = _initial_velocities(s, seed=9)
    k0 = sum(s.kinetic_energy(v, w))
    e = _engine(s)
    e.RigidSetup(0.0005, v, w, prime=True)
    u0 = e.UTotal()["u_tot"]
    tot = [u0 + k0]
    for _ in range(40):
        out = e.VelVer(10)
        tot.append(out["u_tot"] + sum(s.kinetic_energy(out["rod"], out["angvelo"])))
    tot = np.array(tot)
    assert np.abs(tot - tot[0]).max() < 5e-3 * k0, (np.abs(tot - tot[0]).max(), k0)
    e.close()


@pytest.mark.parametrize("ewald", ["spm", "none"])
def test_device_md_run_matches_host_steps(ewald, orc, gpu_lib):
    """mg_poly_md_run (every step on the device) against PolyEngine.VelVer
    (the host between the parts of each step) from the same state: ten
    steps, centres and orientations within 1e-9, the last step's u%tot and
    virial within 1e-9 relative."""
    def system():
        s = configs.water_ions(seed=51, nwater=200, nsalt=10, L=22.0, rcut=9.0)
        s.relpermitt = 78.0
        if ewald == "spm":
            s.ewald, s.ualpha, s.order, s.nmesh = abi.MG_EWALD_SPM, 0.35, 6, 32
        s = s.principal_axes()
        s.build_table(orc.orc_pot_twobody_tab)
        return s
    a, b = system(), system()
    v, w = _initial_velocities(a, seed=4)
    ea, eb = _engine(a), _engine(b)
    ea.RigidSetup(0.0005, v, w, prime=True)
    eb.RigidSetup(0.0005, v, w, prime=True)
    ra = ea.VelVer(10)
    rb = eb.MDRun(10)
    assert np.abs(a.ro - b.ro).max() < 1e-9
    assert np.abs(a.ori - b.ori).max() < 1e-9
    assert np.abs(ra["rod"] - rb["rod"]).max() < 1e-8
    assert abs(ra["u_tot"] - rb["u_tot"]) <= 1e-9 * max(abs(ra["u_tot"]), 1.0)
    assert abs(ra["virial"] - rb["virial"]) <= 1e-9 * max(abs(ra["virial"]), 1.0)
    ea.close()
    eb.close()


def test_device_md_run_graph_replays_the_step(orc, gpu_lib):
    """mg_poly_md_run launches its first step and replays one captured step
    graph for the rest: one ten-step call and ten one-step calls (each step
    launched as a first step) give the same bits."""
    def system():
        s = configs.water_ions(seed=52, nwater=150, nsalt=8, L=20.0, rcut=9.0)
        s.relpermitt = 78.0
        s.ewald, s.ualpha, s.order, s.nmesh = abi.MG_EWALD_SPM, 0.35, 6, 32
        s = s.principal_axes()
        s.build_table(orc.orc_pot_twobody_tab)
        return s
    a, b = system(), system()
    v, w = _initial_velocities(a, seed=5)
    ea, eb = _engine(a), _engine(b)
    ea.RigidSetup(0.0005, v, w, prime=True)
    eb.RigidSetup(0.0005, v, w, prime=True)
    ra = ea.MDRun(10)
    for _ in range(10):
        rb = eb.MDRun(1)
    assert np.array_equal(a.ro, b.ro) and np.array_equal(a.ori, b.ori)
    assert np.array_equal(ra["rod"], rb["rod"])
    assert ra["u_tot"] == rb["u_tot"] and ra["virial"] == rb["virial"]
    ea.close()
    eb.close()
