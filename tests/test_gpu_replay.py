"""The compiled ABI caller (molsim_gb300/harness/mg_replay.cpp) against the
same sequences driven from Python and against the oracle.

mg_replay reads a system and a run from a file and drives the C ABI as the
reference's Fortran drivers would: VelVer steps, BDStep steps, and MC passes
of single-particle moves with the reference's Random generator and
Metropolis rule.  The same library driven through ctypes (the Engine, and
molsim_gb300.mc for the MC passes) must give the same bits; the oracle the
same numbers within the FP64 tolerance of the parity tests.
"""
import numpy as np
import pytest

from molsim_gb300 import Engine, abi, configs, replay
from molsim_gb300.mc import MCPass, MoveParams
from tests.helpers import prepared, rel

pytestmark = pytest.mark.gpu


def _engine(s, lib=None, prefix="mg_"):
    e = Engine(s) if lib is None else Engine(s, lib=lib, prefix=prefix)
    e.SetPositions(s.ro_flat())
    e.NList("write")
    return e


def test_replay_velver(tmp_path, orc, gpu_lib):
    s = prepared(configs.small_system(seed=81), orc)
    v = s.maxwell_velocities(seed=5)
    out = replay.run(str(tmp_path), s, abi.MG_FP64, "velver", 20, tstep=0.002, massip=s.massip(), rod=v,
                     rodd=np.zeros_like(v))
    e = _engine(s)
    e.MDSetup(0.002, v)
    r = e.VelVer(20)
    assert np.array_equal(out["ro"], e.GetPositions().reshape(-1))
    assert np.array_equal(out["rod"], r["rod"].reshape(-1))
    assert out["uout"][0] == r["u_tot"]
    o = _engine(s, orc, "orc_")
    o.MDSetup(0.002, v)
    ro_ = o.VelVer(20)
    assert rel(out["uout"][0], ro_["u_tot"]) <= 1e-9
    assert np.abs(out["ro"] - o.GetPositions().reshape(-1)).max() <= 1e-9


def test_replay_bdstep(tmp_path, orc, gpu_lib):
    s = prepared(configs.small_system(seed=82, mode=abi.MG_BD, chains=3, nseg=8), orc)
    f1, f2 = s.bd_factors(0.01)
    out = replay.run(str(tmp_path), s, abi.MG_FP64, "bdstep", 15, fac1=f1, fac2=f2, iseed=12345)
    e = _engine(s)
    e.BDSetup(0.01, 12345)
    r = e.BDRun(15)
    assert np.array_equal(out["ro"], e.GetPositions().reshape(-1))
    assert out["uout"][0] == r["u_tot"]
    assert int(out["iseed"][0]) == e.BDSeed()
    o = _engine(s, orc, "orc_")
    o.BDSetup(0.01, 12345)
    ro_ = o.BDRun(15)
    assert rel(out["uout"][0], ro_["u_tot"]) <= 1e-9
    assert int(out["iseed"][0]) == o.BDSeed()


@pytest.mark.parametrize("txintlist", [abi.MG_VLIST, abi.MG_CELLLIST], ids=["vlist", "cell"])
def test_replay_mc_passes(txintlist, tmp_path, orc, gpu_lib):
    s = prepared(configs.small_system(seed=83, mode=abi.MG_MC, txintlist=txintlist), orc)
    out = replay.run(str(tmp_path), s, abi.MG_FP64, "mc", 3, iseed=2024, dtran=1.0)
    for lib, prefix in ((None, "mg_"), (orc, "orc_")):
        e = _engine(s, lib, prefix)
        u0 = e.UTotal()["u_tot"]
        mc = MCPass(e, s, iseed=2024, params=MoveParams(pspart=1.0, dtran=1.0))
        for _ in range(3):
            mc.run_pass()
        assert mc.stats.accepted["spart"] == int(out["naccept"][0]), prefix
        assert np.array_equal(out["ro"], mc.ro.reshape(-1)), prefix
        assert abs(out["du_acc"][0] - mc.du_acc) <= 1e-9 * abs(u0)
        u1 = e.UTotal()["u_tot"]
        assert rel(out["uout"][0], u1) <= (0.0 if lib is None else 1e-10)
    assert out["naccept"][0] > 200
