"""Batched replicas: one CUDA graph per step for many independent systems.

Each replica in an ensemble runs the same kernels in the same order as when
it runs alone, so trajectories must agree bit for bit: positions,
velocities, energies and (BD) the GauRandom state.  The autotuner's choice
must meet its force-error target.
"""
import numpy as np
import pytest

from molsim_gb300 import Engine, abi, configs
from molsim_gb300.autotune import tune_spme
from molsim_gb300.ensemble import Ensemble

pytestmark = pytest.mark.gpu


def _replicas(mode, nrep=5):
    rs = configs.replica_set(seed=7, nrep=nrep, nmin=200, nmax=1000, cmin=0.3, cmax=1.0, mode=mode)
    for s in rs:
        s.build_table()
    return rs


def _engine(s, form):
    e = Engine(s, form=form)
    e.SetPositions(s.ro_flat())
    e.NList("write")
    return e


@pytest.mark.parametrize("form", [abi.MG_FP64, abi.MG_MIXED])
def test_md_ensemble_matches_replicas_alone(form, gpu_lib):
    rs = _replicas(abi.MG_MD)
    ens_e, alone = [], []
    for i, s in enumerate(rs):
        v = s.maxwell_velocities(seed=100 + i)
        for lst in (ens_e, alone):
            e = _engine(s, form)
            e.MDSetup(0.002, v)
            lst.append(e)
    ens = Ensemble(ens_e)
    ens.run(0, 25)
    for a, b in zip(ens_e, alone):
        rb = b.VelVer(25)
        ra = a.VelVer(0)
        assert np.array_equal(a.GetPositions(), b.GetPositions())
        assert np.array_equal(ra["rod"], rb["rod"])
        assert ra["u_tot"] == rb["u_tot"]
    # one ensemble step launches every replica's own step kernels
    assert ens.kernels(0) == sum(e.StepKernels(0) for e in alone)
    ens.close()


def test_bd_ensemble_matches_replicas_alone(gpu_lib):
    rs = _replicas(abi.MG_BD, nrep=4)
    ens_e, alone = [], []
    for i, s in enumerate(rs):
        for lst in (ens_e, alone):
            e = _engine(s, abi.MG_FP64)
            e.BDSetup(0.01, 1000 + i)
            lst.append(e)
    ens = Ensemble(ens_e)
    ens.run(1, 12)
    for a, b in zip(ens_e, alone):
        b.BDRun(12)
        a.BDRun(0)
        assert a.BDSeed() == b.BDSeed()
        assert np.array_equal(a.GetPositions(), b.GetPositions())
    ens.close()


def test_ensemble_requires_setup(gpu_lib):
    rs = _replicas(abi.MG_MD, nrep=2)
    es = [_engine(s, abi.MG_FP64) for s in rs]
    ens = Ensemble(es)
    with pytest.raises(Exception):
        ens.run(0, 1)            # no mg_md_setup
    ens.close()


def test_autotuner_meets_its_target(gpu_lib):
    s = configs.replica_set(seed=9, nrep=1, nmin=600, nmax=600, cmin=0.5, cmax=0.5)[0]
    target = 1e-5
    res = tune_spme(s, target=target, form=abi.MG_MIXED, kmax=128)
    assert res["err"] <= target, res["candidates"]
    ok = [c for c in res["candidates"] if c["err"] <= target]
    assert res["ms"] == min(c["ms"] for c in ok)
    # coarser settings that miss the target were measured and rejected
    assert any(c["err"] > target for c in res["candidates"]), res["candidates"]


@pytest.mark.parametrize("conc", [0.01, 0.1, 1.0])
def test_replica_chooser_meets_target(conc, gpu_lib):
    """The batched boxes' SPME chooser (order 6, cutoff and mesh per box):
    the mixed form's forces against a converged FP64 reference (order 10,
    twice the mesh up to 256) stay within the 1e-5 RMS target."""
    import dataclasses

    from molsim_gb300 import autotune
    s = configs.replica_set(seed=11, nrep=1, nmin=2000, nmax=2000, cmin=conc, cmax=conc)[0]
    ch = autotune.choose_spme(s, conc)
    s.rcut, s.ualpha, s.order, s.nmesh = ch["rcut"], ch["ualpha"], ch["order"], ch["nmesh"]
    s.build_table()
    ref = dataclasses.replace(s, order=10, nmesh=min(256, 2 * s.nmesh))
    fr = _engine(ref, abi.MG_FP64).UTotal()["forceo"]
    f = _engine(s, abi.MG_MIXED).UTotal()["forceo"]
    err = np.sqrt(((f - fr) ** 2).mean() / (fr ** 2).mean())
    assert err <= 1e-5, (ch, err)
