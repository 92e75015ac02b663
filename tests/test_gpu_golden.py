"""The GPU against the committed golden fixture (tests/golden/), with no
oracle in the loop: plain FP64 UTotal at 1e-10, the Verlet list as a set,
BD (GauRandom state exact, positions to rounding) and velocity Verlet."""
import os

import numpy as np
import pytest

from molsim_gb300 import Engine, abi, configs
from tests.golden import make_golden
from tests.helpers import TOL_FP64, force_err, rel

pytestmark = pytest.mark.gpu

G = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_small.npz"))


def _system(kw):
    s = configs.small_system(**kw)
    s.build_table()              # the library's own table builder
    return s


@pytest.mark.parametrize("name", sorted(make_golden.CASES))
def test_utotal_matches_golden(name, gpu_lib):
    s = _system(make_golden.CASES[name])
    assert np.array_equal(s.ro_flat(), G[f"{name}/ro"])
    e = Engine(s)
    e.SetPositions(s.ro_flat())
    e.NList("write")
    r = e.UTotal()
    u_tot, u_rec, u_bond, vir = G[f"{name}/scalars"]
    assert rel(r["u_tot"], u_tot) <= TOL_FP64
    assert abs(r["u_rec"] - u_rec) <= TOL_FP64 * max(abs(u_rec), 1.0)
    assert abs(r["u_bond"] - u_bond) <= TOL_FP64 * max(abs(u_bond), 1e-12)
    assert rel(r["virial"], vir) <= TOL_FP64
    ut = G[f"{name}/u_twob"]
    assert np.all(np.abs(r["u_twob"] - ut) <= TOL_FP64 * np.maximum(np.abs(ut), 1e-12))
    assert force_err(r["forceo"].reshape(-1), G[f"{name}/forceo"]) <= TOL_FP64
    if f"{name}/pairs" in G.files:
        nn, lists = e.VList()
        pairs = sorted((min(i + 1, int(j)), max(i + 1, int(j))) for i, js in enumerate(lists) for j in js)
        assert np.array_equal(np.array(pairs, dtype=np.int32), G[f"{name}/pairs"])
    e.close()


def test_bd_matches_golden(gpu_lib):
    s = _system(make_golden.BD_CASE)
    assert np.array_equal(s.ro_flat(), G["bd/ro0"])
    e = Engine(s)
    e.SetPositions(s.ro_flat())
    e.NList("write")
    e.BDSetup(make_golden.BD_DT, make_golden.BD_SEED)
    e.BDRun(make_golden.BD_STEPS)
    assert e.BDSeed() == int(G["bd/seed"][0])
    assert np.abs(e.GetPositions().reshape(-1) - G["bd/ro"]).max() <= 1e-9


def test_md_matches_golden(gpu_lib):
    s = _system(make_golden.MD_CASE)
    rod = s.maxwell_velocities(seed=make_golden.MD_CASE["seed"])
    assert np.array_equal(rod, G["md/rod0"])
    e = Engine(s)
    e.SetPositions(s.ro_flat())
    e.NList("write")
    e.MDSetup(make_golden.MD_DT, rod)
    r = e.VelVer(make_golden.MD_STEPS)
    assert np.abs(e.GetPositions().reshape(-1) - G["md/ro"]).max() <= 1e-9
    assert np.abs(r["rod"].reshape(-1) - G["md/rod"]).max() <= 1e-9 * np.abs(G["md/rod"]).max()
    assert rel(r["u_tot"], G["md/scalars"][0]) <= 1e-9
