"""Parity at the measured configurations, GPU against the oracle (not GPU
against GPU).

  electrolyte_spme   32 768 ions, L = 817 A, SPME order 6 on 64^3, r_c = 12 A,
                     skin 2 A, MD
  polyelectrolyte    64 chains x 200 beads, 12 800 counterions, 20 000 salt
                     pairs (65 600 particles), L = 700 A, SPME order 6 on
                     128^3, r_c = 12 A, bonds, BD
  electrolyte_std    1 000 ions, L = 100 A, standard Ewald |n| <= 8, r_c = 30 A,
                     100 velocity-Verlet steps

Plain FP64 form: Verlet lists equal as sets (SetVListMD's ownership rule,
nlist.F90:724-765); UTotal energies, virial and forces within 1e-10
(energy.F90:280-430).  Mixed form: RMS and largest per-particle force error
and the energy error against the oracle's FP64 UTotal.  The oracle runs with
every host core (threads standing in for the reference's MPI ranks; its
Verlet list is the reference's O(N^2) loop split by rows).
"""
import os

import numpy as np
import pytest

from molsim_gb300 import Engine, abi, configs
from tests.helpers import TOL_FP64, TOL_MIXED_RMS, prepared, rel, utotal_errors

pytestmark = pytest.mark.gpu

MAXN = 96          # list width of both lists (the largest count here is about 30)
# mixed form, largest per-particle force error |dF_i| over the RMS force
TOL_MIXED_MAX = 2e-4


def _threads():
    return max(1, min(16, os.cpu_count() or 1))


def _rows(nn, jl):
    """Each particle's neighbour list sorted, padded with a sentinel."""
    jl = jl.reshape(len(nn), -1).copy()
    for i, n in enumerate(nn):
        jl[i, n:] = np.iinfo(np.int32).max
    return np.sort(jl, axis=1)


def _vlist(e, np_):
    nn = np.zeros(np_, dtype=np.int32)
    jl = np.zeros(np_ * MAXN, dtype=np.int32)
    e._check(e._fn("nlist_get")(e.h, abi.i32(nn), abi.i32(jl), MAXN), "nlist_get")
    return nn, _rows(nn, jl)


def _mixed_errors(g, r):
    d = g["forceo"] - r["forceo"]
    frms = np.sqrt((r["forceo"] ** 2).sum(1).mean())
    return dict(force_rms=float(np.sqrt((d * d).sum(1).mean()) / frms),
                force_max=float(np.sqrt((d * d).sum(1)).max() / frms),
                u_tot=rel(g["u_tot"], r["u_tot"]), u_rec=rel(g["u_rec"], r["u_rec"]),
                virial=rel(g["virial"], r["virial"]))


@pytest.fixture(scope="module", params=["electrolyte_spme", "polyelectrolyte"])
def config_case(request, orc):
    s = getattr(configs, request.param)()
    s.maxnneigh = MAXN
    prepared(s, orc)
    orc.orc_set_threads(_threads())
    try:
        ref = Engine(s, lib=orc, prefix="orc_")
        ref.SetPositions(s.ro_flat())
        ref.NList("write")
        r = ref.UTotal()
        lists = _vlist(ref, s.np_)
        ref.close()
    finally:
        orc.orc_set_threads(1)
    return request.param, s, r, lists


def test_config_vlist_sets(config_case, gpu_lib):
    name, s, _, (nn_r, rows_r) = config_case
    gpu = Engine(s)
    gpu.SetPositions(s.ro_flat())
    gpu.NList("write")
    nn_g, rows_g = _vlist(gpu, s.np_)
    assert np.array_equal(nn_g, nn_r), name
    assert np.array_equal(rows_g, rows_r), name
    assert nn_r.sum() > 0


def test_config_utotal_fp64(config_case, gpu_lib):
    name, s, r, _ = config_case
    gpu = Engine(s)
    gpu.SetPositions(s.ro_flat())
    gpu.NList("write")
    g = gpu.UTotal()
    e = utotal_errors(g, r, s.nptpt)
    bad = {k: v for k, v in e.items() if not v <= TOL_FP64}
    assert not bad, (name, bad, e)


def test_config_utotal_mixed(config_case, gpu_lib):
    name, s, r, _ = config_case
    gpu = Engine(s, form=abi.MG_MIXED)
    gpu.SetPositions(s.ro_flat())
    gpu.NList("write")
    g = gpu.UTotal()
    e = _mixed_errors(g, r)
    print(name, e)
    assert e["force_rms"] <= TOL_MIXED_RMS, (name, e)
    assert e["force_max"] <= TOL_MIXED_MAX, (name, e)
    assert e["u_tot"] <= 1e-5 and e["virial"] <= 1e-5, (name, e)


def test_electrolyte_std_md_100_steps(orc, gpu_lib):
    """The 1 000-ion standard-Ewald workload in full: UTotal of the initial
    configuration, then 100 velocity-Verlet steps (dt = 0.002 ps, Maxwell
    velocities at 298 K), positions, velocities and energies against the
    oracle's VelVer (md.F90:252-357)."""
    s = prepared(configs.electrolyte_std(), orc)
    v = s.maxwell_velocities(seed=11)
    ref = Engine(s, lib=orc, prefix="orc_")
    gpu = Engine(s)
    out0 = []
    for e in (ref, gpu):
        e.SetPositions(s.ro_flat())
        e.NList("write")
        out0.append(e.UTotal())
        e.MDSetup(0.002, v)
    e0 = utotal_errors(out0[1], out0[0], s.nptpt)
    assert max(e0.values()) <= TOL_FP64, e0
    r = ref.VelVer(100)
    g = gpu.VelVer(100)
    L = s.boxlen[0]
    dpos = gpu.GetPositions() - ref.GetPositions()
    dpos -= L * np.round(dpos / L)
    assert np.abs(dpos).max() <= 1e-8, np.abs(dpos).max()
    assert np.abs(g["rod"] - r["rod"]).max() <= 1e-8 * np.abs(r["rod"]).max()
    assert rel(g["u_tot"], r["u_tot"]) <= 1e-9
    assert rel(g["virial"], r["virial"]) <= 1e-9
