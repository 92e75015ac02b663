"""GPU integrators against the oracle.

BD (BDStep, bd.F90:120-155): the device reproduces the reference's serial
GauRandom stream (mollib.F90:2739-2766) in parallel, so after n steps the
LCG seed must be identical and positions equal to rounding.  MD (VelVer,
md.F90:252-420): positions, velocities and energies after n steps.
"""
import ctypes as C

import numpy as np
import pytest

from molsim_gb300 import Engine, abi, configs
from tests.helpers import prepared, rel

pytestmark = pytest.mark.gpu


def _pair(s, orc, form=abi.MG_FP64):
    ref = Engine(s, lib=orc, prefix="orc_")
    gpu = Engine(s, form=form)
    for e in (ref, gpu):
        e.SetPositions(s.ro_flat())
        e.NList("write")
    return ref, gpu


@pytest.mark.parametrize("seed,nstep", [(12345, 1), (987654321, 6), (77, 3)])
def test_bd_stream_and_positions(seed, nstep, orc, gpu_lib):
    s = prepared(configs.small_system(seed=51, n=300, L=36.0, mode=abi.MG_BD), orc)
    ref, gpu = _pair(s, orc)
    for e in (ref, gpu):
        e.BDSetup(0.01, seed)
    r = ref.BDRun(nstep)
    g = gpu.BDRun(nstep)
    assert gpu.BDSeed() == ref.BDSeed()
    dpos = np.abs(gpu.GetPositions() - ref.GetPositions()).max()
    assert dpos <= 1e-9, dpos
    assert rel(g["u_tot"], r["u_tot"]) <= 1e-9


def test_bd_odd_deviate_count_carries_saved_value(orc, gpu_lib):
    """3*np odd: each step leaves one Box-Muller deviate saved for the next."""
    s = prepared(configs.small_system(seed=52, n=310, L=36.0, mode=abi.MG_BD), orc)
    assert (3 * s.np_) % 2 == 1
    ref, gpu = _pair(s, orc)
    for e in (ref, gpu):
        e.BDSetup(0.01, 4242)
    for _ in range(3):
        ref.BDRun(1)
        gpu.BDRun(1)
        assert gpu.BDSeed() == ref.BDSeed()
    assert np.abs(gpu.GetPositions() - ref.GetPositions()).max() <= 1e-9


def test_bd_zero_seed_rejected(orc, gpu_lib):
    s = prepared(configs.small_system(seed=53, n=200, L=30.0, mode=abi.MG_BD), orc)
    gpu = Engine(s)
    with pytest.raises(Exception):
        gpu.BDSetup(0.01, 0)


@pytest.mark.parametrize("ewald", [abi.MG_EWALD_SPM, abi.MG_EWALD_STD])
def test_md_trajectory(ewald, orc, gpu_lib):
    s = prepared(configs.small_system(seed=54, n=300, L=36.0, ewald=ewald, ncut=5), orc)
    v = s.maxwell_velocities(seed=9)
    ref, gpu = _pair(s, orc)
    for e in (ref, gpu):
        e.MDSetup(0.002, v)
    r = ref.VelVer(10)
    g = gpu.VelVer(10)
    assert np.abs(gpu.GetPositions() - ref.GetPositions()).max() <= 1e-9
    assert np.abs(g["rod"] - r["rod"]).max() <= 1e-9 * np.abs(r["rod"]).max()
    assert rel(g["u_tot"], r["u_tot"]) <= 1e-9
    assert rel(g["virial"], r["virial"]) <= 1e-9


def test_md_rebuilds_match(orc, gpu_lib):
    """A hot, small-skin run that rebuilds the Verlet list several times."""
    s = prepared(configs.small_system(seed=55, n=300, L=36.0, drnlist=0.3), orc)
    v = 20.0 * s.maxwell_velocities(seed=10)
    ref, gpu = _pair(s, orc)
    for e in (ref, gpu):
        e.MDSetup(0.002, v)
    ref.VelVer(15)
    gpu.VelVer(15)
    assert np.abs(gpu.GetPositions() - ref.GetPositions()).max() <= 1e-8
    nr, lr = ref.VList()
    ng, lg = gpu.VList()
    assert [sorted(x.tolist()) for x in lr] == [sorted(x.tolist()) for x in lg]


@pytest.mark.parametrize("form", [abi.MG_MIXED, abi.MG_FP64])
def test_bd_step_host_pinned_buffers_match_copies(form, orc, gpu_lib):
    """mg_bd_step_host with pinned host buffers runs the step graph whose
    kernels read and write those buffers in place; with pageable buffers it
    copies.  Both give the same positions, forces and energies, bit for bit,
    as steps of mg_bd_run."""
    torch = pytest.importorskip("torch")
    s = prepared(configs.small_system(seed=54, n=400, L=40.0, mode=abi.MG_BD, chains=2, nseg=10), orc)
    lib = abi.load_library()
    n3 = 3 * s.np_
    runs = []
    for kind in ("pinned", "pageable", "run"):
        e = Engine(s, form=form)
        e.SetPositions(s.ro_flat())
        e.NList("write")
        e.BDSetup(0.01, 2468)
        e.BDRun(0)   # initial forces
        if kind == "run":
            out = e.BDRun(4)
            runs.append((e.GetPositions().reshape(-1), out["forceo"].reshape(-1), out["u_tot"]))
            e.close()
            continue
        if kind == "pinned":
            ro = torch.from_numpy(e.GetPositions().reshape(-1).copy()).pin_memory()
            f = torch.zeros(n3, dtype=torch.float64).pin_memory()
            p_ro, p_f = C.cast(ro.data_ptr(), abi.PF64), C.cast(f.data_ptr(), abi.PF64)
        else:
            ro_np = e.GetPositions().reshape(-1).copy()
            f_np = np.zeros(n3)
            p_ro, p_f = abi.f64(ro_np), abi.f64(f_np)
        u = np.zeros(4)
        for _ in range(4):
            assert lib.mg_bd_step_host(e.h, p_ro, p_f, abi.f64(u)) == 0
        if kind == "pinned":
            runs.append((ro.numpy().copy(), f.numpy().copy(), u[0]))
        else:
            runs.append((ro_np.copy(), f_np.copy(), u[0]))
        e.close()
    (r0, f0, u0), (r1, f1, u1), (r2, f2, u2) = runs
    assert np.array_equal(r0, r1) and np.array_equal(r0, r2)
    assert np.array_equal(f0, f1) and np.array_equal(f0, f2)
    assert u0 == u1 == u2
