"""GPU neighbour lists against the oracle: cell grid and Verlet lists must be
identical as sets (SetVListMD ownership rule for MD/BD, full list for MC).

Reference: InitCellList/SetCellList (celllist.F90:76-410), SetVListMD/MC
(nlist.F90:724-890), NList rebuild rule (nlist.F90:598-621).
"""
import numpy as np
import pytest

from molsim_gb300 import Engine, abi, configs
from tests.helpers import prepared

pytestmark = pytest.mark.gpu


def _lists(e):
    nn, lists = e.VList()
    return [sorted(x.tolist()) for x in lists]


@pytest.mark.parametrize("mode", [abi.MG_MD, abi.MG_MC, abi.MG_BD])
def test_vlist_sets(mode, orc, gpu_lib):
    s = prepared(configs.small_system(seed=41, mode=mode, n=500, L=45.0), orc)
    ref = Engine(s, lib=orc, prefix="orc_")
    gpu = Engine(s)
    for e in (ref, gpu):
        e.SetPositions(s.ro_flat())
        e.NList("write")
    assert _lists(gpu) == _lists(ref)


def test_celllist_cells(orc, gpu_lib):
    s = prepared(configs.small_system(seed=42, txintlist=abi.MG_CELLLIST, n=800, L=60.0), orc)
    ref = Engine(s, lib=orc, prefix="orc_")
    gpu = Engine(s)
    for e in (ref, gpu):
        e.SetPositions(s.ro_flat())
        e.NList("write")
    nc_r, c_r = ref.CellList()
    nc_g, c_g = gpu.CellList()
    assert np.array_equal(nc_r, nc_g)
    assert np.array_equal(c_r, c_g)


def test_rebuild_rule_sequence(orc, gpu_lib):
    """Same rebuild decisions over a sequence of random displacements."""
    s = prepared(configs.small_system(seed=43, n=400, L=40.0, drnlist=1.0), orc)
    ref = Engine(s, lib=orc, prefix="orc_")
    gpu = Engine(s)
    for e in (ref, gpu):
        e.SetPositions(s.ro_flat())
        e.NList("write")
    rng = np.random.default_rng(5)
    ro = s.ro_flat().copy()
    nreb = 0
    for step in range(25):
        d = rng.normal(0, 0.08, ro.shape)
        ro = ro + d
        L = s.boxlen[0]
        ro = ro - L * np.round(ro / L)
        rb = []
        for e in (ref, gpu):
            e.SetPositions(ro)
            rb.append(e.NList("step", d))
        assert rb[0] == rb[1], step
        assert _lists(gpu) == _lists(ref)
        nreb += rb[0]
    assert nreb >= 2
    # VListAver's ncall: the initial build and every rebuild
    assert gpu.NListCalls() == 1 + nreb


def test_rebuild_count_in_device_steps(orc, gpu_lib):
    """Rebuilds inside captured MD steps (the graph's conditional node) are
    counted on the device: the same count as the same steps launched one
    kernel at a time, where the host reads the rebuild flag."""
    s = prepared(configs.small_system(seed=44, n=300, L=36.0, drnlist=0.3), orc)
    v = s.maxwell_velocities(seed=3)
    counts = []
    for uncaptured in (True, False):
        gpu = Engine(s)
        gpu.SetPositions(s.ro_flat())
        gpu.NList("write")
        gpu.MDSetup(0.002, v)
        gpu.PhaseReset(uncaptured)
        gpu.VelVer(40)
        counts.append(gpu.NListCalls())
        gpu.close()
    assert counts[0] == counts[1] and counts[0] >= 3, counts
