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
