"""Edge cases of UTotal against the oracle: the smallest systems, a system
with a net charge, particles on the faces of the box, and a particle
outside the cell grid.

The reference handles each of these without a special case: two ions are an
ordinary system; a net charge only draws a warning (potential.F90:623-625),
the Ewald sums carry no neutralising background; a coordinate of exactly
-L/2 lies in the first cell; a coordinate at +L/2 or beyond gives a cell
index past the grid, which the reference does not check (celllist.F90:303)
and the library reports as MG_ERR_CELL.
"""
import numpy as np
import pytest

from molsim_gb300 import Engine, abi, configs
from molsim_gb300.engine import MolsimError
from molsim_gb300.system import Species, System
from tests.helpers import TOL_FP64, prepared, run_pair, utotal_errors

pytestmark = pytest.mark.gpu


def _system(ro, charges, L=30.0, **kw):
    sp = [Species("A", +1.0, 3.0, 0.2, mass=23.0), Species("B", -1.0, 3.0, 0.2, mass=35.45)]
    iptpn = np.where(np.asarray(charges) > 0, 1, 2).astype(np.int32)
    args = dict(rcut=9.0, drnlist=1.0, ewald=abi.MG_EWALD_SPM, ualpha=0.35, order=6, nmesh=16, relpermitt=78.0)
    args.update(kw)
    return System(species=sp, iptpn=iptpn, ro=np.asarray(ro, dtype=np.float64), boxlen=np.array([L, L, L]),
                  **args)


@pytest.mark.parametrize("ewald", ["spm", "std"])
def test_two_ions(ewald, orc, gpu_lib):
    kw = dict(ewald=abi.MG_EWALD_SPM) if ewald == "spm" else dict(ewald=abi.MG_EWALD_STD, ncut=6)
    s = prepared(_system([[-1.5, 0.2, 0.1], [2.0, -0.4, 0.3]], [1, -1], **kw), orc)
    r, g, _, _ = run_pair(s, orc)
    e = utotal_errors(g, r, s.nptpt)
    assert max(e.values()) <= TOL_FP64, e


@pytest.mark.parametrize("form", [abi.MG_FP64, abi.MG_MIXED])
def test_net_charge(form, orc, gpu_lib):
    s = configs.small_system(seed=51)
    s.iptpn = s.iptpn.copy()
    k = int(np.flatnonzero(s.iptpn == 2)[0])
    s.iptpn[k] = 1                      # one anion becomes a cation: net charge +2
    assert abs(s.az.sum() - 2.0) < 1e-12
    s = prepared(s, orc)
    r, g, _, _ = run_pair(s, orc, form=form)
    e = utotal_errors(g, r, s.nptpt)
    if form == abi.MG_FP64:
        assert max(e.values()) <= TOL_FP64, e
    else:
        assert e["force_rms"] <= 1e-5 and e["u_tot"] <= 1e-5, e


@pytest.mark.parametrize("txintlist", [abi.MG_VLIST, abi.MG_CELLLIST], ids=["vlist", "cell"])
def test_particles_on_the_lower_faces(txintlist, orc, gpu_lib):
    s = configs.small_system(seed=52, txintlist=txintlist)
    L = s.boxlen[0]
    # translate the periodic configuration so that particle 1 sits on the
    # face x = -L/2, particle 2 on y = -L/2 and particle 3 on z = -L/2
    ro = s.ro.copy()
    for m in range(3):
        ro[:, m] += -L / 2 - ro[m, m]
        ro[:, m] -= L * np.round(ro[:, m] / L) * (np.abs(ro[:, m]) > L / 2)
        ro[m, m] = -L / 2
    s.ro = ro
    s = prepared(s, orc)
    r, g, _, _ = run_pair(s, orc)
    e = utotal_errors(g, r, s.nptpt)
    assert max(e.values()) <= TOL_FP64, e


def test_particle_past_the_grid_is_reported(orc, gpu_lib):
    s = configs.small_system(seed=53, txintlist=abi.MG_CELLLIST)
    ro = s.ro.copy()
    ro[5, 2] = s.boxlen[2] / 2        # +L/2: one cell past the grid
    s.ro = ro
    s = prepared(s, orc)
    e = Engine(s)
    e.SetPositions(s.ro_flat())
    with pytest.raises(MolsimError) as ex:
        e.NList("write")
        e.UTotal()
    assert abi.STATUS[ex.value.status] == "MG_ERR_CELL"
    o = Engine(s, lib=orc, prefix="orc_")   # the oracle reports it the same way
    o.SetPositions(s.ro_flat())
    with pytest.raises(MolsimError) as ex:
        o.NList("write")
    assert abi.STATUS[ex.value.status] == "MG_ERR_CELL"
