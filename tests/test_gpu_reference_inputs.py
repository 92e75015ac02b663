"""The reference's own test inputs on the GPU against the oracle.

tests/golden/reference_inputs.json holds the systems that the reference's
Testin/in namelist files describe (read by
molsim_gb300.reference_input.system_from_input; made by
tests/golden/make_reference_inputs.py), or the reason an input is refused.
Each system runs UTotal in the plain FP64 form on the GPU and in the oracle
(energies, virial and forces within 1e-10) and, for MD and BD inputs, a few
steps of its own integrator with its own time step (VelVer md.F90:252-357,
BDStep bd.F90:120-155).  A refused input must name the variable outside the
path.
"""
import json
import os

import numpy as np
import pytest

from molsim_gb300 import Engine, units
from molsim_gb300.engine import MolsimError
from molsim_gb300.system import System
from tests.helpers import TOL_FP64, rel, utotal_errors

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_inputs.json")
with open(FIXTURE) as _fh:
    ENTRIES = json.load(_fh)
RUN = [e for e in ENTRIES if "system" in e]
REFUSED = [e for e in ENTRIES if "refused" in e]

# inputs whose settings the device path does not take, with the variable named
DEVICE_REFUSES = {"mic.mc.ewspm.in": "nmesh = 40"}


def _engines(e, orc):
    s = System.from_dict(e["system"])
    s.build_table(orc.orc_pot_twobody_tab)
    ref = Engine(s, lib=orc, prefix="orc_")
    gpu = Engine(s)
    for x in (ref, gpu):
        x.SetPositions(s.ro_flat())
        x.NList("write")
    return s, ref, gpu


@pytest.mark.parametrize("e", RUN, ids=[e["input"] for e in RUN])
def test_reference_input_utotal(e, orc, gpu_lib):
    if e["input"] in DEVICE_REFUSES:
        s = System.from_dict(e["system"])
        s.build_table(orc.orc_pot_twobody_tab)
        with pytest.raises(MolsimError, match=DEVICE_REFUSES[e["input"]]):
            Engine(s)
        return
    s, ref, gpu = _engines(e, orc)
    r, g = ref.UTotal(), gpu.UTotal()
    err = utotal_errors(g, r, s.nptpt)
    # on a perfect lattice the forces cancel to rounding: scale their errors
    # by the Lennard-Jones force at r = sigma instead of by the largest force
    fscale = max([np.abs(r["forceo"]).max()] + [units.FORCE_FAC * 24.0 * sp.eps / sp.sigma
                                                 for sp in s.species if sp.sigma > 0])
    err["force_max"] = np.abs(g["forceo"] - r["forceo"]).max() / fscale
    err["force_rms"] = np.sqrt(((g["forceo"] - r["forceo"]) ** 2).mean()) / fscale
    bad = {k: v for k, v in err.items() if not v <= TOL_FP64}
    assert not bad, (e["input"], bad)


@pytest.mark.parametrize("e", [e for e in RUN if e["method"] in ("md", "bd") and e["input"] not in DEVICE_REFUSES],
                         ids=[e["input"] for e in RUN if e["method"] in ("md", "bd")
                              and e["input"] not in DEVICE_REFUSES])
def test_reference_input_steps(e, orc, gpu_lib):
    s, ref, gpu = _engines(e, orc)
    nstep = 5
    if e["method"] == "md":
        v = s.maxwell_velocities(seed=e["iseed"])
        for x in (ref, gpu):
            x.MDSetup(e["tstep"], v)
        r, g = ref.VelVer(nstep), gpu.VelVer(nstep)
    else:
        for x in (ref, gpu):
            x.BDSetup(e["tstep"], e["iseed"])
        r, g = ref.BDRun(nstep), gpu.BDRun(nstep)
        assert gpu.BDSeed() == ref.BDSeed()
    L = s.boxlen
    d = gpu.GetPositions() - ref.GetPositions()
    d -= L * np.round(d / L)
    assert np.abs(d).max() <= 1e-9, (e["input"], np.abs(d).max())
    assert rel(g["u_tot"], r["u_tot"]) <= 1e-9, e["input"]


@pytest.mark.parametrize("e", REFUSED, ids=[e["input"] for e in REFUSED])
def test_reference_input_refusal_names_the_variable(e):
    assert any(v in e["refused"] for v in ("natpt", "txelec", "txpot", "npot", "txbc", "txmethod", "iewaldopt",
                                           "txewaldrec", "txintlist", "dipain", "polain", "latweakcharge"))
