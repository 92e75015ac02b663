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
# (none since the device FFT took meshes 2^a 3^b 5^c: mic.mc.ewspm.in's
# nmesh = 40 runs)
DEVICE_REFUSES = {}


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


MC_RUN = [e for e in RUN if e["method"] == "mc"]


@pytest.mark.parametrize("e", MC_RUN, ids=[e["input"] for e in MC_RUN])
def test_reference_input_mc_trials(e, orc, gpu_lib):
    """30 single-particle displacement trials (DUTotal, denergy.F90:98-215;
    steps up to 0.5 A or a fifth of the box)
    of the input's own system on the GPU and in the oracle, every other
    non-overlapping trial accepted (MCUpdate): du%tot within 1e-10 of the
    total energy's parts, the overlap flags equal."""
    s, ref, gpu = _engines(e, orc)
    u = ref.UTotal()
    gpu.UTotal()
    scale = max(abs(u["u_twob"][0]), 1.0) + max(abs(u["u_rec"]), 1.0)
    rng = np.random.default_rng(5)
    L = s.boxlen
    ro = s.ro.copy()
    nacc = nfree = 0
    for it in range(30):
        ip = int(rng.integers(s.np_))
        new = ro[ip] + rng.uniform(-1.0, 1.0, 3) * min(0.5, 0.2 * float(np.min(L)))
        new -= L * np.round(new / L)
        r, ovl_r = ref.DUTotal(np.array([ip + 1]), new[None])
        g, ovl_g = gpu.DUTotal(np.array([ip + 1]), new[None])
        assert ovl_g == ovl_r, it
        if ovl_r:
            continue
        assert abs(g["du_tot"] - r["du_tot"]) <= 1e-10 * scale, (e["input"], it)
        nfree += 1
        if nfree % 2 == 1:
            ref.MCUpdate()
            gpu.MCUpdate()
            ro[ip] = new
            nacc += 1
    assert nfree >= 10 and nacc >= 5
    assert np.array_equal(gpu.GetPositions(), ref.GetPositions())


@pytest.mark.parametrize("e", REFUSED, ids=[e["input"] for e in REFUSED])
def test_reference_input_refusal_names_the_variable(e):
    assert any(v in e["refused"] for v in ("natpt", "txelec", "txpot", "npot", "txbc", "txmethod", "iewaldopt",
                                           "txewaldrec", "txintlist", "dipain", "polain", "latweakcharge"))
