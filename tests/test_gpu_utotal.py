"""GPU parity of UTotal (plain FP64 and mixed forms) against the CPU oracle.

Reference: UTotal, energy.F90:280-430 (pair loop, Ewald std/SPME, self,
surface, bonds, force epilogue).
"""
import numpy as np
import pytest

from molsim_gb300 import Engine, abi, configs
from tests.helpers import (TOL_FP64, TOL_MIXED_RMS, force_err, force_rms_err, prepared, rel,
                           run_pair, small_cases, utotal_errors)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,factory", small_cases(), ids=[c[0] for c in small_cases()])
def test_utotal_fp64(name, factory, orc, gpu_lib):
    s = prepared(factory(), orc)
    r, g, _, _ = run_pair(s, orc)
    e = utotal_errors(g, r, s.nptpt)
    bad = {k: v for k, v in e.items() if not v <= TOL_FP64}
    assert not bad, (bad, e)


@pytest.mark.parametrize("name,factory", small_cases()[:6], ids=[c[0] for c in small_cases()[:6]])
def test_utotal_mixed(name, factory, orc, gpu_lib):
    s = prepared(factory(), orc)
    r, g, _, _ = run_pair(s, orc, form=abi.MG_MIXED)
    e = utotal_errors(g, r, s.nptpt)
    assert e["force_rms"] <= TOL_MIXED_RMS and e["u_tot"] <= 1e-5 and e["virial"] <= 1e-5, e


@pytest.mark.parametrize("nmesh,order", [(40, 6), (96, 6), (60, 8)])
def test_utotal_mixed_generic_meshes(nmesh, order, orc, gpu_lib):
    """The mixed form on meshes 2^a 3^b 5^c that are not powers of two
    (line passes with radices 3 and 5, generic spread and gather): force RMS
    error against the FP64 oracle within the mixed form's bar, and the same
    bits on a second call."""
    s = prepared(configs.small_system(seed=34, nmesh=nmesh, order=order, n=600, L=50.0), orc)
    r, g, _, gpu = run_pair(s, orc, form=abi.MG_MIXED)
    e = utotal_errors(g, r, s.nptpt)
    assert e["force_rms"] <= TOL_MIXED_RMS and e["u_tot"] <= 1e-5 and e["virial"] <= 1e-5, e
    g2 = gpu.UTotal()
    assert np.array_equal(g["forceo"], g2["forceo"]) and g["u_tot"] == g2["u_tot"]


def test_mixed_is_bit_reproducible(orc, gpu_lib):
    s = prepared(configs.small_system(seed=31), orc)
    _, g1, _, gpu = run_pair(s, orc, form=abi.MG_MIXED)
    g2 = gpu.UTotal()
    assert np.array_equal(g1["forceo"], g2["forceo"])
    assert g1["u_tot"] == g2["u_tot"]


@pytest.mark.parametrize("nmesh,order", [(32, 4), (64, 6), (128, 8)])
def test_mixed_fused_planes_reproducible(nmesh, order, orc, gpu_lib):
    """The mixed form's spread inside the forward plane FFT (particles sorted
    by the z plane of their stamp corner, integer shared-memory atomics)
    gives the same bits on every call, in MD and BD handles, and agrees with
    the oracle."""
    for mode in (abi.MG_MD, abi.MG_BD):
        s = prepared(configs.small_system(seed=32, n=900, L=60.0, nmesh=nmesh, order=order, mode=mode,
                                          chains=6, nseg=20), orc)
        r, g1, _, gpu = run_pair(s, orc, form=abi.MG_MIXED)
        g2 = gpu.UTotal()
        assert np.array_equal(g1["forceo"], g2["forceo"]) and g1["u_tot"] == g2["u_tot"]
        e = utotal_errors(g1, r, s.nptpt)
        assert e["force_rms"] <= TOL_MIXED_RMS and e["u_tot"] <= 1e-5 and e["virial"] <= 1e-5, e


def test_mixed_fused_planes_crowded_windows(orc, gpu_lib):
    """Crowded plane windows in the fused spread: 14 000 particles on a 32^3
    mesh at order 6 put 2 500 to 2 700 (particle, plane) items into every
    plane's CTA.  Same bits on every call, and the oracle's energies and
    forces within the mixed form's bar."""
    s = prepared(configs.small_system(seed=33, n=16000, L=150.0, nmesh=32, order=6, mode=abi.MG_BD,
                                      chains=20, nseg=50), orc)
    r, g1, _, gpu = run_pair(s, orc, form=abi.MG_MIXED)
    g2 = gpu.UTotal()
    assert np.array_equal(g1["forceo"], g2["forceo"]) and g1["u_tot"] == g2["u_tot"]
    e = utotal_errors(g1, r, s.nptpt)
    assert e["force_rms"] <= TOL_MIXED_RMS and e["u_tot"] <= 1e-5 and e["virial"] <= 1e-5, e


def test_electrolyte_std_config(orc, gpu_lib):
    """The N=1000 standard-Ewald electrolyte (r_c = 30 A, |n| <= 8)."""
    s = prepared(configs.electrolyte_std(), orc)
    r, g, _, _ = run_pair(s, orc)
    e = utotal_errors(g, r, s.nptpt)
    bad = {k: v for k, v in e.items() if not v <= TOL_FP64}
    assert not bad, (bad, e)


@pytest.mark.parametrize("form", [abi.MG_FP64, abi.MG_MIXED])
def test_angle_energy_matches_oracle(form, orc, gpu_lib):
    """u%angle (UAngle) and the total through mg_energy_terms against the
    oracle: the bonded terms to 1e-10 in both forms (the mixed form computes
    them in FP64 too); the total and the virial to 1e-10 in FP64 and to 1e-5
    in the mixed form (its pair and mesh terms are FP32)."""
    s = prepared(configs.small_system(seed=26, chains=4, nseg=12, angle_kt=1.0, angle_eq=2.2, angle_p=3), orc)
    ref = Engine(s, lib=orc, prefix="orc_")
    gpu = Engine(s, form=form)
    out = []
    for e in (ref, gpu):
        e.SetPositions(s.ro_flat())
        e.NList("write")
        e.UTotal()
        out.append(e.EnergyTerms())
    r, g = out
    tol = 1e-10 if form == abi.MG_FP64 else 1e-5
    assert abs(g["u_angle"] - r["u_angle"]) <= 1e-10 * abs(r["u_angle"])
    # the chains are placed at the bond length, so u%bond is ~0: absolute bar
    assert abs(g["u_bond"] - r["u_bond"]) <= 1e-10 * abs(r["u_tot"])
    assert abs(g["u_tot"] - r["u_tot"]) <= tol * abs(r["u_tot"])
    assert abs(g["virial"] - r["virial"]) <= tol * abs(r["virial"])
