"""GPU parity of UTotal (plain FP64 and mixed forms) against the CPU oracle.

Reference: UTotal, energy.F90:280-430 (pair loop, Ewald std/SPME, self,
surface, bonds, force epilogue).
"""
import numpy as np
import pytest

from molsim_gb300 import abi, configs
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


def test_mixed_is_bit_reproducible(orc, gpu_lib):
    s = prepared(configs.small_system(seed=31), orc)
    _, g1, _, gpu = run_pair(s, orc, form=abi.MG_MIXED)
    g2 = gpu.UTotal()
    assert np.array_equal(g1["forceo"], g2["forceo"])
    assert g1["u_tot"] == g2["u_tot"]


def test_electrolyte_std_config(orc, gpu_lib):
    """The N=1000 standard-Ewald electrolyte (r_c = 30 A, |n| <= 8)."""
    s = prepared(configs.electrolyte_std(), orc)
    r, g, _, _ = run_pair(s, orc)
    e = utotal_errors(g, r, s.nptpt)
    bad = {k: v for k, v in e.items() if not v <= TOL_FP64}
    assert not bad, (bad, e)
