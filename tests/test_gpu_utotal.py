"""GPU parity of UTotal (plain FP64 and mixed forms) against the CPU oracle.

Reference: UTotal, energy.F90:280-430 (pair loop, Ewald std/SPME, self,
surface, bonds, force epilogue).
"""
import numpy as np
import pytest

from molsim_gb300 import abi, configs
from tests.helpers import (TOL_FP64, TOL_MIXED_RMS, force_err, force_rms_err, prepared, rel,
                           run_pair, small_cases)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,factory", small_cases(), ids=[c[0] for c in small_cases()])
def test_utotal_fp64(name, factory, orc, gpu_lib):
    s = prepared(factory(), orc)
    r, g, _, _ = run_pair(s, orc)
    for k in range(1, s.nptpt + 1):
        assert abs(g["u_twob"][k] - r["u_twob"][k]) <= TOL_FP64 * max(abs(r["u_twob"][k]), 1e-12), (k, g["u_twob"], r["u_twob"])
    assert rel(g["u_twob"][0], r["u_twob"][0]) <= TOL_FP64
    assert abs(g["u_rec"] - r["u_rec"]) <= TOL_FP64 * max(abs(r["u_rec"]), 1.0)
    assert abs(g["u_bond"] - r["u_bond"]) <= TOL_FP64 * max(abs(r["u_bond"]), 1e-12)
    assert rel(g["u_tot"], r["u_tot"]) <= TOL_FP64
    assert rel(g["virial"], r["virial"]) <= TOL_FP64
    assert force_err(g["forceo"], r["forceo"]) <= TOL_FP64


@pytest.mark.parametrize("name,factory", small_cases()[:6], ids=[c[0] for c in small_cases()[:6]])
def test_utotal_mixed(name, factory, orc, gpu_lib):
    s = prepared(factory(), orc)
    r, g, _, _ = run_pair(s, orc, form=abi.MG_MIXED)
    assert force_rms_err(g["forceo"], r["forceo"]) <= TOL_MIXED_RMS
    assert rel(g["u_tot"], r["u_tot"]) <= 1e-5
    assert rel(g["virial"], r["virial"]) <= 1e-5


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
    assert rel(g["u_tot"], r["u_tot"]) <= TOL_FP64
    assert rel(g["virial"], r["virial"]) <= TOL_FP64
    assert force_err(g["forceo"], r["forceo"]) <= TOL_FP64
