"""NVE energy conservation of the device velocity Verlet, both forms.

The mixed form (FP32 arithmetic, fixed-point accumulation) must conserve
energy as well as the plain FP64 form: on the 1 000-ion standard-Ewald
electrolyte over 500 steps of 2 fs, its drift stays within 5 % of the FP64
drift and both stay below 0.02 kT per particle per ns.
"""
import pytest

from molsim_gb300 import abi, configs
from molsim_gb300.nve import nve_drift

pytestmark = pytest.mark.gpu


def test_mixed_form_conserves_energy_like_fp64(gpu_lib):
    r64 = nve_drift(configs.electrolyte_std(seed=1), form=abi.MG_FP64, nsteps=500)
    rmx = nve_drift(configs.electrolyte_std(seed=1), form=abi.MG_MIXED, nsteps=500)
    d64, dmx = r64["drift_kt_per_particle_per_ns"], rmx["drift_kt_per_particle_per_ns"]
    assert abs(d64) < 0.02 and abs(dmx) < 0.02, (d64, dmx)
    assert abs(dmx - d64) <= 0.05 * abs(d64) + 1e-5, (d64, dmx)
