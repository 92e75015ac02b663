"""The replay harness's file format and its command line (no GPU needed)."""
import os
import subprocess

import numpy as np

from molsim_gb300 import abi, configs, replay


def test_input_round_trip(tmp_path, orc):
    s = configs.small_system(seed=9, chains=2, nseg=6, angle_kt=0.5)
    s.build_table(orc.orc_pot_twobody_tab)
    path = str(tmp_path / "in.bin")
    replay.write_input(path, s, abi.MG_MIXED, "bdstep", 7, fac1=np.ones(3), fac2=np.ones(3), iseed=5)
    d = replay.read_output(path)   # the same tagged-array format
    assert d["np"][0] == s.np_ and d["form"][0] == abi.MG_MIXED and d["run_kind"][0] == 1
    assert np.array_equal(d["ro"], s.ro_flat())
    assert np.array_equal(d["ubuf"], s.ubuf)
    assert np.array_equal(d["angle_ip"], s.angle_ip) and d["iseed"].dtype == np.int32
    assert d["nstep"][0] == 7 and d["boxlen"].shape == (3,)


def test_harness_is_built_and_checks_its_arguments():
    import molsim_gb300
    molsim_gb300.build()
    assert os.access(replay.HARNESS, os.X_OK)
    r = subprocess.run([replay.HARNESS], capture_output=True, text=True)
    assert r.returncode == 1 and "usage" in r.stderr
