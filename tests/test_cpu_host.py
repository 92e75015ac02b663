"""Host-side logic without a GPU: units, the seeded workload generators
(placement rules, neutrality, bonds) and the integrator factors."""
import math

import numpy as np
import pytest

from molsim_gb300 import abi, configs, units


def _min_image_dist_ok(ro, L, rmin):
    spatial = pytest.importorskip("scipy.spatial")
    t = spatial.cKDTree(np.mod(ro + L / 2, L), boxsize=L)
    return len(t.query_pairs(rmin * (1 - 1e-12))) == 0


def test_bjerrum_length_and_units():
    s = configs.electrolyte_std(seed=1)
    assert abs(s.epsi_four_pi / units.kT(s.temp) - 7.1) < 1e-12
    assert abs(units.ljrcut_default() - 2.0 ** (1.0 / 6.0)) < 1e-6       # single-precision default
    assert abs(math.erfc(s.ualpha * s.rcut) - 1e-5) < 1e-12


def test_electrolyte_std_config():
    s = configs.electrolyte_std(seed=1)
    assert s.np_ == 1000 and np.allclose(s.boxlen, 100.0)
    assert s.az.sum() == 0 and (s.az == 1).sum() == 500
    assert s.ewald == abi.MG_EWALD_STD and s.ncut == 8 and s.rcut == 30.0
    assert np.abs(s.ro).max() <= 50.0
    assert _min_image_dist_ok(s.ro, 100.0, 4.0)


def test_electrolyte_spme_config():
    s = configs.electrolyte_spme(seed=2)
    assert s.np_ == 32768 and np.allclose(s.boxlen, 817.0)
    assert s.az.sum() == 0
    assert (s.order, s.nmesh, s.rcut) == (6, 64, 12.0)
    assert _min_image_dist_ok(s.ro, 817.0, 4.0)


def test_polyelectrolyte_config():
    s = configs.polyelectrolyte(seed=3)
    assert s.np_ == 65600 and np.allclose(s.boxlen, 700.0)
    assert s.az.sum() == 0
    assert (s.az[:12800] == -1).all()
    assert len(s.bond_ip) == 64 * 199
    d = s.ro[s.bond_jp - 1] - s.ro[s.bond_ip - 1]
    d -= 700.0 * np.round(d / 700.0)
    assert np.allclose(np.sqrt((d * d).sum(1)), 5.0, atol=1e-9)
    assert _min_image_dist_ok(s.ro, 700.0, 4.0)
    assert np.allclose(s.bond_eq, 5.0) and (s.bond_p == 2).all()


def test_same_seed_same_system_and_neutral_small_systems():
    a, b = configs.small_system(seed=5), configs.small_system(seed=5)
    assert np.array_equal(a.ro, b.ro)
    assert not np.array_equal(a.ro, configs.small_system(seed=6).ro)
    for kw in (dict(), dict(chains=4, nseg=12), dict(n=600, L=50.0)):
        assert abs(configs.small_system(seed=7, **kw).az.sum()) < 1e-12


def test_bd_factors_einstein_relation():
    """fac1 = D dt / kT (force to displacement), fac2 = sqrt(2 D dt):
    fac2^2 / (2 fac1) is kT in force x length units."""
    f1, f2 = units.bd_factors(0.01, 1.0, 298.0)
    kt_int = f2 * f2 / (2.0 * f1)
    assert f1 > 0 and f2 > 0
    # kT expressed through the force unit: kT [kJ/mol] * FORCE_FAC
    assert abs(kt_int / (units.kT(298.0) * units.FORCE_FAC) - 1.0) < 1e-12


def test_maxwell_velocities_remove_momentum():
    s = configs.small_system(seed=5)
    v = s.maxwell_velocities(seed=1).reshape(-1, 3)
    m = np.array([sp.mass for sp in s.species])[s.iptpn - 1]
    assert np.abs((m[:, None] * v).sum(0)).max() < 1e-9


def test_choose_spme_meets_its_spacing_rule():
    """The replicas' SPME chooser: every box gets order 6, r_c <= L/2, a
    power-of-two mesh of at most 256 whose spacing keeps alpha*h within the
    error model's bound, and alpha from erfc(alpha r_c) = 1e-5."""
    import math

    from molsim_gb300 import autotune, configs
    for s in configs.replica_set(seed=5, nrep=64):
        c = (s.np_ / 2) / (float(np.prod(s.boxlen)) * 1e-27 * configs.AVOGADRO)
        ch = autotune.choose_spme(s, c)
        L = float(s.boxlen.min())
        assert ch["order"] == 6 and ch["rcut"] <= L / 2
        assert ch["nmesh"] <= 256 and ch["nmesh"] & (ch["nmesh"] - 1) == 0
        assert ch["ualpha"] * L / ch["nmesh"] <= autotune.alpha_h_max(1e-5, c) * (1 + 1e-12)
        assert abs(math.erfc(ch["ualpha"] * ch["rcut"]) - 1e-5) < 1e-9
