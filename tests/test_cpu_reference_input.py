"""The reference's input formats: the namelist file (<project>.in) and the
configuration file (<project>.cnf, IOCnf's unformatted records), read into a
System that the oracle and the GPU library run.

The inputs below are written for these tests in the reference's format
(&nmlSystem ... / groups with its variable names and defaults); the last
test checks the fixture made from the reference's own Testin inputs.
"""
import os

import numpy as np
import pytest

from molsim_gb300 import Engine, abi, units
from molsim_gb300.cnf import read_cnf, read_records, write_cnf
from molsim_gb300.namelist import NamelistError, array, parse_namelists, scalar
from molsim_gb300.reference_input import system_from_input

SYNTAX = """
 some text before the first group is ignored
 &nmlA
  txtitle = 'it''s a test',   ! a comment with 'quotes'
  boxlen = 3*50.0,
  temp=298.0 lflag=.t., lother = F,
  nppt(2) = 7, nppt(1) = 5,
  npptct(1,2) = 4, npptct(2,1) = 3,
  zat = 1.0, , -1.0d0,
  bond = 2.5, 2, 5.0,
  angle%k = 0.5, angle%eq = 120.,
 /
 &nmlB x = 2*, 3 /
"""


def test_namelist_syntax():
    g = parse_namelists(SYNTAX)
    a = g["nmla"]
    assert scalar(a, "txtitle") == "it's a test"
    assert list(array(a, "boxlen", 3, 0.0)) == [50.0, 50.0, 50.0]
    assert scalar(a, "temp") == 298.0 and scalar(a, "lflag") is True and scalar(a, "lother") is False
    assert list(array(a, "nppt", 2, 0, dtype=int)) == [5, 7]
    m = array(a, "npptct", (2, 2), 0, dtype=int)
    assert m[0, 1] == 4 and m[1, 0] == 3 and m[0, 0] == 0
    assert list(array(a, "zat", 3, 9.0)) == [1.0, 9.0, -1.0]        # null keeps the preset
    assert a["bond"].values == [2.5, 2, 5.0]
    assert scalar(a, "angle%k") == 0.5 and scalar(a, "angle%eq") == 120.0
    assert list(array(g["nmlb"], "x", 3, 1, dtype=int)) == [1, 1, 3]
    bad = parse_namelists("&nmlC x = 1 &nmlD y = 2 /")   # &nmlC not closed: used, it raises
    assert scalar(bad["nmld"], "y") == 2
    with pytest.raises(NamelistError):
        scalar(bad["nmlc"], "x")
    raw = parse_namelists("&nmlE v(1:3)%l = 3*.t., w(2)%a = 1 /")["nmle"]
    assert raw["__raw__"].items[("v(1:3)%l",)] == [True, True, True]
    with pytest.raises(NamelistError):
        array(parse_namelists("&g v(4) = 1 /")["g"], "v", 3, 0)


def test_cnf_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    ro = rng.uniform(-10, 10, (17, 3))
    rod = rng.standard_normal((17, 3))
    p = tmp_path / "x.cnf"
    write_cnf(p, ro, [20.0, 21.0, 22.0], istep=12, iseed=345, rod=rod)
    recs = read_records(p)
    assert [len(r) for r in recs] == [48, 32, 56 * 17, 56 * 17]
    c = read_cnf(p)
    assert c["np"] == 17 and c["istep"] == 12 and c["iseed"] == 345
    assert np.array_equal(c["ro"], ro) and np.array_equal(c["rod"], rod)
    assert np.array_equal(c["boxlen"], [20.0, 21.0, 22.0])
    assert np.array_equal(c["qua"][:, 0], np.ones(17))
    with open(p, "r+b") as f:                          # a broken record marker
        f.seek(4 + 48)
        f.write(b"\x00\x00\x00\x00")
    with pytest.raises(ValueError):
        read_cnf(p)


def _input(method="bd", ewald="spm", extra_chain=""):
    return f"""
 &nmlSystem txtitle='polyelectrolyte test', txmethod='{method}', txbc='xyz',
  boxlen=3*60.0, temp=298.0, iseed=7, nstep1=1, nstep2=10 /
 &nmlParticle
  nct = 2, txct = 'pe', 'copo', ncct = 2, 1,
  npptct(1,1) = 6, npptct(2,2) = 3, npptct(3,2) = 2,
  npt = 3, txpt = 'bead', 'cat', 'an',
  nppt = 12, 23, 15,
  natpt = 3*1,
  zat = -1.0, 1.0, -1.0,
  sigat = 4.0, 3.5, 4.0, epsat = 3*0.25,
  massat = 3*20.0, radat = 3*0.0,
 /
 &nmlPotential rcut = 12.0, relpermitt = 78.4, lewald=.true., txewaldrec='{ewald}',
  iewaldopt = 0, ualphared = 3.2, ncut = 6, order = 6, nmesh = 32, lsurf = .false.,
  lljcut = .false., utoltab = 1e-7, ftoltab = 1e-6 /
 &nmlPotentialChain bond = 0.8, 2, 5.0, 1.2, 2, 4.5, angle = 0.01, 2, 150.0 {extra_chain} /
 &nmlIntList txintlist = 'celllist', drnlist = 1.5 /
 &nmlBD tstep = 0.02, dcoeff = 3*1.5 /
 &nmlMD tstep = 0.002 /
"""


def test_system_from_input_topology_and_parameters():
    run = system_from_input(_input(), text=True, seed=3)
    s = run.system
    assert run.method == "bd" and run.tstep == 0.02 and run.iseed == 7
    assert s.np_ == 50 and s.mode == abi.MG_BD and s.txintlist == abi.MG_CELLLIST
    assert list(np.bincount(s.iptpn)[1:]) == [12, 23, 15]
    assert [sp.charge for sp in s.species] == [-1.0, 1.0, -1.0] and s.species[1].sigma == 3.5
    assert s.ewald == abi.MG_EWALD_SPM and abs(s.ualpha - 3.2 / 12.0) < 1e-15 and s.lsurf == 0
    # SetObjectParam1 'block' numbering: type-major, chains first within a type.
    # Chains 1-2 (type 'pe'): beads of type 1, particles 1-6 and 7-12; chain 3
    # ('copo'): 3 of type 2 (particles 13-15) then 2 of type 3 (36-37)
    assert list(s.bond_ip[:5]) == [1, 2, 3, 4, 5] and list(s.bond_jp[:5]) == [2, 3, 4, 5, 6]
    assert list(s.bond_ip[5:10]) == [7, 8, 9, 10, 11]
    assert list(s.bond_ip[10:]) == [13, 14, 15, 36] and list(s.bond_jp[10:]) == [14, 15, 36, 37]
    assert np.allclose(s.bond_k, [0.8] * 10 + [1.2] * 4) and np.allclose(s.bond_eq, [5.0] * 10 + [4.5] * 4)
    # angles only for chain type 1 (the second chain type keeps k = 0)
    assert len(s.angle_ip) == 8 and list(s.angle_jm[:2]) == [1, 2] and list(s.angle_jp[:2]) == [3, 4]
    deg = units.Pi / 180.0
    assert np.allclose(s.angle_k, 0.01 / deg ** 2) and np.allclose(s.angle_eq, 150.0 * deg)
    # generated chains sit at their bond lengths
    d = s.ro[s.bond_jp - 1] - s.ro[s.bond_ip - 1]
    d -= s.boxlen * np.round(d / s.boxlen)
    assert np.allclose(np.linalg.norm(d, axis=1), s.bond_eq, atol=1e-9)


@pytest.mark.parametrize("ewald", ["spm", "std"])
def test_reference_input_runs_through_the_oracle(orc, ewald, tmp_path):
    run = system_from_input(_input(ewald=ewald), text=True, seed=4)
    s = run.system
    s.build_table(orc.orc_pot_twobody_tab)
    e = Engine(s, lib=orc, prefix="orc_")
    e.SetPositions(s.ro_flat())
    e.NList("write")
    u = e.UTotal()
    t = e.EnergyTerms()
    assert np.isfinite(u["u_tot"]) and t["u_angle"] > 0 and np.isfinite(u["forceo"]).all()
    e.close()
    # the same configuration through a .cnf gives the same energy
    p = tmp_path / "c.cnf"
    write_cnf(p, s.ro, s.boxlen)
    s2 = system_from_input(_input(ewald=ewald), cnf=p, text=True).system
    s2.build_table(orc.orc_pot_twobody_tab)
    e2 = Engine(s2, lib=orc, prefix="orc_")
    e2.SetPositions(s2.ro_flat())
    e2.NList("write")
    assert e2.UTotal()["u_tot"] == u["u_tot"]
    e2.close()


def test_unsupported_inputs_are_refused():
    with pytest.raises(NotImplementedError):
        system_from_input(_input().replace("txbc='xyz'", "txbc='sph'"), text=True)
    with pytest.raises(NotImplementedError):
        system_from_input(_input().replace("natpt = 3*1", "natpt = 2, 1, 1"), text=True)
    with pytest.raises(NotImplementedError):
        system_from_input(_input().replace("nct = 2,", "txelec = 'dip', nct = 2,"), text=True)
    with pytest.raises(NotImplementedError):
        system_from_input(_input().replace("iewaldopt = 0", "iewaldopt = 2"), text=True)
    with pytest.raises(NotImplementedError):     # SPME reads iewaldopt 0 and 3 only
        system_from_input(_input().replace("iewaldopt = 0", "iewaldopt = 1"), text=True)


def test_ewald_parameter_options():
    """iewaldopt 1 and 3 with the standard Ewald sum: ncut from the
    tolerance (AlphaToNcut); 3: alpha from RcutToAlpha (the oracle's)."""
    from molsim_gb300.reference_input import alpha_to_ncut, ewald_error_ureal
    run1 = system_from_input(_input(ewald="std").replace("iewaldopt = 0", "iewaldopt = 1"), text=True)
    s = run1.system
    q2 = float((s.az ** 2).sum())
    tol = ewald_error_ureal(q2, 60.0, 3.2 / 12.0, 12.0, s.epsi_four_pi)
    assert s.ncut == alpha_to_ncut(tol, q2, 60.0, 3.2 / 12.0, s.epsi_four_pi) and s.ncut > 0
    # more accuracy asks for more k-vectors
    assert alpha_to_ncut(tol / 100, q2, 60.0, 3.2 / 12.0, s.epsi_four_pi) > s.ncut
    run3 = system_from_input(_input(ewald="std").replace("iewaldopt = 0", "iewaldopt = 3, uewaldtol = 1e-4"),
                             text=True)
    assert 0.1 < run3.system.ualpha * 12.0 < 10.0 and run3.system.ncut > 0


def test_reference_input_fixture_is_current():
    """The committed fixture tests/golden/reference_inputs.json is what the
    reference's own input files give today (skipped where the files are
    not present)."""
    import json
    from tests.golden import make_reference_inputs as mk
    if not os.path.isdir(mk.TESTIN):
        pytest.skip("the reference's Testin inputs are not present")
    with open(mk.OUT) as fh:
        stored = json.load(fh)
    fresh = json.loads(json.dumps(mk.make()))
    assert [e["input"] for e in stored] == [e["input"] for e in fresh]
    for a, b in zip(stored, fresh):
        assert a == b, a["input"]
