"""The host-side MC moves (molsim_gb300/mc.py) on the oracle.

Random (mollib.F90:2689-2709) is checked against an independent statement
of its two component generators; the moves against the invariants the
reference's own checks use: the accepted du%tot add up to UTotal (ucheck,
molsim.F90:1728-1745), a pivot about a bond (ipivotrotmode 1) keeps every
bond length, a chain translation keeps the chain's internal distances.
"""
import numpy as np
import pytest

from molsim_gb300 import Engine, abi, configs
from molsim_gb300.mc import MCPass, MoveParams, RefRandom, axis_angle_matrix, chains_from_bonds
from tests.helpers import chain_system


def test_random_components():
    """The Park-Miller part as iy <- 16807 iy mod (2^31 - 1) in exact
    integers, the Marsaglia part as 32-bit xorshifts in numpy uint32, and
    the combination am * ((ix xor iy) and (2^31 - 1) or 1)."""
    r = RefRandom(4711)
    iy = ((888889999 ^ 4711) | 1)
    ix = np.uint32(777755555 ^ 4711)
    am = float(np.float32(1.0 - 2.0 ** -24) / np.float32(2147483647))
    for _ in range(2000):
        x = r()
        iy = (16807 * iy) % 2147483647
        ix = ix ^ (ix << np.uint32(13))
        ix = ix ^ (ix >> np.uint32(17))
        ix = ix ^ (ix << np.uint32(5))
        assert x == am * float(((int(ix) ^ iy) & 0x7FFFFFFF) | 1)
    assert r.iseed == 4712
    xs = np.array([r() for _ in range(200000)])
    assert 0.0 < xs.min() and xs.max() < 1.0
    assert abs(xs.mean() - 0.5) < 3e-3 and abs(xs.std() - 12 ** -0.5) < 3e-3


def test_random_matches_the_oracle(orc):
    """The host generator against the oracle's restatement of Random; a
    non-positive seed re-initialises both."""
    import ctypes as C
    r = RefRandom(-777)
    seed = C.c_int32(-777)
    for _ in range(5000):
        assert r() == orc.orc_random(C.byref(seed))
    assert r.iseed == seed.value


def test_axis_angle_matrix_is_a_rotation():
    rng = np.random.default_rng(3)
    for _ in range(20):
        ax = rng.normal(size=3)
        a = rng.uniform(-np.pi, np.pi)
        R = axis_angle_matrix(ax, a)
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-14)
        assert abs(np.linalg.det(R) - 1.0) < 1e-13
        n = ax / np.linalg.norm(ax)
        assert np.allclose(R @ n, n, atol=1e-13)
        v = np.cross(n, rng.normal(size=3))
        # the reference's matrix rotates by -alpha in the right-handed sense
        # (it is the orientation matrix of the quaternion); the angle is alpha
        c = np.dot(R @ v, v) / np.dot(v, v)
        assert abs(c - np.cos(a)) < 1e-12


def _setup(orc, **kw):
    s = chain_system(txintlist=abi.MG_CELLLIST, **kw)
    s.build_table(orc.orc_pot_twobody_tab)
    e = Engine(s, lib=orc, prefix="orc_")
    e.SetPositions(s.ro_flat())
    e.NList("write")
    return s, e


def _fresh(s, orc, ro):
    e = Engine(s, lib=orc, prefix="orc_")
    e.SetPositions(ro.reshape(-1))
    e.NList("write")
    return e.UTotal()["u_tot"]


def test_chains_from_bonds(orc):
    s, _ = _setup(orc)
    chains, chain_of, seg_of = chains_from_bonds(s.np_, s.bond_ip, s.bond_jp)
    assert len(chains) == 4 and all(len(c) == 10 for c in chains)
    assert chains[1] == list(range(11, 21))
    assert chain_of[15] == 1 and seg_of[15] == 4 and chain_of[s.np_] == -1


@pytest.mark.parametrize("mode", [1, 2, 3])
def test_pivot_moves_ucheck(mode, orc):
    s, e = _setup(orc)
    u0 = e.UTotal()["u_tot"]
    chain_p = MoveParams(pspart=0.2, dtran=1.0, ppivot=0.5, ipivotrotmode=mode, drotpivot=60.0,
                         pchain=0.3, dtranchain=1.0)
    ion_p = MoveParams(pspart=1.0, dtran=2.0)
    mc = MCPass(e, s, iseed=91 + mode, params=[ion_p, ion_p, ion_p, chain_p], record=True)
    for _ in range(2):
        mc.run_pass()
    st = mc.stats
    assert st.trials["pivot"] > 20 and st.accepted["pivot"] > 3
    assert st.trials["chain"] > 10 and st.accepted["spart"] > 100
    u1 = _fresh(s, orc, mc.ro)
    assert abs((u0 + mc.du_acc) - u1) < 1e-9 * abs(u1)
    assert np.array_equal(e.GetPositions(), mc.ro)


def test_pivot_about_a_bond_keeps_bond_lengths(orc):
    s, e = _setup(orc)
    e.UTotal()   # DUTotal needs the Ewald state of a preceding UTotal
    L = s.boxlen[0]

    def bonds(ro):
        d = ro[s.bond_jp - 1] - ro[s.bond_ip - 1]
        d -= L * np.round(d / L)
        return np.linalg.norm(d, axis=1)

    b0 = bonds(s.ro)
    p = MoveParams(pspart=0.0, ppivot=1.0, ipivotrotmode=1, drotpivot=90.0)
    ion = MoveParams(pspart=0.0)   # ions do not move
    mc = MCPass(e, s, iseed=5, params=[ion, ion, ion, p])
    mc.run_pass()
    assert mc.stats.accepted["pivot"] > 3
    assert np.abs(bonds(mc.ro) - b0).max() < 1e-9


def test_clusters_are_connected_components():
    from molsim_gb300.mc import clusters
    lab = clusters(7, [(0, 3), (3, 5), (1, 2), (6, 6)])
    groups = {}
    for i, l in enumerate(lab):
        groups.setdefault(l, []).append(i)
    assert sorted(groups.values()) == [[0, 3, 5], [1, 2], [4], [6]]


@pytest.mark.parametrize("memb", ["ipt", "all"])
def test_cluster_moves_ucheck(memb, orc):
    """SPartCl2Move (mc.F90:1818-1945) beside single-particle moves: clusters
    of several ions move, moves that would change a cluster are rejected,
    and the accepted du%tot add up to the change of UTotal."""
    s, e = _setup(orc)
    u0 = e.UTotal()["u_tot"]
    ion_p = MoveParams(pspart=0.5, dtran=2.0, pspartcl2=0.5, txmembcl2=memb, radcl2=6.0, dtrancl2=3.0)
    chain_p = MoveParams(pspart=1.0, dtran=1.0)
    mc = MCPass(e, s, iseed=17, params=[ion_p, ion_p, ion_p, chain_p], record=True)
    for _ in range(2):
        mc.run_pass()
    st = mc.stats
    sizes = [int(ev[5:]) for ev in st.events if ev.startswith("cl2:") and ev[4] in "aro"]
    assert st.trials["cl2"] > 50 and st.accepted["cl2"] > 5
    assert max(sizes) >= 3
    assert any(ev == "cl2:x" for ev in st.events)
    u1 = _fresh(s, orc, mc.ro)
    assert abs((u0 + mc.du_acc) - u1) < 1e-9 * abs(u1)
    assert np.array_equal(e.GetPositions(), mc.ro)


def test_brush_moves_ucheck(orc):
    """BrushCl2Move (mc.F90:3028-3158) beside single-particle moves: a
    grafting particle's cluster moves with every chain grafted on its
    members, moves that would change the cluster are rejected, the bonds of
    the moved chains keep their lengths, and the accepted du%tot add up to
    the change of UTotal."""
    from tests.helpers import brush_system
    s = brush_system(txintlist=abi.MG_CELLLIST)
    s.build_table(orc.orc_pot_twobody_tab)
    e = Engine(s, lib=orc, prefix="orc_")
    e.SetPositions(s.ro_flat())
    e.NList("write")
    u0 = e.UTotal()["u_tot"]
    L = s.boxlen[0]

    def bonds(ro):
        d = ro[s.bond_jp - 1] - ro[s.bond_ip - 1]
        d -= L * np.round(d / L)
        return np.linalg.norm(d, axis=1)

    b0 = bonds(s.ro)
    ion_p = MoveParams(pspart=1.0, dtran=2.0)
    still = MoveParams(pspart=0.0)   # type 2 holds the chain beads: they move only with their brush
    graft_p = MoveParams(pspart=0.2, dtran=1.0, pbrushcl2=0.8, radcl2=14.0, dtranbrush=2.0)
    mc = MCPass(e, s, iseed=23, params=[ion_p, still, ion_p, graft_p], record=True)
    for _ in range(3):
        mc.run_pass()
    st = mc.stats
    ev = [x for x in st.events if x.startswith("brushcl2:")]
    assert st.trials["brushcl2"] > 5 and st.accepted["brushcl2"] > 0
    moved = [x for x in ev if x[9] in "aro"]
    # a member moves with its 2 chains of 5 beads: 11 particles per member
    assert all(int(x.split(":")[2]) == 11 * int(x.split(":")[1][1:]) for x in moved)
    assert np.abs(bonds(mc.ro) - b0).max() < 1e-9
    u1 = _fresh(s, orc, mc.ro)
    assert abs((u0 + mc.du_acc) - u1) < 1e-9 * abs(u1)
    assert np.array_equal(e.GetPositions(), mc.ro)


def test_brush_rotations_ucheck(orc):
    """BrushMove (mc.F90:2850-3019): a grafting particle with the chains
    grafted on it, translated and rotated about the particle; the bonds of
    the moved chains keep their lengths, the distance from the particle to
    every bead of its brush along the unwrapped chain is kept, and the
    accepted du%tot add up to the change of UTotal."""
    from tests.helpers import brush_system
    s = brush_system(txintlist=abi.MG_CELLLIST)
    s.build_table(orc.orc_pot_twobody_tab)
    e = Engine(s, lib=orc, prefix="orc_")
    e.SetPositions(s.ro_flat())
    e.NList("write")
    u0 = e.UTotal()["u_tot"]
    L = s.boxlen[0]

    def dist(ro, i, j):
        d = ro[np.asarray(j) - 1] - ro[np.asarray(i) - 1]
        d -= L * np.round(d / L)
        return np.linalg.norm(d, axis=-1)

    b0 = dist(s.ro, s.bond_ip, s.bond_jp)
    ng = int(np.count_nonzero(s.iptpn == 4))
    chains, _, _ = chains_from_bonds(s.np_, s.bond_ip, s.bond_jp)
    graft = [(ic % ng) + 1 for ic in range(len(chains))]

    def reach(ro, ic):
        # the beads' distances to the grafting particle along the unwrapped
        # chain (the minimum image from the particle to the first bead, then
        # bond by bond): a rigid move keeps them, whatever the box
        c = chains[ic]
        pts = np.asarray(c) - 1
        d = np.diff(ro[np.concatenate(([graft[ic] - 1], pts))], axis=0)
        d -= L * np.round(d / L)
        return np.linalg.norm(np.cumsum(d, axis=0), axis=1)

    g0 = [reach(s.ro, ic) for ic in range(len(chains))]
    ion_p = MoveParams(pspart=1.0, dtran=2.0)
    still = MoveParams(pspart=0.0)   # type 2 holds the chain beads: they move only with their brush
    # the grafting particles make only brush moves, so that their distances
    # to the beads of their brushes are invariants
    graft_p = MoveParams(pspart=0.0, pbrush=1.0, dtranbrush=1.0, drotbrush=10.0)
    mc = MCPass(e, s, iseed=31, params=[ion_p, still, ion_p, graft_p], record=True)
    for _ in range(3):
        mc.run_pass()
    st = mc.stats
    assert st.trials["brush"] > 5 and st.accepted["brush"] > 1
    assert np.abs(dist(mc.ro, s.bond_ip, s.bond_jp) - b0).max() < 1e-9
    for ic in range(len(chains)):
        assert np.abs(reach(mc.ro, ic) - g0[ic]).max() < 1e-9
    u1 = _fresh(s, orc, mc.ro)
    assert abs((u0 + mc.du_acc) - u1) < 1e-9 * abs(u1)
    assert np.array_equal(e.GetPositions(), mc.ro)
