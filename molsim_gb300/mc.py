"""Monte Carlo passes over an Engine: the reference's trial moves as callers
of DUTotal and MCUpdate.

The moves run on the host and hand their trial positions to the library
(`Engine.DUTotal`, `Engine.MCUpdate`), as the reference's MC driver does
with its own DUTotal and MCUpdate.  Restated from mc.F90:

- MCPass (mc.F90:1470-1581): np trial moves per pass, the particle chosen in
  sequence (isamp = 0) or at random (isamp = 1), the move type by CallMove's
  cumulative probabilities (mc.F90:669-708); NListDriver after the pass.
- SPartMove (mc.F90:1583-1753): one particle, GetRandomTrialPos
  (mc.F90:4527-4580): the same random displacement in a cube of edge dtran
  (or a sphere of diameter |dtran| for dtran < 0) for every moving particle.
- ChainMove (mc.F90:2541-2629): a whole chain, displaced by dtranchain.
- SPartCl2Move (mc.F90:1818-1945): the cluster of the chosen particle (its
  connected component among the particles of its type, or all particles
  with txmembcl2 = 'all', two particles joined when closer than radcl2:
  CalcPartPairListIpt/All molaux.F90:1863-1984, MakeCluster and
  CalcClusterMember mollib.F90:1805-1935), displaced together by one
  GetRandomTrialPos of dtrancl2; after DUTotal the move is rejected without
  a Metropolis draw when a cluster member would come within radcl2 of a
  particle of the type outside the cluster (the cluster would change).
- BrushMove (mc.F90:2850-3019, lcl1brush = .false.): the chosen particle
  and the chains grafted on it (as below), translated by one
  GetRandomTrialPos of dtranbrush and rotated about the particle by alpha =
  drotbrush (Random - 1/2) about a SphRandom axis (RotTranBrush: the chains
  unwrapped from the particle by UndoPBCChain, RotateSetPart, then the
  translation, rotm(ipmove) - ro(ipmove), added to every member).
- BrushCl2Move (mc.F90:3028-3158): the cluster of the chosen particle among
  the particles of its type (radcl2, as SPartCl2Move), and the brush of
  every cluster member: the chains ic = ip, ip + nppt, ip + 2 nppt, ... (ip
  the member's particle number, nppt the number of particles of its type;
  the reference grafts the chains cyclically on the particles of the first
  type), whole, in segment order.  One GetRandomTrialPos of dtranbrush moves
  all of them (the reference draws it with dtranbrush, not dtranbrushcl2);
  after DUTotal the move is rejected without a Metropolis draw when a
  cluster member would come within radcl2 of a particle of its type
  outside the cluster.
- PivotMove (mc.F90:1967-2172): the part of a chain on one side of a pivot
  bead ('short', 'lower' or 'upper'), unwrapped by UndoPBCChain
  (molaux.F90:1266-1325), rotated by alpha = drotpivot (Random - 1/2) about
  an axis through the pivot (ipivotrotmode 1: the bond to the non-moving
  neighbour; 2: the normal of the pivot's two bonds; 3: random, SphRandom
  mollib.F90:2793-2805) with the rotation matrix of AxisAngToOri
  (mollib.F90:2268-2300), RotateSetPart (mc.F90:4687-4732).
- CheckPartBCTM (mc.F90:4810-4858) for periodic boxes: PBC of the trial
  positions; Metropolis (mc.F90:5135-5178); MCUpdate (mc.F90:5203-5236):
  u%tot accumulated, drostep += the displacement.
- Random (mollib.F90:2689-2709): Marsaglia's xorshift combined with
  Park-Miller, the generator every move draws from.

The cluster moves' second shell (radcl1 > 0), the brush move's rotations
of polyatomic particles, the pivot's crosslinked
generations and the non-energetic weights (umbrella, MC weights) are not
part of this path.
"""
from dataclasses import dataclass, field
from typing import Dict, List

import numpy as np

from . import units

__all__ = ["RefRandom", "MoveParams", "MCPass", "chains_from_bonds", "axis_angle_matrix", "clusters"]

_M32 = 0xFFFFFFFF


def _i32(x):
    x &= _M32
    return x - (1 << 32) if x & 0x80000000 else x


class RefRandom:
    """Random(iseed) (mollib.F90:2689-2709).  The generator state (ix, iy,
    am) is module state in the reference; here it lives in the object, with
    the seed.  The first call (iy < 0) initialises from the seed."""

    IA, IM, IQ, IR = 16807, 2147483647, 127773, 2836

    def __init__(self, iseed):
        self.iseed = int(iseed)
        self.ix = -1
        self.iy = -1
        # am = nearest(1.0, -1.0)/im in default (single-precision) real
        self.am = float(np.float32(np.nextafter(np.float32(1.0), np.float32(0.0))) / np.float32(self.IM))

    def __call__(self):
        if self.iseed <= 0 or self.iy < 0:
            a = abs(self.iseed)
            self.iy = _i32((888889999 ^ a) | 1)
            self.ix = _i32(777755555 ^ a)
            self.iseed = a + 1
        ix = self.ix
        ix = _i32(ix ^ ((ix << 13) & _M32))
        ix = _i32(ix ^ ((ix & _M32) >> 17))
        ix = _i32(ix ^ ((ix << 5) & _M32))
        self.ix = ix
        k = self.iy // self.IQ
        iy = self.IA * (self.iy - k * self.IQ) - self.IR * k
        if iy < 0:
            iy += self.IM
        self.iy = iy
        return self.am * float((self.IM & (ix ^ iy)) | 1)

    def sphere(self):
        """SphRandom: a random point on the unit sphere."""
        ct = 2.0 * (self() - 0.5)
        st = np.sqrt(1.0 - ct * ct)
        psi = 6.283185308 * self()
        return np.array([st * np.cos(psi), st * np.sin(psi), ct])


def axis_angle_matrix(rotaxis, alpha):
    """AxisAngToOri: the rotation matrix of angle alpha about rotaxis, built
    from the quaternion (cos(alpha/2), sin(alpha/2) axis)."""
    norm = 1.0 / np.sqrt(rotaxis[0] ** 2 + rotaxis[1] ** 2 + rotaxis[2] ** 2)
    ca, sa = np.cos(0.5 * alpha), np.sin(0.5 * alpha)
    q0, q1, q2, q3 = ca, rotaxis[0] * norm * sa, rotaxis[1] * norm * sa, rotaxis[2] * norm * sa
    return np.array([
        [q0 * q0 + q1 * q1 - q2 * q2 - q3 * q3, 2.0 * (q1 * q2 + q0 * q3), 2.0 * (q1 * q3 - q0 * q2)],
        [2.0 * (q1 * q2 - q0 * q3), q0 * q0 - q1 * q1 + q2 * q2 - q3 * q3, 2.0 * (q2 * q3 + q0 * q1)],
        [2.0 * (q1 * q3 + q0 * q2), 2.0 * (q2 * q3 - q0 * q1), q0 * q0 - q1 * q1 - q2 * q2 + q3 * q3],
    ])


def chains_from_bonds(np_, bond_ip, bond_jp):
    """Chains as lists of 1-based particle numbers in segment order, from a
    bond list in which bond b joins the lower bead bond_ip(b) and the upper
    bead bond_jp(b) (ipnsegcn of the reference); and per particle its chain
    (0-based, -1 none) and segment (0-based)."""
    up = np.zeros(np_ + 1, dtype=np.int64)
    down = np.zeros(np_ + 1, dtype=np.int64)
    for i, j in zip(bond_ip, bond_jp):
        up[i] = j
        down[j] = i
    chains = []
    for ip in range(1, np_ + 1):
        if down[ip] == 0 and up[ip] != 0:
            c = [ip]
            while up[c[-1]] != 0:
                c.append(int(up[c[-1]]))
            chains.append(c)
    chain_of = np.full(np_ + 1, -1, dtype=np.int64)
    seg_of = np.zeros(np_ + 1, dtype=np.int64)
    for ic, c in enumerate(chains):
        for iseg, ip in enumerate(c):
            chain_of[ip] = ic
            seg_of[ip] = iseg
    return chains, chain_of, seg_of


def clusters(n, pairs):
    """Connected components of n objects (0-based) joined by pairs, as a
    label per object (MakeCluster, mollib.F90:1805-1904: the labels differ,
    the membership is the same)."""
    parent = list(range(n))

    def top(i):
        while parent[i] != i:
            parent[i] = parent[parent[i]]
            i = parent[i]
        return i
    for i, j in pairs:
        a, b = top(int(i)), top(int(j))
        if a != b:
            parent[b] = a
    return np.array([top(i) for i in range(n)])


@dataclass
class MoveParams:
    """nmlMC variables of one particle type (mc.F90:959-983 defaults; the
    probabilities are normalised per type as IOMC does)."""
    pspart: float = 1.0
    dtran: float = 0.0
    ppivot: float = 0.0
    txpivot: str = "short"
    drotpivot: float = 360.0      # degrees
    ipivotrotmode: int = 1
    pchain: float = 0.0
    dtranchain: float = 0.0
    pspartcl2: float = 0.0
    txmembcl2: str = "ipt"
    radcl2: float = 0.0
    dtrancl2: float = 0.0
    pbrush: float = 0.0
    drotbrush: float = 0.0        # degrees
    pbrushcl2: float = 0.0
    dtranbrush: float = 0.0


@dataclass
class MCStats:
    trials: Dict[str, int] = field(default_factory=lambda: {"spart": 0, "cl2": 0, "pivot": 0, "chain": 0,
                                                             "brush": 0, "brushcl2": 0})
    accepted: Dict[str, int] = field(default_factory=lambda: {"spart": 0, "cl2": 0, "pivot": 0, "chain": 0,
                                                               "brush": 0, "brushcl2": 0})
    events: List[str] = field(default_factory=list)


class MCPass:
    """Monte Carlo passes of one system through an Engine (the library or the
    oracle) whose positions, list and energies (UTotal) are set, as the
    reference's simulation start leaves them.  params: one MoveParams per
    particle type (1-based types in system.iptpn), or one for all."""

    def __init__(self, engine, system, iseed, params, isamp=1, record=False):
        self.e = engine
        self.s = system
        self.rng = RefRandom(iseed)
        self.beta = units.sclene / (units.GasConstant * system.temp * units.scltem)
        self.isamp = isamp
        npt = system.npt
        plist = params if isinstance(params, (list, tuple)) else [params] * npt
        if len(plist) != npt:
            raise ValueError(f"{len(plist)} move parameter sets for {npt} particle types")
        self.p = plist
        # cumulative probabilities (IOMC, CallMove's order): pspart, then
        # pspartcl2, ppivot, pchain, pbrush and pbrushcl2
        self.cum = []
        for mp in plist:
            tot = max(mp.pspart + mp.pspartcl2 + mp.ppivot + mp.pchain + mp.pbrush + mp.pbrushcl2, 1e-15)
            a = mp.pspart / tot
            a2 = a + mp.pspartcl2 / tot
            b = a2 + mp.ppivot / tot
            c = b + mp.pchain / tot
            c2 = c + mp.pbrush / tot
            self.cum.append((a, a2, b, c, c2, tot > 1e-15))
        self.L = np.asarray(system.boxlen, dtype=np.float64)
        self.half = 0.5 * self.L
        self.Li = 1.0 / self.L
        self.ro = np.asarray(system.ro, dtype=np.float64).reshape(-1, 3).copy()
        nb = 0 if system.bond_ip is None else len(system.bond_ip)
        if nb:
            self.chains, self.chain_of, self.seg_of = chains_from_bonds(
                system.np_, np.asarray(system.bond_ip), np.asarray(system.bond_jp))
        else:
            self.chains, self.chain_of, self.seg_of = [], np.full(system.np_ + 1, -1), np.zeros(system.np_ + 1)
        self.drostep = np.zeros_like(self.ro)
        self.du_acc = 0.0
        self.stats = MCStats()
        self.record = record

    # ---- helpers -----------------------------------------------------------
    def _pbc(self, r):
        """PBC (molaux.F90:104-146, box): r - L anint(r/L) where |r| > L/2."""
        r = np.array(r, dtype=np.float64)
        for m in range(3):
            x = r[..., m]
            big = np.abs(x) > self.half[m]
            t = x * self.Li[m]
            a = np.trunc(t)                                # anint: half away from zero, exactly
            a = a + np.sign(t) * (np.abs(t - a) >= 0.5)
            r[..., m] = np.where(big, x - self.L[m] * a, x)
        return r

    def _pbcr2(self, d):
        """PBCr2 (molaux.F90:149-184): one shift by L where |d| > L/2, then
        r^2 = dx^2 + dy^2 + dz^2 (rows of d)."""
        d = np.array(d, dtype=np.float64)
        for m in range(3):
            x = d[..., m]
            d[..., m] = np.where(np.abs(x) > self.half[m], x - np.copysign(self.L[m], x), x)
        return d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1] + d[..., 2] * d[..., 2]

    def _trial_translation(self, dtran):
        """GetRandomTrialPos: one displacement for all moving particles."""
        if dtran >= 0.0:
            d = np.array([(self.rng() - 0.5) * dtran for _ in range(3)])
        else:
            while True:
                d = np.array([self.rng() - 0.5 for _ in range(3)])
                if d[0] ** 2 + d[1] ** 2 + d[2] ** 2 < 0.25:
                    break
            d = d * abs(dtran)
        return d

    def _metropolis(self, ovl, du_tot, weight=1.0):
        if ovl:
            return False
        dured = du_tot * self.beta
        if dured > 87.0:
            return False
        if dured < -87.0:
            return weight != 0.0
        fac = weight * np.exp(-dured)
        if fac > 1.0:
            return True
        return fac > self.rng()

    def _try(self, kind, ipnptm, rotm, drotm):
        """DUTotal, Metropolis and MCUpdate for one trial."""
        self.stats.trials[kind] += 1
        du, ovl = self.e.DUTotal(ipnptm, rotm)
        acc = self._metropolis(ovl, du["du_tot"])
        if acc:
            self.e.MCUpdate()
            idx = np.asarray(ipnptm) - 1
            self.ro[idx] = rotm
            self.drostep[idx] += drotm
            self.du_acc += du["du_tot"]
            self.stats.accepted[kind] += 1
        if self.record:
            self.stats.events.append(f"{kind}:{'a' if acc else ('o' if ovl else 'r')}")
        return acc

    # ---- moves -------------------------------------------------------------
    def spart(self, ipmove, mp):
        d = self._trial_translation(mp.dtran)
        rotm = self._pbc(self.ro[ipmove - 1] + d).reshape(1, 3)
        return self._try("spart", [ipmove], rotm, d.reshape(1, 3))

    def spartcl2(self, ipmove, mp):
        """SPartCl2Move (radcl1 = 0)."""
        ipt = int(self.s.iptpn[ipmove - 1])
        of_type = np.flatnonzero(self.s.iptpn == ipt) + 1          # iplow .. ipupp
        objs = of_type if mp.txmembcl2 == "ipt" else np.arange(1, self.s.np_ + 1)
        rc2 = mp.radcl2 ** 2
        pos = self.ro[objs - 1]
        pairs = []
        for a in range(len(objs) - 1):
            r2 = self._pbcr2(pos[a] - pos[a + 1:])
            for b in np.flatnonzero(r2 < rc2):
                pairs.append((a, a + 1 + b))
        lab = clusters(len(objs), pairs)
        me = int(np.flatnonzero(objs == ipmove)[0])
        ips = objs[lab == lab[me]]                                  # members in object order
        d = self._trial_translation(mp.dtrancl2)
        rotm = self._pbc(self.ro[ips - 1] + d)
        self.stats.trials["cl2"] += 1
        du, ovl = self.e.DUTotal(ips, rotm)
        if not ovl:
            # a particle of the type outside the cluster within radcl2 of a
            # moved member: the cluster would change, rejected outright
            outside = of_type[~np.isin(of_type, ips)]
            for k in range(len(ips)):
                if outside.size and (self._pbcr2(self.ro[outside - 1] - rotm[k]) < rc2).any():
                    if self.record:
                        self.stats.events.append("cl2:x")
                    return False
        acc = self._metropolis(ovl, du["du_tot"])
        if acc:
            self.e.MCUpdate()
            self.ro[ips - 1] = rotm
            self.drostep[ips - 1] += d
            self.du_acc += du["du_tot"]
            self.stats.accepted["cl2"] += 1
        if self.record:
            self.stats.events.append(f"cl2:{'a' if acc else ('o' if ovl else 'r')}{len(ips)}")
        return acc

    def _brush_chains(self, ip, nppt):
        """The chains grafted on particle ip: ic = ip, ip + nppt, ... <= nc
        (1-based chain numbers, the reference's brush loop)."""
        return list(range(int(ip), len(self.chains) + 1, nppt))

    def brush(self, ipmove, mp):
        """BrushMove: the particle and its chains, translated and rotated."""
        ipt = int(self.s.iptpn[ipmove - 1])
        nppt = int(np.count_nonzero(self.s.iptpn == ipt))
        ics = self._brush_chains(ipmove, nppt)
        ips = [int(ipmove)]
        for ic in ics:
            ips.extend(self.chains[ic - 1])
        ips = np.asarray(ips)
        r0 = self.ro[ipmove - 1]
        d = self._trial_translation(mp.dtranbrush)
        dtr = (r0 + d) - r0                                  # rotm(ipmove) - ro(ipmove)
        axis = self.rng.sphere()
        alpha = (mp.drotbrush * (units.Pi / 180.0)) * (self.rng() - 0.5)   # drotbrush*sclang
        v = {int(ipmove): r0.copy()}
        for ic in ics:
            v.update(self._undo_pbc_chain(ic - 1, ref=r0))
        vaux = np.array([v[int(ip)] for ip in ips])
        rot = axis_angle_matrix(axis, alpha)
        rotm = r0 + (vaux - r0) @ rot.T
        drotm = rotm - vaux
        rotm = self._pbc(rotm + dtr)
        drotm = drotm + dtr
        return self._try("brush", ips, rotm, drotm)

    def brushcl2(self, ipmove, mp):
        """BrushCl2Move: the cluster of ipmove among its type and the chains
        grafted on the cluster's members, moved together."""
        ipt = int(self.s.iptpn[ipmove - 1])
        of_type = np.flatnonzero(self.s.iptpn == ipt) + 1          # iplow .. ipupp
        rc2 = mp.radcl2 ** 2
        pos = self.ro[of_type - 1]
        pairs = []
        for a in range(len(of_type) - 1):
            r2 = self._pbcr2(pos[a] - pos[a + 1:])
            for b in np.flatnonzero(r2 < rc2):
                pairs.append((a, a + 1 + b))
        lab = clusters(len(of_type), pairs)
        me = int(np.flatnonzero(of_type == ipmove)[0])
        prim = of_type[lab == lab[me]]                              # the primary cluster, in particle order
        nppt = len(of_type)
        ips = [int(ip) for ip in prim]
        for ip in prim:                                             # its brush
            for ic in self._brush_chains(ip, nppt):
                ips.extend(self.chains[ic - 1])
        ips = np.asarray(ips)
        d = self._trial_translation(mp.dtranbrush)
        rotm = self._pbc(self.ro[ips - 1] + d)
        self.stats.trials["brushcl2"] += 1
        du, ovl = self.e.DUTotal(ips, rotm)
        if not ovl:
            # a particle of the type outside the moving set within radcl2 of
            # a moved cluster member: the cluster would change, rejected
            outside = of_type[~np.isin(of_type, ips)]
            for k in range(len(prim)):
                if outside.size and (self._pbcr2(self.ro[outside - 1] - rotm[k]) < rc2).any():
                    if self.record:
                        self.stats.events.append("brushcl2:x")
                    return False
        acc = self._metropolis(ovl, du["du_tot"])
        if acc:
            self.e.MCUpdate()
            self.ro[ips - 1] = rotm
            self.drostep[ips - 1] += d
            self.du_acc += du["du_tot"]
            self.stats.accepted["brushcl2"] += 1
        if self.record:
            self.stats.events.append(f"brushcl2:{'a' if acc else ('o' if ovl else 'r')}{len(prim)}:{len(ips)}")
        return acc

    def chain(self, ipmove, mp):
        ic = int(self.chain_of[ipmove])
        if ic < 0:
            raise ValueError(f"chain move based on a non-chain particle {ipmove}")
        ips = np.asarray(self.chains[ic])
        d = self._trial_translation(mp.dtranchain)
        rotm = self._pbc(self.ro[ips - 1] + d)
        return self._try("chain", ips, rotm, np.tile(d, (len(ips), 1)))

    def _undo_pbc_chain(self, ic, ref=None):
        """UndoPBCChain(rref, ic, +1) (molaux.F90:1266-1325): the chain made
        continuous from its first segment, which takes the image nearest to
        rref (by default the first segment itself)."""
        c = self.chains[ic]
        out = {}
        ref = self.ro[c[0] - 1] if ref is None else ref
        out[c[0]] = ref + self._pbc(self.ro[c[0] - 1] - ref)
        for jp, ip in zip(c[:-1], c[1:]):
            out[ip] = out[jp] + self._pbc(self.ro[ip - 1] - self.ro[jp - 1])
        return out

    def pivot(self, ipmove, mp):
        ic = int(self.chain_of[ipmove])
        if ic < 0:
            raise ValueError(f"pivot rotation based on a non-chain particle {ipmove}")
        c = self.chains[ic]
        nseg = len(c)
        isegp = int(self.seg_of[ipmove]) + 1     # 1-based segment of the pivot
        if isegp == 1 or isegp == nseg:
            return None                            # early exit at the chain ends
        seg = lambda k: c[k - 1]
        lower = (mp.txpivot == "lower") or (mp.txpivot == "short" and isegp <= nseg // 2)
        if mp.txpivot not in ("short", "lower", "upper"):
            raise ValueError(f"txpivot = {mp.txpivot!r}")
        ip1 = seg(isegp)
        if lower:
            ip2, ip3, iseg1, iseg2 = seg(isegp + 1), seg(isegp - 1), 1, isegp
        else:
            ip2, ip3, iseg1, iseg2 = seg(isegp - 1), seg(isegp + 1), isegp, nseg
        ips = np.asarray([seg(k) for k in range(iseg1, iseg2 + 1)])
        v = self._undo_pbc_chain(ic)
        if mp.ipivotrotmode == 1:
            axis = v[ip2] - v[ip1]
        elif mp.ipivotrotmode == 2:
            # the reference's cross product, including its use of x of ip1
            # in two of the terms (mc.F90:2111-2113)
            axis = np.array([
                +(v[ip2][1] - v[ip1][1]) * (v[ip3][2] - v[ip1][2]) - (v[ip3][1] - v[ip1][1]) * (v[ip2][2] - v[ip1][0]),
                -(v[ip2][0] - v[ip1][0]) * (v[ip3][2] - v[ip1][2]) + (v[ip3][0] - v[ip1][0]) * (v[ip2][2] - v[ip1][0]),
                +(v[ip2][0] - v[ip1][0]) * (v[ip3][1] - v[ip1][1]) - (v[ip3][0] - v[ip1][0]) * (v[ip2][1] - v[ip1][1]),
            ])
            if np.abs(axis).sum() < 1e-10:
                axis = self.rng.sphere()
        elif mp.ipivotrotmode == 3:
            axis = self.rng.sphere()
        else:
            raise ValueError(f"ipivotrotmode = {mp.ipivotrotmode}")
        alpha = (mp.drotpivot * (units.Pi / 180.0)) * (self.rng() - 0.5)   # drotpivot*sclang
        rot = axis_angle_matrix(axis, alpha)
        origin = v[ip1]
        local = np.array([v[ip] for ip in ips]) - origin
        rotm = origin + local @ rot.T
        drotm = rotm - np.array([v[ip] for ip in ips])
        rotm = self._pbc(rotm)
        return self._try("pivot", ips, rotm, drotm)

    # ---- a pass ------------------------------------------------------------
    def run_pass(self):
        """MCPass: np trial moves, then the list update (NListDriver)."""
        np_ = self.s.np_
        self.drostep[:] = 0.0
        for ipass in range(1, np_ + 1):
            ipmove = ipass if self.isamp == 0 else 1 + int(np_ * self.rng())
            ipmove = max(1, min(ipmove, np_))
            ipt = int(self.s.iptpn[ipmove - 1]) - 1
            a, a2, b, c, c2, moving = self.cum[ipt]
            if not moving:
                continue
            mp = self.p[ipt]
            if a > 1.0 - 1e-15:
                self.spart(ipmove, mp)
                continue
            pr = self.rng()
            if pr < a:
                self.spart(ipmove, mp)
            elif pr < a2:
                self.spartcl2(ipmove, mp)
            elif pr < b:
                self.pivot(ipmove, mp)
            elif pr < c or mp.pbrush + mp.pbrushcl2 <= 0.0:
                self.chain(ipmove, mp)
            elif pr < c2 or mp.pbrushcl2 <= 0.0:
                self.brush(ipmove, mp)
            else:
                self.brushcl2(ipmove, mp)
        self.e.NList("step", self.drostep.reshape(-1))
