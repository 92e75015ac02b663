"""Polyatomic particles: the two-body energy over atom pairs (UTwoBodyP,
energy.F90:786-896) through the library's mg_poly_* entry points.

A `PolySystem` holds atom types (charge, LJ sigma and epsilon), particle
types as rigid sets of atoms (local positions), the particles (type,
centre) and their orientations; `atom_positions` places the atoms as the
reference does (r = ro + ori . local, the local frame rotated by the
particle's orientation matrix).  The pair table runs over atom-type pairs:
PotTwoBodyTab1 (potential.F90:868) with the atom types as its types.
`PolyEngine.UTwoBodyP` evaluates u%twob, the atom forces and the virial for
a particle neighbour list (NList's nneighpn, jpnlist).

Rigid-body molecular dynamics (VelVer with lpolyatom, md.F90:252-420):
`PolySystem.principal_axes` re-expresses each particle type in its
principal axes (PAxesSystem, particle.F90:2350-2420) with the particles'
centres at their centres of mass, `PolyEngine.RigidSetup` puts the
integrator state on the device and `PolyEngine.VelVer` advances it, one
UTotal per step.
"""
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import ctypes as C
import numpy as np

from . import abi, units
from .engine import MolsimError
from .system import iptpt_matrix

__all__ = ["AtomType", "ParticleType", "PolySystem", "PolyEngine", "qua_to_ori", "ori_to_qua"]


@dataclass
class AtomType:
    name: str
    charge: float
    sigma: float
    eps: float
    mass: float = 1.0     # g/mol (massat)


def qua_to_ori(qua):
    """QuaToOri (mollib.F90:2221-2255) for qua (n, 4): ori (n, 3, 3) with
    atom position = ro + ori @ local."""
    q = np.asarray(qua, dtype=np.float64).reshape(-1, 4)
    q0, q1, q2, q3 = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    o = np.empty((len(q), 3, 3))
    o[:, 0, 0] = -q2 * q2 + q1 * q1 - q3 * q3 + q0 * q0
    o[:, 1, 0] = 2.0 * (q0 * q3 - q1 * q2)
    o[:, 2, 0] = 2.0 * (q1 * q3 + q0 * q2)
    o[:, 0, 1] = -2.0 * (q1 * q2 + q0 * q3)
    o[:, 1, 1] = q2 * q2 - q1 * q1 - q3 * q3 + q0 * q0
    o[:, 2, 1] = 2.0 * (q0 * q1 - q2 * q3)
    o[:, 0, 2] = 2.0 * (q1 * q3 - q0 * q2)
    o[:, 1, 2] = -2.0 * (q2 * q3 + q0 * q1)
    o[:, 2, 2] = -q2 * q2 - q1 * q1 + q3 * q3 + q0 * q0
    return o


def ori_to_qua(ori):
    """OriToQua (mollib.F90:2166-2212): the quaternion of each orientation
    matrix from its largest diagonal combination, then normalised."""
    o = np.asarray(ori, dtype=np.float64).reshape(-1, 3, 3)
    out = np.empty((len(o), 4))
    for i, a in enumerate(o):
        tr = a[0, 0] + a[1, 1] + a[2, 2]
        d = [0.25 * (1.0 + tr), 0.25 * (1.0 + 2.0 * a[0, 0] - tr), 0.25 * (1.0 + 2.0 * a[1, 1] - tr),
             0.25 * (1.0 + 2.0 * a[2, 2] - tr)]
        q = np.empty(4)
        if d[0] >= d[1] and d[0] >= d[2] and d[0] >= d[3]:
            q[0] = np.sqrt(d[0]); f = 0.25 / q[0]
            q[1], q[2], q[3] = f * (a[2, 1] - a[1, 2]), f * (a[2, 0] - a[0, 2]), f * (a[1, 0] - a[0, 1])
        elif d[1] >= d[2] and d[1] >= d[3] and d[1] >= d[0]:
            q[1] = np.sqrt(d[1]); f = 0.25 / q[1]
            q[2], q[3], q[0] = f * (-a[1, 0] - a[0, 1]), f * (a[2, 0] + a[0, 2]), f * (a[2, 1] - a[1, 2])
        elif d[2] >= d[3] and d[2] >= d[0] and d[2] >= d[1]:
            q[2] = np.sqrt(d[2]); f = 0.25 / q[2]
            q[3], q[0], q[1] = f * (-a[2, 1] - a[1, 2]), f * (a[2, 0] - a[0, 2]), f * (-a[1, 0] - a[0, 1])
        else:
            q[3] = np.sqrt(d[3]); f = 0.25 / q[3]
            q[0], q[1], q[2] = f * (a[1, 0] - a[0, 1]), f * (a[2, 0] + a[0, 2]), f * (-a[2, 1] - a[1, 2])
        out[i] = q / np.sqrt((q * q).sum())
    return out


@dataclass
class ParticleType:
    name: str
    atoms: List[Tuple[int, Tuple[float, float, float]]]   # (atom type, 0-based; local position)
    # point dipoles of the atoms in the local frame (e A; dipain), for
    # txelec = 'dip'; None: no dipoles
    dipoles: Optional[List[Tuple[float, float, float]]] = None


@dataclass
class PolySystem:
    atom_types: List[AtomType]
    particle_types: List[ParticleType]
    iptpn: np.ndarray                 # (np,) 1-based particle type
    ro: np.ndarray                    # (np, 3) centres
    ori: np.ndarray                   # (np, 3, 3) orientation matrices
    boxlen: np.ndarray
    rcut: float = 10.0
    relpermitt: float = 1.0
    lmc: int = 0
    r2uminin: float = 0.1
    # Ewald over the atom charges (none, standard or SPME, as mg_params)
    ewald: int = abi.MG_EWALD_NONE
    ualpha: float = 0.0
    ncut: int = 0
    order: int = 0
    nmesh: int = 0
    # 'charge': atom charges through the pair table and Ewald; 'dip':
    # charges and point dipoles through UDipole, the table without Coulomb
    txelec: str = "charge"
    lsurf: int = 0
    ubuf: Optional[np.ndarray] = None
    iubuflow: Optional[np.ndarray] = None
    r2umin: Optional[np.ndarray] = None
    keep: dict = field(default_factory=dict)

    @property
    def np_(self):
        return int(len(self.iptpn))

    @property
    def npt(self):
        return len(self.particle_types)

    @property
    def nat(self):
        return len(self.atom_types)

    def napt(self):
        return np.array([len(t.atoms) for t in self.particle_types], dtype=np.int32)

    def ianpn(self):
        """First atom (1-based) of each particle: atoms numbered particle by
        particle, as the reference's ianpn."""
        n = self.napt()[self.iptpn - 1]
        return (np.concatenate([[0], np.cumsum(n)[:-1]]) + 1).astype(np.int32)

    def iatan(self):
        return np.concatenate([[a for a, _ in self.particle_types[t - 1].atoms] for t in self.iptpn]).astype(np.int32) + 1

    def atom_positions(self):
        """r = ro + ori . local for every atom, particle by particle."""
        na = self.napt()[self.iptpn - 1]
        first = self.ianpn() - 1
        out = np.empty((int(na.sum()), 3))
        for t, pt in enumerate(self.particle_types, start=1):
            idx = np.flatnonzero(self.iptpn == t)
            if idx.size == 0:
                continue
            loc = np.array([x for _, x in pt.atoms], dtype=np.float64)          # (a, 3)
            pos = self.ro[idx][:, None, :] + np.einsum("nij,aj->nai", self.ori[idx], loc)
            out[(first[idx][:, None] + np.arange(len(loc))[None, :]).reshape(-1)] = pos.reshape(-1, 3)
        return np.ascontiguousarray(out)

    def aza(self):
        return np.array([self.atom_types[t - 1].charge for t in self.iatan()], dtype=np.float64)

    def atom_dipoles(self):
        """dip(3, na): each atom's local dipole rotated by its particle's
        orientation (SetAtomProp), particle by particle; zero where a type
        has none."""
        na = self.napt()[self.iptpn - 1]
        first = self.ianpn() - 1
        out = np.zeros((int(na.sum()), 3))
        for t, pt in enumerate(self.particle_types, start=1):
            if not pt.dipoles:
                continue
            idx = np.flatnonzero(self.iptpn == t)
            if idx.size == 0:
                continue
            loc = np.array(pt.dipoles, dtype=np.float64)
            d = np.einsum("nij,aj->nai", self.ori[idx], loc)
            out[(first[idx][:, None] + np.arange(len(loc))[None, :]).reshape(-1)] = d.reshape(-1, 3)
        return np.ascontiguousarray(out)

    def type_inertia(self, t):
        """Mass, centre of mass and inertia tensor of particle type t
        (0-based) in its local frame (PAxesSystem, particle.F90:2360-2395,
        with entries below 1e-10 set to zero)."""
        pt = self.particle_types[t]
        m = np.array([self.atom_types[a].mass for a, _ in pt.atoms], dtype=np.float64)
        x = np.array([p for _, p in pt.atoms], dtype=np.float64)
        mass = float(m.sum())
        com = (m[:, None] * x).sum(0) / mass
        d = x - com
        tpi = np.zeros((3, 3))
        for k in range(len(m)):
            tpi += m[k] * (np.dot(d[k], d[k]) * np.eye(3) - np.outer(d[k], d[k]))
        tpi[np.abs(tpi) < 1e-10] = 0.0
        return mass, com, tpi

    def principal_axes(self):
        """The same particles with each type's atoms in its principal axes
        about its centre of mass (ra, particle.F90:2409-2420), the centres
        moved to the centres of mass (folded into the box) and the
        orientations composed with the axes, so that every atom stays where
        it was, up to a box vector."""
        from dataclasses import replace
        types, com, axes = [], [], []
        for t, pt in enumerate(self.particle_types):
            _, c, tpi = self.type_inertia(t)
            _, e = np.linalg.eigh(tpi)
            if np.linalg.det(e) < 0.0:
                e[:, 2] = -e[:, 2]
            loc = np.array([p for _, p in pt.atoms], dtype=np.float64)
            ra = (loc - c) @ e
            dips = None if pt.dipoles is None else [tuple(v) for v in np.array(pt.dipoles, dtype=np.float64) @ e]
            types.append(ParticleType(pt.name, [(a, tuple(ra[k])) for k, (a, _) in enumerate(pt.atoms)], dips))
            com.append(c)
            axes.append(e)
        ti = np.asarray(self.iptpn) - 1
        com, axes = np.array(com), np.array(axes)
        ro = self.ro + np.einsum("nij,nj->ni", self.ori, com[ti])
        # a centre moved past a face goes back into the box (PBC): its atoms
        # move by the same box vector
        L = np.asarray(self.boxlen, dtype=np.float64)
        t = ro / L
        a = np.trunc(t) + np.sign(t) * (np.abs(t - np.trunc(t)) >= 0.5)   # ANINT
        ro = np.where(np.abs(ro) > 0.5 * L, ro - L * a, ro)
        ori = np.einsum("nij,njk->nik", self.ori, axes[ti])
        return replace(self, particle_types=types, ro=np.ascontiguousarray(ro), ori=np.ascontiguousarray(ori),
                       ubuf=self.ubuf, iubuflow=self.iubuflow, r2umin=self.r2umin, keep={})

    def rigid_props(self, tol=1e-8):
        """Per particle: inverse mass (massip) and principal moments (momp),
        for particle types already in their principal axes."""
        mass, momp = [], []
        for t in range(self.npt):
            m, c, tpi = self.type_inertia(t)
            off = tpi - np.diag(np.diag(tpi))
            scale = max(1.0, float(np.abs(tpi).max()))
            if np.abs(c).max() > tol * max(1.0, float(np.abs(c).max()) + 1.0) or np.abs(off).max() > tol * scale:
                raise ValueError(f"particle type {self.particle_types[t].name!r} is not in its principal axes: "
                                 "use PolySystem.principal_axes()")
            mass.append(m)
            momp.append(np.diag(tpi).copy())
        ti = np.asarray(self.iptpn) - 1
        return (np.ascontiguousarray(1.0 / np.array(mass)[ti]), np.ascontiguousarray(np.array(momp)[ti]))

    def kinetic_energy(self, rod, angvelo):
        """Translational and rotational kinetic energy in kJ/mol for
        velocities in A/ps and angular velocities (principal frame) in
        rad/ps: 0.005 * (sum m v^2 + sum I w^2)."""
        massip, momp = self.rigid_props()
        rod = np.asarray(rod).reshape(-1, 3)
        w = np.asarray(angvelo).reshape(-1, 3)
        return 0.005 * float(((rod * rod).sum(1) / massip).sum()), 0.005 * float((momp * w * w).sum())

    @property
    def epsi_four_pi(self):
        return units.Epsi0FourPi / self.relpermitt

    def atoms_in_box(self, r=None):
        """Atom positions folded into the box (PBC, molaux.F90:104-146) for
        the Ewald sums, which are periodic in each atom position: an atom of
        a particle near a face may lie just outside the box."""
        r = self.atom_positions() if r is None else np.array(r, dtype=np.float64).reshape(-1, 3)
        L = np.asarray(self.boxlen, dtype=np.float64)
        out = r.copy()
        for m in range(3):
            big = np.abs(out[:, m]) > 0.5 * L[m]
            t = out[:, m] * (1.0 / L[m])
            a = np.trunc(t)
            a = a + np.sign(t) * (np.abs(t - a) >= 0.5)
            out[:, m] = np.where(big, out[:, m] - L[m] * a, out[:, m])
        return np.ascontiguousarray(out)

    def build_table(self, tabfn):
        """PotTwoBodyTab1 over the atom types: (1,6,12) Lennard-Jones plus
        Coulomb, the real-space Ewald part (CalcEwaldUfac) when Ewald is on."""
        nat = self.nat
        # a dipole system's table holds no Coulomb term (qq = 0 with
        # ldipole, potential.F90:1380): UDipole takes all electrostatics
        dip = self.txelec == "dip"
        keep = {"iptpt": iptpt_matrix(nat),
                "zat": abi.as_f64([0.0 if dip else a.charge for a in self.atom_types]),
                "sigat": abi.as_f64([a.sigma for a in self.atom_types]),
                "epsat": abi.as_f64([a.eps for a in self.atom_types])}
        pp = abi.MgPotParams(npt=nat, iptpt=abi.i32(keep["iptpt"]), zat=abi.f64(keep["zat"]),
                             sigat=abi.f64(keep["sigat"]), epsat=abi.f64(keep["epsat"]), rcut=self.rcut,
                             ualpha=self.ualpha, epsi_four_pi=self.epsi_four_pi,
                             lcharge_ewald=int(self.ewald != abi.MG_EWALD_NONE and not dip),
                             lljcut=0, ljrcut=units.ljrcut_default(), ljushift=1.0, r2uminin=self.r2uminin,
                             utoltab=units.tol_default(), ftoltab=units.tol_default(), umaxtab=20000.0,
                             fmaxtab=20000.0)
        natat = nat * (nat + 1) // 2
        cap = 4000
        while True:
            ubuf = np.zeros(cap)
            used = np.zeros(1, dtype=np.int32)
            iub = np.zeros(natat, dtype=np.int32)
            r2 = np.zeros(natat)
            nug = np.zeros(natat, dtype=np.int32)
            st = tabfn(C.byref(pp), abi.f64(ubuf), cap, abi.i32(used), abi.i32(iub), abi.f64(r2), abi.i32(nug))
            if st == 0:
                break
            if used[0] > cap and cap < 10_000_000:
                cap = max(3 * cap, int(used[0]))
                continue
            raise RuntimeError(f"atom-pair table construction failed: {abi.STATUS.get(st, st)}")
        self.ubuf, self.iubuflow, self.r2umin = np.ascontiguousarray(ubuf[: used[0]]), iub, r2
        return self

    def params(self):
        if self.ubuf is None:
            raise RuntimeError("build_table() must run before params()")
        k = {"iptpn": abi.as_i32(self.iptpn), "iptpt": iptpt_matrix(self.npt), "napt": self.napt(),
             "ianpn": self.ianpn(), "iatan": self.iatan(), "iatat": iptpt_matrix(self.nat),
             "ubuf": abi.as_f64(self.ubuf), "iubuflow": abi.as_i32(self.iubuflow), "r2umin": abi.as_f64(self.r2umin),
             "aza": self.aza(), "r2atat": np.zeros(self.nat * (self.nat + 1) // 2)}
        p = abi.MgPolyParams()
        p.abi_version = abi.MG_ABI_VERSION
        p.np, p.npt, p.nptpt = self.np_, self.npt, self.npt * (self.npt + 1) // 2
        p.iptpn, p.iptpt, p.napt = abi.i32(k["iptpn"]), abi.i32(k["iptpt"]), abi.i32(k["napt"])
        p.na = int(len(k["iatan"]))
        p.ianpn, p.iatan = abi.i32(k["ianpn"]), abi.i32(k["iatan"])
        p.nat, p.natat = self.nat, self.nat * (self.nat + 1) // 2
        p.iatat = abi.i32(k["iatat"])
        p.nbuf = int(len(self.ubuf))
        p.ubuf, p.iubuflow, p.r2umin = abi.f64(k["ubuf"]), abi.i32(k["iubuflow"]), abi.f64(k["r2umin"])
        p.r2atat = abi.f64(k["r2atat"])   # atoms without a hard core
        for m in range(3):
            p.boxlen[m] = float(self.boxlen[m])
        p.rcut = self.rcut
        p.lmc = self.lmc
        p.aza = abi.f64(k["aza"])
        p.ualpha = self.ualpha
        p.epsi_four_pi = self.epsi_four_pi
        p._keep = k        # the arrays live as long as the structure that points at them
        self.keep = k
        return p

    def centre_system(self, skin=1.0):
        """The particle centres as a monoatomic System whose handle keeps the
        particle list on the device (mg_poly_utwobody_list): one species per
        particle type, no charges, no Ewald, a two-body table that is zero."""
        from .system import Species, System
        sp = [Species(t.name, 0.0, 1.0, 0.0) for t in self.particle_types]
        npt = self.npt
        nptpt = npt * (npt + 1) // 2
        ubuf = np.zeros(12 * nptpt)
        ubuf[0::12] = 1e-4
        c = System(species=sp, iptpn=np.asarray(self.iptpn, dtype=np.int32), ro=np.asarray(self.ro),
                   boxlen=np.asarray(self.boxlen), rcut=self.rcut, drnlist=skin, txintlist=abi.MG_VLIST,
                   mode=abi.MG_MD, ewald=abi.MG_EWALD_NONE, name="centres")
        c.ubuf = ubuf
        c.iubuflow = (np.arange(nptpt, dtype=np.int32) * 12 + 1)
        c.r2umin = np.full(nptpt, 1e-4)
        c.nugrid = np.ones(nptpt, dtype=np.int32)
        return c

    def atom_system(self, rlist=3.0, skin=0.5):
        """The atoms as a monoatomic System for the reciprocal Ewald sum (and
        the atomic self term) through a handle: the atom types as species,
        a two-body table that is zero everywhere (the atom pairs' real-space
        terms belong to UTwoBodyP), a short list cutoff."""
        from .system import Species, System
        sp = [Species(a.name, a.charge, 1.0, 0.0) for a in self.atom_types]
        nat = self.nat
        natat = nat * (nat + 1) // 2
        ubuf = np.zeros(12 * natat)
        ubuf[0::12] = 1e-4                       # one zero record from r^2 = 1e-4 up
        s = System(species=sp, iptpn=self.iatan(), ro=self.atoms_in_box(), boxlen=np.asarray(self.boxlen),
                   relpermitt=self.relpermitt, rcut=rlist, drnlist=skin, ewald=self.ewald, ualpha=self.ualpha,
                   ncut=self.ncut, order=self.order, nmesh=self.nmesh, lsurf=0, name="atoms")
        s.ubuf = ubuf
        s.iubuflow = (np.arange(natat, dtype=np.int32) * 12 + 1)
        s.r2umin = np.full(natat, 1e-4)
        s.nugrid = np.ones(natat, dtype=np.int32)
        return s


class PolyEngine:
    """mg_poly_* for one PolySystem; maxnneigh is the list's leading size."""

    def __init__(self, system, maxnneigh, lib=None):
        self.s = system
        self.lib = lib or abi.load_library()
        self.p = system.params()
        self.maxnneigh = int(maxnneigh)
        self.h = C.c_void_p()
        st = self.lib.mg_poly_create(C.byref(self.p), self.maxnneigh, C.byref(self.h))
        if st != 0:
            raise MolsimError(st, "poly_create")

    def UTwoBodyP(self, nneighpn, jpnlist, r=None):
        s = self.s
        r = s.atom_positions() if r is None else np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
        force = np.zeros(3 * len(r))
        ut = np.zeros(self.p.nptpt + 1)
        vir = np.zeros(1)
        nn = abi.as_i32(nneighpn)
        jl = abi.as_i32(np.asarray(jpnlist).reshape(-1))
        st = self.lib.mg_poly_utwobody(self.h, abi.f64(abi.as_f64(s.ro.reshape(-1))), abi.f64(r.reshape(-1)),
                                       abi.i32(nn), abi.i32(jl), abi.f64(force), abi.f64(ut), abi.f64(vir))
        if st != 0:
            buf = C.create_string_buffer(512)
            self.lib.mg_poly_last_error(self.h, buf, 512)
            raise MolsimError(st, f"poly_utwobody: {buf.value.decode(errors='replace')}")
        return dict(force=force.reshape(-1, 3), u_twob=ut, virial=float(vir[0]))

    def UTwoBodyPList(self, r=None):
        """UTwoBodyP with the particle list on the device: a handle of the
        centres (kept between calls) rebuilds its list from the current
        centres, and only the atom positions are copied."""
        from .engine import Engine
        s = self.s
        r = s.atom_positions() if r is None else np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
        if getattr(self, "_centres", None) is None:
            self._centres = Engine(s.centre_system())
        e = self._centres
        e.SetPositions(abi.as_f64(s.ro.reshape(-1)))
        e.NList("write")
        force = np.zeros(3 * len(r))
        ut = np.zeros(self.p.nptpt + 1)
        vir = np.zeros(1)
        st = self.lib.mg_poly_utwobody_list(self.h, e.h, abi.f64(r.reshape(-1)), abi.f64(force), abi.f64(ut),
                                            abi.f64(vir))
        if st != 0:
            buf = C.create_string_buffer(512)
            self.lib.mg_poly_last_error(self.h, buf, 512)
            raise MolsimError(st, f"poly_utwobody_list: {buf.value.decode(errors='replace')}")
        return dict(force=force.reshape(-1, 3), u_twob=ut, virial=float(vir[0]))

    def DUTwoBodyBatch(self, nneighpn, jpnlist, ips, rotm, rtm, r=None):
        """Independent single-particle trials against the current state:
        particle ips[t] to centre rotm[t] with atoms rtm (the trials' atoms
        one after another).  Returns du_twob (u%twob(0) new minus old) and
        the hard-core overlap flags."""
        s = self.s
        r = s.atom_positions() if r is None else np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
        ips = abi.as_i32(np.atleast_1d(ips))
        n = len(ips)
        du = np.zeros(n)
        ovl = np.zeros(n, dtype=np.int32)
        st = self.lib.mg_poly_dutwobody_batch(
            self.h, abi.f64(abi.as_f64(s.ro.reshape(-1))), abi.f64(r.reshape(-1)), abi.i32(abi.as_i32(nneighpn)),
            abi.i32(abi.as_i32(np.asarray(jpnlist).reshape(-1))), n, abi.i32(ips),
            abi.f64(abi.as_f64(np.asarray(rotm).reshape(-1))), abi.f64(abi.as_f64(np.asarray(rtm).reshape(-1))),
            abi.f64(du), abi.i32(ovl))
        if st != 0:
            buf = C.create_string_buffer(512)
            self.lib.mg_poly_last_error(self.h, buf, 512)
            raise MolsimError(st, f"poly_dutwobody_batch: {buf.value.decode(errors='replace')}")
        return du, ovl.astype(bool)

    def DUTwoBodyMulti(self, nneighpn, jpnlist, ips, rotm, rtm, r=None):
        """One trial moving the particles ips (1-based) together to centres
        rotm with atoms rtm (the moving particles' atoms one after another):
        DUTwoBody's UTwoBodyPNew/UTwoBodyPOld for nptm = len(ips).  Returns
        du_twob per particle-type pair (index 0 the total; new minus old) and
        the hard-core overlap flag."""
        s = self.s
        r = s.atom_positions() if r is None else np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
        ips = abi.as_i32(np.atleast_1d(ips))
        du = np.zeros(self.p.nptpt + 1)
        ovl = np.zeros(1, dtype=np.int32)
        st = self.lib.mg_poly_dutwobody_multi(
            self.h, abi.f64(abi.as_f64(s.ro.reshape(-1))), abi.f64(r.reshape(-1)), abi.i32(abi.as_i32(nneighpn)),
            abi.i32(abi.as_i32(np.asarray(jpnlist).reshape(-1))), len(ips), abi.i32(ips),
            abi.f64(abi.as_f64(np.asarray(rotm).reshape(-1))), abi.f64(abi.as_f64(np.asarray(rtm).reshape(-1))),
            abi.f64(du), abi.i32(ovl))
        if st != 0:
            buf = C.create_string_buffer(512)
            self.lib.mg_poly_last_error(self.h, buf, 512)
            raise MolsimError(st, f"poly_dutwobody_multi: {buf.value.decode(errors='replace')}")
        return du, bool(ovl[0])

    def Epilogue(self, force, r=None, torque=None):
        """UTotal's end (energy.F90:405-427): particle forces and torques
        (scaled by force_fac) from the atom forces and, with dipoles, the
        atom torques, and the molecular virial."""
        s = self.s
        r = s.atom_positions() if r is None else np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
        fo = np.zeros(3 * s.np_)
        to = np.zeros(3 * s.np_)
        vm = np.zeros(1)
        tq = None if torque is None else abi.f64(abi.as_f64(np.asarray(torque).reshape(-1)))
        st = self.lib.mg_poly_epilogue(self.h, abi.f64(abi.as_f64(s.ro.reshape(-1))), abi.f64(r.reshape(-1)),
                                       abi.f64(abi.as_f64(np.asarray(force).reshape(-1))), tq, units.FORCE_FAC,
                                       abi.f64(fo), abi.f64(to), abi.f64(vm))
        if st != 0:
            raise MolsimError(st, "poly_epilogue")
        return dict(forceo=fo.reshape(-1, 3), torqueo=to.reshape(-1, 3), virmolecule=float(vm[0]))

    def EwaldIntra(self, r=None):
        """The molecular part of UEwaldSelf: its u%rec share and atom forces."""
        s = self.s
        r = s.atom_positions() if r is None else np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
        force = np.zeros(3 * len(r))
        u = np.zeros(1)
        st = self.lib.mg_poly_ewald_intra(self.h, abi.f64(r.reshape(-1)), abi.f64(force), abi.f64(u))
        if st != 0:
            raise MolsimError(st, "poly_ewald_intra")
        return dict(force=force.reshape(-1, 3), u_rec=float(u[0]))

    def _list(self, nneighpn, jpnlist):
        """The particle list (nneighpn, jpnlist) given, or NList's list of
        the kept handle of the centres."""
        if nneighpn is not None:
            return abi.as_i32(nneighpn), abi.as_i32(np.asarray(jpnlist).reshape(-1))
        from .engine import Engine
        s = self.s
        if getattr(self, "_centres", None) is None:
            self._centres = Engine(s.centre_system())
        e = self._centres
        e.SetPositions(abi.as_f64(s.ro.reshape(-1)))
        e.NList("write")
        nn = np.zeros(s.np_, dtype=np.int32)
        jl = np.zeros(s.np_ * self.maxnneigh, dtype=np.int32)
        e._check(e._fn("nlist_get")(e.h, abi.i32(nn), abi.i32(jl), self.maxnneigh), "nlist_get")
        return nn, jl

    def _atoms_handle(self, engine_factory=None):
        from .engine import Engine
        s = self.s
        if engine_factory is not None:
            return engine_factory(s.atom_system())
        if getattr(self, "_atoms", None) is None:
            self._atoms = Engine(s.atom_system())
        return self._atoms

    def UDipole(self, nneighpn=None, jpnlist=None, dip=None, r=None, engine_factory=None):
        """UDipole (energy.F90:1476-1579) for charges and point dipoles:
        UDipoleP over the particle list, with Ewald the reciprocal part on
        the handle of the atoms, both parts of UDipoleEwaldSelf and (lsurf)
        UDipoleEwaldSurf, then u%stat, atom forces (force(3,na) units) and
        atom torques.  Returns potstat, estat, efg, u_stat, u_rec (u_stat
        minus the real-space part), virial (EpsiFourPi virelec)."""
        s = self.s
        r = s.atom_positions() if r is None else np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
        dip = s.atom_dipoles() if dip is None else np.ascontiguousarray(dip, dtype=np.float64).reshape(-1, 3)
        nn, jl = self._list(nneighpn, jpnlist)
        na = len(r)
        pot, est, efg = np.zeros(na), np.zeros(3 * na), np.zeros(6 * na)
        vir, ureal = np.zeros(1), np.zeros(1)
        self._fail(self.lib.mg_poly_udipole_real(self.h, abi.f64(abi.as_f64(s.ro.reshape(-1))),
                                                 abi.f64(r.reshape(-1)), abi.f64(dip.reshape(-1)), abi.i32(nn),
                                                 abi.i32(jl), abi.f64(pot), abi.f64(est), abi.f64(efg),
                                                 abi.f64(vir), abi.f64(ureal)), "poly_udipole_real")
        if s.ewald != abi.MG_EWALD_NONE:
            e = self._atoms_handle(engine_factory)
            e.SetPositions(s.atoms_in_box(r).reshape(-1))
            e._check(e._fn("dipole_ewald")(e.h, abi.f64(dip.reshape(-1)), abi.f64(pot), abi.f64(est),
                                           abi.f64(efg), abi.f64(vir)), "dipole_ewald")
            if engine_factory is not None:
                e.close()
            self._fail(self.lib.mg_poly_udipole_self(self.h, abi.f64(r.reshape(-1)), abi.f64(dip.reshape(-1)),
                                                     int(s.lsurf), abi.f64(pot), abi.f64(est), abi.f64(efg),
                                                     abi.f64(vir)), "poly_udipole_self")
        force = np.zeros(3 * na)
        torque = np.zeros(3 * na)
        ustat = np.zeros(1)
        self._fail(self.lib.mg_poly_udipole_finish(self.h, abi.f64(dip.reshape(-1)), abi.f64(pot), abi.f64(est),
                                                   abi.f64(efg), abi.f64(force), abi.f64(torque), abi.f64(ustat)),
                   "poly_udipole_finish")
        return dict(potstat=pot, estat=est.reshape(-1, 3), efg=efg.reshape(-1, 6), force=force.reshape(-1, 3),
                    torque=torque.reshape(-1, 3), u_stat=float(ustat[0]), u_rec=float(ustat[0] - ureal[0]),
                    virial=s.epsi_four_pi * float(vir[0]))

    def UTotal(self, nneighpn=None, jpnlist=None, engine_factory=None):
        """UTotal of a polyatomic system: the atom pairs (UTwoBodyP, with the
        real-space Ewald table when Ewald is on), the reciprocal sum and
        atomic self term over the atoms (a handle of the atoms), the
        molecular self term, then UTotal's end: atom forces (force(3,na)
        units), particle forces and torques (forceo, torqueo), the virial."""
        s = self.s
        r = s.atom_positions()
        # no list given: the device-resident list of a centres handle
        tw = self.UTwoBodyPList(r) if nneighpn is None else self.UTwoBodyP(nneighpn, jpnlist, r)
        out = dict(u_twob=tw["u_twob"], virial=tw["virial"], force=tw["force"].copy(), u_rec=0.0)
        if s.txelec == "dip":   # UTwoBodyP then UDipole (energy.F90:366-369)
            d = self.UDipole(nneighpn, jpnlist, r=r, engine_factory=engine_factory)
            out["force"] += d["force"]
            out["virial"] += d["virial"]
            out["u_rec"] = d["u_rec"]
            out["u_stat"] = d["u_stat"]
            out["u_tot"] = out["u_twob"][0] + d["u_stat"]
            ep = self.Epilogue(out["force"], r, torque=d["torque"])
            out.update(forceo=ep["forceo"], torqueo=ep["torqueo"])
            out["virial"] += ep["virmolecule"]
            return out
        if s.ewald != abi.MG_EWALD_NONE:
            e = self._atoms_handle(engine_factory)   # one handle of the atoms, kept for the following calls
            e.SetPositions(s.atoms_in_box(r).reshape(-1))
            e.NList("write")
            rec = e.UTotal()
            intra = self.EwaldIntra(r)
            out["u_rec"] = rec["u_rec"] + intra["u_rec"]
            out["force"] += rec["forceo"] / units.FORCE_FAC + intra["force"]
            out["virial"] += rec["virial"]
        out["u_tot"] = out["u_twob"][0] + out["u_rec"]
        ep = self.Epilogue(out["force"], r)
        out.update(forceo=ep["forceo"], torqueo=ep["torqueo"])
        out["virial"] += ep["virmolecule"]
        return out

    # ---- rigid-body velocity Verlet ---------------------------------------------
    def RigidSetup(self, tstep, rod, angvelo, tvvite=0.0, nvvite=2, rodd=None, quadd=None, prime=False):
        """The integrator state on the device: centres, quaternions
        (OriToQua of the orientations), velocities (A/ps), angular
        velocities (principal frame, rad/ps), accelerations (zero unless
        given, as at the start of a simulation; prime=True takes them from
        a UTotal of the initial state) and tstep (ps), tvvite, nvvite
        (nmlMD)."""
        s = self.s
        massip, momp = s.rigid_props()
        qua = ori_to_qua(s.ori)
        n = s.np_
        rodd = np.zeros(3 * n) if rodd is None else abi.as_f64(np.asarray(rodd).reshape(-1))
        quadd = np.zeros(4 * n) if quadd is None else abi.as_f64(np.asarray(quadd).reshape(-1))
        st = self.lib.mg_poly_rigid_setup(
            self.h, float(tstep), float(tvvite), int(nvvite), abi.f64(massip), abi.f64(abi.as_f64(momp.reshape(-1))),
            abi.f64(abi.as_f64(s.ro.reshape(-1))), abi.f64(abi.as_f64(qua.reshape(-1))),
            abi.f64(abi.as_f64(np.asarray(rod).reshape(-1))), abi.f64(abi.as_f64(np.asarray(angvelo).reshape(-1))),
            abi.f64(rodd), abi.f64(quadd))
        self._fail(st, "poly_rigid_setup")
        if prime:
            u = self.UTotal()
            self._fail(self.lib.mg_poly_rigid_prime(self.h, abi.f64(abi.as_f64(u["forceo"].reshape(-1))),
                                                    abi.f64(abi.as_f64(u["torqueo"].reshape(-1)))),
                       "poly_rigid_prime")
        self.rod = np.asarray(rod, dtype=np.float64).reshape(n, 3).copy()
        self.angvelo = np.asarray(angvelo, dtype=np.float64).reshape(n, 3).copy()

    def VelVer(self, nstep=1, nneighpn=None, jpnlist=None):
        """nstep steps of VelVer: new centres and orientations on the
        device, UTotal (the list of a centres handle unless one is given),
        then the velocity updates.  The system's ro and ori follow.  Returns
        the last step's UTotal with rod and angvelo."""
        s = self.s
        n = s.np_
        ro = np.zeros(3 * n)
        ori = np.zeros(9 * n)
        dro = np.zeros(3 * n)
        rod = np.zeros(3 * n)
        w = np.zeros(3 * n)
        out = None
        for _ in range(nstep):
            self._fail(self.lib.mg_poly_rigid_move(self.h, abi.f64(ro), abi.f64(ori), abi.f64(dro)),
                       "poly_rigid_move")
            s.ro = ro.reshape(n, 3).copy()
            s.ori = np.ascontiguousarray(ori.reshape(n, 3, 3).transpose(0, 2, 1))   # ori(3,3,np) column-major
            out = self.UTotal(nneighpn, jpnlist)
            self._fail(self.lib.mg_poly_rigid_kick(self.h, abi.f64(abi.as_f64(out["forceo"].reshape(-1))),
                                                   abi.f64(abi.as_f64(out["torqueo"].reshape(-1))), abi.f64(rod),
                                                   abi.f64(w)), "poly_rigid_kick")
        self.rod = rod.reshape(n, 3).copy()
        self.angvelo = w.reshape(n, 3).copy()
        out.update(rod=self.rod, angvelo=self.angvelo, drostep=dro.reshape(n, 3).copy())
        return out

    def MDRun(self, nstep=1):
        """nstep steps of VelVer on the device (mg_poly_md_run): the same
        steps as VelVer with the centres' list and the atom handle kept on
        the device and no host arrays between the steps.  The system's ro
        and ori follow; returns u_tot, u_twob0, u_rec, virial, rod,
        angvelo of the last step."""
        from .engine import Engine
        s = self.s
        if s.txelec != "charge":
            raise ValueError("MDRun: charges only (txelec = 'charge')")
        n = s.np_
        if getattr(self, "_centres", None) is None:
            self._centres = Engine(s.centre_system())
            self._centres.SetPositions(abi.as_f64(s.ro.reshape(-1)))
            self._centres.NList("write")
        ha = None
        if s.ewald != abi.MG_EWALD_NONE:
            ha = self._atoms_handle()
            ha.SetPositions(s.atoms_in_box().reshape(-1))
            ha.NList("write")
        ra = abi.as_f64(np.concatenate([np.array([x for _, x in t.atoms], dtype=np.float64).reshape(-1)
                                        for t in s.particle_types]))
        ro, ori = np.zeros(3 * n), np.zeros(9 * n)
        rod, w, uo = np.zeros(3 * n), np.zeros(3 * n), np.zeros(4)
        self._fail(self.lib.mg_poly_md_run(self.h, self._centres.h, ha.h if ha is not None else None, abi.f64(ra),
                                           int(nstep), abi.f64(ro), abi.f64(ori), abi.f64(rod), abi.f64(w),
                                           abi.f64(uo)), "poly_md_run")
        s.ro = ro.reshape(n, 3).copy()
        s.ori = np.ascontiguousarray(ori.reshape(n, 3, 3).transpose(0, 2, 1))
        self.rod = rod.reshape(n, 3).copy()
        self.angvelo = w.reshape(n, 3).copy()
        return dict(u_tot=float(uo[0]), u_twob0=float(uo[1]), u_rec=float(uo[2]), virial=float(uo[3]),
                    rod=self.rod, angvelo=self.angvelo)

    def RigidState(self):
        """The device's quaternions and quaternion velocities, (np, 4) each."""
        n = self.s.np_
        q = np.zeros(4 * n)
        qd = np.zeros(4 * n)
        self._fail(self.lib.mg_poly_rigid_get(self.h, abi.f64(q), abi.f64(qd)), "poly_rigid_get")
        return q.reshape(n, 4), qd.reshape(n, 4)

    def _fail(self, st, what):
        if st != 0:
            buf = C.create_string_buffer(512)
            self.lib.mg_poly_last_error(self.h, buf, 512)
            raise MolsimError(st, f"{what}: {buf.value.decode(errors='replace')}")

    def close(self):
        for k in ("_atoms", "_centres"):
            if getattr(self, k, None) is not None:
                getattr(self, k).close()
                setattr(self, k, None)
        if self.h:
            self.lib.mg_poly_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
