"""Host-side description of a charged monoatomic MOLSIM system.

`System` holds what the reference keeps in MolModule for the hot path
(particle types, charges, box, cutoffs, Ewald and list options, bonds) as
numpy arrays, builds the two-body table with the library's restatement of
PotTwoBodyTab1 (potential.F90:868), and marshals everything into the
mg_params structure of the C ABI.
"""
from dataclasses import dataclass, field
from typing import List, Optional

import ctypes as C
import numpy as np

from . import abi, units


@dataclass
class Species:
    """One particle type (nmlParticle: zat, sigat, epsat, radat, massat;
    nmlBD: dcoeff)."""
    name: str
    charge: float
    sigma: float          # Angstrom
    eps: float            # kJ/mol
    mass: float = 1.0     # g/mol
    dcoeff: float = 1.0   # units of 1e-9 m^2/s
    radat: float = 0.0    # hard-core radius, r2atat = (radat_i + radat_j)**2


def iptpt_matrix(npt):
    """iptpt(ipt,jpt) of the reference (particle.F90:1535-1541), stored
    column-major as a flat array of npt*npt 1-based pair indices."""
    m = np.zeros((npt, npt), dtype=np.int32)
    k = 0
    for i in range(npt):
        for j in range(i, npt):
            k += 1
            m[i, j] = k
            m[j, i] = k
    return np.ascontiguousarray(m.T.reshape(-1))   # column-major flatten


@dataclass
class System:
    species: List[Species]
    iptpn: np.ndarray                 # (np,) 1-based type of each particle
    ro: np.ndarray                    # (np, 3) positions, box centred at 0
    boxlen: np.ndarray                # (3,)
    temp: float = 298.0
    relpermitt: float = 1.0
    rcut: float = 10.0
    drnlist: float = 0.0
    txintlist: int = abi.MG_VLIST
    mode: int = abi.MG_MD
    maxnneigh: int = 0
    ewald: int = abi.MG_EWALD_NONE
    ualpha: float = 0.0
    ncut: int = 0
    ncutregion_cube: int = 0
    order: int = 0
    nmesh: int = 0
    lsurf: int = 0
    lljcut: int = 0
    ljrcut: float = field(default_factory=units.ljrcut_default)
    ljushift: float = 1.0
    r2uminin: float = 0.1
    utoltab: float = field(default_factory=units.tol_default)
    ftoltab: float = field(default_factory=units.tol_default)
    umaxtab: float = 20000.0
    fmaxtab: float = 20000.0
    bond_ip: Optional[np.ndarray] = None
    bond_jp: Optional[np.ndarray] = None
    bond_k: Optional[np.ndarray] = None
    bond_eq: Optional[np.ndarray] = None
    bond_p: Optional[np.ndarray] = None
    # chain angles jm-ip-jp (1-based), u = k*(theta-eq)**p (UAngle)
    angle_jm: Optional[np.ndarray] = None
    angle_ip: Optional[np.ndarray] = None
    angle_jp: Optional[np.ndarray] = None
    angle_k: Optional[np.ndarray] = None
    angle_eq: Optional[np.ndarray] = None
    angle_p: Optional[np.ndarray] = None
    name: str = "system"
    # table (filled by build_table)
    ubuf: Optional[np.ndarray] = None
    iubuflow: Optional[np.ndarray] = None
    r2umin: Optional[np.ndarray] = None
    nugrid: Optional[np.ndarray] = None

    # ---- plain-data form (JSON) ------------------------------------------
    _TABLE_FIELDS = ("ubuf", "iubuflow", "r2umin", "nugrid")

    def to_dict(self):
        """The system as plain data (lists, numbers, strings) for JSON; the
        two-body table is left out (build_table makes it again)."""
        import dataclasses
        out = {}
        for f in dataclasses.fields(self):
            if f.name in self._TABLE_FIELDS:
                continue
            v = getattr(self, f.name)
            if f.name == "species":
                out[f.name] = [dataclasses.asdict(sp) for sp in v]
            elif isinstance(v, np.ndarray):
                out[f.name] = {"dtype": str(v.dtype), "shape": list(v.shape), "data": v.reshape(-1).tolist()}
            elif isinstance(v, (np.integer, np.floating)):
                out[f.name] = v.item()
            else:
                out[f.name] = v
        return out

    @classmethod
    def from_dict(cls, d):
        kw = {}
        for k, v in d.items():
            if k == "species":
                kw[k] = [Species(**sp) for sp in v]
            elif isinstance(v, dict) and "dtype" in v:
                kw[k] = np.asarray(v["data"], dtype=v["dtype"]).reshape(v["shape"])
            else:
                kw[k] = v
        return cls(**kw)

    # ---- derived quantities -------------------------------------------
    @property
    def np_(self):
        return int(self.iptpn.shape[0])

    @property
    def npt(self):
        return len(self.species)

    @property
    def nptpt(self):
        return self.npt * (self.npt + 1) // 2

    @property
    def epsi_four_pi(self):
        return units.Epsi0FourPi / self.relpermitt

    @property
    def az(self):
        z = np.array([s.charge for s in self.species], dtype=np.float64)
        return np.ascontiguousarray(z[self.iptpn - 1])

    @property
    def vol(self):
        return float(self.boxlen[0] * self.boxlen[1] * self.boxlen[2])

    def r2atat(self):
        npt = self.npt
        m = iptpt_matrix(npt).reshape(npt, npt).T
        r2 = np.zeros(self.nptpt)
        for i in range(npt):
            for j in range(i, npt):
                r2[m[i, j] - 1] = (self.species[i].radat + self.species[j].radat) ** 2
        return r2

    def ro_flat(self):
        """ro(3,np) column-major: x,y,z of particle 1, particle 2, ..."""
        return np.ascontiguousarray(np.asarray(self.ro, dtype=np.float64).reshape(-1))

    # ---- two-body table -------------------------------------------------
    def pot_params(self):
        keep = {
            "iptpt": iptpt_matrix(self.npt),
            "zat": abi.as_f64([s.charge for s in self.species]),
            "sigat": abi.as_f64([s.sigma for s in self.species]),
            "epsat": abi.as_f64([s.eps for s in self.species]),
        }
        pp = abi.MgPotParams(
            npt=self.npt, iptpt=abi.i32(keep["iptpt"]), zat=abi.f64(keep["zat"]),
            sigat=abi.f64(keep["sigat"]), epsat=abi.f64(keep["epsat"]),
            rcut=self.rcut, ualpha=self.ualpha, epsi_four_pi=self.epsi_four_pi,
            lcharge_ewald=int(self.ewald != abi.MG_EWALD_NONE),
            lljcut=self.lljcut, ljrcut=self.ljrcut, ljushift=self.ljushift,
            r2uminin=self.r2uminin, utoltab=self.utoltab, ftoltab=self.ftoltab,
            umaxtab=self.umaxtab, fmaxtab=self.fmaxtab)
        return pp, keep

    def build_table(self, tabfn=None):
        """Run PotTwoBodyTab1 through `tabfn` (default: the library's
        mg_pot_twobody_tab; tests pass the oracle's).  Grows the buffer as
        the reference does (nbuf *= 3) until it fits."""
        if tabfn is None:
            tabfn = abi.load_library().mg_pot_twobody_tab
        pp, keep = self.pot_params()
        cap = 1000
        while True:
            ubuf = np.zeros(cap)
            used = np.zeros(1, dtype=np.int32)
            iub = np.zeros(self.nptpt, dtype=np.int32)
            r2umin = np.zeros(self.nptpt)
            nug = np.zeros(self.nptpt, dtype=np.int32)
            st = tabfn(C.byref(pp), abi.f64(ubuf), cap, abi.i32(used), abi.i32(iub),
                       abi.f64(r2umin), abi.i32(nug))
            if st == 0:
                break
            if used[0] > cap and cap < 10_000_000:
                cap = max(3 * cap, int(used[0]))
                continue
            raise RuntimeError(f"two-body table construction failed: {abi.STATUS.get(st, st)}")
        self.ubuf = np.ascontiguousarray(ubuf[: used[0]])
        self.iubuflow, self.r2umin, self.nugrid = iub, r2umin, nug
        return self

    # ---- C ABI marshalling ----------------------------------------------
    def params(self, form=abi.MG_FP64):
        if self.ubuf is None:
            raise RuntimeError("build_table() must run before params()")
        keep = {
            "iptpn": abi.as_i32(self.iptpn), "iptpt": iptpt_matrix(self.npt),
            "az": self.az, "ubuf": abi.as_f64(self.ubuf), "iubuflow": abi.as_i32(self.iubuflow),
            "r2umin": abi.as_f64(self.r2umin), "r2atat": abi.as_f64(self.r2atat()),
        }
        nb = 0 if self.bond_ip is None else int(len(self.bond_ip))
        if nb:
            keep.update(bond_ip=abi.as_i32(self.bond_ip), bond_jp=abi.as_i32(self.bond_jp),
                        bond_k=abi.as_f64(self.bond_k), bond_eq=abi.as_f64(self.bond_eq),
                        bond_p=abi.as_i32(self.bond_p))
        na = 0 if self.angle_ip is None else int(len(self.angle_ip))
        if na:
            keep.update(angle_jm=abi.as_i32(self.angle_jm), angle_ip=abi.as_i32(self.angle_ip),
                        angle_jp=abi.as_i32(self.angle_jp), angle_k=abi.as_f64(self.angle_k),
                        angle_eq=abi.as_f64(self.angle_eq), angle_p=abi.as_i32(self.angle_p))
        p = abi.MgParams()
        p.abi_version = abi.MG_ABI_VERSION
        p.np = self.np_
        p.npt = self.npt
        p.nptpt = self.nptpt
        p.iptpn = abi.i32(keep["iptpn"])
        p.iptpt = abi.i32(keep["iptpt"])
        p.az = abi.f64(keep["az"])
        p.nbuf = int(len(self.ubuf))
        p.ubuf = abi.f64(keep["ubuf"])
        p.iubuflow = abi.i32(keep["iubuflow"])
        p.r2umin = abi.f64(keep["r2umin"])
        p.r2atat = abi.f64(keep["r2atat"])
        for m in range(3):
            p.boxlen[m] = float(self.boxlen[m])
        p.rcut = self.rcut
        p.drnlist = self.drnlist
        p.txintlist = self.txintlist
        p.mode = self.mode
        p.form = form
        p.maxnneigh = self.maxnneigh
        p.ewald = self.ewald
        p.ualpha = self.ualpha
        p.ncut = self.ncut
        p.ncutregion_cube = self.ncutregion_cube
        p.order = self.order
        p.nmesh = self.nmesh
        p.lsurf = self.lsurf
        p.epsi_four_pi = self.epsi_four_pi
        p.force_fac = units.FORCE_FAC
        p.nbond = nb
        if nb:
            p.bond_ip = abi.i32(keep["bond_ip"])
            p.bond_jp = abi.i32(keep["bond_jp"])
            p.bond_k = abi.f64(keep["bond_k"])
            p.bond_eq = abi.f64(keep["bond_eq"])
            p.bond_p = abi.i32(keep["bond_p"])
        p.nangle = na
        if na:
            for f in ("angle_jm", "angle_ip", "angle_jp", "angle_p"):
                setattr(p, f, abi.i32(keep[f]))
            p.angle_k = abi.f64(keep["angle_k"])
            p.angle_eq = abi.f64(keep["angle_eq"])
        return p, keep

    # ---- integrator inputs --------------------------------------------------
    def massip(self):
        m = np.array([s.mass for s in self.species], dtype=np.float64)
        return np.ascontiguousarray(1.0 / m[self.iptpn - 1])

    def bd_factors(self, tstep):
        f = [units.bd_factors(tstep, s.dcoeff, self.temp) for s in self.species]
        return abi.as_f64([a for a, _ in f]), abi.as_f64([b for _, b in f])

    def maxwell_velocities(self, seed=1):
        """Maxwell-Boltzmann velocities (Angstrom/ps) at self.temp with the
        centre-of-mass motion removed."""
        rng = np.random.Generator(np.random.PCG64(seed))
        m = np.array([s.mass for s in self.species])[self.iptpn - 1]
        # kT/m in (Angstrom/ps)^2: J/mol / (kg/mol) = m^2/s^2 = 1e-4 A^2/ps^2
        sd = np.sqrt(units.GasConstant * self.temp / (m * 1e-3)) * 1e-2
        v = rng.standard_normal((self.np_, 3)) * sd[:, None]
        v -= (m[:, None] * v).sum(0) / m.sum()
        return np.ascontiguousarray(v.reshape(-1))
