"""Seeded synthetic workloads for the hot path.

The reference ships no benchmark datasets; these generators build the
systems of the measured configurations from seeds (numpy PCG64), following
the placement rule of the reference's SetRandom (coordinate.F90:1302-1340:
uniform positions, overlaps below a minimum distance rejected) and
SetChainRandom (coordinate.F90:1609-1676: random walks of fixed step).

  electrolyte_std   N=1000 ions, L=100, standard Ewald (r_c=30, |n|<=8)
  electrolyte_spme  N=32768 ions, L=817, SPME order 6, 64^3
  polyelectrolyte   64x200-bead chains + 12800 counterions + 20000 salt
                    pairs (N=65600), L=700, SPME order 6, 128^3, BD
  replica_set       independent electrolyte boxes of uneven size and salt
                    concentration for the batched (ensemble) form
  small_system      a scaled-down charged LJ system for parity tests
"""
import math

import numpy as np

from . import abi, units
from .system import Species, System


def alpha_for_erfc(tol, rcut):
    """alpha with erfc(alpha*rcut) = tol (bisection on math.erfc)."""
    lo, hi = 0.0, 20.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if math.erfc(mid) > tol:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi) / rcut


def lj_shift_at(rc_over_sigma):
    """ljushift (in units of eps) that makes the cut LJ zero at rc."""
    x6 = rc_over_sigma ** -6
    return -4.0 * (x6 * x6 - x6)


class _Grid:
    """Cell grid for overlap rejection during placement: no two particles
    closer than rmin, or, for particles added with a radius, than the sum of
    their radii (rmin is then the largest such sum)."""

    def __init__(self, boxlen, rmin):
        self.L = np.asarray(boxlen, dtype=np.float64)
        self.n = np.maximum(1, np.floor(self.L / max(rmin, 1e-9)).astype(int))
        self.h = self.L / self.n
        self.rmin2 = rmin * rmin
        self.cells = {}
        self.pos = []
        self.rad = []

    def _cell(self, r):
        return tuple((np.floor((r + self.L / 2) / self.h).astype(int)) % self.n)

    def ok(self, r, skip=-1, rad=None):
        c = self._cell(r)
        rng = [range(-1, 2) if self.n[m] >= 3 else range(0, self.n[m]) for m in range(3)]
        for dx in rng[0]:
            for dy in rng[1]:
                for dz in rng[2]:
                    key = ((c[0] + dx) % self.n[0], (c[1] + dy) % self.n[1], (c[2] + dz) % self.n[2]) \
                        if self.n.min() >= 3 else (
                        (c[0] + dx) % self.n[0] if self.n[0] >= 3 else dx,
                        (c[1] + dy) % self.n[1] if self.n[1] >= 3 else dy,
                        (c[2] + dz) % self.n[2] if self.n[2] >= 3 else dz)
                    for j in self.cells.get(key, ()):
                        if j == skip:
                            continue
                        d = r - self.pos[j]
                        d -= self.L * np.round(d / self.L)
                        lim2 = self.rmin2 if rad is None or self.rad[j] is None else (rad + self.rad[j]) ** 2
                        if d @ d < lim2:
                            return False
        return True

    def add(self, r, rad=None):
        self.cells.setdefault(self._cell(r), []).append(len(self.pos))
        self.pos.append(r)
        self.rad.append(rad)


def _wrap(r, L):
    return r - L * np.round(r / L)


def place_uniform(rng, grid, n, maxtry=100000):
    out = []
    for _ in range(n):
        for _t in range(maxtry):
            r = (rng.random(3) - 0.5) * grid.L
            if grid.ok(r):
                grid.add(r)
                out.append(r)
                break
        else:
            raise RuntimeError("could not place particle without overlap")
    return out


def place_chain(rng, grid, nseg, bond):
    for _restart in range(1000):
        start = (rng.random(3) - 0.5) * grid.L
        if not grid.ok(start):
            continue
        chain = [start]
        tmp = _Grid(grid.L, math.sqrt(grid.rmin2))
        tmp.add(start)
        good = True
        for _s in range(1, nseg):
            for _t in range(200):
                u = rng.standard_normal(3)
                u /= np.linalg.norm(u)
                r = _wrap(chain[-1] + bond * u, grid.L)
                if grid.ok(r) and tmp.ok(r, skip=len(chain) - 1):
                    tmp.add(r)
                    chain.append(r)
                    break
            else:
                good = False
                break
        if good:
            for r in chain:
                grid.add(r)
            return chain
    raise RuntimeError("could not grow chain")


def _ions(L, n_plus, n_minus, seed, rmin=4.0):
    rng = np.random.Generator(np.random.PCG64(seed))
    grid = _Grid([L, L, L], rmin)
    pos = place_uniform(rng, grid, n_plus + n_minus)
    types = np.array([1] * n_plus + [2] * n_minus, dtype=np.int32)
    return np.array(pos), types


def electrolyte_std(seed=1, n=1000, L=100.0, lsurf=0):
    """Primitive-model electrolyte with standard Ewald (r_c=30 A, erfc(alpha
    r_c)=1e-5, |n|<=8 sphere), WCA LJ sigma=4 A, eps=1 kT, Bjerrum 7.1 A."""
    T = 298.0
    kt = units.kT(T)
    sp = [Species("Na", +1.0, 4.0, kt, mass=23.0), Species("Cl", -1.0, 4.0, kt, mass=35.45)]
    ro, types = _ions(L, n // 2, n - n // 2, seed)
    rcut = 30.0
    return System(species=sp, iptpn=types, ro=ro, boxlen=np.array([L, L, L]), temp=T,
                  relpermitt=units.relpermitt_from_bjerrum(7.1, T), rcut=rcut, drnlist=2.0,
                  txintlist=abi.MG_VLIST, mode=abi.MG_MD, ewald=abi.MG_EWALD_STD,
                  ualpha=alpha_for_erfc(1e-5, rcut), ncut=8, lsurf=lsurf, lljcut=1,
                  name="electrolyte_std_N1000")


def electrolyte_spme(seed=2, n=32768, L=817.0, nmesh=64, order=6, lsurf=0):
    """SPME electrolyte: sigma=4 A, eps=0.1 kT, LJ truncated at r_c = 12 A.

    The reference cannot tabulate an LJ cut and shifted at 3 sigma: with
    lljcut the force jumps by ~7e-4 kJ/mol/A at the cut, above ftoltab, and
    PotTwoBodyTab3 (potential.F90:1090-1129) never converges.  The LJ is
    therefore truncated by the pair cutoff, as for any (1,6,12) potential."""
    T = 298.0
    kt = units.kT(T)
    sp = [Species("Na", +1.0, 4.0, 0.1 * kt, mass=23.0), Species("Cl", -1.0, 4.0, 0.1 * kt, mass=35.45)]
    ro, types = _ions(L, n // 2, n - n // 2, seed)
    rcut = 12.0
    return System(species=sp, iptpn=types, ro=ro, boxlen=np.array([L, L, L]), temp=T,
                  relpermitt=units.relpermitt_from_bjerrum(7.1, T), rcut=rcut, drnlist=2.0,
                  txintlist=abi.MG_VLIST, mode=abi.MG_MD, ewald=abi.MG_EWALD_SPM,
                  ualpha=alpha_for_erfc(1e-5, rcut), order=order, nmesh=nmesh, lsurf=lsurf,
                  lljcut=0, name=f"electrolyte_spme_N{n}_K{nmesh}")


def polyelectrolyte(seed=3, nchain=64, nseg=200, nsalt=20000, L=700.0, nmesh=128, order=6,
                    dcoeff=1.0):
    """Polyelectrolyte solution: nchain chains of nseg (-1) beads (harmonic
    bonds, reference k = 0.2 kT/A^2 i.e. 0.4 kT/A^2 in the 1/2 k x^2
    convention, r0 = 5 A), nchain*nseg (+1) counterions and nsalt (+1,-1)
    salt pairs in a cube of edge L; SPME order 6, 128^3; overdamped BD."""
    T = 298.0
    kt = units.kT(T)
    eps = 0.1 * kt
    sp = [Species("bead", -1.0, 4.0, eps, mass=100.0, dcoeff=dcoeff),
          Species("cation", +1.0, 4.0, eps, mass=23.0, dcoeff=dcoeff),
          Species("anion", -1.0, 4.0, eps, mass=35.45, dcoeff=dcoeff)]
    rng = np.random.Generator(np.random.PCG64(seed))
    grid = _Grid([L, L, L], 4.0)
    pos, types, bip, bjp = [], [], [], []
    for _c in range(nchain):
        chain = place_chain(rng, grid, nseg, 5.0)
        base = len(pos)
        pos += chain
        types += [1] * nseg
        bip += [base + i + 1 for i in range(nseg - 1)]
        bjp += [base + i + 2 for i in range(nseg - 1)]
    ncounter = nchain * nseg
    pos += place_uniform(rng, grid, ncounter + nsalt)
    types += [2] * (ncounter + nsalt)
    pos += place_uniform(rng, grid, nsalt)
    types += [3] * nsalt
    nb = len(bip)
    rcut = 12.0
    return System(species=sp, iptpn=np.array(types, dtype=np.int32), ro=np.array(pos),
                  boxlen=np.array([L, L, L]), temp=T,
                  relpermitt=units.relpermitt_from_bjerrum(7.1, T), rcut=rcut, drnlist=2.0,
                  txintlist=abi.MG_VLIST, mode=abi.MG_BD, ewald=abi.MG_EWALD_SPM,
                  ualpha=alpha_for_erfc(1e-5, rcut), order=order, nmesh=nmesh, lsurf=0,
                  lljcut=0, bond_ip=np.array(bip, dtype=np.int32), bond_jp=np.array(bjp, dtype=np.int32),
                  bond_k=np.full(nb, 0.2 * kt), bond_eq=np.full(nb, 5.0),
                  bond_p=np.full(nb, 2, dtype=np.int32),
                  name=f"polyelectrolyte_N{len(types)}_K{nmesh}")


def small_system(seed=7, n=400, L=40.0, ewald=abi.MG_EWALD_SPM, nmesh=16, order=6, ncut=6,
                 rcut=9.0, drnlist=1.5, txintlist=abi.MG_VLIST, mode=abi.MG_MD, lsurf=0,
                 chains=0, nseg=10, eps_kt=0.1, rmin=3.0, lljcut=0, angle_kt=0.0, angle_eq=2.5, angle_p=2):
    """A small charged LJ system (three species) for parity tests; chains of
    nseg beads with harmonic bonds and, when angle_kt > 0, angle potentials
    k*(theta - angle_eq)**angle_p at every interior bead (UAngle's order)."""
    T = 298.0
    kt = units.kT(T)
    sp = [Species("A", +1.0, 3.5, eps_kt * kt, mass=23.0),
          Species("B", -1.0, 4.0, eps_kt * kt, mass=35.45),
          Species("C", +2.0, 4.5, 2 * eps_kt * kt, mass=40.0)]
    rng = np.random.Generator(np.random.PCG64(seed))
    grid = _Grid([L, L, L], rmin)
    pos, types, bip, bjp, ajm = [], [], [], [], []
    for _c in range(chains):
        chain = place_chain(rng, grid, nseg, 4.5)
        base = len(pos)
        pos += chain
        types += [2] * nseg
        bip += [base + i + 1 for i in range(nseg - 1)]
        bjp += [base + i + 2 for i in range(nseg - 1)]
        ajm += [base + i + 1 for i in range(nseg - 2)]   # angle (i+1, i+2, i+3), 1-based
    nrest = n - len(pos)
    nC = nrest // 10
    nB_ions = (nrest - nC) // 2
    # neutralise: charges +1*nA - 1*(nB_ions + chain beads) + 2*nC = 0
    nneg = nB_ions + chains * nseg
    nA = nneg - 2 * nC
    if nA < 0:
        raise ValueError("cannot neutralise")
    total_ions = nA + nB_ions + nC
    pos += place_uniform(rng, grid, total_ions)
    types += [1] * nA + [2] * nB_ions + [3] * nC
    ro = np.array(pos)
    types = np.array(types, dtype=np.int32)
    nb = len(bip)
    kw = {}
    if nb:
        kw = dict(bond_ip=np.array(bip, dtype=np.int32), bond_jp=np.array(bjp, dtype=np.int32),
                  bond_k=np.full(nb, 0.3 * kt), bond_eq=np.full(nb, 4.5),
                  bond_p=np.full(nb, 2, dtype=np.int32))
    if angle_kt > 0 and ajm:
        jm = np.array(ajm, dtype=np.int32)
        na = len(jm)
        kw.update(angle_jm=jm, angle_ip=jm + 1, angle_jp=jm + 2, angle_k=np.full(na, angle_kt * kt),
                  angle_eq=np.full(na, angle_eq), angle_p=np.full(na, angle_p, dtype=np.int32))
    return System(species=sp, iptpn=types, ro=ro, boxlen=np.array([L, L, L]), temp=T,
                  relpermitt=units.relpermitt_from_bjerrum(7.1, T), rcut=rcut, drnlist=drnlist,
                  txintlist=txintlist, mode=mode, ewald=ewald, ualpha=alpha_for_erfc(1e-5, rcut),
                  ncut=ncut, order=order, nmesh=nmesh, lsurf=lsurf, lljcut=lljcut,
                  name=f"small_N{len(types)}", **kw)


AVOGADRO = 6.02214076e23


def replica_set(seed=5, nrep=256, nmin=500, nmax=8000, cmin=0.01, cmax=1.0, rcut=12.0, order=5,
                spacing=1.6, mode=abi.MG_MD):
    """nrep electrolyte boxes: N log-uniform in [nmin, nmax] rounded to even,
    salt concentration c uniform in [cmin, cmax] mol/L setting each box edge
    (N/2 ion pairs in V = N/(2 c N_A)), charges +-1 e, LJ sigma = 4 A,
    eps = 0.1 kT truncated at r_c, SPME of the given order on the power-of-
    two mesh with spacing at most `spacing` A (autotune.tune_spme refines
    both).  Returns a list of Systems."""
    T = 298.0
    kt = units.kT(T)
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for r in range(nrep):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax))) / 2)) * 2
        c = rng.uniform(cmin, cmax)
        vol = (n / 2) / (c * AVOGADRO) * 1e27          # A^3 (1 L = 1e27 A^3)
        L = vol ** (1.0 / 3.0)
        k = 8
        while L / k > spacing:
            k *= 2
        sp = [Species("Na", +1.0, 4.0, 0.1 * kt, mass=23.0), Species("Cl", -1.0, 4.0, 0.1 * kt, mass=35.45)]
        ro, types = _ions(L, n // 2, n - n // 2, int(rng.integers(1 << 30)))
        out.append(System(species=sp, iptpn=types, ro=ro, boxlen=np.array([L, L, L]), temp=T,
                          relpermitt=units.relpermitt_from_bjerrum(7.1, T), rcut=rcut, drnlist=2.0,
                          txintlist=abi.MG_VLIST, mode=mode, ewald=abi.MG_EWALD_SPM,
                          ualpha=alpha_for_erfc(1e-5, rcut), order=order, nmesh=k, lsurf=0, lljcut=0,
                          name=f"replica{r}_N{n}_c{c:.3f}"))
    return out


def dipolar_waters(seed=9, nwater=200, nsalt=10, L=22.0, rcut=9.0, rmin=3.0, ewald=abi.MG_EWALD_SPM,
                   ualpha=0.35, order=6, nmesh=32, ncut=8):
    """Rigid three-site waters whose atoms carry charges and point dipoles
    (txelec = 'dip': UDipole takes the electrostatics, the pair table only
    the LJ term), with NaCl ion pairs as one-atom particles; relative
    permittivity 1, Ewald over the atoms.  The dipoles lie in the molecular
    plane: on O along the symmetry axis, on the H atoms along their bonds."""
    s = water_ions(seed=seed, nwater=nwater, nsalt=nsalt, L=L, rcut=rcut, rmin=rmin)
    s.atom_types[0].charge, s.atom_types[1].charge = -0.66, 0.33
    w = s.particle_types[0]
    ho = np.array(w.atoms[1][1]) - np.array(w.atoms[0][1])
    ho2 = np.array(w.atoms[2][1]) - np.array(w.atoms[0][1])
    w.dipoles = [(0.0, 0.0, -0.11), tuple(0.06 * ho / np.linalg.norm(ho)), tuple(0.06 * ho2 / np.linalg.norm(ho2))]
    s.txelec = "dip"
    s.ewald, s.ualpha, s.order, s.nmesh, s.ncut = ewald, ualpha, order, nmesh, ncut
    return s


def water_ions(seed=9, nwater=300, nsalt=20, L=24.0, rcut=9.0, rmin=3.0):
    """A polyatomic system for the UTwoBodyP path: rigid three-site waters
    (O and two H, SPC/E-like charges and geometry) and NaCl ion pairs as
    one-atom particles, centres on a jittered grid at least rmin apart,
    random orientations; Coulomb without Ewald plus (1,6,12) LJ between
    atoms (H without LJ)."""
    from .poly import AtomType, ParticleType, PolySystem
    rng = np.random.Generator(np.random.PCG64(seed))
    atom_types = [AtomType("O", -0.8476, 3.166, 0.650, 15.9994), AtomType("H", 0.4238, 0.0, 0.0, 1.008),
                  AtomType("Na", 1.0, 2.35, 0.544, 22.99), AtomType("Cl", -1.0, 4.40, 0.419, 35.45)]
    hx, hz = 0.8165, 0.5773
    ptypes = [ParticleType("water", [(0, (0.0, 0.0, -0.0656)), (1, (hx, 0.0, hz - 0.0656)),
                                     (1, (-hx, 0.0, hz - 0.0656))]),
              ParticleType("Na", [(2, (0.0, 0.0, 0.0))]), ParticleType("Cl", [(3, (0.0, 0.0, 0.0))])]
    n = nwater + 2 * nsalt
    grid = _Grid([L, L, L], rmin)
    ro = place_uniform(rng, grid, n)
    types = np.array([1] * nwater + [2] * nsalt + [3] * nsalt, dtype=np.int32)
    ori = np.empty((n, 3, 3))
    for i in range(n):
        q, r = np.linalg.qr(rng.standard_normal((3, 3)))
        q = q * np.sign(np.diag(r))
        if np.linalg.det(q) < 0:
            q[:, 0] = -q[:, 0]
        ori[i] = q
    return PolySystem(atom_types=atom_types, particle_types=ptypes, iptpn=types,
                      ro=np.ascontiguousarray(np.asarray(ro, dtype=np.float64)), ori=ori,
                      boxlen=np.array([L, L, L]), rcut=rcut)
