"""A System from the reference's own input: its namelist file (`<project>.in`)
and, optionally, its configuration file (`<project>.cnf`).

The reference reads each group in the routine that owns it; this module
reads the variables of the force/energy path with the reference's defaults
and meaning:

- &nmlSystem (molsim.F90:414-424): txmethod ('md', 'mc', 'bd'), txbc
  (only 'xyz', a rectangular periodic box), boxlen, temp, iseed.
- &nmlParticle (particle.F90:177-187, defaults :200-230): npt, txpt, nppt,
  natpt (1: monoatomic), zat, sigat, epsat, radat, massat; chains nct, txct,
  ncct, npptct, txcopolymer ('block' or 'regular').
- &nmlPotential (potential.F90:307-330, defaults :332-380): rcut,
  relpermitt, txpot ('(1,6,12)' for every pair, or 'default' for every pair
  with only its Coulomb term: npot, ipot, ucoff are refused), lewald,
  txewaldrec ('std', 'spm'), iewaldopt (0: ualpha = ualphared/rcut; 1:
  the same, with ncut from the error estimate (std); 3: alpha from
  uewaldtol, RcutToAlpha, and ncut as for 1 (std)), ncut, ncutregion, lsurf,
  order, nmesh, lljcut,
  ljrcut, ljushift, r2uminin, utoltab, ftoltab, umaxtab, fmaxtab.
- &nmlPotentialChain (potential.F90:3505-3560): bond(nct) and angle(nct) as
  (k, p, eq); angles in degrees in the input, converted as the reference
  does (k / DegToRad**2, eq * DegToRad).
- &nmlIntList (nlist.F90:198-240): txintlist ('vlist', 'celllist';
  'nlist' read as 'vlist'), drnlist.
- &nmlBD (bd.F90:82): tstep, dcoeff(npt).  &nmlMD (md.F90:201): tstep.

Particles are numbered as the reference numbers them: by particle type, and
within a type the chains first (chain type by chain type, 'block' or
'regular' segment order, SetObjectParam1, particle.F90:1080-1130).  Without a
.cnf the positions are generated here (chains as random walks at the bond
length, the other particles uniform, no two closer than the largest radat
sum or 2 Angstrom): the reference's own 'setconf' generators are not
reproduced.  Features outside the path (dipoles, polarisation, weak charges,
polyatomic particles, other boundary conditions or potentials) raise
NotImplementedError.
"""
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import abi, units
from .cnf import read_cnf
from .namelist import array, read_namelists, parse_namelists, scalar
from .system import Species, System

__all__ = ["ReferenceRun", "system_from_input", "ewald_error_ureal", "alpha_to_ncut"]

DegToRad = units.Pi / 180.0


@dataclass
class ReferenceRun:
    system: System
    method: str               # 'md', 'mc' or 'bd'
    tstep: Optional[float]    # ps (MD/BD)
    iseed: int
    nstep1: int
    nstep2: int


def _lower(x):
    return x.strip().lower() if isinstance(x, str) else x


def _chain_indices(nppt, npptct, ncct, txcopolymer):
    """ipnsegcn of SetObjectParam1 (particle.F90:1080-1130) as 1-based
    particle lists, one per chain."""
    npt, nct = npptct.shape
    chains = []
    for ict in range(nct):
        for icloc in range(int(ncct[ict])):
            segs = []
            kind = _lower(txcopolymer[ict])
            if kind == "block":
                for ipt in range(npt):
                    iplow = int(nppt[:ipt].sum()) + int((ncct[:ict] * npptct[ipt, :ict]).sum()) \
                        + icloc * int(npptct[ipt, ict])
                    segs += [iplow + k + 1 for k in range(int(npptct[ipt, ict]))]
            elif kind == "regular":
                nz = [int(npptct[ipt, ict]) for ipt in range(npt) if npptct[ipt, ict] > 0]
                nrep = min(nz)
                for ipt in range(npt):
                    if npptct[ipt, ict] % nrep:
                        raise ValueError("npptct does not repeat regularly")
                for irep in range(nrep):
                    for ipt in range(npt):
                        per = int(npptct[ipt, ict]) // nrep
                        iplow = irep * per + int(nppt[:ipt].sum()) + int((ncct[:ict] * npptct[ipt, :ict]).sum()) \
                            + icloc * int(npptct[ipt, ict])
                        segs += [iplow + k + 1 for k in range(per)]
            else:
                raise NotImplementedError(f"txcopolymer = {txcopolymer[ict]!r}")
            chains.append((ict, segs))
    return chains


def system_from_input(inp, cnf=None, seed=1, text=False):
    """ReferenceRun for the namelist file `inp` (a path, or the text itself
    with text=True) and an optional .cnf path."""
    nml = parse_namelists(inp) if text else read_namelists(inp)
    g = lambda name: nml.get(name.lower(), {})
    sysg, part, pot = g("nmlSystem"), g("nmlParticle"), g("nmlPotential")

    method = _lower(scalar(sysg, "txmethod", "md"))
    mode = {"md": abi.MG_MD, "mc": abi.MG_MC, "bd": abi.MG_BD}.get(method)
    if mode is None:
        raise NotImplementedError(f"txmethod = {method!r}")
    if _lower(scalar(sysg, "txbc", "xyz")) != "xyz":
        raise NotImplementedError("only txbc = 'xyz' (a rectangular periodic box)")
    boxlen = np.array(array(sysg, "boxlen", 3, 0.0), dtype=np.float64)
    if (boxlen <= 0).any():
        raise ValueError("boxlen must be positive")
    temp = float(scalar(sysg, "temp", 298.0))

    # particles (monoatomic: one atom type per particle type)
    npt = int(scalar(part, "npt", 1))
    txelec = _lower(scalar(part, "txelec", "charge"))
    if txelec == "pol":   # induced dipoles (UManyBodyP, energy.F90:2327-2497): not built
        raise NotImplementedError("txelec = 'pol' (polarisation is not built)")
    natpt = array(part, "natpt", npt, 1, dtype=int)
    if (natpt != 1).any():
        raise NotImplementedError("polyatomic particles (natpt > 1): this reader builds monoatomic systems")
    if txelec != "charge":   # particle.F90:307-321: weak charges, dipoles, ...
        raise NotImplementedError(f"txelec = {txelec!r} (this reader builds fixed-charge systems)")
    for name in ("latweakcharge", "dipain", "polain"):
        if name in part:
            vals = part[name].values or []
            if any(v not in (False, 0, 0.0) for v in vals if not isinstance(v, str)):
                raise NotImplementedError(f"{name} is outside the force/energy path")
    txpt = array(part, "txpt", npt, "", dtype=object)
    nppt = array(part, "nppt", npt, 0, dtype=int)
    zat = array(part, "zat", npt, 0.0)
    sigat = array(part, "sigat", npt, 0.0)
    epsat = array(part, "epsat", npt, 0.0)
    radat = array(part, "radat", npt, 0.0)
    massat = array(part, "massat", npt, 1.0)
    nct = int(scalar(part, "nct", 0))
    npptct = array(part, "npptct", (npt, max(nct, 1)), 0, dtype=int)[:, :nct]
    ncct = array(part, "ncct", max(nct, 1), 0, dtype=int)[:nct]
    txcopolymer = array(part, "txcopolymer", max(nct, 1), "block", dtype=object)[:nct]

    bd = g("nmlBD")
    dcoeff = array(bd, "dcoeff", npt, 0.0)
    species = [Species(str(txpt[i]) or f"t{i + 1}", float(zat[i]), float(sigat[i]), float(epsat[i]),
                       mass=float(massat[i]), dcoeff=float(dcoeff[i]), radat=float(radat[i]))
               for i in range(npt)]
    iptpn = np.repeat(np.arange(1, npt + 1, dtype=np.int32), nppt)
    npart = int(nppt.sum())

    # potential
    txpot = [_lower(t) for t in array(pot, "txpot", npt * (npt + 1) // 2, "default", dtype=object)]
    for t in txpot:
        if t not in ("default", "(1,6,12)"):
            raise NotImplementedError(f"txpot = {t!r} (the path tabulates '(1,6,12)' and the Coulomb term)")
    # txpot 'default' is PotDefault (potential.F90:1290-1330): the sum of
    # ucoff(m)/r**ipot(m), whose 1/r term is the Coulomb term EpsiFourPi z z
    # (potential.F90:533-571) -- no Lennard-Jones term.  Only the Coulomb
    # term is read here: further terms are refused.
    for name in ("npot", "ipot", "ucoff"):
        v = pot.get(name)
        if v is not None and any(x not in (0, 0.0) for x in list(v.values or []) +
                                 [y for vv in v.items.values() for y in vv]):
            raise NotImplementedError(f"{name} (terms of txpot = 'default' beyond the Coulomb term)")
    if "default" in txpot and "(1,6,12)" in txpot:
        raise NotImplementedError("txpot = 'default' for some pairs and '(1,6,12)' for others")
    if txpot and txpot[0] == "default":
        epsat = np.zeros(npt)   # Coulomb only
        species = [Species(sp.name, sp.charge, sp.sigma, 0.0, mass=sp.mass, dcoeff=sp.dcoeff, radat=sp.radat)
                   for sp in species]
    rcut = float(scalar(pot, "rcut", 0.0))
    if rcut <= 0:   # potential.F90:418-422: half the box diagonal ('xyz')
        rcut = float(np.sqrt(((0.5 * boxlen) ** 2).sum()))
    relpermitt = float(scalar(pot, "relpermitt", 1.0))
    lewald = bool(scalar(pot, "lewald", False))
    ewald = abi.MG_EWALD_NONE
    ualpha = 0.0
    ncut = int(scalar(pot, "ncut", 0))
    order = int(scalar(pot, "order", 5))
    nmesh = int(scalar(pot, "nmesh", 48))
    if lewald:
        rec = _lower(scalar(pot, "txewaldrec", "std"))
        ewald = {"std": abi.MG_EWALD_STD, "spm": abi.MG_EWALD_SPM}.get(rec)
        if ewald is None:
            raise NotImplementedError(f"txewaldrec = {rec!r}")
        opt = int(scalar(pot, "iewaldopt", -1))
        q = zat[iptpn - 1]
        q2sum, lshort, unit = float((q * q).sum()), float(boxlen.min()), units.Epsi0FourPi / relpermitt
        tol = float(scalar(pot, "uewaldtol", 0.0))
        allowed = (0, 1, 3) if ewald == abi.MG_EWALD_STD else (0, 3)
        if opt not in allowed:
            raise NotImplementedError(f"iewaldopt = {opt} with txewaldrec = {rec!r} (read: {allowed})")
        if opt in (0, 1):
            ualpha = float(scalar(pot, "ualphared", 3.0)) / rcut
            if opt == 1:   # (ualphared, rcut) -> (uewaldtol, ncut)
                tol = ewald_error_ureal(q2sum, lshort, ualpha, rcut, unit)
        else:              # (uewaldtol, rcut) -> alpha (RcutToAlpha)
            a = np.zeros(1)
            st = abi.load_library().mg_rcut_to_alpha(tol, rcut, q2sum, lshort, unit, abi.f64(a))
            if st != 0:
                raise ValueError(f"RcutToAlpha failed ({st})")
            ualpha = float(a[0])
        if ewald == abi.MG_EWALD_STD and opt in (1, 3):
            ncut = alpha_to_ncut(tol, q2sum, lshort, ualpha, unit)
    ncutregion = _lower(scalar(pot, "ncutregion", "sphere"))

    # lists
    il = g("nmlIntList")
    txintlist = _lower(scalar(il, "txintlist", "vlist"))
    txintlist = "vlist" if txintlist == "nlist" else txintlist
    if txintlist not in ("vlist", "celllist"):
        raise NotImplementedError(f"txintlist = {txintlist!r}")
    drnlist = float(scalar(il, "drnlist", 0.0))

    # chains: bonds between consecutive segments, angles at segments 2..npct-1
    chainsg = g("nmlPotentialChain")
    kw = {}
    if nct > 0:
        def bondvar(name, default):
            v = chainsg.get(name)
            k, p, eq = (np.full(nct, default[0], dtype=float), np.full(nct, default[1], dtype=int),
                        np.full(nct, default[2], dtype=float))
            if v is not None:
                vals = [x for x in (v.values or [])]
                for ict in range(nct):   # bond = k, p, eq[, k, p, eq ...] (bond_var components in order)
                    trip = vals[3 * ict:3 * ict + 3]
                    if len(trip) > 0: k[ict] = trip[0]
                    if len(trip) > 1: p[ict] = trip[1]
                    if len(trip) > 2: eq[ict] = trip[2]
                for idx, vv in v.items.items():
                    ict = idx[0] - 1
                    for c, x in enumerate(vv[:3]):
                        (k, p, eq)[c][ict] = x
            for comp, arr in (("k", k), ("p", p), ("eq", eq)):
                cv = chainsg.get(f"{name}%{comp}")
                if cv is not None:
                    arr[:] = array(chainsg, f"{name}%{comp}", nct, arr[0] if nct else 0.0)
            return k, p, eq
        bk, bp, beq = bondvar("bond", (0.0, 2, 0.0))
        ak, ap, aeq = bondvar("angle", (0.0, 2, 180.0))
        ak = ak / DegToRad ** 2      # potential.F90:3555-3556
        aeq = aeq * DegToRad
        chains = _chain_indices(nppt, npptct, ncct, txcopolymer)
        bi, bj, bkk, bee, bpp = [], [], [], [], []
        am, ai, aj, akk, aee, app = [], [], [], [], [], []
        for ict, segs in chains:
            for s in range(len(segs) - 1):
                bi.append(segs[s]); bj.append(segs[s + 1])
                bkk.append(bk[ict]); bee.append(beq[ict]); bpp.append(bp[ict])
            if ak[ict] != 0.0:
                for s in range(1, len(segs) - 1):
                    am.append(segs[s - 1]); ai.append(segs[s]); aj.append(segs[s + 1])
                    akk.append(ak[ict]); aee.append(aeq[ict]); app.append(ap[ict])
        if bi:
            kw.update(bond_ip=np.array(bi, dtype=np.int32), bond_jp=np.array(bj, dtype=np.int32),
                      bond_k=np.array(bkk), bond_eq=np.array(bee), bond_p=np.array(bpp, dtype=np.int32))
        if am:
            kw.update(angle_jm=np.array(am, dtype=np.int32), angle_ip=np.array(ai, dtype=np.int32),
                      angle_jp=np.array(aj, dtype=np.int32), angle_k=np.array(akk),
                      angle_eq=np.array(aee), angle_p=np.array(app, dtype=np.int32))
    else:
        chains = []

    # positions
    if cnf is not None:
        c = read_cnf(cnf)
        if c["np"] != npart:
            raise ValueError(f"the .cnf holds {c['np']} particles, the input {npart}")
        ro = c["ro"]
        boxlen = c["boxlen"] if (c["boxlen"] > 0).all() else boxlen
    else:
        ro, placed = _lattices(g("nmlSetConfiguration"), boxlen, nppt)
        ro = _generate(boxlen, npart, chains, kw, radat, iptpn, seed, ro, placed)

    md = g("nmlMD")
    tstep = scalar(bd, "tstep") if mode == abi.MG_BD else scalar(md, "tstep") if mode == abi.MG_MD else None
    s = System(species=species, iptpn=iptpn, ro=np.ascontiguousarray(ro, dtype=np.float64), boxlen=boxlen,
               temp=temp, relpermitt=relpermitt, rcut=rcut, drnlist=drnlist,
               txintlist=abi.MG_CELLLIST if txintlist == "celllist" else abi.MG_VLIST, mode=mode,
               ewald=ewald, ualpha=ualpha, ncut=ncut, ncutregion_cube=1 if ncutregion == "cube" else 0,
               order=order, nmesh=nmesh, lsurf=1 if (lewald and bool(scalar(pot, "lsurf", True))) else 0,
               lljcut=1 if bool(scalar(pot, "lljcut", False)) else 0,
               ljrcut=float(scalar(pot, "ljrcut", units.ljrcut_default())),
               ljushift=float(scalar(pot, "ljushift", 1.0)),
               r2uminin=float(scalar(pot, "r2uminin", 0.1)),
               utoltab=float(scalar(pot, "utoltab", units.tol_default())),
               ftoltab=float(scalar(pot, "ftoltab", units.tol_default())),
               umaxtab=float(scalar(pot, "umaxtab", 20000.0)), fmaxtab=float(scalar(pot, "fmaxtab", 20000.0)),
               name=str(scalar(sysg, "txtitle", "reference input")).strip(), **kw)
    return ReferenceRun(system=s, method=method, tstep=None if tstep is None else float(tstep),
                        iseed=int(scalar(sysg, "iseed", 1)), nstep1=int(scalar(sysg, "nstep1", 1)),
                        nstep2=int(scalar(sysg, "nstep2", 1)))


def ewald_error_ureal(q2sum, l, alpha, rcut, unit):
    """Real-space Ewald error estimate of a charged system (Kolafa and
    Perram, Mol. Simul. 9, 351 (1992)), as EwaldErrorUReal computes it
    (potential.F90:2995-3018, lq2sum = 0)."""
    fac = (alpha * rcut) ** 2
    return unit * q2sum * np.sqrt(rcut / (2.0 * l ** 3)) / fac * np.exp(-fac)


def alpha_to_ncut(tol, q2sum, l, alpha, unit):
    """k-space cutoff for a tolerance (AlphaToNcut, energy.F90:7071-7086):
    the fixed point of Kolafa and Perram's reciprocal-space estimate."""
    pi = units.Pi
    if not (tol > 0 and q2sum > 0):
        raise ValueError("AlphaToNcut needs a positive tolerance and charges")
    y = (tol / (q2sum * unit)) * (pi ** 2 / (alpha ** 2 * l))
    xold = 1.0
    for _ in range(40):
        xnew = (alpha * l / pi) * np.sqrt(-np.log(y * xold / (1.0 + 1.0 / (alpha * l * np.sqrt(xold)))))
        if abs(xold - xnew) / xnew < 1.0e-6:
            break
        xold = xnew
    else:
        raise ValueError("AlphaToNcut did not converge in 40 iterations")
    return int(xnew + 1.0)


# unit-cell lattice points of SetPC, SetBCC and SetFCC (coordinate.F90:905-976)
_LATTICE_POINTS = {
    "pclattice": [(0.0, 0.0, 0.0)],
    "bcclattice": [(0.0, 0.0, 0.0), (0.5, 0.5, 0.5)],
    "fcclattice": [(0.0, 0.0, 0.0), (0.0, 0.5, 0.5), (0.5, 0.0, 0.5), (0.5, 0.5, 0.0)],
}


def _pbc_position(x, boxlen):
    """PBC for a position in a box (molaux.F90:104-118): one shift by
    boxlen*anint(x/boxlen) where |x| > boxlen/2 (anint rounds half away from
    zero)."""
    for m in range(3):
        if abs(x[m]) > 0.5 * boxlen[m]:
            t = x[m] * (1.0 / boxlen[m])
            x[m] = x[m] - boxlen[m] * float(np.copysign(np.floor(abs(t) + 0.5), t))
    return x


def _lattices(setconf, boxlen, nppt):
    """Particle types placed on a lattice by SetLattice
    (coordinate.F90:713-832) with the &nmlSetConfiguration variables
    txsetconf, nucell, rclow, rcupp, roshift (defaults coordinate.F90:449-510:
    the whole box, no shift).  Returns positions (rows of the other types
    zero) and a mask of the placed particles."""
    npt = len(nppt)
    npart = int(nppt.sum())
    ro = np.zeros((npart, 3))
    placed = np.zeros(npart, dtype=bool)
    if not setconf:
        return ro, placed
    half = 0.5 * boxlen
    txsetconf = array(setconf, "txsetconf", npt, "", dtype=object)
    nucell = array(setconf, "nucell", (3, npt), 0, dtype=int)
    # unassigned elements keep the box defaults (lbcbox)
    rclow = array(setconf, "rclow", (3, npt), np.nan)
    rcupp = array(setconf, "rcupp", (3, npt), np.nan)
    for m in range(3):
        rclow[m, np.isnan(rclow[m])] = -half[m]
        rcupp[m, np.isnan(rcupp[m])] = +half[m]
    roshift = array(setconf, "roshift", (3, npt), 0.0)
    ddelta = 1.0e-10
    for ipt in range(npt):
        kind = _lower(txsetconf[ipt])
        if kind not in _LATTICE_POINTS:
            continue
        ipnpt = int(nppt[:ipt].sum())
        rlen = (rcupp[:, ipt] - rclow[:, ipt]) / nucell[:, ipt]
        rorigin = 0.5 * (rclow[:, ipt] + rcupp[:, ipt])
        nset = 0
        for rol in _LATTICE_POINTS[kind]:
            for iz in range(int(nucell[2, ipt])):
                for iy in range(int(nucell[1, ipt])):
                    for ix in range(int(nucell[0, ipt])):
                        if nset == nppt[ipt]:
                            break
                        idx = (ix, iy, iz)
                        x = np.empty(3)
                        for m in range(3):
                            u = (float(idx[m]) - 0.5 * float(nucell[m, ipt])) + (rol[m] + roshift[m, ipt])
                            x[m] = (rorigin[m] + ddelta) + u * rlen[m]
                        ro[ipnpt + nset] = _pbc_position(x, boxlen)
                        placed[ipnpt + nset] = True
                        nset += 1
        if nset < nppt[ipt]:   # SetLattice: 'lattice set failed'
            raise ValueError(f"{kind} of particle type {ipt + 1} holds {nset} of {nppt[ipt]} particles")
    return ro, placed


def _generate(boxlen, npart, chains, kw, radat, iptpn, seed, ro=None, placed=None):
    """Positions of the particles not placed on a lattice: chains as random
    walks at the bond length, then the other particles uniform, no two
    closer than the sum of their radii radat (at least 1 A each, so that no
    pair comes near r2umin)."""
    from .configs import _Grid, place_chain
    rng = np.random.Generator(np.random.PCG64(seed))
    rad = np.maximum(np.asarray(radat, dtype=float), 1.0)[iptpn - 1]
    grid = _Grid(boxlen, 2.0 * float(rad.max()))
    ro = np.zeros((npart, 3)) if ro is None else ro
    done = np.zeros(npart, dtype=bool) if placed is None else placed.copy()
    for i in np.nonzero(done)[0]:
        grid.add(ro[i], rad[i])
    bond_eq = {}
    if "bond_ip" in kw:
        for i, e in zip(kw["bond_ip"], kw["bond_eq"]):
            bond_eq[int(i)] = float(e)
    for _ict, segs in chains:
        rmin = 2.0 * float(rad[np.asarray(segs) - 1].max())
        b = bond_eq.get(segs[0], 0.0) or rmin * 1.2
        sub = _Grid(boxlen, rmin)
        for i in np.nonzero(done)[0]:
            sub.add(ro[i])
        for s, r in zip(segs, place_chain(rng, sub, len(segs), max(b, rmin * 1.01))):
            ro[s - 1] = r
            done[s - 1] = True
            grid.add(r, rad[s - 1])
    for i in np.nonzero(~done)[0]:
        for _t in range(100000):
            r = (rng.random(3) - 0.5) * grid.L
            if grid.ok(r, rad=rad[i]):
                grid.add(r, rad[i])
                ro[i] = r
                break
        else:
            raise RuntimeError("could not place particle without overlap")
    return ro
