"""Physical constants and unit scales of the reference (mol.F90:59-76,
molsim.F90:786-805).  Internal units: Angstrom, ps, g/mol, kJ/mol, K.

Expressions keep the reference's evaluation order so that derived factors
(EpsiFourPi, the force scale, the BD factors) are bit-identical to what the
Fortran computes.
"""
import math

Pi = 3.1415926535897932
TwoPi = 2.0 * Pi
FourPi = 4.0 * Pi
AvNo = 6.02214179e23          # 1/mol
Boltz = 1.3806504e-23         # J/K
ECh = 1.602176487e-19         # C
GasConstant = 8.314472        # J/(mol K)
Epsi0 = 8.854187817e-12       # F/m

# IOScale defaults (molsim.F90:786-795)
scllen = 1.0e-10
sclmas = 1.0e-03
scltem = 1.0
scltim = 1.0e-12
sclene = 1.0e+03
sclpre = 1.0e+06
scldif = 1.0e-09
sclvol = scllen * scllen * scllen
sclvel = scllen / scltim
sclacc = sclvel / scltim
sclfor = sclacc * sclmas

# Epsi0FourPi = ECh**2/(FourPi*Epsi0*scllen)*AvNo/sclene  (molsim.F90:805)
Epsi0FourPi = (ECh * ECh) / (FourPi * Epsi0 * scllen) * AvNo / sclene

# UTotal force scale: fac = (sclene/scllen)/sclfor  (energy.F90:407)
FORCE_FAC = (sclene / scllen) / sclfor


def kT(temp):
    """Thermal energy in kJ/mol."""
    return GasConstant * temp * scltem / sclene


def relpermitt_from_bjerrum(lb, temp):
    """Relative permittivity giving Bjerrum length lb (Angstrom) at temp."""
    return Epsi0FourPi / (lb * kT(temp))


def bd_factors(tstep, dcoeff, temp):
    """fac1, fac2 of BDStep (bd.F90:136-139) for one particle type."""
    fac1 = tstep * scltim * dcoeff * scldif * sclfor / (GasConstant * temp * scltem) / scllen
    fac2 = math.sqrt(2.0 * dcoeff * scldif * tstep * scltim) / scllen
    return fac1, fac2


def ljrcut_default():
    """Reference default ljrcut = Two**(1.0/6.0) with a single-precision
    exponent (potential.F90:365)."""
    import numpy as np
    return 2.0 ** float(np.float32(1.0) / np.float32(6.0))


def tol_default():
    """Reference default utoltab/ftoltab = 1e-5 written as a single-precision
    literal (potential.F90:341-342)."""
    import numpy as np
    return float(np.float32(1e-5))
