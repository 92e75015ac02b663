/*
 * molsim_oracle.c — TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of MOLSIM's force/energy hot path (reference:
 * joakimstenhammar/molsim, Fortran 90).  Every routine follows the Fortran
 * loop order and expression order of the reference routine it names, so that
 * the GPU library can be compared with it at the 1e-10 level and, for lists,
 * bit-exactly.  Compiled with -ffp-contract=off (no fused multiply-add), as a
 * baseline x86-64 gfortran -O2 build of the reference would evaluate it.
 * Integer powers follow gfortran's -O2 expansion (x**6 = x**3 * x**3).
 *
 * Used only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline.
 * Parity status: unpinned against reference outputs (none ship, and the
 * Fortran cannot be built here); pinned against known answers in tests.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <complex.h>
#include "molsim_oracle.h"
#include "oracle_par.h"

#define Zero 0.0
#define Half 0.5
#define One 1.0
#define Two 2.0
#define Three 3.0
#define Four 4.0
static const double Pi = 3.1415926535897932;   /* mol.F90:63 */
#define TwoPi (Two * Pi)
#define FourPi (Four * Pi)

typedef struct { double re, im; } zc;   /* complex(8) */

/* threads standing in for molsim_par's MPI ranks (oracle_par.h) */
static int g_orc_threads = 1;
int orc_threads(void) { return g_orc_threads; }
int orc_set_threads(int n) {
    if (n < 1 || n > ORC_MAX_THREADS) return MG_ERR_ARG;
    g_orc_threads = n;
    return 0;
}

static inline zc zmul(zc a, zc b) { zc r; r.re = a.re * b.re - a.im * b.im; r.im = a.re * b.im + a.im * b.re; return r; }
static inline zc zconj(zc a) { a.im = -a.im; return a; }
static inline zc zscale(double s, zc a) { zc r; r.re = s * a.re; r.im = s * a.im; return r; }
static inline zc zadd(zc a, zc b) { zc r; r.re = a.re + b.re; r.im = a.im + b.im; return r; }
static inline zc zsub(zc a, zc b) { zc r; r.re = a.re - b.re; r.im = a.im - b.im; return r; }

static inline double pow2(double x) { return x * x; }
static inline double pow3(double x) { return (x * x) * x; }
static inline double pow6(double x) { double x3 = (x * x) * x; return x3 * x3; }
/* gfortran -O2 expands x**n (integer n) with an optimal multiplication chain;
   the chains for the small n used by UBond are written out here. */
static double powi(double x, int n) {
    switch (n) {
    case 0: return One;
    case 1: return x;
    case 2: return x * x;
    case 3: return (x * x) * x;
    case 4: { double x2 = x * x; return x2 * x2; }
    default: { double r = One; for (int i = 0; i < n; ++i) r *= x; return r; }
    }
}
static inline double fsign(double a, double b) { return copysign(fabs(a), b); }   /* Fortran sign(a,b) */

/* ======================================================================
 * mollib.F90
 * ====================================================================== */

/* Erf2, mollib.F90:215-274.  The reference's second branch iterates j from
   ncfd-1 (not ncfc-1) down to 2 after starting from c(ncfc), so c(17) is never
   used and the last term uses c(1) (the loop index ends at 1); both are kept.
   At |x| == xup exactly no branch assigns the result in the reference; sign(1,x)
   is returned there. */
double orc_erf2(double x) {
    static const double sqrtpi = 1.7724538509055160;
    static const double xup = 6.25;
    static const double c[18] = {
        1.9449071068178803, 4.20186582324414e-2, -1.86866103976769e-2,
        5.1281061839107e-3, -1.0683107461726e-3, 1.744737872522e-4,
        -2.15642065714e-5, 1.7282657974e-6, -2.00479241e-8,
        -1.64782105e-8, 2.0008475e-9, 2.57716e-11,
        -3.06343e-11, 1.9158e-12, 3.703e-13,
        -5.43e-14, -4.0e-15, 1.2e-15};
    static const double d[17] = {
        1.4831105640848036, -3.010710733865950e-1, 6.89948306898316e-2,
        -1.39162712647222e-2, 2.4207995224335e-3, -3.658639685849e-4,
        4.86209844323e-5, -5.7492565580e-6, 6.113243578e-7,
        -5.89910153e-8, 5.2070091e-9, -4.232976e-10,
        3.18811e-11, -2.2361e-12, 1.467e-13,
        -9.0e-15, 5.0e-16};
    const int ncfc = 18, ncfd = 17;
    double xv = fabs(x), bj, bjp1, bjp2, x2;
    int j;
    if (xv <= Two) {
        x2 = x * x - Two;
        bjp2 = Zero;
        bjp1 = d[ncfd - 1];
        for (j = ncfd - 1; j >= 2; --j) {
            bj = x2 * bjp1 - bjp2 + d[j - 1];
            bjp2 = bjp1;
            bjp1 = bj;
        }
        bj = x2 * bjp1 - bjp2 + d[0];
        return Half * (bj - bjp2) * x;
    } else if (Two < xv && xv < xup) {
        x2 = Two - 20.0 / (xv + Three);
        bjp2 = Zero;
        bjp1 = c[ncfc - 1];
        for (j = ncfd - 1; j >= 2; --j) {
            bj = x2 * bjp1 - bjp2 + c[j - 1];
            bjp2 = bjp1;
            bjp1 = bj;
        }
        /* j == 1 here */
        bj = x2 * bjp1 - bjp2 + c[j - 1];
        x2 = Half * (bj - bjp2) / xv * exp(-x * x) / sqrtpi;
        return (One - x2) * fsign(One, x);
    }
    return fsign(One, x);
}

/* CardinalBSpline, mollib.F90:1629-1685 (values and first derivatives). */
int orc_cardinal_bspline(int order, double pos, int *kmax, double *values, double *derivs) {
    double lastvals[64];
    int v, n, i;
    double x, a;
    if (order < 1 || order > 64) return -1;
    v = (int)floor(pos);
    x = pos - v;
    *kmax = v;
    for (i = 0; i < order; ++i) lastvals[i] = 0.0;
    values[0] = x;
    if (order > 1) {
        values[1] = (1.0 - x);
        for (n = 3; n <= order; ++n) {
            for (i = 0; i < order; ++i) lastvals[i] = values[i];
            values[0] = x * lastvals[0] / (n - 1);
            for (i = 1; i <= n - 2; ++i) {
                a = i + x;
                values[i] = (a * lastvals[i] + (n - a) * lastvals[i - 1]) / (n - 1);
            }
            values[n - 1] = (1 - x) * lastvals[n - 2] / (n - 1);
        }
        n = order;
        if (derivs) {
            derivs[0] = lastvals[0];
            for (i = 1; i <= n - 2; ++i) derivs[i] = lastvals[i] - lastvals[i - 1];
            derivs[n - 1] = -lastvals[n - 2];
        }
    }
    return 0;
}

/* Random, mollib.F90:2689-2709 (Park-Miller with a Marsaglia shift). */
static double rnd_am;
static int32_t rnd_ix = -1, rnd_iy = -1;
double orc_random(int32_t *idum) {
    const int32_t ia = 16807, im = 2147483647, iq = 127773, ir = 2836;
    int32_t k;
    if (*idum <= 0 || rnd_iy < 0) {
        /* nearest(1.0,-1.0)/im: default (single-precision) real, im converted to it */
        rnd_am = (double)(nextafterf(1.0f, -1.0f) / (float)im);
        rnd_iy = ((888889999 ^ abs(*idum)) | 1);
        rnd_ix = 777755555 ^ abs(*idum);
        *idum = abs(*idum) + 1;
    }
    uint32_t ux = (uint32_t)rnd_ix;
    ux ^= ux << 13;
    ux ^= ux >> 17;   /* ishft(ix,-17) is a logical shift */
    ux ^= ux << 5;
    rnd_ix = (int32_t)ux;
    k = rnd_iy / iq;
    rnd_iy = ia * (rnd_iy - k * iq) - ir * k;
    if (rnd_iy < 0) rnd_iy += im;
    return rnd_am * (double)((im & (rnd_ix ^ rnd_iy)) | 1);
}

/* GauRandom, mollib.F90:2739-2766: polar Box-Muller over the 31-bit LCG
   iseed = ibclr(iseed*16087, 31) (32-bit wrapping product).  The reference
   keeps flag/save as SAVE variables; they are explicit state here. */
double orc_gau_random(int32_t *iseed, int32_t *flag, double *save) {
    const double f = 1.0 / 2147483648.0;   /* 2**(-31) */
    double rx, ry, r, fac;
    if (*flag) {
        for (;;) {
            *iseed = (int32_t)(((uint32_t)*iseed * 16087u) & 0x7fffffffu);
            rx = Two * (f * *iseed - Half);
            *iseed = (int32_t)(((uint32_t)*iseed * 16087u) & 0x7fffffffu);
            ry = Two * (f * *iseed - Half);
            r = rx * rx + ry * ry;
            if (r < One) break;
        }
        fac = sqrt(-Two * log(r) / r);
        *save = ry * fac;
        *flag = 0;
        return rx * fac;
    }
    *flag = 1;
    return *save;
}

/* HeapSortIndex, mollib.F90:1749-1796 (1-based index output). */
static void heap_sort_index(int n, const double *vec, int *index) {
    int l, i, j, ir, indext;
    double vect;
    for (i = 1; i <= n; ++i) index[i - 1] = i;
    if (n <= 1) return;
#define V(k) vec[(k) - 1]
#define IX(k) index[(k) - 1]
    l = n / 2 + 1;
    ir = n;
    for (;;) {
        if (l > 1) {
            l = l - 1;
            indext = IX(l);
            vect = V(indext);
        } else {
            indext = IX(ir);
            vect = V(indext);
            IX(ir) = IX(1);
            ir = ir - 1;
            if (ir == 1) { IX(1) = indext; return; }
        }
        i = l;
        j = l + l;
        while (j <= ir) {
            if (j < ir) {
                if (V(IX(j)) < V(IX(j + 1))) j = j + 1;
            }
            if (vect < V(IX(j))) {
                IX(i) = IX(j);
                i = j;
                j = j + j;
            } else {
                j = ir + 1;
            }
        }
        IX(i) = indext;
    }
#undef V
#undef IX
}

/* ======================================================================
 * potential.F90 : table construction
 * ====================================================================== */

/* CalcEwaldUfac, potential.F90:2938-2966 */
void orc_calc_ewald_ufac(double r1, double ualpha, double *c0fac, double *c1fac, double *c2fac) {
    const double fac = 1.12837916709;
    double ra = ualpha * r1;
    double er = orc_erf2(ra);
    double ex = fac * exp(-(ra * ra));
    *c0fac = One - (er);
    *c1fac = One - (er - ra * ex);
    *c2fac = One - (er - ra * (One + ra * ra) * ex);
}

static inline int iptpt_of(const int32_t *iptpt, int npt, int ipt, int jpt) {   /* 1-based in/out */
    return iptpt[(jpt - 1) * npt + (ipt - 1)];
}

/* Pot_1_6_12 'calc', potential.F90:1386-1428 (one atom per particle type). */
void orc_pot_1_6_12(const mg_pot_params *pp, int iat, int jat, double r1,
                    double *u0, double *u1, double *u2) {
    double qq = pp->zat[iat - 1] * pp->zat[jat - 1] * pp->epsi_four_pi;
    double sig = 0.5 * (pp->sigat[iat - 1] + pp->sigat[jat - 1]);
    double eps = sqrt(pp->epsat[iat - 1] * pp->epsat[jat - 1]);
    double r1i = One / r1;
    double fac = pow6(sig * r1i);
    double c0fac, c1fac, c2fac;
    if (pp->lcharge_ewald) orc_calc_ewald_ufac(r1, pp->ualpha, &c0fac, &c1fac, &c2fac);
    else { c0fac = One; c1fac = One; c2fac = One; }
    double ushort0 = +Four * eps * (fac * fac - fac);
    double ushort1 = -(24.0 * eps * (Two * (fac * fac) - fac) * r1i);
    double ushort2 = +24.0 * eps * (26.0 * (fac * fac) - 7.0 * fac) * (r1i * r1i);
    if (pp->lljcut) {
        if (r1 < pp->ljrcut * sig) {
            ushort0 = ushort0 + pp->ljushift * eps;
        } else {
            ushort0 = Zero; ushort1 = Zero; ushort2 = Zero;
        }
    }
    *u0 = qq * c0fac * r1i + ushort0;
    *u1 = -(qq * c1fac * (r1i * r1i)) + ushort1;
    *u2 = Two * qq * c2fac * pow3(r1i) + ushort2;
}

/* SetUBuffer, potential.F90:1139-1221 */
static void set_ubuffer(double zlow, double u0low, double u1low, double u2low,
                        double zupp, double u0upp, double u1upp, double u2upp, double *ubuft) {
    double dz1, dz2, dz3, rlow, rupp, w0low, w1low, w2low, w0upp, w1upp, w2upp, a, b, c;
    if ((u0low == Zero) && (u0upp == Zero)) {
        ubuft[0] = zlow;
        for (int i = 1; i < 12; ++i) ubuft[i] = Zero;
        return;
    }
    rlow = sqrt(zlow);
    rupp = sqrt(zupp);
    dz1 = zupp - zlow;
    dz2 = dz1 * dz1;
    dz3 = dz2 * dz1;
    w0low = u0low;
    w0upp = u0upp;
    w1low = 0.50 * u1low / rlow;
    w1upp = 0.50 * u1upp / rupp;
    w2low = 0.25 * (u2low - u1low / rlow) / zlow;
    w2upp = 0.25 * (u2upp - u1upp / rupp) / zupp;
    a = 6.0 * (w0upp - w0low - w1low * dz1 - 0.5 * w2low * dz2) / dz3;
    b = 2.0 * (w1upp - w1low - w2low * dz1) / dz2;
    c = (w2upp - w2low) / dz1;
    ubuft[0] = zlow;
    ubuft[1] = w0low;
    ubuft[2] = w1low;
    ubuft[3] = 0.5 * w2low;
    ubuft[4] = (10.0 * a - 12.0 * b + 3.0 * c) / (6.0);
    ubuft[5] = (-15.0 * a + 21.0 * b - 6.0 * c) / (6.0 * dz1);
    ubuft[6] = (2.0 * a - 3.0 * b + c) / (2.0 * dz2);
    ubuft[7] = -2.0 * ubuft[2];
    ubuft[8] = -4.0 * ubuft[3];
    ubuft[9] = -6.0 * ubuft[4];
    ubuft[10] = -8.0 * ubuft[5];
    ubuft[11] = -10.0 * ubuft[6];
}

/* CheckUBuffer, potential.F90:1224-1263 */
static void check_ubuffer(const mg_pot_params *pp, int iat, int jat, double rlow, double rupp,
                          const double *ubuft, int *ok, int *repul) {
    const int ncheck = 11;
    double dr, dz, r1, u0, u1, u2, usum, fsum;
    *ok = 0;
    *repul = 0;
    dr = (rupp - rlow) / (ncheck - 1);
    for (int icheck = 1; icheck <= ncheck; ++icheck) {
        r1 = rlow + dr * (icheck - 1);
        orc_pot_1_6_12(pp, iat, jat, r1, &u0, &u1, &u2);
        dz = r1 * r1 - rlow * rlow;
        usum = ubuft[1] + dz * (ubuft[2] + dz * (ubuft[3] + dz * (ubuft[4] + dz * (ubuft[5] + dz * ubuft[6]))));
        fsum = ubuft[7] + dz * (ubuft[8] + dz * (ubuft[9] + dz * (ubuft[10] + dz * ubuft[11])));
        fsum = r1 * fsum;
        if (fabs(usum - u0) > pp->utoltab) return;
        if (fabs(fsum + u1) > pp->ftoltab) return;
        if (fabs(usum) > pp->umaxtab) *repul = 1;
        if (fabs(fsum) > pp->fmaxtab) *repul = 1;
    }
    *ok = 1;
}

/* PotTwoBodyTab1/2/3, potential.F90:868-1136, for the (1,6,12) potential of a
   monoatomic system (atom type == particle type, racom = 0). */
int orc_pot_twobody_tab(const mg_pot_params *pp, double *ubuf, int32_t nbuf_cap,
                        int32_t *nbuf_used, int32_t *iubuflow, double *r2umin,
                        int32_t *nugrid) {
    const int mnugrid = 1200, ndr = 100;
    const double drfac = 0.9, rumaxfac = 1.1;
    int npt = pp->npt, nptpt = npt * (npt + 1) / 2;
    int cap = 12 * mnugrid * nptpt;
    double *buf = calloc((size_t)cap, sizeof(double));
    int *lset = calloc((size_t)nptpt, sizeof(int));
    int ibuf = 1;
    int status = 0;
    if (!buf || !lset) { free(buf); free(lset); return MG_ERR_ALLOC; }
    for (int ipt = 1; ipt <= npt && !status; ++ipt) {
        for (int jpt = ipt; jpt <= npt && !status; ++jpt) {
            int iatjat = iptpt_of(pp->iptpt, npt, ipt, jpt);
            double r2uminv = pp->r2uminin;                               /* 'init' */
            double r2umaxv = pow2(rumaxfac * (pp->rcut + 0.0 + 0.0));
            if (lset[iatjat - 1]) continue;
            double rumax = sqrt(r2umaxv);
            double rumin = sqrt(r2uminv);
            /* PotTwoBodyTab3 */
            int igrid, idr = 0;
            double rupp, rlow = 0, zlow, zupp, dr, ubuft[12];
            double u0low, u1low, u2low, u0upp, u1upp, u2upp;
            iubuflow[iatjat - 1] = ibuf;
            rupp = rumax;
            dr = Half * (rumax - rumin);
            for (igrid = 1; igrid <= mnugrid; ++igrid) {
                int ok = 0, repul = 0;
                zupp = rupp * rupp;
                for (idr = 1; idr <= ndr; ++idr) {
                    rlow = rupp - dr;
                    rlow = (rumin > rlow) ? rumin : rlow;
                    zlow = rlow * rlow;
                    orc_pot_1_6_12(pp, ipt, jpt, rlow, &u0low, &u1low, &u2low);
                    orc_pot_1_6_12(pp, ipt, jpt, rupp, &u0upp, &u1upp, &u2upp);
                    set_ubuffer(zlow, u0low, u1low, u2low, zupp, u0upp, u1upp, u2upp, ubuft);
                    check_ubuffer(pp, ipt, jpt, rlow, rupp, ubuft, &ok, &repul);
                    if (ok) {
                        rupp = rlow;
                        if (pp->lljcut) dr = Two * dr;
                        break;
                    }
                    dr = dr * drfac;
                }
                if (idr >= ndr + 1) { status = MG_ERR_TABLE; break; }
                if (ibuf + 11 > cap) { status = MG_ERR_TABLE; break; }
                memcpy(buf + ibuf - 1, ubuft, sizeof(ubuft));
                ibuf = ibuf + 12;
                if (repul) rumin = rlow;
                if (rlow <= rumin) break;
                if (repul) break;
            }
            if (status) break;
            if (igrid >= mnugrid + 1) { status = MG_ERR_TABLE; break; }
            nugrid[iatjat - 1] = igrid;
            r2umin[iatjat - 1] = rumin * rumin;
            lset[iatjat - 1] = 1;
        }
    }
    *nbuf_used = ibuf - 1;
    if (!status) {
        if (ibuf - 1 > nbuf_cap || !ubuf) status = MG_ERR_TABLE;
        else memcpy(ubuf, buf, sizeof(double) * (size_t)(ibuf - 1));
    }
    free(buf);
    free(lset);
    return status;
}

/* RcutToAlpha, energy.F90:7090-7106 (lq2sum == 0) */
int orc_rcut_to_alpha(double uewaldtol, double rcut, double q2sum, double boxlenshort,
                      double epsi_four_pi, double *ualpha) {
    double y, xold, xnew = 0;
    int i;
    y = (uewaldtol / (q2sum * epsi_four_pi)) * sqrt(Two * pow3(boxlenshort * rcut));
    xold = 1.0e-1;
    for (i = 1; i <= 40; ++i) {
        xnew = (One / rcut) * sqrt(-log(y * (xold * xold)));
        if (fabs(xold - xnew) / xnew < 1.0e-6) break;
        xold = xnew;
    }
    if (i > 40) return MG_ERR_ARG;
    *ualpha = xnew;
    return 0;
}

/* ======================================================================
 * System state (MolModule / EnergyModule / CellListModule globals)
 * ====================================================================== */

typedef struct { int npart, nneighcell, iphead; int *neigh; } orc_cell;

struct orc_sys {
    int np, npt, nptpt;
    int *iptpn, *iptpt;
    double *az;
    int nbuf;
    double *ubuf, *r2umin, *r2atat;
    int *iubuflow;
    double boxlen[3], boxlen2[3], boxleni[3], dpbc[3], TwoPiBoxi[3], vol, boxlenshort;
    double rcut, rcut2, drnlist;
    int txintlist, mode, maxnneigh;
    int ewald, ncut, ncut2, nkvec, order, nmesh, lsurf;
    double ualpha, ualpha2, EpsiFourPi, force_fac;
    /* bonds */
    int nbond;
    int *bond_ip, *bond_jp, *bond_p;
    double *bond_k, *bond_eq;
    /* angles */
    int nangle;
    int *angle_jm, *angle_ip, *angle_jp, *angle_p;
    double *angle_k, *angle_eq;
    double u_angle;
    /* chain neighbours for DUBond/DUAngle (bondnn of the reference, from the
       bond list: bond b joins lower bond_ip and upper bond_jp), the bond to
       each neighbour, the angle with each particle as vertex (0-based, -1 none) */
    int *nn_lo, *nn_up, *bond_lo, *bond_up, *angle_at;
    double du_bond, du_angle;
    /* state */
    double *ro, *force, *forceo, *u_twob, *utwobnew, *utwobold;
    double u_tot, u_rec, u_bond, virial;
    /* vlist */
    int *nneighpn, *jpnlist;
    double *drosum;
    /* cell list */
    int ncellX, ncellY, ncellZ, maxneighcell;
    double cellSize[3], cellSizei[3];
    orc_cell *cell;
    int *ipnext, *ipprev, *cellip;   /* cellip: 0-based cell id, -1 if none */
    /* std Ewald */
    double *kfac;
    zc *eikx, *eiky, *eikz, *eikyzm, *eikyzp, *eikr, *sumeikr;     /* eik*(na,0:ncut), sumeikr(nkvec,4) */
    zc *eikxtm, *eikytm, *eikztm, *eikyzmtm, *eikyzptm, *sumeikrtm;
    /* SPME */
    int s[3];
    double dkdr[3];
    double *meshfac, *energyfac, *virfac;   /* (0:s/2)^3, x fastest */
    double *Qmesh, *QmeshTM, *FQmesh, *Qspread;
    double *spline, *deriv;                 /* (0:order-1, 3, na) */
    int *meshmax;                           /* (3, na) */
    double *splinetm, *derivtm;
    int *meshmaxtm;
    double urecold, urecnew;
    int have_rec;                           /* a UTotal has set the MC Ewald state */
    /* MC trial */
    int nptm;
    int *ipnptm, *lptm;
    double *rotm;
    double du_twob0, du_rec, du_tot;
    int trial_ok;
    /* MD */
    double tstep, *massip, *rod, *rodd, *roddo, *drostep;
    /* BD */
    double *fac1, *fac2;
    int32_t iseed, gflag;
    double gsave;
    int bd_have_force;
    /* private arrays of the threads (the MPI ranks' replicated arrays) */
    int nthr_alloc;
    double *thr_force, *thr_u, *thr_mesh;
};

/* private arrays for nt threads: force (3 np) and energies (nptpt + 1) per
   thread, and with SPME a charge mesh per thread */
static int thr_arrays(orc_sys *s, int nt) {
    if (s->nthr_alloc >= nt) return 0;
    free(s->thr_force);
    free(s->thr_u);
    free(s->thr_mesh);
    s->thr_force = (double *)malloc(sizeof(double) * (size_t)nt * 3 * s->np);
    s->thr_u = (double *)malloc(sizeof(double) * (size_t)nt * (s->nptpt + 1));
    s->thr_mesh = NULL;
    if (s->ewald == MG_EWALD_SPM)
        s->thr_mesh = (double *)malloc(sizeof(double) * (size_t)nt * s->nmesh * s->nmesh * s->nmesh);
    if (!s->thr_force || !s->thr_u || (s->ewald == MG_EWALD_SPM && !s->thr_mesh)) {
        s->nthr_alloc = 0;
        return MG_ERR_ALLOC;
    }
    s->nthr_alloc = nt;
    return 0;
}

#define RO(m, ip) s->ro[3 * ((ip) - 1) + (m) - 1]
#define FORCE(m, ia) s->force[3 * ((ia) - 1) + (m) - 1]
#define AZ(ia) s->az[(ia) - 1]
#define IPTPN(ip) s->iptpn[(ip) - 1]
#define IPTPT(i, j) s->iptpt[((j) - 1) * s->npt + ((i) - 1)]
#define UBUF(k) s->ubuf[(k) - 1]

static void *xcalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz); }

/* PBCr2, molaux.F90:149-184 (lbcbox) */
static inline void pbcr2(const orc_sys *s, double *dx, double *dy, double *dz, double *r2) {
    if (fabs(*dx) > s->boxlen2[0]) *dx = *dx - fsign(s->dpbc[0], *dx);
    if (fabs(*dy) > s->boxlen2[1]) *dy = *dy - fsign(s->dpbc[1], *dy);
    if (fabs(*dz) > s->boxlen2[2]) *dz = *dz - fsign(s->dpbc[2], *dz);
    *r2 = *dx * *dx + *dy * *dy + *dz * *dz;
}

/* PBC, molaux.F90:104-146 (lbcbox): ANINT rounds half away from zero */
static inline void pbc(const orc_sys *s, double *dx, double *dy, double *dz) {
    if (fabs(*dx) > s->boxlen2[0]) *dx = *dx - s->dpbc[0] * round(*dx * s->boxleni[0]);
    if (fabs(*dy) > s->boxlen2[1]) *dy = *dy - s->dpbc[1] * round(*dy * s->boxleni[1]);
    if (fabs(*dz) > s->boxlen2[2]) *dz = *dz - s->dpbc[2] * round(*dz * s->boxleni[2]);
}

/* ======================================================================
 * EwaldSetup, energy.F90:6601-7049
 * ====================================================================== */
static int ewald_setup(orc_sys *s) {
    if (s->ewald == MG_EWALD_STD) {
        int ncut = s->ncut, nk = 0;
        s->nkvec = (ncut + 1) * (ncut + 1) * (ncut + 1);
        s->kfac = xcalloc((size_t)s->nkvec, sizeof(double));
        double fac0 = TwoPi / s->vol;
        for (int nz = 0; nz <= ncut; ++nz) {
            double facz = Two;
            if (nz == 0) facz = One;
            for (int ny = 0; ny <= ncut; ++ny) {
                double facy = One;
                if (ny == 0) facy = Half;
                for (int nx = 0; nx <= ncut; ++nx) {
                    if (nx * nx + ny * ny + nz * nz > s->ncut2) continue;
                    if (nx == 0 && ny == 0 && nz == 0) continue;
                    nk = nk + 1;
                    double facx = One;
                    if (nx == 0) facx = Half;
                    double k2 = pow2(nx * s->TwoPiBoxi[0]) + pow2(ny * s->TwoPiBoxi[1]) + pow2(nz * s->TwoPiBoxi[2]);
                    s->kfac[nk - 1] = fac0 * facz * facy * facx * exp(-k2 / (Four * (s->ualpha * s->ualpha))) / k2;
                }
            }
        }
        s->nkvec = nk;
        size_t na = (size_t)s->np, nc = (size_t)ncut + 1;
        s->eikx = xcalloc(na * nc, sizeof(zc)); s->eiky = xcalloc(na * nc, sizeof(zc)); s->eikz = xcalloc(na * nc, sizeof(zc));
        s->eikyzm = xcalloc(na, sizeof(zc)); s->eikyzp = xcalloc(na, sizeof(zc));
        s->eikr = xcalloc(na * 4, sizeof(zc));
        s->sumeikr = xcalloc((size_t)nk * 4, sizeof(zc));
        s->eikxtm = xcalloc(na * nc, sizeof(zc)); s->eikytm = xcalloc(na * nc, sizeof(zc)); s->eikztm = xcalloc(na * nc, sizeof(zc));
        s->eikyzmtm = xcalloc(na, sizeof(zc)); s->eikyzptm = xcalloc(na, sizeof(zc));
        s->sumeikrtm = xcalloc((size_t)nk * 4, sizeof(zc));
    } else if (s->ewald == MG_EWALD_SPM) {
        int order = s->order, n = s->nmesh;
        if (n <= 0 || order <= 0 || n % 2 != 0) return MG_ERR_ARG;
        s->s[0] = s->s[1] = s->s[2] = n;
        size_t m3 = (size_t)n * n * n, nh = (size_t)(n / 2 + 1);
        s->Qmesh = xcalloc(m3, sizeof(double));
        s->QmeshTM = xcalloc(m3, sizeof(double));
        s->Qspread = xcalloc(m3, sizeof(double));
        s->FQmesh = xcalloc(2 * nh * n * n, sizeof(double));
        s->meshfac = xcalloc(nh * nh * nh, sizeof(double));
        s->energyfac = xcalloc(nh * nh * nh, sizeof(double));
        s->virfac = xcalloc(nh * nh * nh, sizeof(double));
        s->spline = xcalloc((size_t)order * 3 * s->np, sizeof(double));
        s->deriv = xcalloc((size_t)order * 3 * s->np, sizeof(double));
        s->meshmax = xcalloc((size_t)3 * s->np, sizeof(int));
        s->splinetm = xcalloc((size_t)order * 3 * s->np, sizeof(double));
        s->derivtm = xcalloc((size_t)order * 3 * s->np, sizeof(double));
        s->meshmaxtm = xcalloc((size_t)3 * s->np, sizeof(int));
        for (int m = 0; m < 3; ++m) s->dkdr[m] = s->s[m] / s->boxlen[m];
        /* b(m)**2, eq (4.4) of JCP 1995, 103, 8577.  cmplx(0, x) without a KIND
           argument is single-precision complex in Fortran, so the phase is
           rounded to float and its exponential is a float: reproduced as
           float(angle) and correctly rounded float cos/sin. */
        double spl[64];
        int z;
        double *b2 = xcalloc((size_t)3 * n, sizeof(double));
        orc_cardinal_bspline(order, Zero, &z, spl, NULL);
        for (int i = 0; i < 3; ++i) {
            for (int m = 0; m < s->s[i]; ++m) {
                if ((order % 2 == 1) && (2 * m == s->s[i])) continue;
                double are = Zero, aim = Zero;
                for (int k = 0; k <= order - 2; ++k) {
                    float th = (float)(TwoPi * m * k / s->s[i]);
                    float ce = (float)cos((double)th), se = (float)sin((double)th);
                    /* a = a + spl(k+1)*cmplx(ce,se): real(8) times complex(4) */
                    are = are + spl[k + 1] * (double)ce;
                    aim = aim + spl[k + 1] * (double)se;
                }
                b2[i * n + m] = One / (are * are + aim * aim);
            }
        }
        double fac0 = FourPi / s->vol;
        double expf_ = -One / (Four * (s->ualpha * s->ualpha));
        for (int nz = 0; nz <= n / 2; ++nz)
            for (int ny = 0; ny <= n / 2; ++ny)
                for (int nx = 0; nx <= n / 2; ++nx) {
                    size_t id = ((size_t)nz * nh + ny) * nh + nx;
                    if (nx == 0 && ny == 0 && nz == 0) {
                        s->meshfac[id] = Zero; s->energyfac[id] = Zero; s->virfac[id] = Zero;
                    } else {
                        double m2 = pow2(nx * s->TwoPiBoxi[0]) + pow2(ny * s->TwoPiBoxi[1]) + pow2(nz * s->TwoPiBoxi[2]);
                        double c = exp(m2 * expf_) / m2;
                        double mf = fac0 * c * b2[nx] * b2[n + ny] * b2[2 * n + nz];
                        s->meshfac[id] = mf;
                        if (nx == (n - nx) % n) mf = mf / 2;
                        if (ny == (n - ny) % n) mf = mf / 2;
                        if (nz == (n - nz) % n) mf = mf / 2;
                        s->energyfac[id] = mf;
                        s->virfac[id] = (One + 2 * m2 * expf_) * mf;
                    }
                }
        free(b2);
    }
    s->ualpha2 = s->ualpha * s->ualpha;
    return 0;
}

int orc_create(const mg_params *p, orc_sys **out) {
    if (!p || !out || p->abi_version != MG_ABI_VERSION || p->np < 1 || p->npt < 1) return MG_ERR_ARG;
    orc_sys *s = xcalloc(1, sizeof(orc_sys));
    int np = p->np;
    s->np = np; s->npt = p->npt; s->nptpt = p->nptpt;
    s->iptpn = xcalloc(np, sizeof(int)); memcpy(s->iptpn, p->iptpn, sizeof(int) * np);
    s->iptpt = xcalloc((size_t)p->npt * p->npt, sizeof(int)); memcpy(s->iptpt, p->iptpt, sizeof(int) * p->npt * p->npt);
    s->az = xcalloc(np, sizeof(double)); memcpy(s->az, p->az, sizeof(double) * np);
    s->nbuf = p->nbuf;
    s->ubuf = xcalloc(p->nbuf, sizeof(double)); memcpy(s->ubuf, p->ubuf, sizeof(double) * p->nbuf);
    s->iubuflow = xcalloc(p->nptpt, sizeof(int)); memcpy(s->iubuflow, p->iubuflow, sizeof(int) * p->nptpt);
    s->r2umin = xcalloc(p->nptpt, sizeof(double)); memcpy(s->r2umin, p->r2umin, sizeof(double) * p->nptpt);
    s->r2atat = xcalloc(p->nptpt, sizeof(double)); memcpy(s->r2atat, p->r2atat, sizeof(double) * p->nptpt);
    for (int m = 0; m < 3; ++m) {
        s->boxlen[m] = p->boxlen[m];
        s->boxlen2[m] = p->boxlen[m] / Two;
        s->boxleni[m] = One / p->boxlen[m];
        s->TwoPiBoxi[m] = TwoPi * s->boxleni[m];
        s->dpbc[m] = p->boxlen[m];
    }
    s->vol = p->boxlen[0] * p->boxlen[1] * p->boxlen[2];
    s->boxlenshort = fmin(fmin(p->boxlen[0], p->boxlen[1]), p->boxlen[2]);
    s->rcut = p->rcut; s->rcut2 = p->rcut * p->rcut; s->drnlist = p->drnlist;
    s->txintlist = p->txintlist; s->mode = p->mode;
    s->maxnneigh = p->maxnneigh > 0 ? p->maxnneigh : np - 1;
    if (s->maxnneigh < 1) s->maxnneigh = 1;
    s->ewald = p->ewald; s->ualpha = p->ualpha; s->ncut = p->ncut;
    s->ncut2 = p->ncutregion_cube ? 3 * p->ncut * p->ncut : p->ncut * p->ncut;
    s->order = p->order; s->nmesh = p->nmesh; s->lsurf = p->lsurf;
    s->EpsiFourPi = p->epsi_four_pi; s->force_fac = p->force_fac;
    s->nbond = p->nbond;
    if (s->nbond > 0) {
        s->bond_ip = xcalloc(s->nbond, sizeof(int)); memcpy(s->bond_ip, p->bond_ip, sizeof(int) * s->nbond);
        s->bond_jp = xcalloc(s->nbond, sizeof(int)); memcpy(s->bond_jp, p->bond_jp, sizeof(int) * s->nbond);
        s->bond_p = xcalloc(s->nbond, sizeof(int)); memcpy(s->bond_p, p->bond_p, sizeof(int) * s->nbond);
        s->bond_k = xcalloc(s->nbond, sizeof(double)); memcpy(s->bond_k, p->bond_k, sizeof(double) * s->nbond);
        s->bond_eq = xcalloc(s->nbond, sizeof(double)); memcpy(s->bond_eq, p->bond_eq, sizeof(double) * s->nbond);
    }
    s->nn_lo = xcalloc(s->np, sizeof(int));
    s->nn_up = xcalloc(s->np, sizeof(int));
    s->bond_lo = xcalloc(s->np, sizeof(int));
    s->bond_up = xcalloc(s->np, sizeof(int));
    s->angle_at = xcalloc(s->np, sizeof(int));
    for (int i = 0; i < s->np; ++i) s->bond_lo[i] = s->bond_up[i] = s->angle_at[i] = -1;
    for (int b = 0; b < s->nbond; ++b) {
        int i = p->bond_ip[b], j = p->bond_jp[b];   /* 1-based */
        s->nn_up[i - 1] = j;
        s->bond_up[i - 1] = b;
        s->nn_lo[j - 1] = i;
        s->bond_lo[j - 1] = b;
    }
    for (int a = 0; a < p->nangle; ++a) s->angle_at[p->angle_ip[a] - 1] = a;
    s->nangle = p->nangle;
    if (s->nangle > 0) {
        size_t na = (size_t)s->nangle;
        s->angle_jm = xcalloc(na, sizeof(int)); memcpy(s->angle_jm, p->angle_jm, sizeof(int) * na);
        s->angle_ip = xcalloc(na, sizeof(int)); memcpy(s->angle_ip, p->angle_ip, sizeof(int) * na);
        s->angle_jp = xcalloc(na, sizeof(int)); memcpy(s->angle_jp, p->angle_jp, sizeof(int) * na);
        s->angle_p = xcalloc(na, sizeof(int)); memcpy(s->angle_p, p->angle_p, sizeof(int) * na);
        s->angle_k = xcalloc(na, sizeof(double)); memcpy(s->angle_k, p->angle_k, sizeof(double) * na);
        s->angle_eq = xcalloc(na, sizeof(double)); memcpy(s->angle_eq, p->angle_eq, sizeof(double) * na);
    }
    s->ro = xcalloc((size_t)3 * np, sizeof(double));
    s->force = xcalloc((size_t)3 * np, sizeof(double));
    s->forceo = xcalloc((size_t)3 * np, sizeof(double));
    s->u_twob = xcalloc((size_t)s->nptpt + 1, sizeof(double));
    s->utwobnew = xcalloc((size_t)s->nptpt + 1, sizeof(double));
    s->utwobold = xcalloc((size_t)s->nptpt + 1, sizeof(double));
    s->drosum = xcalloc((size_t)3 * np, sizeof(double));
    s->drostep = xcalloc((size_t)3 * np, sizeof(double));
    s->ipnptm = xcalloc(np, sizeof(int));
    s->lptm = xcalloc(np, sizeof(int));
    s->rotm = xcalloc((size_t)3 * np, sizeof(double));
    s->cellip = xcalloc(np, sizeof(int));
    s->ipnext = xcalloc(np, sizeof(int));
    s->ipprev = xcalloc(np, sizeof(int));
    s->gflag = 1;
    int st = ewald_setup(s);
    if (st) { orc_destroy(s); return st; }
    *out = s;
    return 0;
}

void orc_destroy(orc_sys *s) {
    if (!s) return;
    void *ptrs[] = {s->iptpn, s->iptpt, s->az, s->ubuf, s->r2umin, s->r2atat, s->iubuflow,
                    s->bond_ip, s->bond_jp, s->bond_p, s->bond_k, s->bond_eq,
                    s->angle_jm, s->angle_ip, s->angle_jp, s->angle_p, s->angle_k, s->angle_eq,
                    s->nn_lo, s->nn_up, s->bond_lo, s->bond_up, s->angle_at,
                    s->ro, s->force, s->forceo, s->u_twob, s->utwobnew, s->utwobold,
                    s->nneighpn, s->jpnlist, s->drosum, s->ipnext, s->ipprev, s->cellip,
                    s->kfac, s->eikx, s->eiky, s->eikz, s->eikyzm, s->eikyzp, s->eikr, s->sumeikr,
                    s->eikxtm, s->eikytm, s->eikztm, s->eikyzmtm, s->eikyzptm, s->sumeikrtm,
                    s->meshfac, s->energyfac, s->virfac, s->Qmesh, s->QmeshTM, s->FQmesh, s->Qspread,
                    s->spline, s->deriv, s->meshmax, s->splinetm, s->derivtm, s->meshmaxtm,
                    s->ipnptm, s->lptm, s->rotm, s->massip, s->rod, s->rodd, s->roddo, s->drostep,
                    s->fac1, s->fac2, s->thr_force, s->thr_u, s->thr_mesh};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
    if (s->cell) {
        int nc = s->ncellX * s->ncellY * s->ncellZ;
        for (int i = 0; i < nc; ++i) free(s->cell[i].neigh);
        free(s->cell);
    }
    free(s);
}

int orc_set_positions(orc_sys *s, const double *ro) {
    memcpy(s->ro, ro, sizeof(double) * 3 * s->np);
    return 0;
}
int orc_get_positions(orc_sys *s, double *ro) {
    memcpy(ro, s->ro, sizeof(double) * 3 * s->np);
    return 0;
}

/* ======================================================================
 * celllist.F90
 * ====================================================================== */

static inline int id_cell_pos(const orc_sys *s, int ix, int iy, int iz) {   /* 0-based id */
    return ix + iy * s->ncellX + iz * (s->ncellX * s->ncellY);
}

/* InitCellList, celllist.F90:76-265 */
static int init_cell_list(orc_sys *s, double rcell) {
    int dirRange[3];
    if (rcell <= 0.0) return MG_ERR_ARG;
    int oldX = s->ncellX, oldY = s->ncellY, oldZ = s->ncellZ;
    double ircell = 1.0 / rcell;
    int nc[3];
    for (int m = 0; m < 3; ++m) {
        nc[m] = (int)floor(s->boxlen[m] * ircell);
        if (nc[m] < 1) nc[m] = 1;
        s->cellSize[m] = s->boxlen[m] / nc[m];
        s->cellSizei[m] = 1.0 / s->cellSize[m];
    }
    for (int m = 0; m < 3; ++m) dirRange[m] = (int)ceil(s->rcut * s->cellSizei[m]);
    for (int m = 0; m < 3; ++m) {
        if (2 * dirRange[m] + 1 > nc[m]) {
            nc[m] = 1;
            dirRange[m] = 0;
            s->cellSize[m] = s->boxlen[m];
            s->cellSizei[m] = s->boxleni[m];
        }
    }
    s->ncellX = nc[0]; s->ncellY = nc[1]; s->ncellZ = nc[2];
    if (oldX == nc[0] && oldY == nc[1] && oldZ == nc[2] && s->cell) return 0;
    if (s->cell) {
        int ncold = oldX * oldY * oldZ;
        for (int i = 0; i < ncold; ++i) free(s->cell[i].neigh);
        free(s->cell);
        s->cell = NULL;
    }
    int maxdir = (2 * dirRange[0] + 1) * (2 * dirRange[1] + 1) * (2 * dirRange[2] + 1);
    int *dirs = xcalloc((size_t)3 * maxdir, sizeof(int));
    int *dsorted = xcalloc((size_t)3 * maxdir, sizeof(int));
    int *dindex = xcalloc(maxdir, sizeof(int));
    double *l1 = xcalloc(maxdir, sizeof(double));
    int idir = 0;
    for (int ixd = -dirRange[0]; ixd <= dirRange[0]; ++ixd)
        for (int iyd = -dirRange[1]; iyd <= dirRange[1]; ++iyd)
            for (int izd = -dirRange[2]; izd <= dirRange[2]; ++izd) {
                int d3[3] = {ixd, iyd, izd};
                double dr[3], sum = 0;
                for (int m = 0; m < 3; ++m) {
                    int a = abs(d3[m]) - 1;
                    if (a < 0) a = 0;
                    dr[m] = a * s->cellSize[m];
                }
                sum = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
                if (sum > s->rcut2) continue;
                dirs[3 * idir] = ixd; dirs[3 * idir + 1] = iyd; dirs[3 * idir + 2] = izd;
                idir++;
            }
    s->maxneighcell = idir;
    for (int i = 0; i < idir; ++i) l1[i] = (double)(abs(dirs[3 * i]) + abs(dirs[3 * i + 1]) + abs(dirs[3 * i + 2]));
    heap_sort_index(idir, l1, dindex);
    for (int i = 0; i < idir; ++i)
        for (int m = 0; m < 3; ++m) dsorted[3 * i + m] = dirs[3 * (dindex[i] - 1) + m];
    int ncell = nc[0] * nc[1] * nc[2];
    s->cell = xcalloc(ncell, sizeof(orc_cell));
    for (int ix = 0; ix < nc[0]; ++ix)
        for (int iy = 0; iy < nc[1]; ++iy)
            for (int iz = 0; iz < nc[2]; ++iz) {
                orc_cell *c = &s->cell[id_cell_pos(s, ix, iy, iz)];
                c->neigh = xcalloc(idir, sizeof(int));
                int ineigh = 0;
                for (int k = 0; k < idir; ++k) {
                    int ng[3] = {ix + dsorted[3 * k], iy + dsorted[3 * k + 1], iz + dsorted[3 * k + 2]};
                    for (int m = 0; m < 3; ++m) {
                        if ((ng[m] >= nc[m] || ng[m] < 0) && (s->dpbc[m] == s->boxlen[m])) {
                            ng[m] = ((ng[m] % nc[m]) + nc[m]) % nc[m];   /* Fortran modulo */
                        }
                    }
                    if (ng[0] >= nc[0] || ng[0] < 0 || ng[1] >= nc[1] || ng[1] < 0 || ng[2] >= nc[2] || ng[2] < 0) continue;
                    c->neigh[ineigh++] = id_cell_pos(s, ng[0], ng[1], ng[2]);
                }
                c->nneighcell = ineigh;
            }
    free(dirs); free(dsorted); free(dindex); free(l1);
    return 0;
}

/* pcellro, celllist.F90:295-305 (0-based id; -1 outside the grid) */
static int pcellro(const orc_sys *s, const double *r) {
    int i[3];
    int nc[3] = {s->ncellX, s->ncellY, s->ncellZ};
    for (int m = 0; m < 3; ++m) {
        i[m] = (int)floor((r[m] + s->boxlen2[m]) * s->cellSizei[m]);
        if (i[m] < 0 || i[m] >= nc[m]) return -1;
    }
    return id_cell_pos(s, i[0], i[1], i[2]);
}

/* AddIpToCell, celllist.F90:307-327 (ip 1-based; ipnext/ipprev 0 = none) */
static void add_ip_to_cell(orc_sys *s, int ip, int icell) {
    orc_cell *c = &s->cell[icell];
    c->npart = c->npart + 1;
    int jp = c->iphead;
    c->iphead = ip;
    if (jp != 0) {
        s->ipprev[jp - 1] = ip;
        s->ipnext[ip - 1] = jp;
    } else {
        s->ipnext[ip - 1] = 0;
    }
    s->ipprev[ip - 1] = 0;
    s->cellip[ip - 1] = icell;
}

/* RmIpFromCell, celllist.F90:329-364 */
static void rm_ip_from_cell(orc_sys *s, int ip, int icell) {
    orc_cell *c = &s->cell[icell];
    c->npart = c->npart - 1;
    int nextp = s->ipnext[ip - 1], prevp = s->ipprev[ip - 1];
    if (nextp == 0) {
        if (c->iphead == ip) c->iphead = 0;
        else s->ipnext[prevp - 1] = 0;
    } else {
        if (c->iphead == ip) {
            c->iphead = nextp;
            s->ipprev[nextp - 1] = 0;
        } else {
            s->ipprev[nextp - 1] = prevp;
            s->ipnext[prevp - 1] = nextp;
        }
    }
    s->ipprev[ip - 1] = 0;
    s->ipnext[ip - 1] = 0;
    s->cellip[ip - 1] = -1;
}

/* UpdateCellIp, celllist.F90:366-382 */
static int update_cell_ip(orc_sys *s, int ip) {
    int cold = s->cellip[ip - 1];
    int cnew = pcellro(s, &RO(1, ip));
    if (cnew < 0) return MG_ERR_CELL;
    if (cold != cnew) {
        rm_ip_from_cell(s, ip, cold);
        add_ip_to_cell(s, ip, cnew);
    }
    return 0;
}

/* SetCellList, celllist.F90:384-410 */
static int set_cell_list(orc_sys *s) {
    int nc = s->ncellX * s->ncellY * s->ncellZ;
    for (int i = 0; i < nc; ++i) { s->cell[i].npart = 0; s->cell[i].iphead = 0; }
    memset(s->ipnext, 0, sizeof(int) * s->np);
    memset(s->ipprev, 0, sizeof(int) * s->np);
    for (int ip = 1; ip <= s->np; ++ip) {
        int c = pcellro(s, &RO(1, ip));
        if (c < 0) return MG_ERR_CELL;
        add_ip_to_cell(s, ip, c);
    }
    return 0;
}

/* TestCellList, celllist.F90:447-476: every pair within rcut of a particle
   must be in one of the neighbour cells of its cell.  Returns the number of
   missing pairs. */
int orc_celllist_test(orc_sys *s) {
    int missing = 0;
    for (int ip = 1; ip <= s->np; ++ip) {
        orc_cell *ci = &s->cell[s->cellip[ip - 1]];
        for (int jp = 1; jp <= s->np; ++jp) {
            if (jp == ip) continue;
            double dx = RO(1, ip) - RO(1, jp), dy = RO(2, ip) - RO(2, jp), dz = RO(3, ip) - RO(3, jp), r2;
            pbcr2(s, &dx, &dy, &dz, &r2);
            if (r2 >= s->rcut2) continue;
            int found = 0;
            for (int k = 0; k < ci->nneighcell && !found; ++k)
                if (ci->neigh[k] == s->cellip[jp - 1]) found = 1;
            if (!found) missing++;
        }
    }
    return missing;
}

/* ======================================================================
 * nlist.F90
 * ====================================================================== */

/* SetVListMD, nlist.F90:724-765: the rows of particles ip in [lo, hi)
   (the reference's rank loop over ipmyid; every row depends on the
   positions only, so a split of the rows gives the serial lists) */
static int set_vlist_md_rows(orc_sys *s, int lo, int hi) {
    double rs2cut = pow2(s->rcut + s->drnlist);
    for (int ip = lo + 1; ip <= hi; ++ip) {
        int *nn = &s->nneighpn[ip - 1];
        *nn = 0;
        for (int jp = 1; jp <= s->np; ++jp) {
            int itemp = (ip + jp) % 2;
            if (ip < jp && itemp == 0) continue;
            if (ip > jp && itemp != 0) continue;
            if (ip == jp) continue;
            double dx = RO(1, ip) - RO(1, jp), dy = RO(2, ip) - RO(2, jp), dz = RO(3, ip) - RO(3, jp), r2;
            pbcr2(s, &dx, &dy, &dz, &r2);
            if (r2 < rs2cut) {
                *nn = *nn + 1;
                if (*nn > s->maxnneigh) return MG_ERR_NEIGH_OVERFLOW;
                s->jpnlist[(size_t)(ip - 1) * s->maxnneigh + (*nn - 1)] = jp;
            }
        }
    }
    return 0;
}

typedef struct {
    orc_sys *s;
    int st[ORC_MAX_THREADS];
} vlist_job;

static void vlist_job_run(void *ctx, int t, int nt) {
    vlist_job *j = (vlist_job *)ctx;
    long lo, hi;
    orc_range(j->s->np, t, nt, &lo, &hi);
    j->st[t] = set_vlist_md_rows(j->s, (int)lo, (int)hi);
}

static int set_vlist_md(orc_sys *s) {
    int nt = orc_threads();
    if (nt <= 1) return set_vlist_md_rows(s, 0, s->np);
    vlist_job j;
    j.s = s;
    orc_par_run(vlist_job_run, &j, nt);
    for (int t = 0; t < nt; ++t)
        if (j.st[t]) return j.st[t];
    return 0;
}

/* SetVListMC, nlist.F90:820-890 (serial branch) */
static int set_vlist_mc(orc_sys *s) {
    double rs2cut = pow2(s->rcut + s->drnlist);
    for (int ip = 1; ip <= s->np; ++ip) s->nneighpn[ip - 1] = 0;
    for (int ip = 1; ip <= s->np; ++ip) {
        for (int jp = ip + 1; jp <= s->np; ++jp) {
            double dx = RO(1, ip) - RO(1, jp), dy = RO(2, ip) - RO(2, jp), dz = RO(3, ip) - RO(3, jp), r2;
            pbcr2(s, &dx, &dy, &dz, &r2);
            if (r2 < rs2cut) {
                int ni = ++s->nneighpn[ip - 1], nj = ++s->nneighpn[jp - 1];
                if (ni > s->maxnneigh || nj > s->maxnneigh) return MG_ERR_NEIGH_OVERFLOW;
                s->jpnlist[(size_t)(ip - 1) * s->maxnneigh + (ni - 1)] = jp;
                s->jpnlist[(size_t)(jp - 1) * s->maxnneigh + (nj - 1)] = ip;
            }
        }
    }
    return 0;
}

static int set_vlist(orc_sys *s) {
    if (!s->nneighpn) {
        s->nneighpn = xcalloc(s->np, sizeof(int));
        s->jpnlist = xcalloc((size_t)s->np * s->maxnneigh, sizeof(int));
    }
    if (s->mode == MG_MC) return set_vlist_mc(s);
    return set_vlist_md(s);
}

/* NList(iWriteInput), nlist.F90:568-589 */
int orc_nlist_set(orc_sys *s) {
    int st;
    if (s->txintlist == MG_VLIST) {
        st = set_vlist(s);
    } else {
        st = init_cell_list(s, s->rcut + s->drnlist);
        if (!st) st = set_cell_list(s);
    }
    memset(s->drosum, 0, sizeof(double) * 3 * s->np);
    return st;
}

/* NList(iSimulationStep), nlist.F90:598-621 (inlist == 0).  With the cell
   list the reference relies on UpdateCellIp after MC moves and never
   refreshes cells in MD/BD; here the cell list is refreshed on the same
   displacement rule in MD/BD (the reference's cells would be stale). */
int orc_nlist_update(orc_sys *s, const double *drostep, int32_t *rebuilt) {
    double r2, r2max1 = Zero, r2max2 = Zero;
    const double *d = drostep ? drostep : s->drostep;
    *rebuilt = 0;
    if (s->txintlist == MG_CELLLIST && s->mode == MG_MC) return 0;
    for (int ip = 1; ip <= s->np; ++ip) {
        double *ds = &s->drosum[3 * (ip - 1)];
        ds[0] = ds[0] + d[3 * (ip - 1)];
        ds[1] = ds[1] + d[3 * (ip - 1) + 1];
        ds[2] = ds[2] + d[3 * (ip - 1) + 2];
        r2 = ds[0] * ds[0] + ds[1] * ds[1] + ds[2] * ds[2];
        if (r2 > r2max1) r2max1 = r2;
        else if (r2 > r2max2) r2max2 = r2;
    }
    if (sqrt(r2max1) + sqrt(r2max2) > s->drnlist) {
        memset(s->drosum, 0, sizeof(double) * 3 * s->np);
        *rebuilt = 1;
        if (s->txintlist == MG_VLIST) return set_vlist(s);
        return set_cell_list(s);
    }
    return 0;
}

int orc_nlist_get(orc_sys *s, int32_t *nneighpn, int32_t *jpnlist, int32_t maxnneigh) {
    if (!s->nneighpn) return MG_ERR_STATE;
    for (int ip = 0; ip < s->np; ++ip) {
        int n = s->nneighpn[ip];
        nneighpn[ip] = n;
        if (n > maxnneigh) return MG_ERR_NEIGH_OVERFLOW;
        for (int k = 0; k < n; ++k) jpnlist[(size_t)ip * maxnneigh + k] = s->jpnlist[(size_t)ip * s->maxnneigh + k];
    }
    return 0;
}

int orc_celllist_get(orc_sys *s, int32_t *ncell, int32_t *cellip) {
    if (!s->cell) return MG_ERR_STATE;
    ncell[0] = s->ncellX; ncell[1] = s->ncellY; ncell[2] = s->ncellZ;
    for (int ip = 0; ip < s->np; ++ip) cellip[ip] = s->cellip[ip];
    return 0;
}

/* ======================================================================
 * energy.F90 : two-body
 * ====================================================================== */

/* table lookup shared by the pair routines: energy.F90:481-490 */
static inline int table_eval(const orc_sys *s, int iptjpt, double r2, double *usum, double *fsum) {
    int ibuf = s->iubuflow[iptjpt - 1];
    for (;;) {
        if (r2 >= UBUF(ibuf)) break;
        ibuf = ibuf + 12;
        if (ibuf > s->nbuf) return MG_ERR_IBUF;
    }
    double d = r2 - UBUF(ibuf);
    *usum = UBUF(ibuf + 1) + d * (UBUF(ibuf + 2) + d * (UBUF(ibuf + 3) + d * (UBUF(ibuf + 4) + d * (UBUF(ibuf + 5) + d * UBUF(ibuf + 6)))));
    if (fsum) *fsum = UBUF(ibuf + 7) + d * (UBUF(ibuf + 8) + d * (UBUF(ibuf + 9) + d * (UBUF(ibuf + 10) + d * UBUF(ibuf + 11))));
    return 0;
}

/* The pair loops run over an ip range [lo, hi) (1-based ip = lo+1 .. hi),
   accumulating into the force array F, the per-pair-type energies U and the
   virial *vir: one range and the handle's own arrays is the serial
   reference; several ranges with private arrays are its MPI ranks. */
#define FRC(F, m, ia) (F)[3 * ((ia) - 1) + (m) - 1]

/* UTwoBodyA, energy.F90:445-544 (Verlet list: the MD half list or the MC full list) */
static int utwobody_a_range(orc_sys *s, long lo, long hi, double *F, double *U, double *vir) {
    double virtwob = Zero, fsum = Zero, usum;
    for (int ip = (int)lo + 1; ip <= (int)hi; ++ip) {
        int ipt = IPTPN(ip);
        for (int jploc = 1; jploc <= s->nneighpn[ip - 1]; ++jploc) {
            int jp = s->jpnlist[(size_t)(ip - 1) * s->maxnneigh + jploc - 1];
            if (s->mode == MG_MC && jp < ip) continue;
            int jpt = IPTPN(jp);
            int iptjpt = IPTPT(ipt, jpt);
            double dx = RO(1, ip) - RO(1, jp), dy = RO(2, ip) - RO(2, jp), dz = RO(3, ip) - RO(3, jp), r2;
            pbcr2(s, &dx, &dy, &dz, &r2);
            if (r2 > s->rcut2) continue;
            if (r2 < s->r2atat[iptjpt - 1]) {
                usum = 1e10;   /* fsum keeps its previous value, as in the reference */
            } else if (r2 < s->r2umin[iptjpt - 1]) {
                return MG_ERR_TABLE_UNDERRUN;
            } else {
                int st = table_eval(s, iptjpt, r2, &usum, &fsum);
                if (st) return st;
            }
            U[iptjpt] = U[iptjpt] + usum;
            FRC(F, 1, ip) = FRC(F, 1, ip) + (fsum * dx);
            FRC(F, 2, ip) = FRC(F, 2, ip) + (fsum * dy);
            FRC(F, 3, ip) = FRC(F, 3, ip) + (fsum * dz);
            FRC(F, 1, jp) = FRC(F, 1, jp) - (fsum * dx);
            FRC(F, 2, jp) = FRC(F, 2, jp) - (fsum * dy);
            FRC(F, 3, jp) = FRC(F, 3, jp) - (fsum * dz);
            virtwob = virtwob - (fsum * r2);
        }
    }
    *vir = virtwob;
    return 0;
}

/* UTwoBodyACellList, energy.F90:669-777 */
static int utwobody_a_celllist_range(orc_sys *s, long lo, long hi, double *F, double *U, double *vir) {
    double virtwob = Zero, usum, fsum;
    for (int ip = (int)lo + 1; ip <= (int)hi; ++ip) {
        int ipt = IPTPN(ip);
        orc_cell *ic = &s->cell[s->cellip[ip - 1]];
        for (int incell = 0; incell < ic->nneighcell; ++incell) {
            orc_cell *nc = &s->cell[ic->neigh[incell]];
            int jp = nc->iphead;
            for (int jploc = 1; jploc <= nc->npart; ++jploc) {
                if (jp > ip) {
                    int jpt = IPTPN(jp);
                    int iptjpt = IPTPT(ipt, jpt);
                    double dx = RO(1, ip) - RO(1, jp), dy = RO(2, ip) - RO(2, jp), dz = RO(3, ip) - RO(3, jp), r2;
                    pbcr2(s, &dx, &dy, &dz, &r2);
                    if (r2 < s->rcut2) {
                        if (r2 < s->r2atat[iptjpt - 1]) {
                            usum = 1e10;
                            fsum = 1e10;
                        } else if (r2 < s->r2umin[iptjpt - 1]) {
                            return MG_ERR_TABLE_UNDERRUN;
                        } else {
                            int st = table_eval(s, iptjpt, r2, &usum, &fsum);
                            if (st) return st;
                        }
                        U[iptjpt] = U[iptjpt] + usum;
                        FRC(F, 1, ip) = FRC(F, 1, ip) + (fsum * dx);
                        FRC(F, 2, ip) = FRC(F, 2, ip) + (fsum * dy);
                        FRC(F, 3, ip) = FRC(F, 3, ip) + (fsum * dz);
                        FRC(F, 1, jp) = FRC(F, 1, jp) - (fsum * dx);
                        FRC(F, 2, jp) = FRC(F, 2, jp) - (fsum * dy);
                        FRC(F, 3, jp) = FRC(F, 3, jp) - (fsum * dz);
                        virtwob = virtwob - (fsum * r2);
                    }
                }
                jp = s->ipnext[jp - 1];
            }
        }
    }
    *vir = virtwob;
    return 0;
}

/* the pair loop of either list over the threads' ranges; the private force
   arrays and energies are summed in thread order (the allreduce) */
typedef struct {
    orc_sys *s;
    int cell;
    double *F;     /* nt x 3 np */
    double *U;     /* nt x (nptpt + 1) */
    double vir[ORC_MAX_THREADS];
    int err[ORC_MAX_THREADS];
} pair_job;

static void pair_job_run(void *ctx, int t, int nt) {
    pair_job *j = (pair_job *)ctx;
    long lo, hi;
    orc_range(j->s->np, t, nt, &lo, &hi);
    double *F = j->F + (size_t)t * 3 * j->s->np, *U = j->U + (size_t)t * (j->s->nptpt + 1);
    memset(F, 0, sizeof(double) * 3 * j->s->np);
    memset(U, 0, sizeof(double) * (j->s->nptpt + 1));
    j->err[t] = j->cell ? utwobody_a_celllist_range(j->s, lo, hi, F, U, &j->vir[t])
                        : utwobody_a_range(j->s, lo, hi, F, U, &j->vir[t]);
}

static void force_sum_run(void *ctx, int t, int nt) {
    pair_job *j = (pair_job *)ctx;
    long n3 = 3L * j->s->np, lo, hi;
    orc_range(n3, t, nt, &lo, &hi);
    int ntot = orc_threads();
    for (long i = lo; i < hi; ++i) {
        double f = j->s->force[i];
        for (int k = 0; k < ntot; ++k) f = f + j->F[(size_t)k * n3 + i];
        j->s->force[i] = f;
    }
}

static int utwobody(orc_sys *s, int cell) {
    double virtwob = Zero;
    for (int k = 0; k <= s->nptpt; ++k) s->u_twob[k] = Zero;
    int nt = orc_threads();
    if (nt == 1) {
        int st = cell ? utwobody_a_celllist_range(s, 0, s->np, s->force, s->u_twob, &virtwob)
                      : utwobody_a_range(s, 0, s->np, s->force, s->u_twob, &virtwob);
        if (st) return st;
    } else {
        if (thr_arrays(s, nt)) return MG_ERR_ALLOC;
        pair_job j;
        j.s = s;
        j.cell = cell;
        j.F = s->thr_force;
        j.U = s->thr_u;
        orc_par_run(pair_job_run, &j, nt);
        int st = 0;
        for (int t = 0; t < nt && !st; ++t) st = j.err[t];
        if (!st) {
            orc_par_run(force_sum_run, &j, nt);
            for (int t = 0; t < nt; ++t) {
                for (int k = 1; k <= s->nptpt; ++k) s->u_twob[k] = s->u_twob[k] + j.U[(size_t)t * (s->nptpt + 1) + k];
                virtwob = virtwob + j.vir[t];
            }
        }
        if (st) return st;
    }
    double t = Zero;
    for (int k = 1; k <= s->nptpt; ++k) t = t + s->u_twob[k];
    s->u_twob[0] = t;
    s->u_tot = s->u_tot + s->u_twob[0];
    s->virial = s->virial + virtwob;
    return 0;
}

/* ======================================================================
 * energy.F90 : Ewald
 * ====================================================================== */

#define EIK(a, ia, n) (a)[(size_t)(n) * s->np + ((ia) - 1)]

/* EwaldSetArray, energy.F90:1401-1425 */
static void ewald_set_array(orc_sys *s, int ialow, int iaupp) {
    for (int ia = ialow; ia <= iaupp; ++ia) {
        zc one = {One, Zero};
        EIK(s->eikx, ia, 0) = one; EIK(s->eiky, ia, 0) = one; EIK(s->eikz, ia, 0) = one;
        double ax = s->TwoPiBoxi[0] * RO(1, ia), ay = s->TwoPiBoxi[1] * RO(2, ia), az = s->TwoPiBoxi[2] * RO(3, ia);
        zc ex = {cos(ax), sin(ax)}, ey = {cos(ay), sin(ay)}, ez = {cos(az), sin(az)};
        if (s->ncut >= 1) { EIK(s->eikx, ia, 1) = ex; EIK(s->eiky, ia, 1) = ey; EIK(s->eikz, ia, 1) = ez; }
    }
    for (int icut = 2; icut <= s->ncut; ++icut)
        for (int ia = ialow; ia <= iaupp; ++ia) {
            EIK(s->eikx, ia, icut) = zmul(EIK(s->eikx, ia, icut - 1), EIK(s->eikx, ia, 1));
            EIK(s->eiky, ia, icut) = zmul(EIK(s->eiky, ia, icut - 1), EIK(s->eiky, ia, 1));
            EIK(s->eikz, ia, icut) = zmul(EIK(s->eikz, ia, icut - 1), EIK(s->eikz, ia, 1));
        }
}

/* UEwaldRecStd, energy.F90:964-1102 (serial branch, :1046-1096) */
static void uewald_rec_std(orc_sys *s, double *virrec) {
    int na = s->np, kn = 0;
    ewald_set_array(s, 1, na);
    for (int i = 0; i < s->nkvec * 4; ++i) { s->sumeikr[i].re = Zero; s->sumeikr[i].im = Zero; }
    for (int nz = 0; nz <= s->ncut; ++nz) {
        for (int ny = 0; ny <= s->ncut; ++ny) {
            if (ny * ny + nz * nz > s->ncut2) continue;
            for (int ia = 1; ia <= na; ++ia) {
                s->eikyzm[ia - 1] = zmul(zconj(EIK(s->eiky, ia, ny)), EIK(s->eikz, ia, nz));
                s->eikyzp[ia - 1] = zmul(EIK(s->eiky, ia, ny), EIK(s->eikz, ia, nz));
            }
            for (int nx = 0; nx <= s->ncut; ++nx) {
                if (nx * nx + ny * ny + nz * nz > s->ncut2) continue;
                if (nx == 0 && ny == 0 && nz == 0) continue;
                kn = kn + 1;
                zc *S = &s->sumeikr[(size_t)(kn - 1) * 4];
                for (int ia = 1; ia <= na; ++ia) {
                    zc ex = EIK(s->eikx, ia, nx);
                    zc *er = &s->eikr[(size_t)(ia - 1) * 4];
                    er[0] = zmul(zscale(AZ(ia), zconj(ex)), s->eikyzm[ia - 1]);
                    er[1] = zmul(zscale(AZ(ia), zconj(ex)), s->eikyzp[ia - 1]);
                    er[2] = zmul(zscale(AZ(ia), ex), s->eikyzm[ia - 1]);
                    er[3] = zmul(zscale(AZ(ia), ex), s->eikyzp[ia - 1]);
                    for (int c = 0; c < 4; ++c) S[c] = zadd(S[c], er[c]);
                }
                double term = Zero;
                for (int c = 0; c < 4; ++c) term = term + (S[c].re * S[c].re + S[c].im * S[c].im);
                term = s->kfac[kn - 1] * term;
                s->u_rec = s->u_rec + term;
                double kfac2 = s->EpsiFourPi * Two * s->kfac[kn - 1];
                double kx = kfac2 * nx * s->TwoPiBoxi[0];
                double ky = kfac2 * ny * s->TwoPiBoxi[1];
                double kz = kfac2 * nz * s->TwoPiBoxi[2];
                for (int ia = 1; ia <= na; ++ia) {
                    zc *er = &s->eikr[(size_t)(ia - 1) * 4];
                    double facmm = -er[0].re * S[0].im + er[0].im * S[0].re;
                    double facmp = -er[1].re * S[1].im + er[1].im * S[1].re;
                    double facpm = -er[2].re * S[2].im + er[2].im * S[2].re;
                    double facpp = -er[3].re * S[3].im + er[3].im * S[3].re;
                    FORCE(1, ia) = FORCE(1, ia) + kx * (-facmm - facmp + facpm + facpp);
                    FORCE(2, ia) = FORCE(2, ia) + ky * (-facmm + facmp - facpm + facpp);
                    FORCE(3, ia) = FORCE(3, ia) + kz * (+facmm + facmp + facpm + facpp);
                }
                double k2 = pow2(nx * s->TwoPiBoxi[0]) + pow2(ny * s->TwoPiBoxi[1]) + pow2(nz * s->TwoPiBoxi[2]);
                *virrec = *virrec - (One - k2 / (Two * s->ualpha2)) * term;
            }
        }
    }
}

/* the influence function over the planes nz in [nz0, nz1) of the octant:
   energy and virial sums, then the spectrum times meshfac */
static void spm_influence_range(orc_sys *s, int nz0, int nz1, double *uloc, double *virloc) {
    int n = s->nmesh, nh = n / 2 + 1;
    zc *F = (zc *)s->FQmesh;
#define FQ(x, y, z) F[((size_t)(z) * n + (y)) * nh + (x)]
    for (int nz = nz0; nz < nz1; ++nz) {
        int nza = (n - nz) % n;
        for (int ny = 0; ny <= n / 2; ++ny) {
            int nya = (n - ny) % n;
            for (int nx = 0; nx <= n / 2; ++nx) {
                size_t id = ((size_t)nz * nh + ny) * nh + nx;
                zc v1 = FQ(nx, ny, nz), v2 = FQ(nx, ny, nza), v3 = FQ(nx, nya, nz), v4 = FQ(nx, nya, nza);
                double Qsum = v1.re * v1.re + v1.im * v1.im
                            + v2.re * v2.re + v2.im * v2.im
                            + v3.re * v3.re + v3.im * v3.im
                            + v4.re * v4.re + v4.im * v4.im;
                *uloc = *uloc + Qsum * s->energyfac[id];
                *virloc = *virloc - Qsum * s->virfac[id];
                double mf = s->meshfac[id];
                FQ(nx, ny, nz) = zscale(mf, v1);
                FQ(nx, ny, nza) = zscale(mf, v2);
                FQ(nx, nya, nz) = zscale(mf, v3);
                FQ(nx, nya, nza) = zscale(mf, v4);
            }
        }
    }
#undef FQ
}

typedef struct {
    orc_sys *s;
    double u[ORC_MAX_THREADS], v[ORC_MAX_THREADS];
} infl_job;

static void infl_job_run(void *ctx, int t, int nt) {
    infl_job *j = (infl_job *)ctx;
    long lo, hi;
    orc_range(j->s->nmesh / 2 + 1, t, nt, &lo, &hi);
    j->u[t] = Zero;
    j->v[t] = Zero;
    spm_influence_range(j->s, (int)lo, (int)hi, &j->u[t], &j->v[t]);
}

/* SPMFFTRec, energy.F90:6525-6587 */
static int spm_fft_rec(orc_sys *s, int lsave, double *uloc, double *virloc) {
    int n = s->nmesh;
    if (orc_fft_r2c_3d(n, s->Qmesh, s->FQmesh)) return MG_ERR_ALLOC;
    if (lsave) memcpy(s->QmeshTM, s->Qmesh, sizeof(double) * (size_t)n * n * n);
    *uloc = Zero;
    int nt = orc_threads();
    if (nt > n / 2 + 1) nt = n / 2 + 1;
    if (nt == 1) {
        spm_influence_range(s, 0, n / 2 + 1, uloc, virloc);
    } else {   /* partial sums per thread, combined in thread order */
        infl_job j;
        j.s = s;
        orc_par_run(infl_job_run, &j, nt);
        for (int t = 0; t < nt; ++t) {
            *uloc = *uloc + j.u[t];
            *virloc = *virloc + j.v[t];
        }
    }
    if (orc_fft_c2r_3d(n, s->FQmesh, s->Qmesh)) return MG_ERR_ALLOC;
    return 0;
}

#define SPL(arr, i, m, ia) (arr)[((size_t)((ia) - 1) * 3 + (m) - 1) * s->order + (i)]
#define MESHMAX(arr, m, ia) (arr)[(size_t)((ia) - 1) * 3 + (m) - 1]
#define QM(arr, x, y, z) (arr)[((size_t)(z) * s->s[1] + (y)) * s->s[0] + (x)]

/* splines of particles (lo, hi] (1-based) and their stamps added into Q */
static void spm_spread_range(orc_sys *s, long lo, long hi, double *Q) {
    int order = s->order, *S3 = s->s;
    for (int ia = (int)lo + 1; ia <= (int)hi; ++ia) {
        for (int m = 1; m <= 3; ++m) {
            int kmax;
            orc_cardinal_bspline(order, s->dkdr[m - 1] * RO(m, ia), &kmax, &SPL(s->spline, 0, m, ia), &SPL(s->deriv, 0, m, ia));
            MESHMAX(s->meshmax, m, ia) = (kmax + S3[m - 1]) % S3[m - 1];
        }
        for (int iz = 0; iz <= order - 1; ++iz) {
            int nz = (S3[2] + MESHMAX(s->meshmax, 3, ia) - iz) % S3[2];
            double qz = AZ(ia) * SPL(s->spline, iz, 3, ia);
            for (int iy = 0; iy <= order - 1; ++iy) {
                int ny = (S3[1] + MESHMAX(s->meshmax, 2, ia) - iy) % S3[1];
                double qyz = qz * SPL(s->spline, iy, 2, ia);
                for (int ix = 0; ix <= order - 1; ++ix) {
                    int nx = (S3[0] + MESHMAX(s->meshmax, 1, ia) - ix) % S3[0];
                    double q = qyz * SPL(s->spline, ix, 1, ia);
                    QM(Q, nx, ny, nz) = QM(Q, nx, ny, nz) + q;
                }
            }
        }
    }
}

/* the mesh forces of particles (lo, hi] (1-based) */
static void spm_gather_range(orc_sys *s, long lo, long hi) {
    int order = s->order, *S3 = s->s;
    for (int ia = (int)lo + 1; ia <= (int)hi; ++ia) {
        double esum[3] = {Zero, Zero, Zero};
        for (int iz = 0; iz <= order - 1; ++iz) {
            int nz = (S3[2] + MESHMAX(s->meshmax, 3, ia) - iz) % S3[2];
            double splz = SPL(s->spline, iz, 3, ia), dsdz = SPL(s->deriv, iz, 3, ia);
            for (int iy = 0; iy <= order - 1; ++iy) {
                int ny = (S3[1] + MESHMAX(s->meshmax, 2, ia) - iy) % S3[1];
                double sply = SPL(s->spline, iy, 2, ia), dsdy = SPL(s->deriv, iy, 2, ia);
                for (int ix = 0; ix <= order - 1; ++ix) {
                    int nx = (S3[0] + MESHMAX(s->meshmax, 1, ia) - ix) % S3[0];
                    double splx = SPL(s->spline, ix, 1, ia), dsdx = SPL(s->deriv, ix, 1, ia);
                    double Qval = QM(s->Qmesh, nx, ny, nz);
                    esum[0] = esum[0] + dsdx * sply * splz * Qval;
                    esum[1] = esum[1] + splx * dsdy * splz * Qval;
                    esum[2] = esum[2] + splx * sply * dsdz * Qval;
                }
            }
        }
        for (int m = 1; m <= 3; ++m)
            FORCE(m, ia) = FORCE(m, ia) - AZ(ia) * esum[m - 1] * s->dkdr[m - 1] * s->EpsiFourPi;
    }
}

typedef struct {
    orc_sys *s;
    double *Qt;   /* nt private meshes */
    size_t n3;
    int nt;
} spread_job;

static void spread_job_run(void *ctx, int t, int nt) {
    spread_job *j = (spread_job *)ctx;
    long lo, hi;
    orc_range(j->s->np, t, nt, &lo, &hi);
    memset(j->Qt + (size_t)t * j->n3, 0, sizeof(double) * j->n3);
    spm_spread_range(j->s, lo, hi, j->Qt + (size_t)t * j->n3);
}

static void mesh_sum_run(void *ctx, int t, int nt) {   /* Q = sum of the private meshes, thread order */
    spread_job *j = (spread_job *)ctx;
    long lo, hi;
    orc_range((long)j->n3, t, nt, &lo, &hi);
    for (long i = lo; i < hi; ++i) {
        double q = j->Qt[i];
        for (int k = 1; k < j->nt; ++k) q = q + j->Qt[(size_t)k * j->n3 + i];
        j->s->Qmesh[i] = q;
    }
}

static void gather_job_run(void *ctx, int t, int nt) {
    spread_job *j = (spread_job *)ctx;
    long lo, hi;
    orc_range(j->s->np, t, nt, &lo, &hi);
    spm_gather_range(j->s, lo, hi);
}

/* UEwaldRecSPM, energy.F90:1207-1297 */
static int uewald_rec_spm(orc_sys *s, double *virrec) {
    int *S3 = s->s;
    size_t n3 = (size_t)S3[0] * S3[1] * S3[2];
    int nt = orc_threads();
    spread_job j = {s, NULL, n3, nt};
    if (nt == 1) {
        memset(s->Qmesh, 0, sizeof(double) * n3);
        spm_spread_range(s, 0, s->np, s->Qmesh);
    } else {
        if (thr_arrays(s, nt)) return MG_ERR_ALLOC;
        j.Qt = s->thr_mesh;
        orc_par_run(spread_job_run, &j, nt);
        orc_par_run(mesh_sum_run, &j, nt);
    }
    memcpy(s->Qspread, s->Qmesh, sizeof(double) * n3);
    double urec;
    int st = spm_fft_rec(s, s->mode == MG_MC, &urec, virrec);
    if (st) return st;
    s->u_rec = urec;
    orc_par_run(gather_job_run, &j, nt);   /* each thread its own particles */
    if (s->mode == MG_MC) {
        memcpy(s->Qmesh, s->QmeshTM, sizeof(double) * n3);
        s->urecold = s->u_rec;
    }
    return 0;
}

/* UEwaldSelf, energy.F90:1301-1345 (atomic contribution; monoatomic) */
static void uewald_self(orc_sys *s) {
    double fac = s->ualpha / sqrt(Pi), t = Zero;
    for (int ia = 1; ia <= s->np; ++ia) t = t + AZ(ia) * AZ(ia);
    s->u_rec = s->u_rec - fac * t;
}

/* UEwaldSurf, energy.F90:1349-1371 (3d-periodic) */
static void uewald_surf(orc_sys *s, double *virrec) {
    double fac = TwoPi / (Three * s->vol);
    double sx = Zero, sy = Zero, sz = Zero;
    for (int ia = 1; ia <= s->np; ++ia) sx = sx + AZ(ia) * RO(1, ia);
    for (int ia = 1; ia <= s->np; ++ia) sy = sy + AZ(ia) * RO(2, ia);
    for (int ia = 1; ia <= s->np; ++ia) sz = sz + AZ(ia) * RO(3, ia);
    double term = fac * (sx * sx + sy * sy + sz * sz);
    s->u_rec = s->u_rec + term;
    for (int ia = 1; ia <= s->np; ++ia) {
        FORCE(1, ia) = FORCE(1, ia) - s->EpsiFourPi * (Two * fac) * AZ(ia) * sx;
        FORCE(2, ia) = FORCE(2, ia) - s->EpsiFourPi * (Two * fac) * AZ(ia) * sy;
        FORCE(3, ia) = FORCE(3, ia) - s->EpsiFourPi * (Two * fac) * AZ(ia) * sz;
    }
    *virrec = *virrec - term;
}

static void cardinal_bspline2(int order, double pos, int *kmax, double *values, double *derivs, double *derivs2);
static void dipole_ewald_facs(double ualpha, double *f1, double *f2, double *f3, double *s1, double *s2);

/* UDipoleEwaldRecStd (energy.F90:1830-2040, serial branch :1960-2036):
   structure factors of charges and dipoles, sumeikr with (q + i k.dip) and
   sumeikrd with i k.dip, in the four sign combinations; then per atom the
   potential, field and field gradient of every k-vector, and the virial */
static void dipole_rec_std(orc_sys *s, const double *dip, double *potstat, double *estat, double *efg,
                           double *virelec) {
    int na = s->np, kn = 0;
    ewald_set_array(s, 1, na);
    zc *Sd = (zc *)xcalloc(4, sizeof(zc));
    zc *er = (zc *)xcalloc((size_t)na * 4, sizeof(zc));
    for (int nz = 0; nz <= s->ncut; ++nz) {
        double kz = s->TwoPiBoxi[2] * nz;
        for (int ny = 0; ny <= s->ncut; ++ny) {
            double ky = s->TwoPiBoxi[1] * ny;
            if (ny * ny + nz * nz > s->ncut2) continue;
            for (int ia = 1; ia <= na; ++ia) {
                s->eikyzm[ia - 1] = zmul(zconj(EIK(s->eiky, ia, ny)), EIK(s->eikz, ia, nz));
                s->eikyzp[ia - 1] = zmul(EIK(s->eiky, ia, ny), EIK(s->eikz, ia, nz));
            }
            for (int nx = 0; nx <= s->ncut; ++nx) {
                if (nx * nx + ny * ny + nz * nz > s->ncut2) continue;
                if (nx == 0 && ny == 0 && nz == 0) continue;
                kn = kn + 1;
                double kx = s->TwoPiBoxi[0] * nx;
                zc S[4];
                for (int c = 0; c < 4; ++c) { S[c].re = Zero; S[c].im = Zero; Sd[c].re = Zero; Sd[c].im = Zero; }
                for (int ia = 1; ia <= na; ++ia) {
                    zc ex = EIK(s->eikx, ia, nx);
                    zc *e = &er[(size_t)(ia - 1) * 4];
                    e[0] = zmul(zconj(ex), s->eikyzm[ia - 1]);
                    e[1] = zmul(zconj(ex), s->eikyzp[ia - 1]);
                    e[2] = zmul(ex, s->eikyzm[ia - 1]);
                    e[3] = zmul(ex, s->eikyzp[ia - 1]);
                    double tx = kx * dip[3 * (ia - 1)], ty = ky * dip[3 * (ia - 1) + 1], tz = kz * dip[3 * (ia - 1) + 2];
                    double fac[4] = {-tx - ty + tz, -tx + ty + tz, +tx - ty + tz, +tx + ty + tz};
                    for (int c = 0; c < 4; ++c) {
                        zc g = {AZ(ia), fac[c]}, h = {Zero, fac[c]};
                        S[c] = zadd(S[c], zmul(g, e[c]));
                        Sd[c] = zadd(Sd[c], zmul(h, e[c]));
                    }
                }
                double kfac2 = Two * s->kfac[kn - 1];
                double kxkx = kfac2 * kx * kx, kyky = kfac2 * ky * ky, kzkz = kfac2 * kz * kz;
                double kxky = kfac2 * kx * ky, kxkz = kfac2 * kx * kz, kykz = kfac2 * ky * kz;
                for (int ia = 1; ia <= na; ++ia) {
                    zc *e = &er[(size_t)(ia - 1) * 4];
                    zc cmm = zmul(e[0], zconj(S[0])), cmp = zmul(e[1], zconj(S[1]));
                    zc cpm = zmul(e[2], zconj(S[2])), cpp = zmul(e[3], zconj(S[3]));
                    double *ei = &estat[3 * (ia - 1)], *gi = &efg[6 * (ia - 1)];
                    potstat[ia - 1] = potstat[ia - 1] + kfac2 * (+cmm.re + cmp.re + cpm.re + cpp.re);
                    ei[0] = ei[0] + kfac2 * kx * (-cmm.im - cmp.im + cpm.im + cpp.im);
                    ei[1] = ei[1] + kfac2 * ky * (-cmm.im + cmp.im - cpm.im + cpp.im);
                    ei[2] = ei[2] + kfac2 * kz * (+cmm.im + cmp.im + cpm.im + cpp.im);
                    gi[0] = gi[0] + kxkx * (+cmm.re + cmp.re + cpm.re + cpp.re);
                    gi[1] = gi[1] + kyky * (+cmm.re + cmp.re + cpm.re + cpp.re);
                    gi[2] = gi[2] + kzkz * (+cmm.re + cmp.re + cpm.re + cpp.re);
                    gi[3] = gi[3] + kxky * (+cmm.re - cmp.re - cpm.re + cpp.re);
                    gi[4] = gi[4] + kxkz * (-cmm.re - cmp.re + cpm.re + cpp.re);
                    gi[5] = gi[5] + kykz * (-cmm.re + cmp.re - cpm.re + cpp.re);
                }
                double termx = Zero, termy = Zero;
                for (int c = 0; c < 4; ++c) termx = termx + (Sd[c].re * S[c].re + Sd[c].im * S[c].im);
                for (int c = 0; c < 4; ++c) termy = termy + (S[c].re * S[c].re + S[c].im * S[c].im);
                double termz = One - (kx * kx + ky * ky + kz * kz) / (Two * s->ualpha2);
                *virelec = *virelec - s->kfac[kn - 1] * (Two * termx + termy * termz);
            }
        }
    }
    free(Sd);
    free(er);
}

/* UDipoleEwaldRecSPM (energy.F90:2046-2170): the generalized charge mesh
   (charges and the dipoles through the B-spline derivatives), SPMFFTRec,
   then per atom the potential, field and field gradient (second
   derivatives of the B-splines) and the virial's dipole term */
static int dipole_rec_spm(orc_sys *s, const double *dip, double *potstat, double *estat, double *efg,
                          double *virelec) {
    int order = s->order, *S3 = s->s, na = s->np;
    size_t n3 = (size_t)S3[0] * S3[1] * S3[2];
    double *spl = (double *)xcalloc((size_t)na * 3 * order, sizeof(double));
    double *der = (double *)xcalloc((size_t)na * 3 * order, sizeof(double));
    double *der2 = (double *)xcalloc((size_t)na * 3 * order, sizeof(double));
    int *mm = (int *)xcalloc((size_t)na * 3, sizeof(int));
    if (!spl || !der || !der2 || !mm) { free(spl); free(der); free(der2); free(mm); return MG_ERR_ALLOC; }
#define SP(a, i, m, ia) (a)[((size_t)(ia) * 3 + (m)) * order + (i)]
    memset(s->Qmesh, 0, sizeof(double) * n3);
    for (int ia = 0; ia < na; ++ia) {
        double dipx2 = dip[3 * ia] * s->dkdr[0], dipy2 = dip[3 * ia + 1] * s->dkdr[1], dipz2 = dip[3 * ia + 2] * s->dkdr[2];
        for (int m = 0; m < 3; ++m) {
            int kmax;
            cardinal_bspline2(order, s->dkdr[m] * s->ro[3 * ia + m], &kmax, &SP(spl, 0, m, ia), &SP(der, 0, m, ia),
                              &SP(der2, 0, m, ia));
            mm[3 * ia + m] = (kmax + S3[m]) % S3[m];
        }
        for (int iz = 0; iz <= order - 1; ++iz) {
            int nz = (S3[2] + mm[3 * ia + 2] - iz) % S3[2];
            double splz = SP(spl, iz, 2, ia), dsdz = SP(der, iz, 2, ia);
            for (int iy = 0; iy <= order - 1; ++iy) {
                int ny = (S3[1] + mm[3 * ia + 1] - iy) % S3[1];
                double sply = SP(spl, iy, 1, ia);
                double q1 = s->az[ia] * sply * splz;
                double dipx1 = dipx2 * sply * splz;
                double dipy1 = dipy2 * SP(der, iy, 1, ia) * splz;
                double dipz1 = dipz2 * sply * dsdz;
                for (int ix = 0; ix <= order - 1; ++ix) {
                    int nx = (S3[0] + mm[3 * ia] - ix) % S3[0];
                    double splx = SP(spl, ix, 0, ia);
                    double q = q1 * splx, dx = dipx1 * SP(der, ix, 0, ia), dy = dipy1 * splx, dz = dipz1 * splx;
                    QM(s->Qmesh, nx, ny, nz) = QM(s->Qmesh, nx, ny, nz) + (q + dx + dy + dz);
                }
            }
        }
    }
    double uloc;
    int st = spm_fft_rec(s, 0, &uloc, virelec);
    if (st) { free(spl); free(der); free(der2); free(mm); return st; }
    const double *dk = s->dkdr;
    double d2k[6] = {dk[0] * dk[0], dk[1] * dk[1], dk[2] * dk[2], dk[0] * dk[1], dk[0] * dk[2], dk[1] * dk[2]};
    for (int ia = 0; ia < na; ++ia) {
        double dipx2 = dip[3 * ia] * dk[0], dipy2 = dip[3 * ia + 1] * dk[1], dipz2 = dip[3 * ia + 2] * dk[2];
        double psum = Zero, es[3] = {Zero, Zero, Zero}, gs[6] = {Zero, Zero, Zero, Zero, Zero, Zero};
        for (int iz = 0; iz <= order - 1; ++iz) {
            int nz = (S3[2] + mm[3 * ia + 2] - iz) % S3[2];
            double splz = SP(spl, iz, 2, ia), dsdz = SP(der, iz, 2, ia), d2sdz = SP(der2, iz, 2, ia);
            for (int iy = 0; iy <= order - 1; ++iy) {
                int ny = (S3[1] + mm[3 * ia + 1] - iy) % S3[1];
                double sply = SP(spl, iy, 1, ia), dsdy = SP(der, iy, 1, ia), d2sdy = SP(der2, iy, 1, ia);
                for (int ix = 0; ix <= order - 1; ++ix) {
                    int nx = (S3[0] + mm[3 * ia] - ix) % S3[0];
                    double splx = SP(spl, ix, 0, ia), dsdx = SP(der, ix, 0, ia), d2sdx = SP(der2, ix, 0, ia);
                    double Qval = QM(s->Qmesh, nx, ny, nz);
                    psum = psum + splx * sply * splz * Qval;
                    es[0] = es[0] + dsdx * sply * splz * Qval;
                    es[1] = es[1] + splx * dsdy * splz * Qval;
                    es[2] = es[2] + splx * sply * dsdz * Qval;
                    gs[0] = gs[0] + d2sdx * sply * splz * Qval;
                    gs[1] = gs[1] + splx * d2sdy * splz * Qval;
                    gs[2] = gs[2] + splx * sply * d2sdz * Qval;
                    gs[3] = gs[3] + dsdx * dsdy * splz * Qval;
                    gs[4] = gs[4] + dsdx * sply * dsdz * Qval;
                    gs[5] = gs[5] + splx * dsdy * dsdz * Qval;
                    double Qdip = dipx2 * dsdx * sply * splz + dipy2 * splx * dsdy * splz + dipz2 * splx * sply * dsdz;
                    *virelec = *virelec - Qdip * Qval;
                }
            }
        }
        potstat[ia] = potstat[ia] + psum;
        for (int m = 0; m < 3; ++m) estat[3 * ia + m] = estat[3 * ia + m] - es[m] * dk[m];
        for (int m = 0; m < 6; ++m) efg[6 * ia + m] = efg[6 * ia + m] - gs[m] * d2k[m];
    }
#undef SP
    free(spl); free(der); free(der2); free(mm);
    return 0;
}

/* UDipoleEwald's reciprocal part and the atomic part of UDipoleEwaldSelf
   (energy.F90:1807-1830, 2183-2191) on a handle whose particles are the
   atoms (positions, charges az): adds to potstat, estat, efg and virelec.
   Leaves the handle's mesh and structure factors as scratch. */
int orc_dipole_ewald(orc_sys *s, const double *dip, double *potstat, double *estat, double *efg, double *virelec) {
    if (s->ewald == MG_EWALD_STD) dipole_rec_std(s, dip, potstat, estat, efg, virelec);
    else if (s->ewald == MG_EWALD_SPM) {
        int st = dipole_rec_spm(s, dip, potstat, estat, efg, virelec);
        if (st) return st;
    } else return MG_ERR_STATE;
    double f1, f2, f3, s1, s2;
    dipole_ewald_facs(s->ualpha, &f1, &f2, &f3, &s1, &s2);
    for (int ia = 0; ia < s->np; ++ia) potstat[ia] = potstat[ia] - s1 * s->az[ia];
    for (int ia = 0; ia < s->np; ++ia)
        for (int m = 0; m < 3; ++m) estat[3 * ia + m] = estat[3 * ia + m] + s2 * dip[3 * ia + m];
    for (int ia = 0; ia < s->np; ++ia)
        for (int m = 0; m < 3; ++m) efg[6 * ia + m] = efg[6 * ia + m] - s2 * s->az[ia];
    return 0;
}

/* UEwald, energy.F90:905-960 */
static int uewald(orc_sys *s) {
    double virrec = Zero;
    s->u_rec = Zero;
    if (s->ewald == MG_EWALD_STD) uewald_rec_std(s, &virrec);
    else {
        int st = uewald_rec_spm(s, &virrec);
        if (st) return st;
    }
    uewald_self(s);
    if (s->lsurf) uewald_surf(s, &virrec);
    s->u_rec = s->EpsiFourPi * s->u_rec;
    s->u_tot = s->u_tot + s->u_rec;
    s->virial = s->virial + s->EpsiFourPi * virrec;
    s->have_rec = 1;
    return 0;
}

/* UBond, energy.F90:5335-5386 (the bonds in chain order) */
static void ubond(orc_sys *s) {
    double virbond = Zero;
    s->u_bond = Zero;
    for (int b = 0; b < s->nbond; ++b) {
        int ip = s->bond_ip[b], jp = s->bond_jp[b];
        double dx = RO(1, ip) - RO(1, jp), dy = RO(2, ip) - RO(2, jp), dz = RO(3, ip) - RO(3, jp), r2;
        pbcr2(s, &dx, &dy, &dz, &r2);
        double r1 = sqrt(r2);
        double term = r1 - s->bond_eq[b];
        double fac = s->bond_k[b] * powi(term, s->bond_p[b] - 1);
        s->u_bond = s->u_bond + fac * term;
        fac = -s->bond_p[b] * fac / r1;
        FORCE(1, ip) = FORCE(1, ip) + (fac * dx);
        FORCE(2, ip) = FORCE(2, ip) + (fac * dy);
        FORCE(3, ip) = FORCE(3, ip) + (fac * dz);
        FORCE(1, jp) = FORCE(1, jp) - (fac * dx);
        FORCE(2, jp) = FORCE(2, jp) - (fac * dy);
        FORCE(3, jp) = FORCE(3, jp) - (fac * dz);
        virbond = virbond - (fac * r2);
    }
    s->u_tot = s->u_tot + s->u_bond;
    s->virial = s->virial + virbond;
}

/* UAngle, energy.F90:5409-5506: u = k*(theta - eq)**p at each interior
   segment, theta the angle at ip between ip-jm and ip-jp; forces on jm, jp
   and ip; no contribution to the virial.  The reference carries the unit
   vector of the previous segment into the next angle (dxm = -dxp); the
   angles here are listed in its order and the vector recomputed, which
   gives the same bits (PBC and the norm are symmetric in the sign). */
static void uangle(orc_sys *s) {
    s->u_angle = Zero;
    int any = 0;
    for (int a = 0; a < s->nangle; ++a) any |= s->angle_k[a] != Zero;
    if (!any) return;
    for (int a = 0; a < s->nangle; ++a) {
        int jm = s->angle_jm[a], ip = s->angle_ip[a], jp = s->angle_jp[a];
        double dxm = RO(1, ip) - RO(1, jm), dym = RO(2, ip) - RO(2, jm), dzm = RO(3, ip) - RO(3, jm);
        pbc(s, &dxm, &dym, &dzm);
        double dmi = One / sqrt(pow2(dxm) + pow2(dym) + pow2(dzm));
        dxm = dxm * dmi;
        dym = dym * dmi;
        dzm = dzm * dmi;
        double dxp = RO(1, ip) - RO(1, jp), dyp = RO(2, ip) - RO(2, jp), dzp = RO(3, ip) - RO(3, jp);
        pbc(s, &dxp, &dyp, &dzp);
        double dpi = One / sqrt(pow2(dxp) + pow2(dyp) + pow2(dzp));
        dxp = dxp * dpi;
        dyp = dyp * dpi;
        dzp = dzp * dpi;
        double cosine = dxm * dxp + dym * dyp + dzm * dzp;
        double theta = acos(fmax(-One, fmin(cosine, One)));
        double term = theta - s->angle_eq[a];
        double fac = s->angle_k[a] * powi(term, s->angle_p[a] - 1);
        s->u_angle = s->u_angle + fac * term;
        fac = -s->angle_p[a] * fac / sin(theta);
        double fxm = (fac * dmi) * (dxp - cosine * dxm);
        double fym = (fac * dmi) * (dyp - cosine * dym);
        double fzm = (fac * dmi) * (dzp - cosine * dzm);
        double fxp = (fac * dpi) * (dxm - cosine * dxp);
        double fyp = (fac * dpi) * (dym - cosine * dyp);
        double fzp = (fac * dpi) * (dzm - cosine * dzp);
        FORCE(1, jm) = FORCE(1, jm) + fxm;
        FORCE(2, jm) = FORCE(2, jm) + fym;
        FORCE(3, jm) = FORCE(3, jm) + fzm;
        FORCE(1, jp) = FORCE(1, jp) + fxp;
        FORCE(2, jp) = FORCE(2, jp) + fyp;
        FORCE(3, jp) = FORCE(3, jp) + fzp;
        FORCE(1, ip) = FORCE(1, ip) - (fxm + fxp);
        FORCE(2, ip) = FORCE(2, ip) - (fym + fyp);
        FORCE(3, ip) = FORCE(3, ip) - (fzm + fzp);
    }
    s->u_tot = s->u_tot + s->u_angle;
}

/* UTwoBodyP, energy.F90:786-896: particles iploc in order, their list
   neighbours (in MC only jp > ip), the centre separation folded by PBC2
   (molaux.F90:193-248) and that shift applied to every atom pair; the
   table search of UTwoBodyA per atom-type pair; u%twob(0) the sum of the
   type-pair energies.  Atom forces are not scaled (force(3,na)). */
int orc_poly_utwobody(const mg_poly_params *p, int32_t maxnneigh, const double *ro, const double *r,
                      const int32_t *nneighpn, const int32_t *jpnlist, double *force, double *u_twob,
                      double *virial) {
    int npt = p->npt, nat = p->nat, nptpt = p->nptpt;
    double half[3], rcut2 = p->rcut * p->rcut, virtwob = Zero;
    for (int m = 0; m < 3; ++m) half[m] = p->boxlen[m] / Two;
    for (int k = 0; k <= nptpt; ++k) u_twob[k] = Zero;
    for (int k = 0; k < 3 * p->na; ++k) force[k] = Zero;
    for (int ip = 1; ip <= p->np; ++ip) {
        int ipt = p->iptpn[ip - 1];
        int ialow = p->ianpn[ip - 1], iaupp = ialow + p->napt[ipt - 1] - 1;
        for (int jploc = 1; jploc <= nneighpn[ip - 1]; ++jploc) {
            int jp = jpnlist[(size_t)(ip - 1) * maxnneigh + jploc - 1];
            if (p->lmc && jp < ip) continue;
            int jpt = p->iptpn[jp - 1];
            int iptjpt = p->iptpt[(jpt - 1) * npt + ipt - 1];
            double d[3], sh[3];
            for (int m = 0; m < 3; ++m) {
                d[m] = ro[3 * (ip - 1) + m] - ro[3 * (jp - 1) + m];
                sh[m] = Zero;
                if (fabs(d[m]) > half[m]) sh[m] = fsign(p->boxlen[m], d[m]);
                d[m] = d[m] - sh[m];
            }
            double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (r2 > rcut2) continue;
            double usum = Zero;
            int jalow = p->ianpn[jp - 1], jaupp = jalow + p->napt[jpt - 1] - 1;
            for (int ia = ialow; ia <= iaupp; ++ia) {
                int iat = p->iatan[ia - 1];
                for (int ja = jalow; ja <= jaupp; ++ja) {
                    int jat = p->iatan[ja - 1];
                    int iatjat = p->iatat[(jat - 1) * nat + iat - 1];
                    double dx = r[3 * (ia - 1)] - r[3 * (ja - 1)] - sh[0];
                    double dy = r[3 * (ia - 1) + 1] - r[3 * (ja - 1) + 1] - sh[1];
                    double dz = r[3 * (ia - 1) + 2] - r[3 * (ja - 1) + 2] - sh[2];
                    double ar2 = dx * dx + dy * dy + dz * dz;
                    if (ar2 < p->r2umin[iatjat - 1]) return MG_ERR_TABLE_UNDERRUN;
                    int ibuf = p->iubuflow[iatjat - 1];
                    for (;;) {
                        if (ar2 >= p->ubuf[ibuf - 1]) break;
                        ibuf = ibuf + 12;
                        if (ibuf > p->nbuf) return MG_ERR_IBUF;
                    }
                    const double *u = &p->ubuf[ibuf - 1];
                    double dd = ar2 - u[0];
                    usum = usum + u[1] + dd * (u[2] + dd * (u[3] + dd * (u[4] + dd * (u[5] + dd * u[6]))));
                    double fsum = u[7] + dd * (u[8] + dd * (u[9] + dd * (u[10] + dd * u[11])));
                    force[3 * (ia - 1)] = force[3 * (ia - 1)] + (fsum * dx);
                    force[3 * (ia - 1) + 1] = force[3 * (ia - 1) + 1] + (fsum * dy);
                    force[3 * (ia - 1) + 2] = force[3 * (ia - 1) + 2] + (fsum * dz);
                    force[3 * (ja - 1)] = force[3 * (ja - 1)] - (fsum * dx);
                    force[3 * (ja - 1) + 1] = force[3 * (ja - 1) + 1] - (fsum * dy);
                    force[3 * (ja - 1) + 2] = force[3 * (ja - 1) + 2] - (fsum * dz);
                    virtwob = virtwob - (fsum * ar2);
                }
            }
            u_twob[iptjpt] = u_twob[iptjpt] + usum;
        }
    }
    double s = Zero;
    for (int k = 1; k <= nptpt; ++k) s = s + u_twob[k];
    u_twob[0] = s;
    *virial = virtwob;
    return 0;
}

/* the atom-pair sum of one particle pair for UTwoBodyPNew/Old: centre ci
   and atoms ra (napt of ip's type) against particle jp; returns 1 on a
   hard-core or table underrun (only checked with lnew), -1 past the table */
static int poly_pair_sum(const mg_poly_params *p, int ipt, int ialow, const double *ci, const double *ra,
                         const double *ro, const double *r, int jp, int lnew, double *usum_out, int *inrange) {
    double d[3], sh[3];
    *inrange = 0;
    for (int m = 0; m < 3; ++m) {
        d[m] = ci[m] - ro[3 * (jp - 1) + m];
        sh[m] = Zero;
        if (fabs(d[m]) > p->boxlen[m] / Two) sh[m] = fsign(p->boxlen[m], d[m]);
        d[m] = d[m] - sh[m];
    }
    double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    if (r2 > p->rcut * p->rcut) return 0;
    *inrange = 1;
    int jpt = p->iptpn[jp - 1];
    int jalow = p->ianpn[jp - 1], jaupp = jalow + p->napt[jpt - 1] - 1;
    double usum = Zero;
    for (int k = 0; k < p->napt[ipt - 1]; ++k) {
        int iat = p->iatan[ialow - 1 + k];
        for (int ja = jalow; ja <= jaupp; ++ja) {
            int jat = p->iatan[ja - 1];
            int iatjat = p->iatat[(jat - 1) * p->nat + iat - 1];
            double dx = ra[3 * k] - r[3 * (ja - 1)] - sh[0];
            double dy = ra[3 * k + 1] - r[3 * (ja - 1) + 1] - sh[1];
            double dz = ra[3 * k + 2] - r[3 * (ja - 1) + 2] - sh[2];
            double ar2 = dx * dx + dy * dy + dz * dz;
            if (lnew && ar2 < p->r2atat[iatjat - 1]) return 1;
            if (ar2 < p->r2umin[iatjat - 1]) return 1;
            int ibuf = p->iubuflow[iatjat - 1];
            for (;;) {
                if (ar2 >= p->ubuf[ibuf - 1]) break;
                ibuf = ibuf + 12;
                if (ibuf > p->nbuf) return -1;
            }
            const double *u = &p->ubuf[ibuf - 1];
            double dd = ar2 - u[0];
            usum = usum + u[1] + dd * (u[2] + dd * (u[3] + dd * (u[4] + dd * (u[5] + dd * u[6]))));
        }
    }
    *usum_out = usum;
    return 0;
}

int orc_poly_dutwobody(const mg_poly_params *p, int32_t maxnneigh, const double *ro, const double *r,
                       const int32_t *nneighpn, const int32_t *jpnlist, int32_t ip, const double *rotm,
                       const double *rtm, double *du_twob, int32_t *lhsoverlap) {
    int nptpt = p->nptpt, ipt = p->iptpn[ip - 1], ialow = p->ianpn[ip - 1];
    double unew[64], uold[64];   /* nptpt + 1 entries */
    if (nptpt + 1 > 64) return MG_ERR_ARG;
    for (int k = 0; k <= nptpt; ++k) unew[k] = uold[k] = du_twob[k] = Zero;
    *lhsoverlap = 1;
    for (int pass = 0; pass < 2; ++pass) {   /* UTwoBodyPNew, then UTwoBodyPOld */
        const double *ci = pass ? &ro[3 * (ip - 1)] : rotm;
        const double *ra = pass ? &r[3 * (ialow - 1)] : rtm;
        double *acc = pass ? uold : unew;
        for (int jploc = 1; jploc <= nneighpn[ip - 1]; ++jploc) {
            int jp = jpnlist[(size_t)(ip - 1) * maxnneigh + jploc - 1];
            if (jp == ip) continue;   /* lptm(jp) */
            double usum;
            int inr, st = poly_pair_sum(p, ipt, ialow, ci, ra, ro, r, jp, pass == 0, &usum, &inr);
            if (st < 0) return MG_ERR_IBUF;
            if (st > 0) {
                if (pass == 0) return 0;          /* hard-core overlap: the trial is rejected */
                return MG_ERR_TABLE_UNDERRUN;
            }
            if (!inr) continue;
            int iptjpt = p->iptpt[(p->iptpn[jp - 1] - 1) * p->npt + ipt - 1];
            acc[iptjpt] = acc[iptjpt] + usum;
        }
    }
    *lhsoverlap = 0;
    double s = Zero;
    for (int k = 1; k <= nptpt; ++k) {
        du_twob[k] = unew[k] - uold[k];
        s = s + du_twob[k];
    }
    du_twob[0] = s;
    return 0;
}

/* the atom-pair energy of two particles: centres ci, cj, atoms ra (of ip's
   type, first atom ialow) and rb (of jp's type, first atom jalow); returns
   1 on a hard core or a pair below its table, -1 past the table, and sets
   *inr when the centres are within rcut */
static int poly_pair_sum2(const mg_poly_params *p, int ipt, int ialow, const double *ci, const double *ra,
                          int jpt, int jalow, const double *cj, const double *rb, double *usum_out, int *inr) {
    double d[3], sh[3];
    *inr = 0;
    for (int m = 0; m < 3; ++m) {
        d[m] = ci[m] - cj[m];
        sh[m] = Zero;
        if (fabs(d[m]) > p->boxlen[m] / Two) sh[m] = fsign(p->boxlen[m], d[m]);
        d[m] = d[m] - sh[m];
    }
    double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    if (r2 > p->rcut * p->rcut) return 0;
    *inr = 1;
    double usum = Zero;
    for (int k = 0; k < p->napt[ipt - 1]; ++k) {
        int iat = p->iatan[ialow - 1 + k];
        for (int l = 0; l < p->napt[jpt - 1]; ++l) {
            int jat = p->iatan[jalow - 1 + l];
            int iatjat = p->iatat[(jat - 1) * p->nat + iat - 1];
            double dx = ra[3 * k] - rb[3 * l] - sh[0];
            double dy = ra[3 * k + 1] - rb[3 * l + 1] - sh[1];
            double dz = ra[3 * k + 2] - rb[3 * l + 2] - sh[2];
            double ar2 = dx * dx + dy * dy + dz * dz;
            if (ar2 < p->r2atat[iatjat - 1]) return 1;
            if (ar2 < p->r2umin[iatjat - 1]) return 1;
            int ibuf = p->iubuflow[iatjat - 1];
            for (;;) {
                if (ar2 >= p->ubuf[ibuf - 1]) break;
                ibuf = ibuf + 12;
                if (ibuf > p->nbuf) return -1;
            }
            const double *u = &p->ubuf[ibuf - 1];
            double dd = ar2 - u[0];
            usum = usum + u[1] + dd * (u[2] + dd * (u[3] + dd * (u[4] + dd * (u[5] + dd * u[6]))));
        }
    }
    *usum_out = usum;
    return 0;
}

/* UTwoBodyPNew and UTwoBodyPOld (denergy.F90:937-1231) for nptm moving
   particles ipnptm (1-based) with new centres rotm(3,nptm) and new atoms
   rtm (the moving particles' atoms one after another): each moving
   particle with its list neighbours that do not move, then (lptmdutwob)
   every pair of moving particles once, in the order the reference loops.
   du_twob[nptpt+1] = new - old; *lhsoverlap = 1 on a hard core (or a pair
   below its table) in the new configuration */
int orc_poly_dutwobody_multi(const mg_poly_params *p, int32_t maxnneigh, const double *ro, const double *r,
                             const int32_t *nneighpn, const int32_t *jpnlist, int32_t nptm, const int32_t *ipnptm,
                             const double *rotm, const double *rtm, double *du_twob, int32_t *lhsoverlap) {
    int nptpt = p->nptpt;
    double acc[2][64];
    if (nptpt + 1 > 64 || nptm < 1) return MG_ERR_ARG;
    char *lptm = (char *)calloc((size_t)p->np + 1, 1);
    int *atom0 = (int *)malloc(sizeof(int) * (size_t)nptm);
    if (!lptm || !atom0) { free(lptm); free(atom0); return MG_ERR_ALLOC; }
    int tot = 0;
    for (int k = 0; k < nptm; ++k) {
        lptm[ipnptm[k]] = 1;
        atom0[k] = tot;
        tot += p->napt[p->iptpn[ipnptm[k] - 1] - 1];
    }
    for (int k = 0; k <= nptpt; ++k) acc[0][k] = acc[1][k] = du_twob[k] = Zero;
    *lhsoverlap = 1;
    int st = 0;
    for (int pass = 0; pass < 2 && st == 0; ++pass) {   /* new, then old */
        double *a = acc[pass];
        for (int il = 0; il < nptm && st == 0; ++il) {
            int ip = ipnptm[il], ipt = p->iptpn[ip - 1], ialow = p->ianpn[ip - 1];
            const double *ci = pass ? &ro[3 * (ip - 1)] : &rotm[3 * il];
            const double *ra = pass ? &r[3 * (ialow - 1)] : &rtm[3 * atom0[il]];
            for (int jploc = 1; jploc <= nneighpn[ip - 1]; ++jploc) {
                int jp = jpnlist[(size_t)(ip - 1) * maxnneigh + jploc - 1];
                if (lptm[jp]) continue;
                int jpt = p->iptpn[jp - 1], jalow = p->ianpn[jp - 1];
                double usum;
                int inr, q = poly_pair_sum2(p, ipt, ialow, ci, ra, jpt, jalow, &ro[3 * (jp - 1)],
                                            &r[3 * (jalow - 1)], &usum, &inr);
                if (q < 0) { st = MG_ERR_IBUF; break; }
                if (q > 0) { st = pass == 0 ? 1 : MG_ERR_TABLE_UNDERRUN; break; }
                if (!inr) continue;
                int iptjpt = p->iptpt[(jpt - 1) * p->npt + ipt - 1];
                a[iptjpt] = a[iptjpt] + usum;
            }
        }
        for (int il = 0; il < nptm && st == 0; ++il) {   /* both displaced */
            int ip = ipnptm[il], ipt = p->iptpn[ip - 1], ialow = p->ianpn[ip - 1];
            const double *ci = pass ? &ro[3 * (ip - 1)] : &rotm[3 * il];
            const double *ra = pass ? &r[3 * (ialow - 1)] : &rtm[3 * atom0[il]];
            for (int jl = il + 1; jl < nptm; ++jl) {
                int jp = ipnptm[jl], jpt = p->iptpn[jp - 1], jalow = p->ianpn[jp - 1];
                const double *cj = pass ? &ro[3 * (jp - 1)] : &rotm[3 * jl];
                const double *rb = pass ? &r[3 * (jalow - 1)] : &rtm[3 * atom0[jl]];
                double usum;
                int inr, q = poly_pair_sum2(p, ipt, ialow, ci, ra, jpt, jalow, cj, rb, &usum, &inr);
                if (q < 0) { st = MG_ERR_IBUF; break; }
                if (q > 0) { st = pass == 0 ? 1 : MG_ERR_TABLE_UNDERRUN; break; }
                if (!inr) continue;
                int iptjpt = p->iptpt[(jpt - 1) * p->npt + ipt - 1];
                a[iptjpt] = a[iptjpt] + usum;
            }
        }
    }
    free(lptm);
    free(atom0);
    if (st == 1) return 0;   /* hard-core overlap in the new configuration: rejected */
    if (st) return st;
    *lhsoverlap = 0;
    double sum = Zero;
    for (int k = 1; k <= nptpt; ++k) {
        du_twob[k] = acc[0][k] - acc[1][k];
        sum = sum + du_twob[k];
    }
    du_twob[0] = sum;
    return 0;
}

/* UTotal, energy.F90:405-427: atoms in order, each adding to its particle
   (ipnan) the scaled force, the torque of the scaled force about the
   particle centre, and (r_a - ro_p) . f_a (unscaled) to virmolecule */
int orc_poly_epilogue(const mg_poly_params *p, const double *ro, const double *r, const double *force,
                      const double *torque, double force_fac, double *forceo, double *torqueo,
                      double *virmolecule) {
    double virmol = Zero;
    for (int k = 0; k < 3 * p->np; ++k) forceo[k] = torqueo[k] = Zero;
    for (int ip = 1; ip <= p->np; ++ip) {
        int ialow = p->ianpn[ip - 1], iaupp = ialow + p->napt[p->iptpn[ip - 1] - 1] - 1;
        for (int ia = ialow; ia <= iaupp; ++ia) {
            const double *fa = &force[3 * (ia - 1)];
            double dx = r[3 * (ia - 1)] - ro[3 * (ip - 1)];
            double dy = r[3 * (ia - 1) + 1] - ro[3 * (ip - 1) + 1];
            double dz = r[3 * (ia - 1) + 2] - ro[3 * (ip - 1) + 2];
            virmol = virmol + dx * fa[0] + dy * fa[1] + dz * fa[2];
            double gx = fa[0] * force_fac, gy = fa[1] * force_fac, gz = fa[2] * force_fac;
            double *fo = &forceo[3 * (ip - 1)], *to = &torqueo[3 * (ip - 1)];
            fo[0] = fo[0] + gx;
            fo[1] = fo[1] + gy;
            fo[2] = fo[2] + gz;
            to[0] = to[0] + (dy * gz - dz * gy);
            to[1] = to[1] + (dz * gx - dx * gz);
            to[2] = to[2] + (dx * gy - dy * gx);
            if (torque) {   /* + torque(m,ia)*fac, the atom torques of the dipole electrostatics */
                to[0] = to[0] + torque[3 * (ia - 1)] * force_fac;
                to[1] = to[1] + torque[3 * (ia - 1) + 1] * force_fac;
                to[2] = to[2] + torque[3 * (ia - 1) + 2] * force_fac;
            }
        }
    }
    *virmolecule = virmol;
    return 0;
}

/* UEwaldSelf, molecular contribution (energy.F90:1313-1341), with the
   constants of EwaldSetup (energy.F90:7040-7042) and ErfLocal = Erf2; the
   result scaled by EpsiFourPi as UEwald does at its end (energy.F90:950) */
int orc_poly_ewald_intra(const mg_poly_params *p, const double *r, double *force, double *u_rec) {
    double ualpha = p->ualpha, ualpha2 = ualpha * ualpha;
    double fac0 = One / (sqrt(Pi) * ualpha);
    double ewaldfac1 = fac0 * Two * ualpha2;
    double u = Zero;
    for (int k = 0; k < 3 * p->na; ++k) force[k] = Zero;
    for (int ip = 1; ip <= p->np; ++ip) {
        int ipt = p->iptpn[ip - 1];
        int ialow = p->ianpn[ip - 1], iaupp = p->ianpn[ip - 1] + p->napt[ipt - 1] - 1;
        for (int ia = ialow; ia <= iaupp; ++ia) {
            for (int ja = ia + 1; ja <= iaupp; ++ja) {
                double dx = r[3 * (ia - 1)] - r[3 * (ja - 1)];
                double dy = r[3 * (ia - 1) + 1] - r[3 * (ja - 1) + 1];
                double dz = r[3 * (ia - 1) + 2] - r[3 * (ja - 1) + 2];
                double r2 = dx * dx + dy * dy + dz * dz;
                double r1 = sqrt(r2);
                double r1i = One / r1;
                double r2i = r1i * r1i;
                double ex = exp(-ualpha2 * r2);
                r1i = r1i * orc_erf2(ualpha * r1);
                double r3i = r2i * (r1i - ewaldfac1 * ex);
                double qa = p->aza[ia - 1], qb = p->aza[ja - 1];
                u = u - (qa * qb * r1i);
                double fac = p->epsi_four_pi * qa * qb * r3i;
                force[3 * (ia - 1)] = force[3 * (ia - 1)] - (fac * dx);
                force[3 * (ia - 1) + 1] = force[3 * (ia - 1) + 1] - (fac * dy);
                force[3 * (ia - 1) + 2] = force[3 * (ia - 1) + 2] - (fac * dz);
                force[3 * (ja - 1)] = force[3 * (ja - 1)] + (fac * dx);
                force[3 * (ja - 1) + 1] = force[3 * (ja - 1) + 1] + (fac * dy);
                force[3 * (ja - 1) + 2] = force[3 * (ja - 1) + 2] + (fac * dz);
            }
        }
    }
    *u_rec = p->epsi_four_pi * u;
    return 0;
}

/* ---- electrostatics of charges and point dipoles (UDipole, energy.F90:1476-1579) ----
   potstat(na), estat(3,na), efg(6,na) (xx, yy, zz, xy, xz, yz) and virelec
   as the reference's module arrays; nothing is scaled by EpsiFourPi until
   the UDipole loop (orc_poly_udipole_finish). */

/* CardinalBSpline, mollib.F90:1629-1685, with the second derivatives: they
   come from the values of order-2, saved when the recursion reaches n =
   order-1 (zero for order 3 and below, as there) */
static void cardinal_bspline2(int order, double pos, int *kmax, double *values, double *derivs, double *derivs2) {
    double lastvals[64], lastvals2[64];
    int v = (int)floor(pos), n, i;
    double x = pos - v, a;
    *kmax = v;
    for (i = 0; i < order; ++i) { lastvals[i] = Zero; lastvals2[i] = Zero; values[i] = Zero; }
    values[0] = x;
    if (order > 1) {
        values[1] = (One - x);
        for (n = 3; n <= order; ++n) {
            for (i = 0; i < order; ++i) lastvals[i] = values[i];
            if (n == order - 1)
                for (i = 0; i < order; ++i) lastvals2[i] = values[i];
            values[0] = x * lastvals[0] / (n - 1);
            for (i = 1; i <= n - 2; ++i) {
                a = i + x;
                values[i] = (a * lastvals[i] + (n - a) * lastvals[i - 1]) / (n - 1);
            }
            values[n - 1] = (1 - x) * lastvals[n - 2] / (n - 1);
        }
        n = order;
        derivs[0] = lastvals[0];
        for (i = 1; i <= n - 2; ++i) derivs[i] = lastvals[i] - lastvals[i - 1];
        derivs[n - 1] = -lastvals[n - 2];
        derivs2[0] = lastvals2[0];
        derivs2[1] = lastvals2[1] - 2 * lastvals2[0];
        for (i = 2; i <= n - 3; ++i) derivs2[i] = lastvals2[i] - 2 * lastvals2[i - 1] + lastvals2[i - 2];
        if (n > 3) derivs2[n - 2] = -2 * lastvals2[n - 3] + lastvals2[n - 4];
        if (n > 2) derivs2[n - 1] = lastvals2[n - 3];
    } else {
        derivs[0] = Zero;
        derivs2[0] = Zero;
    }
}

/* the Ewald constants of EwaldSetup, energy.F90:7040-7047 */
static void dipole_ewald_facs(double ualpha, double *f1, double *f2, double *f3, double *s1, double *s2) {
    double ualpha2 = ualpha * ualpha;
    double fac = One / (sqrt(Pi) * ualpha);
    *f1 = fac * Two * ualpha2;
    *f2 = fac * pow2(Two * ualpha2) / Three;
    *f3 = fac * pow3(Two * ualpha2) / (Three * 5.0);
    *s1 = (Two * ualpha) / sqrt(Pi);
    *s2 = (Four * pow3(ualpha)) / (Three * sqrt(Pi));
}

/* UDipoleP, energy.F90:1588-1798: the particle pairs of the list (in MC
   only jp > ip), the centre separation folded by PBC2 and that shift
   applied to every atom pair; with Ewald (ualpha > 0) the erfc-screened
   kernels, otherwise bare ones.  Initialises the arrays.  u_real is
   UDipole's "ureal", EpsiFourPi/2 sum (q pot - dip . e), energy.F90:1494-1498. */
int orc_poly_udipole_real(const mg_poly_params *p, int32_t maxnneigh, const double *ro, const double *r,
                          const double *dip, const int32_t *nneighpn, const int32_t *jpnlist, double *potstat,
                          double *estat, double *efg, double *virelec, double *u_real) {
    const double *az = p->aza;
    double half[3], rcut2 = p->rcut * p->rcut, vir = Zero;
    int lewald = p->ualpha > Zero;
    double ualpha = p->ualpha, ualpha2 = ualpha * ualpha, f1 = Zero, f2 = Zero, f3 = Zero, s1, s2;
    if (lewald) dipole_ewald_facs(ualpha, &f1, &f2, &f3, &s1, &s2);
    for (int m = 0; m < 3; ++m) half[m] = p->boxlen[m] / Two;
    for (int k = 0; k < p->na; ++k) potstat[k] = Zero;
    for (int k = 0; k < 3 * p->na; ++k) estat[k] = Zero;
    for (int k = 0; k < 6 * p->na; ++k) efg[k] = Zero;
    for (int ip = 1; ip <= p->np; ++ip) {
        int ipt = p->iptpn[ip - 1];
        int ialow = p->ianpn[ip - 1], iaupp = ialow + p->napt[ipt - 1] - 1;
        for (int jploc = 1; jploc <= nneighpn[ip - 1]; ++jploc) {
            int jp = jpnlist[(size_t)(ip - 1) * maxnneigh + jploc - 1];
            if (p->lmc && jp < ip) continue;
            int jpt = p->iptpn[jp - 1];
            double d[3], sh[3];
            for (int m = 0; m < 3; ++m) {
                d[m] = ro[3 * (ip - 1) + m] - ro[3 * (jp - 1) + m];
                sh[m] = Zero;
                if (fabs(d[m]) > half[m]) sh[m] = fsign(p->boxlen[m], d[m]);
                d[m] = d[m] - sh[m];
            }
            double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (r2 > rcut2) continue;
            int jalow = p->ianpn[jp - 1], jaupp = jalow + p->napt[jpt - 1] - 1;
            for (int ia = ialow; ia <= iaupp; ++ia) {
                for (int ja = jalow; ja <= jaupp; ++ja) {
                    double dx = r[3 * (ia - 1)] - r[3 * (ja - 1)] - sh[0];
                    double dy = r[3 * (ia - 1) + 1] - r[3 * (ja - 1) + 1] - sh[1];
                    double dz = r[3 * (ia - 1) + 2] - r[3 * (ja - 1) + 2] - sh[2];
                    double ar2 = dx * dx + dy * dy + dz * dz;
                    double r1 = sqrt(ar2);
                    double r1i = One / r1;
                    double r2i = r1i * r1i, r3i, r5i, r7i;
                    if (lewald) {
                        double ex = exp(-ualpha2 * ar2);
                        r1i = r1i * (One - orc_erf2(ualpha * r1));
                        r3i = r2i * (r1i + f1 * ex);
                        r5i = r2i * (r3i + f2 * ex);
                        r7i = r2i * (r5i + f3 * ex);
                    } else {
                        r3i = r2i * r1i;
                        r5i = r2i * r3i;
                        r7i = r2i * r5i;
                    }
                    double threer5i = Three * r5i;
                    const double *di = &dip[3 * (ia - 1)], *dj = &dip[3 * (ja - 1)];
                    double qi = az[ia - 1], qj = az[ja - 1];
                    double doti = di[0] * dx + di[1] * dy + di[2] * dz;
                    double dotj = dj[0] * dx + dj[1] * dy + dj[2] * dz;
                    double dotir5i = Three * r5i * doti;
                    double dotjr5i = Three * r5i * dotj;
                    double dotir7i = (Three * 5.0 * r7i) * doti;
                    double dotjr7i = (Three * 5.0 * r7i) * dotj;
                    potstat[ia - 1] = potstat[ia - 1] + (qj * r1i + dotj * r3i);
                    potstat[ja - 1] = potstat[ja - 1] + (qi * r1i - doti * r3i);
                    double fx = (+qj * dx - dj[0]) * r3i + dotjr5i * dx;
                    double fy = (+qj * dy - dj[1]) * r3i + dotjr5i * dy;
                    double fz = (+qj * dz - dj[2]) * r3i + dotjr5i * dz;
                    double *ei = &estat[3 * (ia - 1)], *ej = &estat[3 * (ja - 1)];
                    ei[0] = ei[0] + fx;
                    ei[1] = ei[1] + fy;
                    ei[2] = ei[2] + fz;
                    vir = vir - qi * (fx * dx + fy * dy + fz * dz);
                    fx = (-qi * dx - di[0]) * r3i + dotir5i * dx;
                    fy = (-qi * dy - di[1]) * r3i + dotir5i * dy;
                    fz = (-qi * dz - di[2]) * r3i + dotir5i * dz;
                    ej[0] = ej[0] + fx;
                    ej[1] = ej[1] + fy;
                    ej[2] = ej[2] + fz;
                    double xx = qj * r3i + (-qj * dx * dx + Two * dj[0] * dx + dotj) * threer5i - dotjr7i * dx * dx;
                    double yy = qj * r3i + (-qj * dy * dy + Two * dj[1] * dy + dotj) * threer5i - dotjr7i * dy * dy;
                    double zz = qj * r3i + (-qj * dz * dz + Two * dj[2] * dz + dotj) * threer5i - dotjr7i * dz * dz;
                    double xy = (-qj * dx * dy + dj[0] * dy + dj[1] * dx) * threer5i - dotjr7i * dx * dy;
                    double xz = (-qj * dx * dz + dj[0] * dz + dj[2] * dx) * threer5i - dotjr7i * dx * dz;
                    double yz = (-qj * dy * dz + dj[1] * dz + dj[2] * dy) * threer5i - dotjr7i * dy * dz;
                    double *gi = &efg[6 * (ia - 1)], *gj = &efg[6 * (ja - 1)];
                    gi[0] = gi[0] + xx; gi[1] = gi[1] + yy; gi[2] = gi[2] + zz;
                    gi[3] = gi[3] + xy; gi[4] = gi[4] + xz; gi[5] = gi[5] + yz;
                    vir = vir - (di[0] * xx * dx + di[0] * xy * dy + di[0] * xz * dz
                               + di[1] * xy * dx + di[1] * yy * dy + di[1] * yz * dz
                               + di[2] * xz * dx + di[2] * yz * dy + di[2] * zz * dz);
                    xx = qi * r3i + (-qi * dx * dx - Two * di[0] * dx - doti) * threer5i + dotir7i * dx * dx;
                    yy = qi * r3i + (-qi * dy * dy - Two * di[1] * dy - doti) * threer5i + dotir7i * dy * dy;
                    zz = qi * r3i + (-qi * dz * dz - Two * di[2] * dz - doti) * threer5i + dotir7i * dz * dz;
                    xy = (-qi * dx * dy - di[0] * dy - di[1] * dx) * threer5i + dotir7i * dx * dy;
                    xz = (-qi * dx * dz - di[0] * dz - di[2] * dx) * threer5i + dotir7i * dx * dz;
                    yz = (-qi * dy * dz - di[1] * dz - di[2] * dy) * threer5i + dotir7i * dy * dz;
                    gj[0] = gj[0] + xx; gj[1] = gj[1] + yy; gj[2] = gj[2] + zz;
                    gj[3] = gj[3] + xy; gj[4] = gj[4] + xz; gj[5] = gj[5] + yz;
                }
            }
        }
    }
    *virelec = vir;
    double ur = Zero;
    for (int ia = 0; ia < p->na; ++ia)
        ur = ur + az[ia] * potstat[ia] - (dip[3 * ia] * estat[3 * ia] + dip[3 * ia + 1] * estat[3 * ia + 1]
                                          + dip[3 * ia + 2] * estat[3 * ia + 2]);
    *u_real = p->epsi_four_pi * Half * ur;
    return 0;
}

/* UDipoleEwaldSelf, molecular contribution (energy.F90:2196-2268), and with
   lsurf UDipoleEwaldSurf (energy.F90:2272-2295; the atom positions r as
   they are, not folded into the box) */
int orc_poly_udipole_self(const mg_poly_params *p, const double *r, const double *dip, int32_t lsurf,
                          double *potstat, double *estat, double *efg, double *virelec) {
    const double *az = p->aza;
    double ualpha = p->ualpha, ualpha2 = ualpha * ualpha, f1, f2, f3, s1, s2;
    dipole_ewald_facs(ualpha, &f1, &f2, &f3, &s1, &s2);
    double vir = *virelec;
    for (int ip = 1; ip <= p->np; ++ip) {
        int ipt = p->iptpn[ip - 1];
        int ialow = p->ianpn[ip - 1], iaupp = ialow + p->napt[ipt - 1] - 1;
        for (int ia = ialow; ia <= iaupp; ++ia) {
            for (int ja = ia + 1; ja <= iaupp; ++ja) {
                double dx = r[3 * (ia - 1)] - r[3 * (ja - 1)];
                double dy = r[3 * (ia - 1) + 1] - r[3 * (ja - 1) + 1];
                double dz = r[3 * (ia - 1) + 2] - r[3 * (ja - 1) + 2];
                double ar2 = dx * dx + dy * dy + dz * dz;
                double r1 = sqrt(ar2);
                double r1i = One / r1;
                double r2i = r1i * r1i;
                double ex = exp(-ualpha2 * ar2);
                r1i = r1i * orc_erf2(ualpha * r1);
                double r3i = r2i * (r1i - f1 * ex);
                double r5i = r2i * (r3i - f2 * ex);
                double r7i = r2i * (r5i - f3 * ex);
                double threer5i = Three * r5i;
                const double *di = &dip[3 * (ia - 1)], *dj = &dip[3 * (ja - 1)];
                double qi = az[ia - 1], qj = az[ja - 1];
                double doti = di[0] * dx + di[1] * dy + di[2] * dz;
                double dotj = dj[0] * dx + dj[1] * dy + dj[2] * dz;
                double dotir5i = Three * r5i * doti;
                double dotjr5i = Three * r5i * dotj;
                double dotir7i = (Three * 5.0 * r7i) * doti;
                double dotjr7i = (Three * 5.0 * r7i) * dotj;
                potstat[ia - 1] = potstat[ia - 1] - (qj * r1i + dotj * r3i);
                potstat[ja - 1] = potstat[ja - 1] - (qi * r1i - doti * r3i);
                double fx = -((qj * dx - dj[0]) * r3i + dotjr5i * dx);
                double fy = -((qj * dy - dj[1]) * r3i + dotjr5i * dy);
                double fz = -((qj * dz - dj[2]) * r3i + dotjr5i * dz);
                double *ei = &estat[3 * (ia - 1)], *ej = &estat[3 * (ja - 1)];
                ei[0] = ei[0] + fx;
                ei[1] = ei[1] + fy;
                ei[2] = ei[2] + fz;
                vir = vir - (qi * (fx * dx + fy * dy + fz * dz));
                fx = -((-qi * dx - di[0]) * r3i + dotir5i * dx);
                fy = -((-qi * dy - di[1]) * r3i + dotir5i * dy);
                fz = -((-qi * dz - di[2]) * r3i + dotir5i * dz);
                ej[0] = ej[0] + fx;
                ej[1] = ej[1] + fy;
                ej[2] = ej[2] + fz;
                double xx = -(qj * r3i + (-qj * dx * dx + Two * dj[0] * dx + dotj) * threer5i - dotjr7i * dx * dx);
                double yy = -(qj * r3i + (-qj * dy * dy + Two * dj[1] * dy + dotj) * threer5i - dotjr7i * dy * dy);
                double zz = -(qj * r3i + (-qj * dz * dz + Two * dj[2] * dz + dotj) * threer5i - dotjr7i * dz * dz);
                double xy = -((-qj * dx * dy + dj[0] * dy + dj[1] * dx) * threer5i - dotjr7i * dx * dy);
                double xz = -((-qj * dx * dz + dj[0] * dz + dj[2] * dx) * threer5i - dotjr7i * dx * dz);
                double yz = -((-qj * dy * dz + dj[1] * dz + dj[2] * dy) * threer5i - dotjr7i * dy * dz);
                double *gi = &efg[6 * (ia - 1)], *gj = &efg[6 * (ja - 1)];
                gi[0] = gi[0] + xx; gi[1] = gi[1] + yy; gi[2] = gi[2] + zz;
                gi[3] = gi[3] + xy; gi[4] = gi[4] + xz; gi[5] = gi[5] + yz;
                vir = vir - (di[0] * xx * dx + di[0] * xy * dy + di[0] * xz * dz
                           + di[1] * xy * dx + di[1] * yy * dy + di[1] * yz * dz
                           + di[2] * xz * dx + di[2] * yz * dy + di[2] * zz * dz);
                xx = -(qi * r3i + (-qi * dx * dx - Two * di[0] * dx - doti) * threer5i + dotir7i * dx * dx);
                yy = -(qi * r3i + (-qi * dy * dy - Two * di[1] * dy - doti) * threer5i + dotir7i * dy * dy);
                zz = -(qi * r3i + (-qi * dz * dz - Two * di[2] * dz - doti) * threer5i + dotir7i * dz * dz);
                xy = -((-qi * dx * dy - di[0] * dy - di[1] * dx) * threer5i + dotir7i * dx * dy);
                xz = -((-qi * dx * dz - di[0] * dz - di[2] * dx) * threer5i + dotir7i * dx * dz);
                yz = -((-qi * dy * dz - di[1] * dz - di[2] * dy) * threer5i + dotir7i * dy * dz);
                gj[0] = gj[0] + xx; gj[1] = gj[1] + yy; gj[2] = gj[2] + zz;
                gj[3] = gj[3] + xy; gj[4] = gj[4] + xz; gj[5] = gj[5] + yz;
            }
        }
    }
    if (lsurf) {
        double vol = p->boxlen[0] * p->boxlen[1] * p->boxlen[2];
        double fac = (Four * Pi / Three) / vol;
        double sqx = Zero, sqy = Zero, sqz = Zero, sdx = Zero, sdy = Zero, sdz = Zero;
        for (int ia = 0; ia < p->na; ++ia) sqx = sqx + az[ia] * r[3 * ia];
        for (int ia = 0; ia < p->na; ++ia) sqy = sqy + az[ia] * r[3 * ia + 1];
        for (int ia = 0; ia < p->na; ++ia) sqz = sqz + az[ia] * r[3 * ia + 2];
        for (int ia = 0; ia < p->na; ++ia) sdx = sdx + dip[3 * ia];
        for (int ia = 0; ia < p->na; ++ia) sdy = sdy + dip[3 * ia + 1];
        for (int ia = 0; ia < p->na; ++ia) sdz = sdz + dip[3 * ia + 2];
        for (int ia = 0; ia < p->na; ++ia)
            potstat[ia] = potstat[ia] + fac * (r[3 * ia] * (sqx + sdx) + r[3 * ia + 1] * (sqy + sdy)
                                               + r[3 * ia + 2] * (sqz + sdz));
        for (int ia = 0; ia < p->na; ++ia) {
            estat[3 * ia] = estat[3 * ia] - fac * (sqx + sdx);
            estat[3 * ia + 1] = estat[3 * ia + 1] - fac * (sqy + sdy);
            estat[3 * ia + 2] = estat[3 * ia + 2] - fac * (sqz + sdz);
        }
        vir = vir - TwoPi / (Three * vol) * ((sqx * sqx + sqy * sqy + sqz * sqz)
                                            + Two * (Two * (sqx * sdx + sqy * sdy + sqz * sdz))
                                            + Three * (sdx * sdx + sdy * sdy + sdz * sdz));
    }
    *virelec = vir;
    return 0;
}

/* UDipole's loop, energy.F90:1510-1545: u%stat = EpsiFourPi/2 sum (q pot -
   dip . e); force(ia) += EpsiFourPi (q e + dip . efg) (added to force, as
   the reference adds to the UTwoBodyP forces); torque(ia) = EpsiFourPi
   dip x e (added to torque) */
int orc_poly_udipole_finish(const mg_poly_params *p, const double *dip, const double *potstat, const double *estat,
                            const double *efg, double *force, double *torque, double *u_stat) {
    const double *az = p->aza;
    double efp = p->epsi_four_pi, us = Zero;
    for (int ia = 0; ia < p->na; ++ia) {
        const double *d = &dip[3 * ia], *e = &estat[3 * ia], *g = &efg[6 * ia];
        double q = az[ia];
        us = us + q * potstat[ia] - (d[0] * e[0] + d[1] * e[1] + d[2] * e[2]);
        double fx = q * e[0] + (d[0] * g[0] + d[1] * g[3] + d[2] * g[4]);
        double fy = q * e[1] + (d[0] * g[3] + d[1] * g[1] + d[2] * g[5]);
        double fz = q * e[2] + (d[0] * g[4] + d[1] * g[5] + d[2] * g[2]);
        force[3 * ia] = force[3 * ia] + efp * fx;
        force[3 * ia + 1] = force[3 * ia + 1] + efp * fy;
        force[3 * ia + 2] = force[3 * ia + 2] + efp * fz;
        torque[3 * ia] = torque[3 * ia] + efp * (d[1] * e[2] - d[2] * e[1]);
        torque[3 * ia + 1] = torque[3 * ia + 1] + efp * (d[2] * e[0] - d[0] * e[2]);
        torque[3 * ia + 2] = torque[3 * ia + 2] + efp * (d[0] * e[1] - d[1] * e[0]);
    }
    *u_stat = efp * Half * us;
    return 0;
}

/* ---- rigid-body velocity Verlet (VelVer, md.F90:252-420, lpolyatom) ----
   Stateless: the caller holds ro(3,np), qua(0:3,np), rod, rodd, quad, quadd,
   angvelo; each routine updates them in place, loop by loop as VelVer
   does. */

/* QuaToOri, mollib.F90:2221-2255: ori(3,3,np), column-major */
static void rigid_qua_to_ori(const double *q, double *ori) {
    double qua00 = q[0] * q[0], qua11 = q[1] * q[1], qua22 = q[2] * q[2], qua33 = q[3] * q[3];
    double qua01 = q[0] * q[1], qua02 = q[0] * q[2], qua03 = q[0] * q[3];
    double qua12 = q[1] * q[2], qua13 = q[1] * q[3], qua23 = q[2] * q[3];
    ori[0] = -qua22 + qua11 - qua33 + qua00;      /* ori(1,1) */
    ori[1] = Two * (qua03 - qua12);               /* ori(2,1) */
    ori[2] = Two * (qua13 + qua02);               /* ori(3,1) */
    ori[3] = -Two * (qua12 + qua03);              /* ori(1,2) */
    ori[4] = qua22 - qua11 - qua33 + qua00;       /* ori(2,2) */
    ori[5] = Two * (qua01 - qua23);               /* ori(3,2) */
    ori[6] = Two * (qua13 - qua02);               /* ori(1,3) */
    ori[7] = -Two * (qua23 + qua01);              /* ori(2,3) */
    ori[8] = -qua22 - qua11 + qua33 + qua00;      /* ori(3,3) */
}

/* AngVelToQuaVel, mollib.F90:2621-2642 */
int orc_angvel_to_quavel(int32_t np, const double *qua, const double *angvelo, double *quad) {
    for (int ip = 0; ip < np; ++ip) {
        const double *q = &qua[4 * ip], *w = &angvelo[3 * ip];
        double *d = &quad[4 * ip];
        d[0] = Half * (-q[1] * w[0] + q[2] * w[1] - q[3] * w[2]);
        d[1] = Half * (+q[0] * w[0] - q[3] * w[1] - q[2] * w[2]);
        d[2] = Half * (-q[3] * w[0] - q[0] * w[1] + q[1] * w[2]);
        d[3] = Half * (+q[2] * w[0] + q[1] * w[1] + q[0] * w[2]);
    }
    return 0;
}

/* VelVer's first part (md.F90:288-306): drostep, ro with PBC (box-like
   cell, molaux.F90:104-118), qua, QuaNorm (mollib.F90:2594-2612),
   QuaToOri */
int orc_rigid_move(int32_t np, double tstep, const double *boxlen, double *ro, double *qua, const double *rod,
                   const double *rodd, const double *quad, const double *quadd, double *drostep, double *ori) {
    double fac = Half * (tstep * tstep);
    for (int ip = 0; ip < np; ++ip) {
        for (int m = 0; m < 3; ++m) {
            drostep[3 * ip + m] = tstep * rod[3 * ip + m] + fac * rodd[3 * ip + m];
            ro[3 * ip + m] = ro[3 * ip + m] + drostep[3 * ip + m];
            double x = ro[3 * ip + m];
            if (fabs(x) > Half * boxlen[m]) x = x - boxlen[m] * round(x * (One / boxlen[m]));
            ro[3 * ip + m] = x;
        }
    }
    for (int ip = 0; ip < np; ++ip)
        for (int k = 0; k < 4; ++k)
            qua[4 * ip + k] = qua[4 * ip + k] + tstep * quad[4 * ip + k] + fac * quadd[4 * ip + k];
    for (int ip = 0; ip < np; ++ip) {
        double *q = &qua[4 * ip];
        double norm = One / sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
        for (int k = 0; k < 4; ++k) q[k] = q[k] * norm;
        rigid_qua_to_ori(q, &ori[9 * ip]);
    }
    return 0;
}

/* VelVer's second part (md.F90:347-402): GetLinAcc (md.F90:601-617), rod;
   quaddo, quado, the trial quad, nvvite times QuaVelToAngVel
   (mollib.F90:2651-2669), GetAngAcc (md.F90:628-663) and quad.  momp are
   the principal moments; momip = InvFlt(momp) (mollib.F90:2814-2819). */
int orc_rigid_kick(int32_t np, double tstep, double tvvite, int32_t nvvite, const double *massip,
                   const double *momp, const double *qua, const double *forceo, const double *torqueo, double *rod,
                   double *rodd, double *quad, double *quadd, double *angvelo) {
    for (int ip = 0; ip < np; ++ip)
        for (int m = 0; m < 3; ++m) {
            double roddo = rodd[3 * ip + m];
            rodd[3 * ip + m] = massip[ip] * forceo[3 * ip + m];
            rod[3 * ip + m] = rod[3 * ip + m] + Half * tstep * (rodd[3 * ip + m] + roddo);
        }
    double *quaddo = (double *)malloc(sizeof(double) * 4 * (size_t)(np > 0 ? np : 1));
    double *quado = (double *)malloc(sizeof(double) * 4 * (size_t)(np > 0 ? np : 1));
    if (!quaddo || !quado) { free(quaddo); free(quado); return MG_ERR_ALLOC; }
    for (int k = 0; k < 4 * np; ++k) quaddo[k] = quadd[k];
    for (int k = 0; k < 4 * np; ++k) {
        quado[k] = quad[k];
        quad[k] = quado[k] + (tvvite * tstep) * quaddo[k];
    }
    for (int it = 1; it <= nvvite; ++it) {
        for (int ip = 0; ip < np; ++ip) {   /* QuaVelToAngVel */
            const double *q = &qua[4 * ip], *d = &quad[4 * ip];
            double *w = &angvelo[3 * ip];
            w[0] = Two * (-q[3] * d[2] + q[0] * d[1] + q[2] * d[3] - q[1] * d[0]);
            w[1] = Two * (-q[0] * d[2] - q[3] * d[1] + q[1] * d[3] + q[2] * d[0]);
            w[2] = Two * (+q[1] * d[2] - q[2] * d[1] + q[0] * d[3] - q[3] * d[0]);
        }
        for (int ip = 0; ip < np; ++ip) {   /* GetAngAcc */
            const double *q = &qua[4 * ip], *d = &quad[4 * ip], *tq = &torqueo[3 * ip], *w = &angvelo[3 * ip];
            const double *mp = &momp[3 * ip];
            double ori[9], mi[3];
            for (int m = 0; m < 3; ++m) mi[m] = mp[m] > Zero ? One / mp[m] : Zero;
            rigid_qua_to_ori(q, ori);
            double tor1 = tq[0] * ori[0] + tq[1] * ori[1] + tq[2] * ori[2];
            double tor2 = tq[0] * ori[3] + tq[1] * ori[4] + tq[2] * ori[5];
            double tor3 = tq[0] * ori[6] + tq[1] * ori[7] + tq[2] * ori[8];
            double a1 = (tor1 + w[1] * w[2] * (mp[1] - mp[2])) * mi[0];
            double a2 = (tor2 + w[2] * w[0] * (mp[2] - mp[0])) * mi[1];
            double a3 = (tor3 + w[0] * w[1] * (mp[0] - mp[1])) * mi[2];
            double fac = -Two * (d[2] * d[2] + d[1] * d[1] + d[3] * d[3] + d[0] * d[0]);
            double *dd = &quadd[4 * ip];
            dd[0] = Half * (-q[1] * a1 + q[2] * a2 - q[3] * a3 + q[0] * fac);
            dd[1] = Half * (+q[0] * a1 - q[3] * a2 - q[2] * a3 + q[1] * fac);
            dd[2] = Half * (-q[3] * a1 - q[0] * a2 + q[1] * a3 + q[2] * fac);
            dd[3] = Half * (+q[2] * a1 + q[1] * a2 + q[0] * a3 + q[3] * fac);
        }
        for (int k = 0; k < 4 * np; ++k) quad[k] = quado[k] + (Half * tstep) * (quadd[k] + quaddo[k]);
    }
    free(quaddo);
    free(quado);
    return 0;
}

/* the energy terms of the last UTotal: u%tot, u%twob(0), u%rec, u%bond,
   u%angle, virial */
int orc_energy_terms(orc_sys *s, double *terms) {
    terms[0] = s->u_tot;
    terms[1] = s->u_twob[0];
    terms[2] = s->u_rec;
    terms[3] = s->u_bond;
    terms[4] = s->u_angle;
    terms[5] = s->virial;
    return 0;
}

/* UTotal, energy.F90:280-430 (charged monoatomic branch) */
static int utotal_core(orc_sys *s) {
    int st = 0;
    s->u_tot = Zero;
    for (int k = 0; k <= s->nptpt; ++k) s->u_twob[k] = Zero;
    memset(s->force, 0, sizeof(double) * 3 * s->np);
    s->virial = Zero;
    s->u_bond = Zero;
    if (s->txintlist == MG_VLIST) {
        if (!s->nneighpn) return MG_ERR_STATE;
        st = utwobody(s, 0);
    } else {
        if (!s->cell) return MG_ERR_STATE;
        st = utwobody(s, 1);
    }
    if (st) return st;
    if (s->ewald != MG_EWALD_NONE) { st = uewald(s); if (st) return st; }
    if (s->nbond > 0) ubond(s);
    if (s->nangle > 0) uangle(s);
    double fac = s->force_fac;
    for (int ia = 1; ia <= s->np; ++ia) {
        /* monoatomic: r == ro, so the molecular virial term is zero */
        for (int m = 1; m <= 3; ++m) {
            FORCE(m, ia) = FORCE(m, ia) * fac;
            s->forceo[3 * (ia - 1) + m - 1] = Zero + FORCE(m, ia);
        }
    }
    return 0;
}

static void copy_out(orc_sys *s, double *forceo, double *u_twob, double *uout) {
    if (forceo) memcpy(forceo, s->forceo, sizeof(double) * 3 * s->np);
    if (u_twob) memcpy(u_twob, s->u_twob, sizeof(double) * (s->nptpt + 1));
    if (uout) { uout[0] = s->u_tot; uout[1] = s->u_rec; uout[2] = s->u_bond; uout[3] = s->virial; }
}

int orc_utotal(orc_sys *s, double *forceo, double *u_twob, double *uout) {
    int st = utotal_core(s);
    if (st) return st;
    copy_out(s, forceo, u_twob, uout);
    return 0;
}

int orc_get_qmesh(orc_sys *s, double *q) {
    if (s->ewald != MG_EWALD_SPM) return MG_ERR_STATE;
    memcpy(q, s->Qspread, sizeof(double) * (size_t)s->nmesh * s->nmesh * s->nmesh);
    return 0;
}

/* ======================================================================
 * denergy.F90
 * ====================================================================== */

/* UTwoBodyANew / UTwoBodyAOld (Verlet list), denergy.F90:289-504, and the
   cell-list versions, denergy.F90:728-935. Returns 1 on overlap. */
static int utwobody_new(orc_sys *s, int *err) {
    for (int k = 0; k <= s->nptpt; ++k) s->utwobnew[k] = Zero;
    for (int iploc = 1; iploc <= s->nptm; ++iploc) {
        int ip = s->ipnptm[iploc - 1], ipt = IPTPN(ip);
        const double *rt = &s->rotm[3 * (iploc - 1)];
        if (s->txintlist == MG_VLIST) {
            for (int jploc = 1; jploc <= s->nneighpn[ip - 1]; ++jploc) {
                int jp = s->jpnlist[(size_t)(ip - 1) * s->maxnneigh + jploc - 1];
                if (s->lptm[jp - 1]) continue;
                int iptjpt = IPTPT(ipt, IPTPN(jp));
                double dx = rt[0] - RO(1, jp), dy = rt[1] - RO(2, jp), dz = rt[2] - RO(3, jp), r2, usum;
                pbcr2(s, &dx, &dy, &dz, &r2);
                if (r2 > s->rcut2) continue;
                if (r2 < s->r2atat[iptjpt - 1]) return 1;
                if (r2 < s->r2umin[iptjpt - 1]) return 1;
                if ((*err = table_eval(s, iptjpt, r2, &usum, NULL))) return 1;
                s->utwobnew[iptjpt] = s->utwobnew[iptjpt] + usum;
            }
        } else {
            int icell = pcellro(s, rt);
            if (icell < 0) { *err = MG_ERR_CELL; return 1; }
            orc_cell *ic = &s->cell[icell];
            for (int incell = 0; incell < ic->nneighcell; ++incell) {
                orc_cell *nc = &s->cell[ic->neigh[incell]];
                int jp = nc->iphead;
                for (int jploc = 1; jploc <= nc->npart; ++jploc) {
                    if (!s->lptm[jp - 1]) {
                        int iptjpt = IPTPT(ipt, IPTPN(jp));
                        double dx = rt[0] - RO(1, jp), dy = rt[1] - RO(2, jp), dz = rt[2] - RO(3, jp), r2, usum;
                        pbcr2(s, &dx, &dy, &dz, &r2);
                        if (r2 < s->rcut2) {
                            if (r2 < s->r2atat[iptjpt - 1]) return 1;
                            if (r2 < s->r2umin[iptjpt - 1]) return 1;
                            if ((*err = table_eval(s, iptjpt, r2, &usum, NULL))) return 1;
                            s->utwobnew[iptjpt] = s->utwobnew[iptjpt] + usum;
                        }
                    }
                    jp = s->ipnext[jp - 1];
                }
            }
        }
    }
    /* pairs where both particles move (lptmdutwob) */
    for (int iploc = 1; iploc <= s->nptm; ++iploc) {
        int ip = s->ipnptm[iploc - 1], ipt = IPTPN(ip);
        for (int jploc = iploc + 1; jploc <= s->nptm; ++jploc) {
            int jp = s->ipnptm[jploc - 1];
            int iptjpt = IPTPT(ipt, IPTPN(jp));
            const double *ri = &s->rotm[3 * (iploc - 1)], *rj = &s->rotm[3 * (jploc - 1)];
            double dx = ri[0] - rj[0], dy = ri[1] - rj[1], dz = ri[2] - rj[2], r2, usum;
            pbcr2(s, &dx, &dy, &dz, &r2);
            if (s->txintlist == MG_VLIST ? (r2 > s->rcut2) : !(r2 < s->rcut2)) continue;
            if (r2 < s->r2atat[iptjpt - 1]) return 1;
            if (r2 < s->r2umin[iptjpt - 1]) return 1;
            if ((*err = table_eval(s, iptjpt, r2, &usum, NULL))) return 1;
            s->utwobnew[iptjpt] = s->utwobnew[iptjpt] + usum;
        }
    }
    double t = Zero;
    for (int k = 1; k <= s->nptpt; ++k) t = t + s->utwobnew[k];
    s->utwobnew[0] = t;
    return 0;
}

static int utwobody_old(orc_sys *s) {
    for (int k = 0; k <= s->nptpt; ++k) s->utwobold[k] = Zero;
    for (int iploc = 1; iploc <= s->nptm; ++iploc) {
        int ip = s->ipnptm[iploc - 1], ipt = IPTPN(ip);
        if (s->txintlist == MG_VLIST) {
            for (int jploc = 1; jploc <= s->nneighpn[ip - 1]; ++jploc) {
                int jp = s->jpnlist[(size_t)(ip - 1) * s->maxnneigh + jploc - 1];
                if (s->lptm[jp - 1]) continue;
                int iptjpt = IPTPT(ipt, IPTPN(jp));
                double dx = RO(1, ip) - RO(1, jp), dy = RO(2, ip) - RO(2, jp), dz = RO(3, ip) - RO(3, jp), r2, usum;
                pbcr2(s, &dx, &dy, &dz, &r2);
                if (r2 > s->rcut2) continue;
                if (r2 < s->r2umin[iptjpt - 1]) return 1;
                int st = table_eval(s, iptjpt, r2, &usum, NULL);
                if (st) return st;
                s->utwobold[iptjpt] = s->utwobold[iptjpt] + usum;
            }
        } else {
            orc_cell *ic = &s->cell[s->cellip[ip - 1]];
            for (int incell = 0; incell < ic->nneighcell; ++incell) {
                orc_cell *nc = &s->cell[ic->neigh[incell]];
                int jp = nc->iphead;
                for (int jploc = 1; jploc <= nc->npart; ++jploc) {
                    if (!s->lptm[jp - 1]) {
                        int iptjpt = IPTPT(ipt, IPTPN(jp));
                        double dx = RO(1, ip) - RO(1, jp), dy = RO(2, ip) - RO(2, jp), dz = RO(3, ip) - RO(3, jp), r2, usum;
                        pbcr2(s, &dx, &dy, &dz, &r2);
                        if (r2 < s->rcut2) {
                            int st = table_eval(s, iptjpt, r2, &usum, NULL);
                            if (st) return st;
                            s->utwobold[iptjpt] = s->utwobold[iptjpt] + usum;
                        }
                    }
                    jp = s->ipnext[jp - 1];
                }
            }
        }
    }
    for (int iploc = 1; iploc <= s->nptm; ++iploc) {
        int ip = s->ipnptm[iploc - 1], ipt = IPTPN(ip);
        for (int jploc = iploc + 1; jploc <= s->nptm; ++jploc) {
            int jp = s->ipnptm[jploc - 1];
            int iptjpt = IPTPT(ipt, IPTPN(jp));
            double dx = RO(1, ip) - RO(1, jp), dy = RO(2, ip) - RO(2, jp), dz = RO(3, ip) - RO(3, jp), r2, usum;
            pbcr2(s, &dx, &dy, &dz, &r2);
            if (s->txintlist == MG_VLIST ? (r2 > s->rcut2) : !(r2 < s->rcut2)) continue;
            int st = table_eval(s, iptjpt, r2, &usum, NULL);
            if (st) return st;
            s->utwobold[iptjpt] = s->utwobold[iptjpt] + usum;
        }
    }
    double t = Zero;
    for (int k = 1; k <= s->nptpt; ++k) t = t + s->utwobold[k];
    s->utwobold[0] = t;
    return 0;
}

/* EwaldSetArrayTM, denergy.F90:1708-1737 */
#define EIKTM(a, ialoc, n) (a)[(size_t)(n) * s->np + ((ialoc) - 1)]
static void ewald_set_array_tm(orc_sys *s) {
    for (int ialoc = 1; ialoc <= s->nptm; ++ialoc) {
        const double *rt = &s->rotm[3 * (ialoc - 1)];
        zc one = {One, Zero};
        EIKTM(s->eikxtm, ialoc, 0) = one; EIKTM(s->eikytm, ialoc, 0) = one; EIKTM(s->eikztm, ialoc, 0) = one;
        double ax = s->TwoPiBoxi[0] * rt[0], ay = s->TwoPiBoxi[1] * rt[1], az = s->TwoPiBoxi[2] * rt[2];
        zc ex = {cos(ax), sin(ax)}, ey = {cos(ay), sin(ay)}, ez = {cos(az), sin(az)};
        if (s->ncut >= 1) { EIKTM(s->eikxtm, ialoc, 1) = ex; EIKTM(s->eikytm, ialoc, 1) = ey; EIKTM(s->eikztm, ialoc, 1) = ez; }
    }
    for (int icut = 2; icut <= s->ncut; ++icut)
        for (int ialoc = 1; ialoc <= s->nptm; ++ialoc) {
            EIKTM(s->eikxtm, ialoc, icut) = zmul(EIKTM(s->eikxtm, ialoc, icut - 1), EIKTM(s->eikxtm, ialoc, 1));
            EIKTM(s->eikytm, ialoc, icut) = zmul(EIKTM(s->eikytm, ialoc, icut - 1), EIKTM(s->eikytm, ialoc, 1));
            EIKTM(s->eikztm, ialoc, icut) = zmul(EIKTM(s->eikztm, ialoc, icut - 1), EIKTM(s->eikztm, ialoc, 1));
        }
}

/* DUTwoBodyEwaldRecStd, denergy.F90:1275-1337 */
static void du_ewald_rec_std(orc_sys *s) {
    int kn = 0;
    ewald_set_array_tm(s);
    for (int nz = 0; nz <= s->ncut; ++nz) {
        for (int ny = 0; ny <= s->ncut; ++ny) {
            if (ny * ny + nz * nz > s->ncut2) continue;
            for (int ialoc = 1; ialoc <= s->nptm; ++ialoc) {
                int ia = s->ipnptm[ialoc - 1];
                s->eikyzm[ia - 1] = zmul(zconj(EIK(s->eiky, ia, ny)), EIK(s->eikz, ia, nz));
                s->eikyzp[ia - 1] = zmul(EIK(s->eiky, ia, ny), EIK(s->eikz, ia, nz));
                s->eikyzmtm[ialoc - 1] = zmul(zconj(EIKTM(s->eikytm, ialoc, ny)), EIKTM(s->eikztm, ialoc, nz));
                s->eikyzptm[ialoc - 1] = zmul(EIKTM(s->eikytm, ialoc, ny), EIKTM(s->eikztm, ialoc, nz));
            }
            for (int nx = 0; nx <= s->ncut; ++nx) {
                if (nx * nx + ny * ny + nz * nz > s->ncut2) continue;
                if (nx == 0 && ny == 0 && nz == 0) continue;
                kn = kn + 1;
                zc *St = &s->sumeikrtm[(size_t)(kn - 1) * 4], *S = &s->sumeikr[(size_t)(kn - 1) * 4];
                for (int c = 0; c < 4; ++c) St[c] = S[c];
                for (int ialoc = 1; ialoc <= s->nptm; ++ialoc) {
                    int ia = s->ipnptm[ialoc - 1];
                    zc ext = EIKTM(s->eikxtm, ialoc, nx), ex = EIK(s->eikx, ia, nx);
                    double q = AZ(ia);
                    St[0] = zadd(St[0], zscale(q, zsub(zmul(zconj(ext), s->eikyzmtm[ialoc - 1]), zmul(zconj(ex), s->eikyzm[ia - 1]))));
                    St[1] = zadd(St[1], zscale(q, zsub(zmul(zconj(ext), s->eikyzptm[ialoc - 1]), zmul(zconj(ex), s->eikyzp[ia - 1]))));
                    St[2] = zadd(St[2], zscale(q, zsub(zmul(ext, s->eikyzmtm[ialoc - 1]), zmul(ex, s->eikyzm[ia - 1]))));
                    St[3] = zadd(St[3], zscale(q, zsub(zmul(ext, s->eikyzptm[ialoc - 1]), zmul(ex, s->eikyzp[ia - 1]))));
                }
                double termnew = St[0].re * St[0].re + St[0].im * St[0].im + St[1].re * St[1].re + St[1].im * St[1].im
                               + St[2].re * St[2].re + St[2].im * St[2].im + St[3].re * St[3].re + St[3].im * St[3].im;
                double termold = S[0].re * S[0].re + S[0].im * S[0].im + S[1].re * S[1].re + S[1].im * S[1].im
                               + S[2].re * S[2].re + S[2].im * S[2].im + S[3].re * S[3].re + S[3].im * S[3].im;
                double term = s->kfac[kn - 1] * (termnew - termold);
                s->du_rec = s->du_rec + term;
            }
        }
    }
}

/* DUTwoBodyEwaldRecSPM, denergy.F90:1413-1495 */
static int du_ewald_rec_spm(orc_sys *s) {
    int order = s->order, *S3 = s->s, n = s->nmesh, nh = n / 2 + 1;
    s->urecnew = Zero;
    memcpy(s->QmeshTM, s->Qmesh, sizeof(double) * (size_t)n * n * n);
    for (int ialoc = 1; ialoc <= s->nptm; ++ialoc) {
        int ia = s->ipnptm[ialoc - 1];
        const double *rt = &s->rotm[3 * (ialoc - 1)];
        for (int m = 1; m <= 3; ++m) {
            int kmax;
            orc_cardinal_bspline(order, s->dkdr[m - 1] * rt[m - 1], &kmax, &SPL(s->splinetm, 0, m, ialoc), &SPL(s->derivtm, 0, m, ialoc));
            MESHMAX(s->meshmaxtm, m, ialoc) = (kmax + S3[m - 1]) % S3[m - 1];
        }
        for (int iz = 0; iz <= order - 1; ++iz) {
            int nz = (S3[2] + MESHMAX(s->meshmax, 3, ia) - iz) % S3[2];
            double qz = AZ(ia) * SPL(s->spline, iz, 3, ia);
            int nztm = (S3[2] + MESHMAX(s->meshmaxtm, 3, ialoc) - iz) % S3[2];
            double qztm = AZ(ia) * SPL(s->splinetm, iz, 3, ialoc);
            for (int iy = 0; iy <= order - 1; ++iy) {
                int ny = (S3[1] + MESHMAX(s->meshmax, 2, ia) - iy) % S3[1];
                double qyz = qz * SPL(s->spline, iy, 2, ia);
                int nytm = (S3[1] + MESHMAX(s->meshmaxtm, 2, ialoc) - iy) % S3[1];
                double qyztm = qztm * SPL(s->splinetm, iy, 2, ialoc);
                for (int ix = 0; ix <= order - 1; ++ix) {
                    int nx = (S3[0] + MESHMAX(s->meshmax, 1, ia) - ix) % S3[0];
                    double q = qyz * SPL(s->spline, ix, 1, ia);
                    int nxtm = (S3[0] + MESHMAX(s->meshmaxtm, 1, ialoc) - ix) % S3[0];
                    double qtm = qyztm * SPL(s->splinetm, ix, 1, ialoc);
                    QM(s->QmeshTM, nx, ny, nz) = QM(s->QmeshTM, nx, ny, nz) - q;
                    QM(s->QmeshTM, nxtm, nytm, nztm) = QM(s->QmeshTM, nxtm, nytm, nztm) + qtm;
                }
            }
        }
    }
    if (orc_fft_r2c_3d(n, s->QmeshTM, s->FQmesh)) return MG_ERR_ALLOC;
    zc *F = (zc *)s->FQmesh;
#define FQ(x, y, z) F[((size_t)(z) * n + (y)) * nh + (x)]
    for (int nz = 0; nz <= n / 2; ++nz) {
        int nza = (n - nz) % n;
        for (int ny = 0; ny <= n / 2; ++ny) {
            int nya = (n - ny) % n;
            for (int nx = 0; nx <= n / 2; ++nx) {
                zc v[4] = {FQ(nx, ny, nz), FQ(nx, ny, nza), FQ(nx, nya, nz), FQ(nx, nya, nza)};
                double Qsum = Zero;
                for (int c = 0; c < 4; ++c) Qsum = Qsum + (v[c].re * v[c].re + v[c].im * v[c].im);
                s->urecnew = s->urecnew + Qsum * s->energyfac[((size_t)nz * nh + ny) * nh + nx];
            }
        }
    }
#undef FQ
    s->du_rec = s->urecnew - s->urecold;
    return 0;
}

/* DUTwoBodyEwaldSurf, denergy.F90:1504-1548 */
static void du_ewald_surf(orc_sys *s) {
    double fac = TwoPi / (Three * s->vol);
    double sx = Zero, sy = Zero, sz = Zero;
    for (int ia = 1; ia <= s->np; ++ia) sx = sx + AZ(ia) * RO(1, ia);
    for (int ia = 1; ia <= s->np; ++ia) sy = sy + AZ(ia) * RO(2, ia);
    for (int ia = 1; ia <= s->np; ++ia) sz = sz + AZ(ia) * RO(3, ia);
    double sxt = sx, syt = sy, szt = sz;
    for (int ialoc = 1; ialoc <= s->nptm; ++ialoc) {
        int ia = s->ipnptm[ialoc - 1];
        const double *rt = &s->rotm[3 * (ialoc - 1)];
        sxt = sxt + AZ(ia) * (rt[0] - RO(1, ia));
        syt = syt + AZ(ia) * (rt[1] - RO(2, ia));
        szt = szt + AZ(ia) * (rt[2] - RO(3, ia));
    }
    double term = fac * ((sxt * sxt + syt * syt + szt * szt) - (sx * sx + sy * sy + sz * sz));
    s->du_rec = s->du_rec + term;
}

/* position of particle jp (1-based) in the moving list, 0-based (iptmpn) */
static int iptmpn(const orc_sys *s, int jp) {
    for (int i = 0; i < s->nptm; ++i)
        if (s->ipnptm[i] == jp) return i;
    return -1;
}

#define ROTM(i) (&s->rotm[3 * (i)])
#define ROP(ip) (&s->ro[3 * ((ip) - 1)])

/* DUBondSub: bond between moving particle iploc (old ro(ip)) and a
   neighbour at ronew (new) / roold (old), parameters of bond b */
static void du_bond_sub(orc_sys *s, int iploc, int ip, int b, const double *ronew, const double *roold) {
    double dx = ROTM(iploc)[0] - ronew[0], dy = ROTM(iploc)[1] - ronew[1], dz = ROTM(iploc)[2] - ronew[2], r2new;
    pbcr2(s, &dx, &dy, &dz, &r2new);
    dx = ROP(ip)[0] - roold[0];
    dy = ROP(ip)[1] - roold[1];
    dz = ROP(ip)[2] - roold[2];
    double r2old;
    pbcr2(s, &dx, &dy, &dz, &r2old);
    s->du_bond = s->du_bond + s->bond_k[b] * (powi(sqrt(r2new) - s->bond_eq[b], s->bond_p[b]) -
                                              powi(sqrt(r2old) - s->bond_eq[b], s->bond_p[b]));
}

/* angle_rad, molaux.F90:836-846 */
static double angle_rad(double x1, double y1, double z1, double x2, double y2, double z2) {
    double term1 = x1 * x2 + y1 * y2 + z1 * z2;
    double term2 = pow2(x1) + pow2(y1) + pow2(z1);
    double term3 = pow2(x2) + pow2(y2) + pow2(z2);
    double term = term1 / sqrt(term2 * term3);
    return acos(fmax(-One, fmin(term, One)));
}

/* DUAngleSub: angle a (vertex 0) from old to new positions */
static void du_angle_sub(orc_sys *s, int a, const double *nm, const double *n0, const double *np_,
                         const double *om, const double *o0, const double *op) {
    double dxm = n0[0] - nm[0], dym = n0[1] - nm[1], dzm = n0[2] - nm[2];
    pbc(s, &dxm, &dym, &dzm);
    double dxp = np_[0] - n0[0], dyp = np_[1] - n0[1], dzp = np_[2] - n0[2];
    pbc(s, &dxp, &dyp, &dzp);
    double thetanew = angle_rad(-dxm, -dym, -dzm, dxp, dyp, dzp);
    dxm = o0[0] - om[0]; dym = o0[1] - om[1]; dzm = o0[2] - om[2];
    pbc(s, &dxm, &dym, &dzm);
    dxp = op[0] - o0[0]; dyp = op[1] - o0[1]; dzp = op[2] - o0[2];
    pbc(s, &dxp, &dyp, &dzp);
    double thetaold = angle_rad(-dxm, -dym, -dzm, dxp, dyp, dzp);
    s->du_angle = s->du_angle + s->angle_k[a] * (powi(thetanew - s->angle_eq[a], s->angle_p[a]) -
                                                 powi(thetaold - s->angle_eq[a], s->angle_p[a]));
}

/* DUBond (denergy.F90:2893-2955) and DUAngle (:2962-3040): the bonds and
   angles of the moving chain segments.  A moving neighbour's new position is
   taken from the previous / next entry of the moving list inside the list
   and from its own entry at the ends, as the reference does (its routines
   assume the moving segments form one string). */
static void du_bonded(orc_sys *s) {
    s->du_bond = Zero;
    s->du_angle = Zero;
    int nptm = s->nptm;
    for (int iploc = 0; iploc < nptm; ++iploc) {
        int ip = s->ipnptm[iploc];
        int jm = s->nn_lo[ip - 1], jp = s->nn_up[ip - 1];
        if (jm == 0 && jp == 0) continue;   /* not a chain segment */
        if (jm != 0) {
            int b = s->bond_lo[ip - 1];
            if (!s->lptm[jm - 1]) du_bond_sub(s, iploc, ip, b, ROP(jm), ROP(jm));
            else du_bond_sub(s, iploc, ip, b, iploc > 0 ? ROTM(iploc - 1) : ROTM(iptmpn(s, jm)), ROP(jm));
        }
        if (jp != 0 && !s->lptm[jp - 1]) du_bond_sub(s, iploc, ip, s->bond_up[ip - 1], ROP(jp), ROP(jp));
    }
    s->du_tot = s->du_tot + s->du_bond;
    int any = 0;
    for (int a = 0; a < s->nangle; ++a) any |= s->angle_k[a] != Zero;
    if (!any) return;
    for (int iploc = 0; iploc < nptm; ++iploc) {
        int ip = s->ipnptm[iploc];
        int jm = s->nn_lo[ip - 1], jp = s->nn_up[ip - 1];
        if (jm == 0 && jp == 0) continue;
        int jmm = jm ? s->nn_lo[jm - 1] : 0, jpp = jp ? s->nn_up[jp - 1] : 0;
        if (jm != 0 && jp != 0 && s->angle_at[ip - 1] >= 0) {
            int a = s->angle_at[ip - 1];
            const double *nm, *np_;
            if (s->lptm[jm - 1]) {
                if (s->lptm[jp - 1]) {
                    int inner = iploc > 0 && iploc < nptm - 1;
                    nm = inner ? ROTM(iploc - 1) : ROTM(iptmpn(s, jm));
                    np_ = inner ? ROTM(iploc + 1) : ROTM(iptmpn(s, jp));
                } else {
                    nm = iploc > 0 ? ROTM(iploc - 1) : ROTM(iptmpn(s, jm));
                    np_ = ROP(jp);
                }
            } else {
                nm = ROP(jm);
                np_ = s->lptm[jp - 1] ? (iploc < nptm - 1 ? ROTM(iploc + 1) : ROTM(iptmpn(s, jp))) : ROP(jp);
            }
            du_angle_sub(s, a, nm, ROTM(iploc), np_, ROP(jm), ROP(ip), ROP(jp));
        }
        if (jm != 0 && jmm != 0 && !s->lptm[jm - 1] && s->angle_at[jm - 1] >= 0)
            du_angle_sub(s, s->angle_at[jm - 1], ROP(jmm), ROP(jm), ROTM(iploc), ROP(jmm), ROP(jm), ROP(ip));
        if (jp != 0 && jpp != 0 && !s->lptm[jp - 1] && s->angle_at[jp - 1] >= 0)
            du_angle_sub(s, s->angle_at[jp - 1], ROTM(iploc), ROP(jp), ROP(jpp), ROP(ip), ROP(jp), ROP(jpp));
    }
    s->du_tot = s->du_tot + s->du_angle;
}

/* DUTotal, denergy.F90:98-215 with DUTwoBody (:246-286), DUTwoBodyEwald
   (:1240-1270), DUBond and DUAngle; charged monoatomic branch. */
int orc_dutotal(orc_sys *s, int32_t nptm, const int32_t *ipnptm, const double *rotm,
                double *du_twob, double *du_rec, double *du_tot, int32_t *lhsoverlap) {
    if (nptm < 1 || nptm > s->np) return MG_ERR_ARG;
    if (s->txintlist == MG_VLIST && !s->nneighpn) return MG_ERR_STATE;
    if (s->txintlist == MG_CELLLIST && !s->cell) return MG_ERR_STATE;
    if (s->ewald != MG_EWALD_NONE && !s->have_rec) return MG_ERR_STATE;
    for (int i = 0; i < s->nptm; ++i) s->lptm[s->ipnptm[i] - 1] = 0;
    s->nptm = nptm;
    for (int i = 0; i < nptm; ++i) {
        s->ipnptm[i] = ipnptm[i];
        s->lptm[ipnptm[i] - 1] = 1;
        for (int m = 0; m < 3; ++m) s->rotm[3 * i + m] = rotm[3 * i + m];
    }
    s->du_tot = Zero;
    s->du_rec = Zero;
    s->du_bond = Zero;
    s->du_angle = Zero;
    double du_tw[64];
    int ntw = s->nptpt + 1;
    for (int k = 0; k < ntw && k < 64; ++k) du_tw[k] = Zero;
    int err = 0;
    int overlap = utwobody_new(s, &err);
    if (err) return err;
    s->trial_ok = 0;
    if (!overlap) {
        for (int k = 0; k < ntw; ++k) du_tw[k] = du_tw[k] + s->utwobnew[k];
        int st = utwobody_old(s);
        if (st < 0) return st;
        if (st == 1) return MG_ERR_TABLE_UNDERRUN;
        for (int k = 0; k < ntw; ++k) du_tw[k] = du_tw[k] - s->utwobold[k];
        s->du_tot = s->du_tot + du_tw[0];
        if (s->ewald != MG_EWALD_NONE) {
            if (s->ewald == MG_EWALD_STD) du_ewald_rec_std(s);
            else { st = du_ewald_rec_spm(s); if (st) return st; }
            if (s->lsurf) du_ewald_surf(s);
            s->du_rec = s->EpsiFourPi * s->du_rec;
            s->du_tot = s->du_tot + s->du_rec;
        }
        if (s->nbond > 0) du_bonded(s);
        s->trial_ok = 1;
    }
    if (du_twob) for (int k = 0; k < ntw; ++k) du_twob[k] = overlap ? Zero : du_tw[k];
    if (du_rec) *du_rec = s->du_rec;
    if (du_tot) *du_tot = s->du_tot;
    if (lhsoverlap) *lhsoverlap = overlap;
    return 0;
}

/* MCUpdate, mc.F90:5203-5235: ro = rotm, EwaldUpdateArray
   (denergy.F90:1776-1820), UpdateCellIp. */
int orc_accept(orc_sys *s) {
    if (!s->trial_ok) return MG_ERR_STATE;
    if (s->ewald == MG_EWALD_STD) {
        for (int icut = 0; icut <= s->ncut; ++icut)
            for (int ialoc = 1; ialoc <= s->nptm; ++ialoc) {
                int ia = s->ipnptm[ialoc - 1];
                EIK(s->eikx, ia, icut) = EIKTM(s->eikxtm, ialoc, icut);
                EIK(s->eiky, ia, icut) = EIKTM(s->eikytm, ialoc, icut);
                EIK(s->eikz, ia, icut) = EIKTM(s->eikztm, ialoc, icut);
            }
        memcpy(s->sumeikr, s->sumeikrtm, sizeof(zc) * 4 * (size_t)s->nkvec);
    } else if (s->ewald == MG_EWALD_SPM) {
        memcpy(s->Qmesh, s->QmeshTM, sizeof(double) * (size_t)s->nmesh * s->nmesh * s->nmesh);
        s->urecold = s->urecnew;
        for (int ialoc = 1; ialoc <= s->nptm; ++ialoc) {
            int ia = s->ipnptm[ialoc - 1];
            for (int m = 1; m <= 3; ++m) {
                for (int i = 0; i < s->order; ++i) {
                    SPL(s->spline, i, m, ia) = SPL(s->splinetm, i, m, ialoc);
                    SPL(s->deriv, i, m, ia) = SPL(s->derivtm, i, m, ialoc);
                }
                MESHMAX(s->meshmax, m, ia) = MESHMAX(s->meshmaxtm, m, ialoc);
            }
        }
    }
    for (int ialoc = 1; ialoc <= s->nptm; ++ialoc) {
        int ip = s->ipnptm[ialoc - 1];
        for (int m = 1; m <= 3; ++m) RO(m, ip) = s->rotm[3 * (ialoc - 1) + m - 1];
        if (s->txintlist == MG_CELLLIST) {
            int st = update_cell_ip(s, ip);
            if (st) return st;
        }
    }
    s->u_tot = s->u_tot + s->du_tot;
    s->u_bond = s->u_bond + s->du_bond;
    s->u_angle = s->u_angle + s->du_angle;
    s->trial_ok = 0;
    return 0;
}

/* ======================================================================
 * md.F90 / bd.F90
 * ====================================================================== */

int orc_md_setup(orc_sys *s, double tstep, const double *massip, const double *rod, const double *rodd) {
    size_t n3 = (size_t)3 * s->np;
    if (!s->massip) {
        s->massip = xcalloc(s->np, sizeof(double));
        s->rod = xcalloc(n3, sizeof(double));
        s->rodd = xcalloc(n3, sizeof(double));
        s->roddo = xcalloc(n3, sizeof(double));
    }
    s->tstep = tstep;
    memcpy(s->massip, massip, sizeof(double) * s->np);
    memcpy(s->rod, rod, sizeof(double) * n3);
    memcpy(s->rodd, rodd, sizeof(double) * n3);
    return 0;
}

/* VelVer, md.F90:252-420, with GetLinAcc (md.F90:601-625) and the list check
   of NListDriver(iSimulationStep) after the step. */
int orc_md_run(orc_sys *s, int32_t nstep, double *forceo, double *uout, double *rod, double *rodd) {
    if (!s->massip) return MG_ERR_STATE;
    double tstep = s->tstep;
    for (int step = 0; step < nstep; ++step) {
        double fac = Half * tstep * tstep;
        for (int ip = 1; ip <= s->np; ++ip) {
            double *d = &s->drostep[3 * (ip - 1)];
            double *v = &s->rod[3 * (ip - 1)], *a = &s->rodd[3 * (ip - 1)];
            d[0] = tstep * v[0] + fac * a[0];
            d[1] = tstep * v[1] + fac * a[1];
            d[2] = tstep * v[2] + fac * a[2];
            RO(1, ip) = RO(1, ip) + d[0];
            RO(2, ip) = RO(2, ip) + d[1];
            RO(3, ip) = RO(3, ip) + d[2];
            pbc(s, &RO(1, ip), &RO(2, ip), &RO(3, ip));
        }
        int st = utotal_core(s);
        if (st) return st;
        for (int i = 0; i < 3 * s->np; ++i) s->roddo[i] = s->rodd[i];
        for (int ip = 1; ip <= s->np; ++ip)
            for (int m = 0; m < 3; ++m)
                s->rodd[3 * (ip - 1) + m] = s->massip[ip - 1] * s->forceo[3 * (ip - 1) + m];
        for (int i = 0; i < 3 * s->np; ++i) s->rod[i] = s->rod[i] + Half * tstep * (s->rodd[i] + s->roddo[i]);
        int32_t rebuilt;
        st = orc_nlist_update(s, s->drostep, &rebuilt);
        if (st) return st;
    }
    copy_out(s, forceo, NULL, uout);
    if (rod) memcpy(rod, s->rod, sizeof(double) * 3 * s->np);
    if (rodd) memcpy(rodd, s->rodd, sizeof(double) * 3 * s->np);
    return 0;
}

int orc_bd_setup(orc_sys *s, const double *fac1, const double *fac2, int32_t iseed) {
    /* a seed that is 0 modulo 2^31 never leaves 0 and GauRandom would loop forever */
    if (((uint32_t)iseed & 0x7fffffffu) == 0) return MG_ERR_ARG;
    if (!s->fac1) { s->fac1 = xcalloc(s->npt, sizeof(double)); s->fac2 = xcalloc(s->npt, sizeof(double)); }
    memcpy(s->fac1, fac1, sizeof(double) * s->npt);
    memcpy(s->fac2, fac2, sizeof(double) * s->npt);
    s->iseed = iseed;
    s->gflag = 1;
    s->gsave = 0;
    s->bd_have_force = 0;
    return 0;
}

/* BDDriver(iSimulationStep), bd.F90:53-59: BDStep (bd.F90:120-155) then
   UTotal, then the list check. */
int orc_bd_run(orc_sys *s, int32_t nstep, double *forceo, double *uout) {
    if (!s->fac1) return MG_ERR_STATE;
    if (!s->bd_have_force) {
        int st = utotal_core(s);
        if (st) return st;
        s->bd_have_force = 1;
    }
    for (int step = 0; step < nstep; ++step) {
        for (int ip = 1; ip <= s->np; ++ip) {
            int ipt = IPTPN(ip);
            double *d = &s->drostep[3 * (ip - 1)];
            const double *f = &s->forceo[3 * (ip - 1)];
            for (int m = 0; m < 3; ++m)
                d[m] = s->fac1[ipt - 1] * f[m] + s->fac2[ipt - 1] * orc_gau_random(&s->iseed, &s->gflag, &s->gsave);
            RO(1, ip) = RO(1, ip) + d[0];
            RO(2, ip) = RO(2, ip) + d[1];
            RO(3, ip) = RO(3, ip) + d[2];
            pbc(s, &RO(1, ip), &RO(2, ip), &RO(3, ip));
        }
        int st = utotal_core(s);
        if (st) return st;
        int32_t rebuilt;
        st = orc_nlist_update(s, s->drostep, &rebuilt);
        if (st) return st;
    }
    copy_out(s, forceo, NULL, uout);
    return 0;
}

int orc_bd_get_seed(orc_sys *s, int32_t *iseed) {
    *iseed = s->iseed;
    return 0;
}
