/*
 * molsim_oracle.h — CPU oracle for the MOLSIM force/energy hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the
 * reference's Fortran (joakimstenhammar/molsim, the Src directory) used to check the
 * GPU library.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline may load it; the product (molsim_gb300/) never does.
 *
 * Parity status: the reference cannot be compiled here (it is Fortran and
 * this image has no Fortran compiler or FFTW) and it ships no numeric
 * outputs, so this oracle is pinned against known answers instead of
 * reference outputs: erf (math library), the NaCl Madelung constant
 * (standard and SPME Ewald), numpy's FFT, the reference's own table
 * tolerance check, brute-force list completeness and finite-difference
 * forces.  Reference-output parity is therefore unpinned.
 *
 * It takes the same mg_params description as the library (the C ABI in
 * include/molsim_gb300.h) so that both see identical inputs.
 */
#ifndef MOLSIM_ORACLE_H
#define MOLSIM_ORACLE_H

#include "../include/molsim_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sys orc_sys;

/* numerical library (mollib.F90, potential.F90) */
double orc_erf2(double x);
void   orc_calc_ewald_ufac(double r1, double ualpha, double *c0, double *c1, double *c2);
int    orc_cardinal_bspline(int order, double pos, int *kmax, double *values, double *derivs);
double orc_random(int32_t *idum);
double orc_gau_random(int32_t *iseed, int32_t *flag, double *save);
int    orc_rcut_to_alpha(double uewaldtol, double rcut, double q2sum, double boxlenshort,
                         double epsi_four_pi, double *ualpha);
int    orc_pot_twobody_tab(const mg_pot_params *pp, double *ubuf, int32_t nbuf_cap,
                           int32_t *nbuf_used, int32_t *iubuflow, double *r2umin,
                           int32_t *nugrid);
void   orc_pot_1_6_12(const mg_pot_params *pp, int iat, int jat, double r1,
                      double *u0, double *u1, double *u2);

/* FFT with FFTW's conventions (forward e^{-i}, unnormalised), mesh q[z][y][x] */
/* threads standing in for the reference's MPI ranks (oracle_par.h); 1 = serial */
int orc_set_threads(int n);

int orc_fft_r2c_3d(int n, const double *q, double *fq /* (n/2+1)*n*n complex */);
int orc_fft_c2r_3d(int n, const double *fq, double *q);

/* system */
int  orc_create(const mg_params *p, orc_sys **s);
void orc_destroy(orc_sys *s);
int  orc_set_positions(orc_sys *s, const double *ro);
int  orc_get_positions(orc_sys *s, double *ro);
int  orc_nlist_set(orc_sys *s);
int  orc_nlist_update(orc_sys *s, const double *drostep, int32_t *rebuilt);
int  orc_nlist_get(orc_sys *s, int32_t *nneighpn, int32_t *jpnlist, int32_t maxnneigh);
int  orc_celllist_get(orc_sys *s, int32_t *ncell, int32_t *cellip);
int  orc_celllist_test(orc_sys *s);   /* TestCellList: brute-force completeness */
int  orc_utotal(orc_sys *s, double *forceo, double *u_twob, double *uout);
int  orc_energy_terms(orc_sys *s, double *terms);
int  orc_dutotal(orc_sys *s, int32_t nptm, const int32_t *ipnptm, const double *rotm,
                 double *du_twob, double *du_rec, double *du_tot, int32_t *lhsoverlap);
int  orc_accept(orc_sys *s);
int  orc_md_setup(orc_sys *s, double tstep, const double *massip, const double *rod,
                  const double *rodd);
int  orc_md_run(orc_sys *s, int32_t nstep, double *forceo, double *uout, double *rod,
                double *rodd);
int  orc_bd_setup(orc_sys *s, const double *fac1, const double *fac2, int32_t iseed);
int  orc_bd_run(orc_sys *s, int32_t nstep, double *forceo, double *uout);
int  orc_bd_get_seed(orc_sys *s, int32_t *iseed);
/* UTwoBodyP (energy.F90:786-896) for polyatomic particles: no state; the
   arguments as mg_poly_utwobody's, with maxnneigh the list's leading size */
int  orc_poly_utwobody(const mg_poly_params *p, int32_t maxnneigh, const double *ro, const double *r,
                       const int32_t *nneighpn, const int32_t *jpnlist, double *force, double *u_twob,
                       double *virial);
/* one single-particle polyatomic trial (UTwoBodyPNew/UTwoBodyPOld,
   denergy.F90:937-1231, nptm = 1): du_twob[nptpt+1] and the overlap flag */
int  orc_poly_dutwobody(const mg_poly_params *p, int32_t maxnneigh, const double *ro, const double *r,
                        const int32_t *nneighpn, const int32_t *jpnlist, int32_t ip, const double *rotm,
                        const double *rtm, double *du_twob, int32_t *lhsoverlap);
/* UTwoBodyPNew/Old for nptm moving particles with the pairs among them
   (denergy.F90:937-1231), arguments as mg_poly_dutwobody_multi's */
int  orc_poly_dutwobody_multi(const mg_poly_params *p, int32_t maxnneigh, const double *ro, const double *r,
                              const int32_t *nneighpn, const int32_t *jpnlist, int32_t nptm,
                              const int32_t *ipnptm, const double *rotm, const double *rtm, double *du_twob,
                              int32_t *lhsoverlap);
/* the end of UTotal for polyatomic particles (energy.F90:405-427),
   arguments as mg_poly_epilogue's */
int  orc_poly_epilogue(const mg_poly_params *p, const double *ro, const double *r, const double *force,
                       const double *torque, double force_fac, double *forceo, double *torqueo,
                       double *virmolecule);
/* UDipole with Ewald (energy.F90:1476-2295), arguments as the library's
   mg_poly_udipole_real/_self/_finish and mg_dipole_ewald (on an atom handle) */
int  orc_poly_udipole_real(const mg_poly_params *p, int32_t maxnneigh, const double *ro, const double *r,
                           const double *dip, const int32_t *nneighpn, const int32_t *jpnlist, double *potstat,
                           double *estat, double *efg, double *virelec, double *u_real);
int  orc_poly_udipole_self(const mg_poly_params *p, const double *r, const double *dip, int32_t lsurf,
                           double *potstat, double *estat, double *efg, double *virelec);
int  orc_poly_udipole_finish(const mg_poly_params *p, const double *dip, const double *potstat,
                             const double *estat, const double *efg, double *force, double *torque,
                             double *u_stat);
int  orc_dipole_ewald(orc_sys *s, const double *dip, double *potstat, double *estat, double *efg,
                      double *virelec);
/* rigid-body VelVer (md.F90:252-420) in parts, the state held by the caller */
int  orc_angvel_to_quavel(int32_t np, const double *qua, const double *angvelo, double *quad);
int  orc_rigid_move(int32_t np, double tstep, const double *boxlen, double *ro, double *qua, const double *rod,
                    const double *rodd, const double *quad, const double *quadd, double *drostep, double *ori);
int  orc_rigid_kick(int32_t np, double tstep, double tvvite, int32_t nvvite, const double *massip,
                    const double *momp, const double *qua, const double *forceo, const double *torqueo,
                    double *rod, double *rodd, double *quad, double *quadd, double *angvelo);
/* the molecular part of UEwaldSelf (energy.F90:1301-1345), arguments as
   mg_poly_ewald_intra's */
int  orc_poly_ewald_intra(const mg_poly_params *p, const double *r, double *force, double *u_rec);
/* the SPME charge mesh after the last spread (before the FFT), n^3 doubles */
int  orc_get_qmesh(orc_sys *s, double *q);

#ifdef __cplusplus
}
#endif
#endif
