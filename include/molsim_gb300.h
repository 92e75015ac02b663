/*
 * molsim_gb300.h — C ABI of the GB300 force/energy hot path of MOLSIM.
 *
 * The reference (MOLSIM, Fortran 90) exposes this path as argument-less
 * subroutines that work on module globals.  Each entry point below replaces
 * one of them; the comment names the subroutine it stands in for
 * (file:line in the reference's Src/ directory).  A Fortran caller binds
 * these with ISO_C_BINDING; a Python caller with ctypes (molsim_gb300/).
 *
 * Conventions
 *   - Every function returns an int status: MG_OK (0) or a negative MG_ERR_*.
 *     The text of the last error (with the offending particle index where
 *     there is one) is read with mg_last_error().  Where the reference calls
 *     Stop(), the library returns the matching error instead; a hard-core
 *     overlap in a trial move is a result (lhsoverlap), not an error.
 *   - Arrays use the reference's layouts: positions/forces ro(3,np) are
 *     column-major, i.e. x,y,z of particle 1, then particle 2 ...
 *     Particle, type and pair indices are 1-based, as in the reference.
 *   - The library copies every input array it keeps; it never frees or
 *     retains caller memory.  One handle = one CUDA stream on the current
 *     device; a handle is not thread safe.  Calls are synchronous: outputs
 *     are valid when the call returns.
 */
#ifndef MOLSIM_GB300_H
#define MOLSIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MG_ABI_VERSION 2

/* ---- status codes ------------------------------------------------------ */
#define MG_OK                   0
#define MG_ERR_ARG             -1  /* bad argument or parameter combination      */
#define MG_ERR_CUDA            -2  /* a CUDA runtime call failed                 */
#define MG_ERR_TABLE_UNDERRUN  -3  /* r2 < r2umin   (energy.F90:478, Stop)       */
#define MG_ERR_NEIGH_OVERFLOW  -4  /* nneighpn > maxnneigh (nlist.F90:752, Stop) */
#define MG_ERR_NAN             -5  /* non-finite force or energy                 */
#define MG_ERR_TIMEOUT         -6  /* a bounded device wait ran out              */
#define MG_ERR_IBUF            -7  /* ibuf > nbuf   (energy.F90:484, Stop)       */
#define MG_ERR_TABLE           -8  /* table build failed (potential.F90:1121,1129) */
#define MG_ERR_STATE           -9  /* call made out of order                     */
#define MG_ERR_ALLOC          -10  /* device or host allocation failed           */
#define MG_ERR_UNSUPPORTED    -11  /* option outside the built path              */
#define MG_ERR_CELL           -12  /* particle outside the cell grid             */

/* ---- option values ----------------------------------------------------- */
enum { MG_EWALD_NONE = 0, MG_EWALD_STD = 1, MG_EWALD_SPM = 2 };   /* txewaldrec */
enum { MG_VLIST = 0, MG_CELLLIST = 1 };                           /* txintlist  */
enum { MG_MD = 0, MG_MC = 1, MG_BD = 2 };                         /* lmd/lmc/lbd */
enum { MG_FP64 = 0, MG_MIXED = 1 };                               /* precision form */

/*
 * System description: the subset of MolModule (mol.F90:1087-1218) and
 * EnergyModule (energy.F90:98-256) that the hot path reads, for a charged
 * monoatomic system in a rectangular periodic box (txbc='xyz').
 */
typedef struct mg_params {
    int32_t abi_version;      /* must be MG_ABI_VERSION                          */
    int32_t np;               /* number of particles (monoatomic: na == np)     */
    int32_t npt;              /* number of particle types                       */
    int32_t nptpt;            /* number of type pairs, npt*(npt+1)/2            */
    const int32_t *iptpn;     /* [np] type of each particle, 1..npt             */
    const int32_t *iptpt;     /* [npt*npt] iptpt(ipt,jpt), column-major, 1..nptpt */
    const double  *az;        /* [np] charge of each particle (units of e)      */

    /* tabulated two-body potential (PotTwoBodyTab1, potential.F90:868) */
    int32_t nbuf;             /* number of doubles in ubuf                      */
    const double  *ubuf;      /* [nbuf] 12 doubles per interval                 */
    const int32_t *iubuflow;  /* [nptpt] 1-based start of each pair's table     */
    const double  *r2umin;    /* [nptpt] lower end of each table                */
    const double  *r2atat;    /* [nptpt] hard-core distance squared             */

    double  boxlen[3];        /* box edges (Angstrom); box centred at origin    */
    double  rcut;             /* real-space cutoff                              */
    double  drnlist;          /* Verlet skin                                    */
    int32_t txintlist;        /* MG_VLIST or MG_CELLLIST                        */
    int32_t mode;             /* MG_MD, MG_MC or MG_BD (list kind and MC state) */
    int32_t form;             /* MG_FP64 or MG_MIXED                            */
    int32_t maxnneigh;        /* neighbour capacity per particle (0 = automatic) */

    /* Ewald summation (EwaldSetup, energy.F90:6601) */
    int32_t ewald;            /* MG_EWALD_NONE / _STD / _SPM                    */
    double  ualpha;           /* Ewald damping parameter (1/Angstrom)           */
    int32_t ncut;             /* std: k-vector cutoff                           */
    int32_t ncutregion_cube;  /* std: 0 = 'sphere', 1 = 'cube'                  */
    int32_t order;            /* SPME: B-spline order                           */
    int32_t nmesh;            /* SPME: mesh points per edge (even)              */
    int32_t lsurf;            /* 1 = add the surface term (UEwaldSurf)          */
    double  epsi_four_pi;     /* EpsiFourPi = Epsi0FourPi/relpermitt            */
    double  force_fac;        /* (sclene/scllen)/sclfor, force -> forceo        */

    /* chain bonds (UBond, energy.F90:5335): u = k*(r-eq)**p per bond */
    int32_t nbond;
    const int32_t *bond_ip;   /* [nbond] first particle, 1-based                */
    const int32_t *bond_jp;   /* [nbond] second particle, 1-based               */
    const double  *bond_k;    /* [nbond]                                        */
    const double  *bond_eq;   /* [nbond]                                        */
    const int32_t *bond_p;    /* [nbond] integer power                          */

    /* chain angles (UAngle, energy.F90:5409): u = k*(theta-eq)**p per angle
       jm-ip-jp, theta the angle at ip; in the reference's order (chains,
       then segments 2..npct-1).  No contribution to the virial. */
    int32_t nangle;
    const int32_t *angle_jm;  /* [nangle] previous segment, 1-based             */
    const int32_t *angle_ip;  /* [nangle] vertex, 1-based                       */
    const int32_t *angle_jp;  /* [nangle] next segment, 1-based                 */
    const double  *angle_k;   /* [nangle]                                       */
    const double  *angle_eq;  /* [nangle] radians                               */
    const int32_t *angle_p;   /* [nangle] integer power                         */
} mg_params;

/* Parameters of the (1,6,12) potential table (Pot_1_6_12, potential.F90:1349). */
typedef struct mg_pot_params {
    int32_t npt;
    const int32_t *iptpt;     /* [npt*npt] column-major, 1-based                */
    const double *zat;        /* [npt] charge per type                          */
    const double *sigat;      /* [npt] LJ sigma per type                        */
    const double *epsat;      /* [npt] LJ epsilon per type                      */
    double rcut;
    double ualpha;
    double epsi_four_pi;
    int32_t lcharge_ewald;    /* 1: charges with Ewald (CalcEwaldUfac factors)  */
    int32_t lljcut;           /* 1: truncate LJ at ljrcut*sig and shift         */
    double ljrcut;
    double ljushift;
    double r2uminin;          /* reference default 0.1                          */
    double utoltab, ftoltab;  /* reference default 1e-5 (a single-precision literal) */
    double umaxtab, fmaxtab;  /* reference default 20000                        */
} mg_pot_params;

typedef struct mg_handle mg_handle;

/* ---- library information ----------------------------------------------- */
int         mg_abi_version(void);
const char *mg_status_string(int status);
/* Text of the last error of this handle (NUL-terminated, truncated to n). */
int         mg_last_error(const mg_handle *h, char *buf, size_t n);

/* ---- host set-up (once per parameter set) -------------------------------- */

/* PotTwoBodyTab1/2/3 + SetUBuffer + CheckUBuffer (potential.F90:868-1263) for
 * the (1,6,12) potential.  Writes up to nbuf_cap doubles into ubuf and always
 * sets *nbuf_used; returns MG_ERR_TABLE if the capacity is too small (call
 * again with a larger buffer) or the interval search does not converge. */
int mg_pot_twobody_tab(const mg_pot_params *pp, double *ubuf, int32_t nbuf_cap,
                       int32_t *nbuf_used, int32_t *iubuflow, double *r2umin,
                       int32_t *nugrid);

/* RcutToAlpha (energy.F90:7090-7106): alpha from tolerance and cutoff
 * (iewaldopt = 3, charged system, lq2sum = 0). */
int mg_rcut_to_alpha(double uewaldtol, double rcut, double q2sum,
                     double boxlenshort, double epsi_four_pi, double *ualpha);

/* ---- handle ---------------------------------------------------------------- */

/* Copies the system, builds the Ewald arrays (kfac, or meshfac/energyfac/
 * virfac as EwaldSetup, energy.F90:6601-7018) and allocates device memory. */
int mg_create(const mg_params *p, mg_handle **h);
int mg_destroy(mg_handle *h);

/* ro(3,np): upload positions (the ro array of MolModule). */
int mg_set_positions(mg_handle *h, const double *ro);
int mg_get_positions(mg_handle *h, double *ro);

/* The device 3D FFT alone, to check it against another FFT library.  It
 * replaces the FFTW r2c/c2r pair of SPMFFTRec (energy.F90:6525-6587) around
 * the influence-function multiply of UEwaldRecSPM.  q: an nmesh^3 mesh
 * (x fastest, then y, then z), loaded in the handle's form as the spread
 * would leave it; mult, ew: octant tables [fz][fy][kx] of (nmesh/2+1)^3
 * values, used at fz = min(kz, nmesh-kz), fy = min(ky, nmesh-ky).  Returns
 * phi = c2r(mult * r2c(q)) (unnormalised, nmesh^3) and *esum = the sum of
 * ew |r2c(q)|^2 over the half spectrum (kx <= nmesh/2, all ky, kz).  The
 * handle (an SPME handle) keeps no result: its next UTotal recomputes the
 * meshes. */
int mg_fft_check(mg_handle *h, const double *q, const double *mult, const double *ew,
                 double *phi, double *esum);

/* The reciprocal part of UDipoleEwald (energy.F90:1807-1830) for charges
 * and point dipoles, on an FP64 handle with Ewald whose particles are the
 * atoms (positions from mg_set_positions, charges az): UDipoleEwaldRecStd
 * (energy.F90:1830-2040: structure factors of q + i k.dip, then per atom
 * the potential, field and field gradient of each k-vector) or
 * UDipoleEwaldRecSPM (:2046-2170: the generalized charge mesh through the
 * B-spline derivatives, SPMFFTRec, then the potential, field and field
 * gradient through the first and second derivatives), followed by the
 * atomic part of UDipoleEwaldSelf (:2183-2191).  dip[3*np] in the lab
 * frame; potstat[np], estat[3*np], efg[6*np] and *virelec are added to, as
 * the reference adds to the real-space part (mg_poly_udipole_real). */
int mg_dipole_ewald(mg_handle *h, const double *dip, double *potstat, double *estat, double *efg,
                    double *virelec);

/* ---- neighbour lists (A1-A4) --------------------------------------------- */

/* NList(iWriteInput) (nlist.F90:553-596): builds the Verlet list
 * (SetVListMD / SetVListMC, nlist.F90:724-890) or the cell list
 * (InitCellList(rcut+drnlist) + SetCellList, celllist.F90:76,384). */
int mg_nlist_set(mg_handle *h);

/* NList(iSimulationStep) (nlist.F90:598-621): accumulates drostep(3,np) and
 * rebuilds the Verlet list when sqrt(r2max1)+sqrt(r2max2) > drnlist.
 * drostep may be NULL to use the displacements of the last device step. */
int mg_nlist_update(mg_handle *h, const double *drostep, int32_t *rebuilt);

/* The number of Verlet-list builds since mg_nlist_set, counting that one:
 * VListAver's ncall (nlist.F90:953-986), "no of neighbour list calls".
 * Rebuilds inside device steps (mg_md_run, mg_bd_run, mg_bench_steps) are
 * counted on the device. */
int mg_nlist_calls(mg_handle *h, int32_t *ncall);

/* Verlet list in the reference's layout: nneighpn(np) and
 * jpnlist(maxnneigh,np), column-major, 1-based.  MD/BD: half list with the
 * (ip+jp) parity owner rule (nlist.F90:742-745); MC: full list. */
int mg_nlist_get(mg_handle *h, int32_t *nneighpn, int32_t *jpnlist,
                 int32_t maxnneigh);

/* Cell list: ncell[3] = ncellX..Z (InitCellList), and for every particle the
 * 0-based cell id  ix + iy*ncellX + iz*ncellX*ncellY  (pcellro). */
int mg_celllist_get(mg_handle *h, int32_t *ncell, int32_t *cellip);

/* ---- energies and forces (A5-A12, A15) ------------------------------------ */

/* UTotal (energy.F90:280-430) for a charged monoatomic system: two-body
 * (UTwoBodyA / UTwoBodyACellList), Ewald (UEwaldRecStd or UEwaldRecSPM,
 * UEwaldSelf, UEwaldSurf), UBond, UAngle and the force epilogue.
 *   forceo  [3*np]  forces scaled by force_fac (may be NULL)
 *   u_twob  [nptpt+1] u%twob(0:nptpt)            (may be NULL)
 *   uout    [4]  u%tot, u%rec, u%bond, virial    (may be NULL)          */
int mg_utotal(mg_handle *h, double *forceo, double *u_twob, double *uout);

/* The energy terms of the last UTotal (or step) of this handle:
 *   terms [6]  u%tot, u%twob(0), u%rec, u%bond, u%angle, virial
 * (UTotal's sums, energy.F90:280-337; u%angle from UAngle, energy.F90:5409). */
int mg_energy_terms(mg_handle *h, double *terms);

/* ---- Monte Carlo trial moves (A13, A14) ------------------------------------ */

/* DUTotal (denergy.F90:98-215) for nptm moving particles ipnptm(1:nptm)
 * at trial positions rotm(3,nptm).  Returns du%twob(0:nptpt) in du_twob,
 * du%rec in *du_rec, du%tot in *du_tot and the hard-core flag.  With bonds,
 * du%tot includes du%bond and du%angle of the moving chain segments (DUBond,
 * DUAngle: denergy.F90:2893-3077; a moved neighbour's trial position is the
 * previous or next entry of ipnptm, as there, so a multi-particle move lists
 * the segments of one string in chain order). */
int mg_dutotal(mg_handle *h, int32_t nptm, const int32_t *ipnptm,
               const double *rotm, double *du_twob, double *du_rec,
               double *du_tot, int32_t *lhsoverlap);

/* MCUpdate for the last mg_dutotal trial (mc.F90:5203-5235): ro = rotm,
 * EwaldUpdateArray (denergy.F90:1776) and UpdateCellIp (celllist.F90:366). */
int mg_accept(mg_handle *h);

/* Many independent single-particle trials against the current
 * configuration: trial t moves particle ip[t] to rtrial(3,t).  Writes
 * du_tot[t] (= du%tot) and lhsoverlap[t]. */
int mg_dutotal_batch(mg_handle *h, int32_t ntrial, const int32_t *ip,
                     const double *rtrial, double *du_tot, int32_t *lhsoverlap);

/* ---- gradients (adjoint form) ------------------------------------------------ */

/* UTotal at the current positions and its gradients with respect to the
 * parameters (the site potentials are the reference's reciprocal-space
 * potential, cf. FieldStatEwaldRecSPM energy.F90:2845-2940, plus the
 * real-space, self and surface parts; the rest has no reference counterpart):
 *   phi     [np]     dU/dq_i per particle (EpsiFourPi applied)
 *   du_deps [nptpt]  dU/d eps_ab of every type pair (Pot_1_6_12 with
 *   du_dsig [nptpt]  sig_ab = (sig_a+sig_b)/2, eps_ab = sqrt(eps_a eps_b))
 *   du_dbox [3]      dU/dL_a for an affine stretch of the box along a;
 *                    sum_a L_a du_dbox[a] equals the scalar virial
 * pp holds the species' sigma, epsilon and lljcut settings the table was
 * built from.  Any output may be NULL. */
int mg_grad(mg_handle *h, const mg_pot_params *pp, double *phi, double *du_deps,
            double *du_dsig, double *du_dbox);

/* The force Jacobian along u: jv[3*np] = d(forceo)/dx . u[3*np] (forceo
 * units per A, i.e. minus force_fac times the Hessian of u%tot applied to
 * u) at the handle's positions, from hand-written derivative kernels: the
 * tabulated pair force (its quartic's derivative in r^2), the bonds, the
 * angles (UAngle's forces in forward-mode dual numbers), and the
 * reciprocal and surface Ewald parts as the field of the dipoles q_j u_j
 * plus the field gradient of the charges along u_i (the dipole kernels of
 * mg_dipole_ewald).  No reference counterpart (the adjoint of MD
 * trajectories needs it).  FP64 handles with a Verlet list in MD or BD
 * mode; runs a UTotal first and leaves the reciprocal scratch (structure
 * factors, meshes) changed. */
int mg_force_jvp(mg_handle *h, const double *u, double *jv);
/* The force's parameter derivatives along u: dq[np] = u . d(forceo)/dq_k
 * for each particle charge, deps[nptpt] and dsig[nptpt] = u . d(forceo)/d
 * eps_ab, d sigma_ab for the (1,6,12) pair parameters (Lorentz-Berthelot
 * from pp's sigat, epsat; lljcut's cut as in mg_grad), at the handle's
 * positions: the Lennard-Jones force differentiated analytically, the
 * real-space Coulomb force through erfc, the reciprocal part as the
 * charges' field along u_k minus the potential of the dipoles q_i u_i (the
 * dipole kernels), and the surface term.  The adjoint of MD trajectories
 * needs it for parameter gradients.  Same handles as mg_force_jvp; runs a
 * UTotal first. */
int mg_force_pvjp(mg_handle *h, const mg_pot_params *pp, const double *u, double *dq, double *deps,
                  double *dsig);
/* UTotal at the current positions and its derivative by an affine strain of
 * the box and the positions, r -> (1 + eps) r: w[9] (row-major, symmetric)
 * = dU/deps_ab, the virial tensor (pairs and bonds r_a f_b, angles through
 * their arms, the reciprocal sum through k -> (1 - eps^T) k and V, the
 * surface term through M and V).  Its trace is the reference's scalar
 * virial (UTotal's `virial`, energy.F90:405-430, of which the reference
 * keeps only the trace); w[0], w[4], w[8] are L_a du_dbox[a] of mg_grad. */
int mg_virial_tensor(mg_handle *h, double *w);

/* ---- integrators ------------------------------------------------------------ */

/* Velocity-Verlet (VelVer, md.F90:252-420 + GetLinAcc md.F90:601-625) for a
 * monoatomic system: massip[np] inverse masses, tstep in ps.  rod/rodd
 * velocity and acceleration arrays (3*np) are uploaded by mg_md_setup. */
int mg_md_setup(mg_handle *h, double tstep, const double *massip,
                const double *rod, const double *rodd);
/* nstep velocity-Verlet steps on the device, each with the Verlet-list
 * check of NList(iSimulationStep).  Outputs as mg_utotal for the last step;
 * rod/rodd (may be NULL) receive the final velocities and accelerations. */
int mg_md_run(mg_handle *h, int32_t nstep, double *forceo, double *uout,
              double *rod, double *rodd);

/* Brownian dynamics (BDStep, bd.F90:120-155): fac1, fac2 per type as the
 * reference computes them; iseed is the GauRandom seed (mollib.F90:2739). */
int mg_bd_setup(mg_handle *h, const double *fac1, const double *fac2,
                int32_t iseed);
/* nstep BD steps on the device (BDStep, then UTotal, then the list check).
 * The first call computes forceo from the current positions before the
 * first step, as BDDriver does at its initial stage. */
int mg_bd_run(mg_handle *h, int32_t nstep, double *forceo, double *uout);
/* One BD step as the host caller sees it: ro_io (3*np, host) is uploaded,
 * one step is taken, and ro_io and forceo (host) are written back. */
int mg_bd_step_host(mg_handle *h, double *ro_io, double *forceo, double *uout);
/* GauRandom state after the BD steps run so far. */
int mg_bd_get_seed(mg_handle *h, int32_t *iseed);

/* ---- ensembles of independent replicas -------------------------------------- */

/* No counterpart in the reference (it runs one system per process).  nrep
 * handles on one device, each set up for MD (mg_md_setup) or BD
 * (mg_bd_setup) after mg_nlist_set, are stepped together: one CUDA graph
 * holds one step of every replica (a branch per replica, each with its own
 * conditional list rebuild), so one launch advances all of them.  A replica
 * follows the same trajectory as when it runs alone.  The handles stay
 * owned by the caller and must outlive the ensemble; read a replica's state
 * with mg_md_run / mg_bd_run (nstep = 0) and mg_get_positions. */
typedef struct mg_ensemble mg_ensemble;
int mg_ensemble_create(int32_t nrep, mg_handle *const *handles, mg_ensemble **e);
/* nstep steps of every replica (kind 0 = velocity Verlet, 1 = BD); *ms (may
 * be NULL) receives the device time of the nstep graph launches. */
int mg_ensemble_run(mg_ensemble *e, int32_t kind, int32_t nstep, double *ms);
/* Kernel launches in one ensemble step (0 before the first run). */
int mg_ensemble_kernels(mg_ensemble *e, int32_t kind, int32_t *nkernels);
int mg_ensemble_last_error(const mg_ensemble *e, char *buf, size_t n);
int mg_ensemble_destroy(mg_ensemble *e);

/* ---- timing ------------------------------------------------------------------ */

/* Average device time per call (ms) of each phase since the last reset,
 * measured with CUDA events on the handle's stream; names in *names
 * (comma separated).  Used for the roofline. */
int mg_phase_times(mg_handle *h, double *ms, int32_t nmax, int32_t *nphase,
                   char *names, size_t names_len);
int mg_phase_reset(mg_handle *h, int32_t enable);

/* Benchmark helper: nstep device steps of the set-up integrator (kind 0 =
 * velocity Verlet, 1 = BD).  Before every step a buffer of flush_bytes is
 * written on the handle's stream (0 = no flush) to evict the L2 cache, then
 * read back, so that the lines the write left dirty are written back before
 * the step rather than during it; CUDA events on the same stream bracket
 * each step (not the flush).  *ms_sum
 * receives the summed device time of the steps.  With phase timing enabled
 * the steps run uncaptured so every kernel can be timed. */
int mg_bench_steps(mg_handle *h, int32_t kind, int32_t nstep, int64_t flush_bytes,
                   double *ms_sum);
/* Number of kernel launches in one captured device step (0 before the first
 * mg_md_run / mg_bd_run / mg_bench_steps). */
int mg_step_kernels(mg_handle *h, int32_t kind, int32_t *nkernels);

/* ---- polyatomic particles (UTwoBodyP) ------------------------------------------ */

/* Particles made of atoms (rigid molecules): the two-body energy is the sum
 * over the atom pairs of every particle pair whose centres are within rcut
 * (UTwoBodyP, energy.F90:786-896).  The atom positions come from the caller
 * (the reference's r(3,na), built from the particle positions and
 * orientations), the particle neighbour list too (jpnlist of NList). */
typedef struct mg_poly_params {
    int32_t abi_version;      /* must be MG_ABI_VERSION                          */
    int32_t np, npt, nptpt;   /* particles, particle types, type pairs          */
    const int32_t *iptpn;     /* [np] particle type, 1..npt                     */
    const int32_t *iptpt;     /* [npt*npt] column-major, 1..nptpt               */
    const int32_t *napt;      /* [npt] atoms per particle of each type          */
    int32_t na;               /* atoms in all                                   */
    const int32_t *ianpn;     /* [np] first atom of each particle, 1-based      */
    const int32_t *iatan;     /* [na] atom type, 1..nat                         */
    int32_t nat, natat;       /* atom types, atom-type pairs                    */
    const int32_t *iatat;     /* [nat*nat] column-major, 1..natat               */
    /* the two-body table over atom-type pairs (PotTwoBodyTab1 with the atom
       types as its types; mg_pot_twobody_tab builds it) */
    int32_t nbuf;
    const double  *ubuf;      /* [nbuf]                                         */
    const int32_t *iubuflow;  /* [natat] 1-based                                */
    const double  *r2umin;    /* [natat]                                        */
    const double  *r2atat;    /* [natat] hard-core distance squared (MC trials) */
    double  boxlen[3];        /* box edges; box centred at the origin           */
    double  rcut;             /* cutoff on the particle-centre distance         */
    int32_t lmc;              /* 1: jpnlist is the full (MC) list: a pair is
                                 taken from its lower-numbered particle         */
    /* Ewald: the atom charges and the damping, for the intramolecular part
       of UEwaldSelf (mg_poly_ewald_intra); aza may be NULL without Ewald */
    const double *aza;        /* [na] atom charges (units of e)                 */
    double  ualpha;
    double  epsi_four_pi;
} mg_poly_params;

typedef struct mg_poly mg_poly;
/* A context on the current device for systems of these parameters; its
 * neighbour list holds up to maxnneigh entries per particle. */
int mg_poly_create(const mg_poly_params *p, int32_t maxnneigh, mg_poly **c);
/* UTwoBodyP for particle centres ro[3*np], atom positions r[3*na] and the
 * neighbour list nneighpn[np], jpnlist[maxnneigh*np] (column-major, 1-based,
 * as NList stores it).  Writes the atom forces force[3*na] (not scaled by
 * force_fac, as force(3,na) in the reference), u%twob(0:nptpt) into
 * u_twob[nptpt+1] and the two-body virial into *virial.  An atom pair
 * closer than its table (r2 < r2umin) returns MG_ERR_TABLE_UNDERRUN. */
int mg_poly_utwobody(mg_poly *c, const double *ro, const double *r, const int32_t *nneighpn,
                     const int32_t *jpnlist, double *force, double *u_twob, double *virial);
/* The molecular part of UEwaldSelf (energy.F90:1301-1345): within every
 * particle, each atom pair removes q_i q_j erf(alpha r)/r (the reciprocal
 * sum counts it, the real-space table does not).  Writes its contribution to
 * u%rec (EpsiFourPi applied) into *u_rec and to the atom forces into
 * force[3*na] (unscaled, as force(3,na)).  The atomic self term and the
 * reciprocal sum over the atoms come from a handle whose particles are the
 * atoms (mg_utotal). */
int mg_poly_ewald_intra(mg_poly *c, const double *r, double *force, double *u_rec);
/* mg_poly_utwobody with the particle list kept on the device: the centres
 * and their neighbour list are those of the handle `centres` (a handle whose
 * particles are the polyatomic particles' centres, after mg_set_positions
 * and mg_nlist_set or mg_nlist_update); only the atom positions r[3*na]
 * travel.  Same outputs; every thread adds the forces of its own particle's
 * atoms only, so the atom forces need no atomics and are reproducible.  The
 * handle's rcut must be at least the pair cutoff p.rcut (its list holds every
 * pair within its rcut, and pairs between rcut and rcut + drnlist only right
 * after a build), else MG_ERR_ARG; a handle whose last list build failed
 * (MG_ERR_NEIGH_OVERFLOW, MG_ERR_CELL) has no list, MG_ERR_STATE. */
int mg_poly_utwobody_list(mg_poly *c, mg_handle *centres, const double *r, double *force, double *u_twob,
                          double *virial);
/* Single-particle MC trials of polyatomic particles (DUTwoBody with
 * UTwoBodyPNew/UTwoBodyPOld, denergy.F90:937-1231, for nptm = 1): trial t
 * moves particle ip[t] (1-based) to centre rotm[3*t] with its atoms at
 * rtm (the atoms of all trials one after another, napt of each particle's
 * type).  Every trial is against the same current state (ro, r and the
 * full MC list nneighpn, jpnlist).  Writes du_twob[t] = u%twob(0) new minus
 * old and lhsoverlap[t] (an atom pair of the trial below r2atat or r2umin:
 * the reference's hard-core rejection); the trials run in parallel. */
int mg_poly_dutwobody_batch(mg_poly *c, const double *ro, const double *r, const int32_t *nneighpn,
                            const int32_t *jpnlist, int32_t ntrial, const int32_t *ip, const double *rotm,
                            const double *rtm, double *du_twob, int32_t *lhsoverlap);
/* One MC trial that moves nptm polyatomic particles together (DUTwoBody
 * with UTwoBodyPNew/UTwoBodyPOld, denergy.F90:937-1231, any nptm, with
 * lptmdutwob for the pairs of moving particles): ipnptm[nptm] the moving
 * particles (1-based, each once), rotm[3*nptm] their new centres, rtm their
 * new atoms one particle after another.  Each moving particle pairs with its
 * list neighbours that stay (nneighpn, jpnlist), and every pair of moving
 * particles counts once.  Writes du_twob[nptpt+1] (index 0 the total, k the
 * particle-type pair k; new minus old) and *lhsoverlap (1: an atom pair of
 * the trial configuration below r2atat or r2umin; du_twob is then zero and
 * the current configuration is not summed).  One block sums the trial. */
int mg_poly_dutwobody_multi(mg_poly *c, const double *ro, const double *r, const int32_t *nneighpn,
                            const int32_t *jpnlist, int32_t nptm, const int32_t *ipnptm, const double *rotm,
                            const double *rtm, double *du_twob, int32_t *lhsoverlap);
/* The end of UTotal for polyatomic particles (energy.F90:405-427): from
 * the total atom forces force[3*na] (unscaled), the atom torques
 * torque[3*na] of the dipole electrostatics (NULL when there are none) and
 * the atom and particle positions, the particle forces forceo[3*np] and
 * torques torqueo[3*np] (both scaled by force_fac, atoms summed in order
 * per particle) and the molecular virial sum (r_a - ro_p) . f_a into
 * *virmolecule. */
int mg_poly_epilogue(mg_poly *c, const double *ro, const double *r, const double *force, const double *torque,
                     double force_fac, double *forceo, double *torqueo, double *virmolecule);
/* Charges and point dipoles of the atoms (UDipole, energy.F90:1476-1579),
 * in the reference's order of calls:
 *   mg_poly_udipole_real    UDipoleP (energy.F90:1588-1798): the atom pairs
 *                           of the particle pairs in the list (NList's
 *                           nneighpn, jpnlist; PBC2 shift of the centres),
 *                           erfc-screened with Ewald (ualpha > 0), bare
 *                           otherwise; sets potstat[na], estat[3*na],
 *                           efg[6*na] (xx, yy, zz, xy, xz, yz) and
 *                           *virelec; *u_real = EpsiFourPi/2 sum (q pot -
 *                           dip . e) of this part (UDipole's ureal)
 *   mg_dipole_ewald         UDipoleEwaldRecStd / UDipoleEwaldRecSPM and the
 *                           atomic part of UDipoleEwaldSelf, on a handle
 *                           of the atoms (below)
 *   mg_poly_udipole_self    the molecular part of UDipoleEwaldSelf
 *                           (energy.F90:2196-2268) and, with lsurf,
 *                           UDipoleEwaldSurf (:2272-2295, the atom
 *                           positions r as they are)
 *   mg_poly_udipole_finish  UDipole's loop (:1510-1545): *u_stat, the atom
 *                           forces added to force[3*na] (EpsiFourPi (q e +
 *                           dip . efg)) and torques added to torque[3*na]
 *                           (EpsiFourPi dip x e)
 * dip[3*na] are the atoms' dipoles in the lab frame (e A); the atom charges
 * are mg_poly_params.aza.  The arrays are read and written on the host at
 * every call.  The pair table of a dipole system holds no Coulomb term
 * (PotTwoBodyTab with ldipole, potential.F90:1380). */
int mg_poly_udipole_real(mg_poly *c, const double *ro, const double *r, const double *dip, const int32_t *nneighpn,
                         const int32_t *jpnlist, double *potstat, double *estat, double *efg, double *virelec,
                         double *u_real);
int mg_poly_udipole_self(mg_poly *c, const double *r, const double *dip, int32_t lsurf, double *potstat,
                         double *estat, double *efg, double *virelec);
int mg_poly_udipole_finish(mg_poly *c, const double *dip, const double *potstat, const double *estat,
                           const double *efg, double *force, double *torque, double *u_stat);
/* Rigid-body velocity Verlet of the polyatomic particles (VelVer with
 * lpolyatom, md.F90:252-420): the state lives on the device.  Set-up takes
 * the inverse masses massip[np], the principal moments momp[3*np], the
 * centres ro[3*np], the quaternions qua[4*np] (qua(0:3,np)), the linear
 * velocities rod[3*np], the angular velocities angvelo[3*np] (principal
 * frame; the quaternion velocities follow by AngVelToQuaVel,
 * mollib.F90:2621-2642), the linear and quaternion accelerations rodd[3*np]
 * and quadd[4*np] (zero at the start of a simulation, as MDDriver sets
 * them, md.F90:131-146), and tvvite, nvvite of the quaternion velocity
 * iteration.  _move advances centres
 * (with PBC) and quaternions (normalised) and writes ro[3*np], the
 * orientation matrices ori[9*np] (ori(3,3,np), column-major, from QuaToOri
 * mollib.F90:2221-2255) and drostep[3*np]; the caller then places the atoms
 * and evaluates UTotal; _kick takes its forceo and torqueo, updates the
 * linear velocities (GetLinAcc md.F90:601-617) and the quaternion
 * velocities (nvvite iterations of GetAngAcc md.F90:628-663) and writes rod
 * and angvelo (that of the last iteration's trial quaternion velocities,
 * as the reference leaves it). */
int mg_poly_rigid_setup(mg_poly *c, double tstep, double tvvite, int32_t nvvite, const double *massip,
                        const double *momp, const double *ro, const double *qua, const double *rod,
                        const double *angvelo, const double *rodd, const double *quadd);
int mg_poly_rigid_move(mg_poly *c, double *ro, double *ori, double *drostep);
int mg_poly_rigid_kick(mg_poly *c, const double *forceo, const double *torqueo, double *rod, double *angvelo);
/* nstep steps of the rigid-body VelVer on the device, without the host
 * between the steps: move, atom placement (SetAtomProp, r = ro + ori ra
 * with ra[3*sum(napt)] the local atom positions of the particle types, type
 * after type), the centres' Verlet list rebuilt on the centres handle hc
 * (an MD handle of the np particle centres with rcut >= the pair cutoff,
 * after mg_set_positions and mg_nlist_set), UTwoBodyP over it, with Ewald
 * (ualpha > 0) the atoms' reciprocal sum and atomic self term on the FP64
 * atom handle ha (its particles the atoms, folded into the box) and the
 * molecular self term, UTotal's end and the kick.  After
 * mg_poly_rigid_setup (and mg_poly_rigid_prime if wanted).  Returns the
 * last step's ro[3*np], ori[9*np] (column-major), rod[3*np], angvelo[3*np]
 * and uout[4] = u%tot, u%twob(0), u%rec, virial.  Charges only (no
 * dipoles).  The first step is launched kernel by kernel; with nstep > 1 the
 * next one is captured on hc's stream into a CUDA graph (ha's streams joined
 * by events) and replayed for the remaining steps, the same kernels in the
 * same order, so the results do not depend on how the steps are split over
 * calls.  With phase timing on either handle every step is launched. */
int mg_poly_md_run(mg_poly *c, mg_handle *hc, mg_handle *ha, const double *ra, int32_t nstep, double *ro,
                   double *ori, double *rod, double *angvelo, double *uout);
/* the accelerations of the current state from forceo and torqueo (a kick
 * of zero length: GetLinAcc, GetAngAcc), for a run that starts from
 * evaluated forces instead of the reference's zero accelerations */
int mg_poly_rigid_prime(mg_poly *c, const double *forceo, const double *torqueo);
/* the quaternions qua[4*np] and quaternion velocities quad[4*np] */
int mg_poly_rigid_get(mg_poly *c, double *qua, double *quad);
int mg_poly_last_error(const mg_poly *c, char *buf, size_t n);
int mg_poly_destroy(mg_poly *c);

/* ---- allocation-free entry point ----------------------------------------------- */

/* Largest ncut that mg_ewald_rec_std_noalloc accepts. */
#define MG_NOALLOC_MAX_NCUT 24

/* No counterpart in the reference.  For callers that cannot allocate device
 * memory -- a host code whose device memory all belongs to its own pool, or
 * one that must not let cudaMalloc/cudaFree synchronise the device inside its
 * step -- the reciprocal part of mg_utotal for standard Ewald
 * (UEwaldRecStd + UEwaldSelf, no surface term), with no handle and no
 * allocation.  Every buffer is caller-owned DEVICE memory:
 *   d_ro [3*np] positions, d_az [np] charges (read)
 *   d_force [3*np]  the reciprocal force is ADDED (EpsiFourPi applied;
 *                   force_fac is not)
 *   d_uout [2]      EpsiFourPi (Urec + Uself), EpsiFourPi Virrec (written)
 * The k-vector set is that of mg_create for the same ncut, ncutregion_cube.
 * Work is queued on `stream` (a cudaStream_t; NULL = default stream) and the
 * call returns without waiting for it.  The working memory is a fixed device
 * array of about 1.2 MB inside the library, held by every GPU that loads it:
 * ncut above MG_NOALLOC_MAX_NCUT is rejected (MG_ERR_ARG).  All calls share
 * that array, so calls that overlap on the GPU (other streams, other threads)
 * race.  The first call on a device looks up the array's device address; make
 * that first call before any stream capture begins.  Every later call made
 * outside stream capture looks the address up again, so a cudaDeviceReset
 * between calls is harmless; a call made during capture uses the address
 * found by the last call outside it.  On error a message is written to err
 * (if non-NULL). */
int mg_ewald_rec_std_noalloc(int32_t np, const double *d_ro, const double *d_az,
                             const double boxlen[3], double ualpha, int32_t ncut,
                             int32_t ncutregion_cube, double epsi_four_pi, double *d_force,
                             double *d_uout, void *stream, char *err, size_t err_len);

#ifdef __cplusplus
}
#endif

#endif /* MOLSIM_GB300_H */
