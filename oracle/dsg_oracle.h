/*
 * dsg_oracle.h -- CPU oracle for the projection hot path of the 3D VOF droplet
 * solver (farzan-t/3D_Droplet_simulation_2007, main.f + input.h).
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C, single-threaded restatement of
 * the reference Fortran routines, kept in the same loop order and operation
 * order, compiled with -O2 -ffp-contract=off so that every double rounding
 * matches a non-contracting Fortran build.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it, and only as the checker.  The
 * GPU product never links or calls it.
 *
 * PARITY UNPINNED: the reference ships no tests, fixtures or golden vectors and
 * no Fortran compiler exists in the build container, so this restatement is not
 * checked against outputs of the reference itself.  It is pinned instead by
 * analytic known-answer tests (AL3D/FL3D round trips, closed-form cut volumes,
 * exact plane translation, manufactured multigrid solutions) and by committed
 * fixtures it generated itself (tests/golden/).
 *
 * Indexing: every 3D array is Fortran column-major A(nx,ny,nz), 1-based, with
 * one ghost layer on each side (interior 2..n-1), exactly as in main.f.
 */
#ifndef DSG_ORACLE_H
#define DSG_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Field identifiers of the fine-level state (same numbering as include/dsg.h). */
enum {
  ORA_CC = 0, ORA_P = 1, ORA_RES = 2, ORA_RHS = 3, ORA_A = 4, ORA_B = 5,
  ORA_C = 6, ORA_EI = 7, ORA_U = 8, ORA_V = 9, ORA_W = 10, ORA_S11 = 11,
  ORA_S22 = 12, ORA_S33 = 13, ORA_S12 = 14, ORA_S13 = 15, ORA_S23 = 16,
  ORA_RHON = 17, ORA_MUN = 18, ORA_NFIELDS = 19,
  /* k-epsilon state (iturb = 3); 19, 20 are the GPU build's pressure history */
  ORA_KTUR = 21, ORA_EPS = 22, ORA_MUT = 23,
  /* interface heights of CalcH3d (hswitch = 1) */
  ORA_HXMIN = 24, ORA_HXMAX = 25, ORA_HYMIN = 26, ORA_HYMAX = 27, ORA_HZMIN = 28, ORA_HZMAX = 29
};

/* Pressure-solver modes. */
enum {
  ORA_MODE_REF_EXACT = 0, /* main.f mglin: FMG, fixed `cycles`, no residual test */
  ORA_MODE_TOL_FP64 = 1   /* same FMG, then extra fine V-cycles until relres < tol */
};

/* The 38 positional values of inputdata.in (main.f:188-234, readinput), in
 * file order, followed by the harness additions. */
typedef struct ora_input {
  int nx, ny, nz, tmax, nfilter, cycles;
  double omega;
  int npre, ntop, npost, restart;
  double maxcfl;
  int iturb, convectype, hswitch;
  double xvel1_si, yvel1_si, zvel1_si, xvel2_si, yvel2_si, zvel2_si;
  double rho2_si, rho1_si, sigma_si, visc2_si, visc1_si, grav_si, grav1_si;
  int icase, ibc;
  double length_si, radius_si, y0_si, z0_si;
  int tprint, ntecplot, tsave, surfacet;
  /* additions (no reference counterpart) */
  int mode;            /* ORA_MODE_* */
  double tol;          /* relative residual target for ORA_MODE_TOL_FP64 */
  int max_vcycles;     /* cap on extra V-cycles */
  double noise_si;     /* half-width of uniform velocity noise [m/s] */
  uint64_t noise_seed; /* counter-based noise seed */
} ora_input;

/* Non-dimensional scalars and adaptive counters (COMMON /PHYSICS/, /DIFF/,
 * /CYCLING/, /dinem/). */
typedef struct ora_scalars {
  double tau, tauh, time, h, rho1, rho2, mu1, mu2, sigma, g, g1;
  double lengthsize, lengthscale, vscale, radius, y0, z0;
  double xvel1, yvel1, zvel1, xvel2, yvel2, zvel2;
  int tauh2; /* INTEGER in input.h:53-55: tau/h^2 truncated */
  int npre, npost, ntop, cycles, tswap, ng;
  int last_vcycles;     /* V-cycles of the last pressure solve (FMG counts as 0) */
  double last_relres;   /* ||rhs - L p||_2 / ||rhs||_2 after the last solve */
  double last_relres_fmg; /* the same right after the FMG part */
  double last_epsdiv;   /* h * max|div u| of the last adaptivity check, -1 if none */
} ora_scalars;

typedef struct ora_state ora_state;

/* ---- whole-solver API --------------------------------------------------- */
int ora_level_count(int nx, int ny, int nz);
ora_state *ora_create(const ora_input *in);
void ora_destroy(ora_state *st);
int ora_nx(const ora_state *st);
int ora_ny(const ora_state *st);
int ora_nz(const ora_state *st);
double *ora_field(ora_state *st, int id);
double *ora_level_field(ora_state *st, int id, int level); /* id in CC..EI, level 1..ng */
void ora_level_dims(const ora_state *st, int level, int *nx, int *ny, int *nz);
void ora_get_scalars(const ora_state *st, ora_scalars *out);
void ora_set_scalars(ora_state *st, const ora_scalars *in);

void ora_vofmethod(ora_state *st);        /* main.f:795-824 (+ fturbdif 1239-1267 when iturb != 0) */
void ora_kepsmodel(ora_state *st);        /* main.f:1888-2025 when iturb = 3, else nothing */
void ora_checktime(ora_state *st);        /* main.f:2152-2171 */
int ora_calch3d(ora_state *st);           /* main.f:1312-1810; nonzero: the reference STOPs */
void ora_sgip(ora_state *st);             /* main.f:2835-3026 */
void ora_sgip2(ora_state *st);            /* main.f:3029-3166 */
int ora_error(const ora_state *st, long long *cell); /* STOP code of the last step (0: none) */
void ora_csf(ora_state *st);              /* main.f:2363-2481 */
void ora_solvelpres(ora_state *st, int t); /* main.f:3236-3439 */
void ora_mglin(ora_state *st);            /* main.f:3645-3763 (+ tol mode) */
void ora_step(ora_state *st, int t);      /* main.f:19-73 loop body (CSF or SGIP, laminar or k-epsilon) */
double ora_relres(ora_state *st);         /* ||rhs - L p|| / ||rhs|| on the fine level */

/* ---- array-level routines (reference subroutine interfaces) ------------- */
void ora_relax(double *u, double lengthsize, const double *rhs, const double *a,
               const double *b, const double *c, const double *ei, int nx, int ny,
               int nz, double omega);
void ora_resid(double lengthsize, double *res, const double *u, const double *rhs,
               const double *a, const double *b, const double *c, int nx, int ny,
               int nz);
void ora_rstrct(double *uc, const double *uf, int ncx, int ncy, int ncz);
void ora_interp(double *uf, const double *uc, int nfx, int nfy, int nfz);
void ora_addint(double *uf, const double *uc, double *res, int nfx, int nfy, int nfz);
void ora_acfromac(double *a, double *b, double *c, double *ei, const double *a2,
                  const double *b2, const double *c2, int nx, int ny, int nz);
void ora_abcei(double *a, double *b, double *c, double *ei, const double *cc,
               double r1, double r2, int nx, int ny, int nz);
void ora_bc_scalar(double *s, int nx, int ny, int nz);
void ora_bc_resid(double *s, int nx, int ny, int nz);
void ora_bc_out(double *s, int nx, int ny, int nz);
void ora_filterc27(const double *cc, double *cf, int nx, int ny, int nz);
/* csf's curvature of a filtered fraction ccf into w11 (interior, then bc_out). */
void ora_csf_curvature(double *w11, const double *ccf, int nx, int ny, int nz);
double ora_al3d(double b1, double b2, double b3, double cc);
double ora_fl3d(double m1, double m2, double m3, double alpha, double r0, double dr0);
/* One split sweep (swp, main.f:848-1000) incl. bc_flux and bc_c; `vof1..3`
 * are caller scratch of the field size. */
void ora_swp(ora_state *st, const double *us, double *cc, double *vof1,
             double *vof2, double *vof3, int d);
double ora_sumfield(const double *u, int nx, int ny, int nz);
double ora_fmodmax(const double *u, int nx, int ny, int nz);
/* counter-based noise shared with the GPU init: uniform in [-1, 1) */
double ora_noise_unit(uint64_t seed, int field, int64_t lin);

#ifdef __cplusplus
}
#endif
#endif
