/*
 * dsg.h -- C ABI of the GB300-native projection hot path of the 3D VOF
 * droplet solver (farzan-t/3D_Droplet_simulation_2007).
 *
 * Two layers of entry points, both plain C (no C++ or torch types):
 *
 *  1. Resident-state API (dsg_create ... dsg_step).  A context owns every
 *     field of the reference COMMON blocks in HBM (one device arena) and runs
 *     the routines of main.f's time loop on one CUDA stream.  This is what the
 *     Fortran driver binds through ISO_C_BINDING in place of VOFmethod, csf,
 *     solvelpres and mglin.
 *  2. Array-level kernels (dsg_relax ... dsg_filterc27) with the argument
 *     lists of the reference subroutines, operating on caller-owned DEVICE
 *     arrays on a caller-given stream.
 *
 * Arrays: Fortran column-major A(nx,ny,nz), FP64 unless stated, one ghost layer
 * on every side (interior 2..n-1), exactly the layout of main.f.  Every function
 * returns DSG_OK (0) or a negative DSG_E* code and never aborts the process;
 * dsg_last_error() gives the message.  A context is not re-entrant: one host
 * thread per context.  Several contexts may coexist.
 */
#ifndef DSG_H
#define DSG_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DSG_OK 0
#define DSG_E_ARG (-1)          /* invalid argument / size */
#define DSG_E_CUDA (-2)         /* CUDA runtime error */
#define DSG_E_NOMEM (-3)        /* device allocation failed */
#define DSG_E_NOT_CONVERGED (-4) /* multigrid hit its V-cycle cap before tol */
#define DSG_E_NONFINITE (-5)    /* NaN/Inf found in a residual or volume reduction */
#define DSG_E_STATE (-6)        /* call out of order (e.g. no net loaded) */

/* Pressure solver modes. */
#define DSG_MODE_REF_EXACT 0 /* mglin as the reference: FMG, fixed `cycles`, no residual test */
#define DSG_MODE_TOL_FP64 1  /* the same FMG, then FP64 V-cycles until relres < tol */
#define DSG_MODE_TOL_MIXED 2 /* FP64 defect correction around FP32 V-cycles, to tol */
#define DSG_MODE_LEARNED 3   /* TOL_MIXED, initial guess from the learned net (guarded) */

/* Fine-level field identifiers (memoryaloc main.f:300-317 order, then the
 * COMMON /surfcom/ and /PHYSICS/ arrays of input.h:31-36, 84-90). */
enum {
  DSG_F_CC = 0,  /* z(icc(ng)): volume fraction */
  DSG_F_P = 1,   /* z(iu(ng)): pressure (also scratch of csf/solvelpres, as in the reference) */
  DSG_F_RES = 2, /* z(ires(ng)) */
  DSG_F_RHS = 3, /* z(irhs(ng)) */
  DSG_F_A = 4, DSG_F_B = 5, DSG_F_C = 6, DSG_F_EI = 7,
  DSG_F_U = 8, DSG_F_V = 9, DSG_F_W = 10,
  DSG_F_S11 = 11, DSG_F_S22 = 12, DSG_F_S33 = 13, DSG_F_S12 = 14, DSG_F_S13 = 15, DSG_F_S23 = 16,
  DSG_F_RHON = 17, DSG_F_MUN = 18,
  DSG_F_PPREV = 19, /* previous-step pressure (build addition: the reference keeps none) */
  DSG_F_PPREV2 = 20, /* spare fine array (not written by the step) */
  DSG_F_KTUR = 21,  /* k-epsilon state (iturb = 3), COMMON /turbulence/ input.h:36-42 */
  DSG_F_EPS = 22,
  DSG_F_MUT = 23,
  DSG_F_HXMIN = 24, /* interface heights of CalcH3d (hswitch = 1): hxmin, hxmax, hymin, hymax, */
  DSG_F_HXMAX = 25, /* hzmin, hzmax (COMMON /NEWW/, input.h:91-95) */
  DSG_F_HYMIN = 26,
  DSG_F_HYMAX = 27,
  DSG_F_HZMIN = 28,
  DSG_F_HZMAX = 29,
  DSG_NFIELDS = 30
};

/* The 38 positional values of inputdata.in (main.f:188-234) in file order,
 * then additions with no reference counterpart. */
typedef struct dsg_config {
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
  /* additions */
  int mode;            /* DSG_MODE_* */
  double tol;          /* relative residual target of the tol modes */
  int max_vcycles;     /* V-cycle / defect-correction cap of the tol modes */
  double noise_si;     /* half-width of the seeded uniform velocity noise [m/s] */
  uint64_t noise_seed; /* seed of the counter-based noise */
  int inner_vcycles;   /* FP32 V-cycles per FP64 defect evaluation in the mixed modes (<= 0: as many
                          as the measured reduction per V-cycle predicts to reach tol, at most 8) */
  int use_graphs;      /* capture the mixed-mode iterations in CUDA graphs (1) or launch directly (0) */
  int tail_nodes;      /* mixed modes: FP32 levels of at most this many nodes run in one single-block
                          launch per V-cycle (0: 18^3 = 5832; < 0: one launch per pass on every level) */
  int warm_start;      /* DSG_MODE_TOL_MIXED initial guess: 0 = FP32 full multigrid, 1 = previous-step
                          pressure, 2 = zero */
  double mg32_omega;   /* relaxation factor of the FP32 V-cycles of the mixed modes (<= 0: omega) */
  int mg32_npre;       /* pre-/post-sweeps of the FP32 V-cycles (<= 0: the adaptive NPRE/NPOST) */
  int mg32_npost;
  int mg32_prolong;    /* prolongation of the FP32 V-cycles and FMG start: 0 = trilinear, 1 = the
                          reference's piecewise-constant injection (interp/addint) */
  int mg32_fmg_cycles; /* V-cycles per level of the FP32 FMG start (<= 0: CYCLES) */
  int mg32_fine_npre;  /* pre-/post-sweeps of the FP32 V-cycles on the finest level (<= 0: as on the
                          other levels) */
  int mg32_fine_npost;
  int mg32_mid_npre;   /* pre-/post-sweeps of the FP32 V-cycles on the level below the finest (<= 0:
                          as on the smaller levels) */
  int mg32_mid_npost;
  int mg32_small_npre; /* pre-/post-sweeps of the FP32 V-cycles on the levels of at most 18^3 nodes below
                          the finest (<= 0: as on the other levels) */
  int mg32_small_npost;
  int fp64_exact;      /* DSG_MODE_TOL_FP64: 0 = sweeps, residuals and norm as fused multiply-adds (fewer
                          FP64 operations, results within ulps of the oracle), 1 = the reference's operation
                          order (bit-identical to the oracle).  DSG_MODE_REF_EXACT always keeps that order. */
  int mg32_krylov;     /* mixed modes: 0 = the FP32 V-cycles between two FP64 defects iterate on one
                          correction, 1 = each V-cycle preconditions one step of GCR (generalised conjugate
                          residual keeping one previous direction; the step minimises the FP32 residual;
                          an option for tolerances of 1e-9 and below) */
  int mg32_fmg_fine_cycles; /* V-cycles of the FP32 FMG start on the finest level (<= 0: as on the others) */
} dsg_config;

/* Non-dimensional scalars and adaptive counters (COMMON /PHYSICS/, /DIFF/,
 * /CYCLING/, /dinem/). */
typedef struct dsg_scalars {
  double tau, tauh, time, h, rho1, rho2, mu1, mu2, sigma, g, g1;
  double lengthsize, lengthscale, vscale, radius, y0, z0;
  double xvel1, yvel1, zvel1, xvel2, yvel2, zvel2;
  int tauh2; /* INTEGER in input.h:53-55: tau/h^2 truncated */
  int npre, npost, ntop, cycles, tswap, ng;
  int last_vcycles;
  double last_relres, last_relres_fmg, last_epsdiv;
} dsg_scalars;

/* Result of one pressure solve. */
typedef struct dsg_mg_stats {
  int mode;           /* mode actually used (a fallback can lower it) */
  int vcycles;        /* V-cycles (fp64 modes) or defect-correction sweeps (mixed) after the initial guess */
  int fine_sweeps;    /* relax calls on the finest level */
  double relres_init; /* relative residual of the initial guess (FMG or learned) */
  double relres;      /* final relative residual (-1 in ref_exact mode) */
  int converged;      /* 1 if relres < tol (tol modes) */
  int fallback;       /* learned mode: 1 if the solve started from the FP32 full-multigrid guess alone
                         (the network's correction was rejected, or the network rested) */
  double epsdiv;      /* h*max|div| of the adaptivity check, -1 if not run this step */
  double relres_base; /* learned mode: relres of the FP32 full-multigrid start (the method without it) */
  double relres_net;  /* learned mode: relres of that start with the network's correction, -1 if not run */
} dsg_mg_stats;

typedef struct dsg_ctx dsg_ctx;

/* ---- lifecycle ---------------------------------------------------------- */
/* readinput + memoryaloc + nondim (main.f:185-446).  Allocates the device
 * arena; requires min(nx,ny,nz) = 2^ng+2 (memoryaloc main.f:295-298). */
int dsg_create(const dsg_config *cfg, dsg_ctx **out);
void dsg_destroy(dsg_ctx *ctx);
const char *dsg_last_error(const dsg_ctx *ctx); /* ctx may be NULL: last error of this host thread */
int dsg_set_stream(dsg_ctx *ctx, void *cuda_stream); /* NULL = the context's own stream */
int dsg_synchronize(dsg_ctx *ctx);
/* Device bytes held by the context arena. */
int64_t dsg_device_bytes(const dsg_ctx *ctx);

/* ---- state transfer ----------------------------------------------------- */
/* Copy a fine field (nx*ny*nz doubles, column-major) host <-> device. */
int dsg_upload(dsg_ctx *ctx, int field, const double *host);
int dsg_download(dsg_ctx *ctx, int field, double *host);
/* Device pointer of a level array (field DSG_F_CC..DSG_F_EI, level 1..ng). */
int dsg_level_ptr(dsg_ctx *ctx, int field, int level, double **dev_ptr, int *nx, int *ny, int *nz);
int dsg_field_ptr(dsg_ctx *ctx, int field, double **dev_ptr);
int dsg_get_scalars(const dsg_ctx *ctx, dsg_scalars *out);
int dsg_set_scalars(dsg_ctx *ctx, const dsg_scalars *in);

/* ---- time-step routines (main.f time loop, main.f:19-73) ----------------- */
/* initialize, restart=0 drop case: smooth2 (+ seeded noise) + bc_c + bc_v +
 * calcrho (main.f:159-178, 5678-5752). */
int dsg_init_drop(dsg_ctx *ctx);
/* VOFmethod(t) main.f:795-824 (+ fturbdif main.f:1239-1267 when iturb != 0) */
int dsg_vofmethod(dsg_ctx *ctx);
/* kepsmodel main.f:1888-2025 (iturb = 3; no-op for iturb = 0) */
int dsg_kepsmodel(dsg_ctx *ctx);
/* checktime(t) main.f:2152-2171 (one device max-reduction, one host read) */
int dsg_checktime(dsg_ctx *ctx);
/* csf(ccc,w11,w22,w33) main.f:2363-2481 (surfacet = 2), SGIP main.f:2835-3026
 * (surfacet = 5) or SGIP2 main.f:3029-3166 (surfacet = 6) */
int dsg_csf(dsg_ctx *ctx);
int dsg_calch3d(dsg_ctx *ctx); /* CalcH3d main.f:1312-1810 (the step calls it when hswitch = 1) */
/* solvelpres(cc,w1..w3,a,b,c,ei,t) main.f:3236-3439, pressure solve per mode */
int dsg_solvelpres(dsg_ctx *ctx, int t, dsg_mg_stats *stats);
/* mglin(r1,r2) main.f:3645-3763 on the resident fine rhs and coefficients */
int dsg_mglin(dsg_ctx *ctx, dsg_mg_stats *stats);
/* One body of the main.f:19-73 loop: VOFmethod (+ CalcH3d when hswitch = 1,
 * + kepsmodel when iturb = 3), checktime, the surface-tension model of
 * surfacet (2 CSF, 5 SGIP, 6 SGIP2) and solvelpres in the context's mode. */
int dsg_step(dsg_ctx *ctx, int t, dsg_mg_stats *stats);
/* dsg_step with the state exchanged through host arrays, as a host that owns
   its fields (the reference's COMMON blocks) needs it: the fields
   in_fields[0..n_in) are copied from in_host[q] and the fields
   out_fields[0..n_out) to out_host[q], each a full nx*ny*nz FP64 array.  The
   copies run on a second stream: each input is waited for only by the first
   phase of the step that touches its field and each output is copied as soon
   as the last phase that writes it is done, so most of the transfer overlaps
   the step's kernels.  Returns once the outputs are on the host.  On an error
   it returns once no copy is in flight any more; outputs whose phase was not
   reached are left unwritten.  Page-locked host arrays (cudaHostRegister or
   cudaMallocHost) make the copies asynchronous. */
int dsg_step_host(dsg_ctx *ctx, int t, dsg_mg_stats *stats, int n_in, const int *in_fields,
                  const double *const *in_host, int n_out, const int *out_fields, double *const *out_host);
/* SUMFIELD(cc) main.f:4783-4801: liquid volume (FP64, deterministic order) */
int dsg_liquid_volume(dsg_ctx *ctx, double *out);
/* h * FMODMAX(div u) on the resident velocity (main.f:3389-3398) */
int dsg_max_divergence(dsg_ctx *ctx, double *out);
/* ||rhs - L p||_2 / ||rhs||_2 on the fine interior (new: the reference has no norm) */
int dsg_relres(dsg_ctx *ctx, double *out);

/* ---- instrumentation ----------------------------------------------------- */
typedef struct dsg_profile {
  int64_t launches;    /* library kernel launches since dsg_profile_enable */
  int64_t relax_calls; /* finest-level relax calls timed with CUDA events */
  double relax_ms;     /* summed event time of those calls */
  double relax_bytes;  /* their algorithmic bytes: 6 words (u r+w, a, b, c, rhs) per cell */
  int relax_bits;      /* word size of the timed relax: 64 (FP64 modes) or 32 (mixed modes) */
  /* CUDA-event time of the phases of dsg_step: 0 VOF advection, 1 CFL check,
   * 2 CSF force, 3 momentum up to the divergence, 4 pressure solve,
   * 5 projection and adaptivity */
  double phase_ms[6];
} dsg_profile;
/* Start (on=1, counters reset) or stop live profiling of the context. */
int dsg_profile_enable(dsg_ctx *ctx, int on);
/* Synchronize the context stream and report the counters. */
int dsg_profile_read(dsg_ctx *ctx, dsg_profile *out);
/* Total kernel launches made by the library in this process. */
int64_t dsg_launch_count(void);

/* ---- learned initial guess (no reference counterpart) ----------------------
 * A 3D convolutional U-Net (4 levels, 16/32/64/64 channels, 3x3x3 kernels,
 * 251649 parameters, BF16 weights/activations, FP32 accumulation, tcgen05
 * tensor-core implicit-GEMM kernels) predicting the correction of the FP32
 * full-multigrid start p0 of a pressure solve from DSG_NET_INPUTS channels:
 * the volume fraction (density), the divergence right-hand side, the FP64
 * defect of p0, p0 and the previous-step pressure.  Its output is in units of
 * h^2 RMS(defect of p0).  A network is sized for one interior grid W x H x D
 * (each a multiple of 8). */
#define DSG_NET_INPUTS 5
typedef struct dsg_net dsg_net;
int64_t dsg_net_param_count(void);
int dsg_net_create(int W, int H, int D, uint64_t seed, dsg_net **out); /* He-initialised */
void dsg_net_destroy(dsg_net *net);
int64_t dsg_net_device_bytes(const dsg_net *net);
/* FP32 parameters, layer by layer: weights [27][cin][cout] then bias[cout] */
int dsg_net_get_params(dsg_net *net, float *host, int64_t count);
int dsg_net_set_params(dsg_net *net, const float *host, int64_t count);
/* forward on host arrays: x = W*H*D voxels x DSG_NET_INPUTS channels (x
 * fastest, channels innermost), y = W*H*D outputs */
int dsg_net_forward_host(dsg_net *net, const float *x, float *y);
/* loss = mean (y - t)^2 and its gradient with respect to every parameter */
int dsg_net_grad_host(dsg_net *net, const float *x, const float *t, float *loss, float *grad);
/* one Adam step on the training pair recorded by the attached context */
int dsg_net_train_step(dsg_net *net, float lr, float *loss);
/* Attach a network to a context (NULL detaches).  record=1: after every
 * mixed-precision pressure solve the context stores (input at the start,
 * solved pressure minus the start) as the net's training pair.
 * DSG_MODE_LEARNED adds the network's correction to the full-multigrid start,
 * scaled to the least FP64 defect, when that cuts the V-cycles the solve
 * expects to need; otherwise it starts from the full-multigrid guess alone
 * and rests the network for 1, 2, 4 .. 32 solves. */
int dsg_attach_net(dsg_ctx *ctx, dsg_net *net, int record);

/* ---- array-level kernels (device pointers, reference argument lists) ----
 * `stream` is a cudaStream_t (NULL = legacy default stream). */
/* relax main.f:3956-3997 */
int dsg_relax(double *u, double lengthsize, const double *rhs, const double *a, const double *b,
              const double *c, const double *ei, int nx, int ny, int nz, double omega, void *stream);
/* resid main.f:3902-3931 (with bc_resid) */
int dsg_resid(double lengthsize, double *res, const double *u, const double *rhs, const double *a,
              const double *b, const double *c, int nx, int ny, int nz, void *stream);
/* rstrct main.f:3765-3791: uc(ncx,ncy,ncz) from uf(2ncx-2, 2ncy-2, 2ncz-2) */
int dsg_rstrct(double *uc, const double *uf, int ncx, int ncy, int ncz, void *stream);
/* interp main.f:3866-3900: uf(nfx,nfy,nfz) from uc(nfx/2+1, ...) */
int dsg_interp(double *uf, const double *uc, int nfx, int nfy, int nfz, void *stream);
/* addint main.f:3934-3954 (res is scratch, as in the reference) */
int dsg_addint(double *uf, const double *uc, double *res, int nfx, int nfy, int nfz, void *stream);
/* acfromac main.f:3793-3844: coarse a,b,c,ei (nx,ny,nz) from fine a2,b2,c2 */
int dsg_acfromac(double *a, double *b, double *c, double *ei, const double *a2, const double *b2,
                 const double *c2, int nx, int ny, int nz, void *stream);
/* abcei main.f:3582-3615 with bc_coef main.f:4465-4494 */
int dsg_abcei(double *a, double *b, double *c, double *ei, const double *cc, double r1, double r2,
              int nx, int ny, int nz, void *stream);
/* bc_scalar main.f:4298-4329, bc_resid 4432-4463, bc_out 4399-4430 */
int dsg_bc_scalar(double *s, int nx, int ny, int nz, void *stream);
int dsg_bc_resid(double *s, int nx, int ny, int nz, void *stream);
int dsg_bc_out(double *s, int nx, int ny, int nz, void *stream);
/* filterc27 main.f:5473-5511 */
int dsg_filterc27(const double *cc, double *cf, int nx, int ny, int nz, void *stream);

/* ---- snapshots and output files ---------------------------------------------
 * A snapshot stages p, u, v, w and cc of step t in device memory (ordered
 * after the work already on the context stream) and copies them to pinned
 * host memory on a separate stream, so the following steps overlap the copy.
 * The writers use the last snapshot (waiting for its copy; taking one if
 * there is none):
 *   dsg_write_tecplot        printtecp, main.f:5105-5153 (X,Y,Z,U,V,W,CC)
 *   dsg_write_pressure_slice printout's pressure plane, main.f:5074-5095
 *   dsg_savedata / iniget    the unformatted restart file, main.f:5414-5467 /
 *                            698-790, as a consistent pair (the reference's
 *                            savedata writes a unit it did not open); iniget
 *                            loads u, v, w, cc into a context of the same grid
 *                            and applies bc_c, bc_v, calcrho (main.f:174-177)
 *   dsg_printout             printout's schedule, main.f:5020-5104:
 *                            main####.plt every ntecplot steps,
 *                            pressure####.plt every 100 steps, save.dat at
 *                            t = tsave, in directory dir (NULL: cwd). */
int dsg_snapshot(dsg_ctx *ctx, int t);
int dsg_snapshot_wait(dsg_ctx *ctx, int *t);
int dsg_snapshot_field(dsg_ctx *ctx, int field, double *host); /* field in p, u, v, w, cc */
int dsg_write_tecplot(dsg_ctx *ctx, const char *path);
int dsg_write_pressure_slice(dsg_ctx *ctx, const char *path);
int dsg_savedata(dsg_ctx *ctx, const char *path, int t0);
int dsg_iniget(dsg_ctx *ctx, const char *path, int *t0);
int dsg_printout(dsg_ctx *ctx, int t, const char *dir);

/* ---- ensemble -------------------------------------------------------------
 * No counterpart in the reference (main.f runs one case per process).  An
 * ensemble holds n independent contexts (cfgs[i], each initialised as
 * dsg_init_drop does) on the current device and steps them together: one
 * dsg_ensemble_step is one time step t of every member.  A pool of `workers`
 * host threads (<= 0: one per hardware thread, at most n) steps the members on
 * their own streams, members assigned to workers by longest-processing-time
 * first on a cost per member.  stats (n entries, may be NULL) receives each
 * member's solve statistics; on failure the first failing member's code is
 * returned and dsg_ensemble_last_error names it.  Members are ordinary
 * contexts for dsg_download/dsg_upload/dsg_get_scalars between steps; they
 * must not be stepped or destroyed individually. */
typedef struct dsg_ensemble dsg_ensemble;
int dsg_ensemble_create(const dsg_config *cfgs, int n, int workers, dsg_ensemble **out);
void dsg_ensemble_destroy(dsg_ensemble *e);
int dsg_ensemble_size(const dsg_ensemble *e);
int dsg_ensemble_workers(const dsg_ensemble *e);
dsg_ctx *dsg_ensemble_member(dsg_ensemble *e, int i);
const char *dsg_ensemble_last_error(const dsg_ensemble *e);
int dsg_ensemble_set_workers(dsg_ensemble *e, int workers);
int dsg_ensemble_step(dsg_ensemble *e, int t, dsg_mg_stats *stats);
/* host wall time of the last ensemble step and of each member's step (ms) */
double dsg_ensemble_last_ms(const dsg_ensemble *e);
int dsg_ensemble_member_ms(const dsg_ensemble *e, double *out);
/* Autotuner: runs real time steps t0, t0+1, ... (the simulation advances):
 * one warm-up step, one step on a single worker that measures every member's
 * step time (the costs of the plan from then on), then steps_per_trial steps
 * per worker count 1, 2, 4, ... up to twice the hardware threads (at most n);
 * keeps the fastest count.  *t_next = the next step index. */
int dsg_ensemble_autotune(dsg_ensemble *e, int t0, int steps_per_trial, int *t_next, int *best_workers);
/* The plan alone: assign[i] = worker of member i for the given costs. */
int dsg_ensemble_plan(const double *cost, int n, int workers, int *assign);
/* Batched mode (groups >= 1): the members split into `groups` cost-balanced
 * groups and each worker steps whole groups: every member of the group up to
 * its pressure solve, the group's pressure solves as one batched
 * mixed-precision solve -- one launch per multigrid pass over all its
 * members, the start and each outer iteration replayed as CUDA graphs on the
 * group's own stream, converged members masked on the device -- then every
 * member after its solve; the groups of different workers overlap on the
 * GPU.  Every member's results are bit for bit those of its own dsg_step.
 * Needs every member in DSG_MODE_TOL_MIXED with the FP32 full-multigrid
 * start, CUDA graphs and the coarse tail on, no network attached (DSG_E_ARG
 * otherwise), and at most 128 members per group.  groups = 0 returns to
 * per-member solves.  mglin
 * main.f:3645-3763 per member.  dsg_ensemble_batched: the group count. */
int dsg_ensemble_set_batched(dsg_ensemble *e, int groups);
int dsg_ensemble_batched(const dsg_ensemble *e);
/* Batched mode: worker time (ms) of the last step's three phases, summed over
 * the workers: members up to their solves, the batched solves, members after
 * their solves. */
int dsg_ensemble_phase_ms(const dsg_ensemble *e, double *out);
/* Autotuner of the batched solves: first the coarse-tail threshold (one
 * batched V-cycle timed per candidate), then the thread-block shape of each
 * sweep, restriction and prolongation launch of an outer iteration (reps
 * timed launches per candidate shape, on the members' own FP32 arrays between
 * steps), keeping the fastest; the results do not change (the cells of a
 * pass are independent).  *slots_tuned = passes tuned over all groups. */
int dsg_ensemble_autotune_tiles(dsg_ensemble *e, int reps, int *slots_tuned);
/* Batched mode: levels of at most this many nodes run in each member's
 * single-block coarse tail (picked by the autotuner; it does not change
 * results); 0 if not batched. */
int64_t dsg_ensemble_batch_tail_nodes(const dsg_ensemble *e);

/* ---- allocation-free pressure solve -------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory when they solve (a host that owns its device arrays under an
 * allocator that forbids cudaMalloc after set-up, or a solve inside a region
 * where an allocation would synchronize the device): the fixed-cycle FMG of
 * mglin (main.f:3645-3763, same kernels and result as dsg_mglin in
 * DSG_MODE_REF_EXACT) on caller-owned device arrays p (in/out: overwritten,
 * ghosts included), rhs, a, b, c, ei of size nx*ny*nz.  Coarse levels and the
 * finest residual live in one static device array sized for grids up to
 * 66x66x66 nodes (about 5.3 MB, held on every device that loads the library
 * until exit); larger grids, and grids whose sides do not all halve evenly
 * down to the coarsest level of min(nx,ny,nz) = 2^ng+2, return DSG_E_ARG.
 * Nothing is allocated.  Calls
 * share that array: each call clears it first, but calls that overlap on the
 * GPU race and must be serialized.  The first call on a device looks up the
 * array's address with that device current; make it before any stream
 * capture. */
int dsg_mglin_noalloc(double *p, const double *rhs, const double *a, const double *b, const double *c,
                      const double *ei, int nx, int ny, int nz, int cycles, int npre, int npost, int ntop,
                      double omega, double lengthsize, double lengthscale, void *stream);

#ifdef __cplusplus
}
#endif
#endif
