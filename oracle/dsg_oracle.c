/*
 * dsg_oracle.c -- CPU oracle (test infrastructure only) restating the
 * projection hot path of farzan-t/3D_Droplet_simulation_2007 (main.f).
 *
 * Every routine cites the main.f lines it follows.  Loop order and the order of
 * every floating-point operation follow the Fortran source (left-to-right
 * evaluation, parentheses honoured, integer powers as repeated products).
 * Default-REAL (single precision) literals of the reference are written as
 * (double)<x>f because gfortran promotes the single-precision value.
 * Build with -O2 -ffp-contract=off (no FMA contraction).
 *
 * PARITY UNPINNED against the reference itself (no Fortran compiler and no
 * reference fixtures exist); pinned by analytic known-answer tests instead.
 */
#include "dsg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define IX(i, j, k) ((size_t)((i) - 1) + (size_t)nx * ((size_t)((j) - 1) + (size_t)ny * (size_t)((k) - 1)))
#define DMAX1(a, b) ((a) > (b) ? (a) : (b))
#define DMIN1(a, b) ((a) < (b) ? (a) : (b))

/* Fortran DMAX1/DMIN1 as gfortran evaluates them for non-NaN arguments. */
static inline double dmax1(double a, double b) { return a >= b ? a : b; }
static inline double dmin1(double a, double b) { return a <= b ? a : b; }

struct ora_state {
  ora_input in;
  int nx, ny, nz;
  ora_scalars s;
  /* level arrays, index 1..ng (main.f:300-317 memoryaloc order) */
  int lnx[32], lny[32], lnz[32];
  double *lv[32][8]; /* [level][CC,P,RES,RHS,A,B,C,EI] */
  double *u, *v, *w, *s11, *s22, *s33, *s12, *s13, *s23, *rhon, *mun;
  double *ktur, *eps, *mut; /* /turbulence/ (input.h:36-42); cmu is 0.09 everywhere for iturb = 3 */
  double *hx0, *hx1, *hy0, *hy1, *hz0, *hz1; /* hxmin, hxmax, hymin, hymax, hzmin, hzmax of CalcH3d */
  int error;                                 /* a STOP of the reference (CalcH3d), 0 = none */
  long long error_cell;
};

static double *zalloc(size_t n) { return (double *)calloc(n, sizeof(double)); }

/* ======================================================================= */
/* boundary conditions                                                     */
/* ======================================================================= */

/* bc_scalar, main.f:4298-4329: x ghost 1 Neumann, x ghost nx Dirichlet 0,
 * y and z Neumann. */
void ora_bc_scalar(double *s, int nx, int ny, int nz) {
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++) {
      s[IX(1, j, k)] = s[IX(2, j, k)];
      s[IX(nx, j, k)] = 0.0;
    }
  for (int k = 2; k <= nz - 1; k++)
    for (int i = 1; i <= nx; i++) {
      s[IX(i, 1, k)] = s[IX(i, 2, k)];
      s[IX(i, ny, k)] = s[IX(i, ny - 1, k)];
    }
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      s[IX(i, j, 1)] = s[IX(i, j, 2)];
      s[IX(i, j, nz)] = s[IX(i, j, nz - 1)];
    }
}

/* bc_resid, main.f:4432-4463 */
void ora_bc_resid(double *s, int nx, int ny, int nz) {
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++) {
      s[IX(1, j, k)] = s[IX(2, j, k)];
      s[IX(nx, j, k)] = s[IX(nx - 1, j, k)];
    }
  for (int k = 2; k <= nz - 1; k++)
    for (int i = 2; i <= nx - 1; i++) {
      s[IX(i, 1, k)] = 0.0;
      s[IX(i, ny, k)] = 0.0;
    }
  for (int j = 1; j <= ny; j++)
    for (int i = 2; i <= nx - 1; i++) {
      s[IX(i, j, 1)] = 0.0;
      s[IX(i, j, nz)] = 0.0;
    }
}

/* bc_out, main.f:4399-4430 */
void ora_bc_out(double *s, int nx, int ny, int nz) {
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++) {
      s[IX(1, j, k)] = s[IX(2, j, k)];
      s[IX(nx, j, k)] = s[IX(nx - 1, j, k)];
    }
  for (int k = 2; k <= nz - 1; k++)
    for (int i = 1; i <= nx; i++) {
      s[IX(i, 1, k)] = s[IX(i, 2, k)];
      s[IX(i, ny, k)] = s[IX(i, ny - 1, k)];
    }
  for (int j = 1; j <= ny; j++)
    for (int i = 2; i <= nx - 1; i++) {
      s[IX(i, j, 1)] = s[IX(i, j, 2)];
      s[IX(i, j, nz)] = s[IX(i, j, nz - 1)];
    }
}

/* bc_c, main.f:4331-4396.  The copy/filterc27/theta block (4347-4375) has no
 * observable effect (both branches at 4378-4382 assign cc(i,2,k)) and is left
 * out. */
static void bc_c(double *cc, int nx, int ny, int nz) {
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++) {
      cc[IX(2, j, k)] = cc[IX(1, j, k)];
      cc[IX(nx, j, k)] = cc[IX(nx - 1, j, k)];
    }
  for (int k = 2; k <= nz - 1; k++)
    for (int i = 2; i <= nx - 1; i++) {
      cc[IX(i, 1, k)] = cc[IX(i, 2, k)];
      if (cc[IX(i, 1, k)] > 1.0) cc[IX(i, 1, k)] = 1.0;
      if (cc[IX(i, 1, k)] < 0.0) cc[IX(i, 1, k)] = 0.0;
      cc[IX(i, ny, k)] = cc[IX(i, ny - 1, k)];
    }
  for (int j = 1; j <= ny; j++)
    for (int i = 2; i <= nx - 1; i++) {
      cc[IX(i, j, 1)] = cc[IX(i, j, 2)];
      cc[IX(i, j, nz)] = cc[IX(i, j, nz - 1)];
    }
}

/* bc_v, main.f:4064-4141 */
static void bc_v(ora_state *st) {
  const int nx = st->nx, ny = st->ny, nz = st->nz;
  double *u = st->u, *v = st->v, *w = st->w;
  const double xvel2 = st->s.xvel2;
  for (int k = 1; k <= nz; k++)
    for (int j = ny; j >= 1; j--) {
      double x = (j * 1.0 - 1.5) / (ny * 1.0 - 1.5) - 1.0;
      u[IX(1, j, k)] = xvel2 * (-(x * x) + 1.0);
      if (j == 1) u[IX(1, 1, k)] = -u[IX(1, 2, k)];
      v[IX(nx, j, k)] = v[IX(nx - 1, j, k)];
      w[IX(nx, j, k)] = w[IX(nx - 1, j, k)];
    }
  for (int k = 2; k <= nz - 1; k++)
    for (int i = 2; i <= nx - 1; i++) {
      u[IX(i, 1, k)] = -u[IX(i, 2, k)];
      u[IX(i, ny, k)] = u[IX(i, ny - 1, k)];
      v[IX(i, 2, k)] = 0.0;
      v[IX(i, 1, k)] = 0.0;
      v[IX(i, ny, k)] = 0.0;
      w[IX(i, 1, k)] = -w[IX(i, 2, k)];
      w[IX(i, ny, k)] = w[IX(i, ny - 1, k)];
    }
  for (int j = 1; j <= ny; j++)
    for (int i = 2; i <= nx - 1; i++) {
      u[IX(i, j, 1)] = u[IX(i, j, 2)];
      u[IX(i, j, nz)] = u[IX(i, j, nz - 1)];
      v[IX(i, j, 1)] = v[IX(i, j, 2)];
      v[IX(i, j, nz)] = v[IX(i, j, nz - 1)];
      w[IX(i, j, 2)] = 0.0;
      w[IX(i, j, nz)] = 0.0;
    }
  double outlet = 0.0, outlet2 = 0.0;
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++) {
      u[IX(2, j, k)] = u[IX(1, j, k)];
      outlet = outlet + u[IX(1, j, k)];
      outlet2 = outlet2 + u[IX(nx - 1, j, k)];
    }
  double vout = outlet / (ny - 2) / (nz - 2);
  double vout2 = outlet2 / (ny - 2) / (nz - 2);
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++) u[IX(nx, j, k)] = u[IX(nx - 1, j, k)] + vout - vout2;
}

/* bc_w, main.f:4143-4220 (note: it overwrites the interior plane i=2 of w1..w3
 * and the plane j=2 of w2 and k=2 of w3, as the reference does). */
static void bc_w(ora_state *st, double *w1, double *w2, double *w3) {
  const int nx = st->nx, ny = st->ny, nz = st->nz;
  const double *u = st->u, *v = st->v, *w = st->w;
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++) {
      w2[IX(1, j, k)] = v[IX(1, j, k)];
      w2[IX(2, j, k)] = w2[IX(1, j, k)];
      w2[IX(nx, j, k)] = v[IX(nx, j, k)];
      w3[IX(1, j, k)] = w[IX(1, j, k)];
      w3[IX(2, j, k)] = w3[IX(1, j, k)];
      w3[IX(nx, j, k)] = w[IX(nx, j, k)];
    }
  for (int k = 2; k <= nz - 1; k++)
    for (int i = 2; i <= nx - 1; i++) {
      w1[IX(i, 1, k)] = -w1[IX(i, 2, k)];
      w1[IX(i, ny, k)] = w1[IX(i, ny - 1, k)];
      w2[IX(i, 1, k)] = 0.0;
      w2[IX(i, 2, k)] = 0.0;
      w2[IX(i, ny, k)] = v[IX(i, ny, k)];
      w3[IX(i, 1, k)] = -w3[IX(i, 2, k)];
      w3[IX(i, ny, k)] = w3[IX(i, ny - 1, k)];
    }
  for (int j = 1; j <= ny; j++)
    for (int i = 2; i <= nx - 1; i++) {
      w1[IX(i, j, 1)] = w1[IX(i, j, 2)];
      w1[IX(i, j, nz)] = w1[IX(i, j, nz - 1)];
      w2[IX(i, j, 1)] = w2[IX(i, j, 2)];
      w2[IX(i, j, nz)] = w2[IX(i, j, nz - 1)];
      w3[IX(i, j, 1)] = w[IX(i, j, 1)];
      w3[IX(i, j, 2)] = w3[IX(i, j, 1)];
      w3[IX(i, j, nz)] = w[IX(i, j, nz)];
    }
  double outlet = 0.0, outlet2 = 0.0;
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++) {
      w1[IX(1, j, k)] = u[IX(1, j, k)];
      w1[IX(2, j, k)] = w1[IX(1, j, k)];
      outlet = outlet + u[IX(1, j, k)];
      outlet2 = outlet2 + w1[IX(nx - 1, j, k)];
    }
  double vout = outlet / (ny - 2) / (nz - 2);
  double vout2 = outlet2 / (ny - 2) / (nz - 2);
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++) w1[IX(nx, j, k)] = w1[IX(nx - 1, j, k)] + vout - vout2;
}

/* bc_tensor, main.f:4222-4296 */
static void bc_tensor(ora_state *st) {
  const int nx = st->nx, ny = st->ny, nz = st->nz;
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++) {
      st->s11[IX(1, j, k)] = 0.0;
      st->s12[IX(nx, j, k)] = 0.0;
      st->s13[IX(nx, j, k)] = 0.0;
    }
  for (int k = 2; k <= nz - 1; k++)
    for (int i = 1; i <= nx; i++) {
      st->s22[IX(i, 1, k)] = st->s22[IX(i, 2, k)];
      st->s12[IX(i, ny, k)] = 0.0;
      st->s23[IX(i, ny, k)] = 0.0;
    }
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      st->s33[IX(i, j, 1)] = 0.0;
      st->s13[IX(i, j, 2)] = 0.0;
      st->s13[IX(i, j, nz)] = 0.0;
      st->s23[IX(i, j, 2)] = 0.0;
      st->s23[IX(i, j, nz)] = 0.0;
    }
}

/* bc_coef, main.f:4465-4494 */
static void bc_coef(double *a, double *b, double *c, const double *cc, double r1,
                    double r2, int nx, int ny, int nz) {
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++) {
      a[IX(1, j, k)] = a[IX(2, j, k)];
      a[IX(nx, j, k)] = a[IX(nx - 1, j, k)];
    }
  for (int k = 2; k <= nz - 1; k++)
    for (int i = 2; i <= nx - 1; i++)
      b[IX(i, 1, k)] = 1.0 / (r1 * (cc[IX(i, 1, k)] + cc[IX(i, 2, k)]) + r2);
  for (int j = 1; j <= ny; j++)
    for (int i = 2; i <= nx - 1; i++)
      c[IX(i, j, 1)] = 1.0 / (r1 * (cc[IX(i, j, 1)] + cc[IX(i, j, 2)]) + r2);
}

/* bc_flux, main.f:4496-4539 */
static void bc_flux(double *vof1, double *vof3, int d, int nx, int ny, int nz) {
  if (d == 1) {
    for (int k = 2; k <= nz - 1; k++)
      for (int j = 2; j <= ny - 1; j++) {
        vof3[IX(1, j, k)] = 0.0;
        vof1[IX(nx, j, k)] = 0.0;
      }
  } else if (d == 2) {
    for (int k = 2; k <= nz - 1; k++)
      for (int i = 2; i <= nx - 1; i++) {
        vof3[IX(i, 1, k)] = 0.0;
        vof1[IX(i, ny, k)] = 0.0;
      }
  } else {
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        vof3[IX(i, j, 1)] = 0.0;
        vof1[IX(i, j, nz)] = 0.0;
      }
  }
}

/* ======================================================================= */
/* multigrid kernels                                                       */
/* ======================================================================= */

/* relax, main.f:3956-3997: omega-over-relaxed red-black Gauss-Seidel, first
 * pass on even i+j+k, bc_scalar before each pass and at the end. */
void ora_relax(double *u, double lengthsize, const double *rhs, const double *a,
               const double *b, const double *c, const double *ei, int nx, int ny,
               int nz, double omega) {
  double h1 = lengthsize / (nx - 2);
  double h2 = h1 * h1;
  int ksw = 1;
  for (int ipass = 1; ipass <= 2; ipass++) {
    ora_bc_scalar(u, nx, ny, nz);
    int jsw = ksw;
    for (int k = 2; k <= nz - 1; k++) {
      int isw = jsw;
      for (int j = 2; j <= ny - 1; j++) {
        for (int i = isw + 1; i <= nx - 1; i += 2) {
          double temp = (a[IX(i, j, k)] * u[IX(i + 1, j, k)] + a[IX(i - 1, j, k)] * u[IX(i - 1, j, k)] +
                         b[IX(i, j, k)] * u[IX(i, j + 1, k)] + b[IX(i, j - 1, k)] * u[IX(i, j - 1, k)] +
                         c[IX(i, j, k)] * u[IX(i, j, k + 1)] + c[IX(i, j, k - 1)] * u[IX(i, j, k - 1)] -
                         h2 * rhs[IX(i, j, k)]) *
                        ei[IX(i, j, k)];
          u[IX(i, j, k)] = omega * temp + (1.0 - omega) * u[IX(i, j, k)];
        }
        isw = 3 - isw;
      }
      jsw = 3 - jsw;
    }
    ksw = 3 - ksw;
  }
  ora_bc_scalar(u, nx, ny, nz);
}

/* resid, main.f:3902-3931 */
void ora_resid(double lengthsize, double *res, const double *u, const double *rhs,
               const double *a, const double *b, const double *c, int nx, int ny,
               int nz) {
  double h1 = lengthsize / (nx - 2);
  double h2i = 1.0 / (h1 * h1);
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        double uc = u[IX(i, j, k)];
        res[IX(i, j, k)] = -h2i * (a[IX(i, j, k)] * (u[IX(i + 1, j, k)] - uc) +
                                   a[IX(i - 1, j, k)] * (u[IX(i - 1, j, k)] - uc) +
                                   b[IX(i, j, k)] * (u[IX(i, j + 1, k)] - uc) +
                                   b[IX(i, j - 1, k)] * (u[IX(i, j - 1, k)] - uc) +
                                   c[IX(i, j, k)] * (u[IX(i, j, k + 1)] - uc) +
                                   c[IX(i, j, k - 1)] * (u[IX(i, j, k - 1)] - uc)) +
                           rhs[IX(i, j, k)];
      }
  ora_bc_resid(res, nx, ny, nz);
}

/* rstrct, main.f:3765-3791: coarse = 1/8 of the 2x2x2 fine children. */
void ora_rstrct(double *uc, const double *uf, int ncx, int ncy, int ncz) {
  const int fx = 2 * ncx - 2, fy = 2 * ncy - 2;
#define FX(i, j, k) ((size_t)((i) - 1) + (size_t)fx * ((size_t)((j) - 1) + (size_t)fy * (size_t)((k) - 1)))
  int nx = ncx, ny = ncy;
  for (int kc = 2; kc <= ncz - 1; kc++) {
    int kf = 2 * kc - 2;
    for (int jc = 2; jc <= ncy - 1; jc++) {
      int jf = 2 * jc - 2;
      for (int ic = 2; ic <= ncx - 1; ic++) {
        int iff = 2 * ic - 2;
        uc[IX(ic, jc, kc)] = 0.125 * (uf[FX(iff, jf, kf)] + uf[FX(iff + 1, jf, kf)] + uf[FX(iff, jf + 1, kf)] +
                                      uf[FX(iff + 1, jf + 1, kf)] + uf[FX(iff, jf, kf + 1)] +
                                      uf[FX(iff + 1, jf, kf + 1)] + uf[FX(iff, jf + 1, kf + 1)] +
                                      uf[FX(iff + 1, jf + 1, kf + 1)]);
      }
    }
  }
#undef FX
  ora_bc_scalar(uc, ncx, ncy, ncz);
}

/* interp, main.f:3866-3900: piecewise-constant injection, then bc_scalar. */
void ora_interp(double *uf, const double *uc, int nfx, int nfy, int nfz) {
  const int ncx = nfx / 2 + 1, ncy = nfy / 2 + 1, ncz = nfz / 2 + 1;
#define CX(i, j, k) ((size_t)((i) - 1) + (size_t)ncx * ((size_t)((j) - 1) + (size_t)ncy * (size_t)((k) - 1)))
  int nx = nfx, ny = nfy;
  for (int kc = 2; kc <= ncz - 1; kc++) {
    int kf = 2 * kc - 2;
    for (int jc = 2; jc <= ncy - 1; jc++) {
      int jf = 2 * jc - 2;
      for (int ic = 2; ic <= ncx - 1; ic++) {
        int ff = 2 * ic - 2;
        double x = uc[CX(ic, jc, kc)];
        uf[IX(ff, jf, kf)] = x;
        uf[IX(ff, jf + 1, kf)] = x;
        uf[IX(ff + 1, jf, kf)] = x;
        uf[IX(ff + 1, jf + 1, kf)] = x;
        uf[IX(ff, jf, kf + 1)] = x;
        uf[IX(ff, jf + 1, kf + 1)] = x;
        uf[IX(ff + 1, jf, kf + 1)] = x;
        uf[IX(ff + 1, jf + 1, kf + 1)] = x;
      }
    }
  }
#undef CX
  (void)ny;
  ora_bc_scalar(uf, nfx, nfy, nfz);
}

/* addint, main.f:3934-3954: res = interp(uc); uf += res over the whole array. */
void ora_addint(double *uf, const double *uc, double *res, int nfx, int nfy, int nfz) {
  ora_interp(res, uc, nfx, nfy, nfz);
  size_t n = (size_t)nfx * nfy * nfz;
  for (size_t q = 0; q < n; q++) uf[q] = uf[q] + res[q];
}

/* acfromac, main.f:3793-3844 */
void ora_acfromac(double *a, double *b, double *c, double *ei, const double *a2,
                  const double *b2, const double *c2, int nx, int ny, int nz) {
  const int fx = 2 * nx - 2, fy = 2 * ny - 2;
#define FX(i, j, k) ((size_t)((i) - 1) + (size_t)fx * ((size_t)((j) - 1) + (size_t)fy * (size_t)((k) - 1)))
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 1; i <= nx - 1; i++)
        a[IX(i, j, k)] = 0.25 * (a2[FX(2 * i - 1, 2 * j - 1, 2 * k - 1)] + a2[FX(2 * i - 1, 2 * j - 2, 2 * k - 1)] +
                                 a2[FX(2 * i - 1, 2 * j - 1, 2 * k - 2)] + a2[FX(2 * i - 1, 2 * j - 2, 2 * k - 2)]);
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 1; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++)
        b[IX(i, j, k)] = 0.25 * (b2[FX(2 * i - 1, 2 * j - 1, 2 * k - 1)] + b2[FX(2 * i - 2, 2 * j - 1, 2 * k - 1)] +
                                 b2[FX(2 * i - 1, 2 * j - 1, 2 * k - 2)] + b2[FX(2 * i - 2, 2 * j - 1, 2 * k - 2)]);
  for (int k = 1; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++)
        c[IX(i, j, k)] = 0.25 * (c2[FX(2 * i - 1, 2 * j - 1, 2 * k - 1)] + c2[FX(2 * i - 2, 2 * j - 1, 2 * k - 1)] +
                                 c2[FX(2 * i - 1, 2 * j - 2, 2 * k - 1)] + c2[FX(2 * i - 2, 2 * j - 2, 2 * k - 1)]);
#undef FX
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++)
        ei[IX(i, j, k)] = 1.0 / (a[IX(i, j, k)] + a[IX(i - 1, j, k)] + b[IX(i, j, k)] + b[IX(i, j - 1, k)] +
                                 c[IX(i, j, k)] + c[IX(i, j, k - 1)]);
}

/* abcei, main.f:3582-3615 (with bc_coef) */
void ora_abcei(double *a, double *b, double *c, double *ei, const double *cc,
               double r1, double r2, int nx, int ny, int nz) {
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        a[IX(i, j, k)] = 1.0 / (r1 * (cc[IX(i, j, k)] + cc[IX(i + 1, j, k)]) + r2);
        b[IX(i, j, k)] = 1.0 / (r1 * (cc[IX(i, j, k)] + cc[IX(i, j + 1, k)]) + r2);
        c[IX(i, j, k)] = 1.0 / (r1 * (cc[IX(i, j, k)] + cc[IX(i, j, k + 1)]) + r2);
      }
  bc_coef(a, b, c, cc, r1, r2, nx, ny, nz);
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++)
        ei[IX(i, j, k)] = 1.0 / (a[IX(i, j, k)] + a[IX(i - 1, j, k)] + b[IX(i, j, k)] + b[IX(i, j - 1, k)] +
                                 c[IX(i, j, k)] + c[IX(i, j, k - 1)]);
}

static void fillzero(double *u, int nx, int ny, int nz) {
  memset(u, 0, sizeof(double) * (size_t)nx * ny * nz);
}

/* ======================================================================= */
/* reductions                                                              */
/* ======================================================================= */

/* SUMFIELD, main.f:4783-4801 */
double ora_sumfield(const double *u, int nx, int ny, int nz) {
  double s = 0.0;
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) s = s + u[IX(i, j, k)];
  return s;
}

/* FMODMAX, main.f:4728-4753 */
double ora_fmodmax(const double *u, int nx, int ny, int nz) {
  double m = -1.0;
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        double r = fabs(u[IX(i, j, k)]);
        if (r > m) m = r;
      }
  return m;
}

/* CFL, main.f:4848-4881 */
static double cfl(ora_state *st) {
  const int nx = st->nx, ny = st->ny, nz = st->nz;
  double c = 0.0;
  const double *f[3] = {st->u, st->v, st->w};
  for (int q = 0; q < 3; q++)
    for (int k = 2; k <= nz - 1; k++)
      for (int j = 2; j <= ny - 1; j++)
        for (int i = 2; i <= nx - 1; i++) c = dmax1(c, fabs(f[q][IX(i, j, k)]));
  return c * st->s.tauh;
}

/* ======================================================================= */
/* multigrid driver                                                        */
/* ======================================================================= */

#define LV(l, f) (st->lv[(l)][(f)])
#define LCC 0
#define LU 1
#define LRES 2
#define LRHS 3
#define LA 4
#define LB 5
#define LC 6
#define LEI 7

/* One V-cycle from level j down to 1 and back (main.f:3705-3759). */
static void vcycle(ora_state *st, int j) {
  const double ls = st->s.lengthsize, om = st->in.omega;
  for (int jj = j; jj >= 2; jj--) {
    int nfx = st->lnx[jj], nfy = st->lny[jj], nfz = st->lnz[jj];
    for (int q = 0; q < st->s.npre; q++)
      ora_relax(LV(jj, LU), ls, LV(jj, LRHS), LV(jj, LA), LV(jj, LB), LV(jj, LC), LV(jj, LEI), nfx, nfy, nfz, om);
    ora_resid(ls, LV(jj, LRES), LV(jj, LU), LV(jj, LRHS), LV(jj, LA), LV(jj, LB), LV(jj, LC), nfx, nfy, nfz);
    int cx = st->lnx[jj - 1], cy = st->lny[jj - 1], cz = st->lnz[jj - 1];
    ora_rstrct(LV(jj - 1, LRHS), LV(jj, LRES), cx, cy, cz);
    fillzero(LV(jj - 1, LU), cx, cy, cz);
  }
  for (int q = 0; q < st->s.ntop; q++)
    ora_relax(LV(1, LU), ls, LV(1, LRHS), LV(1, LA), LV(1, LB), LV(1, LC), LV(1, LEI), st->lnx[1], st->lny[1],
              st->lnz[1], om);
  for (int jj = 2; jj <= j; jj++) {
    int nfx = st->lnx[jj], nfy = st->lny[jj], nfz = st->lnz[jj];
    ora_addint(LV(jj, LU), LV(jj - 1, LU), LV(jj, LRES), nfx, nfy, nfz);
    for (int q = 0; q < st->s.npost; q++)
      ora_relax(LV(jj, LU), ls, LV(jj, LRHS), LV(jj, LA), LV(jj, LB), LV(jj, LC), LV(jj, LEI), nfx, nfy, nfz, om);
  }
}

/* Relative residual ||rhs - L p||_2 / ||rhs||_2 on the fine interior (new; the
 * reference has no norm).  The residual is the expression of resid. */
double ora_relres(ora_state *st) {
  const int ng = st->s.ng;
  const int nx = st->lnx[ng], ny = st->lny[ng], nz = st->lnz[ng];
  const double *u = LV(ng, LU), *rhs = LV(ng, LRHS), *a = LV(ng, LA), *b = LV(ng, LB), *c = LV(ng, LC);
  double h1 = st->s.lengthsize / (nx - 2);
  double h2i = 1.0 / (h1 * h1);
  double rr = 0.0, bb = 0.0;
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        double uc = u[IX(i, j, k)];
        double r = -h2i * (a[IX(i, j, k)] * (u[IX(i + 1, j, k)] - uc) + a[IX(i - 1, j, k)] * (u[IX(i - 1, j, k)] - uc) +
                           b[IX(i, j, k)] * (u[IX(i, j + 1, k)] - uc) + b[IX(i, j - 1, k)] * (u[IX(i, j - 1, k)] - uc) +
                           c[IX(i, j, k)] * (u[IX(i, j, k + 1)] - uc) + c[IX(i, j, k - 1)] * (u[IX(i, j, k - 1)] - uc)) +
                   rhs[IX(i, j, k)];
        rr += r * r;
        bb += rhs[IX(i, j, k)] * rhs[IX(i, j, k)];
      }
  return bb > 0.0 ? sqrt(rr) / sqrt(bb) : sqrt(rr);
}

/* mglin, main.f:3645-3763.  The coefficient arrays of the finest level must
 * already hold abcei's output and the finest rhs the divergence. */
void ora_mglin(ora_state *st) {
  const int ng = st->s.ng;
  const double om = st->in.omega;
  for (int g = ng - 1; g >= 1; g--) {
    int cx = st->lnx[g], cy = st->lny[g], cz = st->lnz[g];
    ora_rstrct(LV(g, LRHS), LV(g + 1, LRHS), cx, cy, cz);
    ora_acfromac(LV(g, LA), LV(g, LB), LV(g, LC), LV(g, LEI), LV(g + 1, LA), LV(g + 1, LB), LV(g + 1, LC), cx, cy,
                 cz);
  }
  fillzero(LV(1, LU), st->lnx[1], st->lny[1], st->lnz[1]);
  /* Q1: the first coarse solve passes lengthscale as lengthsize (3686-3689) */
  for (int q = 0; q < st->s.ntop; q++)
    ora_relax(LV(1, LU), st->s.lengthscale, LV(1, LRHS), LV(1, LA), LV(1, LB), LV(1, LC), LV(1, LEI), st->lnx[1],
              st->lny[1], st->lnz[1], om);
  for (int j = 2; j <= ng; j++) {
    ora_interp(LV(j, LU), LV(j - 1, LU), st->lnx[j], st->lny[j], st->lnz[j]);
    for (int jc = 1; jc <= st->in.cycles; jc++) vcycle(st, j);
  }
  st->s.last_vcycles = 0;
  st->s.last_relres = -1.0;
  st->s.last_relres_fmg = -1.0;
  if (st->in.mode == ORA_MODE_TOL_FP64) {
    double r = ora_relres(st);
    st->s.last_relres_fmg = r;
    int n = 0;
    while (r >= st->in.tol && n < st->in.max_vcycles) {
      vcycle(st, ng);
      n++;
      r = ora_relres(st);
    }
    st->s.last_vcycles = n;
    st->s.last_relres = r;
  }
}

/* ======================================================================= */
/* VOF                                                                     */
/* ======================================================================= */

/* AL3D, main.f:4562-4634 */
double ora_al3d(double b1, double b2, double b3, double cc) {
  const double UNTIER = 1.0 / 3.0;
  double m1 = dmin1(b1, b2), m3 = dmax1(b1, b2), m2 = b3, tmp, res;
  if (m2 < m1) {
    tmp = m1; m1 = m2; m2 = tmp;
  } else if (m2 > m3) {
    tmp = m3; m3 = m2; m2 = tmp;
  }
  double m12 = m1 + m2;
  double pr = dmax1(6.0 * m1 * m2 * m3, 1.0e-50);
  double V1 = m1 * m1 * m1 / pr;
  double V2 = V1 + 0.5 * (m2 - m1) / m3;
  double mm, V3;
  if (m3 < m12) {
    mm = m3;
    V3 = (m3 * m3 * (3.0 * m12 - m3) + m1 * m1 * (m1 - 3.0 * m3) + m2 * m2 * (m2 - 3.0 * m3)) / pr;
  } else {
    mm = m12;
    V3 = 0.5 * mm / m3;
  }
  double ch = dmin1(cc, 1.0 - cc);
  if (ch < V1) {
    res = pow(pr * ch, UNTIER);
  } else if (ch < V2) {
    res = 0.5 * (m1 + sqrt(m1 * m1 + 8.0 * m2 * m3 * (ch - V1)));
  } else if (ch < V3) {
    double p = 2.0 * m1 * m2;
    double q = 1.5 * m1 * m2 * (m12 - 2.0 * m3 * ch);
    double p12 = sqrt(p);
    double cst = q / (p * p12);
    if (cst > 1.0) cst = 1.0;
    if (cst < -1.0) cst = -1.0;
    double teta = acos(cst) / 3.0;
    double cs = cos(teta);
    res = p12 * (sqrt(3.0 * (1.0 - cs * cs)) - cs) + m12;
  } else if (mm == m12) {
    res = m3 * ch + 0.5 * mm;
  } else {
    double p = m1 * (m2 + m3) + m2 * m3 - 0.25;
    double q = 1.5 * m1 * m2 * m3 * (0.5 - ch);
    double p12 = sqrt(p);
    double cst = q / (p * p12);
    if (cst > 1.0) cst = 1.0;
    if (cst < -1.0) cst = -1.0;
    double teta = acos(cst) / 3.0;
    double cs = cos(teta);
    res = p12 * (sqrt(3.0 * (1.0 - cs * cs)) - cs) + 0.5;
  }
  if (cc > 0.5) res = 1.0 - res;
  return res;
}

/* FL3D, main.f:4639-4698 */
double ora_fl3d(double m1, double m2, double m3, double alpha, double r0, double dr0) {
  double al = alpha - m1 * r0;
  al = al + dmax1(0.0, -m1 * dr0) + dmax1(0.0, -m2) + dmax1(0.0, -m3);
  double tmp = fabs(m1) * dr0 + fabs(m2) + fabs(m3);
  double n1 = fabs(m1) / tmp, n2 = fabs(m2) / tmp, n3 = fabs(m3) / tmp;
  al = dmax1(0.0, dmin1(1.0, al / tmp));
  double al0 = dmin1(al, 1.0 - al);
  double b1 = dmin1(n1 * dr0, n2), b3 = dmax1(n1 * dr0, n2), b2 = n3;
  if (b2 < b1) {
    tmp = b1; b1 = b2; b2 = tmp;
  } else if (b2 > b3) {
    tmp = b3; b3 = b2; b2 = tmp;
  }
  double b12 = b1 + b2;
  double bm = dmin1(b12, b3);
  double pr = dmax1(6.0 * b1 * b2 * b3, 1.0e-50);
  if (al0 < b1) {
    tmp = al0 * al0 * al0 / pr;
  } else if (al0 < b2) {
    tmp = 0.5 * al0 * (al0 - b1) / (b2 * b3) + b1 * b1 * b1 / pr;
  } else if (al0 < bm) {
    tmp = (al0 * al0 * (3.0 * b12 - al0) + b1 * b1 * (b1 - 3.0 * al0) + b2 * b2 * (b2 - 3.0 * al0)) / pr;
  } else if (bm == b12) {
    tmp = (al0 - 0.5 * bm) / b3;
  } else {
    tmp = (al0 * al0 * (3.0 - 2.0 * al0) + b1 * b1 * (b1 - 3.0 * al0) + b2 * b2 * (b2 - 3.0 * al0) +
           b3 * b3 * (b3 - 3.0 * al0)) / pr;
  }
  return al <= 0.5 ? tmp * dr0 : (1.0 - tmp) * dr0;
}

/* swp, main.f:848-1000 */
void ora_swp(ora_state *st, const double *us, double *cc, double *vof1, double *vof2,
             double *vof3, int d) {
  const int nx = st->nx, ny = st->ny, nz = st->nz;
  const double tauh = st->s.tauh;
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        double a1 = us[IX(i, j, k)] * tauh, a2;
        if (d == 1) a2 = us[IX(i + 1, j, k)] * tauh;
        else if (d == 2) a2 = us[IX(i, j + 1, k)] * tauh;
        else a2 = us[IX(i, j, k + 1)] * tauh;
        size_t q = IX(i, j, k);
        vof1[q] = 0.0;
        vof2[q] = 0.0;
        vof3[q] = 0.0;
        double c0 = cc[q];
        if (c0 == 1.0) {
          vof1[q] = dmax1(-a1, 0.0);
          vof2[q] = 1.0 - dmax1(a1, 0.0) + dmin1(a2, 0.0);
          vof3[q] = dmax1(a2, 0.0);
        } else if (c0 > 0.0) {
#define C(di, dj, dk) cc[IX(i + (di), j + (dj), k + (dk))]
          double mm1, mm2, mx, my, mz;
          mm1 = C(-1, -1, -1) + C(-1, -1, 1) + C(-1, 1, -1) + C(-1, 1, 1) +
                2.0 * (C(-1, -1, 0) + C(-1, 1, 0) + C(-1, 0, -1) + C(-1, 0, 1)) + 4.0 * C(-1, 0, 0);
          mm2 = C(1, -1, -1) + C(1, -1, 1) + C(1, 1, -1) + C(1, 1, 1) +
                2.0 * (C(1, -1, 0) + C(1, 1, 0) + C(1, 0, -1) + C(1, 0, 1)) + 4.0 * C(1, 0, 0);
          mx = mm1 - mm2;
          mm1 = C(-1, -1, -1) + C(-1, -1, 1) + C(1, -1, -1) + C(1, -1, 1) +
                2.0 * (C(-1, -1, 0) + C(1, -1, 0) + C(0, -1, -1) + C(0, -1, 1)) + 4.0 * C(0, -1, 0);
          mm2 = C(-1, 1, -1) + C(-1, 1, 1) + C(1, 1, -1) + C(1, 1, 1) +
                2.0 * (C(-1, 1, 0) + C(1, 1, 0) + C(0, 1, -1) + C(0, 1, 1)) + 4.0 * C(0, 1, 0);
          my = mm1 - mm2;
          mm1 = C(-1, -1, -1) + C(-1, 1, -1) + C(1, -1, -1) + C(1, 1, -1) +
                2.0 * (C(-1, 0, -1) + C(1, 0, -1) + C(0, -1, -1) + C(0, 1, -1)) + 4.0 * C(0, 0, -1);
          mm2 = C(-1, -1, 1) + C(-1, 1, 1) + C(1, -1, 1) + C(1, 1, 1) +
                2.0 * (C(-1, 0, 1) + C(1, 0, 1) + C(0, -1, 1) + C(0, 1, 1)) + 4.0 * C(0, 0, 1);
          mz = mm1 - mm2;
#undef C
          if (mx == 0.0 && my == 0.0 && mz == 0.0) {
            /* DEVIATION (documented): a symmetric 27-point neighbourhood gives
             * an all-zero Youngs normal; AL3D then returns 0 and FL3D divides
             * 0/0 (NaN in the reference too).  The cell is advected as a
             * uniformly filled cell: donor-cell fluxes scaled by c. */
            vof1[q] = c0 * dmax1(-a1, 0.0);
            vof2[q] = c0 * (1.0 - dmax1(a1, 0.0) + dmin1(a2, 0.0));
            vof3[q] = c0 * dmax1(a2, 0.0);
            continue;
          }
          int invx = 1, invy = 1, invz = 1;
          if (mx < 0.0) { mx = -mx; invx = -1; }
          if (my < 0.0) { my = -my; invy = -1; }
          if (mz < 0.0) { mz = -mz; invz = -1; }
          mm2 = mx + my + mz + (double)1.e-30f; /* default-REAL literal, main.f:927 */
          mx = mx / mm2;
          my = my / mm2;
          mz = mz / mm2;
          double alpha = ora_al3d(mx, my, mz, c0);
          mx = invx * mx;
          my = invy * my;
          mz = invz * mz;
          alpha = alpha + dmin1(0.0, mx) + dmin1(0.0, my) + dmin1(0.0, mz);
          mm1 = dmax1(a1, 0.0);
          mm2 = 1.0 - mm1 + dmin1(0.0, a2);
          if (d == 1) {
            mx = mx / (1.0 - a1 + a2);
            alpha = alpha + mx * a1;
            if (a1 < 0.0) vof1[q] = ora_fl3d(mx, my, mz, alpha, a1, -a1);
            if (a2 > 0.0) vof3[q] = ora_fl3d(mx, my, mz, alpha, 1.0, a2);
            vof2[q] = ora_fl3d(mx, my, mz, alpha, mm1, mm2);
          } else if (d == 2) {
            my = my / (1.0 - a1 + a2);
            alpha = alpha + my * a1;
            if (a1 < 0.0) vof1[q] = ora_fl3d(my, mz, mx, alpha, a1, -a1);
            if (a2 > 0.0) vof3[q] = ora_fl3d(my, mz, mx, alpha, 1.0, a2);
            vof2[q] = ora_fl3d(my, mz, mx, alpha, mm1, mm2);
          } else {
            mz = mz / (1.0 - a1 + a2);
            alpha = alpha + mz * a1;
            if (a1 < 0.0) vof1[q] = ora_fl3d(mz, mx, my, alpha, a1, -a1);
            if (a2 > 0.0) vof3[q] = ora_fl3d(mz, mx, my, alpha, 1.0, a2);
            vof2[q] = ora_fl3d(mz, mx, my, alpha, mm1, mm2);
          }
        }
      }
  bc_flux(vof1, vof3, d, nx, ny, nz);
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        double x;
        if (d == 1) x = vof3[IX(i - 1, j, k)] + vof2[IX(i, j, k)] + vof1[IX(i + 1, j, k)];
        else if (d == 2) x = vof3[IX(i, j - 1, k)] + vof2[IX(i, j, k)] + vof1[IX(i, j + 1, k)];
        else x = vof3[IX(i, j, k - 1)] + vof2[IX(i, j, k)] + vof1[IX(i, j, k + 1)];
        cc[IX(i, j, k)] = dmax1(0.0, dmin1(1.0, x));
      }
  bc_c(cc, nx, ny, nz);
}

/* calcrho, main.f:2177-2190 */
static void calcrho(ora_state *st) {
  const int nx = st->nx, ny = st->ny, nz = st->nz;
  const double *cc = st->lv[st->s.ng][LCC];
  const double rho1 = st->s.rho1, rho2 = st->s.rho2, mu1 = st->s.mu1, mu2 = st->s.mu2;
  for (int i = 1; i <= nx; i++)
    for (int k = 1; k <= nz; k++)
      for (int j = 1; j <= ny; j++) {
        st->rhon[IX(i, j, k)] = rho2 + cc[IX(i, j, k)] * (rho1 - rho2);
        st->mun[IX(i, j, k)] = mu2 + cc[IX(i, j, k)] * (mu1 - mu2);
      }
}

/* VOFmethod, main.f:795-824 (laminar: fturbdif is not called) */
/* ======================================================================= */
/* interface heights (CalcH3d) and the SGIP surface-tension force            */
/* ======================================================================= */

static inline double cube(double x) { return x * x * x; }

/* CalcH3d for one cell (main.f:1312-1770): Youngs normal from the 27-point
 * stencil, the heights of the PLIC polygon on the cell faces in the five
 * geometric cases of the ordered normal (n1 <= n2 <= n3), then assigned to the
 * axes.  h[6] = hxmin, hxmax, hymin, hymax, hzmin, hzmax.  Returns 0, or 1
 * for "NO MATCH CASES FOUND" and 2 for "PROBLEM finding MIN and MAX unit
 * vector components" (the reference STOPs on both). */
static int h3d_cell(const double *c, size_t q, size_t sy, size_t sz, double h[6]) {
#define C(di, dj, dk) c[q + (long)(di) + (long)(dj) * (long)sy + (long)(dk) * (long)sz]
  double mm1, mm2;
  mm1 = C(-1, -1, -1) + C(-1, -1, 1) + C(-1, 1, -1) + C(-1, 1, 1) +
        2.0 * (C(-1, -1, 0) + C(-1, 1, 0) + C(-1, 0, -1) + C(-1, 0, 1)) + 4.0 * C(-1, 0, 0);
  mm2 = C(1, -1, -1) + C(1, -1, 1) + C(1, 1, -1) + C(1, 1, 1) +
        2.0 * (C(1, -1, 0) + C(1, 1, 0) + C(1, 0, -1) + C(1, 0, 1)) + 4.0 * C(1, 0, 0);
  const double normx = mm1 - mm2;
  mm1 = C(-1, -1, -1) + C(-1, -1, 1) + C(1, -1, -1) + C(1, -1, 1) +
        2.0 * (C(-1, -1, 0) + C(1, -1, 0) + C(0, -1, -1) + C(0, -1, 1)) + 4.0 * C(0, -1, 0);
  mm2 = C(-1, 1, -1) + C(-1, 1, 1) + C(1, 1, -1) + C(1, 1, 1) +
        2.0 * (C(-1, 1, 0) + C(1, 1, 0) + C(0, 1, -1) + C(0, 1, 1)) + 4.0 * C(0, 1, 0);
  const double normy = mm1 - mm2;
  mm1 = C(-1, -1, -1) + C(-1, 1, -1) + C(1, -1, -1) + C(1, 1, -1) +
        2.0 * (C(-1, 0, -1) + C(1, 0, -1) + C(0, -1, -1) + C(0, 1, -1)) + 4.0 * C(0, 0, -1);
  mm2 = C(-1, -1, 1) + C(-1, 1, 1) + C(1, -1, 1) + C(1, 1, 1) +
        2.0 * (C(-1, 0, 1) + C(1, 0, 1) + C(0, -1, 1) + C(0, 1, 1)) + 4.0 * C(0, 0, 1);
  const double normz = mm1 - mm2;
  const double cc = C(0, 0, 0);
#undef C
  const double den = sqrt(normx * normx + normy * normy + normz * normz + 1.e-50);
  const double nix = normx / den, niy = normy / den, niz = normz / den;
  const double ccnew = cc > 0.5 ? 1.0 - cc : cc;
  const double absxn = fabs(nix), absyn = fabs(niy), abszn = fabs(niz);
  const double n1 = dmin1(dmin1(absxn, absyn), abszn);
  const double n3 = dmax1(dmax1(absxn, absyn), abszn);
  const double n2 = absxn + absyn + abszn - n1 - n3;
  const double clim1 = sqrt(2.0 * ccnew * n3 * n2);
  double h1a, h1b, h2a, h2b, h3a, h3b, s1, s2, s3, diag;
  if (n1 == 0.0 && n2 > 0.0 && ccnew <= clim1) {
    s2 = sqrt(2.0 * ccnew * n3 / n2);
    s3 = sqrt(2.0 * ccnew * n2 / n3);
    h1a = s2 * s3 / 2.0; h1b = s2 * s3 / 2.0;
    h2a = s3; h2b = 0.0;
    h3a = s2; h3b = 0.0;
  } else if (n1 == 0.0 && n2 > 0.0 && ccnew > clim1) {
    h1a = cc; h1b = cc;
    h2a = cc + n2 / (2.0 * n3); h2b = cc - n2 / (2.0 * n3);
    h3a = 1.0; h3b = 0.0;
  } else if (n1 == 0.0 && n2 == 0.0) {
    h1a = ccnew; h1b = ccnew; h2a = ccnew; h2b = ccnew;
    h3a = 1.0; h3b = 0.0;
  } else if (6.0 * n2 * n3 * ccnew < n1 * n1) {  /* triangle, case (a) */
    diag = pow(6.0 * n1 * n2 * n3 * ccnew, 1.0 / 3.0);
    s1 = diag / n1; s2 = diag / n2; s3 = diag / n3;
    h1a = (s2 * s3) / 2.0; h1b = 0.0;
    h2a = (s1 * s3) / 2.0; h2b = 0.0;
    h3a = (s1 * s2) / 2.0; h3b = 0.0;
  } else if (6.0 * n2 * n3 * ccnew < 3.0 * (n2 * n2) - 3.0 * n1 * n2 + n1 * n1) {  /* quadrilateral A, (b) */
    diag = (3.0 * n1 + sqrt(72.0 * n2 * n3 * ccnew - 3.0 * (n1 * n1))) / 6.0;
    s1 = diag / n1; s2 = diag / n2; s3 = diag / n3;
    const double t = (s1 - 1.0) / s1;
    h1a = (s2 * s3) / 2.0; h1b = (s2 * s3) / 2.0 * (t * t);
    h2a = s3 * (2.0 * s1 - 1.0) / (2.0 * s1); h2b = 0.0;
    h3a = s2 * (2.0 * s1 - 1.0) / (2.0 * s1); h3b = 0.0;
  } else if ((n1 + n2 >= n3 && 6.0 * n1 * n2 * n3 * ccnew < cube(n3) - cube(n3 - n1) - cube(n3 - n2)) ||
             (n1 + n2 < n3 && 2.0 * n3 * ccnew < n1 + n2)) {  /* pentagon, (c): Newton-Raphson */
    const double rsixn3 = 1.0 / (6.0 * n1 * n2 * n3);
    diag = n2;
    for (int loop = 1; loop <= 1000; loop++) {
      const double delta = -(rsixn3 * (cube(diag) - cube(diag - n1) - cube(diag - n2)) - ccnew) /
                           (3.0 * rsixn3 * (diag * diag - (diag - n1) * (diag - n1) - (diag - n2) * (diag - n2)));
      diag = diag + delta;
      if (fabs(delta) < 1.e-6) break;
    }
    s1 = diag / n1; s2 = diag / n2; s3 = diag / n3;
    const double t1 = (s1 - 1.0) / s1, t2 = (s2 - 1.0) / s2;
    h1a = s3 * (2.0 * s2 - 1.0) / (2.0 * s2); h1b = (s2 * s3) / 2.0 * (t1 * t1);
    h2a = s3 * (2.0 * s1 - 1.0) / (2.0 * s1); h2b = (s1 * s3) / 2.0 * (t2 * t2);
    h3a = 2.0 * (s1 + s2) - s1 / s2 - s2 / s1 - s1 * s2 - 1.0; h3b = 0.0;
  } else if ((n1 + n2 > n3) && 6.0 * n1 * n2 * n3 * ccnew >= cube(n3) - cube(n3 - n1) - cube(n3 - n2)) {
    /* hexagon, (d): Newton-Raphson */
    const double rsixn3 = 1.0 / (6.0 * n1 * n2 * n3);
    diag = n3;
    for (int loop = 1; loop <= 1000; loop++) {
      const double delta =
          -(rsixn3 * (cube(diag) - cube(diag - n1) - cube(diag - n2) - cube(diag - n3)) - ccnew) /
          (3.0 * rsixn3 *
           (diag * diag - (diag - n1) * (diag - n1) - (diag - n2) * (diag - n2) - (diag - n3) * (diag - n3)));
      diag = diag + delta;
      if (fabs(delta) < 1.e-6) break;
    }
    s1 = diag / n1; s2 = diag / n2; s3 = diag / n3;
    const double t1 = (s1 - 1.0) / s1, t2 = (s2 - 1.0) / s2, t3 = (s3 - 1.0) / s3;
    h1a = 2.0 * (s2 + s3) - s2 / s3 - s3 / s2 - s2 * s3 - 1.0; h1b = (s2 * s3) / 2.0 * (t1 * t1);
    h2a = 2.0 * (s1 + s3) - s1 / s3 - s3 / s1 - s1 * s3 - 1.0; h2b = (s1 * s3) / 2.0 * (t2 * t2);
    h3a = 2.0 * (s1 + s2) - s1 / s2 - s2 / s1 - s1 * s2 - 1.0; h3b = (s1 * s2) / 2.0 * (t3 * t3);
  } else if ((n1 + n2 < n3) && 6.0 * n1 * n2 * n3 * ccnew >= cube(n1 + n2) - cube(n1) - cube(n2)) {
    /* quadrilateral B, (e) */
    diag = 0.5 * (n1 + n2) + ccnew * n3;
    s1 = diag / n1; s2 = diag / n2; s3 = diag / n3;
    h1a = s3 * (2.0 * s2 - 1.0) / (2.0 * s2); h1b = s3 * (2.0 * s2 - 1.0) * (s1 - 1.0) / (2.0 * s1 * s2);
    h2a = s3 * (2.0 * s1 - 1.0) / (2.0 * s1); h2b = s3 * (2.0 * s1 - 1.0) * (s2 - 1.0) / (2.0 * s1 * s2);
    h3a = 1.0; h3b = 0.0;
  } else {
    return 1;
  }
  if (cc > 0.5) {
    h1a = 1.0 - h1a; h1b = 1.0 - h1b; h2a = 1.0 - h2a; h2b = 1.0 - h2b; h3a = 1.0 - h3a; h3b = 1.0 - h3b;
  }
  /* assignment to the axes (the branches of main.f:1586-1735, including
   * their use of niz's sign for y when z carries the smallest component) */
#define SET(lo, hi, n, a, b) do { if ((n) < 0) { lo = (a); hi = (b); } else { lo = (b); hi = (a); } } while (0)
  double hx0 = 0, hx1 = 0, hy0 = 0, hy1 = 0, hz0 = 0, hz1 = 0;
  if (absxn == n1) {
    SET(hx0, hx1, nix, h1a, h1b);
    if (fabs(absyn - n2) < 1.e-6) { SET(hy0, hy1, niy, h2a, h2b); SET(hz0, hz1, niz, h3a, h3b); }
    else if (fabs(abszn - n2) < 1.e-6) { SET(hy0, hy1, niy, h3a, h3b); SET(hz0, hz1, niz, h2a, h2b); }
    else return 2;
  } else if (absyn == n1) {
    SET(hy0, hy1, niy, h1a, h1b);
    if (fabs(absxn - n2) < 1.e-6) { SET(hx0, hx1, nix, h2a, h2b); SET(hz0, hz1, niz, h3a, h3b); }
    else if (fabs(abszn - n2) < 1.e-6) { SET(hx0, hx1, nix, h3a, h3b); SET(hz0, hz1, niz, h2a, h2b); }
    else return 2;
  } else if (abszn == n1) {
    SET(hz0, hz1, niz, h1a, h1b);
    if (fabs(absxn - n2) < 1.e-6) { SET(hx0, hx1, nix, h2a, h2b); SET(hy0, hy1, niz, h3a, h3b); }
    else if (fabs(absyn - n2) < 1.e-6) { SET(hx0, hx1, nix, h3a, h3b); SET(hy0, hy1, niz, h2a, h2b); }
    else return 2;
  }
#undef SET
  if (cc <= 0.5) {
    double t;
    t = hx0; hx0 = hx1; hx1 = t;
    t = hy0; hy0 = hy1; hy1 = t;
    t = hz0; hz0 = hz1; hz1 = t;
  }
  double *o[6] = {&hx0, &hx1, &hy0, &hy1, &hz0, &hz1};
  for (int m = 0; m < 6; m++) {
    double v = *o[m];
    if (v < 0.0) v = 0.0;
    if (v > 1.0) v = 1.0;
    h[m] = v;
  }
  return 0;
}

/* CalcH3d, main.f:1312-1810: heights of every interior cell; ghosts untouched. */
int ora_calch3d(ora_state *st) {
  const int nx = st->nx, ny = st->ny, nz = st->nz;
  const double *cc = st->lv[st->s.ng][LCC];
  double *H[6] = {st->hx0, st->hx1, st->hy0, st->hy1, st->hz0, st->hz1};
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        const size_t q = IX(i, j, k);
        double h[6];
        const int rc = h3d_cell(cc, q, (size_t)nx, (size_t)nx * ny, h);
        if (rc) {
          if (!st->error) { st->error = rc; st->error_cell = (long long)q; }
          return rc;
        }
        for (int m = 0; m < 6; m++) H[m][q] = h[m];
      }
  return 0;
}

/* SGIP's (and SGIP2's) curvature: csf's formula with the transverse
 * differences summed in SGIP's order (main.f:2880-2913, 3064-3097). */
static void sgip_curvature(double *w11, const double *ccf, int nx, int ny, int nz) {
  for (int j = 2; j <= ny - 1; j++)
    for (int i = 2; i <= nx - 1; i++)
      for (int k = 2; k <= nz - 1; k++) {
#define F(di, dj, dk) ccf[IX(i + (di), j + (dj), k + (dk))]
        double t0, t1, t2;
        t0 = F(1, 0, 0) - F(0, 0, 0);
        t1 = F(0, 1, 0) - F(0, -1, 0) + F(1, 1, 0) - F(1, -1, 0);
        t2 = F(0, 0, 1) - F(0, 0, -1) + F(1, 0, 1) - F(1, 0, -1);
        const double nxu = sqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
        t0 = F(0, 0, 0) - F(-1, 0, 0);
        t1 = F(-1, 1, 0) - F(-1, -1, 0) + F(0, 1, 0) - F(0, -1, 0);
        t2 = F(-1, 0, 1) - F(-1, 0, -1) + F(0, 0, 1) - F(0, 0, -1);
        const double nxd = sqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
        t0 = F(0, 1, 0) - F(0, 0, 0);
        t1 = F(1, 1, 0) - F(-1, 1, 0) + F(1, 0, 0) - F(-1, 0, 0);
        t2 = F(0, 1, 1) - F(0, 1, -1) + F(0, 0, 1) - F(0, 0, -1);
        const double nyu = sqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
        t0 = F(0, 0, 0) - F(0, -1, 0);
        t1 = F(1, 0, 0) - F(-1, 0, 0) + F(1, -1, 0) - F(-1, -1, 0);
        t2 = F(0, 0, 1) - F(0, 0, -1) + F(0, -1, 1) - F(0, -1, -1);
        const double nyd = sqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
        t0 = F(0, 0, 1) - F(0, 0, 0);
        t1 = F(1, 0, 0) - F(-1, 0, 0) + F(1, 0, 1) - F(-1, 0, 1);
        t2 = F(0, 1, 0) - F(0, -1, 0) + F(0, 1, 1) - F(0, -1, 1);
        const double nzu = sqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
        t0 = F(0, 0, 0) - F(0, 0, -1);
        t1 = F(1, 0, -1) - F(-1, 0, -1) + F(1, 0, 0) - F(-1, 0, 0);
        t2 = F(0, 1, -1) - F(0, -1, -1) + F(0, 1, 0) - F(0, -1, 0);
        const double nzd = sqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
        const double d1x = (F(1, 0, 0) - F(0, 0, 0)) / nxu;
        const double d2x = (F(0, 0, 0) - F(-1, 0, 0)) / nxd;
        const double d1y = (F(0, 1, 0) - F(0, 0, 0)) / nyu;
        const double d2y = (F(0, 0, 0) - F(0, -1, 0)) / nyd;
        const double d1z = (F(0, 0, 1) - F(0, 0, 0)) / nzu;
        const double d2z = (F(0, 0, 0) - F(0, 0, -1)) / nzd;
#undef F
        w11[IX(i, j, k)] = -(d1x - d2x + d1y - d2y + d1z - d2z);
      }
}

/* SGIP, main.f:2835-3026: CSF-type force with the curvature of the filtered
 * volume fraction (the terms summed in SGIP's own order) weighted by the jump
 * of the mean interface height between neighbouring cells; on the wall plane
 * j = 2 a contact-angle model sets the direction.  Same scratch aliasing as
 * csf: w11 = pressure array, w22 = residual array, w33 = rhs array. */
void ora_sgip(ora_state *st) {
  const int nx = st->nx, ny = st->ny, nz = st->nz, ng = st->s.ng;
  const size_t n = (size_t)nx * ny * nz;
  double *ccc = LV(ng, LCC), *w11 = LV(ng, LU), *w22 = LV(ng, LRES), *w33 = LV(ng, LRHS);
  double *ccf = zalloc(n);
  memcpy(ccf, ccc, n * sizeof(double));
  ora_filterc27(ccf, w22, nx, ny, nz);
  memcpy(ccf, w22, n * sizeof(double));
  ora_bc_out(ccf, nx, ny, nz);
  if (st->s.sigma == 0.0) {
    memset(st->s11, 0, n * 8); memset(st->s22, 0, n * 8); memset(st->s33, 0, n * 8);
    memset(st->s12, 0, n * 8); memset(st->s13, 0, n * 8); memset(st->s23, 0, n * 8);
    free(ccf);
    return;
  }
  const double tau = st->s.tau, h = st->s.h;
  const double sigh = 0.5 * (tau * tau) * st->s.sigma / (h * h * h);
  sgip_curvature(w11, ccf, nx, ny, nz);
  ora_bc_out(w11, nx, ny, nz);
  const size_t sy = (size_t)nx, sz = (size_t)nx * ny;
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        const size_t q = IX(i, j, k);
        const double Lx = (st->hx1[q] + st->hx0[q]) / 2.0, Lxd = (st->hx1[q - 1] + st->hx0[q - 1]) / 2.0;
        const double Ly = (st->hy1[q] + st->hy0[q]) / 2.0, Lyd = (st->hy1[q - sy] + st->hy0[q - sy]) / 2.0;
        const double Lz = (st->hz1[q] + st->hz0[q]) / 2.0, Lzd = (st->hz1[q - sz] + st->hz0[q - sz]) / 2.0;
        st->s11[q] = sigh * (w11[q] + w11[q - 1]) * (ccf[q + 1] - ccf[q - 1]) * fabs(Lx - Lxd) / 2.0;
        st->s22[q] = sigh * (w11[q] + w11[q - sy]) * (ccf[q + sy] - ccf[q - sy]) * fabs(Ly - Lyd) / 2.0;
        st->s33[q] = sigh * (w11[q] + w11[q - sz]) * (ccf[q + sz] - ccf[q - sz]) * fabs(Lz - Lzd) / 2.0;
        if (j == 2) {
          /* contact angle from the contact-line speed (degrees; dsind/dcosd) */
          const double mx = ccf[q + 1] - ccf[q - 1], mz = ccf[q + sz] - ccf[q - sz];
          const double mmx = mx / sqrt(mz * mz + mx * mx + 1.e-50), mmz = mz / sqrt(mz * mz + mx * mx + 1.e-50);
          double normv = mmx * st->u[q] + mmz * st->w[q];
          normv = -normv;
          double theta;
          if (fabs(normv) > (double)0.1f) theta = normv > 0 ? 115.0 : 45.0;
          else theta = 350.0 * normv + 80.0;
          const double my = ccf[q + sy] - ccf[q - sy];
          const double rad = theta * (3.14159265358979323846 / 180.0);
          const double sind = sin(rad), mmy = cos(rad);
          st->s11[q] = sigh * (w11[q] + w11[q - 1]) * mx * sind / 2.0;
          st->s22[q] = sigh * (w11[q] + w11[q - sy]) * mmy * sqrt(mz * mz + mx * mx + my * my) * -1.0;
          st->s33[q] = sigh * (w11[q] + w11[q - sz]) * mz * sind / 2.0;
        }
      }
  ora_bc_out(st->s11, nx, ny, nz);
  ora_bc_out(st->s22, nx, ny, nz);
  ora_bc_out(st->s33, nx, ny, nz);
  memcpy(w11, st->s11, n * 8);
  memcpy(w22, st->s22, n * 8);
  memcpy(w33, st->s33, n * 8);
  free(ccf);
}

/* SGIP2, main.f:3029-3166: three filter passes, sigh = 0.5 tau sigma / h^2,
 * SGIP's curvature, central differences of the mean heights (no wall model,
 * no bc_out of the forces). */
void ora_sgip2(ora_state *st) {
  const int nx = st->nx, ny = st->ny, nz = st->nz, ng = st->s.ng;
  const size_t n = (size_t)nx * ny * nz;
  double *ccc = LV(ng, LCC), *w11 = LV(ng, LU), *w22 = LV(ng, LRES), *w33 = LV(ng, LRHS);
  double *ccf = zalloc(n);
  memcpy(ccf, ccc, n * sizeof(double));
  for (int pass = 0; pass < 3; pass++) {
    ora_filterc27(ccf, w22, nx, ny, nz);
    memcpy(ccf, w22, n * sizeof(double));
    ora_bc_out(ccf, nx, ny, nz);
  }
  if (st->s.sigma == 0.0) {
    memset(st->s11, 0, n * 8); memset(st->s22, 0, n * 8); memset(st->s33, 0, n * 8);
    memset(st->s12, 0, n * 8); memset(st->s13, 0, n * 8); memset(st->s23, 0, n * 8);
    free(ccf);
    return;
  }
  const double tau = st->s.tau, h = st->s.h;
  const double sigh = 0.5 * tau * st->s.sigma / (h * h);
  sgip_curvature(w11, ccf, nx, ny, nz);
  ora_bc_out(w11, nx, ny, nz);
  const size_t sy = (size_t)nx, sz = (size_t)nx * ny;
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        const size_t q = IX(i, j, k);
        const double Lxu = (st->hx1[q + 1] + st->hx0[q + 1]) / 2.0, Lxd = (st->hx1[q - 1] + st->hx0[q - 1]) / 2.0;
        const double Lyu = (st->hy1[q + sy] + st->hy0[q + sy]) / 2.0, Lyd = (st->hy1[q - sy] + st->hy0[q - sy]) / 2.0;
        const double Lzu = (st->hz1[q + sz] + st->hz0[q + sz]) / 2.0, Lzd = (st->hz1[q - sz] + st->hz0[q - sz]) / 2.0;
        st->s11[q] = sigh * (w11[q + 1] + w11[q - 1]) * (ccf[q + 1] - ccf[q - 1]) * (Lxu - Lxd) * 0.25;
        st->s22[q] = sigh * (w11[q + sy] + w11[q - sy]) * (ccf[q + sy] - ccf[q - sy]) * (Lyu - Lyd) * 0.25;
        st->s33[q] = sigh * (w11[q + sz] + w11[q - sz]) * (ccf[q + sz] - ccf[q - sz]) * (Lzu - Lzd) * 0.25;
      }
  memcpy(w11, st->s11, n * 8);
  memcpy(w22, st->s22, n * 8);
  memcpy(w33, st->s33, n * 8);
  free(ccf);
}

int ora_error(const ora_state *st, long long *cell) {
  if (cell) *cell = st->error_cell;
  return st->error;
}

/* ======================================================================= */
/* k-epsilon turbulence (iturb = 3)                                          */
/* ======================================================================= */

/* Initial ktur, eps, mut of the drop (deviation: the reference never sets
 * them for the drop, so kepsmodel divides 0/0 on its first step).  The
 * values follow inijet's jet formulas (main.f:536-549): ktur = 0.00015 v^2
 * with v the liquid speed in the liquid and (v2 + 0.01 |v1 - v2|) in the gas,
 * eps = 0.09 rho ktur^2 / mu, mut = 0.09 rho ktur^2 / eps, with v the speed
 * of the phase's velocity vector (inijet uses the x component, which is 0 for
 * a drop falling along y) and the two phases mixed by the volume fraction.
 * REAL literals as in the source (0.00015, 0.01, 0.09 single precision). */
static void keps_seed(ora_state *st) {
  const int nx = st->nx, ny = st->ny, nz = st->nz;
  const ora_scalars *s = &st->s;
  const double *cc = st->lv[s->ng][LCC];
  const double v1 = sqrt(s->xvel1 * s->xvel1 + s->yvel1 * s->yvel1 + s->zvel1 * s->zvel1);
  const double v2 = sqrt(s->xvel2 * s->xvel2 + s->yvel2 * s->yvel2 + s->zvel2 * s->zvel2);
  const double dv = sqrt((s->xvel1 - s->xvel2) * (s->xvel1 - s->xvel2) + (s->yvel1 - s->yvel2) * (s->yvel1 - s->yvel2) +
                         (s->zvel1 - s->zvel2) * (s->zvel1 - s->zvel2));
  const double k1 = (double)0.00015f * v1 * v1;
  const double g = v2 + dv * (double)0.01f;
  const double k2 = (double)0.00015f * (g * g);
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        const size_t q = IX(i, j, k);
        const double kt = cc[q] * k1 + (1.0 - cc[q]) * k2;
        st->ktur[q] = kt;
        st->eps[q] = kt > 0.0 ? (double)0.09f * st->rhon[q] * kt * kt / st->mun[q] : 0.0;
        st->mut[q] = kt > 0.0 ? (double)0.09f * st->rhon[q] * kt * kt / st->eps[q] : 0.0;
      }
}

/* fturbdif, main.f:1239-1267: turbulent diffusion of the volume fraction in
 * y and z, updated in place in the loop order i, j, k (cells (i,j-1,k) and
 * (i,j,k-1) are already new when (i,j,k) is computed), then bc_c.  The
 * FINDMIN/FMODMAX warning print has no effect on the state. */
static void fturbdif(ora_state *st, double *cc) {
  const int nx = st->nx, ny = st->ny, nz = st->nz;
  const double *mut = st->mut, *rh = st->rhon;
  const double ftr = 1.0 * (double)st->s.tauh2 * 1.0 / 2.0;
  const size_t sy = (size_t)nx, sz = (size_t)nx * ny;
  for (int i = 2; i <= nx - 1; i++)
    for (int j = 2; j <= ny - 1; j++)
      for (int k = 2; k <= nz - 1; k++) {
        const size_t q = IX(i, j, k);
        const double m0 = mut[q] / rh[q];
        cc[q] = cc[q] + ftr * ((m0 + mut[q + sy] / rh[q + sy]) * (cc[q + sy] - cc[q]) -
                               (m0 + mut[q - sy] / rh[q - sy]) * (cc[q] - cc[q - sy]) +
                               (m0 + mut[q + sz] / rh[q + sz]) * (cc[q + sz] - cc[q]) -
                               (m0 + mut[q - sz] / rh[q - sz]) * (cc[q] - cc[q - sz]));
      }
  bc_c(cc, nx, ny, nz);
}

/* kepsmodel, main.f:1888-2025 with iturb = 3: explicit update of ktur and eps
 * (upwind convection, variable-coefficient diffusion, production from the
 * strain of the staggered velocity), new values into the scratch arrays the
 * reference passes (kturnew = the pressure array, epsnew = the residual
 * array, main.f:39-40), then ktur, eps, mut = cmu rho k^2/eps on the
 * interior and bc_scalar on all three. */
static void kepsmodel(ora_state *st) {
  const int nx = st->nx, ny = st->ny, nz = st->nz, ng = st->s.ng;
  const double *u = st->u, *v = st->v, *w = st->w, *mun = st->mun, *rhon = st->rhon, *mut = st->mut;
  double *ktur = st->ktur, *eps = st->eps;
  double *kn = LV(ng, LU), *en = LV(ng, LRES);
  const double sigk = 1.0, sige = 1.3, c1 = 1.44, c2 = 1.92, cmu = 0.09;
  const double h = st->s.h, tau = st->s.tau, h2 = h * h, h22 = h2 * 2.0;
  const size_t sy = (size_t)nx, sz = (size_t)nx * ny;
  for (int j = 2; j <= ny - 1; j++)
    for (int i = 2; i <= nx - 1; i++)
      for (int k = 2; k <= nz - 1; k++) {
        const size_t q = IX(i, j, k);
        const double *K = ktur, *E = eps;
        double conv = (dmax1(u[q + 1], 0.0) * K[q] + dmin1(u[q + 1], 0.0) * K[q + 1] -
                       dmax1(u[q], 0.0) * K[q - 1] - dmin1(u[q], 0.0) * K[q] +
                       dmax1(v[q + sy], 0.0) * K[q] + dmin1(v[q + sy], 0.0) * K[q + sy] -
                       dmax1(v[q], 0.0) * K[q - sy] - dmin1(v[q], 0.0) * K[q] +
                       dmax1(w[q + sz], 0.0) * K[q] + dmin1(w[q + sz], 0.0) * K[q + sz] -
                       dmax1(w[q], 0.0) * K[q - sz] - dmin1(w[q], 0.0) * K[q]) / h;
        double cip = mun[q + 1] + mun[q] + (mut[q] + mut[q + 1]) / sigk;
        double cim = mun[q - 1] + mun[q] + (mut[q] + mut[q - 1]) / sigk;
        double cjp = mun[q + sy] + mun[q] + (mut[q] + mut[q + sy]) / sigk;
        double cjm = mun[q - sy] + mun[q] + (mut[q] + mut[q - sy]) / sigk;
        double ckp = mun[q + sz] + mun[q] + (mut[q] + mut[q + sz]) / sigk;
        double ckm = mun[q - sz] + mun[q] + (mut[q] + mut[q - sz]) / sigk;
        double diff = 1.0 / (rhon[q] * h22) *
                      (cip * (K[q + 1] - K[q]) - cim * (K[q] - K[q - 1]) + cjp * (K[q + sy] - K[q]) -
                       cjm * (K[q] - K[q - sy]) + ckp * (K[q + sz] - K[q]) - ckm * (K[q] - K[q - sz]));
        const double dudx = u[q + 1] - u[q];
        const double dudy = 0.25 * (u[q] - u[q - sy] + u[q + 1] - u[q + 1 - sy] + u[q + sy] - u[q] +
                                    u[q + 1 + sy] - u[q + 1]);
        const double dudz = 0.25 * (u[q] - u[q - sz] + u[q + 1] - u[q + 1 - sz] + u[q + sz] - u[q] +
                                    u[q + 1 + sz] - u[q + 1]);
        const double dvdx = 0.25 * (v[q] - v[q - 1] + v[q + 1] - v[q] + v[q + sy] - v[q - 1 + sy] +
                                    v[q + 1 + sy] - v[q + sy]);
        const double dvdy = v[q + sy] - v[q];
        const double dvdz = 0.25 * (v[q] - v[q - sz] + v[q + sz] - v[q] + v[q + sy] - v[q + sy - sz] +
                                    v[q + sy + sz] - v[q + sy]);
        const double dwdx = 0.25 * (w[q] - w[q - 1] + w[q + 1] - w[q] + w[q + sz] - w[q - 1 + sz] +
                                    w[q + 1 + sz] - w[q + sz]);
        const double dwdy = 0.25 * (w[q] - w[q - sy] + w[q + sz] - w[q - sy + sz] + w[q + sy] - w[q] +
                                    w[q + sy + sz] - w[q + sz]);
        const double dwdz = w[q + sz] - w[q];
        double prod = mut[q] / rhon[q] / h2 *
                      (2.0 * (dudx * dudx + dvdy * dvdy + dwdz * dwdz + dvdx * dudy + dwdx * dudz + dvdz * dwdy) +
                       dudy * dudy + dudz * dudz + dvdx * dvdx + dvdz * dvdz + dwdx * dwdx + dwdy * dwdy);
        kn[q] = K[q] + tau * (-conv + diff + prod - E[q]);
        conv = (dmax1(u[q + 1], 0.0) * E[q] + dmin1(u[q + 1], 0.0) * E[q + 1] - dmax1(u[q], 0.0) * E[q - 1] -
                dmin1(u[q], 0.0) * E[q] + dmax1(v[q + sy], 0.0) * E[q] + dmin1(v[q + sy], 0.0) * E[q + sy] -
                dmax1(v[q], 0.0) * E[q - sy] - dmin1(v[q], 0.0) * E[q] + dmax1(w[q + sz], 0.0) * E[q] +
                dmin1(w[q + sz], 0.0) * E[q + sz] - dmax1(w[q], 0.0) * E[q - sz] - dmin1(w[q], 0.0) * E[q]) /
               h;
        cip = mun[q + 1] + mun[q] + (mut[q] + mut[q + 1]) / sige;
        cim = mun[q - 1] + mun[q] + (mut[q] + mut[q - 1]) / sige;
        cjp = mun[q + sy] + mun[q] + (mut[q] + mut[q + sy]) / sige;
        cjm = mun[q - sy] + mun[q] + (mut[q] + mut[q - sy]) / sige;
        ckp = mun[q + sz] + mun[q] + (mut[q] + mut[q + sz]) / sige;
        ckm = mun[q - sz] + mun[q] + (mut[q] + mut[q - sz]) / sige;
        diff = 1.0 / (rhon[q] * h22) *
               (cip * (E[q + 1] - E[q]) - cim * (E[q] - E[q - 1]) + cjp * (E[q + sy] - E[q]) -
                cjm * (E[q] - E[q - sy]) + ckp * (E[q + sz] - E[q]) - ckm * (E[q] - E[q - sz]));
        prod = prod * c1 * E[q] / K[q];
        en[q] = E[q] + tau * (-conv + diff + prod - c2 * E[q] * E[q] / K[q]);
      }
  for (int j = 2; j <= ny - 1; j++)
    for (int i = 2; i <= nx - 1; i++)
      for (int k = 2; k <= nz - 1; k++) {
        const size_t q = IX(i, j, k);
        ktur[q] = kn[q];
        eps[q] = en[q];
        st->mut[q] = cmu * rhon[q] * ktur[q] * ktur[q] / eps[q];
      }
  ora_bc_scalar(ktur, nx, ny, nz);
  ora_bc_scalar(eps, nx, ny, nz);
  ora_bc_scalar(st->mut, nx, ny, nz);
}

void ora_vofmethod(ora_state *st) {
  const int ng = st->s.ng;
  double *cc = LV(ng, LCC), *s1 = LV(ng, LEI), *s2 = LV(ng, LRES), *s3 = LV(ng, LRHS);
  st->s.tswap = st->s.tswap + 1;
  if (st->s.tswap > 3) st->s.tswap = 1;
  if (st->s.tswap % 3 == 0) {
    ora_swp(st, st->w, cc, s1, s2, s3, 3);
    ora_swp(st, st->u, cc, s1, s2, s3, 1);
    ora_swp(st, st->v, cc, s1, s2, s3, 2);
  } else if (st->s.tswap % 2 == 0) {
    ora_swp(st, st->v, cc, s1, s2, s3, 2);
    ora_swp(st, st->w, cc, s1, s2, s3, 3);
    ora_swp(st, st->u, cc, s1, s2, s3, 1);
  } else {
    ora_swp(st, st->u, cc, s1, s2, s3, 1);
    ora_swp(st, st->v, cc, s1, s2, s3, 2);
    ora_swp(st, st->w, cc, s1, s2, s3, 3);
  }
  bc_c(cc, st->nx, st->ny, st->nz);
  if (st->in.iturb != 0) fturbdif(st, cc);
  calcrho(st);
}

/* checktime, main.f:2152-2171 */
void ora_checktime(ora_state *st) {
  double cfl1 = cfl(st);
  const double maxcfl = st->in.maxcfl;
  const double h = st->s.h;
  if (cfl1 > maxcfl) {
    st->s.tau = st->s.tau * (maxcfl * (double)0.8f) / cfl1;
    st->s.tauh = st->s.tau / h;
    st->s.tauh2 = (int)(st->s.tau / (h * h));
  }
  if (cfl1 <= maxcfl * (double)0.25f) {
    cfl1 = maxcfl * (double)0.5f;
    st->s.tau = st->s.tau * (maxcfl * (double)0.5f) / cfl1;
    st->s.tauh = st->s.tau / h;
    st->s.tauh2 = (int)(st->s.tau / (h * h));
  }
  st->s.time = st->s.time + st->s.tau;
}

/* ======================================================================= */
/* CSF surface tension                                                     */
/* ======================================================================= */

/* filterc27, main.f:5473-5511 (weights are default-REAL literals) */
void ora_filterc27(const double *cc, double *cf, int nx, int ny, int nz) {
  const double w0 = (double)0.2729f, w1 = (double)0.08185f, w2 = (double)0.0178f, w3 = (double)0.0028f;
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
#define C(di, dj, dk) cc[IX(i + (di), j + (dj), k + (dk))]
        double s6 = C(-1, 0, 0) + C(1, 0, 0) + C(0, -1, 0) + C(0, 1, 0) + C(0, 0, 1) + C(0, 0, -1);
        double s12 = C(-1, -1, 0) + C(-1, 1, 0) + C(1, -1, 0) + C(1, 1, 0) + C(0, 1, 1) + C(0, -1, 1) + C(1, 0, 1) +
                     C(-1, 0, 1) + C(0, 1, -1) + C(0, -1, -1) + C(1, 0, -1) + C(-1, 0, -1);
        double s8 = C(1, 1, 1) + C(1, 1, -1) + C(1, -1, 1) + C(1, -1, -1) + C(-1, 1, 1) + C(-1, 1, -1) +
                    C(-1, -1, 1) + C(-1, -1, -1);
        double x = w0 * C(0, 0, 0) + w1 * s6 + w2 * s12 + w3 * s8;
#undef C
        if (x > 1.0) x = 1.0;
        cf[IX(i, j, k)] = x;
      }
}

/* csf, main.f:2363-2481.  Scratch aliasing as in the reference: w11 is the
 * pressure array, w22 the fine residual array, w33 the fine rhs array. */
/* csf's curvature (main.f:2402-2451): six face-normal magnitudes of the
 * filtered fraction with transverse 4-point means (+1e-50 inside the root),
 * kappa = -(d1x-d2x+d1y-d2y+d1z-d2z) at interior cells, then bc_out. */
void ora_csf_curvature(double *w11, const double *ccf, int nx, int ny, int nz) {
  for (int j = 2; j <= ny - 1; j++)
    for (int i = 2; i <= nx - 1; i++)
      for (int k = 2; k <= nz - 1; k++) {
#define F(di, dj, dk) ccf[IX(i + (di), j + (dj), k + (dk))]
        double t0, t1, t2;
        t0 = F(1, 0, 0) - F(0, 0, 0);
        t1 = F(0, 1, 0) - F(0, -1, 0) + F(1, 1, 0) - F(1, -1, 0);
        t2 = F(0, 0, 1) - F(0, 0, -1) + F(1, 0, 1) - F(1, 0, -1);
        double nxu = sqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
        t0 = F(0, 0, 0) - F(-1, 0, 0);
        t1 = F(0, 1, 0) - F(0, -1, 0) + F(-1, 1, 0) - F(-1, -1, 0);
        t2 = F(0, 0, 1) - F(0, 0, -1) + F(-1, 0, 1) - F(-1, 0, -1);
        double nxd = sqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
        t0 = F(0, 1, 0) - F(0, 0, 0);
        t1 = F(1, 0, 0) - F(-1, 0, 0) + F(1, 1, 0) - F(-1, 1, 0);
        t2 = F(0, 0, 1) - F(0, 0, -1) + F(0, 1, 1) - F(0, 1, -1);
        double nyu = sqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
        t0 = F(0, 0, 0) - F(0, -1, 0);
        t1 = F(1, 0, 0) - F(-1, 0, 0) + F(1, -1, 0) - F(-1, -1, 0);
        t2 = F(0, 0, 1) - F(0, 0, -1) + F(0, -1, 1) - F(0, -1, -1);
        double nyd = sqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
        t0 = F(0, 0, 1) - F(0, 0, 0);
        t1 = F(1, 0, 0) - F(-1, 0, 0) + F(1, 0, 1) - F(-1, 0, 1);
        t2 = F(0, 1, 0) - F(0, -1, 0) + F(0, 1, 1) - F(0, -1, 1);
        double nzu = sqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
        t0 = F(0, 0, 0) - F(0, 0, -1);
        t1 = F(1, 0, 0) - F(-1, 0, 0) + F(1, 0, -1) - F(-1, 0, -1);
        t2 = F(0, 1, 0) - F(0, -1, 0) + F(0, 1, -1) - F(0, -1, -1);
        double nzd = sqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
        double d1x = (F(1, 0, 0) - F(0, 0, 0)) / nxu;
        double d2x = (F(0, 0, 0) - F(-1, 0, 0)) / nxd;
        double d1y = (F(0, 1, 0) - F(0, 0, 0)) / nyu;
        double d2y = (F(0, 0, 0) - F(0, -1, 0)) / nyd;
        double d1z = (F(0, 0, 1) - F(0, 0, 0)) / nzu;
        double d2z = (F(0, 0, 0) - F(0, 0, -1)) / nzd;
#undef F
        w11[IX(i, j, k)] = -(d1x - d2x + d1y - d2y + d1z - d2z);
      }
  ora_bc_out(w11, nx, ny, nz);
}

void ora_csf(ora_state *st) {
  const int nx = st->nx, ny = st->ny, nz = st->nz, ng = st->s.ng;
  const size_t n = (size_t)nx * ny * nz;
  double *ccc = LV(ng, LCC), *w11 = LV(ng, LU), *w22 = LV(ng, LRES), *w33 = LV(ng, LRHS);
  double *ccf = zalloc(n);
  memcpy(ccf, ccc, n * sizeof(double));
  ora_filterc27(ccf, w22, nx, ny, nz);
  memcpy(ccf, w22, n * sizeof(double));
  ora_bc_out(ccf, nx, ny, nz);
  if (st->s.sigma == 0.0) {
    memset(st->s11, 0, n * 8); memset(st->s22, 0, n * 8); memset(st->s33, 0, n * 8);
    memset(st->s12, 0, n * 8); memset(st->s13, 0, n * 8); memset(st->s23, 0, n * 8);
    free(ccf);
    return;
  }
  const double tau = st->s.tau, h = st->s.h;
  const double sigh = 0.5 * (tau * tau) * st->s.sigma / (h * h * h);
  ora_csf_curvature(w11, ccf, nx, ny, nz);
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        double kap = w11[IX(i, j, k)];
        st->s11[IX(i, j, k)] = sigh * (ccf[IX(i, j, k)] - ccf[IX(i - 1, j, k)]) * kap;
        st->s22[IX(i, j, k)] = sigh * (ccf[IX(i, j, k)] - ccf[IX(i, j - 1, k)]) * kap;
        st->s33[IX(i, j, k)] = sigh * (ccf[IX(i, j, k)] - ccf[IX(i, j, k - 1)]) * kap;
      }
  memcpy(w11, st->s11, n * 8);
  memcpy(w22, st->s22, n * 8);
  memcpy(w33, st->s33, n * 8);
  bc_tensor(st);
  free(ccf);
}

/* ======================================================================= */
/* momentum + projection                                                   */
/* ======================================================================= */

/* solvelpres, main.f:3236-3439 (laminar: mut, turbst, u2p.. are zero, so the
 * terms they feed add exact zeros and are left out). */
void ora_solvelpres(ora_state *st, int t) {
  const int nx = st->nx, ny = st->ny, nz = st->nz, ng = st->s.ng;
  double *cc = LV(ng, LCC), *w1 = LV(ng, LU), *w2 = LV(ng, LRES), *w3 = LV(ng, LRHS);
  double *a = LV(ng, LA), *b = LV(ng, LB), *c = LV(ng, LC), *ei = LV(ng, LEI);
  double *u = st->u, *v = st->v, *w = st->w;
  double *S11 = st->s11, *S22 = st->s22, *S33 = st->s33, *S12 = st->s12, *S13 = st->s13, *S23 = st->s23;
  const double tauh2 = (double)st->s.tauh2, mu1 = st->s.mu1, mu2 = st->s.mu2;
  const double tau = st->s.tau, h = st->s.h, tauh = st->s.tauh;
  double r20 = tauh2 * mu2;
  double r10 = 0.25 * tauh2 * (mu1 - mu2);
  double r1 = 2.0 * tauh2 * (mu1 - mu2);
  double r2 = 2.0 * tauh2 * mu2;
  double stdgrav = st->s.g * (tau * tau) / h;
  double horgrav = st->s.g1 * (tau * tau) / h;
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        size_t q = IX(i, j, k);
        double temp = r2 + r1 * cc[q];
        S11[q] = -S11[q] + temp * (u[IX(i + 1, j, k)] - u[q]);
        S22[q] = -S22[q] + temp * (v[IX(i, j + 1, k)] - v[q]);
        S33[q] = -S33[q] + temp * (w[IX(i, j, k + 1)] - w[q]);
        temp = r20 + r10 * (cc[q] + cc[IX(i - 1, j, k)] + cc[IX(i, j - 1, k)] + cc[IX(i - 1, j - 1, k)]);
        S12[q] = -S12[q] + temp * (u[q] - u[IX(i, j - 1, k)] + v[q] - v[IX(i - 1, j, k)]);
        temp = r20 + r10 * (cc[q] + cc[IX(i - 1, j, k)] + cc[IX(i, j, k - 1)] + cc[IX(i - 1, j, k - 1)]);
        S13[q] = -S13[q] + temp * (u[q] - u[IX(i, j, k - 1)] + w[q] - w[IX(i - 1, j, k)]);
        temp = r20 + r10 * (cc[q] + cc[IX(i, j - 1, k)] + cc[IX(i, j, k - 1)] + cc[IX(i, j - 1, k - 1)]);
        S23[q] = -S23[q] + temp * (v[q] - v[IX(i, j, k - 1)] + w[q] - w[IX(i, j - 1, k)]);
      }
  bc_tensor(st);
  r2 = st->s.rho2;
  r1 = 0.5 * (st->s.rho1 - st->s.rho2);
  ora_abcei(a, b, c, ei, cc, r1, r2, nx, ny, nz);
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        size_t q = IX(i, j, k);
        w1[q] = u[q] + a[IX(i - 1, j, k)] * (S11[q] - S11[IX(i - 1, j, k)] + S12[IX(i, j + 1, k)] - S12[q] +
                                             S13[IX(i, j, k + 1)] - S13[q]) + horgrav;
        w2[q] = v[q] + b[IX(i, j - 1, k)] * (S12[IX(i + 1, j, k)] - S12[q] + S22[q] - S22[IX(i, j - 1, k)] +
                                             S23[IX(i, j, k + 1)] - S23[q]) + stdgrav;
        w3[q] = w[q] + c[IX(i, j, k - 1)] * (S13[IX(i + 1, j, k)] - S13[q] + S23[IX(i, j + 1, k)] - S23[q] +
                                             S33[q] - S33[IX(i, j, k - 1)]);
      }
  bc_w(st, w1, w2, w3);
  /* convective, central scheme (main.f:3525-3566) */
  if (st->in.convectype == 2) {
    for (int k = 2; k <= nz - 1; k++)
      for (int j = 2; j <= ny - 1; j++)
        for (int i = 2; i <= nx - 1; i++) {
#define W1(di, dj, dk) w1[IX(i + (di), j + (dj), k + (dk))]
#define W2(di, dj, dk) w2[IX(i + (di), j + (dj), k + (dk))]
#define W3(di, dj, dk) w3[IX(i + (di), j + (dj), k + (dk))]
          double p, m, x;
          p = W1(0, 0, 0) + W1(-1, 0, 0);
          m = W1(1, 0, 0) + W1(0, 0, 0);
          x = p * p - m * m + (W1(0, -1, 0) + W1(0, 0, 0)) * (W2(0, 0, 0) + W2(-1, 0, 0)) -
              (W1(0, 1, 0) + W1(0, 0, 0)) * (W2(0, 1, 0) + W2(-1, 1, 0)) +
              (W1(0, 0, -1) + W1(0, 0, 0)) * (W3(0, 0, 0) + W3(-1, 0, 0)) -
              (W1(0, 0, 1) + W1(0, 0, 0)) * (W3(0, 0, 1) + W3(-1, 0, 1));
          u[IX(i, j, k)] = W1(0, 0, 0) + tauh * (0.25 * x);
          p = W2(0, 0, 0) + W2(0, -1, 0);
          m = W2(0, 1, 0) + W2(0, 0, 0);
          x = p * p - m * m + (W2(-1, 0, 0) + W2(0, 0, 0)) * (W1(0, 0, 0) + W1(0, -1, 0)) -
              (W2(1, 0, 0) + W2(0, 0, 0)) * (W1(1, 0, 0) + W1(1, -1, 0)) +
              (W2(0, 0, -1) + W2(0, 0, 0)) * (W3(0, 0, 0) + W3(0, -1, 0)) -
              (W2(0, 0, 1) + W2(0, 0, 0)) * (W3(0, 0, 1) + W3(0, -1, 1));
          v[IX(i, j, k)] = W2(0, 0, 0) + tauh * (0.25 * x);
          p = W3(0, 0, 0) + W3(0, 0, -1);
          m = W3(0, 0, 1) + W3(0, 0, 0);
          x = p * p - m * m + (W3(-1, 0, 0) + W3(0, 0, 0)) * (W1(0, 0, 0) + W1(0, 0, -1)) -
              (W3(1, 0, 0) + W3(0, 0, 0)) * (W1(1, 0, 0) + W1(1, 0, -1)) +
              (W3(0, -1, 0) + W3(0, 0, 0)) * (W2(0, 0, 0) + W2(0, 0, -1)) -
              (W3(0, 1, 0) + W3(0, 0, 0)) * (W2(0, 1, 0) + W2(0, 1, -1));
          w[IX(i, j, k)] = W3(0, 0, 0) + tauh * (0.25 * x);
#undef W1
#undef W2
#undef W3
        }
  } else {
    for (int k = 2; k <= nz - 1; k++)
      for (int j = 2; j <= ny - 1; j++)
        for (int i = 2; i <= nx - 1; i++) {
          size_t q = IX(i, j, k);
          u[q] = w1[q];
          v[q] = w2[q];
          w[q] = w3[q];
        }
  }
  bc_v(st);
  const double hi2 = 1.0 / (h * h);
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++)
        w3[IX(i, j, k)] = (u[IX(i + 1, j, k)] - u[IX(i, j, k)] + v[IX(i, j + 1, k)] - v[IX(i, j, k)] +
                           w[IX(i, j, k + 1)] - w[IX(i, j, k)]) * hi2;
  ora_mglin(st);
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        size_t q = IX(i, j, k);
        u[q] = u[q] - (w1[q] - w1[IX(i - 1, j, k)]) * a[IX(i - 1, j, k)];
        v[q] = v[q] - (w1[q] - w1[IX(i, j - 1, k)]) * b[IX(i, j - 1, k)];
        w[q] = w[q] - (w1[q] - w1[IX(i, j, k - 1)]) * c[IX(i, j, k - 1)];
      }
  bc_v(st);
  st->s.last_epsdiv = -1.0;
  if (t <= 1 || t % 10 == 0) {
    /* main.f:3389-3416; the divergence goes into w3 (the fine rhs array) */
    for (int k = 2; k <= nz - 1; k++)
      for (int j = 2; j <= ny - 1; j++)
        for (int i = 2; i <= nx - 1; i++)
          w3[IX(i, j, k)] = (u[IX(i + 1, j, k)] - u[IX(i, j, k)] + v[IX(i, j + 1, k)] - v[IX(i, j, k)] +
                             w[IX(i, j, k + 1)] - w[IX(i, j, k)]) * hi2;
    double epsdiv = h * ora_fmodmax(w3, nx, ny, nz);
    st->s.last_epsdiv = epsdiv;
    if (epsdiv > 25.0 && st->s.ntop < 30) {
      st->s.ntop += 2; st->s.npre += 2; st->s.npost += 2;
    } else if (epsdiv < 2.5 && st->s.ntop > 4) {
      st->s.npre -= 1; st->s.ntop -= 1; st->s.npost -= 1;
    }
  }
  if (t % st->in.tprint == 0) {
    /* main.f:3420-3428: the "check calls" divergence also lands in w3 */
    for (int k = 2; k <= nz - 1; k++)
      for (int j = 2; j <= ny - 1; j++)
        for (int i = 2; i <= nx - 1; i++)
          w3[IX(i, j, k)] = (u[IX(i + 1, j, k)] - u[IX(i, j, k)] + v[IX(i, j + 1, k)] - v[IX(i, j, k)] +
                             w[IX(i, j, k + 1)] - w[IX(i, j, k)]) * hi2;
  }
}

/* ======================================================================= */
/* setup                                                                   */
/* ======================================================================= */

double ora_noise_unit(uint64_t seed, int field, int64_t lin) {
  uint64_t z = seed + 0x9E3779B97F4A7C15ULL * ((((uint64_t)field) << 40) + (uint64_t)lin + 1ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z = z ^ (z >> 31);
  double r = (double)(z >> 11) * (1.0 / 9007199254740992.0);
  return 2.0 * r - 1.0;
}

/* nondim, main.f:341-446 (drop case) */
static void nondim(ora_state *st) {
  const ora_input *in = &st->in;
  ora_scalars *s = &st->s;
  s->lengthscale = in->length_si;
  double dx = in->xvel1_si - in->xvel2_si, dy = in->yvel1_si - in->yvel2_si, dz = in->zvel1_si - in->zvel2_si;
  double vscale = sqrt(dx * dx + dy * dy + dz * dz);
  if (vscale == 0.0) vscale = 1.0; /* the drag branch needs gravity; the drop configs set a velocity */
  s->vscale = vscale;
  double timescale = s->lengthscale / vscale;
  s->lengthsize = in->length_si / s->lengthscale;
  s->h = s->lengthsize / (st->nx - 2);
  s->time = 0.0;
  double tau_si = in->maxcfl * (double)0.8f * (in->length_si / (st->nx - 2)) / vscale;
  s->tau = tau_si / timescale;
  s->tauh = s->tau / s->h;
  s->tauh2 = (int)(s->tau / (s->h * s->h));
  s->tswap = 0;
  s->radius = in->radius_si / s->lengthscale;
  s->xvel1 = in->xvel1_si / vscale; s->yvel1 = in->yvel1_si / vscale; s->zvel1 = in->zvel1_si / vscale;
  s->xvel2 = in->xvel2_si / vscale; s->yvel2 = in->yvel2_si / vscale; s->zvel2 = in->zvel2_si / vscale;
  s->y0 = (st->ny - 2) * s->h / 2;
  s->z0 = (st->nz - 2) * s->h / 2;
  s->rho1 = 1.0;
  s->rho2 = in->rho2_si / in->rho1_si;
  double L = s->lengthscale;
  double denom = in->rho1_si * (L * L) / timescale;
  s->mu1 = in->visc1_si / denom;
  s->mu2 = in->visc2_si / denom;
  denom = in->rho1_si * (L * L * L) / (timescale * timescale);
  s->sigma = in->sigma_si / denom;
  denom = L / (timescale * timescale);
  s->g = in->grav_si / denom;
  s->g1 = in->grav1_si / denom;
}

/* smooth2, main.f:5678-5752.  xx(1), yy(1), zz(1) are read uninitialised by
 * the reference (first cell of each line); they are defined here as
 * (1-1.5)*h, which only matters for a drop touching the first cell. */
static void smooth2(ora_state *st) {
  const int nx = st->nx, ny = st->ny, nz = st->nz, ng = st->s.ng;
  ora_scalars *s = &st->s;
  double *cc = LV(ng, LCC);
  const double h = s->h;
  double x0 = (nx - 2) * h / 4.0;
  if (st->in.z0_si != 1000.0) s->z0 = st->in.z0_si / st->in.length_si;
  if (st->in.y0_si != 1000.0) s->y0 = st->in.y0_si / st->in.length_si;
  s->y0 = s->y0 + h / 2.0;
  const double y0 = s->y0, z0 = s->z0, r2 = s->radius * s->radius;
  double *xx = (double *)malloc(sizeof(double) * (nx + 1));
  double *yy = (double *)malloc(sizeof(double) * (ny + 1));
  double *zz = (double *)malloc(sizeof(double) * (nz + 1));
  for (int i = 1; i <= nx; i++) xx[i] = (double)((float)i - 1.5f) * h;
  for (int j = 1; j <= ny; j++) yy[j] = (double)((float)j - 1.5f) * h;
  for (int k = 1; k <= nz; k++) zz[k] = (double)((float)k - 1.5f) * h;
  for (int i = 2; i <= nx - 1; i++)
    for (int j = 2; j <= ny - 1; j++)
      for (int k = 2; k <= nz - 1; k++) {
        double ax = xx[i - 1] - x0, bx = xx[i] - x0, ay = yy[j - 1] - y0, by = yy[j] - y0;
        double az = zz[k - 1] - z0, bz = zz[k] - z0;
        ax *= ax; bx *= bx; ay *= ay; by *= by; az *= az; bz *= bz;
        if (!(dmin1(ax, bx) + dmin1(ay, by) + dmin1(az, bz) < r2)) {
          cc[IX(i, j, k)] = 0.0;
          continue;
        }
        if (!(dmax1(ax, bx) + dmax1(ay, by) + dmax1(az, bz) > r2)) {
          cc[IX(i, j, k)] = 1.0;
          continue;
        }
        const int index = 30;
        const double inc = 1.0 / (double)(index * index * index);
        double c = 0.0;
        for (int l = 1; l <= index; l++)
          for (int m = 1; m <= index; m++)
            for (int nn = 1; nn <= index; nn++) {
              double px = xx[i - 1] + ((double)l - 0.5) / (double)index * h - x0;
              double py = yy[j - 1] + ((double)m - 0.5) / (double)index * h - y0;
              double pz = zz[k - 1] + ((double)nn - 0.5) / (double)index * h - z0;
              if (px * px + py * py + pz * pz < r2) c = c + inc;
            }
        /* DEVIATION (documented): 27000 additions of 1/27000 can round to
         * 1+4e-13; swp then takes that cell as an interface cell with
         * 1-c < 0 and AL3D returns the cube root of a negative number (NaN).
         * The sampled fraction is clamped to 1. */
        if (c > 1.0) c = 1.0;
        cc[IX(i, j, k)] = c;
      }
  free(xx); free(yy); free(zz);
  bc_c(cc, nx, ny, nz);
  for (int i = 1; i <= nx; i++)
    for (int j = 1; j <= ny; j++)
      for (int k = 1; k <= nz; k++) {
        size_t q = IX(i, j, k);
        st->u[q] = 0.0;
        st->v[q] = s->yvel1 * cc[q] + s->yvel2 * (1 - cc[q]);
        st->w[q] = s->zvel1 * cc[q] + s->zvel2 * (1 - cc[q]);
      }
}

/* Number of multigrid levels.  For min(nx,ny,nz) = 2^k+2 this is the count of
 * memoryaloc (main.f:284-298): halve until the smallest interior extent is 2.
 * Other sides, which the reference stops on (main.f:296-297), coarsen while
 * every interior extent is even and the smallest is at least 4, so the
 * coarsest level may have 3 or 5 interior cells (48, 96 and 160 cells per
 * side end at 3, 3 and 5).  Returns 0 for a grid below 2 interior cells. */
int ora_level_count(int nx, int ny, int nz) {
  int mx = nx - 2, my = ny - 2, mz = nz - 2;
  if (mx < 2 || my < 2 || mz < 2) return 0;
  int ng = 1;
  for (;;) {
    int m = mx < my ? mx : my;
    if (mz < m) m = mz;
    if (m < 4 || (mx & 1) || (my & 1) || (mz & 1) || ng >= 31) break;
    mx /= 2; my /= 2; mz /= 2;
    ng++;
  }
  return ng;
}

ora_state *ora_create(const ora_input *in) {
  ora_state *st = (ora_state *)calloc(1, sizeof(ora_state));
  st->in = *in;
  st->nx = in->nx; st->ny = in->ny; st->nz = in->nz;
  /* memoryaloc, main.f:274-322 */
  const int ng = ora_level_count(in->nx, in->ny, in->nz);
  if (ng < 1) { free(st); return NULL; }
  st->s.ng = ng;
  int nnx = in->nx, nny = in->ny, nnz = in->nz;
  for (int l = ng; l >= 1; l--) {
    st->lnx[l] = nnx; st->lny[l] = nny; st->lnz[l] = nnz;
    size_t n = (size_t)nnx * nny * nnz;
    for (int f = 0; f < 8; f++) st->lv[l][f] = zalloc(n);
    nnx = nnx / 2 + 1; nny = nny / 2 + 1; nnz = nnz / 2 + 1;
  }
  size_t n = (size_t)st->nx * st->ny * st->nz;
  st->u = zalloc(n); st->v = zalloc(n); st->w = zalloc(n);
  st->s11 = zalloc(n); st->s22 = zalloc(n); st->s33 = zalloc(n);
  st->s12 = zalloc(n); st->s13 = zalloc(n); st->s23 = zalloc(n);
  st->rhon = zalloc(n); st->mun = zalloc(n);
  st->ktur = zalloc(n); st->eps = zalloc(n); st->mut = zalloc(n);
  st->hx0 = zalloc(n); st->hx1 = zalloc(n); st->hy0 = zalloc(n);
  st->hy1 = zalloc(n); st->hz0 = zalloc(n); st->hz1 = zalloc(n);
  st->s.npre = in->npre; st->s.npost = in->npost; st->s.ntop = in->ntop; st->s.cycles = in->cycles;
  st->s.last_epsdiv = -1.0;
  nondim(st);
  /* initialize, main.f:121-183 (restart=0, drop case) */
  smooth2(st);
  if (in->noise_si != 0.0) {
    const int nx = st->nx, ny = st->ny, nz = st->nz;
    double amp = in->noise_si / st->s.vscale;
    double *f[3] = {st->u, st->v, st->w};
    for (int q = 0; q < 3; q++)
      for (int k = 2; k <= nz - 1; k++)
        for (int jj = 2; jj <= ny - 1; jj++)
          for (int i = 2; i <= nx - 1; i++) {
            size_t lin = IX(i, jj, k);
            f[q][lin] = f[q][lin] + amp * ora_noise_unit(in->noise_seed, q, (int64_t)lin);
          }
  }
  bc_c(LV(ng, LCC), st->nx, st->ny, st->nz);
  bc_v(st);
  calcrho(st);
  if (in->iturb == 3) keps_seed(st);
  return st;
}

void ora_destroy(ora_state *st) {
  if (!st) return;
  for (int l = 1; l <= st->s.ng; l++)
    for (int f = 0; f < 8; f++) free(st->lv[l][f]);
  free(st->u); free(st->v); free(st->w);
  free(st->s11); free(st->s22); free(st->s33); free(st->s12); free(st->s13); free(st->s23);
  free(st->rhon); free(st->mun);
  free(st->ktur); free(st->eps); free(st->mut);
  free(st->hx0); free(st->hx1); free(st->hy0); free(st->hy1); free(st->hz0); free(st->hz1);
  free(st);
}

int ora_nx(const ora_state *st) { return st->nx; }
int ora_ny(const ora_state *st) { return st->ny; }
int ora_nz(const ora_state *st) { return st->nz; }

double *ora_field(ora_state *st, int id) {
  const int ng = st->s.ng;
  switch (id) {
    case ORA_CC: return LV(ng, LCC);
    case ORA_P: return LV(ng, LU);
    case ORA_RES: return LV(ng, LRES);
    case ORA_RHS: return LV(ng, LRHS);
    case ORA_A: return LV(ng, LA);
    case ORA_B: return LV(ng, LB);
    case ORA_C: return LV(ng, LC);
    case ORA_EI: return LV(ng, LEI);
    case ORA_U: return st->u;
    case ORA_V: return st->v;
    case ORA_W: return st->w;
    case ORA_S11: return st->s11;
    case ORA_S22: return st->s22;
    case ORA_S33: return st->s33;
    case ORA_S12: return st->s12;
    case ORA_S13: return st->s13;
    case ORA_S23: return st->s23;
    case ORA_RHON: return st->rhon;
    case ORA_MUN: return st->mun;
    case ORA_KTUR: return st->ktur;
    case ORA_EPS: return st->eps;
    case ORA_MUT: return st->mut;
    case ORA_HXMIN: return st->hx0;
    case ORA_HXMAX: return st->hx1;
    case ORA_HYMIN: return st->hy0;
    case ORA_HYMAX: return st->hy1;
    case ORA_HZMIN: return st->hz0;
    case ORA_HZMAX: return st->hz1;
    default: return NULL;
  }
}

double *ora_level_field(ora_state *st, int id, int level) {
  if (level < 1 || level > st->s.ng || id < 0 || id > 7) return NULL;
  return st->lv[level][id];
}

void ora_level_dims(const ora_state *st, int level, int *nx, int *ny, int *nz) {
  *nx = st->lnx[level]; *ny = st->lny[level]; *nz = st->lnz[level];
}

void ora_get_scalars(const ora_state *st, ora_scalars *out) { *out = st->s; }
void ora_set_scalars(ora_state *st, const ora_scalars *in) { st->s = *in; }

/* main.f:19-73 loop body: VOFmethod, CalcH3d (hswitch = 1), kepsmodel
 * (iturb = 3), checktime, csf (surfacet = 2) or SGIP (surfacet = 5),
 * solvelpres.  A STOP of CalcH3d ends the step (ora_error reports it). */
void ora_kepsmodel(ora_state *st) {
  if (st->in.iturb == 3) kepsmodel(st);
}

void ora_step(ora_state *st, int t) {
  ora_vofmethod(st);
  if (st->in.hswitch == 1 && ora_calch3d(st)) return;
  ora_kepsmodel(st);
  ora_checktime(st);
  if (st->in.surfacet == 5) ora_sgip(st);
  else if (st->in.surfacet == 6) ora_sgip2(st);
  else ora_csf(st);
  ora_solvelpres(st, t);
}
