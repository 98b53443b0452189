// sgip.cu -- interface heights (CalcH3d, main.f:1312-1810) and the SGIP
// surface-tension forces (SGIP, main.f:2835-3026: the reference's default
// surface tension, surfacet = 5 with hswitch = 1 in its inputdata.in; SGIP2,
// main.f:3029-3166, surfacet = 6).  FP64 without
// FP contraction, the reference's operation order: the height case chosen for
// a cell depends on exact comparisons, so the arithmetic matches the oracle's
// bit for bit.
#include "dsg_internal.cuh"

namespace dsg {
namespace {

__device__ __forceinline__ double cube(double x) { return x * x * x; }

// CalcH3d of one cell: Youngs normal from the 27-point stencil, the PLIC
// polygon's heights on the cell faces in the five geometric cases of the
// ordered normal n1 <= n2 <= n3 (Newton-Raphson, at most 1000 steps, for the
// pentagon and hexagon), assigned to the axes and clipped to [0, 1].
// Returns 0, 1 ("NO MATCH CASES FOUND") or 2 ("PROBLEM finding MIN and MAX").
__device__ int h3d_cell(const double *__restrict__ c, size_t q, long sy, long sz, double h[6]) {
#define C(di, dj, dk) c[(long)q + (long)(di) + (long)(dj) * sy + (long)(dk) * sz]
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
    h1a = s2 * s3 / 2.0;
    h1b = s2 * s3 / 2.0;
    h2a = s3;
    h2b = 0.0;
    h3a = s2;
    h3b = 0.0;
  } else if (n1 == 0.0 && n2 > 0.0 && ccnew > clim1) {
    h1a = cc;
    h1b = cc;
    h2a = cc + n2 / (2.0 * n3);
    h2b = cc - n2 / (2.0 * n3);
    h3a = 1.0;
    h3b = 0.0;
  } else if (n1 == 0.0 && n2 == 0.0) {
    h1a = h1b = h2a = h2b = ccnew;
    h3a = 1.0;
    h3b = 0.0;
  } else if (6.0 * n2 * n3 * ccnew < n1 * n1) {  // triangle, case (a)
    diag = pow(6.0 * n1 * n2 * n3 * ccnew, 1.0 / 3.0);
    s1 = diag / n1, s2 = diag / n2, s3 = diag / n3;
    h1a = (s2 * s3) / 2.0;
    h1b = 0.0;
    h2a = (s1 * s3) / 2.0;
    h2b = 0.0;
    h3a = (s1 * s2) / 2.0;
    h3b = 0.0;
  } else if (6.0 * n2 * n3 * ccnew < 3.0 * (n2 * n2) - 3.0 * n1 * n2 + n1 * n1) {  // quadrilateral A, (b)
    diag = (3.0 * n1 + sqrt(72.0 * n2 * n3 * ccnew - 3.0 * (n1 * n1))) / 6.0;
    s1 = diag / n1, s2 = diag / n2, s3 = diag / n3;
    const double t = (s1 - 1.0) / s1;
    h1a = (s2 * s3) / 2.0;
    h1b = (s2 * s3) / 2.0 * (t * t);
    h2a = s3 * (2.0 * s1 - 1.0) / (2.0 * s1);
    h2b = 0.0;
    h3a = s2 * (2.0 * s1 - 1.0) / (2.0 * s1);
    h3b = 0.0;
  } else if ((n1 + n2 >= n3 && 6.0 * n1 * n2 * n3 * ccnew < cube(n3) - cube(n3 - n1) - cube(n3 - n2)) ||
             (n1 + n2 < n3 && 2.0 * n3 * ccnew < n1 + n2)) {  // pentagon, (c)
    const double rsixn3 = 1.0 / (6.0 * n1 * n2 * n3);
    diag = n2;
    for (int loop = 1; loop <= 1000; loop++) {
      const double delta = -(rsixn3 * (cube(diag) - cube(diag - n1) - cube(diag - n2)) - ccnew) /
                           (3.0 * rsixn3 * (diag * diag - (diag - n1) * (diag - n1) - (diag - n2) * (diag - n2)));
      diag = diag + delta;
      if (fabs(delta) < 1.e-6) break;
    }
    s1 = diag / n1, s2 = diag / n2, s3 = diag / n3;
    const double t1 = (s1 - 1.0) / s1, t2 = (s2 - 1.0) / s2;
    h1a = s3 * (2.0 * s2 - 1.0) / (2.0 * s2);
    h1b = (s2 * s3) / 2.0 * (t1 * t1);
    h2a = s3 * (2.0 * s1 - 1.0) / (2.0 * s1);
    h2b = (s1 * s3) / 2.0 * (t2 * t2);
    h3a = 2.0 * (s1 + s2) - s1 / s2 - s2 / s1 - s1 * s2 - 1.0;
    h3b = 0.0;
  } else if ((n1 + n2 > n3) && 6.0 * n1 * n2 * n3 * ccnew >= cube(n3) - cube(n3 - n1) - cube(n3 - n2)) {
    // hexagon, (d)
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
    s1 = diag / n1, s2 = diag / n2, s3 = diag / n3;
    const double t1 = (s1 - 1.0) / s1, t2 = (s2 - 1.0) / s2, t3 = (s3 - 1.0) / s3;
    h1a = 2.0 * (s2 + s3) - s2 / s3 - s3 / s2 - s2 * s3 - 1.0;
    h1b = (s2 * s3) / 2.0 * (t1 * t1);
    h2a = 2.0 * (s1 + s3) - s1 / s3 - s3 / s1 - s1 * s3 - 1.0;
    h2b = (s1 * s3) / 2.0 * (t2 * t2);
    h3a = 2.0 * (s1 + s2) - s1 / s2 - s2 / s1 - s1 * s2 - 1.0;
    h3b = (s1 * s2) / 2.0 * (t3 * t3);
  } else if ((n1 + n2 < n3) && 6.0 * n1 * n2 * n3 * ccnew >= cube(n1 + n2) - cube(n1) - cube(n2)) {
    // quadrilateral B, (e)
    diag = 0.5 * (n1 + n2) + ccnew * n3;
    s1 = diag / n1, s2 = diag / n2, s3 = diag / n3;
    h1a = s3 * (2.0 * s2 - 1.0) / (2.0 * s2);
    h1b = s3 * (2.0 * s2 - 1.0) * (s1 - 1.0) / (2.0 * s1 * s2);
    h2a = s3 * (2.0 * s1 - 1.0) / (2.0 * s1);
    h2b = s3 * (2.0 * s1 - 1.0) * (s2 - 1.0) / (2.0 * s1 * s2);
    h3a = 1.0;
    h3b = 0.0;
  } else {
    return 1;
  }
  if (cc > 0.5) {
    h1a = 1.0 - h1a, h1b = 1.0 - h1b, h2a = 1.0 - h2a;
    h2b = 1.0 - h2b, h3a = 1.0 - h3a, h3b = 1.0 - h3b;
  }
  // axis assignment (main.f:1586-1735, including the use of niz's sign for y
  // when z carries the smallest component)
  double hx0 = 0, hx1 = 0, hy0 = 0, hy1 = 0, hz0 = 0, hz1 = 0;
  auto set = [](double &lo, double &hi, double n, double a, double b) {
    if (n < 0) {
      lo = a;
      hi = b;
    } else {
      lo = b;
      hi = a;
    }
  };
  if (absxn == n1) {
    set(hx0, hx1, nix, h1a, h1b);
    if (fabs(absyn - n2) < 1.e-6) {
      set(hy0, hy1, niy, h2a, h2b);
      set(hz0, hz1, niz, h3a, h3b);
    } else if (fabs(abszn - n2) < 1.e-6) {
      set(hy0, hy1, niy, h3a, h3b);
      set(hz0, hz1, niz, h2a, h2b);
    } else {
      return 2;
    }
  } else if (absyn == n1) {
    set(hy0, hy1, niy, h1a, h1b);
    if (fabs(absxn - n2) < 1.e-6) {
      set(hx0, hx1, nix, h2a, h2b);
      set(hz0, hz1, niz, h3a, h3b);
    } else if (fabs(abszn - n2) < 1.e-6) {
      set(hx0, hx1, nix, h3a, h3b);
      set(hz0, hz1, niz, h2a, h2b);
    } else {
      return 2;
    }
  } else if (abszn == n1) {
    set(hz0, hz1, niz, h1a, h1b);
    if (fabs(absxn - n2) < 1.e-6) {
      set(hx0, hx1, nix, h2a, h2b);
      set(hy0, hy1, niz, h3a, h3b);
    } else if (fabs(absyn - n2) < 1.e-6) {
      set(hx0, hx1, nix, h3a, h3b);
      set(hy0, hy1, niz, h2a, h2b);
    } else {
      return 2;
    }
  }
  if (cc <= 0.5) {  // exchange min and max
    double t;
    t = hx0, hx0 = hx1, hx1 = t;
    t = hy0, hy0 = hy1, hy1 = t;
    t = hz0, hz0 = hz1, hz1 = t;
  }
  const double o[6] = {hx0, hx1, hy0, hy1, hz0, hz1};
#pragma unroll
  for (int m = 0; m < 6; m++) h[m] = o[m] < 0.0 ? 0.0 : (o[m] > 1.0 ? 1.0 : o[m]);
  return 0;
}

struct Heights {
  double *p[6];  // hxmin, hxmax, hymin, hymax, hzmin, hzmax
};

// Heights of every interior cell.  The first failing cell (a STOP of the
// reference) is recorded as (code << 48 | linear index) in *err.
__global__ void k_calch3d(Heights H, const double *__restrict__ cc, Dims d, unsigned long long *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  double h[6];
  const int rc = h3d_cell(cc, q, (long)d.sy(), (long)d.sz(), h);
  if (rc) {
    atomicCAS(err, 0ull, ((unsigned long long)rc << 48) | (unsigned long long)q);
    return;
  }
#pragma unroll
  for (int m = 0; m < 6; m++) H.p[m][q] = h[m];
}

// SGIP's curvature: csf's face-normal formula with the transverse differences
// summed in SGIP's own order (main.f:2880-2913).
__global__ void k_sgip_curvature(double *__restrict__ kap, const double *__restrict__ f, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  const long sy = (long)d.sy(), sz = (long)d.sz();
#define F(di, dj, dk) f[(long)q + (long)(di) + (long)(dj) * sy + (long)(dk) * sz]
  // uniform 19-point neighbourhood: every difference +0, kappa = -0 exactly
  const double f0 = F(0, 0, 0);
#define EQ(di, dj, dk) same_bits(F(di, dj, dk), f0)
  if (EQ(1, 0, 0) && EQ(-1, 0, 0) && EQ(0, 1, 0) && EQ(0, -1, 0) && EQ(0, 0, 1) && EQ(0, 0, -1) && EQ(1, 1, 0) &&
      EQ(1, -1, 0) && EQ(-1, 1, 0) && EQ(-1, -1, 0) && EQ(1, 0, 1) && EQ(1, 0, -1) && EQ(-1, 0, 1) && EQ(-1, 0, -1) &&
      EQ(0, 1, 1) && EQ(0, 1, -1) && EQ(0, -1, 1) && EQ(0, -1, -1)) {
#undef EQ
    kap[q] = -0.0;
    return;
  }
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
  kap[q] = -(d1x - d2x + d1y - d2y + d1z - d2z);
}

// SGIP's face forces: curvature x filtered-fraction difference x the jump of
// the mean interface height between the cell and its lower neighbour; on the
// wall plane j = 2 the contact-angle model (angle from the contact-line
// speed, sin/cos of degrees as dsind/dcosd).
__global__ void k_sgip_force(double *__restrict__ s11, double *__restrict__ s22, double *__restrict__ s33,
                             const double *__restrict__ f, const double *__restrict__ kap, Heights H,
                             const double *__restrict__ u, const double *__restrict__ w, Dims d, double sigh) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  const size_t sy = d.sy(), sz = d.sz();
  const double Lx = (H.p[1][q] + H.p[0][q]) / 2.0, Lxd = (H.p[1][q - 1] + H.p[0][q - 1]) / 2.0;
  const double Ly = (H.p[3][q] + H.p[2][q]) / 2.0, Lyd = (H.p[3][q - sy] + H.p[2][q - sy]) / 2.0;
  const double Lz = (H.p[5][q] + H.p[4][q]) / 2.0, Lzd = (H.p[5][q - sz] + H.p[4][q - sz]) / 2.0;
  if (j != 2) {
    s11[q] = sigh * (kap[q] + kap[q - 1]) * (f[q + 1] - f[q - 1]) * fabs(Lx - Lxd) / 2.0;
    s22[q] = sigh * (kap[q] + kap[q - sy]) * (f[q + sy] - f[q - sy]) * fabs(Ly - Lyd) / 2.0;
    s33[q] = sigh * (kap[q] + kap[q - sz]) * (f[q + sz] - f[q - sz]) * fabs(Lz - Lzd) / 2.0;
    return;
  }
  const double mx = f[q + 1] - f[q - 1], mz = f[q + sz] - f[q - sz];
  const double mmx = mx / sqrt(mz * mz + mx * mx + 1.e-50), mmz = mz / sqrt(mz * mz + mx * mx + 1.e-50);
  double normv = mmx * u[q] + mmz * w[q];
  normv = -normv;
  double theta;
  if (fabs(normv) > (double)0.1f)
    theta = normv > 0 ? 115.0 : 45.0;
  else
    theta = 350.0 * normv + 80.0;
  const double my = f[q + sy] - f[q - sy];
  const double rad = theta * (3.14159265358979323846 / 180.0);
  const double sind = sin(rad), mmy = cos(rad);
  s11[q] = sigh * (kap[q] + kap[q - 1]) * mx * sind / 2.0;
  s22[q] = sigh * (kap[q] + kap[q - sy]) * mmy * sqrt(mz * mz + mx * mx + my * my) * -1.0;
  s33[q] = sigh * (kap[q] + kap[q - sz]) * mz * sind / 2.0;
}

// SGIP2's face forces (main.f:3124-3140): central differences of the mean
// heights, no wall model.
__global__ void k_sgip2_force(double *__restrict__ s11, double *__restrict__ s22, double *__restrict__ s33,
                              const double *__restrict__ f, const double *__restrict__ kap, Heights H, Dims d,
                              double sigh) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  const size_t sy = d.sy(), sz = d.sz();
  const double Lxu = (H.p[1][q + 1] + H.p[0][q + 1]) / 2.0, Lxd = (H.p[1][q - 1] + H.p[0][q - 1]) / 2.0;
  const double Lyu = (H.p[3][q + sy] + H.p[2][q + sy]) / 2.0, Lyd = (H.p[3][q - sy] + H.p[2][q - sy]) / 2.0;
  const double Lzu = (H.p[5][q + sz] + H.p[4][q + sz]) / 2.0, Lzd = (H.p[5][q - sz] + H.p[4][q - sz]) / 2.0;
  s11[q] = sigh * (kap[q + 1] + kap[q - 1]) * (f[q + 1] - f[q - 1]) * (Lxu - Lxd) * 0.25;
  s22[q] = sigh * (kap[q + sy] + kap[q - sy]) * (f[q + sy] - f[q - sy]) * (Lyu - Lyd) * 0.25;
  s33[q] = sigh * (kap[q + sz] + kap[q - sz]) * (f[q + sz] - f[q - sz]) * (Lzu - Lzd) * 0.25;
}

const dim3 kBlk(32, 4, 1);

}  // namespace

cudaError_t calch3d(double *const H[6], const double *cc, Dims d, unsigned long long *err, cudaStream_t st) {
  Heights h;
  for (int m = 0; m < 6; m++) h.p[m] = H[m];
  DSG_COUNT k_calch3d<<<interior_grid(d, kBlk), kBlk, 0, st>>>(h, cc, d, err);
  return cudaGetLastError();
}

// SGIP2 (main.f:3029-3166): three filter passes (each filterc27 into the
// residual array, copied back, bc_out), sigh = 0.5 tau sigma / h^2, SGIP's
// curvature, SGIP2's forces.
cudaError_t sgip2(const double *ccc, double *w11, double *w22, double *w33, double *ccf, double *const S[6],
                  double *const H[6], Dims d, double tau, double sigma, double h, cudaStream_t st) {
  const size_t bytes = d.count() * sizeof(double);
  cudaError_t e;
  for (int pass = 0; pass < 3; pass++) {
    if ((e = filterc27(pass == 0 ? ccc : ccf, w22, d, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(ccf, w22, bytes, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
    if ((e = bc_out(ccf, d, st)) != cudaSuccess) return e;
  }
  if (sigma == 0.0) {
    for (int m = 0; m < 6; m++)
      if ((e = cudaMemsetAsync(S[m], 0, bytes, st)) != cudaSuccess) return e;
    return cudaSuccess;
  }
  const double sigh = 0.5 * tau * sigma / (h * h);
  DSG_COUNT k_sgip_curvature<<<interior_grid(d, kBlk), kBlk, 0, st>>>(w11, ccf, d);
  if ((e = bc_out(w11, d, st)) != cudaSuccess) return e;
  Heights hh;
  for (int m = 0; m < 6; m++) hh.p[m] = H[m];
  DSG_COUNT k_sgip2_force<<<interior_grid(d, kBlk), kBlk, 0, st>>>(S[0], S[1], S[2], ccf, w11, hh, d, sigh);
  if ((e = cudaMemcpyAsync(w11, S[0], bytes, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(w22, S[1], bytes, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
  return cudaMemcpyAsync(w33, S[2], bytes, cudaMemcpyDeviceToDevice, st);
}

// SGIP with the reference's scratch aliasing (as csf): w11 = pressure array,
// w22 = fine residual array, w33 = fine rhs array; ccf is its local array.
cudaError_t sgip(const double *ccc, double *w11, double *w22, double *w33, double *ccf, double *const S[6],
                 double *const H[6], const double *u, const double *w, Dims d, double tau, double sigma, double h,
                 cudaStream_t st) {
  const size_t bytes = d.count() * sizeof(double);
  cudaError_t e = filterc27(ccc, w22, d, st);
  if (e != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(ccf, w22, bytes, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
  if ((e = bc_out(ccf, d, st)) != cudaSuccess) return e;
  if (sigma == 0.0) {
    for (int m = 0; m < 6; m++)
      if ((e = cudaMemsetAsync(S[m], 0, bytes, st)) != cudaSuccess) return e;
    return cudaSuccess;
  }
  const double sigh = 0.5 * (tau * tau) * sigma / (h * h * h);
  DSG_COUNT k_sgip_curvature<<<interior_grid(d, kBlk), kBlk, 0, st>>>(w11, ccf, d);
  if ((e = bc_out(w11, d, st)) != cudaSuccess) return e;
  Heights hh;
  for (int m = 0; m < 6; m++) hh.p[m] = H[m];
  DSG_COUNT k_sgip_force<<<interior_grid(d, kBlk), kBlk, 0, st>>>(S[0], S[1], S[2], ccf, w11, hh, u, w, d, sigh);
  for (int m = 0; m < 3; m++)
    if ((e = bc_out(S[m], d, st)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(w11, S[0], bytes, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(w22, S[1], bytes, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
  return cudaMemcpyAsync(w33, S[2], bytes, cudaMemcpyDeviceToDevice, st);
}

}  // namespace dsg
