// vof.cu -- PLIC-VOF direction-split advection (VOFmethod/swp, main.f:795-1000),
// the plane/volume relations AL3D/FL3D (main.f:4562-4698), bc_flux
// (main.f:4496-4539), bc_c (main.f:4331-4396) and calcrho (main.f:2177-2190).
//
// One sweep = flux kernel (per cell: left-out, stay, right-out volumes written
// to the three scratch arrays the reference uses: z(iei), z(ires), z(irhs) of
// the finest level) -> bc_flux -> update kernel (c = vof3(i-1)+vof2(i)+vof1(i+1)
// clipped to [0,1]) -> bc_c.  Most cells are empty or full and take the cheap
// branches; interface cells evaluate the Youngs normal, AL3D and up to three
// FL3D calls in FP64.
#include "dsg_internal.cuh"

namespace dsg {
namespace {

// AL3D: plane constant alpha of m1 x1 + m2 x2 + m3 x3 = alpha cutting volume cc
// from the unit cube (m1+m2+m3 = 1, all >= 0).  Scardovelli-Zaleski analytic
// inversion with five regimes.
__device__ double al3d(double b1, double b2, double b3, double cc) {
  double m1 = dmin1(b1, b2), m3 = dmax1(b1, b2), m2 = b3, tmp;
  if (m2 < m1) {
    tmp = m1; m1 = m2; m2 = tmp;
  } else if (m2 > m3) {
    tmp = m3; m3 = m2; m2 = tmp;
  }
  const double m12 = m1 + m2;
  const double pr = dmax1(6.0 * m1 * m2 * m3, 1.0e-50);
  const double V1 = m1 * m1 * m1 / pr;
  const double V2 = V1 + 0.5 * (m2 - m1) / m3;
  double mm, V3;
  if (m3 < m12) {
    mm = m3;
    V3 = (m3 * m3 * (3.0 * m12 - m3) + m1 * m1 * (m1 - 3.0 * m3) + m2 * m2 * (m2 - 3.0 * m3)) / pr;
  } else {
    mm = m12;
    V3 = 0.5 * mm / m3;
  }
  const double ch = dmin1(cc, 1.0 - cc);
  double res;
  if (ch < V1) {
    res = pow(pr * ch, 1.0 / 3.0);
  } else if (ch < V2) {
    res = 0.5 * (m1 + sqrt(m1 * m1 + 8.0 * m2 * m3 * (ch - V1)));
  } else if (ch < V3) {
    const double p = 2.0 * m1 * m2;
    const double q = 1.5 * m1 * m2 * (m12 - 2.0 * m3 * ch);
    const double p12 = sqrt(p);
    double cst = q / (p * p12);
    if (cst > 1.0) cst = 1.0;
    if (cst < -1.0) cst = -1.0;
    const double cs = cos(acos(cst) / 3.0);
    res = p12 * (sqrt(3.0 * (1.0 - cs * cs)) - cs) + m12;
  } else if (mm == m12) {
    res = m3 * ch + 0.5 * mm;
  } else {
    const double p = m1 * (m2 + m3) + m2 * m3 - 0.25;
    const double q = 1.5 * m1 * m2 * m3 * (0.5 - ch);
    const double p12 = sqrt(p);
    double cst = q / (p * p12);
    if (cst > 1.0) cst = 1.0;
    if (cst < -1.0) cst = -1.0;
    const double cs = cos(acos(cst) / 3.0);
    res = p12 * (sqrt(3.0 * (1.0 - cs * cs)) - cs) + 0.5;
  }
  if (cc > 0.5) res = 1.0 - res;
  return res;
}

// FL3D: volume of the part of [r0, r0+dr0] x [0,1]^2 below the plane.
__device__ double fl3d(double m1, double m2, double m3, double alpha, double r0, double dr0) {
  double al = alpha - m1 * r0;
  al = al + dmax1(0.0, -m1 * dr0) + dmax1(0.0, -m2) + dmax1(0.0, -m3);
  double tmp = fabs(m1) * dr0 + fabs(m2) + fabs(m3);
  const double n1 = fabs(m1) / tmp, n2 = fabs(m2) / tmp, n3 = fabs(m3) / tmp;
  al = dmax1(0.0, dmin1(1.0, al / tmp));
  const double al0 = dmin1(al, 1.0 - al);
  double b1 = dmin1(n1 * dr0, n2), b3 = dmax1(n1 * dr0, n2), b2 = n3;
  if (b2 < b1) {
    tmp = b1; b1 = b2; b2 = tmp;
  } else if (b2 > b3) {
    tmp = b3; b3 = b2; b2 = tmp;
  }
  const double b12 = b1 + b2;
  const double bm = dmin1(b12, b3);
  const double pr = dmax1(6.0 * b1 * b2 * b3, 1.0e-50);
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

// Fluxes of one interface cell q (0 < c < 1): Youngs normal from the 27-point
// stencil, AL3D plane constant, Lagrangian stretch along D and the FL3D cut
// volumes (swp, main.f:896-995).
template <int D>
__device__ void iface_flux(size_t q, const double *__restrict__ us, const double *__restrict__ cc,
                           double *__restrict__ vof1, double *__restrict__ vof2, double *__restrict__ vof3, Dims d,
                           double tauh) {
  const long sy = (long)d.sy(), sz = (long)d.sz();
  const long sd = D == 1 ? 1 : (D == 2 ? sy : sz);
  const double a1 = us[q] * tauh;
  const double a2 = us[q + sd] * tauh;
  const double c0 = cc[q];
  double f1 = 0.0, f2 = 0.0, f3 = 0.0;
#define C(di, dj, dk) cc[(long)q + (long)(di) + (long)(dj) * sy + (long)(dk) * sz]
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
    // Deviation from swp: a symmetric neighbourhood gives an all-zero Youngs
    // normal, for which FL3D divides 0/0.  Such a cell is advected as a
    // uniformly filled one (donor-cell fluxes scaled by c).
    vof1[q] = c0 * dmax1(-a1, 0.0);
    vof2[q] = c0 * (1.0 - dmax1(a1, 0.0) + dmin1(a2, 0.0));
    vof3[q] = c0 * dmax1(a2, 0.0);
    return;
  }
  double invx = 1.0, invy = 1.0, invz = 1.0;
  if (mx < 0.0) { mx = -mx; invx = -1.0; }
  if (my < 0.0) { my = -my; invy = -1.0; }
  if (mz < 0.0) { mz = -mz; invz = -1.0; }
  mm2 = mx + my + mz + (double)1.e-30f;  // default-REAL literal of main.f:927
  mx = mx / mm2;
  my = my / mm2;
  mz = mz / mm2;
  double alpha = al3d(mx, my, mz, c0);
  mx = invx * mx;
  my = invy * my;
  mz = invz * mz;
  alpha = alpha + dmin1(0.0, mx) + dmin1(0.0, my) + dmin1(0.0, mz);
  mm1 = dmax1(a1, 0.0);
  mm2 = 1.0 - mm1 + dmin1(0.0, a2);
  // The sweep direction's normal component goes first in FL3D.
  double n1, n2, n3;
  if (D == 1) { n1 = mx; n2 = my; n3 = mz; }
  else if (D == 2) { n1 = my; n2 = mz; n3 = mx; }
  else { n1 = mz; n2 = mx; n3 = my; }
  n1 = n1 / (1.0 - a1 + a2);
  alpha = alpha + n1 * a1;
  if (a1 < 0.0) f1 = fl3d(n1, n2, n3, alpha, a1, -a1);
  if (a2 > 0.0) f3 = fl3d(n1, n2, n3, alpha, 1.0, a2);
  f2 = fl3d(n1, n2, n3, alpha, mm1, mm2);
  vof1[q] = f1;
  vof2[q] = f2;
  vof3[q] = f3;
}

// Sweep fluxes, pass 1: full and empty cells directly (the reference's
// c == 1 and c == 0 branches); interface cells are appended to `list`
// (one atomic per warp) for pass 2, so that the PLIC geometry runs on full
// warps instead of one busy lane per warp.
template <int D>
__global__ void k_swp_flux(const double *__restrict__ us, const double *__restrict__ cc,
                           double *__restrict__ vof1, double *__restrict__ vof2, double *__restrict__ vof3, Dims d,
                           double tauh, unsigned *__restrict__ list, unsigned *__restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  const bool inside = i <= d.nx - 1 && j <= d.ny - 1;
  const size_t q = inside ? d.ix(i, j, k) : 0;
  const double c0 = inside ? cc[q] : 0.0;
  const bool iface = inside && positive_bits(c0) && !is_one_bits(c0);
  // warp-aggregated append (a warp is one x-row of the block)
  const unsigned lane = threadIdx.x & 31;
  const unsigned mask = __ballot_sync(0xffffffffu, iface);
  if (mask) {
    unsigned base = 0;
    const int leader = __ffs(mask) - 1;
    if ((int)lane == leader) base = atomicAdd(count, (unsigned)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (iface) list[base + __popc(mask & ((1u << lane) - 1u))] = (unsigned)q;
  }
  if (!inside || iface) return;
  if (!is_one_bits(c0)) {
    // empty cell: no flux.  It returns before the velocity loads and the
    // FP64 arithmetic of full cells, which the compiler otherwise if-converts
    // so that every cell executes them (measured: 9 FP64 operations per cell
    // and 279 us per y/z sweep at 256^3, against 101 us).
    vof1[q] = 0.0;
    vof2[q] = 0.0;
    vof3[q] = 0.0;
    return;
  }
  const long sd = D == 1 ? 1 : (D == 2 ? (long)d.sy() : (long)d.sz());
  const double a1 = us[q] * tauh;
  const double a2 = us[q + sd] * tauh;
  vof1[q] = dmax1(-a1, 0.0);
  vof2[q] = 1.0 - dmax1(a1, 0.0) + dmin1(a2, 0.0);
  vof3[q] = dmax1(a2, 0.0);
}

// Sweep fluxes, pass 2: the listed interface cells, one per thread.
template <int D>
__global__ void k_swp_flux_iface(const unsigned *__restrict__ list, const unsigned *__restrict__ count,
                                 const double *__restrict__ us, const double *__restrict__ cc,
                                 double *__restrict__ vof1, double *__restrict__ vof2, double *__restrict__ vof3,
                                 Dims d, double tauh) {
  const unsigned n = *count;
  for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
    iface_flux<D>(list[t], us, cc, vof1, vof2, vof3, d, tauh);
}

// bc_flux: zero the ghost fluxes entering the domain along D.
template <int D>
__global__ void k_bc_flux(double *__restrict__ vof1, double *__restrict__ vof3, Dims d) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int q = blockIdx.y * blockDim.y + threadIdx.y + 2;
  if (D == 1) {
    if (p > d.ny - 1 || q > d.nz - 1) return;
    vof3[d.ix(1, p, q)] = 0.0;
    vof1[d.ix(d.nx, p, q)] = 0.0;
  } else if (D == 2) {
    if (p > d.nx - 1 || q > d.nz - 1) return;
    vof3[d.ix(p, 1, q)] = 0.0;
    vof1[d.ix(p, d.ny, q)] = 0.0;
  } else {
    if (p > d.nx - 1 || q > d.ny - 1) return;
    vof3[d.ix(p, q, 1)] = 0.0;
    vof1[d.ix(p, q, d.nz)] = 0.0;
  }
}

template <int D>
__global__ void k_swp_update(double *__restrict__ cc, const double *__restrict__ vof1,
                             const double *__restrict__ vof2, const double *__restrict__ vof3, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  const size_t sd = D == 1 ? 1 : (D == 2 ? d.sy() : d.sz());
  const double x = vof3[q - sd] + vof2[q] + vof1[q + sd];
  // dmax1(0, dmin1(1, x)) on the bit patterns (same result for every non-NaN x)
  const double y = __double_as_longlong(x) >= 0x3FF0000000000000LL ? 1.0 : x;
  cc[q] = __double_as_longlong(y) <= 0LL ? 0.0 : y;
}

// bc_c, three ordered steps (main.f:4340-4395 without the dead filter block).
__global__ void k_bc_c_x(double *__restrict__ cc, Dims d) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int k = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (j > d.ny || k > d.nz) return;
  cc[d.ix(2, j, k)] = cc[d.ix(1, j, k)];
  cc[d.ix(d.nx, j, k)] = cc[d.ix(d.nx - 1, j, k)];
}

__global__ void k_bc_c_y(double *__restrict__ cc, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int k = blockIdx.y * blockDim.y + threadIdx.y + 2;
  if (i > d.nx - 1 || k > d.nz - 1) return;
  double x = cc[d.ix(i, 2, k)];
  if (x > 1.0) x = 1.0;
  if (x < 0.0) x = 0.0;
  cc[d.ix(i, 1, k)] = x;
  cc[d.ix(i, d.ny, k)] = cc[d.ix(i, d.ny - 1, k)];
}

__global__ void k_bc_c_z(double *__restrict__ cc, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.nx - 1 || j > d.ny) return;
  cc[d.ix(i, j, 1)] = cc[d.ix(i, j, 2)];
  cc[d.ix(i, j, d.nz)] = cc[d.ix(i, j, d.nz - 1)];
}

// calcrho (main.f:2177-2190); for c = 0 and c = 1 the same operations are
// evaluated once on the host (rho_l = rho2 + 1*(rho1-rho2), ...).
__global__ void k_calcrho(double *__restrict__ rhon, double *__restrict__ mun, const double *__restrict__ cc,
                          size_t n, double rho1, double rho2, double mu1, double mu2, double rho_g, double rho_l,
                          double mu_g, double mu_l) {
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const double c = cc[q];
    if (is_zero_bits(c)) {
      rhon[q] = rho_g;
      mun[q] = mu_g;
    } else if (is_one_bits(c)) {
      rhon[q] = rho_l;
      mun[q] = mu_l;
    } else {
      rhon[q] = rho2 + c * (rho1 - rho2);
      mun[q] = mu2 + c * (mu1 - mu2);
    }
  }
}

const dim3 kBlk(32, 4, 1);

template <int D>
void sweep(const double *us, double *cc, double *v1, double *v2, double *v3, Dims d, double tauh, unsigned *list,
           unsigned *count, cudaStream_t st) {
  cudaMemsetAsync(count, 0, sizeof(unsigned), st);
  DSG_COUNT k_swp_flux<D><<<interior_grid(d, kBlk), kBlk, 0, st>>>(us, cc, v1, v2, v3, d, tauh, list, count);
  DSG_COUNT k_swp_flux_iface<D><<<kRedBlocks, 128, 0, st>>>(list, count, us, cc, v1, v2, v3, d, tauh);
  const dim3 b2(32, 8);
  int p = D == 1 ? d.ny : d.nx, q = D == 3 ? d.ny : d.nz;
  DSG_COUNT k_bc_flux<D><<<dim3((p + 31) / 32, (q + 7) / 8), b2, 0, st>>>(v1, v3, d);
  DSG_COUNT k_swp_update<D><<<interior_grid(d, kBlk), kBlk, 0, st>>>(cc, v1, v2, v3, d);
}

}  // namespace

cudaError_t bc_c(double *cc, Dims d, cudaStream_t st) {
  const dim3 b2(32, 8);
  DSG_COUNT k_bc_c_x<<<dim3((d.ny + 31) / 32, (d.nz + 7) / 8), b2, 0, st>>>(cc, d);
  DSG_COUNT k_bc_c_y<<<dim3((d.nx + 31) / 32, (d.nz + 7) / 8), b2, 0, st>>>(cc, d);
  DSG_COUNT k_bc_c_z<<<dim3((d.nx + 31) / 32, (d.ny + 7) / 8), b2, 0, st>>>(cc, d);
  return cudaGetLastError();
}

cudaError_t swp(const double *us, double *cc, double *vof1, double *vof2, double *vof3, int dir, Dims d,
                double tauh, unsigned *list, unsigned *count, cudaStream_t st) {
  if (dir == 1) sweep<1>(us, cc, vof1, vof2, vof3, d, tauh, list, count, st);
  else if (dir == 2) sweep<2>(us, cc, vof1, vof2, vof3, d, tauh, list, count, st);
  else sweep<3>(us, cc, vof1, vof2, vof3, d, tauh, list, count, st);
  return bc_c(cc, d, st);
}

cudaError_t calcrho(double *rhon, double *mun, const double *cc, Dims d, double rho1, double rho2,
                    double mu1, double mu2, cudaStream_t st) {
  const size_t n = d.count();
  const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
  const double z = 0.0, one = 1.0;
  const double rho_g = rho2 + z * (rho1 - rho2), rho_l = rho2 + one * (rho1 - rho2);
  const double mu_g = mu2 + z * (mu1 - mu2), mu_l = mu2 + one * (mu1 - mu2);
  DSG_COUNT k_calcrho<<<blocks, 256, 0, st>>>(rhon, mun, cc, n, rho1, rho2, mu1, mu2, rho_g, rho_l, mu_g, mu_l);
  return cudaGetLastError();
}

}  // namespace dsg
