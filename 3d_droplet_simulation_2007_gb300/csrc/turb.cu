// turb.cu -- k-epsilon turbulence (iturb = 3): kepsmodel (main.f:1888-2025),
// the turbulent diffusion of the volume fraction fturbdif (main.f:1239-1267)
// and the initial ktur/eps/mut of the drop.  FP64, built without FP
// contraction, same operation order as the reference: results are bit-equal
// to the oracle's.
#include "dsg_internal.cuh"

namespace dsg {
namespace {

// Initial state (the reference never sets ktur/eps for the drop; this follows
// inijet's jet formulas, main.f:536-549, with the phase speeds as vector
// magnitudes and the phases mixed by the volume fraction).  Every cell.
__global__ void k_keps_seed(double *__restrict__ ktur, double *__restrict__ eps, double *__restrict__ mut,
                            const double *__restrict__ cc, const double *__restrict__ rhon,
                            const double *__restrict__ mun, size_t n, double k1, double k2) {
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const double kt = cc[q] * k1 + (1.0 - cc[q]) * k2;
    ktur[q] = kt;
    const double e = kt > 0.0 ? (double)0.09f * rhon[q] * kt * kt / mun[q] : 0.0;
    eps[q] = e;
    mut[q] = kt > 0.0 ? (double)0.09f * rhon[q] * kt * kt / e : 0.0;
  }
}

// Upwind convective flux balance of a cell-centred scalar f (kepsmodel's conv).
__device__ __forceinline__ double upwind(const double *__restrict__ f, const double *__restrict__ u,
                                         const double *__restrict__ v, const double *__restrict__ w, size_t q,
                                         size_t sy, size_t sz, double h) {
  return (dmax1(u[q + 1], 0.0) * f[q] + dmin1(u[q + 1], 0.0) * f[q + 1] - dmax1(u[q], 0.0) * f[q - 1] -
          dmin1(u[q], 0.0) * f[q] + dmax1(v[q + sy], 0.0) * f[q] + dmin1(v[q + sy], 0.0) * f[q + sy] -
          dmax1(v[q], 0.0) * f[q - sy] - dmin1(v[q], 0.0) * f[q] + dmax1(w[q + sz], 0.0) * f[q] +
          dmin1(w[q + sz], 0.0) * f[q + sz] - dmax1(w[q], 0.0) * f[q - sz] - dmin1(w[q], 0.0) * f[q]) /
         h;
}

// Variable-coefficient diffusion of f with the turbulent Prandtl number sig.
__device__ __forceinline__ double diffusion(const double *__restrict__ f, const double *__restrict__ mun,
                                            const double *__restrict__ mut, const double *__restrict__ rhon,
                                            size_t q, size_t sy, size_t sz, double sig, double h22) {
  const double cip = mun[q + 1] + mun[q] + (mut[q] + mut[q + 1]) / sig;
  const double cim = mun[q - 1] + mun[q] + (mut[q] + mut[q - 1]) / sig;
  const double cjp = mun[q + sy] + mun[q] + (mut[q] + mut[q + sy]) / sig;
  const double cjm = mun[q - sy] + mun[q] + (mut[q] + mut[q - sy]) / sig;
  const double ckp = mun[q + sz] + mun[q] + (mut[q] + mut[q + sz]) / sig;
  const double ckm = mun[q - sz] + mun[q] + (mut[q] + mut[q - sz]) / sig;
  return 1.0 / (rhon[q] * h22) *
         (cip * (f[q + 1] - f[q]) - cim * (f[q] - f[q - 1]) + cjp * (f[q + sy] - f[q]) - cjm * (f[q] - f[q - sy]) +
          ckp * (f[q + sz] - f[q]) - ckm * (f[q] - f[q - sz]));
}

// kepsmodel's first loop: new ktur and eps of every interior cell from the
// old ones (into the scratch arrays kn, en).
__global__ void k_keps(double *__restrict__ kn, double *__restrict__ en, const double *__restrict__ ktur,
                       const double *__restrict__ eps, const double *__restrict__ mut,
                       const double *__restrict__ mun, const double *__restrict__ rhon,
                       const double *__restrict__ u, const double *__restrict__ v, const double *__restrict__ w,
                       Dims d, double h, double tau) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const double sigk = 1.0, sige = 1.3, c1 = 1.44, c2 = 1.92;
  const double h2 = h * h, h22 = h2 * 2.0;
  const size_t q = d.ix(i, j, k), sy = d.sy(), sz = d.sz();
  const double *K = ktur, *E = eps;
  double conv = upwind(K, u, v, w, q, sy, sz, h);
  double diff = diffusion(K, mun, mut, rhon, q, sy, sz, sigk, h22);
  const double dudx = u[q + 1] - u[q];
  const double dudy =
      0.25 * (u[q] - u[q - sy] + u[q + 1] - u[q + 1 - sy] + u[q + sy] - u[q] + u[q + 1 + sy] - u[q + 1]);
  const double dudz =
      0.25 * (u[q] - u[q - sz] + u[q + 1] - u[q + 1 - sz] + u[q + sz] - u[q] + u[q + 1 + sz] - u[q + 1]);
  const double dvdx =
      0.25 * (v[q] - v[q - 1] + v[q + 1] - v[q] + v[q + sy] - v[q - 1 + sy] + v[q + 1 + sy] - v[q + sy]);
  const double dvdy = v[q + sy] - v[q];
  const double dvdz =
      0.25 * (v[q] - v[q - sz] + v[q + sz] - v[q] + v[q + sy] - v[q + sy - sz] + v[q + sy + sz] - v[q + sy]);
  const double dwdx =
      0.25 * (w[q] - w[q - 1] + w[q + 1] - w[q] + w[q + sz] - w[q - 1 + sz] + w[q + 1 + sz] - w[q + sz]);
  const double dwdy =
      0.25 * (w[q] - w[q - sy] + w[q + sz] - w[q - sy + sz] + w[q + sy] - w[q] + w[q + sy + sz] - w[q + sz]);
  const double dwdz = w[q + sz] - w[q];
  double prod = mut[q] / rhon[q] / h2 *
                (2.0 * (dudx * dudx + dvdy * dvdy + dwdz * dwdz + dvdx * dudy + dwdx * dudz + dvdz * dwdy) +
                 dudy * dudy + dudz * dudz + dvdx * dvdx + dvdz * dvdz + dwdx * dwdx + dwdy * dwdy);
  kn[q] = K[q] + tau * (-conv + diff + prod - E[q]);
  conv = upwind(E, u, v, w, q, sy, sz, h);
  diff = diffusion(E, mun, mut, rhon, q, sy, sz, sige, h22);
  prod = prod * c1 * E[q] / K[q];
  en[q] = E[q] + tau * (-conv + diff + prod - c2 * E[q] * E[q] / K[q]);
}

// kepsmodel's second loop: commit the new values, mut = cmu rho k^2 / eps.
__global__ void k_keps_commit(double *__restrict__ ktur, double *__restrict__ eps, double *__restrict__ mut,
                              const double *__restrict__ kn, const double *__restrict__ en,
                              const double *__restrict__ rhon, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const double cmu = 0.09;
  const size_t q = d.ix(i, j, k);
  const double kt = kn[q], e = en[q];
  ktur[q] = kt;
  eps[q] = e;
  mut[q] = cmu * rhon[q] * kt * kt / e;
}

// fturbdif: in-place y/z diffusion of cc.  The reference loops i, j, k with k
// innermost, so cell (i,j,k) sees the new values of (i,j-1,k) and (i,j,k-1)
// and the old ones of (i,j+1,k) and (i,j,k+1).  Planes of constant i are
// independent (no x terms); within a plane the cells of one anti-diagonal
// j + k = s depend only on the previous anti-diagonal.  One block per plane
// walks the anti-diagonals in order with a block barrier between them, which
// reproduces the sequential order exactly.
__global__ void k_fturbdif(double *__restrict__ cc, const double *__restrict__ mut,
                           const double *__restrict__ rh, Dims d, double ftr) {
  const int i = blockIdx.x + 2;
  const size_t sy = d.sy(), sz = d.sz();
  for (int s = 4; s <= (d.ny - 1) + (d.nz - 1); s++) {
    const int jlo = s - (d.nz - 1) > 2 ? s - (d.nz - 1) : 2;
    const int jhi = s - 2 < d.ny - 1 ? s - 2 : d.ny - 1;
    for (int j = jlo + (int)threadIdx.x; j <= jhi; j += blockDim.x) {
      const int k = s - j;
      const size_t q = d.ix(i, j, k);
      const double m0 = mut[q] / rh[q];
      cc[q] = cc[q] + ftr * ((m0 + mut[q + sy] / rh[q + sy]) * (cc[q + sy] - cc[q]) -
                             (m0 + mut[q - sy] / rh[q - sy]) * (cc[q] - cc[q - sy]) +
                             (m0 + mut[q + sz] / rh[q + sz]) * (cc[q + sz] - cc[q]) -
                             (m0 + mut[q - sz] / rh[q - sz]) * (cc[q] - cc[q - sz]));
    }
    __syncthreads();
  }
}

const dim3 kBlk(32, 4, 1);

}  // namespace

cudaError_t keps_seed(double *ktur, double *eps, double *mut, const double *cc, const double *rhon,
                      const double *mun, Dims d, double k1, double k2, cudaStream_t st) {
  const size_t n = d.count();
  const int blocks = (int)((n + 255) / 256 < 8192 ? (n + 255) / 256 : 8192);
  DSG_COUNT k_keps_seed<<<blocks, 256, 0, st>>>(ktur, eps, mut, cc, rhon, mun, n, k1, k2);
  return cudaGetLastError();
}

cudaError_t kepsmodel(double *ktur, double *eps, double *mut, double *kn, double *en, const double *mun,
                      const double *rhon, const double *u, const double *v, const double *w, Dims d, double h,
                      double tau, cudaStream_t st) {
  DSG_COUNT k_keps<<<interior_grid(d, kBlk), kBlk, 0, st>>>(kn, en, ktur, eps, mut, mun, rhon, u, v, w, d, h, tau);
  DSG_COUNT k_keps_commit<<<interior_grid(d, kBlk), kBlk, 0, st>>>(ktur, eps, mut, kn, en, rhon, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = bc_scalar(ktur, d, st);
  if (e == cudaSuccess) e = bc_scalar(eps, d, st);
  if (e == cudaSuccess) e = bc_scalar(mut, d, st);
  return e;
}

cudaError_t fturbdif(double *cc, const double *mut, const double *rhon, Dims d, int tauh2, cudaStream_t st) {
  const double ftr = 1.0 * (double)tauh2 * 1.0 / 2.0;
  DSG_COUNT k_fturbdif<<<d.nx - 2, 256, 0, st>>>(cc, mut, rhon, d, ftr);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = bc_c(cc, d, st);
  return e;
}

}  // namespace dsg
