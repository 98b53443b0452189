// momentum.cu -- the step glue of solvelpres (main.f:3236-3439): viscous stress
// update, explicit predictor with gravity, bc_w (main.f:4143-4220), central
// convection (convective, main.f:3525-3566), bc_v (main.f:4064-4141), the
// divergence right-hand side and the pressure projection.
//
// Laminar runs: mut, turbst and the u2p/uvp... arrays of the reference are zero,
// so the terms they feed add exact zeros and are left out.
#include <cmath>

#include "dsg_internal.cuh"

namespace dsg {
namespace {

// Viscosity factors of the stress update: the cell's r2 + r1 c and the edges'
// r20 + r10 (sum of the four cells around the edge).  Where the seven volume
// fractions a cell reads are all exactly 0 or all exactly 1 (tested on the
// integer pipe), the factors are the precomputed values of the same fused
// multiply-adds (pure[0] for 0, pure[1] for 1: cell, edge), which skips 13 of
// the 31 FP64 operations of a cell on GB300's narrow FP64 pipe with the same
// bits.  The branch is taken per warp.
struct StressPure {
  double cell[2], edge[2];
};

__global__ void k_stress(double *__restrict__ S11, double *__restrict__ S22, double *__restrict__ S33,
                         double *__restrict__ S12, double *__restrict__ S13, double *__restrict__ S23,
                         const double *__restrict__ u, const double *__restrict__ v,
                         const double *__restrict__ w, const double *__restrict__ cc, Dims d, double r1,
                         double r2, double r10, double r20, StressPure pure, int k0) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + k0;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  const size_t sy = d.sy(), sz = d.sz();
  const double c0 = cc[q], c1 = cc[q - 1], c2 = cc[q - sy], c3 = cc[q - 1 - sy], c4 = cc[q - sz],
               c5 = cc[q - 1 - sz], c6 = cc[q - sy - sz];
  const bool one = is_one_bits(c0);
  const bool uniform = (one || is_zero_bits(c0)) && same_bits(c1, c0) && same_bits(c2, c0) && same_bits(c3, c0) &&
                       same_bits(c4, c0) && same_bits(c5, c0) && same_bits(c6, c0);
  double tc, t12, t13, t23;
  if (__all_sync(__activemask(), uniform)) {
    tc = one ? pure.cell[1] : pure.cell[0];
    t12 = t13 = t23 = one ? pure.edge[1] : pure.edge[0];
  } else {
    tc = fma(r1, c0, r2);
    t12 = fma(r10, c0 + c1 + c2 + c3, r20);
    t13 = fma(r10, c0 + c1 + c4 + c5, r20);
    t23 = fma(r10, c0 + c2 + c4 + c6, r20);
  }
  S11[q] = -S11[q] + tc * (u[q + 1] - u[q]);
  S22[q] = -S22[q] + tc * (v[q + sy] - v[q]);
  S33[q] = -S33[q] + tc * (w[q + sz] - w[q]);
  S12[q] = -S12[q] + t12 * (u[q] - u[q - sy] + v[q] - v[q - 1]);
  S13[q] = -S13[q] + t13 * (u[q] - u[q - sz] + w[q] - w[q - 1]);
  S23[q] = -S23[q] + t23 * (v[q] - v[q - sz] + w[q] - w[q - sy]);
}

__global__ void k_predictor(double *__restrict__ w1, double *__restrict__ w2, double *__restrict__ w3,
                            const double *__restrict__ u, const double *__restrict__ v,
                            const double *__restrict__ w, const double *__restrict__ a,
                            const double *__restrict__ b, const double *__restrict__ c,
                            const double *__restrict__ S11, const double *__restrict__ S22,
                            const double *__restrict__ S33, const double *__restrict__ S12,
                            const double *__restrict__ S13, const double *__restrict__ S23, Dims d,
                            double horgrav, double stdgrav, int k0) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + k0;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  const size_t sy = d.sy(), sz = d.sz();
  w1[q] = u[q] + a[q - 1] * (S11[q] - S11[q - 1] + S12[q + sy] - S12[q] + S13[q + sz] - S13[q]) + horgrav;
  w2[q] = v[q] + b[q - sy] * (S12[q + 1] - S12[q] + S22[q] - S22[q - sy] + S23[q + sz] - S23[q]) + stdgrav;
  w3[q] = w[q] + c[q - sz] * (S13[q + 1] - S13[q] + S23[q + sy] - S23[q] + S33[q] - S33[q - sz]);
}

// tauq = 0.25*tauh: the reference's tauh*(0.25*x) equals tauq*x bit for bit
// (scaling by 0.25 is exact, so both round the same product once), one FP64
// multiply per component less on GB300's narrow FP64 pipe.
__global__ void k_convective(double *__restrict__ u, double *__restrict__ v, double *__restrict__ w,
                             const double *__restrict__ w1, const double *__restrict__ w2,
                             const double *__restrict__ w3, Dims d, double tauq) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  const long sy = (long)d.sy(), sz = (long)d.sz();
#define W1(di, dj, dk) w1[(long)q + (long)(di) + (long)(dj) * sy + (long)(dk) * sz]
#define W2(di, dj, dk) w2[(long)q + (long)(di) + (long)(dj) * sy + (long)(dk) * sz]
#define W3(di, dj, dk) w3[(long)q + (long)(di) + (long)(dj) * sy + (long)(dk) * sz]
  double p, m, x;
  p = W1(0, 0, 0) + W1(-1, 0, 0);
  m = W1(1, 0, 0) + W1(0, 0, 0);
  x = p * p - m * m + (W1(0, -1, 0) + W1(0, 0, 0)) * (W2(0, 0, 0) + W2(-1, 0, 0)) -
      (W1(0, 1, 0) + W1(0, 0, 0)) * (W2(0, 1, 0) + W2(-1, 1, 0)) +
      (W1(0, 0, -1) + W1(0, 0, 0)) * (W3(0, 0, 0) + W3(-1, 0, 0)) -
      (W1(0, 0, 1) + W1(0, 0, 0)) * (W3(0, 0, 1) + W3(-1, 0, 1));
  u[q] = W1(0, 0, 0) + tauq * x;
  p = W2(0, 0, 0) + W2(0, -1, 0);
  m = W2(0, 1, 0) + W2(0, 0, 0);
  x = p * p - m * m + (W2(-1, 0, 0) + W2(0, 0, 0)) * (W1(0, 0, 0) + W1(0, -1, 0)) -
      (W2(1, 0, 0) + W2(0, 0, 0)) * (W1(1, 0, 0) + W1(1, -1, 0)) +
      (W2(0, 0, -1) + W2(0, 0, 0)) * (W3(0, 0, 0) + W3(0, -1, 0)) -
      (W2(0, 0, 1) + W2(0, 0, 0)) * (W3(0, 0, 1) + W3(0, -1, 1));
  v[q] = W2(0, 0, 0) + tauq * x;
  p = W3(0, 0, 0) + W3(0, 0, -1);
  m = W3(0, 0, 1) + W3(0, 0, 0);
  x = p * p - m * m + (W3(-1, 0, 0) + W3(0, 0, 0)) * (W1(0, 0, 0) + W1(0, 0, -1)) -
      (W3(1, 0, 0) + W3(0, 0, 0)) * (W1(1, 0, 0) + W1(1, 0, -1)) +
      (W3(0, -1, 0) + W3(0, 0, 0)) * (W2(0, 0, 0) + W2(0, 0, -1)) -
      (W3(0, 1, 0) + W3(0, 0, 0)) * (W2(0, 1, 0) + W2(0, 1, -1));
  w[q] = W3(0, 0, 0) + tauq * x;
#undef W1
#undef W2
#undef W3
}

__global__ void k_copy3_interior(double *__restrict__ u, double *__restrict__ v, double *__restrict__ w,
                                 const double *__restrict__ w1, const double *__restrict__ w2,
                                 const double *__restrict__ w3, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  u[q] = w1[q];
  v[q] = w2[q];
  w[q] = w3[q];
}

__global__ void k_div(double *__restrict__ out, const double *__restrict__ u, const double *__restrict__ v,
                      const double *__restrict__ w, Dims d, double hi2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  out[q] = (u[q + 1] - u[q] + v[q + d.sy()] - v[q] + w[q + d.sz()] - w[q]) * hi2;
}

__global__ void k_project(double *__restrict__ u, double *__restrict__ v, double *__restrict__ w,
                          const double *__restrict__ p, const double *__restrict__ a,
                          const double *__restrict__ b, const double *__restrict__ c, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  const size_t sy = d.sy(), sz = d.sz();
  const double pq = p[q];
  u[q] = u[q] - (pq - p[q - 1]) * a[q - 1];
  v[q] = v[q] - (pq - p[q - sy]) * b[q - sy];
  w[q] = w[q] - (pq - p[q - sz]) * c[q - sz];
}

// ---- bc_v (main.f:4064-4141) ---------------------------------------------------
__global__ void k_bcv_1(double *__restrict__ u, double *__restrict__ v, double *__restrict__ w, Dims d,
                        double xvel2) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int k = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (j > d.ny || k > d.nz) return;
  const int jj = j == 1 ? 2 : j;
  const double x = (jj * 1.0 - 1.5) / (d.ny * 1.0 - 1.5) - 1.0;
  const double val = xvel2 * (-(x * x) + 1.0);
  u[d.ix(1, j, k)] = j == 1 ? -val : val;
  v[d.ix(d.nx, j, k)] = v[d.ix(d.nx - 1, j, k)];
  w[d.ix(d.nx, j, k)] = w[d.ix(d.nx - 1, j, k)];
}

__global__ void k_bcv_2(double *__restrict__ u, double *__restrict__ v, double *__restrict__ w, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int k = blockIdx.y * blockDim.y + threadIdx.y + 2;
  if (i > d.nx - 1 || k > d.nz - 1) return;
  u[d.ix(i, 1, k)] = -u[d.ix(i, 2, k)];
  u[d.ix(i, d.ny, k)] = u[d.ix(i, d.ny - 1, k)];
  v[d.ix(i, 2, k)] = 0.0;
  v[d.ix(i, 1, k)] = 0.0;
  v[d.ix(i, d.ny, k)] = 0.0;
  w[d.ix(i, 1, k)] = -w[d.ix(i, 2, k)];
  w[d.ix(i, d.ny, k)] = w[d.ix(i, d.ny - 1, k)];
}

__global__ void k_bcv_3(double *__restrict__ u, double *__restrict__ v, double *__restrict__ w, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.nx - 1 || j > d.ny) return;
  u[d.ix(i, j, 1)] = u[d.ix(i, j, 2)];
  u[d.ix(i, j, d.nz)] = u[d.ix(i, j, d.nz - 1)];
  v[d.ix(i, j, 1)] = v[d.ix(i, j, 2)];
  v[d.ix(i, j, d.nz)] = v[d.ix(i, j, d.nz - 1)];
  w[d.ix(i, j, 2)] = 0.0;
  w[d.ix(i, j, d.nz)] = 0.0;
}

// x2(2,j,k) = x1(1,j,k) over interior j,k (bc_v/bc_w step 4 copies).
__global__ void k_copy_inflow(double *__restrict__ dst, const double *__restrict__ src, int dst_i, Dims d) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int k = blockIdx.y * blockDim.y + threadIdx.y + 2;
  if (j > d.ny - 1 || k > d.nz - 1) return;
  dst[d.ix(dst_i, j, k)] = src[d.ix(1, j, k)];
}

// Sums of f0(1,j,k) and f1(nx-1,j,k) over interior j,k (deterministic order).
__global__ void k_outlet_partial(double *__restrict__ partials, const double *__restrict__ f0,
                                 const double *__restrict__ f1, Dims d) {
  const size_t n = (size_t)(d.ny - 2) * (d.nz - 2);
  double s0 = 0.0, s1 = 0.0;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(t % (size_t)(d.ny - 2)) + 2, k = (int)(t / (size_t)(d.ny - 2)) + 2;
    s0 += f0[d.ix(1, j, k)];
    s1 += f1[d.ix(d.nx - 1, j, k)];
  }
  __shared__ double sh0[256], sh1[256];
  sh0[threadIdx.x] = s0;
  sh1[threadIdx.x] = s1;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sh0[threadIdx.x] += sh0[threadIdx.x + s];
      sh1[threadIdx.x] += sh1[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = sh0[0];
    partials[2 * blockIdx.x + 1] = sh1[0];
  }
}

constexpr int kOutletBlocks = 64;

__global__ void k_outlet_apply(double *__restrict__ x, const double *__restrict__ partials, Dims d) {
  __shared__ double vout, vout2;
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    double s0 = 0.0, s1 = 0.0;
    for (int b = 0; b < kOutletBlocks; b++) {
      s0 += partials[2 * b];
      s1 += partials[2 * b + 1];
    }
    vout = s0 / (d.ny - 2) / (d.nz - 2);
    vout2 = s1 / (d.ny - 2) / (d.nz - 2);
  }
  __syncthreads();
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int k = blockIdx.y * blockDim.y + threadIdx.y + 2;
  if (j > d.ny - 1 || k > d.nz - 1) return;
  x[d.ix(d.nx, j, k)] = x[d.ix(d.nx - 1, j, k)] + vout - vout2;
}

// ---- bc_w (main.f:4143-4220) ---------------------------------------------------
__global__ void k_bcw_1(double *__restrict__ w2, double *__restrict__ w3, const double *__restrict__ v,
                        const double *__restrict__ w, Dims d) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int k = blockIdx.y * blockDim.y + threadIdx.y + 2;
  if (j > d.ny - 1 || k > d.nz - 1) return;
  const double v1 = v[d.ix(1, j, k)], wv1 = w[d.ix(1, j, k)];
  w2[d.ix(1, j, k)] = v1;
  w2[d.ix(2, j, k)] = v1;
  w2[d.ix(d.nx, j, k)] = v[d.ix(d.nx, j, k)];
  w3[d.ix(1, j, k)] = wv1;
  w3[d.ix(2, j, k)] = wv1;
  w3[d.ix(d.nx, j, k)] = w[d.ix(d.nx, j, k)];
}

__global__ void k_bcw_2(double *__restrict__ w1, double *__restrict__ w2, double *__restrict__ w3,
                        const double *__restrict__ v, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int k = blockIdx.y * blockDim.y + threadIdx.y + 2;
  if (i > d.nx - 1 || k > d.nz - 1) return;
  w1[d.ix(i, 1, k)] = -w1[d.ix(i, 2, k)];
  w1[d.ix(i, d.ny, k)] = w1[d.ix(i, d.ny - 1, k)];
  w2[d.ix(i, 1, k)] = 0.0;
  w2[d.ix(i, 2, k)] = 0.0;
  w2[d.ix(i, d.ny, k)] = v[d.ix(i, d.ny, k)];
  w3[d.ix(i, 1, k)] = -w3[d.ix(i, 2, k)];
  w3[d.ix(i, d.ny, k)] = w3[d.ix(i, d.ny - 1, k)];
}

__global__ void k_bcw_3(double *__restrict__ w1, double *__restrict__ w2, double *__restrict__ w3,
                        const double *__restrict__ w, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.nx - 1 || j > d.ny) return;
  w1[d.ix(i, j, 1)] = w1[d.ix(i, j, 2)];
  w1[d.ix(i, j, d.nz)] = w1[d.ix(i, j, d.nz - 1)];
  w2[d.ix(i, j, 1)] = w2[d.ix(i, j, 2)];
  w2[d.ix(i, j, d.nz)] = w2[d.ix(i, j, d.nz - 1)];
  const double wb = w[d.ix(i, j, 1)];
  w3[d.ix(i, j, 1)] = wb;
  w3[d.ix(i, j, 2)] = wb;
  w3[d.ix(i, j, d.nz)] = w[d.ix(i, j, d.nz)];
}

const dim3 kBlk(32, 4, 1);
const dim3 kFace(32, 8, 1);

inline dim3 fgrid(int p, int q) { return dim3((unsigned)((p + 31) / 32), (unsigned)((q + 7) / 8)); }

// Outlet flux balance shared by bc_v and bc_w: x(nx,j,k) = x(nx-1,j,k) + vout - vout2
// with vout the mean of u(1,j,k) and vout2 the mean of x(nx-1,j,k).
void outlet(double *x, const double *u, double *partials, Dims d, cudaStream_t st) {
  DSG_COUNT k_outlet_partial<<<kOutletBlocks, 256, 0, st>>>(partials, u, x, d);
  DSG_COUNT k_outlet_apply<<<fgrid(d.ny, d.nz), kFace, 0, st>>>(x, partials, d);
}

}  // namespace

cudaError_t bc_v(double *u, double *v, double *w, double *partials, Dims d, double xvel2, cudaStream_t st) {
  DSG_COUNT k_bcv_1<<<fgrid(d.ny, d.nz), kFace, 0, st>>>(u, v, w, d, xvel2);
  DSG_COUNT k_bcv_2<<<fgrid(d.nx, d.nz), kFace, 0, st>>>(u, v, w, d);
  DSG_COUNT k_bcv_3<<<fgrid(d.nx, d.ny), kFace, 0, st>>>(u, v, w, d);
  DSG_COUNT k_copy_inflow<<<fgrid(d.ny, d.nz), kFace, 0, st>>>(u, u, 2, d);
  outlet(u, u, partials, d, st);
  return cudaGetLastError();
}

cudaError_t bc_w(double *w1, double *w2, double *w3, const double *u, const double *v, const double *w,
                 double *partials, Dims d, cudaStream_t st) {
  DSG_COUNT k_bcw_1<<<fgrid(d.ny, d.nz), kFace, 0, st>>>(w2, w3, v, w, d);
  DSG_COUNT k_bcw_2<<<fgrid(d.nx, d.nz), kFace, 0, st>>>(w1, w2, w3, v, d);
  DSG_COUNT k_bcw_3<<<fgrid(d.nx, d.ny), kFace, 0, st>>>(w1, w2, w3, w, d);
  DSG_COUNT k_copy_inflow<<<fgrid(d.ny, d.nz), kFace, 0, st>>>(w1, u, 1, d);
  DSG_COUNT k_copy_inflow<<<fgrid(d.ny, d.nz), kFace, 0, st>>>(w1, u, 2, d);
  outlet(w1, u, partials, d, st);
  return cudaGetLastError();
}

// Interior planes k0 .. k1-1 (k1 = 0: all interior planes, 2 .. nz-1).
inline dim3 plane_grid(const Dims &d, int k0, int k1) {
  const dim3 g = interior_grid(d, kBlk);
  return dim3(g.x, g.y, (unsigned)((k1 ? k1 : d.nz) - k0));
}

cudaError_t stress(double *const S[6], const double *u, const double *v, const double *w, const double *cc,
                   Dims d, double r1, double r2, double r10, double r20, cudaStream_t st, int k0, int k1) {
  if ((k1 ? k1 : d.nz) <= k0) return cudaSuccess;
  const StressPure pure{{std::fma(r1, 0.0, r2), std::fma(r1, 1.0, r2)},
                        {std::fma(r10, 0.0, r20), std::fma(r10, 4.0, r20)}};
  DSG_COUNT k_stress<<<plane_grid(d, k0, k1), kBlk, 0, st>>>(S[0], S[1], S[2], S[3], S[4], S[5], u, v, w, cc, d, r1,
                                                              r2, r10, r20, pure, k0);
  return cudaGetLastError();
}

cudaError_t predictor(double *w1, double *w2, double *w3, const double *u, const double *v, const double *w,
                      const double *a, const double *b, const double *c, double *const S[6], Dims d,
                      double horgrav, double stdgrav, cudaStream_t st, int k0, int k1) {
  if ((k1 ? k1 : d.nz) <= k0) return cudaSuccess;
  DSG_COUNT k_predictor<<<plane_grid(d, k0, k1), kBlk, 0, st>>>(w1, w2, w3, u, v, w, a, b, c, S[0], S[1], S[2],
                                                                 S[3], S[4], S[5], d, horgrav, stdgrav, k0);
  return cudaGetLastError();
}

cudaError_t convective(double *u, double *v, double *w, const double *w1, const double *w2, const double *w3,
                       Dims d, double tauh, int convectype, cudaStream_t st) {
  if (convectype == 2)
    DSG_COUNT k_convective<<<interior_grid(d, kBlk), kBlk, 0, st>>>(u, v, w, w1, w2, w3, d, 0.25 * tauh);
  else
    DSG_COUNT k_copy3_interior<<<interior_grid(d, kBlk), kBlk, 0, st>>>(u, v, w, w1, w2, w3, d);
  return cudaGetLastError();
}

cudaError_t divergence(double *out, const double *u, const double *v, const double *w, Dims d, double hi2,
                       cudaStream_t st) {
  DSG_COUNT k_div<<<interior_grid(d, kBlk), kBlk, 0, st>>>(out, u, v, w, d, hi2);
  return cudaGetLastError();
}

cudaError_t project(double *u, double *v, double *w, const double *p, const double *a, const double *b,
                    const double *c, Dims d, cudaStream_t st) {
  DSG_COUNT k_project<<<interior_grid(d, kBlk), kBlk, 0, st>>>(u, v, w, p, a, b, c, d);
  return cudaGetLastError();
}

}  // namespace dsg
