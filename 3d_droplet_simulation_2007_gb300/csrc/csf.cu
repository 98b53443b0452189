// csf.cu -- CSF surface-tension force (csf, main.f:2363-2481): 27-point filter
// of the volume fraction, face-normal curvature kappa = -div(n), and the face
// forces S11/S22/S33 = sigh * (c~_i - c~_{i-1}) * kappa_i, plus bc_tensor
// (main.f:4222-4296).
#include "dsg_internal.cuh"

namespace dsg {
namespace {

// Curvature at interior cells: six face-normal magnitudes with transverse
// 4-point means (+1e-50 inside the root), kappa = -(d1x-d2x+d1y-d2y+d1z-d2z).
__global__ void k_curvature(double *__restrict__ kap, const double *__restrict__ f, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  const long sy = (long)d.sy(), sz = (long)d.sz();
#define F(di, dj, dk) f[(long)q + (long)(di) + (long)(dj) * sy + (long)(dk) * sz]
  // Uniform 19-point neighbourhood (bulk liquid or gas): every difference is
  // +0, every d is 0/sqrt(1e-50) = +0 and kappa = -(+0) = -0 exactly.
  const double f0 = F(0, 0, 0);
#define EQ(di, dj, dk) same_bits(F(di, dj, dk), f0)
  if (EQ(1, 0, 0) && EQ(-1, 0, 0) && EQ(0, 1, 0) && EQ(0, -1, 0) && EQ(0, 0, 1) && EQ(0, 0, -1) && EQ(1, 1, 0) &&
      EQ(1, -1, 0) && EQ(-1, 1, 0) && EQ(-1, -1, 0) && EQ(1, 0, 1) && EQ(1, 0, -1) && EQ(-1, 0, 1) && EQ(-1, 0, -1) &&
      EQ(0, 1, 1) && EQ(0, 1, -1) && EQ(0, -1, 1) && EQ(0, -1, -1)) {
#undef EQ
    kap[q] = -0.0;
    return;
  }
  // d = difference / |normal| as difference * rsqrt(|normal|^2): one FP64
  // reciprocal square root in place of a square root and a division on
  // GB300's narrow FP64 pipe (results within a few ulps of the quotient)
  double t0, t1, t2;
  t0 = F(1, 0, 0) - F(0, 0, 0);
  t1 = F(0, 1, 0) - F(0, -1, 0) + F(1, 1, 0) - F(1, -1, 0);
  t2 = F(0, 0, 1) - F(0, 0, -1) + F(1, 0, 1) - F(1, 0, -1);
  const double d1x = t0 * rsqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
  t0 = F(0, 0, 0) - F(-1, 0, 0);
  t1 = F(0, 1, 0) - F(0, -1, 0) + F(-1, 1, 0) - F(-1, -1, 0);
  t2 = F(0, 0, 1) - F(0, 0, -1) + F(-1, 0, 1) - F(-1, 0, -1);
  const double d2x = t0 * rsqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
  t0 = F(0, 1, 0) - F(0, 0, 0);
  t1 = F(1, 0, 0) - F(-1, 0, 0) + F(1, 1, 0) - F(-1, 1, 0);
  t2 = F(0, 0, 1) - F(0, 0, -1) + F(0, 1, 1) - F(0, 1, -1);
  const double d1y = t0 * rsqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
  t0 = F(0, 0, 0) - F(0, -1, 0);
  t1 = F(1, 0, 0) - F(-1, 0, 0) + F(1, -1, 0) - F(-1, -1, 0);
  t2 = F(0, 0, 1) - F(0, 0, -1) + F(0, -1, 1) - F(0, -1, -1);
  const double d2y = t0 * rsqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
  t0 = F(0, 0, 1) - F(0, 0, 0);
  t1 = F(1, 0, 0) - F(-1, 0, 0) + F(1, 0, 1) - F(-1, 0, 1);
  t2 = F(0, 1, 0) - F(0, -1, 0) + F(0, 1, 1) - F(0, -1, 1);
  const double d1z = t0 * rsqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
  t0 = F(0, 0, 0) - F(0, 0, -1);
  t1 = F(1, 0, 0) - F(-1, 0, 0) + F(1, 0, -1) - F(-1, 0, -1);
  t2 = F(0, 1, 0) - F(0, -1, 0) + F(0, 1, -1) - F(0, -1, -1);
  const double d2z = t0 * rsqrt(t0 * t0 + 0.0625 * (t1 * t1) + 0.0625 * (t2 * t2) + 1.e-50);
#undef F
  kap[q] = -(d1x - d2x + d1y - d2y + d1z - d2z);
}

__global__ void k_csf_force(double *__restrict__ s11, double *__restrict__ s22, double *__restrict__ s33,
                            const double *__restrict__ f, const double *__restrict__ kap, Dims d,
                            double sigh) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  const double kq = kap[q], fq = f[q];
  const double fx = f[q - 1], fy = f[q - d.sy()], fz = f[q - d.sz()];
  if (same_bits(fx, fq) && same_bits(fy, fq) && same_bits(fz, fq)) {
    // bulk cell: every difference is +0, so each force is (sigh * +0) * kappa,
    // a zero whose sign is sign(sigh) xor sign(kappa) (kappa is finite),
    // formed on the integer pipe
    const double z = __longlong_as_double((__double_as_longlong(sigh) ^ __double_as_longlong(kq)) &
                                          (long long)0x8000000000000000ULL);
    s11[q] = z;
    s22[q] = z;
    s33[q] = z;
    return;
  }
  s11[q] = sigh * (fq - fx) * kq;
  s22[q] = sigh * (fq - fy) * kq;
  s33[q] = sigh * (fq - fz) * kq;
}

// bc_tensor, three ordered steps (every cell two steps write gets the same
// constant from both, so the steps also split into ranges of planes: the x
// and y faces of planes kx0 .. kx1-1, the z planes 1, 2 and nz where they
// lie in kz0 .. kz1-1).
__global__ void k_bct_x(double *__restrict__ s11, double *__restrict__ s12, double *__restrict__ s13, Dims d, int kx0,
                        int kx1) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int k = blockIdx.y * blockDim.y + threadIdx.y + kx0;
  if (j > d.ny - 1 || k >= kx1) return;
  s11[d.ix(1, j, k)] = 0.0;
  s12[d.ix(d.nx, j, k)] = 0.0;
  s13[d.ix(d.nx, j, k)] = 0.0;
}

__global__ void k_bct_y(double *__restrict__ s22, double *__restrict__ s12, double *__restrict__ s23, Dims d, int kx0,
                        int kx1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int k = blockIdx.y * blockDim.y + threadIdx.y + kx0;
  if (i > d.nx || k >= kx1) return;
  s22[d.ix(i, 1, k)] = s22[d.ix(i, 2, k)];
  s12[d.ix(i, d.ny, k)] = 0.0;
  s23[d.ix(i, d.ny, k)] = 0.0;
}

__global__ void k_bct_z(double *__restrict__ s33, double *__restrict__ s13, double *__restrict__ s23, Dims d, int kz0,
                        int kz1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.nx || j > d.ny) return;
  if (kz0 <= 1 && 1 < kz1) s33[d.ix(i, j, 1)] = 0.0;
  if (kz0 <= 2 && 2 < kz1) s13[d.ix(i, j, 2)] = 0.0;
  if (kz0 <= d.nz && d.nz < kz1) s13[d.ix(i, j, d.nz)] = 0.0;
  if (kz0 <= 2 && 2 < kz1) s23[d.ix(i, j, 2)] = 0.0;
  if (kz0 <= d.nz && d.nz < kz1) s23[d.ix(i, j, d.nz)] = 0.0;
}

// The off-diagonal part of bc_tensor alone: the constant faces of S12, S13,
// S23 that k_bct_x/y/z write (the same cells and values).
__global__ void k_bct_off_x(double *__restrict__ s12, double *__restrict__ s13, Dims d, int kx0, int kx1) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int k = blockIdx.y * blockDim.y + threadIdx.y + kx0;
  if (j > d.ny - 1 || k >= kx1) return;
  s12[d.ix(d.nx, j, k)] = 0.0;
  s13[d.ix(d.nx, j, k)] = 0.0;
}

__global__ void k_bct_off_y(double *__restrict__ s12, double *__restrict__ s23, Dims d, int kx0, int kx1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int k = blockIdx.y * blockDim.y + threadIdx.y + kx0;
  if (i > d.nx || k >= kx1) return;
  s12[d.ix(i, d.ny, k)] = 0.0;
  s23[d.ix(i, d.ny, k)] = 0.0;
}

__global__ void k_bct_off_z(double *__restrict__ s13, double *__restrict__ s23, Dims d, int kz0, int kz1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.nx || j > d.ny) return;
  if (kz0 <= 2 && 2 < kz1) s13[d.ix(i, j, 2)] = 0.0;
  if (kz0 <= d.nz && d.nz < kz1) s13[d.ix(i, j, d.nz)] = 0.0;
  if (kz0 <= 2 && 2 < kz1) s23[d.ix(i, j, 2)] = 0.0;
  if (kz0 <= d.nz && d.nz < kz1) s23[d.ix(i, j, d.nz)] = 0.0;
}

const dim3 kBlk(32, 4, 1);

}  // namespace

// x and y faces of the interior planes among k0 .. k1-1, and the z planes in
// that range (k0 = 1, k1 = nz + 1: everything).
cudaError_t bc_tensor_offdiag(double *s12, double *s13, double *s23, Dims d, cudaStream_t st, int k0, int k1) {
  const dim3 b2(32, 8);
  const int kx0 = k0 > 2 ? k0 : 2, kx1 = k1 < d.nz ? k1 : d.nz;
  if (kx1 > kx0) {
    DSG_COUNT k_bct_off_x<<<dim3((d.ny + 31) / 32, (kx1 - kx0 + 7) / 8), b2, 0, st>>>(s12, s13, d, kx0, kx1);
    DSG_COUNT k_bct_off_y<<<dim3((d.nx + 31) / 32, (kx1 - kx0 + 7) / 8), b2, 0, st>>>(s12, s23, d, kx0, kx1);
  }
  DSG_COUNT k_bct_off_z<<<dim3((d.nx + 31) / 32, (d.ny + 7) / 8), b2, 0, st>>>(s13, s23, d, k0, k1);
  return cudaGetLastError();
}

cudaError_t bc_tensor(double *const S[6], Dims d, cudaStream_t st, int k0, int k1) {
  // S = {S11, S22, S33, S12, S13, S23}
  const dim3 b2(32, 8);
  const int kx0 = k0 > 2 ? k0 : 2, kx1 = k1 < d.nz ? k1 : d.nz;
  if (kx1 > kx0) {
    DSG_COUNT k_bct_x<<<dim3((d.ny + 31) / 32, (kx1 - kx0 + 7) / 8), b2, 0, st>>>(S[0], S[3], S[4], d, kx0, kx1);
    DSG_COUNT k_bct_y<<<dim3((d.nx + 31) / 32, (kx1 - kx0 + 7) / 8), b2, 0, st>>>(S[1], S[3], S[5], d, kx0, kx1);
  }
  DSG_COUNT k_bct_z<<<dim3((d.nx + 31) / 32, (d.ny + 7) / 8), b2, 0, st>>>(S[2], S[4], S[5], d, k0, k1);
  return cudaGetLastError();
}


// csf with the reference's scratch aliasing: w11 = pressure array, w22 = fine
// residual array, w33 = fine rhs array; ccf is the routine's local array.
// scratch = false (inside a whole step, where the pressure phase overwrites
// all three before reading them): the filtered field goes straight to ccf
// and S11..S33 are not copied into w11..w33; w11 still holds the curvature.
cudaError_t csf(const double *ccc, double *w11, double *w22, double *w33, double *ccf, double *const S[6],
                Dims d, double tau, double sigma, double h, cudaStream_t st, bool scratch) {
  const size_t bytes = d.count() * sizeof(double);
  // copy(ccf,ccc); filterc27(ccf,w22); copy(ccf,w22): filtering ccf == filtering ccc
  cudaError_t e = filterc27(ccc, scratch ? w22 : ccf, d, st);
  if (e != cudaSuccess) return e;
  if (scratch) {
    e = cudaMemcpyAsync(ccf, w22, bytes, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return e;
  }
  e = bc_out(ccf, d, st);
  if (e != cudaSuccess) return e;
  if (sigma == 0.0) {
    for (int m = 0; m < 6; m++) {
      e = cudaMemsetAsync(S[m], 0, bytes, st);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  const double sigh = 0.5 * (tau * tau) * sigma / (h * h * h);
  DSG_COUNT k_curvature<<<interior_grid(d, kBlk), kBlk, 0, st>>>(w11, ccf, d);
  e = bc_out(w11, d, st);
  if (e != cudaSuccess) return e;
  DSG_COUNT k_csf_force<<<interior_grid(d, kBlk), kBlk, 0, st>>>(S[0], S[1], S[2], ccf, w11, d, sigh);
  if (scratch) {
    if ((e = cudaMemcpyAsync(w11, S[0], bytes, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(w22, S[1], bytes, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(w33, S[2], bytes, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
  }
  return bc_tensor(S, d, st);
}

}  // namespace dsg
