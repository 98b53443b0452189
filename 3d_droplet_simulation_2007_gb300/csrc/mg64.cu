// mg64.cu -- FP64 multigrid kernels of the variable-density pressure Poisson
// solve (main.f:3765-3997, 4298-4329, 4432-4494) and the deterministic
// reductions used by the solver.
//
// Ghost handling: bc_scalar's final ghost values are a closed-form function of
// the interior (x ghost 1 = cell 2, x ghost nx = 0, y/z ghosts = the adjacent
// interior cell, edges and corners by composition).  The colour passes of
// relax therefore read "virtual ghosts" (own value or 0) instead of memory,
// which equals running bc_scalar before each pass, and a single bc_scalar at
// the end of a block of relax calls leaves the array exactly as the reference.
// All arithmetic keeps the reference's operation order; this file is built
// without FMA contraction so results are bit-identical to a non-contracting
// Fortran build.
#include "dsg_internal.cuh"

namespace dsg {
namespace {

// ---- bc_scalar, one launch over the six faces (closed form) -----------------
__global__ void k_bc_scalar(double *__restrict__ s, Dims d) {
  const int face = blockIdx.z;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int q = blockIdx.y * blockDim.y + threadIdx.y;
  int i, j, k;
  if (face < 2) {  // x faces: p -> j, q -> k
    if (p >= d.ny || q >= d.nz) return;
    i = face == 0 ? 1 : d.nx; j = p + 1; k = q + 1;
  } else if (face < 4) {  // y faces: p -> i, q -> k
    if (p >= d.nx || q >= d.nz) return;
    i = p + 1; j = face == 2 ? 1 : d.ny; k = q + 1;
  } else {  // z faces: p -> i, q -> j
    if (p >= d.nx || q >= d.ny) return;
    i = p + 1; j = q + 1; k = face == 4 ? 1 : d.nz;
  }
  if (i == d.nx) { s[d.ix(i, j, k)] = 0.0; return; }
  const int ci = i == 1 ? 2 : i;
  const int cj = j == 1 ? 2 : (j == d.ny ? d.ny - 1 : j);
  const int ck = k == 1 ? 2 : (k == d.nz ? d.nz - 1 : k);
  s[d.ix(i, j, k)] = s[d.ix(ci, cj, ck)];
}

// bc_resid step 1 (main.f:4441-4446): x faces over all j,k, reading cell 2 / nx-1.
__global__ void k_bc_xcopy(double *__restrict__ s, Dims d) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int k = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (j > d.ny || k > d.nz) return;
  s[d.ix(1, j, k)] = s[d.ix(2, j, k)];
  s[d.ix(d.nx, j, k)] = s[d.ix(d.nx - 1, j, k)];
}

// bc_resid steps 2-3 (main.f:4450-4461): y and z ghosts of interior i set to 0.
__global__ void k_bc_resid_yz(double *__restrict__ s, Dims d) {
  const int face = blockIdx.z;  // 0: y (i, k in 2..nz-1), 1: z (i, all j)
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int q = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.nx - 1) return;
  if (face == 0) {
    if (q < 2 || q > d.nz - 1) return;
    s[d.ix(i, 1, q)] = 0.0;
    s[d.ix(i, d.ny, q)] = 0.0;
  } else {
    if (q > d.ny) return;
    s[d.ix(i, q, 1)] = 0.0;
    s[d.ix(i, q, d.nz)] = 0.0;
  }
}

// bc_out step 2 (main.f:4413-4418): y faces, all i, interior k.
__global__ void k_bc_out_y(double *__restrict__ s, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int k = blockIdx.y * blockDim.y + threadIdx.y + 2;
  if (i > d.nx || k > d.nz - 1) return;
  s[d.ix(i, 1, k)] = s[d.ix(i, 2, k)];
  s[d.ix(i, d.ny, k)] = s[d.ix(i, d.ny - 1, k)];
}

// bc_out step 3 (main.f:4422-4427): z faces, interior i, all j.
__global__ void k_bc_out_z(double *__restrict__ s, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i > d.nx - 1 || j > d.ny) return;
  s[d.ix(i, j, 1)] = s[d.ix(i, j, 2)];
  s[d.ix(i, j, d.nz)] = s[d.ix(i, j, d.nz - 1)];
}

// ---- relax: one colour pass (main.f:3973-3992) ----------------------------
// colour 0 updates i+j+k even (first pass), colour 1 odd.  Thread (t, j, k)
// updates i = i0 + 2t.  Ghost neighbours are virtual (see file header).
// FMA = false: the reference's operation order, no contraction (17 FP64
// operations per cell, bit-identical to the oracle).  FMA = true: the same
// sum as a fused multiply-add chain and the update written as
// u + omega*(temp - u) (10 FP64 operations); GB300's FP64 pipe, not HBM,
// bounds this kernel, so the operation count sets its speed.
template <bool FMA>
__global__ void k_relax_colour(double *__restrict__ u, const double *__restrict__ rhs,
                               const double *__restrict__ a, const double *__restrict__ b,
                               const double *__restrict__ c, const double *__restrict__ ei, Dims d,
                               double h2, double omega, int colour) {
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (j > d.ny - 1) return;
  const int i = 2 + ((j + k + colour) & 1) + 2 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i > d.nx - 1) return;
  const size_t q = d.ix(i, j, k);
  const size_t sy = d.sy(), sz = d.sz();
  const double uc = u[q];
  const double uxp = (i + 1 == d.nx) ? 0.0 : u[q + 1];
  const double uxm = (i - 1 == 1) ? uc : u[q - 1];
  const double uyp = (j + 1 == d.ny) ? uc : u[q + sy];
  const double uym = (j - 1 == 1) ? uc : u[q - sy];
  const double uzp = (k + 1 == d.nz) ? uc : u[q + sz];
  const double uzm = (k - 1 == 1) ? uc : u[q - sz];
  if (FMA) {
    double t = a[q] * uxp;
    t = __fma_rn(a[q - 1], uxm, t);
    t = __fma_rn(b[q], uyp, t);
    t = __fma_rn(b[q - sy], uym, t);
    t = __fma_rn(c[q], uzp, t);
    t = __fma_rn(c[q - sz], uzm, t);
    t = __fma_rn(-h2, rhs[q], t) * ei[q];
    u[q] = __fma_rn(omega, t - uc, uc);
    return;
  }
  const double temp = (a[q] * uxp + a[q - 1] * uxm + b[q] * uyp + b[q - sy] * uym + c[q] * uzp +
                       c[q - sz] * uzm - h2 * rhs[q]) *
                      ei[q];
  u[q] = omega * temp + (1.0 - omega) * uc;
}

// Residual of one interior cell, rhs - (1/h^2) sum a_nb (u_nb - u) (main.f:3912-3925),
// in the reference's order or as a fused multiply-add chain.
template <bool FMA>
__device__ __forceinline__ double cell_resid(const double *__restrict__ u, const double *__restrict__ rhs,
                                             const double *__restrict__ a, const double *__restrict__ b,
                                             const double *__restrict__ c, size_t q, size_t sy, size_t sz,
                                             double h2i) {
  const double uc = u[q];
  if (FMA) {
    double t = a[q] * (u[q + 1] - uc);
    t = __fma_rn(a[q - 1], u[q - 1] - uc, t);
    t = __fma_rn(b[q], u[q + sy] - uc, t);
    t = __fma_rn(b[q - sy], u[q - sy] - uc, t);
    t = __fma_rn(c[q], u[q + sz] - uc, t);
    t = __fma_rn(c[q - sz], u[q - sz] - uc, t);
    return __fma_rn(-h2i, t, rhs[q]);
  }
  return -h2i * (a[q] * (u[q + 1] - uc) + a[q - 1] * (u[q - 1] - uc) + b[q] * (u[q + sy] - uc) +
                 b[q - sy] * (u[q - sy] - uc) + c[q] * (u[q + sz] - uc) + c[q - sz] * (u[q - sz] - uc)) +
         rhs[q];
}

// ---- resid (main.f:3912-3925), reads the ghosts from memory ----------------
template <bool FMA>
__global__ void k_resid(double *__restrict__ res, const double *__restrict__ u,
                        const double *__restrict__ rhs, const double *__restrict__ a,
                        const double *__restrict__ b, const double *__restrict__ c, Dims d,
                        double h2i) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  res[q] = cell_resid<FMA>(u, rhs, a, b, c, q, d.sy(), d.sz(), h2i);
}

// ---- rstrct fused with the coarse bc_scalar (main.f:3765-3791) ------------
__global__ void k_rstrct(double *__restrict__ uc, const double *__restrict__ uf, Dims dc, Dims df) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > dc.nx || j > dc.ny) return;
  if (i == dc.nx && (j >= 2 && j <= dc.ny - 1 && k >= 2 && k <= dc.nz - 1)) {
    uc[dc.ix(i, j, k)] = 0.0;
    return;
  }
  if (i == dc.nx) { uc[dc.ix(i, j, k)] = 0.0; return; }
  const int ci = i == 1 ? 2 : i;
  const int cj = j == 1 ? 2 : (j == dc.ny ? dc.ny - 1 : j);
  const int ck = k == 1 ? 2 : (k == dc.nz ? dc.nz - 1 : k);
  const int fi = 2 * ci - 2, fj = 2 * cj - 2, fk = 2 * ck - 2;
  const size_t f = df.ix(fi, fj, fk);
  const size_t sy = df.sy(), sz = df.sz();
  uc[dc.ix(i, j, k)] = 0.125 * (uf[f] + uf[f + 1] + uf[f + sy] + uf[f + 1 + sy] + uf[f + sz] +
                                uf[f + 1 + sz] + uf[f + sy + sz] + uf[f + 1 + sy + sz]);
}

// ---- interp fused with the fine bc_scalar (main.f:3866-3900) --------------
__global__ void k_interp(double *__restrict__ uf, const double *__restrict__ uc, Dims df, Dims dc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > df.nx || j > df.ny) return;
  double x = 0.0;
  if (i != df.nx) {
    const int ci = i == 1 ? 2 : i;
    const int cj = j == 1 ? 2 : (j == df.ny ? df.ny - 1 : j);
    const int ck = k == 1 ? 2 : (k == df.nz ? df.nz - 1 : k);
    x = uc[dc.ix((ci >> 1) + 1, (cj >> 1) + 1, (ck >> 1) + 1)];
  }
  uf[df.ix(i, j, k)] = x;
}

// ---- addint: res = interp(uc) (+bc_scalar); uf += res everywhere ----------
__global__ void k_addint(double *__restrict__ uf, double *__restrict__ res, const double *__restrict__ uc,
                         Dims df, Dims dc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > df.nx || j > df.ny) return;
  double x = 0.0;
  if (i != df.nx) {
    const int ci = i == 1 ? 2 : i;
    const int cj = j == 1 ? 2 : (j == df.ny ? df.ny - 1 : j);
    const int ck = k == 1 ? 2 : (k == df.nz ? df.nz - 1 : k);
    x = uc[dc.ix((ci >> 1) + 1, (cj >> 1) + 1, (ck >> 1) + 1)];
  }
  const size_t q = df.ix(i, j, k);
  res[q] = x;
  uf[q] = uf[q] + x;
}

// ---- acfromac (main.f:3793-3844), one thread per coarse cell --------------
__device__ __forceinline__ double ac_a(const double *a2, Dims df, int i, int j, int k) {
  return 0.25 * (a2[df.ix(2 * i - 1, 2 * j - 1, 2 * k - 1)] + a2[df.ix(2 * i - 1, 2 * j - 2, 2 * k - 1)] +
                 a2[df.ix(2 * i - 1, 2 * j - 1, 2 * k - 2)] + a2[df.ix(2 * i - 1, 2 * j - 2, 2 * k - 2)]);
}
__device__ __forceinline__ double ac_b(const double *b2, Dims df, int i, int j, int k) {
  return 0.25 * (b2[df.ix(2 * i - 1, 2 * j - 1, 2 * k - 1)] + b2[df.ix(2 * i - 2, 2 * j - 1, 2 * k - 1)] +
                 b2[df.ix(2 * i - 1, 2 * j - 1, 2 * k - 2)] + b2[df.ix(2 * i - 2, 2 * j - 1, 2 * k - 2)]);
}
__device__ __forceinline__ double ac_c(const double *c2, Dims df, int i, int j, int k) {
  return 0.25 * (c2[df.ix(2 * i - 1, 2 * j - 1, 2 * k - 1)] + c2[df.ix(2 * i - 2, 2 * j - 1, 2 * k - 1)] +
                 c2[df.ix(2 * i - 1, 2 * j - 2, 2 * k - 1)] + c2[df.ix(2 * i - 2, 2 * j - 2, 2 * k - 1)]);
}

__global__ void k_acfromac(double *__restrict__ a, double *__restrict__ b, double *__restrict__ c,
                           double *__restrict__ ei, const double *__restrict__ a2,
                           const double *__restrict__ b2, const double *__restrict__ c2, Dims dc,
                           Dims df) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > dc.nx || j > dc.ny) return;
  const bool ii = i >= 2 && i <= dc.nx - 1, ji = j >= 2 && j <= dc.ny - 1, ki = k >= 2 && k <= dc.nz - 1;
  const size_t q = dc.ix(i, j, k);
  double va = 0.0, vb = 0.0, vc = 0.0;
  if (i <= dc.nx - 1 && ji && ki) { va = ac_a(a2, df, i, j, k); a[q] = va; }
  if (j <= dc.ny - 1 && ii && ki) { vb = ac_b(b2, df, i, j, k); b[q] = vb; }
  if (k <= dc.nz - 1 && ii && ji) { vc = ac_c(c2, df, i, j, k); c[q] = vc; }
  if (ii && ji && ki) {
    const double am = ac_a(a2, df, i - 1, j, k);
    const double bm = ac_b(b2, df, i, j - 1, k);
    const double cm = ac_c(c2, df, i, j, k - 1);
    ei[q] = 1.0 / (va + am + vb + bm + vc + cm);
  }
}

// ---- abcei (main.f:3582-3615) and bc_coef (main.f:4465-4494) --------------
__global__ void k_abc(double *__restrict__ a, double *__restrict__ b, double *__restrict__ c,
                      const double *__restrict__ cc, double r1, double r2, double k_gas, double k_liq, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  const double c0 = cc[q], cx = cc[q + 1], cy = cc[q + d.sy()], cz = cc[q + d.sz()];
  // Faces between two bulk cells of the same phase take the precomputed
  // 1/(r1*(c+c)+r2) (same operations, evaluated once on the host).
  const bool gas = is_zero_bits(c0), bulk = gas || is_one_bits(c0);
  const double kb = gas ? k_gas : k_liq;
  a[q] = (bulk && same_bits(cx, c0)) ? kb : 1.0 / (r1 * (c0 + cx) + r2);
  b[q] = (bulk && same_bits(cy, c0)) ? kb : 1.0 / (r1 * (c0 + cy) + r2);
  c[q] = (bulk && same_bits(cz, c0)) ? kb : 1.0 / (r1 * (c0 + cz) + r2);
}

// bc_coef: face 0 = a x-faces (all j,k), 1 = b(i,1,k) (i,k interior),
// 2 = c(i,j,1) (i interior, all j).
__global__ void k_bc_coef(double *__restrict__ a, double *__restrict__ b, double *__restrict__ c,
                          const double *__restrict__ cc, double r1, double r2, Dims d) {
  const int face = blockIdx.z;
  const int p = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int q = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (face == 0) {
    if (p > d.ny || q > d.nz) return;
    a[d.ix(1, p, q)] = a[d.ix(2, p, q)];
    a[d.ix(d.nx, p, q)] = a[d.ix(d.nx - 1, p, q)];
  } else if (face == 1) {
    if (p < 2 || p > d.nx - 1 || q < 2 || q > d.nz - 1) return;
    b[d.ix(p, 1, q)] = 1.0 / (r1 * (cc[d.ix(p, 1, q)] + cc[d.ix(p, 2, q)]) + r2);
  } else {
    if (p < 2 || p > d.nx - 1 || q > d.ny) return;
    c[d.ix(p, q, 1)] = 1.0 / (r1 * (cc[d.ix(p, q, 1)] + cc[d.ix(p, q, 2)]) + r2);
  }
}

// ei = 1 / (sum of the six face coefficients); with diag non-null the sum
// itself is stored there too (the diagonal of the operator, for the
// mixed solve's flux-form defect).
__global__ void k_ei(double *__restrict__ ei, double *__restrict__ diag, const double *__restrict__ a,
                     const double *__restrict__ b, const double *__restrict__ c, Dims d, double k_gas,
                     double k_liq, double e_gas, double e_liq, double d_gas, double d_liq) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  const double s0 = a[q], s1 = a[q - 1], s2 = b[q], s3 = b[q - d.sy()], s4 = c[q], s5 = c[q - d.sz()];
  // Six equal bulk faces: the precomputed 1/(k+k+k+k+k+k).
  if (same_bits(s0, s1) && same_bits(s0, s2) && same_bits(s0, s3) && same_bits(s0, s4) && same_bits(s0, s5) &&
      (same_bits(s0, k_gas) || same_bits(s0, k_liq))) {
    const bool gas = same_bits(s0, k_gas);
    ei[q] = gas ? e_gas : e_liq;
    if (diag) diag[q] = gas ? d_gas : d_liq;
    return;
  }
  const double sum = s0 + s1 + s2 + s3 + s4 + s5;
  ei[q] = 1.0 / sum;
  if (diag) diag[q] = sum;
}

// diag = the sum of the six face coefficients of every interior cell.
__global__ void k_diag(double *__restrict__ diag, const double *__restrict__ a, const double *__restrict__ b,
                       const double *__restrict__ c, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  diag[q] = a[q] + a[q - 1] + b[q] + b[q - d.sy()] + c[q] + c[q - d.sz()];
}

// ---- filterc27 (main.f:5473-5511), default-REAL weights -------------------
__global__ void k_filterc27(const double *__restrict__ cc, double *__restrict__ cf, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const double w0 = (double)0.2729f, w1 = (double)0.08185f, w2 = (double)0.0178f, w3 = (double)0.0028f;
  const size_t q = d.ix(i, j, k);
  const long sy = (long)d.sy(), sz = (long)d.sz();
#define C(di, dj, dk) cc[(long)q + (long)(di) + (long)(dj) * sy + (long)(dk) * sz]
  // Uniform 27-point neighbourhood of 0 or 1: the partial sums are exact
  // multiples of the value, so the weighted sum equals the precomputed one.
  const double c0 = C(0, 0, 0);
  const bool gas = is_zero_bits(c0);
  if (gas || is_one_bits(c0)) {
    bool uni = true;
#pragma unroll
    for (int dk = -1; dk <= 1; dk++)
#pragma unroll
      for (int dj = -1; dj <= 1; dj++)
#pragma unroll
        for (int di = -1; di <= 1; di++) uni = uni && same_bits(C(di, dj, dk), c0);
    if (uni) {
      double x = gas ? 0.0 : w0 * 1.0 + w1 * 6.0 + w2 * 12.0 + w3 * 8.0;
      if (x > 1.0) x = 1.0;
      cf[q] = x;
      return;
    }
  }
  const double s6 = C(-1, 0, 0) + C(1, 0, 0) + C(0, -1, 0) + C(0, 1, 0) + C(0, 0, 1) + C(0, 0, -1);
  const double s12 = C(-1, -1, 0) + C(-1, 1, 0) + C(1, -1, 0) + C(1, 1, 0) + C(0, 1, 1) + C(0, -1, 1) +
                     C(1, 0, 1) + C(-1, 0, 1) + C(0, 1, -1) + C(0, -1, -1) + C(1, 0, -1) + C(-1, 0, -1);
  const double s8 = C(1, 1, 1) + C(1, 1, -1) + C(1, -1, 1) + C(1, -1, -1) + C(-1, 1, 1) + C(-1, 1, -1) +
                    C(-1, -1, 1) + C(-1, -1, -1);
  double x = w0 * C(0, 0, 0) + w1 * s6 + w2 * s12 + w3 * s8;
#undef C
  if (x > 1.0) x = 1.0;
  cf[q] = x;
}

// ---- deterministic block reductions ----------------------------------------
template <int K>
__device__ __forceinline__ void block_sum_store(double (&v)[K], double *out) {
  __shared__ double sh[K][kRedThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int m = 0; m < K; m++) {
    double x = v[m];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[m][w] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int m = 0; m < K; m++) {
      double x = 0.0;
      for (int q = 0; q < kRedThreads / 32; q++) x += sh[m][q];
      out[(size_t)blockIdx.x * K + m] = x;
    }
  }
}

template <int K>
__device__ __forceinline__ void block_max_store(double (&v)[K], double *out) {
  __shared__ double sh[K][kRedThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int m = 0; m < K; m++) {
    double x = v[m];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_down_sync(0xffffffffu, x, o));
    if (lane == 0) sh[m][w] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int m = 0; m < K; m++) {
      double x = sh[m][0];
      for (int q = 1; q < kRedThreads / 32; q++) x = fmax(x, sh[m][q]);
      out[(size_t)blockIdx.x * K + m] = x;
    }
  }
}

// Second stage: one block folds kRedBlocks partials (fixed order).
template <int K, bool MAX>
__global__ void k_fold(const double *__restrict__ partials, double *__restrict__ out) {
  double v[K];
#pragma unroll
  for (int m = 0; m < K; m++) v[m] = MAX ? -1.0 : 0.0;
  for (int b = threadIdx.x; b < kRedBlocks; b += kRedThreads)
#pragma unroll
    for (int m = 0; m < K; m++) {
      const double x = partials[(size_t)b * K + m];
      v[m] = MAX ? fmax(v[m], x) : v[m] + x;
    }
  __shared__ double sh[K][kRedThreads];
#pragma unroll
  for (int m = 0; m < K; m++) sh[m][threadIdx.x] = v[m];
  __syncthreads();
  for (int s = kRedThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
#pragma unroll
      for (int m = 0; m < K; m++)
        sh[m][threadIdx.x] = MAX ? fmax(sh[m][threadIdx.x], sh[m][threadIdx.x + s])
                                 : sh[m][threadIdx.x] + sh[m][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int m = 0; m < K; m++) out[m] = sh[m][0];
}

// Interior cell of flat interior index t (i fastest).
// Interior cell t -> (i, j, k) with 32-bit division (interior counts stay
// below 2^32; 64-bit division is a long instruction sequence).
__device__ __forceinline__ size_t interior_cell(size_t t, Dims d, int &i, int &j, int &k) {
  const unsigned ni = (unsigned)(d.nx - 2), nj = (unsigned)(d.ny - 2), tt = (unsigned)t;
  const unsigned r = tt / ni;
  i = (int)(tt - r * ni) + 2;
  const unsigned kk = r / nj;
  j = (int)(r - kk * nj) + 2;
  k = (int)kk + 2;
  return d.ix(i, j, k);
}

// |x| as an ordered integer: the bit pattern of a non-negative double orders
// like its value, so maxima of |x| run on the integer pipe (a NaN is the
// largest pattern and propagates).
__device__ __forceinline__ long long abs_bits(double x) {
  return __double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFLL;
}

template <bool FMA>
__global__ void k_relres_partial(double *__restrict__ partials, const double *__restrict__ u,
                                 const double *__restrict__ rhs, const double *__restrict__ a,
                                 const double *__restrict__ b, const double *__restrict__ c, Dims d,
                                 double h2i) {
  const size_t n = (size_t)(d.nx - 2) * (d.ny - 2) * (d.nz - 2);
  const size_t sy = d.sy(), sz = d.sz();
  double v[2] = {0.0, 0.0};
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    const size_t q = interior_cell(t, d, i, j, k);
    const double r = cell_resid<FMA>(u, rhs, a, b, c, q, sy, sz, h2i);
    if (FMA) {
      v[0] = __fma_rn(r, r, v[0]);
      v[1] = __fma_rn(rhs[q], rhs[q], v[1]);
    } else {
      v[0] += r * r;
      v[1] += rhs[q] * rhs[q];
    }
  }
  block_sum_store<2>(v, partials);
}

__global__ void k_sum_partial(double *__restrict__ partials, const double *__restrict__ f, Dims d) {
  const size_t n = (size_t)(d.nx - 2) * (d.ny - 2) * (d.nz - 2);
  double v[1] = {0.0};
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    v[0] += f[interior_cell(t, d, i, j, k)];
  }
  block_sum_store<1>(v, partials);
}

__global__ void k_absmax3_partial(double *__restrict__ partials, const double *__restrict__ f0,
                                  const double *__restrict__ f1, const double *__restrict__ f2, Dims d) {
  const size_t n = (size_t)(d.nx - 2) * (d.ny - 2) * (d.nz - 2);
  long long m = 0;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    const size_t q = interior_cell(t, d, i, j, k);
    m = max(m, abs_bits(f0[q]));
    if (f1) m = max(m, abs_bits(f1[q]));
    if (f2) m = max(m, abs_bits(f2[q]));
  }
  double v[1] = {__longlong_as_double(m)};
  block_max_store<1>(v, partials);
}

__global__ void k_divmax_partial(double *__restrict__ partials, const double *__restrict__ u,
                                 const double *__restrict__ v_, const double *__restrict__ w, Dims d,
                                 double hi2) {
  const size_t n = (size_t)(d.nx - 2) * (d.ny - 2) * (d.nz - 2);
  const size_t sy = d.sy(), sz = d.sz();
  long long m = 0;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    const size_t q = interior_cell(t, d, i, j, k);
    const double dv = (u[q + 1] - u[q] + v_[q + sy] - v_[q] + w[q + sz] - w[q]) * hi2;
    m = max(m, abs_bits(dv));
  }
  double v[1] = {__longlong_as_double(m)};
  block_max_store<1>(v, partials);
}

const dim3 kBlk(32, 4, 1);

dim3 face_grid(Dims d, dim3 blk) {
  int m = d.nx > d.ny ? d.nx : d.ny;
  m = m > d.nz ? m : d.nz;
  return dim3((unsigned)((m + blk.x - 1) / blk.x), (unsigned)((m + blk.y - 1) / blk.y), 6);
}

dim3 full_grid(Dims d, dim3 blk) {
  return dim3((unsigned)((d.nx + blk.x - 1) / blk.x), (unsigned)((d.ny + blk.y - 1) / blk.y), (unsigned)d.nz);
}

}  // namespace

// ---- host launchers ---------------------------------------------------------
cudaError_t bc_scalar(double *s, Dims d, cudaStream_t st) {
  const dim3 blk(32, 8);
  DSG_COUNT k_bc_scalar<<<face_grid(d, blk), blk, 0, st>>>(s, d);
  return cudaGetLastError();
}

cudaError_t bc_resid(double *s, Dims d, cudaStream_t st) {
  const dim3 blk(32, 8);
  DSG_COUNT k_bc_xcopy<<<dim3((d.ny + 31) / 32, (d.nz + 7) / 8), blk, 0, st>>>(s, d);
  const int m = d.ny > d.nz ? d.ny : d.nz;
  DSG_COUNT k_bc_resid_yz<<<dim3((d.nx + 31) / 32, (m + 7) / 8, 2), blk, 0, st>>>(s, d);
  return cudaGetLastError();
}

cudaError_t bc_out(double *s, Dims d, cudaStream_t st) {
  const dim3 blk(32, 8);
  DSG_COUNT k_bc_xcopy<<<dim3((d.ny + 31) / 32, (d.nz + 7) / 8), blk, 0, st>>>(s, d);
  DSG_COUNT k_bc_out_y<<<dim3((d.nx + 31) / 32, (d.nz + 7) / 8), blk, 0, st>>>(s, d);
  DSG_COUNT k_bc_out_z<<<dim3((d.nx + 31) / 32, (d.ny + 7) / 8), blk, 0, st>>>(s, d);
  return cudaGetLastError();
}

static void relax_passes(double *u, double h2, const double *rhs, const double *a, const double *b,
                         const double *c, const double *ei, Dims d, double omega, bool fma, cudaStream_t st) {
  const int half = (d.nx - 2 + 1) / 2;
  const dim3 grid((unsigned)((half + kBlk.x - 1) / kBlk.x), (unsigned)((d.ny - 2 + kBlk.y - 1) / kBlk.y),
                  (unsigned)(d.nz - 2));
  for (int colour = 0; colour < 2; colour++) {
    if (fma)
      DSG_COUNT k_relax_colour<true><<<grid, kBlk, 0, st>>>(u, rhs, a, b, c, ei, d, h2, omega, colour);
    else
      DSG_COUNT k_relax_colour<false><<<grid, kBlk, 0, st>>>(u, rhs, a, b, c, ei, d, h2, omega, colour);
  }
}

cudaError_t relax(double *u, double lengthsize, const double *rhs, const double *a, const double *b,
                  const double *c, const double *ei, Dims d, double omega, cudaStream_t st) {
  return relax_n(1, u, lengthsize, rhs, a, b, c, ei, d, omega, st);
}

cudaError_t relax_n(int n, double *u, double lengthsize, const double *rhs, const double *a,
                    const double *b, const double *c, const double *ei, Dims d, double omega,
                    cudaStream_t st, bool fma) {
  if (n <= 0) return cudaSuccess;
  const double h1 = lengthsize / (d.nx - 2);
  const double h2 = h1 * h1;
  for (int q = 0; q < n; q++) relax_passes(u, h2, rhs, a, b, c, ei, d, omega, fma, st);
  return bc_scalar(u, d, st);
}

cudaError_t resid(double lengthsize, double *res, const double *u, const double *rhs, const double *a,
                  const double *b, const double *c, Dims d, cudaStream_t st, bool fma) {
  const double h1 = lengthsize / (d.nx - 2);
  const double h2i = 1.0 / (h1 * h1);
  if (fma)
    DSG_COUNT k_resid<true><<<interior_grid(d, kBlk), kBlk, 0, st>>>(res, u, rhs, a, b, c, d, h2i);
  else
    DSG_COUNT k_resid<false><<<interior_grid(d, kBlk), kBlk, 0, st>>>(res, u, rhs, a, b, c, d, h2i);
  return bc_resid(res, d, st);
}

cudaError_t rstrct(double *uc, const double *uf, Dims dc, cudaStream_t st) {
  const Dims df{2 * dc.nx - 2, 2 * dc.ny - 2, 2 * dc.nz - 2};
  DSG_COUNT k_rstrct<<<full_grid(dc, kBlk), kBlk, 0, st>>>(uc, uf, dc, df);
  return cudaGetLastError();
}

cudaError_t interp(double *uf, const double *uc, Dims df, cudaStream_t st) {
  const Dims dc{df.nx / 2 + 1, df.ny / 2 + 1, df.nz / 2 + 1};
  DSG_COUNT k_interp<<<full_grid(df, kBlk), kBlk, 0, st>>>(uf, uc, df, dc);
  return cudaGetLastError();
}

cudaError_t addint(double *uf, const double *uc, double *res, Dims df, cudaStream_t st) {
  const Dims dc{df.nx / 2 + 1, df.ny / 2 + 1, df.nz / 2 + 1};
  DSG_COUNT k_addint<<<full_grid(df, kBlk), kBlk, 0, st>>>(uf, res, uc, df, dc);
  return cudaGetLastError();
}

cudaError_t acfromac(double *a, double *b, double *c, double *ei, const double *a2, const double *b2,
                     const double *c2, Dims dc, cudaStream_t st) {
  const Dims df{2 * dc.nx - 2, 2 * dc.ny - 2, 2 * dc.nz - 2};
  DSG_COUNT k_acfromac<<<full_grid(dc, kBlk), kBlk, 0, st>>>(a, b, c, ei, a2, b2, c2, dc, df);
  return cudaGetLastError();
}

cudaError_t abcei(double *a, double *b, double *c, double *ei, const double *cc, double r1, double r2,
                  Dims d, cudaStream_t st, double *diag) {
  // bulk-face constants, same operation order as the kernels
  const double k_gas = 1.0 / (r1 * (0.0 + 0.0) + r2), k_liq = 1.0 / (r1 * (1.0 + 1.0) + r2);
  const double d_gas = k_gas + k_gas + k_gas + k_gas + k_gas + k_gas;
  const double d_liq = k_liq + k_liq + k_liq + k_liq + k_liq + k_liq;
  const double e_gas = 1.0 / d_gas, e_liq = 1.0 / d_liq;
  DSG_COUNT k_abc<<<interior_grid(d, kBlk), kBlk, 0, st>>>(a, b, c, cc, r1, r2, k_gas, k_liq, d);
  const dim3 blk(32, 8);
  DSG_COUNT k_bc_coef<<<face_grid(d, blk), blk, 0, st>>>(a, b, c, cc, r1, r2, d);
  DSG_COUNT k_ei<<<interior_grid(d, kBlk), kBlk, 0, st>>>(ei, diag, a, b, c, d, k_gas, k_liq, e_gas, e_liq, d_gas,
                                                         d_liq);
  return cudaGetLastError();
}

cudaError_t diag_sum(double *diag, const double *a, const double *b, const double *c, Dims d, cudaStream_t st) {
  DSG_COUNT k_diag<<<interior_grid(d, kBlk), kBlk, 0, st>>>(diag, a, b, c, d);
  return cudaGetLastError();
}

cudaError_t filterc27(const double *cc, double *cf, Dims d, cudaStream_t st) {
  DSG_COUNT k_filterc27<<<interior_grid(d, kBlk), kBlk, 0, st>>>(cc, cf, d);
  return cudaGetLastError();
}

cudaError_t relres_sums(double *out, double *partials, double lengthsize, const double *u,
                        const double *rhs, const double *a, const double *b, const double *c, Dims d,
                        cudaStream_t st, bool fma) {
  const double h1 = lengthsize / (d.nx - 2);
  const double h2i = 1.0 / (h1 * h1);
  if (fma)
    DSG_COUNT k_relres_partial<true><<<kRedBlocks, kRedThreads, 0, st>>>(partials, u, rhs, a, b, c, d, h2i);
  else
    DSG_COUNT k_relres_partial<false><<<kRedBlocks, kRedThreads, 0, st>>>(partials, u, rhs, a, b, c, d, h2i);
  DSG_COUNT k_fold<2, false><<<1, kRedThreads, 0, st>>>(partials, out);
  return cudaGetLastError();
}

cudaError_t sumfield(double *out, double *partials, const double *f, Dims d, cudaStream_t st) {
  DSG_COUNT k_sum_partial<<<kRedBlocks, kRedThreads, 0, st>>>(partials, f, d);
  DSG_COUNT k_fold<1, false><<<1, kRedThreads, 0, st>>>(partials, out);
  return cudaGetLastError();
}

cudaError_t absmax3(double *out, double *partials, const double *f0, const double *f1, const double *f2,
                    Dims d, cudaStream_t st) {
  DSG_COUNT k_absmax3_partial<<<kRedBlocks, kRedThreads, 0, st>>>(partials, f0, f1, f2, d);
  DSG_COUNT k_fold<1, true><<<1, kRedThreads, 0, st>>>(partials, out);
  return cudaGetLastError();
}

cudaError_t divmax(double *out, double *partials, const double *u, const double *v, const double *w,
                   double hi2, Dims d, cudaStream_t st) {
  DSG_COUNT k_divmax_partial<<<kRedBlocks, kRedThreads, 0, st>>>(partials, u, v, w, d, hi2);
  DSG_COUNT k_fold<1, true><<<1, kRedThreads, 0, st>>>(partials, out);
  return cudaGetLastError();
}

cudaError_t fill_zero(double *f, size_t n, cudaStream_t st) {
  return cudaMemsetAsync(f, 0, n * sizeof(double), st);
}

}  // namespace dsg

// ---- array-level C ABI --------------------------------------------------------
static int check_dims(int nx, int ny, int nz) {
  return (nx >= 3 && ny >= 3 && nz >= 3) ? DSG_OK : DSG_E_ARG;
}
static int cuda_rc(cudaError_t e) { return e == cudaSuccess ? DSG_OK : DSG_E_CUDA; }

extern "C" int dsg_relax(double *u, double lengthsize, const double *rhs, const double *a, const double *b,
                         const double *c, const double *ei, int nx, int ny, int nz, double omega,
                         void *stream) {
  if (check_dims(nx, ny, nz) || !u || !rhs || !a || !b || !c || !ei) return DSG_E_ARG;
  return cuda_rc(dsg::relax(u, lengthsize, rhs, a, b, c, ei, dsg::Dims{nx, ny, nz}, omega,
                            (cudaStream_t)stream));
}

extern "C" int dsg_resid(double lengthsize, double *res, const double *u, const double *rhs,
                         const double *a, const double *b, const double *c, int nx, int ny, int nz,
                         void *stream) {
  if (check_dims(nx, ny, nz) || !res || !u || !rhs || !a || !b || !c) return DSG_E_ARG;
  return cuda_rc(dsg::resid(lengthsize, res, u, rhs, a, b, c, dsg::Dims{nx, ny, nz}, (cudaStream_t)stream));
}

extern "C" int dsg_rstrct(double *uc, const double *uf, int ncx, int ncy, int ncz, void *stream) {
  if (check_dims(ncx, ncy, ncz) || !uc || !uf) return DSG_E_ARG;
  return cuda_rc(dsg::rstrct(uc, uf, dsg::Dims{ncx, ncy, ncz}, (cudaStream_t)stream));
}

extern "C" int dsg_interp(double *uf, const double *uc, int nfx, int nfy, int nfz, void *stream) {
  if (check_dims(nfx, nfy, nfz) || !uf || !uc || (nfx & 1) || (nfy & 1) || (nfz & 1)) return DSG_E_ARG;
  return cuda_rc(dsg::interp(uf, uc, dsg::Dims{nfx, nfy, nfz}, (cudaStream_t)stream));
}

extern "C" int dsg_addint(double *uf, const double *uc, double *res, int nfx, int nfy, int nfz, void *stream) {
  if (check_dims(nfx, nfy, nfz) || !uf || !uc || !res || (nfx & 1) || (nfy & 1) || (nfz & 1)) return DSG_E_ARG;
  return cuda_rc(dsg::addint(uf, uc, res, dsg::Dims{nfx, nfy, nfz}, (cudaStream_t)stream));
}

extern "C" int dsg_acfromac(double *a, double *b, double *c, double *ei, const double *a2, const double *b2,
                            const double *c2, int nx, int ny, int nz, void *stream) {
  if (check_dims(nx, ny, nz) || !a || !b || !c || !ei || !a2 || !b2 || !c2) return DSG_E_ARG;
  return cuda_rc(dsg::acfromac(a, b, c, ei, a2, b2, c2, dsg::Dims{nx, ny, nz}, (cudaStream_t)stream));
}

extern "C" int dsg_abcei(double *a, double *b, double *c, double *ei, const double *cc, double r1, double r2,
                         int nx, int ny, int nz, void *stream) {
  if (check_dims(nx, ny, nz) || !a || !b || !c || !ei || !cc) return DSG_E_ARG;
  return cuda_rc(dsg::abcei(a, b, c, ei, cc, r1, r2, dsg::Dims{nx, ny, nz}, (cudaStream_t)stream));
}

extern "C" int dsg_bc_scalar(double *s, int nx, int ny, int nz, void *stream) {
  if (check_dims(nx, ny, nz) || !s) return DSG_E_ARG;
  return cuda_rc(dsg::bc_scalar(s, dsg::Dims{nx, ny, nz}, (cudaStream_t)stream));
}

extern "C" int dsg_bc_resid(double *s, int nx, int ny, int nz, void *stream) {
  if (check_dims(nx, ny, nz) || !s) return DSG_E_ARG;
  return cuda_rc(dsg::bc_resid(s, dsg::Dims{nx, ny, nz}, (cudaStream_t)stream));
}

extern "C" int dsg_bc_out(double *s, int nx, int ny, int nz, void *stream) {
  if (check_dims(nx, ny, nz) || !s) return DSG_E_ARG;
  return cuda_rc(dsg::bc_out(s, dsg::Dims{nx, ny, nz}, (cudaStream_t)stream));
}

extern "C" int dsg_filterc27(const double *cc, double *cf, int nx, int ny, int nz, void *stream) {
  if (check_dims(nx, ny, nz) || !cc || !cf) return DSG_E_ARG;
  return cuda_rc(dsg::filterc27(cc, cf, dsg::Dims{nx, ny, nz}, (cudaStream_t)stream));
}
