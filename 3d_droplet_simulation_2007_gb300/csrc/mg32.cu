// mg32.cu -- FP32 multigrid bulk and the FP64 defect-correction kernels of the
// mixed-precision pressure solve (no reference counterpart: the reference
// solves in FP64 only).
//
// The V-cycle follows mglin's structure (main.f:3703-3759): red-black relax
// (main.f:3956-3997), 8-cell restriction of the residual, piecewise-constant
// prolong-and-add, NTOP sweeps on the coarsest grid, on the same operator with
// face coefficients coarsened as acfromac does (main.f:3793-3844).  It runs in
// FP32 on the correction equation L e = r, where r is the FP64 residual of the
// current FP64 pressure; the correction is accumulated in FP64.
//
// Differences from the FP64 kernels of mg64.cu, chosen for bandwidth:
//  * every kernel reads bc_scalar's ghost values virtually (own value / 0), so
//    no ghost-refresh launches exist in the FP32 cycle;
//  * the residual is never stored: one kernel forms the 8 fine residuals of a
//    coarse cell and writes their mean as the coarse right-hand side;
//  * this file is compiled with FMA contraction.
#include "mg32_cells.cuh"

namespace dsg {
namespace {

using namespace mg32;

__global__ void k_relax32_split(float *__restrict__ self, const float *__restrict__ other,
                                const float *__restrict__ rhs_self, const float *__restrict__ cc, Dims d, Split sp,
                                int c, float h2, float omega, float r1, float r2) {
  b_relax32_split(blockIdx, gridDim, self, other, rhs_self, cc, d, sp, c, h2, omega, r1, r2);
}

__global__ void k_resid_restrict32_split(float *__restrict__ rhs_c, float *__restrict__ u_c, const float *__restrict__ ue,
                                         const float *__restrict__ uo, const float *__restrict__ re,
                                         const float *__restrict__ ro, const float *__restrict__ cc, Dims df,
                                         Split sp, Dims dc, float h2i, float r1, float r2) {
  b_resid_restrict32_split(blockIdx, gridDim, rhs_c, u_c, ue, uo, re, ro, cc, df, sp, dc, h2i, r1, r2);
}

template <bool TRI>
__global__ void k_prolong32_split(float *__restrict__ ue, float *__restrict__ uo, const float *__restrict__ uc,
                                  Dims df, Split sp, Dims dc, int add) {
  b_prolong32_split<TRI>(blockIdx, gridDim, ue, uo, uc, df, sp, dc, add);
}

__global__ void k_restrict32_split(float *__restrict__ uc, const float *__restrict__ re,
                                   const float *__restrict__ ro, Dims dc, Split sp) {
  b_restrict32_split(blockIdx, gridDim, uc, re, ro, dc, sp);
}

__global__ void k_split_from64(float *__restrict__ ev, float *__restrict__ od, const double *__restrict__ src,
                               Dims d, Split sp) {
  b_split_from64(blockIdx, gridDim, ev, od, src, d, sp);
}

__global__ void k_relax32(float *__restrict__ u, const float *__restrict__ rhs, const float *__restrict__ a,
                          const float *__restrict__ b, const float *__restrict__ c, const float *__restrict__ ei,
                          Dims d, float h2, float omega, int colour) {
  b_relax32(blockIdx, gridDim, u, rhs, a, b, c, ei, d, h2, omega, colour);
}

__global__ void k_resid_restrict32(float *__restrict__ rhs_c, float *__restrict__ u_c, const float *__restrict__ u,
                                   const float *__restrict__ rhs, const float *__restrict__ a,
                                   const float *__restrict__ b, const float *__restrict__ c, Dims df, Dims dc,
                                   float h2i) {
  b_resid_restrict32(blockIdx, gridDim, rhs_c, u_c, u, rhs, a, b, c, df, dc, h2i);
}

template <bool TRI>
__global__ void k_prolong32(float *__restrict__ uf, const float *__restrict__ uc, Dims df, Dims dc, int add) {
  b_prolong32<TRI>(blockIdx, gridDim, uf, uc, df, dc, add);
}

__global__ void __launch_bounds__(kTailThreads, 1) k_vtail32(TailArgs A) { tail_body(A); }

__global__ void k_restrict32(float *__restrict__ uc, const float *__restrict__ uf, Dims dc, Dims df) {
  b_restrict32(blockIdx, gridDim, uc, uf, dc, df);
}

__global__ void k_acfromac32(float *__restrict__ a, float *__restrict__ b, float *__restrict__ c,
                             float *__restrict__ ei, const float *__restrict__ a2, const float *__restrict__ b2,
                             const float *__restrict__ c2, Dims dc, Dims df) {
  b_acfromac32(blockIdx, gridDim, a, b, c, ei, a2, b2, c2, dc, df);
}

__global__ void k_defect64(float *__restrict__ r_ev, float *__restrict__ r_od, Split sp,
                           double *__restrict__ partials, const double *__restrict__ p,
                           const double *__restrict__ rhs, const double *__restrict__ a,
                           const double *__restrict__ b, const double *__restrict__ c,
                           const double *__restrict__ diag, Dims d, double h2i) {
  b_defect64(blockIdx, gridDim, r_ev, r_od, sp, partials, p, rhs, a, b, c, diag, d, h2i);
}

__global__ void k_fold2(const double *__restrict__ partials, double *__restrict__ out) {
  b_fold2(blockIdx, gridDim, partials, out);
}

__global__ void k_correct64(double *__restrict__ p, const float *__restrict__ ev, const float *__restrict__ od,
                            Dims d, Split sp, int init) {
  b_correct64(blockIdx, gridDim, p, ev, od, d, sp, init);
}

__global__ void k_to32(float *__restrict__ dst, const double *__restrict__ src, size_t n) {
  b_to32(blockIdx, gridDim, dst, src, n);
}

__global__ void k_acfromac64to32(float *__restrict__ a, float *__restrict__ b, float *__restrict__ c,
                                 float *__restrict__ ei, const double *__restrict__ a2,
                                 const double *__restrict__ b2, const double *__restrict__ c2, Dims dc, Dims df) {
  b_acfromac64to32(blockIdx, gridDim, a, b, c, ei, a2, b2, c2, dc, df);
}

const dim3 kBlk(32, 4, 1);

inline int flat_blocks(size_t n) { return (int)((n + 255) / 256 < 8192 ? (n + 255) / 256 : 8192); }

}  // namespace

cudaError_t relax32_n(int n, float *u, float h2, const float *rhs, const float *a, const float *b, const float *c,
                      const float *ei, Dims d, float omega, cudaStream_t st) {
  const int half = (d.nx - 2 + 1) / 2;
  const dim3 grid((unsigned)((half + kBlk.x - 1) / kBlk.x), (unsigned)((d.ny - 2 + kBlk.y - 1) / kBlk.y),
                  (unsigned)(d.nz - 2));
  for (int q = 0; q < n; q++) {
    DSG_COUNT k_relax32<<<grid, kBlk, 0, st>>>(u, rhs, a, b, c, ei, d, h2, omega, 0);
    DSG_COUNT k_relax32<<<grid, kBlk, 0, st>>>(u, rhs, a, b, c, ei, d, h2, omega, 1);
  }
  return cudaGetLastError();
}

// Finest level, colour-split storage: u = {even, odd}, rhs = {even, odd}.
cudaError_t relax32_split_n(int n, float *const u[2], float *const rhs[2], const float *cc, Dims d, float h2,
                            float omega, float r1, float r2, cudaStream_t st) {
  const Split sp{(d.nx - 2) >> 1, d.ny - 2, d.nz - 2};
  const dim3 blk(32, 8, 1);  // a block covers 64 split indices x 8 rows
  const dim3 grid((unsigned)((sp.hx + 63) / 64), (unsigned)((d.ny - 2 + 7) / 8), (unsigned)(d.nz - 2));
  for (int q = 0; q < n; q++)
    for (int c = 0; c < 2; c++)
      DSG_COUNT k_relax32_split<<<grid, blk, 0, st>>>(u[c], u[1 - c], rhs[c], cc, d, sp, c, h2, omega, r1, r2);
  return cudaGetLastError();
}

cudaError_t resid_restrict32_split(float *rhs_c, float *u_c, float *const u[2], float *const rhs[2], const float *cc,
                                   Dims df, float h2i, float r1, float r2, cudaStream_t st) {
  const Dims dc{df.nx / 2 + 1, df.ny / 2 + 1, df.nz / 2 + 1};
  const Split sp{(df.nx - 2) >> 1, df.ny - 2, df.nz - 2};
  DSG_COUNT k_resid_restrict32_split<<<interior_grid(dc, kBlk), kBlk, 0, st>>>(rhs_c, u_c, u[0], u[1], rhs[0], rhs[1],
                                                                            cc, df, sp, dc, h2i, r1, r2);
  return cudaGetLastError();
}

cudaError_t prolong32_split(float *const u[2], const float *uc, Dims df, int add, int tri, cudaStream_t st) {
  const Dims dc{df.nx / 2 + 1, df.ny / 2 + 1, df.nz / 2 + 1};
  const Split sp{(df.nx - 2) >> 1, df.ny - 2, df.nz - 2};
  const dim3 grid((unsigned)((sp.hx + kBlk.x - 1) / kBlk.x), (unsigned)((df.ny - 2 + kBlk.y - 1) / kBlk.y),
                  (unsigned)(df.nz - 2));
  if (tri)
    DSG_COUNT k_prolong32_split<true><<<grid, kBlk, 0, st>>>(u[0], u[1], uc, df, sp, dc, add);
  else
    DSG_COUNT k_prolong32_split<false><<<grid, kBlk, 0, st>>>(u[0], u[1], uc, df, sp, dc, add);
  return cudaGetLastError();
}

cudaError_t restrict32_split(float *uc, float *const rhs[2], Dims dc, cudaStream_t st) {
  const Dims df{2 * dc.nx - 2, 2 * dc.ny - 2, 2 * dc.nz - 2};
  const Split sp{(df.nx - 2) >> 1, df.ny - 2, df.nz - 2};
  DSG_COUNT k_restrict32_split<<<interior_grid(dc, kBlk), kBlk, 0, st>>>(uc, rhs[0], rhs[1], dc, sp);
  return cudaGetLastError();
}

cudaError_t split_from64(float *const dst[2], const double *src, Dims d, cudaStream_t st) {
  const Split sp{(d.nx - 2) >> 1, d.ny - 2, d.nz - 2};
  DSG_COUNT k_split_from64<<<interior_grid(d, kBlk), kBlk, 0, st>>>(dst[0], dst[1], src, d, sp);
  return cudaGetLastError();
}

cudaError_t resid_restrict32(float *rhs_c, float *u_c, const float *u, const float *rhs, const float *a,
                             const float *b, const float *c, Dims df, float h2i, cudaStream_t st) {
  const Dims dc{df.nx / 2 + 1, df.ny / 2 + 1, df.nz / 2 + 1};
  DSG_COUNT k_resid_restrict32<<<interior_grid(dc, kBlk), kBlk, 0, st>>>(rhs_c, u_c, u, rhs, a, b, c, df, dc, h2i);
  return cudaGetLastError();
}

cudaError_t vtail32(const TailArgs &args, cudaStream_t st) {
  DSG_COUNT k_vtail32<<<1, kTailThreads, 0, st>>>(args);
  return cudaGetLastError();
}


cudaError_t prolong32(float *uf, const float *uc, Dims df, int add, int tri, cudaStream_t st) {
  const Dims dc{df.nx / 2 + 1, df.ny / 2 + 1, df.nz / 2 + 1};
  if (tri)
    DSG_COUNT k_prolong32<true><<<interior_grid(df, kBlk), kBlk, 0, st>>>(uf, uc, df, dc, add);
  else
    DSG_COUNT k_prolong32<false><<<interior_grid(df, kBlk), kBlk, 0, st>>>(uf, uc, df, dc, add);
  return cudaGetLastError();
}

cudaError_t restrict32(float *uc, const float *uf, Dims dc, cudaStream_t st) {
  const Dims df{2 * dc.nx - 2, 2 * dc.ny - 2, 2 * dc.nz - 2};
  DSG_COUNT k_restrict32<<<interior_grid(dc, kBlk), kBlk, 0, st>>>(uc, uf, dc, df);
  return cudaGetLastError();
}

cudaError_t acfromac32(float *a, float *b, float *c, float *ei, const float *a2, const float *b2, const float *c2,
                       Dims dc, cudaStream_t st) {
  const Dims df{2 * dc.nx - 2, 2 * dc.ny - 2, 2 * dc.nz - 2};
  const dim3 grid((unsigned)((dc.nx + kBlk.x - 1) / kBlk.x), (unsigned)((dc.ny + kBlk.y - 1) / kBlk.y),
                  (unsigned)dc.nz);
  DSG_COUNT k_acfromac32<<<grid, kBlk, 0, st>>>(a, b, c, ei, a2, b2, c2, dc, df);
  return cudaGetLastError();
}

cudaError_t acfromac64to32(float *a, float *b, float *c, float *ei, const double *a2, const double *b2,
                           const double *c2, Dims dc, cudaStream_t st) {
  const Dims df{2 * dc.nx - 2, 2 * dc.ny - 2, 2 * dc.nz - 2};
  const dim3 grid((unsigned)((dc.nx + kBlk.x - 1) / kBlk.x), (unsigned)((dc.ny + kBlk.y - 1) / kBlk.y),
                  (unsigned)dc.nz);
  DSG_COUNT k_acfromac64to32<<<grid, kBlk, 0, st>>>(a, b, c, ei, a2, b2, c2, dc, df);
  return cudaGetLastError();
}

cudaError_t defect64(float *const r32[2], double *out2, double *partials, const double *p, const double *rhs,
                     const double *a, const double *b, const double *c, const double *diag, Dims d,
                     double lengthsize, cudaStream_t st) {
  const double h1 = lengthsize / (d.nx - 2);
  const double h2i = 1.0 / (h1 * h1);
  const Split sp{(d.nx - 2) >> 1, d.ny - 2, d.nz - 2};
  DSG_COUNT k_defect64<<<kRedBlocks, kRedThreads, 0, st>>>(r32[0], r32[1], sp, partials, p, rhs, a, b, c, diag, d,
                                                           h2i);
  DSG_COUNT k_fold2<<<1, kRedThreads, 0, st>>>(partials, out2);
  return cudaGetLastError();
}

cudaError_t correct64(double *p, float *const e[2], Dims d, int init, cudaStream_t st) {
  const Split sp{(d.nx - 2) >> 1, d.ny - 2, d.nz - 2};
  DSG_COUNT k_correct64<<<interior_grid(d, kBlk), kBlk, 0, st>>>(p, e[0], e[1], d, sp, init);
  return cudaGetLastError();
}

cudaError_t to32(float *dst, const double *src, size_t n, cudaStream_t st) {
  DSG_COUNT k_to32<<<flat_blocks(n), 256, 0, st>>>(dst, src, n);
  return cudaGetLastError();
}

}  // namespace dsg
