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

// ---- GCR over the FP32 V-cycle ----------------------------------------------
//
// The kernels below run over the finest level's colour-split index range
// t = m + hx (j - 2 + ny2 (k - 2)), both colours per index, so that every
// split array is read with unit stride and the FP64 pressure (natural layout)
// in runs of two cells.  Sums are formed per thread in FP32, per block in
// FP64 in a fixed order, and folded by one block: the results are
// deterministic.

// Division by a divisor d >= 1 fixed at launch as a multiply-high, an add and
// a shift (the round-up method of Granlund and Montgomery, 1994): with
// s = ceil(log2 d) and m = floor(2^32 (2^s - d) / d) + 1,
// n / d = (umulhi(n, m) + n) >> s for every 32-bit n (the sum taken in 64
// bits).  It replaces the two integer divisions of each index decode.
struct FastDiv {
  unsigned d, m, s;
};

FastDiv fast_div(unsigned d) {
  unsigned s = 0;
  while ((1ull << s) < d) s++;
  return FastDiv{d, (unsigned)((((1ull << 32) * ((1ull << s) - d)) / d) + 1), s};
}

__device__ __forceinline__ unsigned fdiv(unsigned n, const FastDiv &f) {
  return (unsigned)(((unsigned long long)__umulhi(n, f.m) + n) >> f.s);
}

// Index t's split coordinates (hx and ny2 divisors of the split layout).
struct SplitIx {
  int m, j, k;
};
struct SplitDiv {
  FastDiv hx, ny2;
};
__device__ __forceinline__ SplitIx split_ix(unsigned t, const SplitDiv &sd) {
  const unsigned rem = fdiv(t, sd.hx), kk = fdiv(rem, sd.ny2);
  return SplitIx{(int)(t - rem * sd.hx.d), (int)(rem - kk * sd.ny2.d) + 2, (int)kk + 2};
}

// NS FP64 sums of the block (thread 0 holds them afterwards) written to
// out[NS * block + s].
template <int NS>
__device__ __forceinline__ void block_partials(double (&v)[NS], double *__restrict__ out) {
  __shared__ double sh[NS][kRedThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int s = 0; s < NS; s++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[s] += __shfl_down_sync(0xffffffffu, v[s], o);
    if (lane == 0) sh[s][wid] = v[s];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int s = 0; s < NS; s++) {
      double x = lane < kRedThreads / 32 ? sh[s][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) out[NS * blockIdx.x + s] = x;
    }
  }
}

// w = A z (A z = lap(z) / h^2, the operator whose residual the V-cycle
// restricts), stored when STORE, and the sums (w,w), (r,w), (w,q), (r,q) of
// the current residual r and the previous direction's image q (not read on
// the first iteration).
template <bool FIRST, bool STORE>
__global__ void __launch_bounds__(kRedThreads) k_gcr_apply(float *__restrict__ w_ev, float *__restrict__ w_od,
                                                           double *__restrict__ partials,
                                                           const float *__restrict__ z_ev,
                                                           const float *__restrict__ z_od,
                                                           const float *__restrict__ r_ev,
                                                           const float *__restrict__ r_od,
                                                           const float *__restrict__ q_ev,
                                                           const float *__restrict__ q_od, const float *__restrict__ cc,
                                                           Dims d, Split sp, SplitDiv sd, float h2i, float r1,
                                                           float r2) {
  const unsigned n = (unsigned)sp.hx * (unsigned)sp.ny2 * (unsigned)sp.nz2;
  float ww = 0.f, rw = 0.f, wq = 0.f, rq = 0.f;
  for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const SplitIx x = split_ix(t, sd);
#pragma unroll
    for (int c = 0; c < 2; c++) {
      const float w = h2i * lap32_split_cell(c ? z_od : z_ev, c ? z_ev : z_od, cc, d, sp, c, r1, r2, x.m, x.j, x.k, t);
      if (STORE) (c ? w_od : w_ev)[t] = w;
      const float r = (c ? r_od : r_ev)[t];
      ww = fmaf(w, w, ww);
      rw = fmaf(r, w, rw);
      if (!FIRST) {
        const float q = (c ? q_od : q_ev)[t];
        wq = fmaf(w, q, wq);
        rq = fmaf(r, q, rq);
      }
    }
  }
  double v[4] = {ww, rw, wq, rq};
  block_partials<4>(v, partials);
}

// Step lengths from the sums: new direction d = z - beta d_prev with image
// q = w - beta q_prev orthogonal to q_prev, and the step alpha that minimises
// |r - alpha q|.  coef = {alpha, beta, (w,w), (r,w), (w,q), (r,q), (q,q) of
// the previous direction}.  A breakdown (a non-finite or non-positive
// denominator) gives alpha = beta = 0: no update, and the FP64 defect that
// follows decides.
template <bool FIRST>
__global__ void __launch_bounds__(kRedThreads) k_gcr_fold(const double *__restrict__ p1,
                                                          const double *__restrict__ p2, double *__restrict__ coef,
                                                          int nb) {
  double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nb; b += kRedThreads) {
#pragma unroll
    for (int s = 0; s < 4; s++) v[s] += p1[4 * b + s];
    if (!FIRST) v[4] += p2[2 * b];
  }
  __shared__ double tot[5];
  __shared__ double sh[5][kRedThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int s = 0; s < 5; s++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[s] += __shfl_down_sync(0xffffffffu, v[s], o);
    if (lane == 0) sh[s][wid] = v[s];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int s = 0; s < 5; s++) {
      double x = lane < kRedThreads / 32 ? sh[s][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) tot[s] = x;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double ww = tot[0], rw = tot[1], wq = tot[2], rq = tot[3], qq0 = tot[4];
    double alpha, beta;
    if (FIRST) {
      beta = 0.0;
      alpha = rw / ww;
    } else {
      beta = wq / qq0;
      const double qq = ww - beta * wq;  // |w - beta q_prev|^2
      alpha = (rw - beta * rq) / qq;
      if (!(qq > 0.0) || !(qq0 > 0.0)) alpha = beta = 0.0;
    }
    if (!(ww > 0.0) || !isfinite(alpha) || !isfinite(beta)) alpha = beta = 0.0;
    coef[0] = alpha;
    coef[1] = beta;
#pragma unroll
    for (int s = 0; s < 5; s++) coef[2 + s] = tot[s];
  }
}

// d = z - beta d, q = w - beta q (FIRST: d = z, q = w), r -= alpha q and the
// FP64 pressure p += alpha d; sums (q,q) and (r,r) of the new q and r.
template <bool FIRST>
__global__ void __launch_bounds__(kRedThreads) k_gcr_update(double *__restrict__ p, float *__restrict__ d_ev,
                                                            float *__restrict__ d_od, float *__restrict__ q_ev,
                                                            float *__restrict__ q_od, float *__restrict__ r_ev,
                                                            float *__restrict__ r_od, double *__restrict__ partials,
                                                            const float *__restrict__ z_ev,
                                                            const float *__restrict__ z_od,
                                                            const float *__restrict__ w_ev,
                                                            const float *__restrict__ w_od,
                                                            const double *__restrict__ coef, Dims d, Split sp,
                                                            SplitDiv sd) {
  const double alpha = coef[0];
  const float alpha32 = (float)alpha, beta = (float)coef[1];
  const unsigned n = (unsigned)sp.hx * (unsigned)sp.ny2 * (unsigned)sp.nz2;
  float qq = 0.f, rr = 0.f;
  for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const SplitIx x = split_ix(t, sd);
#pragma unroll
    for (int c = 0; c < 2; c++) {
      float *dc = c ? d_od : d_ev, *qc = c ? q_od : q_ev, *rc = c ? r_od : r_ev;
      const float z = (c ? z_od : z_ev)[t], w = (c ? w_od : w_ev)[t];
      const float dn = FIRST ? z : fmaf(-beta, dc[t], z);
      const float qn = FIRST ? w : fmaf(-beta, qc[t], w);
      const float rn = fmaf(-alpha32, qn, rc[t]);
      dc[t] = dn;
      qc[t] = qn;
      rc[t] = rn;
      const int i = 2 + 2 * x.m + ((x.j + x.k + c) & 1);
      const unsigned q = ix32(d, i, x.j, x.k);
      p[q] = fma(alpha, (double)dn, p[q]);
      qq = fmaf(qn, qn, qq);
      rr = fmaf(rn, rn, rr);
    }
  }
  double v[2] = {qq, rr};
  block_partials<2>(v, partials);
}

// Last iteration: p += alpha (z - beta d) (FIRST: p += alpha z).
template <bool FIRST>
__global__ void __launch_bounds__(kRedThreads) k_gcr_final(double *__restrict__ p, const float *__restrict__ z_ev,
                                                           const float *__restrict__ z_od,
                                                           const float *__restrict__ d_ev,
                                                           const float *__restrict__ d_od,
                                                           const double *__restrict__ coef, Dims d, Split sp,
                                                           SplitDiv sd) {
  const double alpha = coef[0];
  const float beta = (float)coef[1];
  const unsigned n = (unsigned)sp.hx * (unsigned)sp.ny2 * (unsigned)sp.nz2;
  for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const SplitIx x = split_ix(t, sd);
#pragma unroll
    for (int c = 0; c < 2; c++) {
      const float z = (c ? z_od : z_ev)[t];
      const float dn = FIRST ? z : fmaf(-beta, (c ? d_od : d_ev)[t], z);
      const int i = 2 + 2 * x.m + ((x.j + x.k + c) & 1);
      const unsigned q = ix32(d, i, x.j, x.k);
      p[q] = fma(alpha, (double)dn, p[q]);
    }
  }
}

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

cudaError_t gcr_step(int first, int last, const GcrBufs &g, double *p, float *const z[2], float *const r[2],
                     const float *cc, Dims d, float h2i, float r1, float r2, cudaStream_t st) {
  const Split sp{(d.nx - 2) >> 1, d.ny - 2, d.nz - 2};
  const SplitDiv sd{fast_div((unsigned)sp.hx), fast_div((unsigned)sp.ny2)};
  const int nb = kRedBlocks;
  if (first) {
    if (last)
      DSG_COUNT k_gcr_apply<true, false><<<nb, kRedThreads, 0, st>>>(g.w[0], g.w[1], g.p1, z[0], z[1], r[0], r[1],
                                                                    g.q[0], g.q[1], cc, d, sp, sd, h2i, r1, r2);
    else
      DSG_COUNT k_gcr_apply<true, true><<<nb, kRedThreads, 0, st>>>(g.w[0], g.w[1], g.p1, z[0], z[1], r[0], r[1],
                                                                   g.q[0], g.q[1], cc, d, sp, sd, h2i, r1, r2);
    DSG_COUNT k_gcr_fold<true><<<1, kRedThreads, 0, st>>>(g.p1, g.p2, g.coef, nb);
    if (last)
      DSG_COUNT k_gcr_final<true><<<nb, kRedThreads, 0, st>>>(p, z[0], z[1], g.d[0], g.d[1], g.coef, d, sp, sd);
    else
      DSG_COUNT k_gcr_update<true><<<nb, kRedThreads, 0, st>>>(p, g.d[0], g.d[1], g.q[0], g.q[1], r[0], r[1], g.p2,
                                                              z[0], z[1], g.w[0], g.w[1], g.coef, d, sp, sd);
  } else {
    if (last)
      DSG_COUNT k_gcr_apply<false, false><<<nb, kRedThreads, 0, st>>>(g.w[0], g.w[1], g.p1, z[0], z[1], r[0], r[1],
                                                                     g.q[0], g.q[1], cc, d, sp, sd, h2i, r1, r2);
    else
      DSG_COUNT k_gcr_apply<false, true><<<nb, kRedThreads, 0, st>>>(g.w[0], g.w[1], g.p1, z[0], z[1], r[0], r[1],
                                                                    g.q[0], g.q[1], cc, d, sp, sd, h2i, r1, r2);
    DSG_COUNT k_gcr_fold<false><<<1, kRedThreads, 0, st>>>(g.p1, g.p2, g.coef, nb);
    if (last)
      DSG_COUNT k_gcr_final<false><<<nb, kRedThreads, 0, st>>>(p, z[0], z[1], g.d[0], g.d[1], g.coef, d, sp, sd);
    else
      DSG_COUNT k_gcr_update<false><<<nb, kRedThreads, 0, st>>>(p, g.d[0], g.d[1], g.q[0], g.q[1], r[0], r[1], g.p2,
                                                               z[0], z[1], g.w[0], g.w[1], g.coef, d, sp, sd);
  }
  return cudaGetLastError();
}

}  // namespace dsg
