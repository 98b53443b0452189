// mg32_cells.cuh -- per-cell operations and per-block bodies of the FP32
// multigrid and FP64 defect-correction kernels (mg32.cu).
//
// Every kernel of mg32.cu is a thin wrapper that calls its block body here with
// its own blockIdx and gridDim.  The batched kernels of batch.cu call the same
// bodies with the block index a block has inside one ensemble member's grid,
// so a member solved in a batch computes exactly the bits it computes alone.
// Both translation units are compiled with FMA contraction.
#pragma once
#include "dsg_internal.cuh"

namespace dsg {
namespace mg32 {
namespace {  // each including translation unit keeps its own copies

// 32-bit linear index of node (i,j,k) (1-based, ghosts included): grids stay
// below 2^31 nodes, and 32-bit index arithmetic is markedly cheaper than
// 64-bit in these issue-bound sweeps.
__device__ __forceinline__ unsigned ix32(Dims d, int i, int j, int k) {
  return (unsigned)(i - 1) + (unsigned)d.nx * ((unsigned)(j - 1) + (unsigned)d.ny * (unsigned)(k - 1));
}

// Virtual-ghost neighbour reads of bc_scalar semantics on level dims d.
struct Nb {
  float xp, xm, yp, ym, zp, zm;
};

__device__ __forceinline__ Nb neighbours(const float *__restrict__ u, unsigned q, int i, int j, int k, Dims d,
                                         float uc) {
  Nb n;
  const float *uq = u + q;
  const int sy = d.nx, sz = d.nx * d.ny;
  n.xp = (i + 1 == d.nx) ? 0.f : uq[1];
  n.xm = (i - 1 == 1) ? uc : uq[-1];
  n.yp = (j + 1 == d.ny) ? uc : uq[sy];
  n.ym = (j - 1 == 1) ? uc : uq[-sy];
  n.zp = (k + 1 == d.nz) ? uc : uq[sz];
  n.zm = (k - 1 == 1) ? uc : uq[-sz];
  return n;
}

// ---- finest level: colour-split storage --------------------------------------
//
// On the finest level the FP32 correction u and right-hand side are stored
// split by colour: cells with i+j+k even (the first pass of relax) in one
// array, odd in another, each (nx-2)/2 x (ny-2) x (nz-2) over the interior
// only (ghosts are virtual).  In row (j,k) the colour-c cells are
// i = 2 + 2m + p with p = (j+k+c) & 1.  A colour pass then reads the other
// colour, reads and writes its own colour and reads cc for the face
// coefficients, all with full 32-byte sectors: 24 bytes per cell per relax.
// Face coefficients are formed from the FP32 volume fraction as abcei does,
// a = 1/(r1*(c_i+c_{i+1}) + r2), with bc_coef's a(1) = a(2).  (Storing cc
// colour-split as well, so that every load of a pass is a contiguous run, was
// measured slower: 3.88 against 4.25 TB/s at 256^3.)
struct Split {
  int hx, ny2, nz2;  // (nx-2)/2, ny-2, nz-2
  __host__ __device__ __forceinline__ size_t at(int m, int j, int k) const {
    return (size_t)m + (size_t)hx * ((size_t)(j - 2) + (size_t)ny2 * (size_t)(k - 2));
  }
};


__device__ __forceinline__ unsigned at32(Split sp, int m, int j, int k) {
  return (unsigned)m + (unsigned)sp.hx * ((unsigned)(j - 2) + (unsigned)sp.ny2 * (unsigned)(k - 2));
}

// Single-instruction reciprocal (MUFU): the FP32 V-cycle is a preconditioner
// of the FP64 defect correction, so an approximate 1/x is sufficient.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float face_coef(float x, float y, float r1, float r2) {
  return rcp_approx(r1 * (x + y) + r2);
}

// Value of cell (i,j,k) of a colour-split pair {even, odd}.
__device__ __forceinline__ float split_get(const float *__restrict__ ev, const float *__restrict__ od, Split sp,
                                           int i, int j, int k) {
  const unsigned q = at32(sp, (i - 2) >> 1, j, k);
  return ((i + j + k) & 1) ? od[q] : ev[q];
}

// ---- prolongation of a coarse correction ------------------------------------
//
// Two interpolations: the reference's piecewise-constant injection (interp /
// addint, main.f:3866-3954: a fine cell takes its parent's value) and
// cell-centred trilinear interpolation, where a fine cell takes 3/4 of its
// parent plus 1/4 of the parent's neighbour on the fine cell's side along
// each axis (weights 27/64, 9/64, 3/64, 1/64).  Trilinear reaches the
// tolerance in fewer V-cycles (7 against 9 from a zero start on a 128^3
// splash system, V(4,4)).  Coarse ghosts are read virtually as bc_scalar
// sets them: the own value, and 0 beyond the x = nx face.  Explicit fmaf
// fixes the rounding, so that every kernel that interpolates gives the same
// bits.

// Bilinear y-z combination at coarse x-index x (parent row pj, pk; neighbours nj, nk).
__device__ __forceinline__ float tri_yz(const float *__restrict__ uc, Dims dc, int x, int pj, int nj, int pk,
                                        int nk) {
  const float a = uc[ix32(dc, x, pj, pk)], b = uc[ix32(dc, x, nj, pk)];
  const float c = uc[ix32(dc, x, pj, nk)], e = uc[ix32(dc, x, nj, nk)];
  return fmaf(0.0625f, e, fmaf(0.1875f, c, fmaf(0.1875f, b, 0.5625f * a)));
}

// Coarse neighbour of parent p on the side of fine index f (odd f: +1, even:
// -1); a Neumann ghost (index 1 or nc) resolves to the parent itself.
__device__ __forceinline__ int tri_nb(int f, int p, int nc) {
  const int n = p + ((f & 1) ? 1 : -1);
  return (n == 1 || n == nc) ? p : n;
}

// x-combination of the parent's and the neighbour's y-z values.
__device__ __forceinline__ float tri_x(float yp, float yn) { return fmaf(0.25f, yn, 0.75f * yp); }

// Trilinear value of the coarse correction uc at fine cell (i,j,k).
__device__ __forceinline__ float trilin32(const float *__restrict__ uc, Dims dc, int i, int j, int k) {
  const int pi = (i >> 1) + 1, pj = (j >> 1) + 1, pk = (k >> 1) + 1;
  const int nj = tri_nb(j, pj, dc.ny), nk = tri_nb(k, pk, dc.nz);
  const float yp = tri_yz(uc, dc, pi, pj, nj, pk, nk);
  const int ni = pi + ((i & 1) ? 1 : -1);
  const float yn = ni == dc.nx ? 0.f : (ni == 1 ? yp : tri_yz(uc, dc, ni, pj, nj, pk, nk));
  return tri_x(yp, yn);
}

// Coarse correction at fine cell (i,j,k): trilinear (TRI) or injection.
template <bool TRI>
__device__ __forceinline__ float coarse_at(const float *__restrict__ uc, Dims dc, int i, int j, int k) {
  return TRI ? trilin32(uc, dc, i, j, k) : uc[ix32(dc, (i >> 1) + 1, (j >> 1) + 1, (k >> 1) + 1)];
}

// One colour-c update (0 = i+j+k even) of the finest-level cell at split
// index (m, j, k).  Offsets are 32-bit (grids stay below 2^31 nodes) and
// taken from one base pointer per array, which cut the pass from 51.3 to
// 47.2 us at 258^3 against 64-bit indexing, with the same bits.
__device__ __forceinline__ void relax32_split_cell(float *__restrict__ self, const float *__restrict__ other,
                                                   const float *__restrict__ rhs_self, const float *__restrict__ cc,
                                                   Dims d, Split sp, int c, float h2, float omega, float r1, float r2,
                                                   int m, int j, int k) {
  const int p = (j + k + c) & 1;
  const int i = 2 + 2 * m + p;
  const int row = sp.hx, plane = sp.hx * sp.ny2;
  const unsigned qs = (unsigned)m + (unsigned)sp.hx * ((unsigned)(j - 2) + (unsigned)sp.ny2 * (unsigned)(k - 2));
  const float *o = other + qs;
  const float uc = self[qs];
  const float xm = (m == 0 && p == 0) ? uc : o[p - 1];
  const float xp = (m == sp.hx - 1 && p == 1) ? 0.f : o[p];
  const float ym = (j == 2) ? uc : o[-row];
  const float yp = (j == d.ny - 1) ? uc : o[row];
  const float zm = (k == 2) ? uc : o[-plane];
  const float zp = (k == d.nz - 1) ? uc : o[plane];
  const unsigned q = (unsigned)(i - 1) + (unsigned)d.nx * ((unsigned)(j - 1) + (unsigned)d.ny * (unsigned)(k - 1));
  const float *cq = cc + q;
  const int sy = d.nx, sz = d.nx * d.ny;
  const float c0 = cq[0];
  const float ae = face_coef(c0, cq[1], r1, r2);
  const float aw = (i == 2) ? ae : face_coef(cq[-1], c0, r1, r2);
  const float bn = face_coef(c0, cq[sy], r1, r2);
  const float bs = face_coef(cq[-sy], c0, r1, r2);
  const float ct = face_coef(c0, cq[sz], r1, r2);
  const float cb = face_coef(cq[-sz], c0, r1, r2);
  const float ei = rcp_approx(ae + aw + bn + bs + ct + cb);
  const float temp = (ae * xp + aw * xm + bn * yp + bs * ym + ct * zp + cb * zm - h2 * rhs_self[qs]) * ei;
  self[qs] = omega * temp + (1.f - omega) * uc;
}

// Operator of the finest-level FP32 correction equation at the colour-c cell of
// split index (m, j, k) (qs its offset): sum_f a_f (z_f - z) over the six faces,
// with the neighbours, virtual ghosts and face coefficients of
// relax32_split_cell.  The residual of relax is rhs - lap / h^2.
__device__ __forceinline__ float lap32_split_cell(const float *__restrict__ self, const float *__restrict__ other,
                                                  const float *__restrict__ cc, Dims d, Split sp, int c, float r1,
                                                  float r2, int m, int j, int k, unsigned qs) {
  const int p = (j + k + c) & 1;
  const int i = 2 + 2 * m + p;
  const int row = sp.hx, plane = sp.hx * sp.ny2;
  const float *o = other + qs;
  const float uc = self[qs];
  const float xm = (m == 0 && p == 0) ? uc : o[p - 1];
  const float xp = (m == sp.hx - 1 && p == 1) ? 0.f : o[p];
  const float ym = (j == 2) ? uc : o[-row];
  const float yp = (j == d.ny - 1) ? uc : o[row];
  const float zm = (k == 2) ? uc : o[-plane];
  const float zp = (k == d.nz - 1) ? uc : o[plane];
  const unsigned q = (unsigned)(i - 1) + (unsigned)d.nx * ((unsigned)(j - 1) + (unsigned)d.ny * (unsigned)(k - 1));
  const float *cq = cc + q;
  const int sy = d.nx, sz = d.nx * d.ny;
  const float c0 = cq[0];
  const float ae = face_coef(c0, cq[1], r1, r2);
  const float aw = (i == 2) ? ae : face_coef(cq[-1], c0, r1, r2);
  const float bn = face_coef(c0, cq[sy], r1, r2);
  const float bs = face_coef(cq[-sy], c0, r1, r2);
  const float ct = face_coef(c0, cq[sz], r1, r2);
  const float cb = face_coef(cq[-sz], c0, r1, r2);
  return ae * (xp - uc) + aw * (xm - uc) + bn * (yp - uc) + bs * (ym - uc) + ct * (zp - uc) + cb * (zm - uc);
}

// One colour pass on the finest level: each thread updates split indices m
// and m + blockDim.x of its row (two independent cells in flight; 45.7 against
// 47.2 us per pass with one).
__device__ __forceinline__ void b_relax32_split(const uint3 B, const uint3 G, float *__restrict__ self, const float *__restrict__ other,
                                const float *__restrict__ rhs_self, const float *__restrict__ cc, Dims d, Split sp,
                                int c, float h2, float omega, float r1, float r2) {
  const int m = B.x * 2 * blockDim.x + threadIdx.x;
  const int j = B.y * blockDim.y + threadIdx.y + 2;
  const int k = B.z + 2;
  if (j > d.ny - 1) return;
  if (m < sp.hx) relax32_split_cell(self, other, rhs_self, cc, d, sp, c, h2, omega, r1, r2, m, j, k);
  if (m + (int)blockDim.x < sp.hx)
    relax32_split_cell(self, other, rhs_self, cc, d, sp, c, h2, omega, r1, r2, m + blockDim.x, j, k);
}

// Finest-level residual (cc-derived operator, virtual ghosts) restricted to the
// coarse rhs: mean of the 8 fine residuals of each coarse cell.
__device__ __forceinline__ void b_resid_restrict32_split(const uint3 B, const uint3 G, float *__restrict__ rhs_c, float *__restrict__ u_c, const float *__restrict__ ue,
                                         const float *__restrict__ uo, const float *__restrict__ re,
                                         const float *__restrict__ ro, const float *__restrict__ cc, Dims df,
                                         Split sp, Dims dc, float h2i, float r1, float r2) {
  const int ic = B.x * blockDim.x + threadIdx.x + 2;
  const int jc = B.y * blockDim.y + threadIdx.y + 2;
  const int kc = B.z + 2;
  if (ic > dc.nx - 1 || jc > dc.ny - 1) return;
  float acc = 0.f;
#pragma unroll
  for (int dk = 0; dk < 2; dk++)
#pragma unroll
    for (int dj = 0; dj < 2; dj++)
#pragma unroll
      for (int di = 0; di < 2; di++) {
        const int i = 2 * ic - 2 + di, j = 2 * jc - 2 + dj, k = 2 * kc - 2 + dk;
        const float uc = split_get(ue, uo, sp, i, j, k);
        const float xp = (i + 1 == df.nx) ? 0.f : split_get(ue, uo, sp, i + 1, j, k);
        const float xm = (i == 2) ? uc : split_get(ue, uo, sp, i - 1, j, k);
        const float yp = (j + 1 == df.ny) ? uc : split_get(ue, uo, sp, i, j + 1, k);
        const float ym = (j == 2) ? uc : split_get(ue, uo, sp, i, j - 1, k);
        const float zp = (k + 1 == df.nz) ? uc : split_get(ue, uo, sp, i, j, k + 1);
        const float zm = (k == 2) ? uc : split_get(ue, uo, sp, i, j, k - 1);
        const float *cq = cc + ix32(df, i, j, k);
        const int sy = df.nx, sz = df.nx * df.ny;
        const float c0 = cq[0];
        const float ae = face_coef(c0, cq[1], r1, r2);
        const float aw = (i == 2) ? ae : face_coef(cq[-1], c0, r1, r2);
        const float bn = face_coef(c0, cq[sy], r1, r2);
        const float bs = face_coef(cq[-sy], c0, r1, r2);
        const float ct = face_coef(c0, cq[sz], r1, r2);
        const float cb = face_coef(cq[-sz], c0, r1, r2);
        const float lap = ae * (xp - uc) + aw * (xm - uc) + bn * (yp - uc) + bs * (ym - uc) + ct * (zp - uc) +
                          cb * (zm - uc);
        acc += split_get(re, ro, sp, i, j, k) - h2i * lap;
      }
  const unsigned qc = ix32(dc, ic, jc, kc);
  rhs_c[qc] = 0.125f * acc;
  u_c[qc] = 0.f;
}

// Fine (split) u = or += the interpolated coarse correction.
// One thread per colour-split index (m, j, k): its even and odd cells are
// i = 2+2m and 3+2m in some order, both children of coarse cell m+2 along x,
// so both arrays are updated with coalesced accesses.
template <bool TRI>
__device__ __forceinline__ void b_prolong32_split(const uint3 B, const uint3 G, float *__restrict__ ue, float *__restrict__ uo, const float *__restrict__ uc,
                                  Dims df, Split sp, Dims dc, int add) {
  const int m = B.x * blockDim.x + threadIdx.x;
  const int j = B.y * blockDim.y + threadIdx.y + 2;
  const int k = B.z + 2;
  if (m >= sp.hx || j > df.ny - 1) return;
  const int pi = m + 2, pj = (j >> 1) + 1, pk = (k >> 1) + 1;
  float v0, v1;  // cells i = 2+2m and i = 3+2m
  if (TRI) {
    const int nj = tri_nb(j, pj, dc.ny), nk = tri_nb(k, pk, dc.nz);
    const float yc = tri_yz(uc, dc, pi, pj, nj, pk, nk);
    const float yl = pi == 2 ? yc : tri_yz(uc, dc, pi - 1, pj, nj, pk, nk);
    const float yr = pi + 1 == dc.nx ? 0.f : tri_yz(uc, dc, pi + 1, pj, nj, pk, nk);
    v0 = tri_x(yc, yl);
    v1 = tri_x(yc, yr);
  } else {
    v0 = v1 = uc[ix32(dc, pi, pj, pk)];
  }
  const bool odd_first = (j + k) & 1;  // cell 2+2m has odd i+j+k
  const float ve = odd_first ? v1 : v0, vo = odd_first ? v0 : v1;
  const unsigned q = at32(sp, m, j, k);
  ue[q] = add ? ue[q] + ve : ve;
  uo[q] = add ? uo[q] + vo : vo;
}

// 8-cell mean of the split fine rhs into the coarse interior (rstrct).
__device__ __forceinline__ void b_restrict32_split(const uint3 B, const uint3 G, float *__restrict__ uc, const float *__restrict__ re,
                                   const float *__restrict__ ro, Dims dc, Split sp) {
  const int ic = B.x * blockDim.x + threadIdx.x + 2;
  const int jc = B.y * blockDim.y + threadIdx.y + 2;
  const int kc = B.z + 2;
  if (ic > dc.nx - 1 || jc > dc.ny - 1) return;
  float acc = 0.f;
#pragma unroll
  for (int dk = 0; dk < 2; dk++)
#pragma unroll
    for (int dj = 0; dj < 2; dj++)
#pragma unroll
      for (int di = 0; di < 2; di++)
        acc += split_get(re, ro, sp, 2 * ic - 2 + di, 2 * jc - 2 + dj, 2 * kc - 2 + dk);
  uc[dc.ix(ic, jc, kc)] = 0.125f * acc;
}

// FP64 -> split FP32 (the fine rhs of the FMG start).
__device__ __forceinline__ void b_split_from64(const uint3 B, const uint3 G, float *__restrict__ ev, float *__restrict__ od, const double *__restrict__ src,
                               Dims d, Split sp) {
  const int i = B.x * blockDim.x + threadIdx.x + 2;
  const int j = B.y * blockDim.y + threadIdx.y + 2;
  const int k = B.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  float *dst = ((i + j + k) & 1) ? od : ev;
  dst[sp.at((i - 2) >> 1, j, k)] = (float)src[d.ix(i, j, k)];
}

// ---- coarse levels: natural layout ------------------------------------------
//
// The per-cell operations are shared by the one-launch-per-pass kernels and by
// the single-block tail kernel below, so both give the same bits.

// One red-black update of cell (i,j,k) (relax, main.f:3956-3997).
__device__ __forceinline__ void relax32_cell(float *u, const float *rhs, const float *a, const float *b,
                                             const float *c, const float *ei, Dims d, int i, int j, int k,
                                             float h2, float omega) {
  const unsigned q = ix32(d, i, j, k);
  const unsigned sy = (unsigned)d.nx, sz = (unsigned)d.nx * d.ny;
  const float uc = u[q];
  const Nb n = neighbours(u, q, i, j, k, d, uc);
  const float s = a[q] * n.xp + a[q - 1] * n.xm + b[q] * n.yp + b[q - sy] * n.ym + c[q] * n.zp + c[q - sz] * n.zm -
                  h2 * rhs[q];
  u[q] = omega * (s * ei[q]) + (1.f - omega) * uc;
}

// Coarse rhs of coarse cell (ic,jc,kc) = mean of its 8 fine residuals (resid +
// rstrct, main.f:3718-3725); the coarse correction starts at zero (main.f:3726).
__device__ __forceinline__ void resid_restrict32_cell(float *rhs_c, float *u_c, const float *u, const float *rhs,
                                                      const float *a, const float *b, const float *c, Dims df,
                                                      Dims dc, float h2i, int ic, int jc, int kc) {
  const unsigned sy = (unsigned)df.nx, sz = (unsigned)df.nx * df.ny;
  float acc = 0.f;
#pragma unroll
  for (int dk = 0; dk < 2; dk++)
#pragma unroll
    for (int dj = 0; dj < 2; dj++)
#pragma unroll
      for (int di = 0; di < 2; di++) {
        const int i = 2 * ic - 2 + di, j = 2 * jc - 2 + dj, k = 2 * kc - 2 + dk;
        const unsigned q = ix32(df, i, j, k);
        const float uc = u[q];
        const Nb n = neighbours(u, q, i, j, k, df, uc);
        const float lap = a[q] * (n.xp - uc) + a[q - 1] * (n.xm - uc) + b[q] * (n.yp - uc) +
                          b[q - sy] * (n.ym - uc) + c[q] * (n.zp - uc) + c[q - sz] * (n.zm - uc);
        acc += rhs[q] - h2i * lap;
      }
  const unsigned qc = ix32(dc, ic, jc, kc);
  rhs_c[qc] = 0.125f * acc;
  u_c[qc] = 0.f;
}

__device__ __forceinline__ void b_relax32(const uint3 B, const uint3 G, float *__restrict__ u, const float *__restrict__ rhs, const float *__restrict__ a,
                          const float *__restrict__ b, const float *__restrict__ c, const float *__restrict__ ei,
                          Dims d, float h2, float omega, int colour) {
  const int j = B.y * blockDim.y + threadIdx.y + 2;
  const int k = B.z + 2;
  if (j > d.ny - 1) return;
  const int i = 2 + ((j + k + colour) & 1) + 2 * (int)(B.x * blockDim.x + threadIdx.x);
  if (i > d.nx - 1) return;
  relax32_cell(u, rhs, a, b, c, ei, d, i, j, k, h2, omega);
}

// Coarse rhs = mean of the 8 fine residuals; coarse correction = 0 (interior;
// the FP32 kernels never read ghost values).
__device__ __forceinline__ void b_resid_restrict32(const uint3 B, const uint3 G, float *__restrict__ rhs_c, float *__restrict__ u_c, const float *__restrict__ u,
                                   const float *__restrict__ rhs, const float *__restrict__ a,
                                   const float *__restrict__ b, const float *__restrict__ c, Dims df, Dims dc,
                                   float h2i) {
  const int ic = B.x * blockDim.x + threadIdx.x + 2;
  const int jc = B.y * blockDim.y + threadIdx.y + 2;
  const int kc = B.z + 2;
  if (ic > dc.nx - 1 || jc > dc.ny - 1) return;
  resid_restrict32_cell(rhs_c, u_c, u, rhs, a, b, c, df, dc, h2i, ic, jc, kc);
}

// u = or += the interpolated coarse correction (interp / addint,
// main.f:3866-3954), interior.
template <bool TRI>
__device__ __forceinline__ void b_prolong32(const uint3 B, const uint3 G, float *__restrict__ uf, const float *__restrict__ uc, Dims df, Dims dc, int add) {
  const int i = B.x * blockDim.x + threadIdx.x + 2;
  const int j = B.y * blockDim.y + threadIdx.y + 2;
  const int k = B.z + 2;
  if (i > df.nx - 1 || j > df.ny - 1) return;
  const unsigned q = ix32(df, i, j, k);
  const float v = coarse_at<TRI>(uc, dc, i, j, k);
  uf[q] = add ? uf[q] + v : v;
}

// ---- coarse tail: every level at or below `top` in one thread block ---------
//
// On levels of a few thousand cells a launch costs more than its work.  The
// tail kernel runs the rest of a V-cycle from level `top` down to the coarsest
// grid and back (pre-sweeps, residual restriction, NTOP coarsest sweeps,
// prolongation, post-sweeps: mglin's recursion, main.f:3703-3759) inside one
// block, with a block barrier between passes in place of a launch boundary.
// The level arrays stay in L1/L2.
// Threads 0..NT-1 of the block sweep level L n times; WARP: NT = 32 and the
// passes are separated by warp barriers (levels of a few dozen cells), else
// NT = blockDim.x and block barriers.
template <bool WARP>
__device__ void tail_relax(const TailLevel &L, int n, float omega) {
  const int nt = WARP ? 32 : (int)blockDim.x;
  const Dims d = L.d;
  const int hx = (d.nx - 1) / 2;  // cells of one colour per row, rounded up
  const int ny2 = d.ny - 2;
  const int total = hx * ny2 * (d.nz - 2);
  for (int s = 0; s < n; s++)
    for (int colour = 0; colour < 2; colour++) {
      for (int t = threadIdx.x; t < total; t += nt) {
        const int m = t % hx, r = t / hx;
        const int j = 2 + r % ny2, k = 2 + r / ny2;
        const int i = 2 + ((j + k + colour) & 1) + 2 * m;
        if (i <= d.nx - 1) relax32_cell(L.u, L.rhs, L.a, L.b, L.c, L.ei, d, i, j, k, L.h2, omega);
      }
      if (WARP) __syncwarp(); else __syncthreads();
    }
}

// Residual of level F restricted into level C's rhs, C's correction zeroed.
template <bool WARP>
__device__ void tail_restrict(const TailLevel &F, const TailLevel &C) {
  const int nt = WARP ? 32 : (int)blockDim.x;
  const int cx = C.d.nx - 2, cy = C.d.ny - 2, total = cx * cy * (C.d.nz - 2);
  const float h2i = 1.0f / F.h2;
  for (int t = threadIdx.x; t < total; t += nt) {
    const int ic = 2 + t % cx, r = t / cx;
    resid_restrict32_cell(C.rhs, C.u, F.u, F.rhs, F.a, F.b, F.c, F.d, C.d, h2i, ic, 2 + r % cy, 2 + r / cy);
  }
  if (WARP) __syncwarp(); else __syncthreads();
}

// Level F's correction += injection of level C's.
template <bool WARP>
__device__ void tail_addint(const TailLevel &F, const TailLevel &C, bool tri) {
  const int nt = WARP ? 32 : (int)blockDim.x;
  const int fx = F.d.nx - 2, fy = F.d.ny - 2, total = fx * fy * (F.d.nz - 2);
  for (int t = threadIdx.x; t < total; t += nt) {
    const int i = 2 + t % fx, r = t / fx;
    const int j = 2 + r % fy, k = 2 + r / fy;
    const unsigned q = ix32(F.d, i, j, k);
    const float v = tri ? coarse_at<true>(C.u, C.d, i, j, k) : coarse_at<false>(C.u, C.d, i, j, k);
    F.u[q] = F.u[q] + v;
  }
  if (WARP) __syncwarp(); else __syncthreads();
}

// Levels with at most this many interior cells (6^3 nodes and below) run in
// warp 0 alone, at most two cells per lane and pass.
constexpr int kTailWarpCells = 64;

__device__ void tail_body(const TailArgs &A) {
  // lw: the largest level small enough for one warp (0: none)
  int lw = 0;
  for (int l = 1; l <= A.top; l++) {
    const Dims d = A.lv[l].d;
    if ((d.nx - 2) * (d.ny - 2) * (d.nz - 2) <= kTailWarpCells) lw = l;
  }
  for (int l = A.top; l > lw && l >= 2; l--) {
    tail_relax<false>(A.lv[l], A.lv[l].npre, A.omega);
    tail_restrict<false>(A.lv[l], A.lv[l - 1]);
  }
  if (lw == 0) {
    tail_relax<false>(A.lv[1], A.ntop, A.omega);
  } else if (threadIdx.x < 32) {
    for (int l = lw; l >= 2; l--) {
      tail_relax<true>(A.lv[l], A.lv[l].npre, A.omega);
      tail_restrict<true>(A.lv[l], A.lv[l - 1]);
    }
    tail_relax<true>(A.lv[1], A.ntop, A.omega);
    for (int l = 2; l <= lw; l++) {
      tail_addint<true>(A.lv[l], A.lv[l - 1], A.tri);
      tail_relax<true>(A.lv[l], A.lv[l].npost, A.omega);
    }
  }
  if (lw > 0) __syncthreads();
  for (int l = (lw > 1 ? lw : 1) + 1; l <= A.top; l++) {
    tail_addint<false>(A.lv[l], A.lv[l - 1], A.tri);
    tail_relax<false>(A.lv[l], A.lv[l].npost, A.omega);
  }
}



// 8-cell mean of a fine interior field into the coarse interior (rstrct).
__device__ __forceinline__ void b_restrict32(const uint3 B, const uint3 G, float *__restrict__ uc, const float *__restrict__ uf, Dims dc, Dims df) {
  const int ic = B.x * blockDim.x + threadIdx.x + 2;
  const int jc = B.y * blockDim.y + threadIdx.y + 2;
  const int kc = B.z + 2;
  if (ic > dc.nx - 1 || jc > dc.ny - 1) return;
  const size_t f = df.ix(2 * ic - 2, 2 * jc - 2, 2 * kc - 2);
  const size_t sy = df.sy(), sz = df.sz();
  uc[dc.ix(ic, jc, kc)] = 0.125f * (uf[f] + uf[f + 1] + uf[f + sy] + uf[f + 1 + sy] + uf[f + sz] + uf[f + 1 + sz] +
                                    uf[f + sy + sz] + uf[f + 1 + sy + sz]);
}

__device__ __forceinline__ float acf(const float *a2, Dims df, int i1, int j1, int k1, int i2, int j2, int k2,
                                     int i3, int j3, int k3, int i4, int j4, int k4) {
  return 0.25f * (a2[df.ix(i1, j1, k1)] + a2[df.ix(i2, j2, k2)] + a2[df.ix(i3, j3, k3)] + a2[df.ix(i4, j4, k4)]);
}

// acfromac in FP32 (main.f:3793-3844).
__device__ __forceinline__ void b_acfromac32(const uint3 B, const uint3 G, float *__restrict__ a, float *__restrict__ b, float *__restrict__ c,
                             float *__restrict__ ei, const float *__restrict__ a2, const float *__restrict__ b2,
                             const float *__restrict__ c2, Dims dc, Dims df) {
  const int i = B.x * blockDim.x + threadIdx.x + 1;
  const int j = B.y * blockDim.y + threadIdx.y + 1;
  const int k = B.z + 1;
  if (i > dc.nx || j > dc.ny) return;
  const bool ii = i >= 2 && i <= dc.nx - 1, ji = j >= 2 && j <= dc.ny - 1, ki = k >= 2 && k <= dc.nz - 1;
  const size_t q = dc.ix(i, j, k);
#define AA(i, j, k) acf(a2, df, 2 * (i) - 1, 2 * (j) - 1, 2 * (k) - 1, 2 * (i) - 1, 2 * (j) - 2, 2 * (k) - 1, \
                        2 * (i) - 1, 2 * (j) - 1, 2 * (k) - 2, 2 * (i) - 1, 2 * (j) - 2, 2 * (k) - 2)
#define BB(i, j, k) acf(b2, df, 2 * (i) - 1, 2 * (j) - 1, 2 * (k) - 1, 2 * (i) - 2, 2 * (j) - 1, 2 * (k) - 1, \
                        2 * (i) - 1, 2 * (j) - 1, 2 * (k) - 2, 2 * (i) - 2, 2 * (j) - 1, 2 * (k) - 2)
#define CC(i, j, k) acf(c2, df, 2 * (i) - 1, 2 * (j) - 1, 2 * (k) - 1, 2 * (i) - 2, 2 * (j) - 1, 2 * (k) - 1, \
                        2 * (i) - 1, 2 * (j) - 2, 2 * (k) - 1, 2 * (i) - 2, 2 * (j) - 2, 2 * (k) - 1)
  float va = 0.f, vb = 0.f, vc = 0.f;
  if (i <= dc.nx - 1 && ji && ki) { va = AA(i, j, k); a[q] = va; }
  if (j <= dc.ny - 1 && ii && ki) { vb = BB(i, j, k); b[q] = vb; }
  if (k <= dc.nz - 1 && ii && ji) { vc = CC(i, j, k); c[q] = vc; }
  if (ii && ji && ki) ei[q] = 1.f / (va + AA(i - 1, j, k) + vb + BB(i, j - 1, k) + vc + CC(i, j, k - 1));
#undef AA
#undef BB
#undef CC
}

// ---- FP64 defect-correction kernels ----------------------------------------
// r = rhs - L p in FP64 over the interior (resid's operator, main.f:3912-3925,
// with bc_scalar ghosts read virtually), in flux form: L p = h2i (sum of
// a_f p_f - diag p) with p_f the neighbour (the cell itself behind a Neumann
// face, 0 behind the Dirichlet one) and diag the sum of the six face
// coefficients (stored by abcei), the same operator as sum a_f (p_f - p) in
// 11 instead of 17 FP64 operations per cell.  Writes (float)r as the FP32
// fine rhs and per-block partial sums of r^2 and rhs^2.
__device__ __forceinline__ void b_defect64(const uint3 B, const uint3 G, float *__restrict__ r_ev, float *__restrict__ r_od, Split sp,
                           double *__restrict__ partials, const double *__restrict__ p,
                           const double *__restrict__ rhs, const double *__restrict__ a,
                           const double *__restrict__ b, const double *__restrict__ c,
                           const double *__restrict__ diag, Dims d, double h2i) {
  const size_t n = (size_t)(d.nx - 2) * (d.ny - 2) * (d.nz - 2);
  const size_t sy = d.sy(), sz = d.sz();
  double rr = 0.0, bb = 0.0;
  for (size_t t = (size_t)B.x * blockDim.x + threadIdx.x; t < n; t += (size_t)G.x * blockDim.x) {
    const unsigned ni = (unsigned)(d.nx - 2), nj = (unsigned)(d.ny - 2), tt = (unsigned)t;  // < 2^32 cells
    const unsigned rem = tt / ni, kk = rem / nj;
    const int i = (int)(tt - rem * ni) + 2;
    const int j = (int)(rem - kk * nj) + 2, k = (int)kk + 2;
    const size_t q = d.ix(i, j, k);
    const double uc = p[q];
    const double xp = (i + 1 == d.nx) ? 0.0 : p[q + 1];
    const double xm = (i - 1 == 1) ? uc : p[q - 1];
    const double yp = (j + 1 == d.ny) ? uc : p[q + sy];
    const double ym = (j - 1 == 1) ? uc : p[q - sy];
    const double zp = (k + 1 == d.nz) ? uc : p[q + sz];
    const double zm = (k - 1 == 1) ? uc : p[q - sz];
    const double f = rhs[q];
    double lp = a[q] * xp;
    lp = fma(a[q - 1], xm, lp);
    lp = fma(b[q], yp, lp);
    lp = fma(b[q - sy], ym, lp);
    lp = fma(c[q], zp, lp);
    lp = fma(c[q - sz], zm, lp);
    lp = fma(-diag[q], uc, lp);
    const double r = fma(-h2i, lp, f);
    (((i + j + k) & 1) ? r_od : r_ev)[sp.at((i - 2) >> 1, j, k)] = (float)r;
    rr += r * r;
    bb += f * f;
  }
  __shared__ double s0[kRedThreads], s1[kRedThreads];
  s0[threadIdx.x] = rr;
  s1[threadIdx.x] = bb;
  __syncthreads();
  for (int s = kRedThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      s0[threadIdx.x] += s0[threadIdx.x + s];
      s1[threadIdx.x] += s1[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partials[2 * B.x] = s0[0];
    partials[2 * B.x + 1] = s1[0];
  }
}

__device__ __forceinline__ void b_fold2(const uint3 B, const uint3 G, const double *__restrict__ partials, double *__restrict__ out) {
  __shared__ double s0[kRedThreads], s1[kRedThreads];
  double a0 = 0.0, a1 = 0.0;
  for (int b = threadIdx.x; b < kRedBlocks; b += kRedThreads) {
    a0 += partials[2 * b];
    a1 += partials[2 * b + 1];
  }
  s0[threadIdx.x] = a0;
  s1[threadIdx.x] = a1;
  __syncthreads();
  for (int s = kRedThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      s0[threadIdx.x] += s0[threadIdx.x + s];
      s1[threadIdx.x] += s1[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = s0[0];
    out[1] = s1[0];
  }
}

// p += e (FP64 accumulation of the split FP32 correction), interior; `init`
// sets p = e.
__device__ __forceinline__ void b_correct64(const uint3 B, const uint3 G, double *__restrict__ p, const float *__restrict__ ev, const float *__restrict__ od,
                            Dims d, Split sp, int init) {
  const int i = B.x * blockDim.x + threadIdx.x + 2;
  const int j = B.y * blockDim.y + threadIdx.y + 2;
  const int k = B.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const unsigned q = ix32(d, i, j, k);
  const double e = (double)split_get(ev, od, sp, i, j, k);
  p[q] = init ? e : p[q] + e;
}

// Coarse FP32 coefficients (acfromac) straight from the FP64 fine ones.
__device__ __forceinline__ void b_to32(const uint3 B, const uint3 G, float *__restrict__ dst, const double *__restrict__ src, size_t n) {
  for (size_t q = (size_t)B.x * blockDim.x + threadIdx.x; q < n; q += (size_t)G.x * blockDim.x)
    dst[q] = (float)src[q];
}

__device__ __forceinline__ void b_acfromac64to32(const uint3 B, const uint3 G, float *__restrict__ a, float *__restrict__ b, float *__restrict__ c,
                                 float *__restrict__ ei, const double *__restrict__ a2,
                                 const double *__restrict__ b2, const double *__restrict__ c2, Dims dc, Dims df) {
  const int i = B.x * blockDim.x + threadIdx.x + 1;
  const int j = B.y * blockDim.y + threadIdx.y + 1;
  const int k = B.z + 1;
  if (i > dc.nx || j > dc.ny) return;
  const bool ii = i >= 2 && i <= dc.nx - 1, ji = j >= 2 && j <= dc.ny - 1, ki = k >= 2 && k <= dc.nz - 1;
  const size_t q = dc.ix(i, j, k);
#define FA(i, j, k) (0.25 * (a2[df.ix(2 * (i) - 1, 2 * (j) - 1, 2 * (k) - 1)] + a2[df.ix(2 * (i) - 1, 2 * (j) - 2, 2 * (k) - 1)] + \
                             a2[df.ix(2 * (i) - 1, 2 * (j) - 1, 2 * (k) - 2)] + a2[df.ix(2 * (i) - 1, 2 * (j) - 2, 2 * (k) - 2)]))
#define FB(i, j, k) (0.25 * (b2[df.ix(2 * (i) - 1, 2 * (j) - 1, 2 * (k) - 1)] + b2[df.ix(2 * (i) - 2, 2 * (j) - 1, 2 * (k) - 1)] + \
                             b2[df.ix(2 * (i) - 1, 2 * (j) - 1, 2 * (k) - 2)] + b2[df.ix(2 * (i) - 2, 2 * (j) - 1, 2 * (k) - 2)]))
#define FC(i, j, k) (0.25 * (c2[df.ix(2 * (i) - 1, 2 * (j) - 1, 2 * (k) - 1)] + c2[df.ix(2 * (i) - 2, 2 * (j) - 1, 2 * (k) - 1)] + \
                             c2[df.ix(2 * (i) - 1, 2 * (j) - 2, 2 * (k) - 1)] + c2[df.ix(2 * (i) - 2, 2 * (j) - 2, 2 * (k) - 1)]))
  double va = 0.0, vb = 0.0, vc = 0.0;
  if (i <= dc.nx - 1 && ji && ki) { va = FA(i, j, k); a[q] = (float)va; }
  if (j <= dc.ny - 1 && ii && ki) { vb = FB(i, j, k); b[q] = (float)vb; }
  if (k <= dc.nz - 1 && ii && ji) { vc = FC(i, j, k); c[q] = (float)vc; }
  if (ii && ji && ki) ei[q] = (float)(1.0 / (va + FA(i - 1, j, k) + vb + FB(i, j - 1, k) + vc + FC(i, j, k - 1)));
#undef FA
#undef FB
#undef FC
}


}  // namespace
}  // namespace mg32
}  // namespace dsg
