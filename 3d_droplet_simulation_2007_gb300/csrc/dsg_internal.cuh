// dsg_internal.cuh -- shared device helpers, launch helpers and the context
// structure of the GB300 projection hot path.  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <atomic>
#include <string>
#include <vector>

#include "../../include/dsg.h"

namespace dsg {

// Every kernel launch of the library goes through DSG_COUNT so that the
// number of launches in a timed region can be reported.
// The per-thread count lets a graph capture count its own kernel nodes while
// other host threads (ensemble workers) launch concurrently.
extern std::atomic<long long> g_launches;
extern thread_local long long t_launches;
inline void count_launch() {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  t_launches++;
}
#define DSG_COUNT dsg::count_launch(),

// Column-major, 1-based (i,j,k) -> linear offset of an (nx,ny,nz) array.
struct Dims {
  int nx, ny, nz;
  __host__ __device__ __forceinline__ size_t ix(int i, int j, int k) const {
    return (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1));
  }
  __host__ __device__ __forceinline__ size_t count() const { return (size_t)nx * ny * nz; }
  __host__ __device__ __forceinline__ int sx() const { return 1; }
  __host__ __device__ __forceinline__ int sy() const { return nx; }
  __host__ __device__ __forceinline__ size_t sz() const { return (size_t)nx * ny; }
};

// Bit-pattern tests of doubles on the integer pipe.  GB300's FP64 comparisons
// issue on the FP64 pipe (as slow as its FMAs), and the exact fast paths test
// up to 27 values per cell.  same_bits differs from == only for +0/-0 and
// NaN: a -0 then takes the general path, which computes exactly what the
// reference computes.
__device__ __forceinline__ bool same_bits(double a, double b) {
  return __double_as_longlong(a) == __double_as_longlong(b);
}
__device__ __forceinline__ bool is_zero_bits(double a) { return __double_as_longlong(a) == 0LL; }
__device__ __forceinline__ bool is_one_bits(double a) { return __double_as_longlong(a) == 0x3FF0000000000000LL; }
// a > 0 for a finite double (positive bit patterns order like the values)
__device__ __forceinline__ bool positive_bits(double a) { return __double_as_longlong(a) > 0LL; }

__device__ __forceinline__ double dmax1(double a, double b) { return a >= b ? a : b; }
__device__ __forceinline__ double dmin1(double a, double b) { return a <= b ? a : b; }

// Grid over the interior (2..n-1)^3 with 32 x 4 thread blocks, one z plane per
// grid row in z.
inline dim3 interior_grid(const Dims &d, dim3 blk) {
  return dim3((unsigned)((d.nx - 2 + blk.x - 1) / blk.x), (unsigned)((d.ny - 2 + blk.y - 1) / blk.y),
              (unsigned)(d.nz - 2));
}

// Number of multigrid levels.  For min(nx,ny,nz) = 2^k+2 it is memoryaloc's
// count (main.f:284-298), halving until the smallest interior extent is 2.
// Other sides, which the reference refuses (main.f:296-297), coarsen while every
// interior extent is even and the smallest is at least 4 (48, 96 and 160 cells
// per side end at 3, 3 and 5 coarsest cells).  0 below 2 interior cells.
inline int level_count(int nx, int ny, int nz) {
  int mx = nx - 2, my = ny - 2, mz = nz - 2;
  if (mx < 2 || my < 2 || mz < 2) return 0;
  int ng = 1;
  for (;;) {
    int m = mx < my ? mx : my;
    m = mz < m ? mz : m;
    if (m < 4 || (mx & 1) || (my & 1) || (mz & 1) || ng >= 31) break;
    mx /= 2;
    my /= 2;
    mz /= 2;
    ng++;
  }
  return ng;
}

// Number of blocks of the deterministic reductions (fixed so that results do
// not depend on the device).
constexpr int kRedBlocks = 1216;  // 8 x 152 SMs
constexpr int kRedThreads = 256;

// ---- host-side launch helpers (implemented in the kernel .cu files) -------
// All return cudaGetLastError() of the launches.
cudaError_t bc_scalar(double *s, Dims d, cudaStream_t st);
cudaError_t bc_resid(double *s, Dims d, cudaStream_t st);
cudaError_t bc_out(double *s, Dims d, cudaStream_t st);
cudaError_t relax(double *u, double lengthsize, const double *rhs, const double *a, const double *b,
                  const double *c, const double *ei, Dims d, double omega, cudaStream_t st);
// fma = true: the fused multiply-add form of the FP64 sweep and residual
// (fewer FP64 operations, results within ulps of the reference order);
// fma = false: the reference's operation order, bit-identical to the oracle.
cudaError_t relax_n(int n, double *u, double lengthsize, const double *rhs, const double *a,
                    const double *b, const double *c, const double *ei, Dims d, double omega,
                    cudaStream_t st, bool fma = false);
cudaError_t resid(double lengthsize, double *res, const double *u, const double *rhs, const double *a,
                  const double *b, const double *c, Dims d, cudaStream_t st, bool fma = false);
cudaError_t rstrct(double *uc, const double *uf, Dims dc, cudaStream_t st);
cudaError_t interp(double *uf, const double *uc, Dims df, cudaStream_t st);
cudaError_t addint(double *uf, const double *uc, double *res, Dims df, cudaStream_t st);
cudaError_t acfromac(double *a, double *b, double *c, double *ei, const double *a2, const double *b2,
                     const double *c2, Dims dc, cudaStream_t st);
cudaError_t abcei(double *a, double *b, double *c, double *ei, const double *cc, double r1, double r2,
                  Dims d, cudaStream_t st, double *diag = nullptr);
// diag = the sum of the six face coefficients of every interior cell
cudaError_t diag_sum(double *diag, const double *a, const double *b, const double *c, Dims d, cudaStream_t st);
cudaError_t filterc27(const double *cc, double *cf, Dims d, cudaStream_t st);
// relres partial sums: out[0] = sum r^2, out[1] = sum rhs^2 (device, 2 doubles)
cudaError_t relres_sums(double *out, double *partials, double lengthsize, const double *u,
                        const double *rhs, const double *a, const double *b, const double *c, Dims d,
                        cudaStream_t st, bool fma = false);
// out[0] = interior sum of f (SUMFIELD order-independent tree sum)
cudaError_t sumfield(double *out, double *partials, const double *f, Dims d, cudaStream_t st);
// out[0] = max |f| over the interior
cudaError_t absmax3(double *out, double *partials, const double *f0, const double *f1,
                    const double *f2, Dims d, cudaStream_t st);
// out[0] = max |div u| * hi2 over the interior (FMODMAX of the divergence)
cudaError_t divmax(double *out, double *partials, const double *u, const double *v, const double *w,
                   double hi2, Dims d, cudaStream_t st);
cudaError_t fill_zero(double *f, size_t n, cudaStream_t st);

// vof.cu
cudaError_t bc_c(double *cc, Dims d, cudaStream_t st);
// list/count: scratch of the interface-cell list (>= interior cells) and its length
cudaError_t swp(const double *us, double *cc, double *vof1, double *vof2, double *vof3, int dir, Dims d,
                double tauh, unsigned *list, unsigned *count, cudaStream_t st);
cudaError_t calcrho(double *rhon, double *mun, const double *cc, Dims d, double rho1, double rho2,
                    double mu1, double mu2, cudaStream_t st);
// csf.cu (S = {S11,S22,S33,S12,S13,S23})
// The S12/S13/S23 writes of bc_tensor alone (constant faces), for an upload of
// those fields that lands after csf.
// Both on planes k0 .. k1-1 (x and y faces of the interior planes among them,
// the z planes 1, 2, nz in the range); the defaults cover every plane.
cudaError_t bc_tensor_offdiag(double *s12, double *s13, double *s23, Dims d, cudaStream_t st, int k0 = 1,
                              int k1 = 1 << 30);
cudaError_t bc_tensor(double *const S[6], Dims d, cudaStream_t st, int k0 = 1, int k1 = 1 << 30);
cudaError_t csf(const double *ccc, double *w11, double *w22, double *w33, double *ccf, double *const S[6],
                Dims d, double tau, double sigma, double h, cudaStream_t st, bool scratch = true);
// momentum.cu
cudaError_t bc_v(double *u, double *v, double *w, double *partials, Dims d, double xvel2, cudaStream_t st);
cudaError_t bc_w(double *w1, double *w2, double *w3, const double *u, const double *v, const double *w,
                 double *partials, Dims d, cudaStream_t st);
// stress and predictor on the interior planes k0 .. k1-1 (k1 = 0: up to nz-1)
cudaError_t stress(double *const S[6], const double *u, const double *v, const double *w, const double *cc,
                   Dims d, double r1, double r2, double r10, double r20, cudaStream_t st, int k0 = 2, int k1 = 0);
cudaError_t predictor(double *w1, double *w2, double *w3, const double *u, const double *v, const double *w,
                      const double *a, const double *b, const double *c, double *const S[6], Dims d,
                      double horgrav, double stdgrav, cudaStream_t st, int k0 = 2, int k1 = 0);
cudaError_t convective(double *u, double *v, double *w, const double *w1, const double *w2, const double *w3,
                       Dims d, double tauh, int convectype, cudaStream_t st);
cudaError_t divergence(double *out, const double *u, const double *v, const double *w, Dims d, double hi2,
                       cudaStream_t st);
cudaError_t project(double *u, double *v, double *w, const double *p, const double *a, const double *b,
                    const double *c, Dims d, cudaStream_t st);
// sgip.cu (interface heights and the SGIP force, surfacet = 5)
cudaError_t calch3d(double *const H[6], const double *cc, Dims d, unsigned long long *err, cudaStream_t st);
cudaError_t sgip(const double *ccc, double *w11, double *w22, double *w33, double *ccf, double *const S[6],
                 double *const H[6], const double *u, const double *w, Dims d, double tau, double sigma, double h,
                 cudaStream_t st);
cudaError_t sgip2(const double *ccc, double *w11, double *w22, double *w33, double *ccf, double *const S[6],
                  double *const H[6], Dims d, double tau, double sigma, double h, cudaStream_t st);
// turb.cu (k-epsilon, iturb = 3)
cudaError_t keps_seed(double *ktur, double *eps, double *mut, const double *cc, const double *rhon,
                      const double *mun, Dims d, double k1, double k2, cudaStream_t st);
cudaError_t kepsmodel(double *ktur, double *eps, double *mut, double *kn, double *en, const double *mun,
                      const double *rhon, const double *u, const double *v, const double *w, Dims d, double h,
                      double tau, cudaStream_t st);
cudaError_t fturbdif(double *cc, const double *mut, const double *rhon, Dims d, int tauh2, cudaStream_t st);
// mg32.cu (mixed precision)
cudaError_t relax32_n(int n, float *u, float h2, const float *rhs, const float *a, const float *b, const float *c,
                      const float *ei, Dims d, float omega, cudaStream_t st);
cudaError_t resid_restrict32(float *rhs_c, float *u_c, const float *u, const float *rhs, const float *a,
                             const float *b, const float *c, Dims df, float h2i, cudaStream_t st);
// fine u = (add = 0) or += (add = 1) the coarse correction, trilinear (tri) or injected
cudaError_t prolong32(float *uf, const float *uc, Dims df, int add, int tri, cudaStream_t st);
cudaError_t restrict32(float *uc, const float *uf, Dims dc, cudaStream_t st);
cudaError_t acfromac32(float *a, float *b, float *c, float *ei, const float *a2, const float *b2, const float *c2,
                       Dims dc, cudaStream_t st);
cudaError_t acfromac64to32(float *a, float *b, float *c, float *ei, const double *a2, const double *b2,
                           const double *c2, Dims dc, cudaStream_t st);
// coarse tail: levels top..1 of one V-cycle in one thread block
constexpr int kTailThreads = 1024;
constexpr int kTailMaxLevels = 12;
struct TailLevel {
  float *u, *rhs;
  const float *a, *b, *c, *ei;
  Dims d;
  float h2;
  int npre, npost;  // sweeps on this level
};
struct TailArgs {
  TailLevel lv[kTailMaxLevels + 1];  // 1..top
  int top, ntop;
  float omega;
  int tri;  // trilinear prolongation (else injection)
};
cudaError_t vtail32(const TailArgs &args, cudaStream_t st);
// finest level in colour-split storage ({even, odd} arrays of (nx-2)/2 x (ny-2) x (nz-2))
cudaError_t relax32_split_n(int n, float *const u[2], float *const rhs[2], const float *cc, Dims d, float h2,
                            float omega, float r1, float r2, cudaStream_t st);
cudaError_t resid_restrict32_split(float *rhs_c, float *u_c, float *const u[2], float *const rhs[2], const float *cc,
                                   Dims df, float h2i, float r1, float r2, cudaStream_t st);
cudaError_t prolong32_split(float *const u[2], const float *uc, Dims df, int add, int tri, cudaStream_t st);
cudaError_t restrict32_split(float *uc, float *const rhs[2], Dims dc, cudaStream_t st);
cudaError_t split_from64(float *const dst[2], const double *src, Dims d, cudaStream_t st);
cudaError_t defect64(float *const r32[2], double *out2, double *partials, const double *p, const double *rhs,
                     const double *a, const double *b, const double *c, const double *diag, Dims d,
                     double lengthsize, cudaStream_t st);
cudaError_t correct64(double *p, float *const e[2], Dims d, int init, cudaStream_t st);
cudaError_t to32(float *dst, const double *src, size_t n, cudaStream_t st);
// One GCR iteration of the mixed solve on the finest level, after the V-cycle
// that left z = M r in the split correction arrays: w = A z, the step
// lengths, then (not last) d, q, r and p updated, or (last) p += alpha d.
struct GcrBufs {
  float *w[2], *d[2], *q[2];  // colour-split pairs
  double *p1, *p2, *coef;     // block sums of the apply (4 per block) and update (2), step lengths
};
cudaError_t gcr_step(int first, int last, const GcrBufs &g, double *p, float *const z[2], float *const r[2],
                     const float *cc, Dims d, float h2i, float r1, float r2, cudaStream_t st);
// init.cu
cudaError_t init_drop(double *cc, double *u, double *v, double *w, Dims d, double h, double x0, double y0,
                      double z0, double radius, double yvel1, double yvel2, double zvel1, double zvel2,
                      double noise_amp, uint64_t seed, cudaStream_t st);

}  // namespace dsg

struct dsg_net;
namespace dsg {
namespace nn {
// nn.cu: the network at the start of a pressure solve.  net_features: input
// channels from the start pressure p (the FP32 full-multigrid guess), its
// defect (r32: the FP32 colour-split copy the defect pass leaves; red = {sum
// r^2, sum rhs^2} in FP64), cc, rhs and the previous pressure; keeps p as the
// base of the training target.  net_correction: forward pass
// and the minimal-residual step along the network's correction e of p: the
// best alpha and the relative defect of p + alpha e (synchronises the
// stream).  net_apply: p += alpha e.  net_target: after the solve, the
// training pair (p_solved - p_start, in the network's units).
int net_features(dsg_net *n, const double *cc, const double *rhs, const double *p, const double *pprev,
                 const float *const r32[2], const double *red, Dims d, double lengthsize, cudaStream_t st);
int net_correction(dsg_net *n, const double *a, const double *b, const double *c, Dims d, double *relres_pred,
                   double *alpha, cudaStream_t st);
int net_apply(dsg_net *n, double *p, double alpha, Dims d, cudaStream_t st);
int net_target(dsg_net *n, const double *p, Dims d, cudaStream_t st);
void net_begin_solve(dsg_net *n);
}  // namespace nn
}  // namespace dsg

struct dsg_ctx;
namespace dsg {
// dsg.cu: the surface-tension phase (dsg_csf with scratch = true)
int csf_phase(dsg_ctx *ctx, bool scratch);
}  // namespace dsg

// ---- context ---------------------------------------------------------------
// A captured CUDA graph of the mixed-mode pressure solve and the finest-level
// relax event pairs recorded inside it (read back after each replay).
struct GraphRec {
  cudaGraphExec_t exec = nullptr;
  int key[6] = {-1, -1, -1, -1, -1, -1};  // npre, npost, ntop, cycles, inner, profiling
  std::vector<cudaEvent_t> ev;             // start/end event pairs of finest-level relax calls
  std::vector<int> ev_n;                   // relax calls timed by each pair
  long long kernels = 0;                   // kernel nodes in the graph (counted per replay)
};

struct dsg_ctx {
  dsg_config cfg;
  dsg_scalars s;
  int nx, ny, nz, ng;
  int device = 0;             // CUDA device the context was created on
  int tail_top = 0;           // FP32 levels 1..tail_top run in the single-block tail kernel (0: none)
  int lnx[32], lny[32], lnz[32];
  double *lv[32][8];          // [level][CC,P,RES,RHS,A,B,C,EI], level 1..ng
  float *lv32[32][6];         // FP32 hierarchy [level][U,RHS,A,B,C,EI] of the mixed mode;
                              // on the finest level U and RHS are colour-split (even half, odd
                              // half) and A holds cc in FP32
  double *f[DSG_NFIELDS];     // fine fields; 0..7 alias lv[ng]
  double *ccf;                // csf filtered volume fraction (local array of csf)
  double *diag64;             // sum of the six fine face coefficients (the mixed solve's defect)
  bool diag_fresh = false;    // diag64 was formed from the current coefficients (this step's abcei)
  // The mixed solve's FP32 coefficient hierarchy, launched on `side` right
  // after this step's abcei so that it overlaps the rest of the momentum
  // phase; coef_ev marks its end, and the solve waits for it instead of
  // forming the hierarchy itself.
  cudaStream_t side = nullptr;
  cudaEvent_t side_start = nullptr, coef_ev = nullptr;
  bool coef32_async = false;
  double *red_partials;       // reduction partials (kRedBlocks * 4 doubles)
  double *gcr_partials;       // GCR block sums of the mixed solve (kRedBlocks * 6 doubles)
  double *gcr_coef;           // GCR step lengths and sums (16 doubles)
  double *red_out;            // device reduction results (8 doubles)
  double *red_host;           // pinned host mirror of red_out
  unsigned long long *stop_flag;  // device: first cell where CalcH3d would STOP (code << 48 | index)
  unsigned *iface_count;          // device: length of the VOF sweep's interface-cell list (held in ccf)
  void *arena;
  size_t arena_bytes;
  cudaStream_t stream;
  cudaStream_t own_stream;
  std::string err;
  // live profile of the finest-level relaxation (CUDA events on ctx->stream)
  bool prof = false;
  long long prof_launch0 = 0;
  std::vector<cudaEvent_t> prof_ev;
  size_t prof_used = 0;
  long long prof_relax_calls = 0;
  double prof_relax_bytes = 0.0;
  int prof_relax_bits = 64;
  double prof_graph_relax_ms = 0.0;   // relax time read back from graph replays
  static constexpr int kMaxInner = 8;  // FP32 V-cycles of one outer iteration, at most
  GraphRec g_first;                    // FP32 FMG start + first defect
  GraphRec g_iter[kMaxInner + 1];      // one outer iteration of k V-cycles + defect, per k
  double rho_est = 0.3;                // measured residual reduction per FP32 V-cycle
  GraphRec *cap = nullptr;            // graph under capture
  dsg_net *net = nullptr;             // learned initial guess (DSG_MODE_LEARNED)
  int net_record = 0;                 // store a training pair after every solve
  double last_relres_base = -1.0;     // learned mode: relres of the FP32 full-multigrid start
  double last_relres_net = -1.0;      // learned mode: predicted relres of the corrected start
  int net_rest = 0;                   // learned mode: solves left without the network
  int net_backoff = 1;                // learned mode: rest after the next rejection (1, 2, 4 .. 32)
  std::vector<cudaEvent_t> phase_ev;  // phase markers of dsg_step (event pool)
  std::vector<int> phase_id;          // phase that starts at each marker, -1 = end
  size_t phase_used = 0;
  // snapshot (io.cu): p, u, v, w, cc staged in HBM, copied to pinned host memory
  static constexpr int kSnapFields = 5;
  double *snap_dev = nullptr;
  double *snap_host = nullptr;
  cudaStream_t snap_stream = nullptr;
  cudaEvent_t snap_ready = nullptr, snap_done = nullptr;
  bool snap_pending = false;
  int snap_t = -1;
  // host-buffer step (dsg_step_host): upload and download streams, one
  // event per sync point for each (created on first use), and the hook the
  // step calls at its sync points while a host-buffer step runs
  static constexpr int kSyncPoints = 8;
  cudaStream_t xfer_in = nullptr, xfer_out = nullptr;
  cudaEvent_t xfer_in_ev[kSyncPoints] = {};
  cudaEvent_t xfer_out_ev[kSyncPoints] = {};
  cudaEvent_t xfer_start = nullptr;
  // off-diagonal stresses arriving after csf come in kSChunks ranges of
  // planes (chunk c: planes s_chunk_k[c] .. s_chunk_k[c+1]-1, its copies
  // complete at s_chunk_ev[c]); the momentum phase then works through them
  // chunk by chunk.  s_chunks = 0: not in a host-buffer step, or not late.
  static constexpr int kSChunks = 4;
  cudaEvent_t s_chunk_ev[kSChunks] = {};
  int s_chunk_k[kSChunks + 1] = {};
  int s_chunks = 0;
  int (*sync_hook)(dsg_ctx *ctx, int point, void *arg) = nullptr;
  void *sync_arg = nullptr;
  dsg::Dims fine() const { return dsg::Dims{nx, ny, nz}; }
  dsg::Dims level(int l) const { return dsg::Dims{lnx[l], lny[l], lnz[l]}; }
};

namespace dsg {
// ---- settings of the mixed-precision solve, shared by the standalone solve
// (dsg.cu) and the batched ensemble solve (batch.cu) ----------------------
namespace mixed {
enum { U32 = 0, RHS32 = 1, A32 = 2, B32 = 3, C32 = 4, EI32 = 5 };

// Relaxation factor of the FP32 V-cycle (a preconditioner of the FP64 defect
// correction, so free to differ from the reference's OMEGA).
inline float omega32(const dsg_ctx *ctx) {
  return (float)(ctx->cfg.mg32_omega > 0.0 ? ctx->cfg.mg32_omega : ctx->cfg.omega);
}

// Sweeps of the FP32 V-cycle: the reference's (adaptive) NPRE/NPOST unless
// the configuration fixes them.
inline int pre32(const dsg_ctx *ctx) { return ctx->cfg.mg32_npre > 0 ? ctx->cfg.mg32_npre : ctx->s.npre; }
inline int post32(const dsg_ctx *ctx) { return ctx->cfg.mg32_npost > 0 ? ctx->cfg.mg32_npost : ctx->s.npost; }

// Levels of at most this many nodes may have their own sweep counts
// (mg32_small_npre/npost): the levels the coarse tail runs by default.
constexpr long long kSmallLevelNodes = 18LL * 18 * 18;

inline bool small_level(const dsg_ctx *ctx, int l) {
  return (long long)ctx->lnx[l] * ctx->lny[l] * ctx->lnz[l] <= kSmallLevelNodes;
}

// Sweeps on level l: the finest level, the one below it and the small levels
// may have their own counts (a sweep on the finest level costs 8x and on the
// next 2-3x one of the smaller levels, which are bound by launch latency or,
// inside the coarse tail, by one SM's issue rate).
inline int pre32(const dsg_ctx *ctx, int l) {
  if (l == ctx->ng && ctx->cfg.mg32_fine_npre > 0) return ctx->cfg.mg32_fine_npre;
  if (l == ctx->ng - 1 && ctx->cfg.mg32_mid_npre > 0) return ctx->cfg.mg32_mid_npre;
  if (l < ctx->ng && small_level(ctx, l) && ctx->cfg.mg32_small_npre > 0) return ctx->cfg.mg32_small_npre;
  return pre32(ctx);
}
inline int post32(const dsg_ctx *ctx, int l) {
  if (l == ctx->ng && ctx->cfg.mg32_fine_npost > 0) return ctx->cfg.mg32_fine_npost;
  if (l == ctx->ng - 1 && ctx->cfg.mg32_mid_npost > 0) return ctx->cfg.mg32_mid_npost;
  if (l < ctx->ng && small_level(ctx, l) && ctx->cfg.mg32_small_npost > 0) return ctx->cfg.mg32_small_npost;
  return post32(ctx);
}

// Prolongation of the FP32 V-cycles and FMG start: trilinear unless the
// configuration asks for the reference's injection.
// V-cycles of the FP32 FMG start at level l (its own count on the finest
// level when mg32_fmg_fine_cycles > 0).
inline int fmg32_cycles(const dsg_ctx *ctx, int l) {
  if (l == ctx->ng && ctx->cfg.mg32_fmg_fine_cycles > 0) return ctx->cfg.mg32_fmg_fine_cycles;
  return ctx->cfg.mg32_fmg_cycles > 0 ? ctx->cfg.mg32_fmg_cycles : ctx->cfg.cycles;
}

inline int tri32(const dsg_ctx *ctx) { return ctx->cfg.mg32_prolong == 1 ? 0 : 1; }

inline float level_h2(dsg_ctx *ctx, int l) {
  const double h1 = ctx->s.lengthsize / (ctx->lnx[l] - 2);
  return (float)(h1 * h1);
}

// Finest-level colour-split FP32 arrays: {even, odd} halves of U and RHS.
struct FineSplit {
  float *u[2];
  float *r[2];
};

inline FineSplit fine_split(dsg_ctx *ctx) {
  float **L = ctx->lv32[ctx->ng];
  const dsg::Dims d = ctx->fine();
  const size_t half = (size_t)((d.nx - 2) >> 1) * (d.ny - 2) * (d.nz - 2);
  return FineSplit{{L[U32], L[U32] + half}, {L[RHS32], L[RHS32] + half}};
}

inline size_t fine_split_bytes(dsg_ctx *ctx) {
  const dsg::Dims d = ctx->fine();
  return 2 * (size_t)((d.nx - 2) >> 1) * (d.ny - 2) * (d.nz - 2) * sizeof(float);
}

inline void phase_coefs(dsg_ctx *ctx, float *r1, float *r2) {
  *r1 = (float)(0.5 * (ctx->s.rho1 - ctx->s.rho2));
  *r2 = (float)ctx->s.rho2;
}

// Arguments of the coarse-tail kernel for FP32 levels 1..top of ctx.
inline void tail_args(dsg_ctx *ctx, int top, dsg::TailArgs *A) {
  memset(A, 0, sizeof *A);
  for (int l = 1; l <= top; l++) {
    float **L = ctx->lv32[l];
    A->lv[l] = TailLevel{L[U32],       L[RHS32],          L[A32],     L[B32],         L[C32],
                              L[EI32],      ctx->level(l),     level_h2(ctx, l), pre32(ctx, l), post32(ctx, l)};
  }
  A->top = top;
  A->ntop = ctx->s.ntop;
  A->omega = omega32(ctx);
  A->tri = tri32(ctx);
}

}  // namespace mixed

int set_error(dsg_ctx *ctx, int code, const char *fmt, ...);
int cuda_fail(dsg_ctx *ctx, cudaError_t e, const char *where);
// A time step in two halves around its pressure solve (dsg.cu), and the
// bookkeeping after a mixed-precision solve; the batched ensemble solve
// (batch.cu) runs between the halves for all members at once.
int step_pre_solve(dsg_ctx *ctx, int t);
int step_post_solve(dsg_ctx *ctx, int t, dsg_mg_stats *ms, int mg_rc, dsg_mg_stats *stats);
int solvelpres_pre(dsg_ctx *ctx);
int solvelpres_post(dsg_ctx *ctx, int t, dsg_mg_stats *ms, int mg_rc, dsg_mg_stats *stats);
int mixed_finish(dsg_ctx *ctx, dsg_mg_stats *s, dsg_mg_stats *stats);
// batch.cu: the batched mixed-precision solve of ensemble members
struct BatchSolve;
int batch_eligible(const dsg_ctx *c, char *why, size_t nwhy);
BatchSolve *batch_create(const std::vector<dsg_ctx *> &members, int *rc);
void batch_destroy(BatchSolve *b);
int batch_solve(BatchSolve *b, const std::vector<int> &active, std::vector<dsg_mg_stats> &stats,
                std::vector<int> &mg_rc);
int batch_autotune(BatchSolve *b, int reps, int *slots_tuned);
long long batch_tail_nodes(const BatchSolve *b);
// boundary conditions and derived fields after the state was loaded (the
// restart branch of initialize, main.f:174-177), k-epsilon seeding included
int restart_state(dsg_ctx *ctx);
void snapshot_release(dsg_ctx *ctx);
}  // namespace dsg

#define DSG_CK(ctx, expr)                                   \
  do {                                                      \
    cudaError_t _e = (expr);                                \
    if (_e != cudaSuccess) return dsg::cuda_fail((ctx), _e, #expr); \
  } while (0)
