// dsg.cu -- context, device arena and host orchestration of the time step:
// readinput/memoryaloc/nondim (main.f:185-446), the main.f:19-73 loop body,
// solvelpres (main.f:3236-3439) and the FMG driver mglin (main.f:3645-3763).
// Everything runs on one CUDA stream; the only host reads inside a step are the
// CFL maximum of checktime, the residual norm of the tol modes (once per
// V-cycle) and the divergence maximum of the relaxation-count adaptivity
// (every 10 steps).
#include <math.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "dsg_internal.cuh"

// Message of the last failure without a context, per host thread (ensemble
// workers report concurrently).
static thread_local std::string g_last_error;

namespace dsg {

std::atomic<long long> g_launches{0};
thread_local long long t_launches = 0;

int set_error(dsg_ctx *ctx, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (ctx) ctx->err = buf;
  g_last_error = buf;
  return code;
}

int cuda_fail(dsg_ctx *ctx, cudaError_t e, const char *where) {
  return set_error(ctx, e == cudaErrorMemoryAllocation ? DSG_E_NOMEM : DSG_E_CUDA, "CUDA error %d (%s) at %s",
                   (int)e, cudaGetErrorString(e), where);
}

}  // namespace dsg

using dsg::Dims;

namespace {

// nondim, main.f:341-446 (drop case).  Host arithmetic keeps the reference's
// operation order; this translation unit is built without FP contraction.
void nondim(dsg_ctx *ctx) {
  const dsg_config &in = ctx->cfg;
  dsg_scalars &s = ctx->s;
  s.lengthscale = in.length_si;
  const double dx = in.xvel1_si - in.xvel2_si, dy = in.yvel1_si - in.yvel2_si, dz = in.zvel1_si - in.zvel2_si;
  double vscale = sqrt(dx * dx + dy * dy + dz * dz);
  if (vscale == 0.0) vscale = 1.0;
  s.vscale = vscale;
  const double timescale = s.lengthscale / vscale;
  s.lengthsize = in.length_si / s.lengthscale;
  s.h = s.lengthsize / (ctx->nx - 2);
  s.time = 0.0;
  const double tau_si = in.maxcfl * (double)0.8f * (in.length_si / (ctx->nx - 2)) / vscale;
  s.tau = tau_si / timescale;
  s.tauh = s.tau / s.h;
  s.tauh2 = (int)(s.tau / (s.h * s.h));
  s.tswap = 0;
  s.radius = in.radius_si / s.lengthscale;
  s.xvel1 = in.xvel1_si / vscale;
  s.yvel1 = in.yvel1_si / vscale;
  s.zvel1 = in.zvel1_si / vscale;
  s.xvel2 = in.xvel2_si / vscale;
  s.yvel2 = in.yvel2_si / vscale;
  s.zvel2 = in.zvel2_si / vscale;
  s.y0 = (ctx->ny - 2) * s.h / 2;
  s.z0 = (ctx->nz - 2) * s.h / 2;
  s.rho1 = 1.0;
  s.rho2 = in.rho2_si / in.rho1_si;
  const double L = s.lengthscale;
  double denom = in.rho1_si * (L * L) / timescale;
  s.mu1 = in.visc1_si / denom;
  s.mu2 = in.visc2_si / denom;
  denom = in.rho1_si * (L * L * L) / (timescale * timescale);
  s.sigma = in.sigma_si / denom;
  denom = L / (timescale * timescale);
  s.g = in.grav_si / denom;
  s.g1 = in.grav1_si / denom;
}

inline double *S6(dsg_ctx *c, int m) { return c->f[DSG_F_S11 + m]; }

struct Tensor {
  double *p[6];
  explicit Tensor(dsg_ctx *c) {
    for (int m = 0; m < 6; m++) p[m] = S6(c, m);
  }
};

int read_device(dsg_ctx *ctx, int n) {
  DSG_CK(ctx, cudaMemcpyAsync(ctx->red_host, ctx->red_out, n * sizeof(double), cudaMemcpyDeviceToHost,
                              ctx->stream));
  DSG_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return DSG_OK;
}

// Phase marker of the live profile: the phase `id` starts here (-1: the step ends).
cudaError_t phase_mark(dsg_ctx *ctx, int id) {
  if (!ctx->prof) return cudaSuccess;
  if (ctx->phase_used >= ctx->phase_ev.size()) {
    for (int q = 0; q < 64; q++) {
      cudaEvent_t e;
      cudaError_t r = cudaEventCreate(&e);
      if (r != cudaSuccess) return r;
      ctx->phase_ev.push_back(e);
      ctx->phase_id.push_back(-1);
    }
  }
  ctx->phase_id[ctx->phase_used] = id;
  return cudaEventRecord(ctx->phase_ev[ctx->phase_used++], ctx->stream);
}

// The FP64 multigrid of the tolerance mode runs its sweeps, residuals and
// norm in fused multiply-add form unless the configuration asks for the
// reference's exact operation order; the reference's fixed-cycle mode always
// keeps that order.
inline bool fp64_fma(const dsg_ctx *ctx) {
  return ctx->cfg.mode == DSG_MODE_TOL_FP64 && ctx->cfg.fp64_exact == 0;
}

// relax_n on level jj; the finest level is timed with an event pair when the
// live profile is on.
cudaError_t relax_level(dsg_ctx *ctx, int n, int jj, double ls) {
  double **L = ctx->lv[jj];
  const Dims d = ctx->level(jj);
  const bool timed = ctx->prof && jj == ctx->ng && n > 0;
  if (timed) {
    if (ctx->prof_used + 2 > ctx->prof_ev.size()) {
      for (int q = 0; q < 256; q++) {
        cudaEvent_t e;
        cudaError_t r = cudaEventCreate(&e);
        if (r != cudaSuccess) return r;
        ctx->prof_ev.push_back(e);
      }
    }
    cudaError_t r = cudaEventRecord(ctx->prof_ev[ctx->prof_used], ctx->stream);
    if (r != cudaSuccess) return r;
  }
  cudaError_t e =
      dsg::relax_n(n, L[1], ls, L[3], L[4], L[5], L[6], L[7], d, ctx->cfg.omega, ctx->stream, fp64_fma(ctx));
  if (timed) {
    cudaError_t r = cudaEventRecord(ctx->prof_ev[ctx->prof_used + 1], ctx->stream);
    if (r != cudaSuccess) return r;
    ctx->prof_used += 2;
    ctx->prof_relax_calls += n;
    ctx->prof_relax_bytes += (double)n * 6.0 * sizeof(double) * (double)d.count();
    ctx->prof_relax_bits = 64;
  }
  return e;
}

// One V-cycle from level j down to 1 and back (main.f:3705-3759).
int vcycle(dsg_ctx *ctx, int j) {
  const double ls = ctx->s.lengthsize;
  cudaStream_t st = ctx->stream;
  for (int jj = j; jj >= 2; jj--) {
    double **L = ctx->lv[jj];
    const Dims d = ctx->level(jj);
    DSG_CK(ctx, relax_level(ctx, ctx->s.npre, jj, ls));
    DSG_CK(ctx, dsg::resid(ls, L[2], L[1], L[3], L[4], L[5], L[6], d, st, fp64_fma(ctx)));
    const Dims dc = ctx->level(jj - 1);
    DSG_CK(ctx, dsg::rstrct(ctx->lv[jj - 1][3], L[2], dc, st));
    DSG_CK(ctx, dsg::fill_zero(ctx->lv[jj - 1][1], dc.count(), st));
  }
  DSG_CK(ctx, relax_level(ctx, ctx->s.ntop, 1, ls));
  for (int jj = 2; jj <= j; jj++) {
    double **L = ctx->lv[jj];
    const Dims d = ctx->level(jj);
    DSG_CK(ctx, dsg::addint(L[1], ctx->lv[jj - 1][1], L[2], d, st));
    DSG_CK(ctx, relax_level(ctx, ctx->s.npost, jj, ls));
  }
  return DSG_OK;
}

int relres_host(dsg_ctx *ctx, double *out) {
  double **L = ctx->lv[ctx->ng];
  DSG_CK(ctx, dsg::relres_sums(ctx->red_out, ctx->red_partials, ctx->s.lengthsize, L[1], L[3], L[4], L[5],
                               L[6], ctx->fine(), ctx->stream, fp64_fma(ctx)));
  int rc = read_device(ctx, 2);
  if (rc) return rc;
  const double rr = ctx->red_host[0], bb = ctx->red_host[1];
  if (!isfinite(rr) || !isfinite(bb))
    return dsg::set_error(ctx, DSG_E_NONFINITE, "non-finite residual norm (%g, %g)", rr, bb);
  *out = bb > 0.0 ? sqrt(rr) / sqrt(bb) : sqrt(rr);
  return DSG_OK;
}

// ---- mixed precision: FP32 V-cycles inside FP64 defect correction ---------
using namespace dsg::mixed;

cudaError_t relax32_level(dsg_ctx *ctx, int n, int l) {
  float **L = ctx->lv32[l];
  const Dims d = ctx->level(l);
  const bool fine = l == ctx->ng;
  const bool timed = ctx->prof && fine && n > 0;
  if (timed && ctx->cap) {
    // inside a graph capture: the event pair becomes two record nodes, read
    // back after every replay (graph_run)
    cudaEvent_t e0, e1;
    cudaError_t r = cudaEventCreate(&e0);
    if (r == cudaSuccess) r = cudaEventCreate(&e1);
    if (r != cudaSuccess) return r;
    ctx->cap->ev.push_back(e0);
    ctx->cap->ev.push_back(e1);
    ctx->cap->ev_n.push_back(n);
    // External records become event-record nodes that run on every replay
    // (a plain record during capture only marks a dependency).
    r = cudaEventRecordWithFlags(e0, ctx->stream, cudaEventRecordExternal);
    if (r != cudaSuccess) return r;
    FineSplit f = fine_split(ctx);
    float r1, r2;
    phase_coefs(ctx, &r1, &r2);
    cudaError_t e =
        dsg::relax32_split_n(n, f.u, f.r, L[A32], d, level_h2(ctx, l), omega32(ctx), r1, r2, ctx->stream);
    if (e != cudaSuccess) return e;
    return cudaEventRecordWithFlags(e1, ctx->stream, cudaEventRecordExternal);
  }
  if (timed) {
    if (ctx->prof_used + 2 > ctx->prof_ev.size()) {
      for (int q = 0; q < 256; q++) {
        cudaEvent_t e;
        cudaError_t r = cudaEventCreate(&e);
        if (r != cudaSuccess) return r;
        ctx->prof_ev.push_back(e);
      }
    }
    cudaError_t r = cudaEventRecord(ctx->prof_ev[ctx->prof_used], ctx->stream);
    if (r != cudaSuccess) return r;
  }
  cudaError_t e;
  if (fine) {
    FineSplit f = fine_split(ctx);
    float r1, r2;
    phase_coefs(ctx, &r1, &r2);
    e = dsg::relax32_split_n(n, f.u, f.r, L[A32], d, level_h2(ctx, l), omega32(ctx), r1, r2, ctx->stream);
  } else {
    e = dsg::relax32_n(n, L[U32], level_h2(ctx, l), L[RHS32], L[A32], L[B32], L[C32], L[EI32], d,
                       omega32(ctx), ctx->stream);
  }
  if (timed) {
    cudaError_t r = cudaEventRecord(ctx->prof_ev[ctx->prof_used + 1], ctx->stream);
    if (r != cudaSuccess) return r;
    ctx->prof_used += 2;
    ctx->prof_relax_calls += n;
    // colour-split sweep: per colour pass the other colour (half), own colour
    // read+write (half each), own rhs (half) and cc (full): 6 FP32 words per cell
    ctx->prof_relax_bytes += (double)n * 6.0 * sizeof(float) * (double)d.count();
    ctx->prof_relax_bits = 32;
  }
  return e;
}

int vcycle32(dsg_ctx *ctx, int j) {
  cudaStream_t st = ctx->stream;
  const int ng = ctx->ng;
  float r1, r2;
  phase_coefs(ctx, &r1, &r2);
  // levels 1..jt in one single-block launch (0: every level pass by pass)
  const int jt = ctx->tail_top < j ? ctx->tail_top : j;
  for (int jj = j; jj >= 2 && jj > jt; jj--) {
    float **L = ctx->lv32[jj];
    float **Lc = ctx->lv32[jj - 1];
    DSG_CK(ctx, relax32_level(ctx, pre32(ctx, jj), jj));
    if (jj == ng) {
      FineSplit f = fine_split(ctx);
      DSG_CK(ctx, dsg::resid_restrict32_split(Lc[RHS32], Lc[U32], f.u, f.r, L[A32], ctx->level(jj),
                                              1.0f / level_h2(ctx, jj), r1, r2, st));
    } else {
      DSG_CK(ctx, dsg::resid_restrict32(Lc[RHS32], Lc[U32], L[U32], L[RHS32], L[A32], L[B32], L[C32],
                                        ctx->level(jj), 1.0f / level_h2(ctx, jj), st));
    }
  }
  if (jt >= 1) {
    dsg::TailArgs A;
    tail_args(ctx, jt, &A);
    DSG_CK(ctx, dsg::vtail32(A, st));
  } else {
    DSG_CK(ctx, relax32_level(ctx, ctx->s.ntop, 1));
  }
  for (int jj = jt >= 1 ? jt + 1 : 2; jj <= j; jj++) {
    if (jj == ng) {
      FineSplit f = fine_split(ctx);
      DSG_CK(ctx, dsg::prolong32_split(f.u, ctx->lv32[jj - 1][U32], ctx->level(jj), 1, tri32(ctx), st));
    } else {
      DSG_CK(ctx, dsg::prolong32(ctx->lv32[jj][U32], ctx->lv32[jj - 1][U32], ctx->level(jj), 1, tri32(ctx), st));
    }
    DSG_CK(ctx, relax32_level(ctx, post32(ctx, jj), jj));
  }
  return DSG_OK;
}

// FP64 defect into the FP32 finest rhs, its norms copied to the pinned host
// buffer (no synchronization: capturable).
int defect_launch(dsg_ctx *ctx) {
  double **L = ctx->lv[ctx->ng];
  FineSplit f = fine_split(ctx);
  DSG_CK(ctx, dsg::defect64(f.r, ctx->red_out, ctx->red_partials, L[1], L[3], L[4], L[5], L[6], ctx->diag64,
                            ctx->fine(), ctx->s.lengthsize, ctx->stream));
  DSG_CK(ctx, cudaMemcpyAsync(ctx->red_host, ctx->red_out, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                              ctx->stream));
  return DSG_OK;
}

// Relative residual from the norms of the last defect (after a synchronization).
int defect_read(dsg_ctx *ctx, double *relres) {
  const double rr = ctx->red_host[0], bb = ctx->red_host[1];
  if (!isfinite(rr) || !isfinite(bb))
    return dsg::set_error(ctx, DSG_E_NONFINITE, "non-finite defect norm (%g, %g)", rr, bb);
  *relres = bb > 0.0 ? sqrt(rr) / sqrt(bb) : sqrt(rr);
  return DSG_OK;
}

int defect_host(dsg_ctx *ctx, double *relres) {
  int rc = defect_launch(ctx);
  if (rc) return rc;
  DSG_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return defect_read(ctx, relres);
}

void graph_release(GraphRec &g) {
  if (g.exec) cudaGraphExecDestroy(g.exec);
  g.exec = nullptr;
  for (cudaEvent_t e : g.ev) cudaEventDestroy(e);
  g.ev.clear();
  g.ev_n.clear();
  for (int q = 0; q < 6; q++) g.key[q] = -1;
}

// Capture `body` (a sequence of launches on ctx->stream) into g; returns 1 if
// the stream cannot be captured (the caller then launches directly).
template <class F>
int graph_capture(dsg_ctx *ctx, GraphRec &g, const int key[6], F body) {
  graph_release(g);
  if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  ctx->cap = &g;
  const long long launches0 = dsg::t_launches;
  int rc = body();
  // launches made while capturing became graph nodes: count them per replay
  g.kernels = dsg::t_launches - launches0;
  dsg::g_launches.fetch_sub(g.kernels);
  dsg::t_launches -= g.kernels;
  ctx->cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
  if (rc || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    graph_release(g);
    if (rc) return rc;
    return dsg::cuda_fail(ctx, e, "cudaStreamEndCapture");
  }
  e = cudaGraphInstantiate(&g.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    graph_release(g);
    return dsg::cuda_fail(ctx, e, "cudaGraphInstantiate");
  }
  for (int q = 0; q < 6; q++) g.key[q] = key[q];
  return DSG_OK;
}

// Replay g and wait for it; accumulate the relax times recorded inside it.
int graph_run(dsg_ctx *ctx, GraphRec &g) {
  DSG_CK(ctx, cudaGraphLaunch(g.exec, ctx->stream));
  dsg::g_launches.fetch_add(g.kernels);
  DSG_CK(ctx, cudaStreamSynchronize(ctx->stream));
  if (ctx->prof) {
    for (size_t q = 0; q < g.ev_n.size(); q++) {
      float x = 0.f;
      DSG_CK(ctx, cudaEventElapsedTime(&x, g.ev[2 * q], g.ev[2 * q + 1]));
      ctx->prof_graph_relax_ms += x;
      ctx->prof_relax_calls += g.ev_n[q];
      ctx->prof_relax_bytes += (double)g.ev_n[q] * 6.0 * sizeof(float) * (double)ctx->fine().count();
      ctx->prof_relax_bits = 32;
    }
  }
  return DSG_OK;
}

bool graph_matches(const GraphRec &g, const int key[6]) {
  if (!g.exec) return false;
  for (int q = 0; q < 6; q++)
    if (g.key[q] != key[q]) return false;
  return true;
}

// FP32 hierarchy: cc in FP32 on the finest level (its relax forms the face
// coefficients itself), coarse coefficients by acfromac from the FP64 fine
// coefficients of abcei.
int coef_hierarchy32(dsg_ctx *ctx, cudaStream_t st) {
  const int ng = ctx->ng;
  double **F = ctx->lv[ng];
  DSG_CK(ctx, dsg::to32(ctx->lv32[ng][A32], F[0], ctx->fine().count(), st));
  if (ng >= 2) {
    float **C = ctx->lv32[ng - 1];
    DSG_CK(ctx, dsg::acfromac64to32(C[A32], C[B32], C[C32], C[EI32], F[4], F[5], F[6], ctx->level(ng - 1), st));
  }
  for (int g = ng - 2; g >= 1; g--) {
    float **C = ctx->lv32[g], **Fi = ctx->lv32[g + 1];
    DSG_CK(ctx, dsg::acfromac32(C[A32], C[B32], C[C32], C[EI32], Fi[A32], Fi[B32], Fi[C32], ctx->level(g), st));
  }
  return DSG_OK;
}

// In the mixed modes, the FP32 coefficient hierarchy of this step's abcei on
// the side stream (it reads cc and the FP64 a, b, c, which nothing writes
// before the solve): it overlaps the FP64-bound momentum kernels.
int coef_hierarchy_side(dsg_ctx *ctx) {
  ctx->coef32_async = false;
  if (ctx->cfg.mode != DSG_MODE_TOL_MIXED && ctx->cfg.mode != DSG_MODE_LEARNED) return DSG_OK;
  if (!ctx->side) {
    DSG_CK(ctx, cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
    DSG_CK(ctx, cudaEventCreateWithFlags(&ctx->side_start, cudaEventDisableTiming));
    DSG_CK(ctx, cudaEventCreateWithFlags(&ctx->coef_ev, cudaEventDisableTiming));
  }
  DSG_CK(ctx, cudaEventRecord(ctx->side_start, ctx->stream));
  DSG_CK(ctx, cudaStreamWaitEvent(ctx->side, ctx->side_start, 0));
  int rc = coef_hierarchy32(ctx, ctx->side);
  if (rc) return rc;
  DSG_CK(ctx, cudaEventRecord(ctx->coef_ev, ctx->side));
  ctx->coef32_async = true;
  return DSG_OK;
}

// Initial guess by an FP32 full-multigrid pass (the mglin schedule in FP32).
int fmg32(dsg_ctx *ctx) {
  const int ng = ctx->ng;
  cudaStream_t st = ctx->stream;
  FineSplit f = fine_split(ctx);
  DSG_CK(ctx, dsg::split_from64(f.r, ctx->lv[ng][3], ctx->fine(), st));
  if (ng >= 2) DSG_CK(ctx, dsg::restrict32_split(ctx->lv32[ng - 1][RHS32], f.r, ctx->level(ng - 1), st));
  for (int g = ng - 2; g >= 1; g--)
    DSG_CK(ctx, dsg::restrict32(ctx->lv32[g][RHS32], ctx->lv32[g + 1][RHS32], ctx->level(g), st));
  DSG_CK(ctx, cudaMemsetAsync(ctx->lv32[1][U32], 0, ctx->level(1).count() * sizeof(float), st));
  DSG_CK(ctx, relax32_level(ctx, ctx->s.ntop, 1));
  for (int j = 2; j <= ng; j++) {
    if (j == ng)
      DSG_CK(ctx, dsg::prolong32_split(f.u, ctx->lv32[j - 1][U32], ctx->level(j), 0, tri32(ctx), st));
    else
      DSG_CK(ctx, dsg::prolong32(ctx->lv32[j][U32], ctx->lv32[j - 1][U32], ctx->level(j), 0, tri32(ctx), st));
    const int cycles = fmg32_cycles(ctx, j);
    for (int c = 0; c < cycles; c++) {
      int rc = vcycle32(ctx, j);
      if (rc) return rc;
    }
  }
  DSG_CK(ctx, dsg::correct64(ctx->lv[ng][1], f.u, ctx->fine(), 1, st));
  return DSG_OK;
}

// After a solve: the attached network's training pair when recording is on
// (its input was taken from this solve's start, its target is the solved
// pressure's correction of that start).
int record_pair(dsg_ctx *ctx) {
  if (!ctx->net || !ctx->net_record) return DSG_OK;
  return dsg::nn::net_target(ctx->net, ctx->lv[ctx->ng][1], ctx->fine(), ctx->stream);
}

// FP32 V-cycles the mixed solve expects to need from relative residual r at
// the measured reduction per cycle (the count its outer loop would run).
int cycles_needed(const dsg_ctx *ctx, double r) {
  if (r < ctx->cfg.tol) return 0;
  const int n = (int)ceil(log(ctx->cfg.tol / r) / log(ctx->rho_est) + 0.1);
  return n < 1 ? 1 : n;
}

int mixed_solve(dsg_ctx *ctx, dsg_mg_stats *s) {
  const int ng = ctx->ng;
  cudaStream_t st = ctx->stream;
  if ((ctx->nx - 2) & 1)
    return dsg::set_error(ctx, DSG_E_ARG, "mixed mode needs an even number of interior cells along x (%d)",
                          ctx->nx - 2);
  // inner_vcycles > 0: that many FP32 V-cycles per FP64 defect; 0: as many as
  // the measured reduction per V-cycle predicts are needed to reach tol
  const int fixed = ctx->cfg.inner_vcycles;
  int inner = fixed > 0 ? (fixed < dsg_ctx::kMaxInner ? fixed : dsg_ctx::kMaxInner) : 2;
  int key[6] = {pre32(ctx), post32(ctx), ctx->s.ntop, ctx->cfg.cycles, 0, ctx->prof ? 1 : 0};
  // start: FP32 coefficient hierarchy, FP32 FMG guess, first FP64 defect
  auto first = [&]() -> int {
    if (!ctx->coef32_async) {
      int q = coef_hierarchy32(ctx, st);
      if (q) return q;
    }
    int q = fmg32(ctx);
    if (q) return q;
    return defect_launch(ctx);
  };
  // one outer iteration: `inner` FP32 V-cycles on the correction equation,
  // FP64 accumulation, FP64 defect and its norms
  // With mg32_krylov each V-cycle instead starts from zero on the current FP32
  // residual and its result z = M r is one GCR direction: the FP64 pressure
  // takes the step that minimises the FP32 residual along z made orthogonal
  // (in the operator's image) to the previous direction.
  auto iterate = [&]() -> int {
    FineSplit f = fine_split(ctx);
    if (!ctx->cfg.mg32_krylov) {
      DSG_CK(ctx, cudaMemsetAsync(f.u[0], 0, fine_split_bytes(ctx), st));
      for (int q = 0; q < inner; q++) {
        int e = vcycle32(ctx, ng);
        if (e) return e;
      }
      DSG_CK(ctx, dsg::correct64(ctx->lv[ng][1], f.u, ctx->fine(), 0, st));
      return defect_launch(ctx);
    }
    float **L = ctx->lv32[ng];
    const size_t half = fine_split_bytes(ctx) / (2 * sizeof(float));
    const dsg::GcrBufs g{{L[B32], L[B32] + half}, {L[C32], L[C32] + half}, {L[EI32], L[EI32] + half},
                         ctx->gcr_partials, ctx->gcr_partials + 4 * dsg::kRedBlocks, ctx->gcr_coef};
    float r1, r2;
    phase_coefs(ctx, &r1, &r2);
    for (int q = 0; q < inner; q++) {
      DSG_CK(ctx, cudaMemsetAsync(f.u[0], 0, fine_split_bytes(ctx), st));
      int e = vcycle32(ctx, ng);
      if (e) return e;
      DSG_CK(ctx, dsg::gcr_step(q == 0, q == inner - 1, g, ctx->lv[ng][1], f.u, f.r, L[A32], ctx->fine(),
                                1.0f / level_h2(ctx, ng), r1, r2, st));
    }
    return defect_launch(ctx);
  };
  // Run a phase as a replayed CUDA graph (captured once per sweep-count key),
  // or by direct launches when graphs are off or the stream cannot be captured.
  auto run = [&](GraphRec &g, auto &body) -> int {
    if (ctx->cfg.use_graphs) {
      if (!graph_matches(g, key)) {
        int q = graph_capture(ctx, g, key, body);
        if (q < 0) return q;
        if (q == 1) {
          ctx->cfg.use_graphs = 0;  // stream not capturable: launch directly from now on
          goto direct;
        }
      }
      return graph_run(ctx, g);
    }
  direct:
    int q = body();
    if (q) return q;
    DSG_CK(ctx, cudaStreamSynchronize(st));
    return DSG_OK;
  };
  int rc;
  double r;
  if (!ctx->diag_fresh) {  // coefficients not from this step's abcei: form the defect's diagonal
    double **L = ctx->lv[ng];
    DSG_CK(ctx, dsg::diag_sum(ctx->diag64, L[4], L[5], L[6], ctx->fine(), st));
    ctx->diag_fresh = true;
  }
  if (ctx->coef32_async) DSG_CK(ctx, cudaStreamWaitEvent(st, ctx->coef_ev, 0));
  const bool learned = ctx->cfg.mode == DSG_MODE_LEARNED;
  if (learned && !ctx->net) return dsg::set_error(ctx, DSG_E_STATE, "learned mode without an attached network");
  if (ctx->net) dsg::nn::net_begin_solve(ctx->net);
  if (!learned && (ctx->cfg.warm_start == 1 || ctx->cfg.warm_start == 2)) {
    // previous-step pressure (1) or zero (2) as the initial guess
    if (!ctx->coef32_async) {
      rc = coef_hierarchy32(ctx, st);
      if (rc) return rc;
    }
    if (ctx->cfg.warm_start == 1)
      DSG_CK(ctx, cudaMemcpyAsync(ctx->lv[ng][1], ctx->f[DSG_F_PPREV], ctx->fine().count() * sizeof(double),
                                  cudaMemcpyDeviceToDevice, st));
    else
      DSG_CK(ctx, cudaMemsetAsync(ctx->lv[ng][1], 0, ctx->fine().count() * sizeof(double), st));
    rc = defect_host(ctx, &r);
    if (rc) return rc;
  } else {
    key[4] = ctx->coef32_async ? 1 : 0;  // the start with or without the coefficient hierarchy
    rc = run(ctx->g_first, first);
    if (rc) return rc;
    rc = defect_read(ctx, &r);
    if (rc) return rc;
    double **F = ctx->lv[ng];
    // the network's input: when it runs this solve, or to record a training pair
    if (ctx->net && ((learned && ctx->net_rest == 0) || ctx->net_record)) {
      const FineSplit fs = fine_split(ctx);
      rc = dsg::nn::net_features(ctx->net, F[0], F[3], F[1], ctx->f[DSG_F_PPREV], fs.r, ctx->red_out, ctx->fine(),
                                 ctx->s.lengthsize, st);
      if (rc) return rc;
    }
    if (learned) {
      // Guarded learned start.  The method without the network is this FP32
      // full-multigrid start; the network predicts its correction, scaled to
      // the least FP64 defect (one minimal-residual step, whose defect is known
      // from four sums before p changes).  The correction is kept only if it
      // cuts the V-cycles the solve expects to need; after a rejection the
      // network rests for 1, 2, 4 .. 32 solves (reset by an acceptance).
      s->relres_base = r;
      s->relres_net = -1.0;
      s->fallback = 1;
      if (ctx->net_rest > 0) {
        ctx->net_rest--;
      } else {
        double pred = 0.0, alpha = 0.0;
        rc = dsg::nn::net_correction(ctx->net, F[4], F[5], F[6], ctx->fine(), &pred, &alpha, st);
        if (rc) return rc;
        s->relres_net = pred;
        if (cycles_needed(ctx, pred) < cycles_needed(ctx, r)) {
          rc = dsg::nn::net_apply(ctx->net, F[1], alpha, ctx->fine(), st);
          if (rc) return rc;
          DSG_CK(ctx, dsg::bc_scalar(F[1], ctx->fine(), st));
          rc = defect_host(ctx, &r);
          if (rc) return rc;
          s->fallback = 0;
          ctx->net_backoff = 1;
        } else {
          ctx->net_rest = ctx->net_backoff;
          ctx->net_backoff = ctx->net_backoff < 32 ? 2 * ctx->net_backoff : 32;
        }
      }
      ctx->last_relres_base = s->relres_base;
      ctx->last_relres_net = s->relres_net;
    }
  }
  s->relres_init = r;
  int n = 0;
  while (r >= ctx->cfg.tol && n < ctx->cfg.max_vcycles) {
    if (fixed <= 0) {
      const double need = log(ctx->cfg.tol / r) / log(ctx->rho_est);
      inner = (int)ceil(need + 0.1);
      inner = inner < 1 ? 1 : (inner > dsg_ctx::kMaxInner ? dsg_ctx::kMaxInner : inner);
    }
    if (inner > ctx->cfg.max_vcycles - n) inner = ctx->cfg.max_vcycles - n;
    key[4] = inner;
    rc = run(ctx->g_iter[inner], iterate);
    if (rc) return rc;
    s->fine_sweeps += inner * (pre32(ctx, ctx->ng) + post32(ctx, ctx->ng));
    n += inner;
    const double r_old = r;
    rc = defect_read(ctx, &r);
    if (rc) return rc;
    if (r < r_old && r > 0.0) {
      const double obs = pow(r / r_old, 1.0 / inner);
      ctx->rho_est = obs < 0.05 ? 0.05 : (obs > 0.9 ? 0.9 : obs);
    }
  }
  DSG_CK(ctx, dsg::bc_scalar(ctx->lv[ng][1], ctx->fine(), st));
  s->vcycles = n;
  s->relres = r;
  s->converged = r < ctx->cfg.tol;
  return DSG_OK;
}

}  // namespace

// After a mixed-precision solve (standalone or batched): the training pair of
// an attached network, the context's record of the solve, the caller's
// statistics, and DSG_E_NOT_CONVERGED when the cycle cap stopped it.
int dsg::mixed_finish(dsg_ctx *ctx, dsg_mg_stats *s, dsg_mg_stats *stats) {
  ctx->diag_fresh = false;  // the next solve forms it again unless abcei does
  ctx->coef32_async = false;
  int rc = record_pair(ctx);
  if (rc) return rc;
  ctx->s.last_vcycles = s->vcycles;
  ctx->s.last_relres = s->relres;
  ctx->s.last_relres_fmg = s->relres_init;
  if (stats) *stats = *s;
  if (!s->converged)
    return dsg::set_error(ctx, DSG_E_NOT_CONVERGED, "mixed multigrid reached %d cycles at relres %.3e > tol %.3e",
                          s->vcycles, s->relres, ctx->cfg.tol);
  return DSG_OK;
}

namespace {

int mglin(dsg_ctx *ctx, dsg_mg_stats *stats) {
  const int ng = ctx->ng;
  const double om = ctx->cfg.omega;
  cudaStream_t st = ctx->stream;
  int fine_sweeps = 0;
  if (ctx->cfg.mode == DSG_MODE_TOL_MIXED || ctx->cfg.mode == DSG_MODE_LEARNED) {
    dsg_mg_stats s;
    memset(&s, 0, sizeof s);
    s.mode = ctx->cfg.mode;
    s.relres = -1.0;
    s.relres_init = -1.0;
    s.epsdiv = -1.0;
    int rc = mixed_solve(ctx, &s);
    if (rc) return rc;
    return dsg::mixed_finish(ctx, &s, stats);
  }
  for (int g = ng - 1; g >= 1; g--) {
    const Dims dc = ctx->level(g);
    DSG_CK(ctx, dsg::rstrct(ctx->lv[g][3], ctx->lv[g + 1][3], dc, st));
    DSG_CK(ctx, dsg::acfromac(ctx->lv[g][4], ctx->lv[g][5], ctx->lv[g][6], ctx->lv[g][7], ctx->lv[g + 1][4],
                              ctx->lv[g + 1][5], ctx->lv[g + 1][6], dc, st));
  }
  double **L1 = ctx->lv[1];
  DSG_CK(ctx, dsg::fill_zero(L1[1], ctx->level(1).count(), st));
  // First coarse solve with lengthscale in place of lengthsize (main.f:3686-3689).
  DSG_CK(ctx, dsg::relax_n(ctx->s.ntop, L1[1], ctx->s.lengthscale, L1[3], L1[4], L1[5], L1[6], L1[7],
                           ctx->level(1), om, st, fp64_fma(ctx)));
  for (int j = 2; j <= ng; j++) {
    DSG_CK(ctx, dsg::interp(ctx->lv[j][1], ctx->lv[j - 1][1], ctx->level(j), st));
    for (int c = 0; c < ctx->cfg.cycles; c++) {
      int rc = vcycle(ctx, j);
      if (rc) return rc;
      if (j == ng) fine_sweeps += ctx->s.npre + ctx->s.npost;
    }
  }
  dsg_mg_stats s;
  memset(&s, 0, sizeof s);
  s.mode = ctx->cfg.mode;
  s.relres = -1.0;
  s.relres_init = -1.0;
  s.epsdiv = -1.0;
  ctx->s.last_vcycles = 0;
  ctx->s.last_relres = -1.0;
  ctx->s.last_relres_fmg = -1.0;
  if (ctx->cfg.mode == DSG_MODE_TOL_FP64) {
    double r;
    int rc = relres_host(ctx, &r);
    if (rc) return rc;
    s.relres_init = r;
    int n = 0;
    while (r >= ctx->cfg.tol && n < ctx->cfg.max_vcycles) {
      rc = vcycle(ctx, ng);
      if (rc) return rc;
      fine_sweeps += ctx->s.npre + ctx->s.npost;
      n++;
      rc = relres_host(ctx, &r);
      if (rc) return rc;
    }
    s.vcycles = n;
    s.relres = r;
    s.converged = r < ctx->cfg.tol;
    ctx->s.last_vcycles = n;
    ctx->s.last_relres = r;
    ctx->s.last_relres_fmg = s.relres_init;
    int rr = record_pair(ctx);
    if (rr) return rr;
  } else if (ctx->cfg.mode != DSG_MODE_REF_EXACT) {
    return dsg::set_error(ctx, DSG_E_ARG, "pressure mode %d is not available in this build", ctx->cfg.mode);
  }
  s.fine_sweeps = fine_sweeps;
  if (stats) *stats = s;
  if (ctx->cfg.mode == DSG_MODE_TOL_FP64 && !s.converged)
    return dsg::set_error(ctx, DSG_E_NOT_CONVERGED, "multigrid reached %d V-cycles at relres %.3e > tol %.3e",
                          s.vcycles, s.relres, ctx->cfg.tol);
  return DSG_OK;
}

}  // namespace

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

const char *dsg_last_error(const dsg_ctx *ctx) { return ctx ? ctx->err.c_str() : g_last_error.c_str(); }

int dsg_create(const dsg_config *cfg, dsg_ctx **out) {
  if (!cfg || !out) return dsg::set_error(nullptr, DSG_E_ARG, "null argument");
  *out = nullptr;
  if (cfg->nx < 4 || cfg->ny < 4 || cfg->nz < 4)
    return dsg::set_error(nullptr, DSG_E_ARG, "grid %dx%dx%d too small", cfg->nx, cfg->ny, cfg->nz);
  if (cfg->mode < 0 || cfg->mode > DSG_MODE_LEARNED)
    return dsg::set_error(nullptr, DSG_E_ARG, "unknown mode %d", cfg->mode);
  if (cfg->surfacet != 2 && cfg->surfacet != 5 && cfg->surfacet != 6)
    return dsg::set_error(nullptr, DSG_E_ARG, "surfacet = %d is not available (2: CSF, 5: SGIP, 6: SGIP2)",
                          cfg->surfacet);
  if (cfg->hswitch != 0 && cfg->hswitch != 1)
    return dsg::set_error(nullptr, DSG_E_ARG, "hswitch = %d is not available (0 or 1)", cfg->hswitch);
  if (cfg->iturb != 0 && cfg->iturb != 3)
    return dsg::set_error(nullptr, DSG_E_ARG, "iturb = %d is not available (0: laminar, 3: k-epsilon)", cfg->iturb);
  // the kernels index cells with 32-bit offsets (a grid of 2^31 nodes would
  // need over 500 GB of fields)
  if ((size_t)cfg->nx * cfg->ny * cfg->nz >= ((size_t)1 << 31))
    return dsg::set_error(nullptr, DSG_E_ARG, "grid %dx%dx%d has 2^31 nodes or more", cfg->nx, cfg->ny, cfg->nz);
  // memoryaloc, main.f:284-298 (generalised to sides that are not 2^k+2)
  const int ng = dsg::level_count(cfg->nx, cfg->ny, cfg->nz);
  if (ng < 1) return dsg::set_error(nullptr, DSG_E_ARG, "grid %dx%dx%d too small", cfg->nx, cfg->ny, cfg->nz);
  dsg_ctx *ctx = new dsg_ctx();
  ctx->cfg = *cfg;
  ctx->nx = cfg->nx;
  ctx->ny = cfg->ny;
  ctx->nz = cfg->nz;
  ctx->ng = ng;
  memset(&ctx->s, 0, sizeof ctx->s);
  int nnx = cfg->nx, nny = cfg->ny, nnz = cfg->nz;
  size_t total = 0;
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  for (int l = ng; l >= 1; l--) {
    ctx->lnx[l] = nnx;
    ctx->lny[l] = nny;
    ctx->lnz[l] = nnz;
    total += 8 * up((size_t)nnx * nny * nnz * sizeof(double));
    nnx = nnx / 2 + 1;
    nny = nny / 2 + 1;
    nnz = nnz / 2 + 1;
  }
  for (int l = ng; l >= 1; l--)
    total += 6 * up((size_t)ctx->lnx[l] * ctx->lny[l] * ctx->lnz[l] * sizeof(float));
  const size_t fine = up((size_t)cfg->nx * cfg->ny * cfg->nz * sizeof(double));
  const int nextra = DSG_NFIELDS - 8 + 2;  // fine fields beyond the level arrays + ccf + diag64
  total += nextra * fine;
  total += up(dsg::kRedBlocks * 4 * sizeof(double)) + up(16 * sizeof(double)) + up(sizeof(unsigned long long)) +
           up(sizeof(unsigned)) + up(dsg::kRedBlocks * 6 * sizeof(double)) + up(16 * sizeof(double));
  cudaError_t e = cudaMalloc(&ctx->arena, total);
  if (e != cudaSuccess) {
    int rc = dsg::cuda_fail(ctx, e, "cudaMalloc(arena)");
    g_last_error = ctx->err;
    delete ctx;
    return rc;
  }
  ctx->arena_bytes = total;
  char *p = (char *)ctx->arena;
  for (int l = ng; l >= 1; l--)
    for (int f = 0; f < 8; f++) {
      ctx->lv[l][f] = (double *)p;
      p += up((size_t)ctx->lnx[l] * ctx->lny[l] * ctx->lnz[l] * sizeof(double));
    }
  for (int l = ng; l >= 1; l--)
    for (int f = 0; f < 6; f++) {
      ctx->lv32[l][f] = (float *)p;
      p += up((size_t)ctx->lnx[l] * ctx->lny[l] * ctx->lnz[l] * sizeof(float));
    }
  for (int f = 0; f < 8; f++) ctx->f[f] = ctx->lv[ng][f];
  for (int f = 8; f < DSG_NFIELDS; f++) {
    ctx->f[f] = (double *)p;
    p += fine;
  }
  ctx->ccf = (double *)p;
  p += fine;
  ctx->diag64 = (double *)p;
  p += fine;
  ctx->red_partials = (double *)p;
  p += up(dsg::kRedBlocks * 4 * sizeof(double));
  ctx->red_out = (double *)p;
  p += up(16 * sizeof(double));
  ctx->stop_flag = (unsigned long long *)p;
  p += up(sizeof(unsigned long long));
  ctx->iface_count = (unsigned *)p;
  p += up(sizeof(unsigned));
  ctx->gcr_partials = (double *)p;
  p += up(dsg::kRedBlocks * 6 * sizeof(double));
  ctx->gcr_coef = (double *)p;
  e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocHost(&ctx->red_host, 16 * sizeof(double));
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->arena, 0, total, ctx->own_stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->own_stream);
  if (e != cudaSuccess) {
    int rc = dsg::cuda_fail(ctx, e, "context setup");
    g_last_error = ctx->err;
    dsg_destroy(ctx);
    return rc;
  }
  ctx->stream = ctx->own_stream;
  cudaGetDevice(&ctx->device);
  ctx->s.npre = cfg->npre;
  ctx->s.npost = cfg->npost;
  ctx->s.ntop = cfg->ntop;
  ctx->s.cycles = cfg->cycles;
  ctx->s.ng = ng;
  ctx->s.last_epsdiv = -1.0;
  {
    const long long cap = cfg->tail_nodes == 0 ? 18LL * 18 * 18 : cfg->tail_nodes;
    ctx->tail_top = 0;
    for (int l = 1; l < ng && l <= dsg::kTailMaxLevels; l++)
      if ((long long)ctx->lnx[l] * ctx->lny[l] * ctx->lnz[l] <= cap) ctx->tail_top = l;
  }
  nondim(ctx);
  *out = ctx;
  return DSG_OK;
}

void dsg_destroy(dsg_ctx *ctx) {
  if (!ctx) return;
  if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
  dsg::snapshot_release(ctx);
  for (cudaStream_t x : {ctx->xfer_in, ctx->xfer_out})
    if (x) {
      cudaStreamSynchronize(x);
      cudaStreamDestroy(x);
    }
  for (int q = 0; q < dsg_ctx::kSyncPoints; q++) {
    if (ctx->xfer_in_ev[q]) cudaEventDestroy(ctx->xfer_in_ev[q]);
    if (ctx->xfer_out_ev[q]) cudaEventDestroy(ctx->xfer_out_ev[q]);
  }
  for (int q = 0; q < dsg_ctx::kSChunks; q++) {
    if (ctx->s_chunk_ev[q]) cudaEventDestroy(ctx->s_chunk_ev[q]);
  }
  if (ctx->xfer_start) cudaEventDestroy(ctx->xfer_start);
  if (ctx->side) {
    cudaStreamSynchronize(ctx->side);
    cudaStreamDestroy(ctx->side);
  }
  if (ctx->side_start) cudaEventDestroy(ctx->side_start);
  if (ctx->coef_ev) cudaEventDestroy(ctx->coef_ev);
  for (cudaEvent_t e : ctx->prof_ev) cudaEventDestroy(e);
  for (cudaEvent_t e : ctx->phase_ev) cudaEventDestroy(e);
  graph_release(ctx->g_first);
  for (GraphRec &g : ctx->g_iter) graph_release(g);
  if (ctx->arena) cudaFree(ctx->arena);
  if (ctx->red_host) cudaFreeHost(ctx->red_host);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
}

int dsg_set_stream(dsg_ctx *ctx, void *stream) {
  if (!ctx) return DSG_E_ARG;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return DSG_OK;
}

int dsg_synchronize(dsg_ctx *ctx) {
  if (!ctx) return DSG_E_ARG;
  DSG_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return DSG_OK;
}

int64_t dsg_device_bytes(const dsg_ctx *ctx) { return ctx ? (int64_t)ctx->arena_bytes : 0; }

int dsg_upload(dsg_ctx *ctx, int field, const double *host) {
  if (!ctx || !host || field < 0 || field >= DSG_NFIELDS) return dsg::set_error(ctx, DSG_E_ARG, "bad upload");
  if (field == DSG_F_CC || field == DSG_F_A || field == DSG_F_B || field == DSG_F_C) {
    // coefficients or volume fraction replaced: the next solve forms its
    // diagonal and FP32 hierarchy from them
    ctx->diag_fresh = false;
    ctx->coef32_async = false;
  }
  DSG_CK(ctx, cudaMemcpyAsync(ctx->f[field], host, ctx->fine().count() * sizeof(double), cudaMemcpyHostToDevice,
                              ctx->stream));
  DSG_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return DSG_OK;
}

int dsg_download(dsg_ctx *ctx, int field, double *host) {
  if (!ctx || !host || field < 0 || field >= DSG_NFIELDS) return dsg::set_error(ctx, DSG_E_ARG, "bad download");
  DSG_CK(ctx, cudaMemcpyAsync(host, ctx->f[field], ctx->fine().count() * sizeof(double), cudaMemcpyDeviceToHost,
                              ctx->stream));
  DSG_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return DSG_OK;
}

int dsg_level_ptr(dsg_ctx *ctx, int field, int level, double **dev, int *nx, int *ny, int *nz) {
  if (!ctx || field < 0 || field > 7 || level < 1 || level > ctx->ng || !dev)
    return dsg::set_error(ctx, DSG_E_ARG, "bad level field");
  *dev = ctx->lv[level][field];
  if (nx) *nx = ctx->lnx[level];
  if (ny) *ny = ctx->lny[level];
  if (nz) *nz = ctx->lnz[level];
  return DSG_OK;
}

int dsg_field_ptr(dsg_ctx *ctx, int field, double **dev) {
  if (!ctx || field < 0 || field >= DSG_NFIELDS || !dev) return dsg::set_error(ctx, DSG_E_ARG, "bad field");
  *dev = ctx->f[field];
  return DSG_OK;
}

int dsg_get_scalars(const dsg_ctx *ctx, dsg_scalars *out) {
  if (!ctx || !out) return DSG_E_ARG;
  *out = ctx->s;
  return DSG_OK;
}

int dsg_set_scalars(dsg_ctx *ctx, const dsg_scalars *in) {
  if (!ctx || !in) return DSG_E_ARG;
  const int ng = ctx->s.ng;
  ctx->s = *in;
  ctx->s.ng = ng;
  return DSG_OK;
}

int dsg_init_drop(dsg_ctx *ctx) {
  if (!ctx) return DSG_E_ARG;
  dsg_scalars &s = ctx->s;
  const Dims d = ctx->fine();
  // smooth2 geometry (main.f:5684-5691)
  const double x0 = (ctx->nx - 2) * s.h / 4.0;
  if (ctx->cfg.z0_si != 1000.0) s.z0 = ctx->cfg.z0_si / ctx->cfg.length_si;
  if (ctx->cfg.y0_si != 1000.0) s.y0 = ctx->cfg.y0_si / ctx->cfg.length_si;
  s.y0 = s.y0 + s.h / 2.0;
  const double amp = ctx->cfg.noise_si / s.vscale;
  DSG_CK(ctx, dsg::init_drop(ctx->f[DSG_F_CC], ctx->f[DSG_F_U], ctx->f[DSG_F_V], ctx->f[DSG_F_W], d, s.h, x0,
                             s.y0, s.z0, s.radius, s.yvel1, s.yvel2, s.zvel1, s.zvel2, amp, ctx->cfg.noise_seed,
                             ctx->stream));
  return dsg::restart_state(ctx);
}

}  // extern "C"

int dsg::restart_state(dsg_ctx *ctx) {
  const dsg_scalars &s = ctx->s;
  const Dims d = ctx->fine();
  DSG_CK(ctx, dsg::bc_c(ctx->f[DSG_F_CC], d, ctx->stream));
  DSG_CK(ctx, dsg::bc_v(ctx->f[DSG_F_U], ctx->f[DSG_F_V], ctx->f[DSG_F_W], ctx->red_partials, d, s.xvel2,
                        ctx->stream));
  DSG_CK(ctx, dsg::calcrho(ctx->f[DSG_F_RHON], ctx->f[DSG_F_MUN], ctx->f[DSG_F_CC], d, s.rho1, s.rho2, s.mu1,
                           s.mu2, ctx->stream));
  if (ctx->cfg.iturb == 3) {
    // ktur = 0.00015 v^2 per phase (inijet, main.f:536-549), v the phase speed
    const double v1 = sqrt(s.xvel1 * s.xvel1 + s.yvel1 * s.yvel1 + s.zvel1 * s.zvel1);
    const double v2 = sqrt(s.xvel2 * s.xvel2 + s.yvel2 * s.yvel2 + s.zvel2 * s.zvel2);
    const double dv = sqrt((s.xvel1 - s.xvel2) * (s.xvel1 - s.xvel2) + (s.yvel1 - s.yvel2) * (s.yvel1 - s.yvel2) +
                           (s.zvel1 - s.zvel2) * (s.zvel1 - s.zvel2));
    const double k1 = (double)0.00015f * v1 * v1;
    const double g = v2 + dv * (double)0.01f;
    const double k2 = (double)0.00015f * (g * g);
    DSG_CK(ctx, dsg::keps_seed(ctx->f[DSG_F_KTUR], ctx->f[DSG_F_EPS], ctx->f[DSG_F_MUT], ctx->f[DSG_F_CC],
                               ctx->f[DSG_F_RHON], ctx->f[DSG_F_MUN], d, k1, k2, ctx->stream));
  }
  DSG_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return DSG_OK;
}

namespace {

// Sync points of a time step, in order: before each of the three VOF sweeps,
// after the VOF phase (VOFmethod, CalcH3d, kepsmodel), after checktime, after
// the surface-tension phase, after the multigrid solve inside solvelpres, and
// at the end of the step.  A host-buffer step hooks its copies in there.
enum { SP_SWEEP1 = 0, SP_SWEEP2, SP_SWEEP3, SP_VOF, SP_CFL, SP_CSF, SP_MG, SP_END };
static_assert(SP_END + 1 == dsg_ctx::kSyncPoints, "sync points");

inline int sync_point(dsg_ctx *ctx, int point) {
  return ctx->sync_hook ? ctx->sync_hook(ctx, point, ctx->sync_arg) : DSG_OK;
}

// Velocity components of the three sweeps for sweep counter tswap (VOFmethod,
// main.f:795-824: the order rotates with tswap).
void sweep_order(int tswap, int order[3]) {
  if (tswap % 3 == 0) { order[0] = 3; order[1] = 1; order[2] = 2; }
  else if (tswap % 2 == 0) { order[0] = 2; order[1] = 3; order[2] = 1; }
  else { order[0] = 1; order[1] = 2; order[2] = 3; }
}

}  // namespace

extern "C" {

int dsg_vofmethod(dsg_ctx *ctx) {
  if (!ctx) return DSG_E_ARG;
  dsg_scalars &s = ctx->s;
  const Dims d = ctx->fine();
  double *cc = ctx->f[DSG_F_CC], *s1 = ctx->f[DSG_F_EI], *s2 = ctx->f[DSG_F_RES], *s3 = ctx->f[DSG_F_RHS];
  double *vel[4] = {nullptr, ctx->f[DSG_F_U], ctx->f[DSG_F_V], ctx->f[DSG_F_W]};
  s.tswap = s.tswap + 1;
  if (s.tswap > 3) s.tswap = 1;
  int order[3];
  sweep_order(s.tswap, order);
  for (int q = 0; q < 3; q++) {
    int rc = sync_point(ctx, SP_SWEEP1 + q);
    if (rc) return rc;
    DSG_CK(ctx, dsg::swp(vel[order[q]], cc, s1, s2, s3, order[q], d, s.tauh, reinterpret_cast<unsigned *>(ctx->ccf),
                         ctx->iface_count, ctx->stream));
  }
  DSG_CK(ctx, dsg::bc_c(cc, d, ctx->stream));
  // turbulent diffusion of the volume fraction (main.f:820)
  if (ctx->cfg.iturb != 0)
    DSG_CK(ctx, dsg::fturbdif(cc, ctx->f[DSG_F_MUT], ctx->f[DSG_F_RHON], d, s.tauh2, ctx->stream));
  DSG_CK(ctx, dsg::calcrho(ctx->f[DSG_F_RHON], ctx->f[DSG_F_MUN], cc, d, s.rho1, s.rho2, s.mu1, s.mu2,
                           ctx->stream));
  return DSG_OK;
}

// kepsmodel (main.f:39-40): the new values go through the pressure and
// residual arrays, the scratch the reference passes.
int dsg_kepsmodel(dsg_ctx *ctx) {
  if (!ctx) return DSG_E_ARG;
  if (ctx->cfg.iturb != 3) return DSG_OK;
  const dsg_scalars &s = ctx->s;
  DSG_CK(ctx, dsg::kepsmodel(ctx->f[DSG_F_KTUR], ctx->f[DSG_F_EPS], ctx->f[DSG_F_MUT], ctx->f[DSG_F_P],
                             ctx->f[DSG_F_RES], ctx->f[DSG_F_MUN], ctx->f[DSG_F_RHON], ctx->f[DSG_F_U],
                             ctx->f[DSG_F_V], ctx->f[DSG_F_W], ctx->fine(), s.h, s.tau, ctx->stream));
  return DSG_OK;
}

int dsg_checktime(dsg_ctx *ctx) {
  if (!ctx) return DSG_E_ARG;
  dsg_scalars &s = ctx->s;
  DSG_CK(ctx, dsg::absmax3(ctx->red_out, ctx->red_partials, ctx->f[DSG_F_U], ctx->f[DSG_F_V], ctx->f[DSG_F_W],
                           ctx->fine(), ctx->stream));
  int rc = read_device(ctx, 1);
  if (rc) return rc;
  double cfl1 = ctx->red_host[0] * s.tauh;
  if (!isfinite(cfl1)) return dsg::set_error(ctx, DSG_E_NONFINITE, "non-finite velocity in CFL");
  const double maxcfl = ctx->cfg.maxcfl;
  if (cfl1 > maxcfl) {
    s.tau = s.tau * (maxcfl * (double)0.8f) / cfl1;
    s.tauh = s.tau / s.h;
    s.tauh2 = (int)(s.tau / (s.h * s.h));
  }
  if (cfl1 <= maxcfl * (double)0.25f) {
    cfl1 = maxcfl * (double)0.5f;
    s.tau = s.tau * (maxcfl * (double)0.5f) / cfl1;
    s.tauh = s.tau / s.h;
    s.tauh2 = (int)(s.tau / (s.h * s.h));
  }
  s.time = s.time + s.tau;
  return DSG_OK;
}

int dsg_csf(dsg_ctx *ctx) { return dsg::csf_phase(ctx, true); }

}  // extern "C"

// The surface-tension model of surfacet; scratch: csf's copies into the
// pressure, residual and rhs arrays (the reference's aliasing), which a whole
// step overwrites before reading.
int dsg::csf_phase(dsg_ctx *ctx, bool scratch) {
  if (!ctx) return DSG_E_ARG;
  Tensor S(ctx);
  if (ctx->cfg.surfacet == 5 || ctx->cfg.surfacet == 6) {
    double *H[6];
    for (int m = 0; m < 6; m++) H[m] = ctx->f[DSG_F_HXMIN + m];
    if (ctx->cfg.surfacet == 5)
      DSG_CK(ctx, dsg::sgip(ctx->f[DSG_F_CC], ctx->f[DSG_F_P], ctx->f[DSG_F_RES], ctx->f[DSG_F_RHS], ctx->ccf, S.p,
                            H, ctx->f[DSG_F_U], ctx->f[DSG_F_W], ctx->fine(), ctx->s.tau, ctx->s.sigma, ctx->s.h,
                            ctx->stream));
    else
      DSG_CK(ctx, dsg::sgip2(ctx->f[DSG_F_CC], ctx->f[DSG_F_P], ctx->f[DSG_F_RES], ctx->f[DSG_F_RHS], ctx->ccf, S.p,
                             H, ctx->fine(), ctx->s.tau, ctx->s.sigma, ctx->s.h, ctx->stream));
    return DSG_OK;
  }
  DSG_CK(ctx, dsg::csf(ctx->f[DSG_F_CC], ctx->f[DSG_F_P], ctx->f[DSG_F_RES], ctx->f[DSG_F_RHS], ctx->ccf, S.p,
                       ctx->fine(), ctx->s.tau, ctx->s.sigma, ctx->s.h, ctx->stream, scratch));
  return DSG_OK;
}

extern "C" {

// CalcH3d (main.f:30 with hswitch = 1).  The reference STOPs when a cell
// matches none of the polygon cases; here the step returns DSG_E_STATE.
int dsg_calch3d(dsg_ctx *ctx) {
  if (!ctx) return DSG_E_ARG;
  double *H[6];
  for (int m = 0; m < 6; m++) H[m] = ctx->f[DSG_F_HXMIN + m];
  DSG_CK(ctx, cudaMemsetAsync(ctx->stop_flag, 0, sizeof(unsigned long long), ctx->stream));
  DSG_CK(ctx, dsg::calch3d(H, ctx->f[DSG_F_CC], ctx->fine(), ctx->stop_flag, ctx->stream));
  DSG_CK(ctx, cudaMemcpyAsync(ctx->red_host + 15, ctx->stop_flag, sizeof(unsigned long long),
                              cudaMemcpyDeviceToHost, ctx->stream));
  DSG_CK(ctx, cudaStreamSynchronize(ctx->stream));
  unsigned long long v;
  memcpy(&v, ctx->red_host + 15, sizeof v);
  if (v) {
    const long long q = (long long)(v & ((1ull << 48) - 1));
    const int i = (int)(q % ctx->nx) + 1, j = (int)((q / ctx->nx) % ctx->ny) + 1, k = (int)(q / ((long long)ctx->nx * ctx->ny)) + 1;
    return dsg::set_error(ctx, DSG_E_STATE, "CalcH3d: %s at cell (%d,%d,%d)",
                          (v >> 48) == 1 ? "NO MATCH CASES FOUND" : "PROBLEM finding MIN and MAX unit vector components",
                          i, j, k);
  }
  return DSG_OK;
}

int dsg_mglin(dsg_ctx *ctx, dsg_mg_stats *stats) {
  if (!ctx) return DSG_E_ARG;
  return mglin(ctx, stats);
}

int dsg_solvelpres(dsg_ctx *ctx, int t, dsg_mg_stats *stats) {
  if (!ctx) return DSG_E_ARG;
  int rc = dsg::solvelpres_pre(ctx);
  if (rc) return rc;
  dsg_mg_stats ms;
  memset(&ms, 0, sizeof ms);
  rc = mglin(ctx, &ms);
  if (rc && rc != DSG_E_NOT_CONVERGED) return rc;
  return dsg::solvelpres_post(ctx, t, &ms, rc, stats);
}

}  // extern "C"

// solvelpres up to the pressure solve (main.f:3236-3355): stresses, the
// coefficients of abcei, predictor, convection, boundary values and the
// divergence right-hand side.
int dsg::solvelpres_pre(dsg_ctx *ctx) {
  dsg_scalars &s = ctx->s;
  const Dims d = ctx->fine();
  cudaStream_t st = ctx->stream;
  double *cc = ctx->f[DSG_F_CC], *w1 = ctx->f[DSG_F_P], *w2 = ctx->f[DSG_F_RES], *w3 = ctx->f[DSG_F_RHS];
  double *a = ctx->f[DSG_F_A], *b = ctx->f[DSG_F_B], *c = ctx->f[DSG_F_C], *ei = ctx->f[DSG_F_EI];
  double *u = ctx->f[DSG_F_U], *v = ctx->f[DSG_F_V], *w = ctx->f[DSG_F_W];
  Tensor S(ctx);
  const double tauh2 = (double)s.tauh2, mu1 = s.mu1, mu2 = s.mu2;
  const double r20 = tauh2 * mu2;
  const double r10 = 0.25 * tauh2 * (mu1 - mu2);
  double r1 = 2.0 * tauh2 * (mu1 - mu2);
  double r2 = 2.0 * tauh2 * mu2;
  const double stdgrav = s.g * (s.tau * s.tau) / s.h;
  const double horgrav = s.g1 * (s.tau * s.tau) / s.h;
  const double rho_r2 = s.rho2, rho_r1 = 0.5 * (s.rho1 - s.rho2);
  DSG_CK(ctx, phase_mark(ctx, 3));
  if (ctx->s_chunks > 0) {
    // S12/S13/S23 still arriving in chunks of planes (dsg_step_host): abcei
    // (cc only) first; then per chunk, once its copies are in, the csf faces
    // of those stresses written again, stress and bc_tensor on its planes,
    // and the predictor on the previous chunk's planes (it reads the
    // stresses of the planes either side).  The same cells get the same
    // values as in the unsplit order.
    DSG_CK(ctx, dsg::abcei(a, b, c, ei, cc, rho_r1, rho_r2, d, st, ctx->diag64));
    ctx->diag_fresh = true;
    int rc = coef_hierarchy_side(ctx);
    if (rc) return rc;
    const int *K = ctx->s_chunk_k, n = ctx->s_chunks;
    auto lo = [&](int q) { return K[q] > 2 ? K[q] : 2; };
    auto hi = [&](int q) { return K[q + 1] < d.nz ? K[q + 1] : d.nz; };
    for (int q = 0; q < n; q++) {
      DSG_CK(ctx, cudaStreamWaitEvent(st, ctx->s_chunk_ev[q], 0));
      DSG_CK(ctx, dsg::bc_tensor_offdiag(S.p[3], S.p[4], S.p[5], d, st, K[q], K[q + 1]));
      if (hi(q) > lo(q)) DSG_CK(ctx, dsg::stress(S.p, u, v, w, cc, d, r1, r2, r10, r20, st, lo(q), hi(q)));
      DSG_CK(ctx, dsg::bc_tensor(S.p, d, st, K[q], K[q + 1]));
      if (q > 0 && hi(q - 1) > lo(q - 1))
        DSG_CK(ctx, dsg::predictor(w1, w2, w3, u, v, w, a, b, c, S.p, d, horgrav, stdgrav, st, lo(q - 1),
                                   hi(q - 1)));
    }
    if (hi(n - 1) > lo(n - 1))
      DSG_CK(ctx, dsg::predictor(w1, w2, w3, u, v, w, a, b, c, S.p, d, horgrav, stdgrav, st, lo(n - 1),
                                 hi(n - 1)));
  } else {
    DSG_CK(ctx, dsg::stress(S.p, u, v, w, cc, d, r1, r2, r10, r20, st));
    DSG_CK(ctx, dsg::bc_tensor(S.p, d, st));
    DSG_CK(ctx, dsg::abcei(a, b, c, ei, cc, rho_r1, rho_r2, d, st, ctx->diag64));
    ctx->diag_fresh = true;
    int rc = coef_hierarchy_side(ctx);
    if (rc) return rc;
    DSG_CK(ctx, dsg::predictor(w1, w2, w3, u, v, w, a, b, c, S.p, d, horgrav, stdgrav, st));
  }
  DSG_CK(ctx, dsg::bc_w(w1, w2, w3, u, v, w, ctx->red_partials, d, st));
  DSG_CK(ctx, dsg::convective(u, v, w, w1, w2, w3, d, s.tauh, ctx->cfg.convectype, st));
  DSG_CK(ctx, dsg::bc_v(u, v, w, ctx->red_partials, d, s.xvel2, st));
  const double hi2 = 1.0 / (s.h * s.h);
  DSG_CK(ctx, dsg::divergence(w3, u, v, w, d, hi2, st));
  DSG_CK(ctx, phase_mark(ctx, 4));
  return DSG_OK;
}

// solvelpres after the pressure solve (main.f:3371-3439): projection,
// boundary values and the relaxation-count adaptivity.  ms: the solve's
// statistics; mg_rc: its status (DSG_OK or DSG_E_NOT_CONVERGED), returned
// when nothing else fails.
int dsg::solvelpres_post(dsg_ctx *ctx, int t, dsg_mg_stats *ms_in, int mg_rc, dsg_mg_stats *stats) {
  dsg_scalars &s = ctx->s;
  const Dims d = ctx->fine();
  cudaStream_t st = ctx->stream;
  double *w1 = ctx->f[DSG_F_P], *w3 = ctx->f[DSG_F_RHS];
  double *a = ctx->f[DSG_F_A], *b = ctx->f[DSG_F_B], *c = ctx->f[DSG_F_C];
  double *u = ctx->f[DSG_F_U], *v = ctx->f[DSG_F_V], *w = ctx->f[DSG_F_W];
  const double hi2 = 1.0 / (s.h * s.h);
  dsg_mg_stats ms = *ms_in;
  int rc;
  if ((rc = sync_point(ctx, SP_MG))) return rc;
  DSG_CK(ctx, phase_mark(ctx, 5));
  DSG_CK(ctx, cudaMemcpyAsync(ctx->f[DSG_F_PPREV], w1, d.count() * sizeof(double), cudaMemcpyDeviceToDevice, st));
  DSG_CK(ctx, dsg::project(u, v, w, w1, a, b, c, d, st));
  DSG_CK(ctx, dsg::bc_v(u, v, w, ctx->red_partials, d, s.xvel2, st));
  ms.epsdiv = -1.0;
  s.last_epsdiv = -1.0;
  if (t <= 1 || t % 10 == 0) {
    // relaxation-count adaptivity, main.f:3389-3416
    DSG_CK(ctx, dsg::divergence(w3, u, v, w, d, hi2, st));
    DSG_CK(ctx, dsg::absmax3(ctx->red_out, ctx->red_partials, w3, nullptr, nullptr, d, st));
    rc = read_device(ctx, 1);
    if (rc) return rc;
    const double epsdiv = s.h * ctx->red_host[0];
    ms.epsdiv = epsdiv;
    s.last_epsdiv = epsdiv;
    if (epsdiv > 25.0 && s.ntop < 30) {
      s.ntop += 2;
      s.npre += 2;
      s.npost += 2;
    } else if (epsdiv < 2.5 && s.ntop > 4) {
      s.npre -= 1;
      s.ntop -= 1;
      s.npost -= 1;
    }
  }
  if (ctx->cfg.tprint > 0 && t % ctx->cfg.tprint == 0) DSG_CK(ctx, dsg::divergence(w3, u, v, w, d, hi2, st));
  if (stats) *stats = ms;
  return mg_rc;
}

namespace {

// One time step in the order of the main.f:19-73 loop body: VOF (VOFmethod,
// CalcH3d, kepsmodel), CFL (checktime), surface tension (csf / sgip / sgip2)
// and pressure (solvelpres), with the sync points between them.  A pressure
// solve that stops at its cycle cap still completes the step and its
// DSG_E_NOT_CONVERGED is returned after the last sync point.
int step_phases(dsg_ctx *ctx, int t, dsg_mg_stats *stats) {
  int rc = dsg::step_pre_solve(ctx, t);
  if (rc) return rc;
  dsg_mg_stats ms;
  memset(&ms, 0, sizeof ms);
  rc = mglin(ctx, &ms);
  if (rc && rc != DSG_E_NOT_CONVERGED) return rc;
  return dsg::step_post_solve(ctx, t, &ms, rc, stats);
}

}  // namespace

// The step up to the pressure solve: VOF, CFL, surface tension and the first
// part of solvelpres.
int dsg::step_pre_solve(dsg_ctx *ctx, int t) {
  (void)t;
  DSG_CK(ctx, phase_mark(ctx, 0));
  int rc = dsg_vofmethod(ctx);
  if (rc) return rc;
  if (ctx->cfg.hswitch == 1) {
    rc = dsg_calch3d(ctx);
    if (rc) return rc;
  }
  rc = dsg_kepsmodel(ctx);
  if (rc || (rc = sync_point(ctx, SP_VOF))) return rc;
  DSG_CK(ctx, phase_mark(ctx, 1));
  rc = dsg_checktime(ctx);
  if (rc || (rc = sync_point(ctx, SP_CFL))) return rc;
  DSG_CK(ctx, phase_mark(ctx, 2));
  rc = dsg::csf_phase(ctx, false);
  if (rc || (rc = sync_point(ctx, SP_CSF))) return rc;
  return dsg::solvelpres_pre(ctx);
}

// The step after the pressure solve (ms, mg_rc: the solve's statistics and
// status, DSG_OK or DSG_E_NOT_CONVERGED, returned when nothing else fails).
int dsg::step_post_solve(dsg_ctx *ctx, int t, dsg_mg_stats *ms, int mg_rc, dsg_mg_stats *stats) {
  int rc = dsg::solvelpres_post(ctx, t, ms, mg_rc, stats);
  if (rc && rc != DSG_E_NOT_CONVERGED) return rc;
  DSG_CK(ctx, phase_mark(ctx, -1));
  const int rh = sync_point(ctx, SP_END);
  return rh ? rh : rc;
}

namespace {

// Sync point before which an input of field f must have arrived from the
// host: before the first work that reads or writes it.  u, v, w are read first
// by their own VOF sweep (order from the sweep counter the step will use);
// all six stress components are written by the surface-tension phase (csf's
// bc_tensor zeroes ghost faces of S12, S13, S23; with sigma = 0 all six are
// zeroed), so they arrive before it; a, b, c and the previous pressures are
// first touched in the pressure phase.
bool late_offdiag(const dsg_ctx *ctx) { return ctx->cfg.surfacet == 2 && ctx->s.sigma != 0.0; }

int first_touch(const dsg_ctx *ctx, int f) {
  int order[3];
  sweep_order(ctx->s.tswap + 1 > 3 ? 1 : ctx->s.tswap + 1, order);
  switch (f) {
    case DSG_F_U: case DSG_F_V: case DSG_F_W:
      for (int q = 0; q < 3; q++)
        if (order[q] == f - DSG_F_U + 1) return SP_SWEEP1 + q;
      return SP_SWEEP1;
    case DSG_F_S11: case DSG_F_S22: case DSG_F_S33:
      return SP_CFL;
    case DSG_F_S12: case DSG_F_S13: case DSG_F_S23:
      // csf (surfacet 2, sigma != 0) only writes their constant bc_tensor
      // faces, which xfer_hook writes again after a late upload; the
      // momentum phase reads them first.  Otherwise csf or SGIP may write
      // their interiors: before it.
      return late_offdiag(ctx) ? SP_CSF : SP_CFL;
    case DSG_F_A: case DSG_F_B: case DSG_F_C: case DSG_F_PPREV: case DSG_F_PPREV2:
      return SP_CSF;
    default:
      return SP_SWEEP1;
  }
}

// Sync point after which field f no longer changes in the step: the VOF
// fields after the VOF phase, the pressure after the multigrid solve (the
// projection only reads it), everything else at the end.
int last_write(int f) {
  switch (f) {
    case DSG_F_CC: case DSG_F_RHON: case DSG_F_MUN: case DSG_F_KTUR: case DSG_F_EPS: case DSG_F_MUT:
    case DSG_F_HXMIN: case DSG_F_HXMAX: case DSG_F_HYMIN: case DSG_F_HYMAX: case DSG_F_HZMIN: case DSG_F_HZMAX:
      return SP_VOF;
    case DSG_F_P:
      return SP_MG;
    default:
      return SP_END;
  }
}

int xfer_resources(dsg_ctx *ctx) {
  if (ctx->xfer_in) return DSG_OK;
  DSG_CK(ctx, cudaEventCreateWithFlags(&ctx->xfer_start, cudaEventDisableTiming));
  for (int q = 0; q < dsg_ctx::kSyncPoints; q++) {
    DSG_CK(ctx, cudaEventCreateWithFlags(&ctx->xfer_in_ev[q], cudaEventDisableTiming));
    DSG_CK(ctx, cudaEventCreateWithFlags(&ctx->xfer_out_ev[q], cudaEventDisableTiming));
  }
  for (int q = 0; q < dsg_ctx::kSChunks; q++)
    DSG_CK(ctx, cudaEventCreateWithFlags(&ctx->s_chunk_ev[q], cudaEventDisableTiming));
  DSG_CK(ctx, cudaStreamCreateWithFlags(&ctx->xfer_out, cudaStreamNonBlocking));
  DSG_CK(ctx, cudaStreamCreateWithFlags(&ctx->xfer_in, cudaStreamNonBlocking));
  return DSG_OK;
}

// The copies of one host-buffer step.
struct HostXfer {
  int n_in, n_out;
  const int *in_fields, *out_fields;
  double *const *out_host;
  bool need[dsg_ctx::kSyncPoints];
  cudaEvent_t last_in;  // completion of the last upload (null: none)
};

// At a sync point: the library's stream waits for the inputs the following
// work needs, and the outputs final at this point are copied out on the
// download stream.
int xfer_hook(dsg_ctx *ctx, int point, void *arg) {
  const HostXfer &x = *static_cast<const HostXfer *>(arg);
  if (x.need[point]) DSG_CK(ctx, cudaStreamWaitEvent(ctx->stream, ctx->xfer_in_ev[point], 0));
  bool any = false;
  for (int q = 0; q < x.n_out; q++) any = any || last_write(x.out_fields[q]) == point;
  if (!any) return DSG_OK;
  const size_t bytes = ctx->fine().count() * sizeof(double);
  DSG_CK(ctx, cudaEventRecord(ctx->xfer_out_ev[point], ctx->stream));
  DSG_CK(ctx, cudaStreamWaitEvent(ctx->xfer_out, ctx->xfer_out_ev[point], 0));
  // the uploads gate the step and the downloads only its end: the link is
  // left to the uploads until they are all in
  if (x.last_in) DSG_CK(ctx, cudaStreamWaitEvent(ctx->xfer_out, x.last_in, 0));
  for (int q = 0; q < x.n_out; q++)
    if (last_write(x.out_fields[q]) == point)
      DSG_CK(ctx, cudaMemcpyAsync(x.out_host[q], ctx->f[x.out_fields[q]], bytes, cudaMemcpyDeviceToHost,
                                  ctx->xfer_out));
  return DSG_OK;
}

}  // namespace

extern "C" {

int dsg_step(dsg_ctx *ctx, int t, dsg_mg_stats *stats) {
  if (!ctx) return DSG_E_ARG;
  return step_phases(ctx, t, stats);
}

int dsg_step_host(dsg_ctx *ctx, int t, dsg_mg_stats *stats, int n_in, const int *in_fields,
                  const double *const *in_host, int n_out, const int *out_fields, double *const *out_host) {
  if (!ctx) return DSG_E_ARG;
  if (n_in < 0 || n_out < 0 || (n_in > 0 && (!in_fields || !in_host)) || (n_out > 0 && (!out_fields || !out_host)))
    return dsg::set_error(ctx, DSG_E_ARG, "dsg_step_host: bad field lists");
  for (int q = 0; q < n_in; q++)
    if (in_fields[q] < 0 || in_fields[q] >= DSG_NFIELDS || !in_host[q])
      return dsg::set_error(ctx, DSG_E_ARG, "dsg_step_host: bad input %d (field %d)", q, in_fields[q]);
  for (int q = 0; q < n_out; q++)
    if (out_fields[q] < 0 || out_fields[q] >= DSG_NFIELDS || !out_host[q])
      return dsg::set_error(ctx, DSG_E_ARG, "dsg_step_host: bad output %d (field %d)", q, out_fields[q]);
  int rc = xfer_resources(ctx);
  if (rc) return rc;
  const size_t bytes = ctx->fine().count() * sizeof(double);
  HostXfer x{n_in, n_out, in_fields, out_fields, out_host, {}, nullptr};
  // the uploads start after the work already queued on the library's stream,
  // in the order the step needs them, one event after each sync point's group
  DSG_CK(ctx, cudaEventRecord(ctx->xfer_start, ctx->stream));
  DSG_CK(ctx, cudaStreamWaitEvent(ctx->xfer_in, ctx->xfer_start, 0));
  DSG_CK(ctx, cudaStreamWaitEvent(ctx->xfer_out, ctx->xfer_start, 0));
  int late[3], n_late = 0;  // off-diagonal stresses that arrive after csf
  for (int p = 0; p < dsg_ctx::kSyncPoints; p++) {
    for (int q = 0; q < n_in; q++)
      if (first_touch(ctx, in_fields[q]) == p) {
        const int f = in_fields[q];
        if (p == SP_CSF && (f == DSG_F_S12 || f == DSG_F_S13 || f == DSG_F_S23)) {
          if (n_late < 3) late[n_late++] = q;
          continue;
        }
        DSG_CK(ctx, cudaMemcpyAsync(ctx->f[f], in_host[q], bytes, cudaMemcpyHostToDevice, ctx->xfer_in));
        x.need[p] = true;
      }
    if (x.need[p]) {
      DSG_CK(ctx, cudaEventRecord(ctx->xfer_in_ev[p], ctx->xfer_in));
      x.last_in = ctx->xfer_in_ev[p];
    }
    if (p == SP_CSF && n_late > 0) {
      // in chunks of planes, so that the momentum phase starts on the first
      const size_t plane = (size_t)ctx->nx * ctx->ny;
      const int nch = dsg_ctx::kSChunks;
      for (int c = 0; c <= nch; c++) ctx->s_chunk_k[c] = 1 + (int)((long long)c * ctx->nz / nch);
      for (int c = 0; c < nch; c++) {
        const size_t off = (size_t)(ctx->s_chunk_k[c] - 1) * plane;
        const size_t cnt = (size_t)(ctx->s_chunk_k[c + 1] - ctx->s_chunk_k[c]) * plane;
        for (int m = 0; m < n_late; m++)
          DSG_CK(ctx, cudaMemcpyAsync(ctx->f[in_fields[late[m]]] + off, in_host[late[m]] + off,
                                      cnt * sizeof(double), cudaMemcpyHostToDevice, ctx->xfer_in));
        DSG_CK(ctx, cudaEventRecord(ctx->s_chunk_ev[c], ctx->xfer_in));
      }
      ctx->s_chunks = nch;
      x.last_in = ctx->s_chunk_ev[nch - 1];
    }
  }
  ctx->sync_hook = xfer_hook;
  ctx->sync_arg = &x;
  rc = step_phases(ctx, t, stats);
  ctx->sync_hook = nullptr;
  ctx->sync_arg = nullptr;
  ctx->s_chunks = 0;
  // no copy stays in flight into or out of the caller's buffers, also on errors
  const cudaError_t e1 = cudaStreamSynchronize(ctx->xfer_in);
  const cudaError_t e2 = cudaStreamSynchronize(ctx->xfer_out);
  const cudaError_t e3 = cudaStreamSynchronize(ctx->stream);
  if (rc) return rc;
  if (e1 != cudaSuccess) return dsg::cuda_fail(ctx, e1, "dsg_step_host uploads");
  if (e2 != cudaSuccess) return dsg::cuda_fail(ctx, e2, "dsg_step_host downloads");
  if (e3 != cudaSuccess) return dsg::cuda_fail(ctx, e3, "dsg_step_host");
  return DSG_OK;
}

int dsg_liquid_volume(dsg_ctx *ctx, double *out) {
  if (!ctx || !out) return DSG_E_ARG;
  DSG_CK(ctx, dsg::sumfield(ctx->red_out, ctx->red_partials, ctx->f[DSG_F_CC], ctx->fine(), ctx->stream));
  int rc = read_device(ctx, 1);
  if (rc) return rc;
  *out = ctx->red_host[0];
  if (!isfinite(*out)) return dsg::set_error(ctx, DSG_E_NONFINITE, "non-finite liquid volume");
  return DSG_OK;
}

int dsg_max_divergence(dsg_ctx *ctx, double *out) {
  if (!ctx || !out) return DSG_E_ARG;
  const double hi2 = 1.0 / (ctx->s.h * ctx->s.h);
  DSG_CK(ctx, dsg::divmax(ctx->red_out, ctx->red_partials, ctx->f[DSG_F_U], ctx->f[DSG_F_V], ctx->f[DSG_F_W], hi2,
                          ctx->fine(), ctx->stream));
  int rc = read_device(ctx, 1);
  if (rc) return rc;
  *out = ctx->s.h * ctx->red_host[0];
  return DSG_OK;
}

int dsg_relres(dsg_ctx *ctx, double *out) {
  if (!ctx || !out) return DSG_E_ARG;
  return relres_host(ctx, out);
}

int dsg_profile_enable(dsg_ctx *ctx, int on) {
  if (!ctx) return DSG_E_ARG;
  DSG_CK(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->prof = on != 0;
  ctx->prof_used = 0;
  ctx->prof_relax_calls = 0;
  ctx->prof_relax_bytes = 0.0;
  ctx->phase_used = 0;
  ctx->prof_graph_relax_ms = 0.0;
  ctx->prof_launch0 = dsg::g_launches.load();
  return DSG_OK;
}

int dsg_profile_read(dsg_ctx *ctx, dsg_profile *out) {
  if (!ctx || !out) return DSG_E_ARG;
  DSG_CK(ctx, cudaStreamSynchronize(ctx->stream));
  double ms = 0.0;
  for (size_t q = 0; q + 1 < ctx->prof_used; q += 2) {
    float x = 0.f;
    DSG_CK(ctx, cudaEventElapsedTime(&x, ctx->prof_ev[q], ctx->prof_ev[q + 1]));
    ms += x;
  }
  out->launches = dsg::g_launches.load() - ctx->prof_launch0;
  out->relax_calls = ctx->prof_relax_calls;
  out->relax_ms = ms + ctx->prof_graph_relax_ms;
  out->relax_bytes = ctx->prof_relax_bytes;
  out->relax_bits = ctx->prof_relax_bits;
  for (int p = 0; p < 6; p++) out->phase_ms[p] = 0.0;
  for (size_t q = 0; q + 1 < ctx->phase_used; q++) {
    const int id = ctx->phase_id[q];
    if (id < 0 || id > 5) continue;
    float x = 0.f;
    DSG_CK(ctx, cudaEventElapsedTime(&x, ctx->phase_ev[q], ctx->phase_ev[q + 1]));
    out->phase_ms[id] += x;
  }
  return DSG_OK;
}

int64_t dsg_launch_count(void) { return dsg::g_launches.load(); }

int dsg_attach_net(dsg_ctx *ctx, dsg_net *net, int record) {
  if (!ctx) return dsg::set_error(nullptr, DSG_E_ARG, "null context");
  ctx->net = net;
  ctx->net_record = net ? record : 0;
  return DSG_OK;
}

}  // extern "C"
