// batch.cu -- the mixed-precision pressure solve of many ensemble members as
// one batched solve (no reference counterpart: main.f solves one case).
//
// Every pass of the FP32 multigrid (a colour sweep, a residual restriction, a
// prolongation, the coarse tail, the FP64 defect and correction) is one launch
// over all members that take part in it: the launch's virtual blocks are the
// concatenation of each member's own grid, and a block finds its member by a
// binary search over the launch's block bases (an entry per member: its block
// range, its own grid, its arrays and scalars).  The per-cell code is the same
// block body the standalone kernels run (mg32_cells.cuh), with the block index
// the block has inside its member's grid, so every member gets exactly the
// bits of its standalone solve.  Members align at their finest level (depth
// 0); a member whose multigrid has fewer levels, or whose coarse tail starts
// higher, has no entry in the deeper launches.
//
// The solve is the standalone one per member: FP32 coefficient hierarchy and
// FP32 full-multigrid start, then outer iterations of k FP32 V-cycles, FP64
// correction and FP64 defect, with k from the member's own measured reduction
// per V-cycle.  A member takes part in V-cycle q of an outer iteration only if
// q < k (a device gate array read by every block), so converged members are
// masked on the device without a host round trip inside the iteration.  The
// start and each outer iteration of K V-cycles (K = the largest k) are
// captured once as CUDA graphs and replayed; the host reads all members'
// defect norms with one copy per outer iteration.
//
// The coarse tail (one block per member running every level of at most a
// threshold of nodes) computes the same bits as one launch per pass, and in a
// batch the members' tails run side by side on separate SMs; the batch picks
// its own threshold.  Block shapes of the sweep, restriction and prolongation
// passes are free as well (cells of one pass are independent).  An autotuner
// times both on the members' own arrays and keeps the fastest; the
// reductions keep their fixed shape, which fixes their summation order.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <utility>
#include <vector>

#include "mg32_cells.cuh"

namespace dsg {
namespace {

using namespace mg32;
using namespace mixed;

template <class A>
struct Entry {
  unsigned base;        // first virtual block of this member in the launch
  unsigned gx, gy, gz;  // the member's own grid
  int member;           // index into the gate array
  int n;                // sweeps of a relaxation entry (1 otherwise)
  A a;
};

// Argument sets of the batched passes (the parameters of the block bodies).
struct ARelaxSplit { float *u[2]; float *r[2]; const float *cc; Dims d; Split sp; float h2, omega, r1, r2; };
struct ARelax { float *u; const float *rhs, *a, *b, *c, *ei; Dims d; float h2, omega; };
struct ARRSplit {
  float *rhs_c, *u_c;
  const float *ue, *uo, *re, *ro, *cc;
  Dims df;
  Split sp;
  Dims dc;
  float h2i, r1, r2;
};
struct ARR { float *rhs_c, *u_c; const float *u, *rhs, *a, *b, *c; Dims df, dc; float h2i; };
struct AProSplit { float *ue, *uo; const float *uc; Dims df; Split sp; Dims dc; int add; };
struct APro { float *uf; const float *uc; Dims df, dc; int add; };
struct ACorrect { double *p; const float *ev, *od; Dims d; Split sp; int init; };
struct ADefect {
  float *r_ev, *r_od;
  Split sp;
  double *partials;
  const double *p, *rhs, *a, *b, *c, *diag;
  Dims d;
  double h2i;
};
struct AFold { const double *partials; double *out; };
struct AZero { float *p; size_t n; };
struct ATo32 { float *dst; const double *src; size_t n; };
struct AAcf64 { float *a, *b, *c, *ei; const double *a2, *b2, *c2; Dims dc, df; };
struct AAcf32 { float *a, *b, *c, *ei; const float *a2, *b2, *c2; Dims dc, df; };
struct ASplit64 { float *ev, *od; const double *src; Dims d; Split sp; };
struct ARestrSplit { float *uc; const float *re, *ro; Dims dc; Split sp; };
struct ARestr { float *uc; const float *uf; Dims dc, df; };

// Members per batched solve: a launch's entry table travels as a kernel
// parameter (at most 32 KB), so that the member lookup and the members'
// arguments are read through the constant cache like a standalone kernel's.
constexpr int kMaxBatch = 128;

template <class A>
struct Table {
  unsigned total;  // virtual blocks of the launch
  int n;           // entries
  Entry<A> e[kMaxBatch];
};

// A CTA walks the virtual blocks blockIdx.x + i * gridDim.x (one each unless
// the launch is very large).  The member of a virtual block comes from a
// binary search over the entries' block bases; consecutive virtual blocks of
// a CTA mostly belong to the same member.  body(B, G, a) runs one virtual
// block: B its index inside the member's grid G, a the member's arguments.
// Members whose gate is at most q, or whose sweep count is at most `sweep`,
// sit the launch out.
template <class A, class F>
__device__ __forceinline__ void for_member_blocks(const Table<A> &t, const int *__restrict__ gate, int q, int sweep,
                                                  F body) {
  int l = 0;
  unsigned lo = 1, hi = 0;  // block range of the current member (none yet)
  bool run = false;
  for (unsigned vb = blockIdx.x; vb < t.total; vb += gridDim.x) {
    if (vb < lo || vb >= hi) {
      int a = 0, h = t.n - 1;
      while (a < h) {
        const int mid = (a + h + 1) >> 1;
        if (t.e[mid].base <= vb) a = mid;
        else h = mid - 1;
      }
      l = a;
      lo = t.e[l].base;
      hi = l + 1 < t.n ? t.e[l + 1].base : t.total;
      run = gate[t.e[l].member] > q && sweep < t.e[l].n;
    }
    if (!run) continue;
    const Entry<A> &x = t.e[l];
    const unsigned b = vb - lo;
    body(make_uint3(b % x.gx, (b / x.gx) % x.gy, b / (x.gx * x.gy)), make_uint3(x.gx, x.gy, x.gz), x.a);
  }
}

// CTAs of a batched launch of `total` virtual blocks of `threads`: one CTA per
// virtual block up to 64 resident waves.
unsigned launch_grid(unsigned total, unsigned threads) {
  const unsigned per_sm = threads >= 1024 ? 2u : 2048u / threads;
  const unsigned cap = 152u * per_sm * 64u;
  return total < cap ? total : cap;
}

#define BATCH_PARAMS(A) const __grid_constant__ Table<A> t, const int *__restrict__ gate, int q, int sweep
#define FOR_MEMBER_BLOCKS(A) for_member_blocks(t, gate, q, sweep, [&](uint3 B, uint3 G, const A &a)

__global__ void kb_relax32_split(BATCH_PARAMS(ARelaxSplit), int colour) {
  FOR_MEMBER_BLOCKS(ARelaxSplit) {
    b_relax32_split(B, G, a.u[colour], a.u[1 - colour], a.r[colour], a.cc, a.d, a.sp, colour, a.h2, a.omega, a.r1,
                    a.r2);
  });
}

__global__ void kb_relax32(BATCH_PARAMS(ARelax), int colour) {
  FOR_MEMBER_BLOCKS(ARelax) { b_relax32(B, G, a.u, a.rhs, a.a, a.b, a.c, a.ei, a.d, a.h2, a.omega, colour); });
}

__global__ void kb_resid_restrict32_split(BATCH_PARAMS(ARRSplit)) {
  FOR_MEMBER_BLOCKS(ARRSplit) {
    b_resid_restrict32_split(B, G, a.rhs_c, a.u_c, a.ue, a.uo, a.re, a.ro, a.cc, a.df, a.sp, a.dc, a.h2i, a.r1,
                             a.r2);
  });
}

__global__ void kb_resid_restrict32(BATCH_PARAMS(ARR)) {
  FOR_MEMBER_BLOCKS(ARR) { b_resid_restrict32(B, G, a.rhs_c, a.u_c, a.u, a.rhs, a.a, a.b, a.c, a.df, a.dc, a.h2i); });
}

template <bool TRI>
__global__ void kb_prolong32_split(BATCH_PARAMS(AProSplit)) {
  FOR_MEMBER_BLOCKS(AProSplit) { b_prolong32_split<TRI>(B, G, a.ue, a.uo, a.uc, a.df, a.sp, a.dc, a.add); });
}

template <bool TRI>
__global__ void kb_prolong32(BATCH_PARAMS(APro)) {
  FOR_MEMBER_BLOCKS(APro) { b_prolong32<TRI>(B, G, a.uf, a.uc, a.df, a.dc, a.add); });
}

// One virtual block per member; TailArgs is large, so the block reads it in
// place instead of copying it.
__global__ void __launch_bounds__(kTailThreads, 1) kb_vtail32(const Entry<TailArgs> *__restrict__ e, unsigned total,
                                                                const int *__restrict__ gate, int q, int sweep) {
  for (unsigned vb = blockIdx.x; vb < total; vb += gridDim.x) {
    const Entry<TailArgs> &x = e[vb];
    if (gate[x.member] <= q || sweep >= x.n) continue;
    tail_body(x.a);
  }
}

__global__ void kb_correct64(BATCH_PARAMS(ACorrect)) {
  FOR_MEMBER_BLOCKS(ACorrect) { b_correct64(B, G, a.p, a.ev, a.od, a.d, a.sp, a.init); });
}

__global__ void kb_defect64(BATCH_PARAMS(ADefect)) {
  FOR_MEMBER_BLOCKS(ADefect) {
    b_defect64(B, G, a.r_ev, a.r_od, a.sp, a.partials, a.p, a.rhs, a.a, a.b, a.c, a.diag, a.d, a.h2i);
  });
}

__global__ void kb_fold2(BATCH_PARAMS(AFold)) {
  FOR_MEMBER_BLOCKS(AFold) { b_fold2(B, G, a.partials, a.out); });
}

__global__ void kb_zero32(BATCH_PARAMS(AZero)) {
  FOR_MEMBER_BLOCKS(AZero) {
    for (size_t i = (size_t)B.x * blockDim.x + threadIdx.x; i < a.n; i += (size_t)G.x * blockDim.x) a.p[i] = 0.f;
  });
}

__global__ void kb_to32(BATCH_PARAMS(ATo32)) {
  FOR_MEMBER_BLOCKS(ATo32) { b_to32(B, G, a.dst, a.src, a.n); });
}

__global__ void kb_acfromac64to32(BATCH_PARAMS(AAcf64)) {
  FOR_MEMBER_BLOCKS(AAcf64) { b_acfromac64to32(B, G, a.a, a.b, a.c, a.ei, a.a2, a.b2, a.c2, a.dc, a.df); });
}

__global__ void kb_acfromac32(BATCH_PARAMS(AAcf32)) {
  FOR_MEMBER_BLOCKS(AAcf32) { b_acfromac32(B, G, a.a, a.b, a.c, a.ei, a.a2, a.b2, a.c2, a.dc, a.df); });
}

__global__ void kb_split_from64(BATCH_PARAMS(ASplit64)) {
  FOR_MEMBER_BLOCKS(ASplit64) { b_split_from64(B, G, a.ev, a.od, a.src, a.d, a.sp); });
}

__global__ void kb_restrict32_split(BATCH_PARAMS(ARestrSplit)) {
  FOR_MEMBER_BLOCKS(ARestrSplit) { b_restrict32_split(B, G, a.uc, a.re, a.ro, a.dc, a.sp); });
}

__global__ void kb_restrict32(BATCH_PARAMS(ARestr)) {
  FOR_MEMBER_BLOCKS(ARestr) { b_restrict32(B, G, a.uc, a.uf, a.dc, a.df); });
}

#undef FOR_MEMBER_BLOCKS
#undef BATCH_PARAMS

// Kernel parameters are limited to 32764 bytes.
static_assert(sizeof(Table<ARelaxSplit>) <= 32000 && sizeof(Table<ARRSplit>) <= 32000 &&
                  sizeof(Table<ADefect>) <= 32000 && sizeof(Table<AAcf64>) <= 32000 &&
                  sizeof(Table<AAcf32>) <= 32000 && sizeof(Table<ACorrect>) <= 32000,
              "batched entry table exceeds the kernel parameter space");

// ---- host side ---------------------------------------------------------------

enum Kind {
  K_RELAX_SPLIT, K_RELAX, K_RR_SPLIT, K_RR, K_PRO_SPLIT, K_PRO, K_TAIL, K_CORRECT, K_DEFECT, K_FOLD, K_ZERO,
  K_TO32, K_ACF64, K_ACF32, K_SPLIT64, K_RESTR_SPLIT, K_RESTR, K_KINDS
};

// Kinds whose block shape the autotuner may change (independent cells).
inline bool tunable(int k) {
  return k == K_RELAX_SPLIT || k == K_RELAX || k == K_RR_SPLIT || k == K_RR || k == K_PRO_SPLIT || k == K_PRO;
}

// Candidate block shapes of the tunable passes.
const dim3 kShapes[] = {dim3(32, 4), dim3(32, 8), dim3(64, 4), dim3(32, 16), dim3(64, 8), dim3(128, 2), dim3(128, 4),
                        dim3(256, 1)};
constexpr int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);

const dim3 kDefaultShape(32, 4);

dim3 default_shape(int kind) { return kind == K_RELAX_SPLIT ? dim3(32, 8) : kDefaultShape; }

unsigned cdiv(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

// One batched launch of a plan.
struct Launch {
  int kind;
  std::vector<unsigned char> blob;  // the entry table (a kernel parameter)
  size_t off;       // coarse tail: byte offset of its entry table in the device table buffer
  int n;            // entries
  unsigned blocks;  // total virtual blocks
  dim3 blk;
  int q, sweep, colour, tri;
  int gate;         // 0: the all-ones gate, 1: the per-member V-cycle counts
  int slot;         // tuning slot, -1 if not tunable
};

struct MemberPlan {
  dsg_ctx *c;
  int ng, jt;  // levels, top level of the member's tail in the batch
};

}  // namespace

// The batched solve of a group of ensemble members (owned by dsg_ensemble).
struct BatchSolve {
  std::vector<dsg_ctx *> m;
  cudaStream_t st = nullptr;
  cudaEvent_t ev_join = nullptr;
  std::vector<cudaEvent_t> ev_member;
  std::vector<unsigned char> tab;  // host image of the coarse-tail entry tables
  void *tab_dev = nullptr;
  size_t tab_cap = 0;
  int *gate_ones = nullptr, *gate_inner = nullptr;  // device
  int *gate_host = nullptr;                          // pinned
  double *norms_dev = nullptr, *norms_host = nullptr;
  std::vector<Launch> start;
  std::vector<std::vector<Launch>> iter;  // [K] one outer iteration of K V-cycles
  cudaGraphExec_t g_start = nullptr;
  std::vector<cudaGraphExec_t> g_iter;
  long long kernels_start = 0;
  std::vector<long long> kernels_iter;
  // Levels of at most this many nodes run in the per-member single-block tail
  // (chosen by the autotuner).
  long long tail_nodes = 42LL * 42 * 42;
  std::vector<int> key;  // sweep counts and tail threshold the plans were built for
  // tuning slots: a tunable pass is identified by its kind and the level each
  // member runs it on, so the same pass in any plan shares one block shape
  std::vector<std::pair<int, std::vector<int>>> slot_keys;
  std::vector<dim3> slot_shape;
};

namespace {

template <class A>
struct TableBuilder {
  std::vector<Entry<A>> e;
  unsigned blocks = 0;
  void add(int member, dim3 grid, int nsweep, const A &a) {
    Entry<A> x;
    memset(&x, 0, sizeof x);
    x.base = blocks;
    x.gx = grid.x;
    x.gy = grid.y;
    x.gz = grid.z;
    x.member = member;
    x.n = nsweep;
    x.a = a;
    e.push_back(x);
    blocks += grid.x * grid.y * grid.z;
  }
};

// Grid of one member for a pass of kind k with block shape blk (for the
// restrictions d is the coarse level).
dim3 grid_of(int k, const Dims &d, dim3 blk) {
  switch (k) {
    case K_RELAX_SPLIT: {
      const int hx = (d.nx - 2) >> 1;
      return dim3(cdiv(hx, 2 * blk.x), cdiv(d.ny - 2, blk.y), d.nz - 2);
    }
    case K_RELAX: {
      const int half = (d.nx - 2 + 1) / 2;
      return dim3(cdiv(half, blk.x), cdiv(d.ny - 2, blk.y), d.nz - 2);
    }
    case K_PRO_SPLIT: {
      const int hx = (d.nx - 2) >> 1;
      return dim3(cdiv(hx, blk.x), cdiv(d.ny - 2, blk.y), d.nz - 2);
    }
    default:  // interior grid of d
      return dim3(cdiv(d.nx - 2, blk.x), cdiv(d.ny - 2, blk.y), d.nz - 2);
  }
}

struct Planner {
  BatchSolve &b;
  std::vector<MemberPlan> mp;
  explicit Planner(BatchSolve &bs) : b(bs) {
    for (dsg_ctx *c : b.m) mp.push_back(MemberPlan{c, c->ng, batch_tail_top(c, b.tail_nodes)});
  }

  // Top level of a member's tail in the batch: the largest level below the
  // finest with at most `nodes` nodes (at least level 1).
  static int batch_tail_top(const dsg_ctx *c, long long nodes) {
    int top = 1;
    for (int l = 1; l < c->ng && l <= kTailMaxLevels; l++)
      if ((long long)c->lnx[l] * c->lny[l] * c->lnz[l] <= nodes) top = l;
    return top;
  }

  // Tuning slot of a pass of `kind` run on levels lv (one per member, 0: none).
  int slot_of(int kind, const std::vector<int> &lv) {
    for (size_t q = 0; q < b.slot_keys.size(); q++)
      if (b.slot_keys[q].first == kind && b.slot_keys[q].second == lv) return (int)q;
    b.slot_keys.emplace_back(kind, lv);
    b.slot_shape.push_back(default_shape(kind));
    return (int)b.slot_keys.size() - 1;
  }

  template <class A>
  void emit(std::vector<Launch> &out, int kind, TableBuilder<A> &t, dim3 blk, int q, int sweep, int colour, int tri,
            int gate, int slot) {
    if (t.e.empty()) return;
    const size_t bytes = t.e.size() * sizeof(Entry<A>);
    Launch L{kind, {}, 0, (int)t.e.size(), t.blocks, blk, q, sweep, colour, tri, gate, slot};
    if (kind == K_TAIL) {
      const size_t align = 16;
      L.off = (b.tab.size() + align - 1) / align * align;
      b.tab.resize(L.off + bytes);
      memcpy(b.tab.data() + L.off, t.e.data(), bytes);
    } else {
      L.blob.resize(bytes);
      memcpy(L.blob.data(), t.e.data(), bytes);
    }
    out.push_back(std::move(L));
  }

  // Split member levels lv into those on the finest level and the others.
  void split_levels(const std::vector<int> &lv, int min_level, std::vector<int> &ls, std::vector<int> &ln) {
    ls.assign(lv.size(), 0);
    ln.assign(lv.size(), 0);
    for (size_t i = 0; i < mp.size(); i++)
      if (lv[i] >= min_level) (lv[i] == mp[i].ng ? ls : ln)[i] = lv[i];
  }

  // Relaxation of level lv[i] (0: skip) of every member, nsw[i] sweeps.
  void relax(std::vector<Launch> &out, const std::vector<int> &lv, const std::vector<int> &nsw, int q, int gate) {
    int maxn = 0;
    for (size_t i = 0; i < mp.size(); i++)
      if (lv[i] > 0) maxn = std::max(maxn, nsw[i]);
    if (maxn == 0) return;
    std::vector<int> ls, ln;
    split_levels(lv, 1, ls, ln);
    const int slot_s = slot_of(K_RELAX_SPLIT, ls), slot_n = slot_of(K_RELAX, ln);
    const dim3 bs = b.slot_shape[slot_s], bn = b.slot_shape[slot_n];
    TableBuilder<ARelaxSplit> ts;
    TableBuilder<ARelax> tn;
    for (size_t i = 0; i < mp.size(); i++) {
      const int l = lv[i];
      if (l <= 0 || nsw[i] <= 0) continue;
      dsg_ctx *c = mp[i].c;
      const Dims d = c->level(l);
      if (l == c->ng) {
        FineSplit f = fine_split(c);
        float r1, r2;
        phase_coefs(c, &r1, &r2);
        ARelaxSplit a{{f.u[0], f.u[1]}, {f.r[0], f.r[1]}, c->lv32[l][A32], d,
                      Split{(d.nx - 2) >> 1, d.ny - 2, d.nz - 2}, level_h2(c, l), omega32(c), r1, r2};
        ts.add((int)i, grid_of(K_RELAX_SPLIT, d, bs), nsw[i], a);
      } else {
        float **L = c->lv32[l];
        ARelax a{L[U32], L[RHS32], L[A32], L[B32], L[C32], L[EI32], d, level_h2(c, l), omega32(c)};
        tn.add((int)i, grid_of(K_RELAX, d, bn), nsw[i], a);
      }
    }
    for (int s = 0; s < maxn; s++)
      for (int colour = 0; colour < 2; colour++) {
        emit(out, K_RELAX_SPLIT, ts, bs, q, s, colour, 0, gate, slot_s);
        emit(out, K_RELAX, tn, bn, q, s, colour, 0, gate, slot_n);
      }
  }

  // Residual of level lv[i] restricted into level lv[i]-1.
  void resid_restrict(std::vector<Launch> &out, const std::vector<int> &lv, int q, int gate) {
    std::vector<int> ls, ln;
    split_levels(lv, 2, ls, ln);
    const int slot_s = slot_of(K_RR_SPLIT, ls), slot_n = slot_of(K_RR, ln);
    const dim3 bs = b.slot_shape[slot_s], bn = b.slot_shape[slot_n];
    TableBuilder<ARRSplit> ts;
    TableBuilder<ARR> tn;
    for (size_t i = 0; i < mp.size(); i++) {
      const int l = lv[i];
      if (l <= 1) continue;
      dsg_ctx *c = mp[i].c;
      const Dims df = c->level(l), dc = c->level(l - 1);
      float **L = c->lv32[l], **Lc = c->lv32[l - 1];
      if (l == c->ng) {
        FineSplit f = fine_split(c);
        float r1, r2;
        phase_coefs(c, &r1, &r2);
        ARRSplit a{Lc[RHS32], Lc[U32], f.u[0], f.u[1], f.r[0], f.r[1], L[A32], df,
                   Split{(df.nx - 2) >> 1, df.ny - 2, df.nz - 2}, dc, 1.0f / level_h2(c, l), r1, r2};
        ts.add((int)i, grid_of(K_RR_SPLIT, dc, bs), 1, a);
      } else {
        ARR a{Lc[RHS32], Lc[U32], L[U32], L[RHS32], L[A32], L[B32], L[C32], df, dc, 1.0f / level_h2(c, l)};
        tn.add((int)i, grid_of(K_RR, dc, bn), 1, a);
      }
    }
    emit(out, K_RR_SPLIT, ts, bs, q, 0, 0, 0, gate, slot_s);
    emit(out, K_RR, tn, bn, q, 0, 0, 0, gate, slot_n);
  }

  // Level lv[i] = (add 0) or += (add 1) the prolonged correction of level lv[i]-1.
  void prolong(std::vector<Launch> &out, const std::vector<int> &lv, int add, int q, int gate) {
    std::vector<int> ls, ln;
    split_levels(lv, 2, ls, ln);
    const int slot_s = slot_of(K_PRO_SPLIT, ls), slot_n = slot_of(K_PRO, ln);
    const dim3 bs = b.slot_shape[slot_s], bn = b.slot_shape[slot_n];
    TableBuilder<AProSplit> ts;
    TableBuilder<APro> tn;
    const int tri = tri32(mp[0].c);
    for (size_t i = 0; i < mp.size(); i++) {
      const int l = lv[i];
      if (l <= 1) continue;
      dsg_ctx *c = mp[i].c;
      const Dims df = c->level(l), dc = c->level(l - 1);
      if (l == c->ng) {
        FineSplit f = fine_split(c);
        AProSplit a{f.u[0], f.u[1], c->lv32[l - 1][U32], df, Split{(df.nx - 2) >> 1, df.ny - 2, df.nz - 2}, dc,
                    add};
        ts.add((int)i, grid_of(K_PRO_SPLIT, df, bs), 1, a);
      } else {
        APro a{c->lv32[l][U32], c->lv32[l - 1][U32], df, dc, add};
        tn.add((int)i, grid_of(K_PRO, df, bn), 1, a);
      }
    }
    emit(out, K_PRO_SPLIT, ts, bs, q, 0, 0, tri, gate, slot_s);
    emit(out, K_PRO, tn, bn, q, 0, 0, tri, gate, slot_n);
  }

  // One V-cycle of every member from level top[i] (0: not taking part), as
  // vcycle32 in the standalone solve.
  void vcycle(std::vector<Launch> &out, const std::vector<int> &top, int q, int gate) {
    const size_t n = mp.size();
    std::vector<int> jt(n, 0);
    int depth = 0;
    for (size_t i = 0; i < n; i++) {
      if (top[i] <= 0) continue;
      jt[i] = std::min(mp[i].jt, top[i]);
      depth = std::max(depth, top[i] - jt[i]);
    }
    for (int e = 0; e < depth; e++) {
      std::vector<int> lv(n, 0), nsw(n, 0);
      for (size_t i = 0; i < n; i++) {
        const int l = top[i] - e;
        if (top[i] > 0 && l > jt[i] && l >= 2) {
          lv[i] = l;
          nsw[i] = pre32(mp[i].c, l);
        }
      }
      relax(out, lv, nsw, q, gate);
      resid_restrict(out, lv, q, gate);
    }
    TableBuilder<TailArgs> tt;
    for (size_t i = 0; i < n; i++) {
      if (top[i] <= 0) continue;
      TailArgs A;
      tail_args(mp[i].c, jt[i], &A);
      tt.add((int)i, dim3(1, 1, 1), 1, A);
    }
    emit(out, K_TAIL, tt, dim3(kTailThreads), q, 0, 0, 0, gate, -1);
    for (int e = depth - 1; e >= 0; e--) {
      std::vector<int> lv(n, 0), nsw(n, 0);
      for (size_t i = 0; i < n; i++) {
        const int l = top[i] - e;
        if (top[i] > 0 && l > jt[i] && l >= 2) {
          lv[i] = l;
          nsw[i] = post32(mp[i].c, l);
        }
      }
      prolong(out, lv, 1, q, gate);
      relax(out, lv, nsw, q, gate);
    }
  }

  // FP64 correction p (+)= e and the FP64 defect with its norms.
  void correct_defect(std::vector<Launch> &out, int init, int gate, double *norms_dev) {
    TableBuilder<ACorrect> tc;
    TableBuilder<ADefect> td;
    TableBuilder<AFold> tf;
    for (size_t i = 0; i < mp.size(); i++) {
      dsg_ctx *c = mp[i].c;
      const Dims d = c->fine();
      const Split sp{(d.nx - 2) >> 1, d.ny - 2, d.nz - 2};
      FineSplit f = fine_split(c);
      double **L = c->lv[c->ng];
      tc.add((int)i, grid_of(K_CORRECT, d, kDefaultShape), 1, ACorrect{L[1], f.u[0], f.u[1], d, sp, init});
      const double h1 = c->s.lengthsize / (d.nx - 2);
      td.add((int)i, dim3(kRedBlocks), 1,
             ADefect{f.r[0], f.r[1], sp, c->red_partials, L[1], L[3], L[4], L[5], L[6], c->diag64, d,
                     1.0 / (h1 * h1)});
      tf.add((int)i, dim3(1), 1, AFold{c->red_partials, norms_dev + 2 * i});
    }
    emit(out, K_CORRECT, tc, kDefaultShape, 0, 0, 0, 0, gate, -1);
    emit(out, K_DEFECT, td, dim3(kRedThreads), 0, 0, 0, 0, gate, -1);
    emit(out, K_FOLD, tf, dim3(kRedThreads), 0, 0, 0, 0, gate, -1);
  }

  // coef_hierarchy32 + fmg32 + correction + first defect of every member.
  void plan_start(std::vector<Launch> &out, double *norms_dev) {
    const size_t n = mp.size();
    int maxng = 0;
    for (auto &x : mp) maxng = std::max(maxng, x.ng);
    {  // FP32 fine cc, coarse coefficients
      TableBuilder<ATo32> t;
      for (size_t i = 0; i < n; i++) {
        dsg_ctx *c = mp[i].c;
        const size_t cnt = c->fine().count();
        t.add((int)i, dim3(std::min(cdiv(cnt, 256), 8192u)), 1, ATo32{c->lv32[c->ng][A32], c->lv[c->ng][0], cnt});
      }
      emit(out, K_TO32, t, dim3(256), 0, 0, 0, 0, 0, -1);
    }
    {
      TableBuilder<AAcf64> t;
      for (size_t i = 0; i < n; i++) {
        dsg_ctx *c = mp[i].c;
        double **F = c->lv[c->ng];
        float **C = c->lv32[c->ng - 1];
        const Dims dc = c->level(c->ng - 1), df = c->fine();
        t.add((int)i, dim3(cdiv(dc.nx, 32), cdiv(dc.ny, 4), dc.nz), 1,
              AAcf64{C[A32], C[B32], C[C32], C[EI32], F[4], F[5], F[6], dc, df});
      }
      emit(out, K_ACF64, t, kDefaultShape, 0, 0, 0, 0, 0, -1);
    }
    for (int e = 2; e < maxng; e++) {  // level ng - e from level ng - e + 1
      TableBuilder<AAcf32> t;
      for (size_t i = 0; i < n; i++) {
        dsg_ctx *c = mp[i].c;
        const int g = c->ng - e;
        if (g < 1) continue;
        float **C = c->lv32[g], **Fi = c->lv32[g + 1];
        const Dims dc = c->level(g), df = c->level(g + 1);
        t.add((int)i, dim3(cdiv(dc.nx, 32), cdiv(dc.ny, 4), dc.nz), 1,
              AAcf32{C[A32], C[B32], C[C32], C[EI32], Fi[A32], Fi[B32], Fi[C32], dc, df});
      }
      emit(out, K_ACF32, t, kDefaultShape, 0, 0, 0, 0, 0, -1);
    }
    {  // fmg32: split fine rhs, restrict it down, zero the coarsest correction
      TableBuilder<ASplit64> t;
      for (size_t i = 0; i < n; i++) {
        dsg_ctx *c = mp[i].c;
        FineSplit f = fine_split(c);
        const Dims d = c->fine();
        t.add((int)i, grid_of(K_SPLIT64, d, kDefaultShape), 1,
              ASplit64{f.r[0], f.r[1], c->lv[c->ng][3], d, Split{(d.nx - 2) >> 1, d.ny - 2, d.nz - 2}});
      }
      emit(out, K_SPLIT64, t, kDefaultShape, 0, 0, 0, 0, 0, -1);
    }
    {
      TableBuilder<ARestrSplit> t;
      for (size_t i = 0; i < n; i++) {
        dsg_ctx *c = mp[i].c;
        FineSplit f = fine_split(c);
        const Dims dc = c->level(c->ng - 1), df = c->fine();
        t.add((int)i, grid_of(K_RESTR_SPLIT, dc, kDefaultShape), 1,
              ARestrSplit{c->lv32[c->ng - 1][RHS32], f.r[0], f.r[1], dc,
                          Split{(df.nx - 2) >> 1, df.ny - 2, df.nz - 2}});
      }
      emit(out, K_RESTR_SPLIT, t, kDefaultShape, 0, 0, 0, 0, 0, -1);
    }
    for (int e = 2; e < maxng; e++) {
      TableBuilder<ARestr> t;
      for (size_t i = 0; i < n; i++) {
        dsg_ctx *c = mp[i].c;
        const int g = c->ng - e;
        if (g < 1) continue;
        t.add((int)i, grid_of(K_RESTR, c->level(g), kDefaultShape), 1,
              ARestr{c->lv32[g][RHS32], c->lv32[g + 1][RHS32], c->level(g), c->level(g + 1)});
      }
      emit(out, K_RESTR, t, kDefaultShape, 0, 0, 0, 0, 0, -1);
    }
    {
      TableBuilder<AZero> t;
      for (size_t i = 0; i < n; i++) {
        dsg_ctx *c = mp[i].c;
        const size_t cnt = c->level(1).count();
        t.add((int)i, dim3(std::min(cdiv(cnt, 256), 4096u)), 1, AZero{c->lv32[1][U32], cnt});
      }
      emit(out, K_ZERO, t, dim3(256), 0, 0, 0, 0, 0, -1);
    }
    {  // NTOP sweeps on the coarsest level
      std::vector<int> lv(n, 1), nsw(n, 0);
      for (size_t i = 0; i < n; i++) nsw[i] = mp[i].c->s.ntop;
      relax(out, lv, nsw, 0, 0);
    }
    // FMG stages, aligned so that every member reaches its finest level last
    const int stages = maxng - 1;
    for (int k = 0; k < stages; k++) {
      std::vector<int> top(n, 0);
      for (size_t i = 0; i < n; i++) {
        const int j = mp[i].ng - (stages - 1 - k);
        top[i] = j >= 2 ? j : 0;
      }
      prolong(out, top, 0, 0, 0);
      int cycles = 0;
      for (size_t i = 0; i < n; i++)
        if (top[i]) cycles = std::max(cycles, mixed::fmg32_cycles(mp[i].c, top[i]));
      for (int cy = 0; cy < cycles; cy++) {
        std::vector<int> t2(top);
        for (size_t i = 0; i < n; i++)
          if (top[i] && cy >= mixed::fmg32_cycles(mp[i].c, top[i])) t2[i] = 0;
        vcycle(out, t2, 0, 0);
      }
    }
    correct_defect(out, 1, 0, norms_dev);
  }

  // One V-cycle of every member from its finest level, FP32 arrays only (the
  // autotuner's probe: the FP64 state is not touched).
  void plan_probe(std::vector<Launch> &out) {
    std::vector<int> top(mp.size());
    for (size_t i = 0; i < mp.size(); i++) top[i] = mp[i].ng;
    vcycle(out, top, 0, 0);
  }

  // One outer iteration: zero the fine corrections, K V-cycles (member i
  // takes part in V-cycle q while q < its count), FP64 correction and defect.
  void plan_iter(std::vector<Launch> &out, int K, double *norms_dev) {
    const size_t n = mp.size();
    TableBuilder<AZero> t;
    for (size_t i = 0; i < n; i++) {
      dsg_ctx *c = mp[i].c;
      FineSplit f = fine_split(c);
      const size_t cnt = fine_split_bytes(c) / sizeof(float);
      t.add((int)i, dim3(std::min(cdiv(cnt, 256), 4096u)), 1, AZero{f.u[0], cnt});
    }
    emit(out, K_ZERO, t, dim3(256), 0, 0, 0, 0, 1, -1);
    std::vector<int> top(n);
    for (size_t i = 0; i < n; i++) top[i] = mp[i].ng;
    for (int q = 0; q < K; q++) vcycle(out, top, q, 1);
    correct_defect(out, 0, 1, norms_dev);
  }
};

// Launch one batched pass.
template <class A, class K, class... X>
cudaError_t launch_table(K kernel, const Launch &L, const int *gate, cudaStream_t st, X... extra) {
  Table<A> t;
  t.total = L.blocks;
  t.n = L.n;
  memcpy(t.e, L.blob.data(), L.blob.size());
  const unsigned g = launch_grid(L.blocks, L.blk.x * L.blk.y * L.blk.z);
  DSG_COUNT kernel<<<g, L.blk, 0, st>>>(t, gate, L.q, L.sweep, extra...);
  return cudaGetLastError();
}

cudaError_t launch(const BatchSolve &b, const Launch &L, cudaStream_t st) {
  const int *gate = L.gate ? b.gate_inner : b.gate_ones;
  switch (L.kind) {
    case K_RELAX_SPLIT: return launch_table<ARelaxSplit>(kb_relax32_split, L, gate, st, L.colour);
    case K_RELAX: return launch_table<ARelax>(kb_relax32, L, gate, st, L.colour);
    case K_RR_SPLIT: return launch_table<ARRSplit>(kb_resid_restrict32_split, L, gate, st);
    case K_RR: return launch_table<ARR>(kb_resid_restrict32, L, gate, st);
    case K_PRO_SPLIT:
      return L.tri ? launch_table<AProSplit>(kb_prolong32_split<true>, L, gate, st)
                   : launch_table<AProSplit>(kb_prolong32_split<false>, L, gate, st);
    case K_PRO:
      return L.tri ? launch_table<APro>(kb_prolong32<true>, L, gate, st)
                   : launch_table<APro>(kb_prolong32<false>, L, gate, st);
    case K_TAIL: {
      const Entry<TailArgs> *e =
          reinterpret_cast<const Entry<TailArgs> *>(static_cast<const unsigned char *>(b.tab_dev) + L.off);
      DSG_COUNT kb_vtail32<<<L.blocks, L.blk, 0, st>>>(e, L.blocks, gate, L.q, L.sweep);
      return cudaGetLastError();
    }
    case K_CORRECT: return launch_table<ACorrect>(kb_correct64, L, gate, st);
    case K_DEFECT: return launch_table<ADefect>(kb_defect64, L, gate, st);
    case K_FOLD: return launch_table<AFold>(kb_fold2, L, gate, st);
    case K_ZERO: return launch_table<AZero>(kb_zero32, L, gate, st);
    case K_TO32: return launch_table<ATo32>(kb_to32, L, gate, st);
    case K_ACF64: return launch_table<AAcf64>(kb_acfromac64to32, L, gate, st);
    case K_ACF32: return launch_table<AAcf32>(kb_acfromac32, L, gate, st);
    case K_SPLIT64: return launch_table<ASplit64>(kb_split_from64, L, gate, st);
    case K_RESTR_SPLIT: return launch_table<ARestrSplit>(kb_restrict32_split, L, gate, st);
    case K_RESTR: return launch_table<ARestr>(kb_restrict32, L, gate, st);
    default: return cudaErrorInvalidValue;
  }
}

void release_graphs(BatchSolve &b) {
  if (b.g_start) cudaGraphExecDestroy(b.g_start);
  b.g_start = nullptr;
  for (cudaGraphExec_t &g : b.g_iter)
    if (g) cudaGraphExecDestroy(g);
  b.g_iter.clear();
}

// Capture the launches of a plan, then the copy of the norms to the host.
int capture(BatchSolve &b, const std::vector<Launch> &plan, cudaGraphExec_t *out, long long *kernels) {
  cudaError_t e = cudaStreamBeginCapture(b.st, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return set_error(nullptr, DSG_E_CUDA, "batched solve: begin capture: %s", cudaGetErrorString(e));
  const long long l0 = t_launches;
  cudaError_t le = cudaSuccess;
  for (const Launch &L : plan)
    if (le == cudaSuccess) le = launch(b, L, b.st);
  if (le == cudaSuccess)
    le = cudaMemcpyAsync(b.norms_host, b.norms_dev, 2 * b.m.size() * sizeof(double), cudaMemcpyDeviceToHost, b.st);
  *kernels = t_launches - l0;
  g_launches.fetch_sub(*kernels);
  t_launches -= *kernels;
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(b.st, &graph);
  if (le != cudaSuccess || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return set_error(nullptr, DSG_E_CUDA, "batched solve: capture: %s",
                     cudaGetErrorString(le != cudaSuccess ? le : e));
  }
  e = cudaGraphInstantiate(out, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return set_error(nullptr, DSG_E_CUDA, "batched solve: instantiate: %s", cudaGetErrorString(e));
  return DSG_OK;
}

std::vector<int> sweep_key(const BatchSolve &b) {
  std::vector<int> k;
  k.push_back((int)(b.tail_nodes & 0x7fffffff));
  for (dsg_ctx *c : b.m) {
    k.push_back(c->s.ntop);
    for (int l = 1; l <= c->ng; l++) {
      k.push_back(pre32(c, l));
      k.push_back(post32(c, l));
    }
  }
  return k;
}

// Build every plan and its entry tables, upload the tables, capture the graphs.
int build_plans(BatchSolve &b) {
  release_graphs(b);
  b.tab.clear();
  b.start.clear();
  b.iter.assign(dsg_ctx::kMaxInner + 1, {});
  Planner p(b);
  p.plan_start(b.start, b.norms_dev);
  for (int K = 1; K <= dsg_ctx::kMaxInner; K++) p.plan_iter(b.iter[K], K, b.norms_dev);
  if (b.tab.size() > b.tab_cap) {
    if (b.tab_dev) cudaFree(b.tab_dev);
    b.tab_dev = nullptr;
    b.tab_cap = 0;
    cudaError_t e = cudaMalloc(&b.tab_dev, b.tab.size());
    if (e != cudaSuccess) return set_error(nullptr, DSG_E_NOMEM, "batched solve: entry tables (%zu bytes)", b.tab.size());
    b.tab_cap = b.tab.size();
  }
  cudaError_t e = cudaMemcpyAsync(b.tab_dev, b.tab.data(), b.tab.size(), cudaMemcpyHostToDevice, b.st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b.st);
  if (e != cudaSuccess) return set_error(nullptr, DSG_E_CUDA, "batched solve: table upload: %s", cudaGetErrorString(e));
  int rc = capture(b, b.start, &b.g_start, &b.kernels_start);
  if (rc) return rc;
  b.g_iter.assign(dsg_ctx::kMaxInner + 1, nullptr);
  b.kernels_iter.assign(dsg_ctx::kMaxInner + 1, 0);
  for (int K = 1; K <= dsg_ctx::kMaxInner; K++) {
    rc = capture(b, b.iter[K], &b.g_iter[K], &b.kernels_iter[K]);
    if (rc) return rc;
  }
  b.key = sweep_key(b);
  return DSG_OK;
}

int run_graph(BatchSolve &b, cudaGraphExec_t g, long long kernels) {
  cudaError_t e = cudaGraphLaunch(g, b.st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b.st);
  if (e != cudaSuccess) return set_error(nullptr, DSG_E_CUDA, "batched solve: %s", cudaGetErrorString(e));
  g_launches.fetch_add(kernels);
  return DSG_OK;
}

// Time `reps` rounds of one FP32 V-cycle of every member under the current
// tail threshold (direct launches of the probe plan; FP32 scratch only).  The
// probe's coarse-tail table goes to the start of the table buffer; the
// plans' tables there are uploaded again by build_plans before any graph runs.
int time_probe(BatchSolve *b, int reps, float *ms) {
  std::vector<Launch> probe;
  std::vector<unsigned char> saved;
  saved.swap(b->tab);
  Planner p(*b);
  p.plan_probe(probe);
  std::vector<unsigned char> ptab;
  ptab.swap(b->tab);
  b->tab.swap(saved);
  if (ptab.size() > b->tab_cap) return set_error(nullptr, DSG_E_STATE, "autotune: probe tables exceed the table buffer");
  cudaError_t e = ptab.empty() ? cudaSuccess
                               : cudaMemcpyAsync(b->tab_dev, ptab.data(), ptab.size(), cudaMemcpyHostToDevice, b->st);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  for (const Launch &L : probe)
    if (e == cudaSuccess) e = launch(*b, L, b->st);  // warm-up
  if (e == cudaSuccess) e = cudaEventRecord(e0, b->st);
  for (int r = 0; r < reps && e == cudaSuccess; r++)
    for (const Launch &L : probe)
      if (e == cudaSuccess) e = launch(*b, L, b->st);
  if (e == cudaSuccess) e = cudaEventRecord(e1, b->st);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) return set_error(nullptr, DSG_E_CUDA, "autotune probe: %s", cudaGetErrorString(e));
  return DSG_OK;
}

}  // namespace

// ---- entry points used by ensemble.cu ------------------------------------------

// Whether ctx can take part in a batched solve: the mixed mode with the FP32
// full-multigrid start, no network, CUDA graphs on, the coarse tail on and an
// even interior x extent.
int batch_eligible(const dsg_ctx *c, char *why, size_t nwhy) {
  const char *r = nullptr;
  if (c->cfg.mode != DSG_MODE_TOL_MIXED) r = "pressure mode is not DSG_MODE_TOL_MIXED";
  else if (c->net) r = "a network is attached";
  else if (c->cfg.warm_start != 0) r = "the initial guess is not the FP32 full multigrid";
  else if (!c->cfg.use_graphs) r = "CUDA graphs are off";
  else if (c->tail_top < 1) r = "the coarse tail is off";
  else if ((c->nx - 2) & 1) r = "odd interior x extent";
  else if (c->ng < 2) r = "a single multigrid level";
  if (r && why) snprintf(why, nwhy, "%s", r);
  return r ? DSG_E_ARG : DSG_OK;
}

void batch_destroy(BatchSolve *b) {
  if (!b) return;
  if (b->st) cudaStreamSynchronize(b->st);
  release_graphs(*b);
  if (b->tab_dev) cudaFree(b->tab_dev);
  if (b->gate_ones) cudaFree(b->gate_ones);
  if (b->gate_inner) cudaFree(b->gate_inner);
  if (b->norms_dev) cudaFree(b->norms_dev);
  if (b->gate_host) cudaFreeHost(b->gate_host);
  if (b->norms_host) cudaFreeHost(b->norms_host);
  for (cudaEvent_t e : b->ev_member)
    if (e) cudaEventDestroy(e);
  if (b->ev_join) cudaEventDestroy(b->ev_join);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
}

BatchSolve *batch_create(const std::vector<dsg_ctx *> &members, int *rc) {
  *rc = DSG_OK;
  if (members.empty() || members.size() > (size_t)kMaxBatch) {
    *rc = set_error(nullptr, DSG_E_ARG, "batched solve: %zu members (1..%d)", members.size(), kMaxBatch);
    return nullptr;
  }
  for (size_t i = 1; i < members.size(); i++)
    if (tri32(members[i]) != tri32(members[0])) {
      *rc = set_error(nullptr, DSG_E_ARG, "batched solve: members differ in their FP32 prolongation");
      return nullptr;
    }
  BatchSolve *b = new BatchSolve();
  b->m = members;
  const size_t n = members.size();
  auto fail = [&](int code, const char *what, cudaError_t e) {
    *rc = set_error(nullptr, code, "batched solve: %s: %s", what, cudaGetErrorString(e));
    batch_destroy(b);
    return (BatchSolve *)nullptr;
  };
  cudaError_t e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(DSG_E_CUDA, "stream", e);
  if ((e = cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming)) != cudaSuccess)
    return fail(DSG_E_CUDA, "event", e);
  b->ev_member.assign(n, nullptr);
  for (size_t i = 0; i < n; i++)
    if ((e = cudaEventCreateWithFlags(&b->ev_member[i], cudaEventDisableTiming)) != cudaSuccess)
      return fail(DSG_E_CUDA, "event", e);
  if ((e = cudaMalloc(&b->gate_ones, n * sizeof(int))) != cudaSuccess) return fail(DSG_E_NOMEM, "gates", e);
  if ((e = cudaMalloc(&b->gate_inner, n * sizeof(int))) != cudaSuccess) return fail(DSG_E_NOMEM, "gates", e);
  if ((e = cudaMalloc(&b->norms_dev, 2 * n * sizeof(double))) != cudaSuccess) return fail(DSG_E_NOMEM, "norms", e);
  if ((e = cudaMallocHost(&b->gate_host, n * sizeof(int))) != cudaSuccess) return fail(DSG_E_NOMEM, "gates", e);
  if ((e = cudaMallocHost(&b->norms_host, 2 * n * sizeof(double))) != cudaSuccess)
    return fail(DSG_E_NOMEM, "norms", e);
  for (size_t i = 0; i < n; i++) b->gate_host[i] = 1;
  e = cudaMemcpyAsync(b->gate_ones, b->gate_host, n * sizeof(int), cudaMemcpyHostToDevice, b->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
  if (e != cudaSuccess) return fail(DSG_E_CUDA, "gates", e);
  return b;
}

// The pressure solve of every member of the batch, all of whose steps reached
// it (active[i] != 0): each member's stream is joined into the batch stream,
// the batched start and outer iterations run, and each member's stream waits
// for the end.  Per member: stats[i] and mg_rc[i] (DSG_OK,
// DSG_E_NOT_CONVERGED or an error).
int batch_solve(BatchSolve *b, const std::vector<int> &active, std::vector<dsg_mg_stats> &stats,
                std::vector<int> &mg_rc) {
  const size_t n = b->m.size();
  for (size_t i = 0; i < n; i++)
    if (!active[i]) return set_error(nullptr, DSG_E_STATE, "batched solve: member %zu did not reach its solve", i);
  for (size_t i = 0; i < n; i++) {
    mg_rc[i] = DSG_OK;
    dsg_ctx *c = b->m[i];
    cudaError_t e = cudaSuccess;
    if (!c->diag_fresh) {  // coefficients not from this step's abcei: form the defect's diagonal
      double **L = c->lv[c->ng];
      e = dsg::diag_sum(c->diag64, L[4], L[5], L[6], c->fine(), c->stream);
      c->diag_fresh = true;
    }
    // the member's own FP32 hierarchy (side stream) ends before the batch forms it again
    if (e == cudaSuccess && c->coef32_async) e = cudaStreamWaitEvent(c->stream, c->coef_ev, 0);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev_member[i], c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->st, b->ev_member[i], 0);
    if (e != cudaSuccess) return set_error(nullptr, DSG_E_CUDA, "batched solve: join: %s", cudaGetErrorString(e));
  }
  if (b->key != sweep_key(*b) || !b->g_start) {
    int rc = build_plans(*b);
    if (rc) return rc;
  }
  int rc = run_graph(*b, b->g_start, b->kernels_start);
  if (rc) return rc;
  std::vector<double> r(n, 0.0);
  std::vector<int> nv(n, 0), done(n, 0), inner(n, 0);
  for (size_t i = 0; i < n; i++) {
    dsg_ctx *c = b->m[i];
    dsg_mg_stats &s = stats[i];
    memset(&s, 0, sizeof s);
    s.mode = c->cfg.mode;
    s.relres = -1.0;
    s.relres_init = -1.0;
    s.epsdiv = -1.0;
    const double rr = b->norms_host[2 * i], bb = b->norms_host[2 * i + 1];
    if (!isfinite(rr) || !isfinite(bb)) {
      mg_rc[i] = set_error(c, DSG_E_NONFINITE, "non-finite defect norm (%g, %g)", rr, bb);
      done[i] = 1;
      continue;
    }
    r[i] = bb > 0.0 ? sqrt(rr) / sqrt(bb) : sqrt(rr);
    s.relres_init = r[i];
  }
  for (;;) {
    int K = 0;
    for (size_t i = 0; i < n; i++) {
      dsg_ctx *c = b->m[i];
      inner[i] = 0;
      if (done[i] || !(r[i] >= c->cfg.tol && nv[i] < c->cfg.max_vcycles)) continue;
      const int fixed = c->cfg.inner_vcycles;
      int k = fixed > 0 ? (fixed < dsg_ctx::kMaxInner ? fixed : dsg_ctx::kMaxInner) : 2;
      if (fixed <= 0) {
        const double need = log(c->cfg.tol / r[i]) / log(c->rho_est);
        k = (int)ceil(need + 0.1);
        k = k < 1 ? 1 : (k > dsg_ctx::kMaxInner ? dsg_ctx::kMaxInner : k);
      }
      if (k > c->cfg.max_vcycles - nv[i]) k = c->cfg.max_vcycles - nv[i];
      inner[i] = k;
      K = std::max(K, k);
    }
    if (K == 0) break;
    for (size_t i = 0; i < n; i++) b->gate_host[i] = inner[i];
    cudaError_t e = cudaMemcpyAsync(b->gate_inner, b->gate_host, n * sizeof(int), cudaMemcpyHostToDevice, b->st);
    if (e != cudaSuccess) return set_error(nullptr, DSG_E_CUDA, "batched solve: gates: %s", cudaGetErrorString(e));
    rc = run_graph(*b, b->g_iter[K], b->kernels_iter[K]);
    if (rc) return rc;
    for (size_t i = 0; i < n; i++) {
      if (!inner[i]) continue;
      dsg_ctx *c = b->m[i];
      stats[i].fine_sweeps += inner[i] * (pre32(c, c->ng) + post32(c, c->ng));
      nv[i] += inner[i];
      const double rr = b->norms_host[2 * i], bb = b->norms_host[2 * i + 1];
      if (!isfinite(rr) || !isfinite(bb)) {
        mg_rc[i] = set_error(c, DSG_E_NONFINITE, "non-finite defect norm (%g, %g)", rr, bb);
        done[i] = 1;
        continue;
      }
      const double ro = r[i];
      r[i] = bb > 0.0 ? sqrt(rr) / sqrt(bb) : sqrt(rr);
      if (r[i] < ro && r[i] > 0.0) {
        const double obs = pow(r[i] / ro, 1.0 / inner[i]);
        c->rho_est = obs < 0.05 ? 0.05 : (obs > 0.9 ? 0.9 : obs);
      }
    }
  }
  for (size_t i = 0; i < n; i++) {
    dsg_ctx *c = b->m[i];
    cudaError_t e = bc_scalar(c->lv[c->ng][1], c->fine(), b->st);
    if (e != cudaSuccess) return set_error(nullptr, DSG_E_CUDA, "batched solve: bc_scalar: %s", cudaGetErrorString(e));
  }
  cudaError_t e = cudaEventRecord(b->ev_join, b->st);
  if (e != cudaSuccess) return set_error(nullptr, DSG_E_CUDA, "batched solve: %s", cudaGetErrorString(e));
  for (size_t i = 0; i < n; i++) {
    dsg_ctx *c = b->m[i];
    if ((e = cudaStreamWaitEvent(c->stream, b->ev_join, 0)) != cudaSuccess)
      return set_error(nullptr, DSG_E_CUDA, "batched solve: %s", cudaGetErrorString(e));
    if (mg_rc[i]) continue;
    dsg_mg_stats &s = stats[i];
    s.vcycles = nv[i];
    s.relres = r[i];
    s.converged = r[i] < c->cfg.tol;
    mg_rc[i] = mixed_finish(c, &s, &s);
  }
  return DSG_OK;
}

// Autotuner of the batched solve, between steps.  First the coarse-tail
// threshold: one batched FP32 V-cycle is timed per candidate and the fastest
// kept.  Then the block shapes: every tunable launch of an outer iteration of
// one V-cycle is timed with each candidate shape on the members' own FP32
// arrays (scratch between solves: the next solve rewrites every FP32 array
// before reading it) and the fastest shape is kept for its slot.  The plans
// and graphs are rebuilt with the choices.  *slots_tuned: slots timed.
int batch_autotune(BatchSolve *b, int reps, int *slots_tuned) {
  if (!b->g_start) {
    int rc = build_plans(*b);
    if (rc) return rc;
  }
  const size_t n = b->m.size();
  {
    const long long cand[] = {18LL * 18 * 18, 26LL * 26 * 26, 34LL * 34 * 34, 42LL * 42 * 42, 50LL * 50 * 50,
                              66LL * 66 * 66, 82LL * 82 * 82};
    long long best_nodes = b->tail_nodes;
    float best = 1e30f;
    for (long long nodes : cand) {
      b->tail_nodes = nodes;
      float ms = 0.f;
      const size_t slots0 = b->slot_keys.size();
      int rc = time_probe(b, reps, &ms);
      b->slot_keys.resize(slots0);  // probe passes are not plan slots
      b->slot_shape.resize(slots0);
      if (rc) {
        b->tail_nodes = best_nodes;
        build_plans(*b);
        return rc;
      }
      if (ms < best) {
        best = ms;
        best_nodes = nodes;
      }
    }
    b->tail_nodes = best_nodes;
    int rc = build_plans(*b);
    if (rc) return rc;
  }
  for (size_t i = 0; i < n; i++) b->gate_host[i] = dsg_ctx::kMaxInner;
  cudaError_t e = cudaMemcpyAsync(b->gate_inner, b->gate_host, n * sizeof(int), cudaMemcpyHostToDevice, b->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
  if (e != cudaSuccess) return set_error(nullptr, DSG_E_CUDA, "autotune: %s", cudaGetErrorString(e));
  const std::vector<Launch> plan = b->iter[1];
  std::vector<int> seen(b->slot_keys.size(), 0);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  int tuned = 0;
  for (const Launch &L0 : plan) {
    if (e != cudaSuccess) break;
    if (L0.slot < 0 || !tunable(L0.kind) || seen[L0.slot]) continue;
    seen[L0.slot] = 1;
    size_t esz = 0;
    switch (L0.kind) {
      case K_RELAX_SPLIT: esz = sizeof(Entry<ARelaxSplit>); break;
      case K_RELAX: esz = sizeof(Entry<ARelax>); break;
      case K_RR_SPLIT: esz = sizeof(Entry<ARRSplit>); break;
      case K_RR: esz = sizeof(Entry<ARR>); break;
      case K_PRO_SPLIT: esz = sizeof(Entry<AProSplit>); break;
      default: esz = sizeof(Entry<APro>); break;
    }
    float best = 1e30f;
    dim3 best_shape = L0.blk;
    for (int c = 0; c < kNumShapes && e == cudaSuccess; c++) {
      const dim3 blk = kShapes[c];
      Launch L = L0;
      L.blk = blk;
      std::vector<unsigned char> &tab = L.blob;
      unsigned blocks = 0;
      for (int q = 0; q < L.n; q++) {
        unsigned char *p = tab.data() + q * esz;
        Dims d;
        switch (L.kind) {  // the level that sizes the member's grid
          case K_RELAX_SPLIT: d = reinterpret_cast<Entry<ARelaxSplit> *>(p)->a.d; break;
          case K_RELAX: d = reinterpret_cast<Entry<ARelax> *>(p)->a.d; break;
          case K_RR_SPLIT: d = reinterpret_cast<Entry<ARRSplit> *>(p)->a.dc; break;
          case K_RR: d = reinterpret_cast<Entry<ARR> *>(p)->a.dc; break;
          case K_PRO_SPLIT: d = reinterpret_cast<Entry<AProSplit> *>(p)->a.df; break;
          default: d = reinterpret_cast<Entry<APro> *>(p)->a.df; break;
        }
        const dim3 g = grid_of(L.kind, d, blk);
        // the header fields precede the argument set in every Entry<A>
        Entry<char> *hdr = reinterpret_cast<Entry<char> *>(p);
        hdr->base = blocks;
        hdr->gx = g.x;
        hdr->gy = g.y;
        hdr->gz = g.z;
        blocks += g.x * g.y * g.z;
      }
      L.blocks = blocks;
      e = launch(*b, L, b->st);  // warm-up
      if (e == cudaSuccess) e = cudaEventRecord(e0, b->st);
      for (int r = 0; r < reps && e == cudaSuccess; r++) e = launch(*b, L, b->st);
      if (e == cudaSuccess) e = cudaEventRecord(e1, b->st);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e == cudaSuccess && ms < best) {
        best = ms;
        best_shape = blk;
      }
    }
    if (e == cudaSuccess) {
      b->slot_shape[L0.slot] = best_shape;
      tuned++;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  int rc = build_plans(*b);  // new grids in every plan; uploads all tables again
  if (e != cudaSuccess) return set_error(nullptr, DSG_E_CUDA, "autotune: %s", cudaGetErrorString(e));
  if (rc) return rc;
  if (slots_tuned) *slots_tuned = tuned;
  return DSG_OK;
}

long long batch_tail_nodes(const BatchSolve *b) { return b ? b->tail_nodes : 0; }

}  // namespace dsg
