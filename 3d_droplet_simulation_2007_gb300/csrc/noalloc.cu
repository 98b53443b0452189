// noalloc.cu -- a pressure solve that allocates no memory.
//
// Some callers cannot allocate device memory at the time they need a solve:
// a Fortran or C host that hands over device arrays it manages itself and runs
// under an allocator that forbids cudaMalloc between set-up and tear-down, a
// code that solves inside a region where a device allocation would
// synchronize the device, or an embedded loop with a fixed memory budget.
// dsg_mglin_noalloc runs the reference's fixed-cycle full multigrid (mglin,
// main.f:3645-3763) on the caller's finest-level arrays and keeps every coarser
// level and the finest residual in one file-scope device array of fixed size,
// so it calls no cudaMalloc, cudaFree or allocating library routine.
//
// Limits and sharing:
//  * the scratch array holds grids up to 66 x 66 x 66 nodes (64^3 interior
//    cells, the reference's own build size); larger grids are rejected with
//    DSG_E_ARG and a message in dsg_last_error(NULL);
//  * the array exists once per device that loads the library and stays
//    allocated until the process exits;
//  * every call uses the same array and leaves its contents behind; each call
//    first clears it, so results never depend on an earlier call, but calls
//    whose work overlaps on the GPU (different streams, or host threads without
//    ordering) race on the array and must be serialized by the caller;
//  * the first call on each device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it; make that
//    first call before any stream capture is started.
#include <atomic>

#include "dsg_internal.cuh"

namespace {

constexpr int kNoAllocMaxSide = 66;
// finest residual (66^3) + 7 arrays (u, res, rhs, a, b, c, ei) on each coarser
// level of a 66^3 grid (34^3 + 18^3 + 10^3 + 6^3 + 4^3 cells)
constexpr size_t kNoAllocDoubles = (size_t)66 * 66 * 66 + 7 * ((size_t)34 * 34 * 34 + 18 * 18 * 18 + 10 * 10 * 10 +
                                                              6 * 6 * 6 + 4 * 4 * 4);

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

constexpr int kMaxDevices = 64;
// Per-device cache of the array's address.  Host threads that make their first
// call on a device at the same time may both look it up; they store the same
// value, and the atomics make that well defined.
std::atomic<double *> g_scratch_addr[kMaxDevices];

// Device address of the scratch array on the current device (looked up once
// per device; host code cannot use the symbol itself as a device pointer).
int scratch_address(double **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return dsg::set_error(nullptr, DSG_E_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return dsg::set_error(nullptr, DSG_E_ARG, "device %d out of range", dev);
  double *addr = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!addr) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return dsg::set_error(nullptr, DSG_E_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    addr = (double *)p;
    g_scratch_addr[dev].store(addr, std::memory_order_release);
  }
  *out = addr;
  return DSG_OK;
}

struct Level {
  dsg::Dims d;
  double *u, *res, *rhs, *a, *b, *c, *ei;
};

#define NA_CK(expr)                                                                                   \
  do {                                                                                                \
    cudaError_t _e = (expr);                                                                          \
    if (_e != cudaSuccess) return dsg::set_error(nullptr, DSG_E_CUDA, "%s: %s", #expr, cudaGetErrorString(_e)); \
  } while (0)

int vcycle(Level *L, int j, double ls, double omega, int npre, int npost, int ntop, cudaStream_t st) {
  for (int jj = j; jj >= 2; jj--) {
    Level &F = L[jj], &C = L[jj - 1];
    NA_CK(dsg::relax_n(npre, F.u, ls, F.rhs, F.a, F.b, F.c, F.ei, F.d, omega, st));
    NA_CK(dsg::resid(ls, F.res, F.u, F.rhs, F.a, F.b, F.c, F.d, st));
    NA_CK(dsg::rstrct(C.rhs, F.res, C.d, st));
    NA_CK(cudaMemsetAsync(C.u, 0, C.d.count() * sizeof(double), st));
  }
  NA_CK(dsg::relax_n(ntop, L[1].u, ls, L[1].rhs, L[1].a, L[1].b, L[1].c, L[1].ei, L[1].d, omega, st));
  for (int jj = 2; jj <= j; jj++) {
    Level &F = L[jj];
    NA_CK(dsg::addint(F.u, L[jj - 1].u, F.res, F.d, st));
    NA_CK(dsg::relax_n(npost, F.u, ls, F.rhs, F.a, F.b, F.c, F.ei, F.d, omega, st));
  }
  return DSG_OK;
}

}  // namespace

extern "C" int dsg_mglin_noalloc(double *p, const double *rhs, const double *a, const double *b, const double *c,
                                 const double *ei, int nx, int ny, int nz, int cycles, int npre, int npost, int ntop,
                                 double omega, double lengthsize, double lengthscale, void *stream) {
  if (!p || !rhs || !a || !b || !c || !ei)
    return dsg::set_error(nullptr, DSG_E_ARG, "dsg_mglin_noalloc: null array");
  if (nx > kNoAllocMaxSide || ny > kNoAllocMaxSide || nz > kNoAllocMaxSide)
    return dsg::set_error(nullptr, DSG_E_ARG,
                          "dsg_mglin_noalloc: grid %dx%dx%d exceeds the %dx%dx%d capacity of its static scratch",
                          nx, ny, nz, kNoAllocMaxSide, kNoAllocMaxSide, kNoAllocMaxSide);
  if (cycles < 0 || npre < 0 || npost < 0 || ntop < 0)
    return dsg::set_error(nullptr, DSG_E_ARG, "dsg_mglin_noalloc: negative cycle or sweep count");
  // memoryaloc, main.f:284-298
  int nn = nx < ny ? nx : ny;
  nn = nn < nz ? nn : nz;
  int j = nn - 2, ng = 1;
  while (j > 2) {
    j /= 2;
    ng++;
  }
  if (nn < 4 || (1 << ng) + 2 != nn)
    return dsg::set_error(nullptr, DSG_E_ARG, "dsg_mglin_noalloc: min(nx,ny,nz)=%d is not 2**ng+2", nn);
  // every side must halve evenly down to the coarsest level, as in dsg_create
  if (dsg::level_count(nx, ny, nz) != ng)
    return dsg::set_error(nullptr, DSG_E_ARG,
                          "dsg_mglin_noalloc: grid %dx%dx%d does not coarsen evenly over %d levels", nx, ny, nz, ng);
  double *scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;

  Level L[32];
  size_t used = (size_t)nx * ny * nz;  // finest residual
  L[ng] = Level{dsg::Dims{nx, ny, nz}, p, scratch, const_cast<double *>(rhs), const_cast<double *>(a),
                const_cast<double *>(b), const_cast<double *>(c), const_cast<double *>(ei)};
  int cx = nx, cy = ny, cz = nz;
  for (int l = ng - 1; l >= 1; l--) {
    cx = cx / 2 + 1;
    cy = cy / 2 + 1;
    cz = cz / 2 + 1;
    const size_t n = (size_t)cx * cy * cz;
    double *q[7];
    for (int f = 0; f < 7; f++) {
      q[f] = scratch + used;
      used += n;
    }
    L[l] = Level{dsg::Dims{cx, cy, cz}, q[0], q[1], q[2], q[3], q[4], q[5], q[6]};
  }
  if (used > kNoAllocDoubles)
    return dsg::set_error(nullptr, DSG_E_ARG, "dsg_mglin_noalloc: grid needs %zu scratch doubles, capacity %zu", used,
                          kNoAllocDoubles);
  // Clear what a previous call left behind, so results never depend on it.
  NA_CK(cudaMemsetAsync(scratch, 0, used * sizeof(double), st));
  // mglin: restrict rhs and coarsen the coefficients down to the coarsest grid
  for (int g = ng - 1; g >= 1; g--) {
    NA_CK(dsg::rstrct(L[g].rhs, L[g + 1].rhs, L[g].d, st));
    NA_CK(dsg::acfromac(L[g].a, L[g].b, L[g].c, L[g].ei, L[g + 1].a, L[g + 1].b, L[g + 1].c, L[g].d, st));
  }
  NA_CK(cudaMemsetAsync(L[1].u, 0, L[1].d.count() * sizeof(double), st));
  // first coarse solve with lengthscale in place of lengthsize (main.f:3686-3689)
  NA_CK(dsg::relax_n(ntop, L[1].u, lengthscale, L[1].rhs, L[1].a, L[1].b, L[1].c, L[1].ei, L[1].d, omega, st));
  for (int jl = 2; jl <= ng; jl++) {
    NA_CK(dsg::interp(L[jl].u, L[jl - 1].u, L[jl].d, st));
    for (int cyc = 0; cyc < cycles; cyc++) {
      rc = vcycle(L, jl, lengthsize, omega, npre, npost, ntop, st);
      if (rc) return rc;
    }
  }
  return DSG_OK;
}
