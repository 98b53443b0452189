// init.cu -- droplet initial condition on the device: smooth2 (main.f:5678-5752)
// with its 30^3 sub-cell sampling of partial cells, the seeded velocity noise
// of the workload definition, then the same boundary calls as initialize
// (main.f:176-178).
#include "dsg_internal.cuh"

namespace dsg {
namespace {

// Cell-face coordinate xx(i) = (i-1.5)*h with (i-1.5) in default REAL, as in
// smooth2.  xx(1) is read uninitialised by the reference; it is (1-1.5)*h here.
__device__ __forceinline__ double face_coord(int i, double h) { return (double)((float)i - 1.5f) * h; }

__global__ void k_smooth2(double *__restrict__ cc, Dims d, double h, double x0, double y0, double z0,
                          double r2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const double xa = face_coord(i - 1, h), xb = face_coord(i, h);
  const double ya = face_coord(j - 1, h), yb = face_coord(j, h);
  const double za = face_coord(k - 1, h), zb = face_coord(k, h);
  double ax = xa - x0, bx = xb - x0, ay = ya - y0, by = yb - y0, az = za - z0, bz = zb - z0;
  ax *= ax; bx *= bx; ay *= ay; by *= by; az *= az; bz *= bz;
  double c;
  if (!(dmin1(ax, bx) + dmin1(ay, by) + dmin1(az, bz) < r2)) {
    c = 0.0;
  } else if (!(dmax1(ax, bx) + dmax1(ay, by) + dmax1(az, bz) > r2)) {
    c = 1.0;
  } else {
    const int index = 30;
    const double inc = 1.0 / (double)(index * index * index);
    c = 0.0;
    for (int l = 1; l <= index; l++) {
      const double px = xa + ((double)l - 0.5) / (double)index * h - x0;
      for (int m = 1; m <= index; m++) {
        const double py = ya + ((double)m - 0.5) / (double)index * h - y0;
        for (int n = 1; n <= index; n++) {
          const double pz = za + ((double)n - 0.5) / (double)index * h - z0;
          if (px * px + py * py + pz * pz < r2) c = c + inc;
        }
      }
    }
    // Deviation from smooth2: the 27000 sub-sample additions can round to
    // 1+4e-13, which the advection would feed to AL3D as a negative 1-c (NaN);
    // the sampled fraction is clamped to 1.
    if (c > 1.0) c = 1.0;
  }
  cc[d.ix(i, j, k)] = c;
}

__global__ void k_init_velocity(double *__restrict__ u, double *__restrict__ v, double *__restrict__ w,
                                const double *__restrict__ cc, size_t n, double yvel1, double yvel2,
                                double zvel1, double zvel2) {
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const double c = cc[q];
    u[q] = 0.0;
    v[q] = yvel1 * c + yvel2 * (1 - c);
    w[q] = zvel1 * c + zvel2 * (1 - c);
  }
}

// Counter-based uniform noise in [-1,1): SplitMix64 of (seed, field, linear index).
__device__ __forceinline__ double noise_unit(uint64_t seed, int field, uint64_t lin) {
  uint64_t z = seed + 0x9E3779B97F4A7C15ULL * ((((uint64_t)field) << 40) + lin + 1ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z = z ^ (z >> 31);
  const double r = (double)(z >> 11) * (1.0 / 9007199254740992.0);
  return 2.0 * r - 1.0;
}

__global__ void k_noise(double *__restrict__ u, double *__restrict__ v, double *__restrict__ w, Dims d,
                        double amp, uint64_t seed) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1) return;
  const size_t q = d.ix(i, j, k);
  u[q] = u[q] + amp * noise_unit(seed, 0, q);
  v[q] = v[q] + amp * noise_unit(seed, 1, q);
  w[q] = w[q] + amp * noise_unit(seed, 2, q);
}

const dim3 kBlk(32, 4, 1);

}  // namespace

cudaError_t init_drop(double *cc, double *u, double *v, double *w, Dims d, double h, double x0, double y0,
                      double z0, double radius, double yvel1, double yvel2, double zvel1, double zvel2,
                      double noise_amp, uint64_t seed, cudaStream_t st) {
  DSG_COUNT k_smooth2<<<interior_grid(d, kBlk), kBlk, 0, st>>>(cc, d, h, x0, y0, z0, radius * radius);
  cudaError_t e = bc_c(cc, d, st);
  if (e != cudaSuccess) return e;
  const size_t n = d.count();
  const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
  DSG_COUNT k_init_velocity<<<blocks, 256, 0, st>>>(u, v, w, cc, n, yvel1, yvel2, zvel1, zvel2);
  if (noise_amp != 0.0) DSG_COUNT k_noise<<<interior_grid(d, kBlk), kBlk, 0, st>>>(u, v, w, d, noise_amp, seed);
  return cudaGetLastError();
}

}  // namespace dsg
