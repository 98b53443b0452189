// nn.cu -- the learned multigrid initial guess: a small 3D convolutional
// U-Net (no reference counterpart) with hand-written BF16 tensor-core kernels.
//
// Network (~251k parameters), channels-last activations over the interior
// cells (D x H x W, each a multiple of 8):
//   E1 conv 3->16 + ReLU   (full resolution; input padded to 16 channels)
//   E2 conv 16->32 + ReLU  (1/2, after 2x2x2 average pooling)
//   E3 conv 32->64 + ReLU  (1/4)
//   E4 conv 64->64 + ReLU  (1/8)
//   D3 conv 64->32 + ReLU  on up(E4) + E3
//   D2 conv 32->16 + ReLU  on up(D3) + E2
//   D1 conv 16->1          on up(D2) + E1  (linear output, channel padded to 8)
// All convolutions are 3x3x3, zero padded, implicit GEMMs on the tensor cores
// with BF16 inputs and FP32 accumulation.  Forward and data gradient run on
// Blackwell's tcgen05 MMA (k_conv3_tc): M = 128 voxels (an 8 x 16 x 1 tile),
// N = output channels, K = 27 taps x input channels; the input halo arrives
// by TMA, the weights stay in shared memory, the accumulator lives in tensor
// memory.  The data gradient uses flipped, transposed weights.  The weight
// gradient is a second implicit GEMM (M = input channels, N = output channels,
// K = voxels) on mma.sync m16n8k16.
#include <cuda.h>
#include <cuda_bf16.h>

#include <math.h>
#include <string.h>

#include <vector>

#include "dsg_internal.cuh"
#include "tc05.cuh"

namespace dsg {
namespace nn {

typedef __nv_bfloat16 bf16;

// ---- layer table -------------------------------------------------------------
struct LayerDef {
  int cin, cout;   // logical channels
  int cinp, coutp; // padded channels (multiples of 16 / 8)
  int level;       // resolution level (0 = full)
  bool relu;
};
constexpr int kLayers = 7;
constexpr int kIn = DSG_NET_INPUTS;  // logical input channels (padded to 16)
constexpr LayerDef kDefs[kLayers] = {
    {kIn, 16, 16, 16, 0, true}, // E1
    {16, 32, 16, 32, 1, true},  // E2
    {32, 64, 32, 64, 2, true},  // E3
    {64, 64, 64, 64, 3, true},  // E4
    {64, 32, 64, 32, 2, true},  // D3
    {32, 16, 32, 16, 1, true},  // D2
    {16, 1, 16, 8, 0, false},   // D1
};

// channels of a layer's output gradient (the output layer is padded to 16 so
// its gradient feeds the 16-wide data/weight gradient GEMMs)
inline int grad_ch(int l) { return kDefs[l].coutp < 16 ? 16 : kDefs[l].coutp; }

inline long long layer_params(int l) { return 27LL * kDefs[l].cin * kDefs[l].cout + kDefs[l].cout; }
constexpr long long kParams = 27LL * (kIn * 16 + 16 * 32 + 32 * 64 + 64 * 64 + 64 * 32 + 32 * 16 + 16 * 1) +
                              (16 + 32 + 64 + 64 + 32 + 16 + 1);
#define DSG_NET_PARAMS ((size_t)dsg::nn::kParams)

// ---- helpers -------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void ldmatrix_x4(unsigned &r0, unsigned &r1, unsigned &r2, unsigned &r3, unsigned addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}

__device__ __forceinline__ void ldmatrix_x4_trans(unsigned &r0, unsigned &r1, unsigned &r2, unsigned &r3,
                                                  unsigned addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}

__device__ __forceinline__ void ldmatrix_x2_trans(unsigned &r0, unsigned &r1, unsigned addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];" : "=r"(r0), "=r"(r1) : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                         unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Tile geometry of the mma.sync weight-gradient kernel below.
constexpr int CTX = 16, CTY = 8;

// ---- convolution forward / data gradient on tcgen05 ------------------------------
// X: [D][H][W][CIN] bf16 (read through the TMA map xmap), Wt: packed weights
// [9][CIN/8][3][NT][8] bf16 (in-plane tap dy*3+dx, 8-channel input block,
// tap row dz, output channel, 8 inputs); the CTA uses output channels
// co0 .. co0+COUT-1; Y: [D][H][W][ystride] (bf16, or float when OUTF, of which
// channels co0 .. co0+ywrite-1 are written).
//
// A work unit is an 8 (x) x 16 (y) voxel tile -- the 128 rows M of one MMA --
// over a chunk of L output planes z0 .. z0+L-1, marched in z: the input
// planes z0-1 .. z0+L arrive one at a time by TMA (the 10 x 18 halo as CIN/8
// slabs of 8 channels, which is the no-swizzle K-major core-matrix layout:
// 8 voxels along x x 16 bytes per core matrix, the next tile row 160 bytes
// on, the next 8 channels one slab on), and each input plane is multiplied
// once by the weights of all three tap rows dz: per in-plane tap (dy, dx) and
// 16 input channels one MMA with N = 3 x COUT, whose three column groups are
// the accumulators of output planes z'+1, z', z'-1.  Those accumulators sit
// side by side in TMEM with the plane index descending, so each MMA lands on
// the right three planes; at the chunk ends and the domain faces the MMA is
// narrowed to the groups of planes inside the chunk.  An output plane is
// complete after its last input plane; the epilogue then reads it, sets its
// columns back to zero (every MMA accumulates), adds the bias, applies the
// ReLU and stores it.  Per input plane the tensor cores read each A tile once
// for 3 x COUT outputs, and the halo is re-read (L + 2) / L times instead of
// 27 / 9.
//
// Warp roles (192 threads): warp 4 (one thread) issues the TMA loads into a
// ring of STAGES plane buffers, warp 5 (one thread) issues the MMAs into two
// TMEM chunk buffers, warps 0-3 own TMEM lanes 32w .. 32w+31 (= voxels) and
// run the epilogue.  mbarriers hand the buffers over: full[s] (plane bytes
// landed), empty[s] (the MMAs reading stage s are done), pdone[b][p] (plane p
// of chunk buffer b complete), tempty[b] (chunk buffer b read and zeroed).
// The weights arrive once by bulk copies.  Every wait is bounded in time: on
// a timeout the CTA raises a shared abort flag that ends every role's loop,
// waits (again bounded) for its own copies and MMAs in flight, frees its TMEM
// and records the failure in *err.
namespace tc {
constexpr int TX = 8, TY = 16, HX = TX + 2, HY = TY + 2;
constexpr uint32_t PL = 2944;        // 18 x 10 voxels x 16 bytes = 2880, padded to 128 bytes
constexpr uint32_t PL_BYTES = 2880;  // bytes one slab's TMA box delivers
constexpr uint32_t SBO_A = HX * 16;  // next tile row: 8 more M rows
constexpr int EPI_WARPS = 4, PRODUCER_WARP = 4, MMA_WARP = 5;
constexpr int THREADS = 32 * (EPI_WARPS + 2);
constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s bound of every wait

// TMEM columns of two chunk buffers of LMAX planes x COUT channels
__host__ __device__ constexpr int tmem_cols(int cout, int lmax) {
  return 2 * lmax * cout <= 32 ? 32 : 2 * lmax * cout <= 64 ? 64 : 2 * lmax * cout <= 128 ? 128
                                   : 2 * lmax * cout <= 256 ? 256 : 512;
}
template <int CIN, int COUT, int STAGES>
__host__ __device__ constexpr size_t smem_bytes() {
  return 1024 + (size_t)STAGES * (CIN / 8) * PL + (size_t)27 * CIN * COUT * 2 + 512;
}
}  // namespace tc

template <int CIN, int COUT, int STAGES, int LMAX, bool RELU, bool OUTF>
__global__ void __launch_bounds__(tc::THREADS) k_conv3_tc(const __grid_constant__ CUtensorMap xmap,
                                                          const bf16 *__restrict__ Wt, int NT, int co0,
                                                          const float *__restrict__ bias, int nbias,
                                                          void *__restrict__ Yv, int ystride, int ywrite, int W,
                                                          int H, int D, int L, int *__restrict__ err) {
  using namespace tc;
  using namespace dsg::tc05;
  static_assert(COUT % 16 == 0 && 3 * COUT <= 256 && CIN % 16 == 0 && STAGES >= 2 && STAGES <= 8, "MMA shape");
  static_assert(2 * LMAX * COUT <= 512 && LMAX <= 16, "TMEM chunk buffers");
  constexpr uint32_t WBYTES = 27u * CIN * COUT * 2;
  constexpr uint32_t BROW = 3 * COUT * 16;  // bytes of one (tap, 8-channel block) of B
  constexpr int TCOLS = tmem_cols(COUT, LMAX);
  extern __shared__ unsigned char smem_raw[];
  unsigned char *sm = reinterpret_cast<unsigned char *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char *halo = sm;
  unsigned char *wts = sm + (size_t)STAGES * (CIN / 8) * PL;
  uint64_t *full = reinterpret_cast<uint64_t *>(wts + WBYTES);
  uint64_t *empty = full + STAGES, *tempty = empty + STAGES, *pdone = tempty + 2, *wbar = pdone + 2 * LMAX,
           *fin = wbar + 1;
  uint32_t *tslot = reinterpret_cast<uint32_t *>(fin + 1);
  volatile int *abort = reinterpret_cast<volatile int *>(tslot + 1);
  __shared__ float s_bias[COUT];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tilesx = (W + TX - 1) / TX, tilesy = (H + TY - 1) / TY, tiles = tilesx * tilesy;
  const int nunits = tiles * ((D + L - 1) / L);
  const int mine = (int)blockIdx.x < nunits ? (nunits - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  for (int q = tid; q < COUT; q += THREADS) s_bias[q] = (bias && co0 + q < nbias) ? bias[co0 + q] : 0.f;
  if (tid == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&tempty[0], 32 * EPI_WARPS);
    mbar_init(&tempty[1], 32 * EPI_WARPS);
    for (int q = 0; q < 2 * LMAX; q++) mbar_init(&pdone[q], 1);
    mbar_init(wbar, 1);
    mbar_init(fin, 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    tmem_alloc(tslot, TCOLS);
    tmem_relinquish();
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tbase = *tslot;
  // unit u: tile (txi, tyi) of chunk zc; its input planes zlo .. zhi
  auto unit = [&](int i, int &txi, int &tyi, int &z0, int &lc, int &zlo, int &zhi) {
    const int u = (int)blockIdx.x + i * (int)gridDim.x;
    txi = u % tilesx;
    tyi = (u / tilesx) % tilesy;
    z0 = (u / tiles) * L;
    lc = D - z0 < L ? D - z0 : L;
    zlo = z0 > 0 ? z0 - 1 : 0;
    zhi = z0 + lc < D ? z0 + lc : D - 1;
  };

  if (warp == PRODUCER_WARP) {
    if (lane == 0) {
      // weights of output channels co0 .. co0+COUT-1 as [9][CIN/8][3][COUT][8]
      mbar_expect_tx(wbar, WBYTES);
      if (NT == COUT) {
        bulk_g2s(wts, Wt, WBYTES, wbar);
      } else {
        for (int r = 0; r < 27 * (CIN / 8); r++)
          bulk_g2s(wts + (size_t)r * COUT * 16, Wt + ((size_t)r * NT + co0) * 8, COUT * 16, wbar);
      }
      int g = 0;
      bool ok = true;
      for (int i = 0; ok && i < mine; i++) {
        int txi, tyi, z0, lc, zlo, zhi;
        unit(i, txi, tyi, z0, lc, zlo, zhi);
        for (int zp = zlo; zp <= zhi; zp++, g++) {
          const int s = g % STAGES, k = g / STAGES;
          if (k > 0 && !mbar_wait_ns(&empty[s], (k - 1) & 1, kWaitNs, abort)) {
            ok = false;
            break;
          }
          mbar_expect_tx(&full[s], (CIN / 8) * PL_BYTES);
#pragma unroll
          for (int k8 = 0; k8 < CIN / 8; k8++)
            tma_load_4d(halo + ((size_t)s * (CIN / 8) + k8) * PL, &xmap, &full[s], k8 * 8, txi * TX - 1,
                        tyi * TY - 1, zp);
        }
      }
      // copies in flight (after an abort only): the last load of each stage
      for (int s = 0; s < STAGES && s < g; s++) {
        const int last = s + ((g - 1 - s) / STAGES) * STAGES;
        mbar_wait_ns(&full[s], (last / STAGES) & 1, kWaitNs, nullptr);
      }
      mbar_wait_ns(wbar, 0, kWaitNs, nullptr);
    }
  } else if (warp == MMA_WARP) {
    if (lane == 0) {
      const uint64_t bdesc0 = smem_desc(smem_addr(wts), BROW, 128);
      const uint32_t hbase = smem_addr(halo);
      bool ok = mbar_wait_ns(wbar, 0, kWaitNs, abort);
      int g = 0;
      for (int i = 0; ok && i < mine; i++) {
        int txi, tyi, z0, lc, zlo, zhi;
        unit(i, txi, tyi, z0, lc, zlo, zhi);
        const int b = i & 1;
        if (!mbar_wait_ns(&tempty[b], (i >> 1) & 1, kWaitNs, abort)) break;
        fence_after_sync();
        const uint32_t cbase = tbase + (uint32_t)(b * LMAX * COUT);
        int next = 0;  // next plane of the chunk to report complete
        for (int zp = zlo; zp <= zhi; zp++, g++) {
          const int s = g % STAGES, k = g / STAGES;
          if (!mbar_wait_ns(&full[s], k & 1, kWaitNs, abort)) {
            ok = false;
            break;
          }
          // tap rows dz whose output plane zp + 1 - dz lies in the chunk
          const int dlo = zp + 2 - z0 - lc > 0 ? zp + 2 - z0 - lc : 0;
          const int dhi = zp + 1 - z0 < 2 ? zp + 1 - z0 : 2;
          const uint32_t idesc = idesc_bf16(128, (dhi - dlo + 1) * COUT);
          // plane z sits in slot lc - 1 - (z - z0): group dlo is plane zp + 1 - dlo
          const uint32_t dt = cbase + (uint32_t)((lc - 1 - (zp + 1 - dlo - z0)) * COUT);
          const uint64_t adesc0 = smem_desc(hbase + (uint32_t)(s * (CIN / 8)) * PL, PL, SBO_A);
          const uint64_t bdesc1 = bdesc0 + ((uint32_t)(dlo * COUT * 16) >> 4);
          // descriptors hold address / 16 in their low 14 bits: a shared-memory
          // offset is added to them as offset / 16 (no carry below 256 KB)
#pragma unroll
          for (int t9 = 0; t9 < 9; t9++) {
#pragma unroll
            for (int q = 0; q < CIN / 16; q++) {
              const uint32_t aoff = (uint32_t)(((t9 / 3) * HX + t9 % 3) * 16) + (uint32_t)(2 * q) * PL;
              const uint32_t boff = (uint32_t)(t9 * (CIN / 8) + 2 * q) * BROW;
              umma_bf16(dt, adesc0 + (aoff >> 4), bdesc1 + (boff >> 4), idesc, 1u);
            }
          }
          mma_commit(&empty[s]);
          // planes whose last input plane this was
          const int upto = zp == zhi ? lc : (zp - z0 < lc ? zp - z0 : lc);
          for (; next < upto; next++) mma_commit(&pdone[b * LMAX + next]);
        }
      }
      mma_commit(fin);  // arrives once every MMA issued above has completed
      mbar_wait_ns(fin, 0, kWaitNs, nullptr);
    }
  } else {
    // epilogue: warp w holds TMEM lanes 32w .. 32w+31 = tile rows m = 8 * my + mx
    const int m = 32 * warp + lane, mx = m & 7, my = m >> 3;
    const uint32_t lanes = (uint32_t)(32 * warp) << 16;
    uint32_t zero[16];
#pragma unroll
    for (int q = 0; q < 16; q++) zero[q] = 0u;
    // both chunk buffers start at zero
    for (int c = 0; c < 2 * LMAX * COUT; c += 16) tmem_st16(tbase + lanes + (uint32_t)c, zero);
    tmem_wait_st();
    fence_before_sync();
    mbar_arrive(&tempty[0]);
    mbar_arrive(&tempty[1]);
    uint32_t par0 = 0u, par1 = 0u;  // phase parity of each pdone barrier of buffer 0 / 1, one bit per plane
    bool ok = true;
    for (int i = 0; ok && i < mine; i++) {
      int txi, tyi, z0, lc, zlo, zhi;
      unit(i, txi, tyi, z0, lc, zlo, zhi);
      const int b = i & 1;
      const uint32_t cbase = tbase + lanes + (uint32_t)(b * LMAX * COUT);
      const int x = txi * TX + mx, y = tyi * TY + my;
      const bool inside = x < W && y < H;
      for (int p = 0; p < lc; p++) {
        const uint32_t par = b ? par1 : par0;
        const bool got = mbar_wait_ns(&pdone[b * LMAX + p], (par >> p) & 1u, kWaitNs, abort);
        if (b) par1 ^= 1u << p;
        else par0 ^= 1u << p;
        if (!__all_sync(0xffffffffu, got)) {
          ok = false;
          break;
        }
        fence_after_sync();
        const uint32_t dt = cbase + (uint32_t)((lc - 1 - p) * COUT);
        uint32_t r[COUT / 16][16];
#pragma unroll
        for (int c = 0; c < COUT / 16; c++) tmem_ld16_async(dt + (uint32_t)(16 * c), r[c]);
#pragma unroll
        for (int c = 0; c < COUT / 16; c++) tmem_wait_ld16(r[c]);
#pragma unroll
        for (int c = 0; c < COUT / 16; c++) tmem_st16(dt + (uint32_t)(16 * c), zero);
        const size_t vox = ((size_t)(z0 + p) * H + y) * W + x;
#pragma unroll
        for (int c = 0; c < COUT / 16; c++) {
          if (!inside || 16 * c >= ywrite) break;
          float v[16];
#pragma unroll
          for (int q = 0; q < 16; q++) {
            v[q] = __uint_as_float(r[c][q]) + s_bias[16 * c + q];
            if (RELU) v[q] = fmaxf(v[q], 0.f);
          }
          if (OUTF) {
            float *Y = reinterpret_cast<float *>(Yv) + vox * ystride + co0 + 16 * c;
            reinterpret_cast<float4 *>(Y)[0] = make_float4(v[0], v[1], v[2], v[3]);
            reinterpret_cast<float4 *>(Y)[1] = make_float4(v[4], v[5], v[6], v[7]);
            if (ywrite - 16 * c >= 16) {
              reinterpret_cast<float4 *>(Y)[2] = make_float4(v[8], v[9], v[10], v[11]);
              reinterpret_cast<float4 *>(Y)[3] = make_float4(v[12], v[13], v[14], v[15]);
            }
          } else {
            bf16 *Y = reinterpret_cast<bf16 *>(Yv) + vox * ystride + co0 + 16 * c;
            uint4 o[2];
            __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(o);
#pragma unroll
            for (int q = 0; q < 8; q++) h[q] = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
            reinterpret_cast<uint4 *>(Y)[0] = o[0];
            reinterpret_cast<uint4 *>(Y)[1] = o[1];
          }
        }
      }
      if (!ok) break;
      tmem_wait_st();
      fence_before_sync();
      mbar_arrive(&tempty[b]);
    }
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 0) tmem_dealloc(tbase, TCOLS);
  if (tid == 0 && *abort) atomicExch(err, 1);
}

// Weights packed for k_conv3_tc: dst[t9][kin/8][3][ntot][8] bf16 (in-plane tap
// t9 = dy*3+dx, 8-channel input block, tap row dz, output channel, 8 inputs)
// from the FP32 master Wt[27][cin][cout] (tap = dz*9 + t9).  Forward: K =
// input channels, N = output channels.  transpose (data gradient): K = the
// forward outputs, N = the forward inputs, taps mirrored.  Padding channels
// are zero.
__global__ void k_pack_tc(const float *__restrict__ Wt, bf16 *__restrict__ dst, int cin, int cout, int kin, int ntot,
                          int transpose) {
  const int total = 27 * kin * ntot;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int j = e & 7;
    const int n = (e >> 3) % ntot;
    const int dz = (e / (8 * ntot)) % 3;
    const int k8 = (e / (24 * ntot)) % (kin / 8);
    const int t9 = e / (24 * ntot * (kin / 8));
    const int tap = dz * 9 + t9;
    const int k = k8 * 8 + j;
    float w = 0.f;
    if (!transpose) {
      if (k < cin && n < cout) w = Wt[((size_t)tap * cin + k) * cout + n];
    } else {
      if (k < cout && n < cin) w = Wt[((size_t)(26 - tap) * cin + n) * cout + k];
    }
    dst[e] = __float2bfloat16(w);
  }
}

// ---- weight gradient (implicit GEMM over voxels) ----------------------------------
// dW[tap][ci][co] += sum_v X[v + off(tap)][ci] * G[v][co].  A CTA takes a brick of
// CTX x CTY x BZ voxels; warp w owns (tap, ci block) pairs w, w+8, ...; for each
// pair it accumulates a 16 (ci) x COUT tile over the brick with A = X^T and
// B = G loaded by ldmatrix.trans, then adds it to dW with atomics.
constexpr int BZ = 4;

template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_conv3_wgrad(const bf16 *__restrict__ X, const bf16 *__restrict__ G,
                                                     float *__restrict__ dW, int W, int H, int D) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int HX = CTX + 2, HY = CTY + 2, HZ = BZ + 2;
  bf16 *xt = reinterpret_cast<bf16 *>(smem);               // [HZ][HY][HX][CIN]
  bf16 *gt = xt + (size_t)HZ * HY * HX * CIN;               // [BZ][CTY][CTX][COUT]
  const int x0 = blockIdx.x * CTX, y0 = blockIdx.y * CTY, z0 = blockIdx.z * BZ;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  {
    constexpr int VPV = CIN / 8;
    const int nvec = HZ * HY * HX * VPV;
    for (int e = tid; e < nvec; e += 256) {
      const int c8 = e % VPV, v = e / VPV;
      const int hx = v % HX, hy = (v / HX) % HY, hz = v / (HX * HY);
      const int gx = x0 + hx - 1, gy = y0 + hy - 1, gz = z0 + hz - 1;
      uint4 val = make_uint4(0u, 0u, 0u, 0u);
      if (gx >= 0 && gx < W && gy >= 0 && gy < H && gz >= 0 && gz < D)
        val = reinterpret_cast<const uint4 *>(X + (((size_t)gz * H + gy) * W + gx) * CIN)[c8];
      reinterpret_cast<uint4 *>(xt + (size_t)v * CIN)[c8] = val;
    }
    constexpr int GPV = COUT / 8;
    const int ngv = BZ * CTY * CTX * GPV;
    for (int e = tid; e < ngv; e += 256) {
      const int c8 = e % GPV, v = e / GPV;
      const int bx = v % CTX, by = (v / CTX) % CTY, bz = v / (CTX * CTY);
      const int gx = x0 + bx, gy = y0 + by, gz = z0 + bz;
      uint4 val = make_uint4(0u, 0u, 0u, 0u);
      if (gx < W && gy < H && gz < D) val = reinterpret_cast<const uint4 *>(G + (((size_t)gz * H + gy) * W + gx) * COUT)[c8];
      reinterpret_cast<uint4 *>(gt + (size_t)v * COUT)[c8] = val;
    }
  }
  __syncthreads();
  constexpr int KB = CIN / 16;
  const int npairs = 27 * KB;
  // A = X^T (16 ci x 16 voxels): stored rows are voxels with ci contiguous, so
  // ldmatrix.trans of the 4 8x8 blocks gives the row-major A fragment:
  //   m0: ci 0-7,  v 0-7 ; m1: ci 8-15, v 0-7 ; m2: ci 0-7, v 8-15 ; m3: ci 8-15, v 8-15
  // B = G (16 voxels x 8 co): stored rows are voxels with co contiguous; the
  // col-major B fragment is ldmatrix.trans of blocks (v 0-7) and (v 8-15).
  const int lrow = lane & 7, lmat = lane >> 3;
  for (int pr = warp; pr < npairs; pr += 8) {
    const int tap = pr / KB, kb = pr % KB;
    const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
    float acc[COUT / 8][4];
#pragma unroll
    for (int n = 0; n < COUT / 8; n++) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
    for (int bz = 0; bz < BZ; bz++)
      for (int by = 0; by < CTY; by++) {
        // the 16 voxels of this k-step: x = 0..15 of row (by, bz)
        const int av = lrow + ((lmat >> 1) << 3);        // voxel index for this lane's A row address
        const int ach = kb * 16 + ((lmat & 1) << 3);     // ci offset
        const int hv = ((bz + dz) * HY + (by + dy)) * HX + (av + dx);
        unsigned a0, a1, a2, a3;
        ldmatrix_x4_trans(a0, a1, a2, a3, smem_u32(xt + (size_t)hv * CIN + ach));
        const int gvrow = (bz * CTY + by) * CTX;
#pragma unroll
        for (int n = 0; n < COUT / 8; n++) {
          const int bvox = (lane & 15);
          unsigned b0, b1;
          ldmatrix_x2_trans(b0, b1, smem_u32(gt + (size_t)(gvrow + bvox) * COUT + n * 8));
          mma_bf16(acc[n], a0, a1, a2, a3, b0, b1);
        }
      }
    const int g = lane >> 2, t4 = lane & 3;
#pragma unroll
    for (int n = 0; n < COUT / 8; n++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int ci = kb * 16 + g + (q >> 1) * 8;
        const int co = n * 8 + 2 * t4 + (q & 1);
        atomicAdd(dW + ((size_t)tap * CIN + ci) * COUT + co, acc[n][q]);
      }
  }
}

// The elementwise kernels below move 8 channels (16 bytes of bf16) per thread
// with 32-bit voxel indices; C is a multiple of 8 and every level has fewer
// than 2^32 channel groups.
struct V8 {
  float f[8];
};

__device__ __forceinline__ V8 load8(const bf16 *p) {
  const uint4 r = *reinterpret_cast<const uint4 *>(p);
  const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&r);
  V8 v;
#pragma unroll
  for (int c = 0; c < 4; c++) {
    const float2 f = __bfloat1622float2(h[c]);
    v.f[2 * c] = f.x;
    v.f[2 * c + 1] = f.y;
  }
  return v;
}

__device__ __forceinline__ void store8(bf16 *p, const V8 &v) {
  uint4 r;
  __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&r);
#pragma unroll
  for (int c = 0; c < 4; c++) h[c] = __floats2bfloat162_rn(v.f[2 * c], v.f[2 * c + 1]);
  *reinterpret_cast<uint4 *>(p) = r;
}

// 2x2x2 average pooling, channels-last bf16: Y at half resolution.
__global__ void k_pool(const bf16 *__restrict__ X, bf16 *__restrict__ Y, int W, int H, int D, int C) {
  const unsigned C8 = C / 8, Wc = W / 2, Hc = H / 2, Dc = D / 2;
  const unsigned n = Wc * Hc * Dc * C8;
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const unsigned g = q % C8, v = q / C8;
    const unsigned x = v % Wc, y = (v / Wc) % Hc, z = v / (Wc * Hc);
    V8 s;
#pragma unroll
    for (int c = 0; c < 8; c++) s.f[c] = 0.f;
    for (int k = 0; k < 8; k++) {
      const unsigned xx = 2 * x + (k & 1), yy = 2 * y + ((k >> 1) & 1), zz = 2 * z + (k >> 2);
      const V8 a = load8(X + ((size_t)((zz * H + yy) * W + xx)) * C + g * 8);
#pragma unroll
      for (int c = 0; c < 8; c++) s.f[c] += a.f[c];
    }
#pragma unroll
    for (int c = 0; c < 8; c++) s.f[c] = 0.125f * s.f[c];
    store8(Y + (size_t)q * 8, s);
  }
}

// Y = up(A) + B: A at half resolution, Y/B at full, channels-last bf16.
__global__ void k_upadd(const bf16 *__restrict__ A, const bf16 *__restrict__ B, bf16 *__restrict__ Y, int W, int H,
                        int D, int C) {
  const unsigned C8 = C / 8, Wc = W / 2, Hc = H / 2;
  const unsigned n = (unsigned)W * H * D * C8;
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const unsigned g = q % C8, v = q / C8;
    const unsigned x = v % W, y = (v / W) % H, z = v / (W * H);
    const V8 a = load8(A + ((size_t)(((z >> 1) * Hc + (y >> 1)) * Wc + (x >> 1))) * C + g * 8);
    V8 b = load8(B + (size_t)q * 8);
#pragma unroll
    for (int c = 0; c < 8; c++) b.f[c] = a.f[c] + b.f[c];
    store8(Y + (size_t)q * 8, b);
  }
}

// Backward of Y = up(A) + B: dB = dY, dA = sum over the 8 children (FP32).
__global__ void k_upadd_back(const bf16 *__restrict__ dY, float *__restrict__ dA, int W, int H, int D, int C) {
  const unsigned C8 = C / 8, Wc = W / 2, Hc = H / 2, Dc = D / 2;
  const unsigned n = Wc * Hc * Dc * C8;
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const unsigned g = q % C8, v = q / C8;
    const unsigned x = v % Wc, y = (v / Wc) % Hc, z = v / (Wc * Hc);
    float s[8];
#pragma unroll
    for (int c = 0; c < 8; c++) s[c] = 0.f;
    for (int k = 0; k < 8; k++) {
      const unsigned xx = 2 * x + (k & 1), yy = 2 * y + ((k >> 1) & 1), zz = 2 * z + (k >> 2);
      const V8 a = load8(dY + ((size_t)((zz * H + yy) * W + xx)) * C + g * 8);
#pragma unroll
      for (int c = 0; c < 8; c++) s[c] += a.f[c];
    }
    float4 *o = reinterpret_cast<float4 *>(dA + (size_t)q * 8);
    o[0] = make_float4(s[0], s[1], s[2], s[3]);
    o[1] = make_float4(s[4], s[5], s[6], s[7]);
  }
}

// Backward of pooling: dX(child) += dY(parent)/8 (accumulates into an FP32 buffer).
__global__ void k_pool_back_acc(const bf16 *__restrict__ dY, float *__restrict__ dX, int W, int H, int D, int C) {
  const unsigned C8 = C / 8, Wc = W / 2, Hc = H / 2;
  const unsigned n = (unsigned)W * H * D * C8;
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const unsigned g = q % C8, v = q / C8;
    const unsigned x = v % W, y = (v / W) % H, z = v / (W * H);
    const V8 a = load8(dY + ((size_t)(((z >> 1) * Hc + (y >> 1)) * Wc + (x >> 1))) * C + g * 8);
    float4 *o = reinterpret_cast<float4 *>(dX + (size_t)q * 8);
    float4 o0 = o[0], o1 = o[1];
    o0.x += 0.125f * a.f[0], o0.y += 0.125f * a.f[1], o0.z += 0.125f * a.f[2], o0.w += 0.125f * a.f[3];
    o1.x += 0.125f * a.f[4], o1.y += 0.125f * a.f[5], o1.z += 0.125f * a.f[6], o1.w += 0.125f * a.f[7];
    o[0] = o0;
    o[1] = o1;
  }
}

// G = bf16(dAcc * (act > 0)) (ReLU derivative), also the bias gradient.
__global__ void k_relu_back(const float *__restrict__ dacc, const bf16 *__restrict__ act, bf16 *__restrict__ G,
                            float *__restrict__ dbias, size_t nvox, int C, int relu) {
  __shared__ float sb[64];
  if (threadIdx.x < 64) sb[threadIdx.x] = 0.f;
  __syncthreads();
  const unsigned C8 = C / 8;
  const unsigned n = (unsigned)nvox * C8;
  float part[8];
#pragma unroll
  for (int c = 0; c < 8; c++) part[c] = 0.f;
  // a thread always handles the same channel group when blockDim*gridDim is a multiple of C8
  const unsigned stride = gridDim.x * blockDim.x;
  const unsigned q0 = blockIdx.x * blockDim.x + threadIdx.x;
  for (unsigned q = q0; q < n; q += stride) {
    const float4 *d = reinterpret_cast<const float4 *>(dacc + (size_t)q * 8);
    const float4 d0 = d[0], d1 = d[1];
    float g[8] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w};
    if (relu) {
      const V8 a = load8(act + (size_t)q * 8);
#pragma unroll
      for (int c = 0; c < 8; c++)
        if (!(a.f[c] > 0.f)) g[c] = 0.f;
    }
    V8 o;
#pragma unroll
    for (int c = 0; c < 8; c++) {
      o.f[c] = g[c];
      part[c] += g[c];
    }
    store8(G + (size_t)q * 8, o);
  }
  // lanes l and l + C8 hold the same channel group: reduce over them first
  for (int off = 16; off >= (int)C8; off >>= 1)
#pragma unroll
    for (int c = 0; c < 8; c++) part[c] += __shfl_xor_sync(0xffffffffu, part[c], off);
  if ((threadIdx.x & 31) < C8 && q0 < n) {
    const unsigned grp = q0 % C8;  // constant over the loop: stride % C8 == 0
#pragma unroll
    for (int c = 0; c < 8; c++) atomicAdd(&sb[grp * 8 + c], part[c]);
  }
  __syncthreads();
  if (threadIdx.x < C) atomicAdd(&dbias[threadIdx.x], sb[threadIdx.x]);
}

// bf16 -> float accumulate: dst += src (n a multiple of 8).
__global__ void k_acc_bf16(float *__restrict__ dst, const bf16 *__restrict__ src, size_t n) {
  const unsigned n8 = (unsigned)(n / 8);
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n8; q += gridDim.x * blockDim.x) {
    const V8 a = load8(src + (size_t)q * 8);
    float4 *o = reinterpret_cast<float4 *>(dst + (size_t)q * 8);
    float4 o0 = o[0], o1 = o[1];
    o0.x += a.f[0], o0.y += a.f[1], o0.z += a.f[2], o0.w += a.f[3];
    o1.x += a.f[4], o1.y += a.f[5], o1.z += a.f[6], o1.w += a.f[7];
    o[0] = o0;
    o[1] = o1;
  }
}

// Output layer loss: y (float, 8 padded channels, channel 0 used), target t.
// loss = mean (y - t)^2 ; dY (16 channels) channel 0 = 2 (y - t) / N, others 0.
__global__ void k_mse(const float *__restrict__ y, const float *__restrict__ t, float *__restrict__ dy,
                      double *__restrict__ loss, size_t nvox) {
  __shared__ double sh[256];
  double s = 0.0;
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (size_t)gridDim.x * blockDim.x) {
    const float d = y[v * 8] - t[v];
    s += (double)d * d;
#pragma unroll
    for (int c = 0; c < 16; c++) dy[v * 16 + c] = c == 0 ? 2.f * d / (float)nvox : 0.f;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, sh[0] / (double)nvox);
}

// Adam step on FP32 master parameters.
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, size_t n, float lr, float b1, float b2, float eps, float c1, float c2,
                       float clip) {
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    float gq = g[q];
    if (!isfinite(gq)) gq = 0.f;
    gq = fmaxf(-clip, fminf(clip, gq));
    const float mq = b1 * m[q] + (1.f - b1) * gq;
    const float vq = b2 * v[q] + (1.f - b2) * gq * gq;
    m[q] = mq;
    v[q] = vq;
    p[q] -= lr * (mq / c1) / (sqrtf(vq / c2) + eps);
  }
}

// ---- the network at the start of a pressure solve --------------------------------
// The start p is the FP32 full-multigrid guess; r = rhs - L p is its FP64
// defect as the solver's defect pass leaves it: rounded to FP32 in the
// colour-split layout of the finest FP32 level (r_ev / r_od, cell (i, j, k)
// in the half with parity (i + j + k) & 1 at index sp.at((i - 2) / 2, j, k)),
// with red = {sum r^2, sum rhs^2} over the interior in FP64.
// Slots of the network's sums (sums_dev): [0] sum p^2, [1] the correction
// scale h^2 RMS(r), [2..4] sums of the minimal-residual step, [5] sum rhs^2,
// [6] RMS(r); from [10] on, as floats: 1 / RMS(r), 1 / RMS(rhs), 1 / RMS(p).
constexpr int kScaleF = 20;  // float index of the reciprocal scales

// Index into one colour half of the finest FP32 level (the layout of the
// mixed solve: hx = (nx - 2) / 2 cells per row, rows of the interior).
struct Split {
  int hx, ny2, nz2;
  __device__ __forceinline__ size_t at(int m, int j, int k) const {
    return (size_t)m + (size_t)hx * ((size_t)(j - 2) + (size_t)ny2 * (size_t)(k - 2));
  }
};

__device__ __forceinline__ float split_at(const float *__restrict__ r_ev, const float *__restrict__ r_od, Split sp,
                                          int i, int j, int k) {
  return (((i + j + k) & 1) ? r_od : r_ev)[sp.at((i - 2) >> 1, j, k)];
}

// The scales of one solve's start (one thread).
__global__ void k_scales(double *__restrict__ sums, const double *__restrict__ red, double n_int, double h2) {
  if (threadIdx.x != 0) return;
  const double s_r = sqrt(red[0] / n_int) + 1e-300;
  const double s_b = sqrt(red[1] / n_int) + 1e-300;
  const double s_p = sqrt(sums[0] / n_int) + 1e-300;
  sums[1] = h2 * s_r;
  sums[5] = red[1];
  sums[6] = s_r;
  float *f = reinterpret_cast<float *>(sums);
  f[kScaleF] = (float)(1.0 / s_r);
  f[kScaleF + 1] = (float)(1.0 / s_b);
  f[kScaleF + 2] = (float)(1.0 / s_p);
}

// Input channels: cc, rhs / RMS(rhs), r / RMS(r), p / RMS(p), pprev / RMS(p);
// pbase keeps p in FP32 as the base of the training target.  The network
// predicts the correction of p in units of h^2 RMS(r) (the correction scales
// with the defect).
__global__ void k_features(bf16 *__restrict__ Xin, float *__restrict__ pbase, const float *__restrict__ r_ev,
                           const float *__restrict__ r_od, Split sp, const double *__restrict__ cc,
                           const double *__restrict__ rhs, const double *__restrict__ p,
                           const double *__restrict__ pprev, const double *__restrict__ sums, Dims d) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  const int W = d.nx - 2, H = d.ny - 2;
  if (x >= W || y >= H) return;
  const int i = x + 2, j = y + 2, k = z + 2;
  const size_t q = d.ix(i, j, k);
  const float *f = reinterpret_cast<const float *>(sums);
  const float ir = f[kScaleF], ib = f[kScaleF + 1], ip = f[kScaleF + 2];
  const float pc = (float)p[q];
  const size_t v = ((size_t)z * H + y) * W + x;
  uint4 o[2] = {make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u)};
  __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(o);
  h[0] = __floats2bfloat162_rn((float)cc[q], (float)rhs[q] * ib);
  h[1] = __floats2bfloat162_rn(split_at(r_ev, r_od, sp, i, j, k) * ir, pc * ip);
  h[2] = __floats2bfloat162_rn((float)pprev[q] * ip, 0.f);
  uint4 *dst = reinterpret_cast<uint4 *>(Xin + v * 16);
  dst[0] = o[0];
  dst[1] = o[1];
  pbase[v] = pc;
}

// Training target after the solve: (p - pbase) / scale over the interior.
__global__ void k_target(float *__restrict__ target, const double *__restrict__ p, const float *__restrict__ pbase,
                         const double *__restrict__ sums, Dims d) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  const int W = d.nx - 2, H = d.ny - 2;
  if (x >= W || y >= H) return;
  const size_t v = ((size_t)z * H + y) * W + x;
  target[v] = (float)((p[d.ix(x + 2, y + 2, z + 2)] - (double)pbase[v]) / sums[1]);
}

// Block partials of the minimal-residual step along the network's correction
// e = h^2 RMS(r) q (q = channel 0 of the output): L e = RMS(r) l with
// l = sum over the six faces of coefficient x (q_neighbour - q) under the
// solver's operator and boundary rules (main.f resid), evaluated in FP32.
// partials[3B..3B+2] = sums of r r, r l, l l over the block's cells; the
// defect of p + alpha e is r - alpha RMS(r) l.
__global__ void k_line_partials(double *__restrict__ partials, const float *__restrict__ r_ev,
                                const float *__restrict__ r_od, Split sp, const double *__restrict__ a,
                                const double *__restrict__ b, const double *__restrict__ c,
                                const float *__restrict__ qout, Dims d) {
  const int W = d.nx - 2, H = d.ny - 2;
  const size_t n = (size_t)W * H * (d.nz - 2);
  const size_t sy = d.sy(), sz = d.sz();
  const size_t vy = (size_t)W, vz = (size_t)W * H;
  float rr = 0.f, rl = 0.f, ll = 0.f;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const unsigned ni = (unsigned)W, nj = (unsigned)H, t32 = (unsigned)t;  // < 2^32 cells
    const unsigned rem = t32 / ni, kk = rem / nj;
    const int i = (int)(t32 - rem * ni) + 2;
    const int j = (int)(rem - kk * nj) + 2, k = (int)kk + 2;
    const size_t q = d.ix(i, j, k);
    const float r = split_at(r_ev, r_od, sp, i, j, k);
    const float *qv = qout + t * 8;
    const float ec = qv[0];
    const float ex = (i + 1 == d.nx) ? 0.f : qv[8];
    const float exm = (i - 1 == 1) ? ec : qv[-8];
    const float ey = (j + 1 == d.ny) ? ec : qv[8 * vy];
    const float eym = (j - 1 == 1) ? ec : qv[-(ptrdiff_t)(8 * vy)];
    const float ez = (k + 1 == d.nz) ? ec : qv[8 * vz];
    const float ezm = (k - 1 == 1) ? ec : qv[-(ptrdiff_t)(8 * vz)];
    const float l = (float)a[q] * (ex - ec) + (float)a[q - 1] * (exm - ec) + (float)b[q] * (ey - ec) +
                    (float)b[q - sy] * (eym - ec) + (float)c[q] * (ez - ec) + (float)c[q - sz] * (ezm - ec);
    rr += r * r;
    rl += r * l;
    ll += l * l;
  }
  __shared__ double sh[3][256];
  sh[0][threadIdx.x] = rr;
  sh[1][threadIdx.x] = rl;
  sh[2][threadIdx.x] = ll;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int m = 0; m < 3; m++) sh[m][threadIdx.x] += sh[m][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < 3) partials[3 * blockIdx.x + threadIdx.x] = sh[threadIdx.x][0];
}

// Block partials of sum f^2 over the interior (partials[B]).
__global__ void k_sumsq_partials(double *__restrict__ partials, const double *__restrict__ f, Dims d) {
  __shared__ double sh[256];
  const size_t n = (size_t)(d.nx - 2) * (d.ny - 2) * (d.nz - 2);
  double s = 0.0;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const unsigned ni = (unsigned)(d.nx - 2), nj = (unsigned)(d.ny - 2), tt = (unsigned)t;
    const unsigned r = tt / ni, kk = r / nj;
    const int i = (int)(tt - r * ni) + 2;
    const int j = (int)(r - kk * nj) + 2, k = (int)kk + 2;
    const double v = f[d.ix(i, j, k)];
    s += v * v;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = sh[0];
}

// out[m] = sum over nb blocks of partials[w * B + m], m < w (one block, fixed order).
__global__ void k_fold(double *__restrict__ out, const double *__restrict__ partials, int nb, int w) {
  __shared__ double sh[256];
  for (int m = 0; m < w; m++) {
    double s = 0.0;
    for (int q = threadIdx.x; q < nb; q += blockDim.x) s += partials[(size_t)q * w + m];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
      if (threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[m] = sh[0];
    __syncthreads();
  }
}

// p += alpha h^2 RMS(r) q over the interior.
__global__ void k_apply_corr(double *__restrict__ p, const float *__restrict__ qout,
                             const double *__restrict__ sums, double alpha, Dims d) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  const int W = d.nx - 2, H = d.ny - 2;
  if (x >= W || y >= H) return;
  const size_t v = ((size_t)z * H + y) * W + x;
  p[d.ix(x + 2, y + 2, z + 2)] += alpha * sums[1] * (double)qout[v * 8];
}

inline int eblocks(size_t n) { return (int)((n + 255) / 256 < 8192 ? (n + 255) / 256 : 8192); }

}  // namespace nn
}  // namespace dsg

// ============================================================================
// network object
// ============================================================================
using namespace dsg::nn;

struct dsg_net {
  int W[4], H[4], D[4];             // interior sizes per level
  float *params = nullptr;          // FP32 master: per layer W[27][cin][cout] then bias[cout]
  float *grad = nullptr, *adam_m = nullptr, *adam_v = nullptr;
  bf16 *packt[kLayers], *packtb[kLayers];  // forward / data-gradient weights packed for k_conv3_tc
  int *tc_err;                       // set by a tensor-core conv whose bounded wait ran out
  long long poff[kLayers];          // offset of each layer's weights in params
  // activations (bf16 channels-last)
  bf16 *x0;                          // input 16 ch, level 0
  bf16 *e1, *p1, *e2, *p2, *e3, *p3, *e4;  // encoder
  bf16 *u3, *d3, *u2, *d2, *u1;            // decoder inputs/outputs
  float *yout;                      // output 8 ch (channel 0 used), level 0
  float *target;                    // training target, level 0
  // backward buffers
  float *dy_out;                    // dL/dy (8 ch)
  bf16 *gbuf, *gbuf2;               // bf16 gradients
  float *acc_e1, *acc_e2, *acc_e3;  // FP32 gradients of the encoder activations
  float *tmp;                       // FP32 gradient of a decoder output
  float *wscratch;                  // bias (64) + padded weight gradient of one layer
  float *xin_f32, *yhost_f32;       // staging of the host-array entry points
  double *loss_dev;                 // loss
  double *sums_dev;                 // scales and sums of the current solve's start (see k_scales)
  double *partials;                 // block partials of the reductions (kRedBlocks x 4)
  float *pbase;                     // start pressure of the current solve (FP32, interior)
  double *loss_host, *line_host;    // pinned mirrors
  const float *r32[2] = {nullptr, nullptr};  // FP32 split defect of the current solve's start
  bool have_features = false;       // x0 / pbase / scale hold the current solve's start
  long long step = 0;               // Adam steps taken
  bool have_target = false;         // a training pair is recorded
  cudaStream_t stream = 0;          // stream of the attached context (training)
  void *arena = nullptr;
  size_t arena_bytes = 0;
  std::string err;
};

namespace {

// cuTensorMapEncodeTiled from the driver (no link-time dependency on libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<EncodeTiledFn>(f);
  }();
  return fn;
}

// TMA map of a channels-last bf16 activation [D][H][W][C] with the halo box of
// k_conv3_tc: 8 channels x 10 x 18 voxels of one plane.
cudaError_t halo_map(CUtensorMap *m, const bf16 *X, int C, int W, int H, int D) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn) return cudaErrorNotSupported;
  const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)D};
  const cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
  const cuuint32_t box[4] = {8, (cuuint32_t)tc::HX, (cuuint32_t)tc::HY, 1};
  const cuuint32_t es[4] = {1, 1, 1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16 *>(X), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// One tensor-core convolution: input X (CIN channels), weights Wt packed with
// NT output channels, output channels co0 .. co0+COUT-1 of Y (ystride
// channels per voxel, the first ywrite of them written).  Persistent grid: as
// many CTAs as fit on the SMs (shared memory, TMEM columns, registers), at
// most one per work unit; the chunk length L (<= LMAX planes) is the largest
// that still gives every CTA a unit.
template <int CIN, int COUT, int STAGES, int LMAX, bool RELU, bool OUTF>
cudaError_t conv_tc(const bf16 *X, const bf16 *Wt, int NT, int co0, const float *bias, int nbias, void *Y, int ystride,
                    int ywrite, int W, int H, int D, int *err, cudaStream_t st) {
  constexpr size_t smem = tc::smem_bytes<CIN, COUT, STAGES>();
  static_assert(smem <= 232448, "shared memory per CTA");
  auto kern = k_conv3_tc<CIN, COUT, STAGES, LMAX, RELU, OUTF>;
  // resident CTAs on the device, computed once per instantiation (a
  // function-local static: thread-safe initialisation); 0 after a failure
  static const int grid_cap = [&]() -> int {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
      return 0;
    int dev = 0, sms = 0, smem_sm = 0;
    cudaFuncAttributes fa;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, kern) != cudaSuccess)
      return 0;
    // resident CTAs per SM: shared memory (1 KB reserved per CTA), TMEM
    // columns, registers, threads
    constexpr int tcap = 512 / tc::tmem_cols(COUT, LMAX);
    int occ = smem_sm / (int)(smem + fa.sharedSizeBytes + 1024);
    occ = occ < tcap ? occ : tcap;
    const int regs = fa.numRegs > 0 ? fa.numRegs : 64;
    occ = occ < 65536 / (regs * tc::THREADS) ? occ : 65536 / (regs * tc::THREADS);
    occ = occ < 2048 / tc::THREADS ? occ : 2048 / tc::THREADS;
    return sms * (occ > 0 ? occ : 1);
  }();
  if (!grid_cap) return cudaErrorInvalidConfiguration;
  CUtensorMap map;
  cudaError_t e = halo_map(&map, X, CIN, W, H, D);
  if (e != cudaSuccess) return e;
  const int tiles = ((W + tc::TX - 1) / tc::TX) * ((H + tc::TY - 1) / tc::TY);
  const long long span = (long long)tiles * D / grid_cap;
  const int L = span < 1 ? 1 : (span > LMAX ? LMAX : (int)span);
  const int nunits = tiles * ((D + L - 1) / L);
  const int grid = nunits < grid_cap ? nunits : grid_cap;
  DSG_COUNT kern<<<grid, tc::THREADS, smem, st>>>(map, Wt, NT, co0, bias, nbias, Y, ystride, ywrite, W, H, D, L,
                                                  err);
  return cudaGetLastError();
}

template <int CIN, int COUT>
cudaError_t wgrad_launch(const bf16 *X, const bf16 *G, float *dW, int W, int H, int D, cudaStream_t st) {
  const size_t smem = ((size_t)(BZ + 2) * (CTY + 2) * (CTX + 2) * CIN + (size_t)BZ * CTY * CTX * COUT) * sizeof(bf16);
  // set once per instantiation (a function-local static: thread-safe initialisation)
  static const cudaError_t attr =
      cudaFuncSetAttribute(k_conv3_wgrad<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (attr != cudaSuccess) return attr;
  const dim3 grid((unsigned)((W + CTX - 1) / CTX), (unsigned)((H + CTY - 1) / CTY), (unsigned)((D + BZ - 1) / BZ));
  DSG_COUNT k_conv3_wgrad<CIN, COUT><<<grid, 256, smem, st>>>(X, G, dW, W, H, D);
  return cudaGetLastError();
}

// forward conv of layer l (tensor cores); the 64 -> 64 layer runs as two
// launches of 32 output channels each (its weights do not fit in one CTA's
// shared memory next to the halo).
cudaError_t conv_fwd(dsg_net *n, int l, const bf16 *X, void *Y, cudaStream_t st) {
  const int lv = kDefs[l].level;
  const int W = n->W[lv], H = n->H[lv], D = n->D[lv];
  const float *bias = n->params + n->poff[l] + 27LL * kDefs[l].cin * kDefs[l].cout;
  const int nb = kDefs[l].cout;
  const bf16 *Wt = n->packt[l];
  int *err = n->tc_err;
  switch (l) {
    case 0: return conv_tc<16, 16, 4, 8, true, false>(X, Wt, 16, 0, bias, nb, Y, 16, 16, W, H, D, err, st);
    case 1: return conv_tc<16, 32, 4, 4, true, false>(X, Wt, 32, 0, bias, nb, Y, 32, 32, W, H, D, err, st);
    case 2: return conv_tc<32, 64, 4, 4, true, false>(X, Wt, 64, 0, bias, nb, Y, 64, 64, W, H, D, err, st);
    case 3: {
      cudaError_t e = conv_tc<64, 32, 3, 8, true, false>(X, Wt, 64, 0, bias, nb, Y, 64, 32, W, H, D, err, st);
      if (e != cudaSuccess) return e;
      return conv_tc<64, 32, 3, 8, true, false>(X, Wt, 64, 32, bias, nb, Y, 64, 32, W, H, D, err, st);
    }
    case 4: return conv_tc<64, 32, 3, 8, true, false>(X, Wt, 32, 0, bias, nb, Y, 32, 32, W, H, D, err, st);
    case 5: return conv_tc<32, 16, 4, 8, true, false>(X, Wt, 16, 0, bias, nb, Y, 16, 16, W, H, D, err, st);
    default: return conv_tc<16, 16, 4, 8, false, true>(X, Wt, 16, 0, bias, nb, Y, 8, 8, W, H, D, err, st);
  }
}

// data gradient of layer l: dX (bf16, cinp channels) from G (bf16, grad_ch(l)
// channels) with the flipped, transposed weights
cudaError_t conv_dgrad(dsg_net *n, int l, const bf16 *G, bf16 *dX, cudaStream_t st) {
  const int lv = kDefs[l].level;
  const int W = n->W[lv], H = n->H[lv], D = n->D[lv];
  const bf16 *Wt = n->packtb[l];
  int *err = n->tc_err;
  switch (l) {
    case 1: return conv_tc<32, 16, 4, 8, false, false>(G, Wt, 16, 0, nullptr, 0, dX, 16, 16, W, H, D, err, st);
    case 2: return conv_tc<64, 32, 3, 8, false, false>(G, Wt, 32, 0, nullptr, 0, dX, 32, 32, W, H, D, err, st);
    case 3: {
      cudaError_t e = conv_tc<64, 32, 3, 8, false, false>(G, Wt, 64, 0, nullptr, 0, dX, 64, 32, W, H, D, err, st);
      if (e != cudaSuccess) return e;
      return conv_tc<64, 32, 3, 8, false, false>(G, Wt, 64, 32, nullptr, 0, dX, 64, 32, W, H, D, err, st);
    }
    case 4: return conv_tc<32, 64, 4, 4, false, false>(G, Wt, 64, 0, nullptr, 0, dX, 64, 64, W, H, D, err, st);
    case 5: return conv_tc<16, 32, 4, 4, false, false>(G, Wt, 32, 0, nullptr, 0, dX, 32, 32, W, H, D, err, st);
    case 6: return conv_tc<16, 16, 4, 8, false, false>(G, Wt, 16, 0, nullptr, 0, dX, 16, 16, W, H, D, err, st);
    default: return cudaErrorInvalidValue;
  }
}

// weight gradient of layer l into n->grad (FP32 [27][cinp][coutp] scratch then folded)
cudaError_t conv_wgrad(dsg_net *n, int l, const bf16 *X, const bf16 *G, float *dWpad, cudaStream_t st) {
  const int lv = kDefs[l].level;
  const int W = n->W[lv], H = n->H[lv], D = n->D[lv];
  switch (l) {
    case 0: return wgrad_launch<16, 16>(X, G, dWpad, W, H, D, st);
    case 1: return wgrad_launch<16, 32>(X, G, dWpad, W, H, D, st);
    case 2: return wgrad_launch<32, 64>(X, G, dWpad, W, H, D, st);
    case 3: return wgrad_launch<64, 64>(X, G, dWpad, W, H, D, st);
    case 4: return wgrad_launch<64, 32>(X, G, dWpad, W, H, D, st);
    case 5: return wgrad_launch<32, 16>(X, G, dWpad, W, H, D, st);
    default: return wgrad_launch<16, 16>(X, G, dWpad, W, H, D, st);
  }
}

// fold a padded [27][kin][kout] gradient into the logical [27][cin][cout] one
__global__ void k_fold_wgrad(float *__restrict__ dst, const float *__restrict__ src, int cin, int cout, int kin,
                             int kout) {
  const int n = 27 * cin * cout;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int co = q % cout, ci = (q / cout) % cin, tap = q / (cout * cin);
    dst[q] = src[((size_t)tap * kin + ci) * kout + co];
  }
}

int net_fail(dsg_net *n, cudaError_t e, const char *where) {
  char buf[256];
  snprintf(buf, sizeof buf, "CUDA error %d (%s) at %s", (int)e, cudaGetErrorString(e), where);
  if (n) n->err = buf;
  return dsg::set_error(nullptr, e == cudaErrorMemoryAllocation ? DSG_E_NOMEM : DSG_E_CUDA, "%s", buf);
}

#define NCK(n, expr)                                       \
  do {                                                     \
    cudaError_t _e = (expr);                               \
    if (_e != cudaSuccess) return net_fail((n), _e, #expr); \
  } while (0)

size_t vox(const dsg_net *n, int lv) { return (size_t)n->W[lv] * n->H[lv] * n->D[lv]; }

// Output channels of the forward tensor-core conv of layer l (padded to 16).
inline int tc_nout(int l) { return kDefs[l].coutp < 16 ? 16 : kDefs[l].coutp; }

int repack(dsg_net *n, cudaStream_t st) {
  for (int l = 0; l < kLayers; l++) {
    const LayerDef &L = kDefs[l];
    const float *Wt = n->params + n->poff[l];
    DSG_COUNT k_pack_tc<<<eblocks((size_t)27 * L.cinp * tc_nout(l)), 256, 0, st>>>(Wt, n->packt[l], L.cin, L.cout,
                                                                                    L.cinp, tc_nout(l), 0);
    if (l > 0)  // data gradient: K = the forward outputs (gradient channels), N = the forward inputs
      DSG_COUNT k_pack_tc<<<eblocks((size_t)27 * grad_ch(l) * L.cinp), 256, 0, st>>>(Wt, n->packtb[l], L.cin, L.cout,
                                                                                      grad_ch(l), L.cinp, 1);
  }
  NCK(n, cudaGetLastError());
  return DSG_OK;
}

// A tensor-core conv whose bounded wait ran out leaves a flag; read (with a
// synchronisation) by the entry points that synchronise anyway.
int check_tc(dsg_net *n) {
  int f = 0;
  NCK(n, cudaMemcpy(&f, n->tc_err, sizeof f, cudaMemcpyDeviceToHost));
  if (f) {
    n->err = "tensor-core convolution: a bounded wait for a TMA copy or an MMA ran out";
    return dsg::set_error(nullptr, DSG_E_CUDA, "%s", n->err.c_str());
  }
  return DSG_OK;
}

int forward(dsg_net *n, cudaStream_t st) {
  NCK(n, conv_fwd(n, 0, n->x0, n->e1, st));
  DSG_COUNT k_pool<<<eblocks(vox(n, 1) * 2), 256, 0, st>>>(n->e1, n->p1, n->W[0], n->H[0], n->D[0], 16);
  NCK(n, conv_fwd(n, 1, n->p1, n->e2, st));
  DSG_COUNT k_pool<<<eblocks(vox(n, 2) * 4), 256, 0, st>>>(n->e2, n->p2, n->W[1], n->H[1], n->D[1], 32);
  NCK(n, conv_fwd(n, 2, n->p2, n->e3, st));
  DSG_COUNT k_pool<<<eblocks(vox(n, 3) * 8), 256, 0, st>>>(n->e3, n->p3, n->W[2], n->H[2], n->D[2], 64);
  NCK(n, conv_fwd(n, 3, n->p3, n->e4, st));
  DSG_COUNT k_upadd<<<eblocks(vox(n, 2) * 8), 256, 0, st>>>(n->e4, n->e3, n->u3, n->W[2], n->H[2], n->D[2], 64);
  NCK(n, conv_fwd(n, 4, n->u3, n->d3, st));
  DSG_COUNT k_upadd<<<eblocks(vox(n, 1) * 4), 256, 0, st>>>(n->d3, n->e2, n->u2, n->W[1], n->H[1], n->D[1], 32);
  NCK(n, conv_fwd(n, 5, n->u2, n->d2, st));
  DSG_COUNT k_upadd<<<eblocks(vox(n, 0) * 2), 256, 0, st>>>(n->d2, n->e1, n->u1, n->W[0], n->H[0], n->D[0], 16);
  NCK(n, conv_fwd(n, 6, n->u1, n->yout, st));
  NCK(n, cudaGetLastError());
  return DSG_OK;
}

// One layer's backward: dacc (FP32 dL/d(output after activation), coutp channels)
// -> G = bf16(dacc * relu'), bias grad, weight grad (into grad), and the data
// gradient dX (bf16, cinp channels) if want_dx.
int layer_back(dsg_net *n, int l, const float *dacc, const bf16 *act_out, const bf16 *X, bf16 *dX, float *wscratch,
               cudaStream_t st) {
  const LayerDef &L = kDefs[l];
  const int lv = L.level;
  const size_t nv = vox(n, lv);
  float *dbias = n->grad + n->poff[l] + 27LL * L.cin * L.cout;
  // G into gbuf (coutp channels); the bias gradient of padded channels is dropped
  NCK(n, cudaMemsetAsync(wscratch, 0, (size_t)64 * sizeof(float), st));
  const int gc = grad_ch(l);
  DSG_COUNT k_relu_back<<<eblocks(nv * gc / 8), 256, 0, st>>>(dacc, act_out, n->gbuf, wscratch, nv, gc, L.relu ? 1 : 0);
  NCK(n, cudaMemcpyAsync(dbias, wscratch, L.cout * sizeof(float), cudaMemcpyDeviceToDevice, st));
  float *wpad = wscratch + 64;
  const size_t wn = (size_t)27 * L.cinp * gc;
  NCK(n, cudaMemsetAsync(wpad, 0, wn * sizeof(float), st));
  NCK(n, conv_wgrad(n, l, X, n->gbuf, wpad, st));
  DSG_COUNT k_fold_wgrad<<<eblocks(27 * L.cin * L.cout), 256, 0, st>>>(n->grad + n->poff[l], wpad, L.cin, L.cout,
                                                                       L.cinp, gc);
  if (dX) NCK(n, conv_dgrad(n, l, n->gbuf, dX, st));
  NCK(n, cudaGetLastError());
  return DSG_OK;
}

// Backward pass of the U-Net for the loss of the current output/target;
// parameter gradients into n->grad.
int backward(dsg_net *n, cudaStream_t st) {
  const size_t v0 = vox(n, 0), v1 = vox(n, 1), v2 = vox(n, 2), v3 = vox(n, 3);
  float *ws = n->wscratch;
  int rc;
  NCK(n, cudaMemsetAsync(n->grad, 0, DSG_NET_PARAMS * sizeof(float), st));
  NCK(n, cudaMemsetAsync(n->acc_e1, 0, v0 * 16 * sizeof(float), st));
  NCK(n, cudaMemsetAsync(n->acc_e2, 0, v1 * 32 * sizeof(float), st));
  NCK(n, cudaMemsetAsync(n->acc_e3, 0, v2 * 64 * sizeof(float), st));
  // D1: y = conv6(u1), u1 = up(d2) + e1
  if ((rc = layer_back(n, 6, n->dy_out, nullptr, n->u1, n->gbuf2, ws, st))) return rc;
  DSG_COUNT k_acc_bf16<<<eblocks(v0 * 2), 256, 0, st>>>(n->acc_e1, n->gbuf2, v0 * 16);
  DSG_COUNT k_upadd_back<<<eblocks(v1 * 2), 256, 0, st>>>(n->gbuf2, n->tmp, n->W[0], n->H[0], n->D[0], 16);
  // D2: d2 = relu(conv5(u2)), u2 = up(d3) + e2
  if ((rc = layer_back(n, 5, n->tmp, n->d2, n->u2, n->gbuf2, ws, st))) return rc;
  DSG_COUNT k_acc_bf16<<<eblocks(v1 * 4), 256, 0, st>>>(n->acc_e2, n->gbuf2, v1 * 32);
  DSG_COUNT k_upadd_back<<<eblocks(v2 * 4), 256, 0, st>>>(n->gbuf2, n->tmp, n->W[1], n->H[1], n->D[1], 32);
  // D3: d3 = relu(conv4(u3)), u3 = up(e4) + e3
  if ((rc = layer_back(n, 4, n->tmp, n->d3, n->u3, n->gbuf2, ws, st))) return rc;
  DSG_COUNT k_acc_bf16<<<eblocks(v2 * 8), 256, 0, st>>>(n->acc_e3, n->gbuf2, v2 * 64);
  DSG_COUNT k_upadd_back<<<eblocks(v3 * 8), 256, 0, st>>>(n->gbuf2, n->tmp, n->W[2], n->H[2], n->D[2], 64);
  // E4: e4 = relu(conv3(p3)), p3 = pool(e3)
  if ((rc = layer_back(n, 3, n->tmp, n->e4, n->p3, n->gbuf2, ws, st))) return rc;
  DSG_COUNT k_pool_back_acc<<<eblocks(v2 * 8), 256, 0, st>>>(n->gbuf2, n->acc_e3, n->W[2], n->H[2], n->D[2], 64);
  // E3: e3 = relu(conv2(p2)), p2 = pool(e2)
  if ((rc = layer_back(n, 2, n->acc_e3, n->e3, n->p2, n->gbuf2, ws, st))) return rc;
  DSG_COUNT k_pool_back_acc<<<eblocks(v1 * 4), 256, 0, st>>>(n->gbuf2, n->acc_e2, n->W[1], n->H[1], n->D[1], 32);
  // E2: e2 = relu(conv1(p1)), p1 = pool(e1)
  if ((rc = layer_back(n, 1, n->acc_e2, n->e2, n->p1, n->gbuf2, ws, st))) return rc;
  DSG_COUNT k_pool_back_acc<<<eblocks(v0 * 2), 256, 0, st>>>(n->gbuf2, n->acc_e1, n->W[0], n->H[0], n->D[0], 16);
  // E1: e1 = relu(conv0(x0)); no input gradient
  if ((rc = layer_back(n, 0, n->acc_e1, n->e1, n->x0, nullptr, ws, st))) return rc;
  NCK(n, cudaGetLastError());
  return DSG_OK;
}

int loss_grad(dsg_net *n, cudaStream_t st) {
  NCK(n, cudaMemsetAsync(n->loss_dev, 0, sizeof(double), st));
  DSG_COUNT k_mse<<<eblocks(vox(n, 0)), 256, 0, st>>>(n->yout, n->target, n->dy_out, n->loss_dev, vox(n, 0));
  NCK(n, cudaGetLastError());
  return DSG_OK;
}

// x (FP32 host, 3 channels per voxel) -> n->x0 (bf16, 16 channels)
__global__ void k_input_from_f32(bf16 *__restrict__ x0, const float *__restrict__ x, size_t nvox) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (size_t)gridDim.x * blockDim.x)
#pragma unroll
    for (int c = 0; c < 16; c++) x0[v * 16 + c] = __float2bfloat16(c < kIn ? x[v * kIn + c] : 0.f);
}

__global__ void k_output_ch0(float *__restrict__ y, const float *__restrict__ yout, size_t nvox) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (size_t)gridDim.x * blockDim.x)
    y[v] = yout[v * 8];
}

// splitmix64-based normal deviates for He initialisation (host)
double host_normal(uint64_t &state) {
  auto next = [&]() {
    uint64_t z = (state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  };
  const double u1 = next(), u2 = next();
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

}  // namespace

namespace dsg {
namespace nn {

// Solver hooks (used by dsg.cu): features of the current pressure system into
// the network input; optional training target from the solved pressure.
int net_features(dsg_net *n, const double *cc, const double *rhs, const double *p, const double *pprev,
                 const float *const r32[2], const double *red, Dims d, double lengthsize, cudaStream_t st) {
  if (n->W[0] != d.nx - 2 || n->H[0] != d.ny - 2 || n->D[0] != d.nz - 2)
    return dsg::set_error(nullptr, DSG_E_ARG, "network sized %dx%dx%d, grid interior %dx%dx%d", n->W[0], n->H[0],
                          n->D[0], d.nx - 2, d.ny - 2, d.nz - 2);
  const double h1 = lengthsize / (d.nx - 2);
  const Split sp{(d.nx - 2) >> 1, d.ny - 2, d.nz - 2};
  DSG_COUNT k_sumsq_partials<<<kRedBlocks, 256, 0, st>>>(n->partials, p, d);
  DSG_COUNT k_fold<<<1, 256, 0, st>>>(n->sums_dev, n->partials, kRedBlocks, 1);
  DSG_COUNT k_scales<<<1, 32, 0, st>>>(n->sums_dev, red, (double)(d.nx - 2) * (d.ny - 2) * (d.nz - 2), h1 * h1);
  const dim3 blk(32, 8), grid((unsigned)((d.nx - 2 + 31) / 32), (unsigned)((d.ny - 2 + 7) / 8), (unsigned)(d.nz - 2));
  DSG_COUNT k_features<<<grid, blk, 0, st>>>(n->x0, n->pbase, r32[0], r32[1], sp, cc, rhs, p, pprev, n->sums_dev, d);
  NCK(n, cudaGetLastError());
  n->r32[0] = r32[0];
  n->r32[1] = r32[1];
  n->have_features = true;
  return DSG_OK;
}

int net_target(dsg_net *n, const double *p, Dims d, cudaStream_t st) {
  if (!n->have_features) return DSG_OK;
  const dim3 blk(32, 8), grid((unsigned)((d.nx - 2 + 31) / 32), (unsigned)((d.ny - 2 + 7) / 8), (unsigned)(d.nz - 2));
  DSG_COUNT k_target<<<grid, blk, 0, st>>>(n->target, p, n->pbase, n->sums_dev, d);
  NCK(n, cudaGetLastError());
  n->have_target = true;
  n->stream = st;
  return DSG_OK;
}

int net_correction(dsg_net *n, const double *a, const double *b, const double *c, Dims d, double *relres_pred,
                   double *alpha, cudaStream_t st) {
  if (!n->have_features) return dsg::set_error(nullptr, DSG_E_STATE, "network features not computed");
  int rc = forward(n, st);
  if (rc) return rc;
  const Split sp{(d.nx - 2) >> 1, d.ny - 2, d.nz - 2};
  DSG_COUNT k_line_partials<<<kRedBlocks, 256, 0, st>>>(n->partials, n->r32[0], n->r32[1], sp, a, b, c, n->yout, d);
  DSG_COUNT k_fold<<<1, 256, 0, st>>>(n->sums_dev + 2, n->partials, kRedBlocks, 3);
  NCK(n, cudaMemcpyAsync(n->line_host, n->sums_dev, 8 * sizeof(double), cudaMemcpyDeviceToHost, st));
  NCK(n, cudaStreamSynchronize(st));
  rc = check_tc(n);
  if (rc) return rc;
  const double *h = n->line_host;
  const double s_r = h[6], rr = h[2], rt = s_r * h[3], tt = s_r * s_r * h[4], bb = h[5];
  if (!isfinite(rr) || !isfinite(rt) || !isfinite(tt) || !isfinite(bb))
    return dsg::set_error(nullptr, DSG_E_NONFINITE, "non-finite network correction (%g, %g, %g)", rr, rt, tt);
  // defect of p + alpha e: |r - alpha t|^2 = rr - 2 alpha rt + alpha^2 tt, least at alpha = rt / tt
  *alpha = tt > 0.0 ? rt / tt : 0.0;
  double left = tt > 0.0 ? rr - rt * rt / tt : rr;
  if (left < 0.0) left = 0.0;
  *relres_pred = bb > 0.0 ? sqrt(left) / sqrt(bb) : sqrt(left);
  return DSG_OK;
}

int net_apply(dsg_net *n, double *p, double alpha, Dims d, cudaStream_t st) {
  const dim3 blk(32, 8), grid((unsigned)((d.nx - 2 + 31) / 32), (unsigned)((d.ny - 2 + 7) / 8), (unsigned)(d.nz - 2));
  DSG_COUNT k_apply_corr<<<grid, blk, 0, st>>>(p, n->yout, n->sums_dev, alpha, d);
  NCK(n, cudaGetLastError());
  return DSG_OK;
}

void net_begin_solve(dsg_net *n) { n->have_features = false; }


}  // namespace nn
}  // namespace dsg

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

int64_t dsg_net_param_count(void) { return DSG_NET_PARAMS; }

int dsg_net_create(int W, int H, int D, uint64_t seed, dsg_net **out) {
  if (!out) return dsg::set_error(nullptr, DSG_E_ARG, "null output");
  *out = nullptr;
  if (W < 8 || H < 8 || D < 8 || (W % 8) || (H % 8) || (D % 8))
    return dsg::set_error(nullptr, DSG_E_ARG, "network grid %dx%dx%d: sides must be multiples of 8", W, H, D);
  dsg_net *n = new dsg_net();
  for (int l = 0; l < 4; l++) {
    n->W[l] = W >> l;
    n->H[l] = H >> l;
    n->D[l] = D >> l;
  }
  long long off = 0;
  for (int l = 0; l < kLayers; l++) {
    n->poff[l] = off;
    off += layer_params(l);
  }
  const size_t v0 = vox(n, 0), v1 = vox(n, 1), v2 = vox(n, 2), v3 = vox(n, 3);
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  std::vector<std::pair<void **, size_t>> plan;
  plan.push_back({(void **)&n->params, up(DSG_NET_PARAMS * 4)});
  plan.push_back({(void **)&n->grad, up(DSG_NET_PARAMS * 4)});
  plan.push_back({(void **)&n->adam_m, up(DSG_NET_PARAMS * 4)});
  plan.push_back({(void **)&n->adam_v, up(DSG_NET_PARAMS * 4)});
  for (int l = 0; l < kLayers; l++) {
    const LayerDef &L = kDefs[l];
    plan.push_back({(void **)&n->packt[l], up((size_t)27 * L.cinp * tc_nout(l) * sizeof(bf16))});
    plan.push_back({(void **)&n->packtb[l], up((size_t)27 * grad_ch(l) * L.cinp * sizeof(bf16))});
  }
  plan.push_back({(void **)&n->tc_err, 256});
  plan.push_back({(void **)&n->x0, up(v0 * 16 * 2)});
  plan.push_back({(void **)&n->e1, up(v0 * 16 * 2)});
  plan.push_back({(void **)&n->p1, up(v1 * 16 * 2)});
  plan.push_back({(void **)&n->e2, up(v1 * 32 * 2)});
  plan.push_back({(void **)&n->p2, up(v2 * 32 * 2)});
  plan.push_back({(void **)&n->e3, up(v2 * 64 * 2)});
  plan.push_back({(void **)&n->p3, up(v3 * 64 * 2)});
  plan.push_back({(void **)&n->e4, up(v3 * 64 * 2)});
  plan.push_back({(void **)&n->u3, up(v2 * 64 * 2)});
  plan.push_back({(void **)&n->d3, up(v2 * 32 * 2)});
  plan.push_back({(void **)&n->u2, up(v1 * 32 * 2)});
  plan.push_back({(void **)&n->d2, up(v1 * 16 * 2)});
  plan.push_back({(void **)&n->u1, up(v0 * 16 * 2)});
  plan.push_back({(void **)&n->yout, up(v0 * 8 * 4)});
  plan.push_back({(void **)&n->target, up(v0 * 4)});
  plan.push_back({(void **)&n->dy_out, up(v0 * 16 * 4)});
  plan.push_back({(void **)&n->acc_e1, up(v0 * 16 * 4)});
  plan.push_back({(void **)&n->acc_e2, up(v1 * 32 * 4)});
  plan.push_back({(void **)&n->acc_e3, up(v2 * 64 * 4)});
  plan.push_back({(void **)&n->tmp, up(v1 * 16 * 4 > v2 * 32 * 4 ? v1 * 16 * 4 : v2 * 32 * 4)});
  plan.push_back({(void **)&n->gbuf, up(v0 * 16 * 2)});
  plan.push_back({(void **)&n->gbuf2, up(v0 * 16 * 2)});
  plan.push_back({(void **)&n->wscratch, up((64 + 27 * 64 * 64) * 4)});
  plan.push_back({(void **)&n->xin_f32, up(v0 * kIn * 4)});
  plan.push_back({(void **)&n->yhost_f32, up(v0 * 4)});
  plan.push_back({(void **)&n->loss_dev, 256});
  plan.push_back({(void **)&n->sums_dev, 256});
  plan.push_back({(void **)&n->partials, up((size_t)dsg::kRedBlocks * 4 * sizeof(double))});
  plan.push_back({(void **)&n->pbase, up(v0 * 4)});
  size_t total = 0;
  for (auto &e : plan) total += e.second;
  cudaError_t e = cudaMalloc(&n->arena, total);
  if (e == cudaSuccess) e = cudaMemset(n->arena, 0, total);
  if (e == cudaSuccess) e = cudaMallocHost(&n->loss_host, sizeof(double));
  if (e == cudaSuccess) e = cudaMallocHost(&n->line_host, 8 * sizeof(double));
  if (e != cudaSuccess) {
    int rc = net_fail(n, e, "dsg_net_create");
    dsg_net_destroy(n);
    return rc;
  }
  n->arena_bytes = total;
  char *p = (char *)n->arena;
  for (auto &ent : plan) {
    *ent.first = p;
    p += ent.second;
  }
  // He initialisation of the weights, zero biases
  std::vector<float> h(DSG_NET_PARAMS, 0.f);
  uint64_t state = seed * 0x2545F4914F6CDD1DULL + 1;
  for (int l = 0; l < kLayers; l++) {
    const double sd = sqrt(2.0 / (27.0 * kDefs[l].cin)) * (l == kLayers - 1 ? 0.1 : 1.0);
    for (long long q = 0; q < 27LL * kDefs[l].cin * kDefs[l].cout; q++)
      h[n->poff[l] + q] = (float)(sd * host_normal(state));
  }
  e = cudaMemcpy(n->params, h.data(), DSG_NET_PARAMS * sizeof(float), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    int rc = net_fail(n, e, "upload params");
    dsg_net_destroy(n);
    return rc;
  }
  int rc = repack(n, 0);
  if (rc == DSG_OK) {
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) rc = net_fail(n, e, "repack");
  }
  if (rc) {
    dsg_net_destroy(n);
    return rc;
  }
  *out = n;
  return DSG_OK;
}

void dsg_net_destroy(dsg_net *n) {
  if (!n) return;
  if (n->arena) cudaFree(n->arena);
  if (n->loss_host) cudaFreeHost(n->loss_host);
  if (n->line_host) cudaFreeHost(n->line_host);
  delete n;
}

int dsg_net_get_params(dsg_net *n, float *host, int64_t count) {
  if (!n || !host || count != DSG_NET_PARAMS) return dsg::set_error(nullptr, DSG_E_ARG, "bad parameter buffer");
  NCK(n, cudaMemcpy(host, n->params, DSG_NET_PARAMS * sizeof(float), cudaMemcpyDeviceToHost));
  return DSG_OK;
}

int dsg_net_set_params(dsg_net *n, const float *host, int64_t count) {
  if (!n || !host || count != DSG_NET_PARAMS) return dsg::set_error(nullptr, DSG_E_ARG, "bad parameter buffer");
  NCK(n, cudaMemcpy(n->params, host, DSG_NET_PARAMS * sizeof(float), cudaMemcpyHostToDevice));
  int rc = repack(n, 0);
  if (rc) return rc;
  NCK(n, cudaDeviceSynchronize());
  return DSG_OK;
}

int dsg_net_forward_host(dsg_net *n, const float *x, float *y) {
  if (!n || !x || !y) return dsg::set_error(nullptr, DSG_E_ARG, "null argument");
  const size_t v0 = vox(n, 0);
  NCK(n, cudaMemcpy(n->xin_f32, x, v0 * kIn * sizeof(float), cudaMemcpyHostToDevice));
  DSG_COUNT k_input_from_f32<<<eblocks(v0), 256>>>(n->x0, n->xin_f32, v0);
  int rc = forward(n, 0);
  if (rc) return rc;
  DSG_COUNT k_output_ch0<<<eblocks(v0), 256>>>(n->yhost_f32, n->yout, v0);
  NCK(n, cudaMemcpy(y, n->yhost_f32, v0 * sizeof(float), cudaMemcpyDeviceToHost));
  return check_tc(n);
}

int dsg_net_grad_host(dsg_net *n, const float *x, const float *t, float *loss, float *grad) {
  if (!n || !x || !t || !loss || !grad) return dsg::set_error(nullptr, DSG_E_ARG, "null argument");
  const size_t v0 = vox(n, 0);
  NCK(n, cudaMemcpy(n->xin_f32, x, v0 * kIn * sizeof(float), cudaMemcpyHostToDevice));
  DSG_COUNT k_input_from_f32<<<eblocks(v0), 256>>>(n->x0, n->xin_f32, v0);
  NCK(n, cudaMemcpy(n->target, t, v0 * sizeof(float), cudaMemcpyHostToDevice));
  int rc = forward(n, 0);
  if (!rc) rc = loss_grad(n, 0);
  if (!rc) rc = backward(n, 0);
  if (rc) return rc;
  double l = 0.0;
  NCK(n, cudaMemcpy(&l, n->loss_dev, sizeof(double), cudaMemcpyDeviceToHost));
  *loss = (float)l;
  NCK(n, cudaMemcpy(grad, n->grad, DSG_NET_PARAMS * sizeof(float), cudaMemcpyDeviceToHost));
  return check_tc(n);
}

int dsg_net_train_step(dsg_net *n, float lr, float *loss) {
  if (!n) return dsg::set_error(nullptr, DSG_E_ARG, "null network");
  if (!n->have_target) return dsg::set_error(nullptr, DSG_E_STATE, "no recorded training pair");
  cudaStream_t st = n->stream;
  int rc = forward(n, st);
  if (!rc) rc = loss_grad(n, st);
  if (!rc) rc = backward(n, st);
  if (rc) return rc;
  n->step++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)n->step), c2 = 1.f - powf(b2, (float)n->step);
  DSG_COUNT k_adam<<<eblocks(DSG_NET_PARAMS), 256, 0, st>>>(n->params, n->grad, n->adam_m, n->adam_v, DSG_NET_PARAMS,
                                                           lr, b1, b2, 1e-8f, c1, c2, 1.0f);
  rc = repack(n, st);
  if (rc) return rc;
  NCK(n, cudaMemcpyAsync(n->loss_host, n->loss_dev, sizeof(double), cudaMemcpyDeviceToHost, st));
  NCK(n, cudaStreamSynchronize(st));
  if (loss) *loss = (float)*n->loss_host;
  n->have_target = false;
  return check_tc(n);
}

int64_t dsg_net_device_bytes(const dsg_net *n) { return n ? (int64_t)n->arena_bytes : 0; }

}  // extern "C"
