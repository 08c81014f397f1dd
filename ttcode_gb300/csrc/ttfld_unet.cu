// ttfld_unet.cu -- the learned initial guess of SOLVE_WITH_SOR (no reference
// counterpart): a 3-D U-Net (4 levels, 16-32-64-64 channels, 3x3x3 kernels,
// periodic in phi, zero-padded in r and theta) that maps the state of a step
// (log E^n, log kappa_R, log rho, log dt, heating) to the relative energy
// increment delta_ER / E^n.  It is trained on the GPU by the kernels below
// on pairs captured from the solver's own solves; SOLVE_WITH_SOR then starts
// a run's first solve from its prediction instead of zero (ppsor.f:29) and
// iterates to the same tolerance, falling back to zero when the prediction
// is not better.
//
// The network works at half the grid's resolution: the features are
// averaged over 2x2x2 cells, its four levels are 1/2 .. 1/16 of the grid, and
// its output is interpolated back to the grid (trilinear).  The guess is
// worth its smooth part -- the error the red-black sweeps are slow to remove;
// the sweeps remove cell-scale error in a few iterations -- and this costs an
// eighth of a full-resolution network.  The loss is taken on the full grid.
//
// Every convolution is an implicit GEMM on the tensor cores: BF16 operands,
// FP32 accumulation, mma.sync m16n8k16 (one warp computes 16 voxels along r
// times all output channels; A = shifted input voxels x input channels,
// B = weights of one tap).  Activations are channels-last BF16 (voxel-major,
// channels contiguous), so an A fragment row is one voxel's channels.
// Backward-data is the same kernel on flipped, transposed weights; the weight
// gradient is a GEMM over voxels (A = gradient^T, B = shifted input) reduced
// with FP32 atomics (so training is not bitwise reproducible; inference is).
#include <cuda.h>
#include <cuda_bf16.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "ttfld_internal.cuh"

namespace ttfld {

typedef __nv_bfloat16 bf16;

constexpr float kLeak = 0.1f;      // LeakyReLU slope
constexpr int kFeat = 5;           // input channels
constexpr int kFeatPad = 16;       // padded to one mma K step
constexpr double kTargetScale = 0.01;  // target = delta_ER / E / 0.01

// ---- layer table -------------------------------------------------------
struct LayerSpec {
  int cin, cin_pad, cout, level;
};
// 0-7 encoder, 8-13 decoder (their inputs are [upsampled | skip] concatenations)
static const LayerSpec kLayers[14] = {
    {kFeat, 16, 16, 0}, {16, 16, 16, 0}, {16, 16, 32, 1}, {32, 32, 32, 1}, {32, 32, 64, 2},
    {64, 64, 64, 2},  {64, 64, 64, 3}, {64, 64, 64, 3}, {128, 128, 64, 2}, {64, 64, 64, 2},
    {96, 96, 32, 1},  {32, 32, 32, 1}, {48, 48, 16, 0}, {16, 16, 16, 0}};
constexpr int kNumConv = 14;

struct Level {
  int X, Y, Z;
  __host__ __device__ long long vox() const { return (long long)X * Y * Z; }
};

struct Net {
  int ready;
  int wdirty;                  // master weights changed since the BF16 copies were made
  size_t nparams;              // FP32 master parameters (weights, biases, head)
  size_t woff[kNumConv], boff[kNumConv], w16off[kNumConv], hoff;
  size_t nw16;
  float *p, *g, *m, *v;        // params, grads, Adam moments
  bf16 *w16, *w16t;            // [27][cout][cin_pad] and flipped [27][cin_pad][cout]
  long long step;
  Level full;                  // the grid (NX, NY, NZ)
  Level lv[4];                 // network levels: 1/2, 1/4, 1/8, 1/16 of the grid
  // activations (BF16, channels-last) and their gradients
  bf16 *feat, *a0, *cat0, *a12, *a13, *p0, *a2, *cat1, *a10, *a11, *p1, *a4, *cat2, *a8, *a9, *p2, *a6, *a7;
  bf16 *g_a0, *g_cat0, *g_a12, *g_a13, *g_p0, *g_a2, *g_cat1, *g_a10, *g_a11, *g_p1, *g_a4, *g_cat2, *g_a8, *g_a9,
      *g_p2, *g_a6, *g_a7;
  float *pred_half, *gpred_half;   // network output on level 0
  float *pred, *gpred, *target;    // on the grid, one channel
  unsigned char* mask;             // active cells of the grid
  double* loss_acc;
  void* act_mem;
  // dataset (captured pairs)
  int cap, count, capture_next;
  bf16* ds_feat;       // [cap][level-0 vox][kFeatPad] pooled features
  bf16* ds_target;     // [cap][grid vox]
  unsigned char* ds_mask;  // [cap][grid vox]
};

static Net* net_of(ttfld_ctx* c) { return (Net*)c->unet; }

// ---- small device helpers ---------------------------------------------
__device__ __forceinline__ uint32_t ld32(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ void mma_bf16(float* d, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// ---- convolution (forward and backward-data) ----------------------------
struct ConvArgs {
  const bf16* in;
  int in_cs, in_co, cin;   // channel stride / offset of the input buffer, cin % 16 == 0
  const bf16* w;           // [27][cout][cin]
  const float* bias;       // may be null
  bf16* out;
  int out_cs, out_co, cout;  // cout % 8 == 0
  int X, Y, Z;
  int act, accum;
};

// One warp: 16 voxels along x (r) of one (y,z) row times 16 output
// channels, over the taps t with t % KS == ks.  A CTA holds 8/KS such tiles
// and KS warps per tile; with KS > 1 the partial sums of a tile are added in
// shared memory in a fixed order (warp ks = 0 first), so the result does not
// depend on scheduling.  Small levels (a few thousand voxels, 64 channels)
// would otherwise leave most SMs idle while a few warps walk all 27 taps.
template <int KS>
__global__ void __launch_bounds__(256) conv3_fwd_kernel(ConvArgs a) {
  constexpr int TPC = 8 / KS;  // tiles per CTA
  __shared__ float red[KS > 1 ? 8 : 1][8][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int ks = w % KS;
  const long long tile = (long long)blockIdx.x * TPC + w / KS;
  const int XT = (a.X + 15) >> 4, CG = a.cout >> 4;
  const long long ntiles = (long long)XT * a.Y * a.Z * CG;
  const bool active = tile < ntiles;
  const int cg = (int)(tile % CG);
  const long long vt = tile / CG;
  const int xt = (int)(vt % XT);
  const int y = (int)((vt / XT) % a.Y);
  const int z = (int)(vt / ((long long)XT * a.Y));
  const int r = lane >> 2, cq = (lane & 3) * 2;
  const int x0 = xt * 16;
  float acc[2][4];
#pragma unroll
  for (int nb = 0; nb < 2; ++nb) acc[nb][0] = acc[nb][1] = acc[nb][2] = acc[nb][3] = 0.f;
  if (active) {
    for (int tap = ks; tap < 27; tap += KS) {
      const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
      const int zz = z + dz;
      if (zz < 0 || zz >= a.Z) continue;
      int yy = y + dy;
      yy = yy < 0 ? yy + a.Y : (yy >= a.Y ? yy - a.Y : yy);  // periodic phi
      const size_t row = ((size_t)zz * a.Y + yy) * a.X;
      const int xa = x0 + r + dx, xb = xa + 8;
      const bool va = xa >= 0 && xa < a.X, vb = xb >= 0 && xb < a.X;
      const bf16* pa = a.in + (row + (size_t)(va ? xa : 0)) * a.in_cs + a.in_co + cq;
      const bf16* pb = a.in + (row + (size_t)(vb ? xb : 0)) * a.in_cs + a.in_co + cq;
      const bf16* wt = a.w + ((size_t)tap * a.cout + cg * 16) * a.cin;
      for (int kc = 0; kc < a.cin; kc += 16) {
        const uint32_t a0 = va ? ld32(pa + kc) : 0u;
        const uint32_t a1 = vb ? ld32(pb + kc) : 0u;
        const uint32_t a2 = va ? ld32(pa + kc + 8) : 0u;
        const uint32_t a3 = vb ? ld32(pb + kc + 8) : 0u;
#pragma unroll
        for (int nb = 0; nb < 2; ++nb) {
          const bf16* wp = wt + (size_t)(nb * 8 + r) * a.cin + kc + cq;
          mma_bf16(acc[nb], a0, a1, a2, a3, ld32(wp), ld32(wp + 8));
        }
      }
    }
  }
  if (KS > 1) {
#pragma unroll
    for (int q = 0; q < 8; ++q) red[w][q][lane] = acc[q >> 2][q & 3];
    __syncthreads();
    if (ks != 0) return;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      float v = red[w][q][lane];
      for (int o = 1; o < KS; ++o) v += red[w + o][q][lane];
      acc[q >> 2][q & 3] = v;
    }
  }
  if (!active) return;
  // epilogue: rows r, r+8 (voxels), columns cg*16 + nb*8 + cq, +1 (channels)
  const size_t rowo = ((size_t)z * a.Y + y) * a.X;
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    const int x = x0 + r + half * 8;
    if (x >= a.X) continue;
    bf16* po = a.out + (rowo + x) * a.out_cs + a.out_co + cg * 16 + cq;
#pragma unroll
    for (int nb = 0; nb < 2; ++nb) {
      float v0 = acc[nb][half * 2], v1 = acc[nb][half * 2 + 1];
      const int ch = cg * 16 + nb * 8 + cq;
      if (a.bias) { v0 += a.bias[ch]; v1 += a.bias[ch + 1]; }
      if (a.act) { v0 = v0 > 0.f ? v0 : kLeak * v0; v1 = v1 > 0.f ? v1 : kLeak * v1; }
      bf16* q = po + nb * 8;
      if (a.accum) { v0 += __bfloat162float(q[0]); v1 += __bfloat162float(q[1]); }
      *reinterpret_cast<uint32_t*>(q) = pack2(__float2bfloat16_rn(v0), __float2bfloat16_rn(v1));
    }
  }
}

// Shared-memory tiled form for the large levels (few output channels, many
// voxels): a CTA computes 16 (x) x 8 (y) x 2 (z) output voxels and all
// output channels.  The input tile with its one-voxel halo (18 x 10 x 4
// voxels) and, when they fit, the weights are staged in shared memory with
// every voxel/weight row padded by 8 channels, so that the 8 rows an
// A/B-fragment read touches fall in distinct banks.  Warp w computes rows
// (y0 + w, z0) and (y0 + w, z0 + 1), reusing each weight fragment for both.
// Each input voxel is then read from global memory about 2.8 times (the
// halo) instead of once per tap through the caches.
constexpr int kTX = 16, kTY = 8, kTZ = 2;
constexpr int kHX = kTX + 2, kHY = kTY + 2, kHZ = kTZ + 2;
constexpr int kHalo = kHX * kHY * kHZ;

static size_t conv_smem_bytes(int cin, int cout, bool with_w) {
  size_t b = (size_t)kHalo * (cin + 8) * 2;
  if (with_w) b += (size_t)27 * cout * (cin + 8) * 2;
  return b;
}

template <int NB>
__global__ void __launch_bounds__(256) conv3_smem_kernel(ConvArgs a, int w_in_smem) {
  extern __shared__ __align__(16) unsigned char csm[];
  const int cst = a.cin + 8;  // padded row, in bf16
  bf16* tin = reinterpret_cast<bf16*>(csm);
  bf16* tw = tin + (size_t)kHalo * cst;
  const int XT = (a.X + kTX - 1) / kTX, YT = (a.Y + kTY - 1) / kTY;
  const int bx = (int)(blockIdx.x % XT), by = (int)((blockIdx.x / XT) % YT), bz = (int)(blockIdx.x / (XT * YT));
  const int x0 = bx * kTX, y0 = by * kTY, z0 = bz * kTZ;
  const int c8n = a.cin >> 3;
  for (int q = threadIdx.x; q < kHalo * c8n; q += blockDim.x) {
    const int c8 = q % c8n, hv = q / c8n;
    const int hx = hv % kHX, hy = (hv / kHX) % kHY, hz = hv / (kHX * kHY);
    const int x = x0 + hx - 1, z = z0 + hz - 1;
    const int y = ((y0 + hy - 1) % a.Y + a.Y) % a.Y;  // periodic phi
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (x >= 0 && x < a.X && z >= 0 && z < a.Z)
      v = *reinterpret_cast<const uint4*>(a.in + (((size_t)z * a.Y + y) * a.X + x) * a.in_cs + a.in_co + c8 * 8);
    *reinterpret_cast<uint4*>(tin + (size_t)hv * cst + c8 * 8) = v;
  }
  if (w_in_smem) {
    const int rows = 27 * a.cout;
    for (int q = threadIdx.x; q < rows * c8n; q += blockDim.x) {
      const int c8 = q % c8n, row = q / c8n;
      *reinterpret_cast<uint4*>(tw + (size_t)row * cst + c8 * 8) =
          *reinterpret_cast<const uint4*>(a.w + (size_t)row * a.cin + c8 * 8);
    }
  }
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = lane >> 2, cq = (lane & 3) * 2;
  const bf16* wbase = w_in_smem ? tw : a.w;
  const int wst = w_in_smem ? cst : a.cin;
  float acc[2][NB][4];
#pragma unroll
  for (int zz = 0; zz < 2; ++zz)
#pragma unroll
    for (int nb = 0; nb < NB; ++nb) acc[zz][nb][0] = acc[zz][nb][1] = acc[zz][nb][2] = acc[zz][nb][3] = 0.f;
  for (int tap = 0; tap < 27; ++tap) {
    const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;  // 0..2: halo offsets
    const bf16* p0 = tin + ((size_t)((0 + dz) * kHY + (w + dy)) * kHX + r + dx) * cst + cq;
    const bf16* p1 = tin + ((size_t)((1 + dz) * kHY + (w + dy)) * kHX + r + dx) * cst + cq;
    const bf16* wt = wbase + (size_t)tap * a.cout * wst;
    for (int kc = 0; kc < a.cin; kc += 16) {
      const uint32_t a00 = ld32(p0 + kc), a01 = ld32(p0 + 8 * cst + kc);
      const uint32_t a02 = ld32(p0 + kc + 8), a03 = ld32(p0 + 8 * cst + kc + 8);
      const uint32_t a10 = ld32(p1 + kc), a11 = ld32(p1 + 8 * cst + kc);
      const uint32_t a12 = ld32(p1 + kc + 8), a13 = ld32(p1 + 8 * cst + kc + 8);
#pragma unroll
      for (int nb = 0; nb < NB; ++nb) {
        const bf16* wp = wt + (size_t)(nb * 8 + r) * wst + kc + cq;
        const uint32_t b0 = ld32(wp), b1 = ld32(wp + 8);
        mma_bf16(acc[0][nb], a00, a01, a02, a03, b0, b1);
        mma_bf16(acc[1][nb], a10, a11, a12, a13, b0, b1);
      }
    }
  }
  const int y = y0 + w;
  if (y >= a.Y) return;
#pragma unroll
  for (int zz = 0; zz < 2; ++zz) {
    const int z = z0 + zz;
    if (z >= a.Z) continue;
    const size_t rowo = ((size_t)z * a.Y + y) * a.X;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int x = x0 + r + half * 8;
      if (x >= a.X) continue;
      bf16* po = a.out + (rowo + x) * a.out_cs + a.out_co + cq;
#pragma unroll
      for (int nb = 0; nb < NB; ++nb) {
        float v0 = acc[zz][nb][half * 2], v1 = acc[zz][nb][half * 2 + 1];
        const int ch = nb * 8 + cq;
        if (a.bias) { v0 += a.bias[ch]; v1 += a.bias[ch + 1]; }
        if (a.act) { v0 = v0 > 0.f ? v0 : kLeak * v0; v1 = v1 > 0.f ? v1 : kLeak * v1; }
        bf16* q = po + nb * 8;
        if (a.accum) { v0 += __bfloat162float(q[0]); v1 += __bfloat162float(q[1]); }
        *reinterpret_cast<uint32_t*>(q) = pack2(__float2bfloat16_rn(v0), __float2bfloat16_rn(v1));
      }
    }
  }
}

template <int NB>
static int launch_conv_smem(cudaStream_t s, const ConvArgs& a) {
  bool with_w = conv_smem_bytes(a.cin, a.cout, true) <= 100 * 1024;
  const size_t smem = conv_smem_bytes(a.cin, a.cout, with_w);
  static size_t opted = 0;
  if (smem > 48 * 1024 && smem > opted) {
    if (cudaFuncSetAttribute(conv3_smem_kernel<NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
        cudaSuccess)
      return TTFLD_E_CUDA;
    opted = 200 * 1024;
  }
  const long long blocks = (long long)((a.X + kTX - 1) / kTX) * ((a.Y + kTY - 1) / kTY) * ((a.Z + kTZ - 1) / kTZ);
  conv3_smem_kernel<NB><<<(unsigned)blocks, 256, smem, s>>>(a, with_w ? 1 : 0);
  count_launches(1);
  TT_CHECK_LAUNCH();
  return 0;
}

// ---- tcgen05 form for the large levels ------------------------------------
// The same convolution on the 5th-generation tensor cores.  An output tile
// is M = 128 voxels (8 along x times 16 along y, one z-plane) times N = cout
// (16 or 32): 27 * cin/16 tcgen05.mma (kind::f16, BF16 x BF16 -> FP32)
// accumulate it in tensor memory, issued by one thread and completed on an
// mbarrier; four warps read the accumulators back (tcgen05.ld) for the
// epilogue.  Operands sit in shared memory without swizzle in the canonical
// K-major core-matrix layout (8 rows x 16 bytes): the input tile with its
// halo (10 x 18 x 3 voxels) channel-group-major, [cin/8][z][y][x] of 16
// bytes, so that for any tap the 8 x-voxels of an output row are one core
// matrix, consecutive rows one halo row (160 bytes) apart and the next 8
// channels one group apart; the weights likewise as [tap][cin/8][cout].
//
// The CTAs are persistent (one per SM): each stages all 27 taps' weights
// once and walks its share of the tiles.  Each 8-channel group of a tile's
// input is one 4-D tensor-memory-access copy (cp.async.bulk.tensor, box
// 8 channels x 10 x 18 x 3 voxels; the zero padding in r and theta is the
// copy's out-of-bounds fill), into a ring of two stages, so the next tile's
// input streams in while this tile's MMAs and epilogue run.  The periodic
// phi halo rows of the first and last y-tiles are fetched by a one-row copy
// into a side buffer and moved into place by the threads.
constexpr int kUX = 8, kUY = 16;
constexpr int kUHX = kUX + 2, kUHY = kUY + 2, kUHZ = 3;
constexpr int kUHalo = kUHX * kUHY * kUHZ;
constexpr int kUSlab = (kUHalo * 16 + 127) / 128 * 128;   // one channel group of a stage, 128-B aligned
constexpr int kURow = (kUHX * kUHZ * 16 + 127) / 128 * 128;  // one wrapped phi row of one channel group
constexpr long long kUmmaSpins = 1LL << 24;
__device__ int g_umma_error;  // set when a wait of the tcgen05 form ran out

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start, leading (K) and stride (M/N)
// byte offsets in 16-byte units, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t start, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((start >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}
// Instruction descriptor, kind::f16: D F32, A and B BF16, both K-major,
// N = n, M = 128.
__host__ __device__ constexpr uint32_t umma_idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ bool umma_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(saddr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for a phase of an mbarrier.
__device__ __forceinline__ bool umma_wait(uint64_t* bar, uint32_t parity) {
  long long n = 0;
  while (!umma_try_wait(bar, parity))
    if (++n > kUmmaSpins) return false;
  return true;
}

#define TT_LD16(taddr, r)                                                                                          \
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, " \
               "[%16];"                                                                                          \
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), \
                 "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),       \
                 "=r"(r[15])                                                                                     \
               : "r"(taddr))

// Shared memory of the tcgen05 form: two input stages, their side rows
// (two wrapped rows each), the weights.
static size_t conv_tc_smem_bytes(int cin, int cout) {
  const size_t G = cin / 8;
  return 2 * G * kUSlab + 2 * 2 * G * kURow + (size_t)27 * G * cout * 16 + 128;
}

struct TcTile {
  int x0, y0, z0;
  int lo, hi;  // halo rows to take from the wrapped phi rows (0 / 17, or -1)
};
__device__ __forceinline__ TcTile tc_tile(const ConvArgs& a, long long t) {
  const int XT = (a.X + kUX - 1) / kUX, YT = (a.Y + kUY - 1) / kUY;
  TcTile r;
  r.x0 = (int)(t % XT) * kUX;
  r.y0 = (int)((t / XT) % YT) * kUY;
  r.z0 = (int)(t / ((long long)XT * YT));
  r.lo = r.y0 == 0 ? 0 : -1;                 // halo row y0-1 = -1 is row Y-1
  const int h = a.Y - r.y0 + 1;              // the halo row that holds y = Y (row 0)
  r.hi = h <= kUHY - 1 ? h : -1;
  return r;
}

// Thread 0: queue the copies of a tile into stage s (8-channel groups; the
// wrapped rows into the stage's side rows), completing on bar.
__device__ __forceinline__ void tc_issue(const CUtensorMap* tm, const CUtensorMap* tr, const ConvArgs& a,
                                         const TcTile& t, unsigned char* stage, unsigned char* side, uint64_t* bar) {
  const int G = a.cin >> 3;
  const uint32_t bytes = (uint32_t)G * (kUHalo * 16 + ((t.lo >= 0) + (t.hi >= 0)) * kUHX * kUHZ * 16);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
  for (int g = 0; g < G; ++g) {
    const int c = a.in_co + 8 * g;
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(saddr(stage + (size_t)g * kUSlab)),
        "l"((unsigned long long)tm), "r"(c), "r"(t.x0 - 1), "r"(t.y0 - 1), "r"(t.z0 - 1), "r"(saddr(bar))
        : "memory");
    if (t.lo >= 0)
      asm volatile(
          "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
          "[%6];" ::"r"(saddr(side + (size_t)(2 * g) * kURow)),
          "l"((unsigned long long)tr), "r"(c), "r"(t.x0 - 1), "r"(a.Y - 1), "r"(t.z0 - 1), "r"(saddr(bar))
          : "memory");
    if (t.hi >= 0)
      asm volatile(
          "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
          "[%6];" ::"r"(saddr(side + (size_t)(2 * g + 1) * kURow)),
          "l"((unsigned long long)tr), "r"(c), "r"(t.x0 - 1), "r"(0), "r"(t.z0 - 1), "r"(saddr(bar))
          : "memory");
  }
}

template <int N>
__global__ void __launch_bounds__(128, 1) conv3_tc_kernel(ConvArgs a, const __grid_constant__ CUtensorMap tmain,
                                                          const __grid_constant__ CUtensorMap trow, long long ntiles) {
  extern __shared__ __align__(128) unsigned char usm_raw[];
  unsigned char* usm = (unsigned char*)(((uintptr_t)usm_raw + 127) & ~(uintptr_t)127);
  __shared__ __align__(8) uint64_t full_bar[2];
  __shared__ __align__(8) uint64_t mma_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int ok_sh;
  const int G = a.cin >> 3;
  unsigned char* stage[2] = {usm, usm + (size_t)G * kUSlab};
  unsigned char* side[2] = {usm + 2 * (size_t)G * kUSlab, usm + 2 * (size_t)G * kUSlab + 2 * (size_t)G * kURow};
  unsigned char* tw = usm + 2 * (size_t)G * kUSlab + 4 * (size_t)G * kURow;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(&full_bar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(&full_bar[1])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(&mma_bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    ok_sh = 1;
  }
  __syncthreads();
  // the first two tiles' input streams in while the weights are staged
  if (threadIdx.x == 0)
    for (int q = 0; q < 2; ++q) {
      const long long t = blockIdx.x + (long long)q * gridDim.x;
      if (t < ntiles) tc_issue(&tmain, &trow, a, tc_tile(a, t), stage[q], side[q], &full_bar[q]);
    }
  // the weights in batches of kWBatch loads per thread before their stores,
  // so that a thread waits one memory latency per batch, not per 16 bytes
  constexpr int kWBatch = 4;
  const int nw = 27 * G * N;
  for (int q0 = threadIdx.x; q0 < nw; q0 += kWBatch * blockDim.x) {
    uint4 v[kWBatch];
#pragma unroll
    for (int u = 0; u < kWBatch; ++u) {
      const int q = q0 + u * blockDim.x;
      if (q < nw) {
        const int n = q % N, g = (q / N) % G, t = q / (N * G);
        v[u] = *reinterpret_cast<const uint4*>(a.w + ((size_t)t * N + n) * a.cin + g * 8);
      }
    }
#pragma unroll
    for (int u = 0; u < kWBatch; ++u) {
      const int q = q0 + u * blockDim.x;
      if (q < nw) *reinterpret_cast<uint4*>(tw + (size_t)q * 16) = v[u];
    }
  }
  if (threadIdx.x < 32) {  // warp 0 owns the tensor-memory allocation
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(saddr(&tmem_base))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the weights, for the tensor core
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  long long issued = blockIdx.x + 2LL * gridDim.x;  // the next tile to queue
  int it = 0;
  bool mma_pending = false;  // thread 0: MMAs committed but not yet seen complete
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int s = it & 1;
    const TcTile t = tc_tile(a, tile);
    // 1. this tile's input has landed
    if (!umma_wait(&full_bar[s], (uint32_t)((it >> 1) & 1))) atomicExch(&ok_sh, 0);
    // 2. the wrapped phi halo rows into place
    if ((t.lo >= 0 || t.hi >= 0) && ok_sh) {
      for (int q = threadIdx.x; q < 2 * G * kUHX * kUHZ; q += blockDim.x) {
        const int which = q / (G * kUHX * kUHZ), r = q % (G * kUHX * kUHZ);
        const int g = r / (kUHX * kUHZ), v = r % (kUHX * kUHZ), hz = v / kUHX, hx = v % kUHX;
        const int hy = which ? t.hi : t.lo;
        if (hy < 0) continue;
        *reinterpret_cast<uint4*>(stage[s] + (size_t)g * kUSlab + (size_t)((hz * kUHY + hy) * kUHX + hx) * 16) =
            *reinterpret_cast<const uint4*>(side[s] + (size_t)(2 * g + which) * kURow + (size_t)v * 16);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();  // the stage is complete; the last epilogue's tensor-memory reads are done
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok_sh) break;
    // 3. the MMAs of this tile, committed to mma_bar
    if (threadIdx.x == 0) {
      const uint32_t idesc = umma_idesc(N);
      const uint32_t ta = saddr(stage[s]), wa = saddr(tw);
      const uint32_t lbo_a = kUSlab, sbo_a = kUHX * 16;
      const uint32_t lbo_b = N * 16, sbo_b = 8 * 16;
      uint32_t acc = 0;
      for (int tp = 0; tp < 27; ++tp) {
        const int dz = tp / 9, dy = (tp / 3) % 3, dx = tp % 3;
        const uint32_t voff = (uint32_t)((dz * kUHY + dy) * kUHX + dx) * 16;
        for (int k2 = 0; k2 < G; k2 += 2) {
          const uint64_t ad = umma_desc(ta + (uint32_t)k2 * lbo_a + voff, lbo_a, sbo_a);
          const uint64_t bd = umma_desc(wa + (uint32_t)((tp * G + k2) * N) * 16, lbo_b, sbo_b);
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
              "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
              : "memory");
          acc = 1;
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       saddr(&mma_bar))
                   : "memory");
      // 4. the MMAs are done: the accumulators are ready and the stage is free
      mma_pending = !umma_wait(&mma_bar, (uint32_t)(it & 1));
      if (mma_pending) ok_sh = 0;
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok_sh) break;
    // 5. queue the tile two ahead into this stage
    if (threadIdx.x == 0 && issued < ntiles) {
      tc_issue(&tmain, &trow, a, tc_tile(a, issued), stage[s], side[s], &full_bar[s]);
      issued += gridDim.x;
    }
    // 6. epilogue: warp w reads tensor-memory lanes 32w .. 32w+31 (output row m = 32w + lane)
    uint32_t r[N];
    const uint32_t tl = tmem + ((uint32_t)(32 * w) << 16);
    TT_LD16(tl, r);
    if (N == 32) TT_LD16(tl + 16, (r + 16));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    const int m = 32 * w + lane;
    const int x = t.x0 + (m & 7), y = t.y0 + (m >> 3);
    if (x < a.X && y < a.Y) {
      bf16* po = a.out + (((size_t)t.z0 * a.Y + y) * a.X + x) * a.out_cs + a.out_co;
#pragma unroll
      for (int c = 0; c < N; c += 2) {
        float v0 = __uint_as_float(r[c]), v1 = __uint_as_float(r[c + 1]);
        if (a.bias) { v0 += a.bias[c]; v1 += a.bias[c + 1]; }
        if (a.act) { v0 = v0 > 0.f ? v0 : kLeak * v0; v1 = v1 > 0.f ? v1 : kLeak * v1; }
        if (a.accum) { v0 += __bfloat162float(po[c]); v1 += __bfloat162float(po[c + 1]); }
        *reinterpret_cast<uint32_t*>(po + c) = pack2(__float2bfloat16_rn(v0), __float2bfloat16_rn(v1));
      }
    }
  }
  __syncthreads();
  if (!ok_sh) {
    if (threadIdx.x == 0) {
      atomicExch(&g_umma_error, 1);
      // the copies and MMAs in flight end before the shared and tensor
      // memory go (bounded waits): the MMAs of tile `it` if they were left
      // running, and the copies of tiles it and it+1 (a phase already
      // observed passes at once)
      if (mma_pending) {
        long long n = 0;
        while (!umma_try_wait(&mma_bar, (uint32_t)(it & 1)) && ++n < kUmmaSpins) {
        }
      }
      for (int q = 0; q < 2; ++q) {
        if (blockIdx.x + (long long)(it + q) * gridDim.x >= ntiles) continue;  // never queued
        long long n = 0;
        while (!umma_try_wait(&full_bar[(it + q) & 1], (uint32_t)(((it + q) >> 1) & 1)) && ++n < kUmmaSpins) {
        }
      }
    }
    __syncthreads();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(tmem) : "memory");
}

// cuTensorMapEncodeTiled, reached through the runtime (the library links
// only cudart).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static bool looked = false;
  if (!looked) {
    looked = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
    cudaGetLastError();
  }
  return fn;
}

// The input activations as a 4-D BF16 tensor (channels of the whole
// buffer, x, y, z), boxes of 8 channels x 10 x ny x 3 voxels.
static bool tc_tensor_map(CUtensorMap* tm, const ConvArgs& a, int ny) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn) return false;
  const cuuint64_t dims[4] = {(cuuint64_t)a.in_cs, (cuuint64_t)a.X, (cuuint64_t)a.Y, (cuuint64_t)a.Z};
  const cuuint64_t strides[3] = {(cuuint64_t)a.in_cs * 2, (cuuint64_t)a.in_cs * 2 * a.X,
                                 (cuuint64_t)a.in_cs * 2 * a.X * a.Y};
  const cuuint32_t box[4] = {8, (cuuint32_t)kUHX, (cuuint32_t)ny, (cuuint32_t)kUHZ};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return fn(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void*)a.in, dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Whether the tcgen05 form takes this layer: input and weights in the
// supported shapes and a tensor map can be made.
static bool tc_usable(const ConvArgs& a) {
  return a.cin <= 48 && a.cin % 16 == 0 && (a.cout == 16 || a.cout == 32) && a.in_cs % 8 == 0 &&
         a.in_co % 8 == 0 && a.Y >= kUY && ((uintptr_t)a.in & 15) == 0 && encode_tiled() != nullptr;
}

template <int N>
static int launch_conv_tc(cudaStream_t s, const ConvArgs& a) {
  CUtensorMap tm, tr;
  if (!tc_tensor_map(&tm, a, kUHY) || !tc_tensor_map(&tr, a, 1)) return TTFLD_E_UNSUPPORTED;
  const size_t smem = conv_tc_smem_bytes(a.cin, N);
  static int opted = 0, sms = 0, smem_sm = 0, smem_rsv = 0, smem_static = 0;
  if (!opted) {
    if (cudaFuncSetAttribute(conv3_tc_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, 210 * 1024) !=
        cudaSuccess)
      return TTFLD_E_CUDA;
    // the whole unified L1/shared array as shared memory, so that several
    // CTAs fit on an SM (the default carveout left room for one)
    if (cudaFuncSetAttribute(conv3_tc_kernel<N>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
      return TTFLD_E_CUDA;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 152;
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&smem_rsv, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, conv3_tc_kernel<N>) == cudaSuccess) smem_static = (int)fa.sharedSizeBytes;
    opted = 1;
  }
  // as many persistent CTAs as the SM's shared memory holds (at most 4; 32
  // tensor-memory columns each): while one CTA's epilogue reads its
  // accumulators and stores, another's MMAs run.  CTAs beyond what is
  // resident wait for a slot, so an overestimate costs nothing but order.
  const long long per_cta = (long long)smem + smem_static + smem_rsv;
  int per_sm = smem_sm > 0 ? (int)(smem_sm / per_cta) : 1;
  if (per_sm > 4) per_sm = 4;
  if (per_sm < 1) per_sm = 1;
  const long long ntiles = (long long)((a.X + kUX - 1) / kUX) * ((a.Y + kUY - 1) / kUY) * a.Z;
  const long long slots = (long long)sms * per_sm;
  const int blocks = (int)(ntiles < slots ? ntiles : slots);
  conv3_tc_kernel<N><<<blocks, 128, smem, s>>>(a, tm, tr, ntiles);
  count_launches(1);
  TT_CHECK_LAUNCH();
  return 0;
}

// Which layers run on tcgen05: 0 none (mma.sync with shared-memory tiles
// everywhere), 1 every layer the tcgen05 form takes, 2 (default) those with
// 16 output channels.  Measured on the half-resolution grid of 100x256x128
// with up to 4 CTAs per SM: a 16 -> 16 layer takes 52-57 us on tcgen05
// against 76 us on mma.sync, a 16 -> 32 layer 27.6 us against 21.3 us
// (about one tile per CTA, so staging the weights is not amortised).  A
// wait of the tcgen05 form that ran out turns it off for the process and
// fails the pass that saw it.
static int g_conv_tc = 2;

static int check_umma(cudaStream_t s) {
  if (!g_conv_tc) return 0;
  int err = 0;
  TT_CHECK(cudaMemcpyFromSymbolAsync(&err, g_umma_error, sizeof(int), 0, cudaMemcpyDeviceToHost, s));
  TT_CHECK(cudaStreamSynchronize(s));
  if (err) {
    fprintf(stderr, "ttfld: a tcgen05 convolution timed out; using the mma.sync form from now on\n");
    g_conv_tc = 0;
    return TTFLD_E_CUDA;
  }
  return 0;
}

static int conv_fwd(cudaStream_t s, const ConvArgs& a) {
  if (a.cin % 16 || a.cout % 16 || a.in_cs % 2 || a.in_co % 2 || a.out_cs % 2 || a.out_co % 2) return TTFLD_E_ARGS;
  const bool tc = g_conv_tc == 1 || (g_conv_tc == 2 && a.cout == 16);
  if (tc && tc_usable(a)) {
    if (a.cout == 16) return launch_conv_tc<16>(s, a);
    if (a.cout == 32) return launch_conv_tc<32>(s, a);
  }
  // shared-memory tiles up to 96 input channels (a 150 KB input tile; the
  // weights stay in global memory above 100 KB of tile + weights)
  if (a.cin <= 96 && a.in_cs % 8 == 0 && a.in_co % 8 == 0) {
    if (a.cout == 16) return launch_conv_smem<2>(s, a);
    if (a.cout == 32) return launch_conv_smem<4>(s, a);
  }
  const long long tiles = (long long)((a.X + 15) >> 4) * a.Y * a.Z * (a.cout / 16);
  // split the taps over more warps until about two waves of warps are busy
  int ks = 1;
  while (ks < 8 && tiles * ks < 152LL * 128) ks *= 2;
  const long long tpc = 8 / ks;
  const int blocks = (int)((tiles + tpc - 1) / tpc);
  switch (ks) {
    case 1: conv3_fwd_kernel<1><<<blocks, 256, 0, s>>>(a); break;
    case 2: conv3_fwd_kernel<2><<<blocks, 256, 0, s>>>(a); break;
    case 4: conv3_fwd_kernel<4><<<blocks, 256, 0, s>>>(a); break;
    default: conv3_fwd_kernel<8><<<blocks, 256, 0, s>>>(a); break;
  }
  count_launches(1);
  TT_CHECK_LAUNCH();
  return 0;
}

// ---- weight gradient ------------------------------------------------------
// dW[tap][co][ci] = sum_v dZ[v][co] * X[v shifted by tap][ci]: per warp one
// tap, 16 output channels (A = dZ^T, 16 x 16 voxels) and all input channels
// (B = shifted X, 16 voxels x 8 channels per n-block), over a chunk of voxels.
// Each warp stores its chunk's sums (no atomics); a second pass adds the
// chunks in chunk order, so a training run is reproducible bit for bit.
constexpr long long kWgradWarps = 9728;  // about one wave of warps (152 SMs x 64)
struct WgradArgs {
  const bf16* dz;
  int dz_cs, dz_co, cout;
  const bf16* x;
  int x_cs, x_co, cin;  // cin % 8 == 0 (the padded input width)
  float* part;          // [chunk][27][cout][cin] per-chunk sums
  int X, Y, Z;
  long long chunk;      // voxels per warp (multiple of 16)
};

__device__ __forceinline__ long long shifted(long long v, int X, int Y, int Z, int dx, int dy, int dz) {
  const int x = (int)(v % X);
  const int y = (int)((v / X) % Y);
  const int z = (int)(v / ((long long)X * Y));
  const int xx = x + dx, zz = z + dz;
  if (xx < 0 || xx >= X || zz < 0 || zz >= Z) return -1;
  int yy = y + dy;
  yy = yy < 0 ? yy + Y : (yy >= Y ? yy - Y : yy);
  return ((long long)zz * Y + yy) * X + xx;
}

template <int NB>
__global__ void __launch_bounds__(256) conv3_wgrad_kernel(WgradArgs a) {
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long V = (long long)a.X * a.Y * a.Z;
  const long long nchunks = (V + a.chunk - 1) / a.chunk;
  const int cot = a.cout / 16;
  const long long nwarps = 27LL * cot * nchunks;
  if (warp >= nwarps) return;
  const int tap = (int)(warp % 27);
  const int ct = (int)((warp / 27) % cot);
  const long long ck = warp / (27LL * cot);
  const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
  const int r = lane >> 2, cq = (lane & 3) * 2;
  const int co = ct * 16 + r;
  float acc[NB][4];
#pragma unroll
  for (int nb = 0; nb < NB; ++nb) acc[nb][0] = acc[nb][1] = acc[nb][2] = acc[nb][3] = 0.f;
  const bf16 zero = __float2bfloat16_rn(0.f);
  const long long v_end = min(V, (ck + 1) * a.chunk);
  for (long long v0 = ck * a.chunk; v0 < v_end; v0 += 16) {
    long long vv[4] = {v0 + cq, v0 + cq + 1, v0 + cq + 8, v0 + cq + 9};
    bf16 za[4], zb[4];
    long long sv[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const bool in = vv[q] < v_end;
      za[q] = in ? a.dz[(size_t)vv[q] * a.dz_cs + a.dz_co + co] : zero;
      zb[q] = in ? a.dz[(size_t)vv[q] * a.dz_cs + a.dz_co + co + 8] : zero;
      sv[q] = in ? shifted(vv[q], a.X, a.Y, a.Z, dx, dy, dz) : -1;
    }
    // A fragment (row = co, col = voxel): a0 (r, cq..cq+1), a1 (r+8, cq..), a2 (r, cq+8..), a3 (r+8, cq+8..)
    const uint32_t a0 = pack2(za[0], za[1]), a1 = pack2(zb[0], zb[1]);
    const uint32_t a2 = pack2(za[2], za[3]), a3 = pack2(zb[2], zb[3]);
#pragma unroll
    for (int nb = 0; nb < NB; ++nb) {
      const int ci = nb * 8 + r;  // B column n = groupID
      bf16 x0 = sv[0] >= 0 ? a.x[(size_t)sv[0] * a.x_cs + a.x_co + ci] : zero;
      bf16 x1 = sv[1] >= 0 ? a.x[(size_t)sv[1] * a.x_cs + a.x_co + ci] : zero;
      bf16 x2 = sv[2] >= 0 ? a.x[(size_t)sv[2] * a.x_cs + a.x_co + ci] : zero;
      bf16 x3 = sv[3] >= 0 ? a.x[(size_t)sv[3] * a.x_cs + a.x_co + ci] : zero;
      mma_bf16(acc[nb], a0, a1, a2, a3, pack2(x0, x1), pack2(x2, x3));
    }
  }
  // C: (row = co r / r+8, col = ci nb*8+cq, +1), into this chunk's slice
  float* dwt = a.part + ((size_t)ck * 27 + tap) * a.cout * a.cin;
#pragma unroll
  for (int nb = 0; nb < NB; ++nb) {
    const int ci = nb * 8 + cq;
    *reinterpret_cast<float2*>(dwt + (size_t)(ct * 16 + r) * a.cin + ci) = make_float2(acc[nb][0], acc[nb][1]);
    *reinterpret_cast<float2*>(dwt + (size_t)(ct * 16 + r + 8) * a.cin + ci) = make_float2(acc[nb][2], acc[nb][3]);
  }
}

// out[c] = sum over b = 0..nb-1 of part[b * C + c], added in b order
// (accumulate: out[c] += that sum).
template <class T>
__global__ void sum_parts_kernel(const T* part, int nb, long long C, T* out, int accumulate) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < C; c += (long long)gridDim.x * blockDim.x) {
    T s = 0;
    for (int b = 0; b < nb; ++b) s += part[(size_t)b * C + c];
    out[c] = accumulate ? out[c] + s : s;
  }
}

// Weight gradient of one layer into dw [27][cout][cin] (written).
static int conv_wgrad(cudaStream_t s, WgradArgs a, float* dw) {
  if (a.cout % 16 || a.cin % 8) return TTFLD_E_ARGS;
  const long long V = (long long)a.X * a.Y * a.Z;
  // at most one full wave of warps, each summing a long run of voxels
  const long long tiles = 27LL * (a.cout / 16);
  long long nch = kWgradWarps / tiles;
  if (nch < 1) nch = 1;
  long long chunk = (V + nch - 1) / nch;
  chunk = (chunk + 15) / 16 * 16;
  if (chunk < 16) chunk = 16;
  a.chunk = chunk;
  nch = (V + chunk - 1) / chunk;   // <= kWgradWarps / tiles: the partials fit max_wpart()
  const long long warps = tiles * nch;
  const int blocks = (int)((warps * 32 + 255) / 256);
  switch (a.cin / 8) {
    case 2: conv3_wgrad_kernel<2><<<blocks, 256, 0, s>>>(a); break;
    case 4: conv3_wgrad_kernel<4><<<blocks, 256, 0, s>>>(a); break;
    case 6: conv3_wgrad_kernel<6><<<blocks, 256, 0, s>>>(a); break;
    case 8: conv3_wgrad_kernel<8><<<blocks, 256, 0, s>>>(a); break;
    case 12: conv3_wgrad_kernel<12><<<blocks, 256, 0, s>>>(a); break;
    case 16: conv3_wgrad_kernel<16><<<blocks, 256, 0, s>>>(a); break;
    default: return TTFLD_E_UNSUPPORTED;
  }
  const long long C = 27LL * a.cout * a.cin;
  sum_parts_kernel<float><<<grid_for(C), 256, 0, s>>>(a.part, (int)nch, C, dw, 0);
  count_launches(2);
  TT_CHECK_LAUNCH();
  return 0;
}

// ---- elementwise pieces -------------------------------------------------
// dZ = dY * leaky'(Y) in place, on a channel slice
__global__ void act_bwd_kernel(bf16* dy, int dy_cs, int dy_co, const bf16* y, int y_cs, int y_co, int C, long long V) {
  const long long n = V * C;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const long long v = t / C;
    const int c = (int)(t % C);
    bf16* p = dy + (size_t)v * dy_cs + dy_co + c;
    const float yv = __bfloat162float(y[(size_t)v * y_cs + y_co + c]);
    if (!(yv > 0.f)) *p = __float2bfloat16_rn(__bfloat162float(*p) * kLeak);
  }
}

// bias gradient, per block: part[block][c] = sum over the block's voxels of
// dZ[v][c] (the blocks' sums are added in block order afterwards)
__global__ void bias_grad_kernel(const bf16* dz, int cs, int co, int C, long long V, float* part) {
  __shared__ float sh[64 * 8];
  const int c = threadIdx.x % C, lanes = blockDim.x / C, l = threadIdx.x / C;
  float acc = 0.f;
  if (threadIdx.x < C * lanes)
    for (long long v = blockIdx.x * (long long)lanes + l; v < V; v += (long long)gridDim.x * lanes)
      acc += __bfloat162float(dz[(size_t)v * cs + co + c]);
  if (threadIdx.x < C * lanes) sh[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x < C) {
    float t = 0.f;
    for (int q = 0; q < lanes; ++q) t += sh[q * C + threadIdx.x];
    part[(size_t)blockIdx.x * C + threadIdx.x] = t;
  }
}

// 2x2x2 average pooling over the children that exist (ceil sizes), and
// nearest upsampling into a channel slice of the fine buffer: 8 channels
// (16 bytes) per thread, for channel strides, offsets and counts that are
// multiples of 8.
__global__ void pool8_fwd_kernel(const bf16* in, int in_cs, int in_co, Level fi, bf16* out, int out_cs, int out_co,
                                 Level co_, int C) {
  const int C8 = C >> 3;
  const long long n = co_.vox() * C8;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(t % C8) * 8;
    const long long v = t / C8;
    const int x = (int)(v % co_.X), y = (int)((v / co_.X) % co_.Y), z = (int)(v / ((long long)co_.X * co_.Y));
    float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int cnt = 0;
    for (int q = 0; q < 8; ++q) {
      const int xx = 2 * x + (q & 1), yy = 2 * y + ((q >> 1) & 1), zz = 2 * z + (q >> 2);
      if (xx < fi.X && yy < fi.Y && zz < fi.Z) {
        const uint4 u = *reinterpret_cast<const uint4*>(in + (((size_t)zz * fi.Y + yy) * fi.X + xx) * in_cs + in_co + c);
        const bf16* b = reinterpret_cast<const bf16*>(&u);
#pragma unroll
        for (int e = 0; e < 8; ++e) s[e] += __bfloat162float(b[e]);
        ++cnt;
      }
    }
    __align__(16) bf16 o[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) o[e] = __float2bfloat16_rn(s[e] / (float)cnt);
    *reinterpret_cast<uint4*>(out + (size_t)v * out_cs + out_co + c) = *reinterpret_cast<const uint4*>(o);
  }
}

__global__ void up8_fwd_kernel(const bf16* in, int in_cs, Level co_, bf16* out, int out_cs, int out_co, Level fi,
                               int C) {
  const int C8 = C >> 3;
  const long long n = fi.vox() * C8;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(t % C8) * 8;
    const long long v = t / C8;
    const int x = (int)(v % fi.X), y = (int)((v / fi.X) % fi.Y), z = (int)(v / ((long long)fi.X * fi.Y));
    *reinterpret_cast<uint4*>(out + (size_t)v * out_cs + out_co + c) = *reinterpret_cast<const uint4*>(
        in + (((size_t)(z / 2) * co_.Y + y / 2) * co_.X + x / 2) * in_cs + c);
  }
}

// d(fine) += d(coarse) / count (accumulate into a slice of the fine gradient)
__global__ void pool_bwd_kernel(const bf16* gco, int g_cs, int g_co, Level co_, bf16* gfi, int f_cs, int f_co, Level fi,
                                int C) {
  const long long n = fi.vox() * C;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(t % C);
    const long long v = t / C;
    const int x = (int)(v % fi.X), y = (int)((v / fi.X) % fi.Y), z = (int)(v / ((long long)fi.X * fi.Y));
    const int px = x / 2, py = y / 2, pz = z / 2;
    int cnt = 0;
    for (int q = 0; q < 8; ++q) {
      const int xx = 2 * px + (q & 1), yy = 2 * py + ((q >> 1) & 1), zz = 2 * pz + (q >> 2);
      if (xx < fi.X && yy < fi.Y && zz < fi.Z) ++cnt;
    }
    const float g = __bfloat162float(gco[(((size_t)pz * co_.Y + py) * co_.X + px) * g_cs + g_co + c]) / (float)cnt;
    bf16* p = gfi + (size_t)v * f_cs + f_co + c;
    *p = __float2bfloat16_rn(__bfloat162float(*p) + g);
  }
}

// d(coarse) = sum of d(fine children) (written, not accumulated)
__global__ void up_bwd_kernel(const bf16* gfi, int f_cs, int f_co, Level fi, bf16* gco, int g_cs, Level co_, int C) {
  const long long n = co_.vox() * C;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(t % C);
    const long long v = t / C;
    const int x = (int)(v % co_.X), y = (int)((v / co_.X) % co_.Y), z = (int)(v / ((long long)co_.X * co_.Y));
    float s = 0.f;
    for (int q = 0; q < 8; ++q) {
      const int xx = 2 * x + (q & 1), yy = 2 * y + ((q >> 1) & 1), zz = 2 * z + (q >> 2);
      if (xx < fi.X && yy < fi.Y && zz < fi.Z)
        s += __bfloat162float(gfi[(((size_t)zz * fi.Y + yy) * fi.X + xx) * f_cs + f_co + c]);
    }
    gco[(size_t)v * g_cs + c] = __float2bfloat16_rn(s);
  }
}

// head: pred = w . a13 + b (FP32); loss = sum mask (pred - target)^2 / nmask
__global__ void head_fwd_kernel(const bf16* a13, const float* w, float* pred, long long V) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    float s = w[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) s += w[c] * __bfloat162float(a13[(size_t)v * 16 + c]);
    pred[v] = s;
  }
}

__global__ void loss_kernel(const float* pred, const float* target, const unsigned char* mask, long long V, double inv_n,
                            float* gpred, double* part) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    const float d = mask[v] ? pred[v] - target[v] : 0.f;
    acc += (double)d * d;
    gpred[v] = (float)(2.0 * inv_n) * d;
  }
  const double b = block_sum(acc * inv_n, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = b;
}

// d(a13)[v][c] = gpred[v] * w[c]; per block: part[block][c] = sum gpred * a13,
// part[block][16] = sum gpred (added in block order afterwards)
__global__ void head_bwd_kernel(const float* gpred, const bf16* a13, const float* w, bf16* ga13, float* part, long long V) {
  __shared__ float sh[17][32];
  float acc[17];
  for (int c = 0; c < 17; ++c) acc[c] = 0.f;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    const float g = gpred[v];
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      acc[c] += g * __bfloat162float(a13[(size_t)v * 16 + c]);
      ga13[(size_t)v * 16 + c] = __float2bfloat16_rn(g * w[c]);
    }
    acc[16] += g;
  }
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  for (int c = 0; c < 17; ++c) {
    float s = acc[c];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) sh[c][wp] = s;
  }
  __syncthreads();
  if (threadIdx.x < 17) {
    float t = 0.f;
    for (int q = 0; q < nw; ++q) t += sh[threadIdx.x][q];
    part[(size_t)blockIdx.x * 17 + threadIdx.x] = t;
  }
}

// Level-0 output to the grid by cell-centred trilinear interpolation (fine
// cell x sits at coarse coordinate x/2 - 1/4: weights 3/4 and 1/4 on the
// two nearest coarse cells), clamped at the r and theta ends and periodic in
// phi.  A piecewise-constant copy would leave a step every second cell; the
// stencil operator amplifies such cell-scale error, so the guess would start
// with a residual many times ||b||_1.
struct Interp1 {
  int c0, c1;
  float w0, w1;
};
__host__ __device__ __forceinline__ Interp1 interp1(int x, int nc, bool periodic) {
  const int c = x >> 1;
  Interp1 r;
  if (x & 1) { r.c0 = c; r.c1 = c + 1; r.w0 = 0.75f; r.w1 = 0.25f; }
  else { r.c0 = c - 1; r.c1 = c; r.w0 = 0.25f; r.w1 = 0.75f; }
  if (periodic) {
    r.c0 = (r.c0 + nc) % nc;
    r.c1 = r.c1 % nc;
  } else {
    if (r.c0 < 0) r.c0 = 0;
    if (r.c1 > nc - 1) r.c1 = nc - 1;
  }
  return r;
}
// weight fine cell x gives coarse cell c
__device__ __forceinline__ float interp1_weight(int x, int c, int nc, bool periodic) {
  const Interp1 r = interp1(x, nc, periodic);
  return (r.c0 == c ? r.w0 : 0.f) + (r.c1 == c ? r.w1 : 0.f);
}
// the fine cells whose interpolation can touch coarse cell c: the window
// 2c-1 .. 2c+2 (wrapped or clipped); every cell when the extent is small
__device__ __forceinline__ int interp1_window(int c, int nf, bool periodic, int* xs) {
  if (nf <= 4) {
    for (int q = 0; q < nf; ++q) xs[q] = q;
    return nf;
  }
  int m = 0;
  for (int o = -1; o <= 2; ++o) {
    int x = 2 * c + o;
    if (periodic) x = (x + nf) % nf;
    else if (x < 0 || x >= nf) continue;
    xs[m++] = x;
  }
  return m;
}

__global__ void pred_up_kernel(const float* half, Level co_, float* full, Level fi) {
  const long long n = fi.vox();
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(v % fi.X), y = (int)((v / fi.X) % fi.Y), z = (int)(v / ((long long)fi.X * fi.Y));
    const Interp1 ix = interp1(x, co_.X, false), iy = interp1(y, co_.Y, true), iz = interp1(z, co_.Z, false);
    float s = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int cx = (q & 1) ? ix.c1 : ix.c0, cy = (q & 2) ? iy.c1 : iy.c0, cz = (q & 4) ? iz.c1 : iz.c0;
      const float w = ((q & 1) ? ix.w1 : ix.w0) * ((q & 2) ? iy.w1 : iy.w0) * ((q & 4) ? iz.w1 : iz.w0);
      s += w * half[((size_t)cz * co_.Y + cy) * co_.X + cx];
    }
    full[v] = s;
  }
}

// adjoint of pred_up_kernel, as a gather over each coarse cell's window
__global__ void pred_down_kernel(const float* gfull, Level fi, float* ghalf, Level co_) {
  const long long n = co_.vox();
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(v % co_.X), y = (int)((v / co_.X) % co_.Y), z = (int)(v / ((long long)co_.X * co_.Y));
    int xs[4], ys[4], zs[4];
    const int nxw = interp1_window(x, fi.X, false, xs), nyw = interp1_window(y, fi.Y, true, ys),
              nzw = interp1_window(z, fi.Z, false, zs);
    float s = 0.f;
    for (int c = 0; c < nzw; ++c) {
      const float wz = interp1_weight(zs[c], z, co_.Z, false);
      if (wz == 0.f) continue;
      for (int b = 0; b < nyw; ++b) {
        const float wy = interp1_weight(ys[b], y, co_.Y, true);
        if (wy == 0.f) continue;
        for (int a = 0; a < nxw; ++a) {
          const float wx = interp1_weight(xs[a], x, co_.X, false);
          if (wx != 0.f) s += wz * wy * wx * gfull[((size_t)zs[c] * fi.Y + ys[b]) * fi.X + xs[a]];
        }
      }
    }
    ghalf[v] = s;
  }
}

// FP32 master weights -> BF16 [tap][cout][cin_pad] and the flipped transpose
// [26 - tap][cin_pad][cout] used by backward-data
__global__ void wprep_kernel(const float* w, int cin, int cin_pad, int cout, bf16* w16, bf16* w16t) {
  const long long n = 27LL * cout * cin_pad;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int ci = (int)(t % cin_pad);
    const int co = (int)((t / cin_pad) % cout);
    const int tap = (int)(t / ((long long)cin_pad * cout));
    const float v = ci < cin ? w[((size_t)tap * cout + co) * cin + ci] : 0.f;
    const bf16 b = __float2bfloat16_rn(v);
    w16[t] = b;
    w16t[((size_t)(26 - tap) * cin_pad + ci) * cout + co] = b;
  }
}

// Adam on all parameters; padded input channels are not parameters
__global__ void adam_kernel(float* p, const float* g, float* m, float* v, size_t n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const float gt = g[t];
    const float mt = b1 * m[t] + (1.f - b1) * gt;
    const float vt = b2 * v[t] + (1.f - b2) * gt * gt;
    m[t] = mt;
    v[t] = vt;
    p[t] -= lr * (mt / c1) / (sqrtf(vt / c2) + eps);
  }
}

// wgrad accumulates [27][cout][cin_pad]; fold it into the FP32 gradient of
// the real [27][cout][cin] weights
__global__ void wgrad_fold_kernel(const float* gpad, int cin, int cin_pad, int cout, float* g) {
  const long long n = 27LL * cout * cin;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int ci = (int)(t % cin);
    const long long rest = t / cin;
    g[t] += gpad[rest * cin_pad + ci];
  }
}

// ---- features from the step's state ------------------------------------
// L0 voxel (x,y,z) = interior cell (i,j,k) = (x+1, y+1, z+1)
// In FP32: the features are rounded to BF16 anyway, and FP64 logarithms
// would cost more than the network (FP64 is a small fraction of the SM's
// FP32 rate on this part).
__device__ __forceinline__ void cell_features(const Dev& d, int i, int j, int k, float* f) {
  const size_t h = hidx(d, i, j, k);
  const float er = fmaxf((float)d.ER[h], 1e-30f);
  f[0] = (log10f(er) + 1.3f) / 0.6f;
  f[1] = log10f(fmaxf((float)d.XKAPR[h], 1e-30f)) + 4.0f;
  f[2] = (log10f(fmaxf((float)d.RH[h], 1e-30f)) + 4.0f) / 1.2f;
  f[3] = log10f((float)d.delt / 100.0f) / 0.5f;
  const float s = (i <= d.nx) ? (float)d.SI[h] : 0.0f;
  const float q = fminf(fmaxf(s * (float)d.delt * 1e4f / er, -1e30f), 1e30f);
  f[4] = asinhf(q) / 5.0f;
}

__device__ __forceinline__ bool cell_active(const Dev& d, int i, int j, int k) {
  const int ub = PA(UB, j, k);
  return i < ub && i < d.nx && k > 1 && k < d.nz;
}

}  // namespace ttfld

using namespace ttfld;

namespace {

// Parameter layout: per conv layer w[27][cout][cin] then b[cout]; head w[16], b.
void layout(Net* n) {
  size_t o = 0, o16 = 0;
  for (int l = 0; l < kNumConv; ++l) {
    const LayerSpec& s = kLayers[l];
    n->woff[l] = o;
    o += (size_t)27 * s.cout * s.cin;
    n->boff[l] = o;
    o += s.cout;
    n->w16off[l] = o16;
    o16 += (size_t)27 * s.cout * s.cin_pad;
  }
  n->hoff = o;
  o += 17;
  n->nparams = o;
  n->nw16 = o16;
}

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

int ensure_net(ttfld_ctx* c) {
  if (c->unet) return 0;
  Net* n = (Net*)calloc(1, sizeof(Net));
  if (!n) return TTFLD_E_ARGS;
  layout(n);
  const int nx = c->d.nx, ny = c->d.ny, nz = c->d.nz;
  n->full = {nx, ny, nz};
  n->lv[0] = {(nx + 1) / 2, (ny + 1) / 2, (nz + 1) / 2};
  for (int l = 1; l < 4; ++l)
    n->lv[l] = {(n->lv[l - 1].X + 1) / 2, (n->lv[l - 1].Y + 1) / 2, (n->lv[l - 1].Z + 1) / 2};
  // parameters
  float* pm = nullptr;
  if (check_cuda(cudaMalloc((void**)&pm, 4 * align256(n->nparams * 4)), "unet params")) { free(n); return TTFLD_E_CUDA; }
  cudaMemset(pm, 0, 4 * align256(n->nparams * 4));
  n->p = pm;
  n->g = (float*)((char*)pm + align256(n->nparams * 4));
  n->m = (float*)((char*)pm + 2 * align256(n->nparams * 4));
  n->v = (float*)((char*)pm + 3 * align256(n->nparams * 4));
  bf16* w = nullptr;
  if (check_cuda(cudaMalloc((void**)&w, 2 * align256(n->nw16 * 2)), "unet bf16 weights")) { free(n); return TTFLD_E_CUDA; }
  n->w16 = w;
  n->w16t = (bf16*)((char*)w + align256(n->nw16 * 2));
  // activations and gradients
  struct B { bf16** p; bf16** g; int lev, ch; };
  B bufs[] = {{&n->feat, nullptr, 0, 16}, {&n->a0, &n->g_a0, 0, 16}, {&n->cat0, &n->g_cat0, 0, 48},
              {&n->a12, &n->g_a12, 0, 16}, {&n->a13, &n->g_a13, 0, 16}, {&n->p0, &n->g_p0, 1, 16},
              {&n->a2, &n->g_a2, 1, 32}, {&n->cat1, &n->g_cat1, 1, 96}, {&n->a10, &n->g_a10, 1, 32},
              {&n->a11, &n->g_a11, 1, 32}, {&n->p1, &n->g_p1, 2, 32}, {&n->a4, &n->g_a4, 2, 64},
              {&n->cat2, &n->g_cat2, 2, 128}, {&n->a8, &n->g_a8, 2, 64}, {&n->a9, &n->g_a9, 2, 64},
              {&n->p2, &n->g_p2, 3, 64}, {&n->a6, &n->g_a6, 3, 64}, {&n->a7, &n->g_a7, 3, 64}};
  size_t bytes = 0;
  for (const B& b : bufs) bytes += (b.g ? 2 : 1) * align256((size_t)n->lv[b.lev].vox() * b.ch * 2);
  const long long VF = n->full.vox(), V0 = n->lv[0].vox();
  bytes += 2 * align256((size_t)V0 * 4);                        // pred_half, gpred_half
  bytes += 3 * align256((size_t)VF * 4) + align256((size_t)VF) + 256;
  char* mem = nullptr;
  if (check_cuda(cudaMalloc((void**)&mem, bytes), "unet activations")) { free(n); return TTFLD_E_CUDA; }
  cudaMemset(mem, 0, bytes);
  n->act_mem = mem;
  size_t off = 0;
  for (const B& b : bufs) {
    const size_t sz = align256((size_t)n->lv[b.lev].vox() * b.ch * 2);
    *b.p = (bf16*)(mem + off);
    off += sz;
    if (b.g) { *b.g = (bf16*)(mem + off); off += sz; }
  }
  n->pred_half = (float*)(mem + off); off += align256((size_t)V0 * 4);
  n->gpred_half = (float*)(mem + off); off += align256((size_t)V0 * 4);
  n->pred = (float*)(mem + off); off += align256((size_t)VF * 4);
  n->gpred = (float*)(mem + off); off += align256((size_t)VF * 4);
  n->target = (float*)(mem + off); off += align256((size_t)VF * 4);
  n->mask = (unsigned char*)(mem + off); off += align256((size_t)VF);
  n->loss_acc = (double*)(mem + off);
  c->unet = n;
  return 0;
}

// He-normal initialisation from a seeded host generator (Box-Muller).
int init_params(ttfld_ctx* c, uint64_t seed) {
  Net* n = net_of(c);
  std::vector<float> h(n->nparams, 0.f);
  uint64_t st = seed * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL;
  auto u01 = [&]() {
    st ^= st << 13; st ^= st >> 7; st ^= st << 17;
    return ((st >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  };
  for (int l = 0; l < kNumConv; ++l) {
    const LayerSpec& s = kLayers[l];
    const double sd = sqrt(2.0 / (27.0 * s.cin));
    for (size_t q = 0; q < (size_t)27 * s.cout * s.cin; ++q) {
      double z = sqrt(-2.0 * log(u01())) * cos(6.283185307179586 * u01());
      h[n->woff[l] + q] = (float)(sd * z);
    }
  }
  for (int q = 0; q < 16; ++q) h[n->hoff + q] = (float)(0.1 * (u01() - 0.5));
  TT_CHECK(cudaMemcpy(n->p, h.data(), n->nparams * 4, cudaMemcpyHostToDevice));
  TT_CHECK(cudaMemset(n->m, 0, n->nparams * 4));
  TT_CHECK(cudaMemset(n->v, 0, n->nparams * 4));
  n->step = 0;
  n->ready = 1;
  n->wdirty = 1;
  return 0;
}

// BF16 copies (and flipped copies) of the FP32 master weights, when stale.
int prep_weights(ttfld_ctx* c) {
  Net* n = net_of(c);
  if (!n->wdirty) return 0;
  for (int l = 0; l < kNumConv; ++l) {
    const LayerSpec& s = kLayers[l];
    wprep_kernel<<<grid_for(27LL * s.cout * s.cin_pad), 256, 0, c->stream>>>(
        n->p + n->woff[l], s.cin, s.cin_pad, s.cout, n->w16 + n->w16off[l], n->w16t + n->w16off[l]);
    count_launches(1);
  }
  TT_CHECK_LAUNCH();
  n->wdirty = 0;
  return 0;
}

ConvArgs conv_args(Net* n, int l, const bf16* in, int in_cs, int in_co, bf16* out, int out_cs, int out_co, int lev) {
  const LayerSpec& s = kLayers[l];
  ConvArgs a;
  a.in = in; a.in_cs = in_cs; a.in_co = in_co; a.cin = s.cin_pad;
  a.w = n->w16 + n->w16off[l];
  a.bias = n->p + n->boff[l];
  a.out = out; a.out_cs = out_cs; a.out_co = out_co; a.cout = s.cout;
  a.X = n->lv[lev].X; a.Y = n->lv[lev].Y; a.Z = n->lv[lev].Z;
  a.act = 1; a.accum = 0;
  return a;
}

#define GRID(n) grid_for((long long)(n))
#define L(k) n->lv[k]

// Forward pass from n->feat (level 0) to n->pred (the grid).
int forward(ttfld_ctx* c) {
  Net* n = net_of(c);
  cudaStream_t s = c->stream;
  int rc;
#define CONV(l, in, ics, ico, out, ocs, oco, lev) \
  if ((rc = conv_fwd(s, conv_args(n, l, in, ics, ico, out, ocs, oco, lev)))) return rc;
  CONV(0, n->feat, 16, 0, n->a0, 16, 0, 0);
  CONV(1, n->a0, 16, 0, n->cat0, 48, 32, 0);                // s0 -> cat0[32:48]
  pool8_fwd_kernel<<<GRID(L(1).vox() * 2), 256, 0, s>>>(n->cat0, 48, 32, L(0), n->p0, 16, 0, L(1), 16);
  CONV(2, n->p0, 16, 0, n->a2, 32, 0, 1);
  CONV(3, n->a2, 32, 0, n->cat1, 96, 64, 1);                // s1 -> cat1[64:96]
  pool8_fwd_kernel<<<GRID(L(2).vox() * 4), 256, 0, s>>>(n->cat1, 96, 64, L(1), n->p1, 32, 0, L(2), 32);
  CONV(4, n->p1, 32, 0, n->a4, 64, 0, 2);
  CONV(5, n->a4, 64, 0, n->cat2, 128, 64, 2);               // s2 -> cat2[64:128]
  pool8_fwd_kernel<<<GRID(L(3).vox() * 8), 256, 0, s>>>(n->cat2, 128, 64, L(2), n->p2, 64, 0, L(3), 64);
  CONV(6, n->p2, 64, 0, n->a6, 64, 0, 3);
  CONV(7, n->a6, 64, 0, n->a7, 64, 0, 3);
  up8_fwd_kernel<<<GRID(L(2).vox() * 8), 256, 0, s>>>(n->a7, 64, L(3), n->cat2, 128, 0, L(2), 64);
  CONV(8, n->cat2, 128, 0, n->a8, 64, 0, 2);
  CONV(9, n->a8, 64, 0, n->a9, 64, 0, 2);
  up8_fwd_kernel<<<GRID(L(1).vox() * 8), 256, 0, s>>>(n->a9, 64, L(2), n->cat1, 96, 0, L(1), 64);
  CONV(10, n->cat1, 96, 0, n->a10, 32, 0, 1);
  CONV(11, n->a10, 32, 0, n->a11, 32, 0, 1);
  up8_fwd_kernel<<<GRID(L(0).vox() * 4), 256, 0, s>>>(n->a11, 32, L(1), n->cat0, 48, 0, L(0), 32);
  CONV(12, n->cat0, 48, 0, n->a12, 16, 0, 0);
  CONV(13, n->a12, 16, 0, n->a13, 16, 0, 0);
#undef CONV
  head_fwd_kernel<<<GRID(L(0).vox()), 256, 0, s>>>(n->a13, n->p + n->hoff, n->pred_half, L(0).vox());
  pred_up_kernel<<<GRID(n->full.vox()), 256, 0, s>>>(n->pred_half, L(0), n->pred, n->full);
  count_launches(7);
  TT_CHECK_LAUNCH();
  return check_umma(s);
}

// Backward of one conv layer: dY (in place -> dZ), weight/bias gradients,
// and (when gx != null) the input gradient, written or accumulated.
// Gradient workspace of one training call: the padded weight gradient of a
// layer, the per-chunk weight-gradient sums, and the per-block sums of the
// bias, head and loss reductions (each added in a fixed order).
constexpr int kMaxGradBlocks = 4096;  // >= any grid_for() grid
struct GradWork {
  float* gpad;   // max_wpad()
  float* wpart;  // max_wpart()
  float* bpart;  // kMaxGradBlocks x 64
  float* hpart;  // kMaxGradBlocks x 17
  double* lpart; // kMaxGradBlocks
};

int conv_backward(ttfld_ctx* c, GradWork* gw, int l, bf16* gy, int gy_cs, int gy_co, const bf16* y, int y_cs, int y_co,
                  const bf16* x, int x_cs, int x_co, bf16* gx, int gx_cs, int gx_co, int accum, int lev) {
  Net* n = net_of(c);
  const LayerSpec& s = kLayers[l];
  cudaStream_t st = c->stream;
  const long long V = L(lev).vox();
  int rc;
  act_bwd_kernel<<<GRID(V * s.cout), 256, 0, st>>>(gy, gy_cs, gy_co, y, y_cs, y_co, s.cout, V);
  const int bblocks = GRID(V / 8 + 1);
  bias_grad_kernel<<<bblocks, 512, 0, st>>>(gy, gy_cs, gy_co, s.cout, V, gw->bpart);
  sum_parts_kernel<float><<<1, 64, 0, st>>>(gw->bpart, bblocks, s.cout, n->g + n->boff[l], 1);
  count_launches(3);
  WgradArgs wa{gy, gy_cs, gy_co, s.cout, x, x_cs, x_co, s.cin_pad, gw->wpart, L(lev).X, L(lev).Y, L(lev).Z, 0};
  if ((rc = conv_wgrad(st, wa, gw->gpad))) return rc;
  wgrad_fold_kernel<<<GRID(27LL * s.cout * s.cin), 256, 0, st>>>(gw->gpad, s.cin, s.cin_pad, s.cout, n->g + n->woff[l]);
  count_launches(1);
  if (gx) {
    ConvArgs a;
    a.in = gy; a.in_cs = gy_cs; a.in_co = gy_co; a.cin = s.cout;
    a.w = n->w16t + n->w16off[l];
    a.bias = nullptr;
    a.out = gx; a.out_cs = gx_cs; a.out_co = gx_co; a.cout = s.cin_pad;
    a.X = L(lev).X; a.Y = L(lev).Y; a.Z = L(lev).Z;
    a.act = 0; a.accum = accum;
    if ((rc = conv_fwd(st, a))) return rc;
  }
  TT_CHECK_LAUNCH();
  return 0;
}

// Loss against n->target/mask and the gradients of every parameter (n->g).
int backward(ttfld_ctx* c, GradWork* gw, double* loss_out) {
  Net* n = net_of(c);
  cudaStream_t s = c->stream;
  const long long V0 = L(0).vox(), VF = n->full.vox();
  int rc;
  TT_CHECK(cudaMemsetAsync(n->g, 0, n->nparams * 4, s));
  TT_CHECK(cudaMemsetAsync(n->loss_acc, 0, sizeof(double), s));
  // number of active cells
  long long nmask = 0;
  {
    std::vector<unsigned char> hm((size_t)VF);
    TT_CHECK(cudaMemcpyAsync(hm.data(), n->mask, (size_t)VF, cudaMemcpyDeviceToHost, s));
    TT_CHECK(cudaStreamSynchronize(s));
    for (unsigned char m : hm) nmask += m;
  }
  const double inv_n = 1.0 / (double)(nmask > 0 ? nmask : 1);
  const int lblocks = GRID(VF), hblocks = GRID(V0);
  loss_kernel<<<lblocks, 256, 0, s>>>(n->pred, n->target, n->mask, VF, inv_n, n->gpred, gw->lpart);
  sum_parts_kernel<double><<<1, 32, 0, s>>>(gw->lpart, lblocks, 1, n->loss_acc, 0);
  pred_down_kernel<<<GRID(V0), 256, 0, s>>>(n->gpred, n->full, n->gpred_half, L(0));
  head_bwd_kernel<<<hblocks, 256, 0, s>>>(n->gpred_half, n->a13, n->p + n->hoff, n->g_a13, gw->hpart, V0);
  sum_parts_kernel<float><<<1, 32, 0, s>>>(gw->hpart, hblocks, 17, n->g + n->hoff, 1);
  count_launches(5);
#define BWD(l, gy, gcs, gco, y, ycs, yco, x, xcs, xco, gx, gxcs, gxco, acc, lev)                                  \
  if ((rc = conv_backward(c, gw, l, gy, gcs, gco, y, ycs, yco, x, xcs, xco, gx, gxcs, gxco, acc, lev))) return rc;
  BWD(13, n->g_a13, 16, 0, n->a13, 16, 0, n->a12, 16, 0, n->g_a12, 16, 0, 0, 0);
  BWD(12, n->g_a12, 16, 0, n->a12, 16, 0, n->cat0, 48, 0, n->g_cat0, 48, 0, 0, 0);
  up_bwd_kernel<<<GRID(L(1).vox() * 32), 256, 0, s>>>(n->g_cat0, 48, 0, L(0), n->g_a11, 32, L(1), 32);
  BWD(11, n->g_a11, 32, 0, n->a11, 32, 0, n->a10, 32, 0, n->g_a10, 32, 0, 0, 1);
  BWD(10, n->g_a10, 32, 0, n->a10, 32, 0, n->cat1, 96, 0, n->g_cat1, 96, 0, 0, 1);
  up_bwd_kernel<<<GRID(L(2).vox() * 64), 256, 0, s>>>(n->g_cat1, 96, 0, L(1), n->g_a9, 64, L(2), 64);
  BWD(9, n->g_a9, 64, 0, n->a9, 64, 0, n->a8, 64, 0, n->g_a8, 64, 0, 0, 2);
  BWD(8, n->g_a8, 64, 0, n->a8, 64, 0, n->cat2, 128, 0, n->g_cat2, 128, 0, 0, 2);
  up_bwd_kernel<<<GRID(L(3).vox() * 64), 256, 0, s>>>(n->g_cat2, 128, 0, L(2), n->g_a7, 64, L(3), 64);
  BWD(7, n->g_a7, 64, 0, n->a7, 64, 0, n->a6, 64, 0, n->g_a6, 64, 0, 0, 3);
  BWD(6, n->g_a6, 64, 0, n->a6, 64, 0, n->p2, 64, 0, n->g_p2, 64, 0, 0, 3);
  pool_bwd_kernel<<<GRID(L(2).vox() * 64), 256, 0, s>>>(n->g_p2, 64, 0, L(3), n->g_cat2, 128, 64, L(2), 64);
  BWD(5, n->g_cat2, 128, 64, n->cat2, 128, 64, n->a4, 64, 0, n->g_a4, 64, 0, 0, 2);
  BWD(4, n->g_a4, 64, 0, n->a4, 64, 0, n->p1, 32, 0, n->g_p1, 32, 0, 0, 2);
  pool_bwd_kernel<<<GRID(L(1).vox() * 32), 256, 0, s>>>(n->g_p1, 32, 0, L(2), n->g_cat1, 96, 64, L(1), 32);
  BWD(3, n->g_cat1, 96, 64, n->cat1, 96, 64, n->a2, 32, 0, n->g_a2, 32, 0, 0, 1);
  BWD(2, n->g_a2, 32, 0, n->a2, 32, 0, n->p0, 16, 0, n->g_p0, 16, 0, 0, 1);
  pool_bwd_kernel<<<GRID(L(0).vox() * 16), 256, 0, s>>>(n->g_p0, 16, 0, L(1), n->g_cat0, 48, 32, L(0), 16);
  BWD(1, n->g_cat0, 48, 32, n->cat0, 48, 32, n->a0, 16, 0, n->g_a0, 16, 0, 0, 0);
  BWD(0, n->g_a0, 16, 0, n->a0, 16, 0, n->feat, 16, 0, nullptr, 0, 0, 0, 0);
#undef BWD
  count_launches(6);
  TT_CHECK_LAUNCH();
  if ((rc = check_umma(s))) return rc;
  if (loss_out) {
    double h = 0.0;
    TT_CHECK(cudaMemcpyAsync(&h, n->loss_acc, sizeof(double), cudaMemcpyDeviceToHost, s));
    TT_CHECK(cudaStreamSynchronize(s));
    *loss_out = h;
  }
  return 0;
}

// Largest per-chunk weight-gradient sums of a layer: at most kWgradWarps / tiles
// chunks of [27][cout][cin_pad], i.e. kWgradWarps x 16 x cin_pad floats.
size_t max_wpart() {
  size_t m = 0;
  for (int l = 0; l < kNumConv; ++l) {
    size_t v = (size_t)kWgradWarps * 16 * kLayers[l].cin_pad;
    if (v > m) m = v;
  }
  return m;
}

// Largest [27][cout][cin_pad] of the layers (the padded weight-gradient buffer).
size_t max_wpad(const Net* n) {
  size_t m = 0;
  for (int l = 0; l < kNumConv; ++l) {
    size_t v = (size_t)27 * kLayers[l].cout * kLayers[l].cin_pad;
    if (v > m) m = v;
  }
  return m;
}

// One allocation for the gradient workspace (freed with cudaFree(gw->gpad)).
int alloc_gradwork(const Net* n, GradWork* gw) {
  const size_t a = align256(max_wpad(n) * 4), b = align256(max_wpart() * 4);
  const size_t c = align256((size_t)kMaxGradBlocks * 64 * 4), d = align256((size_t)kMaxGradBlocks * 17 * 4);
  const size_t e = align256((size_t)kMaxGradBlocks * 8);
  char* p = nullptr;
  TT_CHECK(cudaMalloc((void**)&p, a + b + c + d + e));
  gw->gpad = (float*)p;
  gw->wpart = (float*)(p + a);
  gw->bpart = (float*)(p + a + b);
  gw->hpart = (float*)(p + a + b + c);
  gw->lpart = (double*)(p + a + b + c + d);
  return 0;
}

// Features of the current state averaged over the 2x2x2 cells of each
// level-0 voxel (BF16, 16 channels, 5 used), and the grid's active-cell mask.
int make_features(ttfld_ctx* c, bf16* feat0, unsigned char* mask) {
  Dev d = c->d;
  const Level l0 = net_of(c)->lv[0];
  launch_box(c->stream, box(0, l0.X - 1, 0, l0.Y - 1, 0, l0.Z - 1), [=] __device__(int x, int y, int z) {
    float acc[kFeat];
    for (int q = 0; q < kFeat; ++q) acc[q] = 0.f;
    int cnt = 0;
    for (int q = 0; q < 8; ++q) {
      const int i = 2 * x + 1 + (q & 1), j = 2 * y + 1 + ((q >> 1) & 1), k = 2 * z + 1 + (q >> 2);
      if (i > d.nx || j > d.ny || k > d.nz) continue;
      float f[kFeat];
      cell_features(d, i, j, k, f);
      for (int t = 0; t < kFeat; ++t) acc[t] += f[t];
      ++cnt;
      mask[(size_t)(i - 1) + (size_t)d.nx * ((size_t)(j - 1) + (size_t)d.ny * (size_t)(k - 1))] =
          cell_active(d, i, j, k) ? 1 : 0;
    }
    __align__(16) bf16 o[kFeatPad];
    for (int t = 0; t < kFeatPad; ++t) o[t] = __float2bfloat16_rn(t < kFeat ? acc[t] / (float)cnt : 0.f);
    uint4* dst = reinterpret_cast<uint4*>(feat0 + ((size_t)(z * l0.Y + y) * l0.X + x) * kFeatPad);
    dst[0] = reinterpret_cast<const uint4*>(o)[0];
    dst[1] = reinterpret_cast<const uint4*>(o)[1];
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// Host features (x, y, z, 5 channels, x fastest, on the grid) averaged
// over the 2x2x2 cells of each level-0 voxel as make_features does, into
// n->feat.
int upload_features(ttfld_ctx* c, const float* feat) {
  Net* n = net_of(c);
  const Level fi = n->full, l0 = n->lv[0];
  std::vector<bf16> hf((size_t)l0.vox() * kFeatPad);
  for (int z = 0; z < l0.Z; ++z)
    for (int y = 0; y < l0.Y; ++y)
      for (int x = 0; x < l0.X; ++x) {
        float acc[kFeat] = {0.f, 0.f, 0.f, 0.f, 0.f};
        int cnt = 0;
        for (int q = 0; q < 8; ++q) {
          const int xx = 2 * x + (q & 1), yy = 2 * y + ((q >> 1) & 1), zz = 2 * z + (q >> 2);
          if (xx >= fi.X || yy >= fi.Y || zz >= fi.Z) continue;
          const float* f = feat + (((size_t)zz * fi.Y + yy) * fi.X + xx) * kFeat;
          for (int t = 0; t < kFeat; ++t) acc[t] += f[t];
          ++cnt;
        }
        bf16* o = hf.data() + (((size_t)z * l0.Y + y) * l0.X + x) * kFeatPad;
        for (int t = 0; t < kFeatPad; ++t) o[t] = __float2bfloat16_rn(t < kFeat ? acc[t] / (float)cnt : 0.f);
      }
  TT_CHECK(cudaMemcpyAsync(n->feat, hf.data(), hf.size() * 2, cudaMemcpyHostToDevice, c->stream));
  return check_cuda(cudaStreamSynchronize(c->stream), "upload features");
}

}  // namespace

namespace ttfld {

void unet_free(ttfld_ctx* c) {
  Net* n = net_of(c);
  if (!n) return;
  if (n->p) cudaFree(n->p);
  if (n->w16) cudaFree(n->w16);
  if (n->act_mem) cudaFree(n->act_mem);
  if (n->ds_feat) cudaFree(n->ds_feat);
  free(n);
  c->unet = nullptr;
}

// Learned initial guess into the interior of x (a halo array, zeroed by the
// caller): delta_ER = pred * 0.01 * E on the active cells, 0 elsewhere.
int unet_guess(ttfld_ctx* c, double* x, double* /*resid_l1*/) {
  Net* n = net_of(c);
  if (!n || !n->ready) return TTFLD_E_NOMODEL;
  int rc;
  if ((rc = prep_weights(c)) || (rc = make_features(c, n->feat, n->mask)) || (rc = forward(c))) return rc;
  Dev d = c->d;
  const float* pred = n->pred;
  const unsigned char* mask = n->mask;
  launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) {
    const size_t v = (size_t)(i - 1) + (size_t)d.nx * ((size_t)(j - 1) + (size_t)d.ny * (size_t)(k - 1));
    const size_t h = hidx(d, i, j, k);
    x[h] = mask[v] ? (double)pred[v] * kTargetScale * d.ER[h] : 0.0;
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// Called after a solve that should become a training pair: features of the
// state the solve started from and its solution delta_ER / E as the target.
int unet_capture(ttfld_ctx* c) {
  Net* n = net_of(c);
  if (!n || !n->capture_next || !n->ds_feat) return 0;
  n->capture_next = 0;
  if (n->count >= n->cap) return 0;
  const long long V0 = L(0).vox(), VF = n->full.vox();
  bf16* feat = n->ds_feat + (size_t)n->count * V0 * kFeatPad;
  unsigned char* mask = n->ds_mask + (size_t)n->count * VF;
  bf16* tgt = n->ds_target + (size_t)n->count * VF;
  int rc = make_features(c, feat, mask);
  if (rc) return rc;
  Dev d = c->d;
  launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) {
    const size_t v = (size_t)(i - 1) + (size_t)d.nx * ((size_t)(j - 1) + (size_t)d.ny * (size_t)(k - 1));
    const size_t h = hidx(d, i, j, k);
    tgt[v] = __float2bfloat16_rn((float)(d.DELTA_ER[h] / d.ER[h] / kTargetScale));
  });
  TT_CHECK_LAUNCH();
  n->count += 1;
  return 0;
}

}  // namespace ttfld

extern "C" {

int ttfld_guess_init(ttfld_ctx* c, uint64_t seed) {
  if (!c) return TTFLD_E_ARGS;
  int rc;
  if ((rc = ensure_net(c)) || (rc = init_params(c, seed))) return rc;
  c->have_model = 1;
  return 0;
}

int ttfld_guess_dataset(ttfld_ctx* c, int capacity) {
  if (!c || capacity < 1) return TTFLD_E_ARGS;
  int rc;
  if ((rc = ensure_net(c))) return rc;
  Net* n = net_of(c);
  if (n->ds_feat) { cudaFree(n->ds_feat); n->ds_feat = nullptr; }
  const long long V0 = L(0).vox(), VF = n->full.vox();
  const size_t fb = align256((size_t)capacity * V0 * kFeatPad * 2);
  const size_t tb = align256((size_t)capacity * VF * 2);
  const size_t mb = align256((size_t)capacity * VF);
  char* mem = nullptr;
  TT_CHECK(cudaMalloc((void**)&mem, fb + tb + mb));
  n->ds_feat = (bf16*)mem;
  n->ds_target = (bf16*)(mem + fb);
  n->ds_mask = (unsigned char*)(mem + fb + tb);
  n->cap = capacity;
  n->count = 0;
  return 0;
}

int ttfld_guess_capture_next(ttfld_ctx* c) {
  if (!c || !c->unet || !net_of(c)->ds_feat) return TTFLD_E_ARGS;
  net_of(c)->capture_next = 1;
  return 0;
}

int ttfld_guess_dataset_count(ttfld_ctx* c) { return (c && c->unet) ? net_of(c)->count : 0; }

// One pass (or several) of Adam over the captured pairs in a seeded order.
int ttfld_guess_train(ttfld_ctx* c, int epochs, double lr, uint64_t seed, double* mean_loss) {
  if (!c || epochs < 1 || !(lr > 0.0)) return TTFLD_E_ARGS;
  Net* n = net_of(c);
  if (!n || !n->ready) return TTFLD_E_NOMODEL;
  if (n->count < 1) return TTFLD_E_ARGS;
  const long long V0 = L(0).vox(), VF = n->full.vox();
  GradWork gw;
  int rc0 = alloc_gradwork(n, &gw);
  if (rc0) return rc0;
  std::vector<int> order(n->count);
  uint64_t st = seed * 0x9E3779B97F4A7C15ULL + 1;
  double tot = 0.0;
  int cnt = 0, rc = 0;
  for (int e = 0; e < epochs && !rc; ++e) {
    for (int q = 0; q < n->count; ++q) order[q] = q;
    for (int q = n->count - 1; q > 0; --q) {
      st ^= st << 13; st ^= st >> 7; st ^= st << 17;
      int r = (int)(st % (uint64_t)(q + 1));
      int t = order[q]; order[q] = order[r]; order[r] = t;
    }
    for (int q = 0; q < n->count && !rc; ++q) {
      const int sidx = order[q];
      // expand the stored pair into the network's input / target buffers
      const bf16* f = n->ds_feat + (size_t)sidx * V0 * kFeatPad;
      const bf16* tg = n->ds_target + (size_t)sidx * VF;
      if (cudaMemcpyAsync(n->feat, f, (size_t)V0 * kFeatPad * 2, cudaMemcpyDeviceToDevice, c->stream) ||
          cudaMemcpyAsync(n->mask, n->ds_mask + (size_t)sidx * VF, (size_t)VF, cudaMemcpyDeviceToDevice, c->stream)) {
        rc = TTFLD_E_CUDA;
        break;
      }
      float* target = n->target;
      launch_box(c->stream, box(0, (int)(VF - 1), 0, 0, 0, 0), [=] __device__(int v, int, int) {
        target[v] = __bfloat162float(tg[v]);
      });
      double loss = 0.0;
      if ((rc = prep_weights(c)) || (rc = forward(c)) || (rc = backward(c, &gw, &loss))) break;
      n->step += 1;
      const float b1 = 0.9f, b2 = 0.999f;
      const float c1 = 1.f - powf(b1, (float)n->step), c2 = 1.f - powf(b2, (float)n->step);
      adam_kernel<<<GRID(n->nparams), 256, 0, c->stream>>>(n->p, n->g, n->m, n->v, n->nparams, (float)lr, b1, b2,
                                                            1e-8f, c1, c2);
      count_launches(1);
      n->wdirty = 1;
      tot += loss;
      ++cnt;
    }
  }
  cudaStreamSynchronize(c->stream);
  cudaFree(gw.gpad);
  if (rc) return rc;
  if (mean_loss) *mean_loss = cnt ? tot / cnt : 0.0;
  c->have_model = 1;
  return 0;
}

// Loss and gradients of all parameters for a given input (x, y, z, 5
// channels, x fastest, on the grid), target and mask: the hook the gradient
// tests use.
int ttfld_guess_gradients(ttfld_ctx* c, const float* feat, const float* target, const unsigned char* mask,
                          double* loss, float* grads) {
  if (!c || !feat || !target || !mask) return TTFLD_E_ARGS;
  Net* n = net_of(c);
  if (!n || !n->ready) return TTFLD_E_NOMODEL;
  const long long VF = n->full.vox();
  int rc = upload_features(c, feat);
  if (rc) return rc;
  TT_CHECK(cudaMemcpy(n->target, target, (size_t)VF * 4, cudaMemcpyHostToDevice));
  TT_CHECK(cudaMemcpy(n->mask, mask, (size_t)VF, cudaMemcpyHostToDevice));
  GradWork gw;
  if ((rc = alloc_gradwork(n, &gw))) return rc;
  rc = prep_weights(c);
  if (!rc) rc = forward(c);
  if (!rc) rc = backward(c, &gw, loss);
  cudaStreamSynchronize(c->stream);
  cudaFree(gw.gpad);
  if (rc) return rc;
  if (grads) TT_CHECK(cudaMemcpy(grads, n->g, n->nparams * 4, cudaMemcpyDeviceToHost));
  return 0;
}

// Prediction (network output, normalised target units) for a given input.
int ttfld_guess_predict(ttfld_ctx* c, const float* feat, float* pred) {
  if (!c || !feat || !pred) return TTFLD_E_ARGS;
  Net* n = net_of(c);
  if (!n || !n->ready) return TTFLD_E_NOMODEL;
  const long long VF = n->full.vox();
  int rc;
  if ((rc = upload_features(c, feat)) || (rc = prep_weights(c)) || (rc = forward(c))) return rc;
  TT_CHECK(cudaStreamSynchronize(c->stream));
  TT_CHECK(cudaMemcpy(pred, n->pred, (size_t)VF * 4, cudaMemcpyDeviceToHost));
  return 0;
}

int ttfld_guess_set_conv(int use_tcgen05) {
  if (use_tcgen05 < 0 || use_tcgen05 > 2) return TTFLD_E_ARGS;
  g_conv_tc = use_tcgen05;
  return 0;
}

size_t ttfld_guess_num_params(void) {
  Net tmp;
  memset(&tmp, 0, sizeof(tmp));
  layout(&tmp);
  return tmp.nparams;
}

// Weights blob: "TTFLDNN2", uint64 nparams, float params[nparams].
int ttfld_guess_save(ttfld_ctx* c, void* blob, size_t bytes, size_t* needed) {
  if (!c) return TTFLD_E_ARGS;
  const size_t np = ttfld_guess_num_params();
  const size_t need = 16 + np * 4;
  if (needed) *needed = need;
  Net* n = net_of(c);
  if (!n || !n->ready) return TTFLD_E_NOMODEL;
  if (!blob) return 0;
  if (bytes < need) return TTFLD_E_ARGS;
  memcpy(blob, "TTFLDNN2", 8);
  uint64_t np64 = np;
  memcpy((char*)blob + 8, &np64, 8);
  TT_CHECK(cudaMemcpy((char*)blob + 16, n->p, np * 4, cudaMemcpyDeviceToHost));
  return 0;
}

int ttfld_guess_load(ttfld_ctx* c, const void* blob, size_t bytes) {
  if (!c || !blob || bytes < 16) return TTFLD_E_ARGS;
  const size_t np = ttfld_guess_num_params();
  uint64_t np64 = 0;
  memcpy(&np64, (const char*)blob + 8, 8);
  if (memcmp(blob, "TTFLDNN2", 8) != 0 || np64 != np || bytes < 16 + np * 4) return TTFLD_E_ARGS;
  int rc = ensure_net(c);
  if (rc) return rc;
  Net* n = net_of(c);
  TT_CHECK(cudaMemcpy(n->p, (const char*)blob + 16, np * 4, cudaMemcpyHostToDevice));
  TT_CHECK(cudaMemset(n->m, 0, np * 4));
  TT_CHECK(cudaMemset(n->v, 0, np * 4));
  n->step = 0;
  n->ready = 1;
  n->wdirty = 1;
  c->have_model = 1;
  return 0;
}

}  // extern "C"
