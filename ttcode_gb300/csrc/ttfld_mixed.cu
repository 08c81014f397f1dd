// ttfld_mixed.cu -- the two fast solvers of SOLVE_WITH_SOR's system:
//
//  * TTFLD_SOLVER_MIXED: FP32 red-black SOR sweeps on the correction
//    equation A e = r inside an FP64 defect-correction loop
//    (x += e; r = b - A x in FP64).  Red-black SOR is a stationary iteration,
//    so m sweeps on A e = r from e = 0 followed by x += e give the same
//    iterate as m more sweeps on A x = b; the FP64 residual re-anchors the
//    iterate so the FP32 rounding never accumulates.  It stops on the true
//    residual ||b - A x||_1 / ||b||_1 <= tol.
//  * TTFLD_SOLVER_SOR64_FAST: the reference's FP64 red-black SOR with its
//    in-sweep stopping rule (ppsor.f:161-177), on Jacobi-scaled
//    coefficients with fused multiply-adds.
//
// Both keep their working arrays colour-compacted: the cells of one colour
// in a (j,k) row are stored contiguously along the radial index, padded to
// a multiple of four, so a half-sweep reads and writes only its own colour
// with 16-byte vector accesses.  For cell (i,j,k) (1-based) the colour is
// (i+j+k)&1 (0 = the reference's first pass, ppsor.f:59-61), its slot is
// h = (i-1)>>1 in row (k-1)*NY + (j-1).  In a row with q = (j+k)&1 (0-based
// j,k) the colour-c cells have i0 = 2h + off, off = (1+q+c)&1; their radial
// neighbours in the other colour sit at h+off-1 and h+off, the phi and
// theta neighbours at the same h.
#include <math.h>

#include "ttfld_internal.cuh"

namespace ttfld {

struct Cmp {
  int nx, ny, nz, nxp;  // nxp: padded slots per colour row (multiple of 4)
  int poles;            // theta rows 1 and NZ-1 read themselves for the mirror; row NZ is not swept
  long long rows;       // ny * nz
  size_t csz;           // slots per colour array (no ghost planes)
  size_t gsz;           // slots per colour array with theta ghost planes
};

static Cmp make_cmp(const Dev& d) {
  Cmp g;
  g.nx = d.nx; g.ny = d.ny; g.nz = d.nz;
  g.poles = d.poles;
  int nxh = (d.nx + 1) / 2;
  g.nxp = (nxh + 3) / 4 * 4;
  g.rows = (long long)d.ny * d.nz;
  g.csz = (size_t)g.rows * g.nxp;
  g.gsz = (size_t)(d.nz + 2) * d.ny * g.nxp;
  return g;
}

struct Mix32 {
  float* a[6][2];   // W E S N B T (xm xp jm jp km kp) over A, per colour
  float* ainv[2];   // 1/A
  float* diag[2];   // A (for the in-sweep residual norm)
  float* rhat[2];   // r / A
  float* e[2];      // correction, with theta ghost planes
};

struct Fast64 {
  double* a[6][2];
  double* bhat[2];  // (b - ghost couplings) / A
  double* diag[2];  // A
  double* x[2];     // iterate, with theta ghost planes
};

// Per-block flags of the neighbour-flag sweep form (below).
constexpr int kFlagStride = 32;        // unsigned ints per flag: one 128-byte line per block
constexpr int kMaxLocalBlocks = 1024;  // flags in the workspace
constexpr size_t kFlagBytes = (size_t)kMaxLocalBlocks * kFlagStride * sizeof(unsigned int);

struct MixWork {
  Cmp g;
  int have32, have64;
  void* mem32;
  void* mem64;
  Mix32 m32;
  Fast64 m64;
  unsigned int* flags;     // per-block half-sweep counters of the neighbour-flag sweep form
  unsigned int flag_base;  // their value when the next launch of that form starts
};

__host__ __device__ __forceinline__ size_t cslot(const Cmp& g, int j0, int k0, int h) {
  return ((size_t)k0 * g.ny + j0) * g.nxp + h;
}
__host__ __device__ __forceinline__ size_t gslot(const Cmp& g, int j0, int k0, int h) {
  return ((size_t)(k0 + 1) * g.ny + j0) * g.nxp + h;
}

static MixWork* work(ttfld_ctx* c) {
  if (!c->mix_slab) {
    MixWork* w = (MixWork*)calloc(1, sizeof(MixWork));
    w->g = make_cmp(c->d);
    c->mix_slab = w;
  }
  return (MixWork*)c->mix_slab;
}

static int ensure32(ttfld_ctx* c) {
  MixWork* w = work(c);
  if (w->have32) return 0;
  const Cmp& g = w->g;
  const size_t flag_floats = kFlagBytes / sizeof(float);  // the flags first: 128-byte lines
  size_t n = flag_floats + 2 * (6 + 3) * g.csz + 2 * g.gsz;
  float* p = nullptr;
  TT_CHECK(cudaMalloc((void**)&p, n * sizeof(float)));
  TT_CHECK(cudaMemset(p, 0, n * sizeof(float)));
  w->mem32 = p;
  w->flags = reinterpret_cast<unsigned int*>(p);
  w->flag_base = 0;
  p += flag_floats;
  for (int q = 0; q < 6; ++q)
    for (int col = 0; col < 2; ++col) { w->m32.a[q][col] = p; p += g.csz; }
  for (int col = 0; col < 2; ++col) { w->m32.ainv[col] = p; p += g.csz; }
  for (int col = 0; col < 2; ++col) { w->m32.diag[col] = p; p += g.csz; }
  for (int col = 0; col < 2; ++col) { w->m32.rhat[col] = p; p += g.csz; }
  for (int col = 0; col < 2; ++col) { w->m32.e[col] = p; p += g.gsz; }
  w->have32 = 1;
  return 0;
}

static int ensure64(ttfld_ctx* c) {
  MixWork* w = work(c);
  if (w->have64) return 0;
  const Cmp& g = w->g;
  size_t n = 2 * (6 + 2) * g.csz + 2 * g.gsz;
  double* p = nullptr;
  TT_CHECK(cudaMalloc((void**)&p, n * sizeof(double)));
  TT_CHECK(cudaMemset(p, 0, n * sizeof(double)));
  w->mem64 = p;
  for (int q = 0; q < 6; ++q)
    for (int col = 0; col < 2; ++col) { w->m64.a[q][col] = p; p += g.csz; }
  for (int col = 0; col < 2; ++col) { w->m64.bhat[col] = p; p += g.csz; }
  for (int col = 0; col < 2; ++col) { w->m64.diag[col] = p; p += g.csz; }
  for (int col = 0; col < 2; ++col) { w->m64.x[col] = p; p += g.gsz; }
  w->have64 = 1;
  return 0;
}

void mix_free(ttfld_ctx* c) {
  MixWork* w = (MixWork*)c->mix_slab;
  if (!w) return;
  if (w->mem32) cudaFree(w->mem32);
  if (w->mem64) cudaFree(w->mem64);
  free(w);
  c->mix_slab = nullptr;
}

// ---- FP32 path ----------------------------------------------------------

// Jacobi-scaled FP32 coefficients of the current SOR_A..G.
static int prep32(ttfld_ctx* c) {
  MixWork* w = work(c);
  Dev d = c->d;
  Cmp g = w->g;
  Mix32 m = w->m32;
  launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) {
    size_t q = cidx(d, i, j, k);
    int col = (i + j + k) & 1;
    size_t s = cslot(g, j - 1, k - 1, (i - 1) >> 1);
    double inv = 1.0 / d.SA[q];
    m.a[0][col][s] = (float)(d.SB[q] * inv);
    m.a[1][col][s] = (float)(d.SC[q] * inv);
    m.a[2][col][s] = (float)(d.SD[q] * inv);
    m.a[3][col][s] = (float)(d.SE[q] * inv);
    m.a[4][col][s] = (float)(d.SF[q] * inv);
    m.a[5][col][s] = (float)(d.SG[q] * inv);
    m.ainv[col][s] = (float)inv;
    m.diag[col][s] = (float)d.SA[q];
  });
  TT_CHECK_LAUNCH();
  return 0;
}

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
// Loads of the correction e are plain coherent loads, never the read-only
// path: the persistent kernels write e in one half-sweep and read it, from
// other SMs, in the next.  The wait between them (acquire loads and a fence
// by the polling threads, then a block barrier) orders those loads after
// the other blocks' writes, as the PTX memory model defines it.
__device__ __forceinline__ float4 lde4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ float lde(const float* p) { return *p; }
// Loads of the coefficients (couplings, r-hat, A: 32 of the 40 bytes of a
// cell update, each read once per sweep) do not allocate in L1, so that the
// stream of them does not evict the lines of e that neighbouring items of
// the same block share.  The sweep kernels never write them.  Timed against
// plain loads on one GB300: 28.1 against 34.1 us per sweep at 160x256x128,
// 120.9 against 129.2 us at 160x512x256, within 1 % at 100x256x128.
__device__ __forceinline__ float4 ldc4(const float* p) {
  float4 v;
  asm("ld.global.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
      : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
      : "l"(p));
  return v;
}

// One colour of FP32 red-black SOR on A e = r (Jacobi-scaled), 4 cells per
// thread: res = (e + sum a_nb e_nb) - rhat (the reference's in-sweep residual
// divided by A, ppsor.f:64-71), e -= omega * res.  NORM sweeps also sum
// |A * res| (per thread in FP32, per block and grid in FP64 in a fixed
// order), i.e. the reference's RNORM (ppsor.f:73) of the iterate x + e.
// Item t is the t-th group of four colour slots (row-major over (k, j, h));
// its coefficients (aw..at: the W E S N B T couplings over A, r: rhat, dg:
// A) come in as arguments, from global or from shared memory.  POLES (a
// compile-time copy of Cmp::poles, so that the kernels without poles carry
// no test of it): theta rows 1 and NZ-1 take the cell itself as their
// neighbour across the edge, and row NZ is not swept.
template <int COL, bool NORM, bool POLES>
__device__ __forceinline__ void update_vec(const Cmp& g, const Mix32& m, float omega, long long t, int nv,
                                           size_t plane, float4 aw, float4 ae, float4 as, float4 an, float4 ab,
                                           float4 at, float4 r, float4 dg, float& nacc) {
  const float* eo = m.e[1 - COL];
  float* es = m.e[COL];
  const int hv = (int)(t % nv);
  const long long rr = t / nv;
  const int j0 = (int)(rr % g.ny), k0 = (int)(rr / g.ny);
  if (POLES && k0 == g.nz - 1) return;  // the north pole's mirror row (zmax_sor_index, ppsor.f:39-43)
  const int off = (1 + ((j0 + k0) & 1) + COL) & 1;
  const int h0 = hv * 4;
  const int ncol = (g.nx - off + 1) >> 1;  // valid slots in this row
  const size_t eb = gslot(g, j0, k0, h0);
  const int jm = j0 == 0 ? g.ny - 1 : j0 - 1;
  const int jp = j0 == g.ny - 1 ? 0 : j0 + 1;
  const float4 o = lde4(eo + eb);
  float xm0, xm1, xm2, xm3, xp0, xp1, xp2, xp3;
  if (off == 0) {
    xm0 = h0 > 0 ? lde(eo + eb - 1) : 0.f; xm1 = o.x; xm2 = o.y; xm3 = o.z;
    xp0 = o.x; xp1 = o.y; xp2 = o.z; xp3 = o.w;
  } else {
    xm0 = o.x; xm1 = o.y; xm2 = o.z; xm3 = o.w;
    xp0 = o.y; xp1 = o.z; xp2 = o.w; xp3 = (h0 + 4 < g.nxp) ? lde(eo + eb + 4) : 0.f;
  }
  const float4 s = lde4(eo + gslot(g, jm, k0, h0));
  const float4 nn = lde4(eo + gslot(g, jp, k0, h0));
  const float4 e = lde4(es + eb);
  // with poles the theta neighbour across either edge is the cell itself
  const float4 b = (POLES && k0 == 0) ? e : lde4(eo + eb - plane);
  const float4 tt = (POLES && k0 == g.nz - 2) ? e : lde4(eo + eb + plane);
  float4 out;
#define UPD(L, IDX, XM, XP)                                                                \
  {                                                                                        \
    float acc = fmaf(aw.L, XM, fmaf(ae.L, XP, fmaf(as.L, s.L, fmaf(an.L, nn.L,             \
                fmaf(ab.L, b.L, at.L * tt.L)))));                                          \
    float res = (e.L + acc) - r.L;                                                         \
    bool ok = h0 + IDX < ncol;                                                             \
    out.L = ok ? fmaf(-omega, res, e.L) : 0.f;                                             \
    if (NORM && ok) nacc += fabsf(dg.L * res);                                            \
  }
  UPD(x, 0, xm0, xp0) UPD(y, 1, xm1, xp1) UPD(z, 2, xm2, xp2) UPD(w, 3, xm3, xp3)
#undef UPD
  st4(es + eb, out);
}

// The same with the coefficients loaded from global memory (item t's four
// slots are floats 4t .. 4t+3 of each coefficient array).
template <int COL, bool NORM, bool POLES>
__device__ __forceinline__ void sweep_vec(const Cmp& g, const Mix32& m, float omega, long long t, int nv,
                                          size_t plane, float& nacc) {
  const size_t cb = (size_t)t * 4;
  const float4 aw = ldc4(m.a[0][COL] + cb), ae = ldc4(m.a[1][COL] + cb);
  const float4 as = ldc4(m.a[2][COL] + cb), an = ldc4(m.a[3][COL] + cb);
  const float4 ab = ldc4(m.a[4][COL] + cb), at = ldc4(m.a[5][COL] + cb);
  const float4 r = ldc4(m.rhat[COL] + cb);
  float4 dg = make_float4(0.f, 0.f, 0.f, 0.f);
  if (NORM) dg = ldc4(m.diag[COL] + cb);
  update_vec<COL, NORM, POLES>(g, m, omega, t, nv, plane, aw, ae, as, an, ab, at, r, dg, nacc);
}

// One colour per launch.  NORM launches of the second colour end with the
// last block applying the stop rule: once RNORM / RHSNORM <= stop_ratio the
// inner loop is done, and sweeps queued after that return at once.
template <int COL, bool NORM, bool POLES>
__global__ void __launch_bounds__(kThreads) sweep32_kernel(Cmp g, Mix32 m, float omega, SolverDev* sol,
                                                           double* partials, double stop_ratio) {
  __shared__ double sh[32];
  __shared__ bool last;
  if (*(volatile int*)&sol->done) return;
  const int nv = g.nxp >> 2;
  const long long n = g.rows * nv;
  const size_t plane = (size_t)g.ny * g.nxp;
  float nacc = 0.f;  // per-thread partial (a few cells): FP32, widened once below
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    sweep_vec<COL, NORM, POLES>(g, m, omega, t, nv, plane, nacc);
  if (COL == 1 && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&sol->iter, 1);
  if (NORM) {
    double sb = block_sum((double)nacc, sh);
    if (threadIdx.x == 0) {
      partials[COL * kMaxPartials + blockIdx.x] = sb;
      if (COL == 1) {
        __threadfence();
        last = (atomicAdd(&sol->ticket, 1u) == gridDim.x - 1);
      }
    }
    if (COL == 1) {
      __syncthreads();
      if (last) {
        __threadfence();
        double r0 = block_sum_array(partials, gridDim.x, sh);
        double r1 = block_sum_array(partials + kMaxPartials, gridDim.x, sh);
        if (threadIdx.x == 0) {
          double rnorm = r0 + r1;
          double ratio = rnorm / sol->rhsnorm;
          sol->rnorm = rnorm;
          sol->ratio = ratio;
          if (!isfinite(rnorm)) { sol->nonfinite = 1; sol->done = 1; }
          else if (!(ratio > stop_ratio)) sol->done = 1;
          sol->ticket = 0;
        }
      }
    }
  }
}

// A norm sweep whose in-sweep ratio is not below kStallFactor times the
// previous one (8 sweeps earlier) ends the inner loop: the FP32 iteration
// has reached its rounding floor relative to the anchor (on stiff,
// high-contrast systems after one or two decades), and re-anchoring in FP64
// continues the same iteration.  A false alarm costs one FP64 residual.
constexpr double kStallFactor = 0.999;

// The decision after a norm sweep, taken by thread 0 of every block on the
// same fixed-order total tot (so every block decides alike): stop at the
// target ratio, on a non-finite norm, or (stall_check) at the FP32 rounding
// floor.  Block 0 records it in sol; the result is 1 to stop.
__device__ __forceinline__ int norm_stop(SolverDev* sol, double tot, double stop_ratio, int stall_check,
                                         double& last_ratio) {
  const double ratio = tot / sol->rhsnorm;
  const bool stall = stall_check && last_ratio > 0.0 && !(ratio < kStallFactor * last_ratio);
  const int stop = !isfinite(tot) || !(ratio > stop_ratio) || stall;
  last_ratio = ratio;
  if (blockIdx.x == 0) {
    sol->rnorm = tot;
    sol->ratio = ratio;
    if (!isfinite(tot)) sol->nonfinite = 1;
    if (stall) sol->stalled = 1;
    if (stop) sol->done = 1;
  }
  return stop;
}

constexpr int kPersistThreads = 768;  // one block per SM: few barrier arrivals

// nsweeps FP32 sweeps in one launch (sweep_form 4, and the product form's
// stand-in where its flags do not cover the grid's blocks): both colours of
// every sweep with a grid barrier after each, every norm_every-th sweep (and
// the last) with the in-sweep norm.  Each block reduces its partial of a norm sweep; after the
// barrier every block adds all partials in the same fixed order, so all of
// them reach the same stop decision and leave the loop together.  Every
// thread keeps the same items from sweep to sweep.
template <bool POLES>
__global__ void __launch_bounds__(kPersistThreads) sweeps32_persistent(Cmp g, Mix32 m, float omega, SolverDev* sol,
                                                                      double* partials, double stop_ratio,
                                                                      int nsweeps, int norm_every, int stall_check) {
  __shared__ double sh[32];
  __shared__ int stop_sh;
  if (*(volatile int*)&sol->done) return;
  const int nv = g.nxp >> 2;
  const long long n = g.rows * nv;
  const size_t plane = (size_t)g.ny * g.nxp;
  const unsigned int nb = gridDim.x;
  const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x, ts = (long long)gridDim.x * blockDim.x;
  double last_ratio = -1.0;  // in-sweep ratio of the previous norm sweep of this launch (thread 0)
  unsigned long long passed = 0;  // grid barriers this block has passed
  for (int sw = 1; sw <= nsweeps; ++sw) {
    const bool norm = norm_every > 0 && (sw % norm_every == 0 || sw == nsweeps);
    float nacc = 0.f;
    if (norm) { for (long long t = t0; t < n; t += ts) sweep_vec<0, true, POLES>(g, m, omega, t, nv, plane, nacc); }
    else { for (long long t = t0; t < n; t += ts) sweep_vec<0, false, POLES>(g, m, omega, t, nv, plane, nacc); }
    if (!grid_sync(sol, nb, passed)) return;
    if (norm) { for (long long t = t0; t < n; t += ts) sweep_vec<1, true, POLES>(g, m, omega, t, nv, plane, nacc); }
    else { for (long long t = t0; t < n; t += ts) sweep_vec<1, false, POLES>(g, m, omega, t, nv, plane, nacc); }
    if (norm) {
      const double sb = block_sum((double)nacc, sh);
      if (threadIdx.x == 0) partials[blockIdx.x] = sb;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) sol->iter += 1;
    if (!grid_sync(sol, nb, passed)) return;
    if (norm) {
      const double tot = block_sum_array(partials, nb, sh);
      if (threadIdx.x == 0) stop_sh = norm_stop(sol, tot, stop_ratio, stall_check, last_ratio);
      __syncthreads();
      if (stop_sh) return;
    }
  }
}

// ---- neighbour flags instead of grid barriers (sweep_form 0, the product) ---
// Block b owns the contiguous items [n b / nb, n (b + 1) / nb).  A
// half-sweep of item t reads the other colour within one theta plane of t
// only (the theta neighbours one plane away, the phi neighbours in the same
// plane, the periodic wrap included, the r neighbours in the same row), so
// before its h-th half-sweep a block needs only the blocks that own items
// within one plane of its own (its neighbours) to have finished h - 1
// half-sweeps.  Each block publishes the half-sweeps it has finished in a
// flag of its own (a block barrier, a fence, a release store) and waits on
// its neighbours' flags (acquire loads, a fence, a block barrier) instead of
// on a grid barrier.  The relation is symmetric, so neighbours are never
// more than one half-sweep apart and no block overwrites a colour that a
// neighbour is still reading: every update reads the values it reads in the
// grid-barrier form, whose iterate this is, bit for bit.  Norm sweeps still
// end with a grid barrier: the stop decision needs every block's partial.
// Flags count half-sweeps from a base that the host advances by 2 nsweeps
// per launch, and every block leaves its flag at base + 2 nsweeps whenever
// it returns, so all flags equal the base when the next launch starts.
// Timed against the grid-barrier kernel in one process on a GB300: 4-6 %
// faster per sweep at 100x128x128, 100x256x128, 100x256x160 and
// 160x512x256, the same at 160x256x128 and 60x512x256 (a slow block holds
// up only its neighbours, not the grid).

__device__ __forceinline__ void st_release(unsigned int* p, unsigned int v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// The block whose items [n b / nb, n (b + 1) / nb) hold item t (0 <= t < n).
__device__ __forceinline__ int owner_block(long long t, long long n, int nb) {
  int b = (int)(t * nb / n);
  while (b + 1 < nb && n * (b + 1) / nb <= t) ++b;
  while (b > 0 && n * b / nb > t) --b;
  return b;
}

// This block has finished v half-sweeps: after every thread's stores.
__device__ __forceinline__ void publish_flag(unsigned int* flag, unsigned int v) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    st_release(flag, v);
  }
}

// Wait until blocks lo..hi other than this one have finished at least
// `target` half-sweeps; warp 0 polls, one flag per lane.  Bounded like the
// grid barriers: false after kBarrierSpins polls or once another block has
// given up.
__device__ __forceinline__ bool wait_flags(const unsigned int* flags, int lo, int hi, unsigned int target,
                                           SolverDev* sol) {
  __shared__ int ok_sh;
  if (threadIdx.x < 32) {
    int ok = 1;
    long long polls = 0;
    for (;;) {
      bool ready = true;
      for (int q = lo + (int)threadIdx.x; q <= hi; q += 32)
        if (q != (int)blockIdx.x && (int)(ld_acquire(flags + (size_t)q * kFlagStride) - target) < 0) ready = false;
      if (__all_sync(0xffffffffu, ready)) break;
      if (__any_sync(0xffffffffu, give_up(++polls, sol))) { ok = 0; break; }
      __nanosleep(32);
    }
    __threadfence();
    if (threadIdx.x == 0) {
      if (!ok) atomicExch(&sol->bar_timeout, 1);
      ok_sh = ok;
    }
  }
  __syncthreads();
  return ok_sh != 0;
}

template <bool POLES>
__global__ void __launch_bounds__(kPersistThreads) sweeps32_local(Cmp g, Mix32 m, float omega, SolverDev* sol,
                                                                 double* partials, double stop_ratio, int nsweeps,
                                                                 int norm_every, int stall_check, unsigned int* flags,
                                                                 unsigned int base) {
  __shared__ double sh[32];
  __shared__ int stop_sh;
  unsigned int* own = flags + (size_t)blockIdx.x * kFlagStride;
  const unsigned int fin = base + 2u * (unsigned int)nsweeps;
  if (*(volatile int*)&sol->done) {  // set before the launch, so the same for every block
    if (threadIdx.x == 0) *own = fin;
    return;
  }
  const int nv = g.nxp >> 2;
  const long long n = g.rows * nv;
  const size_t plane = (size_t)g.ny * g.nxp;
  const int nb = (int)gridDim.x;
  const long long t0 = n * blockIdx.x / nb, t1 = n * (blockIdx.x + 1) / nb;
  const long long reach = (long long)g.ny * nv;  // items within one theta plane
  const int lo = owner_block(t0 > reach ? t0 - reach : 0, n, nb);
  const int hi = owner_block(t1 - 1 + reach < n ? t1 - 1 + reach : n - 1, n, nb);
  const long long ta = t0 + threadIdx.x;
  const int bt = (int)blockDim.x;
  double last_ratio = -1.0;
  unsigned long long passed = 0;  // grid barriers this block has passed
  unsigned int half = base;  // half-sweeps this block has finished
  bool synced = true;        // every block has finished as many (launch start, grid barrier)
  for (int sw = 1; sw <= nsweeps; ++sw) {
    const bool norm = norm_every > 0 && (sw % norm_every == 0 || sw == nsweeps);
    float nacc = 0.f;
    if (!synced && !wait_flags(flags, lo, hi, half, sol)) break;
    if (norm) { for (long long t = ta; t < t1; t += bt) sweep_vec<0, true, POLES>(g, m, omega, t, nv, plane, nacc); }
    else { for (long long t = ta; t < t1; t += bt) sweep_vec<0, false, POLES>(g, m, omega, t, nv, plane, nacc); }
    publish_flag(own, ++half);
    if (!wait_flags(flags, lo, hi, half, sol)) break;
    if (norm) { for (long long t = ta; t < t1; t += bt) sweep_vec<1, true, POLES>(g, m, omega, t, nv, plane, nacc); }
    else { for (long long t = ta; t < t1; t += bt) sweep_vec<1, false, POLES>(g, m, omega, t, nv, plane, nacc); }
    publish_flag(own, ++half);
    synced = false;
    if (norm) {
      const double sb = block_sum((double)nacc, sh);
      if (threadIdx.x == 0) partials[blockIdx.x] = sb;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) sol->iter += 1;
    if (norm) {
      if (!grid_sync(sol, (unsigned int)nb, passed)) break;
      synced = true;
      const double tot = block_sum_array(partials, nb, sh);
      if (threadIdx.x == 0) stop_sh = norm_stop(sol, tot, stop_ratio, stall_check, last_ratio);
      __syncthreads();
      if (stop_sh) break;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) *own = fin;
}

// ---- temporal blocking through L2 (sweep_form 3) ---------------------------
// Two sweeps per pass of a wavefront over windows of win_planes theta
// planes: in phase p the four half-sweeps of the pair (colour 0 and colour 1
// of sweep A, then of sweep B) run on windows p, p - 2, p - 4 and p - 6,
// with a grid barrier after every phase.  A half-sweep of plane k reads the
// other colour at planes k-1, k and k+1 only, so a lag of two windows per
// stage keeps every read after the write it needs and before the write that
// replaces it: the iterate after each pair is the other forms', bit for
// bit.  The seven windows between a window's first and last stage are
// meant to stay in L2, so that each array crosses DRAM once per pair
// instead of once per sweep; the price is nwin + 6 grid barriers per pair
// instead of four.  A pair whose first sweep carries the in-sweep norm, and
// an odd last sweep, run as single sweeps.
constexpr int kWaveLag = 2;

// Items [lo, lo + len) of window w (len 0 outside 0..nwin-1); the form is
// launched only for fewer than 2^31 items.
__device__ __forceinline__ void wave_window(int w, int nwin, int wlen, int n, int& lo, int& len) {
  if (w < 0 || w >= nwin) { lo = 0; len = 0; return; }
  lo = w * wlen;
  len = (lo + wlen < n ? lo + wlen : n) - lo;
}

template <bool POLES>
__global__ void __launch_bounds__(kPersistThreads) sweeps32_wave(Cmp g, Mix32 m, float omega, SolverDev* sol,
                                                                double* partials, double stop_ratio, int nsweeps,
                                                                int norm_every, int stall_check, int win_planes) {
  __shared__ double sh[32];
  __shared__ int stop_sh;
  if (*(volatile int*)&sol->done) return;
  const int nv = g.nxp >> 2;
  const int n = (int)(g.rows * nv);
  const int wlen = win_planes * g.ny * nv;  // items of one window
  const int nwin = (n + wlen - 1) / wlen;
  const size_t plane = (size_t)g.ny * g.nxp;
  const unsigned int nb = gridDim.x;
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x, ts = gridDim.x * blockDim.x;
  double last_ratio = -1.0;
  unsigned long long passed = 0;  // grid barriers this block has passed
  int sw = 0;
  while (sw < nsweeps) {
    const bool norm_a = norm_every > 0 && ((sw + 1) % norm_every == 0 || sw + 1 == nsweeps);
    const bool pair = sw + 2 <= nsweeps && !norm_a;
    const int last = sw + (pair ? 2 : 1);  // the last sweep of this round
    const bool norm = norm_every > 0 && (last % norm_every == 0 || last == nsweeps);
    float nacc = 0.f;
    if (pair) {
      const int nphase = nwin + 3 * kWaveLag;
      for (int p = 0; p < nphase; ++p) {
        // stage st (colour st & 1; sweep B from stage 2) works on window
        // p - kWaveLag * st: its items [lo_st, lo_st + len_st), len 0 when idle
        int lo0, lo1, lo2, lo3, len0, len1, len2, len3;
        wave_window(p, nwin, wlen, n, lo0, len0);
        wave_window(p - kWaveLag, nwin, wlen, n, lo1, len1);
        wave_window(p - 2 * kWaveLag, nwin, wlen, n, lo2, len2);
        wave_window(p - 3 * kWaveLag, nwin, wlen, n, lo3, len3);
        const int total = len0 + len1 + len2 + len3;
        for (int u = t0; u < total; u += ts) {
          int q;
          int t;
          if (u < len0) { q = 0; t = lo0 + u; }
          else if (u < len0 + len1) { q = 1; t = lo1 + (u - len0); }
          else if (u < len0 + len1 + len2) { q = 2; t = lo2 + (u - len0 - len1); }
          else { q = 3; t = lo3 + (u - len0 - len1 - len2); }
          switch (q) {
            case 0: sweep_vec<0, false, POLES>(g, m, omega, t, nv, plane, nacc); break;
            case 1: sweep_vec<1, false, POLES>(g, m, omega, t, nv, plane, nacc); break;
            case 2:
              if (norm) sweep_vec<0, true, POLES>(g, m, omega, t, nv, plane, nacc);
              else sweep_vec<0, false, POLES>(g, m, omega, t, nv, plane, nacc);
              break;
            default:
              if (norm) sweep_vec<1, true, POLES>(g, m, omega, t, nv, plane, nacc);
              else sweep_vec<1, false, POLES>(g, m, omega, t, nv, plane, nacc);
          }
        }
        if (p == nphase - 1) {
          if (norm) {
            const double sb = block_sum((double)nacc, sh);
            if (threadIdx.x == 0) partials[blockIdx.x] = sb;
          }
          if (blockIdx.x == 0 && threadIdx.x == 0) sol->iter += 2;
        }
        if (!grid_sync(sol, nb, passed)) return;
      }
    } else {
      if (norm) { for (int t = t0; t < n; t += ts) sweep_vec<0, true, POLES>(g, m, omega, t, nv, plane, nacc); }
      else { for (int t = t0; t < n; t += ts) sweep_vec<0, false, POLES>(g, m, omega, t, nv, plane, nacc); }
      if (!grid_sync(sol, nb, passed)) return;
      if (norm) { for (int t = t0; t < n; t += ts) sweep_vec<1, true, POLES>(g, m, omega, t, nv, plane, nacc); }
      else { for (int t = t0; t < n; t += ts) sweep_vec<1, false, POLES>(g, m, omega, t, nv, plane, nacc); }
      if (norm) {
        const double sb = block_sum((double)nacc, sh);
        if (threadIdx.x == 0) partials[blockIdx.x] = sb;
      }
      if (blockIdx.x == 0 && threadIdx.x == 0) sol->iter += 1;
      if (!grid_sync(sol, nb, passed)) return;
    }
    if (norm) {  // the persistent kernel's decision, on the same kind of sum
      const double tot = block_sum_array(partials, nb, sh);
      if (threadIdx.x == 0) stop_sh = norm_stop(sol, tot, stop_ratio, stall_check, last_ratio);
      __syncthreads();
      if (stop_sh) return;
    }
    sw = last;
  }
}

// ---- TMA-staged persistent sweeps (measured alternative) -------------------
// The same sweeps as sweeps32_persistent, with each block's coefficients
// streamed through shared memory by bulk asynchronous copies
// (cp.async.bulk, completion on an mbarrier).  Block b owns a contiguous run
// of items, processed per half-sweep in chunks of kTmaThreads items (one per
// thread).  Thread 0 keeps kStages chunks in flight: the chunk's six
// couplings and rhat (and A on norm sweeps) are contiguous spans of 16 bytes
// per item in every array, one bulk copy each.  The coefficients do not
// depend on the sweep, so the copies for the next half-sweep are issued
// before the grid barrier and their latency hides behind it; only the
// correction e is read through the cache after the barrier.
constexpr int kTmaThreads = 512;
constexpr int kStages = 3;
constexpr int kStageArrays = 8;  // aw ae as an ab at rhat A
constexpr size_t kStageBytes = (size_t)kStageArrays * kTmaThreads * 16;
constexpr size_t kTmaSmem = 128 + kStages * kStageBytes;
constexpr long long kMbarSpins = 1LL << 22;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_to_smem(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Bounded wait for phase `parity` of a stage barrier (all threads).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, SolverDev* sol) {
  long long n = 0;
  while (!mbar_try_wait(bar, parity)) {
    if (++n > kMbarSpins) {
      atomicExch(&sol->bar_timeout, 1);
      return false;
    }
  }
  return true;
}

struct TmaPlan {
  long long t0, t1;  // this block's items
  int nk;            // chunks per half-sweep
  int per_sweep;     // chunks per sweep (2 nk)
};

// Thread 0: queue the copies of chunk gi (half-sweep gi / nk, chunk gi % nk)
// into stage gi % kStages.
__device__ __forceinline__ void issue_chunk(const Mix32& m, const TmaPlan& pl, long long gi, int norm_every,
                                            int nsweeps, unsigned char* stages, uint64_t* bars) {
  const int h = (int)(gi / pl.nk), k = (int)(gi % pl.nk);
  const int col = h & 1, sw = h / 2 + 1;
  const bool norm = norm_every > 0 && (sw % norm_every == 0 || sw == nsweeps);
  const long long ta = pl.t0 + (long long)k * kTmaThreads;
  const long long tb = ta + kTmaThreads < pl.t1 ? ta + kTmaThreads : pl.t1;
  const uint32_t bytes = (uint32_t)(tb - ta) * 16u;
  const int st = (int)(gi % kStages);
  unsigned char* base = stages + (size_t)st * kStageBytes;
  const int na = norm ? 8 : 7;
  mbar_expect_tx(bars + st, bytes * na);
  const float* src[8] = {m.a[0][col], m.a[1][col], m.a[2][col], m.a[3][col],
                         m.a[4][col], m.a[5][col], m.rhat[col], m.diag[col]};
  for (int q = 0; q < na; ++q)
    bulk_to_smem(base + (size_t)q * kTmaThreads * 16, src[q] + ta * 4, bytes, bars + st);
}

template <bool POLES>
__global__ void __launch_bounds__(kTmaThreads) sweeps32_tma(Cmp g, Mix32 m, float omega, SolverDev* sol,
                                                            double* partials, double stop_ratio, int nsweeps,
                                                            int norm_every, int stall_check) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  unsigned char* stages = smem + 128;
  __shared__ double sh[32];
  __shared__ int stop_sh;
  if (*(volatile int*)&sol->done) return;  // set before the launch, so the same for every block
  const int nv = g.nxp >> 2;
  const long long n = g.rows * nv;
  const size_t plane = (size_t)g.ny * g.nxp;
  const int nb = (int)gridDim.x;
  TmaPlan pl;
  pl.t0 = n * blockIdx.x / nb;
  pl.t1 = n * (blockIdx.x + 1) / nb;
  pl.nk = (int)((pl.t1 - pl.t0 + kTmaThreads - 1) / kTmaThreads);
  pl.per_sweep = 2 * pl.nk;
  const long long total = (long long)pl.per_sweep * nsweeps;  // chunks of this launch
  if (threadIdx.x == 0) {
    for (int q = 0; q < kStages; ++q) mbar_init(bars + q, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  long long issued = 0, done_chunks = 0;
  if (threadIdx.x == 0)
    for (; issued < kStages && issued < total; ++issued) issue_chunk(m, pl, issued, norm_every, nsweeps, stages, bars);
  bool ok = true, synced = true;  // no barrier before the launch's first half-sweep
  double last_ratio = -1.0;       // in-sweep ratio of the previous norm sweep of this launch (thread 0)
  unsigned long long passed = 0;  // grid barriers this block has passed
  for (int sw = 1; sw <= nsweeps && ok; ++sw) {
    const bool norm = norm_every > 0 && (sw % norm_every == 0 || sw == nsweeps);
    float nacc = 0.f;
    for (int col = 0; col < 2 && ok; ++col) {
      if (!synced && !grid_sync(sol, nb, passed)) { ok = false; break; }
      synced = false;
      for (int k = 0; k < pl.nk; ++k) {
        const int st = (int)(done_chunks % kStages);
        if (!mbar_wait(bars + st, (uint32_t)((done_chunks / kStages) & 1), sol)) { ok = false; break; }
        const long long t = pl.t0 + (long long)k * kTmaThreads + threadIdx.x;
        if (t < pl.t1) {
          const float4* sb = reinterpret_cast<const float4*>(stages + (size_t)st * kStageBytes) + threadIdx.x;
          const float4 dg = norm ? sb[7 * kTmaThreads] : make_float4(0.f, 0.f, 0.f, 0.f);
#define UPD_ARGS g, m, omega, t, nv, plane, sb[0], sb[kTmaThreads], sb[2 * kTmaThreads], sb[3 * kTmaThreads], \
                 sb[4 * kTmaThreads], sb[5 * kTmaThreads], sb[6 * kTmaThreads], dg, nacc
          if (col == 0) { if (norm) update_vec<0, true, POLES>(UPD_ARGS); else update_vec<0, false, POLES>(UPD_ARGS); }
          else { if (norm) update_vec<1, true, POLES>(UPD_ARGS); else update_vec<1, false, POLES>(UPD_ARGS); }
#undef UPD_ARGS
        }
        ++done_chunks;
        __syncthreads();  // the stage is free again
        if (threadIdx.x == 0 && issued < total) {
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          issue_chunk(m, pl, issued, norm_every, nsweeps, stages, bars);
          ++issued;
        }
      }
    }
    if (!ok) break;
    if (norm) {
      const double sb = block_sum((double)nacc, sh);
      if (threadIdx.x == 0) partials[blockIdx.x] = sb;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) sol->iter += 1;
    if (norm) {
      if (!grid_sync(sol, nb, passed)) { ok = false; break; }
      synced = true;
      const double tot = block_sum_array(partials, nb, sh);
      if (threadIdx.x == 0) stop_sh = norm_stop(sol, tot, stop_ratio, stall_check, last_ratio);
      __syncthreads();
      if (stop_sh) break;
    }
  }
  // copies still in flight (issued for chunks that will not run) land before
  // the block leaves; bounded like every other wait
  __syncthreads();
  for (long long c = done_chunks; c < issued; ++c)
    if (!mbar_wait(bars + (int)(c % kStages), (uint32_t)((c / kStages) & 1), sol)) break;
}

// x += e over the interior of a halo array (natural layout).
static int add_correction(ttfld_ctx* c, double* x) {
  MixWork* w = work(c);
  Dev d = c->d;
  Cmp g = w->g;
  const float* e0 = w->m32.e[0];
  const float* e1 = w->m32.e[1];
  launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) {
    int col = (i + j + k) & 1;
    const float* e = col ? e1 : e0;
    size_t q = hidx(d, i, j, k);
    x[q] = x[q] + (double)e[gslot(g, j - 1, k - 1, (i - 1) >> 1)];
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// The same, queued behind the sweeps before their state is read back: it
// does nothing when they made no progress (SOR_ITER still it0) or met a
// non-finite norm, the cases in which the solve loop leaves x as it is.
static int add_correction_unless(ttfld_ctx* c, double* x, int it0) {
  MixWork* w = work(c);
  Dev d = c->d;
  Cmp g = w->g;
  const float* e0 = w->m32.e[0];
  const float* e1 = w->m32.e[1];
  const SolverDev* sol = c->sol;
  launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) {
    if (sol->iter == it0 || sol->nonfinite) return;
    int col = (i + j + k) & 1;
    const float* e = col ? e1 : e0;
    size_t q = hidx(d, i, j, k);
    x[q] = x[q] + (double)e[gslot(g, j - 1, k - 1, (i - 1) >> 1)];
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// r = b - A x in FP64 (FMA), its L1 norm (fixed-order) and rhat = r/A in FP32.
__global__ void __launch_bounds__(kThreads) resid32_kernel(Dev d, Cmp g, Mix32 m, const double* __restrict__ x,
                                                           const double* __restrict__ b, double* partials) {
  __shared__ double sh[32];
  __shared__ bool last;
  const int nx = d.nx, ny = d.ny;
  const long long n = (long long)nx * ny * sor_zmax(d);  // the rows the SOR solves
  const size_t sj = (size_t)(nx + 4), sk = (size_t)(nx + 4) * (ny + 4);
  double acc = 0.0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int i = (int)(t % nx) + 1;
    long long r = t / nx;
    int j = (int)(r % ny) + 1, k = (int)(r / ny) + 1;
    size_t q = hidx(d, i, j, k);
    size_t qjm = (j == 1) ? hidx(d, i, ny, k) : q - sj;
    size_t qjp = (j == ny) ? hidx(d, i, 1, k) : q + sj;
    double ax = d.SA[t] * x[q];
    ax = fma(d.SB[t], x[q - 1], ax);
    ax = fma(d.SC[t], x[q + 1], ax);
    ax = fma(d.SD[t], x[qjm], ax);
    ax = fma(d.SE[t], x[qjp], ax);
    ax = fma(d.SF[t], x_km(d, x, q, k, sk), ax);
    ax = fma(d.SG[t], x_kp(d, x, q, k, sk), ax);
    double rr = b[t] - ax;
    acc += fabs(rr);
    int col = (i + j + k) & 1;
    size_t s = cslot(g, j - 1, k - 1, (i - 1) >> 1);
    m.rhat[col][s] = __double2float_rn(rr) * m.ainv[col][s];
  }
  double sblk = block_sum(acc, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = sblk;
    __threadfence();
    last = (atomicAdd(&d.sol->ticket2, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    double tot = block_sum_array(partials, gridDim.x, sh);
    if (threadIdx.x == 0) {
      d.sol->true_l1 = tot;
      d.sol->ticket2 = 0;
    }
  }
}

// The FP64 anchor queued: SolverDev::true_l1 holds ||b - A x||_1 once it has
// run (read back with the next poll).
static int resid32_launch(ttfld_ctx* c, const double* x, const double* b) {
  MixWork* w = work(c);
  int nb = grid_for((long long)ncell(c->d));
  if (nb > kMaxPartials) nb = kMaxPartials;
  resid32_kernel<<<nb, kThreads, 0, c->stream>>>(c->d, w->g, w->m32, x, b, c->partials + kMaxPartials);
  count_launches(1);
  TT_CHECK_LAUNCH();
  return 0;
}

static int resid32(ttfld_ctx* c, const double* x, const double* b, double* l1) {
  int rc = resid32_launch(c, x, b);
  if (rc) return rc;
  TT_CHECK(cudaMemcpyAsync(c->host_sol, c->sol, sizeof(SolverDev), cudaMemcpyDeviceToHost, c->stream));
  TT_CHECK(cudaStreamSynchronize(c->stream));
  *l1 = c->host_sol->true_l1;
  return 0;
}

// rhat = b / A: the correction equation of the zero initial guess.
static int rhat_of_b(ttfld_ctx* c, const double* b) {
  MixWork* w = work(c);
  Dev d = c->d;
  Cmp g = w->g;
  Mix32 m = w->m32;
  launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) {
    const int col = (i + j + k) & 1;
    const size_t s = cslot(g, j - 1, k - 1, (i - 1) >> 1);
    m.rhat[col][s] = __double2float_rn(b[cidx(d, i, j, k)]) * m.ainv[col][s];
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// Grid of whole waves: the blocks that fit on the SMs at once (occupancy of
// the kernel), walking the rest of the items by grid stride, so the last
// wave of a short streaming kernel is never a partial one.
template <class K>
static int wave_grid(K kernel, long long items) {
  static int per_wave = 0;
  if (per_wave == 0) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0);
    per_wave = (sms > 0 ? sms : 152) * (per_sm > 0 ? per_sm : 4);
    if (per_wave > kMaxPartials) per_wave = kMaxPartials;
  }
  long long need = (items + kThreads - 1) / kThreads;
  return (int)(need < per_wave ? (need < 1 ? 1 : need) : per_wave);
}

// Blocks of a persistent kernel: all resident at once (cooperative launch),
// at most one wave.  0 if cooperative launch is unavailable.
template <class K>
static int persistent_grid(K kernel, int threads, size_t smem, long long items) {
  int dev = 0, sms = 0, per_sm = 0, coop = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
  long long coresident = coop ? (long long)sms * per_sm : 0;
  if (coresident > kMaxPartials) coresident = kMaxPartials;
  if (coresident <= 0 || items <= 0) return 0;
  const long long need = (items + threads - 1) / threads;
  return (int)(need < coresident ? need : coresident);
}

// sweep_form of ttfld_solve_opts: 0 the neighbour-flag kernel (the product
// form), 1 TMA-staged coefficients, 2 two launches per sweep, 3 the
// wavefront, 4 the grid-barrier kernel.
enum SweepForm { kFormNeighbour = 0, kFormTma = 1, kFormSplit = 2, kFormWave = 3, kFormGrid = 4 };

// Theta planes per window of the wavefront form: the seven windows a pair
// keeps in flight should take at most 60 % of L2 (40 B per cell of the FP32
// system).  g_wave_planes > 0 overrides it (timing runs only).
static int g_wave_planes = 0;
static int wave_planes(const Cmp& g) {
  if (g_wave_planes > 0) return g_wave_planes;
  int dev = 0, l2 = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
  if (l2 <= 0) l2 = 126 << 20;
  const double plane_bytes = 2.0 * g.nxp * g.ny * 40.0;
  int p = (int)(0.6 * l2 / (7.0 * plane_bytes));
  if (p < 1) p = 1;
  if (p > g.nz) p = g.nz;
  return p;
}

// Blocks of the persistent kernels for nvec items (0: not available),
// sized once per grid size and pole form.
struct SweepGrids {
  int pers, tma, wave, local;
};
template <bool POLES>
static SweepGrids sweep_grids(long long nvec) {
  static SweepGrids gr = {-1, -1, -1, -1};
  static long long sized_for = -1;
  if (sized_for != nvec) {
    gr.tma = persistent_grid(sweeps32_tma<POLES>, kTmaThreads, kTmaSmem, nvec);
    gr.pers = persistent_grid(sweeps32_persistent<POLES>, kPersistThreads, 0, nvec);
    gr.wave = nvec < (1LL << 31) ? persistent_grid(sweeps32_wave<POLES>, kPersistThreads, 0, nvec) : 0;
    gr.local = persistent_grid(sweeps32_local<POLES>, kPersistThreads, 0, nvec);
    if (gr.local > kMaxLocalBlocks) gr.local = 0;
    sized_for = nvec;
  }
  return gr;
}
static SweepGrids sweep_grids_of(const Cmp& g) {
  const long long nvec = g.rows * (g.nxp >> 2);
  return g.poles ? sweep_grids<true>(nvec) : sweep_grids<false>(nvec);
}
// The form runs as one launch that stops itself.
static bool one_launch_form(const SweepGrids& gr, SweepForm form) {
  return ((form == kFormNeighbour || form == kFormGrid) && (gr.local > 0 || gr.pers > 0)) ||
         (form == kFormTma && gr.tma > 0) || (form == kFormWave && gr.wave > 0);
}

// Queue nsweeps FP32 sweeps; every norm_every-th one (and the last) also
// evaluates the in-sweep norm against stop_ratio (and, with stall_check,
// stops at the FP32 rounding floor).  The product form is one persistent
// launch of the neighbour-flag kernel; the grid-barrier kernel takes its
// place where the flags do not cover the grid's blocks, and two launches
// per sweep where cooperative launch is unavailable.  The TMA-staged and
// wavefront kernels are kept for comparison: both are slower on this
// workload (per-chunk block barriers and cache latencies of e; a grid
// barrier per wavefront phase).
template <bool POLES>
static int launch_sweeps32_form(ttfld_ctx* c, int nsweeps, int norm_every, double stop_ratio, SweepForm form,
                                bool stall_check) {
  MixWork* w = work(c);
  Cmp g = w->g;
  Mix32 m = w->m32;
  long long nvec = g.rows * (g.nxp >> 2);
  float omega = (float)c->d.sorparam;
  SolverDev* sol = c->sol;
  double* partials = c->partials;
  int stall = stall_check ? 1 : 0;
  void* args[] = {&g, &m, &omega, &sol, &partials, &stop_ratio, &nsweeps, &norm_every, &stall};
  const SweepGrids gr = sweep_grids<POLES>(nvec);
  if (form != kFormSplit)  // the grid barrier counts arrivals from zero
    TT_CHECK(cudaMemsetAsync(&sol->arrivals, 0, sizeof(unsigned long long), c->stream));
  if (form == kFormWave && gr.wave > 0) {
    int planes = wave_planes(g);
    void* wargs[] = {&g, &m, &omega, &sol, &partials, &stop_ratio, &nsweeps, &norm_every, &stall, &planes};
    TT_CHECK(cudaLaunchCooperativeKernel((const void*)sweeps32_wave<POLES>, dim3(gr.wave),
                                         dim3(kPersistThreads), wargs, 0, c->stream));
    count_launches(1);
    return 0;
  }
  if (form == kFormNeighbour && gr.local > 0) {
    unsigned int* flags = w->flags;
    unsigned int base = w->flag_base;
    void* largs[] = {&g, &m, &omega, &sol, &partials, &stop_ratio, &nsweeps, &norm_every, &stall, &flags, &base};
    TT_CHECK(cudaLaunchCooperativeKernel((const void*)sweeps32_local<POLES>, dim3(gr.local),
                                         dim3(kPersistThreads), largs, 0, c->stream));
    w->flag_base = base + 2u * (unsigned int)nsweeps;  // every block leaves its flag there
    count_launches(1);
    return 0;
  }
  if (form == kFormTma && gr.tma > 0) {
    TT_CHECK(cudaLaunchCooperativeKernel((const void*)sweeps32_tma<POLES>, dim3(gr.tma), dim3(kTmaThreads),
                                         args, kTmaSmem, c->stream));
    count_launches(1);
    return 0;
  }
  if (form != kFormSplit && gr.pers > 0) {
    TT_CHECK(cudaLaunchCooperativeKernel((const void*)sweeps32_persistent<POLES>, dim3(gr.pers),
                                         dim3(kPersistThreads), args, 0, c->stream));
    count_launches(1);
    return 0;
  }
  int nb = wave_grid(sweep32_kernel<1, true, POLES>, nvec);
  for (int s = 1; s <= nsweeps; ++s) {
    bool norm = norm_every > 0 && (s % norm_every == 0 || s == nsweeps);
    if (norm) {
      sweep32_kernel<0, true, POLES><<<nb, kThreads, 0, c->stream>>>(g, m, omega, c->sol, c->partials, stop_ratio);
      sweep32_kernel<1, true, POLES><<<nb, kThreads, 0, c->stream>>>(g, m, omega, c->sol, c->partials, stop_ratio);
    } else {
      sweep32_kernel<0, false, POLES><<<nb, kThreads, 0, c->stream>>>(g, m, omega, c->sol, c->partials, stop_ratio);
      sweep32_kernel<1, false, POLES><<<nb, kThreads, 0, c->stream>>>(g, m, omega, c->sol, c->partials, stop_ratio);
    }
  }
  count_launches(2 * nsweeps);
  TT_CHECK_LAUNCH();
  return 0;
}

int launch_sweeps32(ttfld_ctx* c, int nsweeps, int norm_every = 0, double stop_ratio = -1.0,
                    SweepForm form = kFormNeighbour, bool stall_check = true) {
  return work(c)->g.poles ? launch_sweeps32_form<true>(c, nsweeps, norm_every, stop_ratio, form, stall_check)
                          : launch_sweeps32_form<false>(c, nsweeps, norm_every, stop_ratio, form, stall_check);
}

static int poll(ttfld_ctx* c) {
  TT_CHECK(cudaMemcpyAsync(c->host_sol, c->sol, sizeof(SolverDev), cudaMemcpyDeviceToHost, c->stream));
  TT_CHECK(cudaStreamSynchronize(c->stream));
  if (c->host_sol->bar_timeout) {
    fprintf(stderr, "ttfld: a wait of the persistent sweep kernel timed out\n");
    return TTFLD_E_CUDA;
  }
  return 0;
}

// Defect correction: anchor r = b - A x in FP64, run FP32 sweeps on
// A e = r until the in-sweep norm of x + e has dropped by 10^-inner_digits
// (default 1e-4, inside FP32's reach even on the stiff shells) relative to
// the anchor or
// reached tol, x += e, repeat;
// stop when the FP64 ||b - A x||_1 / ||b||_1 <= tol.
//
// With guess_test = n > 0, x holds a previous or learned initial guess that
// must beat the zero guess: n sweeps are run from zero and n from the guess,
// and the in-sweep norm of each n-th sweep (the residual the sweeps before
// it left) decides.  The guess keeps its n sweeps and its residual as the
// first anchor; a rejected guess is replaced by zero (*fallback = 1).
int solve_mixed(ttfld_ctx* c, double* x, const double* b, ttfld_solve_stats* st, int guess_test, int* fallback) {
  int rc;
  if ((rc = ensure32(c)) || (rc = prep32(c))) return rc;
  MixWork* w = work(c);
  const Cmp& g = w->g;
  TT_CHECK(cudaMemsetAsync(c->sol, 0, sizeof(SolverDev), c->stream));
  double bl1 = 0.0, l1 = 0.0;
  // ||b||_1 (SolverDev::rhsnorm, which nothing changes during the solve)
  // comes back with the first readback below
  if ((rc = rhs_norm(c, b, nullptr))) return rc;
  const double tol = c->opts.tol;
  const long long budget = c->opts.max_sweeps > 0 ? c->opts.max_sweeps : (long long)c->d.itmax;
  const int period = 8;
  int corrections = 0, stalls = 0, status = TTFLD_OK;
  double tight = 1.0;  // halved each time the in-sweep norm met tol but the FP64 residual did not
  bool hit_tol = false;
  bool resume = false;  // the first anchor and its first sweeps are done already
  if (fallback) *fallback = 0;
  const SweepForm form = c->opts.sweep_form == 1   ? kFormTma
                         : c->opts.sweep_form == 2 ? kFormSplit
                         : c->opts.sweep_form == 3 ? kFormWave
                         : c->opts.sweep_form == 4 ? kFormGrid
                                                   : kFormNeighbour;
  // one launch per anchor needs a persistent kernel (it stops itself)
  const bool one_launch = one_launch_form(sweep_grids_of(g), form);
  if (guess_test) {
    if ((rc = rhat_of_b(c, b))) return rc;
    TT_CHECK(cudaMemsetAsync(w->m32.e[0], 0, 2 * g.gsz * sizeof(float), c->stream));
    if ((rc = launch_sweeps32(c, guess_test, guess_test, -1.0, form))) return rc;
    // the guess's FP64 residual (and its r-hat) queued behind the sweeps from
    // zero: one readback gives their norm, that residual and ||b||_1
    TT_CHECK(cudaMemsetAsync(&c->sol->iter, 0, sizeof(int), c->stream));
    if ((rc = resid32_launch(c, x, b)) || (rc = poll(c))) return rc;
    const double r_zero = c->host_sol->rnorm;
    l1 = c->host_sol->true_l1;
    bl1 = c->host_sol->rhsnorm;
    if (st) st->guess_resid_l1 = l1;
    TT_CHECK(cudaMemsetAsync(w->m32.e[0], 0, 2 * g.gsz * sizeof(float), c->stream));
    if ((rc = launch_sweeps32(c, guess_test, guess_test, -1.0, form)) || (rc = poll(c))) return rc;
    const double r_guess = c->host_sol->rnorm;
    if (r_guess < r_zero) {
      resume = true;
    } else {
      if (fallback) *fallback = 1;
      TT_CHECK(cudaMemsetAsync(x, 0, nhalo(c->d) * 8, c->stream));
      TT_CHECK(cudaMemsetAsync(&c->sol->iter, 0, sizeof(int), c->stream));
      if ((rc = poll(c))) return rc;
    }
  }
  bool anchor_due = !resume;  // the residual of x is still to be formed
  for (;;) {
    if (anchor_due) {
      if ((rc = resid32(c, x, b, &l1))) return rc;
      bl1 = c->host_sol->rhsnorm;
    }
    anchor_due = false;
    ++corrections;
    if (!isfinite(l1)) { status = TTFLD_E_NONFINITE; break; }
    if (!(l1 > tol * bl1)) break;
    if (hit_tol) tight *= 0.5;
    if (c->host_sol->iter >= budget) { status = TTFLD_MAXITER; break; }
    const double anchor = l1 / bl1;
    const double stop = fmax(tol * tight, anchor * pow(10.0, -c->opts.inner_digits));
    hit_tol = stop <= tol;
    if (!resume) TT_CHECK(cudaMemsetAsync(w->m32.e[0], 0, 2 * g.gsz * sizeof(float), c->stream));  // e[0], e[1] adjacent
    TT_CHECK(cudaMemsetAsync(&c->sol->done, 0, sizeof(int), c->stream));
    resume = false;
    int it0 = c->host_sol->iter;
    double r_prev = anchor;
    int it_prev = it0;
    int chunk = 32;
    bool have_norm = false;  // r_prev is an in-sweep norm (the anchor is a true residual)
    if (one_launch) {
      // the persistent kernel stops itself (target reached, FP32 floor, or
      // the budget), so one launch per anchor suffices; x += e and the next
      // anchor's residual are queued behind it, and one readback returns
      // the sweeps' state and that residual
      const long long left = budget - c->host_sol->iter;
      const int n = (int)(left < (1LL << 24) ? (left > 0 ? left : 1) : (1LL << 24));
      if ((rc = launch_sweeps32(c, n, period, stop, form)) || (rc = add_correction_unless(c, x, it0)) ||
          (rc = resid32_launch(c, x, b)) || (rc = poll(c)))
        return rc;
      if (c->host_sol->nonfinite) status = TTFLD_E_NONFINITE;
      if (c->host_sol->stalled) {
        ++stalls;
        TT_CHECK(cudaMemsetAsync(&c->sol->stalled, 0, sizeof(int), c->stream));
      }
      l1 = c->host_sol->true_l1;
    }
    for (; !one_launch;) {
      if ((rc = launch_sweeps32(c, chunk, chunk <= period ? 1 : period, stop, kFormSplit))) return rc;
      if ((rc = poll(c))) return rc;
      const SolverDev* h = c->host_sol;
      if (h->nonfinite) { status = TTFLD_E_NONFINITE; break; }
      if (h->done || h->iter >= budget) break;
      // the in-sweep norm stopped falling over a whole chunk: the FP32
      // iteration has reached its rounding floor relative to this anchor
      // (stiff, high-contrast systems put it well above 1e-5), so re-anchor
      // in FP64; restarting from e = 0 continues the same iteration
      if (have_norm && h->iter - it_prev >= 16 && !(h->ratio < 0.999 * r_prev)) { ++stalls; break; }
      // predict the sweeps left from the last two norms; queue about that many
      double rate = (h->iter > it_prev && h->ratio > 0.0 && r_prev > 0.0)
                        ? pow(h->ratio / r_prev, 1.0 / (h->iter - it_prev)) : 0.0;
      double left = (rate > 0.0 && rate < 1.0) ? log(stop / h->ratio) / log(rate) : 64.0;
      r_prev = h->ratio;
      it_prev = h->iter;
      have_norm = true;
      if (left <= period) chunk = (int)ceil(left) < 1 ? 1 : (int)ceil(left);
      else if (left < 64) chunk = ((int)left / period) * period;
      else chunk = left < 512 ? ((int)(0.75 * left) / period) * period : 384;
      if (chunk < 1) chunk = 1;
    }
    if (status < 0) break;
    if (c->host_sol->iter == it0) { status = TTFLD_MAXITER; break; }  // no progress possible
    if (!one_launch) {
      if ((rc = add_correction(c, x))) return rc;
      anchor_due = true;
    }
  }
  if ((rc = halo_shift(c, x)) || (rc = pole_shift(c, x))) return rc;
  if (st) {
    st->sor_iter = c->host_sol->iter;
    st->corrections = corrections;
    st->rhsnorm = bl1;
    st->rnorm = l1;
    st->true_resid_l1 = l1;
    st->status = status;
    st->stalls = stalls;
  }
  return status;
}

// ---- fast FP64 path -----------------------------------------------------

// Scaled FP64 coefficients; couplings to non-zero ghost values of x (the
// radial and theta ghosts, fixed during a solve) are folded into bhat.
static int prep64(ttfld_ctx* c, const double* x, const double* b) {
  MixWork* w = work(c);
  Dev d = c->d;
  Cmp g = w->g;
  Fast64 m = w->m64;
  launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) {
    size_t q = cidx(d, i, j, k);
    int col = (i + j + k) & 1;
    size_t s = cslot(g, j - 1, k - 1, (i - 1) >> 1);
    double a = d.SA[q];
    double inv = 1.0 / a;
    double bb = b[q];
    if (i == 1) bb = bb - d.SB[q] * x[hidx(d, 0, j, k)];
    if (i == d.nx) bb = bb - d.SC[q] * x[hidx(d, d.nx + 1, j, k)];
    // with poles the theta ghosts are the mirror, read in the sweep as the
    // cell's own value, and row NZ is not swept: nothing to fold
    if (!d.poles && k == 1) bb = bb - d.SF[q] * x[hidx(d, i, j, 0)];
    if (!d.poles && k == d.nz) bb = bb - d.SG[q] * x[hidx(d, i, j, d.nz + 1)];
    m.a[0][col][s] = d.SB[q] * inv;
    m.a[1][col][s] = d.SC[q] * inv;
    m.a[2][col][s] = d.SD[q] * inv;
    m.a[3][col][s] = d.SE[q] * inv;
    m.a[4][col][s] = d.SF[q] * inv;
    m.a[5][col][s] = d.SG[q] * inv;
    m.bhat[col][s] = bb * inv;
    m.diag[col][s] = a;
    m.x[col][gslot(g, j - 1, k - 1, (i - 1) >> 1)] = x[hidx(d, i, j, k)];
  });
  TT_CHECK_LAUNCH();
  return 0;
}

static int unpack64(ttfld_ctx* c, double* x) {
  MixWork* w = work(c);
  Dev d = c->d;
  Cmp g = w->g;
  Fast64 m = w->m64;
  launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) {
    int col = (i + j + k) & 1;
    x[hidx(d, i, j, k)] = m.x[col][gslot(g, j - 1, k - 1, (i - 1) >> 1)];
  });
  TT_CHECK_LAUNCH();
  return 0;
}

__device__ __forceinline__ double2 ld2(const double* p) { return *reinterpret_cast<const double2*>(p); }
__device__ __forceinline__ void st2(double* p, double2 v) { *reinterpret_cast<double2*>(p) = v; }

// One colour of the FP64 red-black sweep on the scaled system, 2 cells per
// thread: rh = x + sum a_nb x_nb - bhat; resid = A*rh (the reference's
// in-sweep residual, ppsor.f:64-73); x -= omega*rh.  POLES as in
// update_vec: theta rows 1 and NZ-1 take the cell itself across the edge,
// row NZ is not swept.
template <int COL, bool POLES>
__global__ void __launch_bounds__(kThreads) sweep64_kernel(Dev d, Cmp g, Fast64 m, double omega, double* partials,
                                                           int itmin, int itmax, double eps) {
  __shared__ double sh[32];
  __shared__ bool last;
  if (solver_done(d)) return;
  const int nv = g.nxp >> 1;
  const long long n = g.rows * nv;
  const double* __restrict__ xo = m.x[1 - COL];
  double* __restrict__ xs = m.x[COL];
  const size_t plane = (size_t)g.ny * g.nxp;
  double acc = 0.0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int hv = (int)(t % nv);
    const long long rr = t / nv;
    const int j0 = (int)(rr % g.ny), k0 = (int)(rr / g.ny);
    if (POLES && k0 == g.nz - 1) continue;  // zmax_sor_index = NZ-1 (ppsor.f:39-43)
    const int off = (1 + ((j0 + k0) & 1) + COL) & 1;
    const int h0 = hv * 2;
    const int ncol = (g.nx - off + 1) >> 1;
    const size_t cb = (size_t)rr * g.nxp + h0;
    const size_t eb = gslot(g, j0, k0, h0);
    const int jm = j0 == 0 ? g.ny - 1 : j0 - 1;
    const int jp = j0 == g.ny - 1 ? 0 : j0 + 1;
    const double2 o = ld2(xo + eb);
    double xm0, xm1, xp0, xp1;
    if (off == 0) {
      xm0 = h0 > 0 ? xo[eb - 1] : 0.0; xm1 = o.x; xp0 = o.x; xp1 = o.y;
    } else {
      xm0 = o.x; xm1 = o.y; xp0 = o.y; xp1 = (h0 + 2 < g.nxp) ? xo[eb + 2] : 0.0;
    }
    const double2 s = ld2(xo + gslot(g, jm, k0, h0));
    const double2 nn = ld2(xo + gslot(g, jp, k0, h0));
    const double2 xv = ld2(xs + eb);
    const double2 bz = (POLES && k0 == 0) ? xv : ld2(xo + eb - plane);
    const double2 tz = (POLES && k0 == g.nz - 2) ? xv : ld2(xo + eb + plane);
    const double2 aw = ld2(m.a[0][COL] + cb), ae = ld2(m.a[1][COL] + cb);
    const double2 as = ld2(m.a[2][COL] + cb), an = ld2(m.a[3][COL] + cb);
    const double2 ab = ld2(m.a[4][COL] + cb), at = ld2(m.a[5][COL] + cb);
    const double2 bh = ld2(m.bhat[COL] + cb), dg = ld2(m.diag[COL] + cb);
    double2 out;
    {
      double rh = fma(aw.x, xm0, fma(ae.x, xp0, fma(as.x, s.x, fma(an.x, nn.x, fma(ab.x, bz.x, fma(at.x, tz.x, xv.x - bh.x))))));
      bool ok = h0 < ncol;
      acc += ok ? fabs(dg.x * rh) : 0.0;
      out.x = ok ? fma(-omega, rh, xv.x) : 0.0;
    }
    {
      double rh = fma(aw.y, xm1, fma(ae.y, xp1, fma(as.y, s.y, fma(an.y, nn.y, fma(ab.y, bz.y, fma(at.y, tz.y, xv.y - bh.y))))));
      bool ok = h0 + 1 < ncol;
      acc += ok ? fabs(dg.y * rh) : 0.0;
      out.y = ok ? fma(-omega, rh, xv.y) : 0.0;
    }
    st2(xs + eb, out);
  }
  double sb = block_sum(acc, sh);
  if (threadIdx.x == 0) {
    partials[COL * kMaxPartials + blockIdx.x] = sb;
    if (COL == 1) {
      __threadfence();
      last = (atomicAdd(&d.sol->ticket, 1u) == gridDim.x - 1);
    }
  }
  if (COL == 1) {
    __syncthreads();
    if (last) {
      __threadfence();
      finalize_sweep(d, partials, gridDim.x, itmin, itmax, eps, sh);
    }
  }
}

int launch_sweeps64(ttfld_ctx* c, int nsweeps, int itmin, int itmax, double eps) {
  MixWork* w = work(c);
  const Cmp& g = w->g;
  long long nvec = g.rows * (g.nxp >> 1);
  int nb = grid_for(nvec);
  if (nb > kMaxPartials) nb = kMaxPartials;
  double omega = c->d.sorparam;
  for (int s = 0; s < nsweeps; ++s) {
    if (g.poles) {
      sweep64_kernel<0, true><<<nb, kThreads, 0, c->stream>>>(c->d, g, w->m64, omega, c->partials, itmin, itmax, eps);
      sweep64_kernel<1, true><<<nb, kThreads, 0, c->stream>>>(c->d, g, w->m64, omega, c->partials, itmin, itmax, eps);
    } else {
      sweep64_kernel<0, false><<<nb, kThreads, 0, c->stream>>>(c->d, g, w->m64, omega, c->partials, itmin, itmax,
                                                               eps);
      sweep64_kernel<1, false><<<nb, kThreads, 0, c->stream>>>(c->d, g, w->m64, omega, c->partials, itmin, itmax,
                                                               eps);
    }
  }
  count_launches(2 * nsweeps);
  TT_CHECK_LAUNCH();
  return 0;
}

int solve_fast64(ttfld_ctx* c, double* x, const double* b, int itmin, int itmax, ttfld_solve_stats* st) {
  int rc;
  if ((rc = ensure64(c))) return rc;
  MixWork* w = work(c);
  TT_CHECK(cudaMemsetAsync(w->m64.x[0], 0, 2 * w->g.gsz * sizeof(double), c->stream));
  if ((rc = prep64(c, x, b))) return rc;
  TT_CHECK(cudaMemsetAsync(c->sol, 0, sizeof(SolverDev), c->stream));
  if ((rc = rhs_norm(c, b, nullptr))) return rc;
  int chunk = 4, launched = 0;
  for (;;) {
    if ((rc = launch_sweeps64(c, chunk, itmin, itmax, c->d.epsmat))) return rc;
    launched += chunk;
    TT_CHECK(cudaMemcpyAsync(c->host_sol, c->sol, sizeof(SolverDev), cudaMemcpyDeviceToHost, c->stream));
    TT_CHECK(cudaStreamSynchronize(c->stream));
    if (c->host_sol->done) break;
    if (launched >= itmax + 2) return TTFLD_E_CUDA;
    chunk = chunk < 128 ? chunk * 2 : 256;
  }
  if ((rc = unpack64(c, x)) || (rc = halo_shift(c, x)) || (rc = pole_shift(c, x))) return rc;
  int status = c->host_sol->nonfinite ? TTFLD_E_NONFINITE : (c->host_sol->maxit ? TTFLD_MAXITER : TTFLD_OK);
  if (st) {
    st->sor_iter = c->host_sol->iter;
    st->rnorm = c->host_sol->rnorm;
    st->rhsnorm = c->host_sol->rhsnorm;
    st->status = status;
  }
  return status;
}

}  // namespace ttfld

namespace ttfld {
int launch_exact_sweeps(ttfld_ctx* c, double* x, const double* b, int nsweeps, int itmin, int itmax, double eps);

// Mean device time of one full sweep of a solver's kernels (measurement).
int time_sweeps(ttfld_ctx* c, int solver, int n, double* ms) {
  int rc;
  if (n < 1) return TTFLD_E_ARGS;
  TT_CHECK(cudaMemsetAsync(c->sol, 0, sizeof(SolverDev), c->stream));
  if ((rc = rhs_norm(c, c->d.RHS, nullptr))) return rc;
  // TTFLD_SOLVER_MIXED times the solver's kernel (one launch of the
  // neighbour-flag kernel for the n sweeps); 3 the same sweeps as two
  // launches per sweep, 4 as one launch of the TMA-staged persistent kernel,
  // 5 as one launch of the wavefront form with its own window size, 16 + P
  // the wavefront with windows of P theta planes, 6 as one launch of the
  // grid-barrier kernel.  No stall test: all n run.
  const bool wave = solver == 5 || solver >= 16;
  const bool mixed = solver == TTFLD_SOLVER_MIXED || (solver >= 3 && solver <= 6) || wave;
  const SweepForm form = solver == 3   ? kFormSplit
                         : solver == 4 ? kFormTma
                         : solver == 6 ? kFormGrid
                         : wave        ? kFormWave
                                       : kFormNeighbour;
  struct PlanesOverride {  // restored however the timing ends
    PlanesOverride(int p) { g_wave_planes = p; }
    ~PlanesOverride() { g_wave_planes = 0; }
  } planes_override(solver >= 16 ? solver - 16 : 0);
  if (mixed) {
    if ((rc = ensure32(c)) || (rc = prep32(c))) return rc;
    double l1;
    if ((rc = resid32(c, c->d.DELTA_ER, c->d.RHS, &l1))) return rc;
    if ((rc = launch_sweeps32(c, 8, 8, -1.0, form, false))) return rc;  // warm
  } else if (solver == TTFLD_SOLVER_SOR64_FAST) {
    if ((rc = ensure64(c)) || (rc = prep64(c, c->d.DELTA_ER, c->d.RHS))) return rc;
    if ((rc = launch_sweeps64(c, 1, n + 8, n + 8, -1.0))) return rc;
  } else {
    if ((rc = launch_exact_sweeps(c, c->d.DELTA_ER, c->d.RHS, 1, n + 8, n + 8, -1.0))) return rc;
  }
  TT_CHECK(cudaEventRecord(c->ev0, c->stream));
  if (mixed) rc = launch_sweeps32(c, n, 8, -1.0, form, false);
  else if (solver == TTFLD_SOLVER_SOR64_FAST) rc = launch_sweeps64(c, n, n + 8, n + 8, -1.0);
  else rc = launch_exact_sweeps(c, c->d.DELTA_ER, c->d.RHS, n, n + 8, n + 8, -1.0);
  if (rc) return rc;
  TT_CHECK(cudaEventRecord(c->ev1, c->stream));
  TT_CHECK(cudaEventSynchronize(c->ev1));
  float t = 0.f;
  TT_CHECK(cudaEventElapsedTime(&t, c->ev0, c->ev1));
  if ((rc = poll(c))) return rc;
  *ms = (double)t / n;
  return 0;
}
}  // namespace ttfld

extern "C" int ttfld_time_sweeps(ttfld_ctx* c, int solver, int n, double* ms) {
  if (!c || !ms || solver < 0 || (solver > 6 && solver < 17) || solver > 16 + 256) return TTFLD_E_ARGS;
  return ttfld::time_sweeps(c, solver, n, ms);
}
