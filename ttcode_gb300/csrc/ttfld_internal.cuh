// ttfld_internal.cuh -- device-side state and helpers shared by the
// libttfld translation units.  All FP64 arithmetic in this library is
// compiled with --fmad=false, so an expression a*b+c is two rounded
// operations exactly as in the reference loops; fused multiply-adds are
// written out explicitly (fma / fmaf) where a kernel wants them.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/ttfld.h"

// global_constants, ppmod.f:1074-1092: REAL*4 literals held in double.
#define TT_FD ((double)2.99792458e10f)
#define TT_ARAD ((double)7.56596e-15f)
#define TT_SBCONST ((double)5.6705e-5f)
#define TT_RGAS ((double)8.315e7f)
#define TT_RSOL ((double)6.9598e10f)

namespace ttfld {

constexpr int kThreads = 256;
constexpr int kMaxPartials = 4096;   // per-colour block partials of a sweep

// Device-side solver bookkeeping (one per context), written by kernels.
struct SolverDev {
  double rhsnorm;      // global_RHSNORM
  double rnorm;        // global_RNORM of the last completed sweep
  double ratio;        // rnorm / rhsnorm
  double true_l1;      // ||b - A x||_1 of the last residual pass
  double scratch[3];
  int iter;            // SOR_ITER
  int done;            // 1 once the stopping rule fired
  int maxit;           // 1 if ITMAX ended the loop
  int nonfinite;       // 1 if a norm was NaN/Inf
  unsigned int ticket; // last-block-done counter
  unsigned int ticket2;
  int bar_timeout;     // 1 if a grid barrier wait ran out (the kernel gave up)
  int stalled;         // 1 if the FP32 inner loop stopped at its rounding floor
  int bad_weights;     // PCG: a row without a valid symmetrising weight
  // arrivals at the grid barrier of the persistent kernels (zeroed by the
  // host before each launch), on a cache line of its own
  alignas(128) unsigned long long arrivals;
};

// Reduction targets of the outer Newton loop.
struct StepDev {
  unsigned long long maxq_bits;   // max |dQ/Q| as IEEE bits (non-negative)
  unsigned long long maxer_bits;  // max |dER/ER|
  int nonpositive_q;              // ppenergy.f:411 guard fired
  int dfq_zero;                   // ppenergy.f:334-340 (eta forced to 0)
  int pad[2];
};

// Every array the step touches, in the reference's Fortran layout.
// 1-D metrics are stored on (-1:N+2) and addressed with G(a, i) = a[i+1].
struct Dev {
  int nx, ny, nz;
  int poles;  // inc_poles: the theta edges are the self-mirrored pole shifts of one rank
  // 1-D grid metrics
  const double *xxa, *xxb, *dxa, *dxb, *xya, *xyb, *dya, *dyb, *xza, *xzb, *dza, *dzb;
  const double *ddx0, *ddx1, *ddy0, *ddy1, *ddz0, *ddz1;
  const double *surxa, *surxb, *surza, *surzb, *geoxg, *geoxh, *geoxga, *geoxha, *geozg, *geozga;
  // halo (-1:NX+2,-1:NY+2,-1:NZ+2)
  double *T, *RH, *CV, *ER, *ER_OLD, *Q, *Q_OLD, *DELTA_ER, *XKAPR, *XKAPP, *XKAPA;
  double *DXKAPP, *DXKAPA, *KMUL, *RHQX, *RHQY, *RHQZ, *STAU, *DTAUS, *SI, *SCALAR;
  // cell (1:NX,1:NY,1:NZ)
  double *E1, *E2, *E3, *E4, *E5, *E6, *E7, *E8, *E16, *ETA, *FQ, *FR, *RHS;
  double *SA, *SB, *SC, *SD, *SE, *SF, *SG, *DIVF, *DIVF_OLD, *DFQ, *DFR, *DQ, *RHS_DIF;
  // face (1:NX+1,1:NY+1,1:NZ+1) internal storage
  double *FLIMX, *FLIMY, *FLIMZ, *DIFRX, *DIFRY, *DIFRZ, *FLUXX, *FLUXY, *FLUXZ;
  // plane (-1:NY+2,-1:NZ+2)
  int* UB;
  double *MU, *TINC;
  // scalars
  double delt, sorparam, epsmat, fbottom, tirr, xnue, pr_num, kap0, sigval;
  int itmax, bcxmin, ibdrad, iflimtyp, f_incident, ieta, isigtyp, iii, kappa_model;
  SolverDev* sol;
  StepDev* stp;
};

__host__ __device__ __forceinline__ size_t hidx(const Dev& d, int i, int j, int k) {
  return (size_t)(i + 1) + (size_t)(d.nx + 4) * ((size_t)(j + 1) + (size_t)(d.ny + 4) * (size_t)(k + 1));
}
__host__ __device__ __forceinline__ size_t cidx(const Dev& d, int i, int j, int k) {
  return (size_t)(i - 1) + (size_t)d.nx * ((size_t)(j - 1) + (size_t)d.ny * (size_t)(k - 1));
}
__host__ __device__ __forceinline__ size_t fidx(const Dev& d, int i, int j, int k) {
  return (size_t)(i - 1) + (size_t)(d.nx + 1) * ((size_t)(j - 1) + (size_t)(d.ny + 1) * (size_t)(k - 1));
}
__host__ __device__ __forceinline__ size_t pidx(const Dev& d, int j, int k) {
  return (size_t)(j + 1) + (size_t)(d.ny + 4) * (size_t)(k + 1);
}
__host__ __device__ __forceinline__ size_t nhalo(const Dev& d) {
  return (size_t)(d.nx + 4) * (d.ny + 4) * (d.nz + 4);
}
__host__ __device__ __forceinline__ size_t ncell(const Dev& d) { return (size_t)d.nx * d.ny * d.nz; }
__host__ __device__ __forceinline__ size_t nface(const Dev& d) {
  return (size_t)(d.nx + 1) * (d.ny + 1) * (d.nz + 1);
}
__host__ __device__ __forceinline__ size_t nplane(const Dev& d) { return (size_t)(d.ny + 4) * (d.nz + 4); }

#define G(a, i) (d.a[(i) + 1])
#define HA(a, i, j, k) (d.a[hidx(d, i, j, k)])
#define CA(a, i, j, k) (d.a[cidx(d, i, j, k)])
#define FA(a, i, j, k) (d.a[fidx(d, i, j, k)])
#define PA(a, j, k) (d.a[pidx(d, j, k)])

__device__ __forceinline__ double p4(double x) { double x2 = x * x; return x2 * x2; }
__device__ __forceinline__ double p3(double x) { return (x * x) * x; }

// An inclusive index box [i0,i1]x[j0,j1]x[k0,k1] walked i fastest.
struct Box {
  int i0, j0, k0, ni, nj, nk;
};
inline Box box(int i0, int i1, int j0, int j1, int k0, int k1) {
  Box b{i0, j0, k0, i1 - i0 + 1, j1 - j0 + 1, k1 - k0 + 1};
  if (b.ni < 0) b.ni = 0;
  if (b.nj < 0) b.nj = 0;
  if (b.nk < 0) b.nk = 0;
  return b;
}

template <class Fn>
__global__ void __launch_bounds__(kThreads) box_kernel(Box b, Fn fn) {
  const long long n = (long long)b.ni * b.nj * b.nk;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    int i = b.i0 + (int)(t % b.ni);
    long long r = t / b.ni;
    int j = b.j0 + (int)(r % b.nj);
    int k = b.k0 + (int)(r / b.nj);
    fn(i, j, k);
  }
}

int grid_for(long long n, int threads = kThreads);
void count_launches(int n);

template <class Fn>
inline void launch_box(cudaStream_t s, Box b, Fn fn) {
  long long n = (long long)b.ni * b.nj * b.nk;
  if (n <= 0) return;
  box_kernel<<<grid_for(n), kThreads, 0, s>>>(b, fn);
  count_launches(1);
}

// Deterministic block sum: every thread passes its value, thread 0 gets the
// block total (fixed shuffle tree, fixed order across warps).
__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    for (int q = 0; q < nw; ++q) t += sh[q];
  }
  __syncthreads();
  return t;
}

// Fixed-order sum of n partials by one block (result valid in thread 0).
__device__ __forceinline__ double block_sum_array(const double* p, int n, double* sh) {
  double v = 0.0;
  for (int q = threadIdx.x; q < n; q += blockDim.x) v += p[q];
  return block_sum(v, sh);
}

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* a, double v) {
  atomicMax(a, (unsigned long long)__double_as_longlong(v));
}

// Grid-wide barrier of the persistent kernels (cooperative launches, so all
// blocks are resident), on a monotonic 64-bit arrival counter that the host
// zeroes before each launch: the k-th barrier of a launch is complete once
// the counter has reached k * nblocks.  Thread 0 of each block releases the
// block's writes (a block barrier, a fence, a release reduction) and polls
// the counter with acquire loads, 32 ns apart, then a fence and a block
// barrier order every thread's later loads after the other blocks' writes.
// With no reset and no generation word, the last block to arrive adds one
// round trip to L2 to the barrier.  `passed` counts this block's barriers
// (the same value in every thread).  The wait is bounded: after
// kBarrierSpins polls (seconds of polling) or once another block has given
// up (tested every kGiveUpPolls polls, so that a poll is one load), the
// block records the timeout and returns false, and the kernel returns
// without further work.
constexpr long long kBarrierSpins = 1LL << 23;
constexpr long long kGiveUpPolls = 256;
__device__ __forceinline__ bool give_up(long long polls, const SolverDev* sol) {
  return polls % kGiveUpPolls == 0 && (polls > kBarrierSpins || *(volatile const int*)&sol->bar_timeout);
}
__device__ __forceinline__ unsigned int ld_acquire(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ bool grid_sync(SolverDev* sol, unsigned int nblocks, unsigned long long& passed) {
  __shared__ int ok_sh;
  __syncthreads();
  ++passed;
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    asm volatile("red.release.gpu.global.add.u64 [%0], 1;" ::"l"(&sol->arrivals) : "memory");
    const unsigned long long target = passed * nblocks;
    long long polls = 0;
    while (ld_acquire64(&sol->arrivals) < target) {
      __nanosleep(32);
      if (give_up(++polls, sol)) {
        atomicExch(&sol->bar_timeout, 1);
        ok = 0;
        break;
      }
    }
    __threadfence();
    ok_sh = ok;
  }
  __syncthreads();
  return ok_sh != 0;
}

__device__ __forceinline__ bool solver_done(const Dev& d) {
  return *(volatile int*)&d.sol->done != 0;
}

// Fixed-order finalisation of one sweep: sum the two colours' partials,
// advance SOR_ITER, apply the stopping rule of ppsor.f:161-177.
__device__ __forceinline__ void finalize_sweep(const Dev& d, const double* partials, int nblk, int itmin, int itmax,
                               double eps, double* sh) {
  double r0 = block_sum_array(partials, nblk, sh);
  double r1 = block_sum_array(partials + kMaxPartials, nblk, sh);
  if (threadIdx.x == 0) {
    double rnorm = r0 + r1;
    SolverDev* s = d.sol;
    int it = s->iter + 1;
    s->iter = it;
    s->rnorm = rnorm;
    double ratio = rnorm / s->rhsnorm;
    s->ratio = ratio;
    if (!isfinite(rnorm)) { s->nonfinite = 1; s->done = 1; }
    else if (it == itmax) { s->maxit = 1; s->done = 1; }
    else if (!(ratio > eps) && it >= itmin) { s->done = 1; }
    s->ticket = 0;
  }
}

}  // namespace ttfld

// Host-side context (the library's one handle per device).
struct ttfld_ctx {
  ttfld::Dev d;              // device pointers + scalars (passed to kernels)
  ttfld_dims dims;
  ttfld_params params;
  ttfld_solve_opts opts;
  int device;
  cudaStream_t stream;
  cudaEvent_t ev0, ev1, evg;
  void* slab;                // one allocation holding every array
  size_t slab_bytes;
  double* staging;           // device staging for box-shaped transfers
  double* partials;          // 2 * kMaxPartials sweep partials
  ttfld::SolverDev* sol;
  ttfld::StepDev* stp;
  ttfld::SolverDev* host_sol;  // pinned mirror
  // mixed-precision workspace (allocated on first use)
  void* mix_slab;
  size_t mix_bytes;
  // learned guess
  void* unet;
  int have_model;
  double prev_scale;        // scale of the previous-solution guess
  int have_prev;
  int solve_idx;            // solves so far in the current step
  double* prev_x;           // previous solution (halo)
  double* guess_tmp;        // scratch halo array of the first-sweep guess test
  void* krylov;             // PCG workspace (allocated on first use)
  void* opac;               // opacity table of kappa_model 2 (device), with its sizes
  int opac_nt, opac_nrh;
  double* divf_tab;         // metric quotients of CALCULATEDIVF_WITHF (allocated on first use)
  int hypre_gs;             // SOLVE_WITH_HYPRE's symmetric line Gauss-Seidel sweeps (0: not yet chosen)
  double* freed;            // Freedman table of kappa_model 3: ross, plnk, abs (42 x 18 each)
  double freed_mu;
  double* wave;             // per-bin opacities (nt x nrh x nbins), then BSTAR_BIN (nbins)
  int wave_nb;
  double wave_rstar, wave_semi;
  double* xkapw;            // per-bin opacities (halo x nbins)
  double* stauw;            // per-bin stellar optical depth (halo x nbins)
  double last_solve_ms;
};

namespace ttfld {
int check_cuda(cudaError_t e, const char* what);
#define TT_CHECK(call)                                   \
  do {                                                   \
    int _rc = ttfld::check_cuda((call), #call);          \
    if (_rc) return _rc;                                 \
  } while (0)
#define TT_CHECK_LAUNCH() TT_CHECK(cudaGetLastError())

// Internal entry points shared across translation units.
int solve_exact64(ttfld_ctx* c, double* x, const double* b, int itmin, int itmax, ttfld_solve_stats* st);
int solve_fast64(ttfld_ctx* c, double* x, const double* b, int itmin, int itmax, ttfld_solve_stats* st);
int solve_mixed(ttfld_ctx* c, double* x, const double* b, ttfld_solve_stats* st, int guess_test = 0,
                int* fallback = nullptr);
int solve_pcg(ttfld_ctx* c, double* x, const double* b, ttfld_solve_stats* st, int guess_test = 0,
              int* fallback = nullptr);
void krylov_free(ttfld_ctx* c);
int fill_sor_matrix(ttfld_ctx* c, bool zero_rhs = true);
int halo_shift(ttfld_ctx* c, double* a);
int pole_shift(ttfld_ctx* c, double* a);

// The last theta row the SOR updates (zmax_sor_index, ppsor.f:39-43): with
// poles the row NZ is the north pole's mirror of NZ-1.
__host__ __device__ __forceinline__ int sor_zmax(const Dev& d) { return d.poles ? d.nz - 1 : d.nz; }
// The theta neighbours of cell (i,j,k) of halo array x at q for the rows the
// SOR updates: with poles the ghost plane 0 holds plane 1 and the plane NZ
// holds NZ-1 (the pole shifts after every colour), which for the cell's own
// column is the cell itself, so its current value is read in their place.
__device__ __forceinline__ double x_km(const Dev& d, const double* x, size_t q, int k, size_t sk) {
  return (d.poles && k == 1) ? x[q] : x[q - sk];
}
__device__ __forceinline__ double x_kp(const Dev& d, const double* x, size_t q, int k, size_t sk) {
  return (d.poles && k == d.nz - 1) ? x[q] : x[q + sk];
}
int rhs_norm(ttfld_ctx* c, const double* b, double* out_host);
int true_residual(ttfld_ctx* c, const double* x, const double* b, double* l1);
int unet_guess(ttfld_ctx* c, double* x_out, double* resid_l1);
void asm_free(ttfld_ctx* c);

// The metric quotients of CALCULATEDIVF_WITHF (ppenergy.f:853-867), formed
// once per context: ax1/ax0 per i, az1/az0 per (i,k), ay per cell.
struct DivfTab {
  double *ax1, *ax0, *az1, *az0, *ay;
};
DivfTab divf_tab(ttfld_ctx* c);

// FILL_EVALUES ppenergy.f:984-1030 for one cell, given its eta.
struct EvalRow {
  double e1, e2, e3, e4, e5, e6, e7, e8, e16;
};
__device__ __forceinline__ EvalRow evalues_cell(const Dev& d, int i, int j, int k, double theta, double eta) {
  EvalRow r;
  r.e1 = -G(surxa, i + 1) * FA(DIFRX, i + 1, j, k) / (G(surxb, i) * G(dxa, i));
  r.e2 = -G(surxa, i) * FA(DIFRX, i, j, k) / (G(surxb, i) * G(dxa, i));
  r.e3 = -FA(DIFRY, i, j + 1, k) / (G(xxb, i) * G(surzb, k) * G(dya, j));
  r.e4 = -FA(DIFRY, i, j, k) / (G(xxb, i) * G(surzb, k) * G(dya, j));
  r.e5 = -FA(DIFRZ, i, j, k + 1) * G(surza, k + 1) / (G(xxb, i) * G(surzb, k) * G(dza, k));
  r.e6 = -FA(DIFRZ, i, j, k) * G(surza, k) / (G(xxb, i) * G(surzb, k) * G(dza, k));
  r.e7 = 1.0 + (1.0 - eta) * d.delt * HA(RH, i, j, k) * HA(XKAPP, i, j, k) * TT_FD;
  r.e8 = (eta * (1.0 - theta) - 1.0) * d.delt;
  r.e16 = r.e1 + r.e2 + r.e3 + r.e4 + r.e5 + r.e6;
  return r;
}
__device__ __forceinline__ void store_evalues(const Dev& d, size_t q, const EvalRow& r) {
  d.E1[q] = r.e1; d.E2[q] = r.e2; d.E3[q] = r.e3; d.E4[q] = r.e4; d.E5[q] = r.e5; d.E6[q] = r.e6;
  d.E7[q] = r.e7; d.E8[q] = r.e8; d.E16[q] = r.e16;
}

// FILL_SOR_MATRIX ppsor.f:189-277 for one cell from its EVAL values, with
// B_VECTOR_BOUNDARIES (ppsor.f:280-329): returns true for the identity rows
// whose right-hand side is zero.
__device__ __forceinline__ bool sor_row(const Dev& d, int i, int j, int k, size_t q, const EvalRow& r) {
  double e8 = r.e8;
  double a = r.e7 + e8 * r.e16;
  double b = -e8 * r.e2, cc = -e8 * r.e1, dd = -e8 * r.e4;
  double e = -e8 * r.e3, f = -e8 * r.e6, g = -e8 * r.e5;
  int ub = PA(UB, j, k);
  // the theta edges are boundary rows only without poles (ppsor.f:228-272)
  bool ident = (i >= ub) || (i == d.nx) || (!d.poles && (k == 1 || k == d.nz));
  if (ident) { a = 1.0; b = 0.0; cc = 0.0; dd = 0.0; e = 0.0; f = 0.0; g = 0.0; }
  if (i == ub - 1) cc = 0.0;
  if (i == d.nx - 1) cc = 0.0;
  if (!d.poles && k == 2) f = 0.0;
  if (!d.poles && k == d.nz - 1) g = 0.0;
  d.SA[q] = a; d.SB[q] = b; d.SC[q] = cc; d.SD[q] = dd; d.SE[q] = e; d.SF[q] = f; d.SG[q] = g;
  return ident;
}

// The divergence of the fluxes of cell (i,j,k), in the reference's operand
// order with its metric quotients read from the table.
__device__ __forceinline__ double divf_cell(const Dev& d, const DivfTab& t, int i, int j, int k) {
  const size_t ik = (size_t)(i - 1) + (size_t)d.nx * (k - 1);
  const double ay = t.ay[cidx(d, i, j, k)];
  return ((t.ax1[i - 1] * FA(FLUXX, i + 1, j, k) - t.ax0[i - 1] * FA(FLUXX, i, j, k)) +
          (ay * FA(FLUXY, i, j + 1, k) - ay * FA(FLUXY, i, j, k))) +
         (t.az1[ik] * FA(FLUXZ, i, j, k + 1) - t.az0[ik] * FA(FLUXZ, i, j, k));
}
int unet_capture(ttfld_ctx* c);
void unet_free(ttfld_ctx* c);
}  // namespace ttfld
