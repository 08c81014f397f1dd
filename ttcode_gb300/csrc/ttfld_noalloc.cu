// ttfld_noalloc.cu -- ttfld_sor_solve_noalloc: the FP64 red-black SOR solve
// of SOLVE_WITH_SOR on arrays the caller already holds on the device, for
// callers that may not allocate GPU memory at all.
//
// Some hosts own every byte of device memory themselves: a Fortran code
// whose arrays live in an OpenACC/OpenMP-offload data region or in its own
// pool, a job that runs under a fixed memory budget next to other work on
// the same GPU, or a caller that must not let a hidden cudaMalloc/cudaFree
// synchronise the device while its own kernels run.  Such a caller cannot
// create a ttfld context (which allocates its arrays and workspaces).  This
// entry point takes the SOR coefficients, the right-hand side and the
// iterate as device pointers and allocates nothing: the only memory it needs
// beyond them -- the per-row partial sums of the residual norm and the
// loop's bookkeeping -- lives in one file-scope __device__ array of fixed
// size, which every GPU that loads the library holds until the process
// exits.
//
// Limits and sharing rules:
//  * NY*NZ <= kNoAllocMaxRows (131072 rows, e.g. 512 x 256); larger grids are
//    rejected with TTFLD_E_ARGS.  The array takes 2 MiB + 256 B per device.
//  * All calls on a device share the array and it keeps the last call's
//    contents; each call clears the bookkeeping it needs at its start.  Two
//    calls whose GPU work overlaps (different streams or host threads on one
//    device) race on it and must be serialised by the caller.
//  * The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (host code must not use the symbol's name as a
//    device pointer).  The address belongs to the CUDA context the module was loaded in, so it is
//    cached per context, keyed by the context's process-unique id
//    (cuCtxGetId): after cudaDeviceReset, or in a context the caller made
//    itself with the driver API, the first call there looks it up again.
//  * Each call returns once its solve has finished on the GPU (it
//    synchronises its stream to read the stopping flag).
#include <mutex>

#include "ttfld_internal.cuh"

namespace ttfld {
namespace {

constexpr int kNoAllocMaxRows = 131072;
constexpr int kNoAllocMaxContexts = 64;

struct NoAllocState {
  double rhsnorm;
  double rnorm;
  int iter;
  int done;
  int maxit;
  int nonfinite;
  unsigned int ticket;
  int pad[7];
};

struct NoAllocScratch {
  NoAllocState st;                       // 64 B, cleared by every call
  double pad[24];                        // keeps partials 256-B aligned
  double partials[2][kNoAllocMaxRows];   // |resid| summed per (j,k) row and colour
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

std::mutex g_noalloc_mu;
struct ScratchEntry {
  unsigned long long ctx_id;  // 0 = free
  NoAllocScratch* ptr;
};
ScratchEntry g_noalloc_cache[kNoAllocMaxContexts];

// The driver's cuCtxGetCurrent / cuCtxGetId, reached through the runtime so
// the library links only cudart.  Returns the current context's unique id,
// or 0 when there is none yet or the driver does not offer the calls.
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);

unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {  // under g_noalloc_mu
    looked_up = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (CtxGetCurrentFn)p;
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (CtxGetIdFn)p;
    cudaGetLastError();
  }
  if (!get_current || !get_id) return 0;
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

// Device address of the scratch array in the current context: looked up
// with cudaGetSymbolAddress (with the caller's device current) the first
// time a context calls, then taken from the cache.  Without a context id the
// address is looked up on every call.
int noalloc_scratch(NoAllocScratch** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  unsigned long long id = current_context_id();
  if (id) {
    for (const ScratchEntry& e : g_noalloc_cache)
      if (e.ctx_id == id) { *out = e.ptr; return 0; }
  }
  void* p = nullptr;
  TT_CHECK(cudaGetSymbolAddress(&p, g_noalloc_scratch));  // makes the device's context current if none was
  if (!id) id = current_context_id();
  if (id) {
    for (ScratchEntry& e : g_noalloc_cache)
      if (e.ctx_id == 0) { e.ctx_id = id; e.ptr = (NoAllocScratch*)p; break; }
  }
  *out = (NoAllocScratch*)p;
  return 0;
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Last block of a grid: fixed-order sums of the two partial arrays.
__device__ __forceinline__ bool last_block(NoAllocScratch* s, bool* flag) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    *flag = (atomicAdd(&s->st.ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (*flag) __threadfence();
  return *flag;
}

// RHSNORM = sum |b| (ppsor.f:33), one warp per (j,k) row.
__global__ void __launch_bounds__(kThreads) noalloc_rhs_kernel(NoAllocScratch* s, const double* __restrict__ b,
                                                                int nx, int rows) {
  __shared__ double sh[32];
  __shared__ bool last;
  const int warp = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (warp < rows) {
    const double* br = b + (size_t)warp * nx;
    double acc = 0.0;
    for (int i = lane; i < nx; i += 32) acc += fabs(br[i]);
    acc = warp_sum(acc);
    if (lane == 0) s->partials[0][warp] = acc;
  }
  if (last_block(s, &last)) {
    double tot = block_sum_array(s->partials[0], rows, sh);
    if (threadIdx.x == 0) {
      s->st.rhsnorm = tot;
      s->st.ticket = 0;
    }
  }
}

// One colour of the red-black loop (ppsor.f:59-88 / :107-136), one warp per
// (j,k) row, the reference's operand order and no FMA (bitwise the same
// iterate as the serial loop).  x is a halo array; phi wraps (NY even).
template <int COLOUR>
__global__ void __launch_bounds__(kThreads) noalloc_sweep_kernel(
    NoAllocScratch* s, const double* __restrict__ A, const double* __restrict__ B, const double* __restrict__ C,
    const double* __restrict__ D, const double* __restrict__ E, const double* __restrict__ F,
    const double* __restrict__ G, const double* __restrict__ rhs, double* __restrict__ x, int nx, int ny, int nz,
    double omega, int itmin, int itmax, double eps) {
  __shared__ double sh[32];
  __shared__ bool last;
  if (*(volatile int*)&s->st.done) return;
  const int rows = ny * nz;
  const int warp = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  const size_t sj = (size_t)(nx + 4), sk = (size_t)(nx + 4) * (ny + 4);
  if (warp < rows) {
    const int j = warp % ny + 1, k = warp / ny + 1;
    const int imin = 2 - ((j + k + COLOUR) & 1);
    double acc = 0.0;
    for (int i = imin + 2 * lane; i <= nx; i += 64) {
      const size_t c = (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1));
      const size_t q = (size_t)(i + 1) + sj * ((size_t)(j + 1) + (size_t)(ny + 4) * (size_t)(k + 1));
      const size_t qjm = (j == 1) ? q + sj * (size_t)(ny - 1) : q - sj;
      const size_t qjp = (j == ny) ? q - sj * (size_t)(ny - 1) : q + sj;
      const double xc = x[q];
      const double resid = A[c] * xc + B[c] * x[q - 1] + C[c] * x[q + 1] + D[c] * x[qjm] + E[c] * x[qjp] +
                           F[c] * x[q - sk] + G[c] * x[q + sk] - rhs[c];
      acc = acc + fabs(resid);
      x[q] = xc - omega * resid / A[c];
    }
    acc = warp_sum(acc);
    if (lane == 0) s->partials[COLOUR][warp] = acc;
  }
  if (COLOUR == 1 && last_block(s, &last)) {
    double r0 = block_sum_array(s->partials[0], rows, sh);
    double r1 = block_sum_array(s->partials[1], rows, sh);
    if (threadIdx.x == 0) {
      NoAllocState& st = s->st;
      const double rnorm = r0 + r1;
      const int it = st.iter + 1;
      st.iter = it;
      st.rnorm = rnorm;
      const double ratio = rnorm / st.rhsnorm;
      if (!isfinite(rnorm)) { st.nonfinite = 1; st.done = 1; }
      else if (it == itmax) { st.maxit = 1; st.done = 1; }
      else if (!(ratio > eps) && it >= itmin) { st.done = 1; }
      st.ticket = 0;
    }
  }
}

// PLANETSHIFT(8) of the iterate with one rank (ppshift.f:1096-1107, 1164-1173).
__global__ void noalloc_shift_kernel(double* x, int nx, int ny, int nz) {
  const long long n = (long long)(nx + 4) * nz;
  const size_t sj = (size_t)(nx + 4), sk = sj * (ny + 4);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % (nx + 4)) - 1, k = (int)(t / (nx + 4)) + 1;
    double* col = x + (size_t)(i + 1) + sk * (size_t)(k + 1);
    col[sj * 1] = col[sj * (size_t)(ny + 1)];        // j = 0    <- j = NY
    col[0] = col[sj * (size_t)ny];                   // j = -1   <- j = NY-1
    col[sj * (size_t)(ny + 2)] = col[sj * 2];        // j = NY+1 <- j = 1
    col[sj * (size_t)(ny + 3)] = col[sj * 3];        // j = NY+2 <- j = 2
  }
}

}  // namespace
}  // namespace ttfld

using namespace ttfld;

extern "C" int ttfld_sor_solve_noalloc(const double* sor_a, const double* sor_b, const double* sor_c,
                                       const double* sor_d, const double* sor_e, const double* sor_f,
                                       const double* sor_g, const double* rhs, double* x, int nx, int ny, int nz,
                                       double omega, double epsmat, int itmin, int itmax, void* stream,
                                       int* sor_iter, double* rnorm, double* rhsnorm) {
  if (!sor_a || !sor_b || !sor_c || !sor_d || !sor_e || !sor_f || !sor_g || !rhs || !x) return TTFLD_E_ARGS;
  if (nx < 4 || ny < 4 || nz < 4 || (ny % 2) || itmax < 1 || itmin < 0) return TTFLD_E_ARGS;
  if ((long long)ny * nz > kNoAllocMaxRows) {
    fprintf(stderr,
            "ttfld_sor_solve_noalloc: NY*NZ = %lld exceeds the fixed scratch of %d rows; "
            "use ttfld_solve_with_sor on a context for larger grids\n",
            (long long)ny * nz, kNoAllocMaxRows);
    return TTFLD_E_ARGS;
  }
  NoAllocScratch* s = nullptr;
  int rc = noalloc_scratch(&s);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int rows = ny * nz;
  const int blocks = (int)(((long long)rows * 32 + kThreads - 1) / kThreads);
  TT_CHECK(cudaMemsetAsync(&s->st, 0, sizeof(NoAllocState), st));
  noalloc_rhs_kernel<<<blocks, kThreads, 0, st>>>(s, rhs, nx, rows);
  count_launches(1);
  TT_CHECK_LAUNCH();
  NoAllocState h;
  int chunk = 4, launched = 0;
  double ratio_prev = 0.0;
  int iter_prev = 0;
  for (;;) {
    for (int q = 0; q < chunk; ++q) {
      noalloc_sweep_kernel<0><<<blocks, kThreads, 0, st>>>(s, sor_a, sor_b, sor_c, sor_d, sor_e, sor_f, sor_g, rhs, x,
                                                           nx, ny, nz, omega, itmin, itmax, epsmat);
      noalloc_sweep_kernel<1><<<blocks, kThreads, 0, st>>>(s, sor_a, sor_b, sor_c, sor_d, sor_e, sor_f, sor_g, rhs, x,
                                                           nx, ny, nz, omega, itmin, itmax, epsmat);
    }
    count_launches(2 * chunk);
    TT_CHECK_LAUNCH();
    launched += chunk;
    TT_CHECK(cudaMemcpyAsync(&h, &s->st, sizeof(h), cudaMemcpyDeviceToHost, st));
    TT_CHECK(cudaStreamSynchronize(st));
    if (h.done) break;
    // the kernel's stopping rule fires at sweep ITMAX at the latest
    if (launched >= itmax) {
      fprintf(stderr, "ttfld_sor_solve_noalloc: %d sweeps queued without the stopping flag\n", launched);
      return TTFLD_E_INTERNAL;
    }
    // queue about the sweeps the last two norms predict are left (sweeps
    // queued after the stop return at once, but each still costs a launch)
    const double ratio = h.rhsnorm > 0.0 ? h.rnorm / h.rhsnorm : 0.0;
    int next = chunk < 128 ? chunk * 2 : 256;
    if (iter_prev > 0 && h.iter > iter_prev && ratio > 0.0 && ratio < ratio_prev) {
      const double rate = pow(ratio / ratio_prev, 1.0 / (h.iter - iter_prev));
      const double left = log(epsmat / ratio) / log(rate);
      if (left > 0.0 && left < next) next = left < 4.0 ? 4 : (int)ceil(left);
    }
    ratio_prev = ratio;
    iter_prev = h.iter;
    chunk = next < itmax - launched ? next : itmax - launched;
  }
  noalloc_shift_kernel<<<grid_for((long long)(nx + 4) * nz), kThreads, 0, st>>>(x, nx, ny, nz);
  count_launches(1);
  TT_CHECK_LAUNCH();
  TT_CHECK(cudaStreamSynchronize(st));
  if (sor_iter) *sor_iter = h.iter;
  if (rnorm) *rnorm = h.rnorm;
  if (rhsnorm) *rhsnorm = h.rhsnorm;
  if (h.nonfinite) return TTFLD_E_NONFINITE;
  return h.maxit ? TTFLD_MAXITER : TTFLD_OK;
}
