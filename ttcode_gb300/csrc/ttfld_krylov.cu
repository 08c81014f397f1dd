// ttfld_krylov.cu -- preconditioned conjugate gradients on the FLD system.
//
//  * ttfld_solve_with_hypre: the IRAD=2 path's SOLVE_WITH_HYPRE
//    (pphypre.f:1-111).  Its system is FILLHYPREMATRIX / FILLHYPREVECTORS
//    (pphypre.f:115-334): SOLVE_WITH_SOR's 7-point matrix (ppsor.f:202-272)
//    with the i = 1 rows made identity rows (pphypre.f:281-294), the west
//    coupling of the i = 2 rows removed (pphypre.f:298-300) and b zero on the
//    same boundary rows (pphypre.f:137-205).  hypre solves it by PCG from
//    x = 1 (pphypre.f:136) to a relative residual of 1e-6 in at most 50
//    iterations (pphypre.f:45-55), preconditioned by one SMG cycle.  Here
//    the same PCG runs on the device with a radial line preconditioner.
//  * TTFLD_SOLVER_PCG: SOLVE_WITH_SOR's own system solved by the same PCG,
//    stopped like the mixed solver on ||b - A x||_1 / ||b||_1 <= tol.
//
// Symmetric form.  Row n of the matrix is (EVAL7 + EVAL8 EVAL_1_6) x_n -
// EVAL8 sum_m EVALm x_m, and each EVALm is a face coefficient shared by the
// two cells of the face divided by the metric factor of cell n
// (ppenergy.f:995-1013).  Multiplied by W_n = V_n / |EVAL8_n| with
// V = surxb dxa dya surzb dza, the rows form a symmetric matrix (the
// identity rows are decoupled and get W = V).  PCG runs on
// S = Sigma sym(W A) Sigma, Sigma = diag(1 / sqrt(W_n A_nn)), which has a
// unit diagonal; sym() is the symmetric part, which differs from W A only
// where the two cells of a face were given different face coefficients (the
// phi seam of the periodic halo).  An FP64 defect correction on the rows as
// they are (r = b - A x, x += Sigma e) removes that difference and the FP32
// rounding of the inner iteration:
//
//   loop: r = b - A x (FP64); stop test; solve S e = Sigma W r by FP32 PCG
//         to a relative reduction of its preconditioned residual norm; x += Sigma e.
//
// Preconditioner.  The radial couplings dominate by two to three orders of
// magnitude (the shell is thin in r), so the preconditioner is built on the
// exact solve of the tridiagonal radial line of a (j,k) column, factored
// once per solve (Thomas algorithm, FP32 pivots): TTFLD_SOLVER_PCG applies
// it to every column (block Jacobi); SOLVE_WITH_HYPRE, whose caller bounds
// the iterations at hypre's 50, applies one symmetric red-black line
// Gauss-Seidel sweep (half the iterations, three times the cost of one).
//
// Layout.  The FP32 inner arrays are line-major, q = (i-1)*NY*NZ +
// (k-1)*NY + (j-1): in a line solve one thread walks one column and the
// threads of a warp touch 32 consecutive columns of the same radius
// (coalesced); in the operator pass the phi and theta neighbours are at q
// +- 1 and q +- NY.  The inner iteration is one persistent cooperative
// kernel with two grid barriers per iteration (after s = S p for alpha,
// after the line solve for beta).
#include <math.h>
#include <stdlib.h>

#include "ttfld_internal.cuh"

namespace ttfld {
namespace {

constexpr int kPcgThreads = 256;   // one block per SM; 248 registers for the batched passes
constexpr int kPcgStall = 25;      // iterations without a new minimum of r.z end an inner run
constexpr double kInnerReduce = 1e-4;  // relative reduction of sqrt(r.z) asked of one inner run
constexpr int kMaxGsSweeps = 32;       // symmetric line Gauss-Seidel sweeps per preconditioner application

struct Kry {
  int nx, ny, nz;
  long long n, ncol;
  // couplings of S to the +i, +j (periodic) and +k neighbour, and the
  // reciprocal pivots of the radial line factorisation (line-major, FP32)
  float *cr, *cp, *ct, *g;
  float *e, *r, *z, *s, *p[2];
  double *sig, *wgt;  // Sigma_n and W_n (cell order, FP64)
};

struct KryWork {
  Kry k;
  void* mem;
};

__host__ __device__ __forceinline__ size_t lq(const Kry& k, int i, int j, int kk) {
  return (size_t)(i - 1) * k.ncol + (size_t)(kk - 1) * k.ny + (size_t)(j - 1);
}

// The rows of the system being solved: SOR_A..G, with the hypre changes.
struct Row {
  double a, b, c, d, e, f, g;
};
// hypre's grid has only its extents (pphypre.f:404-413, no periodicity), so
// the j-1 entry of rows j = 1 and the j+1 entry of rows j = NY reach outside
// it and are dropped.  With poles (SOLVE_WITH_SOR's system only): the theta
// neighbour across either edge is the cell itself (the mirror the pole
// shifts keep), so rows 1 and NZ-1 take that coupling into their diagonal,
// and row NZ, which the SOR does not solve (ppsor.f:39-43) and the pole
// shift overwrites, is a decoupled identity row.  Both keep the symmetric
// form: the couplings between rows 1 and 2, NZ-2 and NZ-1 are unchanged.
__device__ __forceinline__ Row row_of(const Dev& d, size_t t, int i, int j, int k, bool hypre) {
  Row r{d.SA[t], d.SB[t], d.SC[t], d.SD[t], d.SE[t], d.SF[t], d.SG[t]};
  if (hypre) {
    if (i == 1) r = Row{1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};  // pphypre.f:281-294
    else if (i == 2) r.b = 0.0;                               // pphypre.f:298-300
    if (j == 1) r.d = 0.0;
    if (j == d.ny) r.e = 0.0;
  } else if (d.poles) {
    if (k == d.nz) return Row{1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (k == 1) { r.a += r.f; r.f = 0.0; }
    if (k == d.nz - 1) { r.a += r.g; r.g = 0.0; }
  }
  return r;
}

// b of the hypre system (pphypre.f:137-205): zero at i >= upperbnd, i = 1,
// i = NX, k = 1 and k = NZ; with poles, of SOLVE_WITH_SOR's system zero on
// the identity row NZ.
__device__ __forceinline__ double b_of(const Dev& d, const double* b, size_t t, int i, int j, int k, bool hypre) {
  if (hypre && (i >= PA(UB, j, k) || i == 1 || i == d.nx || k == 1 || k == d.nz)) return 0.0;
  if (!hypre && d.poles && k == d.nz) return 0.0;
  return b[t];
}

__device__ __forceinline__ void cell_of(const Dev& d, long long t, int& i, int& j, int& k) {
  i = (int)(t % d.nx) + 1;
  const long long r = t / d.nx;
  j = (int)(r % d.ny) + 1;
  k = (int)(r / d.ny) + 1;
}

// W_n and Sigma_n (cell order).  A coupled row needs EVAL8 < 0.
__global__ void __launch_bounds__(kThreads) kry_weights_kernel(Dev d, Kry kr, int hypre) {
  const long long n = (long long)ncell(d);
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_of(d, t, i, j, k);
    const Row r = row_of(d, t, i, j, k, hypre != 0);
    const bool decoupled = r.b == 0.0 && r.c == 0.0 && r.d == 0.0 && r.e == 0.0 && r.f == 0.0 && r.g == 0.0;
    const double v = G(surxb, i) * G(dxa, i) * G(dya, j) * G(surzb, k) * G(dza, k);
    const double e8 = d.E8[t];
    const double w = decoupled ? v : v / (-e8);
    const double dd = w * r.a;
    bool ok = (decoupled || e8 < 0.0) && dd > 0.0 && isfinite(dd);
    kr.wgt[t] = ok ? w : 0.0;
    kr.sig[t] = ok ? rsqrt(dd) : 0.0;  // any positive scaling serves; it is used consistently
    if (!ok) atomicExch(&d.sol->bad_weights, 1);
  }
}

// Couplings of S (the symmetric part of Sigma W A Sigma) to the +i, +j, +k
// neighbours, written line-major.
__global__ void __launch_bounds__(kThreads) kry_couplings_kernel(Dev d, Kry kr, int hypre) {
  const long long n = (long long)ncell(d);
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_of(d, t, i, j, k);
    const bool h = hypre != 0;
    const Row r = row_of(d, t, i, j, k, h);
    const double wn = kr.wgt[t], sn = kr.sig[t];
    float cr = 0.f, cp = 0.f, ct = 0.f;
    if (i < nx) {
      const size_t m = t + 1;
      const Row rm = row_of(d, m, i + 1, j, k, h);
      cr = (float)(0.5 * (wn * r.c + kr.wgt[m] * rm.b) * sn * kr.sig[m]);
    }
    {
      const int jp = j == ny ? 1 : j + 1;
      const size_t m = cidx(d, i, jp, k);
      const Row rm = row_of(d, m, i, jp, k, h);
      cp = (float)(0.5 * (wn * r.e + kr.wgt[m] * rm.d) * sn * kr.sig[m]);
    }
    if (k < nz) {
      const size_t m = cidx(d, i, j, k + 1);
      const Row rm = row_of(d, m, i, j, k + 1, h);
      ct = (float)(0.5 * (wn * r.g + kr.wgt[m] * rm.f) * sn * kr.sig[m]);
    }
    const size_t q = lq(kr, i, j, k);
    kr.cr[q] = cr;
    kr.cp[q] = cp;
    kr.ct[q] = ct;
  }
}

// Reciprocal pivots of every radial line (diagonal 1, off-diagonal cr):
// u_1 = 1, u_i = 1 - cr_{i-1}^2 / u_{i-1}; g = 1/u.  One thread per column;
// FP32 (the factorisation only preconditions).
__global__ void __launch_bounds__(kThreads) kry_factor_kernel(Kry kr, SolverDev* sol) {
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < kr.ncol;
       c += (long long)gridDim.x * blockDim.x) {
    float g = 1.f, cprev = 0.f;
    size_t q = (size_t)c;
    for (int i = 0; i < kr.nx; ++i, q += kr.ncol) {
      const float u = fmaf(-cprev * cprev, g, 1.f);
      if (!(u > 0.f)) atomicExch(&sol->bad_weights, 1);
      g = 1.f / u;
      kr.g[q] = g;
      cprev = kr.cr[q];
    }
  }
}

// FP64 anchor: r = b - A x, its L1 norm, the scaled right-hand side
// Sigma W r of the inner system (FP32, line-major) and, with L2, its
// squared 2-norm; with WITH_B also ||b||_1 and ||Sigma W b||_2^2 (b does not
// change during a solve).  The last block writes the totals to
// sol->true_l1, sol->scratch[0], sol->rhsnorm, sol->scratch[1].  The
// residual is a chain of FP64 fused multiply-adds: GB300's FP64 pipe, not
// HBM, bounds this kernel.
template <bool L2, bool WITH_B>
__global__ void __launch_bounds__(kThreads) kry_anchor_kernel(Dev d, Kry kr, const double* __restrict__ x,
                                                              const double* __restrict__ b, int hypre,
                                                              double* partials, int nbmax) {
  __shared__ double sh[32];
  __shared__ bool last;
  const int nx = d.nx, ny = d.ny;
  const long long n = (long long)ncell(d);
  const size_t sj = (size_t)(nx + 4), sk = (size_t)(nx + 4) * (ny + 4);
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_of(d, t, i, j, k);
    const Row r = row_of(d, t, i, j, k, hypre != 0);
    const size_t q = hidx(d, i, j, k);
    const size_t qjm = (j == 1) ? hidx(d, i, ny, k) : q - sj;
    const size_t qjp = (j == ny) ? hidx(d, i, 1, k) : q + sj;
    const double bb = b_of(d, b, t, i, j, k, hypre != 0);
    // a zero coupling contributes nothing, whatever the ghost it points at holds
    double ax = r.a * x[q];
    ax = fma(r.b, r.b != 0.0 ? x[q - 1] : 0.0, ax);
    ax = fma(r.c, r.c != 0.0 ? x[q + 1] : 0.0, ax);
    ax = fma(r.d, r.d != 0.0 ? x[qjm] : 0.0, ax);
    ax = fma(r.e, r.e != 0.0 ? x[qjp] : 0.0, ax);
    ax = fma(r.f, r.f != 0.0 ? x[q - sk] : 0.0, ax);
    ax = fma(r.g, r.g != 0.0 ? x[q + sk] : 0.0, ax);
    const double rr = bb - ax;
    const double sw = kr.sig[t] * kr.wgt[t];
    const double rs = sw * rr;
    s[0] += fabs(rr);
    if (L2) s[1] = fma(rs, rs, s[1]);
    if (WITH_B) {
      const double bs = sw * bb;
      s[2] += fabs(hypre ? bb : b[t]);  // RHSNORM over every row (ppsor.f:33)
      s[3] = fma(bs, bs, s[3]);
    }
    const size_t l = lq(kr, i, j, k);
    kr.r[l] = (float)rs;
    kr.e[l] = 0.f;
  }
  for (int m = 0; m < 4; ++m) {
    const double v = block_sum(s[m], sh);
    if (threadIdx.x == 0) partials[m * nbmax + blockIdx.x] = v;
  }
  if (threadIdx.x == 0) {
    __threadfence();
    last = (atomicAdd(&d.sol->ticket2, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    double tot[4];
    for (int m = 0; m < 4; ++m) tot[m] = block_sum_array(partials + m * nbmax, gridDim.x, sh);
    if (threadIdx.x == 0) {
      d.sol->true_l1 = tot[0];
      if (L2) d.sol->scratch[0] = tot[1];
      if (WITH_B) {
        d.sol->rhsnorm = tot[2];
        d.sol->scratch[1] = tot[3];
      }
      d.sol->ticket2 = 0;
    }
  }
}

// x += Sigma e (x a halo array, e line-major).
__global__ void __launch_bounds__(kThreads) kry_update_kernel(Dev d, Kry kr, double* x) {
  const long long n = (long long)ncell(d);
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_of(d, t, i, j, k);
    x[hidx(d, i, j, k)] += kr.sig[t] * (double)kr.e[lq(kr, i, j, k)];
  }
}

// One radial line of the inner iteration for column c.  With UPDATE, first
// r -= alpha s along the line.  Then z = T^-1 r by the factored tridiagonal
// T (forward: y_i = r_i - cr_{i-1} g_{i-1} y_{i-1}, kept in z; backward:
// z_i = (y_i - cr_i z_{i+1}) g_i).  Returns this line's share of r.z.  The
// loads of kLineBatch radii are issued before any of their stores (the
// compiler may not move a load above a store it cannot prove independent,
// and a warp stalls at the first use of a pending load), so a pass waits
// one memory latency per batch, not per radius.
constexpr int kLineBatch = 16;
template <bool UPDATE>
__device__ __forceinline__ float line_pass(const Kry& k, long long c, float alpha) {
  constexpr int U = kLineBatch;
  // 32-bit offsets (a context holds fewer than 2^31 cells per array)
  const unsigned int ncol = (unsigned int)k.ncol;
  const unsigned int c0 = (unsigned int)c;
  const int nx = k.nx;
  float yprev = 0.f, lprev = 0.f;
  for (int i0 = 0; i0 < nx; i0 += U) {
    const unsigned int qb = c0 + (unsigned int)i0 * ncol;
    float rr[U], cc[U], gg[U], ss[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (i0 + u < nx) {
        const unsigned int q = qb + (unsigned int)u * ncol;
        rr[u] = k.r[q];
        cc[u] = k.cr[q];
        gg[u] = k.g[q];
        if (UPDATE) ss[u] = k.s[q];
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (i0 + u < nx) {
        const unsigned int q = qb + (unsigned int)u * ncol;
        float ri = rr[u];
        if (UPDATE) {
          ri = fmaf(-alpha, ss[u], ri);
          k.r[q] = ri;
        }
        const float y = fmaf(-lprev, yprev, ri);
        k.z[q] = y;
        lprev = cc[u] * gg[u];
        yprev = y;
      }
    }
  }
  float dot = 0.f;
  float znext = 0.f;
  for (int i1 = nx - 1; i1 >= 0; i1 -= U) {
    const unsigned int qb = c0 + (unsigned int)i1 * ncol;
    float yy[U], cc[U], gg[U], rr[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (i1 - u >= 0) {
        const unsigned int q = qb - (unsigned int)u * ncol;
        yy[u] = k.z[q];
        cc[u] = k.cr[q];
        gg[u] = k.g[q];
        rr[u] = k.r[q];
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (i1 - u >= 0) {
        const unsigned int q = qb - (unsigned int)u * ncol;
        const float zi = fmaf(-cc[u], znext, yy[u]) * gg[u];
        k.z[q] = zi;
        znext = zi;
        dot = fmaf(rr[u], zi, dot);
      }
    }
  }
  return dot;
}

// One radial line of the red-black line Gauss-Seidel preconditioner for
// column c (j0, k0): with UPDATE first r -= alpha s; then
// z = T^-1 (r - the couplings to the four phi/theta neighbour columns, which
// all have the other colour, times their z).  Returns r.z of the line.
constexpr int kGsBatch = 4;
template <bool UPDATE>
__device__ __forceinline__ float line_gs(const Kry& k, long long c, float alpha) {
  constexpr int U = kGsBatch;
  const unsigned int ncol = (unsigned int)k.ncol;
  const int nx = k.nx, ny = k.ny;
  const int j0 = (int)(c % ny), k0 = (int)(c / ny);
  const unsigned int c0 = (unsigned int)c;
  // neighbour columns (theta neighbours outside the grid read column c with a zero coupling)
  const unsigned int cjp = j0 == ny - 1 ? c0 - (ny - 1) : c0 + 1;
  const unsigned int cjm = j0 == 0 ? c0 + (ny - 1) : c0 - 1;
  const bool hkp = k0 + 1 < k.nz, hkm = k0 > 0;
  const unsigned int ckp = hkp ? c0 + ny : c0, ckm = hkm ? c0 - ny : c0;
  float yprev = 0.f, lprev = 0.f;
  for (int i0 = 0; i0 < nx; i0 += U) {
    const unsigned int qb = (unsigned int)i0 * ncol;
    float rr[U], ss[U], cc[U], gg[U], nb[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (i0 + u < nx) {
        const unsigned int o = qb + (unsigned int)u * ncol;
        rr[u] = k.r[o + c0];
        if (UPDATE) ss[u] = k.s[o + c0];
        cc[u] = k.cr[o + c0];
        gg[u] = k.g[o + c0];
        const float ctm = hkm ? k.ct[o + ckm] : 0.f;
        nb[u] = fmaf(k.cp[o + c0], k.z[o + cjp],
                fmaf(k.cp[o + cjm], k.z[o + cjm], fmaf(k.ct[o + c0], k.z[o + ckp], ctm * k.z[o + ckm])));
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (i0 + u < nx) {
        const unsigned int q = qb + (unsigned int)u * ncol + c0;
        float ri = rr[u];
        if (UPDATE) {
          ri = fmaf(-alpha, ss[u], ri);
          k.r[q] = ri;
        }
        const float y = fmaf(-lprev, yprev, ri - nb[u]);
        k.z[q] = y;
        lprev = cc[u] * gg[u];
        yprev = y;
      }
    }
  }
  float dot = 0.f, znext = 0.f;
  for (int i1 = nx - 1; i1 >= 0; i1 -= U) {
    const unsigned int qb = c0 + (unsigned int)i1 * ncol;
    float yy[U], cc[U], gg[U], rr[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (i1 - u >= 0) {
        const unsigned int q = qb - (unsigned int)u * ncol;
        yy[u] = k.z[q];
        cc[u] = k.cr[q];
        gg[u] = k.g[q];
        rr[u] = k.r[q];
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (i1 - u >= 0) {
        const unsigned int q = qb - (unsigned int)u * ncol;
        const float zi = fmaf(-cc[u], znext, yy[u]) * gg[u];
        k.z[q] = zi;
        znext = zi;
        dot = fmaf(rr[u], zi, dot);
      }
    }
  }
  return dot;
}

// Column m of colour C (0: (j+k) even, 1: odd) in the red-black order of
// the columns; NY is even, so each theta row holds NY/2 of each colour.
__device__ __forceinline__ long long col_of(long long m, int C, int ny) {
  const long long half = ny >> 1;
  const long long k0 = m / half;
  const long long jj = m - k0 * half;
  return k0 * ny + 2 * jj + ((k0 + C) & 1);
}

__device__ __forceinline__ float4 ldf4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void stf4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float4 axpy4(float a, float4 x, float4 y) {
  return make_float4(fmaf(a, x.x, y.x), fmaf(a, x.y, y.y), fmaf(a, x.z, y.z), fmaf(a, x.w, y.w));
}
__device__ __forceinline__ float4 fma4(float4 a, float4 b, float4 c) {
  return make_float4(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y), fmaf(a.z, b.z, c.z), fmaf(a.w, b.w, c.w));
}
__device__ __forceinline__ float4 keep4(bool on, float4 v) { return on ? v : make_float4(0.f, 0.f, 0.f, 0.f); }

// The operator pass on four cells q..q+3 of one phi row (NY a multiple of
// four, q a multiple of four): e += alpha_prev p_old (the previous
// iteration's update of e, deferred to here so that the line pass reads
// fewer arrays), p_new = z + beta p_old, s = S p_new; returns p_new . s.
// Every load is issued before the first arithmetic (neighbours that do not
// exist are read at q and their couplings zeroed), so the quad waits one
// memory latency.
__device__ __forceinline__ float op_quad(const Kry& k, const float* po, float* pn, float beta, float alpha_prev,
                                         long long q) {
  const long long ncol = k.ncol;
  const int ny = k.ny;
  const long long il = q / ncol;
  const long long cc = q - il * ncol;
  const int j0 = (int)(cc % ny);
  const long long k0 = cc / ny;
  const bool hn = il + 1 < k.nx, hs = il > 0, ht = k0 + 1 < k.nz, hb = k0 > 0;
  const long long qn = hn ? q + ncol : q, qs = hs ? q - ncol : q;
  const long long qt = ht ? q + ny : q, qb = hb ? q - ny : q;
  const long long qm = j0 == 0 ? q + ny - 1 : q - 1;   // phi neighbours (periodic)
  const long long qp = j0 + 4 == ny ? q + 4 - ny : q + 4;
  const float4 zc = ldf4(k.z + q), oc = ldf4(po + q), ec = ldf4(k.e + q);
  const float4 zn = ldf4(k.z + qn), on = ldf4(po + qn), zs = ldf4(k.z + qs), os = ldf4(po + qs);
  const float4 zt = ldf4(k.z + qt), ot = ldf4(po + qt), zb = ldf4(k.z + qb), ob = ldf4(po + qb);
  const float4 crn = ldf4(k.cr + q), crs = ldf4(k.cr + qs), ctt = ldf4(k.ct + q), ctb = ldf4(k.ct + qb);
  const float4 cp = ldf4(k.cp + q);
  const float zm = k.z[qm], om = po[qm], zp = k.z[qp], op = po[qp], cl = k.cp[qm];
  stf4(k.e + q, axpy4(alpha_prev, oc, ec));
  const float4 pc = axpy4(beta, oc, zc);
  float4 sv = pc;
  sv = fma4(keep4(hn, crn), axpy4(beta, on, zn), sv);
  sv = fma4(keep4(hs, crs), axpy4(beta, os, zs), sv);
  sv = fma4(keep4(ht, ctt), axpy4(beta, ot, zt), sv);
  sv = fma4(keep4(hb, ctb), axpy4(beta, ob, zb), sv);
  const float pl = fmaf(beta, om, zm), pr = fmaf(beta, op, zp);
  sv.x = fmaf(cp.x, pc.y, fmaf(cl, pl, sv.x));
  sv.y = fmaf(cp.y, pc.z, fmaf(cp.x, pc.x, sv.y));
  sv.z = fmaf(cp.z, pc.w, fmaf(cp.y, pc.y, sv.z));
  sv.w = fmaf(cp.w, pr, fmaf(cp.z, pc.z, sv.w));
  stf4(pn + q, pc);
  stf4(k.s + q, sv);
  return fmaf(pc.x, sv.x, fmaf(pc.y, sv.y, fmaf(pc.z, sv.z, pc.w * sv.w)));
}

// The same for one cell (NY not a multiple of four).
__device__ __forceinline__ float op_one(const Kry& k, const float* po, float* pn, float beta, float alpha_prev,
                                        long long q) {
  const long long ncol = k.ncol;
  const int ny = k.ny;
  const long long il = q / ncol;
  const long long cc = q - il * ncol;
  const int j0 = (int)(cc % ny);
  const long long k0 = cc / ny;
  const bool hn = il + 1 < k.nx, hs = il > 0, ht = k0 + 1 < k.nz, hb = k0 > 0;
  const long long qn = hn ? q + ncol : q, qs = hs ? q - ncol : q;
  const long long qt = ht ? q + ny : q, qb = hb ? q - ny : q;
  const long long qm = j0 == 0 ? q + ny - 1 : q - 1;
  const long long qp = j0 == ny - 1 ? q - (ny - 1) : q + 1;
  const float zc = k.z[q], oc = po[q], ec = k.e[q];
  const float zn = k.z[qn], on = po[qn], zs = k.z[qs], os = po[qs], zt = k.z[qt], ot = po[qt];
  const float zb = k.z[qb], ob = po[qb], zm = k.z[qm], om = po[qm], zp = k.z[qp], op = po[qp];
  const float crn = k.cr[q], crs = k.cr[qs], ctt = k.ct[q], ctb = k.ct[qb], cpp = k.cp[q], cpm = k.cp[qm];
  k.e[q] = fmaf(alpha_prev, oc, ec);
  const float pc = fmaf(beta, oc, zc);
  float sv = pc;
  sv = fmaf(hn ? crn : 0.f, fmaf(beta, on, zn), sv);
  sv = fmaf(hs ? crs : 0.f, fmaf(beta, os, zs), sv);
  sv = fmaf(ht ? ctt : 0.f, fmaf(beta, ot, zt), sv);
  sv = fmaf(hb ? ctb : 0.f, fmaf(beta, ob, zb), sv);
  sv = fmaf(cpp, fmaf(beta, op, zp), sv);
  sv = fmaf(cpm, fmaf(beta, om, zm), sv);
  pn[q] = pc;
  k.s[q] = sv;
  return pc * sv;
}

// z = M^-1 r for the preconditioner M, with UPDATE first r -= alpha s.
// SGS: `sweeps` symmetric red-black line Gauss-Seidel sweeps from z = 0
// (red lines, then black lines against the new red z, red against the new
// black, ...: 2 sweeps + 1 colour passes, a grid barrier between passes; two
// symmetric sweeps in a row share their middle red pass), a symmetric
// preconditioner; otherwise the radial line solve of every column (block
// Jacobi).  acc gains this thread's share of r.z (from each colour's last
// pass).  False if a barrier gave up.
template <bool UPDATE, bool SGS>
__device__ __forceinline__ bool precondition(const Kry& k, SolverDev* sol, unsigned int nb, long long col0,
                                             long long colstride, float alpha, float& acc, int sweeps,
                                             unsigned long long& passed) {
  if (!SGS) {
    for (long long c = col0; c < k.ncol; c += colstride) acc += line_pass<UPDATE>(k, c, alpha);
    return true;
  }
  const long long half = k.ncol >> 1;
  for (long long m = col0; m < half; m += colstride) (void)line_pass<UPDATE>(k, col_of(m, 0, k.ny), alpha);
  if (!grid_sync(sol, nb, passed)) return false;
  float ab = 0.f;  // r.z of the black lines' first pass (their last with one sweep)
  for (long long m = col0; m < half; m += colstride) ab += line_gs<UPDATE>(k, col_of(m, 1, k.ny), alpha);
  if (sweeps == 1) acc += ab;
#pragma unroll 1
  for (int p = 2; p <= 2 * sweeps; ++p) {
    if (!grid_sync(sol, nb, passed)) return false;
    float ap = 0.f;
    for (long long m = col0; m < half; m += colstride) ap += line_gs<false>(k, col_of(m, p & 1, k.ny), 0.f);
    if (p >= 2 * sweeps - 1) acc += ap;  // the last pass of its colour
  }
  return true;
}

// The FP32 PCG iteration on S e = r from e = 0 (r, e set by the anchor).
// Line phases: the warps of all blocks are dealt round-robin over groups of
// 32 consecutive columns.  Operator phase: p_new = z + beta p (p read from
// p[cur], written to p[1-cur], so that neighbours read the old values),
// s = S p_new, and the previous iteration's e += alpha p.  Every block forms
// alpha and beta from all block partials in the same fixed order, so all
// blocks take the same decisions.  The run ends when sqrt(r.z / r0.z0) <=
// stop_ratio, after kPcgStall iterations without a new minimum of r.z (the
// FP32 floor), on a non-positive p.s, or after maxit iterations; the last
// iteration's e update is then applied.  maxit = 0 only computes r0.z0
// (sol->scratch[2]).
template <bool SGS>
__global__ void __launch_bounds__(kPcgThreads, 1) pcg32_persistent(Kry k, SolverDev* sol, double* partials,
                                                                   int maxit, double stop_ratio, int sweeps) {
  __shared__ double sh[32];
  __shared__ double bc[3];
  const unsigned int nb = gridDim.x;
  unsigned long long passed = 0;  // grid barriers this block has passed
  const long long n = k.n;
  const int ny = k.ny;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nth = (long long)gridDim.x * blockDim.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long col0 = ((long long)warp * nb + blockIdx.x) * 32 + lane;
  const long long colstride = (long long)(blockDim.x >> 5) * nb * 32;
  double* pa = partials;                 // operator-phase partials
  double* pb = partials + kMaxPartials;  // line-phase partials

  // z0 = T^-1 r0, gamma0 = r0.z0.  Per-thread partial sums (a few hundred
  // terms) are FP32 -- GB300's FP64 pipe is narrow -- and widened to FP64
  // for the block and grid sums.
  float acc = 0.f;
  if (!precondition<false, SGS>(k, sol, nb, col0, colstride, 0.f, acc, sweeps, passed)) return;
  {
    const double v = block_sum((double)acc, sh);
    if (threadIdx.x == 0) pb[blockIdx.x] = v;
  }
  if (!grid_sync(sol, nb, passed)) return;
  {
    const double tot = block_sum_array(pb, nb, sh);
    if (threadIdx.x == 0) bc[0] = tot;
    __syncthreads();
  }
  double gamma = bc[0];
  const double gamma0 = gamma;
  if (blockIdx.x == 0 && threadIdx.x == 0) sol->scratch[2] = gamma0;
  if (maxit <= 0 || !(gamma0 > 0.0) || !isfinite(gamma0)) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && !isfinite(gamma0)) sol->nonfinite = 1;
    return;
  }
  const double stop2 = stop_ratio * stop_ratio * gamma0;
  double gmin = gamma0;
  int since_min = 0;
  float beta = 0.f, alpha_prev = 0.f;
  int cur = 0;
  bool pending = false;  // e += alpha_prev p[cur] still to be applied
  for (int it = 1; it <= maxit; ++it) {
    const float* po = cur ? k.p[1] : k.p[0];
    float* pn = cur ? k.p[0] : k.p[1];
    // operator phase
    acc = 0.f;
    const float ap = pending ? alpha_prev : 0.f;
    if ((ny & 3) == 0) {
      for (long long g = tid; g < (n >> 2); g += nth) acc += op_quad(k, po, pn, beta, ap, g << 2);
    } else {
      for (long long q = tid; q < n; q += nth) acc += op_one(k, po, pn, beta, ap, q);
    }
    pending = false;
    {
      const double v = block_sum((double)acc, sh);
      if (threadIdx.x == 0) pa[blockIdx.x] = v;
    }
    if (!grid_sync(sol, nb, passed)) return;
    {
      const double tot = block_sum_array(pa, nb, sh);
      if (threadIdx.x == 0) bc[1] = tot;
      __syncthreads();
    }
    const double ps = bc[1];
    if (!(ps > 0.0) || !isfinite(ps)) {  // breakdown: S p_new not positive (rounding)
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        sol->stalled = 1;
        if (!isfinite(ps)) sol->nonfinite = 1;
      }
      break;
    }
    const float alpha = (float)(gamma / ps);
    // line phase: r -= alpha s, z = M^-1 r, r.z
    acc = 0.f;
    if (!precondition<true, SGS>(k, sol, nb, col0, colstride, alpha, acc, sweeps, passed)) return;
    {
      const double v = block_sum((double)acc, sh);
      if (threadIdx.x == 0) pb[blockIdx.x] = v;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) sol->iter += 1;
    alpha_prev = alpha;
    pending = true;
    cur = 1 - cur;  // p[cur] is now this iteration's p
    if (!grid_sync(sol, nb, passed)) return;
    {
      const double tot = block_sum_array(pb, nb, sh);
      if (threadIdx.x == 0) bc[2] = tot;
      __syncthreads();
    }
    const double gnew = bc[2];
    if (!isfinite(gnew)) {
      if (blockIdx.x == 0 && threadIdx.x == 0) sol->nonfinite = 1;
      break;
    }
    if (gnew < gmin) {
      gmin = gnew;
      since_min = 0;
    } else if (++since_min >= kPcgStall) {
      if (blockIdx.x == 0 && threadIdx.x == 0) sol->stalled = 1;
      break;
    }
    if (!(gnew > stop2)) {
      if (blockIdx.x == 0 && threadIdx.x == 0) sol->done = 1;
      break;
    }
    beta = (float)(gnew / gamma);
    gamma = gnew;
  }
  if (pending) {
    const float* pl = cur ? k.p[1] : k.p[0];
    for (long long q = tid; q < n; q += nth) k.e[q] = fmaf(alpha_prev, pl[q], k.e[q]);
  }
}

int grid_cells(long long n) {
  int nb = grid_for(n);
  return nb > 1024 ? 1024 : nb;
}

KryWork* kry_work(ttfld_ctx* c) {
  if (c->krylov) return (KryWork*)c->krylov;
  const Dev& d = c->d;
  KryWork* w = (KryWork*)calloc(1, sizeof(KryWork));
  if (!w) return nullptr;
  Kry& k = w->k;
  k.nx = d.nx; k.ny = d.ny; k.nz = d.nz;
  k.n = (long long)ncell(d);
  k.ncol = (long long)d.ny * d.nz;
  const size_t n = (size_t)k.n;
  const size_t bytes = n * (10 * sizeof(float) + 2 * sizeof(double));
  if (cudaMalloc(&w->mem, bytes) != cudaSuccess) {
    free(w);
    return nullptr;
  }
  double* dp = (double*)w->mem;
  k.sig = dp; dp += n;
  k.wgt = dp; dp += n;
  float* fp = (float*)dp;
  float** arrs[] = {&k.cr, &k.cp, &k.ct, &k.g, &k.e, &k.r, &k.z, &k.s, &k.p[0], &k.p[1]};
  for (float** a : arrs) { *a = fp; fp += n; }
  c->krylov = w;
  return w;
}

int poll_sol(ttfld_ctx* c) {
  TT_CHECK(cudaMemcpyAsync(c->host_sol, c->sol, sizeof(SolverDev), cudaMemcpyDeviceToHost, c->stream));
  TT_CHECK(cudaStreamSynchronize(c->stream));
  if (c->host_sol->bar_timeout) {
    fprintf(stderr, "ttfld: a grid barrier of the PCG kernel timed out\n");
    return TTFLD_E_CUDA;
  }
  return 0;
}

int pcg_blocks(long long ncells) {
  static int blocks = -1;
  if (blocks < 0) {
    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int per_sm_gs = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pcg32_persistent<false>, kPcgThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_gs, pcg32_persistent<true>, kPcgThreads, 0);
    if (per_sm_gs < per_sm) per_sm = per_sm_gs;
    long long b = coop ? (long long)sms * per_sm : 0;
    blocks = (int)(b > kMaxPartials ? kMaxPartials : b);
  }
  const long long need = (ncells + kPcgThreads - 1) / kPcgThreads;
  return (int)(need < blocks ? need : blocks);
}

// One inner run; returns its iterations in *its.
// gs: 0 block-Jacobi radial lines, m >= 1 m symmetric line Gauss-Seidel sweeps.
int launch_inner(ttfld_ctx* c, KryWork* w, int maxit, double stop_ratio, int gs, int* its) {
  const int nb = pcg_blocks(w->k.n);
  if (nb <= 0) {
    fprintf(stderr, "ttfld: the PCG solver needs cooperative launch\n");
    return TTFLD_E_UNSUPPORTED;
  }
  TT_CHECK(cudaMemsetAsync(w->k.p[0], 0, (size_t)w->k.n * sizeof(float), c->stream));
  TT_CHECK(cudaMemsetAsync(&c->sol->iter, 0, sizeof(int), c->stream));
  TT_CHECK(cudaMemsetAsync(&c->sol->done, 0, sizeof(int), c->stream));
  TT_CHECK(cudaMemsetAsync(&c->sol->stalled, 0, sizeof(int), c->stream));
  Kry k = w->k;
  SolverDev* sol = c->sol;
  double* partials = c->partials;
  int sweeps = gs > 0 ? gs : 1;
  void* args[] = {&k, &sol, &partials, &maxit, &stop_ratio, &sweeps};
  const void* kern = gs > 0 ? (const void*)pcg32_persistent<true> : (const void*)pcg32_persistent<false>;
  TT_CHECK(cudaMemsetAsync(&sol->arrivals, 0, sizeof(unsigned long long), c->stream));  // grid barrier
  TT_CHECK(cudaLaunchCooperativeKernel(kern, dim3(nb), dim3(kPcgThreads), args, 0, c->stream));
  count_launches(1);
  int rc = poll_sol(c);
  if (rc) return rc;
  if (c->host_sol->nonfinite) return TTFLD_E_NONFINITE;
  *its = c->host_sol->iter;
  return 0;
}

int anchor(ttfld_ctx* c, KryWork* w, const double* x, const double* b, bool hypre, bool l2, bool with_b) {
  const int nb = grid_cells(w->k.n);
  const int h = hypre ? 1 : 0;
  if (l2 && with_b) kry_anchor_kernel<true, true><<<nb, kThreads, 0, c->stream>>>(c->d, w->k, x, b, h, c->partials, 1024);
  else if (l2) kry_anchor_kernel<true, false><<<nb, kThreads, 0, c->stream>>>(c->d, w->k, x, b, h, c->partials, 1024);
  else if (with_b) kry_anchor_kernel<false, true><<<nb, kThreads, 0, c->stream>>>(c->d, w->k, x, b, h, c->partials, 1024);
  else kry_anchor_kernel<false, false><<<nb, kThreads, 0, c->stream>>>(c->d, w->k, x, b, h, c->partials, 1024);
  count_launches(1);
  TT_CHECK_LAUNCH();
  return poll_sol(c);
}

// Factor the system (weights, couplings, line pivots).
int prepare(ttfld_ctx* c, KryWork* w, bool hypre) {
  const int nb = grid_cells(w->k.n);
  TT_CHECK(cudaMemsetAsync(&c->sol->bad_weights, 0, sizeof(int), c->stream));
  kry_weights_kernel<<<nb, kThreads, 0, c->stream>>>(c->d, w->k, hypre ? 1 : 0);
  kry_couplings_kernel<<<nb, kThreads, 0, c->stream>>>(c->d, w->k, hypre ? 1 : 0);
  kry_factor_kernel<<<grid_cells(w->k.ncol), kThreads, 0, c->stream>>>(w->k, c->sol);
  count_launches(3);
  TT_CHECK_LAUNCH();
  return 0;
}

// PCG with FP64 defect correction on x (halo array, holding the initial
// iterate).  l2 = false: stop on ||b - A x||_1 / ||b||_1 <= tol (the SOR
// system's rule); l2 = true: on ||Sigma W (b - A x)||_2 / ||Sigma W b||_2 <=
// tol (the hypre system's PCG rule on the symmetric form).  budget bounds
// the PCG iterations.  With guess_test, the initial iterate is kept only if
// its preconditioned residual norm r.z is below that of the zero iterate.
int pcg_core(ttfld_ctx* c, double* x, const double* b, bool hypre, double tol, long long budget, bool l2, int gs,
             int guess_test, int* fallback, ttfld_solve_stats* st) {
  KryWork* w = kry_work(c);
  if (!w) return TTFLD_E_CUDA;
  TT_CHECK(cudaMemsetAsync(c->sol, 0, sizeof(SolverDev), c->stream));
  int rc = prepare(c, w, hypre);
  if (rc) return rc;
  if (fallback) *fallback = 0;
  if ((rc = anchor(c, w, x, b, hypre, l2, true))) return rc;
  if (c->host_sol->bad_weights) {
    fprintf(stderr, "ttfld: PCG needs EVAL8 < 0 on every coupled row (the symmetrising weight)\n");
    return TTFLD_E_UNSUPPORTED;
  }
  if (guess_test) {
    int its = 0;
    if ((rc = launch_inner(c, w, 0, 0.0, gs, &its))) return rc;
    const double g_guess = c->host_sol->scratch[2];
    // the zero iterate: r = b
    double* zero_x = c->guess_tmp;
    if (!zero_x) {
      TT_CHECK(cudaMalloc((void**)&c->guess_tmp, nhalo(c->d) * 8));
      zero_x = c->guess_tmp;
    }
    TT_CHECK(cudaMemsetAsync(zero_x, 0, nhalo(c->d) * 8, c->stream));
    if ((rc = anchor(c, w, zero_x, b, hypre, l2, false)) || (rc = launch_inner(c, w, 0, 0.0, gs, &its))) return rc;
    const double g_zero = c->host_sol->scratch[2];
    if (!(g_guess < g_zero)) {
      TT_CHECK(cudaMemsetAsync(x, 0, nhalo(c->d) * 8, c->stream));
      if (fallback) *fallback = 1;
      // the anchor of the zero iterate is current
    } else if ((rc = anchor(c, w, x, b, hypre, l2, false))) {
      return rc;
    }
  }
  long long total = 0;
  int anchors = 0, status = TTFLD_OK, slow = 0, stalls = 0;
  double prev = INFINITY, ratio = INFINITY;
  for (;;) {
    const SolverDev& h = *c->host_sol;
    ratio = l2 ? (h.scratch[1] > 0.0 ? sqrt(h.scratch[0] / h.scratch[1]) : 0.0)
               : (h.rhsnorm > 0.0 ? h.true_l1 / h.rhsnorm : 0.0);
    if (!isfinite(ratio)) return TTFLD_E_NONFINITE;
    if (!(ratio > tol)) break;
    if (total >= budget) { status = TTFLD_MAXITER; break; }
    // an anchor that does not halve the residual twice in a row: the
    // symmetric part is too far from the rows (or FP32 cannot resolve them)
    if (ratio > 0.5 * prev) {
      if (++slow >= 2) { status = TTFLD_MAXITER; break; }
    } else {
      slow = 0;
    }
    prev = ratio;
    double target = 0.3 * tol / ratio;
    if (target < kInnerReduce) target = kInnerReduce;
    long long left = budget - total;
    int its = 0;
    if ((rc = launch_inner(c, w, (int)(left < 1000000 ? left : 1000000), target, gs, &its))) return rc;
    total += its;
    ++anchors;
    if (c->host_sol->stalled) ++stalls;
    kry_update_kernel<<<grid_cells(w->k.n), kThreads, 0, c->stream>>>(c->d, w->k, x);
    count_launches(1);
    TT_CHECK_LAUNCH();
    if ((rc = anchor(c, w, x, b, hypre, l2, false))) return rc;
  }
  // SOLVE_WITH_SOR leaves the phi halo of DELTA_ER refreshed (PLANETSHIFT(8)
  // after the last colour); SOLVE_WITH_HYPRE writes the interior only and its
  // caller shifts (ppenergy.f:353-356)
  if (!hypre && ((rc = halo_shift(c, x)) || (rc = pole_shift(c, x)))) return rc;
  if (st) {
    st->sor_iter = (int)total;
    st->corrections = anchors;
    // rnorm / rhsnorm is the stopping measure (L1, or the scaled 2-norm)
    st->rhsnorm = l2 ? sqrt(c->host_sol->scratch[1]) : c->host_sol->rhsnorm;
    st->rnorm = l2 ? sqrt(c->host_sol->scratch[0]) : c->host_sol->true_l1;
    st->true_resid_l1 = c->host_sol->true_l1;
    st->status = status;
    st->stalls = stalls;
  }
  return status;
}

}  // namespace

int solve_pcg(ttfld_ctx* c, double* x, const double* b, ttfld_solve_stats* st, int guess_test, int* fallback) {
  const long long budget = c->opts.max_sweeps > 0 ? c->opts.max_sweeps : (long long)c->d.itmax;
  return pcg_core(c, x, b, false, c->opts.tol, budget, false, 0, guess_test, fallback, st);
}

void krylov_free(ttfld_ctx* c) {
  KryWork* w = (KryWork*)c->krylov;
  if (!w) return;
  if (w->mem) cudaFree(w->mem);
  free(w);
  c->krylov = nullptr;
}

}  // namespace ttfld

extern "C" {

int ttfld_solve_with_hypre(ttfld_ctx* c, double tol, int maxit, ttfld_solve_stats* st) {
  using namespace ttfld;
  if (!c) return TTFLD_E_ARGS;
  if (c->d.poles) return TTFLD_E_UNSUPPORTED;  // hypre's pole graph (pphypre.f:458-540) is not built
  if (!(tol > 0.0)) tol = 1e-6;  // pphypre.f:45
  if (maxit <= 0) maxit = 50;    // pphypre.f:54-55
  TT_CHECK(cudaSetDevice(c->device));
  ttfld_solve_stats local{};
  if (!st) st = &local;
  int rc = fill_sor_matrix(c, false);  // the 7-point rows; b is taken from RHS_ER as it is
  if (rc) return rc;
  Dev d = c->d;
  double* x = d.DELTA_ER;
  // hypre's PCG is preconditioned by a multigrid cycle, which keeps its
  // iteration count nearly independent of the grid; the line Gauss-Seidel
  // preconditioner here needs more iterations on finer (phi, theta) grids.
  // Its strength is the number m of symmetric sweeps per application: a
  // solve that reaches the iteration cap before tol is run again from
  // x = 1 with m raised from the rate that solve showed (iterations scale
  // about as m^-1/2), and the context keeps m for its later solves.
  int m = c->hypre_gs > 0 ? c->hypre_gs : 1;
  TT_CHECK(cudaEventRecord(c->ev0, c->stream));
  for (;;) {
    // x = 1 in the interior (pphypre.f:136); the halo is left as it is, as
    // SOLVE_WITH_HYPRE only writes delta_ER(1:NX,1:NY,1:NZ) (pphypre.f:84-92)
    launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) { x[hidx(d, i, j, k)] = 1.0; });
    TT_CHECK_LAUNCH();
    rc = pcg_core(c, x, d.RHS, true, tol, maxit, true, m, 0, nullptr, st);
    if (rc != TTFLD_MAXITER || m >= kMaxGsSweeps) break;
    const double ratio = st->rhsnorm > 0.0 ? st->rnorm / st->rhsnorm : 1.0;
    double grow = 4.0;
    if (ratio > 0.0 && ratio < 1.0) {
      const double need = maxit * log(tol) / log(ratio);  // iterations at this m, at this rate
      const double f = need / (0.8 * maxit);
      grow = f * f;
    }
    int m2 = (int)ceil(m * (grow < 2.0 ? 2.0 : grow));
    m = m2 < kMaxGsSweeps ? m2 : kMaxGsSweeps;
  }
  c->hypre_gs = m;
  st->gs_sweeps = m;
  TT_CHECK(cudaEventRecord(c->ev1, c->stream));
  TT_CHECK(cudaEventSynchronize(c->ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  st->solve_ms = ms;
  c->last_solve_ms = ms;
  return rc;
}

}  // extern "C"
