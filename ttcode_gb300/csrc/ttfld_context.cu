// ttfld_context.cu -- context lifetime, parameters and field transfer of
// libttfld (the C ABI declared in include/ttfld.h).
#include <stdlib.h>
#include <string.h>

#include "ttfld_internal.cuh"

namespace ttfld {

void mix_free(ttfld_ctx* c);

int check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return 0;
  fprintf(stderr, "ttfld: CUDA error %s (%d) at %s\n", cudaGetErrorString(e), (int)e, what);
  return TTFLD_E_CUDA;
}

static unsigned long long g_launches = 0;
void count_launches(int n) { __atomic_add_fetch(&g_launches, (unsigned long long)n, __ATOMIC_RELAXED); }
unsigned long long launches() { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

int grid_for(long long n, int threads) {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
  }
  long long blocks = (n + threads - 1) / threads;
  long long cap = (long long)sms * 16;  // 16 resident 256-thread blocks per SM at most
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (int)blocks;
}

// Copy between a box-shaped contiguous buffer and an internal array.
__global__ void box_copy_kernel(double* internal, int ax, int ay, int ox, int oy, int oz,
                                double* packed, int bx, int by, int bz, int to_internal) {
  long long n = (long long)bx * by * bz;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    int i = (int)(t % bx);
    long long r = t / bx;
    int j = (int)(r % by), k = (int)(r / by);
    size_t q = (size_t)(i + ox) + (size_t)ax * ((size_t)(j + oy) + (size_t)ay * (size_t)(k + oz));
    if (to_internal) internal[q] = packed[t];
    else packed[t] = internal[q];
  }
}

}  // namespace ttfld

using namespace ttfld;

namespace {

enum StorageClass { S_HALO, S_CELL, S_FACEX, S_FACEY, S_FACEZ, S_PLANE, S_PLANE_INT, S_SINP, S_STAU };

struct FieldDesc {
  int id;
  size_t off;  // offsetof(Dev, member)
  StorageClass cls;
};

#define FDESC(id, mem, cls) {id, offsetof(Dev, mem), cls}
const FieldDesc kFields[] = {
    FDESC(TTFLD_T, T, S_HALO), FDESC(TTFLD_RH, RH, S_HALO), FDESC(TTFLD_CV, CV, S_HALO),
    FDESC(TTFLD_ER, ER, S_HALO), FDESC(TTFLD_ER_OLD, ER_OLD, S_HALO),
    FDESC(TTFLD_DELTA_ER, DELTA_ER, S_HALO), FDESC(TTFLD_XKAPR, XKAPR, S_HALO),
    FDESC(TTFLD_XKAPP, XKAPP, S_HALO), FDESC(TTFLD_XKAPA, XKAPA, S_HALO),
    FDESC(TTFLD_DXKAPP_DT, DXKAPP, S_HALO), FDESC(TTFLD_DXKAPA_DT, DXKAPA, S_HALO),
    FDESC(TTFLD_KMUL, KMUL, S_HALO), FDESC(TTFLD_Q, Q, S_HALO), FDESC(TTFLD_SCALAR, SCALAR, S_HALO),
    FDESC(TTFLD_EVAL1, E1, S_CELL), FDESC(TTFLD_EVAL2, E2, S_CELL), FDESC(TTFLD_EVAL3, E3, S_CELL),
    FDESC(TTFLD_EVAL4, E4, S_CELL), FDESC(TTFLD_EVAL5, E5, S_CELL), FDESC(TTFLD_EVAL6, E6, S_CELL),
    FDESC(TTFLD_EVAL7, E7, S_CELL), FDESC(TTFLD_EVAL8, E8, S_CELL), FDESC(TTFLD_EVAL_1_6, E16, S_CELL),
    FDESC(TTFLD_JACOB_ETA, ETA, S_CELL), FDESC(TTFLD_RHS_ER, RHS, S_CELL),
    FDESC(TTFLD_SOR_A, SA, S_CELL), FDESC(TTFLD_SOR_B, SB, S_CELL), FDESC(TTFLD_SOR_C, SC, S_CELL),
    FDESC(TTFLD_SOR_D, SD, S_CELL), FDESC(TTFLD_SOR_E, SE, S_CELL), FDESC(TTFLD_SOR_F, SF, S_CELL),
    FDESC(TTFLD_SOR_G, SG, S_CELL), FDESC(TTFLD_FQ, FQ, S_CELL), FDESC(TTFLD_FR, FR, S_CELL),
    FDESC(TTFLD_DIVF, DIVF, S_CELL), FDESC(TTFLD_DELTA_Q, DQ, S_CELL),
    FDESC(TTFLD_FLIMX, FLIMX, S_FACEX), FDESC(TTFLD_FLIMY, FLIMY, S_FACEY),
    FDESC(TTFLD_FLIMZ, FLIMZ, S_FACEZ), FDESC(TTFLD_DIFRX, DIFRX, S_FACEX),
    FDESC(TTFLD_DIFRY, DIFRY, S_FACEY), FDESC(TTFLD_DIFRZ, DIFRZ, S_FACEZ),
    FDESC(TTFLD_FLUX_X, FLUXX, S_FACEX), FDESC(TTFLD_FLUX_Y, FLUXY, S_FACEY),
    FDESC(TTFLD_FLUX_Z, FLUXZ, S_FACEZ),
    FDESC(TTFLD_UPPERBND, UB, S_PLANE_INT), FDESC(TTFLD_MU_STAR, MU, S_PLANE),
    FDESC(TTFLD_TINCIDENT, TINC, S_PLANE),
    FDESC(TTFLD_STELLARINPUT, SI, S_SINP), FDESC(TTFLD_STELLARTAU, STAU, S_STAU),
    FDESC(TTFLD_DTAUS, DTAUS, S_STAU),
};

const FieldDesc* find_field(int id) {
  for (const auto& f : kFields)
    if (f.id == id) return &f;
  return nullptr;
}

// Reference box of a storage class inside the internal array:
// internal dims (ax, ay, az), origin (ox, oy, oz), box size (bx, by, bz).
struct BoxMap {
  int ax, ay, az, ox, oy, oz, bx, by, bz;
};
BoxMap box_of(const Dev& d, StorageClass c) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  switch (c) {
    case S_HALO: return {nx + 4, ny + 4, nz + 4, 0, 0, 0, nx + 4, ny + 4, nz + 4};
    case S_CELL: return {nx, ny, nz, 0, 0, 0, nx, ny, nz};
    case S_FACEX: return {nx + 1, ny + 1, nz + 1, 0, 0, 0, nx + 1, ny, nz};
    case S_FACEY: return {nx + 1, ny + 1, nz + 1, 0, 0, 0, nx, ny + 1, nz};
    case S_FACEZ: return {nx + 1, ny + 1, nz + 1, 0, 0, 0, nx, ny, nz + 1};
    case S_PLANE:
    case S_PLANE_INT: return {ny + 4, nz + 4, 1, 0, 0, 0, ny + 4, nz + 4, 1};
    case S_SINP: return {nx + 4, ny + 4, nz + 4, 2, 0, 0, nx, ny + 4, nz + 4};
    case S_STAU: return {nx + 4, ny + 4, nz + 4, 2, 0, 0, nx + 1, ny + 4, nz + 4};
  }
  return {0, 0, 0, 0, 0, 0, 0, 0, 0};
}

bool is_direct(const BoxMap& m) { return m.ax == m.bx && m.ay == m.by && m.az == m.bz; }

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

void apply_params(ttfld_ctx* c) {
  Dev& d = c->d;
  const ttfld_params& p = c->params;
  d.delt = p.delt; d.sorparam = p.sorparam; d.epsmat = p.epsmat; d.fbottom = p.fbottom;
  d.tirr = p.tirr; d.xnue = p.xnue; d.pr_num = p.pr_num; d.kap0 = p.kap0;
  d.itmax = p.itmax; d.bcxmin = p.bcxmin; d.ibdrad = p.ibdrad; d.iflimtyp = p.iflimtyp;
  d.f_incident = p.f_incident; d.ieta = p.ieta; d.isigtyp = p.isigtyp; d.iii = p.iii;
  d.kappa_model = p.kappa_model;
  d.sigval = (p.isigtyp == 1) ? 0.4 : 0.0;  // SUBSIG pprphy.f:572-581
}

int validate_params(const ttfld_params* p) {
  if (!p) return TTFLD_E_ARGS;
  if (p->itmax < 1 || !(p->delt > 0.0)) return TTFLD_E_ARGS;
  if (p->bcxmin != 9) return TTFLD_E_UNSUPPORTED;
  if (p->iflimtyp != 1 && p->iflimtyp != 2) return TTFLD_E_UNSUPPORTED;
  if (p->f_incident < 0 || p->f_incident > 5) return TTFLD_E_UNSUPPORTED;
  if (p->isigtyp != 0 && p->isigtyp != 1) return TTFLD_E_UNSUPPORTED;
  if (p->ibdrad != 4 && p->ibdrad != 7 && p->ibdrad != 9) return TTFLD_E_UNSUPPORTED;
  if (p->kappa_model < 0 || p->kappa_model > 3) return TTFLD_E_UNSUPPORTED;
  return 0;
}

}  // namespace

extern "C" {

int ttfld_abi_version(void) { return TTFLD_ABI_VERSION; }

uint64_t ttfld_kernel_launches(void) { return (uint64_t)ttfld::launches(); }

const char* ttfld_status_string(int s) {
  switch (s) {
    case TTFLD_OK: return "ok";
    case TTFLD_MAXITER: return "iteration limit reached";
    case TTFLD_FALLBACK: return "learned guess rejected, zero guess used";
    case TTFLD_E_ARGS: return "bad argument";
    case TTFLD_E_CUDA: return "CUDA error";
    case TTFLD_E_UNSUPPORTED: return "configuration not implemented";
    case TTFLD_E_NONPOSITIVE_Q: return "non-positive Q after the update (CLEAN_STOP)";
    case TTFLD_E_NONFINITE: return "non-finite norm";
    case TTFLD_E_NOMODEL: return "no learned-guess model loaded";
    case TTFLD_E_OPACITY: return "opacity table: T <= 0, (T, rho) outside the table or a non-positive opacity";
    case TTFLD_E_INTERNAL: return "internal invariant broken (a library bug)";
  }
  return "unknown status";
}

int ttfld_create(ttfld_ctx** out, const ttfld_dims* dims, const ttfld_metrics* m,
                 const ttfld_params* params, int device) {
  if (!out || !dims || !m || !params) return TTFLD_E_ARGS;
  *out = nullptr;
  if (dims->nx < 4 || dims->ny < 4 || dims->nz < 4) return TTFLD_E_ARGS;
  if (dims->poles != 0 && dims->poles != 1) return TTFLD_E_ARGS;
  if (dims->ny % 2) return TTFLD_E_UNSUPPORTED;  // periodic red-black needs even NY
  int rc = validate_params(params);
  if (rc) return rc;
  TT_CHECK(cudaSetDevice(device));
  ttfld_ctx* c = (ttfld_ctx*)calloc(1, sizeof(ttfld_ctx));
  if (!c) return TTFLD_E_ARGS;
  c->dims = *dims;
  c->params = *params;
  c->device = device;
  c->opts.solver = TTFLD_SOLVER_SOR64_EXACT;
  c->opts.guess = TTFLD_GUESS_ZERO;
  c->opts.tol = 1e-10;
  c->opts.inner_digits = 4;
  c->opts.fallback_rule = 3;
  c->prev_scale = 0.9;
  Dev& d = c->d;
  d.nx = dims->nx; d.ny = dims->ny; d.nz = dims->nz;
  d.poles = dims->poles;
  apply_params(c);

  const size_t H = nhalo(d), Cn = ncell(d), Fn = nface(d), Pn = nplane(d);
  const int n1 = (d.nx > d.ny ? (d.nx > d.nz ? d.nx : d.nz) : (d.ny > d.nz ? d.ny : d.nz)) + 4;
  double** halo[] = {&d.T, &d.RH, &d.CV, &d.ER, &d.ER_OLD, &d.Q, &d.Q_OLD, &d.DELTA_ER,
                     &d.XKAPR, &d.XKAPP, &d.XKAPA, &d.DXKAPP, &d.DXKAPA, &d.KMUL, &d.RHQX,
                     &d.RHQY, &d.RHQZ, &d.STAU, &d.DTAUS, &d.SI, &d.SCALAR};
  double** cell[] = {&d.E1, &d.E2, &d.E3, &d.E4, &d.E5, &d.E6, &d.E7, &d.E8, &d.E16,
                     &d.ETA, &d.FQ, &d.FR, &d.RHS, &d.SA, &d.SB, &d.SC, &d.SD, &d.SE,
                     &d.SF, &d.SG, &d.DIVF, &d.DIVF_OLD, &d.DFQ, &d.DFR, &d.DQ, &d.RHS_DIF};
  double** face[] = {&d.FLIMX, &d.FLIMY, &d.FLIMZ, &d.DIFRX, &d.DIFRY, &d.DIFRZ,
                     &d.FLUXX, &d.FLUXY, &d.FLUXZ};
  const double** g1[] = {&d.xxa, &d.xxb, &d.dxa, &d.dxb, &d.xya, &d.xyb, &d.dya, &d.dyb,
                         &d.xza, &d.xzb, &d.dza, &d.dzb, &d.ddx0, &d.ddx1, &d.ddy0, &d.ddy1,
                         &d.ddz0, &d.ddz1, &d.surxa, &d.surxb, &d.surza, &d.surzb, &d.geoxg,
                         &d.geoxh, &d.geoxga, &d.geoxha, &d.geozg, &d.geozga};
  const size_t A = 256;
  size_t bytes = 0;
  const size_t nh = sizeof(halo) / sizeof(halo[0]), nc = sizeof(cell) / sizeof(cell[0]);
  const size_t nf = sizeof(face) / sizeof(face[0]), ng = sizeof(g1) / sizeof(g1[0]);
  bytes += nh * align_up(H * 8, A) + nc * align_up(Cn * 8, A) + nf * align_up(Fn * 8, A);
  bytes += 3 * align_up(Pn * 8, A) + ng * align_up((size_t)n1 * 8, A);
  bytes += align_up(sizeof(SolverDev), A) + align_up(sizeof(StepDev), A);
  bytes += align_up(2 * kMaxPartials * 8, A);
  size_t staging = H > Fn ? H : Fn;
  bytes += align_up(staging * 8, A);
  char* base = nullptr;
  if (check_cuda(cudaMalloc((void**)&base, bytes), "cudaMalloc slab")) { free(c); return TTFLD_E_CUDA; }
  c->slab = base;
  c->slab_bytes = bytes;
  cudaMemset(base, 0, bytes);
  size_t off = 0;
  auto take = [&](size_t b) { char* p = base + off; off += align_up(b, A); return p; };
  for (size_t q = 0; q < nh; ++q) *halo[q] = (double*)take(H * 8);
  for (size_t q = 0; q < nc; ++q) *cell[q] = (double*)take(Cn * 8);
  for (size_t q = 0; q < nf; ++q) *face[q] = (double*)take(Fn * 8);
  d.UB = (int*)take(Pn * 8);
  d.MU = (double*)take(Pn * 8);
  d.TINC = (double*)take(Pn * 8);
  for (size_t q = 0; q < ng; ++q) *g1[q] = (const double*)take((size_t)n1 * 8);
  c->sol = (SolverDev*)take(sizeof(SolverDev));
  c->stp = (StepDev*)take(sizeof(StepDev));
  c->partials = (double*)take(2 * kMaxPartials * 8);
  c->staging = (double*)take(staging * 8);
  d.sol = c->sol;
  d.stp = c->stp;

  // 1-D metrics with the reference's lower bounds (ttfld.h, ttfld_metrics).
  struct M { const double* src; const double* dst; int lo, hi; };
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  M ms[] = {{m->xxa, d.xxa, 0, nx + 2}, {m->xxb, d.xxb, -1, nx + 2}, {m->dxa, d.dxa, 1, nx + 2},
            {m->dxb, d.dxb, 0, nx + 2}, {m->xya, d.xya, 0, ny + 2}, {m->xyb, d.xyb, -1, ny + 2},
            {m->dya, d.dya, 1, ny + 2}, {m->dyb, d.dyb, 0, ny + 2}, {m->xza, d.xza, 0, nz + 2},
            {m->xzb, d.xzb, -1, nz + 2}, {m->dza, d.dza, 1, nz + 2}, {m->dzb, d.dzb, 0, nz + 2},
            {m->ddx0, d.ddx0, 0, nx + 2}, {m->ddx1, d.ddx1, 0, nx + 2}, {m->ddy0, d.ddy0, 0, ny + 2},
            {m->ddy1, d.ddy1, 0, ny + 2}, {m->ddz0, d.ddz0, 0, nz + 2}, {m->ddz1, d.ddz1, 0, nz + 2},
            {m->surxa, d.surxa, 0, nx + 2}, {m->surxb, d.surxb, 0, nx + 2},
            {m->surza, d.surza, 0, nz + 2}, {m->surzb, d.surzb, 0, nz + 2},
            {m->geoxg, d.geoxg, -1, nx + 2}, {m->geoxh, d.geoxh, -1, nx + 2},
            {m->geoxga, d.geoxga, 0, nx + 2}, {m->geoxha, d.geoxha, 0, nx + 2},
            {m->geozg, d.geozg, -1, nz + 2}, {m->geozga, d.geozga, 0, nz + 2}};
  for (const M& e : ms) {
    if (!e.src) { ttfld_destroy(c); return TTFLD_E_ARGS; }
    if (check_cuda(cudaMemcpy((void*)(e.dst + (e.lo + 1)), e.src, (size_t)(e.hi - e.lo + 1) * 8,
                              cudaMemcpyHostToDevice), "metrics")) {
      ttfld_destroy(c);
      return TTFLD_E_CUDA;
    }
  }
  if (check_cuda(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream") ||
      check_cuda(cudaEventCreate(&c->ev0), "event") || check_cuda(cudaEventCreate(&c->ev1), "event") ||
      check_cuda(cudaEventCreate(&c->evg), "event") ||
      check_cuda(cudaMallocHost((void**)&c->host_sol, sizeof(SolverDev)), "pinned")) {
    ttfld_destroy(c);
    return TTFLD_E_CUDA;
  }
  // CV defaults to nothing: the caller uploads it (GASINIT ppinit.f:1408-1417).
  TT_CHECK(cudaDeviceSynchronize());
  *out = c;
  return TTFLD_OK;
}

int ttfld_destroy(ttfld_ctx* c) {
  if (!c) return TTFLD_E_ARGS;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  unet_free(c);
  asm_free(c);
  mix_free(c);
  krylov_free(c);
  if (c->opac) cudaFree(c->opac);
  if (c->freed) cudaFree(c->freed);
  if (c->wave) cudaFree(c->wave);
  if (c->xkapw) cudaFree(c->xkapw);
  if (c->prev_x) cudaFree(c->prev_x);
  if (c->guess_tmp) cudaFree(c->guess_tmp);
  if (c->slab) cudaFree(c->slab);
  if (c->host_sol) cudaFreeHost(c->host_sol);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->evg) cudaEventDestroy(c->evg);
  if (c->stream) cudaStreamDestroy(c->stream);
  free(c);
  return TTFLD_OK;
}

int ttfld_set_params(ttfld_ctx* c, const ttfld_params* p) {
  if (!c) return TTFLD_E_ARGS;
  int rc = validate_params(p);
  if (rc) return rc;
  c->params = *p;
  apply_params(c);
  return TTFLD_OK;
}

int ttfld_get_params(const ttfld_ctx* c, ttfld_params* p) {
  if (!c || !p) return TTFLD_E_ARGS;
  *p = c->params;
  return TTFLD_OK;
}

int ttfld_set_solver(ttfld_ctx* c, const ttfld_solve_opts* o) {
  if (!c || !o) return TTFLD_E_ARGS;
  if (o->solver < 0 || o->solver > 3 || o->guess < 0 || o->guess > 2) return TTFLD_E_ARGS;
  if (o->solver == TTFLD_SOLVER_MIXED && !(o->tol > 0.0)) return TTFLD_E_ARGS;
  if (o->fallback_rule < 0 || o->fallback_rule > 3) return TTFLD_E_ARGS;
  if (o->sweep_form < 0 || o->sweep_form > 4) return TTFLD_E_ARGS;
  c->opts = *o;
  if (c->opts.inner_digits <= 0) c->opts.inner_digits = 4;
  if (c->opts.inner_digits > 12) c->opts.inner_digits = 12;
  return TTFLD_OK;
}

size_t ttfld_field_size(const ttfld_ctx* c, int field) {
  if (!c) return 0;
  const FieldDesc* f = find_field(field);
  if (!f) return 0;
  BoxMap b = box_of(c->d, f->cls);
  return (size_t)b.bx * b.by * b.bz;
}

void* ttfld_device_ptr(ttfld_ctx* c, int field) {
  if (!c) return nullptr;
  const FieldDesc* f = find_field(field);
  if (!f) return nullptr;
  return *(void**)((char*)&c->d + f->off);
}

int ttfld_upload(ttfld_ctx* c, int field, const void* host) {
  if (!c || !host) return TTFLD_E_ARGS;
  const FieldDesc* f = find_field(field);
  if (!f) return TTFLD_E_ARGS;
  TT_CHECK(cudaSetDevice(c->device));
  void* dst = *(void**)((char*)&c->d + f->off);
  BoxMap b = box_of(c->d, f->cls);
  size_t n = (size_t)b.bx * b.by * b.bz;
  size_t esz = (f->cls == S_PLANE_INT) ? 4 : 8;
  if (is_direct(b)) {
    TT_CHECK(cudaMemcpyAsync(dst, host, n * esz, cudaMemcpyHostToDevice, c->stream));
  } else {
    TT_CHECK(cudaMemcpyAsync(c->staging, host, n * 8, cudaMemcpyHostToDevice, c->stream));
    box_copy_kernel<<<grid_for((long long)n), kThreads, 0, c->stream>>>(
        (double*)dst, b.ax, b.ay, b.ox, b.oy, b.oz, c->staging, b.bx, b.by, b.bz, 1);
    count_launches(1);
    TT_CHECK_LAUNCH();
  }
  TT_CHECK(cudaStreamSynchronize(c->stream));
  return TTFLD_OK;
}

int ttfld_download(ttfld_ctx* c, int field, void* host) {
  if (!c || !host) return TTFLD_E_ARGS;
  const FieldDesc* f = find_field(field);
  if (!f) return TTFLD_E_ARGS;
  TT_CHECK(cudaSetDevice(c->device));
  void* src = *(void**)((char*)&c->d + f->off);
  BoxMap b = box_of(c->d, f->cls);
  size_t n = (size_t)b.bx * b.by * b.bz;
  size_t esz = (f->cls == S_PLANE_INT) ? 4 : 8;
  if (is_direct(b)) {
    TT_CHECK(cudaMemcpyAsync(host, src, n * esz, cudaMemcpyDeviceToHost, c->stream));
  } else {
    box_copy_kernel<<<grid_for((long long)n), kThreads, 0, c->stream>>>(
        (double*)src, b.ax, b.ay, b.ox, b.oy, b.oz, c->staging, b.bx, b.by, b.bz, 0);
    count_launches(1);
    TT_CHECK_LAUNCH();
    TT_CHECK(cudaMemcpyAsync(host, c->staging, n * 8, cudaMemcpyDeviceToHost, c->stream));
  }
  TT_CHECK(cudaStreamSynchronize(c->stream));
  return TTFLD_OK;
}

int ttfld_copy_field(ttfld_ctx* c, int dst_field, int src_field) {
  if (!c) return TTFLD_E_ARGS;
  const FieldDesc* a = find_field(dst_field);
  const FieldDesc* b = find_field(src_field);
  if (!a || !b || a->cls != b->cls) return TTFLD_E_ARGS;
  BoxMap m = box_of(c->d, a->cls);
  size_t n = (size_t)m.ax * m.ay * m.az;
  size_t esz = (a->cls == S_PLANE_INT) ? 4 : 8;
  TT_CHECK(cudaMemcpyAsync(*(void**)((char*)&c->d + a->off), *(void**)((char*)&c->d + b->off),
                           n * esz, cudaMemcpyDeviceToDevice, c->stream));
  return TTFLD_OK;
}

void* ttfld_stream(ttfld_ctx* c) { return c ? (void*)c->stream : nullptr; }

int ttfld_synchronize(ttfld_ctx* c) {
  if (!c) return TTFLD_E_ARGS;
  TT_CHECK(cudaStreamSynchronize(c->stream));
  return TTFLD_OK;
}

}  // extern "C"
