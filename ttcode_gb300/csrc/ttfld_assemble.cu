// ttfld_assemble.cu -- FP64 coefficient assembly of the implicit FLD step:
// KAPPA/SUBSIG/QDENS, FLIM, DIFF, CALCULATEFLUX, FLUX_BC, FILL_EVALUES,
// CALCULATEDIVF_WITHF, the grey stellar heating, BOUNDS for the planet set-up
// and the one-rank PLANETSHIFT.  Each kernel body is one reference loop nest
// (cited), launched over the same index box, with the same operand order.
#include "ttfld_internal.cuh"

namespace ttfld {

// ---- PLANETSHIFT ppshift.f:1009-1214, one rank --------------------------
// Only the "from lower" (:1096-1107) and "from upper" (:1164-1173) copies
// act with one rank; z and corner partners are MPI_PROC_NULL.
int halo_shift(ttfld_ctx* c, double* a) {
  Dev d = c->d;
  launch_box(c->stream, box(-1, d.nx + 2, 0, 0, 1, d.nz), [=] __device__(int i, int, int k) {
    a[hidx(d, i, 0, k)] = a[hidx(d, i, d.ny, k)];
    a[hidx(d, i, -1, k)] = a[hidx(d, i, d.ny - 1, k)];
    a[hidx(d, i, d.ny + 1, k)] = a[hidx(d, i, 1, k)];
    a[hidx(d, i, d.ny + 2, k)] = a[hidx(d, i, 2, k)];
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// NORTH_POLE_SHIFT / SOUTH_POLE_SHIFT ppshift.f:2217-2453 with one rank: the
// partner across each pole (myid -/+ numprocs/2, ppshift.f:820-833) is the
// rank itself, so planes NZ-1, NZ-2, NZ-3 are copied onto NZ, NZ+1, NZ+2 and
// planes 1, 2 onto 0, -1, over the whole (i, j) extent with the ghosts.
// Nothing without poles.
int pole_shift(ttfld_ctx* c, double* a) {
  Dev d = c->d;
  if (!d.poles) return 0;
  launch_box(c->stream, box(-1, d.nx + 2, -1, d.ny + 2, 0, 0), [=] __device__(int i, int j, int) {
    const int nz = d.nz;
    for (int m = 0; m < 3; ++m) a[hidx(d, i, j, nz + m)] = a[hidx(d, i, j, nz - 1 - m)];
    for (int m = 0; m < 2; ++m) a[hidx(d, i, j, -m)] = a[hidx(d, i, j, 1 + m)];
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// Synthetic analytic opacity in KAPPA's IKAPTYP 20:25 branch
// (pprphy.f:321-351): evaluated for i = -1..UPPERBND, then i = UPPERBND..NX+2
// copied from UPPERBND-1.  kappa_P = kappa_A = kappa_R, zero T-derivatives
// (the IKAPTYP=3 convention, pprphy.f:84-87).
__device__ __forceinline__ double kap_formula(const Dev& d, double t, double rh, double kmul) {
  double th = t / 1000.0;
  return ((d.kap0 * sqrt(rh)) * (th * sqrt(th))) * kmul;
}

// The opacity table of kappa_model 2 in device memory: an error word, then
// log10 T (nt), log10 rho (nrh) and the three log10 means (nt x nrh, T
// index fastest).
struct OpacTab {
  int nt, nrh;
  int* err;
  const double *lt, *lrh, *ross, *plnk, *absk;
};

static OpacTab opac_tab(const ttfld_ctx* c) {
  OpacTab t;
  t.nt = c->opac_nt;
  t.nrh = c->opac_nrh;
  t.err = (int*)c->opac;
  const double* p = (const double*)c->opac + 1;
  t.lt = p; p += t.nt;
  t.lrh = p; p += t.nrh;
  t.ross = p; p += (size_t)t.nt * t.nrh;
  t.plnk = p; p += (size_t)t.nt * t.nrh;
  t.absk = p;
  return t;
}

// BurrowsOPC (pprphy.f:1005-1229) for the Rosseland, Planck and absorption
// means: log10 T and log10 rho clamped to the table's interior (REAL*4
// literals, :1045-1049), the first node above each (:1050, :1087), weights
// WS1/WS along T and WS2/WS3 along rho (:1081-1084, :1106-1109), 10^ of the
// bilinear form (:1112-1135), the T-derivative stand-ins of :1180-1185.
// Returns 0, or the reason the reference stops (1: T <= 0, 2: above the
// table, 3: below it, 4: a non-positive opacity).
__device__ __forceinline__ int burrows_opc(const OpacTab& tb, double t, double rh, double& kp, double& kr,
                                           double& ka, double& dkp, double& dka) {
  if (!(t > 0.0)) return 1;
  double rh1 = log10(rh), tm1 = log10(t);
  if (tm1 < (double)1.69896f) tm1 = (double)1.69897f;
  if (tm1 > (double)3.69889f) tm1 = (double)3.69888f;
  if (rh1 < (double)-11.9996f) rh1 = (double)-11.9995f;
  if (rh1 > (double)-1.99993f) rh1 = (double)-1.99994f;
  int it = 1;
  while (it <= tb.nt && !(tb.lt[it - 1] > tm1)) ++it;
  if (it == tb.nt + 1) return 2;
  if (it == 1) return 3;
  const int it1 = it - 1;
  double ws1 = tb.lt[it1 - 1] - tm1;
  double ws = tb.lt[it1 - 1] - tb.lt[it - 1];
  ws1 = ws1 / ws;
  ws = 1.0 - ws1;
  int iw = 1;
  while (iw <= tb.nrh && !(tb.lrh[iw - 1] > rh1)) ++iw;
  if (iw == tb.nrh + 1) return 2;
  if (iw == 1) return 3;
  const int iw1 = iw - 1;
  double ws2 = rh1 - tb.lrh[iw1 - 1];
  double ws3 = tb.lrh[iw - 1] - tb.lrh[iw1 - 1];
  ws2 = ws2 / ws3;
  ws3 = 1.0 - ws2;
  const size_t n00 = (size_t)(it - 1) + (size_t)tb.nt * (iw - 1), n10 = (size_t)(it - 1) + (size_t)tb.nt * (iw1 - 1);
  const size_t n11 = (size_t)(it1 - 1) + (size_t)tb.nt * (iw1 - 1), n01 = (size_t)(it1 - 1) + (size_t)tb.nt * (iw - 1);
  auto interp = [&](const double* a) {
    const double w4 = ws2 * (ws1 * a[n00] + ws * a[n01]);
    const double w5 = ws3 * (ws1 * a[n10] + ws * a[n11]);
    return pow(10.0, w4 + w5);
  };
  kr = interp(tb.ross);
  kp = interp(tb.plnk);
  ka = interp(tb.absk);
  const double dt = pow(10.0, tb.lt[it - 1]) - pow(10.0, tb.lt[it1 - 1]);
  dkp = (pow(10.0, tb.plnk[n00]) - pow(10.0, tb.plnk[n01])) / dt;
  dka = (pow(10.0, tb.absk[n00]) - pow(10.0, tb.absk[n01])) / dt;
  if (kr <= 0.0 || kp <= 0.0 || ka <= 0.0) return 4;
  return 0;
}

// BurrowsOPC's per-bin opacities (pprphy.f:1138-1151): 10** of the bilinear
// form of log BurrowsXKAP_waveopac at burrows_opc's bracketing of (T, rho),
// for the nb bins, into out[l * stride].  Returns 0, or 2/3 off the table.
__device__ __forceinline__ int burrows_wave(const OpacTab& tb, const double* wop, int nb, double t, double rh,
                                           double* out, size_t stride) {
  double rh1 = log10(rh), tm1 = log10(t);
  if (tm1 < (double)1.69896f) tm1 = (double)1.69897f;
  if (tm1 > (double)3.69889f) tm1 = (double)3.69888f;
  if (rh1 < (double)-11.9996f) rh1 = (double)-11.9995f;
  if (rh1 > (double)-1.99993f) rh1 = (double)-1.99994f;
  int it = 1;
  while (it <= tb.nt && !(tb.lt[it - 1] > tm1)) ++it;
  if (it == tb.nt + 1) return 2;
  if (it == 1) return 3;
  const int it1 = it - 1;
  double ws1 = tb.lt[it1 - 1] - tm1;
  double ws = tb.lt[it1 - 1] - tb.lt[it - 1];
  ws1 = ws1 / ws;
  ws = 1.0 - ws1;
  int iw = 1;
  while (iw <= tb.nrh && !(tb.lrh[iw - 1] > rh1)) ++iw;
  if (iw == tb.nrh + 1) return 2;
  if (iw == 1) return 3;
  const int iw1 = iw - 1;
  double ws2 = rh1 - tb.lrh[iw1 - 1];
  double ws3 = tb.lrh[iw - 1] - tb.lrh[iw1 - 1];
  ws2 = ws2 / ws3;
  ws3 = 1.0 - ws2;
  const size_t nn = (size_t)tb.nt * tb.nrh;
  const size_t n00 = (size_t)(it - 1) + (size_t)tb.nt * (iw - 1), n10 = (size_t)(it - 1) + (size_t)tb.nt * (iw1 - 1);
  const size_t n11 = (size_t)(it1 - 1) + (size_t)tb.nt * (iw1 - 1), n01 = (size_t)(it1 - 1) + (size_t)tb.nt * (iw - 1);
  for (int l = 0; l < nb; ++l) {
    const double* a = wop + nn * l;
    const double w4 = ws2 * (ws1 * a[n00] + ws * a[n01]);
    const double w5 = ws3 * (ws1 * a[n10] + ws * a[n11]);
    out[stride * l] = pow(10.0, w4 + w5);
  }
  return 0;
}

// FreedmanTVAL and FreedmanPVAL (ppmod.f:690-700; P in mbar).
__device__ const double kFreedT[42] = {
    75.0, 100.0, 110.0, 120.0, 130.0, 140.0, 150.0, 160.0, 170.0, 180.0, 190.0, 200.0, 210.0, 220.0,
    230.0, 240.0, 250.0, 275.0, 300.0, 400.0, 500.0, 575.0, 650.0, 725.0, 800.0, 900.0, 1000.0, 1100.0,
    1200.0, 1300.0, 1400.0, 1500.0, 1600.0, 1700.0, 1800.0, 1900.0, 2000.0, 2300.0, 2600.0, 3000.0,
    3500.0, 4000.0};
__device__ const double kFreedP[18] = {0.001, 0.003, 0.01, 0.03, 0.1, 0.3, 1.0, 3.0, 10.0,
                                       30.0, 100.0, 300.0, 1000.0, 3000.0, 10000.0, 30000.0, 100000.0, 300000.0};

// FreedmanOPC pprphy.f:800-942 at (T, P_gas in dyn/cm^2): P in mbar, the
// clamps of :830-833, the first node above T and above P, weights linear in
// T and P, 10** of the bilinear log means, the T-derivative stand-ins of
// :895-899.  tab holds ross, plnk, abs (42 x 18 each, T fastest).  Returns
// 0, or 1 T <= 0, 2 above / 3 below the nodes, 4 a non-positive opacity.
__device__ __forceinline__ int freedman_opc(const double* tab, double t, double pg, double& kp, double& kr,
                                            double& ka, double& dkp, double& dka) {
  if (t <= 0.0) return 1;
  double pg1 = pg * (0.001);
  double tm1 = t;
  if (tm1 < 75.0) tm1 = 75.001;
  if (tm1 > 4000.0) tm1 = 3999.9;
  if (pg1 < 0.001) pg1 = 0.001001;
  if (pg1 > 300000.0) pg1 = 299999.9;
  int it = 1;
  while (it <= 42 && !(kFreedT[it - 1] > tm1)) ++it;
  if (it == 43) return 2;
  if (it == 1) return 3;
  const int it1 = it - 1;
  double ws1 = kFreedT[it1 - 1] - tm1;
  double ws = kFreedT[it1 - 1] - kFreedT[it - 1];
  ws1 = ws1 / ws;
  ws = 1.0 - ws1;
  int iw = 1;
  while (iw <= 18 && !(kFreedP[iw - 1] > pg1)) ++iw;
  if (iw == 19) return 2;
  if (iw == 1) return 3;
  const int iw1 = iw - 1;
  double ws2 = pg1 - kFreedP[iw1 - 1];
  double ws3 = kFreedP[iw - 1] - kFreedP[iw1 - 1];
  ws2 = ws2 / ws3;
  ws3 = 1.0 - ws2;
  const size_t n00 = (size_t)(it - 1) + 42 * (size_t)(iw - 1), n10 = (size_t)(it - 1) + 42 * (size_t)(iw1 - 1);
  const size_t n11 = (size_t)(it1 - 1) + 42 * (size_t)(iw1 - 1), n01 = (size_t)(it1 - 1) + 42 * (size_t)(iw - 1);
  const double* ross = tab;
  const double* plnk = tab + 42 * 18;
  const double* absk = tab + 2 * 42 * 18;
  auto interp = [&](const double* a) {
    const double w4 = ws2 * (ws1 * a[n00] + ws * a[n01]);
    const double w5 = ws3 * (ws1 * a[n10] + ws * a[n11]);
    return pow(10.0, w4 + w5);
  };
  kr = interp(ross);
  kp = interp(plnk);
  ka = interp(absk);
  const double dt = kFreedT[it - 1] - kFreedT[it1 - 1];
  dkp = ((pow(10.0, plnk[n00])) - (pow(10.0, plnk[n01]))) / dt;
  dka = ((pow(10.0, absk[n00])) - (pow(10.0, absk[n01]))) / dt;
  if (kr <= 0.0 || kp <= 0.0 || ka <= 0.0) return 4;
  return 0;
}

static int kappa(ttfld_ctx* c) {
  Dev d = c->d;
  if (d.kappa_model == 1) return 0;  // prescribed opacities: KAPPA is the caller's
  if (d.kappa_model == 3) {
    if (!c->freed) {
      fprintf(stderr, "ttfld: kappa_model 3 without a Freedman table (ttfld_set_freedman_table)\n");
      return TTFLD_E_OPACITY;
    }
    // the IKAPTYP 4:5 branch, MODTYP 2 (pprphy.f:88-110): FreedmanOPC for
    // i = -1..UPPERBND on PRESSG's PG = Rgas T RH / mu_gas, the values of
    // UPPERBND above it (each of those cells evaluates UPPERBND itself)
    int* err = (int*)c->freed;
    const double* tab = c->freed + 1;
    const double mu = c->freed_mu;
    TT_CHECK(cudaMemsetAsync(err, 0, sizeof(int), c->stream));
    launch_box(c->stream, box(-1, d.nx + 2, -1, d.ny + 2, -1, d.nz + 2), [=] __device__(int i, int j, int k) {
      const int ub = PA(UB, j, k);
      if (ub < -1 || ub > d.nx + 2) { atomicExch(err, 5); return; }
      const size_t s = hidx(d, i <= ub ? i : ub, j, k), q = hidx(d, i, j, k);
      const double pg = TT_RGAS * d.T[s] * d.RH[s] / mu;
      double kp, kr, ka, dkp, dka;
      const int e = freedman_opc(tab, d.T[s], pg, kp, kr, ka, dkp, dka);
      if (e) atomicExch(err, e);
      d.XKAPR[q] = kr; d.XKAPP[q] = kp; d.XKAPA[q] = ka;
      d.DXKAPP[q] = dkp; d.DXKAPA[q] = dka;
    });
    TT_CHECK_LAUNCH();
    int e = 0;
    TT_CHECK(cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TT_CHECK(cudaStreamSynchronize(c->stream));
    if (e) {
      fprintf(stderr, "ttfld: KAPPA from the Freedman table stopped (reason %d: 1 T<=0, 2 above, 3 below the "
                      "nodes, 4 non-positive opacity, 5 UPPERBND outside the grid)\n", e);
      return TTFLD_E_OPACITY;
    }
    return 0;
  }
  if (d.kappa_model == 2) {
    if (!c->opac) {
      fprintf(stderr, "ttfld: kappa_model 2 without an opacity table (ttfld_set_opacity_table)\n");
      return TTFLD_E_OPACITY;
    }
    const OpacTab tb = opac_tab(c);
    TT_CHECK(cudaMemsetAsync(tb.err, 0, sizeof(int), c->stream));
    // with a wave table, also the per-bin opacities xkapW (pprphy.f:331-341)
    const int nb = c->wave ? c->wave_nb : 0;
    const double* wop = c->wave;
    double* xkapw = c->xkapw;
    const size_t nh = nhalo(d);
    // cells from UPPERBND up take the values of UPPERBND-1 (pprphy.f:336-348)
    launch_box(c->stream, box(-1, d.nx + 2, -1, d.ny + 2, -1, d.nz + 2), [=] __device__(int i, int j, int k) {
      int ub = PA(UB, j, k);
      if (ub < 1 || ub > d.nx + 1) return;
      size_t s = hidx(d, i < ub ? i : ub - 1, j, k);
      size_t q = hidx(d, i, j, k);
      double kp, kr, ka, dkp, dka;
      int e = burrows_opc(tb, d.T[s], d.RH[s], kp, kr, ka, dkp, dka);
      if (nb > 0 && !e) e = burrows_wave(tb, wop, nb, d.T[s], d.RH[s], xkapw + q, nh);
      if (e) atomicExch(tb.err, e);
      d.XKAPR[q] = kr; d.XKAPP[q] = kp; d.XKAPA[q] = ka;
      d.DXKAPP[q] = dkp; d.DXKAPA[q] = dka;
    });
    TT_CHECK_LAUNCH();
    int err = 0;
    TT_CHECK(cudaMemcpyAsync(&err, tb.err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TT_CHECK(cudaStreamSynchronize(c->stream));
    if (err) {
      fprintf(stderr, "ttfld: KAPPA from the opacity table stopped (reason %d: 1 T<=0, 2 above, 3 below the "
                      "table, 4 non-positive opacity)\n", err);
      return TTFLD_E_OPACITY;
    }
    return 0;
  }
  // One thread per cell: the cells from UPPERBND up end with the value of
  // UPPERBND-1, which each of them evaluates itself (same inputs, same bits).
  launch_box(c->stream, box(-1, d.nx + 2, -1, d.ny + 2, -1, d.nz + 2), [=] __device__(int i, int j, int k) {
    int ub = PA(UB, j, k);
    if (ub < 1 || ub > d.nx + 1) return;
    size_t s = hidx(d, i < ub ? i : ub - 1, j, k);
    size_t q = hidx(d, i, j, k);
    double kr = kap_formula(d, d.T[s], d.RH[s], d.KMUL[s]);
    d.XKAPR[q] = kr; d.XKAPP[q] = kr; d.XKAPA[q] = kr;
    d.DXKAPP[q] = 0.0; d.DXKAPA[q] = 0.0;
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// QDENS ppphy.f:47-76
static int qdens(ttfld_ctx* c) {
  Dev d = c->d;
  launch_box(c->stream, box(-1, d.nx + 2, -1, d.ny + 2, -1, d.nz + 2), [=] __device__(int i, int j, int k) {
    size_t q = hidx(d, i, j, k);
    if (i >= 0) d.RHQX[q] = G(ddx1, i) * d.RH[q] + G(ddx0, i) * HA(RH, i - 1, j, k);
    if (j >= 0) d.RHQY[q] = G(ddy1, j) * d.RH[q] + G(ddy0, j) * HA(RH, i, j - 1, k);
    if (k >= 0) d.RHQZ[q] = G(ddz1, k) * d.RH[q] + G(ddz0, k) * HA(RH, i, j, k - 1);
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// ---- FLIM, DIFF, CALCULATEFLUX and FLUX_BC, one face at a time ---------
// Each reference loop nest becomes a device function of one face with the
// reference's operand order, so that a single kernel can form FLIM, DIFF
// and the fluxes of a face together (bit for bit the values of the separate
// loops).

// FLIM's x loop body, pprphy.f:414-448 (IFLIMTYP 2).
__device__ __forceinline__ double flimx_calc(const Dev& d, int i, int j, int k) {
  const double sg = d.sigval;
  double gradx = (HA(ER, i, j, k) - HA(ER, i - 1, j, k)) / G(dxb, i);
  double grady = (G(ddx1, i) * (HA(ER, i, j + 1, k) - HA(ER, i, j - 1, k)) +
                  G(ddx0, i) * (HA(ER, i - 1, j + 1, k) - HA(ER, i - 1, j - 1, k))) /
                 (G(geoxga, i) * G(geozg, k) * (G(xyb, j + 1) - G(xyb, j - 1)));
  double gradz = (G(ddx1, i) * (HA(ER, i, j, k + 1) - HA(ER, i, j, k - 1)) +
                  G(ddx0, i) * (HA(ER, i - 1, j, k + 1) - HA(ER, i - 1, j, k - 1))) /
                 (G(geoxha, i) * (G(xzb, k + 1) - G(xzb, k - 1)));
  double grad = sqrt(gradx * gradx + grady * grady + gradz * gradz) + 1.0e-50;
  double rrx = 2.0 * grad /
               (HA(RHQX, i, j, k) *
                (G(ddx1, i) * (HA(XKAPR, i, j, k) + sg) + G(ddx0, i) * (HA(XKAPR, i - 1, j, k) + sg)) *
                (HA(ER, i, j, k) + HA(ER, i - 1, j, k)));
  return (2.0 + rrx) / (6.0 + 3.0 * rrx + rrx * rrx);
}

// FLIM's y loop body, pprphy.f:462-484.
__device__ __forceinline__ double flimy_calc(const Dev& d, int i, int j, int k) {
  const double sg = d.sigval;
  double gradx = (G(ddy1, j) * (HA(ER, i + 1, j, k) - HA(ER, i - 1, j, k)) +
                  G(ddy0, j) * (HA(ER, i + 1, j - 1, k) - HA(ER, i - 1, j - 1, k))) /
                 (G(xxb, i + 1) - G(xxb, i - 1));
  double grady = (HA(ER, i, j, k) - HA(ER, i, j - 1, k)) / (G(geoxg, i) * G(geozg, k) * G(dyb, j));
  double gradz = (G(ddy1, j) * (HA(ER, i, j, k + 1) - HA(ER, i, j, k - 1)) +
                  G(ddy0, j) * (HA(ER, i, j - 1, k + 1) - HA(ER, i, j - 1, k - 1))) /
                 ((G(xzb, k + 1) - G(xzb, k - 1)) * G(geoxh, i));
  double grad = sqrt(gradx * gradx + grady * grady + gradz * gradz) + 1.0e-50;
  double rry = 2.0 * grad /
               (HA(RHQY, i, j, k) *
                (G(ddy1, j) * (HA(XKAPR, i, j, k) + sg) + G(ddy0, j) * (HA(XKAPR, i, j - 1, k) + sg)) *
                (HA(ER, i, j, k) + HA(ER, i, j - 1, k)));
  return (2.0 + rry) / (6.0 + 3.0 * rry + rry * rry);
}

// FLIM's z loop body, pprphy.f:493-515.
__device__ __forceinline__ double flimz_calc(const Dev& d, int i, int j, int k) {
  const double sg = d.sigval;
  double gradx = (G(ddz1, k) * (HA(ER, i + 1, j, k) - HA(ER, i - 1, j, k)) +
                  G(ddz0, k) * (HA(ER, i + 1, j, k - 1) - HA(ER, i - 1, j, k - 1))) /
                 (G(xxb, i + 1) - G(xxb, i - 1));
  double grady = (G(ddz1, k) * (HA(ER, i, j + 1, k) - HA(ER, i, j - 1, k)) +
                  G(ddz0, k) * (HA(ER, i, j + 1, k - 1) - HA(ER, i, j - 1, k - 1))) /
                 ((G(xyb, j + 1) - G(xyb, j - 1)) * G(geoxg, i) * G(geozga, k));
  double gradz = (HA(ER, i, j, k) - HA(ER, i, j, k - 1)) / (G(geoxh, i) * G(dzb, k));
  double grad = sqrt(gradx * gradx + grady * grady + gradz * gradz) + 1.0e-50;
  double rrz = 2.0 * grad /
               (HA(RHQZ, i, j, k) *
                (G(ddz1, k) * (HA(XKAPR, i, j, k) + sg) + G(ddz0, k) * (HA(XKAPR, i, j, k - 1) + sg)) *
                (HA(ER, i, j, k) + HA(ER, i, j, k - 1)));
  return (2.0 + rrz) / (6.0 + 3.0 * rrz + rrz * rrz);
}

// FLIMX(i,j,k) as FLIM leaves it: formed for i <= UPPERBND-1 (:414-448),
// the value of UPPERBND-1 above (:449-454; re-formed here from the same
// inputs, so the same bits).  With UPPERBND <= 1 the face is neither formed
// nor copied and the array keeps its value.
__device__ __forceinline__ double flimx_at(const Dev& d, int i, int j, int k) {
  if (d.iflimtyp == 1) return 1.0 / 3.0;
  const int ub = PA(UB, j, k);
  if (i > ub - 1 && !(ub >= 2 && ub <= d.nx + 1)) return FA(FLIMX, i, j, k);
  return flimx_calc(d, i <= ub - 1 ? i : ub - 1, j, k);   // one inlined copy of the face
}

// The y and z loops form the faces up to the last x loop's xmax_index,
// UPPERBND(NY,NZ)-1 (:464, :495); the copies of :485-489 and :516-520 then
// give every face from UPPERBND(j,k) up the value of UPPERBND(j,k)-1.
// The face whose value face (i,j,k) ends with: itself, or UPPERBND-1 from
// UPPERBND up (one inlined copy of the face computation).
__device__ __forceinline__ int flim_source(const Dev& d, int i, int j, int k) {
  const int ub = PA(UB, j, k);
  return (ub >= 2 && ub <= d.nx + 1 && i >= ub) ? ub - 1 : i;
}
__device__ __forceinline__ double flimy_at(const Dev& d, int i, int j, int k) {
  if (d.iflimtyp == 1) return 1.0 / 3.0;
  const int is = flim_source(d, i, j, k);
  return is <= PA(UB, d.ny, d.nz) - 1 ? flimy_calc(d, is, j, k) : FA(FLIMY, is, j, k);
}
__device__ __forceinline__ double flimz_at(const Dev& d, int i, int j, int k) {
  if (d.iflimtyp == 1) return 1.0 / 3.0;
  const int is = flim_source(d, i, j, k);
  return is <= PA(UB, d.ny, d.nz) - 1 ? flimz_calc(d, is, j, k) : FA(FLIMZ, is, j, k);
}

// DIFF pprad.f:74-156, one face of each direction (with the ieta = 5 floor).
__device__ __forceinline__ double difrx_of(const Dev& d, int i, int j, int k, double fl) {
  const double sg = d.sigval;
  double v = TT_FD * fl /
             (G(dxb, i) * HA(RHQX, i, j, k) *
              (G(ddx1, i) * (HA(XKAPR, i, j, k) + sg) + G(ddx0, i) * (HA(XKAPR, i - 1, j, k) + sg)));
  if (d.ieta == 5) {
    double mn = HA(RHQX, i, j, k) * HA(CV, i, j, k) * d.xnue /
                (G(dxb, i) * 4.0 * TT_ARAD * p3(G(ddx1, i) * HA(T, i, j, k) + G(ddx0, i) * HA(T, i - 1, j, k)) *
                 d.pr_num);
    v = fmax(v, mn);
  }
  return v;
}
__device__ __forceinline__ double difry_of(const Dev& d, int i, int j, int k, double fl) {
  const double sg = d.sigval;
  double v = TT_FD * fl /
             (G(dyb, j) * G(geoxg, i) * G(geozg, k) * HA(RHQY, i, j, k) *
              (G(ddy1, j) * (HA(XKAPR, i, j, k) + sg) + G(ddy0, j) * (HA(XKAPR, i, j - 1, k) + sg)));
  if (d.ieta == 5) {
    double mn = HA(RHQY, i, j, k) * HA(CV, i, j, k) * d.xnue /
                (G(dyb, j) * G(geoxg, i) * G(geozg, k) * 4.0 * TT_ARAD *
                 p3(G(ddy1, j) * HA(T, i, j, k) + G(ddy0, j) * HA(T, i, j - 1, k)) * d.pr_num);
    v = fmax(v, mn);
  }
  return v;
}
__device__ __forceinline__ double difrz_of(const Dev& d, int i, int j, int k, double fl) {
  const double sg = d.sigval;
  double v = TT_FD * fl /
             (G(dzb, k) * G(geoxh, i) * HA(RHQZ, i, j, k) *
              (G(ddz1, k) * (HA(XKAPR, i, j, k) + sg) + G(ddz0, k) * (HA(XKAPR, i, j, k - 1) + sg)));
  if (d.ieta == 5) {
    double mn = HA(RHQZ, i, j, k) * HA(CV, i, j, k) * d.xnue /
                (G(dzb, k) * G(geoxh, i) * 4.0 * TT_ARAD *
                 p3(G(ddz1, k) * HA(T, i, j, k) + G(ddz0, k) * HA(T, i, j, k - 1)) * d.pr_num);
    v = fmax(v, mn);
  }
  return v;
}

// FLUX_X(i,j,k) as CALCULATEFLUX (ppenergy.f:880-920) and FLUX_BC (:922-982)
// leave it, for i = 1..NX+1, j = 1..NY, k = 1..NZ: the diffusive flux, the
// top value c E_R(UPPERBND-1)/2 from UPPERBND up, Fbottom on the first face.
__device__ __forceinline__ double fluxx_final(const Dev& d, int i, int j, int k, double difr) {
  double f = -difr * (HA(ER, i, j, k) - HA(ER, i - 1, j, k));
  const int ub = PA(UB, j, k);
  if (i >= ub && ub >= 1) f = TT_FD * HA(ER, ub - 1, j, k) / 2.0;
  if (i == 1) f = d.fbottom;
  return f;
}

// FLIM (MODE 0), FLIM + DIFF (1), or FLIM + DIFF + CALCULATEFLUX + FLUX_BC
// (2): one pass per direction over its faces, each face formed whole
// (limiter, diffusion coefficient, flux) by one thread.  KAPPA and QDENS,
// which FLIM calls for energy_iter <= 1 (pprphy.f:396-402), run first unless
// they already ran on the same T and rho in this step (skip_kappa /
// skip_qdens).
template <int MODE>
static int faces(ttfld_ctx* c, int energy_iter, bool skip_kappa, bool skip_qdens) {
  if (energy_iter <= 1) {
    int rc;
    if (!skip_kappa && (rc = kappa(c))) return rc;
    if (!skip_qdens && (rc = qdens(c))) return rc;
  }
  Dev d = c->d;
  launch_box(c->stream, box(1, d.nx + 1, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) {
    const double fl = flimx_at(d, i, j, k);
    FA(FLIMX, i, j, k) = fl;
    if (MODE >= 1) {
      const double dr = difrx_of(d, i, j, k, fl);
      FA(DIFRX, i, j, k) = dr;
      if (MODE == 2) FA(FLUXX, i, j, k) = fluxx_final(d, i, j, k, dr);
    }
  });
  TT_CHECK_LAUNCH();
  launch_box(c->stream, box(1, d.nx, 1, d.ny + 1, 1, d.nz), [=] __device__(int i, int j, int k) {
    const double fl = flimy_at(d, i, j, k);
    FA(FLIMY, i, j, k) = fl;
    if (MODE >= 1) {
      const double dr = difry_of(d, i, j, k, fl);
      FA(DIFRY, i, j, k) = dr;
      if (MODE == 2) {
        double f = -dr * (HA(ER, i, j, k) - HA(ER, i, j - 1, k));
        if (j <= d.ny) {  // FLUX_BC's loop covers j = 1..NY (:940-970)
          const int ub = PA(UB, j, k);
          if (i >= ub && ub >= 1) f = 0.0;
        }
        FA(FLUXY, i, j, k) = f;
      }
    }
  });
  TT_CHECK_LAUNCH();
  launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz + 1), [=] __device__(int i, int j, int k) {
    const double fl = flimz_at(d, i, j, k);
    FA(FLIMZ, i, j, k) = fl;
    if (MODE >= 1) {
      const double dr = difrz_of(d, i, j, k, fl);
      FA(DIFRZ, i, j, k) = dr;
      if (MODE == 2) {
        double f = -dr * (HA(ER, i, j, k) - HA(ER, i, j, k - 1));
        if (k <= d.nz) {
          const int ub = PA(UB, j, k);
          if (i >= ub && ub >= 1) f = 0.0;
        }
        FA(FLUXZ, i, j, k) = f;
      }
    }
  });
  TT_CHECK_LAUNCH();
  return 0;
}

static int diff(ttfld_ctx* c, int energy_iter, bool skip_kappa = false, bool skip_qdens = false) {
  return faces<1>(c, energy_iter, skip_kappa, skip_qdens);
}
static int calculateflux(ttfld_ctx* c, int energy_iter, bool skip_kappa = false, bool skip_qdens = false) {
  return faces<2>(c, energy_iter, skip_kappa, skip_qdens);
}

// The CALCULATEFLUX + FLUX_BC of COUPLED_ENERGY_EQS's set-up (ppenergy.f:
// 74-75) as far as the step reads it: its only reader is the upper boundary
// loop (:80-105), which takes FLUX_X at i >= UPPERBND(j,k), clamped into the
// array for ghost j, k, i = NX+2; the call at :253-255 forms every face again
// before anything else reads them.  Those faces are formed here from the
// same inputs (after KAPPA and QDENS, which that FLIM call runs): from
// UPPERBND up FLUX_BC's c E_R(UPPERBND-1)/2, below it (only reachable from a
// ghost column whose UPPERBND differs from its clamped neighbour's) the full
// FLIM, DIFF and flux of the face.
int asm_top_fluxes(ttfld_ctx* c, bool kappa_done) {
  int rc;
  if (!kappa_done && (rc = kappa(c))) return rc;
  if ((rc = qdens(c))) return rc;
  Dev d = c->d;
  launch_box(c->stream, box(1, d.nx + 2, -1, d.ny + 2, -1, d.nz + 2), [=] __device__(int i, int j, int k) {
    const int ub = PA(UB, j, k);
    if (i < ub || ub < 1) return;
    const int ic = i > d.nx + 1 ? d.nx + 1 : i;
    const int jc = j < 1 ? 1 : (j > d.ny ? d.ny : j);
    const int kc = k < 1 ? 1 : (k > d.nz ? d.nz : k);
    const int ubc = PA(UB, jc, kc);
    double f;
    if (ic >= ubc && ubc >= 1) f = ic == 1 ? d.fbottom : TT_FD * HA(ER, ubc - 1, jc, kc) / 2.0;
    else f = fluxx_final(d, ic, jc, kc, difrx_of(d, ic, jc, kc, flimx_at(d, ic, jc, kc)));
    FA(FLUXX, ic, jc, kc) = f;   // threads that meet on one face write the same value
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// FILL_EVALUES ppenergy.f:984-1030
static int fill_evalues(ttfld_ctx* c, double theta) {
  Dev d = c->d;
  launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) {
    const size_t q = cidx(d, i, j, k);
    store_evalues(d, q, evalues_cell(d, i, j, k, theta, d.ETA[q]));
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// CALCULATEDIVF_WITHF ppenergy.f:825-878, NCOSYS=2 (:853-867).  Its six
// factors are quotients of grid metrics alone, so they are formed once per
// context (the same operations on the same operands, so the same bits) and
// the divergence of a cell costs six products and five sums:
//   ax1(i) = surxa(i+1)/(surxb(i) dxa(i)),  ax0(i) = surxa(i)/(surxb(i) dxa(i)),
//   ay(i,j,k) = 1/(xxb(i) surzb(k) dya(j)),
//   az1(i,k) = surza(k+1)/(xxb(i) surzb(k) dza(k)),  az0(i,k) = surza(k)/(...).
DivfTab divf_tab(ttfld_ctx* c) {
  Dev d = c->d;
  const size_t nx = d.nx, nxz = (size_t)d.nx * d.nz;
  DivfTab t;
  t.ax1 = c->divf_tab;
  t.ax0 = t.ax1 + nx;
  t.az1 = t.ax0 + nx;
  t.az0 = t.az1 + nxz;
  t.ay = t.az0 + nxz;
  return t;
}

static int ensure_divf_tab(ttfld_ctx* c) {
  if (c->divf_tab) return 0;
  Dev d = c->d;
  const size_t n = 2 * (size_t)d.nx + 2 * (size_t)d.nx * d.nz + ncell(d);
  TT_CHECK(cudaMalloc((void**)&c->divf_tab, n * sizeof(double)));
  const DivfTab t = divf_tab(c);
  launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) {
    double xb = G(xxb, i), szb = G(surzb, k);
    if (j == 1 && k == 1) {
      t.ax1[i - 1] = G(surxa, i + 1) / (G(surxb, i) * G(dxa, i));
      t.ax0[i - 1] = G(surxa, i) / (G(surxb, i) * G(dxa, i));
    }
    if (j == 1) {
      t.az1[(i - 1) + (size_t)d.nx * (k - 1)] = G(surza, k + 1) / (xb * szb * G(dza, k));
      t.az0[(i - 1) + (size_t)d.nx * (k - 1)] = G(surza, k) / (xb * szb * G(dza, k));
    }
    t.ay[cidx(d, i, j, k)] = 1.0 / (xb * szb * G(dya, j));
  });
  TT_CHECK_LAUNCH();
  return 0;
}

void asm_free(ttfld_ctx* c) {
  if (c->divf_tab) cudaFree(c->divf_tab);
  c->divf_tab = nullptr;
}

int asm_prepare(ttfld_ctx* c) { return ensure_divf_tab(c); }

static int divf_withf(ttfld_ctx* c, double* out, double theta, bool fill = true) {
  int rc = ensure_divf_tab(c);
  if (rc) return rc;
  Dev d = c->d;
  const DivfTab t = divf_tab(c);
  launch_box(c->stream, box(1, d.nx, 1, d.ny, 1, d.nz), [=] __device__(int i, int j, int k) {
    out[cidx(d, i, j, k)] = divf_cell(d, t, i, j, k);
  });
  TT_CHECK_LAUNCH();
  return fill ? fill_evalues(c, theta) : 0;
}

// CALCSTELLARTAU pprad.f:191-221, STELLAR_DTAU :223-242 and the grey
// STELLARINPUT of STELLARINPUT_HEATING :490-502.  STELLARINPUT is declared
// (1:NX,-1:NY+2,-1:NZ+2) (ppmod.f:341); only i = 1..NX is formed.
// The wavelength-binned branch of STELLARINPUT_HEATING for IKAPTYP 20-24
// (pprad.f:433-448): WAVELENGTH_CALCSTELLARTAU (pprad.f:519-547, per bin the
// optical depth summed from UPPERBND inward, zero elsewhere; one thread per
// column and bin), then per cell WAVELENGTH_STELLAR_DTAU's central
// differences (:549-568, dtaus(1) = dtaus(2)) and the bins summed in order,
// times (RSTAR*RSOL/semi)**2 / dxb(i), for i = 1..NX.
static int stellar_binned(ttfld_ctx* c) {
  Dev d = c->d;
  const int nb = c->wave_nb;
  const size_t nh = nhalo(d);
  double* tau = c->stauw;
  const double* xkapw = c->xkapw;
  const double* bstar = c->wave + (size_t)c->opac_nt * c->opac_nrh * nb;
  TT_CHECK(cudaMemsetAsync(tau, 0, nh * nb * sizeof(double), c->stream));
  launch_box(c->stream, box(0, nb - 1, -1, d.ny + 2, -1, d.nz + 2), [=] __device__(int l, int j, int k) {
    const double dr = G(xxb, 2) - G(xxb, 1);
    int ub = PA(UB, j, k);
    if (ub > d.nx + 1) ub = d.nx + 1;
    const double* kw = xkapw + nh * l;
    double* tw = tau + nh * l;
    double tot = 0.0;
    for (int i = ub; i >= 1; --i) {
      const size_t q = hidx(d, i, j, k);
      tot = tot + (kw[q] * d.RH[q] * dr);
      tw[q] = tot;
    }
  });
  TT_CHECK_LAUNCH();
  const double f = c->wave_rstar * TT_RSOL / c->wave_semi;
  const double geo = f * f;
  launch_box(c->stream, box(1, d.nx, -1, d.ny + 2, -1, d.nz + 2), [=] __device__(int i, int j, int k) {
    const double mu = PA(MU, j, k);
    const int is = i < 2 ? 2 : i;
    const size_t q = hidx(d, i, j, k), qm = hidx(d, is - 1, j, k), qp = hidx(d, is + 1, j, k);
    double si = 0.0;
    for (int l = 0; l < nb; ++l) {
      const double* tw = tau + nh * l;
      const double dtaus = (tw[qm] - tw[qp]) / 2.0;
      si = si + bstar[l] * (exp(-tw[q] / mu)) * dtaus;
    }
    d.SI[q] = si * geo / G(dxb, i);
  });
  TT_CHECK_LAUNCH();
  return 0;
}

static int stellarinput_heating(ttfld_ctx* c) {
  Dev d = c->d;
  if (d.f_incident == 0) {
    TT_CHECK(cudaMemsetAsync(d.SI, 0, nhalo(d) * 8, c->stream));
    return 0;
  }
  if (c->wave && c->wave_nb > 0) {
    if (d.kappa_model != 2) {
      fprintf(stderr, "ttfld: the binned stellar heating needs kappa_model 2 (its per-bin opacities)\n");
      return TTFLD_E_UNSUPPORTED;
    }
    return stellar_binned(c);
  }
  launch_box(c->stream, box(0, 0, -1, d.ny + 2, -1, d.nz + 2), [=] __device__(int, int j, int k) {
    double dr = G(xxb, 2) - G(xxb, 1);
    int ub = PA(UB, j, k);
    if (ub > d.nx + 1) ub = d.nx + 1;
    if (ub < d.nx)
      for (int i = ub + 1; i <= d.nx + 1; ++i) HA(STAU, i, j, k) = 0.0;
    double tot = 0.0;
    for (int i = ub; i >= 1; --i) {
      tot = tot + (HA(XKAPA, i, j, k) * HA(RH, i, j, k) * dr);
      HA(STAU, i, j, k) = tot;
    }
  });
  TT_CHECK_LAUNCH();
  // STELLAR_DTAU and STELLARINPUT of the same cell in one pass
  launch_box(c->stream, box(1, d.nx + 1, -1, d.ny + 2, -1, d.nz + 2), [=] __device__(int i, int j, int k) {
    int is = i < 2 ? 2 : (i > d.nx ? d.nx : i);  // dtaus(1)=dtaus(2), dtaus(NX+1)=dtaus(NX)
    const double dtaus = (HA(STAU, is - 1, j, k) - HA(STAU, is + 1, j, k)) / 2.0;
    HA(DTAUS, i, j, k) = dtaus;
    if (i > d.nx) return;
    double tinc = PA(TINC, j, k), mu = PA(MU, j, k);
    HA(SI, i, j, k) = TT_SBCONST * (p4(tinc) / mu) * (exp(-HA(STAU, i, j, k) / mu)) * dtaus / G(dxb, i);
  });
  TT_CHECK_LAUNCH();
  return 0;
}

// BOUNDS ppbou.f:1-92 for MODTYP=2 (MODVER 0,2-5), T/RH/UPPERBND only:
// UPPERBND from density (ppbou.f:124-138), PASSUPPERBND one rank
// (ppbou.f:522-682), BOUNDXMIN(9) (:1029-1049), BOUNDXMAX(2) (:1269-1384),
// BOUNDZMIN(0)/BOUNDZMAX(0) (:1833-1846, :1946-1958), PLANETSHIFT(1..2).
static int bounds(ttfld_ctx* c) {
  Dev d = c->d;
  int rc;
  if (d.bcxmin != 9) return TTFLD_E_UNSUPPORTED;
  if ((rc = halo_shift(c, d.T)) || (rc = halo_shift(c, d.RH))) return rc;
  if ((rc = pole_shift(c, d.T)) || (rc = pole_shift(c, d.RH))) return rc;
  launch_box(c->stream, box(0, 0, 1, d.ny, 1, d.nz), [=] __device__(int, int j, int k) {
    int ub = d.nx - 1;
    for (int i = 1; i <= d.nx; ++i)
      if (HA(RH, i, j, k) < (double)1.0e-9f) { ub = i; break; }
    PA(UB, j, k) = ub;
  });
  TT_CHECK_LAUNCH();
  // PASSUPPERBND one rank: j ghosts by wrap for k = 1..NZ, then edges.
  launch_box(c->stream, box(0, 0, 0, 0, 1, d.nz), [=] __device__(int, int, int k) {
    PA(UB, 0, k) = PA(UB, d.ny, k); PA(UB, -1, k) = PA(UB, d.ny - 1, k);
    PA(UB, d.ny + 1, k) = PA(UB, 1, k); PA(UB, d.ny + 2, k) = PA(UB, 2, k);
  });
  TT_CHECK_LAUNCH();
  launch_box(c->stream, box(0, 0, -1, d.ny + 2, 0, 0), [=] __device__(int, int j, int) {
    const int nz = d.nz;
    PA(UB, j, 0) = PA(UB, j, 1); PA(UB, j, -1) = PA(UB, j, 1);
    PA(UB, j, nz + 1) = PA(UB, j, nz); PA(UB, j, nz + 2) = PA(UB, j, nz);
  });
  TT_CHECK_LAUNCH();
  // BOUNDXMIN(9); at III = 0 the opacity of cell (1,1,1) comes from the
  // opacity table (ppbou.f:1040-1044) where kappa_model 2 has one, else from
  // the analytic model
  const bool tab = d.kappa_model == 2 && c->opac;
  const OpacTab tb = tab ? opac_tab(c) : OpacTab{};
  launch_box(c->stream, box(0, 0, -1, d.ny + 2, -1, d.nz + 2), [=] __device__(int, int j, int k) {
    double dtdr;
    if (d.ieta == 5) {
      dtdr = -d.fbottom / (HA(RH, 1, j, k) * HA(CV, 1, j, k) * (d.xnue / d.pr_num));
    } else if (d.iii > 0) {
      dtdr = -(3.0 * d.fbottom * HA(XKAPR, 1, j, k) * HA(RH, 1, j, k) /
               (4.0 * TT_ARAD * TT_FD * p3(HA(T, 1, j, k))));
    } else {
      double k111 = kap_formula(d, HA(T, 1, 1, 1), HA(RH, 1, 1, 1), HA(KMUL, 1, 1, 1));
      if (tab) {
        double kp, ka, dkp, dka;
        if (burrows_opc(tb, HA(T, 1, 1, 1), HA(RH, 1, 1, 1), kp, k111, ka, dkp, dka)) atomicExch(tb.err, 5);
      }
      dtdr = -(3.0 * d.fbottom * k111 * HA(RH, 1, 1, 1) / (4.0 * TT_ARAD * TT_FD * p3(HA(T, 1, 1, 1))));
    }
    HA(T, 0, j, k) = HA(T, 1, j, k) - dtdr * (G(xxb, 1) - G(xxb, 0));
    HA(T, -1, j, k) = HA(T, 1, j, k) - dtdr * (G(xxb, 1) - G(xxb, -1));
  });
  TT_CHECK_LAUNCH();
  // BOUNDXMAX(2)
  launch_box(c->stream, box(0, 0, 1, d.ny, 1, d.nz), [=] __device__(int, int j, int k) {
    int ub = PA(UB, j, k);
    double tj;
    if (d.ibdrad == 9) {
      if (d.iii <= 1)
        tj = HA(T, ub - 1, j, k);
      else
        tj = pow((HA(ER, ub - 1, j, k) / TT_ARAD) +
                     (HA(SI, ub - 1, j, k) / (4.0 * TT_SBCONST * HA(RH, ub - 1, j, k) * HA(XKAPP, ub - 1, j, k))),
                 0.25);
    } else if (d.ibdrad == 7) {
      tj = HA(T, ub - 1, j, k);
    } else {
      tj = d.tirr;
    }
    HA(T, ub, j, k) = tj;
    for (int i = ub + 1; i <= d.nx + 2; ++i) {
      HA(T, i, j, k) = tj;
      HA(RH, i, j, k) = (double)1.0e-10f;
    }
    if (ub == d.nx) { HA(RH, d.nx, j, k) = (double)1.0e-10f; HA(T, d.nx, j, k) = tj; }
  });
  TT_CHECK_LAUNCH();
  // BOUNDZMIN(0) then BOUNDZMAX(0), without poles only (ppbou.f:188-193)
  if (!d.poles) launch_box(c->stream, box(-1, d.nx + 2, -1, d.ny + 2, 0, 0), [=] __device__(int i, int j, int) {
    const int nz = d.nz;
    HA(RH, i, j, 1) = HA(RH, i, j, 2); HA(RH, i, j, 0) = HA(RH, i, j, 1); HA(RH, i, j, -1) = HA(RH, i, j, 1);
    HA(T, i, j, 1) = HA(T, i, j, 2); HA(T, i, j, 0) = HA(T, i, j, 1); HA(T, i, j, -1) = HA(T, i, j, 1);
    HA(RH, i, j, nz) = HA(RH, i, j, nz - 1); HA(RH, i, j, nz + 1) = HA(RH, i, j, nz);
    HA(RH, i, j, nz + 2) = HA(RH, i, j, nz);
    HA(T, i, j, nz) = HA(T, i, j, nz - 1); HA(T, i, j, nz + 1) = HA(T, i, j, nz);
    HA(T, i, j, nz + 2) = HA(T, i, j, nz);
  });
  TT_CHECK_LAUNCH();
  if ((rc = halo_shift(c, d.T)) || (rc = halo_shift(c, d.RH))) return rc;
  if ((rc = pole_shift(c, d.T)) || (rc = pole_shift(c, d.RH))) return rc;
  return 0;
}

// ---- exported to the step driver ---------------------------------------
int asm_kappa(ttfld_ctx* c) { return kappa(c); }
int asm_calculateflux(ttfld_ctx* c, int energy_iter, bool skip_kappa, bool skip_qdens) {
  return calculateflux(c, energy_iter, skip_kappa, skip_qdens);
}
int asm_fill_evalues(ttfld_ctx* c, double theta) { return fill_evalues(c, theta); }
int asm_divf(ttfld_ctx* c, double* out, double theta, bool fill) { return divf_withf(c, out, theta, fill); }
int asm_stellar(ttfld_ctx* c) { return stellarinput_heating(c); }
int asm_bounds(ttfld_ctx* c) { return bounds(c); }
int asm_diff(ttfld_ctx* c, int energy_iter) { return diff(c, energy_iter); }

}  // namespace ttfld

using namespace ttfld;

extern "C" {

int ttfld_bounds(ttfld_ctx* c) {
  if (!c) return TTFLD_E_ARGS;
  int rc = bounds(c);
  if (rc) return rc;
  TT_CHECK(cudaStreamSynchronize(c->stream));
  return 0;
}

int ttfld_kappa(ttfld_ctx* c) {
  if (!c) return TTFLD_E_ARGS;
  int rc = kappa(c);
  if (rc) return rc;
  TT_CHECK(cudaStreamSynchronize(c->stream));
  return 0;
}

int ttfld_stellarinput_heating(ttfld_ctx* c) {
  if (!c) return TTFLD_E_ARGS;
  int rc = stellarinput_heating(c);
  if (rc) return rc;
  TT_CHECK(cudaStreamSynchronize(c->stream));
  return 0;
}

int ttfld_set_opacity_table(ttfld_ctx* c, const ttfld_opacity_table* t) {
  if (!c || !t || t->nt < 2 || t->nrh < 2 || !t->log_t || !t->log_rho || !t->log_ross || !t->log_plnk ||
      !t->log_abs)
    return TTFLD_E_ARGS;
  const size_t nn = (size_t)t->nt * t->nrh;
  const size_t bytes = (1 + (size_t)t->nt + t->nrh + 3 * nn) * sizeof(double);
  TT_CHECK(cudaSetDevice(c->device));
  if (c->opac) {
    TT_CHECK(cudaStreamSynchronize(c->stream));
    cudaFree(c->opac);
    c->opac = nullptr;
  }
  TT_CHECK(cudaMalloc(&c->opac, bytes));
  c->opac_nt = t->nt;
  c->opac_nrh = t->nrh;
  double* p = (double*)c->opac + 1;
  TT_CHECK(cudaMemcpy(p, t->log_t, t->nt * sizeof(double), cudaMemcpyHostToDevice));
  p += t->nt;
  TT_CHECK(cudaMemcpy(p, t->log_rho, t->nrh * sizeof(double), cudaMemcpyHostToDevice));
  p += t->nrh;
  TT_CHECK(cudaMemcpy(p, t->log_ross, nn * sizeof(double), cudaMemcpyHostToDevice));
  p += nn;
  TT_CHECK(cudaMemcpy(p, t->log_plnk, nn * sizeof(double), cudaMemcpyHostToDevice));
  p += nn;
  TT_CHECK(cudaMemcpy(p, t->log_abs, nn * sizeof(double), cudaMemcpyHostToDevice));
  return TTFLD_OK;
}

int ttfld_set_wave_table(ttfld_ctx* c, const ttfld_wave_table* t) {
  if (!c || !t || t->nbins < 0) return TTFLD_E_ARGS;
  TT_CHECK(cudaSetDevice(c->device));
  TT_CHECK(cudaStreamSynchronize(c->stream));
  if (c->wave) { cudaFree(c->wave); c->wave = nullptr; }
  if (c->xkapw) { cudaFree(c->xkapw); c->xkapw = nullptr; c->stauw = nullptr; }
  c->wave_nb = 0;
  if (t->nbins == 0) return TTFLD_OK;
  if (!c->opac || !t->log_waveopac || !t->bstar_bin || !(t->semi > 0.0)) return TTFLD_E_ARGS;
  const size_t nn = (size_t)c->opac_nt * c->opac_nrh * t->nbins;
  TT_CHECK(cudaMalloc((void**)&c->wave, (nn + t->nbins) * sizeof(double)));
  TT_CHECK(cudaMemcpy(c->wave, t->log_waveopac, nn * sizeof(double), cudaMemcpyHostToDevice));
  TT_CHECK(cudaMemcpy(c->wave + nn, t->bstar_bin, t->nbins * sizeof(double), cudaMemcpyHostToDevice));
  const size_t nh = nhalo(c->d);
  TT_CHECK(cudaMalloc((void**)&c->xkapw, 2 * nh * t->nbins * sizeof(double)));
  TT_CHECK(cudaMemset(c->xkapw, 0, 2 * nh * t->nbins * sizeof(double)));
  c->stauw = c->xkapw + nh * t->nbins;
  c->wave_nb = t->nbins;
  c->wave_rstar = t->rstar;
  c->wave_semi = t->semi;
  return TTFLD_OK;
}

int ttfld_set_freedman_table(ttfld_ctx* c, const ttfld_freedman_table* t) {
  if (!c || !t || !t->log_ross || !t->log_plnk || !t->log_abs || !(t->mu_gas > 0.0)) return TTFLD_E_ARGS;
  TT_CHECK(cudaSetDevice(c->device));
  TT_CHECK(cudaStreamSynchronize(c->stream));
  if (!c->freed) TT_CHECK(cudaMalloc((void**)&c->freed, (1 + 3 * 42 * 18) * sizeof(double)));
  TT_CHECK(cudaMemcpy(c->freed + 1, t->log_ross, 42 * 18 * sizeof(double), cudaMemcpyHostToDevice));
  TT_CHECK(cudaMemcpy(c->freed + 1 + 42 * 18, t->log_plnk, 42 * 18 * sizeof(double), cudaMemcpyHostToDevice));
  TT_CHECK(cudaMemcpy(c->freed + 1 + 2 * 42 * 18, t->log_abs, 42 * 18 * sizeof(double), cudaMemcpyHostToDevice));
  c->freed_mu = t->mu_gas;
  return TTFLD_OK;
}

int ttfld_diff(ttfld_ctx* c, int energy_iter) {
  if (!c) return TTFLD_E_ARGS;
  int rc = diff(c, energy_iter);
  if (rc) return rc;
  TT_CHECK(cudaStreamSynchronize(c->stream));
  return 0;
}

int ttfld_calculateflux(ttfld_ctx* c, int energy_iter) {
  if (!c) return TTFLD_E_ARGS;
  int rc = calculateflux(c, energy_iter);
  if (rc) return rc;
  TT_CHECK(cudaStreamSynchronize(c->stream));
  return 0;
}

int ttfld_fill_evalues(ttfld_ctx* c, double theta) {
  if (!c) return TTFLD_E_ARGS;
  int rc = fill_evalues(c, theta);
  if (rc) return rc;
  TT_CHECK(cudaStreamSynchronize(c->stream));
  return 0;
}

}  // extern "C"
