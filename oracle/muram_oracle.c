/* CPU restatement of MURaM's MHD time-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY: this file is the oracle the GPU library is checked
 * against.  It is never linked into the product; only tests/, the smoke check
 * and the benchmark's CPU-baseline leg load it.
 *
 * Parity is pinned against the reference itself: tests compare every routine
 * here bit-for-bit with the reference sources compiled unchanged (see
 * oracle/refbuild) on the same inputs, through committed golden fixtures.
 *
 * Each routine cites the reference function whose arithmetic it restates.
 * Expressions are written in the reference's evaluation order so that, built
 * with -ffp-contract=off, every intermediate rounds identically.
 * smax/smin follow std::max/std::min (first argument wins ties and NaNs);
 * fmax/fmin are the C library functions the reference calls by those names.
 */
#include "muram_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define NV 8
#define GH 2

static inline double smax(double a, double b) { return (a < b) ? b : a; }
static inline double smin(double a, double b) { return (b < a) ? b : a; }
static inline int imin(int a, int b) { return a < b ? a : b; }
static inline int imax(int a, int b) { return a > b ? a : b; }

struct mo_eos {
  int N_eps, N_lr, N_lp3, N_s3;
  double del_eps, del_lr, inv_del_eps, inv_del_lr, eps_off, ss_off;
  double *xeps, *xlr;
  float* tab[6]; /* [i_eps*N_lr + j_rho]: ln p, ln T, s, ln ne, ln rhoi, ln amb (pre-divided) */
  /* inverse tables over (ln p, s): [i_lp*N_s3 + j_s], ln eps and ln rho (pre-divided) */
  double del_lp3, del_s3, inv_del_lp3, inv_del_s3;
  double *xlp3, *xs3;
  float *eps3, *d3;
};

/* Geometry helpers */
typedef struct { int sx, sy, sz; long N; } geom;
static inline geom geom_of(const mo_params* p) {
  geom g;
  g.sx = p->nx + 2 * GH;
  g.sy = p->ny + 2 * GH;
  g.sz = p->nz + 2 * GH;
  g.N = (long)g.sx * g.sy * g.sz;
  return g;
}
static inline long at(const geom* g, int i, int j, int k) { return (long)i + (long)g->sx * ((long)j + (long)g->sy * k); }

void mo_default_params(mo_params* p, int nx, int ny, int nz, double dx) {
  memset(p, 0, sizeof *p);
  p->nx = nx; p->ny = ny; p->nz = nz;
  p->periodic_x = 1;
  p->dx[0] = p->dx[1] = p->dx[2] = dx;
  p->CFL = 0.8; p->CFL_tvd = 0.95; p->dt = 0.0; p->autostep = 1;
  p->grav = 0.0; p->va_max = 1e7; p->va_adjust = 0.0; p->max_fill = 1000.;
  for (int i = 0; i < 4; i++) { p->tvd_h[i] = 2.0; p->tvd_cs[i] = 0.2; p->tvd_coeff[i] = 1.0; }
  p->tvd[0] = 1.0e-11; p->tvd[1] = 1.0; p->tvd[2] = 10.0; p->tvd[3] = 0.2; p->tvd[4] = 1.0;
  p->tvd[5] = 1.0; p->tvd[6] = 1.0; p->tvd[7] = 1.0; p->tvd[8] = 0.75; p->tvd[9] = 100.0;
  p->tvd_h_bnd[0] = p->tvd_h_bnd[1] = 1e-6;
  p->tvd_visc_bnd[0] = p->tvd_visc_bnd[1] = 1.0;
  p->tvd_eta_bnd[0] = p->tvd_eta_bnd[1] = 1.0;
  p->tchk[0] = 1.0e11; p->tchk[1] = 1.0e-16; p->tchk[2] = 4.0e15; p->tchk[3] = 100.0e5;
  p->rt_cfl = 0.5; p->rt_tstep = 0.0; p->rt_update = 1;
  p->tau0 = 1.0; p->dt_rad = 1e9;
  p->v_lim = 0.0; p->e_lim = 0.0; p->va_ini_flag = 1;
  p->divB_next_iter = 3;
  p->bnd_bcrit = 1.0e10;
  p->p_bc = -1.0; p->s_bc = -1.0;
  p->bnd_ini = 1;
}

/* ---------------------------------------------------------------- EOS load */
/* Follows eos_init (src/eos_init.C:57-212): axes in double from the float
 * header, table entries divided by del_eps*del_lr in double and stored as float. */
mo_eos* mo_eos_load(const char* path) {
  FILE* f = fopen(path, "rb");
  if (!f) return NULL;
  float h[14];
  if (fread(h, sizeof(float), 14, f) != 14) { fclose(f); return NULL; }
  mo_eos* e = (mo_eos*)calloc(1, sizeof *e);
  e->N_eps = (int)h[0]; e->N_lr = (int)h[1]; e->N_lp3 = (int)h[2]; e->N_s3 = (int)h[3];
  double eps0 = (double)h[4], eps1 = (double)h[5], lr0 = (double)h[6], lr1 = (double)h[7];
  e->eps_off = (double)h[12];
  e->ss_off = (double)h[13];
  e->del_eps = (eps1 - eps0) / ((double)(e->N_eps - 1));
  e->del_lr = (lr1 - lr0) / ((double)(e->N_lr - 1));
  e->inv_del_eps = 1.0 / e->del_eps;
  e->inv_del_lr = 1.0 / e->del_lr;
  e->xeps = (double*)malloc(sizeof(double) * e->N_eps);
  e->xlr = (double*)malloc(sizeof(double) * e->N_lr);
  for (int i = 0; i < e->N_eps; i++) e->xeps[i] = eps0 + e->del_eps * ((double)i);
  for (int i = 0; i < e->N_lr; i++) e->xlr[i] = lr0 + e->del_lr * ((double)i);
  long n = (long)e->N_eps * e->N_lr;
  float* buf = (float*)malloc(sizeof(float) * 6 * n);
  if (fread(buf, sizeof(float), 6 * n, f) != (size_t)(6 * n)) {
    free(buf); fclose(f); mo_eos_free(e); return NULL;
  }
  const double scale = e->del_eps * e->del_lr;
  for (int t = 0; t < 6; t++) {
    e->tab[t] = (float*)malloc(sizeof(float) * n);
    for (int i = 0; i < e->N_eps; i++)
      for (int j = 0; j < e->N_lr; j++)
        e->tab[t][(long)i * e->N_lr + j] = (float)(((double)buf[t * n + (long)j * e->N_eps + i]) / scale);
  }
  free(buf);
  /* inverse tables (src/eos_init.C:120-136, 181-198); missing ones leave them unset */
  const double lp0 = (double)h[8], lp1 = (double)h[9], s0 = (double)h[10], s1 = (double)h[11];
  e->del_lp3 = (lp1 - lp0) / ((double)(e->N_lp3 - 1));
  e->del_s3 = (s1 - s0) / ((double)(e->N_s3 - 1));
  e->inv_del_lp3 = 1.0 / e->del_lp3;
  e->inv_del_s3 = 1.0 / e->del_s3;
  const long n3 = (long)e->N_lp3 * e->N_s3;
  if (n3 > 0) {
    float* b3 = (float*)malloc(sizeof(float) * 2 * n3);
    if (fread(b3, sizeof(float), 2 * n3, f) == (size_t)(2 * n3)) {
      e->xlp3 = (double*)malloc(sizeof(double) * e->N_lp3);
      e->xs3 = (double*)malloc(sizeof(double) * e->N_s3);
      for (int i = 0; i < e->N_lp3; i++) e->xlp3[i] = lp0 + e->del_lp3 * ((double)i);
      for (int i = 0; i < e->N_s3; i++) e->xs3[i] = s0 + e->del_s3 * ((double)i);
      e->eps3 = (float*)malloc(sizeof(float) * n3);
      e->d3 = (float*)malloc(sizeof(float) * n3);
      const double sc3 = e->del_lp3 * e->del_s3;
      for (int i = 0; i < e->N_lp3; i++)
        for (int j = 0; j < e->N_s3; j++) {
          e->eps3[(long)i * e->N_s3 + j] = (float)(((double)b3[(long)j * e->N_lp3 + i]) / sc3);
          e->d3[(long)i * e->N_s3 + j] = (float)(((double)b3[n3 + (long)j * e->N_lp3 + i]) / sc3);
        }
    }
    free(b3);
  }
  fclose(f);
  return e;
}

void mo_eos_free(mo_eos* e) {
  if (!e) return;
  free(e->xeps); free(e->xlr);
  for (int t = 0; t < 6; t++) free(e->tab[t]);
  free(e->xlp3); free(e->xs3); free(e->eps3); free(e->d3);
  free(e);
}

int mo_eos_dims(const mo_eos* e, int* d) {
  d[0] = e->N_eps; d[1] = e->N_lr; d[2] = e->N_lp3; d[3] = e->N_s3;
  return 0;
}

/* --------------------------------------------------------------- SaveCons */
void mo_save_cons(const mo_params* p, const double* U, double* U0) {
  geom g = geom_of(p);
  for (int v = 0; v < NV; v++)
    for (int k = GH; k < GH + p->nz; k++)
      for (int j = GH; j < GH + p->ny; j++)
        for (int i = GH; i < GH + p->nx; i++) {
          long c = at(&g, i, j, k);
          U0[v * g.N + c] = U[v * g.N + c];
        }
}

/* ------------------------------------------------------------- ConsToPrim */
static const double EOS_GAMMA = 1.65, EOS_MU = 0.62, EOS_MU_N = 1.3;
static const double M_HYD = 1.67262158e-24, K_BOLTZ = 1.380622e-16, R_GAS = 8.314e7;

static int invalid_pos(double a) { return (a != a) || (a <= 0.) || (a == INFINITY); }

void mo_cons_to_prim(const mo_params* p, const mo_eos* eos, double* U, double* pres, double* temp,
                     double* ne, double* rhoi, double* amb) {
  geom g = geom_of(p);
  const double eps_max = exp(eos->xeps[eos->N_eps - 1]) - eos->eps_off;
  volatile double gm1 = EOS_GAMMA - 1.;
  const double c_temp = gm1 * EOS_MU / R_GAS;
  const double c_pres = gm1;
  const double mun_mh = EOS_MU_N * M_HYD;
  const int NL = eos->N_lr;
  for (long c = 0; c < g.N; c++) {
    double d = U[c];
    double dn = 1.0 / d;
    double v1 = U[g.N + c] * dn, v2 = U[2 * g.N + c] * dn, v3 = U[3 * g.N + c] * dn;
    double vv = v1 * v1 + v2 * v2 + v3 * v3;
    double ei = U[4 * g.N + c] - 0.5 * vv * d;
    double eps = ei * dn + eos->eps_off;
    double lgr = log(d);
    double ep = log(eps);
    double lr = lgr;
    int i_d = (int)((lr - eos->xlr[0]) * eos->inv_del_lr);
    i_d = imax(0, i_d);
    i_d = imin(eos->N_lr - 2, i_d);
    int i_e = (int)((ep - eos->xeps[0]) * eos->inv_del_eps);
    i_e = imax(0, i_e);
    i_e = imin(eos->N_eps - 2, i_e);
    double c0 = (ep - eos->xeps[i_e]) * (lr - eos->xlr[i_d]);
    double c1 = (ep - eos->xeps[i_e]) * (eos->xlr[i_d + 1] - lr);
    double c2 = (eos->xeps[i_e + 1] - ep) * (lr - eos->xlr[i_d]);
    double c3 = (eos->xeps[i_e + 1] - ep) * (eos->xlr[i_d + 1] - lr);
    long a11 = (long)(i_e + 1) * NL + (i_d + 1), a10 = (long)(i_e + 1) * NL + i_d;
    long a01 = (long)i_e * NL + (i_d + 1), a00 = (long)i_e * NL + i_d;
    double out[6];
    for (int t = 0; t < 6; t++) {
      if (t == 2) continue;
      const float* T = eos->tab[t];
      double s = c0 * (double)T[a11];
      s += c1 * (double)T[a10];
      s += c2 * (double)T[a01];
      s += c3 * (double)T[a00];
      out[t] = exp(s);
    }
    double pr = out[0], tm = out[1], nl = out[3];
    if (lgr < eos->xlr[0]) {
      pr = c_pres * ei;
      tm = c_temp * eps;
      nl = pr / (tm * K_BOLTZ) - d / mun_mh;
    }
    if (eps > 0.8 * eps_max) {
      double xx = smax(0.0, 5.0 * (eps_max - eps) / eps_max);
      pr = pr * xx + (1.0 - xx) * c_pres * ei;
      tm = tm * xx + (1.0 - xx) * c_temp * eps;
      nl = pr / (tm * K_BOLTZ) - d / mun_mh;
    }
    if (invalid_pos(pr) || invalid_pos(tm)) {
      pr = c_pres * ei;
      tm = c_temp * eps;
    }
    if (nl == INFINITY) nl = pr / (tm * K_BOLTZ) - d / mun_mh;
    if ((nl < 1.0) || (nl != nl) || (nl == INFINITY)) nl = 1.0;
    U[g.N + c] = v1; U[2 * g.N + c] = v2; U[3 * g.N + c] = v3; U[4 * g.N + c] = ei;
    pres[c] = pr;
    if (temp) temp[c] = tm;
    if (ne) ne[c] = nl;
    if (rhoi) rhoi[c] = out[4];
    if (amb) amb[c] = out[5];
  }
}

/* --------------------------------------------------------- Adjust_Valf_Max */
void mo_adjust_valf_max(mo_params* p, const double* U, const double* pres, double* stats) {
  geom g = geom_of(p);
  double m0 = 0.0, m1 = 0.0, m2 = 0.0, s0 = 0.0, s1 = 0.0;
  for (int k = GH; k < GH + p->nz; k++)
    for (int j = GH; j < GH + p->ny; j++)
      for (int i = GH; i < GH + p->nx; i++) {
        long c = at(&g, i, j, k);
        double mx = U[g.N + c], my = U[2 * g.N + c], mz = U[3 * g.N + c];
        double vv = sqrt(mx * mx + my * my + mz * mz);
        double ee = U[4 * g.N + c] / U[c];
        m0 = fmax(m0, vv);
        m1 = fmax(m1, 5 / 3. * pres[c] / U[c]);
        m2 = fmax(m2, ee);
        if (vv >= p->v_lim * 0.95) s0 += 1.0;
        if (ee >= p->e_lim * 0.95) s1 += 1.0;
      }
  if (stats) { stats[0] = m0; stats[1] = m1; stats[2] = m2; stats[3] = s0; stats[4] = s1; }
  double gmax0 = m0, gmax1 = sqrt(m1), gmax2 = m2;
  double va_max;
  if (p->va_adjust > 0.0) {
    const double cs_fac = 2.0, vv_fac = 3.0, eps_decay = 0.99;
    if (p->va_ini_flag) {
      p->v_lim = fmin(gmax0, p->tchk[3]);
      p->e_lim = fmin(gmax2, p->tchk[2]);
      p->va_max_old = 0.0;
      p->va_ini_flag = 0;
    } else {
      if (s0 >= 4 * p->max_fill) p->v_lim *= 1.04;
      else if (s0 >= p->max_fill) p->v_lim *= 1.01;
      else if (s0 < 0.5 * p->max_fill) p->v_lim *= 0.99;
      if (s1 >= 4 * p->max_fill) p->e_lim *= 1.04;
      else if (s1 >= p->max_fill) p->e_lim *= 1.01;
      else if (s1 < 0.5 * p->max_fill) p->e_lim *= 0.99;
    }
    va_max = fmax(p->va_max, p->va_adjust * vv_fac * gmax0);
    va_max = fmax(va_max, p->va_adjust * cs_fac * gmax1);
    va_max = fmax(va_max, p->va_max_old * eps_decay);
    p->v_lim = fmax(p->v_lim, p->va_max / vv_fac);
    p->v_lim = fmin(p->v_lim, p->tchk[3]);
    p->e_lim = fmax(p->e_lim, pow(p->va_max / cs_fac, 2));
    p->e_lim = fmin(p->e_lim, p->tchk[2]);
  } else {
    va_max = p->va_max;
    p->v_lim = p->tchk[3];
    p->e_lim = p->tchk[2];
  }
  p->inv_va2max = 1.0 / pow(va_max, 2);
  p->va_max_old = va_max;
}

/* ------------------------------------------------------------ MHD_Residual */
/* Per direction d1 (order x, y, z), each 1-D pencil along d1 over the interior
 * of the two other dimensions: fluxes at every pencil point, 4th-order central
 * derivative, Lorentz force blended between Maxwell stress and curl B x B by
 * the Boris factor, accumulated into R.  cmax covers every pencil point. */
double mo_mhd_residual_ex(const mo_params* p, const double* U, const double* pres, const double* temp, double* R,
                          mo_fields* f) {
  geom g = geom_of(p);
  const int n[3] = {p->nx, p->ny, p->nz};
  const long st[3] = {1, g.sx, (long)g.sx * g.sy};
  static const int order[3][3] = {{0, 1, 2}, {1, 0, 2}, {2, 0, 1}};
  double dxmin = p->dx[0];
  for (int d = 1; d < 3; d++) dxmin = smin(dxmin, p->dx[d]);
  const double inv_va2max = p->inv_va2max;
  double cmax = 0.0;
  int L = 0;
  for (int d = 0; d < 3; d++) L = imax(L, n[d] + 2 * GH);
  double* var = (double*)malloc(sizeof(double) * NV * L);
  double* flx = (double*)malloc(sizeof(double) * NV * L);
  double* ms = (double*)malloc(sizeof(double) * 3 * L);
  double* lf1 = (double*)malloc(sizeof(double) * L);
  /* resistivity (src/mhdres_SR.C:58-61, 112-118, 422-450, 741-765, 815-819):
   * Grid.curlB starts at zero and accumulates the curl over the direction
   * passes; in the last pass R.e gets the ohmic heating eta*|curlB|^2 before
   * that pass's residual, and in every pass B gets eta times the fourth-order
   * second derivative along the pass direction */
  const double eta = p->eta;
  const int needs_curlB = eta > 0.0;
  double* curlB = needs_curlB ? (double*)calloc((size_t)3 * g.N, sizeof(double)) : NULL;
  static const double sgn[3] = {-1., 1., -1.};
  /* hyperbolic Spitzer conduction (src/mhdres_SR.C:33-46, 121-145, 251-253,
   * 355-358, 492-521, 668-692): the heat flux sflx along B enters the energy
   * flux; BgradT accumulates B.grad(T) over the passes, Rflx a hyperdiffusion
   * of sflx per pass and, in the last pass, the relaxation towards the
   * saturated Spitzer flux.  cmax_hyp and friends come from the previous dt. */
  const int spitzer = p->spitzer > 0.0 && f && f->sflx;
  const double CFL_hyp = 1.8, avr_max = 0.25, eps_hyp = 0.02;
  const double k0_spt = p->spitzer;
  const double Rgas = 8.314e7, X_H = 0.7;
  const double sat_flx = (1.0 + X_H) * pow(Rgas, 1.5) * sqrt(1836.) / 8.0;
  double cmax_hyp, nu_hyp_max, hyp_diff;
  if (p->dt > 0.0) {
    cmax_hyp = smin(p->CFL, CFL_hyp) * dxmin / p->dt;
    nu_hyp_max = avr_max / p->dt;
    hyp_diff = eps_hyp / p->dt;
  } else {
    cmax_hyp = 0.0;
    nu_hyp_max = avr_max * cmax_hyp / (smin(p->CFL, CFL_hyp) * dxmin);
    hyp_diff = eps_hyp * cmax_hyp / (smin(p->CFL, CFL_hyp) * dxmin);
  }
  const int dg = p->need_diagnostics && p->diag;
  double* sfl = (double*)malloc(sizeof(double) * L);
  double* vvl = (double*)malloc(sizeof(double) * L);
  double* bbl = (double*)malloc(sizeof(double) * L);
  if (spitzer)
    for (long c = 0; c < g.N; c++) f->BgradT[c] = 0.0;
  for (int d = 0; d < 3; d++) {
    const int d1 = order[d][0], d2 = order[d][1], d3 = order[d][2];
    const double dx = p->dx[d1];
    const double w1 = 8. / (12. * dx), w2 = -1. / (12. * dx);
    const double ww0 = -30. / (12. * dx * dx), ww1 = 16. / (12. * dx * dx), ww2 = -1. / (12. * dx * dx);
    const double signd1 = sgn[d1];
    const double pd[3] = {d1 == 0 ? 1. : 0., d1 == 1 ? 1. : 0., d1 == 2 ? 1. : 0.};
    const int sz = n[d1] + 2 * GH;
    for (int b = GH; b < GH + n[d3]; b++)
      for (int a = GH; a < GH + n[d2]; a++) {
        const long off = a * st[d2] + b * st[d3];
        for (int i = 0; i < sz; i++) {
          long c = off + i * st[d1];
          for (int v = 0; v < NV; v++) var[v * L + i] = U[v * g.N + c];
          double r0 = var[i], r1 = var[L + i], r2 = var[2 * L + i], r3 = var[3 * L + i], r4 = var[4 * L + i];
          double b5 = var[5 * L + i], b6 = var[6 * L + i], b7 = var[7 * L + i];
          double vel = var[(1 + d1) * L + i], mag = var[(5 + d1) * L + i];
          double dn = 1.0 / r0;
          double vv = r1 * r1 + r2 * r2 + r3 * r3;
          double bb = b5 * b5 + b6 * b6 + b7 * b7;
          double va2 = bb * dn;
          double ekin = 0.5 * r0 * vv;
          double pmag = 0.5 * bb;
          double x2 = va2 * inv_va2max, x4 = x2 * x2, s = 1.0 + x2;
          lf1[i] = s / (s + x4);
          double pr = pres[c];
          double cs2 = 5.0 / 3.0 * pr * dn;
          bbl[i] = bb;
          vv = sqrt(vv);
          vvl[i] = vv;
          cmax = smax(cmax, vv + 0.0 + sqrt(smax(cs2, lf1[i] * (cs2 + va2))));
          double mflx = vel * r0;
          flx[0 * L + i] = mflx;
          flx[1 * L + i] = mflx * r1 + pd[0] * pr;
          flx[2 * L + i] = mflx * r2 + pd[1] * pr;
          flx[3 * L + i] = mflx * r3 + pd[2] * pr;
          flx[4 * L + i] = vel * (r4 + ekin + pr);
          if (spitzer) {
            sfl[i] = f->sflx[c];
            flx[4 * L + i] += sfl[i] * var[(5 + d1) * L + i];
          }
          flx[5 * L + i] = vel * b5 - r1 * mag;
          flx[6 * L + i] = vel * b6 - r2 * mag;
          flx[7 * L + i] = vel * b7 - r3 * mag;
          ms[0 * L + i] = mag * b5 - pd[0] * pmag;
          ms[1 * L + i] = mag * b6 - pd[1] * pmag;
          ms[2 * L + i] = mag * b7 - pd[2] * pmag;
        }
        for (int i = GH; i < sz - GH; i++) {
          double res[NV];
          for (int v = 0; v < NV; v++) {
            const double* f = flx + v * L;
            res[v] = 0.0 - (w1 * (f[i + 1] - f[i - 1]) + w2 * (f[i + 2] - f[i - 2]));
          }
          if (dg) {  /* energy-flux divergence, its conduction share (src/mhdres_SR.C:368-384, 689-702) */
            const long cd = off + i * st[d1];
            if (spitzer) {
              const double* Bd = var + (5 + d1) * L;
              const double dn = -(w1 * ((sfl[i + 1] * Bd[i + 1]) - (sfl[i - 1] * Bd[i - 1])) +
                                  w2 * ((sfl[i + 2] * Bd[i + 2]) - (sfl[i - 2] * Bd[i - 2])));
              p->diag[cd] += res[4] - dn;
              p->diag[g.N + cd] += dn;
            } else {
              p->diag[cd] += res[4];
            }
          }
          const double* B2 = var + (5 + d2) * L;
          const double* B3 = var + (5 + d3) * L;
          double dB2 = w1 * (B2[i + 1] - B2[i - 1]) + w2 * (B2[i + 2] - B2[i - 2]);
          double dB3 = w1 * (B3[i + 1] - B3[i - 1]) + w2 * (B3[i + 2] - B3[i - 2]);
          double cbb[3];
          cbb[d1] = -B2[i] * dB2 - B3[i] * dB3;
          cbb[d2] = var[(5 + d1) * L + i] * dB2;
          cbb[d3] = var[(5 + d1) * L + i] * dB3;
          double lrt[3];
          for (int q = 0; q < 3; q++) {
            const double* m = ms + q * L;
            lrt[q] = w1 * (m[i + 1] - m[i - 1]) + w2 * (m[i + 2] - m[i - 2]);
          }
          double lf = lf1[i];
          for (int q = 0; q < 3; q++) lrt[q] = lf * lrt[q] + (1.0 - lf) * cbb[q];
          if (dg)  /* work of the Lorentz force (src/mhdres_SR.C:434-435, 751-752) */
            p->diag[2 * g.N + off + i * st[d1]] += var[L + i] * lrt[0] + var[2 * L + i] * lrt[1] + var[3 * L + i] * lrt[2];
          res[1] += lrt[0];
          res[2] += lrt[1];
          res[3] += lrt[2];
          res[4] += var[L + i] * lrt[0] + var[2 * L + i] * lrt[1] + var[3 * L + i] * lrt[2];
          long c = off + i * st[d1];
          if (needs_curlB) {
            double cb[3];
            cb[d1] = 0;
            cb[d2] = signd1 * dB3;
            cb[d3] = -signd1 * dB2;
            for (int q = 0; q < 3; q++) curlB[q * g.N + c] += cb[q];
            if (d == 2) {  /* the last pass has the whole curl: ohmic heating */
              const double cx = curlB[c], cy = curlB[g.N + c], cz = curlB[2 * g.N + c];
              R[4 * g.N + c] += eta * (cx * cx + cy * cy + cz * cz);
            }
            for (int v = 5; v <= 7; v++) {
              const double* b = var + v * L;
              res[v] += eta * (ww0 * b[i] + ww1 * (b[i + 1] + b[i - 1]) + ww2 * (b[i + 2] + b[i - 2]));
            }
          }
          for (int v = 0; v < NV; v++) R[v * g.N + c] += res[v];
          if (spitzer) {
            const long np1 = c + st[d1], np2 = c + 2 * st[d1], nm1 = c - st[d1], nm2 = c - 2 * st[d1];
            const double* T = temp;
            f->BgradT[c] += (var[(5 + d1) * L + i] * (w1 * (T[np1] - T[nm1]) + w2 * (T[np2] - T[nm2])));
            f->Rflx[c] -= hyp_diff * ((sfl[i + 2] + sfl[i - 2]) - 4. * (sfl[i + 1] + sfl[i - 1]) + 6. * sfl[i]);
            if (d == 2) {  /* the last pass: relaxation to the limited Spitzer flux */
              const double tempi = T[c];
              const double c_lim = cmax_hyp - vvl[i];
              const double tt32 = tempi * sqrt(tempi);
              double kap_spt = k0_spt * tempi * tt32;
              const double F_sat = sat_flx * var[i] * tt32;
              const double invBB = 1.0 / smax(1e-100, bbl[i]);
              double F_spt = -kap_spt * f->BgradT[c];
              const double f_lim = F_sat / (F_sat + fabs(F_spt * sqrt(invBB)));
              F_spt *= invBB * f_lim;
              kap_spt *= f_lim;
              const double nu_hyp = smin(c_lim * c_lim * var[4 * L + i] / (tempi * kap_spt), nu_hyp_max);
              f->Rflx[c] += nu_hyp * (F_spt - sfl[i]);
            }
          }
        }
      }
  }
  free(var); free(flx); free(ms); free(lf1); free(curlB); free(sfl); free(vvl); free(bbl);
  double dt_cfl = dxmin / cmax;
  if (needs_curlB) {
    const double dt_diff_fac = 0.5 / (1. / (p->dx[0] * p->dx[0]) + 1. / (p->dx[1] * p->dx[1]) + 1. / (p->dx[2] * p->dx[2]));
    double dt_res = dt_diff_fac / eta;
    if (p->CFL > 1) dt_res *= 0.5;
    dt_cfl = smin(dt_cfl, dt_res);
  }
  return dt_cfl;
}

double mo_mhd_residual(const mo_params* p, const double* U, const double* pres, double* R) {
  return mo_mhd_residual_ex(p, U, pres, NULL, R, NULL);
}

/* ----------------------------------------------------------- Sync_timestep */
int mo_sync_timestep(mo_params* p, double dt_rad, double dt_mhd, double* cfl) {
  double r0 = dt_rad, r1 = dt_mhd;
  if (invalid_pos(r0)) return -2;
  if (invalid_pos(r1)) return -3;
  double dt_min_rt = p->rt_tstep * p->CFL * r1;
  if (r0 < dt_min_rt) r0 = smax(r0, dt_min_rt);
  double dt_min = smin(r0, r1);
  double dt = smin(r0, p->CFL * r1);
  if (p->outcad > 0) {
    double num = p->time / p->outcad;
    int ce = (int)num;
    double rem = (num == (double)ce) ? 0.0 : (ce + 1) * p->outcad - p->time;
    if (rem > 0.0) dt = smin(dt, rem);
  }
  if (p->autostep) p->dt = dt;
  *cfl = p->dt / dt_min;
  if (*cfl >= 2.) return -4;
  return 0;
}

/* ------------------------------------------------- Source_Integrate_Tcheck */
static void tcheck_cell(const mo_params* p, double* U, long N, long c) {
  const double eps_min = p->tchk[0], rho_min = p->tchk[1];
  const double vmax = p->v_lim > 0.0 ? p->v_lim : p->tchk[3];
  const double eps_max = p->e_lim > 0.0 ? p->e_lim : p->tchk[2];
  double dn = fmax(rho_min, U[c]);
  double mx = U[N + c], my = U[2 * N + c], mz = U[3 * N + c];
  double vv = sqrt(mx * mx + my * my + mz * mz) / dn;
  double s = vmax / fmax(vmax, vv);
  double ekin = 0.5 * dn * vv * vv;
  double ee = U[4 * N + c];
  double lo = eps_min * dn + ekin * s * s;
  double up = eps_max * dn + ekin * s * s;
  U[4 * N + c] = fmin(fmax(ee, lo), up);
  U[c] = dn;
  U[N + c] = mx * s;
  U[2 * N + c] = my * s;
  U[3 * N + c] = mz * s;
}

void mo_source_integrate_ex(const mo_params* p, double* U, const double* U0, double* R, int stage, mo_fields* f) {
  geom g = geom_of(p);
  const long N = g.N;
  const double wdt = p->dt / ((double)(4 + 1 - stage));
  const double gx = -p->grav;
  const double invRdt = p->rt_cfl / p->dt;
  const double Qrad = 0.0, dmp = 0.0;
  /* diagnostics (src/Add_Sources_Integrate_SR.C:122-296): tvar4..6 set, tvar7 += TCheck's energy change / dt */
  const int dg = p->need_diagnostics && p->diag;
  const double invdt = 1.0 / p->dt;
  for (int k = GH; k < GH + p->nz; k++)
    for (int j = GH; j < GH + p->ny; j++)
      for (int i = GH; i < GH + p->nx; i++) {
        long c = at(&g, i, j, k);
        /* gravity + damping + radiation (src/Add_Sources_Integrate_SR.C:331-344) */
        double dn = invRdt * U[4 * N + c];
        double efaci = dn / fmax(dn, fabs(Qrad));
        dn = gx * U[c] - dmp;
        double edmp = dn * U[N + c];
        R[N + c] += dn;
        R[4 * N + c] += edmp + Qrad * efaci;
        if (dg) {
          p->diag[3 * N + c] = efaci;
          p->diag[4 * N + c] = edmp;
        }
        /* Boris correction (:347-392) */
        double rh = U[c], rd = R[c];
        double vx = U[N + c], vy = U[2 * N + c], vz = U[3 * N + c];
        double bx = U[5 * N + c], by = U[6 * N + c], bz = U[7 * N + c];
        double fx = R[N + c], fy = R[2 * N + c], fz = R[3 * N + c];
        double bb = bx * bx + by * by + bz * bz;
        double va2 = bb / rh;
        double x2 = va2 * p->inv_va2max, x4 = x2 * x2;
        double bf = x4 / (1 + x2 + x4);
        fx -= vx * rd;
        fy -= vy * rd;
        fz -= vz * rd;
        double q = (fx * bx + fy * by + fz * bz) / fmax(1e-100, bb);
        double b0 = -bf * (fx - q * bx), b1 = -bf * (fy - q * by), b2 = -bf * (fz - q * bz);
        double b3 = b0 * vx + b1 * vy + b2 * vz;
        R[N + c] += b0;
        R[2 * N + c] += b1;
        R[3 * N + c] += b2;
        R[4 * N + c] += b3;
        if (dg) p->diag[5 * N + c] = b3;
        /* time integration (:394-408) */
        for (int v = 0; v < NV; v++) {
          U[v * N + c] = U0[v * N + c] + wdt * R[v * N + c];
          R[v * N + c] = 0;
        }
        /* Tcheck (:444-465) */
        const double ee = U[4 * N + c];
        tcheck_cell(p, U, N, c);
        if (dg) p->diag[6 * N + c] += (U[4 * N + c] - ee) * invdt;
        /* hyperbolic conduction (:410-419) */
        if (p->spitzer > 0.0 && f && f->sflx) {
          f->sflx[c] = f->sflx0[c] + wdt * f->Rflx[c];
          f->Rflx[c] = 0;
        }
      }
}

void mo_source_integrate_tcheck(const mo_params* p, double* U, const double* U0, double* R, int stage) {
  mo_source_integrate_ex(p, U, U0, R, stage, NULL);
}

/* --------------------------------------------------- ghost fill / boundary */
/* Periodic fill of the periodic dimensions, in the dimension order and with
 * the growing face ranges of exchange_grid_acc (src/exchange.C:532-783). */
static void fill_dim_fields(const mo_params* p, const geom* g, double* U, int v0, int v1, int d, int lo[3], int hi[3]) {
  const int n[3] = {p->nx, p->ny, p->nz};
  int idx[3];
  for (int v = v0; v < v1; v++) {
    double* F = U + v * g->N;
    int a0 = d == 0 ? 1 : 0, a1 = d == 2 ? 1 : 2;
    for (idx[a1] = lo[a1]; idx[a1] <= hi[a1]; idx[a1]++)
      for (idx[a0] = lo[a0]; idx[a0] <= hi[a0]; idx[a0]++)
        for (int gg = 0; gg < GH; gg++) {
          int src[3] = {idx[0], idx[1], idx[2]}, dst[3] = {idx[0], idx[1], idx[2]};
          dst[d] = GH + n[d] + gg; src[d] = GH + gg;
          F[at(g, dst[0], dst[1], dst[2])] = F[at(g, src[0], src[1], src[2])];
          dst[d] = gg; src[d] = n[d] + gg;
          F[at(g, dst[0], dst[1], dst[2])] = F[at(g, src[0], src[1], src[2])];
        }
  }
}

static void fill_dim(const mo_params* p, const geom* g, double* U, int d, int lo[3], int hi[3]) {
  fill_dim_fields(p, g, U, 0, NV, d, lo, hi);
}

/* exchange of fields v0..v1-1 only (exchange_B_acc, exchange_single_acc:
 * src/exchange.C:785-983, 985-1150) */
static void exchange_fields(const mo_params* p, double* U, int v0, int v1) {
  geom g = geom_of(p);
  const int n[3] = {p->nx, p->ny, p->nz};
  int lo[3], hi[3];
  for (int d = 0; d < 3; d++) { lo[d] = GH; hi[d] = GH + n[d] - 1; }
  for (int d = 0; d < 3; d++) {
    if (d == 0 && !p->periodic_x) continue;
    fill_dim_fields(p, &g, U, v0, v1, d, lo, hi);
    lo[d] -= GH;
    hi[d] += GH;
  }
}

void mo_exchange_only(const mo_params* p, double* U) {
  geom g = geom_of(p);
  const int n[3] = {p->nx, p->ny, p->nz};
  int lo[3], hi[3];
  for (int d = 0; d < 3; d++) { lo[d] = GH; hi[d] = GH + n[d] - 1; }
  for (int d = 0; d < 3; d++) {
    if (d == 0 && !p->periodic_x) continue;
    fill_dim(p, &g, U, d, lo, hi);
    lo[d] -= GH;
    hi[d] += GH;
  }
}

void mo_boundaries(const mo_params* p, double* U) {
  mo_exchange_only(p, U);
  if (p->periodic_x) return;
  /* closed x: mirror with M_x, B_y, B_z sign flips over the full (y, z) range */
  geom g = geom_of(p);
  const long N = g.N;
  static const double sg[NV] = {1, -1, 1, 1, 1, 1, -1, -1};
  const int lb = GH, le = GH + p->nx - 1;
  for (int k = 0; k < g.sz; k++)
    for (int j = 0; j < g.sy; j++)
      for (int gg = 1; gg <= GH; gg++)
        for (int v = 0; v < NV; v++) {
          U[v * N + at(&g, le + gg, j, k)] = U[v * N + at(&g, le + 1 - gg, j, k)] * sg[v];
          U[v * N + at(&g, lb - gg, j, k)] = U[v * N + at(&g, lb - 1 + gg, j, k)] * sg[v];
        }
}

/* --------------------------------------------------------------- TVDlimit */
void mo_tvdlimit(const mo_params* p, double* U, const double* pres, double dt_tvd) {
  geom g = geom_of(p);
  const long N = g.N;
  const int n[3] = {p->nx, p->ny, p->nz};
  const long st[3] = {1, g.sx, (long)g.sx * g.sy};
  const double rho_min = p->tchk[1], eps_min = p->tchk[0];
  /* diagnostics (src/tvdlimit_SR.C:115-116): per unit of the full step's time */
  const int dg = p->need_diagnostics && p->diag;
  const double idt_full = 1.0 / p->dt, dt_fac = dt_tvd / p->dt;
  const double rho_lev = pow(p->tvd[0], 2);
  const int rho_log = (int)p->tvd[1];
  const double q_rho_max = log(p->tvd[2]);
  const double visc_coeff_bot = smin(1.0, p->tvd_visc_bnd[0]);
  const double visc_slope_bot = smax(0.0, p->tvd_visc_bnd[0] - 1.0);
  const double visc_coeff_top = smin(1.0, p->tvd_visc_bnd[1]);
  const double visc_slope_top = smax(0.0, p->tvd_visc_bnd[1] - 1.0);
  const double eta_coeff_bot = smin(1.0, p->tvd_eta_bnd[0]);
  const double eta_slope_bot = smax(0.0, p->tvd_eta_bnd[0] - 1.0);
  const double eta_coeff_top = smin(1.0, p->tvd_eta_bnd[1]);
  const double eta_slope_top = smax(0.0, p->tvd_eta_bnd[1] - 1.0);
  const double B_par_diff = p->tvd[3], vhyp = p->tvd[4], Qdiff_bnd = p->tvd[5];
  const double pm_v = p->tvd[6], pm_B = p->tvd[7], vmax_lim = p->tvd[8], CME_thresh = p->tvd[9];
  const double h_bnd_bot = p->tvd_h_bnd[0] < 1 ? p->tvd_h_bnd[0] : p->tvd_h_bnd[0] / (double)p->nx;
  const double h_bnd_top = p->tvd_h_bnd[1] < 1 ? p->tvd_h_bnd[1] : p->tvd_h_bnd[1] / (double)p->nx;
  const double* th = p->tvd_h;
  const double* tc = p->tvd_cs;
  const int is_gbeg0 = !p->periodic_x, is_gend0 = !p->periodic_x;
  const int need_coeff = (p->tvd_coeff[0] * p->tvd_coeff[1] * p->tvd_coeff[2] * p->tvd_coeff[3] != 1.0);
  const double v_lim = p->v_lim;
  const double vsqr_diff = vmax_lim < 1.0 ? pow(vmax_lim * v_lim, 2.0) : pow(vmax_lim, 2.0);
  /* vertical boundary profiles (src/tvdlimit_SR.C:137-149) */
  const int sx = g.sx;
  double* hfb = (double*)malloc(sizeof(double) * sx);
  double* hft = (double*)malloc(sizeof(double) * sx);
  double* qft = (double*)malloc(sizeof(double) * sx);
  const double gxmax0 = p->dx[0] * p->nx;
  for (int i = 0; i < sx; i++) {
    double hh = (0.0 + (0.5 + (i - GH)) * p->dx[0]) / gxmax0;
    double vv = smax(0.0, 1.0 - 0.5 * (1.0 - hh) / h_bnd_top);
    hft[i] = smin(1.0, vv * vv);
    vv = smax(0.0, 1.0 - 0.5 * hh / h_bnd_bot);
    hfb[i] = smin(1.0, vv * vv);
    qft[i] = (hh < 1 - 2 * h_bnd_top) ? 1.0 : Qdiff_bnd;
  }
  const double CZ_val = (double)(p->tau0 > 1.0e-5);
  int L = 0;
  for (int d = 0; d < 3; d++) L = imax(L, n[d] + 2 * GH);
  double *var = malloc(sizeof(double) * NV * L), *slp = malloc(sizeof(double) * NV * L);
  double *flx = malloc(sizeof(double) * NV * L), *res = malloc(sizeof(double) * NV * L);
  double *qrho = malloc(sizeof(double) * L), *h_b = malloc(sizeof(double) * L), *h_t = malloc(sizeof(double) * L);
  double *q_t = malloc(sizeof(double) * L), *cm = malloc(sizeof(double) * L), *bsqr = malloc(sizeof(double) * L);
  double *vsqr = malloc(sizeof(double) * L), *BC2 = malloc(sizeof(double) * L), *hyd = malloc(sizeof(double) * L);
  double *hyp_e = malloc(sizeof(double) * L), *hyp_v = malloc(sizeof(double) * L), *hyp_B = malloc(sizeof(double) * L);
  double* CZ = malloc(sizeof(double) * L);
  static const int order[3][3] = {{0, 1, 2}, {1, 0, 2}, {2, 0, 1}};
  int blo[3], bhi[3];
  for (int d = 0; d < 3; d++) { blo[d] = 0; bhi[d] = n[d] + 2 * GH - 1; }
  for (int d = 0; d < 3; d++) {
    const int d1 = order[d][0], d2 = order[d][1], d3 = order[d][2];
    const double cmax = 0.975 * p->dx[d1] / dt_tvd;
    const int sz = n[d1] + 2 * GH;
    const double idx1 = 1. / p->dx[d1];
    for (int b = blo[d3]; b <= bhi[d3]; b++)
      for (int a = blo[d2]; a <= bhi[d2]; a++) {
        const long off = a * st[d2] + b * st[d3];
        for (int i = 0; i < sz; i++) {
          long c = off + i * st[d1];
          var[i] = smax(rho_min, U[c]);
          for (int v = 1; v < NV; v++) var[v * L + i] = U[v * N + c];
          CZ[i] = CZ_val;
          int xi = d1 == 0 ? i : (d2 == 0 ? a : b);
          h_b[i] = hfb[xi]; h_t[i] = hft[xi]; q_t[i] = qft[xi];
        }
        for (int i = 0; i < sz; i++) {
          long c = off + i * st[d1];
          double dn = 1.0 / var[i];
          var[L + i] = var[L + i] * dn;
          var[2 * L + i] = var[2 * L + i] * dn;
          var[3 * L + i] = var[3 * L + i] * dn;
          double vv = var[L + i] * var[L + i] + var[2 * L + i] * var[2 * L + i] + var[3 * L + i] * var[3 * L + i];
          double bb = var[5 * L + i] * var[5 * L + i] + var[6 * L + i] * var[6 * L + i] + var[7 * L + i] * var[7 * L + i];
          var[4 * L + i] = var[4 * L + i] * dn - 0.5 * vv;
          vsqr[i] = vv;
          bsqr[i] = bb;
          vv = sqrt(vv);
          double va2 = bb * dn;
          double x2 = va2 * p->inv_va2max, x4 = x2 * x2, s = 1.0 + x2;
          double lf = s / (s + x4);
          double cs2 = 5.0 / 3.0 * pres[c] * dn;
          double cfast = sqrt(va2 + cs2);
          double CME = (1.0 - CZ[i]) * ((double)(vv >= CME_thresh * cfast));
          dn = var[i] * var[i];
          double rf = smin(lf, dn / (dn + rho_lev));
          double hh = 1.0 - h_b[i] - h_t[i];
          double cf = h_b[i] * tc[0] + (rf * tc[1] + (1.0 - rf) * tc[2]) * hh + h_t[i] * tc[3];
          cf = smax(cf, CME);
          cs2 *= cf * cf;
          double vv_amb = 0.0;
          cm[i] = vv_amb + vv + sqrt(smax(cs2, lf * (cs2 + va2)));
          hyp_e[i] = h_b[i] * th[0] + (rf * th[1] + (1.0 - rf) * th[2]) * hh + h_t[i] * th[3];
          hyp_v[i] = h_b[i] * th[0] + (rf * th[1] + (1.0 - rf) * th[2] * pm_v) * hh + h_t[i] * th[3] * pm_v;
          hyp_B[i] = h_b[i] * th[0] + (rf * th[1] + (1.0 - rf) * th[2] * pm_B) * hh + h_t[i] * th[3] * pm_B;
          hyp_e[i] *= (1.0 - CME);
          hyp_v[i] *= (1.0 - CME);
          BC2[i] = 1.0 - lf;
        }
        if ((d1 == 0) && (vhyp > 0.0)) {
          for (int i = 0; i < sz; i++) {
            hyd[i] = vhyp * sqrt(vsqr[i]);
            hyd[i] = 0.5 * idx1 * smax(0.0, smin(hyd[i], cmax - cm[i]));
          }
        }
        if (rho_log) {
          for (int i = 0; i < sz; i++) {
            var[i] = log(var[i]);
            var[4 * L + i] = log(var[4 * L + i]);
          }
          for (int i = 0; i < sz - 1; i++) qrho[i] = fabs(var[i] - var[i + 1]);
        } else {
          for (int i = 0; i < sz - 1; i++) qrho[i] = fabs(log(var[i]) - log(var[i + 1]));
        }
        for (int v = 0; v < NV; v++) {
          const double* q = var + v * L;
          for (int i = 1; i < sz - 1; i++) {
            double sl = q[i] - q[i - 1];
            double sr = q[i + 1] - q[i];
            double slm = 0.25 * (sl + sr);
            double lower = smin(smin(sl, sr), slm);
            double upper = smax(smax(sl, sr), slm);
            slp[v * L + i] = smax(0.0, lower) + smin(0.0, upper);
          }
        }
        if ((visc_slope_bot > 0.0) || (visc_slope_top > 0.0)) {
          for (int i = 1; i < sz - 1; i++) {
            double cf = (1.0 - visc_slope_bot * h_b[i]) * (1.0 - visc_slope_top * h_t[i]);
            slp[L + i] *= cf; slp[2 * L + i] *= cf; slp[3 * L + i] *= cf;
          }
        }
        if ((eta_slope_bot > 0.0) || (eta_slope_top > 0.0)) {
          for (int i = 1; i < sz - 1; i++) {
            double cf = (1.0 - eta_slope_bot * h_b[i]) * (1.0 - eta_slope_top * h_t[i]);
            slp[5 * L + i] *= cf; slp[6 * L + i] *= cf; slp[7 * L + i] *= cf;
          }
        }
        for (int i = 1; i < sz - 1; i++)
          if (qrho[i] > q_rho_max) slp[i] = 0.0;
        if (vmax_lim > 0.0) {
          for (int i = 1; i < sz - 1; i++)
            if (vsqr[i] > vsqr_diff) { slp[L + i] = 0.0; slp[2 * L + i] = 0.0; slp[3 * L + i] = 0.0; }
        }
        for (int v = 0; v < NV; v++) {
          const double* q = var + v * L;
          const double* sp = slp + v * L;
          const double* hy = (v >= 1 && v <= 3) ? hyp_v : ((v >= 5 && v <= 7) ? hyp_B : hyp_e);
          for (int i = 1; i < sz - 2; i++) {
            double sl = q[i + 1] - q[i];
            double sl_lim = q[i + 1] - q[i] - (sp[i] + sp[i + 1]);
            double dn = hy[i];
            double rf = fabs(sl_lim) / smax(1e-100, fabs(sl));
            double cf = smax(0.0, smin(sl_lim, sl)) + smin(0.0, smax(sl_lim, sl));
            flx[v * L + i] = smax(0.0, 1.0 + dn * (rf - 1.0)) * cf;
          }
        }
        for (int i = 1; i < sz - 2; i++) {
          double fac = 0.5 * idx1 * smin(cmax, smax(cm[i], cm[i + 1]));
          for (int v = 0; v < NV; v++) flx[v * L + i] *= fac;
          flx[(5 + d1) * L + i] *= B_par_diff;
        }
        if (need_coeff) {
          for (int i = 1; i < sz - 2; i++) {
            flx[i] *= p->tvd_coeff[0];
            double cf = smax(p->tvd_coeff[1], visc_coeff_bot * h_b[i] + visc_coeff_top * h_t[i]);
            flx[L + i] *= cf; flx[2 * L + i] *= cf; flx[3 * L + i] *= cf;
            flx[4 * L + i] *= p->tvd_coeff[2];
            cf = smax(p->tvd_coeff[3], eta_coeff_bot * h_b[i] + eta_coeff_top * h_t[i]);
            flx[5 * L + i] *= cf; flx[6 * L + i] *= cf; flx[7 * L + i] *= cf;
          }
        }
        if ((d1 == 0) && (vhyp > 0.0)) {
          int istart = 1;
          if (is_gbeg0) istart += GH;
          for (int i = istart; i < sz - 2; i++) {
            double dn = smax(hyd[i], hyd[i + 1]);
            static const int hv[3] = {0, 1, 4};
            for (int q = 0; q < 3; q++) {
              const double* u = var + hv[q] * L;
              flx[hv[q] * L + i] -= dn * (0.125 * (u[i + 2] - u[i - 1]) - 0.375 * (u[i + 1] - u[i]));
            }
          }
        }
        for (int i = 1; i < sz - 2; i++) {
          double f0 = flx[i], f1 = flx[L + i], f2 = flx[2 * L + i], f3 = flx[3 * L + i], f4 = flx[4 * L + i];
          double u[5];
          for (int v = 0; v < 5; v++)
            u[v] = 0.5 * (var[v * L + i] + slp[v * L + i] + var[v * L + i + 1] - slp[v * L + i + 1]);
          if (rho_log) {
            u[0] = exp(u[0]);
            f0 *= u[0];
            u[4] = exp(u[4]);
            f4 *= u[4];
          }
          double min_cz = f0 * smin(CZ[i], CZ[i + 1]);
          f1 *= u[0]; f1 += u[1] * min_cz;
          f2 *= u[0]; f2 += u[2] * min_cz;
          f3 *= u[0]; f3 += u[3] * min_cz;
          f4 *= u[0];
          f4 += (u[4] * min_cz) + q_t[i] * (u[1] * f1 + u[2] * f2 + u[3] * f3);
          flx[i] = f0; flx[L + i] = f1; flx[2 * L + i] = f2; flx[3 * L + i] = f3; flx[4 * L + i] = f4;
        }
        if (d1 == 0) {
          if (is_gend0) flx[5 * L + sz - GH - 1] = 0.0;
          if (is_gbeg0) flx[5 * L + GH - 1] = 0.0;
        }
        for (int v = 0; v < NV; v++)
          for (int i = GH; i < sz - GH; i++) res[v * L + i] = dt_tvd * (flx[v * L + i] - flx[v * L + i - 1]);
        for (int i = GH; i < sz - GH; i++)
          res[4 * L + i] += (1.0 - q_t[i]) * (res[L + i] * var[L + i] + res[2 * L + i] * var[2 * L + i] +
                                              res[3 * L + i] * var[3 * L + i]);
        if (dg)  /* energy change of the sweep (src/tvdlimit_SR.C:577-584) */
          for (int i = GH; i < sz - GH; i++) p->diag[7 * N + off + i * st[d1]] += res[4 * L + i] * idt_full;
        for (int i = GH; i < sz - GH; i++) {
          double dn = (res[L + i] * var[5 * L + i] + res[2 * L + i] * var[6 * L + i] + res[3 * L + i] * var[7 * L + i]) /
                      smax(1e-100, bsqr[i]);
          double b0 = -BC2[i] * (res[L + i] - dn * var[5 * L + i]);
          double b1 = -BC2[i] * (res[2 * L + i] - dn * var[6 * L + i]);
          double b2 = -BC2[i] * (res[3 * L + i] - dn * var[7 * L + i]);
          double b3 = b0 * var[L + i] + b1 * var[2 * L + i] + b2 * var[3 * L + i];
          res[L + i] += b0; res[2 * L + i] += b1; res[3 * L + i] += b2; res[4 * L + i] += b3;
          if (dg) p->diag[5 * N + off + i * st[d1]] += b3 * idt_full;  /* (:601-604) */
        }
        for (int i = 1; i < sz - 2; i++)
          qrho[i] = (var[5 * L + i + 1] - var[5 * L + i]) * flx[5 * L + i] +
                    (var[6 * L + i + 1] - var[6 * L + i]) * flx[6 * L + i] +
                    (var[7 * L + i + 1] - var[7 * L + i]) * flx[7 * L + i];
        for (int i = GH; i < sz - GH; i++) {
          double qres = 0.5 * (qrho[i] + qrho[i - 1]) * q_t[i];
          res[4 * L + i] += dt_tvd * qres;
          if (dg) p->diag[8 * N + off + i * st[d1]] += dt_fac * qres;  /* Qres (:617-624) */
        }
        if (dg)  /* viscous heating, for the diagnostics only (:626-635) */
          for (int i = 1; i < sz - 2; i++)
            qrho[i] = (var[L + i + 1] - var[L + i]) * flx[L + i] + (var[2 * L + i + 1] - var[2 * L + i]) * flx[2 * L + i] +
                      (var[3 * L + i + 1] - var[3 * L + i]) * flx[3 * L + i];
        for (int i = GH; i < sz - GH; i++) {
          long c = off + i * st[d1];
          for (int v = 0; v < NV; v++) U[v * N + c] += res[v * L + i];
          U[c] = smax(rho_min, U[c]);
          double mx = U[N + c], my = U[2 * N + c], mz = U[3 * N + c];
          const double eb = U[4 * N + c];
          U[4 * N + c] = smax(U[4 * N + c], eps_min * U[c] + 0.5 * (mx * mx + my * my + mz * mz) / U[c]);
          if (dg) {  /* the energy floor's change and Qvis (:659-667) */
            p->diag[6 * N + c] += (U[4 * N + c] - eb) * idt_full;
            p->diag[9 * N + c] += dt_fac * (0.5 * (qrho[i] + qrho[i - 1]) * q_t[i]);
          }
        }
      }
    blo[d1] = GH;
    bhi[d1] = GH + n[d1] - 1;
  }
  free(var); free(slp); free(flx); free(res); free(qrho); free(h_b); free(h_t); free(q_t); free(cm);
  free(bsqr); free(vsqr); free(BC2); free(hyd); free(hyp_e); free(hyp_v); free(hyp_B); free(CZ);
  free(hfb); free(hft); free(qft);
}

/* ------------------------------------------------------------------ TCheck */
void mo_tcheck(const mo_params* p, double* U) {
  geom g = geom_of(p);
  /* diagnostics: tvar7 += energy change / dt (src/Add_Sources_Integrate_SR.C:560-564, 618-620) */
  const int dg = p->need_diagnostics && p->diag;
  const double invdt = p->dt > 0.0 ? 1.0 / p->dt : 0.0;
  for (int k = GH; k < GH + p->nz; k++)
    for (int j = GH; j < GH + p->ny; j++)
      for (int i = GH; i < GH + p->nx; i++) {
        const long c = at(&g, i, j, k);
        const double eei = U[4 * g.N + c];
        tcheck_cell(p, U, g.N, c);
        if (dg) p->diag[6 * g.N + c] += (U[4 * g.N + c] - eei) * invdt;
      }
}

/* ------------------------------------------------- physical x boundaries */
/* Scalar EOS lookups of src/eos_init.C (their bilinear terms are summed in
 * another order than ConsToPrim's): p_interp :319-343, s_interp :268-292,
 * d3_interp :216-240, eps3_interp :242-266. */
static double eos_fwd(const mo_eos* e, int t, double ee, double dd) {
  const double ee1 = log(ee + e->eps_off);
  const double logr = log(dd);
  int i = (int)((ee1 - e->xeps[0]) * e->inv_del_eps);
  if (i < 0) i = 0;
  if (i > e->N_eps - 2) i = e->N_eps - 2;
  int j = (int)((logr - e->xlr[0]) * e->inv_del_lr);
  if (j < 0) j = 0;
  if (j > e->N_lr - 2) j = e->N_lr - 2;
  const float* T = e->tab[t];
  const long L = e->N_lr;
  return (logr - e->xlr[j]) * (ee1 - e->xeps[i]) * (double)T[(i + 1) * L + j + 1] +
         (logr - e->xlr[j]) * (e->xeps[i + 1] - ee1) * (double)T[i * L + j + 1] +
         (e->xlr[j + 1] - logr) * (ee1 - e->xeps[i]) * (double)T[(i + 1) * L + j] +
         (e->xlr[j + 1] - logr) * (e->xeps[i + 1] - ee1) * (double)T[i * L + j];
}
static double eos_p_interp(const mo_eos* e, double ee, double dd) { return exp(eos_fwd(e, 0, ee, dd)); }
static double eos_s_interp(const mo_eos* e, double ee, double dd) { return eos_fwd(e, 2, ee, dd) - e->ss_off; }
static double eos_inv(const mo_eos* e, const float* T, double pp, double ss) {
  const double ss1 = ss + e->ss_off;
  const double logp = log(pp);
  int i = (int)((logp - e->xlp3[0]) * e->inv_del_lp3);
  if (i < 0) i = 0;
  if (i > e->N_lp3 - 2) i = e->N_lp3 - 2;
  int j = (int)((ss1 - e->xs3[0]) * e->inv_del_s3);
  if (j < 0) j = 0;
  if (j > e->N_s3 - 2) j = e->N_s3 - 2;
  const long L = e->N_s3;
  return (logp - e->xlp3[i]) * (ss1 - e->xs3[j]) * (double)T[(i + 1) * L + j + 1] +
         (logp - e->xlp3[i]) * (e->xs3[j + 1] - ss1) * (double)T[(i + 1) * L + j] +
         (e->xlp3[i + 1] - logp) * (ss1 - e->xs3[j]) * (double)T[i * L + j + 1] +
         (e->xlp3[i + 1] - logp) * (e->xs3[j + 1] - ss1) * (double)T[i * L + j];
}
static double eos_d3_interp(const mo_eos* e, double pp, double ss) { return exp(eos_inv(e, e->d3, pp, ss)); }
static double eos_eps3_interp(const mo_eos* e, double pp, double ss) {
  return exp(eos_inv(e, e->eps3, pp, ss)) - e->eps_off;
}

/* set_p_s_bc (src/boundary_pdmp_1_fftw3.C:496-565): p_bc from the mean
 * pressures of the two bottom layers, s_bc from the mean entropy of the
 * upflows (or of all cells) of the first one; only the negative ones are set. */
static void set_p_s_bc(mo_params* p, const mo_eos* e, const double* U) {
  geom g = geom_of(p);
  const long N = g.N;
  double b0 = 0, b1 = 0, b2 = 0, b3 = 0, b4 = 0;
  for (int k = GH; k < GH + p->nz; k++)
    for (int j = GH; j < GH + p->ny; j++) {
      const long c1 = at(&g, GH, j, k), c2 = at(&g, GH + 1, j, k);
      const double d1 = U[c1], d2 = U[c2];
      const double m1 = U[N + c1], m2 = U[2 * N + c1], m3 = U[3 * N + c1];
      const double q1 = U[N + c2], q2 = U[2 * N + c2], q3 = U[3 * N + c2];
      const double e1 = U[4 * N + c1] - 0.5 * (m1 * m1 + m2 * m2 + m3 * m3) / d1;
      const double e2 = U[4 * N + c2] - 0.5 * (q1 * q1 + q2 * q2 + q3 * q3) / d2;
      const double eps1 = e1 / d1, eps2 = e2 / d2;
      b0 += eos_p_interp(e, eps1, d1);
      b1 += eos_p_interp(e, eps2, d2);
      if (m1 > 0.0) {
        b2 += 1.0;
        b3 += eos_s_interp(e, eps1, d1);
      }
      b4 += eos_s_interp(e, eps1, d1);
    }
  const double n = (double)(p->ny * p->nz);
  b0 /= n;
  b1 /= n;
  if (p->p_bc < 0.0) p->p_bc = b0 * sqrt(b0 / b1);
  if (p->s_bc < 0.0) p->s_bc = (b2 > 0.0) ? b3 / b2 : b4 / n;
}

/* SetBoundaryConditions (src/boundary_pdmp_1_fftw3.C:81-493) without the
 * potential-field top: at the bottom, ghost pressures extrapolated
 * exponentially from the mean pressure of the two first layers to p_bc with
 * their fluctuations damped (p1_dmp = 0.8), entropy s_bc in upflows and the
 * cell's own entropy in downflows, density and energy from the inverse EOS,
 * momentum scaled down where |B_x| nears B_crit; at the top, M_x mirrored
 * (always, or only in downflows with bnd_top = 1), B_y and B_z mirrored, and
 * the internal energy fixed at eps_top when it is positive.  Covers the y and
 * z ghost columns too; the caller has exchanged the periodic dimensions. */
static void set_boundary_conditions(mo_params* p, const mo_eos* e, double* U) {
  geom g = geom_of(p);
  const long N = g.N;
  const int lb = GH, le = GH + p->nx - 1;
  const double p1_dmp = 0.8;
  const double B_crit = p->bnd_bcrit / sqrt(8.0 * asin(1.0));
  if (p->bnd_ini) {
    if ((p->p_bc < 0.0) || (p->s_bc < 0.0)) set_p_s_bc(p, e, U);
    p->bnd_ini = 0;
  }
  double l5 = 0, l6 = 0;
  for (int k = GH; k < GH + p->nz; k++)
    for (int j = GH; j < GH + p->ny; j++) {
      const long c1 = at(&g, lb, j, k), c2 = at(&g, lb + 1, j, k);
      const double d1 = U[c1], d2 = U[c2];
      const double m1 = U[N + c1], m2 = U[2 * N + c1], m3 = U[3 * N + c1];
      const double q1 = U[N + c2], q2 = U[2 * N + c2], q3 = U[3 * N + c2];
      const double e1 = U[4 * N + c1] - 0.5 * ((m1 * m1 + m2 * m2 + m3 * m3) / d1);
      const double e2 = U[4 * N + c2] - 0.5 * ((q1 * q1 + q2 * q2 + q3 * q3) / d2);
      l5 += eos_p_interp(e, e1 / d1, d1);
      l6 += eos_p_interp(e, e2 / d2, d2);
    }
  const double cn = 1.0 / ((double)(p->ny * p->nz));
  const double pmean1 = l5 * cn, pmean2 = l6 * cn;
  for (int k = 0; k < g.sz; k++)
    for (int j = 0; j < g.sy; j++) {
      const long c1 = at(&g, lb, j, k), c2 = at(&g, lb + 1, j, k);
      double u1[NV], u2[NV];
      for (int v = 0; v < NV; v++) { u1[v] = U[v * N + c1]; u2[v] = U[v * N + c2]; }
      u1[4] -= 0.5 * (u1[1] * u1[1] + u1[2] * u1[2] + u1[3] * u1[3]) / u1[0];
      u2[4] -= 0.5 * (u2[1] * u2[1] + u2[2] * u2[2] + u2[3] * u2[3]) / u2[0];
      double eps1 = u1[4] / u1[0], eps2 = u2[4] / u2[0];
      const double pmag = 0.5 * u1[5] * u1[5];
      const double pmin1 = eos_p_interp(e, eps1, u1[0]) - pmean1;
      const double pmin2 = eos_p_interp(e, eps2, u2[0]) - pmean2;
      const double smin1 = eos_s_interp(e, eps1, u1[0]);
      const double smin2 = eos_s_interp(e, eps2, u2[0]);
      double s1, s2;
      if (u1[1] >= 0.e0) { s1 = p->s_bc; s2 = p->s_bc; }
      else { s1 = smin1; s2 = smin2; }
      double c = p->p_bc / sqrt(pmean1 * pmean2);
      double p1 = pmean1 * c;
      double p2 = pmean1 * c * c;
      p1 += pmin1 * p1_dmp;
      p2 += pmin1 * p1_dmp * p1_dmp;
      p1 -= pmag * (1.0 - p1_dmp);
      p2 -= pmag * (1.0 - p1_dmp * p1_dmp);
      (void)pmin2;
      c = u1[5] / B_crit;
      c = pow(c, 4);
      c = (1.0 - c) / (1.0 + c);
      for (int v = 1; v <= 3; v++) { u1[v] *= c; u2[v] *= c; }
      const double rho1 = eos_d3_interp(e, p1, s1), rho2 = eos_d3_interp(e, p2, s2);
      eps1 = eos_eps3_interp(e, p1, s1);
      eps2 = eos_eps3_interp(e, p2, s2);
      u1[0] = rho1;
      u2[0] = rho2;
      u1[4] = eps1 * rho1 + 0.5 * (u1[1] * u1[1] + u1[2] * u1[2] + u1[3] * u1[3]) / u1[0];
      u2[4] = eps2 * rho2 + 0.5 * (u2[1] * u2[1] + u2[2] * u2[2] + u2[3] * u2[3]) / u2[0];
      const long g1 = at(&g, lb - 1, j, k), g2 = at(&g, lb - 2, j, k);
      for (int v = 0; v < NV; v++) { U[v * N + g1] = u1[v]; U[v * N + g2] = u2[v]; }
    }
  for (int k = 0; k < g.sz; k++)
    for (int j = 0; j < g.sy; j++) {
      const long c1 = at(&g, le, j, k), c2 = at(&g, le - 1, j, k);
      double u1[NV], u2[NV];
      for (int v = 0; v < NV; v++) { u1[v] = U[v * N + c1]; u2[v] = U[v * N + c2]; }
      if (p->bnd_top == 1) {
        if (u1[1] < 0.0) { u1[1] *= -1; u2[1] *= -1; }
      } else {
        u1[1] *= -1;
        u2[1] *= -1;
      }
      if (p->bnd_eps_top > 0.0) {
        u1[4] = p->bnd_eps_top * u1[0] + 0.5 * (u1[1] * u1[1] + u1[2] * u1[2] + u1[3] * u1[3]) / u1[0];
        u2[4] = p->bnd_eps_top * u2[0] + 0.5 * (u2[1] * u2[1] + u2[2] * u2[2] + u2[3] * u2[3]) / u2[0];
      }
      u1[6] *= -1; u2[6] *= -1;
      u1[7] *= -1; u2[7] *= -1;
      const long g1 = at(&g, le + 1, j, k), g2 = at(&g, le + 2, j, k);
      for (int v = 0; v < NV; v++) { U[v * N + g1] = u1[v]; U[v * N + g2] = u2[v]; }
    }
}

/* the heat flux's boundary values (src/boundary_pdmp_1_fftw3.C:302-306, 426-438):
 * zero in the bottom ghosts; at the top symmetric with eps_top > 0, else zero
 * in the two top layers and their ghosts */
static void sflx_boundaries(const mo_params* p, double* sflx) {
  geom g = geom_of(p);
  const int lb = GH, le = GH + p->nx - 1;
  for (int k = 0; k < g.sz; k++)
    for (int j = 0; j < g.sy; j++) {
      sflx[at(&g, lb - 1, j, k)] = 0.0;
      sflx[at(&g, lb - 2, j, k)] = 0.0;
      if (p->bnd_eps_top > 0.0) {
        sflx[at(&g, le + 1, j, k)] = sflx[at(&g, le, j, k)];
        sflx[at(&g, le + 2, j, k)] = sflx[at(&g, le - 1, j, k)];
      } else {
        sflx[at(&g, le - 1, j, k)] = 0.0;
        sflx[at(&g, le, j, k)] = 0.0;
        sflx[at(&g, le + 1, j, k)] = 0.0;
        sflx[at(&g, le + 2, j, k)] = 0.0;
      }
    }
}

void mo_boundaries_ex(mo_params* p, const mo_eos* e, double* U, mo_fields* f, int needs_sflx) {
  const int spitzer = p->spitzer > 0.0 && f && f->sflx;
  if (p->xbnd == 1 && !p->periodic_x) {
    mo_exchange_only(p, U);
    if (spitzer && needs_sflx) exchange_fields(p, f->sflx, 0, 1);
    set_boundary_conditions(p, e, U);
    if (spitzer) sflx_boundaries(p, f->sflx);
  } else {
    mo_boundaries(p, U);
    if (spitzer && needs_sflx) exchange_fields(p, f->sflx, 0, 1);
  }
}

void mo_boundaries_eos(mo_params* p, const mo_eos* e, double* U) { mo_boundaries_ex(p, e, U, NULL, 1); }

/* ------------------------------------------------------------- Clean_divB */
/* Fourth-order divergence of B at interior cell (i, j, k), summed over the
 * dimensions from zero as src/clean_divB.C:136-156 does. */
static double divb_cell(const geom* g, const double* U, const double w1[3], const double w2[3], int i, int j, int k) {
  const long c = at(g, i, j, k);
  const long st[3] = {1, g->sx, (long)g->sx * g->sy};
  double d = 0.0;
  for (int v = 0; v < 3; v++) {
    const double* B = U + (5 + v) * g->N;
    const long s = st[v];
    d += (w1[v] * (B[c + s] - B[c - s]) + w2[v] * (B[c + 2 * s] - B[c - 2 * s]));
  }
  return d;
}

static double divb_pass(const mo_params* p, const geom* g, const double* U, const double w1[3], const double w2[3],
                        double* divB) {
  double err = 0.0;
  for (int k = GH; k < GH + p->nz; k++)
    for (int j = GH; j < GH + p->ny; j++)
      for (int i = GH; i < GH + p->nx; i++) {
        const double d = divb_cell(g, U, w1, w2, i, j, k);
        divB[at(g, i, j, k)] = d;
        err = smax(err, fabs(d));
      }
  return err;
}

/* src/clean_divB.C:35-369 on one rank: damped iterations phi += fac*divB -
 * damp*phi, B += grad(phi), e += phi*divB, with the iteration count adapted
 * from call to call (next_iter, a function static there, lives in p).  phi
 * persists between calls; divB receives the last divergence.  A closed x
 * dimension keeps B's x ghosts as the caller left them (exchange_B_acc does
 * not fill physical boundaries) and makes phi antisymmetric across it. */
void mo_clean_divB(mo_params* p, double* U, double* phi, double* divB) {
  geom g = geom_of(p);
  const long N = g.N;
  const int it_max = (int)p->divB_itmax;
  const double divB_coeff = 1.0, divB_damp = 0.65;
  double w1[3], w2[3], err_unit = 0.0;
  for (int v = 0; v < 3; v++) {
    err_unit += 1.0 / p->dx[v];
    w1[v] = 8. / (12. * p->dx[v]);
    w2[v] = -1. / (12. * p->dx[v]);
  }
  err_unit = 0.5 / err_unit * 3.5449;
  double dxmin = smin(p->dx[0], p->dx[1]);
  double dxmax = smax(p->dx[0], p->dx[1]);
  dxmin = smin(dxmin, p->dx[2]);
  dxmax = smax(dxmin, p->dx[2]);  /* as written there: the new dxmin, not dxmax */
  const double divB_fac = divB_coeff * smin(dxmin, 0.4 * dxmax) * dxmin;

  exchange_fields(p, U, 5, 8);
  double err0 = divb_pass(p, &g, U, w1, w2, divB), err1 = 0.0;
  const int n = p->divB_next_iter;
  const long st[3] = {1, g.sx, (long)g.sx * g.sy};
  int iter;
  for (iter = 0; iter < n; iter++) {
    for (int k = GH; k < GH + p->nz; k++)
      for (int j = GH; j < GH + p->ny; j++)
        for (int i = GH; i < GH + p->nx; i++) {
          const long c = at(&g, i, j, k);
          phi[c] += divB_fac * divB[c] - divB_damp * phi[c];
        }
    exchange_fields(p, phi, 0, 1);
    if (!p->periodic_x) {
      const int lb = GH, le = GH + p->nx - 1;
      for (int k = GH; k < GH + p->nz; k++)
        for (int j = GH; j < GH + p->ny; j++) {
          phi[at(&g, lb - 1, j, k)] = -phi[at(&g, lb, j, k)];
          phi[at(&g, lb - 2, j, k)] = -phi[at(&g, lb + 1, j, k)];
          phi[at(&g, le + 1, j, k)] = -phi[at(&g, le, j, k)];
          phi[at(&g, le + 2, j, k)] = -phi[at(&g, le - 1, j, k)];
        }
    }
    for (int k = GH; k < GH + p->nz; k++)
      for (int j = GH; j < GH + p->ny; j++)
        for (int i = GH; i < GH + p->nx; i++) {
          const long c = at(&g, i, j, k);
          for (int v = 0; v < 3; v++) {
            const long s = st[v];
            U[(5 + v) * N + c] += (w1[v] * (phi[c + s] - phi[c - s]) + w2[v] * (phi[c + 2 * s] - phi[c - 2 * s]));
          }
          U[4 * N + c] += phi[c] * divB[c];
        }
    exchange_fields(p, U, 5, 8);
    err1 = divb_pass(p, &g, U, w1, w2, divB);
  }
  err0 *= err_unit;
  err1 *= err_unit;
  const double err = err1 / err0;
  int next = n;
  if (err > p->divB_err) next += 1;
  else next -= 1;
  next = next < it_max ? next : it_max;
  next = next > 1 ? next : 1;
  p->divB_next_iter = next;
  p->divB_last_iters = iter;
  p->divB_err0 = err0;
  p->divB_err1 = err1;
}

/* --------------------------------------------------------------- full step */
int mo_step_ex(mo_params* p, const mo_eos* eos, double* U, double* U0, double* R, double* aux5, mo_fields* f) {
  geom g = geom_of(p);
  const long N = g.N;
  double* pres = aux5;
  double cfl = 0.0;
  const int spitzer = p->spitzer > 0.0;
  if (spitzer && !(f && f->sflx && f->sflx0 && f->Rflx && f->BgradT)) return -11;
  mo_save_cons(p, U, U0);
  if (spitzer)  /* SaveCons's heat-flux copy (src/Add_Sources_Integrate_SR.C:503-516) */
    for (int k = GH; k < GH + p->nz; k++)
      for (int j = GH; j < GH + p->ny; j++)
        for (int i = GH; i < GH + p->nx; i++) f->sflx0[at(&g, i, j, k)] = f->sflx[at(&g, i, j, k)];
  const int diag_step = p->diagnostics_next_step && p->diag;
  p->need_diagnostics = 0;
  for (int stage = 1; stage <= 4; stage++) {
    mo_cons_to_prim(p, eos, U, pres, aux5 + N, aux5 + 2 * N, aux5 + 3 * N, aux5 + 4 * N);
    if (stage == 1) mo_adjust_valf_max(p, U, pres, NULL);
    if (stage == 4 && diag_step) {  /* an output step's diagnostics (src/solver.C:264-289) */
      p->need_diagnostics = 1;
      for (long c = 0; c < 10 * N; c++) p->diag[c] = 0.0;
    }
    double dt_mhd = mo_mhd_residual_ex(p, U, pres, aux5 + N, R, f);
    if (stage == 1) {
      int rc = mo_sync_timestep(p, p->dt_rad, dt_mhd, &cfl);
      if (rc) return rc;
      p->last_cfl = cfl;
    }
    mo_source_integrate_ex(p, U, U0, R, stage, f);
    mo_boundaries_ex(p, eos, U, f, 1);
  }
  if (cfl <= p->CFL_tvd) {
    p->tvd_two_half_steps = 0;
    mo_tvdlimit(p, U, pres, p->dt);
  } else {
    p->tvd_two_half_steps = 1;
    mo_tvdlimit(p, U, pres, 0.5 * p->dt);
    mo_exchange_only(p, U);
    mo_tvdlimit(p, U, pres, 0.5 * p->dt);
  }
  if (p->divB_switch > 0) {
    if (!(f && f->phi && f->divB)) return -10;
    mo_clean_divB(p, U, f->phi, f->divB);
  }
  mo_tcheck(p, U);
  p->need_diagnostics = 0;
  p->diagnostics_next_step = 0;
  mo_boundaries_ex(p, eos, U, f, 0);
  p->time += p->dt;
  return 0;
}

int mo_step_divb(mo_params* p, const mo_eos* eos, double* U, double* U0, double* R, double* aux5, double* phi,
                 double* divB) {
  mo_fields f = {phi, divB, NULL, NULL, NULL, NULL};
  return mo_step_ex(p, eos, U, U0, R, aux5, &f);
}

int mo_step(mo_params* p, const mo_eos* eos, double* U, double* U0, double* R, double* aux5) {
  return mo_step_divb(p, eos, U, U0, R, aux5, NULL, NULL);
}
