// Host side of the gpumhd C ABI (include/gpumhd.h).
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <vector>

#include "../../include/gpumhd.h"
#include "gpumhd_adjoint.cuh"
#include "gpumhd_launch.cuh"

using namespace gpumhd;

struct gpumhd_ctx {
  gpumhd_params p;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool f32 = false;
  size_t rsz = 8;
  Consts c{};
  // device memory
  void* S[3] = {nullptr, nullptr, nullptr};   // state buffers (8N each)
  int iU = 0, iU0 = 1, iRes = 2;              // per-routine roles
  void* P[2] = {nullptr, nullptr};            // pressure buffers (N each)
  int iP = 0;
  void* aux[4] = {nullptr, nullptr, nullptr, nullptr};  // temp, ne, rhoi, amb
  void* T = nullptr;                          // TVD scratch of the per-routine path (8N)
  double* staging = nullptr;                  // host-layout transfer buffer (8N doubles)
  // asynchronous transfers: their own copy streams and two host-layout
  // buffers per direction (used in turn), ordered against the context's
  // stream by events (created on first use)
  cudaStream_t s_in = nullptr, s_out = nullptr;
  cudaStream_t s_cond = nullptr;              // captures the bodies of conditional graph nodes
  bool cond_tvd2 = false;                     // the captured step holds the second TVD pass in a conditional node
  double* astage_in[2] = {nullptr, nullptr};  // 8N doubles each
  double* astage_out[2] = {nullptr, nullptr};
  cudaEvent_t ev_in_ready[2] = {}, ev_in_free[2] = {}, ev_out_ready[2] = {}, ev_out_free[2] = {};
  unsigned n_up = 0, n_down = 0;              // asynchronous transfers so far (buffer turn)
  Dyn* dyn = nullptr;
  double* dt_hist = nullptr;
  int dt_hist_cap = 0;
  Dyn hdyn{};                                  // host mirror of the per-routine scalars
  // EOS
  double* d_xeps = nullptr;
  double* d_xlr = nullptr;
  float* d_tab[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  float4* d_pquad = nullptr;
  float* d_inv_xeps = nullptr;
  float* d_inv_xlr = nullptr;
  double* d_prof = nullptr;
  float* d_prof_f = nullptr;
  bool eos_loaded = false;
  // per-routine state flags
  bool have_pres = false;
  // fused path
  bool fused_ready = false;
  cudaGraphExec_t graph = nullptr;
  long long launches = 0;
  // TMA descriptors of the state (x, y, z, variable) and pressure (x, y, z)
  // buffers for the TMA / tensor-memory stage kernel; tma = false: plain loads
  bool tma = false;
  CUtensorMap mapS[3];
  CUtensorMap mapP[2];
  // launch shapes of the fused step (0: defaults); set by gpumhd_set_tuning / gpumhd_autotune
  int tune_zc = 0, tune_td = 0;
  // test hook of the TMA stage kernel's bounded waits (gpumhd_test_tma_wait)
  int tm_withhold_last = 0;
  long long tm_wait_cycles = 0;
  void* comp = nullptr;  // FP32 compensated mode: per-cell remainders of the RK update (8N floats)
  // diagnostics of an output step (RunData::need_diagnostics): tvar1..tvar8,
  // Qres, Qvis (GridData, 10 x N), allocated when first switched on
  void* diag = nullptr;
  bool need_diag = false;
  // Res holds zeros as far as the API is concerned, but the buffer was not
  // cleared: Source_Integrate_Tcheck and the fused steps leave it so, the next
  // MHD_Residual writes it without adding, any other access clears it first
  bool res_zero_pending = false;
  bool aux_pending = false;  // temp and ne hold ConsToPrim's density and internal energy (see field_ptr)
  void* phi = nullptr;   // divB cleaning potential (GridData::phi, N), persists between calls
  void* divb = nullptr;  // last divergence of B (GridData::divB, N)
  double* bnd_part = nullptr;  // per-plane sums of the physical x boundaries (nz * BND_NQ)
  // Spitzer conduction (N each): spt[0] the heat flux (step start = sflx0 of
  // the fused step), spt[1], spt[2] the stages' outputs (per routine: sflx0 and
  // Rflx), spt[3] the temperature, spt[4] the energy residual's share
  void* spt[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  float *d_d3 = nullptr, *d_eps3 = nullptr;  // inverse EOS tables
  float eos_hdr[14] = {0};                    // the EOS file's header (axes of the boundary lookups)
  char err[1024] = {0};
};

static char g_create_err[1024];

static int fail(gpumhd_ctx* ctx, int code, const char* fmt, ...) {
  char* buf = ctx ? ctx->err : g_create_err;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, 1024, fmt, ap);
  va_end(ap);
  return code;
}

#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) return fail(ctx, GPUMHD_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

static int check_launch(gpumhd_ctx* ctx, int n) {
  ctx->launches += n;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(ctx, GPUMHD_E_CUDA, "kernel launch: %s", cudaGetErrorString(e));
  return GPUMHD_OK;
}

extern "C" int gpumhd_default_params(gpumhd_params* p, int nx, int ny, int nz, double dx) {
  if (!p) return GPUMHD_E_INVALID;
  memset(p, 0, sizeof *p);
  p->nx = nx; p->ny = ny; p->nz = nz;
  p->periodic_x = 1;
  p->precision = 64;
  p->dx[0] = p->dx[1] = p->dx[2] = dx;
  p->CFL = 0.8; p->CFL_tvd = 0.95; p->dt = 0.0; p->autostep = 1; p->time = 0.0; p->outcad = 0.0;
  p->grav = 0.0; p->va_max = 1e7; p->va_adjust = 0.0; p->max_fill = 1000.;
  for (int i = 0; i < 4; i++) { p->tvd_h[i] = 2.0; p->tvd_cs[i] = 0.2; p->tvd_coeff[i] = 1.0; }
  const double tvd[10] = {1.0e-11, 1.0, 10.0, 0.2, 1.0, 1.0, 1.0, 1.0, 0.75, 100.0};
  for (int i = 0; i < 10; i++) p->tvd[i] = tvd[i];
  p->tvd_h_bnd[0] = p->tvd_h_bnd[1] = 1e-6;
  p->tvd_visc_bnd[0] = p->tvd_visc_bnd[1] = 1.0;
  p->tvd_eta_bnd[0] = p->tvd_eta_bnd[1] = 1.0;
  p->tchk[0] = 1.0e11; p->tchk[1] = 1.0e-16; p->tchk[2] = 4.0e15; p->tchk[3] = 100.0e5;
  p->rt_cfl = 0.5; p->rt_tstep = 0.0; p->rt_update = 1;
  p->tau0 = 1.0; p->dt_rad = 1e9;
  p->divB_switch = 0; p->divB_itmax = 5; p->divB_err = 0.2;  // off; the reference's test settings when on
  p->xbnd = 0; p->bnd_top = 0; p->bnd_bcrit = 1.0e10; p->bnd_eps_top = 0.0;  // include/physics.H defaults
  p->p_bc = -1.0; p->s_bc = -1.0;
  p->spitzer = 0.0;
  return GPUMHD_OK;
}

static inline double stdmax(double a, double b) { return (a < b) ? b : a; }
static inline double stdmin(double a, double b) { return (b < a) ? b : a; }

// Copy the run constants into the kernels' per-type sets (FP64: unchanged
// values; FP32: rounded once here).
template <class R>
static void fill_kc(const Consts& c, KC<R>& k, const R* prof) {
  k.eps_off = (R)c.eps_off; k.xeps0 = (R)c.xeps0; k.xlr0 = (R)c.xlr0; k.xepsN = (R)c.xepsN; k.xlrN = (R)c.xlrN;
  k.inv_del_eps = (R)c.inv_del_eps; k.inv_del_lr = (R)c.inv_del_lr; k.eps_max = (R)c.eps_max;
  k.rho_min = (R)c.rho_min; k.eps_min = (R)c.eps_min; k.rho_lev = (R)c.rho_lev; k.q_rho_max = (R)c.q_rho_max;
  k.visc_coeff_bot = (R)c.visc_coeff_bot; k.visc_slope_bot = (R)c.visc_slope_bot;
  k.visc_coeff_top = (R)c.visc_coeff_top; k.visc_slope_top = (R)c.visc_slope_top;
  k.eta_coeff_bot = (R)c.eta_coeff_bot; k.eta_slope_bot = (R)c.eta_slope_bot;
  k.eta_coeff_top = (R)c.eta_coeff_top; k.eta_slope_top = (R)c.eta_slope_top;
  k.B_par_diff = (R)c.B_par_diff; k.vhyp = (R)c.vhyp; k.pm_v = (R)c.pm_v; k.pm_B = (R)c.pm_B;
  k.CME_thresh = (R)c.CME_thresh;
  for (int i = 0; i < 4; i++) { k.tvd_h[i] = (R)c.tvd_h[i]; k.tvd_cs[i] = (R)c.tvd_cs[i]; k.tvd_coeff[i] = (R)c.tvd_coeff[i]; }
  k.CZ = (R)c.CZ; k.tchk_vmax = (R)c.tchk_vmax; k.tchk_eps_max = (R)c.tchk_eps_max; k.gx = (R)c.gx;
  for (int d = 0; d < 3; d++) { k.w1[d] = (R)c.w1[d]; k.w2[d] = (R)c.w2[d]; }
  k.eta = (R)c.eta;
  for (int d = 0; d < 3; d++) {
    k.ww0[d] = (R)(-30. / (12. * c.dx[d] * c.dx[d]));
    k.ww1[d] = (R)(16. / (12. * c.dx[d] * c.dx[d]));
    k.ww2[d] = (R)(-1. / (12. * c.dx[d] * c.dx[d]));
  }
  k.divb_fac = (R)c.divb_fac_d;
  k.del_eps = (R)(c.inv_del_eps > 0.0 ? 1.0 / c.inv_del_eps : 0.0);
  k.del_lr = (R)(c.inv_del_lr > 0.0 ? 1.0 / c.inv_del_lr : 0.0);
  k.divb_damp = (R)0.65;
  k.hfb = prof; k.hft = prof + c.g.sx; k.qft = prof + 2 * c.g.sx;
  k.has_visc_slope = (c.visc_slope_bot > 0.0 || c.visc_slope_top > 0.0);
  k.has_eta_slope = (c.eta_slope_bot > 0.0 || c.eta_slope_top > 0.0);
  k.has_vmax_lim = (c.vmax_lim > 0.0);
  k.has_vhyp = (c.vhyp > 0.0);
}

static void fill_kcs(gpumhd_ctx* ctx) {
  fill_kc<double>(ctx->c, ctx->c.kd, ctx->d_prof);
  fill_kc<float>(ctx->c, ctx->c.kf, ctx->d_prof_f);
}

// The physical boundaries' lookup constants from the EOS header, as
// eos_init forms its axes (src/eos_init.C:92-146), and B_crit, eps_top.
template <class R>
static void fill_bndk1(const float* h, const gpumhd_params& p, BndK<R>& b) {
  const int N_eps = (int)h[0], N_lr = (int)h[1], N_lp3 = (int)h[2], N_s3 = (int)h[3];
  const double eps0 = (double)h[4], eps1 = (double)h[5], lr0 = (double)h[6], lr1 = (double)h[7];
  const double lp0 = (double)h[8], lp1 = (double)h[9], s0 = (double)h[10], s1 = (double)h[11];
  const double del_eps = N_eps > 1 ? (eps1 - eps0) / (double(N_eps - 1)) : 1.0;
  const double del_lr = N_lr > 1 ? (lr1 - lr0) / (double(N_lr - 1)) : 1.0;
  const double del_lp3 = N_lp3 > 1 ? (lp1 - lp0) / (double(N_lp3 - 1)) : 1.0;
  const double del_s3 = N_s3 > 1 ? (s1 - s0) / (double(N_s3 - 1)) : 1.0;
  b.eps0 = (R)eps0; b.del_eps = (R)del_eps; b.inv_del_eps = (R)(1.0 / del_eps);
  b.lr0 = (R)lr0; b.del_lr = (R)del_lr; b.inv_del_lr = (R)(1.0 / del_lr);
  b.lp30 = (R)lp0; b.del_lp3 = (R)del_lp3; b.inv_del_lp3 = (R)(1.0 / del_lp3);
  b.s30 = (R)s0; b.del_s3 = (R)del_s3; b.inv_del_s3 = (R)(1.0 / del_s3);
  b.eps_off = (R)(double)h[12];
  b.ss_off = (R)(double)h[13];
  b.bcrit = (R)(p.bnd_bcrit / sqrt(8.0 * asin(1.0)));  // G to code units (src/boundary_pdmp_1_fftw3.C:90)
  b.eps_top = (R)p.bnd_eps_top;
}
static void fill_bndk(gpumhd_ctx* ctx) {
  fill_bndk1<double>(ctx->eos_hdr, ctx->p, ctx->c.bndd);
}

// Run constants derived from the parameters, computed with the host math
// library exactly as the reference computes them.
static int fill_consts(gpumhd_ctx* ctx) {
  const gpumhd_params& p = ctx->p;
  Consts& c = ctx->c;
  Geom& g = c.g;
  g.nx = p.nx; g.ny = p.ny; g.nz = p.nz;
  g.sx = p.nx + 2 * GH; g.sy = p.ny + 2 * GH; g.sz = p.nz + 2 * GH;
  g.N = (long long)g.sx * g.sy * g.sz;
  g.N32 = (unsigned)g.N;
  g.periodic_x = p.periodic_x ? 1 : 0;
  c.tm_withhold_last = ctx->tm_withhold_last;
  c.tm_wait_cycles = ctx->tm_wait_cycles;
  g.xmirror = (!p.periodic_x && p.xbnd == 0) ? 1 : 0;
  c.xbnd = (!p.periodic_x && p.xbnd == 1) ? 1 : 0;
  c.bnd_top = p.bnd_top;
  c.spitzer = p.spitzer;
  c.has_spitzer = p.spitzer > 0.0 ? 1 : 0;
  c.spt_sat_flx = (1.0 + 0.7) * pow(8.314e7, 1.5) * sqrt(1836.) / 8.0;  // src/mhdres_SR.C:42-46
  c.spt_rsp = ctx->spt[4];
  for (int d = 0; d < 3; d++) {
    c.dx[d] = p.dx[d];
    c.w1[d] = 8. / (12. * p.dx[d]);
    c.w2[d] = -1. / (12. * p.dx[d]);
    c.idx[d] = 1. / p.dx[d];
  }
  c.dxmin = p.dx[0];
  for (int d = 1; d < 3; d++) c.dxmin = stdmin(c.dxmin, p.dx[d]);
  c.rho_min = p.tchk[1];
  c.eps_min = p.tchk[0];
  c.rho_lev = pow(p.tvd[0], 2);
  c.rho_log = (int)p.tvd[1];
  c.q_rho_max = log(p.tvd[2]);
  c.visc_coeff_bot = stdmin(1.0, p.tvd_visc_bnd[0]);
  c.visc_slope_bot = stdmax(0.0, p.tvd_visc_bnd[0] - 1.0);
  c.visc_coeff_top = stdmin(1.0, p.tvd_visc_bnd[1]);
  c.visc_slope_top = stdmax(0.0, p.tvd_visc_bnd[1] - 1.0);
  c.eta_coeff_bot = stdmin(1.0, p.tvd_eta_bnd[0]);
  c.eta_slope_bot = stdmax(0.0, p.tvd_eta_bnd[0] - 1.0);
  c.eta_coeff_top = stdmin(1.0, p.tvd_eta_bnd[1]);
  c.eta_slope_top = stdmax(0.0, p.tvd_eta_bnd[1] - 1.0);
  c.B_par_diff = p.tvd[3]; c.vhyp = p.tvd[4];
  c.pm_v = p.tvd[6]; c.pm_B = p.tvd[7]; c.vmax_lim = p.tvd[8]; c.CME_thresh = p.tvd[9];
  for (int i = 0; i < 4; i++) { c.tvd_h[i] = p.tvd_h[i]; c.tvd_cs[i] = p.tvd_cs[i]; c.tvd_coeff[i] = p.tvd_coeff[i]; }
  c.need_coeff = (p.tvd_coeff[0] * p.tvd_coeff[1] * p.tvd_coeff[2] * p.tvd_coeff[3] != 1.0) ? 1 : 0;
  c.CZ = (double)(p.tau0 > 1.0e-5);
  c.tchk_vmax = p.tchk[3];
  c.tchk_eps_max = p.tchk[2];
  c.gx = -p.grav;
  // resistivity: time-step limit dt_diff_fac / eta, halved for CFL > 1 (src/mhdres_SR.C:47-62, 815-819)
  c.eta = p.eta;
  c.has_eta = p.eta > 0.0 ? 1 : 0;
  c.dt_res = 0.0;
  if (c.has_eta) {
    const double dt_diff_fac = 0.5 / (1. / (p.dx[0] * p.dx[0]) + 1. / (p.dx[1] * p.dx[1]) + 1. / (p.dx[2] * p.dx[2]));
    c.dt_res = dt_diff_fac / p.eta;
    if (p.CFL > 1) c.dt_res *= 0.5;
  }
  // divB cleaning constants (src/clean_divB.C:47-101): error unit 0.5/sum(1/dx)*3.5449 and
  // fac = coeff*min(dxmin, 0.4*dxmax)*dxmin, where dxmax is formed from the updated dxmin
  c.divb_on = p.divB_switch > 0 ? 1 : 0;
  c.divb_itmax = p.divB_itmax;
  c.divb_err = p.divB_err;
  {
    double eu = 0.0;
    for (int d = 0; d < 3; d++) eu += 1.0 / p.dx[d];
    c.divb_err_unit = 0.5 / eu * 3.5449;
    double dxmin = stdmin(p.dx[0], p.dx[1]);
    double dxmax = stdmax(p.dx[0], p.dx[1]);
    dxmin = stdmin(dxmin, p.dx[2]);
    dxmax = stdmax(dxmin, p.dx[2]);
    c.divb_fac_d = 1.0 * stdmin(dxmin, 0.4 * dxmax) * dxmin;
  }
  c.rt_cfl = p.rt_cfl;
  c.CFL = p.CFL; c.CFL_tvd = p.CFL_tvd; c.dt_rad = p.dt_rad; c.rt_tstep = p.rt_tstep; c.outcad = p.outcad;
  c.spt_cfl_dx = (1.8 < c.CFL ? 1.8 : c.CFL) * c.dxmin;  // smin(CFL, CFL_hyp) * dxmin
  c.va_max = p.va_max; c.va_adjust = p.va_adjust; c.max_fill = p.max_fill;
  c.autostep = p.autostep;
  // vertical boundary profiles of TVDlimit (src/tvdlimit_SR.C:132-149)
  const double h_bnd_bot = p.tvd_h_bnd[0] < 1 ? p.tvd_h_bnd[0] : p.tvd_h_bnd[0] / double(p.nx);
  const double h_bnd_top = p.tvd_h_bnd[1] < 1 ? p.tvd_h_bnd[1] : p.tvd_h_bnd[1] / double(p.nx);
  std::vector<double> prof(3 * (size_t)g.sx);
  const double gxmax0 = p.dx[0] * p.nx;
  for (int i = 0; i < g.sx; i++) {
    double hh = (0.0 + (0.5 + (i - GH)) * p.dx[0]) / gxmax0;
    double vv = stdmax(0.0, 1.0 - 0.5 * (1.0 - hh) / h_bnd_top);
    prof[g.sx + i] = stdmin(1.0, vv * vv);  // hft
    vv = stdmax(0.0, 1.0 - 0.5 * hh / h_bnd_bot);
    prof[i] = stdmin(1.0, vv * vv);          // hfb
    prof[2 * g.sx + i] = (hh < 1 - 2 * h_bnd_top) ? 1.0 : p.tvd[5];
  }
  if (!ctx->d_prof) CK(cudaMalloc(&ctx->d_prof, sizeof(double) * 3 * g.sx));
  CK(cudaMemcpy(ctx->d_prof, prof.data(), sizeof(double) * 3 * g.sx, cudaMemcpyHostToDevice));
  std::vector<float> proff(prof.begin(), prof.end());
  if (!ctx->d_prof_f) CK(cudaMalloc(&ctx->d_prof_f, sizeof(float) * 3 * g.sx));
  CK(cudaMemcpy(ctx->d_prof_f, proff.data(), sizeof(float) * 3 * g.sx, cudaMemcpyHostToDevice));
  c.hfb = ctx->d_prof;
  c.hft = ctx->d_prof + g.sx;
  c.qft = ctx->d_prof + 2 * g.sx;
  fill_kcs(ctx);
  fill_bndk(ctx);
  return GPUMHD_OK;
}

// Host restatement of the Adjust_Valf_Max limit update (src/Adjust_Valf_Max.C:83-144)
// from the five reduced statistics.
static void adjust_limits(gpumhd_ctx* ctx, const double st[5]) {
  const gpumhd_params& p = ctx->p;
  Dyn& d = ctx->hdyn;
  const double g0 = st[0], g1 = sqrt(st[1]), g2 = st[2];
  double va_max;
  if (p.va_adjust > 0.0) {
    const double cs_fac = 2.0, vv_fac = 3.0, eps_decay = 0.99;
    if (d.va_ini_flag) {
      d.v_lim = fmin(g0, p.tchk[3]);
      d.e_lim = fmin(g2, p.tchk[2]);
      d.va_max_old = 0.0;
      d.va_ini_flag = 0;
    } else {
      if (st[3] >= 4 * p.max_fill) d.v_lim *= 1.04;
      else if (st[3] >= p.max_fill) d.v_lim *= 1.01;
      else if (st[3] < 0.5 * p.max_fill) d.v_lim *= 0.99;
      if (st[4] >= 4 * p.max_fill) d.e_lim *= 1.04;
      else if (st[4] >= p.max_fill) d.e_lim *= 1.01;
      else if (st[4] < 0.5 * p.max_fill) d.e_lim *= 0.99;
    }
    va_max = fmax(p.va_max, p.va_adjust * vv_fac * g0);
    va_max = fmax(va_max, p.va_adjust * cs_fac * g1);
    va_max = fmax(va_max, d.va_max_old * eps_decay);
    d.v_lim = fmax(d.v_lim, p.va_max / vv_fac);
    d.v_lim = fmin(d.v_lim, p.tchk[3]);
    d.e_lim = fmax(d.e_lim, pow(p.va_max / cs_fac, 2));
    d.e_lim = fmin(d.e_lim, p.tchk[2]);
  } else {
    va_max = p.va_max;
    d.v_lim = p.tchk[3];
    d.e_lim = p.tchk[2];
  }
  d.inv_va2max = 1.0 / pow(va_max, 2);
  d.va_max_old = va_max;
  const double vml = p.tvd[8];
  d.vsqr_diff = vml < 1.0 ? pow(vml * d.v_lim, 2.0) : pow(vml, 2.0);
}

static int push_dyn(gpumhd_ctx* ctx) {
  const Consts& c = ctx->c;
  derive_one<float>(ctx->hdyn, c.dx, c.idx, c.rt_cfl, c.tchk_vmax, c.tchk_eps_max, ctx->hdyn.rf, c.spt_cfl_dx);
  derive_one<double>(ctx->hdyn, c.dx, c.idx, c.rt_cfl, c.tchk_vmax, c.tchk_eps_max, ctx->hdyn.rd, c.spt_cfl_dx);
  CK(cudaMemcpyAsync(ctx->dyn, &ctx->hdyn, sizeof(Dyn), cudaMemcpyHostToDevice, ctx->stream));
  return GPUMHD_OK;
}
static int pull_dyn(gpumhd_ctx* ctx) {
  CK(cudaMemcpyAsync(&ctx->hdyn, ctx->dyn, sizeof(Dyn), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return GPUMHD_OK;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled_fn() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(f);
  }
  return fn;
}

// Tensor maps of the three state and two pressure buffers, boxes of one plane
// tile with its halo ((TX+4) x (TY+4) x 1 [x 8 variables]).  TMA needs every
// row stride to be a multiple of 16 bytes: (nx+4)*sizeof(real) % 16 == 0.
template <class R>
static bool make_tensor_maps(gpumhd_ctx* ctx) {
  constexpr int TX = StageTileTm<R>::TX, TY = StageTileTm<R>::TY;
  const Geom& g = ctx->c.g;
  const cuuint64_t esz = sizeof(R);
  if (((cuuint64_t)g.sx * esz) % 16 != 0) return false;
  EncodeTiledFn enc = encode_tiled_fn();
  if (!enc) return false;
  const CUtensorMapDataType dt = sizeof(R) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  const cuuint64_t dimU[4] = {(cuuint64_t)g.sx, (cuuint64_t)g.sy, (cuuint64_t)g.sz, 8};
  const cuuint64_t strU[3] = {g.sx * esz, (cuuint64_t)g.sx * g.sy * esz, (cuuint64_t)g.N * esz};
  const cuuint32_t boxU[4] = {TX + 4, TY + 4, 1, 8};
  const cuuint32_t one[4] = {1, 1, 1, 1};
  for (int b = 0; b < 3; b++)
    if (enc(&ctx->mapS[b], dt, 4, ctx->S[b], dimU, strU, boxU, one, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
        CUDA_SUCCESS)
      return false;
  for (int b = 0; b < 2; b++)
    if (enc(&ctx->mapP[b], dt, 3, ctx->P[b], dimU, strU, boxU, one, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
        CUDA_SUCCESS)
      return false;
  return true;
}

// Tensor maps for a stage launch reading state buffer b and pressure buffer pb
// (both null: the plain-load kernel).
static const CUtensorMap* map_u(const gpumhd_ctx* ctx, int b) {
  return (ctx->tma && ctx->p.stage_kernel == 0) ? &ctx->mapS[b] : nullptr;
}
static const CUtensorMap* map_p(const gpumhd_ctx* ctx, int pb) {
  return (ctx->tma && ctx->p.stage_kernel == 0) ? &ctx->mapP[pb] : nullptr;
}

extern "C" int gpumhd_create(const gpumhd_params* p, int device, gpumhd_ctx** out) {
  gpumhd_ctx* ctx = nullptr;
  if (!p || !out) return fail(nullptr, GPUMHD_E_INVALID, "null argument");
  *out = nullptr;
  if (p->nx < 4 || p->ny < 4 || p->nz < 4) return fail(nullptr, GPUMHD_E_INVALID, "grid must have >= 4 interior cells per dimension");
  if (p->precision != 64 && p->precision != 32) return fail(nullptr, GPUMHD_E_INVALID, "precision must be 32 or 64");
  if (p->stage_kernel != 0 && p->stage_kernel != 1) return fail(nullptr, GPUMHD_E_INVALID, "stage_kernel must be 0 or 1");
  if (!(p->eta >= 0.0)) return fail(nullptr, GPUMHD_E_INVALID, "eta must be >= 0");
  if (p->divB_switch > 0 && !(p->divB_err >= 0.0)) return fail(nullptr, GPUMHD_E_INVALID, "divB_err must be >= 0");
  if (p->xbnd != 0 && p->xbnd != 1) return fail(nullptr, GPUMHD_E_INVALID, "xbnd must be 0 or 1");
  if (!(p->spitzer >= 0.0)) return fail(nullptr, GPUMHD_E_INVALID, "spitzer must be >= 0");
  if ((long long)(p->nx + 4) * (p->ny + 4) * (p->nz + 4) > GPUMHD_MAX_CELLS)
    return fail(nullptr, GPUMHD_E_INVALID, "grid too large: (nx+4)(ny+4)(nz+4) must not exceed %lld cells",
                (long long)GPUMHD_MAX_CELLS);
  if (!(p->dx[0] > 0 && p->dx[1] > 0 && p->dx[2] > 0)) return fail(nullptr, GPUMHD_E_INVALID, "dx must be positive");
  ctx = new gpumhd_ctx();
  ctx->p = *p;
  ctx->device = device;
  ctx->f32 = (p->precision == 32);
  ctx->rsz = ctx->f32 ? 4 : 8;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    fail(nullptr, GPUMHD_E_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e));
    delete ctx;
    return GPUMHD_E_CUDA;
  }
  int rc = GPUMHD_OK;
  do {
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) { rc = GPUMHD_E_CUDA; break; }
    if (cudaStreamCreateWithFlags(&ctx->s_cond, cudaStreamNonBlocking) != cudaSuccess) { rc = GPUMHD_E_CUDA; break; }
    e = ctx->f32 ? Launch<float>::setup() : Launch<double>::setup();
    if (e != cudaSuccess) { rc = fail(ctx, GPUMHD_E_CUDA, "kernel setup: %s", cudaGetErrorString(e)); break; }
    rc = fill_consts(ctx);
    if (rc) break;
    const long long N = ctx->c.g.N;
    for (int b = 0; b < 3; b++)
      if (cudaMalloc(&ctx->S[b], 8 * N * ctx->rsz) != cudaSuccess) { rc = GPUMHD_E_NOMEM; break; }
    if (rc) break;
    for (int b = 0; b < 2; b++)
      if (cudaMalloc(&ctx->P[b], N * ctx->rsz) != cudaSuccess) { rc = GPUMHD_E_NOMEM; break; }
    if (rc) break;
    if (cudaMalloc(&ctx->dyn, sizeof(Dyn)) != cudaSuccess) { rc = GPUMHD_E_NOMEM; break; }
    ctx->tma = ctx->f32 ? make_tensor_maps<float>(ctx) : make_tensor_maps<double>(ctx);
    for (int b = 0; b < 3; b++) cudaMemsetAsync(ctx->S[b], 0, 8 * N * ctx->rsz, ctx->stream);
    for (int b = 0; b < 2; b++) cudaMemsetAsync(ctx->P[b], 0, N * ctx->rsz, ctx->stream);
    memset(&ctx->hdyn, 0, sizeof(Dyn));
    ctx->hdyn.dt = p->dt;
    ctx->hdyn.time = p->time;
    ctx->hdyn.va_ini_flag = 1;
    ctx->hdyn.divb_next = 3;  // Clean_divB's static next_iter starts at 3 (src/clean_divB.C:51)
    ctx->hdyn.p_bc = p->p_bc;
    ctx->hdyn.s_bc = p->s_bc;
    ctx->hdyn.bnd_ini = 1;
    ctx->hdyn.inv_va2max = 1.0 / pow(p->va_max, 2);
    ctx->hdyn.v_lim = 0.0;
    ctx->hdyn.e_lim = 0.0;
    const double vml = p->tvd[8];
    ctx->hdyn.vsqr_diff = vml < 1.0 ? pow(vml * p->tchk[3], 2.0) : pow(vml, 2.0);
    rc = push_dyn(ctx);
    if (rc) break;
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) { rc = GPUMHD_E_CUDA; break; }
  } while (0);
  if (rc) {
    if (rc == GPUMHD_E_NOMEM) fail(nullptr, rc, "device allocation of the grid state failed");
    else fail(nullptr, rc, "%s", ctx->err[0] ? ctx->err : "context creation failed");
    gpumhd_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return GPUMHD_OK;
}

extern "C" int gpumhd_destroy(gpumhd_ctx* ctx) {
  if (!ctx) return GPUMHD_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
  for (void* q : ctx->S) cudaFree(q);
  for (void* q : ctx->P) cudaFree(q);
  for (void* q : ctx->aux) cudaFree(q);
  cudaFree(ctx->T);
  cudaFree(ctx->staging);
  if (ctx->s_in) cudaStreamSynchronize(ctx->s_in);
  if (ctx->s_out) cudaStreamSynchronize(ctx->s_out);
  for (int b = 0; b < 2; b++) {
    cudaFree(ctx->astage_in[b]);
    cudaFree(ctx->astage_out[b]);
    for (cudaEvent_t e : {ctx->ev_in_ready[b], ctx->ev_in_free[b], ctx->ev_out_ready[b], ctx->ev_out_free[b]})
      if (e) cudaEventDestroy(e);
  }
  if (ctx->s_in) cudaStreamDestroy(ctx->s_in);
  if (ctx->s_out) cudaStreamDestroy(ctx->s_out);
  if (ctx->s_cond) cudaStreamDestroy(ctx->s_cond);
  cudaFree(ctx->comp);
  cudaFree(ctx->diag);
  cudaFree(ctx->phi);
  cudaFree(ctx->divb);
  cudaFree(ctx->bnd_part);
  for (void* q : ctx->spt) cudaFree(q);
  cudaFree(ctx->d_d3); cudaFree(ctx->d_eps3);
  cudaFree(ctx->dyn);
  cudaFree(ctx->dt_hist);
  cudaFree(ctx->d_xeps);
  cudaFree(ctx->d_xlr);
  for (float* q : ctx->d_tab) cudaFree(q);
  cudaFree(ctx->d_pquad);
  cudaFree(ctx->d_inv_xeps);
  cudaFree(ctx->d_inv_xlr);
  cudaFree(ctx->d_prof);
  cudaFree(ctx->d_prof_f);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return GPUMHD_OK;
}

extern "C" const char* gpumhd_last_error(gpumhd_ctx* ctx) { return ctx ? ctx->err : g_create_err; }

extern "C" int gpumhd_get_params(gpumhd_ctx* ctx, gpumhd_params* p) {
  if (!ctx || !p) return GPUMHD_E_INVALID;
  *p = ctx->p;
  p->dt = ctx->hdyn.dt;
  p->time = ctx->hdyn.time;
  return GPUMHD_OK;
}

extern "C" int gpumhd_set_params(gpumhd_ctx* ctx, const gpumhd_params* p) {
  if (!ctx || !p) return GPUMHD_E_INVALID;
  if (p->nx != ctx->p.nx || p->ny != ctx->p.ny || p->nz != ctx->p.nz || p->precision != ctx->p.precision ||
      (p->periodic_x != 0) != (ctx->p.periodic_x != 0))
    return fail(ctx, GPUMHD_E_INVALID, "grid shape, boundaries and precision are fixed at creation");
  if (p->divB_switch > 0 && !(p->divB_err >= 0.0)) return fail(ctx, GPUMHD_E_INVALID, "divB_err must be >= 0");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  {
    int rc0 = pull_dyn(ctx);  // the device's copy is current (the cleaning's count lives there)
    if (rc0) return rc0;
  }
  const Consts keep = ctx->c;
  if (p->p_bc != ctx->p.p_bc || p->s_bc != ctx->p.s_bc) {
    ctx->hdyn.p_bc = p->p_bc;
    ctx->hdyn.s_bc = p->s_bc;
    ctx->hdyn.bnd_ini = 1;
  }
  ctx->p = *p;
  int rc = fill_consts(ctx);
  if (rc) return rc;
  // EOS pointers and values survive a parameter change
  Consts& c = ctx->c;
  c.N_eps = keep.N_eps; c.N_lr = keep.N_lr; c.eps_off = keep.eps_off; c.xeps0 = keep.xeps0; c.xlr0 = keep.xlr0;
  c.xepsN = keep.xepsN; c.xlrN = keep.xlrN; c.inv_del_eps = keep.inv_del_eps; c.inv_del_lr = keep.inv_del_lr;
  c.eps_max = keep.eps_max; c.xeps = keep.xeps; c.xlr = keep.xlr;
  for (int t = 0; t < 6; t++) c.tab[t] = keep.tab[t];
  c.pquad = keep.pquad; c.inv_exp_xeps = keep.inv_exp_xeps; c.inv_exp_xlr = keep.inv_exp_xlr;
  c.c_pres = keep.c_pres; c.c_temp = keep.c_temp; c.kb = keep.kb; c.mun_mh = keep.mun_mh;
  c.N_lp3 = keep.N_lp3; c.N_s3 = keep.N_s3;
  c.d3 = keep.d3; c.eps3 = keep.eps3;
  c.spt_rsp = ctx->spt[4];
  fill_kcs(ctx);
  fill_bndk(ctx);
  ctx->hdyn.dt = p->dt;
  ctx->hdyn.time = p->time;
  if (ctx->graph) { cudaGraphExecDestroy(ctx->graph); ctx->graph = nullptr; }
  return push_dyn(ctx);
}

// eos_init (src/eos_init.C:57-212): table axes in double from the float header,
// entries divided by del_eps*del_lr in double and stored as float.
extern "C" int gpumhd_eos_init(gpumhd_ctx* ctx, const char* path) {
  if (!ctx || !path) return GPUMHD_E_INVALID;
  FILE* f = fopen(path, "rb");
  if (!f) return fail(ctx, GPUMHD_E_EOS, "eos_init: EOS file - %s not found", path);
  float h[14];
  if (fread(h, sizeof(float), 14, f) != 14) { fclose(f); return fail(ctx, GPUMHD_E_EOS, "eos_init: short header in %s", path); }
  const int N_eps = (int)h[0], N_lr = (int)h[1], N_lp3 = (int)h[2], N_s3 = (int)h[3];
  if (N_eps < 2 || N_lr < 2 || N_eps > 100000 || N_lr > 100000 || N_lp3 < 0 || N_s3 < 0 || N_lp3 > 100000 ||
      N_s3 > 100000)
    { fclose(f); return fail(ctx, GPUMHD_E_EOS, "eos_init: bad table sizes in %s", path); }
  const double eps0 = (double)h[4], eps1 = (double)h[5], lr0 = (double)h[6], lr1 = (double)h[7];
  const double eps_off = (double)h[12];
  const double del_eps = (eps1 - eps0) / (double(N_eps - 1));
  const double del_lr = (lr1 - lr0) / (double(N_lr - 1));
  std::vector<double> xeps(N_eps), xlr(N_lr);
  for (int i = 0; i < N_eps; i++) xeps[i] = eps0 + del_eps * ((double)i);
  for (int i = 0; i < N_lr; i++) xlr[i] = lr0 + del_lr * ((double)i);
  const size_t n = (size_t)N_eps * N_lr;
  std::vector<float> buf(6 * n);
  if (fread(buf.data(), sizeof(float), 6 * n, f) != 6 * n) { fclose(f); return fail(ctx, GPUMHD_E_EOS, "eos_init: truncated tables in %s", path); }
  // inverse tables eps(p, s), rho(p, s) (src/eos_init.C:120-136, 181-198); a file
  // without them serves every boundary but the open bottom
  const double lp0 = (double)h[8], lp1 = (double)h[9], s0 = (double)h[10], s1 = (double)h[11];
  const size_t n3 = (size_t)N_lp3 * N_s3;
  std::vector<float> b3(2 * n3);
  const bool have_inv = N_lp3 >= 2 && N_s3 >= 2 && fread(b3.data(), sizeof(float), 2 * n3, f) == 2 * n3;
  fclose(f);
  std::vector<float> tab(6 * n);
  const double scale = del_eps * del_lr;
  for (int t = 0; t < 6; t++)
    for (int i = 0; i < N_eps; i++)
      for (int j = 0; j < N_lr; j++)
        tab[t * n + (size_t)i * N_lr + j] = (float)(((double)buf[t * n + (size_t)j * N_eps + i]) / scale);
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(ctx->d_xeps); cudaFree(ctx->d_xlr);
  for (float*& q : ctx->d_tab) { cudaFree(q); q = nullptr; }
  cudaFree(ctx->d_pquad); cudaFree(ctx->d_inv_xeps); cudaFree(ctx->d_inv_xlr);
  ctx->d_pquad = nullptr; ctx->d_inv_xeps = nullptr; ctx->d_inv_xlr = nullptr;
  CK(cudaMalloc(&ctx->d_xeps, sizeof(double) * N_eps));
  CK(cudaMalloc(&ctx->d_xlr, sizeof(double) * N_lr));
  CK(cudaMemcpy(ctx->d_xeps, xeps.data(), sizeof(double) * N_eps, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_xlr, xlr.data(), sizeof(double) * N_lr, cudaMemcpyHostToDevice));
  for (int t = 0; t < 6; t++) {
    CK(cudaMalloc(&ctx->d_tab[t], sizeof(float) * n));
    CK(cudaMemcpy(ctx->d_tab[t], tab.data() + t * n, sizeof(float) * n, cudaMemcpyHostToDevice));
  }
  if (ctx->f32) {
    // pressure patches: ln p = T00 + fe*a/.. re-expanded about the lower corner
    std::vector<float4> quad(n);
    for (int i = 0; i < N_eps - 1; i++)
      for (int j = 0; j < N_lr - 1; j++) {
        const double T00 = (double)tab[(size_t)i * N_lr + j] * scale;
        const double T01 = (double)tab[(size_t)i * N_lr + j + 1] * scale;
        const double T10 = (double)tab[(size_t)(i + 1) * N_lr + j] * scale;
        const double T11 = (double)tab[(size_t)(i + 1) * N_lr + j + 1] * scale;
        float4 q;
        q.x = (float)exp(T00);
        q.y = (float)((T10 - T00) / del_eps);
        q.z = (float)((T01 - T00) / del_lr);
        q.w = (float)((T11 - T10 - T01 + T00) / (del_eps * del_lr));
        quad[(size_t)i * N_lr + j] = q;
      }
    std::vector<float> ie(N_eps), ir(N_lr);
    for (int i = 0; i < N_eps; i++) ie[i] = (float)exp(-xeps[i]);
    for (int j = 0; j < N_lr; j++) ir[j] = (float)exp(-xlr[j]);
    CK(cudaMalloc(&ctx->d_pquad, sizeof(float4) * n));
    CK(cudaMemcpy(ctx->d_pquad, quad.data(), sizeof(float4) * n, cudaMemcpyHostToDevice));
    CK(cudaMalloc(&ctx->d_inv_xeps, sizeof(float) * N_eps));
    CK(cudaMalloc(&ctx->d_inv_xlr, sizeof(float) * N_lr));
    CK(cudaMemcpy(ctx->d_inv_xeps, ie.data(), sizeof(float) * N_eps, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_inv_xlr, ir.data(), sizeof(float) * N_lr, cudaMemcpyHostToDevice));
  }
  cudaFree(ctx->d_d3); cudaFree(ctx->d_eps3);
  ctx->d_d3 = ctx->d_eps3 = nullptr;
  if (have_inv) {
    const double del_lp3 = (lp1 - lp0) / (double(N_lp3 - 1));
    const double del_s3 = (s1 - s0) / (double(N_s3 - 1));
    std::vector<float> eps3(n3), d3(n3);
    const double sc3 = del_lp3 * del_s3;
    for (int i = 0; i < N_lp3; i++)
      for (int j = 0; j < N_s3; j++) {
        eps3[(size_t)i * N_s3 + j] = (float)(((double)b3[(size_t)j * N_lp3 + i]) / sc3);
        d3[(size_t)i * N_s3 + j] = (float)(((double)b3[n3 + (size_t)j * N_lp3 + i]) / sc3);
      }
    CK(cudaMalloc(&ctx->d_eps3, sizeof(float) * n3));
    CK(cudaMalloc(&ctx->d_d3, sizeof(float) * n3));
    CK(cudaMemcpy(ctx->d_eps3, eps3.data(), sizeof(float) * n3, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_d3, d3.data(), sizeof(float) * n3, cudaMemcpyHostToDevice));
  }
  Consts& c = ctx->c;
  c.N_lp3 = have_inv ? N_lp3 : 0;
  c.N_s3 = have_inv ? N_s3 : 0;
  c.d3 = ctx->d_d3; c.eps3 = ctx->d_eps3;
  memcpy(ctx->eos_hdr, h, sizeof(h));
  fill_bndk(ctx);
  c.N_eps = N_eps; c.N_lr = N_lr;
  c.eps_off = eps_off;
  c.xeps0 = xeps[0]; c.xlr0 = xlr[0]; c.xepsN = xeps[N_eps - 1]; c.xlrN = xlr[N_lr - 1];
  c.inv_del_eps = 1.0 / del_eps;
  c.inv_del_lr = 1.0 / del_lr;
  c.eps_max = exp(xeps[N_eps - 1]) - eps_off;
  c.xeps = ctx->d_xeps; c.xlr = ctx->d_xlr;
  for (int t = 0; t < 6; t++) c.tab[t] = ctx->d_tab[t];
  c.pquad = ctx->d_pquad; c.inv_exp_xeps = ctx->d_inv_xeps; c.inv_exp_xlr = ctx->d_inv_xlr;
  // ConsToPrim's ideal-gas constants (src/cons_to_prim.C:60-99)
  volatile double eos_gamma = 1.65, eos_mu = 0.62, eos_mu_n = 1.3, mh = 1.67262158e-24, kb = 1.380622e-16;
  const double Rgas = 8.314e7;
  c.c_temp = (eos_gamma - 1.) * eos_mu / Rgas;
  c.c_pres = (eos_gamma - 1.);
  c.kb = kb;
  c.mun_mh = eos_mu_n * mh;
  fill_kcs(ctx);
  ctx->eos_loaded = true;
  if (ctx->graph) { cudaGraphExecDestroy(ctx->graph); ctx->graph = nullptr; }
  return GPUMHD_OK;
}

// Clears Res where the context only marked it as zero.
static void materialize_res(gpumhd_ctx* ctx) {
  if (!ctx->res_zero_pending) return;
  cudaMemsetAsync(ctx->S[ctx->iRes], 0, 8 * ctx->c.g.N * ctx->rsz, ctx->stream);
  ctx->res_zero_pending = false;
}

// ConsToPrim's outputs temp, ne, rhoi, amb (t = 0..3), allocated zeroed on first use.
static void* aux_alloc(gpumhd_ctx* ctx, int t, int* rc) {
  void*& a = ctx->aux[t];
  if (!a) {
    if (cudaMalloc(&a, ctx->c.g.N * ctx->rsz) != cudaSuccess) { *rc = GPUMHD_E_NOMEM; return nullptr; }
    cudaMemsetAsync(a, 0, ctx->c.g.N * ctx->rsz, ctx->stream);
  }
  return a;
}

static void* field_ptr(gpumhd_ctx* ctx, int which, int* nf, int* rc) {
  *rc = GPUMHD_OK;
  if (which >= 0 && which <= 2) {
    *nf = 8;
    if (which == 2) materialize_res(ctx);
    return ctx->S[which == 0 ? ctx->iU : (which == 1 ? ctx->iU0 : ctx->iRes)];
  }
  *nf = 1;
  if (which == 3) return ctx->P[ctx->iP];
  if (which == 10) {
    void*& a = ctx->spt[0];
    if (!a) {
      if (cudaMalloc(&a, ctx->c.g.N * ctx->rsz) != cudaSuccess) { *rc = GPUMHD_E_NOMEM; return nullptr; }
      cudaMemsetAsync(a, 0, ctx->c.g.N * ctx->rsz, ctx->stream);
    }
    return a;
  }
  if (which == 8 || which == 9) {
    void*& a = which == 8 ? ctx->phi : ctx->divb;
    if (!a) {
      if (cudaMalloc(&a, ctx->c.g.N * ctx->rsz) != cudaSuccess) { *rc = GPUMHD_E_NOMEM; return nullptr; }
      cudaMemsetAsync(a, 0, ctx->c.g.N * ctx->rsz, ctx->stream);
    }
    return a;
  }
  if (which >= 11 && which <= 20) {  // diagnostics: tvar1..tvar8, Qres, Qvis
    if (!ctx->diag) {
      if (cudaMalloc(&ctx->diag, 10 * ctx->c.g.N * ctx->rsz) != cudaSuccess) { *rc = GPUMHD_E_NOMEM; return nullptr; }
      cudaMemsetAsync(ctx->diag, 0, 10 * ctx->c.g.N * ctx->rsz, ctx->stream);
    }
    return (char*)ctx->diag + (size_t)(which - 11) * ctx->c.g.N * ctx->rsz;
  }
  if (which >= 4 && which <= 7) {
    void* a = aux_alloc(ctx, which - 4, rc);
    if (a && ctx->aux_pending) {  // ConsToPrim left its EOS inputs: form the outputs now
      if (ctx->f32)
        Launch<float>::aux_of_snapshot(ctx->c, (float*)ctx->aux[0], (float*)ctx->aux[1], (float*)ctx->aux[2],
                                       (float*)ctx->aux[3], ctx->stream);
      else
        Launch<double>::aux_of_snapshot(ctx->c, (double*)ctx->aux[0], (double*)ctx->aux[1], (double*)ctx->aux[2],
                                        (double*)ctx->aux[3], ctx->stream);
      ctx->aux_pending = false;
      ctx->launches += 1;
      if (cudaGetLastError() != cudaSuccess) { *rc = GPUMHD_E_CUDA; return nullptr; }
    }
    return a;
  }
  *rc = GPUMHD_E_INVALID;
  return nullptr;
}

// phi and divB exist (zero-initialised) before the first cleaning.
static int ensure_divb(gpumhd_ctx* ctx) {
  int nf, rc;
  field_ptr(ctx, 8, &nf, &rc);
  if (rc) return fail(ctx, rc, "allocation of the divB cleaning fields failed");
  field_ptr(ctx, 9, &nf, &rc);
  if (rc) return fail(ctx, rc, "allocation of the divB cleaning fields failed");
  return GPUMHD_OK;
}

// Spitzer conduction's buffers (zero-initialised).
static int ensure_spitzer(gpumhd_ctx* ctx) {
  if (!ctx->c.has_spitzer) return GPUMHD_OK;
  if (!ctx->eos_loaded) return fail(ctx, GPUMHD_E_ORDER, "Spitzer conduction before eos_init");
  for (int b = 0; b < 5; b++)
    if (!ctx->spt[b]) {
      CK(cudaMalloc(&ctx->spt[b], ctx->c.g.N * ctx->rsz));
      CK(cudaMemsetAsync(ctx->spt[b], 0, ctx->c.g.N * ctx->rsz, ctx->stream));
    }
  ctx->c.spt_rsp = ctx->spt[4];
  return GPUMHD_OK;
}

// The physical x boundaries need the EOS's inverse tables and a plane-sum buffer.
static int ensure_bnd(gpumhd_ctx* ctx) {
  if (!ctx->c.xbnd) return GPUMHD_OK;
  if (!ctx->eos_loaded) return fail(ctx, GPUMHD_E_ORDER, "physical x boundaries before eos_init");
  if (!ctx->c.d3) return fail(ctx, GPUMHD_E_EOS, "the open bottom needs the EOS file's inverse tables");
  if (!ctx->bnd_part) {
    const long long nb = (long long)((ctx->c.g.ny + BND_BX - 1) / BND_BX) * ((ctx->c.g.nz + BND_BY - 1) / BND_BY);
    CK(cudaMalloc(&ctx->bnd_part, sizeof(double) * BND_NQ * nb));
  }
  return GPUMHD_OK;
}

// MURaM's physical x boundaries on state buffer U (P, cmax: see Launch::bc).
static int enqueue_bc(gpumhd_ctx* ctx, void* U, void* P, int with_cmax) {
  void* sf = ctx->c.has_spitzer ? ctx->spt[0] : nullptr;  // the heat flux's boundary values too
  if (ctx->f32)
    return Launch<float>::bc(ctx->c, (float*)U, (float*)P, ctx->dyn, ctx->bnd_part, with_cmax, ctx->stream, (float*)sf);
  return Launch<double>::bc(ctx->c, (double*)U, (double*)P, ctx->dyn, ctx->bnd_part, with_cmax, ctx->stream,
                            (double*)sf);
}

static int ensure_staging(gpumhd_ctx* ctx) {
  if (!ctx->staging) CK(cudaMalloc(&ctx->staging, sizeof(double) * 8 * ctx->c.g.N));
  return GPUMHD_OK;
}

// Host element type H: double (MURaM's default build) or float (SINGLE_PRECISION).
template <class H>
static int upload_impl(gpumhd_ctx* ctx, int which, const H* host) {
  if (!ctx || !host) return GPUMHD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  int nf, rc;
  void* dst = field_ptr(ctx, which, &nf, &rc);
  if (rc) return fail(ctx, rc, "upload: bad field %d", which);
  rc = ensure_staging(ctx);
  if (rc) return rc;
  const long long N = ctx->c.g.N;
  H* const stg = reinterpret_cast<H*>(ctx->staging);
  CK(cudaMemcpyAsync(stg, host, sizeof(H) * nf * N, cudaMemcpyHostToDevice, ctx->stream));
  if (ctx->f32) Launch<float>::aos_to_soa(N, nf, stg, (float*)dst, ctx->stream);
  else Launch<double>::aos_to_soa(N, nf, stg, (double*)dst, ctx->stream);
  if (which == 0) {
    ctx->fused_ready = false;
    if (ctx->comp) CK(cudaMemsetAsync(ctx->comp, 0, sizeof(Rem<float>) * 8 * N, ctx->stream));
  }
  if (which == 3) ctx->have_pres = true;
  return check_launch(ctx, 1);
}
extern "C" int gpumhd_upload(gpumhd_ctx* ctx, int which, const double* host) { return upload_impl(ctx, which, host); }
extern "C" int gpumhd_upload_f32(gpumhd_ctx* ctx, int which, const float* host) { return upload_impl(ctx, which, host); }

// dst's state (U) = periodic tiling of src's state; same precision, and dst's
// interior sizes multiples of src's.  Ghosts filled with dst's boundary rule.
extern "C" int gpumhd_tile_from(gpumhd_ctx* ctx, gpumhd_ctx* src) {
  if (!ctx || !src || ctx->device != src->device) return GPUMHD_E_INVALID;
  const Geom& gd = ctx->c.g;
  const Geom& gs = src->c.g;
  if (ctx->f32 != src->f32 || gd.nx % gs.nx || gd.ny % gs.ny || gd.nz % gs.nz)
    return fail(ctx, GPUMHD_E_INVALID, "tile_from: precision differs or sizes are not multiples");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(src->stream));
  if (ctx->f32) {
    Launch<float>::tile_state(gd, gs, (const float*)src->S[src->iU], (float*)ctx->S[ctx->iU], ctx->stream);
    Launch<float>::fill_ghosts(ctx->c, (float*)ctx->S[ctx->iU], 8, 1, ctx->stream);
  } else {
    Launch<double>::tile_state(gd, gs, (const double*)src->S[src->iU], (double*)ctx->S[ctx->iU], ctx->stream);
    Launch<double>::fill_ghosts(ctx->c, (double*)ctx->S[ctx->iU], 8, 1, ctx->stream);
  }
  if (ctx->comp) CK(cudaMemsetAsync(ctx->comp, 0, sizeof(Rem<float>) * 8 * gd.N, ctx->stream));
  ctx->fused_ready = false;
  return check_launch(ctx, 2);
}

// The asynchronous transfers' streams, events and buffers.
static int ensure_async(gpumhd_ctx* ctx) {
  if (ctx->s_in) return GPUMHD_OK;
  const size_t B = sizeof(double) * 8 * (size_t)ctx->c.g.N;
  for (int b = 0; b < 2; b++) {
    CK(cudaMalloc(&ctx->astage_in[b], B));
    CK(cudaMalloc(&ctx->astage_out[b], B));
    for (cudaEvent_t* e : {&ctx->ev_in_ready[b], &ctx->ev_in_free[b], &ctx->ev_out_ready[b], &ctx->ev_out_free[b]})
      CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  }
  CK(cudaStreamCreateWithFlags(&ctx->s_out, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&ctx->s_in, cudaStreamNonBlocking));
  return GPUMHD_OK;
}

// Upload through the copy-in stream: the host-to-device copy waits only for
// the conversion of the upload before last (two buffers in turn), so it
// overlaps the steps enqueued before it; the conversion into the field runs
// in stream order.
template <class H>
static int upload_async_impl(gpumhd_ctx* ctx, int which, const H* host) {
  if (!ctx || !host) return GPUMHD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  int nf, rc;
  void* dst = field_ptr(ctx, which, &nf, &rc);
  if (rc) return fail(ctx, rc, "upload_async: bad field %d", which);
  rc = ensure_async(ctx);
  if (rc) return rc;
  const long long N = ctx->c.g.N;
  const int b = (int)(ctx->n_up++ & 1u);
  CK(cudaStreamWaitEvent(ctx->s_in, ctx->ev_in_free[b], 0));
  H* const stg = reinterpret_cast<H*>(ctx->astage_in[b]);
  CK(cudaMemcpyAsync(stg, host, sizeof(H) * nf * N, cudaMemcpyHostToDevice, ctx->s_in));
  CK(cudaEventRecord(ctx->ev_in_ready[b], ctx->s_in));
  CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_in_ready[b], 0));
  if (ctx->f32) Launch<float>::aos_to_soa(N, nf, stg, (float*)dst, ctx->stream);
  else Launch<double>::aos_to_soa(N, nf, stg, (double*)dst, ctx->stream);
  CK(cudaEventRecord(ctx->ev_in_free[b], ctx->stream));
  if (which == 0) {
    ctx->fused_ready = false;
    if (ctx->comp) CK(cudaMemsetAsync(ctx->comp, 0, sizeof(Rem<float>) * 8 * N, ctx->stream));
  }
  if (which == 3) ctx->have_pres = true;
  return check_launch(ctx, 1);
}
extern "C" int gpumhd_upload_async(gpumhd_ctx* ctx, int which, const double* host) {
  return upload_async_impl(ctx, which, host);
}
extern "C" int gpumhd_upload_async_f32(gpumhd_ctx* ctx, int which, const float* host) {
  return upload_async_impl(ctx, which, host);
}

// Download through the copy-out stream: the field is converted in stream
// order into a copy-out buffer (once the download before last has left it)
// and copied to the host while later steps run.
template <class H>
static int download_async_impl(gpumhd_ctx* ctx, int which, H* host) {
  if (!ctx || !host) return GPUMHD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  int nf, rc;
  void* src = field_ptr(ctx, which, &nf, &rc);
  if (rc) return fail(ctx, rc, "download_async: bad field %d", which);
  rc = ensure_async(ctx);
  if (rc) return rc;
  const long long N = ctx->c.g.N;
  const int b = (int)(ctx->n_down++ & 1u);
  CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_out_free[b], 0));
  H* const stg = reinterpret_cast<H*>(ctx->astage_out[b]);
  if (ctx->f32) Launch<float>::soa_to_aos(N, nf, (const float*)src, stg, ctx->stream);
  else Launch<double>::soa_to_aos(N, nf, (const double*)src, stg, ctx->stream);
  rc = check_launch(ctx, 1);
  if (rc) return rc;
  CK(cudaEventRecord(ctx->ev_out_ready[b], ctx->stream));
  CK(cudaStreamWaitEvent(ctx->s_out, ctx->ev_out_ready[b], 0));
  CK(cudaMemcpyAsync(host, stg, sizeof(H) * nf * N, cudaMemcpyDeviceToHost, ctx->s_out));
  CK(cudaEventRecord(ctx->ev_out_free[b], ctx->s_out));
  return GPUMHD_OK;
}
extern "C" int gpumhd_download_async(gpumhd_ctx* ctx, int which, double* host) {
  return download_async_impl(ctx, which, host);
}
extern "C" int gpumhd_download_async_f32(gpumhd_ctx* ctx, int which, float* host) {
  return download_async_impl(ctx, which, host);
}

template <class H>
static int download_impl(gpumhd_ctx* ctx, int which, H* host) {
  if (!ctx || !host) return GPUMHD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  int nf, rc;
  void* src = field_ptr(ctx, which, &nf, &rc);
  if (rc) return fail(ctx, rc, "download: bad field %d", which);
  rc = ensure_staging(ctx);
  if (rc) return rc;
  const long long N = ctx->c.g.N;
  H* const stg = reinterpret_cast<H*>(ctx->staging);
  if (ctx->f32) Launch<float>::soa_to_aos(N, nf, (const float*)src, stg, ctx->stream);
  else Launch<double>::soa_to_aos(N, nf, (const double*)src, stg, ctx->stream);
  rc = check_launch(ctx, 1);
  if (rc) return rc;
  CK(cudaMemcpyAsync(host, stg, sizeof(H) * nf * N, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return GPUMHD_OK;
}
extern "C" int gpumhd_download(gpumhd_ctx* ctx, int which, double* host) { return download_impl(ctx, which, host); }
extern "C" int gpumhd_download_f32(gpumhd_ctx* ctx, int which, float* host) { return download_impl(ctx, which, host); }

#define DISPATCH(call_f, call_d) (ctx->f32 ? (call_f) : (call_d))

extern "C" int gpumhd_set_need_diagnostics(gpumhd_ctx* ctx, int on) {
  if (!ctx) return GPUMHD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  if (on) {  // src/solver.C:271-289: the arrays start the output step at zero
    int nf, rc;
    field_ptr(ctx, 11, &nf, &rc);
    if (rc) return fail(ctx, rc, "diagnostics allocation failed");
    CK(cudaMemsetAsync(ctx->diag, 0, 10 * ctx->c.g.N * ctx->rsz, ctx->stream));
  }
  ctx->need_diag = on != 0;
  return GPUMHD_OK;
}

extern "C" int gpumhd_save_cons(gpumhd_ctx* ctx) {
  if (!ctx) return GPUMHD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  if (ctx->f32) Launch<float>::save_cons(ctx->c, (const float*)ctx->S[ctx->iU], (float*)ctx->S[ctx->iU0], ctx->stream);
  else Launch<double>::save_cons(ctx->c, (const double*)ctx->S[ctx->iU], (double*)ctx->S[ctx->iU0], ctx->stream);
  if (ctx->c.has_spitzer) {  // sflx0 = sflx (src/Add_Sources_Integrate_SR.C:503-516)
    int rc = ensure_spitzer(ctx);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->spt[1], ctx->spt[0], ctx->c.g.N * ctx->rsz, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  return check_launch(ctx, 1);
}

extern "C" int gpumhd_cons_to_prim(gpumhd_ctx* ctx) {
  if (!ctx) return GPUMHD_E_INVALID;
  if (!ctx->eos_loaded) return fail(ctx, GPUMHD_E_ORDER, "ConsToPrim before eos_init");
  CK(cudaSetDevice(ctx->device));
  int rc = GPUMHD_OK;
  void* a[4];
  for (int t = 0; t < 4; t++) {
    a[t] = aux_alloc(ctx, t, &rc);
    if (rc) return fail(ctx, rc, "allocation of the EOS output fields failed");
  }
  // Temperature, n_e, rho_i and amb are read only when downloaded (or by the
  // Spitzer residual): the kernel stores the density and internal energy they
  // come from, and the first access forms them (field_ptr).  With Spitzer
  // conduction, which reads the temperature every stage, they are formed here.
  const bool snap = !ctx->c.has_spitzer;
  if (ctx->f32)
    Launch<float>::cons_to_prim(ctx->c, (float*)ctx->S[ctx->iU], (float*)ctx->P[ctx->iP], (float*)a[0], (float*)a[1],
                                (float*)a[2], (float*)a[3], snap, ctx->stream);
  else
    Launch<double>::cons_to_prim(ctx->c, (double*)ctx->S[ctx->iU], (double*)ctx->P[ctx->iP], (double*)a[0],
                                 (double*)a[1], (double*)a[2], (double*)a[3], snap, ctx->stream);
  ctx->aux_pending = snap;
  ctx->have_pres = true;
  ctx->fused_ready = false;
  return check_launch(ctx, 1);
}

static int reset_accumulators(gpumhd_ctx* ctx) {
  ctx->hdyn.cmax_bits = 0;
  ctx->hdyn.stat_max_bits[0] = ctx->hdyn.stat_max_bits[1] = ctx->hdyn.stat_max_bits[2] = 0;
  ctx->hdyn.stat_cnt[0] = ctx->hdyn.stat_cnt[1] = 0;
  return push_dyn(ctx);
}

static double bits_to_double(unsigned long long b) {
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
}

extern "C" int gpumhd_adjust_valf_max(gpumhd_ctx* ctx) {
  if (!ctx) return GPUMHD_E_INVALID;
  if (!ctx->have_pres) return fail(ctx, GPUMHD_E_ORDER, "Adjust_Valf_Max needs ConsToPrim first");
  CK(cudaSetDevice(ctx->device));
  int rc = reset_accumulators(ctx);
  if (rc) return rc;
  if (ctx->f32) Launch<float>::adjust_stats(ctx->c, (const float*)ctx->S[ctx->iU], (const float*)ctx->P[ctx->iP], ctx->dyn, ctx->stream);
  else Launch<double>::adjust_stats(ctx->c, (const double*)ctx->S[ctx->iU], (const double*)ctx->P[ctx->iP], ctx->dyn, ctx->stream);
  rc = check_launch(ctx, 1);
  if (rc) return rc;
  rc = pull_dyn(ctx);
  if (rc) return rc;
  double st[5];
  for (int q = 0; q < 3; q++) st[q] = bits_to_double(ctx->hdyn.stat_max_bits[q]);
  st[3] = (double)ctx->hdyn.stat_cnt[0];
  st[4] = (double)ctx->hdyn.stat_cnt[1];
  adjust_limits(ctx, st);
  return push_dyn(ctx);
}

extern "C" int gpumhd_get_limits(gpumhd_ctx* ctx, double* inv_va2max, double* v_lim, double* e_lim) {
  if (!ctx) return GPUMHD_E_INVALID;
  if (inv_va2max) *inv_va2max = ctx->hdyn.inv_va2max;
  if (v_lim) *v_lim = ctx->hdyn.v_lim;
  if (e_lim) *e_lim = ctx->hdyn.e_lim;
  return GPUMHD_OK;
}

extern "C" int gpumhd_mhd_residual(gpumhd_ctx* ctx, double* dt_mhd) {
  if (!ctx) return GPUMHD_E_INVALID;
  if (!ctx->have_pres) return fail(ctx, GPUMHD_E_ORDER, "MHD_Residual needs ConsToPrim first");
  CK(cudaSetDevice(ctx->device));
  int rc = reset_accumulators(ctx);
  if (rc) return rc;
  int nl = 2;
  if (ctx->c.has_spitzer) {
    // heat flux residual into Rflx (spt[2]) and the energy share, from the
    // primitive state and ConsToPrim's temperature
    rc = ensure_spitzer(ctx);
    if (rc) return rc;
    int nf;
    void* Tm = field_ptr(ctx, 4, &nf, &rc);
    if (rc) return fail(ctx, rc, "temperature field allocation failed");
    if (ctx->f32)
      Launch<float>::spitzer(ctx->c, (const float*)ctx->S[ctx->iU], true, (const float*)Tm, (const float*)ctx->spt[0],
                             nullptr, nullptr, (float*)ctx->spt[2], (float*)ctx->spt[4], ctx->dyn, 0, ctx->stream);
    else
      Launch<double>::spitzer(ctx->c, (const double*)ctx->S[ctx->iU], true, (const double*)Tm,
                              (const double*)ctx->spt[0], nullptr, nullptr, (double*)ctx->spt[2],
                              (double*)ctx->spt[4], ctx->dyn, 0, ctx->stream);
    nl += 1;
  }
  // Res += residual; a Res only marked as zero is written without being read
  const void* res_in = ctx->res_zero_pending ? nullptr : ctx->S[ctx->iRes];
  ctx->res_zero_pending = false;
  if (ctx->f32) {
    Launch<float>::stage(ctx->c, (const float*)ctx->S[ctx->iU], (const float*)ctx->P[ctx->iP], (const float*)res_in,
                         nullptr, nullptr, (float*)ctx->S[ctx->iRes], ctx->dyn, 0, true, 0, ctx->stream,
                         map_u(ctx, ctx->iU), map_p(ctx, ctx->iP));
    Launch<float>::cmax_faces(ctx->c, (const float*)ctx->S[ctx->iU], (const float*)ctx->P[ctx->iP], ctx->dyn, ctx->stream);
  } else {
    Launch<double>::stage(ctx->c, (const double*)ctx->S[ctx->iU], (const double*)ctx->P[ctx->iP],
                          (const double*)res_in, nullptr, nullptr, (double*)ctx->S[ctx->iRes], ctx->dyn, 0, true, 0,
                          ctx->stream, map_u(ctx, ctx->iU), map_p(ctx, ctx->iP));
    Launch<double>::cmax_faces(ctx->c, (const double*)ctx->S[ctx->iU], (const double*)ctx->P[ctx->iP], ctx->dyn, ctx->stream);
  }
  if (ctx->need_diag) {  // tvar1..3 of the output step
    if (ctx->f32)
      Launch<float>::diag_residual(ctx->c, (const float*)ctx->S[ctx->iU], (const float*)ctx->P[ctx->iP],
                                   ctx->c.has_spitzer ? (const float*)ctx->spt[0] : nullptr, (float*)ctx->diag,
                                   ctx->dyn, ctx->stream);
    else
      Launch<double>::diag_residual(ctx->c, (const double*)ctx->S[ctx->iU], (const double*)ctx->P[ctx->iP],
                                    ctx->c.has_spitzer ? (const double*)ctx->spt[0] : nullptr, (double*)ctx->diag,
                                    ctx->dyn, ctx->stream);
    nl += 1;
  }
  rc = check_launch(ctx, nl);
  if (rc) return rc;
  rc = pull_dyn(ctx);
  if (rc) return rc;
  if (ctx->hdyn.err == ERR_WAIT_TIMEOUT) {  // the residual is incomplete; report it once
    ctx->hdyn.err = 0;
    push_dyn(ctx);
    return fail(ctx, GPUMHD_E_CUDA, "a device-side wait for a TMA copy timed out");
  }
  const double cmax = bits_to_double(ctx->hdyn.cmax_bits);
  if (dt_mhd) {
    double dt = ctx->c.dxmin / cmax;
    if (ctx->c.has_eta) dt = stdmin(dt, ctx->c.dt_res);
    *dt_mhd = dt;
  }
  return GPUMHD_OK;
}

// Sync_timestep (src/solver.C:487-548) for one rank.
extern "C" int gpumhd_sync_timestep(gpumhd_ctx* ctx, double dt_rad, double dt_mhd, double* cfl) {
  if (!ctx) return GPUMHD_E_INVALID;
  const gpumhd_params& p = ctx->p;
  auto bad = [](double a) { return (a != a) || (a <= 0.) || (a == INFINITY); };
  double r0 = dt_rad, r1 = dt_mhd;
  if (bad(r0)) return fail(ctx, GPUMHD_E_BAD_DT, "Invalid time step: dt_rad = %g", r0);
  if (bad(r1)) return fail(ctx, GPUMHD_E_BAD_DT, "Invalid time step: dt_mhd = %g", r1);
  const double dt_min_rt = p.rt_tstep * p.CFL * r1;
  if (r0 < dt_min_rt) r0 = stdmax(r0, dt_min_rt);
  const double dt_min = stdmin(r0, r1);
  double dt = stdmin(r0, p.CFL * r1);
  if (p.outcad > 0) {
    const double num = ctx->hdyn.time / p.outcad;
    const int ce = (int)num;
    const double rem = (num == (double)ce) ? 0.0 : (ce + 1) * p.outcad - ctx->hdyn.time;
    if (rem > 0.0) dt = stdmin(dt, rem);
  }
  if (p.autostep) ctx->hdyn.dt = dt;
  const double c = ctx->hdyn.dt / dt_min;
  ctx->hdyn.cfl = c;
  if (cfl) *cfl = c;
  if (c >= 2.) return fail(ctx, GPUMHD_E_CFL, "Invalid time step: CFL = %g", c);
  return push_dyn(ctx);
}

extern "C" int gpumhd_source_integrate_tcheck(gpumhd_ctx* ctx, int stage) {
  if (!ctx || stage < 1 || stage > 4) return GPUMHD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  materialize_res(ctx);  // it reads Res
  const double invdt = 1.0 / ctx->hdyn.dt;  // src/Add_Sources_Integrate_SR.C:84
  if (ctx->f32)
    Launch<float>::source_integrate(ctx->c, (float*)ctx->S[ctx->iU], (const float*)ctx->S[ctx->iU0],
                                    (float*)ctx->S[ctx->iRes], ctx->dyn, stage, ctx->stream,
                                    ctx->need_diag ? (float*)ctx->diag : nullptr, (float)invdt);
  else
    Launch<double>::source_integrate(ctx->c, (double*)ctx->S[ctx->iU], (const double*)ctx->S[ctx->iU0],
                                     (double*)ctx->S[ctx->iRes], ctx->dyn, stage, ctx->stream,
                                     ctx->need_diag ? (double*)ctx->diag : nullptr, invdt);
  ctx->res_zero_pending = true;  // Res = 0 (src/Add_Sources_Integrate_SR.C:394-408), not stored
  int nl = 1;
  if (ctx->c.has_spitzer) {  // sflx = sflx0 + wdt*Rflx, Rflx = 0 (src/Add_Sources_Integrate_SR.C:410-419)
    int rc = ensure_spitzer(ctx);
    if (rc) return rc;
    if (ctx->f32)
      Launch<float>::sflx_update(ctx->c, (float*)ctx->spt[0], (const float*)ctx->spt[1], (float*)ctx->spt[2], ctx->dyn,
                                 stage, ctx->stream);
    else
      Launch<double>::sflx_update(ctx->c, (double*)ctx->spt[0], (const double*)ctx->spt[1], (double*)ctx->spt[2],
                                  ctx->dyn, stage, ctx->stream);
    nl += 1;
  }
  return check_launch(ctx, nl);
}

extern "C" int gpumhd_exchange(gpumhd_ctx* ctx, int with_bc) {
  if (!ctx) return GPUMHD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  const bool phys = with_bc && ctx->c.xbnd;
  if (phys) {
    int rc = ensure_bnd(ctx);
    if (rc) return rc;
  }
  // exchange (periodic images; the mirror rule too when it is the x boundary)
  const int mirror = (with_bc && ctx->c.g.xmirror) ? 1 : 0;
  if (ctx->f32) Launch<float>::fill_ghosts(ctx->c, (float*)ctx->S[ctx->iU], 8, mirror, ctx->stream);
  else Launch<double>::fill_ghosts(ctx->c, (double*)ctx->S[ctx->iU], 8, mirror, ctx->stream);
  int n = 1;
  if (ctx->c.has_spitzer) {  // the heat flux's periodic images (src/exchange.C:590-760)
    int rc = ensure_spitzer(ctx);
    if (rc) return rc;
    if (ctx->f32) Launch<float>::fill_ghosts(ctx->c, (float*)ctx->spt[0], 1, 0, ctx->stream);
    else Launch<double>::fill_ghosts(ctx->c, (double*)ctx->spt[0], 1, 0, ctx->stream);
    n += 1;
  }
  if (phys) n += enqueue_bc(ctx, ctx->S[ctx->iU], nullptr, 0);
  int rc = check_launch(ctx, n);
  if (rc || !phys || !ctx->hdyn.bnd_ini) return rc;
  // the first call sets p_bc and s_bc on the device: bring the host copy up to
  // date before a later push of the per-step scalars could overwrite them
  CK(cudaStreamSynchronize(ctx->stream));
  return pull_dyn(ctx);
}

extern "C" int gpumhd_boundary_info(gpumhd_ctx* ctx, double* p_bc, double* s_bc) {
  if (!ctx) return GPUMHD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  int rc = pull_dyn(ctx);
  if (rc) return rc;
  if (p_bc) *p_bc = ctx->hdyn.p_bc;
  if (s_bc) *s_bc = ctx->hdyn.s_bc;
  return GPUMHD_OK;
}

extern "C" int gpumhd_tcheck(gpumhd_ctx* ctx) {
  if (!ctx) return GPUMHD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  const double invdt = ctx->hdyn.dt > 0.0 ? 1.0 / ctx->hdyn.dt : 0.0;  // src/Add_Sources_Integrate_SR.C:560-564
  if (ctx->f32)
    Launch<float>::tcheck(ctx->c, (float*)ctx->S[ctx->iU], ctx->dyn, ctx->stream,
                          ctx->need_diag ? (float*)ctx->diag : nullptr, (float)invdt);
  else
    Launch<double>::tcheck(ctx->c, (double*)ctx->S[ctx->iU], ctx->dyn, ctx->stream,
                           ctx->need_diag ? (double*)ctx->diag : nullptr, invdt);
  return check_launch(ctx, 1);
}

// TVDlimit: three in-place sweeps; each sweep reads a copy of the state so that
// pencil chunks never see a neighbour's partial update.
// Clean_divB (src/clean_divB.C:35-369): the damped iterations on the
// context's state with its persistent phi; B's ghosts of the periodic
// dimensions are refreshed at the end as exchange_B_acc leaves them.
extern "C" int gpumhd_clean_divB(gpumhd_ctx* ctx) {
  if (!ctx) return GPUMHD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  int rc = ensure_divb(ctx);
  if (rc) return rc;
  Consts c = ctx->c;
  c.divb_on = 1;
  int n;
  if (ctx->f32) {
    float* U = (float*)ctx->S[ctx->iU];
    n = Launch<float>::divb_clean(c, U, (float*)ctx->phi, (float*)ctx->divb, ctx->dyn, ctx->stream);
    Launch<float>::fill_ghosts(c, U + 5 * c.g.N, 3, 0, ctx->stream);
  } else {
    double* U = (double*)ctx->S[ctx->iU];
    n = Launch<double>::divb_clean(c, U, (double*)ctx->phi, (double*)ctx->divb, ctx->dyn, ctx->stream);
    Launch<double>::fill_ghosts(c, U + 5 * c.g.N, 3, 0, ctx->stream);
  }
  rc = check_launch(ctx, n + 1);
  if (rc) return rc;
  // the adaptive count lives on the device: bring the host copy up to date
  CK(cudaStreamSynchronize(ctx->stream));
  return pull_dyn(ctx);
}

extern "C" int gpumhd_set_divb_iters(gpumhd_ctx* ctx, int next_iters) {
  if (!ctx) return GPUMHD_E_INVALID;
  const int cap = ctx->p.divB_itmax > 3 ? ctx->p.divB_itmax : 3;  // the count starts at 3 whatever itmax is
  if (next_iters < 1 || next_iters > cap)
    return fail(ctx, GPUMHD_E_INVALID, "divB iteration count %d outside [1, %d]", next_iters, cap);
  CK(cudaSetDevice(ctx->device));
  k_set_counter<<<1, 32, 0, ctx->stream>>>(&ctx->dyn->divb_next, next_iters);  // stream-ordered
  ctx->hdyn.divb_next = next_iters;
  return check_launch(ctx, 1);
}

extern "C" int gpumhd_divb_info(gpumhd_ctx* ctx, int* last_iters, int* next_iters, double* err_before,
                                double* err_after) {
  if (!ctx) return GPUMHD_E_INVALID;
  if (last_iters) *last_iters = ctx->hdyn.divb_last;
  if (next_iters) *next_iters = ctx->hdyn.divb_next;
  if (err_before) *err_before = ctx->hdyn.divb_err0;
  if (err_after) *err_after = ctx->hdyn.divb_err1;
  return GPUMHD_OK;
}

extern "C" int gpumhd_tvdlimit(gpumhd_ctx* ctx, double dt_tvd) {
  if (!ctx) return GPUMHD_E_INVALID;
  if (!ctx->have_pres) return fail(ctx, GPUMHD_E_ORDER, "TVDlimit needs the pressure of a ConsToPrim call");
  CK(cudaSetDevice(ctx->device));
  const long long N = ctx->c.g.N;
  if (!ctx->T) CK(cudaMalloc(&ctx->T, 8 * N * ctx->rsz));
  ctx->hdyn.dt_tvd = dt_tvd;
  ctx->hdyn.two_half = 0;
  int rc = push_dyn(ctx);
  if (rc) return rc;
  // The sweeps update U in place in the reference; here each reads one
  // buffer and writes another: x T -> U, y U -> T, z T -> U, from one copy of
  // U into T.  A sweep writes only the cells it updates (x: interior x, every
  // y and z row; y: interior x and y, every z row; z: the interior), so every
  // cell a sweep reads holds the previous sweep's value, and at the end U holds
  // the reference's values everywhere but in the z ghost planes at interior y,
  // which the y sweep updated in T: those rows are copied back.
  CK(cudaMemcpyAsync(ctx->T, ctx->S[ctx->iU], 8 * N * ctx->rsz, cudaMemcpyDeviceToDevice, ctx->stream));
  // an output step's diagnostics (src/tvdlimit_SR.C:115-116): per unit of the full step's time
  const double idt_full = 1.0 / ctx->hdyn.dt, dt_fac = dt_tvd / ctx->hdyn.dt;
  const TvdDiag<float> dgf{(float*)ctx->diag, (float)idt_full, (float)dt_fac};
  const TvdDiag<double> dgd{(double*)ctx->diag, idt_full, dt_fac};
  void* const bufs[2] = {ctx->T, ctx->S[ctx->iU]};  // [d & 1]: the input of sweep d
  for (int d = 0; d < 3; d++) {
    const void* in = bufs[d & 1];
    void* out = bufs[1 - (d & 1)];
    if (ctx->f32)
      Launch<float>::tvd(ctx->c, d, 0, 0, (const float*)in, (const float*)ctx->P[ctx->iP], (float*)out, ctx->dyn,
                         ctx->stream, 0, ctx->need_diag ? &dgf : nullptr);
    else
      Launch<double>::tvd(ctx->c, d, 0, 0, (const double*)in, (const double*)ctx->P[ctx->iP], (double*)out,
                          ctx->dyn, ctx->stream, 0, ctx->need_diag ? &dgd : nullptr);
    rc = check_launch(ctx, 1);
    if (rc) return rc;
  }
  {  // the z ghost planes' rows at interior y: the y sweep's values (in T)
    const Geom& g = ctx->c.g;
    const size_t plane = (size_t)g.sx * g.sy * ctx->rsz, row = (size_t)g.sx * ctx->rsz;
    for (int f = 0; f < 8; f++)
      for (int side = 0; side < 2; side++) {
        const size_t k0 = side == 0 ? 0 : (size_t)(GH + g.nz);
        const size_t off = (size_t)f * N * ctx->rsz + k0 * plane + GH * row;
        CK(cudaMemcpy2DAsync((char*)ctx->S[ctx->iU] + off, plane, (const char*)ctx->T + off, plane,
                             (size_t)g.ny * row, GH, cudaMemcpyDeviceToDevice, ctx->stream));
      }
  }
  return GPUMHD_OK;
}

// ------------------------------------------------------------- fused path
// Launches of one fused step: step control, four RK stages, six TVD sweeps,
// the end-of-step pass; with divB cleaning also the cleaning passes, with the
// physical x boundaries their three launches after each stage and the step.
static int step_launches(const gpumhd_ctx* ctx) {
  int n = 12;
  if (ctx->c.divb_on) n += 3 + 2 * (ctx->c.divb_itmax > 3 ? ctx->c.divb_itmax : 3);
  if (ctx->c.xbnd) n += 5 * 3;  // the boundaries after each stage and at the end of the step
  if (ctx->c.has_spitzer) n += 4 * 2;  // temperature and heat flux before each stage
  if (ctx->c.va_adjust > 0.0) n += ctx->c.xbnd ? 3 : 2;  // adaptive limits, then the CFL speed with them
  return n;
}
// Kernels one replay of the captured step always launches: the second TVD
// half pass sits in a conditional node (k_step_begin counts it when taken).
static int graph_step_launches(const gpumhd_ctx* ctx) { return step_launches(ctx) - (ctx->cond_tvd2 ? 3 : 0); }

// During a capture on the context's stream: an IF node, controlled by handle
// h, after the work captured so far; body(q) enqueues its contents on stream q.
template <class F>
static int capture_if(gpumhd_ctx* ctx, cudaGraphConditionalHandle h, F body) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  cudaGraph_t cg = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  const cudaGraphEdgeData* ed = nullptr;
  size_t nd = 0;
  CK(cudaStreamGetCaptureInfo(ctx->stream, &st, nullptr, &cg, &deps, &ed, &nd));
  if (st != cudaStreamCaptureStatusActive || !cg) return fail(ctx, GPUMHD_E_CUDA, "conditional node outside a capture");
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeIf;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, cg, deps, ed, nd, &np));
  CK(cudaStreamBeginCaptureToGraph(ctx->s_cond, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                   cudaStreamCaptureModeThreadLocal));
  body(ctx->s_cond);
  cudaGraph_t bg = nullptr;
  CK(cudaStreamEndCapture(ctx->s_cond, &bg));
  CK(cudaStreamUpdateCaptureDependencies(ctx->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  return GPUMHD_OK;
}

// One fused step: step control, four RK stages, two TVD passes (the second
// returns at once unless the step takes two half passes), Clean_divB when it
// is on, and the end-of-step pass (TCheck, ghost images, the next step's
// pressure, CFL speed and statistics; src/solver.C:324-365).  With ev != NULL
// an event is recorded before each of the 11 launches up to the TVD passes,
// before the cleaning, before the end-of-step pass and after it (14 events).
static int enqueue_one_step(gpumhd_ctx* ctx, cudaEvent_t* ev = nullptr) {
  const Consts& c = ctx->c;
  cudaStream_t s = ctx->stream;
  int k = 0;
  auto mark = [&]() { if (ev) cudaEventRecord(ev[k++], s); };
  const int a = ctx->iU, b = ctx->iU0, d = ctx->iRes;  // a: state, b and d: work buffers
  const int pa = ctx->iP, pb = 1 - ctx->iP;
  const bool xb = c.xbnd != 0;
  const bool sp = c.has_spitzer != 0;
  // Under stream capture the second TVD half pass (which most steps skip)
  // becomes an IF node that k_step_begin switches on only for steps that take
  // it; launched directly, its kernels return at once when not taken.
  cudaGraphConditionalHandle tvd2 = 0;
  bool cond = false;
  {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    cudaGraph_t cg = nullptr;
    if (cudaStreamGetCaptureInfo(s, &st, nullptr, &cg, nullptr, nullptr, nullptr) == cudaSuccess &&
        st == cudaStreamCaptureStatusActive && cg) {
      if (cudaGraphConditionalHandleCreate(&tvd2, cg, 0, cudaGraphCondAssignDefault) == cudaSuccess) cond = true;
      else cudaGetLastError();
    }
  }
  ctx->cond_tvd2 = cond;
  mark();
  if (c.va_adjust > 0.0) {
    // Adjust_Valf_Max with adaptive limits, then the stage-1 CFL speed under
    // the new inv_va2max (interior, and the physical boundaries' face ghosts)
    k_step_limits<<<1, 32, 0, s>>>(c, ctx->dyn);
    if (ctx->f32) {
      Launch<float>::cfl_cons(c, (const float*)ctx->S[ctx->iU], (const float*)ctx->P[ctx->iP], ctx->dyn, s);
      if (c.xbnd) Launch<float>::cmax_faces(c, (const float*)ctx->S[ctx->iU], (const float*)ctx->P[ctx->iP], ctx->dyn, s);
    } else {
      Launch<double>::cfl_cons(c, (const double*)ctx->S[ctx->iU], (const double*)ctx->P[ctx->iP], ctx->dyn, s);
      if (c.xbnd) Launch<double>::cmax_faces(c, (const double*)ctx->S[ctx->iU], (const double*)ctx->P[ctx->iP], ctx->dyn, s);
    }
  }
  k_step_begin<<<1, 32, 0, s>>>(c, ctx->dyn, ctx->dt_hist, ctx->dt_hist_cap, tvd2, cond ? 1 : 0);
  if (ctx->f32) {
    using L = Launch<float>;
    // Spitzer conduction before each stage: temperature, then the heat flux's
    // residual (the energy share for the stage kernel) and its update
    float* const* SF = (float* const*)ctx->spt;
    static const int sf_in[5] = {0, 0, 1, 2, 1}, sf_out[5] = {0, 1, 2, 1, 0};
    auto spz = [&](const float* Uin, int st) {
      if (!sp) return;
      L::temp(c, Uin, SF[3], s);
      L::spitzer(c, Uin, false, SF[3], SF[sf_in[st]], SF[0], SF[sf_out[st]], nullptr, SF[4], ctx->dyn, st, s);
    };
    float* const sf1 = sp ? SF[1] : nullptr;
    float* const sf2 = sp ? SF[2] : nullptr;
    float* const sf0 = sp ? SF[0] : nullptr;
    Rem<float>* const comp = (ctx->p.compensated && ctx->comp) ? (Rem<float>*)ctx->comp : nullptr;
    float* const* S = (float* const*)ctx->S;
    float* const* P = (float* const*)ctx->P;
    mark();
    spz(S[a], 1);
    L::stage(c, S[a], P[pa], S[a], S[b], P[pb], nullptr, ctx->dyn, 1, false, 1, s,
              map_u(ctx, a), map_p(ctx, pa), ctx->tune_zc, comp);
    if (xb) L::bc(c, S[b], P[pb], ctx->dyn, ctx->bnd_part, 0, s, sf1);
    mark();
    spz(S[b], 2);
    L::stage(c, S[b], P[pb], S[a], S[d], P[pa], nullptr, ctx->dyn, 2, false, 1, s,
              map_u(ctx, b), map_p(ctx, pb), ctx->tune_zc, comp);
    if (xb) L::bc(c, S[d], P[pa], ctx->dyn, ctx->bnd_part, 0, s, sf2);
    mark();
    spz(S[d], 3);
    L::stage(c, S[d], P[pa], S[a], S[b], P[pb], nullptr, ctx->dyn, 3, false, 1, s,
              map_u(ctx, d), map_p(ctx, pa), ctx->tune_zc, comp);
    if (xb) L::bc(c, S[b], P[pb], ctx->dyn, ctx->bnd_part, 0, s, sf1);
    mark();
    spz(S[b], 4);
    L::stage(c, S[b], P[pb], S[a], S[a], nullptr, nullptr, ctx->dyn, 4, false, 0, s,
              map_u(ctx, b), map_p(ctx, pb), ctx->tune_zc, comp);
    if (xb) L::bc(c, S[a], (float*)nullptr, ctx->dyn, ctx->bnd_part, 0, s, sf0);  // TVD keeps the stale pressure
    mark();
    L::tvd(c, 0, 0, 0, S[a], P[pb], S[d], ctx->dyn, s, ctx->tune_td, nullptr, comp);
    mark();
    L::tvd(c, 1, 0, 0, S[d], P[pb], S[b], ctx->dyn, s, ctx->tune_td, nullptr, comp);
    mark();
    L::tvd(c, 2, 1, 0, S[b], P[pb], S[a], ctx->dyn, s, ctx->tune_td, nullptr, comp);
    if (cond) {
      const int rc2 = capture_if(ctx, tvd2, [&](cudaStream_t q) {
        L::tvd(c, 0, 0, 1, S[a], P[pb], S[d], ctx->dyn, q, ctx->tune_td, nullptr, comp);
        L::tvd(c, 1, 0, 1, S[d], P[pb], S[b], ctx->dyn, q, ctx->tune_td, nullptr, comp);
        L::tvd(c, 2, 2, 1, S[b], P[pb], S[a], ctx->dyn, q, ctx->tune_td, nullptr, comp);
      });
      if (rc2) return rc2;
    } else {
      mark();
      L::tvd(c, 0, 0, 1, S[a], P[pb], S[d], ctx->dyn, s, ctx->tune_td, nullptr, comp);
      mark();
      L::tvd(c, 1, 0, 1, S[d], P[pb], S[b], ctx->dyn, s, ctx->tune_td, nullptr, comp);
      mark();
      L::tvd(c, 2, 2, 1, S[b], P[pb], S[a], ctx->dyn, s, ctx->tune_td, nullptr, comp);
    }
    mark();
    if (c.divb_on) L::divb_clean(c, S[a], (float*)ctx->phi, (float*)ctx->divb, ctx->dyn, s);
    mark();
    {
      L::step_finish(c, S[a], P[pa], ctx->dyn, s, comp);
    }
    if (xb) {
      L::bc(c, S[a], P[pa], ctx->dyn, ctx->bnd_part, 1, s, sf0);  // the next step's ghosts, pressure and CFL speed
    }
  } else {
    using L = Launch<double>;
    // Spitzer conduction before each stage: temperature, then the heat flux's
    // residual (the energy share for the stage kernel) and its update
    double* const* SF = (double* const*)ctx->spt;
    static const int sf_in[5] = {0, 0, 1, 2, 1}, sf_out[5] = {0, 1, 2, 1, 0};
    auto spz = [&](const double* Uin, int st) {
      if (!sp) return;
      L::temp(c, Uin, SF[3], s);
      L::spitzer(c, Uin, false, SF[3], SF[sf_in[st]], SF[0], SF[sf_out[st]], nullptr, SF[4], ctx->dyn, st, s);
    };
    double* const sf1 = sp ? SF[1] : nullptr;
    double* const sf2 = sp ? SF[2] : nullptr;
    double* const sf0 = sp ? SF[0] : nullptr;
    double* const* S = (double* const*)ctx->S;
    double* const* P = (double* const*)ctx->P;
    mark();
    spz(S[a], 1);
    L::stage(c, S[a], P[pa], S[a], S[b], P[pb], nullptr, ctx->dyn, 1, false, 1, s,
              map_u(ctx, a), map_p(ctx, pa), ctx->tune_zc);
    if (xb) L::bc(c, S[b], P[pb], ctx->dyn, ctx->bnd_part, 0, s, sf1);
    mark();
    spz(S[b], 2);
    L::stage(c, S[b], P[pb], S[a], S[d], P[pa], nullptr, ctx->dyn, 2, false, 1, s,
              map_u(ctx, b), map_p(ctx, pb), ctx->tune_zc);
    if (xb) L::bc(c, S[d], P[pa], ctx->dyn, ctx->bnd_part, 0, s, sf2);
    mark();
    spz(S[d], 3);
    L::stage(c, S[d], P[pa], S[a], S[b], P[pb], nullptr, ctx->dyn, 3, false, 1, s,
              map_u(ctx, d), map_p(ctx, pa), ctx->tune_zc);
    if (xb) L::bc(c, S[b], P[pb], ctx->dyn, ctx->bnd_part, 0, s, sf1);
    mark();
    spz(S[b], 4);
    L::stage(c, S[b], P[pb], S[a], S[a], nullptr, nullptr, ctx->dyn, 4, false, 0, s,
              map_u(ctx, b), map_p(ctx, pb), ctx->tune_zc);
    if (xb) L::bc(c, S[a], (double*)nullptr, ctx->dyn, ctx->bnd_part, 0, s, sf0);  // TVD keeps the stale pressure
    mark();
    L::tvd(c, 0, 0, 0, S[a], P[pb], S[d], ctx->dyn, s, ctx->tune_td);
    mark();
    L::tvd(c, 1, 0, 0, S[d], P[pb], S[b], ctx->dyn, s, ctx->tune_td);
    mark();
    L::tvd(c, 2, 1, 0, S[b], P[pb], S[a], ctx->dyn, s, ctx->tune_td);
    if (cond) {
      const int rc2 = capture_if(ctx, tvd2, [&](cudaStream_t q) {
        L::tvd(c, 0, 0, 1, S[a], P[pb], S[d], ctx->dyn, q, ctx->tune_td);
        L::tvd(c, 1, 0, 1, S[d], P[pb], S[b], ctx->dyn, q, ctx->tune_td);
        L::tvd(c, 2, 2, 1, S[b], P[pb], S[a], ctx->dyn, q, ctx->tune_td);
      });
      if (rc2) return rc2;
    } else {
      mark();
      L::tvd(c, 0, 0, 1, S[a], P[pb], S[d], ctx->dyn, s, ctx->tune_td);
      mark();
      L::tvd(c, 1, 0, 1, S[d], P[pb], S[b], ctx->dyn, s, ctx->tune_td);
      mark();
      L::tvd(c, 2, 2, 1, S[b], P[pb], S[a], ctx->dyn, s, ctx->tune_td);
    }
    mark();
    if (c.divb_on) L::divb_clean(c, S[a], (double*)ctx->phi, (double*)ctx->divb, ctx->dyn, s);
    mark();
    {
      L::step_finish(c, S[a], P[pa], ctx->dyn, s);
    }
    if (xb) {
      L::bc(c, S[a], P[pa], ctx->dyn, ctx->bnd_part, 1, s, sf0);  // the next step's ghosts, pressure and CFL speed
    }
  }
  mark();
  return check_launch(ctx, step_launches(ctx));
}

static int fused_prepare(gpumhd_ctx* ctx, int nsteps) {
  if (!ctx->eos_loaded) return fail(ctx, GPUMHD_E_ORDER, "time steps before eos_init");
  if (ctx->need_diag)
    return fail(ctx, GPUMHD_E_INVALID, "an output step's diagnostics come from the per-routine calls; "
                "switch them off (gpumhd_set_need_diagnostics) before fused steps");
  if (nsteps > ctx->dt_hist_cap) {
    if (ctx->graph) { cudaGraphExecDestroy(ctx->graph); ctx->graph = nullptr; }
    cudaFree(ctx->dt_hist);
    ctx->dt_hist = nullptr;
    int cap = nsteps < 1024 ? 1024 : nsteps;
    CK(cudaMalloc(&ctx->dt_hist, sizeof(double) * cap));
    ctx->dt_hist_cap = cap;
  }
  if (ctx->c.divb_on) {
    int rc1 = ensure_divb(ctx);
    if (rc1) return rc1;
  }
  {
    int rc1 = ensure_bnd(ctx);
    if (rc1) return rc1;
    rc1 = ensure_spitzer(ctx);
    if (rc1) return rc1;
  }
  if (ctx->f32 && ctx->p.compensated && !ctx->comp) {
    CK(cudaMalloc(&ctx->comp, sizeof(Rem<float>) * 8 * ctx->c.g.N));
    CK(cudaMemsetAsync(ctx->comp, 0, sizeof(Rem<float>) * 8 * ctx->c.g.N, ctx->stream));
  }
  if (!ctx->fused_ready) {
    // exchange + boundaries before the loop (src/solver.C:80-81), then the
    // pressure, CFL speed and statistics of the initial state
    // The limits, error flag and accumulators are reset by a kernel rather
    // than a host round trip of Dyn: no host synchronisation and no small
    // copy queued behind large asynchronous transfers.  The host mirror gets
    // the same values (its other fields are refreshed by the next pull).
    // With adaptive limits (va_adjust > 0) the limits and their history stay
    // as the device holds them: k_step_limits updates them at every step.
    Dyn& d = ctx->hdyn;
    if (!(ctx->p.va_adjust > 0.0)) {
      d.va_ini_flag = 0;
      d.inv_va2max = 1.0 / pow(ctx->p.va_max, 2);
      d.v_lim = ctx->p.tchk[3];
      d.e_lim = ctx->p.tchk[2];
      const double vml = ctx->p.tvd[8];
      d.vsqr_diff = vml < 1.0 ? pow(vml * d.v_lim, 2.0) : pow(vml, 2.0);
    }
    d.err = 0;
    d.cmax_bits = 0;
    d.stat_max_bits[0] = d.stat_max_bits[1] = d.stat_max_bits[2] = 0;
    d.stat_cnt[0] = d.stat_cnt[1] = 0;
    k_fused_reinit<<<1, 32, 0, ctx->stream>>>(ctx->c, ctx->dyn, d.inv_va2max, d.v_lim, d.e_lim, d.vsqr_diff);
    int rc = GPUMHD_OK;
    // physical x boundaries: their ghosts, with the CFL speed of the x ghosts
    // (no longer images of interior cells), before the pressures and statistics
    int n = 3;
    if (ctx->c.has_spitzer) {  // the heat flux's periodic images
      if (ctx->f32) Launch<float>::fill_ghosts(ctx->c, (float*)ctx->spt[0], 1, 0, ctx->stream);
      else Launch<double>::fill_ghosts(ctx->c, (double*)ctx->spt[0], 1, 0, ctx->stream);
      n += 1;
    }
    if (ctx->f32) {
      Launch<float>::fill_ghosts(ctx->c, (float*)ctx->S[ctx->iU], 8, 1, ctx->stream);
      if (ctx->c.xbnd) n += enqueue_bc(ctx, ctx->S[ctx->iU], ctx->P[ctx->iP], 1);
      Launch<float>::init_pass(ctx->c, (const float*)ctx->S[ctx->iU], (float*)ctx->P[ctx->iP], ctx->dyn, ctx->stream);
    } else {
      Launch<double>::fill_ghosts(ctx->c, (double*)ctx->S[ctx->iU], 8, 1, ctx->stream);
      if (ctx->c.xbnd) n += enqueue_bc(ctx, ctx->S[ctx->iU], ctx->P[ctx->iP], 1);
      Launch<double>::init_pass(ctx->c, (const double*)ctx->S[ctx->iU], (double*)ctx->P[ctx->iP], ctx->dyn, ctx->stream);
    }
    rc = check_launch(ctx, n);
    if (rc) return rc;
    ctx->fused_ready = true;
  }
  return GPUMHD_OK;
}

extern "C" int gpumhd_enqueue_steps(gpumhd_ctx* ctx, int nsteps) {
  if (!ctx || nsteps < 0) return GPUMHD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  int rc = fused_prepare(ctx, nsteps);
  if (rc) return rc;
  for (int s = 0; s < nsteps; s++) {
    if (ctx->graph) {
      CK(cudaGraphLaunch(ctx->graph, ctx->stream));
      ctx->launches += graph_step_launches(ctx);
    } else {
      rc = enqueue_one_step(ctx);
      if (rc) return rc;
    }
  }
  // the fused step uses U0 and Res as work space; Res counts as zero again, as
  // after Source_Integrate_Tcheck, so per-routine calls can follow
  if (nsteps > 0) ctx->res_zero_pending = true;
  ctx->have_pres = true;
  return GPUMHD_OK;
}

static int capture_graph(gpumhd_ctx* ctx) {
  if (ctx->graph) return GPUMHD_OK;
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_one_step(ctx);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (rc) { if (g) cudaGraphDestroy(g); return rc; }
  if (e != cudaSuccess) return fail(ctx, GPUMHD_E_CUDA, "graph capture: %s", cudaGetErrorString(e));
  ctx->launches -= step_launches(ctx);  // capture records, it does not launch
  e = cudaGraphInstantiate(&ctx->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) { ctx->graph = nullptr; return fail(ctx, GPUMHD_E_CUDA, "graph instantiate: %s", cudaGetErrorString(e)); }
  return GPUMHD_OK;
}

extern "C" int gpumhd_synchronize(gpumhd_ctx* ctx) {
  if (!ctx) return GPUMHD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->s_out) CK(cudaStreamSynchronize(ctx->s_out));
  if (ctx->s_in) CK(cudaStreamSynchronize(ctx->s_in));
  int rc = pull_dyn(ctx);
  if (rc) return rc;
  switch (ctx->hdyn.err) {
    case 0: return GPUMHD_OK;
    case ERR_BAD_DT_RAD: return fail(ctx, GPUMHD_E_BAD_DT, "Invalid time step: dt_rad");
    case ERR_BAD_DT_MHD: return fail(ctx, GPUMHD_E_BAD_DT, "Invalid time step: dt_mhd = %g", ctx->hdyn.dt_mhd);
    case ERR_CFL: return fail(ctx, GPUMHD_E_CFL, "Invalid time step: CFL = %g", ctx->hdyn.cfl);
    case ERR_WAIT_TIMEOUT: return fail(ctx, GPUMHD_E_CUDA, "a device-side wait for a TMA copy timed out");
    default: return fail(ctx, GPUMHD_E_CUDA, "device error flag %d", ctx->hdyn.err);
  }
}

extern "C" int gpumhd_run_steps(gpumhd_ctx* ctx, int nsteps, double* dt_out, int capture) {
  if (!ctx || nsteps < 0) return GPUMHD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  int rc = fused_prepare(ctx, nsteps);
  if (rc) return rc;
  // dt history restarts at this call
  ctx->hdyn.steps_done = 0;
  CK(cudaMemcpyAsync(&ctx->dyn->steps_done, &ctx->hdyn.steps_done, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  if (capture) {
    rc = capture_graph(ctx);
    if (rc) return rc;
  }
  rc = gpumhd_enqueue_steps(ctx, nsteps);
  if (rc) return rc;
  rc = gpumhd_synchronize(ctx);
  if (rc) return rc;
  if (dt_out && nsteps > 0)
    CK(cudaMemcpy(dt_out, ctx->dt_hist, sizeof(double) * nsteps, cudaMemcpyDeviceToHost));
  return GPUMHD_OK;
}

extern "C" int gpumhd_profile_steps(gpumhd_ctx* ctx, int nsteps, double* ms_phase) {
  if (!ctx || nsteps < 1 || !ms_phase) return GPUMHD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  int rc = fused_prepare(ctx, nsteps);
  if (rc) return rc;
  cudaEvent_t ev[14];
  for (int q = 0; q < 14; q++) CK(cudaEventCreate(&ev[q]));
  for (int q = 0; q < 13; q++) ms_phase[q] = 0.0;
  for (int st = 0; st < nsteps && rc == 0; st++) {
    rc = enqueue_one_step(ctx, ev);
    if (rc) break;
    if (cudaEventSynchronize(ev[13]) != cudaSuccess) { rc = fail(ctx, GPUMHD_E_CUDA, "event sync failed"); break; }
    for (int q = 0; q < 13; q++) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[q], ev[q + 1]);
      ms_phase[q] += ms / nsteps;
    }
  }
  for (int q = 0; q < 14; q++) cudaEventDestroy(ev[q]);
  if (rc) return rc;
  ctx->res_zero_pending = true;
  return gpumhd_synchronize(ctx);
}

extern "C" int gpumhd_step_info(gpumhd_ctx* ctx, double* dt, double* cfl, double* time, int* tvd_two_half) {
  if (!ctx) return GPUMHD_E_INVALID;
  if (dt) *dt = ctx->hdyn.dt;
  if (cfl) *cfl = ctx->hdyn.cfl;
  if (time) *time = ctx->hdyn.time;
  if (tvd_two_half) *tvd_two_half = ctx->hdyn.two_half;
  return GPUMHD_OK;
}

extern "C" void* gpumhd_stream(gpumhd_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }
// After gpumhd_synchronize: the host-counted launches plus those the device
// enabled in captured steps' conditional nodes.
extern "C" long long gpumhd_launch_count(gpumhd_ctx* ctx) {
  if (!ctx) return 0;
  unsigned long long cl = 0;
  if (cudaSetDevice(ctx->device) != cudaSuccess ||
      cudaMemcpy(&cl, &ctx->dyn->cond_launches, sizeof cl, cudaMemcpyDeviceToHost) != cudaSuccess)
    cl = 0;
  return ctx->launches + (long long)cl;
}

// ------------------------------------------------------------- launch shapes
extern "C" int gpumhd_test_tma_wait(gpumhd_ctx* ctx, long long wait_cycles, int withhold_last) {
  if (!ctx || wait_cycles < 0) return GPUMHD_E_INVALID;
  ctx->tm_wait_cycles = wait_cycles;
  ctx->tm_withhold_last = withhold_last ? 1 : 0;
  ctx->c.tm_wait_cycles = ctx->tm_wait_cycles;
  ctx->c.tm_withhold_last = ctx->tm_withhold_last;
  if (ctx->graph) {  // the captured step holds the old launch parameters
    cudaGraphExecDestroy(ctx->graph);
    ctx->graph = nullptr;
  }
  return GPUMHD_OK;
}

extern "C" int gpumhd_set_tuning(gpumhd_ctx* ctx, int stage_zchunk, int tvd_chunk) {
  if (!ctx || stage_zchunk < 0 || tvd_chunk < 0 || tvd_chunk > 1024) return GPUMHD_E_INVALID;
  ctx->tune_zc = stage_zchunk;
  ctx->tune_td = tvd_chunk;
  if (ctx->graph) { cudaGraphExecDestroy(ctx->graph); ctx->graph = nullptr; }
  return GPUMHD_OK;
}

extern "C" int gpumhd_get_tuning(gpumhd_ctx* ctx, int* stage_kernel, int* stage_zchunk, int* tvd_chunk) {
  if (!ctx) return GPUMHD_E_INVALID;
  if (stage_kernel) *stage_kernel = (ctx->tma && ctx->p.stage_kernel == 0) ? 0 : 1;
  if (stage_zchunk) *stage_zchunk = ctx->tune_zc;
  if (tvd_chunk) *tvd_chunk = ctx->tune_td;
  return GPUMHD_OK;
}

// Mean time of `steps` fused steps (after one untimed step), CUDA events on the
// context's stream.
// What trial steps change and must give back: the state, its pressure, the
// divB cleaning potential, the Spitzer heat flux and the step-control block.
// Compensated remainders are left alone by running the trials uncompensated.
struct TrialSave {
  void* U = nullptr;
  void* P = nullptr;
  void* phi = nullptr;
  void* sflx = nullptr;
  Dyn dyn{};
  int comp = 0;
};

static void trial_free(TrialSave& t) {
  for (void* q : {t.U, t.P, t.phi, t.sflx})
    if (q) cudaFree(q);
  t.U = t.P = t.phi = t.sflx = nullptr;
}

static int trial_save(gpumhd_ctx* ctx, TrialSave& t) {
  gpumhd_ctx* const x = ctx;
  const size_t n = (size_t)x->c.g.N * x->rsz;
  t.comp = x->p.compensated;
  CK(cudaMalloc(&t.U, 8 * n));
  CK(cudaMalloc(&t.P, n));
  CK(cudaMemcpyAsync(t.U, x->S[x->iU], 8 * n, cudaMemcpyDeviceToDevice, x->stream));
  CK(cudaMemcpyAsync(t.P, x->P[x->iP], n, cudaMemcpyDeviceToDevice, x->stream));
  if (x->phi) {
    CK(cudaMalloc(&t.phi, n));
    CK(cudaMemcpyAsync(t.phi, x->phi, n, cudaMemcpyDeviceToDevice, x->stream));
  }
  if (x->spt[0]) {
    CK(cudaMalloc(&t.sflx, n));
    CK(cudaMemcpyAsync(t.sflx, x->spt[0], n, cudaMemcpyDeviceToDevice, x->stream));
  }
  const int rc = pull_dyn(x);
  if (rc) return rc;
  t.dyn = x->hdyn;
  x->p.compensated = 0;
  return GPUMHD_OK;
}

static int trial_restore(gpumhd_ctx* ctx, const TrialSave& t) {
  gpumhd_ctx* const x = ctx;
  const size_t n = (size_t)x->c.g.N * x->rsz;
  CK(cudaMemcpyAsync(x->S[x->iU], t.U, 8 * n, cudaMemcpyDeviceToDevice, x->stream));
  CK(cudaMemcpyAsync(x->P[x->iP], t.P, n, cudaMemcpyDeviceToDevice, x->stream));
  if (t.phi) CK(cudaMemcpyAsync(x->phi, t.phi, n, cudaMemcpyDeviceToDevice, x->stream));
  if (t.sflx) CK(cudaMemcpyAsync(x->spt[0], t.sflx, n, cudaMemcpyDeviceToDevice, x->stream));
  x->hdyn = t.dyn;
  return push_dyn(x);
}

static int time_steps(gpumhd_ctx* ctx, int steps, double* ms) {
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  int rc = enqueue_one_step(ctx);
  cudaEventRecord(e0, ctx->stream);
  for (int s = 0; s < steps && rc == 0; s++) rc = enqueue_one_step(ctx);
  cudaEventRecord(e1, ctx->stream);
  float t = 0.f;
  if (rc == 0) {
    if (cudaEventSynchronize(e1) != cudaSuccess) rc = fail(ctx, GPUMHD_E_CUDA, "autotune: event sync failed");
    else cudaEventElapsedTime(&t, e0, e1);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = (double)t / (steps > 0 ? steps : 1);
  return rc;
}

// Times candidate launch shapes -- stage kernel (TMA / plain loads), z planes
// per stage block, cells per thread of the y / z TVD sweeps -- on the
// context's own state, and keeps the fastest.  The state, its pressure and the
// step-control block are restored afterwards, so the run is unchanged.
extern "C" int gpumhd_autotune(gpumhd_ctx* ctx, int trial_steps, double* best_ms) {
  if (!ctx || trial_steps < 1) return GPUMHD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  int rc = fused_prepare(ctx, trial_steps + 1);
  if (rc) return rc;
  TrialSave sv;
  rc = trial_save(ctx, sv);
  if (rc) { ctx->p.compensated = sv.comp; trial_free(sv); return rc; }
  auto restore = [&]() { return trial_restore(ctx, sv); };
  const int nz = ctx->c.g.nz;
  std::vector<int> zcs = {0, nz};
  for (int f = 2; f <= 16; f *= 2)
    if ((nz + f - 1) / f >= 4) zcs.push_back((nz + f - 1) / f);
  std::vector<int> kernels = {1};
  if (ctx->tma) kernels.insert(kernels.begin(), 0);
  const int keep_kernel = ctx->p.stage_kernel, keep_td = ctx->tune_td;
  double best = 1e300;
  int bk = keep_kernel, bz = 0, btd = keep_td;
  for (int kern : kernels) {
    for (int zc : zcs) {
      if (rc) break;
      ctx->p.stage_kernel = kern;
      ctx->tune_zc = zc;
      double ms = 0.0;
      rc = restore();
      if (!rc) rc = time_steps(ctx, trial_steps, &ms);
      if (!rc && ms < best) { best = ms; bk = kern; bz = zc; }
    }
  }
  ctx->p.stage_kernel = bk;
  ctx->tune_zc = bz;
  const int tds[] = {32, 16, 64};
  for (int td : tds) {
    if (rc) break;
    ctx->tune_td = td;
    double ms = 0.0;
    rc = restore();
    if (!rc) rc = time_steps(ctx, trial_steps, &ms);
    if (!rc && ms < best) { best = ms; btd = td; }
  }
  ctx->tune_td = btd;
  ctx->p.compensated = sv.comp;
  if (!rc) rc = restore();
  cudaStreamSynchronize(ctx->stream);
  trial_free(sv);
  if (ctx->graph) { cudaGraphExecDestroy(ctx->graph); ctx->graph = nullptr; }
  if (rc) return rc;
  if (best_ms) *best_ms = best;
  return gpumhd_synchronize(ctx);
}

// ------------------------------------------------------------------ ensemble
// Independent boxes (contexts of any sizes on one device) advanced together:
// one CUDA graph whose while-node body is one step of every box, the boxes as
// parallel branches, so that a single graph launch runs all requested steps.
struct gpumhd_ensemble {
  std::vector<gpumhd_ctx*> box;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr;
  std::vector<cudaEvent_t> join;
  int* d_counter = nullptr;
  cudaGraphExec_t exec = nullptr;    // body: one step of every box
  cudaGraphExec_t exec_k = nullptr;  // body: unroll steps of every box (unroll > 1)
  int unroll = 1;                    // steps of each box per loop iteration
  bool largest_first = false;        // branches captured in order of decreasing cell count
  long long launches = 0;
  char err[1024] = {0};
};

static int efail(gpumhd_ensemble* e, int code, const char* msg) {
  if (e) snprintf(e->err, sizeof e->err, "%s", msg);
  snprintf(g_create_err, sizeof g_create_err, "%s", msg);
  return code;
}

#define ECK(call)                                                  \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) return efail(e, GPUMHD_E_CUDA, cudaGetErrorString(e_)); \
  } while (0)

static void ensemble_free(gpumhd_ensemble* e) {
  if (!e) return;
  if (e->exec) cudaGraphExecDestroy(e->exec);
  if (e->exec_k) cudaGraphExecDestroy(e->exec_k);
  for (cudaEvent_t ev : e->join) cudaEventDestroy(ev);
  if (e->fork) cudaEventDestroy(e->fork);
  if (e->done) cudaEventDestroy(e->done);
  if (e->d_counter) cudaFree(e->d_counter);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
}

// The loop graph whose body advances every box by nstep steps (a chain of
// nstep fused steps per box, the boxes as parallel branches between a fork
// and a join), into *exec.
static int ensemble_build(gpumhd_ensemble* e, int nstep, cudaGraphExec_t* exec) {
  cudaGraph_t g = nullptr;
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return efail(e, GPUMHD_E_CUDA, "cudaGraphCreate failed");
  cudaGraphConditionalHandle h;
  if (cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) {
    cudaGraphDestroy(g);
    return efail(e, GPUMHD_E_CUDA, "cudaGraphConditionalHandleCreate failed");
  }
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  if (cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np) != cudaSuccess) {
    cudaGraphDestroy(g);
    return efail(e, GPUMHD_E_CUDA, "adding the while node failed");
  }
  cudaGraph_t body = np.conditional.phGraph_out[0];
  int rc = GPUMHD_OK;
  if (cudaStreamBeginCaptureToGraph(e->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) !=
      cudaSuccess) {
    cudaGraphDestroy(g);
    return efail(e, GPUMHD_E_CUDA, "capture into the loop body failed");
  }
  cudaEventRecord(e->fork, e->stream);
  std::vector<size_t> order(e->box.size());
  for (size_t b = 0; b < order.size(); b++) order[b] = b;
  if (e->largest_first)
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t u, size_t v) { return e->box[u]->c.g.N > e->box[v]->c.g.N; });
  for (size_t o = 0; o < order.size() && rc == 0; o++) {
    const size_t b = order[o];
    gpumhd_ctx* x = e->box[b];
    cudaStreamWaitEvent(x->stream, e->fork, 0);
    for (int t = 0; t < nstep && rc == 0; t++) {
      rc = enqueue_one_step(x);
      x->launches -= step_launches(x);  // recorded into the graph, not launched
    }
    cudaEventRecord(e->join[b], x->stream);
    cudaStreamWaitEvent(e->stream, e->join[b], 0);
  }
  k_loop_tick<<<1, 32, 0, e->stream>>>(e->d_counter, h);
  cudaGraph_t out = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(e->stream, &out);
  if (rc == 0 && ce != cudaSuccess) rc = efail(e, GPUMHD_E_CUDA, cudaGetErrorString(ce));
  if (rc == 0 && cudaGraphInstantiate(exec, g, 0) != cudaSuccess) {
    *exec = nullptr;
    rc = efail(e, GPUMHD_E_CUDA, "instantiating the ensemble graph failed");
  }
  cudaGraphDestroy(g);
  return rc;
}

extern "C" int gpumhd_ensemble_create(gpumhd_ctx* const* boxes, int n, gpumhd_ensemble** out) {
  if (!boxes || n < 1 || !out) return efail(nullptr, GPUMHD_E_INVALID, "ensemble: no boxes");
  *out = nullptr;
  gpumhd_ensemble* e = new gpumhd_ensemble();
  e->device = boxes[0] ? boxes[0]->device : 0;
  for (int b = 0; b < n; b++) {
    gpumhd_ctx* x = boxes[b];
    if (!x || x->device != e->device) { ensemble_free(e); return efail(nullptr, GPUMHD_E_INVALID, "ensemble: null box or boxes on different devices"); }
    for (int a = 0; a < b; a++)
      if (boxes[a] == x) { ensemble_free(e); return efail(nullptr, GPUMHD_E_INVALID, "ensemble: a box appears twice"); }
    e->box.push_back(x);
  }
  int rc = GPUMHD_OK;
  if (cudaSetDevice(e->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->done, cudaEventDisableTiming) != cudaSuccess ||
      cudaMalloc(&e->d_counter, sizeof(int)) != cudaSuccess)
    rc = efail(e, GPUMHD_E_CUDA, "ensemble: stream/event/counter setup failed");
  for (int b = 0; b < n && rc == 0; b++) {
    cudaEvent_t ev;
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) { rc = efail(e, GPUMHD_E_CUDA, "ensemble: event"); break; }
    e->join.push_back(ev);
    rc = fused_prepare(e->box[b], 1024);
    if (rc) efail(e, rc, e->box[b]->err);
  }
  for (int b = 0; b < n && rc == 0; b++)
    if (cudaStreamSynchronize(e->box[b]->stream) != cudaSuccess) rc = efail(e, GPUMHD_E_CUDA, "ensemble: box stream");
  if (rc == 0) rc = ensemble_build(e, 1, &e->exec);
  if (rc) { ensemble_free(e); return rc; }
  *out = e;
  return GPUMHD_OK;
}

extern "C" int gpumhd_ensemble_set_schedule(gpumhd_ensemble* e, int steps_per_iteration, int largest_first) {
  if (!e || steps_per_iteration < 1 || steps_per_iteration > 64) return GPUMHD_E_INVALID;
  ECK(cudaSetDevice(e->device));
  ECK(cudaStreamSynchronize(e->stream));
  for (gpumhd_ctx* x : e->box) ECK(cudaStreamSynchronize(x->stream));
  if (e->exec) cudaGraphExecDestroy(e->exec);
  if (e->exec_k) cudaGraphExecDestroy(e->exec_k);
  e->exec = e->exec_k = nullptr;
  e->unroll = steps_per_iteration;
  e->largest_first = largest_first != 0;
  int rc = ensemble_build(e, 1, &e->exec);
  if (rc == 0 && e->unroll > 1) rc = ensemble_build(e, e->unroll, &e->exec_k);
  return rc;
}

// Launch shapes inside an ensemble.  A box's own autotuned shapes are the
// fastest for the box alone, which must fill the GPU by itself (short z
// chunks, short TVD chunks: many blocks, each with its own prologue planes and
// stencil halo); inside an ensemble the other boxes fill it, so longer
// marches can pay.  Candidates: each box's current shapes, and stage z chunks
// of half or all of the box's z extent with TVD chunks of 64 or 128 cells;
// timed over trial_steps steps of the whole ensemble (branches largest box
// first) from the boxes' current states, which are restored afterwards.
extern "C" int gpumhd_ensemble_autotune(gpumhd_ensemble* e, int trial_steps, double* best_ms) {
  if (!e || trial_steps < 1) return GPUMHD_E_INVALID;
  ECK(cudaSetDevice(e->device));
  ECK(cudaStreamSynchronize(e->stream));
  const size_t nb = e->box.size();
  std::vector<TrialSave> sv(nb);
  std::vector<int> zc0(nb), td0(nb);
  const int keep_unroll = e->unroll;
  int rc = GPUMHD_OK;
  size_t saved = 0;  // boxes whose trial_save ran (its buffers and flag to give back)
  for (; saved < nb && rc == 0; saved++) {
    gpumhd_ctx* x = e->box[saved];
    zc0[saved] = x->tune_zc;
    td0[saved] = x->tune_td;
    rc = trial_save(x, sv[saved]);
  }
  const bool all_saved = rc == 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (rc == 0 && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
    rc = efail(e, GPUMHD_E_CUDA, "ensemble autotune: events");
  struct Cand { int z; int td; };  // z: 0 = each box's own shapes, 1 = half the z extent, 2 = all of it
  const Cand cands[] = {{0, 0}, {1, 64}, {1, 128}, {2, 64}, {2, 128}};
  auto apply = [&](const Cand& k) {
    for (size_t b = 0; b < nb; b++) {
      gpumhd_ctx* x = e->box[b];
      const int nz = x->c.g.nz;
      x->tune_zc = k.z == 0 ? zc0[b] : (k.z == 1 ? std::max(1, nz / 2) : nz);
      x->tune_td = k.z == 0 ? td0[b] : k.td;
      if (x->graph) { cudaGraphExecDestroy(x->graph); x->graph = nullptr; }
    }
  };
  auto restore_all = [&]() {
    int r = GPUMHD_OK;
    for (size_t b = 0; b < nb && r == 0; b++) r = trial_restore(e->box[b], sv[b]);
    return r;
  };
  double best = 1e300;
  int bi = 0;
  for (int ci = 0; ci < (int)(sizeof(cands) / sizeof(cands[0])) && rc == 0; ci++) {
    apply(cands[ci]);
    rc = gpumhd_ensemble_set_schedule(e, 1, 1);
    if (!rc) rc = restore_all();
    if (!rc) rc = gpumhd_ensemble_enqueue_steps(e, 1);  // untimed first step
    if (rc) break;
    float t = 0.f;
    if (cudaEventRecord(e0, e->stream) != cudaSuccess) { rc = efail(e, GPUMHD_E_CUDA, "ensemble autotune: event"); break; }
    rc = gpumhd_ensemble_enqueue_steps(e, trial_steps);
    if (rc) break;
    if (cudaEventRecord(e1, e->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&t, e0, e1) != cudaSuccess) {
      rc = efail(e, GPUMHD_E_CUDA, "ensemble autotune: timing failed");
      break;
    }
    rc = gpumhd_ensemble_synchronize(e);
    const double ms = (double)t / trial_steps;
    if (!rc && ms < best) { best = ms; bi = ci; }
  }
  // keep the fastest candidate; the boxes' states, compensation and graphs as before
  apply(cands[bi]);
  for (size_t b = 0; b < saved; b++) e->box[b]->p.compensated = sv[b].comp;
  const int rc2 = gpumhd_ensemble_set_schedule(e, keep_unroll, 1);
  if (!rc) rc = rc2;
  if (all_saved) {
    const int rc3 = restore_all();
    if (!rc) rc = rc3;
  }
  for (size_t b = 0; b < nb; b++) cudaStreamSynchronize(e->box[b]->stream);
  for (size_t b = 0; b < saved; b++) trial_free(sv[b]);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (rc) return rc;
  if (best_ms) *best_ms = best;
  return GPUMHD_OK;
}

extern "C" int gpumhd_ensemble_destroy(gpumhd_ensemble* e) {
  if (!e) return GPUMHD_E_INVALID;
  cudaSetDevice(e->device);
  if (e->stream) cudaStreamSynchronize(e->stream);
  ensemble_free(e);
  return GPUMHD_OK;
}

// nsteps steps of every box in one graph launch (stream-ordered after work
// already queued on the boxes' own streams; later calls on a box wait for it).
extern "C" int gpumhd_ensemble_enqueue_steps(gpumhd_ensemble* e, int nsteps) {
  if (!e || nsteps < 0) return GPUMHD_E_INVALID;
  if (nsteps == 0) return GPUMHD_OK;
  ECK(cudaSetDevice(e->device));
  for (size_t b = 0; b < e->box.size(); b++) {
    ECK(cudaEventRecord(e->join[b], e->box[b]->stream));
    ECK(cudaStreamWaitEvent(e->stream, e->join[b], 0));
  }
  if (!e->exec) return efail(e, GPUMHD_E_INVALID, "ensemble has no graph (a failed schedule change)");
  // nsteps / unroll iterations of the unrolled body, the rest one step at a time
  const int nk = e->unroll > 1 ? nsteps / e->unroll : 0;
  const int n1 = nsteps - nk * e->unroll;
  if (nk > 0) {
    k_set_counter<<<1, 32, 0, e->stream>>>(e->d_counter, nk);
    ECK(cudaGraphLaunch(e->exec_k, e->stream));
  }
  if (n1 > 0) {
    k_set_counter<<<1, 32, 0, e->stream>>>(e->d_counter, n1);
    ECK(cudaGraphLaunch(e->exec, e->stream));
  }
  for (gpumhd_ctx* x : e->box) {
    x->res_zero_pending = true;  // Res served as work space
    x->have_pres = true;
    x->launches += (long long)graph_step_launches(x) * nsteps;
  }
  long long per_step = 0;
  for (gpumhd_ctx* x : e->box) per_step += graph_step_launches(x);
  // the boxes' steps, one loop tick per iteration, one counter set per graph launch
  e->launches += per_step * nsteps + (nk + n1) + (nk > 0) + (n1 > 0);
  ECK(cudaEventRecord(e->done, e->stream));
  for (gpumhd_ctx* x : e->box) ECK(cudaStreamWaitEvent(x->stream, e->done, 0));
  return GPUMHD_OK;
}

extern "C" int gpumhd_ensemble_synchronize(gpumhd_ensemble* e) {
  if (!e) return GPUMHD_E_INVALID;
  ECK(cudaSetDevice(e->device));
  if (cudaStreamSynchronize(e->stream) != cudaSuccess) return efail(e, GPUMHD_E_CUDA, "ensemble stream failed");
  for (size_t b = 0; b < e->box.size(); b++) {
    const int rc = gpumhd_synchronize(e->box[b]);
    if (rc) {
      char msg[1024];
      snprintf(msg, sizeof msg, "box %zu: %.900s", b, e->box[b]->err);
      return efail(e, rc, msg);
    }
  }
  return GPUMHD_OK;
}

extern "C" const char* gpumhd_ensemble_last_error(gpumhd_ensemble* e) { return e ? e->err : g_create_err; }
extern "C" void* gpumhd_ensemble_stream(gpumhd_ensemble* e) { return e ? (void*)e->stream : nullptr; }
extern "C" long long gpumhd_ensemble_launch_count(gpumhd_ensemble* e) { return e ? e->launches : 0; }

// ------------------------------------------------------------------- adjoint
// Gradient of an objective J(U_T) with respect to the initial state U_0 over
// nsteps fused FP64 steps of fixed dt, by the hand-written adjoint step
// (adjoint.cu) run backwards in time.  Forward states are kept only every
// checkpoint_every steps; the steps in between are recomputed from the
// nearest checkpoint when the reverse sweep reaches them (memory: one
// checkpoint per segment plus one step's intermediates).
namespace {

struct AdjMem {
  std::vector<void*> all;
  double* get(gpumhd_ctx* ctx, size_t count, int* rc) {
    void* p = nullptr;
    if (*rc) return nullptr;
    if (cudaMalloc(&p, count * sizeof(double)) != cudaSuccess) {
      *rc = fail(ctx, GPUMHD_E_NOMEM, "adjoint: device allocation of %zu doubles failed", count);
      return nullptr;
    }
    all.push_back(p);
    return (double*)p;
  }
  ~AdjMem() {
    for (void* p : all) cudaFree(p);
  }
};

}  // namespace

extern "C" int gpumhd_adjoint(gpumhd_ctx* ctx, int nsteps, int checkpoint_every, const double* dJ_dUT,
                              double* dJ_dU0) {
  if (!ctx || nsteps < 1 || checkpoint_every < 1 || !dJ_dUT || !dJ_dU0) return GPUMHD_E_INVALID;
  if (ctx->f32) return fail(ctx, GPUMHD_E_INVALID, "adjoint: FP64 contexts only");
  if (!ctx->p.periodic_x) return fail(ctx, GPUMHD_E_INVALID, "adjoint: periodic boxes only");
  if (ctx->p.autostep) return fail(ctx, GPUMHD_E_INVALID, "adjoint: needs a fixed time step (autostep = 0, dt > 0)");
  if (!(ctx->p.dt > 0.0)) return fail(ctx, GPUMHD_E_INVALID, "adjoint: dt must be positive");
  if (ctx->c.has_eta) return fail(ctx, GPUMHD_E_INVALID, "adjoint: ideal MHD only (eta = 0)");
  if (ctx->c.divb_on) return fail(ctx, GPUMHD_E_INVALID, "adjoint: without divB cleaning (divB_switch = 0)");
  if (ctx->c.has_spitzer) return fail(ctx, GPUMHD_E_INVALID, "adjoint: without Spitzer conduction (spitzer = 0)");
  if (ctx->c.va_adjust > 0.0) return fail(ctx, GPUMHD_E_INVALID, "adjoint: with fixed limits (va_adjust = 0)");
  CK(cudaSetDevice(ctx->device));
  int rc = fused_prepare(ctx, nsteps);
  if (rc) return rc;
  cudaStream_t s = ctx->stream;
  const Consts& c = ctx->c;
  const size_t N = (size_t)c.g.N;
  const size_t n = (size_t)c.g.nx * c.g.ny * c.g.nz;
  const int ncp = (nsteps + checkpoint_every - 1) / checkpoint_every;
  AdjMem m;
  double *A = m.get(ctx, 8 * N, &rc), *An = m.get(ctx, 8 * N, &rc), *B1 = m.get(ctx, 8 * N, &rc);
  double *B2 = m.get(ctx, 8 * N, &rc), *B3 = m.get(ctx, 8 * N, &rc), *B4 = m.get(ctx, 8 * N, &rc);
  double *V1 = m.get(ctx, 8 * N, &rc), *V2 = m.get(ctx, 8 * N, &rc);
  double *Q0 = m.get(ctx, N, &rc), *Qn = m.get(ctx, N, &rc), *Q1 = m.get(ctx, N, &rc);
  double *Q2 = m.get(ctx, N, &rc), *Q3 = m.get(ctx, N, &rc);
  double* cpU = m.get(ctx, 8 * N * ncp, &rc);
  double* cpP = m.get(ctx, N * ncp, &rc);
  double *lA = m.get(ctx, 8 * n, &rc), *lB = m.get(ctx, 8 * n, &rc), *lC = m.get(ctx, 8 * n, &rc);
  double *lU0 = m.get(ctx, 8 * n, &rc), *lP3 = m.get(ctx, n, &rc), *lP = m.get(ctx, n, &rc);
  double *bdq = m.get(ctx, 36 * n, &rc), *bwc = m.get(ctx, 11 * n, &rc);
  double* tv = m.get(ctx, (size_t)ADJ_TVD_DOUBLES * n, &rc);
  double* tcell = m.get(ctx, 19 * N, &rc);
  Dyn* adyn = nullptr;
  if (!rc && cudaMalloc(&adyn, sizeof(Dyn)) != cudaSuccess) rc = fail(ctx, GPUMHD_E_NOMEM, "adjoint: Dyn");
  if (rc) { cudaFree(adyn); return rc; }
  m.all.push_back(adyn);
  rc = ensure_staging(ctx);
  if (rc) return rc;
  AdjTvdScratch w;
  w.in = tv;
  w.cell = w.in + 8 * n;
  w.fp = w.cell + 19 * n;
  w.fm = w.fp + 9 * n;
  w.iface = w.fm + 9 * n;
  w.slope = w.iface + 92 * n;
  w.tcell = tcell;
  using L = Launch<double>;
  // one recorded forward step: (A, Q0) -> (An, Qn), intermediates kept
  auto record = [&]() {
    k_step_begin<<<1, 32, 0, s>>>(c, adyn, nullptr, 0, 0, 0);
    L::stage(c, A, Q0, A, B1, Q1, nullptr, adyn, 1, false, 1, s);
    L::stage(c, B1, Q1, A, B2, Q2, nullptr, adyn, 2, false, 1, s);
    L::stage(c, B2, Q2, A, B3, Q3, nullptr, adyn, 3, false, 1, s);
    L::stage(c, B3, Q3, A, B4, nullptr, nullptr, adyn, 4, false, 0, s);
    L::tvd(c, 0, 0, 0, B4, Q3, V1, adyn, s);
    L::tvd(c, 1, 0, 0, V1, Q3, V2, adyn, s);
    L::tvd(c, 2, 1, 0, V2, Q3, An, adyn, s);
    L::step_finish(c, An, Qn, adyn, s);
    std::swap(A, An);
    std::swap(Q0, Qn);
  };
  // forward pass: checkpoints every checkpoint_every steps
  CK(cudaMemcpyAsync(adyn, ctx->dyn, sizeof(Dyn), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(A, ctx->S[ctx->iU], 8 * N * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(Q0, ctx->P[ctx->iP], N * sizeof(double), cudaMemcpyDeviceToDevice, s));
  std::vector<Dyn> cpd(ncp);  // step-control block at each checkpoint
  for (int t = 0; t < nsteps; t++) {
    if (t % checkpoint_every == 0) {
      const int q = t / checkpoint_every;
      CK(cudaMemcpyAsync(cpU + 8 * N * q, A, 8 * N * sizeof(double), cudaMemcpyDeviceToDevice, s));
      CK(cudaMemcpyAsync(cpP + N * q, Q0, N * sizeof(double), cudaMemcpyDeviceToDevice, s));
      CK(cudaMemcpyAsync(&cpd[q], adyn, sizeof(Dyn), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
    }
    record();
  }
  ctx->launches += 9LL * nsteps;
  Dyn dchk;
  CK(cudaMemcpyAsync(&dchk, adyn, sizeof(Dyn), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (dchk.err) return fail(ctx, GPUMHD_E_BAD_DT, "adjoint: the forward run failed (device error %d)", dchk.err);
  if (dchk.two_half)
    return fail(ctx, GPUMHD_E_INVALID, "adjoint: the fixed dt needs two TVD half steps (cfl > CFL_tvd); use a smaller dt");
  // reverse pass
  CK(cudaMemcpyAsync(ctx->staging, dJ_dUT, 8 * N * sizeof(double), cudaMemcpyHostToDevice, s));
  adjoint_from_cstate(c, ctx->staging, lA, s);
  for (int t = nsteps - 1; t >= 0; t--) {
    const int q = t / checkpoint_every;
    CK(cudaMemcpyAsync(A, cpU + 8 * N * q, 8 * N * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(Q0, cpP + N * q, N * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(adyn, &cpd[q], sizeof(Dyn), cudaMemcpyHostToDevice, s));
    for (int u = q * checkpoint_every; u < t; u++) record();
    // step t's intermediates: recorded by the last call; inputs back in A, Q0
    record();
    std::swap(A, An);
    std::swap(Q0, Qn);
    ctx->launches += 9LL * (t - q * checkpoint_every + 1);
    CK(cudaMemsetAsync(lP3, 0, n * sizeof(double), s));
    CK(cudaMemsetAsync(lU0, 0, 8 * n * sizeof(double), s));
    adjoint_tvd(c, adyn, 2, V2, Q3, lA, 1, lB, lP3, w, s);
    adjoint_tvd(c, adyn, 1, V1, Q3, lB, 0, lC, lP3, w, s);
    adjoint_tvd(c, adyn, 0, B4, Q3, lC, 0, lB, lP3, w, s);
    adjoint_stage(c, adyn, B3, Q3, A, lB, lU0, lC, lP3, bdq, bwc, 4, s);
    adjoint_eos(c, B3, lP3, lC, s);
    CK(cudaMemsetAsync(lP, 0, n * sizeof(double), s));
    adjoint_stage(c, adyn, B2, Q2, A, lC, lU0, lB, lP, bdq, bwc, 3, s);
    adjoint_eos(c, B2, lP, lB, s);
    CK(cudaMemsetAsync(lP, 0, n * sizeof(double), s));
    adjoint_stage(c, adyn, B1, Q1, A, lB, lU0, lC, lP, bdq, bwc, 2, s);
    adjoint_eos(c, B1, lP, lC, s);
    CK(cudaMemsetAsync(lP, 0, n * sizeof(double), s));
    adjoint_stage(c, adyn, A, Q0, A, lC, lU0, lB, lP, bdq, bwc, 1, s);
    adjoint_eos(c, A, lP, lB, s);
    adjoint_add(c, lB, lU0, lA, s);
    ctx->launches += 12 + 8 + 5;
    rc = check_launch(ctx, 0);
    if (rc) return rc;
  }
  CK(cudaMemsetAsync(ctx->staging, 0, 8 * N * sizeof(double), s));
  adjoint_to_cstate(c, lA, ctx->staging, s);
  CK(cudaMemcpyAsync(dJ_dU0, ctx->staging, 8 * N * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return check_launch(ctx, 0);
}
