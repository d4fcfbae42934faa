// FP64 kernels: compiled with --fmad=false so that every product and sum
// rounds separately, as in the reference's no-FMA builds.
#define GPUMHD_LAUNCH_IMPL
#include "gpumhd_launch.cuh"

namespace gpumhd {

template struct Launch<double>;

__device__ __forceinline__ void step_begin(const Consts& c, Dyn* dyn, double* dt_hist, int dt_hist_cap);

__global__ void k_step_begin(Consts c, Dyn* dyn, double* dt_hist, int dt_hist_cap, cudaGraphConditionalHandle tvd2,
                             int use_cond) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  step_begin(c, dyn, dt_hist, dt_hist_cap);
  if (use_cond) {  // the captured step's second TVD half pass runs only when this step takes it
    const bool take = !dyn->err && dyn->two_half;
    if (take) dyn->cond_launches += 3ULL;
    cudaGraphSetConditional(tvd2, take ? 1u : 0u);
  }
}

// Adjust_Valf_Max with adaptive limits (src/Adjust_Valf_Max.C:92-144) from the
// maxima and near-limit counts the previous pass reduced over the step's
// stage-1 state: the first call takes v_lim and e_lim from the maxima, later
// calls scale them by 1.04 / 1.01 / 0.99 from the counts; va_max follows the
// velocity and sound-speed maxima and decays by at most 1 % per call.  The
// function statics of the reference (ini_flag, va_max_old) live in Dyn.
// Where the reference squares with pow(x, 2.0), this squares with one
// multiplication: the correctly rounded square, which glibc's pow misses by
// one ulp for about 0.1 % of arguments.
__global__ void k_step_limits(Consts c, Dyn* dyn) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (dyn->err) return;
  const double g0 = __longlong_as_double((long long)dyn->stat_max_bits[0]);
  const double g1 = sqrt(__longlong_as_double((long long)dyn->stat_max_bits[1]));
  const double g2 = __longlong_as_double((long long)dyn->stat_max_bits[2]);
  const double n0 = (double)dyn->stat_cnt[0], n1 = (double)dyn->stat_cnt[1];
  const double cs_fac = 2.0, vv_fac = 3.0, eps_decay = 0.99, mf = c.max_fill;
  double v_lim = dyn->v_lim, e_lim = dyn->e_lim;
  if (dyn->va_ini_flag) {
    v_lim = fmin(g0, c.tchk_vmax);
    e_lim = fmin(g2, c.tchk_eps_max);
    dyn->va_max_old = 0.0;
    dyn->va_ini_flag = 0;
  } else {
    if (n0 >= 4 * mf) v_lim *= 1.04;
    else if (n0 >= mf) v_lim *= 1.01;
    else if (n0 < 0.5 * mf) v_lim *= 0.99;
    if (n1 >= 4 * mf) e_lim *= 1.04;
    else if (n1 >= mf) e_lim *= 1.01;
    else if (n1 < 0.5 * mf) e_lim *= 0.99;
  }
  double va_max = fmax(c.va_max, c.va_adjust * vv_fac * g0);
  va_max = fmax(va_max, c.va_adjust * cs_fac * g1);
  va_max = fmax(va_max, dyn->va_max_old * eps_decay);
  v_lim = fmax(v_lim, c.va_max / vv_fac);
  v_lim = fmin(v_lim, c.tchk_vmax);
  const double ef = c.va_max / cs_fac;
  e_lim = fmax(e_lim, ef * ef);
  e_lim = fmin(e_lim, c.tchk_eps_max);
  dyn->v_lim = v_lim;
  dyn->e_lim = e_lim;
  dyn->inv_va2max = 1.0 / (va_max * va_max);
  dyn->va_max_old = va_max;
  // TVDlimit's velocity cap (src/tvdlimit_SR.C:194-197); with vmax_lim >= 1
  // it does not depend on v_lim and keeps the host's value
  if (c.vmax_lim < 1.0) {
    const double vl = c.vmax_lim * v_lim;
    dyn->vsqr_diff = vl * vl;
  }
  derive_one<float>(*dyn, c.dx, c.idx, c.rt_cfl, c.tchk_vmax, c.tchk_eps_max, dyn->rf, c.spt_cfl_dx);
  derive_one<double>(*dyn, c.dx, c.idx, c.rt_cfl, c.tchk_vmax, c.tchk_eps_max, dyn->rd, c.spt_cfl_dx);
  dyn->cmax_bits = 0ULL;  // the CFL pass that follows uses the new inv_va2max
}

__device__ __forceinline__ void step_begin(const Consts& c, Dyn* dyn, double* dt_hist, int dt_hist_cap) {
  if (dyn->err) return;
  // Adjust_Valf_Max (src/Adjust_Valf_Max.C:136-142): without va_adjust the
  // limits are the run constants; with it k_step_limits has set them.
  if (!(c.va_adjust > 0.0)) {
    dyn->v_lim = c.tchk_vmax;
    dyn->e_lim = c.tchk_eps_max;
  }
  dyn->dt_prev = dyn->dt;  // Run.dt as MHD_Residual sees it at stage 1
  const double cmax = __longlong_as_double((long long)dyn->cmax_bits);
  double dt_mhd = c.dxmin / cmax;
  if (c.has_eta) dt_mhd = smin(dt_mhd, c.dt_res);  // resistive limit (src/mhdres_SR.C:815-819)
  dyn->dt_mhd = dt_mhd;
  // Sync_timestep (src/solver.C:487-548) on one rank
  double r0 = c.dt_rad, r1 = dt_mhd;
  if (bad_pos(r0)) { dyn->err = ERR_BAD_DT_RAD; return; }
  if (bad_pos(r1)) { dyn->err = ERR_BAD_DT_MHD; return; }
  const double dt_min_rt = c.rt_tstep * c.CFL * r1;
  if (r0 < dt_min_rt) r0 = smax(r0, dt_min_rt);
  const double dt_min = smin(r0, r1);
  double dt = smin(r0, c.CFL * r1);
  if (c.outcad > 0) {
    const double num = dyn->time / c.outcad;
    const int ce = cvt_x86(num);
    const double rem = (num == (double)ce) ? 0.0 : (ce + 1) * c.outcad - dyn->time;
    if (rem > 0.0) dt = smin(dt, rem);
  }
  if (c.autostep) dyn->dt = dt;
  const double cfl = dyn->dt / dt_min;
  dyn->cfl = cfl;
  if (cfl >= 2.) { dyn->err = ERR_CFL; return; }
  // TVD branch (src/solver.C:325-339)
  dyn->two_half = (cfl <= c.CFL_tvd) ? 0 : 1;
  dyn->dt_tvd = dyn->two_half ? 0.5 * dyn->dt : dyn->dt;
  if (dt_hist && dyn->steps_done >= 0 && dyn->steps_done < dt_hist_cap) dt_hist[dyn->steps_done] = dyn->dt;
  dyn->steps_done += 1;
  dyn->time += dyn->dt;
  derive_one<float>(*dyn, c.dx, c.idx, c.rt_cfl, c.tchk_vmax, c.tchk_eps_max, dyn->rf, c.spt_cfl_dx);
  derive_one<double>(*dyn, c.dx, c.idx, c.rt_cfl, c.tchk_vmax, c.tchk_eps_max, dyn->rd, c.spt_cfl_dx);
  // the last TVD pass of this step accumulates the next step's values
  dyn->cmax_bits = 0ULL;
  dyn->stat_max_bits[0] = dyn->stat_max_bits[1] = dyn->stat_max_bits[2] = 0ULL;
  dyn->stat_cnt[0] = dyn->stat_cnt[1] = 0ULL;
}

}  // namespace gpumhd

namespace gpumhd {

// Loop control of the ensemble's while-graph: one tick per step.
__global__ void k_loop_tick(int* counter, cudaGraphConditionalHandle h) {
  if (threadIdx.x == 0) {
    const int left = --(*counter);
    cudaGraphSetConditional(h, left > 0 ? 1u : 0u);
  }
}

__global__ void k_set_counter(int* counter, int n) {
  if (threadIdx.x == 0) *counter = n;
}

__global__ void k_fused_reinit(Consts c, Dyn* dyn, double inv_va2max, double v_lim, double e_lim, double vsqr_diff) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (!(c.va_adjust > 0.0)) {  // adaptive limits keep their history (the reference's function statics)
    dyn->va_ini_flag = 0;
    dyn->inv_va2max = inv_va2max;
    dyn->v_lim = v_lim;
    dyn->e_lim = e_lim;
    dyn->vsqr_diff = vsqr_diff;
  }
  dyn->err = 0;
  dyn->cmax_bits = 0ULL;
  dyn->stat_max_bits[0] = dyn->stat_max_bits[1] = dyn->stat_max_bits[2] = 0ULL;
  dyn->stat_cnt[0] = dyn->stat_cnt[1] = 0ULL;
  derive_one<float>(*dyn, c.dx, c.idx, c.rt_cfl, c.tchk_vmax, c.tchk_eps_max, dyn->rf, c.spt_cfl_dx);
  derive_one<double>(*dyn, c.dx, c.idx, c.rt_cfl, c.tchk_vmax, c.tchk_eps_max, dyn->rd, c.spt_cfl_dx);
}

__global__ void k_divb_begin(Dyn* dyn) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (dyn->err) return;
  dyn->divb_iters = dyn->divb_next;
  dyn->divb_err_bits[0] = 0ULL;
  dyn->divb_err_bits[1] = 0ULL;
}

// Clean_divB: error ratio and the next call's iteration count (src/clean_divB.C:335-354).
__global__ void k_divb_end(Consts c, Dyn* dyn) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (dyn->err) return;
  const int n = dyn->divb_iters;
  const double e0 = __longlong_as_double((long long)dyn->divb_err_bits[0]) * c.divb_err_unit;
  const double e1 = __longlong_as_double((long long)dyn->divb_err_bits[1]) * c.divb_err_unit;
  const double err = e1 / e0;
  int next = n;
  if (err > c.divb_err) next += 1;
  else next -= 1;
  next = min(next, c.divb_itmax);
  next = max(1, next);
  dyn->divb_next = next;
  dyn->divb_last = n;
  dyn->divb_err0 = e0;
  dyn->divb_err1 = e1;
}


__global__ void k_bc_setup(Consts c, Dyn* dyn, const double* __restrict__ part, int nb) {
  if (dyn->err) return;
  __shared__ double sh[BND_NQ][BND_SETUP_THREADS];
  const int tid = threadIdx.x;
  double t[BND_NQ];
  for (int q = 0; q < BND_NQ; q++) t[q] = 0.0;
  for (int k = tid; k < nb; k += BND_SETUP_THREADS)
    for (int q = 0; q < BND_NQ; q++) t[q] += part[(long long)k * BND_NQ + q];
  for (int q = 0; q < BND_NQ; q++) sh[q][tid] = t[q];
  __syncthreads();
  for (int st = BND_SETUP_THREADS / 2; st > 0; st >>= 1) {
    if (tid < st)
      for (int q = 0; q < BND_NQ; q++) sh[q][tid] += sh[q][tid + st];
    __syncthreads();
  }
  if (tid != 0) return;
  for (int q = 0; q < BND_NQ; q++) t[q] = sh[q][0];
  const double n = (double)(c.g.ny * c.g.nz);
  if (dyn->bnd_ini) {
    const double b0 = t[2] / n, b1 = t[3] / n;
    if (dyn->p_bc < 0.0) dyn->p_bc = b0 * sqrt(b0 / b1);
    if (dyn->s_bc < 0.0) dyn->s_bc = (t[4] > 0.0) ? t[5] / t[4] : t[6] / n;
    dyn->bnd_ini = 0;
  }
  const double cn = 1.0 / n;
  dyn->pmean1 = t[0] * cn;
  dyn->pmean2 = t[1] * cn;
}

}  // namespace gpumhd
