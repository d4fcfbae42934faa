// Hyperbolic Spitzer heat conduction (src/mhdres_SR.C:33-46, 121-145,
// 251-253, 355-358, 492-521, 668-692; src/Add_Sources_Integrate_SR.C:410-419).
//
// A ninth field, the heat flux along B (sflx), enters the energy flux as
// sflx * B_d in each direction d.  Its residual Rflx is a hyperdiffusion of
// sflx per direction plus, once B.grad T is complete, a relaxation towards
// the saturation-limited Spitzer flux -kappa(T) B.grad T / |B|^2 at the rate
// nu_hyp, capped by the previous time step.  The RK stage then updates
// sflx = sflx0 + wdt * Rflx.
//
// Here one kernel per stage does all of it for a cell: the three directions'
// share of the energy residual (-D_d(sflx * B_d), summed into Rsp for the
// stage kernel, which adds it to R.e), B.grad T, Rflx and -- in the fused
// step -- the update of sflx into the next buffer.  The reference adds
// sflx * B_d to the energy flux before differencing; summing the two
// differences separately changes the residual at the rounding level only.
#pragma once
#include "gpumhd_kernels.cuh"

namespace gpumhd {

constexpr int SPT_BX = 32, SPT_BY = 8;

// the floor of |B|^2 in 1/|B|^2: 1e-100 (src/mhdres_SR.C:511), in FP32 a
// normal float instead
template <class R> __device__ __forceinline__ R spt_bbmin();
template <> __device__ __forceinline__ double spt_bbmin<double>() { return 1e-100; }
template <> __device__ __forceinline__ float spt_bbmin<float>() { return 1e-30f; }

// ConsToPrim's temperature (src/cons_to_prim.C:148-243), with the pressure its
// fallback tests: c2p_eos_full's arithmetic for those two outputs.
__device__ inline double c2p_temp(const Consts& c, double d, double ei, double dn) {
  const double eps = ei * dn + c.eps_off;
  const double lgr = log(d);
  const double ep = log(eps);
  const double lr = lgr;
  int i_d = cvt_x86((lr - c.xlr0) * c.inv_del_lr);
  i_d = max(0, i_d);
  i_d = min(c.N_lr - 2, i_d);
  int i_e = cvt_x86((ep - c.xeps0) * c.inv_del_eps);
  i_e = max(0, i_e);
  i_e = min(c.N_eps - 2, i_e);
  const double xe0 = c.xeps[i_e], xe1 = c.xeps[i_e + 1];
  const double xr0 = c.xlr[i_d], xr1 = c.xlr[i_d + 1];
  const double c0 = (ep - xe0) * (lr - xr0);
  const double c1 = (ep - xe0) * (xr1 - lr);
  const double c2 = (xe1 - ep) * (lr - xr0);
  const double c3 = (xe1 - ep) * (xr1 - lr);
  const long long a11 = (long long)(i_e + 1) * c.N_lr + (i_d + 1);
  const long long a10 = (long long)(i_e + 1) * c.N_lr + i_d;
  const long long a01 = (long long)i_e * c.N_lr + (i_d + 1);
  const long long a00 = (long long)i_e * c.N_lr + i_d;
  double out[2];
#pragma unroll
  for (int t = 0; t < 2; t++) {
    const float* T = c.tab[t];
    double s = c0 * (double)T[a11];
    s += c1 * (double)T[a10];
    s += c2 * (double)T[a01];
    s += c3 * (double)T[a00];
    out[t] = exp(s);
  }
  double pr = out[0], tm = out[1];
  if (lgr < c.xlr0) {
    pr = c.c_pres * ei;
    tm = c.c_temp * eps;
  }
  if (eps > 0.8 * c.eps_max) {
    double xx = smax(0.0, 5.0 * (c.eps_max - eps) / c.eps_max);
    pr = pr * xx + (1.0 - xx) * c.c_pres * ei;
    tm = tm * xx + (1.0 - xx) * c.c_temp * eps;
  }
  if (bad_pos(pr) || bad_pos(tm)) tm = c.c_temp * eps;
  return tm;
}

// Temperature of every cell, ghosts included, of a conserved state.
template <class R>
__global__ void __launch_bounds__(256) k_temp(Consts c, const R* __restrict__ U, R* __restrict__ T) {
  const Geom& g = c.g;
  for (long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < g.N; id += (long long)gridDim.x * blockDim.x) {
    R v1, v2, v3, ei;
    const R d = U[id];
    prim_from_cons(d, U[g.N + id], U[2 * g.N + id], U[3 * g.N + id], U[4 * g.N + id], v1, v2, v3, ei);
    T[id] = (R)c2p_temp(c, (double)d, (double)ei, 1.0 / (double)d);
  }
}

// One interior cell per thread (block 32 x 8 over x, y; z planes by the
// grid's third dimension).  U: conserved (fused step) or primitive (after
// ConsToPrim, PRIM).  T: temperature; S: sflx with its ghosts; stage: 1-4
// in the fused step (stage 1 takes the previous step's dt for the relaxation
// caps, as MHD_Residual runs before Sync_timestep there), 0 per routine
// (the context's dt).  Outputs: Rsp (the energy residual's share), and
// either Sout = S0 + wdt*Rflx with its periodic images (fused; Sout may be
// S0 itself, each cell reading its own value before writing it) or Rflx.
template <class R, bool PRIM>
__global__ void __launch_bounds__(SPT_BX* SPT_BY) k_spitzer(Consts c, const R* __restrict__ U, const R* __restrict__ T,
                                                           const R* __restrict__ S, const R* S0, R* Sout,
                                                           R* __restrict__ Rflx,
                                                           R* __restrict__ Rsp, const Dyn* __restrict__ dyn,
                                                           int stage) {
  if (dyn->err) return;
  const Geom& g = c.g;
  const int i = GH + blockIdx.x * SPT_BX + threadIdx.x;
  const int j = GH + blockIdx.y * SPT_BY + threadIdx.y;
  if (i >= GH + g.nx || j >= GH + g.ny) return;
  // the relaxation's caps from the time step (src/mhdres_SR.C:137-145)
  const double dt_h = (stage == 1) ? dyn->dt_prev : dyn->dt;
  const double CFL_hyp = 1.8, avr_max = 0.25, eps_hyp = 0.02;
  double cmax_hyp_d, nu_hyp_max_d, hyp_diff_d;
  if (dt_h > 0.0) {
    cmax_hyp_d = smin(c.CFL, CFL_hyp) * c.dxmin / dt_h;
    nu_hyp_max_d = avr_max / dt_h;
    hyp_diff_d = eps_hyp / dt_h;
  } else {
    cmax_hyp_d = 0.0;
    nu_hyp_max_d = avr_max * cmax_hyp_d / (smin(c.CFL, CFL_hyp) * c.dxmin);
    hyp_diff_d = eps_hyp * cmax_hyp_d / (smin(c.CFL, CFL_hyp) * c.dxmin);
  }
  const R cmax_hyp = (R)cmax_hyp_d, nu_hyp_max = (R)nu_hyp_max_d, hyp_diff = (R)hyp_diff_d;
  const R k0 = (R)c.spitzer, sat_flx = (R)c.spt_sat_flx;
  const R wdt = dynr<R>(dyn).wdt[stage > 0 ? stage : 0];
  const auto& kk = kc<R>(c);
  const unsigned st[3] = {1u, (unsigned)g.sx, (unsigned)g.sx * (unsigned)g.sy};
  for (int k = GH + blockIdx.z; k < GH + g.nz; k += gridDim.z) {
    const unsigned id = cidx32(g, i, j, k);
    R rsp = (R)0, bgt = (R)0, rfl = (R)0;
    const R s0 = S[id];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const R* Bd = U + (unsigned)(5 + d) * g.N32;
      const unsigned sd = st[d];
      const R w1 = kk.w1[d], w2 = kk.w2[d];
      const R sp1 = S[id + sd], sm1 = S[id - sd], sp2 = S[id + 2 * sd], sm2 = S[id - 2 * sd];
      const R bp1 = Bd[id + sd], bm1 = Bd[id - sd], bp2 = Bd[id + 2 * sd], bm2 = Bd[id - 2 * sd];
      rsp += (R)0 - (w1 * (sp1 * bp1 - sm1 * bm1) + w2 * (sp2 * bp2 - sm2 * bm2));
      bgt += (Bd[id] * (w1 * (T[id + sd] - T[id - sd]) + w2 * (T[id + 2 * sd] - T[id - 2 * sd])));
      rfl -= hyp_diff * ((sp2 + sm2) - (R)4. * (sp1 + sm1) + (R)6. * s0);
    }
    // relaxation to the limited Spitzer flux (src/mhdres_SR.C:503-519)
    const R d = U[id];
    R v1, v2, v3, ei;
    if (PRIM) {
      v1 = U[g.N32 + id]; v2 = U[2u * g.N32 + id]; v3 = U[3u * g.N32 + id]; ei = U[4u * g.N32 + id];
    } else {
      prim_from_cons(d, U[g.N32 + id], U[2u * g.N32 + id], U[3u * g.N32 + id], U[4u * g.N32 + id], v1, v2, v3, ei);
    }
    const R b5 = U[5u * g.N32 + id], b6 = U[6u * g.N32 + id], b7 = U[7u * g.N32 + id];
    const R vv = d_sqrt(v1 * v1 + v2 * v2 + v3 * v3);
    const R bb = b5 * b5 + b6 * b6 + b7 * b7;
    const R tempi = T[id];
    const R c_lim = cmax_hyp - vv;
    const R tt32 = tempi * d_sqrt(tempi);
    R kap_spt = k0 * tempi * tt32;
    const R F_sat = sat_flx * d * tt32;
    const R invBB = (R)1.0 / smax(spt_bbmin<R>(), bb);
    R F_spt = -kap_spt * bgt;
    const R f_lim = F_sat / (F_sat + d_fabs(F_spt * d_sqrt(invBB)));
    F_spt *= invBB * f_lim;
    kap_spt *= f_lim;
    const R nu_hyp = smin(c_lim * c_lim * ei / (tempi * kap_spt), nu_hyp_max);
    rfl += nu_hyp * (F_spt - s0);
    Rsp[id] = rsp;
    if (Rflx) Rflx[id] = rfl;
    if (Sout) {
      const R sn = S0[id] + wdt * rfl;
      // the cell and its periodic images (the exchange of the heat flux)
      const Images im = images_of(g, i, j, k, false);
      for_images<true>(g, i, j, k, im, [&](unsigned long long gid, bool) { Sout[(unsigned)gid] = sn; });
    }
  }
}

// The per-routine update of the heat flux in Source_Integrate
// (src/Add_Sources_Integrate_SR.C:410-419): sflx = sflx0 + wdt*Rflx, Rflx = 0.
template <class R>
__global__ void k_sflx_update(Consts c, R* __restrict__ S, const R* __restrict__ S0, R* __restrict__ Rflx,
                              const Dyn* __restrict__ dyn, int stage) {
  const Geom& g = c.g;
  const R wdt = dynr<R>(dyn).wdt[stage];
  const long long n = (long long)g.nx * g.ny * g.nz;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = GH + (int)(t % g.nx), j = GH + (int)((t / g.nx) % g.ny), k = GH + (int)(t / ((long long)g.nx * g.ny));
    const long long id = cidx(g, i, j, k);
    S[id] = S0[id] + wdt * Rflx[id];
    Rflx[id] = (R)0;
  }
}

}  // namespace gpumhd
