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

// Temperature in FP32, as eos_pres's FP32 path does the pressure: inside the
// table (and away from the high-eps blend) the offsets from the cell's lower
// corner come from ln of ratios near one, and the bilinear weights are the
// offsets and the cell width minus them (so that they sum to the cell area the
// table values are divided by); elsewhere the FP64 routine decides.
__device__ __forceinline__ float eos_temp(const Consts& c, float d, float ei, float dn) {
  constexpr float LN2 = 0.69314718f;
  const KC<float>& k = c.kf;
  const float eps = ei * dn + k.eps_off;
  const float lgr = __log2f(d) * LN2;
  const float ep = __log2f(eps) * LN2;
  if (!(lgr >= k.xlr0 + 0.01f && lgr < k.xlrN + 1.0f && ep > k.xeps0 - 1.0f && ep < k.xepsN + 1.0f &&
        !(eps > 0.8f * k.eps_max)))
    return (float)c2p_temp(c, (double)d, (double)ei, 1.0 / (double)d);
  int i_d = (int)((lgr - k.xlr0) * k.inv_del_lr);
  i_d = max(0, min(c.N_lr - 2, i_d));
  int i_e = (int)((ep - k.xeps0) * k.inv_del_eps);
  i_e = max(0, min(c.N_eps - 2, i_e));
  const float fe = log1p_small(eps * __ldg(c.inv_exp_xeps + i_e) - 1.0f);
  const float fr = log1p_small(d * __ldg(c.inv_exp_xlr + i_d) - 1.0f);
  const float ge = k.del_eps - fe, gr = k.del_lr - fr;
  const float* T = c.tab[1];
  const long long r1 = (long long)(i_e + 1) * c.N_lr + i_d;
  const long long r0 = (long long)i_e * c.N_lr + i_d;
  const float s = fe * fr * __ldg(T + r1 + 1) + fe * gr * __ldg(T + r1) + ge * fr * __ldg(T + r0 + 1) +
                  ge * gr * __ldg(T + r0);
  return expf(s);
}
__device__ __forceinline__ float temp_of(const Consts& c, float d, float ei) { return eos_temp(c, d, ei, 1.0f / d); }
__device__ __forceinline__ double temp_of(const Consts& c, double d, double ei) { return c2p_temp(c, d, ei, 1.0 / d); }

// Temperature of every cell, ghosts included, of a conserved state.
template <class R>
__global__ void __launch_bounds__(256, EwBlocks<R>::v) k_temp(Consts c, const R* __restrict__ U, R* __restrict__ T) {
  const Geom& g = c.g;
  const unsigned N = g.N32;
  for (unsigned id = gs_first(); id < N; id += gs_step()) {
    R v1, v2, v3, ei;
    const R d = U[id];
    prim_from_cons(d, U[N + id], U[2 * N + id], U[3 * N + id], U[4 * N + id], v1, v2, v3, ei);
    T[id] = temp_of(c, d, ei);
  }
}

// One thread per (x, y) column of a chunk of zc interior z planes (block
// 32 x 8); the z stencils of the heat flux, the temperature and B_z move
// through five-value register windows, so a plane costs three new z loads,
// and those and the cell's own values are loaded a plane ahead of their use
// (80 registers; 0.34 -> 0.24 ms per launch at 128 x 384 x 384, FP32).
// U: conserved (fused step) or primitive (after ConsToPrim, PRIM).  T:
// temperature; S: sflx with its ghosts; stage: 1-4 in the fused step (stage
// 1 takes the previous step's dt for the relaxation caps, as MHD_Residual
// runs before Sync_timestep there), 0 per routine (the context's dt).
// Outputs: Rsp (the energy residual's share), and either Sout = S0 + wdt*Rflx
// with its periodic images (fused; Sout may be S0 itself, each cell reading
// its own value before writing it) or Rflx.
template <class R, bool PRIM>
__global__ void __launch_bounds__(SPT_BX* SPT_BY) k_spitzer(Consts c, const R* __restrict__ U, const R* __restrict__ T,
                                                           const R* __restrict__ S, const R* S0, R* Sout,
                                                           R* __restrict__ Rflx, R* __restrict__ Rsp,
                                                           const Dyn* __restrict__ dyn, int stage, int zc) {
  if (dyn->err) return;
  const Geom& g = c.g;
  const int i = GH + blockIdx.x * SPT_BX + threadIdx.x;
  const int j = GH + blockIdx.y * SPT_BY + threadIdx.y;
  if (i >= GH + g.nx || j >= GH + g.ny) return;
  const int k0 = GH + blockIdx.z * zc;
  const int k1 = min(k0 + zc, GH + g.nz);
  // the relaxation's caps from the time step (src/mhdres_SR.C:137-145),
  // derived once per step with the step scalars: stage 1 of a fused step
  // takes the previous step's dt, everything else the current one
  const int qd = (stage == 1) ? 0 : 1;
  const DynR<R>& drr = dynr<R>(dyn);
  const R cmax_hyp = drr.spt_cmax[qd], nu_hyp_max = drr.spt_numax[qd], hyp_diff = drr.spt_hyp[qd];
  const R k0s = (R)c.spitzer, sat_flx = (R)c.spt_sat_flx;
  const R wdt = dynr<R>(dyn).wdt[stage > 0 ? stage : 0];
  const auto& kk = kc<R>(c);
  const unsigned sy = (unsigned)g.sx, sz = (unsigned)g.sx * (unsigned)g.sy;
  const R* Bx = U + 5u * g.N32;
  const R* By = U + 6u * g.N32;
  const R* Bz = U + 7u * g.N32;
  const unsigned col = (unsigned)i + (unsigned)j * sy;
  // z windows at k-2 .. k+2, plus the plane k+3 values loaded a plane ahead
  R sw[5], tw[5], bw[5];
#pragma unroll
  for (int o = 0; o < 5; o++) {
    const unsigned id = col + (unsigned)(k0 - 2 + o) * sz;
    sw[o] = S[id]; tw[o] = T[id]; bw[o] = Bz[id];
  }
  // the cell's own values, loaded a plane ahead
  struct Own { R d, a1, a2, a3, a4, bx, by, s0; };
  auto load_own = [&](unsigned id, Own& o) {
    o.d = U[id]; o.a1 = U[g.N32 + id]; o.a2 = U[2u * g.N32 + id]; o.a3 = U[3u * g.N32 + id];
    o.a4 = U[4u * g.N32 + id]; o.bx = Bx[id]; o.by = By[id]; o.s0 = Sout ? S0[id] : (R)0;
  };
  Own cur;
  load_own(col + (unsigned)k0 * sz, cur);
  for (int k = k0; k < k1; k++) {
    const unsigned id = col + (unsigned)k * sz;
    R sn3 = (R)0, tn3 = (R)0, bn3 = (R)0;
    Own nxt = cur;
    if (k + 1 < k1) {
      const unsigned id3 = id + 3 * sz;
      sn3 = S[id3]; tn3 = T[id3]; bn3 = Bz[id3];
      load_own(id + sz, nxt);
    }
    const R s0 = sw[2];
    R rsp = (R)0, bgt = (R)0, rfl = (R)0;
    auto dir = [&](R w1, R w2, R sp1, R sm1, R sp2, R sm2, R bp1, R bm1, R bp2, R bm2, R b0, R tp1, R tm1, R tp2,
                   R tm2) {
      rsp += (R)0 - (w1 * (sp1 * bp1 - sm1 * bm1) + w2 * (sp2 * bp2 - sm2 * bm2));
      bgt += (b0 * (w1 * (tp1 - tm1) + w2 * (tp2 - tm2)));
      rfl -= hyp_diff * ((sp2 + sm2) - (R)4. * (sp1 + sm1) + (R)6. * s0);
    };
    dir(kk.w1[0], kk.w2[0], S[id + 1], S[id - 1], S[id + 2], S[id - 2], Bx[id + 1], Bx[id - 1], Bx[id + 2],
        Bx[id - 2], cur.bx, T[id + 1], T[id - 1], T[id + 2], T[id - 2]);
    dir(kk.w1[1], kk.w2[1], S[id + sy], S[id - sy], S[id + 2 * sy], S[id - 2 * sy], By[id + sy], By[id - sy],
        By[id + 2 * sy], By[id - 2 * sy], cur.by, T[id + sy], T[id - sy], T[id + 2 * sy], T[id - 2 * sy]);
    dir(kk.w1[2], kk.w2[2], sw[3], sw[1], sw[4], sw[0], bw[3], bw[1], bw[4], bw[0], bw[2], tw[3], tw[1], tw[4],
        tw[0]);
    // relaxation to the limited Spitzer flux (src/mhdres_SR.C:503-519)
    const R d = cur.d;
    R v1, v2, v3, ei;
    if (PRIM) {
      v1 = cur.a1; v2 = cur.a2; v3 = cur.a3; ei = cur.a4;
    } else {
      prim_from_cons(d, cur.a1, cur.a2, cur.a3, cur.a4, v1, v2, v3, ei);
    }
    const R b5 = cur.bx, b6 = cur.by, b7 = bw[2];
    const R vv = d_sqrt(v1 * v1 + v2 * v2 + v3 * v3);
    const R bb = b5 * b5 + b6 * b6 + b7 * b7;
    const R tempi = tw[2];
    const R c_lim = cmax_hyp - vv;
    const R tt32 = tempi * d_sqrt(tempi);
    R kap_spt = k0s * tempi * tt32;
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
      const R sn = cur.s0 + wdt * rfl;
      // the cell and its periodic images (the exchange of the heat flux)
      const Images im = images_of(g, i, j, k, false);
      for_images<true>(g, i, j, k, im, [&](unsigned long long gid, bool) { Sout[(unsigned)gid] = sn; });
    }
#pragma unroll
    for (int o = 0; o < 4; o++) { sw[o] = sw[o + 1]; tw[o] = tw[o + 1]; bw[o] = bw[o + 1]; }
    sw[4] = sn3; tw[4] = tn3; bw[4] = bn3;
    cur = nxt;
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
  for (unsigned t = gs_first(); t < (unsigned)n; t += gs_step()) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const unsigned id = cidx32(g, i, j, k);
    S[id] = S0[id] + wdt * Rflx[id];
    Rflx[id] = (R)0;
  }
}

}  // namespace gpumhd
