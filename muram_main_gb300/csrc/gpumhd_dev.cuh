// Device-side data structures and per-cell arithmetic of the MURaM MHD step.
//
// Templates take the state type R (double or float).  The FP64 instantiation
// is compiled without FMA contraction and follows the reference's operation
// order term by term, so that it rounds like the reference's CPU build; the
// FP32 instantiation uses the same formulas in float (with contraction) and
// an interpolation form of the pressure lookup that keeps float accuracy.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace gpumhd {

constexpr int NV = 8;   // rho, M_x, M_y, M_z, e, B_x, B_y, B_z
constexpr int GH = 2;   // ghost layers

struct Geom {
  int nx, ny, nz;       // interior
  int sx, sy, sz;       // with ghosts
  long long N;          // sx*sy*sz
  int periodic_x;
  unsigned N32;         // N as 32-bit: every offset q*N + cell of the 8 state arrays is below 2^32
  int xmirror;          // closed x with the mirror rule at both ends (0: periodic, or MURaM's physical boundaries)
  int pad_g;
};

// Run constants in the kernel's own type, converted once on the host: the
// FP32 kernels never touch the (slow) FP64 pipe for them, and the FP64 copies
// are the original values.
template <class R>
struct KC {
  R eps_off, xeps0, xlr0, xepsN, xlrN, inv_del_eps, inv_del_lr, eps_max;
  R rho_min, eps_min, rho_lev, q_rho_max;
  R visc_coeff_bot, visc_slope_bot, visc_coeff_top, visc_slope_top;
  R eta_coeff_bot, eta_slope_bot, eta_coeff_top, eta_slope_top;
  R B_par_diff, vhyp, pm_v, pm_B, CME_thresh;
  R tvd_h[4], tvd_cs[4], tvd_coeff[4];
  R CZ, tchk_vmax, tchk_eps_max, gx;
  R w1[3], w2[3];
  R eta, ww0[3], ww1[3], ww2[3];  // resistivity and the second-derivative stencil
  R divb_fac, divb_damp;          // divB cleaning: phi += fac*divB - damp*phi
  R del_eps, del_lr;              // EOS cell widths (FP32 temperature lookup)
  const R* hfb;   // vertical boundary profiles, length sx
  const R* hft;
  const R* qft;
  int has_visc_slope, has_eta_slope, has_vmax_lim, has_vhyp;
};

// Constants of the physical x boundaries' EOS lookups and formulas: table
// axes as x0 + del*i (src/eos_init.C:125-146), offsets, B_crit (code units)
// and eps_top.
template <class R>
struct BndK {
  R eps0, del_eps, inv_del_eps, lr0, del_lr, inv_del_lr;
  R lp30, del_lp3, inv_del_lp3, s30, del_s3, inv_del_s3;
  R eps_off, ss_off, bcrit, eps_top;
};

// Constants of a run (copied by value into every kernel).
struct Consts {
  Geom g;
  double dx[3], w1[3], w2[3], idx[3], dxmin;
  // EOS (src/eos_init.C:57-212)
  int N_eps, N_lr;
  double eps_off, xeps0, xlr0, xepsN, xlrN, inv_del_eps, inv_del_lr, eps_max;
  const double* xeps;
  const double* xlr;
  const float* tab[6];         // [i_eps*N_lr + j_rho], divided by del_eps*del_lr
  const float4* pquad;         // FP32 pressure patches {exp(T00), a, b, c}
  const float* inv_exp_xeps;   // exp(-xeps[i])
  const float* inv_exp_xlr;    // exp(-xlr[j])
  double c_pres, c_temp, kb, mun_mh;
  // TVD (src/tvdlimit_SR.C:41-205)
  double rho_min, eps_min, rho_lev, q_rho_max;
  int rho_log, need_coeff;
  double visc_coeff_bot, visc_slope_bot, visc_coeff_top, visc_slope_top;
  double eta_coeff_bot, eta_slope_bot, eta_coeff_top, eta_slope_top;
  double B_par_diff, vhyp, pm_v, pm_B, vmax_lim, CME_thresh;
  double tvd_h[4], tvd_cs[4], tvd_coeff[4];
  double CZ;                   // (double)(Tau > 1e-5) for the constant optical depth
  const double* hfb;           // vertical boundary profiles, length sx
  const double* hft;
  const double* qft;
  // Tcheck and sources
  double tchk_vmax, tchk_eps_max;
  double gx;                   // PhysicsData::g[0] = -grav
  double eta, dt_res;          // resistivity and its time-step limit (eta > 0 only)
  int has_eta, pad3;
  // divB cleaning (src/clean_divB.C:43-101): on, iteration cap, target ratio, error unit
  int divb_on, divb_itmax;
  double divb_err, divb_err_unit, divb_fac_d;
  // physical x boundaries (src/boundary_pdmp_1_fftw3.C:81-565): on, top mode,
  // the EOS's inverse tables and the lookup constants per precision
  int xbnd, bnd_top;
  int N_lp3, N_s3;
  const float* d3;     // ln rho (p, s), [i_lp*N_s3 + j_s], pre-divided
  const float* eps3;   // ln eps (p, s)
  BndK<double> bndd;
  // hyperbolic Spitzer conduction: coefficient (0: off), saturation flux
  // factor (1+X_H) Rgas^1.5 sqrt(1836)/8 (src/mhdres_SR.C:40-46)
  double spitzer, spt_sat_flx;
  double spt_cfl_dx;  // min(CFL, 1.8) * dxmin, the hyperbolic speed cap's numerator (src/mhdres_SR.C:137-145)
  int has_spitzer, pad_spt;
  const void* spt_rsp;  // the energy residual's Spitzer share for this stage (N, state precision)
  double rt_cfl;
  double CFL, CFL_tvd, dt_rad, rt_tstep, outcad;
  double va_max, va_adjust, max_fill;
  int autostep;
  // test hook of the TMA stage kernel's bounded waits: withhold the copy of
  // each block's last plane (its wait then runs out); the wait limit in clock
  // cycles for the planes' copies
  int tm_withhold_last;
  long long tm_wait_cycles;
  KC<float> kf;
  KC<double> kd;
};

// Run constants for arithmetic type R (a trait, so that other arithmetic
// types -- the adjoint's dual numbers -- can map to one of the two sets).
template <class R> struct KCSel;
template <> struct KCSel<float> {
  using T = KC<float>;
  static __device__ __forceinline__ const T& get(const Consts& c) { return c.kf; }
};
template <> struct KCSel<double> {
  using T = KC<double>;
  static __device__ __forceinline__ const T& get(const Consts& c) { return c.kd; }
};
template <class R> __device__ __forceinline__ const typename KCSel<R>::T& kc(const Consts& c) {
  return KCSel<R>::get(c);
}

// Per-step scalars in a kernel's type, derived from the double values once
// per step (host for the per-routine calls, k_step_begin on the device).
template <class R>
struct DynR {
  R dt_tvd, cmax_t[3], fac0[3];      // TVDlimit: dt, 0.975*dx/dt, 0.5/dx (src/tvdlimit_SR.C:230, 455-457)
  R inv_va2max, vsqr_diff;
  R vmax, emax, vlim95, elim95;      // Tcheck limits, Adjust_Valf_Max thresholds
  R wdt[5], invRdt;                  // dt/(5-stage), rt_cfl/dt (src/Add_Sources_Integrate_SR.C:44, 85)
  // Spitzer relaxation caps (src/mhdres_SR.C:137-145) for [0] the previous
  // step's dt (stage 1 of a fused step) and [1] the current dt
  R spt_cmax[2], spt_numax[2], spt_hyp[2];
};

// Values that change during a run; live in device memory.
struct Dyn {
  double dt, cfl, time;
  double inv_va2max, v_lim, e_lim, va_max_old;
  int va_ini_flag, two_half, err, steps_done;
  double dt_tvd;
  double vsqr_diff;     // pow(vmax_lim*v_lim, 2) or pow(vmax_lim, 2), from the host (src/tvdlimit_SR.C:194-197)
  // accumulators of the last reduction pass
  unsigned long long cmax_bits;
  unsigned long long stat_max_bits[3];
  unsigned long long stat_cnt[2];
  double dt_mhd;
  DynR<float> rf;
  DynR<double> rd;
  // divB cleaning: the adaptive iteration count (a function static of
  // Clean_divB, starts at 3), this call's count, max|divB| before the
  // iterations and after the latest one (bit patterns, reduced by atomics),
  // and the last call's errors in G
  int divb_next, divb_iters;
  unsigned long long divb_err_bits[2];
  double divb_err0, divb_err1;
  int divb_last, divb_pad;
  // physical x boundaries: the bottom's pressure and entropy (negative: set
  // by the first call), the first call still pending, the latest mean pressures
  double p_bc, s_bc, pmean1, pmean2;
  int bnd_ini, bnd_pad;
  double dt_prev;       // the previous step's dt (Spitzer relaxation caps at stage 1)
  // kernels a captured step launched through its conditional nodes (the
  // second TVD half pass), counted by k_step_begin when it enables them
  unsigned long long cond_launches;
};

template <class R> __device__ __forceinline__ const DynR<R>& dynr(const Dyn* d);
template <> __device__ __forceinline__ const DynR<float>& dynr<float>(const Dyn* d) { return d->rf; }
template <> __device__ __forceinline__ const DynR<double>& dynr<double>(const Dyn* d) { return d->rd; }

enum { ERR_BAD_DT_RAD = 1, ERR_BAD_DT_MHD = 2, ERR_CFL = 3 };

template <class R>
__host__ __device__ inline void derive_one(const Dyn& d, const double dx[3], const double idx[3], double rt_cfl,
                                           double tchk_vmax, double tchk_eps_max, DynR<R>& r,
                                           double spt_cfl_dx = 0.0) {
  r.dt_tvd = (R)d.dt_tvd;
  for (int q = 0; q < 3; q++) {
    r.cmax_t[q] = (R)(0.975 * dx[q] / d.dt_tvd);
    r.fac0[q] = (R)(0.5 * idx[q]);
  }
  r.inv_va2max = (R)d.inv_va2max;
  r.vsqr_diff = (R)d.vsqr_diff;
  r.vmax = (R)(d.v_lim > 0.0 ? d.v_lim : tchk_vmax);
  r.emax = (R)(d.e_lim > 0.0 ? d.e_lim : tchk_eps_max);
  r.vlim95 = (R)(d.v_lim * 0.95);
  r.elim95 = (R)(d.e_lim * 0.95);
  r.wdt[0] = (R)0;
  for (int st = 1; st <= 4; st++) r.wdt[st] = (R)(d.dt / (double)(4 + 1 - st));
  r.invRdt = (R)(rt_cfl / d.dt);
  // spt_cfl_dx = min(CFL, CFL_hyp = 1.8) * dxmin
  for (int q = 0; q < 2; q++) {
    const double dth = q == 0 ? d.dt_prev : d.dt;
    double cm, nu, hy;
    if (dth > 0.0) {
      cm = spt_cfl_dx / dth;
      nu = 0.25 / dth;
      hy = 0.02 / dth;
    } else {
      cm = 0.0;
      nu = 0.25 * cm / spt_cfl_dx;
      hy = 0.02 * cm / spt_cfl_dx;
    }
    r.spt_cmax[q] = (R)cm;
    r.spt_numax[q] = (R)nu;
    r.spt_hyp[q] = (R)hy;
  }
}

// ---------------------------------------------------------------- helpers
// std::max / std::min semantics: the first argument wins ties and NaNs.
template <class R> __device__ __forceinline__ R smax(R a, R b) { return (a < b) ? b : a; }
template <class R> __device__ __forceinline__ R smin(R a, R b) { return (b < a) ? b : a; }
// FP32 mode: one min/max instruction instead of a compare and a select; it
// differs from std::max/min only in which operand a NaN or a signed zero
// yields, which the FP32 mode does not reproduce anyway.
template <> __device__ __forceinline__ float smax<float>(float a, float b) { return fmaxf(a, b); }
template <> __device__ __forceinline__ float smin<float>(float a, float b) { return fminf(a, b); }

// The reference's 1e-100 floors; float cannot hold 1e-100, so FP32 uses 1e-30.
template <class R> struct Tiny100 { static __device__ __forceinline__ double get() { return 1e-100; } };
template <> struct Tiny100<float> { static __device__ __forceinline__ float get() { return 1e-30f; } };
template <class R> __device__ __forceinline__ R tiny100() { return (R)Tiny100<R>::get(); }

// Storage of the FP32 compensated mode's rounding remainders: bfloat16.  A
// remainder is below half an ulp of the value it belongs to, so its 8
// significant bits carry the state to about 2^-33 relative, at half the
// bytes of a float (the other precisions keep their own type, unused).
template <class R> struct RemOf { using T = R; };
template <> struct RemOf<float> { using T = __nv_bfloat16; };
template <class R> using Rem = typename RemOf<R>::T;
template <class R> __device__ __forceinline__ R rem_ld(const Rem<R>* p) { return (R)*p; }
template <> __device__ __forceinline__ float rem_ld<float>(const __nv_bfloat16* p) { return __bfloat162float(*p); }
template <class R> __device__ __forceinline__ void rem_st(Rem<R>* p, R v) { *p = v; }
template <> __device__ __forceinline__ void rem_st<float>(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }

__device__ __forceinline__ double d_log(double x) { return log(x); }
__device__ __forceinline__ float d_log(float x) { return logf(x); }
__device__ __forceinline__ double d_exp(double x) { return exp(x); }
__device__ __forceinline__ float d_exp(float x) { return expf(x); }
__device__ __forceinline__ double d_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float d_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double d_fmax(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ float d_fmax(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double d_fmin(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ float d_fmin(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ double d_fabs(double a) { return fabs(a); }
__device__ __forceinline__ float d_fabs(float a) { return fabsf(a); }

// Double -> int conversion as x86-64 performs it for the reference's (int)
// casts: out-of-range and NaN give INT_MIN.
__device__ __forceinline__ int cvt_x86(double x) {
  return (x >= -2147483648.0 && x < 2147483648.0) ? (int)x : (int)0x80000000;
}

__device__ __forceinline__ bool bad_pos(double a) { return (a != a) || (a <= 0.) || (a == (double)INFINITY); }

__device__ __forceinline__ long long cidx(const Geom& g, int i, int j, int k) {
  return (long long)i + (long long)g.sx * ((long long)j + (long long)g.sy * (long long)k);
}

// 32-bit cell offset for the hot kernels (8*N < 2^32 is enforced at context creation).
__device__ __forceinline__ unsigned cidx32(const Geom& g, int i, int j, int k) {
  return (unsigned)i + (unsigned)g.sx * ((unsigned)j + (unsigned)g.sy * (unsigned)k);
}

// (i, j, k) of interior cell t (x fastest) and of box node id, in 32-bit
// arithmetic (8 N < 2^32 for every context, so both fit).
__device__ __forceinline__ void interior_ijk(const Geom& g, unsigned t, int& i, int& j, int& k) {
  const unsigned nx = (unsigned)g.nx, ny = (unsigned)g.ny;
  const unsigned q = t / nx;
  i = GH + (int)(t - q * nx);
  j = GH + (int)(q % ny);
  k = GH + (int)(q / ny);
}
__device__ __forceinline__ void node_ijk(const Geom& g, unsigned id, int& i, int& j, int& k) {
  const unsigned sx = (unsigned)g.sx, sy = (unsigned)g.sy;
  const unsigned q = id / sx;
  i = (int)(id - q * sx);
  j = (int)(q % sy);
  k = (int)(q / sy);
}
// Grid-stride loop bounds in 32 bits.
__device__ __forceinline__ unsigned gs_first() { return blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ unsigned gs_step() { return gridDim.x * blockDim.x; }

// Order-preserving bits for non-negative doubles (cmax, maxima); NaN never stored.
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* dst, double v) {
  if (v == v && v > 0.0) atomicMax(dst, (unsigned long long)__double_as_longlong(v));
}

template <class R>
__device__ __forceinline__ R warp_max_nonnan(R v) {
  // NaN-ignoring maximum across the warp (values >= 0)
  for (int o = 16; o > 0; o >>= 1) {
    R w = __shfl_xor_sync(0xffffffffu, v, o);
    v = (v < w) ? w : v;   // NaN in w is never taken; NaN in v is replaced by any w
    if (v != v) v = w;
  }
  return v;
}

// NaN-ignoring maximum over the block (values >= 0), valid in thread 0;
// every thread of the block calls it.
template <class R>
__device__ __forceinline__ R block_max_nonnan(R v) {
  __shared__ R sw[32];
  v = warp_max_nonnan(v);
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
  if ((tid & 31) == 0) sw[tid >> 5] = v;
  __syncthreads();
  if (tid < 32) v = warp_max_nonnan(tid < nw ? sw[tid] : (R)0);
  return v;
}

// ------------------------------------------------------------------- EOS
struct C2POut {
  double pres, temp, ne, rhoi, amb;
};

// Full ConsToPrim arithmetic for one cell given primitives (src/cons_to_prim.C:148-243).
__device__ inline C2POut c2p_eos_full(const Consts& c, double d, double ei, double dn) {
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
  double out[6];
#pragma unroll
  for (int t = 0; t < 6; t++) {
    if (t == 2) { out[t] = 0.0; continue; }
    const float* T = c.tab[t];
    double s = c0 * (double)T[a11];
    s += c1 * (double)T[a10];
    s += c2 * (double)T[a01];
    s += c3 * (double)T[a00];
    out[t] = exp(s);
  }
  double pr = out[0], tm = out[1], nl = out[3];
  if (lgr < c.xlr0) {
    pr = c.c_pres * ei;
    tm = c.c_temp * eps;
    nl = pr / (tm * c.kb) - d / c.mun_mh;
  }
  if (eps > 0.8 * c.eps_max) {
    double xx = smax(0.0, 5.0 * (c.eps_max - eps) / c.eps_max);
    pr = pr * xx + (1.0 - xx) * c.c_pres * ei;
    tm = tm * xx + (1.0 - xx) * c.c_temp * eps;
    nl = pr / (tm * c.kb) - d / c.mun_mh;
  }
  if (bad_pos(pr) || bad_pos(tm)) {
    pr = c.c_pres * ei;
    tm = c.c_temp * eps;
  }
  if (nl == (double)INFINITY) nl = pr / (tm * c.kb) - d / c.mun_mh;
  if ((nl < 1.0) || (nl != nl) || (nl == (double)INFINITY)) nl = 1.0;
  C2POut o;
  o.pres = pr; o.temp = tm; o.ne = nl; o.rhoi = out[4]; o.amb = out[5];
  return o;
}

// Pressure only, FP64.  Inside the table (and away from the high-eps blend)
// none of ConsToPrim's fallbacks can fire, so the result is exp() of the
// bilinear sum; elsewhere the full routine decides.
__device__ __forceinline__ double eos_pres(const Consts& c, double d, double ei, double dn) {
  const double eps = ei * dn + c.eps_off;
  const double lgr = log(d);
  const double ep = log(eps);
  if (!(lgr >= c.xlr0 && lgr < c.xlrN + 1.0 && ep > c.xeps0 - 1.0 && ep < c.xepsN + 1.0 &&
        !(eps > 0.8 * c.eps_max)))
    return c2p_eos_full(c, d, ei, dn).pres;
  const double lr = lgr;
  int i_d = (int)((lr - c.xlr0) * c.inv_del_lr);
  i_d = max(0, i_d);
  i_d = min(c.N_lr - 2, i_d);
  int i_e = (int)((ep - c.xeps0) * c.inv_del_eps);
  i_e = max(0, i_e);
  i_e = min(c.N_eps - 2, i_e);
  const double xe0 = __ldg(c.xeps + i_e), xe1 = __ldg(c.xeps + i_e + 1);
  const double xr0 = __ldg(c.xlr + i_d), xr1 = __ldg(c.xlr + i_d + 1);
  const double c0 = (ep - xe0) * (lr - xr0);
  const double c1 = (ep - xe0) * (xr1 - lr);
  const double c2 = (xe1 - ep) * (lr - xr0);
  const double c3 = (xe1 - ep) * (xr1 - lr);
  const float* T = c.tab[0];
  const long long r1 = (long long)(i_e + 1) * c.N_lr + i_d;
  const long long r0 = (long long)i_e * c.N_lr + i_d;
  double s = c0 * (double)__ldg(T + r1 + 1);
  s += c1 * (double)__ldg(T + r1);
  s += c2 * (double)__ldg(T + r0 + 1);
  s += c3 * (double)__ldg(T + r0);
  return exp(s);
}

// ln(1+t) and exp(d) for the small arguments of the FP32 pressure patch:
// truncated Taylor series (errors below 1e-9 for |t| <= 0.03, |d| <= 0.1),
// the library functions outside that range.
__device__ __forceinline__ float log1p_small(float t) {
  if (fabsf(t) > 0.03f) return logf(1.0f + t);
  return t * (1.0f + t * (-0.5f + t * (0.33333334f + t * (-0.25f + t * 0.2f))));
}
__device__ __forceinline__ float exp_small(float d) {
  if (fabsf(d) > 0.1f) return expf(d);
  return 1.0f + d * (1.0f + d * (0.5f + d * (0.16666667f + d * (0.041666668f + d * (0.008333334f + d * 0.0013888889f)))));
}

// Pressure only, FP32.  The bilinear patch of ln p is re-expanded around its
// lower corner, p = P00 * exp(fe*a + fr*b + fe*fr*c), with the offsets
// fe = ln(eps) - xeps[i] and fr = ln(rho) - xlr[j] taken as ln of ratios near
// one; this keeps ~1e-7 relative accuracy where the direct float sum of the
// pre-divided table terms would lose ~1e-6.  The cell index only needs the
// hardware log2: an index off by one at a cell edge selects the neighbouring
// patch, which agrees there to the table's rounding.
__device__ __forceinline__ float eos_pres(const Consts& c, float d, float ei, float dn) {
  constexpr float LN2 = 0.69314718f;
  const KC<float>& k = c.kf;
  const float eps = ei * dn + k.eps_off;
  const float lgr = __log2f(d) * LN2;
  const float ep = __log2f(eps) * LN2;
  if (!(lgr >= k.xlr0 + 0.01f && lgr < k.xlrN + 1.0f && ep > k.xeps0 - 1.0f && ep < k.xepsN + 1.0f &&
        !(eps > 0.8f * k.eps_max)))
    return (float)c2p_eos_full(c, (double)d, (double)ei, 1.0 / (double)d).pres;
  int i_d = (int)((lgr - k.xlr0) * k.inv_del_lr);
  i_d = max(0, min(c.N_lr - 2, i_d));
  int i_e = (int)((ep - k.xeps0) * k.inv_del_eps);
  i_e = max(0, min(c.N_eps - 2, i_e));
  const float fe = log1p_small(eps * __ldg(c.inv_exp_xeps + i_e) - 1.0f);
  const float fr = log1p_small(d * __ldg(c.inv_exp_xlr + i_d) - 1.0f);
  const float4 q = __ldg(c.pquad + (long long)i_e * c.N_lr + i_d);
  return q.x * exp_small(fe * q.y + fr * q.z + fe * fr * q.w);
}

// All ConsToPrim outputs in FP32 (src/cons_to_prim.C:148-243): the pressure
// from eos_pres; temperature, n_e, rho_i and the ambipolar coefficient as
// exp of float bilinear sums whose weights are the offsets from the cell's
// corners taken as ln of ratios near one (table values are pre-divided by
// the cell area, so the weights must be formed to float accuracy); outside
// the table or in the high-eps blend the FP64 routine decides.
__device__ inline void c2p_outputs(const Consts& c, float d, float ei, float dn, float& pr, float& tm, float& ne,
                                   float& ri, float& am) {
  constexpr float LN2 = 0.69314718f;
  const KC<float>& k = c.kf;
  const float eps = ei * dn + k.eps_off;
  const float lgr = __log2f(d) * LN2;
  const float ep = __log2f(eps) * LN2;
  if (!(lgr >= k.xlr0 + 0.01f && lgr < k.xlrN + 1.0f && ep > k.xeps0 - 1.0f && ep < k.xepsN + 1.0f &&
        !(eps > 0.8f * k.eps_max))) {
    const C2POut o = c2p_eos_full(c, (double)d, (double)ei, 1.0 / (double)d);
    pr = (float)o.pres; tm = (float)o.temp; ne = (float)o.ne; ri = (float)o.rhoi; am = (float)o.amb;
    return;
  }
  int i_d = (int)((lgr - k.xlr0) * k.inv_del_lr);
  i_d = max(0, min(c.N_lr - 2, i_d));
  int i_e = (int)((ep - k.xeps0) * k.inv_del_eps);
  i_e = max(0, min(c.N_eps - 2, i_e));
  const float fe = log1p_small(eps * __ldg(c.inv_exp_xeps + i_e) - 1.0f);
  const float fr = log1p_small(d * __ldg(c.inv_exp_xlr + i_d) - 1.0f);
  const float ge = k.del_eps - fe, gr = k.del_lr - fr;
  const long long r1 = (long long)(i_e + 1) * c.N_lr + i_d;
  const long long r0 = (long long)i_e * c.N_lr + i_d;
  auto look = [&](int t) {
    const float* T = c.tab[t];
    return expf(fe * fr * __ldg(T + r1 + 1) + fe * gr * __ldg(T + r1) + ge * fr * __ldg(T + r0 + 1) +
                ge * gr * __ldg(T + r0));
  };
  pr = eos_pres(c, d, ei, dn);
  tm = look(1);
  ne = look(3);
  ri = look(4);
  am = look(5);
  const float inf = __int_as_float(0x7f800000);
  if (!(pr > 0.0f && pr < inf) || !(tm > 0.0f && tm < inf)) {
    pr = (float)(c.c_pres * (double)ei);
    tm = (float)(c.c_temp * (double)eps);
  }
  if (!(ne >= 1.0f) || ne == inf) ne = 1.0f;
}
__device__ inline void c2p_outputs(const Consts& c, double d, double ei, double dn, double& pr, double& tm, double& ne,
                                   double& ri, double& am) {
  const C2POut o = c2p_eos_full(c, d, ei, dn);
  pr = o.pres; tm = o.temp; ne = o.ne; ri = o.rhoi; am = o.amb;
}

// The pressure lookup split in two, so that a kernel can issue the table
// loads of one cell and finish the value later (after other work): begin()
// computes the cell index and starts the loads, end() returns eos_pres's
// value.  Outside the fast path (and in FP64) begin() computes it at once.
template <class R>
struct PresLookup {
  float4 q;
  float ix, id, eps, d;
  R done;
  int ready;
};

__device__ __forceinline__ void eos_pres_begin(const Consts& c, double d, double ei, double dn, PresLookup<double>& L) {
  L.done = eos_pres(c, d, ei, dn);
  L.ready = 1;
}
__device__ __forceinline__ double eos_pres_end(const PresLookup<double>& L) { return L.done; }

__device__ __forceinline__ void eos_pres_begin(const Consts& c, float d, float ei, float dn, PresLookup<float>& L) {
  constexpr float LN2 = 0.69314718f;
  const KC<float>& k = c.kf;
  const float eps = ei * dn + k.eps_off;
  const float lgr = __log2f(d) * LN2;
  const float ep = __log2f(eps) * LN2;
  if (!(lgr >= k.xlr0 + 0.01f && lgr < k.xlrN + 1.0f && ep > k.xeps0 - 1.0f && ep < k.xepsN + 1.0f &&
        !(eps > 0.8f * k.eps_max))) {
    L.done = (float)c2p_eos_full(c, (double)d, (double)ei, 1.0 / (double)d).pres;
    L.ready = 1;
    return;
  }
  int i_d = (int)((lgr - k.xlr0) * k.inv_del_lr);
  i_d = max(0, min(c.N_lr - 2, i_d));
  int i_e = (int)((ep - k.xeps0) * k.inv_del_eps);
  i_e = max(0, min(c.N_eps - 2, i_e));
  L.ix = __ldg(c.inv_exp_xeps + i_e);
  L.id = __ldg(c.inv_exp_xlr + i_d);
  L.q = __ldg(c.pquad + (long long)i_e * c.N_lr + i_d);
  L.eps = eps;
  L.d = d;
  L.ready = 0;
}
__device__ __forceinline__ float eos_pres_end(const PresLookup<float>& L) {
  if (L.ready) return L.done;
  const float fe = log1p_small(L.eps * L.ix - 1.0f);
  const float fr = log1p_small(L.d * L.id - 1.0f);
  return L.q.x * exp_small(fe * L.q.y + fr * L.q.z + fe * fr * L.q.w);
}

// ------------------------------------------------------------ Tcheck cell
// src/Add_Sources_Integrate_SR.C:444-465 and :600-617
template <class R>
__device__ __forceinline__ void tcheck_cell(const Consts& c, R vmax, R eps_max, R& d, R& m1, R& m2, R& m3, R& e) {
  const R rho_min = kc<R>(c).rho_min, eps_min = kc<R>(c).eps_min;
  R dn = d_fmax(rho_min, d);
  R vv = d_sqrt(m1 * m1 + m2 * m2 + m3 * m3) / dn;
  R s = vmax / d_fmax(vmax, vv);
  R ekin = (R)0.5 * dn * vv * vv;
  R lo = eps_min * dn + ekin * s * s;
  R up = eps_max * dn + ekin * s * s;
  e = d_fmin(d_fmax(e, lo), up);
  d = dn;
  m1 *= s;
  m2 *= s;
  m3 *= s;
}

// Characteristic speed of MHD_Residual's CFL condition (src/mhdres_SR.C:310-328)
template <class R>
__device__ __forceinline__ R cmax_cell(R d, R v1, R v2, R v3, R b1, R b2, R b3, R p, R inv_va2max) {
  R dn = (R)1.0 / d;
  R vv = v1 * v1 + v2 * v2 + v3 * v3;
  R bb = b1 * b1 + b2 * b2 + b3 * b3;
  R va2 = bb * dn;
  R x2 = va2 * inv_va2max, x4 = x2 * x2, s = (R)1.0 + x2;
  R lf = s / (s + x4);
  R cs2 = (R)(5.0 / 3.0) * p * dn;
  vv = d_sqrt(vv);
  return vv + (R)0.0 + d_sqrt(smax(cs2, lf * (cs2 + va2)));
}

}  // namespace gpumhd
