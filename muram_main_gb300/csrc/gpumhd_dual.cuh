// Forward-mode dual numbers for the adjoint's local Jacobians.
//
// Dual<K> carries a value and K directional derivatives.  The cell-local
// functions of the forward step (primitives, fluxes, residual assembly,
// sources, Tcheck, the TVD cell / slope / flux / update, the EOS pressure) are
// templates on their arithmetic type; instantiated with Dual they return the
// derivative of each output along the seeded input directions.  Comparisons
// and min / max act on values, so a limiter kink or a clamp contributes the
// derivative of the branch it takes (a one-sided subgradient).
#pragma once
#include "gpumhd_dev.cuh"

namespace gpumhd {

template <int K>
struct Dual {
  double v;
  double d[K];
  __device__ __forceinline__ Dual() {}
  __device__ __forceinline__ Dual(double x) : v(x) {
#pragma unroll
    for (int k = 0; k < K; k++) d[k] = 0.0;
  }
};

template <int K> struct KCSel<Dual<K>> {
  using T = KC<double>;
  static __device__ __forceinline__ const T& get(const Consts& c) { return c.kd; }
};

__device__ __forceinline__ double val(double x) { return x; }
__device__ __forceinline__ float val(float x) { return x; }
template <int K> __device__ __forceinline__ double val(const Dual<K>& x) { return x.v; }

#define GPUMHD_DUAL_BINOP(OP, VAL, DER)                                                        \
  template <int K>                                                                             \
  __device__ __forceinline__ Dual<K> operator OP(const Dual<K>& a, const Dual<K>& b) {        \
    Dual<K> r;                                                                                 \
    r.v = VAL;                                                                                 \
    _Pragma("unroll") for (int k = 0; k < K; k++) r.d[k] = DER;                                \
    return r;                                                                                  \
  }                                                                                            \
  template <int K>                                                                             \
  __device__ __forceinline__ Dual<K> operator OP(const Dual<K>& a, double bv) {               \
    return a OP Dual<K>(bv);                                                                   \
  }                                                                                            \
  template <int K>                                                                             \
  __device__ __forceinline__ Dual<K> operator OP(double av, const Dual<K>& b) {               \
    return Dual<K>(av) OP b;                                                                   \
  }

GPUMHD_DUAL_BINOP(+, a.v + b.v, a.d[k] + b.d[k])
GPUMHD_DUAL_BINOP(-, a.v - b.v, a.d[k] - b.d[k])
GPUMHD_DUAL_BINOP(*, a.v * b.v, a.d[k] * b.v + a.v * b.d[k])
GPUMHD_DUAL_BINOP(/, a.v / b.v, (a.d[k] * b.v - a.v * b.d[k]) / (b.v * b.v))
#undef GPUMHD_DUAL_BINOP

template <int K> __device__ __forceinline__ Dual<K> operator-(const Dual<K>& a) {
  Dual<K> r;
  r.v = -a.v;
#pragma unroll
  for (int k = 0; k < K; k++) r.d[k] = -a.d[k];
  return r;
}
template <int K> __device__ __forceinline__ Dual<K>& operator+=(Dual<K>& a, const Dual<K>& b) { return a = a + b; }
template <int K> __device__ __forceinline__ Dual<K>& operator-=(Dual<K>& a, const Dual<K>& b) { return a = a - b; }
template <int K> __device__ __forceinline__ Dual<K>& operator*=(Dual<K>& a, const Dual<K>& b) { return a = a * b; }
template <int K> __device__ __forceinline__ Dual<K>& operator/=(Dual<K>& a, const Dual<K>& b) { return a = a / b; }
template <int K> __device__ __forceinline__ Dual<K>& operator+=(Dual<K>& a, double b) { return a = a + b; }
template <int K> __device__ __forceinline__ Dual<K>& operator-=(Dual<K>& a, double b) { return a = a - b; }
template <int K> __device__ __forceinline__ Dual<K>& operator*=(Dual<K>& a, double b) { return a = a * b; }

#define GPUMHD_DUAL_CMP(OP)                                                                                     \
  template <int K> __device__ __forceinline__ bool operator OP(const Dual<K>& a, const Dual<K>& b) { return a.v OP b.v; } \
  template <int K> __device__ __forceinline__ bool operator OP(const Dual<K>& a, double b) { return a.v OP b; }           \
  template <int K> __device__ __forceinline__ bool operator OP(double a, const Dual<K>& b) { return a OP b.v; }
GPUMHD_DUAL_CMP(<)
GPUMHD_DUAL_CMP(>)
GPUMHD_DUAL_CMP(<=)
GPUMHD_DUAL_CMP(>=)
GPUMHD_DUAL_CMP(==)
GPUMHD_DUAL_CMP(!=)
#undef GPUMHD_DUAL_CMP

template <int K> __device__ __forceinline__ Dual<K> dual_chain(const Dual<K>& a, double fv, double dfdx) {
  Dual<K> r;
  r.v = fv;
#pragma unroll
  for (int k = 0; k < K; k++) r.d[k] = dfdx * a.d[k];
  return r;
}
template <int K> __device__ __forceinline__ Dual<K> d_sqrt(const Dual<K>& a) {
  const double s = sqrt(a.v);
  return dual_chain(a, s, s > 0.0 ? 0.5 / s : 0.0);
}
template <int K> __device__ __forceinline__ Dual<K> d_log(const Dual<K>& a) { return dual_chain(a, log(a.v), 1.0 / a.v); }
template <int K> __device__ __forceinline__ Dual<K> d_exp(const Dual<K>& a) {
  const double e = exp(a.v);
  return dual_chain(a, e, e);
}
template <int K> __device__ __forceinline__ Dual<K> d_fabs(const Dual<K>& a) {
  return dual_chain(a, fabs(a.v), a.v < 0.0 ? -1.0 : 1.0);
}
template <int K> __device__ __forceinline__ Dual<K> d_fmax(const Dual<K>& a, const Dual<K>& b) { return (a.v < b.v) ? b : a; }
template <int K> __device__ __forceinline__ Dual<K> d_fmin(const Dual<K>& a, const Dual<K>& b) { return (b.v < a.v) ? b : a; }
// mixed (constant, dual) arguments of the min / max helpers
template <int K> __device__ __forceinline__ Dual<K> smax(double a, const Dual<K>& b) { return smax(Dual<K>(a), b); }
template <int K> __device__ __forceinline__ Dual<K> smax(const Dual<K>& a, double b) { return smax(a, Dual<K>(b)); }
template <int K> __device__ __forceinline__ Dual<K> smin(double a, const Dual<K>& b) { return smin(Dual<K>(a), b); }
template <int K> __device__ __forceinline__ Dual<K> smin(const Dual<K>& a, double b) { return smin(a, Dual<K>(b)); }
template <int K> __device__ __forceinline__ Dual<K> d_fmax(double a, const Dual<K>& b) { return d_fmax(Dual<K>(a), b); }
template <int K> __device__ __forceinline__ Dual<K> d_fmax(const Dual<K>& a, double b) { return d_fmax(a, Dual<K>(b)); }

// ------------------------------------------------------------- EOS, generic
// ConsToPrim's pressure (src/cons_to_prim.C:148-243) for any arithmetic type:
// the bilinear table sum in (ln eps, ln rho), exp, and the ideal-gas
// fallbacks; the table cell comes from the values.  For double it gives
// c2p_eos_full's pressure.
template <class R>
__device__ __forceinline__ R eos_pres_t(const Consts& c, R d, R ei, R dn) {
  const R eps = ei * dn + c.eps_off;
  const R lgr = d_log(d);
  const R ep = d_log(eps);
  int i_d = cvt_x86((val(lgr) - c.xlr0) * c.inv_del_lr);
  i_d = max(0, min(c.N_lr - 2, i_d));
  int i_e = cvt_x86((val(ep) - c.xeps0) * c.inv_del_eps);
  i_e = max(0, min(c.N_eps - 2, i_e));
  const double xe0 = c.xeps[i_e], xe1 = c.xeps[i_e + 1];
  const double xr0 = c.xlr[i_d], xr1 = c.xlr[i_d + 1];
  const R c0 = (ep - xe0) * (lgr - xr0);
  const R c1 = (ep - xe0) * (xr1 - lgr);
  const R c2 = (xe1 - ep) * (lgr - xr0);
  const R c3 = (xe1 - ep) * (xr1 - lgr);
  const float* T = c.tab[0];
  const long long r1 = (long long)(i_e + 1) * c.N_lr + i_d;
  const long long r0 = (long long)i_e * c.N_lr + i_d;
  R s = c0 * (double)T[r1 + 1];
  s += c1 * (double)T[r1];
  s += c2 * (double)T[r0 + 1];
  s += c3 * (double)T[r0];
  R pr = d_exp(s);
  if (val(lgr) < c.xlr0) pr = c.c_pres * ei;
  if (val(eps) > 0.8 * c.eps_max) {
    const double xx = smax(0.0, 5.0 * (c.eps_max - val(eps)) / c.eps_max);
    const R xr = 5.0 * (c.eps_max - eps) / c.eps_max;
    const R xd = (xx > 0.0) ? xr : R(0.0);
    pr = pr * xd + (1.0 - xd) * c.c_pres * ei;
  }
  if (bad_pos(val(pr))) pr = c.c_pres * ei;
  return pr;
}

}  // namespace gpumhd
