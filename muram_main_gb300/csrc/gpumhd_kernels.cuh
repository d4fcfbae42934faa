// Kernels of the MURaM MHD time step (templated on the state type R).
//
//  k_stage      one RK stage: residual (MHD_Residual), sources, Boris
//               correction, update and Tcheck (Source_Integrate_Tcheck), and
//               the next stage's pressure (ConsToPrim), in one pass; or, in
//               residual mode, MHD_Residual alone (Res += residual).
//  k_tvd_sweep  one directional TVDlimit sweep; the last sweep of a step
//               also applies TCheck, the ghost fill and the next step's
//               pressure, CFL speed and Adjust_Valf_Max statistics.
//  small kernels: ConsToPrim, Adjust_Valf_Max statistics, Source_Integrate,
//               SaveCons, TCheck, ghost fill, layout conversion, step control.
#pragma once
#include <type_traits>

#include "gpumhd_dev.cuh"

namespace gpumhd {

// ----------------------------------------------------------- ghost images
// Every interior cell within two cells of a face has a ghost image across it:
// periodic dimensions copy, the closed x dimension mirrors (M_x, B_y, B_z
// change sign).  xmirror = 0 restricts the images to the periodic dimensions
// (the exchange between TVD half steps does not apply the x boundary rule).
struct Images {
  int xa, ya, za;   // index of the image across x / y / z, -1 if none
  int xf;           // the x image is a mirror (sign flips)
};

__device__ __forceinline__ Images images_of(const Geom& g, int i, int j, int k, bool xmirror) {
  Images im;
  im.xa = -1; im.ya = -1; im.za = -1; im.xf = 0;
  const int I = i - GH, J = j - GH, K = k - GH;
  if (g.periodic_x) {
    if (I < GH) im.xa = i + g.nx;
    else if (I >= g.nx - GH) im.xa = i - g.nx;
  } else if (xmirror && g.xmirror) {
    if (I < GH) { im.xa = 2 * GH - 1 - i; im.xf = 1; }
    else if (I >= g.nx - GH) { im.xa = 2 * GH + 2 * g.nx - 1 - i; im.xf = 1; }
  }
  if (J < GH) im.ya = j + g.ny;
  else if (J >= g.ny - GH) im.ya = j - g.ny;
  if (K < GH) im.za = k + g.nz;
  else if (K >= g.nz - GH) im.za = k - g.nz;
  return im;
}

// Calls f(index, mirrored) for the cell itself and each of its ghost images.
// IDX32: 32-bit offsets (the stage kernel) or 64-bit (the TVD sweeps, where
// the 64-bit form compiles to fewer registers).
template <bool IDX32, class F>
__device__ __forceinline__ void for_images(const Geom& g, int i, int j, int k, const Images& im, F f) {
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const int kk = c ? im.za : k;
    if (kk < 0) continue;
#pragma unroll
    for (int b = 0; b < 2; b++) {
      const int jj = b ? im.ya : j;
      if (jj < 0) continue;
#pragma unroll
      for (int a = 0; a < 2; a++) {
        const int ii = a ? im.xa : i;
        if (ii < 0) continue;
        if (IDX32) f((unsigned long long)cidx32(g, ii, jj, kk), a && im.xf);
        else f((unsigned long long)cidx(g, ii, jj, kk), a && im.xf);
      }
    }
  }
}

// The ghost images of the cells of one (i, j) column as 32-bit index offsets:
// the x and y parts (0: none) are fixed along the column, the z part depends
// on the plane only (uniform over a block that shares k).  Writes the same
// (index, mirrored) set as images_of / for_images.
struct ColImg {
  int ox, oy;  // offsets of the x and y images
  int xf;      // the x image is a mirror (sign flips)
};
__device__ __forceinline__ ColImg col_images(const Geom& g, int i, int j, bool xmirror) {
  ColImg ci;
  ci.ox = 0; ci.oy = 0; ci.xf = 0;
  const int I = i - GH, J = j - GH;
  if (g.periodic_x) {
    if (I < GH) ci.ox = g.nx;
    else if (I >= g.nx - GH) ci.ox = -g.nx;
  } else if (xmirror && g.xmirror) {
    if (I < GH) { ci.ox = 2 * GH - 1 - 2 * i; ci.xf = 1; }
    else if (I >= g.nx - GH) { ci.ox = 2 * GH + 2 * g.nx - 1 - 2 * i; ci.xf = 1; }
  }
  if (J < GH) ci.oy = g.ny * g.sx;
  else if (J >= g.ny - GH) ci.oy = -g.ny * g.sx;
  return ci;
}
__device__ __forceinline__ int z_image_off(const Geom& g, int k) {
  const int K = k - GH;
  const int pl = g.sx * g.sy;
  return K < GH ? g.nz * pl : (K >= g.nz - GH ? -g.nz * pl : 0);
}
// f(index, mirrored) for the cell id and each of its images.
template <class F>
__device__ __forceinline__ void for_col_images(unsigned id, const ColImg& ci, int oz, F f) {
  f(id, false);
  if (ci.ox) f(id + (unsigned)ci.ox, ci.xf != 0);
  if (ci.oy) {
    f(id + (unsigned)ci.oy, false);
    if (ci.ox) f(id + (unsigned)(ci.oy + ci.ox), ci.xf != 0);
  }
  if (oz) {
    f(id + (unsigned)oz, false);
    if (ci.ox) f(id + (unsigned)(oz + ci.ox), ci.xf != 0);
    if (ci.oy) {
      f(id + (unsigned)(oz + ci.oy), false);
      if (ci.ox) f(id + (unsigned)(oz + ci.oy + ci.ox), ci.xf != 0);
    }
  }
}
template <class R>
__device__ __forceinline__ void store_state_col(const Geom& g, R* __restrict__ U, unsigned id, const ColImg& ci, int oz,
                                                const R v[NV]) {
  for_col_images(id, ci, oz, [&](unsigned t, bool f) {
#pragma unroll
    for (int q = 0; q < NV; q++) {
      R x = v[q];
      if (f && (q == 1 || q == 6 || q == 7)) x = -x;
      U[t + (unsigned)q * g.N32] = x;
    }
  });
}

template <class R, bool IDX32 = false>
__device__ __forceinline__ void store_state(const Geom& g, R* __restrict__ U, int i, int j, int k, const Images& im,
                                            const R v[NV]) {
  for_images<IDX32>(g, i, j, k, im, [&](unsigned long long id, bool f) {
#pragma unroll
    for (int q = 0; q < NV; q++) {
      R x = v[q];
      if (f && (q == 1 || q == 6 || q == 7)) x = -x;
      if (IDX32) U[(unsigned)id + (unsigned)q * g.N32] = x;
      else U[(long long)q * g.N + (long long)id] = x;
    }
  });
}

template <class R, bool IDX32 = false>
__device__ __forceinline__ void store_scalar(const Geom& g, R* __restrict__ P, int i, int j, int k, const Images& im,
                                             R v) {
  for_images<IDX32>(g, i, j, k, im, [&](unsigned long long id, bool) { P[id] = v; });
}

// -------------------------------------------------------------- primitives
// 11 per-cell values the residual's fluxes need.
enum { P_D, P_V1, P_V2, P_V3, P_EI, P_B1, P_B2, P_B3, P_P, P_EK, P_PM, NPRIM };

// From conserved variables as ConsToPrim forms them (src/cons_to_prim.C:148-159),
// then the residual's kinetic and magnetic pressure terms (src/mhdres_SR.C:310-317).
template <class R>
__device__ __forceinline__ void prim_from_cons(R d, R m1, R m2, R m3, R e, R& v1, R& v2, R& v3, R& ei) {
  R dn = (R)1.0 / d;
  v1 = m1 * dn;
  v2 = m2 * dn;
  v3 = m3 * dn;
  R vv = v1 * v1 + v2 * v2 + v3 * v3;
  ei = e - (R)0.5 * vv * d;
}

// The 9 stored values of a cell (state and pressure), as loaded from memory.
template <class R>
struct Raw9 {
  R v[9];
};

template <class R>
__device__ __forceinline__ void load_raw(const Geom& g, const R* __restrict__ U, const R* __restrict__ P, unsigned id,
                                         Raw9<R>& r) {
#pragma unroll
  for (int q = 0; q < NV; q++) r.v[q] = U[id + (unsigned)q * g.N32];
  r.v[8] = P[id];
}

template <class R>
__device__ __forceinline__ void load_raw64(const Geom& g, const R* __restrict__ U, const R* __restrict__ P, long long id,
                                           Raw9<R>& r) {
#pragma unroll
  for (int q = 0; q < NV; q++) r.v[q] = U[(long long)q * g.N + id];
  r.v[8] = P[id];
}

__device__ __forceinline__ void fill_raw_one(Raw9<float>& r) {
#pragma unroll
  for (int q = 0; q < 9; q++) r.v[q] = 1.0f;
}
__device__ __forceinline__ void fill_raw_one(Raw9<double>& r) {
#pragma unroll
  for (int q = 0; q < 9; q++) r.v[q] = 1.0;
}

template <class R, bool PRIM_IN>
__device__ __forceinline__ void prim_of_raw(const Raw9<R>& r, R* out) {
  R d = r.v[0];
  R a1 = r.v[1], a2 = r.v[2], a3 = r.v[3], a4 = r.v[4];
  R b1 = r.v[5], b2 = r.v[6], b3 = r.v[7];
  R v1, v2, v3, ei;
  if (PRIM_IN) { v1 = a1; v2 = a2; v3 = a3; ei = a4; }
  else prim_from_cons(d, a1, a2, a3, a4, v1, v2, v3, ei);
  R vv = v1 * v1 + v2 * v2 + v3 * v3;
  R bb = b1 * b1 + b2 * b2 + b3 * b3;
  out[P_D] = d;
  out[P_V1] = v1;
  out[P_V2] = v2;
  out[P_V3] = v3;
  out[P_EI] = ei;
  out[P_B1] = b1;
  out[P_B2] = b2;
  out[P_B3] = b3;
  out[P_P] = r.v[8];
  out[P_EK] = (R)0.5 * d * vv;
  out[P_PM] = (R)0.5 * bb;
}

// The 12 directional quantities whose 4th-order derivative the residual takes
// along D1 (src/mhdres_SR.C:330-347): F0..F4, the two induction fluxes other
// than component D1 (which is identically zero), the Maxwell stress (3), and
// B along the two other directions (for curl B x B).
template <int D1> struct Dirs;
template <> struct Dirs<0> { static constexpr int d2 = 1, d3 = 2, fa = 6, fb = 7; };
template <> struct Dirs<1> { static constexpr int d2 = 0, d3 = 2, fa = 5, fb = 7; };
template <> struct Dirs<2> { static constexpr int d2 = 0, d3 = 1, fa = 5, fb = 6; };
constexpr int NF = 12;

template <class R, int D1>
__device__ __forceinline__ void flux12(const R* p, int s, R* f, int fs) {
  const R d = p[P_D * s], v1 = p[P_V1 * s], v2 = p[P_V2 * s], v3 = p[P_V3 * s];
  const R ei = p[P_EI * s], b1 = p[P_B1 * s], b2 = p[P_B2 * s], b3 = p[P_B3 * s];
  const R pr = p[P_P * s], ekin = p[P_EK * s], pmag = p[P_PM * s];
  const R vel = D1 == 0 ? v1 : (D1 == 1 ? v2 : v3);
  const R mag = D1 == 0 ? b1 : (D1 == 1 ? b2 : b3);
  const R p1 = D1 == 0 ? (R)1.0 : (R)0.0, p2 = D1 == 1 ? (R)1.0 : (R)0.0, p3 = D1 == 2 ? (R)1.0 : (R)0.0;
  const R mflx = vel * d;
  f[0 * fs] = mflx;
  f[1 * fs] = mflx * v1 + p1 * pr;
  f[2 * fs] = mflx * v2 + p2 * pr;
  f[3 * fs] = mflx * v3 + p3 * pr;
  f[4 * fs] = vel * (ei + ekin + pr);
  const R F5 = vel * b1 - v1 * mag, F6 = vel * b2 - v2 * mag, F7 = vel * b3 - v3 * mag;
  f[5 * fs] = Dirs<D1>::fa == 5 ? F5 : F6;
  f[6 * fs] = Dirs<D1>::fb == 7 ? F7 : F6;
  f[7 * fs] = mag * b1 - p1 * pmag;
  f[8 * fs] = mag * b2 - p2 * pmag;
  f[9 * fs] = mag * b3 - p3 * pmag;
  f[10 * fs] = Dirs<D1>::d2 == 0 ? b1 : b2;
  f[11 * fs] = Dirs<D1>::d3 == 1 ? b2 : b3;
}

// One direction's contribution (src/mhdres_SR.C:361-412) added to R in place:
// res = 0 - D(F); res[1..3] += Lorentz; res[4] += v . Lorentz; R += res.
// fm2..fp2 point at the 12 consecutive quantities of cells c-2, c-1, c+1, c+2.
__device__ __forceinline__ void deriv12(double* Dq, const double* fm2, const double* fm1, const double* fp1,
                                        const double* fp2, double w1, double w2) {
#pragma unroll
  for (int q = 0; q < NF; q++) Dq[q] = w1 * (fp1[q] - fm1[q]) + w2 * (fp2[q] - fm2[q]);
}
__device__ __forceinline__ void deriv12(float* Dq, const float* fm2, const float* fm1, const float* fp1,
                                        const float* fp2, float w1, float w2) {
  const float2 neg = make_float2(-1.0f, -1.0f), W1 = make_float2(w1, w1), W2 = make_float2(w2, w2);
#pragma unroll
  for (int q = 0; q < NF; q += 2) {
    const float2 d1 = __ffma2_rn(make_float2(fm1[q], fm1[q + 1]), neg, make_float2(fp1[q], fp1[q + 1]));
    const float2 d2 = __ffma2_rn(make_float2(fm2[q], fm2[q + 1]), neg, make_float2(fp2[q], fp2[q + 1]));
    const float2 r = __ffma2_rn(W1, d1, __fmul2_rn(W2, d2));
    Dq[q] = r.x;
    Dq[q + 1] = r.y;
  }
}

// Residual terms of one direction from its derivatives Dq (src/mhdres_SR.C:
// 373-412), added to Racc: res = 0 - D(F); res[1..3] += Lorentz; res[4] +=
// v . Lorentz; Racc += res.  ETA (resistivity, src/mhdres_SR.C:422-450,
// 741-765): the direction's curl B parts accumulate in cb; the last direction
// (z) adds the ohmic heating eta*|cb|^2 to Racc[4] before its residual; lap3
// is eta times the fourth-order second derivative of B along the direction.
template <class R, int D1, bool ETA = false>
__device__ __forceinline__ void apply_direction(R* Racc, const R* Dq, const R* cen, R lf, R eta = (R)0,
                                                R* cb = nullptr, const R* lap3 = nullptr) {
  R res[NV];
  res[0] = (R)0.0 - Dq[0];
  res[1] = (R)0.0 - Dq[1];
  res[2] = (R)0.0 - Dq[2];
  res[3] = (R)0.0 - Dq[3];
  res[4] = (R)0.0 - Dq[4];
  res[5] = (R)0.0;
  res[6] = (R)0.0;
  res[7] = (R)0.0;
  res[Dirs<D1>::fa] = (R)0.0 - Dq[5];
  res[Dirs<D1>::fb] = (R)0.0 - Dq[6];
  const R dB2 = Dq[10], dB3 = Dq[11];
  const R Bd1 = cen[P_B1 + D1];
  const R Bd2 = cen[P_B1 + Dirs<D1>::d2], Bd3 = cen[P_B1 + Dirs<D1>::d3];
  R cbb[3];
  cbb[D1] = -Bd2 * dB2 - Bd3 * dB3;
  cbb[Dirs<D1>::d2] = Bd1 * dB2;
  cbb[Dirs<D1>::d3] = Bd1 * dB3;
  const R lrt0 = lf * Dq[7] + ((R)1.0 - lf) * cbb[0];
  const R lrt1 = lf * Dq[8] + ((R)1.0 - lf) * cbb[1];
  const R lrt2 = lf * Dq[9] + ((R)1.0 - lf) * cbb[2];
  res[1] += lrt0;
  res[2] += lrt1;
  res[3] += lrt2;
  res[4] += cen[P_V1] * lrt0 + cen[P_V2] * lrt1 + cen[P_V3] * lrt2;
  if (ETA) {
    const R signd1 = D1 == 1 ? (R)1.0 : (R)-1.0;
    cb[Dirs<D1>::d2] += signd1 * dB3;
    cb[Dirs<D1>::d3] += -signd1 * dB2;
    if (D1 == 2) Racc[4] += eta * (cb[0] * cb[0] + cb[1] * cb[1] + cb[2] * cb[2]);
    res[5] += lap3[0];
    res[6] += lap3[1];
    res[7] += lap3[2];
  }
#pragma unroll
  for (int q = 0; q < NV; q++) Racc[q] += res[q];
}

// eta times the fourth-order second derivative of B along a direction of
// stride sd at cell id (src/mhdres_SR.C:441-450); cen: the cell's primitives.
template <class R>
__device__ __forceinline__ void eta_lap(const Consts& c, const R* __restrict__ U, unsigned id, unsigned sd, int d,
                                        const R* cen, R* lap3) {
  const auto& k = kc<R>(c);
#pragma unroll
  for (int q = 0; q < 3; q++) {
    const R* B = U + (unsigned)(5 + q) * c.g.N32;
    const R bp1 = B[id + sd], bm1 = B[id - sd], bp2 = B[id + 2 * sd], bm2 = B[id - 2 * sd];
    lap3[q] = k.eta * (k.ww0[d] * cen[P_B1 + q] + k.ww1[d] * (bp1 + bm1) + k.ww2[d] * (bp2 + bm2));
  }
}

template <class R, int D1, bool ETA = false>
__device__ __forceinline__ void add_direction(R* Racc, const R* __restrict__ fm2, const R* __restrict__ fm1,
                                              const R* __restrict__ fp1, const R* __restrict__ fp2, R w1,
                                              R w2, const R* cen, R lf, R eta = (R)0, R* cb = nullptr,
                                              const R* lap3 = nullptr) {
  R Dq[NF];
  deriv12(Dq, fm2, fm1, fp1, fp2, w1, w2);
  apply_direction<R, D1, ETA>(Racc, Dq, cen, lf, eta, cb, lap3);
}

// ------------------------------------------------------------ stage kernel
// Shared memory holds 12 values per cell contiguously (primitives padded to
// 12, or the 12 flux quantities), moved with 16-byte vector accesses.  With a
// 12-float stride the 128-bit accesses of a quarter warp to consecutive cells
// hit distinct banks; FP64 keeps the 12-value stride (2-way conflicts) to fit
// two blocks per SM.
template <class R> struct CellW { static constexpr int W = 12; };

__device__ __forceinline__ void load_cell(const float* p, float v[12]) {
  const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
  for (int a = 0; a < 3; a++) {
    float4 t = q[a];
    v[4 * a] = t.x; v[4 * a + 1] = t.y; v[4 * a + 2] = t.z; v[4 * a + 3] = t.w;
  }
}
__device__ __forceinline__ void store_cell(float* p, const float v[12]) {
  float4* q = reinterpret_cast<float4*>(p);
#pragma unroll
  for (int a = 0; a < 3; a++) q[a] = make_float4(v[4 * a], v[4 * a + 1], v[4 * a + 2], v[4 * a + 3]);
}
__device__ __forceinline__ void load_cell(const double* p, double v[12]) {
  const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
  for (int a = 0; a < 6; a++) {
    double2 t = q[a];
    v[2 * a] = t.x; v[2 * a + 1] = t.y;
  }
}
__device__ __forceinline__ void store_cell(double* p, const double v[12]) {
  double2* q = reinterpret_cast<double2*>(p);
#pragma unroll
  for (int a = 0; a < 6; a++) q[a] = make_double2(v[2 * a], v[2 * a + 1]);
}

// RK update of one cell, un = base + wdt * R, then Tcheck.  With Cc (FP32
// compensated mode) Cc holds, per interior cell, what rounding the state to
// FP32 dropped at the last stage 4: every stage adds it back
// (un = base + (wdt * R + C)) and stage 4 stores the new remainder -- zero
// where Tcheck changed the value.
template <class R>
__device__ __forceinline__ void rk_update(const Consts& c, Rem<R>* __restrict__ Cc, unsigned id, int stage, R wdt,
                                          const R* base, const R* Racc, R vmax, R emax, R* un) {
  if (Cc == nullptr) {
#pragma unroll
    for (int v = 0; v < NV; v++) un[v] = base[v] + wdt * Racc[v];
    tcheck_cell<R>(c, vmax, emax, un[0], un[1], un[2], un[3], un[4]);
    return;
  }
  const unsigned N32 = c.g.N32;
  R y[NV], t[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) {
    y[v] = wdt * Racc[v] + rem_ld<R>(Cc + id + (unsigned)v * N32);
    t[v] = base[v] + y[v];
    un[v] = t[v];
  }
  tcheck_cell<R>(c, vmax, emax, un[0], un[1], un[2], un[3], un[4]);
  if (stage == 4) {
#pragma unroll
    for (int v = 0; v < NV; v++)
      rem_st<R>(Cc + id + (unsigned)v * N32, (un[v] == t[v]) ? y[v] - (t[v] - base[v]) : (R)0);
  }
}

// Boris factor of MHD_Residual's Lorentz-force blend at a cell (src/mhdres_SR.C:310-323).
template <class R>
__device__ __forceinline__ R boris_lf(const R* cen, R inv_va2max) {
  const R dn = (R)1.0 / cen[P_D];
  const R bb = cen[P_B1] * cen[P_B1] + cen[P_B2] * cen[P_B2] + cen[P_B3] * cen[P_B3];
  const R va2 = bb * dn;
  const R x2 = va2 * inv_va2max, x4 = x2 * x2, s = (R)1.0 + x2;
  return s / (s + x4);
}

// Sources and semi-relativistic (Boris) correction added to the residual Racc
// of a cell with primitives cen (src/Add_Sources_Integrate_SR.C:331-392):
// gravity along x, the radiative term (zero here), then the correction.
template <class R>
__device__ __forceinline__ void stage_sources(R* Racc, const R* cen, R gx, R inv_va2max, R invRdt) {
  const R rh = cen[P_D], vx = cen[P_V1], vy = cen[P_V2], vz = cen[P_V3];
  const R bx = cen[P_B1], by = cen[P_B2], bz = cen[P_B3];
  R dn = invRdt * cen[P_EI];
  R efaci = (dn > (R)0 && dn < (R)INFINITY) ? (R)1.0 : dn / d_fmax(dn, (R)0.0);
  dn = gx * rh - (R)0.0;
  const R edmp = dn * vx;
  Racc[1] += dn;
  Racc[4] += edmp + (R)0.0 * efaci;
  const R rd = Racc[0];
  R fx = Racc[1], fy = Racc[2], fz = Racc[3];
  const R bb = bx * bx + by * by + bz * bz;
  const R va2 = bb / rh;
  const R x2 = va2 * inv_va2max, x4 = x2 * x2;
  const R bf = x4 / ((R)1 + x2 + x4);
  fx -= vx * rd;
  fy -= vy * rd;
  fz -= vz * rd;
  const R q = (fx * bx + fy * by + fz * bz) / d_fmax(tiny100<R>(), bb);
  const R b0 = -bf * (fx - q * bx), b1 = -bf * (fy - q * by), b2 = -bf * (fz - q * bz);
  const R b3 = b0 * vx + b1 * vy + b2 * vz;
  Racc[1] += b0;
  Racc[2] += b1;
  Racc[3] += b2;
  Racc[4] += b3;
}

// Shared memory of one stage block: the x fluxes of (TX+4) x TY cells, the y
// fluxes of TX x (TY+4) cells (12 quantities each) and each thread's ring of
// five z-flux planes.
template <int TX, int TY>
struct StageSmem {
  static constexpr int PW = TX + 4, PH = TY + 4;
  static constexpr int FXN = PW * TY;
  static constexpr int FYN = TX * PH;
  static constexpr int NZ = TX * TY;
  template <class R>
  static constexpr size_t bytes() {
    return sizeof(R) * CellW<R>::W * ((size_t)FXN + (size_t)FYN + (size_t)5 * NZ);
  }
};

// RESID = false: fused RK stage.  Uin: conserved state with filled ghosts,
//   Pin: its pressure (ghosts included), U0: the step's initial state,
//   Uout/Pout: the new state and its pressure (interior and ghost images).
// RESID = true: MHD_Residual.  Uin holds primitives (after ConsToPrim),
//   Res = U0 + residual over the interior (U0: the residual accumulated so
//   far, null when it is zero), dyn->cmax_bits gets the interior CFL speed.
//
// A block owns a TX x TY column tile and marches along z.  Per plane, each
// thread converts its own cell to primitives and computes that cell's x and y
// fluxes (into shared memory) and its column's z flux two planes ahead (into
// its private ring); the first 4*(TX+TY) threads also compute the x or y flux
// of one cell of the tile's two-cell halo.  After one barrier every thread
// takes the three fourth-order derivatives of its cell.  All global loads of
// the next plane are issued before the barrier, so their latency overlaps this
// plane's arithmetic.
template <class R, int TX, int TY, bool RESID>
__global__ void __launch_bounds__(TX* TY, 2) k_stage(Consts c, const R* __restrict__ Uin, const R* __restrict__ Pin,
                                                     const R* __restrict__ U0, R* __restrict__ Uout,
                                                     R* __restrict__ Pout, R* __restrict__ Res, Dyn* __restrict__ dyn,
                                                     int stage, int zc, int write_pres, Rem<R>* __restrict__ Cc) {
  using S = StageSmem<TX, TY>;
  constexpr int CW = CellW<R>::W;
  constexpr int NT = TX * TY;
  constexpr int NH = 4 * TY + 4 * TX;  // halo cells: two columns each side (x), two rows each side (y)
  static_assert(NH <= NT, "every halo cell needs a thread");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* FX = reinterpret_cast<R*>(smem_raw);   // x flux of (lx, ly) at ((ly * PW) + lx + 2) * CW
  R* FY = FX + CW * S::FXN;                 // y flux of (lx, ly) at (((ly + 2) * TX) + lx) * CW
  R* FZ = FY + CW * S::FYN;
  const Geom& g = c.g;
  if (!RESID && dyn->err) return;
  const int tid = threadIdx.x;
  const int tx = tid % TX, ty = tid / TX;
  const int x0 = GH + blockIdx.x * TX, y0 = GH + blockIdx.y * TY;
  const int zb = GH + blockIdx.z * zc;
  const int ze = min(zb + zc, GH + g.nz);
  const int i = x0 + tx, j = y0 + ty;
  const bool active = (i < GH + g.nx) && (j < GH + g.ny);
  const bool own_in = (i < g.sx) && (j < g.sy);
  // this thread's halo cell (tid < NH): x-halo cells first (4 per row), then y-halo rows
  int hlx = 0, hly = 0;
  const bool hx = tid < 4 * TY;
  if (tid < NH) {
    if (hx) {
      const int c4 = tid & 3;
      hlx = c4 < 2 ? c4 - 2 : TX + c4 - 2;
      hly = tid >> 2;
    } else {
      const int r = tid - 4 * TY;
      hlx = r % TX;
      const int q = r / TX;
      hly = q < 2 ? q - 2 : TY + q - 2;
    }
  }
  const int hi = x0 + hlx, hj = y0 + hly;
  const bool h_in = (tid < NH) && hi >= 0 && hi < g.sx && hj >= 0 && hj < g.sy;
  const KC<R>& kk_ = kc<R>(c);
  const DynR<R>& dr = dynr<R>(dyn);
  const R inv_va2max = dr.inv_va2max;
  const R w1x = kk_.w1[0], w2x = kk_.w2[0], w1y = kk_.w1[1], w2y = kk_.w2[1], w1z = kk_.w1[2], w2z = kk_.w2[2];
  // per-step scalars (src/Add_Sources_Integrate_SR.C:44, 84-85)
  const R wdt = dr.wdt[(stage >= 1 && stage <= 4) ? stage : 0];
  const R invRdt = dr.invRdt;
  const R vmax = dr.vmax;
  const R emax = dr.emax;
  R cm_acc = (R)0;  // residual mode: this thread's largest CFL speed
  R prim[NF];
  R fl[NF];
  prim[NPRIM] = (R)0;
  fl[NPRIM] = (R)0;

  // z-flux ring: slot of plane kk is (kk - zb + 2) mod 5
  R* const zring = FZ + (size_t)tid * CW;
  auto zcell = [&](int sl) { return zring + sl * (S::NZ * CW); };
  auto slot_add = [](int sl, int d) { return sl + d >= 5 ? sl + d - 5 : sl + d; };
  // zr: the column at plane k+2; orw: the own cell at plane k; hrw: the halo
  // cell at plane k (cells outside the array read as 1, their fluxes unused)
  Raw9<R> zr, orw, hrw;
  fill_raw_one(orw);
  fill_raw_one(hrw);
  const unsigned plane = (unsigned)g.sx * (unsigned)g.sy;
  const unsigned own0 = cidx32(g, i, j, 0), halo0 = cidx32(g, hi, hj, 0);
  for (int kk = zb - 2; kk < zb + 2; kk++) {
    if (active) {
      load_raw<R>(g, Uin, Pin, own0 + (unsigned)kk * plane, zr);
      prim_of_raw<R, RESID>(zr, prim);
      flux12<R, 2>(prim, 1, fl, 1);
      store_cell(zcell(kk - zb + 2), fl);
    }
  }
  if (active) load_raw<R>(g, Uin, Pin, own0 + (unsigned)(zb + 2) * plane, zr);
  if (own_in) load_raw<R>(g, Uin, Pin, own0 + (unsigned)zb * plane, orw);
  if (h_in) load_raw<R>(g, Uin, Pin, halo0 + (unsigned)zb * plane, hrw);

  int s0 = 2;  // ring slot of plane k
  for (int k = zb; k < ze; k++, s0 = slot_add(s0, 1)) {
    R cen[NF];
    if (active) {
      prim_of_raw<R, RESID>(zr, prim);
      flux12<R, 2>(prim, 1, fl, 1);
      store_cell(zcell(slot_add(s0, 2)), fl);
    }
    prim_of_raw<R, RESID>(orw, cen);
    cen[NPRIM] = (R)0;
    flux12<R, 0>(cen, 1, fl, 1);
    store_cell(FX + (ty * S::PW + tx + 2) * CW, fl);
    flux12<R, 1>(cen, 1, fl, 1);
    store_cell(FY + ((ty + 2) * TX + tx) * CW, fl);
    if (tid < NH) {
      prim_of_raw<R, RESID>(hrw, prim);
      if (hx) {
        flux12<R, 0>(prim, 1, fl, 1);
        store_cell(FX + (hly * S::PW + hlx + 2) * CW, fl);
      } else {
        flux12<R, 1>(prim, 1, fl, 1);
        store_cell(FY + ((hly + 2) * TX + hlx) * CW, fl);
      }
    }
    // next plane's loads, in flight during this plane's derivatives
    const unsigned id = own0 + (unsigned)k * plane;
    if (k + 1 < ze) {
      if (active) load_raw<R>(g, Uin, Pin, id + 3 * plane, zr);
      if (own_in) load_raw<R>(g, Uin, Pin, id + plane, orw);
      if (h_in) load_raw<R>(g, Uin, Pin, halo0 + (unsigned)(k + 1) * plane, hrw);
    }
    // this cell's U0 (fused stage) or Res (residual mode), used at the end
    R base[NV];
    if (active) {
      // RESID: U0 is the residual to add to (null: start from zero)
      if (!RESID || U0) {
#pragma unroll
        for (int q = 0; q < NV; q++) base[q] = U0[id + (unsigned)q * g.N32];
      } else {
#pragma unroll
        for (int q = 0; q < NV; q++) base[q] = (R)0;
      }
    }
    __syncthreads();
    if (active) {
      R Racc[NV];
      if (RESID) {
#pragma unroll
        for (int q = 0; q < NV; q++) Racc[q] = base[q];
      } else {
#pragma unroll
        for (int q = 0; q < NV; q++) Racc[q] = (R)0.0;
      }
      // Boris factor at the cell (src/mhdres_SR.C:310-323)
      const R lf = boris_lf<R>(cen, inv_va2max);
      // the three directions, with the resistive terms when eta > 0
      auto directions = [&](auto eta_on) {
        constexpr bool ETA = decltype(eta_on)::value;
        R cb[3] = {(R)0, (R)0, (R)0};
        R lap[3];
        R n0[NF], n1[NF], n2[NF], n3[NF];
        {
          const R* fb = FX + (ty * S::PW + tx + 2) * CW;
          load_cell(fb - 2 * CW, n0);
          load_cell(fb - CW, n1);
          load_cell(fb + CW, n2);
          load_cell(fb + 2 * CW, n3);
          if (ETA) eta_lap<R>(c, Uin, id, 1u, 0, cen, lap);
          add_direction<R, 0, ETA>(Racc, n0, n1, n2, n3, w1x, w2x, cen, lf, kk_.eta, cb, lap);
        }
        {
          const R* fb = FY + ((ty + 2) * TX + tx) * CW;
          load_cell(fb - 2 * TX * CW, n0);
          load_cell(fb - TX * CW, n1);
          load_cell(fb + TX * CW, n2);
          load_cell(fb + 2 * TX * CW, n3);
          if (ETA) eta_lap<R>(c, Uin, id, (unsigned)g.sx, 1, cen, lap);
          add_direction<R, 1, ETA>(Racc, n0, n1, n2, n3, w1y, w2y, cen, lf, kk_.eta, cb, lap);
        }
        load_cell(zcell(slot_add(s0, 3)), n0);
        load_cell(zcell(slot_add(s0, 4)), n1);
        load_cell(zcell(slot_add(s0, 1)), n2);
        load_cell(zcell(slot_add(s0, 2)), n3);
        if (ETA) eta_lap<R>(c, Uin, id, plane, 2, cen, lap);
        add_direction<R, 2, ETA>(Racc, n0, n1, n2, n3, w1z, w2z, cen, lf, kk_.eta, cb, lap);
      };
      if (c.has_eta) directions(std::true_type());
      else directions(std::false_type());
      // Spitzer conduction's share of the energy residual (-sum_d D_d(sflx B_d))
      if (c.has_spitzer) Racc[4] += ((const R*)c.spt_rsp)[id];
      if (RESID) {
#pragma unroll
        for (int q = 0; q < NV; q++) Res[id + (unsigned)q * g.N32] = Racc[q];
        const R cm = cmax_cell<R>(cen[P_D], cen[P_V1], cen[P_V2], cen[P_V3], cen[P_B1], cen[P_B2], cen[P_B3],
                                  cen[P_P], inv_va2max);
        if (cm > cm_acc) cm_acc = cm;  // a NaN speed is skipped, as the atomic maximum skips it
      } else {
        // sources, Boris correction, update, Tcheck (src/Add_Sources_Integrate_SR.C:331-465)
        stage_sources<R>(Racc, cen, kk_.gx, inv_va2max, invRdt);
        R un[NV];
        rk_update<R>(c, Cc, id, stage, wdt, base, Racc, vmax, emax, un);
        const Images im = images_of(g, i, j, k, true);
        store_state<R, true>(g, Uout, i, j, k, im, un);
        if (write_pres) {
          R v1, v2, v3, ei;
          prim_from_cons(un[0], un[1], un[2], un[3], un[4], v1, v2, v3, ei);
          const R pr = eos_pres(c, un[0], ei, (R)1.0 / un[0]);
          store_scalar<R, true>(g, Pout, i, j, k, im, pr);
        }
      }
    }
    __syncthreads();
  }
  if (RESID) {  // one atomic per block
    const R m = block_max_nonnan(cm_acc);
    if (threadIdx.x == 0 && threadIdx.y == 0) atomic_max_nonneg(&dyn->cmax_bits, (double)m);
  }
}

// --------------------------------------------------------------- TVD sweep
// y or z index t (0..n+3) of a cell -> the interior cell it images under the
// periodic fill (itself when interior).
__device__ __forceinline__ int wrap_interior(int t, int n) { return t < GH ? t + n : (t >= GH + n ? t - n : t); }

// Per-cell quantities of TVDlimit's pencil (src/tvdlimit_SR.C:269-377).
template <class R>
struct TCell {
  R q[NV];        // rho (log), v, eps (log), B
  R cm, he, hv, hB, BC2, bsqr, vsqr, hd, hb, ht, qt;
};

struct TvdArgs {
  int dir;               // 0, 1, 2
  int mode;              // 0: plain sweep; 1: z sweep of the first (or only) TVD pass; 2: z sweep of the second half pass
  int only_two_half;     // return at once unless the step takes two half TVD passes
  int td;                // chunk length along the sweep
  int na, nb, a0, b0;    // pencil ranges: a fastest (coalesced), b second
  long long sa, sb, sd;  // strides of a, b and along the sweep
  int n1;                // interior cells along the sweep
};

// An output step's TVDlimit diagnostics (src/tvdlimit_SR.C:577-667): the ten
// diagnostic arrays (tvar1..tvar8, Qres, Qvis; N each), 1 / Run.dt and
// dt_tvd / Run.dt.
template <class R>
struct TvdDiag {
  R* d;
  R idt_full, dt_fac;
};

// Per-cell quantities from the cell's stored values r (state and pressure)
// and its vertical boundary profiles hb, ht, qt.
template <class R>
__device__ __forceinline__ void tvd_cell(const Consts& c, const Raw9<R>& r, R hb, R ht, R qt, R cmax_t, R fac0,
                                         bool hyper, R inv_va2max, TCell<R>& t) {
  const auto& k = kc<R>(c);
  const R rho_min = k.rho_min;
  R d = smax(rho_min, r.v[0]);
  R v1 = r.v[1], v2 = r.v[2], v3 = r.v[3], e = r.v[4];
  R b5 = r.v[5], b6 = r.v[6], b7 = r.v[7];
  t.hb = hb;
  t.ht = ht;
  t.qt = qt;
  R dn = (R)1.0 / d;
  v1 = v1 * dn;
  v2 = v2 * dn;
  v3 = v3 * dn;
  R vv = v1 * v1 + v2 * v2 + v3 * v3;
  R bb = b5 * b5 + b6 * b6 + b7 * b7;
  e = e * dn - (R)0.5 * vv;
  t.vsqr = vv;
  t.bsqr = bb;
  vv = d_sqrt(vv);
  R va2 = bb * dn;
  R x2 = va2 * inv_va2max, x4 = x2 * x2, s = (R)1.0 + x2;
  R lf = s / (s + x4);
  R cs2 = (R)(5.0 / 3.0) * r.v[8] * dn;
  R cfast = d_sqrt(va2 + cs2);
  const R CZ = k.CZ;
  R CME = ((R)1.0 - CZ) * ((R)(vv >= k.CME_thresh * cfast));
  dn = d * d;
  R rf = smin(lf, dn / (dn + k.rho_lev));
  R hh = (R)1.0 - t.hb - t.ht;
  R cf = t.hb * k.tvd_cs[0] + (rf * k.tvd_cs[1] + ((R)1.0 - rf) * k.tvd_cs[2]) * hh + t.ht * k.tvd_cs[3];
  cf = smax(cf, CME);
  cs2 *= cf * cf;
  t.cm = (R)0.0 + vv + d_sqrt(smax(cs2, lf * (cs2 + va2)));
  const R h0 = k.tvd_h[0], h1 = k.tvd_h[1], h2 = k.tvd_h[2], h3 = k.tvd_h[3];
  t.he = t.hb * h0 + (rf * h1 + ((R)1.0 - rf) * h2) * hh + t.ht * h3;
  t.hv = t.hb * h0 + (rf * h1 + ((R)1.0 - rf) * h2 * k.pm_v) * hh + t.ht * h3 * k.pm_v;
  t.hB = t.hb * h0 + (rf * h1 + ((R)1.0 - rf) * h2 * k.pm_B) * hh + t.ht * h3 * k.pm_B;
  t.he *= ((R)1.0 - CME);
  t.hv *= ((R)1.0 - CME);
  t.BC2 = (R)1.0 - lf;
  t.hd = (R)0;
  if (hyper) {
    R h = k.vhyp * d_sqrt(t.vsqr);
    t.hd = fac0 * smax((R)0.0, smin(h, cmax_t - t.cm));
  }
  if (c.rho_log) {
    d = d_log(d);
    e = d_log(e);
  }
  t.q[0] = d; t.q[1] = v1; t.q[2] = v2; t.q[3] = v3; t.q[4] = e; t.q[5] = b5; t.q[6] = b6; t.q[7] = b7;
}

template <class R>
__device__ __forceinline__ void tvd_load(const Consts& c, const R* __restrict__ U, const R* __restrict__ P, long long id,
                                         int xi, R cmax_t, R fac0, bool hyper, R inv_va2max, TCell<R>& t) {
  const Geom& g = c.g;
  const auto& k = kc<R>(c);
  Raw9<R> r;
#pragma unroll
  for (int q = 0; q < NV; q++) r.v[q] = U[(long long)q * g.N + id];
  r.v[8] = P[id];
  tvd_cell<R>(c, r, k.hfb[xi], k.hft[xi], k.qft[xi], cmax_t, fac0, hyper, inv_va2max, t);
}

// Limited slope at the middle cell b (src/tvdlimit_SR.C:388-434)
template <class R>
__device__ __forceinline__ void tvd_slope(const Consts& c, const TCell<R>& a, const TCell<R>& b, const TCell<R>& n,
                                          R vsqr_diff, R* slp) {
#pragma unroll
  for (int v = 0; v < NV; v++) {
    R sl = b.q[v] - a.q[v];
    R sr = n.q[v] - b.q[v];
    R slm = (R)0.25 * (sl + sr);
    R lower = smin(smin(sl, sr), slm);
    R upper = smax(smax(sl, sr), slm);
    slp[v] = smax((R)0.0, lower) + smin((R)0.0, upper);
  }
  const auto& k = kc<R>(c);
  if (k.has_visc_slope) {
    R cf = ((R)1.0 - k.visc_slope_bot * b.hb) * ((R)1.0 - k.visc_slope_top * b.ht);
    slp[1] *= cf; slp[2] *= cf; slp[3] *= cf;
  }
  if (k.has_eta_slope) {
    R cf = ((R)1.0 - k.eta_slope_bot * b.hb) * ((R)1.0 - k.eta_slope_top * b.ht);
    slp[5] *= cf; slp[6] *= cf; slp[7] *= cf;
  }
  R qr = c.rho_log ? d_fabs(b.q[0] - n.q[0]) : d_fabs(d_log(b.q[0]) - d_log(n.q[0]));
  if (qr > k.q_rho_max) slp[0] = (R)0.0;
  if (k.has_vmax_lim && b.vsqr > vsqr_diff) { slp[1] = (R)0.0; slp[2] = (R)0.0; slp[3] = (R)0.0; }
}

// Interface flux between cells a (index ia) and b, plus its resistive-heating
// term (src/tvdlimit_SR.C:436-557, 559-563, 608-614).  am = cell left of a,
// bp = cell right of b (hyperdiffusion stencil).
template <class R, int DIR, bool DIAG = false>
__device__ __forceinline__ void tvd_flux(const Consts& c, const TCell<R>& am, const TCell<R>& a, const TCell<R>& b,
                                         const TCell<R>& bp, const R* sa, const R* sb, int ia, int sz, R fac0,
                                         R cmax_t, bool hyper, int istart, R* F, R& qres, R* qvis = nullptr) {
#pragma unroll
  for (int v = 0; v < NV; v++) {
    R sl = b.q[v] - a.q[v];
    R sl_lim = b.q[v] - a.q[v] - (sa[v] + sb[v]);
    R dn = (v >= 1 && v <= 3) ? a.hv : ((v >= 5) ? a.hB : a.he);
    R rf = d_fabs(sl_lim) / smax(tiny100<R>(), d_fabs(sl));
    R cf = smax((R)0.0, smin(sl_lim, sl)) + smin((R)0.0, smax(sl_lim, sl));
    F[v] = smax((R)0.0, (R)1.0 + dn * (rf - (R)1.0)) * cf;
  }
  R fac = fac0 * smin(cmax_t, smax(a.cm, b.cm));
#pragma unroll
  for (int v = 0; v < NV; v++) F[v] *= fac;
  const auto& k = kc<R>(c);
  F[5 + DIR] *= k.B_par_diff;
  if (c.need_coeff) {
    F[0] *= k.tvd_coeff[0];
    R cf = smax(k.tvd_coeff[1], k.visc_coeff_bot * a.hb + k.visc_coeff_top * a.ht);
    F[1] *= cf; F[2] *= cf; F[3] *= cf;
    F[4] *= k.tvd_coeff[2];
    cf = smax(k.tvd_coeff[3], k.eta_coeff_bot * a.hb + k.eta_coeff_top * a.ht);
    F[5] *= cf; F[6] *= cf; F[7] *= cf;
  }
  if (DIR == 0 && hyper && ia >= istart) {
    R dn = smax(a.hd, b.hd);
    F[0] -= dn * ((R)0.125 * (bp.q[0] - am.q[0]) - (R)0.375 * (b.q[0] - a.q[0]));
    F[1] -= dn * ((R)0.125 * (bp.q[1] - am.q[1]) - (R)0.375 * (b.q[1] - a.q[1]));
    F[4] -= dn * ((R)0.125 * (bp.q[4] - am.q[4]) - (R)0.375 * (b.q[4] - a.q[4]));
  }
  R f0 = F[0], f1 = F[1], f2 = F[2], f3 = F[3], f4 = F[4];
  R u[5];
#pragma unroll
  for (int v = 0; v < 5; v++) u[v] = (R)0.5 * (a.q[v] + sa[v] + b.q[v] - sb[v]);
  if (c.rho_log) {
    u[0] = d_exp(u[0]);
    f0 *= u[0];
    u[4] = d_exp(u[4]);
    f4 *= u[4];
  }
  const R CZ = k.CZ;
  R min_cz = f0 * smin(CZ, CZ);
  f1 *= u[0]; f1 += u[1] * min_cz;
  f2 *= u[0]; f2 += u[2] * min_cz;
  f3 *= u[0]; f3 += u[3] * min_cz;
  f4 *= u[0];
  f4 += (u[4] * min_cz) + a.qt * (u[1] * f1 + u[2] * f2 + u[3] * f3);
  F[0] = f0; F[1] = f1; F[2] = f2; F[3] = f3; F[4] = f4;
  if (DIR == 0 && !c.g.periodic_x) {
    if (ia == sz - GH - 1) F[5] = (R)0.0;
    if (ia == GH - 1) F[5] = (R)0.0;
  }
  qres = (b.q[5] - a.q[5]) * F[5] + (b.q[6] - a.q[6]) * F[6] + (b.q[7] - a.q[7]) * F[7];
  // viscous heating at the interface, for the diagnostics (src/tvdlimit_SR.C:626-635)
  if (DIAG) *qvis = (b.q[1] - a.q[1]) * F[1] + (b.q[2] - a.q[2]) * F[2] + (b.q[3] - a.q[3]) * F[3];
}

// Update of one cell by a TVD sweep (src/tvdlimit_SR.C:565-657): the flux
// difference, its kinetic-energy and Boris parts, the resistive heating, and
// the density and energy floors.  u_in: the cell's stored state; Fp / Fm: the
// fluxes at its right / left interfaces, qp / qm their heating terms.
// DIAG (an output step): the sweep's diagnostics of cell id accumulate in
// dg (src/tvdlimit_SR.C:577-584, 601-604, 617-624, 659-667); qvp / qvm: the
// viscous heating terms of its right / left interfaces.
// Cin (FP32 compensated mode, else null): the remainders of the cell's
// state, at stride N -- what rounding the state to FP32 has dropped so far;
// the update then adds them (u = u_in + (res + C)) and Cout (null for a
// ghost image, whose source cell keeps them) receives the new remainders,
// zero where a floor changed the value.
template <class R, bool DIAG = false>
__device__ __forceinline__ void tvd_update(const Consts& c, R dtt, const R* Fp, const R* Fm, R qp, R qm,
                                           const TCell<R>& c0, const R* u_in, R* u, const TvdDiag<R>* dg = nullptr,
                                           long long id = 0, R qvp = (R)0, R qvm = (R)0, const Rem<R>* Cin = nullptr,
                                           Rem<R>* Cout = nullptr) {
  const auto& kk_ = kc<R>(c);
  const long long N = c.g.N;
  R res[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) res[v] = dtt * (Fp[v] - Fm[v]);
  res[4] += ((R)1.0 - c0.qt) * (res[1] * c0.q[1] + res[2] * c0.q[2] + res[3] * c0.q[3]);
  if (DIAG) dg->d[7 * N + id] += res[4] * dg->idt_full;
  {
    R dn = (res[1] * c0.q[5] + res[2] * c0.q[6] + res[3] * c0.q[7]) / smax(tiny100<R>(), c0.bsqr);
    R b0 = -c0.BC2 * (res[1] - dn * c0.q[5]);
    R b1 = -c0.BC2 * (res[2] - dn * c0.q[6]);
    R b2 = -c0.BC2 * (res[3] - dn * c0.q[7]);
    R b3 = b0 * c0.q[1] + b1 * c0.q[2] + b2 * c0.q[3];
    res[1] += b0; res[2] += b1; res[3] += b2; res[4] += b3;
    if (DIAG) dg->d[5 * N + id] += b3 * dg->idt_full;
  }
  {
    R qres = (R)0.5 * (qp + qm) * c0.qt;
    res[4] += dtt * qres;
    if (DIAG) dg->d[8 * N + id] += dg->dt_fac * qres;
  }
  if constexpr (std::is_same<R, float>::value) {
    if (Cin) {  // compensated sum and the floors
      R rem[NV];
#pragma unroll
      for (int v = 0; v < NV; v++) {
        const R y = res[v] + rem_ld<R>(Cin + (long long)v * N);
        u[v] = u_in[v] + y;
        rem[v] = y - (u[v] - u_in[v]);
      }
      const R d0 = u[0];
      u[0] = smax((R)kk_.rho_min, u[0]);
      const R e0 = u[4];
      u[4] = smax(u[4], kk_.eps_min * u[0] + (R)0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) / u[0]);
      if (Cout) {
        if (u[0] != d0) rem[0] = (R)0;
        if (u[4] != e0) rem[4] = (R)0;
#pragma unroll
        for (int v = 0; v < NV; v++) rem_st<R>(Cout + (long long)v * N, rem[v]);
      }
      return;
    }
  }
#pragma unroll
  for (int v = 0; v < NV; v++) u[v] = u_in[v] + res[v];
  u[0] = smax((R)kk_.rho_min, u[0]);
  const R eb = u[4];
  u[4] = smax(u[4], kk_.eps_min * u[0] + (R)0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) / u[0]);
  if (DIAG) {
    dg->d[6 * N + id] += (u[4] - eb) * dg->idt_full;
    dg->d[9 * N + id] += dg->dt_fac * ((R)0.5 * (qvp + qvm) * c0.qt);
  }
}

// The end of a step for one interior cell with its updated state u: TCheck,
// the state's ghost images (closed-x mirror included), and the next step's
// stage-1 pressure, CFL speed and Adjust_Valf_Max statistics, accumulated in
// FinishAcc and reduced once per warp by flush().
template <class R>
struct FinishAcc {
  R cmax = (R)0, v = (R)0, cs = (R)0, e = (R)0;
  unsigned long long nv = 0, ne = 0;
  // Warp reductions, then lane 0 of each warp parks its values in shared
  // memory and warp 0 combines them: one atomic per statistic and block
  // (same-address atomics from every warp serialise in L2).  Every thread of
  // the block calls this.
  __device__ __forceinline__ void flush(Dyn* dyn) {
    __shared__ R sr[32][4];
    __shared__ unsigned long long sn[32][2];
    R a0 = warp_max_nonnan(cmax);
    R a1 = warp_max_nonnan(v), a2 = warp_max_nonnan(cs), a3 = warp_max_nonnan(e);
    for (int o = 16; o > 0; o >>= 1) {
      nv += __shfl_xor_sync(0xffffffffu, nv, o);
      ne += __shfl_xor_sync(0xffffffffu, ne, o);
    }
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
    const int w = tid >> 5, lane = tid & 31;
    if (lane == 0) {
      sr[w][0] = a0; sr[w][1] = a1; sr[w][2] = a2; sr[w][3] = a3;
      sn[w][0] = nv; sn[w][1] = ne;
    }
    __syncthreads();
    if (w == 0) {
      const bool h = lane < nw;
      a0 = warp_max_nonnan(h ? sr[lane][0] : (R)0);
      a1 = warp_max_nonnan(h ? sr[lane][1] : (R)0);
      a2 = warp_max_nonnan(h ? sr[lane][2] : (R)0);
      a3 = warp_max_nonnan(h ? sr[lane][3] : (R)0);
      unsigned long long c0 = h ? sn[lane][0] : 0ULL, c1 = h ? sn[lane][1] : 0ULL;
      for (int o = 16; o > 0; o >>= 1) {
        c0 += __shfl_xor_sync(0xffffffffu, c0, o);
        c1 += __shfl_xor_sync(0xffffffffu, c1, o);
      }
      if (lane == 0) {
        atomic_max_nonneg(&dyn->cmax_bits, (double)a0);
        atomic_max_nonneg(&dyn->stat_max_bits[0], (double)a1);
        atomic_max_nonneg(&dyn->stat_max_bits[1], (double)a2);
        atomic_max_nonneg(&dyn->stat_max_bits[2], (double)a3);
        if (c0) atomicAdd(&dyn->stat_cnt[0], c0);
        if (c1) atomicAdd(&dyn->stat_cnt[1], c1);
      }
    }
  }
};

// End of a fused step, after the TVD sweeps (and Clean_divB): per interior
// cell TCheck (src/Add_Sources_Integrate_SR.C:534-625) in place -- a field is
// stored only where TCheck changed its bits, so most cells cost reads only --,
// the cell's ghost images (closed-x mirror included), and the next step's
// stage-1 pressure, CFL speed and Adjust_Valf_Max statistics.  Block 32 x 8
// over (x, y), z planes by the grid's third dimension.
constexpr int FIN_BX = 32, FIN_BY = 8;

template <class R>
__device__ __forceinline__ bool same_bits(R a, R b);
template <>
__device__ __forceinline__ bool same_bits<float>(float a, float b) { return __float_as_uint(a) == __float_as_uint(b); }
template <>
__device__ __forceinline__ bool same_bits<double>(double a, double b) {
  return __double_as_longlong(a) == __double_as_longlong(b);
}

// resident blocks per SM the register budget is set for (FP32: 64 registers)
template <class R> struct FinBlocks { static constexpr int v = sizeof(R) == 4 ? 4 : 2; };

// COMP (FP32 compensated mode; Cc its remainders): a field TCheck changes loses its remainder.
template <class R, bool COMP = false>
__global__ void __launch_bounds__(FIN_BX* FIN_BY, FinBlocks<R>::v) k_step_finish(Consts c, R* __restrict__ U, R* __restrict__ Pout,
                                                               Dyn* __restrict__ dyn, Rem<R>* __restrict__ Cc) {
  if (dyn->err) return;
  const Geom& g = c.g;
  const DynR<R>& dr = dynr<R>(dyn);
  const R vmax = dr.vmax, emax = dr.emax, inv_va2max = dr.inv_va2max, vlim95 = dr.vlim95, elim95 = dr.elim95;
  FinishAcc<R> acc;
  const int i = GH + blockIdx.x * FIN_BX + threadIdx.x;
  const int j = GH + blockIdx.y * FIN_BY + threadIdx.y;
  if (i < GH + g.nx && j < GH + g.ny) {
#pragma unroll 2
    for (int k = GH + blockIdx.z; k < GH + g.nz; k += gridDim.z) {
      const unsigned id = cidx32(g, i, j, k);
      R u[NV], u0[5];
#pragma unroll
      for (int v = 0; v < NV; v++) u[v] = U[(unsigned)v * g.N32 + id];
#pragma unroll
      for (int v = 0; v < 5; v++) u0[v] = u[v];
      tcheck_cell<R>(c, vmax, emax, u[0], u[1], u[2], u[3], u[4]);
#pragma unroll
      for (int v = 0; v < 5; v++)
        if (!same_bits(u[v], u0[v])) {
          U[(unsigned)v * g.N32 + id] = u[v];
          if (COMP) rem_st<R>(Cc + (unsigned)v * g.N32 + id, (R)0);
        }
      R v1, v2, v3, ei;
      prim_from_cons(u[0], u[1], u[2], u[3], u[4], v1, v2, v3, ei);
      const R pr = eos_pres(c, u[0], ei, (R)1.0 / u[0]);
      Pout[id] = pr;
      const Images im = images_of(g, i, j, k, true);
      if (im.xa >= 0 || im.ya >= 0 || im.za >= 0) {
        // the ghost images (every combination but the cell itself)
        for (int q = 1; q < 8; q++) {
          const int ii = (q & 1) ? im.xa : i, jj = (q & 2) ? im.ya : j, kk = (q & 4) ? im.za : k;
          if (ii < 0 || jj < 0 || kk < 0) continue;
          const unsigned gid = cidx32(g, ii, jj, kk);
          const bool f = (q & 1) && im.xf;
#pragma unroll
          for (int v = 0; v < NV; v++) {
            R x = u[v];
            if (f && (v == 1 || v == 6 || v == 7)) x = -x;
            U[(unsigned)v * g.N32 + gid] = x;
          }
          Pout[gid] = pr;
        }
      }
      R cmv = cmax_cell<R>(u[0], v1, v2, v3, u[5], u[6], u[7], pr, inv_va2max);
      acc.cmax = smax(acc.cmax, cmv);
      R vabs = d_sqrt(v1 * v1 + v2 * v2 + v3 * v3);
      R cs = (R)(5 / 3.) * pr / u[0];
      R ee = ei / u[0];
      acc.v = d_fmax(acc.v, vabs);
      acc.cs = d_fmax(acc.cs, cs);
      acc.e = d_fmax(acc.e, ee);
      if (vabs >= vlim95) acc.nv++;
      if (ee >= elim95) acc.ne++;
    }
  }
  acc.flush(dyn);
}

// Resident blocks of 128 threads the TVD sweeps are compiled for (FP32; FP64
// keeps the compiler's register choice).  Measured at 128 x 384 x 384: y / z
// sweeps 0.496 / 0.489 -> 0.490 / 0.482 ms with 4 blocks (128 registers, a
// few spilled), the x sweep 0.623 -> 0.603 ms with 6 (85 registers).
template <class R> struct TvdBlocks { static constexpr int pencil = sizeof(R) == 4 ? 4 : 1, lanes = sizeof(R) == 4 ? 6 : 1; };

// COMP: FP32 compensated fused steps (Cc: the state's rounding remainders).
template <class R, int DIR, bool DIAG = false, bool COMP = false>
__global__ void __launch_bounds__(128, TvdBlocks<R>::pencil) k_tvd_sweep(Consts c, const R* __restrict__ Uin, const R* __restrict__ Pst,
                                                   R* __restrict__ Uout, Dyn* __restrict__ dyn, TvdArgs ta,
                                                   TvdDiag<R> dg, Rem<R>* __restrict__ Cc) {
  const Geom& g = c.g;
  if (dyn->err) return;
  if (ta.only_two_half && !dyn->two_half) return;   // second half pass not taken this step
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned nch = (unsigned)((ta.n1 + ta.td - 1) / ta.td);
  const unsigned total = (unsigned)ta.na * (unsigned)ta.nb * nch;
  bool live = t < total;
  int a = 0, b = 0, ch = 0;
  if (live) {
    a = (int)(t % (unsigned)ta.na);
    const unsigned r = t / (unsigned)ta.na;
    b = (int)(r % (unsigned)ta.nb);
    ch = (int)(r / (unsigned)ta.nb);
  }
  const int aa = ta.a0 + a, bb = ta.b0 + b;
  const long long base = (long long)aa * ta.sa + (long long)bb * ta.sb;
  const int sz = ta.n1 + 2 * GH;
  const int p0 = GH + ch * ta.td;
  const int p1 = min(p0 + ta.td, GH + ta.n1);
  const DynR<R>& dr = dynr<R>(dyn);
  const R dtt = dr.dt_tvd;
  const R cmax_t = dr.cmax_t[DIR];
  const R fac0 = dr.fac0[DIR];
  const R inv_va2max = dr.inv_va2max;
  const R vsqr_diff = dr.vsqr_diff;
  const bool hyper = (DIR == 0) && kc<R>(c).has_vhyp;
  const KC<R>& kk_ = kc<R>(c);
  const int istart = 1 + (c.g.periodic_x ? 0 : GH);
  // after the first of two half passes the z sweep also writes the periodic
  // images (the exchange between the halves); otherwise the interior only --
  // k_step_finish ends the step (TCheck, images, next pressure, statistics)
  const bool half_images = (ta.mode == 1) && dyn->two_half;
  if (live) {
    auto xi_of = [&](int pos) { return DIR == 0 ? pos : aa; };
    TCell<R> cm1, c0, c1, c2;
    R s0[NV], s1[NV], Fm[NV], F0[NV];
    R qm, q0;
    R qvm = (R)0, qv0 = (R)0;  // viscous heating at the interfaces (diagnostics)
    {
      TCell<R> cmm;
      tvd_load<R>(c, Uin, Pst, base + (long long)(p0 - 2) * ta.sd, xi_of(p0 - 2), cmax_t, fac0, hyper, inv_va2max, cmm);
      tvd_load<R>(c, Uin, Pst, base + (long long)(p0 - 1) * ta.sd, xi_of(p0 - 1), cmax_t, fac0, hyper, inv_va2max, cm1);
      tvd_load<R>(c, Uin, Pst, base + (long long)p0 * ta.sd, xi_of(p0), cmax_t, fac0, hyper, inv_va2max, c0);
      tvd_load<R>(c, Uin, Pst, base + (long long)(p0 + 1) * ta.sd, xi_of(p0 + 1), cmax_t, fac0, hyper, inv_va2max, c1);
      R sm[NV];
      tvd_slope<R>(c, cmm, cm1, c0, vsqr_diff, sm);
      tvd_slope<R>(c, cm1, c0, c1, vsqr_diff, s0);
      tvd_flux<R, DIR, DIAG>(c, cmm, cm1, c0, c1, sm, s0, p0 - 1, sz, fac0, cmax_t, hyper, istart, Fm, qm, &qvm);
    }
    // the boundary profiles depend on x only: fixed along a y or z pencil
    R hb_f = (R)0, ht_f = (R)0, qt_f = (R)0;
    if (DIR != 0) { hb_f = kk_.hfb[aa]; ht_f = kk_.hft[aa]; qt_f = kk_.qft[aa]; }
    // the next cell's stored values are loaded one step ahead of their use
    Raw9<R> nxt;
    load_raw64<R>(g, Uin, Pst, base + (long long)(p0 + 2) * ta.sd, nxt);
    for (int pos = p0; pos < p1; pos++) {
      const long long id = base + (long long)pos * ta.sd;
      R uc[NV];
#pragma unroll
      for (int v = 0; v < NV; v++) uc[v] = Uin[(long long)v * g.N + id];
      if (DIR == 0)
        tvd_cell<R>(c, nxt, kk_.hfb[pos + 2], kk_.hft[pos + 2], kk_.qft[pos + 2], cmax_t, fac0, hyper, inv_va2max, c2);
      else
        tvd_cell<R>(c, nxt, hb_f, ht_f, qt_f, cmax_t, fac0, hyper, inv_va2max, c2);
      if (pos + 1 < p1) load_raw64<R>(g, Uin, Pst, base + (long long)(pos + 3) * ta.sd, nxt);
      tvd_slope<R>(c, c0, c1, c2, vsqr_diff, s1);
      tvd_flux<R, DIR, DIAG>(c, cm1, c0, c1, c2, s0, s1, pos, sz, fac0, cmax_t, hyper, istart, F0, q0, &qv0);
      // update of cell pos (src/tvdlimit_SR.C:565-657)
      R u[NV];
      const Rem<R>* cin = nullptr;
      Rem<R>* cout = nullptr;
      if (COMP) {  // FP32 compensated: the remainders of the interior cell this one is or images
        const int ci = DIR == 0 ? pos : aa, cj = DIR == 1 ? pos : (DIR == 0 ? aa : bb), ck = DIR == 2 ? pos : bb;
        const int sj = wrap_interior(cj, g.ny), sk = wrap_interior(ck, g.nz);
        const long long src = (long long)ci + (long long)g.sx * ((long long)sj + (long long)g.sy * sk);
        cin = Cc + src;
        if (sj == cj && sk == ck) cout = Cc + id;
      }
      tvd_update<R, DIAG>(c, dtt, F0, Fm, q0, qm, c0, uc, u, &dg, id, qv0, qvm, cin, cout);
      if (!half_images) {
#pragma unroll
        for (int v = 0; v < NV; v++) Uout[(long long)v * g.N + id] = u[v];
      } else {
        // first of two half steps: exchange (periodic dimensions) only
        int ci = DIR == 0 ? pos : aa, cj = DIR == 1 ? pos : (DIR == 0 ? aa : bb), ck = DIR == 2 ? pos : bb;
        store_state<R>(g, Uout, ci, cj, ck, images_of(g, ci, cj, ck, false), u);
      }
      // shift the window
      cm1 = c0; c0 = c1; c1 = c2;
#pragma unroll
      for (int v = 0; v < NV; v++) { s0[v] = s1[v]; Fm[v] = F0[v]; }
      qm = q0;
      qvm = qv0;
    }
  }
}

// --------------------------------------------------- TVD sweep along x, by lanes
// The x pencils are contiguous in memory, so here a warp holds 32 consecutive
// cells of one pencil, one per lane (coalesced loads and stores), and the
// stencil neighbours come from warp shuffles: 28 cells are updated per warp,
// the two lanes at each end are the sweep's halo.  Same arithmetic as
// k_tvd_sweep<R, 0>; used for the plain (mode 0) x sweep.
template <class R>
__device__ __forceinline__ R shfl(R v, int src) { return __shfl_sync(0xffffffffu, v, src); }

template <class R, bool COMP = false>
__global__ void __launch_bounds__(128, TvdBlocks<R>::lanes) k_tvd_sweep_xlanes(Consts c, const R* __restrict__ Uin, const R* __restrict__ Pst,
                                                          R* __restrict__ Uout, Dyn* __restrict__ dyn, int only_two_half,
                                                          Rem<R>* __restrict__ Cc) {
  const Geom& g = c.g;
  if (dyn->err) return;
  if (only_two_half && !dyn->two_half) return;
  constexpr int OUT = 28;
  const int lane = threadIdx.x & 31;
  const unsigned nseg = (unsigned)((g.nx + OUT - 1) / OUT);
  const unsigned total = (unsigned)g.sy * (unsigned)g.sz * nseg;
  const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
  const DynR<R>& dr = dynr<R>(dyn);
  const R dtt = dr.dt_tvd;
  const R cmax_t = dr.cmax_t[0];
  const R fac0 = dr.fac0[0];
  const R inv_va2max = dr.inv_va2max;
  const R vsqr_diff = dr.vsqr_diff;
  const bool hyper = kc<R>(c).has_vhyp;
  const KC<R>& kk_ = kc<R>(c);
  const int istart = 1 + (g.periodic_x ? 0 : GH);
  const int sz = g.nx + 2 * GH;
  const int lm = max(lane - 1, 0), lp = min(lane + 1, 31), lpp = min(lane + 2, 31);
  // whole warps stride over (pencil, segment) pairs together
  for (unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; warp < total; warp += nwarps) {
    const unsigned seg = warp % nseg;
    const unsigned pen = warp / nseg;
    const unsigned j = pen % (unsigned)g.sy, k = pen / (unsigned)g.sy;
    const long long base = (long long)g.sx * ((long long)j + (long long)g.sy * (long long)k);
    const int pos = GH + OUT * (int)seg - 2 + lane;     // this lane's cell along x
    const int posc = min(pos, g.sx - 1);                 // clamped for the tail of the last segment
    TCell<R> c0, cl, cr, crr;
    tvd_load<R>(c, Uin, Pst, base + posc, posc, cmax_t, fac0, hyper, inv_va2max, c0);
    // from the neighbours only what the slope and the interface flux read:
    // q of both, cm and hd of the right one, q[0,1,4] two to the right (hyperdiffusion)
#pragma unroll
    for (int v = 0; v < NV; v++) {
      cl.q[v] = shfl(c0.q[v], lm);
      cr.q[v] = shfl(c0.q[v], lp);
    }
    cr.cm = shfl(c0.cm, lp);
    cr.hd = shfl(c0.hd, lp);
    if (hyper) {
      crr.q[0] = shfl(c0.q[0], lpp);
      crr.q[1] = shfl(c0.q[1], lpp);
      crr.q[4] = shfl(c0.q[4], lpp);
    }
    R s0[NV], s1[NV], F[NV], Fm[NV];
    tvd_slope<R>(c, cl, c0, cr, vsqr_diff, s0);
#pragma unroll
    for (int v = 0; v < NV; v++) s1[v] = shfl(s0[v], lp);
    R qr;
    tvd_flux<R, 0>(c, cl, c0, cr, crr, s0, s1, pos, sz, fac0, cmax_t, hyper, istart, F, qr);
#pragma unroll
    for (int v = 0; v < NV; v++) Fm[v] = shfl(F[v], lm);
    const R qm = shfl(qr, lm);
    if (lane < 2 || lane >= 30 || pos >= GH + g.nx) continue;
    const long long id = base + pos;
    R uc[NV], u[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) uc[v] = Uin[(long long)v * g.N + id];
    const Rem<R>* cin = nullptr;
    Rem<R>* cout = nullptr;
    if (COMP) {  // FP32 compensated: the remainders of the interior cell this one is or images
      const int sj = wrap_interior((int)j, g.ny), sk = wrap_interior((int)k, g.nz);
      cin = Cc + ((long long)g.sx * ((long long)sj + (long long)g.sy * sk) + pos);
      if (sj == (int)j && sk == (int)k) cout = Cc + id;
    }
    tvd_update<R>(c, dtt, F, Fm, qr, qm, c0, uc, u, nullptr, 0, (R)0, (R)0, cin, cout);
#pragma unroll
    for (int v = 0; v < NV; v++) Uout[(long long)v * g.N + id] = u[v];
  }
}

// ---------------------------------------------------------- small kernels
// ConsToPrim over the whole box (src/cons_to_prim.C:78-266).  FP32: compiled
// for 6 resident blocks of 256 (at most 42 registers; the spills are in the
// FP64 fallback of cells outside the table): 0.71 -> 0.52 ms at 19.9 M nodes,
// the EOS gathers' latency hidden by more warps.  The same bound serves the
// temperature and Source_Integrate kernels (0.97 -> 0.75 ms).
template <class R> struct EwBlocks { static constexpr int v = sizeof(R) == 4 ? 6 : 1; };
template <class R, bool SNAP>
__global__ void __launch_bounds__(256, EwBlocks<R>::v) k_cons_to_prim(Consts c, R* __restrict__ U, R* __restrict__ P, R* __restrict__ T, R* __restrict__ Ne,
                               R* __restrict__ Ri, R* __restrict__ Am) {
  const Geom& g = c.g;
  const unsigned N = g.N32;
  for (unsigned id = gs_first(); id < N; id += gs_step()) {
    R d = U[id];
    R v1, v2, v3, ei;
    prim_from_cons(d, U[N + id], U[2 * N + id], U[3 * N + id], U[4 * N + id], v1, v2, v3, ei);
    const R dn = (R)1.0 / d;
    R pr, tm, ne, ri, am;
    c2p_outputs(c, d, ei, dn, pr, tm, ne, ri, am);
    U[N + id] = v1;
    U[2 * N + id] = v2;
    U[3 * N + id] = v3;
    U[4 * N + id] = ei;
    P[id] = pr;
    if (SNAP) {  // the EOS inputs, from which k_aux_of_snapshot forms the other outputs
      T[id] = d;
      Ne[id] = ei;
    } else if (T) {
      T[id] = tm; Ne[id] = ne; Ri[id] = ri; Am[id] = am;
    }
  }
}

// ConsToPrim's temperature, n_e, rho_i and ambipolar coefficient from the
// density and internal energy that k_cons_to_prim<R, true> left in T and Ne:
// the same routine on the same inputs, so the same values as computing them
// there.
template <class R>
__global__ void __launch_bounds__(256, EwBlocks<R>::v) k_aux_of_snapshot(Consts c, R* __restrict__ T, R* __restrict__ Ne,
                                                                    R* __restrict__ Ri, R* __restrict__ Am) {
  const unsigned N = c.g.N32;
  for (unsigned id = gs_first(); id < N; id += gs_step()) {
    const R d = T[id], ei = Ne[id];
    const R dn = (R)1.0 / d;
    R pr, tm, ne, ri, am;
    c2p_outputs(c, d, ei, dn, pr, tm, ne, ri, am);
    T[id] = tm; Ne[id] = ne; Ri[id] = ri; Am[id] = am;
  }
}

// Fused-path initial pass: pressure of the conserved state over the whole box,
// CFL speed and Adjust_Valf_Max statistics over the interior.
template <class R>
__global__ void k_init_pass(Consts c, const R* __restrict__ U, R* __restrict__ P, Dyn* __restrict__ dyn) {
  const Geom& g = c.g;
  R cm_loc = 0, sv = 0, sc = 0, se = 0;
  unsigned long long nv = 0, ne = 0;
  const R inv_va2max = dynr<R>(dyn).inv_va2max;
  const R vlim95 = dynr<R>(dyn).vlim95, elim95 = dynr<R>(dyn).elim95;
  const unsigned N = g.N32;
  for (unsigned id = gs_first(); id < N; id += gs_step()) {
    R d = U[id];
    R v1, v2, v3, ei;
    prim_from_cons(d, U[N + id], U[2 * N + id], U[3 * N + id], U[4 * N + id], v1, v2, v3, ei);
    R pr = eos_pres(c, d, ei, (R)1.0 / d);
    P[id] = pr;
    int i, j, k;
    node_ijk(g, id, i, j, k);
    if (i >= GH && i < GH + g.nx && j >= GH && j < GH + g.ny && k >= GH && k < GH + g.nz) {
      cm_loc = smax(cm_loc, cmax_cell<R>(d, v1, v2, v3, U[5 * N + id], U[6 * N + id], U[7 * N + id], pr, inv_va2max));
      R vabs = d_sqrt(v1 * v1 + v2 * v2 + v3 * v3);
      R cs = (R)(5 / 3.) * pr / d;
      R ee = ei / d;
      sv = d_fmax(sv, vabs);
      sc = d_fmax(sc, cs);
      se = d_fmax(se, ee);
      if (vabs >= vlim95) nv++;
      if (ee >= elim95) ne++;
    }
  }
  R m = warp_max_nonnan(cm_loc);
  R a1 = warp_max_nonnan(sv), a2 = warp_max_nonnan(sc), a3 = warp_max_nonnan(se);
  for (int o = 16; o > 0; o >>= 1) {
    nv += __shfl_xor_sync(0xffffffffu, nv, o);
    ne += __shfl_xor_sync(0xffffffffu, ne, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_max_nonneg(&dyn->cmax_bits, (double)m);
    atomic_max_nonneg(&dyn->stat_max_bits[0], (double)a1);
    atomic_max_nonneg(&dyn->stat_max_bits[1], (double)a2);
    atomic_max_nonneg(&dyn->stat_max_bits[2], (double)a3);
    if (nv) atomicAdd(&dyn->stat_cnt[0], nv);
    if (ne) atomicAdd(&dyn->stat_cnt[1], ne);
  }
}

// Adjust_Valf_Max statistics over the interior of a primitive state
// (src/Adjust_Valf_Max.C:58-81).
template <class R>
__global__ void k_adjust_stats(Consts c, const R* __restrict__ U, const R* __restrict__ P, Dyn* __restrict__ dyn) {
  const Geom& g = c.g;
  const unsigned n = (unsigned)g.nx * (unsigned)g.ny * (unsigned)g.nz, N = g.N32;
  R sv = 0, sc = 0, se = 0;
  unsigned long long nv = 0, ne = 0;
  const R vlim95 = dynr<R>(dyn).vlim95, elim95 = dynr<R>(dyn).elim95;
  for (unsigned t = gs_first(); t < n; t += gs_step()) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const unsigned id = cidx32(g, i, j, k);
    R d = U[id], v1 = U[N + id], v2 = U[2 * N + id], v3 = U[3 * N + id], ei = U[4 * N + id];
    R vabs = d_sqrt(v1 * v1 + v2 * v2 + v3 * v3);
    R ee = ei / d;
    sv = d_fmax(sv, vabs);
    sc = d_fmax(sc, (R)(5 / 3.) * P[id] / d);
    se = d_fmax(se, ee);
    if (vabs >= vlim95) nv++;
    if (ee >= elim95) ne++;
  }
  R a1 = warp_max_nonnan(sv), a2 = warp_max_nonnan(sc), a3 = warp_max_nonnan(se);
  for (int o = 16; o > 0; o >>= 1) {
    nv += __shfl_xor_sync(0xffffffffu, nv, o);
    ne += __shfl_xor_sync(0xffffffffu, ne, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_max_nonneg(&dyn->stat_max_bits[0], (double)a1);
    atomic_max_nonneg(&dyn->stat_max_bits[1], (double)a2);
    atomic_max_nonneg(&dyn->stat_max_bits[2], (double)a3);
    if (nv) atomicAdd(&dyn->stat_cnt[0], nv);
    if (ne) atomicAdd(&dyn->stat_cnt[1], ne);
  }
}

// MHD_Residual's diagnostics on an output step (src/mhdres_SR.C:368-384,
// 434-435, 689-702, 751-752), per interior cell and direction in the
// residual's order x, y, z: tvar1 += the energy-flux divergence (without the
// conduction share, which goes to tvar2) and tvar3 += the work of the
// Boris-blended Lorentz force, each formed as the residual forms it (the same
// flux, derivative and blend functions).  U: primitives as ConsToPrim leaves
// them; P: the pressure; S: the heat flux (null without conduction); diag:
// tvar1..3 at 0, N, 2N.
template <class R>
__global__ void __launch_bounds__(256) k_diag_residual(Consts c, const R* __restrict__ U, const R* __restrict__ P,
                                                       const R* __restrict__ S, R* __restrict__ diag,
                                                       const Dyn* __restrict__ dyn) {
  const Geom& g = c.g;
  const unsigned n = (unsigned)g.nx * (unsigned)g.ny * (unsigned)g.nz, N = g.N32;
  const KC<R>& k = kc<R>(c);
  const R inv_va2max = dynr<R>(dyn).inv_va2max;
  for (unsigned t = gs_first(); t < n; t += gs_step()) {
    int i, j, kk;
    interior_ijk(g, t, i, j, kk);
    const unsigned id = cidx32(g, i, j, kk);
    Raw9<R> r;
    load_raw(g, U, P, id, r);
    R cen[NF];
    prim_of_raw<R, true>(r, cen);
    cen[NPRIM] = (R)0;
    const R lf = boris_lf<R>(cen, inv_va2max);
    R t1 = diag[id], t2 = diag[N + id], t3 = diag[2 * N + id];
    auto direction = [&](auto dim) {
      constexpr int D1 = decltype(dim)::value;
      const unsigned sd = D1 == 0 ? 1u : (D1 == 1 ? (unsigned)g.sx : (unsigned)g.sx * (unsigned)g.sy);
      const unsigned nb[4] = {id - 2 * sd, id - sd, id + sd, id + 2 * sd};  // c-2, c-1, c+1, c+2
      R fl[4][NF], sb[4];
#pragma unroll
      for (int m = 0; m < 4; m++) {
        Raw9<R> rm;
        load_raw(g, U, P, nb[m], rm);
        R pm[NF];
        prim_of_raw<R, true>(rm, pm);
        pm[NPRIM] = (R)0;
        flux12<R, D1>(pm, 1, fl[m], 1);
        sb[m] = S ? S[nb[m]] * pm[P_B1 + D1] : (R)0;
      }
      R Dq[NF];
      deriv12(Dq, fl[0], fl[1], fl[2], fl[3], k.w1[D1], k.w2[D1]);
      const R w1 = k.w1[D1], w2 = k.w2[D1];
      if (S) {  // the reference's energy flux carries sflx * B_d
        const R f0 = fl[0][4] + sb[0], f1 = fl[1][4] + sb[1], f2 = fl[2][4] + sb[2], f3 = fl[3][4] + sb[3];
        const R r4 = (R)0.0 - (w1 * (f2 - f1) + w2 * (f3 - f0));
        const R dn = -(w1 * (sb[2] - sb[1]) + w2 * (sb[3] - sb[0]));
        t1 += r4 - dn;
        t2 += dn;
      } else {
        t1 += (R)0.0 - Dq[4];
      }
      const R dB2 = Dq[10], dB3 = Dq[11];
      const R Bd1 = cen[P_B1 + D1];
      const R Bd2 = cen[P_B1 + Dirs<D1>::d2], Bd3 = cen[P_B1 + Dirs<D1>::d3];
      R cbb[3];
      cbb[D1] = -Bd2 * dB2 - Bd3 * dB3;
      cbb[Dirs<D1>::d2] = Bd1 * dB2;
      cbb[Dirs<D1>::d3] = Bd1 * dB3;
      const R lrt0 = lf * Dq[7] + ((R)1.0 - lf) * cbb[0];
      const R lrt1 = lf * Dq[8] + ((R)1.0 - lf) * cbb[1];
      const R lrt2 = lf * Dq[9] + ((R)1.0 - lf) * cbb[2];
      t3 += cen[P_V1] * lrt0 + cen[P_V2] * lrt1 + cen[P_V3] * lrt2;
    };
    direction(std::integral_constant<int, 0>());
    direction(std::integral_constant<int, 1>());
    direction(std::integral_constant<int, 2>());
    diag[id] = t1;
    diag[N + id] = t2;
    diag[2 * N + id] = t3;
  }
}

// Stage-1 CFL speed of a conserved state over the interior, with the limits
// the step's Adjust_Valf_Max has just set (MHD_Residual's cmax from
// ConsToPrim's velocities, src/cons_to_prim.C:148-159, src/mhdres_SR.C:
// 310-327).  A fused step runs it only with adaptive limits (va_adjust > 0):
// the end-of-step pass's speeds used the previous step's inv_va2max, and the
// speed depends on it cell by cell.  Same expression as k_step_finish; one
// atomic per block.
template <class R>
__global__ void __launch_bounds__(256) k_cfl_cons(Consts c, const R* __restrict__ U, const R* __restrict__ P,
                                                  Dyn* __restrict__ dyn) {
  if (dyn->err) return;
  const Geom& g = c.g;
  const unsigned n = (unsigned)g.nx * (unsigned)g.ny * (unsigned)g.nz, N = g.N32;
  const R inv_va2max = dynr<R>(dyn).inv_va2max;
  R cm = (R)0;
  for (unsigned t = gs_first(); t < n; t += gs_step()) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const unsigned id = cidx32(g, i, j, k);
    const R d = U[id];
    R v1, v2, v3, ei;
    prim_from_cons(d, U[N + id], U[2 * N + id], U[3 * N + id], U[4 * N + id], v1, v2, v3, ei);
    cm = smax(cm, cmax_cell<R>(d, v1, v2, v3, U[5 * N + id], U[6 * N + id], U[7 * N + id], P[id], inv_va2max));
  }
  const R m = block_max_nonnan(cm);
  if (threadIdx.x == 0) atomic_max_nonneg(&dyn->cmax_bits, (double)m);
}

// CFL speed on the face ghost cells the residual's pencils include
// (one coordinate in the ghost range, the other two interior).
template <class R>
__global__ void k_cmax_faces(Consts c, const R* __restrict__ U, const R* __restrict__ P, Dyn* __restrict__ dyn) {
  const Geom& g = c.g;
  const long long nfx = 2LL * GH * g.ny * g.nz, nfy = 2LL * GH * g.nx * g.nz, nfz = 2LL * GH * g.nx * g.ny;
  const R inv_va2max = dynr<R>(dyn).inv_va2max;
  R cm = 0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nfx + nfy + nfz; t += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    if (t < nfx) {
      int q = (int)(t % (2 * GH)); long long r = t / (2 * GH);
      i = q < GH ? q : g.nx + q; j = GH + (int)(r % g.ny); k = GH + (int)(r / g.ny);
    } else if (t < nfx + nfy) {
      long long u = t - nfx; int q = (int)(u % (2 * GH)); long long r = u / (2 * GH);
      j = q < GH ? q : g.ny + q; i = GH + (int)(r % g.nx); k = GH + (int)(r / g.nx);
    } else {
      long long u = t - nfx - nfy; int q = (int)(u % (2 * GH)); long long r = u / (2 * GH);
      k = q < GH ? q : g.nz + q; i = GH + (int)(r % g.nx); j = GH + (int)(r / g.nx);
    }
    const long long id = cidx(g, i, j, k);
    cm = smax(cm, cmax_cell<R>(U[id], U[g.N + id], U[2 * g.N + id], U[3 * g.N + id], U[5 * g.N + id], U[6 * g.N + id],
                               U[7 * g.N + id], P[id], inv_va2max));
  }
  R m = warp_max_nonnan(cm);
  if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&dyn->cmax_bits, (double)m);
}

// Source_Integrate_Tcheck (src/Add_Sources_Integrate_SR.C:297-467) on a primitive U.
// diag (an output step, else null): tvar4 = the radiation factor, tvar5 = the
// gravity work, tvar6 = the Boris correction's energy, tvar7 += Tcheck's
// energy change * invdt (src/Add_Sources_Integrate_SR.C:122-296).
template <class R>
__global__ void __launch_bounds__(256, EwBlocks<R>::v) k_source_integrate(Consts c, R* __restrict__ U, const R* __restrict__ U0, R* __restrict__ Res,
                                   const Dyn* __restrict__ dyn, int stage, R* __restrict__ diag, R invdt) {
  const Geom& g = c.g;
  const unsigned n = (unsigned)g.nx * (unsigned)g.ny * (unsigned)g.nz, N = g.N32;
  const DynR<R>& dr = dynr<R>(dyn);
  const R wdt = dr.wdt[stage];
  const R invRdt = dr.invRdt;
  const R inv_va2max = dr.inv_va2max;
  const R vmax = dr.vmax;
  const R emax = dr.emax;
  for (unsigned t = gs_first(); t < n; t += gs_step()) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const unsigned id = cidx32(g, i, j, k);
    R r[NV], u[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) { r[v] = Res[(unsigned)v * N + id]; u[v] = U[(unsigned)v * N + id]; }
    R dn = invRdt * u[4];
    R efaci = dn / d_fmax(dn, (R)0.0);
    dn = kc<R>(c).gx * u[0] - (R)0.0;
    R edmp = dn * u[1];
    r[1] += dn;
    r[4] += edmp + (R)0.0 * efaci;
    const R rh = u[0], rd = r[0], vx = u[1], vy = u[2], vz = u[3], bx = u[5], by = u[6], bz = u[7];
    R fx = r[1], fy = r[2], fz = r[3];
    const R bb = bx * bx + by * by + bz * bz;
    const R va2 = bb / rh;
    const R x2 = va2 * inv_va2max, x4 = x2 * x2;
    const R bf = x4 / ((R)1 + x2 + x4);
    fx -= vx * rd;
    fy -= vy * rd;
    fz -= vz * rd;
    const R q = (fx * bx + fy * by + fz * bz) / d_fmax(tiny100<R>(), bb);
    const R b0 = -bf * (fx - q * bx), b1 = -bf * (fy - q * by), b2 = -bf * (fz - q * bz);
    const R b3 = b0 * vx + b1 * vy + b2 * vz;
    r[1] += b0; r[2] += b1; r[3] += b2; r[4] += b3;
    R un[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) un[v] = U0[(unsigned)v * N + id] + wdt * r[v];
    // Res is zero for the next MHD_Residual: the host marks it so and the
    // next residual writes it without reading it (no pass stores the zeros)
    const R ee = un[4];
    tcheck_cell<R>(c, vmax, emax, un[0], un[1], un[2], un[3], un[4]);
    if (diag) {
      diag[3 * N + id] = efaci;
      diag[4 * N + id] = edmp;
      diag[5 * N + id] = b3;
      diag[6 * N + id] += (un[4] - ee) * invdt;
    }
#pragma unroll
    for (int v = 0; v < NV; v++) U[(unsigned)v * N + id] = un[v];
  }
}

template <class R>
__global__ void k_save_cons(Geom g, const R* __restrict__ U, R* __restrict__ U0) {
  const unsigned n = (unsigned)g.nx * (unsigned)g.ny * (unsigned)g.nz, N = g.N32;
  for (unsigned t = gs_first(); t < n; t += gs_step()) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const unsigned id = cidx32(g, i, j, k);
#pragma unroll
    for (int v = 0; v < NV; v++) U0[(unsigned)v * N + id] = U[(unsigned)v * N + id];
  }
}

// diag (an output step, else null): tvar7 += the energy change * invdt
// (src/Add_Sources_Integrate_SR.C:560-564, 618-620).
template <class R>
__global__ void k_tcheck(Consts c, R* __restrict__ U, const Dyn* __restrict__ dyn, R* __restrict__ diag, R invdt) {
  const Geom& g = c.g;
  const unsigned n = (unsigned)g.nx * (unsigned)g.ny * (unsigned)g.nz, N = g.N32;
  const R vmax = dynr<R>(dyn).vmax;
  const R emax = dynr<R>(dyn).emax;
  for (unsigned t = gs_first(); t < n; t += gs_step()) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const unsigned id = cidx32(g, i, j, k);
    R d = U[id], m1 = U[N + id], m2 = U[2 * N + id], m3 = U[3 * N + id], e = U[4 * N + id];
    const R eei = e;
    tcheck_cell<R>(c, vmax, emax, d, m1, m2, m3, e);
    U[id] = d; U[N + id] = m1; U[2 * N + id] = m2; U[3 * N + id] = m3; U[4 * N + id] = e;
    if (diag) diag[6 * N + id] += (e - eei) * invdt;
  }
}

// Ghost fill: each ghost cell takes the value of the interior cell it images
// (periodic wrap; for closed x with with_bc, mirror with M_x, B_y, B_z flipped).
// Without with_bc a closed x leaves the x ghosts and the y/z ghosts outside the
// interior x range untouched, like exchange_grid_acc without the boundary call.
// Interior of a box filled by periodic tiling of a smaller box's interior
// (benchmark and test set-up): cell (i, j, k) takes the source cell
// (i mod nx_s, j mod ny_s, k mod nz_s).  Ghosts are filled afterwards.
template <class R>
__global__ void k_tile_state(Geom gd, Geom gs, const R* __restrict__ Us, R* __restrict__ Ud) {
  const long long n = (long long)gd.nx * gd.ny * gd.nz;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % gd.nx);
    const long long r = t / gd.nx;
    const int j = (int)(r % gd.ny), k = (int)(r / gd.ny);
    const long long d = cidx(gd, GH + i, GH + j, GH + k);
    const long long sidx = cidx(gs, GH + i % gs.nx, GH + j % gs.ny, GH + k % gs.nz);
#pragma unroll
    for (int q = 0; q < NV; q++) Ud[(long long)q * gd.N + d] = Us[(long long)q * gs.N + sidx];
  }
}

template <class R>
__global__ void k_fill_ghosts(Geom g, R* __restrict__ U, int nfield, int with_bc) {
  const unsigned N = g.N32;
  // the ghost nodes only, in three x-fastest groups: the z-ghost planes, the
  // y-ghost rows of interior planes, the x-ghost nodes of interior rows
  const unsigned sx = (unsigned)g.sx, sy = (unsigned)g.sy;
  const unsigned nA = 2u * GH * sx * sy;
  const unsigned nB = 2u * GH * sx * (unsigned)g.nz;
  const unsigned nC = 2u * GH * (unsigned)g.ny * (unsigned)g.nz;
  for (unsigned t = gs_first(); t < nA + nB + nC; t += gs_step()) {
    int i, j, k;
    if (t < nA) {
      const unsigned q = t / sx, p = q / sy;
      i = (int)(t - q * sx);
      j = (int)(q - p * sy);
      k = p < (unsigned)GH ? (int)p : (int)p + g.nz;
    } else if (t < nA + nB) {
      const unsigned u = t - nA, q = u / sx, jj = q % (2u * GH);
      i = (int)(u - q * sx);
      j = jj < (unsigned)GH ? (int)jj : (int)jj + g.ny;
      k = GH + (int)(q / (2u * GH));
    } else {
      const unsigned u = t - nA - nB, ii = u % (2u * GH), q = u / (2u * GH);
      i = ii < (unsigned)GH ? (int)ii : (int)ii + g.nx;
      j = GH + (int)(q % (unsigned)g.ny);
      k = GH + (int)(q / (unsigned)g.ny);
    }
    const unsigned id = cidx32(g, i, j, k);
    const bool gx = (i < GH || i >= GH + g.nx), gy = (j < GH || j >= GH + g.ny), gz = (k < GH || k >= GH + g.nz);
    bool flip = false;
    if (gx) {
      if (g.periodic_x) i = i < GH ? i + g.nx : i - g.nx;
      else if (with_bc && g.xmirror) { i = i < GH ? 2 * GH - 1 - i : 2 * GH + 2 * g.nx - 1 - i; flip = true; }
      else continue;
    }
    if (gy) j = j < GH ? j + g.ny : j - g.ny;
    if (gz) k = k < GH ? k + g.nz : k - g.nz;
    const unsigned src = cidx32(g, i, j, k);
    for (int v = 0; v < nfield; v++) {
      R x = U[(unsigned)v * N + src];
      if (flip && (v == 1 || v == 6 || v == 7)) x = -x;
      U[(unsigned)v * N + id] = x;
    }
  }
}

// Host cState (AoS, double) <-> device SoA (R)
template <class R, class H>
__global__ void k_aos_to_soa(long long N, int nf, const H* __restrict__ A, R* __restrict__ S) {
  for (long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < N; id += (long long)gridDim.x * blockDim.x)
    for (int v = 0; v < nf; v++) S[(long long)v * N + id] = (R)A[id * nf + v];
}
template <class R, class H>
__global__ void k_soa_to_aos(long long N, int nf, const R* __restrict__ S, H* __restrict__ A) {
  for (long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < N; id += (long long)gridDim.x * blockDim.x)
    for (int v = 0; v < nf; v++) A[id * nf + v] = (H)S[(long long)v * N + id];
}

}  // namespace gpumhd
