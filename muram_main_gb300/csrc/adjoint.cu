// Adjoint (reverse-mode) kernels of one fused MHD step, FP64, periodic box.
//
// The step is U0 -> four RK stages (residual MHD_Residual, sources and Boris
// correction, update from U0, Tcheck, ghost fill) -> three TVD sweeps (the last
// with TCheck).  Its adjoint runs the same pieces backwards.  The stencil
// structure -- which cell's output depends on which neighbours, the transposes
// of the fourth-order differences and of the TVD interface fluxes -- is
// written out here; the Jacobians of the cell-local functions (fluxes,
// residual assembly, sources, Tcheck, EOS pressure, the TVD cell quantities,
// slopes, interface flux and update) come from forward-mode dual numbers run
// through the same templates the forward kernels use, so both always agree.
// Limiter kinks and clamps take the derivative of the branch the forward step
// took (one-sided subgradients).
//
// Adjoint fields live on the interior only (nx*ny*nz per variable, x fastest)
// with periodic neighbours; forward fields are the ghost-filled arrays the
// forward kernels wrote.  Compiled without FMA contraction like the FP64
// forward kernels, so the recomputed forward values equal the forward run's.
#include "gpumhd_adjoint.cuh"
#include "gpumhd_dual.cuh"

namespace gpumhd {
namespace adj {

using D1 = Dual<1>;

struct Box {
  int nx, ny, nz;
  long long n;  // interior cells
};

__device__ __forceinline__ int wrap(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }
__device__ __forceinline__ long long lin(const Box& b, int i, int j, int k) {
  return (long long)i + (long long)b.nx * ((long long)j + (long long)b.ny * (long long)k);
}
// forward array offset of interior cell (i, j, k); i, j, k may reach two
// cells into the ghosts
__device__ __forceinline__ long long fwd(const Geom& g, int i, int j, int k) { return cidx(g, GH + i, GH + j, GH + k); }

__device__ __forceinline__ void raw_at(const Geom& g, const double* U, const double* P, long long id, Raw9<double>& r) {
#pragma unroll
  for (int q = 0; q < NV; q++) r.v[q] = U[(long long)q * g.N + id];
  r.v[8] = P[id];
}

template <int K>
__device__ __forceinline__ void to_dual(const double* x, Dual<K>* y, int m) {
  for (int q = 0; q < m; q++) y[q] = Dual<K>(x[q]);
}

// ------------------------------------------------------------- stage, part A
// Per cell c: recompute the stage's forward residual G(c) and pre-Tcheck state
// U0 + wdt*G, then: lamU0 += Tcheck^T lam_out; from lam_G = wdt * that, the
// adjoints of the three directions' derivative vectors Dq_d(c) (bufDq, 36
// per cell) and of the cell's own primitives (bufWc, 11 per cell).
__global__ void k_stage_a(Consts c, const Dyn* dyn, Box b, const double* __restrict__ Uin,
                          const double* __restrict__ Pin, const double* __restrict__ U0,
                          const double* __restrict__ lam_out, double* __restrict__ lam_u0,
                          double* __restrict__ buf_dq, double* __restrict__ buf_wc, int stage) {
  const Geom& g = c.g;
  const KC<double>& k = c.kd;
  const DynR<double>& dr = dyn->rd;
  const double inv_va2max = dr.inv_va2max, invRdt = dr.invRdt, vmax = dr.vmax, emax = dr.emax;
  const double wdt = dr.wdt[stage];
  for (long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x; li < b.n;
       li += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(li % b.nx), j = (int)((li / b.nx) % b.ny), kk = (int)(li / ((long long)b.nx * b.ny));
    double cen[NF];
    Raw9<double> r;
    raw_at(g, Uin, Pin, fwd(g, i, j, kk), r);
    prim_of_raw<double, false>(r, cen);
    cen[NPRIM] = 0.0;
    // derivative vectors of the three directions, as the forward computes them
    double Dq[3][NF];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      double f[4][NF];
      const int off[4] = {-2, -1, 1, 2};
#pragma unroll
      for (int s = 0; s < 4; s++) {
        const int ii = i + (d == 0 ? off[s] : 0), jj = j + (d == 1 ? off[s] : 0), zz = kk + (d == 2 ? off[s] : 0);
        double w[NF];
        Raw9<double> rn;
        raw_at(g, Uin, Pin, fwd(g, ii, jj, zz), rn);
        prim_of_raw<double, false>(rn, w);
        w[NPRIM] = 0.0;
        if (d == 0) flux12<double, 0>(w, 1, f[s], 1);
        else if (d == 1) flux12<double, 1>(w, 1, f[s], 1);
        else flux12<double, 2>(w, 1, f[s], 1);
      }
      for (int q = 0; q < NF; q++) Dq[d][q] = k.w1[d] * (f[2][q] - f[1][q]) + k.w2[d] * (f[3][q] - f[0][q]);
    }
    const double lf = boris_lf<double>(cen, inv_va2max);
    double R[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) R[q] = 0.0;
    apply_direction<double, 0>(R, Dq[0], cen, lf);
    apply_direction<double, 1>(R, Dq[1], cen, lf);
    apply_direction<double, 2>(R, Dq[2], cen, lf);
    double G[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) G[q] = R[q];
    stage_sources<double>(G, cen, k.gx, inv_va2max, invRdt);
    const long long id = fwd(g, i, j, kk);
    double pre[NV], lo[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) {
      pre[q] = U0[(long long)q * g.N + id] + wdt * G[q];
      lo[q] = lam_out[(long long)q * b.n + li];
    }
    // Tcheck (density, momentum, energy) transposed; the field passes through
    double lp[NV];
    for (int q = 5; q < NV; q++) lp[q] = lo[q];
    for (int q = 0; q < 5; q++) {
      D1 x[5];
      to_dual(pre, x, 5);
      x[q].d[0] = 1.0;
      tcheck_cell<D1>(c, D1(vmax), D1(emax), x[0], x[1], x[2], x[3], x[4]);
      double s = 0.0;
      for (int o = 0; o < 5; o++) s += x[o].d[0] * lo[o];
      lp[q] = s;
    }
#pragma unroll
    for (int q = 0; q < NV; q++) lam_u0[(long long)q * b.n + li] += lp[q];
    double lg[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) lg[q] = wdt * lp[q];
    // sources and Boris correction: G = sources(R, cen)
    double lR[NV], lcen[NF];
    for (int q = 0; q < NF; q++) lcen[q] = 0.0;
    for (int q = 0; q < NV + 8; q++) {
      D1 Ra[NV], cd[NF];
      to_dual(R, Ra, NV);
      to_dual(cen, cd, NF);
      const int cq[8] = {P_D, P_V1, P_V2, P_V3, P_EI, P_B1, P_B2, P_B3};
      if (q < NV) Ra[q].d[0] = 1.0;
      else cd[cq[q - NV]].d[0] = 1.0;
      stage_sources<D1>(Ra, cd, D1(k.gx), D1(inv_va2max), D1(invRdt));
      double s = 0.0;
      for (int o = 0; o < NV; o++) s += Ra[o].d[0] * lg[o];
      if (q < NV) lR[q] = s;
      else lcen[cq[q - NV]] += s;
    }
    // residual assembly per direction: R += res_d(Dq_d, cen, lf)
    double llf = 0.0;
    const int cu[6] = {P_V1, P_V2, P_V3, P_B1, P_B2, P_B3};
#pragma unroll
    for (int d = 0; d < 3; d++) {
      for (int q = 0; q < NF + 7; q++) {
        D1 acc[NV], dq[NF], cd[NF], lfd(lf);
        for (int o = 0; o < NV; o++) acc[o] = D1(0.0);
        to_dual(Dq[d], dq, NF);
        to_dual(cen, cd, NF);
        if (q < NF) dq[q].d[0] = 1.0;
        else if (q < NF + 6) cd[cu[q - NF]].d[0] = 1.0;
        else lfd.d[0] = 1.0;
        if (d == 0) apply_direction<D1, 0>(acc, dq, cd, lfd);
        else if (d == 1) apply_direction<D1, 1>(acc, dq, cd, lfd);
        else apply_direction<D1, 2>(acc, dq, cd, lfd);
        double s = 0.0;
        for (int o = 0; o < NV; o++) s += acc[o].d[0] * lR[o];
        if (q < NF) buf_dq[(long long)(d * NF + q) * b.n + li] = s;
        else if (q < NF + 6) lcen[cu[q - NF]] += s;
        else llf += s;
      }
    }
    // Boris factor from the cell's primitives
    {
      const int cb[4] = {P_D, P_B1, P_B2, P_B3};
      for (int t = 0; t < 4; t++) {
        D1 cd[NF];
        to_dual(cen, cd, NF);
        cd[cb[t]].d[0] = 1.0;
        const D1 l = boris_lf<D1>(cd, D1(inv_va2max));
        lcen[cb[t]] += l.d[0] * llf;
      }
    }
    for (int q = 0; q < NPRIM; q++) buf_wc[(long long)q * b.n + li] = lcen[q];
  }
}

// ------------------------------------------------------------- stage, part B
// Per cell n: the flux adjoints (transpose of the fourth-order differences of
// the neighbours' Dq adjoints), through flux12 and the primitive conversion to
// the stage input: lam_uin = (overwritten), lam_pin += .
__global__ void k_stage_b(Consts c, Box b, const double* __restrict__ Uin, const double* __restrict__ Pin,
                          const double* __restrict__ buf_dq, const double* __restrict__ buf_wc,
                          double* __restrict__ lam_uin, double* __restrict__ lam_pin) {
  const Geom& g = c.g;
  const KC<double>& k = c.kd;
  for (long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x; li < b.n;
       li += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(li % b.nx), j = (int)((li / b.nx) % b.ny), kk = (int)(li / ((long long)b.nx * b.ny));
    Raw9<double> r;
    raw_at(g, Uin, Pin, fwd(g, i, j, kk), r);
    double w[NF];
    prim_of_raw<double, false>(r, w);
    w[NPRIM] = 0.0;
    double lw[NF];
    for (int q = 0; q < NPRIM; q++) lw[q] = buf_wc[(long long)q * b.n + li];
    lw[NPRIM] = 0.0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      long long nb[4];
      const int off[4] = {-2, -1, 1, 2};
      for (int s = 0; s < 4; s++) {
        const int ii = d == 0 ? wrap(i + off[s], b.nx) : i, jj = d == 1 ? wrap(j + off[s], b.ny) : j;
        const int zz = d == 2 ? wrap(kk + off[s], b.nz) : kk;
        nb[s] = lin(b, ii, jj, zz);
      }
      double lF[NF];
      for (int q = 0; q < NF; q++) {
        const double* B = buf_dq + (long long)(d * NF + q) * b.n;
        lF[q] = k.w1[d] * (B[nb[1]] - B[nb[2]]) + k.w2[d] * (B[nb[0]] - B[nb[3]]);
      }
      for (int q = 0; q < NPRIM; q++) {
        D1 wd[NF], f[NF];
        to_dual(w, wd, NF);
        wd[q].d[0] = 1.0;
        if (d == 0) flux12<D1, 0>(wd, 1, f, 1);
        else if (d == 1) flux12<D1, 1>(wd, 1, f, 1);
        else flux12<D1, 2>(wd, 1, f, 1);
        double s = 0.0;
        for (int o = 0; o < NF; o++) s += f[o].d[0] * lF[o];
        lw[q] += s;
      }
    }
    for (int q = 0; q < 9; q++) {
      Raw9<D1> rd;
      for (int t = 0; t < 9; t++) rd.v[t] = D1(r.v[t]);
      rd.v[q].d[0] = 1.0;
      D1 wd[NF];
      prim_of_raw<D1, false>(rd, wd);
      double s = 0.0;
      for (int o = 0; o < NPRIM; o++) s += wd[o].d[0] * lw[o];
      if (q < NV) lam_uin[(long long)q * b.n + li] = s;
      else lam_pin[li] += s;
    }
  }
}

// --------------------------------------------------------------- EOS pressure
// lam_u += (dp/dU)^T lam_p, p = ConsToPrim's pressure of the conserved state U.
__global__ void k_eos(Consts c, Box b, const double* __restrict__ U, const double* __restrict__ lam_p,
                      double* __restrict__ lam_u) {
  const Geom& g = c.g;
  for (long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x; li < b.n;
       li += (long long)gridDim.x * blockDim.x) {
    const double lp = lam_p[li];
    if (lp == 0.0) continue;
    const int i = (int)(li % b.nx), j = (int)((li / b.nx) % b.ny), kk = (int)(li / ((long long)b.nx * b.ny));
    const long long id = fwd(g, i, j, kk);
    double u[5];
    for (int q = 0; q < 5; q++) u[q] = U[(long long)q * g.N + id];
    for (int q = 0; q < 5; q++) {
      D1 x[5];
      to_dual(u, x, 5);
      x[q].d[0] = 1.0;
      D1 v1, v2, v3, ei;
      prim_from_cons(x[0], x[1], x[2], x[3], x[4], v1, v2, v3, ei);
      const D1 p = eos_pres_t<D1>(c, x[0], ei, 1.0 / x[0]);
      lam_u[(long long)q * b.n + li] += p.d[0] * lp;
    }
  }
}

// ----------------------------------------------------------------- TVD sweeps
// TCell fields in declaration order: q[0..7], cm 8, he 9, hv 10, hB 11, BC2 12,
// bsqr 13, vsqr 14, hd 15, hb 16, ht 17, qt 18.
constexpr int NT = 19;
enum { T_CM = 8, T_HE = 9, T_HV = 10, T_HB = 11, T_BC2 = 12, T_BSQR = 13, T_VSQR = 14, T_HD = 15, T_HBOT = 16,
       T_HTOP = 17, T_QT = 18 };
template <class R> __device__ __forceinline__ R* tf(TCell<R>& t) { return reinterpret_cast<R*>(&t); }
template <class R> __device__ __forceinline__ const R* tf(const TCell<R>& t) { return reinterpret_cast<const R*>(&t); }

__device__ __forceinline__ TCell<D1> dual_cell(const TCell<double>& t) {
  TCell<D1> o;
  for (int f = 0; f < NT; f++) tf(o)[f] = D1(tf(t)[f]);
  return o;
}

struct Sweep {
  double dtt, cmax_t, fac0, inv_va2max, vsqr_diff;
  bool hyper;
  int istart, sz;
};

template <int DIR>
__device__ __forceinline__ Sweep sweep_of(const Consts& c, const Dyn* dyn) {
  Sweep s;
  const DynR<double>& dr = dyn->rd;
  s.dtt = dr.dt_tvd;
  s.cmax_t = dr.cmax_t[DIR];
  s.fac0 = dr.fac0[DIR];
  s.inv_va2max = dr.inv_va2max;
  s.vsqr_diff = dr.vsqr_diff;
  s.hyper = (DIR == 0) && c.kd.has_vhyp;
  s.istart = 1 + (c.g.periodic_x ? 0 : GH);
  s.sz = (DIR == 0 ? c.g.nx : (DIR == 1 ? c.g.ny : c.g.nz)) + 2 * GH;
  return s;
}

// forward cell quantities of the cell `o` steps along DIR from interior (i, j, k)
template <int DIR>
__device__ __forceinline__ void cell_at(const Consts& c, const Sweep& s, const double* V, const double* P, int i, int j,
                                        int k, int o, TCell<double>& t, Raw9<double>* raw = nullptr) {
  const Geom& g = c.g;
  const int ii = i + (DIR == 0 ? o : 0), jj = j + (DIR == 1 ? o : 0), kk = k + (DIR == 2 ? o : 0);
  Raw9<double> r;
  raw_at(g, V, P, fwd(g, ii, jj, kk), r);
  if (raw) *raw = r;
  const int xi = GH + ii;  // the boundary profiles depend on x
  tvd_cell<double>(c, r, c.kd.hfb[xi], c.kd.hft[xi], c.kd.qft[xi], s.cmax_t, s.fac0, s.hyper, s.inv_va2max, t);
}

template <int DIR>
__device__ __forceinline__ long long nbr(const Box& b, int i, int j, int k, int o) {
  if (DIR == 0) return lin(b, wrap(i + o, b.nx), j, k);
  if (DIR == 1) return lin(b, i, wrap(j + o, b.ny), k);
  return lin(b, i, j, wrap(k + o, b.nz));
}
__device__ __forceinline__ void ijk(const Box& b, long long li, int& i, int& j, int& k) {
  i = (int)(li % b.nx);
  j = (int)((li / b.nx) % b.ny);
  k = (int)(li / ((long long)b.nx * b.ny));
}
// memory index along the sweep of interior position p (for the flux's boundary tests)
template <int DIR> __device__ __forceinline__ int pos_of(int i, int j, int k) {
  return GH + (DIR == 0 ? i : (DIR == 1 ? j : k));
}

// T1: per cell i, the update transposed.  Outputs: lam_in_direct (8), the
// adjoint of the cell's TCell (19), and of its right / left interface fluxes
// and heating terms (9 + 9).
template <int DIR>
__global__ void k_tvd_t1(Consts c, const Dyn* dyn, Box b, const double* __restrict__ V, const double* __restrict__ P,
                         const double* __restrict__ lam_out, int final_pass, double* __restrict__ o_in,
                         double* __restrict__ o_cell, double* __restrict__ o_fp, double* __restrict__ o_fm) {
  const Sweep s = sweep_of<DIR>(c, dyn);
  const DynR<double>& dr = dyn->rd;
  for (long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x; li < b.n;
       li += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    ijk(b, li, i, j, k);
    TCell<double> T[5];
    Raw9<double> r0;
    for (int o = -2; o <= 2; o++) cell_at<DIR>(c, s, V, P, i, j, k, o, T[o + 2], o == 0 ? &r0 : nullptr);
    double sl[3][NV];
    for (int o = 0; o < 3; o++) tvd_slope<double>(c, T[o], T[o + 1], T[o + 2], s.vsqr_diff, sl[o]);
    const int p = pos_of<DIR>(i, j, k);
    double Fm[NV], Fp[NV], qm, qp;
    tvd_flux<double, DIR>(c, T[0], T[1], T[2], T[3], sl[0], sl[1], p - 1, s.sz, s.fac0, s.cmax_t, s.hyper, s.istart,
                          Fm, qm);
    tvd_flux<double, DIR>(c, T[1], T[2], T[3], T[4], sl[1], sl[2], p, s.sz, s.fac0, s.cmax_t, s.hyper, s.istart, Fp,
                          qp);
    double lo[NV];
    for (int q = 0; q < NV; q++) lo[q] = lam_out[(long long)q * b.n + li];
    if (final_pass) {
      // TCheck of the final sweep, transposed
      double u[NV];
      tvd_update<double>(c, s.dtt, Fp, Fm, qp, qm, T[2], r0.v, u);
      double l5[5];
      for (int q = 0; q < 5; q++) {
        D1 x[5];
        to_dual(u, x, 5);
        x[q].d[0] = 1.0;
        tcheck_cell<D1>(c, D1(dr.vmax), D1(dr.emax), x[0], x[1], x[2], x[3], x[4]);
        double acc = 0.0;
        for (int o = 0; o < 5; o++) acc += x[o].d[0] * lo[o];
        l5[q] = acc;
      }
      for (int q = 0; q < 5; q++) lo[q] = l5[q];
    }
    // inputs of tvd_update: u_in (8), c0 {q 0..7, BC2, bsqr, qt}, Fp (8), Fm (8), qp, qm
    const int cf[11] = {0, 1, 2, 3, 4, 5, 6, 7, T_BC2, T_BSQR, T_QT};
    for (int q = 0; q < 37; q++) {
      D1 ui[NV], fp[NV], fm[NV], u[NV];
      D1 qpd(qp), qmd(qm);
      to_dual(r0.v, ui, NV);
      to_dual(Fp, fp, NV);
      to_dual(Fm, fm, NV);
      TCell<D1> t0 = dual_cell(T[2]);
      if (q < 8) ui[q].d[0] = 1.0;
      else if (q < 19) tf(t0)[cf[q - 8]].d[0] = 1.0;
      else if (q < 27) fp[q - 19].d[0] = 1.0;
      else if (q < 35) fm[q - 27].d[0] = 1.0;
      else if (q == 35) qpd.d[0] = 1.0;
      else qmd.d[0] = 1.0;
      tvd_update<D1>(c, D1(s.dtt), fp, fm, qpd, qmd, t0, ui, u);
      double acc = 0.0;
      for (int o = 0; o < NV; o++) acc += u[o].d[0] * lo[o];
      if (q < 8) o_in[(long long)q * b.n + li] = acc;
      else if (q < 19) o_cell[(long long)cf[q - 8] * b.n + li] = acc;
      else if (q < 27) o_fp[(long long)(q - 19) * b.n + li] = acc;
      else if (q < 35) o_fm[(long long)(q - 27) * b.n + li] = acc;
      else if (q == 35) o_fp[(long long)8 * b.n + li] = acc;
      else o_fm[(long long)8 * b.n + li] = acc;
    }
    const int unused[8] = {T_CM, T_HE, T_HV, T_HB, T_VSQR, T_HD, T_HBOT, T_HTOP};
    for (int f = 0; f < 8; f++) o_cell[(long long)unused[f] * b.n + li] = 0.0;
  }
}

// T2: per interface i+1/2 (stored at its left cell i), the interface flux
// transposed onto its four cells' TCells (am, a, b, bp: 19 each) and its two
// slopes (8 each): 92 values per interface.
template <int DIR>
__global__ void k_tvd_t2(Consts c, const Dyn* dyn, Box b, const double* __restrict__ V, const double* __restrict__ P,
                         const double* __restrict__ i_fp, const double* __restrict__ i_fm, double* __restrict__ o_if) {
  const Sweep s = sweep_of<DIR>(c, dyn);
  for (long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x; li < b.n;
       li += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    ijk(b, li, i, j, k);
    const long long lr = nbr<DIR>(b, i, j, k, 1);
    double lF[NV + 1];
    for (int q = 0; q <= NV; q++) lF[q] = i_fp[(long long)q * b.n + li] + i_fm[(long long)q * b.n + lr];
    TCell<double> T[4];
    for (int o = -1; o <= 2; o++) cell_at<DIR>(c, s, V, P, i, j, k, o, T[o + 1]);
    double sa[NV], sb[NV];
    tvd_slope<double>(c, T[0], T[1], T[2], s.vsqr_diff, sa);
    tvd_slope<double>(c, T[1], T[2], T[3], s.vsqr_diff, sb);
    const int p = pos_of<DIR>(i, j, k);
    for (int t = 0; t < 4 * NT + 2 * NV; t++) o_if[(long long)t * b.n + li] = 0.0;
    // seeds: (role, field)
    const int fa[16] = {0, 1, 2, 3, 4, 5, 6, 7, T_CM, T_HE, T_HV, T_HB, T_HD, T_HBOT, T_HTOP, T_QT};
    const int fb[10] = {0, 1, 2, 3, 4, 5, 6, 7, T_CM, T_HD};
    const int fh[3] = {0, 1, 4};
    const int nseed = 16 + 10 + 16 + (s.hyper ? 6 : 0);
    for (int q = 0; q < nseed; q++) {
      TCell<D1> am = dual_cell(T[0]), a = dual_cell(T[1]), bb = dual_cell(T[2]), bp = dual_cell(T[3]);
      D1 sad[NV], sbd[NV], F[NV], qr;
      to_dual(sa, sad, NV);
      to_dual(sb, sbd, NV);
      int role, f;
      if (q < 16) { role = 1; f = fa[q]; tf(a)[f].d[0] = 1.0; }
      else if (q < 26) { role = 2; f = fb[q - 16]; tf(bb)[f].d[0] = 1.0; }
      else if (q < 34) { role = 4; f = q - 26; sad[f].d[0] = 1.0; }
      else if (q < 42) { role = 5; f = q - 34; sbd[f].d[0] = 1.0; }
      else if (q < 45) { role = 0; f = fh[q - 42]; tf(am)[f].d[0] = 1.0; }
      else { role = 3; f = fh[q - 45]; tf(bp)[f].d[0] = 1.0; }
      tvd_flux<D1, DIR>(c, am, a, bb, bp, sad, sbd, p, s.sz, D1(s.fac0), D1(s.cmax_t), s.hyper, s.istart, F, qr);
      double acc = qr.d[0] * lF[NV];
      for (int o = 0; o < NV; o++) acc += F[o].d[0] * lF[o];
      const int slot = role < 4 ? role * NT + f : 4 * NT + (role - 4) * NV + f;
      o_if[(long long)slot * b.n + li] = acc;
    }
  }
}

// T3: per cell i, its slope transposed onto the three cells it reads
// (i-1: q; i: q, hb, ht, vsqr; i+1: q): 3 x 19 values.
template <int DIR>
__global__ void k_tvd_t3(Consts c, const Dyn* dyn, Box b, const double* __restrict__ V, const double* __restrict__ P,
                         const double* __restrict__ i_if, double* __restrict__ o_sl) {
  const Sweep s = sweep_of<DIR>(c, dyn);
  for (long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x; li < b.n;
       li += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    ijk(b, li, i, j, k);
    const long long ll = nbr<DIR>(b, i, j, k, -1);
    double ls[NV];
    for (int q = 0; q < NV; q++)
      ls[q] = i_if[(long long)(4 * NT + q) * b.n + li] + i_if[(long long)(4 * NT + NV + q) * b.n + ll];
    TCell<double> T[3];
    for (int o = -1; o <= 1; o++) cell_at<DIR>(c, s, V, P, i, j, k, o, T[o + 1]);
    for (int t = 0; t < 3 * NT; t++) o_sl[(long long)t * b.n + li] = 0.0;
    const int fc[11] = {0, 1, 2, 3, 4, 5, 6, 7, T_HBOT, T_HTOP, T_VSQR};
    for (int q = 0; q < 27; q++) {
      TCell<D1> a = dual_cell(T[0]), bb = dual_cell(T[1]), n = dual_cell(T[2]);
      int role, f;
      if (q < 8) { role = 0; f = q; tf(a)[f].d[0] = 1.0; }
      else if (q < 19) { role = 1; f = fc[q - 8]; tf(bb)[f].d[0] = 1.0; }
      else { role = 2; f = q - 19; tf(n)[f].d[0] = 1.0; }
      D1 sl[NV];
      tvd_slope<D1>(c, a, bb, n, D1(s.vsqr_diff), sl);
      double acc = 0.0;
      for (int o = 0; o < NV; o++) acc += sl[o].d[0] * ls[o];
      o_sl[(long long)(role * NT + f) * b.n + li] = acc;
    }
  }
}

// T4: per cell j, the TCell adjoint gathered from the update, the four
// interfaces and three slopes that read the cell, through the cell quantities
// to the sweep input: lam_in = direct + ..., lam_p += .
template <int DIR>
__global__ void k_tvd_t4(Consts c, const Dyn* dyn, Box b, const double* __restrict__ V, const double* __restrict__ P,
                         const double* __restrict__ i_in, const double* __restrict__ i_cell,
                         const double* __restrict__ i_if, const double* __restrict__ i_sl,
                         double* __restrict__ lam_in, double* __restrict__ lam_p) {
  const Sweep s = sweep_of<DIR>(c, dyn);
  for (long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x; li < b.n;
       li += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    ijk(b, li, i, j, k);
    const long long m1 = nbr<DIR>(b, i, j, k, -1), m2 = nbr<DIR>(b, i, j, k, -2), p1 = nbr<DIR>(b, i, j, k, 1);
    double lt[NT];
    for (int f = 0; f < NT; f++) {
      double a = i_cell[(long long)f * b.n + li];
      a += i_if[(long long)(1 * NT + f) * b.n + li];   // as a of interface j+1/2
      a += i_if[(long long)(2 * NT + f) * b.n + m1];   // as b of interface j-1/2
      a += i_if[(long long)(0 * NT + f) * b.n + p1];   // as am of interface j+3/2
      a += i_if[(long long)(3 * NT + f) * b.n + m2];   // as bp of interface j-3/2
      a += i_sl[(long long)(1 * NT + f) * b.n + li];   // middle of its own slope
      a += i_sl[(long long)(0 * NT + f) * b.n + p1];   // left cell of slope j+1
      a += i_sl[(long long)(2 * NT + f) * b.n + m1];   // right cell of slope j-1
      lt[f] = a;
    }
    Raw9<double> r;
    const Geom& g = c.g;
    raw_at(g, V, P, fwd(g, i, j, k), r);
    const int xi = GH + i;
    for (int q = 0; q < 9; q++) {
      Raw9<D1> rd;
      for (int t = 0; t < 9; t++) rd.v[t] = D1(r.v[t]);
      rd.v[q].d[0] = 1.0;
      TCell<D1> t;
      tvd_cell<D1>(c, rd, D1(c.kd.hfb[xi]), D1(c.kd.hft[xi]), D1(c.kd.qft[xi]), D1(s.cmax_t), D1(s.fac0), s.hyper,
                   D1(s.inv_va2max), t);
      double acc = 0.0;
      for (int f = 0; f < NT; f++) acc += tf(t)[f].d[0] * lt[f];
      if (q < NV) lam_in[(long long)q * b.n + li] = i_in[(long long)q * b.n + li] + acc;
      else lam_p[li] += acc;
    }
  }
}

// host cState records (8 per cell, ghosts included) <-> interior adjoint fields
__global__ void k_from_cstate(Geom g, Box b, const double* __restrict__ aos, double* __restrict__ lam) {
  for (long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x; li < b.n;
       li += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    ijk(b, li, i, j, k);
    const long long id = fwd(g, i, j, k);
    for (int q = 0; q < NV; q++) lam[(long long)q * b.n + li] = aos[id * NV + q];
  }
}
__global__ void k_to_cstate(Geom g, Box b, const double* __restrict__ lam, double* __restrict__ aos) {
  for (long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x; li < b.n;
       li += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    ijk(b, li, i, j, k);
    const long long id = fwd(g, i, j, k);
    for (int q = 0; q < NV; q++) aos[id * NV + q] = lam[(long long)q * b.n + li];
  }
}
__global__ void k_add(long long m, const double* __restrict__ x, const double* __restrict__ y, double* __restrict__ o) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (long long)gridDim.x * blockDim.x)
    o[t] = x[t] + y[t];
}

}  // namespace adj

// ------------------------------------------------------------------ launchers
static inline int adj_grid(long long n) {
  long long bl = (n + 127) / 128;
  if (bl > 152LL * 64) bl = 152LL * 64;
  return (int)(bl < 1 ? 1 : bl);
}

static adj::Box box_of(const Consts& c) {
  adj::Box b;
  b.nx = c.g.nx;
  b.ny = c.g.ny;
  b.nz = c.g.nz;
  b.n = (long long)b.nx * b.ny * b.nz;
  return b;
}

void adjoint_stage(const Consts& c, const Dyn* dyn, const double* Uin, const double* Pin, const double* U0,
                   const double* lam_out, double* lam_u0, double* lam_uin, double* lam_pin, double* buf_dq,
                   double* buf_wc, int stage, cudaStream_t s) {
  const adj::Box b = box_of(c);
  adj::k_stage_a<<<adj_grid(b.n), 128, 0, s>>>(c, dyn, b, Uin, Pin, U0, lam_out, lam_u0, buf_dq, buf_wc, stage);
  adj::k_stage_b<<<adj_grid(b.n), 128, 0, s>>>(c, b, Uin, Pin, buf_dq, buf_wc, lam_uin, lam_pin);
}

void adjoint_eos(const Consts& c, const double* U, const double* lam_p, double* lam_u, cudaStream_t s) {
  const adj::Box b = box_of(c);
  adj::k_eos<<<adj_grid(b.n), 128, 0, s>>>(c, b, U, lam_p, lam_u);
}

template <int DIR>
static void tvd_dir(const Consts& c, const Dyn* dyn, const adj::Box& b, const double* V, const double* P,
                    const double* lam_out, int final_pass, double* lam_in, double* lam_p, const AdjTvdScratch& w,
                    cudaStream_t s) {
  const int gr = adj_grid(b.n);
  adj::k_tvd_t1<DIR><<<gr, 128, 0, s>>>(c, dyn, b, V, P, lam_out, final_pass, w.in, w.cell, w.fp, w.fm);
  adj::k_tvd_t2<DIR><<<gr, 128, 0, s>>>(c, dyn, b, V, P, w.fp, w.fm, w.iface);
  adj::k_tvd_t3<DIR><<<gr, 128, 0, s>>>(c, dyn, b, V, P, w.iface, w.slope);
  adj::k_tvd_t4<DIR><<<gr, 128, 0, s>>>(c, dyn, b, V, P, w.in, w.cell, w.iface, w.slope, lam_in, lam_p);
}

void adjoint_tvd(const Consts& c, const Dyn* dyn, int dir, const double* V, const double* P, const double* lam_out,
                 int final_pass, double* lam_in, double* lam_p, const AdjTvdScratch& w, cudaStream_t s) {
  const adj::Box b = box_of(c);
  if (dir == 0) tvd_dir<0>(c, dyn, b, V, P, lam_out, final_pass, lam_in, lam_p, w, s);
  else if (dir == 1) tvd_dir<1>(c, dyn, b, V, P, lam_out, final_pass, lam_in, lam_p, w, s);
  else tvd_dir<2>(c, dyn, b, V, P, lam_out, final_pass, lam_in, lam_p, w, s);
}

void adjoint_from_cstate(const Consts& c, const double* aos, double* lam, cudaStream_t s) {
  const adj::Box b = box_of(c);
  adj::k_from_cstate<<<adj_grid(b.n), 128, 0, s>>>(c.g, b, aos, lam);
}
void adjoint_to_cstate(const Consts& c, const double* lam, double* aos, cudaStream_t s) {
  const adj::Box b = box_of(c);
  adj::k_to_cstate<<<adj_grid(b.n), 128, 0, s>>>(c.g, b, lam, aos);
}
void adjoint_add(const Consts& c, const double* x, const double* y, double* out, cudaStream_t s) {
  const adj::Box b = box_of(c);
  adj::k_add<<<adj_grid(8 * b.n), 128, 0, s>>>(8 * b.n, x, y, out);
}

}  // namespace gpumhd
