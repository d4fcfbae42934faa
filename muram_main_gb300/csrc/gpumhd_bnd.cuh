// MURaM's physical x boundaries (SetBoundaryConditions without the
// potential-field top, src/boundary_pdmp_1_fftw3.C:81-565) on the device.
//
// Bottom (open): the ghost pressures are extrapolated exponentially from the
// mean pressure of the two first interior layers to p_bc, with the cell's
// pressure fluctuation damped (p1_dmp = 0.8) and the magnetic pressure kept;
// entropy s_bc in upflows, the cell's own in downflows; density and internal
// energy from the inverse EOS (d3_interp, eps3_interp); momenta scaled by
// (1 - (B_x/B_crit)^4) / (1 + (B_x/B_crit)^4).  Top: M_x mirrored (always,
// or only in downflows with bnd_top = 1), B_y and B_z mirrored, the internal
// energy fixed at eps_top when positive.  Both cover the y and z ghost
// columns, which the periodic images filled before.
//
// Three launches: sums over the first two layers per block of columns (the
// two mean pressures, and on the first call the sums that set p_bc and
// s_bc), their total, then the ghost columns (one thread per column and
// side).  The arithmetic is FP64 in both precisions: in float, the bilinear
// sums over tables divided by the cell area lose ~1e-6 of ln p and ln rho,
// which the ghost states carry into the interior (FP32 runs reach 2e-5 rel.
// L2 within 40 steps that way, against 5e-6 in FP64 arithmetic).  The sums are reduced in a
// fixed order, so a run repeats bit for bit; the reference sums them in
// another order (differences of an ulp in the means).  The EOS lookups are
// eos_init's (src/eos_init.C:216-343), whose bilinear terms are summed in
// another order than ConsToPrim's.
#pragma once
#include "gpumhd_kernels.cuh"

namespace gpumhd {

constexpr int BND_NQ = 7;         // l5, l6 (mean pressures), b0..b4 (set_p_s_bc)
constexpr int BND_BX = 32, BND_BY = 4;
constexpr int BND_THREADS = BND_BX * BND_BY;
constexpr int BND_SETUP_THREADS = 256;

// Axes x0 + del*i as eos_init stores them (src/eos_init.C:125-146).
__device__ __forceinline__ void bnd_w(double x, double x0, double del, int i, double& lo, double& hi) {
  lo = x - (x0 + del * ((double)i));
  hi = (x0 + del * ((double)(i + 1))) - x;
}

// p_interp / s_interp (src/eos_init.C:268-343): ln p or s + ss_off
__device__ __forceinline__ double bnd_fwd(const Consts& c, const float* T, double ee, double dd) {
  const BndK<double>& b = c.bndd;
  const double ee1 = log(ee + b.eps_off);
  const double logr = log(dd);
  int i = cvt_x86((ee1 - b.eps0) * b.inv_del_eps);
  if (i < 0) i = 0;
  if (i > c.N_eps - 2) i = c.N_eps - 2;
  int j = cvt_x86((logr - b.lr0) * b.inv_del_lr);
  if (j < 0) j = 0;
  if (j > c.N_lr - 2) j = c.N_lr - 2;
  double we0, we1, wr0, wr1;
  bnd_w(ee1, b.eps0, b.del_eps, i, we0, we1);
  bnd_w(logr, b.lr0, b.del_lr, j, wr0, wr1);
  const long long L = c.N_lr;
  return wr0 * we0 * (double)T[(i + 1) * L + j + 1] + wr0 * we1 * (double)T[i * L + j + 1] +
         wr1 * we0 * (double)T[(i + 1) * L + j] + wr1 * we1 * (double)T[i * L + j];
}
// The same two lookups as bnd_fwd on two tables (ln p and s + ss_off) at one
// (ee, dd): logs, cell and weights formed once, each sum as bnd_fwd's.
__device__ __forceinline__ void bnd_fwd2(const Consts& c, const float* T1, const float* T2, double ee, double dd,
                                         double& o1, double& o2) {
  const BndK<double>& b = c.bndd;
  const double ee1 = log(ee + b.eps_off);
  const double logr = log(dd);
  int i = cvt_x86((ee1 - b.eps0) * b.inv_del_eps);
  if (i < 0) i = 0;
  if (i > c.N_eps - 2) i = c.N_eps - 2;
  int j = cvt_x86((logr - b.lr0) * b.inv_del_lr);
  if (j < 0) j = 0;
  if (j > c.N_lr - 2) j = c.N_lr - 2;
  double we0, we1, wr0, wr1;
  bnd_w(ee1, b.eps0, b.del_eps, i, we0, we1);
  bnd_w(logr, b.lr0, b.del_lr, j, wr0, wr1);
  const long long L = c.N_lr;
  o1 = wr0 * we0 * (double)T1[(i + 1) * L + j + 1] + wr0 * we1 * (double)T1[i * L + j + 1] +
       wr1 * we0 * (double)T1[(i + 1) * L + j] + wr1 * we1 * (double)T1[i * L + j];
  o2 = wr0 * we0 * (double)T2[(i + 1) * L + j + 1] + wr0 * we1 * (double)T2[i * L + j + 1] +
       wr1 * we0 * (double)T2[(i + 1) * L + j] + wr1 * we1 * (double)T2[i * L + j];
}
__device__ __forceinline__ double bnd_p(const Consts& c, double ee, double dd) { return exp(bnd_fwd(c, c.tab[0], ee, dd)); }
__device__ __forceinline__ double bnd_s(const Consts& c, double ee, double dd) {
  return bnd_fwd(c, c.tab[2], ee, dd) - c.bndd.ss_off;
}
// d3_interp and eps3_interp (src/eos_init.C:216-266) at one (pp, ss): ln rho
// and ln(eps + eps_off), the log, cell and weights formed once for both.
__device__ __forceinline__ void bnd_inv2(const Consts& c, double pp, double ss, double& lrho, double& leps) {
  const BndK<double>& b = c.bndd;
  const double ss1 = ss + b.ss_off;
  const double logp = log(pp);
  int i = cvt_x86((logp - b.lp30) * b.inv_del_lp3);
  if (i < 0) i = 0;
  if (i > c.N_lp3 - 2) i = c.N_lp3 - 2;
  int j = cvt_x86((ss1 - b.s30) * b.inv_del_s3);
  if (j < 0) j = 0;
  if (j > c.N_s3 - 2) j = c.N_s3 - 2;
  double wp0, wp1, ws0, ws1;
  bnd_w(logp, b.lp30, b.del_lp3, i, wp0, wp1);
  bnd_w(ss1, b.s30, b.del_s3, j, ws0, ws1);
  const long long L = c.N_s3;
  const float* D = c.d3;
  const float* E = c.eps3;
  lrho = wp0 * ws0 * (double)D[(i + 1) * L + j + 1] + wp0 * ws1 * (double)D[(i + 1) * L + j] +
         wp1 * ws0 * (double)D[i * L + j + 1] + wp1 * ws1 * (double)D[i * L + j];
  leps = wp0 * ws0 * (double)E[(i + 1) * L + j + 1] + wp0 * ws1 * (double)E[(i + 1) * L + j] +
         wp1 * ws0 * (double)E[i * L + j + 1] + wp1 * ws1 * (double)E[i * L + j];
}

// Per block of 32 (y) x 4 (z) interior columns: sums over the first two
// layers' pressures (the means of src/boundary_pdmp_1_fftw3.C:157-216) and,
// before the first call, set_p_s_bc's sums (:510-538); block partials in a
// fixed order, added up by k_bc_setup.
template <class R>
__global__ void __launch_bounds__(BND_THREADS) k_bc_sums(Consts c, const R* __restrict__ U,
                                                        const Dyn* __restrict__ dyn, double* __restrict__ part) {
  if (dyn->err) return;
  const Geom& g = c.g;
  const int tid = threadIdx.x + BND_BX * threadIdx.y;
  const int j = GH + blockIdx.x * BND_BX + threadIdx.x, k = GH + blockIdx.y * BND_BY + threadIdx.y;
  const bool ini = dyn->bnd_ini != 0;
  double q[BND_NQ];
#pragma unroll
  for (int t = 0; t < BND_NQ; t++) q[t] = 0.0;
  if (j < GH + g.ny && k < GH + g.nz) {
    const long long c1 = cidx(g, GH, j, k), c2 = cidx(g, GH + 1, j, k);
    const double d1 = (double)U[c1], d2 = (double)U[c2];
    const double m1 = (double)U[g.N + c1], m2 = (double)U[2 * g.N + c1], m3 = (double)U[3 * g.N + c1];
    const double n1 = (double)U[g.N + c2], n2 = (double)U[2 * g.N + c2], n3 = (double)U[3 * g.N + c2];
    const double e1 = (double)U[4 * g.N + c1], e2 = (double)U[4 * g.N + c2];
    const double mm1 = m1 * m1 + m2 * m2 + m3 * m3, mm2 = n1 * n1 + n2 * n2 + n3 * n3;
    const double ea1 = e1 - 0.5 * (mm1 / d1), ea2 = e2 - 0.5 * (mm2 / d2);
    q[0] = bnd_p(c, ea1 / d1, d1);
    q[1] = bnd_p(c, ea2 / d2, d2);
    if (ini) {
      const double eb1 = e1 - 0.5 * mm1 / d1, eb2 = e2 - 0.5 * mm2 / d2;
      q[2] = bnd_p(c, eb1 / d1, d1);
      q[3] = bnd_p(c, eb2 / d2, d2);
      const double s1 = bnd_s(c, eb1 / d1, d1);
      if (m1 > 0.0) {
        q[4] = 1.0;
        q[5] = s1;
      }
      q[6] = s1;
    }
  }
  __shared__ double sh[BND_NQ][BND_THREADS];
#pragma unroll
  for (int t = 0; t < BND_NQ; t++) sh[t][tid] = q[t];
  __syncthreads();
  for (int st = BND_THREADS / 2; st > 0; st >>= 1) {
    if (tid < st)
      for (int t = 0; t < BND_NQ; t++) sh[t][tid] += sh[t][tid + st];
    __syncthreads();
  }
  if (tid < BND_NQ) part[((long long)blockIdx.y * gridDim.x + blockIdx.x) * BND_NQ + tid] = sh[tid][0];
}

// The block partials' totals (one block, fixed order), p_bc and s_bc on the
// first call (src/boundary_pdmp_1_fftw3.C:540-552), and the two mean
// pressures (:205-207).  nb: number of partials.
__global__ void k_bc_setup(Consts c, Dyn* dyn, const double* __restrict__ part, int nb);

// Ghost columns: one thread per (y, z) column and side (bottom, top), ghosts
// included.  P (may be null) receives the ghosts' pressure as ConsToPrim
// forms it; with cmax the CFL speeds of the ghosts at interior (y, z) -- the
// cells MHD_Residual's x pencils reach -- join the step's maximum.
template <class R>
__global__ void __launch_bounds__(BND_THREADS) k_bc_ghosts(Consts c, R* __restrict__ U, R* __restrict__ P,
                                                          Dyn* __restrict__ dyn, int with_cmax,
                                                          R* __restrict__ sflx) {
  if (dyn->err) return;
  const Geom& g = c.g;
  const long long ncol = (long long)g.sy * g.sz;
  const long long t = (long long)blockIdx.x * BND_THREADS + threadIdx.x;
  R cm = (R)0;
  if (t < 2 * ncol) {
    const bool top = t >= ncol;
    const long long col = top ? t - ncol : t;
    const int j = (int)(col % g.sy), k = (int)(col / g.sy);
    const int lb = GH, le = GH + g.nx - 1;
    const BndK<double>& b = c.bndd;
    const bool cm_col = with_cmax && j >= GH && j < GH + g.ny && k >= GH && k < GH + g.nz;
    auto out = [&](int i, const double* u) {
      const long long id = cidx(g, i, j, k);
      R w[NV];
#pragma unroll
      for (int v = 0; v < NV; v++) {
        w[v] = (R)u[v];
        U[(long long)v * g.N + id] = w[v];
      }
      if (P || cm_col) {
        R v1, v2, v3, ei;
        prim_from_cons(w[0], w[1], w[2], w[3], w[4], v1, v2, v3, ei);
        const R pr = eos_pres(c, w[0], ei, (R)1.0 / w[0]);
        if (P) P[id] = pr;
        if (cm_col) cm = smax(cm, cmax_cell<R>(w[0], v1, v2, v3, w[5], w[6], w[7], pr, dynr<R>(dyn).inv_va2max));
      }
    };
    double u1[NV], u2[NV];
    const long long c1 = cidx(g, top ? le : lb, j, k), c2 = cidx(g, top ? le - 1 : lb + 1, j, k);
#pragma unroll
    for (int v = 0; v < NV; v++) {
      u1[v] = (double)U[(long long)v * g.N + c1];
      u2[v] = (double)U[(long long)v * g.N + c2];
    }
    if (!top) {
      // bottom (src/boundary_pdmp_1_fftw3.C:227-310)
      const double p1_dmp = 0.8;
      const double pmean1 = dyn->pmean1, pmean2 = dyn->pmean2, p_bc = dyn->p_bc, s_bc = dyn->s_bc;
      u1[4] -= 0.5 * (u1[1] * u1[1] + u1[2] * u1[2] + u1[3] * u1[3]) / u1[0];
      u2[4] -= 0.5 * (u2[1] * u2[1] + u2[2] * u2[2] + u2[3] * u2[3]) / u2[0];
      double eps1 = u1[4] / u1[0], eps2 = u2[4] / u2[0];
      const double pmag = 0.5 * u1[5] * u1[5];
      // p_interp and s_interp of the first layer share their logs and weights
      double lnp1, ss1;
      bnd_fwd2(c, c.tab[0], c.tab[2], eps1, u1[0], lnp1, ss1);
      const double pmin1 = exp(lnp1) - pmean1;
      double s1, s2;
      if (u1[1] >= 0.e0) {
        s1 = s_bc;
        s2 = s_bc;
      } else {
        s1 = ss1 - c.bndd.ss_off;
        s2 = bnd_s(c, eps2, u2[0]);
      }
      double cc = p_bc / sqrt(pmean1 * pmean2);
      double p1 = pmean1 * cc;
      double p2 = pmean1 * cc * cc;
      p1 += pmin1 * p1_dmp;
      p2 += pmin1 * p1_dmp * p1_dmp;
      p1 -= pmag * (1.0 - p1_dmp);
      p2 -= pmag * (1.0 - p1_dmp * p1_dmp);
      cc = u1[5] / b.bcrit;
      cc = (cc * cc) * (cc * cc);  // pow(cc, 4) to the last bit or two
      cc = (1.0 - cc) / (1.0 + cc);
#pragma unroll
      for (int v = 1; v <= 3; v++) {
        u1[v] *= cc;
        u2[v] *= cc;
      }
      double lr1, le1, lr2, le2;
      bnd_inv2(c, p1, s1, lr1, le1);
      bnd_inv2(c, p2, s2, lr2, le2);
      const double rho1 = exp(lr1), rho2 = exp(lr2);
      eps1 = exp(le1) - b.eps_off;
      eps2 = exp(le2) - b.eps_off;
      u1[0] = rho1;
      u2[0] = rho2;
      u1[4] = eps1 * rho1 + 0.5 * (u1[1] * u1[1] + u1[2] * u1[2] + u1[3] * u1[3]) / u1[0];
      u2[4] = eps2 * rho2 + 0.5 * (u2[1] * u2[1] + u2[2] * u2[2] + u2[3] * u2[3]) / u2[0];
      out(lb - 1, u1);
      out(lb - 2, u2);
      if (sflx) {  // heat flux: zero in the bottom ghosts (src/boundary_pdmp_1_fftw3.C:302-306)
        sflx[cidx(g, lb - 1, j, k)] = (R)0;
        sflx[cidx(g, lb - 2, j, k)] = (R)0;
      }
    } else {
      // top (src/boundary_pdmp_1_fftw3.C:398-450)
      if (c.bnd_top == 1) {
        if (u1[1] < 0.0) {
          u1[1] *= -1;
          u2[1] *= -1;
        }
      } else {
        u1[1] *= -1;
        u2[1] *= -1;
      }
      if (b.eps_top > 0.0) {
        u1[4] = b.eps_top * u1[0] + 0.5 * (u1[1] * u1[1] + u1[2] * u1[2] + u1[3] * u1[3]) / u1[0];
        u2[4] = b.eps_top * u2[0] + 0.5 * (u2[1] * u2[1] + u2[2] * u2[2] + u2[3] * u2[3]) / u2[0];
      }
      u1[6] *= -1;
      u2[6] *= -1;
      u1[7] *= -1;
      u2[7] *= -1;
      out(le + 1, u1);
      out(le + 2, u2);
      if (sflx) {  // heat flux: symmetric under a hot top, else zero in the top layers (:426-438)
        if (b.eps_top > 0.0) {
          sflx[cidx(g, le + 1, j, k)] = sflx[cidx(g, le, j, k)];
          sflx[cidx(g, le + 2, j, k)] = sflx[cidx(g, le - 1, j, k)];
        } else {
          sflx[cidx(g, le - 1, j, k)] = (R)0;
          sflx[cidx(g, le, j, k)] = (R)0;
          sflx[cidx(g, le + 1, j, k)] = (R)0;
          sflx[cidx(g, le + 2, j, k)] = (R)0;
        }
      }
    }
  }
  if (with_cmax) {
    const R m = block_max_nonnan(cm);
    if (threadIdx.x == 0) atomic_max_nonneg(&dyn->cmax_bits, (double)m);
  }
}

}  // namespace gpumhd
