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

// Reverse of apply_direction<double, D1> (eta = 0; src/mhdres_SR.C:373-412):
// lR, the adjoint of the residual it adds to, back to the direction's 12
// derivatives (l_dq, written), the cell's velocity and field (l_cen, added)
// and the Boris factor (l_lf, added).
template <int D1>
__device__ __forceinline__ void apply_direction_rev(const double* Dq, const double* cen, double lf, const double* lR,
                                                    double* l_dq, double* l_cen, double& l_lf) {
  constexpr int d2 = Dirs<D1>::d2, d3 = Dirs<D1>::d3;
  const double dB2 = Dq[10], dB3 = Dq[11];
  const double Bd1 = cen[P_B1 + D1], Bd2 = cen[P_B1 + d2], Bd3 = cen[P_B1 + d3];
  double cbb[3];
  cbb[D1] = -Bd2 * dB2 - Bd3 * dB3;
  cbb[d2] = Bd1 * dB2;
  cbb[d3] = Bd1 * dB3;
  double l_cbb[3];
  for (int i = 0; i < 3; i++) {  // lrt_i = lf*Dq[7+i] + (1-lf)*cbb_i; res[1+i] += lrt_i; res[4] += v_i*lrt_i
    const double lrt = lf * Dq[7 + i] + (1.0 - lf) * cbb[i];
    const double l_lrt = lR[1 + i] + lR[4] * cen[P_V1 + i];
    l_cen[P_V1 + i] += lR[4] * lrt;
    l_dq[7 + i] = l_lrt * lf;
    l_lf += l_lrt * (Dq[7 + i] - cbb[i]);
    l_cbb[i] = l_lrt * (1.0 - lf);
  }
  l_dq[10] = -l_cbb[D1] * Bd2 + l_cbb[d2] * Bd1;
  l_dq[11] = -l_cbb[D1] * Bd3 + l_cbb[d3] * Bd1;
  l_cen[P_B1 + d2] -= l_cbb[D1] * dB2;
  l_cen[P_B1 + d3] -= l_cbb[D1] * dB3;
  l_cen[P_B1 + D1] += l_cbb[d2] * dB2 + l_cbb[d3] * dB3;
  for (int q = 0; q < 5; q++) l_dq[q] = -lR[q];
  l_dq[5] = -lR[Dirs<D1>::fa];
  l_dq[6] = -lR[Dirs<D1>::fb];
}

// Reverse of stage_sources<double> (gravity and the Boris correction,
// src/Add_Sources_Integrate_SR.C:331-392): lG, the adjoint of the residual
// after them, back to the residual before them (l_R, written) and the cell's
// density, velocity and field (l_cen, added); every max takes the forward's
// branch.  The radiative term is zero on this path.
__device__ __forceinline__ void stage_sources_rev(const double* R, const double* cen, double gx, double inv_va2max,
                                                  const double* lG, double* l_R, double* l_cen) {
  const double tiny = tiny100<double>();
  const double rh = cen[P_D];
  const double v[3] = {cen[P_V1], cen[P_V2], cen[P_V3]}, B[3] = {cen[P_B1], cen[P_B2], cen[P_B3]};
  // ---- forward
  const double dn2 = gx * rh - 0.0;
  const double F[3] = {R[1] + dn2, R[2], R[3]};
  const double rd = R[0];
  const double bb = B[0] * B[0] + B[1] * B[1] + B[2] * B[2];
  const double va2 = bb / rh;
  const double x2 = va2 * inv_va2max, x4 = x2 * x2;
  const double D = 1.0 + x2 + x4;
  const double bf = x4 / D;
  double f[3], bo[3];
  for (int i = 0; i < 3; i++) f[i] = F[i] - v[i] * rd;
  const double bq = d_fmax(tiny, bb);
  const double q = (f[0] * B[0] + f[1] * B[1] + f[2] * B[2]) / bq;
  for (int i = 0; i < 3; i++) bo[i] = -bf * (f[i] - q * B[i]);
  // ---- reverse
  double l_v[3] = {0.0, 0.0, 0.0}, l_B[3] = {0.0, 0.0, 0.0}, l_f[3];
  double l_bf = 0.0, l_q = 0.0;
  for (int i = 0; i < 3; i++) {  // R[1+i] += bo_i, R[4] += sum bo_i * v_i, bo_i = -bf*(f_i - q*B_i)
    const double l_bo = lG[1 + i] + lG[4] * v[i];
    l_v[i] += lG[4] * bo[i];
    l_bf -= l_bo * (f[i] - q * B[i]);
    l_f[i] = -bf * l_bo;
    l_q += bf * l_bo * B[i];
    l_B[i] += bf * l_bo * q;
  }
  const double l_Nq = l_q / bq;  // q = (f . B) / max(tiny, bb)
  double l_bb = (tiny < bb) ? -l_q * q / bq : 0.0;
  for (int i = 0; i < 3; i++) {
    l_f[i] += l_Nq * B[i];
    l_B[i] += l_Nq * f[i];
  }
  double l_rd = 0.0, l_F[3];
  for (int i = 0; i < 3; i++) {  // f_i = F_i - v_i * rd
    l_F[i] = l_f[i];
    l_v[i] -= l_f[i] * rd;
    l_rd -= l_f[i] * v[i];
  }
  const double l_D = -l_bf * bf / D;  // bf = x4 / ((1 + x2) + x4)
  const double l_x4 = l_bf / D + l_D;
  const double l_x2 = l_D + l_x4 * 2.0 * x2;
  const double l_va2 = l_x2 * inv_va2max;
  l_bb += l_va2 / rh;
  double l_rh = -l_va2 * va2 / rh;
  for (int i = 0; i < 3; i++) l_B[i] += l_bb * 2.0 * B[i];
  const double l_R1 = lG[1] + l_F[0];  // R[1] + dn2 is both the output and fx
  l_R[0] = lG[0] + l_rd;
  l_R[1] = l_R1;
  l_R[2] = lG[2] + l_F[1];
  l_R[3] = lG[3] + l_F[2];
  for (int o = 4; o < NV; o++) l_R[o] = lG[o];
  const double l_dn2 = l_R1 + lG[4] * v[0];  // R[4] += dn2 * vx
  l_v[0] += lG[4] * dn2;
  l_rh += l_dn2 * gx;
  l_cen[P_D] += l_rh;
  for (int i = 0; i < 3; i++) {
    l_cen[P_V1 + i] += l_v[i];
    l_cen[P_B1 + i] += l_B[i];
  }
}

// Reverse of boris_lf<double> (src/mhdres_SR.C:310-323): l_lf back to the
// cell's density and field (l_cen, added).
__device__ __forceinline__ void boris_lf_rev(const double* cen, double inv_va2max, double l_lf, double* l_cen) {
  const double dn = 1.0 / cen[P_D];
  const double B[3] = {cen[P_B1], cen[P_B2], cen[P_B3]};
  const double bb = B[0] * B[0] + B[1] * B[1] + B[2] * B[2];
  const double va2 = bb * dn;
  const double x2 = va2 * inv_va2max, x4 = x2 * x2, s = 1.0 + x2;
  const double E = s + x4, lf = s / E;
  const double l_s = l_lf * (1.0 - lf) / E;  // lf = s / (s + x4)
  const double l_x4 = -l_lf * lf / E;
  const double l_x2 = l_s + l_x4 * 2.0 * x2;
  const double l_va2 = l_x2 * inv_va2max;
  const double l_bb = l_va2 * dn, l_dn = l_va2 * bb;
  l_cen[P_D] += -l_dn * dn * dn;
  for (int i = 0; i < 3; i++) l_cen[P_B1 + i] += l_bb * 2.0 * B[i];
}

// Reverse of flux12<double, D1> (src/mhdres_SR.C:330-347): lF, the adjoints
// of the 12 directional quantities, back to the cell's primitives (lw, added).
template <int D1>
__device__ __forceinline__ void flux12_rev(const double* p, const double* lF, double* lw) {
  const double d = p[P_D], v[3] = {p[P_V1], p[P_V2], p[P_V3]}, ei = p[P_EI], B[3] = {p[P_B1], p[P_B2], p[P_B3]};
  const double pr = p[P_P], ekin = p[P_EK];
  const double vel = v[D1], mag = B[D1];
  const double mflx = vel * d;
  double l_v[3] = {0.0, 0.0, 0.0}, l_B[3] = {0.0, 0.0, 0.0};
  double l_mflx = lF[0], l_vel = 0.0, l_mag = 0.0;
  for (int t = 0; t < 3; t++) {  // f(1+t) = mflx * v_t + (t == D1) * pr
    l_mflx += lF[1 + t] * v[t];
    l_v[t] += lF[1 + t] * mflx;
  }
  lw[P_P] += lF[1 + D1];
  l_vel += lF[4] * (ei + ekin + pr);  // f4 = vel * (ei + ekin + pr)
  lw[P_EI] += lF[4] * vel;
  lw[P_EK] += lF[4] * vel;
  lw[P_P] += lF[4] * vel;
  for (int t = 0; t < 3; t++) {  // induction flux of component t: vel * B_t - v_t * mag
    const double l = (Dirs<D1>::fa == 5 + t ? lF[5] : 0.0) + (Dirs<D1>::fb == 5 + t ? lF[6] : 0.0);
    l_vel += l * B[t];
    l_B[t] += l * vel;
    l_v[t] -= l * mag;
    l_mag -= l * v[t];
  }
  for (int t = 0; t < 3; t++) {  // Maxwell stress: mag * B_t - (t == D1) * pmag
    l_mag += lF[7 + t] * B[t];
    l_B[t] += lF[7 + t] * mag;
  }
  lw[P_PM] -= lF[7 + D1];
  l_B[Dirs<D1>::d2] += lF[10];
  l_B[Dirs<D1>::d3] += lF[11];
  l_vel += l_mflx * d;  // mflx = vel * d
  lw[P_D] += l_mflx * vel;
  l_v[D1] += l_vel;
  l_B[D1] += l_mag;
  for (int t = 0; t < 3; t++) {
    lw[P_V1 + t] += l_v[t];
    lw[P_B1 + t] += l_B[t];
  }
}

// Reverse of prim_of_raw<double, false> (src/cons_to_prim.C:148-159 and the
// residual's kinetic and magnetic pressures): lw, the adjoints of the 11
// primitives, back to the cell's 9 stored values (lr, written).
__device__ __forceinline__ void prim_of_raw_rev(const Raw9<double>& r, const double* lw, double* lr) {
  const double d = r.v[0], dn = 1.0 / d;
  const double m[3] = {r.v[1], r.v[2], r.v[3]};
  double v[3];
  for (int t = 0; t < 3; t++) v[t] = m[t] * dn;
  const double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  double l_d = lw[P_D] + lw[P_EK] * 0.5 * vv;  // ekin = 0.5 * d * vv
  double l_vv = lw[P_EK] * 0.5 * d;
  const double l_e = lw[P_EI];  // ei = e - 0.5 * vv * d
  l_vv -= lw[P_EI] * 0.5 * d;
  l_d -= lw[P_EI] * 0.5 * vv;
  double l_dn = 0.0;
  for (int t = 0; t < 3; t++) {
    const double l_v = lw[P_V1 + t] + l_vv * 2.0 * v[t];
    lr[1 + t] = l_v * dn;  // v = m * dn
    l_dn += l_v * m[t];
  }
  l_d -= l_dn * dn * dn;  // dn = 1 / d
  lr[0] = l_d;
  lr[4] = l_e;
  for (int t = 0; t < 3; t++) lr[5 + t] = lw[P_B1 + t] + lw[P_PM] * r.v[5 + t];  // pmag = 0.5 * |B|^2
  lr[8] = lw[P_P];
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
    // sources and Boris correction (G = sources(R, cen)), the residual
    // assembly of each direction (R = sum_d res_d(Dq_d, cen, lf)) and the
    // Boris factor lf(cen), each transposed in one reverse pass
    double lR[NV], lcen[NF];
    for (int q = 0; q < NF; q++) lcen[q] = 0.0;
    stage_sources_rev(R, cen, k.gx, inv_va2max, lg, lR, lcen);
    double llf = 0.0;
    {
      double ldq[NF];
      apply_direction_rev<0>(Dq[0], cen, lf, lR, ldq, lcen, llf);
      for (int q = 0; q < NF; q++) buf_dq[(long long)(0 * NF + q) * b.n + li] = ldq[q];
      apply_direction_rev<1>(Dq[1], cen, lf, lR, ldq, lcen, llf);
      for (int q = 0; q < NF; q++) buf_dq[(long long)(1 * NF + q) * b.n + li] = ldq[q];
      apply_direction_rev<2>(Dq[2], cen, lf, lR, ldq, lcen, llf);
      for (int q = 0; q < NF; q++) buf_dq[(long long)(2 * NF + q) * b.n + li] = ldq[q];
    }
    boris_lf_rev(cen, inv_va2max, llf, lcen);
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
      if (d == 0) flux12_rev<0>(w, lF, lw);  // flux12 transposed onto the cell's primitives
      else if (d == 1) flux12_rev<1>(w, lF, lw);
      else flux12_rev<2>(w, lF, lw);
    }
    double lr[9];  // the primitive conversion transposed onto the stage input
    prim_of_raw_rev(r, lw, lr);
    for (int q = 0; q < NV; q++) lam_uin[(long long)q * b.n + li] = lr[q];
    lam_pin[li] += lr[8];
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

// Reverse mode of tvd_flux<double, DIR> (DIAG off; src/tvdlimit_SR.C:436-563
// as gpumhd_kernels.cuh restates it): the forward intermediates are
// recomputed, then the adjoints lF (the 8 interface fluxes) and lq (the
// resistive-heating term) are carried back to the inputs, each min / max /
// |.| taking the branch the forward took -- the one-sided subgradient the
// dual numbers give, in one pass instead of one dual pass per input.  Adds
// into l_am, l_a, l_b, l_bp (NT TCell fields each) and l_sa, l_sb (slopes).
template <int DIR>
__device__ void tvd_flux_rev(const Consts& c, const TCell<double>& am, const TCell<double>& a, const TCell<double>& b,
                             const TCell<double>& bp, const double* sa, const double* sb, int ia, int sz, double fac0,
                             double cmax_t, bool hyper, int istart, const double* lF, double lq, double* l_am,
                             double* l_a, double* l_b, double* l_bp, double* l_sa, double* l_sb) {
  const KC<double>& k = c.kd;
  const double tiny = tiny100<double>();
  auto dn_field = [](int v) { return (v >= 1 && v <= 3) ? T_HV : ((v >= 5) ? T_HB : T_HE); };
  // ---- forward
  double sl[NV], sll[NV], den[NV], rf[NV], cfv[NV], G[NV], F0[NV], F[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) {
    sl[v] = b.q[v] - a.q[v];
    sll[v] = b.q[v] - a.q[v] - (sa[v] + sb[v]);
    const double dnv = tf(a)[dn_field(v)];
    den[v] = smax(tiny, fabs(sl[v]));
    rf[v] = fabs(sll[v]) / den[v];
    cfv[v] = smax(0.0, smin(sll[v], sl[v])) + smin(0.0, smax(sll[v], sl[v]));
    G[v] = smax(0.0, 1.0 + dnv * (rf[v] - 1.0));
    F0[v] = G[v] * cfv[v];
  }
  const double M = smax(a.cm, b.cm);
  const double fac = fac0 * smin(cmax_t, M);
#pragma unroll
  for (int v = 0; v < NV; v++) F[v] = F0[v] * fac;
  F[5 + DIR] *= k.B_par_diff;
  double F2[NV];  // before the coefficients
#pragma unroll
  for (int v = 0; v < NV; v++) F2[v] = F[v];
  double argv = 0.0, arge = 0.0, cv = 1.0, ce = 1.0;
  if (c.need_coeff) {
    F[0] *= k.tvd_coeff[0];
    argv = k.visc_coeff_bot * a.hb + k.visc_coeff_top * a.ht;
    cv = smax(k.tvd_coeff[1], argv);
    F[1] *= cv; F[2] *= cv; F[3] *= cv;
    F[4] *= k.tvd_coeff[2];
    arge = k.eta_coeff_bot * a.hb + k.eta_coeff_top * a.ht;
    ce = smax(k.tvd_coeff[3], arge);
    F[5] *= ce; F[6] *= ce; F[7] *= ce;
  }
  const bool hy = DIR == 0 && hyper && ia >= istart;
  double dh = 0.0, X[NV] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (hy) {
    dh = smax(a.hd, b.hd);
    const int hv[3] = {0, 1, 4};
    for (int t = 0; t < 3; t++) {
      const int v = hv[t];
      X[v] = 0.125 * (bp.q[v] - am.q[v]) - 0.375 * (b.q[v] - a.q[v]);
      F[v] -= dh * X[v];
    }
  }
  double u[5];
#pragma unroll
  for (int v = 0; v < 5; v++) u[v] = 0.5 * (a.q[v] + sa[v] + b.q[v] - sb[v]);
  double U0 = u[0], U4 = u[4], f0 = F[0], f4a = F[4];
  if (c.rho_log) {
    U0 = exp(u[0]);
    f0 = F[0] * U0;
    U4 = exp(u[4]);
    f4a = F[4] * U4;
  }
  const double CZ = smin(k.CZ, k.CZ);
  const double mcz = f0 * CZ;
  double fn[4];
  for (int t = 1; t <= 3; t++) fn[t] = F[t] * U0 + u[t] * mcz;
  const double S = u[1] * fn[1] + u[2] * fn[2] + u[3] * fn[3];
  const bool zero5 = DIR == 0 && !c.g.periodic_x && (ia == sz - GH - 1 || ia == GH - 1);
  const double Fq[3] = {zero5 ? 0.0 : F[5], F[6], F[7]};
  // ---- reverse
  double lo[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) lo[v] = lF[v];
  for (int t = 0; t < 3; t++) {  // qres = sum (b.q - a.q) * F, v = 5..7
    const int v = 5 + t;
    lo[v] += lq * (b.q[v] - a.q[v]);
    l_b[v] += lq * Fq[t];
    l_a[v] -= lq * Fq[t];
  }
  if (zero5) lo[5] = 0.0;
  // F4 = (f4a*U0 + U4*mcz) + qt*S
  double l_u[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  double l_U4 = lo[4] * mcz, l_mcz = lo[4] * U4;
  l_a[T_QT] += lo[4] * S;
  const double l_S = lo[4] * a.qt;
  double l_U0 = lo[4] * f4a;
  const double l_f4a = lo[4] * U0;
  double lFc[NV] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};  // adjoints of F after coefficients and hyperdiffusion
  for (int t = 1; t <= 3; t++) {  // fn = F*U0 + u*mcz
    const double l_fn = lo[t] + l_S * u[t];
    l_u[t] += l_S * fn[t] + l_fn * mcz;
    lFc[t] += l_fn * U0;
    l_U0 += l_fn * F[t];
    l_mcz += l_fn * u[t];
  }
  const double l_f0 = lo[0] + l_mcz * CZ;
  if (c.rho_log) {
    lFc[0] += l_f0 * U0;
    l_U0 += l_f0 * F[0];
    lFc[4] += l_f4a * U4;
    l_U4 += l_f4a * F[4];
    l_u[0] += l_U0 * U0;
    l_u[4] += l_U4 * U4;
  } else {
    lFc[0] += l_f0;
    lFc[4] += l_f4a;
    l_u[0] += l_U0;
    l_u[4] += l_U4;
  }
  for (int v = 5; v < NV; v++) lFc[v] += lo[v];
#pragma unroll
  for (int v = 0; v < 5; v++) {  // u = 0.5 * (a.q + sa + b.q - sb)
    const double h = 0.5 * l_u[v];
    l_a[v] += h;
    l_sa[v] += h;
    l_b[v] += h;
    l_sb[v] -= h;
  }
  if (hy) {  // F -= dh * X
    double l_dh = 0.0;
    const int hv[3] = {0, 1, 4};
    for (int t = 0; t < 3; t++) {
      const int v = hv[t];
      l_dh -= lFc[v] * X[v];
      const double lX = -lFc[v] * dh;
      l_bp[v] += 0.125 * lX;
      l_am[v] -= 0.125 * lX;
      l_b[v] -= 0.375 * lX;
      l_a[v] += 0.375 * lX;
    }
    if (a.hd < b.hd) l_b[T_HD] += l_dh;
    else l_a[T_HD] += l_dh;
  }
  double l1[NV];  // adjoints of F after the scaling by fac (and B_par_diff)
  if (c.need_coeff) {
    l1[0] = lFc[0] * k.tvd_coeff[0];
    l1[4] = lFc[4] * k.tvd_coeff[2];
    double l_cv = 0.0, l_ce = 0.0;
    for (int v = 1; v <= 3; v++) { l1[v] = lFc[v] * cv; l_cv += lFc[v] * F2[v]; }
    for (int v = 5; v <= 7; v++) { l1[v] = lFc[v] * ce; l_ce += lFc[v] * F2[v]; }
    if (k.tvd_coeff[1] < argv) { l_a[T_HBOT] += l_cv * k.visc_coeff_bot; l_a[T_HTOP] += l_cv * k.visc_coeff_top; }
    if (k.tvd_coeff[3] < arge) { l_a[T_HBOT] += l_ce * k.eta_coeff_bot; l_a[T_HTOP] += l_ce * k.eta_coeff_top; }
  } else {
#pragma unroll
    for (int v = 0; v < NV; v++) l1[v] = lFc[v];
  }
  l1[5 + DIR] *= k.B_par_diff;
  double l_fac = 0.0;
#pragma unroll
  for (int v = 0; v < NV; v++) l_fac += l1[v] * F0[v];
  if (M < cmax_t) {  // fac = fac0 * min(cmax_t, max(a.cm, b.cm))
    const double l_M = l_fac * fac0;
    if (a.cm < b.cm) l_b[T_CM] += l_M;
    else l_a[T_CM] += l_M;
  }
#pragma unroll
  for (int v = 0; v < NV; v++) {
    const double l_F0 = l1[v] * fac;
    const double l_G = l_F0 * cfv[v], l_cf = l_F0 * G[v];
    const int df = dn_field(v);
    const double dnv = tf(a)[df];
    double l_rf = 0.0;
    if (0.0 < 1.0 + dnv * (rf[v] - 1.0)) {  // G = max(0, 1 + dn*(rf - 1))
      l_a[df] += l_G * (rf[v] - 1.0);
      l_rf = l_G * dnv;
    }
    double l_sl = 0.0, l_sll = 0.0;
    l_sll += (l_rf / den[v]) * (sll[v] < 0.0 ? -1.0 : 1.0);  // rf = |sll| / den
    if (tiny < fabs(sl[v])) l_sl += (-l_rf * rf[v] / den[v]) * (sl[v] < 0.0 ? -1.0 : 1.0);
    if (0.0 < smin(sll[v], sl[v])) {  // cf = max(0, min(sll, sl)) + min(0, max(sll, sl))
      if (sl[v] < sll[v]) l_sl += l_cf;
      else l_sll += l_cf;
    }
    if (smax(sll[v], sl[v]) < 0.0) {
      if (sll[v] < sl[v]) l_sl += l_cf;
      else l_sll += l_cf;
    }
    l_b[v] += l_sl + l_sll;  // sl = b.q - a.q, sll = sl - (sa + sb)
    l_a[v] -= l_sl + l_sll;
    l_sa[v] -= l_sll;
    l_sb[v] -= l_sll;
  }
}

// Reverse mode of tvd_update<double> (DIAG off, no compensation;
// src/tvdlimit_SR.C:565-657): given lu (the adjoint of the updated state),
// the adjoints of u_in (l_in), of the cell's TCell (l_c0: q, BC2, bsqr, qt),
// of the fluxes at its right / left interfaces (l_fp, l_fm) and of their
// heating terms (l_qp, l_qm), each floor taking the forward's branch.
__device__ void tvd_update_rev(const Consts& c, double dtt, const double* Fp, const double* Fm, double qp, double qm,
                               const TCell<double>& c0, const double* u_in, const double* lu, double* l_in,
                               double* l_c0, double* l_fp, double* l_fm, double& l_qp, double& l_qm) {
  const KC<double>& k = c.kd;
  const double tiny = tiny100<double>();
  // ---- forward
  double res[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) res[v] = dtt * (Fp[v] - Fm[v]);
  const double W = res[1] * c0.q[1] + res[2] * c0.q[2] + res[3] * c0.q[3];
  const double r4a = res[4] + (1.0 - c0.qt) * W;
  const double bs = smax(tiny, c0.bsqr);
  const double num = res[1] * c0.q[5] + res[2] * c0.q[6] + res[3] * c0.q[7];
  const double dn = num / bs;
  double bb[3];
  for (int t = 0; t < 3; t++) bb[t] = -c0.BC2 * (res[1 + t] - dn * c0.q[5 + t]);
  const double b3 = bb[0] * c0.q[1] + bb[1] * c0.q[2] + bb[2] * c0.q[3];
  double r[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) r[v] = res[v];
  for (int t = 0; t < 3; t++) r[1 + t] += bb[t];
  const double qres = 0.5 * (qp + qm) * c0.qt;
  r[4] = (r4a + b3) + dtt * qres;
  double u[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) u[v] = u_in[v] + r[v];
  const double u0f = smax(k.rho_min, u[0]);
  const double K = u[1] * u[1] + u[2] * u[2] + u[3] * u[3];
  const double ef = k.eps_min * u0f + 0.5 * K / u0f;
  // ---- reverse
  double l_u[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) l_u[v] = lu[v];
  double l_ef = 0.0;
  if (u[4] < ef) {  // u4 = max(u4, ef)
    l_ef = lu[4];
    l_u[4] = 0.0;
  }
  double l_u0f = lu[0] + l_ef * (k.eps_min - 0.5 * K / (u0f * u0f));
  for (int t = 1; t <= 3; t++) l_u[t] += l_ef * u[t] / u0f;
  l_u[0] = (k.rho_min < u[0]) ? l_u0f : 0.0;  // u0 = max(rho_min, u0)
#pragma unroll
  for (int v = 0; v < NV; v++) l_in[v] = l_u[v];
  // r4 = (r4a + b3) + dtt * 0.5 * (qp + qm) * qt
  const double l_qres = l_u[4] * dtt;
  l_qp = 0.5 * l_qres * c0.qt;
  l_qm = l_qp;
  l_c0[T_QT] += l_qres * 0.5 * (qp + qm);
  double l_res[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) l_res[v] = l_u[v];  // r = res (+ bb on 1..3)
  const double l_b3 = l_u[4];
  double l_bb[3];
  for (int t = 0; t < 3; t++) {
    l_bb[t] = l_u[1 + t] + l_b3 * c0.q[1 + t];  // b3 = sum bb * q(1..3)
    l_c0[1 + t] += l_b3 * bb[t];
  }
  double l_dn = 0.0;
  for (int t = 0; t < 3; t++) {  // bb = -BC2 * (res - dn * qB)
    const double in = res[1 + t] - dn * c0.q[5 + t];
    l_c0[T_BC2] -= l_bb[t] * in;
    const double l_inn = -c0.BC2 * l_bb[t];
    l_res[1 + t] += l_inn;
    l_dn -= l_inn * c0.q[5 + t];
    l_c0[5 + t] -= l_inn * dn;
  }
  const double l_num = l_dn / bs;  // dn = num / bs
  if (tiny < c0.bsqr) l_c0[T_BSQR] += -l_dn * dn / bs;
  for (int t = 0; t < 3; t++) {
    l_res[1 + t] += l_num * c0.q[5 + t];
    l_c0[5 + t] += l_num * res[1 + t];
  }
  // r4a = res4 + (1 - qt) * W, W = sum res(1..3) * q(1..3)
  const double l_r4a = l_u[4];
  l_res[4] = l_r4a;
  l_c0[T_QT] -= l_r4a * W;
  const double l_W = l_r4a * (1.0 - c0.qt);
  for (int t = 1; t <= 3; t++) {
    l_res[t] += l_W * c0.q[t];
    l_c0[t] += l_W * res[t];
  }
#pragma unroll
  for (int v = 0; v < NV; v++) {  // res = dtt * (Fp - Fm)
    l_fp[v] = l_res[v] * dtt;
    l_fm[v] = -l_res[v] * dtt;
  }
}

// Reverse of tvd_slope<double> (src/tvdlimit_SR.C:388-434): ls, the adjoint
// of the limited slope at the middle cell b, back to the TCells of a, b, n
// (added): q of all three, and b's boundary profiles hb, ht.  The zeroings
// (large density jump, speed limit) pass nothing back, as for the dual
// numbers, and every min / max takes the forward's branch.
__device__ void tvd_slope_rev(const Consts& c, const TCell<double>& a, const TCell<double>& b, const TCell<double>& n,
                              double vsqr_diff, const double* ls_in, double* l_a, double* l_b, double* l_n) {
  const KC<double>& k = c.kd;
  double ls[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) ls[v] = ls_in[v];
  const double qr = c.rho_log ? fabs(b.q[0] - n.q[0]) : fabs(log(b.q[0]) - log(n.q[0]));
  if (qr > k.q_rho_max) ls[0] = 0.0;
  if (k.has_vmax_lim && b.vsqr > vsqr_diff) ls[1] = ls[2] = ls[3] = 0.0;
  double s0[NV];  // the limited slopes before the boundary factors
#pragma unroll
  for (int v = 0; v < NV; v++) {
    const double sl = b.q[v] - a.q[v], sr = n.q[v] - b.q[v];
    const double slm = 0.25 * (sl + sr);
    const double lower = smin(smin(sl, sr), slm), upper = smax(smax(sl, sr), slm);
    s0[v] = smax(0.0, lower) + smin(0.0, upper);
  }
  if (k.has_visc_slope) {
    const double fb = 1.0 - k.visc_slope_bot * b.hb, ft = 1.0 - k.visc_slope_top * b.ht;
    const double cf = fb * ft;
    double l_cf = 0.0;
    for (int v = 1; v <= 3; v++) { l_cf += ls[v] * s0[v]; ls[v] *= cf; }
    l_b[T_HBOT] -= l_cf * ft * k.visc_slope_bot;
    l_b[T_HTOP] -= l_cf * fb * k.visc_slope_top;
  }
  if (k.has_eta_slope) {
    const double fb = 1.0 - k.eta_slope_bot * b.hb, ft = 1.0 - k.eta_slope_top * b.ht;
    const double cf = fb * ft;
    double l_cf = 0.0;
    for (int v = 5; v <= 7; v++) { l_cf += ls[v] * s0[v]; ls[v] *= cf; }
    l_b[T_HBOT] -= l_cf * ft * k.eta_slope_bot;
    l_b[T_HTOP] -= l_cf * fb * k.eta_slope_top;
  }
#pragma unroll
  for (int v = 0; v < NV; v++) {
    const double sl = b.q[v] - a.q[v], sr = n.q[v] - b.q[v];
    const double slm = 0.25 * (sl + sr);
    const double m = smin(sl, sr), M = smax(sl, sr);
    const double lower = smin(m, slm), upper = smax(M, slm);
    double l_sl = 0.0, l_sr = 0.0, l_slm = 0.0;
    if (0.0 < lower) {  // max(0, lower), lower = min(min(sl, sr), slm)
      if (slm < m) l_slm += ls[v];
      else if (sr < sl) l_sr += ls[v];
      else l_sl += ls[v];
    }
    if (upper < 0.0) {  // min(0, upper), upper = max(max(sl, sr), slm)
      if (M < slm) l_slm += ls[v];
      else if (sl < sr) l_sr += ls[v];
      else l_sl += ls[v];
    }
    l_sl += 0.25 * l_slm;
    l_sr += 0.25 * l_slm;
    l_b[v] += l_sl - l_sr;
    l_a[v] -= l_sl;
    l_n[v] += l_sr;
  }
}

// Reverse of tvd_cell<double> (src/tvdlimit_SR.C:269-377): lt, the adjoints
// of a cell's TCell fields, back to its 9 stored values (lr, written).  The
// boundary profiles hb, ht, qt are fixed by x; the switch CME is a step in
// the values and passes nothing back; every min / max / floor takes the
// forward's branch, as the dual numbers do.
__device__ void tvd_cell_rev(const Consts& c, const Raw9<double>& r, double hb, double ht, double cmax_t, double fac0,
                             bool hyper, double inv_va2max, const double* lt, double* lr) {
  const KC<double>& k = c.kd;
  // ---- forward
  const double d0 = r.v[0];
  const double d = smax(k.rho_min, d0);
  const double dn = 1.0 / d;
  double v[3], Bc[3];
  for (int t = 0; t < 3; t++) { v[t] = r.v[1 + t] * dn; Bc[t] = r.v[5 + t]; }
  const double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  const double bb = Bc[0] * Bc[0] + Bc[1] * Bc[1] + Bc[2] * Bc[2];
  const double e = r.v[4] * dn - 0.5 * vv;
  const double vs = sqrt(vv);
  const double va2 = bb * dn;
  const double x2 = va2 * inv_va2max, x4 = x2 * x2, s = 1.0 + x2, E = s + x4;
  const double lf = s / E;
  const double cs2 = (5.0 / 3.0) * r.v[8] * dn;
  const double cfast = sqrt(va2 + cs2);
  const double CME = (1.0 - k.CZ) * ((double)(vs >= k.CME_thresh * cfast));
  const double d2 = d * d;
  const double rl = d2 / (d2 + k.rho_lev);
  const double rf = smin(lf, rl);
  const double hh = 1.0 - hb - ht;
  const double cfa = hb * k.tvd_cs[0] + (rf * k.tvd_cs[1] + (1.0 - rf) * k.tvd_cs[2]) * hh + ht * k.tvd_cs[3];
  const double cf = smax(cfa, CME);
  const double cs2b = cs2 * (cf * cf);
  const double A = lf * (cs2b + va2);
  const double mx = smax(cs2b, A);
  const double sq = sqrt(mx);
  const double cm = 0.0 + vs + sq;
  // ---- reverse
  double l_d = c.rho_log ? lt[0] / d : lt[0];
  const double l_e = c.rho_log ? lt[4] / e : lt[4];
  double l_v[3], l_B[3];
  for (int t = 0; t < 3; t++) { l_v[t] = lt[1 + t]; l_B[t] = lt[5 + t]; }
  double l_cm = lt[T_CM], l_vv = lt[T_VSQR], l_bb = lt[T_BSQR], l_lf = -lt[T_BC2];
  if (hyper) {  // hd = fac0 * max(0, min(vhyp * sqrt(vsqr), cmax_t - cm))
    const double hv = k.vhyp * vs, g = cmax_t - cm;
    const double mn = smin(hv, g);
    if (0.0 < mn) {
      const double l_mn = lt[T_HD] * fac0;
      if (g < hv) l_cm -= l_mn;
      else if (vs > 0.0) l_vv += l_mn * k.vhyp * 0.5 / vs;
    }
  }
  const double h1 = k.tvd_h[1], h2 = k.tvd_h[2];
  double l_rf = (lt[T_HE] * (1.0 - CME) * (h1 - h2) + lt[T_HV] * (1.0 - CME) * (h1 - h2 * k.pm_v) +
                 lt[T_HB] * (h1 - h2 * k.pm_B)) * hh;
  double l_vs = l_cm;  // cm = (0 + vs) + sqrt(mx)
  const double l_mx = sq > 0.0 ? l_cm * 0.5 / sq : 0.0;
  double l_cs2b = 0.0, l_A = 0.0;
  if (cs2b < A) l_A = l_mx;
  else l_cs2b = l_mx;
  l_lf += l_A * (cs2b + va2);
  l_cs2b += l_A * lf;
  double l_va2 = l_A * lf;
  double l_cs2 = l_cs2b * (cf * cf);
  const double l_cf = l_cs2b * cs2 * 2.0 * cf;
  if (!(cfa < CME)) l_rf += l_cf * (k.tvd_cs[1] - k.tvd_cs[2]) * hh;
  if (rl < lf) l_d += l_rf * k.rho_lev / ((d2 + k.rho_lev) * (d2 + k.rho_lev)) * 2.0 * d;
  else l_lf += l_rf;
  double l_dn = l_cs2 * (5.0 / 3.0) * r.v[8];
  lr[8] = l_cs2 * (5.0 / 3.0) * dn;
  const double l_x2 = l_lf * (1.0 - lf) / E + (-l_lf * lf / E) * 2.0 * x2;  // lf = s / (s + x4)
  l_va2 += l_x2 * inv_va2max;
  l_bb += l_va2 * dn;  // va2 = bb * dn
  l_dn += l_va2 * bb;
  if (vs > 0.0) l_vv += l_vs * 0.5 / vs;
  lr[4] = l_e * dn;  // e = r4 * dn - 0.5 * vv
  l_dn += l_e * r.v[4];
  l_vv -= 0.5 * l_e;
  for (int t = 0; t < 3; t++) {
    const double lvt = l_v[t] + l_vv * 2.0 * v[t];
    lr[1 + t] = lvt * dn;
    l_dn += lvt * r.v[1 + t];
    lr[5 + t] = l_B[t] + l_bb * 2.0 * Bc[t];
  }
  l_d -= l_dn * dn * dn;
  lr[0] = (k.rho_min < d0) ? l_d : 0.0;
}

// T0: the per-cell TVD quantities of every cell the sweep's transposes read
// (interior in the other directions, two ghosts on either side along the
// sweep), once, into tc (19 per node of the ghosted box).
template <int DIR>
__global__ void k_tvd_t0(Consts c, const Dyn* dyn, Box b, const double* __restrict__ V, const double* __restrict__ P,
                         double* __restrict__ tc) {
  const Sweep s = sweep_of<DIR>(c, dyn);
  const Geom& g = c.g;
  const int na = DIR == 0 ? b.nx + 2 * GH : b.nx, nb = DIR == 1 ? b.ny + 2 * GH : b.ny;
  const int nc = DIR == 2 ? b.nz + 2 * GH : b.nz;
  const long long m = (long long)na * nb * nc;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (long long)gridDim.x * blockDim.x) {
    int i = (int)(t % na), j = (int)((t / na) % nb), k = (int)(t / ((long long)na * nb));
    if (DIR == 0) i -= GH;
    if (DIR == 1) j -= GH;
    if (DIR == 2) k -= GH;
    TCell<double> T;
    cell_at<DIR>(c, s, V, P, i, j, k, 0, T);
    const long long id = fwd(g, i, j, k);
    for (int f = 0; f < NT; f++) tc[(long long)f * g.N + id] = tf(T)[f];
  }
}

// the cell `o` steps along DIR from interior (i, j, k), from k_tvd_t0's store
template <int DIR>
__device__ __forceinline__ void cell_load(const Geom& g, const double* __restrict__ tc, int i, int j, int k, int o,
                                          TCell<double>& t) {
  const long long id = fwd(g, i + (DIR == 0 ? o : 0), j + (DIR == 1 ? o : 0), k + (DIR == 2 ? o : 0));
  for (int f = 0; f < NT; f++) tf(t)[f] = tc[(long long)f * g.N + id];
}

// T1: per cell i, the update transposed.  Outputs: lam_in_direct (8), the
// adjoint of the cell's TCell (19), and of its right / left interface fluxes
// and heating terms (9 + 9).
template <int DIR>
__global__ void k_tvd_t1(Consts c, const Dyn* dyn, Box b, const double* __restrict__ V, const double* __restrict__ P,
                         const double* __restrict__ tc, const double* __restrict__ lam_out, int final_pass,
                         double* __restrict__ o_in, double* __restrict__ o_cell, double* __restrict__ o_fp,
                         double* __restrict__ o_fm) {
  const Sweep s = sweep_of<DIR>(c, dyn);
  const DynR<double>& dr = dyn->rd;
  for (long long li = (long long)blockIdx.x * blockDim.x + threadIdx.x; li < b.n;
       li += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    ijk(b, li, i, j, k);
    TCell<double> T[5];
    Raw9<double> r0;
    raw_at(c.g, V, P, fwd(c.g, i, j, k), r0);
    for (int o = -2; o <= 2; o++) cell_load<DIR>(c.g, tc, i, j, k, o, T[o + 2]);
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
    // the update transposed in one reverse pass (inputs: u_in, the cell's
    // q, BC2, bsqr, qt, the fluxes and heating terms of both interfaces)
    {
      double l_in[NV], l_c0[NT], l_fp[NV], l_fm[NV], l_qp = 0.0, l_qm = 0.0;
      for (int f = 0; f < NT; f++) l_c0[f] = 0.0;
      tvd_update_rev(c, s.dtt, Fp, Fm, qp, qm, T[2], r0.v, lo, l_in, l_c0, l_fp, l_fm, l_qp, l_qm);
      for (int q = 0; q < NV; q++) {
        o_in[(long long)q * b.n + li] = l_in[q];
        o_cell[(long long)q * b.n + li] = l_c0[q];
        o_fp[(long long)q * b.n + li] = l_fp[q];
        o_fm[(long long)q * b.n + li] = l_fm[q];
      }
      o_cell[(long long)T_BC2 * b.n + li] = l_c0[T_BC2];
      o_cell[(long long)T_BSQR * b.n + li] = l_c0[T_BSQR];
      o_cell[(long long)T_QT * b.n + li] = l_c0[T_QT];
      o_fp[(long long)8 * b.n + li] = l_qp;
      o_fm[(long long)8 * b.n + li] = l_qm;
    }
    const int unused[8] = {T_CM, T_HE, T_HV, T_HB, T_VSQR, T_HD, T_HBOT, T_HTOP};
    for (int f = 0; f < 8; f++) o_cell[(long long)unused[f] * b.n + li] = 0.0;
  }
}

// T2: per interface i+1/2 (stored at its left cell i), the interface flux
// transposed onto its four cells' TCells (am, a, b, bp: 19 each) and its two
// slopes (8 each): 92 values per interface.
template <int DIR>
__global__ void k_tvd_t2(Consts c, const Dyn* dyn, Box b, const double* __restrict__ tc,
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
    for (int o = -1; o <= 2; o++) cell_load<DIR>(c.g, tc, i, j, k, o, T[o + 1]);
    double sa[NV], sb[NV];
    tvd_slope<double>(c, T[0], T[1], T[2], s.vsqr_diff, sa);
    tvd_slope<double>(c, T[1], T[2], T[3], s.vsqr_diff, sb);
    const int p = pos_of<DIR>(i, j, k);
    // the interface flux transposed in one reverse pass onto its four cells'
    // TCells (am, a, b, bp) and its two slopes
    double l_t[4][NT], l_s[2][NV];
    for (int r = 0; r < 4; r++)
      for (int f = 0; f < NT; f++) l_t[r][f] = 0.0;
    for (int q = 0; q < NV; q++) l_s[0][q] = l_s[1][q] = 0.0;
    tvd_flux_rev<DIR>(c, T[0], T[1], T[2], T[3], sa, sb, p, s.sz, s.fac0, s.cmax_t, s.hyper, s.istart, lF, lF[NV],
                      l_t[0], l_t[1], l_t[2], l_t[3], l_s[0], l_s[1]);
    for (int r = 0; r < 4; r++)
      for (int f = 0; f < NT; f++) o_if[(long long)(r * NT + f) * b.n + li] = l_t[r][f];
    for (int r = 0; r < 2; r++)
      for (int q = 0; q < NV; q++) o_if[(long long)(4 * NT + r * NV + q) * b.n + li] = l_s[r][q];
  }
}

// T3: per cell i, its slope transposed onto the three cells it reads
// (i-1: q; i: q, hb, ht, vsqr; i+1: q): 3 x 19 values.
template <int DIR>
__global__ void k_tvd_t3(Consts c, const Dyn* dyn, Box b, const double* __restrict__ tc,
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
    for (int o = -1; o <= 1; o++) cell_load<DIR>(c.g, tc, i, j, k, o, T[o + 1]);
    // the slope transposed in one reverse pass onto its three cells
    double l_t[3][NT];
    for (int r = 0; r < 3; r++)
      for (int f = 0; f < NT; f++) l_t[r][f] = 0.0;
    tvd_slope_rev(c, T[0], T[1], T[2], s.vsqr_diff, ls, l_t[0], l_t[1], l_t[2]);
    for (int r = 0; r < 3; r++)
      for (int f = 0; f < NT; f++) o_sl[(long long)(r * NT + f) * b.n + li] = l_t[r][f];
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
    double lr[9];  // the cell quantities transposed onto the sweep input
    tvd_cell_rev(c, r, c.kd.hfb[xi], c.kd.hft[xi], s.cmax_t, s.fac0, s.hyper, s.inv_va2max, lt, lr);
    for (int q = 0; q < NV; q++) lam_in[(long long)q * b.n + li] = i_in[(long long)q * b.n + li] + lr[q];
    lam_p[li] += lr[8];
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
  adj::k_tvd_t0<DIR><<<gr, 128, 0, s>>>(c, dyn, b, V, P, w.tcell);
  adj::k_tvd_t1<DIR><<<gr, 128, 0, s>>>(c, dyn, b, V, P, w.tcell, lam_out, final_pass, w.in, w.cell, w.fp, w.fm);
  adj::k_tvd_t2<DIR><<<gr, 128, 0, s>>>(c, dyn, b, w.tcell, w.fp, w.fm, w.iface);
  adj::k_tvd_t3<DIR><<<gr, 128, 0, s>>>(c, dyn, b, w.tcell, w.iface, w.slope);
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
