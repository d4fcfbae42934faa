// divB cleaning (Clean_divB, src/clean_divB.C:35-369).
//
// One call: the divergence pass (k_divb_div, pass 0) gives divB and its
// maximum; then each of n iterations is a gradient pass (k_divb_grad:
// B += grad(phi), e += phi*divB) followed by a divergence pass on the new B.
// The reference's first statement of an iteration, phi += fac*divB -
// damp*phi, is pointwise, so the divergence pass that precedes the iteration
// applies it to its own cell right after forming divB there (and the last
// divergence pass does not).  n is Clean_divB's adaptive count (a function
// static there) and lives in Dyn: k_divb_begin copies it for this call,
// k_divb_end updates it from the two error maxima.  The host enqueues
// max(3, itmax) iterations; the passes beyond n return at once.
//
// Ghosts: the reference exchanges B and phi before each use.  Here periodic
// neighbours are read from the interior directly (the wrapped index), which
// is the value that exchange puts in the ghost.  Across a closed x boundary
// exchange_B_acc fills nothing, so B's stored x ghosts are read as the step
// left them, and phi is antisymmetric (src/clean_divB.C:198-225).
#pragma once
#include "gpumhd_kernels.cuh"

namespace gpumhd {

constexpr int DIVB_BX = 32, DIVB_BY = 4;

// Interior neighbour index at offset o along a periodic dimension of n cells.
__device__ __forceinline__ int wrap_i(int i, int o, int n) {
  int I = i - GH + o;
  if (I < 0) I += n;
  else if (I >= n) I -= n;
  return I + GH;
}

// x neighbour of phi at offset o: periodic wraps; closed mirrors with a sign
// change (phi[lb-1] = -phi[lb], phi[lb-2] = -phi[lb+1], and alike at the top).
__device__ __forceinline__ int phi_x(const Geom& g, int i, int o, bool& neg) {
  neg = false;
  if (g.periodic_x) return wrap_i(i, o, g.nx);
  const int I = i - GH + o;
  if (I < 0) { neg = true; return GH - 1 - I; }
  if (I >= g.nx) { neg = true; return GH + 2 * g.nx - 1 - I; }
  return i + o;
}

// k_divb_begin (copies the adaptive count for this call, clears the error
// slots) and k_divb_end (the error ratio and the next count,
// src/clean_divB.C:335-354) are defined once, in kernels_f64.cu.
__global__ void k_divb_begin(Dyn* dyn);
__global__ void k_divb_end(Consts c, Dyn* dyn);

// Divergence pass q (0: before the iterations, q >= 1: after iteration q-1):
// divB = sum over dimensions of w1*(B[+1]-B[-1]) + w2*(B[+2]-B[-2]) from zero
// (src/clean_divB.C:125-165, 289-327), its NaN-ignoring maximum, and, when an
// iteration follows, phi += fac*divB - damp*phi (src/clean_divB.C:171-183).
// Threads: x (coalesced) by y in the block, z planes marched with B_z's five
// values along z in registers.
template <class R>
__global__ void __launch_bounds__(DIVB_BX* DIVB_BY) k_divb_div(Consts c, const R* __restrict__ U, R* __restrict__ phi,
                                                              R* __restrict__ divb, Dyn* __restrict__ dyn, int q,
                                                              int zc) {
  if (dyn->err) return;
  const int n = dyn->divb_iters;
  if (q > n) return;
  const Geom& g = c.g;
  const int i = GH + blockIdx.x * DIVB_BX + threadIdx.x;
  const int j = GH + blockIdx.y * DIVB_BY + threadIdx.y;
  const int k0 = GH + blockIdx.z * zc;
  const int k1 = min(k0 + zc, GH + g.nz);
  R err = (R)0;
  if (i < GH + g.nx && j < GH + g.ny) {
    const auto& kk = kc<R>(c);
    const R w1x = kk.w1[0], w2x = kk.w2[0], w1y = kk.w1[1], w2y = kk.w2[1], w1z = kk.w1[2], w2z = kk.w2[2];
    const R fac = kk.divb_fac, damp = kk.divb_damp;
    const bool upd = q < n;
    const unsigned sy = (unsigned)g.sx, sz = (unsigned)g.sx * (unsigned)g.sy;
    const int xm2 = g.periodic_x ? wrap_i(i, -2, g.nx) : i - 2;
    const int xm1 = g.periodic_x ? wrap_i(i, -1, g.nx) : i - 1;
    const int xp1 = g.periodic_x ? wrap_i(i, 1, g.nx) : i + 1;
    const int xp2 = g.periodic_x ? wrap_i(i, 2, g.nx) : i + 2;
    const unsigned ym2 = (unsigned)wrap_i(j, -2, g.ny) * sy, ym1 = (unsigned)wrap_i(j, -1, g.ny) * sy;
    const unsigned yp1 = (unsigned)wrap_i(j, 1, g.ny) * sy, yp2 = (unsigned)wrap_i(j, 2, g.ny) * sy;
    const R* Bx = U + 5u * g.N32;
    const R* By = U + 6u * g.N32;
    const R* Bz = U + 7u * g.N32;
    const unsigned col = (unsigned)i + (unsigned)j * sy;
    // one plane's loads (B_x along the row, B_y along the column, the next
    // B_z of the z window, phi) are issued a plane ahead of their use
    struct In { R x[4], y[4], z, ph; };
    auto load = [&](int k, In& v) {
      const unsigned pl = (unsigned)k * sz;
      const unsigned row = pl + (unsigned)j * sy;
      v.x[0] = Bx[row + xm2]; v.x[1] = Bx[row + xm1]; v.x[2] = Bx[row + xp1]; v.x[3] = Bx[row + xp2];
      v.y[0] = By[pl + ym2 + i]; v.y[1] = By[pl + ym1 + i]; v.y[2] = By[pl + yp1 + i]; v.y[3] = By[pl + yp2 + i];
      v.z = Bz[col + (unsigned)wrap_i(k, 2, g.nz) * sz];
      v.ph = upd ? phi[row + (unsigned)i] : (R)0;
    };
    R zm2 = Bz[col + (unsigned)wrap_i(k0, -2, g.nz) * sz];
    R zm1 = Bz[col + (unsigned)wrap_i(k0, -1, g.nz) * sz];
    R z0 = Bz[col + (unsigned)k0 * sz];
    R zp1 = Bz[col + (unsigned)wrap_i(k0, 1, g.nz) * sz];
    In cur;
    load(k0, cur);
    for (int k = k0; k < k1; k++) {
      In nxt;
      if (k + 1 < k1) load(k + 1, nxt);
      const R zp2 = cur.z;
      R d = (R)0;
      d += (w1x * (cur.x[2] - cur.x[1]) + w2x * (cur.x[3] - cur.x[0]));
      d += (w1y * (cur.y[2] - cur.y[1]) + w2y * (cur.y[3] - cur.y[0]));
      d += (w1z * (zp1 - zm1) + w2z * (zp2 - zm2));
      const unsigned id = (unsigned)k * sz + col;
      divb[id] = d;
      if (upd) phi[id] = cur.ph + (fac * d - damp * cur.ph);
      err = smax(err, d_fabs(d));  // std::max semantics: a NaN divergence is skipped
      zm2 = zm1; zm1 = z0; z0 = zp1; zp1 = zp2;
      cur = nxt;
    }
  }
  const R m = block_max_nonnan(err);  // one atomic per block
  if (threadIdx.x == 0 && threadIdx.y == 0) atomic_max_nonneg(&dyn->divb_err_bits[q == 0 ? 0 : 1], (double)m);
}

// Gradient pass of iteration it: B_v += w1*(phi[+1]-phi[-1]) + w2*(phi[+2]-phi[-2])
// along v, then e += phi*divB (src/clean_divB.C:227-264).  Also clears the
// "after" error slot for the divergence pass that follows.
template <class R>
__global__ void __launch_bounds__(DIVB_BX* DIVB_BY) k_divb_grad(Consts c, R* __restrict__ U, const R* __restrict__ phi,
                                                               const R* __restrict__ divb, Dyn* __restrict__ dyn,
                                                               int it, int zc) {
  if (dyn->err) return;
  if (it >= dyn->divb_iters) return;
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 && threadIdx.y == 0)
    dyn->divb_err_bits[1] = 0ULL;
  const Geom& g = c.g;
  const int i = GH + blockIdx.x * DIVB_BX + threadIdx.x;
  const int j = GH + blockIdx.y * DIVB_BY + threadIdx.y;
  if (i >= GH + g.nx || j >= GH + g.ny) return;
  const int k0 = GH + blockIdx.z * zc;
  const int k1 = min(k0 + zc, GH + g.nz);
  const auto& kk = kc<R>(c);
  const R w1x = kk.w1[0], w2x = kk.w2[0], w1y = kk.w1[1], w2y = kk.w2[1], w1z = kk.w1[2], w2z = kk.w2[2];
  const unsigned sy = (unsigned)g.sx, sz = (unsigned)g.sx * (unsigned)g.sy;
  bool nm2, nm1, np1, np2;
  const int xm2 = phi_x(g, i, -2, nm2), xm1 = phi_x(g, i, -1, nm1);
  const int xp1 = phi_x(g, i, 1, np1), xp2 = phi_x(g, i, 2, np2);
  const unsigned ym2 = (unsigned)wrap_i(j, -2, g.ny) * sy, ym1 = (unsigned)wrap_i(j, -1, g.ny) * sy;
  const unsigned yp1 = (unsigned)wrap_i(j, 1, g.ny) * sy, yp2 = (unsigned)wrap_i(j, 2, g.ny) * sy;
  R* E = U + 4u * g.N32;
  R* Bx = U + 5u * g.N32;
  R* By = U + 6u * g.N32;
  R* Bz = U + 7u * g.N32;
  const unsigned col = (unsigned)i + (unsigned)j * sy;
  // one plane's loads issued a plane ahead of their use
  struct In { R x[4], y[4], pz, bx, by, bz, e, dv; };
  auto load = [&](int k, In& v) {
    const unsigned pl = (unsigned)k * sz;
    const unsigned row = pl + (unsigned)j * sy;
    const unsigned id = row + (unsigned)i;
    v.x[0] = phi[row + xm2]; v.x[1] = phi[row + xm1]; v.x[2] = phi[row + xp1]; v.x[3] = phi[row + xp2];
    v.y[0] = phi[pl + ym2 + i]; v.y[1] = phi[pl + ym1 + i]; v.y[2] = phi[pl + yp1 + i]; v.y[3] = phi[pl + yp2 + i];
    v.pz = phi[col + (unsigned)wrap_i(k, 2, g.nz) * sz];
    v.bx = Bx[id]; v.by = By[id]; v.bz = Bz[id]; v.e = E[id]; v.dv = divb[id];
  };
  R pm2 = phi[col + (unsigned)wrap_i(k0, -2, g.nz) * sz];
  R pm1 = phi[col + (unsigned)wrap_i(k0, -1, g.nz) * sz];
  R p0 = phi[col + (unsigned)k0 * sz];
  R pp1 = phi[col + (unsigned)wrap_i(k0, 1, g.nz) * sz];
  In cur;
  load(k0, cur);
  for (int k = k0; k < k1; k++) {
    In nxt;
    if (k + 1 < k1) load(k + 1, nxt);
    const R pp2 = cur.pz;
    const unsigned id = (unsigned)k * sz + col;
    R a2 = cur.x[0], a1 = cur.x[1], b1 = cur.x[2], b2 = cur.x[3];
    if (nm2) a2 = -a2;
    if (nm1) a1 = -a1;
    if (np1) b1 = -b1;
    if (np2) b2 = -b2;
    Bx[id] = cur.bx + (w1x * (b1 - a1) + w2x * (b2 - a2));
    By[id] = cur.by + (w1y * (cur.y[2] - cur.y[1]) + w2y * (cur.y[3] - cur.y[0]));
    Bz[id] = cur.bz + (w1z * (pp1 - pm1) + w2z * (pp2 - pm2));
    E[id] = cur.e + p0 * cur.dv;
    pm2 = pm1; pm1 = p0; p0 = pp1; pp1 = pp2;
    cur = nxt;
  }
}

}  // namespace gpumhd
