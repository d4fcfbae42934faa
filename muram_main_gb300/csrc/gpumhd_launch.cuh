// Kernel launchers, instantiated once per state type in its own translation
// unit (FP64 without FMA contraction, FP32 with it).
#pragma once
#include "gpumhd_stage_tm.cuh"
#include "gpumhd_divb.cuh"
#include "gpumhd_bnd.cuh"
#include "gpumhd_spitzer.cuh"

namespace gpumhd {

// Step control for the fused path (one thread): the Adjust_Valf_Max limits,
// Sync_timestep (src/solver.C:487-548) on the CFL speed accumulated by the
// previous pass, the TVD branch (src/solver.C:325-339) and Run.Advance.
// With use_cond (a captured step) it also sets the conditional node of the
// second TVD half pass (tvd2) from the branch it chose.
__global__ void k_step_begin(Consts c, Dyn* dyn, double* dt_hist, int dt_hist_cap, cudaGraphConditionalHandle tvd2,
                             int use_cond);
// Step counter of a graph's while loop: k_set_counter before the launch,
// k_loop_tick at the end of each pass (sets the loop condition).
__global__ void k_loop_tick(int* counter, cudaGraphConditionalHandle h);
__global__ void k_set_counter(int* counter, int n);
__global__ void k_divb_begin(Dyn* dyn);
// Start of a fused run on a new state (one thread): the step limits, the
// error flag, the reduction accumulators and the per-precision derived
// scalars, set on the device so that no host copy sits in the stream.
__global__ void k_fused_reinit(Consts c, Dyn* dyn, double inv_va2max, double v_lim, double e_lim, double vsqr_diff);
__global__ void k_divb_end(Consts c, Dyn* dyn);
// Adjust_Valf_Max with adaptive limits (va_adjust > 0) at the start of a fused
// step (one thread): the limits from the statistics the previous pass
// reduced, and a cleared CFL accumulator for the pass that follows.
__global__ void k_step_limits(Consts c, Dyn* dyn);

template <class R>
struct Launch {
  static int resident_stage_blocks;   // stage blocks resident on the whole GPU at once
  static int resident_tm_blocks;      // the same for the TMA / tensor-memory stage kernel
  static int stage_smem_bytes();
  static cudaError_t setup();
  // mu / mp: tensor maps of Uin / Pin for the TMA kernel (both null: k_stage)
  // zc: z planes per block (0: chosen from the occupancy, see stage())
  static void stage(const Consts& c, const R* Uin, const R* Pin, const R* U0, R* Uout, R* Pout, R* Res, Dyn* dyn,
                    int stage, bool resid, int write_pres, cudaStream_t s, const CUtensorMap* mu = nullptr,
                    const CUtensorMap* mp = nullptr, int zc = 0, Rem<R>* Cc = nullptr);
  // td: cells per thread along the y / z sweeps (0: 32); the sweeps store the
  // interior (and after a first half pass the periodic images), step_finish
  // then ends the step
  // dg (per-routine TVDlimit on an output step): the diagnostics, through the
  // pencil kernel in every direction
  // Cc (FP32 compensated fused steps, else null): the state's rounding remainders
  static void tvd(const Consts& c, int dir, int mode, int only_two_half, const R* Uin, const R* Pst, R* Uout,
                  Dyn* dyn, cudaStream_t s, int td = 0, const TvdDiag<R>* dg = nullptr, Rem<R>* Cc = nullptr);
  // Clean_divB on U (phi, divb: N each); returns the number of launches
  static int divb_clean(const Consts& c, R* U, R* phi, R* divb, Dyn* dyn, cudaStream_t s);
  static void step_finish(const Consts& c, R* U, R* P, Dyn* dyn, cudaStream_t s, Rem<R>* Cc = nullptr);
  // MURaM's physical x boundaries on U (P: ghost pressures, may be null;
  // with_cmax: ghost CFL speeds join the step maximum); part: nz*BND_NQ doubles.
  // Returns the number of launches.
  static int bc(const Consts& c, R* U, R* P, Dyn* dyn, double* part, int with_cmax, cudaStream_t s,
                R* sflx = nullptr);
  // Spitzer conduction: the temperature of a conserved state; the per-stage
  // residual of the heat flux (prim: U after ConsToPrim; Sout: the fused
  // step's update of sflx, else Rflx receives the residual)
  static void temp(const Consts& c, const R* U, R* T, cudaStream_t s);
  static void spitzer(const Consts& c, const R* U, bool prim, const R* T, const R* S, const R* S0, R* Sout, R* Rflx,
                      R* Rsp, const Dyn* dyn, int stage, cudaStream_t s);
  static void sflx_update(const Consts& c, R* S, const R* S0, R* Rflx, const Dyn* dyn, int stage, cudaStream_t s);
  // snapshot: T and Ne receive the density and internal energy, aux_of_snapshot the outputs later
  static void cons_to_prim(const Consts& c, R* U, R* P, R* T, R* Ne, R* Ri, R* Am, bool snapshot, cudaStream_t s);
  static void aux_of_snapshot(const Consts& c, R* T, R* Ne, R* Ri, R* Am, cudaStream_t s);
  static void init_pass(const Consts& c, const R* U, R* P, Dyn* dyn, cudaStream_t s);
  static void adjust_stats(const Consts& c, const R* U, const R* P, Dyn* dyn, cudaStream_t s);
  static void cmax_faces(const Consts& c, const R* U, const R* P, Dyn* dyn, cudaStream_t s);
  // interior CFL speed of a conserved state with the step's limits (adaptive limits only)
  static void cfl_cons(const Consts& c, const R* U, const R* P, Dyn* dyn, cudaStream_t s);
  // diag (an output step, else null): tvar1..Qvis, N each; invdt = 1 / Run.dt
  static void source_integrate(const Consts& c, R* U, const R* U0, R* Res, const Dyn* dyn, int stage, cudaStream_t s,
                               R* diag = nullptr, R invdt = (R)0);
  static void save_cons(const Consts& c, const R* U, R* U0, cudaStream_t s);
  static void tcheck(const Consts& c, R* U, const Dyn* dyn, cudaStream_t s, R* diag = nullptr, R invdt = (R)0);
  // MHD_Residual's diagnostics (tvar1..3) of a primitive state
  static void diag_residual(const Consts& c, const R* U, const R* P, const R* S, R* diag, const Dyn* dyn,
                            cudaStream_t s);
  static void fill_ghosts(const Consts& c, R* U, int nfield, int with_bc, cudaStream_t s);
  static void tile_state(const Geom& gd, const Geom& gs, const R* Us, R* Ud, cudaStream_t s);
  // host cState layout (double, or float as in MURaM's SINGLE_PRECISION build) <-> device SoA
  static void aos_to_soa(long long N, int nf, const double* A, R* S, cudaStream_t s);
  static void soa_to_aos(long long N, int nf, const R* S, double* A, cudaStream_t s);
  static void aos_to_soa(long long N, int nf, const float* A, R* S, cudaStream_t s);
  static void soa_to_aos(long long N, int nf, const R* S, float* A, cudaStream_t s);
};

// Tile shapes of the stage kernel per state type.
template <class R> struct StageTile;
template <> struct StageTile<double> { static constexpr int TX = 16, TY = 8; };
template <> struct StageTile<float> { static constexpr int TX = 16, TY = 16; };
// Tile shapes of the TMA / tensor-memory stage kernel.
template <class R> struct StageTileTm;
template <> struct StageTileTm<double> { static constexpr int TX = 16, TY = 8; };
template <> struct StageTileTm<float> { static constexpr int TX = 32, TY = 8; };

inline int grid_for(long long n, int block) {
  long long b = (n + block - 1) / block;
  if (b > 152LL * 32) b = 152LL * 32;
  if (b < 1) b = 1;
  return (int)b;
}

#ifdef GPUMHD_LAUNCH_IMPL
template <class R>
int Launch<R>::stage_smem_bytes() {
  return (int)StageSmem<StageTile<R>::TX, StageTile<R>::TY>::template bytes<R>();
}

template <class R>
int Launch<R>::resident_stage_blocks = 0;
template <class R>
int Launch<R>::resident_tm_blocks = 0;

template <class R>
cudaError_t Launch<R>::setup() {
  constexpr int TX = StageTile<R>::TX, TY = StageTile<R>::TY;
  const int bytes = stage_smem_bytes();
  cudaError_t e = cudaFuncSetAttribute(k_stage<R, TX, TY, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_stage<R, TX, TY, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stage<R, TX, TY, false>, TX * TY, bytes);
  if (e != cudaSuccess) return e;
  resident_stage_blocks = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  constexpr int MX = StageTileTm<R>::TX, MY = StageTileTm<R>::TY;
  const int tb = (int)StageTm<R, MX, MY, false>::BYTES;
  e = cudaFuncSetAttribute(k_stage_tm<R, MX, MY, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, tb);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_stage_tm<R, MX, MY, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, tb);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stage_tm<R, MX, MY, false, false>, MX * MY, tb);
  if (e != cudaSuccess) return e;
  int per_sm_db = per_sm;
  if constexpr (sizeof(R) == 4) {
    const int tdb = (int)StageTm<R, MX, MY, true>::BYTES;
    e = cudaFuncSetAttribute(k_stage_tm<R, MX, MY, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, tdb);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_stage_tm<R, MX, MY, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, tdb);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_db, k_stage_tm<R, MX, MY, false, true>, MX * MY, tdb);
    if (e != cudaSuccess) return e;
  }
  // the z chunking assumes the smaller residency of the two layouts
  per_sm = per_sm_db < per_sm ? per_sm_db : per_sm;
  resident_tm_blocks = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  return cudaSuccess;
}

template <class R>
void Launch<R>::stage(const Consts& c, const R* Uin, const R* Pin, const R* U0, R* Uout, R* Pout, R* Res, Dyn* dyn,
                      int stage, bool resid, int write_pres, cudaStream_t s, const CUtensorMap* mu,
                      const CUtensorMap* mp, int zc_force, Rem<R>* Cc) {
  const bool tma = mu && mp;
  const int TX = tma ? StageTileTm<R>::TX : StageTile<R>::TX, TY = tma ? StageTileTm<R>::TY : StageTile<R>::TY;
  const Geom& g = c.g;
  const int bx = (g.nx + TX - 1) / TX, by = (g.ny + TY - 1) / TY;
  // z chunk length: each block computes 4 extra z-flux planes before its
  // first output plane, and a partly filled last wave idles the GPU; pick the
  // chunk count that maximises (useful share of the waves) / (1 + 4/zc).
  const long long bxy = (long long)bx * by;
  const int res0 = tma ? resident_tm_blocks : resident_stage_blocks;
  const int res = res0 > 0 ? res0 : 304;
  int zc = g.nz;
  double best = -1.0;
  for (int nzc = 1; nzc <= 64 && nzc <= g.nz; nzc++) {
    const int zcc = (g.nz + nzc - 1) / nzc;
    if (zcc < 4 && nzc > 1) break;
    const long long blocks = bxy * ((g.nz + zcc - 1) / zcc);
    const long long waves = (blocks + res - 1) / res;
    const double eff = ((double)blocks / (double)(waves * res)) / (1.0 + 4.0 / zcc);
    if (eff > best + 1e-9) { best = eff; zc = zcc; }
  }
  if (zc_force > 0) zc = zc_force < g.nz ? zc_force : g.nz;
  const int bz = (g.nz + zc - 1) / zc;
  dim3 grid(bx, by, bz);
  if (tma) {
    constexpr int MX = StageTileTm<R>::TX, MY = StageTileTm<R>::TY;
    // FP32: the double-buffered layout for the residual and for stages 1
    // and 4 (no separate U0 stream), the four-slot one for stages 2 and 3.
    // With three slots a block's first planes wait for their tiles twice
    // (the fourth prologue plane and the first output plane), so short z
    // chunks (small boxes, ensembles) keep the four-slot layout.
    bool db = false;
    if constexpr (sizeof(R) == 4) db = (resid || stage == 1 || stage == 4) && zc >= 16;
    auto go = [&](auto dbt) {
      constexpr bool DB = decltype(dbt)::value;
      const int bytes = (int)StageTm<R, MX, MY, DB>::BYTES;
      if (resid)
        k_stage_tm<R, MX, MY, true, DB><<<grid, MX * MY, bytes, s>>>(*mu, *mp, c, Uin, U0, Uout, Pout, Res, dyn,
                                                                     stage, zc, write_pres, nullptr);
      else
        k_stage_tm<R, MX, MY, false, DB><<<grid, MX * MY, bytes, s>>>(*mu, *mp, c, Uin, U0, Uout, Pout, Res, dyn,
                                                                      stage, zc, write_pres, Cc);
    };
    if constexpr (sizeof(R) == 4) {
      if (db) go(std::true_type());
      else go(std::false_type());
    } else {
      go(std::false_type());
    }
    return;
  }
  constexpr int PX = StageTile<R>::TX, PY = StageTile<R>::TY;
  const int bytes = stage_smem_bytes();
  if (resid)
    k_stage<R, PX, PY, true><<<grid, PX * PY, bytes, s>>>(c, Uin, Pin, U0, Uout, Pout, Res, dyn, stage, zc, write_pres,
                                                          nullptr);
  else
    k_stage<R, PX, PY, false><<<grid, PX * PY, bytes, s>>>(c, Uin, Pin, U0, Uout, Pout, Res, dyn, stage, zc, write_pres,
                                                           Cc);
}

template <class R>
void Launch<R>::tvd(const Consts& c, int dir, int mode, int only_two_half, const R* Uin, const R* Pst, R* Uout,
                    Dyn* dyn, cudaStream_t s, int td, const TvdDiag<R>* dg, Rem<R>* Cc) {
  const Geom& g = c.g;
  TvdArgs ta;
  ta.dir = dir;
  ta.mode = mode;
  ta.only_two_half = only_two_half;
  ta.td = td > 0 ? td : 32;
  const long long sx = 1, sy = g.sx, sz = (long long)g.sx * g.sy;
  // pencil ranges of TVDlimit's three sweeps (src/tvdlimit_SR.C:199-205, 671-672)
  if (dir == 0) {
    ta.na = g.sy; ta.a0 = 0; ta.sa = sy;
    ta.nb = g.sz; ta.b0 = 0; ta.sb = sz;
    ta.sd = sx; ta.n1 = g.nx;
  } else if (dir == 1) {
    ta.na = g.nx; ta.a0 = GH; ta.sa = sx;
    ta.nb = g.sz; ta.b0 = 0; ta.sb = sz;
    ta.sd = sy; ta.n1 = g.ny;
  } else {
    ta.na = g.nx; ta.a0 = GH; ta.sa = sx;
    ta.nb = g.ny; ta.b0 = GH; ta.sb = sy;
    ta.sd = sz; ta.n1 = g.nz;
  }
  const long long nch = (ta.n1 + ta.td - 1) / ta.td;
  const long long total = (long long)ta.na * ta.nb * nch;
  const int block = 128;
  const long long blocks = (total + block - 1) / block;
  if (dg) {
    if (dir == 0) k_tvd_sweep<R, 0, true><<<(unsigned)blocks, block, 0, s>>>(c, Uin, Pst, Uout, dyn, ta, *dg, nullptr);
    else if (dir == 1) k_tvd_sweep<R, 1, true><<<(unsigned)blocks, block, 0, s>>>(c, Uin, Pst, Uout, dyn, ta, *dg, nullptr);
    else k_tvd_sweep<R, 2, true><<<(unsigned)blocks, block, 0, s>>>(c, Uin, Pst, Uout, dyn, ta, *dg, nullptr);
    return;
  }
  const TvdDiag<R> nod{nullptr, (R)0, (R)0};
  if (dir == 0 && mode == 0) {
    // contiguous pencils: one cell per lane, 28 updates per warp
    const long long warps = (long long)g.sy * g.sz * ((g.nx + 27) / 28);
    long long nb = (warps * 32 + block - 1) / block;
    if (nb > 152LL * 16) nb = 152LL * 16;   // grid-stride: a few waves of resident blocks
    (Cc ? k_tvd_sweep_xlanes<R, true> : k_tvd_sweep_xlanes<R, false>)<<<(unsigned)nb, block, 0, s>>>(c, Uin, Pst, Uout, dyn, only_two_half, Cc);
    return;
  }
  if (dir == 0) (Cc ? k_tvd_sweep<R, 0, false, true> : k_tvd_sweep<R, 0, false, false>)<<<(unsigned)blocks, block, 0, s>>>(c, Uin, Pst, Uout, dyn, ta, nod, Cc);
  else if (dir == 1) (Cc ? k_tvd_sweep<R, 1, false, true> : k_tvd_sweep<R, 1, false, false>)<<<(unsigned)blocks, block, 0, s>>>(c, Uin, Pst, Uout, dyn, ta, nod, Cc);
  else (Cc ? k_tvd_sweep<R, 2, false, true> : k_tvd_sweep<R, 2, false, false>)<<<(unsigned)blocks, block, 0, s>>>(c, Uin, Pst, Uout, dyn, ta, nod, Cc);
}

template <class R>
int Launch<R>::divb_clean(const Consts& c, R* U, R* phi, R* divb, Dyn* dyn, cudaStream_t s) {
  const Geom& g = c.g;
  const dim3 block(DIVB_BX, DIVB_BY);
  const int bx = (g.nx + DIVB_BX - 1) / DIVB_BX, by = (g.ny + DIVB_BY - 1) / DIVB_BY;
  // z chunks: about 64 blocks per SM (short z marches keep more loads in flight)
  int nzch = (152 * 64 + bx * by - 1) / (bx * by);
  nzch = nzch < 1 ? 1 : (nzch > g.nz ? g.nz : nzch);
  const int zc = (g.nz + nzch - 1) / nzch;
  const dim3 grid(bx, by, (g.nz + zc - 1) / zc);
  const int maxit = c.divb_itmax > 3 ? c.divb_itmax : 3;
  k_divb_begin<<<1, 32, 0, s>>>(dyn);
  k_divb_div<R><<<grid, block, 0, s>>>(c, U, phi, divb, dyn, 0, zc);
  for (int it = 0; it < maxit; it++) {
    k_divb_grad<R><<<grid, block, 0, s>>>(c, U, phi, divb, dyn, it, zc);
    k_divb_div<R><<<grid, block, 0, s>>>(c, U, phi, divb, dyn, it + 1, zc);
  }
  k_divb_end<<<1, 32, 0, s>>>(c, dyn);
  return 3 + 2 * maxit;
}
template <class R>
int Launch<R>::bc(const Consts& c, R* U, R* P, Dyn* dyn, double* part, int with_cmax, cudaStream_t s, R* sflx) {
  const Geom& g = c.g;
  const dim3 gs((g.ny + BND_BX - 1) / BND_BX, (g.nz + BND_BY - 1) / BND_BY);
  k_bc_sums<R><<<gs, dim3(BND_BX, BND_BY), 0, s>>>(c, U, dyn, part);
  k_bc_setup<<<1, BND_SETUP_THREADS, 0, s>>>(c, dyn, part, (int)(gs.x * gs.y));
  const long long cols = (long long)g.sy * g.sz;
  k_bc_ghosts<R><<<(unsigned)((2 * cols + BND_THREADS - 1) / BND_THREADS), BND_THREADS, 0, s>>>(c, U, P, dyn, with_cmax,
                                                                                              sflx);
  return 3;
}
template <class R>
void Launch<R>::temp(const Consts& c, const R* U, R* T, cudaStream_t s) {
  k_temp<R><<<grid_for(c.g.N, 256), 256, 0, s>>>(c, U, T);
}
template <class R>
void Launch<R>::spitzer(const Consts& c, const R* U, bool prim, const R* T, const R* S, const R* S0, R* Sout, R* Rflx,
                        R* Rsp, const Dyn* dyn, int stage, cudaStream_t s) {
  const Geom& g = c.g;
  const int bx = (g.nx + SPT_BX - 1) / SPT_BX, by = (g.ny + SPT_BY - 1) / SPT_BY;
  // z chunks: about 16 blocks per SM
  int nzch = (152 * 16 + bx * by - 1) / (bx * by);
  nzch = nzch < 1 ? 1 : (nzch > g.nz ? g.nz : nzch);
  const int zc = (g.nz + nzch - 1) / nzch;
  const dim3 grid(bx, by, (g.nz + zc - 1) / zc), block(SPT_BX, SPT_BY);
  if (prim) k_spitzer<R, true><<<grid, block, 0, s>>>(c, U, T, S, S0, Sout, Rflx, Rsp, dyn, stage, zc);
  else k_spitzer<R, false><<<grid, block, 0, s>>>(c, U, T, S, S0, Sout, Rflx, Rsp, dyn, stage, zc);
}
template <class R>
void Launch<R>::sflx_update(const Consts& c, R* S, const R* S0, R* Rflx, const Dyn* dyn, int stage, cudaStream_t s) {
  k_sflx_update<R><<<grid_for((long long)c.g.nx * c.g.ny * c.g.nz, 256), 256, 0, s>>>(c, S, S0, Rflx, dyn, stage);
}
template <class R>
void Launch<R>::step_finish(const Consts& c, R* U, R* P, Dyn* dyn, cudaStream_t s, Rem<R>* Cc) {
  const Geom& g = c.g;
  const dim3 block(FIN_BX, FIN_BY);
  // z planes per block: one wave of resident blocks (each block marches
  // through its share of the planes), so that the statistics atomics (one per
  // statistic and block) stay few
  const int bxy = ((g.nx + FIN_BX - 1) / FIN_BX) * ((g.ny + FIN_BY - 1) / FIN_BY);
  int gz = (152 * FinBlocks<R>::v) / bxy;
  gz = gz < 1 ? 1 : (gz > g.nz ? g.nz : gz);
  const dim3 grid((g.nx + FIN_BX - 1) / FIN_BX, (g.ny + FIN_BY - 1) / FIN_BY, gz);
  (Cc ? k_step_finish<R, true> : k_step_finish<R, false>)<<<grid, block, 0, s>>>(c, U, P, dyn, Cc);
}
template <class R>
void Launch<R>::cons_to_prim(const Consts& c, R* U, R* P, R* T, R* Ne, R* Ri, R* Am, bool snapshot, cudaStream_t s) {
  (snapshot ? k_cons_to_prim<R, true> : k_cons_to_prim<R, false>)<<<grid_for(c.g.N, 256), 256, 0, s>>>(c, U, P, T, Ne,
                                                                                                      Ri, Am);
}
template <class R>
void Launch<R>::aux_of_snapshot(const Consts& c, R* T, R* Ne, R* Ri, R* Am, cudaStream_t s) {
  k_aux_of_snapshot<R><<<grid_for(c.g.N, 256), 256, 0, s>>>(c, T, Ne, Ri, Am);
}
template <class R>
void Launch<R>::init_pass(const Consts& c, const R* U, R* P, Dyn* dyn, cudaStream_t s) {
  k_init_pass<R><<<grid_for(c.g.N, 256), 256, 0, s>>>(c, U, P, dyn);
}
template <class R>
void Launch<R>::adjust_stats(const Consts& c, const R* U, const R* P, Dyn* dyn, cudaStream_t s) {
  k_adjust_stats<R><<<grid_for((long long)c.g.nx * c.g.ny * c.g.nz, 256), 256, 0, s>>>(c, U, P, dyn);
}
template <class R>
void Launch<R>::cmax_faces(const Consts& c, const R* U, const R* P, Dyn* dyn, cudaStream_t s) {
  const Geom& g = c.g;
  long long n = 2LL * GH * ((long long)g.ny * g.nz + (long long)g.nx * g.nz + (long long)g.nx * g.ny);
  k_cmax_faces<R><<<grid_for(n, 256), 256, 0, s>>>(c, U, P, dyn);
}
template <class R>
void Launch<R>::cfl_cons(const Consts& c, const R* U, const R* P, Dyn* dyn, cudaStream_t s) {
  const long long n = (long long)c.g.nx * c.g.ny * c.g.nz;
  k_cfl_cons<R><<<grid_for(n, 256), 256, 0, s>>>(c, U, P, dyn);
}
template <class R>
void Launch<R>::source_integrate(const Consts& c, R* U, const R* U0, R* Res, const Dyn* dyn, int stage, cudaStream_t s,
                                 R* diag, R invdt) {
  // one cell per thread: more loads in flight than a capped grid-stride loop (0.93 against 1.14 ms at 18.9 M cells)
  const long long n = (long long)c.g.nx * c.g.ny * c.g.nz;
  k_source_integrate<R><<<(int)((n + 255) / 256), 256, 0, s>>>(c, U, U0, Res, dyn, stage, diag, invdt);
}
template <class R>
void Launch<R>::save_cons(const Consts& c, const R* U, R* U0, cudaStream_t s) {
  k_save_cons<R><<<grid_for((long long)c.g.nx * c.g.ny * c.g.nz, 256), 256, 0, s>>>(c.g, U, U0);
}
template <class R>
void Launch<R>::tcheck(const Consts& c, R* U, const Dyn* dyn, cudaStream_t s, R* diag, R invdt) {
  k_tcheck<R><<<grid_for((long long)c.g.nx * c.g.ny * c.g.nz, 256), 256, 0, s>>>(c, U, dyn, diag, invdt);
}
template <class R>
void Launch<R>::diag_residual(const Consts& c, const R* U, const R* P, const R* S, R* diag, const Dyn* dyn,
                              cudaStream_t s) {
  k_diag_residual<R><<<grid_for((long long)c.g.nx * c.g.ny * c.g.nz, 256), 256, 0, s>>>(c, U, P, S, diag, dyn);
}
template <class R>
void Launch<R>::tile_state(const Geom& gd, const Geom& gs, const R* Us, R* Ud, cudaStream_t s) {
  k_tile_state<R><<<grid_for((long long)gd.nx * gd.ny * gd.nz, 256), 256, 0, s>>>(gd, gs, Us, Ud);
}

template <class R>
void Launch<R>::fill_ghosts(const Consts& c, R* U, int nfield, int with_bc, cudaStream_t s) {
  const Geom& g = c.g;
  const long long ng = 2LL * GH * ((long long)g.sx * g.sy + (long long)g.sx * g.nz + (long long)g.ny * g.nz);
  k_fill_ghosts<R><<<grid_for(ng, 256), 256, 0, s>>>(g, U, nfield, with_bc);
}
template <class R>
void Launch<R>::aos_to_soa(long long N, int nf, const double* A, R* S, cudaStream_t s) {
  k_aos_to_soa<R, double><<<grid_for(N, 256), 256, 0, s>>>(N, nf, A, S);
}
template <class R>
void Launch<R>::soa_to_aos(long long N, int nf, const R* S, double* A, cudaStream_t s) {
  k_soa_to_aos<R, double><<<grid_for(N, 256), 256, 0, s>>>(N, nf, S, A);
}
template <class R>
void Launch<R>::aos_to_soa(long long N, int nf, const float* A, R* S, cudaStream_t s) {
  k_aos_to_soa<R, float><<<grid_for(N, 256), 256, 0, s>>>(N, nf, A, S);
}
template <class R>
void Launch<R>::soa_to_aos(long long N, int nf, const R* S, float* A, cudaStream_t s) {
  k_soa_to_aos<R, float><<<grid_for(N, 256), 256, 0, s>>>(N, nf, S, A);
}
#endif

}  // namespace gpumhd
