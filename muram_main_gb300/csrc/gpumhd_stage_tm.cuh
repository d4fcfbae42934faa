// RK stage kernel with TMA plane loads and a tensor-memory z-flux ring.
//
// Same arithmetic as k_stage (gpumhd_kernels.cuh), different data movement:
//
//  * the state and pressure of each z plane under the block's tile, with its
//    two-cell halo ((TX+4) x (TY+4) cells, 9 arrays), arrive in shared memory
//    by one cp.async.bulk.tensor per array group, issued by one thread three
//    planes ahead and tracked by an mbarrier per slot of a four-plane ring;
//  * each thread's five-plane ring of z fluxes (12 quantities) lives in tensor
//    memory (tcgen05.st / tcgen05.ld, one TMEM lane per thread), which leaves
//    shared memory to the plane tiles and the x / y flux buffers.
//
// Every mbarrier wait is bounded (about one second, or the test hook's limit);
// on expiry the kernel sets ERR_WAIT_TIMEOUT in the step-control block, waits
// (bounded, about one second) for the copies it issued, releases its tensor
// memory and returns.
#pragma once
#include <cuda.h>

#include "gpumhd_kernels.cuh"

namespace gpumhd {

enum { ERR_WAIT_TIMEOUT = 4 };

namespace tm {

constexpr long long WAIT_CYCLES = 2000000000LL;  // ~1 s at the GB300 SM clock

__device__ __forceinline__ unsigned su32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(su32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Wait for completion of phase `parity`; false after `limit` clock cycles.
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, unsigned parity, long long limit = WAIT_CYCLES) {
  if (mbar_try_wait(b, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(b, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* m, int c0, int c1, int c2, int c3,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(su32(dst)),
      "l"(reinterpret_cast<unsigned long long>(m)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(su32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* m, int c0, int c1, int c2,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(su32(dst)),
      "l"(reinterpret_cast<unsigned long long>(m)), "r"(c0), "r"(c1), "r"(c2), "r"(su32(bar))
      : "memory");
}

// Tensor memory: allocation by one warp, per-thread lane access (32x32b shape).
__device__ __forceinline__ void tmem_alloc(unsigned* dst, unsigned ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(dst)), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(unsigned taddr, unsigned ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_st4(unsigned t, unsigned a, unsigned b, unsigned c, unsigned d) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(t), "r"(a), "r"(b), "r"(c),
               "r"(d)
               : "memory");
}
__device__ __forceinline__ void tmem_ld4(unsigned t, unsigned& a, unsigned& b, unsigned& c, unsigned& d) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(a), "=r"(b), "=r"(c), "=r"(d)
               : "r"(t)
               : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
// Waits for this thread's tensor-memory loads; the 16 registers pass through
// the instruction so that no use of them is scheduled before it.
__device__ __forceinline__ void tmem_wait_ld16(unsigned* r) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
               :
               : "memory");
}

}  // namespace tm

// Shared-memory layout of one k_stage_tm block.
template <class R, int TX, int TY, bool DB_>
struct StageTm {
  static constexpr int BX = TX + 4, BY = TY + 4;  // TMA box of one plane (x, y)
  static constexpr int BOXN = BX * BY;
  static constexpr unsigned UB = (unsigned)(sizeof(R) * BOXN * NV);  // state box bytes ([v][y][x])
  static constexpr unsigned PB = (unsigned)(sizeof(R) * BOXN);       // pressure box bytes, right after
  static constexpr size_t TILE = ((size_t)UB + PB + 127) / 128 * 128;
  // DB: three plane slots and two x / y flux buffers used in turn, so that
  // one barrier per plane suffices (the next plane's fluxes go to the other
  // buffer; a slot is refilled right after the barrier of the plane that
  // last reads it).  Otherwise four slots and one flux buffer, two barriers
  // per plane.  Two blocks per SM fit either way in FP32; FP64 uses the
  // latter only.  Measured at 128 x 384 x 384 (FP32): DB is faster for the
  // stages that read no separate U0 (stage 1: 0.76 against 0.79 ms; stage 4,
  // whose U0 is its output, 0.62 against 0.67 ms; the residual), slower for
  // stages 2 and 3 (0.80 against 0.78 ms), whose U0 loads and EOS gathers
  // then have less L1 beside the larger shared memory.
  static constexpr bool DB = DB_;
  static constexpr int NSLOT = DB ? 3 : 4;
  static constexpr int NFB = DB ? 2 : 1;
  static constexpr int FXN = BX * TY, FYN = TX * BY;
  static constexpr size_t FSET = sizeof(R) * 12 * (FXN + FYN);  // one x + y flux buffer pair
  static constexpr size_t OFF_FX = NSLOT * TILE;                  // set b: x at OFF_FX + b * FSET, y after it
  static constexpr size_t OFF_BAR = OFF_FX + NFB * FSET;
  static constexpr size_t OFF_MISC = OFF_BAR + 8 * NSLOT;  // TMEM address, flags
  static constexpr size_t BYTES = OFF_MISC + 16 + 128;     // + alignment slack
  // tensor memory: per thread 5 slots x 12 quantities (32-bit columns)
  static constexpr int WPQ = sizeof(R) / 4;              // columns per value
  static constexpr int SLOT_COLS = 12 * WPQ;
  static constexpr int NWARP = TX * TY / 32;
  static constexpr int WARP_COLS = 64 * WPQ;             // column block of each warp sharing a lane quadrant
  static constexpr int TMEM_COLS = ((NWARP + 3) / 4) * WARP_COLS;
  static_assert(5 * SLOT_COLS <= WARP_COLS, "z ring fits the warp's column block");
  static_assert(TMEM_COLS == 32 || TMEM_COLS == 64 || TMEM_COLS == 128 || TMEM_COLS == 256, "TMEM allocation size");
};

// 12 flux quantities to tensor-memory slot `col` of this thread's lane.
__device__ __forceinline__ void tm_store12(unsigned ta, const float* f) {
#pragma unroll
  for (int a = 0; a < 3; a++)
    tm::tmem_st4(ta + 4 * a, __float_as_uint(f[4 * a]), __float_as_uint(f[4 * a + 1]), __float_as_uint(f[4 * a + 2]),
                 __float_as_uint(f[4 * a + 3]));
}
__device__ __forceinline__ void tm_store12(unsigned ta, const double* f) {
#pragma unroll
  for (int a = 0; a < 6; a++) {
    const unsigned long long u0 = __double_as_longlong(f[2 * a]), u1 = __double_as_longlong(f[2 * a + 1]);
    tm::tmem_st4(ta + 4 * a, (unsigned)u0, (unsigned)(u0 >> 32), (unsigned)u1, (unsigned)(u1 >> 32));
  }
}

// z derivative of the 12 quantities from the ring slots of planes k-2, k-1,
// k+1, k+2 (column addresses m2, m1, p1, p2), in the order of deriv12.
__device__ __forceinline__ void tm_deriv12(float* Dq, unsigned m2, unsigned m1, unsigned p1, unsigned p2, float w1,
                                           float w2) {
  const float2 neg = make_float2(-1.0f, -1.0f), W1 = make_float2(w1, w1), W2 = make_float2(w2, w2);
#pragma unroll
  for (int a = 0; a < 3; a++) {
    unsigned r[16];
    tm::tmem_ld4(m2 + 4 * a, r[0], r[1], r[2], r[3]);
    tm::tmem_ld4(m1 + 4 * a, r[4], r[5], r[6], r[7]);
    tm::tmem_ld4(p1 + 4 * a, r[8], r[9], r[10], r[11]);
    tm::tmem_ld4(p2 + 4 * a, r[12], r[13], r[14], r[15]);
    tm::tmem_wait_ld16(r);
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const float2 a2 = make_float2(__uint_as_float(r[2 * h]), __uint_as_float(r[2 * h + 1]));
      const float2 a1 = make_float2(__uint_as_float(r[4 + 2 * h]), __uint_as_float(r[5 + 2 * h]));
      const float2 b1 = make_float2(__uint_as_float(r[8 + 2 * h]), __uint_as_float(r[9 + 2 * h]));
      const float2 b2 = make_float2(__uint_as_float(r[12 + 2 * h]), __uint_as_float(r[13 + 2 * h]));
      const float2 d1 = __ffma2_rn(a1, neg, b1);
      const float2 d2 = __ffma2_rn(a2, neg, b2);
      const float2 res = __ffma2_rn(W1, d1, __fmul2_rn(W2, d2));
      Dq[4 * a + 2 * h] = res.x;
      Dq[4 * a + 2 * h + 1] = res.y;
    }
  }
}
__device__ __forceinline__ void tm_deriv12(double* Dq, unsigned m2, unsigned m1, unsigned p1, unsigned p2, double w1,
                                           double w2) {
#pragma unroll
  for (int a = 0; a < 6; a++) {
    unsigned r[16];
    tm::tmem_ld4(m2 + 4 * a, r[0], r[1], r[2], r[3]);
    tm::tmem_ld4(m1 + 4 * a, r[4], r[5], r[6], r[7]);
    tm::tmem_ld4(p1 + 4 * a, r[8], r[9], r[10], r[11]);
    tm::tmem_ld4(p2 + 4 * a, r[12], r[13], r[14], r[15]);
    tm::tmem_wait_ld16(r);
#pragma unroll
    for (int h = 0; h < 2; h++) {
      auto dbl = [&](int o) {
        return __longlong_as_double((long long)(((unsigned long long)r[o + 1] << 32) | (unsigned long long)r[o]));
      };
      const double a2 = dbl(2 * h), a1 = dbl(4 + 2 * h), b1 = dbl(8 + 2 * h), b2 = dbl(12 + 2 * h);
      Dq[2 * a + h] = w1 * (b1 - a1) + w2 * (b2 - a2);
    }
  }
}

// Launch: grid (ceil(nx/TX), ceil(ny/TY), z chunks), TX*TY threads,
// StageTm::BYTES of dynamic shared memory.  mapU: the input state as a 4-D
// tensor (x, y, z, variable), box (TX+4, TY+4, 1, 8); mapP: its pressure,
// box (TX+4, TY+4, 1); Ug: the same state as a pointer (read for the
// resistive terms only).  Other arguments as k_stage.
template <class R, int TX, int TY, bool RESID, bool DB>
__global__ void __launch_bounds__(TX* TY, 2)
    k_stage_tm(const __grid_constant__ CUtensorMap mapU, const __grid_constant__ CUtensorMap mapP, Consts c,
               const R* __restrict__ Ug, const R* __restrict__ U0, R* __restrict__ Uout, R* __restrict__ Pout,
               R* __restrict__ Res,
               Dyn* __restrict__ dyn, int stage, int zc, int write_pres, Rem<R>* __restrict__ Cc) {
  using L = StageTm<R, TX, TY, DB>;
  static_assert(!DB || sizeof(R) == 4, "the double-buffered layout is for FP32");
  constexpr int CW = CellW<R>::W;
  constexpr int NT = TX * TY;
  constexpr int NH = 4 * TY + 4 * TX;
  static_assert(NH <= NT, "every halo cell needs a thread");
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = smem_raw + ((128u - (tm::su32(smem_raw) & 127u)) & 127u);
  auto fx_of = [&](int b) { return reinterpret_cast<R*>(sm + L::OFF_FX + (size_t)b * L::FSET); };
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(sm + L::OFF_BAR);
  unsigned* misc = reinterpret_cast<unsigned*>(sm + L::OFF_MISC);  // [0] TMEM base, [1] skip, [2] timeout
  const Geom& g = c.g;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int tx = tid % TX, ty = tid / TX;
  if (tid == 0) {
    misc[1] = RESID ? 0u : (unsigned)(*(volatile int*)&dyn->err);
    misc[2] = 0u;
    for (int s = 0; s < L::NSLOT; s++) tm::mbar_init(&bar[s], 1);
    tm::fence_mbar_init();
    tm::fence_proxy_async();
  }
  __syncthreads();
  if (misc[1]) return;  // an earlier launch of the step failed (uniform for the block)
  if (warp == 0) {
    tm::tmem_alloc(&misc[0], L::TMEM_COLS);
    tm::tmem_relinquish();
  }
  tm::tc_fence_before();
  __syncthreads();
  tm::tc_fence_after();
  const unsigned tmem = misc[0];
  // this thread's lane (its warp's quadrant) and its warp's column block
  const unsigned ta = tmem + ((unsigned)((warp & 3) * 32) << 16) + (unsigned)((warp >> 2) * L::WARP_COLS);

  const int bx0 = blockIdx.x * TX, by0 = blockIdx.y * TY;  // box origin = tile origin - 2 (x0 - GH, y0 - GH)
  const int x0 = GH + bx0, y0 = GH + by0;
  const int zb = GH + blockIdx.z * zc;
  const int ze = min(zb + zc, GH + g.nz);
  const int i = x0 + tx, j = y0 + ty;
  const bool active = (i < GH + g.nx) && (j < GH + g.ny);
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
  const KC<R>& kk_ = kc<R>(c);
  const DynR<R>& dr = dynr<R>(dyn);
  const R inv_va2max = dr.inv_va2max;
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

  // plane tiles: plane p is tile t = p - (zb - 2), slot t % NSLOT, phase (t / NSLOT) % 2
  const int p_first = zb - 2;
  auto tile = [&](int p) { return reinterpret_cast<const R*>(sm + (size_t)((p - p_first) % L::NSLOT) * L::TILE); };
  // test hook: the last plane's copy is never issued, so its wait runs out
  const int withheld = c.tm_withhold_last ? ze + 1 : -1;
  const long long wait_limit = c.tm_wait_cycles > 0 ? c.tm_wait_cycles : tm::WAIT_CYCLES;
  auto issue = [&](int p) {  // one thread
    if (p == withheld) return;
    const int t = p - p_first, sl = t % L::NSLOT;
    unsigned char* dst = sm + (size_t)sl * L::TILE;
    tm::fence_proxy_async();
    tm::mbar_arrive_expect_tx(&bar[sl], L::UB + L::PB);
    tm::tma_load_4d(dst, &mapU, bx0, by0, p, 0, &bar[sl]);
    tm::tma_load_3d(dst + L::UB, &mapP, bx0, by0, p, &bar[sl]);
  };
  bool timed_out = false;
  auto wait_tile = [&](int p) {
    const int t = p - p_first;
    if (!tm::mbar_wait(&bar[t % L::NSLOT], (unsigned)((t / L::NSLOT) & 1), wait_limit)) timed_out = true;
  };
  // cell offsets inside a tile: own cell and halo cell
  const int o_own = (ty + 2) * L::BX + (tx + 2);
  const int o_halo = (hly + 2) * L::BX + (hlx + 2);
  auto raw_at = [&](const R* T, int o, Raw9<R>& r) {
#pragma unroll
    for (int q = 0; q < 9; q++) r.v[q] = T[q * L::BOXN + o];
  };
  // z-flux ring in tensor memory: slot s at columns s * SLOT_COLS
  auto zcol = [&](int s) { return ta + (unsigned)(s * L::SLOT_COLS); };
  auto slot_add = [](int sl, int d) { return sl + d >= 5 ? sl + d - 5 : sl + d; };

  if (tid == 0)
    for (int p = zb - 2; p < zb - 2 + L::NSLOT; p++) issue(p);
  for (int p = zb - 2; p < zb + 2; p++) {
    if (L::DB && p == zb + 1) {  // the fourth prologue plane takes the first plane's slot
      tm::tmem_wait_st();
      __syncthreads();
      if (tid == 0) issue(p);
    }
    wait_tile(p);
    __syncwarp();
    Raw9<R> r;
    raw_at(tile(p), o_own, r);
    prim_of_raw<R, RESID>(r, prim);
    flux12<R, 2>(prim, 1, fl, 1);
    tm_store12(zcol(p - zb + 2), fl);
  }
  tm::tmem_wait_st();
  __syncthreads();
  if (tid == 0) issue(zb + 2);

  const unsigned plane = (unsigned)g.sx * (unsigned)g.sy;
  const unsigned own0 = cidx32(g, i, j, 0);
  // The new state's pressure of plane k is looked up at the end of plane k
  // and stored during plane k+1, so the table loads overlap that plane's work.
  PresLookup<R> plook;
  bool pend = false;
  auto finish_pressure = [&](int kp) {
    const R pr = eos_pres_end(plook);
    for_col_images(own0 + (unsigned)kp * plane, col_images(g, i, j, true), z_image_off(g, kp),
                   [&](unsigned t, bool) { Pout[t] = pr; });
    pend = false;
  };
  int s0 = 2;  // ring slot of plane k
  for (int k = zb; k < ze; k++, s0 = slot_add(s0, 1)) {
    if (!L::DB && tid == 0 && k + 1 < ze) issue(k + 3);
    R* const FX = fx_of(L::DB ? ((k - zb) & 1) : 0);
    R* const FY = FX + 12 * L::FXN;
    // z flux of plane k+2 (all lanes: tensor-memory stores are warp-wide)
    wait_tile(k + 2);
    __syncwarp();
    {
      Raw9<R> r;
      raw_at(tile(k + 2), o_own, r);
      prim_of_raw<R, RESID>(r, prim);
      flux12<R, 2>(prim, 1, fl, 1);
      tm_store12(zcol(slot_add(s0, 2)), fl);
    }
    // own cell: primitives and x / y fluxes; halo cell: its x or y flux
    R cen[NF];
    {
      const R* T = tile(k);
      Raw9<R> r;
      raw_at(T, o_own, r);
      prim_of_raw<R, RESID>(r, cen);
      cen[NPRIM] = (R)0;
      flux12<R, 0>(cen, 1, fl, 1);
      store_cell(FX + (ty * L::BX + tx + 2) * CW, fl);
      flux12<R, 1>(cen, 1, fl, 1);
      store_cell(FY + ((ty + 2) * TX + tx) * CW, fl);
      if (tid < NH) {
        raw_at(T, o_halo, r);
        prim_of_raw<R, RESID>(r, prim);
        if (hx) {
          flux12<R, 0>(prim, 1, fl, 1);
          store_cell(FX + (hly * L::BX + hlx + 2) * CW, fl);
        } else {
          flux12<R, 1>(prim, 1, fl, 1);
          store_cell(FY + ((hly + 2) * TX + hlx) * CW, fl);
        }
      }
    }
    const unsigned id = own0 + (unsigned)k * plane;
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
    if (pend) finish_pressure(k - 1);
    tm::tmem_wait_st();
    __syncthreads();
    // FP32: plane k's slot is free (its last reads were this plane's own and
    // halo cells), refill it with plane k+3, read in the next plane
    if (L::DB && tid == 0 && k + 1 < ze) issue(k + 3);
    // z derivative (all lanes), then the cell's residual and update
    R Dz[NF];
    __syncwarp();
    tm_deriv12(Dz, zcol(slot_add(s0, 3)), zcol(slot_add(s0, 4)), zcol(slot_add(s0, 1)), zcol(slot_add(s0, 2)),
               kk_.w1[2], kk_.w2[2]);
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
        {
          R Dq[NF];
          const R* fb = FX + (ty * L::BX + tx + 2) * CW;
          deriv12(Dq, fb - 2 * CW, fb - CW, fb + CW, fb + 2 * CW, kk_.w1[0], kk_.w2[0]);
          if (ETA) eta_lap<R>(c, Ug, id, 1u, 0, cen, lap);
          apply_direction<R, 0, ETA>(Racc, Dq, cen, lf, kk_.eta, cb, lap);
        }
        {
          R Dq[NF];
          const R* fb = FY + ((ty + 2) * TX + tx) * CW;
          deriv12(Dq, fb - 2 * TX * CW, fb - TX * CW, fb + TX * CW, fb + 2 * TX * CW, kk_.w1[1], kk_.w2[1]);
          if (ETA) eta_lap<R>(c, Ug, id, (unsigned)g.sx, 1, cen, lap);
          apply_direction<R, 1, ETA>(Racc, Dq, cen, lf, kk_.eta, cb, lap);
        }
        if (ETA) eta_lap<R>(c, Ug, id, plane, 2, cen, lap);
        apply_direction<R, 2, ETA>(Racc, Dz, cen, lf, kk_.eta, cb, lap);
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
        store_state_col<R>(g, Uout, id, col_images(g, i, j, true), z_image_off(g, k), un);
        if (write_pres) {
          R v1, v2, v3, ei;
          prim_from_cons(un[0], un[1], un[2], un[3], un[4], v1, v2, v3, ei);
          eos_pres_begin(c, un[0], ei, (R)1.0 / un[0], plook);
          pend = true;
        }
      }
    }
    if (!L::DB) __syncthreads();  // FP64: the flux buffer is rewritten by the next plane
  }
  if (pend) finish_pressure(ze - 1);
  if (RESID) {  // one atomic per block
    const R m = block_max_nonnan(cm_acc);
    if (tid == 0) atomic_max_nonneg(&dyn->cmax_bits, (double)m);
  }

  // teardown: report an expired wait, let issued copies land, free tensor memory
  if (timed_out) atomicExch(&misc[2], 1u);
  tm::tc_fence_before();
  __syncthreads();
  if (misc[2]) {
    if (tid == 0) {
      atomicExch(&dyn->err, (int)ERR_WAIT_TIMEOUT);
      // the last NSLOT tiles issued are the only ones that can be in flight
      const int p_last = max(ze + 1, zb + 2);
      for (int p = max(p_first, p_last - (L::NSLOT - 1)); p <= p_last; p++) {
        if (p == withheld) continue;  // never issued
        const int t = p - p_first;
        tm::mbar_wait(&bar[t % L::NSLOT], (unsigned)((t / L::NSLOT) & 1));
      }
    }
    __syncthreads();
  }
  if (warp == 0) {
    __syncwarp();
    tm::tmem_dealloc(tmem, L::TMEM_COLS);
  }
}

}  // namespace gpumhd
