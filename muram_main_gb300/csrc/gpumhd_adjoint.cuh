// Launchers of the adjoint kernels (adjoint.cu): one RK stage, the EOS
// pressure and one TVD sweep of the fused step, transposed.  FP64, periodic
// boxes; adjoint fields are interior-only (nx*ny*nz per variable).
#pragma once
#include "gpumhd_launch.cuh"

namespace gpumhd {

// Work arrays of one TVD-sweep adjoint (interior-sized, doubles):
// in 8, cell 19, fp 9, fm 9, iface 92, slope 57 values per cell.
struct AdjTvdScratch {
  double* in;
  double* cell;
  double* fp;
  double* fm;
  double* iface;
  double* slope;
  double* tcell;  // the sweep's per-cell TVD quantities, 19 per node of the ghosted box
};
constexpr int ADJ_TVD_DOUBLES = 8 + 19 + 9 + 9 + 92 + 57;
constexpr int ADJ_STAGE_DOUBLES = 36 + 11;

// Stage `stage` (1..4) with input Uin / Pin (its pressure) and step state U0;
// lam_out: adjoint of the stage's output.  lam_u0 += the U0 part;
// lam_uin = the input part; lam_pin += the pressure part.  buf_dq (36 per
// cell) and buf_wc (11 per cell) are work arrays.
void adjoint_stage(const Consts& c, const Dyn* dyn, const double* Uin, const double* Pin, const double* U0,
                   const double* lam_out, double* lam_u0, double* lam_uin, double* lam_pin, double* buf_dq,
                   double* buf_wc, int stage, cudaStream_t s);
// lam_u += (dp/dU)^T lam_p for the pressure p(U) of ConsToPrim.
void adjoint_eos(const Consts& c, const double* U, const double* lam_p, double* lam_u, cudaStream_t s);
// TVD sweep along dir of input V with stale pressure P (final_pass: the last
// sweep, with TCheck); lam_in = adjoint of V; lam_p += the pressure part.
void adjoint_tvd(const Consts& c, const Dyn* dyn, int dir, const double* V, const double* P, const double* lam_out,
                 int final_pass, double* lam_in, double* lam_p, const AdjTvdScratch& w, cudaStream_t s);

// Host cState records (8 doubles per cell, ghosts included) to / from the
// interior adjoint layout; out = x + y over the 8 interior fields.
void adjoint_from_cstate(const Consts& c, const double* aos, double* lam, cudaStream_t s);
void adjoint_to_cstate(const Consts& c, const double* lam, double* aos, cudaStream_t s);
void adjoint_add(const Consts& c, const double* x, const double* y, double* out, cudaStream_t s);

}  // namespace gpumhd
