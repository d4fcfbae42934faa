// MURaM-side binding of the gpumhd library.
//
// Drop this file into MURaM's src/ and link libgpumhd.so in place of the
// objects of the hot-path routines it defines (src/Makefile:10-42):
//   cons_to_prim.o (ConsToPrim only; keep eos_init.o for the host EOS tables),
//   mhdres_SR.o, tvdlimit_SR.o, Add_Sources_Integrate_SR.o, Adjust_Valf_Max.o,
//   boundary_pdmp_1_fftw3.o (SetBoundaryConditions), clean_divB.o (Clean_divB),
//   the exchange_grid_acc of exchange.o, and ACCH::UpdateCPU/UpdateGPU of ACCH.o.
// Link with -Wl,--wrap=_Z8eos_initR8GridDataR7RunDataRK11PhysicsData (that is,
// eos_init): the reference's eos_init still builds the host EOS tables (other
// host code reads them), and the wrapper then creates the GPU context.  ComputeSolution (src/solver.C) is unchanged: each routine it
// calls keeps its signature and meaning, and works on the GPU-resident copy of
// GridData.
// Host arrays are refreshed only at ACCH::UpdateCPU, and the device copy
// only at ACCH::UpdateGPU, as with the reference's OpenACC build.
//
// Scope: MHD with the Boris correction, gravity, constant resistivity eta,
// hyperbolic Spitzer conduction, divB cleaning, periodic y/z, periodic x or
// MURaM's physical x boundaries without the potential-field top, constant Tau
// and Qtot = 0 (radiation outside the path).  Every other
// setting reports an error and aborts, as the reference does on invalid input.
#include <mpi.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "grid.H"
#include "physics.H"
#include "run.H"
#include "eos.H"
#include "mhd_tvd.H"
#include "src_int_tck.H"
#include "limit_va.H"
#include "exchange.H"
#include "ACCH.h"
#include "icbc.H"
#include "divB.H"
#include "gpumhd.h"

// include/limit_va.H:5 -- defined by Adjust_Valf_Max.C in the reference
double inv_va2max, v_lim = 0.0, e_lim = 0.0;
// the open bottom's pressure and entropy (src/boundary_pdmp_1_fftw3.C:31; read
// from backup.dat by ReadBackupFile, negative: set from the first boundary call)
double p_bc, s_bc;

namespace {

gpumhd_ctx* g_ctx = nullptr;
const GridData* g_grid = nullptr;

void die(const char* where, int rc) {
  fprintf(stderr, "gpumhd: %s failed (%d): %s\n", where, rc, gpumhd_last_error(g_ctx));
  MPI_Abort(MPI_COMM_WORLD, 1);
}

void check(const char* where, int rc) {
  if (rc != GPUMHD_OK) die(where, rc);
}

// GridData's cState arrays (U, U0) hold `real`: float in a SINGLE_PRECISION
// build (include/precision.h:4-10, include/physics.H:77), double otherwise;
// its other arrays are double in both (include/grid.H:53-100).
int upload_cstate(int which, const void* ptr) {
#ifdef SINGLE_PRECISION
  return gpumhd_upload_f32(g_ctx, which, static_cast<const float*>(ptr));
#else
  return gpumhd_upload(g_ctx, which, static_cast<const double*>(ptr));
#endif
}
int download_cstate(int which, void* ptr) {
#ifdef SINGLE_PRECISION
  return gpumhd_download_f32(g_ctx, which, static_cast<float*>(ptr));
#else
  return gpumhd_download(g_ctx, which, static_cast<double*>(ptr));
#endif
}

void fill_params(gpumhd_params& p, const RunData& Run, const GridData& Grid, const PhysicsData& Physics) {
  gpumhd_default_params(&p, Grid.lsize[0], Grid.lsize[1], Grid.lsize[2], Grid.dx[0]);
#ifdef GPUMHD_FP32
  p.precision = 32;
#endif
  p.periodic_x = Grid.periods[0];
  for (int d = 0; d < 3; d++) p.dx[d] = Grid.dx[d];
  p.CFL = Run.CFL;
  p.CFL_tvd = Run.CFL_tvd;
  p.dt = Run.dt;
  p.time = Run.time;
  p.outcad = Run.outcad;
  p.autostep = Run.autostep;
  p.grav = Physics.params[i_param_grav];
  p.va_max = Physics.params[i_param_va_max];
  p.va_adjust = Physics.params[i_param_va_adjust];
  p.max_fill = Physics.params[i_param_max_fill];
  for (int i = 0; i < 4; i++) {
    p.tvd_h[i] = Physics.tvd_h[i];
    p.tvd_cs[i] = Physics.tvd_cs[i];
    p.tvd_coeff[i] = Physics.tvd_coeff[i];
    p.tchk[i] = Physics.tchk[i];
  }
  for (int i = 0; i < 10; i++) p.tvd[i] = Physics.tvd[i];
  for (int i = 0; i < 2; i++) {
    p.tvd_h_bnd[i] = Physics.tvd_h_bnd[i];
    p.tvd_visc_bnd[i] = Physics.tvd_visc_bnd[i];
    p.tvd_eta_bnd[i] = Physics.tvd_eta_bnd[i];
  }
  p.rt_cfl = Physics.rt[i_rt_cfl];
  p.rt_tstep = Physics.rt[i_rt_tstep];
  p.rt_update = Physics.rt[i_rt_update];
  p.tau0 = Grid.Tau ? Grid.Tau[0] : 1.0;
  p.eta = Physics.params[i_param_eta];
  p.divB_switch = (int)Physics.divB[i_divB_switch];
  p.divB_itmax = (int)Physics.divB[i_divB_itmax];
  p.divB_err = Physics.divB[i_divB_err];
  // a closed x gets MURaM's physical boundaries (src/boundary_pdmp_1_fftw3.C:81-493)
  p.xbnd = Grid.periods[0] ? 0 : 1;
  p.bnd_top = (int)Physics.bnd[i_bnd_top];
  p.bnd_bcrit = Physics.bnd[i_bnd_bcrit];
  p.bnd_eps_top = Physics.bnd[i_bnd_eps_top];
  p.p_bc = p_bc;
  p.s_bc = s_bc;
  p.spitzer = Physics.params[i_param_spitzer];
}

const RunData* g_run = nullptr;
const PhysicsData* g_phys = nullptr;
double g_dt = -1.0, g_time = -1.0;
int g_need_diag = 0;

// Run.need_diagnostics (set by ComputeSolution per stage, src/solver.C:264-289):
// switching it on zeroes the diagnostic arrays as the reference does there.
void sync_diagnostics(gpumhd_ctx* c, const RunData& Run) {
  const int on = Run.need_diagnostics ? 1 : 0;
  if (on != g_need_diag) {
    check("need_diagnostics", gpumhd_set_need_diagnostics(c, on));
    g_need_diag = on;
  }
}

// The run parameters the device needs change only through Run.dt / Run.time
// (Sync_timestep, Run.Advance); push them when they did.
gpumhd_ctx* ctx() {
  if (!g_ctx) {
    fprintf(stderr, "gpumhd: hot-path routine called before eos_init\n");
    MPI_Abort(MPI_COMM_WORLD, 1);
  }
  if (g_run->dt != g_dt || g_run->time != g_time) {
    gpumhd_params p;
    fill_params(p, *g_run, *g_grid, *g_phys);
    check("set_params", gpumhd_set_params(g_ctx, &p));
    g_dt = g_run->dt;
    g_time = g_run->time;
  }
  return g_ctx;
}

}  // namespace

// eos_init (include/eos.H:38) keeps the reference's host tables; the wrapper
// then creates the GPU context and loads the same table file on the device.
// The linker's --wrap works on the mangled name of
// void eos_init(GridData&, RunData&, const PhysicsData&).
#define GPUMHD_EOS_INIT_MANGLED _Z8eos_initR8GridDataR7RunDataRK11PhysicsData
#define GPUMHD_CAT2(a, b) a##b
#define GPUMHD_CAT(a, b) GPUMHD_CAT2(a, b)
extern "C" void GPUMHD_CAT(__real_, GPUMHD_EOS_INIT_MANGLED)(GridData&, RunData&, const PhysicsData&);
extern "C" void GPUMHD_CAT(__wrap_, GPUMHD_EOS_INIT_MANGLED)(GridData& Grid, RunData& Run,
                                                            const PhysicsData& Physics) {
  GPUMHD_CAT(__real_, GPUMHD_EOS_INIT_MANGLED)(Grid, Run, Physics);
  if (Physics.params[i_param_ambipolar] > 0 || Physics.bnd[i_bnd_pot] > 0 || Physics.dmp[i_dmp_switch] > 0 ||
      Physics.rt_ext[i_ext_cor] > 0 || Grid.procs[0] * Grid.procs[1] * Grid.procs[2] != 1) {
    fprintf(stderr, "gpumhd: configuration outside the GPU path\n");
    MPI_Abort(MPI_COMM_WORLD, 1);
  }
  gpumhd_params p;
  fill_params(p, Run, Grid, Physics);
  check("create", gpumhd_create(&p, 0, &g_ctx));
  check("eos_init", gpumhd_eos_init(g_ctx, Run.eos_name));
  g_grid = &Grid;
  g_run = &Run;
  g_phys = &Physics;
  g_dt = Run.dt;
  g_time = Run.time;
}

// ---- the routines ComputeSolution calls (signatures from the reference headers)

void SaveCons(GridData& Grid, const PhysicsData& Physics) {          // include/src_int_tck.H:10
  check("SaveCons", gpumhd_save_cons(ctx()));
}

void ConsToPrim(GridData& Grid, const PhysicsData& Physics, const RunData& Run) {  // include/eos.H:39
  check("ConsToPrim", gpumhd_cons_to_prim(ctx()));
}

void Adjust_Valf_Max(const RunData& Run, const GridData& Grid, const PhysicsData& Physics) {  // include/limit_va.H:7
  gpumhd_ctx* c = ctx();
  check("Adjust_Valf_Max", gpumhd_adjust_valf_max(c));
  check("get_limits", gpumhd_get_limits(c, &inv_va2max, &v_lim, &e_lim));
}

double lfac(double va2) {  // include/limit_va.H:9
  double x2 = va2 * inv_va2max, x4 = x2 * x2, s = 1.0 + x2;
  return s / (s + x4);
}

double MHD_Residual(const RunData& Run, GridData& Grid, const PhysicsData& Physics) {  // include/mhd_tvd.H:5
  double dt_mhd = 0.0;
  gpumhd_ctx* c = ctx();
  sync_diagnostics(c, Run);
  check("MHD_Residual", gpumhd_mhd_residual(c, &dt_mhd));
  return dt_mhd;
}

void Source_Integrate_Tcheck(const RunData& Run, GridData& Grid, const PhysicsData& Physics,
                             const int stage) {  // include/src_int_tck.H:8-9
  gpumhd_ctx* c = ctx();
  sync_diagnostics(c, Run);
  check("Source_Integrate_Tcheck", gpumhd_source_integrate_tcheck(c, stage));
}

void TVDlimit(const RunData& Run, GridData& Grid, const PhysicsData& Physics, const double dt_tvd) {  // include/mhd_tvd.H:6
  gpumhd_ctx* c = ctx();
  sync_diagnostics(c, Run);
  check("TVDlimit", gpumhd_tvdlimit(c, dt_tvd));
}

void TCheck(const RunData& Run, GridData& Grid, const PhysicsData& Physics) {  // include/src_int_tck.H:7
  gpumhd_ctx* c = ctx();
  sync_diagnostics(c, Run);
  check("TCheck", gpumhd_tcheck(c));
}

void Clean_divB(const RunData& Run, GridData& Grid, const PhysicsData& Physics) {  // include/divB.H:5
  check("Clean_divB", gpumhd_clean_divB(ctx()));
}

void exchange_grid_acc(GridData& Grid, const PhysicsData& Physics, const int) {  // include/exchange.H:8
  if (!g_ctx) return;  // before eos_init the host state is still authoritative
  check("exchange", gpumhd_exchange(g_ctx, 0));
}

// SetBoundaryConditions (include/icbc.H:10-12): periodic x needs nothing
// beyond the exchange; a closed x gets MURaM's physical boundaries (open
// bottom, top per bnd_top; src/boundary_pdmp_1_fftw3.C:81-565), and p_bc /
// s_bc, which the first call may set, return to the globals for backup.dat.
// The potential-field top is outside the GPU path.
void SetBoundaryConditions(const RunData& Run, GridData& Grid, const PhysicsData& Physics, const int,
                           const int, RTS*) {
  if (!g_ctx || Grid.periods[0]) return;
  check("boundaries", gpumhd_exchange(ctx(), 1));
  check("boundary info", gpumhd_boundary_info(g_ctx, &p_bc, &s_bc));
}

// ACCH::UpdateCPU / UpdateGPU (src/ACCH.C:114-158) for the arrays the library owns.
namespace ACCH {
void UpdateCPU(void* ptr, std::size_t) {
  if (!g_ctx || !g_grid) return;
  if (ptr == g_grid->U) check("download U", download_cstate(0, ptr));
  else if (ptr == g_grid->U0) check("download U0", download_cstate(1, ptr));
  else if (ptr == g_grid->pres) check("download pres", gpumhd_download(g_ctx, 3, (double*)ptr));
  else if (ptr == g_grid->temp) check("download temp", gpumhd_download(g_ctx, 4, (double*)ptr));
  else if (ptr == g_grid->ne) check("download ne", gpumhd_download(g_ctx, 5, (double*)ptr));
  else if (ptr == g_grid->rhoi) check("download rhoi", gpumhd_download(g_ctx, 6, (double*)ptr));
  else if (ptr == g_grid->amb) check("download amb", gpumhd_download(g_ctx, 7, (double*)ptr));
  else if (ptr == g_grid->phi) check("download phi", gpumhd_download(g_ctx, 8, (double*)ptr));
  else if (ptr == g_grid->divB) check("download divB", gpumhd_download(g_ctx, 9, (double*)ptr));
  else if (g_grid->sflx && ptr == g_grid->sflx) check("download sflx", gpumhd_download(g_ctx, 10, (double*)ptr));
  else {  // the diagnostics of an output step (solver.C:162-172): tvar1..tvar8, Qres, Qvis
    double* const dg[10] = {g_grid->tvar1, g_grid->tvar2, g_grid->tvar3, g_grid->tvar4, g_grid->tvar5,
                            g_grid->tvar6, g_grid->tvar7, g_grid->tvar8, g_grid->Qres, g_grid->Qvis};
    for (int q = 0; q < 10; q++)
      if (dg[q] && ptr == dg[q]) check("download diagnostics", gpumhd_download(g_ctx, 11 + q, (double*)ptr));
  }
}
void UpdateGPU(void* ptr, std::size_t) {
  if (!g_ctx || !g_grid) return;
  if (ptr == g_grid->U) check("upload U", upload_cstate(0, ptr));
  else if (ptr == g_grid->U0) check("upload U0", upload_cstate(1, ptr));
  else if (ptr == g_grid->divB) check("upload divB", gpumhd_upload(g_ctx, 9, (const double*)ptr));
  else if (g_grid->sflx && ptr == g_grid->sflx) check("upload sflx", gpumhd_upload(g_ctx, 10, (const double*)ptr));
}
}  // namespace ACCH
