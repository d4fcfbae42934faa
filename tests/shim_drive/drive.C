// Drives the MURaM-side shim (muram_main_gb300/shim/gpumhd_muram_shim.C) the
// way MURaM's ComputeSolution (src/solver.C:109-365) calls the hot-path
// routines -- by their MURaM names and signatures, over GridData / RunData /
// PhysicsData (stand-in declarations in standin/) -- so that the shim's own
// mechanisms run on a GPU: the eos_init wrapper that creates the context, the
// parameter push when Run.dt or Run.time changes, Run.need_diagnostics, and
// the ACCH::UpdateGPU / UpdateCPU routing of GridData's arrays.
//
// Usage: shim_drive <dir>
//   in:  <dir>/params.bin  gpumhd_params (the run's parameters, bytes)
//        <dir>/run.txt     eos table path, dt_rad, steps, diagnostics step (0: none)
//        <dir>/input.bin   cState array incl. ghosts, float64, x fastest
//   out: <dir>/final.bin   the state after the steps (cState, float64)
//        <dir>/pres.bin    GridData::pres after the last step
//        <dir>/dts.txt     dt and cfl of every step
//        <dir>/diag.bin    tvar1..tvar8, Qres, Qvis of the diagnostics step
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ACCH.h"
#include "divB.H"
#include "eos.H"
#include "exchange.H"
#include "gpumhd.h"
#include "grid.H"
#include "icbc.H"
#include "limit_va.H"
#include "mhd_tvd.H"
#include "run.H"
#include "src_int_tck.H"

extern double p_bc, s_bc;  // defined by the shim (MURaM: src/boundary_pdmp_1_fftw3.C)

static void die(const char* what) {
  fprintf(stderr, "shim_drive: %s\n", what);
  std::exit(1);
}

static std::vector<char> slurp(const std::string& path) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) die(("cannot open " + path).c_str());
  std::vector<char> b;
  char buf[1 << 16];
  size_t n;
  while ((n = fread(buf, 1, sizeof buf, f)) > 0) b.insert(b.end(), buf, buf + n);
  fclose(f);
  return b;
}

static void spill(const std::string& path, const void* p, size_t n) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f || fwrite(p, 1, n, f) != n) die(("cannot write " + path).c_str());
  fclose(f);
}

// MURaM's Sync_timestep (src/solver.C:476-548) for one rank: dt from the
// radiative and MHD limits, clipped to the next output time, and the CFL
// number; an invalid step ends the run as the reference's does.
static double sync_timestep(RunData& Run, const PhysicsData& Physics, double dt_rad, double dt_mhd) {
  auto bad = [](double a) { return (a != a) || (a <= 0.) || (a > 1e300); };
  if (bad(dt_rad) || bad(dt_mhd)) die("invalid time step");
  double r0 = dt_rad;
  const double r1 = dt_mhd;
  const double dt_min_rt = Physics.rt[i_rt_tstep] * Run.CFL * r1;
  if (r0 < dt_min_rt) r0 = r0 > dt_min_rt ? r0 : dt_min_rt;
  const double dt_min = r0 < r1 ? r0 : r1;
  double dt = (Run.CFL * r1 < r0) ? Run.CFL * r1 : r0;
  if (Run.outcad > 0) {
    const double num = Run.time / Run.outcad;
    const int ce = (int)num;
    const double rem = (num == (double)ce) ? 0.0 : (ce + 1) * Run.outcad - Run.time;
    if (rem > 0.0 && rem < dt) dt = rem;
  }
  if (Run.autostep) Run.dt = dt;
  const double cfl = Run.dt / dt_min;
  if (cfl >= 2.) die("CFL >= 2");
  return cfl;
}

int main(int argc, char** argv) {
  if (argc != 2) die("usage: shim_drive <dir>");
  const std::string dir = argv[1];
  const std::vector<char> pb = slurp(dir + "/params.bin");
  if (pb.size() != sizeof(gpumhd_params)) die("params.bin does not hold one gpumhd_params");
  gpumhd_params p;
  memcpy(&p, pb.data(), sizeof p);
  char eos[512] = {0};
  double dt_rad = 0.0;
  int steps = 0, diag_step = 0;
  {
    FILE* f = fopen((dir + "/run.txt").c_str(), "r");
    if (!f || fscanf(f, "%511s %lf %d %d", eos, &dt_rad, &steps, &diag_step) != 4) die("bad run.txt");
    fclose(f);
  }

  GridData Grid;
  RunData Run;
  PhysicsData Physics;
  memset(&Grid, 0, sizeof Grid);
  memset(&Run, 0, sizeof Run);
  memset(&Physics, 0, sizeof Physics);
  const int n[3] = {p.nx, p.ny, p.nz};
  long long N = 1;
  for (int d = 0; d < 3; d++) {
    Grid.lsize[d] = n[d];
    Grid.procs[d] = 1;
    Grid.periods[d] = d == 0 ? p.periodic_x : 1;
    Grid.dx[d] = (real)p.dx[d];
    N *= n[d] + 4;
  }
  Grid.bufsize = (int)N;
  Grid.U = new cState[N];
  Grid.U0 = new cState[N];
  Grid.Res = new cState[N];
  double** const scal[] = {&Grid.pres, &Grid.temp, &Grid.ne, &Grid.rhoi, &Grid.amb, &Grid.Tau, &Grid.divB,
                           &Grid.phi, &Grid.tvar1, &Grid.tvar2, &Grid.tvar3, &Grid.tvar4, &Grid.tvar5,
                           &Grid.tvar6, &Grid.tvar7, &Grid.tvar8, &Grid.Qres, &Grid.Qvis};
  for (double** a : scal) *a = new double[N]();
  for (long long i = 0; i < N; i++) Grid.Tau[i] = p.tau0;
  if (p.spitzer > 0) Grid.sflx = new double[N]();

  Run.CFL = p.CFL;
  Run.CFL_tvd = p.CFL_tvd;
  Run.dt = p.dt;
  Run.time = p.time;
  Run.outcad = p.outcad;
  Run.autostep = p.autostep;
  Run.diagnostics = diag_step > 0;
  snprintf(Run.eos_name, sizeof Run.eos_name, "%s", eos);

  Physics.params[i_param_grav] = p.grav;
  Physics.params[i_param_va_max] = p.va_max;
  Physics.params[i_param_va_adjust] = p.va_adjust;
  Physics.params[i_param_max_fill] = p.max_fill;
  Physics.params[i_param_eta] = p.eta;
  Physics.params[i_param_spitzer] = p.spitzer;
  for (int i = 0; i < 4; i++) {
    Physics.tvd_h[i] = p.tvd_h[i];
    Physics.tvd_cs[i] = p.tvd_cs[i];
    Physics.tvd_coeff[i] = p.tvd_coeff[i];
    Physics.tchk[i] = p.tchk[i];
  }
  for (int i = 0; i < 10; i++) Physics.tvd[i] = p.tvd[i];
  for (int i = 0; i < 2; i++) {
    Physics.tvd_h_bnd[i] = p.tvd_h_bnd[i];
    Physics.tvd_visc_bnd[i] = p.tvd_visc_bnd[i];
    Physics.tvd_eta_bnd[i] = p.tvd_eta_bnd[i];
  }
  Physics.rt[i_rt_cfl] = p.rt_cfl;
  Physics.rt[i_rt_tstep] = p.rt_tstep;
  Physics.rt[i_rt_update] = p.rt_update;
  Physics.divB[i_divB_switch] = p.divB_switch;
  Physics.divB[i_divB_itmax] = p.divB_itmax;
  Physics.divB[i_divB_err] = p.divB_err;
  Physics.bnd[i_bnd_top] = p.bnd_top;
  Physics.bnd[i_bnd_bcrit] = p.bnd_bcrit;
  Physics.bnd[i_bnd_eps_top] = p.bnd_eps_top;
  p_bc = p.p_bc;
  s_bc = p.s_bc;

  {  // the initial state into GridData::U (cState of `real`)
    const std::vector<char> ub = slurp(dir + "/input.bin");
    if (ub.size() != sizeof(double) * 8 * (size_t)N) die("input.bin does not hold the box's cState array");
    const double* u = reinterpret_cast<const double*>(ub.data());
    for (long long i = 0; i < N; i++)
      for (int v = 0; v < 8; v++) Grid.U[i].v[v] = (real)u[8 * i + v];
  }

  // MURaM's start-up: the EOS (the shim's wrapper creates the GPU context and
  // loads the same table), the state to the device, ghosts and boundaries
  eos_init(Grid, Run, Physics);
  ACCH::UpdateGPU(Grid.U, sizeof(cState) * N);
  exchange_grid_acc(Grid, Physics, 1);
  SetBoundaryConditions(Run, Grid, Physics, 0, 1, nullptr);

  FILE* fdt = fopen((dir + "/dts.txt").c_str(), "w");
  if (!fdt) die("cannot write dts.txt");
  for (int it = 1; it <= steps; it++) {
    // ComputeSolution (src/solver.C:109-365), one step
    SaveCons(Grid, Physics);
    double cfl = 0.0;
    for (int stage = 1; stage <= 4; stage++) {
      Run.need_diagnostics = (stage == 4 && it == diag_step) ? 1 : 0;
      ConsToPrim(Grid, Physics, Run);
      if (stage == 1) Adjust_Valf_Max(Run, Grid, Physics);
      const double dt_mhd = MHD_Residual(Run, Grid, Physics);
      if (stage == 1) cfl = sync_timestep(Run, Physics, dt_rad, dt_mhd);
      Source_Integrate_Tcheck(Run, Grid, Physics, stage);
      exchange_grid_acc(Grid, Physics, 1);
      SetBoundaryConditions(Run, Grid, Physics, stage, 0, nullptr);
    }
    if (cfl <= Run.CFL_tvd) {
      TVDlimit(Run, Grid, Physics, Run.dt);
    } else {
      TVDlimit(Run, Grid, Physics, 0.5 * Run.dt);
      exchange_grid_acc(Grid, Physics, 0);
      TVDlimit(Run, Grid, Physics, 0.5 * Run.dt);
    }
    if (Physics.divB[i_divB_switch] > 0) Clean_divB(Run, Grid, Physics);
    TCheck(Run, Grid, Physics);
    exchange_grid_acc(Grid, Physics, 0);
    SetBoundaryConditions(Run, Grid, Physics, 5, 1, nullptr);
    fprintf(fdt, "%.17g %.17g\n", Run.dt, cfl);
    if (it == diag_step) {  // the output step's diagnostics, as MURaM's output reads them
      std::vector<double> dg;
      double* const arr[10] = {Grid.tvar1, Grid.tvar2, Grid.tvar3, Grid.tvar4, Grid.tvar5,
                               Grid.tvar6, Grid.tvar7, Grid.tvar8, Grid.Qres, Grid.Qvis};
      for (double* a : arr) {
        ACCH::UpdateCPU(a, sizeof(double) * N);
        dg.insert(dg.end(), a, a + N);
      }
      spill(dir + "/diag.bin", dg.data(), sizeof(double) * dg.size());
    }
    Run.time += Run.dt;  // RunData::Advance
  }
  fclose(fdt);

  ACCH::UpdateCPU(Grid.U, sizeof(cState) * N);
  ACCH::UpdateCPU(Grid.pres, sizeof(double) * N);
  std::vector<double> out(8 * (size_t)N);
  for (long long i = 0; i < N; i++)
    for (int v = 0; v < 8; v++) out[8 * i + v] = (double)Grid.U[i].v[v];
  spill(dir + "/final.bin", out.data(), sizeof(double) * out.size());
  spill(dir + "/pres.bin", Grid.pres, sizeof(double) * N);
  return 0;
}
