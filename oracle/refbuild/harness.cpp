// Test infrastructure: drives the reference MURaM hot-path functions, compiled
// unchanged from the reference sources, through the time-step loop of
// ComputeSolution (src/solver.C:109-365) on a seeded initial state, and dumps
// the arrays the GPU path is compared against.  Only tests and the CPU
// baseline run this program; the product never links it.
//
// With xbnd = 1 a closed x dimension gets the reference's own physical
// boundaries (SetBoundaryConditions, src/boundary_pdmp_1_fftw3.C:81-493:
// open bottom, top per bnd_top; no potential field) instead of the mirror.
// With spitzer > 0 the hyperbolic heat conduction runs (heat flux sflx from zero).
// With divB_switch > 0 the reference's Clean_divB runs after the TVD pass, as
// in src/solver.C:341-345; phi starts at zero.
//
// What the harness supplies around the reference functions:
//  * RT stub: Qtot = 0, Tau = tau0 everywhere, dt_rad = a large constant
//    (replaces rts->wrapper, src/solver.C:141);
//  * Sync_timestep, restated from src/solver.C:476-548 (file-local there);
//  * the boundary shim: periodic dimensions are filled by the reference's own
//    exchange_grid_acc; a non-periodic x dimension ("closed") gets the
//    reference's OPEN_TOP=0 mirror rule (src/boundary_pdmp_1_fftw3.C:415-447:
//    M.x, B.y, B.z change sign) at both the bottom and the top;
//  * I/O of the state as raw float64 cState arrays (AoS, ghosts included).
//
// Usage: muram_ref_harness <params.txt> <state_in.bin> <out_dir>
#include <mpi.h>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <vector>
#include <fstream>
#include <sstream>
#include <iostream>
#include <algorithm>

#include "physics.H"
#include "grid.H"
#include "run.H"
#include "eos.H"
#include "limit_va.H"
#include "mhd_tvd.H"
#include "src_int_tck.H"
#include "exchange.H"
#include "divB.H"
#include "icbc.H"
#include "comm_split.H"

MPI_Comm cart_comm;  // defined in comm_split.C, which the harness does not need
// the rest of comm_split.C's globals: one rank, every sub-communicator is the world
MPI_Comm XY_COMM = 0, XZ_COMM = 0, YZ_COMM = 0, XCOL_COMM = 0, YCOL_COMM = 0, ZCOL_COMM = 0;
MPI_Datatype xy_subarray, xz_subarray, yz_subarray;
int xy_rank = 0, xz_rank = 0, yz_rank = 0, xcol_rank = 0, ycol_rank = 0, zcol_rank = 0;
// the potential-field top needs FFTs; the harness runs with bnd_pot = 0
void potential_ext_heffte(const GridData&, double*, double*) {
  fprintf(stderr, "potential-field boundary not available in the harness\n");
  exit(6);
}
extern double p_bc, s_bc;  // src/boundary_pdmp_1_fftw3.C:31
static int g_xbnd = 0;

static std::map<std::string, std::string> g_par;

static double par_d(const char* k, double def) {
  auto it = g_par.find(k);
  return it == g_par.end() ? def : atof(it->second.c_str());
}
static int par_i(const char* k, int def) {
  auto it = g_par.find(k);
  return it == g_par.end() ? def : atoi(it->second.c_str());
}
static std::string par_s(const char* k, const char* def) {
  auto it = g_par.find(k);
  return it == g_par.end() ? std::string(def) : it->second;
}
static void par_arr(const char* k, double* dst, int n) {
  auto it = g_par.find(k);
  if (it == g_par.end()) return;
  std::istringstream is(it->second);
  for (int i = 0; i < n; i++) is >> dst[i];
}

static std::string g_out;

static void dump(const char* name, const void* p, size_t bytes) {
  std::string fn = g_out + "/" + name + ".bin";
  FILE* f = fopen(fn.c_str(), "wb");
  if (!f) { perror(fn.c_str()); exit(2); }
  fwrite(p, 1, bytes, f);
  fclose(f);
}

static void dump_aux(const char* name, const GridData& G) {
  std::vector<double> buf(5 * (size_t)G.bufsize);
  const double* src[5] = {G.pres, G.temp, G.ne, G.rhoi, G.amb};
  for (int v = 0; v < 5; v++) memcpy(&buf[(size_t)v * G.bufsize], src[v], G.bufsize * sizeof(double));
  dump(name, buf.data(), buf.size() * sizeof(double));
}

// Restatement of Sync_timestep (src/solver.C:487-548) for one rank.
static void sync_timestep(RunData& Run, const PhysicsData& Physics, double dt_rad, double dt_mhd,
                          int* rt_upd, double* cfl) {
  auto invalid = [](double a) {
    return (a != a) || (a <= 0.) || (a == std::numeric_limits<double>::infinity());
  };
  double r0 = dt_rad, r1 = dt_mhd;
  if (invalid(r0)) { fprintf(stderr, "Invalid time step: dt_rad = %g\n", r0); exit(5); }
  if (invalid(r1)) { fprintf(stderr, "Invalid time step: dt_mhd = %g\n", r1); exit(5); }
  double dt_min_rt = Physics.rt[i_rt_tstep] * Run.CFL * r1;
  if (r0 < dt_min_rt) r0 = std::max(r0, dt_min_rt);
  double dt_min = std::min(r0, r1);
  double dt = std::min(r0, Run.CFL * r1);
  if (Run.outcad > 0) {
    double rem = Run.dt_rem();
    if (rem > 0.0) dt = std::min(dt, rem);
  }
  if (Run.autostep) Run.dt = dt;
  *cfl = Run.dt / dt_min;
  if (*cfl >= 2.) { fprintf(stderr, "Invalid time step: CFL = %g\n", *cfl); exit(5); }
  *rt_upd = (int)(r0 / Run.dt);
  *rt_upd = std::max(1, std::min(*rt_upd, (int)Physics.rt[i_rt_update]));
}

// Closed-x mirror rule at both ends (harness boundary shim).
static void closed_x_bc(GridData& G) {
  const int lb = G.lbeg[0], le = G.lend[0];
  for (int k = G.lbeg[2] - G.ghosts[2]; k <= G.lend[2] + G.ghosts[2]; k++)
    for (int j = G.lbeg[1] - G.ghosts[1]; j <= G.lend[1] + G.ghosts[1]; j++) {
      for (int g = 1; g <= 2; g++) {
        cState top = G.U[G.node(le + 1 - g, j, k)];
        top.M.x *= -1; top.B.y *= -1; top.B.z *= -1;
        G.U[G.node(le + g, j, k)] = top;
        cState bot = G.U[G.node(lb - 1 + g, j, k)];
        bot.M.x *= -1; bot.B.y *= -1; bot.B.z *= -1;
        G.U[G.node(lb - g, j, k)] = bot;
      }
    }
}

// xbnd = 1: the reference's own SetBoundaryConditions (open bottom, top per
// bnd_top); its stage argument only selects logging, so 0 is passed.
static RunData* g_run = nullptr;
static void boundaries(GridData& G, const PhysicsData& P, int needs_sflx) {
  exchange_grid_acc(G, P, needs_sflx);
  if (G.periods[0]) return;
  if (g_xbnd == 1) SetBoundaryConditions(*g_run, G, P, 0, 0, nullptr);
  else closed_x_bc(G);
}

int main(int argc, char** argv) {
  if (argc < 4) {
    fprintf(stderr, "usage: %s params.txt state_in.bin out_dir\n", argv[0]);
    return 1;
  }
  {
    std::ifstream in(argv[1]);
    std::string line;
    while (std::getline(in, line)) {
      auto eq = line.find('=');
      if (eq == std::string::npos || line[0] == '#') continue;
      std::string k = line.substr(0, eq), v = line.substr(eq + 1);
      k.erase(std::remove_if(k.begin(), k.end(), ::isspace), k.end());
      g_par[k] = v;
    }
  }
  g_out = argv[3];

  RunData Run;
  GridData Grid;
  PhysicsData Physics;

  Grid.NDIM = 3;
  const int n[3] = {par_i("nx", 16), par_i("ny", 16), par_i("nz", 16)};
  const double dx0 = par_d("dx", 3.2e6);
  const double dx[3] = {dx0, par_d("dy", dx0), par_d("dz", dx0)};
  for (int d = 0; d < 3; d++) {
    Grid.gsize[d] = n[d];
    Grid.gxmin[d] = 0.0;
    Grid.gxmax[d] = dx[d] * n[d];
    Grid.ghosts[d] = 2;
    Grid.procs[d] = 1;
    Grid.pardim[d] = 1;
  }
  Grid.periods[0] = par_i("periodic_x", 1);
  Grid.periods[1] = 1;
  Grid.periods[2] = 1;

  Run.CFL = par_d("CFL", 0.8);
  Run.CFL_tvd = par_d("CFL_tvd", 0.95);
  Run.dt = 0.0;
  Run.maxiter = 1000000;
  Run.Tmax = 1e30;
  Run.outcad = 0.0;
  strncpy(Run.eos_name, par_s("eos", "eos.dat").c_str(), sizeof(Run.eos_name) - 1);

  Physics.params[i_param_grav] = par_d("grav", 0.0);
  Physics.params[i_param_va_max] = par_d("va_max", 1e7);
  Physics.params[i_param_va_adjust] = par_d("va_adjust", 0.0);
  Physics.params[i_param_max_fill] = par_d("max_fill", 1000.);
  Physics.params[i_param_spitzer] = par_d("spitzer", 0.0);
  Physics.params[i_param_eta] = par_d("eta", 0.0);
  Physics.params[i_param_ambipolar] = 0.0;
  par_arr("tvd_h", Physics.tvd_h, 4);
  par_arr("tvd_cs", Physics.tvd_cs, 4);
  par_arr("tvd_coeff", Physics.tvd_coeff, 4);
  Physics.tvd_h_bnd[0] = Physics.tvd_h_bnd[1] = 1e-6;
  Physics.tvd_visc_bnd[0] = Physics.tvd_visc_bnd[1] = 1.0;
  Physics.tvd_eta_bnd[0] = Physics.tvd_eta_bnd[1] = 1.0;
  par_arr("tvd_h_bnd", Physics.tvd_h_bnd, 2);
  par_arr("tvd_visc_bnd", Physics.tvd_visc_bnd, 2);
  par_arr("tvd_eta_bnd", Physics.tvd_eta_bnd, 2);
  Physics.tvd[i_tvd_rholev] = par_d("tvd_rholev", Physics.tvd[i_tvd_rholev]);
  Physics.tvd[i_tvd_rholog] = par_d("tvd_rholog", Physics.tvd[i_tvd_rholog]);
  Physics.tvd[i_tvd_qrho] = par_d("tvd_qrho", Physics.tvd[i_tvd_qrho]);
  Physics.tvd[i_tvd_Bpar] = par_d("tvd_Bpar", Physics.tvd[i_tvd_Bpar]);
  Physics.tvd[i_tvd_vhyp] = par_d("tvd_vhyp", Physics.tvd[i_tvd_vhyp]);
  Physics.tvd[i_tvd_Qdiff_bnd] = par_d("tvd_Qdiff_bnd", 1.0);
  Physics.tvd[i_tvd_pm_v] = par_d("tvd_pm_v", Physics.tvd[i_tvd_pm_v]);
  Physics.tvd[i_tvd_pm_B] = par_d("tvd_pm_B", Physics.tvd[i_tvd_pm_B]);
  Physics.tvd[i_tvd_vmax_lim] = par_d("tvd_vmax_lim", Physics.tvd[i_tvd_vmax_lim]);
  Physics.tvd[i_tvd_CME_thresh] = par_d("tvd_CME_thresh", Physics.tvd[i_tvd_CME_thresh]);
  Physics.divB[i_divB_switch] = par_d("divB_switch", 0.0);
  Physics.divB[i_divB_itmax] = par_d("divB_itmax", 5.0);
  Physics.divB[i_divB_err] = par_d("divB_err", 0.2);
  Physics.tchk[i_tchk_eps_min] = par_d("tchk_eps_min", Physics.tchk[i_tchk_eps_min]);
  Physics.tchk[i_tchk_rho_min] = par_d("tchk_rho_min", Physics.tchk[i_tchk_rho_min]);
  Physics.tchk[i_tchk_eps_max] = par_d("tchk_eps_max", Physics.tchk[i_tchk_eps_max]);
  Physics.tchk[i_tchk_vmax] = par_d("tchk_vmax", Physics.tchk[i_tchk_vmax]);
  Physics.dmp[i_dmp_switch] = 0;
  Physics.rt[i_rt_update] = 1;
  Physics.rt[i_rt_tstep] = 0.0;
  Physics.rt_ext[i_ext_cor] = 0;
  Physics.bnd[i_bnd_pot] = 0;
  Physics.bnd[i_bnd_top] = par_d("bnd_top", 0.0);
  Physics.bnd[i_bnd_bcrit] = par_d("bnd_bcrit", 1.0e10);
  Physics.bnd[i_bnd_eps_top] = par_d("bnd_eps_top", 0.0);
  g_xbnd = par_i("xbnd", 0);
  p_bc = par_d("p_bc", -1.0);
  s_bc = par_d("s_bc", -1.0);

  Run.Init(0);
  Run.verbose = par_i("verbose", 0);
  // diag_step > 0: the diagnostics of that (1-based) step, as ComputeSolution
  // sets them on an output step (src/solver.C:264-289); GridData::Init
  // allocates the arrays only with Run.diagnostics (src/grid.C:318-334)
  const int diag_step = par_i("diag_step", 0);
  Run.diagnostics = diag_step > 0 ? 1 : 0;
  g_run = &Run;
  Physics.Init();
  Grid.Init(Run, Physics);
  if (Grid.periods[0]) {  // truly periodic x: no physical x boundary inside the TVD
    Grid.is_gbeg[0] = 0;
    Grid.is_gend[0] = 0;
  }

  const double tau0 = par_d("tau0", 1.0);
  const double dt_rad_const = par_d("dt_rad", 1e9);
  for (int i = 0; i < Grid.bufsize; i++) {
    Grid.Qtot[i] = 0.0;
    Grid.Tau[i] = tau0;
    Grid.Res[i].zero();
    Grid.U0[i].zero();
    Grid.pres[i] = Grid.temp[i] = Grid.ne[i] = Grid.rhoi[i] = Grid.amb[i] = 0.0;
    Grid.phi[i] = Grid.divB[i] = 0.0;  // Grid.C:284-285 leaves them unset; the cleaning starts from phi = 0
    if (Grid.sflx) Grid.sflx[i] = Grid.sflx0[i] = Grid.Rflx[i] = Grid.BgradT[i] = 0.0;  // heat flux starts at zero
  }

  eos_init(Grid, Run, Physics);

  {
    FILE* f = fopen(argv[2], "rb");
    if (!f) { perror(argv[2]); return 2; }
    size_t got = fread(Grid.U, sizeof(cState), Grid.bufsize, f);
    fclose(f);
    if ((int)got != Grid.bufsize) {
      fprintf(stderr, "state file has %zu cells, expected %d\n", got, Grid.bufsize);
      return 2;
    }
  }
  boundaries(Grid, Physics, 1);

  const int steps = par_i("steps", 1);
  const int trace_step = par_i("trace_step", 0);  // 1-based step to dump, 0 = none
  const size_t ubytes = (size_t)Grid.bufsize * sizeof(cState);

  dump("init_U", Grid.U, ubytes);

  std::vector<double> dts;
  std::vector<double> limits;
  double dt_rad = 0.0, dt_mhd = 0.0, cfl = 0.0;
  int rt_upd = 1;
  int tvd_two = 0;
  char name[64];
  for (int it = 1; it <= steps; it++) {
    const bool tr = (it == trace_step);
    SaveCons(Grid, Physics);
    for (int stage = 1; stage <= maxstage; stage++) {
      ConsToPrim(Grid, Physics, Run);
      if (tr) {
        snprintf(name, sizeof name, "s%d_c2p_U", stage); dump(name, Grid.U, ubytes);
        snprintf(name, sizeof name, "s%d_c2p_aux", stage); dump_aux(name, Grid);
      }
      if (stage == 1) {
        Adjust_Valf_Max(Run, Grid, Physics);
        limits.push_back(inv_va2max);
        limits.push_back(v_lim);
        limits.push_back(e_lim);
        dt_rad = dt_rad_const;  // RT stub (Qtot = 0, Tau = tau0 set once above)
      }
      Run.need_diagnostics = (it == diag_step && stage == maxstage) ? 1 : 0;
      if (Run.need_diagnostics) {
        double* dg[10] = {Grid.tvar1, Grid.tvar2, Grid.tvar3, Grid.tvar4, Grid.tvar5,
                          Grid.tvar6, Grid.tvar7, Grid.tvar8, Grid.Qres, Grid.Qvis};
        for (int q = 0; q < 10; q++)
          for (int i = 0; i < Grid.bufsize; i++) dg[q][i] = 0.0;
      }
      dt_mhd = MHD_Residual(Run, Grid, Physics);
      if (tr) {
        snprintf(name, sizeof name, "s%d_res_R", stage); dump(name, Grid.Res, ubytes);
        snprintf(name, sizeof name, "s%d_res_dt", stage); dump(name, &dt_mhd, sizeof(double));
      }
      if (stage == 1) {
        sync_timestep(Run, Physics, dt_rad, dt_mhd, &rt_upd, &cfl);
        dts.push_back(Run.dt);
        dts.push_back(cfl);
        dts.push_back(dt_mhd);
      }
      Source_Integrate_Tcheck(Run, Grid, Physics, stage);
      if (tr) { snprintf(name, sizeof name, "s%d_si_U", stage); dump(name, Grid.U, ubytes); }
      boundaries(Grid, Physics, 1);
      if (tr) { snprintf(name, sizeof name, "s%d_bc_U", stage); dump(name, Grid.U, ubytes); }
    }
    if (cfl <= Run.CFL_tvd) {
      TVDlimit(Run, Grid, Physics, Run.dt);
    } else {
      tvd_two = 1;
      TVDlimit(Run, Grid, Physics, 0.5 * Run.dt);
      exchange_grid_acc(Grid, Physics, 0);  // src/solver.C:334: exchange only, no BC call
      TVDlimit(Run, Grid, Physics, 0.5 * Run.dt);
    }
    if (tr) dump("tvd_U", Grid.U, ubytes);
    if (Physics.divB[i_divB_switch] > 0) {  // src/solver.C:341-345
      if (tr) dump("divb_phi_in", Grid.phi, Grid.bufsize * sizeof(double));
      Clean_divB(Run, Grid, Physics);
      if (tr) dump("divb_U", Grid.U, ubytes);
    }
    TCheck(Run, Grid, Physics);
    if (tr) dump("tck_U", Grid.U, ubytes);
    if (it == diag_step) {
      const double* dg[10] = {Grid.tvar1, Grid.tvar2, Grid.tvar3, Grid.tvar4, Grid.tvar5,
                              Grid.tvar6, Grid.tvar7, Grid.tvar8, Grid.Qres, Grid.Qvis};
      std::vector<double> all;
      for (int q = 0; q < 10; q++) all.insert(all.end(), dg[q], dg[q] + Grid.bufsize);
      dump("diag", all.data(), all.size() * sizeof(double));
      dump("diag_U", Grid.U, ubytes);  // the state after TCheck of that step
    }
    Run.need_diagnostics = 0;
    boundaries(Grid, Physics, 0);
    if (tr) dump("end_U", Grid.U, ubytes);
    Run.Advance();
  }
  dump("final_U", Grid.U, ubytes);
  if (Grid.sflx) dump("final_sflx", Grid.sflx, Grid.bufsize * sizeof(double));
  if (Physics.divB[i_divB_switch] > 0) {
    dump("final_phi", Grid.phi, Grid.bufsize * sizeof(double));
    dump("final_divB", Grid.divB, Grid.bufsize * sizeof(double));
  }
  dump("dts", dts.data(), dts.size() * sizeof(double));
  dump("limits", limits.data(), limits.size() * sizeof(double));
  {
    std::string fn = g_out + "/summary.txt";
    FILE* f = fopen(fn.c_str(), "w");
    fprintf(f, "steps=%d\ntime=%.17g\ndt=%.17g\ncfl=%.17g\ntvd_two_half_steps=%d\n", steps, Run.time,
            Run.dt, cfl, tvd_two);
    if (g_xbnd == 1) fprintf(f, "p_bc=%.17g\ns_bc=%.17g\n", p_bc, s_bc);
    fclose(f);
  }
  return 0;
}
