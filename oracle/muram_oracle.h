/* CPU restatement of MURaM's MHD time-step hot path (test infrastructure).
 *
 * This oracle is the checker for the GPU library: only tests, the smoke check
 * and the CPU-baseline leg of the benchmark call it.  Every routine restates
 * the arithmetic of the reference function it names, in the same operation
 * order (built with -ffp-contract=off), on a structure-of-arrays state:
 *
 *   U[v*N + i + sx*(j + sy*k)],  v = rho, M_x, M_y, M_z, e, B_x, B_y, B_z
 *   sx = nx+4, sy = ny+4, sz = nz+4, N = sx*sy*sz   (two ghost layers)
 */
#ifndef MURAM_ORACLE_H
#define MURAM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int nx, ny, nz;       /* interior cells per dimension (dimension 0 = x = vertical) */
  int periodic_x;       /* 1: periodic x; 0: closed x (mirror ghosts, physical x boundaries) */
  double dx[3];
  /* RunData subset */
  double CFL, CFL_tvd, dt, time, outcad;
  int autostep;
  /* PhysicsData subset */
  double grav, va_max, va_adjust, max_fill;
  double tvd_h[4], tvd_cs[4], tvd[10], tvd_h_bnd[2], tvd_visc_bnd[2], tvd_eta_bnd[2], tvd_coeff[4];
  double tchk[4];
  double rt_cfl, rt_tstep, rt_update;
  /* RT stub: constant optical depth, zero Qtot, constant dt_rad */
  double tau0, dt_rad;
  /* values the reference keeps in globals / function statics */
  double inv_va2max, v_lim, e_lim, va_max_old;
  int va_ini_flag;
  double last_cfl;
  int tvd_two_half_steps;
  /* PhysicsData::params[i_param_eta]: resistivity (cm^2/s); 0 = ideal MHD */
  double eta;
  /* PhysicsData::divB: cleaning on (> 0), iteration cap, target error ratio */
  int divB_switch, divB_itmax;
  double divB_err;
  /* Clean_divB's adaptive iteration count (a function static there, starts
   * at 3) and the last call's iterations and max|divB| before / after (G) */
  int divB_next_iter, divB_last_iters;
  double divB_err0, divB_err1;
  /* x boundaries of a closed box: 0 = mirror at both ends; 1 = MURaM's physical
   * boundaries (open bottom, closed or half-open top).  PhysicsData::bnd: top
   * mode (0 closed, 1 open to outflows), B_crit (G), eps_top; p_bc and s_bc
   * (negative: set from the first call's bottom layers); bnd_ini: first call pending */
  int xbnd, bnd_top;
  double bnd_bcrit, bnd_eps_top, p_bc, s_bc;
  int bnd_ini;
  /* PhysicsData::params[i_param_spitzer]: Spitzer coefficient of the hyperbolic
   * heat conduction (0: off) */
  double spitzer;
  /* RunData::need_diagnostics (src/solver.C:264-289) and the ten diagnostic
   * arrays tvar1..tvar8, Qres, Qvis (10 x N, NULL: none).  mo_step_ex sets
   * need_diagnostics at stage 4 of a step requested by diagnostics_next_step,
   * zeroes the arrays there, and clears both flags after that step's TCheck. */
  int need_diagnostics, diagnostics_next_step;
  double* diag;
} mo_params;

typedef struct mo_eos mo_eos;

/* Fields beyond the state that some settings evolve (NULL where unused):
 * divB cleaning's phi and last divergence; Spitzer conduction's heat flux
 * sflx, its stage-start copy sflx0, its residual Rflx and B.grad(T). N each. */
typedef struct {
  double *phi, *divB, *sflx, *sflx0, *Rflx, *BgradT;
} mo_fields;

void mo_default_params(mo_params* p, int nx, int ny, int nz, double dx);
mo_eos* mo_eos_load(const char* path);
void mo_eos_free(mo_eos* e);
int mo_eos_dims(const mo_eos* e, int* dims4);

/* src/Add_Sources_Integrate_SR.C:475-502 */
void mo_save_cons(const mo_params* p, const double* U, double* U0);
/* src/cons_to_prim.C:78-266 (aux may be NULL to skip T, n_e, rho_i, nu_in) */
void mo_cons_to_prim(const mo_params* p, const mo_eos* eos, double* U, double* pres, double* temp,
                     double* ne, double* rhoi, double* amb);
/* src/Adjust_Valf_Max.C:25-150; stats[5] receives the local max/sum values */
void mo_adjust_valf_max(mo_params* p, const double* U, const double* pres, double* stats);
/* src/mhdres_SR.C:27-854 (ideal MHD branch); returns dt_mhd */
double mo_mhd_residual(const mo_params* p, const double* U, const double* pres, double* R);
/* the same with the Spitzer terms when p->spitzer > 0 (temp: ConsToPrim's T) */
double mo_mhd_residual_ex(const mo_params* p, const double* U, const double* pres, const double* temp, double* R,
                          mo_fields* f);
/* src/solver.C:487-548; returns 0 or a negative error code */
int mo_sync_timestep(mo_params* p, double dt_rad, double dt_mhd, double* cfl);
/* src/Add_Sources_Integrate_SR.C:38-472 (no-diagnostics branch) */
void mo_source_integrate_tcheck(const mo_params* p, double* U, const double* U0, double* R, int stage);
void mo_source_integrate_ex(const mo_params* p, double* U, const double* U0, double* R, int stage, mo_fields* f);
/* src/exchange.C:532-783 on one rank plus the closed-x mirror rule */
void mo_boundaries(const mo_params* p, double* U);
void mo_exchange_only(const mo_params* p, double* U);
/* exchange, then the x boundaries p->xbnd selects (src/boundary_pdmp_1_fftw3.C:81-565
 * for xbnd = 1, which needs the EOS's inverse tables) */
void mo_boundaries_eos(mo_params* p, const mo_eos* eos, double* U);
/* the same with the heat flux: exchanged when needs_sflx (src/exchange.C:590-760),
 * and its boundary values with the physical x boundaries */
void mo_boundaries_ex(mo_params* p, const mo_eos* eos, double* U, mo_fields* f, int needs_sflx);
/* src/tvdlimit_SR.C:33-695 */
void mo_tvdlimit(const mo_params* p, double* U, const double* pres, double dt_tvd);
/* src/Add_Sources_Integrate_SR.C:534-625 */
void mo_tcheck(const mo_params* p, double* U);
/* src/clean_divB.C:35-369; phi (N, persists between calls), divB (N) */
void mo_clean_divB(mo_params* p, double* U, double* phi, double* divB);
/* One full step in the order of src/solver.C:109-365; returns 0 or a negative error code.
 * Scratch: U0, R (8N each) and pres, temp, ne, rhoi, amb (N each). */
int mo_step(mo_params* p, const mo_eos* eos, double* U, double* U0, double* R, double* aux5);
/* The same with divB cleaning after the TVD pass (src/solver.C:341-345) when
 * p->divB_switch > 0; phi and divB as for mo_clean_divB. */
int mo_step_divb(mo_params* p, const mo_eos* eos, double* U, double* U0, double* R, double* aux5, double* phi,
                 double* divB);
/* One step with every optional field (divB cleaning, Spitzer conduction) */
int mo_step_ex(mo_params* p, const mo_eos* eos, double* U, double* U0, double* R, double* aux5, mo_fields* f);

#ifdef __cplusplus
}
#endif
#endif
