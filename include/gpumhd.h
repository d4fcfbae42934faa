/* gpumhd: GB300-native MURaM MHD time-step hot path, C ABI.
 *
 * The library owns the grid state on one GPU and exposes one entry point per
 * reference routine on MURaM's time-step path (src/solver.C:109-365), so a
 * MURaM build can route each call through it, plus a fused entry point that
 * advances whole time steps on the device.
 *
 * State layout seen by the host: MURaM's GridData arrays, i.e. cState records
 * of 8 doubles (rho, M_x, M_y, M_z, e, B_x, B_y, B_z) in x-fastest order over
 * the local box including 2 ghost layers, node = i + sx*(j + sy*k),
 * sx = nx+4, sy = ny+4 (include/grid.H:109-121, src/grid.C:197-199).
 * Dimension 0 (x) is vertical.  On the device the state is stored as a
 * structure of arrays in FP64 or FP32 (gpumhd_params.precision).
 *
 * Every function returns GPUMHD_OK (0) or a negative status; the reference
 * calls MPI_Abort in the corresponding situations instead.
 * A context is bound to one device and one CUDA stream and is not thread-safe.
 * Calls are ordered on the context's stream; functions that return host
 * scalars synchronise on them.
 */
#ifndef GPUMHD_H
#define GPUMHD_H

#ifdef __cplusplus
extern "C" {
#endif

#define GPUMHD_OK 0
#define GPUMHD_E_INVALID (-1)   /* bad argument or unsupported configuration */
#define GPUMHD_E_CUDA (-2)      /* CUDA runtime error (message in gpumhd_last_error) */
#define GPUMHD_E_EOS (-3)       /* EOS file missing or malformed (src/eos_init.C:74-77 aborts) */
#define GPUMHD_E_BAD_DT (-4)    /* invalid dt_rad or dt_mhd (src/solver.C:497-507 aborts) */
#define GPUMHD_E_CFL (-5)       /* cfl >= 2 (src/solver.C:530-534 aborts) */
#define GPUMHD_E_ORDER (-6)     /* call made before the state it needs exists */
#define GPUMHD_E_NOMEM (-7)     /* device allocation failed */

/* Largest box, ghosts included ((nx+4)(ny+4)(nz+4)), that a context accepts:
 * the kernels address the 8 state arrays with 32-bit offsets (8*N < 2^32).
 * 1024 x 1024 x 256 interior cells is 2.75e8. */
#define GPUMHD_MAX_CELLS 536870911LL

/* Plain-data mirror of the RunData / PhysicsData / GridData fields the path
 * reads (include/run.H:6-80, include/physics.H:80-206, include/grid.H:8-125). */
typedef struct gpumhd_params {
  int nx, ny, nz;        /* interior cells (GridData::lsize); each >= 4 */
  int periodic_x;        /* GridData::periods[0]; y and z are periodic */
  int precision;         /* 64: FP64 state and arithmetic; 32: FP32 state and arithmetic */
  int stage_kernel;      /* 0: TMA / tensor-memory stage kernel where the box allows it
                            ((nx+4)*sizeof(real) a multiple of 16 bytes), else plain loads;
                            1: always the plain-load stage kernel (same results) */
  double dx[3];          /* GridData::dx */
  /* RunData */
  double CFL, CFL_tvd, dt, time, outcad;
  int autostep;          /* RunData::autostep (dt computed from the CFL condition) */
  int compensated;       /* FP32 fused steps only: 1 = compensated (Kahan) updates -- a per-cell
                            remainder (stored as bfloat16) carries what rounding the state has dropped: every
                            RK stage sum adds it, stage 4 and each TVD sweep store the new one
                            (zero where Tcheck or a floor changed the value); 0 = plain */
  /* PhysicsData::params */
  double grav, va_max, va_adjust, max_fill;
  /* PhysicsData TVD settings */
  double tvd_h[4], tvd_cs[4], tvd[10], tvd_h_bnd[2], tvd_visc_bnd[2], tvd_eta_bnd[2], tvd_coeff[4];
  double tchk[4];        /* eps_min, rho_min, eps_max, vmax */
  double rt_cfl, rt_tstep, rt_update;
  /* radiative transfer stays outside the path: constant optical depth,
   * zero radiative heating, constant radiative time step */
  double tau0, dt_rad;
  /* PhysicsData::params[i_param_eta]: resistivity in cm^2/s (0: ideal MHD).
   * MHD_Residual then adds eta times the fourth-order Laplacian of B, the ohmic
   * heating eta*|curl B|^2, and the resistive time-step limit
   * (src/mhdres_SR.C:58-61, 422-450, 741-765, 815-819). */
  double eta;
  /* PhysicsData::divB (include/physics.H:43-45): divB_switch > 0 runs Clean_divB
   * after the TVD pass of every fused step (src/solver.C:341-345); divB_itmax caps
   * its adaptive iteration count, divB_err is the target ratio of max|divB|
   * after / before the iterations (src/clean_divB.C:35-369). */
  int divB_switch, divB_itmax;
  double divB_err;
  /* x boundaries of a closed box (periodic_x = 0).  xbnd = 0: mirror rule at
   * both ends (M_x, B_y, B_z change sign).  xbnd = 1: MURaM's physical
   * boundaries, SetBoundaryConditions of src/boundary_pdmp_1_fftw3.C:81-565
   * without the potential-field top: open bottom (mean pressure extrapolated
   * to p_bc, entropy s_bc in upflows, density and energy from the EOS's
   * inverse tables), top closed (bnd_top = 0) or open to outflows (1), top
   * internal energy fixed at bnd_eps_top when positive; bnd_bcrit is
   * PhysicsData::bnd[i_bnd_bcrit] in G.  p_bc, s_bc: the values backup.dat
   * carries; negative ones are set from the bottom layers by the first
   * boundary call (set_p_s_bc), gpumhd_boundary_info reads them back. */
  int xbnd, bnd_top;
  double bnd_bcrit, bnd_eps_top, p_bc, s_bc;
  /* PhysicsData::params[i_param_spitzer]: hyperbolic Spitzer heat conduction
   * (0: off).  A ninth field, the heat flux along B (which = 10 in
   * upload/download, zero at creation), evolves with the RK stages
   * (src/mhdres_SR.C:33-46, 121-145, 355-358, 492-521, 668-692;
   * src/Add_Sources_Integrate_SR.C:410-419). */
  double spitzer;
} gpumhd_params;

typedef struct gpumhd_ctx gpumhd_ctx;

/* Fill p with the reference defaults (src/run.C:8-56, include/physics.H:111-198). */
int gpumhd_default_params(gpumhd_params* p, int nx, int ny, int nz, double dx);

/* Create a context on CUDA device `device`; allocates the device state
 * (GridData::Init, src/grid.C:147-348). */
int gpumhd_create(const gpumhd_params* p, int device, gpumhd_ctx** out);
int gpumhd_destroy(gpumhd_ctx* ctx);
/* Replace the run parameters (e.g. after the host changed Run.dt); the grid
 * shape and precision must not change. */
int gpumhd_set_params(gpumhd_ctx* ctx, const gpumhd_params* p);
int gpumhd_get_params(gpumhd_ctx* ctx, gpumhd_params* p);
/* Text of the last error on this context (or on context creation when ctx is NULL). */
const char* gpumhd_last_error(gpumhd_ctx* ctx);

/* eos_init (src/eos_init.C:57-212): read the binary EOS table and upload it. */
int gpumhd_eos_init(gpumhd_ctx* ctx, const char* path);

/* ACCH::UpdateGPU / ACCH::UpdateCPU of the GridData arrays (src/ACCH.C:114-158):
 * which = 0: U, 1: U0, 2: Res (cState arrays, 8 doubles per node);
 * which = 3..7: pres, temp, ne, rhoi, amb; 8: phi, 9: divB (the divB cleaning's
 * potential and last divergence, GridData::phi / divB); 10: sflx (the Spitzer
 * heat flux, GridData::sflx); 11..20: the diagnostics tvar1..tvar8, Qres, Qvis
 * (GridData, see gpumhd_set_need_diagnostics); one double per node. */
int gpumhd_upload(gpumhd_ctx* ctx, int which, const double* host);
int gpumhd_download(gpumhd_ctx* ctx, int which, double* host);
/* The same with float host arrays: the cState arrays (U, U0) of GridData in
 * MURaM built with SINGLE_PRECISION (include/precision.h:4-10,
 * include/physics.H:77: cState<real>, 8 floats per node; GridData's other
 * arrays stay double, include/grid.H:53-100).  Any field takes either layout,
 * and either precision of context accepts both. */
int gpumhd_upload_f32(gpumhd_ctx* ctx, int which, const float* host);
int gpumhd_download_f32(gpumhd_ctx* ctx, int which, float* host);
/* The same transfers without waiting (no reference counterpart): each one
 * is ordered with the context's steps as the synchronous call is, but its
 * host copy runs on a copy stream of its own, so that the upload of one
 * step's input and the download of another step's result overlap the steps
 * in between.  The host buffer must stay valid (and, for an upload,
 * unchanged) until gpumhd_synchronize, which also waits for these copies;
 * pinned host memory makes the copies asynchronous.  Each direction has two
 * device-side buffers used in turn (2 x 8 doubles per node, allocated on the
 * first asynchronous call); a third transfer waits for the first one's
 * buffer, so any number may be queued. */
int gpumhd_upload_async(gpumhd_ctx* ctx, int which, const double* host);
int gpumhd_download_async(gpumhd_ctx* ctx, int which, double* host);
/* The asynchronous transfers with float host arrays (SINGLE_PRECISION layout). */
int gpumhd_upload_async_f32(gpumhd_ctx* ctx, int which, const float* host);
int gpumhd_download_async_f32(gpumhd_ctx* ctx, int which, float* host);

/* Clean_divB (include/divB.H:5, src/clean_divB.C:35-369): damped iterations
 * phi += fac*divB - 0.65*phi, B += grad phi, e += phi*divB on U, their count
 * adapted from call to call as the reference's function static does (starts
 * at 3).  phi persists in the context (zero at creation; which = 8 above).
 * gpumhd_divb_info: the last call's iteration count, the next call's, and
 * max|divB| before / after it in G (the reference's verbose log line). */
int gpumhd_clean_divB(gpumhd_ctx* ctx);
/* The open bottom's current p_bc and s_bc (WriteBackupFile,
 * src/boundary_pdmp_1_fftw3.C:44-50, writes them to backup.dat). */
int gpumhd_boundary_info(gpumhd_ctx* ctx, double* p_bc, double* s_bc);
int gpumhd_divb_info(gpumhd_ctx* ctx, int* last_iters, int* next_iters, double* err_before, double* err_after);
/* Set the iteration count the next Clean_divB call (per routine or inside a
 * fused step) starts from: the function static next_iter of src/clean_divB.C
 * (starts at 3), which MURaM keeps only in memory and restarts at 3.  For
 * carrying it across a restart, or for running two contexts on one iteration
 * sequence; 1 <= next_iters <= max(3, divB_itmax), else GPUMHD_E_INVALID.
 * Stream-ordered with the context's other calls. */
int gpumhd_set_divb_iters(gpumhd_ctx* ctx, int next_iters);

/* RunData::need_diagnostics (include/run.H; set per stage by src/solver.C:
 * 264-289): on = 1 zeroes the ten diagnostic arrays (which = 11..20) and makes
 * the per-routine calls that follow fill them as the reference's do on an
 * output step -- MHD_Residual: tvar1 the energy-flux divergence (tvar2 its
 * conduction share), tvar3 the Lorentz force's work (src/mhdres_SR.C:
 * 368-384, 434-435, 689-702, 751-752); Source_Integrate_Tcheck: tvar4 the
 * radiation factor, tvar5 the gravity work, tvar6 the Boris energy, tvar7
 * += Tcheck's energy change / dt (src/Add_Sources_Integrate_SR.C:122-296);
 * TVDlimit: tvar8 its energy change, tvar6 its Boris part, Qres and Qvis the
 * resistive and viscous heating, tvar7 its energy floor's change, per unit
 * of Run.dt (src/tvdlimit_SR.C:577-667); TCheck: tvar7 (:618-620).  MURaM
 * sets it at stage 4 of an output step and clears it at the next stage 1.
 * Fused steps refuse to run while it is on. */
int gpumhd_set_need_diagnostics(gpumhd_ctx* ctx, int on);
/* SaveCons (include/src_int_tck.H:10, src/Add_Sources_Integrate_SR.C:475-531). */
int gpumhd_save_cons(gpumhd_ctx* ctx);
/* ConsToPrim (include/eos.H:39, src/cons_to_prim.C:78-266).  The state
 * becomes primitive in place and the pressure is stored; temperature, n_e,
 * rho_i and amb (fields 4-7) are formed on their first access (download,
 * upload of one of them, the Spitzer residual) from the density and internal
 * energy this call saw, so they hold this call's values whatever happens to
 * the state in between. */
int gpumhd_cons_to_prim(gpumhd_ctx* ctx);
/* Adjust_Valf_Max (include/limit_va.H:7, src/Adjust_Valf_Max.C:25-150). */
int gpumhd_adjust_valf_max(gpumhd_ctx* ctx);
/* The globals inv_va2max, v_lim, e_lim (include/limit_va.H:5). */
int gpumhd_get_limits(gpumhd_ctx* ctx, double* inv_va2max, double* v_lim, double* e_lim);
/* MHD_Residual (include/mhd_tvd.H:5, src/mhdres_SR.C:27-854): Res += residual,
 * *dt_mhd = dxmin / cmax. */
int gpumhd_mhd_residual(gpumhd_ctx* ctx, double* dt_mhd);
/* Sync_timestep (src/solver.C:487-548, file-local in the reference). */
int gpumhd_sync_timestep(gpumhd_ctx* ctx, double dt_rad, double dt_mhd, double* cfl);
/* Source_Integrate_Tcheck (include/src_int_tck.H:8-9, src/Add_Sources_Integrate_SR.C:38-472). */
int gpumhd_source_integrate_tcheck(gpumhd_ctx* ctx, int stage);
/* TVDlimit (include/mhd_tvd.H:6, src/tvdlimit_SR.C:33-695). */
int gpumhd_tvdlimit(gpumhd_ctx* ctx, double dt_tvd);
/* TCheck (include/src_int_tck.H:7, src/Add_Sources_Integrate_SR.C:534-625). */
int gpumhd_tcheck(gpumhd_ctx* ctx);
/* exchange_grid_acc (include/exchange.H:8, src/exchange.C:532-783) on one GPU:
 * periodic ghost fill; with_bc = 1 also applies the closed-x mirror rule
 * (SetBoundaryConditions with OPEN_TOP = 0, src/boundary_pdmp_1_fftw3.C:415-447). */
int gpumhd_exchange(gpumhd_ctx* ctx, int with_bc);

/* Fused path: advance `nsteps` full time steps (SaveCons, 4 RK stages,
 * Sync_timestep, TVD, TCheck, boundaries; src/solver.C:109-365) entirely on
 * the device.  Equivalent to the per-routine calls above on U in conserved
 * form with filled ghosts.  With adaptive limits (va_adjust > 0) each step
 * also updates the limits on the device from the previous pass's statistics
 * and takes the stage-1 CFL speed in one more pass; the limits' history (the
 * reference's function statics) carries over between per-routine and fused
 * calls.  dt_out (may be NULL) receives dt of each step.
 * With capture = 1 the step sequence is recorded once as a CUDA graph and
 * replayed. */
int gpumhd_run_steps(gpumhd_ctx* ctx, int nsteps, double* dt_out, int capture);
/* Enqueue `nsteps` fused steps without synchronising or reading results. */
int gpumhd_enqueue_steps(gpumhd_ctx* ctx, int nsteps);
/* Wait for the context's stream and report any device-side error flag. */
int gpumhd_synchronize(gpumhd_ctx* ctx);
/* Device-side step diagnostics after gpumhd_synchronize: dt, cfl, time,
 * and whether the last step took the two-half-step TVD branch. */
int gpumhd_step_info(gpumhd_ctx* ctx, double* dt, double* cfl, double* time, int* tvd_two_half);

/* Run `nsteps` fused steps without graph capture, timing each launch with CUDA
 * events on the context's stream; ms_phase[13] receives the mean duration of:
 * step control, RK stages 1-4, TVD x/y/z sweeps, second-half TVD x/y/z sweeps,
 * divB cleaning (0 when divB_switch = 0), the end-of-step pass (TCheck, ghost
 * images, next pressure and statistics). */
int gpumhd_profile_steps(gpumhd_ctx* ctx, int nsteps, double* ms_phase);
/* MHD_Residual's CFL time step, dt_mhd = dxmin / cmax, computed with no device
 * allocation at all.  No counterpart in the reference: it exists for callers
 * that own their device arrays and must not allocate -- e.g. a MURaM build
 * whose fields belong to the OpenACC runtime, or a time-step loop that cannot
 * afford cudaMalloc's device-wide synchronisation.  Inputs are the caller's
 * device arrays in this library's FP64 layout: U_prim holds primitives as
 * ConsToPrim leaves them (8 fields of (nx+4)(ny+4)(nz+4) doubles, x fastest),
 * pres the pressure; dx[3] and inv_va2max are host values; dt_out is a device
 * double the result is written to, in stream order on `stream` (a
 * cudaStream_t, NULL for the default stream).  The result is the CFL term
 * only: MHD_Residual also takes min(dt, dt_diff_fac/eta) when resistivity is
 * on (src/mhdres_SR.C:815-819), so a resistive run takes that minimum itself.
 * The speeds are those of MHD_Residual's pencils: interior cells and face
 * ghosts (one index in a ghost layer), not edge or corner ghosts.
 * Scratch: a fixed 32 KiB __device__ array, one partial per z plane, so
 * nz + 4 must not exceed 4096 (GPUMHD_E_INVALID otherwise).  The first call
 * on each device looks up that array's device address and keeps it for the
 * life of the process; make it before any stream capture, and do not call
 * the function again after a cudaDeviceReset (the library may then sit at
 * another address).  All calls share the array: calls that overlap on the
 * GPU race. */
int gpumhd_cfl_dt_noalloc(const double* U_prim, const double* pres, int nx, int ny, int nz, const double dx[3],
                          double inv_va2max, void* stream, double* dt_out);
/* The CUDA stream the context enqueues on (a cudaStream_t). */
void* gpumhd_stream(gpumhd_ctx* ctx);
/* Number of kernels the context has launched so far: those it enqueued plus
 * those that captured steps ran through their conditional nodes (the second
 * TVD half pass); exact after gpumhd_synchronize. */
long long gpumhd_launch_count(gpumhd_ctx* ctx);

/* Benchmark / test set-up, no counterpart in the reference: the state of ctx
 * becomes the periodic tiling of src's state (same precision; ctx's interior
 * sizes multiples of src's), ghosts filled by ctx's boundary rule. */
int gpumhd_tile_from(gpumhd_ctx* ctx, gpumhd_ctx* src);

/* ---- launch shapes (no counterpart in the reference: GPU tiling only) ----
 * stage_zchunk: z planes per stage-kernel block (0: chosen from the GPU's
 * occupancy); tvd_chunk: cells per thread of the y / z TVD sweeps (0: 32).
 * Results do not depend on them. */
int gpumhd_set_tuning(gpumhd_ctx* ctx, int stage_zchunk, int tvd_chunk);
/* Test hook of the TMA stage kernel's bounded waits (no counterpart in the
 * reference; for testing the error path only).  wait_cycles limits each wait
 * for a plane's copy in SM clock cycles (0: the default, about one second);
 * withhold_last = 1 makes every block of the kernel skip the copy of the last
 * plane it needs, so that its wait for that plane runs out: the block records
 * ERR_WAIT_TIMEOUT, waits for the copies it did issue, frees its tensor memory
 * and returns; the rest of the step returns at once, and gpumhd_synchronize
 * (or MHD_Residual) reports GPUMHD_E_CUDA.  Drops the captured step graph;
 * ensembles built before keep their launch parameters. */
int gpumhd_test_tma_wait(gpumhd_ctx* ctx, long long wait_cycles, int withhold_last);
/* stage_kernel: 0 when the TMA / tensor-memory stage kernel runs, 1 for the
 * plain-load kernel. */
int gpumhd_get_tuning(gpumhd_ctx* ctx, int* stage_kernel, int* stage_zchunk, int* tvd_chunk);
/* Autotuner: times the candidate stage kernels, z chunks and TVD chunks on
 * the context's own state (trial_steps timed steps each; the state, its
 * pressure and the step scalars are restored afterwards) and keeps the
 * fastest; *best_ms receives its time per step. */
int gpumhd_autotune(gpumhd_ctx* ctx, int trial_steps, double* best_ms);

/* ---- adjoint (no counterpart in the reference) ----
 * Gradient of an objective J(U_T) with respect to the initial state U_0, where
 * U_0 is the context's current state and U_T the state after nsteps fused
 * steps of fixed dt (FP64 context, periodic box, autostep = 0, dt > 0, one TVD
 * pass per step, fixed limits: va_adjust = 0).  dJ_dUT: dJ/dU_T in the host
 * cState layout (8 doubles per cell, ghosts included and ignored); dJ_dU0
 * receives dJ/dU_0 in the same layout (ghost records zero).  The hand-written adjoint of the step (stages
 * with MHD_Residual, sources, Boris correction and Tcheck, ConsToPrim's
 * pressure, the three TVD sweeps) runs backwards in time; forward states are
 * kept every checkpoint_every steps and recomputed in between.  Limiter kinks
 * and clamps take the derivative of the branch the forward step took.  The
 * context's state is left unchanged. */
int gpumhd_adjoint(gpumhd_ctx* ctx, int nsteps, int checkpoint_every, const double* dJ_dUT, double* dJ_dU0);

/* ---- ensembles of independent boxes (no counterpart in the reference) ----
 * An ensemble advances several contexts (boxes of any sizes and precisions on
 * one device) together: one CUDA graph whose while-loop body is one fused step
 * of every box, the boxes running as parallel branches, so that a single graph
 * launch runs all requested steps.  The boxes must have their EOS and state
 * loaded; the ensemble does not own them (destroy it before them). */
typedef struct gpumhd_ensemble gpumhd_ensemble;
int gpumhd_ensemble_create(gpumhd_ctx* const* boxes, int n, gpumhd_ensemble** out);
int gpumhd_ensemble_destroy(gpumhd_ensemble* e);
/* nsteps steps of every box in one graph launch; ordered after the work
 * already queued on the boxes' streams, and later calls on a box wait for it. */
int gpumhd_ensemble_enqueue_steps(gpumhd_ensemble* e, int nsteps);
/* Waits for the ensemble and returns the first box error (as gpumhd_synchronize). */
int gpumhd_ensemble_synchronize(gpumhd_ensemble* e);
const char* gpumhd_ensemble_last_error(gpumhd_ensemble* e);
void* gpumhd_ensemble_stream(gpumhd_ensemble* e);
long long gpumhd_ensemble_launch_count(gpumhd_ensemble* e);
/* The ensemble's schedule: steps_per_iteration (1..64) steps of each box per
 * loop iteration (a chain of fused steps per box between one fork and one
 * join, so the boxes meet once per that many steps; a call's remaining
 * nsteps % steps_per_iteration steps run one per iteration), and
 * largest_first != 0 captures the branches in order of decreasing cell
 * count.  Rebuilds the graphs after waiting for the ensemble and its boxes;
 * results do not depend on the schedule. */
int gpumhd_ensemble_set_schedule(gpumhd_ensemble* e, int steps_per_iteration, int largest_first);
/* Launch shapes of the boxes for running inside the ensemble: each box's
 * current shapes, or stage z chunks of half or all of its z extent with TVD
 * chunks of 64 or 128 cells (longer marches pay when the other boxes fill the
 * GPU), timed over trial_steps steps of the ensemble from the boxes' current
 * states and restored states afterwards (state, pressure, divB potential,
 * heat flux, step control); keeps the fastest, branches largest box first.
 * *best_ms: its time per ensemble step. */
int gpumhd_ensemble_autotune(gpumhd_ensemble* e, int trial_steps, double* best_ms);

#ifdef __cplusplus
}
#endif
#endif
