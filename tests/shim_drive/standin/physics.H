/* Stand-in declarations of the MURaM types and parameter indices that the
 * shim (muram_main_gb300/shim/gpumhd_muram_shim.C) reads: the member names
 * must match MURaM's, the index values and array sizes are this harness's own. */
#pragma once
#include "precision.h"

namespace MHD {
template <class T>
struct cState {
  T v[8];  // rho, M (3), e, B (3): one grid node
};
}  // namespace MHD
typedef MHD::cState<real> cState;

enum { i_param_grav, i_param_va_max, i_param_va_adjust, i_param_max_fill, i_param_eta, i_param_spitzer,
       i_param_ambipolar, n_param_standin };
enum { i_rt_cfl, i_rt_tstep, i_rt_update, n_rt_standin };
enum { i_divB_switch, i_divB_itmax, i_divB_err, n_divB_standin };
enum { i_bnd_top, i_bnd_bcrit, i_bnd_eps_top, i_bnd_pot, n_bnd_standin };
enum { i_dmp_switch, n_dmp_standin };
enum { i_ext_cor, n_ext_standin };

class PhysicsData {
 public:
  double params[n_param_standin];
  double tvd_h[4], tvd_cs[4], tvd_coeff[4], tchk[4], tvd[10];
  double tvd_h_bnd[2], tvd_visc_bnd[2], tvd_eta_bnd[2];
  double rt[n_rt_standin], divB[n_divB_standin], bnd[n_bnd_standin], dmp[n_dmp_standin], rt_ext[n_ext_standin];
};
