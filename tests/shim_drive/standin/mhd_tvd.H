/* Stand-in declarations with MURaM's signatures (include/mhd_tvd.H). */
#pragma once
#include "grid.H"
#include "run.H"
double MHD_Residual(const RunData& Run, GridData& Grid, const PhysicsData& Physics);
void TVDlimit(const RunData& Run, GridData& Grid, const PhysicsData& Physics, const double dt_tvd);
