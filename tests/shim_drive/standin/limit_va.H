/* Stand-in declarations with MURaM's signatures (include/limit_va.H). */
#pragma once
#include "grid.H"
#include "run.H"
extern double inv_va2max, v_lim, e_lim;
void Adjust_Valf_Max(const RunData& Run, const GridData& Grid, const PhysicsData& Physics);
double lfac(double va2);
