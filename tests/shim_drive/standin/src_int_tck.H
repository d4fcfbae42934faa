/* Stand-in declarations with MURaM's signatures (include/src_int_tck.H). */
#pragma once
#include "grid.H"
#include "run.H"
void TCheck(const RunData& Run, GridData& Grid, const PhysicsData& Physics);
void Source_Integrate_Tcheck(const RunData& Run, GridData& Grid, const PhysicsData& Physics, const int stage);
void SaveCons(GridData& Grid, const PhysicsData& Physics);
