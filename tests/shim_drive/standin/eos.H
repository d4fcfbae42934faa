/* Stand-in declarations with MURaM's signatures (include/eos.H). */
#pragma once
#include "grid.H"
#include "run.H"
void eos_init(GridData& Grid, RunData& Run, const PhysicsData& Physics);
void ConsToPrim(GridData& Grid, const PhysicsData& Physics, const RunData& Run);
