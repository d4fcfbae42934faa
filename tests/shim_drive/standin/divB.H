/* Stand-in declaration with MURaM's signature (include/divB.H). */
#pragma once
#include "grid.H"
#include "run.H"
void Clean_divB(const RunData& Run, GridData& Grid, const PhysicsData& Physics);
