/* Stand-in declaration with MURaM's signature (include/icbc.H). */
#pragma once
#include "grid.H"
#include "run.H"
class RTS;
void SetBoundaryConditions(const RunData& Run, GridData& Grid, const PhysicsData& Physics, const int stage,
                           const int pt_update, RTS* rts);
