/* Stand-in declaration with MURaM's signature (include/exchange.H). */
#pragma once
#include "grid.H"
void exchange_grid_acc(GridData& Grid, const PhysicsData& Physics, const int with_bc);
