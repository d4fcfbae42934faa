/* Stand-in GridData: the members the shim reads (see physics.H). */
#pragma once
#include "physics.H"

class GridData {
 public:
  int lsize[3], procs[3], periods[3];
  real dx[3];
  int bufsize;
  cState *U, *U0, *Res;
  double *pres, *temp, *ne, *rhoi, *amb, *Tau, *sflx, *divB, *phi;
  double *tvar1, *tvar2, *tvar3, *tvar4, *tvar5, *tvar6, *tvar7, *tvar8, *Qres, *Qvis;
};
