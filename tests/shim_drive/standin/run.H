/* Stand-in RunData: the members the shim reads (see physics.H). */
#pragma once

class RunData {
 public:
  double CFL, CFL_tvd, dt, time, outcad;
  int autostep, diagnostics, need_diagnostics;
  char eos_name[512];
};
