// MURaM's host eos_init builds the host EOS tables that code outside the hot
// path reads; nothing here reads them.  It sits in a translation unit of its
// own so that drive.C's call is an undefined reference, which the linker's
// --wrap sends to the shim's wrapper (and the wrapper's __real_ call here).
#include "eos.H"

void eos_init(GridData&, RunData&, const PhysicsData&) {}
