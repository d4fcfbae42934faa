/* Stand-in for MURaM's precision header, for driving the MURaM-side shim on a
 * machine without MURaM's sources: `real` is the cState element type. */
#pragma once
#ifdef SINGLE_PRECISION
typedef float real;
#else
typedef double real;
#endif
