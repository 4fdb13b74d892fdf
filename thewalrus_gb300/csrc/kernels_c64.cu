// The sieve kernel for complex FP64 terms.
#define WG_UNIT_SCALAR c64
#define WG_UNIT_NAME c64
#include "kernels_unit.cuh"
