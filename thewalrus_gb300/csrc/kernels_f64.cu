// The sieve kernel for real FP64 terms.
#define WG_UNIT_SCALAR double
#define WG_UNIT_NAME f64
#include "kernels_unit.cuh"
