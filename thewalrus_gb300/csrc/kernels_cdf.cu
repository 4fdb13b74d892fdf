// The sieve kernel for complex double-float terms.
#define WG_UNIT_SCALAR cdf
#define WG_UNIT_NAME cdf
#include "kernels_unit.cuh"
