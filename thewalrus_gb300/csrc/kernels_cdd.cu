// The sieve kernel for complex double-double terms.
#define WG_UNIT_SCALAR cdd
#define WG_UNIT_NAME cdd
#include "kernels_unit.cuh"
