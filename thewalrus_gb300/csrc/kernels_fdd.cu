// The sieve kernel for real double-double terms.
#define WG_UNIT_SCALAR ddr
#define WG_UNIT_NAME fdd
#include "kernels_unit.cuh"
