// The sieve kernel for real double-float terms.
#define WG_UNIT_SCALAR dfr
#define WG_UNIT_NAME fdf
#include "kernels_unit.cuh"
