// The sieve kernel for residues modulo 2147483629 (exact sieves of integer inputs).
#include "arith.cuh"
#define WG_UNIT_PRIME 2147483629u
#define WG_UNIT_SCALAR wg::modp<2147483629u>
#define WG_UNIT_NAME mod1
#include "kernels_unit.cuh"
