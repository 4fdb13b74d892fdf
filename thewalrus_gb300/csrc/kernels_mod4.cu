// The sieve kernel for residues modulo 2147483563 (exact sieves of integer inputs).
#include "arith.cuh"
#define WG_UNIT_PRIME 2147483563u
#define WG_UNIT_SCALAR wg::modp<2147483563u>
#define WG_UNIT_NAME mod4
#include "kernels_unit.cuh"
