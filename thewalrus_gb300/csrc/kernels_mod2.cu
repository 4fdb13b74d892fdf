// The sieve kernel for residues modulo 2147483587 (exact sieves of integer inputs).
#include "arith.cuh"
#define WG_UNIT_PRIME 2147483587u
#define WG_UNIT_SCALAR wg::modp<2147483587u>
#define WG_UNIT_NAME mod2
#include "kernels_unit.cuh"
