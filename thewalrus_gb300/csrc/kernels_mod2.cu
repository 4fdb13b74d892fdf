// Sieve kernels for residues modulo 2147483587 (exact sieves of integer inputs), one per register
// class (the classes of pick_ns).
#include "arith.cuh"
#define WG_UNIT_PRIME 2147483587u
#define WG_UNIT_SCALAR wg::modp<2147483587u>
#define WG_UNIT_NAME mod2
#define WG_UNIT_CLASSES(X) X(4) X(8) X(12)
#include "kernels_unit.cuh"
