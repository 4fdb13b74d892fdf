// Sieve kernels for complex double-float terms, one per register class (the classes of pick_ns).
#define WG_UNIT_SCALAR cdf
#define WG_UNIT_NAME cdf
#define WG_UNIT_CLASSES(X) X(4) X(6) X(8) X(10)
#include "kernels_unit.cuh"
