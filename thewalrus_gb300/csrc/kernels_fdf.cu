// Sieve kernels for real double-float terms, one per register class (the classes of pick_ns).
#define WG_UNIT_SCALAR dfr
#define WG_UNIT_NAME fdf
#define WG_UNIT_CLASSES(X) X(4) X(8) X(12)
#include "kernels_unit.cuh"
