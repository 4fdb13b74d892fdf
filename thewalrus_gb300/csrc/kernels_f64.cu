// Sieve kernels for real FP64 terms, one per register class (the classes of pick_ns).
#define WG_UNIT_SCALAR double
#define WG_UNIT_NAME f64
#define WG_UNIT_CLASSES(X) X(4) X(8) X(12)
#include "kernels_unit.cuh"
