// Sieve kernels for complex FP64 terms, one per register class (the classes of pick_ns).
#define WG_UNIT_SCALAR c64
#define WG_UNIT_NAME c64
#define WG_UNIT_CLASSES(X) X(4) X(6) X(8) X(10)
#include "kernels_unit.cuh"
