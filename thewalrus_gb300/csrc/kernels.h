// Sieve-kernel instantiations live in one translation unit per scalar class (kernels_c64.cu,
// kernels_cdf.cu, kernels_f64.cu, kernels_fdf.cu, kernels_cdd.cu, kernels_fdd.cu,
// kernels_mod{0..4}.cu: residues modulo one prime each) so that they compile in parallel.  Each unit
// instantiates sieve_kernel<S> and holds its own copy of the constant tables (binomials,
// reciprocals), which the host fills through sieve_tables_*.
#pragma once
#include <cuda_runtime.h>

#include "sieve_kernel.cuh"

namespace wg {

#define WG_KERNEL_UNIT_DECL(T)                                                                      \
  cudaError_t sieve_launch_##T(const SieveParams& p, int ctas, int wpc, cudaStream_t st); \
  int sieve_occupancy_##T(int wpc, int smem);                                             \
  cudaError_t sieve_tables_##T(const double* binom, const double* inv);

WG_KERNEL_UNIT_DECL(c64)
WG_KERNEL_UNIT_DECL(cdf)
WG_KERNEL_UNIT_DECL(f64)
WG_KERNEL_UNIT_DECL(fdf)
WG_KERNEL_UNIT_DECL(cdd)
WG_KERNEL_UNIT_DECL(fdd)
WG_KERNEL_UNIT_DECL(mod0)
WG_KERNEL_UNIT_DECL(mod1)
WG_KERNEL_UNIT_DECL(mod2)
WG_KERNEL_UNIT_DECL(mod3)
WG_KERNEL_UNIT_DECL(mod4)
#undef WG_KERNEL_UNIT_DECL

}  // namespace wg
