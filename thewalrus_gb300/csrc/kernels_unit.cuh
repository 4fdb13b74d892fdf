// Body of one kernel translation unit: define WG_UNIT_SCALAR (the scalar type), WG_UNIT_NAME (the
// suffix of the entry points) and, for the residue types, WG_UNIT_PRIME, then include this file.
#include "kernels.h"

namespace wg {

#define WG_CAT2(a, b) a##b
#define WG_CAT(a, b) WG_CAT2(a, b)

cudaError_t WG_CAT(sieve_launch_, WG_UNIT_NAME)(const SieveParams& p, int ctas, int wpc, cudaStream_t st) {
  auto k = sieve_kernel<WG_UNIT_SCALAR>;
  const int smem = wpc * p.L.bytes;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  k<<<ctas, 32 * wpc, smem, st>>>(p);
  return cudaGetLastError();
}

int WG_CAT(sieve_occupancy_, WG_UNIT_NAME)(int wpc, int smem) {
  int nb = 0;
  auto k = sieve_kernel<WG_UNIT_SCALAR>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, 32 * wpc, smem) != cudaSuccess) return 0;
  return nb;
}

cudaError_t WG_CAT(sieve_tables_, WG_UNIT_NAME)(const double* binom, const double* inv) {
  cudaError_t e = cudaMemcpyToSymbol(c_binom, binom, sizeof(c_binom));
  if (e != cudaSuccess) return e;
  e = cudaMemcpyToSymbol(c_inv, inv, sizeof(c_inv));
#ifdef WG_UNIT_PRIME
  if (e != cudaSuccess) return e;
  uint32_t invmod[256];  // 1/k mod p by k * inv(k) = 1: inv(k) = -(p / k) inv(p mod k)
  invmod[0] = 0;
  invmod[1] = 1;
  const uint64_t P = WG_UNIT_PRIME;
  for (uint64_t k = 2; k < 256; ++k) invmod[k] = (uint32_t)((P - (P / k) * invmod[P % k] % P) % P);
  for (int k = 0; k < 256; ++k) invmod[k] = Montgomery<WG_UNIT_PRIME>::to_mont(invmod[k]);
  e = cudaMemcpyToSymbol(c_invmod, invmod, sizeof(invmod));
#endif
  return e;
}

#undef WG_CAT
#undef WG_CAT2

}  // namespace wg
