// Device helpers shared by the kernel units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "wpic_internal.h"

namespace wpic {

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): counter-based generator used by the device loader.
__device__ __forceinline__ uint4 philox4x32(uint4 ctr, uint2 key) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const unsigned hi0 = __umulhi(0xD2511F53u, ctr.x), lo0 = 0xD2511F53u * ctr.x;
    const unsigned hi1 = __umulhi(0xCD9E8D57u, ctr.z), lo1 = 0xCD9E8D57u * ctr.z;
    ctr = make_uint4(hi1 ^ ctr.y ^ key.x, lo1, hi0 ^ ctr.w ^ key.y, lo0);
    key.x += 0x9E3779B9u;
    key.y += 0xBB67AE85u;
  }
  return ctr;
}

// uniform double in (0, 1] from 53 random bits
__device__ __forceinline__ double u01(unsigned a, unsigned b) {
  const unsigned long long m = ((unsigned long long)(a >> 5) << 26) | (b >> 6);
  return ((double)m + 1.0) * (1.0 / 9007199254740992.0);
}

}  // namespace wpic
