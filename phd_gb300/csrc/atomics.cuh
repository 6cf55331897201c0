// Atomic maxima of non-negative doubles kept as 64-bit patterns (for
// non-negative IEEE doubles the order of the bit patterns is the order of
// the values).
#pragma once
#include <cuda_runtime.h>

__device__ inline void atomic_max_nonneg(unsigned long long* addr, double v) {
  atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// atomic_max_nonneg with the lanes of the warp that name the same address
// combined first (one atomic per address and warp instead of one per lane;
// the maximum of non-negative doubles is the maximum of their bit patterns,
// taken on the high, then the low 32 bits).  Every active lane calls it.
__device__ inline void atomic_max_nonneg_warp(unsigned long long* addr, double v) {
  const unsigned act = __activemask();
  const unsigned grp = __match_any_sync(act, (unsigned long long)addr);
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned mhi = __reduce_max_sync(grp, hi);
  const unsigned mlo = __reduce_max_sync(grp, hi == mhi ? lo : 0u);
  if ((int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicMax(addr, ((unsigned long long)mhi << 32) | mlo);
}
