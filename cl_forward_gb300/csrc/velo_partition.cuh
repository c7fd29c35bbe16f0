// velo_partition.cuh -- the reference's per-module sort step on the device:
// the first-element-pivot partition of Tools.cpp:125-157, with x, y, z and
// the hit IDs moving together, replayed where the permutation it makes is
// not simply "ascending x" (equal x values: it swaps equal neighbours).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace velo {

__device__ __forceinline__ void swap4(float* a, float* b, float* c, uint32_t* d, int i, int j) {
  float t = a[i]; a[i] = a[j]; a[j] = t;
  t = b[i]; b[i] = b[j]; b[j] = t;
  t = c[i]; c[i] = c[j]; c[j] = t;
  const uint32_t u = d[i]; d[i] = d[j]; d[j] = u;
}

__device__ __forceinline__ int partition4(float* a, float* b, float* c, uint32_t* d, int lo, int hi) {
  const float pivot = a[lo];
  int l = lo, r = hi;
  while (l < r) {
    while (a[r] > pivot) r--;   // stops at lo at the latest: a[lo] == pivot
    while (l < r && a[l] <= pivot) l++;
    if (l < r) swap4(a, b, c, d, l, r);
  }
  swap4(a, b, c, d, r, lo);
  return r;
}

constexpr int kSortStack = 64;   // >= 2 * log2(VELO_MAX_MODULE_HITS + 1) + 2

// The reference's partition steps over [lo0, hi0] (one thread), the
// smaller side first so that the explicit stack stays within 2 log2(n)
// entries.  x must be finite (the reference's sort does not return on NaN).
__device__ inline void quicksort4(float* x, float* y, float* z, uint32_t* id, int lo0, int hi0) {
  int lo_s[kSortStack], hi_s[kSortStack];
  int sp = 0;
  lo_s[sp] = lo0;
  hi_s[sp] = hi0;
  sp++;
  while (sp > 0 && sp <= kSortStack - 2) {
    --sp;
    const int lo = lo_s[sp], hi = hi_s[sp];
    if (lo >= hi) continue;
    const int p = partition4(x, y, z, id, lo, hi);
    if (p - lo > hi - p) {
      lo_s[sp] = lo; hi_s[sp] = p - 1; sp++;
      lo_s[sp] = p + 1; hi_s[sp] = hi; sp++;
    } else {
      lo_s[sp] = p + 1; hi_s[sp] = hi; sp++;
      lo_s[sp] = lo; hi_s[sp] = p - 1; sp++;
    }
  }
}

}  // namespace velo
