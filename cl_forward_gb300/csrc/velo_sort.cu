// velo_sort.cu -- the reference's per-module x-sort (preorder_by_x,
// Tools.cpp:46-66) on the device, in place on staged events.
//
// One thread sorts one module's hits (x, y, z and ID move together) with the
// first-element-pivot partition of Tools.cpp:125-157, so the permutation --
// equal x values included -- is the reference's: output hit indices refer to
// the sorted order, so it has to be.  Subranges are disjoint, so their order
// of processing does not change the result; taking the smaller one first
// bounds the explicit stack at 2 log2(n) entries.
#include <cuda_runtime.h>

#include "velo_internal.h"

namespace velo {
namespace {

__device__ __forceinline__ void swap4(float* a, float* b, float* c, uint32_t* d, int i, int j) {
  float t = a[i]; a[i] = a[j]; a[j] = t;
  t = b[i]; b[i] = b[j]; b[j] = t;
  t = c[i]; c[i] = c[j]; c[j] = t;
  const uint32_t u = d[i]; d[i] = d[j]; d[j] = u;
}

__device__ int partition4(float* a, float* b, float* c, uint32_t* d, int lo, int hi) {
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

constexpr int kStack = 64;   // >= 2 * log2(VELO_MAX_MODULE_HITS + 1) + 2

__global__ void sort_modules_kernel(uint8_t* input, const uint64_t* offsets, const uint32_t* valid, int n_events) {
  const int e = blockIdx.x;
  if (e >= n_events || !valid[e]) return;
  int32_t* hdr = reinterpret_cast<int32_t*>(input + offsets[e]);
  const int S = hdr[0], H = hdr[1];
  const int32_t* start = hdr + 2 + S;
  const int32_t* num = start + S;
  uint32_t* id = reinterpret_cast<uint32_t*>(hdr + 2 + 3 * S);
  float* x = reinterpret_cast<float*>(id + H);
  float* y = x + H;
  float* z = y + H;
  // the module table must tile [0, H) in order before anything moves
  bool bad = threadIdx.x == 0 && S == 0 && H != 0;
  for (int m = threadIdx.x; m < S; m += blockDim.x) {
    const int64_t expect = m == 0 ? 0 : (int64_t)start[m - 1] + (int64_t)num[m - 1];
    bad |= num[m] < 0 || num[m] > VELO_MAX_MODULE_HITS || (int64_t)start[m] != expect ||
           (m == S - 1 && (int64_t)start[m] + (int64_t)num[m] != (int64_t)H);
  }
  if (__syncthreads_or(bad)) return;
  for (int m = threadIdx.x; m < S; m += blockDim.x) {
    // a non-finite x would stall the partition (the reference's sort never
    // returns on a NaN); such a module stays unsorted and the search marks
    // its event invalid
    bool finite = true;
    for (int i = start[m]; i < start[m] + num[m]; ++i) finite &= isfinite(x[i]) != 0;
    if (!finite) continue;
    int lo_s[kStack], hi_s[kStack];
    int sp = 0;
    lo_s[sp] = start[m];
    hi_s[sp] = start[m] + num[m] - 1;
    sp++;
    while (sp > 0 && sp <= kStack - 2) {
      --sp;
      const int lo = lo_s[sp], hi = hi_s[sp];
      if (lo >= hi) continue;
      const int p = partition4(x, y, z, id, lo, hi);
      // push the larger side first so the smaller one is processed next
      if (p - lo > hi - p) {
        lo_s[sp] = lo; hi_s[sp] = p - 1; sp++;
        lo_s[sp] = p + 1; hi_s[sp] = hi; sp++;
      } else {
        lo_s[sp] = p + 1; hi_s[sp] = hi; sp++;
        lo_s[sp] = lo; hi_s[sp] = p - 1; sp++;
      }
    }
  }
}

}  // namespace

int launch_sort_modules(uint8_t* input, const uint64_t* offsets, const uint32_t* valid, int n_events, void* stream) {
  if (n_events <= 0) return 0;
  sort_modules_kernel<<<n_events, 64, 0, (cudaStream_t)stream>>>(input, offsets, valid, n_events);
  return (int)cudaGetLastError();
}

}  // namespace velo
